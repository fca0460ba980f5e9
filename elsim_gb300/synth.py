"""Seeded synthetic microstructures standing in for the reference's inputs.

The reference reads production voxel/distance files that are not in its
repository (SBMES:138-151, LevelSet_3D.f90:60-63), so every input here is
generated: overlapping spheres with radii uniform in [rmin, rmax] voxels,
added at uniform random centres until the solid fraction reaches the target,
optionally a cylindrical tunnel carved out of the solid along a random axis.
The signed distance comes from the sign field by level-set reinitialisation
(ReDist3D_XYZ, run on the GPU), and psi = 0.5 (1 + tanh(d / zeta)).

All arrays use the reference's Fortran layout indexed [i, j, k] = (y, x, z).
"""
from __future__ import annotations

import math

import numpy as np

ZETA_CFG = math.sqrt(2.0) * 1.5  # psi width of the synthetic workloads


def spheres(shape, seed: int, solid_fraction: float = 0.6, rmin: float = 4.0,
            rmax: float = 10.0) -> np.ndarray:
    """Boolean solid mask (interior shape) of overlapping random spheres."""
    ny, nx, nz = shape
    rng = np.random.default_rng(seed)
    solid = np.zeros(shape, dtype=bool, order="F")
    target = int(round(solid_fraction * solid.size))
    count = 0
    while count < target:
        cy, cx, cz = rng.uniform(0, ny), rng.uniform(0, nx), rng.uniform(0, nz)
        r = rng.uniform(rmin, rmax)
        y0, y1 = max(int(cy - r), 0), min(int(cy + r) + 2, ny)
        x0, x1 = max(int(cx - r), 0), min(int(cx + r) + 2, nx)
        z0, z1 = max(int(cz - r), 0), min(int(cz + r) + 2, nz)
        if y0 >= y1 or x0 >= x1 or z0 >= z1:
            continue
        yy = (np.arange(y0, y1) + 0.5 - cy)[:, None, None]
        xx = (np.arange(x0, x1) + 0.5 - cx)[None, :, None]
        zz = (np.arange(z0, z1) + 0.5 - cz)[None, None, :]
        ball = (yy * yy + xx * xx + zz * zz) <= r * r
        sub = solid[y0:y1, x0:x1, z0:z1]
        count += int(np.count_nonzero(ball & ~sub))
        sub |= ball
    return solid


def carve_tunnel(solid: np.ndarray, seed: int, radius: float = 6.0) -> np.ndarray:
    """Removes an infinite cylinder of the given radius around a random
    axis through a random point of the box (returns a new mask)."""
    rng = np.random.default_rng(seed + 7919)
    ny, nx, nz = solid.shape
    p0 = rng.uniform(0, 1, 3) * np.array([ny, nx, nz])
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    out = solid.copy(order="F")
    yy = np.arange(ny)[:, None] + 0.5 - p0[0]
    xx = np.arange(nx)[None, :] + 0.5 - p0[1]
    for k in range(nz):
        zz = k + 0.5 - p0[2]
        dot = yy * d[0] + xx * d[1] + zz * d[2]
        r2 = yy * yy + xx * xx + zz * zz - dot * dot
        out[:, :, k] &= ~(r2 < radius * radius)
    return out


def sign_field(solid: np.ndarray) -> np.ndarray:
    """Halo-padded sign field: +1 in the solid, -1 outside, ghosts copied
    from the nearest interior cell (LevelSet_3D.f90:122, :140-144)."""
    ds = np.pad(solid.astype(np.float64), 1, mode="edge")
    return np.asfortranarray(np.where(ds > 0.5, 1.0, -1.0))


def psi_from_distance(d: np.ndarray, zeta: float = ZETA_CFG) -> np.ndarray:
    """psi = 0.5(1 + tanh(d/zeta)) clamped to [0, 1] (SBMES:155-161)."""
    return np.asfortranarray(np.clip(0.5 * (1.0 + np.tanh(d / zeta)), 0.0, 1.0))


def microstructure(shape, seed: int, solid_fraction: float = 0.6, tunnel: bool = False,
                   reinit_steps: int = 175, zeta: float = ZETA_CFG, redist=None) -> dict:
    """Solid mask, signed distance (halo-padded, from reinitialisation on the
    GPU unless another ``redist(lit, sg, f, dt)`` is given) and psi
    (halo-padded) of one seeded microstructure."""
    if redist is None:
        from .sbm import redist3d_xyz as redist

    solid = spheres(shape, seed, solid_fraction)
    if tunnel:
        solid = carve_tunnel(solid, seed)
    sg = sign_field(solid)
    d = redist(reinit_steps, sg, np.zeros_like(sg), 1.0e-1)
    return dict(solid=solid, sg=sg, dist=d, psi=psi_from_distance(d, zeta), seed=seed,
                solid_fraction=float(solid.mean()))


def potential_problem(psi: np.ndarray, k_solid: float = 1.0, k_elec: float = 0.1,
                      phi_lo: float = 0.0, phi_hi: float = 1.0) -> dict:
    """The plain SBM potential solve: node conductivity psi*k_s + (1-psi)*k_e
    (halo-padded), zero right-hand side, Dirichlet phi_lo on the x = 0 ghost
    plane and phi_hi on x = nx+1, Neumann elsewhere."""
    coef = np.asfortranarray(psi * k_solid + (1.0 - psi) * k_elec)
    x = np.zeros_like(coef, order="F")
    x[:, 0, :] = phi_lo
    x[:, -1, :] = phi_hi
    rhs = np.zeros_like(coef, order="F")
    return dict(coef=coef, x=x, rhs=rhs, weight=np.asfortranarray(psi.copy()))


CONC_SCALE = 0.1  # dt D / dx^2 of the synthetic concentration solve


def concentration_problem(psi: np.ndarray, seed: int = 0) -> dict:
    """An implicit concentration step in the CnE form of the reference
    (SBMES:515-521): psE c - s div(psE grad c) = psE c_old, psE = 1 - psi +
    1e-6 (its floor, SBMES:258), face coefficients from psE, s = CONC_SCALE,
    Neumann on every face; c_old = 1 + 0.1 x smoothed noise, also the
    initial guess.  Fields for OP_GENERIC_DIAG: coef, diag, rhs, x, weight."""
    from scipy.ndimage import gaussian_filter

    pse = np.asfortranarray(1.0 - psi + 1.0e-6)
    rng = np.random.default_rng(seed + 7)
    c0 = 1.0 + 0.1 * gaussian_filter(rng.standard_normal(psi.shape), 2.0, mode="nearest")
    c0 = np.asfortranarray(c0)
    return dict(coef=pse.copy(order="F"), diag=pse, rhs=np.asfortranarray(pse * c0), x=c0,
                weight=pse.copy(order="F"), scale=CONC_SCALE)


def reference_tables(params):
    """Fills the five 101-point property tables of the reference
    (C_Li_X / M6 / Mb5 / J2 / O3, SBMES:210-242, not in its repository) with
    smooth synthetic curves of plausible magnitude: chemical potential,
    mobility (already scaled as SBMES:242 does), exchange current and
    open-circuit voltage against the Li fraction on [0, 1]."""
    x = np.arange(101) * 0.01
    params.set_table("tbl_x", x)
    params.set_table("tbl_mu", 0.05 * (2.0 * x - 1.0) + 0.02 * np.sin(6.0 * np.pi * x))
    params.set_table("tbl_mb", 1.0e-9 * (1.0 + x))
    params.set_table("tbl_i0", 1.0 + 0.5 * x * (1.0 - x))
    params.set_table("tbl_ocv", 0.2 - 0.1 * x)
    return params


def full_step_params(params):
    """The 128^3 full-electrochemical-step workload: Cahn-Hilliard with the
    analytic double well of height W = 1, gradient coefficient kappa = 1
    voxel^2 and mobility M = 1 voxel^2 per unit time -- in the reference's
    physical grid spacing dx that is eps = dx^2 and a mobility table of dx^2,
    so the update equals the voxel-unit one -- and Butler-Volmer linearised
    in the potential jump with a uniform exchange current i0 = i0_scale =
    1e-3 (a table of ones) and zero open-circuit voltage; everything else
    (dx, the potentials, CnE) as the reference."""
    from .sbm import BV_LINEAR, CH_DOUBLE_WELL

    x = np.arange(101) * 0.01
    dx2 = params.dx * params.dx
    params.eps = dx2
    params.ch_mode = CH_DOUBLE_WELL
    params.ch_w = 1.0
    params.bv_mode = BV_LINEAR
    params.i0_scale = 1.0e-3
    params.set_table("tbl_x", x)
    params.set_table("tbl_mu", np.zeros(101))
    params.set_table("tbl_mb", np.full(101, dx2))
    params.set_table("tbl_i0", np.ones(101))
    params.set_table("tbl_ocv", np.zeros(101))
    return params


def full_step_concentration(shape, seed: int) -> np.ndarray:
    """Halo-padded initial particle concentration 0.5 + U(-0.01, 0.01),
    ghosts copied from the nearest interior cell."""
    rng = np.random.default_rng(seed + 104729)
    c = 0.5 + rng.uniform(-0.01, 0.01, size=shape)
    return np.asfortranarray(np.pad(c, 1, mode="edge"))


FULL_STEP_DT = 1.0e-3


def step_schedule(xrf: float, dcrnt: float, trgi: float):
    """dt and voltage-scan rate of one time step as the reference's time
    loop chooses them (SBMES:360-383); all literals REAL(4) as there."""
    f = lambda v: float(np.float32(v))
    vsr0 = 1.0e-2 * 1.0e1 / f(3.25 ** 2) * f(2.5)
    if dcrnt < f(0.07) * abs(trgi):
        vsr = vsr0 * f(0.5)
    elif dcrnt < f(0.20) * abs(trgi):
        vsr = vsr0
    elif dcrnt < f(0.40) * abs(trgi):
        vsr = vsr0 * f(3.0)
    elif dcrnt < f(0.75) * abs(trgi):
        vsr = vsr0 * f(5.0)
    else:
        vsr = vsr0 * f(8.0)
    base = np.float32(np.float32(1.05625e-02) * np.float32(0.125))
    if xrf < f(0.12):
        dt = float(np.float32(base * np.float32(0.75)))
        vsr = vsr * 2
    elif xrf < f(0.20):
        dt = float(np.float32(base * np.float32(0.5)))
        vsr = vsr * 10
    else:
        dt = float(np.float32(base * np.float32(0.5)))
        vsr = vsr * 15
    return dt, vsr
