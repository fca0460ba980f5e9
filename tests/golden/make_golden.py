"""Generates the golden fixtures of tests/golden/ from an independent NumPy
restatement of the reference Fortran (AffanMalik90/Elsim, src/frtrn/).

The reference ships no tests, golden vectors or fixtures and cannot be
compiled here (no Fortran compiler, no MPI), so these vectors come from a
second restatement written in NumPy array syntax -- which maps one for one
onto the Fortran array statements and WHERE blocks -- and independently of
the C oracle (oracle/sbm_oracle.c).  tests/test_oracle_golden.py checks the
oracle against them: bit for bit where the arithmetic is free of
transcendental library calls and reductions, within a few ulp otherwise.

Each NumPy operation is a single IEEE-754 double operation (no fused
multiply-add), and expressions keep the Fortran evaluation order.  REAL(4)
literals are promoted from float32 exactly as gfortran promotes them.

Run:  python tests/golden/make_golden.py   (writes tests/golden/*.npz)
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
f4 = lambda v: float(np.float32(v))  # REAL(4) literal promoted to REAL(8)


# ---------------------------------------------------------------- helpers
def nogrdbc(f):
    """NoGrdBc3D, LevelSet_3D.f90:164-190 (f indexed [i, j, k], halo 0/n+1)."""
    f[0, 1:-1, 1:-1] = f[1, 1:-1, 1:-1]
    f[-1, 1:-1, 1:-1] = f[-2, 1:-1, 1:-1]
    f[:, 0, 1:-1] = f[:, 1, 1:-1]
    f[:, -1, 1:-1] = f[:, -2, 1:-1]
    f[:, :, 0] = f[:, :, 1]
    f[:, :, -1] = f[:, :, -2]
    return f


def allen_cahn(d, iters):
    """LevelSet_3D.f90:116-136 in array syntax: NoGrdBc3D, then per step
    sgF = 2*d*(1.0-d)*(1.0-2*d) - 0.64*(neighbours - 6*d), d = d - 0.05*sgF,
    NoGrdBc3D (0.64, 0.05 REAL(4))."""
    d = nogrdbc(d.copy())
    I = slice(1, -1)
    for _ in range(iters):
        c = d[I, I, I]
        nb = d[2:, I, I] + d[:-2, I, I] + d[I, 2:, I] + d[I, :-2, I] + d[I, I, 2:] + d[I, I, :-2] - 6 * c
        sg = 2 * c * (1.0 - c) * (1.0 - 2 * c) - f4(0.64) * nb
        d[I, I, I] = c - f4(0.05) * sg
        nogrdbc(d)
    return d


def absgrd(sg, f):
    """AbsGrd3DUW_XYZ, LevelSet_3D.f90:289-320, interior result."""
    c = f[1:-1, 1:-1, 1:-1]
    ag = c - f[:-2, 1:-1, 1:-1]
    bg = f[2:, 1:-1, 1:-1] - c
    cg = c - f[1:-1, :-2, 1:-1]
    dg = f[1:-1, 2:, 1:-1] - c
    eg = c - f[1:-1, 1:-1, :-2]
    fg = f[1:-1, 1:-1, 2:] - c
    mx = np.maximum
    sq = lambda a: a * a
    gp = np.sqrt((mx(sq(mx(ag, 0.0)), sq(mx(-bg, 0.0))) + mx(sq(mx(cg, 0.0)), sq(mx(-dg, 0.0))))
                 + mx(sq(mx(eg, 0.0)), sq(mx(-fg, 0.0))))
    gn = np.sqrt((mx(sq(mx(-ag, 0.0)), sq(mx(bg, 0.0))) + mx(sq(mx(-cg, 0.0)), sq(mx(dg, 0.0))))
                 + mx(sq(mx(-eg, 0.0)), sq(mx(fg, 0.0))))
    s = sg[1:-1, 1:-1, 1:-1]
    return np.where(s == 0.0, 0.0, np.where(s > 0.0, gp, gn))


def redist(lit, dt, sg, f):
    """ReDist3D_XYZ, LevelSet_3D.f90:226-259."""
    f = f.copy()
    gf = np.zeros_like(f)
    for _ in range(lit):
        gf[1:-1, 1:-1, 1:-1] = absgrd(sg, f)
        nogrdbc(gf)
        nf = f + (sg * (1.0 - gf)) * dt
        bad = ~(nf * f > 0.0)
        nf[bad] = f[bad] + (dt * 1.0e-7) * sg[bad]
        f = nf
    return f


def accdiff(psi, cn, term, dirichlet_x):
    """AccDiff_3D.f90:111-169 (dirichlet_x=1) / :185-243 (dirichlet_x=0)."""
    cn = cn.copy()
    dt = float(np.float32(np.float32(1.25e-1) * np.float32(0.5)))
    idh2 = 1.0 / (1.0 ** 2)
    thr, cmin = f4(4.0e-1), f4(1.0e-4)
    div = np.zeros(tuple(s - 2 for s in psi.shape))
    P = psi[1:-1, 1:-1, 1:-1]
    mask = P >= thr
    for it in range(2, term + 1):
        C = cn[1:-1, 1:-1, 1:-1]
        t = (psi[2:, 1:-1, 1:-1] + P) * (cn[2:, 1:-1, 1:-1] - C)
        t = t - (P + psi[:-2, 1:-1, 1:-1]) * (C - cn[:-2, 1:-1, 1:-1])
        t = t + (psi[1:-1, 2:, 1:-1] + P) * (cn[1:-1, 2:, 1:-1] - C)
        t = t - (P + psi[1:-1, :-2, 1:-1]) * (C - cn[1:-1, :-2, 1:-1])
        t = t + (psi[1:-1, 1:-1, 2:] + P) * (cn[1:-1, 1:-1, 2:] - C)
        t = t - (P + psi[1:-1, 1:-1, :-2]) * (C - cn[1:-1, 1:-1, :-2])
        d = ((0.5 * idh2) / P) * t
        div[mask] = d[mask]
        C[mask] = C[mask] + dt * div[mask]
        if it % 5 == 1:
            C[(C > cmin) & (P > thr)] = 1.0
        cn[0, 1:-1, 1:-1] = cn[1, 1:-1, 1:-1]
        cn[-1, 1:-1, 1:-1] = cn[-2, 1:-1, 1:-1]
        if dirichlet_x:
            cn[:, 0, 1:-1] = cn[:, 1, 1:-1]
            cn[:, -1, 1:-1] = 1.0
        else:
            cn[:, 0, 1:-1] = 1.0
            cn[:, -1, 1:-1] = cn[:, -2, 1:-1]
        cn[:, :, 0] = cn[:, :, 1]
        cn[:, :, -1] = cn[:, :, -2]
    return cn


def table(cord, vals, cn):
    """Tbl_Chk_Pln_3DA, SBMES:998-1026 (1-based lb restated 0-based)."""
    t = cn.copy()
    t[t < 0.0] = 1.0e-6
    t[t > 1.0] = 1.0
    ditv = cord[1] - cord[0]
    lb = np.floor(t / ditv).astype(np.int64)
    sz = cord.size
    lb[lb == 0] = 1
    lb[lb == sz] = sz - 1
    lb = np.minimum(lb, sz - 1)
    return vals[lb - 1] + ((t - cord[lb - 1]) / ditv) * (vals[lb] - vals[lb - 1])


def faces(K):
    """The six face arrays (K_nb + K_c)*0.5 of SBMES:326-331, order 1..6 =
    y-, y+, x-, x+, z-, z+."""
    c = K[1:-1, 1:-1, 1:-1]
    return [(K[:-2, 1:-1, 1:-1] + c) * 0.5, (K[2:, 1:-1, 1:-1] + c) * 0.5,
            (K[1:-1, :-2, 1:-1] + c) * 0.5, (K[1:-1, 2:, 1:-1] + c) * 0.5,
            (K[1:-1, 1:-1, :-2] + c) * 0.5, (K[1:-1, 1:-1, 2:] + c) * 0.5]


def S(pk, P):
    """Flux sum of SBMES:516-521 with face arrays pk (1-based pk(...,n) = pk[n-1])."""
    C = P[1:-1, 1:-1, 1:-1]
    t = pk[1] * (P[2:, 1:-1, 1:-1] - C)
    t = t - pk[0] * (C - P[:-2, 1:-1, 1:-1])
    t = t + pk[3] * (P[1:-1, 2:, 1:-1] - C)
    t = t - pk[2] * (C - P[1:-1, :-2, 1:-1])
    t = t + pk[5] * (P[1:-1, 1:-1, 2:] - C)
    t = t - pk[4] * (C - P[1:-1, 1:-1, :-2])
    return t


def apply_cne(psE, pce, P, dt, dx):
    """WMX of SBMES:515-521."""
    return psE[1:-1, 1:-1, 1:-1] * P[1:-1, 1:-1, 1:-1] - dt / dx ** 2 * S(faces(pce), P)


def apply_php(kap, P, dx):
    """WMX of SBMES:670-676."""
    return 1.0 / dx ** 2 * S(faces(kap), P)


def avp(psP, psE, dx):
    """SBMES:274-291."""
    def grad(p):
        a = (p[2:, 1:-1, 1:-1] - p[:-2, 1:-1, 1:-1]) / 2
        b = (p[1:-1, 2:, 1:-1] - p[1:-1, :-2, 1:-1]) / 2
        e = (p[1:-1, 1:-1, 2:] - p[1:-1, 1:-1, :-2]) / 2
        return np.sqrt(a ** 2 + b ** 2 + e ** 2)
    v = np.sqrt(grad(psP) * grad(psE))
    v[v < 1.0e-2] = 0.0
    return v, v / dx


def ch_update(cnp, psP, mb_tbl, mu_tbl, cord, rxn, avpx, dt, dx, eps, rho):
    """Cahn-Hilliard block SBMES:398-438 for one rank owning the grid."""
    C = cnp[1:-1, 1:-1, 1:-1]
    lap = (cnp[1:-1, :-2, 1:-1] - 2 * C + cnp[1:-1, 2:, 1:-1] + cnp[:-2, 1:-1, 1:-1] - 2 * C
           + cnp[2:, 1:-1, 1:-1] + cnp[1:-1, 1:-1, :-2] - 2 * C + cnp[1:-1, 1:-1, 2:]) / dx ** 2
    mu = np.zeros_like(cnp)
    mb = np.zeros_like(cnp)
    mu[1:-1, 1:-1, 1:-1] = table(cord, mu_tbl, C)
    mb[1:-1, 1:-1, 1:-1] = table(cord, mb_tbl, C)
    edge = lambda f: (nogrdbc(f))
    edge(mb)
    mu[1:-1, 1:-1, 1:-1] = mu[1:-1, 1:-1, 1:-1] - eps * lap
    edge(mu)
    pm = psP * mb
    M = mu[1:-1, 1:-1, 1:-1]
    Pc = pm[1:-1, 1:-1, 1:-1]
    t = 0.5 * (pm[2:, 1:-1, 1:-1] + Pc) * (mu[2:, 1:-1, 1:-1] - M)
    t = t - 0.5 * (Pc + pm[:-2, 1:-1, 1:-1]) * (M - mu[:-2, 1:-1, 1:-1])
    t = t + 1.0 * 0.5 * (pm[1:-1, 2:, 1:-1] + Pc) * (mu[1:-1, 2:, 1:-1] - M)
    t = t - 1.0 * 0.5 * (Pc + pm[1:-1, :-2, 1:-1]) * (M - mu[1:-1, :-2, 1:-1])
    t = t + 0.5 * (pm[1:-1, 1:-1, 2:] + Pc) * (mu[1:-1, 1:-1, 2:] - M)
    t = t - 0.5 * (Pc + pm[1:-1, 1:-1, :-2]) * (M - mu[1:-1, 1:-1, :-2])
    dvc = t / dx ** 2
    ps = psP[1:-1, 1:-1, 1:-1]
    out = cnp.copy()
    o = out[1:-1, 1:-1, 1:-1]
    msk = ps > 1.0e-5
    o[msk] = C[msk] + dt * (dvc[msk] + (rxn[msk] / rho) * avpx[msk]) / ps[msk]
    nogrdbc(out)
    return out


def main():
    rng = np.random.default_rng(20240601)
    out = {}
    # level set: sign field of a few blobs
    ny, nx, nz = 11, 13, 9
    yy, xx, zz = np.meshgrid(np.arange(ny + 2), np.arange(nx + 2), np.arange(nz + 2), indexing="ij")
    blob = ((yy - 4.2) ** 2 + (xx - 5.1) ** 2 + (zz - 3.3) ** 2 < 10) | (
        (yy - 8.7) ** 2 + (xx - 10.2) ** 2 + (zz - 6.5) ** 2 < 6)
    sg = np.where(blob, 1.0, -1.0)
    out["redist_sg"] = sg
    out["redist_out_d"] = redist(9, 1.0e-1, sg, np.zeros_like(sg))
    out["redist_out_f"] = redist(9, f4(1.0e-1), sg, np.zeros_like(sg))
    # AccDiff: psi from a smooth random field, ghosts Neumann
    d = rng.normal(size=(ny, nx, nz)) * 2.0
    psi = np.zeros((ny + 2, nx + 2, nz + 2))
    psi[1:-1, 1:-1, 1:-1] = 0.5 * (1.0 + np.tanh(d / 0.75))
    nogrdbc(psi)
    out["acc_psi"] = psi
    out["acc_solid"] = accdiff(psi, np.zeros_like(psi), 23, 1)
    pe = psi.copy()
    pe[1:-1, 1:-1, 1:-1] = 1.0 - pe[1:-1, 1:-1, 1:-1]
    out["acc_psi_e"] = pe
    out["acc_elec"] = accdiff(pe, np.zeros_like(pe), 23, 0)
    # tables
    cord = np.arange(101) * 0.01
    vals = np.cumsum(rng.normal(size=101))
    cn = np.concatenate([rng.uniform(-0.1, 1.1, 3000), cord, [0.0, 1.0, 1e-6, 0.005, 0.995]])
    out["tbl_cord"], out["tbl_vals"], out["tbl_cn"] = cord, vals, cn
    out["tbl_out"] = table(cord, vals, cn)
    # operators (phP and CnE forms) with random node coefficients
    K = rng.uniform(0.1, 3.3, (ny + 2, nx + 2, nz + 2))
    P = rng.normal(size=(ny + 2, nx + 2, nz + 2))
    psE = rng.uniform(1e-6, 1.0, (ny + 2, nx + 2, nz + 2))
    dx, dt = 3.25e-5 * 0.5, float(np.float32(np.float32(1.05625e-02) * np.float32(0.125)) * np.float32(0.75))
    out["op_K"], out["op_P"], out["op_psE"] = K, P, psE
    out["op_php"] = apply_php(K, P, dx)
    out["op_cne"] = apply_cne(psE, K * psE, P, dt, dx)
    out["op_dx"], out["op_dt"] = np.array(dx), np.array(dt)
    # interface measure
    psP = np.clip(psi + 1e-7, 0, 1.1)
    av, avx = avp(psP, pe + 1e-6, dx)
    out["avp_psP"], out["avp_psE"], out["avp"], out["avpx"] = psP, pe + 1e-6, av, avx
    # Cahn-Hilliard block
    cnp = rng.uniform(0.0, 1.0, (ny + 2, nx + 2, nz + 2))
    nogrdbc(cnp)
    mu_t = np.sin(cord * 3.0)
    mb_t = 1.0 + cord
    rxn = rng.normal(size=(ny, nx, nz)) * 1e-6
    avpx = rng.uniform(0, 1.0 / dx, (ny, nx, nz))
    ch = ch_update(cnp, psP, mb_t, mu_t, cord, rxn, avpx, dt, dx, 6.76e-10, f4(0.0312))
    out.update(ch_cnp=cnp, ch_psP=psP, ch_mu_t=mu_t, ch_mb_t=mb_t, ch_rxn=rxn, ch_avpx=avpx,
               ch_out=ch)
    # Allen-Cahn pre-smoothing of a noisy 0/1 voxel field (ghosts arbitrary)
    vox = (rng.uniform(size=(ny + 2, nx + 2, nz + 2)) < 0.55).astype(np.float64)
    vox += rng.normal(size=vox.shape) * 0.05
    out["ac_in"] = vox
    out["ac_out"] = allen_cahn(vox, 17)
    np.savez_compressed(HERE / "golden_v1.npz", **out)
    print("wrote", HERE / "golden_v1.npz", sorted(out))


if __name__ == "__main__":
    main()
