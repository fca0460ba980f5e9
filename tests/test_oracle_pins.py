"""Analytic known-answer tests of the C oracle (CPU only).

The reference ships no test vectors; besides its own results run by the
Fortran-subset interpreter (tests/test_oracle_reference.py), the restatement
is pinned here by cases whose answer is known in closed form or by an
independent direct solver.
"""
import numpy as np
import pytest

from elsim_gb300 import sbm
from oracle import sbm_oracle as orc


def _pad(shape):
    return np.zeros(tuple(s + 2 for s in shape), order="F")


def test_uniform_laplace_is_linear_between_dirichlet_planes():
    ny, nx, nz = 6, 17, 5
    K = _pad((ny, nx, nz)) + 1.0
    x = _pad((ny, nx, nz))
    x[:, -1, :] = 1.0  # phi = 1 on the x = nx+1 ghost plane, 0 on x = 0
    sol, info = orc.cg(K, np.zeros_like(K), x, 1.0, sbm.BC_ZERO, sbm.BC_ZERO, sbm.STOP_REL_RES,
                       1e-14, 1000)
    assert info["status"] == 0
    exact = np.arange(1, nx + 1) / (nx + 1)
    got = sol[1:-1, 1:-1, 1:-1]
    assert np.abs(got - exact[None, :, None]).max() < 1e-12


def _homog(p, bc0, bc1):
    p = np.asfortranarray(p.copy())
    ny, nx, nz = (s - 2 for s in p.shape)
    orc.lib().orc_bc_yz(ny, nx, nz, orc._p(p))
    orc.lib().orc_bc_x(ny, nx, nz, orc._p(p), 0, nz + 1, bc0, 0.0, bc1, 0.0)
    return p


@pytest.mark.parametrize("bc", [(0, 1), (1, 0), (1, 1), (0, 0)])
@pytest.mark.parametrize("diag", [False, True])
def test_operator_is_symmetric(bc, diag):
    rng = np.random.default_rng(1)
    shp = (7, 9, 6)
    K = np.asfortranarray(rng.uniform(0.1, 2.0, tuple(s + 2 for s in shp)))
    dg = np.asfortranarray(rng.uniform(0.5, 1.0, K.shape)) if diag else None
    a = _homog(rng.normal(size=K.shape), *bc)
    b = _homog(rng.normal(size=K.shape), *bc)
    Aa = orc.apply(K, a, 0.7, diag=dg)
    Ab = orc.apply(K, b, 0.7, diag=dg)
    i = (slice(1, -1),) * 3
    lhs, rhs = float((Aa[i] * b[i]).sum()), float((a[i] * Ab[i]).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
    # the phP form is negative semi-definite, the CnE form positive definite
    aa = float((Aa[i] * a[i]).sum())
    assert (aa > 0) if diag else (aa < 0)


def test_cg_matches_direct_solve():
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    rng = np.random.default_rng(4)
    shp = (5, 6, 4)
    n = int(np.prod(shp))
    K = np.asfortranarray(rng.uniform(0.2, 2.0, tuple(s + 2 for s in shp)))
    rhs = np.asfortranarray(rng.normal(size=K.shape))
    x0 = _pad(shp)
    x0[:, 0, :] = 0.3
    x0[:, -1, :] = -0.2
    sol, info = orc.cg(K, rhs, x0, 1.0, sbm.BC_ZERO, sbm.BC_ZERO, sbm.STOP_REL_RES, 1e-14, 5000)
    # assemble A (homogeneous) column by column and the boundary contribution
    cols = []
    for c in range(n):
        e = np.zeros(shp)
        e.flat[c] = 1.0
        p = _pad(shp)
        p[1:-1, 1:-1, 1:-1] = e
        cols.append(orc.apply(K, _homog(p, 1, 1), 1.0)[1:-1, 1:-1, 1:-1].ravel())
    A = sp.csr_matrix(np.array(cols).T)
    b = orc.residual(K, rhs, x0, 1.0)[1:-1, 1:-1, 1:-1].ravel()
    d = spl.spsolve(A.tocsc(), b)
    assert np.abs(sol[1:-1, 1:-1, 1:-1].ravel() - d).max() < 1e-10


def test_redistancing_recovers_planar_distance():
    ny, nx, nz = 4, 40, 4
    sg = np.full((ny + 2, nx + 2, nz + 2), -1.0, order="F")
    sg[:, :21, :] = 1.0  # solid for x index <= 20: interface between 20 and 21
    f = orc.redist(175, sg, np.zeros_like(sg), 1.0e-1)
    prof = f[2, 1:-1, 2]
    # the cells next to the interface sit at exactly +-0.5, the profile is
    # antisymmetric, and |grad f| -> 1 near the interface (the first-order
    # upwind front is still converging farther out)
    assert abs(prof[19] - 0.5) < 1e-12 and abs(prof[20] + 0.5) < 1e-12
    assert np.array_equal(prof, -prof[::-1])
    diffs = np.diff(prof)
    assert np.allclose(diffs[15:24], -1.0, atol=1e-4)
    assert (diffs < 0).all()


def test_accdiff_labels_connected_and_isolated_regions():
    ny, nx, nz = 12, 30, 12
    psi = _pad((ny, nx, nz))
    psi[:, 21:, :] = 1.0          # slab touching the Dirichlet face x = nx+1
    yy, xx, zz = np.meshgrid(np.arange(ny + 2), np.arange(nx + 2), np.arange(nz + 2),
                             indexing="ij")
    ball = (yy - 6) ** 2 + (xx - 8) ** 2 + (zz - 6) ** 2 <= 9
    psi[ball] = 1.0               # isolated particle
    cn = orc.accdiff(psi, np.zeros_like(psi), 1501, 1)
    assert (cn[1:-1, 21:-1, 1:-1] > 1e-4).all()
    assert (cn[ball] == 0.0).all()
    # electrolyte phase: the gap region connects to x = 0
    pe = psi.copy()
    pe[1:-1, 1:-1, 1:-1] = 1.0 - pe[1:-1, 1:-1, 1:-1]
    ce = orc.accdiff(pe, np.zeros_like(pe), 1501, 0)
    assert (ce[1:-1, 1:5, 1:-1] > 1e-4).all()


def test_rm_mask_thresholds_at_real4_literal():
    thr = float(np.float32(1e-4))
    cn = np.array([thr, np.nextafter(thr, 0), 0.0, 1.0, 1e-4])
    out = orc.rm_mask(np.ones(5), cn)
    assert out.tolist() == [1.0, 0.0, 0.0, 1.0, 0.0 if 1e-4 < thr else 1.0]


def test_table_of_linear_function_is_exact():
    cord = np.arange(101) * 0.01
    vals = 2.0 * cord + 0.5
    c = np.linspace(0.0, 1.0, 997)
    assert np.allclose(orc.table(cord, vals, c), 2.0 * c + 0.5, rtol=0, atol=1e-13)
    # clamps: below 0 -> 1e-6, above 1 -> 1
    assert np.allclose(orc.table(cord, vals, np.array([-5.0, 7.0])), [0.5 + 2e-6, 2.5])


def test_allen_cahn_fixed_points_and_direction():
    """LevelSet_3D.f90:116-136: 0, 1/2 and 1 are fixed points of the double
    well (constant fields do not move, the Laplacian of a constant is 0);
    values below 1/2 move toward 0, above toward 1; the ghosts end as
    zero-gradient copies."""
    for v in (0.0, 0.5, 1.0):
        f = np.full((6, 7, 5), v)
        assert np.array_equal(orc.allen_cahn(30, f), f)
    f = np.full((6, 7, 22), 0.4)
    f[:, :, 11:] = 0.6  # two thick slabs: each relaxes toward its well
    g = orc.allen_cahn(40, f)
    assert g[3, 3, 1] < 0.1 and g[3, 3, -2] > 0.9
    assert np.all(np.diff(g[3, 3, 1:-1]) >= 0)  # a monotone interface between them
    assert np.array_equal(g[0], g[1]) and np.array_equal(g[:, -1], g[:, -2])
    assert np.array_equal(g[:, :, 0], g[:, :, 1])



def test_double_well_cahn_hilliard_pin():
    """The double-well chemical potential of the full-step workload:
    mu = W*2c(1-c)(1-2c) - eps*Lap c, restated in NumPy, against the oracle's
    Cahn-Hilliard update on a random field with psP = 1 and no reaction."""
    from elsim_gb300 import sbm, synth
    from oracle import sbm_oracle as orc
    shape = (9, 7, 6)
    p = synth.full_step_params(orc.params_reference())
    p.ch_w = 1.7
    st = orc.State(*shape, p)
    rng = np.random.default_rng(3)
    dist = rng.uniform(2.0, 3.0, size=shape).astype(np.float32)
    st.setup_domain(dist, -dist)
    c = np.pad(rng.uniform(0.3, 0.7, size=shape), 1, mode="edge")
    st.set_field(sbm.F_CNP, np.asfortranarray(c))
    psp = st.field(sbm.F_PSP)
    st.set_field(sbm.F_RXN, np.zeros_like(c, order="F"))
    dt = 1e-3
    st.ch_step(dt)
    got = st.field(sbm.F_CNP)[1:-1, 1:-1, 1:-1]
    dx2 = p.dx * p.dx

    def lap(u):
        return ((u[2:, 1:-1, 1:-1] + u[:-2, 1:-1, 1:-1] + u[1:-1, 2:, 1:-1] + u[1:-1, :-2, 1:-1]
                 + u[1:-1, 1:-1, 2:] + u[1:-1, 1:-1, :-2] - 6 * u[1:-1, 1:-1, 1:-1]) / dx2)

    ci = c[1:-1, 1:-1, 1:-1]
    mu = np.pad(1.7 * 2 * ci * (1 - ci) * (1 - 2 * ci) - p.eps * lap(c), 1, mode="edge")
    pm = np.pad(psp[1:-1, 1:-1, 1:-1] * dx2, 1, mode="edge")
    m0 = mu[1:-1, 1:-1, 1:-1]
    p0 = pm[1:-1, 1:-1, 1:-1]
    dvc = np.zeros_like(ci)
    for sl in ((slice(2, None), slice(1, -1), slice(1, -1)), (slice(None, -2), slice(1, -1), slice(1, -1)),
               (slice(1, -1), slice(2, None), slice(1, -1)), (slice(1, -1), slice(None, -2), slice(1, -1)),
               (slice(1, -1), slice(1, -1), slice(2, None)), (slice(1, -1), slice(1, -1), slice(None, -2))):
        dvc += 0.5 * (pm[sl] + p0) * (mu[sl] - m0)
    want = ci + dt * (dvc / dx2) / psp[1:-1, 1:-1, 1:-1]
    assert np.allclose(got, want, rtol=1e-12, atol=1e-14)
    assert not np.allclose(got, ci, rtol=0, atol=1e-9)  # the step did move c


def test_cg_error_energy_decreases_monotonically():
    """CG on a small SPD system (the CnE form, diagonal + scaled diffusion,
    Neumann faces): the energy norm of the error, e.A e, must fall with every
    further iteration -- the defining property of CG."""
    rng = np.random.default_rng(7)
    shp = (6, 5, 4)
    K = np.asfortranarray(rng.uniform(0.2, 2.0, tuple(s + 2 for s in shp)))
    dg = np.asfortranarray(rng.uniform(0.5, 1.5, K.shape))
    rhs = np.asfortranarray(rng.normal(size=K.shape))
    x0 = _pad(shp)
    i = (slice(1, -1),) * 3
    xs, _ = orc.cg(K, rhs, x0, 0.3, sbm.BC_COPY, sbm.BC_COPY, sbm.STOP_REL_RES, 1e-15, 5000,
                   diag=dg)
    energies = []
    for m in range(1, 16):
        xm, _ = orc.cg(K, rhs, x0, 0.3, sbm.BC_COPY, sbm.BC_COPY, sbm.STOP_REL_RES, 0.0, m,
                       diag=dg)
        e = _pad(shp)
        e[i] = xm[i] - xs[i]
        e = _homog(e, 0, 0)
        energies.append(float((orc.apply(K, e, 0.3, diag=dg)[i] * e[i]).sum()))
    assert all(a > 0 for a in energies)
    assert all(b < a for a, b in zip(energies, energies[1:])), energies
