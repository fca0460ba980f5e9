"""GPU parity of the SBM operator and CG solvers against the oracle.

FP64 CG (the drop-in) must reproduce the oracle's iteration count (within a
few iterations: the sums are tree- rather than sequentially ordered) and its
solution to rel-L2 <= 1e-9; the mixed-precision solver must reach the same
FP64 true residual and match the FP64 oracle solution to rel-L2 <= 1e-6.
"""
import numpy as np
import pytest

from conftest import interior, rel_l2
from elsim_gb300 import sbm, synth
from oracle import sbm_oracle as orc

pytestmark = pytest.mark.gpu


def _problem(shape, seed, tunnel=False):
    m = synth.microstructure(shape, seed=seed, tunnel=tunnel, reinit_steps=60, redist=orc.redist)
    return m, synth.potential_problem(m["psi"])


def _load(ctx, prob):
    for name in ("coef", "x", "rhs", "weight"):
        ctx.upload(name, prob[name])


def _true_relres(prob, x):
    xg = x.copy(order="F")
    orc.lib().orc_bc_yz(*orc.hdims(xg), orc._p(xg))
    r = orc.residual(prob["coef"], prob["rhs"], xg, 1.0)
    r0 = orc.residual(prob["coef"], prob["rhs"], prob["x"], 1.0)
    return np.linalg.norm(interior(r)) / np.linalg.norm(interior(r0))


@pytest.mark.parametrize("shape", [(32, 32, 32), (40, 27, 33), (8, 64, 5)])
def test_fp64_cg_matches_oracle(built, shape):
    m, prob = _problem(shape, 7)
    with sbm.Context(*shape) as ctx:
        _load(ctx, prob)
        info = ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0,
                            tol=1e-10, max_it=20000, stop_rule=sbm.STOP_REL_RES)
        x = ctx.download("x")
    xo, io = orc.cg(prob["coef"], prob["rhs"], prob["x"], 1.0, sbm.BC_ZERO, sbm.BC_ZERO,
                    sbm.STOP_REL_RES, 1e-10, 20000)
    assert io["status"] == 0 and info["status"] == 0
    assert abs(info["iters"] - io["iters"]) <= 3
    assert rel_l2(x, xo) < 1e-9
    assert _true_relres(prob, x) < 2e-10
    # ghosts after the solve: Dirichlet faces kept, y/z faces copy the edge
    assert np.array_equal(x[:, 0, 1:-1], prob["x"][:, 0, 1:-1])
    assert np.array_equal(x[0, 1:-1, 1:-1], x[1, 1:-1, 1:-1])


@pytest.mark.parametrize("bcs", [(sbm.BC_COPY, sbm.BC_ZERO), (sbm.BC_ZERO, sbm.BC_COPY)])
def test_reference_update_rule_matches_oracle(built, bcs):
    """The phP / phE loop: weighted update norm < tol (SBMES:699-705)."""
    shape = (24, 28, 20)
    m, prob = _problem(shape, 9)
    rng = np.random.default_rng(0)
    rhs = np.asfortranarray(rng.normal(size=prob["x"].shape) * 1e-2)
    prob["rhs"] = rhs
    w = prob["weight"] + 1e-7
    prob["weight"] = w
    wsum = float(interior(w).sum())
    with sbm.Context(*shape) as ctx:
        _load(ctx, prob)
        info = ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=bcs[0], bc_x1=bcs[1], scale=1.0, tol=1e-9,
                            max_it=30001, stop_rule=sbm.STOP_REF_UPDATE)
        x = ctx.download("x")
    xo, io = orc.cg(prob["coef"], rhs, prob["x"], 1.0, bcs[0], bcs[1], sbm.STOP_REF_UPDATE, 1e-9,
                    30001, w=w, wsum=wsum)
    assert abs(info["iters"] - io["iters"]) <= 3, (info, io)
    assert rel_l2(x, xo) < 1e-7


def test_cne_form_residual_rule_matches_oracle(built):
    """The CnE loop: q = psE p - dt/dx^2 div(pce grad p), weighted residual
    norm (SBMES:515-547), through a full electrochemical set-up."""
    shape = (20, 24, 16)
    p = orc.params_reference()
    p.crt_cne = 1e-12
    dist_p, dist_e = _distances(shape, 4)
    with sbm.Context(*shape, params=p) as ctx:
        ctx.setup_domain(dist_p, dist_e)
        st = orc.State(*shape, p)
        st.setup_domain(dist_p, dist_e)
        dt = float(np.float32(np.float32(1.05625e-02) * np.float32(0.125)) * np.float32(0.75))
        # perturb CnE so the solve has work to do
        rng = np.random.default_rng(3)
        cne = st.field(sbm.F_CNE) + rng.uniform(0, 1e-4, st.field(sbm.F_CNE).shape)
        st.set_field(sbm.F_CNE, cne)
        ctx.upload("CnE", cne)
        g = ctx.cne_step(2, dt)
        o = st.cne_step(2, dt)
        # thousands of iterations on an ill-conditioned system: tree- versus
        # plane-ordered sums shift the stopping iteration by a fraction of a percent
        assert abs(g["it_cne"] - o["it_cne"]) <= max(3, 0.01 * o["it_cne"]), (g["it_cne"], o["it_cne"])
        # psE has a 1e-6 floor in the solid, where the CnE system is nearly
        # singular and the stopping norm (weighted by psE) barely looks: there
        # two converged solves agree to ~1e-7; in the electrolyte far closer.
        got, ref = ctx.download("CnE"), st.field(sbm.F_CNE)
        assert rel_l2(got, ref) < 1e-6
        w = interior(st.field(sbm.F_PSE))
        werr = np.sqrt((w * (interior(got) - interior(ref)) ** 2).sum() / (w * interior(ref) ** 2).sum())
        assert werr < 1e-8, werr
        assert abs(g["infx"] - o["infx"]) <= 1e-12 * max(1.0, abs(o["infx"]))


def _distances(shape, seed):
    m = synth.microstructure(shape, seed=seed, reinit_steps=60, redist=orc.redist)
    d = m["dist"][1:-1, 1:-1, 1:-1]
    return d.astype(np.float32), (-d).astype(np.float32)


@pytest.mark.parametrize("precond", [sbm.PC_NONE, sbm.PC_JACOBI])
@pytest.mark.parametrize("shape", [(48, 48, 48), (44, 30, 21), (42, 36, 40)])
def test_mixed_precision_matches_fp64(built, precond, shape):
    # y extents a multiple of 4 (the four-cell double-float residual
    # kernels; 44 x 30: partial tiles in y and x) and not (the one-cell ones)
    m, prob = _problem(shape, 13, tunnel=True)
    xo, io = orc.cg(prob["coef"], prob["rhs"], prob["x"], 1.0, sbm.BC_ZERO, sbm.BC_ZERO,
                    sbm.STOP_REL_RES, 1e-12, 50000)
    with sbm.Context(*shape) as ctx:
        _load(ctx, prob)
        info = ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0,
                            tol=1e-8, max_it=50000, stop_rule=sbm.STOP_REL_RES,
                            precision=sbm.PREC_MIXED, precond=precond)
        x = ctx.download("x")
    assert info["status"] == 0
    assert _true_relres(prob, x) <= 1.05e-8
    assert rel_l2(x, xo) < 1e-6


def test_jacobi_fp64_matches(built):
    shape = (32, 30, 28)
    m, prob = _problem(shape, 17)
    xo, _ = orc.cg(prob["coef"], prob["rhs"], prob["x"], 1.0, sbm.BC_ZERO, sbm.BC_ZERO,
                   sbm.STOP_REL_RES, 1e-12, 50000)
    with sbm.Context(*shape) as ctx:
        _load(ctx, prob)
        info = ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0,
                            tol=1e-10, max_it=50000, stop_rule=sbm.STOP_REL_RES,
                            precond=sbm.PC_JACOBI)
        x = ctx.download("x")
    assert info["status"] == 0
    assert rel_l2(x, xo) < 1e-8


def test_iteration_cap_reports_maxit(built):
    shape = (16, 16, 16)
    m, prob = _problem(shape, 2)
    with sbm.Context(*shape) as ctx:
        _load(ctx, prob)
        info = ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0,
                            tol=1e-14, max_it=5, stop_rule=sbm.STOP_REL_RES,
                            raise_on_maxit=False)
    assert info["status"] == sbm.ERR_MAXIT and info["iters"] == 5
    xo, io = orc.cg(prob["coef"], prob["rhs"], prob["x"], 1.0, sbm.BC_ZERO, sbm.BC_ZERO,
                    sbm.STOP_REL_RES, 1e-14, 5)
    assert io["iters"] == 5


def test_zero_rhs_zero_boundary_converges_immediately(built):
    shape = (8, 8, 8)
    with sbm.Context(*shape) as ctx:
        ctx.upload("coef", np.ones((10, 10, 10)))
        info = ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0,
                            tol=1e-8, max_it=100, stop_rule=sbm.STOP_REL_RES)
        assert info["iters"] == 0 and info["status"] == 0
        assert not ctx.download("x").any()


def test_expired_device_wait_reports_timeout_and_the_context_recovers(built):
    """The TMA-staged stencil kernel's bounded waits: with the consumer-side
    limit at 0 every wait gives up at once (no fault, no hang: each CTA still
    waits out its own copies), the solve reports SBM_ERR_TIMEOUT, and after
    the limit is restored the same context solves normally."""
    shape = (64, 40, 24)  # ny a multiple of 4: the TMA-staged kernel runs
    m, prob = _problem(shape, 21)
    lib = sbm.load_library()
    kw = dict(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0, tol=1e-8,
              max_it=20000, stop_rule=sbm.STOP_REL_RES, precision=sbm.PREC_MIXED,
              precond=sbm.PC_JACOBI)
    with sbm.Context(*shape) as ctx:
        _load(ctx, prob)
        assert lib.sbm_set_wait_limit(0) == sbm.OK
        try:
            with pytest.raises(sbm.SbmError) as exc:
                ctx.cg_solve(**kw)
        finally:
            assert lib.sbm_set_wait_limit(-1) == sbm.OK
        assert exc.value.code == sbm.ERR_TIMEOUT
        ctx.upload("x", prob["x"])
        info = ctx.cg_solve(**kw)
        x = ctx.download("x")
    assert info["status"] == 0
    assert _true_relres(prob, x) <= 1.05e-8


@pytest.mark.parametrize("precond", [sbm.PC_JACOBI, sbm.PC_NONE])
def test_host_driven_chunks_equal_the_device_loop(built, precond):
    """The mixed solver loops its captured chunk on the device (a WHILE
    conditional node); SBM_TUNE_HOST_LOOP drives the same chunk from the host
    (for profilers).  Both run the same kernels on the same state, so the
    iterations and the solution agree bit for bit."""
    shape = (48, 40, 36)
    m, prob = _problem(shape, 23, tunnel=True)
    out = []
    with sbm.Context(*shape) as ctx:
        _load(ctx, prob)
        for host in (False, True, False):
            ctx.set_tuning(host_loop=host)
            ctx.upload("x", prob["x"])
            info = ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO,
                                scale=1.0, tol=1e-8, max_it=50000, stop_rule=sbm.STOP_REL_RES,
                                precision=sbm.PREC_MIXED, precond=precond)
            assert info["status"] == 0
            out.append((info["iters"], info["final_res"], ctx.download("x")))
    for iters, res, x in out[1:]:
        assert iters == out[0][0] and res == out[0][1]
        np.testing.assert_array_equal(x, out[0][2])
