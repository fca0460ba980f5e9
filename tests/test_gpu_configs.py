"""GPU parity against the oracle on the stated workloads themselves, not on
reduced grids:

* the plain 64^3 potential solve (spheres r ~ U[4,10], solid 0.6, 175
  reinitialisation steps, Dirichlet 0 / 1 on the two x faces, FP64 CG to
  rel-res 1e-8) -- the reference's potential CG loop
  (SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90:661-714) with the
  rel-res stopping rule;
* the 128^3 full electrochemical step (double-well Cahn-Hilliard,
  linearised Butler-Volmer, 20 reinitialisation steps): fields and scalars
  after the first two steps (SBMES:397-840);
* the 256^3 potential solve with a tunnel (the benchmarked solve): the
  production mixed-precision solve with the learned preconditioner, and the
  GPU's plain FP64 CG, against the oracle's FP64 CG;
* the 256^3 concentration system of the same microstructure in the CnE form
  (SBMES:509-554): psE c - s div(psE grad c) = psE c_old, Neumann faces.

Tolerances: FP64 CG against the oracle's FP64 CG within 3 iterations and
rel-L2 <= 1e-9 (tree- versus plane-ordered sums); mixed precision rel-L2 <=
1e-6 against the FP64 oracle solution at the same rel-res 1e-8 (for the
potentials also the true FP64 residual <= 1.05e-8); time-step fields within 1e-7 in their own phase
(weighted as the reference's convergence norms weight them) except phE,
whose CG tolerance is 1e-6 (SBMES:98); scalars within 1e-6 relative.
"""
import numpy as np
import pytest

from elsim_gb300 import sbm, synth
from oracle import sbm_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-8


def _i(a):
    return a[1:-1, 1:-1, 1:-1]


def _rel(a, b):
    return float(np.linalg.norm(_i(a) - _i(b)) / np.linalg.norm(_i(b)))


def _true_relres(prob, x):
    """FP64 rel-res of a potential solution (Dirichlet x faces kept in the
    ghosts, y / z ghosts copied from the edge)."""
    xg = x.copy(order="F")
    orc.lib().orc_bc_yz(*orc.hdims(xg), orc._p(xg))
    r = orc.residual(prob["coef"], prob["rhs"], xg, 1.0)
    r0 = orc.residual(prob["coef"], prob["rhs"], prob["x"], 1.0)
    return np.linalg.norm(_i(r)) / np.linalg.norm(_i(r0))


def _solve(ctx, prob, precision, precond, op=sbm.OP_GENERIC):
    ctx.upload("x", prob["x"])
    bc = sbm.BC_COPY if op == sbm.OP_GENERIC_DIAG else sbm.BC_ZERO
    info = ctx.cg_solve(op=op, bc_x0=bc, bc_x1=bc, scale=prob.get("scale", 1.0), tol=TOL,
                        max_it=200000, stop_rule=sbm.STOP_REL_RES, precision=precision,
                        precond=precond)
    return info, ctx.download("x")


def _oracle(prob):
    bc = sbm.BC_COPY if "diag" in prob else sbm.BC_ZERO
    return orc.cg(prob["coef"], prob["rhs"], prob["x"], prob.get("scale", 1.0), bc, bc,
                  sbm.STOP_REL_RES, TOL, 200000, diag=prob.get("diag"))


def test_c1_plain_solve_64_matches_oracle(built):
    from elsim_gb300 import learned
    n = 64
    m = synth.microstructure((n, n, n), seed=1)
    assert abs(m["solid_fraction"] - 0.6) < 0.01
    prob = synth.potential_problem(m["psi"])
    xo, io = _oracle(prob)
    assert io["status"] == 0
    with sbm.Context(n, n, n) as ctx:
        for k in ("coef", "x", "rhs", "weight"):
            ctx.upload(k, prob[k])
        g, x = _solve(ctx, prob, sbm.PREC_FP64, sbm.PC_NONE)
        assert g["status"] == 0 and abs(g["iters"] - io["iters"]) <= 3, (g, io)
        assert _rel(x, xo) <= 1e-9
        ctx.set_net(learned.load())
        gm, xm = _solve(ctx, prob, sbm.PREC_MIXED, sbm.PC_LEARNED)
        assert gm["status"] == 0 and ctx.last_precond() == sbm.PC_LEARNED
    assert _rel(xm, xo) <= 1e-6
    assert _true_relres(prob, xm) <= 1.05e-8


def test_c2_first_two_full_steps_128_match_oracle(built):
    shape = (128, 128, 128)
    p = synth.full_step_params(orc.params_reference())
    m = synth.microstructure(shape, seed=1, reinit_steps=20)
    d = _i(m["dist"])
    dp, de = d.astype(np.float32), (-d).astype(np.float32)
    c0 = synth.full_step_concentration(shape, 1)
    dt = synth.FULL_STEP_DT
    st = orc.State(*shape, p)
    so = st.setup_domain(dp, de)
    st.set_field(sbm.F_CNP, c0)
    with sbm.Context(*shape, params=p) as ctx:
        sg = ctx.setup_domain(dp, de)
        ctx.upload(sbm.F_CNP, c0)
        for key in ("tPP", "tPE", "xrf", "trgI"):
            assert abs(sg[key] - so[key]) <= 1e-12 * abs(so[key]), key
        vsr = synth.step_schedule(so["xrf"], 0.0, so["trgI"])[1]
        for it in (1, 2):
            so = st.time_step(it, dt, vsr)
            sg = ctx.time_step(it, dt, vsr)
        for key in ("xrf", "scrnt", "bve", "infx"):
            assert abs(sg[key] - so[key]) <= 1e-6 * max(abs(so[key]), 1e-12), (key, sg[key], so[key])
        tol = {sbm.F_CNP: 1e-7, sbm.F_CNE: 1e-7, sbm.F_PHP: 1e-7, sbm.F_PHE: 1e-6}
        wf = {sbm.F_CNP: sbm.F_PSP, sbm.F_PHP: sbm.F_PSP, sbm.F_CNE: sbm.F_PSE,
              sbm.F_PHE: sbm.F_PSE}
        for f, t in tol.items():
            w = _i(st.field(wf[f]))
            a, b = _i(ctx.download(f)), _i(st.field(f))
            err = np.sqrt((w * (a - b) ** 2).sum() / (w * b * b).sum())
            assert err < t, (f, err)
    st.close()


@pytest.fixture(scope="module")
def c3():
    """The benchmarked 256^3 microstructure (seed 1, one tunnel of radius 6)."""
    n = 256
    m = synth.microstructure((n, n, n), seed=1, tunnel=True)
    return m


def test_c3_potential_256_matches_oracle(built, c3):
    from elsim_gb300 import learned
    n = 256
    prob = synth.potential_problem(c3["psi"])
    xo, io = _oracle(prob)
    assert io["status"] == 0
    with sbm.Context(n, n, n) as ctx:
        for k in ("coef", "x", "rhs", "weight"):
            ctx.upload(k, prob[k])
        g, x = _solve(ctx, prob, sbm.PREC_FP64, sbm.PC_NONE)
        assert g["status"] == 0 and abs(g["iters"] - io["iters"]) <= 3, (g, io)
        assert _rel(x, xo) <= 1e-9
        ctx.set_net(learned.load())
        gm, xm = _solve(ctx, prob, sbm.PREC_MIXED, sbm.PC_LEARNED)
        assert gm["status"] == 0 and ctx.last_precond() == sbm.PC_LEARNED
        gj, _ = _solve(ctx, prob, sbm.PREC_MIXED, sbm.PC_JACOBI)
    assert _rel(xm, xo) <= 1e-6
    assert _true_relres(prob, xm) <= 1.05e-8
    # the learned preconditioner's gain at this size
    assert gm["iters"] < 0.2 * gj["iters"], (gm["iters"], gj["iters"])


def test_c3_concentration_256_matches_oracle(built, c3):
    n = 256
    prob = synth.concentration_problem(c3["psi"], 1)
    xo, io = _oracle(prob)
    assert io["status"] == 0
    with sbm.Context(n, n, n) as ctx:
        for k in ("coef", "x", "rhs", "weight", "diag"):
            ctx.upload(k, prob[k])
        g, x = _solve(ctx, prob, sbm.PREC_FP64, sbm.PC_NONE, op=sbm.OP_GENERIC_DIAG)
        assert g["status"] == 0 and abs(g["iters"] - io["iters"]) <= 3, (g, io)
        assert _rel(x, xo) <= 1e-9
        gm, xm = _solve(ctx, prob, sbm.PREC_MIXED, sbm.PC_LEARNED, op=sbm.OP_GENERIC_DIAG)
        assert gm["status"] == 0
    assert _rel(xm, xo) <= 1e-6
