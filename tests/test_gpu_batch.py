"""Batched uneven sub-volume solves (one parent CUDA graph per round) must
give every volume the same iterations and solution as solving it alone, and
the FP64-oracle accuracy of the mixed solver."""
import numpy as np
import pytest

from conftest import rel_l2
from elsim_gb300 import sbm, synth
from oracle import sbm_oracle as orc

pytestmark = pytest.mark.gpu


def _vol(n, seed, frac):
    m = synth.microstructure((n, n, n), seed=seed, solid_fraction=frac, reinit_steps=60,
                             redist=orc.redist)
    return synth.potential_problem(m["psi"])


def test_batch_equals_individual_solves(built):
    sizes = [24, 32, 16, 40, 24, 28]
    probs = [_vol(n, 100 + v, 0.5 + 0.04 * v) for v, n in enumerate(sizes)]
    ctxs = [sbm.Context(n, n, n) for n in sizes]
    for c, p in zip(ctxs, probs):
        for k in ("coef", "x", "rhs", "weight"):
            c.upload(k, p[k])
    out = sbm.batch_solve(ctxs, tol=1e-8, precond=sbm.PC_JACOBI)
    assert out["status"] == [0] * len(sizes)
    xs = [c.download("x") for c in ctxs]
    for v, (c, p) in enumerate(zip(ctxs, probs)):
        c.upload("x", p["x"])
        info = c.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0,
                          tol=1e-8, max_it=100000, stop_rule=sbm.STOP_REL_RES,
                          precision=sbm.PREC_MIXED, precond=sbm.PC_JACOBI)
        assert info["iters"] == out["iters"][v]
        assert np.array_equal(c.download("x"), xs[v])
        xo, _ = orc.cg(p["coef"], p["rhs"], p["x"], 1.0, sbm.BC_ZERO, sbm.BC_ZERO,
                       sbm.STOP_REL_RES, 1e-12, 50000)
        assert rel_l2(xs[v], xo) < 1e-6
        assert out["final_res"][v] <= 1e-8
    # a second batch call reuses the cached parent graph
    for c, p in zip(ctxs, probs):
        c.upload("x", p["x"])
    again = sbm.batch_solve(ctxs, tol=1e-8, precond=sbm.PC_JACOBI)
    assert again["iters"] == out["iters"]
    for c in ctxs:
        c.close()


def test_batch_with_learned_preconditioner(built):
    # 64^3 and 128^3 volumes take the learned preconditioner, the 48^3 one
    # falls back to Jacobi; each equals its single solve
    from elsim_gb300 import learned
    net = learned.load()
    sizes = [64, 48, 128, 64]
    probs = [_vol(n, 300 + v, 0.55 + 0.03 * v) for v, n in enumerate(sizes)]
    ctxs = [sbm.Context(n, n, n) for n in sizes]
    for c, p in zip(ctxs, probs):
        for k in ("coef", "x", "rhs", "weight"):
            c.upload(k, p[k])
        c.set_net(net)
    out = sbm.batch_solve(ctxs, tol=1e-8, precond=sbm.PC_LEARNED)
    assert out["status"] == [0] * len(sizes)
    assert [c.last_precond() for c in ctxs] == [sbm.PC_LEARNED, sbm.PC_JACOBI, sbm.PC_LEARNED,
                                                sbm.PC_LEARNED]
    xs = [c.download("x") for c in ctxs]
    for v, (c, p) in enumerate(zip(ctxs, probs)):
        c.upload("x", p["x"])
        info = c.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0,
                          tol=1e-8, max_it=100000, stop_rule=sbm.STOP_REL_RES,
                          precision=sbm.PREC_MIXED, precond=sbm.PC_LEARNED)
        assert info["iters"] == out["iters"][v]
        assert np.array_equal(c.download("x"), xs[v])
        assert out["final_res"][v] <= 1e-8
    for c in ctxs:
        c.close()

