"""Checkpoint / resume through the C-ABI: a context restored from a snapshot
(in memory or through a checkpoint file) continues bit for bit like the
context it was taken from -- electrochemical time steps in FP64 and mixed
precision, and GENERIC solves -- and foreign snapshots are rejected."""
import numpy as np
import pytest

from elsim_gb300 import sbm, synth
from oracle import sbm_oracle as orc

pytestmark = pytest.mark.gpu

STATE = [sbm.F_CNP, sbm.F_CNE, sbm.F_PHP, sbm.F_PHE, sbm.F_RXN, sbm.F_PSP, sbm.F_PSE,
         sbm.F_AVP, sbm.F_AVPX]


def _setup(shape, seed=4):
    m = synth.microstructure(shape, seed=seed, reinit_steps=60, redist=orc.redist)
    d = m["dist"][1:-1, 1:-1, 1:-1]
    p = synth.reference_tables(orc.params_reference())
    ctx = sbm.Context(*shape, params=p)
    s = ctx.setup_domain(d.astype(np.float32), (-d).astype(np.float32))
    return ctx, p, s


def _steps(ctx, s, first, n, precision):
    out = []
    for it in range(first, first + n):
        dt, vsr = synth.step_schedule(s["xrf"], abs(s["trgI"] - s["scrnt"]), s["trgI"])
        s = ctx.time_step(it, dt, vsr, precision=precision)
        out.append(s)
    return s, out


@pytest.mark.parametrize("precision", [sbm.PREC_FP64, sbm.PREC_MIXED])
def test_resume_time_steps_bit_for_bit(built, tmp_path, precision):
    shape = (20, 24, 16)
    a, p, s = _setup(shape)
    s, _ = _steps(a, s, 1, 2, precision)
    path = a.save(tmp_path / "run.ckpt", iter=2, tm=1.5e-3)
    s_a, hist_a = _steps(a, s, 3, 2, precision)
    b = sbm.Context(*shape)  # reference parameters; the snapshot brings the run's
    meta = b.load(path)
    assert meta == {"iter": 2, "tm": 1.5e-3}
    assert b.scalars() == s
    assert b.params.tbl_n == p.tbl_n and b.params.bv_mode == p.bv_mode
    s_b, hist_b = _steps(b, b.scalars(), meta["iter"] + 1, 2, precision)
    assert hist_a == hist_b
    for f in STATE:
        assert np.array_equal(a.download(f), b.download(f)), f
    a.close()
    b.close()


def test_snapshot_round_trip_and_generic_solve(built):
    shape = (32, 24, 20)
    m = synth.microstructure(shape, seed=7)
    prob = synth.potential_problem(m["psi"])
    a = sbm.Context(*shape)
    for k in ("coef", "x", "rhs", "weight"):
        a.upload(k, prob[k])
    blob = a.snapshot()
    b = sbm.Context(*shape)
    b.restore(blob)
    assert np.array_equal(b.snapshot(), blob)
    kw = dict(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO, scale=1.0, tol=1e-9,
              max_it=5000, stop_rule=sbm.STOP_REL_RES, precision=sbm.PREC_MIXED,
              precond=sbm.PC_JACOBI)
    ia, ib = a.cg_solve(**kw), b.cg_solve(**kw)
    assert ia["iters"] == ib["iters"]
    assert np.array_equal(a.download("x"), b.download("x"))
    a.close()
    b.close()


def test_restore_rejects_foreign_snapshots(built):
    a = sbm.Context(16, 12, 8)
    blob = a.snapshot()
    with sbm.Context(16, 12, 10) as other, pytest.raises(sbm.SbmError):
        other.restore(blob)
    bad = blob.copy()
    bad[0] ^= 0xFF
    with pytest.raises(sbm.SbmError):
        a.restore(bad)
    with pytest.raises(sbm.SbmError):
        a.restore(blob[:-8])
    a.close()
