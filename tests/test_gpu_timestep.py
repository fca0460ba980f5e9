"""GPU parity of whole electrochemical time steps (SBMES:357-840) against the
oracle: set-up from two REAL(4) distance fields, then Cahn-Hilliard, the CnE
solve with its flux condition and mean correction, the potentials with the
Butler-Volmer Picard loop, and the voltage control -- for the reference's
exponential Butler-Volmer and for the linearised form.
"""
import numpy as np
import pytest

from conftest import rel_l2
from elsim_gb300 import sbm, synth
from oracle import sbm_oracle as orc

pytestmark = pytest.mark.gpu

FIELDS = [sbm.F_CNP, sbm.F_CNE, sbm.F_PHP, sbm.F_PHE, sbm.F_RXN]
# each field is compared in its own phase, weighted as the reference's
# convergence norms weight it (SBMES:545, :702, :783): outside its phase the
# domain parameter floors at 1e-7 / 1e-6 and the systems are near-singular.
WEIGHT = {sbm.F_CNP: sbm.F_PSP, sbm.F_PHP: sbm.F_PSP, sbm.F_CNE: sbm.F_PSE,
          sbm.F_PHE: sbm.F_PSE, sbm.F_RXN: None}


def _werr(got, ref, w):
    i = (slice(1, -1),) * 3
    w = np.ones_like(ref[i]) if w is None else w[i]
    d = got[i] - ref[i]
    return float(np.sqrt((w * d * d).sum() / max((w * ref[i] * ref[i]).sum(), 1e-300)))


def _dist(shape, seed):
    m = synth.microstructure(shape, seed=seed, reinit_steps=60, redist=orc.redist)
    d = m["dist"][1:-1, 1:-1, 1:-1]
    return d.astype(np.float32), (-d).astype(np.float32)


def _params(tight, bv_mode):
    p = synth.reference_tables(orc.params_reference())
    p.bv_mode = bv_mode
    if tight:
        # tighter CG tolerances so both sides land on the same fields; the
        # Picard tolerance stays the reference's 1e-8 (SBMES:627) -- pushed
        # further, the explicit Butler-Volmer fixed point diverges (Rxn
        # overflows) on small geometries, in the oracle as on the GPU
        p.crt_cne = p.crt_php = p.crt_phe = 1e-11
    return p


def _run(shape, p, steps, seed=4, mean_every=None):
    if mean_every:
        p.cne_mean_every = mean_every
    dp, de = _dist(shape, seed)
    st = orc.State(*shape, p)
    so = st.setup_domain(dp, de)
    ctx = sbm.Context(*shape, params=p)
    sg = ctx.setup_domain(dp, de)
    for key in ("tPP", "tPE", "xrf", "trgI"):
        assert abs(sg[key] - so[key]) <= 1e-12 * abs(so[key]), key
    hist = []
    for it in range(1, steps + 1):
        dt, vsr = synth.step_schedule(so["xrf"], abs(so["trgI"] - so["scrnt"]), so["trgI"])
        so = st.time_step(it, dt, vsr)
        sg = ctx.time_step(it, dt, vsr)
        hist.append((sg, so))
    return ctx, st, hist


@pytest.mark.parametrize("bv_mode", [sbm.BV_EXP, sbm.BV_LINEAR])
def test_time_steps_match_oracle_tight(built, bv_mode):
    shape = (20, 24, 16)
    ctx, st, hist = _run(shape, _params(True, bv_mode), 3, mean_every=2)
    sg, so = hist[-1]
    for key in ("xrf", "scrnt", "bve", "infx"):
        assert abs(sg[key] - so[key]) <= 1e-7 * max(abs(so[key]), 1e-12), (key, sg[key], so[key])
    for f in FIELDS:
        w = st.field(WEIGHT[f]) if WEIGHT[f] is not None else None
        assert _werr(ctx.download(f), st.field(f), w) < 1e-7, f
    # the set-up fields are bit-for-bit functions of psi except for tanh
    assert rel_l2(ctx.download(sbm.F_PSP), st.field(sbm.F_PSP)) < 1e-14
    assert rel_l2(ctx.download(sbm.F_AVP), st.field(sbm.F_AVP)) < 1e-12
    ctx.close()


def test_time_steps_reference_tolerances(built):
    """With the reference's own tolerances both sides stop on the same norms;
    iteration counts agree to a couple of iterations, fields to the solver
    tolerance."""
    shape = (24, 20, 18)
    ctx, st, hist = _run(shape, _params(False, sbm.BV_EXP), 3, seed=6)
    for sg, so in hist:
        for key in ("it_cne", "it_php", "it_phe", "n_picard"):
            assert abs(sg[key] - so[key]) <= max(2, 0.02 * so[key]), (key, sg[key], so[key])
    sg, so = hist[-1]
    assert abs(sg["xrf"] - so["xrf"]) <= 1e-9 * abs(so["xrf"])
    for f in (sbm.F_CNP, sbm.F_CNE):
        assert _werr(ctx.download(f), st.field(f), st.field(WEIGHT[f])) < 1e-6, f
    ctx.close()


def test_stage_calls_equal_full_step(built):
    shape = (12, 16, 10)
    p = _params(False, sbm.BV_EXP)
    dp, de = _dist(shape, 8)
    a = sbm.Context(*shape, params=p)
    b = sbm.Context(*shape, params=p)
    a.setup_domain(dp, de)
    b.setup_domain(dp, de)
    dt, vsr = 1e-3, 0.02
    for it in (1, 2):
        a.time_step(it, dt, vsr)
        b.ch_step(dt)
        b.cne_step(it, dt)
        b.bv_update()
        b.voltage_step(dt, vsr)
    for f in FIELDS:
        assert np.array_equal(a.download(f), b.download(f))
    a.close()
    b.close()


def test_step_before_setup_is_a_state_error(built):
    with sbm.Context(8, 8, 8) as ctx:
        with pytest.raises(sbm.SbmError) as e:
            ctx.time_step(1, 1e-3, 0.01)
        assert e.value.code == sbm.ERR_STATE


def test_diverging_picard_loop_is_reported_not_hidden(built):
    """On this small geometry with CG tolerances tightened to 1e-11 the
    explicit Butler-Volmer fixed point diverges (the oracle overflows too);
    the GPU step must stop with SBM_ERR_NONFINITE, not loop or go on."""
    shape = (12, 16, 10)
    p = _params(True, sbm.BV_EXP)
    dp, de = _dist(shape, 8)
    st = orc.State(*shape, p)
    so = st.setup_domain(dp, de)
    with pytest.raises(RuntimeError):
        for it in (1, 2, 3):
            dt, vsr = synth.step_schedule(so["xrf"], abs(so["trgI"] - so["scrnt"]), so["trgI"])
            so = st.time_step(it, dt, vsr)
    with sbm.Context(*shape, params=p) as ctx:
        sg = ctx.setup_domain(dp, de)
        with pytest.raises(sbm.SbmError) as e:
            for it in (1, 2, 3):
                dt, vsr = synth.step_schedule(sg["xrf"], abs(sg["trgI"] - sg["scrnt"]), sg["trgI"])
                sg = ctx.time_step(it, dt, vsr)
        assert e.value.code == sbm.ERR_NONFINITE


def test_mixed_precision_time_steps_match_oracle(built):
    """The whole step with the mixed-precision stage solves (FP32 Jacobi-PCG
    inside FP64 refinement to rel-res 1e-10) against the FP64 oracle with
    tightened CG tolerances: the same fields to 1e-6 in their phases."""
    shape = (20, 24, 16)
    p = _params(True, sbm.BV_EXP)
    dp, de = _dist(shape, 4)
    st = orc.State(*shape, p)
    so = st.setup_domain(dp, de)
    with sbm.Context(*shape, params=p) as ctx:
        ctx.setup_domain(dp, de)
        for it in (1, 2, 3):
            dt, vsr = synth.step_schedule(so["xrf"], abs(so["trgI"] - so["scrnt"]), so["trgI"])
            so = st.time_step(it, dt, vsr)
            sg = ctx.time_step(it, dt, vsr, precision=sbm.PREC_MIXED)
        for key in ("xrf", "scrnt", "bve"):
            assert abs(sg[key] - so[key]) <= 1e-6 * max(abs(so[key]), 1e-12), (key, sg[key], so[key])
        for f in FIELDS:
            w = st.field(WEIGHT[f]) if WEIGHT[f] is not None else None
            assert _werr(ctx.download(f), st.field(f), w) < 1e-6, f


def _full_step_setup(shape, seed, tight):
    """The full-step workload (double-well Cahn-Hilliard, linearised
    Butler-Volmer, i0 = 1e-3, 20 reinitialisation steps, c0 = 0.5 +- 0.01)."""
    p = synth.full_step_params(orc.params_reference())
    if tight:
        p.crt_cne = p.crt_php = p.crt_phe = 1e-11
    m = synth.microstructure(shape, seed=seed, reinit_steps=20, redist=orc.redist)
    d = m["dist"][1:-1, 1:-1, 1:-1]
    return p, d.astype(np.float32), (-d).astype(np.float32), synth.full_step_concentration(shape, seed)


def test_full_step_workload_matches_oracle(built):
    shape = (20, 24, 16)
    p, dp, de, c0 = _full_step_setup(shape, 4, True)
    st = orc.State(*shape, p)
    so = st.setup_domain(dp, de)
    st.set_field(sbm.F_CNP, c0)
    with sbm.Context(*shape, params=p) as ctx:
        ctx.setup_domain(dp, de)
        ctx.upload(sbm.F_CNP, c0)
        vsr = synth.step_schedule(so["xrf"], 0.0, so["trgI"])[1]
        for it in range(1, 6):
            so = st.time_step(it, synth.FULL_STEP_DT, vsr)
            sg = ctx.time_step(it, synth.FULL_STEP_DT, vsr)
        for key in ("xrf", "scrnt", "bve"):
            assert abs(sg[key] - so[key]) <= 1e-7 * max(abs(so[key]), 1e-12), (key, sg[key], so[key])
        for f in FIELDS:
            w = st.field(WEIGHT[f]) if WEIGHT[f] is not None else None
            assert _werr(ctx.download(f), st.field(f), w) < 1e-7, f


def test_full_step_workload_128(built):
    """128^3, 100 steps of the full-step workload on the GPU: every solve
    converges, the concentration stays finite and inside [0, 1], the mean
    moves only by the reaction, and a second run from the same state is
    bit-identical (deterministic reductions)."""
    shape = (128, 128, 128)
    p, dp, de, c0 = _full_step_setup(shape, 1, False)
    with sbm.Context(*shape, params=p) as ctx:
        s0 = ctx.setup_domain(dp, de)
        ctx.upload(sbm.F_CNP, c0)
        vsr = synth.step_schedule(s0["xrf"], 0.0, s0["trgI"])[1]
        snap = None
        hist = []
        for it in range(1, 101):
            if it == 91:
                snap = ctx.snapshot()
            hist.append(ctx.time_step(it, synth.FULL_STEP_DT, vsr))
        c = ctx.download(sbm.F_CNP)[1:-1, 1:-1, 1:-1]
        assert np.isfinite(c).all() and c.min() >= 0.0 and c.max() <= 1.0
        assert all(h["it_cne"] < p.max_it_cne - 1 and h["n_picard"] < p.max_picard for h in hist)
        assert abs(hist[-1]["xrf"] - 0.5) < 0.05
        ctx.restore(snap)
        again = [ctx.time_step(it, synth.FULL_STEP_DT, vsr) for it in range(91, 101)]
        assert again == hist[90:]
        assert np.array_equal(ctx.download(sbm.F_CNP)[1:-1, 1:-1, 1:-1], c)
