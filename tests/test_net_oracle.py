"""CPU checks of the learned preconditioner's oracle and host logic: the
NumPy backward pass against central finite differences (float64, no
rounding), the product's feature computation against the oracle's, the
prolongation's exactness on constant / linear fields, the parameter layout
shared with the CUDA library, and the stored weights file."""
import numpy as np
import pytest

from oracle import net_oracle as no
from elsim_gb300 import learned


def _params(seed, bias=0.1):
    rng = np.random.default_rng(seed)
    p = np.zeros(no.NPARAM)
    for l in range(10):
        taps = 1 if l == no.OUT else 27
        n = no.CO[l] * taps * no.CI[l]
        p[no.OFF[l]:no.OFF[l] + n] = rng.normal(size=n) * np.sqrt(2.0 / (taps * no.CI[l]))
        p[no.BOFF[l]:no.BOFF[l] + no.CO[l]] = rng.normal(size=no.CO[l]) * bias
    return p


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = _params(1)
    x = rng.normal(size=(1, 16, 16, 16, 16))
    t = rng.normal(size=(1, 16, 16, 16))
    _, g = no.loss_grad(p, x, t, rounding=False)
    errs = []
    for l in range(10):
        for i in rng.integers(no.OFF[l], no.BOFF[l] + no.CO[l], size=2):
            e = 1e-5 * max(1.0, abs(p[i]))
            pp = p.copy()
            pp[i] += e
            lp = ((no.forward(pp, x, False)[0] - t) ** 2).mean()
            pp[i] -= 2 * e
            lm = ((no.forward(pp, x, False)[0] - t) ** 2).mean()
            fd = (lp - lm) / (2 * e)
            errs.append(abs(fd - g[i]) / max(abs(g[i]), 1e-6))
    assert max(errs) < 1e-4


@pytest.mark.parametrize("cne", [False, True])
def test_features_match_oracle(cne):
    rng = np.random.default_rng(4)
    r = rng.normal(size=(32, 16, 24))
    k = rng.uniform(0.1, 1.0, size=(32, 16, 24))
    d = rng.uniform(0.0, 1.0, size=(32, 16, 24)) if cne else None
    f1, s1, c1 = learned.features(r, k, 1, 0, d, 0.3)
    f2, s2, c2, v = no.features(r, k, 1, 0, d, 0.3)
    assert f1.shape == (8 * 4 * 6, 16) and v == (8, 4, 6)
    # the oracle pads the coarse grid with zero cells to multiples of 16
    assert f2.shape == (1, 16, 16, 16, 16)
    assert not f2[0, 6:].any() and not f2[0, :, 4:].any() and not f2[0, :, :, 8:].any()
    np.testing.assert_allclose(f1, f2[0, :6, :4, :8].reshape(-1, 16), rtol=1e-6, atol=1e-6)
    assert s1 == pytest.approx(s2) and c1 == pytest.approx(c2)
    assert f1[:, 3].sum() == 8 * 6 and f1[:, 4].sum() == 0  # x0 face only
    if cne:
        x = no.restrict(d) / (0.3 * c2)
        np.testing.assert_allclose(f2[0, :6, :4, :8, 5], np.transpose(x / (1 + x), (2, 1, 0)),
                                   rtol=1e-12)
    else:
        assert not f1[:, 5].any()


def test_padded_forward_equals_unpadded_where_the_grid_is_whole():
    """A 16^3 grid zero-padded to 32^3 with the padding masked runs the
    network exactly as the 16^3 grid itself: the zero padding stands for the
    convolutions' zero fill beyond the faces."""
    rng = np.random.default_rng(8)
    p = _params(2)
    x = rng.normal(size=(1, 16, 16, 16, 16))
    want, _ = no.forward(p, x, rounding=False)
    xp = np.zeros((1, 32, 32, 32, 16))
    xp[:, :16, :16, :16] = x
    got, _ = no.forward(p, xp, rounding=False, valid=(16, 16, 16))
    np.testing.assert_allclose(got[:, :16, :16, :16], want, rtol=1e-12, atol=1e-12)


def test_target_is_restricted_scaled_error():
    rng = np.random.default_rng(5)
    e = rng.normal(size=(16, 16, 16))
    t = learned.target(e, s=2.0, cref=0.5, scale=3.0, kout=4.0)
    ref = no.restrict(e) * 3.0 * 0.5 / (2.0 * 4.0)
    np.testing.assert_allclose(t, np.transpose(ref, (2, 1, 0)).ravel(), rtol=1e-6)


def test_prolongation_exact_on_constants_and_interior_linear():
    assert np.abs(no.prolong(np.full((4, 5, 6), 2.5)) - 2.5).max() == 0.0
    c = np.arange(8, dtype=float)[:, None, None] * np.ones((8, 3, 3))
    f = no.prolong(c)
    pos = (np.arange(32) + 0.5) / 4 - 0.5
    np.testing.assert_allclose(f[2:-2, 1, 1], pos[2:-2], atol=1e-12)
    assert f[0, 0, 0] == 0.0 and f[-1, 0, 0] == 7.0  # clamped at the faces


def test_parameter_layout_matches_library(built):
    from elsim_gb300 import sbm
    assert sbm.Net.param_count() == no.NPARAM


def test_stored_weights():
    p, kout = learned.read()
    assert p.dtype == np.float32 and p.size == no.NPARAM
    assert np.isfinite(p).all() and kout > 0


def test_weights_file_round_trip(tmp_path):
    class _Net:  # what save() reads from a network
        out_scale = 2.5

        def params(self):
            return np.arange(no.NPARAM, dtype=np.float32)

    learned.save(tmp_path / "w.bin", _Net(), {"sizes": [[64, 1]], "loss": np.ones(30)})
    p, kout = learned.read(tmp_path / "w.bin")
    assert kout == 2.5 and np.array_equal(p, np.arange(no.NPARAM, dtype=np.float32))
    assert (tmp_path / "w.json").exists()


def test_apply_dir_matches_c_oracle():
    """The NumPy operator of the multiplicative preconditioner step equals
    the C oracle's operator with the search-direction ghost rules."""
    from oracle import sbm_oracle as orc
    rng = np.random.default_rng(0)
    coef = np.asfortranarray(rng.uniform(0.1, 1.0, size=(10, 12, 9)))
    p = rng.normal(size=(8, 10, 7))
    for bc0, bc1 in ((1, 1), (0, 1), (1, 0)):
        ph = np.pad(p, 1, mode="edge")
        if bc0:
            ph[:, 0, :] = 0.0
        if bc1:
            ph[:, -1, :] = 0.0
        want = orc.apply(coef, np.asfortranarray(ph), 0.7)[1:-1, 1:-1, 1:-1]
        assert np.array_equal(no.apply_dir(coef, p, 0.7, bc0, bc1), want)


def test_multiplicative_form_cuts_iterations():
    """Flexible CG (FP64, NumPy) on a 64^3 tunnelled structure with the
    stored network: the multiplicative form (coarse correction, then one
    Jacobi step with the GPU's omega on the remaining residual) needs clearly
    fewer iterations than the additive form."""
    from elsim_gb300 import learned, synth
    from oracle import sbm_oracle as orc
    m = synth.microstructure((64, 64, 64), seed=5, tunnel=True, redist=orc.redist)
    prob = synth.potential_problem(m["psi"])
    params, kout = learned.read()
    params = params.astype(np.float64)
    I = (slice(1, -1),) * 3

    def fcg(mult, tol=1e-8, cap=400):
        r = orc.residual(prob["coef"], prob["rhs"], prob["x"], 1.0)
        r0 = np.linalg.norm(r[I])
        z = no.pc_apply(params, kout, prob["coef"], r, multiplicative=mult)
        p, rz = z.copy(), (z * r).sum()
        for it in range(1, cap + 1):
            q = np.zeros_like(r)
            q[I] = no.apply_dir(prob["coef"], p[I], 1.0, 1, 1)
            pq = (p * q).sum()
            r -= (rz / pq) * q
            if np.linalg.norm(r[I]) <= tol * r0:
                return it
            z = no.pc_apply(params, kout, prob["coef"], r, multiplicative=mult)
            beta = -(z * q).sum() / pq
            rz = (z * r).sum()
            p = z + beta * p
        return cap

    add, mult = fcg(False), fcg(True)
    assert mult <= 0.75 * add, (add, mult)
