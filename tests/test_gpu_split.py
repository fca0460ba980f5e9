"""The double-float split of FP64 values, through the C-ABI.

The mixed-precision solver carries the operator, the initial iterate and the
right-hand side as FP32 pairs hi + lo, hi = (float)x, lo = (float)(x - hi).
sbm_split_f64 (and the solver's set-up, which uses the same device routine)
forms them with integer instructions; the pairs must equal those two FP64
expressions bit for bit -- including ties, roundings that carry into the
next binade, signed zeros, subnormal results and the values outside the
integer path's range, which take the FP64 expressions themselves.
"""
import numpy as np
import pytest

from elsim_gb300 import sbm

pytestmark = pytest.mark.gpu


def _split_gpu(x):
    import torch
    lib = sbm.load_library()
    d_x = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    d_hi = torch.empty(x.size, dtype=torch.float32, device="cuda")
    d_lo = torch.empty(x.size, dtype=torch.float32, device="cuda")
    rc = lib.sbm_split_f64(x.size, d_x.data_ptr(), d_hi.data_ptr(), d_lo.data_ptr(), None)
    assert rc == sbm.OK, lib.sbm_last_error()
    torch.cuda.synchronize()
    return d_hi.cpu().numpy(), d_lo.cpu().numpy()


def _split_ref(x):
    with np.errstate(invalid="ignore", over="ignore"):
        hi = x.astype(np.float32)
        lo = (x - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def _same_bits(a, b):
    nan = np.isnan(a)
    assert np.array_equal(nan, np.isnan(b))
    return np.array_equal(a[~nan].view(np.uint32), b[~nan].view(np.uint32))


def _cases():
    one = 1.0
    special = [
        0.0, -0.0, 1.0, -1.0, 0.1, -0.1, 1.0 / 3.0, np.pi, 2.0 / 3.0 * 1e-5,
        # ties: halfway between two floats, to even (down) and to even (up)
        one + 2.0**-24, one + 3 * 2.0**-24, -(one + 2.0**-24), 3.0 + 2.0**-22,
        # a tie one unit of the double's last place either side
        one + 2.0**-24 + 2.0**-52, one + 2.0**-24 - 2.0**-52,
        # rounding that carries into the next binade
        2.0 - 2.0**-53, 2.0 - 2.0**-25, 4.0 - 2.0**-24, -(1.0 - 2.0**-54),
        # the integer path's range ends and the FP64 path beyond them
        2.0**-70, 2.0**-70 * (1 + 2.0**-30), 2.0**-71, 2.0**126 * 1.5, 2.0**127,
        1.9999999 * 2.0**126, 2.0**127 * 1.99999999, 1e-30, 1e-40, 1e-45, 5e-324,
        2.0**-126, 2.0**-149, 1e300, -1e300, 3.5e38, 3.4e38, np.inf, -np.inf, np.nan,
    ]
    rng = np.random.default_rng(11)
    wide = rng.standard_normal(200_000) * 10.0 ** rng.uniform(-45, 40, 200_000)
    unit = rng.uniform(-2, 2, 200_000)
    bits = rng.integers(0, 2**63, 100_000, dtype=np.uint64)
    bits[::2] |= np.uint64(1) << np.uint64(63)
    raw = bits.view(np.float64)
    return np.concatenate([np.array(special), wide, unit, raw])


def test_split_matches_the_fp64_expressions_bit_for_bit(built):
    x = _cases()
    hi, lo = _split_gpu(x)
    rhi, rlo = _split_ref(x)
    assert _same_bits(hi, rhi)
    assert _same_bits(lo, rlo)
    # the pair carries the value to about 48 bits where both parts are normal
    ok = np.isfinite(x) & (np.abs(x) > 1e-30) & (np.abs(x) < 1e30)
    back = hi[ok].astype(np.float64) + lo[ok].astype(np.float64)
    assert np.max(np.abs(back - x[ok]) / np.abs(x[ok])) < 2.0**-47


def test_split_of_nothing_and_bad_arguments(built):
    lib = sbm.load_library()
    assert lib.sbm_split_f64(0, None, None, None, None) == sbm.OK
    assert lib.sbm_split_f64(-1, None, None, None, None) == sbm.ERR_ARG
    assert lib.sbm_split_f64(4, None, None, None, None) == sbm.ERR_ARG
