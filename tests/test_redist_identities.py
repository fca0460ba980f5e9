"""The operation-saving form of AbsGrd3DUW_XYZ and the ReDist3D_XYZ update
that the GPU kernels use (one subtraction and one square per direction,
integer comparisons; elsim_gb300/csrc/sbm_levelset.cu), restated in NumPy
and checked bit for bit against the oracle's literal form on fields with
ties, zeros of both signs and tiny values."""
import numpy as np
import pytest

from oracle import sbm_oracle as orc


def _okey(x):
    b = x.view(np.int64)
    return b ^ ((b >> 63) & np.int64(0x7FFFFFFFFFFFFFFF))


def _imin(a, b):
    return np.where(_okey(a) <= _okey(b), a, b)


def _imax(a, b):
    return np.where(_okey(a) >= _okey(b), a, b)


def _pos0(x):
    return np.where(x.view(np.int64) > 0, x, 0.0)


def _absgrd_fast(sg, f):
    c = f[1:-1, 1:-1, 1:-1]
    ym, yp = f[:-2, 1:-1, 1:-1], f[2:, 1:-1, 1:-1]
    xm, xp = f[1:-1, :-2, 1:-1], f[1:-1, 2:, 1:-1]
    zm, zp = f[1:-1, 1:-1, :-2], f[1:-1, 1:-1, 2:]
    pos = [_pos0(c - _imin(m, p)) for m, p in ((ym, yp), (xm, xp), (zm, zp))]
    neg = [_pos0(_imax(m, p) - c) for m, p in ((ym, yp), (xm, xp), (zm, zp))]
    gp = np.sqrt((pos[0] * pos[0] + pos[1] * pos[1]) + pos[2] * pos[2])
    gn = np.sqrt((neg[0] * neg[0] + neg[1] * neg[1]) + neg[2] * neg[2])
    s = sg[1:-1, 1:-1, 1:-1]
    sb = s.view(np.int64)
    out = np.where(sb > 0, gp, gn)
    return np.where((sb << 1) == 0, 0.0, out)


def _prod_pos(v, f):
    a, b = v.view(np.int64), f.view(np.int64)
    zero = ((a << 1) == 0) | ((b << 1) == 0) | ((a ^ b) < 0)
    ea, eb = (a >> 52) & 0x7FF, (b >> 52) & 0x7FF
    sure = (ea != 0) & (eb != 0) & (ea != 0x7FF) & (eb != 0x7FF) & (ea + eb >= 972)
    with np.errstate(under="ignore"):
        slow = (v * f) > 0.0
    return ~zero & (sure | slow)


def _field(shape, seed):
    rng = np.random.default_rng(seed)
    f = rng.normal(size=shape)
    # ties between neighbours, signed zeros and tiny values
    f[rng.random(shape) < 0.2] = 0.5
    f[rng.random(shape) < 0.05] = 0.0
    f[rng.random(shape) < 0.05] = -0.0
    f[rng.random(shape) < 0.03] = 1e-170
    f[rng.random(shape) < 0.03] = -3e-160
    return np.asfortranarray(f)


@pytest.mark.parametrize("seed", range(4))
def test_absgrd_identity(seed):
    shape = (14, 11, 9)
    f = _field(shape, seed)
    sg = np.asfortranarray(np.random.default_rng(seed + 50).choice([-1.0, 0.0, 1.0, -0.0, 0.7, -2.5],
                                                                   size=shape))
    want = orc.absgrd(sg, f)[1:-1, 1:-1, 1:-1]
    got = _absgrd_fast(sg, f)
    assert np.array_equal(got.view(np.int64), want.view(np.int64))


@pytest.mark.parametrize("seed", range(3))
def test_sign_check_identity(seed):
    rng = np.random.default_rng(seed)
    v = _field((4000,), seed + 10)
    f = _field((4000,), seed + 20)
    v[:200] = rng.choice([1e-160, -1e-160, 2e-300, 5e-324], size=200)
    f[:200] = rng.choice([1e-160, 3e-170, -2e-300, 1e10], size=200)
    with np.errstate(under="ignore"):
        want = (v * f) > 0.0
    assert np.array_equal(_prod_pos(v, f), want)
