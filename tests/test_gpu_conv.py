"""The tcgen05 BF16 implicit-GEMM 3x3x3 convolution against the CUDA-core
kernel and a float64 NumPy convolution of the same BF16 values.

BF16 x BF16 products are exact in FP32, so the only difference is the FP32
summation order: tolerance 1e-5 relative to the largest output.
"""
import ctypes as C

import numpy as np
import pytest

from elsim_gb300 import sbm

pytestmark = pytest.mark.gpu


def to_bf16(a):
    b = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
    b = b + np.uint32(0x7FFF) + ((b >> np.uint32(16)) & np.uint32(1))
    return (b >> np.uint32(16)).astype(np.uint16)


def from_bf16(h):
    return (h.astype(np.uint32) << np.uint32(16)).view(np.float32)


def np_conv(x, w, b, shape, relu, flip):
    ny, nx, nz = shape
    cin = x.shape[1]
    cout = w.shape[0]
    X = x.reshape(nz, nx, ny, cin).astype(np.float64)  # v = i + ny*(j + nx*k)
    Xp = np.zeros((nz + 2, nx + 2, ny + 2, cin))
    Xp[1:-1, 1:-1, 1:-1] = X
    W = w.reshape(cout, 27, cin).astype(np.float64)
    out = np.zeros((nz, nx, ny, cout)) + (b if b is not None else 0.0)
    for t in range(27):
        di, dj, dk = t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1
        if flip:
            di, dj, dk = -di, -dj, -dk
        sl = Xp[1 + dk:1 + dk + nz, 1 + dj:1 + dj + nx, 1 + di:1 + di + ny]
        out += sl @ W[:, t, :].T
    if relu:
        out = np.maximum(out, 0)
    return out.reshape(-1, cout)


def run(shape, cin, cout, relu, flip, use_tc, x16, w16, bias):
    lib = sbm.load_library()
    nv = int(np.prod(shape))
    y = np.zeros((nv, cout), dtype=np.float32)
    u16 = C.POINTER(C.c_uint16)
    rc = lib.sbm_conv3d_bf16(*shape, cin, cout, x16.ctypes.data_as(u16), w16.ctypes.data_as(u16),
                             bias.ctypes.data_as(C.POINTER(C.c_float)), relu, flip, use_tc,
                             y.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == 0, lib.sbm_last_error()
    return y


# z extents: odd -> one plane per CTA, even -> two, multiples of 4 with at
# most 32 output channels -> four.  The last three have more voxel tiles
# than one wave of CTAs holds (one, two and four planes; two, three and
# four input chunks with one pipeline stage per CTA).
@pytest.mark.parametrize("shape,cin,cout", [((5, 6, 7), 16, 16), ((8, 8, 8), 32, 48),
                                            ((9, 4, 10), 112, 48), ((16, 16, 3), 48, 64),
                                            ((3, 3, 3), 16, 32), ((7, 9, 12), 48, 16),
                                            ((8, 16, 8), 16, 32), ((48, 48, 13), 64, 32),
                                            ((64, 64, 12), 48, 48), ((64, 64, 24), 32, 16)])
@pytest.mark.parametrize("relu,flip", [(0, 0), (1, 0), (0, 1)])
def test_tensor_core_conv_matches_references(built, shape, cin, cout, relu, flip):
    rng = np.random.default_rng(cin * 7 + cout + relu + 3 * flip)
    nv = int(np.prod(shape))
    x16 = to_bf16(rng.normal(size=(nv, cin)))
    w16 = to_bf16(rng.normal(size=(cout, 27 * cin)) * 0.1)
    bias = rng.normal(size=cout).astype(np.float32)
    ref = np_conv(from_bf16(x16), from_bf16(w16), bias, shape, relu, flip)
    y_tc = run(shape, cin, cout, relu, flip, 1, x16, w16, bias)
    y_cc = run(shape, cin, cout, relu, flip, 0, x16, w16, bias)
    scale = np.abs(ref).max()
    assert np.abs(y_cc - ref).max() <= 1e-5 * scale
    assert np.abs(y_tc - ref).max() <= 1e-5 * scale
