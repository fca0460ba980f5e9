"""The allocation-free ReDist3D_XYZ entry point, through the C-ABI.

sbm_redist_noalloc serves callers that cannot allocate device memory -- a
host program whose GPU memory is all owned by another allocator or
framework, or one held to a fixed memory budget: the caller passes device
buffers and the library's only scratch is a fixed array built into it.  Its
output must equal the allocating entry point's (sbm_redist) bit for bit --
the tolerance every reinitialisation test here uses -- on two calls in a
row, so the scratch that the first call leaves behind cannot leak into the
second.  This file is collected last on purpose.
"""
import numpy as np
import pytest

from elsim_gb300 import sbm, synth

pytestmark = pytest.mark.gpu


def _noalloc(lit, sg, f0, dt):
    import torch
    lib = sbm.load_library()
    d_sg = torch.from_numpy(np.ascontiguousarray(sg.ravel(order="F"))).cuda()
    d_f = torch.from_numpy(np.ascontiguousarray(f0.ravel(order="F"))).cuda()
    torch.cuda.synchronize()
    py, px, pz = (s - 2 for s in sg.shape)
    rc = lib.sbm_redist_noalloc(lit, py, px, pz, dt, d_sg.data_ptr(), d_f.data_ptr(), None)
    assert rc == sbm.OK, lib.sbm_last_error()
    return d_f.cpu().numpy().reshape(sg.shape, order="F")


def test_noalloc_redist_equals_allocating_entry_point_twice(built):
    # first call: a sphere packing, odd iteration count (result lands in the scratch)
    sg1 = synth.sign_field(synth.spheres((30, 26, 22), seed=2, solid_fraction=0.5, rmin=2, rmax=5))
    f1 = np.zeros_like(sg1)
    got1 = _noalloc(33, sg1, f1, 1.0e-1)
    assert np.array_equal(got1, sbm.redist3d_xyz(33, sg1, f1, 1.0e-1))
    # second call right after: other shape, non-zero start, REAL(4) dt, even count
    sg2 = synth.sign_field(synth.spheres((17, 40, 12), seed=9, solid_fraction=0.4, rmin=2, rmax=4))
    f2 = np.asfortranarray(np.random.default_rng(7).normal(size=sg2.shape))
    dt = float(np.float32(0.1))
    got2 = _noalloc(20, sg2, f2, dt)
    assert np.array_equal(got2, sbm.redist3d_xyz(20, sg2, f2, dt))


def test_noalloc_fills_the_whole_scratch(built):
    # (126+2)(126+2)(62+2) = 2^20 padded cells: exactly the scratch's size; an
    # odd iteration count leaves the result in the scratch before the copy back
    shape = (126, 126, 62)
    assert (shape[0] + 2) * (shape[1] + 2) * (shape[2] + 2) == 1 << 20
    sg = synth.sign_field(synth.spheres(shape, seed=4, solid_fraction=0.5, rmin=3, rmax=8))
    f0 = np.zeros_like(sg)
    for _ in range(2):
        got = _noalloc(7, sg, f0, 1.0e-1)
        assert np.array_equal(got, sbm.redist3d_xyz(7, sg, f0, 1.0e-1))


def test_noalloc_rejects_grid_beyond_scratch(built):
    import torch
    lib = sbm.load_library()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    n = 128  # (n+2)^3 padded cells > SBM_NOALLOC_REDIST_MAX_CELLS
    assert (n + 2) ** 3 > (1 << 20)
    rc = lib.sbm_redist_noalloc(1, n, n, n, 0.1, buf.data_ptr(), buf.data_ptr(), None)
    assert rc == sbm.ERR_ARG
    assert b"scratch" in lib.sbm_last_error()
    # a thin grid within the cell limit whose z extent the launch grid cannot hold
    rc = lib.sbm_redist_noalloc(1, 1, 1, 70000, 0.1, buf.data_ptr(), buf.data_ptr(), None)
    assert rc == sbm.ERR_ARG
    assert b"65535" in lib.sbm_last_error()
    # extents whose padded sizes overflow 32-bit arithmetic
    big = 2 ** 31 - 2
    rc = lib.sbm_redist_noalloc(1, big, big, big, 0.1, buf.data_ptr(), buf.data_ptr(), None)
    assert rc == sbm.ERR_ARG
    assert not buf.cpu().numpy().any()
