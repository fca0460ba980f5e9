"""Geometry front end on the GPU (LevelSet_3D.f90:80-150) through the C-ABI,
bit-exact against the oracle: Allen-Cahn pre-smoothing, the stacked field
with tunnels, and whole frames (stack, Allen-Cahn, sign, reinitialisation)."""
import numpy as np
import pytest

from oracle import sbm_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sbm():
    from elsim_gb300 import sbm as m

    m.load_library()
    return m


def _field(shape, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.uniform(-0.2, 1.2, size=tuple(s + 2 for s in shape)))


@pytest.mark.parametrize("shape,iters", [((13, 9, 7), 0), ((13, 9, 7), 1), ((33, 17, 5), 17),
                                         ((64, 40, 24), 50), ((1, 1, 1), 3)])
def test_allen_cahn(sbm, shape, iters):
    f = _field(shape, 10 + iters)
    assert np.array_equal(sbm.allen_cahn(iters, f), orc.allen_cahn(iters, f))


GEOMETRIES = [
    # (voxel shape, yg, zg, xoff, nthick, tr)
    ((12, 14, 5), 7, 9, 3, 4, 2.5),
    ((40, 52, 17), 31, 48, 5, 4, float(np.float32(12.764))),
    ((33, 30, 21), 33, 30, 0, 1, 9.0),
    ((20, 25, 6), 9, 11, 2, 3, 0.0),
]


@pytest.mark.parametrize("g", GEOMETRIES)
def test_geometry(sbm, g):
    shape, yg, zg, xoff, nthick, tr = g
    vox = np.asfortranarray(np.random.default_rng(sum(shape)).uniform(0.0, 1.0, size=shape))
    got = sbm.ls_geometry(vox, yg, zg, xoff, nthick, tr)
    assert np.array_equal(got, orc.ls_geometry(vox, yg, zg, xoff, nthick, tr))


def test_geometry_rejects_out_of_range(sbm):
    vox = np.zeros((12, 14, 5), order="F")
    with pytest.raises(sbm.SbmError):
        sbm.ls_geometry(vox, 13, 9, 3, 4, 1.0)  # yg > yo
    with pytest.raises(sbm.SbmError):
        sbm.ls_geometry(vox, 7, 9, 3, 30, 1.0)  # tunnel loop leaves TmpB


@pytest.mark.parametrize("ac,lit", [(50, 175), (0, 7), (3, 0)])
def test_frame(sbm, ac, lit):
    from elsim_gb300 import geometry

    vox = geometry.synthetic_voxels((48, 60, 20), seed=ac + lit, blob=2.0)
    args = (37, 44, 6, 4, float(geometry.TUNNEL_RADII[4]))
    got = sbm.ls_frontend(vox, *args, ac_iters=ac, lit=lit)
    want = orc.ls_frontend(vox, *args, ac_iters=ac, lit=lit)
    assert np.array_equal(got, want)


def test_frame_file(sbm, tmp_path):
    from elsim_gb300 import fortran_io, geometry

    vox = geometry.synthetic_voxels((30, 40, 12), seed=5, blob=2.0)
    kw = {"yg": 21, "zg": 33, "xoff": 4, "nthick": 4, "ac_iters": 10, "lit": 30}
    (path,) = geometry.run(vox, frames=[5], directory=tmp_path, **kw)
    assert path.name == "L24Z1005.dat"
    d = fortran_io.read_array(path, np.float64, (21, 4 + 4 * 12, 33))
    want = orc.ls_frontend(vox, 21, 33, 4, 4, geometry.TUNNEL_RADII[5], 10, 30)
    assert np.array_equal(d, want[1:-1, 1:-1, 1:-1])
