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


def _frame_distance(shape=(40, 52, 14), seed=11):
    from elsim_gb300 import geometry

    vox = geometry.synthetic_voxels(shape, seed=seed, blob=1.5)
    ds = orc.ls_frontend(vox, 23, 37, 4, 4, float(geometry.TUNNEL_RADII[3]), 20, 60)
    return np.asfortranarray(ds[1:-1, 1:-1, 1:-1])


def test_connectivity_program(sbm):
    d = _frame_distance()
    got = sbm.connectivity(d, 0.75, 1501)
    want = orc.connectivity(d, 0.75, 1501)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_rm_ucnct_program(sbm):
    d = _frame_distance(seed=12)
    cs, ce = orc.connectivity(d, 0.75, 1501)
    i = (slice(1, -1),) * 3
    # the structure has disconnected pieces in at least one phase
    psa = 0.5 * (1.0 + np.tanh(d))
    assert ((cs[i] < 1e-4) & (psa > 0.5)).any() or ((ce[i] < 1e-4) & (psa < 0.5)).any()
    got = sbm.rm_ucnct(d, cs[i], ce[i], 175)
    want = orc.rm_ucnct(d, cs[i], ce[i], 175)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_geometry_chain(sbm):
    from elsim_gb300 import geometry

    d = _frame_distance(seed=13)
    ds, de, cs, ce = geometry.connected(d, term=301, lit=50)
    wcs, wce = orc.connectivity(d, 0.75, 301)
    i = (slice(1, -1),) * 3
    wds, wde = orc.rm_ucnct(d, wcs[i], wce[i], 50)
    assert np.array_equal(cs, wcs[i]) and np.array_equal(ce, wce[i])
    assert np.array_equal(ds, wds[i]) and np.array_equal(de, wde[i])
