"""Geometry front end (LevelSet_3D.f90:61-150) on the CPU: the oracle's
literal restatement of the stacking and tunnel loops against independent
restatements here, and the host side of elsim_gb300.geometry."""
import numpy as np
import pytest

from oracle import sbm_oracle as orc

# small sizes that keep the reference's shape: xg = xoff + 4*zo well above
# zo, so the tunnel loop writes past TmpB's second extent
SMALL = {"yg": 7, "zg": 9, "xoff": 3, "nthick": 4}
VOX = (12, 14, 5)


def _vox(shape=VOX, seed=0):
    return np.asfortranarray(np.random.default_rng(seed).uniform(0.1, 1.0, size=shape))


def _interior(a):
    return a[1:-1, 1:-1, 1:-1]


def _literal(vox, yg, zg, xoff, nthick, tr, alias=True):
    """LevelSet_3D.f90:80-119 as plain loops over a flat column-major TmpB."""
    yo, xo, zo = vox.shape
    xg = xoff + nthick * zo
    flat = np.zeros(yo * zo * xo)
    for k in range(1, zo + 1):
        for j in range(1, xo + 1):
            for i in range(1, yo + 1):
                flat[(i - 1) + yo * ((k - 1) + zo * (j - 1))] = vox[i - 1, j - 1, zo - k]
    for k in range(1, zg + 1):
        for j in range(1, (xg if alias else zo) + 1):
            for i in range(1, yg + 1):
                at = (i - 1) + yo * ((j - 1) + zo * (k - 1))
                if np.sqrt((i - 1.0) ** 2 + (k - float(zg)) ** 2) < tr:
                    flat[at] = 0.0
                if np.sqrt((i - float(yg)) ** 2 + (k - 1.0) ** 2) < tr:
                    flat[at] = 0.0
    tb = flat.reshape((yo, zo, xo), order="F")
    ds = np.zeros((yg, xg, zg))
    for j in range(xoff + 1, xg + 1):
        t, r = divmod(j - xoff - 1, zo)
        c = r + 1 if t % 2 == 0 else zo - r
        ds[:, j - 1, :] = tb[:yg, c - 1, :zg]
    return ds


def test_stack_without_tunnels():
    vox = _vox()
    ds = orc.ls_geometry(vox, tr=0.0, **SMALL)
    yg, zg, xoff = SMALL["yg"], SMALL["zg"], SMALL["xoff"]
    tmpb = vox[:, :, ::-1].transpose(0, 2, 1)  # TmpB(i,k,j) = TmpA(i,j,zo-k+1)
    straight = tmpb[:yg, :, :zg]
    want = np.concatenate([np.zeros((yg, xoff, zg)), straight, straight[:, ::-1],
                           straight, straight[:, ::-1]], axis=1)
    assert np.array_equal(_interior(ds), want)


@pytest.mark.parametrize("tr", [1.0, 2.5, np.float64(np.float32(3.7)), 6.0])
def test_tunnels_follow_the_reference_loop(tr):
    vox = _vox(seed=1)
    ds = orc.ls_geometry(vox, tr=tr, **SMALL)
    want = _literal(vox, tr=tr, **SMALL)
    assert np.array_equal(_interior(ds), want)
    # the writes past TmpB's second extent change the result
    if tr >= 2.5:
        assert not np.array_equal(want, _literal(vox, tr=tr, alias=False, **SMALL))


def test_ghosts_are_zero_gradient():
    ds = orc.ls_geometry(_vox(seed=2), tr=2.0, **SMALL)
    ref = ds.copy()
    orc.nogrdbc(ref)
    assert np.array_equal(ds, ref)


@pytest.mark.parametrize("bad", [{"yg": 13}, {"zg": 15}, {"nthick": 30}])
def test_out_of_range(bad):
    args = dict(SMALL, **bad)
    with pytest.raises(ValueError):
        orc.ls_geometry(_vox(), tr=1.0, **args)


def test_reference_sizes_stay_inside_tmpb():
    from elsim_gb300.geometry import REFERENCE as R

    xg = R["xoff"] + R["nthick"] * R["zo"]
    assert xg == 170 * 4 + 50
    assert (xg - 1) + R["zo"] * (R["zg"] - 1) < R["zo"] * R["xo"]


def test_tunnel_radii_are_real4():
    from elsim_gb300.geometry import TUNNEL_RADII

    assert TUNNEL_RADII.dtype == np.float64 and TUNNEL_RADII.shape == (14,)
    assert TUNNEL_RADII[1] == float(np.float32(6.3826)) and TUNNEL_RADII[1] != 6.3826
    assert TUNNEL_RADII[0] == 0.0


def test_read_voxels(tmp_path):
    from elsim_gb300.geometry import read_voxels

    vox = _vox((3, 4, 2), seed=3)
    p = tmp_path / "a.txt"
    vals = vox.ravel(order="F")
    p.write_text(" ".join(f"{v:.17g}" for v in vals[:10]) + "\n" +
                 ",".join(f"{v:.17g}" for v in vals[10:]) + "\n")
    assert np.array_equal(read_voxels(p, 3, 4, 2), vox)
    q = tmp_path / "b.txt"
    q.write_text("5*1.0 2*0 1.5D0,\n 1 1 1 1 1 1 1 1 1 1 1 1 1 1 1 9 / 7 7")
    got = read_voxels(q, 3, 4, 2).ravel(order="F")
    assert np.array_equal(got[:8], [1, 1, 1, 1, 1, 0, 0, 1.5]) and got[-1] == 9
    with pytest.raises(ValueError):
        read_voxels(q, 3, 4, 3)


def test_frontend_oracle_signs():
    # after the front end the distance is positive where the smoothed field
    # exceeded 0.5 and negative elsewhere
    vox = (_vox(seed=4) > 0.5).astype(np.float64)
    d = orc.ls_frontend(vox, tr=2.0, ac_iters=5, lit=20, **SMALL)
    sm = orc.allen_cahn(5, orc.ls_geometry(vox, tr=2.0, **SMALL))
    assert np.array_equal(d > 0, sm > 0.5)


def _slab_and_ball(shape=(20, 28, 16)):
    """Interior distance-like field: +2 in a solid slab touching the x = px+1
    face and in an isolated ball, -2 elsewhere."""
    ny, nx, nz = shape
    i, j, k = np.meshgrid(np.arange(ny), np.arange(nx), np.arange(nz), indexing="ij")
    slab = j >= nx - 6
    ball = (i - ny / 2) ** 2 + (j - nx / 3) ** 2 + (k - nz / 2) ** 2 <= 16
    return np.asfortranarray(np.where(slab | ball, 2.0, -2.0)), slab, ball


def test_connectivity_removes_isolated_solid():
    # AccDiff_3D + RM_UCNCT_3D: the ball has no path to the solid's Dirichlet
    # face, so its Cn stays 0 and the solid distance drops it; the slab keeps
    # Cn = 1 and stays solid; the electrolyte (Dirichlet face x = 0) is one
    # connected region and keeps its sign
    d, slab, ball = _slab_and_ball()
    cs, ce = orc.connectivity(d, 0.75, 1501)
    i = (slice(1, -1),) * 3
    assert cs[i][ball].max() < 1e-4 and cs[i][slab].min() == 1.0
    elec = ~(slab | ball)
    assert ce[i][elec].min() > 1e-4
    ds, de = orc.rm_ucnct(d, cs[i], ce[i], lit=40)
    assert (ds[i][ball] < 0).all() and (ds[i][slab] > 0).all()
    assert np.array_equal(de[i] > 0, elec)
