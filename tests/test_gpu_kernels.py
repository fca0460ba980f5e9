"""GPU parity of the bit-exact kernels against the oracle, through the C-ABI.

ReDist3D_XYZ, the AccDiff sweep, the RM mask, the sign function and
Tbl_Chk_Pln_3DA must match the oracle bit for bit (integer/compare-heavy
FP64 work with every operation IEEE round-to-nearest and no contraction).
"""
import numpy as np
import pytest

from elsim_gb300 import sbm, synth
from oracle import sbm_oracle as orc

pytestmark = pytest.mark.gpu

SHAPES = [(24, 24, 24), (33, 17, 20), (1, 5, 3), (64, 8, 9)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("lit,dt", [(1, 1.0e-1), (20, 1.0e-1), (175, float(np.float32(0.1)))])
def test_redist_bit_exact(built, shape, lit, dt):
    solid = synth.spheres(shape, seed=11, solid_fraction=0.5, rmin=2, rmax=5)
    sg = synth.sign_field(solid)
    f0 = np.zeros_like(sg)
    got = sbm.redist3d_xyz(lit, sg, f0, dt)
    ref = orc.redist(lit, sg, f0, dt)
    assert np.array_equal(got, ref)


def test_redist_zero_sign_and_nonzero_start(built):
    rng = np.random.default_rng(5)
    sg = rng.choice([-1.0, 0.0, 1.0], size=(12, 14, 10))
    f0 = rng.normal(size=(12, 14, 10))
    got = sbm.redist3d_xyz(7, sg, f0, 1.0e-1)
    ref = orc.redist(7, sg, f0, 1.0e-1)
    assert np.array_equal(got, ref)


def _psi(shape, seed):
    m = synth.microstructure(shape, seed=seed, solid_fraction=0.55, reinit_steps=30,
                             redist=orc.redist)
    # AccDiff_3D.f90:84 uses width 0.75 on the distance
    return np.asfortranarray(0.5 * (1.0 + np.tanh(m["dist"] / 0.75)))


@pytest.mark.parametrize("shape", [(20, 24, 18), (7, 31, 5)])
@pytest.mark.parametrize("dirichlet_x", [1, 0])
@pytest.mark.parametrize("term", [2, 6, 300])
def test_accdiff_bit_exact(built, shape, dirichlet_x, term):
    psi = _psi(shape, 21)
    if dirichlet_x == 0:
        psi = psi.copy(order="F")
        psi[1:-1, 1:-1, 1:-1] = 1.0 - psi[1:-1, 1:-1, 1:-1]  # AccDiff_3D.f90:175 (ghosts kept)
    cn0 = np.zeros_like(psi)
    got = sbm.accdiff(psi, cn0, term, dirichlet_x)
    ref = orc.accdiff(psi, cn0, term, dirichlet_x)
    assert np.array_equal(got, ref)


def test_accdiff_full_length_and_nonzero_start(built):
    psi = _psi((16, 20, 12), 4)
    cn0 = np.asfortranarray(np.random.default_rng(1).uniform(0, 1, psi.shape))
    got = sbm.accdiff(psi, cn0, 1501, 1)
    ref = orc.accdiff(psi, cn0, 1501, 1)
    assert np.array_equal(got, ref)


def test_rm_mask_and_sign_bit_exact(built):
    rng = np.random.default_rng(2)
    psa = rng.uniform(0, 1, 5000)
    cn = np.concatenate([rng.uniform(0, 2e-4, 4990),
                         [np.float32(1e-4), 1e-4, 0.0, -0.0, 1.0, 2e-4, 9.99e-5, 1.0000001e-4,
                          np.nextafter(float(np.float32(1e-4)), 0), float(np.float32(1e-4))]])
    assert np.array_equal(sbm.rm_mask(psa, cn), orc.rm_mask(psa, cn))
    ds = np.concatenate([rng.uniform(-1, 2, 4995), [0.5, np.nextafter(0.5, 1), 0.0, -0.0, 1.0]])
    assert np.array_equal(sbm.sign(ds, 0.5), orc.sign(ds, 0.5))
    assert sbm.rm_mask(np.zeros(0), np.zeros(0)).size == 0


@pytest.mark.parametrize("seed", [0, 1])
def test_table_bit_exact(built, seed):
    rng = np.random.default_rng(seed)
    x = np.arange(101) * 0.01
    v = np.cumsum(rng.normal(size=101))
    c = np.concatenate([rng.uniform(-0.2, 1.2, 20000), x, [0.0, 1.0, -1e-300, 1e-6, 0.999999999,
                                                           0.005, 1.5, -3.0]])
    got = sbm.tbl_chk_pln_3da(x, v, c)
    ref = orc.table(x, v, c)
    assert np.array_equal(got, ref)


def test_table_one_segment_left_quirk(built):
    # c = 0.015 floors to lb = 1 -> segment [X(1), X(2)] = [0, 0.01], i.e. the
    # value is extrapolated from the left segment (SBMES:1013-1021)
    x = np.arange(101) * 0.01
    v = (x ** 2)
    got = sbm.tbl_chk_pln_3da(x, v, np.array([0.015, 0.5]))
    assert got[0] == v[0] + (0.015 - x[0]) / 0.01 * (v[1] - v[0])
    lb = int(np.floor(0.5 / 0.01))
    assert got[1] == v[lb - 1] + (0.5 - x[lb - 1]) / 0.01 * (v[lb] - v[lb - 1])


def test_bad_arguments_are_errors(built):
    with pytest.raises(sbm.SbmError) as e:
        sbm.accdiff(np.zeros((3, 3, 3)), np.zeros((3, 3, 3)), 10, 2)
    assert e.value.code == sbm.ERR_ARG
    with pytest.raises(sbm.SbmError):
        sbm.Context(0, 4, 4)
