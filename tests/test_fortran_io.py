"""The reference's file formats (elsim_gb300/fortran_io.py): record layout of
gfortran unformatted sequential files at the byte level, the distance input,
the per-rank dumps and the combine program's global file, the rank
decomposition (known answers for the production grid) and the TmFx log."""
import numpy as np
import pytest

from elsim_gb300 import fortran_io as fio


def test_record_bytes(tmp_path):
    a = np.arange(24, dtype=np.float32).reshape(2, 3, 4, order="F")
    p = fio.write_distance(tmp_path / "d.dat", a, double=False)
    raw = p.read_bytes()
    assert len(raw) == 4 + 96 + 4
    assert raw[:4] == (96).to_bytes(4, "little") and raw[-4:] == raw[:4]
    # Fortran order: the first index runs fastest
    vals = np.frombuffer(raw[4:-4], "<f4")
    assert vals[1] == a[1, 0, 0] and vals[2] == a[0, 1, 0] and vals[6] == a[0, 0, 1]


def test_distance_round_trip_and_mode_2(tmp_path):
    rng = np.random.default_rng(1)
    d = np.asfortranarray(rng.normal(size=(5, 7, 3)).astype(np.float32))
    fio.write_distance(tmp_path / "s.dat", d, double=False)
    assert np.array_equal(fio.read_distance(tmp_path / "s.dat", 5, 7, 3), d)
    fio.write_distance(tmp_path / "d.dat", d.astype(np.float64), double=True)
    assert np.array_equal(fio.read_array(tmp_path / "d.dat", np.float64, (5, 7, 3)), d)
    with pytest.raises(ValueError):
        fio.read_distance(tmp_path / "s.dat", 5, 7, 4)


def test_bad_markers_are_rejected(tmp_path):
    p = tmp_path / "bad.dat"
    p.write_bytes((8).to_bytes(4, "little") + b"\0" * 8 + (9).to_bytes(4, "little"))
    with pytest.raises(ValueError):
        fio.read_records(p)


def test_output3d_a_name_and_content(tmp_path):
    a = np.linspace(0, 1, 60).reshape(3, 4, 5)
    p = fio.output3d_a(7, "CP1003", a, tmp_path)
    assert p.name == "CP10031007.dat"
    assert np.array_equal(fio.read_array(p, np.float32, a.shape), a.astype(np.float32))
    t = fio.output3d_a(7, "CP1003", a, tmp_path, mode=1)
    assert t.name == "CP10031007.txt"
    assert np.array_equal(np.loadtxt(t).astype(np.float32), a.astype(np.float32).ravel(order="F"))


def test_rank_decomposition_production_grid():
    # gy = 186, gz = 320 on rnb = 12 z blocks x cnb = 16 y blocks
    idx = fio.rank_decomposition(186, 320, 12, 16)
    assert idx.shape == (192, 6)
    # 320 = 12 * 26 + 8: the first 8 z blocks hold 27 planes
    assert tuple(idx[0]) == (1, 12, 12, 1, 27, 27)
    assert tuple(idx[7][3:]) == (190, 216, 27) and tuple(idx[8][3:]) == (217, 242, 26)
    assert tuple(idx[11][3:]) == (295, 320, 26)
    # 186 = 16 * 11 + 10: the first 10 y blocks hold 12 columns; rank -> y block rank // 12
    assert tuple(idx[12 * 9][:3]) == (109, 120, 12) and tuple(idx[12 * 10][:3]) == (121, 131, 11)
    assert tuple(idx[191][:3]) == (176, 186, 11)
    # the blocks tile the domain exactly once
    cover = np.zeros((186, 320), dtype=int)
    for lwy, upy, ny, lwz, upz, nz in idx:
        assert upy - lwy + 1 == ny and upz - lwz + 1 == nz
        cover[lwy - 1:upy, lwz - 1:upz] += 1
    assert (cover == 1).all()


def test_rank_dumps_combine_to_the_global_field(tmp_path):
    rng = np.random.default_rng(2)
    g = np.asfortranarray(rng.normal(size=(13, 6, 11)))
    paths = fio.write_rank_outputs(135, "CP", g, rnb=3, cnb=4, directory=tmp_path)
    assert [p.name for p in paths[:2]] == ["CP10001135.dat", "CP10011135.dat"]
    und, path = fio.combine(135, "CP", 13, 6, 11, rnb=3, cnb=4, directory=tmp_path)
    assert path.name == "CPASMB1135.dat"
    assert np.array_equal(und, g.astype(np.float32))
    assert np.array_equal(fio.read_array(path, np.float32, g.shape), g.astype(np.float32))


def test_tmfx_log(tmp_path):
    fio.rec_tmfx(1, "GBQ105", 10, 0.5, 0.02, 1.5e-3, -2e-3, 0.1, tmp_path)
    fio.rec_tmfx(2, "GBQ105", 20, 1.0, 0.025, 1.6e-3, -2e-3, 0.11, tmp_path)
    rows = fio.read_tmfx(tmp_path / "GBQ105TmFx.txt")
    assert rows.shape == (2, 7)
    assert rows[1].tolist() == [2, 20, 1.0, 0.025, 1.6e-3, -2e-3, 0.11]
    fio.rec_tmfx(1, "GBQ105", 5, 0.1, 0.0, 0.0, 0.0, 0.0, tmp_path)  # frame 1 restarts
    assert fio.read_tmfx(tmp_path / "GBQ105TmFx.txt").shape == (1, 7)
