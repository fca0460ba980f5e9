"""elsim_gb300.cell on the host: a bounded run, and the per-rank dumps of a
decomposed run reassembled by the combine program's restatement.  CPU only
(a stand-in context; the loop control itself is checked against the
reference in tests/test_oracle_reference.py)."""
import numpy as np

from elsim_gb300 import cell, sbm
from elsim_gb300 import fortran_io as fio

SHAPE = (9, 11, 7)


class _Ctx:
    """Xrf rising 0.003 per step from 0.0202, a constant current error and
    BvE far from the stop condition; each field a distinct ramp."""

    def __init__(self):
        self.s = dict(xrf=0.0202, scrnt=0.017, trgI=0.018, bve=-0.4495)
        self.k = 0

    def scalars(self):
        return dict(self.s)

    def time_step(self, it, dt, vsr, precision=0):
        self.k = it
        self.s["xrf"] = 0.0202 + 0.003 * it
        return dict(self.s)

    def download(self, fid, haloed=True):
        n = int(np.prod(SHAPE))
        return np.asfortranarray((np.arange(n, dtype=np.float64) + 1000.0 * fid)
                                 .reshape(SHAPE, order="F"))


def test_bounded_run_stops_and_reports(tmp_path):
    res = cell.run(_Ctx(), max_steps=5, directory=None)
    assert res["why"] == "max_steps" and res["iter"] == 6
    assert [e[1] for e in res["events"] if e[0] == "step"] == [1, 2, 3, 4, 5]
    assert not list(tmp_path.iterdir())


def test_rank_dumps_combine_to_the_fields(tmp_path):
    rnb, cnb = 3, 2
    ctx = _Ctx()
    cell.write_setup(ctx, tmp_path, rnb, cnb)
    res = cell.run(ctx, max_steps=3, directory=tmp_path, rnb=rnb, cnb=cnb)
    dumps = [e for e in res["events"] if e[0] == "dump"]
    assert {(e[1], e[2]) for e in dumps} == {(p, 1) for p in ("CP", "CE", "PP", "PE")}
    gy, gx, gz = SHAPE
    for pred, fid in (("PS", sbm.F_PSP), ("CP", sbm.F_CNP), ("PE", sbm.F_PHE)):
        assert len(list(tmp_path.glob(f"{pred}10??1001.dat"))) == rnb * cnb
        und, _ = fio.combine(1, pred, gy, gx, gz, rnb, cnb, tmp_path)
        assert np.array_equal(und, ctx.download(fid).astype(np.float32))
    rows = fio.read_tmfx(tmp_path / "GBQ105TmFx.txt")
    assert rows.shape[0] == sum(1 for e in res["events"] if e[0] == "tmfx") > 0
