"""The reference's cell program -- the time loop of the SBMES main program
(SBMES:351-877) -- as a host loop over the C-ABI.

`sbm_time_step` runs one pass of the loop body on the GPU (Cahn-Hilliard,
the CnE solve, the Butler-Volmer Picard loop, the voltage control); this
module keeps what the reference's host does around it, REAL(4) literals
and all:

* the loop runs while Xrf < 0.971 (SBMES:357), from sCrnt = trgI, cnt = 1,
  iter = 1, tm = 0 (SBMES:339-355);
* each step's dt and voltage scan rate come from the Li fraction and the
  current error |trgI - sCrnt| left by the previous step
  (`synth.step_schedule`, SBMES:360-383); tm accumulates dt (SBMES:840);
* after a step with Xrf > 0.02 + (cnt-1)*0.005 (evaluated in REAL(4)):
  every rank's block of CnP, CnE, phP and phE when MOD(cnt,10) == 1
  (OutPut3D_A, files CP/CE/PP/PE//I4(1000+rank)//I4(1000+cnt)//'.dat'), a
  ReC_TmFX line, then cnt = cnt + 1 (SBMES:842-859);
* the loop ends after a step with BvE >= BvP + 0.005 or Xrf > 0.97, with a
  ReC_TmFX line and the four dumps of frame cnt (SBMES:861-873).

`write_setup` writes the set-up dumps PS and PL (SBMES:348-349).  Files go
to `directory` through elsim_gb300.fortran_io (the per-rank blocks of an
rnb x cnb decomposition, as the combine program reads them); with
directory=None nothing is written and only the event log is returned.
"""
from __future__ import annotations

import numpy as np

from . import fortran_io, sbm, synth

_F4 = lambda v: float(np.float32(v))  # a REAL(4) literal promoted to REAL(8)
BVP = _F4(-0.1)  # the particle potential's boundary value (SBMES:106)
DUMPS = (("CP", sbm.F_CNP), ("CE", sbm.F_CNE), ("PP", sbm.F_PHP), ("PE", sbm.F_PHE))


def _output_threshold(cnt: int) -> float:
    """0.02 + (cnt-1)*0.005 as the reference evaluates it: INTEGER times a
    REAL(4) literal, plus a REAL(4) literal, all in REAL(4)."""
    return float(np.float32(np.float32(0.02) + np.float32(cnt - 1) * np.float32(0.005)))


def write_setup(ctx, directory, rnb: int = 1, cnb: int = 1) -> None:
    """The set-up dumps of psP and psE, frame 1 (SBMES:348-349)."""
    for pred, fid in (("PS", sbm.F_PSP), ("PL", sbm.F_PSE)):
        fortran_io.write_rank_outputs(1, pred, ctx.download(fid, haloed=False), rnb, cnb,
                                      directory)


def run(ctx, max_steps: int | None = None, directory=None, outpf: str = "GBQ105",
        rnb: int = 1, cnb: int = 1, bvp: float = BVP, precision=sbm.PREC_FP64) -> dict:
    """Runs the reference's time loop on a context whose domain is set up
    (`Context.setup_domain`).  Returns the step count, tm, cnt, why the loop
    ended ("xrf" when Xrf reached 0.971, "stop" for the BvE / Xrf condition,
    "max_steps") and the event log: ("step", iter, dt, vsr), ("dump", pred,
    frame, iter) and ("tmfx", frame, iter, tm, Xrf, sCrnt, trgI, BvE)."""
    s = ctx.scalars()
    tm, cnt, it = 0.0, 1, 1
    events = []
    why = "xrf"

    def dump(frame):
        for pred, fid in DUMPS:
            events.append(("dump", pred, frame, it))
            if directory is not None:
                fortran_io.write_rank_outputs(frame, pred, ctx.download(fid, haloed=False), rnb,
                                              cnb, directory)

    def tmfx(frame):
        rec = (frame, it, tm, s["xrf"], s["scrnt"], s["trgI"], s["bve"])
        events.append(("tmfx",) + rec)
        if directory is not None:
            fortran_io.rec_tmfx(frame, outpf, it, *rec[2:], directory=directory)

    while s["xrf"] < _F4(0.971):
        if max_steps is not None and it > max_steps:
            why = "max_steps"
            break
        dt, vsr = synth.step_schedule(s["xrf"], abs(s["trgI"] - s["scrnt"]), s["trgI"])
        events.append(("step", it, dt, vsr))
        s = ctx.time_step(it, dt, vsr, precision=precision)
        tm = tm + dt
        if s["xrf"] > _output_threshold(cnt):
            if cnt % 10 == 1:
                dump(cnt)
            tmfx(cnt)
            cnt = cnt + 1
        if s["bve"] >= bvp + _F4(0.005) or s["xrf"] > _F4(0.97):
            tmfx(cnt)
            dump(cnt)
            why = "stop"
            break
        it = it + 1
    return dict(iter=it, tm=tm, cnt=cnt, why=why, events=events, scalars=s)
