"""File formats of the reference program, on the host.

The reference (SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90, SBMES below;
LevelSet_3D.f90; SBMES_3D_Cmbn_MPI_v2.f90, Cmbn below) reads and writes
gfortran *unformatted sequential* files: every WRITE is one record framed
by a 4-byte little-endian length marker before and after the payload; the
arrays are stored in Fortran (column-major) order.  This module writes and
reads exactly those records, so its files and the reference's are
interchangeable:

* ``read_distance``   -- the REAL(4) distance input, SBMES:148-151 / 180-186;
* ``write_distance``  -- LevelSet_3D.f90 OutPut3D, modes 2 (REAL(8)) and 3 (REAL(4));
* ``output3d_a``      -- SBMES:892-919 (per-rank field dumps, REAL(4));
* ``rank_decomposition`` -- MyDmnCmpn_YZ, SBMES:947-982 (= Cmbn:27-67);
* ``write_rank_outputs`` / ``combine`` -- the per-rank dumps the MPI program
  writes for a decomposition, and the combine program's global
  ``<pred>ASMB`` file (Cmbn:75-129);
* ``rec_tmfx``        -- the time / fraction / current log, SBMES:922-943.

Records larger than 2**31 - 1 bytes (gfortran splits those into
subrecords) are rejected.  The list-directed text variants (OutPut3D_A
mode 1, the TmFx log) are written value-compatible -- whitespace-separated
values that a list-directed READ accepts -- not byte-identical, since the
spacing of list-directed output is compiler-specific.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

_MAX_RECORD = 2**31 - 1


def write_record(f, a: np.ndarray) -> None:
    """One unformatted sequential record of `a` in Fortran order."""
    data = np.asfortranarray(a).tobytes(order="F")
    if len(data) > _MAX_RECORD:
        raise ValueError("record larger than 2**31 - 1 bytes (gfortran subrecords not written)")
    marker = np.int32(len(data)).astype("<i4").tobytes()
    f.write(marker)
    f.write(data)
    f.write(marker)


def read_records(path) -> list[bytes]:
    """Payloads of every record of an unformatted sequential file."""
    raw = Path(path).read_bytes()
    out, pos = [], 0
    while pos < len(raw):
        if pos + 4 > len(raw):
            raise ValueError("truncated record marker")
        n = int(np.frombuffer(raw[pos:pos + 4], "<i4")[0])
        if n < 0:
            raise ValueError("gfortran subrecords are not supported")
        end = pos + 4 + n
        if end + 4 > len(raw) or raw[end:end + 4] != raw[pos:pos + 4]:
            raise ValueError("record markers do not match")
        out.append(raw[pos + 4:end])
        pos = end + 4
    return out


def read_array(path, dtype, shape, record: int = 0) -> np.ndarray:
    """Record `record` of a file as an array of `shape` (Fortran order)."""
    rec = read_records(path)[record]
    need = int(np.prod(shape)) * np.dtype(dtype).itemsize
    if len(rec) != need:
        raise ValueError(f"record holds {len(rec)} bytes, {need} expected for {shape}")
    return np.frombuffer(rec, dtype=np.dtype(dtype).newbyteorder("<")).reshape(shape, order="F")


def read_distance(path, gy: int, gx: int, gz: int) -> np.ndarray:
    """SBMES:148-151: READ(20) DmyT(1:gy,1:gx,1:gz) with DmyT REAL(4)."""
    return np.asfortranarray(read_array(path, np.float32, (gy, gx, gz)))


def write_distance(path, d: np.ndarray, double: bool = True) -> Path:
    """LevelSet_3D.f90 OutPut3D mode 2 (REAL(8), `double`) or 3 (SNGL)."""
    path = Path(path)
    with open(path, "wb") as f:
        write_record(f, np.asarray(d, dtype=np.float64 if double else np.float32))
    return path


def _frame(fr: int) -> str:
    s = f"{1000 + fr:4d}"  # WRITE(fs,"(I4)") 1000+fr
    if len(s) != 4:
        raise ValueError("frame number outside the reference's I4 field")
    return s


def output3d_a(fr: int, prfn: str, cn: np.ndarray, directory=".", mode: int = 2) -> Path:
    """SBMES:892-919: file prfn//I4(1000+fr)//'.dat' holding SNGL(Cn1) as one
    record (mode 2), or '.txt' with the values as text (mode 1)."""
    if len(prfn) != 6:
        raise ValueError("prfn is CHARACTER(LEN=6)")
    a = np.asarray(cn, dtype=np.float32)
    if mode == 2:
        path = Path(directory) / f"{prfn}{_frame(fr)}.dat"
        with open(path, "wb") as f:
            write_record(f, a)
    elif mode == 1:
        path = Path(directory) / f"{prfn}{_frame(fr)}.txt"
        np.savetxt(path, a.ravel(order="F")[None, :], fmt="%.9E")
    else:
        raise ValueError("mode is 1 (text) or 2 (binary)")
    return path


def rank_decomposition(gy: int, gz: int, rnb: int, cnb: int) -> np.ndarray:
    """MyDmnCmpn_YZ (SBMES:947-982): for every rank of rnb x cnb, the columns
    (lwy, upy, ny, lwz, upz, nz) -- 1-based global y / z ranges and sizes
    (the combine program's IdxAry).  rank -> z block MOD(rank, rnb),
    y block rank / rnb; the first MOD(n, blocks) blocks get one cell more."""
    out = np.zeros((rnb * cnb, 6), dtype=np.int64)
    for rank in range(rnb * cnb):
        ddc, ddr = rank // rnb, rank % rnb
        bz, rz = divmod(gz, rnb)
        nz = bz + 1 if ddr <= rz - 1 else bz
        lwz = ddr * nz + 1 + (rz if ddr >= rz else 0)
        by, ry = divmod(gy, cnb)
        ny = by + 1 if ddc <= ry - 1 else by
        lwy = ddc * ny + 1 + (ry if ddc >= ry else 0)
        out[rank] = (lwy, lwy + ny - 1, ny, lwz, lwz + nz - 1, nz)
    return out


def write_rank_outputs(fr: int, pred: str, field: np.ndarray, rnb: int, cnb: int,
                       directory=".") -> list[Path]:
    """The per-rank dumps the MPI program writes for the global interior
    field (gy, gx, gz): rank r's block under pred//I4(1000+r)//I4(1000+fr)
    (SBMES:346, :847-851)."""
    if len(pred) != 2:
        raise ValueError("pred is CHARACTER(LEN=2)")
    gy, _, gz = field.shape
    paths = []
    for rank, (lwy, upy, _, lwz, upz, _) in enumerate(rank_decomposition(gy, gz, rnb, cnb)):
        block = field[lwy - 1:upy, :, lwz - 1:upz]
        paths.append(output3d_a(fr, f"{pred}{1000 + rank:4d}", block, directory))
    return paths


def combine(fr: int, pred: str, gy: int, gx: int, gz: int, rnb: int, cnb: int,
            directory=".") -> tuple[np.ndarray, Path]:
    """Cmbn:75-129: reads every rank's REAL(4) dump of frame fr, places it at
    its global position and writes pred//'ASMB'//I4(1000+fr)//'.dat'
    (REAL(4), one record).  Returns the global array and the file."""
    und = np.zeros((gy, gx, gz), dtype=np.float32, order="F")
    for rank, (lwy, upy, ny, lwz, upz, nz) in enumerate(rank_decomposition(gy, gz, rnb, cnb)):
        path = Path(directory) / f"{pred}{1000 + rank:4d}{_frame(fr)}.dat"
        und[lwy - 1:upy, :, lwz - 1:upz] = read_array(path, np.float32, (int(ny), gx, int(nz)))
    return und, output3d_a(fr, f"{pred}ASMB", und, directory)


def rec_tmfx(fr: int, prfn: str, it: int, tm: float, frx: float, crnt: float, tg: float,
             bve: float, directory=".") -> Path:
    """SBMES:922-943: one line fr, iter, tm, Xrf, crnt, trgI, BvE in
    prfn//'TmFx.txt'; frame 1 starts the file, later frames append."""
    path = Path(directory) / f"{prfn}TmFx.txt"
    line = f"{int(fr):12d}{int(it):12d}" + "".join(f"{float(v):26.17E}"
                                                   for v in (tm, frx, crnt, tg, bve)) + "\n"
    with open(path, "w" if fr == 1 else "a") as f:
        f.write(line)
    return path


def read_tmfx(path) -> np.ndarray:
    """The TmFx log as rows (fr, iter, tm, Xrf, crnt, trgI, BvE)."""
    return np.loadtxt(path, ndmin=2)
