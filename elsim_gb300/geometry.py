"""Geometry front end of the reference (LevelSet_3D.f90) on the GPU.

The reference program turns one voxelated microstructure into the signed
distance the SBM solver reads, once per tunnel radius (frames 3..13):

1. read TmpA(500,520,170) from a list-directed text file   (:61-64)
2. reorient, carve two cylindrical tunnels, stack four
   thicknesses in x after 50 empty columns, NoGrdBc3D       (:80-122)
3. 50 Allen-Cahn pre-smoothing steps                       (:124-136)
4. sign (> 0.5 -> +1, else -1), 175 reinitialisation steps
   from zero                                               (:138-147)
5. OutPut3D mode 2: the REAL(8) interior, one unformatted
   record, file prefix//I4(1000+fr)//'.dat'               (:150, :357-362)

Steps 2-4 run on the GPU (``sbm.ls_frontend``: one gather kernel for the
stacked field, then the Allen-Cahn, sign and reinitialisation kernels, all
bit-exact with the reference arithmetic); steps 1 and 5 are host I/O.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import fortran_io, sbm

# DATA TuRd (LevelSet_3D.f90:54-56): REAL(4) literals stored into REAL(8).
TUNNEL_RADII = np.array([0, 6.3826e+00, 1.2764e+01, 1.9171e+01, 2.5566e+01, 3.1941e+01,
                         3.8331e+01, 4.4729e+01, 5.1114e+01, 5.7506e+01, 6.3890e+01,
                         7.0280e+01, 7.6674e+01, 8.3061e+01], dtype=np.float32).astype(np.float64)

# Sizes of the reference program (LevelSet_3D.f90:9-11): voxel input
# (yo, xo, zo), computational grid yg x (xoff + nthick*zo) x zg.
REFERENCE = {"yo": 500, "xo": 520, "zo": 170, "yg": 93, "zg": 160, "xoff": 50, "nthick": 4}
FRAMES = range(3, 14)
PREFIX = "L24Z"
AC_ITERS = 50
REDIST_ITERS = 175
DT = 1.0e-1


def read_voxels(path, yo: int, xo: int, zo: int) -> np.ndarray:
    """READ(20,*) TmpA(1:yo,1:xo,1:zo) (LevelSet_3D.f90:61-64): the first
    yo*xo*zo values of a list-directed text file (separators blank, comma or
    newline; ``r*c`` repeat counts; D exponents; a slash ends the input) in
    Fortran order."""
    text = Path(path).read_text().split("/", 1)[0].replace(",", " ")
    text = text.replace("d", "e").replace("D", "e")
    toks = text.split()
    n = yo * xo * zo
    if any("*" in t for t in toks):
        vals: list[float] = []
        for t in toks:
            if "*" in t:
                r, c = t.split("*", 1)
                vals.extend([float(c)] * int(r))
            else:
                vals.append(float(t))
            if len(vals) >= n:
                break
        a = np.asarray(vals[:n], dtype=np.float64)
    else:
        a = np.asarray(toks[:n], dtype=np.float64)
    if a.size < n:
        raise ValueError(f"{path}: {a.size} values, {n} expected")
    return a.reshape((yo, xo, zo), order="F")


def synthetic_voxels(shape=(REFERENCE["yo"], REFERENCE["xo"], REFERENCE["zo"]), seed: int = 0,
                     solid: float = 0.6, blob: float = 3.0) -> np.ndarray:
    """Seeded 0/1 voxel data in place of the reference's scanned
    microstructure: thresholded Gaussian-smoothed white noise, ``solid`` of
    the voxels 1."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    a = gaussian_filter(rng.standard_normal(shape, dtype=np.float32), blob, mode="wrap")
    thr = np.quantile(a[:: max(1, shape[0] // 64), :: max(1, shape[1] // 64)], 1.0 - solid)
    return np.asfortranarray((a > thr).astype(np.float64))


def frame(vox: np.ndarray, n: int, yg: int = REFERENCE["yg"], zg: int = REFERENCE["zg"],
          xoff: int = REFERENCE["xoff"], nthick: int = REFERENCE["nthick"],
          ac_iters: int = AC_ITERS, lit: int = REDIST_ITERS, dt: float = DT) -> np.ndarray:
    """Distance of frame n (tunnel radius TuRd(n)) on the GPU: the interior
    (yg, xoff + nthick*zo, zg) the reference writes."""
    ds = sbm.ls_frontend(vox, yg, zg, xoff, nthick, float(TUNNEL_RADII[n]), ac_iters, lit, dt)
    return ds[1:-1, 1:-1, 1:-1]


def connected(dist: np.ndarray, term: int = 1501, lit: int = REDIST_ITERS):
    """The AccDiff_3D and RM_UCNCT_3D programs for one interior distance
    field (a frame's output) on the GPU: connectivity of each phase, then the
    solid and electrolyte distances with their disconnected regions removed
    (the GRP_LS / POR_LS fields the cell model reads).  Returns
    (d_solid, d_elec, cn_solid, cn_elec), all interior."""
    cs, ce = sbm.connectivity(dist, 0.75, term)
    i = (slice(1, -1),) * 3
    ds, de = sbm.rm_ucnct(dist, cs[i], ce[i], lit)
    return ds[i], de[i], cs[i], ce[i]


def run(vox: np.ndarray, frames=FRAMES, prefix: str = PREFIX, directory=".",
        **kw) -> list[Path]:
    """The reference's frame loop (LevelSet_3D.f90:72-152): one REAL(8)
    distance file prefix//I4(1000+fr)//'.dat' per frame."""
    if len(prefix) != 4:
        raise ValueError("prefix is CHARACTER(LEN=4)")
    out = []
    for n in frames:
        d = frame(vox, n, **kw)
        out.append(fortran_io.write_distance(Path(directory) / f"{prefix}{1000 + n:4d}.dat", d))
    return out
