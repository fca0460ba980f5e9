"""Host-side mirror of the reference's SBM solver interface over the C-ABI.

The reference (AffanMalik90/Elsim, src/frtrn/SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90,
called SBMES here) is one Fortran program whose solver loops are inline; its
only subroutines on the path are Tbl_Chk_Pln_3DA (SBMES:987), ReDist3D_XYZ
(LevelSet_3D.f90:194) and the AccDiff sweep (AccDiff_3D.f90:111).  This
module binds ``libsbm_gb300.so`` with ctypes exactly as a Fortran
``bind(C)`` interface would, and offers:

* ``Context`` -- one device-resident domain: field upload/download in the
  reference's halo-padded (y, x, z) layout, ``setup_domain`` (SBMES:154-341),
  ``cg_solve`` (the inline CG loops), and the time-step stages;
* ``tbl_chk_pln_3da``, ``redist3d_xyz``, ``accdiff``, ``rm_mask``, ``sign``
  -- one-for-one replacements of the reference subroutines/blocks.

Arrays are numpy arrays in Fortran order, indexed ``A[i, j, k]`` with the
halo at index 0 and n+1, as in the reference.  Errors raise ``SbmError``
carrying the C status code.  There is no CPU fallback: if the CUDA library
is missing the import of a ``Context`` fails.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libsbm_gb300.so"

# status codes (include/sbm_capi.h)
OK, ERR_ARG, ERR_CUDA, ERR_MAXIT, ERR_NONFINITE, ERR_BREAKDOWN, ERR_NOMEM, ERR_STATE, ERR_TIMEOUT = (
    0, -1, -2, -3, -4, -5, -6, -7, -8)
TUNE_NO_TMA = 1
TUNE_PC_ADDITIVE = 2
TUNE_HOST_LOOP = 4
BC_COPY, BC_ZERO = 0, 1
OP_CNE, OP_PHP, OP_PHE, OP_GENERIC, OP_GENERIC_DIAG = 0, 1, 2, 3, 4
STOP_REF_UPDATE, STOP_REF_RESID, STOP_REL_RES = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
PC_NONE, PC_JACOBI, PC_LEARNED = 0, 1, 2
BV_EXP, BV_LINEAR = 0, 1
CH_TABLE, CH_DOUBLE_WELL = 0, 1
(F_PSP, F_PSE, F_AVP, F_AVPX, F_CNP, F_CNE, F_PHP, F_PHE, F_RXN, F_COEF, F_RHS, F_X, F_WEIGHT,
 F_DIAG) = range(14)
FIELDS = dict(psP=F_PSP, psE=F_PSE, AvP=F_AVP, AvPx=F_AVPX, CnP=F_CNP, CnE=F_CNE, phP=F_PHP,
              phE=F_PHE, Rxn=F_RXN, coef=F_COEF, rhs=F_RHS, x=F_X, weight=F_WEIGHT, diag=F_DIAG)
TBL_MAX = 128

_ERRNAMES = {ERR_ARG: "bad argument", ERR_CUDA: "CUDA error", ERR_MAXIT: "iteration cap",
             ERR_NONFINITE: "non-finite value", ERR_BREAKDOWN: "CG breakdown",
             ERR_NOMEM: "out of device memory", ERR_STATE: "invalid state",
             ERR_TIMEOUT: "device wait expired"}


class SbmError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        msg = f"{where}: {_ERRNAMES.get(code, 'error')} ({code})"
        if detail:
            msg += f" [{detail}]"
        super().__init__(msg)


class Params(C.Structure):
    """Mirror of ``sbm_params`` (include/sbm_capi.h)."""
    _fields_ = [(n, C.c_double) for n in (
        "dx", "rho", "eps", "ch_mask", "d0", "tc1", "tc2", "t_minus", "dab_c0", "dab_c1", "dab_c2",
        "dab_c3", "cne_ref", "cst1", "frd", "bvp", "bve", "kap_scale", "avp_mask", "i0_scale",
        "kfw_c", "crt_cne", "crt_php", "crt_phe", "crt_picard")] + [
        (n, C.c_int) for n in ("max_it_cne", "max_it_php", "max_it_phe", "max_picard",
                               "cne_mean_every", "bv_mode", "tbl_n", "ch_mode")] + [
        (n, C.c_double * TBL_MAX) for n in ("tbl_x", "tbl_mu", "tbl_mb", "tbl_i0", "tbl_ocv")] + [
        ("ch_w", C.c_double)]

    def set_table(self, name: str, values) -> None:
        v = np.asarray(values, dtype=np.float64)
        if v.size > TBL_MAX:
            raise ValueError("table longer than SBM_TBL_MAX")
        arr = getattr(self, name)
        for t, x in enumerate(v):
            arr[t] = float(x)
        if name == "tbl_x":
            self.tbl_n = int(v.size)

    def table(self, name: str) -> np.ndarray:
        return np.array(getattr(self, name)[: self.tbl_n])


class Scalars(C.Structure):
    """Mirror of ``sbm_scalars``."""
    _fields_ = [(n, C.c_double) for n in ("tPP", "tPE", "xrf", "infx", "scrnt", "trgI", "bve",
                                          "cvgp", "cvgl")] + [
        (n, C.c_int) for n in ("it_cne", "it_php", "it_phe", "n_picard")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


def load_library(path: os.PathLike | None = None) -> C.CDLL:
    """Loads the CUDA library (fails loudly when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the SBM path has no CPU fallback)")
    lib = C.CDLL(str(p))
    dp, fp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int), C.c_void_p
    i64 = C.c_int64
    sig = {
        "sbm_version": (C.c_char_p, []),
        "sbm_launch_count": (i64, []),
        "sbm_last_error": (C.c_char_p, []),
        "sbm_params_reference": (C.c_int, [C.POINTER(Params)]),
        "sbm_ctx_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(Params), C.POINTER(vp)]),
        "sbm_ctx_destroy": (C.c_int, [vp]),
        "sbm_ctx_set_params": (C.c_int, [vp, C.POINTER(Params)]),
        "sbm_ctx_set_tuning": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]),
        "sbm_ctx_stream": (C.c_int, [vp, C.POINTER(vp)]),
        "sbm_ctx_sync": (C.c_int, [vp]),
        "sbm_ctx_get_params": (C.c_int, [vp, C.POINTER(Params)]),
        "sbm_ctx_get_scalars": (C.c_int, [vp, C.POINTER(Scalars)]),
        "sbm_ctx_snapshot_size": (C.c_int, [vp, C.POINTER(C.c_size_t)]),
        "sbm_ctx_snapshot": (C.c_int, [vp, vp, C.c_size_t]),
        "sbm_ctx_restore": (C.c_int, [vp, vp, C.c_size_t]),
        "sbm_upload": (C.c_int, [vp, C.c_int, dp, C.c_int]),
        "sbm_download": (C.c_int, [vp, C.c_int, dp, C.c_int]),
        "sbm_field_ptr": (C.c_int, [vp, C.c_int, C.POINTER(dp)]),
        "sbm_setup_domain": (C.c_int, [vp, fp, fp, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.POINTER(Scalars)]),
        "sbm_cg_solve": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                   C.c_int, C.c_int, C.c_int, ip, dp, fp]),
        "sbm_bench_kernel": (C.c_int, [vp, C.c_int, C.c_int, fp, dp]),
        "sbm_time_step": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_int,
                                    C.POINTER(Scalars)]),
        "sbm_ch_step": (C.c_int, [vp, C.c_double, C.POINTER(Scalars)]),
        "sbm_cne_step": (C.c_int, [vp, C.c_int, C.c_double, C.c_int, C.POINTER(Scalars)]),
        "sbm_bv_update": (C.c_int, [vp, C.c_int, C.POINTER(Scalars)]),
        "sbm_voltage_step": (C.c_int, [vp, C.c_double, C.c_double, C.POINTER(Scalars)]),
        "sbm_batch_solve": (C.c_int, [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_double,
                                      C.c_double, C.c_int, C.c_int, ip, dp, ip, fp]),
        "sbm_batch_solve_ops": (C.c_int, [C.POINTER(vp), ip, ip, ip, dp, C.c_int, C.c_double,
                                          C.c_int, C.c_int, ip, dp, ip, fp]),
        "sbm_table_lookup": (C.c_int, [i64, C.c_int, dp, dp, dp, dp]),
        "sbm_conv3d_bf16": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.POINTER(C.c_uint16), C.POINTER(C.c_uint16),
                                      C.POINTER(C.c_float), C.c_int, C.c_int, C.c_int, fp]),
        "sbm_redist": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, dp, dp]),
        "sbm_accdiff": (C.c_int, [C.c_int, C.c_int, C.c_int, dp, dp, C.c_int, C.c_int]),
        "sbm_allen_cahn": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, dp]),
        "sbm_ls_geometry": (C.c_int, [dp] + [C.c_int] * 7 + [C.c_double, dp]),
        "sbm_connectivity": (C.c_int, [C.c_int] * 3 + [dp, C.c_double, C.c_int, dp, dp]),
        "sbm_rm_ucnct": (C.c_int, [C.c_int] * 3 + [dp, dp, dp, C.c_int, dp, dp]),
        "sbm_ls_frontend": (C.c_int, [dp] + [C.c_int] * 7 + [C.c_double, C.c_int, C.c_int,
                                                              C.c_double, dp]),
        "sbm_ls_frontend_device": (C.c_int, [C.c_void_p] + [C.c_int] * 7 +
                                   [C.c_double, C.c_int, C.c_int, C.c_double] +
                                   [C.c_void_p] * 4),
        "sbm_redist_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                         C.c_void_p, C.c_void_p, C.c_void_p]),
        "sbm_set_wait_limit": (C.c_int, [C.c_int]),
        "sbm_split_f64": (C.c_int, [i64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
        "sbm_rm_mask": (C.c_int, [i64, dp, dp, dp]),
        "sbm_sign": (C.c_int, [i64, dp, C.c_double, dp]),
        "sbm_net_param_count": (i64, []),
        "sbm_net_create": (C.c_int, [C.c_uint64, C.POINTER(vp)]),
        "sbm_net_destroy": (C.c_int, [vp]),
        "sbm_net_get_params": (C.c_int, [vp, fp, i64]),
        "sbm_net_set_params": (C.c_int, [vp, fp, i64]),
        "sbm_net_forward": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, fp, fp]),
        "sbm_net_loss_grad": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, fp, fp, dp, fp]),
        "sbm_net_train": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, fp, fp, C.c_int,
                                    C.c_int, C.c_float, C.c_uint64, fp]),
        "sbm_net_set_data": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, fp, fp]),
        "sbm_net_train_steps": (C.c_int, [vp, C.c_int, C.c_int, C.c_float, C.c_uint64, fp]),
        "sbm_ctx_set_net": (C.c_int, [vp, vp, C.c_double]),
        "sbm_net_load": (C.c_int, [C.c_char_p, C.POINTER(vp), dp]),
        "sbm_ctx_last_precond": (C.c_int, [vp]),
        "sbm_learned_pc_apply": (C.c_int, [vp, C.c_int, C.c_int, C.c_double, dp, dp]),
        "sbm_learned_pc_apply_op": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double, dp,
                                              dp]),
        "sbm_net_set_mass_channel": (C.c_int, [vp, C.c_int]),
        "sbm_net_get_mass_channel": (C.c_int, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def declared_symbols() -> list[str]:
    """Every function name declared in include/sbm_capi.h."""
    import re
    hdr = (_PKG.parent / "include" / "sbm_capi.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w]+\**\s+\**(sbm_\w+)\s*\(", hdr, re.M)))


def _check(rc: int, where: str) -> int:
    if rc != OK:
        detail = ""
        if rc == ERR_CUDA and _lib is not None:
            detail = _lib.sbm_last_error().decode(errors="replace")
        raise SbmError(rc, where, detail)
    return rc


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a, shape=None) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return np.asfortranarray(a)


def reference_params() -> Params:
    """The reference's constants (SBMES:90-136) with flat synthetic tables."""
    p = Params()
    _check(load_library().sbm_params_reference(C.byref(p)), "sbm_params_reference")
    return p


def launch_count() -> int:
    return int(load_library().sbm_launch_count())


CKPT_MAGIC = b"SBMCKPT1"


def write_checkpoint(path, blob, meta: dict) -> Path:
    """Checkpoint file: 8-byte magic, u64 length of the JSON meta, the meta,
    zero padding to a multiple of 64 bytes, the snapshot bytes.  Written to a
    temporary name, flushed to stable storage (fsync of the file, then of its
    directory after the rename), so a process crash or a power loss leaves
    either the previous file or the new one whole."""
    path = Path(path)
    js = json.dumps(meta, sort_keys=True).encode()
    head = CKPT_MAGIC + np.uint64(len(js)).astype("<u8").tobytes() + js
    head += b"\0" * (-len(head) % 64)
    tmp = path.with_name(path.name + ".tmp")
    with open(tmp, "wb") as f:
        f.write(head)
        f.write(memoryview(np.ascontiguousarray(blob, dtype=np.uint8)))
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)
    try:
        dfd = os.open(path.parent if str(path.parent) else ".", os.O_RDONLY)
    except OSError:
        return path  # a directory that cannot be opened for reading
    try:
        os.fsync(dfd)
    except OSError:
        pass  # file systems that do not sync directories
    finally:
        os.close(dfd)
    return path


def read_checkpoint(path) -> tuple[dict, np.ndarray]:
    """(meta, snapshot bytes) of a checkpoint file."""
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size < 16 or raw[:8].tobytes() != CKPT_MAGIC:
        raise ValueError(f"{path}: not a checkpoint file")
    n = int(raw[8:16].view("<u8")[0])
    if 16 + n > raw.size:
        raise ValueError(f"{path}: truncated checkpoint")
    meta = json.loads(raw[16:16 + n].tobytes())
    start = 16 + n + (-(16 + n) % 64)
    return meta, raw[start:]


class Context:
    """One device-resident SBM domain of ny x nx x nz interior voxels."""

    def __init__(self, ny: int, nx: int, nz: int, params: Params | None = None):
        self.lib = load_library()
        self.shape = (ny, nx, nz)
        self.hshape = (ny + 2, nx + 2, nz + 2)
        self.params = params if params is not None else reference_params()
        h = C.c_void_p()
        _check(self.lib.sbm_ctx_create(ny, nx, nz, C.byref(self.params), C.byref(h)),
               "sbm_ctx_create")
        self._h = h

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.sbm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- configuration
    def set_params(self, params: Params) -> None:
        self.params = params
        _check(self.lib.sbm_ctx_set_params(self._h, C.byref(params)), "sbm_ctx_set_params")

    def set_tuning(self, zc64=0, zc32=0, chunk=0, delta=0.0, no_tma=False,
                   pc_additive=False, host_loop=False) -> None:
        """Launch-shape knobs (0 = built-in), the reliable-update factor, the
        choice of the register-tiled instead of the TMA-staged stencil, of
        the additive instead of the multiplicative learned preconditioner and
        of host-driven instead of device-looped iteration chunks (for
        profilers that cannot see kernels inside conditional graphs)."""
        flags = ((TUNE_NO_TMA if no_tma else 0) | (TUNE_PC_ADDITIVE if pc_additive else 0) |
                 (TUNE_HOST_LOOP if host_loop else 0))
        _check(self.lib.sbm_ctx_set_tuning(self._h, zc64, zc32, chunk, delta, flags),
               "sbm_ctx_set_tuning")

    def bench_kernel(self, which: int, reps: int = 20) -> tuple[float, float]:
        """(ms per launch, algorithmic bytes per launch) of a solver kernel."""
        ms = C.c_float(0)
        b = C.c_double(0)
        _check(self.lib.sbm_bench_kernel(self._h, which, reps, C.byref(ms), C.byref(b)),
               "sbm_bench_kernel")
        return ms.value, b.value

    def stream(self) -> int:
        s = C.c_void_p()
        _check(self.lib.sbm_ctx_stream(self._h, C.byref(s)), "sbm_ctx_stream")
        return s.value or 0

    def sync(self) -> None:
        _check(self.lib.sbm_ctx_sync(self._h), "sbm_ctx_sync")

    def scalars(self) -> dict:
        s = Scalars()
        _check(self.lib.sbm_ctx_get_scalars(self._h, C.byref(s)), "sbm_ctx_get_scalars")
        return s.as_dict()

    # -- checkpoint / resume
    def snapshot(self) -> np.ndarray:
        """The context's state (parameters, scalars, every FP64 field a later
        step reads) as a host byte array; see sbm_ctx_snapshot."""
        n = C.c_size_t(0)
        _check(self.lib.sbm_ctx_snapshot_size(self._h, C.byref(n)), "sbm_ctx_snapshot_size")
        buf = np.empty(n.value, dtype=np.uint8)
        _check(self.lib.sbm_ctx_snapshot(self._h, buf.ctypes.data, n.value), "sbm_ctx_snapshot")
        return buf

    def restore(self, buf) -> None:
        """Loads a snapshot of a context with the same grid."""
        buf = np.ascontiguousarray(np.frombuffer(buf, dtype=np.uint8))
        _check(self.lib.sbm_ctx_restore(self._h, buf.ctypes.data, buf.size), "sbm_ctx_restore")
        p = Params()
        _check(self.lib.sbm_ctx_get_params(self._h, C.byref(p)), "sbm_ctx_get_params")
        self.params = p

    def save(self, path, **meta) -> Path:
        """Writes a checkpoint file: the snapshot plus the caller's run
        counters (``meta``, e.g. iteration, time, frame) as JSON."""
        return write_checkpoint(path, self.snapshot(), meta)

    def load(self, path) -> dict:
        """Restores a checkpoint file written by ``save``; returns its meta."""
        meta, blob = read_checkpoint(path)
        self.restore(blob)
        return meta

    # -- fields
    def upload(self, field, a, haloed: bool = True) -> None:
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        a = _f64(a, self.hshape if haloed else self.shape)
        _check(self.lib.sbm_upload(self._h, fid, _dptr(a), int(haloed)), "sbm_upload")

    def download(self, field, haloed: bool = True) -> np.ndarray:
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        out = np.zeros(self.hshape if haloed else self.shape, dtype=np.float64, order="F")
        _check(self.lib.sbm_download(self._h, fid, _dptr(out), int(haloed)), "sbm_download")
        return out

    def field_ptr(self, field) -> int:
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        p = C.POINTER(C.c_double)()
        _check(self.lib.sbm_field_ptr(self._h, fid, C.byref(p)), "sbm_field_ptr")
        return C.cast(p, C.c_void_p).value

    # -- set-up and solves
    def setup_domain(self, dist_p, dist_e, zeta=0.5, cnp0=2.02e-2, cne0=1.0e-3, cr=6.0) -> dict:
        """SBMES:154-341 from two REAL(4) distance fields (interior shape)."""
        dp = np.asfortranarray(np.asarray(dist_p, dtype=np.float32))
        de = np.asfortranarray(np.asarray(dist_e, dtype=np.float32))
        if dp.shape != self.shape or de.shape != self.shape:
            raise ValueError("distance fields must have the interior shape")
        s = Scalars()
        fpt = C.POINTER(C.c_float)
        _check(self.lib.sbm_setup_domain(self._h, dp.ctypes.data_as(fpt), de.ctypes.data_as(fpt),
                                         zeta, cnp0, cne0, cr, C.byref(s)), "sbm_setup_domain")
        return s.as_dict()

    def cg_solve(self, op=OP_GENERIC, bc_x0=BC_COPY, bc_x1=BC_COPY, scale=1.0, tol=1e-8,
                 max_it=100000, stop_rule=STOP_REL_RES, precision=PREC_FP64, precond=PC_NONE,
                 raise_on_maxit: bool = True) -> dict:
        it = C.c_int(0)
        res = C.c_double(0)
        ms = C.c_float(0)
        rc = self.lib.sbm_cg_solve(self._h, op, bc_x0, bc_x1, scale, tol, max_it, stop_rule,
                                   precision, precond, C.byref(it), C.byref(res), C.byref(ms))
        if rc != OK and not (rc == ERR_MAXIT and not raise_on_maxit):
            _check(rc, "sbm_cg_solve")
        return dict(iters=it.value, final_res=res.value, ms=ms.value, status=rc)

    def set_net(self, net: "Net | None", out_scale: float = 1.0) -> None:
        """Attach the learned preconditioner (SBM_PC_LEARNED); None detaches.
        The context keeps a reference so the network outlives it."""
        self._net = net
        _check(self.lib.sbm_ctx_set_net(self._h, net._h if net is not None else None,
                                        out_scale if net is None else net.out_scale),
               "sbm_ctx_set_net")

    def last_precond(self) -> int:
        """Preconditioner the last mixed-precision solve used (PC_*)."""
        return int(self.lib.sbm_ctx_last_precond(self._h))

    def learned_pc_apply(self, r, bc_x0=BC_ZERO, bc_x1=BC_ZERO, scale=1.0,
                         op=OP_GENERIC) -> np.ndarray:
        """z = M(r) of the attached network for the GENERIC (or, with
        op=OP_GENERIC_DIAG, the diagonal CnE-form) operator of the uploaded
        coefficient (halo-padded arrays)."""
        r = _f64(r, self.hshape)
        z = np.zeros(self.hshape, dtype=np.float64, order="F")
        _check(self.lib.sbm_learned_pc_apply_op(self._h, op, bc_x0, bc_x1, scale, _dptr(r),
                                                _dptr(z)), "sbm_learned_pc_apply_op")
        return z

    def time_step(self, it: int, dt: float, vsr: float, precision=PREC_FP64) -> dict:
        s = Scalars()
        _check(self.lib.sbm_time_step(self._h, it, dt, vsr, precision, C.byref(s)),
               "sbm_time_step")
        return s.as_dict()

    def ch_step(self, dt: float) -> dict:
        s = Scalars()
        _check(self.lib.sbm_ch_step(self._h, dt, C.byref(s)), "sbm_ch_step")
        return s.as_dict()

    def cne_step(self, it: int, dt: float, precision=PREC_FP64) -> dict:
        s = Scalars()
        _check(self.lib.sbm_cne_step(self._h, it, dt, precision, C.byref(s)), "sbm_cne_step")
        return s.as_dict()

    def bv_update(self, precision=PREC_FP64) -> dict:
        s = Scalars()
        _check(self.lib.sbm_bv_update(self._h, precision, C.byref(s)), "sbm_bv_update")
        return s.as_dict()

    def voltage_step(self, dt: float, vsr: float) -> dict:
        s = Scalars()
        _check(self.lib.sbm_voltage_step(self._h, dt, vsr, C.byref(s)), "sbm_voltage_step")
        return s.as_dict()


def batch_solve(contexts, bc_x0=BC_ZERO, bc_x1=BC_ZERO, scale=1.0, tol=1e-8, max_it=100000,
                precond=PC_JACOBI) -> dict:
    """Mixed-precision GENERIC solves of many independent contexts advanced
    together by one CUDA-graph launch per round (sbm_batch_solve)."""
    lib = load_library()
    n = len(contexts)
    hs = (C.c_void_p * n)(*[c._h for c in contexts])
    it = (C.c_int * n)()
    res = (C.c_double * n)()
    stt = (C.c_int * n)()
    ms = C.c_float(0)
    _check(lib.sbm_batch_solve(hs, n, bc_x0, bc_x1, scale, tol, max_it, precond, it, res, stt,
                               C.byref(ms)), "sbm_batch_solve")
    return dict(iters=list(it), final_res=list(res), status=list(stt), ms=ms.value)


def batch_solve_ops(contexts, ops, bc_x0, bc_x1, scales, tol=1e-8, max_it=100000,
                    precond=PC_JACOBI) -> dict:
    """As batch_solve with one system per context of either GENERIC form
    (OP_GENERIC or OP_GENERIC_DIAG) and its own x-face rules and scale
    (sbm_batch_solve_ops)."""
    lib = load_library()
    n = len(contexts)
    if not (len(ops) == len(bc_x0) == len(bc_x1) == len(scales) == n):
        raise ValueError("one op, x-face rule pair and scale per context")
    hs = (C.c_void_p * n)(*[c._h for c in contexts])
    it = (C.c_int * n)()
    res = (C.c_double * n)()
    stt = (C.c_int * n)()
    ms = C.c_float(0)
    arr = lambda t, v: (t * n)(*v)
    _check(lib.sbm_batch_solve_ops(hs, arr(C.c_int, ops), arr(C.c_int, bc_x0),
                                   arr(C.c_int, bc_x1), arr(C.c_double, scales), n, tol, max_it,
                                   precond, it, res, stt, C.byref(ms)), "sbm_batch_solve_ops")
    return dict(iters=list(it), final_res=list(res), status=list(stt), ms=ms.value)


class Net:
    """The learned preconditioner's U-Net (sbm_net_*): parameters, forward
    pass, loss gradient and on-GPU training.  Inputs are channels-last
    (voxel v = i + ny*(j + nx*k), 16 channels), nb samples stacked along z."""

    def __init__(self, seed: int = 0, params: np.ndarray | None = None, out_scale: float = 1.0,
                 mass: bool = False):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.sbm_net_create(seed, C.byref(h)), "sbm_net_create")
        self._h = h
        self.out_scale = float(out_scale)
        if params is not None:
            self.set_params(params)
        self.mass = mass

    @property
    def mass(self) -> bool:
        """True when the network reads input channel 5, the mass term of the
        CnE form (it then also preconditions GENERIC_DIAG / CnE solves)."""
        return bool(self.lib.sbm_net_get_mass_channel(self._h))

    @mass.setter
    def mass(self, on: bool) -> None:
        _check(self.lib.sbm_net_set_mass_channel(self._h, 1 if on else 0),
               "sbm_net_set_mass_channel")

    @staticmethod
    def param_count() -> int:
        return int(load_library().sbm_net_param_count())

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.sbm_net_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.empty(self.param_count(), dtype=np.float32)
        _check(self.lib.sbm_net_get_params(self._h, _fptr(out), out.size), "sbm_net_get_params")
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(self.lib.sbm_net_set_params(self._h, _fptr(p), p.size), "sbm_net_set_params")

    def forward(self, x, dims, nb: int = 1) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.empty(x.shape[0], dtype=np.float32)
        _check(self.lib.sbm_net_forward(self._h, *dims, nb, _fptr(x), _fptr(out)),
               "sbm_net_forward")
        return out

    def loss_grad(self, x, target, dims, nb: int = 1) -> tuple[float, np.ndarray]:
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        g = np.empty(self.param_count(), dtype=np.float32)
        loss = C.c_double(0)
        _check(self.lib.sbm_net_loss_grad(self._h, *dims, nb, _fptr(x), _fptr(t), C.byref(loss),
                                          _fptr(g)), "sbm_net_loss_grad")
        return loss.value, g

    def set_data(self, x, target, dims) -> None:
        """Keeps a training set (x: (samples*V) x 16, target: samples*V) on the
        device for train_steps."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        ns = t.size // int(np.prod(dims))
        _check(self.lib.sbm_net_set_data(self._h, *dims, ns, _fptr(x), _fptr(t)),
               "sbm_net_set_data")

    def train_steps(self, steps: int, batch: int, lr: float, seed: int = 0) -> np.ndarray:
        """Adam steps on the resident training set; returns the loss per step."""
        hist = np.empty(steps, dtype=np.float32)
        _check(self.lib.sbm_net_train_steps(self._h, steps, batch, lr, seed, _fptr(hist)),
               "sbm_net_train_steps")
        return hist

    def train(self, x, target, dims, steps: int, batch: int, lr: float, seed: int = 0) -> np.ndarray:
        """x: (samples*V) x 16, target: samples*V; returns the loss per step."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        nv = int(np.prod(dims))
        ns = t.size // nv
        hist = np.empty(steps, dtype=np.float32)
        _check(self.lib.sbm_net_train(self._h, *dims, ns, _fptr(x), _fptr(t), steps, batch, lr,
                                      seed, _fptr(hist)), "sbm_net_train")
        return hist


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


# ------------------------------------------------------- stateless routines

def tbl_chk_pln_3da(cord, vals, cn) -> np.ndarray:
    """Tbl_Chk_Pln_3DA (SBMES:987-1028) on the GPU; any array shape."""
    lib = load_library()
    cord = np.ascontiguousarray(cord, dtype=np.float64)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    c = np.asarray(cn, dtype=np.float64)
    flat = np.ascontiguousarray(c).ravel()
    out = np.empty_like(flat)
    _check(lib.sbm_table_lookup(flat.size, cord.size, _dptr(cord), _dptr(vals), _dptr(flat),
                                _dptr(out)), "sbm_table_lookup")
    return out.reshape(c.shape)


def redist3d_xyz(lit: int, sg, f, dt: float = 1.0e-1) -> np.ndarray:
    """ReDist3D_XYZ (LevelSet_3D.f90:194-261) on the GPU; returns the new f.

    ``dt`` is 1.0d-1 in LevelSet_3D.f90 and the REAL(4) 1.0e-1 (pass
    ``float(np.float32(0.1))``) in RM_UCNCT_3D.f90."""
    lib = load_library()
    sg = _f64(sg)
    f = _f64(f).copy(order="F")
    py, px, pz = (s - 2 for s in sg.shape)
    _check(lib.sbm_redist(lit, py, px, pz, dt, _dptr(sg), _dptr(f)), "sbm_redist")
    return f


def allen_cahn(iters: int, f) -> np.ndarray:
    """Allen-Cahn pre-smoothing (LevelSet_3D.f90:116-136) on the GPU;
    returns the new halo-padded field (ghosts zero-gradient)."""
    lib = load_library()
    f = _f64(f).copy(order="F")
    py, px, pz = (s - 2 for s in f.shape)
    _check(lib.sbm_allen_cahn(iters, py, px, pz, _dptr(f)), "sbm_allen_cahn")
    return f


def ls_geometry(vox, yg: int, zg: int, xoff: int, nthick: int, tr: float) -> np.ndarray:
    """Stacked voxel field of LevelSet_3D.f90:80-122 on the GPU from
    TmpA = vox (yo, xo, zo); returns the halo-padded (yg+2, xg+2, zg+2)
    field, xg = xoff + nthick*zo."""
    lib = load_library()
    vox = _f64(vox)
    yo, xo, zo = vox.shape
    ds = np.zeros((yg + 2, xoff + nthick * zo + 2, zg + 2), order="F")
    _check(lib.sbm_ls_geometry(_dptr(vox), yo, xo, zo, yg, zg, xoff, nthick, float(tr),
                               _dptr(ds)), "sbm_ls_geometry")
    return ds


def ls_frontend(vox, yg: int, zg: int, xoff: int, nthick: int, tr: float, ac_iters: int = 50,
                lit: int = 175, dt: float = 1.0e-1) -> np.ndarray:
    """One frame of the LevelSet_3D front end (LevelSet_3D.f90:80-150) on the
    GPU; returns the halo-padded distance."""
    lib = load_library()
    vox = _f64(vox)
    yo, xo, zo = vox.shape
    ds = np.zeros((yg + 2, xoff + nthick * zo + 2, zg + 2), order="F")
    _check(lib.sbm_ls_frontend(_dptr(vox), yo, xo, zo, yg, zg, xoff, nthick, float(tr),
                               ac_iters, lit, float(dt), _dptr(ds)), "sbm_ls_frontend")
    return ds


def connectivity(dist, width: float = 0.75, term: int = 1501) -> tuple[np.ndarray, np.ndarray]:
    """AccDiff_3D program body for one interior distance field on the GPU:
    halo-padded Cn of the solid and of the electrolyte."""
    lib = load_library()
    d = _f64(dist)
    py, px, pz = d.shape
    cs = np.zeros((py + 2, px + 2, pz + 2), order="F")
    ce = np.zeros_like(cs)
    _check(lib.sbm_connectivity(py, px, pz, _dptr(d), width, term, _dptr(cs), _dptr(ce)),
           "sbm_connectivity")
    return cs, ce


def rm_ucnct(dist, cn_solid, cn_elec, lit: int = 175) -> tuple[np.ndarray, np.ndarray]:
    """RM_UCNCT_3D program body on the GPU: halo-padded (solid, electrolyte)
    distances with the disconnected regions removed; all inputs interior."""
    lib = load_library()
    d = _f64(dist)
    cs, ce = _f64(cn_solid, d.shape), _f64(cn_elec, d.shape)
    py, px, pz = d.shape
    ds = np.zeros((py + 2, px + 2, pz + 2), order="F")
    de = np.zeros_like(ds)
    _check(lib.sbm_rm_ucnct(py, px, pz, _dptr(d), _dptr(cs), _dptr(ce), lit, _dptr(ds),
                            _dptr(de)), "sbm_rm_ucnct")
    return ds, de


def accdiff(psi, cn, term: int = 1501, dirichlet_x: int = 1) -> np.ndarray:
    """One AccDiff_3D phase (AccDiff_3D.f90:111-169 solid with dirichlet_x=1,
    :185-243 electrolyte with dirichlet_x=0) on the GPU; returns the new Cn."""
    lib = load_library()
    psi = _f64(psi)
    cn = _f64(cn).copy(order="F")
    py, px, pz = (s - 2 for s in psi.shape)
    _check(lib.sbm_accdiff(py, px, pz, _dptr(psi), _dptr(cn), term, dirichlet_x), "sbm_accdiff")
    return cn


def rm_mask(psA, cn) -> np.ndarray:
    """RM_UCNCT_3D.f90:79-82: psB = psA, 0 where Cn < 1e-4 (REAL(4))."""
    lib = load_library()
    a = np.ascontiguousarray(psA, dtype=np.float64)
    c = np.ascontiguousarray(cn, dtype=np.float64)
    out = np.empty_like(a)
    _check(lib.sbm_rm_mask(a.size, _dptr(a), _dptr(c), _dptr(out)), "sbm_rm_mask")
    return out


def sign(ds, thr: float = 0.5) -> np.ndarray:
    """LevelSet_3D.f90:140-144: 1 where ds > thr, else -1."""
    lib = load_library()
    d = np.ascontiguousarray(ds, dtype=np.float64)
    out = np.empty_like(d)
    _check(lib.sbm_sign(d.size, _dptr(d), thr, _dptr(out)), "sbm_sign")
    return out
