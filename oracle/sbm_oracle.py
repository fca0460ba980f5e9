"""ctypes bindings of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg
as the checker; the product (elsim_gb300) never imports it.  The oracle is a
line-by-line FP64 C restatement of the reference Fortran, pinned against the
reference's own results on small seeded cases (its Fortran sources run by
the interpreter tests/golden/fortran_subset.py, fixtures
tests/golden/reference_v1.npz) and by analytic known-answer tests.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from elsim_gb300.sbm import Params, Scalars  # struct layouts only

from .build_oracle import build

HERE = Path(__file__).resolve().parent

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = build()
    L = C.CDLL(str(path))
    dp, fp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int), C.c_void_p
    i, d, i64 = C.c_int, C.c_double, C.c_int64
    sig = {
        "orc_nogrdbc": (None, [i, i, i, dp]),
        "orc_bc_yz": (None, [i, i, i, dp]),
        "orc_bc_x": (None, [i, i, i, dp, i, i, i, d, i, d]),
        "orc_absgrd": (None, [i, i, i, dp, dp, dp]),
        "orc_redist": (None, [i, d, i, i, i, dp, dp]),
        "orc_accdiff": (None, [i, i, i, dp, dp, i, i]),
        "orc_connectivity": (None, [i, i, i, dp, d, i, dp, dp]),
        "orc_rm_mask": (None, [i64, dp, dp, dp]),
        "orc_sign": (None, [i64, dp, d, dp]),
        "orc_allen_cahn": (None, [i, i, i, i, dp]),
        "orc_ls_geometry": (i, [dp, i, i, i, i, i, i, i, d, dp]),
        "orc_rm_ucnct": (None, [i, i, i, dp, dp, dp, i, dp, dp]),
        "orc_psi_from_dist": (None, [i, i, i, fp, d, dp]),
        "orc_avp": (None, [i, i, i, dp, dp, d, d, dp, dp]),
        "orc_table": (None, [i64, i, dp, dp, dp, dp]),
        "orc_apply": (None, [i, i, i, dp, dp, d, dp, dp]),
        "orc_residual": (None, [i, i, i, dp, dp, d, dp, dp, dp]),
        "orc_cg": (i, [i, i, i, dp, dp, d, i, i, dp, dp, dp, d, i, d, i, ip, dp]),
        "orc_dot": (d, [i, i, i, dp, dp]),
        "orc_state_new": (vp, [i, i, i, C.POINTER(Params)]),
        "orc_state_free": (None, [vp]),
        "orc_state_field": (dp, [vp, i]),
        "orc_setup_domain": (i, [vp, fp, fp, d, d, d, d, C.POINTER(Scalars)]),
        "orc_ch_step": (i, [vp, d, C.POINTER(Scalars)]),
        "orc_cne_step": (i, [vp, i, d, C.POINTER(Scalars)]),
        "orc_bv_update": (i, [vp, C.POINTER(Scalars)]),
        "orc_voltage_step": (i, [vp, d, d, C.POINTER(Scalars)]),
        "orc_time_step": (i, [vp, i, d, d, C.POINTER(Scalars)]),
        "orc_params_reference": (i, [C.POINTER(Params)]),
        "orc_num_threads": (i, []),
        "orc_set_num_threads": (None, [i]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _F(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def hdims(a):
    return tuple(s - 2 for s in a.shape)


def nogrdbc(f):
    f = _F(f).copy(order="F")
    lib().orc_nogrdbc(*hdims(f), _p(f))
    return f


def allen_cahn(iters, f):
    """LevelSet_3D.f90:116-136 on a halo-padded field (returns a new array)."""
    f = _F(f).copy(order="F")
    lib().orc_allen_cahn(iters, *hdims(f), _p(f))
    return f


def ls_geometry(vox, yg, zg, xoff, nthick, tr):
    """LevelSet_3D.f90:80-122 (reorient, tunnels, stacking, NoGrdBc3D) on
    TmpA = vox (yo, xo, zo); returns the halo-padded stacked field."""
    vox = _F(vox)
    yo, xo, zo = vox.shape
    ds = np.zeros((yg + 2, xoff + nthick * zo + 2, zg + 2), order="F")
    rc = lib().orc_ls_geometry(_p(vox), yo, xo, zo, yg, zg, xoff, nthick, float(tr), _p(ds))
    if rc:
        raise ValueError("geometry arguments out of range")
    return ds


def ls_frontend(vox, yg, zg, xoff, nthick, tr, ac_iters=50, lit=175, dt=1.0e-1):
    """One frame of LevelSet_3D.f90:80-150: stacked field, Allen-Cahn,
    sign, reinitialisation from zero; returns the halo-padded distance."""
    ds = allen_cahn(ac_iters, ls_geometry(vox, yg, zg, xoff, nthick, tr))
    sg = np.asfortranarray(sign(ds.ravel(order="F")).reshape(ds.shape, order="F"))
    return redist(lit, sg, np.zeros_like(ds, order="F"), dt)


def redist(lit, sg, f, dt=1.0e-1):
    sg, f = _F(sg), _F(f).copy(order="F")
    lib().orc_redist(lit, dt, *hdims(f), _p(sg), _p(f))
    return f


def absgrd(sg, f):
    sg, f = _F(sg), _F(f)
    gr = np.zeros_like(f, order="F")
    lib().orc_absgrd(*hdims(f), _p(sg), _p(f), _p(gr))
    return gr


def accdiff(psi, cn, term=1501, dirichlet_x=1):
    psi, cn = _F(psi), _F(cn).copy(order="F")
    lib().orc_accdiff(*hdims(psi), _p(psi), _p(cn), term, dirichlet_x)
    return cn


def connectivity(dist_interior, width=0.75, term=1501):
    d = _F(dist_interior)
    ny, nx, nz = d.shape
    cs = np.zeros((ny + 2, nx + 2, nz + 2), order="F")
    ce = np.zeros_like(cs)
    lib().orc_connectivity(ny, nx, nz, _p(d), width, term, _p(cs), _p(ce))
    return cs, ce


def rm_ucnct(dist_interior, cn_solid, cn_elec, lit=175):
    """RM_UCNCT_3D.f90:68-141 for one frame: (solid, electrolyte) distance,
    halo-padded, from the interior distance and the phases' interior Cn."""
    d = _F(dist_interior)
    ny, nx, nz = d.shape
    cs, ce = _F(cn_solid), _F(cn_elec)
    out_s = np.zeros((ny + 2, nx + 2, nz + 2), order="F")
    out_e = np.zeros_like(out_s)
    lib().orc_rm_ucnct(ny, nx, nz, _p(d), _p(cs), _p(ce), lit, _p(out_s), _p(out_e))
    return out_s, out_e


def rm_mask(psA, cn):
    a, c = np.ascontiguousarray(psA, dtype=np.float64), np.ascontiguousarray(cn, dtype=np.float64)
    out = np.empty_like(a)
    lib().orc_rm_mask(a.size, _p(a), _p(c), _p(out))
    return out


def sign(ds, thr=0.5):
    d = np.ascontiguousarray(ds, dtype=np.float64)
    out = np.empty_like(d)
    lib().orc_sign(d.size, _p(d), thr, _p(out))
    return out


def table(cord, vals, cn):
    cord = np.ascontiguousarray(cord, dtype=np.float64)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    c = np.ascontiguousarray(cn, dtype=np.float64)
    out = np.empty_like(c)
    lib().orc_table(c.size, cord.size, _p(cord), _p(vals), _p(c), _p(out))
    return out


def psi_from_dist(d_interior_f32, zeta):
    d = np.asfortranarray(np.asarray(d_interior_f32, dtype=np.float32))
    ny, nx, nz = d.shape
    psi = np.zeros((ny + 2, nx + 2, nz + 2), order="F")
    lib().orc_psi_from_dist(ny, nx, nz, d.ctypes.data_as(C.POINTER(C.c_float)), zeta, _p(psi))
    return psi


def apply(K, p, scale, diag=None):
    K, p = _F(K), _F(p)
    q = np.zeros_like(p, order="F")
    dg = _p(_F(diag)) if diag is not None else None
    lib().orc_apply(*hdims(p), _p(K), dg, scale, _p(p), _p(q))
    return q


def residual(K, rhs, x, scale, diag=None):
    K, rhs, x = _F(K), _F(rhs), _F(x)
    r = np.zeros_like(x, order="F")
    dg = _p(_F(diag)) if diag is not None else None
    lib().orc_residual(*hdims(x), _p(K), dg, scale, _p(rhs), _p(x), _p(r))
    return r


def cg(K, rhs, x, scale, bc_x0, bc_x1, stop_rule, tol, max_it, w=None, wsum=1.0, diag=None):
    K, rhs = _F(K), _F(rhs)
    x = _F(x).copy(order="F")
    w = _F(w) if w is not None else np.ones_like(x, order="F")
    it = C.c_int(0)
    res = C.c_double(0)
    dg = _p(_F(diag)) if diag is not None else None
    rc = lib().orc_cg(*hdims(x), _p(K), dg, scale, bc_x0, bc_x1, _p(rhs), _p(x), _p(w), wsum,
                      stop_rule, tol, max_it, C.byref(it), C.byref(res))
    return x, dict(iters=it.value, final_res=res.value, status=rc)


def params_reference() -> Params:
    p = Params()
    lib().orc_params_reference(C.byref(p))
    return p


class State:
    """Oracle mirror of the reference program state (orc_state)."""

    def __init__(self, ny, nx, nz, params: Params):
        self.shape = (ny, nx, nz)
        self.params = params
        self._h = lib().orc_state_new(ny, nx, nz, C.byref(params))

    def close(self):
        if self._h:
            lib().orc_state_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self, fid) -> np.ndarray:
        ny, nx, nz = self.shape
        ptr = lib().orc_state_field(self._h, fid)
        n = (ny + 2) * (nx + 2) * (nz + 2)
        a = np.ctypeslib.as_array(ptr, shape=(n,)).copy()
        return a.reshape((ny + 2, nx + 2, nz + 2), order="F")

    def set_field(self, fid, a):
        ny, nx, nz = self.shape
        ptr = lib().orc_state_field(self._h, fid)
        n = (ny + 2) * (nx + 2) * (nz + 2)
        dst = np.ctypeslib.as_array(ptr, shape=(n,))
        dst[:] = _F(a).ravel(order="F")

    def _call(self, name, *args):
        s = Scalars()
        rc = getattr(lib(), name)(self._h, *args, C.byref(s))
        if rc != 0:
            raise RuntimeError(f"{name} -> {rc}")
        return s.as_dict()

    def setup_domain(self, dist_p, dist_e, zeta=0.5, cnp0=2.02e-2, cne0=1.0e-3, cr=6.0):
        dp = np.asfortranarray(np.asarray(dist_p, dtype=np.float32))
        de = np.asfortranarray(np.asarray(dist_e, dtype=np.float32))
        fpt = C.POINTER(C.c_float)
        return self._call("orc_setup_domain", dp.ctypes.data_as(fpt), de.ctypes.data_as(fpt),
                          zeta, cnp0, cne0, cr)

    def ch_step(self, dt):
        return self._call("orc_ch_step", dt)

    def cne_step(self, it, dt):
        return self._call("orc_cne_step", it, dt)

    def bv_update(self):
        return self._call("orc_bv_update")

    def voltage_step(self, dt, vsr):
        return self._call("orc_voltage_step", dt, vsr)

    def time_step(self, it, dt, vsr):
        return self._call("orc_time_step", it, dt, vsr)
