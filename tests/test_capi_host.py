"""CPU checks of the C-ABI boundary and the host-side logic (no GPU calls).

* the CUDA library loads and exports every function include/sbm_capi.h
  declares;
* the ctypes mirrors of sbm_params / sbm_scalars have the C layout;
* the reference parameters keep the Fortran literal kinds;
* the synthetic generator is deterministic and hits its targets.
"""
import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_declared_symbol(built):
    from elsim_gb300 import sbm
    lib = sbm.load_library()
    declared = sbm.declared_symbols()
    assert len(declared) >= 25
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(sbm.LIB_PATH)], capture_output=True,
                         text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(declared) <= exported
    assert sbm.load_library().sbm_version().startswith(b"elsim_gb300")


def test_struct_layout_matches_header(tmp_path):
    from elsim_gb300.sbm import Params, Scalars
    src = tmp_path / "lay.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "sbm_capi.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu\\n\", sizeof(sbm_params),"
        " offsetof(sbm_params, max_it_cne), offsetof(sbm_params, tbl_x),"
        " offsetof(sbm_params, tbl_ocv), sizeof(sbm_scalars), offsetof(sbm_scalars, it_cne));"
        "return 0;}\n")
    exe = tmp_path / "lay"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), "-o", str(exe), str(src)], check=True)
    c_vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True,
                                             text=True).stdout.split()]
    py_vals = [C.sizeof(Params), Params.max_it_cne.offset, Params.tbl_x.offset,
               Params.tbl_ocv.offset, C.sizeof(Scalars), Scalars.it_cne.offset]
    assert c_vals == py_vals


def test_reference_parameters_keep_literal_kinds(built):
    from elsim_gb300 import sbm
    from oracle import sbm_oracle as orc
    p = sbm.reference_params()
    f4 = lambda v: float(np.float32(v))
    assert p.dx == 3.25e-5 * 0.5
    assert p.rho == f4(0.0312) and p.frd == f4(96485.3365)
    assert p.kap_scale == f4(3.3) and p.bvp == f4(-0.1) and p.bve == f4(-0.4495)
    assert p.dab_c0 == f4(-7.02) and p.dab_c2 == f4(0.05)
    assert p.max_it_php == 30001 and p.max_it_cne == 50001 and p.max_it_phe == 100001
    q = orc.params_reference()
    for name, _ in type(p)._fields_:
        a, b = getattr(p, name), getattr(q, name)
        if hasattr(a, "__len__"):
            assert list(a) == list(b), name
        else:
            assert a == b, name


def test_synthetic_generator_is_deterministic_and_hits_fraction():
    from elsim_gb300 import synth
    a = synth.spheres((40, 36, 32), seed=5, solid_fraction=0.6)
    b = synth.spheres((40, 36, 32), seed=5, solid_fraction=0.6)
    assert np.array_equal(a, b)
    assert 0.6 <= a.mean() < 0.62
    t = synth.carve_tunnel(a, seed=5, radius=6)
    assert t.sum() < a.sum() and not (t & ~a).any()
    sg = synth.sign_field(a)
    assert sg.shape == (42, 38, 34) and set(np.unique(sg)) <= {-1.0, 1.0}


def test_missing_library_fails_loudly(tmp_path):
    code = ("import sys; sys.path.insert(0, %r); from elsim_gb300 import sbm; "
            "sbm.LIB_PATH = sbm.Path(%r); sbm._lib = None\n"
            "try:\n    sbm.load_library()\nexcept FileNotFoundError as e:\n"
            "    print('loud', 'no CPU fallback' in str(e))\n") % (str(ROOT), str(tmp_path / "x.so"))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True).stdout
    assert "loud True" in out


def test_entry_points_reject_bad_arguments_before_any_device_work(built):
    """The geometry, connectivity, batch and checkpoint entry points check
    their arguments on the host and return SBM_ERR_ARG (-1) without touching
    the GPU: out-of-range stacking geometries, negative iteration counts,
    unknown operators, null buffers."""
    from elsim_gb300 import sbm
    lib = sbm.load_library()
    dp = C.POINTER(C.c_double)
    vox = np.zeros(12 * 14 * 5)
    out = np.zeros(100000)
    v, o = vox.ctypes.data_as(dp), out.ctypes.data_as(dp)
    # yg > yo; zg > xo; the tunnel loop would leave TmpB; negative offset
    assert lib.sbm_ls_geometry(v, 12, 14, 5, 13, 9, 3, 4, 1.0, o) == sbm.ERR_ARG
    assert lib.sbm_ls_geometry(v, 12, 14, 5, 7, 15, 3, 4, 1.0, o) == sbm.ERR_ARG
    assert lib.sbm_ls_geometry(v, 12, 14, 5, 7, 9, 3, 30, 1.0, o) == sbm.ERR_ARG
    assert lib.sbm_ls_geometry(v, 12, 14, 5, 7, 9, -1, 4, 1.0, o) == sbm.ERR_ARG
    assert lib.sbm_ls_geometry(v, 12, 14, 5, 7, 9, 3, 4, float("nan"), o) == sbm.ERR_ARG
    assert lib.sbm_ls_frontend(v, 12, 14, 5, 7, 9, 3, 4, 1.0, -1, 10, 0.1, o) == sbm.ERR_ARG
    assert lib.sbm_ls_frontend(v, 12, 14, 5, 7, 9, 3, 4, 1.0, 5, -2, 0.1, o) == sbm.ERR_ARG
    assert lib.sbm_allen_cahn(-1, 4, 4, 4, o) == sbm.ERR_ARG
    assert lib.sbm_allen_cahn(3, 0, 4, 4, o) == sbm.ERR_ARG
    assert lib.sbm_connectivity(0, 4, 4, o, 0.75, 10, o, o) == sbm.ERR_ARG
    assert lib.sbm_connectivity(4, 4, 4, o, 0.0, 10, o, o) == sbm.ERR_ARG
    assert lib.sbm_rm_ucnct(4, 4, 4, o, o, o, -1, o, o) == sbm.ERR_ARG
    # batches: null contexts, an unknown operator
    ops = (C.c_int * 1)(7)
    bc = (C.c_int * 1)(0)
    sc = (C.c_double * 1)(1.0)
    hs = (C.c_void_p * 1)(None)
    assert lib.sbm_batch_solve_ops(hs, ops, bc, bc, sc, 1, 1e-8, 100, 1, None, None, None,
                                   None) == sbm.ERR_ARG
    assert lib.sbm_batch_solve(None, 1, 0, 0, 1.0, 1e-8, 100, 1, None, None, None,
                               None) == sbm.ERR_ARG
    # checkpoints: no context
    n = C.c_size_t(0)
    assert lib.sbm_ctx_snapshot_size(None, C.byref(n)) == sbm.ERR_ARG
    assert lib.sbm_ctx_restore(None, None, 0) == sbm.ERR_ARG
