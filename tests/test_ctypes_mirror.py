"""The ctypes mirror elsim_gb300/sbm.py against include/sbm_capi.h, on the
CPU (the library loads without a GPU): every declared function is typed by
load_library(), with the header's arity, a pointer type exactly where the C
parameter is a pointer (with the same element type for scalar and struct
pointers), the C scalar type otherwise, and the C return type."""
import ctypes as C

from capi_header import c_prototypes

SCALAR = {"int": C.c_int, "double": C.c_double, "float": C.c_float, "int64_t": C.c_int64,
          "size_t": C.c_size_t, "uint64_t": C.c_uint64, "uint16_t": C.c_uint16,
          "char": C.c_char}


def _pointee(t):
    return t._type_ if isinstance(t, type) and issubclass(t, C._Pointer) else None


def _check(lib):
    from elsim_gb300 import sbm

    structs = {"sbm_params": sbm.Params, "sbm_scalars": sbm.Scalars}
    protos = c_prototypes()
    assert len(protos) >= 50
    for name, (rbase, rstars, params) in protos.items():
        fn = getattr(lib, name)
        assert fn.argtypes is not None, f"{name} is not typed"
        assert len(fn.argtypes) == len(params), name
        for t, (base, stars, pname) in zip(fn.argtypes, params):
            where = (name, pname, base, stars, t)
            if stars == 0:
                assert t is SCALAR[base], where
                continue
            assert t in (C.c_void_p, C.c_char_p) or _pointee(t) is not None, where
            target = _pointee(t)
            if stars == 1 and target is not None:
                if base in SCALAR:
                    assert target is SCALAR[base], where
                elif base in structs:
                    assert target is structs[base], where
            if t is C.c_char_p:
                assert base == "char" and stars == 1, where
            if stars == 2:
                assert target is not None and (target is C.c_void_p or _pointee(target)), where
        if rstars:
            assert fn.restype in (C.c_char_p, C.c_void_p), name
        else:
            assert fn.restype is SCALAR[rbase], (name, rbase, fn.restype)


def test_every_function_has_the_header_signature(built):
    from elsim_gb300 import sbm

    _check(sbm.load_library())


def test_the_check_catches_a_planted_mismatch(built):
    import pytest
    from elsim_gb300 import sbm

    lib = sbm.load_library()
    fn = lib.sbm_upload
    saved = fn.argtypes
    try:
        fn.argtypes = [saved[0], C.c_int, C.POINTER(C.c_float), C.c_int]  # double* -> float*
        with pytest.raises(AssertionError):
            _check(lib)
    finally:
        fn.argtypes = saved
    _check(lib)
