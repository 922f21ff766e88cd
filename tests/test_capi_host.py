"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every entry point include/nt2cuda.h declares, and validates arguments and
the tuning table without touching a device."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "nt2cuda.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nt2cuda_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_abi():
    syms = header_symbols()
    assert "nt2cuda_blackscholes_f32" in syms and "nt2cuda_sum_outer_f32" in syms
    assert len(syms) >= 50


def test_library_exports_every_declared_symbol(cuda_lib):
    missing = [s for s in header_symbols() if not hasattr(cuda_lib, s)]
    assert not missing, missing


def test_python_binding_matches_header(cuda_lib):
    from nt2_gb300._lib import declared_symbols
    assert sorted(declared_symbols()) == header_symbols()


def test_status_strings(cuda_lib):
    for code in range(10):
        s = cuda_lib.nt2cuda_status_string(code)
        assert s and s != b"unknown status"
    assert cuda_lib.nt2cuda_status_string(99) == b"unknown status"


def test_argument_validation_without_device(cuda_lib):
    L = cuda_lib
    assert L.nt2cuda_saxpy_f32(2.0, None, None, 10, 0, None) == 1
    assert L.nt2cuda_blackscholes_f32(None, None, None, 0.02, 0.3, None, None, 5, 0, 0, None) == 1
    assert L.nt2cuda_dot_f32(None, None, 7, None, 1, None) == 1
    assert L.nt2cuda_sum_outer_f32(None, 3, 3, None, 1, None) == 1
    assert L.nt2cuda_server_create(None, None) == 1
    assert L.nt2cuda_server_submit(None, None, None, None, 0.0, 0.0, 1, None) == 1
    from nt2_gb300._lib import SdStream
    arr = (SdStream * 1)()
    assert L.nt2cuda_sigmadelta_batch_u8(arr, 1, 0, 1, None) == 1
    assert L.nt2cuda_sigmadelta_batch_u8(arr, 0, 4, 1, None) == 1
    assert L.nt2cuda_map_f32(99, None, None, 0, 0, None) in (0, 1)   # unknown op
    assert L.nt2cuda_map_f32(12, None, None, 0, 4, None) == 1     # unknown flag bit
    assert L.nt2cuda_map_f64(14, None, None, 5, 2, None) == 1     # null tables
    assert L.nt2cuda_pow_f32(None, None, None, 5, 0, None) == 1   # null tables
    assert L.nt2cuda_pow_f64(None, None, None, 0, 2, None) == 1   # SIMD128 is not a pow flag
    assert L.nt2cuda_map2_f32(4, None, None, None, 3, 0, None) == 1  # null tables
    assert L.nt2cuda_sincos_f32(0, None, None, None, 3, 0, None) == 1  # null tables
    assert L.nt2cuda_sincos_f64(9, None, None, None, 0, 0, None) == 1  # unknown form
    assert L.nt2cuda_map2_f64(4, None, None, None, 0, 2, None) == 1  # SIMD128 is not a map2 flag


def test_tuning_table_roundtrip(cuda_lib):
    L = cuda_lib
    n = C.c_int()
    assert L.nt2cuda_tuning_import(b"bs_f32@24 4 2\nsaxpy_f32@24 1 1\nbogus@3 9 1\n", C.byref(n)) == 0
    assert n.value == 2
    need = C.c_size_t()
    assert L.nt2cuda_tuning_export(None, 0, C.byref(need)) == 0
    buf = C.create_string_buffer(need.value)
    assert L.nt2cuda_tuning_export(buf, need.value, C.byref(need)) == 0
    text = buf.value.decode()
    assert "bs_f32@24 4 2" in text and "saxpy_f32@24 1 1" in text and "bogus" not in text
    small = C.create_string_buffer(4)
    assert L.nt2cuda_tuning_export(small, 4, C.byref(need)) == 1


def test_demo_programs_compile():
    """NT2's demo statements written against the C++ front end compile (nvcc cross-compiles
    for sm_103a without a GPU), so a change to the kernels' templates cannot break them unseen."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "nt2_gb300", "demo"))
    import build_demos
    assert os.path.exists(build_demos.build())
