"""CPU checks of the drop-in boundary: the CUDA library loads without a GPU and exports every
entry point include/oems_cuda.h declares (no compute call is made here)."""
import ctypes
import os
import re

from openems_gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "oems_cuda.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(oems_cuda_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    declared = _header_symbols()
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    assert sorted(_native.HEADER_SYMBOLS) == _header_symbols()


def test_load_cuda_binds_all_functions():
    build.build()
    lib = _native.load_cuda()
    for name in list(_native.SIGNATURES) + list(_native.CUDA_ONLY) + ["create"]:
        assert callable(getattr(lib, name))


def test_null_handle_calls_are_rejected_without_a_gpu():
    lib = _native.load_cuda()
    assert lib.init(None, 10) == 1
    assert lib.iterate(None, 1) == 1
    assert lib.num_timesteps(None) == 0
    assert lib.last_error(None) == b"null engine handle"
    lib.destroy(None)
