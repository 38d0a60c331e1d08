"""The openEMS-side binding (openems_gb300/binding/engine_cuda.{h,cpp}: Operator_CUDA and
Engine_CUDA) compiles against the reference's own headers, unchanged, and links with the
reference's engine objects and the CUDA engine library with every symbol resolved.  Loading the
result needs no GPU.  Needs the openEMS source tree; skipped without it."""
import ctypes
import subprocess

import pytest

from oracle import refengine
from oracle.refbuild import build_ref

pytestmark = pytest.mark.skipif(not build_ref.available(), reason="openEMS source tree not available")


def test_binding_compiles_links_and_loads():
    from openems_gb300 import build
    build.build()
    path = build_ref.build_binding()
    lib = ctypes.CDLL(path)        # RTLD_NOW: fails on any unresolved symbol
    assert lib is not None
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", path], capture_output=True, text=True).stdout
    for sym in ("Engine_CUDA::IterateTS(unsigned int)", "Engine_CUDA::Init()", "Operator_CUDA::CreateEngine()",
                "Operator_CUDA::New()"):
        assert sym in out, sym
