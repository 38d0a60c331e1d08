"""GPU test of oems_cuda_energy_noalloc, the entry point for callers that cannot allocate device
memory: their device memory is owned by a framework's pool or arena, or they run inside stream
capture.  The caller owns the device fields; the entry point reduces them with the library's
fixed scratch array and must agree with the engine's own energy (oems_cuda_energy) within the
tolerance of the other energy checks (relative 1e-12), on two calls in a row.

This file is collected last so that a failure here does not hide any other test."""
import ctypes as C

import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.engine import Engine_CUDA

pytestmark = pytest.mark.gpu


def _device_copy(torch, field, z_stride):
    """Caller-owned device copy of a host N-I-J-K field with a padded z stride."""
    n, nx, ny, nz = field.shape
    padded = np.zeros((n, nx, ny, z_stride), np.float32)
    padded[..., :nz] = field
    return torch.from_numpy(padded).to("cuda")


def test_energy_noalloc_matches_engine_energy_twice(cuda_lib):
    torch = pytest.importorskip("torch")
    op = configs.small_mixed(steps=120)
    eng = Engine_CUDA(op, 120)
    nl = (C.c_uint * 3)(*[int(v) for v in op.num_lines])
    for steps in (60, 60):                     # two calls in a row, on different field states
        eng.IterateTS(steps)
        ref = eng.CalcFastEnergy()
        z_stride = int(op.num_lines[2]) + 5     # exercise a padded stride
        V = _device_copy(torch, eng.read_field(0), z_stride)
        I = _device_copy(torch, eng.read_field(1), z_stride)
        torch.cuda.synchronize()
        out = C.c_double(-1.0)
        rc = cuda_lib.energy_noalloc(C.c_void_p(V.data_ptr()), C.c_void_p(I.data_ptr()), nl, z_stride,
                                     None, C.byref(out))
        assert rc == 0
        assert ref > 0
        assert abs(out.value - ref) <= 1e-12 * abs(ref)


def test_energy_noalloc_rejects_meshes_beyond_its_scratch(cuda_lib):
    big = (C.c_uint * 3)(8194, 4, 4)
    out = C.c_double(0.0)
    # sizes are checked before any device access, so dummy pointers are never dereferenced
    rc = cuda_lib.energy_noalloc(C.c_void_p(16), C.c_void_p(16), big, 4, None, C.byref(out))
    assert rc == 7                              # OEMS_ERR_TOO_LARGE
