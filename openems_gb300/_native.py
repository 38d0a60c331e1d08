"""ctypes binding of the engine C ABI (include/oems_cuda.h).

``load_cuda()`` loads the in-tree CUDA library and raises if it is missing: the engine has no
CPU fallback.  ``bind(lib, prefix)`` attaches argument types for any library exporting the same
ABI shape under ``prefix`` (the tests use this to drive their CPU checker with identical calls).
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CUDA_LIB = os.path.join(HERE, "_build", "liboems_cuda.so")

OEMS_OK = 0
ERRORS = {1: "OEMS_ERR_ARG", 2: "OEMS_ERR_CUDA", 3: "OEMS_ERR_STATE", 4: "OEMS_ERR_UNSUPPORTED",
          5: "OEMS_ERR_DEVICE", 6: "OEMS_ERR_NOMEM", 7: "OEMS_ERR_TOO_LARGE", 8: "OEMS_ERR_IO"}

P = C.c_void_p
U = C.c_uint
I = C.c_int
D = C.c_double
F = C.c_float
SZ = C.c_size_t
PU = C.POINTER(C.c_uint)
PI_ = C.POINTER(C.c_int)
PF = C.POINTER(C.c_float)
PD = C.POINTER(C.c_double)
PUS = C.POINTER(C.c_ushort)
PSZ = C.POINTER(C.c_size_t)

# name -> (restype, argtypes); the create call differs per library and is bound separately
SIGNATURES = {
    "destroy": (None, [P]),
    "last_error": (C.c_char_p, [P]),
    "set_operator": (I, [P, PF, PF, PF, PF, U]),
    "operator_classes": (I, [P, PU]),
    "set_excitation": (I, [P, U, PU, PUS, PF, PU, U, PU, PUS, PF, PU, PF, PF, U, U]),
    "add_upml": (I, [P, PU, PU, PF, PF, PF, PF, PF, PF]),
    "add_mur": (I, [P, I, U, U, U, PF, PF]),
    "add_lorentz_order": (I, [P, U, PU, I, I, I, I, PF, PF, PF, PF, PF, PF]),
    "set_tfsf": (I, [P, U, PU, PUS, PU, PF, PF, U, PU, PUS, PU, PF, PF, PF, PF, U, U, U]),
    "set_lumped_rlc": (I, [P, U, PU, PI_, PF, PF, PF, PF, PF, PF, PF, PF, PF]),
    "add_voltage_probe": (I, [P, PU, PU, D, U, U, U, PI_]),
    "add_current_probe": (I, [P, PU, PU, I, PI_, PI_, D, U, U, U, PI_]),
    "add_field_probe": (I, [P, I, PU, PD, D, U, U, U, PI_]),
    "set_cylinder": (I, [P, I, I, PF, PF]),
    "set_dump_rho": (I, [P, I, PD]),
    "set_probe_dft": (I, [P, I, U, U, PD]),
    "add_fd_dump": (I, [P, I, I, PU, PU, U, U, PD, PD, PD, PI_]),
    "add_td_dump": (I, [P, I, I, PU, PU, U, U, U, PD, PD, PD, C.c_char_p, PI_]),
    "init": (I, [P, U]),
    "iterate": (I, [P, U]),
    "sync": (I, [P]),
    "num_timesteps": (U, [P]),
    "read_field": (I, [P, I, PF]),
    "write_field": (I, [P, I, PF]),
    "get_value": (I, [P, I, U, U, U, U, PF]),
    "set_value": (I, [P, I, U, U, U, U, F]),
    "read_probe": (I, [P, I, PD, SZ, PSZ]),
    "read_probe_dft": (I, [P, I, PD]),
    "read_fd_dump": (I, [P, I, PF, SZ]),
    "energy": (I, [P, PD]),
}

CUDA_ONLY = {
    "set_operator_sse_compressed": (I, [P, U, PF, PF, PF, PF, PU]),
    "snapshot_size": (I, [P, PSZ]),
    "snapshot": (I, [P, P, SZ]),
    "restore": (I, [P, P, SZ]),
    "launches_per_step": (I, [P, PU]),
    "update_kernels": (I, [P, C.c_char_p, C.c_char_p, SZ]),
    "timed_iterate": (I, [P, U, PF]),
    "profile_steps": (I, [P, U, PF, PU]),
    "read_probe_range": (I, [P, I, SZ, SZ, PD]),
    "flush_dumps": (I, [P]),
    "write_fd_dump": (I, [P, I, C.c_char_p, PD]),
    "energy_noalloc": (I, [P, P, PU, U, P, PD]),
    "batch_create": (I, [C.POINTER(P), U, C.POINTER(P)]),
    "batch_run": (I, [P, PU, U, U]),
    "batch_config": (I, [P, PU, PU, PI_, PF, PU]),
    "batch_destroy": (None, [P]),
    "adjoint_setup": (I, [P, U, PU, PU]),
    "adjoint_forward": (I, [P, U]),
    "adjoint_backward": (I, [P, U, PI_, PD, PD, PD]),
    "adjoint_timing": (I, [P, PF, PF, PU]),
    "nf2ff": (I, [P, U, PI_, PI_, PD, U, D, U, PD, U, PD, PD, D, D, D, PD, PD, PD, PD, PD]),
    "opbuild_create": (I, [PU, PD, D, U, PD, PD, PD, PD, C.POINTER(P)]),
    "opbuild_ec": (I, [P, PF, PF, PF, PF, PD]),
    "opbuild_coefficients": (I, [P, D, PF, PF, PF, PF]),
    "opbuild_last_error": (C.c_char_p, [P]),
    "opbuild_destroy": (None, [P]),
}

KERNEL_CLASSES = ["update_v", "update_i", "mur", "lorentz", "excite", "step_end"]

# every symbol include/oems_cuda.h declares
HEADER_SYMBOLS = ["oems_cuda_create"] + ["oems_cuda_" + k for k in list(SIGNATURES) + list(CUDA_ONLY)]


class Lib:
    """Bound function table of one library (``fn.<name>`` without the prefix)."""

    def __init__(self, cdll, prefix, extra=None):
        self.cdll = cdll
        self.prefix = prefix
        table = dict(SIGNATURES)
        if extra:
            table.update(extra)
        self.fn = {}
        for name, (res, args) in table.items():
            f = getattr(cdll, prefix + name)
            f.restype = res
            f.argtypes = args
            self.fn[name] = f

    def __getattr__(self, name):
        try:
            return self.__dict__["fn"][name]
        except KeyError:
            raise AttributeError(name)


_CUDA = None


def load_cuda() -> Lib:
    """Load the CUDA engine library; raises RuntimeError if it was not built."""
    global _CUDA
    if _CUDA is None:
        if not os.path.exists(CUDA_LIB):
            raise RuntimeError(f"CUDA engine library missing: {CUDA_LIB} (run __graft_entry__.build())")
        cdll = C.CDLL(CUDA_LIB)
        lib = Lib(cdll, "oems_cuda_", CUDA_ONLY)
        f = cdll.oems_cuda_create
        f.restype = I
        f.argtypes = [PU, D, I, C.POINTER(P)]
        lib.fn["create"] = f
        _CUDA = lib
    return _CUDA
