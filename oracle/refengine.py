"""ORACLE -- test infrastructure only: ctypes driver of openEMS's own engine (oracle/_ref).

``RefEngine(op, max_ts, kind=...)`` runs the reference's compiled engine classes through the same
ABI shape as the CUDA engine (``oracle/refbuild/harness.cpp``):

- ``kind="basic"``: ``Engine`` (FDTD/engine.cpp), one thread;
- ``kind="sse"``: ``Engine_sse``;
- ``kind="sse_compressed"``: ``Engine_SSE_Compressed`` over the reference's ``CompressOperator``;
- ``kind="multithread"``: ``Engine_Multithread`` (openEMS's default engine) with ``threads`` workers.

``ftz=True`` loads the library built as the reference runs on x86-64 (its SSE engines flush
denormals to zero); the default keeps denormals, as the reference does on arm64 and as the CUDA
engine does.  The excitation signal is rebuilt by the reference's ``Excitation`` from the operator's
excitation parameters, and the harness rejects a table whose signal, period or probe DFT interval
differs from the reference's.  Field dumps are not driven: ``RefEngine`` drops them from its copy of
the operator data.
"""
import ctypes as C
import dataclasses
import os
import tempfile

import numpy as np

from openems_gb300 import _native
from openems_gb300.engine import EngineBase, EngineError, _p

from .refbuild import build_ref

KINDS = {"basic": 0, "sse": 1, "sse_compressed": 2, "multithread": 3}
_LIBS = {}


def available() -> bool:
    """True when the reference engine was built (it needs the openEMS source tree)."""
    return os.path.exists(build_ref.lib_path(False)) or build_ref.available()


def load(ftz: bool = False):
    key = bool(ftz)
    if key not in _LIBS:
        path = build_ref.lib_path(ftz)
        if build_ref.available():
            build_ref.build()
        if not os.path.exists(path):
            raise RuntimeError(f"reference engine library missing: {path}")
        cdll = C.CDLL(path)
        lib = _native.Lib(cdll, "oems_refeng_")
        f = cdll.oems_refeng_create_ex
        f.restype = C.c_int
        f.argtypes = [_native.PU, _native.PD, C.c_double, C.c_double, C.c_int, C.c_uint, C.c_char_p,
                      C.POINTER(C.c_void_p)]
        lib.fn["create_ex"] = f
        g = cdll.oems_refeng_set_signal
        g.restype = C.c_int
        g.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint]
        lib.fn["set_signal"] = g
        r = cdll.oems_refeng_read_signal
        r.restype = C.c_int
        r.argtypes = [C.c_void_p, _native.PF, _native.PF, C.c_uint, _native.PU, _native.PU, _native.PU]
        lib.fn["read_signal"] = r
        t = cdll.oems_refeng_thread_lines
        t.restype = C.c_int
        t.argtypes = [C.c_void_p, _native.PU, _native.PU, _native.PU, C.c_uint]
        lib.fn["thread_lines"] = t
        _LIBS[key] = lib
    return _LIBS[key]


class RefEngine(EngineBase):
    def __init__(self, op, max_timesteps, kind="multithread", threads=4, ftz=False, scratch=None):
        lib = load(ftz)
        self._tmp = None
        if scratch is None:
            self._tmp = tempfile.TemporaryDirectory(prefix="oems_refeng_")
            scratch = self._tmp.name
        h = C.c_void_p()
        nl = np.ascontiguousarray(op.num_lines, np.uint32)
        if op.grid is not None:
            lines = np.ascontiguousarray(np.concatenate([np.asarray(l, np.float64) for l in op.grid.lines]))
            unit = float(op.grid.unit)
        else:
            lines, unit = None, 1.0
        rc = lib.create_ex(_p(nl, C.c_uint), _p(lines, C.c_double) if lines is not None else None, unit,
                           float(op.dt), KINDS[kind], int(threads), scratch.encode(), C.byref(h))
        if rc != 0:
            raise EngineError(f"oems_refeng_create_ex failed: {_native.ERRORS.get(rc, rc)}")
        ex = getattr(op, "excitation", None)
        if ex is not None and ex.kind is not None:
            rc = lib.set_signal(h, int(ex.kind), float(ex.f0), float(ex.fc), float(ex.f_max), int(ex.length))
            if rc != 0:
                raise EngineError(f"oems_refeng_set_signal failed: {lib.last_error(h)!r}")
        op = dataclasses.replace(op, dumps=[], td_dumps=[])
        self._kind = kind
        super().__init__(lib, h, op, max_timesteps)

    def signal(self):
        """(volt, curr, nyquist, period steps) of the signal the reference's Excitation built."""
        n = C.c_uint()
        self._ck(self.lib.read_signal(self.h, None, None, 0, C.byref(n), None, None), "read_signal")
        v = np.zeros(max(n.value, 1), np.float32)
        c = np.zeros(max(n.value, 1), np.float32)
        ny, per = C.c_uint(), C.c_uint()
        self._ck(self.lib.read_signal(self.h, _p(v, C.c_float), _p(c, C.c_float), n.value, C.byref(n),
                                      C.byref(ny), C.byref(per)), "read_signal")
        return v[:n.value], c[:n.value], ny.value, per.value

    def close(self):
        super().close()
        if self._tmp is not None:
            self._tmp.cleanup()
            self._tmp = None
