"""ORACLE -- test infrastructure only: ctypes driver of the C oracle (oems_oracle.c).

``OracleEngine(op, max_ts)`` runs the basic (single-thread, N-I-J-K) restatement;
``OracleEngine(op, max_ts, threads=T)`` runs the multithreaded SSE-compressed restatement used
as the CPU baseline.  Both are driven through the same ABI shape as the CUDA engine.
"""
import ctypes as C

import numpy as np

from openems_gb300 import _native
from openems_gb300.engine import EngineBase, EngineError, _p

from . import build as _build

_LIB = None


def load():
    global _LIB
    if _LIB is None:
        path = _build.build()
        cdll = C.CDLL(path)
        lib = _native.Lib(cdll, "oems_ref_")
        f = cdll.oems_ref_create
        f.restype = C.c_int
        f.argtypes = [_native.PU, C.c_double, C.c_int, C.POINTER(C.c_void_p)]
        lib.fn["create"] = f
        g = cdll.oems_ref_create_mt
        g.restype = C.c_int
        g.argtypes = [_native.PU, C.c_double, C.c_int, C.POINTER(C.c_void_p)]
        lib.fn["create_mt"] = g
        r = cdll.oems_ref_read_td_sample
        r.restype = C.c_int
        r.argtypes = [C.c_void_p, C.c_int, C.c_uint, _native.PF, _native.PU, _native.PU]
        lib.fn["read_td_sample"] = r
        _LIB = lib
    return _LIB


class OracleEngine(EngineBase):
    def td_samples(self, did):
        """(steps, samples float [n][3][sx][sy][sz]) of time-domain dump `did`."""
        cnt = C.c_uint()
        self._ck(self.lib.read_td_sample(self.h, did, 0, None, None, C.byref(cnt)), "read_td_sample")
        d = self.op.td_dumps[self.td_dump_ids.index(did)]
        shape = (3,) + tuple(int(b) - int(a) + 1 for a, b in zip(d.start, d.stop))
        out = np.zeros((cnt.value,) + shape, np.float32)
        ts = np.zeros(cnt.value, np.int64)
        for k in range(cnt.value):
            t = C.c_uint()
            self._ck(self.lib.read_td_sample(self.h, did, k, _p(out[k], C.c_float), C.byref(t), None), "read_td_sample")
            ts[k] = t.value
        return ts, out

    def __init__(self, op, max_timesteps, threads=0):
        lib = load()
        h = C.c_void_p()
        nl = np.ascontiguousarray(op.num_lines, np.uint32)
        if threads:
            rc = lib.create_mt(_p(nl, C.c_uint), float(op.dt), int(threads), C.byref(h))
        else:
            rc = lib.create(_p(nl, C.c_uint), float(op.dt), 0, C.byref(h))
        if rc != 0:
            raise EngineError(f"oems_ref_create failed: {rc}")
        super().__init__(lib, h, op, max_timesteps)
