"""Batched form over the engine C ABI: many Engine_CUDA instances advanced together
(oems_cuda_batch_*).  Each instance keeps its own probes; results equal the serial runs."""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence

import numpy as np

from . import _native
from .engine import Engine_CUDA, EngineError


class BatchEngine:
    def __init__(self, engines: Sequence[Engine_CUDA]):
        self.lib = _native.load_cuda()
        self.engines = list(engines)
        arr = (C.c_void_p * len(self.engines))(*[e.h.value for e in self.engines])
        self.h = C.c_void_p()
        rc = self.lib.batch_create(arr, len(self.engines), C.byref(self.h))
        if rc != 0:
            self.h = None
            raise EngineError(f"oems_cuda_batch_create failed: {_native.ERRORS.get(rc, rc)}")

    PHASES = 0x80000000      # depth flag: per-phase launches instead of one persistent launch
    GROUPED = 0xC0000000     # depth flag: per-phase launches over L2-sized instance groups
    CONCURRENT = 0x20000000  # depth flag: one graph branch per instance with its own step kernels
    CONCURRENT_GROUPED = 0x10000000  # depth flag: CONCURRENT over L2-sized instance groups

    def run(self, steps: Sequence[int], block_size: int = 0, depth: int = 0):
        st = (C.c_uint * len(steps))(*[int(s) for s in steps])
        rc = self.lib.batch_run(self.h, st, int(block_size), int(depth))
        if rc != 0:
            raise EngineError(f"oems_cuda_batch_run failed: {_native.ERRORS.get(rc, rc)}")

    def config(self):
        b, d, n = C.c_uint(), C.c_uint(), C.c_uint()
        g = C.c_int()
        ms = (C.c_float * 16)()
        self.lib.batch_config(self.h, C.byref(b), C.byref(d), C.byref(g), ms, C.byref(n))
        mode = "persistent"
        if d.value & 0x10000000:
            mode = "concurrent per-instance graph branches, L2-sized groups"
        elif d.value & 0x20000000:
            mode = "concurrent per-instance graph branches"
        elif d.value & 0x40000000:
            mode = "per-phase launches, L2-sized groups"
        elif d.value & 0x80000000:
            mode = "per-phase launches"
        return {"block_size": b.value, "depth": d.value & 0x0FFFFFFF, "mode": mode,
                "graph": bool(g.value), "tune_ms": [ms[i] for i in range(n.value)]}

    def close(self):
        if self.h:
            self.lib.batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
