"""Python mirror of openEMS's ``Engine`` + ``Processing`` interface over the engine C ABI.

``Engine_CUDA(op_data)`` plays the role of ``Operator::CreateEngine()`` + ``Engine::Init`` for an
``OperatorData`` built by ``openems_gb300.operator.Operator``: it hands the coefficients and every
extension table to the engine library, registers the probes / FD dumps and captures the step
graph.  ``IterateTS``, ``GetVolt``/``GetCurr``/``SetVolt``/``SetCurr`` and
``GetNumberOfTimesteps`` keep the reference's names (FDTD/engine.h:44-101).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import _native
from .operator import OperatorData

VOLT, CURR = 0, 1


def _p(arr, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


class EngineError(RuntimeError):
    pass


class EngineBase:
    """Drives any library that exports the engine ABI (``lib`` from ``_native``)."""

    def __init__(self, lib: _native.Lib, handle, op: OperatorData, max_timesteps: int, max_classes: int = 0,
                 dump_path: Optional[str] = None):
        self.lib = lib
        self.h = handle
        self.op = op
        self.N = [int(v) for v in op.num_lines]
        self.max_ts = int(max_timesteps)
        self._keep = []
        self.vprobe_ids, self.iprobe_ids, self.dump_ids = [], [], []
        self.fprobe_ids = []
        self.td_dump_ids = []
        # time-domain dump files go to <dump_path>/<dump name>_<numTS>.vtr, as the reference
        # writes them into the simulation path
        self.dump_path = dump_path if dump_path is not None else os.getcwd()
        self._setup(max_classes)

    # --- error handling -------------------------------------------------------------------
    def _ck(self, rc, what):
        if rc != 0:
            msg = self.lib.last_error(self.h)
            msg = msg.decode() if msg else ""
            raise EngineError(f"{what} failed: {_native.ERRORS.get(rc, rc)} {msg}")

    def _a(self, arr, dtype):
        a = np.ascontiguousarray(arr, dtype=dtype)
        self._keep.append(a)
        return a

    # --- setup (Engine::Init + InitExtensions, FDTD/engine.cpp:51-73) ---------------------
    def _setup(self, max_classes):
        op = self.op
        L = self.lib
        f32 = np.float32
        vv, vi, ii, iv = (self._a(a, f32) for a in (op.vv, op.vi, op.ii, op.iv))
        self._ck(L.set_operator(self.h, _p(vv, C.c_float), _p(vi, C.c_float), _p(ii, C.c_float), _p(iv, C.c_float),
                                int(max_classes)), "set_operator")
        self._keep.clear()
        ex = op.exc
        vidx = self._a(ex.volt_index, np.uint32)
        cidx = self._a(ex.curr_index, np.uint32)
        vdir = self._a(ex.volt_dir, np.uint16)
        cdir = self._a(ex.curr_dir, np.uint16)
        vamp = self._a(ex.volt_amp, f32)
        camp = self._a(ex.curr_amp, f32)
        vdel = self._a(ex.volt_delay, np.uint32)
        cdel = self._a(ex.curr_delay, np.uint32)
        sv = self._a(ex.signal_volt, f32)
        sc = self._a(ex.signal_curr, f32)
        self._ck(L.set_excitation(self.h, vamp.size, _p(vidx, C.c_uint), _p(vdir, C.c_ushort), _p(vamp, C.c_float),
                                  _p(vdel, C.c_uint), camp.size, _p(cidx, C.c_uint), _p(cdir, C.c_ushort),
                                  _p(camp, C.c_float), _p(cdel, C.c_uint), _p(sv, C.c_float), _p(sc, C.c_float),
                                  sv.size, int(ex.period)), "set_excitation")
        for u in op.upml:
            st = self._a(u.start, np.uint32)
            nl = self._a(u.num_lines, np.uint32)
            tabs = [self._a(getattr(u, k), f32) for k in ("vv", "vvfo", "vvfn", "ii", "iifo", "iifn")]
            self._ck(L.add_upml(self.h, _p(st, C.c_uint), _p(nl, C.c_uint), *[_p(t, C.c_float) for t in tabs]),
                     "add_upml")
        for m in op.mur:
            cp = self._a(m.coeff_nyP, f32)
            cpp = self._a(m.coeff_nyPP, f32)
            self._ck(L.add_mur(self.h, int(m.ny), int(m.line_nr), int(m.line_nr_shift), int(m.start_ts),
                               _p(cp, C.c_float), _p(cpp, C.c_float)), "add_mur")
        for o in op.lorentz:
            pos = self._a(o.pos, np.uint32)
            t = [self._a(getattr(o, k), f32) for k in ("v_int", "v_ext", "v_lor", "i_int", "i_ext", "i_lor")]
            self._ck(L.add_lorentz_order(self.h, pos.shape[1], _p(pos, C.c_uint), int(o.volt_ade_on),
                                         int(o.curr_ade_on), int(o.volt_lor_on), int(o.curr_lor_on),
                                         *[_p(a, C.c_float) for a in t]), "add_lorentz_order")
        t = getattr(op, "tfsf", None)
        if t is not None:
            a = [self._a(t.volt_index, np.uint32), self._a(t.volt_dir, np.uint16), self._a(t.volt_delay, np.uint32),
                 self._a(t.volt_delta, f32), self._a(t.volt_amp, f32)]
            b = [self._a(t.curr_index, np.uint32), self._a(t.curr_dir, np.uint16), self._a(t.curr_delay, np.uint32),
                 self._a(t.curr_delta, f32), self._a(t.curr_amp, f32)]
            ctypes_of = (C.c_uint, C.c_ushort, C.c_uint, C.c_float, C.c_float)
            sv = self._a(t.signal_volt, f32)
            sc = self._a(t.signal_curr, f32)
            self._ck(L.set_tfsf(self.h, a[4].size, *[_p(x, ct) for x, ct in zip(a, ctypes_of)],
                                b[4].size, *[_p(x, ct) for x, ct in zip(b, ctypes_of)],
                                _p(sv, C.c_float), _p(sc, C.c_float), sv.size, int(t.period), int(t.max_delay)),
                     "set_tfsf")
        cyl = getattr(op, "cylinder", None)
        if cyl is not None:
            vv0 = self._a(cyl.vv_r0, np.float32)
            vi0 = self._a(cyl.vi_r0, np.float32)
            self._ck(L.set_cylinder(self.h, int(cyl.closed_alpha), int(cyl.r0_included),
                                    _p(vv0, C.c_float) if vv0.size else None,
                                    _p(vi0, C.c_float) if vi0.size else None), "set_cylinder")
        r = getattr(op, "rlc", None)
        if r is not None:
            pos = self._a(r.pos, np.uint32)
            dr = self._a(r.dir, np.int32)
            cs = [self._a(getattr(r, k), f32) for k in ("ilv", "i2v", "vv2", "vj1", "vj2", "vvd", "ib0", "b1", "b2")]
            self._ck(L.set_lumped_rlc(self.h, dr.size, _p(pos, C.c_uint), _p(dr, C.c_int),
                                      *[_p(c, C.c_float) for c in cs]), "set_lumped_rlc")
        for p in op.vprobes:
            pid = C.c_int(-1)
            s = self._a(p.start, np.uint32)
            e = self._a(p.stop, np.uint32)
            self._ck(L.add_voltage_probe(self.h, _p(s, C.c_uint), _p(e, C.c_uint), float(p.weight), int(p.interval),
                                         int(p.start_ts), int(min(p.stop_ts, 0xFFFFFFFF)), C.byref(pid)),
                     "add_voltage_probe")
            self._probe_dft(pid.value, p)
            self.vprobe_ids.append(pid.value)
        for p in op.iprobes:
            pid = C.c_int(-1)
            s = self._a(p.start, np.uint32)
            e = self._a(p.stop, np.uint32)
            si = self._a(p.start_inside, np.int32)
            ei = self._a(p.stop_inside, np.int32)
            self._ck(L.add_current_probe(self.h, _p(s, C.c_uint), _p(e, C.c_uint), int(p.norm_dir),
                                         _p(si, C.c_int), _p(ei, C.c_int), float(p.weight), int(p.interval),
                                         int(p.start_ts), int(min(p.stop_ts, 0xFFFFFFFF)), C.byref(pid)),
                     "add_current_probe")
            self._probe_dft(pid.value, p)
            self.iprobe_ids.append(pid.value)
        for p in list(getattr(op, "fprobes", []) or []):
            pid = C.c_int(-1)
            pos = self._a(p.pos, np.uint32)
            el = self._a(p.el, np.float64)     # GetEdgeLength(n, pos) of the main (E) or dual (H) mesh
            self._ck(L.add_field_probe(self.h, int(p.field), _p(pos, C.c_uint), _p(el, C.c_double),
                                       float(p.weight), int(p.interval), int(p.start_ts),
                                       int(min(p.stop_ts, 0xFFFFFFFF)), C.byref(pid)), "add_field_probe")
            self._probe_dft(pid.value, p)
            self.fprobe_ids.append(pid.value)
        td = list(getattr(op, "td_dumps", []) or [])
        if op.dumps or td:
            g = op.grid
            from .operator import _main_delta, _dual_delta, _dual_line
            el = self._a(np.concatenate([_main_delta(l) * g.unit for l in g.lines]), np.float64)
            dl = self._a(np.concatenate([_dual_delta(l) * g.unit for l in g.lines]), np.float64)
            for d in op.dumps:
                did = C.c_int(-1)
                s = self._a(d.start, np.uint32)
                e = self._a(d.stop, np.uint32)
                fr = self._a(d.freqs, np.float64)
                self._ck(L.add_fd_dump(self.h, int(d.field), int(getattr(d, "interp", 2)), _p(s, C.c_uint),
                                       _p(e, C.c_uint), int(d.fd_interval),
                                       fr.size, _p(fr, C.c_double), _p(el, C.c_double), _p(dl, C.c_double),
                                       C.byref(did)), "add_fd_dump")
                rl = getattr(op, "rho_lines", None)
                if rl is not None:         # cylindrical mesh: alpha edges scale with rho
                    rho = self._a(rl[1] if d.dual else rl[0], np.float64)
                    self._ck(L.set_dump_rho(self.h, did.value, _p(rho, C.c_double)), "set_dump_rho")
                self.dump_ids.append(did.value)
            for d in td:
                did = C.c_int(-1)
                s = self._a(d.start, np.uint32)
                e = self._a(d.stop, np.uint32)
                lines = [(_dual_line(np.asarray(l, np.float64)) if d.dual else np.asarray(l, np.float64)) * g.unit
                         for l in g.lines]
                xyz = self._a(np.concatenate([lines[a][int(d.start[a]):int(d.stop[a]) + 1] for a in range(3)]),
                              np.float64)
                prefix = os.path.join(self.dump_path, d.name).encode()
                self._ck(L.add_td_dump(self.h, int(d.field), int(d.interp), _p(s, C.c_uint), _p(e, C.c_uint),
                                       int(d.interval), int(d.start_ts), int(min(d.stop_ts, 0xFFFFFFFF)),
                                       _p(el, C.c_double), _p(dl, C.c_double), _p(xyz, C.c_double), prefix,
                                       C.byref(did)), "add_td_dump")
                self.td_dump_ids.append(did.value)
        self._ck(L.init(self.h, self.max_ts), "init")
        self._keep.clear()

    def _probe_dft(self, pid, p):
        if p.fd_interval and p.freqs:
            fr = self._a(p.freqs, np.float64)
            self._ck(self.lib.set_probe_dft(self.h, pid, int(p.fd_interval), fr.size, _p(fr, C.c_double)),
                     "set_probe_dft")

    # --- Engine API ----------------------------------------------------------------------
    def IterateTS(self, n: int):
        self._ck(self.lib.iterate(self.h, int(n)), "iterate")
        return True

    def sync(self):
        self._ck(self.lib.sync(self.h), "sync")

    def GetNumberOfTimesteps(self) -> int:
        return int(self.lib.num_timesteps(self.h))

    def read_field(self, which: int) -> np.ndarray:
        out = np.empty((3, *self.N), np.float32)
        self._ck(self.lib.read_field(self.h, which, _p(out, C.c_float)), "read_field")
        return out

    def write_field(self, which: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, np.float32)
        self._ck(self.lib.write_field(self.h, which, _p(a, C.c_float)), "write_field")

    def GetVolt(self, n, x, y, z) -> float:
        v = C.c_float()
        self._ck(self.lib.get_value(self.h, VOLT, n, x, y, z, C.byref(v)), "get_value")
        return v.value

    def GetCurr(self, n, x, y, z) -> float:
        v = C.c_float()
        self._ck(self.lib.get_value(self.h, CURR, n, x, y, z, C.byref(v)), "get_value")
        return v.value

    def SetVolt(self, n, x, y, z, value):
        self._ck(self.lib.set_value(self.h, VOLT, n, x, y, z, float(value)), "set_value")

    def SetCurr(self, n, x, y, z, value):
        self._ck(self.lib.set_value(self.h, CURR, n, x, y, z, float(value)), "set_value")

    def _ncomp(self, pid: int) -> int:
        return 3 if pid in self.fprobe_ids else 1

    def probe_series(self, pid: int) -> np.ndarray:
        """Samples of probe `pid` (NaN where no sample was taken); a field probe gives [n][3]."""
        nc = self._ncomp(pid)
        cap = (self.max_ts + 1) * nc
        out = np.empty(cap, np.float64)
        cnt = C.c_size_t(0)
        self._ck(self.lib.read_probe(self.h, pid, _p(out, C.c_double), cap, C.byref(cnt)), "read_probe")
        out = out[:cnt.value]
        return out.reshape(-1, 3) if nc == 3 else out

    def probe_dft(self, pid: int, nf: int) -> np.ndarray:
        """Accumulated DFT of probe `pid` at its nf frequencies; a field probe gives [nf][3]."""
        nc = self._ncomp(pid)
        n = nf * nc
        out = np.zeros(2 * max(n, 1), np.float64)
        self._ck(self.lib.read_probe_dft(self.h, pid, _p(out, C.c_double)), "read_probe_dft")
        z = out[0:2 * n:2] + 1j * out[1:2 * n:2]
        return z.reshape(nf, 3) if nc == 3 else z

    def fd_dump(self, did: int) -> np.ndarray:
        d = self.op.dumps[self.dump_ids.index(did)]
        sz = [int(b) - int(a) + 1 for a, b in zip(d.start, d.stop)]
        n = len(d.freqs) * 3 * sz[0] * sz[1] * sz[2] * 2
        out = np.zeros(max(n, 1), np.float32)
        self._ck(self.lib.read_fd_dump(self.h, did, _p(out, C.c_float), out.size), "read_fd_dump")
        out = out[:n].reshape(len(d.freqs), 3, *sz, 2)
        return out[..., 0] + 1j * out[..., 1]

    def CalcFastEnergy(self) -> float:
        e = C.c_double()
        self._ck(self.lib.energy(self.h, C.byref(e)), "energy")
        return e.value

    def operator_classes(self) -> int:
        n = C.c_uint()
        self._ck(self.lib.operator_classes(self.h, C.byref(n)), "operator_classes")
        return n.value

    def close(self):
        if self.h:
            self.lib.destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine_CUDA(EngineBase):
    """The GB300 engine (``--engine=cuda``): the only product engine, no CPU fallback."""

    def __init__(self, op: OperatorData, max_timesteps: int, device: int = 0, max_classes: int = 0,
                 dump_path: Optional[str] = None):
        lib = _native.load_cuda()
        h = C.c_void_p()
        nl = np.ascontiguousarray(op.num_lines, np.uint32)
        rc = lib.create(_p(nl, C.c_uint), float(op.dt), int(device), C.byref(h))
        if rc != 0:
            msg = lib.last_error(h) if h.value else b""
            raise EngineError(f"oems_cuda_create failed: {_native.ERRORS.get(rc, rc)} {msg!r}")
        super().__init__(lib, h, op, max_timesteps, max_classes, dump_path)

    def write_fd_dump(self, did: int, prefix: Optional[str] = None):
        """Write FD dump `did` as the reference's VTK files (<prefix>_f=<freq>_p=<deg>.vtr,
        _abs, _arg); the prefix defaults to <dump_path>/<dump name>."""
        d = self.op.dumps[self.dump_ids.index(did)]
        g = self.op.grid
        from .operator import _dual_line
        lines = [(_dual_line(np.asarray(l, np.float64)) if d.dual else np.asarray(l, np.float64)) * g.unit
                 for l in g.lines]
        xyz = np.ascontiguousarray(np.concatenate([lines[a][int(d.start[a]):int(d.stop[a]) + 1] for a in range(3)]),
                                   np.float64)
        if prefix is None:
            prefix = os.path.join(self.dump_path, d.name)
        self._ck(self.lib.write_fd_dump(self.h, int(did), prefix.encode(), _p(xyz, C.c_double)), "write_fd_dump")

    def flush_dumps(self):
        """Wait until every time-domain dump file of the steps issued so far is written."""
        self._ck(self.lib.flush_dumps(self.h), "flush_dumps")

    def launches_per_step(self) -> int:
        n = C.c_uint()
        self._ck(self.lib.launches_per_step(self.h, C.byref(n)), "launches_per_step")
        return n.value

    def update_kernels(self):
        """(voltage, current) update kernel names of this engine's configuration."""
        v = C.create_string_buffer(64)
        i = C.create_string_buffer(64)
        self._ck(self.lib.update_kernels(self.h, v, i, 64), "update_kernels")
        return v.value.decode(), i.value.decode()

    def timed_iterate(self, n: int) -> float:
        ms = C.c_float()
        self._ck(self.lib.timed_iterate(self.h, int(n), C.byref(ms)), "timed_iterate")
        return ms.value

    def profile(self, n: int):
        """Run n steps with per-kernel CUDA events: (ms per kernel class, launches per class)."""
        ms = (C.c_float * 6)()
        cnt = (C.c_uint * 6)()
        self._ck(self.lib.profile_steps(self.h, int(n), ms, cnt), "profile_steps")
        return list(ms), list(cnt)

    def probe_range(self, pid: int, first: int, count: int) -> np.ndarray:
        """Sample slots [first, first+count) of probe `pid` ([count][3] for a field probe)."""
        nc = self._ncomp(pid)
        out = np.empty(max(count * nc, 1), np.float64)
        self._ck(self.lib.read_probe_range(self.h, pid, int(first), int(count), _p(out, C.c_double)),
                 "read_probe_range")
        out = out[:count * nc]
        return out.reshape(-1, 3) if nc == 3 else out

    def snapshot(self) -> bytes:
        sz = C.c_size_t()
        self._ck(self.lib.snapshot_size(self.h, C.byref(sz)), "snapshot_size")
        buf = C.create_string_buffer(sz.value)
        self._ck(self.lib.snapshot(self.h, buf, sz.value), "snapshot")
        return buf.raw

    def restore(self, blob: bytes):
        buf = C.create_string_buffer(blob, len(blob))
        self._ck(self.lib.restore(self.h, buf, len(blob)), "restore")
