"""CPU tests of the time-domain field dumps (ProcessFieldsTD) in the oracle.

Pinned by
* the sampling schedule of Processing::CheckTimestep (every Nyquist/OverSampling steps from
  numTS = 0, within the start/stop window of a dump);
* a numpy restatement of the three interpolation types of Engine_Interface_FDTD
  (FDTD/engine_interface_fdtd.cpp:63-204) applied to the final fields, against the last sample;
* basic-vs-multithreaded oracle equality of every sample.
"""
import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.operator import _dual_delta, _main_delta
from oracle.oracle import OracleEngine

from helpers import bits_equal


def _raw(F, el, n):
    """GetRawField / GetRawDualField of component n: value / edge length (0 for a zero length)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        d = el[n].reshape([-1 if a == n else 1 for a in range(3)])
        return np.where(d != 0, F[n].astype(np.float64) / d, 0.0)


def interpolate(op, field, interp, F):
    """The reference's interpolated E (field 0) or H (field 1) at every mesh position, float64 [3][N]."""
    g = op.grid
    el = [(_main_delta(l) if field == 0 else _dual_delta(l)) * g.unit for l in g.lines]
    N = [int(v) for v in op.num_lines]
    out = np.zeros((3,) + tuple(N))
    for n in range(3):
        nP, nPP = (n + 1) % 3, (n + 2) % 3
        r = _raw(F, el, n)
        if interp == 0:
            out[n] = r
            continue
        edge = np.zeros(N, bool)
        for a in range(3):
            idx = [slice(None)] * 3
            idx[a] = N[a] - 1
            edge[tuple(idx)] = True

        def sh(a, k):       # r at index i+k along axis a (wrapped; the wrapped rows are masked below)
            return np.roll(r, -k, axis=a)
        if field == 0 and interp == 1:
            dn = el[n].reshape([-1 if a == n else 1 for a in range(3)])
            down = np.roll(dn, 1, axis=n)
            rel = dn / (dn + down)
            o = r * (1.0 - rel) + sh(n, -1) * rel
            idx0 = [slice(None)] * 3
            idx0[n] = 0
            o[tuple(idx0)] = r[tuple(idx0)]
            o = np.where(np.broadcast_to(dn, o.shape) == 0, 0.0, o)
            idxN = [slice(None)] * 3
            idxN[n] = N[n] - 1
            o[tuple(idxN)] = r[tuple([slice(None) if a != n else N[n] - 2 for a in range(3)])]
            out[n] = o
        elif field == 0:
            a = sh(nP, 1)
            b = np.roll(a, -1, axis=nPP)
            c = sh(nPP, 1)
            out[n] = np.where(edge, 0.0, (((r + a) + b) + c) / 4)
        elif interp == 1:
            a = sh(nP, -1)
            b = np.roll(a, 1, axis=nPP)
            c = sh(nPP, -1)
            o = (((r + a) + b) + c) / 4
            lowP = np.zeros(N, bool)
            idx = [slice(None)] * 3
            idx[nP] = 0
            lowP[tuple(idx)] = True
            lowPP = np.zeros(N, bool)
            idx = [slice(None)] * 3
            idx[nPP] = 0
            lowPP[tuple(idx)] = True
            out[n] = np.where(edge | lowP | lowPP, 0.0, o)
        else:
            dn = el[n].reshape([-1 if a == n else 1 for a in range(3)])
            up = np.roll(dn, -1, axis=n)
            rel = dn / (dn + up)
            o = r * (1.0 - rel) + sh(n, 1) * rel
            idxN = [slice(None)] * 3
            idxN[n] = N[n] - 1
            o[tuple(idxN)] = 0.0
            out[n] = o
    return out


def test_schedule_and_interpolation_known_answers():
    steps = 120                      # a multiple of the dumps' interval (5): the last step is a sample
    op = configs.td_dumps(steps=steps)
    eng = OracleEngine(op, steps)
    eng.IterateTS(steps)
    V, I = eng.read_field(0), eng.read_field(1)
    for did, d in zip(eng.td_dump_ids, op.td_dumps):
        ts, smp = eng.td_samples(did)
        want = [t for t in range(0, steps + 1) if t % d.interval == 0 and d.start_ts <= t <= d.stop_ts]
        assert ts.tolist() == want, d.name
        assert not smp[0].any() or d.start_ts > 0           # numTS = 0: all fields zero
        if ts[-1] != steps:
            continue
        ref = interpolate(op, d.field, d.interp, V if d.field == 0 else I)
        box = ref[:, d.start[0]:d.stop[0] + 1, d.start[1]:d.stop[1] + 1, d.start[2]:d.stop[2] + 1].astype(np.float32)
        assert bits_equal(smp[-1], box), d.name
        assert np.abs(box).max() > 0, d.name


def test_basic_equals_multithreaded_td_samples():
    steps = 90
    op = configs.td_dumps(steps=steps)
    a = OracleEngine(op, steps)
    b = OracleEngine(op, steps, threads=3)
    for n in (31, 59):
        a.IterateTS(n)
        b.IterateTS(n)
    for did in a.td_dump_ids:
        ta, sa = a.td_samples(did)
        tb, sb = b.td_samples(did)
        assert np.array_equal(ta, tb) and bits_equal(sa, sb)
