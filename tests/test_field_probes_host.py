"""CPU tests of the E/H field probes (probe types 2/3, ProcessFieldProbe) in the oracle.

Pinned by the reference's own contract, TESTSUITE/probes/fieldprobes.m (at a smaller extent, see
``configs.fieldprobes``): a field probe at a point gives, sample for sample, the values of a
time-domain field dump without interpolation at the same Yee node --
* the same number of samples, at the same times (within 1e-13 s; H on the dual time),
* amplitudes within 1e-7 relative (the dump stores float, the probe double),
* max |Ez| of every E probe >= 5e-3 V/m and max |Hx|, |Hy| of every H probe >= 1e-7 A/m;
and by a known answer of the probe DFT (ProcessIntegral::Process, processintegral.cpp:156-167)
restated from the time series, and by basic-vs-multithreaded oracle equality.
"""
import math

import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.operator import _dual_line
from oracle.oracle import OracleEngine

STEPS = 600


@pytest.fixture(scope="module")
def run():
    op = configs.fieldprobes(steps=STEPS)
    e = OracleEngine(op, STEPS)
    e.IterateTS(STEPS)
    return op, e


def _lines(op, dual):
    g = op.grid
    return [(_dual_line(np.asarray(l, np.float64)) if dual else np.asarray(l, np.float64)) for l in g.lines]


@pytest.mark.parametrize("field", [0, 1])
def test_probe_equals_td_dump_at_its_node(run, field):
    op, e = run
    dt = op.dt
    pre = "Et_" if field == 0 else "Ht_"
    faces = ["xn", "xp", "yn", "yp", "zn", "zp"]
    fps = [(pid, p) for pid, p in zip(e.fprobe_ids, op.fprobes) if p.field == field]
    assert len(fps) == 6
    for k, (pid, p) in enumerate(fps):
        di = [d.name for d in op.td_dumps].index(pre + faces[k])
        d = op.td_dumps[di]
        ts, smp = e.td_samples(e.td_dump_ids[di])
        # the dump node nearest the probe's coordinate, as the reference's test looks it up
        lines = _lines(op, d.dual)
        coord = op.fieldprobe_coords[k]
        idx = []
        for a in range(3):
            seg = lines[a][int(d.start[a]):int(d.stop[a]) + 1]
            i = 0 if seg.size == 1 else int(np.argmin(np.abs(seg - coord[a])))
            idx.append(i)
            assert int(d.start[a]) + i == int(p.pos[a])
        dump = smp[:, :, idx[0], idx[1], idx[2]].astype(np.float64)
        s = e.probe_series(pid)
        ok = ~np.isnan(s[:, 0])
        probe = s[ok]
        # vector length and absolute time
        assert probe.shape[0] == dump.shape[0]
        t_probe = (np.nonzero(ok)[0] * p.interval + 0.5 * field) * dt
        t_dump = (ts + 0.5 * field) * dt
        assert np.abs(t_probe - t_dump).max() <= 1e-13
        # amplitudes (0 == 0 passes, as the reference's NaN ratio does)
        assert np.all(np.abs(dump - probe) <= 1e-7 * np.abs(dump)), (p.name, np.abs(dump - probe).max())
        if field == 0:
            assert np.abs(probe[:, 2]).max() >= 5e-3, p.name
        else:
            assert np.abs(probe[:, 0]).max() >= 1e-7 and np.abs(probe[:, 1]).max() >= 1e-7, p.name


def test_probe_dft_known_answer():
    op = configs.fieldprobes(steps=STEPS, freqs=(4e8, 7e8), interval=1)
    e = OracleEngine(op, STEPS)
    e.IterateTS(STEPS)
    dt = op.dt
    for pid, p in zip(e.fprobe_ids, op.fprobes):
        s = e.probe_series(pid)
        assert p.fd_interval > 0
        ts = np.arange(0, STEPS + 1, p.fd_interval)
        t = (ts + 0.5 * p.field) * dt
        want = np.zeros((len(p.freqs), 3), complex)
        for fi, f in enumerate(p.freqs):
            ph = np.exp(-2j * math.pi * f * t)
            want[fi] = (s[ts] * ph[:, None]).sum(axis=0) * 2.0 * dt * p.fd_interval
        got = e.probe_dft(pid, len(p.freqs))
        assert np.allclose(got, want, rtol=1e-9, atol=1e-12 * np.abs(want).max()), p.name


def test_basic_equals_multithreaded():
    op = configs.fieldprobes(half=6, steps=300)
    a = OracleEngine(op, 300)
    b = OracleEngine(op, 300, threads=3)
    for n in (100, 200):
        a.IterateTS(n)
        b.IterateTS(n)
    for pid in a.fprobe_ids:
        assert np.array_equal(a.probe_series(pid), b.probe_series(pid), equal_nan=True)
        assert np.array_equal(a.probe_dft(pid, 1), b.probe_dft(pid, 1))
