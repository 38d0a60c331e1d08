"""Physics contracts of the reference's own test suite, run on the oracle (CPU).

* TESTSUITE/combinedtests/Coax.m: a PEC coaxial line (radii 100 / 230 / 240 mm, 5 mm mesh, 1 m
  long, PML_8 at the far end, radially weighted excitation) must show |U/I| within +3 % / -1 % of
  the analytic Z0 = sqrt(mu0/eps0) ln(230/100) / (2 pi) at every FFT frequency from 0 to 1 GHz
  (the FFT of ReadUI/FFT_time2freq: zero padded to the next power of two).  This pins the
  cylinder primitives, the weighted excitation, the PML grading of a one-sided PML and both
  probe types.
* UPML absorption: a point source in a 30^3 box with an 8-cell UPML on every wall matches the
  same source in a 90^3 box (whose walls are out of reach in the time window) within 2 %.
"""
import math
import os

import numpy as np

from openems_gb300 import configs
from openems_gb300.excitation import Excitation
from openems_gb300.operator import EPS0, MUE0, Grid, Operator, Structure
from oracle.oracle import OracleEngine

THREADS = min(16, os.cpu_count() or 1)


def coax_impedance(eng, op):
    u = eng.probe_series(eng.vprobe_ids[0])
    i = eng.probe_series(eng.iprobe_ids[0])
    nfft = 1 << int(math.ceil(math.log2(len(u))))
    U = np.fft.rfft(u, nfft)
    I = np.fft.rfft(i, nfft)
    f = np.fft.rfftfreq(nfft, op.dt)
    sel = f <= 1e9
    return f[sel], np.abs(U[sel] / I[sel])


def coax_z0():
    return math.sqrt(MUE0 / EPS0) * math.log(230 / 100) / (2 * math.pi)


def test_coax_impedance_reference_contract():
    op = configs.coax(steps=5000)
    eng = OracleEngine(op, 5000, threads=THREADS)
    eng.IterateTS(5000)
    f, Z = coax_impedance(eng, op)
    Z0 = coax_z0()
    assert f.size > 50
    assert (Z <= Z0 * 1.03).all() and (Z >= Z0 * 0.99).all(), (Z.min() / Z0, Z.max() / Z0)


def _point_source(n, steps):
    g = Grid([np.arange(n, dtype=float)] * 3, unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(10e9, 8e9)
    c = n // 2
    csx.AddExcitation("s", 0, [0, 0, 1.0]).AddBox([c, c, c], [c, c, c + 1])
    csx.AddProbe("p", 0, interval=1).AddBox([c + 6, c, c], [c + 6, c, c + 1])
    op = Operator(csx, g, exc, bc=(3,) * 6, pml_size=(8,) * 6)
    eng = OracleEngine(op.build(steps), steps, threads=THREADS)
    eng.IterateTS(steps)
    return eng.probe_series(eng.vprobe_ids[0])


def test_upml_absorbs_like_open_space():
    steps = 220
    big = _point_source(90, steps)
    small = _point_source(30, steps)
    assert np.abs(small - big).max() < 2e-2 * np.abs(big).max()
