"""CPU tests of the lumped RLC restatement (Operator_Ext_LumpedRLC + Engine_Ext_LumpedRLC).

No reference test covers the lumped RLC loads, so they are pinned here by
* known answers of the table build: the element count of each box (edges along the direction
  times the parallel cross-section), the parallel coefficients ilv = dT/dL and
  i2v = (dT/dC)/(1 + dT dG/(2 dC)) with the per-edge dL, dC of the reference's split, and the
  short-circuit series coefficients for C = 0;
* engine cross-equality (basic and multithreaded oracle bit for bit);
* a physics contract: a parallel LC on one edge of a PEC box, kicked by a soft source, rings at
  1/(2 pi sqrt(LC)) within 2 % (the edge's own capacitance lowers it slightly).
"""
import math

import numpy as np
import pytest

from openems_gb300 import configs
from oracle.oracle import OracleEngine

from helpers import bits_equal


def test_table_known_answers():
    op = configs.lumped_rlc(steps=50)
    r = op.rlc
    # series_rlc: 2 z edges x 1; series_rl: 2 x edges x 2 parallel; parallel_rlc: 2 y edges;
    # parallel_l: 1 z edge -- in the order the properties were defined
    assert r.dir.tolist() == [2, 2, 0, 0, 0, 0, 1, 1, 2]
    dT = op.dt
    # parallel RLC: N0 = 2 edges in series, Npar = 1 -> dL = L/2, dC = 2C, dG = 2/R
    dL, dC, dG = 3e-9 / 2, 0.2e-12 * 2, (1 / 100.0) * 2
    assert r.ilv[6] == np.float32(dT / dL)
    assert r.i2v[6] == np.float32((dT / dC) / (1.0 + dT * dG / (2.0 * dC)))
    assert r.vvd[6] == 1 and r.ib0[6] == 0
    # series RL with C = 0: N0 = 2, Npar = 2 -> dL = L, dR = R
    dL, dR = 1e-9, 20.0
    assert r.ib0[2] == np.float32(dT / (2.0 * dL + dT * dR))
    assert r.b1[2] == np.float32(-4.0 * dL / dT)
    assert r.b2[2] == np.float32((2.0 * dL - dT * dR) / dT)
    assert (r.ilv[:6] == 0).all() and (r.i2v[:6] == 0).all()
    # the element edges' coefficients were rewritten from the modified EC (Calc_ECOperatorPos)
    for k in range(r.dir.size):
        x, y, z = (int(v) for v in r.pos[:, k])
        assert op.vi[r.dir[k], x, y, z] > 0


@pytest.mark.parametrize("name,kw,steps", [
    ("mur", dict(), 300),
    ("upml_dispersive", dict(bc=(3,) * 6, dispersive=True), 240),
    ("pec", dict(bc=(0,) * 6), 240),
])
def test_basic_equals_multithreaded_with_lumped_rlc(name, kw, steps):
    op = configs.lumped_rlc(steps=steps, **kw)
    a = OracleEngine(op, steps)
    b = OracleEngine(op, steps, threads=3)
    for n in (steps // 3, steps - steps // 3):
        a.IterateTS(n)
        b.IterateTS(n)
    for w in (0, 1):
        assert bits_equal(a.read_field(w), b.read_field(w)), (name, w)
    for pid in a.vprobe_ids + a.iprobe_ids:
        s = a.probe_series(pid)
        assert np.array_equal(s, b.probe_series(pid), equal_nan=True)
        assert np.isfinite(s[~np.isnan(s)]).all()


@pytest.mark.parametrize("L,C", [(1e-9, 1e-12), (0.5e-9, 4e-12)])
def test_lc_tank_rings_at_the_lc_frequency(L, C):
    steps = 8000
    op = configs.lc_tank(L=L, C=C, steps=steps)
    e = OracleEngine(op, steps)
    e.IterateTS(steps)
    u = e.probe_series(e.vprobe_ids[0])[2000:]
    u = u - u.mean()
    nf = 1 << 20
    spec = np.abs(np.fft.rfft(u * np.hanning(len(u)), nf))
    f = np.fft.rfftfreq(nf, op.dt)
    f_peak = f[np.argmax(spec)]
    f0 = 1 / (2 * math.pi * math.sqrt(L * C))
    assert abs(f_peak / f0 - 1) < 2e-2, (f_peak, f0)
