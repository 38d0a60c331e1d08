"""CPU tests of the oracle (the checker of the CUDA engine) and of the host operator.

Pins, in the order the reference's own tests hold them:
* engine cross-equality (TESTSUITE/enginetests/cavity.m): the basic and the multithreaded
  SSE-compressed restatements agree bit for bit on every geometry;
* the resonance contract of TESTSUITE/combinedtests/cavity.m (analytic TE/TM modes, same limits);
* known answers: the uniform-vacuum Rennings timestep, CalcNyquistNum, the Gaussian length and the
  excitation index sequence of Engine_Ext_Excitation;
* the committed oracle fixtures (tests/golden/oracle_small.npz).
"""
import json
import math
import os

import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.excitation import Excitation, calc_nyquist_num
from openems_gb300.operator import C0
from oracle.oracle import OracleEngine

from helpers import bits_equal, rel_l2

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name,fn,steps", [
    ("smoke", configs.smoke_case, 60),
    ("mixed", configs.small_mixed, 150),
    ("mixed_pec", lambda: configs.small_mixed(bc=(0, 1, 2, 0, 3, 3), seed=3), 120),
    ("cube", lambda: configs.plain_cube(n=21, steps=200), 200),
    ("stress_small", lambda: configs.stress(shape=(26, 22, 18), steps=120, nblocks=12), 120),
    ("mur_corners", configs.mur_corners, 600),
    ("mur_corners_lanes", lambda: configs.mur_corners(n=(16, 14, 33), wall_source=False, steps=300), 300),
])
def test_basic_equals_multithreaded_sse_compressed(name, fn, steps):
    op = fn()
    a = OracleEngine(op, steps)
    b = OracleEngine(op, steps, threads=3)
    a.IterateTS(steps // 2)
    b.IterateTS(steps // 2)
    a.IterateTS(steps - steps // 2)
    b.IterateTS(steps - steps // 2)
    for w in (0, 1):
        assert bits_equal(a.read_field(w), b.read_field(w)), (name, w)
    for pid in a.vprobe_ids + a.iprobe_ids:
        assert np.array_equal(a.probe_series(pid), b.probe_series(pid), equal_nan=True)
    assert a.CalcFastEnergy() == b.CalcFastEnergy()


def test_vacuum_timestep_known_answer():
    op = configs.plain_cube(n=12, steps=10)
    expect = 1e-3 / (C0 * math.sqrt(3.0))
    assert abs(op.dt / expect - 1) < 1e-7          # float32 EC values, Rennings eq. 4.77
    assert op.nyquist == calc_nyquist_num(3e9, op.dt)


def test_gaussian_and_nyquist_known_answers():
    dt = 1e-3 / (C0 * math.sqrt(3.0))
    e = Excitation()
    e.SetupGaussianPulse(2e9, 1e9)
    e.Reset(dt)
    e.buildExcitationSignal(100000)
    assert e.GetLength() == math.ceil(2.0 * 9.0 / (2.0 * math.pi * 1e9) / dt) == 1488
    assert e.GetNyquistNum() == 86
    assert calc_nyquist_num(0, dt) == 0xFFFFFFFF
    # signal peaks at t0 = 9/(2 pi fc)
    assert abs(e.GetMaxExcitationTimestep() * dt - 9.0 / (2 * math.pi * 1e9)) < 2 * dt
    # truncation to the number of timesteps
    e.buildExcitationSignal(500)
    assert e.GetLength() == 500


def _exc_pos(numTS, delay, p, length):
    e = numTS - delay
    e *= (e > 0)
    e %= p
    e *= (e < length)
    return e


def test_excitation_index_sequence():
    """Engine_Ext_Excitation index arithmetic (engine_ext_excitation.cpp:48-53) against the oracle:
    a single soft source on a 1-edge mesh region reproduces sig[exc_pos(numTS)] increments."""
    op = configs.plain_cube(n=10, steps=40)
    op.exc.volt_delay[:] = 7
    eng = OracleEngine(op, 40)
    x, y, z = (int(v) for v in op.exc.volt_index[:, 0])
    n = int(op.exc.volt_dir[0])
    amp = float(op.exc.volt_amp[0])
    sig = op.exc.signal_volt
    for ts in range(40):
        # isolate the excitation: zero the fields, step once, the source edge holds amp*sig[pos]
        eng.write_field(0, np.zeros((3, 10, 10, 10), np.float32))
        eng.write_field(1, np.zeros((3, 10, 10, 10), np.float32))
        eng.IterateTS(1)
        k = _exc_pos(ts, 7, ts + 1, len(sig))
        assert eng.GetVolt(n, x, y, z) == np.float32(np.float32(0) + np.float32(amp) * sig[k])
    assert [_exc_pos(t, 3, 5, 4) for t in range(12)] == [0, 0, 0, 0, 1, 2, 3, 0, 0, 1, 2, 3]


def test_cavity_resonances_reference_contract():
    """TESTSUITE/combinedtests/cavity.m restated on the oracle (limits in tests/golden)."""
    with open(os.path.join(GOLDEN, "cavity_contract.json")) as fh:
        c = json.load(fh)
    op = configs.cavity(steps=c["steps"])
    eng = OracleEngine(op, c["steps"])
    eng.IterateTS(c["steps"])
    uy = eng.probe_series(eng.vprobe_ids[1])
    uz = eng.probe_series(eng.vprobe_ids[2])
    assert _cavity_check(c, op.dt, uy, uz)


def _fft_time2freq(t, val):
    """matlab/FFT_time2freq.m"""
    dt = t[1] - t[0]
    L = len(val)
    nfft = 1 << int(math.ceil(math.log2(L)))
    v = np.fft.fft(val, nfft) * dt
    f = 1 / (2 * dt) * np.linspace(0, 1, nfft // 2 + 1)
    return f, 2 * v[:nfft // 2 + 1]


def _check_frequency(f, val, f_upper, f_lower, rel_amp, kind):
    """TESTSUITE/helperscripts/check_frequency.m"""
    max1 = val.max()
    for f1, f2 in zip(f_lower, f_upper):
        i1 = int(np.argmin(np.abs(f - f1)))
        i2 = int(np.argmin(np.abs(f - f2)))
        m = val[i1:i2 + 1].max()
        if kind == "inside" and m < max1 * rel_amp:
            return False
        if kind == "outside" and m > max1 * rel_amp:
            return False
    return True


def _cavity_check(c, dt, uy, uz):
    t = np.arange(len(uy)) * dt
    i0 = int(np.argmin(np.abs(t - c["t_start"])))
    f, vy = _fft_time2freq(t[i0:], uy[i0:])
    _, vz = _fft_time2freq(t[i0:], uz[i0:])
    a = int(np.argmin(np.abs(f - c["f_start"])))
    b = int(np.argmin(np.abs(f - c["f_stop"])))
    f, vy, vz = f[a:b + 1], np.abs(vy[a:b + 1]), np.abs(vz[a:b + 1])
    fte, ftm = np.array(c["f_TE"]), np.array(c["f_TM"])

    def outer(fr):
        temp = [c["f_start"]] + list(fr) + [c["f_stop"]]
        o1 = [temp[n] * (1 + c["outer_rel_limit"]) for n in range(len(temp) - 1)]
        o2 = [temp[n + 1] * (1 - c["outer_rel_limit"]) for n in range(len(temp) - 1)]
        return o2, o1
    p1 = _check_frequency(f, vy, fte * (1 + c["upper_rel_limit"]), fte * (1 - c["lower_rel_limit"]),
                          c["min_rel_amplitude"], "inside")
    p2 = _check_frequency(f, vz, ftm * (1 + c["upper_rel_limit_TM"]), ftm * (1 - c["lower_rel_limit_TM"]),
                          c["min_rel_amplitude_TM"], "inside")
    o2, o1 = outer(fte)
    p3 = _check_frequency(f, vy, o2, o1, c["max_rel_amplitude"], "outside")
    o2, o1 = outer(ftm)
    p4 = _check_frequency(f, vz, o2, o1, c["max_rel_amplitude"], "outside")
    return p1 and p2 and p3 and p4


def test_oracle_matches_committed_fixtures():
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    g = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    for name in make_golden.CASES:
        out = make_golden.oracle_case(name)
        for k, v in out.items():
            ref = g[k]
            if np.iscomplexobj(v):
                assert rel_l2(v.real, ref.real) < 1e-6 and rel_l2(v.imag, ref.imag) < 1e-6, k
            else:
                assert rel_l2(v, ref) < 1e-6, k


def test_operator_vacuum_coefficients():
    """Calc_ECOperatorPos on vacuum: vv=1, vi=dt/C, ii=1, iv=dt/L; PEC walls zero the
    tangential vv/vi; the last current lines are zeroed (ApplyMagneticBC)."""
    op = configs.plain_cube(n=8, steps=10)
    eps0, mu0 = 8.85418781762e-12, 1.256637062e-6
    d = 1e-3
    C = np.float32(eps0 * d * d / d)
    L = np.float32(mu0 * d * d / d)
    assert op.vv[0, 3, 3, 3] == 1.0 and op.ii[0, 3, 3, 3] == 1.0
    assert op.vi[0, 3, 3, 3] == np.float32((op.dt / float(C)) / (1.0 + 0.0))
    assert op.iv[0, 3, 3, 3] == np.float32((op.dt / float(L)) / (1.0 + 0.0))
    assert (op.vv[1, 0] == 0).all() and (op.vv[2, 0] == 0).all()     # x=0 wall: Ey, Ez tangential
    assert (op.vv[0, -1] == 0).all()                                   # upper wall: all three
    assert (op.ii[:, -1] == 0).all() and (op.iv[:, :, -1] == 0).all()
