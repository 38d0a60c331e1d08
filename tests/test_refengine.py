"""CPU tests that pin the oracle and the host operator tables to openEMS's own engine.

``oracle/refengine.py`` drives the reference's engine classes compiled unmodified from the openEMS
sources (``oracle/refbuild/build_ref.py``).  Pins:

* every reference engine type (Engine, Engine_sse, Engine_SSE_Compressed, Engine_Multithread) equals
  the C restatement (``oracle/oems_oracle.c``) bit for bit: fields, probe time series, probe DFTs
  and the fast energy, over uneven chunks of steps;
* the excitation signals of ``openems_gb300/excitation.py`` equal the reference's
  ``Excitation::buildExcitationSignal`` bit for bit (the harness rejects a table whose signal,
  period or probe DFT interval differs from the reference's, so every run above checks them too);
* the reference's x86 flush-to-zero build agrees with the denormal-keeping one within round-off.

The reference tree is needed to build the library; without it these tests are skipped.
"""
import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.excitation import Excitation
from oracle import refengine
from oracle.oracle import OracleEngine

from helpers import bits_equal, rel_l2

pytestmark = pytest.mark.skipif(not refengine.available(), reason="openEMS source tree not available")

KINDS = ["basic", "sse", "sse_compressed", "multithread"]

CASES = {
    "smoke": (configs.smoke_case, 60),
    "mixed": (configs.small_mixed, 150),
    "mixed_pec": (lambda: configs.small_mixed(bc=(0, 1, 2, 0, 3, 3), seed=3), 120),
    "cube": (lambda: configs.plain_cube(n=21, steps=200), 200),
    "stress_small": (lambda: configs.stress(shape=(26, 22, 18), steps=120, nblocks=12), 120),
    "mur_corners": (configs.mur_corners, 600),
    "mur_corners_lanes": (lambda: configs.mur_corners(n=(16, 14, 33), wall_source=False, steps=300), 300),
    "patch_small": (lambda: configs.patch(shape=(40, 38, 24), steps=300, with_nf2ff=False), 300),
}


def _run(e, steps):
    first = steps // 3
    e.IterateTS(first)
    e.IterateTS(1)
    e.IterateTS(steps - first - 1)


def _compare(a, b, op):
    for w in (0, 1):
        assert bits_equal(a.read_field(w), b.read_field(w)), f"field {w}"
    for pid in a.vprobe_ids + a.iprobe_ids:
        sa, sb = a.probe_series(pid), b.probe_series(pid)
        assert np.array_equal(np.isnan(sa), np.isnan(sb)) and bits_equal(np.nan_to_num(sa), np.nan_to_num(sb)), \
            f"probe {pid}"
    for pid, p in zip(a.vprobe_ids + a.iprobe_ids, op.vprobes + op.iprobes):
        if p.fd_interval and p.freqs:
            assert bits_equal(a.probe_dft(pid, len(p.freqs)), b.probe_dft(pid, len(p.freqs))), f"dft {pid}"
    assert a.CalcFastEnergy() == b.CalcFastEnergy()


@pytest.mark.parametrize("name", list(CASES))
def test_reference_engines_equal_oracle(name):
    fn, steps = CASES[name]
    op = fn()
    basic = OracleEngine(op, steps)
    mt = OracleEngine(op, steps, threads=3)
    _run(basic, steps)
    _run(mt, steps)
    for kind in KINDS:
        ref = refengine.RefEngine(op, steps, kind=kind, threads=3)
        _run(ref, steps)
        assert ref.GetNumberOfTimesteps() == steps
        _compare(ref, basic, op)
        _compare(ref, mt, op)
        if kind in ("sse_compressed", "multithread"):
            # CompressOperator dedups per 4-lane vector, like the oracle's mt storage
            assert ref.operator_classes() == mt.operator_classes()
        ref.close()


@pytest.mark.parametrize("kind,f0,fc,dt", [
    (Excitation.GAUSSIAN, 2e9, 1e9, 1.9258e-12),
    (Excitation.GAUSSIAN, 3e9, 2e9, 7.3e-13),
    (Excitation.GAUSSIAN, 4.2e9, 2.1e9, 5.1e-13),
    (Excitation.SINUS, 1e9, 0.0, 1.9258e-12),
    (Excitation.SINUS, 7.7e9, 0.0, 3.3e-13),
    (Excitation.DIRAC, 0.0, 0.0, 1.9258e-12),
    (Excitation.STEP, 0.0, 0.0, 1.9258e-12),
])
def test_excitation_signal_equals_reference(kind, f0, fc, dt):
    e = Excitation()
    fmax = 5e9
    if kind == Excitation.GAUSSIAN:
        e.SetupGaussianPulse(f0, fc)
        fmax = f0 + fc
    elif kind == Excitation.SINUS:
        e.SetupSinusoidal(f0)
        fmax = f0
    elif kind == Excitation.DIRAC:
        e.SetupDiracPulse(fmax)
    else:
        e.SetupStepExcite(fmax)
    e.Reset(dt)
    e.buildExcitationSignal(100000)
    op = configs.plain_cube(n=8, steps=10)
    op.excitation = e
    op.dt = dt
    ex = op.exc
    ex.signal_volt = e.volt
    ex.signal_curr = e.curr
    ex.period = e.period_steps()
    # the harness rebuilds the signal with the reference's Excitation and rejects any difference
    ref = refengine.RefEngine(op, 10, kind="basic")
    v, c, nyq, per = ref.signal()
    assert bits_equal(v, e.volt) and bits_equal(c, e.curr)
    assert nyq == e.GetNyquistNum()
    assert per == e.period_steps()
    ref.close()


def test_signal_mismatch_is_rejected():
    op = configs.smoke_case()
    op.exc.signal_volt = op.exc.signal_volt.copy()
    op.exc.signal_volt[5] = np.nextafter(op.exc.signal_volt[5], np.float32(1))
    with pytest.raises(Exception, match="differs from the reference"):
        refengine.RefEngine(op, 10, kind="basic")


def test_flush_to_zero_build_within_roundoff():
    """The reference on x86 flushes denormals in its SSE engines; the difference to the
    denormal-keeping build stays at round-off on the probe series."""
    op = configs.small_mixed()
    a = refengine.RefEngine(op, 300, kind="multithread", threads=3)
    b = refengine.RefEngine(op, 300, kind="multithread", threads=3, ftz=True)
    a.IterateTS(300)
    b.IterateTS(300)
    for pid in a.vprobe_ids + a.iprobe_ids:
        assert rel_l2(b.probe_series(pid), a.probe_series(pid)) < 1e-6
    a.close()
    b.close()


def test_thread_split_is_the_references():
    """Engine_Multithread's x-slab split (Operator_Multithread::CalcStartStopLines)."""
    import ctypes as C
    op = configs.smoke_case()
    ref = refengine.RefEngine(op, 10, kind="multithread", threads=4)
    n = C.c_uint()
    st = (C.c_uint * 8)()
    sp = (C.c_uint * 8)()
    ref._ck(ref.lib.thread_lines(ref.h, C.byref(n), st, sp, 8), "thread_lines")
    nx = int(op.num_lines[0])
    assert n.value == 4
    assert st[0] == 0 and sp[n.value - 1] == nx - 1
    assert all(st[k + 1] == sp[k] + 1 for k in range(n.value - 1))
    ref.close()
