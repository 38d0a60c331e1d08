"""CPU tests of the TFSF plane-wave restatement (Operator_Ext_TFSF + Engine_Ext_TFSF).

The reference has no test that pins the plane-wave tables, so they are pinned here by
* known answers of the build: H = k x E / Z0, the active faces of a box that touches the mesh
  walls, the polarisation correction, the term count and order of the engine tables;
* the numerical dispersion relation: the phase velocity CalcNumericPhaseVelocity returns makes
  the Yee relation sum_n (sin(k d_n Dn / 2) / Dn)^2 = (sin(w dt / 2) / (c dt))^2 hold;
* engine cross-equality (basic and multithreaded oracle bit for bit, TESTSUITE/enginetests style);
* the physics contract of a total-field/scattered-field source: in vacuum the scattered-field
  region stays empty (energy below 1e-4 of the total-field peak), while a metal brick inside the
  box scatters into it.
"""
import math

import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.operator import C0, Z0
from oracle.oracle import OracleEngine

from helpers import bits_equal

OBLIQUE = dict(k_dir=(1.0, 0.5, -0.3), e_dir=(0.0, 0.5, 1.0), frequency=10e9, graded=True)


def test_tables_known_answers():
    op = configs.plane_wave(steps=50, scatterer=False)
    t = op.tfsf
    assert t.phase_velocity == C0                      # no frequency: c0 / sqrt(eps mu)
    np.testing.assert_array_equal(t.h_amp, [0.0, -1.0 / Z0, 0.0])
    assert t.active.all()
    nl = t.stop - t.start + 1
    # two components per position on each of the six face planes
    count = sum(2 * 2 * int(nl[(n + 1) % 3] * nl[(n + 2) % 3]) for n in range(3))
    assert t.volt_amp.size == count and t.curr_amp.size == count
    # first terms: x lower plane, component y then z, voltage at the Start line, current one line below
    assert tuple(t.volt_index[:, 0]) == tuple(t.start) and t.volt_dir[0] == 1 and t.volt_dir[1] == 2
    assert t.curr_index[0, 0] == t.start[0] - 1
    # x lower plane: with E = z and H = -y, V_y (driven by H_z) and I_z (driven by E_y) get nothing
    face = 2 * int(nl[1] * nl[2])
    assert not t.volt_amp[0:face:2].any() and t.volt_amp[1:face:2].any()
    assert not t.curr_amp[1:face:2].any() and t.curr_amp[0:face:2].any()
    assert int(t.volt_delay.max()) + 1 <= t.max_delay and int(t.curr_delay.max()) + 1 <= t.max_delay


def test_box_on_walls_turns_faces_off():
    op = configs.plane_wave(steps=50, scatterer=False, box=([0, 6, 5], [20, 23, 19]))
    t = op.tfsf
    assert t.active.tolist() == [[False, True], [True, False], [True, True]]
    nl = t.stop - t.start + 1
    count = sum(2 * int(t.active[n].sum()) * int(nl[(n + 1) % 3] * nl[(n + 2) % 3]) for n in range(3))
    assert t.volt_amp.size == count and t.curr_amp.size == count
    # the only x plane left is the upper one
    xs = t.volt_index[0][:2 * int(nl[1] * nl[2])]
    assert (xs == t.stop[0]).all()


def test_polarisation_is_made_orthogonal():
    op = configs.plane_wave(steps=50, scatterer=False, **OBLIQUE)
    t = op.tfsf
    d = np.array(OBLIQUE["k_dir"]) / np.linalg.norm(OBLIQUE["k_dir"])
    np.testing.assert_allclose(t.prop_dir, d, rtol=0, atol=1e-15)
    assert abs(float(np.dot(t.e_amp, t.prop_dir))) < 1e-15
    np.testing.assert_allclose(t.h_amp, np.cross(t.prop_dir, t.e_amp) / Z0, rtol=1e-14)


@pytest.mark.parametrize("k_dir", [(1.0, 0.0, 0.0), (0.0, -1.0, 0.0), (1.0, 0.5, -0.3), (0.2, 1.0, 0.7)])
def test_numeric_phase_velocity_satisfies_yee_dispersion(k_dir):
    f = 12e9
    op = configs.plane_wave(steps=50, scatterer=False, k_dir=k_dir, e_dir=(0.0, 0.0, 1.0) if k_dir[2] == 0 else
                            (1.0, 0.0, 0.0), frequency=f)
    t = op.tfsf
    d = t.prop_dir
    # the mesh is uniform, so the mean deltas are the pitch (1 mm) on every axis
    dx = 1e-3
    ff = float(np.float32(f))
    k = 2 * math.pi * ff / t.phase_velocity
    lhs = sum((math.sin(d[n] * k * dx / 2) / dx) ** 2 for n in range(3))
    rhs = (math.sin(2 * math.pi * ff * op.dt / 2) / C0 / op.dt) ** 2
    assert abs(lhs - rhs) <= 1e-6 * rhs
    assert t.phase_velocity < C0


@pytest.mark.parametrize("name,kw,steps", [
    ("upml", dict(), 160),
    ("oblique_mur_dispersive", dict(bc=(2,) * 6, dispersive=True, box=([0, 6, 5], [20, 23, 19]), **OBLIQUE), 160),
    ("sinus_periodic", dict(k_dir=(-0.2, -1.0, 0.4), e_dir=(1.0, 0.0, 0.5), sinus=True), 160),
])
def test_basic_equals_multithreaded_with_tfsf(name, kw, steps):
    op = configs.plane_wave(steps=steps, **kw)
    a = OracleEngine(op, steps)
    b = OracleEngine(op, steps, threads=3)
    for n in (steps // 3, steps - steps // 3):
        a.IterateTS(n)
        b.IterateTS(n)
    for w in (0, 1):
        assert bits_equal(a.read_field(w), b.read_field(w)), (name, w)
    for pid in a.vprobe_ids + a.iprobe_ids:
        assert np.array_equal(a.probe_series(pid), b.probe_series(pid), equal_nan=True)
    assert np.nanmax(np.abs(a.probe_series(a.vprobe_ids[0]))) > 0


def _region_energies(op, steps, every=10, pml=5):
    eng = OracleEngine(op, steps)
    t = op.tfsf
    N = tuple(int(v) for v in op.num_lines)
    tf = np.zeros(N, bool)
    tf[t.start[0]:t.stop[0] + 1, t.start[1]:t.stop[1] + 1, t.start[2]:t.stop[2] + 1] = True
    core = np.zeros(N, bool)
    core[pml + 1:-pml - 1, pml + 1:-pml - 1, pml + 1:-pml - 1] = True
    sf = core & ~tf
    e_tf, e_sf = [], []
    for _ in range(steps // every):
        eng.IterateTS(every)
        V = eng.read_field(0).astype(np.float64)
        e_tf.append(float((V[:, tf] ** 2).sum()))
        e_sf.append(float((V[:, sf] ** 2).sum()))
    return max(e_tf), max(e_sf)


def test_vacuum_scattered_field_region_stays_empty():
    for kw in (dict(), OBLIQUE):
        e_tf, e_sf = _region_energies(configs.plane_wave(steps=300, scatterer=False, **kw), 300)
        assert e_tf > 0
        assert e_sf < 1e-4 * e_tf, (kw, e_sf / e_tf)


def test_metal_brick_scatters_into_the_scattered_field_region():
    e_tf, e_sf = _region_energies(configs.plane_wave(steps=300, scatterer=True), 300)
    assert e_sf > 1e-3 * e_tf
