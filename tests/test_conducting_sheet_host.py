"""CPU tests of the conducting-sheet restatement (Operator_Ext_ConductingSheet on the dispersive
engine path).

No reference test covers the sheet model, so it is pinned by
* the DC sheet conductance: in steady state a voltage ADE branch carries J = v_ext V / (1 - v_int),
  i.e. a conductance v_ext / ((1 - v_int) vi), and the edge's own conductance follows from vv and
  vi.  Their sum over a sheet edge of a uniform mesh (edge length = node width) must be
  G0 (g + 1/r1 + 1/r2) of the model's row for the frequency range (w_max / w0), with
  G0 = conductivity * thickness and w0 = 8 / (G0 thickness mu0), or half of it on the sheet's
  rim (the reference's factor 2); a thin, low-conductance sheet uses the first row, whose DC
  conductance is G0 itself;
* the fallback to PEC for a volume of sheet material and inside the boundary layer;
* engine cross-equality (basic and multithreaded oracle bit for bit);
* shielding: a copper sheet between a source and a probe passes no more than a metal plate does,
  within a factor of two, and both less than 1e-3 of the field on the source side.
"""
import numpy as np
import pytest

from openems_gb300 import condsheet_table as T
from openems_gb300 import configs
from openems_gb300.excitation import Excitation
from openems_gb300.operator import MUE0, Grid, Operator, Structure
from oracle.oracle import OracleEngine

from helpers import bits_equal


def _uniform_sheet(sigma, thickness, fmax):
    g = Grid([np.arange(16.0), np.arange(14.0), np.arange(12.0)], unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(fmax / 2, fmax / 2)
    csx.AddConductingSheet("s", sigma, thickness).AddBox([3, 3, 6], [12, 10, 6])
    csx.AddExcitation("src", 0, [0, 0, 1.0]).AddBox([7, 7, 3], [7, 7, 4])
    op = Operator(csx, g, exc, bc=(0,) * 6)
    return op.build(50)


@pytest.mark.parametrize("sigma,thickness", [(5.8e7, 35e-6), (1e6, 2e-6), (1e3, 1e-6)])
def test_dc_sheet_conductance(sigma, thickness):
    op = _uniform_sheet(sigma, thickness, 10e9)
    o1, o2 = op.lorentz
    G0 = float(np.float32(np.float32(sigma) * np.float32(thickness)))
    w0 = float(np.float32(8.0 / G0 / float(np.float32(thickness)) / MUE0))
    om = float(np.float32(np.float32(op.excitation.f_max * 2 * np.pi) / np.float32(w0)))
    k = next(i for i, w in enumerate(T.OMEGA_STOP) if w > om)
    S = T.G[k] + 1 / T.R1[k] + 1 / T.R2[k]        # the row's DC conductance in units of G0
    ratios = []
    for i in range(o1.pos.shape[1]):
        x, y, z = (int(v) for v in o1.pos[:, i])
        for n in range(2):                        # the tangential components of the z-normal sheet
            if o1.v_ext[n, i] == 0:
                continue
            vv = float(op.vv[n, x, y, z])
            vi = float(op.vi[n, x, y, z])
            xg = (1 - vv) / (1 + vv)
            G = 2 * xg / (vi * (1 + xg))
            for o in (o1, o2):
                G += float(o.v_ext[n, i]) / ((1 - float(o.v_int[n, i])) * vi)
            ratios.append(G / G0 / S)
    if k == 0:
        assert abs(S - 1) < 2e-3                  # the first row keeps the DC conductance G0
    ratios = np.array(ratios)
    assert ratios.size > 50
    near = np.minimum(np.abs(ratios - 1), np.abs(ratios - 0.5))
    assert near.max() < 2e-3, near.max()
    assert (np.abs(ratios - 1) < 2e-3).sum() > ratios.size // 2      # mostly interior edges


def test_volume_and_boundary_fall_back_to_pec():
    op = configs.conducting_sheet(steps=20)
    # the 4..6 x 4..7 x 4..6 volume of sheet material: its inner edges are PEC
    assert op.vi[0, 4, 5, 5] == 0 and op.vv[0, 4, 5, 5] == 0
    # the "edge" sheet reaches x = 0 (Mur: boundary layer of one line): PEC there, a sheet inside
    c1 = 10
    assert op.vi[2, 1, c1, 3] == 0
    pos = {tuple(int(v) for v in op.lorentz[0].pos[:, i]) for i in range(op.lorentz[0].pos.shape[1])}
    assert (3, c1, 3) in pos


@pytest.mark.parametrize("name,kw,steps", [
    ("mur", dict(), 240),
    ("upml_dispersive", dict(bc=(3,) * 6, dispersive=True), 200),
])
def test_basic_equals_multithreaded_with_sheets(name, kw, steps):
    op = configs.conducting_sheet(steps=steps, **kw)
    a = OracleEngine(op, steps)
    b = OracleEngine(op, steps, threads=3)
    for n in (steps // 3, steps - steps // 3):
        a.IterateTS(n)
        b.IterateTS(n)
    for w in (0, 1):
        assert bits_equal(a.read_field(w), b.read_field(w)), (name, w)
    for pid in a.vprobe_ids:
        assert np.array_equal(a.probe_series(pid), b.probe_series(pid), equal_nan=True)


def test_copper_sheet_shields_like_a_plate():
    out = {}
    for tag, kw in (("sheet", {}), ("plate", dict(pec=True))):
        op = configs.conducting_sheet(steps=1200, **kw)
        e = OracleEngine(op, 1200)
        e.IterateTS(1200)
        below, above = (np.nanmax(np.abs(e.probe_series(p))) for p in e.vprobe_ids)
        out[tag] = (below, above)
    for below, above in out.values():
        assert above < 1e-3 * below
    assert out["sheet"][1] < 2 * out["plate"][1]
