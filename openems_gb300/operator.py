"""Host-side Operator: the equivalent-circuit (EC) coefficient build that feeds the CUDA engine.

This restates the parts of openEMS's Cartesian ``Operator`` (FDTD/operator.cpp) and of its
operator extensions that the engine consumes, for rectilinear meshes holding axis-aligned box
primitives (the CSXCAD geometry library is not part of this package; ``Structure`` below holds
the boxes and their properties, with CSXCAD's python API names).  Everything is vectorised with
numpy so that 67 M-cell meshes build in well under a minute.

What is computed, and where it follows the reference:

* quarter-cell material averaging ``AverageMatQuarterCell`` (FDTD/operator.cpp:1447-1564) and
  ``Calc_ECPos`` (FDTD/operator.cpp:1189-1254) -> EC_C/G/L/R, stored as float32 like the
  reference's ``FDTD_FLOAT* EC_*`` arrays;
* the Rennings timestep ``CalcTimestep_Var3`` (FDTD/operator.cpp:1956-2030) including the
  ``AdrOp`` reflection at the mesh border (tools/AdrOp.cpp:183-221);
* ``Calc_ECOperatorPos`` (FDTD/operator.cpp:956-984) -> vv/vi/ii/iv (float64 math, float32 store);
* ``ApplyElectricBC`` / ``CalcPEC_Range`` / ``Calc_LumpedElements`` / ``ApplyMagneticBC``
  (FDTD/operator.cpp:1099-1187, 2045-2083, 1586-1763) in the order of ``CalcECOperator``
  (FDTD/operator.cpp:986-1097);
* operator extensions in insertion order (openems.cpp:1186-1243): excitation
  (FDTD/extensions/operator_ext_excitation.cpp:105-297), Mur ABC
  (FDTD/extensions/operator_ext_mur_abc.cpp:107-186), UPML
  (FDTD/extensions/operator_ext_upml.cpp:69-445), Lorentz/Drude
  (FDTD/extensions/operator_ext_lorentzmaterial.cpp:120-445);
* probe snapping (Common/processing.cpp:180-189, Common/processvoltage.cpp:38-42,
  Common/processcurrent.cpp:40-88).

CSXCAD's ``GetPropertyByCoordPriority`` is restated as: among the boxes of the requested
property kinds that contain the coordinate (bounds inclusive), the highest priority wins and
ties go to the box defined first.
"""
from __future__ import annotations

import math
import os
from concurrent.futures import ThreadPoolExecutor
from contextlib import contextmanager
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .excitation import Excitation, calc_nyquist_num

EPS0 = 8.85418781762e-12    # tools/constants.h:23
MUE0 = 1.256637062e-6       # tools/constants.h:24
C0 = 299792458.0            # tools/constants.h:25
Z0 = 376.730313461          # tools/constants.h:26
PI = 3.141592653589793238462643383279

# property kinds (bit flags, like CSProperties::PropertyType); a conducting sheet is a metal
# property of its own type (METAL | CONDSHEET), so the PEC pass does not take it for metal
MATERIAL, METAL, EXCITATION, LUMPED, PROBE, DUMP, CONDSHEET = 1, 2, 4, 8, 16, 32, 64


# =========================================================================================
# geometry container (CSXCAD-like)
# =========================================================================================
class Property:
    def __init__(self, structure, kind, name, **params):
        self.structure = structure
        self.kind = kind
        self.name = name
        self.params = params
        self.boxes = []

    def AddBox(self, start, stop, priority=0):
        self.structure._add_box(self, np.asarray(start, float), np.asarray(stop, float), priority)
        return self

    def AddCylinder(self, start, stop, radius, priority=0):
        """Solid cylinder (CSPrimCylinder) whose axis runs from start to stop along one mesh axis:
        the points within `radius` of the axis, ends included."""
        self.structure._add_cylinder(self, start, stop, float(radius), None, priority)
        return self

    def AddCylindricalShell(self, start, stop, radius, shell_width, priority=0):
        """Cylindrical shell (CSPrimCylindricalShell) along one mesh axis: the points whose
        distance to the axis is within shell_width/2 of `radius`."""
        self.structure._add_cylinder(self, start, stop, float(radius), float(shell_width), priority)
        return self

    # plane-wave excitation (exc_type 10) parameters, named like CSPropExcitation's setters
    def SetPropagationDir(self, val):
        self.params["prop_dir"] = np.asarray(val, float)
        return self

    def SetFrequency(self, val):
        self.params["frequency"] = float(val)
        return self


class Structure:
    """Holds properties and their box primitives (the subset of CSXCAD used by the engine path)."""

    def __init__(self):
        self.props: List[Property] = []
        self.boxes = []          # (start, stop, priority, seq, prop)
        self._seq = 0

    def _add_box(self, prop, start, stop, priority, shape=None):
        lo = np.minimum(start, stop)
        hi = np.maximum(start, stop)
        rec = (lo, hi, int(priority), self._seq, prop, start.copy(), stop.copy(), shape)
        self._seq += 1
        prop.boxes.append(rec)
        self.boxes.append(rec)

    def _add_cylinder(self, prop, start, stop, radius, width, priority):
        """A cylinder or shell along one axis; the record carries its bounding box and the shape
        (axis, centre in the two other axes, radius, shell width or None)."""
        start = np.asarray(start, float)
        stop = np.asarray(stop, float)
        d = np.nonzero(start != stop)[0]
        if d.size != 1:
            raise ValueError("cylinders must run along one mesh axis")
        a = int(d[0])
        b, c = (a + 1) % 3, (a + 2) % 3
        r_out = radius + (0.5 * width if width is not None else 0.0)
        lo = start.copy()
        hi = stop.copy()
        lo[a], hi[a] = min(start[a], stop[a]), max(start[a], stop[a])
        for k in (b, c):
            lo[k], hi[k] = start[k] - r_out, start[k] + r_out
        shape = (a, float(start[b]), float(start[c]), radius, width)
        self._add_box(prop, lo, hi, priority, shape)
        prop.boxes[-1] = prop.boxes[-1][:5] + (start.copy(), stop.copy(), shape)
        self.boxes[-1] = prop.boxes[-1]

    def _add(self, kind, name, **params):
        p = Property(self, kind, name, **params)
        self.props.append(p)
        return p

    def AddMaterial(self, name, epsilon=1.0, mue=1.0, kappa=0.0, sigma=0.0):
        return self._add(MATERIAL, name, epsilon=float(epsilon), mue=float(mue), kappa=float(kappa), sigma=float(sigma))

    def AddLorentzMaterial(self, name, epsilon=1.0, mue=1.0, kappa=0.0, sigma=0.0,
                           eps_plasma_freq=(), eps_relax_time=(), eps_lor_pole_freq=(),
                           mue_plasma_freq=(), mue_relax_time=(), mue_lor_pole_freq=()):
        """Drude/Lorentz dispersive material, one entry per dispersion order (CSPropLorentzMaterial)."""
        order = max(len(eps_plasma_freq), len(mue_plasma_freq), 1)

        def pad(v):
            v = list(v)
            return v + [0.0] * (order - len(v))
        return self._add(MATERIAL, name, epsilon=float(epsilon), mue=float(mue), kappa=float(kappa),
                         sigma=float(sigma), lorentz=True, order=order,
                         eps_plasma=pad(eps_plasma_freq), eps_relax=pad(eps_relax_time),
                         eps_pole=pad(eps_lor_pole_freq), mue_plasma=pad(mue_plasma_freq),
                         mue_relax=pad(mue_relax_time), mue_pole=pad(mue_lor_pole_freq))

    def AddVoxelMaterial(self, name, start, stop, epsilon, kappa=0.0, priority=0):
        """Per-cell relative permittivity and conductivity on a box whose faces lie on mesh lines:
        ``epsilon`` (and ``kappa``, scalar or array) hold one value per mesh cell of the box
        (shape = cells per axis).  Used for design regions."""
        eps = np.asarray(epsilon, np.float64)
        kap = np.broadcast_to(np.asarray(kappa, np.float64), eps.shape).copy()
        p = self._add(MATERIAL, name, epsilon=1.0, mue=1.0, kappa=0.0, sigma=0.0, voxel=True,
                      eps_array=eps, kappa_array=kap)
        p.AddBox(start, stop, priority)
        return p

    def AddMetal(self, name):
        return self._add(METAL, name)

    def AddConductingSheet(self, name, conductivity, thickness):
        """Thin conducting sheet (CSPropConductingSheet): conductivity in S/m, thickness in metres,
        on two-dimensional boxes; modelled by Operator_Ext_ConductingSheet."""
        return self._add(METAL | CONDSHEET, name, conductivity=float(conductivity), thickness=float(thickness))

    def AddLumpedElement(self, name, ny, R=float('nan'), C=float('nan'), caps=True, L=float('nan'), LEtype=0):
        """Lumped element (CSPropLumpedElement): LEtype 0 = parallel, 1 = series, -1 = invalid.
        A parallel element without L > 0 is the parallel RC of the main operator
        (Operator::Calc_LumpedElements); a parallel element with L > 0 and every series element
        go through the lumped RLC extension (Operator_Ext_LumpedRLC)."""
        return self._add(LUMPED, name, ny=int(ny), R=float(R), C=float(C), caps=bool(caps), L=float(L),
                         LEtype=int(LEtype))

    def AddExcitation(self, name, exc_type, exc_val, delay=0.0, weight=None):
        """Excitation property; `weight` = three functions f(x, y, z) of the drawing-unit
        coordinates that scale the components (CSPropExcitation's weight functions)."""
        return self._add(EXCITATION, name, exc_type=int(exc_type),
                         exc_val=np.asarray(exc_val, float), delay=float(delay), weight=weight)

    def AddProbe(self, name, p_type, weight=1.0, norm_dir=-1, frequency=(), start_time=0.0, stop_time=0.0,
                 interval=0):
        """Voltage (p_type 0), current (1), E-field (2) or H-field (3) probe; ``interval``
        overrides the default sampling interval Nyquist/OverSampling (openems.cpp:568)."""
        return self._add(PROBE, name, p_type=int(p_type), weight=float(weight), norm_dir=int(norm_dir),
                         frequency=list(frequency), start_time=float(start_time), stop_time=float(stop_time),
                         interval=int(interval))

    def AddDump(self, name, dump_type=0, dump_mode=1, frequency=(), start_time=0.0, stop_time=0.0):
        """Field dump box: dump_type 0/1 = E/H time domain, 10/11 = E/H frequency domain;
        dump_mode 0 = no interpolation, 1 = node interpolation, 2 = cell interpolation
        (Common/processfields.h, Common/engine_interface_base.h:33); start/stop time in seconds
        limit a time-domain dump (Processing::SetProcessStartStopTime)."""
        return self._add(DUMP, name, dump_type=int(dump_type), dump_mode=int(dump_mode), frequency=list(frequency),
                         start_time=float(start_time), stop_time=float(stop_time))


@dataclass
class Grid:
    """Rectilinear mesh: ``lines[n]`` in drawing units, ``unit`` = metres per drawing unit."""
    lines: list
    unit: float = 1.0

    def __post_init__(self):
        self.lines = [np.asarray(sorted(set(float(v) for v in l)), np.float64) for l in self.lines]


# =========================================================================================
# engine-facing tables (what the operator extensions hand to their engine extensions)
# =========================================================================================
@dataclass
class ExcitationTable:
    """Operator_Ext_Excitation arrays (FDTD/extensions/operator_ext_excitation.h:80-94)."""
    volt_index: np.ndarray
    volt_dir: np.ndarray
    volt_amp: np.ndarray
    volt_delay: np.ndarray
    curr_index: np.ndarray
    curr_dir: np.ndarray
    curr_amp: np.ndarray
    curr_delay: np.ndarray
    signal_volt: np.ndarray
    signal_curr: np.ndarray
    period: int = 0


@dataclass
class UPMLRegion:
    """Operator_Ext_UPML tables (FDTD/extensions/operator_ext_upml.h:74-96)."""
    start: np.ndarray
    num_lines: np.ndarray
    vv: np.ndarray
    vvfo: np.ndarray
    vvfn: np.ndarray
    ii: np.ndarray
    iifo: np.ndarray
    iifn: np.ndarray


@dataclass
class MurWall:
    """Operator_Ext_Mur_ABC (FDTD/extensions/operator_ext_mur_abc.h) + engine m_start_TS."""
    ny: int
    line_nr: int
    line_nr_shift: int
    start_ts: int
    coeff_nyP: np.ndarray
    coeff_nyPP: np.ndarray


@dataclass
class LorentzOrder:
    """One dispersion order of Operator_Ext_LorentzMaterial (operator_ext_dispersive.h:60-75)."""
    pos: np.ndarray               # uint32 [3, M]
    volt_ade_on: bool
    curr_ade_on: bool
    volt_lor_on: bool
    curr_lor_on: bool
    v_int: np.ndarray
    v_ext: np.ndarray
    v_lor: np.ndarray
    i_int: np.ndarray
    i_ext: np.ndarray
    i_lor: np.ndarray


@dataclass
class TFSFTable:
    """Operator_Ext_TFSF (FDTD/extensions/operator_ext_tfsf.h:55-84), flattened.

    ``volt_*`` / ``curr_*`` hold one term per (face, position, component) in the order
    Engine_Ext_TFSF::DoPostVoltageUpdates / DoPostCurrentUpdates apply them
    (engine_ext_tfsf.cpp:36-215): faces n = x, y, z, lower plane before upper, positions with
    the nP line outer and the nPP line inner, component nP before nPP.  ``index`` [3, K] is the
    cell, ``dir`` the field component, ``delay``/``delta``/``amp`` the reference's
    m_*Delay / m_*DelayDelta / m_*Amp entries.  ``max_delay`` is m_maxDelay (already +1)."""
    start: np.ndarray
    stop: np.ndarray
    active: np.ndarray            # bool [3, 2]: lower/upper plane of each direction
    prop_dir: np.ndarray
    e_amp: np.ndarray
    h_amp: np.ndarray
    phase_velocity: float
    max_delay: int
    volt_index: np.ndarray
    volt_dir: np.ndarray
    volt_delay: np.ndarray
    volt_delta: np.ndarray
    volt_amp: np.ndarray
    curr_index: np.ndarray
    curr_dir: np.ndarray
    curr_delay: np.ndarray
    curr_delta: np.ndarray
    curr_amp: np.ndarray
    signal_volt: np.ndarray
    signal_curr: np.ndarray
    period: int = 0


@dataclass
class LumpedRLCTable:
    """Operator_Ext_LumpedRLC (FDTD/extensions/operator_ext_lumpedRLC.h:58-82): one entry per
    lumped edge, in the reference's build order."""
    pos: np.ndarray               # uint32 [3, K]
    dir: np.ndarray               # int32 [K]
    ilv: np.ndarray               # parallel inductor: dT/dL
    i2v: np.ndarray               # parallel: (dT/dC)/(1 + dT*dG/(2*dC))
    vv2: np.ndarray               # series coefficients
    vj1: np.ndarray
    vj2: np.ndarray
    vvd: np.ndarray
    ib0: np.ndarray
    b1: np.ndarray
    b2: np.ndarray


@dataclass
class VoltageProbe:
    name: str
    start: np.ndarray
    stop: np.ndarray
    weight: float
    interval: int
    fd_interval: int
    freqs: list
    start_ts: int = 0
    stop_ts: int = 0xFFFFFFFF


@dataclass
class CurrentProbe:
    name: str
    start: np.ndarray
    stop: np.ndarray
    norm_dir: int
    start_inside: np.ndarray
    stop_inside: np.ndarray
    weight: float
    interval: int
    fd_interval: int
    freqs: list
    start_ts: int = 0
    stop_ts: int = 0xFFFFFFFF


@dataclass
class FieldProbe:
    """E (field 0, probe type 2) or H (field 1, probe type 3) point probe: the three Yee values at
    ``pos`` (main mesh for E, dual mesh for H) over their edge lengths, no interpolation
    (ProcessFieldProbe, Common/processfieldprobe.cpp:77-92); H samples carry the dual time."""
    name: str
    field: int
    pos: np.ndarray
    weight: float
    interval: int
    fd_interval: int
    freqs: list
    start_ts: int = 0
    stop_ts: int = 0xFFFFFFFF
    el: tuple = ()                # GetEdgeLength(n, pos) of each component (E main, H dual mesh)


@dataclass
class FieldDumpFD:
    """FD dump box (Common/processfields_fd.cpp): E (field=0) or H (field=1); interp = the dump
    mode (0 none, 1 node, 2 cell interpolation); dual = the box was snapped to the dual mesh."""
    name: str
    field: int
    start: np.ndarray
    stop: np.ndarray
    freqs: list
    fd_interval: int
    interp: int = 2
    dual: bool = True


@dataclass
class FieldDumpTD:
    """Time-domain dump box (Common/processfields_td.cpp): E (field=0) or H (field=1) every
    ``interval`` steps within [start_ts, stop_ts]; interp/dual as for FieldDumpFD.  ``name`` is the
    file name stem (the property name, with _<box number> when the property has several boxes)."""
    name: str
    field: int
    start: np.ndarray
    stop: np.ndarray
    interval: int
    interp: int
    dual: bool
    start_ts: int = 0
    stop_ts: int = 0xFFFFFFFF


@dataclass
class OperatorData:
    num_lines: np.ndarray
    dt: float
    vv: np.ndarray
    vi: np.ndarray
    ii: np.ndarray
    iv: np.ndarray
    exc: ExcitationTable
    upml: list = field(default_factory=list)
    mur: list = field(default_factory=list)
    lorentz: list = field(default_factory=list)
    vprobes: list = field(default_factory=list)
    iprobes: list = field(default_factory=list)
    dumps: list = field(default_factory=list)
    nyquist: int = 0
    excitation: Optional[Excitation] = None
    grid: Optional[Grid] = None
    tfsf: Optional[TFSFTable] = None
    rlc: Optional[LumpedRLCTable] = None
    td_dumps: list = field(default_factory=list)
    fprobes: list = field(default_factory=list)
    cylinder: Optional["CylinderTable"] = None


# lumped element types (CSPropLumpedElement::LEtype)
LE_INVALID, LE_PARALLEL, LE_SERIES = -1, 0, 1
LUMPED_RLC_Z_FACT = 20.0      # FDTD/extensions/operator_ext_lumpedRLC.h:30


def _dump_mesh(field, dump_mode):
    """Interpolation type and snapping mesh of a dump box (openems.cpp:629-665,
    Common/processfields.cpp:200-208): H dumps default to the dual mesh, cell interpolation
    selects the dual mesh and node interpolation the main mesh; no interpolation keeps the
    default."""
    interp = int(dump_mode)
    if interp not in (0, 1, 2):
        raise ValueError(f"dump mode {dump_mode} is not 0, 1 or 2")
    dual = field == 1
    if interp == 2:
        dual = True
    elif interp == 1:
        dual = False
    return interp, dual


def _is_par_rc(prop):
    """Operator::IsLEparRC (FDTD/operator.cpp:1765-1775)."""
    L = prop.params.get("L", float("nan"))
    return prop.params.get("LEtype", LE_PARALLEL) == LE_PARALLEL and not (L > 0.0)


def _is_lumped_rlc(prop):
    """Operator_Ext_LumpedRLC::IsLElumpedRLC (operator_ext_lumpedRLC.cpp:550-561)."""
    t = prop.params.get("LEtype", LE_PARALLEL)
    L = prop.params.get("L", float("nan"))
    return (t == LE_PARALLEL and L > 0.0) or t == LE_SERIES


# =========================================================================================
# mesh helpers
# =========================================================================================
def _main_delta(L):
    """GetDiscDelta(n,pos,false) for pos in [0,N-1] (FDTD/operator.cpp:159-171)."""
    d = np.empty_like(L)
    d[:-1] = L[1:] - L[:-1]
    d[-1] = L[-1] - L[-2]
    return d


def _dual_line(L):
    """GetDiscLine(n,pos,true) (FDTD/operator.cpp:144-157)."""
    dl = np.empty_like(L)
    dl[:-1] = 0.5 * (L[:-1] + L[1:])
    dl[-1] = L[-1] + 0.5 * (L[-1] - L[-2])
    return dl


def _dual_delta(L):
    """GetDiscDelta(n,pos,true) (FDTD/operator.cpp:172-179)."""
    dl = _dual_line(L)
    d = np.empty_like(L)
    d[0] = L[1] - L[0]
    d[1:] = dl[1:] - dl[:-1]
    return d


def _raw_delta(L, idx):
    """GetRawDiscDelta (FDTD/operator.cpp:1256-1266) for an index array (may hold -1 or N-1)."""
    N = len(L)
    idx = np.asarray(idx)
    out = np.empty(idx.shape, np.float64)
    lo = idx < 0
    hi = idx >= N - 1
    mid = ~(lo | hi)
    out[lo] = L[0] - L[1]
    out[hi] = L[N - 2] - L[N - 1]
    out[mid] = L[idx[mid] + 1] - L[idx[mid]]
    return out


class _Painter:
    """Vectorised GetPropertyByCoordPriority over separable sample coordinates."""

    def __init__(self, structure: Structure, kinds: int):
        recs = [b for b in structure.boxes if b[4].kind & kinds]
        # paint ascending priority; among equal priorities the earliest-defined box is painted last (wins)
        self.recs = sorted(recs, key=lambda r: (r[2], -r[3]))
        self.props = []
        self.prop_index = {}
        for r in self.recs:
            if id(r[4]) not in self.prop_index:
                self.prop_index[id(r[4])] = len(self.props)
                self.props.append(r[4])

    @staticmethod
    def _range(c, lo, hi):
        m = np.nonzero((c >= lo) & (c <= hi))[0]
        if m.size == 0:
            return None
        if m[-1] - m[0] + 1 == m.size:
            return slice(int(m[0]), int(m[-1]) + 1)
        return m

    @staticmethod
    def rec_cells(rec, cx, cy, cz):
        """Index arrays (ix, iy, iz) of the sample grid and a boolean mask over them (None = all)
        of the points inside primitive `rec`; None when its bounding box holds no point."""
        lo, hi = rec[0], rec[1]
        cs = (cx, cy, cz)
        idx = [np.nonzero((cs[k] >= lo[k]) & (cs[k] <= hi[k]))[0] for k in range(3)]
        if any(i.size == 0 for i in idx):
            return None
        shape = rec[7] if len(rec) > 7 else None
        if shape is None:
            return idx, None
        a, pb, pc, radius, width = shape
        b, c = (a + 1) % 3, (a + 2) % 3
        db = np.asarray(cs[b], np.float64)[idx[b]] - pb
        dc = np.asarray(cs[c], np.float64)[idx[c]] - pc
        dist = np.sqrt(db[:, None] ** 2 + dc[None, :] ** 2)       # [b][c]
        inside = dist <= radius if width is None else np.abs(dist - radius) <= 0.5 * width
        # broadcast [b][c] to the index order (x, y, z)
        m = inside.T if b > c else inside
        m = np.expand_dims(m, a)
        m = np.broadcast_to(m, tuple(i.size for i in idx))
        return idx, m

    def paint_bbox(self, cx, cy, cz):
        """paint() over the smallest index box that holds every sample point inside one of the
        primitives (all other points are background): (map of that box, its index offsets)."""
        cs = (np.asarray(cx), np.asarray(cy), np.asarray(cz))
        lo = [None] * 3
        hi = [None] * 3
        for rec in self.recs:
            for k in range(3):
                idx = np.nonzero((cs[k] >= rec[0][k]) & (cs[k] <= rec[1][k]))[0]
                if idx.size:
                    lo[k] = int(idx[0]) if lo[k] is None else min(lo[k], int(idx[0]))
                    hi[k] = int(idx[-1]) if hi[k] is None else max(hi[k], int(idx[-1]))
        if any(v is None for v in lo):
            return np.full((0, 0, 0), -1, np.int32), (0, 0, 0)
        m = self.paint(cs[0][lo[0]:hi[0] + 1], cs[1][lo[1]:hi[1] + 1], cs[2][lo[2]:hi[2] + 1])
        return m, (lo[0], lo[1], lo[2])

    def paint(self, cx, cy, cz):
        """Return int32 array [len(cx),len(cy),len(cz)] of property indices (-1 = background)."""
        out = np.full((len(cx), len(cy), len(cz)), -1, np.int32)
        for rec in self.recs:
            lo, hi, _prio, _seq, prop = rec[:5]
            pid = self.prop_index[id(prop)]
            if len(rec) > 7 and rec[7] is not None:
                hit = self.rec_cells(rec, cx, cy, cz)
                if hit is None:
                    continue
                (ax, ay, az), m = hit
                sub = out[np.ix_(ax, ay, az)]
                sub[m] = pid
                out[np.ix_(ax, ay, az)] = sub
                continue
            rx = self._range(cx, lo[0], hi[0])
            ry = self._range(cy, lo[1], hi[1])
            rz = self._range(cz, lo[2], hi[2])
            if rx is None or ry is None or rz is None:
                continue
            if isinstance(rx, slice) and isinstance(ry, slice) and isinstance(rz, slice):
                out[rx, ry, rz] = pid
            else:
                ax = np.arange(len(cx))[rx]
                ay = np.arange(len(cy))[ry]
                az = np.arange(len(cz))[rz]
                out[np.ix_(ax, ay, az)] = pid
        return out

    def param(self, idx_map, key, background):
        table = np.array([p.params.get(key, background) if p.kind == MATERIAL else background
                          for p in self.props] + [background], np.float64)
        return table[idx_map]   # -1 selects the trailing background entry


def _axes(n):
    return n, (n + 1) % 3, (n + 2) % 3


def _bcast(n, arr_n, arr_p, arr_pp):
    """Broadcast three 1-D arrays given in (n, nP, nPP) axis order into an x,y,z grid; the
    reshaped arrays are returned in the same (n, nP, nPP) order."""
    out = [None, None, None]
    a, b, c = _axes(n)
    shapes = {a: arr_n, b: arr_p, c: arr_pp}
    for ax in range(3):
        v = shapes[ax]
        shp = [1, 1, 1]
        shp[ax] = len(v)
        out[ax] = v.reshape(shp)
    return out[a], out[b], out[c]


def _coords_xyz(n, cn, cp, cpp):
    """Return (cx, cy, cz) 1-D coordinate arrays from (n, nP, nPP)-ordered arrays."""
    a, b, c = _axes(n)
    d = {a: cn, b: cp, c: cpp}
    return d[0], d[1], d[2]


def _slabs(n, parts):
    """Split range(n) into at most ``parts`` contiguous (x0, x1) chunks."""
    parts = max(1, min(parts, n))
    edges = np.linspace(0, n, parts + 1).round().astype(int)
    return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]


def _parallel(fn, items):
    """Run fn over items on a thread pool (numpy releases the GIL inside its kernels)."""
    workers = min(len(items), os.cpu_count() or 1)
    if workers <= 1:
        return [fn(*it) for it in items]
    with ThreadPoolExecutor(max_workers=workers) as ex:
        return list(ex.map(lambda it: fn(*it), items))


# =========================================================================================
# the operator
# =========================================================================================
_BUILD_DEVICE = ["cpu"]


@contextmanager
def build_device(device: str):
    """Default device of Operator.build inside the block ("cpu" or "cuda")."""
    _BUILD_DEVICE.append(device)
    try:
        yield
    finally:
        _BUILD_DEVICE.pop()


class Operator:
    """Builds EC-FDTD coefficients plus extension tables for the engine.

    ``bc``: 6 boundary codes as in openEMS (0 PEC, 1 PMC, 2 Mur, 3 PML), order xmin,xmax,...
    """

    def __init__(self, structure: Structure, grid: Grid, excitation: Excitation, bc=(0,) * 6,
                 pml_size=(8,) * 6, timestep=0.0, timestep_factor=1.0, over_sampling=4,
                 background=(1.0, 1.0, 0.0, 0.0), fdtd_float=np.float32):
        self.ft = np.dtype(fdtd_float).type   # FDTD_FLOAT: float32 like the reference, float64 for FP64 runs
        self.csx = structure
        self.grid = grid
        self.exc = excitation
        self.bc = [int(b) for b in bc]
        # every wall keeps its configured PML size (openEMS defaults all six to 8,
        # openems.cpp:129), PML or not: Operator_Ext_UPML grades an upper PML with the lower
        # wall's size (operator_ext_upml.cpp:315, width/m_Size[2*n]), so a PML on the upper wall
        # alone depends on the size of the wall below
        self.pml_size = [int(s) for s in pml_size]
        self.forced_dt = float(timestep)
        self.ts_factor = float(timestep_factor)
        self.over_sampling = int(over_sampling)
        self.bg = dict(epsilon=background[0], mue=background[1], kappa=background[2], sigma=background[3])
        self.L = grid.lines
        self.unit = float(grid.unit)
        self.N = np.array([len(l) for l in self.L], np.int64)
        if (self.N < 3).any():
            raise ValueError("Operator: at least 3 mesh lines per direction are required")
        self.md = [_main_delta(l) for l in self.L]        # main deltas (drawing units)
        self.dd = [_dual_delta(l) for l in self.L]        # dual deltas (drawing units)
        self.dl = [_dual_line(l) for l in self.L]
        self._mat = _Painter(structure, MATERIAL)
        self._matmetal = _Painter(structure, MATERIAL | METAL)
        self._bind_voxels()

    # ---- material lookup ------------------------------------------------------------------
    def _lookup(self, n, cn, cp, cpp, keys, painter=None):
        painter = painter or self._mat
        cx, cy, cz = _coords_xyz(n, cn, cp, cpp)
        m = painter.paint(cx, cy, cz)
        out = [painter.param(m, k, self.bg[k]) for k in keys]
        vkeys = [(keys.index(k), k + "_array" if k == "kappa" else "eps_array")
                 for k in ("epsilon", "kappa") if k in keys]
        if vkeys:
            for prop in painter.props:
                if not prop.params.get("voxel"):
                    continue
                pid = painter.prop_index[id(prop)]
                mask = m == pid
                if not mask.any():
                    continue
                cl = prop.params["cell_lines"]
                idx = [np.clip(np.searchsorted(cl[a], c, side="right") - 1, 0, len(cl[a]) - 2)
                       for a, c in enumerate((cx, cy, cz))]
                for ki, arr in vkeys:
                    vox = prop.params[arr][np.ix_(*idx)]
                    out[ki] = np.where(mask, vox, out[ki])
        return out

    def _bind_voxels(self):
        """Record the cell boundaries of every voxel material box on this mesh."""
        for prop in self.csx.props:
            if not prop.params.get("voxel"):
                continue
            lo, hi = prop.boxes[0][0], prop.boxes[0][1]
            cl = []
            for a in range(3):
                L = self.L[a]
                tol = 1e-9 * max(1.0, abs(L[-1] - L[0]))
                cl.append(L[(L >= lo[a] - tol) & (L <= hi[a] + tol)])
            shape = tuple(len(c) - 1 for c in cl)
            if shape != prop.params["eps_array"].shape:
                raise ValueError(f"voxel material {prop.name}: {prop.params['eps_array'].shape} values for "
                                 f"{shape} mesh cells")
            prop.params["cell_lines"] = cl

    # ---- effective material (FDTD/operator.cpp:1447-1564) ----------------------------------
    def eff_mat(self, n):
        """Quarter-cell averaged eps (abs), kappa, mue (abs), sigma for edge direction n, full grid."""
        a, p, pp = _axes(n)
        L, Lp, Lpp = self.L[a], self.L[p], self.L[pp]
        N, Np, Npp = len(L), len(Lp), len(Lpp)
        i_n, i_p, i_pp = np.arange(N), np.arange(Np), np.arange(Npp)
        delta = _raw_delta(L, i_n)
        deltaP = _raw_delta(Lp, i_p)
        deltaPP = _raw_delta(Lpp, i_pp)
        delta_M = _raw_delta(L, i_n - 1)
        deltaP_M = _raw_delta(Lp, i_p - 1)
        deltaPP_M = _raw_delta(Lpp, i_pp - 1)
        u = self.unit

        def wmain(k, idx):   # GetNodeWidth(k, int pos, dual=true) = main delta * unit, 0 for idx<0
            d = self.md[k]
            out = np.zeros(len(idx))
            ok = idx >= 0
            out[ok] = d[idx[ok]] * u
            return out

        cn = L + delta * 0.5
        cp_up, cp_dn = Lp + deltaP * 0.25, Lp - deltaP_M * 0.25
        cpp_up, cpp_dn = Lpp + deltaPP * 0.25, Lpp - deltaPP_M * 0.25
        Wp, WpM = wmain(p, i_p), wmain(p, i_p - 1)
        Wpp, WppM = wmain(pp, i_pp), wmain(pp, i_pp - 1)

        samples = [(cp_up, cpp_up, Wp, Wpp), (cp_dn, cpp_up, WpM, Wpp),
                   (cp_up, cpp_dn, Wp, WppM), (cp_dn, cpp_dn, WpM, WppM)]
        eps_acc = kap_acc = area = None
        for cpv, cppv, wa, wb in samples:
            e, k = self._lookup(n, cn, cpv, cppv, ("epsilon", "kappa"))
            _, A_p, A_pp = _bcast(n, np.ones(N), wa, wb)
            A = A_p * A_pp                       # shape broadcastable (1 along n)
            if eps_acc is None:
                eps_acc = e * A
                kap_acc = k * A
                area = np.broadcast_to(A, e.shape).copy()
            else:
                eps_acc += e * A
                kap_acc += k * A
                area = area + A
        eff0 = eps_acc * (EPS0 / area)
        eff1 = kap_acc / area
        del eps_acc, kap_acc

        # mu / sigma: two samples along n
        cpm = Lp + deltaP * 0.5
        cppm = Lpp + deltaPP * 0.5
        d_dn = wmain(a, i_n - 1)
        d_up = wmain(a, i_n)
        mu_dn, sg_dn = self._lookup(n, L - delta_M * 0.25, cpm, cppm, ("mue", "sigma"))
        Ddn, _, _ = _bcast(n, d_dn, np.ones(Np), np.ones(Npp))
        Dup, _, _ = _bcast(n, d_up, np.ones(Np), np.ones(Npp))
        with np.errstate(divide="ignore", invalid="ignore"):
            eff2 = Ddn / mu_dn
            eff3 = np.where(sg_dn != 0, Ddn / np.where(sg_dn != 0, sg_dn, 1.0), 0.0)
            length = np.broadcast_to(Ddn, eff2.shape)
            mu_up, sg_up = self._lookup(n, L + delta * 0.25, cpm, cppm, ("mue", "sigma"))
            eff2 = eff2 + Dup / mu_up
            eff3 = np.where(sg_up != 0, eff3 + Dup / np.where(sg_up != 0, sg_up, 1.0), 0.0)
            length = length + Dup
            eff2 = length * MUE0 / eff2
            eff3 = np.where(eff3 != 0, length / np.where(eff3 != 0, eff3, 1.0), eff3)
        for arr in (eff0, eff1, eff2, eff3):
            if not np.isfinite(arr).all():
                raise ValueError("Operator: an effective material parameter is not finite")
        return eff0, eff1, eff2, eff3

    def _sub(self, lo, hi):
        """Operator over the sub-mesh lines[a][lo[a]:hi[a]] (same geometry and background).

        Every per-edge quantity of EffMat/EC depends only on lines within +-1 of the edge, so
        with one halo line on each internal side the sub-mesh reproduces the full mesh's values
        at its interior positions."""
        g = Grid([self.L[a][lo[a]:hi[a]] for a in range(3)], unit=self.unit)
        sub = Operator.__new__(Operator)
        sub.csx, sub.grid, sub.exc, sub.bg, sub.ft = self.csx, g, self.exc, self.bg, self.ft
        sub.L, sub.unit = g.lines, self.unit
        sub.N = np.array([len(l) for l in g.lines], np.int64)
        sub.md = [_main_delta(l) for l in g.lines]
        sub.dd = [_dual_delta(l) for l in g.lines]
        sub.dl = [_dual_line(l) for l in g.lines]
        sub._mat, sub._matmetal = self._mat, self._matmetal
        return sub

    def _halo(self, axis, a0, a1):
        lo = [0, 0, 0]
        hi = [int(v) for v in self.N]
        lo[axis] = max(a0 - 1, 0)
        hi[axis] = min(a1 + 1, int(self.N[axis]))
        return lo, hi

    # ---- EC (FDTD/operator.cpp:1189-1254, 1839-1870) ---------------------------------------
    def _ec_local(self):
        """EC_C/G/L/R (float32) on this operator's own mesh."""
        shape = tuple(int(v) for v in self.N)
        out = [np.empty((3,) + shape, self.ft) for _ in range(4)]
        u = self.unit
        for n in range(3):
            a, p, pp = _axes(n)
            e0, e1, e2, e3 = self.eff_mat(n)
            Dn, Ap, App = _bcast(n, self.md[a] * u, self.dd[p] * u, self.dd[pp] * u)
            area_e = Ap * App
            with np.errstate(divide="ignore", invalid="ignore"):
                out[0][n] = np.where(Dn != 0, e0 * area_e / Dn, 0.0)
                out[1][n] = np.where(Dn != 0, e1 * area_e / Dn, 0.0)
                Dh, Bp, Bpp = _bcast(n, self.dd[a] * u, self.md[p] * u, self.md[pp] * u)
                area_h = Bp * Bpp
                out[2][n] = np.where(Dh != 0, e2 * area_h / Dh, 0.0)
                out[3][n] = np.where(Dh != 0, e3 * area_h / Dh, 0.0)
        return out

    def calc_ec(self):
        shape = tuple(int(v) for v in self.N)
        self.EC_C = np.empty((3,) + shape, self.ft)
        self.EC_G = np.empty((3,) + shape, self.ft)
        self.EC_L = np.empty((3,) + shape, self.ft)
        self.EC_R = np.empty((3,) + shape, self.ft)
        dst = (self.EC_C, self.EC_G, self.EC_L, self.EC_R)

        def work(x0, x1):
            lo, hi = self._halo(0, x0, x1)
            res = self._sub(lo, hi)._ec_local()
            for d, r in zip(dst, res):
                d[:, x0:x1] = r[:, x0 - lo[0]:x1 - lo[0]]
        _parallel(work, _slabs(int(self.N[0]), 2 * (os.cpu_count() or 1)))

    def eff_region(self, n, start, nl):
        """eff_Mat (eps abs, kappa, mue abs, sigma) of direction n on the box start..start+nl."""
        lo = [max(int(start[a]) - 1, 0) for a in range(3)]
        hi = [min(int(start[a] + nl[a]) + 1, int(self.N[a])) for a in range(3)]
        e = self._sub(lo, hi).eff_mat(n)
        sl = tuple(slice(int(start[a]) - lo[a], int(start[a]) - lo[a] + int(nl[a])) for a in range(3))
        return [x[sl] for x in e]

    # ---- the same numerics on the GPU -----------------------------------------------------------
    def _gpu_core(self):
        """EC_C/G/L/R and the Var3 timestep from the device builder; returns (builder, dt_var3)."""
        if np.dtype(self.ft) != np.float32:
            raise ValueError("Operator.build(device='cuda'): float32 operators only")
        recs = self._mat.recs
        if any(len(r) > 7 and r[7] is not None for r in recs):
            raise ValueError("Operator.build(device='cuda'): cylinder materials are built on the host")
        if any(r[4].params.get("voxel") for r in recs):
            raise ValueError("Operator.build(device='cuda'): voxel materials are built on the host")
        keys = ("epsilon", "kappa", "mue", "sigma")
        lo = np.array([np.asarray(r[0], np.float64) for r in recs], np.float64).reshape(-1, 3)
        hi = np.array([np.asarray(r[1], np.float64) for r in recs], np.float64).reshape(-1, 3)
        par = np.array([[r[4].params.get(k, self.bg[k]) if r[4].kind == MATERIAL else self.bg[k] for k in keys]
                        for r in recs], np.float64).reshape(-1, 4)
        b = GpuOperatorBuilder(self.L, self.unit, lo, hi, par, [self.bg[k] for k in keys])
        shape = (3,) + tuple(int(v) for v in self.N)
        self.EC_C, self.EC_G, self.EC_L, self.EC_R = (np.empty(shape, np.float32) for _ in range(4))
        dt = b.ec(self.EC_C, self.EC_G, self.EC_L, self.EC_R, self.forced_dt <= 0)
        return b, dt

    # ---- timestep (FDTD/operator.cpp:1956-2030) --------------------------------------------
    def calc_timestep(self):
        """Operator::CalcTimestep (FDTD/operator.cpp:1880-1889): the Rennings Var3 timestep."""
        return self.calc_timestep_var3()

    def calc_timestep_var3(self):
        def work(x0, x1):
            h0, h1 = max(x0 - 1, 0), min(x1 + 1, int(self.N[0]))
            return self._var3_local(self.EC_C[:, h0:h1], self.EC_L[:, h0:h1], x0 - h0, x1 - h0)
        dts = _parallel(work, _slabs(int(self.N[0]), 2 * (os.cpu_count() or 1)))
        dT = min(dts)
        if dT == 0 or dT >= 1e200:
            raise ValueError("Operator: timestep is zero")
        return dT

    @staticmethod
    def _var3_local(C32, L32, i0, i1):
        """Minimum Rennings timestep over x-positions [i0, i1) of the given EC slab (the slab
        carries one halo plane on each internal side)."""
        C = C32.astype(np.float64)
        Lh = L32.astype(np.float64)

        def sh(arr, shifts):
            """arr at pos+shift with AdrOp cell reflection (-1 -> 0, N -> N-1)."""
            out = arr
            for ax, s in shifts:
                if s == 0:
                    continue
                Nn = arr.shape[ax]
                idx = np.clip(np.arange(Nn) + s, 0, Nn - 1)
                out = np.take(out, idx, axis=ax)
            return out

        dT = 1e200
        with np.errstate(divide="ignore", invalid="ignore"):
            for n in range(3):
                a, p, pp = _axes(n)
                Cn = C[n]
                wqp = 1 / (Lh[pp] * sh(Cn, [(p, 1)])) + 1 / (Lh[pp] * Cn)
                wqp += 1 / (Lh[p] * sh(Cn, [(pp, 1)])) + 1 / (Lh[p] * Cn)
                Lpp_m = sh(Lh[pp], [(p, -1)])
                wqp += 1 / (Lpp_m * Cn) + 1 / (Lpp_m * sh(Cn, [(p, -1)]))
                # AdrOp shifts are cumulative: after Shift(nP,-1), Shift(nPP,-1) -> pos - eP - ePP
                Lp_mm = sh(Lh[p], [(p, -1), (pp, -1)])
                wqp += 1 / (Lp_mm * sh(Cn, [(p, -1)])) + 1 / (Lp_mm * sh(Cn, [(p, -1), (pp, -1)]))

                Lpp_pm = sh(Lh[pp], [(p, -1)])
                Lp_ppm = sh(Lh[p], [(pp, -1)])
                w4 = [1 / (Lh[pp] * C[p]), 1 / (Lpp_pm * C[p]), 1 / (Lh[p] * C[pp]), 1 / (Lp_ppm * C[pp])]
                wt1 = w4[0] + w4[1] + w4[2] + w4[3] - 2 * np.minimum(np.minimum(w4[0], w4[1]), np.minimum(w4[2], w4[3]))
                Cp_n = sh(C[p], [(a, 1)])
                Cpp_n = sh(C[pp], [(a, 1)])
                w4 = [1 / (Lh[pp] * Cp_n), 1 / (Lpp_pm * Cp_n), 1 / (Lh[p] * Cpp_n), 1 / (Lp_ppm * Cpp_n)]
                wt2 = w4[0] + w4[1] + w4[2] + w4[3] - 2 * np.minimum(np.minimum(w4[0], w4[1]), np.minimum(w4[2], w4[3]))
                newT = (2 / np.sqrt(wqp + wt1 + wt2))[i0:i1]
                cand = newT[np.isfinite(newT) & (newT > 0)]
                if cand.size:
                    dT = min(dT, float(cand.min()))
        return dT

    # ---- coefficients (FDTD/operator.cpp:956-984) ------------------------------------------
    def _ec_op(self, C, G, L, R, dT):
        with np.errstate(divide="ignore", invalid="ignore"):
            C = C.astype(np.float64)
            G = G.astype(np.float64)
            L = L.astype(np.float64)
            R = R.astype(np.float64)
            okc = C > 0
            okl = L > 0
            Cs = np.where(okc, C, 1.0)
            Ls = np.where(okl, L, 1.0)
            vv = np.where(okc, (1.0 - dT * G / 2.0 / Cs) / (1.0 + dT * G / 2.0 / Cs), 0.0)
            vi = np.where(okc, (dT / Cs) / (1.0 + dT * G / 2.0 / Cs), 0.0)
            ii = np.where(okl, (1.0 - dT * R / 2.0 / Ls) / (1.0 + dT * R / 2.0 / Ls), 0.0)
            iv = np.where(okl, (dT / Ls) / (1.0 + dT * R / 2.0 / Ls), 0.0)
        return vv.astype(self.ft), vi.astype(self.ft), ii.astype(self.ft), iv.astype(self.ft)

    # ---- snapping (FDTD/operator.cpp:252-372) ----------------------------------------------
    def _num_lines(self, ny, full):
        """GetNumberOfLines(ny, fullMesh): every line on a Cartesian mesh."""
        return int(self.N[ny])

    def snap_line(self, ny, coord, dual=False, full=False):
        """SnapToMeshLine (FDTD/operator.cpp:252-280) over GetNumberOfLines(ny, full) lines."""
        L = self.L[ny]
        nl = self._num_lines(ny, full)
        if coord < L[0]:
            return 0, False
        if coord > L[nl - 1]:
            return nl - 1, False
        if not dual:
            dl = self.dl[ny]
            for n in range(nl):
                if coord <= dl[n]:
                    return n, True
        else:
            for n in range(1, nl):
                if coord <= L[n]:
                    return n - 1, True
        return 0, True

    def snap_box(self, start, stop, dual=False, method=0, full=False):
        """SnapBox2Mesh; returns (dim, uiStart, uiStop, startIn, stopIn) or dim=-2 if outside."""
        lstart = np.minimum(start, stop)
        lstop = np.maximum(start, stop)
        nl = [self._num_lines(n, full) for n in range(3)]
        for n in range(3):
            mn, mx = self.L[n][0], self.L[n][nl[n] - 1]
            if (lstart[n] < mn and lstop[n] < mn) or (lstart[n] > mx and lstop[n] > mx):
                return -2, None, None, None, None
        s, si, e, ei = [0] * 3, [False] * 3, [0] * 3, [False] * 3
        for n in range(3):
            s[n], si[n] = self.snap_line(n, lstart[n], dual, full)
            e[n], ei[n] = self.snap_line(n, lstop[n], dual, full)
        dim = 0

        def line(n, i):
            return self.dl[n][i] if dual else self.L[n][i]
        for n in range(3):
            if method == 1 and e[n] > s[n]:
                if line(n, s[n]) > lstart[n] and s[n] > 0:
                    s[n] -= 1
                if line(n, e[n]) < lstop[n] and e[n] < nl[n] - 1:
                    e[n] += 1
            elif method == 2 and e[n] > s[n]:
                if line(n, s[n]) < lstart[n] and s[n] < nl[n] - 1:
                    s[n] += 1
                if line(n, e[n]) > lstop[n] and e[n] > 0:
                    e[n] -= 1
            if e[n] > s[n]:
                dim += 1
        return dim, np.array(s), np.array(e), np.array(si), np.array(ei)

    # ---- the build --------------------------------------------------------------------------
    def build(self, num_ts: int, device: Optional[str] = None) -> OperatorData:
        """CalcECOperator (FDTD/operator.cpp:986-1097) + extension builds + processing setup.

        device="cuda" computes the equivalent circuit, the Var3 timestep and the coefficients on
        the GPU (oems_cuda_opbuild_*, bit-identical to the host path) for float32 operators
        without voxel materials; everything else is built on the host either way."""
        gpu = None
        device = device or _BUILD_DEVICE[-1]
        if device == "cuda":
            gpu = self._gpu_core()
        elif device != "cpu":
            raise ValueError(f"Operator.build: unknown device {device!r}")
        else:
            self.calc_ec()
        if self.forced_dt > 0:
            dT = self.forced_dt
        elif gpu is not None:
            dT = gpu[1]
            if dT == 0 or dT >= 1e200:
                gpu[0].close()
                raise ValueError("Operator: timestep is zero")
        else:
            dT = self.calc_timestep()
        dT *= self.ts_factor
        if self.exc.period > 0:
            TS = math.ceil(self.exc.period / dT)
            dT = self.exc.period / TS
        self.dT = dT
        self.exc.ft = self.ft
        self.exc.Reset(dT)
        self.exc.buildExcitationSignal(num_ts)

        shape = (3,) + tuple(int(v) for v in self.N)
        self.vv, self.vi, self.ii, self.iv = (np.empty(shape, self.ft) for _ in range(4))

        def coef(x0, x1):
            for n in range(3):
                r = self._ec_op(self.EC_C[n, x0:x1], self.EC_G[n, x0:x1], self.EC_L[n, x0:x1],
                                self.EC_R[n, x0:x1], dT)
                for d, v in zip((self.vv, self.vi, self.ii, self.iv), r):
                    d[n, x0:x1] = v
        if gpu is not None:
            try:
                gpu[0].coefficients(dT, self.vv, self.vi, self.ii, self.iv)
            finally:
                gpu[0].close()
        else:
            _parallel(coef, _slabs(int(self.N[0]), 2 * (os.cpu_count() or 1)))

        self._apply_electric_bc([b != -1 for b in self.bc])
        self._calc_pec()
        self._calc_lumped()
        self._apply_magnetic_bc([b == 1 for b in self.bc])
        # the cylinder extension is added with the grid (Operator_Cylinder::SetupCSXGrid), before
        # every other extension, so it is built first
        cyl = self._build_cylinder()

        exc = self._build_excitation()
        # Operator_Ext_TFSF is added right after the excitation extension (openems.cpp:1186-1188)
        # and built in that order, so it reads vi/iv before any later extension rewrites them
        tfsf = self._build_tfsf()
        mur = self._build_mur(exc)
        upml = self._build_upml()
        lorentz = self._build_lorentz()
        # Operator_Ext_ConductingSheet follows Operator_Ext_LorentzMaterial (openems.cpp:1236-1239)
        # and hands its tables to the same engine extension
        lorentz = lorentz + self._build_conducting_sheet()
        # Operator_Ext_LumpedRLC is added after the dispersive extensions (openems.cpp:1236-1241)
        rlc = self._build_lumped_rlc()
        vprobes, iprobes, dumps = self._build_processing()
        data = OperatorData(num_lines=self.N.astype(np.uint32), dt=dT, vv=self.vv, vi=self.vi, ii=self.ii,
                            iv=self.iv, exc=exc, upml=upml, mur=mur, lorentz=lorentz, vprobes=vprobes,
                            iprobes=iprobes, dumps=dumps, nyquist=self.exc.GetNyquistNum(),
                            excitation=self.exc, grid=self.grid, tfsf=tfsf, rlc=rlc, td_dumps=self.td_dumps,
                            fprobes=self.fprobes, cylinder=cyl)
        return data

    def _build_cylinder(self):
        """Cartesian meshes have no cylinder extension."""
        return None

    def _node_width_at(self, ny, pos, dual=False):
        """GetNodeWidth(ny, pos, dual) = GetEdgeLength(ny, pos, !dual) for one position."""
        return self._edge_length(ny, pos, not dual)

    def _area_over_length(self, ny, pos):
        """GetEdgeArea(ny, pos) / GetEdgeLength(ny, pos) of one edge; the area is the product of
        the two node widths (GetNodeArea, FDTD/operator.cpp:235-240)."""
        u = self.unit
        nyP, nyPP = (ny + 1) % 3, (ny + 2) % 3
        area = (self.dd[nyP][pos[nyP]] * u) * (self.dd[nyPP][pos[nyPP]] * u)
        return area / (self.md[ny][pos[ny]] * u)

    def _edge_geometry(self, n, pos_axes):
        """GetEdgeLength(n, pos), GetEdgeArea(n, pos) and their dual versions over the box of
        positions pos_axes (broadcastable arrays, metres)."""
        a, p, pp = _axes(n)
        u = self.unit
        De, Ap, App = _bcast(n, self.md[a][pos_axes[a]] * u, self.dd[p][pos_axes[p]] * u, self.dd[pp][pos_axes[pp]] * u)
        Dh, Bp, Bpp = _bcast(n, self.dd[a][pos_axes[a]] * u, self.md[p][pos_axes[p]] * u, self.md[pp][pos_axes[pp]] * u)
        return De, Ap * App, Dh, Bp * Bpp

    def _weight_coords(self, cs, x, y, z):
        """The Yee coordinates (drawing units) an excitation weight function is evaluated at."""
        return float(cs[0][x]), float(cs[1][y]), float(cs[2][z])

    def _yee_painter(self, kinds):
        """Property lookup at Yee coordinates (GetYeeCoords + GetPropertyByCoordPriority)."""
        return _Painter(self.csx, kinds)

    def _mur_painter(self):
        """Material lookup at the Mur wall's mesh coordinates (operator_ext_mur_abc.cpp:125-160)."""
        return self._mat

    # ---- boundary conditions ---------------------------------------------------------------
    def _apply_electric_bc(self, dirs):
        """ApplyElectricBC (FDTD/operator.cpp:1099-1138)."""
        for n in range(3):
            a, p, pp = _axes(n)
            sl0 = [slice(None)] * 3
            sl0[n] = 0
            sl1 = [slice(None)] * 3
            sl1[n] = int(self.N[n]) - 1
            if dirs[2 * n]:
                for c in (p, pp):
                    self.vv[c][tuple(sl0)] = 0
                    self.vi[c][tuple(sl0)] = 0
            if dirs[2 * n + 1]:
                for c in (n, p, pp):
                    self.vv[c][tuple(sl1)] = 0
                    self.vi[c][tuple(sl1)] = 0

    def _apply_magnetic_bc(self, dirs):
        """ApplyMagneticBC (FDTD/operator.cpp:1140-1187)."""
        for n in range(3):
            a, p, pp = _axes(n)
            def sl(i):
                s = [slice(None)] * 3
                s[n] = i
                return tuple(s)
            if dirs[2 * n]:
                for c in (n, p, pp):
                    self.ii[c][sl(0)] = 0
                    self.iv[c][sl(0)] = 0
            if dirs[2 * n + 1]:
                for c in (p, pp):
                    self.ii[c][sl(int(self.N[n]) - 2)] = 0
                    self.iv[c][sl(int(self.N[n]) - 2)] = 0
            for c in (n, p, pp):
                self.ii[c][sl(int(self.N[n]) - 1)] = 0
                self.iv[c][sl(int(self.N[n]) - 1)] = 0

    def _calc_pec(self):
        """CalcPEC_Range (FDTD/operator.cpp:2045-2083): edges whose Yee point is in a METAL box."""
        if not any(p.kind == METAL for p in self.csx.props):
            return
        painter = self._matmetal
        metal_ids = np.array([p.kind == METAL for p in painter.props] + [False])
        for n in range(3):
            cs = [self.L[0], self.L[1], self.L[2]]
            cs[n] = self.dl[n]
            m = painter.paint(cs[0], cs[1], cs[2])
            is_metal = metal_ids[m]
            self.vv[n][is_metal] = 0
            self.vi[n][is_metal] = 0

    def _calc_lumped(self):
        """Calc_LumpedElements (FDTD/operator.cpp:1586-1763), parallel RC boxes only."""
        u = self.unit
        for prop in self.csx.props:
            if prop.kind != LUMPED:
                continue
            if not _is_par_rc(prop):      # Operator::IsLEparRC (FDTD/operator.cpp:1765-1775)
                continue
            C = prop.params["C"]
            R = prop.params["R"]
            if not (C > 0):
                C = float("nan")
            if R < 0:
                R = float("nan")
            if math.isnan(R) and math.isnan(C):
                continue
            ny = prop.params["ny"]
            nyP, nyPP = (ny + 1) % 3, (ny + 2) % 3
            for lo, hi, _pr, _sq, _p, *_ in prop.boxes:
                # the base SnapBox2Mesh on the full mesh (Operator::SnapBox2Mesh, qualified)
                dim, s, e, _, _ = Operator.snap_box(self, lo, hi, dual=False, method=0, full=True)
                if dim <= 0 or s[ny] == e[ny]:
                    continue
                def gc(pos):
                    return self._area_over_length(ny, pos)
                unitGC = 0.0
                pos = [0, 0, 0]
                for pos[ny] in range(s[ny], e[ny]):
                    plane = 0.0
                    for pos[nyP] in range(s[nyP], e[nyP] + 1):
                        for pos[nyPP] in range(s[nyPP], e[nyPP] + 1):
                            plane += gc(pos)
                    unitGC += 1 / plane
                unitGC = 1 / unitGC
                kappa = 1 / R / unitGC if R > 0 else 0.0
                epsilon = 0.0
                if C > 0:
                    epsilon = C / unitGC
                    if epsilon < EPS0:
                        C = 0
                for pos[ny] in range(s[ny], e[ny]):
                    for pos[nyP] in range(s[nyP], e[nyP] + 1):
                        for pos[nyPP] in range(s[nyPP], e[nyPP] + 1):
                            x, y, z = pos
                            if C > 0:
                                self.EC_C[ny, x, y, z] = epsilon * gc(pos)
                            if R > 0:
                                self.EC_G[ny, x, y, z] = kappa * gc(pos)
                            if R == 0:
                                self.vv[ny, x, y, z] = 0
                                self.vi[ny, x, y, z] = 0
                            else:
                                a_, b_, c_, d_ = self._ec_op(self.EC_C[ny, x, y, z], self.EC_G[ny, x, y, z],
                                                             self.EC_L[ny, x, y, z], self.EC_R[ny, x, y, z], self.dT)
                                self.vv[ny, x, y, z], self.vi[ny, x, y, z] = a_, b_
                                self.ii[ny, x, y, z], self.iv[ny, x, y, z] = c_, d_
                if prop.params["caps"]:
                    for pos[nyP] in range(s[nyP], e[nyP] + 1):
                        for pos[nyPP] in range(s[nyPP], e[nyPP] + 1):
                            for pos[ny] in (s[ny], e[ny]):
                                x, y, z = pos
                                if pos[nyP] < e[nyP]:
                                    self.vv[nyP, x, y, z] = 0
                                    self.vi[nyP, x, y, z] = 0
                                if pos[nyPP] < e[nyPP]:
                                    self.vv[nyPP, x, y, z] = 0
                                    self.vi[nyPP, x, y, z] = 0

    # ---- excitation extension ----------------------------------------------------------------
    def _build_excitation(self) -> ExcitationTable:
        """Operator_Ext_Excitation::BuildExtension (operator_ext_excitation.cpp:105-297), boxes only.

        List order follows the reference's loops: z outer, then y, then x, then the component.
        """
        u = self.unit
        painter = self._yee_painter(EXCITATION)
        vrec, crec = [], []
        if painter.props:
            for n in range(3):
                # electric: Yee point of the main mesh, skip pos[n] >= N-1 (painted only over the
                # index box that holds the excitation primitives: the rest is background)
                cs = [self.L[0], self.L[1], self.L[2]]
                cs[n] = self.dl[n]
                m, (ox, oy, oz) = painter.paint_bbox(*cs)
                valid = np.ones(m.shape, bool)
                sl = [slice(None)] * 3
                sl[n] = slice(max(0, int(self.N[n]) - 1 - (ox, oy, oz)[n]), None)
                valid[tuple(sl)] = False
                for sx, sy, sz in zip(*np.nonzero((m >= 0) & valid)):
                    x, y, z = int(sx) + ox, int(sy) + oy, int(sz) + oz
                    prop = painter.props[m[sx, sy, sz]]
                    et = prop.params["exc_type"]
                    if et not in (0, 1):
                        continue
                    ex = prop.params["exc_val"][n]
                    wf = prop.params.get("weight")
                    if wf is not None:       # GetWeightedExcitation at the Yee point (drawing units)
                        ex = ex * float(wf[n](*self._weight_coords(cs, x, y, z)))
                    amp = ex * self._edge_length(n, (x, y, z))
                    if amp != 0:
                        vrec.append((z, y, x, n, amp, int(prop.params["delay"] / self.dT)))
                    if et == 1:
                        self.vv[n, x, y, z] = 0
                        self.vi[n, x, y, z] = 0
                # magnetic: dual Yee point, skip the last H line in every direction
                cs = [self.dl[0], self.dl[1], self.dl[2]]
                cs[n] = self.L[n]
                m, (ox, oy, oz) = painter.paint_bbox(*cs)
                valid = np.zeros(m.shape, bool)
                valid[:max(0, int(self.N[0]) - 1 - ox), :max(0, int(self.N[1]) - 1 - oy),
                      :max(0, int(self.N[2]) - 1 - oz)] = True
                for sx, sy, sz in zip(*np.nonzero((m >= 0) & valid)):
                    x, y, z = int(sx) + ox, int(sy) + oy, int(sz) + oz
                    prop = painter.props[m[sx, sy, sz]]
                    et = prop.params["exc_type"]
                    if et not in (2, 3):
                        continue
                    amp = prop.params["exc_val"][n] * self._edge_length(n, (x, y, z), dual=True)
                    if amp != 0:
                        crec.append((z, y, x, n, amp, int(prop.params["delay"] / self.dT)))
                    if et == 3:
                        self.ii[n, x, y, z] = 0
                        self.iv[n, x, y, z] = 0
        vrec.sort(key=lambda r: (r[0], r[1], r[2], r[3]))
        crec.sort(key=lambda r: (r[0], r[1], r[2], r[3]))

        def pack(rec):
            K = len(rec)
            idx = np.zeros((3, K), np.uint32)
            for i, r in enumerate(rec):
                idx[:, i] = (r[2], r[1], r[0])
            return (idx, np.array([r[3] for r in rec], np.uint16), np.array([r[4] for r in rec], self.ft),
                    np.array([r[5] for r in rec], np.uint32))
        vi_, vd, va, vdl = pack(vrec)
        ci_, cd, ca, cdl = pack(crec)
        return ExcitationTable(vi_, vd, va, vdl, ci_, cd, ca, cdl, self.exc.volt.copy(), self.exc.curr.copy(),
                               self.exc.period_steps())

    # ---- TFSF plane wave (operator_ext_tfsf.cpp:84-406) ----------------------------------------
    def _disc_line(self, n, pos, dual=False):
        """GetDiscLine (FDTD/operator.cpp:144-157); 0.0 outside the mesh, as there."""
        if pos < 0 or pos >= self.N[n]:
            return 0.0
        return float(self.dl[n][pos] if dual else self.L[n][pos])

    def _edge_length(self, n, pos, dual=False):
        """GetEdgeLength (FDTD/operator.cpp:212-215) = GetDiscDelta * gridDelta."""
        p = pos[n]
        if p < 0 or p >= self.N[n]:
            return 0.0
        return float((self.dd[n][p] if dual else self.md[n][p]) * self.unit)

    def _yee_coords(self, ny, pos, dual):
        """GetYeeCoords (FDTD/operator.cpp:182-201), coordinates only."""
        c = [self._disc_line(k, pos[k], dual) for k in range(3)]
        c[ny] = self._disc_line(ny, pos[ny], not dual)
        return c

    def numeric_phase_velocity(self, start, stop, prop_dir, freq):
        """Operator::CalcNumericPhaseVelocity (FDTD/operator.cpp:2150-2215).  ``freq`` is rounded
        to float first, as the reference's signature takes a float."""
        freq = float(np.float32(freq))
        dT = self.dT
        c0 = C0 / math.sqrt(self.bg["epsilon"] * self.bg["mue"])
        avg = [abs(self._disc_line(n, int(start[n])) - self._disc_line(n, int(stop[n]))) * self.unit
               / abs(float(int(stop[n]) - int(start[n]))) for n in range(3)]
        for n in range(3):
            nP, nPP = (n + 1) % 3, (n + 2) % 3
            if abs(prop_dir[n]) == 1 and prop_dir[nP] == 0 and prop_dir[nPP] == 0:
                # the reference uses the x-axis mean delta for every Cartesian direction
                kx = math.asin(avg[0] / c0 / dT * math.sin(2 * PI * freq * dT / 2)) * 2 / avg[0]
                return 2 * PI * freq / kx
        k0 = 2 * PI * freq / c0
        k = k0
        rhs = math.pow(math.sin(2 * PI * freq * dT / 2) / c0 / dT, 2)
        old_phv, phv, it = 0.0, c0, 0
        while abs(old_phv - phv) > 1e-6:
            it += 1
            old_phv = phv
            fk = 0.0
            fdk = 0.0
            for n in range(3):
                fk += math.pow(math.sin(prop_dir[n] * k * avg[n] / 2) / avg[n], 2)
                fdk += prop_dir[n] * math.sin(prop_dir[n] * k * avg[n] / 2) * math.cos(prop_dir[n] * k * avg[n] / 2) / avg[n]
            fk -= rhs
            k -= fk / fdk
            if k < k0:
                k = k0
            phv = 2 * PI * freq / k
            if it > 99:
                break
        return phv

    def _build_tfsf(self):
        """Operator_Ext_TFSF::BuildExtension (operator_ext_tfsf.cpp:84-406): the first plane-wave
        excitation (exc_type 10) with exactly one box.  Returns None when there is none, like
        the reference's SetActive(false); raises where the reference rejects the setup."""
        ft = self.ft
        for prop in self.csx.props:
            if prop.kind != EXCITATION or prop.params.get("exc_type") != 10:
                continue
            if len(prop.boxes) != 1:
                continue   # "more (or less) than one primitive, skipping"
            rec = prop.boxes[0]
            d = np.asarray(prop.params.get("prop_dir", (0.0, 0.0, 0.0)), float)
            d = [float(v) for v in d]
            norm = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
            if norm == 0:
                raise ValueError("TFSF: plane wave direction is zero")
            d = [d[0] / norm, d[1] / norm, d[2] / norm]
            dim, St, Sp, _, _ = self.snap_box(rec[5], rec[6])
            if dim != 3:
                raise ValueError("TFSF: plane wave box dimension is invalid")
            St = [int(v) for v in St]
            Sp = [int(v) for v in Sp]
            ref_index = math.sqrt(self.bg["epsilon"] * self.bg["mue"])
            freq = float(prop.params.get("frequency", 0.0))
            if freq <= 0:
                phv = C0 / ref_index
            else:
                phv = self.numeric_phase_velocity(St, Sp, d, freq)
            if phv < 0 or phv > C0 / ref_index or math.isnan(phv):
                phv = C0 / ref_index
            E = [float(v) for v in prop.params["exc_val"]]
            nl = [Sp[n] - St[n] + 1 for n in range(3)]
            active = np.zeros((3, 2), bool)
            origin = [0.0] * 3
            for n in range(3):
                active[n, 0] = St[n] != 0
                active[n, 1] = Sp[n] != int(self.N[n]) - 1
                ui = St[n] - 1 if d[n] >= 0 else Sp[n] + 1   # -1 wraps to an unsigned index: 0.0
                origin[n] = self._disc_line(n, ui)
            dotEk = E[0] * d[0] + E[1] * d[1] + E[2] * d[2]
            angle = math.acos(dotEk / (E[0] * E[0] + E[1] * E[1] + E[2] * E[2])) / PI * 180
            if angle == 0:
                raise ValueError("TFSF: plane wave direction and polarization are identical")
            if angle != 90:
                E = [E[n] - d[n] * dotEk for n in range(3)]
            H = [0.0] * 3
            for n in range(3):
                nP, nPP = (n + 1) % 3, (n + 2) % 3
                H[n] = d[nP] * E[nPP] - d[nPP] * E[nP]
                H[n] /= Z0 * math.sqrt(self.bg["mue"] / self.bg["epsilon"])
            unit, dT = self.unit, self.dT

            def dist_delay(ny, pos, dual, extra):
                c = self._yee_coords(ny, pos, dual)
                dist = abs((c[0] - origin[0]) * d[0]) + abs((c[1] - origin[1]) * d[1]) + abs((c[2] - origin[2]) * d[2])
                return dist * unit / phv / dT + extra

            max_delay = 0
            # per (n, l, c): lists of (delay, delta, amp) in ui_pos order
            vt = {}
            ct = {}
            for n in range(3):
                nP, nPP = (n + 1) % 3, (n + 2) % 3
                if not active[n, 0] and not active[n, 1]:
                    continue
                numP = nl[nP] * nl[nPP]
                for l in range(2):
                    for c in range(2):
                        if active[n, l]:
                            vt[n, l, c] = [np.zeros(numP, np.uint32), np.zeros(numP, ft), np.zeros(numP, ft)]
                            ct[n, l, c] = [np.zeros(numP, np.uint32), np.zeros(numP, ft), np.zeros(numP, ft)]
                pos = [0, 0, 0]
                pos[nP] = St[nP]
                ui = 0
                for i in range(nl[nP]):
                    pos[nPP] = St[nPP]
                    for j in range(nl[nPP]):
                        def put(tab, key, delay, amp):
                            nonlocal max_delay
                            max_delay = max(int(delay), max_delay)
                            fl = math.floor(delay)
                            tab[key][0][ui] = int(fl)
                            tab[key][1][ui] = ft(delay - fl)
                            tab[key][2][ui] = ft(amp)
                        # current updates
                        pos[n] = St[n]
                        if active[n, 0]:
                            put(ct, (n, 0, 1), dist_delay(nP, pos, False, 0.0), E[nP] * self._edge_length(nP, pos))
                            put(ct, (n, 0, 0), dist_delay(nPP, pos, False, 0.0), E[nPP] * self._edge_length(nPP, pos))
                            pos[n] -= 1
                            ct[n, 0, 0][2][ui] = ft(ct[n, 0, 0][2][ui] * self.iv[nP, pos[0], pos[1], pos[2]])
                            ct[n, 0, 1][2][ui] = ft(ct[n, 0, 1][2][ui] * self.iv[nPP, pos[0], pos[1], pos[2]])
                        if active[n, 1]:
                            pos[n] = Sp[n]
                            put(ct, (n, 1, 1), dist_delay(nP, pos, False, 0.0), E[nP] * self._edge_length(nP, pos))
                            put(ct, (n, 1, 0), dist_delay(nPP, pos, False, 0.0), E[nPP] * self._edge_length(nPP, pos))
                            ct[n, 1, 0][2][ui] = ft(ct[n, 1, 0][2][ui] * self.iv[nP, pos[0], pos[1], pos[2]])
                            ct[n, 1, 1][2][ui] = ft(ct[n, 1, 1][2][ui] * self.iv[nPP, pos[0], pos[1], pos[2]])
                        if active[n, 0]:
                            ct[n, 0, 0][2][ui] = -ct[n, 0, 0][2][ui]
                        if active[n, 1]:
                            ct[n, 1, 1][2][ui] = -ct[n, 1, 1][2][ui]
                        if pos[nP] == Sp[nP]:
                            if active[n, 0]:
                                ct[n, 0, 1][2][ui] = 0
                            if active[n, 1]:
                                ct[n, 1, 1][2][ui] = 0
                        if pos[nPP] == Sp[nPP]:
                            if active[n, 0]:
                                ct[n, 0, 0][2][ui] = 0
                            if active[n, 1]:
                                ct[n, 1, 0][2][ui] = 0
                        # voltage updates
                        pos[n] = St[n] - 1
                        if active[n, 0]:
                            put(vt, (n, 0, 1), dist_delay(nP, pos, True, 1.0), H[nP] * self._edge_length(nP, pos, True))
                            put(vt, (n, 0, 0), dist_delay(nPP, pos, True, 1.0), H[nPP] * self._edge_length(nPP, pos, True))
                            pos[n] += 1
                            vt[n, 0, 0][2][ui] = ft(vt[n, 0, 0][2][ui] * self.vi[nP, pos[0], pos[1], pos[2]])
                            vt[n, 0, 1][2][ui] = ft(vt[n, 0, 1][2][ui] * self.vi[nPP, pos[0], pos[1], pos[2]])
                        pos[n] = Sp[n]
                        if active[n, 1]:
                            put(vt, (n, 1, 1), dist_delay(nP, pos, True, 1.0), H[nP] * self._edge_length(nP, pos, True))
                            put(vt, (n, 1, 0), dist_delay(nPP, pos, True, 1.0), H[nPP] * self._edge_length(nPP, pos, True))
                            vt[n, 1, 0][2][ui] = ft(vt[n, 1, 0][2][ui] * self.vi[nP, pos[0], pos[1], pos[2]])
                            vt[n, 1, 1][2][ui] = ft(vt[n, 1, 1][2][ui] * self.vi[nPP, pos[0], pos[1], pos[2]])
                        if active[n, 1]:
                            vt[n, 1, 0][2][ui] = -vt[n, 1, 0][2][ui]
                        if active[n, 0]:
                            vt[n, 0, 1][2][ui] = -vt[n, 0, 1][2][ui]
                        if pos[nP] == Sp[nP]:
                            if active[n, 0]:
                                vt[n, 0, 0][2][ui] = 0
                            if active[n, 1]:
                                vt[n, 1, 0][2][ui] = 0
                        if pos[nPP] == Sp[nPP]:
                            if active[n, 0]:
                                vt[n, 0, 1][2][ui] = 0
                            if active[n, 1]:
                                vt[n, 1, 1][2][ui] = 0
                        pos[nPP] += 1
                        ui += 1
                    pos[nP] += 1
            max_delay += 1
            volt = self._tfsf_terms(vt, St, Sp, nl, active, False)
            curr = self._tfsf_terms(ct, St, Sp, nl, active, True)
            return TFSFTable(np.array(St, np.uint32), np.array(Sp, np.uint32), active, np.array(d), np.array(E),
                             np.array(H), phv, max_delay, *volt, *curr, self.exc.volt.copy(), self.exc.curr.copy(),
                             self.exc.period_steps())
        return None

    @staticmethod
    def _tfsf_terms(tab, St, Sp, nl, active, curr):
        """Flatten the per-face tables into the application order of Engine_Ext_TFSF."""
        idx, dirs, dl, dd, am = [], [], [], [], []
        for n in range(3):
            nP, nPP = (n + 1) % 3, (n + 2) % 3
            for l in range(2):
                if not active[n, l]:
                    continue
                line = (St[n] - 1 if curr else St[n]) if l == 0 else Sp[n]
                ui = 0
                for i in range(nl[nP]):
                    for j in range(nl[nPP]):
                        pos = [0, 0, 0]
                        pos[n], pos[nP], pos[nPP] = line, St[nP] + i, St[nPP] + j
                        for c, comp in ((0, nP), (1, nPP)):
                            t = tab[n, l, c]
                            idx.append(pos)
                            dirs.append(comp)
                            dl.append(t[0][ui])
                            dd.append(t[1][ui])
                            am.append(t[2][ui])
                        ui += 1
        ft = type(dd[0]) if dd else np.float32
        return (np.array(idx, np.uint32).T.reshape(3, -1).copy(), np.array(dirs, np.uint16),
                np.array(dl, np.uint32), np.array(dd, ft), np.array(am, ft))

    # ---- Mur ABC (operator_ext_mur_abc.cpp:80-186, engine_ext_mur_abc.cpp:30-57) -------------
    def _build_mur(self, exc: ExcitationTable):
        walls = []
        u = self.unit
        for w in range(6):
            if self.bc[w] != 2:
                continue
            ny, top = w // 2, w % 2
            nyP, nyPP = (ny + 1) % 3, (ny + 2) % 3
            if not top:
                line, shift = 0, 1
            else:
                line, shift = int(self.N[ny]) - 1, int(self.N[ny]) - 2
            delta = abs(self.md[ny][line] * u)
            c_ny = self.L[ny][line] + (delta / 2 / u if line == 0 else -delta / 2 / u)
            cs = [None, None, None]
            cs[ny] = np.array([c_ny])
            cs[nyP] = self.L[nyP]
            cs[nyPP] = self.L[nyPP]
            m = self._mur_painter().paint(*cs)
            m2 = np.moveaxis(m, ny, 0)[0]            # axes now (nyP? ...) -> reorder below
            # moveaxis leaves the remaining axes in increasing order; we need [nyP][nyPP]
            if nyP > nyPP:
                m2 = m2.T
            eps = self._mat.param(m2, "epsilon", self.bg["epsilon"])
            mue = self._mat.param(m2, "mue", self.bg["mue"])
            c0t = C0 * self.dT / np.sqrt(eps * mue)
            coeff = ((c0t - delta) / (c0t + delta)).astype(self.ft)
            bg = C0 / math.sqrt(self.bg["epsilon"] * self.bg["mue"]) * self.dT
            coeff_bg = self.ft((bg - delta) / (bg + delta))
            coeff = np.where(m2 >= 0, coeff, coeff_bg).astype(self.ft)
            # excitation inside the wall delays the ABC (engine_ext_mur_abc.cpp:44-60)
            max_delay = -1
            for i in range(exc.volt_dir.size):
                if exc.volt_dir[i] in (nyP, nyPP) and exc.volt_index[ny, i] == line:
                    max_delay = max(max_delay, int(exc.volt_delay[i]))
            start_ts = 0
            if max_delay >= 0:
                start_ts = max_delay + int(self.exc.GetLength()) + 10
            walls.append(MurWall(ny, line, shift, start_ts, coeff.copy(), coeff.copy()))
        return walls

    # ---- UPML (operator_ext_upml.cpp:69-445) -------------------------------------------------
    @staticmethod
    def _grading(D, dl, W, Z, N):
        """Default grading " -log(1e-6)*log(2.5)/(2*dl*Z*(pow(2.5,W/dl)-1)) * pow(2.5, D/dl) "."""
        return -math.log(1e-6) * math.log(2.5) / (2 * dl * Z * (np.power(2.5, W / dl) - 1)) * np.power(2.5, D / dl)

    def _upml_regions(self):
        BC = list(self.bc)
        size = list(self.pml_size)
        for n in range(3):
            if size[2 * n] * (BC[2 * n] == 3) + size[2 * n + 1] * (BC[2 * n + 1] == 3) >= self.N[n]:
                BC[2 * n] = BC[2 * n + 1] = 0
                size[2 * n] = size[2 * n + 1] = 0
        self._pml_bc, self._pml_sz = BC, size
        regs = []
        N = [int(v) for v in self.N]
        start, stop = [0, 0, 0], [N[0] - 1, N[1] - 1, N[2] - 1]
        if BC[0] == 3:
            regs.append(([0, start[1], start[2]], [size[0], stop[1], stop[2]]))
        if BC[1] == 3:
            regs.append(([N[0] - 1 - size[1], start[1], start[2]], [N[0] - 1, stop[1], stop[2]]))
        start[0] = (size[0] + 1) * (BC[0] == 3)
        stop[0] = N[0] - 1 - (size[0] + 1) * (BC[1] == 3)
        if BC[2] == 3:
            regs.append(([start[0], 0, start[2]], [stop[0], size[2], stop[2]]))
        if BC[3] == 3:
            regs.append(([start[0], N[1] - 1 - size[3], start[2]], [stop[0], N[1] - 1, stop[2]]))
        start[1] = (size[2] + 1) * (BC[2] == 3)
        stop[1] = N[1] - 1 - (size[3] + 1) * (BC[3] == 3)
        if BC[4] == 3:
            regs.append(([start[0], start[1], 0], [stop[0], stop[1], size[4]]))
        if BC[5] == 3:
            regs.append(([start[0], start[1], N[2] - 1 - size[5]], [stop[0], stop[1], N[2] - 1]))
        return regs

    def _grading_kappa(self, ny, pos_axes):
        """CalcGradingKappa (operator_ext_upml.cpp:269-343) vectorised per axis: returns
        kappa_v[3], kappa_i[3] as 1-D arrays over that axis' region indices."""
        kv, ki = [], []
        u = self.unit
        BC, sz = self._pml_bc, self._pml_sz
        for n in range(3):
            pos = pos_axes[n]
            L = self.L[n]
            N = int(self.N[n])
            el = self.md[n][pos] * u
            kvn = np.zeros(len(pos))
            kin = np.zeros(len(pos))
            low = (pos <= sz[2 * n]) & (BC[2 * n] == 3)
            up = (~low) & (pos >= N - 1 - sz[2 * n + 1]) & (BC[2 * n + 1] == 3)
            if low.any():
                width = (L[sz[2 * n]] - L[0]) * u
                depth = width - (L[pos] - L[0]) * u
                if n == ny:
                    depth = depth - el / 2
                dl = width / sz[2 * n]
                with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
                    g = self._grading(depth, dl, width, Z0, float(sz[2 * n]))
                kvn = np.where(low & (depth > 0), g, kvn)
                if n == ny:
                    depth = depth + el / 2
                if n != ny:
                    depth = depth - el / 2
                depth = np.where(depth < 0, 0.0, depth)
                with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
                    g = self._grading(depth, dl, width, Z0, float(sz[2 * n]))
                kin = np.where(low & (depth > 0), g, kin)
            if up.any():
                width = (L[N - 1] - L[N - sz[2 * n + 1] - 1]) * u
                depth = width - (L[N - 1] - L[pos]) * u
                if n == ny:
                    depth = depth + el / 2
                dl = width / sz[2 * n] if sz[2 * n] else float("inf")    # the lower wall's size, as the reference
                with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
                    g = self._grading(depth, dl, width, Z0, float(sz[2 * n]))
                kvn = np.where(up & (depth > 0), g, kvn)
                if n == ny:
                    depth = depth - el / 2
                if n != ny:
                    depth = depth + el / 2
                depth = np.where(depth > width, 0.0, depth)
                with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
                    g = self._grading(depth, dl, width, Z0, float(sz[2 * n]))
                kin = np.where(up & (depth > 0), g, kin)
            kv.append(np.nan_to_num(kvn))
            ki.append(np.nan_to_num(kin))
        return kv, ki

    def _build_upml(self):
        regs = self._upml_regions()
        out = []
        dT = self.dT
        u = self.unit
        for start, stop in regs:
            start = np.array(start)
            nl = np.array(stop) - start + 1
            sl = tuple(slice(int(start[k]), int(start[k] + nl[k])) for k in range(3))
            pos_axes = [np.arange(start[k], start[k] + nl[k]) for k in range(3)]
            shape = tuple(int(v) for v in nl)
            arrs = {k: np.zeros((3,) + shape, self.ft) for k in ("vv", "vvfo", "vvfn", "ii", "iifo", "iifn")}
            for n in range(3):
                a, p, pp = _axes(n)
                kv1, ki1 = self._grading_kappa(n, pos_axes)
                # 1-D gradings along their axis, or arrays that already broadcast over the region
                KV = [kv1[k] if kv1[k].ndim == 3 else kv1[k].reshape([-1 if j == k else 1 for j in range(3)])
                      for k in range(3)]
                KI = [ki1[k] if ki1[k].ndim == 3 else ki1[k].reshape([-1 if j == k else 1 for j in range(3)])
                      for k in range(3)]
                ksum_v = np.broadcast_to(KV[0] + KV[1] + KV[2], shape)
                ksum_i = np.broadcast_to(KI[0] + KI[1] + KI[2], shape)
                eff_eps, eff_kap, eff_mue, _ = self.eff_region(n, start, nl)
                op_vv = self.vv[n][sl]
                op_vi = self.vi[n][sl]
                op_ii = self.ii[n][sl]
                op_iv = self.iv[n][sl]
                # GetEdgeLength(n,pos)/GetEdgeArea(n,pos) and their dual versions
                De, Ae, Dh, Ah = self._edge_geometry(n, pos_axes)
                kvp = np.broadcast_to(KV[p], shape)
                kvpp = np.broadcast_to(KV[pp], shape)
                kvn = np.broadcast_to(KV[a], shape)
                kip = np.broadcast_to(KI[p], shape)
                kipp = np.broadcast_to(KI[pp], shape)
                kin = np.broadcast_to(KI[a], shape)
                # ---- voltages
                act_v = (ksum_v != 0) & (eff_kap < 1e3)
                not_pec = (op_vv + op_vi) != 0
                mod = act_v & not_pec
                new_vv = ((2 * EPS0 - kvp * dT) / (2 * EPS0 + kvp * dT)).astype(self.ft)
                new_vi = ((2 * EPS0 * dT) / (2 * EPS0 + kvp * dT) * De / Ae).astype(self.ft)
                e_vv = ((2 * EPS0 - kvpp * dT) / (2 * EPS0 + kvpp * dT)).astype(self.ft)
                e_vvfn = ((2 * EPS0 + kvn * dT) / (2 * EPS0 + kvpp * dT) / eff_eps).astype(self.ft)
                e_vvfo = ((2 * EPS0 - kvn * dT) / (2 * EPS0 + kvpp * dT) / eff_eps).astype(self.ft)
                arrs["vv"][n] = np.where(mod, e_vv, np.where(act_v, 0, op_vv))
                arrs["vvfn"][n] = np.where(mod, e_vvfn, np.where(act_v, 0, 1))
                arrs["vvfo"][n] = np.where(mod, e_vvfo, 0)
                self.vv[n][sl] = np.where(mod, new_vv, np.where(act_v, op_vv, 0))
                self.vi[n][sl] = np.where(mod, new_vi, op_vi)
                # ---- currents
                act_i = ksum_i != 0
                not_pmc = (op_ii + op_iv) != 0
                mod = act_i & not_pmc
                new_ii = ((2 * EPS0 - kip * dT) / (2 * EPS0 + kip * dT)).astype(self.ft)
                new_iv = ((2 * EPS0 * dT) / (2 * EPS0 + kip * dT) * Dh / Ah).astype(self.ft)
                e_ii = ((2 * EPS0 - kipp * dT) / (2 * EPS0 + kipp * dT)).astype(self.ft)
                e_iifn = ((2 * EPS0 + kin * dT) / (2 * EPS0 + kipp * dT) / eff_mue).astype(self.ft)
                e_iifo = ((2 * EPS0 - kin * dT) / (2 * EPS0 + kipp * dT) / eff_mue).astype(self.ft)
                arrs["ii"][n] = np.where(mod, e_ii, np.where(act_i, 0, op_ii))
                arrs["iifn"][n] = np.where(mod, e_iifn, np.where(act_i, 0, 1))
                arrs["iifo"][n] = np.where(mod, e_iifo, 0)
                self.ii[n][sl] = np.where(mod, new_ii, np.where(act_i, op_ii, 0))
                self.iv[n][sl] = np.where(mod, new_iv, op_iv)
            out.append(UPMLRegion(start.astype(np.uint32), nl.astype(np.uint32), **arrs))
        return out

    # ---- Lorentz / Drude (operator_ext_lorentzmaterial.cpp:120-445) ---------------------------
    def _build_lumped_rlc(self):
        """Operator_Ext_LumpedRLC::BuildExtension (operator_ext_lumpedRLC.cpp:111-528): series RLC
        elements and parallel elements with an inductor, boxes only.  Rewrites EC_C/EC_G and the
        coefficients of the element edges (Calc_ECOperatorPos) and builds the ADE table; None
        when there is no such element."""
        dT = self.dT
        fmax = self.exc.f0 + self.exc.fc        # GetCenterFreq() + GetCutOffFreq()
        ft = self.ft
        cols = {k: [] for k in ("ilv", "i2v", "vv2", "vj1", "vj2", "vvd", "ib0", "b1", "b2")}
        P, D = [], []
        for prop in self.csx.props:
            if prop.kind != LUMPED:
                continue
            prm = prop.params
            d = prm["ny"]
            t = prm.get("LEtype", LE_PARALLEL)
            if t == LE_INVALID:
                t = LE_PARALLEL
            C, R, L = prm["C"], prm["R"], prm.get("L", float("nan"))
            if C < 0.0:
                C = 0.0
            if R < 0.0:
                R = 0.0
            if L < 0.0:
                L = 0.0
            if math.isnan(C):
                C = 0.0
            if math.isnan(L):
                L = 0.0
            if math.isnan(R):
                R = 0.0
            if not _is_lumped_rlc(prop):
                continue
            if d < 0 or d > 2:
                continue
            d1, d2 = (d + 1) % 3, (d + 2) % 3
            for lo, hi, *_ in prop.boxes:
                dim, s0, e0, _, _ = self.snap_box(lo, hi, dual=False, method=0, full=True)
                if dim <= 0:
                    continue
                s0 = [int(v) for v in s0]
                e0 = [int(v) for v in e0]
                if s0[d] == e0[d]:
                    continue
                n0 = e0[d] - s0[d]
                n1 = e0[d1] - s0[d1] + 1
                n2 = e0[d2] - s0[d2] + 1
                npar = n1 * n2
                dL = L * npar / n0
                dR = R * npar / n0
                dG = (1 / R) * n0 / npar if R != 0 else math.inf
                dC = C * n0 / npar
                # series RLC coefficients (only the series elements use them); a series element
                # with C = 0 is a short for the capacitor
                ib0 = b1 = b2 = 0.0
                if t == LE_SERIES and C == 0:
                    ib0 = dT / (2.0 * dL + dT * dR)
                    b1 = -4.0 * dL / dT
                    b2 = (2.0 * dL - dT * dR) / dT
                elif t == LE_SERIES:
                    ib0 = 2.0 * dT * dC / (4.0 * dL * dC + 2.0 * dT * dR * dC + dT * dT)
                    b1 = (dT * dT - 4.0 * dL * dC) / (dT * dC)
                    b2 = (4.0 * dL * dC - 2.0 * dT * dR * dC + dT * dT) / (2.0 * dT * dC)
                if t == LE_PARALLEL and R == 0.0:
                    dG = 0.0
                pos = [0, 0, 0]
                for pos[d] in range(s0[d], e0[d]):
                    for pos[d1] in range(s0[d1], e0[d1] + 1):
                        for pos[d2] in range(s0[d2], e0[d2] + 1):
                            x, y, z = pos
                            if t == LE_PARALLEL:
                                if dC > 0:
                                    self.EC_C[d, x, y, z] = dC
                                else:
                                    dC = float(self.EC_C[d, x, y, z])   # the natural capacitor, kept for the next edges
                                with np.errstate(divide="ignore", invalid="ignore"):
                                    c64 = np.float64(dC)
                                    cols["i2v"].append(float((dT / c64) / (1.0 + dT * dG / (2.0 * c64))))
                                if R >= 0:
                                    self.EC_G[d, x, y, z] = dG
                                cols["ilv"].append(dT / dL if L > 0 else 0.0)
                                if dC == 0:
                                    Cd = float(self.EC_C[d, x, y, z])
                                    zmin = max(dR, 2 * PI * fmax * dL)
                                    zcd = 1.0 / (2.0 * PI * fmax * Cd) if Cd != 0 else math.inf
                                    if zcd < LUMPED_RLC_Z_FACT * zmin:
                                        self.EC_C[d, x, y, z] = 1.0 / (2 * PI * fmax * zmin * LUMPED_RLC_Z_FACT)
                                for k, v in (("vv2", 0.0), ("vj1", 0.0), ("vj2", 0.0), ("vvd", 1.0), ("ib0", 0.0),
                                             ("b1", 0.0), ("b2", 0.0)):
                                    cols[k].append(v)
                            else:
                                self.EC_G[d, x, y, z] = 0.0
                                Cd = float(self.EC_C[d, x, y, z])       # FDTD_FLOAT Cd
                                if dC:
                                    zmin = math.sqrt(math.pow(dR, 2) + math.pow(2 * PI * fmax * dL - 1.0 / (dC * 2 * PI * fmax), 2))
                                else:
                                    zmin = math.sqrt(math.pow(dR, 2) + math.pow(2 * PI * fmax * dL, 2))
                                zcd = 1.0 / (2.0 * PI * fmax * Cd) if Cd != 0 else math.inf
                                if zcd < LUMPED_RLC_Z_FACT * zmin:
                                    Cd = float(ft(1.0 / (2 * PI * fmax * zmin * LUMPED_RLC_Z_FACT)))
                                    self.EC_C[d, x, y, z] = Cd
                                cols["ilv"].append(0.0)
                                cols["i2v"].append(0.0)
                                cols["vv2"].append(0.5 * dT * ib0 / Cd)
                                cols["vj1"].append(0.5 * dT * (b1 * ib0 - 1.0) / Cd)
                                cols["vj2"].append(0.5 * dT * b2 * ib0 / Cd)
                                cols["vvd"].append(1.0 / (1.0 + 0.5 * dT * ib0 / Cd))
                                cols["ib0"].append(ib0)
                                cols["b1"].append(b1)
                                cols["b2"].append(b2)
                            a_, b_, c_, d_ = self._ec_op(self.EC_C[d, x, y, z], self.EC_G[d, x, y, z],
                                                         self.EC_L[d, x, y, z], self.EC_R[d, x, y, z], dT)
                            self.vv[d, x, y, z], self.vi[d, x, y, z] = a_, b_
                            self.ii[d, x, y, z], self.iv[d, x, y, z] = c_, d_
                            D.append(d)
                            P.append(tuple(pos))
                if prm["caps"]:
                    for pos[d1] in range(s0[d1], e0[d1] + 1):
                        for pos[d2] in range(s0[d2], e0[d2] + 1):
                            for pos[d] in (s0[d], e0[d]):
                                x, y, z = pos
                                if pos[d1] < e0[d1]:
                                    self.vv[d1, x, y, z] = 0
                                    self.vi[d1, x, y, z] = 0
                                if pos[d2] < e0[d2]:
                                    self.vv[d2, x, y, z] = 0
                                    self.vi[d2, x, y, z] = 0
        if not D:
            return None
        with np.errstate(over="ignore", invalid="ignore"):
            arr = {k: np.array(v, np.float64).astype(ft) for k, v in cols.items()}
        return LumpedRLCTable(np.array(P, np.uint32).T.copy(), np.array(D, np.int32), **arr)

    def _build_conducting_sheet(self):
        """Operator_Ext_ConductingSheet::BuildExtension (operator_ext_conductingsheet.cpp:42-263):
        two voltage ADE orders on the edges of two-dimensional conducting-sheet boxes, with the
        sheet's EC_G/EC_C rewritten from the fitted model (condsheet_table).  Edges of sheets that
        are not two-dimensional, lie in a boundary layer or have no conductance fall back to PEC."""
        from . import condsheet_table as T
        if not any(p.kind & CONDSHEET for p in self.csx.props):
            return []
        ft = self.ft
        N = [int(v) for v in self.N]
        dT = self.dT
        u = self.unit
        # GetBCSize: 0 for PEC/PMC, 1 for Mur, the PML size for UPML (openems.cpp:388-403)
        bcs = [0 if b in (0, 1) else (1 if b == 2 else int(self.pml_size[w])) for w, b in enumerate(self.bc)]
        recs = self._matmetal.recs
        tan = np.full((3,) + tuple(N), -1, np.int64)
        cond = np.zeros((3,) + tuple(N), ft)
        thick = np.zeros((3,) + tuple(N), ft)
        on = np.zeros(tuple(N), bool)
        ax = [np.arange(k) for k in N]
        disable = np.zeros(tuple(N), bool)
        for m in range(3):
            bad = (ax[m] <= bcs[2 * m]) | (ax[m] >= N[m] - bcs[2 * m + 1] - 1)
            sh = [1, 1, 1]
            sh[m] = N[m]
            disable |= bad.reshape(sh)
        for n in range(3):
            nP, nPP = (n + 1) % 3, (n + 2) % 3
            cs = [self.L[0], self.L[1], self.L[2]]
            cs[n] = self.dl[n]
            # the winning record at every Yee point (GetPropertyByCoordPriority with its primitive)
            win = np.full(tuple(N), -1, np.int64)
            for ri, rec in enumerate(recs):
                hit = _Painter.rec_cells(rec, cs[0], cs[1], cs[2])
                if hit is None:
                    continue
                (rx, ry, rz), msk = hit
                if msk is None:
                    win[np.ix_(rx, ry, rz)] = ri
                else:
                    sub = win[np.ix_(rx, ry, rz)]
                    sub[msk] = ri
                    win[np.ix_(rx, ry, rz)] = sub
            valid = np.ones(tuple(N), bool)
            sl = [slice(None)] * 3
            sl[n] = slice(N[n] - 1, None)
            valid[tuple(sl)] = False          # GetYeeCoords is false for pos[n] >= N-1
            for x, y, z in zip(*np.nonzero((win >= 0) & valid)):
                lo, hi, _pr, _sq, prop = recs[win[x, y, z]][:5]
                if not (prop.kind & CONDSHEET):
                    continue
                dim = int(sum(lo[k] != hi[k] for k in range(3)))
                if dim != 2 or disable[x, y, z] or not (ft(prop.params["conductivity"]) > 0) or \
                        not (ft(prop.params["thickness"]) > 0):
                    self.vv[n, x, y, z] = 0      # fallback to PEC
                    self.vi[n, x, y, z] = 0
                    continue
                cond[n, x, y, z] = prop.params["conductivity"]
                thick[n, x, y, z] = prop.params["thickness"]
                if lo[nP] != hi[nP]:
                    tan[n, x, y, z] = nP
                if lo[nPP] != hi[nPP]:
                    tan[n, x, y, z] = nPP
                on[x, y, z] = True
        pos = np.array(np.nonzero(on), np.int64)       # x-major scan order
        M = pos.shape[1]
        if M == 0:
            return []
        vint = [np.zeros((3, M), ft), np.zeros((3, M), ft)]
        vext = [np.zeros((3, M), ft), np.zeros((3, M), ft)]
        w_stop = ft(self.exc.f_max * 2 * PI)
        for i in range(M):
            p = [int(pos[0, i]), int(pos[1, i]), int(pos[2, i])]
            for n in range(3):
                t_dir = int(tan[n, p[0], p[1], p[2]])
                G0 = ft(cond[n, p[0], p[1], p[2]] * thick[n, p[0], p[1], p[2]])
                tk = thick[n, p[0], p[1], p[2]]
                with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
                    w0 = ft(np.float64(8.0) / np.float64(G0) / np.float64(tk) / MUE0)
                    omega_max = ft(w_stop / w0)
                k = 0
                while k < len(T.OMEGA_STOP) and not (T.OMEGA_STOP[k] > float(omega_max)):
                    k += 1
                if k >= len(T.OMEGA_STOP):
                    k = len(T.OMEGA_STOP) - 1
                if t_dir < 0:
                    continue
                # GetEdgeLength(n, pos) / GetNodeWidth(t_dir, pos)
                wtl = ft(self._edge_length(n, p) / self._node_width_at(t_dir, p))
                factor = ft(1)
                if tan[t_dir, p[0], p[1], p[2]] < 0:
                    factor = ft(2)
                q = list(p)
                q[t_dir] -= 1
                if tan[t_dir, q[0], q[1], q[2]] < 0:
                    factor = ft(2)
                L1 = ft(T.L1[k] / float(G0) / float(w0) * float(factor))
                L2 = ft(T.L2[k] / float(G0) / float(w0) * float(factor))
                R1 = ft(T.R1[k] / float(G0) * float(factor))
                R2 = ft(T.R2[k] / float(G0) * float(factor))
                G = ft(float(G0) * T.G[k] / float(factor))
                L1 = ft(L1 * wtl)
                L2 = ft(L2 * wtl)
                R1 = ft(R1 * wtl)
                R2 = ft(R2 * wtl)
                G = ft(G / wtl)
                Lmin = L2 if L2 < L1 else L1
                x, y, z = p
                self.EC_G[n, x, y, z] = G
                self.EC_C[n, x, y, z] = ft(dT * dT / 4.0 * (16.0 / float(Lmin) + float(ft(1) / L1) + float(ft(1) / L2)))
                a_, b_, c_, d_ = self._ec_op(self.EC_C[n, x, y, z], self.EC_G[n, x, y, z],
                                             self.EC_L[n, x, y, z], self.EC_R[n, x, y, z], dT)
                self.vv[n, x, y, z], self.vi[n, x, y, z] = a_, b_
                self.ii[n, x, y, z], self.iv[n, x, y, z] = c_, d_
                vi_ = float(self.vi[n, x, y, z])
                for o, (Lk, Rk) in enumerate(((L1, R1), (L2, R2))):
                    Lf, Rf = float(Lk), float(Rk)
                    vint[o][n, i] = ft((2.0 * Lf - dT * Rf) / (2.0 * Lf + dT * Rf))
                    vext[o][n, i] = ft(dT / (Lf + dT * Rf / 2.0) * vi_)
        pos32 = pos.astype(np.uint32)
        z = np.zeros((3, M), ft)
        return [LorentzOrder(pos32.copy(), True, False, False, False, vint[o], vext[o], z.copy(), z.copy(), z.copy(),
                             z.copy()) for o in range(2)]

    def _build_lorentz(self):
        """Operator_Ext_LorentzMaterial::BuildExtension, evaluated in parallel x-slabs; positions
        come out in the reference's x-major scan order."""
        lor_props = [p for p in self.csx.props if p.kind == MATERIAL and p.params.get("lorentz")]
        if not lor_props:
            return []
        order_max = max(p.params["order"] for p in lor_props)
        painter = self._matmetal
        dT = self.dT
        Nx = int(self.N[0])
        Ny, Nz = int(self.N[1]), int(self.N[2])
        # per dispersive primitive, the index box that holds its sample points (primary or dual
        # lines): outside these boxes no edge can be dispersive, so only they are painted (the
        # painted material at a point depends only on the point, so boxes that overlap give the
        # same values there, merged below)
        boxes = []
        for rec in painter.recs:
            if not (rec[4].kind == MATERIAL and rec[4].params.get("lorentz")):
                continue
            b = []
            for k in range(3):
                hit = np.zeros(int(self.N[k]), bool)
                for c in (np.asarray(self.L[k]), np.asarray(self.dl[k])):
                    hit |= (c >= rec[0][k]) & (c <= rec[1][k])
                idx = np.nonzero(hit)[0]
                if not idx.size:
                    b = None
                    break
                b.append((int(idx[0]), int(idx[-1]) + 1))
            if b:
                boxes.append(b)
        if not boxes:
            return []
        orders = []
        for o in range(order_max):
            def ptab(key):
                vals = []
                for p in painter.props:
                    if p.kind == MATERIAL and p.params.get("lorentz") and o < p.params["order"]:
                        vals.append(p.params[key][o])
                    else:
                        vals.append(0.0)
                return np.array(vals + [0.0], np.float64)
            tab = {k: ptab(k) for k in ("eps_plasma", "eps_relax", "eps_pole", "mue_plasma", "mue_relax", "mue_pole")}

            def slab(x0, x1, y0, y1, z0, z1):
                per_n = []
                on_mask = np.zeros((x1 - x0, y1 - y0, z1 - z0), bool)
                flags = [False, False, False, False]
                for n in range(3):
                    # voltage part: main Yee point, skip pos[n] >= N-1 and edges with VI == 0
                    cs = [self.L[0][x0:x1], self.L[1][y0:y1], self.L[2][z0:z1]]
                    if n == 0:
                        cs[0] = self.dl[0][x0:x1]
                    else:
                        cs[n] = self.dl[n][(y0, z0)[n - 1]:(y1, z1)[n - 1]]
                    m = painter.paint(*cs)
                    valid = self.vi[n, x0:x1, y0:y1, z0:z1] != 0
                    if n == 0:
                        if x1 == Nx:
                            valid[-1] = False
                    else:
                        sl = [slice(None)] * 3
                        sl[n] = slice(max(0, int(self.N[n]) - 1 - (y0, z0)[n - 1]), None)
                        valid[tuple(sl)] = False
                    wp = tab["eps_plasma"][m] * 2 * PI
                    trel = tab["eps_relax"][m]
                    wl = tab["eps_pole"][m] * 2 * PI
                    C = self.EC_C[n, x0:x1, y0:y1, z0:z1].astype(np.float64)
                    with np.errstate(divide="ignore", invalid="ignore"):
                        LD = np.where(valid & (wp > 0) & (C > 0), 1 / (wp * wp * C), 0.0)
                        RD = np.where((LD > 0) & (trel > 0), LD / np.where(trel > 0, trel, 1), 0.0)
                        CL = np.where((LD > 0) & (wl > 0), 1 / (wl * wl * np.where(LD > 0, LD, 1)), 0.0)
                    flags[0] |= bool((LD > 0).any())
                    flags[2] |= bool((CL > 0).any())
                    # current part: dual Yee point, skip the last H lines and IV == 0
                    cs = [self.dl[0][x0:x1], self.dl[1][y0:y1], self.dl[2][z0:z1]]
                    if n == 0:
                        cs[0] = self.L[0][x0:x1]
                    else:
                        cs[n] = self.L[n][(y0, z0)[n - 1]:(y1, z1)[n - 1]]
                    m2 = painter.paint(*cs)
                    valid2 = self.iv[n, x0:x1, y0:y1, z0:z1] != 0
                    if x1 == Nx:
                        valid2[-1] = False
                    if y1 == Ny:
                        valid2[:, -1, :] = False
                    if z1 == Nz:
                        valid2[:, :, -1] = False
                    wpm = tab["mue_plasma"][m2] * 2 * PI
                    trelm = tab["mue_relax"][m2]
                    wlm = tab["mue_pole"][m2] * 2 * PI
                    Lh = self.EC_L[n, x0:x1, y0:y1, z0:z1].astype(np.float64)
                    with np.errstate(divide="ignore", invalid="ignore"):
                        CD = np.where(valid2 & (wpm > 0) & (Lh > 0), 1 / (wpm * wpm * Lh), 0.0)
                        GD = np.where((CD > 0) & (trelm > 0), CD / np.where(trelm > 0, trelm, 1), 0.0)
                        LL = np.where((CD > 0) & (wlm > 0), 1 / (wlm * wlm * np.where(CD > 0, CD, 1)), 0.0)
                    flags[1] |= bool((CD > 0).any())
                    flags[3] |= bool((LL > 0).any())
                    on_mask |= (LD > 0) | (CD > 0)
                    per_n.append((LD, RD, CL, CD, GD, LL))
                pos = np.array(np.nonzero(on_mask), dtype=np.int64)
                sel = tuple(pos)
                M = pos.shape[1]
                tabs = {k: np.zeros((3, M), self.ft) for k in ("v_int", "v_ext", "v_lor", "i_int", "i_ext", "i_lor")}
                with np.errstate(divide="ignore", invalid="ignore"):
                    for n in range(3):
                        LD, RD, CL, CD, GD, LL = (t[sel] for t in per_n[n])
                        VI = self.vi[n, x0:x1, y0:y1, z0:z1][sel].astype(np.float64)
                        IV = self.iv[n, x0:x1, y0:y1, z0:z1][sel].astype(np.float64)
                        drude = LD > 0
                        tabs["v_int"][n] = np.where(drude, (2.0 * LD - dT * RD) / (2.0 * LD + dT * RD), 1.0)
                        tabs["v_ext"][n] = np.where(drude, dT / (LD + dT * RD / 2.0) * VI, 0.0)
                        tabs["i_int"][n] = np.where(CD > 0, (2.0 * CD - dT * GD) / (2.0 * CD + dT * GD), 1.0)
                        tabs["i_ext"][n] = np.where(CD > 0, dT / (CD + dT * GD / 2.0) * IV, 0.0)
                        tabs["v_lor"][n] = np.where(CL > 0, dT / CL / VI, 0.0)
                        tabs["i_lor"][n] = np.where(LL > 0, dT / LL / IV, 0.0)
                pos[0] += x0
                pos[1] += y0
                pos[2] += z0
                return pos.astype(np.uint32), tabs, flags

            vol = sum((b[0][1] - b[0][0]) * (b[1][1] - b[1][0]) * (b[2][1] - b[2][0]) for b in boxes)
            per_task = max(1, vol // (2 * (os.cpu_count() or 1)))
            tasks = []
            for (bx0, bx1), (y0, y1), (z0, z1) in boxes:
                nparts = max(1, ((bx1 - bx0) * (y1 - y0) * (z1 - z0)) // per_task)
                tasks += [(bx0 + a, bx0 + b, y0, y1, z0, z1) for a, b in _slabs(bx1 - bx0, nparts)]
            parts = _parallel(slab, tasks)
            pos = np.concatenate([p[0] for p in parts], axis=1)
            tabs = {k: np.concatenate([p[1][k] for p in parts], axis=1) for k in parts[0][1]}
            fl = [any(p[2][i] for p in parts) for i in range(4)]
            # the reference's x-major scan order, each position once
            lin = (pos[0].astype(np.int64) * Ny + pos[1]) * Nz + pos[2]
            _, first = np.unique(lin, return_index=True)
            pos = np.ascontiguousarray(pos[:, first])
            tabs = {k: np.ascontiguousarray(v[:, first]) for k, v in tabs.items()}
            orders.append(LorentzOrder(pos, fl[0], fl[1], fl[2], fl[3], **tabs))
        return orders

    # ---- processing (probes, FD dumps) ---------------------------------------------------------
    def _build_processing(self):
        vprobes, iprobes, dumps = [], [], []
        td_dumps = self.td_dumps = []
        fprobes = self.fprobes = []
        nyq = self.exc.GetNyquistNum()
        for prop in self.csx.props:
            if prop.kind == PROBE:
                pt = prop.params["p_type"]
                interval = max(1, nyq // self.over_sampling)
                if prop.params.get("interval"):
                    interval = int(prop.params["interval"])
                fd_interval = 0
                freqs = []
                for f in prop.params["frequency"]:
                    nts = calc_nyquist_num(f, self.dT)
                    if nts == 0:
                        continue
                    if fd_interval == 0:
                        fd_interval = nyq
                    if fd_interval > nts:
                        fd_interval = nts
                    freqs.append(float(f))
                start_ts, stop_ts = 0, 0xFFFFFFFF
                if prop.params["start_time"] > 0:
                    start_ts = int(math.floor(prop.params["start_time"] / self.dT))
                if prop.params["stop_time"] > 0:
                    stop_ts = int(math.ceil(prop.params["stop_time"] / self.dT))
                for lo, hi, _pr, _sq, _p, b_start, b_stop, *_ in prop.boxes:
                    if pt == 0:
                        s = np.array([self.snap_line(n, b_start[n], False)[0] for n in range(3)])
                        e = np.array([self.snap_line(n, b_stop[n], False)[0] for n in range(3)])
                        # keep the user's start/stop order (the sign of the integral follows it)
                        vprobes.append(VoltageProbe(prop.name, s, e, prop.params["weight"], interval, fd_interval,
                                                    freqs, start_ts, stop_ts))
                    elif pt == 1:
                        dim, s, e, si, ei = self.snap_box(lo, hi, dual=True, method=1)
                        if dim < 0:
                            continue
                        nd = prop.params["norm_dir"]
                        if nd < 0 or nd > 2:
                            if dim != 2:
                                continue
                            for n in range(3):
                                if e[n] == s[n]:
                                    nd = n
                        else:
                            for n in range(3):
                                if n == nd:
                                    continue
                                if lo[n] == hi[n]:
                                    if self.dl[n][s[n]] > lo[n] and s[n] > 0:
                                        s[n] -= 1
                                    if self.dl[n][s[n]] < lo[n] and e[n] < self.N[n] - 1:
                                        e[n] += 1
                        if s[nd] != e[nd]:
                            continue
                        iprobes.append(CurrentProbe(prop.name, s, e, nd, si, ei, prop.params["weight"], interval,
                                                    fd_interval, freqs, start_ts, stop_ts))
                    elif pt in (2, 3):
                        # field probes snap to the main (E) or dual (H) mesh, SnapMethod 0
                        # (openems.cpp:559-577, Processing::DefineStartStopCoord)
                        dim, s, e, _, _ = self.snap_box(lo, hi, dual=pt == 3, method=0)
                        if dim < 0:
                            continue
                        el = tuple(self._edge_length(n, tuple(int(v) for v in s), dual=pt == 3) for n in range(3))
                        fprobes.append(FieldProbe(prop.name, pt - 2, s, prop.params["weight"], interval,
                                                  fd_interval, freqs, start_ts, stop_ts, el))
            elif prop.kind == DUMP and prop.params["dump_type"] in (0, 1):
                # ProcessFieldsTD (openems.cpp:611-690): interval Nyquist/OverSampling
                field_ = prop.params["dump_type"]
                interp, dual = _dump_mesh(field_, prop.params["dump_mode"])
                interval = max(1, nyq // self.over_sampling)
                start_ts, stop_ts = 0, 0xFFFFFFFF
                st, sp = prop.params.get("start_time", 0.0), prop.params.get("stop_time", 0.0)
                if st > 0:
                    start_ts = int(math.floor(st / self.dT))
                if sp > 0:
                    stop_ts = int(math.ceil(sp / self.dT))
                if stop_ts <= start_ts:
                    start_ts, stop_ts = 0, 0xFFFFFFFF
                multi = len(prop.boxes) > 1
                for nb, (lo, hi, *_r) in enumerate(prop.boxes):
                    dim, s, e, _, _ = self.snap_box(lo, hi, dual=dual, method=0)
                    if dim < 0:
                        continue
                    name = f"{prop.name}_{nb}" if multi else prop.name
                    td_dumps.append(FieldDumpTD(name, field_, s, e, interval, interp, dual, start_ts, stop_ts))
            elif prop.kind == DUMP:
                dt_ = prop.params["dump_type"]
                if dt_ not in (10, 11):
                    continue
                fd_interval = 0
                freqs = []
                for f in prop.params["frequency"]:
                    nts = calc_nyquist_num(f, self.dT)
                    if nts == 0:
                        continue
                    if fd_interval == 0:
                        fd_interval = nyq
                    if fd_interval > nts:
                        fd_interval = nts
                    freqs.append(float(f))
                field_ = dt_ - 10
                interp, dual = _dump_mesh(field_, prop.params["dump_mode"])
                for lo, hi, _pr, _sq, _p, *_ in prop.boxes:
                    dim, s, e, _, _ = self.snap_box(lo, hi, dual=dual, method=0)
                    if dim < 0:
                        continue
                    dumps.append(FieldDumpFD(prop.name, field_, s, e, freqs, fd_interval, interp, dual))
        return vprobes, iprobes, dumps


def box_lines(start, stop, n):
    """Uniform helper: n+1 equally spaced lines between start and stop."""
    return np.linspace(start, stop, n + 1)


class GpuOperatorBuilder:
    """ctypes handle of oems_cuda_opbuild_* (the CUDA library is required)."""

    def __init__(self, lines, unit, lo, hi, par, background):
        import ctypes as C
        from . import _native
        self.C = C
        self.lib = _native.load_cuda()
        nl = np.array([len(l) for l in lines], np.uint32)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(l, np.float64) for l in lines]))
        self._keep = [nl, flat, np.ascontiguousarray(lo), np.ascontiguousarray(hi), np.ascontiguousarray(par),
                      np.ascontiguousarray(background, np.float64)]
        P = lambda a, t: a.ctypes.data_as(C.POINTER(t))
        self.h = C.c_void_p()
        rc = self.lib.opbuild_create(P(nl, C.c_uint), P(flat, C.c_double), float(unit), len(lo),
                                     P(self._keep[2], C.c_double), P(self._keep[3], C.c_double),
                                     P(self._keep[4], C.c_double), P(self._keep[5], C.c_double), C.byref(self.h))
        self._check(rc, "opbuild_create")

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.opbuild_last_error(self.h) if self.h else b""
            self.close()
            raise RuntimeError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def ec(self, Cc, G, L, R, var3=True):
        C = self.C
        P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        dt = C.c_double(0.0)
        self._check(self.lib.opbuild_ec(self.h, P(Cc), P(G), P(L), P(R), C.byref(dt) if var3 else None), "opbuild_ec")
        return dt.value

    def coefficients(self, dt, vv, vi, ii, iv):
        C = self.C
        P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        self._check(self.lib.opbuild_coefficients(self.h, float(dt), P(vv), P(vi), P(ii), P(iv)),
                    "opbuild_coefficients")

    def close(self):
        if self.h:
            self.lib.opbuild_destroy(self.h)
            self.h = None
