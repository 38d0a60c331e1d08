"""The operator in cylindrical coordinates: Operator_Cylinder (FDTD/operator_cylinder.cpp) and
the build half of Operator_Ext_Cylinder (FDTD/extensions/operator_ext_cylinder.cpp:44-112).

The mesh is (rho, alpha, z): ``lines[0]`` radii and ``lines[2]`` heights in drawing units,
``lines[1]`` angles in radians.  Material, metal, excitation and probe boxes are boxes in these
coordinates.  The update equations are the Cartesian ones; only the equivalent circuit changes:
alpha edges are rho times their angle (GetEdgeLength, :204-210), z faces are annular sectors
(GetNodeArea, :158-189) and the node widths of alpha carry the radius (GetNodeWidth, :134-143).

* Closed alpha (a span of 2*pi within 1e-6, SetupCSXGrid :469-487): the last angle is set to
  a0 + 2*pi and the line a1 + 2*pi is appended, so alpha line N-2 is line 0 once more; the engine
  copies the tangential voltages of line N-2 onto line 0 after each voltage update and the
  tangential currents of line 0 onto line N-2 after each current update.
* rho = 0 on a closed mesh (CC_R0_included): the z voltages on the axis are updated from the
  sum of the alpha currents around it with the coefficients ``vv_r0``/``vi_r0`` built here from
  the summed capacitance and conductance of every z edge on the axis; metal on the axis zeroes
  them.  A mesh that includes rho = 0 uses the conservative Var1 timestep (CalcTimestep, :88-95).

Built here: materials (eps, kappa, mue, sigma) and metal (PEC) on boxes and on cylinder primitives
whose axis is the z axis, soft/hard and weighted excitations,
Mur walls that the reference accepts in cylindrical coordinates (operator_ext_mur_abc.cpp:47-54;
the others are dropped as there, leaving PEC), UPML on the rho and z walls and on the alpha
walls of an open mesh (graded with rho along alpha), Drude/Lorentz
materials (their tables read only the equivalent circuit, which carries the geometry), parallel
RC lumped elements (Calc_LumpedElements with the cylindrical edge area over length), lumped RLC
elements (Operator_Ext_LumpedRLC reads the equivalent circuit and snaps on the full mesh),
conducting sheets (their edge length over node width taken cylindrically), voltage, current and
field probes.  Not built for this mesh: TFSF (rejected by the reference too) and field dumps.
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass

import numpy as np

from .operator import DUMP, EPS0, MATERIAL, METAL, MUE0, Z0, Grid, Operator, _axes

CLOSED_ALPHA_THRESHOLD = 1e-6     # OPERATOR_CYLINDER_CLOSED_ALPHA_THRESHOLD (operator_cylinder.h:21)
TWO_PI = 2.0 * math.pi


@dataclass
class CylinderTable:
    """Engine_Ext_Cylinder's inputs (FDTD/extensions/engine_ext_cylinder.cpp:23-101)."""
    closed_alpha: bool
    r0_included: bool
    vv_r0: np.ndarray             # float32 [Nz]: z voltage on the axis (empty without rho = 0)
    vi_r0: np.ndarray             # float32 [Nz]: weight of each alpha current around it


class _AlphaWrapPainter:
    """A painter whose alpha coordinates are folded back by 2*pi on a closed mesh first: above
    a0 + 2*pi as Operator_Cylinder::GetMaterial does (operator_cylinder.cpp:74-87), or from
    a0 + 2*pi on (``inclusive``) as its GetYeeCoords does (:119-129); below a0 both add 2*pi."""

    def __init__(self, inner, a0, inclusive):
        self._p = inner
        self.a0 = float(a0)
        self.inclusive = inclusive

    def __getattr__(self, k):
        return getattr(self._p, k)

    def paint(self, cx, cy, cz):
        cy = np.asarray(cy, np.float64)
        top = cy >= self.a0 + TWO_PI if self.inclusive else cy > self.a0 + TWO_PI
        cy = np.where(top, cy - TWO_PI, np.where(cy < self.a0, cy + TWO_PI, cy))
        return self._p.paint(cx, cy, cz)


class OperatorCylinder(Operator):
    """Operator (FDTD/operator.cpp) with Operator_Cylinder's geometry."""

    def __init__(self, structure, grid: Grid, excitation, bc=(0,) * 6, **kw):
        lines = [np.array(l, np.float64) for l in grid.lines]
        a = lines[1]
        span = abs(a[-1] - a[0])
        closed = abs(span - TWO_PI) < CLOSED_ALPHA_THRESHOLD
        if closed:
            a[-1] = TWO_PI + a[0]
            lines[1] = np.append(a, TWO_PI + a[1])
        elif span > TWO_PI:
            raise ValueError("OperatorCylinder: the alpha span must not exceed 2*pi")
        if lines[0][0] < 0:
            raise ValueError("OperatorCylinder: rho < 0 is not allowed")
        self.closed_alpha = bool(closed)
        # on an open mesh rho = 0 needs no special treatment (E_alpha/E_z there are PEC anyway)
        self.r0_included = bool(lines[0][0] == 0.0 and closed)
        bc = [int(b) for b in bc]
        # UPML: on the alpha walls of an open mesh only (a closed mesh has none), and not at rho = 0
        if closed and (bc[2] == 3 or bc[3] == 3):
            raise ValueError("OperatorCylinder: a closed alpha mesh has no alpha walls for a UPML")
        if bc[0] == 3 and lines[0][0] == 0.0:
            raise ValueError("OperatorCylinder: no UPML at rho = 0")
        # Mur walls the reference rejects in cylindrical coordinates are dropped (PEC remains)
        self.dropped_mur = []
        for w in range(6):
            if bc[w] != 2:
                continue
            ny, top = w // 2, w % 2
            if (ny == 0 and not top and (self.r0_included or self.closed_alpha)) or (ny == 1 and self.closed_alpha):
                bc[w] = 0
                self.dropped_mur.append(w)
        structure = self._axial_boxes(structure)
        super().__init__(structure, Grid(lines, unit=grid.unit), excitation, bc=bc, **kw)
        self._mat_raw, self._matmetal_raw = self._mat, self._matmetal
        if self.closed_alpha:
            self._mat = _AlphaWrapPainter(self._mat, self.L[1][0], inclusive=False)
            # PEC (CalcPEC_Range) looks the metal up at Yee coordinates
            self._matmetal = _AlphaWrapPainter(self._matmetal, self.L[1][0], inclusive=True)
        for prop in structure.props:
            if prop.kind == DUMP and (prop.params["dump_type"] not in (10, 11) or prop.params["dump_mode"] != 0):
                raise ValueError(f"OperatorCylinder: {prop.name}: on a cylindrical mesh only frequency-domain "
                                 "dumps without interpolation are built")
            if prop.params.get("exc_type") == 10:
                raise ValueError("OperatorCylinder: TFSF is not cylinder-safe (operator_ext_tfsf.h:40)")


    @staticmethod
    def _axial_boxes(structure):
        """CSXCAD's cylinder primitives are Cartesian. A cylinder (or shell) whose axis is the z
        axis is the box rho <= R (|rho - R| <= width/2) over every alpha in (rho, alpha, z), and is
        painted as that box; others are rejected.  Works on a shallow copy of the structure."""
        recs = []
        for r in structure.boxes:
            shape = r[7] if len(r) > 7 else None
            if shape is None:
                recs.append(r)
                continue
            a, pb, pc, radius, width = shape
            if r[4].kind not in (MATERIAL, METAL):
                # excitations, probes, dumps, lumped elements and sheets snap their property's own
                # box list, which keeps the Cartesian bounding box of the primitive
                raise ValueError(f"OperatorCylinder: {r[4].name}: cylinder primitives are built for "
                                 "materials and metal only; give this property boxes in (rho, alpha, z)")
            if a != 2 or pb != 0.0 or pc != 0.0:
                raise ValueError("OperatorCylinder: only cylinder primitives on the z axis are built; "
                                 "use boxes in (rho, alpha, z)")
            r_lo, r_hi = (0.0, radius) if width is None else (radius - 0.5 * width, radius + 0.5 * width)
            lo = np.array([max(r_lo, 0.0), -1e30, r[0][2]])
            hi = np.array([r_hi, 1e30, r[1][2]])
            recs.append((lo, hi) + tuple(r[2:7]) + (None,))
        out = copy.copy(structure)
        out.boxes = recs
        return out

    # ---- geometry on index arrays (all lengths in metres) -------------------------------------
    def _line(self, k, idx, dual):
        """GetDiscLine: 0 outside [0, N)."""
        idx = np.asarray(idx)
        src = self.dl[k] if dual else self.L[k]
        ok = (idx >= 0) & (idx < self.N[k])
        return np.where(ok, src[np.clip(idx, 0, self.N[k] - 1)], 0.0)

    def _cart_len(self, k, idx, dual):
        """Operator::GetEdgeLength = GetDiscDelta * gridDelta (0 outside [0, N))."""
        idx = np.asarray(idx)
        src = self.dd[k] if dual else self.md[k]
        ok = (idx >= 0) & (idx < self.N[k])
        return np.where(ok, src[np.clip(idx, 0, self.N[k] - 1)] * self.unit, 0.0)

    def _cyl_len(self, k, pos, dual):
        """Operator_Cylinder::GetEdgeLength (:204-210): alpha edges times rho (drawing units)."""
        v = self._cart_len(k, pos[k], dual)
        return v * self._line(0, pos[0], dual) if k == 1 else v

    def _node_width(self, ny, pos, dual):
        """GetNodeWidth, unsigned positions (:134-143)."""
        w = self._cart_len(ny, pos[ny], not dual)
        if ny == 1:
            w = w * self._line(0, pos[0], dual)
        return np.where(np.asarray(pos[ny]) >= self.N[ny], 0.0, w)

    def _wrap_int(self, pos):
        """The int-position wrappers (:145-156, :191-202): 0 for a negative rho or z position or
        a negative alpha position on an open mesh; a closed mesh folds alpha -1 to N-3."""
        p = [np.asarray(v) for v in pos]
        bad = (p[0] < 0) | (p[2] < 0)
        if self.closed_alpha:
            p[1] = np.where(p[1] < 0, p[1] + int(self.N[1]) - 2, p[1])
        else:
            bad = bad | (p[1] < 0)
        return p, bad

    def _node_width_i(self, ny, pos, dual):
        p, bad = self._wrap_int(pos)
        return np.where(bad, 0.0, self._node_width(ny, p, dual))

    def _node_area(self, ny, pos, dual):
        """GetNodeArea, unsigned positions (:158-189): z faces are annular sectors."""
        out_of = (np.asarray(pos[ny]) >= self.N[ny]) | (np.asarray(pos[0]) >= self.N[0])
        if ny == 2:
            da = self._cart_len(1, pos[1], dual) / self.unit
            if dual:
                r1 = self._line(0, pos[0], False) * self.unit
                r2 = r1 + self._cyl_len(0, pos, False)
            else:
                r2 = self._line(0, pos[0], True) * self.unit
                r1 = r2 - self._cyl_len(0, pos, True)
            area = np.where(r1 <= 0, da / 2 * r2 ** 2, da / 2 * (r2 ** 2 - r1 ** 2))
        else:
            area = self._node_width((ny + 1) % 3, pos, dual) * self._node_width((ny + 2) % 3, pos, dual)
        return np.where(out_of, 0.0, area)

    def _node_area_i(self, ny, pos, dual):
        p, bad = self._wrap_int(pos)
        return np.where(bad, 0.0, self._node_area(ny, p, dual))

    def _edge_area(self, ny, pos, dual):
        """GetEdgeArea (:219-225)."""
        if ny != 0:
            return self._node_area(ny, pos, dual)
        return self._cyl_len(1, pos, not dual) * self._cyl_len(2, pos, not dual)

    def _raw_delta_c(self, k, idx):
        """GetRawDiscDelta with the closed-alpha wrap (:65-73)."""
        L = self.L[k]
        N = len(L)
        idx = np.asarray(idx)
        out = np.where(idx < 0, L[0] - L[1],
                       np.where(idx >= N - 1, L[N - 2] - L[N - 1], L[np.clip(idx + 1, 0, N - 1)] - L[np.clip(idx, 0, N - 1)]))
        if self.closed_alpha and k == 1:
            out = np.where(idx == -1, L[N - 2] - L[N - 3], out)
            out = np.where(idx == N - 1, L[2] - L[1], out)
        return out

    def _grid_pos(self):
        N = [int(v) for v in self.N]
        return [np.arange(N[0]).reshape(-1, 1, 1), np.arange(N[1]).reshape(1, -1, 1), np.arange(N[2]).reshape(1, 1, -1)]

    def _edge_length(self, n, pos, dual=False):
        """Operator_Cylinder::GetEdgeLength for one position (metres)."""
        return float(self._cyl_len(n, [np.asarray(int(v)) for v in pos], dual))

    # ---- effective material, AverageMatQuarterCell (FDTD/operator.cpp:1447-1564) --------------
    def eff_mat(self, n):
        a, p, pp = _axes(n)
        P = self._grid_pos()
        N = [int(v) for v in self.N]
        i_n, i_p, i_pp = np.arange(N[a]), np.arange(N[p]), np.arange(N[pp])
        delta, deltaP, deltaPP = self._raw_delta_c(a, i_n), self._raw_delta_c(p, i_p), self._raw_delta_c(pp, i_pp)
        delta_M = self._raw_delta_c(a, i_n - 1)
        deltaP_M = self._raw_delta_c(p, i_p - 1)
        deltaPP_M = self._raw_delta_c(pp, i_pp - 1)
        L, Lp, Lpp = self.L[a], self.L[p], self.L[pp]

        def shifted(offsets):
            """The position grid moved by {axis: offset}."""
            q = list(P)
            for ax, off in offsets.items():
                q[ax] = q[ax] + off
            return q
        cn = L + delta * 0.5
        cp_up, cp_dn = Lp + deltaP * 0.25, Lp - deltaP_M * 0.25
        cpp_up, cpp_dn = Lpp + deltaPP * 0.25, Lpp - deltaPP_M * 0.25
        samples = [(cp_up, cpp_up, {}), (cp_dn, cpp_up, {p: -1}),
                   (cp_up, cpp_dn, {pp: -1}), (cp_dn, cpp_dn, {p: -1, pp: -1})]
        eps_acc = kap_acc = area = None
        for cpv, cppv, sh in samples:
            e, k = self._lookup(n, cn, cpv, cppv, ("epsilon", "kappa"))
            A = np.broadcast_to(self._node_area_i(n, shifted(sh), True), e.shape)
            if eps_acc is None:
                eps_acc, kap_acc, area = e * A, k * A, A.copy()
            else:
                eps_acc = eps_acc + e * A
                kap_acc = kap_acc + k * A
                area = area + A
        eff0 = eps_acc * (EPS0 / area)
        eff1 = kap_acc / area
        cpm = Lp + deltaP * 0.5
        cppm = Lpp + deltaPP * 0.5
        with np.errstate(divide="ignore", invalid="ignore"):
            mu_dn, sg_dn = self._lookup(n, L - delta_M * 0.25, cpm, cppm, ("mue", "sigma"))
            Ddn = np.broadcast_to(self._node_width_i(n, shifted({a: -1}), True), mu_dn.shape)
            eff2 = Ddn / mu_dn
            eff3 = np.where(sg_dn != 0, Ddn / np.where(sg_dn != 0, sg_dn, 1.0), 0.0)
            length = Ddn
            mu_up, sg_up = self._lookup(n, L + delta * 0.25, cpm, cppm, ("mue", "sigma"))
            Dup = np.broadcast_to(self._node_width_i(n, P, True), mu_up.shape)
            eff2 = eff2 + Dup / mu_up
            eff3 = np.where(sg_up != 0, eff3 + Dup / np.where(sg_up != 0, sg_up, 1.0), 0.0)
            length = length + Dup
            eff2 = length * MUE0 / eff2
            eff3 = np.where(eff3 != 0, length / np.where(eff3 != 0, eff3, 1.0), eff3)
        for arr in (eff0, eff1, eff2, eff3):
            if not np.isfinite(arr).all():
                raise ValueError("OperatorCylinder: an effective material parameter is not finite")
        return eff0, eff1, eff2, eff3

    # ---- equivalent circuit, Calc_ECPos (FDTD/operator.cpp:1189-1254) ------------------------
    def _ec_double(self):
        P = self._grid_pos()
        out = []
        self._eff = {}
        for n in range(3):
            e0, e1, e2, e3 = self._eff[n] = self.eff_mat(n)
            D, A = self._cyl_len(n, P, False), self._edge_area(n, P, False)
            Dh, Ah = self._cyl_len(n, P, True), self._edge_area(n, P, True)
            with np.errstate(divide="ignore", invalid="ignore"):
                out.append((np.where(D != 0, e0 * A / D, 0.0), np.where(D != 0, e1 * A / D, 0.0),
                            np.where(Dh != 0, e2 * Ah / Dh, 0.0), np.where(Dh != 0, e3 * Ah / Dh, 0.0)))
        return out

    def eff_region(self, n, start, nl):
        """The effective material of direction n on the box start..start+nl (from the full mesh)."""
        if not hasattr(self, "_eff"):
            self._eff = {k: self.eff_mat(k) for k in range(3)}
        sl = tuple(slice(int(start[a]), int(start[a] + nl[a])) for a in range(3))
        return [x[sl] for x in self._eff[n]]

    def _node_width_at(self, ny, pos, dual=False):
        """Operator_Cylinder::GetNodeWidth (:134-143) for one position (metres)."""
        return float(self._node_width(ny, [np.asarray(int(v)) for v in pos], dual))

    def _area_over_length(self, ny, pos):
        P = [np.asarray(int(v)) for v in pos]
        return float(self._edge_area(ny, P, False)) / float(self._cyl_len(ny, P, False))

    def _grading_kappa(self, ny, pos_axes):
        """CalcGradingKappa (operator_ext_upml.cpp:269-343) on this mesh: along rho and z as on a
        Cartesian mesh; along alpha the width, the depth and the edge length are scaled by the
        main rho line of the position (:280-284, :313-317), so that grading is returned as a
        [rho][alpha][1] array over the region."""
        kv, ki = super()._grading_kappa(ny, pos_axes)
        BC, sz = self._pml_bc, self._pml_sz
        n = 1
        if not (BC[2] == 3 or BC[3] == 3):
            return kv, ki
        u = self.unit
        L = self.L[n]
        N = int(self.N[n])
        pos = np.asarray(pos_axes[1])[None, :]
        rho = self.L[0][np.asarray(pos_axes[0])][:, None]
        el = (self.md[n][pos] * u) * rho                     # Operator_Cylinder::GetEdgeLength(1, pos)
        shape = (rho.shape[0], pos.shape[1])
        kvn = np.zeros(shape)
        kin = np.zeros(shape)
        low = np.broadcast_to((pos <= sz[2]) & (BC[2] == 3), shape)
        up = np.broadcast_to((pos >= N - 1 - sz[3]) & (BC[3] == 3), shape) & ~low
        err = dict(divide="ignore", invalid="ignore", over="ignore")
        if low.any():
            width = (L[sz[2]] - L[0]) * u
            depth = width - (L[pos] - L[0]) * u
            width = width * rho
            depth = depth * rho
            if n == ny:
                depth = depth - el / 2
            dl = width / sz[2]
            with np.errstate(**err):
                g = self._grading(depth, dl, width, Z0, float(sz[2]))
            kvn = np.where(low & (depth > 0), g, kvn)
            if n == ny:
                depth = depth + el / 2
            if n != ny:
                depth = depth - el / 2
            depth = np.where(depth < 0, 0.0, depth)
            with np.errstate(**err):
                g = self._grading(depth, dl, width, Z0, float(sz[2]))
            kin = np.where(low & (depth > 0), g, kin)
        if up.any():
            width = (L[N - 1] - L[N - sz[3] - 1]) * u
            depth = width - (L[N - 1] - L[pos]) * u
            width = width * rho
            depth = depth * rho
            if n == ny:
                depth = depth + el / 2
            with np.errstate(**err):
                dl = width / sz[2] if sz[2] else np.full(shape, np.inf)   # the lower wall's size
                g = self._grading(depth, dl, width, Z0, float(sz[2]))
            kvn = np.where(up & (depth > 0), g, kvn)
            if n == ny:
                depth = depth - el / 2
            if n != ny:
                depth = depth + el / 2
            depth = np.where(depth > width, 0.0, depth)
            with np.errstate(**err):
                g = self._grading(depth, dl, width, Z0, float(sz[2]))
            kin = np.where(up & (depth > 0), g, kin)
        kv[1] = np.nan_to_num(kvn)[:, :, None]
        ki[1] = np.nan_to_num(kin)[:, :, None]
        return kv, ki

    def _edge_geometry(self, n, pos_axes):
        P = [np.asarray(pos_axes[0]).reshape(-1, 1, 1), np.asarray(pos_axes[1]).reshape(1, -1, 1),
             np.asarray(pos_axes[2]).reshape(1, 1, -1)]
        return (self._cyl_len(n, P, False), self._edge_area(n, P, False),
                self._cyl_len(n, P, True), self._edge_area(n, P, True))

    def calc_ec(self):
        ec = self._ec_double()
        shape = (3,) + tuple(int(v) for v in self.N)
        self.EC_C, self.EC_G, self.EC_L, self.EC_R = (np.empty(shape, self.ft) for _ in range(4))
        for n in range(3):
            for d, v in zip((self.EC_C, self.EC_G, self.EC_L, self.EC_R), ec[n]):
                d[n] = v
        # Calc_ECPos of the z edges on the axis, in double, for the rho = 0 extension
        self._r0_CG = (ec[2][0][0], ec[2][1][0])

    # ---- snapping (operator_cylinder.cpp:100-108, 227-296) ---------------------------------
    def _num_lines(self, ny, full):
        """GetNumberOfLines: a closed mesh hides its last two alpha lines from processing."""
        if not full and ny == 1 and self.closed_alpha:
            return int(self.N[1]) - 2
        return int(self.N[ny])

    def fit_to_alpha_range(self, a, full=False):
        """FitToAlphaRange (:227-249): a coordinate shifted by 2*pi into the alpha lines' range."""
        lo = float(self.L[1][0])
        hi = float(self.L[1][self._num_lines(1, full) - 1])
        if lo <= a <= hi:
            return a
        while a < lo:
            a += TWO_PI
            if a > hi:
                return a - TWO_PI
            if a > lo:
                return a
        while a > hi:
            a -= TWO_PI
            if a < lo:
                return a + TWO_PI
            if a < hi:
                return a
        return a

    def snap_line(self, ny, coord, dual=False, full=False):
        if ny == 1:
            coord = self.fit_to_alpha_range(float(coord))
        return super().snap_line(ny, coord, dual, full)

    def snap_box(self, start, stop, dual=False, method=0, full=False):
        """SnapBox2Mesh (:270-290): the alpha span is centred by FitToAlphaRange and clamped to
        the alpha lines before the Cartesian snapping."""
        a_min = float(self.L[1][0])
        a_max = float(self.L[1][self._num_lines(1, full) - 1])
        a_size = float(stop[1]) - float(start[1])
        a_center = self.fit_to_alpha_range(0.5 * (float(stop[1]) + float(start[1])))
        a_start = a_center - a_size / 2
        a_stop = a_start + a_size
        a_stop = min(max(a_stop, a_min), a_max)
        a_start = min(max(a_start, a_min), a_max)
        l_start = np.array([start[0], a_start, start[2]], np.float64)
        l_stop = np.array([stop[0], a_stop, stop[2]], np.float64)
        return super().snap_box(l_start, l_stop, dual, method, full)

    def _weight_coords(self, cs, x, y, z):
        """GetYeeCoords folds alpha from a0 + 2*pi on back by 2*pi on a closed mesh (:119-129)."""
        r, a, zz = super()._weight_coords(cs, x, y, z)
        if self.closed_alpha:
            a0 = float(self.L[1][0])
            # two independent tests in the reference's order: a value that rounding leaves below
            # a0 after the first fold is folded back up by the second
            if a >= a0 + TWO_PI:
                a -= TWO_PI
            if a < a0:
                a += TWO_PI
        return r, a, zz

    def _yee_painter(self, kinds):
        p = super()._yee_painter(kinds)
        return _AlphaWrapPainter(p, self.L[1][0], inclusive=True) if self.closed_alpha else p

    def _mur_painter(self):
        return self._mat_raw

    def _gpu_core(self):
        raise ValueError("OperatorCylinder: the device operator build is Cartesian only")

    # ---- timestep ------------------------------------------------------------------------------
    def calc_timestep(self):
        """Operator_Cylinder::CalcTimestep (:88-95): Var1 when the mesh includes rho = 0."""
        if self.L[0][0] == 0.0:
            return self.calc_timestep_var1()
        return self.calc_timestep_var3()

    def calc_timestep_var1(self):
        """Operator::CalcTimestep_Var1 (FDTD/operator.cpp:1892-1942), with AdrOp cell reflection
        at the mesh ends; double arithmetic on the float equivalent circuit."""
        C = self.EC_C.astype(np.float64)
        Lh = self.EC_L.astype(np.float64)

        def sh(arr, ax):
            idx = np.clip(np.arange(arr.shape[ax]) - 1, 0, arr.shape[ax] - 1)
            return np.take(arr, idx, axis=ax)
        dT = 1e200
        with np.errstate(divide="ignore", invalid="ignore"):
            for n in range(3):
                _, p, pp = _axes(n)
                s = 4 / Lh[p] + 4 / sh(Lh[p], pp) + 4 / Lh[pp] + 4 / sh(Lh[pp], p)
                newT = 2 / np.sqrt(s / C[n])
                cand = newT[np.isfinite(newT) & (newT > 0)]
                if cand.size:
                    dT = min(dT, float(cand.min()))
        if dT == 0 or dT >= 1e200:
            raise ValueError("OperatorCylinder: timestep is zero")
        return dT

    # ---- boundary conditions -------------------------------------------------------------------
    def _apply_magnetic_bc(self, dirs):
        """Operator_Cylinder::ApplyMagneticBC (:510-523): no PMC on closed alpha walls nor at rho = 0."""
        dirs = list(dirs)
        if self.closed_alpha:
            dirs[2] = dirs[3] = False
        if self.r0_included:
            dirs[0] = False
        return super()._apply_magnetic_bc(dirs)

    # ---- Operator_Ext_Cylinder::BuildExtension (operator_ext_cylinder.cpp:44-112) -------------
    def _build_cylinder(self):
        if not (self.closed_alpha or self.r0_included):
            return None
        Nz = int(self.N[2])
        if not self.r0_included:
            return CylinderTable(self.closed_alpha, False, np.zeros(0, self.ft), np.zeros(0, self.ft))
        Cd, Gd = self._r0_CG                     # [alpha][z], double
        Na = int(self.N[1])
        C = np.zeros(Nz)
        G = np.zeros(Nz)
        for ia in range(Na - 2):                 # in the reference's summation order
            C = C + Cd[ia]
            G = G + Gd[ia]
        dT = self.dT
        with np.errstate(divide="ignore", invalid="ignore"):
            vv_r0 = ((1 - dT * G / 2 / C) / (1 + dT * G / 2 / C)).astype(self.ft)
            vi_r0 = ((dT / C) / (1 + dT * G / 2 / C)).astype(self.ft)
        self.vv[2, 0, 0, :] = 1
        self.EC_C[2, 0, :, :] = C.astype(self.ft)[None, :]
        self.EC_G[2, 0, :, :] = G.astype(self.ft)[None, :]
        # metal on the axis: the Yee point of z edge (0, N-2, z), alpha folded to a0 (GetYeeCoords)
        m = self._matmetal_raw.paint(np.array([self.L[0][0]]), np.array([self.L[1][0]]), self.dl[2])
        for z in range(Nz):
            pid = int(m[0, 0, z])
            if pid >= 0 and self._matmetal.props[pid].kind == METAL:
                self.vv[2, 0, 0, z] = 0
                vv_r0[z] = 0
                vi_r0[z] = 0
                self.EC_C[2, 0, 0, z] = 0
                self.EC_G[2, 0, 0, z] = 0
        return CylinderTable(True, True, vv_r0, vi_r0)

    def build(self, num_ts, device=None):
        if device not in (None, "cpu"):
            raise ValueError("OperatorCylinder: the operator is built on the host")
        data = super().build(num_ts, device="cpu")
        data.rho_lines = (np.array(self.L[0], np.float64), np.array(self.dl[0], np.float64))   # main, dual
        data.closed_alpha = self.closed_alpha
        data.r0_included = self.r0_included
        return data
