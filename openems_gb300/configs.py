"""Synthetic workloads with the shapes of the engine's benchmark configurations.

No public dataset is involved: every geometry is generated here from a fixed seed.

* ``plain_cube``   -- 100^3 lines, 1 mm, vacuum, PEC walls, soft Ez point source (f0 2 GHz,
                      fc 1 GHz), a 5-edge Ez voltage probe and a 1-cell H loop, sampled every step.
* ``patch``        -- 160x160x80 graded mesh (0.3-2 mm, ratio <= 1.4), FR4-like slab
                      (eps_r 3.38, kappa 1e-3 S/m, 1.524 mm) with PEC ground + 32x40 mm patch,
                      UPML 8 on all sides, 50 Ohm lumped port (f0 2 GHz, fc 1.5 GHz), port U/I
                      probes and an NF2FF box (6 faces, E and H FD dumps) at 1.5/2/2.5 GHz.
* ``stress``       -- 512x512x256 lines, 1 mm, 64 seeded random blocks (eps_r U[1,10],
                      kappa U[0,0.1] S/m), 10 % of them Drude/Lorentz (plasma 1-10 GHz, damping
                      1e8-1e9 1/s), first-order Mur on all walls, 4 seeded Gaussian point sources.
* ``batch_instance`` -- one simulation of the batched form: lines U[48,160]^3, pitch 0.5-2 mm,
                      UPML 8, one dielectric block eps_r U[2,12], a 50 Ohm lumped port with a
                      Gaussian (f0 U[1,5] GHz, fc = f0/2), steps U[4000,12000].
* ``smoke_case`` / ``cavity`` / ``small_mixed`` -- small cases for tests.

Every builder accepts a ``scale`` (or explicit sizes) so the tests can run the same geometry
at sizes the CPU checker finishes in seconds.
"""
from __future__ import annotations

import numpy as np

from .excitation import Excitation
from .operator import Grid, Operator, Structure


# ------------------------------------------------------------------------------------------
def _uniform(n, pitch=1.0):
    return np.arange(n, dtype=np.float64) * pitch


def graded_lines(n, fine_lo, fine_hi, d_fine, d_max, ratio=1.3, must=()):
    """Exactly ``n`` lines: uniform spacing d_fine on [fine_lo, fine_hi] (plus the ``must``
    coordinates), growing geometrically by ``ratio`` outward (capped at d_max), alternating
    sides until n lines exist."""
    core = list(np.arange(fine_lo, fine_hi + 0.5 * d_fine, d_fine))
    core = sorted(set([round(c, 9) for c in core] + [round(m, 9) for m in must]))
    lines = list(core)
    dl = dh = d_fine
    side = 0
    while len(lines) < n:
        if side == 0:
            dl = min(dl * ratio, d_max)
            lines.insert(0, lines[0] - dl)
        else:
            dh = min(dh * ratio, d_max)
            lines.append(lines[-1] + dh)
        side ^= 1
    while len(lines) > n:
        lines.pop(-1 if side else 0)
        side ^= 1
    return np.array(lines)


# ------------------------------------------------------------------------------------------
def plain_cube(n=100, steps=5000, pitch_mm=1.0):
    """100^3 vacuum cube with PEC walls and a soft Ez point source at the centre edge."""
    g = Grid([_uniform(n, pitch_mm)] * 3, unit=1e-3)
    csx = Structure()
    c = (n // 2) * pitch_mm
    exc = Excitation()
    exc.SetupGaussianPulse(2e9, 1e9)
    csx.AddExcitation("excite", 0, [0, 0, 1]).AddBox([c, c, c], [c, c, c + pitch_mm])
    csx.AddProbe("ut1", 0, weight=1.0, interval=1).AddBox([c, c, c - 2 * pitch_mm], [c, c, c + 3 * pitch_mm])
    h = 0.5 * pitch_mm
    csx.AddProbe("it1", 1, weight=1.0, norm_dir=2, interval=1).AddBox([c - h, c - h, c + h], [c + h, c + h, c + h])
    op = Operator(csx, g, exc, bc=(0,) * 6)
    return op.build(steps)


def smoke_case(n=(17, 13, 15), steps=60):
    """Small mixed case touching UPML, Mur, a dielectric block and both probe types."""
    lines = [_uniform(k, 1.0) for k in n]
    g = Grid(lines, unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(8e9, 6e9)
    csx.AddMaterial("diel", epsilon=3.0, kappa=0.02).AddBox([4, 3, 3], [9, 8, 9])
    c = [k // 2 for k in n]
    csx.AddExcitation("excite", 0, [0, 0, 1]).AddBox([c[0], c[1], c[2]], [c[0], c[1], c[2] + 1])
    csx.AddProbe("ut1", 0, interval=1).AddBox([c[0], c[1], c[2] - 2], [c[0], c[1], c[2] + 2])
    csx.AddProbe("it1", 1, norm_dir=2, interval=1).AddBox([c[0] - .5, c[1] - .5, c[2] + .5], [c[0] + .5, c[1] + .5, c[2] + .5])
    op = Operator(csx, g, exc, bc=(3, 0, 2, 2, 0, 3), pml_size=(4, 4, 4, 4, 4, 4))
    return op.build(steps)


def small_mixed(n=(18, 16, 14), steps=200, bc=(3, 3, 2, 2, 0, 3), pml=4, seed=1, dispersive=True, dump=True):
    """Everything at once on a small mesh: UPML + Mur + PEC walls, dielectric and Drude/Lorentz
    blocks, a metal plate, a lumped port with U/I probes and DFTs, and E/H FD dumps."""
    rng = np.random.default_rng(seed)
    lines = [np.cumsum(np.concatenate([[0.0], rng.uniform(0.6, 1.2, k - 1)])) for k in n]
    g = Grid(lines, unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(6e9, 5e9)
    L = [l[-1] for l in g.lines]
    csx.AddMaterial("diel", epsilon=4.0, kappa=0.05).AddBox([0.3 * L[0], 0.2 * L[1], 0.2 * L[2]], [0.6 * L[0], 0.7 * L[1], 0.5 * L[2]])
    if dispersive:
        csx.AddLorentzMaterial("drude", epsilon=1.5, eps_plasma_freq=[5e9], eps_relax_time=[2e-9]).AddBox(
            [0.55 * L[0], 0.4 * L[1], 0.4 * L[2]], [0.8 * L[0], 0.8 * L[1], 0.8 * L[2]], priority=5)
        csx.AddLorentzMaterial("lor", epsilon=2.0, eps_plasma_freq=[8e9], eps_relax_time=[1e-9],
                               eps_lor_pole_freq=[3e9]).AddBox([0.2 * L[0], 0.6 * L[1], 0.55 * L[2]],
                                                              [0.4 * L[0], 0.85 * L[1], 0.75 * L[2]], priority=6)
    csx.AddMetal("plate").AddBox([0.25 * L[0], 0.25 * L[1], 0.3 * L[2]], [0.45 * L[0], 0.45 * L[1], 0.3 * L[2]], priority=10)
    gl = g.lines
    px, py = gl[0][n[0] // 2], gl[1][n[1] // 2]
    z0, z1 = gl[2][n[2] // 2 - 1], gl[2][n[2] // 2 + 1]
    csx.AddLumpedElement("port_R", ny=2, R=50.0, caps=True).AddBox([px, py, z0], [px, py, z1], priority=20)
    csx.AddExcitation("port_exc", 0, [0, 0, -1.0]).AddBox([px, py, z0], [px, py, z1], priority=20)
    freqs = [3e9, 5e9, 7e9]
    csx.AddProbe("port_ut", 0, weight=-1.0, interval=1, frequency=freqs).AddBox([px, py, z0], [px, py, z1])
    zm = 0.5 * (z0 + z1)
    csx.AddProbe("port_it", 1, weight=1.0, norm_dir=2, interval=1, frequency=freqs).AddBox([px, py, zm], [px, py, zm])
    if dump:
        lo = [l[2] for l in gl]
        hi = [l[-3] for l in gl]
        for f_idx, name in ((10, "nf2ff_E"), (11, "nf2ff_H")):
            d = csx.AddDump(name, dump_type=f_idx, dump_mode=1, frequency=[4e9, 6e9])
            d.AddBox([lo[0], lo[1], lo[2]], [hi[0], hi[1], lo[2]])
            d.AddBox([lo[0], lo[1], lo[2]], [lo[0], hi[1], hi[2]])
        # the other two interpolation types: cell-interpolated (dual mesh) and raw Yee values
        for f_idx, name in ((10, "cell_E"), (11, "cell_H")):
            csx.AddDump(name, dump_type=f_idx, dump_mode=2, frequency=[5e9]).AddBox(
                [lo[0], lo[1], hi[2]], [hi[0], hi[1], hi[2]])
        for f_idx, name in ((10, "raw_E"), (11, "raw_H")):
            csx.AddDump(name, dump_type=f_idx, dump_mode=0, frequency=[5e9]).AddBox(
                [gl[0][0], gl[1][0], gl[2][0]], [gl[0][-1], gl[1][-1], gl[2][3]])
    op = Operator(csx, g, exc, bc=bc, pml_size=(pml,) * 6)
    return op.build(steps)


# ------------------------------------------------------------------------------------------
def stress(shape=(512, 512, 256), steps=2000, nblocks=64, seed=20261204, pitch_mm=1.0, bc=(2,) * 6,
           dispersive=True):
    """Bandwidth-stress mesh: random dielectric/lossy blocks, 10 % dispersive, Mur walls (``bc``
    and ``dispersive`` give the PEC / non-dispersive variants of the same blocks)."""
    rng = np.random.default_rng(seed)
    g = Grid([_uniform(k, pitch_mm) for k in shape], unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(3e9, 2e9)
    ndisp = max(1, int(round(0.1 * nblocks)))
    disp = set(rng.choice(nblocks, size=ndisp, replace=False).tolist())
    scale = min(shape) / 256.0
    for b in range(nblocks):
        side = rng.integers(max(2, int(16 * scale)), max(3, int(128 * scale)) + 1, size=3)
        side = np.minimum(side, np.array(shape) - 2)
        lo = np.array([rng.integers(0, shape[k] - side[k]) for k in range(3)])
        hi = lo + side
        eps = rng.uniform(1.0, 10.0)
        kap = rng.uniform(0.0, 0.1)
        start = lo * pitch_mm
        stop = hi * pitch_mm
        if b in disp and dispersive:
            fp = rng.uniform(1e9, 10e9)
            tr = 1.0 / rng.uniform(1e8, 1e9)
            if b % 2:
                m = csx.AddLorentzMaterial(f"disp{b}", epsilon=eps, kappa=kap, eps_plasma_freq=[fp],
                                           eps_relax_time=[tr], eps_lor_pole_freq=[0.5 * fp])
            else:
                m = csx.AddLorentzMaterial(f"disp{b}", epsilon=eps, kappa=kap, eps_plasma_freq=[fp],
                                           eps_relax_time=[tr])
        else:
            m = csx.AddMaterial(f"blk{b}", epsilon=eps, kappa=kap)
        m.AddBox(start, stop, priority=b)
    for s in range(4):
        p = np.array([rng.integers(8, shape[k] - 8) for k in range(3)])
        d = int(rng.integers(0, 3))
        val = [0.0, 0.0, 0.0]
        val[d] = float(rng.choice([-1.0, 1.0]))
        stop = p.astype(float).copy()
        stop[d] += 1
        csx.AddExcitation(f"src{s}", 0, val).AddBox(p * pitch_mm, stop * pitch_mm, priority=1000)
        # a 3-edge voltage monitor through each source edge, sampled every step
        a = p.astype(float).copy()
        b = p.astype(float).copy()
        a[d] -= 1
        b[d] += 2
        csx.AddProbe(f"mon{s}", 0, interval=1).AddBox(a * pitch_mm, b * pitch_mm)
    op = Operator(csx, g, exc, bc=bc)
    return op.build(steps)


def mur_corners(n=(16, 14, 12), steps=600, seed=7, wall_source=True):
    """Mur on all six walls with the hooks' corner cases: dispersive blocks that reach five walls
    (their apply hooks run between the Mur post and apply hooks; the blocks meet on the wall
    edges), and (wall_source) a soft source on the x = 0 wall line, which switches that wall on
    only after the excitation (engine_ext_mur_abc.cpp:44-60).  An odd z count such as 33 puts
    the upper z wall's line and shift cells of some rows in neighbouring warps of the engine."""
    rng = np.random.default_rng(seed)
    lines = [np.cumsum(np.concatenate([[0.0], rng.uniform(0.6, 1.2, k - 1)])) for k in n]
    g = Grid(lines, unit=1e-3)
    gl = g.lines
    L = [l[-1] for l in gl]
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(6e9, 5e9)
    csx.AddMaterial("diel", epsilon=3.0, kappa=0.02).AddBox([0.3 * L[0], 0.3 * L[1], 0.3 * L[2]],
                                                            [0.7 * L[0], 0.6 * L[1], 0.7 * L[2]])
    csx.AddLorentzMaterial("drude_wall", epsilon=1.5, eps_plasma_freq=[5e9], eps_relax_time=[2e-9]).AddBox(
        [0.0, 0.0, 0.3 * L[2]], [0.4 * L[0], 0.5 * L[1], L[2]], priority=5)
    csx.AddLorentzMaterial("lor_wall", epsilon=2.0, eps_plasma_freq=[8e9], eps_relax_time=[1e-9],
                           eps_lor_pole_freq=[3e9]).AddBox([0.6 * L[0], 0.5 * L[1], 0.0], [L[0], L[1], 0.4 * L[2]],
                                                          priority=6)
    # y-directed source on the x = 0 line (tangential to that wall) and a z-directed one inside
    if wall_source:
        csx.AddExcitation("wall_src", 0, [0, 1.0, 0]).AddBox([gl[0][0], gl[1][5], gl[2][6]],
                                                             [gl[0][0], gl[1][6], gl[2][6]], priority=20)
    cx, cy, cz = (gl[k][n[k] // 2] for k in range(3))
    csx.AddExcitation("mid_src", 0, [0, 0, 1.0]).AddBox([cx, cy, cz], [cx, cy, gl[2][n[2] // 2 + 1]], priority=20)
    csx.AddProbe("wall_ut", 0, interval=1).AddBox([gl[0][0], gl[1][5], gl[2][6]], [gl[0][0], gl[1][6], gl[2][6]])
    op = Operator(csx, g, exc, bc=(2,) * 6)
    return op.build(steps)


# ------------------------------------------------------------------------------------------
def plane_wave(n=(28, 24, 26), steps=300, bc=(3,) * 6, pml=5, k_dir=(1.0, 0.0, 0.0), e_dir=(0.0, 0.0, 1.0),
               frequency=0.0, graded=False, scatterer=True, dispersive=False, box=None, sinus=False, seed=3):
    """Plane-wave (TFSF, exc_type 10) excitation of a total-field box, as the reference's
    RCS_Sphere tutorial sets it up (python/Tutorials/RCS_Sphere.py:61-71): a metal brick and a
    dielectric block inside the box, voltage probes inside and outside it.  ``box`` = (lo, hi)
    line indices per axis (default: 7 lines in from every wall); a lower index of 0 or an upper
    index of N-1 turns that face off, as in the reference."""
    rng = np.random.default_rng(seed)
    if graded:
        lines = [np.cumsum(np.concatenate([[0.0], rng.uniform(0.7, 1.3, k - 1)])) for k in n]
    else:
        lines = [_uniform(k) for k in n]
    g = Grid(lines, unit=1e-3)
    gl = g.lines
    csx = Structure()
    exc = Excitation()
    if sinus:
        exc.SetupSinusoidal(10e9)
    else:
        exc.SetupGaussianPulse(10e9, 8e9)
    if box is None:
        box = ([7, 7, 7], [k - 8 for k in n])
    lo, hi = box
    pw = csx.AddExcitation("plane_wave", 10, list(e_dir))
    pw.SetPropagationDir(list(k_dir))
    if frequency:
        pw.SetFrequency(frequency)
    pw.AddBox([gl[a][lo[a]] for a in range(3)], [gl[a][hi[a]] for a in range(3)])
    mid = [gl[a][(lo[a] + hi[a]) // 2] for a in range(3)]
    if scatterer:
        csx.AddMetal("brick").AddBox([mid[0] + 1.0, mid[1] - 2.0, mid[2] - 2.0], [mid[0] + 2.0, mid[1] + 2.0, mid[2] + 2.0],
                                     priority=10)
        csx.AddMaterial("diel", epsilon=4.0, kappa=0.05).AddBox([mid[0] - 4.0, mid[1] - 3.0, mid[2] - 3.0],
                                                               [mid[0] - 1.0, mid[1] + 1.0, mid[2] + 3.0])
    if dispersive:
        csx.AddLorentzMaterial("drude", epsilon=1.2, eps_plasma_freq=[8e9], eps_relax_time=[1e-9]).AddBox(
            [gl[0][lo[0] + 1], gl[1][lo[1] + 1], gl[2][lo[2] + 1]], [gl[0][lo[0] + 4], gl[1][hi[1] - 1], gl[2][lo[2] + 4]],
            priority=5)
    # probes: one z-line inside the total-field box, one in the scattered-field region
    zi = (lo[2] + hi[2]) // 2
    xi = lo[0] + 2
    yi = (lo[1] + hi[1]) // 2
    csx.AddProbe("ut_inside", 0, interval=1).AddBox([gl[0][xi], gl[1][yi], gl[2][zi]], [gl[0][xi], gl[1][yi], gl[2][zi + 1]])
    xo = max(lo[0] - 2, 1)
    csx.AddProbe("ut_outside", 0, interval=1).AddBox([gl[0][xo], gl[1][yi], gl[2][zi]], [gl[0][xo], gl[1][yi], gl[2][zi + 1]])
    op = Operator(csx, g, exc, bc=bc, pml_size=(pml,) * 6)
    return op.build(steps)


def lumped_rlc(n=(22, 20, 24), steps=600, bc=(2,) * 6, dispersive=False, seed=11):
    """Lumped RLC loads of every kind the reference's Operator_Ext_LumpedRLC builds, fed by a 50 Ohm
    lumped port: a series RLC, a series RL (C = 0: the capacitor is a short), a parallel RLC and
    a parallel L without C (the edge keeps its own capacitance, raised to the reference's minimum
    if it is too small), on a graded mesh with Mur walls (or the given boundaries).  Every element
    stays out of a 4-cell UPML: the UPML rewrites the coefficients of its cells, which a lumped
    element rewritten after it would break."""
    rng = np.random.default_rng(seed)
    lines = [np.cumsum(np.concatenate([[0.0], rng.uniform(0.8, 1.2, k - 1)])) for k in n]
    g = Grid(lines, unit=1e-3)
    gl = g.lines
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(5e9, 4e9)
    c = [k // 2 for k in n]

    def P(i, j, k):
        return [gl[0][i], gl[1][j], gl[2][k]]
    csx.AddLumpedElement("port", 2, R=50.0, caps=True).AddBox(P(c[0] - 4, c[1], c[2] - 1), P(c[0] - 4, c[1], c[2] + 1))
    csx.AddExcitation("port_exc", 0, [0, 0, -1.0]).AddBox(P(c[0] - 4, c[1], c[2] - 1), P(c[0] - 4, c[1], c[2] + 1))
    csx.AddLumpedElement("series_rlc", 2, R=10.0, L=2e-9, C=0.5e-12, LEtype=1, caps=True).AddBox(
        P(c[0] + 3, c[1], c[2] - 1), P(c[0] + 3, c[1], c[2] + 1))
    csx.AddLumpedElement("series_rl", 0, R=20.0, L=1e-9, LEtype=1, caps=False).AddBox(
        P(c[0] - 1, c[1] + 3, c[2] + 3), P(c[0] + 1, c[1] + 4, c[2] + 3))
    csx.AddLumpedElement("parallel_rlc", 1, R=100.0, C=0.2e-12, L=3e-9, LEtype=0, caps=True).AddBox(
        P(c[0], c[1] - 5, c[2] - 3), P(c[0], c[1] - 3, c[2] - 3))
    csx.AddLumpedElement("parallel_l", 2, L=2e-9, LEtype=0).AddBox(P(c[0] + 5, c[1] - 2, c[2]), P(c[0] + 5, c[1] - 2, c[2] + 1))
    if dispersive:
        csx.AddLorentzMaterial("drude", epsilon=1.5, eps_plasma_freq=[6e9], eps_relax_time=[1e-9]).AddBox(
            P(5, 5, 5), P(c[0] - 2, n[1] - 6, c[2]), priority=2)
    csx.AddProbe("u_port", 0, interval=1).AddBox(P(c[0] - 4, c[1], c[2] - 1), P(c[0] - 4, c[1], c[2] + 1))
    csx.AddProbe("u_series", 0, interval=1).AddBox(P(c[0] + 3, c[1], c[2] - 1), P(c[0] + 3, c[1], c[2] + 1))
    csx.AddProbe("i_series", 1, norm_dir=2, interval=1).AddBox(P(c[0] + 3, c[1], c[2]), P(c[0] + 3, c[1], c[2]))
    op = Operator(csx, g, exc, bc=bc, pml_size=(4,) * 6)
    return op.build(steps)


def lc_tank(L=1e-9, C=1e-12, steps=6000, n=20):
    """A parallel LC lumped element (LEtype 0, R open) on one z edge at the centre of a PEC box of
    n^3 lines at 0.5 mm, kicked by a soft source on the same edge.  After the pulse the node rings
    at 1/(2 pi sqrt(L C)) as long as C dominates the edge's own capacitance."""
    g = Grid([_uniform(n, 0.5) for _ in range(3)], unit=1e-3)
    gl = g.lines
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(4e9, 4e9)
    c = n // 2
    box = ([gl[0][c], gl[1][c], gl[2][c]], [gl[0][c], gl[1][c], gl[2][c + 1]])
    csx.AddLumpedElement("tank", 2, C=C, L=L, LEtype=0, caps=False).AddBox(*box)
    csx.AddExcitation("kick", 0, [0, 0, 1.0]).AddBox(*box)
    csx.AddProbe("u_tank", 0, interval=1).AddBox(*box)
    op = Operator(csx, g, exc, bc=(0,) * 6)
    return op.build(steps)


def td_dumps(n=(16, 14, 12), steps=120, bc=(2, 2, 3, 3, 0, 0), seed=5):
    """Time-domain field dumps (dump types 0/1) of every interpolation type on a small graded mesh
    with a dielectric block and a point source: E and H volumes with node interpolation, an E plane
    with cell interpolation, an H line without interpolation that starts and stops at given times,
    and a two-box E dump (files named <name>_0 and <name>_1)."""
    rng = np.random.default_rng(seed)
    lines = [np.cumsum(np.concatenate([[0.0], rng.uniform(0.7, 1.3, k - 1)])) for k in n]
    g = Grid(lines, unit=1e-3)
    gl = g.lines
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(8e9, 6e9)
    c = [k // 2 for k in n]
    csx.AddMaterial("diel", epsilon=3.0, kappa=0.01).AddBox([gl[0][2], gl[1][2], gl[2][2]], [gl[0][c[0]], gl[1][-4], gl[2][c[2]]])
    csx.AddExcitation("src", 0, [0, 0, 1.0]).AddBox([gl[0][c[0]], gl[1][c[1]], gl[2][c[2]]],
                                                   [gl[0][c[0]], gl[1][c[1]], gl[2][c[2] + 1]])
    csx.AddProbe("ut", 0, interval=1).AddBox([gl[0][c[0]], gl[1][c[1]], gl[2][c[2]]], [gl[0][c[0]], gl[1][c[1]], gl[2][c[2] + 1]])
    lo = [l[0] for l in gl]
    hi = [l[-1] for l in gl]
    csx.AddDump("Et_node", dump_type=0, dump_mode=1).AddBox(lo, hi)
    csx.AddDump("Ht_node", dump_type=1, dump_mode=1).AddBox(lo, hi)
    csx.AddDump("Et_cell", dump_type=0, dump_mode=2).AddBox([lo[0], lo[1], gl[2][c[2]]], [hi[0], hi[1], gl[2][c[2]]])
    dt_guess = 1.0 / (3e8 * np.sqrt(3) / 0.7e-3)     # about the mesh's timestep, for the window
    csx.AddDump("Ht_raw", dump_type=1, dump_mode=0, start_time=20 * dt_guess, stop_time=90 * dt_guess).AddBox(
        [gl[0][1], gl[1][c[1]], gl[2][c[2]]], [gl[0][-2], gl[1][c[1]], gl[2][c[2]]])
    two = csx.AddDump("Et_two", dump_type=0, dump_mode=1)
    two.AddBox([gl[0][1], gl[1][1], gl[2][1]], [gl[0][4], gl[1][3], gl[2][5]])
    two.AddBox([gl[0][c[0]], gl[1][c[1]], gl[2][0]], [gl[0][c[0]], gl[1][c[1]], gl[2][-1]])
    op = Operator(csx, g, exc, bc=bc, pml_size=(3,) * 6)
    return op.build(steps)


def conducting_sheet(n=(24, 20, 22), steps=400, bc=(2,) * 6, sigma=5.8e7, thickness=35e-6, pec=False, seed=9,
                     dispersive=False):
    """Conducting sheets (Operator_Ext_ConductingSheet): a z-normal sheet across most of the cross
    section between a point source and a probe, a small x-normal sheet, a three-dimensional box of
    the sheet material (PEC fallback) and a sheet reaching the boundary layer (PEC fallback there),
    on a graded mesh.  pec=True puts a metal plate where the main sheet is (for comparisons)."""
    rng = np.random.default_rng(seed)
    lines = [np.cumsum(np.concatenate([[0.0], rng.uniform(0.8, 1.2, k - 1)])) for k in n]
    g = Grid(lines, unit=1e-3)
    gl = g.lines
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(5e9, 4e9)
    c = [k // 2 for k in n]

    def P(i, j, k):
        return [gl[0][i], gl[1][j], gl[2][k]]
    if pec:
        csx.AddMetal("plate").AddBox(P(3, 3, c[2]), P(n[0] - 4, n[1] - 4, c[2]), priority=10)
    else:
        sheet = csx.AddConductingSheet("sheet", sigma, thickness)
        sheet.AddBox(P(3, 3, c[2]), P(n[0] - 4, n[1] - 4, c[2]), priority=10)
        sheet.AddBox(P(4, 4, 4), P(6, 7, 6), priority=10)                      # a volume: PEC fallback
        csx.AddConductingSheet("small", 1e5, 2e-6).AddBox(P(c[0] + 4, 3, 4), P(c[0] + 4, 8, 8), priority=11)
        csx.AddConductingSheet("edge", 3e6, 10e-6).AddBox(P(0, c[1], 2), P(5, c[1], 6), priority=11)
    if dispersive:
        csx.AddLorentzMaterial("drude", epsilon=1.5, eps_plasma_freq=[6e9], eps_relax_time=[1e-9]).AddBox(
            P(3, 3, c[2] + 2), P(9, 9, c[2] + 5), priority=2)
    csx.AddMaterial("diel", epsilon=2.5).AddBox(P(2, 2, c[2] - 4), P(n[0] - 3, n[1] - 3, c[2] - 1))
    csx.AddExcitation("src", 0, [1.0, 0, 0]).AddBox(P(c[0], c[1], c[2] - 3), P(c[0] + 1, c[1], c[2] - 3))
    csx.AddProbe("u_below", 0, interval=1).AddBox(P(c[0], c[1], c[2] - 2), P(c[0] + 1, c[1], c[2] - 2))
    csx.AddProbe("u_above", 0, interval=1).AddBox(P(c[0], c[1], c[2] + 3), P(c[0] + 1, c[1], c[2] + 3))
    op = Operator(csx, g, exc, bc=bc, pml_size=(4,) * 6)
    return op.build(steps)


def coax(steps=5000, length=1000.0, res=5.0):
    """The reference's coax test (TESTSUITE/combinedtests/Coax.m:24-90): a PEC coaxial line of
    inner radius 100 and outer radii 230/240 (drawing units, mm) on a 5 mm mesh, PEC on every wall
    but a PML_8 at the far end, a radially weighted soft excitation at z = 0 and, half way down,
    a voltage probe across the gap and a current probe around the inner conductor."""
    r_i, r_ai, r_aa = 100.0, 230.0, 240.0
    xs = np.arange(-2.5 * res - r_aa, r_aa + 2.5 * res + 1e-9, res)
    nz = int(round(length / res)) + 1
    zs = np.linspace(0.0, length, nz)
    g = Grid([xs, xs.copy(), zs], unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(0.0, 1e9)
    pec = csx.AddMetal("PEC")
    pec.AddCylinder([0, 0, 0], [0, 0, length], r_i, priority=1)
    pec.AddCylindricalShell([0, 0, 0], [0, 0, length], 0.5 * (r_aa + r_ai), r_aa - r_ai, priority=0)
    weight = (lambda x, y, z: x / (x * x + y * y), lambda x, y, z: y / (x * x + y * y), lambda x, y, z: 0.0)
    csx.AddExcitation("excite", 0, [1, 1, 0], weight=weight).AddCylindricalShell(
        [0, 0, 0], [0, 0, res / 2], 0.5 * (r_i + r_ai), r_ai - r_i)
    csx.AddProbe("ut1", 0, interval=1).AddBox([r_i, 0, length / 2], [r_ai, 0, length / 2])
    mid = r_i + 3 * res
    csx.AddProbe("it1", 1, interval=1).AddBox([-mid, -mid, length / 2], [mid, mid, length / 2])
    op = Operator(csx, g, exc, bc=(0, 0, 0, 0, 0, 3), pml_size=(8,) * 6)
    return op.build(steps)


def fieldprobes(half=8, steps=600, freqs=(5e8,), interval=0):
    """The reference's field probe test (TESTSUITE/probes/fieldprobes.m:36-116) at a smaller
    extent: an infinitesimal dipole (hard Ez over lambda/50, lambda at 1 GHz, drawing unit 1 um)
    on a uniform lambda/100 mesh of +-half dipole lengths, Mur on every wall, a Gaussian pulse
    (f0 0, fc 1 GHz), OverSampling 10; six E and six H time-domain dumps without interpolation on
    the faces of the cube +-2.25 dipole lengths, and E (type 2) and H (type 3) point probes at the
    face centres (the given frequencies add a DFT to the probes; ``interval`` overrides the
    probes' sampling interval)."""
    c0 = 299792458.0
    unit = 1e-6
    dl = c0 / 1e9 / unit / 50
    m = np.arange(-2 * half, 2 * half + 1) * (dl / 2)
    g = Grid([m, m.copy(), m.copy()], unit=unit)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(0.0, 1e9)
    csx.AddExcitation("infDipole", 1, [0, 0, 1.0]).AddBox([0, 0, -dl / 2], [0, 0, dl / 2])
    s1 = [-4.5 * dl / 2] * 3
    s2 = [4.5 * dl / 2] * 3
    faces = {"xn": (s1, [s1[0], s2[1], s2[2]]), "xp": ([s2[0], s1[1], s1[2]], s2),
             "yn": (s1, [s2[0], s1[1], s2[2]]), "yp": ([s1[0], s2[1], s1[2]], s2),
             "zn": (s1, [s2[0], s2[1], s1[2]]), "zp": ([s1[0], s1[1], s2[2]], s2)}
    for f, (a, b) in faces.items():
        csx.AddDump("Et_" + f, dump_type=0, dump_mode=0).AddBox(a, b)
        csx.AddDump("Ht_" + f, dump_type=1, dump_mode=0).AddBox(a, b)
    coords = [[s1[0], 0, 0], [s2[0], 0, 0], [0, s1[1], 0], [0, s2[1], 0], [0, 0, s1[2]], [0, 0, s2[2]]]
    for k, c in enumerate(coords):
        csx.AddProbe("et%d" % (k + 1), 2, frequency=freqs, interval=interval).AddBox(c, c)
    for k, c in enumerate(coords):
        csx.AddProbe("ht%d" % (k + 1), 3, frequency=freqs, interval=interval).AddBox(c, c)
    op = Operator(csx, g, exc, bc=(2,) * 6, over_sampling=10)
    data = op.build(steps)
    data.fieldprobe_coords = coords
    return data


def coax_cyl(steps=5000, length=1000.0, res=10.0, n_alpha=71, pml=False, load=None, rlc=False, shield=None):
    """``coax_cyl_operator`` built for ``steps`` timesteps."""
    return coax_cyl_operator(length, res, n_alpha, pml, load, rlc, shield).build(steps)


def coax_cyl_operator(length=1000.0, res=10.0, n_alpha=71, pml=False, load=None, rlc=False, shield=None):
    """The reference's coax example in cylindrical coordinates
    (matlab/examples/waveguide/Coax_CylinderCoords.m:25-123): rho from the inner radius 100 to the
    outer radius 230 on a 10 mm mesh, 71 alpha lines over 2*pi (a closed mesh), z over 1000 mm; PEC
    on every wall but Mur at the far end; a radial soft excitation weighted 1/rho on the z = 0 plane
    (f0 = fc = 0.5 GHz); half way down, a voltage probe across the gap at alpha = 0 and a current
    loop around the inner conductor on the dual mesh (one full turn of alpha).  ``pml``: a PML_8 at
    the far end instead of Mur (the example's use_pml option).  ``load``: a radial lumped resistor
    of that many ohms across the gap one line in front of the far end (one parallel RC element, or
    with ``rlc`` a parallel R || 1 uH element of the lumped RLC extension), so the line sees it
    in parallel with the matched remainder.  ``shield``: "sheet" (a 35 um copper conducting sheet)
    or "metal" (PEC) across the gap a quarter of the way down, between source and probes."""
    from .operator_cyl import OperatorCylinder
    r_i, r_a = 100.0, 230.0
    rs = np.arange(r_i, r_a + 0.5 * res, res)
    al = np.linspace(0.0, 2 * np.pi, n_alpha)
    zs = np.arange(0.0, length + 0.5 * res, res)
    g = Grid([rs, al, zs], unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(0.5e9, 0.5e9)
    weight = (lambda r, a, z: 1.0 / r, lambda r, a, z: 0.0, lambda r, a, z: 0.0)
    csx.AddExcitation("excite", 0, [1.0, 0, 0], weight=weight).AddBox([r_i, al[0], 0.0], [r_a, al[-1], 0.0])
    zm = zs[len(zs) // 2]
    csx.AddProbe("ut1", 0, interval=1).AddBox([r_i, 0.0, zm], [r_a, 0.0, zm])
    mid = 0.5 * (r_i + r_a)
    a1 = al[1]
    # the loop starts below the mesh (no inner side) and runs over dual alpha lines 0 .. N-2
    csx.AddProbe("it1", 1, norm_dir=2, interval=1).AddBox([0.0, 0.5 * a1, zm], [mid, 2 * np.pi + 0.5 * a1, zm])
    if shield is not None:
        zq = zs[len(zs) // 4]
        box = ([r_i, al[0], zq], [r_a, al[-1], zq])
        if shield == "sheet":
            csx.AddConductingSheet("shield", conductivity=5.8e7, thickness=35e-6).AddBox(*box)
        else:
            csx.AddMetal("shield").AddBox(*box)
    if load is not None:
        # up to the last distinct angle: snapping folds alpha = 2*pi back to 0 on a closed mesh
        # (SnapToMeshLine + FitToAlphaRange), which would leave a single radial edge chain
        # rlc: a parallel R || 1 uH element, which the lumped RLC extension builds
        csx.AddLumpedElement("load", ny=0, R=float(load), caps=False, L=1e-6 if rlc else float("nan")).AddBox(
            [r_i, al[0], zs[-2]], [r_a, al[-2], zs[-2]])
    far = 3 if pml else 2
    return OperatorCylinder(csx, g, exc, bc=(0, 0, 0, 0, 0, far), pml_size=(8,) * 6)


def cavity_cyl(steps=20000, radius=50.0, height=20.0, res=2.5, n_alpha=37, probe_r=0.0, dispersive=False,
               field_probes=False, fd_dumps=False):
    """A pillbox cavity in cylindrical coordinates with rho = 0 on the mesh: radius 50 mm, height
    20 mm, PEC walls, a 2.5 mm rho/z mesh and 10 degree alpha steps (a closed mesh), a soft Ez
    point source off the axis (f0 3 GHz, fc 2 GHz) and an Ez voltage probe at ``probe_r`` (on the
    axis by default, where the TM010 field is largest and the axis hook computes it).
    ``dispersive``: a Drude rod on the axis and a Lorentz sector across the alpha seam.
    ``field_probes``: E and H point probes off the axis (probe types 2 and 3), sampled every step.
    ``fd_dumps``: E and H frequency-domain dumps without interpolation at 2.3 GHz over a box
    around the field probes' node."""
    from .operator_cyl import OperatorCylinder
    rs = np.arange(0.0, radius + 0.5 * res, res)
    al = np.linspace(0.0, 2 * np.pi, n_alpha)
    zs = np.arange(0.0, height + 0.5 * res, res)
    g = Grid([rs, al, zs], unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(3e9, 2e9)
    k = len(zs) // 2
    rs_src = rs[len(rs) // 3]
    csx.AddExcitation("src", 0, [0, 0, 1.0]).AddBox([rs_src, al[3], zs[k]], [rs_src, al[3], zs[k + 1]])
    csx.AddProbe("uz", 0, interval=1).AddBox([probe_r, 0.0, zs[1]], [probe_r, 0.0, zs[-2]])
    if field_probes:
        pt = [0.4 * radius, al[5], zs[k]]
        csx.AddProbe("et", 2, interval=1, frequency=[2.3e9]).AddBox(pt, pt)
        csx.AddProbe("ht", 3, interval=1, frequency=[2.3e9]).AddBox(pt, pt)
    if fd_dumps:
        lo, hi = [0.3 * radius, al[3], zs[k - 1]], [0.5 * radius, al[7], zs[k + 1]]
        csx.AddDump("Ef", dump_type=10, dump_mode=0, frequency=[2.3e9]).AddBox(lo, hi)
        csx.AddDump("Hf", dump_type=11, dump_mode=0, frequency=[2.3e9]).AddBox(lo, hi)
    if dispersive:
        csx.AddLorentzMaterial("drude", epsilon=1.5, eps_plasma_freq=[4e9], eps_relax_time=[1e-9]).AddBox(
            [0.0, 0.0, zs[2]], [3 * res, 2 * np.pi, zs[-3]])
        csx.AddLorentzMaterial("lor", epsilon=2.0, eps_plasma_freq=[6e9], eps_relax_time=[2e-9],
                               eps_lor_pole_freq=[3e9]).AddBox([0.5 * radius, al[-4], zs[1]], [0.8 * radius, 2 * np.pi, zs[-2]])
        csx.AddLorentzMaterial("lor2", epsilon=2.0, eps_plasma_freq=[6e9], eps_relax_time=[2e-9],
                               eps_lor_pole_freq=[3e9]).AddBox([0.5 * radius, 0.0, zs[1]], [0.8 * radius, al[3], zs[-2]])
    op = OperatorCylinder(csx, g, exc, bc=(0,) * 6)
    return op.build(steps)


def sector_cyl(steps=1500, alpha_bc=3, pml=8, rho_bc=0):
    """An open quarter-circle sector in cylindrical coordinates: rho 20-60 mm (2 mm), alpha over
    pi/2 in 61 lines, z 0-16 mm between PEC plates, ``rho_bc`` on both rho walls (PEC: the alpha
    walls are the only way out) and ``alpha_bc`` (3 = a UPML of ``pml`` cells) on both alpha walls;
    a soft Ez source in the middle of the sector (f0 8 GHz, fc 3 GHz: above the 3.75 GHz cutoff of
    the curved guide between the rho walls) and an Ez probe near one alpha wall."""
    from .operator_cyl import OperatorCylinder
    rs = np.arange(20.0, 60.0 + 1e-9, 2.0)
    al = np.linspace(0.0, 0.5 * np.pi, 61)
    zs = np.arange(0.0, 16.0 + 1e-9, 2.0)
    g = Grid([rs, al, zs], unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(8e9, 3e9)
    csx.AddExcitation("src", 0, [0, 0, 1.0]).AddBox([rs[10], al[30], zs[4]], [rs[10], al[30], zs[5]])
    csx.AddProbe("uz", 0, interval=1).AddBox([rs[10], al[12], zs[4]], [rs[10], al[12], zs[5]])
    op = OperatorCylinder(csx, g, exc, bc=(rho_bc, rho_bc, alpha_bc, alpha_bc, 0, 0), pml_size=(pml,) * 6)
    return op.build(steps)


def patch(shape=(160, 160, 80), steps=20000, with_nf2ff=True):
    """Microstrip patch antenna on a graded mesh with UPML, lumped port and NF2FF box."""
    nx, ny, nz = shape
    sub_t = 1.524
    patch_w, patch_l = 32.0, 40.0
    sub_w = 60.0
    feed = -6.0
    xl = graded_lines(nx, -sub_w / 2, sub_w / 2, 0.5 * 160 / max(nx, 40) if nx < 160 else 0.5, 2.0, 1.3,
                      must=(feed, -patch_w / 2, patch_w / 2))
    yl = graded_lines(ny, -sub_w / 2, sub_w / 2, 0.5 * 160 / max(ny, 40) if ny < 160 else 0.5, 2.0, 1.3,
                      must=(0.0, -patch_l / 2, patch_l / 2))
    zfine = np.linspace(0.0, sub_t, 5)
    zl = graded_lines(nz, 0.0, sub_t, sub_t / 4, 2.0, 1.35, must=tuple(zfine))
    g = Grid([xl, yl, zl], unit=1e-3)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(2e9, 1.5e9)
    csx.AddMaterial("substrate", epsilon=3.38, kappa=1e-3).AddBox([-sub_w / 2, -sub_w / 2, 0], [sub_w / 2, sub_w / 2, sub_t])
    csx.AddMetal("gnd").AddBox([-sub_w / 2, -sub_w / 2, 0], [sub_w / 2, sub_w / 2, 0], priority=10)
    csx.AddMetal("patch").AddBox([-patch_w / 2, -patch_l / 2, sub_t], [patch_w / 2, patch_l / 2, sub_t], priority=10)
    # 50 Ohm lumped port from ground to patch (python/openEMS/ports.py:155-209)
    start, stop = np.array([feed, 0, 0]), np.array([feed, 0, sub_t])
    csx.AddLumpedElement("port_resist", ny=2, R=50.0, caps=True).AddBox(start, stop, priority=5)
    csx.AddExcitation("port_excite", 0, [0, 0, -1.0]).AddBox(start, stop, priority=5)
    csx.AddProbe("port_ut1", 0, weight=-1.0, interval=1, frequency=[1.5e9, 2e9, 2.5e9]).AddBox(start, stop)
    zm = 0.5 * sub_t
    csx.AddProbe("port_it1", 1, weight=1.0, norm_dir=2, interval=1, frequency=[1.5e9, 2e9, 2.5e9]).AddBox(
        [feed, 0, zm], [feed, 0, zm])
    if with_nf2ff:
        k = 11  # inside the 8-cell UPML
        lo = [xl[k], yl[k], zl[k]]
        hi = [xl[-k - 1], yl[-k - 1], zl[-k - 1]]
        for dt, name in ((10, "nf2ff_E"), (11, "nf2ff_H")):
            d = csx.AddDump(name, dump_type=dt, dump_mode=1, frequency=[1.5e9, 2e9, 2.5e9])
            for ax in range(3):
                for side in (lo, hi):
                    a = list(lo)
                    b = list(hi)
                    a[ax] = b[ax] = side[ax]
                    d.AddBox(a, b)
    op = Operator(csx, g, exc, bc=(3,) * 6, pml_size=(8,) * 6)
    return op.build(steps)


# ------------------------------------------------------------------------------------------
def cavity(steps=4000):
    """The reference's resonance-test cavity (TESTSUITE/combinedtests/cavity.m:46-111): a PEC box
    a=5 cm, b=2 cm, d=6 cm on 26x11x32 lines, Gaussian f0=fc=4.5 GHz, soft E source on the three
    edges from the 2/3 point, Ex/Ey/Ez voltage probes."""
    a, b, d = 5e-2, 2e-2, 6e-2
    mx = np.linspace(0, a, 26)
    my = np.linspace(0, b, 11)
    mz = np.linspace(0, d, 32)
    g = Grid([mx, my, mz], unit=1.0)
    csx = Structure()
    exc = Excitation()
    exc.SetupGaussianPulse(4.5e9, 4.5e9)
    i = [int(np.floor(len(m) * 2 / 3)) - 1 for m in (mx, my, mz)]
    p1 = [mx[i[0]], my[i[1]], mz[i[2]]]
    # the reference's curve from p1 to p1+one cell in every direction walks one edge per axis
    csx.AddExcitation("excite_x", 0, [1, 0, 0]).AddBox(p1, [mx[i[0] + 1], my[i[1]], mz[i[2]]])
    csx.AddExcitation("excite_y", 0, [0, 1, 0]).AddBox([mx[i[0] + 1], my[i[1]], mz[i[2]]], [mx[i[0] + 1], my[i[1] + 1], mz[i[2]]])
    csx.AddExcitation("excite_z", 0, [0, 0, 1]).AddBox([mx[i[0] + 1], my[i[1] + 1], mz[i[2]]], [mx[i[0] + 1], my[i[1] + 1], mz[i[2] + 1]])
    f = lambda m, frac: int(np.floor(len(m) * frac)) - 1  # noqa: E731  (MATLAB end*frac, 1-based)
    csx.AddProbe("ut1x", 0, interval=1).AddBox([mx[f(mx, .25)], my[f(my, .5)], mz[f(mz, .2)]],
                                              [mx[f(mx, .25) + 1], my[f(my, .5)], mz[f(mz, .2)]])
    csx.AddProbe("ut1y", 0, interval=1).AddBox([mx[f(mx, .25)], my[f(my, .5)], mz[f(mz, .2)]],
                                              [mx[f(mx, .25)], my[f(my, .5) + 1], mz[f(mz, .2)]])
    csx.AddProbe("ut1z", 0, interval=1).AddBox([mx[f(mx, .5)], my[f(my, .5)], mz[f(mz, .2)]],
                                              [mx[f(mx, .5)], my[f(my, .5)], mz[f(mz, .2) + 1]])
    op = Operator(csx, g, exc, bc=(0,) * 6)
    return op.build(steps)


# ------------------------------------------------------------------------------------------
def batch_instance(seed, size_range=(48, 160), pitch_range=(0.5, 2.0), steps_range=(4000, 12000), pml=8):
    """One simulation of the batched form: lines U[size_range]^3 at a uniform pitch
    U[pitch_range] mm, UPML on all sides, one dielectric block (eps_r U[2,12]), a 50 Ohm lumped
    port along z at the centre with a Gaussian excitation (f0 U[1,5] GHz, fc = f0/2), port U/I
    probes every step.  Returns (OperatorData, steps)."""
    rng = np.random.default_rng(seed)
    n = [int(rng.integers(size_range[0], size_range[1] + 1)) for _ in range(3)]
    pitch = float(rng.uniform(*pitch_range))
    steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
    g = Grid([_uniform(k, pitch) for k in n], unit=1e-3)
    csx = Structure()
    exc = Excitation()
    f0 = float(rng.uniform(1e9, 5e9))
    exc.SetupGaussianPulse(f0, f0 / 2)
    lo_i = [pml + 2 + int(rng.integers(0, max(1, k // 4))) for k in n]
    hi_i = [max(lo_i[a] + 2, n[a] - pml - 3 - int(rng.integers(0, max(1, n[a] // 4)))) for a in range(3)]
    csx.AddMaterial("block", epsilon=float(rng.uniform(2.0, 12.0))).AddBox(
        [lo_i[a] * pitch for a in range(3)], [hi_i[a] * pitch for a in range(3)])
    c = [k // 2 for k in n]
    z0, z1 = (c[2] - 1) * pitch, (c[2] + 1) * pitch
    px, py = c[0] * pitch, c[1] * pitch
    csx.AddLumpedElement("port_R", ny=2, R=50.0, caps=True).AddBox([px, py, z0], [px, py, z1], priority=10)
    csx.AddExcitation("port_exc", 0, [0, 0, -1.0]).AddBox([px, py, z0], [px, py, z1], priority=10)
    csx.AddProbe("port_ut", 0, weight=-1.0, interval=1).AddBox([px, py, z0], [px, py, z1])
    zm = 0.5 * (z0 + z1)
    csx.AddProbe("port_it", 1, weight=1.0, norm_dir=2, interval=1).AddBox([px, py, zm], [px, py, zm])
    op = Operator(csx, g, exc, bc=(3,) * 6, pml_size=(pml,) * 6)
    return op.build(steps), steps


# ------------------------------------------------------------------------------------------
class DesignCase:
    """The differentiable form: a uniform mesh with UPML on all sides, a box of per-cell
    eps_r / kappa (the design region) and two 50 Ohm lumped ports along z, each about ``gap``
    cells (Euclidean, diagonally in x-y) from the nearest design cell.  The input port carries
    a Gaussian pulse; the output port has U/I probes sampled every step.

    ``build(eps, kappa, fdtd_float)`` makes the operator for one design at a fixed timestep
    (just below the one of the initial design), so every design of an optimisation or a finite-difference
    stencil runs with the same dt and excitation signal."""

    def __init__(self, lines=(200, 200, 100), pitch_mm=0.5, design=(64, 64, 16), gap=60, steps=8000, pml=8,
                 freqs=(4e9, 5e9, 6e9), f0=5e9, fc=2e9, seed=0, eps_range=(1.0, 6.0), dt=None):
        self.lines = tuple(int(v) for v in lines)
        self.pitch = float(pitch_mm)
        self.design = tuple(int(v) for v in design)
        self.steps = int(steps)
        self.pml = int(pml)
        self.freqs = tuple(float(f) for f in freqs)
        self.f0, self.fc = float(f0), float(fc)
        cells = [n - 1 for n in self.lines]
        self.c0 = [(cells[a] - self.design[a]) // 2 for a in range(3)]     # first design cell
        off = int(np.ceil(gap / np.sqrt(2.0)))
        zc = self.c0[2] + self.design[2] // 2
        self.port_in = (self.c0[0] - off, self.c0[1] - off, zc)
        self.port_out = (self.c0[0] + self.design[0] + off, self.c0[1] + self.design[1] + off, zc)
        for p in (self.port_in, self.port_out):
            for a in range(2):
                if not (pml + 3 <= p[a] <= self.lines[a] - pml - 4):
                    raise ValueError(f"DesignCase: port {p} is too close to the UPML")
        if not (pml + 2 <= zc - 1 and zc + 1 <= self.lines[2] - pml - 3):
            raise ValueError("DesignCase: ports too close to the z UPML")
        for a in range(3):
            if self.c0[a] < pml + 1 or self.c0[a] + self.design[a] > cells[a] - pml - 1:
                raise ValueError("DesignCase: design region overlaps the UPML")
        rng = np.random.default_rng(seed)
        self.eps0 = rng.uniform(eps_range[0], eps_range[1], self.design)
        self.kappa0 = np.zeros(self.design)
        # fixed timestep: 0.995 x the Var3 timestep of the initial design, so that designs a
        # little below it (finite-difference stencils at eps_r near 1) stay within the bound
        self.dt = None
        self.dt = float(dt) if dt else 0.995 * self.build(self.eps0, self.kappa0)[1].dt

    @property
    def box_nodes(self):
        """Mesh nodes whose edges touch the design cells: [start, stop) per axis."""
        return [self.c0[a] for a in range(3)], [self.c0[a] + self.design[a] + 1 for a in range(3)]

    def build(self, eps, kappa=None, fdtd_float=np.float32):
        """(Operator, OperatorData) for one design."""
        p = self.pitch
        g = Grid([_uniform(k, p) for k in self.lines], unit=1e-3)
        csx = Structure()
        exc = Excitation()
        exc.SetupGaussianPulse(self.f0, self.fc)
        lo = [self.c0[a] * p for a in range(3)]
        hi = [(self.c0[a] + self.design[a]) * p for a in range(3)]
        kap = self.kappa0 if kappa is None else kappa
        csx.AddVoxelMaterial("design", lo, hi, np.asarray(eps, np.float64), kappa=np.asarray(kap, np.float64))
        for name, (x, y, z), src in (("in", self.port_in, True), ("out", self.port_out, False)):
            z0, z1 = (z - 1) * p, (z + 1) * p
            csx.AddLumpedElement(f"port_{name}_R", ny=2, R=50.0, caps=True).AddBox([x * p, y * p, z0], [x * p, y * p, z1],
                                                                                 priority=10)
            if src:
                csx.AddExcitation(f"port_{name}_exc", 0, [0, 0, -1.0]).AddBox([x * p, y * p, z0], [x * p, y * p, z1],
                                                                             priority=10)
            else:
                csx.AddProbe(f"port_{name}_ut", 0, weight=-1.0, interval=1).AddBox([x * p, y * p, z0],
                                                                                  [x * p, y * p, z1])
                zm = 0.5 * (z0 + z1)
                csx.AddProbe(f"port_{name}_it", 1, weight=1.0, norm_dir=2, interval=1).AddBox([x * p, y * p, zm],
                                                                                             [x * p, y * p, zm])
        op = Operator(csx, g, exc, bc=(3,) * 6, pml_size=(self.pml,) * 6, timestep=self.dt or 0.0,
                      fdtd_float=fdtd_float)
        return op, op.build(self.steps)
