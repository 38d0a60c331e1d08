"""Host side of the differentiable form (no GPU): the objective's derivative, the material chain
eps_r/kappa -> C/G -> vv/vi, voxel materials, and the array restatement of the timestep used as
the FP64 / autograd checker, pinned bit-exact against the C oracle in float32."""
import numpy as np
import pytest

from openems_gb300.adjoint import material_chain, port_power
from openems_gb300.configs import DesignCase
from openems_gb300.operator import Grid, Operator, Structure
from openems_gb300.excitation import Excitation

from helpers import bits_equal


def tiny_case(**kw):
    """26x26x20 lines at 0.5 mm, UPML 4, 4x4x2 design cells, fast pulse (f0 20 GHz)."""
    args = dict(lines=(26, 26, 20), design=(4, 4, 2), gap=4, steps=200, pml=4, freqs=(15e9, 20e9, 25e9),
                f0=20e9, fc=15e9, seed=3)
    args.update(kw)
    return DesignCase(**args)


def test_port_power_derivative_matches_finite_differences():
    rng = np.random.default_rng(0)
    n = 64
    u, i = rng.standard_normal(n), rng.standard_normal(n)
    dt, freqs = 1e-12, (4e9, 5e9, 6e9)
    J, su, si = port_power(u, i, dt, freqs)
    h = 1e-6
    for k in (0, 7, 31, 63):
        e = np.zeros(n)
        e[k] = h
        fd_u = (port_power(u + e, i, dt, freqs)[0] - port_power(u - e, i, dt, freqs)[0]) / (2 * h)
        fd_i = (port_power(u, i + e, dt, freqs)[0] - port_power(u, i - e, dt, freqs)[0]) / (2 * h)
        assert abs(fd_u - su[k]) <= 1e-7 * max(abs(su).max(), 1e-300)
        assert abs(fd_i - si[k]) <= 1e-7 * max(abs(si).max(), 1e-300)


def test_voxel_material_equals_plain_material():
    def build(vox):
        g = Grid([np.arange(n) * 0.5 for n in (22, 20, 18)], unit=1e-3)
        csx, exc = Structure(), Excitation()
        exc.SetupGaussianPulse(5e9, 2e9)
        lo, hi = [4.0, 3.5, 3.0], [7.0, 6.5, 5.0]
        if vox:
            csx.AddVoxelMaterial("d", lo, hi, np.full((6, 6, 4), 3.0), kappa=np.full((6, 6, 4), 0.02))
        else:
            csx.AddMaterial("d", epsilon=3.0, kappa=0.02).AddBox(lo, hi)
        csx.AddExcitation("e", 0, [0, 0, 1.0]).AddBox([2.5, 2.5, 6.0], [2.5, 2.5, 6.5])
        return Operator(csx, g, exc, bc=(3,) * 6, pml_size=(3,) * 6).build(50)
    a, b = build(False), build(True)
    for k in ("vv", "vi", "ii", "iv"):
        assert bits_equal(getattr(a, k), getattr(b, k)), k


def test_voxel_shape_is_checked():
    g = Grid([np.arange(n) * 0.5 for n in (12, 12, 12)], unit=1e-3)
    csx = Structure()
    csx.AddVoxelMaterial("d", [1.0, 1.0, 1.0], [3.0, 3.0, 2.0], np.ones((3, 3, 3)))
    with pytest.raises(ValueError, match="mesh cells"):
        Operator(csx, g, Excitation())


def test_material_chain_matches_fp64_operator_differences():
    """d/d eps_c and d/d kappa_c of L = sum(g_vv * vv + g_vi * vi) over the design box, from the
    analytic chain and from central differences of FP64 operator builds."""
    case = tiny_case(steps=10)
    rng = np.random.default_rng(5)
    kap0 = rng.uniform(0.0, 0.5, case.design)
    bs, be = case.box_nodes
    box = tuple(slice(s, e) for s, e in zip(bs, be))
    shape = (3,) + tuple(e - s for s, e in zip(bs, be))
    g_vv, g_vi = rng.standard_normal(shape), rng.standard_normal(shape)

    def L(eps, kap):
        op, d = case.build(eps, kap, fdtd_float=np.float64)
        return float(np.sum(g_vv * d.vv[(slice(None),) + box]) + np.sum(g_vi * d.vi[(slice(None),) + box]))

    op, _ = case.build(case.eps0, kap0, fdtd_float=np.float64)
    ge, gk = material_chain(op, case.c0, case.design, g_vv, g_vi)
    cells = [(0, 0, 0), (3, 2, 1), (1, 3, 0), (2, 1, 1)]
    for c in cells:
        he, hk = 1e-4, 1e-3
        e = np.zeros(case.design)
        e[c] = 1.0
        fd_e = (L(case.eps0 + he * e, kap0) - L(case.eps0 - he * e, kap0)) / (2 * he)
        fd_k = (L(case.eps0, kap0 + hk * e) - L(case.eps0, kap0 - hk * e)) / (2 * hk)
        assert abs(ge[c] - fd_e) <= 1e-6 * abs(fd_e), (c, ge[c], fd_e)
        assert abs(gk[c] - fd_k) <= 1e-5 * abs(fd_k), (c, gk[c], fd_k)


def test_design_case_geometry_is_validated():
    with pytest.raises(ValueError):
        DesignCase(lines=(26, 26, 20), design=(4, 4, 2), gap=12, steps=10, pml=4)


def test_array_restatement_matches_c_oracle_bitwise():
    from oracle.fdtd_ref import RefEngine
    from oracle.oracle import OracleEngine
    case = tiny_case(steps=120)
    _, data = case.build(case.eps0)
    o = OracleEngine(data, case.steps)
    o.IterateTS(case.steps)
    r = RefEngine(data, dtype=np.float32).run(case.steps)
    for k, pid in enumerate(o.vprobe_ids + o.iprobe_ids):
        a = o.probe_series(pid)
        assert bits_equal(a, r.probe_series(k)[:len(a)])
    assert bits_equal(o.read_field(0).reshape(r.V.shape), r.V)
    assert bits_equal(o.read_field(1).reshape(r.I.shape), r.I)
