"""Differentiable form on the GPU: the adjoint kernels behind oems_cuda_adjoint_* and the
torch.autograd.Function, against
  * the forward series of the array restatement in float32 (bit-exact),
  * a reverse-mode reference (torch autograd through the float64 restatement) for dJ/dvv, dJ/dvi,
  * FP64 central finite differences (h = 1e-3) of dJ/d eps_r on 16 random design cells and of
    dJ/d kappa on 4, with the relative error bound 1e-3 written below,
  * itself with another checkpoint interval (bit-exact: recomputation is deterministic)."""
import multiprocessing as mp
import os

import numpy as np
import pytest

from helpers import bits_equal, rel_l2
from test_adjoint_host import tiny_case

pytestmark = pytest.mark.gpu

FD_TOL = 1e-3          # relative L2 error of the adjoint gradient vs FP64 central differences
AUTOGRAD_TOL = 1e-4    # relative L2 error of the float32 adjoint vs float64 reverse mode


def fd_case_kwargs():
    """44x44x34 lines at 0.5 mm, UPML 8, 8x8x4 design cells, ports 8 cells from the region,
    Gaussian f0 5 GHz / fc 2 GHz, objective at 4/5/6 GHz over 700 steps."""
    return dict(lines=(44, 44, 34), design=(8, 8, 4), gap=8, steps=700, pml=8, seed=11)


@pytest.fixture(scope="module")
def fd_pool():
    # spawn: a forked child of a process that has touched CUDA can hang
    ctx = mp.get_context("spawn")
    pool = ctx.Pool(max(1, min(16, os.cpu_count() or 1)))
    yield pool
    pool.close()
    pool.join()


def test_adjoint_forward_series_bit_exact(cuda_lib):
    from oracle.fdtd_ref import RefEngine
    from openems_gb300.adjoint import AdjointRun
    case = tiny_case()
    run = AdjointRun(case, case.eps0, checkpoint_every=64)
    try:
        r = RefEngine(run.data, dtype=np.float32).run(case.steps)
        assert bits_equal(run.u, r.probe_series(0))
        assert bits_equal(run.i, r.probe_series(1))
    finally:
        run.close()


def test_edge_gradient_matches_reverse_mode_reference(cuda_lib):
    from oracle.fdtd_ref import reference_edge_gradient
    from openems_gb300.adjoint import AdjointRun
    case = tiny_case()
    run = AdjointRun(case, case.eps0, checkpoint_every=64)
    try:
        gvv, gvi = run.edge_gradient()
        J_ref, rvv, rvi = reference_edge_gradient(run.data, case.steps, *case.box_nodes, case.freqs)
        assert abs(run.J - J_ref) <= 1e-4 * abs(J_ref)
        e_vv, e_vi = rel_l2(gvv, rvv), rel_l2(gvi, rvi)
        print(f"edge gradient rel L2 vs float64 reverse mode: vv {e_vv:.2e} vi {e_vi:.2e}")
        assert e_vv <= AUTOGRAD_TOL and e_vi <= AUTOGRAD_TOL
        # the engine is back at its forward end state
        assert run.eng.GetNumberOfTimesteps() == case.steps
    finally:
        run.close()


def test_checkpoint_interval_does_not_change_the_gradient(cuda_lib):
    """K = 0 records the factors during the forward run; K > 0 recomputes them from checkpoints.
    Both give the factors of the same bit-exact trajectory, so the gradients are identical."""
    from openems_gb300.adjoint import AdjointRun
    case = tiny_case()
    out = []
    for K in (0, 7, 64, 1000):
        run = AdjointRun(case, case.eps0, checkpoint_every=K)
        try:
            out.append(run.edge_gradient())
        finally:
            run.close()
    for gvv, gvi in out[1:]:
        assert bits_equal(gvv, out[0][0]) and bits_equal(gvi, out[0][1])


def test_gradient_matches_fp64_central_differences(cuda_lib, fd_pool):
    from openems_gb300.adjoint import AdjointRun
    from openems_gb300.configs import DesignCase
    from oracle.fdtd_ref import fp64_port_power
    kw = fd_case_kwargs()
    case = DesignCase(**kw)
    kw["dt"] = case.dt
    rng = np.random.default_rng(2024)
    kappa0 = np.full(case.design, 0.05)
    run = AdjointRun(case, case.eps0, kappa0, checkpoint_every=256)
    try:
        g_eps, g_kap = run.gradient()
    finally:
        run.close()
    flat = rng.choice(int(np.prod(case.design)), size=16, replace=False)
    cells = [tuple(int(v) for v in np.unravel_index(k, case.design)) for k in flat]
    kcells = cells[:4]
    h = 1e-3
    jobs = []
    for c in cells:
        for s in (1, -1):
            e = case.eps0.copy()
            e[c] += s * h
            jobs.append((kw, e, kappa0))
    for c in kcells:
        for s in (1, -1):
            k = kappa0.copy()
            k[c] += s * h
            jobs.append((kw, case.eps0, k))
    J = fd_pool.starmap(fp64_port_power, jobs)
    fd_e = np.array([(J[2 * k] - J[2 * k + 1]) / (2 * h) for k in range(len(cells))])
    off = 2 * len(cells)
    fd_k = np.array([(J[off + 2 * k] - J[off + 2 * k + 1]) / (2 * h) for k in range(len(kcells))])
    ad_e = np.array([g_eps[c] for c in cells])
    ad_k = np.array([g_kap[c] for c in kcells])
    err_e, err_k = rel_l2(ad_e, fd_e), rel_l2(ad_k, fd_k)
    print(f"dJ/deps rel L2 vs FP64 FD: {err_e:.2e}; dJ/dkappa: {err_k:.2e}")
    assert err_e <= FD_TOL
    assert err_k <= FD_TOL


def test_record_mode_matches_reverse_mode_reference(cuda_lib):
    from oracle.fdtd_ref import reference_edge_gradient
    from openems_gb300.adjoint import AdjointRun
    case = tiny_case()
    run = AdjointRun(case, case.eps0, checkpoint_every=0)
    try:
        gvv, gvi = run.edge_gradient()
        gvv2, gvi2 = run.edge_gradient()          # a second reverse sweep gives the same result
        assert bits_equal(gvv, gvv2) and bits_equal(gvi, gvi2)
        _, rvv, rvi = reference_edge_gradient(run.data, case.steps, *case.box_nodes, case.freqs)
        assert rel_l2(gvv, rvv) <= AUTOGRAD_TOL and rel_l2(gvi, rvi) <= AUTOGRAD_TOL
        assert run.eng.GetNumberOfTimesteps() == case.steps
    finally:
        run.close()


def test_autograd_function(cuda_lib):
    import torch
    from openems_gb300.adjoint import AdjointRun, port_power_objective
    case = tiny_case()
    eps = torch.tensor(case.eps0, requires_grad=True)
    kap = torch.zeros(case.design, dtype=torch.float64, requires_grad=True)
    J = port_power_objective(eps, kap, case, 64)
    J.backward()
    run = AdjointRun(case, case.eps0, checkpoint_every=64)
    try:
        ge, gk = run.gradient()
        assert float(J.detach()) == run.J
    finally:
        run.close()
    assert bits_equal(eps.grad.numpy(), ge)
    assert bits_equal(kap.grad.numpy(), gk)


def test_adjoint_rejects_unsupported_setups(cuda_lib):
    import ctypes as C
    from openems_gb300 import configs
    from openems_gb300.engine import Engine_CUDA, _p
    bs = np.array([6, 6, 6], np.uint32)
    be = np.array([9, 9, 9], np.uint32)
    eng = Engine_CUDA(configs.smoke_case(), 20)           # has Mur walls
    try:
        assert eng.lib.adjoint_setup(eng.h, 16, _p(bs, C.c_uint), _p(be, C.c_uint)) == 4   # OEMS_ERR_UNSUPPORTED
    finally:
        eng.close()
    case = tiny_case(steps=20)
    _, data = case.build(case.eps0)
    eng = Engine_CUDA(data, case.steps)
    try:
        L = eng.lib
        upml_box = np.array([0, 0, 0], np.uint32)
        assert L.adjoint_setup(eng.h, 16, _p(upml_box, C.c_uint), _p(be, C.c_uint)) == 1        # overlaps UPML
        assert L.adjoint_backward(eng.h, 0, None, None, None, None) == 3                       # not set up
        s, e = (np.asarray(v, np.uint32) for v in case.box_nodes)
        assert L.adjoint_setup(eng.h, 16, _p(s, C.c_uint), _p(e, C.c_uint)) == 0
        assert L.adjoint_setup(eng.h, 16, _p(s, C.c_uint), _p(e, C.c_uint)) == 3                # twice
        g = np.zeros(3 * int(np.prod(e - s)))
        assert L.adjoint_backward(eng.h, 0, None, None, _p(g, C.c_double), _p(g, C.c_double)) == 3   # no forward
        assert L.adjoint_forward(eng.h, case.steps + 1) == 1                                    # > max_ts
        assert L.adjoint_forward(eng.h, case.steps) == 0
        assert L.adjoint_forward(eng.h, case.steps) == 3                                        # numTS != 0
    finally:
        eng.close()


@pytest.mark.skipif(os.environ.get("OEMS_FULL_C5") != "1", reason="full-size check: set OEMS_FULL_C5=1 (about 15 min)")
def test_full_design_case_gradient_vs_fp64_central_differences(cuda_lib):
    """The full differentiable-form configuration (200x200x100 lines, 0.5 mm, UPML 8, 64x64x16
    design cells of eps_r U[1,6], ports 60 cells from the region, 4/5/6 GHz, 8000 steps,
    checkpoints every 256 steps): adjoint dJ/d eps_r on 16 random design cells against FP64
    central differences with h = 1e-3.  The FP64 forward runs are the array restatement on torch
    tensors on the GPU (float64 throughout), the only way to run 32 of them at this size."""
    import json
    import torch
    from openems_gb300.adjoint import AdjointRun, port_power
    from openems_gb300.configs import DesignCase
    from oracle.fdtd_ref import RefEngine

    def J64(case, eps):
        _, d = case.build(eps, case.kappa0, fdtd_float=np.float64)
        eng = RefEngine(d, dtype=np.float64, backend="torch", device="cuda").run(case.steps)
        u = eng.probe_series(0).cpu().numpy()
        i = eng.probe_series(len(d.vprobes)).cpu().numpy()
        return port_power(u, i, d.dt, case.freqs)[0]

    case = DesignCase()
    run = AdjointRun(case, case.eps0, case.kappa0, checkpoint_every=256)
    try:
        ge, _ = run.gradient()
        print(json.dumps({"objective": run.J, **run.timing()}), flush=True)
    finally:
        run.close()
    rng = np.random.default_rng(555)
    flat = rng.choice(int(np.prod(case.design)), size=16, replace=False)
    cells = [tuple(int(v) for v in np.unravel_index(k, case.design)) for k in flat]
    h = 1e-3
    fd, ad = [], []
    for c in cells:
        e1, e2 = case.eps0.copy(), case.eps0.copy()
        e1[c] += h
        e2[c] -= h
        fd.append((J64(case, e1) - J64(case, e2)) / (2 * h))
        ad.append(ge[c])
        print(json.dumps({"cell": c, "fd": fd[-1], "adjoint": ad[-1], "rel": abs(fd[-1] - ad[-1]) / abs(fd[-1])}),
              flush=True)
        torch.cuda.empty_cache()
    err = rel_l2(np.array(ad), np.array(fd))
    print(json.dumps({"rel_l2": err, "max_rel": float(np.max(np.abs(np.array(ad) - fd) / np.abs(fd)))}), flush=True)
    assert err <= FD_TOL
