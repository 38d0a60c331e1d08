"""Differentiable form: the gradient of a port-power DFT objective with respect to per-cell
eps_r and kappa of a design region, from the adjoint (time-reversed) engine kernels, behind a
``torch.autograd.Function``.

The chain is
    J(u, i)  --dJ/du, dJ/di-->  oems_cuda_adjoint_backward  --dJ/dvv, dJ/dvi (edges)-->
    Calc_ECOperatorPos  (FDTD/operator.cpp:956-984: vv, vi from C, G and dt)  --dJ/dC, dJ/dG-->
    AverageMatQuarterCell + Calc_ECPos (FDTD/operator.cpp:1447-1564, 1189-1254: C and G of an
    edge are area-weighted sums over the four cells around it)  --> dJ/d eps_r, dJ/d kappa.
The timestep is held fixed across designs (the operator's forced-timestep path,
FDTD/operator.cpp:994-1012), so dt does not enter the derivative.

The objective is the power delivered to the output port, summed over the design frequencies,
    J = sum_f 1/2 Re(U_f conj(I_f)),   U_f = sum_n u[n] 2 dt exp(-2 pi j f n dt),
    I_f = sum_n i[n] 2 dt exp(-2 pi j f (n + 1/2) dt),
i.e. the DFT of Common/processintegral.cpp:134-171 with the current sampled half a step later,
and port power P = 1/2 Re(U conj(I)) as in python/openEMS/ports.py (CalcPort).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _native
from .engine import Engine_CUDA, EngineError, _p
from .operator import EPS0, _axes


# ------------------------------------------------------------------------------------------
def port_power(u: np.ndarray, i: np.ndarray, dt: float, freqs: Sequence[float]):
    """J and dJ/du[n], dJ/di[n] for sample series u, i at numTS = 0..len-1 (float64)."""
    u = np.asarray(u, np.float64)
    i = np.asarray(i, np.float64)
    n = np.arange(len(u), dtype=np.float64)
    J = 0.0
    su = np.zeros(len(u))
    si = np.zeros(len(i))
    for f in freqs:
        cu = 2.0 * dt * np.exp(-2j * np.pi * f * n * dt)
        ci = 2.0 * dt * np.exp(-2j * np.pi * f * (n + 0.5) * dt)
        U = np.dot(u, cu)
        I = np.dot(i, ci)
        J += 0.5 * (U * np.conj(I)).real
        su += 0.5 * (cu * np.conj(I)).real
        si += 0.5 * (U * np.conj(ci)).real
    return float(J), su, si


# ------------------------------------------------------------------------------------------
def material_chain(op, c0, design, g_vv: np.ndarray, g_vi: np.ndarray):
    """dJ/d eps_r and dJ/d kappa of the design cells from dJ/dvv, dJ/dvi of the edges at the
    design-box nodes c0 .. c0+design (inclusive), arrays [3][bx][by][bz].

    For an edge of direction n at node (i_n, i_p, i_pp), the quarter-cell average gives
        C = EPS0 * sum_q eps_q A_q / sum_q A_q * area / length,
    the four cells q = (i_n, i_p - {0,1}, i_pp - {0,1}) with A_q = width_p(q) * width_pp(q),
    sum_q A_q = (w_p(i_p) + w_p(i_p-1)) (w_pp(i_pp) + w_pp(i_pp-1)), area = dual widths at the
    node, length = the edge's main width; G likewise with kappa and without EPS0."""
    dt = float(op.dT)
    u = float(op.unit)
    d = [int(v) for v in design]
    c0 = [int(v) for v in c0]
    box = tuple(slice(c0[a], c0[a] + d[a] + 1) for a in range(3))
    g_eps = np.zeros(d)
    g_kap = np.zeros(d)
    for n in range(3):
        a, p, pp = _axes(n)
        Cn = op.EC_C[n][box].astype(np.float64)
        Gn = op.EC_G[n][box].astype(np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            x = dt * Gn / (2.0 * Cn)
            den = Cn + dt * Gn / 2.0
            dvv_dC = 2.0 * x / (Cn * (1.0 + x) ** 2)
            dvv_dG = -dt / (Cn * (1.0 + x) ** 2)
            dvi_dC = -dt / den ** 2
            dvi_dG = -(dt * dt / 2.0) / den ** 2
        gC = np.where(Cn > 0, g_vv[n] * dvv_dC + g_vi[n] * dvi_dC, 0.0)
        gG = np.where(Cn > 0, g_vv[n] * dvv_dG + g_vi[n] * dvi_dG, 0.0)
        md, dd = op.md, op.dd
        cells = [np.arange(c0[k], c0[k] + d[k]) for k in range(3)]

        def shaped(ax, v):
            s = [1, 1, 1]
            s[ax] = len(v)
            return v.reshape(s)

        fa = shaped(a, u / md[a][cells[a]])
        for dp in (0, 1):
            ip = cells[p] + dp
            fp = shaped(p, md[p][cells[p]] * dd[p][ip] / (md[p][ip] + md[p][ip - 1]))
            for dpp in (0, 1):
                ipp = cells[pp] + dpp
                fpp = shaped(pp, md[pp][cells[pp]] * dd[pp][ipp] / (md[pp][ipp] + md[pp][ipp - 1]))
                w = fa * fp * fpp
                sl = [slice(0, d[0]), slice(0, d[1]), slice(0, d[2])]
                sl[p] = slice(dp, dp + d[p])
                sl[pp] = slice(dpp, dpp + d[pp])
                sl = tuple(sl)
                g_eps += EPS0 * w * gC[sl]
                g_kap += w * gG[sl]
    return g_eps, g_kap


# ------------------------------------------------------------------------------------------
class AdjointRun:
    """One design on the GPU: forward run with checkpoints, then (on demand) the reverse sweep."""

    def __init__(self, case, eps, kappa=None, checkpoint_every: int = 256, device: int = 0):
        self.case = case
        self.op, self.data = case.build(eps, kappa)
        self.eng = Engine_CUDA(self.data, case.steps, device=device)
        self.lib = self.eng.lib
        bs, be = case.box_nodes
        self.bs = np.asarray(bs, np.uint32)
        self.be = np.asarray(be, np.uint32)
        self.eng._ck(self.lib.adjoint_setup(self.eng.h, int(checkpoint_every), _p(self.bs, C.c_uint),
                                            _p(self.be, C.c_uint)), "adjoint_setup")
        self.eng._ck(self.lib.adjoint_forward(self.eng.h, int(case.steps)), "adjoint_forward")
        n = case.steps + 1
        self.vid = self.eng.vprobe_ids[0]
        self.iid = self.eng.iprobe_ids[0]
        self.u = self._series(self.vid, n)
        self.i = self._series(self.iid, n)
        self.J, self.su, self.si = port_power(self.u, self.i, self.data.dt, case.freqs)

    def _series(self, pid, n):
        s = self.eng.probe_series(pid)
        out = np.zeros(n)
        out[:min(n, len(s))] = s[:n]
        return out

    def edge_gradient(self):
        """dJ/dvv and dJ/dvi of the design-box edges, [3][bx][by][bz] each."""
        shape = (3,) + tuple(int(e) - int(s) for s, e in zip(self.bs, self.be))
        gvv = np.zeros(shape)
        gvi = np.zeros(shape)
        ids = np.asarray([self.vid, self.iid], np.int32)
        # the reverse sweep is linear in its sources: run it on sources scaled to a maximum of 1
        # (port powers in SI units are tiny; this keeps the float32 adjoint state well above
        # the denormal range) and scale the result back in double
        scale = float(max(np.abs(self.su).max(), np.abs(self.si).max()))
        if scale == 0.0:
            return gvv, gvi
        src = np.ascontiguousarray(np.stack([self.su, self.si]) / scale)
        self.eng._ck(self.lib.adjoint_backward(self.eng.h, 2, _p(ids, C.c_int), _p(src, C.c_double),
                                               _p(gvv, C.c_double), _p(gvi, C.c_double)), "adjoint_backward")
        return gvv * scale, gvi * scale

    def gradient(self):
        gvv, gvi = self.edge_gradient()
        return material_chain(self.op, self.case.c0, self.case.design, gvv, gvi)

    def timing(self):
        f, b = C.c_float(), C.c_float()
        L = C.c_uint()
        self.eng._ck(self.lib.adjoint_timing(self.eng.h, C.byref(f), C.byref(b), C.byref(L)), "adjoint_timing")
        return {"forward_ms": f.value, "backward_ms": b.value, "launches_per_reverse_step": L.value}

    def close(self):
        if self.eng is not None:
            self.eng.close()
            self.eng = None


# ------------------------------------------------------------------------------------------
try:
    import torch

    class PortPowerObjective(torch.autograd.Function):
        """J(eps_r, kappa) of a ``configs.DesignCase`` on the GPU engine.  The forward pass runs
        the simulation with checkpoints; the backward pass runs the reverse sweep."""

        @staticmethod
        def forward(ctx, eps, kappa, case, checkpoint_every=256, device=0):
            run = AdjointRun(case, eps.detach().cpu().double().numpy(), kappa.detach().cpu().double().numpy(),
                             checkpoint_every=checkpoint_every, device=device)
            ctx.run = run
            ctx.dtypes = (eps.dtype, kappa.dtype, eps.device, kappa.device)
            return torch.tensor(run.J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            run = ctx.run
            try:
                ge, gk = run.gradient()
            finally:
                run.close()
            de, dk, deve, devk = ctx.dtypes
            g = float(gJ)
            return (torch.from_numpy(ge * g).to(dtype=de, device=deve),
                    torch.from_numpy(gk * g).to(dtype=dk, device=devk), None, None, None)

    def port_power_objective(eps, kappa, case, checkpoint_every=256, device=0):
        return PortPowerObjective.apply(eps, kappa, case, checkpoint_every, device)

except ImportError:   # torch is optional for the numpy interface above
    pass
