"""ORACLE (test infrastructure only): array-level restatement of the EC-FDTD timestep for the
differentiable form, in any floating type, on numpy or torch arrays.

It restates, for engines with excitation, UPML and probes (no Mur walls, no dispersive
materials):

* Engine::UpdateVoltages / UpdateCurrents (FDTD/engine.cpp:110-222): separate multiply and add
  in the reference's evaluation order ((a - b) - c) + d; at index 0 the "previous" neighbour is
  the cell itself (the reference's shift of 0).
* Engine_Ext_UPML pre/post voltage and current hooks (FDTD/extensions/engine_ext_upml.cpp:52-229).
* Engine_Ext_Excitation::Apply2Voltages/Apply2Current (FDTD/extensions/engine_ext_excitation.cpp:33-94),
  with the excitation position rule of the reference.
* ProcessVoltage / ProcessCurrent line integrals (FDTD/engine_interface_fdtd.cpp:206-232,
  Common/processcurrent.cpp:96-171) sampled after every step at numTS (Common/processintegral.cpp:134-171).

Three uses, all as a checker:
* float32 on numpy: bit-identical to the C oracle (pins this restatement);
* float64 on numpy: the FP64 forward run behind central finite differences;
* float64 on torch (CPU) with coefficient tensors that require grad: a reverse-mode
  reference gradient through the time loop, independent of the hand-written adjoint.
"""
from __future__ import annotations

import numpy as np


class _NP:
    def __init__(self, dtype):
        self.dtype = np.dtype(dtype)

    def asarray(self, a):
        return np.asarray(a, dtype=self.dtype)

    def zeros(self, shape):
        return np.zeros(shape, self.dtype)

    def cat(self, parts, axis):
        return np.concatenate(parts, axis=axis)

    @staticmethod
    def copy(a):
        return a.copy()

    @staticmethod
    def scalar(a):
        return a


class _Torch:
    def __init__(self, dtype, device="cpu"):
        import torch
        self.torch = torch
        self.dtype = dtype
        self.device = device

    def asarray(self, a):
        t = self.torch
        if isinstance(a, t.Tensor):
            return a.to(self.dtype)
        return t.as_tensor(np.asarray(a), dtype=self.dtype, device=self.device)

    def zeros(self, shape):
        return self.torch.zeros(shape, dtype=self.dtype, device=self.device)

    def cat(self, parts, axis):
        return self.torch.cat(parts, dim=axis)

    @staticmethod
    def copy(a):
        return a.clone()

    @staticmethod
    def scalar(a):
        return a


def _prev(xp, a, axis):
    """a[i-1] along `axis` with a[-1] replaced by a[0] (the engine's zero shift at index 0)."""
    sl0 = [slice(None)] * a.ndim
    sl0[axis] = slice(0, 1)
    slm = [slice(None)] * a.ndim
    slm[axis] = slice(0, a.shape[axis] - 1)
    return xp.cat([a[tuple(sl0)], a[tuple(slm)]], axis)


def voltage_terms(p):
    """(component, x, y, z, sign) in the order of Engine_Interface_FDTD::CalcVoltageIntegral."""
    out = []
    s = [int(v) for v in p.start]
    t = [int(v) for v in p.stop]
    for n in range(3):
        if s[n] < t[n]:
            pos = list(s)
            while pos[n] < t[n]:
                out.append((n, pos[0], pos[1], pos[2], 1))
                pos[n] += 1
        else:
            pos = list(t)
            while pos[n] < s[n]:
                out.append((n, pos[0], pos[1], pos[2], -1))
                pos[n] += 1
    return out


def current_terms(p):
    """(component, x, y, z, sign) in the order of ProcessCurrent::CalcIntegral."""
    s = [int(v) for v in p.start]
    t = [int(v) for v in p.stop]
    si = [int(v) for v in p.start_inside]
    ei = [int(v) for v in p.stop_inside]
    out = []

    def run(cond, comp, rng, fix, sign):
        if cond:
            for i in rng:
                pos = list(fix)
                pos[comp] = i
                out.append((comp, pos[0], pos[1], pos[2], sign))

    nd = int(p.norm_dir)
    if nd == 0:
        run(ei[0] and si[2], 1, range(s[1] + 1, t[1] + 1), (t[0], 0, s[2]), 1)
        run(ei[0] and ei[1], 2, range(s[2] + 1, t[2] + 1), (t[0], t[1], 0), 1)
        run(si[0] and ei[2], 1, range(s[1] + 1, t[1] + 1), (s[0], 0, t[2]), -1)
        run(si[0] and si[1], 2, range(s[2] + 1, t[2] + 1), (s[0], s[1], 0), -1)
    elif nd == 1:
        run(si[0] and si[1], 2, range(s[2] + 1, t[2] + 1), (s[0], s[1], 0), 1)
        run(ei[1] and ei[2], 0, range(s[0] + 1, t[0] + 1), (0, t[1], t[2]), 1)
        run(ei[0] and ei[1], 2, range(s[2] + 1, t[2] + 1), (t[0], t[1], 0), -1)
        run(si[1] and si[2], 0, range(s[0] + 1, t[0] + 1), (0, s[1], s[2]), -1)
    elif nd == 2:
        run(si[1] and si[2], 0, range(s[0] + 1, t[0] + 1), (0, s[1], s[2]), 1)
        run(ei[0] and si[2], 1, range(s[1] + 1, t[1] + 1), (t[0], 0, s[2]), 1)
        run(ei[1] and ei[2], 0, range(s[0] + 1, t[0] + 1), (0, t[1], t[2]), -1)
        run(si[0] and ei[2], 1, range(s[1] + 1, t[1] + 1), (s[0], 0, t[2]), -1)
    return out


class RefEngine:
    """Time loop over `op` (an OperatorData). ``backend`` is "numpy" or "torch" (``device`` may
    then be "cuda"); ``coef`` may replace (vv, vi, ii, iv) by arrays of the backend (e.g. torch
    tensors that require grad).  The three field components are updated together as stacked
    [3][Nx][Ny][Nz] arrays; element by element the arithmetic is the reference's."""

    def __init__(self, op, dtype=np.float64, backend="numpy", coef=None, device="cpu"):
        if op.mur or op.lorentz:
            raise ValueError("RefEngine: Mur walls and dispersive materials are not restated here")
        self.torch = backend != "numpy"
        if not self.torch:
            self.xp = _NP(dtype)
        else:
            import torch
            self.xp = _Torch({np.float32: torch.float32, np.float64: torch.float64}.get(dtype, dtype), device)
        xp = self.xp
        self.op = op
        self.N = [int(v) for v in op.num_lines]
        c = coef if coef is not None else (op.vv, op.vi, op.ii, op.iv)
        self.vv, self.vi, self.ii, self.iv = (xp.asarray(a) for a in c)
        self.V = xp.zeros((3,) + tuple(self.N))
        self.I = xp.zeros((3,) + tuple(self.N))
        self.upml = []
        for u in op.upml:
            tabs = {k: xp.asarray(getattr(u, k)) for k in ("vv", "vvfo", "vvfn", "ii", "iifo", "iifn")}
            start = [int(v) for v in u.start]
            nl = tuple(int(n) for n in u.num_lines)
            self.upml.append((start, nl, tabs, [xp.zeros((3,) + nl), xp.zeros((3,) + nl)]))
        ex = op.exc
        self.exc = []
        for idx, dr, amp, dl, sig in ((ex.volt_index, ex.volt_dir, ex.volt_amp, ex.volt_delay, ex.signal_volt),
                                      (ex.curr_index, ex.curr_dir, ex.curr_amp, ex.curr_delay, ex.signal_curr)):
            idx = np.asarray(idx, np.int64).reshape(3, -1)
            sel = (np.asarray(dr, np.int64), idx[0], idx[1], idx[2])
            if self.torch:
                sel = tuple(xp.torch.as_tensor(a, device=device) for a in sel)
            self.exc.append((sel, xp.asarray(amp), np.asarray(dl, np.int64), xp.asarray(sig), idx.shape[1]))
        self.sig_len = len(ex.signal_volt)
        self.period = int(ex.period)
        self.probes = []
        for typ, plist in ((0, op.vprobes), (1, op.iprobes)):
            for p in plist:
                terms = voltage_terms(p) if typ == 0 else current_terms(p)
                gat = None
                if self.torch and terms:
                    t = xp.torch
                    arr = np.asarray(terms, np.int64)
                    gat = (tuple(t.as_tensor(arr[:, k], device=device) for k in range(4)),
                           t.as_tensor(arr[:, 4], dtype=xp.dtype, device=device))
                self.probes.append((typ, terms, gat, float(p.weight), int(p.start_ts), int(p.stop_ts)))
        self.series = [[] for _ in self.probes]
        self.numTS = 0
        self._sample()                  # the initial state is sampled too (numTS = 0)

    # ---- curls -------------------------------------------------------------------------------
    def _curl_v(self, I):
        xp = self.xp
        i0, i1, i2 = I[0], I[1], I[2]
        c0 = ((i2 - _prev(xp, i2, 1)) - i1) + _prev(xp, i1, 2)
        c1 = ((i0 - _prev(xp, i0, 2)) - i2) + _prev(xp, i2, 0)
        c2 = ((i1 - _prev(xp, i1, 0)) - i0) + _prev(xp, i0, 1)
        return self._stack([c0, c1, c2])

    def _curl_i(self, V):
        v0, v1, v2 = V[0], V[1], V[2]
        a = (slice(0, -1),) * 3
        xs = (slice(1, None), slice(0, -1), slice(0, -1))
        ys = (slice(0, -1), slice(1, None), slice(0, -1))
        zs = (slice(0, -1), slice(0, -1), slice(1, None))
        c0 = ((v2[a] - v2[ys]) - v1[a]) + v1[zs]
        c1 = ((v0[a] - v0[zs]) - v2[a]) + v2[xs]
        c2 = ((v1[a] - v1[xs]) - v0[a]) + v0[ys]
        return self._stack([c0, c1, c2])

    def _stack(self, parts):
        if self.torch:
            return self.xp.torch.stack(parts)
        return np.stack(parts)

    # ---- one half-step -----------------------------------------------------------------------
    def _update(self, F, curl, cf, cc, hi, which):
        """F' = cf*F + cc*curl on [0, hi) per axis, with the UPML pre/post hooks inside it."""
        xp = self.xp
        reg = (slice(None),) + tuple(slice(0, h) for h in hi)
        out = xp.copy(F)
        out[reg] = F[reg] * cf[reg] + cc[reg] * curl
        for start, nl, tabs, flux in self.upml:
            cvv, cfo, cfn = (tabs["vv"], tabs["vvfo"], tabs["vvfn"]) if which == 0 else \
                            (tabs["ii"], tabs["iifo"], tabs["iifn"])
            stop = [min(start[a] + nl[a], hi[a]) for a in range(3)]
            if any(stop[a] <= start[a] for a in range(3)):
                continue
            g = (slice(None),) + tuple(slice(start[a], stop[a]) for a in range(3))
            loc = (slice(None),) + tuple(slice(0, stop[a] - start[a]) for a in range(3))
            psi = flux[which]
            ps = psi[loc]
            pre = F[g] * cvv[loc] - cfo[loc] * ps                  # f = vv*V - vvfo*flux
            vn = ps * cf[g] + cc[g] * curl[g]                      # the update on V = flux
            newpsi = xp.copy(psi)
            newpsi[loc] = vn                                       # flux = V
            flux[which] = newpsi
            out[g] = pre + cfn[loc] * vn                           # V = f + vvfn*flux
        return out

    def _excite(self, F, k):
        sel, amp, dl, sig, cnt = self.exc[k]
        if cnt == 0:
            return F
        p = self.numTS + 1 if self.period <= 0 else self.period
        pos = self.numTS - dl
        pos = pos * (pos > 0)
        pos = pos % p
        pos = pos * (pos < self.sig_len)
        if self.torch:
            t = self.xp.torch
            vals = amp * sig[t.as_tensor(pos, device=sig.device)]
            return F.index_put(sel, vals, accumulate=True)          # distinct source edges
        out = F.copy()
        out[sel] = out[sel] + amp * sig[pos]
        return out

    def _sample(self):
        ts = self.numTS
        for k, (typ, terms, gat, w, t0, t1) in enumerate(self.probes):
            if ts < t0 or ts > t1:
                self.series[k].append(0.0 * w)
                continue
            F = self.V if typ == 0 else self.I
            if self.torch:
                acc = (F[gat[0]] * gat[1]).sum() if gat is not None else 0.0
                self.series[k].append(acc * w)
                continue
            # voltage: double accumulation; current: accumulation in the field type
            acc = np.float64(0.0) if typ == 0 else F.dtype.type(0.0)
            for (n, x, y, z, s) in terms:
                v = F[n, x, y, z]
                if typ == 0:
                    v = np.float64(v)
                acc = acc + v if s > 0 else acc - v
            self.series[k].append(np.float64(acc) * w)

    def step(self):
        N = self.N
        self.V = self._update(self.V, self._curl_v(self.I), self.vv, self.vi, N, 0)
        self.V = self._excite(self.V, 0)
        self.I = self._update(self.I, self._curl_i(self.V), self.ii, self.iv, [n - 1 for n in N], 1)
        self.I = self._excite(self.I, 1)
        self.numTS += 1
        self._sample()

    def run(self, steps):
        for _ in range(int(steps)):
            self.step()
        return self

    def probe_series(self, k):
        """Samples at numTS = 0..numTS."""
        s = self.series[k]
        if not self.torch:
            return np.asarray(s, np.float64)
        t = self.xp.torch
        return t.stack([x if isinstance(x, t.Tensor) else t.tensor(x, dtype=self.xp.dtype, device=self.xp.device)
                        for x in s])


def port_power_torch(u, i, dt, freqs):
    """J = sum_f 1/2 Re(U_f conj(I_f)) on torch series (the objective of the differentiable form)."""
    import torch
    n = torch.arange(u.shape[0], dtype=torch.float64, device=u.device)
    J = torch.zeros((), dtype=torch.float64, device=u.device)
    for f in freqs:
        th_u = -2.0 * np.pi * f * n * dt
        th_i = -2.0 * np.pi * f * (n + 0.5) * dt
        Ur, Ui = (u * torch.cos(th_u)).sum() * 2 * dt, (u * torch.sin(th_u)).sum() * 2 * dt
        Ir, Ii = (i * torch.cos(th_i)).sum() * 2 * dt, (i * torch.sin(th_i)).sum() * 2 * dt
        J = J + 0.5 * (Ur * Ir + Ui * Ii)
    return J


def reference_edge_gradient(op, steps, box_start, box_stop, freqs, vprobe=0, iprobe=None, device="cpu"):
    """Reverse-mode reference: torch autograd (CPU, float64) through `steps` timesteps of `op`
    for J = port_power(voltage probe `vprobe`, current probe `iprobe`).  Returns
    (J, dJ/dvv, dJ/dvi) with the gradients restricted to the nodes box_start..box_stop-1."""
    import torch
    vv = torch.tensor(np.asarray(op.vv, np.float64), device=device, requires_grad=True)
    vi = torch.tensor(np.asarray(op.vi, np.float64), device=device, requires_grad=True)
    eng = RefEngine(op, dtype=np.float64, backend="torch", coef=(vv, vi, op.ii, op.iv), device=device)
    eng.run(steps)
    ip = len(op.vprobes) + (0 if iprobe is None else iprobe)
    J = port_power_torch(eng.probe_series(vprobe), eng.probe_series(ip), float(op.dt), freqs)
    J.backward()
    box = (slice(None),) + tuple(slice(int(s), int(e)) for s, e in zip(box_start, box_stop))
    return float(J.detach()), vv.grad[box].cpu().numpy().copy(), vi.grad[box].cpu().numpy().copy()


def fp64_port_power(case_kwargs, eps, kappa):
    """The objective of a DesignCase design from an FP64 forward run on the host (a worker for
    central finite differences; picklable arguments so it can run in a spawn pool)."""
    from openems_gb300.adjoint import port_power
    from openems_gb300.configs import DesignCase
    case = DesignCase(**case_kwargs)
    _, data = case.build(eps, kappa, fdtd_float=np.float64)
    eng = RefEngine(data, dtype=np.float64).run(case.steps)
    return port_power(eng.probe_series(0), eng.probe_series(len(data.vprobes)), float(data.dt), case.freqs)[0]
