"""ORACLE (test infrastructure only): numpy restatement of the NF2FF far-field transform of
nf2ff/nf2ff_calc.cpp, Cartesian meshes without mirror planes.

Per face (a planar set of FD-dump samples, E and H complex vectors at sample coordinates in metres):
* normal direction = the axis with one line (nf2ff_calc::GetNormalDir, :233-245), outward sign
  from the face position against the centre (:329-336);
* sample areas = half the distance to the neighbouring lines along both tangential axes, half
  the end interval at the ends (:338-353);
* radiated power += 1/2 area Re(E_P conj(H_PP) - E_PP conj(H_P)) n (:409-418);
* Js = n x H, Ms = -n x E (eq. 8.15a/b, :66-76); radiation vectors
  N_theta, N_phi, L_theta, L_phi = sum area exp(j k r.r_hat) (J or M projected) (:104-150);
Then (:489-528) E_theta = -f (L_phi + Z0 N_theta), E_phi = f (L_theta - Z0 N_phi),
f = j k / (4 pi r) exp(-j k r), P_rad = |E|^2 / (2 Z0), Dmax = max P_rad 4 pi r^2 / P_total.

Precision follows the reference where it matters for the result: float32 geometry and phase
(k r.r_hat formed in float32, exp in complex64), complex128 accumulation.
"""
from __future__ import annotations

import numpy as np

C0 = 299792458.0          # tools/constants.h:25
Z0 = 376.730313461        # tools/constants.h:26


def face_normal(lines):
    n = [len(l) for l in lines]
    ny = -1
    for a in range(3):
        if n[a] == 1 and n[(a + 1) % 3] > 2 and n[(a + 2) % 3] > 2:
            ny = a
    if ny < 0:
        raise ValueError("nf2ff: cannot determine the normal direction of a face")
    return ny


def _edge_lengths(l):
    l = np.asarray(l, np.float32)
    e = np.empty(len(l), np.float32)
    e[1:-1] = np.float32(0.5) * np.abs(l[2:] - l[:-2])
    e[0] = np.float32(0.5) * np.abs(l[1] - l[0])
    e[-1] = np.float32(0.5) * np.abs(l[-1] - l[-2])
    return e


def nf2ff(faces, freq, theta, phi, center=(0.0, 0.0, 0.0), radius=1.0, eps_r=1.0, mu_r=1.0):
    """faces: list of (lines (3 arrays, metres), E, H) with E, H complex arrays [3][n0][n1][n2].
    Returns dict(E_theta, E_phi, P_rad [ntheta][nphi], Prad, Dmax)."""
    theta = np.asarray(theta, np.float32)
    phi = np.asarray(phi, np.float32)
    center = np.asarray(center, np.float32)
    k = np.float32(2 * np.pi * freq / C0 * np.sqrt(eps_r * mu_r))
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    sp, cp = np.sin(phi)[None, :], np.cos(phi)[None, :]
    Nt = np.zeros((len(theta), len(phi)), np.complex128)
    Np = np.zeros_like(Nt)
    Lt = np.zeros_like(Nt)
    Lp = np.zeros_like(Nt)
    prad = 0.0
    for lines, E, H in faces:
        lines = [np.asarray(l, np.float32) for l in lines]
        ny = face_normal(lines)
        nP, nPP = (ny + 1) % 3, (ny + 2) % 3
        nd = np.zeros(3, np.float32)
        nd[ny] = 1.0 if lines[ny][0] >= center[ny] else -1.0
        eP = _edge_lengths(lines[nP])
        ePP = _edge_lengths(lines[nPP])
        E = np.asarray(E, np.complex64)
        H = np.asarray(H, np.complex64)
        # area of each sample in x,y,z order
        shp = [1, 1, 1]
        shp[nP] = len(eP)
        a1 = eP.reshape(shp)
        shp = [1, 1, 1]
        shp[nPP] = len(ePP)
        area = (a1 * ePP.reshape(shp)).astype(np.float64)
        pw = E[nP] * np.conj(H[nPP]) - E[nPP] * np.conj(H[nP])
        prad += float(np.sum(0.5 * area * pw.real.astype(np.float64)) * nd[ny])
        # surface currents
        Js = np.stack([nd[1] * H[2] - nd[2] * H[1], nd[2] * H[0] - nd[0] * H[2], nd[0] * H[1] - nd[1] * H[0]])
        Ms = np.stack([nd[2] * E[1] - nd[1] * E[2], nd[0] * E[2] - nd[2] * E[0], nd[1] * E[0] - nd[0] * E[1]])
        X, Y, Z = np.meshgrid(lines[0] - center[0], lines[1] - center[1], lines[2] - center[2], indexing="ij")
        X, Y, Z = X.ravel(), Y.ravel(), Z.ravel()
        A = area.astype(np.float32).ravel()
        J = Js.reshape(3, -1)
        M = Ms.reshape(3, -1)
        for tn in range(len(theta)):
            for pn in range(len(phi)):
                s_t, c_t = np.float32(st[tn, 0]), np.float32(ct[tn, 0])
                s_p, c_p = np.float32(sp[0, pn]), np.float32(cp[0, pn])
                r_cos_psi = X * (c_p * s_t) + Y * (s_p * s_t) + Z * c_t
                ejkr = np.exp(1j * (k * r_cos_psi)).astype(np.complex64) * A
                Nt[tn, pn] += np.sum((ejkr * (J[0] * (c_t * c_p) + J[1] * (c_t * s_p) - J[2] * s_t)).astype(np.complex128))
                Np[tn, pn] += np.sum((ejkr * (J[1] * c_p - J[0] * s_p)).astype(np.complex128))
                Lt[tn, pn] += np.sum((ejkr * (M[0] * (c_t * c_p) + M[1] * (c_t * s_p) - M[2] * s_t)).astype(np.complex128))
                Lp[tn, pn] += np.sum((ejkr * (M[1] * c_p - M[0] * s_p)).astype(np.complex128))
    z0 = Z0 * np.sqrt(mu_r / eps_r)
    f = 1j * k / (4 * np.pi * radius) * np.exp(-1j * k * radius)
    Eth = -f * (Lp + z0 * Nt)
    Eph = f * (Lt - z0 * Np)
    P = np.abs(Eth * np.conj(Eth) + Eph * np.conj(Eph)) / (2 * z0)
    dmax = float(P.max() * 4 * np.pi * radius ** 2 / prad) if prad != 0 else 0.0
    return {"E_theta": Eth, "E_phi": Eph, "P_rad": P, "Prad": prad, "Dmax": dmax}
