"""NF2FF far-field transform on the device (oems_cuda_nf2ff), the counterpart of openEMS's
nf2ff box (python/openEMS/nf2ff.py: CalcNF2FF) for an engine whose FD dumps record the box faces.

``NF2FFResult`` carries the fields the reference's nf2ff result object exposes for a single
frequency: E_theta, E_phi, P_rad, Dmax and Prad."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np

from .engine import EngineError, _p
from .operator import _dual_line


@dataclass
class NF2FFResult:
    freq: float
    theta: np.ndarray
    phi: np.ndarray
    E_theta: np.ndarray          # [ntheta][nphi] complex
    E_phi: np.ndarray
    P_rad: np.ndarray            # W/m^2 at the radius
    Prad: float                  # W through the faces
    Dmax: float


def box_faces(engine) -> List[Tuple[int, int, List[np.ndarray]]]:
    """(E dump id, H dump id, sample coordinates in metres) of every planar face recorded by an
    E FD dump with a matching H FD dump (same box and mesh).  Coordinates are the mesh lines the
    dump was snapped to: the main lines for node interpolation, the dual lines for cell
    interpolation (Common/processfields.cpp:200-208, 229-243)."""
    op = engine.op
    g = op.grid
    main = [np.asarray(l, np.float64) * g.unit for l in g.lines]
    dual = [_dual_line(np.asarray(l, np.float64)) * g.unit for l in g.lines]
    faces = []
    for ie, de in zip(engine.dump_ids, op.dumps):
        if de.field != 0:
            continue
        for ih, dh in zip(engine.dump_ids, op.dumps):
            if (dh.field == 1 and np.array_equal(de.start, dh.start) and np.array_equal(de.stop, dh.stop)
                    and de.dual == dh.dual):
                lines = dual if de.dual else main
                coords = [lines[a][int(de.start[a]):int(de.stop[a]) + 1] for a in range(3)]
                faces.append((ie, ih, coords))
                break
    return faces


def calc_nf2ff(engine, freq_index: int, theta: Sequence[float], phi: Sequence[float], center=(0.0, 0.0, 0.0),
               radius: float = 1.0, eps_r: float = 1.0, mu_r: float = 1.0, faces=None) -> NF2FFResult:
    """The far field of the recorded faces at the dumps' frequency number ``freq_index``; theta
    and phi in radians, center in metres."""
    faces = box_faces(engine) if faces is None else faces
    if not faces:
        raise EngineError("calc_nf2ff: no E/H FD dump pair found")
    d = engine.op.dumps[engine.dump_ids.index(faces[0][0])]
    freq = float(d.freqs[freq_index])
    eids = np.asarray([f[0] for f in faces], np.int32)
    hids = np.asarray([f[1] for f in faces], np.int32)
    coords = np.ascontiguousarray(np.concatenate([np.concatenate(f[2]) for f in faces]), np.float64)
    th = np.ascontiguousarray(theta, np.float64)
    ph = np.ascontiguousarray(phi, np.float64)
    ctr = np.ascontiguousarray(center, np.float64)
    nt, npp = len(th), len(ph)
    et = np.zeros(2 * nt * npp)
    ep = np.zeros(2 * nt * npp)
    pr = np.zeros(nt * npp)
    prad, dmax = C.c_double(), C.c_double()
    engine._ck(engine.lib.nf2ff(engine.h, len(faces), _p(eids, C.c_int), _p(hids, C.c_int), _p(coords, C.c_double),
                                int(freq_index), freq, nt, _p(th, C.c_double), npp, _p(ph, C.c_double),
                                _p(ctr, C.c_double), float(radius), float(eps_r), float(mu_r), _p(et, C.c_double),
                                _p(ep, C.c_double), _p(pr, C.c_double), C.byref(prad), C.byref(dmax)), "nf2ff")
    shape = (nt, npp)
    return NF2FFResult(freq, th, ph, (et[0::2] + 1j * et[1::2]).reshape(shape), (ep[0::2] + 1j * ep[1::2]).reshape(shape),
                       pr.reshape(shape), prad.value, dmax.value)
