"""Excitation time signals, restating openEMS ``Excitation`` (FDTD/excitation.cpp).

The signals are built on the host in float64 with the C library's ``cos``/``exp``/``pow``
(Python's ``math`` module calls them), then stored as float32 exactly like the reference's
``FDTD_FLOAT* Signal_volt / Signal_curr`` arrays.  The engine only consumes the two arrays,
their length and the optional period.
"""
from __future__ import annotations

import math

import numpy as np

PI = 3.141592653589793238462643383279  # tools/constants.h:27


def calc_nyquist_num(fmax: float, dt: float) -> int:
    """``CalcNyquistNum`` (tools/useful.cpp:30-36)."""
    if fmax == 0:
        return 0xFFFFFFFF
    if dt == 0:
        return 1
    t0 = 1.0 / fmax
    return int(math.floor(t0 / 2 / dt))


class Excitation:
    """Mirror of ``Excitation`` (FDTD/excitation.h:26-110): one time signal shared by all sources."""

    GAUSSIAN, SINUS, DIRAC, STEP = 0, 1, 2, 3

    def __init__(self):
        self.ft = np.float32       # FDTD_FLOAT (tools/constants.h:21); float64 for FP64 checks
        self.kind = None
        self.f0 = 0.0
        self.fc = 0.0
        self.f_max = 0.0
        self.period = 0.0          # m_SignalPeriod (seconds); >0 only for periodic signals
        self.dt = 0.0
        self.length = 0
        self.nyquist = 0
        self.volt = np.zeros(0, self.ft)
        self.curr = np.zeros(0, self.ft)

    # --- setup (FDTD/excitation.cpp:55-93) -------------------------------------------------
    def SetupGaussianPulse(self, f0: float, fc: float):
        self.kind, self.f0, self.fc, self.f_max, self.period = self.GAUSSIAN, f0, fc, f0 + fc, 0.0

    def SetupSinusoidal(self, f0: float):
        self.kind, self.f0, self.f_max, self.period = self.SINUS, f0, f0, 1.0 / f0

    def SetupDiracPulse(self, fmax: float):
        self.kind, self.f_max, self.period = self.DIRAC, fmax, 0.0

    def SetupStepExcite(self, fmax: float):
        self.kind, self.f_max, self.period = self.STEP, fmax, 0.0

    # --- signal (FDTD/excitation.cpp:95-133, 150-230) --------------------------------------
    def Reset(self, dt: float):
        self.dt = float(dt)

    def buildExcitationSignal(self, max_ts: int):
        if self.dt <= 0:
            raise ValueError("Excitation: invalid timestep")
        if self.kind == self.GAUSSIAN:
            self._gauss(self.f0, self.fc, int(max_ts))
        elif self.kind == self.SINUS:
            self._sinus(self.f0, int(max_ts))
        elif self.kind == self.DIRAC:
            self.length = 2
            self.volt = np.array([0.0, 1.0], self.ft)
            self.curr = np.array([0.0, 1.0], self.ft)
            self.nyquist = 1
        elif self.kind == self.STEP:
            self.length = 2
            self.volt = np.array([1.0, 1.0], self.ft)
            self.curr = np.array([1.0, 1.0], self.ft)
            self.nyquist = 1
        else:
            raise ValueError("Excitation: unknown excitation type")
        if self.nyquist == 0:
            raise ValueError("Excitation: setup failed (nyquist number is zero)")

    def _gauss(self, f0, fc, nts):
        """``CalcGaussianPulsExcitation`` (FDTD/excitation.cpp:150-176)."""
        dt = self.dt
        length = int(math.ceil(2.0 * 9.0 / (2.0 * PI * fc) / dt))
        if length > nts:
            length = nts
        v = np.empty(length, np.float64)
        c = np.empty(length, np.float64)
        for n in range(length):
            t = n * dt
            v[n] = math.cos(2.0 * PI * f0 * (t - 9.0 / (2.0 * PI * fc))) * math.exp(-1 * math.pow(2.0 * PI * fc * t / 3.0 - 3, 2))
            t += 0.5 * dt
            c[n] = math.cos(2.0 * PI * f0 * (t - 9.0 / (2.0 * PI * fc))) * math.exp(-1 * math.pow(2.0 * PI * fc * t / 3.0 - 3, 2))
        self.length = length
        self.volt = v.astype(self.ft)
        self.curr = c.astype(self.ft)
        self.f_max = f0 + fc
        self.nyquist = calc_nyquist_num(f0 + fc, dt)

    def _sinus(self, f0, nts):
        """``CalcSinusExcitation`` (FDTD/excitation.cpp:252-275): two periods, index 0 forced to 0."""
        dt = self.dt
        length = int(math.floor(2.0 / f0 / dt + 0.5))  # C round(): half away from zero
        v = np.zeros(length, np.float64)
        c = np.zeros(length, np.float64)
        for n in range(1, length):
            t = n * dt
            v[n] = math.sin(2.0 * PI * f0 * t)
            t += 0.5 * dt
            c[n] = math.sin(2.0 * PI * f0 * t)
        self.length = length
        self.volt = v.astype(self.ft)
        self.curr = c.astype(self.ft)
        self.nyquist = calc_nyquist_num(f0, dt)

    def GetLength(self) -> int:
        return self.length

    def GetNyquistNum(self) -> int:
        return self.nyquist

    def period_steps(self) -> int:
        """``p`` of Engine_Ext_Excitation (FDTD/extensions/engine_ext_excitation.cpp:41-43); 0 = not periodic."""
        if self.period > 0:
            return int(self.period / self.dt)
        return 0

    def GetMaxExcitationTimestep(self) -> int:
        """FDTD/excitation.cpp:135-148."""
        if self.length == 0:
            return 0
        return int(np.argmax(np.abs(self.volt)))
