"""Inlet waveforms -> per-step amplitude tables for ``lbm_set_inlet_table``.

* :func:`pulsatile` / :func:`inlet_velocity` restate the reference's
  ``Pulsatile`` polynomials (pulsatile.h:8-30) and
  ``Simulation::getInletVelocity`` (Simulation.cpp:548-563): three piecewise
  polynomials over ``fmod(t, 0.9)``, zero on [0.81, 0.9).
* :func:`reference_table` reproduces the times ``Iterate()`` visits
  (``t`` starts at 0 and accumulates ``t += dt`` in FP64,
  Simulation.cpp:571-599), so table[s] is the exact inlet value of step s.
* :func:`sinusoid_table` is the benchmark waveform
  u(t) = U (1 + 0.5 sin(2 pi t / T) + 0.2 sin(4 pi t / T)), t in steps.
"""
from __future__ import annotations

import math

import numpy as np

PERIOD = 0.9


def _eq1(x):
    return (-8.579e+08 * x ** 8 + 4.059e+08 * x ** 7 - 7.817e+07 * x ** 6 + 7.994e+06 * x ** 5
            - 4.835e+05 * x ** 4 + 1.782e+04 * x ** 3 - 321.6 * x ** 2 + 3.215 * x + 0.1423)


def _eq2(x):
    return (-4.32e+06 * x ** 8 + 7.94e+06 * x ** 7 - 6.298e+06 * x ** 6 + 2.82e+06 * x ** 5
            - 7.809e+05 * x ** 4 + 1.37e+05 * x ** 3 - 1.484e+04 * x ** 2 + 901.9 * x - 22.87)


def _eq3(x):
    return -5.123 * x ** 4 + 14.15 * x ** 3 - 14.21 * x ** 2 + 5.865 * x - 0.5696


def inlet_velocity(t: float, period: float = PERIOD) -> float:
    """getInletVelocity(t, period) (Simulation.cpp:548-563)."""
    vel = 0.0
    xn = math.fmod(t, period)
    if 0 <= xn < 0.1 * period:
        vel = _eq1(xn)
    elif 0.1 * period <= xn < 0.3 * period:
        vel = _eq2(xn)
    elif 0.3 * period <= xn < 0.9 * period:
        vel = _eq3(xn)
    return vel


def reference_table(dt: float, nsteps: int, period: float = PERIOD) -> np.ndarray:
    """Inlet value of each step of Iterate() for nsteps steps."""
    out = np.empty(nsteps, np.float64)
    t = 0.0
    for s in range(nsteps):
        out[s] = inlet_velocity(t, period)
        t += dt
    return out


def pulsatile(x: float) -> float:
    """Alias kept for callers that evaluate the waveform at a phase."""
    return inlet_velocity(x)


def sinusoid_table(mean: float, period_steps: float, n: int | None = None) -> np.ndarray:
    """u(s) = mean (1 + 0.5 sin(2 pi s/T) + 0.2 sin(4 pi s/T)); one period by default."""
    n = int(round(period_steps)) if n is None else n
    s = np.arange(n, dtype=np.float64)
    w = 2.0 * math.pi * s / period_steps
    return mean * (1.0 + 0.5 * np.sin(w) + 0.2 * np.sin(2.0 * w))
