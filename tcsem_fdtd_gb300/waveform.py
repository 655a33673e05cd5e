"""Post-processing of receiver traces into the responses of other source waveforms.

The time loop injects a narrow Gaussian pulse of unit area (SourceWave.cpp,
centred at 3 sigma_t), so every trace is, to that pulse's width, the impulse
response h(t) of its receiver component.  Responses to other transmitter
current waveforms follow by integration, without running the solver again:

* :func:`step_off` -- current switched off at t = 0 after a long on-time:
  s(t) = integral_t^inf h(tau) dtau;
* :func:`convolve` -- any current waveform I(t) given by samples (piecewise
  linear, zero outside the given times): y(t) = integral h(tau) I(t - tau) dtau.

The time loop starts at t = 0 with the pulse centred at t = 3 sigma_t
(main.cu:151-152), so a trace sampled at time t belongs to the delay
tau = t - 3 sigma_t; both functions take that shift as ``delay`` (3 sigma_t is
half the last time that ``Simulation.waveform()`` returns).

The traces are sampled at few, usually log-spaced, times (Receiver.in), so h is
interpolated by a cubic spline of tau h(tau) in u = ln tau, where it is smooth,
and the integrals are taken in u.  Beyond the last sample h is continued by the
late-time form t^-p exp(-a/t) fitted to the last three samples (step_off only).
"""
from __future__ import annotations

import os

import numpy as np


def sampling_times(directory):
    """The receiver sampling times of a survey directory (Receiver.in, logspace.cpp:5-19)."""
    with open(os.path.join(directory, "Receiver.in")) as f:
        tok = f.read().split()
    t0, tn, nt, islog = float(tok[0]), float(tok[1]), int(tok[2]), int(tok[3])
    if islog:
        return 10.0 ** (np.log10(t0) + np.arange(nt) * (np.log10(tn) - np.log10(t0)) / (nt - 1))
    return t0 + np.arange(nt) * (tn - t0) / (nt - 1)


def _spline(t, h):
    from scipy.interpolate import CubicSpline

    if np.any(t <= 0) or np.any(np.diff(t) <= 0):
        raise ValueError("sampling times must be positive and increasing")
    return CubicSpline(np.log(t), t * np.asarray(h, dtype=float), axis=-1)


def _tail(t, h):
    """integral_{T_N}^inf h for each trace, from its last three samples.

    The late-time form of a diffusive field, h = C t^-p exp(-a/t) (exact for a
    uniform half-space), is fitted through the last three samples and
    integrated in closed form, C a^(1-p) Gamma(p-1) P(p-1, a/T_N) (P the
    regularised lower incomplete gamma function).  Where that fit does not
    decay (p <= 1 or a < 0) the power law through the last two samples is used;
    a trace that still changes sign, or decays as t^-1 or slower, has no finite
    tail and gets NaN.  A trace that ends at 0 gets 0.
    """
    from scipy.special import gamma, gammainc

    tt = t[-3:]
    hh = h[..., -3:].reshape(-1, 3)
    out = np.full(hh.shape[0], np.nan)
    G = np.stack([np.ones(3), -np.log(tt), -1.0 / tt], axis=1)
    for r, v in enumerate(hh):
        if v[-1] == 0 and v[-2] == 0:
            out[r] = 0.0
            continue
        if not (np.all(v > 0) or np.all(v < 0)):
            continue
        c, p, a = np.linalg.solve(G, np.log(np.abs(v)))
        sgn = np.sign(v[-1])
        if p > 1 and a > 0:
            out[r] = sgn * np.exp(c) * a ** (1 - p) * gamma(p - 1) * gammainc(p - 1, a / tt[-1])
            continue
        q = np.log(v[-2] / v[-1]) / np.log(tt[-1] / tt[-2])
        if q > 1:
            out[r] = v[-1] * tt[-1] / (q - 1)
    return out.reshape(h.shape[:-1])


def step_off(times, traces, delay=0.0):
    """Step-off responses at the sampling times: traces [..., Nt] of impulse responses -> [..., Nt]."""
    t = np.asarray(times, dtype=float) - delay
    h = np.asarray(traces, dtype=float)
    sp = _spline(t, h)
    u = np.log(t)
    # integral_t^T_N h dt = integral_u^u_N (t h)(u) du
    rest = np.stack([sp.integrate(u[i], u[-1]) for i in range(len(t))], axis=-1)
    return rest + _tail(t, h)[..., None]


def convolve(times, traces, wave_t, wave_i, out_times=None, delay=0.0, order=8):
    """Responses to the source current I(t) sampled at wave_t (piecewise linear, 0 outside).

    Returns [..., len(out_times)] at the delays out_times (default: the sampling
    delays).  The impulse response is taken as 0 outside the sampled delays.  For
    each output delay t the integral over u = ln tau is split at the spline knots
    and at the current's breakpoints tau = t - wave_t, where the integrand has
    kinks or jumps, and each piece is summed by Gauss-Legendre of the given order.
    """
    t = np.asarray(times, dtype=float) - delay
    h = np.asarray(traces, dtype=float)
    wt, wi = np.asarray(wave_t, dtype=float), np.asarray(wave_i, dtype=float)
    if wt.ndim != 1 or wt.shape != wi.shape or len(wt) < 2 or np.any(np.diff(wt) <= 0):
        raise ValueError("the current needs at least two samples at increasing times")
    ot = t if out_times is None else np.asarray(out_times, dtype=float)
    sp = _spline(t, h)
    u = np.log(t)
    gx, gw = np.polynomial.legendre.leggauss(order)
    out = np.zeros(h.shape[:-1] + (len(ot),))
    for q, tq in enumerate(ot):
        br = tq - wt
        br = np.log(br[(br > t[0]) & (br < t[-1])])
        edges = np.union1d(u, br)
        a, b = edges[:-1], edges[1:]
        uu = (0.5 * (b - a)[:, None] * gx[None, :] + 0.5 * (a + b)[:, None]).ravel()
        ww = (0.5 * (b - a)[:, None] * gw[None, :]).ravel()
        cur = np.interp(tq - np.exp(uu), wt, wi, left=0.0, right=0.0)
        out[..., q] = sp(uu) @ (ww * cur)  # integral of (tau h)(u) I(t - tau) du
    return out
