"""Waveform post-processing of impulse traces (tcsem_fdtd_gb300.waveform).

The impulse response h(t) = t^(-5/2) exp(-a/t) has the shape of a late-time
diffusive field and closed-form integrals:
  integral_t^inf h = a^(-3/2) * Gamma(3/2) * P(3/2, a/t)   (P: regularised lower gamma),
so the step-off response and the response to a box current of width w,
y(t) = integral_{t-w}^{t} h, are known exactly.  Sampled like Receiver.in
(100 log-spaced times over 3 decades) the step-off and the box, long-box and
ramp-off responses match within 1e-5 of their peaks (measured: 4e-7, 1e-7,
3e-8, 5e-8).
"""
import numpy as np
import pytest

from tcsem_fdtd_gb300 import waveform

scipy_special = pytest.importorskip("scipy.special")

A = 0.05


def h(t):
    return t ** -2.5 * np.exp(-A / t)


def tail(t):
    """integral_t^inf h."""
    return A ** -1.5 * scipy_special.gamma(1.5) * scipy_special.gammainc(1.5, A / t)


def test_sampling_times_follow_receiver_in(tmp_path):
    (tmp_path / "Receiver.in").write_text("0.01 10.0\n100 1\n1 1 0 1 1 1\n1\n1 0 0 0\n")
    t = waveform.sampling_times(tmp_path)
    assert len(t) == 100 and t[0] == pytest.approx(0.01) and t[-1] == pytest.approx(10.0)
    assert np.allclose(np.diff(np.log10(t)), 3.0 / 99)
    (tmp_path / "Receiver.in").write_text("0.5 2.0\n4 0\n1 1 0 1 1 1\n1\n1 0 0 0\n")
    assert np.allclose(waveform.sampling_times(tmp_path), [0.5, 1.0, 1.5, 2.0])


def test_step_off_of_a_closed_form_impulse():
    t = np.logspace(-2, 1, 100)
    traces = np.stack([h(t), -2.0 * h(t)])[None]  # [1, 2, Nt]: a scale and a sign change
    got = waveform.step_off(t, traces)
    exp = np.stack([tail(t), -2.0 * tail(t)])[None]
    assert got.shape == traces.shape
    assert np.abs(got - exp).max() / np.abs(exp).max() <= 1e-4


def test_step_off_with_the_pulse_delay():
    """Traces sampled at absolute times t respond at delays t - 3 sigma_t."""
    d = 1.5e-3
    t = np.logspace(-2, 1, 100)
    got = waveform.step_off(t, h(t - d), delay=d)
    assert np.abs(got - tail(t - d)).max() / tail(t - d).max() <= 1e-4


def test_box_current_of_a_closed_form_impulse():
    t = np.logspace(-2, 1, 100)
    w = 0.05
    out = np.logspace(-1.0, 0.5, 20)
    got = waveform.convolve(t, h(t)[None], [0.0, w], [1.0, 1.0], out_times=out)[0]
    exp = tail(out - w) - tail(out)
    assert np.abs(got - exp).max() / np.abs(exp).max() <= 1e-5


def test_long_box_converges_to_step_off():
    """A current on for a long time and switched off at 0 gives the step-off response."""
    t = np.logspace(-2, 1, 100)
    on = 1e3
    out = t[40:80]
    got = waveform.convolve(t, h(t)[None], [-on, 0.0], [1.0, 1.0], out_times=out)[0]
    # the convolution stops at the last sampling time; the step-off adds the tail beyond it
    exp = tail(out) - tail(t[-1])
    assert np.abs(got - exp).max() / np.abs(exp).max() <= 1e-5


def test_ramp_off_against_adaptive_quadrature():
    """Current on for a long time, then falling linearly to 0 over r."""
    quad = pytest.importorskip("scipy.integrate").quad
    t = np.logspace(-2, 1, 100)
    r = 0.02
    wt, wi = [-1e3, 0.0, r], [1.0, 1.0, 0.0]
    out = np.logspace(-1.0, 0.5, 15)
    got = waveform.convolve(t, h(t)[None], wt, wi, out_times=out)[0]

    def y(tq):
        f = lambda tau: h(tau) * np.interp(tq - tau, wt, wi, left=0.0, right=0.0)
        return quad(f, t[0], t[-1], points=[tq - r, tq], limit=500)[0]

    exp = np.array([y(tq) for tq in out])
    assert np.abs(got - exp).max() / np.abs(exp).max() <= 1e-5


def test_tail_of_a_pure_power_law_and_of_undecided_traces():
    t = np.logspace(-2, 1, 60)
    traces = np.stack([t ** -3.0, np.zeros_like(t), np.where(t < 9.0, t ** -3.0, -(t ** -3.0))])
    got = waveform.step_off(t, traces)
    assert np.abs(got[0] - 0.5 * t ** -2.0).max() / (0.5 * t[0] ** -2.0) <= 1e-5
    assert np.all(got[1] == 0)
    assert np.all(np.isnan(got[2]))  # the sign still changes within the last samples: no finite tail


def test_rejects_unordered_times():
    with pytest.raises(ValueError):
        waveform.step_off(np.array([0.1, 0.05, 0.2]), np.ones(3))
    with pytest.raises(ValueError):
        waveform.convolve(np.array([0.1, 0.2, 0.3]), np.ones(3), [0.0, 0.0], [1.0, 1.0])
