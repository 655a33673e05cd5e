"""Comparison of receiver traces [nr][NComp][Nt] between two runs, shared by the parity tests.

The recorded components split into two fields, E (the first nefcmp) and B.  A trace
carries a signal when its peak exceeds `floor` x the largest trace of its field; it is then
compared relative to its own peak.  The other traces are the components that vanish by
symmetry (Ey and Bz on the inline receivers of an x-directed source): they hold round-off
or interpolation residue of a zero field, and are compared relative to the largest trace of
their field.
"""
import numpy as np


def compare(got, exp, nefcmp, floor):
    """(worst error of the signal traces, worst error of the residue traces, {component: worst
    error}); NaN anywhere in either run counts as an infinite error."""
    if not (np.isfinite(got).all() and np.isfinite(exp).all()):
        return np.inf, np.inf, {}
    sig = res = 0.0
    per = {}
    for grp in (range(0, nefcmp), range(nefcmp, exp.shape[1])):
        grp = list(grp)
        if not grp:
            continue
        gmax = float(np.abs(exp[:, grp]).max())
        if gmax == 0.0:
            res = max(res, float(np.abs(got[:, grp]).max()))
            continue
        for c in grp:
            pk = np.abs(exp[:, c]).max(axis=1)
            d = np.abs(got[:, c] - exp[:, c]).max(axis=1)
            s = pk > floor * gmax
            e = 0.0
            if s.any():
                e = float((d[s] / pk[s]).max())
                sig = max(sig, e)
            if (~s).any():
                res = max(res, float(d[~s].max() / gmax))
            per[c] = e
    return sig, res, per


def check_fp64(got, exp, nefcmp, tol=1e-8):
    """The FP64 build against an FP64 run of the same scheme: every signal trace within `tol`
    of its peak (the survey's criterion is 1e-4 above a noise floor at 1e-6), the residue
    within `tol` of its field's largest trace."""
    sig, res, per = compare(got, exp, nefcmp, 1e-6)
    assert sig < tol and res < tol, (sig, res, per)
    return max(sig, res)


def check_fp32(got, exp, nefcmp, tol=1e-2):
    """FP32 production against FP64: the traces with a signal (peak above 1e-3 of their field's
    largest trace) within `tol` of their peak; the symmetry residue within `tol` of the field."""
    sig, res, per = compare(got, exp, nefcmp, 1e-3)
    assert sig < tol and res < tol, (sig, res, per)
    return sig, res, per


def field_error(got, exp, nefcmp):
    """max over the two fields of max|got - exp| / (largest trace of the field): the error on
    the survey's own amplitude scale, for runs whose weak traces carry noise of the reference
    (see tests/test_oracle_reference_kernels.py)."""
    if not (np.isfinite(got).all() and np.isfinite(exp).all()):
        return np.inf
    worst = 0.0
    for grp in (range(0, nefcmp), range(nefcmp, exp.shape[1])):
        grp = list(grp)
        if grp:
            gmax = float(np.abs(exp[:, grp]).max())
            if gmax > 0:
                worst = max(worst, float(np.abs(got[:, grp] - exp[:, grp]).max()) / gmax)
    return worst
