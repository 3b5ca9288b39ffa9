"""Tolerance of the fast-fp kernels against the oracle (test helper).

Bar, per field: max |got - oracle| over the interior <= 1e-12 * max |oracle|
(normwise relative error). The pointwise relative error |d| / max(|oracle|,
1e-300) is bounded by 1e-9 where the oracle is not itself a cancellation
residue (|oracle| >= 1e-3 of the field's maximum).
"""

import numpy as np

NORMWISE = 1e-12
POINTWISE = 1e-9


def errors(got, ref):
    """(normwise, pointwise) relative errors of one field."""
    d = np.abs(got - ref)
    scale = np.abs(ref).max()
    if scale == 0:  # an exactly vanishing tendency (e.g. one periodic cell): the residue itself is the error
        return float(d.max()), 0.0
    normwise = d.max() / scale
    big = np.abs(ref) >= 1e-3 * scale
    pointwise = (d[big] / np.maximum(np.abs(ref[big]), 1e-300)).max()
    return float(normwise), float(pointwise)


def check(got, ref, name=""):
    assert np.isfinite(got).all(), f"{name}: a point was not written"
    normwise, pointwise = errors(got, ref)
    assert normwise <= NORMWISE, f"{name}: normwise relative error {normwise:.3e}"
    assert pointwise <= POINTWISE, f"{name}: pointwise relative error {pointwise:.3e}"
    return normwise, pointwise
