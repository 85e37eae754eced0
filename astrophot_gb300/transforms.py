"""Value <-> representation maps of the fitted parameters (float64, host side).

``boundaries`` / ``inv_boundaries`` / ``cyclic_boundaries`` of
``astrophot/utils/conversions/optimization.py:6-54``: two-sided limits use tan/arctan,
one-sided limits ``v - 1/(v - lim)``, cyclic parameters wrap with a modulo, and free
parameters are the identity.  The LM works in representation space.
"""

from __future__ import annotations

import math

import numpy as np

# (limits, cyclic) of each full-vector slot [cx, cy, q, PA, n, Re, Ie, F]
# (models/galaxy_model_object.py:44-53, sersic_model.py:61-65, flatsky_model.py:23-25)
SLOT_LIMITS = (
    ((None, None), False),
    ((None, None), False),
    ((0.0, 1.0), False),
    ((0.0, math.pi), True),
    ((0.36, 8.0), False),
    ((0.0, None), False),
    ((None, None), False),
    ((None, None), False),
)


def to_rep(limits, cyclic, val):
    lo, hi = limits
    val = np.asarray(val, dtype=np.float64)
    if cyclic:
        return lo + np.mod(val - lo, hi - lo)
    if lo is None and hi is None:
        return val
    if lo is None:
        return val - 1.0 / (val - hi)
    if hi is None:
        return val - 1.0 / (val - lo)
    return np.tan((val - lo) * np.pi / (hi - lo) - np.pi / 2)


def to_value(limits, cyclic, rep):
    lo, hi = limits
    rep = np.asarray(rep, dtype=np.float64)
    if cyclic:
        return lo + np.mod(rep - lo, hi - lo)
    if lo is None and hi is None:
        return rep
    if lo is None:
        return (rep + hi - np.sqrt((rep - hi) ** 2 + 4)) * 0.5
    if hi is None:
        return (rep + lo + np.sqrt((rep - lo) ** 2 + 4)) * 0.5
    return (np.arctan(rep) + np.pi / 2) * (hi - lo) / np.pi + lo


def drep_dvalue(limits, cyclic, rep):
    """d value / d representation (``d_inv_boundaries_dval``, optimization.py:40-47); 1 for
    cyclic and unbounded parameters."""
    lo, hi = limits
    rep = np.asarray(rep, dtype=np.float64)
    if cyclic or (lo is None and hi is None):
        return np.ones_like(rep)
    if lo is None:
        return 0.5 - 0.5 * (rep - hi) / np.sqrt((rep - hi) ** 2 + 4)
    if hi is None:
        return 0.5 + 0.5 * (rep - lo) / np.sqrt((rep - lo) ** 2 + 4)
    return (hi - lo) / (np.pi * (rep**2 + 1))


def slots_to_rep(values: np.ndarray, free_mask: int) -> np.ndarray:
    """[n, 8] value-space rows -> [n, n_free] representation rows (fitted slots, in order)."""
    values = np.atleast_2d(np.asarray(values, dtype=np.float64))
    cols = [to_rep(*SLOT_LIMITS[i], values[:, i]) for i in range(8) if free_mask & (1 << i)]
    return np.stack(cols, axis=1) if cols else np.zeros((values.shape[0], 0))


def rep_to_slots(rep: np.ndarray, fixed: np.ndarray, free_mask: int) -> np.ndarray:
    """[n, n_free] representation rows + [n, 8] fixed values -> [n, 8] value rows."""
    rep = np.atleast_2d(np.asarray(rep, dtype=np.float64))
    out = np.array(np.atleast_2d(fixed), dtype=np.float64, copy=True)
    k = 0
    for i in range(8):
        if free_mask & (1 << i):
            out[:, i] = to_value(*SLOT_LIMITS[i], rep[:, k])
            k += 1
    return out
