"""NumPy restatement of the 2D-table event location objective.

TEST INFRASTRUCTURE ONLY: used by tests/ as the checker of the GPU loss and
gradient (adt_locate_loss_grad) -- never by the product path.

Follows tests/Eikonal/eikoloc.py: _interp (:119-145, bilinear with the cell
index clamped to the table), traveltime (:148-156, r = horizontal distance,
z = |z_event| - z_station), and the closure of invert (:169-204: position
clamped to the bounds, mean weighted Huber loss per phase, optional
double-difference term weighted by gamma).  Pinned: tests/test_oracle.py
checks it against tests/golden/loc_eikoloc.npz, the loss and autograd
gradient of the script's own _interp, traveltime and invert closure on seeded
tables and picks (generated by tests/golden/make_location_golden.py, which
executes those functions from the script's source).
"""
from __future__ import annotations

import numpy as np


def interp(T, r, z, r0, z0, h):
    m, n = T.shape
    ir0 = np.clip(np.floor((r - r0) / h), 0, m - 2).astype(np.int64)
    iz0 = np.clip(np.floor((z - z0) / h), 0, n - 2).astype(np.int64)
    ir1, iz1 = ir0 + 1, iz0 + 1
    x1, x2 = ir0 * h + r0, ir1 * h + r0
    y1, y2 = iz0 * h + z0, iz1 * h + z0
    q11, q12, q21, q22 = T[ir0, iz0], T[ir0, iz1], T[ir1, iz0], T[ir1, iz1]
    return 1 / (x2 - x1) / (y2 - y1) * (q11 * (x2 - r) * (y2 - z) + q21 * (r - x1) * (y2 - z) +
                                        q12 * (x2 - r) * (z - y1) + q22 * (r - x1) * (z - y1))


def huber(d):
    a = np.abs(d)
    return np.where(a < 1.0, 0.5 * d * d, a - 0.5)


def event_loss(params, sta, t, phase, w, tp, ts, r0, z0, h, bounds, gamma=0.0):
    """Loss of one event at params = (t0, x, y, z); phase 0 = P, 1 = S."""
    t0 = params[0]
    b = np.asarray(bounds, np.float64).reshape(3, 2)
    loc = np.maximum(np.minimum(np.asarray(params[1:], np.float64), b[:, 1]), b[:, 0])
    loc = np.nan_to_num(loc, nan=0.0)
    total = 0.0
    for ph, T in ((0, tp), (1, ts)):
        sel = phase == ph
        if not sel.any():
            continue
        s = sta[sel]
        r = np.sqrt(np.sum((loc[None, :2] - s[:, :2]) ** 2, axis=-1))
        z = np.abs(loc[2]) - s[:, 2]
        tt = interp(T, r, z, r0, z0, h)
        total += np.mean(huber(t[sel] - (t0 + tt)) * w[sel])
        if gamma != 0.0:
            dd_tt = tt[:, None] - tt[None, :]
            dd_t = t[sel][:, None] - t[sel][None, :]
            total += gamma * np.mean(huber(dd_tt - dd_t) * w[sel][:, None] * w[sel][None, :])
    return total
