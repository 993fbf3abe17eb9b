"""Event location from 2D (r, z) travel-time tables (tests/Eikonal/eikoloc.py).

The reference builds P and S travel-time tables on a radial grid (horizontal
distance r, depth z) with a 2D fast-sweeping solve from a surface source
(eikoloc.py:283-306), reads them by bilinear interpolation with the cell
index clamped to the table (:119-145), and locates every event
independently: origin time t0 and position (x, y, z), clamped to search
bounds, minimise the mean weighted Huber misfit of its P and S picks, plus
optionally a double-difference term (:157-206), with torch's L-BFGS.

Here the tables come from the 2D GPU solver (adt_eikonal, FP64), and all
events are located together: one launch of adt_locate_loss_grad evaluates
every event's loss and analytic gradient, and a batched L-BFGS on the host
(history 10, Armijo backtracking per event) updates all events at once.
torch's L-BFGS uses a strong-Wolfe line search instead; both converge to
the same local minimum of the same objective, not along the same path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib
from .ops import _ptr, eikonal


def traveltime_tables(zz, vp, vp_vs_ratio, rlim, zlim, h, edge=3):
    """P and S tables on the grid of eikoloc.py:270-306.

    zz, vp: the 1D model (depth knots, km, and P velocity, km/s), linearly
    interpolated; rlim, zlim: (min, max) of the horizontal distance and depth;
    edge: cells of margin below the minima.  Returns (tp, ts, r0, z0) with
    tp, ts of shape (len(rgrid), len(zgrid)) indexed [ir, iz], and r0, z0 the
    first grid coordinates; the source is the node (edge, edge)."""
    rgrid = np.arange(rlim[0] - edge * h, rlim[1], h)
    zgrid = np.arange(zlim[0] - edge * h, zlim[1], h)
    m, n = len(rgrid), len(zgrid)
    vp1d = np.interp(zgrid, zz, vp)
    out = []
    for v1d in (vp1d, vp1d / vp_vs_ratio):
        # the 2D op's array is (depth, width): rows z, columns r
        f = np.ascontiguousarray(np.repeat((1.0 / v1d)[:, None], m, axis=1))
        u = eikonal(f, edge + 1, edge + 1, h)
        out.append(np.ascontiguousarray(u.T))
    return out[0], out[1], float(rgrid[0]), float(zgrid[0])


def _picks(picks):
    offs = np.ascontiguousarray(picks["offs"], np.int64)
    sta = np.ascontiguousarray(picks["sta"], np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(picks["t"], np.float64)
    ph = picks["phase"]
    ph = np.array([0 if str(p).upper() == "P" else 1 for p in ph], np.int32) \
        if len(ph) and not np.issubdtype(np.asarray(ph).dtype, np.integer) \
        else np.ascontiguousarray(ph, np.int32)
    w = np.ascontiguousarray(picks.get("w", np.ones(len(t))), np.float64)
    return offs, sta, t, ph, w


class Locator:
    """Batched event location with P/S tables (see traveltime_tables).

    bounds: ((xmin, xmax), (ymin, ymax), (zmin, zmax)) for the clamp of the
    position; gamma: weight of the double-difference term (0 = off, as the
    reference's default add_eqt=False)."""

    def __init__(self, tp, ts, r0, z0, h, bounds, gamma=0.0):
        self.tp = np.ascontiguousarray(tp, np.float64)
        self.ts = np.ascontiguousarray(ts, np.float64)
        if self.tp.shape != self.ts.shape or self.tp.ndim != 2:
            raise ValueError("tables must be two arrays of the same (nr, nz) shape")
        self.r0, self.z0, self.h = float(r0), float(z0), float(h)
        self.bounds = np.ascontiguousarray(bounds, np.float64).reshape(6)
        self.gamma = float(gamma)

    def loss_grad(self, params, picks):
        """Loss (E,) and gradient (E, 4) at params (E, 4) = (t0, x, y, z)."""
        params = np.ascontiguousarray(params, np.float64).reshape(-1, 4)
        offs, sta, t, ph, w = _picks(picks)
        E = len(params)
        if len(offs) != E + 1:
            raise ValueError("picks['offs'] must have one entry per event plus one")
        loss = np.empty(E)
        grad = np.empty((E, 4))
        m, n = self.tp.shape
        check(lib().adt_locate_loss_grad(E, _ptr(params), _ptr(offs), _ptr(sta), _ptr(t),
                                         _ptr(ph), _ptr(w), _ptr(self.tp), _ptr(self.ts), m, n,
                                         self.r0, self.z0, self.h, _ptr(self.bounds), self.gamma,
                                         _ptr(loss), _ptr(grad)))
        return loss, grad

    def locate(self, picks, t0=0.0, loc0=(0.0, 0.0, 5.0), max_iter=1000, history=10,
               tol_grad=1e-7, tol_change=1e-9):
        """Locate every event; returns (params (E, 4), loss (E,), iterations (E,))."""
        offs = np.asarray(picks["offs"])
        E = len(offs) - 1
        x = np.tile(np.array([t0, *loc0], np.float64), (E, 1))
        f, g = self.loss_grad(x, picks)
        S = np.zeros((E, history, 4))
        Y = np.zeros((E, history, 4))
        rho = np.zeros((E, history))
        nh = np.zeros(E, np.int64)  # pairs stored per event (ring of `history`)
        active = np.abs(g).max(axis=1) > tol_grad
        iters = np.zeros(E, np.int64)
        for _ in range(max_iter):
            if not active.any():
                break
            # two-loop recursion, vectorised over events (newest pair first)
            q = -g.copy()
            alpha = np.zeros((E, history))
            for k in range(history):
                idx = (nh - 1 - k) % history
                ok = k < np.minimum(nh, history)
                s_k = S[np.arange(E), idx]
                y_k = Y[np.arange(E), idx]
                a = np.where(ok, rho[np.arange(E), idx] * np.einsum("ij,ij->i", s_k, q), 0.0)
                alpha[:, k] = a
                q -= a[:, None] * y_k
            last = (nh - 1) % history
            sy = np.einsum("ij,ij->i", S[np.arange(E), last], Y[np.arange(E), last])
            yy = np.einsum("ij,ij->i", Y[np.arange(E), last], Y[np.arange(E), last])
            scale = np.where((nh > 0) & (yy > 0), sy / np.where(yy > 0, yy, 1.0), 1.0)
            q *= scale[:, None]
            for k in reversed(range(history)):
                idx = (nh - 1 - k) % history
                ok = k < np.minimum(nh, history)
                s_k = S[np.arange(E), idx]
                y_k = Y[np.arange(E), idx]
                b = rho[np.arange(E), idx] * np.einsum("ij,ij->i", y_k, q)
                q += np.where(ok, alpha[:, k] - b, 0.0)[:, None] * s_k
            d = q
            dphi = np.einsum("ij,ij->i", g, d)
            bad = dphi >= 0  # not a descent direction: restart from steepest descent
            d[bad] = -g[bad]
            nh[bad] = 0
            dphi = np.einsum("ij,ij->i", g, d)
            # Armijo backtracking, every event its own step
            step = np.where(nh == 0, np.minimum(1.0, 1.0 / np.maximum(np.abs(g).sum(axis=1),
                                                                     1e-300)), 1.0)
            todo = active.copy()
            xn, fn, gn = x.copy(), f.copy(), g.copy()
            for _ls in range(60):
                if not todo.any():
                    break
                xt = np.where(todo[:, None], x + step[:, None] * d, x)
                ft, gt = self.loss_grad(xt, picks)
                ok = todo & (ft <= f + 1e-4 * step * dphi)
                xn[ok], fn[ok], gn[ok] = xt[ok], ft[ok], gt[ok]
                todo &= ~ok
                step = np.where(todo, step * 0.5, step)
            moved = active & ~todo
            s_new = xn - x
            y_new = gn - g
            sy_new = np.einsum("ij,ij->i", s_new, y_new)
            keep = moved & (sy_new > 1e-300)
            slot = nh % history
            S[keep, slot[keep]] = s_new[keep]
            Y[keep, slot[keep]] = y_new[keep]
            rho[keep, slot[keep]] = 1.0 / sy_new[keep]
            nh[keep] += 1
            iters += active
            done = ~moved | (np.abs(gn).max(axis=1) <= tol_grad) | (np.abs(fn - f) <= tol_change)
            x, f, g = np.where(active[:, None], xn, x), np.where(active, fn, f), \
                np.where(active[:, None], gn, g)
            active &= ~done
        return x, f, iters
