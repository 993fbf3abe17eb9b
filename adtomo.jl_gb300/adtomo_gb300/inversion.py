"""Host driver of the travel-time inversion (the loop around the hot path).

scripts/inversion.jl builds, for every station, one eikonal3d solve with the
station as the source (reciprocity), samples the travel times at the events,
forms the weighted misfit  sum qua * (uobs - t)^2  over the picks
(uobs == -1 marks a missing pick), adds the smoothness penalty
lambda_p * sum |v - S v| (S: circular box mean, :107-121) and minimises over a
sigmoid-bounded velocity  v = 2 sigmoid(x) - 1 + vel0  (:42-43) with
Optim's L-BFGS and BackTracking line search (src/mpi_optimize.jl:3-72).

Here the misfit and its slowness gradient come from one batched GPU plan
(adt_batch_*), the penalty from adt_smooth_l1 (both in libadtomo_gpu.so),
and the optimiser stays on the host, as in the reference.  Coordinates are
0-based fractional node positions (Julia's 1-based x becomes x - 1).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Callable

import numpy as np

from ._lib import ADT_F32, check, lib
from .ops import Batch3D, _f64, _ptr


def smooth_l1(v, sh: int, sv: int, lam: float = 1.0, grad: bool = True):
    """lam * sum |v - S v| and its gradient (scripts/inversion.jl:107-121).

    v: (m, n, l) model, C order.  S: mean over an sh x sh x sv box centred on
    each cell, wrapping around the grid edges.  Returns (penalty, grad or None).
    """
    v = _f64(v, "v")
    if v.ndim != 3:
        raise ValueError("v must be (m, n, l)")
    m, n, l = v.shape
    pen = C.c_double(0.0)
    g = np.empty_like(v) if grad else None
    check(lib().adt_smooth_l1(_ptr(v), m, n, l, sh, sv, lam, C.byref(pen),
                              _ptr(g) if grad else None))
    return pen.value, g


# ------------------------------------------------------------------ L-BFGS
def _backtracking(phi, alpha, phi0, dphi0, c1=1e-4, rho_hi=0.5, rho_lo=0.1, iterations=1000):
    """Armijo backtracking with quadratic, then cubic, interpolation of the
    step (the BackTracking line search Optim's LBFGS uses in
    src/mpi_optimize.jl:39-42: order 3, c_1 = 1e-4, step shrink kept in
    [0.1, 0.5] per trial).  phi(a) returns the objective at step a.
    Returns (a, phi(a))."""
    a1 = a2 = alpha
    phi_prev = phi0
    phi2 = phi(a2)
    tries = 0
    while not np.isfinite(phi2) and tries < 50:  # first reach a finite value
        tries += 1
        a1, a2 = a2, a2 / 2
        phi2 = phi(a2)
    it = 0
    while phi2 > phi0 + c1 * a2 * dphi0:
        it += 1
        if it > iterations:
            raise RuntimeError("line search did not find a sufficient decrease")
        if it == 1:  # minimiser of the quadratic through phi(0), phi'(0), phi(a2)
            a_new = -(dphi0 * a2 * a2) / (2.0 * (phi2 - phi0 - dphi0 * a2))
        else:  # minimiser of the cubic through phi(0), phi'(0), phi(a1), phi(a2)
            r2 = phi2 - phi0 - dphi0 * a2
            r1 = phi_prev - phi0 - dphi0 * a1
            div = 1.0 / (a1 * a1 * a2 * a2 * (a2 - a1))
            ca = (a1 * a1 * r2 - a2 * a2 * r1) * div
            cb = (-a1 ** 3 * r2 + a2 ** 3 * r1) * div
            if abs(ca) <= np.finfo(float).eps:
                a_new = dphi0 / (2.0 * cb)
            else:
                disc = max(cb * cb - 3.0 * ca * dphi0, 0.0)
                a_new = (-cb + np.sqrt(disc)) / (3.0 * ca)
        a1 = a2
        hi, lo = a2 * rho_hi, a2 * rho_lo
        a_new = hi if not np.isfinite(a_new) else min(a_new, hi)
        a2 = max(a_new, lo)
        phi_prev, phi2 = phi2, phi(a2)
    return a2, phi2


def lbfgs(fg: Callable, x0, m: int = 10, iterations: int = 1000, g_tol: float = 1e-8,
          callback: Callable | None = None):
    """Minimise f with L-BFGS (history m, initial inverse Hessian scaled by
    s'y / y'y) and the backtracking line search above, starting every line
    search at step 1 (Optim's LBFGS with InitialStatic + BackTracking, as
    src/mpi_optimize.jl configures it).  fg(x) returns (f, grad).
    Stops after `iterations` iterations or when max|grad| <= g_tol.
    callback(k, x, f, g) runs after every iteration; returning True stops.
    Returns (x, f, history) with history the list of f after each iteration."""
    x = np.array(x0, dtype=np.float64, copy=True).ravel()
    cache = {}

    def eval_at(xx):
        f, g = fg(xx)
        cache["x"], cache["f"], cache["g"] = xx, float(f), np.asarray(g, np.float64).ravel()
        return cache["f"]

    f = eval_at(x)
    g = cache["g"]
    S, Y = [], []
    hist = []
    for k in range(iterations):
        if np.max(np.abs(g)) <= g_tol:
            break
        # two-loop recursion
        q = -g.copy()
        alphas = []
        for s, y in zip(reversed(S), reversed(Y)):
            a = np.dot(s, q) / np.dot(y, s)
            alphas.append(a)
            q -= a * y
        if S:
            q *= np.dot(S[-1], Y[-1]) / np.dot(Y[-1], Y[-1])
        for (s, y), a in zip(zip(S, Y), reversed(alphas)):
            b = np.dot(y, q) / np.dot(y, s)
            q += (a - b) * s
        d = q
        dphi0 = float(np.dot(g, d))
        if not dphi0 < 0.0:  # not a descent direction: restart from steepest descent
            S.clear()
            Y.clear()
            d = -g
            dphi0 = float(np.dot(g, d))
        alpha, f_new = _backtracking(lambda a: eval_at(x + a * d), 1.0, f, dphi0)
        if cache.get("x") is None or not np.array_equal(cache["x"], x + alpha * d):
            eval_at(x + alpha * d)
        x_new, g_new = cache["x"], cache["g"]
        s, y = x_new - x, g_new - g
        if np.dot(s, y) > 0.0:  # keep the pair only with positive curvature
            S.append(s)
            Y.append(y)
            if len(S) > m:
                S.pop(0)
                Y.pop(0)
        x, f, g = x_new, cache["f"], g_new
        hist.append(f)
        if callback is not None and callback(k + 1, x, f, g):
            break
    return x, f, hist


# -------------------------------------------------------------- inversion
def _sigmoid(x):
    return 0.5 * (1.0 + np.tanh(0.5 * x))


class TravelTimeInversion:
    """The objective and driver of scripts/inversion.jl on one GPU.

    grid: (m, n, l, h); vel0: (m, n, l) starting velocity (km/s);
    stations: (S, 3), events: (E, 3) 0-based fractional node coordinates;
    uobs, qua: (S, E) picked times (-1 = missing) and weights.
    Every station is one source; the travel times are sampled at the events.
    lambda_p, smooth_hor, smooth_ver: the smoothness penalty (smooth_* odd box
    sizes; lambda_p = 0 disables it).  tol, max_iter: forward stopping rule
    (the script passes tol = 1e-3 to eikonal3d, whose cap is 20 iterations).
    The near-source initial values come from vel0 for the whole run, as in
    the script (:52-60).  autotune > 0 (FP32): time the plan's launch shapes
    on the starting model with that many evaluations per candidate first.
    """

    def __init__(self, grid, vel0, stations, events, uobs, qua, lambda_p=0.0, smooth_hor=1,
                 smooth_ver=1, tol=1e-3, max_iter=20, precision=ADT_F32, autotune=0, **plan_kw):
        m, n, l, h = grid
        self.shape = (int(m), int(n), int(l))
        self.vel0 = _f64(vel0, "vel0").reshape(self.shape)
        if not np.all(self.vel0 > 0):
            raise ValueError("vel0 must be > 0")
        self.stations = np.asarray(stations, np.float64).reshape(-1, 3)
        self.events = np.asarray(events, np.float64).reshape(-1, 3)
        S, E = len(self.stations), len(self.events)
        self.uobs = np.asarray(uobs, np.float64).reshape(S, E)
        self.qua = np.asarray(qua, np.float64).reshape(S, E)
        self.lambda_p, self.sh, self.sv = float(lambda_p), int(smooth_hor), int(smooth_ver)
        self.plan = Batch3D([(m, n, l, h)], [self.events], np.zeros(S, np.int32), self.stations,
                            precision=precision, tol=tol, max_iter=max_iter, **plan_kw)
        self.plan.set_source_velocity([self.vel0])
        if autotune and precision == ADT_F32:
            # launch shapes timed on the starting model (adt_batch_autotune, `autotune` reps)
            self.plan.upload([1.0 / self.vel0], self.uobs, self.qua)
            self.plan.autotune(reps=int(autotune))
        self.evaluations = 0
        self.last_status = None

    def close(self):
        self.plan.close()

    def velocity(self, x):
        return 2.0 * _sigmoid(np.asarray(x, np.float64).reshape(self.shape)) - 1.0 + self.vel0

    def loss_and_grad(self, x):
        """(loss, d loss / d x) at the parameters x (shape of vel0)."""
        x = np.asarray(x, np.float64).reshape(self.shape)
        sig = _sigmoid(x)
        v = 2.0 * sig - 1.0 + self.vel0
        if not np.all(v > 0):
            return np.inf, np.zeros(x.size)
        mis, _, grads, status = self.plan.run([1.0 / v], self.uobs, self.qua)
        self.evaluations += 1
        self.last_status = status
        dv = -grads[0].reshape(self.shape) / (v * v)
        loss = mis
        if self.lambda_p != 0.0:
            pen, gp = smooth_l1(v, self.sh, self.sv, self.lambda_p)
            loss += pen
            dv += gp
        return loss, (dv * 2.0 * sig * (1.0 - sig)).ravel()

    def optimize(self, x0=None, iterations=10, steps=0, checkpoint_dir=None, callback=None):
        """L-BFGS over x (zeros = vel0).  Every `steps` iterations x is saved
        to checkpoint_dir/iter_<k>.npy (the reference writes iter_<k>.h5,
        src/mpi_optimize.jl:22-27).  Returns (x, loss, history)."""
        x0 = np.zeros(self.shape) if x0 is None else np.asarray(x0, np.float64)

        def cb(k, x, f, g):
            if steps and checkpoint_dir and k % steps == 0:
                os.makedirs(checkpoint_dir, exist_ok=True)
                np.save(os.path.join(checkpoint_dir, f"iter_{k}.npy"), x.reshape(self.shape))
            return callback(k, x, f, g) if callback else False

        x, f, hist = lbfgs(self.loss_and_grad, x0, iterations=iterations, callback=cb)
        return x.reshape(self.shape), f, hist
