"""The reference's Julia API (src/eikonal_op.jl) over the GB300 library.

eikonal(f, srcx, srcy, h)                        -- src/eikonal_op.jl:3-21
eikonal3d(u0, f, h, m, n, l, tol, verbose)       -- src/eikonal_op.jl:24-32
and their gradient ops (EikonalGrad, EikonalThreeDGrad) as eikonal_grad /
eikonal3d_grad.  Same argument order and meaning: srcx/srcy are 1-based, f for
eikonal has shape (n+1, m+1) (depth x width), arrays for eikonal3d have shape
(m, n, l) or are flat in C order.  Invalid input raises AdtError
(ADT_EINVAL) instead of reaching the solver.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (ADT_ADJ_AUTO, ADT_ADJ_CAUSAL, ADT_ADJ_SWEEPS, ADT_F32, ADT_F64, AdtError, BatchOpts,
                   BatchStats, SolveStatus, check, lib)

__all__ = ["eikonal", "eikonal_grad", "eikonal_batch", "eikonal3d", "eikonal3d_grad", "Batch3D",
           "AdtError", "ADT_F32", "ADT_F64"]


def _f64(a, name):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if not a.flags.c_contiguous:
        raise AdtError(-1, f"{name} must be contiguous")
    return a


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------------- 2D ----
def eikonal(f, srcx: int, srcy: int, h: float, return_status: bool = False):
    """Travel times on the (n+1) x (m+1) grid of slowness f from the node
    (srcx, srcy) (1-based, srcx along the width)."""
    f = _f64(f, "f")
    if f.ndim != 2:
        raise AdtError(-1, "eikonal: f must be 2-D (n+1, m+1)")
    n1, m1 = f.shape
    u = np.empty_like(f)
    st = SolveStatus()
    check(lib().adt_eikonal(_ptr(f), m1 - 1, n1 - 1, int(srcx), int(srcy), float(h), _ptr(u),
                            C.byref(st)))
    return (u, st) if return_status else u


def eikonal_grad(grad_u, u, f, srcx: int, srcy: int, h: float):
    """dL/df for dL/du = grad_u at the converged u (EikonalGrad)."""
    f = _f64(f, "f")
    n1, m1 = f.shape
    gu = _f64(grad_u, "grad_u").reshape(f.shape)
    uu = _f64(u, "u").reshape(f.shape)
    g = np.empty_like(f)
    check(lib().adt_eikonal_grad(_ptr(gu), _ptr(uu), _ptr(f), m1 - 1, n1 - 1, int(srcx), int(srcy),
                                 float(h), _ptr(g)))
    return g


def eikonal_batch(f, srcx, srcy, h: float):
    """Many 2D solves on one grid; returns (count, n+1, m+1) travel times."""
    f = _f64(f, "f")
    n1, m1 = f.shape
    sx = np.ascontiguousarray(srcx, np.int64)
    sy = np.ascontiguousarray(srcy, np.int64)
    u = np.empty((len(sx), n1, m1))
    st = (SolveStatus * len(sx))()
    check(lib().adt_eikonal_batch(_ptr(f), m1 - 1, n1 - 1, len(sx), _ptr(sx), _ptr(sy), float(h),
                                  _ptr(u), st))
    return u, [(s.iters, s.converged) for s in st]


# ------------------------------------------------------------------- 3D ----
def _shape3(a, m, n, l, name):
    a = _f64(a, name)
    if a.size != m * n * l:
        raise AdtError(-1, f"{name} has {a.size} entries, expected m*n*l = {m * n * l}")
    return a.reshape(m, n, l)


def eikonal3d(u0, f, h: float, m: int, n: int, l: int, tol: float, verbose: bool = False,
              return_status: bool = False):
    """Travel times for initial values u0 and slowness f on an m x n x l grid
    (FP64, the reference's stopping rule, at most 20 iterations)."""
    u0 = _shape3(u0, m, n, l, "u0")
    f = _shape3(f, m, n, l, "f")
    u = np.empty_like(u0)
    st = SolveStatus()
    check(lib().adt_eikonal_three_d(_ptr(u0), _ptr(f), float(h), int(m), int(n), int(l), float(tol),
                                    int(bool(verbose)), _ptr(u), C.byref(st)))
    return (u, st) if return_status else u


def eikonal3d_grad(grad_u, u, u0, f, h: float, m: int, n: int, l: int, tol: float = 0.0,
                   verbose: bool = False):
    """(grad_u0, grad_f) of EikonalThreeDGrad."""
    gu = _shape3(grad_u, m, n, l, "grad_u")
    uu = _shape3(u, m, n, l, "u")
    u0 = _shape3(u0, m, n, l, "u0")
    f = _shape3(f, m, n, l, "f")
    g0 = np.empty_like(uu)
    gf = np.empty_like(uu)
    check(lib().adt_eikonal_three_d_grad(_ptr(gu), _ptr(uu), _ptr(u0), _ptr(f), float(h), int(m),
                                         int(n), int(l), float(tol), int(bool(verbose)), _ptr(g0),
                                         _ptr(gf)))
    return g0, gf


# --------------------------------------------------------------- batch -----
class Batch3D:
    """Batched misfit + slowness gradient for many sources on several fields.

    fields:   list of (m, n, l, h)
    stations: list of (S_f, 3) arrays of fractional 0-based node coordinates
    solve_field, src_xyz: per solve, the field index and the source position
    The near-source initial values follow scripts/gene_obs.jl:42-51 (the
    evaluation's slowness at the source's (ceil x, ceil y) column, one value
    per depth plane); set_source_velocity switches to scripts/inversion.jl's
    rule (a fixed vel0 per node).
    Each evaluation (run) takes the slowness of every field, t_obs and weight
    (concatenated per solve over the stations of its field; t_obs == -1 is a
    missing pick) and returns (misfit, t_pred, [grad per field], status).
    Options are the fields of adt_batch_opts (include/adtomo_gpu.h); in
    particular wake_tol / adj_wake_tol (FP32 only, default 0 = exact brick
    skipping) let bricks that moved by at most that much (seconds; relative
    for the adjoint) leave their neighbours asleep.  adj_solver "causal"
    (ADT_ADJ_CAUSAL) solves each adjoint system once in reverse causal order
    instead of by sweeps ("sweeps", ADT_ADJ_SWEEPS); "auto" (the default)
    starts with the causal solve and, in FP32, lets autotune() keep whichever
    of the two is faster on the uploaded inputs (stats().adj_solver).
    """

    def __init__(self, fields, stations, solve_field, src_xyz, precision=ADT_F32, tol=1e-6,
                 max_iter=200, adj_max_iter=200, ref_compat=False, near_src_f64=2, chunk=0,
                 bk=0, warps=0, groups=0, use_graph=True, wake_tol=0.0, adj_wake_tol=0.0,
                 adj_order_filter=True, fwd_order_filter=True, overlap_chunks=False,
                 adj_warps=0, adj_groups=0, adj_solver="auto"):
        L = lib()
        self._L = L
        self.fields = [tuple(x) for x in fields]
        dims = np.array([[f[0], f[1], f[2]] for f in self.fields], np.int32).ravel()
        hs = np.array([f[3] for f in self.fields], np.float64)
        self.nsta = np.array([len(s) for s in stations], np.int32)
        sta = (np.concatenate([np.asarray(s, np.float64).reshape(-1, 3) for s in stations]).ravel()
               if len(stations) and self.nsta.sum() else np.zeros(3))
        self.solve_field = np.ascontiguousarray(solve_field, np.int32)
        src = np.ascontiguousarray(src_xyz, np.float64).reshape(-1, 3)
        self.n_solves = len(self.solve_field)
        self.n_obs = int(sum(self.nsta[f] for f in self.solve_field if 0 <= f < len(self.nsta)))
        self.ncell = [f[0] * f[1] * f[2] for f in self.fields]
        o = BatchOpts()
        L.adt_batch_opts_default(C.byref(o))
        o.precision, o.tol, o.max_iter, o.adj_max_iter = precision, tol, max_iter, adj_max_iter
        o.ref_compat, o.near_src_f64, o.chunk = int(ref_compat), near_src_f64, chunk
        o.bk, o.warps, o.groups, o.use_graph = bk, warps, groups, int(use_graph)
        o.wake_tol, o.adj_wake_tol = wake_tol, adj_wake_tol
        o.adj_order_filter = int(bool(adj_order_filter))
        o.fwd_order_filter = int(bool(fwd_order_filter))
        o.overlap_chunks = int(bool(overlap_chunks))
        o.adj_warps, o.adj_groups = adj_warps, adj_groups
        solvers = {"sweeps": ADT_ADJ_SWEEPS, "causal": ADT_ADJ_CAUSAL, "auto": ADT_ADJ_AUTO}
        o.adj_solver = solvers[adj_solver] if isinstance(adj_solver, str) else int(adj_solver)
        self._keep = (dims, hs, sta, src)
        h = C.c_void_p()
        check(L.adt_batch_create(C.byref(h), len(self.fields), _ptr(dims), _ptr(hs),
                                 _ptr(self.nsta), _ptr(sta), self.n_solves,
                                 _ptr(self.solve_field), _ptr(src), C.byref(o)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.adt_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _inputs(self, slowness, t_obs, weight):
        # one field: the caller's buffer itself (no host copy, so pinned memory stays pinned)
        slow = (_f64(slowness[0], "slowness").ravel() if len(slowness) == 1 else
                np.concatenate([_f64(s, "slowness").ravel() for s in slowness]))
        if slow.size != sum(self.ncell):
            raise AdtError(-1, "slowness size does not match the fields")
        t_obs = _f64(t_obs, "t_obs").ravel()
        weight = _f64(weight, "weight").ravel()
        if t_obs.size != self.n_obs or weight.size != self.n_obs:
            raise AdtError(-1, f"t_obs/weight need {self.n_obs} entries")
        return slow, t_obs, weight

    def _split(self, grad):
        out, off = [], 0
        for (m, n, l, _), nc in zip(self.fields, self.ncell):
            out.append(grad[off:off + nc].reshape(m, n, l))
            off += nc
        return out

    def run(self, slowness, t_obs, weight, out=None):
        """One evaluation end to end through adt_batch_run (host buffers).
        out: optional (t_pred, grad) float64 buffers of n_obs and total-cell
        entries to write into (e.g. pinned memory) instead of new arrays."""
        slow, t_obs, weight = self._inputs(slowness, t_obs, weight)
        mis = C.c_double(0)
        if out is None:
            tp, gr = np.empty(self.n_obs), np.empty(sum(self.ncell))
        else:
            tp, gr = out
            if (tp.dtype != np.float64 or gr.dtype != np.float64 or not tp.flags.c_contiguous or
                    not gr.flags.c_contiguous or tp.size != self.n_obs or
                    gr.size != sum(self.ncell)):
                raise AdtError(-1, "out must be contiguous float64 (t_pred, grad) buffers "
                                   f"of {self.n_obs} and {sum(self.ncell)} entries")
        st = (SolveStatus * self.n_solves)()
        check(self._L.adt_batch_run(self._h, _ptr(slow), _ptr(t_obs), _ptr(weight), C.byref(mis),
                                    _ptr(tp), _ptr(gr), st))
        return mis.value, tp, self._split(gr), st

    # device-resident use
    def upload(self, slowness=None, t_obs=None, weight=None):
        slow = (np.concatenate([_f64(s, "slowness").ravel() for s in slowness])
                if slowness is not None else None)
        to = _f64(t_obs, "t_obs").ravel() if t_obs is not None else None
        w = _f64(weight, "weight").ravel() if weight is not None else None
        self._upl = (slow, to, w)
        check(self._L.adt_batch_upload(self._h, _ptr(slow) if slow is not None else None,
                                       _ptr(to) if to is not None else None,
                                       _ptr(w) if w is not None else None))

    def run_resident(self):
        check(self._L.adt_batch_run_resident(self._h))

    def set_source_velocity(self, vel0):
        """Near-source initial values from the fixed velocity models vel0 (one
        per field): r * h / vel0[node] at the 8 nodes around each source, the
        rule of scripts/inversion.jl:52-60 (adt_batch_set_source_velocity).
        None returns to the default rule of scripts/gene_obs.jl:42-51, which
        uses the evaluation's own slowness."""
        if vel0 is None:
            check(self._L.adt_batch_set_source_velocity(self._h, None))
            return
        v = np.concatenate([_f64(a, "vel0").ravel() for a in vel0])
        if v.size != sum(self.ncell):
            raise AdtError(-1, "vel0 size does not match the fields")
        check(self._L.adt_batch_set_source_velocity(self._h, _ptr(v)))

    def download(self):
        mis = C.c_double(0)
        tp = np.empty(self.n_obs)
        gr = np.empty(sum(self.ncell))
        st = (SolveStatus * self.n_solves)()
        check(self._L.adt_batch_download(self._h, C.byref(mis), _ptr(tp), _ptr(gr), st))
        return mis.value, tp, self._split(gr), st

    def stream(self) -> int:
        return self._L.adt_batch_stream(self._h) or 0

    def autotune(self, reps: int = 2) -> BatchStats:
        """Time the sweep kernels over candidate launch shapes on the uploaded
        inputs and keep the fastest (adt_batch_autotune); returns the stats
        of the chosen shape."""
        check(self._L.adt_batch_autotune(self._h, int(reps)))
        return self.stats()

    def stats(self) -> BatchStats:
        s = BatchStats()
        check(self._L.adt_batch_stats_get(self._h, C.byref(s)))
        return s
