"""ctypes wrapper around the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check in
__graft_entry__.py and by the cpu_baseline / reference arm of bench.py, always
as the checker or as the timed CPU baseline -- never by the product path.

Parity status: pinned against the reference's own sources compiled into
oracle/_ref (see tests/golden/make_golden.py).

Array conventions follow the reference ops:
  2D: f has shape (n+1, m+1) (depth x width); flat index j*(m+1)+i.
  3D: arrays have shape (m, n, l) in C order; flat index i*n*l + j*l + k.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_ip64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and _ref/libadtomo_ref.so when ref=True)."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", _HERE] + targets, check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_eik2d_forward.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, _dp,
                                        C.POINTER(C.c_int)]
        L.orc_eik2d_forward.restype = C.c_int
        L.orc_eik2d_backward.argtypes = [_dp, _dp, _dp, C.c_int, C.c_int, C.c_double, C.c_int,
                                         C.c_int, _dp]
        L.orc_eik2d_backward.restype = C.c_int
        L.orc_eik3d_forward.argtypes = [_dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double,
                                        C.c_int, _dp, C.POINTER(C.c_double)]
        L.orc_eik3d_forward.restype = C.c_int
        L.orc_eik3d_backward.argtypes = [_dp, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int,
                                         _dp, _dp]
        L.orc_eik3d_backward.restype = C.c_int
        L.orc_assemble.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int64, _ip64, _ip64, _dp, _dp]
        L.orc_assemble.restype = C.c_int64
        L.orc_src_u0.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_int, _dp]
        L.orc_src_u0.restype = None
        L.orc_sample.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                 C.c_double, C.c_void_p, C.c_void_p]
        L.orc_sample.restype = C.c_double
        L.orc_batch_misfit_grad.argtypes = [C.c_int, _ip32, _dp, _dp, _ip32, _dp, C.c_int, _ip32,
                                            _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                            C.c_int, C.c_void_p, C.POINTER(C.c_double), _dp, _dp,
                                            _ip32]
        L.orc_batch_misfit_grad.restype = C.c_int
        _LIB = L
    return _LIB


def ref_lib(required: bool = True):
    """The reference's own functions compiled by `make ref` (this container only)."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libadtomo_ref.so")
        if not os.path.exists(path):
            if not required:
                return None
            build(ref=True)
        R = C.CDLL(path)
        R.ref_eik2d_forward.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int]
        R.ref_eik2d_backward.argtypes = [_dp, _dp, _dp, _dp, C.c_int, C.c_int, C.c_double, C.c_int,
                                         C.c_int]
        R.ref_eik3d_forward.argtypes = [_dp, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int,
                                        C.c_double, C.c_int]
        R.ref_eik3d_backward.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                         C.c_int]
        for fn in (R.ref_eik2d_forward, R.ref_eik2d_backward, R.ref_eik3d_forward,
                   R.ref_eik3d_backward):
            fn.restype = None
        _REF = R
    return _REF


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ---------------------------------------------------------------- 2D ------
def eik2d_forward(f, ix, jx, h):
    """Travel times for slowness f (shape (n+1, m+1)); ix, jx are 0-based."""
    f = _c(f)
    n1, m1 = f.shape
    u = np.empty_like(f)
    it = C.c_int(0)
    conv = lib().orc_eik2d_forward(f.ravel(), m1 - 1, n1 - 1, float(h), int(ix), int(jx),
                                   u.ravel(), C.byref(it))
    return u, it.value, bool(conv)


def eik2d_backward(grad_u, u, f, ix, jx, h):
    f = _c(f)
    n1, m1 = f.shape
    g = np.empty_like(f)
    rc = lib().orc_eik2d_backward(_c(grad_u).ravel(), _c(u).ravel(), f.ravel(), m1 - 1, n1 - 1,
                                  float(h), int(ix), int(jx), g.ravel())
    if rc != 0:
        raise ArithmeticError("2D adjoint system is singular (a cell has no upwind direction)")
    return g


# ---------------------------------------------------------------- 3D ------
def eik3d_forward(u0, f, h, tol, max_iter=20):
    u0 = _c(u0)
    m, n, l = u0.shape
    u = np.empty_like(u0)
    err = C.c_double(0.0)
    it = lib().orc_eik3d_forward(u0.ravel(), _c(f).ravel(), float(h), m, n, l, float(tol),
                                 int(max_iter), u.ravel(), C.byref(err))
    return u, it, err.value


def eik3d_backward(grad_u, u, u0, f, h):
    u = _c(u)
    m, n, l = u.shape
    gu0 = np.empty_like(u)
    gf = np.empty_like(u)
    lib().orc_eik3d_backward(_c(grad_u).ravel(), u.ravel(), _c(u0).ravel(), _c(f).ravel(),
                             float(h), m, n, l, gu0.ravel(), gf.ravel())
    return gu0, gf


def assemble(dim, u, u0=None, ix=0, jx=0):
    """COO triplets (rows, cols, vals) of the adjoint matrix A and the seed mask."""
    u = _c(u)
    if dim == 2:
        n1, m1 = u.shape
        m, n, l = m1 - 1, n1 - 1, 1
        u0 = np.zeros(1)
    else:
        m, n, l = u.shape
    N = u.size
    cap = 8 * N + 8
    rows = np.empty(cap, np.int64)
    cols = np.empty(cap, np.int64)
    vals = np.empty(cap, np.float64)
    mask = np.empty(N, np.float64)
    nt = lib().orc_assemble(dim, u.ravel(), _c(u0).ravel(), m, n, l, int(ix), int(jx), cap, rows,
                            cols, vals, mask)
    assert nt >= 0
    return rows[:nt], cols[:nt], vals[:nt], mask


SRC_MODES = {"gene_obs": 0, "inversion": 1, "node": 2}


def src_u0(a, h, src, mode="gene_obs"):
    """u0 = 1000 except the 8 nodes around the fractional 0-based source.

    mode "gene_obs": a is the slowness; distance * a[ceil x, ceil y, k] * h
        (scripts/gene_obs.jl:42-51: one slowness per depth plane);
    mode "inversion": a is the velocity vel0; distance * h / a[node]
        (scripts/inversion.jl:52-60);
    mode "node": a is the slowness; distance * a[node] * h."""
    a = _c(a)
    m, n, l = a.shape
    u0 = np.empty_like(a)
    lib().orc_src_u0(a.ravel(), m, n, l, float(h), float(src[0]), float(src[1]), float(src[2]),
                     SRC_MODES[mode], u0.ravel())
    return u0


def sample(u, xyz):
    u = _c(u)
    m, n, l = u.shape
    idx = np.zeros(8, np.int64)
    w = np.zeros(8, np.float64)
    t = lib().orc_sample(u.ravel(), m, n, l, float(xyz[0]), float(xyz[1]), float(xyz[2]),
                         idx.ctypes.data, w.ctypes.data)
    return t, idx, w


def batch_misfit_grad(fields, stations, solve_field, src_xyz, t_obs, weight, tol=1e-6,
                      max_iter=20, nthreads=1, src_mode="gene_obs", src_model=None):
    """FP64 misfit + summed slowness gradient over solves.

    fields: list of (slowness (m,n,l) array, h); stations: list of (S_f, 3) arrays.
    t_obs / weight: 1-D arrays, concatenated per solve (nsta of the solve's field).
    src_mode / src_model: the near-source rule of src_u0 and its arrays (one
    per field; None: the evaluation's own slowness, not for "inversion").
    Returns (misfit, t_pred, [grad per field], iters)."""
    dims = np.array([f.shape for f, _ in fields], np.int32).ravel()
    hs = np.array([h for _, h in fields], np.float64)
    slow = np.concatenate([_c(f).ravel() for f, _ in fields])
    nsta = np.array([len(s) for s in stations], np.int32)
    sta = np.concatenate([_c(s).ravel() for s in stations]) if len(stations) else np.zeros(0)
    sf = np.ascontiguousarray(solve_field, np.int32)
    src = _c(src_xyz).ravel()
    t_obs = _c(t_obs).ravel()
    weight = _c(weight).ravel()
    t_pred = np.empty_like(t_obs)
    grad = np.empty_like(slow)
    iters = np.empty(len(sf), np.int32)
    mis = C.c_double(0.0)
    model = (np.concatenate([_c(a).ravel() for a in src_model]) if src_model is not None
             else None)
    rc = lib().orc_batch_misfit_grad(len(fields), dims, hs, slow, nsta, sta, len(sf), sf, src,
                                     t_obs, weight, float(tol), int(max_iter), int(nthreads),
                                     SRC_MODES[src_mode],
                                     model.ctypes.data if model is not None else None,
                                     C.byref(mis), t_pred, grad, iters)
    assert rc == 0
    out, off = [], 0
    for f, _ in fields:
        out.append(grad[off:off + f.size].reshape(f.shape))
        off += f.size
    return mis.value, t_pred, out, iters


# ------------------------------------------------ reference (_ref) ------
def ref_eik2d_forward(f, ix, jx, h):
    f = _c(f)
    n1, m1 = f.shape
    u = np.empty_like(f)
    ref_lib().ref_eik2d_forward(u.ravel(), f.ravel(), m1 - 1, n1 - 1, float(h), int(ix), int(jx))
    return u


def ref_eik2d_backward(grad_u, u, f, ix, jx, h):
    f = _c(f)
    n1, m1 = f.shape
    g = np.empty_like(f)
    ref_lib().ref_eik2d_backward(g.ravel(), _c(grad_u).ravel(), _c(u).ravel(), f.ravel(), m1 - 1,
                                 n1 - 1, float(h), int(ix), int(jx))
    return g


def ref_eik3d_forward(u0, f, h, tol):
    u0 = _c(u0)
    m, n, l = u0.shape
    u = np.empty_like(u0)
    ref_lib().ref_eik3d_forward(u.ravel(), u0.ravel(), _c(f).ravel(), float(h), m, n, l,
                                float(tol), 0)
    return u


def ref_eik3d_backward(grad_u, u, u0, f, h):
    u = _c(u)
    m, n, l = u.shape
    gu0 = np.empty_like(u)
    gf = np.empty_like(u)
    ref_lib().ref_eik3d_backward(gu0.ravel(), gf.ravel(), _c(grad_u).ravel(), u.ravel(),
                                 _c(u0).ravel(), _c(f).ravel(), float(h), m, n, l)
    return gu0, gf


def smooth_l1(v, sh, sv, lam=1.0):
    """lam * sum |v - S v| and its gradient lam * (s - S s), s = sign(v - S v),
    S the circular box mean over sh x sh x sv cells: the penalty of
    scripts/inversion.jl:107-121 (the tf.concat wrap-around padding followed by
    a VALID conv3d with weights 1/(sh*sh*sv)).  Plain NumPy, FP64."""
    v = np.asarray(v, np.float64)
    rh, rv = (sh - 1) // 2, (sv - 1) // 2

    def box(a):
        out = np.zeros_like(a)
        for dx in range(-rh, rh + 1):
            for dy in range(-rh, rh + 1):
                for dz in range(-rv, rv + 1):
                    out += np.roll(a, (-dx, -dy, -dz), axis=(0, 1, 2))
        return out / (sh * sh * sv)

    r = v - box(v)
    s = np.sign(r)
    return lam * np.abs(r).sum(), lam * (s - box(s))
