"""The CPU oracle against the reference's golden vectors and known answers.

The oracle (oracle/eikonal_oracle.c) restates deps/CustomOps/Eikonal/Eikonal.h
and deps/CustomOps/Eikonal3D/Eikonal3D.cpp.  These tests pin it: the FP64
forward must be bit-identical to the reference outputs stored in tests/golden
(generated by tests/golden/make_golden.py from the reference sources), and the
adjoint must agree to rounding (the reference factorises with SparseLU; the
oracle substitutes in causal order).
"""
import glob
import os

import numpy as np
import pytest

from adtomo_gb300 import synth
from oracle import oracle as O

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "g[23]d_*.npz")))


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_oracle_matches_reference_golden(path):
    g = np.load(path)
    if str(g["kind"]) == "2d":
        u, _, _ = O.eik2d_forward(g["f"], int(g["ix"]), int(g["jx"]), float(g["h"]))
        assert np.array_equal(u, g["u"]), "2D forward must be bit-identical to the reference"
        gf = O.eik2d_backward(g["grad_u"], g["u"], g["f"], int(g["ix"]), int(g["jx"]), float(g["h"]))
        scale = np.abs(g["grad_f"]).max()
        assert np.abs(gf - g["grad_f"]).max() <= 1e-12 * scale
    else:
        u, _, _ = O.eik3d_forward(g["u0"], g["f"], float(g["h"]), float(g["tol"]))
        assert np.array_equal(u, g["u"]), "3D forward must be bit-identical to the reference"
        gu0, gf = O.eik3d_backward(g["grad_u"], g["u"], g["u0"], g["f"], float(g["h"]))
        assert np.array_equal(gu0, g["grad_u0"])
        scale = max(np.abs(g["grad_f"]).max(), 1e-300)
        assert np.abs(gf - g["grad_f"]).max() <= 1e-12 * scale


def test_homogeneous_on_axis_exact_3d():
    """Point source in a homogeneous medium: along grid lines through the
    source the first-order scheme is exact, u = |d| f h."""
    m, n, l, h = 15, 12, 10, 0.25
    f = np.full((m, n, l), 0.5)
    s = (7, 5, 4)
    u0 = np.full((m, n, l), 1000.0)
    u0[s] = 0.0
    u, it, _ = O.eik3d_forward(u0, f, h, 1e-12, 50)
    ax = np.arange(m)
    np.testing.assert_allclose(u[:, s[1], s[2]], np.abs(ax - s[0]) * 0.5 * h, rtol=0, atol=1e-14)
    np.testing.assert_allclose(u[s[0], :, s[2]], np.abs(np.arange(n) - s[1]) * 0.5 * h, atol=1e-14)
    np.testing.assert_allclose(u[s[0], s[1], :], np.abs(np.arange(l) - s[2]) * 0.5 * h, atol=1e-14)
    # monotone away from the source along every axis line through it
    assert np.all(np.diff(u[s[0]:, s[1], s[2]]) > 0)
    assert np.all(np.diff(u[:s[0] + 1, s[1], s[2]]) < 0)


def test_symmetry_centred_source_3d():
    m = n = l = 11
    f = np.ones((m, n, l))
    u0 = np.full((m, n, l), 1000.0)
    u0[5, 5, 5] = 0.0
    u, _, _ = O.eik3d_forward(u0, f, 1.0, 1e-12, 50)
    np.testing.assert_allclose(u, u[::-1, :, :], atol=1e-12)
    np.testing.assert_allclose(u, u[:, ::-1, :], atol=1e-12)
    np.testing.assert_allclose(u, np.transpose(u, (1, 0, 2)), atol=1e-12)


def test_homogeneous_on_axis_exact_2d():
    f = np.full((21, 31), 2.0)
    u, _, conv = O.eik2d_forward(f, 10, 7, 0.5)
    assert conv
    np.testing.assert_allclose(u[7, :], np.abs(np.arange(31) - 10) * 2.0 * 0.5, atol=1e-13)
    np.testing.assert_allclose(u[:, 10], np.abs(np.arange(21) - 7) * 2.0 * 0.5, atol=1e-13)


def test_adjoint_matches_sparse_lu_3d():
    """The causal substitution equals a general sparse LU (SuperLU, the same
    family as Eigen's SparseLU) on the identical assembled matrix."""
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "g3d_layered.npz"))
    u, u0, f, h = g["u"], g["u0"], g["f"], float(g["h"])
    rows, cols, vals, mask = O.assemble(3, u, u0)
    N = u.size
    A = sp.csc_matrix((vals, (rows, cols)), shape=(N, N))
    lam = spla.spsolve(A.T.tocsc(), g["grad_u"].ravel() * mask)
    gf_lu = 2 * f.ravel() * h * h * lam
    _, gf = O.eik3d_backward(g["grad_u"], u, u0, f, h)
    assert np.abs(gf.ravel() - gf_lu).max() <= 1e-10 * np.abs(gf_lu).max()


def test_adjoint_matches_sparse_lu_2d():
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "g2d_band.npz"))
    u, f, h, ix, jx = g["u"], g["f"], float(g["h"]), int(g["ix"]), int(g["jx"])
    rows, cols, vals, _ = O.assemble(2, u, None, ix, jx)
    N = u.size
    A = sp.csc_matrix((vals, (rows, cols)), shape=(N, N))
    lam = spla.spsolve(A.T.tocsc(), g["grad_u"].ravel())
    dfdf = -2 * f.ravel() * h * h
    dfdf[jx * f.shape[1] + ix] = 0.0
    gf_lu = -lam * dfdf
    gf = O.eik2d_backward(g["grad_u"], u, f, ix, jx, h)
    assert np.abs(gf.ravel() - gf_lu).max() <= 1e-10 * np.abs(gf_lu).max()


def test_taylor_gradient_3d():
    """Taylor test in the style of deps/CustomOps/Eikonal3D/gradtest.jl:49-63,
    but with respect to the slowness: the first-order remainder must shrink
    like gamma^2."""
    rng = np.random.default_rng(3)
    m, n, l, h = 12, 11, 9, 0.5
    f = 0.2 + 0.05 * rng.random((m, n, l))
    u0 = O.src_u0(f, h, (5.4, 4.7, 3.2))
    u, _, _ = O.eik3d_forward(u0, f, h, 1e-14, 60)
    J = lambda uu: float(np.sum(uu ** 2))
    _, gf = O.eik3d_backward(2 * u, u, u0, f, h)
    v = rng.random((m, n, l))
    v[u0 < 1000] = 0.0  # keep the initial values fixed
    r1, r2 = [], []
    for gam in (1e-3, 1e-4, 1e-5):
        up, _, _ = O.eik3d_forward(u0, f + gam * v, h, 1e-14, 60)
        d = J(up) - J(u)
        r1.append(abs(d))
        r2.append(abs(d - gam * np.sum(v * gf)))
    assert r2[1] < r2[0] * 0.05 and r2[2] < r2[1] * 0.05
    assert r1[2] > r1[1] * 0.05


def test_batch_matches_single_solves():
    rng = np.random.default_rng(5)
    m, n, l, h = 10, 9, 8, 0.5
    f = 0.25 + 0.02 * rng.random((m, n, l))
    sta = np.column_stack([rng.uniform(0, m - 1, 6), rng.uniform(0, n - 1, 6), np.zeros(6)])
    src = np.column_stack([rng.uniform(1, m - 2, 3), rng.uniform(1, n - 2, 3), rng.uniform(1, l - 2, 3)])
    t_obs = rng.uniform(0.5, 2.0, 18)
    t_obs[4] = -1.0
    w = rng.uniform(0.5, 1.0, 18)
    mis, tp, grads, iters = O.batch_misfit_grad([(f, h)], [sta], np.zeros(3, np.int32), src, t_obs, w,
                                                nthreads=2)
    mis1, g1 = 0.0, np.zeros_like(f)
    for s in range(3):
        u0 = O.src_u0(f, h, src[s])
        u, _, _ = O.eik3d_forward(u0, f, h, 1e-6)
        gu = np.zeros_like(u)
        for q in range(6):
            t, idx, wt = O.sample(u, sta[q])
            assert t == tp[6 * s + q]
            if t_obs[6 * s + q] == -1:
                continue
            r = t_obs[6 * s + q] - t
            mis1 += w[6 * s + q] * r * r
            np.add.at(gu.ravel(), idx, -2 * w[6 * s + q] * r * wt)
        g1 += O.eik3d_backward(gu, u, u0, f, h)[1]
    assert abs(mis - mis1) <= 1e-12 * mis1
    np.testing.assert_allclose(grads[0], g1, rtol=0, atol=1e-12 * np.abs(g1).max())


def _julia_u0(a, h, ix, iy, iz, rule):
    """Line-by-line restatement of the two Julia caller blocks on Julia's
    1-based coordinates (ix, iy, iz): scripts/gene_obs.jl:39-51 (rule
    "gene_obs", a = slowness) and scripts/inversion.jl:48-60 (rule
    "inversion", a = vel0)."""
    ixu, ixd = int(np.ceil(ix)), int(np.floor(ix))
    iyu, iyd = int(np.ceil(iy)), int(np.floor(iy))
    izu, izd = int(np.ceil(iz)), int(np.floor(iz))
    u0 = 1000 * np.ones(a.shape)
    A = lambda i, j, k: a[i - 1, j - 1, k - 1]  # noqa: E731  (1-based read)

    def put(i, j, k, v):
        u0[i - 1, j - 1, k - 1] = v

    if rule == "gene_obs":
        pu, pd = A(ixu, iyu, izu), A(ixu, iyu, izd)
        for i in (ixu, ixd):
            for j in (iyu, iyd):
                for k, s in ((izu, pu), (izd, pd)):
                    put(i, j, k, np.sqrt((ix - i) * (ix - i) + (iy - j) * (iy - j) +
                                         (iz - k) * (iz - k)) * s * h)
    else:
        for i in (ixu, ixd):
            for j in (iyu, iyd):
                for k in (izu, izd):
                    put(i, j, k, np.sqrt((ix - i) * (ix - i) + (iy - j) * (iy - j) +
                                         (iz - k) * (iz - k)) * h / A(i, j, k))
    return u0


@pytest.mark.parametrize("src1", [(4.6, 8.3, 4.5), (12.25, 4.8, 8.1), (5.0, 7.0, 3.0),
                                  (1.0, 1.3, 14.0), (20.0, 18.0, 1.75), (7.123456789, 9.87, 2.2)])
def test_src_u0_rules_follow_the_reference_callers(src1):
    """orc_src_u0 reproduces the caller code bit for bit: gene_obs.jl's one
    slowness per depth plane from the (ceil x, ceil y) column, and
    inversion.jl's h / vel0 per node (including integral coordinates and grid
    edges).  The callers read 1-based coordinates; the library takes x - 1,
    which is exact for x >= 1, so the distances are the same bits."""
    m, n, l, h = 20, 18, 14, 0.5
    f = synth.layered_checkerboard(m, n, l, block=4)
    v0 = 1.0 / synth.layered_checkerboard(m, n, l, block=2)
    src0 = tuple(x - 1.0 for x in src1)
    assert all((x0 + 1.0) - 1.0 == x0 for x0 in src0)
    assert np.array_equal(O.src_u0(f, h, src0, mode="gene_obs"),
                          _julia_u0(f, h, *src1, "gene_obs"))
    assert np.array_equal(O.src_u0(v0, h, src0, mode="inversion"),
                          _julia_u0(v0, h, *src1, "inversion"))


def test_location_oracle_matches_the_reference_script(golden_dir):
    """The NumPy restatement of the location objective against the loss and
    autograd gradient of tests/Eikonal/eikoloc.py's own _interp, traveltime
    and invert closure (fixture from tests/golden/make_location_golden.py):
    loss to 1e-12 relative, central differences of the loss to the gradient
    to 1e-6."""
    from oracle import location_oracle as LO
    d = np.load(os.path.join(golden_dir, "loc_eikoloc.npz"))
    offs, b = d["offs"], d["bounds"]
    args = (d["tp"], d["ts"], float(d["r0"]), float(d["z0"]), float(d["h"]), b)
    for c in range(len(d["params"])):
        sl = slice(offs[c], offs[c + 1])
        pick = (d["sta"][sl], d["t"][sl], d["phase"][sl], d["w"][sl])

        def f(p):
            return LO.event_loss(p, *pick, *args, gamma=float(d["gamma"][c]))
        p0 = d["params"][c]
        assert abs(f(p0) - d["loss"][c]) <= 1e-12 * abs(d["loss"][c]), c
        for a in range(4):
            e = np.zeros(4)
            e[a] = 1e-6
            fd = (f(p0 + e) - f(p0 - e)) / 2e-6
            assert abs(fd - d["grad"][c][a]) <= 1e-6 * max(1.0, abs(d["grad"][c][a])), (c, a)
