"""The inversion driver around the hot path (scripts/inversion.jl, src/mpi_optimize.jl):
smoothness penalty, L-BFGS with backtracking, and the full objective's gradient.

CPU tests check the optimiser and the NumPy restatement of the penalty; GPU
tests check the CUDA penalty and the batched objective through the C ABI.
"""
import numpy as np
import pytest

import adtomo_gb300 as A
from adtomo_gb300 import inversion as I
from adtomo_gb300 import synth
from oracle import oracle as O


# ------------------------------------------------------------- CPU -----
def _rosen(x):
    f = np.sum(100.0 * (x[1:] - x[:-1] ** 2) ** 2 + (1.0 - x[:-1]) ** 2)
    g = np.zeros_like(x)
    g[:-1] = -400.0 * x[:-1] * (x[1:] - x[:-1] ** 2) - 2.0 * (1.0 - x[:-1])
    g[1:] += 200.0 * (x[1:] - x[:-1] ** 2)
    return f, g


def test_lbfgs_rosenbrock():
    x, f, hist = I.lbfgs(_rosen, np.full(10, -1.2), iterations=500, g_tol=1e-10)
    assert f < 1e-16
    assert np.allclose(x, 1.0, atol=1e-7)
    # every accepted step decreases the objective (Armijo condition)
    assert all(b < a for a, b in zip(hist, hist[1:]))


def test_lbfgs_quadratic_exact_in_n_steps():
    rng = np.random.default_rng(1)
    M = rng.standard_normal((6, 6))
    H = M @ M.T + 6 * np.eye(6)
    b = rng.standard_normal(6)
    x, f, _ = I.lbfgs(lambda x: (0.5 * x @ H @ x - b @ x, H @ x - b), np.zeros(6),
                      iterations=200, g_tol=1e-12)
    assert np.allclose(x, np.linalg.solve(H, b), rtol=1e-9, atol=1e-10)


def test_backtracking_sufficient_decrease():
    # phi(a) = (a - 0.1)^2 from phi'(0) = -0.2: step 1 fails, backtracking must
    # return a step with phi(a) <= phi(0) + c1 a phi'(0)
    phi = lambda a: (a - 0.1) ** 2
    a, pa = I._backtracking(phi, 1.0, phi(0.0), -0.2)
    assert pa <= phi(0.0) + 1e-4 * a * -0.2
    assert 0.0 < a < 1.0


def test_oracle_smooth_l1_against_scipy():
    ndimage = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(2)
    v = rng.uniform(4.0, 8.0, (9, 7, 5))
    pen, g = O.smooth_l1(v, 5, 3, 0.7)
    box = ndimage.uniform_filter(v, size=(5, 5, 3), mode="wrap")
    r = v - box
    assert np.isclose(pen, 0.7 * np.abs(r).sum(), rtol=1e-13)
    s = np.sign(r)
    assert np.allclose(g, 0.7 * (s - ndimage.uniform_filter(s, size=(5, 5, 3), mode="wrap")),
                       rtol=1e-12, atol=1e-14)


def test_oracle_smooth_l1_gradient_fd():
    rng = np.random.default_rng(3)
    v = rng.uniform(4.0, 8.0, (6, 5, 4))
    _, g = O.smooth_l1(v, 3, 3, 1.0)
    for c in [(0, 0, 0), (2, 3, 1), (5, 4, 3)]:
        e = np.zeros_like(v)
        e[c] = 1e-7
        fd = (O.smooth_l1(v + e, 3, 3)[0] - O.smooth_l1(v - e, 3, 3)[0]) / 2e-7
        assert abs(fd - g[c]) < 1e-6


def test_smooth_l1_rejects_bad_sizes():
    with pytest.raises(A.AdtError):
        I.smooth_l1(np.ones((4, 4, 4)), 4, 3)  # even box
    with pytest.raises(A.AdtError):
        I.smooth_l1(np.ones((2, 2, 8)), 7, 1)  # half-width beyond the grid


# ------------------------------------------------------------- GPU -----
@pytest.mark.gpu
def test_smooth_l1_matches_oracle():
    rng = np.random.default_rng(4)
    v = rng.uniform(4.0, 8.0, (20, 18, 12))
    for sh, sv in [(1, 1), (3, 3), (5, 3), (7, 5)]:
        pen, g = I.smooth_l1(v, sh, sv, 0.3)
        po, go = O.smooth_l1(v, sh, sv, 0.3)
        assert abs(pen - po) <= 1e-12 * abs(po) + 1e-15
        assert np.allclose(g, go, rtol=1e-12, atol=1e-13)
        pen2, g2 = I.smooth_l1(v, sh, sv, 0.3)
        assert pen2 == pen and np.array_equal(g2, g)  # fixed reduction order


def _small_problem(rng, shape=(24, 20, 14), h=0.5, nsta=6, neve=10):
    m, n, l = shape
    vtrue = 1.0 / synth.layered_checkerboard(m, n, l, block=4)
    vel0 = np.full(shape, vtrue.mean())
    sta = synth.surface_stations(m, n, nsta, rng)
    eve = synth.volume_sources(m, n, l, neve, rng)
    # synthetic picks: FP64 forward on the true model through the same plan
    P = A.Batch3D([(m, n, l, h)], [eve], np.zeros(nsta, np.int32), sta, precision=A.ADT_F64,
                  tol=1e-9, max_iter=200)
    _, tp, _, _ = P.run([1.0 / vtrue], np.full(nsta * neve, 1.0), np.ones(nsta * neve))
    P.close()
    uobs = tp.reshape(nsta, neve).copy()
    uobs[0, 3] = -1.0  # a missing pick
    qua = rng.uniform(0.5, 1.0, (nsta, neve))
    return (m, n, l, h), vel0, sta, eve, uobs, qua


@pytest.mark.gpu
def test_inversion_gradient_fd():
    rng = np.random.default_rng(6)
    grid, vel0, sta, eve, uobs, qua = _small_problem(rng)
    inv = I.TravelTimeInversion(grid, vel0, sta, eve, uobs, qua, lambda_p=0.05, smooth_hor=3,
                                smooth_ver=3, tol=0.0, max_iter=200, precision=A.ADT_F64)
    x = 0.3 * rng.standard_normal(vel0.shape)
    f0, g = inv.loss_and_grad(x)
    assert np.isfinite(f0) and f0 > 0
    cells = [tuple(rng.integers(0, d) for d in vel0.shape) for _ in range(8)]
    for c in cells:
        e = np.zeros_like(x)
        e[c] = 1e-5
        fp, _ = inv.loss_and_grad(x + e)
        fm, _ = inv.loss_and_grad(x - e)
        fd = (fp - fm) / 2e-5
        gi = g.reshape(vel0.shape)[c]
        assert abs(fd - gi) <= 1e-3 * max(abs(gi), 1e-3 * np.abs(g).max()), (c, fd, gi)
    inv.close()


@pytest.mark.gpu
def test_inversion_lbfgs_decreases_loss(tmp_path):
    rng = np.random.default_rng(7)
    grid, vel0, sta, eve, uobs, qua = _small_problem(rng)
    # a tight forward tolerance keeps the objective smooth enough for the
    # line search (the script's 1e-3 s makes it step-wise at this scale)
    inv = I.TravelTimeInversion(grid, vel0, sta, eve, uobs, qua, lambda_p=0.01, smooth_hor=3,
                                smooth_ver=1, tol=1e-6, max_iter=200)
    f0, _ = inv.loss_and_grad(np.zeros(vel0.shape))
    x, f, hist = inv.optimize(iterations=4, steps=2, checkpoint_dir=str(tmp_path))
    assert len(hist) == 4 and hist[0] < f0
    assert all(b < a for a, b in zip(hist, hist[1:]))
    assert (tmp_path / "iter_2.npy").exists() and (tmp_path / "iter_4.npy").exists()
    v = inv.velocity(x)
    assert np.all(v > vel0 - 1.0) and np.all(v < vel0 + 1.0)  # sigmoid bounds
    inv.close()
