"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference's own C++ functions (deps/CustomOps/Eikonal/Eikonal.h,
deps/CustomOps/Eikonal3D/Eikonal3D.cpp) are compiled in place by
`make -C oracle ref` into oracle/_ref/libadtomo_ref.so and run here on seeded
inputs; inputs and outputs are written as compressed .npz files.  The reference
sources do not exist on GPU machines, so the fixtures are committed.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def layered_checker(m, n, l, block, rng=None, amp=0.05):
    """Velocity rising linearly 4 -> 8 km/s with depth (k) times a +-amp
    checkerboard of `block`-cell blocks; returns slowness."""
    z = np.arange(l)
    v = 4.0 + 4.0 * z / max(l - 1, 1)
    ii, jj, kk = np.meshgrid(np.arange(m), np.arange(n), np.arange(l), indexing="ij")
    sgn = (-1.0) ** ((ii // block) + (jj // block) + (kk // block))
    return 1.0 / (v[None, None, :] * (1.0 + amp * sgn))


def gauss2d(n1, m1, rng):
    """6 km/s background with 3 Gaussian anomalies of +-10%, sigma 8 cells."""
    jj, ii = np.meshgrid(np.arange(n1), np.arange(m1), indexing="ij")
    v = np.full((n1, m1), 6.0)
    for _ in range(3):
        cj, ci = rng.uniform(8, n1 - 8), rng.uniform(8, m1 - 8)
        amp = rng.choice([-0.1, 0.1])
        v *= 1.0 + amp * np.exp(-((jj - cj) ** 2 + (ii - ci) ** 2) / (2 * 8.0 ** 2))
    return 1.0 / v


def case2d(name, f, ix, jx, h, gu):
    u = O.ref_eik2d_forward(f, ix, jx, h)
    gf = O.ref_eik2d_backward(gu, u, f, ix, jx, h)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), kind="2d", f=f, ix=ix, jx=jx, h=h,
                        grad_u=gu, u=u, grad_f=gf)
    print(name, f.shape, "max u", u.max())


def case3d(name, u0, f, h, tol, gu):
    u = O.ref_eik3d_forward(u0, f, h, tol)
    gu0, gf = O.ref_eik3d_backward(gu, u, u0, f, h)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), kind="3d", u0=u0, f=f, h=h, tol=tol,
                        grad_u=gu, u=u, grad_u0=gu0, grad_f=gf)
    print(name, f.shape, "max u", u.max())


def main():
    O.build(ref=True)
    rng = np.random.default_rng(0)

    # 2D: the gradient-test model of deps/CustomOps/Eikonal/gradtest.jl:41-51
    m, n, h = 60, 30, 0.1
    f = np.ones((n + 1, m + 1))
    f[11:18, :] = 10.0
    case2d("g2d_band", f, 29, 2, h, rng.random(f.shape))

    # 2D: 101x101 Gaussian-anomaly model, interior source, 20 receivers
    f = gauss2d(101, 101, rng)
    ix, jx = (int(v) for v in rng.integers(5, 96, size=2))
    gu = np.zeros_like(f)
    rec = rng.integers(0, 101, size=(20, 2))
    gu[rec[:, 0], rec[:, 1]] = rng.standard_normal(20)
    case2d("g2d_gauss101", f, ix, jx, 1.0, gu)

    # 2D: small ragged grid, random slowness, corner source
    f = rng.uniform(0.5, 2.0, size=(12, 7))
    case2d("g2d_ragged", f, 0, 0, 0.5, rng.standard_normal(f.shape))

    # 3D: gradient-test setup of deps/CustomOps/Eikonal3D/gradtest.jl:14-23
    m = n = l = 21
    u0 = np.full((m, n, l), 1000.0)
    u0[10, 10, 11] = 0.0
    case3d("g3d_unit21", u0, np.ones((m, n, l)), 0.01, 1e-6, rng.random((m, n, l)))

    # 3D: layered + checkerboard, fractional source, receivers on the top face
    m, n, l = 17, 13, 11
    f = layered_checker(m, n, l, 4)
    u0 = O.src_u0(f, 1.0, (5.3, 7.6, 4.2), mode="node")
    gu = np.zeros((m, n, l))
    gu[:, :, 0] = rng.standard_normal((m, n))
    case3d("g3d_layered", u0, f, 1.0, 1e-6, gu)

    # 3D: random initial values (gradtest.jl:43 style), unit slowness
    m = n = l = 9
    case3d("g3d_randu0", rng.random((m, n, l)) * 1000, np.ones((m, n, l)), 0.01, 1e-6,
           rng.random((m, n, l)))

    # 3D: ragged extents, random slowness, integer corner source
    m, n, l = 5, 19, 7
    f = rng.uniform(0.5, 2.0, size=(m, n, l))
    u0 = np.full((m, n, l), 1000.0)
    u0[0, 0, 0] = 0.0
    case3d("g3d_ragged", u0, f, 0.5, 1e-6, rng.standard_normal((m, n, l)))

    # 3D: smallest legal grid
    f = rng.uniform(0.5, 2.0, size=(2, 2, 2))
    u0 = np.full((2, 2, 2), 1000.0)
    u0[1, 0, 1] = 0.0
    case3d("g3d_min", u0, f, 1.0, 1e-6, rng.standard_normal((2, 2, 2)))

    # 3D: medium layered model with 8-cell checkerboard, loose tolerance (1e-3
    # as in scripts/inversion.jl:61) so the reference stops before full
    # convergence
    m, n, l = 40, 36, 20
    f = layered_checker(m, n, l, 8)
    u0 = O.src_u0(f, 1.0, (20.5, 11.25, 9.75), mode="node")
    gu = np.zeros((m, n, l))
    gu[:, :, 0] = rng.standard_normal((m, n))
    case3d("g3d_layered_tol1e3", u0, f, 1.0, 1e-3, gu)


if __name__ == "__main__":
    main()
