"""The branch-free FP32 cell update of the batched sweeps (upd3_f32 in
eik3d_brick.cuh), restated in NumPy float32, against the local solve of the
reference (Eikonal3D.cpp:11-33: sort, one-, two- then three-axis root, each
taken while it does not exceed the next neighbour value) in FP64.  Checks the
algebra the kernel relies on: the three-axis root formed relative to the
lane's own z value, the two-axis admissibility tested as r2 <= 2 d3 - d2, the
unclamped two-axis discriminant, and +inf ghost neighbours.  CPU only."""
import numpy as np

f32 = np.float32


def upd3_f32_model(ax, ay, az, fh):
    """Same operations as the kernel, in float32 (sqrt correctly rounded here,
    the hardware approximation there)."""
    with np.errstate(invalid="ignore", over="ignore"):
        ax, ay, az, fh = (np.asarray(v, f32) for v in (ax, ay, az, fh))
        lo = np.minimum(np.minimum(ax, ay), az)
        hi = np.maximum(np.maximum(ax, ay), az)
        mid = np.minimum(np.minimum(np.maximum(ax, ay), np.maximum(ax, az)), np.maximum(ay, az))
        F2 = fh * fh
        d2, d3 = mid - lo, hi - lo
        x1 = lo + fh
        r2 = np.sqrt(-d2 * d2 + f32(2) * F2)  # NaN only where x1 is taken
        x2 = f32(0.5) * (d2 + r2) + lo
        bx, by, bxy = ax - az, ay - az, ax - ay
        disc = -bxy * bxy + (-by * by + (-bx * bx + f32(3) * F2))
        r3 = np.sqrt(np.maximum(disc, f32(0)))
        x3 = (bx + by + r3) * f32(1.0 / 3.0) + az
        c2 = r2 <= f32(2) * d3 - d2
        return np.where(x1 <= mid, x1, np.where(c2, x2, x3))


def local_solve_ref(ax, ay, az, fh):
    """FP64: sorted a1 <= a2 <= a3; x = a1 + F; if x > a2 the two-axis root
    of (x-a1)^2 + (x-a2)^2 = F^2; if that exceeds a3 the three-axis root."""
    a = np.sort(np.stack([ax, ay, az]).astype(np.float64), axis=0)
    F = np.asarray(fh, np.float64)
    with np.errstate(invalid="ignore"):
        x = a[0] + F
        two = x > a[1]
        x2 = (a[0] + a[1] + np.sqrt(2 * F * F - (a[1] - a[0]) ** 2)) / 2
        x = np.where(two, x2, x)
        three = two & (x > a[2])
        s = a.sum(axis=0)
        x3 = (s + np.sqrt(s * s - 3 * ((a ** 2).sum(axis=0) - F * F))) / 3
        return np.where(three, x3, x)


def test_update_matches_local_solve():
    rng = np.random.default_rng(3)
    n = 200000
    fh = rng.uniform(1e-3, 1.0, n)
    base = rng.uniform(5.0, 20.0, n)
    # neighbour values within a few F of each other: every branch occurs
    ax = base + rng.uniform(0, 2.0, n) * fh
    ay = base + rng.uniform(0, 2.0, n) * fh
    az = base + rng.uniform(0, 2.0, n) * fh
    got = upd3_f32_model(ax, ay, az, fh).astype(np.float64)
    # the reference solve on the float32-rounded inputs
    ref = local_solve_ref(*(np.asarray(v, f32) for v in (ax, ay, az, fh)))
    assert np.all(np.isfinite(got))
    assert np.max(np.abs(got - ref) / ref) < 2e-6
    # every branch is exercised: one, two and three upwind axes
    a = np.sort(np.stack([ax, ay, az]), axis=0)
    one = a[0] + fh <= a[1]
    three = ref > a[2]
    assert one.mean() > 0.05 and three.mean() > 0.05 and (~one & ~three).mean() > 0.05


def test_update_with_ghost_neighbours():
    rng = np.random.default_rng(4)
    n = 20000
    fh = rng.uniform(1e-2, 1.0, n)
    vals = rng.uniform(5.0, 6.0, (3, n))
    for ghosts in ([0], [1], [2], [0, 1], [0, 2], [1, 2]):
        v = vals.copy()
        for gi in ghosts:
            v[gi] = np.inf
        got = upd3_f32_model(v[0], v[1], v[2], fh).astype(np.float64)
        ref = local_solve_ref(*(np.asarray(x, f32) for x in (v[0], v[1], v[2], fh)))
        assert np.all(np.isfinite(got)), ghosts
        assert np.max(np.abs(got - ref) / ref) < 2e-6, ghosts
    # all three neighbours ghosts: +inf, never NaN
    inf = np.full(4, np.inf)
    assert np.all(np.isposinf(upd3_f32_model(inf, inf, inf, np.ones(4))))
