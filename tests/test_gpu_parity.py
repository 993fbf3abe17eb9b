"""GPU parity: the CUDA library through its C ABI against the oracle.

Tolerances (stated per test):
  * plain FP64 path (adt_eikonal, adt_eikonal_three_d): travel times
    bit-identical to the oracle and to the reference golden vectors; adjoint
    bit-identical to the oracle (same per-cell formula and summation order)
    and within 1e-12 relative of the reference's SparseLU solution.
  * batched FP64 with the reference stopping rule: misfit, predicted times and
    summed gradient bit-identical to the oracle's batch.
  * batched FP32: relative travel-time error <= 1e-4 (max over picks) and
    relative gradient error <= 1e-3 (L2 norm) against the FP64 oracle.
"""
import glob
import os

import numpy as np
import pytest

import adtomo_gb300 as A
from adtomo_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "g[23]d_*.npz")))


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if A.lib().adt_device_count() < 1:
        pytest.skip("no GPU")


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# ------------------------------------------------------------ golden ----
@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_plain_fp64_matches_reference_golden(path):
    g = np.load(path)
    if str(g["kind"]) == "2d":
        ix, jx, h = int(g["ix"]), int(g["jx"]), float(g["h"])
        u = A.eikonal(g["f"], ix + 1, jx + 1, h)
        assert np.array_equal(u, g["u"])
        gf = A.eikonal_grad(g["grad_u"], g["u"], g["f"], ix + 1, jx + 1, h)
        assert rel_max(gf, g["grad_f"]) <= 1e-12
        assert np.array_equal(gf, O.eik2d_backward(g["grad_u"], g["u"], g["f"], ix, jx, h))
    else:
        m, n, l = g["f"].shape
        h, tol = float(g["h"]), float(g["tol"])
        u = A.eikonal3d(g["u0"], g["f"], h, m, n, l, tol)
        assert np.array_equal(u, g["u"])
        g0, gf = A.eikonal3d_grad(g["grad_u"], g["u"], g["u0"], g["f"], h, m, n, l)
        assert np.array_equal(g0, g["grad_u0"])
        assert rel_max(gf, g["grad_f"]) <= 1e-12
        r0, rf = O.eik3d_backward(g["grad_u"], g["u"], g["u0"], g["f"], h)
        assert np.array_equal(gf, rf)


# ------------------------------------------------- plain FP64, seeded ----
CASES3 = [
    # (m, n, l, source) -- ragged extents, k longer than a brick, tiny grids
    (9, 13, 37, (4.5, 6.2, 17.9)),
    (17, 6, 70, (0.0, 0.0, 0.0)),
    (2, 2, 2, (1.0, 0.0, 1.0)),
    (33, 5, 3, (32.0, 4.0, 2.0)),
    (24, 20, 66, (11.7, 3.1, 64.6)),
]


@pytest.mark.parametrize("case", CASES3, ids=[f"{c[0]}x{c[1]}x{c[2]}" for c in CASES3])
def test_plain_fp64_random_models(case):
    m, n, l, src = case
    rng = np.random.default_rng(m * 1000 + n * 10 + l)
    f = rng.uniform(0.15, 0.35, size=(m, n, l))
    h = 0.5
    u0 = O.src_u0(f, h, src)
    u, st = A.eikonal3d(u0, f, h, m, n, l, 1e-9, return_status=True)
    ur, it, _ = O.eik3d_forward(u0, f, h, 1e-9)
    assert np.array_equal(u, ur)
    assert st.iters == it
    gu = rng.standard_normal((m, n, l))
    g0, gf = A.eikonal3d_grad(gu, u, u0, f, h, m, n, l)
    r0, rf = O.eik3d_backward(gu, ur, u0, f, h)
    assert np.array_equal(g0, r0)
    assert np.array_equal(gf, rf)


def test_plain_fp64_iteration_cap_and_status():
    m, n, l = 20, 18, 16
    f = synth.layered_checkerboard(m, n, l, block=4)
    u0 = O.src_u0(f, 1.0, (10.2, 9.1, 8.3))
    u, st = A.eikonal3d(u0, f, 1.0, m, n, l, 0.0, return_status=True)
    ur, it, err = O.eik3d_forward(u0, f, 1.0, 0.0, 20)
    assert it == 20 and st.iters == 20 and st.converged == 0
    assert np.array_equal(u, ur)
    assert st.final_err == err


def test_c2_config_fp64_forward_adjoint_and_fd():
    """64x64x32, h=1 km, layered 4->8 km/s x (1 +- 5%) checkerboard of 8-cell
    blocks, random interior source, 50 receivers on the top surface; central
    finite differences on 20 random cells agree with the adjoint gradient to
    1e-3 relative with delta = 1e-6 f (round-off limited) and to 1e-5 with
    delta = 1e-4 f."""
    rng = np.random.default_rng(1)
    m, n, l, h = 64, 64, 32, 1.0
    f = synth.layered_checkerboard(m, n, l, block=8)
    src = synth.volume_sources(m, n, l, 1, rng)[0]
    sta = synth.surface_stations(m, n, 50, rng)
    u0 = O.src_u0(f, h, src)
    tol = 0.0
    u = A.eikonal3d(u0, f, h, m, n, l, tol)
    ur, _, _ = O.eik3d_forward(u0, f, h, tol)
    assert np.array_equal(u, ur)
    f_obs = f * (1 + 0.02 * rng.standard_normal(f.shape))
    uo = A.eikonal3d(O.src_u0(f_obs, h, src), f_obs, h, m, n, l, tol)
    t_obs = np.array([O.sample(uo, s)[0] for s in sta])

    def misfit(uu):
        return sum((t_obs[q] - O.sample(uu, sta[q])[0]) ** 2 for q in range(len(sta)))

    gu = np.zeros_like(u)
    for q in range(len(sta)):
        t, idx, w = O.sample(u, sta[q])
        np.add.at(gu.ravel(), idx, -2 * (t_obs[q] - t) * w)
    _, gf = A.eikonal3d_grad(gu, u, u0, f, h, m, n, l)
    _, rf = O.eik3d_backward(gu, ur, u0, f, h)
    assert np.array_equal(gf, rf)
    # FD on 20 random cells with non-negligible sensitivity (u0 held fixed).
    # With delta = 1e-6 f the FD quotient carries ~1e-4 relative round-off
    # (one ulp of a ~10 s travel time over a ~1e-10 misfit change), so it is
    # checked to 1e-3; delta = 1e-4 f is checked to 1e-5.
    cand = np.flatnonzero((np.abs(gf.ravel()) > 1e-3 * np.abs(gf).max()) & (u0.ravel() >= 1000))
    cells = rng.choice(cand, size=20, replace=False)
    for c in cells:
        for rel, tol_fd in ((1e-6, 1e-3), (1e-4, 1e-5)):
            d = rel * f.ravel()[c]
            fp = f.copy().ravel()
            fp[c] += d
            fm = f.copy().ravel()
            fm[c] -= d
            # tol 0: all 20 iterations, so both solves sit on their fixed points
            up = A.eikonal3d(u0, fp.reshape(f.shape), h, m, n, l, 0.0)
            um = A.eikonal3d(u0, fm.reshape(f.shape), h, m, n, l, 0.0)
            fd = (misfit(up) - misfit(um)) / (2 * d)
            g = gf.ravel()[c]
            assert abs(fd - g) <= tol_fd * abs(g), (c, rel, fd, g)


def test_2d_c1_config_forward_and_grad():
    """101x101, h=1, 6 km/s with 3 Gaussian anomalies, interior source, L2
    misfit at 20 receivers against times from a +2%-noise velocity."""
    rng = np.random.default_rng(2)
    v = synth.gaussian_anomalies_2d(101, 101, rng)
    f = 1.0 / v
    ix, jx = (int(x) for x in rng.integers(5, 96, size=2))
    u, st = A.eikonal(f, ix + 1, jx + 1, 1.0, return_status=True)
    ur, it, conv = O.eik2d_forward(f, ix, jx, 1.0)
    assert np.array_equal(u, ur) and st.iters == it and st.converged == conv
    f_obs = 1.0 / (v * (1 + 0.02 * rng.standard_normal(v.shape)))
    uo = A.eikonal(f_obs, ix + 1, jx + 1, 1.0)
    rec = rng.integers(0, 101, size=(20, 2))
    gu = np.zeros_like(u)
    for r in rec:
        gu[r[0], r[1]] += -2 * (uo[r[0], r[1]] - u[r[0], r[1]])
    gf = A.eikonal_grad(gu, u, f, ix + 1, jx + 1, 1.0)
    assert np.array_equal(gf, O.eik2d_backward(gu, ur, f, ix, jx, 1.0))


@pytest.mark.parametrize("shape,src", [((120, 121), (60, 2)), ((140, 150), (3, 130)),
                                       ((161, 200), (150, 7))])
def test_2d_grids_beyond_the_shared_memory_paths(shape, src):
    """Grids of 14520, 21000 and 32200 nodes: the forward keeps its travel
    times and change flags in shared memory up to 25600 nodes; the adjoint
    by levels keeps its working set there up to 17600 (the travel times too
    up to 12200), and beyond that the causal adjoint works in global memory.
    Bit-identical to the oracle, with the exact skipping of unchanged nodes
    in the forward."""
    rng = np.random.default_rng(5)
    f = rng.uniform(0.4, 1.6, size=shape)
    jx, ix = src
    u, st = A.eikonal(f, ix + 1, jx + 1, 0.3, return_status=True)
    ur, it, conv = O.eik2d_forward(f, ix, jx, 0.3)
    assert np.array_equal(u, ur) and st.iters == it and st.converged == conv
    gu = np.zeros_like(u)
    gu[rng.integers(0, shape[0], 40), rng.integers(0, shape[1], 40)] = rng.standard_normal(40)
    gf = A.eikonal_grad(gu, u, f, ix + 1, jx + 1, 0.3)
    assert np.array_equal(gf, O.eik2d_backward(gu, ur, f, ix, jx, 0.3))


@pytest.mark.parametrize("src", [(0, 0), (36, 52), (0, 52), (36, 0), (18, 0), (0, 26)])
def test_2d_sources_on_corners_and_edges(src):
    """Sources on the grid's corners and edges: the one-sided neighbour rule
    (Eikonal.h:14-20 callers) through the forward's exact skipping and the
    adjoint by levels, bit-identical to the oracle."""
    rng = np.random.default_rng(6)
    f = rng.uniform(0.5, 1.5, size=(37, 53))
    jx, ix = src
    u, st = A.eikonal(f, ix + 1, jx + 1, 0.5, return_status=True)
    ur, it, conv = O.eik2d_forward(f, ix, jx, 0.5)
    assert np.array_equal(u, ur) and st.iters == it and st.converged == conv
    gu = np.zeros_like(u)
    gu[rng.integers(0, 37, 12), rng.integers(0, 53, 12)] = rng.standard_normal(12)
    gf = A.eikonal_grad(gu, u, f, ix + 1, jx + 1, 0.5)
    assert np.array_equal(gf, O.eik2d_backward(gu, ur, f, ix, jx, 0.5))


def test_2d_batch_beyond_shared_memory():
    """Several sources on a 32200-node grid: the forward's global-memory path
    with a change-flag array per solve."""
    rng = np.random.default_rng(7)
    f = rng.uniform(0.5, 1.5, size=(161, 200))
    sx = rng.integers(1, 201, size=3)
    sy = rng.integers(1, 162, size=3)
    u, st = A.eikonal_batch(f, sx, sy, 0.4)
    for k in range(3):
        ur, it, conv = O.eik2d_forward(f, sx[k] - 1, sy[k] - 1, 0.4)
        assert np.array_equal(u[k], ur)
        assert st[k] == (it, int(conv))


def test_2d_adjoint_singular_row_is_an_error():
    """A non-source cell with no upwind direction (u smaller than all four
    neighbours away from the source) leaves its adjoint row without a
    diagonal: ADT_ESINGULAR, where the reference's SparseLU fails silently.
    The same travel times without that minimum give a finite gradient."""
    m = n = 12
    f = np.ones((n + 1, m + 1))
    u = A.eikonal(f, 4, 4, 1.0)
    gu = np.ones_like(u)
    assert np.all(np.isfinite(A.eikonal_grad(gu, u, f, 4, 4, 1.0)))
    bad = u.copy()
    bad[9, 9] = min(bad[8, 9], bad[10, 9], bad[9, 8], bad[9, 10]) - 0.5
    with pytest.raises(A.AdtError) as e:
        A.eikonal_grad(gu, bad, f, 4, 4, 1.0)
    assert e.value.name == "ADT_ESINGULAR"


def test_2d_batch_matches_single_solves():
    rng = np.random.default_rng(4)
    f = rng.uniform(0.5, 1.5, size=(23, 31))
    sx = rng.integers(1, 32, size=5)
    sy = rng.integers(1, 24, size=5)
    u, st = A.eikonal_batch(f, sx, sy, 0.7)
    for k in range(5):
        ur, it, conv = O.eik2d_forward(f, sx[k] - 1, sy[k] - 1, 0.7)
        assert np.array_equal(u[k], ur)
        assert st[k] == (it, int(conv))


# --------------------------------------------------------- batched ------
def make_batch(rng, fields_dims, n_src, n_sta, missing=0.1):
    fields, stations, slow = [], [], []
    for (m, n, l, h) in fields_dims:
        fields.append((m, n, l, h))
        slow.append(synth.layered_checkerboard(m, n, l, block=4))
        sta = synth.surface_stations(m, n, n_sta, rng)
        sta[0] = [0.0, 0.0, 0.0]  # integer position: x1 == x2 branches
        sta[1] = [m - 1, 2.5, 0.0]
        stations.append(sta)
    solve_field, src = [], []
    for s in range(n_src):
        fi = s % len(fields_dims)
        m, n, l, _ = fields_dims[fi]
        solve_field.append(fi)
        src.append(synth.volume_sources(m, n, l, 1, rng)[0])
    src[0] = [0.0, 0.0, 0.0]  # a corner source
    n_obs = sum(len(stations[fi]) for fi in solve_field)
    t_obs = rng.uniform(0.5, 3.0, n_obs)
    t_obs[rng.random(n_obs) < missing] = -1.0
    w = rng.uniform(0.5, 1.0, n_obs)
    w[3] = 0.0
    return fields, stations, slow, np.array(solve_field), np.array(src), t_obs, w


def oracle_batch(fields, stations, slow, sf, src, t_obs, w, tol, max_iter):
    return O.batch_misfit_grad([(s, f[3]) for s, f in zip(slow, fields)], stations, sf, src, t_obs,
                               w, tol=tol, max_iter=max_iter)


def test_batch_fp64_ref_compat_bit_exact():
    rng = np.random.default_rng(7)
    fields, stations, slow, sf, src, t_obs, w = make_batch(
        rng, [(20, 17, 13, 0.5), (12, 26, 40, 0.25)], 6, 9)
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F64, tol=1e-6, ref_compat=True,
                  adj_solver="sweeps")
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, ito = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-6, 20)
    assert np.array_equal(tp, tpo)
    assert mis == mo
    for g, r in zip(grads, go):
        assert np.array_equal(g, r)
    assert [s.iters for s in st] == list(ito)
    B.close()


def test_batch_near_source_rules_bit_exact():
    """The batched plan builds u0 exactly as the reference's callers do, for
    sources whose 8-node box straddles checkerboard block edges in x, y and z
    (so every node of the box has its own slowness):
    - default: scripts/gene_obs.jl:42-51, r * f * h with f taken at the
      (ceil x, ceil y) column, one value per depth plane;
    - set_source_velocity(vel0): scripts/inversion.jl:52-60, r * h / vel0[node].
    FP64 with the reference stopping rule: misfit, predicted times, gradient
    and iteration counts bit-identical to the oracle in both modes."""
    rng = np.random.default_rng(31)
    m, n, l, h = 20, 18, 14, 0.5
    f = synth.layered_checkerboard(m, n, l, block=4)
    vel0 = 1.0 / synth.layered_checkerboard(m, n, l, block=2)
    sta = synth.surface_stations(m, n, 7, rng)
    # block edges at multiples of 4: every source box straddles one in x and y,
    # the first two in z as well
    src = np.array([[3.6, 7.3, 3.5], [11.25, 3.8, 7.1], [7.5, 11.6, 5.4]])
    sf = np.zeros(len(src), np.int32)
    t_obs = rng.uniform(0.5, 3.0, 7 * len(src))
    t_obs[4] = -1.0
    w = rng.uniform(0.5, 1.0, t_obs.size)
    B = A.Batch3D([(m, n, l, h)], [sta], sf, src, precision=A.ADT_F64, tol=1e-6, ref_compat=True)
    out = {}
    for mode in ("gene_obs", "inversion"):
        B.set_source_velocity([vel0] if mode == "inversion" else None)
        mis, tp, (g,), st = B.run([f], t_obs, w)
        mo, tpo, (go,), ito = O.batch_misfit_grad(
            [(f, h)], [sta], sf, src, t_obs, w, tol=1e-6, max_iter=20, src_mode=mode,
            src_model=[vel0] if mode == "inversion" else None)
        assert mis == mo, mode
        assert np.array_equal(tp, tpo), mode
        assert np.array_equal(g, go), mode
        assert [s.iters for s in st] == list(ito), mode
        out[mode] = tp
    # the per-node slowness variant differs here, so the test sees the rule
    _, tpn, _, _ = O.batch_misfit_grad([(f, h)], [sta], sf, src, t_obs, w, tol=1e-6, max_iter=20,
                                       src_mode="node")
    assert not np.array_equal(tpn, out["gene_obs"])
    assert not np.array_equal(out["inversion"], out["gene_obs"])
    B.close()


def test_batch_fp32_accuracy_against_fp64():
    rng = np.random.default_rng(8)
    fields, stations, slow, sf, src, t_obs, w = make_batch(
        rng, [(40, 36, 24, 0.5), (24, 24, 48, 0.5)], 8, 12)
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-7)
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, _ = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-12, 100)
    ok = tpo > 0
    assert np.max(np.abs(tp[ok] - tpo[ok]) / tpo[ok]) <= 1e-4
    assert abs(mis - mo) <= 1e-3 * mo
    for g, r in zip(grads, go):
        assert np.linalg.norm(g - r) <= 1e-3 * np.linalg.norm(r)
    assert all(s.converged and s.adj_converged for s in st)
    B.close()


def test_batch_causal_adjoint_fp64_bit_exact():
    """The causal-order adjoint (adj_solver "causal") in FP64 with the
    reference stopping rule: misfit, predicted times and gradient
    bit-identical to the oracle (whose adjoint is the same substitution in
    travel-time order), on two fields whose depths are not multiples of 4
    (the per-cell code passes), a corner source and missing picks."""
    rng = np.random.default_rng(7)
    fields, stations, slow, sf, src, t_obs, w = make_batch(
        rng, [(20, 17, 13, 0.5), (12, 26, 41, 0.25)], 6, 9)
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F64, tol=1e-6, ref_compat=True,
                  adj_solver="causal")
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, ito = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-6, 20)
    assert np.array_equal(tp, tpo)
    assert mis == mo
    for g, r in zip(grads, go):
        assert np.array_equal(g, r)
    assert all(s.adj_converged == 1 and s.adj_iters == 1 for s in st)  # one pass
    stats = B.stats()
    assert stats.adj_groups == 1 and stats.adj_bricks == 0
    assert stats.adj_cell_updates > 0
    B.close()


@pytest.mark.parametrize("dims", [[(40, 36, 24, 0.5), (24, 24, 48, 0.5)],
                                  [(33, 29, 21, 0.5), (18, 22, 30, 0.4)]],
                         ids=["l8", "ragged"])
def test_batch_causal_adjoint_fp32_equals_exact_sweeps(dims):
    """FP32: the causal-order adjoint evaluates every cell once with the
    sweeping adjoint's formula, so its gradient equals the exact sweeps'
    fixed point (adj_wake_tol 0).  Bit for bit where both use the vector
    code passes and tiles (depths multiple of 8); on ragged depths the sweeps'
    per-cell tile path sums in another order, so there to 1e-5 relative.
    Both against the FP64 oracle as well."""
    rng = np.random.default_rng(11)
    fields, stations, slow, sf, src, t_obs, w = make_batch(rng, dims, 8, 12)
    out = {}
    for solver in ("sweeps", "causal"):
        B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-7,
                      adj_solver=solver)
        out[solver] = B.run(slow, t_obs, w)
        assert all(s.converged and s.adj_converged for s in out[solver][3])
        B.close()
    (ms, tps, gs, _), (mc, tpc, gc, stc) = out["sweeps"], out["causal"]
    assert np.array_equal(tps, tpc) and ms == mc  # same forward
    assert all(s.adj_iters == 1 for s in stc)  # one pass of the causal solve
    exact = all(f[2] % 8 == 0 for f in dims)
    for a, b in zip(gs, gc):
        if exact:
            assert np.array_equal(a, b)
        else:
            assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(a)
    mo, tpo, go, _ = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-12, 100)
    for g, r in zip(gc, go):
        assert np.linalg.norm(g - r) <= 1e-3 * np.linalg.norm(r)


def test_batch_causal_adjoint_chunking_and_overlap():
    """Chunks of 3 solves, one or two resident: the gradient (FP64 sum in
    solve order) is the same bits as all solves at once."""
    rng = np.random.default_rng(12)
    fields, stations, slow, sf, src, t_obs, w = make_batch(
        rng, [(32, 28, 24, 0.5), (20, 24, 16, 0.5)], 8, 10)
    ref = None
    for kw in ({}, {"chunk": 3}, {"chunk": 3, "overlap_chunks": True}):
        B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-7,
                      adj_solver="causal", **kw)
        mis, tp, grads, st = B.run(slow, t_obs, w)
        B.close()
        if ref is None:
            ref = (mis, tp, grads)
            continue
        assert mis == ref[0] and np.array_equal(tp, ref[1]), kw
        for g, r in zip(grads, ref[2]):
            assert np.array_equal(g, r), kw


def _fp32_vs_fp64_full_grid(fields, stations, slow, slow_obs, sf, src, **kw):
    """FP32 plan with the bench's wake tolerances against the reference's FP64
    op (the oracle: tol 1e-6, 20 iterations, exact causal adjoint) on the same
    picks: FP64 travel times on the perturbed model (the library's FP64 plan
    with the reference stopping rule, bit-exact to the oracle)."""
    n_obs = sum(len(stations[fi]) for fi in sf)
    w = np.ones(n_obs)
    P = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F64, tol=1e-6, ref_compat=True)
    _, t_obs, _, _ = P.run(slow_obs, np.full(n_obs, 1.0), w)
    P.close()
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-6, wake_tol=1e-6,
                  **({"adj_wake_tol": 1e-5} | kw))
    mis, tp, grads, st = B.run(slow, t_obs, w)
    B.close()
    assert all(s.converged and s.adj_converged for s in st)
    mo, tpo, go, _ = O.batch_misfit_grad([(s_, f_[3]) for s_, f_ in zip(slow, fields)], stations,
                                         sf, src, t_obs, w, tol=1e-6, max_iter=20,
                                         nthreads=os.cpu_count() or 1)
    # tolerances: travel times 1e-4 relative (max over picks), gradient 1e-3
    # relative (L2, each field), misfit 1e-3 relative
    assert np.max(np.abs(tp - tpo) / tpo) <= 1e-4
    assert abs(mis - mo) <= 1e-3 * mo
    for g, r in zip(grads, go):
        assert np.linalg.norm(g - r) <= 1e-3 * np.linalg.norm(r)


def test_batch_fp32_c3_full_grid_against_fp64():
    """The headline configuration's grid at full size: 128x128x64, h = 0.5 km,
    layered 4-8 km/s x (1 +- 5%) 8-cell checkerboard, 100 surface stations,
    8 events uniform in the volume, picks from a +2%-noise model."""
    rng = np.random.default_rng(0)
    m, n, l, h = 128, 128, 64, 0.5
    f = synth.layered_checkerboard(m, n, l, block=8)
    sta = synth.surface_stations(m, n, 100, rng)
    src = synth.volume_sources(m, n, l, 8, rng)
    f_obs = f / (1.0 + 0.02 * rng.standard_normal(f.shape))
    _fp32_vs_fp64_full_grid([(m, n, l, h)], [sta], [f], [f_obs], np.zeros(8, np.int32), src)


def test_batch_fp32_c3_full_grid_causal_adjoint_against_fp64():
    """As above with the causal-order adjoint (no adjoint wake tolerance)."""
    rng = np.random.default_rng(0)
    m, n, l, h = 128, 128, 64, 0.5
    f = synth.layered_checkerboard(m, n, l, block=8)
    sta = synth.surface_stations(m, n, 100, rng)
    src = synth.volume_sources(m, n, l, 8, rng)
    f_obs = f / (1.0 + 0.02 * rng.standard_normal(f.shape))
    _fp32_vs_fp64_full_grid([(m, n, l, h)], [sta], [f], [f_obs], np.zeros(8, np.int32), src,
                            adj_solver="causal")


def test_batch_fp32_c4_largest_grid_p_and_s_against_fp64():
    """The uneven P/S configuration's largest grid at full size: 160x160x80,
    h = 0.5 km, Vp layered 4-8 km/s x (1 +- 5%) smooth, Vs = Vp / 1.73, 150
    surface stations, 2 events with a P and an S solve each."""
    rng = np.random.default_rng(4)
    m, n, l, h = 160, 160, 80, 0.5
    vp = synth.layered_smooth(m, n, l, rng)
    sta = synth.surface_stations(m, n, 150, rng)
    ev = synth.volume_sources(m, n, l, 2, rng)
    fields = [(m, n, l, h), (m, n, l, h)]
    slow = [1.0 / vp, 1.73 / vp]
    slow_obs = [s_ * 1.02 for s_ in slow]
    sf = np.array([0, 1, 0, 1], np.int32)
    src = np.repeat(ev, 2, axis=0)
    _fp32_vs_fp64_full_grid(fields, [sta, sta], slow, slow_obs, sf, src)


def test_batch_fp32_wake_tolerances_against_fp64():
    """Bricks that moved by at most wake_tol (forward, seconds) or adj_wake_tol
    (adjoint, relative) wake no neighbours: results stay within the FP32
    tolerances of the converged FP64 oracle, and stay independent of the
    launch shape."""
    rng = np.random.default_rng(8)
    fields, stations, slow, sf, src, t_obs, w = make_batch(
        rng, [(40, 36, 24, 0.5), (24, 24, 48, 0.5)], 8, 12)
    mo, tpo, go, _ = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-12, 100)
    ok = tpo > 0
    first = None
    for kw in ({"wake_tol": 1e-6, "adj_wake_tol": 1e-5}, {"wake_tol": 1e-6, "adj_wake_tol": 1e-5,
                                                          "warps": 3, "groups": 2},
               {"wake_tol": 1e-5, "adj_wake_tol": 1e-4}):
        B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-6,
                      adj_solver="sweeps", **kw)
        mis, tp, grads, st = B.run(slow, t_obs, w)
        # tolerances: travel times 1e-4 relative, gradient 1e-3 relative (L2)
        assert np.max(np.abs(tp[ok] - tpo[ok]) / tpo[ok]) <= 1e-4, kw
        assert abs(mis - mo) <= 1e-3 * mo, kw
        for g, r in zip(grads, go):
            assert np.linalg.norm(g - r) <= 1e-3 * np.linalg.norm(r), kw
        assert all(s.converged and s.adj_converged for s in st), kw
        if first is None:
            first = (tp, grads[0])
        elif "warps" in kw:
            assert np.array_equal(tp, first[0]) and np.array_equal(grads[0], first[1])
        B.close()
    with pytest.raises(A.AdtError):
        A.Batch3D(fields, stations, sf, src, wake_tol=-1.0)
    with pytest.raises(A.AdtError):
        A.Batch3D(fields, stations, sf, src, adj_wake_tol=float("nan"))


def test_batch_adjoint_order_filter_is_exact():
    """Sweeping each adjoint brick only in the orderings that follow its flow
    (adt_batch_opts.adj_order_filter, the default) reaches the same unique
    fixed point of the triangular adjoint system: with exact skipping the
    predicted times, misfit and gradient are bit-identical with and without
    the filter, in FP32 and FP64, while fewer bricks are swept."""
    rng = np.random.default_rng(21)
    fields, stations, slow, sf, src, t_obs, w = make_batch(
        rng, [(40, 36, 24, 0.5), (24, 24, 48, 0.5)], 8, 12)
    for prec in (A.ADT_F32, A.ADT_F64):
        out = []
        for filt in (True, False):
            B = A.Batch3D(fields, stations, sf, src, precision=prec, tol=1e-7,
                          adj_order_filter=filt, adj_solver="sweeps")
            mis, tp, grads, st = B.run(slow, t_obs, w)
            out.append((mis, tp, grads, B.stats().adj_bricks, st))
            B.close()
        (m1, tp1, g1, b1, st1), (m0, tp0, g0, b0, st0) = out
        assert m1 == m0 and np.array_equal(tp1, tp0), prec
        for a, b in zip(g1, g0):
            assert np.array_equal(a, b), prec
        assert all(s.adj_converged for s in st1) and all(s.adj_converged for s in st0)
        assert b1 < b0, (prec, b1, b0)


def test_batch_fp32_forward_order_filter_against_fp64():
    """FP32 forward sweeping each brick only in the orderings that follow the
    upwind directions its sweeps have seen (adt_batch_opts.fwd_order_filter):
    the same fixed point along another iteration path, so results stay within
    the FP32 tolerances of the converged FP64 oracle (travel times 1e-4
    relative, gradient 1e-3 relative L2), alone and with the wake tolerances,
    and do not depend on the launch shape."""
    rng = np.random.default_rng(8)
    fields, stations, slow, sf, src, t_obs, w = make_batch(
        rng, [(40, 36, 24, 0.5), (24, 24, 48, 0.5)], 8, 12)
    mo, tpo, go, _ = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-12, 100)
    ok = tpo > 0
    first = None
    for kw in ({}, {"warps": 3, "groups": 2}, {"wake_tol": 1e-6, "adj_wake_tol": 1e-5}):
        B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-7,
                      fwd_order_filter=True, **kw)
        mis, tp, grads, st = B.run(slow, t_obs, w)
        B.close()
        assert np.max(np.abs(tp[ok] - tpo[ok]) / tpo[ok]) <= 1e-4, kw
        assert abs(mis - mo) <= 1e-3 * mo, kw
        for g, r in zip(grads, go):
            assert np.linalg.norm(g - r) <= 1e-3 * np.linalg.norm(r), kw
        assert all(s.converged and s.adj_converged for s in st), kw
        if first is None:
            first = (tp, grads[0])
        elif "warps" in kw:
            assert np.array_equal(tp, first[0]) and np.array_equal(grads[0], first[1])


def test_batch_run_into_caller_buffers():
    rng = np.random.default_rng(12)
    fields, stations, slow, sf, src, t_obs, w = make_batch(rng, [(18, 14, 20, 0.5)], 5, 6)
    B = A.Batch3D(fields, stations, sf, src)
    mis, tp, grads, _ = B.run(slow, t_obs, w)
    out = (np.full(tp.size, np.nan), np.full(grads[0].size, np.nan))
    mis2, tp2, grads2, _ = B.run(slow, t_obs, w, out=out)
    assert mis2 == mis and np.array_equal(tp2, tp) and np.array_equal(grads2[0], grads[0])
    assert np.shares_memory(tp2, out[0]) and np.shares_memory(grads2[0], out[1])
    with pytest.raises(A.AdtError):
        B.run(slow, t_obs, w, out=(np.empty(tp.size), np.empty(3)))
    with pytest.raises(A.AdtError):
        B.run(slow, t_obs, w, out=(np.empty(tp.size, np.float32), out[1]))
    B.close()


def test_batch_chunking_and_graph_do_not_change_results():
    """Chunking (one chunk at a time, or two overlapping on two streams), graph
    replay and launch shapes change only the schedule: the same bits and
    iteration counts.  The brick depth changes the bricks the
    ordering filters work on: without the forward filter (the adjoint's is
    exact) the results are still the same bits; with it (the FP32 default) the
    forward stops at its tolerance after another iteration path, within 1e-6
    relative of the same result."""
    rng = np.random.default_rng(9)
    fields, stations, slow, sf, src, t_obs, w = make_batch(rng, [(18, 14, 20, 0.5)], 7, 6)
    ref = A.Batch3D(fields, stations, sf, src, use_graph=False)
    r = ref.run(slow, t_obs, w)
    ref_x = A.Batch3D(fields, stations, sf, src, use_graph=False, fwd_order_filter=False)
    rx = ref_x.run(slow, t_obs, w)
    for kw in ({"chunk": 3}, {"chunk": 1, "use_graph": True}, {"bk": 64}, {"bk": 16}, {"warps": 3},
               {"warps": 1, "groups": 1}, {"warps": 2, "groups": 5},
               {"chunk": 3, "overlap_chunks": True}, {"chunk": 2, "overlap_chunks": True},
               {"chunk": 2, "overlap_chunks": True, "use_graph": False}):
        B = A.Batch3D(fields, stations, sf, src, **kw)
        out = B.run(slow, t_obs, w)
        if "bk" in kw:
            assert np.all(np.abs(out[1] - r[1]) <= 1e-6 * np.abs(r[1])), kw
            assert np.linalg.norm(out[2][0] - r[2][0]) <= 1e-5 * np.linalg.norm(r[2][0]), kw
            X = A.Batch3D(fields, stations, sf, src, fwd_order_filter=False, **kw)
            ox = X.run(slow, t_obs, w)
            X.close()
            assert ox[0] == rx[0] and np.array_equal(ox[1], rx[1]), kw
            assert np.array_equal(ox[2][0], rx[2][0]), kw
            assert [x.iters for x in ox[3]] == [x.iters for x in rx[3]], kw
        else:
            assert out[0] == r[0], kw
            assert np.array_equal(out[1], r[1]), kw
            assert np.array_equal(out[2][0], r[2][0]), kw
            assert ([(x.iters, x.adj_iters) for x in out[3]] ==
                    [(x.iters, x.adj_iters) for x in r[3]]), kw
        # a second evaluation of the same plan reproduces the first
        out2 = B.run(slow, t_obs, w)
        assert np.array_equal(out2[2][0], out[2][0]), kw
        B.close()
    ref.close()
    ref_x.close()


def test_batch_overlapping_chunks_uneven_fields():
    """Two chunks resident on two streams (overlap_chunks) with solves on
    fields of different size, ragged chunk counts and graph replay on and
    off: the same bits as one chunk of all solves, FP32 and FP64; with the
    reference stopping rule (one buffer set, overlap ignored) bit-exact to
    the oracle."""
    rng = np.random.default_rng(17)
    fields, stations, slow, sf, src, t_obs, w = make_batch(
        rng, [(20, 18, 14, 0.5), (12, 26, 40, 0.25)], 9, 7)
    for prec in (A.ADT_F32, A.ADT_F64):
        R = A.Batch3D(fields, stations, sf, src, precision=prec, tol=1e-6)
        r = R.run(slow, t_obs, w)
        R.close()
        for kw in ({"chunk": 2}, {"chunk": 4, "use_graph": False}, {"chunk": 5}):
            B = A.Batch3D(fields, stations, sf, src, precision=prec, tol=1e-6, overlap_chunks=True,
                          **kw)
            for _ in range(2):  # replays reuse both buffer sets
                out = B.run(slow, t_obs, w)
                assert out[0] == r[0] and np.array_equal(out[1], r[1]), (prec, kw)
                for a, b in zip(out[2], r[2]):
                    assert np.array_equal(a, b), (prec, kw)
            B.close()
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F64, tol=1e-6, ref_compat=True,
                  chunk=3, overlap_chunks=True)
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, ito = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-6, 20)
    assert mis == mo and np.array_equal(tp, tpo)
    for g, r_ in zip(grads, go):
        assert np.array_equal(g, r_)
    assert [x.iters for x in st] == list(ito)
    B.close()


def test_batch_nonconvergence_is_reported():
    rng = np.random.default_rng(10)
    fields, stations, slow, sf, src, t_obs, w = make_batch(rng, [(30, 30, 20, 0.5)], 2, 5)
    B = A.Batch3D(fields, stations, sf, src, max_iter=1, adj_max_iter=1)
    _, _, _, st = B.run(slow, t_obs, w)
    assert all(s.iters == 1 and s.converged == 0 for s in st)
    B.close()


def test_batch_rejects_bad_geometry():
    with pytest.raises(A.AdtError):
        A.Batch3D([(10, 10, 10, 1.0)], [np.array([[11.0, 0.0, 0.0]])], [0], [[1.0, 1.0, 1.0]])
    with pytest.raises(A.AdtError):
        A.Batch3D([(10, 10, 10, 1.0)], [np.zeros((1, 3))], [0], [[-0.5, 1.0, 1.0]])
    with pytest.raises(A.AdtError):
        A.Batch3D([(10, 10, 10, 1.0)], [np.zeros((1, 3))], [1], [[1.0, 1.0, 1.0]])


def test_batch_c4_multi_field_uneven_grids():
    """The C4 layout at reduced size: four grids of different sizes, each with
    a P and an S field (Vs = Vp / 1.73, layered + smooth random), every event
    solved on both fields; FP32 plan against the FP64 oracle, gradients with
    respect to all eight slownesses."""
    rng = np.random.default_rng(11)
    grids = [(16, 16, 8, 0.5), (24, 24, 12, 0.5), (32, 32, 16, 0.5), (40, 40, 20, 0.5)]
    fields, stations, slow = [], [], []
    for (m, n, l, h) in grids:
        vp = synth.layered_smooth(m, n, l, rng, corr=3.0)
        sta = synth.surface_stations(m, n, 12, rng)
        for v in (vp, vp / 1.73):
            fields.append((m, n, l, h))
            slow.append(1.0 / v)
            stations.append(sta)
    sf, src = [], []
    for gi, (m, n, l, _) in enumerate(grids):
        for e in synth.volume_sources(m, n, l, 3, rng):
            for ph in range(2):
                sf.append(2 * gi + ph)
                src.append(e)
    sf, src = np.array(sf), np.array(src)
    n_obs = sum(len(stations[f]) for f in sf)
    t_obs = rng.uniform(0.5, 3.0, n_obs)
    t_obs[rng.random(n_obs) < 0.1] = -1.0
    w = rng.uniform(0.5, 1.0, n_obs)
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-7)
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, _ = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-12, 100)
    ok = tpo > 0
    assert np.max(np.abs(tp[ok] - tpo[ok]) / tpo[ok]) <= 1e-4
    assert abs(mis - mo) <= 1e-3 * mo
    assert len(grads) == 8
    for g, r in zip(grads, go):
        assert np.linalg.norm(g - r) <= 1e-3 * np.linalg.norm(r)
    assert all(s.converged and s.adj_converged for s in st)
    B.close()


def test_batch_fp32_mixed_fields_alignment():
    """A field whose cell count is not a multiple of 4 ahead of a field that
    takes the 16-byte-access FP32 path: every solve's buffers must still start
    aligned (results against the FP64 oracle)."""
    rng = np.random.default_rng(12)
    fields, stations, slow, sf, src, t_obs, w = make_batch(
        rng, [(9, 7, 13, 0.5), (16, 12, 20, 0.5), (11, 9, 7, 0.5), (12, 16, 24, 0.5)], 8, 6)
    assert fields[0][0] * fields[0][1] * fields[0][2] % 4 != 0
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-7)
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, _ = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-12, 100)
    ok = tpo > 0
    assert np.max(np.abs(tp[ok] - tpo[ok]) / tpo[ok]) <= 1e-4
    for g, r in zip(grads, go):
        assert np.linalg.norm(g - r) <= 1e-3 * np.linalg.norm(r)
    assert all(s.converged and s.adj_converged for s in st)
    B.close()


def test_batch_many_bricks_global_meta():
    """A grid with more bricks (33 x 65 x 1 = 2145) than the per-group
    shared-memory metadata holds, so brick timestamps live in global memory,
    as on the 256x256x128 grids of the largest configuration: FP64 with the
    reference stopping rule bit-exact, FP32 within tolerance."""
    rng = np.random.default_rng(13)
    fields, stations, slow, sf, src, t_obs, w = make_batch(rng, [(264, 260, 8, 0.5)], 2, 10)
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F64, tol=1e-6, ref_compat=True)
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, ito = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-6, 20)
    assert np.array_equal(tp, tpo) and mis == mo
    assert np.array_equal(grads[0], go[0])
    assert [s.iters for s in st] == list(ito)
    B.close()
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-7)
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, _ = oracle_batch(fields, stations, slow, sf, src, t_obs, w, 1e-12, 100)
    ok = tpo > 0
    assert np.max(np.abs(tp[ok] - tpo[ok]) / tpo[ok]) <= 1e-4
    assert np.linalg.norm(grads[0] - go[0]) <= 1e-3 * np.linalg.norm(go[0])
    assert all(s.converged and s.adj_converged for s in st)
    B.close()


def test_batch_autotune_keeps_results():
    rng = np.random.default_rng(14)
    fields, stations, slow, sf, src, t_obs, w = make_batch(rng, [(32, 24, 16, 0.5)], 6, 8)
    ref = A.Batch3D(fields, stations, sf, src)
    r = ref.run(slow, t_obs, w)
    B = A.Batch3D(fields, stations, sf, src)
    with pytest.raises(A.AdtError):
        B.autotune()  # inputs not uploaded yet
    B.upload(slow, t_obs, w)
    st = B.autotune(reps=1)
    assert st.warps >= 1 and st.groups >= 1 and st.adj_warps >= 1 and st.adj_groups >= 1
    out = B.run(slow, t_obs, w)
    assert out[0] == r[0] and np.array_equal(out[1], r[1]) and np.array_equal(out[2][0], r[2][0])
    B.close()
    ref.close()
    P = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F64, ref_compat=True)
    P.upload(slow, t_obs, w)
    with pytest.raises(A.AdtError):
        P.autotune()
    P.close()


def test_batch_many_receivers_global_merge():
    """More receivers per field (1500) than the shared-memory seed merge takes,
    as when events are the receivers (scripts/inversion.jl uses stations as
    sources): FP64 bit-exact, FP32 within tolerance."""
    rng = np.random.default_rng(15)
    m, n, l, h = 40, 36, 16, 0.5
    slow = [synth.layered_checkerboard(m, n, l, block=4)]
    rec = np.c_[rng.uniform(0, m - 1, 1500), rng.uniform(0, n - 1, 1500), rng.uniform(0, l - 1, 1500)]
    rec[:40] = np.round(rec[:40])  # integer positions share nodes with neighbours
    src = synth.surface_stations(m, n, 3, rng)
    sf = np.zeros(3, np.int32)
    t_obs = rng.uniform(0.5, 3.0, 4500)
    t_obs[rng.random(4500) < 0.1] = -1.0
    w = rng.uniform(0.5, 1.0, 4500)
    fields = [(m, n, l, h)]
    B = A.Batch3D(fields, [rec], sf, src, precision=A.ADT_F64, tol=1e-6, ref_compat=True)
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, _ = oracle_batch(fields, [rec], slow, sf, src, t_obs, w, 1e-6, 20)
    assert np.array_equal(tp, tpo) and mis == mo and np.array_equal(grads[0], go[0])
    B.close()
    B = A.Batch3D(fields, [rec], sf, src, precision=A.ADT_F32, tol=1e-7)
    mis, tp, grads, st = B.run(slow, t_obs, w)
    mo, tpo, go, _ = oracle_batch(fields, [rec], slow, sf, src, t_obs, w, 1e-12, 100)
    ok = tpo > 0
    assert np.max(np.abs(tp[ok] - tpo[ok]) / tpo[ok]) <= 1e-4
    assert np.linalg.norm(grads[0] - go[0]) <= 1e-3 * np.linalg.norm(go[0])
    B.close()
