"""Index arithmetic of the 3D brick sweeps, enumerated on the CPU against the
library's own tile layout (adt_tile_layout): the pipelined FP32 sweep steps
are bank-conflict-free in every ordering, every shared address a sweep
touches (lanes outside their window included) stays inside the warp's
tiles, and the unchecked staging of full bricks issues exactly the copies of
the generic staging loops.  (The adjoint's uint16 code load, two codes per
word on the same column stride, takes two passes; every float access one.)
No GPU needed.

The address model restates eik3d_brick.cuh: lane L owns column (L >> 2,
L & 3), mirrored per ordering; at step tau it works on cell kk = tau - s
(s = li + lj) and touches the offsets listed below."""
import ctypes as C

import numpy as np
import pytest

import adtomo_gb300 as A

BI, BJ, SKEW = 8, 4, 10
ORDERINGS = [(si, sj, sk) for sk in (1, -1) for sj in (1, -1) for si in (1, -1)]


def layout(bk):
    out = (C.c_int32 * 6)()
    assert A.lib().adt_tile_layout(bk, out) == 0
    rs, irs, cs_same, cs_diff, te, ite = out
    return rs, irs, cs_same, cs_diff, te, ite


def lanes(si, sj):
    lane = np.arange(32)
    li, lj = lane >> 2, lane & 3
    pi = li if si > 0 else BI - 1 - li
    pj = lj if sj > 0 else BJ - 1 - lj
    return pi, pj, li + lj


def wavefronts(word_addrs):
    """Shared-memory passes for one warp access: the most distinct 4-byte
    words that fall in one of the 32 banks."""
    words = np.unique(np.asarray(word_addrs))
    return int(np.bincount(words % 32, minlength=32).max())


@pytest.mark.parametrize("bk", [16, 32, 64])
def test_layout_constants(bk):
    rs, irs, cs_same, cs_diff, te, ite = layout(bk)
    assert rs % 32 == 0 and irs % 32 == 0
    assert cs_same % 16 == 9 and cs_diff % 16 == 7
    assert min(cs_same, cs_diff) >= bk + 2 and 6 * max(cs_same, cs_diff) <= rs
    assert te == (BI + 2) * rs and ite == BI * irs
    out = (C.c_int32 * 6)()
    assert A.lib().adt_tile_layout(8, out) != 0


@pytest.mark.parametrize("bk", [16, 32, 64])
@pytest.mark.parametrize("order", ORDERINGS)
def test_sweep_steps_are_bank_conflict_free(bk, order):
    si, sj, sk = order
    rs, irs, cs_same, cs_diff, te, ite = layout(bk)
    cs = cs_same if sj == sk else cs_diff
    pi, pj, s = lanes(si, sj)
    kb = 0 if sk > 0 else bk - 1
    own = (pi + 1) * rs + (pj + 1) * cs + 1 + kb
    fown = pi * irs + pj * cs + kb
    xu, xd, yu, yd = -rs * si, rs * si, -cs * sj, cs * sj
    # travel-time / adjoint tile (float): the step's two upstream loads, the
    # next step's loads and the store; slowness (float) and codes (uint16)
    offs = [xu, yu, 2 * sk, xd + sk, yd + sk, xu + sk, yu + sk, 0]
    for tau in range(bk + SKEW):
        kk = tau - s
        act = (kk >= 0) & (kk < bk)
        for off in offs:
            a = own + sk * kk + off
            if off == 0:
                a = a[act]  # the store is predicated on the window
            assert wavefronts(a) == 1, (tau, off)
        assert wavefronts(fown + sk * (kk + 1)) == 1
        # uint16 codes, two per word, on the same odd column stride: the one
        # access of the step that takes two passes
        assert wavefronts((fown + sk * (kk + 1)) // 2) <= 2


@pytest.mark.parametrize("bk", [16, 32, 64])
def test_sweep_addresses_stay_in_tiles(bk):
    rs, irs, cs_same, cs_diff, te, ite = layout(bk)
    for si, sj, sk in ORDERINGS:
        cs = cs_same if sj == sk else cs_diff
        pi, pj, s = lanes(si, sj)
        xu, xd, yu, yd = -rs * si, rs * si, -cs * sj, cs * sj
        offs = np.array([0, -sk, sk, 2 * sk, xu, xd, yu, yd, xu + sk, xd + sk, yu + sk, yd + sk])
        for pnk in sorted({1, 2, 3, bk // 2, bk - 1, bk}):
            kb = 0 if sk > 0 else pnk - 1
            own = (pi + 1) * rs + (pj + 1) * cs + 1 + kb
            fown = pi * irs + pj * cs + kb
            # every cell position a lane's pointer visits, the final advance included
            kk = np.arange(-s.max(), pnk + SKEW + 1)[None, :]
            valid = (kk >= -s[:, None]) & (kk <= pnk + SKEW - s[:, None])
            base = (own[:, None] + sk * kk)[valid]
            a = base[:, None] + offs[None, :]
            assert a.min() >= 0 and a.max() < te, (si, sj, sk, pnk)
            fa = (fown[:, None] + sk * kk)[valid]
            fa = np.concatenate([fa, fa + sk])
            # slowness / codes tiles may reach back into the warp's tile before them
            assert fa.min() >= -te and fa.max() < ite, (si, sj, sk, pnk)


def _halo_col(c):
    if c < BI * BJ:
        return (c >> 2) + 1, (c & 3) + 1
    h = c - BI * BJ
    if h < 2 * BJ:
        return (0 if h < BJ else BI + 1), (h & 3) + 1
    q = h - 2 * BJ
    return (q >> 1) + 1, (BJ + 1 if q & 1 else 0)


@pytest.mark.parametrize("same", [True, False])
def test_staging_fast_paths_match_generic_copies(same):
    """Full bricks (BK = 32) skip the per-copy checks: same (shared, global)
    copies as the generic loops, from per-lane bases."""
    bk = 32
    rs, irs, cs_same, cs_diff, te, ite = layout(bk)
    cs = cs_same if same else cs_diff
    n, l = 30, 64
    i0, j0, k0 = 8, 8, 32
    ch_n = bk // 4
    gen, fast = set(), set()
    for lane in range(32):  # halo tile
        for t in range((BI * BJ + 2 * BI + 2 * BJ) * ch_n // 32):
            e = lane + 32 * t
            ci, cj = _halo_col(e // ch_n)
            k = 4 * (e % ch_n)
            for w in range(4):
                gen.add((ci * rs + cj * cs + 1 + k + w,
                         ((i0 + ci - 1) * n + (j0 + cj - 1)) * l + k0 + k + w))
        gq, k = lane >> 3, 4 * (lane & 7)
        for ci in range(BI + 2):
            for w in range(4):
                fast.add((ci * rs + (gq + 1) * cs + 1 + k + w,
                          ((i0 - 1 + ci) * n + (j0 + gq)) * l + k0 + k + w))
        cib, cjb = (gq >> 1) + 1, (BJ + 1 if gq & 1 else 0)
        for r in range(BI // 2):
            for w in range(4):
                fast.add(((cib + 2 * r) * rs + cjb * cs + 1 + k + w,
                          ((i0 + cib + 2 * r - 1) * n + (j0 + cjb - 1)) * l + k0 + k + w))
    assert gen == fast
    gen, fast, sgen, sfast, cgen, cfast = set(), set(), set(), set(), set(), set()
    for lane in range(32):  # interior tile, write-back, codes
        for t in range(BI * BJ * ch_n // 32):
            e = lane + 32 * t
            c, k = e // ch_n, 4 * (e % ch_n)
            ci, cj = c >> 2, c & 3
            g0 = ((i0 + ci) * n + (j0 + cj)) * l + k0 + k
            for w in range(4):
                gen.add((ci * irs + cj * cs + k + w, g0 + w))
            sgen.add(((ci + 1) * rs + (cj + 1) * cs + 1 + k, g0))
        for t in range(BI * BJ * (bk // 8) // 32):
            e = lane + 32 * t
            c, k = e // (bk // 8), 8 * (e % (bk // 8))
            ci, cj = c >> 2, c & 3
            cgen.add((ci * irs + cj * cs + k, ((i0 + ci) * n + (j0 + cj)) * l + k0 + k))
        gq, k = lane >> 3, 4 * (lane & 7)
        for t in range(BI):
            g0 = ((i0 + t) * n + (j0 + gq)) * l + k0 + k
            for w in range(4):
                fast.add((t * irs + gq * cs + k + w, g0 + w))
            sfast.add((rs + (gq + 1) * cs + 1 + k + t * rs, g0))
        ci, cj, k = lane >> 4, (lane >> 2) & 3, 8 * (lane & 3)
        for t in range(BI * BJ * (bk // 8) // 32):
            cfast.add((ci * irs + cj * cs + k + 2 * t * irs,
                       ((i0 + ci + 2 * t) * n + (j0 + cj)) * l + k0 + k))
    assert gen == fast and sgen == sfast and cgen == cfast
