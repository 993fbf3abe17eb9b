"""2D-table event location (tests/Eikonal/eikoloc.py): the GPU loss/gradient
against the NumPy restatement, and event recovery on synthetic picks."""
import numpy as np
import pytest

import adtomo_gb300 as A
from adtomo_gb300 import location as Lc
from oracle import location_oracle as LO

pytestmark = pytest.mark.gpu

ZZ, VP = [0.0, 5.5, 16.0, 32.0, 50.0], [5.5, 5.5, 6.7, 7.8, 7.8]  # eikoloc.py:292-294
BOUNDS = ((-60.0, 60.0), (-60.0, 60.0), (0.0, 30.0))


def _setup(rng, n_events=12, n_sta=15, h=1.0):
    tp, ts, r0, z0 = Lc.traveltime_tables(ZZ, VP, 1.73, (0.0, 120.0), (0.0, 40.0), h)
    sta = np.c_[rng.uniform(-50, 50, (n_sta, 2)), rng.uniform(0.0, 1.5, n_sta)]
    true = np.c_[rng.uniform(-1, 1, n_events), rng.uniform(-30, 30, (n_events, 2)),
                 rng.uniform(3, 20, n_events)]
    offs, S, T, P, W = [0], [], [], [], []
    for e in range(n_events):
        for q in range(n_sta):
            for ph, tab in ((0, tp), (1, ts)):
                if rng.random() < 0.2:
                    continue
                r = np.hypot(*(true[e, 1:3] - sta[q, :2]))
                z = abs(true[e, 3]) - sta[q, 2]
                S.append(sta[q]); P.append(ph); W.append(rng.uniform(0.5, 1.0))
                T.append(true[e, 0] + LO.interp(tab, np.array([r]), np.array([z]), r0, z0, h)[0])
        offs.append(len(T))
    picks = {"offs": np.array(offs), "sta": np.array(S), "t": np.array(T),
             "phase": np.array(P, np.int32), "w": np.array(W)}
    return tp, ts, r0, z0, h, picks, true


def _oracle_losses(params, picks, tp, ts, r0, z0, h, gamma):
    o = picks["offs"]
    return np.array([LO.event_loss(params[e], picks["sta"][o[e]:o[e + 1]], picks["t"][o[e]:o[e + 1]],
                                   picks["phase"][o[e]:o[e + 1]], picks["w"][o[e]:o[e + 1]],
                                   tp, ts, r0, z0, h, BOUNDS, gamma) for e in range(len(o) - 1)])


@pytest.mark.parametrize("gamma", [0.0, 0.5])
def test_loss_and_gradient_match_numpy(gamma):
    rng = np.random.default_rng(1)
    tp, ts, r0, z0, h, picks, true = _setup(rng)
    loc = Lc.Locator(tp, ts, r0, z0, h, BOUNDS, gamma=gamma)
    params = true + np.c_[rng.normal(0, 0.3, len(true)), rng.normal(0, 3, (len(true), 3))]
    params[0, 3] = 45.0  # beyond the depth bound: clamped, no z gradient
    loss, grad = loc.loss_grad(params, picks)
    ref = _oracle_losses(params, picks, tp, ts, r0, z0, h, gamma)
    assert np.allclose(loss, ref, rtol=1e-12, atol=1e-14)
    assert grad[0, 3] == 0.0
    eps = 1e-6
    for a in range(4):
        dp = np.zeros_like(params)
        dp[:, a] = eps
        fd = (_oracle_losses(params + dp, picks, tp, ts, r0, z0, h, gamma) -
              _oracle_losses(params - dp, picks, tp, ts, r0, z0, h, gamma)) / (2 * eps)
        assert np.allclose(grad[:, a], fd, rtol=1e-5, atol=1e-7), a


def test_loss_and_gradient_match_the_reference_script(golden_dir):
    """adt_locate_loss_grad against the loss and autograd gradient of the
    reference's own location code (tests/Eikonal/eikoloc.py: _interp,
    traveltime and the closure of invert, executed by
    tests/golden/make_location_golden.py): loss to 1e-12 relative, gradient to
    1e-9 relative, with and without the double-difference term."""
    import os
    d = np.load(os.path.join(golden_dir, "loc_eikoloc.npz"))
    offs = d["offs"]
    for gamma in np.unique(d["gamma"]):
        ev = np.flatnonzero(d["gamma"] == gamma)
        sub_offs, idx = [0], []
        for e in ev:
            idx.extend(range(offs[e], offs[e + 1]))
            sub_offs.append(len(idx))
        picks = {"offs": np.array(sub_offs), "sta": d["sta"][idx], "t": d["t"][idx],
                 "phase": d["phase"][idx].astype(np.int32), "w": d["w"][idx]}
        loc = Lc.Locator(d["tp"], d["ts"], float(d["r0"]), float(d["z0"]), float(d["h"]),
                         d["bounds"], gamma=float(gamma))
        loss, grad = loc.loss_grad(d["params"][ev], picks)
        assert np.allclose(loss, d["loss"][ev], rtol=1e-12, atol=0), gamma
        assert np.allclose(grad, d["grad"][ev], rtol=1e-9, atol=1e-12), gamma


def test_tables_match_the_2d_solver():
    tp, ts, r0, z0 = Lc.traveltime_tables(ZZ, VP, 1.73, (0.0, 30.0), (0.0, 20.0), 1.0)
    assert tp.shape == ts.shape == (33, 23) and (r0, z0) == (-3.0, -3.0)
    assert tp[3, 3] == 0.0 and ts[3, 3] == 0.0
    assert np.all(ts >= tp)  # S is slower everywhere
    # straight-line bound: a layered medium is never slower than its slowest layer
    r = np.arange(33) - 3.0
    assert tp[33 - 1, 3] <= np.hypot(r[-1], 0) / 5.5 + 1e-12


def test_locate_recovers_synthetic_events():
    rng = np.random.default_rng(2)
    tp, ts, r0, z0, h, picks, true = _setup(rng, n_events=20)
    loc = Lc.Locator(tp, ts, r0, z0, h, BOUNDS)
    est, loss, iters = loc.locate(picks, loc0=(0.0, 0.0, 5.0))
    assert np.all(loss < 1e-6)
    assert np.max(np.abs(est[:, 1:] - true[:, 1:])) < 0.05
    assert np.max(np.abs(est[:, 0] - true[:, 0])) < 0.01


def test_locate_rejects_bad_input():
    tp = np.zeros((4, 4))
    loc = Lc.Locator(tp, tp, 0.0, 0.0, 1.0, BOUNDS)
    with pytest.raises(A.AdtError):
        loc.loss_grad(np.zeros((1, 4)), {"offs": [0, 1], "sta": [[0, 0, 0]], "t": [1.0],
                                         "phase": np.array([2], np.int32), "w": [1.0]})
