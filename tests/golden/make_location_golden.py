"""Generate tests/golden/loc_eikoloc.npz from the reference's own location code.

The reference locates events with tests/Eikonal/eikoloc.py: `_interp`
(:119-140, bilinear read of a travel-time table), `traveltime` (:142-152,
horizontal distance and |z| - z_station) and the loss closure inside
`invert` (:155-206: clamp to the bounds, mean weighted Huber loss per phase,
optional double-difference term).  The script imports pandas and
matplotlib at the top and runs torch's L-BFGS, so it is not imported here:
this generator parses it with `ast`, executes those two functions and the
statements of `invert` that build the closure's inputs, replaces only the
optimiser object by a stub (the closure calls optimizer.zero_grad()), calls
the closure once and records the loss and torch's autograd gradient with
respect to t0 and the event position.

The script creates t0 and loc0 as FP32 tensors; the generator runs the same
code with torch.float32 mapped to FP64, so that the fixture pins the
arithmetic of the objective rather than FP32 rounding (the library computes
in FP64).  Inputs are seeded synthetic tables and picks (no dataset is
shipped with the reference).  Positions are kept off the bounds, where
torch splits the gradient of min/max ties.

Run in a container that has the reference sources and torch:
    python tests/golden/make_location_golden.py [path/to/eikoloc.py]
The default path is $ADTOMO_REFERENCE/tests/Eikonal/eikoloc.py, with
ADTOMO_REFERENCE defaulting to the read-only reference mount.
"""
from __future__ import annotations

import ast
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "loc_eikoloc.npz")


def load_reference_functions(path):
    """(_interp, traveltime, invert_once) executed from the script's source."""
    import torch
    import torch.nn.functional as F

    tree = ast.parse(open(path).read(), filename=path)
    defs = {n.name: n for n in tree.body if isinstance(n, ast.FunctionDef)}
    inv = defs["invert"]
    # statements of invert up to the optimiser, then the closure definition
    pre, closure = [], None
    for st in inv.body:
        if isinstance(st, ast.Assign) and any(isinstance(t, ast.Name) and t.id == "optimizer"
                                              for t in st.targets):
            continue
        if isinstance(st, ast.FunctionDef) and st.name == "closure":
            closure = st
            break
        pre.append(st)
    assert closure is not None, "closure of invert not found"
    ret = ast.parse("return closure(), t0, loc0").body
    once = ast.FunctionDef(name="invert_once", args=inv.args, body=pre + [closure] + ret,
                           decorator_list=[], returns=None, type_comment=None, type_params=[])
    mod = ast.Module(body=[defs["_interp"], defs["traveltime"], once], type_ignores=[])
    ast.fix_missing_locations(mod)

    class _Optimizer:  # the closure only calls zero_grad(); the step is not run
        def zero_grad(self):
            pass

    torch64 = types.SimpleNamespace(**{k: getattr(torch, k) for k in dir(torch)
                                       if not k.startswith("__")})
    torch64.float32 = torch.float64
    ns = {"torch": torch64, "F": F, "np": np, "optimizer": _Optimizer()}
    exec(compile(mod, path, "exec"), ns)
    return ns["_interp"], ns["traveltime"], ns["invert_once"]


def tables(r0, z0, h, m, n):
    """Smooth P and S tables on r = r0 + i h, z = z0 + j h (a layered-like
    analytic field: straight-ray time in a velocity rising with depth)."""
    r = r0 + h * np.arange(m)
    z = z0 + h * np.arange(n)
    R, Z = np.meshgrid(r, z, indexing="ij")
    v = 5.5 + 0.05 * np.clip(Z, 0, None)
    tp = np.sqrt(R ** 2 + (Z - z0) ** 2) / v + 0.01 * np.sin(0.3 * R) * np.cos(0.2 * Z)
    return tp, tp * 1.73, R, Z


def main():
    import torch

    ref = os.environ.get("ADTOMO_REFERENCE", "/root/reference")
    path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ref, "tests", "Eikonal",
                                                              "eikoloc.py")
    _interp, traveltime, invert_once = load_reference_functions(path)
    rng = np.random.default_rng(2024)
    h, r0, z0, m, n = 1.0, -3.0, -3.0, 130, 46
    tp, ts, R, Z = tables(r0, z0, h, m, n)
    up, us = torch.tensor(tp), torch.tensor(ts)
    rgrid, zgrid = torch.tensor(R), torch.tensor(Z)
    bounds = ((-60.0, 60.0), (-60.0, 60.0), (0.0, 30.0))
    cases = []
    for e in range(10):
        nsta = int(rng.integers(4, 14))
        sta = np.c_[rng.uniform(-50, 50, (nsta, 2)), rng.uniform(0.0, 1.5, nsta)]
        # P and S picks of random stations (an event may lack one phase)
        phase = rng.integers(0, 2, nsta) if e % 3 else np.zeros(nsta, np.int64)
        t = rng.uniform(2.0, 20.0, nsta)
        w = rng.uniform(0.3, 1.0, nsta)
        params = np.r_[rng.uniform(-1, 1), rng.uniform(-40, 40, 2), rng.uniform(2, 25)]
        if e == 4:
            params[3] = -params[3]  # a negative depth: |z| in traveltime
        for add_eqt, gamma in ((False, 0.1), (True, 0.1), (True, 1.0)):
            loss, t0, loc0 = invert_once(
                torch.tensor(t), torch.tensor(sta), np.array(["P", "S"])[phase], torch.tensor(w),
                up, us, rgrid, zgrid, h, t0=[params[0]], loc0=list(params[1:]), bounds=bounds,
                add_eqt=add_eqt, gamma=gamma)
            grad = np.r_[t0.grad.numpy(), loc0.grad.numpy()]
            cases.append(dict(sta=sta, t=t, w=w, phase=phase.astype(np.int32), params=params,
                              gamma=gamma if add_eqt else 0.0, loss=float(loss.item()),
                              grad=grad))
    offs = np.cumsum([0] + [len(c["t"]) for c in cases])
    np.savez_compressed(
        OUT, tp=tp, ts=ts, r0=r0, z0=z0, h=h, bounds=np.array(bounds), offs=offs,
        sta=np.concatenate([c["sta"] for c in cases]), t=np.concatenate([c["t"] for c in cases]),
        w=np.concatenate([c["w"] for c in cases]),
        phase=np.concatenate([c["phase"] for c in cases]),
        params=np.array([c["params"] for c in cases]), gamma=np.array([c["gamma"] for c in cases]),
        loss=np.array([c["loss"] for c in cases]), grad=np.array([c["grad"] for c in cases]))
    print(f"wrote {OUT}: {len(cases)} cases, {offs[-1]} picks")


if __name__ == "__main__":
    main()
