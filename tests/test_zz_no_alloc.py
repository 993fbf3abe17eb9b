"""The no-allocation 3D forward entry point (adt_eikonal_three_d_device_noalloc).

Some callers cannot allocate device memory (a framework that owns the whole
device heap, a host with a memory budget fixed at start-up).  This entry
point runs the plain FP64 3D forward on caller-provided device buffers and
takes its scratch from a fixed array inside the library.  Its results must
equal the existing entry point adt_eikonal_three_d_device, which uses the
same kernels, and the oracle's restatement of the reference's forward
(Eikonal3D.cpp:71-94, same tolerance and 20-iteration cap): FP64 travel times
bit-identical (the tolerance of the plain FP64 parity tests), on two calls in
a row, so the shared scratch carries nothing over from one call to the next.

This file is collected last so that, when it fails, a run stopping at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import adtomo_gb300 as A
from adtomo_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    if A.lib().adt_device_count() < 1:
        pytest.skip("no GPU")
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch sees no GPU")
    return torch


def _run(fn, torch, u0, f, h, tol):
    m, n, l = u0.shape
    d0 = torch.from_numpy(u0).cuda()
    df = torch.from_numpy(f).cuda()
    du = torch.empty_like(d0)
    st = A._lib.SolveStatus()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(C.c_void_p(d0.data_ptr()), C.c_void_p(df.data_ptr()), float(h), m, n, l, float(tol), 0,
            C.c_void_p(du.data_ptr()), C.byref(st), stream)
    A._lib.check(rc)
    torch.cuda.synchronize()
    return du.cpu().numpy(), (st.iters, st.converged, st.final_err)


CASES = [
    ("c2_64x64x32", (64, 64, 32), 1.0, 1e-6),
    ("ragged_9x13x37", (9, 13, 37), 0.5, 1e-9),
    ("tiny_2x2x2", (2, 2, 2), 1.0, 1e-6),
]


@pytest.mark.parametrize("name,dims,h,tol", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_existing_entry_point(torch_cuda, name, dims, h, tol):
    torch = torch_cuda
    L = A.lib()
    m, n, l = dims
    rng = np.random.default_rng(m * 7 + n * 3 + l)
    if name.startswith("c2"):
        f = synth.layered_checkerboard(m, n, l, block=8)
    else:
        f = rng.uniform(0.15, 0.35, size=dims)
    src = (rng.uniform(0, m - 1), rng.uniform(0, n - 1), rng.uniform(0, l - 1))
    u0 = O.src_u0(f, h, src)
    ref, ref_st = _run(L.adt_eikonal_three_d_device, torch, u0, f, h, tol)
    orc, orc_it, orc_err = O.eik3d_forward(u0, f, h, tol)
    for _ in range(2):  # two calls in a row share the same scratch
        got, st = _run(L.adt_eikonal_three_d_device_noalloc, torch, u0, f, h, tol)
        assert np.array_equal(got, ref)
        assert st == ref_st
        assert np.array_equal(got, orc)
        assert st[0] == orc_it and st[2] == orc_err


def test_noalloc_rejects_grids_above_the_scratch_limit(torch_cuda):
    L = A.lib()
    limit = 262144
    m, n, l = 64, 64, limit // (64 * 64) + 1
    st = A._lib.SolveStatus()
    rc = L.adt_eikonal_three_d_device_noalloc(None, None, 1.0, m, n, l, 1e-6, 0, None, C.byref(st),
                                              None)
    assert rc == -1
    assert b"scratch limit" in L.adt_last_error()
