"""The C-ABI library: it loads, exports every symbol the header declares, and
rejects invalid input before any device work (CPU only, no GPU needed)."""
import os
import re

import numpy as np
import pytest

import adtomo_gb300 as A
from adtomo_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "adtomo_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(adt_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = A.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(_lib.SIGNATURES), "ctypes signatures must cover the header exactly"


def test_struct_mirrors_match_the_library():
    import ctypes as C
    sizes = (C.c_int64 * 3)()
    assert A.lib().adt_abi_struct_sizes(sizes, 3) == 3
    assert tuple(sizes) == (C.sizeof(_lib.SolveStatus), C.sizeof(_lib.BatchOpts),
                            C.sizeof(_lib.BatchStats))


def test_version_and_device_count_do_not_fail():
    L = A.lib()
    assert b"sm_103a" in L.adt_version()
    assert L.adt_device_count() >= 0


@pytest.mark.parametrize("dims", [(1, 4, 4), (4, 1, 4), (4, 4, 1), (0, 3, 3)])
def test_eikonal3d_rejects_small_grids(dims):
    m, n, l = dims
    with pytest.raises(A.AdtError) as e:
        A.eikonal3d(np.zeros(max(m * n * l, 1)), np.ones(max(m * n * l, 1)), 1.0, m, n, l, 1e-6)
    assert e.value.code == -1


def test_eikonal3d_rejects_bad_slowness_and_h():
    u0 = np.full(27, 1000.0)
    f = np.ones(27)
    f[5] = -1.0
    with pytest.raises(A.AdtError) as e:
        A.eikonal3d(u0, f, 1.0, 3, 3, 3, 1e-6)
    assert e.value.code == -1
    f[5] = np.nan
    with pytest.raises(A.AdtError):
        A.eikonal3d(u0, f, 1.0, 3, 3, 3, 1e-6)
    with pytest.raises(A.AdtError):
        A.eikonal3d(u0, np.ones(27), 0.0, 3, 3, 3, 1e-6)
    with pytest.raises(A.AdtError):
        A.eikonal3d(u0, np.ones(27), 1.0, 3, 3, 3, -1.0)


def test_eikonal2d_rejects_source_outside():
    f = np.ones((5, 7))
    for sx, sy in [(0, 1), (8, 1), (1, 0), (1, 6)]:
        with pytest.raises(A.AdtError) as e:
            A.eikonal(f, sx, sy, 1.0)
        assert e.value.code == -1


def test_size_mismatch_is_rejected_host_side():
    with pytest.raises(A.AdtError):
        A.eikonal3d(np.zeros(10), np.ones(10), 1.0, 3, 3, 3, 1e-6)


@pytest.mark.parametrize("kw", [{"wake_tol": -1.0}, {"adj_wake_tol": float("nan")}, {"bk": 8},
                                {"precision": 7}, {"max_iter": 0}, {"tol": -1.0},
                                {"ref_compat": True}, {"max_iter": 100001},
                                {"adj_max_iter": 100001}, {"adj_solver": 3}])
def test_batch_options_rejected_host_side(kw):
    with pytest.raises(A.AdtError) as e:
        A.Batch3D([(8, 8, 8, 1.0)], [np.zeros((1, 3))], [0], [[1.0, 1.0, 1.0]], **kw)
    assert e.value.name == "ADT_EINVAL"


def test_batch_null_handle_is_rejected():
    import ctypes as C
    L = A.lib()
    one = np.zeros(4)
    assert L.adt_batch_upload(None, None, None, None) == -1
    assert L.adt_batch_run_resident(None) == -1
    assert L.adt_batch_autotune(None, 1) == -1
    assert L.adt_batch_set_source_velocity(None, None) == -1
    assert L.adt_batch_download(None, None, None, None, None) == -1
    assert L.adt_batch_run(None, one.ctypes.data_as(C.c_void_p), None, None, None, None, None,
                           None) == -1
    assert L.adt_batch_stats_get(None, None) == -1
    assert L.adt_batch_stream(None) is None
    assert L.adt_batch_device_buffer(None, 0) is None
    assert L.adt_batch_destroy(None) == 0
    assert b"null handle" in L.adt_last_error() or b"null" in L.adt_last_error()


@pytest.mark.skipif(A.lib().adt_device_count() > 0, reason="a GPU is present")
def test_valid_call_without_gpu_reports_nodev():
    with pytest.raises(A.AdtError) as e:
        A.eikonal3d(np.full(27, 1000.0), np.ones(27), 1.0, 3, 3, 3, 1e-6)
    assert e.value.name == "ADT_ENODEV"


def test_eikonal3d_rejects_grids_deeper_than_the_brick_packing():
    """Brick coordinates are packed in 11/11/10 bits: more than 1023 bricks of
    16 cells (the plain path's brick depth) along k would wrap, so the plain 3D
    entry points reject such a grid before any device work."""
    import ctypes as C
    L = A.lib()
    st = _lib.SolveStatus()
    for l in (16 * 1023 + 1, 40000):
        assert L.adt_eikonal_three_d_device(None, None, 1.0, 2, 2, l, 1e-6, 0, None,
                                            C.byref(st), None) == -1
        assert b"too deep" in L.adt_last_error()
    # the deepest accepted grid passes the size checks (and fails on the null arrays)
    assert L.adt_eikonal_three_d_device(None, None, 1.0, 2, 2, 16 * 1023, 1e-6, 0, None,
                                        C.byref(st), None) == -1
    assert b"null array" in L.adt_last_error()


@pytest.mark.parametrize("dims,msg", [((2, 2, 40000), b"too deep"),
                                      ((16376, 8188, 1 << 40), b"scratch limit"),
                                      ((8, 8, (1 << 62) // 64 + 1), b"scratch limit"),
                                      ((64, 64, 65), b"scratch limit")])
def test_noalloc_rejects_sizes_host_side(dims, msg):
    """The no-allocation entry point bounds every extent before forming the
    cell count (a huge l must not wrap the product below the limit) and
    rejects grids deeper than the brick packing, before any device work."""
    import ctypes as C
    L = A.lib()
    st = _lib.SolveStatus()
    m, n, l = dims
    assert L.adt_eikonal_three_d_device_noalloc(None, None, 1.0, m, n, l, 1e-6, 0, None,
                                                C.byref(st), None) == -1
    assert msg in L.adt_last_error()


def test_noalloc_rejects_infinite_spacing_like_the_plain_entry_point():
    import ctypes as C
    L = A.lib()
    st = _lib.SolveStatus()
    for fn in (L.adt_eikonal_three_d_device_noalloc, L.adt_eikonal_three_d_device):
        assert fn(None, None, float("inf"), 4, 4, 4, 1e-6, 0, None, C.byref(st), None) == -1
        assert b"finite" in L.adt_last_error()
