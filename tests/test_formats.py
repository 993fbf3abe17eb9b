"""Plain-text inputs of the inversion workflow (scripts/sta_eve.jl, scripts/inversion.jl)."""
import numpy as np
import pytest

from adtomo_gb300 import formats as F


def test_range_roundtrip_and_reference_layout(tmp_path):
    p = tmp_path / "range.txt"
    # what sta_eve.jl's println calls produce
    p.write_text("128\n128\n64\n0.5\n12\n9\n3\n")
    r = F.read_range(str(p))
    assert r == {"m": 128, "n": 128, "l": 64, "h": 0.5, "dx": 12, "dy": 9, "dz": 3}
    F.write_range(str(p), **r)
    assert F.read_range(str(p)) == r
    p.write_text("1\n2\n")
    with pytest.raises(ValueError):
        F.read_range(str(p))


def test_points_csv_roundtrip(tmp_path):
    p = tmp_path / "allsta.csv"
    p.write_text("x,y,z,lon,lat\n13.25,4.5,1.0,-117.5,35.7\n1.0,2.0,3.5,-117.2,35.9\n")
    xyz, extra = F.read_points_csv(str(p))
    assert np.array_equal(xyz, [[13.25, 4.5, 1.0], [1.0, 2.0, 3.5]])
    assert extra["lon"] == ["-117.5", "-117.2"]
    assert np.array_equal(F.node_coords(xyz), xyz - 1.0)
    q = tmp_path / "out.csv"
    F.write_points_csv(str(q), xyz, lon=extra["lon"], lat=extra["lat"])
    xyz2, extra2 = F.read_points_csv(str(q))
    assert np.array_equal(xyz2, xyz) and extra2 == extra


def test_read_matrix_formats(tmp_path):
    a = np.array([[0.5, -1.0, 2.0], [1.5, 2.5, -1.0]])
    np.save(tmp_path / "u.npy", a)
    np.savez(tmp_path / "u.npz", matrix=a)
    np.savetxt(tmp_path / "u.csv", a, delimiter=",")
    for f in ("u.npy", "u.npz", "u.csv"):
        assert np.array_equal(F.read_matrix(str(tmp_path / f)), a)
    with pytest.raises(ValueError):
        F.read_matrix(str(tmp_path / "uobs_p.h5"))
