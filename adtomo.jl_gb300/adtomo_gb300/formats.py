"""Readers and writers for the plain-text inputs of the inversion workflow.

scripts/sta_eve.jl writes, per region:
  range.txt    seven lines: m, n, l, h, dx, dy, dz (sta_eve.jl:130-132), read
               back by scripts/inversion.jl:25-27;
  allsta.csv / alleve.csv   DataFrames written by CSV.write, with columns
               x, y, z (1-based fractional grid coordinates, already shifted
               by dx, dy, dz), lon, lat, and for events a picks column.
The pick matrices (uobs_p.h5 / qua_p.h5, "matrix", stations x events, -1
for a missing pick) and the starting model (vel0_p.h5, "data") are HDF5
files; this package reads the same arrays from .npy / .npz / CSV instead,
because no HDF5 library is available to it.

Grid coordinates in the files are 1-based, as Julia indexes; the batched
plan (adtomo_gb300.Batch3D) takes 0-based coordinates: node_coords() does
the conversion.
"""
from __future__ import annotations

import csv
import os

import numpy as np

RANGE_KEYS = ("m", "n", "l", "h", "dx", "dy", "dz")


def read_range(path: str) -> dict:
    """range.txt -> {"m", "n", "l" (int), "h" (float), "dx", "dy", "dz" (int)}."""
    with open(path) as fh:
        lines = [ln.strip() for ln in fh if ln.strip()]
    if len(lines) < 7:
        raise ValueError(f"{path}: expected 7 lines (m, n, l, h, dx, dy, dz), got {len(lines)}")
    out = {}
    for key, text in zip(RANGE_KEYS, lines[:7]):
        out[key] = float(text) if key == "h" else int(text)
    return out


def write_range(path: str, m: int, n: int, l: int, h: float, dx: int, dy: int, dz: int) -> None:
    """Write range.txt the way scripts/sta_eve.jl does (one value per line)."""
    with open(path, "w") as fh:
        for v in (int(m), int(n), int(l), float(h), int(dx), int(dy), int(dz)):
            fh.write(f"{v}\n")


def read_points_csv(path: str):
    """allsta.csv / alleve.csv -> (xyz (N, 3) float64, 1-based as stored; the
    other columns as a dict of string lists)."""
    with open(path, newline="") as fh:
        rows = list(csv.DictReader(fh))
    if rows and not all(k in rows[0] for k in ("x", "y", "z")):
        raise ValueError(f"{path}: needs columns x, y, z")
    xyz = np.array([[float(r["x"]), float(r["y"]), float(r["z"])] for r in rows],
                   dtype=np.float64).reshape(-1, 3)
    extra = {}
    if rows:
        for k in rows[0]:
            if k not in ("x", "y", "z"):
                extra[k] = [r[k] for r in rows]
    return xyz, extra


def write_points_csv(path: str, xyz, **columns) -> None:
    """Write x, y, z (and further columns) with a header line, as CSV.write does."""
    xyz = np.asarray(xyz, np.float64).reshape(-1, 3)
    names = ["x", "y", "z"] + list(columns)
    with open(path, "w", newline="") as fh:
        w = csv.writer(fh)
        w.writerow(names)
        for q in range(len(xyz)):
            w.writerow([repr(float(v)) for v in xyz[q]] + [columns[k][q] for k in columns])


def node_coords(xyz_1based):
    """1-based grid coordinates (the files, Julia) -> 0-based (Batch3D)."""
    return np.asarray(xyz_1based, np.float64) - 1.0


def read_matrix(path: str, name: str = "matrix"):
    """A pick matrix or a model array from .npy, .npz (array `name`) or CSV."""
    ext = os.path.splitext(path)[1].lower()
    if ext == ".npy":
        return np.load(path)
    if ext == ".npz":
        with np.load(path) as z:
            return z[name]
    if ext in (".csv", ".txt"):
        return np.loadtxt(path, delimiter=",", ndmin=2)
    raise ValueError(f"{path}: unsupported format {ext} (HDF5 needs a library this package "
                     "does not have; convert to .npy/.npz/CSV)")
