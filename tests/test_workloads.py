"""CPU checks of the synthetic workloads bench.py measures: the 192x96x96 bracket
(void cylinder r = 16 through y at the x-z centre, four passive 6x6 full-height
bolt-pad columns inset 6 voxels from the x-y corners, three seeded point loads of
magnitude U(0.5, 1.5) on the top face, clamped x = 0 face), the 256x128x128
cantilever (total -z load 1 on the 33x33 nodes of the central 32x32 patch of
x = max), the 48x24x12 cantilever (unit -z line load along x = 48, z = 6) and the
256 seeded uneven cantilevers of the batched workload."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _node(shape, i, j, k):
    nx, ny, nz = shape
    return (i * (ny + 1) + j) * (nz + 1) + k


def _clamped_x0(W):
    nx, ny, nz = W["shape"]
    fixed = np.sort(W["fixed"])
    expect = np.sort((3 * np.array([_node(W["shape"], 0, j, k) for j in range(ny + 1) for k in range(nz + 1)])[:, None]
                      + np.arange(3)).ravel())
    return np.array_equal(fixed, expect)


def test_bracket192():
    W = bench.build_workload("bracket192")
    nx, ny, nz = W["shape"]
    assert (nx, ny, nz) == (192, 96, 96) and W["rmin"] == 2.0 and W["vf"] == 0.3
    assert W["F"].size == 3 * 193 * 97 * 97 == 5447811
    assert _clamped_x0(W)
    rho = W["rho0"]
    # void cylinder through y: element centres within 16 of the x-z centre
    i = np.arange(nx) + 0.5
    k = np.arange(nz) + 0.5
    cyl = (i[:, None] - nx / 2) ** 2 + (k[None, :] - nz / 2) ** 2 <= 256.0
    assert np.all(rho[np.broadcast_to(cyl[:, None, :], rho.shape)] == 0.0)
    # four 6x6 full-height pads at density 1, inset 6 from the x-y corners
    pads = np.zeros((nx, ny), bool)
    for x0 in (6, nx - 12):
        for y0 in (6, ny - 12):
            pads[x0:x0 + 6, y0:y0 + 6] = True
    assert np.all(rho[pads] == 1.0)
    assert int(pads.sum()) == 4 * 36
    rest = ~np.broadcast_to(cyl[:, None, :], rho.shape) & ~np.broadcast_to(pads[:, :, None], rho.shape)
    assert np.all(rho[rest] == 0.3)
    # three point loads on the top face (k = nz), magnitudes in [0.5, 1.5]
    F = W["F"].reshape(-1, 3)
    loaded = np.nonzero(np.linalg.norm(F, axis=1))[0]
    assert loaded.size == 3
    assert np.all(loaded % (nz + 1) == nz)
    mags = np.linalg.norm(F[loaded], axis=1)
    assert np.all((mags >= 0.5) & (mags <= 1.5))
    # seeded: the same loads every time
    assert np.array_equal(bench.build_workload("bracket192")["F"], W["F"])


def test_cantilevers():
    W = bench.build_workload("cantilever256")
    nx, ny, nz = W["shape"]
    assert (nx, ny, nz) == (256, 128, 128) and W["rmin"] == 2.5 and W["vf"] == 0.25
    assert _clamped_x0(W)
    F = W["F"].reshape(-1, 3)
    loaded = np.nonzero(F[:, 2])[0]
    assert loaded.size == 33 * 33 and np.all(F[:, :2] == 0.0)
    assert abs(F[:, 2].sum() + 1.0) < 1e-12
    assert np.all(loaded // ((ny + 1) * (nz + 1)) == nx)
    W = bench.build_workload("cantilever48")
    nx, ny, nz = W["shape"]
    assert (nx, ny, nz) == (48, 24, 12) and W["rmin"] == 1.5
    F = W["F"].reshape(-1, 3)
    loaded = np.nonzero(F[:, 2])[0]
    assert loaded.size == ny + 1 and abs(F[:, 2].sum() + 1.0) < 1e-12
    assert np.all(loaded % (nz + 1) == nz // 2) and np.all(loaded // ((ny + 1) * (nz + 1)) == nx)


def test_batch256():
    probs = bench.build_batch256()
    assert len(probs) == 256
    for pr in probs:
        nx, ny, nz = pr["shape"]
        assert 32 <= nx <= 96 and 16 <= ny <= 48 and 8 <= nz <= 48
        assert 0.2 <= pr["vf"] <= 0.5 and 1.2 <= pr["rmin"] <= 2.5
        F = pr["F"].reshape(-1, 3)
        loaded = np.nonzero(np.linalg.norm(F, axis=1))[0]
        assert loaded.size == 1 and loaded[0] // ((ny + 1) * (nz + 1)) == nx
        assert abs(np.linalg.norm(F[loaded[0]]) - 1.0) < 1e-12
    sizes = {pr["shape"] for pr in probs}
    assert len(sizes) > 200  # uneven sizes
    again = bench.build_batch256()
    assert all(a["shape"] == b["shape"] and np.array_equal(a["F"], b["F"]) for a, b in zip(probs, again))
