"""Host-side logic of the batched solver and the serving loop, on CPU: the
tiling depends only on a system's own size (what makes a system's bits
independent of the batch), tile tables are laid out as the C ABI expects,
the request stream has the configured mix and sizes, and the memory
estimate grows with the system."""
import ctypes

import numpy as np
import pytest

from fealpy_gb300 import _lib
from fealpy_gb300.batch import BatchSolver
from fealpy_gb300.serving import resident_estimate
from fealpy_gb300.workloads import serving_requests, batched_tri_meshes, tri_box_dofs, tet_box_dofs


class _Tiler:
    max_tiles_per_system = 256
    _tile_bounds = BatchSolver._tile_bounds
    _tiles = BatchSolver._tiles


def test_tile_bounds_cover_each_system_once():
    t = _Tiler()
    for lim, per in ((1, 16), (15, 16), (16, 16), (1000, 16), (100000, 16), (4096, 4096), (5000, 4096)):
        b = t._tile_bounds(lim, per)
        assert b[0, 0] == 0 and b[-1, 1] == lim
        assert np.all(b[1:, 0] == b[:-1, 1]) and np.all(b[:, 1] > b[:, 0])
        assert len(b) <= max(t.max_tiles_per_system, -(-lim // per))
        assert len(b) <= t.max_tiles_per_system or per * t.max_tiles_per_system >= lim


def test_tiles_table_layout_and_pointers():
    t = _Tiler()
    parts = [t._tile_bounds(100, 16), None, t._tile_bounds(33, 16)]
    tiles, ptr, n = t._tiles(parts)
    assert n == 7 + 3 and list(ptr) == [0, 7, 7, 10]
    assert tiles.dtype == np.int32 and tiles.shape == (10, 4) and tiles.flags["C_CONTIGUOUS"]
    assert list(tiles[:7, 0]) == [0] * 7 and list(tiles[7:, 0]) == [2] * 3
    # one row of the array is one fgb_batch_tile
    assert ctypes.sizeof(_lib.BatchTile) == tiles.itemsize * 4
    # a system's tiles are the same wherever it sits in the table
    alone, _, _ = t._tiles([t._tile_bounds(33, 16)])
    assert np.array_equal(alone[:, 1:], tiles[7:, 1:])


def test_struct_sizes_match_the_header():
    # fgb_batch_system: 2 int64 + 14 pointers + 2 int32; fgb_batch_state: 11 double,
    # 2 int64, 6 int32, 1 double, 2 int64
    assert ctypes.sizeof(_lib.BatchSystem) == 2 * 8 + 14 * 8 + 2 * 4
    assert ctypes.sizeof(_lib.BatchState) == 11 * 8 + 2 * 8 + 6 * 4 + 8 + 2 * 8


def test_serving_stream_mix_and_sizes():
    reqs = serving_requests(2000, rate=100.0, seed=3)
    t = np.array([r["t"] for r in reqs])
    assert np.all(np.diff(t) >= 0) and abs(len(reqs) / t[-1] - 100.0) < 10.0
    kinds = np.array([r["kind"] for r in reqs])
    assert abs(np.mean(kinds == "tri") - 0.7) < 0.04
    for r in reqs:
        d = tri_box_dofs(r["n"], r["p"]) if r["kind"] == "tri" else tet_box_dofs(r["n"])
        assert d == r["dofs"] and 300 <= d <= 2.5e6
        assert r["p"] in ((1, 2) if r["kind"] == "tri" else (1,))


def test_batched_meshes_configuration():
    ms = batched_tri_meshes(64)
    assert all(16 <= m["nx"] <= 512 and m["p"] in (1, 2, 3) for m in ms)
    for m in ms[:4]:
        assert m["cell"].shape[0] == 2 * m["nx"] ** 2 and m["kappa"].shape == (m["cell"].shape[0],)
        assert 0.1 <= m["kappa"].min() and m["kappa"].max() <= 10.0
        assert len(np.unique(m["kappa"])) <= 16


def test_resident_estimate_monotone():
    a = resident_estimate(1000, 7000, False)
    assert resident_estimate(2000, 14000, False) > a and resident_estimate(1000, 7000, True) > a
    with pytest.raises(TypeError):
        resident_estimate(1000)
