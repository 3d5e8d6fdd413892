"""The host-side quiet start (particles/startPosition/QuietImpl.hpp) in the exchange format: no GPU."""
import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import global_cells


def test_lattice_positions_counts_and_layout():
    g = pg.Grid(16, 16, 8, dx=0.5, dy=1.0, dz=2.0)
    p = pg.quiet_start(g, per_cell=(3, 2, 1), density=0.25, with_ids=True)
    n_cells = 16 * 16 * 8
    assert p["w"].size == 6 * n_cells
    assert np.allclose(p["w"], 0.25 * 0.5 * 1.0 * 2.0 / 6)
    # every cell holds the 3 x 2 x 1 lattice i s + s/2, s = 1/n, in float32
    cells = global_cells(g.as_dict(), p)
    key = cells[0] + 16 * (cells[1] + 16 * cells[2])
    assert np.array_equal(np.bincount(key, minlength=n_cells), np.full(n_cells, 6))
    s3, s2 = np.float32(1) / np.float32(3), np.float32(1) / np.float32(2)
    want_x = {np.float32(i) * s3 + s3 * np.float32(0.5) for i in range(3)}
    want_y = {np.float32(i) * s2 + s2 * np.float32(0.5) for i in range(2)}
    assert set(np.unique(p["pos"][0])) == want_x and set(np.unique(p["pos"][1])) == want_y
    assert np.all(p["pos"][2] == np.float32(0.5))
    first = key == 0
    pts = {(float(a), float(b)) for a, b in p["pos"][:2, first].T}
    assert len(pts) == 6  # six distinct lattice points in one cell
    # supercell-major, consecutive particles in consecutive cells of a supercell
    assert np.all(np.diff(p["sc"]) >= 0)
    assert np.array_equal(p["lcell"][:256], np.arange(256))
    assert np.unique(p["id"]).size == p["id"].size


def test_drifts_split_and_temperature():
    g = pg.Grid(8, 16, 4)
    p = pg.quiet_start(g, per_cell=(2, 2, 1), density=1.0, mass=2.0, drift_lo=(0.2, 0, 0), drift_hi=(-0.2, 0, 0),
                       split_axis=1, split_cell=8)
    y = global_cells(g.as_dict(), p)[1]
    u = p["mom"] / (2.0 * p["w"])  # gamma beta
    assert np.allclose(u[0][y < 8], 0.2) and np.allclose(u[0][y >= 8], -0.2)
    assert np.all(u[1:] == 0.0)
    q = pg.quiet_start(g, per_cell=(2, 2, 1), u_th=0.05, seed=3)
    uq = q["mom"] / q["w"]
    assert abs(float(uq.std()) - 0.05) < 0.005


def test_invalid_arguments():
    g = pg.Grid(8, 8, 4)
    with pytest.raises(ValueError):
        pg.quiet_start(g, per_cell=(0, 1, 1))
    with pytest.raises(ValueError):
        pg.quiet_start(g, split_axis=3)
