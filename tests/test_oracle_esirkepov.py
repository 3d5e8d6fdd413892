"""Oracle Esirkepov deposit vs. the reference's numpy Esirkepov implementation.

Fixture: tests/golden/esirkepov_single_particle.npz, written by
tests/golden/make_esirkepov_golden.py from
share/picongpu/tests/CurrentDeposition/lib/python/test/CurrentDeposition/grid_class.py.
Tolerance |dJ| < 1e-5 as in MainTest.py:152.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "esirkepov_single_particle.npz"))
NC = int(Z["ncases"])
N = int(Z["grid_n"])


def case(i):
    return {k.split("_", 1)[1]: Z[k] for k in Z.files if k.startswith(f"c{i}_")}


@pytest.mark.parametrize("i", range(NC))
def test_single_particle_deposit(orc, i):
    c = case(i)
    g = dict(nx=N, ny=N, nz=N, sx=4, sy=4, sz=4, dx=1, dy=1, dz=1, dt=float(c["dt"]), c=1, eps0=1)
    J = np.zeros((3, N, N, N), np.float32)
    orc.esirkepov_one(g, int(c["order"]), c["cell1"], c["pos1"], c["vel"], float(c["charge"]), J)
    for d, k in enumerate(("jx", "jy", "jz")):
        assert np.abs(J[d] - c[k]).max() < 1e-5, (i, k)
    if bool(c["jx_ref_valid"]):
        assert np.abs(J[0] - c["jx_ref"]).max() < 1e-5


def test_fixture_covers_reference_ci_cases():
    dirs = set()
    for i in range(NC):
        c = case(i)
        if np.allclose(c["pos0"], [0.9, 0.8, 0.7]):
            dirs.add((int(c["order"]), tuple(np.sign(np.round(c["vel"], 3)).astype(int))))
    for order in (1, 2, 3):
        for d in ((1, 0, 0), (1, 1, 0), (1, 1, 1)):
            assert (order, d) in dirs


def _single_axis(c):
    v = np.round(np.asarray(c["vel"], np.float64), 6)
    return np.count_nonzero(v) == 1


@pytest.mark.parametrize("i", range(NC))
def test_emz_single_particle(orc, i):
    """EmZ (fields/currentDeposition/EmZ/EmZ.hpp) of the same particles.  Along one axis the
    relay-point split changes nothing: the current of a 1D motion is fixed by charge
    conservation, so EmZ must reproduce the reference's Esirkepov golden J there.  In every
    case EmZ conserves charge against the charge-assignment density."""
    c = case(i)
    g = dict(nx=N, ny=N, nz=N, sx=4, sy=4, sz=4, dx=1, dy=1, dz=1, dt=float(c["dt"]), c=1, eps0=1)
    J = np.zeros((3, N, N, N), np.float32)
    orc.emz_one(g, int(c["order"]), c["cell1"], c["pos1"], c["vel"], float(c["charge"]), J)
    if _single_axis(c):
        for d, k in enumerate(("jx", "jy", "jz")):
            assert np.abs(J[d] - c[k]).max() < 1e-5, (i, k)
    # continuity: (rho1 - rho0)/dt + div J = 0 with rho from the assignment function
    order = int(c["order"])
    rho = []
    for cell, pos in ((c["cell0"], c["pos0"]), (c["cell1"], c["pos1"])):
        p = dict(pos=np.asarray(pos, np.float32).reshape(3, 1), mom=np.zeros((3, 1), np.float32),
                 w=np.ones(1, np.float32), sc=np.zeros(1, np.int32), lcell=np.zeros(1, np.uint16))
        cell = np.asarray(cell, np.int64) % N
        sc4 = cell // 4
        p["sc"][0] = sc4[0] + (N // 4) * (sc4[1] + (N // 4) * sc4[2])
        lc = cell % 4
        p["lcell"][0] = lc[0] + 4 * (lc[1] + 4 * lc[2])
        r = np.zeros((N, N, N), np.float32)
        orc.charge_density(g, dict(charge=float(c["charge"]), mass=1.0, shape=order, pusher=1, current=2), p, r)
        rho.append(r.astype(np.float64))
    divJ = ((J[0] - np.roll(J[0], 1, axis=2)) + (J[1] - np.roll(J[1], 1, axis=1))
            + (J[2] - np.roll(J[2], 1, axis=0))).astype(np.float64)
    res = (rho[1] - rho[0]) / float(c["dt"]) + divJ
    assert np.abs(res).max() < 1e-5 * np.abs(rho[0]).max() / float(c["dt"])
