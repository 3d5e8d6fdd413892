"""The GPU deposit against the reference's own single-particle Esirkepov numbers.

The numbers are those of share/picongpu/tests/CurrentDeposition: the reference's numpy Esirkepov
(lib/python/test/CurrentDeposition/grid_class.py, assignment_and_W_func.py) evaluated by
tests/golden/make_esirkepov_golden.py into the committed fixture
tests/golden/esirkepov_single_particle.npz.  Its cases are the reference CI's (start offset
(0.9, 0.8, 0.7), directions (1,0,0), (1,1,0), (1,1,1), beta = 0.999, dt = 0.5 dx/c) and seeded
random ones, for CIC, TSC and PQS.

Each case runs through the product path: one electron (w = 1) starts at the fixture's cell and
in-cell position with the momentum gamma beta of its velocity, moves one step of the full
single-box step with the Free pusher on a 12^3 periodic grid of 4^3 supercells, and J after the
step matches the fixture within |dJ| < 1e-5, the tolerance of the reference test
(MainTest.py:152).
"""
import os

import numpy as np
import pytest

import picongpu_gb300 as pg

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "esirkepov_single_particle.npz"))
NC = int(Z["ncases"])
N = int(Z["grid_n"])
SHAPE = {1: "CIC", 2: "TSC", 3: "PQS"}


def case(i):
    return {k.split("_", 1)[1]: Z[k] for k in Z.files if k.startswith(f"c{i}_")}


@pytest.mark.parametrize("i", range(NC))
def test_gpu_deposit_matches_reference_numbers(i):
    c = case(i)
    g = pg.Grid(N, N, N, dt=float(c["dt"]), supercell=(4, 4, 4))
    vel = np.asarray(c["vel"], np.float64)
    gamma = 1.0 / np.sqrt(1.0 - float(vel @ vel))
    cx, cy, cz = (int(v) for v in c["cell0"])
    ns = N // 4
    p = dict(pos=np.asarray(c["pos0"], np.float32).reshape(3, 1),
             mom=(gamma * vel).astype(np.float32).reshape(3, 1), w=np.ones(1, np.float32),
             sc=np.array([cx // 4 + ns * (cy // 4 + ns * (cz // 4))], np.int32),
             lcell=np.array([cx % 4 + 4 * (cy % 4 + 4 * (cz % 4))], np.uint16))
    with pg.Simulation(g) as sim:
        sim.add_species(pg.Species("e", float(c["charge"]), 1.0, pusher="Free", shape=SHAPE[int(c["order"])],
                                   current="Esirkepov"))
        sim.set_particles("e", p)
        sim.step()
        J = sim.get_field("J")
        q = sim.get_particles("e")
    # the particle ended where the reference's numbers put it
    sc, lc = int(q["sc"][0]), int(q["lcell"][0])
    cell = np.array([(sc % ns) * 4 + lc % 4, ((sc // ns) % ns) * 4 + (lc // 4) % 4, (sc // (ns * ns)) * 4 + lc // 16])
    assert np.array_equal(cell, np.asarray(c["cell1"]) % N), (cell, c["cell1"])
    assert np.abs(q["pos"][:, 0] - np.asarray(c["pos1"], np.float32)).max() < 1e-6
    for d, k in enumerate(("jx", "jy", "jz")):
        assert np.abs(J[d] - c[k]).max() < 1e-5, (i, k, float(np.abs(J[d] - c[k]).max()))
