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
