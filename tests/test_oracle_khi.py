"""The electron-scale Kelvin-Helmholtz instability in the oracle (CPU): the reference's KHI
growth-rate test (share/picongpu/tests/KHI_growthRate, checked by
lib/python/test/setups/ESKHI/config.py) on a coarser grid that the CPU runs in half a minute.

Quasi-neutral electron-proton flows along +x and -x (gamma = 1.021) in two slabs of y, periodic
box, TSC, Boris, Esirkepov, Yee, particles started on a 3 x 3 x 1 lattice per cell as the
reference's quiet start does (``picongpu_gb300.quiet_start``).  The magnetic field energy grows exponentially, and its largest
growth rate 0.5 d ln(E_B)/dt, in units of the relativistic plasma frequency, approaches the
theory value 1 / (sqrt(8) gamma) = 0.346 as the grid is refined: the oracle measured 0.25 with
cells of 0.2 c/omega_p (this test), 0.29 with 0.1 c/omega_p, while the reference's setup uses
0.048 c/omega_p and accepts 20 %.  The test therefore asks for 60 % to 110 % of the theory value
at this resolution, and for more than three decades of exponential growth.
"""
import os

import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import grid

GAMMA = 1.021
NX, NY, NZ = 32, 64, 4
WP = 0.2  # plasma frequency in c / cell: cells of 0.2 c / omega_p
STEPS = 420
LATTICE = 3
MASS_P = 1836.15267343


@pytest.fixture(scope="module")
def orc():
    import oracle

    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    return oracle


def test_eskhi_growth_rate(orc):
    g = grid(n=(NX, NY, NZ))
    u = np.sqrt(GAMMA ** 2 - 1.0)
    start = dict(per_cell=(LATTICE, LATTICE, 1), density=WP ** 2, drift_lo=(u, 0.0, 0.0), drift_hi=(-u, 0.0, 0.0),
                 split_axis=1, split_cell=NY // 2)  # density omega_p^2 with q = m = eps0 = 1
    pg_grid = pg.Grid(NX, NY, NZ, dt=g["dt"])
    pe = pg.quiet_start(pg_grid, mass=1.0, u_th=1e-3, seed=1, **start)
    pi = pg.quiet_start(pg_grid, mass=MASS_P, **start)
    se = dict(charge=-1.0, mass=1.0, shape=2, pusher=0, current=1)  # TSC, Boris, Esirkepov
    si = dict(charge=1.0, mass=MASS_P, shape=2, pusher=0, current=1)
    shp = (3, NZ, NY, NX)
    E, B, J = (np.zeros(shp, np.float32) for _ in range(3))
    t, eb = [], []
    for step in range(STEPS + 1):
        if step:
            orc.step(g, [se, si], [pe, pi], E, B, J, os.cpu_count() or 1)
        if step % 5 == 0:
            t.append(step * g["dt"])
            eb.append(orc.field_energy(g, E, B)[1])
    t = np.asarray(t) * WP / np.sqrt(GAMMA)
    eb = np.asarray(eb)
    # central differences over +-15 steps, after the start-up (t >= 5 / omega_p)
    k = 3
    rate = 0.5 * np.log(eb[2 * k + 1:] / eb[1:-2 * k]) / (t[2 * k + 1:] - t[1:-2 * k])
    rate = rate[t[1:-2 * k] >= 5.0]
    theory = 1.0 / (np.sqrt(8.0) * GAMMA)
    assert 0.6 * theory <= rate.max() <= 1.1 * theory, (rate.max(), theory)
    assert eb.max() > 1e3 * eb[t >= 5.0][0]
