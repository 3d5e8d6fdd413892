"""The electron-scale Kelvin-Helmholtz instability in the oracle (CPU): the reference's KHI
growth-rate test (share/picongpu/tests/KHI_growthRate, checked by
lib/python/test/setups/ESKHI/config.py) on a coarser grid that the CPU runs in half a minute.

Quasi-neutral electron-proton flows along +x and -x (gamma = 1.021) in two slabs of y, periodic
box, TSC, Boris, Esirkepov, Yee, particles started on a 3 x 3 x 1 lattice per cell as the
reference's quiet start does.  The magnetic field energy grows exponentially, and its largest
growth rate 0.5 d ln(E_B)/dt, in units of the relativistic plasma frequency, approaches the
theory value 1 / (sqrt(8) gamma) = 0.346 as the grid is refined: the oracle measured 0.256 with
cells of 0.2 c/omega_p (this test), 0.29 with 0.1 c/omega_p, while the reference's setup uses
0.048 c/omega_p and accepts 20 %.  The test therefore asks for 60 % to 110 % of the theory value
at this resolution, and for more than three decades of exponential growth.
"""
import os

import numpy as np
import pytest

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


def _species(g, cells, pos, drift, mass, w, u_th, rng):
    n = cells.shape[1]
    u = np.zeros((3, n))
    u[0] = drift
    if u_th > 0.0:
        u += rng.normal(0.0, u_th, u.shape)
    sc = (cells[0] // g["sx"]) + (g["nx"] // g["sx"]) * ((cells[1] // g["sy"]) + (g["ny"] // g["sy"]) * (cells[2] // g["sz"]))
    lc = (cells[0] % g["sx"]) + g["sx"] * ((cells[1] % g["sy"]) + g["sy"] * (cells[2] % g["sz"]))
    return dict(pos=np.ascontiguousarray(pos.copy()), mom=np.ascontiguousarray((u * mass * w).astype(np.float32)),
                w=np.full(n, w, np.float32), sc=sc.astype(np.int32), lcell=lc.astype(np.uint16))


def test_eskhi_growth_rate(orc):
    g = grid(n=(NX, NY, NZ))
    ppc = LATTICE * LATTICE
    w = WP ** 2 / ppc  # density omega_p^2 with q = m = eps0 = 1
    cx, cy, cz = np.meshgrid(np.arange(NX), np.arange(NY), np.arange(NZ), indexing="ij")
    cells = np.repeat(np.stack([cx.ravel(), cy.ravel(), cz.ravel()]), ppc, axis=1)
    ox, oy = np.meshgrid((np.arange(LATTICE) + 0.5) / LATTICE, (np.arange(LATTICE) + 0.5) / LATTICE, indexing="ij")
    offsets = np.stack([ox.ravel(), oy.ravel(), np.full(ppc, 0.5)])
    pos = np.tile(offsets, (1, NX * NY * NZ)).astype(np.float32)
    u = np.sqrt(GAMMA ** 2 - 1.0)
    drift = np.where(cells[1] < NY // 2, u, -u)
    rng = np.random.default_rng(1)
    pe = _species(g, cells, pos, drift, 1.0, w, 1e-3, rng)
    pi = _species(g, cells, pos, drift, MASS_P, w, 0.0, rng)
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
