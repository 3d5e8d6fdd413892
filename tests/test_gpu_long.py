"""100-step runs of the 32^3 thermal electron-proton plasma (CIC, Boris, Esirkepov,
Yee, FP32) on the CUDA path and on the CPU oracle from identical inputs.

Contract:
* FP64 field and kinetic energies agree within 1e-4 relative at every 10th step
  (the J deposit sums in a different order on the two sides, so the runs are
  not bit-identical after the first step);
* charge conservation: max |eps0 div E - rho| stays <= 1e-5 * max|rho_e| on the
  GPU (protons start on the electrons, so the total density starts at zero and
  Esirkepov's continuity keeps div E - rho/eps0 constant).
"""
import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import random_particles

pytestmark = pytest.mark.gpu

DT = float(np.float32(0.99 / np.sqrt(3.0)))
N = 32
PPC = 4
STEPS = 100


def thermal_32(rng):
    g = pg.Grid(N, N, N, dt=DT)
    gd = g.as_dict()
    n = (0.1 / DT) ** 2  # omega_p dt = 0.1, q = m = eps0 = 1
    w = n / PPC
    pe = random_particles(gd, PPC, rng, u_th=0.01, mass=1.0, weight=w)
    pi = random_particles(gd, PPC, rng, u_th=0.01 / np.sqrt(1836.0), mass=1836.0, weight=w)
    pi["pos"] = pe["pos"].copy()
    return g, pe, pi


@pytest.fixture(scope="module")
def orc():
    import oracle

    import os

    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    return oracle


def test_energies_and_charge_conservation_over_100_steps(orc):
    rng = np.random.default_rng(2024)
    g, pe, pi = thermal_32(rng)
    gd = g.as_dict()
    se = pg.Species("e", -1.0, 1.0, shape="CIC")
    si = pg.Species("i", 1.0, 1836.0, shape="CIC")
    shp = (3, N, N, N)
    E = np.zeros(shp, np.float32)
    B = np.zeros(shp, np.float32)
    J = np.zeros(shp, np.float32)
    ref_e = {k: v.copy() for k, v in pe.items()}
    ref_i = {k: v.copy() for k, v in pi.items()}
    rho_e = np.zeros(shp[1:], np.float32)
    orc.charge_density(gd, se.as_dict(), pe, rho_e)
    rho_max = float(np.abs(rho_e).max())
    with pg.Simulation(g) as sim:
        sim.add_species(se)
        sim.add_species(si)
        sim.set_particles("e", pe)
        sim.set_particles("i", pi)
        res0, _ = sim.charge_residual()
        assert res0 <= 1e-5 * rho_max
        for step in range(1, STEPS + 1):
            sim.step()
            orc.step(gd, [se.as_dict(), si.as_dict()], [ref_e, ref_i], E, B, J, threads=1)
            if step % 10 == 0:
                eg = sim.energies()
                fe = orc.field_energy(gd, E, B)
                ke = orc.kinetic_energy(gd, se.as_dict(), ref_e)
                ki = orc.kinetic_energy(gd, si.as_dict(), ref_i)
                for got, want in ((eg["E"], fe[0]), (eg["B"], fe[1]), (eg["e"], ke), (eg["i"], ki)):
                    assert abs(got - want) <= 1e-4 * abs(want), (step, got, want)
                res, _ = sim.charge_residual()
                assert res <= 1e-5 * rho_max, (step, res, rho_max)
