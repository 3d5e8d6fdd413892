"""Conservation laws of the oracle's full step (CPU, no GPU): the invariants that the
reference's ChargeConservation and Energy plugins watch (plugins/ChargeConservation.tpp,
plugins/EnergyFields.x.cpp, plugins/EnergyParticles.x.cpp), over many steps.

* Gauss's law: protons start on the electrons, so rho = 0 and E = 0 satisfy
  eps0 div E = rho at the start, and a charge-conserving deposit (Esirkepov, EmZ) keeps
  max |eps0 div E - rho| within 1e-5 of max |rho_e| at every step, for every shape.
* Energy: field plus kinetic energy of a thermal plasma drifts by less than 3 % over the run
  (the Debye length is 0.3 cells, and CIC heats by about 1 % in 30 steps).
"""
import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import grid, random_particles

STEPS = 30
PPC = 3


@pytest.fixture(scope="module")
def orc():
    import oracle

    oracle.build()
    oracle.set_threads(1)
    return oracle


def _plasma(g, rng, u_th):
    n = (0.1 / g["dt"]) ** 2  # omega_p dt = 0.1 with q = m = eps0 = 1
    w = n / PPC
    pe = random_particles(g, PPC, rng, u_th=u_th, mass=1.0, weight=w)
    pi = random_particles(g, PPC, rng, u_th=u_th / np.sqrt(1836.0), mass=1836.0, weight=w)
    pi["pos"] = pe["pos"].copy()
    return pe, pi


@pytest.mark.parametrize("current", ["Esirkepov", "EmZ"])
@pytest.mark.parametrize("shape", ["CIC", "TSC", "PQS", "PCS"])
def test_gauss_law_and_energy_over_steps(orc, shape, current):
    g = grid(n=(16, 16, 8))
    rng = np.random.default_rng(11 + len(current))
    pe, pi = _plasma(g, rng, u_th=0.05)
    se = pg.Species("e", -1.0, 1.0, shape=shape, current=current).as_dict()
    si = pg.Species("i", 1.0, 1836.0, shape=shape, current=current).as_dict()
    shp = (g["nz"], g["ny"], g["nx"])
    E, B, J = (np.zeros((3,) + shp, np.float32) for _ in range(3))
    rho_e = np.zeros(shp, np.float32)
    orc.charge_density(g, se, pe, rho_e)
    rho_max = float(np.abs(rho_e).max())

    def total_energy():
        fe = orc.field_energy(g, E, B)
        return float(fe[0] + fe[1]) + orc.kinetic_energy(g, se, pe) + orc.kinetic_energy(g, si, pi)

    w0 = total_energy()
    crossed = np.zeros(pe["w"].size, bool)
    cell0 = pe["lcell"].copy(), pe["sc"].copy()
    for step in range(STEPS):
        orc.step(g, [se, si], [pe, pi], E, B, J)
        rho = np.zeros(shp, np.float32)
        rho_i = np.zeros(shp, np.float32)
        orc.charge_density(g, se, pe, rho)
        orc.charge_density(g, si, pi, rho_i)
        rho = rho.astype(np.float64) + rho_i
        res, _ = orc.charge_residual(g, E, rho.astype(np.float32))
        assert res <= 1e-5 * rho_max, (step, res, rho_max)
    crossed |= (pe["lcell"] != cell0[0]) | (pe["sc"] != cell0[1])
    assert crossed.mean() > 0.05  # the electrons did change cells
    assert abs(total_energy() - w0) <= 0.03 * w0
