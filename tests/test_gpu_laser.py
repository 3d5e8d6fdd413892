"""Laser-driven plasma on the single-box path: a Gaussian pulse (a0 = 2, wavelength 16)
entering through the TF/SF surface into an electron gas (PQS) over immobile ions.

Contract after 120 steps: the pulse has reached the plasma (electron kinetic energy
grows by orders of magnitude from the cold start), and charge is conserved to the
float32 rounding of the laser field: max|eps0 div E - rho| <= 1e-5 eps0 E0 / dx
(E0 = a0 omega, far above the plasma's charge density).  The pulse is transversely
uniform here: the incident field has no longitudinal component, so only a plane
pulse is divergence-free; a finite waist leaves a charge on the TF/SF surface.
"""
import math

import pytest

import picongpu_gb300 as pg

pytestmark = pytest.mark.gpu


def test_laser_drives_the_plasma_and_conserves_charge():
    lam = 16.0
    omega = 2 * math.pi / lam
    dens = 0.01 * omega * omega
    g = pg.Grid(32, 128, 32)
    with pg.Simulation(g) as sim:
        sim.add_species(pg.Species("e", -1.0, 1.0, shape="PQS"))
        sim.add_species(pg.Species("i", 1.0, 1836.0, pusher=None, shape="PQS", current=None))
        sim.init_plasma("e", 2, dens, 1e-4, seed=1, position_seed=2)
        sim.init_plasma("i", 2, dens, 0.0, seed=3, position_seed=2)
        fwhm = 10 * g.dt
        sigma = fwhm / (2 * math.sqrt(math.log(2)))
        sim.set_incident_field(a0=2.0, wavelength=lam, waist=1e6, duration_fwhm=fwhm, t_center=4 * sigma, surface=8)
        e0 = sim.energies()["e"]
        res0, _ = sim.charge_residual()
        assert res0 <= 1e-5 * dens
        sim.run(120)
        en = sim.energies()
        res, _ = sim.charge_residual()
    assert en["E"] + en["B"] > 0
    assert en["e"] > 100 * e0
    assert res <= 1e-5 * 2.0 * omega, (res, dens)
