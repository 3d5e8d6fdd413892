"""Incident field through the total-field/scattered-field surface (fields/incidentField).

Vacuum box 16 x 256 x 16 (periodic), surface at y = 32, a transversely uniform
pulse (wavelength 16 cells, intensity FWHM 20 dt) travelling +y, polarised along x
or z.  A transversely uniform wave on the 3D Yee grid obeys the 1D Yee scheme
exactly, so a float64 numpy restatement of the 1D split update with the same
TF/SF corrections is the reference (the pulse of profiles/GaussianPulse.hpp with its waist
going to infinity).  Contract after 200 steps:
* the tangential E and B on every (x, z) line match the 1D reference within 1e-4
  of the amplitude;
* the scattered-field region holds less than 1e-5 of the amplitude (no backward leak);
* the pulse follows the analytic form (carrier with the grid's numerical wavenumber)
  within 12% of its amplitude (the rest is the grid's dispersion of a 3-cycle pulse).
"""
import math

import numpy as np
import pytest

import picongpu_gb300 as pg

pytestmark = pytest.mark.gpu

NX, NY, NZ = 16, 256, 16
J0 = 32
LAM = 16.0
STEPS = 200


def phase_velocity(g, omega):
    """The Yee grid's phase velocity along y: sin(k dy / 2) / dy = sin(omega dt / 2) / (c dt)."""
    dt = float(np.float32(g.dt))
    k = 2.0 / g.dy * math.asin(g.dy / (g.c * dt) * math.sin(omega * dt / 2))
    return omega / k


def incident(y, t, g, fwhm, tc):
    """The plane pulse (waist -> infinity) of profiles/GaussianPulse.hpp: the local time runs from
    the Huygens surface J0 - 1/4 at the grid's phase velocity, zero before it starts, cosine
    carrier, envelope exp(-(time / 2 tau)^2) with tau the rms duration of the intensity."""
    omega = 2 * math.pi * g.c / LAM
    tau2 = fwhm / math.sqrt(2 * math.log(2))
    tloc = t - (y - (J0 - 0.25)) * g.dy / phase_velocity(g, omega)
    time = tloc - tc
    return np.where(tloc < 0, 0.0, omega * np.exp(-(time / tau2) ** 2) * np.cos(omega * time))


def yee_1d(g, fwhm, tc, steps):
    """Tangential E (at integer y) and B (at y + 1/2) of the 1D split Yee update with the
    TF/SF corrections, for polarisation x (E_x, B_z); polarisation z is the mirror image
    (E_z, -B_x)."""
    E = np.zeros(NY)
    Bt = np.zeros(NY)
    dt, dy, c = float(np.float32(g.dt)), g.dy, g.c
    for n in range(steps):
        t = n * dt
        Bt += 0.5 * dt * (np.roll(E, -1) - E) / dy
        Bt[J0 - 1] -= 0.5 * dt / dy * incident(J0, t, g, fwhm, tc)
        E += c * c * dt * (Bt - np.roll(Bt, 1)) / dy
        E[J0] += c * dt / dy * incident(J0 - 0.5, t + 0.5 * dt, g, fwhm, tc)
        Bt += 0.5 * dt * (np.roll(E, -1) - E) / dy
        Bt[J0 - 1] -= 0.5 * dt / dy * incident(J0, t + dt, g, fwhm, tc)
    return E, Bt


def analytic(t, y, g, fwhm, tc):
    """The pulse with its carrier at the Yee grid's wavenumber k for omega,
    sin(k dy / 2) / dy = sin(omega dt / 2) / (c dt), and its envelope moving at c."""
    omega = 2 * math.pi * g.c / LAM
    k = omega / phase_velocity(g, omega)
    tau2 = fwhm / math.sqrt(2 * math.log(2))
    y0 = J0 - 0.25
    env = t - (y - y0) * g.dy / g.c - tc
    out = omega * np.exp(-(env / tau2) ** 2) * np.cos(omega * (t - tc) - k * (y - y0) * g.dy)
    out[y < J0] = 0.0
    return out


@pytest.mark.parametrize("pol", [0, 1])
def test_pulse_enters_through_the_surface(pol):
    g = pg.Grid(NX, NY, NZ)
    fwhm = 20 * g.dt
    tc = 40.0
    with pg.Simulation(g) as sim:
        sim.set_incident_field(a0=1.0, wavelength=LAM, waist=1e6, duration_fwhm=fwhm, t_center=tc, surface=J0,
                               polarisation=pol)
        sim.run(STEPS)
        E = sim.get_field("E")
        B = sim.get_field("B")
        en = sim.energies()
    E0 = 2 * math.pi / LAM
    e1, b1 = yee_1d(g, fwhm, tc, STEPS)
    ce, cb, sb = (0, 2, 1.0) if pol == 0 else (2, 0, -1.0)
    for k in (0, NZ // 2):
        for i in (0, NX // 3):
            assert np.abs(E[ce, k, :, i] - e1).max() <= 1e-4 * E0
            assert np.abs(B[cb, k, :, i] - sb * b1).max() <= 1e-4 * E0
    assert np.abs(E[:, :, : J0 - 2, :]).max() <= 1e-5 * E0
    assert np.abs(B[:, :, : J0 - 2, :]).max() <= 1e-5 * E0
    y = np.arange(NY, dtype=np.float64)
    assert np.abs(e1 - analytic(STEPS * float(np.float32(g.dt)), y, g, fwhm, tc)).max() <= 0.12 * E0
    want = 0.5 * NX * NZ * (np.sum(e1 ** 2) + np.sum(b1 ** 2))
    assert abs(en["E"] + en["B"] - want) <= 1e-4 * want, (en, want)


def test_incident_field_is_validated():
    g = pg.Grid(16, 64, 16)
    with pg.Simulation(g) as sim:
        with pytest.raises(pg.PicError):
            sim.set_incident_field(a0=1.0, wavelength=16.0, waist=4.0, duration_fwhm=5.0, t_center=10.0, surface=0)
        with pytest.raises(pg.PicError):
            sim.set_incident_field(a0=1.0, wavelength=-1.0, waist=4.0, duration_fwhm=5.0, t_center=10.0, surface=8)
        sim.clear_incident_field()
