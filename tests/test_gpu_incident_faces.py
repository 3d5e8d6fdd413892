"""Incident field through every face of the total-field/scattered-field box
(fields/incidentField/Solver.hpp: XMin ... ZMax profiles, propagation along the face normal).

* Every axis, both directions and both polarisations: a transversely uniform pulse
  (wavelength 16 cells, intensity FWHM 20 dt) in a vacuum box 256 cells long along the axis
  and 16 across obeys the 1D Yee scheme exactly, so a float64 restatement of the 1D split
  update with the TF/SF corrections of either direction, fed with the plane pulse of
  profiles/GaussianPulse.hpp (waist -> infinity), is the reference: the tangential
  E and B on two lines along the axis match it within 1e-4 of the amplitude, and the
  scattered-field region beyond the surface holds less than 1e-5 of it.
* A focused beam (waist 6, wavelength 8, focus 5 cells beyond the surface) through the +x
  and +z faces equals the +y run with the axes swapped (E as a polar, B as an axial
  vector), through the -y face the +y run mirrored, within 1e-5 of the largest field.
* Two faces at once give the sum of the two single-face runs within 1e-5 (linearity).
* Invalid faces, surfaces and surfaces inside an absorber are refused.
"""
import math

import numpy as np
import pytest

import picongpu_gb300 as pg
from incident_1d import line, yee_1d

pytestmark = pytest.mark.gpu

LONG, ACROSS = 256, 16
LAM = 16.0
STEPS = 200
OFF = 32  # surface distance from the entering end


def dims(axis, long, across):
    d = [across] * 3
    d[axis] = long
    return d


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("direction", [1, -1])
@pytest.mark.parametrize("pol", [0, 1])
def test_pulse_through_every_face(axis, direction, pol):
    g = pg.Grid(*dims(axis, LONG, ACROSS))
    fwhm = 20 * g.dt
    tc = 40.0
    P = OFF if direction > 0 else LONG - 1 - OFF
    with pg.Simulation(g) as sim:
        sim.set_incident_field(a0=1.0, wavelength=LAM, waist=1e6, duration_fwhm=fwhm, t_center=tc, surface=P,
                               polarisation=pol, axis=axis, direction=direction)
        sim.run(STEPS)
        E = sim.get_field("E")
        B = sim.get_field("B")
    E0 = 2 * math.pi / LAM
    e1, b1 = yee_1d(LONG, P, direction, g, LAM, fwhm, tc, STEPS)
    t1, t2 = [d for d in range(3) if d != axis]
    p = t1 if pol == 0 else t2
    o = t2 if pol == 0 else t1
    eta = 1.0 if p == (axis + 2) % 3 else -1.0
    assert np.abs(e1).max() > 0.5 * E0  # the pulse is inside
    for u1, u2 in ((0, 0), (ACROSS // 3, ACROSS // 2)):
        assert np.abs(line(E, p, axis, u1, u2) - e1).max() <= 1e-4 * E0
        assert np.abs(line(B, o, axis, u1, u2) - eta * b1).max() <= 1e-4 * E0
        assert np.abs(line(E, o, axis, u1, u2)).max() <= 1e-6 * E0
        assert np.abs(line(E, axis, axis, u1, u2)).max() <= 1e-6 * E0
    # nothing leaks into the scattered region behind the surface
    sl = [slice(None)] * 3
    sl[2 - axis] = slice(0, P - 2) if direction > 0 else slice(P + 3, LONG)
    for F in (E, B):
        assert np.abs(F[(slice(None),) + tuple(sl)]).max() <= 1e-5 * E0


# ---------------------------------------------------------------- focused beam, other faces
N1, NL = 32, 96  # across, along the propagation
J0 = 16
FOCUSED = dict(a0=1.0, wavelength=8.0, waist=6.0, duration_fwhm=12.0, t_center=20.0, focus=5.0, phase=0.3)
FSTEPS = 90


def focused_run(axis, direction, surface, pol=0, center=(13.0, 17.5), extra=None):
    g = pg.Grid(*dims(axis, NL, N1))
    with pg.Simulation(g) as sim:
        sim.set_incident_field(surface=surface, polarisation=pol, center=center, axis=axis, direction=direction,
                               **FOCUSED)
        if extra is not None:
            sim.set_incident_field(**extra)
        sim.run(FSTEPS)
        return sim.get_field("E"), sim.get_field("B")


def swap(F, a, b, axial):
    """Fields of the run with spatial axes a and b exchanged: components a <-> b, array axes
    (2 - a) <-> (2 - b); an axial vector changes sign under the reflection."""
    perm = [0, 1, 2]
    perm[a], perm[b] = b, a
    out = np.stack([F[perm[c]] for c in range(3)])
    out = np.swapaxes(out, 1 + (2 - a), 1 + (2 - b))
    return -out if axial else out


def test_focused_beam_through_x_and_z_faces_matches_y():
    Ey, By = focused_run(1, 1, J0)
    scale = max(np.abs(Ey).max(), np.abs(By).max())
    assert scale > 0.1
    for axis in (0, 2):
        Ea, Ba = focused_run(axis, 1, J0)
        # the +y run with y exchanged for `axis` (transverse order and polarisation follow)
        assert np.abs(Ea - swap(Ey, 1, axis, False)).max() <= 1e-5 * scale, axis
        assert np.abs(Ba - swap(By, 1, axis, True)).max() <= 1e-5 * scale, axis


def test_focused_beam_through_the_high_y_face_is_the_mirror_image():
    Ey, By = focused_run(1, 1, J0)
    Y0 = NL - 1
    Em, Bm = focused_run(1, -1, Y0 - J0)
    scale = max(np.abs(Ey).max(), np.abs(By).max())
    j = np.arange(NL)
    whole = (Y0 - j) % NL  # integer y positions map to Y0 - j
    half = (Y0 - 1 - j) % NL  # half-integer ones to Y0 - 1 - j
    # E_x, E_z and B_y sit at integer y; E_y, B_x, B_z at half-integer y.  Under y -> -y the
    # polar E_y and the axial B_x, B_z change sign.
    want_E = np.stack([Ey[0][:, whole, :], -Ey[1][:, half, :], Ey[2][:, whole, :]])
    want_B = np.stack([-By[0][:, half, :], By[1][:, whole, :], -By[2][:, half, :]])
    assert np.abs(Em - want_E).max() <= 1e-5 * scale
    assert np.abs(Bm - want_B).max() <= 1e-5 * scale


def test_two_faces_add():
    Ea, Ba = focused_run(1, 1, J0)
    Eb, Bb = focused_run(1, -1, NL - 1 - J0, pol=1, center=(15.0, 14.0))
    both = dict(FOCUSED, surface=NL - 1 - J0, polarisation=1, center=(15.0, 14.0), axis=1, direction=-1)
    Ec, Bc = focused_run(1, 1, J0, extra=both)
    scale = max(np.abs(Ea).max(), np.abs(Eb).max())
    assert np.abs(Ec - (Ea + Eb)).max() <= 1e-5 * scale
    assert np.abs(Bc - (Ba + Bb)).max() <= 1e-5 * scale


def test_faces_are_validated():
    g = pg.Grid(32, 64, 32)
    base = dict(a0=1.0, wavelength=16.0, waist=4.0, duration_fwhm=5.0, t_center=10.0)
    with pg.Simulation(g) as sim:
        for bad in (dict(axis=3, surface=8), dict(axis=1, direction=2, surface=8), dict(axis=1, direction=-1, surface=64),
                    dict(axis=0, direction=1, surface=0), dict(axis=2, direction=1, surface=32)):
            with pytest.raises(pg.PicError):
                sim.set_incident_field(**base, **bad)
        sim.set_incident_field(**base, axis=1, direction=-1, surface=62)
        sim.set_incident_field(**base, axis=0, direction=1, surface=1)
        sim.clear_incident_field(axis=1, direction=-1)
        sim.clear_incident_field()
        # an open y axis with 8-cell absorbers: the surface must keep out of them
        sim.set_boundaries(open_axes=(False, True, False), thickness=((0, 0), (8, 8), (0, 0)))
        with pytest.raises(pg.PicError):
            sim.set_incident_field(**base, axis=1, direction=1, surface=8)
        with pytest.raises(pg.PicError):
            sim.set_incident_field(**base, axis=1, direction=-1, surface=56)
        sim.set_incident_field(**base, axis=1, direction=1, surface=9)
        sim.set_incident_field(**base, axis=1, direction=-1, surface=55)
        sim.run(2)
        # thicker absorbers set afterwards: the next field stage refuses the surfaces
        sim.set_boundaries(open_axes=(False, True, False), thickness=((0, 0), (12, 12), (0, 0)))
        with pytest.raises(pg.PicError):
            sim.step()
