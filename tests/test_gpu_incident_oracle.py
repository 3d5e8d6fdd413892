"""The incident field against the oracle's restatement of the reference
(profiles/GaussianPulse.hpp with Functors.hpp BaseFunctorE / ApproximateIncidentB, and the
TF/SF update of incidentField/Solver.kernel), element by element.

Vacuum boxes 32 x 96 x 32 (long along the propagation axis), a focused Gaussian beam
(wavelength 8, waist 5, focus 6 cells beyond the Huygens surface, off-centre, phase 0.7,
intensity FWHM 12, t_center 40), 140 steps.  The oracle runs the same split Yee update
(B half, E, B half) with its TF/SF corrections of each face after every field update, in
the reference's vector formulation (origin on the Huygens surface, internal coordinates by
dot products, updated[comp2] += base * inc[comp1], updated[comp1] -= base * inc[comp2]).
Contract: E and B agree within 2e-6 of the amplitude E0 = a0 omega (measured on GB300: 2e-7
to 3e-7), for faces on all three axes, both directions and both polarisations, for two faces
at once, at oblique incidence (s and p polarised), with circular polarisation, with a sum of
Laguerre-Gauss modes and TIME_DELAY, and for the PlaneWave, Wavepacket and Polynom profiles; the rest is float rounding of the carrier's argument (up to about 40 rad) and
the GPU's fused multiply-adds.  A structural difference (a quarter cell in the origin, a sign,
a staggering) shows at 1e-2 E0 or more.
"""
import math

import numpy as np
import pytest

import oracle as orc
import picongpu_gb300 as pg

pytestmark = pytest.mark.gpu

ACROSS, LONG = 32, 96
STEPS = 140
BEAM = dict(a0=1.0, wavelength=8.0, waist=5.0, duration_fwhm=12.0, t_center=40.0, focus=6.0, phase=0.7)
TOL = 2e-6
E0 = 2 * math.pi / BEAM["wavelength"]  # a0 omega with c = e/m = 1


def dims(axis):
    d = [ACROSS] * 3
    d[axis] = LONG
    return d


def oracle_face(gd, axis, direction, surface, pol, center, prop=None, polvec=None, circular=False, delay=0.0,
                modes=None, phases=None, profile="GaussianPulse", ramp_init=0.0, plateau=0.0, pulse_duration=0.0,
                waist_axis=None, pulse_init=0.0):
    """The face in the reference's parameters: the origin is the beam axis on the Huygens plane (a
    quarter cell before the first or last total E plane) at the transverse centre, the focus lies
    `focus` face-axis cells from it along the propagation."""
    cell = (gd["dx"], gd["dy"], gd["dz"])
    t1, t2 = [d for d in range(3) if d != axis]
    d = [float(np.float32(v)) for v in prop] if prop is not None else [float(direction) if a == axis else 0.0
                                                                        for a in range(3)]
    origin = [0.0, 0.0, 0.0]
    origin[t1] = center[0] * cell[t1]
    origin[t2] = center[1] * cell[t2]
    origin[axis] = (surface - 0.25 * direction) * cell[axis]
    focus = [origin[a] + BEAM["focus"] * cell[axis] * d[a] for a in range(3)]
    # PULSE_DURATION: given, or the rms duration of the intensity from its FWHM
    tau = pulse_duration if pulse_duration > 0 else BEAM["duration_fwhm"] / (2 * math.sqrt(2 * math.log(2)))
    pv = [float(np.float32(v)) for v in polvec] if polvec is not None else None
    return orc.incident_face(gd, axis, direction, surface, pol, BEAM["a0"], BEAM["wavelength"], BEAM["waist"], tau,
                             -BEAM["t_center"], BEAM["phase"], focus, propagation=d if prop is not None else None,
                             polarisation_vector=pv, circular=circular, time_delay=delay, laguerre_modes=modes,
                             laguerre_phases=phases,
                             profile={"GaussianPulse": 0, "PlaneWave": 1, "Wavepacket": 2, "Polynom": 3}[profile],
                             ramp_init=ramp_init, plateau=plateau, pulse_init=pulse_init, waist_axis=waist_axis)


def run_both(axis, faces):
    g = pg.Grid(*dims(axis))
    gd = g.as_dict()
    with pg.Simulation(g) as sim:
        for f in faces:
            sim.set_incident_field(surface=f["surface"], polarisation=f["pol"], center=f["center"], axis=f["axis"],
                                   direction=f["dir"], propagation=f.get("prop"), polarisation_vector=f.get("polvec"),
                                   circular=f.get("circular", False), time_delay=f.get("delay", 0.0),
                                   laguerre_modes=f.get("modes"), laguerre_phases=f.get("phases"),
                                   profile=f.get("profile", "GaussianPulse"), ramp_init=f.get("ramp_init", 0.0),
                                   plateau=f.get("plateau", 0.0), pulse_duration=f.get("pulse_duration", 0.0),
                                   waist_axis=f.get("waist_axis"), pulse_init=f.get("pulse_init", 0.0), **BEAM)
        sim.run(STEPS)
        Eg, Bg = sim.get_field("E"), sim.get_field("B")
    E = np.zeros_like(Eg)
    B = np.zeros_like(Bg)
    of = [oracle_face(gd, f["axis"], f["dir"], f["surface"], f["pol"], f["center"], f.get("prop"), f.get("polvec"),
                      f.get("circular", False), f.get("delay", 0.0), f.get("modes"), f.get("phases"),
                      f.get("profile", "GaussianPulse"), f.get("ramp_init", 0.0), f.get("plateau", 0.0),
                      f.get("pulse_duration", 0.0), f.get("waist_axis"), f.get("pulse_init", 0.0)) for f in faces]
    dt = np.float32(g.dt)
    for s in range(STEPS):
        # the times of the field stages: step dt, step dt + dt/2, (step + 1) dt, in float
        t0 = np.float32(np.float64(s) * np.float64(dt))
        th = np.float32(t0 + np.float32(0.5) * dt)
        t1 = np.float32(np.float64(s + 1) * np.float64(dt))
        orc.yee_b_half(gd, E, B)
        for f in of:
            orc.incident_update(gd, f, B, True, float(t0))
        orc.yee_e(gd, B, E)
        for f in of:
            orc.incident_update(gd, f, E, False, float(th))
        orc.yee_b_half(gd, E, B)
        for f in of:
            orc.incident_update(gd, f, B, True, float(t1))
    return Eg, Bg, E, B


@pytest.mark.parametrize("axis,direction,pol", [(1, 1, 0), (1, -1, 1), (0, 1, 1), (0, -1, 0), (2, 1, 0), (2, -1, 1)])
def test_face_matches_the_oracle(axis, direction, pol):
    surface = 16 if direction > 0 else LONG - 1 - 16
    Eg, Bg, E, B = run_both(axis, [dict(axis=axis, dir=direction, surface=surface, pol=pol, center=(13.0, 18.5))])
    scale = max(np.abs(E).max(), np.abs(B).max())
    assert scale > 0.1  # the pulse is inside (spread 34 cells past its focus: about 0.28 of E0 = 0.785)
    assert np.abs(Eg - E).max() <= TOL * E0, np.abs(Eg - E).max() / E0
    assert np.abs(Bg - B).max() <= TOL * E0, np.abs(Bg - B).max() / E0


def test_two_faces_match_the_oracle():
    faces = [dict(axis=1, dir=1, surface=16, pol=0, center=(13.0, 18.5)),
             dict(axis=1, dir=-1, surface=LONG - 1 - 16, pol=1, center=(17.0, 14.0))]
    Eg, Bg, E, B = run_both(1, faces)
    assert np.abs(Eg - E).max() <= TOL * E0, np.abs(Eg - E).max() / E0
    assert np.abs(Bg - B).max() <= TOL * E0, np.abs(Bg - B).max() / E0


def unit(v):
    v = np.asarray(v, np.float64)
    return tuple(v / np.linalg.norm(v))


TH = math.radians(25.0)
OBLIQUE = [
    # s-polarised through the low y face, 25 degrees off the normal in the x-y plane
    dict(axis=1, dir=1, surface=16, pol=0, center=(13.0, 18.5), prop=(math.sin(TH), math.cos(TH), 0.0),
         polvec=(0.0, 0.0, 1.0)),
    # p-polarised (E in the plane of incidence)
    dict(axis=1, dir=1, surface=16, pol=0, center=(13.0, 18.5), prop=(math.sin(TH), math.cos(TH), 0.0),
         polvec=(math.cos(TH), -math.sin(TH), 0.0)),
    # through the high x face, 30 degrees towards +z
    dict(axis=0, dir=-1, surface=LONG - 1 - 16, pol=0, center=(13.0, 18.5),
         prop=(-math.cos(math.radians(30)), 0.0, math.sin(math.radians(30))), polvec=(0.0, 1.0, 0.0)),
    # circular, normal incidence through the low z face
    dict(axis=2, dir=1, surface=16, pol=0, center=(13.0, 18.5), circular=True),
    # circular and oblique through the high y face
    dict(axis=1, dir=-1, surface=LONG - 1 - 16, pol=0, center=(15.0, 14.0), prop=unit((0.3, -0.85, 0.4)),
         polvec=unit(np.cross(unit((0.3, -0.85, 0.4)), (1.0, 0.0, 0.0))), circular=True),


    # a sum of three Laguerre-Gauss modes with phases, and TIME_DELAY
    dict(axis=1, dir=1, surface=16, pol=1, center=(13.0, 18.5), delay=7.5, modes=(1.0, 0.5, -0.25),
         phases=(0.0, 0.3, -0.2)),
    # the same, circular and oblique
    dict(axis=1, dir=1, surface=16, pol=0, center=(13.0, 18.5), prop=(math.sin(TH), math.cos(TH), 0.0),
         polvec=(0.0, 0.0, 1.0), circular=True, delay=3.0, modes=(0.8, 0.4, 0.2, 0.1), phases=(0.1, 0.0, 0.5, 1.0)),
    # the PlaneWave profile: ramps of 4 PULSE_DURATIONs around a plateau of 20
    dict(axis=1, dir=1, surface=16, pol=0, center=(13.0, 18.5), profile="PlaneWave", ramp_init=4.0, plateau=20.0),
    # PlaneWave, circular, oblique, through the high z face, with TIME_DELAY
    dict(axis=2, dir=-1, surface=LONG - 1 - 16, pol=0, center=(13.0, 18.5), profile="PlaneWave", ramp_init=3.0,
         plateau=10.0, prop=unit((0.2, 0.3, -0.9)), polvec=unit(np.cross(unit((0.2, 0.3, -0.9)), (0.0, 1.0, 0.0))),
         circular=True, delay=2.0),
    # Wavepacket: separate transverse waists, PULSE_INIT, a plateau; circular and oblique
    dict(axis=1, dir=1, surface=16, pol=0, center=(13.0, 18.5), profile="Wavepacket", waist_axis=(5.0, 8.0),
         pulse_init=4.0, plateau=6.0, prop=(math.sin(TH), math.cos(TH), 0.0), polvec=(0.0, 0.0, 1.0), circular=True),
    # Polynom with an explicit PULSE_DURATION, through the low x face
    dict(axis=0, dir=1, surface=16, pol=1, center=(13.0, 18.5), profile="Polynom", waist_axis=(6.0, 4.0),
         pulse_duration=30.0),
]


@pytest.mark.parametrize("face", OBLIQUE, ids=["s-pol", "p-pol", "x-high", "circular", "oblique-circular",
                                               "laguerre-delay", "laguerre-circular-oblique", "plane-wave",
                                               "plane-wave-circular-oblique", "wavepacket", "polynom"])
def test_oblique_and_circular_faces_match_the_oracle(face):
    Eg, Bg, E, B = run_both(face["axis"], [face])
    scale = max(np.abs(E).max(), np.abs(B).max())
    assert scale > 0.05
    assert np.abs(Eg - E).max() <= TOL * E0, np.abs(Eg - E).max() / E0
    assert np.abs(Bg - B).max() <= TOL * E0, np.abs(Bg - B).max() / E0


def test_oblique_pulse_travels_along_its_direction():
    """The E-field energy centroid of a 30-degree pulse through the low y face moves along the
    propagation direction: the angle of its displacement between two times is within 3 degrees."""
    th = math.radians(30.0)
    g = pg.Grid(128, 96, 32)
    with pg.Simulation(g) as sim:
        sim.set_incident_field(a0=1.0, wavelength=8.0, waist=8.0, duration_fwhm=12.0, t_center=30.0, surface=8,
                               center=(32.0, 16.0), focus=20.0, propagation=(math.sin(th), math.cos(th), 0.0),
                               polarisation_vector=(0.0, 0.0, 1.0))
        cents = []
        for steps in (110, 50):
            sim.run(steps)
            Ez = sim.get_field("E")[2].astype(np.float64)
            w = (Ez ** 2).sum(axis=0)  # over z: [y][x]
            w[:12, :] = 0.0  # the region next to the surface
            y, x = np.mgrid[0:96, 0:128]
            cents.append(((w * x).sum() / w.sum(), (w * y).sum() / w.sum()))
    dx, dy = cents[1][0] - cents[0][0], cents[1][1] - cents[0][1]
    ang = math.degrees(math.atan2(dx, dy))
    assert abs(ang - 30.0) < 3.0, ang
    assert math.hypot(dx, dy) > 15.0
