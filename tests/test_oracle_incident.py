"""The oracle's incident field (its restatement of profiles/GaussianPulse.hpp and of the TF/SF
update of incidentField/Solver.kernel) against the float64 1D Yee reference, on the CPU.

A transversely uniform pulse (waist 1e6, wavelength 16, intensity FWHM 20 dt, t_center 40)
through one face of a vacuum box 256 cells long along the axis and 16 across, 200 steps of
the oracle's split Yee update with the face's corrections after every field update.
Contract: the tangential E and B on two lines along the axis match the 1D reference within
1e-4 of the amplitude, the other components stay below 1e-6 of it, and the scattered-field
region behind the surface holds less than 1e-5 of it.
"""
import math

import numpy as np
import pytest

import oracle as orc
import picongpu_gb300 as pg
from incident_1d import line, yee_1d

LONG, ACROSS = 256, 16
LAM = 16.0
STEPS = 200
OFF = 32


@pytest.mark.parametrize("axis,direction,pol", [(1, 1, 0), (0, -1, 1), (2, 1, 1)])
def test_oracle_face_matches_the_1d_reference(axis, direction, pol):
    d = [ACROSS] * 3
    d[axis] = LONG
    g = pg.Grid(*d)
    gd = g.as_dict()
    fwhm = 20 * float(np.float32(g.dt))
    tc = 40.0
    P = OFF if direction > 0 else LONG - 1 - OFF
    tau = fwhm / (2 * math.sqrt(2 * math.log(2)))
    t1, t2 = [a for a in range(3) if a != axis]
    focus = [0.0, 0.0, 0.0]
    focus[t1], focus[t2] = ACROSS / 2.0, ACROSS / 2.0
    focus[axis] = P - 0.25 * direction
    face = orc.incident_face(gd, axis, direction, P, pol, 1.0, LAM, 1e6, tau, -tc, 0.0, focus)
    E = np.zeros((3, d[2], d[1], d[0]), np.float32)
    B = np.zeros_like(E)
    dt = np.float32(g.dt)
    for s in range(STEPS):
        t0 = np.float32(np.float64(s) * np.float64(dt))
        th = np.float32(t0 + np.float32(0.5) * dt)
        t1_ = np.float32(np.float64(s + 1) * np.float64(dt))
        orc.yee_b_half(gd, E, B)
        orc.incident_update(gd, face, B, True, float(t0))
        orc.yee_e(gd, B, E)
        orc.incident_update(gd, face, E, False, float(th))
        orc.yee_b_half(gd, E, B)
        orc.incident_update(gd, face, B, True, float(t1_))
    E0 = 2 * math.pi / LAM
    e1, b1 = yee_1d(LONG, P, direction, g, LAM, fwhm, tc, STEPS)
    p = t1 if pol == 0 else t2
    o = t2 if pol == 0 else t1
    eta = 1.0 if p == (axis + 2) % 3 else -1.0
    assert np.abs(e1).max() > 0.5 * E0
    for u1, u2 in ((0, 0), (ACROSS // 3, ACROSS // 2)):
        assert np.abs(line(E, p, axis, u1, u2) - e1).max() <= 1e-4 * E0
        assert np.abs(line(B, o, axis, u1, u2) - eta * b1).max() <= 1e-4 * E0
        assert np.abs(line(E, o, axis, u1, u2)).max() <= 1e-6 * E0
        assert np.abs(line(E, axis, axis, u1, u2)).max() <= 1e-6 * E0
    sl = [slice(None)] * 3
    sl[2 - axis] = slice(0, P - 2) if direction > 0 else slice(P + 3, LONG)
    for F in (E, B):
        assert np.abs(F[(slice(None),) + tuple(sl)]).max() <= 1e-5 * E0
