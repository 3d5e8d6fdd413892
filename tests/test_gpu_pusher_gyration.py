"""The reference's Pusher integration test (share/picongpu/tests/Pusher) at its own size on the GPU.

Setup of the reference's test:
* one electron at 0.5c (gamma 1.1547, particle.param DriftParam) moving along x, perpendicular to
  a uniform B_z;
* 64 x 64 x 32 periodic cells, CIC shape, Esirkepov current (species.param);
* 50 steps per gyration period (simulation.param: DELTA_T_SI = T_GYRO_SI / 50), so that
  c dt / dx = 0.57518 with its cell of 8.6 um and step of 16.5 fs;
* start in cell (32, 5, 16) at in-cell offset 0 (density.param, OnePositionParameter).

Here c = dx = m = |q| = eps0 = 1 and B_z = 2 pi gamma / (50 dt).  In the reference B = 50 T enters
only the pusher (fieldBackground.param) and the one real electron's own field is some 1e-11 of the
Lorentz force; the weighting 1e-9 keeps the electron's field as negligible here while B_z sits in
the grid (a uniform field is a static solution of the Yee update).

Pass criteria of lib/python/test/Pusher/MainTest.py:177,212 and README.rst, between consecutive
turns over 10 turns:
* the radius from the momentum (p / (q B)) changes by less than 1e-5;
* the radius from the positions (circle fit) changes by less than 5e-5;
* the phase changes by less than 0.16 rad.
Boris is the test's pusher; Vay and HigueraCary as its pusher variants (cmakeFlags).
"""
import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import global_cells

pytestmark = pytest.mark.gpu

NX, NY, NZ = 64, 64, 32
DT = 299792458.0 * (0.825e-12 / 50.0) / 8.6e-6  # c dt / dx of the reference's setup
GAMMA = 1.1547
W = 1e-9
STEPS_PER_TURN = 50
TURNS = 10


def fit_circle(x, y):
    A = np.stack([x, y, np.ones_like(x)], axis=1)
    s = np.linalg.lstsq(A, x * x + y * y, rcond=None)[0]
    return s[0] / 2, s[1] / 2


@pytest.mark.parametrize("pusher", ["Boris", "Vay", "HigueraCary"])
def test_reference_pusher_setup(pusher):
    g = pg.Grid(NX, NY, NZ, dt=float(np.float32(DT)))
    gd = g.as_dict()
    u = GAMMA * np.sqrt(1.0 - 1.0 / GAMMA ** 2)  # gamma beta c
    B0 = 2 * np.pi * GAMMA / (STEPS_PER_TURN * g.dt)
    B = np.zeros((3, NZ, NY, NX), np.float32)
    B[2] = np.float32(B0)
    # cell (32, 5, 16): supercell (4, 0, 4) of the 8 x 8 x 4 supercells, cell (0, 5, 0) in it
    p = dict(pos=np.zeros((3, 1), np.float32), mom=np.array([[u * W], [0.0], [0.0]], np.float32),
             w=np.array([W], np.float32), sc=np.array([4 + 8 * (0 + 8 * 4)], np.int32),
             lcell=np.array([0 + 8 * (5 + 8 * 0)], np.uint16))
    with pg.Simulation(g) as sim:
        sim.add_species(pg.Species("e", -1.0, 1.0, pusher=pusher, shape="CIC", current="Esirkepov"))
        sim.set_particles("e", p)
        sim.set_field("B", B)
        q = sim.get_particles("e")
        assert np.array_equal(global_cells(gd, q)[:, 0], [32, 5, 16])
        xs, ys, rp = [], [], []
        for _ in range(STEPS_PER_TURN * TURNS + 1):
            q = sim.get_particles("e")
            cell = global_cells(gd, q)[:, 0]
            xs.append(cell[0] + float(q["pos"][0, 0]))
            ys.append(cell[1] + float(q["pos"][1, 0]))
            rp.append(np.hypot(float(q["mom"][0, 0]), float(q["mom"][1, 0])) / (W * B0))
            sim.step()
    xs, ys, rp = map(np.asarray, (xs, ys, rp))
    cx, cy = fit_circle(xs[:STEPS_PER_TURN], ys[:STEPS_PER_TURN])
    r = np.hypot(xs - cx, ys - cy)
    ph = np.unwrap(np.arctan2(ys - cy, xs - cx))
    for t in range(TURNS):
        i0, i1 = STEPS_PER_TURN * t, STEPS_PER_TURN * (t + 1)
        assert abs(rp[i1] - rp[i0]) / rp[i0] < 1e-5, (t, rp[i0], rp[i1])
        assert abs(r[i1] - r[i0]) / r[i0] < 5e-5, (t, r[i0], r[i1])
        dph = (ph[i1] - ph[i0]) % (2 * np.pi)
        assert min(dph, 2 * np.pi - dph) < 0.16, (t, dph)
    # the radius p / (q B) = gamma beta c / B, about 2.29 cells as in the reference's SI setup
    assert abs(r.mean() - u / B0) / (u / B0) < 0.02
