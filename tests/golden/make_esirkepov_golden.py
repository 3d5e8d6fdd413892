"""Generate single-particle Esirkepov golden vectors from the reference's own numpy code.

The reference validates its Esirkepov deposit in the CurrentDeposition
integration test (share/picongpu/tests/CurrentDeposition): one electron moving
one step with the Free pusher, the deposited J compared with a numpy
implementation (lib/python/test/CurrentDeposition/grid_class.py:97-199 and
assignment_and_W_func.py:15-117) within |dJ| < 1e-5 (MainTest.py:152).

This script imports that numpy implementation from a PIConGPU source tree and
evaluates it for the reference's own test cases (start offset (0.9, 0.8, 0.7),
directions (1,0,0), (1,1,0), (1,1,1), beta = 0.999, dt = 0.5 dx/c) and for
seeded random cases, for the CIC, TSC and PQS shapes.  With unit cells the
reference's normalisation (1/H)**order equals 1/V for every order, so every
shape is pinned.

What comes straight from the reference code:
  * ``wx``, ``wy``, ``wz``: the current deposition vector W on the minimal
    grid (grid.current_deposition_field, grid_class.py:97-131);
  * ``jx_ref``: the x current as grid.current_density_field returns it.
That last function is exact only for motion along +x with CIC or TSC, which is
what the reference CI runs: its loop ends use ``np.min`` of start and end
(grid_class.py:167), its y and z loops are ``range(start[2], start[2])``
(grid_class.py:184,192) and its grid offset ``r`` is one cell too large for
PQS (num_cells = order + 4 puts the particle in minimal cell 3, so the
minimal-to-global offset is cell0 - 3, while r evaluates to cell0 - 2).
``jx``, ``jy``, ``jz`` are therefore derived from the reference's W with the
Esirkepov definition J = -q/dt * dx * cumsum(W) along the component axis, over
the whole minimal grid, placed at global node = minimal node + cell0 -
start_cell.  The script asserts that the derived jx equals the reference's
own jx_ref on the cases where the latter is valid.

Usage (needs the reference tree; the fixture it writes is committed):
    python tests/golden/make_esirkepov_golden.py /path/to/picongpu
"""
import os
import sys

import numpy as np

N = 12  # periodic test grid, cells per axis
START = 5  # start cell per axis


def load_reference(ref_root):
    d = os.path.join(ref_root, "share/picongpu/tests/CurrentDeposition/lib/python/test/CurrentDeposition")
    sys.path.insert(0, d)
    from grid_class import grid  # noqa: E402

    return grid


def move(pos, cell):
    """Split a float32 position into (cell, in-cell) like particles/MoveParticle.hpp."""
    pos = pos.astype(np.float32)
    cell = cell.copy()
    out = np.zeros(3, np.float32)
    for d in range(3):
        p = np.float32(pos[d] - np.float32(0.5))
        mv = np.float32(0.0)
        if p < np.float32(-0.5):
            mv = np.float32(-1.0)
        if p >= np.float32(0.5):
            mv = np.float32(1.0)
        p = np.float32(p - mv)
        out[d] = np.float32(p + np.float32(0.5))
        cell[d] += int(mv)
    return out, cell


def run_case(grid, order, pos0, beta_vec, dt, charge):
    cell0 = np.array([START, START, START])
    vel = np.asarray(beta_vec, np.float32)  # c = 1
    dx = np.float32(1.0)
    new = np.array([pos0[d] + (vel[d] * np.float32(dt)) / dx for d in range(3)], np.float32)
    pos1, cell1 = move(new, cell0)

    g = grid(order)
    gx, gy, gz = g.create_grid()
    s, e = g.particle_step(pos0.astype(np.float64), pos1.astype(np.float64), cell0, cell1)
    wx, wy, wz = g.current_deposition_field(s, e, gx, gy, gz)
    params = dict(cell_width=1.0, cell_height=1.0, cell_depth=1.0, dt=float(dt), unit_time=1.0,
                  unit_length=1.0, unit_charge=1.0)
    shape = (N, N, N)
    jx_ref, _, _ = g.current_density_field(wx, wy, wz, s, e, charge, params, shape)

    comb = (-charge) / params["dt"]
    off = cell0 - int((g.num_cells - 1) / 2)  # global node = minimal node + off
    n = g.num_cells
    J = []
    for comp, W in enumerate((wx, wy, wz)):
        axis = 2 - comp  # W is indexed [z][y][x]
        C = comb * np.cumsum(W, axis=axis)
        full = np.zeros(shape)
        full[off[2]:off[2] + n, off[1]:off[1] + n, off[0]:off[0] + n] = C
        J.append(full.astype(np.float32))
    valid_ref = order in (1, 2) and beta_vec[1] == 0 and beta_vec[2] == 0 and beta_vec[0] > 0
    if valid_ref:
        assert np.abs(J[0] - jx_ref).max() < 1e-6, "derived jx disagrees with the reference's jx"
    return dict(order=order, pos0=pos0, cell0=cell0, vel=vel, dt=np.float32(dt), charge=np.float32(charge),
                pos1=pos1, cell1=cell1, wx=np.asarray(wx, np.float32), wy=np.asarray(wy, np.float32),
                wz=np.asarray(wz, np.float32), jx_ref=jx_ref.astype(np.float32), jx_ref_valid=np.array(valid_ref),
                jx=J[0], jy=J[1], jz=J[2])


def main():
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of a PIConGPU source tree>")
    grid = load_reference(sys.argv[1])
    cases = []
    beta = 0.999
    dt = 0.5
    for order in (1, 2, 3):
        for direc in ((1, 0, 0), (1, 1, 0), (1, 1, 1)):
            v = np.asarray(direc, np.float64)
            v = beta * v / np.linalg.norm(v)
            cases.append(run_case(grid, order, np.array([0.9, 0.8, 0.7], np.float32), v, dt, -1.0))
    rng = np.random.default_rng(20231)
    for order in (1, 2, 3):
        for _ in range(6):
            pos0 = rng.random(3).astype(np.float32)
            v = rng.normal(size=3)
            v = rng.uniform(0.05, 0.999) * v / np.linalg.norm(v)
            cases.append(run_case(grid, order, pos0, v, dt, float(rng.choice([-1.0, 1.0]))))
    out = {}
    for i, c in enumerate(cases):
        for k, v in c.items():
            out[f"c{i}_{k}"] = np.asarray(v)
    out["ncases"] = np.array(len(cases))
    out["grid_n"] = np.array(N)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "esirkepov_single_particle.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {len(cases)} cases to {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
