"""Host-side start distributions in the particle exchange format of ``Simulation.set_particles``.

``quiet_start`` places the macro particles of every cell on a regular in-cell lattice, the
reference's ``startPosition::Quiet`` (particles/startPosition/QuietImpl.hpp:40-110): with n_d
particles along axis d the in-cell position is i * s + s / 2, s = 1 / n_d, evaluated in float32
as two rounded operations.  Momenta follow ``manipulators::unary::Drift`` (a drift gamma*beta along
x, optionally of opposite sign beyond a plane) plus ``Temperature`` (a normal spread u_th per
component), as the device initialisation ``init_plasma`` does.

Differences to the reference: the weighting is density * cell volume / particles per cell in the
simulation's units, and the reference's MIN_WEIGHTING reduction of the lattice (which works on
SI real-particle counts) is left to the caller's choice of ``per_cell``.  Particles are ordered
supercell by supercell, and inside a supercell with consecutive particles in consecutive cells,
the order that keeps a warp's particles in different cells on the GPU.
"""
from __future__ import annotations

import numpy as np

from .simulation import Grid


def quiet_start(grid: Grid, per_cell=(2, 2, 2), density: float = 1.0, mass: float = 1.0, u_th: float = 0.0,
                drift_lo=(0.0, 0.0, 0.0), drift_hi=None, split_axis: int = -1, split_cell: int = 0, seed: int = 0,
                with_ids: bool = False) -> dict:
    """Particles of one species on a per_cell[0] x per_cell[1] x per_cell[2] lattice in every cell.

    density is in the simulation's units (the weighting of a macro particle is density * dx dy dz /
    particles per cell).  u_th and the drifts are gamma*beta; momenta are macro-weighted
    (u * mass * weighting * c), as the exchange format stores them.  Cells with a coordinate along
    split_axis at or beyond split_cell take drift_hi (when given) instead of drift_lo.
    """
    per = tuple(int(v) for v in per_cell)
    if len(per) != 3 or min(per) < 1:
        raise ValueError(f"per_cell needs three positive counts, got {per_cell!r}")
    if split_axis not in (-1, 0, 1, 2):
        raise ValueError(f"split_axis must be -1, 0, 1 or 2, got {split_axis}")
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    sx, sy, sz = grid.supercell
    vol = sx * sy * sz
    ppc = per[0] * per[1] * per[2]
    nsx, nsy, nsz = nx // sx, ny // sy, nz // sz
    nsc = nsx * nsy * nsz

    # in-cell lattice (x fastest), float32 with two roundings: i * s + s * 0.5
    f32 = np.float32
    axes = []
    for d in range(3):
        s = f32(1.0) / f32(per[d])
        axes.append((np.arange(per[d], dtype=f32) * s + s * f32(0.5)).astype(f32))
    lz, ly, lx = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    lattice = np.stack([lx.ravel(), ly.ravel(), lz.ravel()])  # [3][ppc]

    # slot k of a supercell: particle p = k // vol of local cell lc = k % vol
    k = np.arange(vol * ppc)
    lc, p = k % vol, k // vol
    sc = np.repeat(np.arange(nsc, dtype=np.int64), vol * ppc)
    lc_all = np.tile(lc, nsc)
    p_all = np.tile(p, nsc)
    scx, scy, scz = sc % nsx, (sc // nsx) % nsy, sc // (nsx * nsy)
    cx = scx * sx + lc_all % sx
    cy = scy * sy + (lc_all // sx) % sy
    cz = scz * sz + lc_all // (sx * sy)
    n = sc.size

    pos = np.ascontiguousarray(lattice[:, p_all])
    w = f32(density * grid.dx * grid.dy * grid.dz / ppc)
    u = np.zeros((3, n))
    u[:] = np.asarray(drift_lo, dtype=np.float64)[:, None]
    if drift_hi is not None and split_axis >= 0:
        hi = (cx, cy, cz)[split_axis] >= split_cell
        u[:, hi] = np.asarray(drift_hi, dtype=np.float64)[:, None]
    if u_th > 0.0:
        u += np.random.default_rng(seed).normal(0.0, u_th, size=(3, n))
    out = dict(pos=pos, mom=np.ascontiguousarray((u * mass * float(w) * grid.c).astype(f32)),
               w=np.full(n, w, f32), sc=sc.astype(np.int32), lcell=lc_all.astype(np.uint16))
    if with_ids:
        gc = cx + nx * (cy + ny * cz)
        out["id"] = (gc * ppc + p_all).astype(np.uint32)
    return out
