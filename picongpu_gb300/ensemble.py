"""Batched ensemble: many independent periodic boxes of uneven size stepped together.

Each box is a complete single-box simulation (``box(i)`` returns a
``Simulation`` view of it, so particles, fields and diagnostics are read and
written as usual).  ``run(n)`` advances every box with the batched step: each
kernel of Simulation::runOneStep runs once over all boxes, the push as one
launch per species over every supercell of every box, and the step is one CUDA
graph launch.  ``run_sequential(n)`` advances the boxes one after the other
through the single-box path instead.  ``autotune`` picks the supercell size
and the threads per supercell of the batched push by timing each candidate.
"""
from __future__ import annotations

import ctypes
from dataclasses import replace

import numpy as np

from . import _lib as L
from .simulation import CURRENTS, PUSHERS, SHAPES, SOLVERS, SUPERCELLS, Grid, Simulation, Species

CANDIDATES = [(sc, t) for sc in ((8, 8, 4), (4, 4, 4), (8, 8, 8)) for t in (128, 256, 512)]


def _config(dims, grid: Grid, threads: int):
    dims = np.ascontiguousarray(np.asarray(dims, dtype=np.int32).reshape(-1, 3))
    g = L.GridConfig(0, 0, 0, SUPERCELLS[tuple(grid.supercell)], grid.dx, grid.dy, grid.dz, grid.dt, grid.c, grid.eps0,
                     SOLVERS[grid.solver], 1, grid.device)
    cfg = L.EnsembleConfig(g, dims.shape[0], dims.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), threads)
    return cfg, dims


def _species_config(sp: Species) -> L.SpeciesConfig:
    return L.SpeciesConfig(sp.name.encode(), sp.charge, sp.mass, PUSHERS.get(sp.pusher, L.PUSHER_NONE),
                           SHAPES[sp.shape], CURRENTS[sp.current], sp.capacity, int(sp.with_ids))


def plasma_init(ppc: int, density: float, u_th: float, drift_lo=(0.0, 0.0, 0.0), drift_hi=None, split_axis: int = -1,
                split_cell: int = 0, seed: int = 42, position_seed: int = 42, quiet=None) -> L.PlasmaInit:
    """One box's seeded plasma (the fields of picgb_plasma_init); quiet=(nx, ny, nz) selects the
    lattice start."""
    return L.PlasmaInit(ppc, density, u_th, (ctypes.c_float * 3)(*drift_lo),
                        (ctypes.c_float * 3)(*(drift_hi if drift_hi is not None else drift_lo)), split_axis,
                        split_cell, seed, position_seed, (ctypes.c_uint32 * 3)(*(quiet or (0, 0, 0))))


class Ensemble:
    def __init__(self, dims, grid: Grid | None = None, threads: int = 256):
        self.grid = grid if grid is not None else Grid(8, 8, 4)
        cfg, self.dims = _config(dims, self.grid, threads)
        h = ctypes.c_void_p()
        L.call("picgb_ensemble_create", ctypes.byref(cfg), ctypes.byref(h))
        self.handle = h
        self.threads = threads
        self.species: list[Species] = []

    def __len__(self) -> int:
        return int(self.dims.shape[0])

    def close(self):
        if self.handle:
            L.load().picgb_ensemble_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_species(self, sp: Species) -> int:
        cfg = _species_config(sp)
        idx = ctypes.c_int32()
        L.call("picgb_ensemble_add_species", self.handle, ctypes.byref(cfg), ctypes.byref(idx))
        self.species.append(sp)
        return idx.value

    def init_plasma(self, name: str, per_box: list[L.PlasmaInit]) -> None:
        if len(per_box) != len(self):
            raise ValueError("one plasma init per box is needed")
        arr = (L.PlasmaInit * len(per_box))(*per_box)
        L.call("picgb_ensemble_init_plasma", self.handle, self._index(name), arr)

    def _index(self, name: str) -> int:
        for i, s in enumerate(self.species):
            if s.name == name:
                return i
        raise RuntimeError(f"unknown species '{name}'")

    def box(self, i: int) -> Simulation:
        h = ctypes.c_void_p()
        L.call("picgb_ensemble_box", self.handle, i, ctypes.byref(h))
        nx, ny, nz = (int(v) for v in self.dims[i])
        return Simulation.borrowed(h, replace(self.grid, nx=nx, ny=ny, nz=nz, fuse_deposit=True), self.species)

    def run(self, n: int) -> None:
        L.call("picgb_ensemble_run", self.handle, n)

    def set_sort_interval(self, steps: int) -> None:
        """Restore the interleaved cell order every `steps` steps (0: never), in the batched step
        and in every box's single-box step; see picgb_ensemble_set_sort_interval."""
        L.call("picgb_ensemble_set_sort_interval", self.handle, int(steps))

    def run_sequential(self, n: int) -> None:
        L.call("picgb_ensemble_run_sequential", self.handle, n)

    def launch_count(self) -> int:
        v = ctypes.c_uint64()
        L.call("picgb_ensemble_launch_count", self.handle, ctypes.byref(v))
        return v.value

    def particle_count(self) -> int:
        total = 0
        for i in range(len(self)):
            b = self.box(i)
            total += sum(b.particle_count(s.name) for s in self.species if s.pusher is not None)
        return total


def autotune(dims, species: list[Species], inits: list[list[L.PlasmaInit]], grid: Grid | None = None,
             warmup: int = 2, steps: int = 3):
    """Times every (supercell, threads) candidate on the ensemble; returns
    (supercell, threads, {candidate: particle-steps/s})."""
    grid = grid if grid is not None else Grid(8, 8, 4)
    cfg, dims_arr = _config(dims, grid, 256)
    nbox = dims_arr.shape[0]
    scfg = (L.SpeciesConfig * len(species))(*[_species_config(s) for s in species])
    flat = [p for per in inits for p in per]
    if len(flat) != len(species) * nbox:
        raise ValueError("inits needs one list of per-box inits per species")
    ini = (L.PlasmaInit * len(flat))(*flat)
    sc, th = ctypes.c_int32(), ctypes.c_int32()
    rates = (ctypes.c_double * len(CANDIDATES))()
    L.call("picgb_ensemble_autotune", ctypes.byref(cfg), len(species), scfg, ini, warmup, steps, ctypes.byref(sc),
           ctypes.byref(th), rates)
    inv = {v: k for k, v in SUPERCELLS.items()}
    return inv[sc.value], th.value, {CANDIDATES[i]: rates[i] for i in range(len(CANDIDATES))}
