"""The interleaved cell order restored inside every supercell (picgb_set_sort_interval, kReorder).

* A step with the reorder is bit-exact in the particles (sorted by id) with the same step
  without it, and J agrees within 1e-6 of its maximum: the reorder only moves particles
  between slots of their supercell (single box and batched ensemble).
* After the reorder every supercell's slots are in the interleaved order: the key
  (rank of the particle among those of its cell, cell) increases along the slots, so the
  slots of the first m rounds (m = the smallest count of a cell) hold cell k mod vol.
* Over 30 steps with a reorder every 7 steps the FP64 energies follow the run without
  reorders within 1e-4 (the deposit sums in another order).
* The reorder of a step also compacts the slots the push vacated (kCompactReorder in place of
  kCompact): bit-exact with hole filling after one step, also for a supercell with a cell of
  more than 64 particles, where the sort gives way to hole filling.
* A species that leaves its supercells often (more than 3 % of it per step, measured by the
  reorder of the first step after its device initialisation and of every sort step) is
  reordered every step from then on; a cold one only in that first step and every sort
  interval.
"""
import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import random_field

pytestmark = pytest.mark.gpu

DT = float(np.float32(0.99 / np.sqrt(3.0)))


def make(sort_interval):
    g = pg.Grid(32, 32, 16, dt=DT)
    sim = pg.Simulation(g)
    sim.add_species(pg.Species("e", -1.0, 1.0, shape="TSC", with_ids=True))
    sim.add_species(pg.Species("i", 1.0, 1836.0, shape="TSC", with_ids=True))
    n = (0.1 / DT) ** 2
    sim.init_plasma("e", 8, n, 0.1, drift_lo=(0.2, 0.0, 0.0), seed=5, position_seed=6)
    sim.init_plasma("i", 8, n, 0.1 / np.sqrt(1836.0), seed=7, position_seed=6)
    rng = np.random.default_rng(3)
    sim.set_field("E", random_field(g.as_dict(), rng, 0.01))
    sim.set_field("B", random_field(g.as_dict(), rng, 0.01))
    sim.set_sort_interval(sort_interval)
    return g, sim


def sorted_by_id(p):
    o = np.argsort(p["id"], kind="stable")
    return {k: (v[:, o] if v.ndim == 2 else v[o]) for k, v in p.items()}


def test_reorder_moves_particles_only():
    # one step: the global J flush adds float atomics in any order, so two runs differ in
    # rounding after their first field update, with or without the reorder
    g, a = make(1)
    _, b = make(0)
    with a, b:
        a.step()
        b.step()
        for name in ("e", "i"):
            pa, pb = sorted_by_id(a.get_particles(name)), sorted_by_id(b.get_particles(name))
            for k in ("id", "pos", "mom", "w", "sc", "lcell"):
                assert np.array_equal(pa[k], pb[k]), (name, k)
        Ja, Jb = a.get_field("J"), b.get_field("J")
        assert np.abs(Ja - Jb).max() <= 1e-6 * np.abs(Jb).max()


def test_reorder_restores_the_interleaved_order():
    g, sim = make(0)
    vol = g.sx * g.sy * g.sz
    with sim:
        sim.run(15)  # drifted: particles kept their slots while they changed cells
        sim.set_sort_interval(1)
        sim.step()
        for name in ("e", "i"):
            p = sim.get_particles(name)  # supercell by supercell, slots in order
            sc = p["sc"]
            starts = np.flatnonzero(np.r_[True, sc[1:] != sc[:-1]])
            ends = np.r_[starts[1:], sc.size]
            for s0, s1 in zip(starts, ends):
                lc = p["lcell"][s0:s1].astype(np.int64)
                # rank of every particle among the earlier slots of its cell
                rank = np.zeros_like(lc)
                seen = np.zeros(vol, np.int64)
                for k, c in enumerate(lc):
                    rank[k] = seen[c]
                    seen[c] += 1
                key = rank * vol + lc
                assert np.all(np.diff(key) > 0), (name, int(sc[s0]))
                m = int(np.bincount(lc, minlength=vol).min())
                assert np.array_equal(lc[: m * vol], np.tile(np.arange(vol), m))


def test_energies_with_periodic_reorders():
    _, a = make(7)
    _, b = make(0)
    with a, b:
        for step in range(30):
            a.step()
            b.step()
        ea, eb = a.energies(), b.energies()
        for k in ("E", "B", "e", "i"):
            assert abs(ea[k] - eb[k]) <= 1e-4 * abs(eb[k]), (k, ea[k], eb[k])


def test_batched_reorder_moves_particles_only():
    """The batched step's reorder (one launch per species over every box) against the batched
    step without it: bit-exact particles, and every box in the interleaved order."""
    dims = [(16, 16, 8), (24, 16, 16)]
    runs = []
    for interval in (1, 0):
        ens = pg.Ensemble(dims)
        ens.add_species(pg.Species("e", -1.0, 1.0, shape="TSC", with_ids=True))
        ens.init_plasma("e", [pg.plasma_init(6, 0.03, 0.2, drift_lo=(0.3, 0.0, 0.0), seed=9 + b) for b in range(2)])
        ens.set_sort_interval(interval)
        ens.run(1)  # one step (see test_reorder_moves_particles_only)
        runs.append([ens.box(b).get_particles("e") for b in range(2)])
        ens.close()
    for pa, pb in zip(*runs):
        a, b = sorted_by_id(pa), sorted_by_id(pb)
        for k in ("id", "pos", "mom", "sc", "lcell"):
            assert np.array_equal(a[k], b[k]), k
    vol = 8 * 8 * 4
    for p in runs[0]:
        sc = p["sc"]
        starts = np.flatnonzero(np.r_[True, sc[1:] != sc[:-1]])
        for s0, s1 in zip(starts, np.r_[starts[1:], sc.size]):
            lc = p["lcell"][s0:s1].astype(np.int64)
            seen = np.zeros(vol, np.int64)
            key = np.empty_like(lc)
            for k, c in enumerate(lc):
                key[k] = seen[c] * vol + c
                seen[c] += 1
            assert np.all(np.diff(key) > 0)


def crowded(sort_interval):
    """A 4 ppc plasma plus 120 particles in cell (3, 3, 3), which some of them leave."""
    g = pg.Grid(32, 32, 16, dt=DT)
    sim = pg.Simulation(g)
    sim.add_species(pg.Species("e", -1.0, 1.0, shape="TSC", with_ids=True))
    sim.init_plasma("e", 4, 0.02, 0.2, seed=11, position_seed=12)
    p = sim.get_particles("e")
    rng = np.random.default_rng(13)
    m = 120
    extra = dict(pos=rng.random((3, m), dtype=np.float32), mom=(0.3 * rng.standard_normal((3, m))).astype(np.float32),
                 w=np.full(m, p["w"][0], np.float32), sc=np.zeros(m, np.int32),
                 lcell=np.full(m, 3 + 8 * (3 + 8 * 3), np.uint16),
                 id=np.arange(p["id"].max() + 1, p["id"].max() + 1 + m, dtype=np.uint32))
    sim.set_particles("e", {k: np.concatenate([p[k], extra[k]], axis=-1) for k in p})
    sim.set_sort_interval(sort_interval)
    return sim


def test_compacting_reorder_falls_back_for_a_crowded_cell():
    a, b = crowded(1), crowded(0)
    with a, b:
        n0 = a.particle_count("e")
        a.step()
        b.step()
        pa, pb = sorted_by_id(a.get_particles("e")), sorted_by_id(b.get_particles("e"))
        assert pa["id"].size == n0
        for k in ("id", "pos", "mom", "w", "sc", "lcell"):
            assert np.array_equal(pa[k], pb[k]), k
        assert a.device_status() == 0


def reorder_launches(u_th, steps):
    g = pg.Grid(32, 32, 16, dt=DT)
    with pg.Simulation(g) as sim:
        sim.add_species(pg.Species("e", -1.0, 1.0, shape="TSC"))
        sim.init_plasma("e", 4, 0.02, u_th, seed=15, position_seed=16)
        n0 = sim.particle_count("e")
        sim.profile(True)
        sim.run(steps)
        kt = sim.kernel_times()
        assert sim.particle_count("e") == n0
        return kt["reorder"][1], kt["compact"][1]


def test_hot_species_is_reordered_every_step():
    # default interval 20: the reorders of steps 1 and 20 measure the leave fraction
    assert reorder_launches(0.001, 25) == (2, 23)  # cold: hole filling between the reorders
    assert reorder_launches(0.5, 25) == (25, 0)  # hot: every step from step 2 on
