"""Checkpoint and restart of a simulation through the openPMD files (Checkpoint::notify and
Simulation::restart of the reference): the restored state is bit-identical to the written
one, a restart onto another supercell size keeps every particle in its cell, and a
restarted run continues the original one."""
import numpy as np
import pytest

import picongpu_gb300 as pg
from picongpu_gb300 import openpmd
from plasma import global_cells, random_field, random_particles

pytestmark = pytest.mark.gpu


def _sim(sc=(8, 8, 4)):
    g = pg.Grid(32, 32, 16, supercell=sc)
    sim = pg.Simulation(g)
    sim.add_species(pg.Species("e", -1.0, 1.0, shape="TSC", with_ids=True))
    sim.add_species(pg.Species("i", 1.0, 1836.0, pusher="Vay", shape="TSC"))
    return g, sim


def _seed(sim, g):
    gd = g.as_dict()
    rng = np.random.default_rng(17)
    pe = random_particles(gd, 4, rng, u_th=0.1, weight=0.01)
    pi = random_particles(gd, 4, rng, u_th=0.002, mass=1836.0, weight=0.01)
    pi["pos"] = pe["pos"].copy()
    del pi["id"]
    sim.set_particles("e", pe)
    sim.set_particles("i", pi)
    sim.set_field("E", random_field(gd, rng, 0.02))
    sim.set_field("B", random_field(gd, rng, 0.02))


def _by_id(p):
    o = np.argsort(p["id"], kind="stable")
    return {k: (v[:, o] if v.ndim == 2 else v[o]) for k, v in p.items()}


def _canonical(g, p):
    """Particles without ids in a canonical order (global cell, then position and momentum)."""
    cell = global_cells(g.as_dict(), p)
    keys = np.vstack([p["mom"][::-1], p["pos"][::-1], cell[::-1]])
    o = np.lexsort(keys)
    return cell[:, o], p["pos"][:, o], p["mom"][:, o], p["w"][o]


def test_round_trip_is_bit_exact(tmp_path):
    d = str(tmp_path / "ckpt")
    g, a = _sim()
    with a:
        _seed(a, g)
        a.run(3)
        a.write_checkpoint(d)
        E, B = a.get_field("E"), a.get_field("B")
        pe, pi = _by_id(a.get_particles("e")), a.get_particles("i")
        assert np.array_equal(openpmd.read_mesh(d, 3, "E"), E)
    g, b = _sim()
    with b:
        b.read_checkpoint(d, 3)
        assert b.current_step == 3
        assert np.array_equal(b.get_field("E"), E) and np.array_equal(b.get_field("B"), B)
        assert not b.get_field("J").any()
        qe, qi = _by_id(b.get_particles("e")), b.get_particles("i")
    for k in ("pos", "mom", "w", "sc", "lcell", "id"):
        assert np.array_equal(qe[k], pe[k]), k
    for x, y in zip(_canonical(g, qi), _canonical(g, pi)):
        assert np.array_equal(x, y)


def test_restart_onto_another_supercell(tmp_path):
    d = str(tmp_path / "ckpt")
    g, a = _sim()
    with a:
        _seed(a, g)
        a.run(2)
        a.write_checkpoint(d)
        pe = _by_id(a.get_particles("e"))
    g4, b = _sim(sc=(4, 4, 4))
    with b:
        b.read_checkpoint(d, 2)
        qe = _by_id(b.get_particles("e"))
        b.run(1)  # the restored layout steps
        assert b.device_status() == 0
    assert np.array_equal(global_cells(g4.as_dict(), qe), global_cells(g.as_dict(), pe))
    for k in ("pos", "mom", "w", "id"):
        assert np.array_equal(qe[k], pe[k]), k


def test_restart_continues_the_run(tmp_path):
    """Three more steps after a restart agree with three more steps of the original run.
    J is summed with float atomics in an arbitrary order, so the two runs agree to rounding,
    not bit for bit."""
    d = str(tmp_path / "ckpt")
    g, a = _sim()
    with a:
        _seed(a, g)
        a.run(3)
        a.write_checkpoint(d)
        a.run(3)
        Ea, pa = a.get_field("E"), _by_id(a.get_particles("e"))
        ena = a.energies()
    g, b = _sim()
    with b:
        b.read_checkpoint(d, 3)
        b.run(3)
        Eb, pb = b.get_field("E"), _by_id(b.get_particles("e"))
        enb = b.energies()
    assert np.abs(Eb - Ea).max() <= 1e-5 * np.abs(Ea).max()
    assert np.array_equal(pa["id"], pb["id"])
    assert np.allclose(pb["mom"], pa["mom"], rtol=1e-4, atol=1e-7)
    moved = np.any(global_cells(g.as_dict(), pa) != global_cells(g.as_dict(), pb), axis=0)
    assert moved.mean() < 1e-4  # only particles within rounding of a cell face may differ
    for k in ena:
        assert enb[k] == pytest.approx(ena[k], rel=1e-5)


def test_restart_needs_every_species(tmp_path):
    d = str(tmp_path / "ckpt")
    g, a = _sim()
    with a:
        _seed(a, g)
        a.write_checkpoint(d)
    g = pg.Grid(32, 32, 16)
    with pg.Simulation(g) as b:
        b.add_species(pg.Species("p", 1.0, 1836.0))
        with pytest.raises(pg.PicError) as e:
            b.read_checkpoint(d, 0)
        assert e.value.code == pg._lib.ERR_NOT_FOUND
    with pg.Simulation(pg.Grid(16, 32, 16)) as c:
        with pytest.raises(pg.PicError) as e:
            c.read_checkpoint(d, 0)
        assert e.value.code == pg._lib.ERR_IO


def test_restart_with_open_boundaries_is_exact(tmp_path):
    """A pulse in a box open along y with a PML: the checkpoint keeps the PML's convolution
    fields, so the fields after a restart continue bit for bit (no particles, no atomics)."""
    import os
    import sys

    sys.path.insert(0, os.path.dirname(__file__))
    from test_oracle_pml import _pulse

    d = str(tmp_path / "ckpt")
    g = pg.Grid(8, 96, 8)
    E, B = _pulse(g.as_dict(), y0=70.0)
    bnd = dict(open_axes=(False, True, False), thickness=((0, 0), (12, 12), (0, 0)), alpha_max=(0.0, 0.2, 0.0))
    with pg.Simulation(g) as a:
        a.set_boundaries(**bnd)
        a.set_field("E", E)
        a.set_field("B", B)
        a.run(20)  # the pulse is inside the positive PML now
        a.write_checkpoint(d)
        a.run(20)
        Ea, Ba = a.get_field("E"), a.get_field("B")
    with pg.Simulation(g) as b:
        b.set_boundaries(**bnd)
        b.read_checkpoint(d, 20)
        b.run(20)
        Eb, Bb = b.get_field("E"), b.get_field("B")
    assert np.array_equal(Ea, Eb) and np.array_equal(Ba, Bb)
    assert os.path.exists(os.path.join(d, "simData_20", "meshes_PmlPsiB_zy.bin"))
