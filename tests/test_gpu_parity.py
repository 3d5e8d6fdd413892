"""CUDA path vs. the CPU oracle on identical seeded inputs, through the C-ABI.

Contract (parity bar of the PIC hot path):
* Yee updates, gathered fields, momenta, positions, supercell indices,
  localCellIdx and per-cell particle counts after one step: bit-exact (the
  CUDA kernels evaluate the same IEEE operations in the same order, with a
  correctly rounded 1/sqrt on both sides);
* J after a step: |dJ| <= 1e-6 * max|J| (the deposit sums with atomics, in a
  different order than the oracle);
* E after a full step (it absorbs J): |dE| <= 1e-6 * max|E|.
"""
import ctypes

import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import random_field, random_particles

pytestmark = pytest.mark.gpu

REL = 1e-6


def make_grid(n=(32, 32, 32), sc=(8, 8, 4), fuse=True, dt=None):
    g = pg.Grid(*n, supercell=sc, fuse_deposit=fuse)
    if dt is not None:
        g.dt = float(np.float32(dt))
    return g


def sorted_by_id(p):
    o = np.argsort(p["id"], kind="stable")
    return {k: (v[:, o] if v.ndim == 2 else v[o]) for k, v in p.items()}


def counts_per_cell(g, p):
    nsx, nsy = g.nx // g.sx, g.ny // g.sy
    vol = g.sx * g.sy * g.sz
    key = p["sc"].astype(np.int64) * vol + p["lcell"].astype(np.int64)
    return np.bincount(key, minlength=(g.nx // g.sx) * nsy * (g.nz // g.sz) * vol)


def max_rel(a, b):
    scale = max(float(np.abs(b).max()), 1e-30)
    return float(np.abs(a.astype(np.float64) - b).max()) / scale


@pytest.fixture(scope="module")
def orc():
    import oracle

    oracle.build()
    oracle.set_threads(1)
    return oracle


def test_library_loads_native():
    L = pg.load()
    assert L.picgb_abi_version() == 1


def test_yee_bit_exact(orc):
    g = make_grid((32, 16, 24), sc=(8, 8, 4))
    rng = np.random.default_rng(11)
    E, B, J = random_field(g.as_dict(), rng), random_field(g.as_dict(), rng), random_field(g.as_dict(), rng)
    with pg.Simulation(g) as sim:
        sim.set_field("E", E)
        sim.set_field("B", B)
        sim.set_field("J", J)
        sim.stage("field_before")  # B half, E (+ coeff J with the fused deposit)
        sim.stage("field_after")  # B half
        Eg, Bg = sim.get_field("E"), sim.get_field("B")
    gd = g.as_dict()
    orc.yee_b_half(gd, E, B)
    orc.yee_e(gd, B, E)
    orc.add_current(gd, J, E)
    orc.yee_b_half(gd, E, B)
    assert np.array_equal(Eg, E)
    assert np.array_equal(Bg, B)


@pytest.mark.parametrize("shape", ["CIC", "TSC", "PQS", "PCS"])
@pytest.mark.parametrize("sc", [(8, 8, 4), (4, 4, 4), (8, 8, 8)])
def test_push_and_deposit_one_step(orc, shape, sc):
    """Gather + Boris + move + sort bit-exact; fused Esirkepov deposit within 1e-6."""
    _push_and_deposit(orc, shape, sc, "Boris")


@pytest.mark.parametrize("pusher", ["HigueraCary", "Vay"])
@pytest.mark.parametrize("shape", ["CIC", "TSC", "PQS", "PCS"])
def test_higuera_cary_and_vay_one_step(orc, pusher, shape):
    """The HigueraCary and Vay pushers (square-root stages in double) bit-exact with the oracle."""
    _push_and_deposit(orc, shape, (8, 8, 4), pusher, amp=0.3)


def test_photon_push_bit_exact(orc):
    """Photon species (particlePusherPhoton.hpp, no charge, no current): positions bit-exact."""
    g = make_grid((32, 32, 32))
    gd = g.as_dict()
    rng = np.random.default_rng(41)
    p = random_particles(gd, 2, rng, u_th=1.0, weight=0.01)
    sp = pg.Species("ph", charge=0.0, mass=0.0, pusher="Photon", shape="TSC", current=None, with_ids=True)
    zero = np.zeros((3, g.nz, g.ny, g.nx), np.float32)
    with pg.Simulation(g) as sim:
        sim.add_species(sp)
        sim.set_particles("ph", p)
        sim.stage("push")
        q = sorted_by_id(sim.get_particles("ph"))
    orc.push(gd, sp.as_dict(), p, zero, zero)
    for k in ("pos", "mom", "sc", "lcell"):
        assert np.array_equal(q[k], p[k]), k


@pytest.mark.parametrize("pusher", ["Boris", "HigueraCary"])
@pytest.mark.parametrize("shape", ["CIC", "TSC", "PQS", "PCS"])
def test_emz_one_step(orc, pusher, shape):
    """The EmZ deposit (fields/currentDeposition/EmZ/EmZ.hpp) fused into the push, within 1e-6."""
    _push_and_deposit(orc, shape, (8, 8, 4), pusher, current="EmZ")


def _push_and_deposit(orc, shape, sc, pusher, amp=0.05, current="Esirkepov"):
    g = make_grid((32, 32, 32) if sc != (8, 8, 8) else (32, 32, 16), sc=sc)
    gd = g.as_dict()
    rng = np.random.default_rng(100 + len(shape) + sc[2] + len(pusher))
    p = random_particles(gd, 4, rng, u_th=0.2, weight=0.01)  # hot: many cell and supercell crossings
    E = random_field(gd, rng, amp=amp)
    B = random_field(gd, rng, amp=amp)
    sp = pg.Species("e", charge=-1.0, mass=1.0, pusher=pusher, shape=shape, current=current, with_ids=True)
    with pg.Simulation(g) as sim:
        sim.add_species(sp)
        sim.set_particles("e", p)
        sim.set_field("E", E)
        sim.set_field("B", B)
        sim.stage("current_reset")
        sim.stage("push")
        q = sorted_by_id(sim.get_particles("e"))
        Jg = sim.get_field("J")
        assert sim.device_status() == 0
    ref = {k: v.copy() for k, v in p.items()}
    orc.push(gd, sp.as_dict(), ref, E, B)
    for k in ("pos", "mom", "w", "sc", "lcell"):
        assert np.array_equal(q[k], ref[k]), k
    assert np.array_equal(counts_per_cell(g, q), counts_per_cell(g, ref))
    Jo = np.zeros_like(E)
    orc.deposit(gd, sp.as_dict(), ref, Jo)
    assert max_rel(Jg, Jo) <= REL


@pytest.mark.parametrize("current", ["Esirkepov", "EmZ"])
@pytest.mark.parametrize("fuse", [True, False])
def test_full_step_two_species(orc, fuse, current):
    """One Simulation::runOneStep of an electron-proton plasma (CIC), both deposit orders."""
    g = make_grid((32, 32, 32), fuse=fuse)
    gd = g.as_dict()
    rng = np.random.default_rng(5)
    pe = random_particles(gd, 4, rng, u_th=0.05, weight=0.01)
    pi = random_particles(gd, 4, rng, u_th=0.05 / np.sqrt(1836.0), mass=1836.0, weight=0.01)
    pi["pos"] = pe["pos"].copy()  # protons start on the electrons: quasi-neutral
    E, B = random_field(gd, rng, 0.02), random_field(gd, rng, 0.02)
    se = pg.Species("e", -1.0, 1.0, shape="CIC", current=current, with_ids=True)
    si = pg.Species("i", 1.0, 1836.0, shape="CIC", current=current, with_ids=True)
    with pg.Simulation(g) as sim:
        sim.add_species(se)
        sim.add_species(si)
        sim.set_particles("e", pe)
        sim.set_particles("i", pi)
        sim.set_field("E", E)
        sim.set_field("B", B)
        sim.step()
        qe, qi = sorted_by_id(sim.get_particles("e")), sorted_by_id(sim.get_particles("i"))
        Eg, Bg, Jg = sim.get_field("E"), sim.get_field("B"), sim.get_field("J")
    J = np.zeros_like(E)
    orc.step(gd, [se.as_dict(), si.as_dict()], [pe, pi], E, B, J)
    for q, r in ((qe, pe), (qi, pi)):
        for k in ("pos", "mom", "sc", "lcell"):
            assert np.array_equal(q[k], r[k]), k
    assert max_rel(Jg, J) <= REL
    assert max_rel(Eg, E) <= REL
    assert max_rel(Bg, B) <= REL


def test_counts_bit_exact_with_drift(orc):
    """Strong drift: most particles change cell, many change supercell."""
    g = make_grid((32, 32, 32))
    gd = g.as_dict()
    rng = np.random.default_rng(9)
    p = random_particles(gd, 8, rng, u_th=0.05, drift=(0.9, -0.7, 0.5), weight=0.01)
    sp = pg.Species("e", -1.0, 1.0, shape="TSC", with_ids=True)
    zeros = np.zeros((3, g.nz, g.ny, g.nx), np.float32)
    sc0 = p["sc"].copy()
    with pg.Simulation(g) as sim:
        sim.add_species(sp)
        sim.set_particles("e", p)
        sim.stage("current_reset")
        sim.stage("push")
        q = sorted_by_id(sim.get_particles("e"))
    orc.push(gd, sp.as_dict(), p, zeros, zeros)
    assert np.array_equal(q["sc"], p["sc"]) and np.array_equal(q["lcell"], p["lcell"])
    assert np.array_equal(counts_per_cell(g, q), counts_per_cell(g, p))
    assert (q["sc"] != sc0).mean() > 0.05


def test_overflow_relayout_keeps_every_particle():
    """Counter-streaming halves double the density where they overlap; with a
    tight capacity the spill + relayout path runs and no particle is lost."""
    g = make_grid((32, 16, 8))
    gd = g.as_dict()
    rng = np.random.default_rng(21)
    p = random_particles(gd, 2, rng, u_th=0.0, weight=0.01)
    from plasma import global_cells

    x = global_cells(gd, p)[0]
    u = np.where(x < g.nx // 2, 0.9, -0.9).astype(np.float32)
    p["mom"][0] = u * np.float32(0.01)
    n0 = p["w"].shape[0]
    sp = pg.Species("e", -1.0, 1.0, pusher="Free", shape="CIC", with_ids=True, capacity=544)
    with pg.Simulation(g) as sim:
        sim.add_species(sp)
        sim.set_particles("e", p)
        cap0 = sim.data_connector.get("e").capacity
        for _ in range(12):
            sim.step()
        q = sim.get_particles("e")
        cap1 = sim.data_connector.get("e").capacity
    assert q["w"].shape[0] == n0
    assert np.array_equal(np.sort(q["id"]), np.arange(n0, dtype=np.uint32))
    assert cap0 == 544 and cap1 > cap0


def test_data_connector_contract():
    g = make_grid((16, 16, 8))
    with pg.Simulation(g) as sim:
        sim.add_species(pg.Species("e", -1.0, 1.0))
        ids = set(sim.data_connector.ids())
        assert {"E", "B", "J", "FieldTmp0", "FieldSolverFDTD", "e"} <= ids
        d = sim.data_connector.get("E")
        assert d.kind == pg._lib.BUFFER_FIELD and d.ncomp == 3 and tuple(d.dims) == (16, 16, 8)
        assert tuple(d.guard) == (0, 0, 0) and d.ptr[0] and d.ptr[1] - d.ptr[0] == 16 * 16 * 8 * 4
        with pytest.raises(pg.PicError) as e:
            sim.data_connector.get("nope")
        assert e.value.code == pg._lib.ERR_NOT_FOUND
        with pytest.raises(pg.PicError) as e:
            sim.data_connector.share("E", d)
        assert e.value.code == pg._lib.ERR_DUPLICATE
        sim.data_connector.share("myE", d)
        assert sim.data_connector.get("myE").ptr[0] == d.ptr[0]
        sim.data_connector.unshare("myE")


def test_invalid_configs_are_rejected():
    with pytest.raises(pg.PicError) as e:
        pg.Simulation(pg.Grid(16, 16, 8, dt=1.0))  # CFL violated
    assert e.value.code == pg._lib.ERR_INVALID
    with pytest.raises(pg.PicError):
        pg.Simulation(pg.Grid(12, 16, 8))  # not a multiple of the supercell
    g = make_grid((16, 16, 8))
    with pg.Simulation(g) as sim:
        sim.add_species(pg.Species("e", -1.0, 1.0))
        bad = random_particles(g.as_dict(), 1, np.random.default_rng(0))
        bad["sc"][3] = 10_000
        with pytest.raises(pg.PicError) as e:
            sim.set_particles("e", bad)
        assert e.value.code == pg._lib.ERR_INVALID
        with pytest.raises(ValueError):
            sim.add_species(pg.Species("x", -1.0, 1.0, pusher="Axel"))
        with pytest.raises(ValueError):
            sim.add_species(pg.Species("x", -1.0, 1.0, shape="NGP"))
        with pytest.raises(ValueError):
            sim.add_species(pg.Species("x", -1.0, 1.0, current="None"))
        cfg = pg._lib.SpeciesConfig(b"y", -1.0, 1.0, 9, pg._lib.SHAPE_TSC, 1, 0, 0)  # no pusher 9
        idx = ctypes.c_int32()
        assert pg.load().picgb_add_species(sim.handle, ctypes.byref(cfg), ctypes.byref(idx)) == pg._lib.ERR_INVALID
        cfg = pg._lib.SpeciesConfig(b"z", -1.0, 0.0, pg._lib.PUSHER_BORIS, pg._lib.SHAPE_TSC, 1, 0, 0)  # massless Boris
        assert pg.load().picgb_add_species(sim.handle, ctypes.byref(cfg), ctypes.byref(idx)) == pg._lib.ERR_INVALID
