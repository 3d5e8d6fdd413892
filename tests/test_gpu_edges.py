"""Edge cases of one PIC step, CUDA path vs. the CPU oracle through the C-ABI.

* In-cell positions on the cell and half-cell boundaries (0, 1/2 and their float
  neighbours, the largest float below 1) with momenta that reach, cross or just miss a
  boundary: the cases of moveParticle (share/picongpu/unit/MoveParticle.cpp) and of the
  relay point of the deposits (Esirkepov.hpp:62-242, relayPoint.hpp:48-64).
* Particles in the corner cells of supercells, including the corners of the periodic box,
  leaving towards each of the 26 neighbours in one step (ParticlesBase.kernel:361-631).
* An empty species and a species that occupies three supercells only.

The parity bar is the one of test_gpu_parity.py: particles bit-exact, J and E within 1e-6
of their largest magnitude.
"""
import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import random_field, random_particles

pytestmark = pytest.mark.gpu

REL = 1e-6
F32 = np.float32


def _sorted(p):
    o = np.argsort(p["id"], kind="stable")
    return {k: (v[:, o] if v.ndim == 2 else v[o]) for k, v in p.items()}


def _max_rel(a, b):
    scale = max(float(np.abs(b).max()), 1e-30)
    return float(np.abs(a.astype(np.float64) - b).max()) / scale


def _layout(g, cells):
    """(sc, lcell) of global cells [3][n] for the grid's supercell layout."""
    x, y, z = (np.asarray(c, np.int64) for c in cells)
    nsx, nsy = g.nx // g.sx, g.ny // g.sy
    sc = (x // g.sx) + nsx * ((y // g.sy) + nsy * (z // g.sz))
    lc = (x % g.sx) + g.sx * ((y % g.sy) + g.sy * (z % g.sz))
    return sc.astype(np.int32), lc.astype(np.uint16)


def _particles(g, cells, pos, u, mass=1.0, weight=0.01):
    sc, lc = _layout(g, cells)
    n = sc.size
    mom = (np.asarray(u, np.float64) * mass * weight * g.c).astype(F32)
    return dict(pos=np.ascontiguousarray(np.asarray(pos, F32)), mom=np.ascontiguousarray(mom),
                w=np.full(n, weight, F32), sc=sc, lcell=lc, id=np.arange(n, dtype=np.uint32))


def _one_push(orc, g, sp, p, E, B):
    """One push (with the fused deposit) on the GPU and in the oracle; both compared."""
    gd = g.as_dict()
    with pg.Simulation(g) as sim:
        sim.add_species(sp)
        sim.set_particles(sp.name, p)
        sim.set_field("E", E)
        sim.set_field("B", B)
        sim.stage("current_reset")
        sim.stage("push")
        q = _sorted(sim.get_particles(sp.name))
        Jg = sim.get_field("J")
        assert sim.device_status() == 0
    ref = {k: v.copy() for k, v in p.items()}
    orc.push(gd, sp.as_dict(), ref, E, B)
    for k in ("pos", "mom", "w", "sc", "lcell"):
        assert np.array_equal(q[k], ref[k]), k
    Jo = np.zeros_like(E)
    orc.deposit(gd, sp.as_dict(), ref, Jo)
    assert _max_rel(Jg, Jo) <= REL
    return q, ref


@pytest.fixture(scope="module")
def orc():
    import oracle

    oracle.build()
    oracle.set_threads(1)
    return oracle


BOUNDARY_POS = np.array([0.0, np.nextafter(F32(0), F32(1)), 2.0 ** -24, 0.25, np.nextafter(F32(0.5), F32(0)), 0.5,
                         np.nextafter(F32(0.5), F32(1)), 0.75, np.nextafter(F32(1), F32(0))], F32)
# normalised momenta u = gamma v / c: zero, tiny (a displacement far below one ulp of 1), and
# large enough to cross a cell boundary from anywhere near it (|v| dt < 1 cell always)
BOUNDARY_U = np.array([0.0, 1e-7, -1e-7, 1e-3, -1e-3, 0.3, -0.3, 3.0, -3.0])


@pytest.mark.parametrize("current", ["Esirkepov", "EmZ"])
@pytest.mark.parametrize("shape", ["CIC", "TSC", "PQS", "PCS"])
def test_boundary_positions_bit_exact(orc, shape, current):
    g = pg.Grid(32, 32, 32, supercell=(8, 8, 4))
    gd = g.as_dict()
    rng = np.random.default_rng(7 + len(shape) + len(current))
    # cells on supercell faces and at the corners of the box
    cx = np.array([0, 7, 8, 15, 31])
    cz = np.array([0, 3, 4, 7, 31])
    n = 6000
    cells = np.stack([rng.choice(cx, n), rng.choice(cx, n), rng.choice(cz, n)])
    pos = np.stack([rng.choice(BOUNDARY_POS, n) for _ in range(3)])
    u = np.stack([rng.choice(BOUNDARY_U, n) for _ in range(3)])
    p = _particles(g, cells, pos, u)
    E, B = random_field(gd, rng, 0.05), random_field(gd, rng, 0.05)
    sp = pg.Species("e", -1.0, 1.0, shape=shape, current=current, with_ids=True)
    q, ref = _one_push(orc, g, sp, p, E, B)
    assert (q["sc"] != p["sc"]).any() and (q["lcell"] != p["lcell"]).any()


@pytest.mark.parametrize("shape", ["CIC", "TSC", "PQS"])
def test_diagonal_migration_to_all_26_neighbours(orc, shape):
    """Every particle leaves its supercell through a face, an edge or a corner, some through
    the corners of the periodic box; each lands in the neighbour the oracle names."""
    g = pg.Grid(32, 32, 16, supercell=(8, 8, 4))
    gd = g.as_dict()
    rng = np.random.default_rng(26)
    size = (g.sx, g.sy, g.sz)
    dirs = [(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1) if (a, b, c) != (0, 0, 0)]
    scs = [(0, 0, 0), (3, 3, 3), (1, 2, 1), (0, 3, 2)]  # box corners and inner supercells
    cells, pos, u = [], [], []
    for (sx, sy, sz) in scs:
        for d in dirs:
            for _ in range(4):
                c, x, v = [], [], []
                for a in range(3):
                    lo = (sx, sy, sz)[a] * size[a]
                    if d[a] > 0:
                        c.append(lo + size[a] - 1)
                        x.append(rng.uniform(0.7, 0.99))
                        v.append(3.0)
                    elif d[a] < 0:
                        c.append(lo)
                        x.append(rng.uniform(0.01, 0.3))
                        v.append(-3.0)
                    else:
                        c.append(lo + rng.integers(1, size[a] - 1))
                        x.append(rng.uniform(0.3, 0.7))
                        v.append(rng.uniform(-0.01, 0.01))
                cells.append(c)
                pos.append(x)
                u.append(v)
    p = _particles(g, np.array(cells).T, np.array(pos).T, np.array(u).T)
    E, B = random_field(gd, rng, 0.01), random_field(gd, rng, 0.01)
    sp = pg.Species("e", -1.0, 1.0, shape=shape, with_ids=True)
    q, _ = _one_push(orc, g, sp, p, E, B)
    assert (q["sc"] != p["sc"]).all()  # every particle changed supercell
    nsx, nsy, nsz = g.nx // g.sx, g.ny // g.sy, g.nz // g.sz
    moved = np.stack([(q["sc"] % nsx) - (p["sc"] % nsx), (q["sc"] // nsx) % nsy - (p["sc"] // nsx) % nsy,
                      q["sc"] // (nsx * nsy) - p["sc"] // (nsx * nsy)])
    # the supercell step along each axis, with the periodic wrap undone
    for a, n_a in enumerate((nsx, nsy, nsz)):
        moved[a] = (moved[a] + 1) % n_a - 1
    seen = {tuple(m) for m in moved.T}
    assert seen == set(dirs)


def test_empty_and_sparse_species(orc):
    """A full step with an empty species beside one that occupies three supercells."""
    g = pg.Grid(32, 32, 16, supercell=(8, 8, 4))
    gd = g.as_dict()
    rng = np.random.default_rng(3)
    p = random_particles(gd, 2, rng, u_th=0.2, weight=0.01)
    keep = np.isin(p["sc"], [0, 5, 63])
    p = {k: np.ascontiguousarray(v[:, keep] if v.ndim == 2 else v[keep]) for k, v in p.items()}
    p["id"] = np.arange(p["w"].size, dtype=np.uint32)
    empty = {k: np.ascontiguousarray(v[:, :0] if v.ndim == 2 else v[:0]) for k, v in p.items()}
    E, B = random_field(gd, rng, 0.02), random_field(gd, rng, 0.02)
    se = pg.Species("e", -1.0, 1.0, shape="TSC", with_ids=True)
    sn = pg.Species("none", 1.0, 1836.0, shape="TSC", with_ids=True)
    with pg.Simulation(g) as sim:
        sim.add_species(se)
        sim.add_species(sn)
        sim.set_particles("e", p)
        sim.set_particles("none", empty)
        sim.set_field("E", E)
        sim.set_field("B", B)
        sim.step()
        q = _sorted(sim.get_particles("e"))
        qn = sim.get_particles("none")
        Eg, Jg = sim.get_field("E"), sim.get_field("J")
        energies = sim.energies()
        assert sim.device_status() == 0
    J = np.zeros_like(E)
    orc.step(gd, [se.as_dict(), sn.as_dict()], [p, empty], E, B, J)
    assert qn["w"].size == 0
    for k in ("pos", "mom", "sc", "lcell"):
        assert np.array_equal(q[k], p[k]), k
    assert _max_rel(Jg, J) <= REL
    assert _max_rel(Eg, E) <= REL
    assert energies["none"] == 0.0
    ke = orc.kinetic_energy(gd, se.as_dict(), p)
    assert energies["e"] == pytest.approx(ke, rel=1e-6)


def test_overflow_before_separate_deposit(orc):
    """Arrivals that overflow their destination supercell are parked and re-inserted inside the
    push stage, so the separate deposit stage (fuse_deposit off) deposits every particle."""
    g = pg.Grid(32, 32, 16, supercell=(8, 8, 4), fuse_deposit=False)
    gd = g.as_dict()
    rng = np.random.default_rng(64)
    n = 60
    # 60 particles in the last x column of supercell 0 leave along +x into supercell 1, which
    # holds 60 particles of its own; 64 slots per supercell
    movers = [np.full(n, 7), rng.integers(0, 8, n), rng.integers(0, 4, n)]
    stayers = [rng.integers(9, 15, n), rng.integers(1, 7, n), rng.integers(1, 3, n)]
    cells = np.concatenate([np.stack(movers), np.stack(stayers)], axis=1)
    pos = np.concatenate([np.stack([rng.uniform(0.8, 0.99, n), rng.uniform(0.2, 0.8, n), rng.uniform(0.2, 0.8, n)]),
                          rng.uniform(0.2, 0.8, (3, n))], axis=1)
    u = np.concatenate([np.stack([np.full(n, 3.0), np.zeros(n), np.zeros(n)]), np.zeros((3, n))], axis=1)
    p = _particles(g, cells, pos, u)
    E, B = random_field(gd, rng, 0.01), random_field(gd, rng, 0.01)
    sp = pg.Species("e", -1.0, 1.0, shape="TSC", capacity=64, with_ids=True)
    with pg.Simulation(g) as sim:
        sim.add_species(sp)
        sim.set_particles("e", p)
        sim.set_field("E", E)
        sim.set_field("B", B)
        sim.stage("current_reset")
        sim.stage("push")
        sim.stage("deposit")
        q = _sorted(sim.get_particles("e"))
        Jg = sim.get_field("J")
        assert sim.device_status() == 0
    ref = {k: v.copy() for k, v in p.items()}
    orc.push(gd, sp.as_dict(), ref, E, B)
    assert np.bincount(ref["sc"])[1] == 2 * n  # the destination holds more than its 64 slots
    for k in ("pos", "mom", "sc", "lcell"):
        assert np.array_equal(q[k], ref[k]), k
    Jo = np.zeros_like(E)
    orc.deposit(gd, sp.as_dict(), ref, Jo)
    assert _max_rel(Jg, Jo) <= REL
