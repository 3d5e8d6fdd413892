"""The benchmarked configurations under parity: the CUDA path against the CPU oracle
on the distributions the bench measures, started from the device initialiser's own
output (kInitPlasma, downloaded through the C-ABI and handed to the oracle).

* Two-stream slice (the headline workload on 64^3 cells): electrons in two slabs
  along y drifting at +-0.2c along x (u_th 0.005) over protons at the same
  positions, 2 x 16 ppc, TSC, Boris, Esirkepov, Yee, omega_p dt = 0.1.
  - the initialiser: exact counts per cell, uniform in-cell positions, the drift
    of each slab and the thermal spread within sampling error
    (startPosition::Random, particles/startPosition/RandomImpl.hpp; Temperature,
    particles/manipulators/unary/Temperature.hpp:61-108; Drift);
  - one step: positions, momenta, cell and supercell indices and per-cell counts
    bit-exact; J and E within 1e-6 of their maximum; the charge density in
    FieldTmp0 element by element within 1e-5 of max|rho| before and after the step
    (each cell sums about 430 float contributions per species, in another order on
    each side; 1e-5 is also the charge-conservation bar);
  - 100 steps: the four FP64 energies within 1e-4 relative at every 10th step and
    the charge residual <= 1e-5 max|rho_e| on the GPU.
* Laser slice (the laser-wake workload's species and shape): electrons at
  n/n_c = 0.01, 8 ppc, PQS, over immobile protons, in a plane pulse (a0 = 2,
  wavelength 16 cells) set in E and B: one step bit-exact, 20 steps of energies
  within 1e-4.
* Ensemble boxes (the batched workload's distribution): uneven boxes with 4-16 ppc,
  u_th in [0.005, 0.05] and omega_p dt in [0.05, 0.2], CIC and TSC; one batched
  step against the oracle's step of every box.
"""
import math
import os

import numpy as np
import pytest

import picongpu_gb300 as pg

pytestmark = pytest.mark.gpu

DT = float(np.float32(0.99 / np.sqrt(3.0)))
MASS_P = 1836.0
REL = 1e-6
REL_RHO = 1e-5


@pytest.fixture(scope="module")
def orc():
    import oracle

    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    return oracle


def sorted_by_id(p):
    o = np.argsort(p["id"], kind="stable")
    return {k: (v[:, o] if v.ndim == 2 else v[o]) for k, v in p.items()}


def max_rel(a, b):
    scale = max(float(np.abs(b).max()), 1e-30)
    return float(np.abs(a.astype(np.float64) - b).max()) / scale


def counts_per_cell(g, p):
    vol = g.sx * g.sy * g.sz
    nsc = (g.nx // g.sx) * (g.ny // g.sy) * (g.nz // g.sz)
    return np.bincount(p["sc"].astype(np.int64) * vol + p["lcell"].astype(np.int64), minlength=nsc * vol)


def global_cells(g, p):
    nsx, nsy = g.nx // g.sx, g.ny // g.sy
    sc = p["sc"].astype(np.int64)
    lc = p["lcell"].astype(np.int64)
    x = (sc % nsx) * g.sx + lc % g.sx
    y = ((sc // nsx) % nsy) * g.sy + (lc // g.sx) % g.sy
    z = (sc // (nsx * nsy)) * g.sz + lc // (g.sx * g.sy)
    return x, y, z


# ------------------------------------------------------------------ two-stream slice
N2 = 64
PPC2 = 16
U_TH = 0.005
DRIFT = 0.2 / math.sqrt(1.0 - 0.04)  # gamma beta of 0.2c


def density(wpdt=0.1):
    wp = wpdt / DT
    return wp * wp  # q = m = eps0 = 1


def two_stream_sim():
    g = pg.Grid(N2, N2, N2, dt=DT)
    sim = pg.Simulation(g)
    sim.add_species(pg.Species("e", -1.0, 1.0, shape="TSC", with_ids=True))
    sim.add_species(pg.Species("i", 1.0, MASS_P, shape="TSC", with_ids=True))
    n = density()
    # the bench's initialisation of the two-stream workload
    sim.init_plasma("e", PPC2, n, U_TH, drift_lo=(DRIFT, 0, 0), drift_hi=(-DRIFT, 0, 0), split_axis=1,
                    split_cell=N2 // 2, seed=1, position_seed=7)
    sim.init_plasma("i", PPC2, n, U_TH / math.sqrt(MASS_P), seed=2, position_seed=7)
    return g, sim


def test_device_initialiser_statistics():
    g, sim = two_stream_sim()
    with sim:
        pe = sim.get_particles("e")
        pi = sim.get_particles("i")
    ncell = N2 ** 3
    n = density()
    w = np.float32(n / PPC2)
    for p, mass in ((pe, 1.0), (pi, MASS_P)):
        assert p["w"].size == ncell * PPC2
        # exactly ppc particles in every cell, ids unique
        assert np.array_equal(counts_per_cell(g, p), np.full(ncell, PPC2))
        assert np.unique(p["id"]).size == p["id"].size
        assert np.all(p["w"] == w)
        # uniform in-cell positions: [0, 1), mean 1/2 and variance 1/12 within 6 sigma
        pos = p["pos"].astype(np.float64)
        assert pos.min() >= 0.0 and pos.max() < 1.0
        m = pos.size
        assert abs(pos.mean() - 0.5) < 6 * math.sqrt(1 / 12 / m)
        assert abs(pos.var() - 1 / 12) < 6 * math.sqrt(1 / 180 / m)
        # the ten deciles along each axis are equally filled (chi-square, 9 dof, p ~ 1e-6)
        for d in range(3):
            h = np.bincount(np.minimum((pos[d] * 10).astype(int), 9), minlength=10)
            chi2 = float(((h - m / 30) ** 2 / (m / 30)).sum())
            assert chi2 < 45.0, (d, chi2)
    # the species share positions (one position seed): a neutral start
    oe, oi = np.argsort(pe["id"]), np.argsort(pi["id"])
    assert np.array_equal(pe["pos"][:, oe], pi["pos"][:, oi])
    # momenta: u = p / (m w c); slabs along y at +-drift in x, Maxwellian spread u_th
    for p, mass, uth, split in ((pe, 1.0, U_TH, True), (pi, MASS_P, U_TH / math.sqrt(MASS_P), False)):
        u = p["mom"].astype(np.float64) / (mass * float(w))
        _, y, _ = global_cells(g, p)
        groups = [(y < N2 // 2, DRIFT), (y >= N2 // 2, -DRIFT)] if split else [(np.ones_like(y, bool), 0.0)]
        for sel, ux in groups:
            k = int(sel.sum())
            for d, mean in ((0, ux), (1, 0.0), (2, 0.0)):
                ud = u[d][sel]
                assert abs(ud.mean() - mean) < 6 * uth / math.sqrt(k), (d, ud.mean(), mean)
                assert abs(ud.std() / uth - 1.0) < 6 / math.sqrt(2 * k), (d, ud.std(), uth)
            # Gaussian tails: the fraction beyond 2 sigma (two-sided) is 4.55 %
            tail = float((np.abs(u[0][sel] - ux) > 2 * uth).mean())
            assert abs(tail - 0.0455) < 6 * math.sqrt(0.0455 * 0.9545 / k), tail


def oracle_rho(orc, gd, species, parts):
    rho = np.zeros((gd["nz"], gd["ny"], gd["nx"]), np.float32)
    for s, p in zip(species, parts):
        r = np.zeros_like(rho)
        orc.charge_density(gd, s.as_dict(), p, r)
        rho += r
    return rho


def gpu_rho(g, sp, p):
    """FieldTmp0 of a simulation holding one species with particles p (kChargeDensity)."""
    with pg.Simulation(g) as sim:
        sim.add_species(sp)
        sim.set_particles(sp.name, p)
        sim.charge_residual()
        return sim.get_field("FieldTmp0")[0]


def kinetic_energy_f64(p, mass0, c=1.0):
    """KinEnergy (algorithms/KinEnergy.hpp:38-66) per particle in float32, as the kernel
    evaluates it, summed in float64 over all particles."""
    f = np.float32
    m = f(mass0) * p["w"]
    u = p["mom"]
    mom2 = (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]
    c2 = f(c) * f(c)
    gamma = np.sqrt(f(1.0) + mom2 * (f(1.0) / ((m * m) * c2)))
    e = np.where(gamma < f(1.005), mom2 / (f(2.0) * m), ((gamma - f(1.0)) * m) * c2)
    return float(e.astype(np.float64).sum())


def test_two_stream_slice_one_step(orc):
    g, sim = two_stream_sim()
    gd = g.as_dict()
    with sim:
        pe, pi = sim.get_particles("e"), sim.get_particles("i")
        ses = [sim.species[0], sim.species[1]]
        # the kinetic energies are FP64 sums: against a float64 sum of the same float
        # per-particle energies over the 4.2e6 particles of each species
        en = sim.energies()
        for name, p, m0 in (("e", pe, 1.0), ("i", pi, MASS_P)):
            want = kinetic_energy_f64(p, m0)
            assert abs(en[name] - want) <= 1e-12 * want, (name, en[name], want)
        # charge density of the initial state (FieldTmp0) against the oracle's
        sim.charge_residual()
        rho0 = sim.get_field("FieldTmp0")[0]
        sim.step()
        qe, qi = sim.get_particles("e"), sim.get_particles("i")
        Jg, Eg = sim.get_field("J"), sim.get_field("E")
        res, _ = sim.charge_residual()
        rho1 = sim.get_field("FieldTmp0")[0]
    # the protons sit on the electrons: the total density is zero up to rounding, so the
    # total is compared on the scale of the electron density, and each species alone
    # element by element below
    want0 = oracle_rho(orc, gd, ses, [pe, pi])
    rho_e0 = oracle_rho(orc, gd, ses[:1], [pe])
    assert float(np.abs(rho0.astype(np.float64) - want0).max()) <= REL_RHO * float(np.abs(rho_e0).max())
    shp = (3, N2, N2, N2)
    E, B, J = (np.zeros(shp, np.float32) for _ in range(3))
    orc.step(gd, [s.as_dict() for s in ses], [pe, pi], E, B, J, threads=os.cpu_count() or 1)
    for got, want in ((qe, pe), (qi, pi)):
        a, b = sorted_by_id(got), sorted_by_id(want)
        assert np.array_equal(a["id"], b["id"])
        for k in ("pos", "mom", "sc", "lcell"):
            assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(counts_per_cell(g, got), counts_per_cell(g, want))
    assert max_rel(Jg, J) <= REL
    assert max_rel(Eg, E) <= REL
    want1 = oracle_rho(orc, gd, ses, [pe, pi])
    rho_e = oracle_rho(orc, gd, ses[:1], [pe])
    assert float(np.abs(rho1.astype(np.float64) - want1).max()) <= REL_RHO * float(np.abs(rho_e).max())
    for s, got, want in ((ses[0], qe, pe), (ses[1], qi, pi)):
        assert max_rel(gpu_rho(g, s, got), oracle_rho(orc, gd, [s], [want])) <= REL_RHO, s.name
    assert res <= 1e-5 * float(np.abs(rho_e).max())


def test_two_stream_slice_100_steps(orc):
    g, sim = two_stream_sim()
    gd = g.as_dict()
    threads = os.cpu_count() or 1
    with sim:
        pe, pi = sim.get_particles("e"), sim.get_particles("i")
        ses = [s.as_dict() for s in sim.species]
        rho_e = np.zeros((N2, N2, N2), np.float32)
        orc.charge_density(gd, ses[0], pe, rho_e)
        rho_max = float(np.abs(rho_e).max())
        shp = (3, N2, N2, N2)
        E, B, J = (np.zeros(shp, np.float32) for _ in range(3))
        for step in range(1, 101):
            sim.step()
            orc.step(gd, ses, [pe, pi], E, B, J, threads=threads)
            if step % 10 == 0:
                eg = sim.energies()
                fe = orc.field_energy(gd, E, B)
                want = {"E": fe[0], "B": fe[1], "e": orc.kinetic_energy(gd, ses[0], pe),
                        "i": orc.kinetic_energy(gd, ses[1], pi)}
                for k, v in want.items():
                    assert abs(eg[k] - v) <= 1e-4 * abs(v), (step, k, eg[k], v)
                res, _ = sim.charge_residual()
                assert res <= 1e-5 * rho_max, (step, res, rho_max)


# ------------------------------------------------------------------ laser slice
def plane_pulse(g, a0=2.0, lam=16.0, y0=40.0, sigma_y=12.0):
    """A plane pulse travelling +y, polarised along x, on the Yee grid: E_x at
    (i + 1/2, j, k), B_z = -E_x / c at (i + 1/2, j + 1/2, k), Gaussian envelope along y."""
    k = 2 * math.pi / lam
    E0 = a0 * k  # a0 m c omega / e with m = c = e = 1
    E = np.zeros((3, g.nz, g.ny, g.nx), np.float32)
    B = np.zeros_like(E)
    for arr, comp, y_off, sign in ((E, 0, 0.0, 1.0), (B, 2, 0.5, -1.0)):
        y = np.arange(g.ny) + y_off
        f = sign * E0 * np.exp(-((y - y0) ** 2) / (2 * sigma_y ** 2)) * np.sin(k * (y - y0))
        arr[comp] = f.astype(np.float32)[None, :, None]
    return E, B


def test_laser_slice_against_the_oracle(orc):
    lam = 16.0
    omega = 2 * math.pi / lam
    dens = 0.01 * omega * omega
    g = pg.Grid(32, 128, 32, dt=DT)
    gd = g.as_dict()
    E, B = plane_pulse(g)
    se = pg.Species("e", -1.0, 1.0, shape="PQS", with_ids=True)
    si = pg.Species("i", 1.0, MASS_P, pusher=None, shape="PQS", current=None, with_ids=True)
    with pg.Simulation(g) as sim:
        sim.add_species(se)
        sim.add_species(si)
        sim.init_plasma("e", 8, dens, 0.0, seed=21, position_seed=22)
        sim.init_plasma("i", 8, dens, 0.0, seed=23, position_seed=22)
        sim.set_field("E", E)
        sim.set_field("B", B)
        pe, pi = sim.get_particles("e"), sim.get_particles("i")
        sim.step()
        qe = sim.get_particles("e")
        Eg = sim.get_field("E")
        J = np.zeros_like(E)
        orc.step(gd, [se.as_dict(), si.as_dict()], [pe, pi], E, B, J, threads=os.cpu_count() or 1)
        a, b = sorted_by_id(qe), sorted_by_id(pe)
        for k in ("pos", "mom", "sc", "lcell"):
            assert np.array_equal(a[k], b[k]), k
        assert max_rel(Eg, E) <= REL
        for step in range(2, 21):
            sim.step()
            orc.step(gd, [se.as_dict(), si.as_dict()], [pe, pi], E, B, J, threads=os.cpu_count() or 1)
        eg = sim.energies()
        fe = orc.field_energy(gd, E, B)
        ke = orc.kinetic_energy(gd, se.as_dict(), pe)
        for got, want in ((eg["E"], fe[0]), (eg["B"], fe[1]), (eg["e"], ke)):
            assert abs(got - want) <= 1e-4 * abs(want), (got, want)
        # the electrons started cold: the pulse has given them their energy
        assert ke > 0.0


# ------------------------------------------------------------------ ensemble boxes
def test_ensemble_boxes_against_the_oracle(orc):
    """Boxes of the batched workload's distribution, each one stepped by the oracle
    from the device-initialised particles the batched step started from."""
    rng = np.random.default_rng(4)
    edges = (16, 24, 32)
    nbox = 4
    dims = [tuple(int(x) for x in rng.choice(edges, size=3)) for _ in range(nbox)]
    ppc = rng.integers(4, 17, size=nbox)
    u_th = rng.uniform(0.005, 0.05, size=nbox)
    dens = (rng.uniform(0.05, 0.2, size=nbox) / DT) ** 2
    for shape in ("CIC", "TSC"):
        species = [pg.Species("e", -1.0, 1.0, shape=shape, with_ids=True),
                   pg.Species("i", 1.0, MASS_P, shape=shape, with_ids=True)]
        with pg.Ensemble(dims) as ens:
            for sp in species:
                ens.add_species(sp)
            ens.init_plasma("e", [pg.plasma_init(int(ppc[b]), float(dens[b]), float(u_th[b]), seed=1000 + b,
                                                 position_seed=5000 + b) for b in range(nbox)])
            ens.init_plasma("i", [pg.plasma_init(int(ppc[b]), float(dens[b]), float(u_th[b] / math.sqrt(MASS_P)),
                                                 seed=3000 + b, position_seed=5000 + b) for b in range(nbox)])
            before = [[ens.box(b).get_particles(s.name) for s in species] for b in range(nbox)]
            ens.run(1)
            for b, (nx, ny, nz) in enumerate(dims):
                box = ens.box(b)
                gd = pg.Grid(nx, ny, nz, dt=DT).as_dict()
                E, B, J = (np.zeros((3, nz, ny, nx), np.float32) for _ in range(3))
                orc.step(gd, [s.as_dict() for s in species], before[b], E, B, J, threads=os.cpu_count() or 1)
                for s, want in zip(species, before[b]):
                    a, w = sorted_by_id(box.get_particles(s.name)), sorted_by_id(want)
                    for k in ("pos", "mom", "sc", "lcell"):
                        assert np.array_equal(a[k], w[k]), (shape, b, s.name, k)
                assert max_rel(box.get_field("J"), J) <= REL, (shape, b)
                assert max_rel(box.get_field("E"), E) <= REL, (shape, b)
