"""Batched ensemble (one push launch per species over every box, the step as one CUDA
graph) against the single-box path on the same boxes.

Contract:
* after one step from identical particles and random E/B, momenta, positions,
  supercell and cell indices of every box are bit-exact with the single-box
  step (the same per-particle arithmetic); J, E, B agree within 1e-6 of their
  maximum (atomic summation order);
* over 10 steps the FP64 energies of every box agree within 1e-5 relative;
* an overflowing supercell inside a batched step is re-laid out and no
  particle is lost;
* the autotuner times every candidate and returns the fastest;
* the boxes stay periodic and without incident field (the batched field kernels have
  neither): a box's handle refuses open boundaries and an incident pulse.
"""
import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import random_field, random_particles

pytestmark = pytest.mark.gpu

REL = 1e-6
DIMS = [(16, 16, 8), (24, 16, 16), (32, 24, 8), (16, 32, 12)]


def sorted_by_id(p):
    o = np.argsort(p["id"], kind="stable")
    return {k: (v[:, o] if v.ndim == 2 else v[o]) for k, v in p.items()}


def max_rel(a, b):
    scale = max(float(np.abs(b).max()), 1e-30)
    return float(np.abs(a.astype(np.float64) - b).max()) / scale


def species(shape="TSC", ids=True, capacity=0, pusher="Boris", current="Esirkepov"):
    return [pg.Species("e", -1.0, 1.0, pusher=pusher, shape=shape, current=current, with_ids=ids, capacity=capacity),
            pg.Species("i", 1.0, 1836.0, pusher=pusher, shape=shape, current=current, with_ids=ids,
                       capacity=capacity)]


def box_inputs(dims, seed):
    """Per box: electrons, protons on the electrons, random E and B."""
    out = []
    for b, (nx, ny, nz) in enumerate(dims):
        g = pg.Grid(nx, ny, nz)
        gd = g.as_dict()
        rng = np.random.default_rng(seed + b)
        ppc = 2 + b % 3
        pe = random_particles(gd, ppc, rng, u_th=0.05 + 0.02 * b, weight=0.01)
        pi = random_particles(gd, ppc, rng, u_th=0.002, mass=1836.0, weight=0.01)
        pi["pos"] = pe["pos"].copy()
        out.append((pe, pi, random_field(gd, rng, 0.02), random_field(gd, rng, 0.02)))
    return out


def make_ensemble(dims, inputs, shape="TSC", threads=256, fields=True, pusher="Boris", current="Esirkepov"):
    ens = pg.Ensemble(dims, threads=threads)
    for sp in species(shape, pusher=pusher, current=current):
        ens.add_species(sp)
    for b, (pe, pi, E, B) in enumerate(inputs):
        box = ens.box(b)
        box.set_particles("e", pe)
        box.set_particles("i", pi)
        if fields:
            box.set_field("E", E)
            box.set_field("B", B)
    return ens


@pytest.mark.parametrize("threads", [128, 256, 512])
@pytest.mark.parametrize("shape", ["CIC", "TSC"])
def test_batched_step_matches_single_box_step(shape, threads):
    inputs = box_inputs(DIMS, 11)
    with make_ensemble(DIMS, inputs, shape, threads) as a, make_ensemble(DIMS, inputs, shape) as b:
        a.run(1)
        b.run_sequential(1)
        assert a.launch_count() == 8  # J reset, 2 pushes, 2 compactions, 3 Yee
        for i in range(len(DIMS)):
            ba, bb = a.box(i), b.box(i)
            for name in ("e", "i"):
                qa, qb = sorted_by_id(ba.get_particles(name)), sorted_by_id(bb.get_particles(name))
                for k in ("pos", "mom", "w", "sc", "lcell", "id"):
                    assert np.array_equal(qa[k], qb[k]), (i, name, k)
            for f in ("J", "E", "B"):
                assert max_rel(ba.get_field(f), bb.get_field(f)) <= REL, (i, f)


def test_batched_energies_follow_single_box_path():
    """Quasi-neutral start with E = B = 0, so eps0 div E - rho starts (and stays) at zero."""
    inputs = box_inputs(DIMS, 23)
    with make_ensemble(DIMS, inputs, fields=False) as a, make_ensemble(DIMS, inputs, fields=False) as b:
        a.run(10)
        b.run_sequential(10)
        for i in range(len(DIMS)):
            ea, eb = a.box(i).energies(), b.box(i).energies()
            for k in ("E", "B", "e", "i"):
                assert abs(ea[k] - eb[k]) <= 1e-5 * abs(eb[k]), (i, k, ea[k], eb[k])
            res, rho = a.box(i).charge_residual()
            assert res <= 1e-5 * rho


def test_batched_overflow_is_relaid_out():
    """Slots per supercell exactly the initial count: every net arrival overflows."""
    dims = [(16, 16, 8), (24, 24, 8)]
    with pg.Ensemble(dims) as ens:
        ens.add_species(pg.Species("e", -1.0, 1.0, shape="TSC", capacity=4 * 256))
        inits = [pg.plasma_init(4, 0.05, 0.3, drift_lo=(0.4, 0.0, 0.0), seed=3 + b) for b in range(len(dims))]
        ens.init_plasma("e", inits)
        n0 = ens.particle_count()
        ens.run(4)
        assert ens.particle_count() == n0
        for i in range(len(dims)):
            assert ens.box(i).device_status() == 0


def test_autotune_times_every_candidate():
    dims = [(16, 16, 16), (24, 16, 32), (32, 32, 16)]
    sp = species(ids=False)
    inits = [[pg.plasma_init(4, 0.03, 0.02, seed=s * 10 + b, position_seed=b) for b in range(len(dims))]
             for s in range(len(sp))]
    sc, th, rates = pg.autotune(dims, sp, inits, warmup=1, steps=2)
    assert len(rates) == 9 and all(r > 0 for r in rates.values()), rates
    assert rates[(sc, th)] == max(rates.values())


@pytest.mark.parametrize("shape,pusher,current", [("PCS", "Boris", "Esirkepov"), ("TSC", "Boris", "EmZ"),
                                                   ("PQS", "HigueraCary", "EmZ"), ("PCS", "Vay", "EmZ")])
def test_batched_pcs_and_emz_match_single_box(shape, pusher, current):
    """The PCS and EmZ variants of the batched push (the Thermal benchmark's policies) against the
    single-box path: particles bit-exact, J, E, B within 1e-6."""
    inputs = box_inputs(DIMS[:2], 29)
    with make_ensemble(DIMS[:2], inputs, shape, 512, pusher=pusher, current=current) as a, \
            make_ensemble(DIMS[:2], inputs, shape, pusher=pusher, current=current) as b:
        a.run(1)
        b.run_sequential(1)
        for i in range(2):
            ba, bb = a.box(i), b.box(i)
            for name in ("e", "i"):
                pa, pb = sorted_by_id(ba.get_particles(name)), sorted_by_id(bb.get_particles(name))
                for k in ("pos", "mom", "sc", "lcell"):
                    assert np.array_equal(pa[k], pb[k]), (shape, current, i, name, k)
            for f in ("J", "E", "B"):
                assert max_rel(ba.get_field(f), bb.get_field(f)) <= REL, (shape, current, i, f)


@pytest.mark.parametrize("pusher", ["HigueraCary", "Vay"])
def test_batched_higuera_cary_and_vay_match_single_box(pusher):
    """The batched push's HigueraCary/Vay kernel variant against the single-box path."""
    inputs = box_inputs(DIMS[:2], 23)
    with make_ensemble(DIMS[:2], inputs, "PQS", 512, pusher=pusher) as a, \
            make_ensemble(DIMS[:2], inputs, "PQS", pusher=pusher) as b:
        a.run(1)
        b.run_sequential(1)
        for i in range(2):
            for name in ("e", "i"):
                pa, pb = sorted_by_id(a.box(i).get_particles(name)), sorted_by_id(b.box(i).get_particles(name))
                for k in ("pos", "mom", "sc", "lcell"):
                    assert np.array_equal(pa[k], pb[k]), (pusher, i, name, k)


def test_ensemble_boxes_refuse_open_boundaries_and_incident_fields():
    dims = [(16, 32, 16), (16, 32, 16)]
    pulse = dict(a0=1.0, wavelength=16.0, waist=4.0, duration_fwhm=5.0, t_center=10.0, axis=1, surface=8)
    with pg.Ensemble(dims) as ens:
        ens.add_species(pg.Species("e", -1.0, 1.0, shape="TSC"))
        ens.init_plasma("e", [pg.plasma_init(2, 0.02, 0.01, seed=b) for b in range(len(dims))])
        with pytest.raises(pg.PicError):
            ens.box(1).set_boundaries(open_axes=(False, True, False), thickness=((0, 0), (4, 4), (0, 0)))
        with pytest.raises(pg.PicError):
            ens.box(1).set_incident_field(**pulse)
        ens.box(1).clear_incident_field()
        ens.box(1).clear_incident_field(axis=1)
        ens.run(1)
