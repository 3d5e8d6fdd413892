"""Open boundaries on the GPU (the reference's non-periodic axes with fields/absorber): the
PML Yee updates are bit-exact with the oracle, a plane pulse is absorbed, and particles that
leave through an open face are absorbed while the others push and deposit as in the oracle."""
import numpy as np
import pytest

import picongpu_gb300 as pg
from plasma import random_field, random_particles

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def orc():
    import oracle

    oracle.build()
    oracle.set_threads(1)
    return oracle


def _by_id(p):
    o = np.argsort(p["id"], kind="stable")
    return {k: (v[:, o] if v.ndim == 2 else v[o]) for k, v in p.items()}


def test_pml_updates_match_oracle(orc):
    g = pg.Grid(24, 40, 16)
    gd = g.as_dict()
    gd["open"] = 3  # x and y open, z periodic
    cells = ((4, 0), (6, 6), (0, 0))
    sigma, kappa, alpha = (3.0, 4.0, 0.0), (1.5, 2.0, 1.0), (0.1, 0.2, 0.0)
    rng = np.random.default_rng(21)
    E, B = random_field(gd, rng, 0.1), random_field(gd, rng, 0.1)
    with pg.Simulation(g) as sim:
        sim.set_boundaries(open_axes=(True, True, False), thickness=cells, sigma_max=sigma, kappa_max=kappa,
                           alpha_max=alpha, grading_order=3.0, alpha_grading_order=1.0)
        sim.set_field("E", E)
        sim.set_field("B", B)
        for _ in range(5):
            sim.stage("current_reset")
            sim.stage("field_before")
            sim.stage("field_after")
        Eg, Bg = sim.get_field("E"), sim.get_field("B")
    p = orc.pml(cells, sigma, kappa, alpha, order=3.0, alpha_order=1.0)
    psiE = np.zeros((6,) + E.shape[1:], np.float32)
    psiB = np.zeros_like(psiE)
    for _ in range(5):
        orc.yee_b_half_open(gd, p, E, B, psiB, update=False)
        orc.yee_e_open(gd, p, B, E, psiE)
        orc.yee_b_half_open(gd, p, E, B, psiB, update=True)
    assert np.array_equal(Eg, E) and np.array_equal(Bg, B)


def test_pml_absorbs_a_plane_pulse():
    """The pulse of the oracle test, with the default sigma (0.8 (m + 1) c / dy, m = 4)."""
    import sys, os

    sys.path.insert(0, os.path.dirname(__file__))
    from test_oracle_pml import _energy, _interior, _pulse

    g = pg.Grid(8, 96, 8)
    E, B = _pulse(g.as_dict())
    e0 = _energy(E, B)
    with pg.Simulation(g) as sim:
        sim.set_boundaries(open_axes=(False, True, False), thickness=((0, 0), (12, 12), (0, 0)))
        sim.set_field("E", E)
        sim.set_field("B", B)
        sim.run(200)
        Eg, Bg = sim.get_field("E"), sim.get_field("B")
    assert _interior(Eg, Bg, 12, 84) < 1e-7 * e0


def test_particles_absorbed_at_open_faces_and_the_rest_match_oracle(orc):
    """Hot electrons (u_th 0.3) in a box open along x: particles crossing x = 0 or x = nx are
    removed; positions, momenta and cells of the others match the oracle, and so does J away
    from the open faces.  (The GPU deposits a leaving particle's current before removing it,
    the oracle drops that particle; the difference stays within the shape's reach of the face,
    inside the PML.)"""
    g = pg.Grid(32, 16, 16)
    gd = g.as_dict()
    gd["open"] = 1
    rng = np.random.default_rng(8)
    p = random_particles(gd, 4, rng, u_th=0.3, weight=0.01)
    E, B = random_field(gd, rng, 0.05), random_field(gd, rng, 0.05)
    sp = pg.Species("e", -1.0, 1.0, shape="TSC", with_ids=True)
    with pg.Simulation(g) as sim:
        sim.set_boundaries(open_axes=(True, False, False), thickness=((4, 4), (0, 0), (0, 0)))
        sim.add_species(sp)
        sim.set_particles("e", p)
        sim.set_field("E", E)
        sim.set_field("B", B)
        sim.stage("current_reset")
        sim.stage("push")
        assert sim.device_status() == 0
        q = _by_id(sim.get_particles("e"))
        Jg = sim.get_field("J")
    ref = {k: v.copy() for k, v in p.items()}
    orc.push(gd, sp.as_dict(), ref, E, B)
    Jo = np.zeros_like(E)
    orc.deposit(gd, sp.as_dict(), ref, Jo)
    kept = ref["sc"] >= 0
    assert 0 < (~kept).sum() < kept.sum()  # some, not all, left through the open faces
    r = {k: v[..., kept] for k, v in ref.items()}
    for k in ("id", "pos", "mom", "sc", "lcell"):
        assert np.array_equal(q[k], r[k]), k
    inner = (slice(None), slice(None), slice(None), slice(4, 28))
    assert np.abs(Jg[inner] - Jo[inner]).max() <= 1e-6 * np.abs(Jo).max()


def test_ensemble_boxes_stay_periodic():
    ens = pg.Ensemble([(16, 16, 16)])
    with pytest.raises(pg.PicError) as e:
        ens.box(0).set_boundaries(open_axes=(True, False, False), thickness=((4, 4), (0, 0), (0, 0)))
    assert e.value.code == pg._lib.ERR_UNSUPPORTED
    ens.close()


def _exp_damp(n, thick, strength):
    """Damping factors of one axis (Exponential.kernel:50-90) rounded from double to float."""
    d = np.ones(n)
    i = np.arange(n)
    f_neg = thick[0] - 1 - i
    d = np.where(f_neg > 0, d * np.exp(-float(np.float32(strength[0])) * f_neg), d)
    f_pos = i - n + thick[1]
    d = np.where(f_pos > 0, d * np.exp(-float(np.float32(strength[1])) * f_pos), d)
    return d.astype(np.float32)


def test_exponential_absorber_matches_restatement(orc):
    """fields/absorber/exponential: the plain open-face Yee updates, then E and B multiplied by
    exp(-strength f) in the layers, factor by factor in x, y, z order (bit-exact)."""
    g = pg.Grid(24, 32, 16)
    gd = g.as_dict()
    gd["open"] = 3
    thick, strength = ((5, 3), (6, 6), (0, 0)), ((0.1, 0.2), (0.05, 0.3), (0.0, 0.0))
    rng = np.random.default_rng(5)
    E, B = random_field(gd, rng, 0.1), random_field(gd, rng, 0.1)
    with pg.Simulation(g) as sim:
        sim.set_boundaries(open_axes=(True, True, False), thickness=thick, absorber="Exponential", strength=strength)
        sim.set_field("E", E)
        sim.set_field("B", B)
        for _ in range(4):
            sim.stage("current_reset")
            sim.stage("field_before")
            sim.stage("field_after")
        Eg, Bg = sim.get_field("E"), sim.get_field("B")
    p = orc.pml(((0, 0),) * 3, [0.0] * 3, [1.0] * 3, [0.0] * 3)
    psi = np.zeros((6,) + E.shape[1:], np.float32)
    dx, dy = _exp_damp(24, thick[0], strength[0]), _exp_damp(32, thick[1], strength[1])

    def damp(F):
        for c in range(3):
            v = F[c]
            m = dx != 1.0
            v[:, :, m] = v[:, :, m] * dx[m][None, None, :]
            m = dy != 1.0
            v[:, m, :] = v[:, m, :] * dy[m][None, :, None]

    for _ in range(4):
        orc.yee_b_half_open(gd, p, E, B, psi, update=False)
        orc.yee_e_open(gd, p, B, E, psi)
        damp(E)
        orc.yee_b_half_open(gd, p, E, B, psi, update=True)
        damp(B)
    assert np.array_equal(Eg, E) and np.array_equal(Bg, B)


def test_invalid_boundaries_are_rejected():
    with pg.Simulation(pg.Grid(16, 16, 8)) as sim:
        with pytest.raises(pg.PicError) as e:  # layers thicker than the axis
            sim.set_boundaries(open_axes=(True, False, False), thickness=((10, 10), (0, 0), (0, 0)))
        assert e.value.code == pg._lib.ERR_INVALID
        with pytest.raises(pg.PicError) as e:
            sim.set_boundaries(open_axes=(True, False, False), thickness=((4, 4), (0, 0), (0, 0)),
                               absorber="Exponential", strength=((-1.0, 0.1), (0, 0), (0, 0)))
        assert e.value.code == pg._lib.ERR_INVALID
        with pytest.raises(pg.PicError) as e:
            sim.set_boundaries(open_axes=(True, False, False), thickness=((4, 4), (0, 0), (0, 0)), kappa_max=(0.5, 1, 1))
        assert e.value.code == pg._lib.ERR_INVALID
        with pytest.raises(ValueError):
            sim.set_boundaries(open_axes=(True, False, False), absorber="Mur")
        sim.set_boundaries()  # all periodic again
        sim.run(1)
        assert sim.device_status() == 0
