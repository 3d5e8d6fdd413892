"""Differentiable run: hand-written adjoint against FP64 central finite differences.

Case: 16^3 periodic cells, TSC, electrons and protons (1 ppc each, u_th = 0.02),
a Gaussian pulse (a0 = 1, waist 4, wavelength 8) in E/B, 8 steps with
checkpoints every 3 steps; loss = electron kinetic energy after the run.
Contract:
* FP64 adjoint gradients with respect to a0, the waist and single initial
  momenta agree with FP64 central differences (h = 1e-4 relative) within 1e-4;
* the FP32 adjoint agrees with the FP64 one within 1e-3;
* the checkpoint interval does not change the gradient (1e-9, FP64);
* one forward step agrees with the single-box step on the same particles
  (positions and momenta within 1e-5 of their scale).
"""
import math

import numpy as np
import pytest

import picongpu_gb300 as pg
from picongpu_gb300 import adjoint as A

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

N = 16
STEPS = 8
DT = 0.99 / math.sqrt(3.0)
DENSITY = (0.1 / DT) ** 2


def make(precision, K=3, ppc=1):
    n = N ** 3 * ppc
    sp = [A.DiffSpecies("e", -1.0, 1.0, n), A.DiffSpecies("i", 1.0, 1836.0, n)]
    pic = A.DiffPIC(N, N, N, sp, dt=DT, shape="TSC", precision=precision, checkpoint_every=K)
    e = A.thermal_species(pic, 0, ppc, DENSITY, 0.02, seed=3)
    i = A.thermal_species(pic, 1, ppc, DENSITY, 0.02 / math.sqrt(1836.0), seed=4, position_seed=3)
    return pic, [e, i]


def loss_of(pic, parts, a0, waist, steps=STEPS):
    E, B = A.gaussian_pulse(pic, a0, waist, 8.0, 4.0, (8.0, 8.0, 8.0))
    E1, B1, out = A.run(pic, steps, E, B, parts)
    return A.kinetic_energy(out[0]["mom"], parts[0]["w"], 1.0)


def gradients(pic, parts, a0=1.0, waist=4.0):
    a = torch.tensor(a0, dtype=pic.dtype, device="cuda", requires_grad=True)
    w = torch.tensor(waist, dtype=pic.dtype, device="cuda", requires_grad=True)
    mom = parts[0]["mom"].clone().requires_grad_(True)
    p = [dict(parts[0], mom=mom), parts[1]]
    L = loss_of(pic, p, a, w)
    L.backward()
    return float(L.detach()), float(a.grad), float(w.grad), mom.grad.detach().clone()


def value(pic, parts, a0=1.0, waist=4.0):
    with torch.no_grad():
        a = torch.tensor(a0, dtype=pic.dtype, device="cuda")
        w = torch.tensor(waist, dtype=pic.dtype, device="cuda")
        return float(loss_of(pic, parts, a, w))


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def test_fp64_adjoint_matches_central_differences():
    pic, parts = make(8)
    L, ga, gw, gmom = gradients(pic, parts)
    assert L > 0
    h = 1e-4
    fa = (value(pic, parts, 1.0 + h) - value(pic, parts, 1.0 - h)) / (2 * h)
    fw = (value(pic, parts, 1.0, 4.0 * (1 + h)) - value(pic, parts, 1.0, 4.0 * (1 - h))) / (2 * 4.0 * h)
    assert rel(ga, fa) <= 1e-4, (ga, fa)
    assert rel(gw, fw) <= 1e-4, (gw, fw)
    # single initial momenta of the electrons with the largest gradients
    idx = torch.topk(gmom.abs().flatten(), 3).indices.tolist()
    for flat in idx:
        d, p = divmod(flat, gmom.shape[1])
        m0 = float(parts[0]["mom"][d, p])
        hp = 1e-4 * abs(m0)
        vals = []
        for s in (+1, -1):
            mom = parts[0]["mom"].clone()
            mom[d, p] = m0 + s * hp
            vals.append(value(pic, [dict(parts[0], mom=mom), parts[1]]))
        fd = (vals[0] - vals[1]) / (2 * hp)
        assert rel(float(gmom[d, p]), fd) <= 1e-4, (d, p, float(gmom[d, p]), fd)
    pic.close()


def test_fp32_adjoint_follows_fp64():
    p64, parts64 = make(8)
    p32, parts32 = make(4)
    _, ga64, gw64, _ = gradients(p64, parts64)
    _, ga32, gw32, _ = gradients(p32, parts32)
    assert rel(ga32, ga64) <= 1e-3, (ga32, ga64)
    assert rel(gw32, gw64) <= 1e-3, (gw32, gw64)


@pytest.mark.parametrize("K", [1, 8])
def test_checkpoint_interval_does_not_change_the_gradient(K):
    p3, parts3 = make(8, K=3)
    pk, partsk = make(8, K=K)
    _, ga3, gw3, gm3 = gradients(p3, parts3)
    _, gak, gwk, gmk = gradients(pk, partsk)
    assert rel(gak, ga3) <= 1e-9 and rel(gwk, gw3) <= 1e-9
    assert float((gmk - gm3).abs().max()) <= 1e-9 * float(gm3.abs().max())


def test_backward_needs_the_latest_forward():
    pic, parts = make(4)
    a = torch.tensor(1.0, device="cuda", requires_grad=True)
    L1 = loss_of(pic, parts, a, torch.tensor(4.0, device="cuda"), steps=2)
    loss_of(pic, parts, a, torch.tensor(4.0, device="cuda"), steps=2)
    with pytest.raises(RuntimeError):
        L1.backward()


def test_forward_step_matches_single_box_step():
    pic, parts = make(4, ppc=2)
    a0 = torch.tensor(1.0, device="cuda")
    E, B = A.gaussian_pulse(pic, a0, torch.tensor(4.0, device="cuda"), 8.0, 4.0, (8.0, 8.0, 8.0))
    with torch.no_grad():
        E1, B1, out = A.run(pic, 1, E, B, parts)
    g = pg.Grid(N, N, N, dt=float(np.float32(DT)))
    with pg.Simulation(g) as sim:
        for k, (name, mass) in enumerate((("e", 1.0), ("i", 1836.0))):
            sim.add_species(pg.Species(name, -1.0 if k == 0 else 1.0, mass, shape="TSC", with_ids=True))
        for k, name in enumerate(("e", "i")):
            c = parts[k]["cell"].cpu().numpy().astype(np.int64)
            sc = (c[0] // 8) + (N // 8) * ((c[1] // 8) + (N // 8) * (c[2] // 4))
            lc = (c[0] % 8) + 8 * ((c[1] % 8) + 8 * (c[2] % 4))
            n = c.shape[1]
            sim.set_particles(name, dict(pos=parts[k]["pos"].cpu().numpy(), mom=parts[k]["mom"].cpu().numpy(),
                                         w=parts[k]["w"].cpu().numpy(), sc=sc.astype(np.int32),
                                         lcell=lc.astype(np.uint16), id=np.arange(n, dtype=np.uint32)))
        sim.set_field("E", E.cpu().numpy())
        sim.set_field("B", B.cpu().numpy())
        sim.step()
        for k, name in enumerate(("e", "i")):
            q = sim.get_particles(name)
            o = np.argsort(q["id"])
            mom = q["mom"][:, o]
            ref = out[k]["mom"].cpu().numpy()
            assert np.abs(mom - ref).max() <= 1e-5 * np.abs(ref).max()
            gx = (q["sc"][o] % (N // 8)) * 8 + q["lcell"][o] % 8
            pos_ref = out[k]["pos"].cpu().numpy()
            cx = out[k]["cell"].cpu().numpy()[0]
            assert np.array_equal(gx, cx)
            assert np.abs(q["pos"][:, o] - pos_ref).max() <= 1e-5
        Eg = sim.get_field("E")
    assert np.abs(Eg - E1.cpu().numpy()).max() <= 1e-5 * np.abs(Eg).max()
