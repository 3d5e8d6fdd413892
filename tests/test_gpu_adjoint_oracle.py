"""The GPU adjoint against an independent FP64 reference gradient from the CPU oracle.

Case: 16^3 periodic cells, TSC, electrons and protons (1 ppc each, u_th = 0.02), a
Gaussian pulse (a0 = 1, waist 4, wavelength 8) in E/B, 8 steps; loss = electron kinetic
energy after the run, sum of u^2 / (sqrt(1 + u^2) + 1) m w c^2.  The reference gradient is
taken by FP64 central differences (h = 1e-4 relative) through the oracle's double
instantiation of the PIC step (oracle.step_f64: the reference's gather, Boris push,
moveParticle, Esirkepov deposit and Yee update, every float_X operation in double), from
the same initial particles and fields; it shares no code with the GPU's adjoint kernels.
The GPU FP64 adjoint (transposed curls, Jacobian-transposed Boris, gather and deposit as
each other's transposes, checkpoint replay) must agree within 1e-4 relative for dL/da0,
dL/dwaist and the initial momenta with the largest gradients.
"""
import math
import os

import numpy as np
import pytest

from picongpu_gb300 import adjoint as A

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

N = 16
STEPS = 8
DT = float(np.float32(0.99 / math.sqrt(3.0)))  # one value for the float grid of the oracle and the GPU
DENSITY = (0.1 / DT) ** 2
MASS_P = 1836.0
H = 1e-4


@pytest.fixture(scope="module")
def orc():
    import oracle

    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    return oracle


def make():
    n = N ** 3
    sp = [A.DiffSpecies("e", -1.0, 1.0, n), A.DiffSpecies("i", 1.0, MASS_P, n)]
    pic = A.DiffPIC(N, N, N, sp, dt=DT, shape="TSC", precision=8, checkpoint_every=3)
    e = A.thermal_species(pic, 0, 1, DENSITY, 0.02, seed=3)
    i = A.thermal_species(pic, 1, 1, DENSITY, 0.02 / math.sqrt(MASS_P), seed=4, position_seed=3)
    return pic, [e, i]


def pulse(pic, a0, waist):
    return A.gaussian_pulse(pic, torch.tensor(a0, dtype=torch.float64, device="cuda"),
                            torch.tensor(waist, dtype=torch.float64, device="cuda"), 8.0, 4.0, (8.0, 8.0, 8.0))


def to_oracle(parts):
    """Initial particles of the differentiable run in the oracle's exchange format (float64)."""
    out = []
    for p in parts:
        c = p["cell"].cpu().numpy().astype(np.int64)
        sc = (c[0] // 8) + (N // 8) * ((c[1] // 8) + (N // 8) * (c[2] // 4))
        lc = (c[0] % 8) + 8 * ((c[1] % 8) + 8 * (c[2] % 4))
        out.append(dict(pos=np.ascontiguousarray(p["pos"].cpu().numpy()),
                        mom=np.ascontiguousarray(p["mom"].cpu().numpy()),
                        w=np.ascontiguousarray(p["w"].cpu().numpy()), sc=sc.astype(np.int32),
                        lcell=lc.astype(np.uint16)))
    return out


def oracle_loss(orc, parts, E, B):
    gd = dict(nx=N, ny=N, nz=N, sx=8, sy=8, sz=4, dx=1.0, dy=1.0, dz=1.0, dt=DT, c=1.0, eps0=1.0)
    species = [dict(charge=-1.0, mass=1.0, shape=2, pusher=0, current=1),
               dict(charge=1.0, mass=MASS_P, shape=2, pusher=0, current=1)]
    ps = [{k: v.copy() for k, v in p.items()} for p in parts]
    E, B = E.copy(), B.copy()
    J = np.zeros_like(E)
    for _ in range(STEPS):
        orc.step_f64(gd, species, ps, E, B, J, threads=os.cpu_count() or 1)
    mw = 1.0 * ps[0]["w"]
    u2 = (ps[0]["mom"] ** 2).sum(0) / (mw * mw)
    return float((u2 / (np.sqrt(1.0 + u2) + 1.0) * mw).sum())


def test_adjoint_matches_the_oracle_fp64_gradient(orc):
    pic, parts = make()
    a = torch.tensor(1.0, dtype=torch.float64, device="cuda", requires_grad=True)
    w = torch.tensor(4.0, dtype=torch.float64, device="cuda", requires_grad=True)
    mom = parts[0]["mom"].clone().requires_grad_(True)
    E, B = A.gaussian_pulse(pic, a, w, 8.0, 4.0, (8.0, 8.0, 8.0))
    _, _, out = A.run(pic, STEPS, E, B, [dict(parts[0], mom=mom), parts[1]])
    L = A.kinetic_energy(out[0]["mom"], parts[0]["w"], 1.0)
    L.backward()
    ga, gw, gmom = float(a.grad), float(w.grad), mom.grad.detach().cpu().numpy()
    base = to_oracle(parts)

    def fields(a0, waist):
        with torch.no_grad():
            Ef, Bf = pulse(pic, a0, waist)
        return np.ascontiguousarray(Ef.cpu().numpy()), np.ascontiguousarray(Bf.cpu().numpy())

    E0, B0 = fields(1.0, 4.0)
    L0 = oracle_loss(orc, base, E0, B0)
    assert abs(float(L.detach()) - L0) <= 1e-7 * L0, (float(L.detach()), L0)  # the forward runs agree
    # dL/da0: the fields are linear in a0
    fa = (oracle_loss(orc, base, E0 * (1 + H), B0 * (1 + H)) - oracle_loss(orc, base, E0 * (1 - H), B0 * (1 - H))) \
        / (2 * H)
    Ep, Bp = fields(1.0, 4.0 * (1 + H))
    Em, Bm = fields(1.0, 4.0 * (1 - H))
    fw = (oracle_loss(orc, base, Ep, Bp) - oracle_loss(orc, base, Em, Bm)) / (2 * 4.0 * H)
    assert abs(ga - fa) <= 1e-4 * abs(fa), (ga, fa)
    assert abs(gw - fw) <= 1e-4 * abs(fw), (gw, fw)
    # initial momenta of the electrons with the largest gradients
    for flat in np.argsort(np.abs(gmom).ravel())[-4:]:
        d, p = divmod(int(flat), gmom.shape[1])
        m0 = float(base[0]["mom"][d, p])
        hp = H * abs(m0)
        vals = []
        for s in (+1, -1):
            ps = [dict(base[0], mom=base[0]["mom"].copy()), base[1]]
            ps[0]["mom"][d, p] = m0 + s * hp
            vals.append(oracle_loss(orc, ps, E0, B0))
        fd = (vals[0] - vals[1]) / (2 * hp)
        assert abs(gmom[d, p] - fd) <= 1e-4 * abs(fd), (d, p, gmom[d, p], fd)
    pic.close()
