"""Analytic invariants of the oracle: gyration of the Boris, HigueraCary and Vay
pushers (share/picongpu/tests/Pusher), their phase-lag order
(share/picongpu/tests/PusherScaling), the E x B drift that HigueraCary and Vay keep,
discrete charge continuity of the Esirkepov deposit, and the Yee update against an
independent numpy restatement."""
import numpy as np
import pytest

from plasma import grid, random_particles, random_field, global_cells


def _fit_circle(x, y):
    A = np.stack([x, y, np.ones_like(x)], axis=1)
    b = x * x + y * y
    s = np.linalg.lstsq(A, b, rcond=None)[0]
    return s[0] / 2, s[1] / 2


PUSHERS = {"Boris": 0, "HigueraCary": 3, "Vay": 4}


@pytest.mark.parametrize("pusher", list(PUSHERS))
def test_gyration(orc, pusher):
    """Electron at 0.5c in uniform B_z, 50 steps per turn (Pusher/README.rst, MainTest.py:177,212):
    radius change per turn < 1e-5 (momentum) and < 5e-5 (position), phase change < 0.16 rad."""
    g = grid(n=(16, 16, 16), sc=(8, 8, 4), dt=0.5)
    gamma = 1.0 / np.sqrt(1 - 0.25)
    u = gamma * 0.5
    B0 = 2 * np.pi * gamma / (50 * g["dt"])  # |q| = m = c = 1: period = 50 dt
    E = np.zeros((3, 16, 16, 16), np.float32)
    B = np.zeros_like(E)
    B[2] = np.float32(B0)
    p = dict(pos=np.full((3, 1), 0.5, np.float32), mom=np.array([[u], [0], [0]], np.float32),
             w=np.ones(1, np.float32), sc=np.array([1 + 2 * (1 + 2 * 2)], np.int32),
             lcell=np.array([0], np.uint16))
    sp = dict(charge=-1.0, mass=1.0, shape=2, pusher=PUSHERS[pusher], current=1)
    xs, ys, rp = [], [], []
    last = None
    off = np.zeros(2)
    for k in range(500):
        orc.push(g, sp, p, E, B)
        cell = global_cells(g, p)[:, 0]
        xy = np.array([cell[0] + p["pos"][0, 0], cell[1] + p["pos"][1, 0]], np.float64)
        if last is not None:
            jump = xy + off - last
            off -= 16 * np.round(jump / 16)
        last = xy + off
        xs.append(last[0])
        ys.append(last[1])
        rp.append(np.hypot(p["mom"][0, 0], p["mom"][1, 0]) / B0)
    xs, ys, rp = map(np.asarray, (xs, ys, rp))
    cx, cy = _fit_circle(xs[:50], ys[:50])
    r = np.hypot(xs - cx, ys - cy)
    ph = np.unwrap(np.arctan2(ys - cy, xs - cx))
    for t in range(1, 9):
        i0, i1 = 50 * t, 50 * (t + 1)
        assert abs(rp[i1] - rp[i0]) / rp[i0] < 1e-5
        assert abs(r[i1] - r[i0]) / r[i0] < 5e-5
        assert abs((ph[i1] - ph[i0]) % (2 * np.pi)) < 0.16 or abs((ph[i1] - ph[i0]) % (2 * np.pi) - 2 * np.pi) < 0.16
    assert abs(r.mean() - u / B0) / (u / B0) < 0.02  # radius p/(qB)


def _single(g, mom, pusher):
    p = dict(pos=np.full((3, 1), 0.5, np.float32), mom=np.array(mom, np.float32).reshape(3, 1),
             w=np.ones(1, np.float32), sc=np.array([0], np.int32), lcell=np.array([0], np.uint16))
    return p, dict(charge=-1.0, mass=1.0, shape=2, pusher=PUSHERS[pusher], current=1)


def _phase_lag(orc, pusher, steps_per_turn, turns=4):
    """|phase of the momentum after `turns` nominal periods - turns * 2 pi| (gyration at 0.5c)."""
    g = grid(n=(16, 16, 16), sc=(8, 8, 4), dt=0.5)
    gamma = 1.0 / np.sqrt(1 - 0.25)
    B0 = 2 * np.pi * gamma / (steps_per_turn * g["dt"])
    E = np.zeros((3, 16, 16, 16), np.float32)
    B = np.zeros_like(E)
    B[2] = np.float32(B0)
    p, sp = _single(g, [gamma * 0.5, 0, 0], pusher)
    ang = [0.0]
    for _ in range(steps_per_turn * turns):
        orc.push(g, sp, p, E, B)
        ang.append(np.arctan2(p["mom"][1, 0], p["mom"][0, 0]))
    return abs(abs(np.unwrap(np.array(ang))[-1]) - 2 * np.pi * turns)


@pytest.mark.parametrize("pusher", list(PUSHERS))
def test_phase_lag_is_second_order(orc, pusher):
    """PusherScaling/README.rst: with 10, 20, 40, 80 and 160 steps per turn the phase lag falls
    by 2^x per halving of dt with x within 0.1 of 2 and a standard deviation of x below 0.05."""
    lags = np.array([_phase_lag(orc, pusher, n) for n in (10, 20, 40, 80, 160)])
    x = np.log2(lags[:-1] / lags[1:])
    assert abs(x.mean() - 2.0) < 0.1, x
    assert x.std() < 0.05, x


def test_exb_drift_kept_by_higuera_cary_and_vay(orc):
    """A particle at the relativistic E x B drift velocity (0.9c) feels no force: HigueraCary and
    Vay keep its momentum to float rounding over 200 steps (the property both were built for);
    Boris does not (its velocity average is not the drift), the reason they exist."""
    g = grid(n=(16, 16, 16), sc=(8, 8, 4), dt=0.5)
    vd = 0.9
    E = np.zeros((3, 16, 16, 16), np.float32)
    B = np.zeros_like(E)
    E[1] = np.float32(vd)  # E x B / B^2 = vd x-hat for B = z-hat
    B[2] = 1.0
    dev = {}
    for pusher in PUSHERS:
        p, sp = _single(g, [vd / np.sqrt(1 - vd * vd), 0, 0], pusher)
        m0 = p["mom"].copy()
        worst = 0.0
        for _ in range(200):
            orc.push(g, sp, p, E, B)
            worst = max(worst, float(np.abs(p["mom"] - m0).max() / np.abs(m0).max()))
        dev[pusher] = worst
    assert dev["HigueraCary"] < 1e-5 and dev["Vay"] < 1e-5, dev
    assert dev["Boris"] > 1e-2, dev


@pytest.mark.parametrize("current", [1, 2], ids=["Esirkepov", "EmZ"])
@pytest.mark.parametrize("shape", [1, 2, 3])
def test_charge_continuity(orc, shape, current):
    """(rho1 - rho0)/dt + div J = 0 on every node, the defining property of Esirkepov and EmZ."""
    g = grid(n=(16, 16, 8))
    rng = np.random.default_rng(7 + shape)
    p = random_particles(g, 3, rng, u_th=0.3)
    sp = dict(charge=-1.0, mass=1.0, shape=shape, pusher=1, current=current)
    shp = (g["nz"], g["ny"], g["nx"])
    rho0 = np.zeros(shp, np.float32)
    orc.charge_density(g, sp, p, rho0)
    E = np.zeros((3,) + shp, np.float32)
    orc.push(g, sp, p, E, E.copy())
    rho1 = np.zeros(shp, np.float32)
    orc.charge_density(g, sp, p, rho1)
    J = np.zeros((3,) + shp, np.float32)
    orc.deposit(g, sp, p, J)
    divJ = ((J[0] - np.roll(J[0], 1, axis=2)) / g["dx"] + (J[1] - np.roll(J[1], 1, axis=1)) / g["dy"]
            + (J[2] - np.roll(J[2], 1, axis=0)) / g["dz"]).astype(np.float64)
    res = (rho1.astype(np.float64) - rho0) / g["dt"] + divJ
    scale = np.abs(rho0).max() / g["dt"]
    assert np.abs(res).max() < 1e-5 * scale


def test_yee_matches_numpy_restatement(orc):
    g = grid(n=(16, 8, 12), sc=(8, 4, 4), d=(1.0, 1.5, 0.75))
    rng = np.random.default_rng(3)
    E = random_field(g, rng)
    B = random_field(g, rng)
    J = random_field(g, rng)
    f32 = np.float32
    dt, dx, dy, dz = f32(g["dt"]), f32(g["dx"]), f32(g["dy"]), f32(g["dz"])

    def curl(F, fwd):
        s = -1 if fwd else 1
        ax = {0: 2, 1: 1, 2: 0}

        def d(c, a, h):
            r = np.roll(F[c], s, axis=ax[a])
            return ((r - F[c]) if fwd else (F[c] - r)) / h
        return [d(2, 1, dy) - d(1, 2, dz), d(0, 2, dz) - d(2, 0, dx), d(1, 0, dx) - d(0, 1, dy)]

    Bn = B.copy()
    cE = curl(E, True)
    for c in range(3):
        Bn[c] = Bn[c] - cE[c] * f32(0.5) * dt
    Bo = B.copy()
    orc.yee_b_half(g, E, Bo)
    assert np.array_equal(Bo, Bn)
    En = E.copy()
    cB = curl(Bo, False)
    for c in range(3):
        En[c] = En[c] + cB[c] * (f32(g["c"]) * f32(g["c"])) * dt
    Eo = E.copy()
    orc.yee_e(g, Bo, Eo)
    assert np.array_equal(Eo, En)
    coeff = -(f32(1.0) / f32(g["eps0"])) * dt
    En2 = (En + coeff * J).astype(np.float32)
    orc.add_current(g, J, Eo)
    assert np.array_equal(Eo, En2)


def test_photon_pusher_moves_at_c(orc):
    """particlePusherPhoton.hpp: free streaming at |v| = c along the momentum, whatever |p|."""
    g = grid(n=(16, 16, 16), sc=(8, 8, 4), dt=0.5)
    rng = np.random.default_rng(4)
    n = 256
    mom = rng.normal(size=(3, n)).astype(np.float32) * np.float32(10.0) ** rng.uniform(-3, 3, n).astype(np.float32)
    p = dict(pos=np.full((3, n), 0.5, np.float32), mom=mom, w=np.ones(n, np.float32),
             sc=np.zeros(n, np.int32), lcell=np.zeros(n, np.uint16))
    sp = dict(charge=0.0, mass=0.0, shape=2, pusher=5, current=0)
    zero = np.zeros((3, 16, 16, 16), np.float32)
    before = global_cells(g, p) + p["pos"].astype(np.float64)
    orc.push(g, sp, p, zero, zero)
    after = global_cells(g, p) + p["pos"].astype(np.float64)
    d = (after - before + 8) % 16 - 8  # periodic unwrap
    speed = np.sqrt((d ** 2).sum(axis=0)) / g["dt"]
    assert np.allclose(speed, g["c"], rtol=1e-5)
