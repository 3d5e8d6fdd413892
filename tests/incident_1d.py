"""Float64 restatement of the 1D split Yee update with the total-field/scattered-field
corrections of one face, fed with the plane pulse (waist -> infinity) of
profiles/GaussianPulse.hpp: a transversely uniform pulse on the 3D Yee grid obeys the 1D
scheme exactly, so this is the reference for the tangential fields along the axis."""
import math

import numpy as np


def plane_pulse(u, t, P, direction, g, lam, fwhm, tc):
    """E of the pulse at position u (cells) along the axis and time t: the local time runs from
    the Huygens surface P - direction / 4 at the Yee grid's phase velocity and the field is zero
    before it starts; cosine carrier; envelope exp(-(time / 2 tau)^2) with tau the rms duration
    of the intensity (intensity FWHM = 2 sqrt(2 ln 2) tau); E0 = a0 omega c / (e/m) with a0 = 1."""
    omega = 2 * math.pi * g.c / lam
    dt = float(np.float32(g.dt))
    kn = 2.0 / g.dx * math.asin(g.dx / (g.c * dt) * math.sin(omega * dt / 2))
    tau2 = fwhm / math.sqrt(2 * math.log(2))
    tloc = t - direction * (u - (P - 0.25 * direction)) * g.dx * kn / omega
    time = tloc - tc
    return np.where(tloc < 0, 0.0, omega * np.exp(-(time / tau2) ** 2) * np.cos(omega * time))


def yee_1d(n, P, direction, g, lam, fwhm, tc, steps):
    """E_p (integer positions) and B' (half-integer positions, B' = eta B_o with eta = +1 when
    (axis, p, o) is anticyclic, i.e. p = (axis + 2) % 3) of the split update
    dB'/dt = dE/du, dE/dt = c^2 dB'/du with the corrections of the face whose first (+1) or
    last (-1) total E plane is P: the scattered-side B plane is P - 1 (+1) or P (-1)."""
    E = np.zeros(n)
    Bt = np.zeros(n)
    dt, da, c = float(np.float32(g.dt)), g.dx, g.c
    bidx = P - 1 if direction > 0 else P
    sgn = -1.0 if direction > 0 else 1.0
    for s in range(steps):
        t = s * dt
        Bt += 0.5 * dt * (np.roll(E, -1) - E) / da
        Bt[bidx] += sgn * 0.5 * dt / da * plane_pulse(P, t, P, direction, g, lam, fwhm, tc)
        E += c * c * dt * (Bt - np.roll(Bt, 1)) / da
        E[P] += c * dt / da * plane_pulse(P - 0.5 * direction, t + 0.5 * dt, P, direction, g, lam, fwhm, tc)
        Bt += 0.5 * dt * (np.roll(E, -1) - E) / da
        Bt[bidx] += sgn * 0.5 * dt / da * plane_pulse(P, t + dt, P, direction, g, lam, fwhm, tc)
    return E, Bt


def line(F, comp, axis, u1, u2):
    """Values of component comp along `axis` at transverse cells (u1, u2) (first, second
    transverse axis in increasing order); F is [3][nz][ny][nx]."""
    A = F[comp]
    if axis == 0:
        return A[u2, u1, :]
    if axis == 1:
        return A[u2, :, u1]
    return A[:, u2, u1]
