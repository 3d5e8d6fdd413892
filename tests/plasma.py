"""Small seeded particle/field inputs for CPU tests (numpy; exchange format of oracle/)."""
import numpy as np


def grid(n=(16, 16, 8), sc=(8, 8, 4), dt=0.99 / np.sqrt(3.0), d=(1.0, 1.0, 1.0), c=1.0, eps0=1.0):
    return dict(nx=n[0], ny=n[1], nz=n[2], sx=sc[0], sy=sc[1], sz=sc[2], dx=d[0], dy=d[1], dz=d[2],
                dt=float(np.float32(dt)), c=c, eps0=eps0)


def random_particles(g, ppc, rng, u_th=0.01, mass=1.0, weight=0.01, drift=(0.0, 0.0, 0.0)):
    nsx, nsy, nsz = g["nx"] // g["sx"], g["ny"] // g["sy"], g["nz"] // g["sz"]
    ncell = g["nx"] * g["ny"] * g["nz"]
    n = ncell * ppc
    cells = np.repeat(np.arange(ncell), ppc)
    cx = cells % g["nx"]
    cy = (cells // g["nx"]) % g["ny"]
    cz = cells // (g["nx"] * g["ny"])
    sc = (cx // g["sx"]) + nsx * ((cy // g["sy"]) + nsy * (cz // g["sz"]))
    lc = (cx % g["sx"]) + g["sx"] * ((cy % g["sy"]) + g["sy"] * (cz % g["sz"]))
    pos = rng.random((3, n), dtype=np.float32)
    u = rng.normal(0.0, u_th, size=(3, n)) + np.asarray(drift)[:, None]
    w = np.full(n, weight, np.float32)
    mom = (u * mass * weight * g["c"]).astype(np.float32)
    return dict(pos=np.ascontiguousarray(pos), mom=np.ascontiguousarray(mom), w=w, sc=sc.astype(np.int32),
                lcell=lc.astype(np.uint16), id=np.arange(n, dtype=np.uint32))


def global_cells(g, p):
    nsx, nsy = g["nx"] // g["sx"], g["ny"] // g["sy"]
    sc = p["sc"].astype(np.int64)
    lc = p["lcell"].astype(np.int64)
    scx, scy, scz = sc % nsx, (sc // nsx) % nsy, sc // (nsx * nsy)
    x = scx * g["sx"] + lc % g["sx"]
    y = scy * g["sy"] + (lc // g["sx"]) % g["sy"]
    z = scz * g["sz"] + lc // (g["sx"] * g["sy"])
    return np.stack([x, y, z])


def random_field(g, rng, amp=0.01):
    return np.ascontiguousarray((amp * rng.standard_normal((3, g["nz"], g["ny"], g["nx"]))).astype(np.float32))
