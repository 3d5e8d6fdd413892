"""Species transfers through page-locked host memory against pageable memory.

Page-locked arrays are read by a copy kernel over the host link on upload and written by the
gather kernel on download; pageable arrays go through cudaMemcpyAsync and a staging buffer.
Contract, for two species with ids on a 32 x 32 x 16 box:
* an upload and download through page-locked arrays returns the same particles (sorted by id)
  bit for bit as through pageable arrays, for arrays starting on 16-byte boundaries and for
  arrays misaligned by one element, and for an odd particle count;
* one step after either upload gives bit-identical particles.
"""
import numpy as np
import pytest

import picongpu_gb300 as pg

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

DT = float(np.float32(0.99 / np.sqrt(3.0)))


def make():
    g = pg.Grid(32, 32, 16, dt=DT)
    sim = pg.Simulation(g)
    sim.add_species(pg.Species("e", -1.0, 1.0, shape="TSC", with_ids=True))
    sim.add_species(pg.Species("i", 1.0, 1836.0, shape="TSC", with_ids=True))
    return sim


def pinned(p, offset, keep):
    """A copy of the exchange dict in page-locked memory, each array starting `offset` elements
    into its own page-locked buffer (offset 1 breaks the 16-byte alignment)."""
    out = {}
    for k, v in p.items():
        tdt = torch.int16 if v.dtype == np.uint16 else getattr(torch, str(v.dtype))
        t = torch.empty(v.size + offset, dtype=tdt, pin_memory=True)
        keep.append(t)
        flat = t.numpy().view(v.dtype)
        a = flat[offset:offset + v.size].reshape(v.shape)
        a[...] = v
        out[k] = a
    return out


def by_id(p):
    o = np.argsort(p["id"], kind="stable")
    return {k: (v[:, o] if v.ndim == 2 else v[o]) for k, v in p.items()}


def take(p, n):
    return {k: (v[:, :n].copy() if v.ndim == 2 else v[:n].copy()) for k, v in p.items()}


@pytest.mark.parametrize("offset", [0, 1])
def test_page_locked_round_trip_and_step(offset):
    src = make()
    with src:
        src.init_plasma("e", 6, 0.02, 0.05, drift_lo=(0.1, 0.0, 0.0), seed=3, position_seed=4)
        src.init_plasma("i", 6, 0.02, 0.002, seed=5, position_seed=4)
        p = {name: src.get_particles(name) for name in ("e", "i")}
    p["e"] = take(p["e"], p["e"]["w"].size - 3)  # an odd count
    keep = []
    a, b = make(), make()
    with a, b:
        for name in ("e", "i"):
            a.set_particles(name, p[name])
            b.set_particles(name, pinned(p[name], offset, keep))
        for name in ("e", "i"):
            n = b.particle_count(name)
            assert n == p[name]["w"].size
            out = pinned({k: np.zeros_like(v) for k, v in p[name].items()}, offset, keep)
            got = by_id(b.get_particles(name, out=out))
            want = by_id(a.get_particles(name))
            ref = by_id(p[name])
            for k in ("id", "pos", "mom", "w", "sc", "lcell"):
                assert np.array_equal(got[k], want[k]), (name, k)
                assert np.array_equal(got[k], ref[k]), (name, k)
        a.step()
        b.step()
        for name in ("e", "i"):
            x, y = by_id(a.get_particles(name)), by_id(b.get_particles(name))
            for k in ("id", "pos", "mom", "sc", "lcell"):
                assert np.array_equal(x[k], y[k]), (name, k)
