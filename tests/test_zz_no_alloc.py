"""The allocation-free charge-conservation entry point against the simulation handle's.

picgb_charge_residual_noalloc serves callers that cannot call cudaMalloc (for
instance a plugin inside an application that already reserved the device
memory); it keeps its charge density in a static device array of at most
picgb_noalloc_max_cells() cells.  Here it reads the same particles and E field
as picgb_charge_residual on a simulation handle, through the C-ABI, twice in a
row (the shared scratch must be cleared between calls), and must agree within
the tolerance of the other charge tests: both sum the density with float
atomics in different orders.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import picongpu_gb300 as pg
from picongpu_gb300 import _lib as L
from plasma import random_field, random_particles

pytestmark = pytest.mark.gpu

REL = 1e-5


def _device_particles(torch, p):
    """Copy a host particle dict to CUDA tensors; returns (descriptor, tensors to keep alive)."""
    keep = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in p.items() if k in ("pos", "w", "sc")}
    keep["lcell"] = torch.from_numpy(p["lcell"].astype(np.int16)).cuda()
    d = L.Particles()
    d.n = p["w"].size
    for k in range(3):
        d.pos[k] = keep["pos"][k].data_ptr()
        d.mom[k] = None
    d.w = keep["w"].data_ptr()
    d.sc = keep["sc"].data_ptr()
    d.lcell = keep["lcell"].data_ptr()
    d.id = None
    return d, keep


def test_noalloc_residual_matches_simulation_handle():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    lib = L.load()
    g = pg.Grid(32, 32, 16)
    gd = g.as_dict()
    rng = np.random.default_rng(77)
    pe = random_particles(gd, 4, rng, u_th=0.1, weight=0.02)
    pi = random_particles(gd, 4, rng, u_th=0.1 / np.sqrt(1836.0), mass=1836.0, weight=0.02)
    with pg.Simulation(g) as sim:
        sim.add_species(pg.Species("e", -1.0, 1.0, shape="TSC"))
        sim.add_species(pg.Species("i", 1.0, 1836.0, shape="CIC"))
        sim.set_particles("e", pe)
        sim.set_particles("i", pi)
        sim.set_field("E", random_field(gd, rng, 0.01))
        sim.step()
        ref_res, ref_rho = sim.charge_residual()
        E = sim.data_connector.get("E")
        qe, qi = sim.get_particles("e"), sim.get_particles("i")
        de, ke = _device_particles(torch, qe)
        di, ki = _device_particles(torch, qi)
        species = (L.Particles * 2)(de, di)
        charge = (ctypes.c_float * 2)(-1.0, 1.0)
        shape = (ctypes.c_int32 * 2)(L.SHAPE_TSC, L.SHAPE_CIC)
        Eptr = (ctypes.c_void_p * 3)(E.ptr[0], E.ptr[1], E.ptr[2])
        cfg = L.GridConfig(g.nx, g.ny, g.nz, L.SUPERCELL_8x8x4, g.dx, g.dy, g.dz, g.dt, g.c, g.eps0, 0, 1, 0)
        for call in range(2):
            r, m = ctypes.c_double(), ctypes.c_double()
            rc = lib.picgb_charge_residual_noalloc(ctypes.byref(cfg), Eptr, 2, species, charge, shape, None,
                                                   ctypes.byref(r), ctypes.byref(m))
            assert rc == L.OK, lib.picgb_noalloc_last_error()
            assert ref_rho > 0
            assert abs(m.value - ref_rho) <= REL * ref_rho, (call, m.value, ref_rho)
            assert abs(r.value - ref_res) <= REL * ref_rho, (call, r.value, ref_res)
        del ke, ki


def test_noalloc_rejects_grids_beyond_the_scratch():
    lib = L.load()
    big = int(round(lib.picgb_noalloc_max_cells() ** (1 / 3))) * 2
    big -= big % 8
    cfg = L.GridConfig(big, big, big, L.SUPERCELL_8x8x4, 1.0, 1.0, 1.0, 0.5, 1.0, 1.0, 0, 1, 0)
    Eptr = (ctypes.c_void_p * 3)(1, 1, 1)  # never dereferenced: the size check comes first
    r, m = ctypes.c_double(), ctypes.c_double()
    rc = lib.picgb_charge_residual_noalloc(ctypes.byref(cfg), Eptr, 0, None, None, None, None, ctypes.byref(r),
                                           ctypes.byref(m))
    assert rc == L.ERR_INVALID
    assert b"static scratch" in lib.picgb_noalloc_last_error()
