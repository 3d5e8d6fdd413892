"""The allocation-free charge-conservation entry point, through the C-ABI.

picgb_charge_residual_noalloc serves callers that cannot call cudaMalloc (for
instance a plugin inside an application that already reserved the device
memory); it keeps its charge density in a static device array of at most
picgb_noalloc_max_cells() cells.  Here it reads particles of three species (CIC,
TSC, PQS) and an E field in device memory, twice in a row (the shared scratch
must be cleared between calls), and must agree with
* the CPU oracle's charge density (max|rho|) and residual max|eps0 div E - rho|
  on the same particles and E, and
* picgb_charge_residual of a simulation handle holding the same particles,
within 1e-5 of max|rho| (float atomics sum the density in another order).
Around the second call the device's free memory must not change, and the
caller's current device must be the same afterwards.  This file is collected
last on purpose.
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


def test_noalloc_residual_matches_oracle_and_simulation_handle(orc):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    lib = L.load()
    g = pg.Grid(32, 32, 16)
    gd = g.as_dict()
    rng = np.random.default_rng(77)
    spec = [pg.Species("e", -1.0, 1.0, shape="TSC"), pg.Species("i", 1.0, 1836.0, shape="CIC"),
            pg.Species("p", -1.0, 1.0, shape="PQS")]
    parts = [random_particles(gd, 4, rng, u_th=0.1, weight=0.02),
             random_particles(gd, 4, rng, u_th=0.1 / np.sqrt(1836.0), mass=1836.0, weight=0.02),
             random_particles(gd, 2, rng, u_th=0.1, weight=0.01)]
    with pg.Simulation(g) as sim:
        for s, p in zip(spec, parts):
            sim.add_species(s)
            sim.set_particles(s.name, p)
        sim.set_field("E", random_field(gd, rng, 0.01))
        sim.step()
        ref_res, ref_rho = sim.charge_residual()
        E = sim.data_connector.get("E")
        Eh = sim.get_field("E")
        got = [sim.get_particles(s.name) for s in spec]
        # the oracle on the same particles and E
        rho = np.zeros((g.nz, g.ny, g.nx), np.float32)
        for s, q in zip(spec, got):
            r = np.zeros_like(rho)
            orc.charge_density(gd, s.as_dict(), q, r)
            rho += r
        orc_rho = float(np.abs(rho).max())
        orc_res, _ = orc.charge_residual(gd, Eh, rho)
        dev = [_device_particles(torch, q) for q in got]
        species = (L.Particles * 3)(*[d for d, _ in dev])
        charge = (ctypes.c_float * 3)(*[s.charge for s in spec])
        shape = (ctypes.c_int32 * 3)(L.SHAPE_TSC, L.SHAPE_CIC, L.SHAPE_PQS)
        Eptr = (ctypes.c_void_p * 3)(E.ptr[0], E.ptr[1], E.ptr[2])
        cfg = L.GridConfig(g.nx, g.ny, g.nz, L.SUPERCELL_8x8x4, g.dx, g.dy, g.dz, g.dt, g.c, g.eps0, 0, 1, 0)
        assert orc_rho > 0 and ref_rho > 0
        for call in range(2):
            torch.cuda.synchronize()
            free0, _ = torch.cuda.mem_get_info()
            r, m = ctypes.c_double(), ctypes.c_double()
            rc = lib.picgb_charge_residual_noalloc(ctypes.byref(cfg), Eptr, 3, species, charge, shape, None,
                                                   ctypes.byref(r), ctypes.byref(m))
            assert rc == L.OK, lib.picgb_noalloc_last_error()
            free1, _ = torch.cuda.mem_get_info()
            if call == 1:  # the first call may load the library's device code (and its scratch)
                assert free1 == free0, (free0, free1)
            assert torch.cuda.current_device() == 0
            assert abs(m.value - orc_rho) <= REL * orc_rho, (call, m.value, orc_rho)
            assert abs(r.value - orc_res) <= REL * orc_rho, (call, r.value, orc_res)
            assert abs(m.value - ref_rho) <= REL * ref_rho, (call, m.value, ref_rho)
            assert abs(r.value - ref_res) <= REL * ref_rho, (call, r.value, ref_res)
        del dev


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
