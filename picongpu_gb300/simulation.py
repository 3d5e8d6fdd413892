"""Python mirror of the reference's operator surface for the PIC hot path.

``Simulation`` follows simulation/control/Simulation.hpp: fields "E", "B", "J"
and "FieldTmp0" exist from construction, species are added with the
``.param`` flags of param/speciesDefinition.param (pusher, shape, current
solver, charge and mass), ``step()`` runs Simulation::runOneStep and
``data_connector.get(id)`` resolves a registered id like
pmacc::DataConnector::get (raising on an unknown id).  All work runs in the
CUDA library libpicgb.so through its C-ABI.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import _lib as L

# .param policy names -> C-ABI enums (param/species.param:49-90, param/fieldSolver.param:57)
PUSHERS = {"Boris": L.PUSHER_BORIS, "Free": L.PUSHER_FREE, "HigueraCary": L.PUSHER_HIGUERA_CARY,
           "Vay": L.PUSHER_VAY, "Photon": L.PUSHER_PHOTON, None: L.PUSHER_NONE}
SHAPES = {"CIC": L.SHAPE_CIC, "TSC": L.SHAPE_TSC, "PQS": L.SHAPE_PQS, "PCS": L.SHAPE_PCS}
CURRENTS = {"Esirkepov": L.CURRENT_ESIRKEPOV, "EmZ": L.CURRENT_EMZ, None: L.CURRENT_NONE}
SOLVERS = {"Yee": L.SOLVER_YEE}
SUPERCELLS = {(8, 8, 4): L.SUPERCELL_8x8x4, (4, 4, 4): L.SUPERCELL_4x4x4, (8, 8, 8): L.SUPERCELL_8x8x8}


@dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    dx: float = 1.0
    dy: float = 1.0
    dz: float = 1.0
    dt: float = float(np.float32(0.99 / np.sqrt(3.0)))
    c: float = 1.0
    eps0: float = 1.0
    supercell: tuple = (8, 8, 4)
    solver: str = "Yee"
    fuse_deposit: bool = True
    device: int = 0

    def config(self) -> L.GridConfig:
        """The C-ABI picgb_grid_config of this grid."""
        return L.GridConfig(self.nx, self.ny, self.nz, SUPERCELLS[tuple(self.supercell)], self.dx, self.dy, self.dz,
                            self.dt, self.c, self.eps0, SOLVERS[self.solver], int(bool(self.fuse_deposit)),
                            self.device)

    @property
    def sx(self):
        return self.supercell[0]

    @property
    def sy(self):
        return self.supercell[1]

    @property
    def sz(self):
        return self.supercell[2]

    def as_dict(self):
        return dict(nx=self.nx, ny=self.ny, nz=self.nz, sx=self.sx, sy=self.sy, sz=self.sz, dx=self.dx, dy=self.dy,
                    dz=self.dz, dt=self.dt, c=self.c, eps0=self.eps0)


@dataclass
class Species:
    name: str
    charge: float
    mass: float
    pusher: str | None = "Boris"
    shape: str = "TSC"
    current: str | None = "Esirkepov"
    capacity: int = 0
    with_ids: bool = False

    def as_dict(self):
        return dict(charge=self.charge, mass=self.mass, shape=SHAPES[self.shape],
                    pusher=PUSHERS[self.pusher] if self.pusher in PUSHERS else L.PUSHER_NONE,
                    current=CURRENTS[self.current])


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


class DataConnector:
    """Named registry of simulation data (pmacc/dataManagement/DataConnector.hpp:48-136)."""

    def __init__(self, sim: "Simulation"):
        self._sim = sim

    def get(self, name: str) -> L.BufferDesc:
        d = L.BufferDesc()
        L.call("picgb_get_buffer", self._sim.handle, name.encode(), ctypes.byref(d))
        return d

    def share(self, name: str, desc: L.BufferDesc) -> None:
        L.call("picgb_share", self._sim.handle, name.encode(), ctypes.byref(desc))

    def unshare(self, name: str) -> None:
        L.call("picgb_unshare", self._sim.handle, name.encode())

    def ids(self) -> list[str]:
        n = ctypes.c_int32()
        L.call("picgb_registry_size", self._sim.handle, ctypes.byref(n))
        out = []
        buf = ctypes.create_string_buffer(256)
        for i in range(n.value):
            L.call("picgb_registry_name", self._sim.handle, i, buf, 256)
            out.append(buf.value.decode())
        return out


class Simulation:
    def __init__(self, grid: Grid):
        self.grid = grid
        cfg = grid.config()
        h = ctypes.c_void_p()
        L.call("picgb_create", ctypes.byref(cfg), ctypes.byref(h))
        self._init_handle(h, grid, owned=True)

    def _init_handle(self, h, grid: Grid, owned: bool):
        self.grid = grid
        self.handle = h
        self._owned = owned
        self.species: list[Species] = []
        self.data_connector = DataConnector(self)
        self.current_step = 0

    @classmethod
    def borrowed(cls, handle: ctypes.c_void_p, grid: Grid, species: list[Species]) -> "Simulation":
        """Wrapper of a handle owned elsewhere (a box of an ensemble); close() leaves it alive."""
        self = cls.__new__(cls)
        self._init_handle(handle, grid, owned=False)
        self.species = list(species)
        return self

    # ------------------------------------------------------------ lifetime
    def close(self):
        if self.handle:
            if self._owned:
                L.load().picgb_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ species
    def add_species(self, sp: Species) -> int:
        if sp.pusher not in PUSHERS:
            raise ValueError(f"unknown pusher {sp.pusher!r}; available: {[k for k in PUSHERS if k]} or None")
        if sp.shape not in SHAPES:
            raise ValueError(f"unknown shape {sp.shape!r}; available: {list(SHAPES)}")
        if sp.current not in CURRENTS:
            raise ValueError(f"unknown current solver {sp.current!r}; available: {[k for k in CURRENTS if k]} or None")
        pusher = PUSHERS[sp.pusher]
        cfg =L.SpeciesConfig(sp.name.encode(), sp.charge, sp.mass, pusher, SHAPES[sp.shape],
                              CURRENTS[sp.current], sp.capacity, int(sp.with_ids))
        idx = ctypes.c_int32()
        L.call("picgb_add_species", self.handle, ctypes.byref(cfg), ctypes.byref(idx))
        self.species.append(sp)
        return idx.value

    def species_index(self, name: str) -> int:
        for i, s in enumerate(self.species):
            if s.name == name:
                return i
        raise RuntimeError(f"unknown species '{name}'")

    def set_particles(self, name: str, p: dict) -> None:
        i = self.species_index(name)
        arrs = {k: np.ascontiguousarray(p[k]) for k in ("pos", "mom", "w", "sc", "lcell")}
        assert arrs["pos"].dtype == np.float32 and arrs["mom"].dtype == np.float32 and arrs["w"].dtype == np.float32
        arrs["sc"] = arrs["sc"].astype(np.int32, copy=False)
        arrs["lcell"] = arrs["lcell"].astype(np.uint16, copy=False)
        ids = np.ascontiguousarray(p["id"], dtype=np.uint32) if "id" in p else None
        d = L.Particles()
        d.n = arrs["w"].shape[0]
        for k in range(3):
            d.pos[k] = arrs["pos"][k].ctypes.data
            d.mom[k] = arrs["mom"][k].ctypes.data
        d.w = arrs["w"].ctypes.data
        d.sc = arrs["sc"].ctypes.data
        d.lcell = arrs["lcell"].ctypes.data
        d.id = ids.ctypes.data if ids is not None else None
        L.call("picgb_species_set", self.handle, i, ctypes.byref(d))

    def init_plasma(self, name: str, ppc: int, density: float, u_th: float, drift_lo=(0, 0, 0), drift_hi=None,
                    split_axis: int = -1, split_cell: int = 0, seed: int = 42, position_seed: int = 42,
                    quiet=None) -> None:
        """Seeded plasma on the device: random in-cell positions (startPosition::Random), or with
        quiet=(nx, ny, nz) the in-cell lattice of startPosition::Quiet (ppc 0 or nx*ny*nz)."""
        ip = L.PlasmaInit(ppc, density, u_th, (ctypes.c_float * 3)(*drift_lo),
                          (ctypes.c_float * 3)(*(drift_hi if drift_hi is not None else drift_lo)), split_axis,
                          split_cell, seed, position_seed, (ctypes.c_uint32 * 3)(*(quiet or (0, 0, 0))))
        L.call("picgb_species_init_plasma", self.handle, self.species_index(name), ctypes.byref(ip))

    def particle_count(self, name: str) -> int:
        n = ctypes.c_uint64()
        L.call("picgb_species_count", self.handle, self.species_index(name), ctypes.byref(n))
        return n.value

    def get_particles(self, name: str, with_ids: bool | None = None, out: dict | None = None) -> dict:
        """Copy a species out in the host exchange format; ``out`` may hold preallocated
        (e.g. pinned) arrays with room for every particle."""
        i = self.species_index(name)
        n = self.particle_count(name)
        if with_ids is None:
            with_ids = self.species[i].with_ids
        if out is None:
            out = dict(pos=np.empty((3, n), np.float32), mom=np.empty((3, n), np.float32),
                       w=np.empty(n, np.float32), sc=np.empty(n, np.int32), lcell=np.empty(n, np.uint16))
            if with_ids:
                out["id"] = np.empty(n, np.uint32)
        else:
            with_ids = "id" in out
            if out["w"].shape[0] < n or out["pos"].shape[1] < n:
                raise ValueError(f"output arrays hold fewer than {n} particles")
        d = L.Particles()
        d.n = n
        for k in range(3):
            d.pos[k] = out["pos"][k].ctypes.data
            d.mom[k] = out["mom"][k].ctypes.data
        d.w = out["w"].ctypes.data
        d.sc = out["sc"].ctypes.data
        d.lcell = out["lcell"].ctypes.data
        d.id = out["id"].ctypes.data if with_ids else None
        L.call("picgb_species_get", self.handle, i, ctypes.byref(d))
        return out

    # ------------------------------------------------------------ fields
    def _field_shape(self, name):
        nc = 1 if name == "FieldTmp0" else 3
        return (nc, self.grid.nz, self.grid.ny, self.grid.nx)

    def set_field(self, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float32).reshape(self._field_shape(name))
        ptrs = (ctypes.c_void_p * a.shape[0])(*[a[c].ctypes.data for c in range(a.shape[0])])
        L.call("picgb_field_set", self.handle, name.encode(), ptrs)

    def get_field(self, name: str) -> np.ndarray:
        a = np.empty(self._field_shape(name), np.float32)
        ptrs = (ctypes.c_void_p * a.shape[0])(*[a[c].ctypes.data for c in range(a.shape[0])])
        L.call("picgb_field_get", self.handle, name.encode(), ptrs)
        return a

    # ------------------------------------------------------------ boundaries
    def set_boundaries(self, open_axes=(False, False, False), thickness=((0, 0), (0, 0), (0, 0)), absorber="PML",
                       sigma_max=None, kappa_max=(1.0, 1.0, 1.0), alpha_max=(0.0, 0.0, 0.0), grading_order: float = 4.0,
                       alpha_grading_order: float = 1.0, strength=((1e-3, 1e-3),) * 3) -> None:
        """Open axes (absorbing layers, absorbing particles) as the reference's non-periodic
        boundaries; absorber "PML" (fields/absorber/pml; sigma_max None: 0.8 (m + 1) c / cell edge)
        or "Exponential" (fields/absorber/exponential, damping strength per face)."""
        if absorber not in ("PML", "Exponential"):
            raise ValueError(f"unknown absorber {absorber!r}: 'PML' or 'Exponential'")
        b = L.BoundaryConfig()
        b.absorber = 0 if absorber == "PML" else 1
        for a in range(3):
            b.open[a] = int(bool(open_axes[a]))
            b.thickness[a][0], b.thickness[a][1] = int(thickness[a][0]), int(thickness[a][1])
            b.sigma_max[a] = -1.0 if sigma_max is None else float(sigma_max[a])
            b.kappa_max[a] = float(kappa_max[a])
            b.alpha_max[a] = float(alpha_max[a])
            b.strength[a][0], b.strength[a][1] = float(strength[a][0]), float(strength[a][1])
        b.grading_order = grading_order
        b.alpha_grading_order = alpha_grading_order
        L.call("picgb_set_boundaries", self.handle, ctypes.byref(b))

    # ------------------------------------------------------------ checkpoints
    def write_checkpoint(self, directory: str, step: int | None = None) -> str:
        """openPMD checkpoint of E, B and every species as iteration ``step`` (default: the
        current step, i.e. the state after that many steps); returns the iteration directory."""
        step = self.current_step if step is None else int(step)
        L.call("picgb_checkpoint_write", self.handle, os.fsencode(directory), step)
        return os.path.join(directory, f"simData_{step}")

    def read_checkpoint(self, directory: str, step: int) -> None:
        """Restart from iteration ``step``: E, B and the species of this simulation (by name);
        J is zeroed and the next step index becomes ``step``."""
        L.call("picgb_checkpoint_read", self.handle, os.fsencode(directory), int(step))
        self.current_step = int(step)

    # ------------------------------------------------------------ stepping
    def set_incident_field(self, a0: float, wavelength: float, waist: float, duration_fwhm: float, t_center: float,
                           surface: int, polarisation: int = 0, center=None, phase: float = 0.0,
                           e_over_m: float = 1.0, focus: float = 0.0, axis: int = 1, direction: int = 1,
                           propagation=None, polarisation_vector=None, circular: bool = False,
                           time_delay: float = 0.0, laguerre_modes=None, laguerre_phases=None,
                           profile: str = "GaussianPulse", ramp_init: float = 0.0, plateau: float = 0.0,
                           pulse_duration: float = 0.0, waist_axis=None, pulse_init: float = 0.0) -> None:
        """Focused Gaussian pulse entering through the TF/SF face normal to `axis` (0, 1, 2):
        direction +1 from the low face along +axis, -1 from the high face along -axis
        (fields/incidentField/Solver.hpp, profiles/GaussianPulse.hpp).  `surface` is the first
        (+1) or last (-1) E plane of the total-field region, the focus lies `focus` cells beyond
        the Huygens surface (a quarter cell before that plane), `center` is the beam centre on
        the two transverse axes in increasing order (default: the middle), `polarisation` 0 or 1
        puts E along the first or the second of them, `phase` is the reference's LASER_PHASE of
        the cosine carrier and `t_center` its PULSE_INIT * PULSE_DURATION / 2.  `propagation`
        and `polarisation_vector` (unit 3-vectors, DIRECTION_* and POLARISATION_DIRECTION_*) give
        oblique incidence through the face, `circular` circular polarisation; `time_delay` is
        TIME_DELAY and `laguerre_modes` / `laguerre_phases` (up to 8) the Laguerre-Gauss mode sum
        of GaussianPulse.  profile "PlaneWave" is profiles/PlaneWave.hpp with `ramp_init` (RAMP_INIT)
        and `plateau` (LASER_NOFOCUS_CONSTANT), "Wavepacket" and "Polynom" their profiles with
        `waist_axis` (W0_AXIS_1, W0_AXIS_2) and, for the Wavepacket, `pulse_init` (PULSE_INIT) and
        `plateau`; `pulse_duration` > 0 gives PULSE_DURATION directly.  Each face holds its own
        pulse; see picgb_set_incident_field."""
        profiles = {"GaussianPulse": 0, "PlaneWave": 1, "Wavepacket": 2, "Polynom": 3}
        if profile not in profiles:
            raise ValueError(f"unknown incident profile {profile!r}: one of {sorted(profiles)}")
        cells = (self.grid.nx, self.grid.ny, self.grid.nz)
        t1, t2 = [d for d in range(3) if d != axis] if axis in (0, 1, 2) else (0, 2)
        c1, c2 = center if center is not None else (cells[t1] / 2.0, cells[t2] / 2.0)
        f = L.IncidentField(1, axis, surface, polarisation, a0, e_over_m, wavelength, waist, duration_fwhm, t_center,
                            c1, c2, phase, focus, direction, (ctypes.c_float * 3)(*(propagation or (0, 0, 0))),
                            (ctypes.c_float * 3)(*(polarisation_vector or (0, 0, 0))), int(bool(circular)),
                            float(time_delay), len(laguerre_modes or ()),
                            (ctypes.c_float * 8)(*(laguerre_modes or ())),
                            (ctypes.c_float * 8)(*(laguerre_phases or ())), profiles[profile], float(ramp_init),
                            float(plateau), float(pulse_duration), (ctypes.c_float * 2)(*(waist_axis or (0.0, 0.0))),
                            float(pulse_init))
        L.call("picgb_set_incident_field", self.handle, ctypes.byref(f))

    def clear_incident_field(self, axis: int | None = None, direction: int = 1) -> None:
        """Switch off the pulse of one face (axis, direction), or of every face (axis None)."""
        if axis is None:
            L.call("picgb_set_incident_field", self.handle, None)
            return
        f = L.IncidentField()
        f.axis = axis
        f.direction = direction
        L.call("picgb_set_incident_field", self.handle, ctypes.byref(f))

    def step(self) -> None:
        L.call("picgb_step", self.handle, self.current_step)
        self.current_step += 1

    def run(self, n: int) -> None:
        L.call("picgb_run", self.handle, self.current_step, n)
        self.current_step += n

    def stage(self, name: str) -> None:
        fn = "picgb_stage_" + name
        if name in ("current_reset", "add_current"):
            L.call(fn, self.handle)
        else:
            L.call(fn, self.handle, self.current_step)

    def synchronize(self) -> None:
        L.call("picgb_synchronize", self.handle)

    def set_sort_interval(self, steps: int) -> None:
        """Restore the interleaved cell order of every supercell every `steps` steps (0: never);
        see picgb_set_sort_interval."""
        L.call("picgb_set_sort_interval", self.handle, int(steps))

    def set_stream(self, stream_ptr: int | None) -> None:
        L.call("picgb_set_stream", self.handle, ctypes.c_void_p(stream_ptr) if stream_ptr else None)

    # ------------------------------------------------------------ diagnostics
    def energies(self) -> dict:
        n = 2 + len(self.species)
        out = (ctypes.c_double * n)()
        L.call("picgb_energies", self.handle, out, n)
        d = {"E": out[0], "B": out[1]}
        for i, s in enumerate(self.species):
            d[s.name] = out[2 + i]
        return d

    def charge_residual(self) -> tuple[float, float]:
        r = ctypes.c_double()
        m = ctypes.c_double()
        L.call("picgb_charge_residual", self.handle, ctypes.byref(r), ctypes.byref(m))
        return r.value, m.value

    def launch_count(self) -> int:
        n = ctypes.c_uint64()
        L.call("picgb_launch_count", self.handle, ctypes.byref(n))
        return n.value

    def profile(self, on: bool = True) -> None:
        """Per-kernel CUDA-event timing on the launching stream; enabling resets the counters."""
        L.call("picgb_profile_enable", self.handle, int(on))

    def kernel_times(self) -> dict:
        """{kernel class: (total device ms, launches)} since profiling was enabled."""
        out = {}
        for name, k in L.KERNEL_CLASSES.items():
            ms = ctypes.c_double()
            n = ctypes.c_uint64()
            L.call("picgb_profile_read", self.handle, k, ctypes.byref(ms), ctypes.byref(n))
            out[name] = (ms.value, n.value)
        return out

    def deposit_kinds(self) -> tuple[int, int]:
        """(deposits with the short footprint, general deposits) since profiling was enabled."""
        out = (ctypes.c_uint64 * 2)()
        L.call("picgb_profile_deposit_kinds", self.handle, out)
        return out[0], out[1]

    def device_status(self, reset: bool = False) -> int:
        b = ctypes.c_uint32()
        L.call("picgb_device_status", self.handle, ctypes.byref(b), int(reset))
        return b.value
