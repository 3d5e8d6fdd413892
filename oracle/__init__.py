"""CPU oracle for the PIC-cycle hot path -- TEST INFRASTRUCTURE ONLY.

The oracle is a plain C++ restatement (``pic_oracle.hpp``) of PIConGPU's
reference algorithms for the electromagnetic PIC step: Yee field solver
(fields/MaxwellSolver/FDTD/FDTDBase.kernel), form-factor gather
(algorithms/FieldToParticleInterpolation.hpp), Boris push
(particles/pusher/particlePusherBoris.hpp, particlePusherHigueraCary.hpp,
particlePusherVay.hpp), moveParticle
(particles/MoveParticle.hpp), Esirkepov deposition
(fields/currentDeposition/Esirkepov/Esirkepov.hpp) and the energy and charge
conservation diagnostics.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may load it, and only as the checker.

Data conventions (shared with the CUDA library's host exchange format):

* fields: float32 arrays of shape ``(3, nz, ny, nx)``, no guard cells, periodic;
* particles: dict with ``pos`` (3, n) float32 in-cell positions in [0, 1),
  ``mom`` (3, n) float32 macro-weighted momenta, ``w`` (n,) float32 weightings,
  ``sc`` (n,) int32 supercell index, ``lcell`` (n,) uint16 cell index inside
  the supercell and optionally ``id`` (n,) uint32.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


class OrcGrid(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("nx", "ny", "nz", "sx", "sy", "sz")] + [
        (n, ctypes.c_float) for n in ("dx", "dy", "dz", "dt", "c", "eps0")
    ] + [("open", ctypes.c_int)]


class OrcPml(ctypes.Structure):
    _fields_ = [("cells", (ctypes.c_int * 2) * 3), ("sigma_max", ctypes.c_double * 3),
                ("kappa_max", ctypes.c_double * 3), ("alpha_max", ctypes.c_double * 3),
                ("order", ctypes.c_double), ("alpha_order", ctypes.c_double)]


class OrcSpecies(ctypes.Structure):
    _fields_ = [
        ("charge", ctypes.c_float),
        ("mass", ctypes.c_float),
        ("shape", ctypes.c_int),
        ("pusher", ctypes.c_int),
        ("current", ctypes.c_int),
    ]


class OrcField(ctypes.Structure):
    _fields_ = [("c", ctypes.c_void_p * 3)]


class OrcIncidentFace(ctypes.Structure):
    _fields_ = [("axis", ctypes.c_int), ("dir", ctypes.c_int), ("surface", ctypes.c_int),
                ("dirv", ctypes.c_float * 3), ("polv", ctypes.c_float * 3), ("focus", ctypes.c_float * 3),
                ("circular", ctypes.c_int),
                ("amplitude", ctypes.c_float), ("wavelength", ctypes.c_float), ("w0", ctypes.c_float),
                ("pulse_duration", ctypes.c_float), ("time_shift", ctypes.c_float), ("laser_phase", ctypes.c_float),
                ("phase_velocity", ctypes.c_float), ("time_delay", ctypes.c_float), ("nmodes", ctypes.c_int),
                ("modes", ctypes.c_float * 8), ("mode_phases", ctypes.c_float * 8), ("profile", ctypes.c_int),
                ("ramp_init", ctypes.c_float), ("nofocus", ctypes.c_float), ("pulse_init", ctypes.c_float),
                ("w0_axis1", ctypes.c_float), ("w0_axis2", ctypes.c_float)]


class OrcParticles64(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint64),
        ("pos", ctypes.c_void_p * 3),
        ("mom", ctypes.c_void_p * 3),
        ("w", ctypes.c_void_p),
        ("sc", ctypes.c_void_p),
        ("lcell", ctypes.c_void_p),
    ]


class OrcParticles(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint64),
        ("pos", ctypes.c_void_p * 3),
        ("mom", ctypes.c_void_p * 3),
        ("w", ctypes.c_void_p),
        ("sc", ctypes.c_void_p),
        ("lcell", ctypes.c_void_p),
    ]


def _stale() -> bool:
    t = os.path.getmtime(_LIB_PATH)
    return any(os.path.getmtime(os.path.join(_HERE, f)) > t for f in ("oracle_capi.cpp", "pic_oracle.hpp", "Makefile"))


def build(force: bool = False) -> str:
    """Compile the oracle shared library with its Makefile (g++, OpenMP); make rebuilds
    it when a source is newer than the library."""
    if force or not os.path.exists(_LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        vp = ctypes.c_void_p
        L.orc_shape_value.restype = ctypes.c_float
        L.orc_shape_value.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float]
        L.orc_shape_ca_array.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_int, vp]
        L.orc_shape_os_array.argtypes = [ctypes.c_int, ctypes.c_float, vp]
        L.orc_move_particle.restype = ctypes.c_int
        L.orc_move_particle.argtypes = [P(OrcGrid), vp, vp, vp]
        L.orc_gather.argtypes = [P(OrcGrid), ctypes.c_int, P(OrcField), ctypes.c_int, vp, vp, vp]
        L.orc_yee_b_half.argtypes = [P(OrcGrid), P(OrcField), P(OrcField)]
        L.orc_incident_update.argtypes = [P(OrcGrid), P(OrcIncidentFace), P(OrcField), ctypes.c_int, ctypes.c_float]
        L.orc_yee_e.argtypes = [P(OrcGrid), P(OrcField), P(OrcField)]
        L.orc_add_current.argtypes = [P(OrcGrid), P(OrcField), P(OrcField)]
        L.orc_push.argtypes = [P(OrcGrid), P(OrcSpecies), P(OrcParticles), P(OrcField), P(OrcField)]
        L.orc_deposit.argtypes = [P(OrcGrid), P(OrcSpecies), P(OrcParticles), P(OrcField), ctypes.c_int]
        L.orc_esirkepov_one.argtypes = [P(OrcGrid), ctypes.c_int, vp, vp, vp, ctypes.c_float, P(OrcField)]
        L.orc_yee_b_half_open.argtypes = [P(OrcGrid), vp, P(OrcField), P(OrcField), vp, ctypes.c_int]
        L.orc_yee_e_open.argtypes = [P(OrcGrid), vp, P(OrcField), P(OrcField), vp]
        L.orc_emz_one.argtypes = [P(OrcGrid), ctypes.c_int, vp, vp, vp, ctypes.c_float, P(OrcField)]
        L.orc_step.argtypes = [
            P(OrcGrid),
            ctypes.c_int,
            P(OrcSpecies),
            P(OrcParticles),
            P(OrcField),
            P(OrcField),
            P(OrcField),
            ctypes.c_int,
        ]
        L.orc_step_f64.argtypes = [P(OrcGrid), ctypes.c_int, P(OrcSpecies), P(OrcParticles64), P(OrcField),
                                   P(OrcField), P(OrcField), ctypes.c_int]
        L.orc_charge_density.argtypes = [P(OrcGrid), P(OrcSpecies), P(OrcParticles), vp]
        L.orc_charge_residual.restype = ctypes.c_double
        L.orc_charge_residual.argtypes = [P(OrcGrid), P(OrcField), vp, vp]
        L.orc_kinetic_energy.restype = ctypes.c_double
        L.orc_kinetic_energy.argtypes = [P(OrcGrid), P(OrcSpecies), P(OrcParticles)]
        L.orc_field_energy.argtypes = [P(OrcGrid), P(OrcField), P(OrcField), vp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


# ----------------------------------------------------------------- helpers
def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"], "arrays handed to the oracle must be C-contiguous"
    return a.ctypes.data


def grid(g) -> OrcGrid:
    """Build the ctypes grid from any object/dict with nx..eps0 attributes."""
    get = (lambda k: g[k]) if isinstance(g, dict) else (lambda k: getattr(g, k))
    opn = g.get("open", 0) if isinstance(g, dict) else getattr(g, "open", 0)
    return OrcGrid(*[int(get(k)) for k in ("nx", "ny", "nz", "sx", "sy", "sz")],
                   *[float(get(k)) for k in ("dx", "dy", "dz", "dt", "c", "eps0")], int(opn))


def pml(cells, sigma_max, kappa_max, alpha_max, order=4.0, alpha_order=1.0) -> OrcPml:
    """PML parameters: cells[a] = (negative, positive) thickness, per-axis sigma/kappa/alpha maxima."""
    p = OrcPml()
    for a in range(3):
        p.cells[a][0], p.cells[a][1] = int(cells[a][0]), int(cells[a][1])
        p.sigma_max[a], p.kappa_max[a], p.alpha_max[a] = float(sigma_max[a]), float(kappa_max[a]), float(alpha_max[a])
    p.order, p.alpha_order = float(order), float(alpha_order)
    return p


def _psi(psi: np.ndarray):
    assert psi.dtype == np.float32 and psi.shape[0] == 6 and psi.flags["C_CONTIGUOUS"]
    return (ctypes.c_void_p * 6)(*[psi[k].ctypes.data for k in range(6)])


def yee_b_half_open(g, p: OrcPml, E, B, psiB, update: bool):
    lib().orc_yee_b_half_open(grid(g), ctypes.byref(p), field(E), field(B), _psi(psiB), int(bool(update)))


def yee_e_open(g, p: OrcPml, B, E, psiE):
    lib().orc_yee_e_open(grid(g), ctypes.byref(p), field(B), field(E), _psi(psiE))


def species(s) -> OrcSpecies:
    get = (lambda k: s[k]) if isinstance(s, dict) else (lambda k: getattr(s, k))
    return OrcSpecies(float(get("charge")), float(get("mass")), int(get("shape")),
                      int(get("pusher")), int(get("current")))


def field(F: np.ndarray) -> OrcField:
    assert F.dtype == np.float32 and F.shape[0] == 3 and F.flags["C_CONTIGUOUS"]
    f = OrcField()
    for d in range(3):
        f.c[d] = F[d].ctypes.data
    return f


def particles(p: dict) -> OrcParticles:
    for k, dt in (("pos", np.float32), ("mom", np.float32), ("w", np.float32), ("sc", np.int32),
                  ("lcell", np.uint16)):
        assert p[k].dtype == dt and p[k].flags["C_CONTIGUOUS"], k
    o = OrcParticles()
    o.n = p["w"].shape[0]
    for d in range(3):
        o.pos[d] = p["pos"][d].ctypes.data
        o.mom[d] = p["mom"][d].ctypes.data
    o.w = _ptr(p["w"])
    o.sc = _ptr(p["sc"])
    o.lcell = _ptr(p["lcell"])
    return o


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def incident_face(g, axis, direction, surface, polarisation, a0, wavelength, waist, pulse_duration, time_shift,
                  laser_phase, focus_position, e_over_m=1.0, propagation=None, polarisation_vector=None,
                  circular=False, time_delay=0.0, laguerre_modes=None, laguerre_phases=None, profile=0,
                  ramp_init=0.0, plateau=0.0, pulse_init=0.0, waist_axis=None):
    """One incident-field face in the reference's parameters (profiles/BaseParam.def,
    GaussianPulse.def): the propagation direction is `propagation` (DIRECTION_*) or the face
    normal, the E polarisation `polarisation_vector` (POLARISATION_DIRECTION_*) or the unit vector
    along the transverse axis `polarisation` (0: the first of the two other axes in increasing
    order, 1: the second), focus_position is absolute (length units), pulse_duration the rms
    duration of the intensity (PULSE_DURATION), time_shift = -PULSE_INIT * PULSE_DURATION / 2, and
    the phase velocity solves the Yee dispersion relation along the direction
    (calculatePhaseVelocity.hpp) by bisection."""
    import math
    f = OrcIncidentFace()
    f.axis, f.dir, f.surface = int(axis), int(direction), int(surface)
    t = [d for d in range(3) if d != axis]
    dv = list(propagation) if propagation is not None else [float(direction) if d == axis else 0.0 for d in range(3)]
    pv = list(polarisation_vector) if polarisation_vector is not None else [1.0 if d == t[polarisation] else 0.0
                                                                             for d in range(3)]
    for d in range(3):
        f.dirv[d], f.polv[d], f.focus[d] = float(dv[d]), float(pv[d]), float(focus_position[d])
    f.circular = int(bool(circular))
    c, dt = float(g["c"]), float(g["dt"])
    h = [float(g["dx"]), float(g["dy"]), float(g["dz"])]
    omega = 2 * math.pi * c / wavelength
    rhs = (math.sin(omega * dt / 2) / (c * dt)) ** 2
    lhs = lambda k: sum((math.sin(k * dv[a] * h[a] / 2) / h[a]) ** 2 for a in range(3))
    lo, hi = 0.0, math.pi / max(abs(dv[a]) * h[a] for a in range(3))
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        lo, hi = (mid, hi) if lhs(mid) < rhs else (lo, mid)
    f.phase_velocity = omega / (0.5 * (lo + hi))
    f.amplitude = a0 * omega * c / e_over_m
    f.wavelength, f.w0, f.pulse_duration = wavelength, waist, pulse_duration
    f.time_shift, f.laser_phase = time_shift, laser_phase
    f.time_delay = time_delay  # TIME_DELAY
    modes = list(laguerre_modes) if laguerre_modes else [1.0]  # laguerreModes, laguerrePhases
    phases = list(laguerre_phases) if laguerre_phases else [0.0] * len(modes)
    f.nmodes = len(modes)
    for m in range(len(modes)):
        f.modes[m], f.mode_phases[m] = modes[m], phases[m]
    f.profile, f.ramp_init, f.nofocus = int(profile), ramp_init, plateau  # PlaneWave: RAMP_INIT, LASER_NOFOCUS_CONSTANT
    f.pulse_init = pulse_init  # Wavepacket PULSE_INIT
    f.w0_axis1, f.w0_axis2 = waist_axis if waist_axis else (waist, waist)  # W0_AXIS_1, W0_AXIS_2
    return f


def incident_update(g, face: OrcIncidentFace, F, update_b: bool, t: float):
    """TF/SF correction of one face (incidentField/Solver.kernel) after a B half step
    (update_b, incident E at t) or the E step (incident B at t), in place on F."""
    lib().orc_incident_update(grid(g), ctypes.byref(face), field(F), int(bool(update_b)), float(t))


def yee_b_half(g, E, B):
    lib().orc_yee_b_half(grid(g), field(E), field(B))


def yee_e(g, B, E):
    lib().orc_yee_e(grid(g), field(B), field(E))


def add_current(g, J, E):
    lib().orc_add_current(grid(g), field(J), field(E))


def push(g, s, p, E, B):
    lib().orc_push(grid(g), species(s), particles(p), field(E), field(B))


def deposit(g, s, p, J, threads: int = 1):
    lib().orc_deposit(grid(g), species(s), particles(p), field(J), int(threads))


def esirkepov_one(g, shape, cell, pos, vel, charge, J):
    cell = np.ascontiguousarray(cell, dtype=np.int32)
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    vel = np.ascontiguousarray(vel, dtype=np.float32)
    lib().orc_esirkepov_one(grid(g), int(shape), _ptr(cell), _ptr(pos), _ptr(vel), float(charge), field(J))


def emz_one(g, shape, cell, pos, vel, charge, J):
    cell = np.ascontiguousarray(cell, dtype=np.int32)
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    vel = np.ascontiguousarray(vel, dtype=np.float32)
    lib().orc_emz_one(grid(g), int(shape), _ptr(cell), _ptr(pos), _ptr(vel), float(charge), field(J))


def step(g, species_list, plist, E, B, J, threads: int = 1):
    n = len(species_list)
    S = (OrcSpecies * n)(*[species(s) for s in species_list])
    P = (OrcParticles * n)(*[particles(p) for p in plist])
    lib().orc_step(grid(g), n, S, P, field(E), field(B), field(J), int(threads))


def _field64(F: np.ndarray) -> OrcField:
    assert F.dtype == np.float64 and F.shape[0] == 3 and F.flags["C_CONTIGUOUS"]
    f = OrcField()
    for d in range(3):
        f.c[d] = F[d].ctypes.data
    return f


def _particles64(p: dict) -> OrcParticles64:
    for k, dt in (("pos", np.float64), ("mom", np.float64), ("w", np.float64), ("sc", np.int32),
                  ("lcell", np.uint16)):
        assert p[k].dtype == dt and p[k].flags["C_CONTIGUOUS"], k
    o = OrcParticles64()
    o.n = p["w"].shape[0]
    for d in range(3):
        o.pos[d] = p["pos"][d].ctypes.data
        o.mom[d] = p["mom"][d].ctypes.data
    o.w = _ptr(p["w"])
    o.sc = _ptr(p["sc"])
    o.lcell = _ptr(p["lcell"])
    return o


def step_f64(g, species_list, plist, E, B, J, threads: int = 1):
    """One step of the FP64 instantiation: particles and fields as float64 arrays (in place)."""
    n = len(species_list)
    S = (OrcSpecies * n)(*[species(s) for s in species_list])
    P = (OrcParticles64 * n)(*[_particles64(p) for p in plist])
    lib().orc_step_f64(grid(g), n, S, P, _field64(E), _field64(B), _field64(J), int(threads))


def gather(g, shape, F, is_b, cell, pos):
    cell = np.ascontiguousarray(cell, dtype=np.int32)
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    out = np.zeros(3, np.float32)
    lib().orc_gather(grid(g), int(shape), field(F), int(bool(is_b)), _ptr(cell), _ptr(pos), _ptr(out))
    return out


def charge_density(g, s, p, rho):
    lib().orc_charge_density(grid(g), species(s), particles(p), _ptr(rho))


def charge_residual(g, E, rho):
    out = np.zeros_like(rho)
    m = lib().orc_charge_residual(grid(g), field(E), _ptr(rho), _ptr(out))
    return m, out


def kinetic_energy(g, s, p) -> float:
    return lib().orc_kinetic_energy(grid(g), species(s), particles(p))


def field_energy(g, E, B):
    out = np.zeros(2, np.float64)
    lib().orc_field_energy(grid(g), field(E), field(B), _ptr(out))
    return out


def move_particle(g, pos, lcell):
    pos = np.array(pos, dtype=np.float32)
    lc = np.array([lcell], dtype=np.uint16)
    d = np.zeros(3, np.int32)
    mm = lib().orc_move_particle(grid(g), _ptr(pos), _ptr(lc), _ptr(d))
    return pos, int(lc[0]), int(mm), d
