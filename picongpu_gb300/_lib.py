"""ctypes binding of the C-ABI in include/picgb.h (libpicgb.so, built in-tree).

There is no fallback: if the CUDA library cannot be loaded, every entry point
raises.  Structures mirror picgb.h field by field.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

c_int, c_uint32, c_uint64, c_float, c_double, c_void_p, c_char_p = (
    ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float, ctypes.c_double, ctypes.c_void_p,
    ctypes.c_char_p)
P = ctypes.POINTER

# status codes (enum picgb_status)
OK, ERR_INVALID, ERR_CUDA, ERR_OVERFLOW, ERR_NOT_FOUND, ERR_DUPLICATE, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_LOST, ERR_IO = range(10)
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "OVERFLOW", 4: "NOT_FOUND", 5: "DUPLICATE", 6: "TIMEOUT",
                7: "UNSUPPORTED", 8: "LOST", 9: "IO"}

PUSHER_BORIS, PUSHER_FREE, PUSHER_NONE, PUSHER_HIGUERA_CARY, PUSHER_VAY, PUSHER_PHOTON = 0, 1, 2, 3, 4, 5
SHAPE_NGP, SHAPE_CIC, SHAPE_TSC, SHAPE_PQS, SHAPE_PCS = range(5)
CURRENT_NONE, CURRENT_ESIRKEPOV, CURRENT_EMZ = 0, 1, 2
SOLVER_YEE = 0
SUPERCELL_8x8x4, SUPERCELL_4x4x4, SUPERCELL_8x8x8 = 0, 1, 2
SUPERCELL_SIZES = {0: (8, 8, 4), 1: (4, 4, 4), 2: (8, 8, 8)}
BUFFER_FIELD, BUFFER_SPECIES, BUFFER_OPAQUE = 0, 1, 2


class GridConfig(ctypes.Structure):
    _fields_ = [("nx", c_int), ("ny", c_int), ("nz", c_int), ("supercell", c_int),
                ("dx", c_float), ("dy", c_float), ("dz", c_float), ("dt", c_float), ("c", c_float),
                ("eps0", c_float), ("field_solver", c_int), ("fuse_deposit", c_int), ("device", c_int)]


class SpeciesConfig(ctypes.Structure):
    _fields_ = [("name", c_char_p), ("charge", c_float), ("mass", c_float), ("pusher", c_int), ("shape", c_int),
                ("current", c_int), ("capacity", c_uint32), ("with_ids", c_int)]


class Particles(ctypes.Structure):
    _fields_ = [("n", c_uint64), ("pos", c_void_p * 3), ("mom", c_void_p * 3), ("w", c_void_p), ("sc", c_void_p),
                ("lcell", c_void_p), ("id", c_void_p)]


class OpenPMDSpecies(ctypes.Structure):
    _fields_ = [("name", c_char_p), ("charge", c_float), ("mass", c_float), ("pusher", c_int), ("shape", c_int),
                ("current", c_int), ("particles", Particles)]


class BoundaryConfig(ctypes.Structure):
    _fields_ = [("open", c_int * 3), ("absorber", c_int), ("thickness", (c_int * 2) * 3), ("sigma_max", c_float * 3),
                ("kappa_max", c_float * 3), ("alpha_max", c_float * 3), ("grading_order", c_float),
                ("alpha_grading_order", c_float), ("strength", (c_float * 2) * 3)]


class BufferDesc(ctypes.Structure):
    _fields_ = [("kind", c_int), ("ncomp", c_int), ("ptr", c_void_p * 10), ("dims", ctypes.c_int64 * 3),
                ("stride", ctypes.c_int64 * 3), ("guard", c_int * 3), ("elem_bytes", c_int), ("capacity", c_uint32),
                ("layout", c_int)]


class PlasmaInit(ctypes.Structure):
    _fields_ = [("ppc", c_uint32), ("density", c_float), ("u_th", c_float), ("drift_lo", c_float * 3),
                ("drift_hi", c_float * 3), ("split_axis", c_int), ("split_cell", c_int), ("seed", c_uint64),
                ("position_seed", c_uint64), ("quiet", c_uint32 * 3)]


class IncidentField(ctypes.Structure):
    _fields_ = [("enabled", c_int), ("axis", c_int), ("surface", c_int), ("polarisation", c_int), ("a0", c_float),
                ("e_over_m", c_float), ("wavelength", c_float), ("waist", c_float), ("duration_fwhm", c_float),
                ("t_center", c_float), ("center_x", c_float), ("center_z", c_float), ("phase", c_float),
                ("focus", c_float), ("direction", c_int), ("propagation", c_float * 3),
                ("polarisation_vector", c_float * 3), ("circular", c_int), ("time_delay", c_float),
                ("laguerre_count", c_int), ("laguerre_modes", c_float * 8), ("laguerre_phases", c_float * 8),
                ("profile", c_int), ("ramp_init", c_float), ("plateau", c_float), ("pulse_duration", c_float),
                ("waist_axis", c_float * 2), ("pulse_init", c_float)]


class EnsembleConfig(ctypes.Structure):
    _fields_ = [("grid", GridConfig), ("nbox", c_int), ("dims", P(c_int)), ("threads", c_int)]


DIFF_MAX_SPECIES = 4


class DiffConfig(ctypes.Structure):
    _fields_ = [("nx", c_int), ("ny", c_int), ("nz", c_int), ("dx", c_double), ("dy", c_double), ("dz", c_double),
                ("dt", c_double), ("c", c_double), ("eps0", c_double), ("shape", c_int), ("precision", c_int),
                ("checkpoint_every", c_int), ("device", c_int)]


class DiffSpecies(ctypes.Structure):
    _fields_ = [("charge", c_double), ("mass", c_double), ("n", c_uint64)]


class DiffState(ctypes.Structure):
    _fields_ = [("E", c_void_p), ("B", c_void_p), ("nspecies", c_int), ("cell", c_void_p * DIFF_MAX_SPECIES),
                ("pos", c_void_p * DIFF_MAX_SPECIES), ("mom", c_void_p * DIFF_MAX_SPECIES),
                ("w", c_void_p * DIFF_MAX_SPECIES)]


# (name, restype, argtypes) of every symbol declared in include/picgb.h
SIGNATURES = [
    ("picgb_abi_version", c_int, []),
    ("picgb_last_error", c_char_p, []),
    ("picgb_create", c_int, [P(GridConfig), P(c_void_p)]),
    ("picgb_destroy", c_int, [c_void_p]),
    ("picgb_add_species", c_int, [c_void_p, P(SpeciesConfig), P(c_int)]),
    ("picgb_species_set", c_int, [c_void_p, c_int, P(Particles)]),
    ("picgb_species_count", c_int, [c_void_p, c_int, P(c_uint64)]),
    ("picgb_species_init_plasma", c_int, [c_void_p, c_int, P(PlasmaInit)]),
    ("picgb_species_get", c_int, [c_void_p, c_int, P(Particles)]),
    ("picgb_field_set", c_int, [c_void_p, c_char_p, P(c_void_p)]),
    ("picgb_field_get", c_int, [c_void_p, c_char_p, P(c_void_p)]),
    ("picgb_get_buffer", c_int, [c_void_p, c_char_p, P(BufferDesc)]),
    ("picgb_share", c_int, [c_void_p, c_char_p, P(BufferDesc)]),
    ("picgb_unshare", c_int, [c_void_p, c_char_p]),
    ("picgb_registry_size", c_int, [c_void_p, P(c_int)]),
    ("picgb_registry_name", c_int, [c_void_p, c_int, c_char_p, ctypes.c_size_t]),
    ("picgb_step", c_int, [c_void_p, c_uint32]),
    ("picgb_run", c_int, [c_void_p, c_uint32, c_uint32]),
    ("picgb_stage_current_reset", c_int, [c_void_p]),
    ("picgb_stage_push", c_int, [c_void_p, c_uint32]),
    ("picgb_stage_field_before", c_int, [c_void_p, c_uint32]),
    ("picgb_stage_deposit", c_int, [c_void_p, c_uint32]),
    ("picgb_stage_add_current", c_int, [c_void_p]),
    ("picgb_stage_field_after", c_int, [c_void_p, c_uint32]),
    ("picgb_set_incident_field", c_int, [c_void_p, P(IncidentField)]),
    ("picgb_energies", c_int, [c_void_p, P(c_double), ctypes.c_size_t]),
    ("picgb_charge_residual", c_int, [c_void_p, P(c_double), P(c_double)]),
    ("picgb_set_stream", c_int, [c_void_p, c_void_p]),
    ("picgb_set_sort_interval", c_int, [c_void_p, c_uint32]),
    ("picgb_ensemble_set_sort_interval", c_int, [c_void_p, c_uint32]),
    ("picgb_synchronize", c_int, [c_void_p]),
    ("picgb_launch_count", c_int, [c_void_p, P(c_uint64)]),
    ("picgb_device_status", c_int, [c_void_p, P(c_uint32), c_int]),
    ("picgb_profile_enable", c_int, [c_void_p, c_int]),
    ("picgb_profile_read", c_int, [c_void_p, c_int, P(c_double), P(c_uint64)]),
    ("picgb_profile_deposit_kinds", c_int, [c_void_p, P(c_uint64)]),
    ("picgb_noalloc_max_cells", c_uint64, []),
    ("picgb_noalloc_last_error", c_char_p, []),
    ("picgb_charge_residual_noalloc", c_int,
     [P(GridConfig), P(c_void_p), c_int, P(Particles), P(c_float), P(c_int), c_void_p, P(c_double), P(c_double)]),
    ("picgb_ensemble_create", c_int, [P(EnsembleConfig), P(c_void_p)]),
    ("picgb_ensemble_destroy", c_int, [c_void_p]),
    ("picgb_ensemble_size", c_int, [c_void_p, P(c_int)]),
    ("picgb_ensemble_box", c_int, [c_void_p, c_int, P(c_void_p)]),
    ("picgb_ensemble_add_species", c_int, [c_void_p, P(SpeciesConfig), P(c_int)]),
    ("picgb_ensemble_init_plasma", c_int, [c_void_p, c_int, P(PlasmaInit)]),
    ("picgb_ensemble_run", c_int, [c_void_p, c_uint32]),
    ("picgb_ensemble_run_sequential", c_int, [c_void_p, c_uint32]),
    ("picgb_ensemble_launch_count", c_int, [c_void_p, P(c_uint64)]),
    ("picgb_ensemble_autotune", c_int,
     [P(EnsembleConfig), c_int, P(SpeciesConfig), P(PlasmaInit), c_uint32, c_uint32, P(c_int), P(c_int),
      P(c_double)]),
    ("picgb_openpmd_write", c_int, [c_char_p, c_uint32, P(GridConfig), P(c_void_p), P(c_void_p), c_int,
                                    P(OpenPMDSpecies)]),
    ("picgb_openpmd_species_count", c_int, [c_char_p, c_uint32, c_char_p, P(c_uint64)]),
    ("picgb_openpmd_read_species", c_int, [c_char_p, c_uint32, c_char_p, P(GridConfig), P(Particles)]),
    ("picgb_openpmd_read_mesh", c_int, [c_char_p, c_uint32, c_char_p, P(GridConfig), P(c_void_p)]),
    ("picgb_checkpoint_write", c_int, [c_void_p, c_char_p, c_uint32]),
    ("picgb_set_boundaries", c_int, [c_void_p, P(BoundaryConfig)]),
    ("picgb_checkpoint_read", c_int, [c_void_p, c_char_p, c_uint32]),
    ("picgb_diff_create", c_int, [P(DiffConfig), c_int, P(DiffSpecies), P(c_void_p)]),
    ("picgb_diff_destroy", c_int, [c_void_p]),
    ("picgb_diff_forward", c_int, [c_void_p, P(DiffState), c_uint32, c_void_p]),
    ("picgb_diff_backward", c_int, [c_void_p, P(DiffState), c_void_p]),
    ("picgb_diff_kinetic_energy", c_int, [c_void_p, P(DiffState), c_int, P(c_double), c_void_p]),
]

KERNEL_CLASSES = {"push": 0, "compact": 1, "yee_b": 2, "yee_e": 3, "deposit": 4, "add_current": 5, "reorder": 6}

_lib = None


class PicError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libpicgb.so (building it first if it is absent); raises if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; run picongpu_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(code: int, where: str) -> None:
    if code != OK:
        msg = load().picgb_last_error()
        raise PicError(code, where, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
