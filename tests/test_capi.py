"""The C-ABI library builds, loads without a GPU and exports every symbol of include/picgb.h."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "picgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|uint64_t)\s+(picgb_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from picongpu_gb300 import _lib

    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "picgb_step" in names and "picgb_create" in names and len(names) >= 25


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    from picongpu_gb300 import _lib

    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_abi_version(lib):
    assert lib.picgb_abi_version() == 1


def test_struct_sizes_match_header():
    """Layouts of the ctypes mirrors, checked against the C compiler's view of picgb.h."""
    import ctypes
    import subprocess
    import tempfile

    from picongpu_gb300 import _lib

    prog = r"""
#include <stdio.h>
#include "picgb.h"
int main(void){printf("%zu %zu %zu %zu %zu %zu\n", sizeof(picgb_grid_config), sizeof(picgb_species_config),
 sizeof(picgb_particles), sizeof(picgb_buffer_desc), sizeof(picgb_plasma_init), sizeof(picgb_ensemble_config));
 printf("%zu %zu %zu %zu\n", sizeof(picgb_diff_config), sizeof(picgb_diff_species), sizeof(picgb_diff_state),
 sizeof(picgb_incident_field));
 printf("%zu %zu\n", sizeof(picgb_openpmd_species), sizeof(picgb_boundary_config));
 return 0;}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        open(c, "w").write(prog)
        exe = os.path.join(d, "s")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        sizes = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    mine = [ctypes.sizeof(t) for t in (_lib.GridConfig, _lib.SpeciesConfig, _lib.Particles, _lib.BufferDesc,
                                       _lib.PlasmaInit, _lib.EnsembleConfig, _lib.DiffConfig, _lib.DiffSpecies,
                                       _lib.DiffState, _lib.IncidentField, _lib.OpenPMDSpecies, _lib.BoundaryConfig)]
    assert mine == sizes


def test_errors_are_reported_not_raised(lib):
    """Without a usable device the library returns a status and a message (no abort, no CPU fallback)."""
    import ctypes

    import picongpu_gb300 as pg

    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(pg.PicError) as e:
        pg.Simulation(pg.Grid(16, 16, 8))
    assert e.value.code in (pg._lib.ERR_CUDA, pg._lib.ERR_INVALID)
    with pytest.raises(pg.PicError):
        pg.Ensemble([(16, 16, 8), (24, 16, 8)])
    assert lib.picgb_step(None, 0) == pg._lib.ERR_INVALID
    assert lib.picgb_ensemble_run(None, 1) == pg._lib.ERR_INVALID
    assert b"null" in lib.picgb_last_error()
