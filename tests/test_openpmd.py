"""openPMD checkpoint files on the host (no GPU): the C-ABI writer against an independent
numpy reader that follows only the openPMD tree, the C-ABI reader's round trip (also onto
another supercell size), the openPMD 1.1.0 / ED-PIC attributes the reference's openPMD
plugin writes (plugins/openPMD/openPMDWriter.hpp), and the error paths."""
import ctypes
import json
import os

import numpy as np
import pytest

import picongpu_gb300 as pg
from picongpu_gb300 import openpmd
from plasma import global_cells, random_field, random_particles


def _state(seed=3):
    g = pg.Grid(16, 16, 8, dx=1.0, dy=0.5, dz=0.25, dt=0.1)
    gd = g.as_dict()
    rng = np.random.default_rng(seed)
    E, B = random_field(gd, rng), random_field(gd, rng)
    pe = random_particles(gd, 3, rng, u_th=0.1)
    pi = random_particles(gd, 2, rng, u_th=0.01, mass=1836.0)
    del pi["id"]
    se = pg.Species("e", -1.0, 1.0, pusher="Vay", shape="TSC", with_ids=True)
    si = pg.Species("i", 1.0, 1836.0, pusher="HigueraCary", shape="PQS", current="EmZ")
    return g, E, B, [(se, pe), (si, pi)]


def _attr(node, name):
    return node["attributes"][name]["value"]


def test_index_attributes_and_numpy_reader(tmp_path):
    g, E, B, species = _state()
    d = str(tmp_path / "ckpt")
    it_dir = openpmd.write(d, 7, g, E, B, species)
    assert os.path.isdir(it_dir)
    idx = openpmd.read_index(d, 7)
    assert _attr(idx, "openPMD") == "1.1.0"
    assert _attr(idx, "openPMDextension") == 1
    assert _attr(idx, "basePath") == "/data/%T/"
    assert _attr(idx, "meshesPath") == "meshes/" and _attr(idx, "particlesPath") == "particles/"
    assert _attr(idx, "iterationEncoding") == "fileBased" and _attr(idx, "iterationFormat") == "simData_%T"
    it = idx["data"]["7"]
    assert _attr(it, "dt") == pytest.approx(np.float32(0.1)) and _attr(it, "time") == pytest.approx(7 * np.float32(0.1))
    meshes = it["meshes"]
    assert _attr(meshes, "fieldSolver") == "Yee"
    stag = {"E": {"x": [0, 0, 0.5], "y": [0, 0.5, 0], "z": [0.5, 0, 0]},
            "B": {"x": [0.5, 0.5, 0], "y": [0.5, 0, 0.5], "z": [0, 0.5, 0.5]}}
    units = {"E": [1, 1, -3, -1, 0, 0, 0], "B": [0, 1, -2, -1, 0, 0, 0]}
    for name, F in (("E", E), ("B", B)):
        m = meshes[name]
        assert _attr(m, "geometry") == "cartesian" and _attr(m, "dataOrder") == "C"
        assert _attr(m, "axisLabels") == ["z", "y", "x"]
        assert _attr(m, "gridSpacing") == [0.25, 0.5, 1.0]
        assert _attr(m, "unitDimension") == units[name]
        for c in "xyz":
            assert _attr(m[c], "position") == stag[name][c]
            assert m[c]["extent"] == [8, 16, 16] and m[c]["datatype"] == "FLOAT"
        assert np.array_equal(openpmd.read_mesh(d, 7, name), F)
    gd = g.as_dict()
    for sp, p in species:
        s = it["particles"][sp.name]
        assert _attr(s, "particlePush") == sp.pusher
        assert _attr(s, "particleShape") == {"TSC": 2, "PQS": 3}[sp.shape]
        assert _attr(s, "currentDeposition") == sp.current
        assert _attr(s["position"], "unitDimension") == [1, 0, 0, 0, 0, 0, 0]
        assert [_attr(s["position"][c], "unitSI") for c in "xyz"] == [1.0, 0.5, 0.25]
        assert _attr(s["momentum"], "macroWeighted") == 1 and _attr(s["momentum"], "weightingPower") == 1
        n = p["w"].size
        assert s["particlePatches"]["numParticles"]["data"] == [n]
        assert [s["particlePatches"]["extent"][c]["data"][0] for c in "xyz"] == [16, 16, 8]
        q = openpmd.read_species(d, 7, sp.name)
        assert np.array_equal(q["pos"], p["pos"]) and np.array_equal(q["mom"], p["mom"])
        assert np.array_equal(q["w"], p["w"])
        assert np.array_equal(q["cell"], global_cells(gd, p))
        assert q["charge"] == sp.charge and q["mass"] == sp.mass
        assert ("id" in q) == ("id" in p)
        if "id" in p:
            assert np.array_equal(q["id"], p["id"])


@pytest.mark.parametrize("supercell", [(8, 8, 4), (4, 4, 4)])
def test_c_reader_round_trip(tmp_path, supercell):
    """The C-ABI reader returns the written particles; onto another supercell size it
    recomputes (supercell, cell) from the global cell."""
    g, E, B, species = _state(seed=5)
    d = str(tmp_path / "ckpt")
    openpmd.write(d, 0, g, E, B, species)
    g2 = pg.Grid(16, 16, 8, dx=1.0, dy=0.5, dz=0.25, dt=0.1, supercell=supercell)
    for sp, p in species:
        q = openpmd.read_species_for_grid(d, 0, sp.name, g2, with_ids="id" in p)
        for k in ("pos", "mom", "w"):
            assert np.array_equal(q[k], p[k]), k
        assert np.array_equal(global_cells(g2.as_dict(), q), global_cells(g.as_dict(), p))
        if supercell == (8, 8, 4):
            assert np.array_equal(q["sc"], p["sc"]) and np.array_equal(q["lcell"], p["lcell"])
    Eh = np.empty_like(E)
    ptrs = (ctypes.c_void_p * 3)(*[Eh[c].ctypes.data for c in range(3)])
    cfg = g2.config()
    assert pg.load().picgb_openpmd_read_mesh(os.fsencode(d), 0, b"E", ctypes.byref(cfg), ptrs) == 0
    assert np.array_equal(Eh, E)


def test_error_paths(tmp_path):
    g, E, B, species = _state()
    d = str(tmp_path / "ckpt")
    openpmd.write(d, 2, g, E, B, species)
    with pytest.raises(pg.PicError) as e:  # no such iteration
        openpmd.read_species_for_grid(d, 3, "e", g)
    assert e.value.code == pg._lib.ERR_IO
    with pytest.raises(pg.PicError) as e:  # no such species
        openpmd.read_species_for_grid(d, 2, "x", g)
    assert e.value.code == pg._lib.ERR_NOT_FOUND
    with pytest.raises(pg.PicError) as e:  # the ions carry no ids
        openpmd.read_species_for_grid(d, 2, "i", g, with_ids=True)
    assert e.value.code == pg._lib.ERR_NOT_FOUND
    with pytest.raises(pg.PicError) as e:  # a smaller grid than the file's
        openpmd.read_species_for_grid(d, 2, "e", pg.Grid(8, 8, 8, dt=0.1))
    assert e.value.code == pg._lib.ERR_IO
    with pytest.raises(pg.PicError) as e:  # names become file names: no path separators
        openpmd.write(d, 4, g, E, B, [(pg.Species("a/b", -1.0, 1.0), species[0][1])])
    assert e.value.code == pg._lib.ERR_INVALID
    # a truncated dataset file
    f = os.path.join(openpmd.iteration_dir(d, 2), "particles_e_weighting.bin")
    with open(f, "r+b") as fh:
        fh.truncate(8)
    with pytest.raises(pg.PicError) as e:
        openpmd.read_species_for_grid(d, 2, "e", g)
    assert e.value.code == pg._lib.ERR_IO
    # an index that is not JSON
    idx = os.path.join(openpmd.iteration_dir(d, 2), "simData_2.json")
    with open(idx, "w") as fh:
        fh.write('{"attributes": {"openPMD": ')
    with pytest.raises(pg.PicError) as e:
        openpmd.read_species_for_grid(d, 2, "i", g)
    assert e.value.code == pg._lib.ERR_IO


def test_index_is_valid_json_with_escapes(tmp_path):
    """The index parses as standard JSON, and the C reader parses what the writer wrote
    after a round trip through Python's json (reordered whitespace, same values)."""
    g, E, B, species = _state()
    d = str(tmp_path / "ckpt")
    openpmd.write(d, 1, g, E, B, species)
    idx_path = os.path.join(openpmd.iteration_dir(d, 1), "simData_1.json")
    with open(idx_path) as fh:
        idx = json.load(fh)
    idx["attributes"]["comment"] = {"datatype": "STRING", "value": "quote \" backslash \\ tab \t unicode é"}
    with open(idx_path, "w") as fh:
        json.dump(idx, fh, indent=None, separators=(",", ":"))
    q = openpmd.read_species_for_grid(d, 1, "e", g, with_ids=True)
    assert np.array_equal(q["id"], species[0][1]["id"])
