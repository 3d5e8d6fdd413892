"""openPMD checkpoint files of the PIC state (the reference's Checkpoint and openPMD
plugins, plugins/Checkpoint.x.cpp and plugins/openPMD/openPMDWriter.hpp).

One iteration is the directory ``<dir>/simData_<step>/``: the series index
``simData_<step>.json`` holds the openPMD 1.1.0 tree (ED-PIC extension) in the
attribute/dataset form of openPMD-api's JSON backend, and the large datasets live
beside it as raw little-endian C-order files named by ``"external"``.

``write`` and ``read_species_for_grid`` go through the C-ABI's host-side writer and
reader (no device work).  ``read_index``, ``read_mesh`` and ``read_species`` read the
files with numpy alone, following only the openPMD tree, as an independent reader.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

from . import _lib as L

DTYPES = {"FLOAT": np.float32, "DOUBLE": np.float64, "INT": np.int32, "UINT": np.uint32, "ULONG": np.uint64,
          "LONG": np.int64}


def iteration_dir(directory: str, step: int) -> str:
    return os.path.join(directory, f"simData_{int(step)}")


def read_index(directory: str, step: int) -> dict:
    with open(os.path.join(iteration_dir(directory, step), f"simData_{int(step)}.json")) as f:
        return json.load(f)


def _dataset(directory: str, step: int, node: dict) -> np.ndarray:
    dt = np.dtype(DTYPES[node["datatype"]]).newbyteorder("<")
    if "data" in node:
        return np.asarray(node["data"], dtype=dt)
    path = os.path.join(iteration_dir(directory, step), node["external"])
    return np.fromfile(path, dtype=dt).reshape([int(e) for e in node["extent"]])


def _iteration(index: dict, step: int) -> dict:
    return index["data"][str(int(step))]


def read_mesh(directory: str, step: int, name: str) -> np.ndarray:
    """Mesh ``name`` as a (3, nz, ny, nx) float32 array."""
    it = _iteration(read_index(directory, step), step)
    m = it["meshes"][name]
    return np.stack([_dataset(directory, step, m[c]) for c in "xyz"])


def read_species(directory: str, step: int, name: str) -> dict:
    """Species ``name``: in-cell ``pos`` (3, n), global cell ``cell`` (3, n), ``mom`` (3, n), ``w``,
    ``id`` when stored, and the constant records ``charge`` and ``mass``."""
    it = _iteration(read_index(directory, step), step)
    s = it["particles"][name]
    out = dict(pos=np.stack([_dataset(directory, step, s["position"][c]) for c in "xyz"]),
               cell=np.stack([_dataset(directory, step, s["positionOffset"][c]) for c in "xyz"]),
               mom=np.stack([_dataset(directory, step, s["momentum"][c]) for c in "xyz"]),
               w=_dataset(directory, step, s["weighting"]),
               charge=s["charge"]["attributes"]["value"]["value"], mass=s["mass"]["attributes"]["value"]["value"])
    if "id" in s:
        out["id"] = _dataset(directory, step, s["id"])
    return out


def _particles_struct(p: dict, keep: list) -> L.Particles:
    d = L.Particles()
    d.n = int(p["w"].shape[0])
    for k in range(3):
        d.pos[k] = p["pos"][k].ctypes.data
        d.mom[k] = p["mom"][k].ctypes.data
    d.w = p["w"].ctypes.data
    d.sc = p["sc"].ctypes.data
    d.lcell = p["lcell"].ctypes.data
    d.id = p["id"].ctypes.data if p.get("id") is not None else None
    keep.append(p)
    return d


def write(directory: str, step: int, grid, E: np.ndarray, B: np.ndarray, species: list) -> str:
    """Write iteration ``step`` from host arrays through the C-ABI writer.  ``species`` is a
    list of (``Species``, particles in the exchange format) pairs."""
    from .simulation import CURRENTS, PUSHERS, SHAPES

    keep = []
    fields = []
    for F in (E, B):
        a = np.ascontiguousarray(F, dtype=np.float32).reshape(3, grid.nz, grid.ny, grid.nx)
        keep.append(a)
        fields.append((ctypes.c_void_p * 3)(*[a[c].ctypes.data for c in range(3)]))
    arr = (L.OpenPMDSpecies * max(1, len(species)))()
    for i, (sp, p) in enumerate(species):
        q = {k: np.ascontiguousarray(p[k]) for k in ("pos", "mom", "w")}
        q["sc"] = np.ascontiguousarray(p["sc"], dtype=np.int32)
        q["lcell"] = np.ascontiguousarray(p["lcell"], dtype=np.uint16)
        q["id"] = np.ascontiguousarray(p["id"], dtype=np.uint32) if "id" in p else None
        name = sp.name.encode()
        keep.append(name)
        arr[i] = L.OpenPMDSpecies(name, sp.charge, sp.mass, PUSHERS.get(sp.pusher, L.PUSHER_NONE), SHAPES[sp.shape],
                                  CURRENTS[sp.current], _particles_struct(q, keep))
    cfg = grid.config()
    L.call("picgb_openpmd_write", os.fsencode(directory), int(step), ctypes.byref(cfg), fields[0], fields[1],
           len(species), arr)
    return iteration_dir(directory, step)


def read_species_for_grid(directory: str, step: int, name: str, grid, with_ids: bool = False) -> dict:
    """Species ``name`` in the exchange format of ``grid`` (supercell index and cell inside the
    supercell for grid.supercell), through the C-ABI reader."""
    n = ctypes.c_uint64()
    L.call("picgb_openpmd_species_count", os.fsencode(directory), int(step), name.encode(), ctypes.byref(n))
    n = n.value
    p = dict(pos=np.empty((3, n), np.float32), mom=np.empty((3, n), np.float32), w=np.empty(n, np.float32),
             sc=np.empty(n, np.int32), lcell=np.empty(n, np.uint16))
    if with_ids:
        p["id"] = np.empty(n, np.uint32)
    keep = []
    d = _particles_struct(p, keep)
    cfg = grid.config()
    L.call("picgb_openpmd_read_species", os.fsencode(directory), int(step), name.encode(), ctypes.byref(cfg),
           ctypes.byref(d))
    return p
