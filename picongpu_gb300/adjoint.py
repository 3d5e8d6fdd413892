"""Differentiable PIC runs: the C-ABI adjoint (picgb_diff_*) as a torch.autograd.Function.

``DiffPIC`` owns a handle (grid, shape, precision, checkpoint interval and the
species); ``run(pic, nsteps, E, B, species)`` advances the state on the GPU and
returns the final fields and particles as tensors whose backward pass is the
hand-written adjoint (transposed curls, Jacobian-transposed Boris, deposit and
gather as each other's transposes), replayed from checkpoints every K steps.
Any torch expression of the initial state (a laser pulse built from its
amplitude and waist, say) and of the final state (a kinetic-energy loss) can be
differentiated through it.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

from . import _lib as L
from .simulation import SHAPES


@dataclass
class DiffSpecies:
    name: str
    charge: float
    mass: float
    n: int


class DiffPIC:
    def __init__(self, nx, ny, nz, species: list[DiffSpecies], dt=0.99 / math.sqrt(3.0), dx=1.0, dy=1.0, dz=1.0,
                 c=1.0, eps0=1.0, shape="TSC", precision=4, checkpoint_every=20, device=0):
        if len(species) > L.DIFF_MAX_SPECIES:
            raise ValueError(f"at most {L.DIFF_MAX_SPECIES} species")
        self.shape = (nz, ny, nx)
        self.dt, self.c, self.eps0 = dt, c, eps0
        self.cell = (dx, dy, dz)
        self.species = list(species)
        self.precision = precision
        self.device = device
        cfg = L.DiffConfig(nx, ny, nz, dx, dy, dz, dt, c, eps0, SHAPES[shape], precision, checkpoint_every, device)
        sp = (L.DiffSpecies * max(len(species), 1))(*[L.DiffSpecies(s.charge, s.mass, s.n) for s in species])
        h = ctypes.c_void_p()
        L.call("picgb_diff_create", ctypes.byref(cfg), len(species), sp, ctypes.byref(h))
        self.handle = h
        self.generation = 0  # forward runs so far: a backward pass needs the latest one

    @property
    def dtype(self):
        import torch

        return torch.float64 if self.precision == 8 else torch.float32

    def close(self):
        if self.handle:
            L.load().picgb_diff_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def state(self, E, B, cells=None, pos=None, mom=None, w=None) -> L.DiffState:
        st = L.DiffState()
        st.E, st.B = E.data_ptr(), B.data_ptr()
        st.nspecies = len(self.species)
        for k in range(len(self.species)):
            st.cell[k] = cells[k].data_ptr() if cells is not None else None
            st.pos[k] = pos[k].data_ptr()
            st.mom[k] = mom[k].data_ptr()
            st.w[k] = w[k].data_ptr() if w is not None else None
        return st

    def kinetic_energy(self, k: int, mom, w) -> float:
        """FP64 sum of (gamma - 1) m w c^2 of species k (device reduction)."""
        import torch

        st = L.DiffState()
        st.nspecies = len(self.species)
        st.mom[k], st.w[k] = mom.data_ptr(), w.data_ptr()
        out = ctypes.c_double()
        L.call("picgb_diff_kinetic_energy", self.handle, ctypes.byref(st), k, ctypes.byref(out),
               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        return out.value


def _check(pic: DiffPIC, t, shape, name, dtype=None):
    import torch

    if not t.is_cuda or not t.is_contiguous():
        raise ValueError(f"{name}: a contiguous CUDA tensor is needed")
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name}: shape {tuple(t.shape)}, expected {tuple(shape)}")
    if t.dtype != (dtype or pic.dtype):
        raise ValueError(f"{name}: dtype {t.dtype}, expected {dtype or pic.dtype}")
    return torch


class _Run:
    """torch.autograd.Function built lazily (torch is imported on first use)."""

    fn = None

    @classmethod
    def get(cls):
        if cls.fn is not None:
            return cls.fn
        import torch

        class PICRun(torch.autograd.Function):
            @staticmethod
            def forward(ctx, pic, nsteps, E, B, *flat):
                ns = len(pic.species)
                cells = [flat[4 * k].clone() for k in range(ns)]
                pos = [flat[4 * k + 1].detach().clone() for k in range(ns)]
                mom = [flat[4 * k + 2].detach().clone() for k in range(ns)]
                w = [flat[4 * k + 3].detach() for k in range(ns)]
                E1, B1 = E.detach().clone(), B.detach().clone()
                st = pic.state(E1, B1, cells, pos, mom, w)
                stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
                L.call("picgb_diff_forward", pic.handle, ctypes.byref(st), nsteps, stream)
                pic.generation += 1
                ctx.pic = pic
                ctx.generation = pic.generation
                ctx.keep = w  # the weights must outlive the backward pass
                ctx.mark_non_differentiable(*cells)
                out = [E1, B1]
                for k in range(ns):
                    out += [cells[k], pos[k], mom[k]]
                return tuple(out)

            @staticmethod
            def backward(ctx, gE, gB, *gflat):
                pic = ctx.pic
                if ctx.generation != pic.generation:
                    raise RuntimeError("the handle's checkpoints belong to a later forward run; "
                                       "call backward before the next run() on the same DiffPIC")
                ns = len(pic.species)
                z = torch.zeros
                gE = gE.contiguous().clone() if gE is not None else z((3,) + pic.shape, dtype=pic.dtype, device="cuda")
                gB = gB.contiguous().clone() if gB is not None else z((3,) + pic.shape, dtype=pic.dtype, device="cuda")
                gpos, gmom = [], []
                for k in range(ns):
                    n = pic.species[k].n
                    gp, gm = gflat[3 * k + 1], gflat[3 * k + 2]
                    gpos.append(gp.contiguous().clone() if gp is not None else z((3, n), dtype=pic.dtype, device="cuda"))
                    gmom.append(gm.contiguous().clone() if gm is not None else z((3, n), dtype=pic.dtype, device="cuda"))
                st = pic.state(gE, gB, None, gpos, gmom, None)
                stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
                L.call("picgb_diff_backward", pic.handle, ctypes.byref(st), stream)
                grads = [None, None, gE, gB]
                for k in range(ns):
                    grads += [None, gpos[k], gmom[k], None]
                return tuple(grads)

        cls.fn = PICRun
        return PICRun


def run(pic: DiffPIC, nsteps: int, E, B, species: list[dict]):
    """Differentiable nsteps-step run.  species[k] = {"cell": int32 (3, n), "pos": (3, n), "mom": (3, n),
    "w": (n,)}; returns (E, B, [{"cell", "pos", "mom"} per species]) after the run."""
    import torch

    nz, ny, nx = pic.shape
    _check(pic, E, (3, nz, ny, nx), "E")
    _check(pic, B, (3, nz, ny, nx), "B")
    flat = []
    for k, s in enumerate(species):
        n = pic.species[k].n
        _check(pic, s["cell"], (3, n), "cell", torch.int32)
        for key in ("pos", "mom"):
            _check(pic, s[key], (3, n), key)
        _check(pic, s["w"], (n,), "w")
        flat += [s["cell"], s["pos"], s["mom"], s["w"]]
    out = _Run.get().apply(pic, nsteps, E, B, *flat)
    parts = [{"cell": out[2 + 3 * k], "pos": out[3 + 3 * k], "mom": out[4 + 3 * k]} for k in range(len(species))]
    return out[0], out[1], parts


def kinetic_energy(mom, w, mass: float, c: float = 1.0):
    """Differentiable total (gamma - 1) m w c^2 of one species (torch), with gamma - 1
    written as u^2 / (gamma + 1), u^2 = p^2 / (m w c)^2, so that slow particles keep
    their precision."""
    mw = mass * w
    u2 = (mom * mom).sum(0) / (mw * mw * c * c)
    return (u2 / ((1.0 + u2).sqrt() + 1.0) * mw * c * c).sum()


def gaussian_pulse(pic: DiffPIC, a0, waist, wavelength: float, length: float, center, axis: int = 0):
    """Linearly polarised Gaussian pulse travelling along +x with E along y and B along z,
    evaluated at the Yee positions (fields/YeeCell.hpp:70-131): amplitude a0 (normalised,
    E0 = a0 m c omega / q with m = q = 1), transverse 1/e radius `waist`, longitudinal 1/e
    half length `length`, centred at `center` (cells).  a0 and waist may be tensors
    (gradients flow to them).  Returns E, B of shape (3, nz, ny, nx)."""
    import torch

    if axis != 0:
        raise ValueError("the pulse travels along x")
    nz, ny, nx = pic.shape
    dt = pic.dtype
    dev = "cuda"
    k = 2.0 * math.pi / wavelength
    omega = k * pic.c

    def profile(ox, oy, oz):
        x = (torch.arange(nx, dtype=dt, device=dev) + ox - center[0])[None, None, :]
        y = (torch.arange(ny, dtype=dt, device=dev) + oy - center[1])[None, :, None]
        z = (torch.arange(nz, dtype=dt, device=dev)[:, None, None] + oz - center[2])
        r2 = y * y + z * z
        return torch.exp(-r2 / (waist * waist)) * torch.exp(-(x * x) / (length * length)) * torch.sin(k * x)

    E0 = a0 * omega * pic.c
    E = torch.zeros((3, nz, ny, nx), dtype=dt, device=dev)
    B = torch.zeros((3, nz, ny, nx), dtype=dt, device=dev)
    ey = E0 * profile(0.0, 0.5, 0.0)  # E_y at (0, 1/2, 0)
    bz = E0 / pic.c * profile(0.5, 0.5, 0.0)  # B_z at (1/2, 1/2, 0)
    E = torch.stack([E[0], ey, E[2]])
    B = torch.stack([B[0], B[1], bz])
    return E.contiguous(), B.contiguous()


def thermal_species(pic: DiffPIC, k: int, ppc: int, density: float, u_th: float, seed: int, position_seed=None):
    """Seeded uniform plasma of species k: ppc particles per cell (particle i in cell i mod ncell)
    at uniform in-cell positions,
    momenta u_th * N(0,1) * m w c per component, weighting density * V / ppc."""
    import torch

    nz, ny, nx = pic.shape
    n = nx * ny * nz * ppc
    if pic.species[k].n != n:
        raise ValueError(f"species {k} was declared with {pic.species[k].n} particles, {n} needed")
    gpos = torch.Generator(device="cuda").manual_seed(seed if position_seed is None else position_seed)
    gmom = torch.Generator(device="cuda").manual_seed(seed + 7919)
    # cell of particle k = k mod ncell: the 32 particles of a warp sit in 32 different cells, so
    # the atomics of one instruction (deposit, gather transpose) never hit the same address
    cells = torch.arange(nx * ny * nz, device="cuda", dtype=torch.int64).repeat(ppc)
    cell = torch.stack([cells % nx, (cells // nx) % ny, cells // (nx * ny)]).to(torch.int32).contiguous()
    pos = torch.rand((3, n), generator=gpos, device="cuda", dtype=torch.float64).to(pic.dtype).contiguous()
    dx, dy, dz = pic.cell
    w = torch.full((n,), density * dx * dy * dz / ppc, dtype=pic.dtype, device="cuda")
    mw = pic.species[k].mass * w
    u = torch.randn((3, n), generator=gmom, device="cuda", dtype=torch.float64).to(pic.dtype) * u_th
    mom = (u * mw * pic.c).contiguous()
    return {"cell": cell, "pos": pos, "mom": mom, "w": w}
