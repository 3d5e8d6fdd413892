"""Throughput of the PIC cycle in particle-steps/s on GB300 (one JSON line).

Workload (default ``two_stream_256``): 256^3 periodic cells, electrons in two
slabs along y drifting at +-0.2c along x (u_th = 0.005) over a proton
background at the same positions, 16 macro particles per cell per species
(5.4e8 particles), TSC shape, Boris pusher, Esirkepov deposition, Yee solver,
FP32, omega_p dt = 0.1.  A step is one Simulation::runOneStep over all
particles.  ``thermal_32`` is the 32^3 CIC electron-proton thermal plasma.

* value: particle-steps/s with everything resident in HBM, timed with CUDA
  events on the launching stream (max over ranks); the particle arrays
  (21 GB) are far larger than L2, so no flush is needed between steps.
* roofline: the fused push kernel; achieved = algorithmic bytes per launch /
  mean launch time from events recorded around each launch.
* e2e: the same metric through the C-ABI from pinned host buffers: upload of
  both species, K steps each followed by the FP64 energy read-back, download
  of both species.
* cpu_baseline: the CPU oracle (C++, OpenMP, all host threads) on a bounded
  sample of the same workload (64^3 cells, same ppc/shape/solvers).
* --impl reference: that CPU implementation alone, as the reference arm.
Multi-GPU (torchrun): independent replicas, one per GPU (the path is a
single periodic box; it has no exchange step to shard).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "two_stream_256": dict(n=(256, 256, 256), ppc=16, shape="TSC", u_th=0.005, drift=0.2, split=True,
                           sample_n=(64, 64, 64)),
    "thermal_32": dict(n=(32, 32, 32), ppc=4, shape="CIC", u_th=0.01, drift=0.0, split=False,
                       sample_n=(32, 32, 32)),
    # the two-stream workload on 64^3 cells (8.4e6 particles, 270 MB of particle arrays): profiling case
    "two_stream_64": dict(n=(64, 64, 64), ppc=16, shape="TSC", u_th=0.005, drift=0.2, split=True,
                          sample_n=(64, 64, 64)),
    # on 128^3 cells (6.7e7 particles, 2.5 GB): the DRAM-traffic capture, working set ~20x L2
    "two_stream_128": dict(n=(128, 128, 128), ppc=16, shape="TSC", u_th=0.005, drift=0.2, split=True,
                           sample_n=(64, 64, 64)),
}
DT = float(np.float32(0.99 / np.sqrt(3.0)))
MASS_P = 1836.0
# algorithmic bytes: particle read x,u,w,cell (30 B) + write x,u (24 B); per cell and step the
# gather reads E,B (24 B), J is written (12 B), the Yee updates read E,B,J (36 B) and write E,B (24 B)
B_PARTICLE = 54.0
B_CELL = 96.0
B_PUSH_CELL = 36.0  # per push launch: E,B tile read + J write


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def density():
    wp = 0.1 / DT  # omega_p dt = 0.1 with q = m = eps0 = 1
    return wp * wp


def drift_u(beta):
    return beta / np.sqrt(1.0 - beta * beta) if beta else 0.0


# ---------------------------------------------------------------------- CPU sample (oracle)
def numpy_plasma(n, ppc, u_th, drift, split, mass, seed, pos_seed, sc=(8, 8, 4)):
    nx, ny, nz = n
    ncell = nx * ny * nz
    cells = np.repeat(np.arange(ncell, dtype=np.int64), ppc)
    cx, cy, cz = cells % nx, (cells // nx) % ny, cells // (nx * ny)
    nsx, nsy = nx // sc[0], ny // sc[1]
    scidx = (cx // sc[0]) + nsx * ((cy // sc[1]) + nsy * (cz // sc[2]))
    lc = (cx % sc[0]) + sc[0] * ((cy % sc[1]) + sc[1] * (cz % sc[2]))
    pos = np.random.default_rng(pos_seed).random((3, cells.size), dtype=np.float32)
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((3, cells.size), dtype=np.float32) * np.float32(u_th)
    ud = drift_u(drift)
    if ud:
        u[0] += np.where(cy < ny // 2, ud, -ud).astype(np.float32) if split else np.float32(ud)
    w = np.float32(density() / ppc)
    mom = (u * np.float32(mass * w)).astype(np.float32)
    return dict(pos=np.ascontiguousarray(pos), mom=np.ascontiguousarray(mom), w=np.full(cells.size, w, np.float32),
                sc=scidx.astype(np.int32), lcell=lc.astype(np.uint16))


def cpu_sample_rate(wl, steps, warmup, budget_s=20.0):
    """Oracle particle-steps/s on the bounded sample, all host threads."""
    import oracle

    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    n = wl["sample_n"]
    g = dict(nx=n[0], ny=n[1], nz=n[2], sx=8, sy=8, sz=4, dx=1.0, dy=1.0, dz=1.0, dt=DT, c=1.0, eps0=1.0)
    shape = {"CIC": 1, "TSC": 2, "PQS": 3}[wl["shape"]]
    pe = numpy_plasma(n, wl["ppc"], wl["u_th"], wl["drift"], wl["split"], 1.0, 11, 7)
    pi = numpy_plasma(n, wl["ppc"], wl["u_th"] / np.sqrt(MASS_P), 0.0, False, MASS_P, 12, 7)
    se = dict(charge=-1.0, mass=1.0, shape=shape, pusher=0, current=1)
    si = dict(charge=1.0, mass=MASS_P, shape=shape, pusher=0, current=1)
    shp = (3, n[2], n[1], n[0])
    E, B, J = (np.zeros(shp, np.float32) for _ in range(3))
    npart = pe["w"].size + pi["w"].size
    for _ in range(max(warmup, 1)):
        oracle.step(g, [se, si], [pe, pi], E, B, J, threads)
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        oracle.step(g, [se, si], [pe, pi], E, B, J, threads)
        done += 1
        if time.perf_counter() - t0 > budget_s and done >= 1:
            break
    dt = time.perf_counter() - t0
    sample = (f"{n[0]}x{n[1]}x{n[2]} cells, 2x{wl['ppc']} ppc ({npart} particles), {wl['shape']}, {done} steps "
              f"of the oracle step (push, Yee, Esirkepov, J add) on {threads} threads")
    return npart * done / dt, threads, sample


# ---------------------------------------------------------------------- clocks
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "100", "-i",
                 str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = [r.split(", ") for r in out.strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------- replicas
def max_over_ranks(x: float, device: str) -> float:
    """Largest value over the ranks of the default process group (the slowest replica's time)."""
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_rate(npart_per_rank: int, steps: int, ms: float, world: int) -> float:
    """Whole-job particle-steps/s of `world` independent replicas that each advanced npart_per_rank
    particles by `steps` steps, timed by the slowest replica (ms)."""
    return world * npart_per_rank * steps / (ms / 1e3)


# ---------------------------------------------------------------------- GPU arm
def build_sim(pg, wl, device):
    g = pg.Grid(*wl["n"], dt=DT, supercell=(8, 8, 4), device=device)
    sim = pg.Simulation(g)
    sim.add_species(pg.Species("e", -1.0, 1.0, pusher="Boris", shape=wl["shape"], current="Esirkepov"))
    sim.add_species(pg.Species("i", 1.0, MASS_P, pusher="Boris", shape=wl["shape"], current="Esirkepov"))
    return sim


def init_plasma(sim, wl):
    n = density()
    ud = drift_u(wl["drift"])
    if wl["split"]:
        sim.init_plasma("e", wl["ppc"], n, wl["u_th"], drift_lo=(ud, 0, 0), drift_hi=(-ud, 0, 0), split_axis=1,
                        split_cell=wl["n"][1] // 2, seed=1, position_seed=7)
    else:
        sim.init_plasma("e", wl["ppc"], n, wl["u_th"], drift_lo=(ud, 0, 0), seed=1, position_seed=7)
    sim.init_plasma("i", wl["ppc"], n, wl["u_th"] / np.sqrt(MASS_P), seed=2, position_seed=7)


def pinned_like(torch, p):
    out = {}
    for k, v in p.items():
        t = torch.empty(v.shape, dtype=getattr(torch, str(v.dtype)) if str(v.dtype) != "uint16" else torch.int16,
                        pin_memory=True)
        a = t.numpy()
        if str(v.dtype) == "uint16":
            a = a.view(np.uint16)
        a[...] = v
        out[k] = (a, t)
    return {k: a for k, (a, _) in out.items()}, [t for _, t in out.values()]


def run_gpu(args, wl, rank, world, local_rank):
    import torch

    import picongpu_gb300 as pg

    torch.cuda.set_device(local_rank)
    stream = torch.cuda.Stream()
    sim = build_sim(pg, wl, local_rank)
    sim.set_stream(stream.cuda_stream)
    init_plasma(sim, wl)
    npart = sim.particle_count("e") + sim.particle_count("i")
    ncell = wl["n"][0] * wl["n"][1] * wl["n"][2]
    for _ in range(args.warmup):
        sim.step()
    sim.profile(True)
    launches0 = sim.launch_count()
    dist = world > 1
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        sim.step()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = sim.launch_count() - launches0
    kt = sim.kernel_times()
    kinds = sim.deposit_kinds()
    sim.profile(False)
    if dist:
        ms = max_over_ranks(ms, f"cuda:{local_rank}")
        torch.distributed.barrier()
    value = replica_rate(npart, args.steps, ms, world)

    # roofline of the fused push kernel (dominant kernel)
    push_ms, push_n = kt["push"]
    push_bytes = args.steps * (B_PARTICLE * npart + 2 * B_PUSH_CELL * ncell)
    peak, peak_kind = peaks()
    achieved = push_bytes / (push_ms / 1e3) / 1e9 if push_ms > 0 else None
    traffic, traffic_pp = push_traffic(npart / 2, ncell)
    roof = {"kernel": "kPush (gather+Boris+move+Esirkepov+migration, per species)", "bound": "hbm",
            "achieved": round(achieved, 1) if achieved else None, "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4) if achieved else None, "peak_kind": peak_kind,
            "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one kPush launch on the 128^3 "
                              f"two-stream case (33.5e6 particles, {traffic_pp} B each), scaled by the particle count "
                              "(profiles/push_tsc_two_stream_128_dram.md)",
            "algorithmic_bytes_per_launch": (B_PARTICLE * npart + 2 * B_PUSH_CELL * ncell) / 2,
            "mean_launch_ms": push_ms / max(push_n, 1),
            "step_frac_of_peak": round(value / world * (B_PARTICLE + B_CELL / (2 * wl["ppc"])) / (peak * 1e9), 4),
            "kernel_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in kt.items() if v[1]},
            "deposit_short_footprint_frac": round(kinds[0] / max(kinds[0] + kinds[1], 1), 4)}

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, wl, sim, pg, torch, local_rank, world)
    sim.close()
    return dict(value=value, ms=ms, npart=npart, ncell=ncell, roof=roof, clocks=clk, launches=launches, e2e=e2e)


def push_traffic(n_per_launch, ncell):
    """DRAM bytes per push launch from the committed ncu summary of one 128^3 launch (bytes per
    particle), scaled to the launch's particle count, and the bytes per particle; else (None, None)."""
    p = os.path.join(ROOT, "profiles", "push_tsc_two_stream_128_dram.md")
    if not os.path.exists(p):
        return None, None
    for line in open(p):
        if line.startswith("dram_bytes_per_particle:"):
            pp = float(line.split(":")[1])
            return pp * n_per_launch, pp
    return None, None


def run_e2e(args, wl, sim, pg, torch, local_rank, world):
    """Same metric through the C-ABI from pinned host memory (upload, K steps + energies, download)."""
    host = {}
    keep = []
    for name in ("e", "i"):
        p = sim.get_particles(name)
        host[name], ts = pinned_like(torch, p)
        keep += ts
    # the fields from page-locked host memory too
    E0t = torch.empty(sim._field_shape("E"), dtype=torch.float32, pin_memory=True)
    B0t = torch.empty(sim._field_shape("B"), dtype=torch.float32, pin_memory=True)
    E0, B0 = E0t.numpy(), B0t.numpy()
    E0[...] = sim.get_field("E")
    B0[...] = sim.get_field("B")
    keep += [E0t, B0t]
    sim2 = build_sim(pg, wl, local_rank)
    npart = sum(host[n]["w"].size for n in host)
    h2d = sum(a.nbytes for n in host for a in host[n].values()) + E0.nbytes + B0.nbytes
    # set-up outside the timed region: one upload allocates the particle storage and the staging
    # buffer, as a host that reuses a simulation for new inputs has them
    for name in ("e", "i"):
        sim2.set_particles(name, host[name])
    sim2.synchronize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim2.set_field("E", E0)
    sim2.set_field("B", B0)
    t_fields = time.perf_counter()
    t_sp = {}
    for name in ("e", "i"):
        ts0 = time.perf_counter()
        sim2.set_particles(name, host[name])
        t_sp[name] = round(time.perf_counter() - ts0, 4)
    t_up = time.perf_counter()
    for _ in range(args.steps):
        sim2.step()
        sim2.energies()
    t_steps = time.perf_counter()
    d2h = 0
    for name in ("e", "i"):
        out = sim2.get_particles(name, out=host[name])
        d2h += sum(a.nbytes for a in out.values())
    t1 = time.perf_counter()
    dt = t1 - t0
    if world > 1:
        dt = max_over_ranks(dt, f"cuda:{local_rank}")
    d2h += args.steps * 8 * (2 + 2)
    sim2.close()
    del keep
    return {"value": world * npart * args.steps / dt, "unit": "particle-steps/s",
            "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps),
            "wall_s": round(dt, 4),
            "timed": "uploads of both species and E, B from pinned memory, the steps with an FP64 energy read-back "
                     "after each, downloads of both species into pinned memory; the particle storage was allocated "
                     "by one untimed upload before",
            "phases_s": {"upload": round(t_up - t0, 4), "upload_fields": round(t_fields - t0, 4),
                         "upload_species": t_sp, "steps_with_energies": round(t_steps - t_up, 4),
                         "download": round(t1 - t_steps, 4)}}


# ---------------------------------------------------------------------- batched ensemble
EDGES = (16, 24, 32, 48, 64)


def ensemble_boxes(nbox, seed=4):
    """Seeded uneven boxes: edges from EDGES per axis, 4-16 ppc, u_th in [0.005, 0.05],
    omega_p dt in [0.05, 0.2] (the density follows from omega_p with q = m = eps0 = 1)."""
    rng = np.random.default_rng(seed)
    dims = rng.choice(EDGES, size=(nbox, 3))
    ppc = rng.integers(4, 17, size=nbox)
    u_th = rng.uniform(0.005, 0.05, size=nbox)
    wpdt = rng.uniform(0.05, 0.2, size=nbox)
    return dims, ppc, u_th, (wpdt / DT) ** 2


def ensemble_inits(pg, ppc, u_th, dens):
    e = [pg.plasma_init(int(ppc[b]), float(dens[b]), float(u_th[b]), seed=1000 + b, position_seed=5000 + b)
         for b in range(len(ppc))]
    i = [pg.plasma_init(int(ppc[b]), float(dens[b]), float(u_th[b] / np.sqrt(MASS_P)), seed=3000 + b,
                        position_seed=5000 + b) for b in range(len(ppc))]
    return [e, i]


def run_ensemble(args, local_rank):
    """512 boxes, the batched workload with each of its shapes (CIC and TSC): the autotuned
    batched step (one graph launch per step) against the single-box path box by box, both
    over the same number of steps (200 by default, the workload's run length)."""
    import picongpu_gb300 as pg

    dims, ppc, u_th, dens = ensemble_boxes(args.ensemble_boxes)
    ntune = min(64, len(dims))
    out = {"workload": f"{len(dims)} periodic boxes, edges from {list(EDGES)} per axis, 4-16 ppc per species, "
                       f"u_th in [0.005, 0.05], omega_p dt in [0.05, 0.2], CIC and TSC, Boris, Esirkepov, Yee, fp32",
           "cells": int(np.prod(dims, axis=1).sum()), "autotune_boxes": ntune, "unit": "particle-steps/s",
           "steps": args.ensemble_steps,
           "timing": "host clock around run() and run_sequential() with the stream synchronised on both sides; "
                     "every step ends with a status read"}
    for shape in ("TSC", "CIC"):
        species = [pg.Species("e", -1.0, 1.0, shape=shape), pg.Species("i", 1.0, MASS_P, shape=shape)]
        g = pg.Grid(8, 8, 4, dt=DT, device=local_rank)
        if args.no_ensemble_tune:
            sc, th, rates = (8, 8, 4), args.ensemble_threads, {}
        else:
            sc, th, rates = pg.autotune(dims[:ntune], species,
                                        ensemble_inits(pg, ppc[:ntune], u_th[:ntune], dens[:ntune]), grid=g,
                                        warmup=2, steps=3)
        g = pg.Grid(8, 8, 4, dt=DT, supercell=sc, device=local_rank)
        with pg.Ensemble(dims, grid=g, threads=th) as ens:
            for sp in species:
                ens.add_species(sp)
            inits = ensemble_inits(pg, ppc, u_th, dens)
            ens.init_plasma("e", inits[0])
            ens.init_plasma("i", inits[1])
            npart = ens.particle_count()
            ens.run(args.warmup)
            l0 = ens.launch_count()
            t0 = time.perf_counter()
            ens.run(args.ensemble_steps)
            t_batched = time.perf_counter() - t0
            launches = ens.launch_count() - l0
            ens.run_sequential(1)
            t0 = time.perf_counter()
            ens.run_sequential(args.ensemble_steps)
            t_seq = time.perf_counter() - t0
        out[shape] = {"supercell": list(sc), "threads_per_supercell": th,
                      "autotune": {f"{c[0][0]}x{c[0][1]}x{c[0][2]}/{c[1]}": round(r, 1) for c, r in rates.items()},
                      "particles": npart, "value": npart * args.ensemble_steps / t_batched,
                      "plain_sequential": npart * args.ensemble_steps / t_seq, "speedup": t_seq / t_batched,
                      "ms_per_step": 1e3 * t_batched / args.ensemble_steps, "gpu_launches": launches}
    # the headline figures of this leg: the TSC runs
    out.update({k: out["TSC"][k] for k in ("value", "plain_sequential", "speedup", "particles", "ms_per_step")})
    return out


# ---------------------------------------------------------------------- laser-driven wake
LASER_FOCUS = 2 * np.pi * 8.0 ** 2 / 16.0  # two Rayleigh lengths of the waist-8, wavelength-16 beam
def run_laser_wake(args, local_rank):
    """128 x 1024 x 128 cells, a Gaussian pulse (a0 = 2, waist 8, 10 dt FWHM, wavelength 16)
    entering through the TF/SF surface y = 8 into an electron gas at n/n_c = 0.01 (8 ppc) over
    immobile ions; PQS, Boris, Esirkepov, Yee.  By default the configuration's 1500 steps run: the
    warm-up steps untimed, the rest timed.  The gas starts cold, and a particle at rest skips its
    deposit, so the first steps run about twice as fast as the warm gas later in the run."""
    import torch

    import picongpu_gb300 as pg

    n = (128, 1024, 128)
    lam = 16.0
    omega = 2 * np.pi / lam
    dens = 0.01 * omega * omega  # n_c = omega^2 eps0 m / q^2 with eps0 = m = q = 1
    g = pg.Grid(*n, dt=DT, supercell=(8, 8, 4), device=local_rank)
    with pg.Simulation(g) as sim:
        sim.add_species(pg.Species("e", -1.0, 1.0, shape="PQS"))
        sim.add_species(pg.Species("i", 1.0, MASS_P, pusher=None, shape="PQS", current=None))
        sim.init_plasma("e", 8, dens, 0.0, seed=21, position_seed=22)
        sim.init_plasma("i", 8, dens, 0.0, seed=23, position_seed=22)
        fwhm = 10 * DT
        sigma = fwhm / (2 * np.sqrt(np.log(2)))
        sim.set_incident_field(a0=2.0, wavelength=lam, waist=8.0, duration_fwhm=fwhm, t_center=4 * sigma, surface=8,
                               focus=LASER_FOCUS)
        npart = sim.particle_count("e")
        for _ in range(args.warmup):
            sim.step()
        sim.synchronize()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        steps = args.laser_steps if args.laser_steps is not None else max(1500 - args.warmup, 1)
        for _ in range(steps):
            sim.step()
        sim.synchronize()
        dt_wall = time.perf_counter() - t0
        en = sim.energies()
        res, rho = sim.charge_residual()
        # the same residual without the E plane of the TF/SF surface, where the injection of the
        # transverse profile (as the reference's GaussianPulse) carries a divergence of its own
        E = sim.get_field("E")
        rho_g = sim.get_field("FieldTmp0")[0]
        div = ((E[0] - np.roll(E[0], 1, axis=2)) + (E[1] - np.roll(E[1], 1, axis=1))
               + (E[2] - np.roll(E[2], 1, axis=0)))  # unit cells, eps0 = 1
        r = np.abs(div - rho_g)
        r[:, 8, :] = 0.0
        res_away = float(r.max())
        del E, div, r
    e0 = 2.0 * omega  # a0 omega c with m = q = c = 1
    return {"workload": "laser-driven wake: 128x1024x128 cells, e 8 ppc at n/n_c = 0.01 over immobile ions, "
                        "focused Gaussian pulse a0 = 2, waist 8, 10 dt FWHM, wavelength 16, TF/SF surface y = 8, "
                        f"focus {LASER_FOCUS:g} cells beyond it, PQS, Boris, Esirkepov, Yee, fp32",
            "steps": steps, "after_steps": args.warmup + steps, "particles_pushed": npart,
            "value": npart * steps / dt_wall, "unit": "particle-steps/s",
            "ms_per_step": 1e3 * dt_wall / steps, "field_energy": en["E"] + en["B"],
            "electron_energy": en["e"], "charge_residual_over_electron_density": res / dens,
            "charge_residual_off_surface_over_electron_density": res_away / dens,
            "charge_residual_off_surface_over_E0": res_away / e0,
            "timing": "host clock around the steps, stream synchronised on both sides"}


def run_pushers(args, local_rank):
    """The two-stream workload on 128^3 cells with each field pusher: Boris, HigueraCary and Vay
    (the last two with their square-root stages in double, the reference's default).  Host clock
    around the timed steps, stream synchronised on both sides."""
    import picongpu_gb300 as pg

    wl = dict(WORKLOADS["two_stream_256"], n=(128, 128, 128))
    out = {"workload": "two-stream 128^3 cells, 2 species x 16 ppc, TSC, Esirkepov, Yee, fp32 (pusher square "
                       "roots in fp64 for HigueraCary and Vay)", "steps": args.pusher_steps, "unit": "particle-steps/s"}
    for pusher in ("Boris", "HigueraCary", "Vay"):
        g = pg.Grid(*wl["n"], dt=DT, supercell=(8, 8, 4), device=local_rank)
        with pg.Simulation(g) as sim:
            sim.add_species(pg.Species("e", -1.0, 1.0, pusher=pusher, shape=wl["shape"]))
            sim.add_species(pg.Species("i", 1.0, MASS_P, pusher=pusher, shape=wl["shape"]))
            init_plasma(sim, wl)
            npart = sim.particle_count("e") + sim.particle_count("i")
            for _ in range(args.warmup):
                sim.step()
            sim.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.pusher_steps):
                sim.step()
            sim.synchronize()
            dt_wall = time.perf_counter() - t0
        out[pusher] = npart * args.pusher_steps / dt_wall
    return out


def run_thermal(args, local_rank):
    """The reference's Thermal benchmark (share/picongpu/benchmarks/Thermal: 192^3 cells, 25
    electrons per cell at kT = 17.5 mc^2, HigueraCary pusher, PQS shape) with its EmZ and
    Esirkepov variants (cmakeFlags flags[2], flags[5]).  Synthetic seeded start: the
    Temperature manipulator's normal momenta with u_th = sqrt(kT / mc^2).  Host clock around
    the timed steps, stream synchronised on both sides."""
    import picongpu_gb300 as pg

    out = {"workload": "Thermal: 192^3 cells, e 25 ppc, kT = 17.5 mc^2, HigueraCary, PQS, Yee, fp32",
           "steps": args.thermal_steps, "unit": "particle-steps/s"}
    for current in ("EmZ", "Esirkepov"):
        g = pg.Grid(192, 192, 192, dt=DT, supercell=(8, 8, 4), device=local_rank)
        with pg.Simulation(g) as sim:
            sim.add_species(pg.Species("e", -1.0, 1.0, pusher="HigueraCary", shape="PQS", current=current))
            sim.init_plasma("e", 25, density(), float(np.sqrt(17.5)), seed=31, position_seed=32)
            npart = sim.particle_count("e")
            for _ in range(args.warmup):
                sim.step()
            sim.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.thermal_steps):
                sim.step()
            sim.synchronize()
            dt_wall = time.perf_counter() - t0
            ok = sim.device_status() == 0
        out[current] = npart * args.thermal_steps / dt_wall
        out[current + "_status_ok"] = bool(ok)
    out["particles"] = npart
    return out


def run_checkpoint(args, local_rank):
    """openPMD checkpoint write and restart read of the two-stream workload on 64^3 cells
    (E, B and 2 x 4.2e6 particles) to a temporary directory, timed with the host clock
    around the C-ABI calls (device copies and file IO included)."""
    import shutil
    import tempfile

    import picongpu_gb300 as pg

    wl = WORKLOADS["two_stream_64"]
    d = tempfile.mkdtemp(prefix="picgb_ckpt_")
    try:
        sim = build_sim(pg, wl, local_rank)
        with sim:
            init_plasma(sim, wl)
            sim.run(2)
            sim.synchronize()
            t0 = time.perf_counter()
            it = sim.write_checkpoint(d)
            t_write = time.perf_counter() - t0
            nbytes = sum(os.path.getsize(os.path.join(it, f)) for f in os.listdir(it))
            npart = sim.particle_count("e") + sim.particle_count("i")
        sim2 = build_sim(pg, wl, local_rank)
        with sim2:
            t0 = time.perf_counter()
            sim2.read_checkpoint(d, 2)
            sim2.synchronize()
            t_read = time.perf_counter() - t0
            same = sim2.particle_count("e") + sim2.particle_count("i") == npart
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return {"workload": "two-stream 64^3 cells, 2 species x 16 ppc (E, B, positions, cell offsets, momenta, "
                        "weightings)", "bytes": nbytes, "particles": npart, "write_s": t_write, "read_s": t_read,
            "write_GBps": nbytes / t_write / 1e9, "read_GBps": nbytes / t_read / 1e9, "restored_all": bool(same),
            "timing": "host clock around picgb_checkpoint_write / picgb_checkpoint_read"}


# ---------------------------------------------------------------------- differentiable run
def adjoint_case(A, n, ppc, precision, checkpoint_every):
    dens = (0.1 / DT) ** 2
    npart = n ** 3 * ppc
    sp = [A.DiffSpecies("e", -1.0, 1.0, npart), A.DiffSpecies("i", 1.0, MASS_P, npart)]
    pic = A.DiffPIC(n, n, n, sp, dt=DT, shape="TSC", precision=precision, checkpoint_every=checkpoint_every)
    parts = [A.thermal_species(pic, 0, ppc, dens, 0.02, seed=11),
             A.thermal_species(pic, 1, ppc, dens, 0.02 / np.sqrt(MASS_P), seed=12, position_seed=11)]
    return pic, parts


def adjoint_loss(A, torch, pic, parts, a0, waist, steps, n):
    E, B = A.gaussian_pulse(pic, a0, waist, 12.0, 6.0, (n / 4.0, n / 2.0, n / 2.0))
    _, _, out = A.run(pic, steps, E, B, parts)
    return A.kinetic_energy(out[0]["mom"], parts[0]["w"], 1.0)


def run_adjoint(args):
    """64^3 TSC e/p plasma with a Gaussian pulse (a0 = 1, waist 6, wavelength 12): forward and
    adjoint timing over the full run (FP32, checkpoints every 20 steps), the plain single-box
    step on the same plasma, and an FP64 central-difference check of dL/da0 on a shorter run."""
    import torch

    import picongpu_gb300 as pg
    from picongpu_gb300 import adjoint as A

    n, ppc, K = 64, 8, 20
    steps = args.adjoint_steps
    pic, parts = adjoint_case(A, n, ppc, 4, K)
    a0 = torch.tensor(1.0, device="cuda", requires_grad=True)
    waist = torch.tensor(6.0, device="cuda", requires_grad=True)
    # warm-up (builds the kernels' caches and the checkpoint buffers)
    adjoint_loss(A, torch, pic, parts, a0, waist, 2, n).backward()
    a0.grad = None
    waist.grad = None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L = adjoint_loss(A, torch, pic, parts, a0, waist, steps, n)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    L.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    fwd_ms, bwd_ms = 1e3 * (t1 - t0) / steps, 1e3 * (t2 - t1) / steps
    grad_a0 = float(a0.grad)
    pic.close()
    # the plain single-box step on the same plasma (production path)
    g = pg.Grid(n, n, n, dt=DT)
    with pg.Simulation(g) as sim:
        sim.add_species(pg.Species("e", -1.0, 1.0, shape="TSC"))
        sim.add_species(pg.Species("i", 1.0, MASS_P, shape="TSC"))
        dens = (0.1 / DT) ** 2
        sim.init_plasma("e", ppc, dens, 0.02, seed=1, position_seed=7)
        sim.init_plasma("i", ppc, dens, 0.02 / np.sqrt(MASS_P), seed=2, position_seed=7)
        for _ in range(3):
            sim.step()
        sim.synchronize()
        t0 = time.perf_counter()
        for _ in range(20):
            sim.step()
        sim.synchronize()
        plain_ms = 1e3 * (time.perf_counter() - t0) / 20
    # FP64: adjoint against central differences (h = 1e-4 relative) on a shorter run
    fd_steps = args.adjoint_fd_steps
    p64, parts64 = adjoint_case(A, n, ppc, 8, 10)
    a = torch.tensor(1.0, dtype=torch.float64, device="cuda", requires_grad=True)
    w = torch.tensor(6.0, dtype=torch.float64, device="cuda")
    adjoint_loss(A, torch, p64, parts64, a, w, fd_steps, n).backward()
    g64 = float(a.grad)
    h = 1e-4
    with torch.no_grad():
        lp = float(adjoint_loss(A, torch, p64, parts64, torch.tensor(1 + h, dtype=torch.float64, device="cuda"), w,
                                fd_steps, n))
        lm = float(adjoint_loss(A, torch, p64, parts64, torch.tensor(1 - h, dtype=torch.float64, device="cuda"), w,
                                fd_steps, n))
    fd = (lp - lm) / (2 * h)
    p64.close()
    return {"workload": f"{n}^3 cells, TSC, e/p 2 x {ppc} ppc (u_th 0.02), Gaussian pulse a0 = 1, waist 6, "
                        f"wavelength 12 in E/B, loss = electron kinetic energy after {steps} steps, "
                        f"checkpoints every {K} steps, fp32",
            "steps": steps, "loss": float(L.detach()), "grad_a0": grad_a0,
            "forward_ms_per_step": round(fwd_ms, 4), "adjoint_ms_per_step": round(bwd_ms, 4),
            "adjoint_over_forward": round(bwd_ms / fwd_ms, 3),
            "plain_step_ms": round(plain_ms, 4), "adjoint_over_plain_step": round(bwd_ms / plain_ms, 3),
            "fd_check": {"precision": "fp64", "steps": fd_steps, "h_rel": h, "adjoint": g64, "central_difference": fd,
                         "rel_err": abs(g64 - fd) / abs(fd) if fd else None},
            "timing": "host clock around forward and backward with device synchronisation"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="two_stream_256", choices=sorted(WORKLOADS))
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--ensemble-boxes", type=int, default=512)
    ap.add_argument("--ensemble-steps", type=int, default=200)
    ap.add_argument("--no-ensemble-tune", action="store_true",
                    help="8x8x4 supercells and --ensemble-threads threads per supercell, no autotuning")
    ap.add_argument("--ensemble-threads", type=int, default=256, choices=(128, 256, 512),
                    help="threads per supercell of the batched push with --no-ensemble-tune")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-laser", action="store_true")
    ap.add_argument("--laser-steps", type=int, default=None,
                    help="timed steps of the laser-wake leg (default: the configuration's 1500 steps less the warm-up)")
    ap.add_argument("--no-pushers", action="store_true")
    ap.add_argument("--no-checkpoint", action="store_true")
    ap.add_argument("--no-thermal", action="store_true")
    ap.add_argument("--thermal-steps", type=int, default=20)
    ap.add_argument("--pusher-steps", type=int, default=20)
    ap.add_argument("--adjoint-steps", type=int, default=300)
    ap.add_argument("--adjoint-fd-steps", type=int, default=20)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    wl = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    n = wl["n"]
    config = {"workload": f"{args.workload}: {n[0]}x{n[1]}x{n[2]} cells, 2 species x {wl['ppc']} ppc, "
                          f"{wl['shape']}, Boris, Esirkepov, Yee, fp32",
              "cells": list(n), "ppc_per_species": wl["ppc"], "species": ["e (q=-1, m=1)", "i (q=+1, m=1836)"],
              "shape": wl["shape"], "supercell": [8, 8, 4], "dt": DT, "omega_p_dt": 0.1,
              "l2": "inputs larger than L2 (particle SoA of both species streamed every step)",
              "parallelism": f"replicas x{args.gpus}"}
    metric = "particle-steps/s"

    if args.impl == "reference":
        if rank != 0:
            return
        val, cores, sample = cpu_sample_rate(wl, args.steps, args.warmup, budget_s=60.0)
        sn = wl["sample_n"]
        ref_config = dict(config, workload=f"{config['workload']}; the CPU arm times a bounded sample of it: "
                                           f"{sn[0]}x{sn[1]}x{sn[2]} cells with the same ppc, shape, solvers and "
                                           f"distribution (particle-steps/s is per particle, so the rates compare)",
                          sample_cells=list(sn))
        print(json.dumps({"impl": "reference", "metric": metric, "value": val, "unit": metric, "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": ref_config,
                          "cpu_baseline": {"value": val, "unit": metric, "cores": cores, "kind": "port",
                                           "sample": sample},
                          "e2e": {"value": val, "unit": metric, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
              flush=True)
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl", device_id=torch.device(f"cuda:{local_rank}"))
    r = run_gpu(args, wl, rank, world, local_rank)
    if rank != 0:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()
        return
    batched = None
    if not args.no_ensemble:
        batched = run_ensemble(args, local_rank)
    adjoint = None
    if not args.no_adjoint:
        adjoint = run_adjoint(args)
    laser = None
    if not args.no_laser:
        laser = run_laser_wake(args, local_rank)
    pushers = None
    if not args.no_pushers:
        pushers = run_pushers(args, local_rank)
    checkpoint = None
    if not args.no_checkpoint:
        checkpoint = run_checkpoint(args, local_rank)
    thermal = None
    if not args.no_thermal:
        thermal = run_thermal(args, local_rank)
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        val, cores, sample = cpu_sample_rate(wl, 10, 1, budget_s=20.0)
        cpu = {"value": val, "unit": metric, "cores": cores, "kind": "port", "sample": sample}
    line = {"metric": metric, "value": r["value"], "unit": metric, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded device init)", "config": config,
            "particles": r["npart"], "roofline": r["roof"], "cpu_baseline": cpu, "e2e": r["e2e"],
            "clocks": r["clocks"], "gpu_launches": r["launches"], "batched": batched, "adjoint": adjoint,
            "laser_wake": laser, "pushers": pushers, "checkpoint": checkpoint, "thermal": thermal}
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
