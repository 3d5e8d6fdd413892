// Fused particle kernel of one PIC step: form-factor gather of E and B from a
// shared-memory tile, Boris push, moveParticle, Esirkepov deposit into a
// shared-memory J tile, and the supercell migration of leaving particles.
// One thread block per supercell.
//
// Reference path: KernelMoveAndMarkParticles + PushParticlePerFrame
// (particles/Particles.kernel:170-316), KernelComputeCurrent + ComputePerFrame
// (fields/FieldJ.kernel:52-142) and KernelShiftParticles/KernelFillGaps
// (pmacc/particles/ParticlesBase.kernel:61-631).
#pragma once

#include "picgb_device.cuh"
#include "picgb_internal.hpp"

namespace picgb
{
#ifndef PICGB_PUSH_THREADS
    // threads per supercell block of the single-box push kernel: 16 warps, two blocks
    // per SM (two-stream 256^3, TSC, ms per launch: 256 threads 30.7, 448 28.5, 512 27.1)
#    define PICGB_PUSH_THREADS 512
#endif
    constexpr int kPushThreads = PICGB_PUSH_THREADS;
#ifndef PICGB_PUSH_MIN_BLOCKS
    // resident blocks per SM the push kernel's register budget is sized for (64
    // registers at 512 threads, no spills)
#    define PICGB_PUSH_MIN_BLOCKS 2
#endif

    // Per-warp queue of deposit jobs of particles that cross a cell boundary
    // (see kPush): kQueueCap jobs (32 or more) of kJobWords words for every warp.
#ifndef PICGB_QUEUE_CAP
    // 32 keeps the 16 queues of a 512-thread block at 18 KB, so two blocks fit an SM
#    define PICGB_QUEUE_CAP 32
#endif
    constexpr int kQueueCap = PICGB_QUEUE_CAP;

#ifndef PICGB_TILE_PITCH_MIN
    // smallest row and plane pitch (words) of the E/B tiles of 8 x 8 supercell planes
    // (TileGeom); 0 keeps the unpadded widths
#    define PICGB_TILE_PITCH_MIN 12
#endif
#ifndef PICGB_J_PLANE_PAD
#    define PICGB_J_PLANE_PAD 1
#endif
#ifndef PICGB_GATHER_PAIRS
#    define PICGB_GATHER_PAIRS 1 // the six field components gathered in three f32x2 pairs
#endif
#ifndef PICGB_POOL_LEFTOVERS
#    define PICGB_POOL_LEFTOVERS 1 // the warps' leftover deposit jobs drained together after the loop
#endif
    static_assert(kQueueCap >= 32, "a warp drains 32 jobs at a time");
    constexpr int kJobWords = 9;

    template<typename SH, typename SC, int THREADS = kPushThreads>
    struct TileGeom
    {
        static constexpr int GX = SC::SX + SH::gLo + SH::gHi;
        static constexpr int GY = SC::SY + SH::gLo + SH::gHi;
        static constexpr int GZ = SC::SZ + SH::gLo + SH::gHi;
        // Row and plane pitch of the E/B tiles.  With 8 x 8 supercell planes the 32 lanes of
        // a warp gather from 32 cells of an 8 x 4 patch, each shifted by its particle's
        // sub-cell position; a bank-conflict model of that access (random in-cell
        // positions) gives 2.1 shared-memory wavefronts per load with a pitch of 12 words
        // against 2.3 to 2.4 with the unpadded 10 (CIC) and 11 (TSC); PQS (12) and PCS (13)
        // keep their widths, and so do the small 4 x 4 x 4 supercells.
        static constexpr int PX = (SC::SX == 8 && GX < PICGB_TILE_PITCH_MIN) ? PICGB_TILE_PITCH_MIN : GX;
        static constexpr int PY = (SC::SY == 8 && GY < PICGB_TILE_PITCH_MIN) ? PICGB_TILE_PITCH_MIN : GY;
        static constexpr int GT = PX * PY * GZ; // words of one component's tile
        static constexpr int JX = SC::SX + SH::jLo + SH::jHi;
        static constexpr int JY = SC::SY + SH::jLo + SH::jHi;
        static constexpr int JZ = SC::SZ + SH::jLo + SH::jHi;
        // Plane pitch of the J tile.  A deposit instruction of a warp adds at one node
        // offset for 32 particles, whose origins differ by their cells (an 8 x 4 patch in
        // the interleaved order, random after a drift) and, for the odd shapes, by a
        // random shift of 0 or 1 per axis.  With the unpadded planes (225 words for TSC,
        // 1 mod 32) a shift along z lands in the bank of a shift along x.  A bank model
        // of these accesses gives the fewest wavefronts per atomic for plane pitches of
        // 8 mod 16 words: TSC 3.3 (patch) and 3.5 (random cells) against 4.2 and 4.0
        // unpadded, PCS alike, CIC and PQS (no random shift) 3.5 against 3.6 and 4.1 for
        // random cells.  The pitch is the smallest such one above the plane; 4 x 4 x 4
        // supercells keep theirs.
        static constexpr int JP = (SC::SX == 8 && SC::SY == 8 && PICGB_J_PLANE_PAD)
            ? JX * JY + ((8 - JX * JY % 16) + 16) % 16
            : JX * JY;
        static constexpr int JT = JP * JZ;
        // tile word of node (x, y, z), counted from the tile's corner
        __device__ __forceinline__ static int jIndex(int x, int y, int z) { return x + JX * y + JP * z; }
        // E and B tiles, the J tile, the per-warp queues of deposit jobs
        static constexpr int JWords = (PICGB_J_FIXED ? 6 : 3) * JT; // words of the J tile
        static constexpr int QueueWords = (THREADS / 32) * kQueueCap * kJobWords;
        static constexpr size_t pushSmem = sizeof(float) * (6 * GT + JWords) + sizeof(float) * QueueWords;
        static constexpr size_t depositSmem = sizeof(float) * JWords;
    };

    __device__ __forceinline__ void scCoords(int sc, GridParams const& g, int& x, int& y, int& z)
    {
        x = sc % g.nscx;
        y = (sc / g.nscx) % g.nscy;
        z = sc / (g.nscx * g.nscy);
    }

    // Stage a TX x TY x TZ tile of a 3-component SoA field with periodic wrap, stored with
    // row pitch PX and plane pitch PX * PY (component stride PT words).
    template<int TX, int TY, int TZ, int PX, int PY, int PT>
    __device__ __forceinline__ void loadTile(
        float* __restrict__ dst,
        float const* __restrict__ src,
        int ox,
        int oy,
        int oz,
        GridParams const& g,
        size_t ncell)
    {
        bool const anyOpen = g.open != 0; // uniform: the periodic box takes the plain wrap
        for(int e = threadIdx.x; e < TX * TY * TZ; e += blockDim.x)
        {
            int const tx = e % TX, ty = (e / TX) % TY, tz = e / (TX * TY);
            int const t = tx + PX * (ty + PY * tz);
            constexpr int TT = PT;
            int gx, gy, gz;
            if(!anyOpen)
            {
                gx = wrapi(ox + tx, g.nx);
                gy = wrapi(oy + ty, g.ny);
                gz = wrapi(oz + tz, g.nz);
            }
            else
            {
                gx = wrapOrOutside(ox + tx, g.nx, g.open & 1);
                gy = wrapOrOutside(oy + ty, g.ny, g.open & 2);
                gz = wrapOrOutside(oz + tz, g.nz, g.open & 4);
                if((gx | gy | gz) < 0) // beyond an open face the fields are zero
                {
                    dst[t] = dst[TT + t] = dst[2 * TT + t] = 0.0f;
                    continue;
                }
            }
            size_t const gi = size_t(gx) + size_t(g.nx) * (size_t(gy) + size_t(g.ny) * size_t(gz));
            dst[t] = __ldg(src + gi);
            dst[TT + t] = __ldg(src + ncell + gi);
            dst[2 * TT + t] = __ldg(src + 2 * ncell + gi);
        }
    }

    // Add a shared-memory J tile into the global J with periodic wrap (the
    // reference's guard add of FieldJ, FieldJ.x.cpp:156-169, folded in).  Beyond an
    // open face the current is dropped, as the reference's guard current at a
    // non-periodic boundary is.
    template<int TX, int TY, int TP, int TT>
    __device__ __forceinline__ void flushTile(
        float const* __restrict__ Js,
        float* __restrict__ J,
        int ox,
        int oy,
        int oz,
        GridParams const& g,
        size_t ncell,
        JFixed const& f)
    {
        bool const anyOpen = g.open != 0;
        for(int t = threadIdx.x; t < TT; t += blockDim.x)
        {
            float const vx = tileValue<TT>(Js, t, f), vy = tileValue<TT>(Js, TT + t, f),
                        vz = tileValue<TT>(Js, 2 * TT + t, f);
            if(vx == 0.0f && vy == 0.0f && vz == 0.0f)
                continue;
            int const tz = t / TP, ty = (t - tz * TP) / TX, tx = t - tz * TP - ty * TX;
            if(ty >= TY)
                continue; // plane padding (never written)
            int gx, gy, gz;
            if(!anyOpen)
            {
                gx = wrapi(ox + tx, g.nx);
                gy = wrapi(oy + ty, g.ny);
                gz = wrapi(oz + tz, g.nz);
            }
            else
            {
                gx = wrapOrOutside(ox + tx, g.nx, g.open & 1);
                gy = wrapOrOutside(oy + ty, g.ny, g.open & 2);
                gz = wrapOrOutside(oz + tz, g.nz, g.open & 4);
                if((gx | gy | gz) < 0)
                    continue;
            }
            size_t const gi = size_t(gx) + size_t(g.nx) * (size_t(gy) + size_t(g.ny) * size_t(gz));
            if(vx != 0.0f)
                atomicAdd(J + gi, vx);
            if(vy != 0.0f)
                atomicAdd(J + ncell + gi, vy);
            if(vz != 0.0f)
                atomicAdd(J + 2 * ncell + gi, vz);
        }
    }

    __device__ __forceinline__ unsigned laneMaskLt() { return (1u << (threadIdx.x & 31)) - 1u; }

    // Per-warp queue of deposit jobs: trajectory in the virtual coordinate
    // system, charge, tile origin and packed status bits.
    struct WarpQueue
    {
        float* w; // kQueueCap jobs, structure of arrays of kJobWords words

        __device__ __forceinline__ void put(
            int i,
            float const p0[3],
            float const p1[3],
            float q,
            int org,
            int const st[3]) const
        {
#pragma unroll
            for(int d = 0; d < 3; ++d)
            {
                w[d * kQueueCap + i] = p0[d];
                w[(3 + d) * kQueueCap + i] = p1[d];
            }
            w[6 * kQueueCap + i] = q;
            w[7 * kQueueCap + i] = __int_as_float(org);
            w[8 * kQueueCap + i] = __int_as_float(st[0] | (st[1] << 3) | (st[2] << 6));
        }

        __device__ __forceinline__ void get(int i, float p0[3], float p1[3], float& q, int& org, int st[3]) const
        {
#pragma unroll
            for(int d = 0; d < 3; ++d)
            {
                p0[d] = w[d * kQueueCap + i];
                p1[d] = w[(3 + d) * kQueueCap + i];
            }
            q = w[6 * kQueueCap + i];
            org = __float_as_int(w[7 * kQueueCap + i]);
            int const pk = __float_as_int(w[8 * kQueueCap + i]);
            st[0] = pk & 7;
            st[1] = (pk >> 3) & 7;
            st[2] = (pk >> 6) & 7;
        }

        __device__ __forceinline__ void move(int from, int to) const
        {
#pragma unroll
            for(int r = 0; r < kJobWords; ++r)
                w[r * kQueueCap + to] = w[r * kQueueCap + from];
        }
    };

#ifndef PICGB_DRAIN_OUT_OF_LINE
#    define PICGB_DRAIN_OUT_OF_LINE 1
#endif

    // Deposit of the queued jobs of lanes [0, njobs) of a warp with the general footprint
    // (EmZ: the second virtual particles).  The tile and the queue are addressed as word
    // offsets into the block's dynamic shared memory, so the accesses stay shared-memory
    // atomics and loads.  Out of line when PICGB_DRAIN_OUT_OF_LINE: the path runs once per
    // 32 queued jobs, and keeping its code out of the particle loop keeps the loop small
    // for the instruction cache.
    template<typename SH, int TX, int TP, int TT, bool EMZ>
#if PICGB_DRAIN_OUT_OF_LINE
    __device__ __noinline__
#else
    __device__ __forceinline__
#endif
        void drainQueue(int jOff, int qOff, int idx, bool active, JFixed jf, float dx, float dy, float dz, float dt, float invVdt)
    {
        extern __shared__ __align__(16) float smem[];
        if(!active)
            return;
        WarpQueue const queue{smem + qOff};
        float q0[3], q1[3], qc;
        int qo, qs[3];
        queue.get(idx, q0, q1, qc, qo, qs);
        GridParams g{};
        g.dx = dx;
        g.dy = dy;
        g.dz = dz;
        g.dt = dt;
        using Tile = TileJ<TX, TP, TT>;
        if constexpr(EMZ)
            Esirkepov<SH>::runEmZ(Tile{smem + jOff, qo, jf}, q0, q1, qc, g);
        else
            Esirkepov<SH>::template run<true>(Tile{smem + jOff, qo, jf}, q0, q1, qs, qc, g, invVdt);
    }

    // The hook pushSupercell runs after the block has loaded its tiles (or found its supercell
    // empty): nothing in the single-box kernel.
    struct NoHook
    {
        __device__ void operator()() const {}
    };

    // Push of the particles of supercell `sc` by one block of THREADS threads.
    // Each thread pushes one particle per round; then the warp deposits at once
    // the lanes whose particle stays in its assignment cell along every axis
    // (the short fixed footprint, most particles), and queues the other lanes'
    // jobs in its shared-memory queue, which it drains 32 at a time with the
    // general footprint.  Without the split every warp would pay, through
    // divergence, the largest footprint of any of its lanes.  `smem` holds
    // TileGeom::pushSmem bytes; the block must be synchronised before a second
    // call reuses it.  ALT: the kernel variant for the HigueraCary and Vay pushers;
    // the other variant serves Boris and Free, so neither carries the other's code.
    // EMZ: the EmZ deposit (each particle's first virtual particle at once, the second,
    // for the particles that change cell, through the warp's queue) instead of Esirkepov.
    // Every thread calls hook() once: after the tile loads and their barrier, or at once
    // when the supercell is empty (the batched kernel fetches its next work item there).
    template<int SHAPE, int SX, int SY, int SZ, int THREADS, bool ALT, bool EMZ, typename Hook = NoHook>
    __device__ __forceinline__ void pushSupercell(
        SpeciesDev const& sp,
        float const* __restrict__ E,
        float const* __restrict__ B,
        float* __restrict__ J,
        GridParams const& g,
        PushParams const& pp,
        unsigned* __restrict__ status,
        int const sc,
        float* const smem,
        unsigned& s_nhole,
        Hook const& hook = Hook{})
    {
        using SH = Shape<SHAPE>;
        using SC = SuperCell<SX, SY, SZ>;
        using TG = TileGeom<SH, SC, THREADS>;
        using ES = Esirkepov<SH>;
        using Tile = TileJ<TG::JX, TG::JP, TG::JT>;
        float* const Es = smem;
        float* const Bs = smem + 3 * TG::GT;
        float* const Js = smem + 6 * TG::GT;
        int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        int const qOff = 6 * TG::GT + TG::JWords + warp * kQueueCap * kJobWords; // word offset of this warp's queue
        WarpQueue const queue{smem + qOff};

        uint32_t const n = sp.count[sc];
        if(threadIdx.x == 0)
            s_nhole = 0u;
        if(n == 0)
        {
            if(threadIdx.x == 0)
                sp.nhole[sc] = 0u;
            hook();
            return;
        }
        int scx, scy, scz;
        scCoords(sc, g, scx, scy, scz);
        int const ox = scx * SX, oy = scy * SY, oz = scz * SZ;
        size_t const ncell = size_t(g.nx) * g.ny * g.nz;
        bool const useFields = pp.pusher != kPusherFree && pp.pusher != kPusherPhoton; // Boris, HigueraCary, Vay
        if(useFields)
        {
            loadTile<TG::GX, TG::GY, TG::GZ, TG::PX, TG::PY, TG::GT>(Es, E, ox - SH::gLo, oy - SH::gLo, oz - SH::gLo, g,
                                                                  ncell);
            loadTile<TG::GX, TG::GY, TG::GZ, TG::PX, TG::PY, TG::GT>(Bs, B, ox - SH::gLo, oy - SH::gLo, oz - SH::gLo, g,
                                                                  ncell);
        }
        if(pp.deposit)
            for(int t = threadIdx.x; t < TG::JWords; t += blockDim.x)
                Js[t] = 0.0f;
        __syncthreads();
        hook();

        size_t const base = size_t(sc) * sp.cap;
        int queued = 0; // jobs in this warp's queue (warp-uniform)
        for(uint32_t c0 = 0; c0 < n; c0 += THREADS)
        {
            uint32_t const k = c0 + threadIdx.x;
            int kind = -1; // 0: stays in its assignment cell, 1: crosses a cell boundary
            float p0[3], p1[3], charge = 0.0f;
            int stat[3] = {0, 0, 0}, org = 0;
            float b0[3], b1[3]; // EmZ: the second virtual particle
            int orgB = 0;
            if(k < n)
            {
                size_t const slot = base + k;
                float pos[3] = {sp.px[slot], sp.py[slot], sp.pz[slot]};
                float mom[3] = {sp.ux[slot], sp.uy[slot], sp.uz[slot]};
                float const w = sp.w[slot];
                int const lc = sp.lcell[slot];
                int const lx = lc % SX, ly = (lc / SX) % SY, lz = lc / (SX * SY);
                float const mass = fm(pp.mass, w);
                charge = fm(pp.charge, w);
                float vel[3];
                if(useFields)
                {
                    float Ev[3], Bv[3];
                    GatherWeights<SH> gw;
                    gw.compute(pos);
                    // Yee positions (fields/YeeCell.hpp:70-131): E_x (1/2,0,0) ... B_x (0,1/2,1/2) ...
#if PICGB_GATHER_PAIRS
                    // pairs sharing the staggering along two axes, with packed f32x2 FMAs
                    float2 const bxEy = gw.template gather2<TG::PX, TG::PY, 0, 1, 1, 0, 1, 0>(Bs, Es + TG::GT, lx, ly, lz);
                    float2 const byEz = gw.template gather2<TG::PX, TG::PY, 1, 0, 1, 0, 0, 1>(Bs + TG::GT, Es + 2 * TG::GT, lx, ly, lz);
                    float2 const bzEx = gw.template gather2<TG::PX, TG::PY, 1, 1, 0, 1, 0, 0>(Bs + 2 * TG::GT, Es, lx, ly, lz);
                    Bv[0] = bxEy.x;
                    Ev[1] = bxEy.y;
                    Bv[1] = byEz.x;
                    Ev[2] = byEz.y;
                    Bv[2] = bzEx.x;
                    Ev[0] = bzEx.y;
#else
                    Bv[0] = gw.template gather<TG::PX, TG::PY, 0, 1, 1>(Bs, lx, ly, lz);
                    Bv[1] = gw.template gather<TG::PX, TG::PY, 1, 0, 1>(Bs + TG::GT, lx, ly, lz);
                    Bv[2] = gw.template gather<TG::PX, TG::PY, 1, 1, 0>(Bs + 2 * TG::GT, lx, ly, lz);
                    Ev[0] = gw.template gather<TG::PX, TG::PY, 1, 0, 0>(Es, lx, ly, lz);
                    Ev[1] = gw.template gather<TG::PX, TG::PY, 0, 1, 0>(Es + TG::GT, lx, ly, lz);
                    Ev[2] = gw.template gather<TG::PX, TG::PY, 0, 0, 1>(Es + 2 * TG::GT, lx, ly, lz);
#endif
                    if constexpr(!ALT)
                        boris(charge, mass, Ev, Bv, pp.dt, pp.c2, pp.rc2, mom, vel);
                    else
                    {
                        float3 const e3 = make_float3(Ev[0], Ev[1], Ev[2]), b3 = make_float3(Bv[0], Bv[1], Bv[2]);
                        float3 const m3 = make_float3(mom[0], mom[1], mom[2]);
                        float3 const r = pp.pusher == kPusherHigueraCary
                            ? higueraCary(charge, mass, e3, b3, pp.dt, pp.c, pp.c2, m3)
                            : vay(charge, mass, e3, b3, pp.dt, pp.c, pp.c2, pp.rc2, m3);
                        mom[0] = r.x;
                        mom[1] = r.y;
                        mom[2] = r.z;
                        velocity(mom, mass, pp.rc2, vel);
                    }
                }
                else if(pp.pusher == kPusherPhoton)
                {
                    // Photon (particlePusherPhoton.hpp:66-74): vel = mom * (c / |mom|)
                    float const f = fdv(pp.c, fsq(l2n2(mom[0], mom[1], mom[2])));
#pragma unroll
                    for(int d = 0; d < 3; ++d)
                        vel[d] = fm(mom[d], f);
                }
                else
                    velocity(mom, mass, pp.rc2, vel);
#pragma unroll
                for(int d = 0; d < 3; ++d)
                    pos[d] = fa(pos[d], divCell(fm(vel[d], pp.dt), d, g));
                int nlc = lc;
                int mv[3], dir[3];
                bool const leave = moveParticle<SC>(pos, nlc, mv, dir);
                if constexpr(EMZ)
                {
                    int sS[3], sE[3];
                    bool two;
                    if(pp.deposit && !ES::prepareEmZ(pos, vel, g, p0, p1, sS, b0, b1, sE, two))
                        atomicOr(status, ST_BAD_CELL);
                    else if(pp.deposit)
                    {
                        // tile indices of the two virtual particles' cells
                        org = TG::jIndex(lx + mv[0] + sS[0] + SH::jLo, ly + mv[1] + sS[1] + SH::jLo, lz + mv[2] + sS[2] + SH::jLo);
                        orgB = TG::jIndex(lx + mv[0] + sE[0] + SH::jLo, ly + mv[1] + sE[1] + SH::jLo, lz + mv[2] + sE[2] + SH::jLo);
                        kind = two ? 1 : 0;
                    }
                }
                else if(pp.deposit)
                {
                    int gs[3];
                    if(!ES::prepare(pos, vel, g, p0, p1, gs, stat))
                        atomicOr(status, ST_BAD_CELL);
                    else
                    {
                        // tile index of the Esirkepov origin; the new cell lies in [-1, S]
                        org = TG::jIndex(lx + mv[0] + gs[0] + SH::jLo, ly + mv[1] + gs[1] + SH::jLo, lz + mv[2] + gs[2] + SH::jLo);
                        kind = (stat[0] == ES::kInCell && stat[1] == ES::kInCell && stat[2] == ES::kInCell) ? 0 : 1;
                    }
                }
                if(!leave)
                {
                    sp.px[slot] = pos[0];
                    sp.py[slot] = pos[1];
                    sp.pz[slot] = pos[2];
                    sp.ux[slot] = mom[0];
                    sp.uy[slot] = mom[1];
                    sp.uz[slot] = mom[2];
                    if(nlc != lc)
                        sp.lcell[slot] = uint16_t(nlc);
                }
                else
                {
                    int const dx = wrapOrOutside(scx + dir[0], g.nscx, g.open & 1),
                              dy = wrapOrOutside(scy + dir[1], g.nscy, g.open & 2),
                              dz = wrapOrOutside(scz + dir[2], g.nscz, g.open & 4);
                    int const dsc = dx + g.nscx * (dy + g.nscy * dz);
                    uint32_t const id = sp.id ? sp.id[slot] : 0u;
                    // a particle that leaves the box through an open face is absorbed: it only
                    // vacates its slot (the reference's absorbing particle boundary)
                    if((dx | dy | dz) >= 0)
                    {
                        uint32_t const s = atomicAdd(sp.tail + dsc, 1u);
                        if(s < sp.cap)
                        {
                            size_t const d = size_t(dsc) * sp.cap + s;
                            sp.px[d] = pos[0];
                            sp.py[d] = pos[1];
                            sp.pz[d] = pos[2];
                            sp.ux[d] = mom[0];
                            sp.uy[d] = mom[1];
                            sp.uz[d] = mom[2];
                            sp.w[d] = w;
                            sp.lcell[d] = uint16_t(nlc);
                            if(sp.id)
                                sp.id[d] = id;
                        }
                        else
                        {
                            uint32_t const q = atomicAdd(sp.sp_count, 1u);
                            if(q < sp.spill_cap)
                            {
                                float* a = sp.sp_attr;
                                size_t const C = sp.spill_cap;
                                a[q] = pos[0];
                                a[C + q] = pos[1];
                                a[2 * C + q] = pos[2];
                                a[3 * C + q] = mom[0];
                                a[4 * C + q] = mom[1];
                                a[5 * C + q] = mom[2];
                                a[6 * C + q] = w;
                                sp.sp_sc[q] = dsc;
                                sp.sp_lcell[q] = uint16_t(nlc);
                                sp.sp_id[q] = id;
                                atomicOr(status, ST_OVERFLOW);
                            }
                            else
                                atomicOr(status, ST_OVERFLOW | ST_LOST);
                        }
                    }
                    uint32_t const h = atomicAdd(&s_nhole, 1u);
                    sp.holes[base + h] = uint16_t(k);
                }
            }
            if(!pp.deposit)
                continue;
            // particles that stay in their cell: deposit now with the short footprint (EmZ:
            // every particle's first virtual particle)
            if constexpr(EMZ)
            {
                if(kind >= 0)
                    ES::runEmZ(Tile{Js, org, pp.jf}, p0, p1, charge, g);
            }
            else if(kind == 0)
                ES::template run<false>(Tile{Js, org, pp.jf}, p0, p1, stat, charge, g, pp.invVdt);
            // the others: into the warp's queue, drained 32 at a time
            unsigned const crossing = __ballot_sync(0xffffffffu, kind == 1);
            if(pp.kindCount)
            {
                unsigned const shortFp = __ballot_sync(0xffffffffu, kind == 0);
                if(lane == 0)
                {
                    atomicAdd(pp.kindCount, (unsigned long long) __popc(shortFp));
                    atomicAdd(pp.kindCount + 1, (unsigned long long) __popc(crossing));
                }
            }
            // the lanes that fit go in now; a queue that reaches 32 jobs is drained; the
            // lanes that did not fit go in after the drain (only with kQueueCap < 63)
            int const nc = __popc(crossing);
            int const room = kQueueCap - queued;
            int const rank = __popc(crossing & laneMaskLt());
            auto enqueue = [&](int at)
            {
                if constexpr(EMZ)
                    queue.put(at, b0, b1, charge, orgB, stat);
                else
                    queue.put(at, p0, p1, charge, org, stat);
            };
            if(kind == 1 && rank < room)
                enqueue(queued + rank);
            queued += nc < room ? nc : room;
            __syncwarp();
            if(queued >= 32)
            {
                drainQueue<SH, TG::JX, TG::JP, TG::JT, EMZ>(
                    int(Js - smem), qOff, lane, true, pp.jf, g.dx, g.dy, g.dz, g.dt, pp.invVdt);
                __syncwarp();
                if(lane < queued - 32)
                    queue.move(32 + lane, lane);
                queued -= 32;
                __syncwarp();
            }
            if(nc > room)
            {
                if(kind == 1 && rank >= room)
                    enqueue(queued + rank - room);
                queued += nc - room;
                __syncwarp();
            }
        }
        // The jobs still queued (fewer than 32 per warp), pooled over the block: job p of the
        // pool is job p - (jobs of the warps before) of its warp's queue, and warp w drains pool
        // jobs 32 w .. 32 w + 31.  A warp draining only its own few leftovers would run the whole
        // general footprint for a handful of lanes.
#if !PICGB_POOL_LEFTOVERS
        if(pp.deposit && queued > 0)
            drainQueue<SH, TG::JX, TG::JP, TG::JT, EMZ>(
                int(Js - smem), qOff, lane, lane < queued, pp.jf, g.dx, g.dy, g.dz, g.dt, pp.invVdt);
#else
        if(pp.deposit)
        {
            __shared__ int s_left[THREADS / 32];
            if(lane == 0)
                s_left[warp] = queued;
            __syncthreads(); // every warp's queue is complete
            int const p = warp * 32 + lane;
            int total = 0, owner = 0, idx = 0;
#pragma unroll
            for(int q = 0; q < THREADS / 32; ++q)
            {
                int const c = s_left[q];
                if(p >= total && p < total + c)
                {
                    owner = q;
                    idx = p - total;
                }
                total += c;
            }
            if(warp * 32 < total)
                drainQueue<SH, TG::JX, TG::JP, TG::JT, EMZ>(int(Js - smem),
                    6 * TG::GT + TG::JWords + owner * kQueueCap * kJobWords, idx, p < total, pp.jf, g.dx, g.dy, g.dz,
                    g.dt, pp.invVdt);
        }
#endif
        __syncthreads(); // every hole is recorded and every deposit done
        if(threadIdx.x == 0)
            sp.nhole[sc] = s_nhole;
        if(pp.deposit)
            flushTile<TG::JX, TG::JY, TG::JP, TG::JT>(Js, J, ox - SH::jLo, oy - SH::jLo, oz - SH::jLo, g, ncell, pp.jf);
    }

    // Fused push kernel of one box: one block per supercell.
    template<int SHAPE, int SX, int SY, int SZ, bool ALT, bool EMZ>
    __global__ void __launch_bounds__(kPushThreads, PICGB_PUSH_MIN_BLOCKS) kPush(
        SpeciesDev sp,
        float const* __restrict__ E,
        float const* __restrict__ B,
        float* __restrict__ J,
        GridParams g,
        PushParams pp,
        unsigned* __restrict__ status)
    {
        extern __shared__ __align__(16) float smem[];
        __shared__ unsigned s_nhole;
        pushSupercell<SHAPE, SX, SY, SZ, kPushThreads, ALT, EMZ>(sp, E, B, J, g, pp, status, blockIdx.x, smem, s_nhole);
    }

    // Deposit-only kernel over the sorted particles (the reference's separate
    // CurrentDeposition stage, simulation/stage/CurrentDeposition.x.cpp:105).
    template<int SHAPE, int SX, int SY, int SZ, bool EMZ>
    __global__ void __launch_bounds__(kPushThreads)
        kDeposit(SpeciesDev sp, float* __restrict__ J, GridParams g, PushParams pp, unsigned* __restrict__ status)
    {
        using SH = Shape<SHAPE>;
        using SC = SuperCell<SX, SY, SZ>;
        using TG = TileGeom<SH, SC>;
        extern __shared__ __align__(16) float jsm[];
        float* const Js = jsm;
        int const sc = blockIdx.x;
        uint32_t const n = sp.count[sc];
        if(n == 0)
            return;
        int scx, scy, scz;
        scCoords(sc, g, scx, scy, scz);
        size_t const ncell = size_t(g.nx) * g.ny * g.nz;
        for(int t = threadIdx.x; t < TG::JWords; t += blockDim.x)
            Js[t] = 0.0f;
        __syncthreads();
        size_t const base = size_t(sc) * sp.cap;
        for(uint32_t k = threadIdx.x; k < n; k += blockDim.x)
        {
            size_t const slot = base + k;
            float const pos[3] = {sp.px[slot], sp.py[slot], sp.pz[slot]};
            float const mom[3] = {sp.ux[slot], sp.uy[slot], sp.uz[slot]};
            float const w = sp.w[slot];
            int const lc = sp.lcell[slot];
            int const cellRel[3] = {lc % SX, (lc / SX) % SY, lc / (SX * SY)};
            float vel[3];
            velocity(mom, fm(pp.mass, w), pp.rc2, vel);
            float p0[3], p1[3];
            int gs[3], stat[3];
            if constexpr(EMZ)
            {
                float b0[3], b1[3];
                int sE[3];
                bool two;
                if(!Esirkepov<SH>::prepareEmZ(pos, vel, g, p0, p1, gs, b0, b1, sE, two))
                {
                    atomicOr(status, ST_BAD_CELL);
                    continue;
                }
                float const q = fm(pp.charge, w);
                Esirkepov<SH>::runEmZ(
                    TileJ<TG::JX, TG::JP, TG::JT>{
                        Js,
                        TG::jIndex(cellRel[0] + gs[0] + SH::jLo, cellRel[1] + gs[1] + SH::jLo, cellRel[2] + gs[2] + SH::jLo),
                        pp.jf},
                    p0,
                    p1,
                    q,
                    g);
                if(two)
                    Esirkepov<SH>::runEmZ(
                        TileJ<TG::JX, TG::JP, TG::JT>{
                            Js,
                            TG::jIndex(cellRel[0] + sE[0] + SH::jLo, cellRel[1] + sE[1] + SH::jLo, cellRel[2] + sE[2] + SH::jLo),
                            pp.jf},
                        b0,
                        b1,
                        q,
                        g);
                continue;
            }
            if(!Esirkepov<SH>::prepare(pos, vel, g, p0, p1, gs, stat))
            {
                atomicOr(status, ST_BAD_CELL);
                continue;
            }
            TileJ<TG::JX, TG::JP, TG::JT> const acc{
                Js,
                TG::jIndex(cellRel[0] + gs[0] + SH::jLo, cellRel[1] + gs[1] + SH::jLo, cellRel[2] + gs[2] + SH::jLo),
                pp.jf};
            Esirkepov<SH>::template run<true>(acc, p0, p1, stat, fm(pp.charge, w), g, pp.invVdt);
        }
        __syncthreads();
        flushTile<TG::JX, TG::JY, TG::JP, TG::JT>(
            Js,
            J,
            scx * SX - SH::jLo,
            scy * SY - SH::jLo,
            scz * SZ - SH::jLo,
            g,
            ncell,
            pp.jf);
    }

    // Charge density at the cell origin with ChargeAssignment
    // (particles/particleToGrid/ComputeGridValuePerFrame.hpp:66-117); validation only.
    template<int SHAPE, int SX, int SY, int SZ>
    __global__ void kChargeDensity(SpeciesDev sp, float* __restrict__ rho, GridParams g, float charge, float cellVolume)
    {
        using SH = Shape<SHAPE>;
        constexpr int lo = SH::supp / 2, up = (SH::supp + 1) / 2, span = lo + up + 1;
        int const sc = blockIdx.x;
        uint32_t const n = sp.count[sc];
        int scx, scy, scz;
        scCoords(sc, g, scx, scy, scz);
        size_t const base = size_t(sc) * sp.cap;
        for(uint32_t k = threadIdx.x; k < n; k += blockDim.x)
        {
            size_t const slot = base + k;
            float const pos[3] = {sp.px[slot], sp.py[slot], sp.pz[slot]};
            int const lc = sp.lcell[slot];
            int const cx = scx * SX + lc % SX, cy = scy * SY + (lc / SX) % SY, cz = scz * SZ + lc / (SX * SY);
            float const attr = fdv(fm(charge, sp.w[slot]), cellVolume); // ChargeDensity.hpp:46
            for(int i = 0; i < span * span * span; ++i)
            {
                int const o[3] = {i % span - lo, (i / span) % span - lo, i / (span * span) - lo};
                float a = 1.0f;
#pragma unroll
                for(int d = 0; d < 3; ++d)
                    a = fm(a, SH::ca(fs(float(o[d]), pos[d])));
                if(a != 0.0f)
                {
                    int const gx = wrapi(cx + o[0], g.nx), gy = wrapi(cy + o[1], g.ny), gz = wrapi(cz + o[2], g.nz);
                    atomicAdd(rho + size_t(gx) + size_t(g.nx) * (size_t(gy) + size_t(g.ny) * gz), fm(a, attr));
                }
            }
        }
    }

    template<int SHAPE, int SX, int SY, int SZ, bool ALT>
    cudaError_t launchPushT(
        SpeciesDev const& sp,
        float const* E,
        float const* B,
        float* J,
        GridParams const& g,
        PushParams const& pp,
        unsigned* status,
        cudaStream_t stream)
    {
        using TG = TileGeom<Shape<SHAPE>, SuperCell<SX, SY, SZ>>;
        auto k = pp.current == kCurrentEmZ ? kPush<SHAPE, SX, SY, SZ, ALT, true> : kPush<SHAPE, SX, SY, SZ, ALT, false>;
        size_t const smem = TG::pushSmem;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if(e != cudaSuccess)
            return e;
        int const nsc = g.nscx * g.nscy * g.nscz;
        k<<<nsc, kPushThreads, smem, stream>>>(sp, E, B, J, g, pp, status);
        return cudaGetLastError();
    }

    template<int SHAPE, int SX, int SY, int SZ>
    cudaError_t launchDepositT(
        SpeciesDev const& sp,
        float* J,
        GridParams const& g,
        PushParams const& pp,
        unsigned* status,
        cudaStream_t stream)
    {
        using TG = TileGeom<Shape<SHAPE>, SuperCell<SX, SY, SZ>>;
        auto k = pp.current == kCurrentEmZ ? kDeposit<SHAPE, SX, SY, SZ, true> : kDeposit<SHAPE, SX, SY, SZ, false>;
        size_t const smem = TG::depositSmem;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if(e != cudaSuccess)
            return e;
        int const nsc = g.nscx * g.nscy * g.nscz;
        k<<<nsc, kPushThreads, smem, stream>>>(sp, J, g, pp, status);
        return cudaGetLastError();
    }

    template<int SHAPE, int SX, int SY, int SZ>
    cudaError_t launchChargeDensityT(
        SpeciesDev const& sp,
        float* rho,
        GridParams const& g,
        float charge,
        float cellVolume,
        cudaStream_t stream)
    {
        int const nsc = g.nscx * g.nscy * g.nscz;
        kChargeDensity<SHAPE, SX, SY, SZ><<<nsc, 256, 0, stream>>>(sp, rho, g, charge, cellVolume);
        return cudaGetLastError();
    }

// Instantiates the push launcher of one shape and pusher variant (ALT: HigueraCary and
// Vay) for the supported supercell sizes; each (shape, variant) pair has its own
// translation unit, so the heaviest instantiations compile in parallel.
#define PICGB_PUSH_LAUNCHER(SHAPE, NAME, ALT)                                                                         \
    cudaError_t launchPush##NAME(                                                                                     \
        int scId,                                                                                                     \
        SpeciesDev const& sp,                                                                                         \
        float const* E,                                                                                               \
        float const* B,                                                                                               \
        float* J,                                                                                                     \
        GridParams const& g,                                                                                          \
        PushParams const& pp,                                                                                         \
        unsigned* status,                                                                                             \
        cudaStream_t stream)                                                                                          \
    {                                                                                                                 \
        switch(scId)                                                                                                  \
        {                                                                                                             \
        case 0:                                                                                                       \
            return launchPushT<SHAPE, 8, 8, 4, ALT>(sp, E, B, J, g, pp, status, stream);                              \
        case 1:                                                                                                       \
            return launchPushT<SHAPE, 4, 4, 4, ALT>(sp, E, B, J, g, pp, status, stream);                              \
        case 2:                                                                                                       \
            return launchPushT<SHAPE, 8, 8, 8, ALT>(sp, E, B, J, g, pp, status, stream);                              \
        }                                                                                                             \
        return cudaErrorInvalidValue;                                                                                 \
    }

// Instantiates the deposit and charge-density launchers of one shape for the supported
// supercell sizes.
#define PICGB_SHAPE_LAUNCHERS(SHAPE, NAME)                                                                            \
    cudaError_t launchDeposit##NAME(                                                                                  \
        int scId,                                                                                                     \
        SpeciesDev const& sp,                                                                                         \
        float* J,                                                                                                     \
        GridParams const& g,                                                                                          \
        PushParams const& pp,                                                                                         \
        unsigned* status,                                                                                             \
        cudaStream_t stream)                                                                                          \
    {                                                                                                                 \
        switch(scId)                                                                                                  \
        {                                                                                                             \
        case 0:                                                                                                       \
            return launchDepositT<SHAPE, 8, 8, 4>(sp, J, g, pp, status, stream);                                      \
        case 1:                                                                                                       \
            return launchDepositT<SHAPE, 4, 4, 4>(sp, J, g, pp, status, stream);                                      \
        case 2:                                                                                                       \
            return launchDepositT<SHAPE, 8, 8, 8>(sp, J, g, pp, status, stream);                                      \
        }                                                                                                             \
        return cudaErrorInvalidValue;                                                                                 \
    }                                                                                                                 \
    cudaError_t launchChargeDensity##NAME(                                                                            \
        int scId,                                                                                                     \
        SpeciesDev const& sp,                                                                                         \
        float* rho,                                                                                                   \
        GridParams const& g,                                                                                          \
        float charge,                                                                                                 \
        float cellVolume,                                                                                             \
        cudaStream_t stream)                                                                                          \
    {                                                                                                                 \
        switch(scId)                                                                                                  \
        {                                                                                                             \
        case 0:                                                                                                       \
            return launchChargeDensityT<SHAPE, 8, 8, 4>(sp, rho, g, charge, cellVolume, stream);                            \
        case 1:                                                                                                       \
            return launchChargeDensityT<SHAPE, 4, 4, 4>(sp, rho, g, charge, cellVolume, stream);                            \
        case 2:                                                                                                       \
            return launchChargeDensityT<SHAPE, 8, 8, 8>(sp, rho, g, charge, cellVolume, stream);                            \
        }                                                                                                             \
        return cudaErrorInvalidValue;                                                                                 \
    }
} // namespace picgb
