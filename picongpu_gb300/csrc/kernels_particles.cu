// Particle bookkeeping kernels: shape dispatch of the push/deposit launchers,
// hole compaction after the migration (the reference's KernelFillGaps,
// pmacc/particles/ParticlesBase.kernel:183-359), upload scatter into the
// supercell layout, download gather, and the FP64 kinetic-energy reduction
// (plugins/EnergyParticles.x.cpp:58-160).
#include "picgb_batch.hpp"
#include "picgb_device.cuh"
#include "picgb_internal.hpp"

namespace picgb
{
#define PICGB_DECL_BATCH(NAME)                                                                                        \
    cudaError_t launchPushBatch##NAME(int, int, BatchSpecies const*, uint32_t const*, uint32_t, uint32_t*, unsigned*, \
                                      GridParams const&, PushParams const&, cudaStream_t);
#define PICGB_DECL_BATCH_SHAPE(NAME)                                                                                  \
    PICGB_DECL_BATCH(NAME)                                                                                            \
    PICGB_DECL_BATCH(NAME##Alt)                                                                                       \
    PICGB_DECL_BATCH(NAME##EmZ)                                                                                       \
    PICGB_DECL_BATCH(NAME##AltEmZ)
    PICGB_DECL_BATCH_SHAPE(CIC)
    PICGB_DECL_BATCH_SHAPE(TSC)
    PICGB_DECL_BATCH_SHAPE(PQS)
    PICGB_DECL_BATCH_SHAPE(PCS)

#define PICGB_DECL_SHAPE(NAME)                                                                                        \
    cudaError_t launchPush##NAME(                                                                                     \
        int,                                                                                                          \
        SpeciesDev const&,                                                                                            \
        float const*,                                                                                                 \
        float const*,                                                                                                 \
        float*,                                                                                                       \
        GridParams const&,                                                                                            \
        PushParams const&,                                                                                            \
        unsigned*,                                                                                                    \
        cudaStream_t);                                                                                                \
    cudaError_t launchPush##NAME##Alt(                                                                                \
        int,                                                                                                          \
        SpeciesDev const&,                                                                                            \
        float const*,                                                                                                 \
        float const*,                                                                                                 \
        float*,                                                                                                       \
        GridParams const&,                                                                                            \
        PushParams const&,                                                                                            \
        unsigned*,                                                                                                    \
        cudaStream_t);                                                                                                \
    cudaError_t launchDeposit##NAME(                                                                                  \
        int,                                                                                                          \
        SpeciesDev const&,                                                                                            \
        float*,                                                                                                       \
        GridParams const&,                                                                                            \
        PushParams const&,                                                                                            \
        unsigned*,                                                                                                    \
        cudaStream_t);                                                                                                \
    cudaError_t launchChargeDensity##NAME(int, SpeciesDev const&, float*, GridParams const&, float, float, cudaStream_t);
    PICGB_DECL_SHAPE(CIC)
    PICGB_DECL_SHAPE(TSC)
    PICGB_DECL_SHAPE(PQS)
    cudaError_t launchPushPCS(int, SpeciesDev const&, float const*, float const*, float*, GridParams const&, PushParams const&,
                              unsigned*, cudaStream_t);
    cudaError_t launchPushPCSAlt(int, SpeciesDev const&, float const*, float const*, float*, GridParams const&,
                                 PushParams const&, unsigned*, cudaStream_t);
    cudaError_t launchDepositPCS(int, SpeciesDev const&, float*, GridParams const&, PushParams const&, unsigned*, cudaStream_t);
    cudaError_t launchChargeDensityPCS(int, SpeciesDev const&, float*, GridParams const&, float, float, cudaStream_t);

    cudaError_t launchPush(
        int shape,
        int scId,
        SpeciesDev const& sp,
        float const* E,
        float const* B,
        float* J,
        GridParams const& g,
        PushParams const& pp,
        unsigned* status,
        cudaStream_t stream)
    {
        bool const alt = pp.pusher == kPusherHigueraCary || pp.pusher == kPusherVay;
        switch(shape * 2 + (alt ? 1 : 0))
        {
        case 2:
            return launchPushCIC(scId, sp, E, B, J, g, pp, status, stream);
        case 3:
            return launchPushCICAlt(scId, sp, E, B, J, g, pp, status, stream);
        case 4:
            return launchPushTSC(scId, sp, E, B, J, g, pp, status, stream);
        case 5:
            return launchPushTSCAlt(scId, sp, E, B, J, g, pp, status, stream);
        case 6:
            return launchPushPQS(scId, sp, E, B, J, g, pp, status, stream);
        case 7:
            return launchPushPQSAlt(scId, sp, E, B, J, g, pp, status, stream);
        case 8:
            return launchPushPCS(scId, sp, E, B, J, g, pp, status, stream);
        case 9:
            return launchPushPCSAlt(scId, sp, E, B, J, g, pp, status, stream);
        }
        return cudaErrorInvalidValue;
    }

    cudaError_t launchPushBatch(
        int shape,
        int scId,
        int threads,
        int pusher,
        int current,
        BatchSpecies const* table,
        uint32_t const* items,
        uint32_t nitems,
        uint32_t* counter,
        unsigned* status,
        GridParams const& g0,
        PushParams const& pp0,
        cudaStream_t stream)
    {
        bool const alt = pusher == kPusherHigueraCary || pusher == kPusherVay;
        bool const emz = current == kCurrentEmZ;
#define PICGB_BATCH_DISPATCH(NAME)                                                                                    \
    return emz ? (alt ? launchPushBatch##NAME##AltEmZ(scId, threads, table, items, nitems, counter, status, g0, pp0, stream)    \
                      : launchPushBatch##NAME##EmZ(scId, threads, table, items, nitems, counter, status, g0, pp0, stream))      \
               : (alt ? launchPushBatch##NAME##Alt(scId, threads, table, items, nitems, counter, status, g0, pp0, stream)       \
                      : launchPushBatch##NAME(scId, threads, table, items, nitems, counter, status, g0, pp0, stream));
        switch(shape)
        {
        case 1:
            PICGB_BATCH_DISPATCH(CIC)
        case 2:
            PICGB_BATCH_DISPATCH(TSC)
        case 3:
            PICGB_BATCH_DISPATCH(PQS)
        case 4:
            PICGB_BATCH_DISPATCH(PCS)
        }
#undef PICGB_BATCH_DISPATCH
        return cudaErrorInvalidValue;
    }

    cudaError_t launchDeposit(
        int shape,
        int scId,
        SpeciesDev const& sp,
        float* J,
        GridParams const& g,
        PushParams const& pp,
        unsigned* status,
        cudaStream_t stream)
    {
        switch(shape)
        {
        case 1:
            return launchDepositCIC(scId, sp, J, g, pp, status, stream);
        case 2:
            return launchDepositTSC(scId, sp, J, g, pp, status, stream);
        case 3:
            return launchDepositPQS(scId, sp, J, g, pp, status, stream);
        case 4:
            return launchDepositPCS(scId, sp, J, g, pp, status, stream);
        }
        return cudaErrorInvalidValue;
    }

    cudaError_t launchChargeDensity(
        int shape,
        int scId,
        SpeciesDev const& sp,
        float* rho,
        GridParams const& g,
        float charge,
        float cellVolume,
        cudaStream_t stream)
    {
        switch(shape)
        {
        case 1:
            return launchChargeDensityCIC(scId, sp, rho, g, charge, cellVolume, stream);
        case 2:
            return launchChargeDensityTSC(scId, sp, rho, g, charge, cellVolume, stream);
        case 3:
            return launchChargeDensityPQS(scId, sp, rho, g, charge, cellVolume, stream);
        case 4:
            return launchChargeDensityPCS(scId, sp, rho, g, charge, cellVolume, stream);
        }
        return cudaErrorInvalidValue;
    }

    __device__ __forceinline__ uint32_t maskBelow(int w, uint32_t limit)
    {
        // bits j of word w with 32 * w + j < limit
        int64_t const r = int64_t(limit) - 32 * int64_t(w);
        if(r <= 0)
            return 0u;
        if(r >= 32)
            return 0xffffffffu;
        return (1u << r) - 1u;
    }

    __device__ __forceinline__ void copyParticle(SpeciesDev const& sp, size_t dst, size_t src)
    {
        sp.px[dst] = sp.px[src];
        sp.py[dst] = sp.py[src];
        sp.pz[dst] = sp.pz[src];
        sp.ux[dst] = sp.ux[src];
        sp.uy[dst] = sp.uy[src];
        sp.uz[dst] = sp.uz[src];
        sp.w[dst] = sp.w[src];
        sp.lcell[dst] = sp.lcell[src];
        if(sp.id)
            sp.id[dst] = sp.id[src];
    }

    // Fill the slots vacated by leaving particles with the last valid particles of supercell
    // `sc` so that slots [0, count) are dense again.  One warp per supercell (a supercell loses a
    // few percent of its particles per step, so a block per supercell spent its time in barriers):
    // a bitmap of the holes, per 32-slot word the number of holes below the new count
    // (destinations) and of particles at or above it (sources), their exclusive prefix sums by
    // warp scans, and the r-th destination takes the r-th source.  Destinations and sources are
    // disjoint slots, so the lanes' copies never conflict.  `csm` holds 3 * ceil(cap / 32) words
    // for this warp.
    __device__ __forceinline__ void compactSupercell(SpeciesDev const& sp, int const sc, uint32_t* csm)
    {
        int const lane = threadIdx.x & 31;
        uint32_t const tail = sp.tail[sc];
        uint32_t const n = tail < sp.cap ? tail : sp.cap;
        uint32_t const h = sp.nhole[sc];
        if(h == 0)
        {
            if(lane == 0)
            {
                sp.count[sc] = n;
                sp.tail[sc] = n;
            }
            return;
        }
        uint32_t const newc = n - h;
        int const W = int((n + 31) / 32);
        uint32_t* bm = csm;
        uint32_t* dpre = csm + W;
        uint32_t* spre = csm + 2 * W;
        for(int i = lane; i < W; i += 32)
            bm[i] = 0u;
        __syncwarp();
        size_t const base = size_t(sc) * sp.cap;
        for(uint32_t i = lane; i < h; i += 32)
        {
            uint32_t const s = sp.holes[base + i];
            atomicOr(bm + (s >> 5), 1u << (s & 31));
        }
        __syncwarp();
        uint32_t carryD = 0, carryS = 0;
        for(int w0 = 0; w0 < W; w0 += 32)
        {
            int const w = w0 + lane;
            uint32_t d = 0, c = 0;
            if(w < W)
            {
                uint32_t const lo = maskBelow(w, newc);
                uint32_t const hi = maskBelow(w, n) & ~lo;
                d = __popc(bm[w] & lo);
                c = __popc(~bm[w] & hi);
            }
            uint32_t id = d, ic = c; // inclusive warp scans
#pragma unroll
            for(int o = 1; o < 32; o <<= 1)
            {
                uint32_t const vd = __shfl_up_sync(0xffffffffu, id, o);
                uint32_t const vc = __shfl_up_sync(0xffffffffu, ic, o);
                if(lane >= o)
                {
                    id += vd;
                    ic += vc;
                }
            }
            if(w < W)
            {
                dpre[w] = carryD + id - d;
                spre[w] = carryS + ic - c;
            }
            carryD += __shfl_sync(0xffffffffu, id, 31);
            carryS += __shfl_sync(0xffffffffu, ic, 31);
        }
        __syncwarp();
        for(int w = lane; w < W; w += 32)
        {
            uint32_t m = bm[w] & maskBelow(w, newc);
            uint32_t r = dpre[w];
            while(m)
            {
                int const b = __ffs(m) - 1;
                m &= m - 1u;
                // source word: last ws with spre[ws] <= r
                int lo = 0, hi = W - 1;
                while(lo < hi)
                {
                    int const mid = (lo + hi + 1) >> 1;
                    if(spre[mid] <= r)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                int const ws = lo;
                uint32_t sm = ~bm[ws] & (maskBelow(ws, n) & ~maskBelow(ws, newc));
                for(uint32_t q = r - spre[ws]; q > 0; --q)
                    sm &= sm - 1u;
                int const sb = __ffs(sm) - 1;
                if(sb < 0)
                    break; // unreachable for consistent ranks; never index with it
                copyParticle(sp, base + 32u * w + b, base + 32u * ws + sb);
                ++r;
            }
        }
        __syncwarp();
        if(lane == 0)
        {
            sp.count[sc] = newc;
            sp.tail[sc] = newc;
            sp.nhole[sc] = 0u;
        }
    }

    // Warps per block of the compaction: eight, fewer when a warp's 3 ceil(cap / 32) words of
    // shared memory would take more than 48 KB for the block.
    int compactWarps(uint32_t cap)
    {
        size_t const perWarp = sizeof(uint32_t) * 3 * ((cap + 31) / 32);
        size_t const w = (48 * 1024) / (perWarp ? perWarp : 1);
        return int(w < 1 ? 1 : (w > 8 ? 8 : w));
    }

    __global__ void __launch_bounds__(256) kCompact(SpeciesDev sp, int nsc, int words)
    {
        extern __shared__ uint32_t csm[];
        int const warp = threadIdx.x >> 5;
        int const sc = blockIdx.x * (blockDim.x >> 5) + warp;
        if(sc < nsc)
            compactSupercell(sp, sc, csm + warp * 3 * words);
    }

    // Compaction over the supercells of every box of an ensemble: warp k of block b handles
    // work item b * (warps per block) + k (box, supercell).
    __global__ void __launch_bounds__(256)
        kCompactBatch(BatchSpecies const* __restrict__ boxes, uint32_t const* __restrict__ items, uint32_t nitems, int words)
    {
        extern __shared__ uint32_t csm[];
        int const warp = threadIdx.x >> 5;
        uint32_t const k = blockIdx.x * (blockDim.x >> 5) + warp;
        if(k >= nitems)
            return;
        uint32_t const it = items[k];
        compactSupercell(boxes[batchBox(it)].sp, int(batchSc(it)), csm + warp * 3 * words);
    }

    cudaError_t launchCompactBatch(
        BatchSpecies const* boxes,
        uint32_t const* items,
        uint32_t nitems,
        uint32_t maxCap,
        cudaStream_t stream)
    {
        if(nitems == 0)
            return cudaSuccess;
        int const warps = compactWarps(maxCap);
        int const words = int((maxCap + 31) / 32);
        size_t const smem = sizeof(uint32_t) * 3 * size_t(words) * warps;
        if(smem > 48 * 1024)
        {
            cudaError_t e = cudaFuncSetAttribute(kCompactBatch, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if(e != cudaSuccess)
                return e;
        }
        kCompactBatch<<<(nitems + warps - 1) / warps, 32 * warps, smem, stream>>>(boxes, items, nitems, words);
        return cudaGetLastError();
    }

    // ------------------------------------------------------------ re-interleave
    // The push keeps a particle in its slot while it moves between the cells of its supercell,
    // so the cells of a warp's 32 particles drift away from the 8 x 4 patches that the tile
    // pitches are chosen for, and the shared-memory bank conflicts of the gather and the deposit
    // grow (two-stream 256^3: 25.5 ms per push launch after the initialisation, 27.0 ms 200
    // steps later).  kReorder restores the interleaved order of the initialisation in place:
    // round r holds the r-th particle of every cell with more than r particles, cells in
    // index order, so slot k of a supercell whose cells all hold m particles is in cell
    // k mod vol for k < m vol.  A counting sort in shared memory: per-cell ranks by shared
    // atomics, one bitmap of occupied cells per round, positions from popcounts, then every
    // attribute moved once through shared memory.  A supercell with a cell of more than
    // kReorderRounds particles keeps its order.
    constexpr int kReorderRounds = 64;
    constexpr int kReorderThreads = 512;

    struct ReorderSmem
    {
        // word offsets of the parts of the dynamic shared memory
        __host__ __device__ static int cnt(int) { return 0; }
        __host__ __device__ static int bm(int vol) { return vol; }
        __host__ __device__ static int starts(int vol) { return vol + kReorderRounds * (vol / 32); }
        __host__ __device__ static int rank(int vol) { return starts(vol) + kReorderRounds + 1; } // uint16 [cap]
        __host__ __device__ static int inv(int vol, uint32_t cap) { return rank(vol) + int((cap + 1) / 2); } // uint16 [cap]
        __host__ __device__ static int buf(int vol, uint32_t cap) { return inv(vol, cap) + int((cap + 1) / 2); } // uint32 [cap]
        // bitmap of the vacated slots (the compacting form)
        __host__ __device__ static int holes(int vol, uint32_t cap) { return buf(vol, cap) + int(cap); } // uint32 [cap / 32]
        __host__ __device__ static size_t bytes(int vol, uint32_t cap)
        {
            return sizeof(uint32_t) * (size_t(holes(vol, cap)) + (cap + 31) / 32);
        }
    };

    // Loads per thread issued before the first shared-memory store of a staging pass, so
    // that a pass costs one memory latency instead of one per loop iteration.
    constexpr int kReorderLoads = 8;

    // a[j] = a_old[inv[j]] for j < nOut, staged through buf (slots [0, n) are read).  The bits
    // of a 32-bit or 16-bit attribute pass through buf unchanged.
    template<typename T>
    __device__ __forceinline__ void permuteInPlace(
        T* __restrict__ a,
        uint32_t n,
        uint32_t nOut,
        uint32_t* buf,
        uint16_t const* inv)
    {
        static_assert(sizeof(T) == 4 || sizeof(T) == 2, "32-bit or 16-bit attributes");
        using Bits = typename std::conditional<sizeof(T) == 4, uint32_t, uint16_t>::type;
        Bits* const ab = reinterpret_cast<Bits*>(a);
        uint32_t const step = blockDim.x * kReorderLoads;
        for(uint32_t k0 = threadIdx.x; k0 < n; k0 += step)
        {
            Bits v[kReorderLoads];
#pragma unroll
            for(int u = 0; u < kReorderLoads; ++u)
            {
                uint32_t const k = k0 + u * blockDim.x;
                v[u] = k < n ? ab[k] : Bits(0);
            }
#pragma unroll
            for(int u = 0; u < kReorderLoads; ++u)
            {
                uint32_t const k = k0 + u * blockDim.x;
                if(k < n)
                    buf[k] = uint32_t(v[u]);
            }
        }
        __syncthreads();
        for(uint32_t j = threadIdx.x; j < nOut; j += blockDim.x)
            ab[j] = Bits(buf[inv[j]]);
        __syncthreads();
    }

    // Reorder of supercell sc by one block (rsm: ReorderSmem::bytes(vol, sp.cap) of shared memory).
    // COMPACT: the supercell as the push left it (slots [0, min(tail, cap)), the vacated slots in
    // `holes`) is compacted by the same pass, in place of kCompact: the vacated slots are left
    // out of the sort and the count becomes the particles that remain.  Where the sort cannot
    // run (a cell of more than kReorderRounds particles) warp 0 compacts the supercell as
    // kCompact does.  counters (COMPACT, or nullptr): [64][2] sums of the vacated slots and of
    // the particles after the step, one slot pair per block index mod 64.
    template<bool COMPACT>
    __device__ void reorderSupercell(
        SpeciesDev const& sp,
        int sc,
        int vol,
        uint32_t* rsm,
        int& s_tooFull,
        unsigned long long* counters = nullptr)
    {
        uint32_t n, h = 0;
        if constexpr(COMPACT)
        {
            uint32_t const tail = sp.tail[sc];
            n = tail < sp.cap ? tail : sp.cap;
            h = sp.nhole[sc];
            if(threadIdx.x == 0 && counters)
            {
                atomicAdd(counters + 2 * (blockIdx.x & 63u), (unsigned long long) h);
                atomicAdd(counters + 2 * (blockIdx.x & 63u) + 1, (unsigned long long) (n - h));
            }
            if(n < 2 || h == n)
            {
                if(threadIdx.x < 32)
                    compactSupercell(sp, sc, rsm);
                return;
            }
        }
        else
        {
            n = sp.count[sc];
            if(n < 2)
                return;
        }
        uint32_t const newc = n - h;
        int const words = vol / 32;
        uint32_t* cnt = rsm + ReorderSmem::cnt(vol);
        uint32_t* bm = rsm + ReorderSmem::bm(vol);
        uint32_t* starts = rsm + ReorderSmem::starts(vol);
        uint16_t* rank = reinterpret_cast<uint16_t*>(rsm + ReorderSmem::rank(vol));
        uint16_t* inv = reinterpret_cast<uint16_t*>(rsm + ReorderSmem::inv(vol, sp.cap));
        uint32_t* buf = rsm + ReorderSmem::buf(vol, sp.cap);
        uint32_t* hb = rsm + ReorderSmem::holes(vol, sp.cap);
        size_t const base = size_t(sc) * sp.cap;
        for(int i = threadIdx.x; i < ReorderSmem::starts(vol); i += blockDim.x)
            rsm[i] = 0u;
        if constexpr(COMPACT)
            for(uint32_t i = threadIdx.x; i < (n + 31) / 32; i += blockDim.x)
                hb[i] = 0u;
        if(threadIdx.x == 0)
            s_tooFull = 0;
        __syncthreads();
        if constexpr(COMPACT)
        {
            for(uint32_t i = threadIdx.x; i < h; i += blockDim.x)
            {
                uint32_t const v = sp.holes[base + i];
                atomicOr(hb + (v >> 5), 1u << (v & 31u));
            }
            __syncthreads();
        }
        auto vacated = [&](uint32_t k) { return COMPACT && ((hb[k >> 5] >> (k & 31u)) & 1u); };
        for(uint32_t k0 = threadIdx.x; k0 < n; k0 += blockDim.x * kReorderLoads)
        {
            uint16_t lcs[kReorderLoads];
#pragma unroll
            for(int u = 0; u < kReorderLoads; ++u)
            {
                uint32_t const k = k0 + u * blockDim.x;
                lcs[u] = k < n ? sp.lcell[base + k] : uint16_t(0);
            }
#pragma unroll
            for(int u = 0; u < kReorderLoads; ++u)
            {
                uint32_t const k = k0 + u * blockDim.x;
                if(k >= n)
                    break;
                uint32_t const lc = lcs[u];
                buf[k] = lc;
                if(vacated(k))
                    continue;
                if(lc >= uint32_t(vol)) // not a cell of this supercell: leave the order alone
                {
                    s_tooFull = 1;
                    continue;
                }
                uint32_t const r = atomicAdd(cnt + lc, 1u);
                rank[k] = uint16_t(r < 65535u ? r : 65535u);
                if(r < uint32_t(kReorderRounds))
                    atomicOr(bm + r * words + lc / 32, 1u << (lc % 32));
                else
                    s_tooFull = 1;
            }
        }
        __syncthreads();
        if(s_tooFull) // uniform: every thread read it after the barrier
        {
            if constexpr(COMPACT)
            {
                __syncthreads(); // every thread is past its read of s_tooFull before rsm is reused
                if(threadIdx.x < 32)
                    compactSupercell(sp, sc, rsm);
            }
            return;
        }
        // first slot of every round: a prefix over the rounds' occupied cells
        if(threadIdx.x < 32)
        {
            uint32_t carry = 0;
            for(int r0 = 0; r0 < kReorderRounds; r0 += 32)
            {
                int const r = r0 + int(threadIdx.x);
                uint32_t tot = 0;
                for(int w = 0; w < words; ++w)
                    tot += __popc(bm[r * words + w]);
                uint32_t incl = tot;
#pragma unroll
                for(int o = 1; o < 32; o <<= 1)
                {
                    uint32_t const v = __shfl_up_sync(0xffffffffu, incl, o);
                    if(threadIdx.x >= unsigned(o))
                        incl += v;
                }
                starts[r] = carry + incl - tot;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
            if(threadIdx.x == 0)
                starts[kReorderRounds] = carry;
        }
        __syncthreads();
        for(uint32_t k = threadIdx.x; k < n; k += blockDim.x)
        {
            if(vacated(k))
                continue;
            uint32_t const lc = buf[k], r = rank[k];
            uint32_t const* row = bm + r * words;
            uint32_t before = 0;
            for(uint32_t w = 0; w < lc / 32; ++w)
                before += __popc(row[w]);
            before += __popc(row[lc / 32] & ((1u << (lc % 32)) - 1u));
            inv[starts[r] + before] = uint16_t(k);
        }
        __syncthreads();
        permuteInPlace(sp.px + base, n, newc, buf, inv);
        permuteInPlace(sp.py + base, n, newc, buf, inv);
        permuteInPlace(sp.pz + base, n, newc, buf, inv);
        permuteInPlace(sp.ux + base, n, newc, buf, inv);
        permuteInPlace(sp.uy + base, n, newc, buf, inv);
        permuteInPlace(sp.uz + base, n, newc, buf, inv);
        permuteInPlace(sp.w + base, n, newc, buf, inv);
        permuteInPlace(sp.lcell + base, n, newc, buf, inv);
        if(sp.id)
            permuteInPlace(sp.id + base, n, newc, buf, inv);
        if constexpr(COMPACT)
            if(threadIdx.x == 0)
            {
                sp.count[sc] = newc;
                sp.tail[sc] = newc;
                sp.nhole[sc] = 0u;
            }
    }

    __global__ void __launch_bounds__(kReorderThreads) kReorder(SpeciesDev sp, int vol)
    {
        extern __shared__ uint32_t rsm[];
        __shared__ int s_tooFull;
        reorderSupercell<false>(sp, int(blockIdx.x), vol, rsm, s_tooFull);
    }

    __global__ void __launch_bounds__(kReorderThreads) kCompactReorder(SpeciesDev sp, int vol, unsigned long long* counters)
    {
        extern __shared__ uint32_t rsm[];
        __shared__ int s_tooFull;
        reorderSupercell<true>(sp, int(blockIdx.x), vol, rsm, s_tooFull, counters);
    }

    // The reorder over the supercells of every box of an ensemble: block b handles work item b.
    __global__ void __launch_bounds__(kReorderThreads)
        kReorderBatch(BatchSpecies const* __restrict__ boxes, uint32_t const* __restrict__ items, int vol)
    {
        extern __shared__ uint32_t rsm[];
        __shared__ int s_tooFull;
        uint32_t const it = items[blockIdx.x];
        reorderSupercell<false>(boxes[batchBox(it)].sp, int(batchSc(it)), vol, rsm, s_tooFull);
    }

    size_t reorderSmemBytes(int vol, uint32_t cap) { return ReorderSmem::bytes(vol, cap); }

    cudaError_t launchReorder(SpeciesDev const& sp, int nsc, int vol, cudaStream_t stream)
    {
        size_t const smem = ReorderSmem::bytes(vol, sp.cap);
        if(smem > 48 * 1024)
        {
            cudaError_t e = cudaFuncSetAttribute(kReorder, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if(e != cudaSuccess)
                return e;
        }
        kReorder<<<nsc, kReorderThreads, smem, stream>>>(sp, vol);
        return cudaGetLastError();
    }

    cudaError_t launchCompactReorder(SpeciesDev const& sp, int nsc, int vol, unsigned long long* counters, cudaStream_t stream)
    {
        size_t const smem = ReorderSmem::bytes(vol, sp.cap);
        if(smem > 48 * 1024)
        {
            cudaError_t e = cudaFuncSetAttribute(kCompactReorder, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if(e != cudaSuccess)
                return e;
        }
        kCompactReorder<<<nsc, kReorderThreads, smem, stream>>>(sp, vol, counters);
        return cudaGetLastError();
    }

    cudaError_t launchReorderBatch(
        BatchSpecies const* boxes,
        uint32_t const* items,
        uint32_t nitems,
        int vol,
        uint32_t maxCap,
        cudaStream_t stream)
    {
        if(nitems == 0)
            return cudaSuccess;
        size_t const smem = ReorderSmem::bytes(vol, maxCap);
        if(smem > 48 * 1024)
        {
            cudaError_t e = cudaFuncSetAttribute(kReorderBatch, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if(e != cudaSuccess)
                return e;
        }
        kReorderBatch<<<nitems, kReorderThreads, smem, stream>>>(boxes, items, vol);
        return cudaGetLastError();
    }

    cudaError_t launchCompact(SpeciesDev const& sp, int nsc, cudaStream_t stream)
    {
        int const warps = compactWarps(sp.cap);
        int const words = int((sp.cap + 31) / 32);
        size_t const smem = sizeof(uint32_t) * 3 * size_t(words) * warps;
        if(smem > 48 * 1024)
        {
            cudaError_t e = cudaFuncSetAttribute(kCompact, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if(e != cudaSuccess)
                return e;
        }
        kCompact<<<(nsc + warps - 1) / warps, 32 * warps, smem, stream>>>(sp, nsc, words);
        return cudaGetLastError();
    }

    // ------------------------------------------------------------ upload
    // Occupancy per supercell; also validates the input: supercell and cell
    // indices in range and in-cell positions in [0, 1) (the kernels assume a
    // particle moves at most one cell per step from a valid in-cell position).
    // counter[key] += 1 for every lane of the warp with take set, as one atomic per group of
    // lanes with the same key: the group's lowest lane adds the group's size, and each lane
    // gets the old value plus its rank in the group.  Called by all 32 lanes together.
    __device__ __forceinline__ uint32_t warpAggregatedInc(uint32_t* counter, int key, bool take)
    {
        unsigned const lane = threadIdx.x & 31u;
        unsigned const takers = __ballot_sync(0xffffffffu, take);
        unsigned const peers = __match_any_sync(0xffffffffu, take ? key : -1) & takers;
        uint32_t old = 0u;
        if(take && lane == unsigned(__ffs(peers) - 1))
            old = atomicAdd(counter + key, unsigned(__popc(peers)));
        old = __shfl_sync(0xffffffffu, old, take ? __ffs(peers) - 1 : int(lane));
        return old + unsigned(__popc(peers & ((1u << lane) - 1u)));
    }

    __global__ void kHistogram(
        uint64_t n,
        int32_t const* __restrict__ sc,
        uint16_t const* __restrict__ lcell,
        float const* __restrict__ px,
        float const* __restrict__ py,
        float const* __restrict__ pz,
        uint32_t* count,
        int nsc,
        int vol,
        unsigned* status)
    {
        // warp-uniform trip count (blockDim.x is a multiple of 32), so the warp-wide
        // aggregation below has every lane present
        uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
        for(uint64_t i0 = blockIdx.x * uint64_t(blockDim.x) + (threadIdx.x & ~31u); i0 < n; i0 += stride)
        {
            uint64_t const i = i0 + (threadIdx.x & 31u);
            bool const valid = i < n;
            int s = -1;
            bool bad = false;
            if(valid)
            {
                s = sc[i];
                bad = s < 0 || s >= nsc || int(lcell[i]) >= vol;
                if(px)
                {
                    float const x = px[i], y = py[i], z = pz[i];
                    bad |= !(x >= 0.0f && x < 1.0f && y >= 0.0f && y < 1.0f && z >= 0.0f && z < 1.0f);
                }
                if(bad)
                    atomicOr(status, ST_BAD_CELL);
            }
            warpAggregatedInc(count, s, valid && !bad);
        }
    }

    // Largest |w| of n values as the bits of a non-negative float (ordered like the values; a
    // NaN reads above the bits of infinity).  *bits must be zero on entry.
    __global__ void kMaxAbsBits(uint64_t n, float const* __restrict__ w, unsigned* bits)
    {
        unsigned m = 0u;
        for(uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
        {
            unsigned const b = __float_as_uint(w[i]) & 0x7FFFFFFFu;
            m = b > m ? b : m;
        }
#pragma unroll
        for(int o = 16; o > 0; o >>= 1)
        {
            unsigned const v = __shfl_xor_sync(0xffffffffu, m, o);
            m = v > m ? v : m;
        }
        if((threadIdx.x & 31) == 0 && m)
            atomicMax(bits, m);
    }

    cudaError_t launchMaxAbsBits(float const* w, uint64_t n, unsigned* bits, cudaStream_t stream)
    {
        if(n == 0)
            return cudaSuccess;
        int const blocks = int(std::min<uint64_t>((n + 255) / 256, uint64_t(smCount()) * 16));
        kMaxAbsBits<<<blocks, 256, 0, stream>>>(n, w, bits);
        return cudaGetLastError();
    }

    cudaError_t launchHistogram(
        int scId,
        uint64_t n,
        int32_t const* sc,
        uint16_t const* lcell,
        float const* const* pos,
        uint32_t* count,
        int nsc,
        unsigned* status,
        cudaStream_t stream)
    {
        int const vol = scId == 0 ? 256 : (scId == 1 ? 64 : 512);
        if(n == 0)
            return cudaSuccess;
        int const blocks = int(std::min<uint64_t>((n + 255) / 256, uint64_t(smCount()) * 64));
        float const* px = pos ? pos[0] : nullptr;
        float const* py = pos ? pos[1] : nullptr;
        float const* pz = pos ? pos[2] : nullptr;
        kHistogram<<<blocks, 256, 0, stream>>>(n, sc, lcell, px, py, pz, count, nsc, vol, status);
        return cudaGetLastError();
    }

    struct Attr7
    {
        float const* a[7];
    };

    __global__ void kScatter(
        uint64_t n,
        Attr7 attr,
        int32_t const* __restrict__ sc,
        uint16_t const* __restrict__ lcell,
        uint32_t const* __restrict__ id,
        SpeciesDev sp,
        unsigned* status)
    {
        // warp-uniform trip count (blockDim.x is a multiple of 32); the input's supercell
        // indices were checked by kHistogram.  The lanes of a warp that share a supercell take
        // consecutive slots in lane order.
        uint64_t const stride = uint64_t(gridDim.x) * blockDim.x;
        for(uint64_t i0 = blockIdx.x * uint64_t(blockDim.x) + (threadIdx.x & ~31u); i0 < n; i0 += stride)
        {
            uint64_t const i = i0 + (threadIdx.x & 31u);
            bool const valid = i < n;
            int const s = valid ? sc[i] : -1;
            uint32_t const slot = warpAggregatedInc(sp.count, s, valid);
            if(!valid)
                continue;
            if(slot >= sp.cap)
            {
                atomicOr(status, ST_LOST);
                continue;
            }
            size_t const d = size_t(s) * sp.cap + slot;
            sp.px[d] = attr.a[0][i];
            sp.py[d] = attr.a[1][i];
            sp.pz[d] = attr.a[2][i];
            sp.ux[d] = attr.a[3][i];
            sp.uy[d] = attr.a[4][i];
            sp.uz[d] = attr.a[5][i];
            sp.w[d] = attr.a[6][i];
            sp.lcell[d] = lcell[i];
            if(sp.id)
                sp.id[d] = id ? id[i] : uint32_t(i);
        }
    }

    cudaError_t launchScatter(
        uint64_t n,
        float const* const* attr,
        int32_t const* sc,
        uint16_t const* lcell,
        uint32_t const* id,
        SpeciesDev const& sp,
        unsigned* status,
        cudaStream_t stream)
    {
        if(n == 0)
            return cudaSuccess;
        Attr7 a;
        for(int i = 0; i < 7; ++i)
            a.a[i] = attr[i];
        int const blocks = int(std::min<uint64_t>((n + 255) / 256, uint64_t(smCount()) * 64));
        kScatter<<<blocks, 256, 0, stream>>>(n, a, sc, lcell, id, sp, status);
        return cudaGetLastError();
    }

    // ------------------------------------------------------------ download
    struct OutAttr
    {
        float* a[7];
    };

    // Copy of `n` units of type T by the whole grid, four loads per thread and round in flight.
    template<typename T>
    __device__ __forceinline__ void copyUnits(T* __restrict__ d, T const* __restrict__ s, size_t n)
    {
        size_t const stride = size_t(gridDim.x) * blockDim.x;
        size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
        for(; i + 3 * stride < n; i += 4 * stride)
        {
            T const a = s[i], b = s[i + stride], c = s[i + 2 * stride], e = s[i + 3 * stride];
            d[i] = a;
            d[i + stride] = b;
            d[i + 2 * stride] = c;
            d[i + 3 * stride] = e;
        }
        for(; i < n; i += stride)
            d[i] = s[i];
    }

    // Host-to-device copy by the SMs: segment blockIdx.y in 16-byte units when both ends are
    // 16-byte aligned, else in 4-byte units when both are 4-byte aligned (an array offset by one
    // float), the rest byte by byte.
    __global__ void __launch_bounds__(256) kCopyIn(CopyJobs jobs)
    {
        CopySeg const sg = jobs.s[blockIdx.y];
        char* const d = static_cast<char*>(sg.dst);
        char const* const src = static_cast<char const*>(sg.src);
        uintptr_t const misalign = reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(src);
        size_t done = 0;
        if((misalign & 15u) == 0)
        {
            done = sg.bytes / 16 * 16;
            copyUnits(reinterpret_cast<uint4*>(d), reinterpret_cast<uint4 const*>(src), sg.bytes / 16);
        }
        else if((misalign & 3u) == 0)
        {
            done = sg.bytes / 4 * 4;
            copyUnits(reinterpret_cast<uint32_t*>(d), reinterpret_cast<uint32_t const*>(src), sg.bytes / 4);
        }
        size_t const stride = size_t(gridDim.x) * blockDim.x;
        for(size_t j = done + size_t(blockIdx.x) * blockDim.x + threadIdx.x; j < sg.bytes; j += stride)
            d[j] = src[j];
    }

    cudaError_t launchCopyIn(CopyJobs const& jobs, cudaStream_t stream)
    {
        if(jobs.n <= 0)
            return cudaSuccess;
        dim3 const grid(unsigned(smCount() * 2), unsigned(jobs.n));
        kCopyIn<<<grid, 256, 0, stream>>>(jobs);
        return cudaGetLastError();
    }

    // Output-major gather of a species into the host exchange format: output d belongs to the
    // last supercell whose offset is at most d (empty supercells share the offset of the next),
    // and is its slot d - offset.  Consecutive threads write consecutive outputs, so a warp's
    // stores to each array are whole aligned 128-byte lines even when the supercells' counts put
    // their ranges at arbitrary offsets (a supercell-major loop straddled lines, which costs
    // about a third of the host link's bandwidth when the arrays are host memory written over
    // the link); the reads stay contiguous within a supercell.
    __global__ void kGatherOut(
        SpeciesDev sp,
        uint64_t const* __restrict__ offsets,
        int nsc,
        uint64_t total,
        OutAttr out,
        int32_t* __restrict__ osc,
        uint16_t* __restrict__ olc,
        uint32_t* __restrict__ oid)
    {
        for(uint64_t d = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; d < total; d += uint64_t(gridDim.x) * blockDim.x)
        {
            int lo = 0, hi = nsc - 1;
            while(lo < hi)
            {
                int const mid = (lo + hi + 1) >> 1;
                if(__ldg(offsets + mid) <= d)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            int const sc = lo;
            size_t const s = size_t(sc) * sp.cap + size_t(d - __ldg(offsets + sc));
            out.a[0][d] = sp.px[s];
            out.a[1][d] = sp.py[s];
            out.a[2][d] = sp.pz[s];
            out.a[3][d] = sp.ux[s];
            out.a[4][d] = sp.uy[s];
            out.a[5][d] = sp.uz[s];
            out.a[6][d] = sp.w[s];
            osc[d] = sc;
            olc[d] = sp.lcell[s];
            if(oid)
                oid[d] = sp.id ? sp.id[s] : 0u;
        }
    }

    cudaError_t launchGatherOut(
        SpeciesDev const& sp,
        int nsc,
        uint64_t const* offsets,
        uint64_t total,
        float* const* attr,
        int32_t* sc,
        uint16_t* lcell,
        uint32_t* id,
        cudaStream_t stream)
    {
        if(total == 0)
            return cudaSuccess;
        OutAttr o;
        for(int i = 0; i < 7; ++i)
            o.a[i] = attr[i];
        uint64_t const blocks = std::min<uint64_t>((total + 255) / 256, uint64_t(smCount()) * 16);
        kGatherOut<<<unsigned(blocks), 256, 0, stream>>>(sp, offsets, nsc, total, o, sc, lcell, id);
        return cudaGetLastError();
    }

    // ------------------------------------------------------------ energies
    __device__ __forceinline__ double blockSumD(double v)
    {
        __shared__ double ws[32];
#pragma unroll
        for(int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if(lane == 0)
            ws[warp] = v;
        __syncthreads();
        double r = 0.0;
        if(warp == 0)
        {
            r = lane < int(blockDim.x >> 5) ? ws[lane] : 0.0;
#pragma unroll
            for(int o = 16; o > 0; o >>= 1)
                r += __shfl_down_sync(0xffffffffu, r, o);
        }
        __syncthreads();
        return r;
    }

    // KinEnergy (algorithms/KinEnergy.hpp:43-66) per macro particle in float,
    // summed in FP64.  A grid of resident blocks walks the supercells (one FP64 atomic per
    // block at the end instead of one per supercell).
    __global__ void kKineticEnergy(SpeciesDev sp, int nsc, float mass0, float c, double* out)
    {
        float const c2 = fm(c, c);
        // per thread and supercell a compensated float sum (compensatedAdd), as the reference
        // sums per thread in float_X, carried into an FP64 sum per thread after each supercell.
        // An FP64 add per particle runs on this GPU's narrow FP64 pipe.
        // The loads of kBatch particles are issued before their arithmetic, so a thread waits
        // for memory once per batch; the particles are summed in the same order as one at a time.
        constexpr int kBatch = 8;
        double acc = 0.0;
        for(int sc = blockIdx.x; sc < nsc; sc += gridDim.x)
        {
            uint32_t const n = sp.count[sc];
            size_t const base = size_t(sc) * sp.cap;
            float sum = 0.0f, comp = 0.0f;
            for(uint32_t k0 = threadIdx.x; k0 < n; k0 += kBatch * blockDim.x)
            {
                float wv[kBatch], uxv[kBatch], uyv[kBatch], uzv[kBatch];
#pragma unroll
                for(int b = 0; b < kBatch; ++b)
                {
                    uint32_t const k = k0 + b * blockDim.x;
                    size_t const s = base + (k < n ? k : 0u);
                    wv[b] = sp.w[s];
                    uxv[b] = sp.ux[s];
                    uyv[b] = sp.uy[s];
                    uzv[b] = sp.uz[s];
                }
#pragma unroll
                for(int b = 0; b < kBatch; ++b)
                {
                    if(k0 + b * blockDim.x >= n)
                        break;
                    float const m = fm(mass0, wv[b]);
                    float const mom2 = l2n2(uxv[b], uyv[b], uzv[b]);
                    float e;
                    if(m == 0.0f)
                        e = fm(c, fsq(mom2));
                    else
                    {
                        float const r = fdv(1.0f, fm(fm(m, m), c2));
                        float const gamma = fsq(fa(1.0f, fm(mom2, r)));
                        if(gamma < 1.005f)
                            e = fdv(mom2, fm(2.0f, m));
                        else
                            e = fm(fm(fs(gamma, 1.0f), m), c2);
                    }
                    compensatedAdd(sum, comp, e);
                }
            }
            acc += double(sum) + double(comp);
        }
        double const s = blockSumD(acc);
        if(threadIdx.x == 0 && s != 0.0)
            atomicAdd(out, s);
    }

    cudaError_t launchKineticEnergy(SpeciesDev const& sp, int nsc, float mass, float c, double* out, cudaStream_t stream)
    {
        if(nsc <= 0)
            return cudaSuccess;
        int const blocks = std::min(nsc, smCount() * 8);
        kKineticEnergy<<<blocks, 256, 0, stream>>>(sp, nsc, mass, c, out);
        return cudaGetLastError();
    }
} // namespace picgb
