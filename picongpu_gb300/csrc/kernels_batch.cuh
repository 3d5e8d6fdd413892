// Push kernel of a batched ensemble: many independent periodic boxes of uneven
// size in one launch per species, so large and small boxes share the GPU without
// a launch per box.  Each work item (box, supercell) runs the same supercell push
// as the single-box kernel (kernels_push.cuh) on that box's fields and particles.
// The items are ordered with the largest boxes first.  By default each item is one
// block and the hardware's block scheduler hands them out in order; the persistent
// form (PICGB_BATCH_PERSISTENT=1: a grid of resident blocks taking items from a
// global counter) gives the same results and measured 4 to 5 % slower, its blocks
// meeting at a barrier between items.
//
// The grid and push parameters that every box of the launch shares (cell size, time
// step, speed of light, the species' charge, mass and pusher) are kernel arguments, as
// in the single-box kernel: the compiler uses them as constant-bank operands.  Only
// what differs between boxes comes from the work item's descriptor in shared memory:
// the box's extent, its storage and field pointers and the fixed-point format of its J
// tile.  With the whole GridParams and PushParams taken from the shared descriptor, the
// 512-thread kernel held those values in registers and spilled 104 bytes per thread
// inside the particle loop (2.3 GB of local-memory loads per launch on one 128^3
// two-stream box, 17 % slower than the single-box kernel on the same box).
#pragma once

#include "kernels_push.cuh"
#include "picgb_batch.hpp"

namespace picgb
{
#ifndef PICGB_BATCH_MIN_BLOCKS
    // resident 256-thread blocks per SM the batched kernel's register budget is sized for
#    define PICGB_BATCH_MIN_BLOCKS 3
#endif

    // Resident blocks the batched kernel's register budget is sized for (512 threads:
    // two blocks at 64 registers, as the single-box kernel).
    template<int THREADS>
    constexpr int batchMinBlocks()
    {
        return THREADS >= 512 ? 2 : (THREADS >= 256 ? PICGB_BATCH_MIN_BLOCKS : 2 * PICGB_BATCH_MIN_BLOCKS);
    }

#ifndef PICGB_BATCH_PERSISTENT
    // 1: a grid of resident blocks takes work items from a counter; 0: one block per work
    // item, in the items' order, handed out by the hardware's block scheduler
#    define PICGB_BATCH_PERSISTENT 0
#endif

    // Copy of work item `it`'s box descriptor (it < nitems) into shared memory by `nthreads`
    // threads (thread index t).
    __device__ __forceinline__ void loadBox(
        BatchSpecies const* __restrict__ table,
        uint32_t const* __restrict__ items,
        uint32_t it,
        int t,
        int nthreads,
        BatchSpecies& dst)
    {
        static_assert(sizeof(BatchSpecies) % 4 == 0, "BatchSpecies is copied as 32-bit words");
        constexpr int kWords = int(sizeof(BatchSpecies) / 4);
        uint32_t const* src = reinterpret_cast<uint32_t const*>(table + batchBox(__ldg(items + it)));
        for(int i = t; i < kWords; i += nthreads)
            reinterpret_cast<uint32_t*>(&dst)[i] = __ldg(src + i);
    }

    // The persistent kernel's hook inside the supercell push: thread 0 takes the next work
    // item from the counter while the block pushes particles, so the hand-over at the end of
    // the item does not wait for the counter.
    struct NextItem
    {
        uint32_t* counter;
        uint32_t* item; // the block's next item (>= nitems: no more work)

        __device__ void operator()() const
        {
            if(threadIdx.x == 0)
                *item = atomicAdd(counter, 1u);
        }
    };

    // One work item v = (box, supercell) whose descriptor is in s_box: the supercell push
    // with the launch's shared parameters and the box's own extent and J tile.
    template<int SHAPE, int SX, int SY, int SZ, int THREADS, bool ALT, bool EMZ, typename Hook>
    __device__ __forceinline__ void pushItem(
        BatchSpecies const& s_box,
        uint32_t const v,
        unsigned* __restrict__ status,
        GridParams const& g0,
        PushParams const& pp0,
        float* const smem,
        unsigned& s_nhole,
        Hook const& hook)
    {
        GridParams g = g0; // the box's extent over the shared grid parameters
        g.nx = s_box.g.nx;
        g.ny = s_box.g.ny;
        g.nz = s_box.g.nz;
        g.nscx = s_box.g.nscx;
        g.nscy = s_box.g.nscy;
        g.nscz = s_box.g.nscz;
        PushParams pp = pp0; // the box's J-tile format over the species' parameters
        pp.jf = s_box.pp.jf;
        pushSupercell<SHAPE, SX, SY, SZ, THREADS, ALT, EMZ>(
            s_box.sp,
            s_box.E,
            s_box.B,
            s_box.J,
            g,
            pp,
            status,
            int(batchSc(v)),
            smem,
            s_nhole,
            hook);
    }

    template<int SHAPE, int SX, int SY, int SZ, int THREADS, bool ALT, bool EMZ>
    __global__ void __launch_bounds__(THREADS, batchMinBlocks<THREADS>()) kPushBatch(
        BatchSpecies const* __restrict__ table,
        uint32_t const* __restrict__ items,
        uint32_t nitems,
        uint32_t* __restrict__ counter,
        unsigned* __restrict__ status,
        GridParams const g0,
        PushParams const pp0)
    {
        extern __shared__ __align__(16) float smem[];
        __shared__ unsigned s_nhole;
#if PICGB_BATCH_PERSISTENT
        __shared__ __align__(16) BatchSpecies s_box;
        __shared__ uint32_t s_item;
        if(threadIdx.x == 0)
            s_item = atomicAdd(counter, 1u);
        __syncthreads();
        for(;;)
        {
            uint32_t const it = s_item;
            if(it >= nitems)
                break;
            loadBox(table, items, it, int(threadIdx.x), THREADS, s_box);
            __syncthreads(); // every thread has read s_item; the descriptor is complete
            pushItem<SHAPE, SX, SY, SZ, THREADS, ALT, EMZ>(s_box, __ldg(items + it), status, g0, pp0, smem, s_nhole,
                                                            NextItem{counter, &s_item});
            __syncthreads(); // the next item reuses the tiles and the descriptor; s_item is set
        }
#else
        __shared__ __align__(16) BatchSpecies s_box;
        if(blockIdx.x >= nitems)
            return;
        loadBox(table, items, blockIdx.x, int(threadIdx.x), THREADS, s_box);
        __syncthreads();
        pushItem<SHAPE, SX, SY, SZ, THREADS, ALT, EMZ>(s_box, __ldg(items + blockIdx.x), status, g0, pp0, smem, s_nhole,
                                                        NoHook{});
#endif
    }

    template<int SHAPE, int SX, int SY, int SZ, int THREADS, bool ALT, bool EMZ>
    cudaError_t launchPushBatchT(
        BatchSpecies const* table,
        uint32_t const* items,
        uint32_t nitems,
        uint32_t* counter,
        unsigned* status,
        GridParams const& g0,
        PushParams const& pp0,
        cudaStream_t stream)
    {
        using TG = TileGeom<Shape<SHAPE>, SuperCell<SX, SY, SZ>, THREADS>;
        auto k = kPushBatch<SHAPE, SX, SY, SZ, THREADS, ALT, EMZ>;
        size_t const smem = TG::pushSmem;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if(e != cudaSuccess)
            return e;
        int occ = 0, dev = 0, nsm = 0;
        if((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, THREADS, smem)) != cudaSuccess)
            return e;
        if((e = cudaGetDevice(&dev)) != cudaSuccess)
            return e;
        if((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
            return e;
        if(occ < 1)
            return cudaErrorInvalidConfiguration;
        uint32_t const blocks = PICGB_BATCH_PERSISTENT ? std::min<uint32_t>(uint32_t(occ) * uint32_t(nsm), nitems) : nitems;
        if(blocks == 0)
            return cudaSuccess;
        k<<<blocks, THREADS, smem, stream>>>(table, items, nitems, counter, status, g0, pp0);
        return cudaGetLastError();
    }

// Instantiates the batched launcher of one shape, pusher variant (ALT: HigueraCary and Vay)
// and current scheme (EMZ: EmZ, else Esirkepov) for the supercell sizes 8x8x4, 4x4x4,
// 8x8x8 and 128, 256 or 512 threads per supercell.  Each combination has its own
// translation unit, so the heaviest instantiations compile in parallel.
#define PICGB_BATCH_CASES(F, SHAPE, ALT, EMZ, ...)                                                                    \
    switch(scId * 3 + (threads == 128 ? 0 : (threads == 256 ? 1 : 2)))                                               \
    {                                                                                                                 \
    case 0:                                                                                                           \
        return F<SHAPE, 8, 8, 4, 128, ALT, EMZ>(__VA_ARGS__);                                                         \
    case 1:                                                                                                           \
        return F<SHAPE, 8, 8, 4, 256, ALT, EMZ>(__VA_ARGS__);                                                         \
    case 2:                                                                                                           \
        return F<SHAPE, 8, 8, 4, 512, ALT, EMZ>(__VA_ARGS__);                                                         \
    case 3:                                                                                                           \
        return F<SHAPE, 4, 4, 4, 128, ALT, EMZ>(__VA_ARGS__);                                                         \
    case 4:                                                                                                           \
        return F<SHAPE, 4, 4, 4, 256, ALT, EMZ>(__VA_ARGS__);                                                         \
    case 5:                                                                                                           \
        return F<SHAPE, 4, 4, 4, 512, ALT, EMZ>(__VA_ARGS__);                                                         \
    case 6:                                                                                                           \
        return F<SHAPE, 8, 8, 8, 128, ALT, EMZ>(__VA_ARGS__);                                                         \
    case 7:                                                                                                           \
        return F<SHAPE, 8, 8, 8, 256, ALT, EMZ>(__VA_ARGS__);                                                         \
    case 8:                                                                                                           \
        return F<SHAPE, 8, 8, 8, 512, ALT, EMZ>(__VA_ARGS__);                                                         \
    }

#define PICGB_BATCH_LAUNCHERS(SHAPE, NAME, ALT, EMZ)                                                                  \
    cudaError_t launchPushBatch##NAME(                                                                                \
        int scId,                                                                                                     \
        int threads,                                                                                                  \
        BatchSpecies const* table,                                                                                    \
        uint32_t const* items,                                                                                        \
        uint32_t nitems,                                                                                              \
        uint32_t* counter,                                                                                            \
        unsigned* status,                                                                                             \
        GridParams const& g0,                                                                                         \
        PushParams const& pp0,                                                                                        \
        cudaStream_t stream)                                                                                          \
    {                                                                                                                 \
        if(threads != 128 && threads != 256 && threads != 512)                                                        \
            return cudaErrorInvalidValue;                                                                             \
        PICGB_BATCH_CASES(launchPushBatchT, SHAPE, ALT, EMZ, table, items, nitems, counter, status, g0, pp0, stream)\
        return cudaErrorInvalidValue;                                                                                 \
    }
} // namespace picgb
