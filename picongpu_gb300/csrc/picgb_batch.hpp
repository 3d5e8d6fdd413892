// Device tables of a batched ensemble: many independent periodic boxes whose
// particle and field kernels run as single launches over all boxes.  Not part
// of the C-ABI.
#pragma once

#include "picgb_device.cuh"
#include "picgb_internal.hpp"

namespace picgb
{
    // One box's fields and the range of field blocks it owns in a batched field launch.
    struct BatchBox
    {
        GridParams g;
        float* E;
        float* B;
        float* J;
        float coeffJ; // -dt / eps0 (FDTD.hpp:84)
        uint32_t block0; // first block of this box in the field launches
    };

    // One species of one box: everything the push of one of its supercells needs.
    struct BatchSpecies
    {
        SpeciesDev sp;
        PushParams pp;
        GridParams g;
        float const* E;
        float const* B;
        float* J;
    };

    // Work item = (box, supercell of that box), packed in 32 bits.
    constexpr int kBatchScBits = 20;
    constexpr uint32_t kBatchMaxSc = 1u << kBatchScBits;
    constexpr uint32_t kBatchMaxBoxes = 1u << (32 - kBatchScBits);
    constexpr int kBatchFieldThreads = 256;

    __host__ __device__ inline uint32_t batchItem(uint32_t box, uint32_t sc) { return (box << kBatchScBits) | sc; }
    __host__ __device__ inline uint32_t batchBox(uint32_t it) { return it >> kBatchScBits; }
    __host__ __device__ inline uint32_t batchSc(uint32_t it) { return it & (kBatchMaxSc - 1u); }

    // Push over every work item, one launch per species: one block per item, or (built with
    // PICGB_BATCH_PERSISTENT=1) resident blocks taking items from `*counter`, which is zero
    // at launch.  g0 and pp0
    // hold what every box shares (cell size, time step, c, eps0, the open-axis bits; the
    // species' charge, mass, pusher and current); the table supplies each box's extent,
    // storage, fields and J-tile format.
    cudaError_t launchPushBatch(
        int shape,
        int scId,
        int threads,
        int pusher, // selects the kernel variant (Boris/Free or HigueraCary/Vay)
        int current, // Esirkepov or EmZ
        BatchSpecies const* table,
        uint32_t const* items,
        uint32_t nitems,
        uint32_t* counter,
        unsigned* status,
        GridParams const& g0,
        PushParams const& pp0,
        cudaStream_t stream);
    // kReorder over every work item; maxCap = the largest slots per supercell of any box.
    cudaError_t launchReorderBatch(
        BatchSpecies const* boxes,
        uint32_t const* items,
        uint32_t nitems,
        int vol,
        uint32_t maxCap,
        cudaStream_t stream);
    cudaError_t launchCompactBatch(
        BatchSpecies const* boxes,
        uint32_t const* items,
        uint32_t nitems,
        uint32_t maxCap,
        cudaStream_t stream);
    // Field kernels over all boxes: block b works on box blockBox[b].
    cudaError_t launchYeeBHalfBatch(BatchBox const* boxes, uint32_t const* blockBox, uint32_t nblocks, cudaStream_t stream);
    cudaError_t launchYeeEBatch(BatchBox const* boxes, uint32_t const* blockBox, uint32_t nblocks, cudaStream_t stream);
    cudaError_t launchZeroJBatch(BatchBox const* boxes, uint32_t const* blockBox, uint32_t nblocks, cudaStream_t stream);
} // namespace picgb
