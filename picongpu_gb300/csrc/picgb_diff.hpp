// Launchers of the differentiable PIC step (kernels_diff.cu).  Not part of the C-ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace picgb::diff
{
    struct DiffGridDesc
    {
        int nx, ny, nz;
        double dx, dy, dz, dt, c, eps0;
    };

    // One species in device memory: cell [3][n] int32, pos and mom [3][n] T, w [n] T.
    struct DiffSpeciesPtr
    {
        int32_t* cell;
        void* pos;
        void* mom;
        void const* w;
        uint64_t n;
        double charge, mass; // per real particle
        // where the push writes the new cell, pos, mom (null: in place)
        int32_t* cellOut = nullptr;
        void* posOut = nullptr;
        void* momOut = nullptr;
    };

    // precision: 4 (float) or 8 (double); shape: 1 CIC, 2 TSC, 3 PQS
    cudaError_t launchDiffPush(
        int precision,
        int shape,
        DiffSpeciesPtr const& s,
        void const* E,
        void const* B,
        void* J,
        void* gathered, // [24][n]: gathered E, B and their position gradients are stored here, or null
        DiffGridDesc const& g,
        cudaStream_t st);
    cudaError_t launchDiffAdjoint(
        int precision,
        int shape,
        DiffSpeciesPtr const& s,
        void const* E,
        void const* B,
        void const* lamJ,
        void* lamE,
        void* lamB,
        void* lamPos,
        void* lamMom,
        void const* gathered, // [24][n] from launchDiffPush of the same step, or null (gathered again)
        DiffGridDesc const& g,
        cudaStream_t st);
    // A += alpha * curl(F) (3-component SoA fields), forward or backward differences
    cudaError_t launchDiffCurlAdd(
        int precision,
        void* A,
        void const* F,
        double alpha,
        bool forward,
        DiffGridDesc const& g,
        cudaStream_t st);
    // y = a x + b y over n values
    cudaError_t launchDiffAxpby(int precision, void* y, double a, void const* x, double b, size_t n, cudaStream_t st);
    // out += sum of (gamma - 1) m w c^2 in FP64
    cudaError_t launchDiffKinetic(int precision, DiffSpeciesPtr const& s, double c, double* out, cudaStream_t st);
} // namespace picgb::diff
