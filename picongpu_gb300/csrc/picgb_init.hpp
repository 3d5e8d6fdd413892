// Parameters of the seeded plasma initialisation (kernels_init.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace picgb
{
    struct GridParams;
    struct SpeciesDev;

    struct InitParams
    {
        uint32_t ppc; // macro particles per cell
        float weight; // macro weighting
        float mass; // mass of one real particle
        float c; // speed of light
        float u_th; // thermal spread of u = gamma * beta per component
        float drift_lo[3]; // mean u where the split coordinate is below split_cell
        float drift_hi[3]; // mean u at and above split_cell
        int split_axis; // -1: drift_lo everywhere
        int split_cell;
        uint64_t seed; // momenta
        uint64_t position_seed; // positions (species sharing it get identical positions)
        uint32_t quiet[3]; // lattice per axis (startPosition::Quiet); quiet[0] == 0: random positions
    };

    cudaError_t launchInitPlasma(
        SpeciesDev const& sp,
        GridParams const& g,
        InitParams const& ip,
        int const* supercell,
        cudaStream_t stream);
} // namespace picgb
