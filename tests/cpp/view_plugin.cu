// A C++ host program that drives the PIC step through include/picgb.h stage by stage
// (the loop of Simulation::runOneStep, simulation/control/Simulation.hpp:522-542) and
// runs two plugins written the way PIConGPU's EnergyFields and EnergyParticles read the
// hot path's data, through the reference-layout views of include/picgb_view.hpp:
//   * EnergyFields::reduceField (plugins/EnergyFields.x.cpp:241-261): the DataBox of E
//     and B shifted by the guard, squares per component in float, cast to double,
//     summed over the core cells, times eps0 V / 2 and V / (2 mu0);
//   * EnergyParticles (plugins/EnergyParticles.x.cpp:58-160, algorithms/KinEnergy.hpp:38-66):
//     every supercell's frames from getFirstFrame to the end of getNextFrame, the
//     kinetic energy of every particle slot that holds a particle.
// Both must match picgb_energies (E and B within 1e-12 relative: the same float
// squares summed in double in another order; kinetic energy within 1e-6: float energies
// per particle, FP64 sums), the frames must visit every particle once, and guard indices
// of the DataBox must read the periodic neighbours.  Exit status 0 when all hold.
#include "picgb.h"
#include "picgb_view.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

using picgb::view::DataSpace3;
using picgb::view::FieldBox;
using picgb::view::Float3;
using picgb::view::FramePtr;
using picgb::view::ParticlesBox;

#define CHECK(call)                                                                                                   \
    do                                                                                                                \
    {                                                                                                                 \
        int r_ = (call);                                                                                              \
        if(r_ != PICGB_OK)                                                                                            \
        {                                                                                                             \
            std::fprintf(stderr, "%s failed (%d): %s\n", #call, r_, picgb_last_error());                              \
            return 1;                                                                                                 \
        }                                                                                                             \
    } while(0)

#define CUDA_CHECK(call)                                                                                              \
    do                                                                                                                \
    {                                                                                                                 \
        cudaError_t e_ = (call);                                                                                      \
        if(e_ != cudaSuccess)                                                                                         \
        {                                                                                                             \
            std::fprintf(stderr, "%s failed: %s\n", #call, cudaGetErrorString(e_));                                   \
            return 1;                                                                                                 \
        }                                                                                                             \
    } while(0)

// squareComponentWise then cast64Bit, reduced over the core cells of the shifted box
__global__ void kReduceFieldSquares(FieldBox box, DataSpace3 size, double* out3)
{
    double acc[3] = {0.0, 0.0, 0.0};
    int64_t const n = size.productOfComponents();
    for(int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        DataSpace3 const c{int(i % size.x), int((i / size.x) % size.y), int(i / (int64_t(size.x) * size.y))};
        Float3 const v = box(c);
        for(int d = 0; d < 3; ++d)
            acc[d] += double(__fmul_rn(v[d], v[d]));
    }
    for(int d = 0; d < 3; ++d)
        atomicAdd(out3 + d, acc[d]);
}

// kinetic energy of every particle reached through the frame lists, and the particle count
__global__ void kParticleEnergy(ParticlesBox box, float mass0, float c, double* energy, unsigned long long* count)
{
    int64_t const sc = blockIdx.x;
    DataSpace3 const idx{int(sc % box.superCells.x), int((sc / box.superCells.x) % box.superCells.y),
                         int(sc / (int64_t(box.superCells.x) * box.superCells.y))};
    double acc = 0.0;
    unsigned long long n = 0;
    for(FramePtr f = box.getFirstFrame(idx); f.isValid(); f = box.getNextFrame(f))
        for(uint32_t i = threadIdx.x; i < box.frameSize; i += blockDim.x)
        {
            if(!f.isParticle(i))
                continue;
            Float3 const p = f.momentum(i);
            float const m = mass0 * f.weighting(i);
            float const mom2 = p.x * p.x + p.y * p.y + p.z * p.z;
            float const gamma = sqrtf(1.0f + mom2 / (m * m * c * c));
            float const e = gamma < 1.005f ? mom2 / (2.0f * m) : (gamma - 1.0f) * m * c * c;
            acc += double(e);
            ++n;
        }
    atomicAdd(energy, acc);
    atomicAdd(count, n);
}

// the box read at guard indices: the periodic neighbours of the first and last core cells
__global__ void kGuardProbe(FieldBox raw, FieldBox core, DataSpace3 size, float* out)
{
    DataSpace3 const lowGuard{-1, 0, 0}, lastCore{size.x - 1, 0, 0};
    out[0] = Float3(core(lowGuard)).y;
    out[1] = Float3(core(lastCore)).y;
    // the unshifted box starts at the lower guard corner
    DataSpace3 const g = raw.getGridLayout().guardSizeND();
    out[2] = Float3(raw(g)).z;
    out[3] = Float3(core(DataSpace3{0, 0, 0})).z;
    out[4] = Float3(core(DataSpace3{size.x, size.y, size.z})).x; // upper guard corner = core (0,0,0)
    out[5] = Float3(core(DataSpace3{0, 0, 0})).x;
}

int main()
{
    picgb_grid_config g{};
    g.nx = 32;
    g.ny = 32;
    g.nz = 32;
    g.supercell = PICGB_SUPERCELL_8x8x4;
    g.dx = g.dy = g.dz = 1.0f;
    g.c = 1.0f;
    g.eps0 = 1.0f;
    g.dt = 0.99f / std::sqrt(3.0f);
    g.field_solver = PICGB_SOLVER_YEE;
    g.fuse_deposit = 1;
    g.device = 0;
    picgb_sim* sim = nullptr;
    CHECK(picgb_create(&g, &sim));
    picgb_species_config e{"e", -1.0f, 1.0f, PICGB_PUSHER_BORIS, PICGB_SHAPE_TSC, PICGB_CURRENT_ESIRKEPOV, 0, 0};
    picgb_species_config i{"i", 1.0f, 1836.0f, PICGB_PUSHER_BORIS, PICGB_SHAPE_TSC, PICGB_CURRENT_ESIRKEPOV, 0, 0};
    int32_t ie = -1, ii = -1;
    CHECK(picgb_add_species(sim, &e, &ie));
    CHECK(picgb_add_species(sim, &i, &ii));
    float const wp = 0.1f / g.dt;
    float const drift = 0.2f / std::sqrt(1.0f - 0.04f);
    picgb_plasma_init pe{8, wp * wp, 0.01f, {drift, 0.0f, 0.0f}, {-drift, 0.0f, 0.0f}, 1, 16, 1, 7};
    picgb_plasma_init pi{8, wp * wp, 0.01f / std::sqrt(1836.0f), {0, 0, 0}, {0, 0, 0}, -1, 0, 2, 7};
    CHECK(picgb_species_init_plasma(sim, ie, &pe));
    CHECK(picgb_species_init_plasma(sim, ii, &pi));
    for(uint32_t step = 0; step < 20; ++step)
    {
        CHECK(picgb_stage_current_reset(sim));
        CHECK(picgb_stage_push(sim, step));
        CHECK(picgb_stage_field_before(sim, step));
        CHECK(picgb_stage_deposit(sim, step));
        CHECK(picgb_stage_add_current(sim));
        CHECK(picgb_stage_field_after(sim, step));
    }
    CHECK(picgb_synchronize(sim));

    double lib[4] = {0, 0, 0, 0};
    CHECK(picgb_energies(sim, lib, 4));

    // the plugins: DataConnector::get through picgb_get_buffer, reference-layout views
    DataSpace3 const guard{8, 8, 4}; // one supercell, param/memory.param:73
    FieldBox fe, fb;
    CHECK(picgb::view::makeFieldBox(sim, "E", guard, &fe));
    CHECK(picgb::view::makeFieldBox(sim, "B", guard, &fb));
    DataSpace3 const size = fe.getGridLayout().sizeWithoutGuardND();
    double* d = nullptr;
    unsigned long long* cnt = nullptr;
    float* probe = nullptr;
    CUDA_CHECK(cudaMalloc(&d, 8 * sizeof(double)));
    CUDA_CHECK(cudaMalloc(&cnt, 2 * sizeof(unsigned long long)));
    CUDA_CHECK(cudaMalloc(&probe, 6 * sizeof(float)));
    CUDA_CHECK(cudaMemset(d, 0, 8 * sizeof(double)));
    CUDA_CHECK(cudaMemset(cnt, 0, 2 * sizeof(unsigned long long)));
    kReduceFieldSquares<<<64, 256>>>(fe.shift(fe.getGridLayout().guardSizeND()), size, d);
    kReduceFieldSquares<<<64, 256>>>(fb.shift(fb.getGridLayout().guardSizeND()), size, d + 3);
    ParticlesBox pbe, pbi;
    CHECK(picgb::view::makeParticlesBox(sim, "e", guard, &pbe));
    CHECK(picgb::view::makeParticlesBox(sim, "i", guard, &pbi));
    int const nsc = int(pbe.superCells.productOfComponents());
    kParticleEnergy<<<nsc, 128>>>(pbe, e.mass, g.c, d + 6, cnt);
    kParticleEnergy<<<nsc, 128>>>(pbi, i.mass, g.c, d + 7, cnt + 1);
    kGuardProbe<<<1, 1>>>(fe, fe.shift(guard), size, probe);
    CUDA_CHECK(cudaGetLastError());
    double h[8];
    unsigned long long hc[2];
    float hp[6];
    CUDA_CHECK(cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost));
    CUDA_CHECK(cudaMemcpy(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost));
    CUDA_CHECK(cudaMemcpy(hp, probe, sizeof(hp), cudaMemcpyDeviceToHost));

    double const V = double(g.dx) * g.dy * g.dz;
    double const eps0 = g.eps0, mu0 = 1.0 / (double(g.eps0) * g.c * g.c);
    double const plugE = (h[0] + h[1] + h[2]) * eps0 * V * 0.5;
    double const plugB = (h[3] + h[4] + h[5]) * 0.5 / mu0 * V;
    uint64_t ne = 0, ni = 0;
    CHECK(picgb_species_count(sim, ie, &ne));
    CHECK(picgb_species_count(sim, ii, &ni));
    int fails = 0;
    auto rel = [](double a, double b) { return std::fabs(a - b) / std::fmax(std::fabs(b), 1e-300); };
    std::printf("field E: plugin %.15e library %.15e\n", plugE, lib[0]);
    std::printf("field B: plugin %.15e library %.15e\n", plugB, lib[1]);
    std::printf("kinetic e: plugin %.15e library %.15e; i: %.15e %.15e\n", h[6], lib[2], h[7], lib[3]);
    std::printf("frames visited %llu + %llu particles, species hold %llu + %llu\n", hc[0], hc[1],
                (unsigned long long) ne, (unsigned long long) ni);
    if(!(lib[0] > 0.0 && rel(plugE, lib[0]) <= 1e-12))
        ++fails, std::printf("FAIL: E field energy\n");
    if(!(lib[1] > 0.0 && rel(plugB, lib[1]) <= 1e-12))
        ++fails, std::printf("FAIL: B field energy\n");
    if(!(rel(h[6], lib[2]) <= 1e-6 && rel(h[7], lib[3]) <= 1e-6))
        ++fails, std::printf("FAIL: kinetic energies\n");
    if(hc[0] != ne || hc[1] != ni)
        ++fails, std::printf("FAIL: particle counts through the frames\n");
    if(hp[0] != hp[1] || hp[2] != hp[3] || hp[4] != hp[5])
        ++fails, std::printf("FAIL: guard indices do not read the periodic neighbours\n");
    cudaFree(d);
    cudaFree(cnt);
    cudaFree(probe);
    CHECK(picgb_destroy(sim));
    std::printf(fails ? "view plugin: %d failures\n" : "view plugin: OK\n", fails);
    return fails ? 1 : 0;
}
