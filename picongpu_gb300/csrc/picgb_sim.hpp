// Host-side state of one simulation handle (picgb_sim) and the helpers the
// host translation units share: error reporting, device allocation, species
// storage, the DataConnector-style registry entries.  Not part of the C-ABI.
#pragma once

#include "picgb.h"
#include "picgb_device.cuh"
#include "picgb_internal.hpp"
#include "picgb_pml.hpp"

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace picgb::host
{
    // Records the message for picgb_last_error() and returns `code`.
    int fail(int code, char const* fmt, ...);

#define CUDA_TRY(expr)                                                                                                \
    do                                                                                                                \
    {                                                                                                                 \
        cudaError_t e_ = (expr);                                                                                      \
        if(e_ != cudaSuccess)                                                                                         \
            return ::picgb::host::fail(                                                                               \
                PICGB_ERR_CUDA,                                                                                       \
                "%s failed: %s (%s:%d)",                                                                              \
                #expr,                                                                                                \
                cudaGetErrorString(e_),                                                                               \
                __FILE__,                                                                                             \
                __LINE__);                                                                                            \
    } while(0)

    template<typename T>
    cudaError_t dalloc(T*& p, size_t n)
    {
        p = nullptr;
        if(n == 0)
            return cudaSuccess;
        return cudaMalloc(reinterpret_cast<void**>(&p), n * sizeof(T));
    }

    template<typename T>
    void dfree(T*& p)
    {
        if(p)
            cudaFree(p);
        p = nullptr;
    }

    inline int scSize(int id, int* s)
    {
        static int const tab[3][3] = {{8, 8, 4}, {4, 4, 4}, {8, 8, 8}};
        if(id < 0 || id > 2)
            return 0;
        s[0] = tab[id][0];
        s[1] = tab[id][1];
        s[2] = tab[id][2];
        return 1;
    }

    struct Species
    {
        std::string name;
        picgb_species_config cfg{};
        SpeciesDev dev{};
        int nsc = 0;
        bool allocated = false;
        float wmax = 0.0f; // largest |weighting| (bounds a single J contribution)
        // compaction by the compacting reorder: its counters ([64][2] sums of vacated slots and of
        // remaining particles), whether the last launch wrote them, and whether the species
        // leaves its supercells often enough to take that path every step
        unsigned long long* leaveCount = nullptr;
        bool counted = false;
        bool hot = false;
        bool probe = false; // the next step measures the leave fraction (set by the plasma initialisation)

        void freeAll()
        {
            dfree(dev.px);
            dfree(dev.py);
            dfree(dev.pz);
            dfree(dev.ux);
            dfree(dev.uy);
            dfree(dev.uz);
            dfree(dev.w);
            dfree(dev.lcell);
            dfree(dev.id);
            dfree(dev.count);
            dfree(dev.tail);
            dfree(dev.nhole);
            dfree(dev.holes);
            dfree(dev.sp_attr);
            dfree(dev.sp_sc);
            dfree(dev.sp_lcell);
            dfree(dev.sp_id);
            dfree(dev.sp_count);
            dfree(leaveCount);
            counted = false;
            allocated = false;
        }
    };

    // Registry entry (pmacc/dataManagement/DataConnector.hpp:48-136): either an
    // internal buffer (field or species, resolved at lookup so relayouts are
    // seen) or caller-shared device data.
    struct Entry
    {
        enum Kind
        {
            FieldE,
            FieldB,
            FieldJ,
            FieldTmp,
            SpeciesBuf,
            Opaque,
            External
        } kind;
        int index = 0;
        picgb_buffer_desc desc{};
    };
} // namespace picgb::host

struct picgb_sim
{
    picgb_grid_config cfg{};
    picgb::GridParams g{};
    int sc[3] = {8, 8, 4};
    int nsc = 0;
    size_t ncell = 0;
    float* E = nullptr;
    float* B = nullptr;
    float* J = nullptr;
    float* rho = nullptr;
    unsigned* status = nullptr; // device status word
    unsigned* hostStatus = nullptr; // pinned
    void* ioBuf = nullptr; // staging of species uploads and downloads, kept between calls
    size_t ioBytes = 0;
    double* energy = nullptr; // device accumulators
    unsigned* maxBits = nullptr; // device: residual max, rho max
    unsigned long long* kindCount = nullptr; // device: deposits by footprint (profiling)
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    bool inEnsemble = false; // owned by a picgb_ensemble: not destroyed through picgb_destroy
    picgb::IncidentParams inc[picgb::kIncidentFaces]{}; // incident pulses by TF/SF face, all disabled by default
    int absorberThick[3][2] = {}; // absorber cells at the low and high face of each open axis (0 when periodic)
    picgb::PmlDev pml{}; // open boundaries: convolution fields and coefficient tables (g.open != 0)
    float* pmlTab = nullptr;
    float* expDamp = nullptr; // exponential absorber: damping factors [3][pml.nmax], or null
    uint64_t launches = 0;
    std::vector<std::unique_ptr<picgb::host::Species>> species;
    std::map<std::string, picgb::host::Entry> registry;
    // per-kernel event timing (picgb_profile_enable)
    bool prof = false;
    struct Pending
    {
        int cls;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> eventPool;
    double profMs[PICGB_KERNEL_CLASSES] = {};
    uint64_t profN[PICGB_KERNEL_CLASSES] = {};
    // interleaved order restored every sortInterval steps (0: never)
    uint32_t sortInterval = 20;
    uint32_t stepsSinceSort = 0;

    float coeffJ() const { return -(1.0f / cfg.eps0) * cfg.dt; } // FDTD.hpp:84
    float cellVolume() const
    {
        float v = cfg.dx * cfg.dy;
        v = v * cfg.dz;
        return v;
    }
    // Push parameters of one species, including the fixed-point format of the J tile.
    picgb::PushParams pushParams(picgb::host::Species const& s, bool deposit) const;
};

namespace picgb::host
{
    int checkSim(picgb_sim* s);
    bool hasCurrent(Species const& sp);
    // Reads (and optionally clears) the device status word; synchronises the stream.
    int readStatus(picgb_sim* s, unsigned* bits, bool reset);
    // Re-inserts spilled particles after an overflow; synchronises the stream.
    int afterStep(picgb_sim* s);
    // Frees every device resource of a handle.
    int destroySim(picgb_sim* s);
} // namespace picgb::host
