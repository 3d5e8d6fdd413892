// Internal declarations shared by the host runtime (picgb_api.cu) and the
// kernel translation units.  Not part of the C-ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace picgb
{
    struct GridParams; // picgb_device.cuh

    // Multiprocessors of the current device, for sizing grid-stride launches (queried once
    // per device; 152, the GB300's count, if the query fails).
    inline int smCount()
    {
        static int cache[64] = {};
        int dev = 0;
        if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
            return 152;
        if(cache[dev] == 0)
        {
            int n = 0;
            if(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
                n = 152;
            cache[dev] = n;
        }
        return cache[dev];
    }

#ifndef PICGB_J_FIXED
    // 1: the shared-memory J tile holds 32-bit fixed-point high and low parts
    // added with native fire-and-forget integer atomics; 0: floats added with
    // atomicAdd, which for shared memory is a load/compare-and-swap loop on this
    // target that retries whenever another warp updated the node in between
    // (measured on the 256^3 two-stream workload: 30.9 vs 39.7 ms per launch)
#    define PICGB_J_FIXED 1
#endif

    // Fixed-point format of the shared-memory J tile (PICGB_J_FIXED): a value v
    // becomes v * 2^s units, split into a high part a = rint(v 2^s / 2^k) and the
    // low part v 2^s - a 2^k, each rounded to an integer.  The host picks s and k
    // so that both parts stay below 2^22 in magnitude and neither part's sum over
    // the values of one tile node can leave the int32 range.
    struct JFixed
    {
        float scale; // 2^s
        float invScale; // 2^-s
        float hiStep; // 2^-k
        float hiUnit; // 2^k
        int k;
    };


    // Status bits written by kernels into a device word (never a trap).
    enum StatusBits : unsigned
    {
        ST_OVERFLOW = 1u, // a supercell ran out of slots; particles were parked in the spill buffer
        ST_LOST = 2u, // the spill buffer was full as well: particles were dropped
        ST_BAD_CELL = 4u, // an input particle had an out-of-range supercell or cell index
        ST_TIMEOUT = 8u // a bounded wait gave up (persistent kernels)
    };

    // Particle storage of one species on the device: supercell-major SoA with
    // a fixed number of slots per supercell.  Slots [0, count[sc]) of supercell
    // sc are valid particles, stored at sc * cap + slot.
    struct SpeciesDev
    {
        float* px;
        float* py;
        float* pz;
        float* ux;
        float* uy;
        float* uz;
        float* w;
        uint16_t* lcell;
        uint32_t* id; // optional (nullptr)
        uint32_t* count; // [nsc] valid particles per supercell
        uint32_t* tail; // [nsc] append cursor during the push (starts at count)
        uint32_t* nhole; // [nsc] slots vacated by leaving particles
        uint16_t* holes; // [nsc * cap] vacated slot indices
        uint32_t cap; // slots per supercell (multiple of 32, <= 65535)
        // spill buffer for arrivals that found their supercell full
        float* sp_attr; // [7 * spill_cap]: px,py,pz,ux,uy,uz,w
        int32_t* sp_sc; // [spill_cap] destination supercell
        uint16_t* sp_lcell; // [spill_cap]
        uint32_t* sp_id; // [spill_cap]
        uint32_t* sp_count;
        uint32_t spill_cap;
    };

    // PushParams::pusher values (the C-ABI's enum picgb_pusher)
    constexpr int kPusherBoris = 0;
    constexpr int kPusherFree = 1;
    constexpr int kPusherHigueraCary = 3;
    constexpr int kPusherVay = 4;
    constexpr int kPusherPhoton = 5;
    // PushParams::current values (the C-ABI's enum picgb_current)
    constexpr int kCurrentNone = 0;
    constexpr int kCurrentEsirkepov = 1;
    constexpr int kCurrentEmZ = 2;

    struct PushParams
    {
        float charge; // per real particle
        float mass; // per real particle
        float dt;
        float c2; // c * c
        float rc2; // 1 / (c * c)
        float invVdt; // 1 / (dx * dy * dz * dt)
        float c; // speed of light (HigueraCary and Vay)
        int pusher; // 0 Boris, 1 Free, 3 HigueraCary, 4 Vay, 5 Photon (2 = not pushed, never launched)
        int current; // 1 Esirkepov, 2 EmZ (0: no current, the deposit is off)
        int deposit; // deposit the current inside the push kernel
        unsigned long long* kindCount; // profiling only: [0] deposits with the short footprint, [1] general; or nullptr
        JFixed jf; // fixed-point format of the J tile (used when built with PICGB_J_FIXED)
    };

    // One face of the total-field/scattered-field box and its pulse (fields/incidentField/
    // Solver.hpp:500-533, the profiles of fields/incidentField/profiles/), in the vector form of
    // fields/incidentField/Functors.hpp (BaseFunctorE): propagation direction d, polarisation
    // vectors, origin on the face's Huygens plane.
    struct IncidentParams
    {
        int enabled;
        int axis; // face normal
        int dir; // +1: the low face (the pulse enters towards +axis); -1: the high face
        int plane; // first (dir +1) or last (dir -1) E plane of the total-field region along axis
        int circular; // 0: E = pv1 value; 1: E = pv1 value(phase + pi/2) + pv2 value(phase)
        float E0, omega, w0, tc;
        float tau2; // twice the rms duration of the intensity (the envelope is exp(-(t / tau2)^2))
        float phase;
        float d[3]; // unit propagation direction
        float pv1[3]; // linear: the unit polarisation; circular: polarisation / sqrt(2)
        float pv2[3]; // circular: d x pv1 (zero for linear)
        float pol[3]; // the unit polarisation (internal coordinate axis 1)
        float pol2[3]; // d x pol (internal coordinate axis 2)
        float o[3]; // origin: the beam axis on the face's Huygens plane (length)
        float focusDist; // distance of the focus from the origin along d (length)
        float invVph; // 1 / the Yee grid's phase velocity at omega along d
        float zR; // Rayleigh length pi w0^2 / wavelength
        float k; // wave number omega / c
        float timeDelay; // TIME_DELAY
        int nmodes; // Laguerre-Gauss modes 0 .. nmodes-1 (1: the fundamental mode)
        float modes[8], modePhases[8];
        float modeNorm; // the sum of the mode amplitudes
        int profile; // 0: GaussianPulse, 1: PlaneWave, 2: Wavepacket, 3: Polynom
        float pwMu, pwTau, pwPlateau; // PlaneWave: end of the rising ramp, ramp width tau sqrt(2), plateau
        float pulseDuration; // PULSE_DURATION (Wavepacket, Polynom)
        float wpMu; // Wavepacket: centre of the plateau, INIT_TIME / 2
        float w01, w02; // W0_AXIS_1, W0_AXIS_2 of the transversal Gaussian
        int lo[2], hi[2]; // transverse extent of the face in cells, [lo, hi) on each transverse axis
    };
    constexpr int kIncidentFaces = 6; // face = 2 axis + (dir < 0)

    // ---- launchers (kernels_*.cu); all asynchronous on `stream`
    // shape: 1 CIC, 2 TSC, 3 PQS; scId: 0 -> 8x8x4, 1 -> 4x4x4, 2 -> 8x8x8
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
        cudaStream_t stream);
    cudaError_t launchDeposit(
        int shape,
        int scId,
        SpeciesDev const& sp,
        float* J,
        GridParams const& g,
        PushParams const& pp,
        unsigned* status,
        cudaStream_t stream);
    cudaError_t launchCompact(SpeciesDev const& sp, int nsc, cudaStream_t stream);
    // Interleaved cell order restored in every supercell (kReorder); vol = cells per supercell.
    cudaError_t launchReorder(SpeciesDev const& sp, int nsc, int vol, cudaStream_t stream);
    // Compaction of the push's vacated slots and the interleaved order in one pass per supercell
    // (in place of launchCompact); counters: [64][2] sums of vacated slots and of the particles
    // that remain, added to (or nullptr).
    cudaError_t launchCompactReorder(
        SpeciesDev const& sp,
        int nsc,
        int vol,
        unsigned long long* counters,
        cudaStream_t stream);
    // Shared memory kReorder needs for slots of `cap` particles per supercell.
    size_t reorderSmemBytes(int vol, uint32_t cap);
    cudaError_t launchMaxAbsBits(float const* w, uint64_t n, unsigned* bits, cudaStream_t stream);
    cudaError_t launchHistogram(
        int scId,
        uint64_t n,
        int32_t const* sc,
        uint16_t const* lcell,
        float const* const* pos, // 3 position arrays to validate, or nullptr
        uint32_t* count,
        int nsc,
        unsigned* status,
        cudaStream_t stream);
    cudaError_t launchScatter(
        uint64_t n,
        float const* const* attr, // 7 arrays: px py pz ux uy uz w
        int32_t const* sc,
        uint16_t const* lcell,
        uint32_t const* id,
        SpeciesDev const& sp,
        unsigned* status,
        cudaStream_t stream);
    // Copy of up to kCopySegs host-mapped (page-locked) arrays into device memory by a kernel:
    // the SMs read the host memory over the link, as the download's gather writes it.
    constexpr int kCopySegs = 10;
    struct CopySeg
    {
        void* dst;
        void const* src;
        size_t bytes;
    };
    struct CopyJobs
    {
        CopySeg s[kCopySegs];
        int n;
    };
    cudaError_t launchCopyIn(CopyJobs const& jobs, cudaStream_t stream);
    // offsets[sc]: first output of supercell sc (a prefix of its counts); total: the sum
    cudaError_t launchGatherOut(
        SpeciesDev const& sp,
        int nsc,
        uint64_t const* offsets,
        uint64_t total,
        float* const* attr,
        int32_t* sc,
        uint16_t* lcell,
        uint32_t* id,
        cudaStream_t stream);
    cudaError_t launchChargeDensity(
        int shape,
        int scId,
        SpeciesDev const& sp,
        float* rho,
        GridParams const& g,
        float charge,
        float cellVolume,
        cudaStream_t stream);
    cudaError_t launchKineticEnergy(
        SpeciesDev const& sp,
        int nsc,
        float mass,
        float c,
        double* out,
        cudaStream_t stream);

    // fields (kernels_fields.cu); fields are SoA [3][nz][ny][nx]
    cudaError_t launchYeeBHalf(float const* E, float* B, GridParams const& g, cudaStream_t stream);
    cudaError_t launchYeeE(float const* B, float* E, float const* J, float coeff, GridParams const& g, cudaStream_t stream);
    cudaError_t launchAddCurrent(float* E, float const* J, float coeff, size_t ncell, cudaStream_t stream);
    // TF/SF corrections after a B half step (incident E at time t, coefficient dt/2) and
    // after the E step (incident B at time t, coefficient c^2 dt)
    cudaError_t launchIncidentB(float* B, GridParams const& g, IncidentParams const& inc, float t, cudaStream_t stream);
    cudaError_t launchIncidentE(float* E, GridParams const& g, IncidentParams const& inc, float t, cudaStream_t stream);
    cudaError_t launchFieldEnergy(float const* F, size_t ncell, double* out3, cudaStream_t stream);
    cudaError_t launchChargeResidual(
        float const* E,
        float const* rho,
        GridParams const& g,
        float* out,
        unsigned* maxBits,
        unsigned* maxRhoBits,
        cudaStream_t stream);
} // namespace picgb
