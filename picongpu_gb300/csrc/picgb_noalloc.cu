// Charge-conservation residual that allocates no device memory.
//
// Who needs it: code that runs inside a host application which has already
// reserved the GPU's memory for itself -- a plugin of a PIC code whose particle
// heap was sized to nearly all free device memory at start-up (the way the
// reference sizes its frame heap), or a caller in a memory-pool-restricted
// process -- cannot call cudaMalloc for a temporary charge-density grid.  This
// entry point therefore keeps its scratch (the charge density and two maxima)
// in file-scope static device arrays of a fixed maximum size.  CUDA loads a
// library's device code lazily by default: the arrays are reserved on a device
// when this file's device code is first used there, i.e. by the first call on
// that device, and held until the process exits.  A host that reserves device
// memory for itself should make that first call before it does so.
#include "picgb.h"
#include "picgb_device.cuh"
#include "picgb_internal.hpp"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

namespace
{
    // largest grid (cells) the scratch holds: 2^22 floats = 16 MiB
    constexpr size_t kMaxCells = size_t(1) << 22;

    __device__ __align__(256) float g_rho[kMaxCells];
    __device__ __align__(256) unsigned g_max[2];

    struct ScratchPtrs
    {
        float* rho = nullptr;
        unsigned* max = nullptr;
    };

    thread_local std::string g_err;

    // Makes `device` current for the lifetime of the guard and gives the calling
    // thread its previous current device back on every return path.
    struct DeviceGuard
    {
        int previous = -1;
        cudaError_t err = cudaSuccess;

        explicit DeviceGuard(int device)
        {
            err = cudaGetDevice(&previous);
            if(err == cudaSuccess && previous != device)
                err = cudaSetDevice(device);
        }

        ~DeviceGuard()
        {
            int now = -1;
            if(previous >= 0 && cudaGetDevice(&now) == cudaSuccess && now != previous)
                cudaSetDevice(previous);
        }
    };

    int failNa(int code, char const* fmt, ...)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        g_err = buf;
        return code;
    }

    // Charge density at the cell origins from a flat particle list in the host
    // exchange format (ComputeGridValuePerFrame.hpp:66-117 with ChargeDensity).
    template<int SHAPE>
    __global__ void kRhoFlat(
        uint64_t n,
        float const* __restrict__ px,
        float const* __restrict__ py,
        float const* __restrict__ pz,
        float const* __restrict__ w,
        int32_t const* __restrict__ sc,
        uint16_t const* __restrict__ lcell,
        float* __restrict__ rho,
        picgb::GridParams g,
        int SX,
        int SY,
        int SZ,
        float charge,
        float cellVolume,
        unsigned* status)
    {
        using SH = picgb::Shape<SHAPE>;
        constexpr int lo = SH::supp / 2, up = (SH::supp + 1) / 2, span = lo + up + 1;
        int const nsc = g.nscx * g.nscy * g.nscz;
        for(uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
        {
            int const s = sc[i];
            int const lc = lcell[i];
            if(s < 0 || s >= nsc || lc >= SX * SY * SZ)
            {
                atomicOr(status, picgb::ST_BAD_CELL);
                continue;
            }
            int const scx = s % g.nscx, scy = (s / g.nscx) % g.nscy, scz = s / (g.nscx * g.nscy);
            int const cx = scx * SX + lc % SX, cy = scy * SY + (lc / SX) % SY, cz = scz * SZ + lc / (SX * SY);
            float const pos[3] = {px[i], py[i], pz[i]};
            float const attr = picgb::fdv(picgb::fm(charge, w[i]), cellVolume);
            for(int k = 0; k < span * span * span; ++k)
            {
                int const o[3] = {k % span - lo, (k / span) % span - lo, k / (span * span) - lo};
                float a = 1.0f;
#pragma unroll
                for(int d = 0; d < 3; ++d)
                    a = picgb::fm(a, SH::ca(picgb::fs(float(o[d]), pos[d])));
                if(a != 0.0f)
                {
                    int const gx = picgb::wrapi(cx + o[0], g.nx), gy = picgb::wrapi(cy + o[1], g.ny),
                              gz = picgb::wrapi(cz + o[2], g.nz);
                    atomicAdd(rho + size_t(gx) + size_t(g.nx) * (size_t(gy) + size_t(g.ny) * gz), picgb::fm(a, attr));
                }
            }
        }
    }

    // |eps0 div E - rho| and max|rho|; the same arithmetic as the residual kernel
    // of the simulation handle (plugins/ChargeConservation.tpp:121-135, 211-240)
    __global__ void kResidualNa(float const* __restrict__ Ex, float const* __restrict__ Ey, float const* __restrict__ Ez,
                                float const* __restrict__ rho, picgb::GridParams g, unsigned* maxBits)
    {
        using picgb::fa;
        using picgb::fdv;
        using picgb::fm;
        using picgb::fs;
        int const x = blockIdx.x * blockDim.x + threadIdx.x;
        int const y = blockIdx.y, z = blockIdx.z;
        float r = 0.0f, ar = 0.0f;
        if(x < g.nx)
        {
            size_t const row = size_t(g.nx) * (size_t(y) + size_t(g.ny) * z);
            size_t const i = row + x;
            size_t const ix = row + (x == 0 ? g.nx - 1 : x - 1);
            size_t const iy = size_t(g.nx) * (size_t(y == 0 ? g.ny - 1 : y - 1) + size_t(g.ny) * z) + x;
            size_t const iz = size_t(g.nx) * (size_t(y) + size_t(g.ny) * (z == 0 ? g.nz - 1 : z - 1)) + x;
            float const rw = fdv(1.0f, g.dx), rh = fdv(1.0f, g.dy), rd = fdv(1.0f, g.dz);
            float const div = fa(fa(fm(fs(Ex[i], Ex[ix]), rw), fm(fs(Ey[i], Ey[iy]), rh)), fm(fs(Ez[i], Ez[iz]), rd));
            r = fabsf(fs(fm(div, g.eps0), rho[i]));
            ar = fabsf(rho[i]);
        }
#pragma unroll
        for(int o = 16; o > 0; o >>= 1)
        {
            r = fmaxf(r, __shfl_down_sync(0xffffffffu, r, o));
            ar = fmaxf(ar, __shfl_down_sync(0xffffffffu, ar, o));
        }
        if((threadIdx.x & 31) == 0)
        {
            atomicMax(maxBits, __float_as_uint(r));
            atomicMax(maxBits + 1, __float_as_uint(ar));
        }
    }

    // Device addresses of the scratch arrays on the current device.  Looked up on every
    // call (cheap once the device code is loaded), so a context that the host tore down
    // and created again never sees a stale address.  The first lookup on a device loads
    // this file's device code there, which reserves the arrays.
    int scratchOnCurrentDevice(ScratchPtrs* out)
    {
        ScratchPtrs p;
        cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p.rho), g_rho);
        if(e != cudaSuccess)
            return failNa(PICGB_ERR_CUDA, "cudaGetSymbolAddress(rho scratch) failed: %s", cudaGetErrorString(e));
        e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p.max), g_max);
        if(e != cudaSuccess)
            return failNa(PICGB_ERR_CUDA, "cudaGetSymbolAddress(max scratch) failed: %s", cudaGetErrorString(e));
        *out = p;
        return PICGB_OK;
    }
} // namespace

#define NA_TRY(expr)                                                                                                  \
    do                                                                                                                \
    {                                                                                                                 \
        cudaError_t e_ = (expr);                                                                                      \
        if(e_ != cudaSuccess)                                                                                         \
            return failNa(PICGB_ERR_CUDA, "%s failed: %s", #expr, cudaGetErrorString(e_));                           \
    } while(0)

extern "C"
{
    uint64_t picgb_noalloc_max_cells(void) { return kMaxCells; }

    const char* picgb_noalloc_last_error(void) { return g_err.c_str(); }

    int picgb_charge_residual_noalloc(
        const picgb_grid_config* cfg,
        const float* const* E,
        int32_t nspecies,
        const picgb_particles* species,
        const float* charge,
        const int32_t* shape,
        void* stream,
        double* max_residual,
        double* max_rho)
    {
        if(!cfg || !E || !E[0] || !E[1] || !E[2] || (nspecies > 0 && (!species || !charge || !shape)))
            return failNa(PICGB_ERR_INVALID, "null argument");
        static int const scTab[3][3] = {{8, 8, 4}, {4, 4, 4}, {8, 8, 8}};
        if(cfg->supercell < 0 || cfg->supercell > 2)
            return failNa(PICGB_ERR_INVALID, "unknown supercell id %d", int(cfg->supercell));
        int const* scs = scTab[cfg->supercell];
        if(cfg->nx <= 0 || cfg->ny <= 0 || cfg->nz <= 0 || cfg->nx % scs[0] || cfg->ny % scs[1] || cfg->nz % scs[2])
            return failNa(PICGB_ERR_INVALID, "grid %dx%dx%d is not a positive multiple of the supercell", int(cfg->nx),
                          int(cfg->ny), int(cfg->nz));
        size_t const ncell = size_t(cfg->nx) * cfg->ny * cfg->nz;
        if(ncell > kMaxCells)
            return failNa(PICGB_ERR_INVALID,
                          "grid of %zu cells exceeds the %zu cells of this entry point's static scratch; use "
                          "picgb_charge_residual on a simulation handle instead",
                          ncell, kMaxCells);
        for(int s = 0; s < nspecies; ++s)
            if(shape[s] < PICGB_SHAPE_CIC || shape[s] > PICGB_SHAPE_PQS)
                return failNa(PICGB_ERR_UNSUPPORTED, "species %d: shape %d has no kernel", s, int(shape[s]));
        if(cfg->device < 0)
            return failNa(PICGB_ERR_INVALID, "device %d is not a device index", int(cfg->device));
        DeviceGuard guard(cfg->device); // the caller's current device comes back on return
        NA_TRY(guard.err);
        ScratchPtrs p;
        if(int r = scratchOnCurrentDevice(&p))
            return r;
        int sms = 0;
        NA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg->device));
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        picgb::GridParams g{};
        g.nx = cfg->nx;
        g.ny = cfg->ny;
        g.nz = cfg->nz;
        g.nscx = cfg->nx / scs[0];
        g.nscy = cfg->ny / scs[1];
        g.nscz = cfg->nz / scs[2];
        g.dx = cfg->dx;
        g.dy = cfg->dy;
        g.dz = cfg->dz;
        g.dt = cfg->dt;
        g.c = cfg->c;
        g.eps0 = cfg->eps0;
        // the scratch keeps the previous call's contents: clear what accumulates
        NA_TRY(cudaMemsetAsync(p.rho, 0, sizeof(float) * ncell, st));
        NA_TRY(cudaMemsetAsync(p.max, 0, sizeof(unsigned) * 2, st));
        float V = cfg->dx * cfg->dy;
        V = V * cfg->dz;
        for(int s = 0; s < nspecies; ++s)
        {
            picgb_particles const& q = species[s];
            if(q.n == 0)
                continue;
            // grid-stride loop: 8 blocks of 256 threads per SM of this device at most
            int const blocks = int(std::min<uint64_t>((q.n + 255) / 256, uint64_t(sms) * 8));
            // the first maximum word doubles as the status word of the density pass;
            // it is read and cleared before the residual pass
            unsigned* status = p.max;
            switch(shape[s])
            {
            case PICGB_SHAPE_CIC:
                kRhoFlat<1><<<blocks, 256, 0, st>>>(q.n, q.pos[0], q.pos[1], q.pos[2], q.w, q.sc, q.lcell, p.rho, g,
                                                    scs[0], scs[1], scs[2], charge[s], V, status);
                break;
            case PICGB_SHAPE_TSC:
                kRhoFlat<2><<<blocks, 256, 0, st>>>(q.n, q.pos[0], q.pos[1], q.pos[2], q.w, q.sc, q.lcell, p.rho, g,
                                                    scs[0], scs[1], scs[2], charge[s], V, status);
                break;
            default:
                kRhoFlat<3><<<blocks, 256, 0, st>>>(q.n, q.pos[0], q.pos[1], q.pos[2], q.w, q.sc, q.lcell, p.rho, g,
                                                    scs[0], scs[1], scs[2], charge[s], V, status);
                break;
            }
            NA_TRY(cudaGetLastError());
        }
        unsigned bad = 0;
        NA_TRY(cudaMemcpyAsync(&bad, p.max, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        NA_TRY(cudaStreamSynchronize(st));
        if(bad & picgb::ST_BAD_CELL)
            return failNa(PICGB_ERR_INVALID, "a particle has an out-of-range supercell or cell index");
        NA_TRY(cudaMemsetAsync(p.max, 0, sizeof(unsigned) * 2, st));
        dim3 grid((cfg->nx + 127) / 128, cfg->ny, cfg->nz);
        kResidualNa<<<grid, 128, 0, st>>>(E[0], E[1], E[2], p.rho, g, p.max);
        NA_TRY(cudaGetLastError());
        unsigned bits[2];
        NA_TRY(cudaMemcpyAsync(bits, p.max, sizeof(bits), cudaMemcpyDeviceToHost, st));
        NA_TRY(cudaStreamSynchronize(st));
        float f0, f1;
        std::memcpy(&f0, &bits[0], 4);
        std::memcpy(&f1, &bits[1], 4);
        if(max_residual)
            *max_residual = f0;
        if(max_rho)
            *max_rho = f1;
        return PICGB_OK;
    }
}
