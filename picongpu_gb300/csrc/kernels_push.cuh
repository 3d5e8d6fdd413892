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
    constexpr int kPushThreads = 256;

    template<typename SH, typename SC>
    struct TileGeom
    {
        static constexpr int GX = SC::SX + SH::gLo + SH::gHi;
        static constexpr int GY = SC::SY + SH::gLo + SH::gHi;
        static constexpr int GZ = SC::SZ + SH::gLo + SH::gHi;
        static constexpr int GT = GX * GY * GZ;
        static constexpr int JX = SC::SX + SH::jLo + SH::jHi;
        static constexpr int JY = SC::SY + SH::jLo + SH::jHi;
        static constexpr int JZ = SC::SZ + SH::jLo + SH::jHi;
        static constexpr int JT = JX * JY * JZ;
        static constexpr size_t pushSmem = sizeof(float) * (6 * GT + 3 * JT);
        static constexpr size_t depositSmem = sizeof(float) * (3 * JT);
    };

    __device__ __forceinline__ void scCoords(int sc, GridParams const& g, int& x, int& y, int& z)
    {
        x = sc % g.nscx;
        y = (sc / g.nscx) % g.nscy;
        z = sc / (g.nscx * g.nscy);
    }

    // Stage a (S + lo + hi)^3 tile of a 3-component SoA field with periodic wrap.
    template<int TX, int TY, int TT>
    __device__ __forceinline__ void loadTile(
        float* __restrict__ dst,
        float const* __restrict__ src,
        int ox,
        int oy,
        int oz,
        GridParams const& g,
        size_t ncell)
    {
        for(int t = threadIdx.x; t < TT; t += blockDim.x)
        {
            int const tx = t % TX, ty = (t / TX) % TY, tz = t / (TX * TY);
            int const gx = wrapi(ox + tx, g.nx), gy = wrapi(oy + ty, g.ny), gz = wrapi(oz + tz, g.nz);
            size_t const gi = size_t(gx) + size_t(g.nx) * (size_t(gy) + size_t(g.ny) * size_t(gz));
            dst[t] = __ldg(src + gi);
            dst[TT + t] = __ldg(src + ncell + gi);
            dst[2 * TT + t] = __ldg(src + 2 * ncell + gi);
        }
    }

    // Add a shared-memory J tile into the global J with periodic wrap (the
    // reference's guard add of FieldJ, FieldJ.x.cpp:156-169, folded in).
    template<int TX, int TY, int TT>
    __device__ __forceinline__ void flushTile(
        float const* __restrict__ Js,
        float* __restrict__ J,
        int ox,
        int oy,
        int oz,
        GridParams const& g,
        size_t ncell)
    {
        for(int t = threadIdx.x; t < TT; t += blockDim.x)
        {
            float const vx = Js[t], vy = Js[TT + t], vz = Js[2 * TT + t];
            if(vx == 0.0f && vy == 0.0f && vz == 0.0f)
                continue;
            int const tx = t % TX, ty = (t / TX) % TY, tz = t / (TX * TY);
            int const gx = wrapi(ox + tx, g.nx), gy = wrapi(oy + ty, g.ny), gz = wrapi(oz + tz, g.nz);
            size_t const gi = size_t(gx) + size_t(g.nx) * (size_t(gy) + size_t(g.ny) * size_t(gz));
            if(vx != 0.0f)
                atomicAdd(J + gi, vx);
            if(vy != 0.0f)
                atomicAdd(J + ncell + gi, vy);
            if(vz != 0.0f)
                atomicAdd(J + 2 * ncell + gi, vz);
        }
    }

    template<int SHAPE, int SX, int SY, int SZ>
    __global__ void __launch_bounds__(kPushThreads) kPush(
        SpeciesDev sp,
        float const* __restrict__ E,
        float const* __restrict__ B,
        float* __restrict__ J,
        GridParams g,
        PushParams pp,
        unsigned* __restrict__ status)
    {
        using SH = Shape<SHAPE>;
        using SC = SuperCell<SX, SY, SZ>;
        using TG = TileGeom<SH, SC>;
        extern __shared__ float smem[];
        float* const Es = smem;
        float* const Bs = smem + 3 * TG::GT;
        float* const Js = smem + 6 * TG::GT;
        __shared__ unsigned s_nhole;

        int const sc = blockIdx.x;
        uint32_t const n = sp.count[sc];
        if(threadIdx.x == 0)
            s_nhole = 0u;
        if(n == 0)
        {
            if(threadIdx.x == 0)
                sp.nhole[sc] = 0u;
            return;
        }
        int scx, scy, scz;
        scCoords(sc, g, scx, scy, scz);
        int const ox = scx * SX, oy = scy * SY, oz = scz * SZ;
        size_t const ncell = size_t(g.nx) * g.ny * g.nz;
        bool const useBoris = (pp.pusher == 0);
        if(useBoris)
        {
            loadTile<TG::GX, TG::GY, TG::GT>(Es, E, ox - SH::gLo, oy - SH::gLo, oz - SH::gLo, g, ncell);
            loadTile<TG::GX, TG::GY, TG::GT>(Bs, B, ox - SH::gLo, oy - SH::gLo, oz - SH::gLo, g, ncell);
        }
        if(pp.deposit)
            for(int t = threadIdx.x; t < 3 * TG::JT; t += blockDim.x)
                Js[t] = 0.0f;
        __syncthreads();

        float const cs[3] = {g.dx, g.dy, g.dz};
        size_t const base = size_t(sc) * sp.cap;
        for(uint32_t k = threadIdx.x; k < n; k += blockDim.x)
        {
            size_t const slot = base + k;
            float pos[3] = {sp.px[slot], sp.py[slot], sp.pz[slot]};
            float mom[3] = {sp.ux[slot], sp.uy[slot], sp.uz[slot]};
            float const w = sp.w[slot];
            int const lc = sp.lcell[slot];
            int const lx = lc % SX, ly = (lc / SX) % SY, lz = lc / (SX * SY);
            float const mass = fm(pp.mass, w);
            float const charge = fm(pp.charge, w);
            float vel[3];
            if(useBoris)
            {
                float Ev[3], Bv[3];
                // Yee positions (fields/YeeCell.hpp:70-131)
                Bv[0] = gatherComponent<SH, TG::GX, TG::GY>(Bs, lx, ly, lz, pos[0], pos[1], pos[2], 0.f, .5f, .5f);
                Bv[1] = gatherComponent<SH, TG::GX, TG::GY>(
                    Bs + TG::GT, lx, ly, lz, pos[0], pos[1], pos[2], .5f, 0.f, .5f);
                Bv[2] = gatherComponent<SH, TG::GX, TG::GY>(
                    Bs + 2 * TG::GT, lx, ly, lz, pos[0], pos[1], pos[2], .5f, .5f, 0.f);
                Ev[0] = gatherComponent<SH, TG::GX, TG::GY>(Es, lx, ly, lz, pos[0], pos[1], pos[2], .5f, 0.f, 0.f);
                Ev[1] = gatherComponent<SH, TG::GX, TG::GY>(
                    Es + TG::GT, lx, ly, lz, pos[0], pos[1], pos[2], 0.f, .5f, 0.f);
                Ev[2] = gatherComponent<SH, TG::GX, TG::GY>(
                    Es + 2 * TG::GT, lx, ly, lz, pos[0], pos[1], pos[2], 0.f, 0.f, .5f);
                boris(charge, mass, Ev, Bv, pp.dt, pp.c2, pp.rc2, mom, vel);
            }
            else
                velocity(mom, mass, pp.rc2, vel);
#pragma unroll
            for(int d = 0; d < 3; ++d)
                pos[d] = fa(pos[d], fdv(fm(vel[d], pp.dt), cs[d]));
            int nlc = lc;
            int mv[3], dir[3];
            bool const leave = moveParticle<SC>(pos, nlc, mv, dir);
            if(pp.deposit)
            {
                int const cellRel[3] = {lx + mv[0], ly + mv[1], lz + mv[2]};
                if(!Esirkepov<SH, TG::JX, TG::JY>::deposit(
                       Js,
                       Js + TG::JT,
                       Js + 2 * TG::JT,
                       cellRel,
                       pos,
                       vel,
                       charge,
                       g,
                       pp.invVdt))
                    atomicOr(status, ST_BAD_CELL);
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
                int const dx = wrapi(scx + dir[0], g.nscx), dy = wrapi(scy + dir[1], g.nscy),
                          dz = wrapi(scz + dir[2], g.nscz);
                int const dsc = dx + g.nscx * (dy + g.nscy * dz);
                uint32_t const id = sp.id ? sp.id[slot] : 0u;
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
                uint32_t const h = atomicAdd(&s_nhole, 1u);
                sp.holes[base + h] = uint16_t(k);
            }
        }
        __syncthreads();
        if(threadIdx.x == 0)
            sp.nhole[sc] = s_nhole;
        if(pp.deposit)
            flushTile<TG::JX, TG::JY, TG::JT>(
                Js,
                J,
                ox - SH::jLo,
                oy - SH::jLo,
                oz - SH::jLo,
                g,
                ncell);
    }

    // Deposit-only kernel over the sorted particles (the reference's separate
    // CurrentDeposition stage, simulation/stage/CurrentDeposition.x.cpp:105).
    template<int SHAPE, int SX, int SY, int SZ>
    __global__ void __launch_bounds__(kPushThreads)
        kDeposit(SpeciesDev sp, float* __restrict__ J, GridParams g, PushParams pp, unsigned* __restrict__ status)
    {
        using SH = Shape<SHAPE>;
        using SC = SuperCell<SX, SY, SZ>;
        using TG = TileGeom<SH, SC>;
        extern __shared__ float smem[];
        float* const Js = smem;
        int const sc = blockIdx.x;
        uint32_t const n = sp.count[sc];
        if(n == 0)
            return;
        int scx, scy, scz;
        scCoords(sc, g, scx, scy, scz);
        size_t const ncell = size_t(g.nx) * g.ny * g.nz;
        for(int t = threadIdx.x; t < 3 * TG::JT; t += blockDim.x)
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
            if(!Esirkepov<SH, TG::JX, TG::JY>::deposit(
                   Js,
                   Js + TG::JT,
                   Js + 2 * TG::JT,
                   cellRel,
                   pos,
                   vel,
                   fm(pp.charge, w),
                   g,
                   pp.invVdt))
                atomicOr(status, ST_BAD_CELL);
        }
        __syncthreads();
        flushTile<TG::JX, TG::JY, TG::JT>(
            Js,
            J,
            scx * SX - SH::jLo,
            scy * SY - SH::jLo,
            scz * SZ - SH::jLo,
            g,
            ncell);
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

    template<int SHAPE, int SX, int SY, int SZ>
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
        auto k = kPush<SHAPE, SX, SY, SZ>;
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
        auto k = kDeposit<SHAPE, SX, SY, SZ>;
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

// Instantiates the three launchers of one shape for the supported supercell sizes.
#define PICGB_SHAPE_LAUNCHERS(SHAPE, NAME)                                                                            \
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
            return launchPushT<SHAPE, 8, 8, 4>(sp, E, B, J, g, pp, status, stream);                                   \
        case 1:                                                                                                       \
            return launchPushT<SHAPE, 4, 4, 4>(sp, E, B, J, g, pp, status, stream);                                   \
        case 2:                                                                                                       \
            return launchPushT<SHAPE, 8, 8, 8>(sp, E, B, J, g, pp, status, stream);                                   \
        }                                                                                                             \
        return cudaErrorInvalidValue;                                                                                 \
    }                                                                                                                 \
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
