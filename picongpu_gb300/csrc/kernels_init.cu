// Seeded plasma initialisation directly into the supercell layout: uniform
// random in-cell positions (startPosition::Random,
// particles/startPosition/RandomImpl.hpp) or the in-cell lattice of
// startPosition::Quiet (particles/startPosition/QuietImpl.hpp:40-110), Maxwellian momenta plus a drift
// (manipulators Temperature/Drift, particles/manipulators/unary/Temperature.hpp:61-108).
// Counter-based random numbers: the value of every attribute depends only on
// (seed, global cell, particle-in-cell, attribute), not on the launch shape.
#include "picgb_device.cuh"
#include "picgb_init.hpp"
#include "picgb_internal.hpp"

namespace picgb
{
    __device__ __forceinline__ uint64_t splitmix64(uint64_t x)
    {
        x += 0x9e3779b97f4a7c15ull;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
        return x ^ (x >> 31);
    }

    // uniform in [0, 1) with 24 random bits
    __device__ __forceinline__ float uniform01(uint64_t seed, uint64_t counter)
    {
        uint64_t const h = splitmix64(seed ^ splitmix64(counter));
        return float(h >> 40) * (1.0f / 16777216.0f);
    }

    // standard normal by the Box-Muller transform
    __device__ __forceinline__ float normal01(uint64_t seed, uint64_t counter)
    {
        float const u1 = 1.0f - uniform01(seed, 2 * counter); // (0, 1]
        float const u2 = uniform01(seed, 2 * counter + 1);
        return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    }

    __global__ void kInitPlasma(SpeciesDev sp, GridParams g, InitParams ip, int SX, int SY, int SZ)
    {
        int const sc = blockIdx.x;
        int const vol = SX * SY * SZ;
        int scx = sc % g.nscx, scy = (sc / g.nscx) % g.nscy, scz = sc / (g.nscx * g.nscy);
        uint32_t const n = uint32_t(vol) * ip.ppc;
        size_t const base = size_t(sc) * sp.cap;
        for(uint32_t k = threadIdx.x; k < n; k += blockDim.x)
        {
            // slot k holds particle p of cell lc with consecutive slots in consecutive
            // cells, so the lanes of a warp deposit into different cells
            uint32_t const lc = k % uint32_t(vol), p = k / uint32_t(vol);
            int const lx = lc % SX, ly = (lc / SX) % SY, lz = lc / (SX * SY);
            int const c[3] = {scx * SX + lx, scy * SY + ly, scz * SZ + lz};
            uint64_t const gc = uint64_t(c[0]) + uint64_t(g.nx) * (uint64_t(c[1]) + uint64_t(g.ny) * c[2]);
            uint64_t const pid = gc * ip.ppc + p;
            size_t const s = base + k;
            if(ip.quiet[0] == 0u)
            {
                sp.px[s] = uniform01(ip.position_seed, 3 * pid);
                sp.py[s] = uniform01(ip.position_seed, 3 * pid + 1);
                sp.pz[s] = uniform01(ip.position_seed, 3 * pid + 2);
            }
            else
            {
                // lattice coordinate of particle p (x fastest, pmacc::math::mapToND) and
                // position coordinate * spacing + spacing * 0.5 in float_X
                uint32_t const q[3] = {p % ip.quiet[0], (p / ip.quiet[0]) % ip.quiet[1], p / (ip.quiet[0] * ip.quiet[1])};
                float pos[3];
#pragma unroll
                for(int d = 0; d < 3; ++d)
                {
                    float const spacing = fdv(1.0f, float(ip.quiet[d]));
                    pos[d] = fa(fm(float(q[d]), spacing), fm(spacing, 0.5f));
                }
                sp.px[s] = pos[0];
                sp.py[s] = pos[1];
                sp.pz[s] = pos[2];
            }
            bool const hi = ip.split_axis >= 0 && c[ip.split_axis] >= ip.split_cell;
            float const* drift = hi ? ip.drift_hi : ip.drift_lo;
            float const mw = ip.mass * ip.weight * ip.c; // u (units of c) -> macro momentum
            sp.ux[s] = (drift[0] + ip.u_th * normal01(ip.seed, 3 * pid)) * mw;
            sp.uy[s] = (drift[1] + ip.u_th * normal01(ip.seed, 3 * pid + 1)) * mw;
            sp.uz[s] = (drift[2] + ip.u_th * normal01(ip.seed, 3 * pid + 2)) * mw;
            sp.w[s] = ip.weight;
            sp.lcell[s] = uint16_t(lc);
            if(sp.id)
                sp.id[s] = uint32_t(pid);
        }
        if(threadIdx.x == 0)
        {
            sp.count[sc] = n;
            sp.tail[sc] = n;
            sp.nhole[sc] = 0u;
        }
    }

    cudaError_t launchInitPlasma(SpeciesDev const& sp, GridParams const& g, InitParams const& ip, int const* scs, cudaStream_t stream)
    {
        int const nsc = g.nscx * g.nscy * g.nscz;
        kInitPlasma<<<nsc, 256, 0, stream>>>(sp, g, ip, scs[0], scs[1], scs[2]);
        return cudaGetLastError();
    }
} // namespace picgb
