// Yee FDTD field kernels and field diagnostics.
//
// Fields are SoA [component][z][y][x] without guard cells; the periodic
// neighbour is reached by index wrap, which replaces the reference's guard
// exchange of E and B (MaxwellSolver/FDTD/FDTDBase.hpp:111,168,181).
#include "picgb_batch.hpp"
#include "picgb_device.cuh"
#include "picgb_internal.hpp"

namespace picgb
{
    constexpr int kFieldBX = 128;

    // B -= curl(E) * 0.5 * dt with forward differences at cell (x, y, z)
    // (FDTDBase.kernel:92-121 UpdateBHalfFunctor, differentiation/ForwardDerivative.hpp:45-63, Curl.hpp:84-89).
    __device__ __forceinline__ void yeeBHalfAt(
        float const* __restrict__ E,
        float* __restrict__ B,
        GridParams const& g,
        int const x,
        int const y,
        int const z)
    {
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const row = size_t(g.nx) * (size_t(y) + size_t(g.ny) * z);
        size_t const i = row + x;
        size_t const ix = row + (x + 1 == g.nx ? 0 : x + 1);
        size_t const iy = size_t(g.nx) * (size_t(y + 1 == g.ny ? 0 : y + 1) + size_t(g.ny) * z) + x;
        size_t const iz = size_t(g.nx) * (size_t(y) + size_t(g.ny) * (z + 1 == g.nz ? 0 : z + 1)) + x;
        float const* Ex = E;
        float const* Ey = E + nc;
        float const* Ez = E + 2 * nc;
        float const ex = __ldg(Ex + i), ey = __ldg(Ey + i), ez = __ldg(Ez + i);
        float const dFdx_y = divCell(fs(__ldg(Ey + ix), ey), 0, g);
        float const dFdx_z = divCell(fs(__ldg(Ez + ix), ez), 0, g);
        float const dFdy_x = divCell(fs(__ldg(Ex + iy), ex), 1, g);
        float const dFdy_z = divCell(fs(__ldg(Ez + iy), ez), 1, g);
        float const dFdz_x = divCell(fs(__ldg(Ex + iz), ex), 2, g);
        float const dFdz_y = divCell(fs(__ldg(Ey + iz), ey), 2, g);
        float const c0 = fs(dFdy_z, dFdz_y), c1 = fs(dFdz_x, dFdx_z), c2 = fs(dFdx_y, dFdy_x);
        B[i] = fs(B[i], fm(fm(c0, 0.5f), g.dt));
        B[nc + i] = fs(B[nc + i], fm(fm(c1, 0.5f), g.dt));
        B[2 * nc + i] = fs(B[2 * nc + i], fm(fm(c2, 0.5f), g.dt));
    }

    __global__ void __launch_bounds__(kFieldBX) kYeeBHalf(float const* __restrict__ E, float* __restrict__ B, GridParams g)
    {
        int const x = blockIdx.x * blockDim.x + threadIdx.x;
        if(x < g.nx)
            yeeBHalfAt(E, B, g, x, blockIdx.y, blockIdx.z);
    }

    // ---- vectorised Yee updates: four cells along x per thread
    // With nx a multiple of 4 every row and every component plane starts on a 16-byte
    // boundary, so the four cells' values of a component are one 128-bit load or store; the
    // neighbour beyond the four cells along x is one scalar load.  The arithmetic per cell is
    // that of yeeBHalfAt / yeeEAt.  A grid-stride loop over the (nx/4) ny nz quads.
    constexpr int kYeeVecThreads = 256;

    __device__ __forceinline__ float4 ld4(float const* p) { return __ldg(reinterpret_cast<float4 const*>(p)); }
    __device__ __forceinline__ float at4(float4 const& v, int m) { return m == 0 ? v.x : (m == 1 ? v.y : (m == 2 ? v.z : v.w)); }
    __device__ __forceinline__ void set4(float4& v, int m, float a)
    {
        if(m == 0)
            v.x = a;
        else if(m == 1)
            v.y = a;
        else if(m == 2)
            v.z = a;
        else
            v.w = a;
    }

    __global__ void __launch_bounds__(kYeeVecThreads) kYeeBHalf4(float const* __restrict__ E, float* __restrict__ B, GridParams g)
    {
        int const nq = g.nx >> 2;
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const quads = size_t(nq) * g.ny * g.nz;
        float const* Ex = E;
        float const* Ey = E + nc;
        float const* Ez = E + 2 * nc;
        for(size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x; t < quads; t += size_t(gridDim.x) * blockDim.x)
        {
            size_t const r = t / nq; // row y + ny z
            int const x = int(t - r * nq) * 4;
            int const y = int(r % g.ny), z = int(r / g.ny);
            size_t const i = r * g.nx + x;
            size_t const iy = (size_t(y + 1 == g.ny ? 0 : y + 1) + size_t(g.ny) * z) * g.nx + x;
            size_t const iz = (size_t(y) + size_t(g.ny) * (z + 1 == g.nz ? 0 : z + 1)) * g.nx + x;
            size_t const ix4 = r * g.nx + (x + 4 == g.nx ? 0 : x + 4); // the cell after the four
            float4 const ex = ld4(Ex + i), ey = ld4(Ey + i), ez = ld4(Ez + i);
            float const eyN = __ldg(Ey + ix4), ezN = __ldg(Ez + ix4);
            float4 const exY = ld4(Ex + iy), ezY = ld4(Ez + iy), exZ = ld4(Ex + iz), eyZ = ld4(Ey + iz);
            float4 b0 = *reinterpret_cast<float4 const*>(B + i);
            float4 b1 = *reinterpret_cast<float4 const*>(B + nc + i);
            float4 b2 = *reinterpret_cast<float4 const*>(B + 2 * nc + i);
#pragma unroll
            for(int m = 0; m < 4; ++m)
            {
                float const cx = at4(ex, m), cy = at4(ey, m), cz = at4(ez, m);
                float const dFdx_y = divCell(fs(m < 3 ? at4(ey, m + 1) : eyN, cy), 0, g);
                float const dFdx_z = divCell(fs(m < 3 ? at4(ez, m + 1) : ezN, cz), 0, g);
                float const dFdy_x = divCell(fs(at4(exY, m), cx), 1, g);
                float const dFdy_z = divCell(fs(at4(ezY, m), cz), 1, g);
                float const dFdz_x = divCell(fs(at4(exZ, m), cx), 2, g);
                float const dFdz_y = divCell(fs(at4(eyZ, m), cy), 2, g);
                float const c0 = fs(dFdy_z, dFdz_y), c1 = fs(dFdz_x, dFdx_z), c2 = fs(dFdx_y, dFdy_x);
                set4(b0, m, fs(at4(b0, m), fm(fm(c0, 0.5f), g.dt)));
                set4(b1, m, fs(at4(b1, m), fm(fm(c1, 0.5f), g.dt)));
                set4(b2, m, fs(at4(b2, m), fm(fm(c2, 0.5f), g.dt)));
            }
            *reinterpret_cast<float4*>(B + i) = b0;
            *reinterpret_cast<float4*>(B + nc + i) = b1;
            *reinterpret_cast<float4*>(B + 2 * nc + i) = b2;
        }
    }

    __global__ void __launch_bounds__(kYeeVecThreads)
        kYeeE4(float const* __restrict__ B, float* __restrict__ E, float const* __restrict__ J, float coeff, GridParams g)
    {
        int const nq = g.nx >> 2;
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const quads = size_t(nq) * g.ny * g.nz;
        float const* Bx = B;
        float const* By = B + nc;
        float const* Bz = B + 2 * nc;
        float const c2 = fm(g.c, g.c);
        for(size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x; t < quads; t += size_t(gridDim.x) * blockDim.x)
        {
            size_t const r = t / nq;
            int const x = int(t - r * nq) * 4;
            int const y = int(r % g.ny), z = int(r / g.ny);
            size_t const i = r * g.nx + x;
            size_t const iy = (size_t(y == 0 ? g.ny - 1 : y - 1) + size_t(g.ny) * z) * g.nx + x;
            size_t const iz = (size_t(y) + size_t(g.ny) * (z == 0 ? g.nz - 1 : z - 1)) * g.nx + x;
            size_t const ixP = r * g.nx + (x == 0 ? g.nx - 1 : x - 1); // the cell before the four
            float4 const bx = ld4(Bx + i), by = ld4(By + i), bz = ld4(Bz + i);
            float const byP = __ldg(By + ixP), bzP = __ldg(Bz + ixP);
            float4 const bxY = ld4(Bx + iy), bzY = ld4(Bz + iy), bxZ = ld4(Bx + iz), byZ = ld4(By + iz);
            float4 e[3] = {*reinterpret_cast<float4 const*>(E + i), *reinterpret_cast<float4 const*>(E + nc + i),
                           *reinterpret_cast<float4 const*>(E + 2 * nc + i)};
            float4 j[3];
            if(J)
            {
                j[0] = ld4(J + i);
                j[1] = ld4(J + nc + i);
                j[2] = ld4(J + 2 * nc + i);
            }
#pragma unroll
            for(int m = 0; m < 4; ++m)
            {
                float const cx = at4(bx, m), cy = at4(by, m), cz = at4(bz, m);
                float const dFdx_y = divCell(fs(cy, m > 0 ? at4(by, m - 1) : byP), 0, g);
                float const dFdx_z = divCell(fs(cz, m > 0 ? at4(bz, m - 1) : bzP), 0, g);
                float const dFdy_x = divCell(fs(cx, at4(bxY, m)), 1, g);
                float const dFdy_z = divCell(fs(cz, at4(bzY, m)), 1, g);
                float const dFdz_x = divCell(fs(cx, at4(bxZ, m)), 2, g);
                float const dFdz_y = divCell(fs(cy, at4(byZ, m)), 2, g);
                float const cu[3] = {fs(dFdy_z, dFdz_y), fs(dFdz_x, dFdx_z), fs(dFdx_y, dFdy_x)};
#pragma unroll
                for(int d = 0; d < 3; ++d)
                {
                    float v = fa(at4(e[d], m), fm(fm(cu[d], c2), g.dt));
                    if(J)
                        v = fa(v, fm(coeff, at4(j[d], m)));
                    set4(e[d], m, v);
                }
            }
#pragma unroll
            for(int d = 0; d < 3; ++d)
                *reinterpret_cast<float4*>(E + d * nc + i) = e[d];
        }
    }

    int yeeVecBlocks(GridParams const& g)
    {
        size_t const quads = size_t(g.nx >> 2) * g.ny * g.nz;
        size_t const cap = size_t(smCount()) * 8; // 8 blocks of 256 threads per SM
        return int(std::min<size_t>((quads + kYeeVecThreads - 1) / kYeeVecThreads, cap));
    }

    // E += curl(B) * c^2 * dt with backward differences at cell (x, y, z) (FDTDBase.kernel:51-81
    // UpdateEFunctor, BackwardDerivative.hpp:45-63); optionally followed by E += coeff * J
    // (currentInterpolation/None.hpp:60-65) as a separate rounding step.
    __device__ __forceinline__ void yeeEAt(
        float const* __restrict__ B,
        float* __restrict__ E,
        float const* __restrict__ J,
        float const coeff,
        GridParams const& g,
        int const x,
        int const y,
        int const z)
    {
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const row = size_t(g.nx) * (size_t(y) + size_t(g.ny) * z);
        size_t const i = row + x;
        size_t const ix = row + (x == 0 ? g.nx - 1 : x - 1);
        size_t const iy = size_t(g.nx) * (size_t(y == 0 ? g.ny - 1 : y - 1) + size_t(g.ny) * z) + x;
        size_t const iz = size_t(g.nx) * (size_t(y) + size_t(g.ny) * (z == 0 ? g.nz - 1 : z - 1)) + x;
        float const* Bx = B;
        float const* By = B + nc;
        float const* Bz = B + 2 * nc;
        float const bx = __ldg(Bx + i), by = __ldg(By + i), bz = __ldg(Bz + i);
        float const dFdx_y = divCell(fs(by, __ldg(By + ix)), 0, g);
        float const dFdx_z = divCell(fs(bz, __ldg(Bz + ix)), 0, g);
        float const dFdy_x = divCell(fs(bx, __ldg(Bx + iy)), 1, g);
        float const dFdy_z = divCell(fs(bz, __ldg(Bz + iy)), 1, g);
        float const dFdz_x = divCell(fs(bx, __ldg(Bx + iz)), 2, g);
        float const dFdz_y = divCell(fs(by, __ldg(By + iz)), 2, g);
        float const c2 = fm(g.c, g.c);
        float const cu[3] = {fs(dFdy_z, dFdz_y), fs(dFdz_x, dFdx_z), fs(dFdx_y, dFdy_x)};
#pragma unroll
        for(int d = 0; d < 3; ++d)
        {
            size_t const k = d * nc + i;
            float e = fa(E[k], fm(fm(cu[d], c2), g.dt));
            if(J)
                e = fa(e, fm(coeff, __ldg(J + k)));
            E[k] = e;
        }
    }

    __global__ void __launch_bounds__(kFieldBX)
        kYeeE(float const* __restrict__ B, float* __restrict__ E, float const* __restrict__ J, float coeff, GridParams g)
    {
        int const x = blockIdx.x * blockDim.x + threadIdx.x;
        if(x < g.nx)
            yeeEAt(B, E, J, coeff, g, x, blockIdx.y, blockIdx.z);
    }

    // ------------------------------------------------------------ incident field (TF/SF)
    __device__ __forceinline__ float pick3(float v0, float v1, float v2, int i) { return i == 0 ? v0 : (i == 1 ? v1 : v2); }

    // Incident E at (x, y, z) in cell units and time t: the focused Gaussian beam of
    // profiles/GaussianPulse.hpp:206-290 in its fundamental mode, in the reference's order of
    // operations.  Internal coordinates are dot products of the offset from the origin with the
    // propagation direction and the two polarisation axes (Functors.hpp getInternalCoordinates);
    // the local time runs from the origin at the grid's phase velocity along the direction
    // (getCurrentTime) and the field is zero before it starts there; the waist w(z_f), the phase
    // omega (time - z_f / c) + phase, the wavefront curvature, the Gouy phase, the cosine carrier,
    // the envelope exp(-(t_s / 2 tau)^2) of the curvature-delayed time and the amplitude w0 / w
    // follow GaussianPulse.hpp:214-290; circular polarisation adds the carrier shifted by pi/2
    // along the first vector (GaussianPulseFunctorIncidentE::operator()).
    __device__ __forceinline__ void incidentE(IncidentParams const& p, GridParams const& g, float x, float y, float z, float t, float E[3])
    {
        E[0] = E[1] = E[2] = 0.0f;
        float const s0 = x * g.dx - p.o[0], s1 = y * g.dy - p.o[1], s2 = z * g.dz - p.o[2];
        float const pos0 = s0 * p.d[0] + s1 * p.d[1] + s2 * p.d[2];
        float const tcur = t - (pos0 * p.invVph + p.timeDelay);
        if(tcur < 0.0f)
            return;
        if(p.profile != 0)
        {
            // separable functors (BaseSeparableFunctorE): E = polarisation (longitudinal(t_loc) transversal)
            float transversal = 1.0f;
            if(p.profile >= 2)
            {
                // BaseSeparableTransversalGaussianFunctorE::getTransversal: exp(-|x / W0|^2) in the
                // internal coordinates, the propagation coordinate set to 0
                float const a1 = (s0 * p.pol[0] + s1 * p.pol[1] + s2 * p.pol[2]) / p.w01;
                float const a2 = (s0 * p.pol2[0] + s1 * p.pol2[1] + s2 * p.pol2[2]) / p.w02;
                transversal = expf(-(0.0f + a1 * a1 + a2 * a2));
            }
            auto longitudinal = [&](float ph)
            {
                if(p.profile == 2)
                {
                    // Wavepacket (profiles/Wavepacket.hpp getLongitudinal)
                    float const runTime = tcur - p.wpMu;
                    float const tau = p.pulseDuration * sqrtf(2.0f);
                    float envelope = p.E0, corr = 0.0f;
                    float const startDown = 0.5f * p.pwPlateau, endUp = -0.5f * p.pwPlateau;
                    if(runTime > startDown)
                    {
                        float const ex = (runTime - startDown) / p.pulseDuration / sqrtf(2.0f);
                        envelope *= expf(-0.5f * ex * ex);
                        corr = (runTime - startDown) / (tau * tau * p.omega);
                    }
                    else if(runTime < endUp)
                    {
                        float const ex = (runTime - endUp) / p.pulseDuration / sqrtf(2.0f);
                        envelope *= expf(-0.5f * ex * ex);
                        corr = (runTime - endUp) / (tau * tau * p.omega);
                    }
                    float const phase = p.omega * runTime + p.phase + ph;
                    return (sinf(phase) + corr * cosf(phase)) * envelope;
                }
                if(p.profile == 3)
                {
                    // Polynom (profiles/Polynom.hpp getLongitudinal, polynomial)
                    float const riseTime = 0.5f * p.pulseDuration;
                    float const u = tcur / riseTime;
                    float const phase = p.omega * (tcur - riseTime) + p.phase + ph;
                    float poly = 0.0f;
                    if(u >= 0.0f && u <= 1.0f)
                        poly = u * u * u * (10.0f - 15.0f * u + 6.0f * u * u);
                    else if(u > 1.0f && u <= 2.0f)
                        poly = (2.0f - u) * (2.0f - u) * (2.0f - u) * (4.0f - 9.0f * u + 6.0f * u * u);
                    return sinf(phase) * (p.E0 * poly);
                }
                // PlaneWave (profiles/PlaneWave.hpp getLongitudinal): Gaussian ramps of width
                // tau sqrt(2) around a plateau, and the integration correction of the sine carrier
                float envelope = p.E0, corr = 0.0f;
                float const startDown = p.pwMu + p.pwPlateau;
                if(tcur > startDown)
                {
                    float const ex = (tcur - startDown) / p.pwTau;
                    envelope *= expf(-0.5f * ex * ex);
                    corr = (tcur - startDown) / (p.omega * p.pwTau * p.pwTau);
                }
                else if(tcur < p.pwMu)
                {
                    float const ex = (tcur - p.pwMu) / p.pwTau;
                    envelope *= expf(-0.5f * ex * ex);
                    corr = (tcur - p.pwMu) / (p.omega * p.pwTau * p.pwTau);
                }
                float const phase = p.omega * (tcur - p.pwMu) + p.phase + ph;
                return (sinf(phase) + cosf(phase) * corr) * envelope;
            };
            if(!p.circular)
            {
                float const v = longitudinal(0.0f) * transversal;
#pragma unroll
                for(int c = 0; c < 3; ++c)
                    E[c] = p.pv1[c] * v;
                return;
            }
            float const v1 = longitudinal(1.57079633f) * transversal, v2 = longitudinal(0.0f) * transversal;
#pragma unroll
            for(int c = 0; c < 3; ++c)
                E[c] = p.pv1[c] * v1 + p.pv2[c] * v2;
            return;
        }
        float const time = tcur - p.tc;
        float const a1 = s0 * p.pol[0] + s1 * p.pol[1] + s2 * p.pol[2];
        float const a2 = s0 * p.pol2[0] + s1 * p.pol2[1] + s2 * p.pol2[2];
        float const r2 = a1 * a1 + a2 * a2;
        float const fp = p.focusDist - pos0; // distance to the focus along the propagation
        float const w = p.w0 * sqrtf(1.0f + (fp / p.zR) * (fp / p.zR));
        float const phase = p.omega * (time - fp / g.c) + p.phase;
        float const rInv = -fp / (p.zR * p.zR + fp * fp); // inverse radius of curvature
        float const xi = atanf(-fp / p.zR); // Gouy phase
        float const r2OverW2 = r2 / w / w;
        float const rc = 0.5f * r2 * rInv;
        float const e = (time - rc / g.c) / p.tau2;
        float const gt = expf(-r2OverW2), ge = expf(-e * e), amp = p.E0 * (p.w0 / w);
        // E0 (w0 / w) ((sum_m a_m L_m(2 r^2/w^2) exp(-r^2/w^2) cos(... + (2m+1) xi + phi_m)) exp(-e^2))
        // / sum_m a_m, the loop and association of the reference (GaussianPulse.hpp:260-289)
        auto value = [&](float ph)
        {
            float et = 0.0f;
            float const x = 2.0f * r2OverW2;
            float lm1 = 1.0f, lm = 1.0f; // L_{m-1}, L_m (simpleLaguerre's recursion)
            for(int m = 0; m < p.nmodes; ++m)
            {
                if(m == 1)
                    lm = 1.0f - x;
                else if(m > 1)
                {
                    float const next = ((2.0f * float(m - 1) + 1.0f - x) * lm - float(m - 1) * lm1) / float(m);
                    lm1 = lm;
                    lm = next;
                }
                et += p.modes[m] * lm * gt
                    * cosf(p.k * fp - p.k * rc + (2.0f * float(m) + 1.0f) * xi + ph + p.modePhases[m]);
            }
            et *= ge;
            return amp * et / p.modeNorm;
        };
        float const v2 = value(phase);
        if(!p.circular)
        {
#pragma unroll
            for(int c = 0; c < 3; ++c)
                E[c] = p.pv1[c] * v2;
            return;
        }
        float const v1 = value(p.omega * (time - fp / g.c) + p.phase + 1.57079633f); // + pi/2
#pragma unroll
        for(int c = 0; c < 3; ++c)
            E[c] = p.pv1[c] * v1 + p.pv2[c] * v2;
    }

    // Cell (i, j, k) of a face node: `planeIdx` along the axis, (u1, u2) on the transverse axes.
    __device__ __forceinline__ void faceCell(int a, int planeIdx, int u1, int u2, int& i, int& j, int& k)
    {
        i = a == 0 ? planeIdx : u1;
        j = a == 1 ? planeIdx : (a == 0 ? u1 : u2);
        k = a == 2 ? planeIdx : u2;
    }

    __constant__ float kYeePosE[3][3] = {{0.5f, 0.f, 0.f}, {0.f, 0.5f, 0.f}, {0.f, 0.f, 0.5f}};
    __constant__ float kYeePosB[3][3] = {{0.f, 0.5f, 0.5f}, {0.5f, 0.f, 0.5f}, {0.5f, 0.5f, 0.f}};

    // The incident field of component c at the Yee position of that component in cell (i, j, k)
    // shifted by `shift` cells along the face axis: E (wantB false) or B = d x E / c.
    __device__ __forceinline__ float incidentComponent(
        IncidentParams const& p, GridParams const& g, int c, bool wantB, int i, int j, int k, float shift, float t)
    {
        float const(*pos)[3] = wantB ? kYeePosB : kYeePosE;
        float x = float(i) + pos[c][0], y = float(j) + pos[c][1], z = float(k) + pos[c][2];
        if(p.axis == 0)
            x += shift;
        else if(p.axis == 1)
            y += shift;
        else
            z += shift;
        float E[3];
        incidentE(p, g, x, y, z, t, E);
        if(!wantB)
            return E[c];
        int const c1 = (c + 1) % 3, c2 = (c + 2) % 3;
        return (p.d[c1] * E[c2] - p.d[c2] * E[c1]) / g.c;
    }

    // TF/SF correction of a face after a field update (incidentField/Solver.kernel UpdateFunctor
    // with the Yee curl): updated[comp2] += base * incident[comp1], updated[comp1] -= base *
    // incident[comp2], comp1 = (axis + 2) % 3, comp2 = (axis + 1) % 3, base = curl coefficient /
    // d_axis * face direction.  After a B half step (curl coefficient -dt/2) the B plane on the
    // scattered side of the surface (plane - 1 for a low face, plane for a high face) takes the
    // incident E one plane further in on a low face (Solver.hpp:343-356); after the E step
    // (c^2 dt) the E plane `plane` takes the incident B half a plane out.  For a wave along +y
    // polarised along x: B_z -= dt/2 E_x,inc / dy and E_x += c^2 dt E_x,inc(at B_z) / (c dy).
    __global__ void kIncidentB(float* __restrict__ B, GridParams g, IncidentParams p, float t)
    {
        int const u1 = p.lo[0] + int(blockIdx.x * blockDim.x + threadIdx.x), u2 = p.lo[1] + int(blockIdx.y);
        if(u1 >= p.hi[0])
            return;
        int const a = p.axis, comp1 = (a + 2) % 3, comp2 = (a + 1) % 3;
        float const da = pick3(g.dx, g.dy, g.dz, a);
        float const base = -0.5f * g.dt / da * float(p.dir);
        float const shift = p.dir > 0 ? 1.0f : 0.0f;
        int i, j, k;
        faceCell(a, p.dir > 0 ? p.plane - 1 : p.plane, u1, u2, i, j, k);
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const idx = size_t(i) + size_t(g.nx) * (size_t(j) + size_t(g.ny) * size_t(k));
        if(p.pv1[comp1] != 0.0f || p.pv2[comp1] != 0.0f)
            B[size_t(comp2) * nc + idx] += base * incidentComponent(p, g, comp1, false, i, j, k, shift, t);
        if(p.pv1[comp2] != 0.0f || p.pv2[comp2] != 0.0f)
            B[size_t(comp1) * nc + idx] -= base * incidentComponent(p, g, comp2, false, i, j, k, shift, t);
    }

    __global__ void kIncidentE(float* __restrict__ E, GridParams g, IncidentParams p, float t)
    {
        int const u1 = p.lo[0] + int(blockIdx.x * blockDim.x + threadIdx.x), u2 = p.lo[1] + int(blockIdx.y);
        if(u1 >= p.hi[0])
            return;
        int const a = p.axis, comp1 = (a + 2) % 3, comp2 = (a + 1) % 3;
        float const da = pick3(g.dx, g.dy, g.dz, a);
        float const base = g.c * g.c * g.dt / da * float(p.dir);
        float const shift = p.dir > 0 ? -1.0f : 0.0f;
        int i, j, k;
        faceCell(a, p.plane, u1, u2, i, j, k);
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const idx = size_t(i) + size_t(g.nx) * (size_t(j) + size_t(g.ny) * size_t(k));
        E[size_t(comp2) * nc + idx] += base * incidentComponent(p, g, comp1, true, i, j, k, shift, t);
        E[size_t(comp1) * nc + idx] -= base * incidentComponent(p, g, comp2, true, i, j, k, shift, t);
    }

    cudaError_t launchIncidentB(float* B, GridParams const& g, IncidentParams const& inc, float t, cudaStream_t stream)
    {
        if(!inc.enabled || inc.hi[0] <= inc.lo[0] || inc.hi[1] <= inc.lo[1])
            return cudaSuccess;
        kIncidentB<<<dim3((inc.hi[0] - inc.lo[0] + 127) / 128, inc.hi[1] - inc.lo[1]), 128, 0, stream>>>(B, g, inc, t);
        return cudaGetLastError();
    }

    cudaError_t launchIncidentE(float* E, GridParams const& g, IncidentParams const& inc, float t, cudaStream_t stream)
    {
        if(!inc.enabled || inc.hi[0] <= inc.lo[0] || inc.hi[1] <= inc.lo[1])
            return cudaSuccess;
        kIncidentE<<<dim3((inc.hi[0] - inc.lo[0] + 127) / 128, inc.hi[1] - inc.lo[1]), 128, 0, stream>>>(E, g, inc, t);
        return cudaGetLastError();
    }

    // ------------------------------------------------------------ ensemble of boxes
    // Block b of a batched field launch covers kBatchFieldThreads consecutive
    // cells of box blockBox[b]; returns false for threads past the box's end.
    __device__ __forceinline__ bool batchCell(
        BatchBox const* __restrict__ boxes,
        uint32_t const* __restrict__ blockBox,
        BatchBox const*& box,
        int& x,
        int& y,
        int& z)
    {
        box = boxes + __ldg(blockBox + blockIdx.x);
        GridParams const& g = box->g;
        size_t const cell = size_t(blockIdx.x - box->block0) * kBatchFieldThreads + threadIdx.x;
        if(cell >= size_t(g.nx) * g.ny * g.nz)
            return false;
        x = int(cell % unsigned(g.nx));
        size_t const r = cell / unsigned(g.nx);
        y = int(r % unsigned(g.ny));
        z = int(r / unsigned(g.ny));
        return true;
    }

    __global__ void __launch_bounds__(kBatchFieldThreads)
        kYeeBHalfBatch(BatchBox const* __restrict__ boxes, uint32_t const* __restrict__ blockBox)
    {
        BatchBox const* b;
        int x, y, z;
        if(batchCell(boxes, blockBox, b, x, y, z))
            yeeBHalfAt(b->E, b->B, b->g, x, y, z);
    }

    // E update with the J add of the fused deposit (as kYeeE with J).
    __global__ void __launch_bounds__(kBatchFieldThreads)
        kYeeEBatch(BatchBox const* __restrict__ boxes, uint32_t const* __restrict__ blockBox)
    {
        BatchBox const* b;
        int x, y, z;
        if(batchCell(boxes, blockBox, b, x, y, z))
            yeeEAt(b->B, b->E, b->J, b->coeffJ, b->g, x, y, z);
    }

    __global__ void __launch_bounds__(kBatchFieldThreads)
        kZeroJBatch(BatchBox const* __restrict__ boxes, uint32_t const* __restrict__ blockBox)
    {
        BatchBox const* b;
        int x, y, z;
        if(batchCell(boxes, blockBox, b, x, y, z))
        {
            size_t const nc = size_t(b->g.nx) * b->g.ny * b->g.nz;
            size_t const i = size_t(x) + size_t(b->g.nx) * (size_t(y) + size_t(b->g.ny) * z);
            b->J[i] = 0.0f;
            b->J[nc + i] = 0.0f;
            b->J[2 * nc + i] = 0.0f;
        }
    }

    cudaError_t launchYeeBHalfBatch(BatchBox const* boxes, uint32_t const* blockBox, uint32_t nblocks, cudaStream_t stream)
    {
        if(nblocks)
            kYeeBHalfBatch<<<nblocks, kBatchFieldThreads, 0, stream>>>(boxes, blockBox);
        return cudaGetLastError();
    }

    cudaError_t launchYeeEBatch(BatchBox const* boxes, uint32_t const* blockBox, uint32_t nblocks, cudaStream_t stream)
    {
        if(nblocks)
            kYeeEBatch<<<nblocks, kBatchFieldThreads, 0, stream>>>(boxes, blockBox);
        return cudaGetLastError();
    }

    cudaError_t launchZeroJBatch(BatchBox const* boxes, uint32_t const* blockBox, uint32_t nblocks, cudaStream_t stream)
    {
        if(nblocks)
            kZeroJBatch<<<nblocks, kBatchFieldThreads, 0, stream>>>(boxes, blockBox);
        return cudaGetLastError();
    }

    __global__ void kAddCurrent(float* __restrict__ E, float const* __restrict__ J, float coeff, size_t n)
    {
        for(size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
            E[i] = fa(E[i], fm(coeff, J[i]));
    }

    cudaError_t launchYeeBHalf(float const* E, float* B, GridParams const& g, cudaStream_t stream)
    {
        if(g.nx % 4 == 0)
        {
            kYeeBHalf4<<<yeeVecBlocks(g), kYeeVecThreads, 0, stream>>>(E, B, g);
            return cudaGetLastError();
        }
        dim3 grid((g.nx + kFieldBX - 1) / kFieldBX, g.ny, g.nz);
        kYeeBHalf<<<grid, kFieldBX, 0, stream>>>(E, B, g);
        return cudaGetLastError();
    }

    cudaError_t launchYeeE(float const* B, float* E, float const* J, float coeff, GridParams const& g, cudaStream_t stream)
    {
        if(g.nx % 4 == 0)
        {
            kYeeE4<<<yeeVecBlocks(g), kYeeVecThreads, 0, stream>>>(B, E, J, coeff, g);
            return cudaGetLastError();
        }
        dim3 grid((g.nx + kFieldBX - 1) / kFieldBX, g.ny, g.nz);
        kYeeE<<<grid, kFieldBX, 0, stream>>>(B, E, J, coeff, g);
        return cudaGetLastError();
    }

    cudaError_t launchAddCurrent(float* E, float const* J, float coeff, size_t ncell, cudaStream_t stream)
    {
        size_t const n = 3 * ncell;
        int const blocks = int(std::min<size_t>((n + 255) / 256, size_t(smCount()) * 32));
        kAddCurrent<<<blocks, 256, 0, stream>>>(E, J, coeff, n);
        return cudaGetLastError();
    }

    // ------------------------------------------------------------ diagnostics
    __device__ __forceinline__ double warpSumD(double v)
    {
#pragma unroll
        for(int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        return v;
    }

    // Sum over cells of F_c^2 per component c (plugins/EnergyFields.x.cpp:240-261: the squares
    // in float, squareComponentWise, then cast64Bit and an FP64 reduction).  Each thread sums
    // its squares as a compensated float pair (compensatedAdd) carried into FP64, where the
    // block and grid sums go on; the result differs from a plain FP64 sum of the same float
    // squares by about 1e-13 of it.  One FP64 conversion and add per square, as in the
    // reference, ran on this GPU's narrow FP64 pipe: 204 us for the 201 MB of one 256^3
    // field, 1 TB/s.  VEC: four cells per load (the cell count a multiple of 4).
    template<bool VEC>
    __global__ void kFieldEnergy(float const* __restrict__ F, size_t nc, double* out3)
    {
        __shared__ double ws[3][32];
        float sum[3] = {0.0f, 0.0f, 0.0f}, comp[3] = {0.0f, 0.0f, 0.0f};
        size_t const stride = size_t(gridDim.x) * blockDim.x;
        if constexpr(VEC)
        {
            float4 const* F4 = reinterpret_cast<float4 const*>(F);
            size_t const nc4 = nc / 4;
            for(size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < nc4; i += stride)
            {
#pragma unroll
                for(int d = 0; d < 3; ++d)
                {
                    float4 const v = F4[d * nc4 + i];
                    compensatedAdd(sum[d], comp[d], fm(v.x, v.x));
                    compensatedAdd(sum[d], comp[d], fm(v.y, v.y));
                    compensatedAdd(sum[d], comp[d], fm(v.z, v.z));
                    compensatedAdd(sum[d], comp[d], fm(v.w, v.w));
                }
            }
        }
        else
        {
            for(size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < nc; i += stride)
            {
#pragma unroll
                for(int d = 0; d < 3; ++d)
                {
                    float const v = F[d * nc + i];
                    compensatedAdd(sum[d], comp[d], fm(v, v));
                }
            }
        }
        int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for(int d = 0; d < 3; ++d)
        {
            double const s = warpSumD(double(sum[d]) + double(comp[d]));
            if(lane == 0)
                ws[d][warp] = s;
        }
        __syncthreads();
        if(warp == 0)
        {
#pragma unroll
            for(int d = 0; d < 3; ++d)
            {
                double v = lane < int(blockDim.x >> 5) ? ws[d][lane] : 0.0;
                v = warpSumD(v);
                if(lane == 0 && v != 0.0)
                    atomicAdd(out3 + d, v);
            }
        }
    }

    cudaError_t launchFieldEnergy(float const* F, size_t ncell, double* out3, cudaStream_t stream)
    {
        bool const vec = ncell % 4 == 0 && reinterpret_cast<uintptr_t>(F) % 16 == 0;
        size_t const work = vec ? ncell / 4 : ncell;
        int const blocks = int(std::min<size_t>((work + 255) / 256, size_t(smCount()) * 8));
        if(vec)
            kFieldEnergy<true><<<blocks, 256, 0, stream>>>(F, ncell, out3);
        else
            kFieldEnergy<false><<<blocks, 256, 0, stream>>>(F, ncell, out3);
        return cudaGetLastError();
    }

    // |eps0 * div E - rho| (plugins/ChargeConservation.tpp:121-135, 211-240) and its max;
    // max|rho| alongside.  Non-negative floats order like their bit patterns.
    __global__ void kChargeResidual(
        float const* __restrict__ E,
        float const* __restrict__ rho,
        GridParams g,
        float* __restrict__ out,
        unsigned* maxBits,
        unsigned* maxRhoBits)
    {
        int const x = blockIdx.x * blockDim.x + threadIdx.x;
        int const y = blockIdx.y, z = blockIdx.z;
        float r = 0.0f, ar = 0.0f;
        if(x < g.nx)
        {
            size_t const nc = size_t(g.nx) * g.ny * g.nz;
            size_t const row = size_t(g.nx) * (size_t(y) + size_t(g.ny) * z);
            size_t const i = row + x;
            size_t const ix = row + (x == 0 ? g.nx - 1 : x - 1);
            size_t const iy = size_t(g.nx) * (size_t(y == 0 ? g.ny - 1 : y - 1) + size_t(g.ny) * z) + x;
            size_t const iz = size_t(g.nx) * (size_t(y) + size_t(g.ny) * (z == 0 ? g.nz - 1 : z - 1)) + x;
            float const rw = fdv(1.0f, g.dx), rh = fdv(1.0f, g.dy), rd = fdv(1.0f, g.dz);
            float const div = fa(fa(fm(fs(E[i], E[ix]), rw), fm(fs(E[nc + i], E[nc + iy]), rh)),
                                 fm(fs(E[2 * nc + i], E[2 * nc + iz]), rd));
            r = fabsf(fs(fm(div, g.eps0), rho[i]));
            ar = fabsf(rho[i]);
            if(out)
                out[i] = r;
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
            atomicMax(maxRhoBits, __float_as_uint(ar));
        }
    }

    cudaError_t launchChargeResidual(
        float const* E,
        float const* rho,
        GridParams const& g,
        float* out,
        unsigned* maxBits,
        unsigned* maxRhoBits,
        cudaStream_t stream)
    {
        dim3 grid((g.nx + kFieldBX - 1) / kFieldBX, g.ny, g.nz);
        kChargeResidual<<<grid, kFieldBX, 0, stream>>>(E, rho, g, out, maxBits, maxRhoBits);
        return cudaGetLastError();
    }
} // namespace picgb
