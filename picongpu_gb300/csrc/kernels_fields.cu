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
    // Incident pulse value at (x, y, z) in cell units and time t: the focused Gaussian beam of
    // profiles/GaussianPulse.hpp:223-290 in its fundamental mode (waist w(z_f), wavefront
    // curvature, Gouy phase, amplitude w0/w, the envelope shifted by the curvature's delay).
    __device__ __forceinline__ float incidentValue(IncidentParams const& p, GridParams const& g, float x, float y, float z, float t)
    {
        float const rx = (x - p.cx) * g.dx, rz = (z - p.cz) * g.dz;
        float const r2 = rx * rx + rz * rz;
        float const tau = t - (y - float(p.j0)) * g.dy / g.c - p.tc;
        float const zf = (p.yf - y) * g.dy; // distance to the focus along the propagation
        float const q = zf / p.zR;
        float const w2 = p.w0 * p.w0 * (1.0f + q * q);
        float const rc = 0.5f * r2 * (-zf / (p.zR * p.zR + zf * zf)); // r^2/2 times the inverse curvature radius
        float const xi = atanf(-q); // Gouy phase
        float const ts = tau - rc / g.c;
        float const env = sqrtf(p.w0 * p.w0 / w2) * expf(-r2 / w2) * expf(-(ts * ts) / (2.0f * p.sigma * p.sigma));
        return p.E0 * env * sinf(p.omega * tau - p.k * rc + xi + p.phase);
    }

    // After B -= dt/2 curl E: the B plane j0 - 1 (scattered side) used the total E of plane j0;
    // removing the incident part gives B_x += dt/2 E_z,inc / dy and B_z -= dt/2 E_x,inc / dy.
    __global__ void kIncidentB(float* __restrict__ B, GridParams g, IncidentParams p, float t)
    {
        int const i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
        if(i >= g.nx)
            return;
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const idx = size_t(i) + size_t(g.nx) * (size_t(p.j0 - 1) + size_t(g.ny) * k);
        float const h = 0.5f * g.dt / g.dy;
        if(p.pol == 0) // E_x at (i + 1/2, j0, k)
            B[2 * nc + idx] -= h * incidentValue(p, g, i + 0.5f, float(p.j0), float(k), t);
        else // E_z at (i, j0, k + 1/2)
            B[idx] += h * incidentValue(p, g, float(i), float(p.j0), k + 0.5f, t);
    }

    // After E += c^2 dt curl B: the E plane j0 (total side) used the scattered B of plane j0 - 1;
    // adding the incident part gives E_x -= c^2 dt B_z,inc / dy and E_z += c^2 dt B_x,inc / dy,
    // with B_z,inc = -E_x,inc / c (pol 0) and B_x,inc = E_z,inc / c (pol 1) for a wave along +y.
    __global__ void kIncidentE(float* __restrict__ E, GridParams g, IncidentParams p, float t)
    {
        int const i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
        if(i >= g.nx)
            return;
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const idx = size_t(i) + size_t(g.nx) * (size_t(p.j0) + size_t(g.ny) * k);
        float const h = g.c * g.c * g.dt / g.dy;
        float const yb = float(p.j0) - 0.5f;
        if(p.pol == 0) // B_z at (i + 1/2, j0 - 1/2, k)
            E[idx] -= h * (-incidentValue(p, g, i + 0.5f, yb, float(k), t) / g.c);
        else // B_x at (i, j0 - 1/2, k + 1/2)
            E[2 * nc + idx] += h * (incidentValue(p, g, float(i), yb, k + 0.5f, t) / g.c);
    }

    cudaError_t launchIncidentB(float* B, GridParams const& g, IncidentParams const& inc, float t, cudaStream_t stream)
    {
        if(!inc.enabled)
            return cudaSuccess;
        kIncidentB<<<dim3((g.nx + 127) / 128, g.nz), 128, 0, stream>>>(B, g, inc, t);
        return cudaGetLastError();
    }

    cudaError_t launchIncidentE(float* E, GridParams const& g, IncidentParams const& inc, float t, cudaStream_t stream)
    {
        if(!inc.enabled)
            return cudaSuccess;
        kIncidentE<<<dim3((g.nx + 127) / 128, g.nz), 128, 0, stream>>>(E, g, inc, t);
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
        dim3 grid((g.nx + kFieldBX - 1) / kFieldBX, g.ny, g.nz);
        kYeeBHalf<<<grid, kFieldBX, 0, stream>>>(E, B, g);
        return cudaGetLastError();
    }

    cudaError_t launchYeeE(float const* B, float* E, float const* J, float coeff, GridParams const& g, cudaStream_t stream)
    {
        dim3 grid((g.nx + kFieldBX - 1) / kFieldBX, g.ny, g.nz);
        kYeeE<<<grid, kFieldBX, 0, stream>>>(B, E, J, coeff, g);
        return cudaGetLastError();
    }

    cudaError_t launchAddCurrent(float* E, float const* J, float coeff, size_t ncell, cudaStream_t stream)
    {
        size_t const n = 3 * ncell;
        int const blocks = int(std::min<size_t>((n + 255) / 256, 152 * 32));
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

    // sum over cells of F_c^2 (square in float, cast to FP64, summed in FP64:
    // plugins/EnergyFields.x.cpp:240-261 squareComponentWise + cast64Bit)
    __global__ void kFieldEnergy(float const* __restrict__ F, size_t nc, double* out3)
    {
        __shared__ double ws[3][32];
        double acc[3] = {0.0, 0.0, 0.0};
        for(size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < nc; i += size_t(gridDim.x) * blockDim.x)
        {
#pragma unroll
            for(int d = 0; d < 3; ++d)
            {
                float const v = F[d * nc + i];
                acc[d] += double(fm(v, v));
            }
        }
        int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for(int d = 0; d < 3; ++d)
        {
            double const s = warpSumD(acc[d]);
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
        int const blocks = int(std::min<size_t>((ncell + 255) / 256, 152 * 8));
        kFieldEnergy<<<blocks, 256, 0, stream>>>(F, ncell, out3);
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
