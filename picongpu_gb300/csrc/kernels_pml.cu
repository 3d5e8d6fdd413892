// Yee updates of a box with open axes: beyond an open face the fields are zero, and in the
// PML layers the convolutional PML of fields/absorber/pml/Pml.kernel:400-590 replaces the
// plain update (Taflove & Hagness eqs. 7.105-7.110 with B on the right-hand side).  Cells
// outside the layers take exactly the operations of kYeeBHalf / kYeeE, so a box whose open
// axes carry no PML evolves bit for bit as the plain solver would with zero exterior fields.
#include "picgb_device.cuh"
#include "picgb_pml.hpp"

namespace picgb
{
    namespace
    {
        constexpr int kPmlBX = 128;

        // b, c, kappa of field f (0: E at cell i, 1: B at cell i + 1/2) along axis a
        __device__ __forceinline__ void pmlCoef(PmlDev const& p, int f, int a, int i, float& b, float& c, float& k)
        {
            float const* t = p.tab + size_t((f * 3 + a) * 3) * p.nmax;
            b = __ldg(t + i);
            c = __ldg(t + p.nmax + i);
            k = __ldg(t + 2 * p.nmax + i);
        }

        __device__ __forceinline__ size_t cellIndex(GridParams const& g, int x, int y, int z)
        {
            return size_t(x) + size_t(g.nx) * (size_t(y) + size_t(g.ny) * size_t(z));
        }
    } // namespace

    // B -= dt/2 curl E with forward differences (FDTDBase.kernel UpdateBHalfFunctor); in the PML,
    // Pml.kernel:522-581, the convolution fields updated once per step (updatePsi).
    __global__ void __launch_bounds__(kPmlBX)
        kYeeBHalfOpen(float const* __restrict__ E, float* __restrict__ B, GridParams g, PmlDev p, int updatePsi)
    {
        int const x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
        if(x >= g.nx)
            return;
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const i = cellIndex(g, x, y, z);
        int const xn = wrapOrOutside(x + 1, g.nx, g.open & 1), yn = wrapOrOutside(y + 1, g.ny, g.open & 2),
                  zn = wrapOrOutside(z + 1, g.nz, g.open & 4);
        float const ex = __ldg(E + i), ey = __ldg(E + nc + i), ez = __ldg(E + 2 * nc + i);
        auto at = [&](int c, int xx, int yy, int zz)
        { return (xx | yy | zz) < 0 ? 0.0f : __ldg(E + c * nc + cellIndex(g, xx, yy, zz)); };
        float const dFdx_y = divCell(fs(at(1, xn, y, z), ey), 0, g);
        float const dFdx_z = divCell(fs(at(2, xn, y, z), ez), 0, g);
        float const dFdy_x = divCell(fs(at(0, x, yn, z), ex), 1, g);
        float const dFdy_z = divCell(fs(at(2, x, yn, z), ez), 1, g);
        float const dFdz_x = divCell(fs(at(0, x, y, zn), ex), 2, g);
        float const dFdz_y = divCell(fs(at(1, x, y, zn), ey), 2, g);
        float bx, cx, kx, by, cy, ky, bz, cz, kz;
        pmlCoef(p, 1, 0, x, bx, cx, kx);
        pmlCoef(p, 1, 1, y, by, cy, ky);
        pmlCoef(p, 1, 2, z, bz, cz, kz);
        if(fm(fm(bx, by), bz) == 1.0f) // outside the PML (Pml.kernel:269-275)
        {
            float const c0 = fs(dFdy_z, dFdz_y), c1 = fs(dFdz_x, dFdx_z), c2 = fs(dFdx_y, dFdy_x);
            B[i] = fs(B[i], fm(fm(c0, 0.5f), g.dt));
            B[nc + i] = fs(B[nc + i], fm(fm(c1, 0.5f), g.dt));
            B[2 * nc + i] = fs(B[2 * nc + i], fm(fm(c2, 0.5f), g.dt));
            return;
        }
        float* ps = p.psiB;
        float yx = ps[kPsiYX * nc + i], zx = ps[kPsiZX * nc + i], xy = ps[kPsiXY * nc + i];
        float zy = ps[kPsiZY * nc + i], xz = ps[kPsiXZ * nc + i], yz = ps[kPsiYZ * nc + i];
        if(updatePsi)
        {
            yx = fa(fm(bx, yx), fm(cx, dFdx_z));
            zx = fa(fm(bx, zx), fm(cx, dFdx_y));
            xy = fa(fm(by, xy), fm(cy, dFdy_z));
            zy = fa(fm(by, zy), fm(cy, dFdy_x));
            xz = fa(fm(bz, xz), fm(cz, dFdz_y));
            yz = fa(fm(bz, yz), fm(cz, dFdz_x));
            ps[kPsiYX * nc + i] = yx;
            ps[kPsiZX * nc + i] = zx;
            ps[kPsiXY * nc + i] = xy;
            ps[kPsiZY * nc + i] = zy;
            ps[kPsiXZ * nc + i] = xz;
            ps[kPsiYZ * nc + i] = yz;
        }
        float const h = fm(0.5f, g.dt);
        B[i] = fa(B[i], fm(h, fs(fa(fs(fdv(dFdz_y, kz), fdv(dFdy_z, ky)), xz), xy)));
        B[nc + i] = fa(B[nc + i], fm(h, fs(fa(fs(fdv(dFdx_z, kx), fdv(dFdz_x, kz)), yx), yz)));
        B[2 * nc + i] = fa(B[2 * nc + i], fm(h, fs(fa(fs(fdv(dFdy_x, ky), fdv(dFdx_y, kx)), zy), zx)));
    }

    // E += curl(B) c^2 dt with backward differences, then E += coeff J as its own rounding step;
    // in the PML, Pml.kernel:424-475 with the convolution fields updated every call.
    __global__ void __launch_bounds__(kPmlBX) kYeeEOpen(
        float const* __restrict__ B,
        float* __restrict__ E,
        float const* __restrict__ J,
        float coeff,
        GridParams g,
        PmlDev p)
    {
        int const x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
        if(x >= g.nx)
            return;
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const i = cellIndex(g, x, y, z);
        int const xp = wrapOrOutside(x - 1, g.nx, g.open & 1), yp = wrapOrOutside(y - 1, g.ny, g.open & 2),
                  zp = wrapOrOutside(z - 1, g.nz, g.open & 4);
        float const bx0 = __ldg(B + i), by0 = __ldg(B + nc + i), bz0 = __ldg(B + 2 * nc + i);
        auto at = [&](int c, int xx, int yy, int zz)
        { return (xx | yy | zz) < 0 ? 0.0f : __ldg(B + c * nc + cellIndex(g, xx, yy, zz)); };
        float const dFdx_y = divCell(fs(by0, at(1, xp, y, z)), 0, g);
        float const dFdx_z = divCell(fs(bz0, at(2, xp, y, z)), 0, g);
        float const dFdy_x = divCell(fs(bx0, at(0, x, yp, z)), 1, g);
        float const dFdy_z = divCell(fs(bz0, at(2, x, yp, z)), 1, g);
        float const dFdz_x = divCell(fs(bx0, at(0, x, y, zp)), 2, g);
        float const dFdz_y = divCell(fs(by0, at(1, x, y, zp)), 2, g);
        float const c2 = fm(g.c, g.c);
        float bx, cx, kx, by, cy, ky, bz, cz, kz;
        pmlCoef(p, 0, 0, x, bx, cx, kx);
        pmlCoef(p, 0, 1, y, by, cy, ky);
        pmlCoef(p, 0, 2, z, bz, cz, kz);
        float e[3] = {E[i], E[nc + i], E[2 * nc + i]};
        if(fm(fm(bx, by), bz) == 1.0f)
        {
            float const cu[3] = {fs(dFdy_z, dFdz_y), fs(dFdz_x, dFdx_z), fs(dFdx_y, dFdy_x)};
#pragma unroll
            for(int d = 0; d < 3; ++d)
                e[d] = fa(e[d], fm(fm(cu[d], c2), g.dt));
        }
        else
        {
            float* ps = p.psiE;
            float const yx = fa(fm(bx, ps[kPsiYX * nc + i]), fm(cx, dFdx_z));
            float const zx = fa(fm(bx, ps[kPsiZX * nc + i]), fm(cx, dFdx_y));
            float const xy = fa(fm(by, ps[kPsiXY * nc + i]), fm(cy, dFdy_z));
            float const zy = fa(fm(by, ps[kPsiZY * nc + i]), fm(cy, dFdy_x));
            float const xz = fa(fm(bz, ps[kPsiXZ * nc + i]), fm(cz, dFdz_y));
            float const yz = fa(fm(bz, ps[kPsiYZ * nc + i]), fm(cz, dFdz_x));
            ps[kPsiYX * nc + i] = yx;
            ps[kPsiZX * nc + i] = zx;
            ps[kPsiXY * nc + i] = xy;
            ps[kPsiZY * nc + i] = zy;
            ps[kPsiXZ * nc + i] = xz;
            ps[kPsiYZ * nc + i] = yz;
            float const c2dt = fm(c2, g.dt);
            e[0] = fa(e[0], fm(c2dt, fs(fa(fs(fdv(dFdy_z, ky), fdv(dFdz_y, kz)), xy), xz)));
            e[1] = fa(e[1], fm(c2dt, fs(fa(fs(fdv(dFdz_x, kz), fdv(dFdx_z, kx)), yz), yx)));
            e[2] = fa(e[2], fm(c2dt, fs(fa(fs(fdv(dFdx_y, kx), fdv(dFdy_x, ky)), zx), zy)));
        }
#pragma unroll
        for(int d = 0; d < 3; ++d)
        {
            if(J)
                e[d] = fa(e[d], fm(coeff, __ldg(J + d * nc + i)));
            E[d * nc + i] = e[d];
        }
    }

    // The exponential absorber (fields/absorber/exponential/Exponential.kernel:50-90) on one field.
    __global__ void __launch_bounds__(kPmlBX) kAbsorbExponential(float* __restrict__ F, GridParams g, float const* __restrict__ damp, int nmax)
    {
        int const x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
        if(x >= g.nx)
            return;
        float const f[3] = {__ldg(damp + x), __ldg(damp + nmax + y), __ldg(damp + 2 * nmax + z)};
        if(f[0] == 1.0f && f[1] == 1.0f && f[2] == 1.0f)
            return;
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const i = cellIndex(g, x, y, z);
#pragma unroll
        for(int c = 0; c < 3; ++c)
        {
            float v = F[c * nc + i];
#pragma unroll
            for(int a = 0; a < 3; ++a)
                if(f[a] != 1.0f)
                    v = fm(v, f[a]);
            F[c * nc + i] = v;
        }
    }

    cudaError_t launchAbsorbExponential(float* F, GridParams const& g, float const* damp, int nmax, cudaStream_t stream)
    {
        dim3 const grid((g.nx + kPmlBX - 1) / kPmlBX, g.ny, g.nz);
        kAbsorbExponential<<<grid, kPmlBX, 0, stream>>>(F, g, damp, nmax);
        return cudaGetLastError();
    }

    cudaError_t launchYeeBHalfOpen(float const* E, float* B, GridParams const& g, PmlDev const& p, bool updatePsi, cudaStream_t stream)
    {
        dim3 const grid((g.nx + kPmlBX - 1) / kPmlBX, g.ny, g.nz);
        kYeeBHalfOpen<<<grid, kPmlBX, 0, stream>>>(E, B, g, p, updatePsi ? 1 : 0);
        return cudaGetLastError();
    }

    cudaError_t launchYeeEOpen(
        float const* B,
        float* E,
        float const* J,
        float coeff,
        GridParams const& g,
        PmlDev const& p,
        cudaStream_t stream)
    {
        dim3 const grid((g.nx + kPmlBX - 1) / kPmlBX, g.ny, g.nz);
        kYeeEOpen<<<grid, kPmlBX, 0, stream>>>(B, E, J, coeff, g, p);
        return cudaGetLastError();
    }
} // namespace picgb
