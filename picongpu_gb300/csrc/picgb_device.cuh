// Device-side math of the PIC hot path: assignment shapes, form-factor gather,
// Boris, HigueraCary and Vay pushes, moveParticle and the Esirkepov deposit.
//
// Operations that decide particle positions (shapes, gather, push, move) use
// the explicit round-to-nearest intrinsics (__fmul_rn, __fadd_rn, __fmaf_rn,
// ...) so the compiler can neither contract nor reorder them: the result is
// bit-identical to the CPU oracle, which evaluates the same operations in the
// reference's association order (fused multiply-adds exactly where the gather
// accumulates `result += value * weight`).  That is what makes positions,
// momenta and the per-cell particle counts after a step bit-exact.
#pragma once

#include "picgb_internal.hpp"

#include <cstdint>
#include <cuda_runtime.h>

namespace picgb
{
    // ------------------------------------------------------------ exact ops
    __device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
    __device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
    __device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
    __device__ __forceinline__ float fdv(float a, float b) { return __fdiv_rn(a, b); }
    __device__ __forceinline__ float fsq(float a) { return __fsqrt_rn(a); }

    // One step of Neumaier's compensated summation (the improved Kahan-Babuska sum): e is
    // added to sum, and the rounding error of that addition is collected in comp.  The pair
    // (sum, comp), carried into FP64 as double(sum) + double(comp), holds the float sum with
    // an error of order n 2^-48 of the sum of |e|.
    __device__ __forceinline__ void compensatedAdd(float& sum, float& comp, float e)
    {
        float const t = fa(sum, e);
        comp = fa(comp, fabsf(sum) >= fabsf(e) ? fa(fs(sum, t), e) : fa(fs(e, t), sum));
        sum = t;
    }

    // ------------------------------------------------------------ shapes
    // particles/shapes/{NGP,CIC,TSC,PQS,PCS}.hpp; SHAPE = assignment order, support = SHAPE + 1.
    template<int SHAPE>
    struct Shape
    {
        static constexpr int supp = SHAPE + 1;
        static constexpr bool even = (supp % 2) == 0;
        // ChargeAssignment::begin / end
        static constexpr int caBegin = (SHAPE == 0 || SHAPE == 1) ? 0 : (SHAPE == 4 ? -2 : -1);
        static constexpr int caEnd = caBegin + supp;
        // ChargeAssignmentOnSupport begin (FieldToParticleInterpolation.hpp:65)
        static constexpr int osBegin = -supp / 2 + (supp + 1) % 2;
        // gather margins (FieldToParticleInterpolation.hpp:43-44)
        static constexpr int gLo = supp / 2;
        static constexpr int gHi = (supp + 1) / 2;
        // deposit node range relative to a cell in [-1, S] (a particle may have
        // left the supercell by one cell): gridShift in [-1, even ? 0 : 1],
        // node offset in [caBegin, caEnd]
        static constexpr int jLo = 2 - caBegin;
        static constexpr int jHi = (even ? 0 : 1) + caEnd + 1;

        // ---- radius helpers, exact arithmetic
        __device__ static float tsc1(float x) { return fs(0.75f, fm(x, x)); }
        __device__ static float tsc2(float x)
        {
            float t = fs(1.5f, x);
            return fm(0.5f, fm(t, t));
        }
        __device__ static float pqs1(float x)
        {
            float sq = fm(x, x);
            float tr = fm(sq, x);
            return fm(1.0f / 6.0f, fa(fs(4.0f, fm(6.0f, sq)), fm(3.0f, tr)));
        }
        __device__ static float pqs2(float x)
        {
            float t = fs(2.0f, x);
            return fm(1.0f / 6.0f, fm(fm(t, t), t));
        }
        __device__ static float pcs1(float x)
        {
            float sq = fm(x, x);
            return fa(115.f / 192.f, fm(sq, fa(-5.f / 8.f, fm(1.0f / 4.0f, sq))));
        }
        __device__ static float pcs2(float x)
        {
            // 1/96 * (55 + 4x(5 - 2x(15 + 2x(-5 + x))))
            float a = fa(-5.f, x);
            float b = fa(15.f, fm(fm(2.f, x), a));
            float c = fs(5.f, fm(fm(2.f, x), b));
            return fm(1.f / 96.f, fa(55.f, fm(fm(4.f, x), c)));
        }
        __device__ static float pcs3(float x)
        {
            float t = fs(5.f, fm(2.f, x));
            float sq = fm(t, t);
            return fm(1.f / 384.f, fm(sq, sq));
        }

        // detail::<Shape>::shapeArray(x): support values on the support grid points
        __device__ static void base(float x, float* s)
        {
            if constexpr(SHAPE == 0)
                s[0] = 1.0f;
            else if constexpr(SHAPE == 1)
            {
                s[0] = fs(1.0f, x);
                s[1] = x;
            }
            else if constexpr(SHAPE == 2)
            {
                s[0] = tsc2(fabsf(fs(-1.f, x)));
                s[1] = tsc1(fabsf(x));
                s[2] = fs(1.0f, fa(s[0], s[1]));
            }
            else if constexpr(SHAPE == 3)
            {
                s[0] = pqs2(fabsf(fs(-1.f, x)));
                s[1] = pqs1(x);
                s[3] = pqs2(fs(2.f, x));
                s[2] = fs(1.0f, fa(fa(s[0], s[1]), s[3]));
            }
            else
            {
                s[0] = pcs3(fabsf(fs(-2.f, x)));
                s[1] = pcs2(fabsf(fs(-1.f, x)));
                s[2] = pcs1(fabsf(x));
                s[4] = pcs3(fs(2.f, x));
                s[3] = fs(1.0f, fa(fa(fa(s[0], s[1]), s[2]), s[4]));
            }
        }

        // ChargeAssignment::shapeArray(pos, isOutOfRange): supp + 1 values
        __device__ static void caArray(float pos, bool oor, float* s)
        {
            float x = oor ? fs(pos, 1.0f) : pos;
            float v[supp + 1];
            base(x, v);
            s[supp] = oor ? v[supp - 1] : 0.0f;
#pragma unroll
            for(int k = supp - 1; k >= 1; --k)
                s[k] = oor ? v[k - 1] : v[k];
            s[0] = oor ? 0.0f : v[0];
        }

        // ChargeAssignment::operator()(x): the piecewise function
        __device__ static float ca(float x)
        {
            float ax = fabsf(x);
            if constexpr(SHAPE == 0)
                return (-0.5f <= x && x < 0.5f) ? 1.0f : 0.0f;
            else if constexpr(SHAPE == 1)
                return ax < 1.0f ? fs(1.0f, ax) : 0.0f;
            else if constexpr(SHAPE == 2)
            {
                float r1 = tsc1(ax), r2 = tsc2(ax);
                return ax < 0.5f ? r1 : (ax < 1.5f ? r2 : 0.0f);
            }
            else if constexpr(SHAPE == 3)
            {
                float r1 = pqs1(ax), r2 = pqs2(ax);
                return ax < 1.0f ? r1 : (ax < 2.0f ? r2 : 0.0f);
            }
            else
            {
                float r1 = pcs1(ax), r2 = pcs2(ax), r3 = pcs3(ax);
                float on = ax < 0.5f ? r1 : (ax < 1.5f ? r2 : r3);
                return ax < 2.5f ? on : 0.0f;
            }
        }
    };

    // ------------------------------------------------------------ geometry
    template<int SX_, int SY_, int SZ_>
    struct SuperCell
    {
        static constexpr int SX = SX_, SY = SY_, SZ = SZ_;
        static constexpr int volume = SX * SY * SZ;
    };

    // Per-launch grid constants (all in the units the caller chose).
    struct GridParams
    {
        int nx, ny, nz; // cells
        int nscx, nscy, nscz; // supercells
        float dx, dy, dz, dt, c, eps0;
        float rd[3]; // 1/dx, 1/dy, 1/dz
        int recipExact; // all cell sizes are powers of two: x / d == x * (1/d) exactly
        int open; // bit a set: axis a is open (no wrap; PML fields, absorbing particles)
    };

    // Index along an axis of n cells: periodic wrap, or -1 outside the box on an open axis.
    __device__ __forceinline__ int wrapOrOutside(int i, int n, bool open)
    {
        if(open)
            return (i < 0 || i >= n) ? -1 : i;
        return i < 0 ? i + n : (i >= n ? i - n : i);
    }

    // x / cellSize[d]: a multiplication by the exact reciprocal when the cell size is a
    // power of two (bit-identical to the IEEE division), the division otherwise.
    __device__ __forceinline__ float divCell(float x, int d, GridParams const& g)
    {
        if(g.recipExact)
            return fm(x, g.rd[d]);
        return fdv(x, d == 0 ? g.dx : (d == 1 ? g.dy : g.dz));
    }

    __device__ __forceinline__ float frcp(float x) { return __frcp_rn(x); } // == 1.0f / x, correctly rounded

    __device__ __forceinline__ int wrapi(int i, int n)
    {
        // valid for i in [-n, 2n)
        return i < 0 ? i + n : (i >= n ? i - n : i);
    }

    // ------------------------------------------------------------ gather
    // AssignedTrilinearInterpolation::interpolate (algorithms/AssignedTrilinearInterpolation.hpp:54-86):
    // z-y-x nested weighted sums over the support, each accumulation one fused
    // multiply-add (the contraction the reference's CUDA build applies to
    // `result += value * weight`; the oracle uses std::fma at the same places).
    // The tile origin is the supercell origin minus Shape::gLo in every direction.
    template<typename SH, int TX, int TY>
    __device__ __forceinline__ float interpolate(
        float const* __restrict__ tile,
        int lx,
        int ly,
        int lz,
        int shx,
        int shy,
        int shz,
        float const* sx,
        float const* sy,
        float const* sz)
    {
        constexpr int S = SH::supp;
        int const bx = lx + SH::gLo + shx + SH::osBegin;
        int const by = ly + SH::gLo + shy + SH::osBegin;
        int const bz = lz + SH::gLo + shz + SH::osBegin;
        float const* base = tile + (bx + TX * (by + TY * bz));
        float rz = 0.0f;
#pragma unroll
        for(int z = 0; z < S; ++z)
        {
            float ry = 0.0f;
#pragma unroll
            for(int y = 0; y < S; ++y)
            {
                float rx = 0.0f;
                float const* row = base + TX * (y + TY * z);
#pragma unroll
                for(int x = 0; x < S; ++x)
                    rx = __fmaf_rn(row[x], sx[x], rx);
                ry = __fmaf_rn(rx, sy[y], ry);
            }
            rz = __fmaf_rn(ry, sz[z], rz);
        }
        return rz;
    }

    // Two components gathered together with packed f32x2 fused multiply-adds (each half is the
    // scalar chain of `interpolate`, so both results are bit-identical to two scalar gathers).
    template<typename SH, int TX, int TY>
    __device__ __forceinline__ float2 interpolate2(
        float const* __restrict__ tileA,
        float const* __restrict__ tileB,
        int lx,
        int ly,
        int lz,
        int const shA[3],
        int const shB[3],
        float const* axA,
        float const* ayA,
        float const* azA,
        float const* axB,
        float const* ayB,
        float const* azB)
    {
        constexpr int S = SH::supp;
        float const* baseA = tileA
            + ((lx + SH::gLo + shA[0] + SH::osBegin)
               + TX * ((ly + SH::gLo + shA[1] + SH::osBegin) + TY * (lz + SH::gLo + shA[2] + SH::osBegin)));
        float const* baseB = tileB
            + ((lx + SH::gLo + shB[0] + SH::osBegin)
               + TX * ((ly + SH::gLo + shB[1] + SH::osBegin) + TY * (lz + SH::gLo + shB[2] + SH::osBegin)));
        float2 rz = make_float2(0.0f, 0.0f);
#pragma unroll
        for(int z = 0; z < S; ++z)
        {
            float2 ry = make_float2(0.0f, 0.0f);
#pragma unroll
            for(int y = 0; y < S; ++y)
            {
                float2 rx = make_float2(0.0f, 0.0f);
                float const* rowA = baseA + TX * (y + TY * z);
                float const* rowB = baseB + TX * (y + TY * z);
#pragma unroll
                for(int x = 0; x < S; ++x)
                    rx = __ffma2_rn(make_float2(rowA[x], rowB[x]), make_float2(axA[x], axB[x]), rx);
                ry = __ffma2_rn(rx, make_float2(ayA[y], ayB[y]), ry);
            }
            rz = __ffma2_rn(ry, make_float2(azA[z], azB[z]), rz);
        }
        return rz;
    }

    // ShiftCoordinateSystem (algorithms/ShiftCoordinateSystem.hpp:54-79) and the
    // on-support shape array for the two staggering offsets a Yee component can
    // have along an axis (0 and 1/2, fields/YeeCell.hpp:70-131).  The six
    // components of E and B reuse these six weight arrays.
    template<typename SH>
    struct GatherWeights
    {
        int sh[2][3];
        float w[2][3][SH::supp];

        __device__ __forceinline__ void compute(float const pos[3])
        {
#pragma unroll
            for(int a = 0; a < 2; ++a)
#pragma unroll
                for(int d = 0; d < 3; ++d)
                {
                    float const v = fs(fs(pos[d], a ? 0.5f : 0.0f), 0.5f);
                    int s;
                    if constexpr(SH::even)
                        s = v >= -0.5f ? 0 : -1;
                    else
                        s = v >= 0.0f ? 1 : 0;
                    sh[a][d] = s;
                    SH::base(fa(fs(v, float(s)), 0.5f), w[a][d]);
                }
        }

        // components A (staggering ax, ay, az) and B (bx, by, bz) together
        template<int TX, int TY, int ax, int ay, int az, int bx, int by, int bz>
        __device__ __forceinline__ float2 gather2(float const* __restrict__ tileA, float const* __restrict__ tileB, int lx, int ly, int lz) const
        {
            int const shA[3] = {sh[ax][0], sh[ay][1], sh[az][2]};
            int const shB[3] = {sh[bx][0], sh[by][1], sh[bz][2]};
            return interpolate2<SH, TX, TY>(
                tileA, tileB, lx, ly, lz, shA, shB, w[ax][0], w[ay][1], w[az][2], w[bx][0], w[by][1], w[bz][2]);
        }

        // ax, ay, az: staggering (0 or 1) of the component along x, y, z
        template<int TX, int TY, int ax, int ay, int az>
        __device__ __forceinline__ float gather(float const* __restrict__ tile, int lx, int ly, int lz) const
        {
            return interpolate<SH, TX, TY>(
                tile,
                lx,
                ly,
                lz,
                sh[ax][0],
                sh[ay][1],
                sh[az][2],
                w[ax][0],
                w[ay][1],
                w[az][2]);
        }
    };

    // ------------------------------------------------------------ push
    __device__ __forceinline__ float l2n2(float a, float b, float c) { return fa(fa(fm(a, a), fm(b, b)), fm(c, c)); }

    // Velocity (algorithms/Velocity.hpp:31-37) with a correctly rounded 1/sqrt
    __device__ __forceinline__ void velocity(float const mom[3], float mass, float rc2, float vel[3])
    {
        float const m0_2 = fm(mass, mass);
        float const fMom2 = l2n2(mom[0], mom[1], mom[2]);
        float const t = frcp(fsq(fa(m0_2, fm(fMom2, rc2))));
#pragma unroll
        for(int d = 0; d < 3; ++d)
            vel[d] = fm(t, mom[d]);
    }

    // Boris (particles/pusher/particlePusherBoris.hpp:42-90); mom updated in place, vel returned
    __device__ __forceinline__ void boris(
        float charge,
        float mass,
        float const E[3],
        float const B[3],
        float dt,
        float c2,
        float rc2,
        float mom[3],
        float vel[3])
    {
        float const QoM = fdv(charge, mass);
        float const hq = fm(0.5f, charge);
        float mm[3];
#pragma unroll
        for(int d = 0; d < 3; ++d)
            mm[d] = fa(mom[d], fm(fm(hq, E[d]), dt));
        // Gamma (algorithms/Gamma.hpp:30-37)
        float const m2_c2_reci = frcp(fm(fm(mass, mass), c2));
        float const gamma = fsq(fa(1.0f, fm(l2n2(mm[0], mm[1], mm[2]), m2_c2_reci)));
        float const gamma_reci = frcp(gamma);
        float const hqm = fm(0.5f, QoM);
        float t[3];
#pragma unroll
        for(int d = 0; d < 3; ++d)
            t[d] = fm(fm(fm(hqm, B[d]), gamma_reci), dt);
        float const sf = frcp(fa(1.0f, l2n2(t[0], t[1], t[2])));
        float s[3];
#pragma unroll
        for(int d = 0; d < 3; ++d)
            s[d] = fm(fm(2.0f, t[d]), sf);
        float mp[3], mq[3];
        mp[0] = fa(mm[0], fs(fm(mm[1], t[2]), fm(mm[2], t[1])));
        mp[1] = fa(mm[1], fs(fm(mm[2], t[0]), fm(mm[0], t[2])));
        mp[2] = fa(mm[2], fs(fm(mm[0], t[1]), fm(mm[1], t[0])));
        mq[0] = fa(mm[0], fs(fm(mp[1], s[2]), fm(mp[2], s[1])));
        mq[1] = fa(mm[1], fs(fm(mp[2], s[0]), fm(mp[0], s[2])));
        mq[2] = fa(mm[2], fs(fm(mp[0], s[1]), fm(mp[1], s[0])));
#pragma unroll
        for(int d = 0; d < 3; ++d)
            mom[d] = fa(mq[d], fm(fm(hq, E[d]), dt));
        velocity(mom, mass, rc2, vel);
    }

    // ---- HigueraCary and Vay.  Their square-root stages run in double, the
    // reference's default (param/pusher.param:56-72, precision64Bit); the rest in
    // float, with every float<->double cast where the reference's types put it.
    __device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
    __device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
    __device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
    __device__ __forceinline__ double ddv(double a, double b) { return __ddiv_rn(a, b); }
    __device__ __forceinline__ double dsq(double a) { return __dsqrt_rn(a); }
    __device__ __forceinline__ double dl2n2(double a, double b, double c) { return da(da(dm(a, a), dm(b, b)), dm(c, c)); }

    // Gamma<float_X> (algorithms/Gamma.hpp:30-37)
    __device__ __forceinline__ float gammaOf(float a, float b, float c, float mass, float c2)
    {
        float const m2_c2_reci = frcp(fm(fm(mass, mass), c2));
        return fsq(fa(1.0f, fm(l2n2(a, b, c), m2_c2_reci)));
    }

    // HigueraCary (particles/pusher/particlePusherHigueraCary.hpp:85-135): the new
    // momentum.  Kept out of line so the Boris kernels keep their register budget.
    static __device__ __noinline__ float3 higueraCary(float charge, float mass, float3 E, float3 B, float dt, float c, float c2, float3 mom)
    {
        float const hq = fm(0.5f, charge);
        // mom_minus = mom + 0.5 q E dt (float), then held in double
        float const mf[3] = {fa(mom.x, fm(fm(hq, E.x), dt)), fa(mom.y, fm(fm(hq, E.y), dt)), fa(mom.z, fm(fm(hq, E.z), dt))};
        double const mm[3] = {mf[0], mf[1], mf[2]};
        double const gm = gammaOf(mf[0], mf[1], mf[2], mass, c2);
        // tau = 0.5 B q dt / m (float), then held in double
        double const tau[3] = {fdv(fm(fm(fm(0.5f, B.x), charge), dt), mass), fdv(fm(fm(fm(0.5f, B.y), charge), dt), mass),
                               fdv(fm(fm(fm(0.5f, B.z), charge), dt), mass)};
        double const tau2 = dl2n2(tau[0], tau[1], tau[2]);
        double const sigma = ds(dm(gm, gm), tau2);
        double const ustar = ddv(da(da(dm(mm[0], tau[0]), dm(mm[1], tau[1])), dm(mm[2], tau[2])), double(fm(mass, c)));
        double const gp = dsq(dm(0.5, da(sigma, dsq(da(dm(sigma, sigma), dm(4.0, da(tau2, dm(ustar, ustar))))))));
        double const t[3] = {ddv(tau[0], gp), ddv(tau[1], gp), ddv(tau[2], gp)};
        double const s = ddv(1.0, da(1.0, dl2n2(t[0], t[1], t[2])));
        double const mt = da(da(dm(mm[0], t[0]), dm(mm[1], t[1])), dm(mm[2], t[2]));
        double const cr[3] = {ds(dm(mm[1], t[2]), dm(mm[2], t[1])), ds(dm(mm[2], t[0]), dm(mm[0], t[2])),
                              ds(dm(mm[0], t[1]), dm(mm[1], t[0]))};
        double mp[3];
#pragma unroll
        for(int d = 0; d < 3; ++d)
            mp[d] = dm(s, da(da(mm[d], dm(mt, t[d])), cr[d]));
        // the second half acceleration plus the rotation term cross(mom_plus, t), summed in float
        float const d2[3] = {__double2float_rn(ds(dm(mp[1], t[2]), dm(mp[2], t[1]))),
                             __double2float_rn(ds(dm(mp[2], t[0]), dm(mp[0], t[2]))),
                             __double2float_rn(ds(dm(mp[0], t[1]), dm(mp[1], t[0])))};
        float3 r;
        r.x = fa(__double2float_rn(mp[0]), fa(fm(fm(hq, E.x), dt), d2[0]));
        r.y = fa(__double2float_rn(mp[1]), fa(fm(fm(hq, E.y), dt), d2[1]));
        r.z = fa(__double2float_rn(mp[2]), fa(fm(fm(hq, E.z), dt), d2[2]));
        return r;
    }

    // Vay (particles/pusher/particlePusherVay.hpp:72-103): the new momentum.
    static __device__ __noinline__ float3 vay(float charge, float mass, float3 E, float3 B, float dt, float c, float c2, float rc2, float3 mom)
    {
        float const factor = fm(fm(0.5f, charge), dt);
        float const m[3] = {mom.x, mom.y, mom.z};
        float v[3];
        velocity(m, mass, rc2, v);
        float const Ev[3] = {E.x, E.y, E.z}, Bv[3] = {B.x, B.y, B.z};
        float const cvb[3] = {fs(fm(v[1], Bv[2]), fm(v[2], Bv[1])), fs(fm(v[2], Bv[0]), fm(v[0], Bv[2])),
                              fs(fm(v[0], Bv[1]), fm(v[1], Bv[0]))};
        float mp[3];
#pragma unroll
        for(int d = 0; d < 3; ++d)
            mp[d] = fa(fa(m[d], fm(factor, fa(Ev[d], cvb[d]))), fm(factor, Ev[d])); // momentum_atZero, momentum_prime
        float const gprime = gammaOf(mp[0], mp[1], mp[2], mass, c2);
        float const fom = fdv(factor, mass);
        double const tau[3] = {fm(fom, Bv[0]), fm(fom, Bv[1]), fm(fom, Bv[2])};
        double const tau2 = dl2n2(tau[0], tau[1], tau[2]);
        double const ustar = ddv(da(da(dm(mp[0], tau[0]), dm(mp[1], tau[1])), dm(mp[2], tau[2])), double(fm(c, mass)));
        double const sigma = ds(double(fm(gprime, gprime)), tau2);
        double const gph = dsq(dm(0.5, da(sigma, dsq(da(dm(sigma, sigma), dm(4.0, da(tau2, dm(ustar, ustar))))))));
        double const rg = ddv(1.0, gph);
        float const t[3] = {__double2float_rn(dm(tau[0], rg)), __double2float_rn(dm(tau[1], rg)),
                            __double2float_rn(dm(tau[2], rg))};
        float const s = frcp(fa(1.0f, l2n2(t[0], t[1], t[2])));
        float const mt = fa(fa(fm(mp[0], t[0]), fm(mp[1], t[1])), fm(mp[2], t[2]));
        float const cr[3] = {fs(fm(mp[1], t[2]), fm(mp[2], t[1])), fs(fm(mp[2], t[0]), fm(mp[0], t[2])),
                             fs(fm(mp[0], t[1]), fm(mp[1], t[0]))};
        float3 r;
        r.x = fm(s, fa(fa(mp[0], fm(mt, t[0])), cr[0]));
        r.y = fm(s, fa(fa(mp[1], fm(mt, t[1])), cr[1]));
        r.z = fm(s, fa(fa(mp[2], fm(mt, t[2])), cr[2]));
        return r;
    }

    // moveParticle (particles/MoveParticle.hpp:48-160).  pos in [-1,2) on entry,
    // [0,1) on exit; mv = cell move per axis; returns the supercell leave
    // direction through dir (0 when the particle stays inside its supercell).
    template<typename SC>
    __device__ __forceinline__ bool moveParticle(float pos[3], int& lcell, int mv[3], int dir[3])
    {
        bool moved = false;
#pragma unroll
        for(int i = 0; i < 3; ++i)
        {
            float p = fs(pos[i], 0.5f);
            float m = 0.0f;
            if(p < -0.5f)
                m = -1.0f;
            if(p >= 0.5f)
                m = 1.0f;
            p = fs(p, m);
            pos[i] = fa(p, 0.5f);
            mv[i] = int(m);
            moved |= (mv[i] != 0);
        }
        dir[0] = dir[1] = dir[2] = 0;
        if(!moved)
            return false;
        int lc[3] = {lcell % SC::SX, (lcell / SC::SX) % SC::SY, lcell / (SC::SX * SC::SY)};
        int const scs[3] = {SC::SX, SC::SY, SC::SZ};
        bool leave = false;
#pragma unroll
        for(int i = 0; i < 3; ++i)
        {
            lc[i] += mv[i];
            dir[i] = (unsigned(lc[i]) >= unsigned(scs[i])) ? mv[i] : 0;
            lc[i] -= dir[i] * scs[i];
            leave |= (dir[i] != 0);
        }
        lcell = lc[0] + SC::SX * (lc[1] + SC::SY * lc[2]);
        return leave;
    }

    // ------------------------------------------------------------ J accumulators
    // Maps the rotated axes (i, j, k) of current component C to real axes:
    // J_x: i->y, j->z, k->x; J_y: i->z, j->x, k->y; J_z: i->x, j->y, k->z
    // (rotateOrigin / PermutatedFieldValueAccess, Esirkepov.hpp:112-129).
    template<int C>
    __device__ __forceinline__ void rotToReal(int ri, int rj, int rk, int& x, int& y, int& z)
    {
        if constexpr(C == 0)
        {
            x = rk;
            y = ri;
            z = rj;
        }
        else if constexpr(C == 1)
        {
            x = rj;
            y = rk;
            z = ri;
        }
        else
        {
            x = ri;
            y = rj;
            z = rk;
        }
    }

    // Shared-memory J tile of one supercell: [3][TT] floats, or [2][3][TT] ints in fixed point.
#ifndef PICGB_SHORT_LOOP
    // 1: the short-footprint deposit runs its three components in a runtime loop
#    define PICGB_SHORT_LOOP 1
#endif

    // TX: row pitch, TP: plane pitch, TT: words of one component's tile
    template<int TX, int TP, int TT>
    struct TileJ
    {
        static constexpr int kTT = TT;
        float* J;
        int base; // tile index of the particle's Esirkepov origin (cell + gridShift)
        JFixed f;

        // Scale of the values passed to add(): 2^s in fixed point, 1 for floats.
        __device__ __forceinline__ float unit() const
        {
#if PICGB_J_FIXED
            return f.scale;
#else
            return 1.0f;
#endif
        }

        // v in units of unit().  In fixed point: a = rint(v / 2^k) and the remainder
        // r = v - a 2^k (exact), both rounded to integers by adding 1.5 * 2^23 (valid
        // for magnitudes below 2^22, which the host's choice of s and k guarantees),
        // so the whole conversion runs on the FMA pipe.
        template<int C>
        __device__ __forceinline__ void add(int ri, int rj, int rk, float v) const
        {
            int x, y, z;
            rotToReal<C>(ri, rj, rk, x, y, z);
            addAt(C * TT + base + x + TX * y + TP * z, v);
        }

        // word stride of real axis a (0 x, 1 y, 2 z)
        __device__ __forceinline__ static int stride(int a) { return a == 0 ? 1 : (a == 1 ? TX : TP); }

        // T * cum at tile word idx (component offset included by the caller); cumHi =
        // cum * 2^-k (exact).  In fixed point the high part a = rint(T cum 2^-k) comes from
        // one fused multiply-add on the exact product, the low part r = T cum - a 2^k from
        // another (one rounding), so a 2^k + rint(r) is the value rounded to a unit.
        __device__ __forceinline__ void addProduct(int idx, float T, float cum, float cumHi, float magicHi) const
        {
#if PICGB_J_FIXED
            constexpr float kMagic = 12582912.0f; // 1.5 * 2^23
            constexpr int kMagicBits = 0x4B400000;
            int* w = reinterpret_cast<int*>(J);
            float const t = __fmaf_rn(T, cumHi, kMagic); // kMagic + a
            float const na = __fmaf_rn(-t, f.hiUnit, magicHi); // -a 2^k, exact
            float const r = __fmaf_rn(T, cum, na);
            atomicAdd(w + idx, __float_as_int(t) - kMagicBits);
            atomicAdd(w + 3 * TT + idx, __float_as_int(__fadd_rn(r, kMagic)) - kMagicBits);
#else
            (void) cumHi;
            (void) magicHi;
            atomicAdd(J + idx, fm(T, cum));
#endif
        }

        // kMagic * 2^k, the constant of addProduct
        __device__ __forceinline__ float magicHi() const
        {
#if PICGB_J_FIXED
            return fm(12582912.0f, f.hiUnit);
#else
            return 0.0f;
#endif
        }

        __device__ __forceinline__ float hiStep() const
        {
#if PICGB_J_FIXED
            return f.hiStep;
#else
            return 1.0f;
#endif
        }

        // v at tile word idx of the first plane (component offset included by the caller)
        __device__ __forceinline__ void addAt(int idx, float v) const
        {
#if PICGB_J_FIXED
            constexpr float kMagic = 12582912.0f; // 1.5 * 2^23
            constexpr int kMagicBits = 0x4B400000;
            int* w = reinterpret_cast<int*>(J);
            float const t = __fmaf_rn(v, f.hiStep, kMagic); // kMagic + rint(v / 2^k)
            float const a = __fsub_rn(t, kMagic);
            float const r = __fmaf_rn(-a, f.hiUnit, v); // exact (Sterbenz)
            atomicAdd(w + idx, __float_as_int(t) - kMagicBits);
            atomicAdd(w + 3 * TT + idx, __float_as_int(__fadd_rn(r, kMagic)) - kMagicBits);
#else
            atomicAdd(J + idx, v);
#endif
        }
    };

    // Value of tile node t of component c (the flush of the tile).
    template<int TT>
    __device__ __forceinline__ float tileValue(float const* J, int i, JFixed const& f)
    {
#if PICGB_J_FIXED
        int const* hi = reinterpret_cast<int const*>(J);
        long long const t = (static_cast<long long>(hi[i]) << f.k) + hi[3 * TT + i];
        return fm(__ll2float_rn(t), f.invScale);
#else
        (void) f;
        return J[i];
#endif
    }

    // ------------------------------------------------------------ Esirkepov
    // Esirkepov::operator() (fields/currentDeposition/Esirkepov/Esirkepov.hpp:62-134),
    // cptCurrent1D (:147-242), relayPoint (relayPoint.hpp:48-64).
    template<typename SH>
    struct Esirkepov
    {
        static constexpr int S = SH::supp;
        static constexpr int begin = SH::caBegin;
        static constexpr int end = SH::caEnd;

        // status bits (Esirkepov/bitPacking.hpp:37-47): particle stays in its assignment cell
        static constexpr int kInCell = 2 | 4;

        // Trajectory of the particle in the virtual coordinate system: pos = in-cell
        // position after the move, vel from the new momentum.  Returns false when
        // the relay shift is out of range, which valid inputs (|v| dt < cell size)
        // never produce.
        __device__ __forceinline__ static bool prepare(
            float const pos[3],
            float const vel[3],
            GridParams const& g,
            float p0[3],
            float p1[3],
            int gs[3],
            int stat[3])
        {
#pragma unroll
            for(int d = 0; d < 3; ++d)
            {
                float const dp = divCell(fm(vel[d], g.dt), d, g);
                p0[d] = fs(pos[d], dp);
                p1[d] = pos[d];
                int iS, iE;
                if constexpr(SH::even)
                {
                    iS = int(floorf(p0[d]));
                    iE = int(floorf(p1[d]));
                }
                else
                {
                    iS = int(floorf(fa(p0[d], 0.5f)));
                    iE = int(floorf(fa(p1[d], 0.5f)));
                }
                gs[d] = iS < iE ? iS : iE;
                stat[d] = (gs[d] == iS ? 2 : 0) | (gs[d] == iE ? 4 : 0) | (iS != iE ? 1 : 0);
                p0[d] = fs(p0[d], float(gs[d]));
                p1[d] = fs(p1[d], float(gs[d]));
            }
            constexpr int gsHi = SH::even ? 0 : 1;
            bool ok = true;
#pragma unroll
            for(int d = 0; d < 3; ++d)
                ok &= (gs[d] >= -1 && gs[d] <= gsHi);
            return ok;
        }

        // One rotated 1D current (cptCurrent1D); the running sum runs along k.
        // kGeneral = false: the particle stays in its assignment cell along every
        // axis (status kInCell everywhere), so the loops have their short fixed
        // extent and the cached shapes need no out-of-range shift.
        template<int C, bool kGeneral, typename Acc>
        __device__ __forceinline__ static void cpt1D(
            Acc const& acc,
            int const stat[3],
            float const q0[3],
            float const q1[3],
            float csd)
        {
            if(q0[2] == q1[2])
                return;
            float sj0[S + 1], sj1[S + 1], sk0[S + 1], sk1[S + 1];
            SH::caArray(q0[1], kGeneral && !(stat[1] & 2), sj0);
            SH::caArray(q1[1], kGeneral && !(stat[1] & 4), sj1);
            SH::caArray(q0[2], kGeneral && !(stat[2] & 2), sk0);
            SH::caArray(q1[2], kGeneral && !(stat[2] & 4), sk1);
            float dsk[S];
#pragma unroll
            for(int k = 0; k < S; ++k)
                dsk[k] = fs(sk1[k], sk0[k]);
            int const leaveI = kGeneral ? (stat[0] & 1) : 0;
            int const leaveJ = kGeneral ? (stat[1] & 1) : 0;
            int const leaveK = kGeneral ? (stat[2] & 1) : 0;
            constexpr int endIJ = kGeneral ? end + 1 : end; // loop bound before the leave guard
            constexpr int endK = kGeneral ? end : end - 1;
            float const ncsd = -csd;
#pragma unroll
            for(int i = begin; i < endIJ; ++i)
                if(i < end + leaveI)
                {
                    float const s0i = SH::ca(fs(float(i), q0[0]));
                    float const dsi = fs(SH::ca(fs(float(i), q1[0])), s0i);
#pragma unroll
                    for(int j = begin; j < endIJ; ++j)
                        if(j < end + leaveJ)
                        {
                            float const s0j = sj0[j - begin];
                            float const dsj = fs(sj1[j - begin], s0j);
                            // s0i s0j + 1/2 (dsi s0j + s0i dsj) + 1/3 dsj dsi (Esirkepov.hpp:214-215),
                            // contracted to fused multiply-adds; J is compared within tolerance
                            float const half = fm(0.5f, __fmaf_rn(dsi, s0j, fm(s0i, dsj)));
                            float const tmp = fm(ncsd, __fmaf_rn(fm(1.0f / 3.0f, dsj), dsi, __fmaf_rn(s0i, s0j, half)));
                            float run = 0.0f;
#pragma unroll
                            for(int k = begin; k < endK; ++k)
                                if(k < end + leaveK - 1)
                                {
                                    run = __fmaf_rn(dsk[k - begin], tmp, run);
                                    acc.template add<C>(i, j, k, run);
                                }
                        }
                }
        }

        // The short footprint (the particle stays in its assignment cell along every axis) of
        // the three rotated components.  The on-support weights S0 (start) and S1 (end) of
        // each axis are evaluated once and shared by the components (ChargeAssignment of
        // the shape, TSC.hpp:85 etc.; the reference evaluates the same functions per node).
        // The Esirkepov weight of node (i, j) (Esirkepov.hpp:214-215),
        //   S0i S0j + 1/2 (dSi S0j + S0i dSj) + 1/3 dSi dSj = Ai Aj + dSi dSj / 12,
        // with A = (S0 + S1) / 2 and dS = S1 - S0, is one product and one fused
        // multiply-add; the running sum along k is the prefix sum of dSk.  The three
        // components run in one runtime loop, so the particle loop holds one copy of the
        // unrolled (i, j, k) body, and pick their axes' weights by selects.  J agrees with
        // the per-node evaluation to rounding (the tile sums in another order anyway).  Used
        // for the Esirkepov deposit of CIC and TSC, whose 2 x 3 x 3 weights fit the register
        // budget beside the rest of the push.
        template<typename Acc>
        __device__ __forceinline__ static void runShort(
            Acc const& acc,
            float const p0[3],
            float const p1[3],
            float const csd[3],
            int tileTT)
        {
            float A[3][S], D[3][S];
#pragma unroll
            for(int d = 0; d < 3; ++d)
            {
                float s0[S + 1], s1[S + 1];
                SH::caArray(p0[d], false, s0);
                SH::caArray(p1[d], false, s1);
#pragma unroll
                for(int m = 0; m < S; ++m)
                {
                    D[d][m] = fs(s1[m], s0[m]);
                    A[d][m] = fm(0.5f, fa(s0[m], s1[m]));
                }
            }
            float const magicHi = acc.magicHi(), hiStep = acc.hiStep();
#pragma unroll 1
            for(int C = 0; C < 3; ++C)
            {
                // rotated axes: i -> C + 1, j -> C + 2, k -> C (mod 3)
                bool const c0 = C == 0, c1 = C == 1;
                if(c0 ? p0[0] == p1[0] : (c1 ? p0[1] == p1[1] : p0[2] == p1[2]))
                    continue; // no motion along k: no current
                int const ai = C == 2 ? 0 : C + 1;
                int const aj = c0 ? 2 : C - 1;
                auto pick = [](float const (&X)[3][S], int a, int m)
                { return a == 0 ? X[0][m] : (a == 1 ? X[1][m] : X[2][m]); };
                int const si = Acc::stride(ai), sj = Acc::stride(aj), sk = Acc::stride(C);
                float const ncsd = -(c0 ? csd[0] : (c1 ? csd[1] : csd[2]));
                float const ncsd12 = fm(ncsd, 1.0f / 12.0f);
                float cum[S - 1], cumHi[S - 1];
                {
                    float run = 0.0f;
#pragma unroll
                    for(int k = 0; k < S - 1; ++k)
                    {
                        run = fa(run, pick(D, C, k));
                        cum[k] = run;
                        cumHi[k] = fm(run, hiStep);
                    }
                }
                float Aj[S], Dj[S];
#pragma unroll
                for(int m = 0; m < S; ++m)
                {
                    Aj[m] = pick(A, aj, m);
                    Dj[m] = pick(D, aj, m);
                }
                int const base = acc.base + C * tileTT + begin * (si + sj + sk);
#pragma unroll
                for(int i = 0; i < S; ++i)
                {
                    float const ai_ = fm(ncsd, pick(A, ai, i));
                    float const di_ = fm(ncsd12, pick(D, ai, i));
#pragma unroll
                    for(int j = 0; j < S; ++j)
                    {
                        float const T = __fmaf_rn(ai_, Aj[j], fm(di_, Dj[j]));
                        int const row = base + i * si + j * sj;
#pragma unroll
                        for(int k = 0; k < S - 1; ++k)
                            acc.addProduct(row + k * sk, T, cum[k], cumHi[k], magicHi);
                    }
                }
            }
        }

        // The short footprint with the weights evaluated per component and node, the
        // arithmetic of cpt1D<C, false> (Esirkepov.hpp:200-241): fewer values live at once
        // than in runShort, which keeps the register budget of the PQS and PCS kernels and of
        // the EmZ variants (whose second virtual particle stays live across this deposit)
        // without spills.  The three rotated components run in one runtime loop; the rotation
        // maps rotated axes i, j, k to real axes C+1, C+2, C.
        template<typename Acc>
        __device__ __forceinline__ static void runShortPerNode(
            Acc const& acc,
            float const p0[3],
            float const p1[3],
            float const csd[3],
            int tileTT)
        {
            auto sel = [](float const* p, int a) { return a == 0 ? p[0] : (a == 1 ? p[1] : p[2]); };
#pragma unroll 1
            for(int C = 0; C < 3; ++C)
            {
                int const ai = C == 2 ? 0 : C + 1;
                int const aj = C == 0 ? 2 : C - 1;
                float const q0[3] = {sel(p0, ai), sel(p0, aj), sel(p0, C)};
                float const q1[3] = {sel(p1, ai), sel(p1, aj), sel(p1, C)};
                if(q0[2] == q1[2])
                    continue;
                int const si = Acc::stride(ai), sj = Acc::stride(aj), sk = Acc::stride(C);
                int const base = acc.base + C * tileTT;
                float sj0[S + 1], sj1[S + 1], sk0[S + 1], sk1[S + 1];
                SH::caArray(q0[1], false, sj0);
                SH::caArray(q1[1], false, sj1);
                SH::caArray(q0[2], false, sk0);
                SH::caArray(q1[2], false, sk1);
                float dsk[S];
#pragma unroll
                for(int k = 0; k < S; ++k)
                    dsk[k] = fs(sk1[k], sk0[k]);
                float const ncsd = -sel(csd, C);
#pragma unroll
                for(int i = begin; i < end; ++i)
                {
                    float const s0i = SH::ca(fs(float(i), q0[0]));
                    float const dsi = fs(SH::ca(fs(float(i), q1[0])), s0i);
#pragma unroll
                    for(int j = begin; j < end; ++j)
                    {
                        float const s0j = sj0[j - begin];
                        float const dsj = fs(sj1[j - begin], s0j);
                        float const half = fm(0.5f, __fmaf_rn(dsi, s0j, fm(s0i, dsj)));
                        float const tmp = fm(ncsd, __fmaf_rn(fm(1.0f / 3.0f, dsj), dsi, __fmaf_rn(s0i, s0j, half)));
                        float run = 0.0f;
                        int const row = base + i * si + j * sj;
#pragma unroll
                        for(int k = begin; k < end - 1; ++k)
                        {
                            run = __fmaf_rn(dsk[k - begin], tmp, run);
                            acc.addAt(row + k * sk, run);
                        }
                    }
                }
            }
        }

        // the three rotated calls; csd = charge * (1/(V*dt)) * cellEdgeLength (Esirkepov.hpp:188-190)
        template<bool kGeneral, typename Acc>
        __device__ __forceinline__ static void run(
            Acc const& acc,
            float const p0[3],
            float const p1[3],
            int const stat[3],
            float charge,
            GridParams const& g,
            float invVdt)
        {
            float const qv = fm(charge, invVdt);
            // the accumulator's unit (a power of two) is applied to csd: exact, and the
            // deposited values arrive already scaled
            float const u = acc.unit();
#if PICGB_SHORT_LOOP
            if constexpr(!kGeneral)
            {
                float const csd[3] = {fm(fm(qv, g.dx), u), fm(fm(qv, g.dy), u), fm(fm(qv, g.dz), u)};
                if constexpr(S <= 3)
                    runShort(acc, p0, p1, csd, Acc::kTT);
                else
                    runShortPerNode(acc, p0, p1, csd, Acc::kTT);
                return;
            }
#endif
            {
                int const st[3] = {stat[1], stat[2], stat[0]};
                float const a0[3] = {p0[1], p0[2], p0[0]}, a1[3] = {p1[1], p1[2], p1[0]};
                cpt1D<0, kGeneral>(acc, st, a0, a1, fm(fm(qv, g.dx), u));
            }
            {
                int const st[3] = {stat[2], stat[0], stat[1]};
                float const a0[3] = {p0[2], p0[0], p0[1]}, a1[3] = {p1[2], p1[0], p1[1]};
                cpt1D<1, kGeneral>(acc, st, a0, a1, fm(fm(qv, g.dy), u));
            }
            cpt1D<2, kGeneral>(acc, stat, p0, p1, fm(fm(qv, g.dz), u));
        }

        // ---- EmZ (fields/currentDeposition/EmZ/EmZ.hpp:72-120): the trajectory is split at
        // the relay point (relayPoint.hpp:48-64) into at most two virtual particles, each
        // on support, so each deposits with the short footprint of cpt1D<C, false>
        // (EmZ/DepositCurrent.hpp:76-126: on-support shapes, loops [begin, begin + supp)).
        // a0 -> a1 in the frame of cell shift sS, b0 -> b1 in the frame of sE; returns
        // false when a shift is out of range, which valid inputs (|v| dt < cell) never give.
        __device__ __forceinline__ static bool prepareEmZ(
            float const pos[3],
            float const vel[3],
            GridParams const& g,
            float a0[3],
            float a1[3],
            int sS[3],
            float b0[3],
            float b1[3],
            int sE[3],
            bool& two)
        {
            two = false;
            bool ok = true;
#pragma unroll
            for(int d = 0; d < 3; ++d)
            {
                float const x2 = pos[d];
                float const x1 = fs(x2, divCell(fm(vel[d], g.dt), d, g));
                int i1, i2;
                float relay;
                if constexpr(SH::even)
                {
                    i1 = int(floorf(x1));
                    i2 = int(floorf(x2));
                    relay = i1 == i2 ? x2 : float(i1 > i2 ? i1 : i2);
                }
                else
                {
                    i1 = int(floorf(fa(x1, 0.5f)));
                    i2 = int(floorf(fa(x2, 0.5f)));
                    relay = i1 == i2 ? x2 : fdv(float(i1 + i2), 2.0f);
                }
                sS[d] = i1;
                sE[d] = i2;
                a0[d] = fs(x1, float(i1));
                a1[d] = fs(relay, float(i1));
                b0[d] = fs(relay, float(i2));
                b1[d] = fs(x2, float(i2));
                two |= (i1 != i2);
                ok &= (i1 >= -1 && i1 <= (SH::even ? 1 : 2) && i2 >= 0 && i2 <= (SH::even ? 0 : 1));
            }
            return ok;
        }

        // One EmZ virtual particle (EmZ/DepositCurrent.hpp:38-63): chargeDensity = q / V and
        // currentSurfaceDensity = cellEdge * chargeDensity / dt, in the reference's order.
        template<typename Acc>
        __device__ __forceinline__ static void runEmZ(
            Acc const& acc,
            float const p0[3],
            float const p1[3],
            float charge,
            GridParams const& g)
        {
            int const st[3] = {kInCell, kInCell, kInCell};
            float const rho = fdv(charge, fm(fm(g.dx, g.dy), g.dz));
            float const u = acc.unit();
#if PICGB_SHORT_LOOP
            {
                float const csd[3] = {fm(fdv(fm(g.dx, rho), g.dt), u), fm(fdv(fm(g.dy, rho), g.dt), u),
                                      fm(fdv(fm(g.dz, rho), g.dt), u)};
                runShortPerNode(acc, p0, p1, csd, Acc::kTT);
                return;
            }
#endif
            {
                float const a0[3] = {p0[1], p0[2], p0[0]}, a1[3] = {p1[1], p1[2], p1[0]};
                cpt1D<0, false>(acc, st, a0, a1, fm(fdv(fm(g.dx, rho), g.dt), u));
            }
            {
                float const a0[3] = {p0[2], p0[0], p0[1]}, a1[3] = {p1[2], p1[0], p1[1]};
                cpt1D<1, false>(acc, st, a0, a1, fm(fdv(fm(g.dy, rho), g.dt), u));
            }
            cpt1D<2, false>(acc, st, p0, p1, fm(fdv(fm(g.dz, rho), g.dt), u));
        }
    };

} // namespace picgb
