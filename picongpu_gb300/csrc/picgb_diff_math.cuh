// Differentiable PIC step: the forward operations of one step on particles kept
// in a fixed order (no supercell sort), and their hand-written adjoints.
// Templated on the real type T (float or double) so that the same code gives
// the FP32 run and the FP64 reference gradient.
//
// Forward (per particle, as in the single-box step): form-factor gather of E
// and B (algorithms/FieldToParticleInterpolation.hpp:97-124 with
// ShiftCoordinateSystem.hpp:54-79), Boris (particles/pusher/particlePusherBoris.hpp:49-89),
// Velocity (algorithms/Velocity.hpp:31-37), the move (particles/MoveParticle.hpp:48-160)
// and the Esirkepov deposit (fields/currentDeposition/Esirkepov/Esirkepov.hpp:62-242).
// Adjoint: the transposed Jacobian of each of these maps, applied in reverse
// order.  The gather's transpose is a deposit of the adjoint force with the
// same weights; the deposit's transpose gathers the adjoint current with the
// derivatives of the Esirkepov weights.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace picgb::diff
{
    // constant factors as multiplications (a division by a constant is a full IEEE divide)
    template<typename T>
    __host__ __device__ constexpr T third()
    {
        return T(1.0 / 3.0);
    }
    template<typename T>
    __host__ __device__ constexpr T sixth()
    {
        return T(1.0 / 6.0);
    }

    template<typename T>
    struct DiffGrid
    {
        int nx, ny, nz;
        T dx, dy, dz, dt, c, eps0;
    };

    // periodic index for i in [-n, 2n) (stencil offsets of a few cells; grids have n >= 4)
    __device__ __forceinline__ int wrapIdx(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

    template<typename T>
    __device__ __forceinline__ T cellSize(DiffGrid<T> const& g, int d)
    {
        return d == 0 ? g.dx : (d == 1 ? g.dy : g.dz);
    }

    template<typename T>
    __device__ __forceinline__ size_t cellIndex(DiffGrid<T> const& g, int x, int y, int z)
    {
        return size_t(wrapIdx(x, g.nx)) + size_t(g.nx) * (size_t(wrapIdx(y, g.ny)) + size_t(g.ny) * size_t(wrapIdx(z, g.nz)));
    }

    // B-spline assignment functions (particles/shapes/CIC.hpp, TSC.hpp, PQS.hpp) and derivatives.
    template<int SHAPE, typename T>
    struct DShape
    {
        static constexpr int supp = SHAPE + 1;
        static constexpr bool even = (supp % 2) == 0;
        static constexpr int caBegin = SHAPE == 1 ? 0 : -1;
        static constexpr int caEnd = caBegin + supp;
        static constexpr int osBegin = -supp / 2 + (supp + 1) % 2;

        // on-support weights at the shifted position x (gather) and their derivatives
        __device__ static void base(T x, T* s, T* ds)
        {
            if constexpr(SHAPE == 1)
            {
                s[0] = T(1) - x;
                s[1] = x;
                ds[0] = T(-1);
                ds[1] = T(1);
            }
            else if constexpr(SHAPE == 2)
            {
                T const a = T(0.5) - x, b = T(0.5) + x;
                s[0] = T(0.5) * a * a;
                s[1] = T(0.75) - x * x;
                s[2] = T(0.5) * b * b;
                ds[0] = -a;
                ds[1] = T(-2) * x;
                ds[2] = b;
            }
            else
            {
                T const a = T(1) - x, x2 = x * x;
                s[0] = a * a * a * sixth<T>();
                s[1] = (T(4) - T(6) * x2 + T(3) * x2 * x) * sixth<T>();
                s[3] = x2 * x * sixth<T>();
                s[2] = T(1) - s[0] - s[1] - s[3];
                ds[0] = T(-0.5) * a * a;
                ds[1] = T(-2) * x + T(1.5) * x2;
                ds[3] = T(0.5) * x2;
                ds[2] = -(ds[0] + ds[1] + ds[3]);
            }
        }

        // ChargeAssignment (the piecewise function of the distance) and its derivative
        // both branches are evaluated and selected (no divergence between lanes)
        __device__ static T ca(T t)
        {
            T const a = t < T(0) ? -t : t;
            if constexpr(SHAPE == 1)
                return a < T(1) ? T(1) - a : T(0);
            else if constexpr(SHAPE == 2)
            {
                T const b = T(1.5) - a;
                T const inner = T(0.75) - t * t, outer = T(0.5) * b * b;
                return a < T(0.5) ? inner : (a < T(1.5) ? outer : T(0));
            }
            else
            {
                T const b = T(2) - a;
                T const inner = (T(4) - T(6) * t * t + T(3) * a * a * a) * sixth<T>(), outer = b * b * b * sixth<T>();
                return a < T(1) ? inner : (a < T(2) ? outer : T(0));
            }
        }

        __device__ static T dca(T t)
        {
            T const a = t < T(0) ? -t : t;
            T const sg = t < T(0) ? T(-1) : T(1);
            if constexpr(SHAPE == 1)
                return a < T(1) ? -sg : T(0);
            else if constexpr(SHAPE == 2)
            {
                T const inner = T(-2) * t, outer = -(T(1.5) - a) * sg;
                return a < T(0.5) ? inner : (a < T(1.5) ? outer : T(0));
            }
            else
            {
                T const b = T(2) - a;
                T const inner = T(-2) * t + T(1.5) * t * a, outer = T(-0.5) * b * b * sg;
                return a < T(1) ? inner : (a < T(2) ? outer : T(0));
            }
        }
    };

    // Yee staggering of the six components (fields/YeeCell.hpp:70-131): E_x (1/2,0,0) ... B_x (0,1/2,1/2) ...
    __host__ __device__ constexpr int stagger(int comp, int axis)
    {
        // comp 0..2 = E_x..E_z, 3..5 = B_x..B_z
        return comp < 3 ? (comp == axis ? 1 : 0) : ((comp - 3) == axis ? 0 : 1);
    }

    // Gather weights of one particle: for both Yee staggerings (0, 1/2) along each axis,
    // the first node and the on-support weights with their position derivatives.
    template<int SHAPE, typename T>
    struct DGather
    {
        using SH = DShape<SHAPE, T>;
        static constexpr int S = SH::supp;
        uint32_t off[2][3][S]; // wrapped node index times the axis stride
        T w[2][3][S];
        T dw[2][3][S];

        __device__ void compute(int const cell[3], T const pos[3], DiffGrid<T> const& g)
        {
            int const n3[3] = {g.nx, g.ny, g.nz};
            uint32_t const stride[3] = {1u, uint32_t(g.nx), uint32_t(g.nx) * uint32_t(g.ny)};
#pragma unroll
            for(int a = 0; a < 2; ++a)
#pragma unroll
                for(int d = 0; d < 3; ++d)
                {
                    T const v = pos[d] - (a ? T(0.5) : T(0)) - T(0.5);
                    int s;
                    if constexpr(SH::even)
                        s = v >= T(-0.5) ? 0 : -1;
                    else
                        s = v >= T(0) ? 1 : 0;
                    int const first = cell[d] + s + SH::osBegin;
#pragma unroll
                    for(int t = 0; t < S; ++t)
                        off[a][d][t] = uint32_t(wrapIdx(first + t, n3[d])) * stride[d];
                    SH::base(v - T(s) + T(0.5), w[a][d], dw[a][d]);
                }
        }

        // weights and node offsets of one axis for staggering a (0 or 1), without dynamic indexing
        __device__ __forceinline__ void axis(int d, int a, T wt[S], T dwt[S], uint32_t o[S]) const
        {
#pragma unroll
            for(int t = 0; t < S; ++t)
            {
                T const w0 = d == 0 ? w[0][0][t] : (d == 1 ? w[0][1][t] : w[0][2][t]);
                T const w1 = d == 0 ? w[1][0][t] : (d == 1 ? w[1][1][t] : w[1][2][t]);
                T const d0 = d == 0 ? dw[0][0][t] : (d == 1 ? dw[0][1][t] : dw[0][2][t]);
                T const d1 = d == 0 ? dw[1][0][t] : (d == 1 ? dw[1][1][t] : dw[1][2][t]);
                uint32_t const o0 = d == 0 ? off[0][0][t] : (d == 1 ? off[0][1][t] : off[0][2][t]);
                uint32_t const o1 = d == 0 ? off[1][0][t] : (d == 1 ? off[1][1][t] : off[1][2][t]);
                wt[t] = a ? w1 : w0;
                dwt[t] = a ? d1 : d0;
                o[t] = a ? o1 : o0;
            }
        }

        // component comp (0..2 E_x..E_z, 3..5 B_x..B_z, a runtime value) of field F
        __device__ T valueAt(T const* __restrict__ F, int comp) const
        {
            T wx[S], wy[S], wz[S], dx[S], dy[S], dz[S];
            uint32_t ox[S], oy[S], oz[S];
            axis(0, stagger(comp, 0), wx, dx, ox);
            axis(1, stagger(comp, 1), wy, dy, oy);
            axis(2, stagger(comp, 2), wz, dz, oz);
            T rz = T(0);
#pragma unroll
            for(int z = 0; z < S; ++z)
            {
                T ry = T(0);
#pragma unroll
                for(int y = 0; y < S; ++y)
                {
                    T rx = T(0);
#pragma unroll
                    for(int x = 0; x < S; ++x)
                        rx += wx[x] * F[oz[z] + oy[y] + ox[x]];
                    ry += wy[y] * rx;
                }
                rz += wz[z] * ry;
            }
            return rz;
        }

        // valueAt() and its gradient with respect to the particle position (nested sums)
        __device__ T valueGradAt(T const* __restrict__ F, int comp, T grad[3]) const
        {
            T wx[S], wy[S], wz[S], dx[S], dy[S], dz[S];
            uint32_t ox[S], oy[S], oz[S];
            axis(0, stagger(comp, 0), wx, dx, ox);
            axis(1, stagger(comp, 1), wy, dy, oy);
            axis(2, stagger(comp, 2), wz, dz, oz);
            T v = T(0), gx = T(0), gy = T(0), gz = T(0);
#pragma unroll
            for(int z = 0; z < S; ++z)
            {
                T pz = T(0), pdx = T(0), pdy = T(0);
#pragma unroll
                for(int y = 0; y < S; ++y)
                {
                    T sx = T(0), sdx = T(0);
#pragma unroll
                    for(int x = 0; x < S; ++x)
                    {
                        T const f = F[oz[z] + oy[y] + ox[x]];
                        sx += f * wx[x];
                        sdx += f * dx[x];
                    }
                    pz += wy[y] * sx;
                    pdx += wy[y] * sdx;
                    pdy += dy[y] * sx;
                }
                v += wz[z] * pz;
                gx += wz[z] * pdx;
                gy += wz[z] * pdy;
                gz += dz[z] * pz;
            }
            grad[0] = gx;
            grad[1] = gy;
            grad[2] = gz;
            return v;
        }

        // scatter part of adjointAt() alone: lam * weights added into lamF
        __device__ void scatterAt(T* __restrict__ lamF, int comp, T lam) const
        {
            if(lam == T(0))
                return;
            T wx[S], wy[S], wz[S], dx[S], dy[S], dz[S];
            uint32_t ox[S], oy[S], oz[S];
            axis(0, stagger(comp, 0), wx, dx, ox);
            axis(1, stagger(comp, 1), wy, dy, oy);
            axis(2, stagger(comp, 2), wz, dz, oz);
#pragma unroll
            for(int z = 0; z < S; ++z)
#pragma unroll
                for(int y = 0; y < S; ++y)
                {
                    T const lyz = lam * wy[y] * wz[z];
#pragma unroll
                    for(int x = 0; x < S; ++x)
                        atomicAdd(lamF + oz[z] + oy[y] + ox[x], lyz * wx[x]);
                }
        }

        // adjoint of valueAt(): lam * weights scattered into lamF, and the position gradient
        __device__ void adjointAt(T const* __restrict__ F, T* __restrict__ lamF, int comp, T lam, T gpos[3]) const
        {
            if(lam == T(0))
                return;
            T wx[S], wy[S], wz[S], dx[S], dy[S], dz[S];
            uint32_t ox[S], oy[S], oz[S];
            axis(0, stagger(comp, 0), wx, dx, ox);
            axis(1, stagger(comp, 1), wy, dy, oy);
            axis(2, stagger(comp, 2), wz, dz, oz);
            // nested sums as in the gather: per row the value and its x-derivative, per plane
            // the y-derivative, then z; the scattered value per node is (lam wy wz) wx
            T gx = T(0), gy = T(0), gz = T(0);
#pragma unroll
            for(int z = 0; z < S; ++z)
            {
                T pz = T(0), pdx = T(0), pdy = T(0);
#pragma unroll
                for(int y = 0; y < S; ++y)
                {
                    T const lyz = lam * wy[y] * wz[z];
                    T sx = T(0), sdx = T(0);
#pragma unroll
                    for(int x = 0; x < S; ++x)
                    {
                        uint32_t const i = oz[z] + oy[y] + ox[x];
                        atomicAdd(lamF + i, lyz * wx[x]);
                        T const f = F[i];
                        sx += f * wx[x];
                        sdx += f * dx[x];
                    }
                    pz += wy[y] * sx;
                    pdx += wy[y] * sdx;
                    pdy += dy[y] * sx;
                }
                gx += wz[z] * pdx;
                gy += wz[z] * pdy;
                gz += dz[z] * pz;
            }
            gpos[0] += lam * gx;
            gpos[1] += lam * gy;
            gpos[2] += lam * gz;
        }
    };

    // Boris step with the intermediates its adjoint needs.
    template<typename T>
    struct DBoris
    {
        T mm[3], t[3], s[3], mp[3], gamma, sf;

        __device__ void forward(T qw, T mw, T const E[3], T const B[3], T dt, T c, T const p[3], T out[3])
        {
            T const hq = T(0.5) * qw * dt;
            for(int d = 0; d < 3; ++d)
                mm[d] = p[d] + hq * E[d];
            T const mm2 = mm[0] * mm[0] + mm[1] * mm[1] + mm[2] * mm[2];
            gamma = sqrt(T(1) + mm2 / (mw * mw * c * c));
            T const f = T(0.5) * (qw / mw) * dt / gamma;
            for(int d = 0; d < 3; ++d)
                t[d] = f * B[d];
            sf = T(1) / (T(1) + t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
            for(int d = 0; d < 3; ++d)
                s[d] = T(2) * t[d] * sf;
            mp[0] = mm[0] + (mm[1] * t[2] - mm[2] * t[1]);
            mp[1] = mm[1] + (mm[2] * t[0] - mm[0] * t[2]);
            mp[2] = mm[2] + (mm[0] * t[1] - mm[1] * t[0]);
            T mq[3];
            mq[0] = mm[0] + (mp[1] * s[2] - mp[2] * s[1]);
            mq[1] = mm[1] + (mp[2] * s[0] - mp[0] * s[2]);
            mq[2] = mm[2] + (mp[0] * s[1] - mp[1] * s[0]);
            for(int d = 0; d < 3; ++d)
                out[d] = mq[d] + hq * E[d];
        }

        // given lamOut = dL/d(out): dL/dp, dL/dE, dL/dB
        __device__ void adjoint(T qw, T mw, T const B[3], T dt, T c, T const lamOut[3], T lp[3], T lE[3], T lB[3]) const
        {
            T const hq = T(0.5) * qw * dt;
            T lmq[3], lmm[3], lmp[3], ls[3], lt[3];
            for(int d = 0; d < 3; ++d)
            {
                lmq[d] = lamOut[d];
                lE[d] = hq * lamOut[d];
            }
            // mq = mm + mp x s
            for(int d = 0; d < 3; ++d)
                lmm[d] = lmq[d];
            cross(s, lmq, lmp); // d(mp x s)/dmp^T lam = s x lam
            cross(lmq, mp, ls); // d(mp x s)/ds^T lam = lam x mp
            // mp = mm + mm x t
            T tmp[3];
            cross(t, lmp, tmp);
            for(int d = 0; d < 3; ++d)
                lmm[d] += lmp[d] + tmp[d];
            cross(lmp, mm, lt);
            // s = 2 t sf, sf = 1 / (1 + t.t)
            T const tls = t[0] * ls[0] + t[1] * ls[1] + t[2] * ls[2];
            for(int d = 0; d < 3; ++d)
                lt[d] += T(2) * sf * ls[d] - T(4) * sf * sf * tls * t[d];
            // t = (qw / mw) dt B / (2 gamma)
            T const f = T(0.5) * (qw / mw) * dt / gamma;
            T const tlt = t[0] * lt[0] + t[1] * lt[1] + t[2] * lt[2];
            for(int d = 0; d < 3; ++d)
                lB[d] = f * lt[d];
            T const lgamma = -tlt / gamma;
            // gamma = sqrt(1 + mm.mm / (mw c)^2)
            T const g2 = lgamma / (gamma * mw * mw * c * c);
            for(int d = 0; d < 3; ++d)
                lmm[d] += g2 * mm[d];
            // mm = p + hq E
            for(int d = 0; d < 3; ++d)
            {
                lp[d] = lmm[d];
                lE[d] += hq * lmm[d];
            }
            (void) B;
        }

        __device__ static void cross(T const a[3], T const b[3], T out[3])
        {
            out[0] = a[1] * b[2] - a[2] * b[1];
            out[1] = a[2] * b[0] - a[0] * b[2];
            out[2] = a[0] * b[1] - a[1] * b[0];
        }
    };

    // v = p / sqrt(mw^2 + p.p / c^2) and the transpose of its Jacobian
    template<typename T>
    __device__ void dVelocity(T mw, T c, T const p[3], T v[3])
    {
        T const D = sqrt(mw * mw + (p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) / (c * c));
        for(int d = 0; d < 3; ++d)
            v[d] = p[d] / D;
    }

    template<typename T>
    __device__ void dVelocityAdjoint(T mw, T c, T const p[3], T const lv[3], T lp[3])
    {
        T const D = sqrt(mw * mw + (p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) / (c * c));
        T const pl = p[0] * lv[0] + p[1] * lv[1] + p[2] * lv[2];
        for(int d = 0; d < 3; ++d)
            lp[d] += lv[d] / D - p[d] * pl / (c * c * D * D * D);
    }

    // a[i] for a runtime axis i without dynamic register indexing
    template<typename V>
    __device__ __forceinline__ V sel3(V const a[3], int i)
    {
        return i == 0 ? a[0] : (i == 1 ? a[1] : a[2]);
    }

    template<typename V>
    __device__ __forceinline__ void add3(V a[3], int i, V v)
    {
        a[0] += i == 0 ? v : V(0);
        a[1] += i == 1 ? v : V(0);
        a[2] += i == 2 ? v : V(0);
    }

    // Rotations of the three current components: rotated axis r of component C is real axis rot(C, r)
    // (J_x: i->y, j->z, k->x; J_y: i->z, j->x, k->y; J_z: i->x, j->y, k->z).
    __host__ __device__ constexpr int rot(int C, int r)
    {
        return C == 0 ? (r == 0 ? 1 : (r == 1 ? 2 : 0)) : (C == 1 ? (r == 0 ? 2 : (r == 1 ? 0 : 1)) : r);
    }

    // Esirkepov trajectory in the virtual grid: start q0 and end q1 relative to the
    // origin cell (new cell + shift), the per-axis leave flags, and the wrapped,
    // strided offsets of the N = supp + 1 nodes per axis the deposit can touch.
    template<int SHAPE, typename T>
    struct DTrajectory
    {
        using SH = DShape<SHAPE, T>;
        static constexpr int B0 = SH::caBegin;
        static constexpr int N = SH::caEnd - SH::caBegin + 1;
        T q0[3], q1[3];
        int leave[3];
        uint32_t node[3][N];
        T s0[3][N], s1[3][N]; // S(node - q0), S(node - q1) per axis

        __device__ void compute(int const newCell[3], T const pos[3], T const dp[3], DiffGrid<T> const& g)
        {
            int const n3[3] = {g.nx, g.ny, g.nz};
            uint32_t const stride[3] = {1u, uint32_t(g.nx), uint32_t(g.nx) * uint32_t(g.ny)};
#pragma unroll
            for(int d = 0; d < 3; ++d)
            {
                T const p0 = pos[d] - dp[d], p1 = pos[d];
                int iS, iE;
                if constexpr(SH::even)
                {
                    iS = int(floor(p0));
                    iE = int(floor(p1));
                }
                else
                {
                    iS = int(floor(p0 + T(0.5)));
                    iE = int(floor(p1 + T(0.5)));
                }
                int const gs = iS < iE ? iS : iE;
                leave[d] = iS != iE ? 1 : 0;
                q0[d] = p0 - T(gs);
                q1[d] = p1 - T(gs);
                int const o = newCell[d] + gs + B0;
#pragma unroll
                for(int t = 0; t < N; ++t)
                {
                    node[d][t] = uint32_t(wrapIdx(o + t, n3[d])) * stride[d];
                    s0[d][t] = SH::ca(T(B0 + t) - q0[d]);
                    s1[d][t] = SH::ca(T(B0 + t) - q1[d]);
                }
            }
        }

        // shape values at the N nodes of axis d for the start and end positions, and the node offsets
        __device__ __forceinline__ void line(int d, T a0[], T a1[], uint32_t nd[]) const
        {
#pragma unroll
            for(int t = 0; t < N; ++t)
            {
                a0[t] = d == 0 ? s0[0][t] : (d == 1 ? s0[1][t] : s0[2][t]);
                a1[t] = d == 0 ? s1[0][t] : (d == 1 ? s1[1][t] : s1[2][t]);
                nd[t] = d == 0 ? node[0][t] : (d == 1 ? node[1][t] : node[2][t]);
            }
        }

        // derivatives S'(node - q) of axis d for the start and end positions
        __device__ __forceinline__ void slope(int d, T a0[], T a1[]) const
        {
            T const u = sel3(q0, d), v = sel3(q1, d);
#pragma unroll
            for(int t = 0; t < N; ++t)
            {
                a0[t] = SH::dca(T(B0 + t) - u);
                a1[t] = SH::dca(T(B0 + t) - v);
            }
        }
    };

    // One rotated component C of the Esirkepov deposit (cptCurrent1D, Esirkepov.hpp:147-242):
    // loops with fixed extents and the leave flags as predicates, so everything stays in registers.
    template<int SHAPE, typename T>
    __device__ __forceinline__ void esirkepovComponent(
        int const C,
        DTrajectory<SHAPE, T> const& tr,
        T qvdt,
        DiffGrid<T> const& g,
        T* __restrict__ J)
    {
        using TR = DTrajectory<SHAPE, T>;
        constexpr int N = TR::N;
        int const ai = rot(C, 0), aj = rot(C, 1), ak = rot(C, 2);
        if(sel3(tr.q0, ak) == sel3(tr.q1, ak))
            return;
        T const csd = qvdt * cellSize(g, ak);
        T s0i[N], s1i[N], s0j[N], s1j[N], s0k[N], s1k[N];
        uint32_t ndi[N], ndj[N], ndk[N];
        tr.line(ai, s0i, s1i, ndi);
        tr.line(aj, s0j, s1j, ndj);
        tr.line(ak, s0k, s1k, ndk);
        // node counts: N - 1 without the leave node; the running sum along k has one node less
        int const ni = N - 1 + sel3(tr.leave, ai), nj = N - 1 + sel3(tr.leave, aj), nk = N - 2 + sel3(tr.leave, ak);
        T* const Jc = J + size_t(C) * g.nx * g.ny * g.nz;
#pragma unroll
        for(int i = 0; i < N; ++i)
#pragma unroll
            for(int j = 0; j < N; ++j)
            {
                if(i >= ni || j >= nj)
                    continue;
                // -csd (S0i S0j / 3 + S1i S0j / 6 + S0i S1j / 6 + S1i S1j / 3) (Esirkepov.hpp:214-215)
                T const tmp = -csd
                    * (s0i[i] * s0j[j] * third<T>() + (s1i[i] * s0j[j] + s0i[i] * s1j[j]) * sixth<T>() + s1i[i] * s1j[j] * third<T>());
                T run = T(0);
                uint32_t const base = ndi[i] + ndj[j];
#pragma unroll
                for(int k = 0; k < N - 1; ++k)
                    if(k < nk)
                    {
                        run += (s1k[k] - s0k[k]) * tmp;
                        atomicAdd(Jc + base + ndk[k], run);
                    }
            }
    }

    template<int SHAPE, typename T>
    __device__ void esirkepovDeposit(DTrajectory<SHAPE, T> const& tr, T qvdt, DiffGrid<T> const& g, T* __restrict__ J)
    {
#pragma unroll 1
        for(int C = 0; C < 3; ++C)
            esirkepovComponent(C, tr, qvdt, g, J);
    }

    // Adjoint of esirkepovComponent: with J(i, j, k) = tmp(i, j) D_k, D_k = sum_{k' <= k} dS_k',
    // tmp = -csd (S0i S0j / 3 + S1i S0j / 6 + S0i S1j / 6 + S1i S1j / 3), the gradients of the
    // loss with respect to the rotated start/end positions are accumulated in gq0, gq1
    // (real axes) through dS(n - q)/dq = -S'(n - q).
    template<int SHAPE, typename T>
    __device__ __forceinline__ void esirkepovComponentAdjoint(
        int const C,
        DTrajectory<SHAPE, T> const& tr,
        T qvdt,
        DiffGrid<T> const& g,
        T const* __restrict__ lamJ,
        T gq0[3],
        T gq1[3])
    {
        using TR = DTrajectory<SHAPE, T>;
        using SH = DShape<SHAPE, T>;
        constexpr int N = TR::N;
        int const ai = rot(C, 0), aj = rot(C, 1), ak = rot(C, 2);
        if(sel3(tr.q0, ak) == sel3(tr.q1, ak))
            return;
        T const csd = qvdt * cellSize(g, ak);
        T s0i[N], s1i[N], s0j[N], s1j[N], s0k[N], s1k[N];
        uint32_t ndi[N], ndj[N], ndk[N];
        tr.line(ai, s0i, s1i, ndi);
        tr.line(aj, s0j, s1j, ndj);
        tr.line(ak, s0k, s1k, ndk);
        int const ni = N - 1 + sel3(tr.leave, ai), nj = N - 1 + sel3(tr.leave, aj), nk = N - 2 + sel3(tr.leave, ak);
        T const* const Lc = lamJ + size_t(C) * g.nx * g.ny * g.nz;
        T ls0i[N], ls1i[N], ls0j[N], ls1j[N], lds[N];
#pragma unroll
        for(int t = 0; t < N; ++t)
            ls0i[t] = ls1i[t] = ls0j[t] = ls1j[t] = lds[t] = T(0);
#pragma unroll
        for(int i = 0; i < N; ++i)
#pragma unroll
            for(int j = 0; j < N; ++j)
            {
                if(i >= ni || j >= nj)
                    continue;
                T const tmp = -csd
                    * (s0i[i] * s0j[j] * third<T>() + (s1i[i] * s0j[j] + s0i[i] * s1j[j]) * sixth<T>() + s1i[i] * s1j[j] * third<T>());
                uint32_t const base = ndi[i] + ndj[j];
                // ltmp = sum_k lam_k D_k; dL/d(dS_k') = sum_{k >= k'} lam_k tmp
                T ltmp = T(0), D = T(0), lamk[N];
#pragma unroll
                for(int k = 0; k < N - 1; ++k)
                {
                    lamk[k] = T(0);
                    if(k < nk)
                    {
                        D += s1k[k] - s0k[k];
                        T const lam = Lc[base + ndk[k]];
                        ltmp += lam * D;
                        lamk[k] = lam * tmp;
                    }
                }
                T acc = T(0);
#pragma unroll
                for(int k = N - 2; k >= 0; --k)
                {
                    acc += lamk[k];
                    lds[k] += acc;
                }
                T const lt = -csd * ltmp;
                ls0i[i] += lt * (s0j[j] * third<T>() + s1j[j] * sixth<T>());
                ls1i[i] += lt * (s0j[j] * sixth<T>() + s1j[j] * third<T>());
                ls0j[j] += lt * (s0i[i] * third<T>() + s1i[i] * sixth<T>());
                ls1j[j] += lt * (s0i[i] * sixth<T>() + s1i[i] * third<T>());
            }
        T g0i = T(0), g1i = T(0), g0j = T(0), g1j = T(0), g0k = T(0), g1k = T(0);
        T d0[N], d1[N];
        tr.slope(ai, d0, d1);
#pragma unroll
        for(int t = 0; t < N; ++t)
        {
            g0i -= ls0i[t] * d0[t];
            g1i -= ls1i[t] * d1[t];
        }
        tr.slope(aj, d0, d1);
#pragma unroll
        for(int t = 0; t < N; ++t)
        {
            g0j -= ls0j[t] * d0[t];
            g1j -= ls1j[t] * d1[t];
        }
        tr.slope(ak, d0, d1);
#pragma unroll
        for(int t = 0; t < N; ++t)
        {
            // dS_k = S1_k - S0_k
            g1k -= lds[t] * d1[t];
            g0k += lds[t] * d0[t];
        }
        add3(gq0, ai, g0i);
        add3(gq1, ai, g1i);
        add3(gq0, aj, g0j);
        add3(gq1, aj, g1j);
        add3(gq0, ak, g0k);
        add3(gq1, ak, g1k);
    }

    template<int SHAPE, typename T>
    __device__ void esirkepovAdjoint(
        DTrajectory<SHAPE, T> const& tr,
        T qvdt,
        DiffGrid<T> const& g,
        T const* __restrict__ lamJ,
        T gq0[3],
        T gq1[3])
    {
#pragma unroll 1
        for(int C = 0; C < 3; ++C)
            esirkepovComponentAdjoint(C, tr, qvdt, g, lamJ, gq0, gq1);
    }

} // namespace picgb::diff
