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
    template<typename T>
    struct DiffGrid
    {
        int nx, ny, nz;
        T dx, dy, dz, dt, c, eps0;
    };

    __device__ __forceinline__ int wrapIdx(int i, int n)
    {
        i %= n;
        return i < 0 ? i + n : i;
    }

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
                s[0] = a * a * a / T(6);
                s[1] = (T(4) - T(6) * x2 + T(3) * x2 * x) / T(6);
                s[3] = x2 * x / T(6);
                s[2] = T(1) - s[0] - s[1] - s[3];
                ds[0] = T(-0.5) * a * a;
                ds[1] = T(-2) * x + T(1.5) * x2;
                ds[3] = T(0.5) * x2;
                ds[2] = -(ds[0] + ds[1] + ds[3]);
            }
        }

        // ChargeAssignment (the piecewise function of the distance) and its derivative
        __device__ static T ca(T t)
        {
            T const a = t < T(0) ? -t : t;
            if constexpr(SHAPE == 1)
                return a < T(1) ? T(1) - a : T(0);
            else if constexpr(SHAPE == 2)
            {
                if(a < T(0.5))
                    return T(0.75) - t * t;
                T const b = T(1.5) - a;
                return a < T(1.5) ? T(0.5) * b * b : T(0);
            }
            else
            {
                if(a < T(1))
                    return (T(4) - T(6) * t * t + T(3) * a * a * a) / T(6);
                T const b = T(2) - a;
                return a < T(2) ? b * b * b / T(6) : T(0);
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
                if(a < T(0.5))
                    return T(-2) * t;
                return a < T(1.5) ? -(T(1.5) - a) * sg : T(0);
            }
            else
            {
                if(a < T(1))
                    return T(-2) * t + T(1.5) * t * a;
                T const b = T(2) - a;
                return a < T(2) ? T(-0.5) * b * b * sg : T(0);
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
        int first[2][3];
        T w[2][3][S];
        T dw[2][3][S];

        __device__ void compute(int const cell[3], T const pos[3])
        {
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
                    first[a][d] = cell[d] + s + SH::osBegin;
                    SH::base(v - T(s) + T(0.5), w[a][d], dw[a][d]);
                }
        }

        // component COMP (0..2 E_x..E_z, 3..5 B_x..B_z) of field F
        template<int COMP>
        __device__ T value(T const* __restrict__ F, DiffGrid<T> const& g) const
        {
            constexpr int ax = stagger(COMP, 0), ay = stagger(COMP, 1), az = stagger(COMP, 2);
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
                        rx += w[ax][0][x]
                            * F[cellIndex(g, first[ax][0] + x, first[ay][1] + y, first[az][2] + z)];
                    ry += w[ay][1][y] * rx;
                }
                rz += w[az][2][z] * ry;
            }
            return rz;
        }

        // adjoint of value(): lam * weights scattered into lamF, and the position gradient
        template<int COMP>
        __device__ void adjoint(T const* __restrict__ F, T* __restrict__ lamF, DiffGrid<T> const& g, T lam, T gpos[3])
            const
        {
            constexpr int ax = stagger(COMP, 0), ay = stagger(COMP, 1), az = stagger(COMP, 2);
            if(lam == T(0))
                return;
#pragma unroll
            for(int z = 0; z < S; ++z)
#pragma unroll
                for(int y = 0; y < S; ++y)
#pragma unroll
                    for(int x = 0; x < S; ++x)
                    {
                        size_t const i = cellIndex(g, first[ax][0] + x, first[ay][1] + y, first[az][2] + z);
                        T const wx = w[ax][0][x], wy = w[ay][1][y], wz = w[az][2][z];
                        atomicAdd(lamF + i, lam * wx * wy * wz);
                        T const f = F[i] * lam;
                        gpos[0] += f * dw[ax][0][x] * wy * wz;
                        gpos[1] += f * wx * dw[ay][1][y] * wz;
                        gpos[2] += f * wx * wy * dw[az][2][z];
                    }
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

    // Esirkepov trajectory in the virtual grid: start q0 and end q1 relative to the
    // origin cell (new cell + shift), and the per-axis leave flags.
    template<int SHAPE, typename T>
    struct DTrajectory
    {
        T q0[3], q1[3];
        int origin[3];
        int leave[3];

        __device__ void compute(int const newCell[3], T const pos[3], T const dp[3])
        {
            for(int d = 0; d < 3; ++d)
            {
                T const p0 = pos[d] - dp[d], p1 = pos[d];
                int iS, iE;
                if constexpr(DShape<SHAPE, T>::even)
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
                origin[d] = newCell[d] + gs;
                q0[d] = p0 - T(gs);
                q1[d] = p1 - T(gs);
            }
        }
    };

    // Rotations of the three current components: rotated axis r of component C is real axis rot(C, r)
    // (J_x: i->y, j->z, k->x; J_y: i->z, j->x, k->y; J_z: i->x, j->y, k->z).
    __host__ __device__ constexpr int rot(int C, int r)
    {
        return C == 0 ? (r == 0 ? 1 : (r == 1 ? 2 : 0)) : (C == 1 ? (r == 0 ? 2 : (r == 1 ? 0 : 1)) : r);
    }

    // Esirkepov deposit of one particle (all three components) into J with atomics.
    template<int SHAPE, typename T>
    __device__ void esirkepovDeposit(
        DTrajectory<SHAPE, T> const& tr,
        T qvdt, // charge * weighting / (V dt)
        DiffGrid<T> const& g,
        T* __restrict__ J)
    {
        using SH = DShape<SHAPE, T>;
        constexpr int B0 = SH::caBegin, E0 = SH::caEnd;
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        for(int C = 0; C < 3; ++C)
        {
            int const ai = rot(C, 0), aj = rot(C, 1), ak = rot(C, 2);
            if(tr.q0[ak] == tr.q1[ak])
                continue;
            T const csd = qvdt * cellSize(g, ak);
            int const ei = E0 + tr.leave[ai], ej = E0 + tr.leave[aj], ek = E0 + tr.leave[ak] - 1;
            for(int i = B0; i < ei; ++i)
            {
                T const s0i = SH::ca(T(i) - tr.q0[ai]), s1i = SH::ca(T(i) - tr.q1[ai]);
                for(int j = B0; j < ej; ++j)
                {
                    T const s0j = SH::ca(T(j) - tr.q0[aj]), s1j = SH::ca(T(j) - tr.q1[aj]);
                    // -csd (S0i S0j / 3 + S1i S0j / 6 + S0i S1j / 6 + S1i S1j / 3) (Esirkepov.hpp:214-215)
                    T const tmp = -csd
                        * (s0i * s0j / T(3) + (s1i * s0j + s0i * s1j) / T(6) + s1i * s1j / T(3));
                    T run = T(0);
                    for(int k = B0; k < ek; ++k)
                    {
                        run += (SH::ca(T(k) - tr.q1[ak]) - SH::ca(T(k) - tr.q0[ak])) * tmp;
                        int n[3];
                        n[ai] = tr.origin[ai] + i;
                        n[aj] = tr.origin[aj] + j;
                        n[ak] = tr.origin[ak] + k;
                        atomicAdd(J + C * nc + cellIndex(g, n[0], n[1], n[2]), run);
                    }
                }
            }
        }
    }

    // Adjoint of esirkepovDeposit: given lamJ, the gradients with respect to q0 and q1 (real axes).
    template<int SHAPE, typename T>
    __device__ void esirkepovAdjoint(
        DTrajectory<SHAPE, T> const& tr,
        T qvdt,
        DiffGrid<T> const& g,
        T const* __restrict__ lamJ,
        T gq0[3],
        T gq1[3])
    {
        using SH = DShape<SHAPE, T>;
        constexpr int B0 = SH::caBegin, E0 = SH::caEnd;
        constexpr int N = E0 - B0 + 1; // nodes per axis with the leave node
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        for(int C = 0; C < 3; ++C)
        {
            int const ai = rot(C, 0), aj = rot(C, 1), ak = rot(C, 2);
            if(tr.q0[ak] == tr.q1[ak])
                continue;
            T const csd = qvdt * cellSize(g, ak);
            int const ei = E0 + tr.leave[ai], ej = E0 + tr.leave[aj], ek = E0 + tr.leave[ak] - 1;
            T s0k[N], s1k[N], lds[N];
            for(int k = B0; k < ek; ++k)
            {
                s0k[k - B0] = SH::ca(T(k) - tr.q0[ak]);
                s1k[k - B0] = SH::ca(T(k) - tr.q1[ak]);
                lds[k - B0] = T(0);
            }
            for(int i = B0; i < ei; ++i)
            {
                T const s0i = SH::ca(T(i) - tr.q0[ai]), s1i = SH::ca(T(i) - tr.q1[ai]);
                T ls0i = T(0), ls1i = T(0);
                for(int j = B0; j < ej; ++j)
                {
                    T const s0j = SH::ca(T(j) - tr.q0[aj]), s1j = SH::ca(T(j) - tr.q1[aj]);
                    T const tmp = -csd
                        * (s0i * s0j / T(3) + (s1i * s0j + s0i * s1j) / T(6) + s1i * s1j / T(3));
                    // J(k) = tmp * D_k with D_k = sum_{k' <= k} ds_k'
                    T ltmp = T(0), D = T(0);
                    T lamk[N];
                    for(int k = B0; k < ek; ++k)
                    {
                        D += s1k[k - B0] - s0k[k - B0];
                        int n[3];
                        n[ai] = tr.origin[ai] + i;
                        n[aj] = tr.origin[aj] + j;
                        n[ak] = tr.origin[ak] + k;
                        T const lam = lamJ[C * nc + cellIndex(g, n[0], n[1], n[2])];
                        ltmp += lam * D;
                        lamk[k - B0] = lam * tmp;
                    }
                    // dL/d(ds_k') = sum_{k >= k'} lam_k tmp
                    T acc = T(0);
                    for(int k = ek - 1; k >= B0; --k)
                    {
                        acc += lamk[k - B0];
                        lds[k - B0] += acc;
                    }
                    T const lt = -csd * ltmp;
                    ls0i += lt * (s0j / T(3) + s1j / T(6));
                    ls1i += lt * (s0j / T(6) + s1j / T(3));
                    T const ls0j = lt * (s0i / T(3) + s1i / T(6));
                    T const ls1j = lt * (s0i / T(6) + s1i / T(3));
                    // S(j - q): d/dq = -ca'(j - q)
                    gq0[aj] -= ls0j * SH::dca(T(j) - tr.q0[aj]);
                    gq1[aj] -= ls1j * SH::dca(T(j) - tr.q1[aj]);
                }
                gq0[ai] -= ls0i * SH::dca(T(i) - tr.q0[ai]);
                gq1[ai] -= ls1i * SH::dca(T(i) - tr.q1[ai]);
            }
            for(int k = B0; k < ek; ++k)
            {
                // ds_k = S1_k - S0_k
                gq1[ak] -= lds[k - B0] * SH::dca(T(k) - tr.q1[ak]);
                gq0[ak] += lds[k - B0] * SH::dca(T(k) - tr.q0[ak]);
            }
        }
    }
} // namespace picgb::diff
