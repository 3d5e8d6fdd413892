// Device-side math of the PIC hot path: assignment shapes, form-factor gather,
// Boris push, moveParticle and the Esirkepov deposit.
//
// Operations that decide particle positions (shapes, gather, push, move) use
// the explicit round-to-nearest intrinsics (__fmul_rn, __fadd_rn, ...) so the
// compiler cannot contract them into FMAs: the result is bit-identical to a
// scalar IEEE evaluation in the reference's association order, which is what
// makes the per-cell particle counts after a step bit-exact.
#pragma once

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
        // deposit node range relative to a cell in [-1, S] (particle may have
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
    };

    __device__ __forceinline__ int wrapi(int i, int n)
    {
        // valid for i in [-n, 2n)
        return i < 0 ? i + n : (i >= n ? i - n : i);
    }

    // ------------------------------------------------------------ gather
    // FieldToParticleInterpolation (algorithms/FieldToParticleInterpolation.hpp:97-124),
    // ShiftCoordinateSystem (ShiftCoordinateSystem.hpp:54-79), AssignedTrilinearInterpolation
    // (AssignedTrilinearInterpolation.hpp:54-86), reading a shared-memory tile whose
    // origin is the supercell origin minus Shape::gLo in every direction.
    template<typename SH, int TX, int TY>
    __device__ __forceinline__ float gatherComponent(
        float const* __restrict__ tile,
        int lx,
        int ly,
        int lz,
        float px,
        float py,
        float pz,
        float fx,
        float fy,
        float fz)
    {
        constexpr int S = SH::supp;
        float const pin[3] = {px, py, pz};
        float const fp[3] = {fx, fy, fz};
        int shift[3];
        float p[3];
#pragma unroll
        for(int d = 0; d < 3; ++d)
        {
            float v = fs(fs(pin[d], fp[d]), 0.5f);
            if constexpr(SH::even)
                shift[d] = v >= -0.5f ? 0 : -1;
            else
                shift[d] = v >= 0.0f ? 1 : 0;
            p[d] = fa(fs(v, float(shift[d])), 0.5f);
        }
        float sx[S], sy[S], sz[S];
        SH::base(p[0], sx);
        SH::base(p[1], sy);
        SH::base(p[2], sz);
        int const bx = lx + SH::gLo + shift[0] + SH::osBegin;
        int const by = ly + SH::gLo + shift[1] + SH::osBegin;
        int const bz = lz + SH::gLo + shift[2] + SH::osBegin;
        float rz = 0.0f;
#pragma unroll
        for(int z = 0; z < S; ++z)
        {
            float ry = 0.0f;
#pragma unroll
            for(int y = 0; y < S; ++y)
            {
                float rx = 0.0f;
                float const* row = tile + (bx + TX * ((by + y) + TY * (bz + z)));
#pragma unroll
                for(int x = 0; x < S; ++x)
                    rx = fa(rx, fm(row[x], sx[x]));
                ry = fa(ry, fm(rx, sy[y]));
            }
            rz = fa(rz, fm(ry, sz[z]));
        }
        return rz;
    }

    // ------------------------------------------------------------ push
    __device__ __forceinline__ float l2n2(float a, float b, float c) { return fa(fa(fm(a, a), fm(b, b)), fm(c, c)); }

    // Velocity (algorithms/Velocity.hpp:31-37) with a correctly rounded 1/sqrt
    __device__ __forceinline__ void velocity(float const mom[3], float mass, float rc2, float vel[3])
    {
        float const m0_2 = fm(mass, mass);
        float const fMom2 = l2n2(mom[0], mom[1], mom[2]);
        float const t = fdv(1.0f, fsq(fa(m0_2, fm(fMom2, rc2))));
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
        float const m2_c2_reci = fdv(1.0f, fm(fm(mass, mass), c2));
        float const gamma = fsq(fa(1.0f, fm(l2n2(mm[0], mm[1], mm[2]), m2_c2_reci)));
        float const gamma_reci = fdv(1.0f, gamma);
        float const hqm = fm(0.5f, QoM);
        float t[3];
#pragma unroll
        for(int d = 0; d < 3; ++d)
            t[d] = fm(fm(fm(hqm, B[d]), gamma_reci), dt);
        float const sf = fdv(1.0f, fa(1.0f, l2n2(t[0], t[1], t[2])));
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

    // ------------------------------------------------------------ Esirkepov
    // Deposits into a shared-memory J tile (3 arrays of TX*TY*TZ floats) whose
    // origin is the supercell origin minus Shape::jLo per axis.  cellRel = new
    // cell of the particle relative to the supercell origin (in [-1, S]).
    // Esirkepov::operator() (fields/currentDeposition/Esirkepov/Esirkepov.hpp:62-134),
    // cptCurrent1D (:147-242), relayPoint (relayPoint.hpp:48-64).
    template<typename SH, int TX, int TY>
    struct Esirkepov
    {
        static constexpr int S = SH::supp;
        static constexpr int begin = SH::caBegin;
        static constexpr int end = SH::caEnd;

        // one rotated 1D current: axes (i,j,k) of the rotated frame map to the
        // tile strides st[0..2]; the running sum runs along k.
        __device__ static void cpt1D(
            float* __restrict__ Jc,
            int const stat[3],
            float const q0[3],
            float const q1[3],
            int base,
            int const st[3],
            float csd)
        {
            if(q0[2] == q1[2])
                return;
            float sj0[S + 1], sj1[S + 1], sk0[S + 1], sk1[S + 1];
            SH::caArray(q0[1], !(stat[1] & 2), sj0);
            SH::caArray(q1[1], !(stat[1] & 4), sj1);
            SH::caArray(q0[2], !(stat[2] & 2), sk0);
            SH::caArray(q1[2], !(stat[2] & 4), sk1);
            float dsk[S];
#pragma unroll
            for(int k = 0; k < S; ++k)
                dsk[k] = fs(sk1[k], sk0[k]);
            int const leaveI = stat[0] & 1, leaveJ = stat[1] & 1, leaveK = stat[2] & 1;
            float const ncsd = -csd;
#pragma unroll
            for(int i = begin; i < end + 1; ++i)
                if(i < end + leaveI)
                {
                    float const s0i = SH::ca(fs(float(i), q0[0]));
                    float const dsi = fs(SH::ca(fs(float(i), q1[0])), s0i);
#pragma unroll
                    for(int j = begin; j < end + 1; ++j)
                        if(j < end + leaveJ)
                        {
                            float const s0j = sj0[j - begin];
                            float const dsj = fs(sj1[j - begin], s0j);
                            float const tmp = fm(
                                ncsd,
                                fa(fa(fm(s0i, s0j), fm(0.5f, fa(fm(dsi, s0j), fm(s0i, dsj)))),
                                   fm(fm(1.0f / 3.0f, dsj), dsi)));
                            float acc = 0.0f;
                            int const ij = base + i * st[0] + j * st[1];
#pragma unroll
                            for(int k = begin; k < end; ++k)
                                if(k < end + leaveK - 1)
                                {
                                    acc = fa(acc, fm(dsk[k - begin], tmp));
                                    atomicAdd(Jc + ij + k * st[2], acc);
                                }
                        }
                }
        }

        // pos = in-cell position after the move, vel from the new momentum.
        // Returns false (and deposits nothing) when the trajectory would leave
        // the tile, which valid inputs (|v| dt < cell size) never do.
        __device__ static bool deposit(
            float* __restrict__ Jx,
            float* __restrict__ Jy,
            float* __restrict__ Jz,
            int const cellRel[3],
            float const pos[3],
            float const vel[3],
            float charge,
            GridParams const& g,
            float invVdt)
        {
            float const cs[3] = {g.dx, g.dy, g.dz};
            float p0[3], p1[3];
            int gs[3], stat[3];
#pragma unroll
            for(int d = 0; d < 3; ++d)
            {
                float const dp = fdv(fm(vel[d], g.dt), cs[d]);
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
#pragma unroll
            for(int d = 0; d < 3; ++d)
                if(gs[d] < -1 || gs[d] > gsHi || cellRel[d] < -1)
                    return false;
            constexpr int TYX = TX * TY;
            int const base =(cellRel[0] + gs[0] + SH::jLo) + TX * (cellRel[1] + gs[1] + SH::jLo)
                + TYX * (cellRel[2] + gs[2] + SH::jLo);
            // currentSurfaceDensity = charge * (1/(V*dt)) * cellEdgeLength (Esirkepov.hpp:188-190)
            {
                // J_x: rotation (1,2,0): i->y, j->z, k->x
                int const st[3] = {stat[1], stat[2], stat[0]};
                float const a0[3] = {p0[1], p0[2], p0[0]}, a1[3] = {p1[1], p1[2], p1[0]};
                int const stride[3] = {TX, TYX, 1};
                cpt1D(Jx, st, a0, a1, base, stride, fm(fm(charge, invVdt), g.dx));
            }
            {
                // J_y: rotation (2,0,1): i->z, j->x, k->y
                int const st[3] = {stat[2], stat[0], stat[1]};
                float const a0[3] = {p0[2], p0[0], p0[1]}, a1[3] = {p1[2], p1[0], p1[1]};
                int const stride[3] = {TYX, 1, TX};
                cpt1D(Jy, st, a0, a1, base, stride, fm(fm(charge, invVdt), g.dy));
            }
            {
                int const stride[3] = {1, TX, TYX};
                cpt1D(Jz, stat, p0, p1, base, stride, fm(fm(charge, invVdt), g.dz));
            }
            return true;
        }
    };
} // namespace picgb
