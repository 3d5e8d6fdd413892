// CPU oracle for the PIC-cycle hot path — TEST INFRASTRUCTURE ONLY.
//
// This header restates, in plain C++, the reference algorithms of PIConGPU's
// electromagnetic PIC step so that the CUDA path can be checked against it on
// identical inputs.  It is the checker, never the product: only tests/, the
// smoke check and bench.py's CPU-baseline leg may load it.
//
// Every function cites the reference file:line it follows (paths relative to
// the PIConGPU source tree).  Floating-point operations are written in the same
// association order as the reference so that the CUDA kernels, which use the
// same order without FMA contraction in the push/gather/Yee paths, agree
// bit-for-bit there.  Build with -ffp-contract=off (see oracle/Makefile).
//
// Parity pins: shape partition of unity (share/picongpu/unit/shape.cpp:176-207),
// moveParticle known answers (share/picongpu/unit/MoveParticle.cpp:98-258),
// single-particle Esirkepov vs. the reference's numpy implementation
// (share/picongpu/tests/CurrentDeposition/lib/python/test/CurrentDeposition/
// grid_class.py:97-199, fixtures in tests/golden/), Boris gyration invariants
// (share/picongpu/tests/Pusher/README.rst).  The reference itself cannot be
// compiled on this machine (Boost/MPI absent), so there is no oracle/_ref.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#    include <omp.h>
#endif

namespace orc
{
    // ---------------------------------------------------------------- grid
    struct Grid
    {
        int nx, ny, nz; // cells (periodic box)
        int sx, sy, sz; // supercell size in cells
        float dx, dy, dz; // cell edge lengths
        float dt; // time step
        float c; // speed of light
        float eps0; // vacuum permittivity
        int open = 0; // bit a: axis a is open (no wrap; fields zero beyond the box, particles absorbed)

        static constexpr size_t kOutside = ~size_t(0); // idx() of a point beyond an open face

        int nscx() const { return nx / sx; }
        int nscy() const { return ny / sy; }
        int nscz() const { return nz / sz; }
        int nsc() const { return nscx() * nscy() * nscz(); }
        int scVolume() const { return sx * sy * sz; }
        size_t ncells() const { return size_t(nx) * ny * nz; }

        static inline int wrap(int i, int n)
        {
            i %= n;
            return i < 0 ? i + n : i;
        }
        size_t idx(int x, int y, int z) const
        {
            if(((open & 1) && (x < 0 || x >= nx)) || ((open & 2) && (y < 0 || y >= ny))
               || ((open & 4) && (z < 0 || z >= nz)))
                return kOutside;
            return size_t(wrap(x, nx)) + size_t(nx) * (size_t(wrap(y, ny)) + size_t(ny) * size_t(wrap(z, nz)));
        }
        // component value at a flat index, zero beyond an open face
        template<typename T>
        static T at(T const* f, size_t i)
        {
            return i == kOutside ? T(0) : f[i];
        }
    };

    // Three-component field in SoA layout, x fastest, no guard cells: the
    // periodic neighbour is reached by index wrap (Grid::idx).
    template<typename T>
    struct Field3
    {
        T* c[3];
    };

    // Particle exchange format (one species): SoA arrays of n particles.
    // pos = in-cell position in [0,1), mom = macro-weighted momentum
    // (param/speciesAttributes.param:71-80), w = weighting, sc = supercell
    // linear index, lcell = cell index inside the supercell
    // (pmacc/particles/memory/frames/Frame.hpp:58-85 attribute set).
    template<typename T>
    struct Particles
    {
        size_t n;
        T* pos[3];
        T* mom[3];
        T* w;
        int32_t* sc;
        uint16_t* lcell;
    };

    enum Shape
    {
        NGP = 0,
        CIC = 1,
        TSC = 2,
        PQS = 3,
        PCS = 4
    };
    enum Pusher
    {
        BORIS = 0,
        FREE = 1,
        HIGUERA_CARY = 3,
        VAY = 4,
        PHOTON = 5
    };

    struct SpeciesParam
    {
        float charge; // charge of one real particle (macro charge = charge * w)
        float mass; // mass of one real particle (macro mass = mass * w)
        int shape; // Shape
        int pusher; // Pusher
        int current; // 1 = Esirkepov deposit, 2 = EmZ, 0 = no current
    };
    constexpr int EMZ_CURRENT = 2;

    // ---------------------------------------------------------------- shapes
    // particles/shapes/{NGP,CIC,TSC,PQS,PCS}.hpp.  support = order + 1.
    inline int support(int shape) { return shape + 1; }

    template<typename T>
    struct ShapeFn
    {
        // ---- TSC helpers (particles/shapes/TSC.hpp:46-63)
        static T tsc1(T x) { T sq = x * x; return T(0.75) - sq; }
        static T tsc2(T x) { T tmp = T(1.5) - x; T sq = tmp * tmp; return T(0.5) * sq; }
        // ---- PQS helpers (particles/shapes/PQS.hpp:45-67)
        static T pqs1(T x)
        {
            T sq = x * x;
            T tr = sq * x;
            return (T(1.0) / T(6.0)) * (T(4.0) - T(6.0) * sq + T(3.0) * tr);
        }
        static T pqs2(T x)
        {
            T tmp = T(2.0) - x;
            T tr = tmp * tmp * tmp;
            return (T(1.0) / T(6.0)) * tr;
        }
        // ---- PCS helpers (particles/shapes/PCS.hpp:47-75)
        static T pcs1(T x)
        {
            T sq = x * x;
            return T(115.) / T(192.) + sq * (T(-5.) / T(8.) + T(1.0) / T(4.0) * sq);
        }
        static T pcs2(T x)
        {
            return T(1.) / T(96.) * (T(55.) + T(4.) * x * (T(5.) - T(2.) * x * (T(15.) + T(2.) * x * (T(-5.) + x))));
        }
        static T pcs3(T x)
        {
            T tmp = T(5.) - T(2.) * x;
            T sq = tmp * tmp;
            T bq = sq * sq;
            return T(1.) / T(384.) * bq;
        }

        // detail::<Shape>::shapeArray<size>(x): values on the support grid points.
        // CIC.hpp:42-53, TSC.hpp:65-76, PQS.hpp:69-82, NGP.hpp:42-50, PCS.hpp:85-101
        static void baseArray(int shape, T x, T* s)
        {
            switch(shape)
            {
            case NGP:
                s[0] = T(1.0);
                break;
            case CIC:
                s[0] = T(1.0) - x;
                s[1] = x;
                break;
            case TSC:
                s[0] = tsc2(std::abs(T(-1.) - x));
                s[1] = tsc1(std::abs(x));
                s[2] = T(1.0) - (s[0] + s[1]);
                break;
            case PQS:
                s[0] = pqs2(std::abs(T(-1.) - x));
                s[1] = pqs1(x);
                s[3] = pqs2(T(2.) - x);
                s[2] = T(1.0) - (s[0] + s[1] + s[3]);
                break;
            case PCS:
                s[0] = pcs3(std::abs(T(-2.) - x));
                s[1] = pcs2(std::abs(T(-1.) - x));
                s[2] = pcs1(std::abs(x));
                s[4] = pcs3(T(2.) - x);
                s[3] = T(1.0) - (s[0] + s[1] + s[2] + s[4]);
                break;
            }
        }

        // <Shape>::ChargeAssignment::begin (CIC.hpp:72, TSC.hpp:90, PQS.hpp:90, NGP.hpp:65, PCS.hpp:119)
        static int caBegin(int shape)
        {
            static const int b[5] = {0, 0, -1, -1, -2};
            return b[shape];
        }
        // <Shape>::ChargeAssignmentOnSupport::begin (shape files, OnSupport struct)
        static int osBegin(int shape)
        {
            static const int b[5] = {0, 0, -1, -1, -2};
            return b[shape];
        }

        // ChargeAssignment::shapeArray(pos, isOutOfRange): support+1 values,
        // shifted by one when the particle sits one cell above the assignment cell.
        // CIC.hpp:95-109, TSC.hpp:116-132, PQS.hpp:119-137, NGP.hpp:83-95, PCS.hpp:154-170
        static void caArray(int shape, T pos, bool isOutOfRange, T* s)
        {
            int supp = support(shape);
            T x = isOutOfRange ? pos - T(1.0) : pos;
            T v[6] = {0, 0, 0, 0, 0, 0};
            baseArray(shape, x, v);
            s[supp] = isOutOfRange ? v[supp - 1] : T(0.0);
            for(int k = supp - 1; k >= 1; --k)
                s[k] = isOutOfRange ? v[k - 1] : v[k];
            s[0] = isOutOfRange ? T(0.0) : v[0];
        }

        // ChargeAssignment::operator()(x): the piecewise assignment function.
        // CIC.hpp:78-93, TSC.hpp:96-114, PQS.hpp:96-117, NGP.hpp:71-81, PCS.hpp:125-140
        static T ca(int shape, T x)
        {
            T ax = std::abs(x);
            switch(shape)
            {
            case NGP:
                return (T(-0.5) <= x && x < T(0.5)) ? T(1.0) : T(0.0);
            case CIC:
            {
                T on = T(1.0) - ax;
                return ax < T(1.0) ? on : T(0.0);
            }
            case TSC:
            {
                T r1 = tsc1(ax), r2 = tsc2(ax);
                T res = T(0.0);
                if(ax < T(0.5))
                    res = r1;
                else if(ax < T(1.5))
                    res = r2;
                return res;
            }
            case PQS:
            {
                T r1 = pqs1(ax), r2 = pqs2(ax);
                T res = T(0.0);
                if(ax < T(1.0))
                    res = r1;
                else if(ax < T(2.0))
                    res = r2;
                return res;
            }
            case PCS:
            {
                T on = os(PCS, ax);
                return ax < T(2.5) ? on : T(0.0);
            }
            }
            return T(0);
        }

        // ChargeAssignmentOnSupport::operator()(x) (shape files, OnSupport struct)
        static T os(int shape, T x)
        {
            T ax = std::abs(x);
            switch(shape)
            {
            case NGP:
                return T(1.0);
            case CIC:
                return T(1.0) - ax;
            case TSC:
            {
                T r1 = tsc1(ax), r2 = tsc2(ax);
                return ax < T(0.5) ? r1 : r2;
            }
            case PQS:
            {
                T r1 = pqs1(ax), r2 = pqs2(ax);
                return ax < T(1.0) ? r1 : r2;
            }
            case PCS:
            {
                T r1 = pcs1(ax), r2 = pcs2(ax), r3 = pcs3(ax);
                T res = r3;
                if(ax < T(0.5))
                    res = r1;
                else if(ax < T(1.5))
                    res = r2;
                return res;
            }
            }
            return T(0);
        }
    };

    // ---------------------------------------------------------------- Yee solver
    // fields/differentiation/ForwardDerivative.hpp:45-63 (upper - cur)/d,
    // BackwardDerivative.hpp:45-63 (cur - lower)/d, Curl.hpp:84-89.
    template<typename T>
    inline void curlForward(Grid const& g, Field3<T> const& F, int x, int y, int z, T out[3])
    {
        size_t i0 = g.idx(x, y, z), ix = g.idx(x + 1, y, z), iy = g.idx(x, y + 1, z), iz = g.idx(x, y, z + 1);
        // dF/dx, dF/dy, dF/dz as full vectors (only the needed components are used)
        T dFdx_y = (Grid::at(F.c[1], ix) - F.c[1][i0]) / T(g.dx);
        T dFdx_z = (Grid::at(F.c[2], ix) - F.c[2][i0]) / T(g.dx);
        T dFdy_x = (Grid::at(F.c[0], iy) - F.c[0][i0]) / T(g.dy);
        T dFdy_z = (Grid::at(F.c[2], iy) - F.c[2][i0]) / T(g.dy);
        T dFdz_x = (Grid::at(F.c[0], iz) - F.c[0][i0]) / T(g.dz);
        T dFdz_y = (Grid::at(F.c[1], iz) - F.c[1][i0]) / T(g.dz);
        out[0] = dFdy_z - dFdz_y;
        out[1] = dFdz_x - dFdx_z;
        out[2] = dFdx_y - dFdy_x;
    }

    template<typename T>
    inline void curlBackward(Grid const& g, Field3<T> const& F, int x, int y, int z, T out[3])
    {
        size_t i0 = g.idx(x, y, z), ix = g.idx(x - 1, y, z), iy = g.idx(x, y - 1, z), iz = g.idx(x, y, z - 1);
        T dFdx_y = (F.c[1][i0] - Grid::at(F.c[1], ix)) / T(g.dx);
        T dFdx_z = (F.c[2][i0] - Grid::at(F.c[2], ix)) / T(g.dx);
        T dFdy_x = (F.c[0][i0] - Grid::at(F.c[0], iy)) / T(g.dy);
        T dFdy_z = (F.c[2][i0] - Grid::at(F.c[2], iy)) / T(g.dy);
        T dFdz_x = (F.c[0][i0] - Grid::at(F.c[0], iz)) / T(g.dz);
        T dFdz_y = (F.c[1][i0] - Grid::at(F.c[1], iz)) / T(g.dz);
        out[0] = dFdy_z - dFdz_y;
        out[1] = dFdz_x - dFdx_z;
        out[2] = dFdx_y - dFdy_x;
    }

    // B -= curl(E) * 0.5 * dt  (MaxwellSolver/FDTD/FDTDBase.kernel:92-121, UpdateBHalfFunctor).
    // The source field is read-only during the update (it is cached per supercell
    // in the reference, FDTDBase.kernel:170-176), so B never aliases E.
    template<typename T>
    void yeeBHalf(Grid const& g, Field3<T> const& E, Field3<T>& B)
    {
#pragma omp parallel for schedule(static)
        for(int z = 0; z < g.nz; ++z)
            for(int y = 0; y < g.ny; ++y)
                for(int x = 0; x < g.nx; ++x)
                {
                    T curl[3];
                    curlForward(g, E, x, y, z, curl);
                    size_t i = g.idx(x, y, z);
                    for(int d = 0; d < 3; ++d)
                        B.c[d][i] = B.c[d][i] - curl[d] * T(0.5) * T(g.dt);
                }
    }

    // E += curl(B) * c^2 * dt  (FDTDBase.kernel:51-81, UpdateEFunctor)
    template<typename T>
    void yeeE(Grid const& g, Field3<T> const& B, Field3<T>& E)
    {
        T const c2 = T(g.c) * T(g.c);
#pragma omp parallel for schedule(static)
        for(int z = 0; z < g.nz; ++z)
            for(int y = 0; y < g.ny; ++y)
                for(int x = 0; x < g.nx; ++x)
                {
                    T curl[3];
                    curlBackward(g, B, x, y, z, curl);
                    size_t i = g.idx(x, y, z);
                    for(int d = 0; d < 3; ++d)
                        E.c[d][i] = E.c[d][i] + curl[d] * c2 * T(g.dt);
                }
    }

    // E(idx) += coeff * J(idx), coeff = -(1/eps0) * dt
    // (currentInterpolation/None.hpp:60-65, coefficient MaxwellSolver/FDTD/FDTD.hpp:84)
    template<typename T>
    void addCurrent(Grid const& g, Field3<T> const& J, Field3<T>& E)
    {
        T const coeff = -(T(1.0) / T(g.eps0)) * T(g.dt);
        size_t n = g.ncells();
#pragma omp parallel for schedule(static)
        for(size_t i = 0; i < n; ++i)
            for(int d = 0; d < 3; ++d)
                E.c[d][i] = E.c[d][i] + coeff * J.c[d][i];
    }

    // ---------------------------------------------------------------- gather
    // Yee staggering of the components (fields/YeeCell.hpp:70-131).
    static const float kPosE[3][3] = {{0.5f, 0.f, 0.f}, {0.f, 0.5f, 0.f}, {0.f, 0.f, 0.5f}};
    static const float kPosB[3][3] = {{0.f, 0.5f, 0.5f}, {0.5f, 0.f, 0.5f}, {0.5f, 0.5f, 0.f}};

    // FieldToParticleInterpolation::operator() (algorithms/FieldToParticleInterpolation.hpp:97-124) with
    // ShiftCoordinateSystem (algorithms/ShiftCoordinateSystem.hpp:37-79) and
    // AssignedTrilinearInterpolation::interpolate (algorithms/AssignedTrilinearInterpolation.hpp:54-86).
    // cell = global cell of the particle; pos = in-cell position.
    template<typename T>
    void gather(
        Grid const& g,
        int shape,
        Field3<T> const& F,
        float const fieldPos[3][3],
        int const cell[3],
        T const pos[3],
        T out[3])
    {
        int const supp = support(shape);
        bool const isEven = (supp % 2) == 0;
        int const begin = -supp / 2 + (supp + 1) % 2;
        int const end = begin + supp - 1;
        for(int comp = 0; comp < 3; ++comp)
        {
            int shift[3];
            T p[3];
            for(int d = 0; d < 3; ++d)
            {
                T const v_pos = pos[d] - T(fieldPos[comp][d]) - T(0.5);
                if(isEven)
                    shift[d] = v_pos >= T(-0.5) ? 0 : -1;
                else
                    shift[d] = v_pos >= T(0.0) ? 1 : 0;
                p[d] = v_pos - T(shift[d]) + T(0.5);
            }
            T sx[6] = {}, sy[6] = {}, sz[6] = {};
            ShapeFn<T>::baseArray(shape, p[0], sx);
            ShapeFn<T>::baseArray(shape, p[1], sy);
            ShapeFn<T>::baseArray(shape, p[2], sz);
            // `result += value * weight` evaluated as one fused multiply-add, the
            // contraction the reference's CUDA build (nvcc, -fmad=true) applies here
            T result_z = T(0.0);
            for(int z = begin; z <= end; ++z)
            {
                T result_y = T(0.0);
                for(int y = begin; y <= end; ++y)
                {
                    T result_x = T(0.0);
                    for(int x = begin; x <= end; ++x)
                    {
                        size_t i = g.idx(cell[0] + shift[0] + x, cell[1] + shift[1] + y, cell[2] + shift[2] + z);
                        result_x = std::fma(Grid::at(F.c[comp], i), sx[x - begin], result_x);
                    }
                    result_y = std::fma(result_x, sy[y - begin], result_y);
                }
                result_z = std::fma(result_y, sz[z - begin], result_z);
            }
            out[comp] = result_z;
        }
    }

    // ---------------------------------------------------------------- push
    template<typename T>
    inline T l2norm2(T const v[3])
    {
        T r = v[0] * v[0];
        r += v[1] * v[1];
        r += v[2] * v[2];
        return r;
    }

    // Gamma (algorithms/Gamma.hpp:30-37)
    template<typename T>
    inline T gammaOf(T const mom[3], T mass, T c)
    {
        T const fMom2 = l2norm2(mom);
        T const c2 = c * c;
        T const m2_c2_reci = T(1.0) / (mass * mass * c2);
        return std::sqrt(T(1.0) + fMom2 * m2_c2_reci);
    }

    // Velocity (algorithms/Velocity.hpp:31-37).  The reference calls math::rsqrt;
    // the correctly rounded 1/sqrt is used here and in the CUDA path so both agree
    // bit for bit.
    template<typename T>
    inline void velocityOf(T const mom[3], T mass, T c, T vel[3])
    {
        T const rc2 = T(1.0) / (c * c); // sim.pic.getMue0Eps0() (unitless/simulation.unitless:98-101)
        T const m0_2 = mass * mass;
        T const fMom2 = l2norm2(mom);
        T const t = T(1.0) / std::sqrt(m0_2 + fMom2 * rc2);
        for(int d = 0; d < 3; ++d)
            vel[d] = t * mom[d];
    }

    // Boris push (particles/pusher/particlePusherBoris.hpp:42-90)
    template<typename T>
    inline void borisPush(Grid const& g, T charge, T mass, T const E[3], T const B[3], T mom[3], T pos[3])
    {
        T const QoM = charge / mass;
        T const deltaT = T(g.dt);
        T mom_minus[3];
        for(int d = 0; d < 3; ++d)
            mom_minus[d] = mom[d] + T(0.5) * charge * E[d] * deltaT;
        T const gamma_reci = T(1.0) / gammaOf(mom_minus, mass, T(g.c));
        T t[3];
        for(int d = 0; d < 3; ++d)
            t[d] = T(0.5) * QoM * B[d] * gamma_reci * deltaT;
        T const sfac = T(1.0) / (T(1.0) + l2norm2(t));
        T s[3];
        for(int d = 0; d < 3; ++d)
            s[d] = T(2.0) * t[d] * sfac;
        T mom_prime[3], mom_plus[3];
        // pmacc::math::cross (pmacc/math/vector/Vector.tpp:71-77)
        mom_prime[0] = mom_minus[0] + (mom_minus[1] * t[2] - mom_minus[2] * t[1]);
        mom_prime[1] = mom_minus[1] + (mom_minus[2] * t[0] - mom_minus[0] * t[2]);
        mom_prime[2] = mom_minus[2] + (mom_minus[0] * t[1] - mom_minus[1] * t[0]);
        mom_plus[0] = mom_minus[0] + (mom_prime[1] * s[2] - mom_prime[2] * s[1]);
        mom_plus[1] = mom_minus[1] + (mom_prime[2] * s[0] - mom_prime[0] * s[2]);
        mom_plus[2] = mom_minus[2] + (mom_prime[0] * s[1] - mom_prime[1] * s[0]);
        for(int d = 0; d < 3; ++d)
            mom[d] = mom_plus[d] + T(0.5) * charge * E[d] * deltaT;
        T vel[3];
        velocityOf(mom, mass, T(g.c), vel);
        T const cs[3] = {T(g.dx), T(g.dy), T(g.dz)};
        for(int d = 0; d < 3; ++d)
            pos[d] += (vel[d] * deltaT) / cs[d];
    }

    template<typename T>
    inline T dot3(T const a[3], T const b[3])
    {
        T r = a[0] * b[0];
        r += a[1] * b[1];
        r += a[2] * b[2];
        return r;
    }

    // pmacc::math::cross (pmacc/math/vector/Vector.tpp:71-77)
    template<typename T>
    inline void cross3(T const a[3], T const b[3], T r[3])
    {
        r[0] = a[1] * b[2] - a[2] * b[1];
        r[1] = a[2] * b[0] - a[0] * b[2];
        r[2] = a[0] * b[1] - a[1] * b[0];
    }

    // Position update shared by the pushers: pos += vel dt / cellSize
    template<typename T>
    inline void advance(Grid const& g, T mass, T const mom[3], T pos[3])
    {
        T vel[3];
        velocityOf(mom, mass, T(g.c), vel);
        T const cs[3] = {T(g.dx), T(g.dy), T(g.dz)};
        for(int d = 0; d < 3; ++d)
            pos[d] += (vel[d] * T(g.dt)) / cs[d];
    }

    // HigueraCary (particles/pusher/particlePusherHigueraCary.hpp:85-135).  T is
    // float_X; D is the precision of the square-root stages (param/pusher.param:65-72,
    // precision64Bit by default).  Every cast sits where the reference's types put it.
    template<typename T, typename D>
    inline void higueraCaryPush(Grid const& g, T charge, T mass, T const E[3], T const B[3], T mom[3], T pos[3])
    {
        T const deltaT = T(g.dt);
        T const c = T(g.c);
        T mmT[3];
        for(int d = 0; d < 3; ++d)
            mmT[d] = mom[d] + T(0.5) * charge * E[d] * deltaT;
        D const mm[3] = {D(mmT[0]), D(mmT[1]), D(mmT[2])};
        D const gamma_minus = D(gammaOf(mmT, mass, c)); // Gamma<float_X> casts the momentum back
        D tau[3];
        for(int d = 0; d < 3; ++d)
            tau[d] = D(T(0.5) * B[d] * charge * deltaT / mass);
        D const sigma = gamma_minus * gamma_minus - l2norm2(tau);
        D const u_star = dot3(mm, tau) / D(mass * c);
        D const gamma_plus = std::sqrt(D(0.5) * (sigma + std::sqrt(sigma * sigma + D(4.0) * (l2norm2(tau) + u_star * u_star))));
        D tv[3];
        for(int d = 0; d < 3; ++d)
            tv[d] = tau[d] / gamma_plus;
        D const s = D(1.0) / (D(1.0) + l2norm2(tv));
        D const mt = dot3(mm, tv);
        D cr[3], mp[3], cr2[3];
        cross3(mm, tv, cr);
        for(int d = 0; d < 3; ++d)
            mp[d] = s * (mm[d] + mt * tv[d] + cr[d]);
        cross3(mp, tv, cr2);
        for(int d = 0; d < 3; ++d)
        {
            T const diff = T(0.5) * charge * E[d] * deltaT + T(cr2[d]);
            mom[d] = T(mp[d]) + diff;
        }
        advance(g, mass, mom, pos);
    }

    // Vay (particles/pusher/particlePusherVay.hpp:72-110), precisions as in higueraCaryPush.
    template<typename T, typename D>
    inline void vayPush(Grid const& g, T charge, T mass, T const E[3], T const B[3], T mom[3], T pos[3])
    {
        T const deltaT = T(g.dt);
        T const c = T(g.c);
        T const factor = T(0.5 * double(charge) * double(deltaT));
        T v[3], cvb[3], mp[3];
        velocityOf(mom, mass, c, v);
        cross3(v, B, cvb);
        for(int d = 0; d < 3; ++d)
        {
            T const atZero = mom[d] + factor * (E[d] + cvb[d]);
            mp[d] = atZero + factor * E[d];
        }
        T const gamma_prime = gammaOf(mp, mass, c);
        T const fom = factor / mass;
        D const tau[3] = {D(fom * B[0]), D(fom * B[1]), D(fom * B[2])};
        D const mpD[3] = {D(mp[0]), D(mp[1]), D(mp[2])};
        D const u_star = dot3(mpD, tau) / D(c * mass);
        D const sigma = D(gamma_prime * gamma_prime) - l2norm2(tau);
        D const gamma_half = std::sqrt(D(0.5) * (sigma + std::sqrt(sigma * sigma + D(4.0) * (l2norm2(tau) + u_star * u_star))));
        D const rg = D(T(1.0)) / gamma_half;
        T const t[3] = {T(tau[0] * rg), T(tau[1] * rg), T(tau[2] * rg)};
        T const s = T(1.0) / (T(1.0) + l2norm2(t));
        T const mt = dot3(mp, t);
        T cr[3];
        cross3(mp, t, cr);
        for(int d = 0; d < 3; ++d)
            mom[d] = s * (mp[d] + mt * t[d] + cr[d]);
        advance(g, mass, mom, pos);
    }

    // Free streaming (particles/pusher/particlePusherFree.hpp:40-72)
    template<typename T>
    inline void freePush(Grid const& g, T mass, T const mom[3], T pos[3])
    {
        T vel[3];
        velocityOf(mom, mass, T(g.c), vel);
        T const cs[3] = {T(g.dx), T(g.dy), T(g.dz)};
        for(int d = 0; d < 3; ++d)
            pos[d] += (vel[d] * T(g.dt)) / cs[d];
    }

    // moveParticle (particles/MoveParticle.hpp:48-160).  Updates pos to [0,1),
    // localCellIdx when the cell changes, and returns the supercell exchange
    // direction (multiMask-1, 0 when the particle stays in its supercell).
    template<typename T>
    inline int moveParticle(Grid const& g, T pos[3], uint16_t& lcell, int dirOut[3])
    {
        T const shift = T(0.5);
        int dir[3];
        for(int i = 0; i < 3; ++i)
        {
            T p = pos[i] - shift;
            T moveDir = T(0.0);
            if(p < T(-0.5))
                moveDir = T(-1.0);
            if(p >= T(0.5))
                moveDir = T(1.0);
            p -= moveDir;
            pos[i] = p + shift;
            dir[i] = int(moveDir);
        }
        int newMultimask = 1;
        dirOut[0] = dirOut[1] = dirOut[2] = 0;
        if(dir[0] != 0 || dir[1] != 0 || dir[2] != 0)
        {
            int const scs[3] = {g.sx, g.sy, g.sz};
            int lc[3] = {lcell % g.sx, (lcell / g.sx) % g.sy, lcell / (g.sx * g.sy)};
            for(int i = 0; i < 3; ++i)
                lc[i] += dir[i];
            for(int i = 0; i < 3; ++i)
                dir[i] = uint32_t(lc[i]) >= uint32_t(scs[i]) ? dir[i] : 0;
            for(int i = 0; i < 3; ++i)
                lc[i] -= dir[i] * scs[i];
            lcell = uint16_t(lc[0] + g.sx * (lc[1] + g.sy * lc[2]));
            int exchangeType = 1;
            for(int i = 0; i < 3; ++i)
            {
                newMultimask += (dir[i] == -1 ? 2 : dir[i]) * exchangeType;
                exchangeType *= 3;
            }
            for(int i = 0; i < 3; ++i)
                dirOut[i] = dir[i];
        }
        return newMultimask;
    }

    inline void cellOf(Grid const& g, int32_t sc, uint16_t lcell, int cell[3])
    {
        int const ncx = g.nscx(), ncy = g.nscy();
        int scx = sc % ncx, scy = (sc / ncx) % ncy, scz = sc / (ncx * ncy);
        cell[0] = scx * g.sx + lcell % g.sx;
        cell[1] = scy * g.sy + (lcell / g.sx) % g.sy;
        cell[2] = scz * g.sz + lcell / (g.sx * g.sy);
    }

    // Supercell index after leaving in direction dir; periodic wrap replaces the
    // reference's guard exchange (pmacc/particles/ParticlesBase.kernel:361-631).
    inline int32_t neighbourSc(Grid const& g, int32_t sc, int const dir[3])
    {
        int const ncx = g.nscx(), ncy = g.nscy(), ncz = g.nscz();
        int scx = sc % ncx, scy = (sc / ncx) % ncy, scz = sc / (ncx * ncy);
        // leaving through an open face: absorbed (-1)
        if(((g.open & 1) && (scx + dir[0] < 0 || scx + dir[0] >= ncx))
           || ((g.open & 2) && (scy + dir[1] < 0 || scy + dir[1] >= ncy))
           || ((g.open & 4) && (scz + dir[2] < 0 || scz + dir[2] >= ncz)))
            return -1;
        scx = Grid::wrap(scx + dir[0], ncx);
        scy = Grid::wrap(scy + dir[1], ncy);
        scz = Grid::wrap(scz + dir[2], ncz);
        return int32_t(scx + ncx * (scy + ncy * scz));
    }

    // One species: gather + push + move + supercell shift
    // (particles/Particles.kernel:276-316 PushParticlePerFrame; Particles.tpp:322-368).
    template<typename T>
    void push(Grid const& g, SpeciesParam const& sp, Particles<T>& P, Field3<T> const& E, Field3<T> const& B)
    {
#pragma omp parallel for schedule(static)
        for(long long k = 0; k < (long long) P.n; ++k)
        {
            if(P.sc[k] < 0) // absorbed at an open face in an earlier step
                continue;
            int cell[3];
            cellOf(g, P.sc[k], P.lcell[k], cell);
            T pos[3] = {P.pos[0][k], P.pos[1][k], P.pos[2][k]};
            T mom[3] = {P.mom[0][k], P.mom[1][k], P.mom[2][k]};
            T const w = P.w[k];
            T const mass = T(sp.mass) * w; // traits/attribute/GetMass.hpp:34-37
            T const charge = T(sp.charge) * w; // traits/attribute/GetCharge.hpp:46
            if(sp.pusher == BORIS || sp.pusher == HIGUERA_CARY || sp.pusher == VAY)
            {
                T Bv[3], Ev[3];
                gather(g, sp.shape, B, kPosB, cell, pos, Bv);
                gather(g, sp.shape, E, kPosE, cell, pos, Ev);
                if(sp.pusher == BORIS)
                    borisPush(g, charge, mass, Ev, Bv, mom, pos);
                else if(sp.pusher == HIGUERA_CARY)
                    higueraCaryPush<T, double>(g, charge, mass, Ev, Bv, mom, pos);
                else
                    vayPush<T, double>(g, charge, mass, Ev, Bv, mom, pos);
            }
            else if(sp.pusher == PHOTON)
            {
                // Photon (particles/pusher/particlePusherPhoton.hpp:66-74): vel = mom * (c / |mom|)
                T const normMom = std::sqrt(l2norm2(mom));
                T const f = T(g.c) / normMom;
                T const cs[3] = {T(g.dx), T(g.dy), T(g.dz)};
                for(int d = 0; d < 3; ++d)
                    pos[d] += (mom[d] * f * T(g.dt)) / cs[d];
            }
            else
                freePush(g, mass, mom, pos);
            uint16_t lc = P.lcell[k];
            int dir[3];
            int mm = moveParticle(g, pos, lc, dir);
            for(int d = 0; d < 3; ++d)
            {
                P.pos[d][k] = pos[d];
                P.mom[d][k] = mom[d];
            }
            P.lcell[k] = lc;
            if(mm >= 2)
                P.sc[k] = neighbourSc(g, P.sc[k], dir);
        }
    }

    // ---------------------------------------------------------------- Esirkepov
    // relayPoint (fields/currentDeposition/relayPoint.hpp:48-64)
    template<typename T>
    inline void relayPoint(bool isEven, int& i1, int& i2, T x1, T x2)
    {
        if(isEven)
        {
            i1 = int(std::floor(x1));
            i2 = int(std::floor(x2));
            return;
        }
        i1 = int(std::floor(x1 + T(0.5)));
        i2 = int(std::floor(x2 + T(0.5)));
    }

    enum Status
    {
        LEAVE_CELL = 1,
        START_IN_CELL = 2,
        END_IN_CELL = 4
    }; // Esirkepov/bitPacking.hpp:37-47

    // J accumulator used by the deposit: one component at a global node.
    template<typename T>
    struct JAccess
    {
        Grid const* g;
        Field3<T>* J;
        void add(int comp, int x, int y, int z, T v)
        {
            size_t const i = g->idx(x, y, z);
            if(i != Grid::kOutside) // current beyond an open face is dropped
                J->c[comp][i] += v;
        }
    };

    // cptCurrent1D (fields/currentDeposition/Esirkepov/Esirkepov.hpp:147-242) in the rotated frame:
    // i,j,k are the rotated axes, perm[] maps rotated axis -> real axis, comp = real J component.
    template<typename T, typename Acc>
    void cptCurrent1D(
        Grid const& g,
        int shape,
        int const status[3],
        T const p0[3],
        T const p1[3],
        int const base[3],
        int const perm[3],
        int comp,
        T cellEdgeLength,
        T charge,
        Acc& acc)
    {
        if(p0[2] == p1[2])
            return;
        int const supp = support(shape);
        int const begin = ShapeFn<T>::caBegin(shape);
        int const end = begin + supp;
        // outer loop: Jit shape (shapes/ShapeSelector.hpp:33-52), middle/inner: Cached (:54-75)
        // (Strategy.def:44-53, detail::ShapeStrategy)
        T sj0[6] = {}, sj1[6] = {}, sk0[6] = {}, sk1[6] = {};
        ShapeFn<T>::caArray(shape, p0[1], !(status[1] & START_IN_CELL), sj0);
        ShapeFn<T>::caArray(shape, p1[1], !(status[1] & END_IN_CELL), sj1);
        ShapeFn<T>::caArray(shape, p0[2], !(status[2] & START_IN_CELL), sk0);
        ShapeFn<T>::caArray(shape, p1[2], !(status[2] & END_IN_CELL), sk1);
        T const V = T(g.dx) * T(g.dy) * T(g.dz);
        T const currentSurfaceDensity = charge * (T(1.0) / T(V * T(g.dt))) * cellEdgeLength;
        int const leaveI = status[0] & LEAVE_CELL;
        int const leaveJ = status[1] & LEAVE_CELL;
        int const leaveK = status[2] & LEAVE_CELL;
        for(int i = begin; i < end + 1; ++i)
            if(i < end + leaveI)
            {
                T const s0i = ShapeFn<T>::ca(shape, T(i) - p0[0]);
                T const dsi = ShapeFn<T>::ca(shape, T(i) - p1[0]) - s0i;
                for(int j = begin; j < end + 1; ++j)
                    if(j < end + leaveJ)
                    {
                        T const s0j = sj0[j - begin];
                        T const dsj = sj1[j - begin] - s0j;
                        T tmp = -currentSurfaceDensity
                            * (s0i * s0j + T(0.5) * (dsi * s0j + s0i * dsj) + (T(1.0) / T(3.0)) * dsj * dsi);
                        T accumulated_J = T(0.0);
                        for(int k = begin; k < end; ++k)
                            if(k < end + leaveK - 1)
                            {
                                T const W = (sk1[k - begin] - sk0[k - begin]) * tmp;
                                accumulated_J += W;
                                int r[3] = {i, j, k};
                                int node[3];
                                for(int a = 0; a < 3; ++a)
                                    node[perm[a]] = base[perm[a]] + r[a];
                                acc.add(comp, node[0], node[1], node[2], accumulated_J);
                            }
                    }
            }
    }

    // Esirkepov::operator() (Esirkepov/Esirkepov.hpp:62-134).  cell = global cell of
    // the particle after the move, pos = in-cell position after the move, vel from
    // the new momentum (fields/FieldJ.kernel:110-142 ComputePerFrame).
    template<typename T, typename Acc>
    void esirkepov(Grid const& g, int shape, int const cell[3], T const pos[3], T const vel[3], T charge, Acc& acc)
    {
        int const supp = support(shape);
        bool const isEven = (supp % 2) == 0;
        T const cs[3] = {T(g.dx), T(g.dy), T(g.dz)};
        T p0[3], p1[3];
        for(int d = 0; d < 3; ++d)
        {
            T const deltaPos = vel[d] * T(g.dt) / cs[d];
            p0[d] = pos[d] - deltaPos;
            p1[d] = pos[d];
        }
        int gridShift[3], status[3] = {0, 0, 0};
        for(int d = 0; d < 3; ++d)
        {
            int iStart, iEnd;
            relayPoint(isEven, iStart, iEnd, p0[d], p1[d]);
            gridShift[d] = iStart < iEnd ? iStart : iEnd;
            status[d] |= (gridShift[d] == iStart) ? START_IN_CELL : 0;
            status[d] |= (gridShift[d] == iEnd) ? END_IN_CELL : 0;
            status[d] |= (iStart != iEnd) ? LEAVE_CELL : 0;
            p0[d] -= T(gridShift[d]);
            p1[d] -= T(gridShift[d]);
        }
        int base[3] = {cell[0] + gridShift[0], cell[1] + gridShift[1], cell[2] + gridShift[2]};
        // J_x: rotation (1,2,0) (Esirkepov.hpp:112-117)
        {
            int const st[3] = {status[1], status[2], status[0]};
            T const q0[3] = {p0[1], p0[2], p0[0]}, q1[3] = {p1[1], p1[2], p1[0]};
            int const perm[3] = {1, 2, 0};
            cptCurrent1D(g, shape, st, q0, q1, base, perm, 0, cs[0], charge, acc);
        }
        // J_y: rotation (2,0,1) (Esirkepov.hpp:118-123)
        {
            int const st[3] = {status[2], status[0], status[1]};
            T const q0[3] = {p0[2], p0[0], p0[1]}, q1[3] = {p1[2], p1[0], p1[1]};
            int const perm[3] = {2, 0, 1};
            cptCurrent1D(g, shape, st, q0, q1, base, perm, 1, cs[1], charge, acc);
        }
        // J_z: identity (Esirkepov.hpp:124-129)
        {
            int const perm[3] = {0, 1, 2};
            cptCurrent1D(g, shape, status, p0, p1, base, perm, 2, cs[2], charge, acc);
        }
    }

    // ---------------------------------------------------------------- EmZ
    // One rotated 1D current of an EmZ virtual particle (EmZ/DepositCurrent.hpp:76-126):
    // on-support shapes, Jit for the outer loop and Cached for the middle and inner loops
    // (Strategy.def:44-61), loops [begin, begin + supp) and [begin, begin + supp - 1).
    template<typename T, typename Acc>
    void emzCurrent1D(
        int shape,
        T const p0[3],
        T const p1[3],
        int const base[3],
        int const perm[3],
        int comp,
        T currentSurfaceDensity,
        Acc& acc)
    {
        if(p0[2] == p1[2])
            return;
        int const supp = support(shape);
        int const begin = ShapeFn<T>::osBegin(shape);
        int const end = begin + supp;
        T sj0[6] = {}, sj1[6] = {}, sk0[6] = {}, sk1[6] = {};
        ShapeFn<T>::baseArray(shape, p0[1], sj0);
        ShapeFn<T>::baseArray(shape, p1[1], sj1);
        ShapeFn<T>::baseArray(shape, p0[2], sk0);
        ShapeFn<T>::baseArray(shape, p1[2], sk1);
        for(int i = begin; i < end; ++i)
        {
            T const s0i = ShapeFn<T>::os(shape, T(i) - p0[0]);
            T const dsi = ShapeFn<T>::os(shape, T(i) - p1[0]) - s0i;
            for(int j = begin; j < end; ++j)
            {
                T const s0j = sj0[j - begin];
                T const dsj = sj1[j - begin] - s0j;
                T tmp = -currentSurfaceDensity
                    * (s0i * s0j + T(0.5) * (dsi * s0j + s0i * dsj) + (T(1.0) / T(3.0)) * dsj * dsi);
                T accumulated_J = T(0.0);
                for(int k = begin; k < end - 1; ++k)
                {
                    T const W = (sk1[k - begin] - sk0[k - begin]) * tmp;
                    accumulated_J += W;
                    int r[3] = {i, j, k};
                    int node[3];
                    for(int a = 0; a < 3; ++a)
                        node[perm[a]] = base[perm[a]] + r[a];
                    acc.add(comp, node[0], node[1], node[2], accumulated_J);
                }
            }
        }
    }

    // One EmZ virtual particle from p0 to p1 in the frame of cell `base`
    // (EmZ/DepositCurrent.hpp:38-63): the three rotated calls.
    template<typename T, typename Acc>
    void emzVirtual(Grid const& g, int shape, T const p0[3], T const p1[3], int const base[3], T chargeDensity, Acc& acc)
    {
        T const cs[3] = {T(g.dx), T(g.dy), T(g.dz)};
        T const dt = T(g.dt);
        {
            T const q0[3] = {p0[1], p0[2], p0[0]}, q1[3] = {p1[1], p1[2], p1[0]};
            int const perm[3] = {1, 2, 0};
            emzCurrent1D(shape, q0, q1, base, perm, 0, cs[0] * chargeDensity / dt, acc);
        }
        {
            T const q0[3] = {p0[2], p0[0], p0[1]}, q1[3] = {p1[2], p1[0], p1[1]};
            int const perm[3] = {2, 0, 1};
            emzCurrent1D(shape, q0, q1, base, perm, 1, cs[1] * chargeDensity / dt, acc);
        }
        {
            int const perm[3] = {0, 1, 2};
            emzCurrent1D(shape, p0, p1, base, perm, 2, cs[2] * chargeDensity / dt, acc);
        }
    }

    // EmZ::operator() (fields/currentDeposition/EmZ/EmZ.hpp:72-120): the trajectory is
    // split at the relay point (relayPoint.hpp:48-64) into at most two virtual particles,
    // each on support.  Arguments as for esirkepov().
    template<typename T, typename Acc>
    void emz(Grid const& g, int shape, int const cell[3], T const pos[3], T const vel[3], T charge, Acc& acc)
    {
        int const supp = support(shape);
        bool const isEven = (supp % 2) == 0;
        T const cs[3] = {T(g.dx), T(g.dy), T(g.dz)};
        T posStart[3], relay[3];
        int shiftStart[3], shiftEnd[3];
        bool two = false;
        for(int d = 0; d < 3; ++d)
        {
            T const deltaPos = (vel[d] * T(g.dt)) / cs[d];
            posStart[d] = pos[d] - deltaPos;
            relayPoint(isEven, shiftStart[d], shiftEnd[d], posStart[d], pos[d]);
            if(shiftStart[d] == shiftEnd[d])
                relay[d] = pos[d];
            else if(isEven)
                relay[d] = T(std::max(shiftStart[d], shiftEnd[d]));
            else
                relay[d] = T(shiftStart[d] + shiftEnd[d]) / T(2.0);
            two |= shiftStart[d] != shiftEnd[d];
        }
        T const chargeDensity = charge / (cs[0] * cs[1] * cs[2]);
        T a0[3], a1[3];
        int base[3];
        for(int d = 0; d < 3; ++d)
        {
            a0[d] = posStart[d] - T(shiftStart[d]);
            a1[d] = relay[d] - T(shiftStart[d]);
            base[d] = cell[d] + shiftStart[d];
        }
        emzVirtual(g, shape, a0, a1, base, chargeDensity, acc);
        if(two)
        {
            for(int d = 0; d < 3; ++d)
            {
                a1[d] = pos[d] - T(shiftEnd[d]);
                a0[d] = relay[d] - T(shiftEnd[d]);
                base[d] = cell[d] + shiftEnd[d];
            }
            emzVirtual(g, shape, a0, a1, base, chargeDensity, acc);
        }
    }

    // The species' current solver (param/species.param: UsedParticleCurrentSolver).
    template<typename T, typename Acc>
    void depositOne(Grid const& g, SpeciesParam const& sp, int const cell[3], T const pos[3], T const vel[3], T charge, Acc& acc)
    {
        if(sp.current == EMZ_CURRENT)
            emz(g, sp.shape, cell, pos, vel, charge, acc);
        else
            esirkepov(g, sp.shape, cell, pos, vel, charge, acc);
    }

    // Deposit all particles of one species into J (FieldJ.kernel:52-142; the guard
    // add of CurrentInterpolationAndAdditionToEMF.hpp:110 is the periodic wrap here).
    // Single-threaded in particle order so that the result is reproducible.
    template<typename T>
    void deposit(Grid const& g, SpeciesParam const& sp, Particles<T> const& P, Field3<T>& J)
    {
        JAccess<T> acc{&g, &J};
        for(size_t k = 0; k < P.n; ++k)
        {
            if(P.sc[k] < 0)
                continue;
            int cell[3];
            cellOf(g, P.sc[k], P.lcell[k], cell);
            T const pos[3] = {P.pos[0][k], P.pos[1][k], P.pos[2][k]};
            T const mom[3] = {P.mom[0][k], P.mom[1][k], P.mom[2][k]};
            T const w = P.w[k];
            T const charge = T(sp.charge) * w;
            T vel[3];
            velocityOf(mom, T(sp.mass) * w, T(g.c), vel);
            depositOne(g, sp, cell, pos, vel, charge, acc);
        }
    }

    // Multi-threaded deposit: each thread deposits a static slice of the particles
    // into a private J, the private J are summed in thread order.  Used for the
    // CPU baseline timing.
    template<typename T>
    void depositThreaded(Grid const& g, SpeciesParam const& sp, Particles<T> const& P, Field3<T>& J, int nthreads)
    {
        if(nthreads <= 1)
        {
            deposit(g, sp, P, J);
            return;
        }
        size_t const nc = g.ncells();
        std::vector<std::vector<T>> priv(nthreads, std::vector<T>(3 * nc, T(0)));
#pragma omp parallel num_threads(nthreads)
        {
#ifdef _OPENMP
            int const t = omp_get_thread_num();
#else
            int const t = 0;
#endif
            Field3<T> Jt{{priv[t].data(), priv[t].data() + nc, priv[t].data() + 2 * nc}};
            JAccess<T> acc{&g, &Jt};
            size_t const chunk = (P.n + nthreads - 1) / nthreads;
            size_t const k0 = std::min(P.n, chunk * t), k1 = std::min(P.n, k0 + chunk);
            for(size_t k = k0; k < k1; ++k)
            {
                if(P.sc[k] < 0)
                    continue;
                int cell[3];
                cellOf(g, P.sc[k], P.lcell[k], cell);
                T const pos[3] = {P.pos[0][k], P.pos[1][k], P.pos[2][k]};
                T const mom[3] = {P.mom[0][k], P.mom[1][k], P.mom[2][k]};
                T const w = P.w[k];
                T vel[3];
                velocityOf(mom, T(sp.mass) * w, T(g.c), vel);
                depositOne(g, sp, cell, pos, vel, T(sp.charge) * w, acc);
            }
        }
#pragma omp parallel for schedule(static)
        for(long long i = 0; i < (long long) nc; ++i)
            for(int d = 0; d < 3; ++d)
                for(int t = 0; t < nthreads; ++t)
                    J.c[d][i] += priv[t][d * nc + i];
    }

    // ---------------------------------------------------------------- diagnostics
    // Charge density with ChargeAssignment at the cell origin
    // (particles/particleToGrid/ComputeGridValuePerFrame.hpp:66-117,
    //  derivedAttributes/ChargeDensity.hpp:39-50).
    template<typename T>
    void chargeDensity(Grid const& g, SpeciesParam const& sp, Particles<T> const& P, T* rho)
    {
        int const supp = support(sp.shape);
        int const lo = supp / 2, up = (supp + 1) / 2;
        int const span = lo + up + 1;
        T const V = T(g.dx) * T(g.dy) * T(g.dz);
        for(size_t k = 0; k < P.n; ++k)
        {
            if(P.sc[k] < 0)
                continue;
            int cell[3];
            cellOf(g, P.sc[k], P.lcell[k], cell);
            T const attr = (T(sp.charge) * P.w[k]) / V;
            for(int i = 0; i < span * span * span; ++i)
            {
                int const off[3] = {i % span - lo, (i / span) % span - lo, i / (span * span) - lo};
                T assign = T(1.0);
                for(int d = 0; d < 3; ++d)
                    assign *= ShapeFn<T>::ca(sp.shape, T(off[d]) - P.pos[d][k]);
                size_t const ri = g.idx(cell[0] + off[0], cell[1] + off[1], cell[2] + off[2]);
                if(ri != Grid::kOutside)
                    rho[ri] += assign * attr;
            }
        }
    }

    // |eps0 * div E - rho| per cell (plugins/ChargeConservation.tpp:121-135, 211-240); returns the max.
    template<typename T>
    double chargeResidual(Grid const& g, Field3<T> const& E, T const* rho, T* out)
    {
        T const rw = T(1.0) / T(g.dx), rh = T(1.0) / T(g.dy), rd = T(1.0) / T(g.dz);
        double mx = 0.0;
        for(int z = 0; z < g.nz; ++z)
            for(int y = 0; y < g.ny; ++y)
                for(int x = 0; x < g.nx; ++x)
                {
                    size_t i = g.idx(x, y, z);
                    T div = (E.c[0][i] - Grid::at(E.c[0], g.idx(x - 1, y, z))) * rw
                        + (E.c[1][i] - Grid::at(E.c[1], g.idx(x, y - 1, z))) * rh
                        + (E.c[2][i] - Grid::at(E.c[2], g.idx(x, y, z - 1))) * rd;
                    T r = std::abs(div * T(g.eps0) - rho[i]);
                    if(out)
                        out[i] = r;
                    mx = std::max(mx, double(r));
                }
        return mx;
    }

    // Kinetic energy of one macro particle (algorithms/KinEnergy.hpp:43-66).
    template<typename T>
    inline T kinEnergy(T const mom[3], T mass, T c)
    {
        if(mass == T(0.0))
            return c * std::sqrt(l2norm2(mom));
        T const gamma = gammaOf(mom, mass, c);
        if(gamma < T(1.005)) // GAMMA_THRESH (param/speciesConstants.param:39)
            return l2norm2(mom) / (T(2.0) * mass);
        T const c2 = c * c;
        return (gamma - T(1.0)) * mass * c2;
    }

    // Sum of kinetic energies in FP64 (plugins/EnergyParticles.x.cpp:58-160).
    template<typename T>
    double kineticEnergy(Grid const& g, SpeciesParam const& sp, Particles<T> const& P)
    {
        double sum = 0.0;
        for(size_t k = 0; k < P.n; ++k)
        {
            if(P.sc[k] < 0)
                continue;
            T const mom[3] = {P.mom[0][k], P.mom[1][k], P.mom[2][k]};
            sum += double(kinEnergy(mom, T(sp.mass) * P.w[k], T(g.c)));
        }
        return sum;
    }

    // Field energies in FP64 (plugins/EnergyFields.x.cpp:211-225, 240-261):
    // out[0] = eps0/2 * V * sum E^2, out[1] = 1/(2 mu0) * V * sum B^2.
    template<typename T>
    void fieldEnergy(Grid const& g, Field3<T> const& E, Field3<T> const& B, double out[2])
    {
        double sE[3] = {0, 0, 0}, sB[3] = {0, 0, 0};
        size_t n = g.ncells();
        for(size_t i = 0; i < n; ++i)
            for(int d = 0; d < 3; ++d)
            {
                T e = E.c[d][i], b = B.c[d][i];
                sE[d] += double(e * e);
                sB[d] += double(b * b);
            }
        double const V = double(g.dx) * double(g.dy) * double(g.dz);
        double const mu0 = 1.0 / (double(g.eps0) * double(g.c) * double(g.c));
        out[0] = out[1] = 0.0;
        for(int d = 0; d < 3; ++d)
        {
            out[0] += sE[d] * (double(g.eps0) * V * 0.5);
            out[1] += sB[d] * (0.5 / mu0 * V);
        }
    }

    // ---------------------------------------------------------------- incident field (TF/SF)
    // One face of the Huygens box carrying the focused Gaussian pulse of
    // profiles/GaussianPulse.hpp:206-290 (linear polarisation, fundamental Laguerre mode), in the
    // reference's vector form (fields/incidentField/Functors.hpp BaseFunctorE): the origin is the
    // focus projected along the propagation direction onto the Huygens surface (0.75 cells
    // inside POSITION, getOrigin), the local time runs from it at the grid's phase velocity
    // (getCurrentTime), internal coordinates are dot products with the direction (axis0), the
    // polarisation (axis1) and their cross product (axis2).  POSITION: the first total E plane
    // of a low face is POSITION + 1, the last of a high face POSITION - 1.
    struct IncidentFace
    {
        int axis = 1, dir = 1; // face normal and side (+1: low face, -1: high face)
        int surface = 1; // first (dir +1) or last (dir -1) E plane of the total-field region
        float dirv[3] = {0.f, 1.f, 0.f}; // unit propagation direction (DIRECTION_*), entering through the face
        float polv[3] = {1.f, 0.f, 0.f}; // unit E polarisation, orthogonal to dirv
        int circular = 0; // PolarisationType::Circular
        float focus[3] = {0.f, 0.f, 0.f}; // focus position (length units)
        float amplitude = 1.f; // E0
        float wavelength = 1.f, w0 = 1.f;
        float pulseDuration = 1.f; // rms duration of the intensity (PULSE_DURATION)
        float timeShift = 0.f; // GaussianPulseEnvelope::TIME_SHIFT = -PULSE_INIT * PULSE_DURATION / 2
        float laserPhase = 0.f;
        float phaseVelocity = 1.f; // calculatePhaseVelocity, times c
        float timeDelay = 0.f; // TIME_DELAY
        int nmodes = 1; // laguerreModes / laguerrePhases
        float modes[8] = {1.f}, modePhases[8] = {0.f};
        int profile = 0; // 0 GaussianPulse, 1 PlaneWave, 2 Wavepacket, 3 Polynom
        float rampInit = 0.f, nofocus = 0.f; // PlaneWave RAMP_INIT, LASER_NOFOCUS_CONSTANT
        float pulseInit = 0.f; // Wavepacket PULSE_INIT
        float w0Axis1 = 1.f, w0Axis2 = 1.f; // W0_AXIS_1, W0_AXIS_2
    };

    // WavepacketFunctorIncidentE::getLongitudinal (profiles/Wavepacket.hpp:118-151)
    inline float wavepacketLongitudinal(IncidentFace const& f, float omega, float time, float phaseShift)
    {
        float const initTime = f.pulseInit * f.pulseDuration + f.nofocus;
        float const endUpramp = -0.5f * f.nofocus, startDownramp = 0.5f * f.nofocus;
        float const mue = 0.5f * initTime;
        float const runTime = time - mue;
        float const tau = f.pulseDuration * std::sqrt(2.f);
        float envelope = f.amplitude, correctionFactor = 0.f;
        if(runTime > startDownramp)
        {
            float const exponent = ((runTime - startDownramp) / f.pulseDuration / std::sqrt(2.f));
            envelope *= std::exp(-0.5f * exponent * exponent);
            correctionFactor = (runTime - startDownramp) / (tau * tau * omega);
        }
        else if(runTime < endUpramp)
        {
            float const exponent = ((runTime - endUpramp) / f.pulseDuration / std::sqrt(2.f));
            envelope *= std::exp(-0.5f * exponent * exponent);
            correctionFactor = (runTime - endUpramp) / (tau * tau * omega);
        }
        float const phase = omega * runTime + f.laserPhase + phaseShift;
        return (std::sin(phase) + correctionFactor * std::cos(phase)) * envelope;
    }

    // PolynomFunctorIncidentE::getLongitudinal and polynomial (profiles/Polynom.hpp:113-136)
    inline float polynomLongitudinal(IncidentFace const& f, float omega, float time, float phaseShift)
    {
        float const riseTime = 0.5f * f.pulseDuration;
        float const tau = time / riseTime;
        float const phase = omega * (time - riseTime) + f.laserPhase + phaseShift;
        float result = 0.f;
        if(tau >= 0.f && tau <= 1.f)
            result = tau * tau * tau * (10.f - 15.f * tau + 6.f * tau * tau);
        else if(tau > 1.f && tau <= 2.f)
            result = (2.f - tau) * (2.f - tau) * (2.f - tau) * (4.f - 9.f * tau + 6.f * tau * tau);
        float const amplitude = f.amplitude * result;
        return std::sin(phase) * amplitude;
    }

    // PlaneWaveFunctorIncidentE::getLongitudinal (profiles/PlaneWave.hpp:79-106)
    inline float planeWaveLongitudinal(IncidentFace const& f, float omega, float time, float phaseShift)
    {
        float envelope = f.amplitude;
        float const mue = 0.5f * f.rampInit * f.pulseDuration;
        float const tau = f.pulseDuration * std::sqrt(2.0f);
        float const endUpramp = mue;
        float const startDownramp = mue + f.nofocus;
        float integrationCorrectionFactor = 0.f;
        if(time > startDownramp)
        {
            float const exponent = (time - startDownramp) / tau;
            envelope *= std::exp(-0.5f * exponent * exponent);
            integrationCorrectionFactor = (time - startDownramp) / (omega * tau * tau);
        }
        else if(time < endUpramp)
        {
            float const exponent = (time - endUpramp) / tau;
            envelope *= std::exp(-0.5f * exponent * exponent);
            integrationCorrectionFactor = (time - endUpramp) / (omega * tau * tau);
        }
        float const timeOszi = time - endUpramp;
        float const phase = omega * timeOszi + f.laserPhase + phaseShift;
        return (std::sin(phase) + std::cos(phase) * integrationCorrectionFactor) * envelope;
    }

    // simpleLaguerre (GaussianPulse.hpp:298-323): the Laguerre polynomial L_n(x) by its recursion
    inline float simpleLaguerre(int n, float x)
    {
        if(n == 0)
            return 1.f;
        int cur = 1;
        float lm1 = 1.f, l = 1.f - x, lp = 0.f;
        while(cur < n)
        {
            lp = ((2.f * float(cur) + 1.f - x) * l - float(cur) * lm1) / float(cur + 1);
            lm1 = l;
            l = lp;
            ++cur;
        }
        return l;
    }

    inline float dotf(float const a[3], float const b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

    // E (or B = direction x E / c: ApproximateIncidentB) of the face at total cell index idx
    // (fractional, cells) and time t.
    inline void incidentFieldAt(Grid const& g, IncidentFace const& f, float const idx[3], float t, bool wantB, float out[3])
    {
        float const cell[3] = {g.dx, g.dy, g.dz};
        float const* dirv = f.dirv;
        // getOrigin: the focus moved back along the direction onto the Huygens surface of the face
        // (the reference takes the latest crossing of the box's planes; the face's own plane here)
        float const minPos = (float(f.surface - 1) + 0.75f) * cell[f.axis];
        float const maxPos = (float(f.surface + 1) - 0.75f) * cell[f.axis];
        float const originP = ((f.dir > 0 ? minPos : maxPos) - f.focus[f.axis]) / dirv[f.axis];
        float origin[3];
        for(int d = 0; d < 3; ++d)
            origin[d] = f.focus[d] + originP * dirv[d];
        origin[f.axis] = f.dir > 0 ? minPos : maxPos;
        float shift[3];
        for(int d = 0; d < 3; ++d)
            shift[d] = idx[d] * cell[d] - origin[d];
        float const pos0 = dotf(shift, dirv);
        float const currentTime = t - (pos0 / f.phaseVelocity + f.timeDelay);
        float value = 0.f, value1 = 0.f; // value1: with the phase shifted by pi/2 (circular)
        if(f.profile != 0 && !(currentTime < 0.f))
        {
            // BaseSeparableFunctorE: longitudinal(time) times the transversal factor, 1 for PlaneWave,
            // exp(-|internal position / (1, W0_AXIS_1, W0_AXIS_2)|^2) with the propagation coordinate set
            // to 0 for Wavepacket and Polynom (BaseSeparableTransversalGaussianFunctorE)
            float const omega = 2.f * 3.14159265358979323846f * g.c / f.wavelength;
            float transversal = 1.f;
            if(f.profile >= 2)
            {
                float const axis2[3] = {dirv[1] * f.polv[2] - dirv[2] * f.polv[1],
                                        dirv[2] * f.polv[0] - dirv[0] * f.polv[2],
                                        dirv[0] * f.polv[1] - dirv[1] * f.polv[0]};
                float const q[3] = {0.f / 1.f, dotf(shift, f.polv) / f.w0Axis1, dotf(shift, axis2) / f.w0Axis2};
                transversal = std::exp(-(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]));
            }
            auto lon = [&](float ph)
            {
                if(f.profile == 2)
                    return wavepacketLongitudinal(f, omega, currentTime, ph);
                if(f.profile == 3)
                    return polynomLongitudinal(f, omega, currentTime, ph);
                return planeWaveLongitudinal(f, omega, currentTime, ph);
            };
            value = lon(0.f) * transversal;
            value1 = lon(1.57079633f) * transversal;
        }
        else if(!(currentTime < 0.f)) // cut off before the pulse reaches this point
        {
            float const time = currentTime + f.timeShift;
            float const axis2[3] = {dirv[1] * f.polv[2] - dirv[2] * f.polv[1], dirv[2] * f.polv[0] - dirv[0] * f.polv[2],
                                    dirv[0] * f.polv[1] - dirv[1] * f.polv[0]};
            float const pos1 = dotf(shift, f.polv), pos2 = dotf(shift, axis2);
            float focusRel[3];
            for(int d = 0; d < 3; ++d)
                focusRel[d] = f.focus[d] - origin[d];
            float const focusPos = dotf(focusRel, dirv) - pos0;
            float const zR = 3.14159265358979323846f * f.w0 * f.w0 / f.wavelength;
            float const w = f.w0 * std::sqrt(1.f + (focusPos / zR) * (focusPos / zR));
            float const omega = 2.f * 3.14159265358979323846f * g.c / f.wavelength;
            float const phase = omega * (time - focusPos / g.c) + f.laserPhase;
            float const r2 = pos1 * pos1 + pos2 * pos2;
            float const rInv = -focusPos / (zR * zR + focusPos * focusPos);
            float const xi = std::atan(-focusPos / zR);
            float const r2OverW2 = r2 / w / w;
            float const r = 0.5f * r2 * rInv;
            float const k = 2.f * 3.14159265358979323846f / f.wavelength;
            float const shiftedTime = time - r / g.c;
            float const exponent = shiftedTime / (2.f * f.pulseDuration);
            float norm = 0.f;
            for(int m = 0; m < f.nmodes; ++m)
                norm += f.modes[m];
            auto modesSum = [&](float ph)
            {
                float etrans = 0.f;
                for(int m = 0; m < f.nmodes; ++m)
                    etrans += f.modes[m] * simpleLaguerre(m, 2.f * r2OverW2) * std::exp(-r2OverW2)
                        * std::cos(k * focusPos - k * r + (2.f * float(m) + 1.f) * xi + ph + f.modePhases[m]);
                etrans *= std::exp(-exponent * exponent);
                return f.amplitude * (f.w0 / w) * etrans / norm;
            };
            value = modesSum(phase);
            if(f.circular)
                value1 = modesSum(omega * (time - focusPos / g.c) + f.laserPhase + 1.57079633f);
        }
        float E[3];
        if(!f.circular)
            for(int d = 0; d < 3; ++d)
                E[d] = f.polv[d] * value;
        else
        {
            // getCircularPolarizationVector1 = polarisation / sqrt(2), vector2 = direction x vector1
            float v1[3], v2[3];
            for(int d = 0; d < 3; ++d)
                v1[d] = f.polv[d] / std::sqrt(2.f);
            v2[0] = dirv[1] * v1[2] - dirv[2] * v1[1];
            v2[1] = dirv[2] * v1[0] - dirv[0] * v1[2];
            v2[2] = dirv[0] * v1[1] - dirv[1] * v1[0];
            for(int d = 0; d < 3; ++d)
                E[d] = v1[d] * value1 + v2[d] * value;
        }
        if(!wantB)
        {
            for(int d = 0; d < 3; ++d)
                out[d] = E[d];
            return;
        }
        out[0] = (dirv[1] * E[2] - dirv[2] * E[1]) / g.c;
        out[1] = (dirv[2] * E[0] - dirv[0] * E[2]) / g.c;
        out[2] = (dirv[0] * E[1] - dirv[1] * E[0]) / g.c;
    }

    // TF/SF correction of one face after a field update (incidentField/Solver.kernel
    // UpdateFunctor for the Yee curl, margin 1):
    //   updated[comp2] += base * incident[comp1](shift1), updated[comp1] -= base * incident[comp2](shift2),
    //   comp1 = (axis + 2) % 3, comp2 = (axis + 1) % 3, base = curlCoefficient / d_axis * dir,
    // curlCoefficient = -dt/2 for a B half step (incident E) and c^2 dt for the E step (incident B).
    // The updated plane along the axis is the first total E plane (E) or the scattered B plane
    // before it (B) for a low face, the last total E plane and the B plane after it for a high
    // face (Solver.hpp:206-266); the incident field is taken at the updated cell plus its Yee
    // position, shifted along the axis by -1 (E) or +1 (B) on a low face (Solver.hpp:343-356).
    inline void incidentUpdate(Grid const& g, IncidentFace const& f, Field3<float>& F, bool updateB, float t)
    {
        int const a = f.axis, comp1 = (a + 2) % 3, comp2 = (a + 1) % 3;
        float const cell[3] = {g.dx, g.dy, g.dz};
        float const curl = updateB ? -0.5f * g.dt : g.c * g.c * g.dt;
        float const base = curl / cell[a] * (f.dir > 0 ? 1.f : -1.f);
        int const plane = (updateB && f.dir > 0) ? f.surface - 1 : f.surface;
        float baseShift = 0.f;
        if(f.dir > 0)
            baseShift = updateB ? 1.f : -1.f;
        // Yee positions of the incident field's components (B when E is updated, E when B is)
        auto const& incPos = updateB ? kPosE : kPosB;
        int const n[3] = {g.nx, g.ny, g.nz};
        int const u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
        for(int j = 0; j < n[v]; ++j)
            for(int i = 0; i < n[u]; ++i)
            {
                int c[3];
                c[a] = plane;
                c[u] = i;
                c[v] = j;
                float s1[3], s2[3];
                for(int d = 0; d < 3; ++d)
                {
                    s1[d] = float(c[d]) + incPos[comp1][d];
                    s2[d] = float(c[d]) + incPos[comp2][d];
                }
                s1[a] += baseShift;
                s2[a] += baseShift;
                float inc1[3], inc2[3];
                incidentFieldAt(g, f, s1, t, !updateB, inc1);
                incidentFieldAt(g, f, s2, t, !updateB, inc2);
                size_t const id = g.idx(c[0], c[1], c[2]);
                F.c[comp2][id] += base * inc1[comp1];
                F.c[comp1][id] -= base * inc2[comp2];
            }
    }

    // ---------------------------------------------------------------- full step
    // Simulation::runOneStep (simulation/control/Simulation.hpp:522-542):
    // CurrentReset, ParticlePush (+shift), update_beforeCurrent (B half, E),
    // CurrentDeposition, AddCurrent (E += coeff J), update_afterCurrent (B half).
    template<typename T>
    void step(
        Grid const& g,
        int nspecies,
        SpeciesParam const* sp,
        Particles<T>* P,
        Field3<T>& E,
        Field3<T>& B,
        Field3<T>& J,
        int depositThreads)
    {
        size_t const n = g.ncells();
        for(int d = 0; d < 3; ++d)
            std::fill(J.c[d], J.c[d] + n, T(0));
        for(int s = 0; s < nspecies; ++s)
            push(g, sp[s], P[s], E, B);
        yeeBHalf(g, E, B);
        yeeE(g, B, E);
        for(int s = 0; s < nspecies; ++s)
            if(sp[s].current)
                depositThreaded(g, sp[s], P[s], J, depositThreads);
        addCurrent(g, J, E);
        yeeBHalf(g, E, B);
    }
    // ---------------------------------------------------------------- open boundaries, PML
    // Convolutional PML of fields/absorber/pml/Pml.kernel for the open axes of g.open.
    struct PmlConfig
    {
        int cells[3][2]; // thickness at the negative and positive face of each open axis
        double sigmaMax[3], kappaMax[3], alphaMax[3]; // normalized (divided by eps0), 1/time
        double order, alphaOrder; // grading orders
    };

    // b, c, kappa at position x (cells) along axis a (Pml.kernel:130-267): relative depth d,
    // sigma = sigmaMax d^m, kappa = 1 + (kappaMax - 1) d^m, alpha = alphaMax (1 - d)^ma,
    // b = exp(-(sigma / kappa + alpha) dt), c = sigma (b - 1) / (kappa (sigma + alpha kappa)).
    inline void pmlCoef(Grid const& g, PmlConfig const& p, int a, double x, float out[3])
    {
        int const n = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
        double depth = 0.0;
        if(g.open & (1 << a))
        {
            double const neg = p.cells[a][0], pos = p.cells[a][1];
            double const rightStart = double(n) - pos;
            if(x < neg)
                depth = (neg - x) / neg;
            else if(x > rightStart && pos > 0)
                depth = (x - rightStart) / pos;
        }
        double sigma = 0.0, alpha = 0.0, kappa = 1.0;
        if(depth != 0.0)
        {
            double const grade = std::pow(depth, p.order);
            sigma = p.sigmaMax[a] * grade;
            kappa = 1.0 + (p.kappaMax[a] - 1.0) * grade;
            alpha = p.alphaMax[a] * std::pow(1.0 - depth, p.alphaOrder);
        }
        double const b = std::exp(-(sigma / kappa + alpha) * double(g.dt));
        double const den = kappa * (sigma + alpha * kappa);
        out[0] = float(b);
        out[1] = float(den != 0.0 ? sigma * (b - 1.0) / den : 0.0);
        out[2] = float(kappa);
    }

    // psi component order: xy, xz, yx, yz, zx, zy (psi.ab: field component a, derivative along b)
    enum
    {
        PSI_XY,
        PSI_XZ,
        PSI_YX,
        PSI_YZ,
        PSI_ZX,
        PSI_ZY
    };

    // B half step with the PML (Pml.kernel:522-581); the convolution fields advance when updatePsi.
    inline void yeeBHalfOpen(Grid const& g, PmlConfig const& p, Field3<float> const& E, Field3<float>& B, float* const psi[6], bool updatePsi)
    {
#pragma omp parallel for schedule(static)
        for(int z = 0; z < g.nz; ++z)
            for(int y = 0; y < g.ny; ++y)
                for(int x = 0; x < g.nx; ++x)
                {
                    size_t const i = g.idx(x, y, z), ix = g.idx(x + 1, y, z), iy = g.idx(x, y + 1, z),
                                 iz = g.idx(x, y, z + 1);
                    float const dFdx_y = (Grid::at(E.c[1], ix) - E.c[1][i]) / g.dx;
                    float const dFdx_z = (Grid::at(E.c[2], ix) - E.c[2][i]) / g.dx;
                    float const dFdy_x = (Grid::at(E.c[0], iy) - E.c[0][i]) / g.dy;
                    float const dFdy_z = (Grid::at(E.c[2], iy) - E.c[2][i]) / g.dy;
                    float const dFdz_x = (Grid::at(E.c[0], iz) - E.c[0][i]) / g.dz;
                    float const dFdz_y = (Grid::at(E.c[1], iz) - E.c[1][i]) / g.dz;
                    float cx[3], cy[3], cz[3];
                    pmlCoef(g, p, 0, x + 0.5, cx);
                    pmlCoef(g, p, 1, y + 0.5, cy);
                    pmlCoef(g, p, 2, z + 0.5, cz);
                    if(cx[0] * cy[0] * cz[0] == 1.0f)
                    {
                        B.c[0][i] = B.c[0][i] - (dFdy_z - dFdz_y) * 0.5f * g.dt;
                        B.c[1][i] = B.c[1][i] - (dFdz_x - dFdx_z) * 0.5f * g.dt;
                        B.c[2][i] = B.c[2][i] - (dFdx_y - dFdy_x) * 0.5f * g.dt;
                        continue;
                    }
                    if(updatePsi)
                    {
                        psi[PSI_YX][i] = cx[0] * psi[PSI_YX][i] + cx[1] * dFdx_z;
                        psi[PSI_ZX][i] = cx[0] * psi[PSI_ZX][i] + cx[1] * dFdx_y;
                        psi[PSI_XY][i] = cy[0] * psi[PSI_XY][i] + cy[1] * dFdy_z;
                        psi[PSI_ZY][i] = cy[0] * psi[PSI_ZY][i] + cy[1] * dFdy_x;
                        psi[PSI_XZ][i] = cz[0] * psi[PSI_XZ][i] + cz[1] * dFdz_y;
                        psi[PSI_YZ][i] = cz[0] * psi[PSI_YZ][i] + cz[1] * dFdz_x;
                    }
                    float const h = 0.5f * g.dt;
                    B.c[0][i] += h * (dFdz_y / cz[2] - dFdy_z / cy[2] + psi[PSI_XZ][i] - psi[PSI_XY][i]);
                    B.c[1][i] += h * (dFdx_z / cx[2] - dFdz_x / cz[2] + psi[PSI_YX][i] - psi[PSI_YZ][i]);
                    B.c[2][i] += h * (dFdy_x / cy[2] - dFdx_y / cx[2] + psi[PSI_ZY][i] - psi[PSI_ZX][i]);
                }
    }

    // E step with the PML (Pml.kernel:424-475); the convolution fields advance every call.
    inline void yeeEOpen(Grid const& g, PmlConfig const& p, Field3<float> const& B, Field3<float>& E, float* const psi[6])
    {
        float const c2 = g.c * g.c;
#pragma omp parallel for schedule(static)
        for(int z = 0; z < g.nz; ++z)
            for(int y = 0; y < g.ny; ++y)
                for(int x = 0; x < g.nx; ++x)
                {
                    size_t const i = g.idx(x, y, z), ix = g.idx(x - 1, y, z), iy = g.idx(x, y - 1, z),
                                 iz = g.idx(x, y, z - 1);
                    float const dFdx_y = (B.c[1][i] - Grid::at(B.c[1], ix)) / g.dx;
                    float const dFdx_z = (B.c[2][i] - Grid::at(B.c[2], ix)) / g.dx;
                    float const dFdy_x = (B.c[0][i] - Grid::at(B.c[0], iy)) / g.dy;
                    float const dFdy_z = (B.c[2][i] - Grid::at(B.c[2], iy)) / g.dy;
                    float const dFdz_x = (B.c[0][i] - Grid::at(B.c[0], iz)) / g.dz;
                    float const dFdz_y = (B.c[1][i] - Grid::at(B.c[1], iz)) / g.dz;
                    float cx[3], cy[3], cz[3];
                    pmlCoef(g, p, 0, x, cx);
                    pmlCoef(g, p, 1, y, cy);
                    pmlCoef(g, p, 2, z, cz);
                    if(cx[0] * cy[0] * cz[0] == 1.0f)
                    {
                        E.c[0][i] = E.c[0][i] + (dFdy_z - dFdz_y) * c2 * g.dt;
                        E.c[1][i] = E.c[1][i] + (dFdz_x - dFdx_z) * c2 * g.dt;
                        E.c[2][i] = E.c[2][i] + (dFdx_y - dFdy_x) * c2 * g.dt;
                        continue;
                    }
                    psi[PSI_YX][i] = cx[0] * psi[PSI_YX][i] + cx[1] * dFdx_z;
                    psi[PSI_ZX][i] = cx[0] * psi[PSI_ZX][i] + cx[1] * dFdx_y;
                    psi[PSI_XY][i] = cy[0] * psi[PSI_XY][i] + cy[1] * dFdy_z;
                    psi[PSI_ZY][i] = cy[0] * psi[PSI_ZY][i] + cy[1] * dFdy_x;
                    psi[PSI_XZ][i] = cz[0] * psi[PSI_XZ][i] + cz[1] * dFdz_y;
                    psi[PSI_YZ][i] = cz[0] * psi[PSI_YZ][i] + cz[1] * dFdz_x;
                    float const c2dt = c2 * g.dt;
                    E.c[0][i] += c2dt * (dFdy_z / cy[2] - dFdz_y / cz[2] + psi[PSI_XY][i] - psi[PSI_XZ][i]);
                    E.c[1][i] += c2dt * (dFdz_x / cz[2] - dFdx_z / cx[2] + psi[PSI_YZ][i] - psi[PSI_YX][i]);
                    E.c[2][i] += c2dt * (dFdx_y / cx[2] - dFdy_x / cy[2] + psi[PSI_ZX][i] - psi[PSI_ZY][i]);
                }
    }
} // namespace orc
