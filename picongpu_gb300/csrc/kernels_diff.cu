// Kernels of the differentiable PIC step (picgb_diff_* in picgb.h): the
// forward step on particles in a fixed order and its adjoint, for float and
// double, CIC/TSC/PQS.  One thread per particle; fields, J and the adjoint
// fields are read and scattered in global memory.
#include "picgb_diff.hpp"
#include "picgb_diff_math.cuh"

namespace picgb::diff
{
    constexpr int kDiffThreads = 128;
    // rows per particle of the fields kept by the replay: 6 values and 6 x 3 position gradients
    constexpr int kGatherRows = 24;

    template<typename T>
    struct DiffParticles
    {
        int32_t* cell; // [3][n]
        T* pos; // [3][n]
        T* mom; // [3][n]
        T const* w; // [n]
        uint64_t n;
        T charge, mass;
        int32_t* cellOut; // new state (may equal the inputs)
        T* posOut;
        T* momOut;
    };

    // Everything one particle's step computes from its start state and the fields.
    template<int SHAPE, typename T>
    struct ParticleStep
    {
        int cell[3], newCell[3];
        T pos[3], mom[3], newPos[3], newMom[3], vel[3], dp[3];
        T qw, mw;
        T Ef[3], Bf[3];
        DBoris<T> boris;
        DTrajectory<SHAPE, T> traj;

        // gathered: this particle's six field values and their position gradients from an
        // earlier pass ([kGatherRows][n]), or null
        __device__ void run(
            DiffParticles<T> const& sp,
            uint64_t p,
            T const* E,
            T const* B,
            DiffGrid<T> const& g,
            T const* gathered = nullptr,
            T* keep = nullptr)
        {
            size_t const nc = size_t(g.nx) * g.ny * g.nz;
            for(int d = 0; d < 3; ++d)
            {
                cell[d] = sp.cell[d * sp.n + p];
                pos[d] = sp.pos[d * sp.n + p];
                mom[d] = sp.mom[d * sp.n + p];
            }
            T const w = sp.w[p];
            qw = sp.charge * w;
            mw = sp.mass * w;
            // the gather weights are not kept: the adjoint recomputes them at its end, which keeps
            // them out of the registers during the deposit adjoint
            T f6[6];
            if(gathered)
            {
                for(int comp = 0; comp < 6; ++comp)
                    f6[comp] = gathered[comp * sp.n + p];
            }
            else if(keep)
            {
                // the fields and their gradients, kept for the adjoint of this step
                DGather<SHAPE, T> gw;
                gw.compute(cell, pos, g);
#pragma unroll 1
                for(int comp = 0; comp < 6; ++comp)
                {
                    T gr[3];
                    f6[comp] = gw.valueGradAt(comp < 3 ? E + comp * nc : B + (comp - 3) * nc, comp, gr);
                    keep[comp * sp.n + p] = f6[comp];
                    for(int d = 0; d < 3; ++d)
                        keep[(6 + 3 * comp + d) * sp.n + p] = gr[d];
                }
            }
            else
            {
                DGather<SHAPE, T> gw;
                gw.compute(cell, pos, g);
#pragma unroll 1
                for(int comp = 0; comp < 6; ++comp)
                    f6[comp] = gw.valueAt(comp < 3 ? E + comp * nc : B + (comp - 3) * nc, comp);
            }
            for(int d = 0; d < 3; ++d)
            {
                Ef[d] = f6[d];
                Bf[d] = f6[3 + d];
            }
            boris.forward(qw, mw, Ef, Bf, g.dt, g.c, mom, newMom);
            dVelocity(mw, g.c, newMom, vel);
            int const n3[3] = {g.nx, g.ny, g.nz};
            for(int d = 0; d < 3; ++d)
            {
                dp[d] = vel[d] * g.dt / cellSize(g, d);
                // moveParticle: recentred position, at most one cell per step
                T const x = pos[d] + dp[d] - T(0.5);
                int m = 0;
                if(x < T(-0.5))
                    m = -1;
                if(x >= T(0.5))
                    m = 1;
                newPos[d] = (x - T(m)) + T(0.5);
                newCell[d] = wrapIdx(cell[d] + m, n3[d]);
            }
            traj.compute(newCell, newPos, dp, g);
        }

        __device__ T qvdt(DiffGrid<T> const& g) const { return qw / (g.dx * g.dy * g.dz * g.dt); }
    };

    template<int SHAPE, typename T>
    __global__ void __launch_bounds__(kDiffThreads)
        kDiffPush(
            DiffParticles<T> sp,
            T const* __restrict__ E,
            T const* __restrict__ B,
            T* __restrict__ J,
            DiffGrid<T> g,
            T* __restrict__ gathered)
    {
        uint64_t const p = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        if(p >= sp.n)
            return;
        ParticleStep<SHAPE, T> st;
        st.run(sp, p, E, B, g, nullptr, gathered);
        if(J) // the replay of the backward pass moves the particles only
            esirkepovDeposit(st.traj, st.qvdt(g), g, J);
        for(int d = 0; d < 3; ++d)
        {
            sp.cellOut[d * sp.n + p] = st.newCell[d];
            sp.posOut[d * sp.n + p] = st.newPos[d];
            sp.momOut[d * sp.n + p] = st.newMom[d];
        }
    }

    // Adjoint of kDiffPush for the particles: lamPos/lamMom hold dL/d(state after the step)
    // on entry and dL/d(state before the step) on exit; dL/dE, dL/dB of the gather are
    // added to lamE, lamB.  lamJ = dL/dJ of this step.
    template<int SHAPE, typename T>
#ifndef PICGB_ADJOINT_MIN_BLOCKS
#    define PICGB_ADJOINT_MIN_BLOCKS 3 // resident blocks of 128 threads the adjoint's register budget is sized for
#endif
    __global__ void __launch_bounds__(kDiffThreads, PICGB_ADJOINT_MIN_BLOCKS) kDiffAdjoint(
        DiffParticles<T> sp,
        T const* __restrict__ E,
        T const* __restrict__ B,
        T const* __restrict__ lamJ,
        T* __restrict__ lamE,
        T* __restrict__ lamB,
        T* __restrict__ lamPos,
        T* __restrict__ lamMom,
        DiffGrid<T> g,
        T const* __restrict__ gathered)
    {
        uint64_t const p = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        if(p >= sp.n)
            return;
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        ParticleStep<SHAPE, T> st;
        st.run(sp, p, E, B, g, gathered);
        T lpos[3], lmom[3];
        for(int d = 0; d < 3; ++d)
        {
            lpos[d] = lamPos[d * sp.n + p];
            lmom[d] = lamMom[d * sp.n + p];
        }
        // deposit: J(q0 = newPos - dp - shift, q1 = newPos - shift)
        T gq0[3] = {T(0), T(0), T(0)}, gq1[3] = {T(0), T(0), T(0)};
        esirkepovAdjoint(st.traj, st.qvdt(g), g, lamJ, gq0, gq1);
        // newPos = pos + v dt / d (- integer move); dp = v dt / d
        T lv[3], lposOld[3];
        for(int d = 0; d < 3; ++d)
        {
            T const lnew = lpos[d] + gq0[d] + gq1[d];
            lposOld[d] = lnew;
            lv[d] = (lnew - gq0[d]) * g.dt / cellSize(g, d);
        }
        dVelocityAdjoint(st.mw, g.c, st.newMom, lv, lmom);
        T lp[3], lE[3], lB[3];
        st.boris.adjoint(st.qw, st.mw, st.Bf, g.dt, g.c, lmom, lp, lE, lB);
        T gpos[3] = {T(0), T(0), T(0)};
        DGather<SHAPE, T> gw;
        gw.compute(st.cell, st.pos, g);
        T const l6[6] = {lE[0], lE[1], lE[2], lB[0], lB[1], lB[2]};
#pragma unroll 1
        for(int comp = 0; comp < 6; ++comp)
        {
            size_t const o = size_t(comp % 3) * nc;
            T const lam = comp == 0 ? l6[0] : comp == 1 ? l6[1] : comp == 2 ? l6[2] : comp == 3 ? l6[3] : comp == 4 ? l6[4] : l6[5];
            if(gathered)
            {
                // position gradient from the kept field gradients; only the scatter remains
                for(int d = 0; d < 3; ++d)
                    gpos[d] += lam * gathered[(6 + 3 * comp + d) * sp.n + p];
                gw.scatterAt(comp < 3 ? lamE + o : lamB + o, comp, lam);
            }
            else
                gw.adjointAt(comp < 3 ? E + o : B + o, comp < 3 ? lamE + o : lamB + o, comp, lam, gpos);
        }
        for(int d = 0; d < 3; ++d)
        {
            lamPos[d * sp.n + p] = lposOld[d] + gpos[d];
            lamMom[d * sp.n + p] = lp[d];
        }
    }

    // A += alpha * curl(F) with forward (FWD) or backward differences, periodic.
    template<typename T, bool FWD>
    __global__ void kCurlAdd(T* __restrict__ A, T const* __restrict__ F, T alpha, DiffGrid<T> g)
    {
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        size_t const i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
        if(i >= nc)
            return;
        int const x = int(i % g.nx), y = int((i / g.nx) % g.ny), z = int(i / (size_t(g.nx) * g.ny));
        int const o = FWD ? 1 : -1;
        size_t const ix = cellIndex(g, x + o, y, z), iy = cellIndex(g, x, y + o, z), iz = cellIndex(g, x, y, z + o);
        T const* Fx = F;
        T const* Fy = F + nc;
        T const* Fz = F + 2 * nc;
        auto d = [&](T const* f, size_t j, T h) { return (FWD ? (f[j] - f[i]) : (f[i] - f[j])) / h; };
        T const cx = d(Fz, iy, g.dy) - d(Fy, iz, g.dz);
        T const cy = d(Fx, iz, g.dz) - d(Fz, ix, g.dx);
        T const cz = d(Fy, ix, g.dx) - d(Fx, iy, g.dy);
        A[i] += alpha * cx;
        A[nc + i] += alpha * cy;
        A[2 * nc + i] += alpha * cz;
    }

    template<typename T>
    __global__ void kAxpby(T* __restrict__ y, T a, T const* __restrict__ x, T b, size_t n)
    {
        size_t const i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
        if(i < n)
            y[i] = a * x[i] + b * y[i];
    }

    template<typename T>
    __global__ void kKinetic(DiffParticles<T> sp, T c, double* out)
    {
        uint64_t const p = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        double e = 0.0;
        if(p < sp.n)
        {
            T const mw = sp.mass * sp.w[p];
            T const p2 = sp.mom[p] * sp.mom[p] + sp.mom[sp.n + p] * sp.mom[sp.n + p]
                + sp.mom[2 * sp.n + p] * sp.mom[2 * sp.n + p];
            // gamma - 1 = u^2 / (gamma + 1): no cancellation for slow particles
            T const u2 = p2 / (mw * mw * c * c);
            e = double(u2 / (sqrt(T(1) + u2) + T(1)) * mw * c * c);
        }
        for(int o = 16; o > 0; o >>= 1)
            e += __shfl_down_sync(0xffffffffu, e, o);
        if((threadIdx.x & 31) == 0)
            atomicAdd(out, e);
    }

    // ---------------------------------------------------------------- launchers
    template<typename T>
    DiffParticles<T> particles(DiffSpeciesPtr const& s)
    {
        return DiffParticles<T>{
            s.cell,
            static_cast<T*>(s.pos),
            static_cast<T*>(s.mom),
            static_cast<T const*>(s.w),
            s.n,
            T(s.charge),
            T(s.mass),
            s.cellOut ? s.cellOut : s.cell,
            static_cast<T*>(s.posOut ? s.posOut : s.pos),
            static_cast<T*>(s.momOut ? s.momOut : s.mom)};
    }

    template<typename T>
    DiffGrid<T> grid(DiffGridDesc const& d)
    {
        return DiffGrid<T>{d.nx, d.ny, d.nz, T(d.dx), T(d.dy), T(d.dz), T(d.dt), T(d.c), T(d.eps0)};
    }

    inline unsigned blocksFor(uint64_t n, int threads) { return unsigned((n + threads - 1) / threads); }

    template<typename T, int SHAPE>
    cudaError_t pushT(
        DiffSpeciesPtr const& s,
        void const* E,
        void const* B,
        void* J,
        void* gathered,
        DiffGridDesc const& g,
        cudaStream_t st)
    {
        if(s.n == 0)
            return cudaSuccess;
        kDiffPush<SHAPE, T><<<blocksFor(s.n, kDiffThreads), kDiffThreads, 0, st>>>(
            particles<T>(s),
            static_cast<T const*>(E),
            static_cast<T const*>(B),
            static_cast<T*>(J),
            grid<T>(g),
            static_cast<T*>(gathered));
        return cudaGetLastError();
    }

    template<typename T, int SHAPE>
    cudaError_t adjointT(
        DiffSpeciesPtr const& s,
        void const* E,
        void const* B,
        void const* lamJ,
        void* lamE,
        void* lamB,
        void* lamPos,
        void* lamMom,
        void const* gathered,
        DiffGridDesc const& g,
        cudaStream_t st)
    {
        if(s.n == 0)
            return cudaSuccess;
        kDiffAdjoint<SHAPE, T><<<blocksFor(s.n, kDiffThreads), kDiffThreads, 0, st>>>(
            particles<T>(s),
            static_cast<T const*>(E),
            static_cast<T const*>(B),
            static_cast<T const*>(lamJ),
            static_cast<T*>(lamE),
            static_cast<T*>(lamB),
            static_cast<T*>(lamPos),
            static_cast<T*>(lamMom),
            grid<T>(g),
            static_cast<T const*>(gathered));
        return cudaGetLastError();
    }

    template<typename T>
    cudaError_t dispatchPush(
        int shape,
        DiffSpeciesPtr const& s,
        void const* E,
        void const* B,
        void* J,
        void* gathered,
        DiffGridDesc const& g,
        cudaStream_t st)
    {
        switch(shape)
        {
        case 1:
            return pushT<T, 1>(s, E, B, J, gathered, g, st);
        case 2:
            return pushT<T, 2>(s, E, B, J, gathered, g, st);
        case 3:
            return pushT<T, 3>(s, E, B, J, gathered, g, st);
        }
        return cudaErrorInvalidValue;
    }

    template<typename T>
    cudaError_t dispatchAdjoint(
        int shape,
        DiffSpeciesPtr const& s,
        void const* E,
        void const* B,
        void const* lamJ,
        void* lamE,
        void* lamB,
        void* lamPos,
        void* lamMom,
        void const* gathered,
        DiffGridDesc const& g,
        cudaStream_t st)
    {
        switch(shape)
        {
        case 1:
            return adjointT<T, 1>(s, E, B, lamJ, lamE, lamB, lamPos, lamMom, gathered, g, st);
        case 2:
            return adjointT<T, 2>(s, E, B, lamJ, lamE, lamB, lamPos, lamMom, gathered, g, st);
        case 3:
            return adjointT<T, 3>(s, E, B, lamJ, lamE, lamB, lamPos, lamMom, gathered, g, st);
        }
        return cudaErrorInvalidValue;
    }

    cudaError_t launchDiffPush(
        int precision,
        int shape,
        DiffSpeciesPtr const& s,
        void const* E,
        void const* B,
        void* J,
        void* gathered,
        DiffGridDesc const& g,
        cudaStream_t st)
    {
        return precision == 8 ? dispatchPush<double>(shape, s, E, B, J, gathered, g, st)
                              : dispatchPush<float>(shape, s, E, B, J, gathered, g, st);
    }

    cudaError_t launchDiffAdjoint(
        int precision,
        int shape,
        DiffSpeciesPtr const& s,
        void const* E,
        void const* B,
        void const* lamJ,
        void* lamE,
        void* lamB,
        void* lamPos,
        void* lamMom,
        void const* gathered,
        DiffGridDesc const& g,
        cudaStream_t st)
    {
        return precision == 8
            ? dispatchAdjoint<double>(shape, s, E, B, lamJ, lamE, lamB, lamPos, lamMom, gathered, g, st)
            : dispatchAdjoint<float>(shape, s, E, B, lamJ, lamE, lamB, lamPos, lamMom, gathered, g, st);
    }

    template<typename T>
    cudaError_t curlT(void* A, void const* F, double alpha, bool forward, DiffGridDesc const& g, cudaStream_t st)
    {
        size_t const nc = size_t(g.nx) * g.ny * g.nz;
        if(forward)
            kCurlAdd<T, true><<<blocksFor(nc, 256), 256, 0, st>>>(
                static_cast<T*>(A),
                static_cast<T const*>(F),
                T(alpha),
                grid<T>(g));
        else
            kCurlAdd<T, false><<<blocksFor(nc, 256), 256, 0, st>>>(
                static_cast<T*>(A),
                static_cast<T const*>(F),
                T(alpha),
                grid<T>(g));
        return cudaGetLastError();
    }

    cudaError_t launchDiffCurlAdd(
        int precision,
        void* A,
        void const* F,
        double alpha,
        bool forward,
        DiffGridDesc const& g,
        cudaStream_t st)
    {
        return precision == 8 ? curlT<double>(A, F, alpha, forward, g, st) : curlT<float>(A, F, alpha, forward, g, st);
    }

    cudaError_t launchDiffAxpby(int precision, void* y, double a, void const* x, double b, size_t n, cudaStream_t st)
    {
        if(n == 0)
            return cudaSuccess;
        if(precision == 8)
            kAxpby<double><<<blocksFor(n, 256), 256, 0, st>>>(static_cast<double*>(y), a, static_cast<double const*>(x), b, n);
        else
            kAxpby<float>
                <<<blocksFor(n, 256), 256, 0, st>>>(static_cast<float*>(y), float(a), static_cast<float const*>(x), float(b), n);
        return cudaGetLastError();
    }

    cudaError_t launchDiffKinetic(int precision, DiffSpeciesPtr const& s, double c, double* out, cudaStream_t st)
    {
        if(s.n == 0)
            return cudaSuccess;
        if(precision == 8)
            kKinetic<double><<<blocksFor(s.n, 256), 256, 0, st>>>(particles<double>(s), c, out);
        else
            kKinetic<float><<<blocksFor(s.n, 256), 256, 0, st>>>(particles<float>(s), float(c), out);
        return cudaGetLastError();
    }
} // namespace picgb::diff
