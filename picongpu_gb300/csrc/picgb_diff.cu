// Differentiable PIC run (picgb_diff_* in picgb.h): forward steps on caller
// arrays with checkpoints every K steps, and the backward pass that replays
// each segment from its checkpoint and runs the adjoint steps in reverse.
//
// Checkpoints: the particles every K steps, the fields (E, B: a few MB per step) at
// every step when they fit in a quarter of the free device memory.  The replay of a
// segment then only moves the particles through the stored fields (gather, push,
// move: no deposit, no field update), and the adjoint steps read the forward's own
// fields.  Otherwise the replay runs the whole step from the segment's checkpoint.
//
// Adjoint of one step (forward: J = push(x, u, E, B); B1 = B - dt/2 Cf E;
// E1 = E + c^2 dt Cb B1 + coeff J; B2 = B1 - dt/2 Cf E1, with Cf / Cb the
// forward / backward difference curls of FDTDBase.hpp:97-183 and Cf^T = Cb):
//   lamE += -dt/2 Cb lamB;  lamB += c^2 dt Cf lamE;  lamJ = coeff lamE;
//   lamE += -dt/2 Cb lamB;  particles: (lamX, lamU, lamJ) -> (lamX, lamU), += lamE, lamB.
#include "picgb.h"
#include "picgb_diff.hpp"
#include "picgb_sim.hpp"

#include <algorithm>
#include <vector>

using namespace picgb::diff;
using picgb::host::fail;

namespace
{
    constexpr int kMaxSpecies = PICGB_DIFF_MAX_SPECIES;

    // Device addresses of one full state: fields and every species' cell, pos, mom.
    struct StatePtrs
    {
        void* E;
        void* B;
        int32_t* cell[kMaxSpecies];
        void* pos[kMaxSpecies];
        void* mom[kMaxSpecies];
    };
} // namespace

struct picgb_diff
{
    picgb_diff_config cfg{};
    DiffGridDesc g{};
    int prec = 4;
    size_t esz = 4;
    size_t nc = 0;
    std::vector<picgb_diff_species> species;
    std::vector<void const*> weights; // from the last forward call (caller-owned)
    void* J = nullptr;
    void* lamJ = nullptr;
    size_t blobBytes = 0;
    std::vector<void*> ckpts; // state at steps 0, K, 2K, ...
    std::vector<void*> seg; // states of one segment during the backward pass
    std::vector<void*> gathered; // per step of a segment: the particles' gathered E, B and gradients ([24][n])
    void* fieldHist = nullptr; // E and B at the start of every forward step (histSteps entries)
    size_t histSteps = 0;
    bool denseFields = false; // the last forward stored its fields at every step
    uint32_t nsteps = 0;
    bool haveForward = false;

    size_t fieldBytes() const { return 3 * nc * esz; }
    size_t fieldStride() const { return (fieldBytes() + 255) / 256 * 256; }

    // E and B of forward step i in the dense field history
    void* histE(size_t i) const { return static_cast<char*>(fieldHist) + 2 * i * fieldStride(); }
    void* histB(size_t i) const { return static_cast<char*>(fieldHist) + (2 * i + 1) * fieldStride(); }

    // offsets of a state blob: E, B, then per species cell, pos, mom (256-byte aligned)
    StatePtrs blobPtrs(void* blob) const
    {
        StatePtrs s{};
        auto* b = static_cast<char*>(blob);
        size_t off = 0;
        auto take = [&](size_t bytes)
        {
            char* p = b + off;
            off += (bytes + 255) / 256 * 256;
            return p;
        };
        s.E = take(fieldBytes());
        s.B = take(fieldBytes());
        for(size_t k = 0; k < species.size(); ++k)
        {
            s.cell[k] = reinterpret_cast<int32_t*>(take(3 * species[k].n * sizeof(int32_t)));
            s.pos[k] = take(3 * species[k].n * esz);
            s.mom[k] = take(3 * species[k].n * esz);
        }
        return s;
    }

    size_t computeBlobBytes() const
    {
        size_t off = 2 * ((fieldBytes() + 255) / 256 * 256);
        for(auto const& sp : species)
        {
            off += (3 * sp.n * sizeof(int32_t) + 255) / 256 * 256;
            off += 2 * ((3 * sp.n * esz + 255) / 256 * 256);
        }
        return off;
    }

    size_t gatheredBytes() const
    {
        size_t b = 0;
        for(auto const& sp : species)
            b += (24 * sp.n * esz + 255) / 256 * 256;
        return b;
    }

    // species k's part of a gathered-field buffer, or null
    void* gatheredPtr(void* buf, size_t k) const
    {
        if(!buf)
            return nullptr;
        size_t off = 0;
        for(size_t i = 0; i < k; ++i)
            off += (24 * species[i].n * esz + 255) / 256 * 256;
        return static_cast<char*>(buf) + off;
    }

    DiffSpeciesPtr speciesPtr(StatePtrs const& s, size_t k) const
    {
        return DiffSpeciesPtr{s.cell[k], s.pos[k], s.mom[k], weights[k], species[k].n, species[k].charge, species[k].mass};
    }
};

namespace
{
    StatePtrs callerPtrs(picgb_diff const* d, picgb_diff_state const* st)
    {
        StatePtrs s{};
        s.E = st->E;
        s.B = st->B;
        for(size_t k = 0; k < d->species.size(); ++k)
        {
            s.cell[k] = st->cell[k];
            s.pos[k] = st->pos[k];
            s.mom[k] = st->mom[k];
        }
        return s;
    }

    int copyState(picgb_diff const* d, StatePtrs const& dst, StatePtrs const& src, cudaStream_t st)
    {
        CUDA_TRY(cudaMemcpyAsync(dst.E, src.E, d->fieldBytes(), cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(dst.B, src.B, d->fieldBytes(), cudaMemcpyDeviceToDevice, st));
        for(size_t k = 0; k < d->species.size(); ++k)
        {
            size_t const n = d->species[k].n;
            CUDA_TRY(cudaMemcpyAsync(dst.cell[k], src.cell[k], 3 * n * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(cudaMemcpyAsync(dst.pos[k], src.pos[k], 3 * n * d->esz, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(cudaMemcpyAsync(dst.mom[k], src.mom[k], 3 * n * d->esz, cudaMemcpyDeviceToDevice, st));
        }
        return PICGB_OK;
    }

    // One forward step (Simulation::runOneStep with the fused deposit) from state s into state
    // o (o == s: in place; otherwise s is left unchanged); the particles' gathered fields go to
    // `gathered` when it is not null.
    int stepForward(picgb_diff* d, StatePtrs const& s, StatePtrs const& o, cudaStream_t st, void* gathered = nullptr)
    {
        double const dt = d->g.dt, c2 = d->g.c * d->g.c;
        CUDA_TRY(cudaMemsetAsync(d->J, 0, d->fieldBytes(), st));
        for(size_t k = 0; k < d->species.size(); ++k)
        {
            DiffSpeciesPtr sp = d->speciesPtr(s, k);
            sp.cellOut = o.cell[k];
            sp.posOut = o.pos[k];
            sp.momOut = o.mom[k];
            CUDA_TRY(launchDiffPush(d->prec, d->cfg.shape, sp, s.E, s.B, d->J, d->gatheredPtr(gathered, k), d->g, st));
        }
        if(o.E != s.E)
        {
            CUDA_TRY(cudaMemcpyAsync(o.E, s.E, d->fieldBytes(), cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(cudaMemcpyAsync(o.B, s.B, d->fieldBytes(), cudaMemcpyDeviceToDevice, st));
        }
        StatePtrs const& s2 = o; // the field update runs on the output fields
        CUDA_TRY(launchDiffCurlAdd(d->prec, s2.B, s2.E, -0.5 * dt, true, d->g, st));
        CUDA_TRY(launchDiffCurlAdd(d->prec, s2.E, s2.B, c2 * dt, false, d->g, st));
        CUDA_TRY(launchDiffAxpby(d->prec, s2.E, -dt / d->g.eps0, d->J, 1.0, 3 * d->nc, st));
        CUDA_TRY(launchDiffCurlAdd(d->prec, s2.B, s2.E, -0.5 * dt, true, d->g, st));
        return PICGB_OK;
    }

    // Replay of forward step i for the particles only, through the stored fields of that step:
    // particles of state s -> state o, the gathered fields to `gathered`.
    int stepReplayParticles(picgb_diff* d, size_t i, StatePtrs const& s, StatePtrs const& o, cudaStream_t st, void* gathered)
    {
        for(size_t k = 0; k < d->species.size(); ++k)
        {
            DiffSpeciesPtr sp = d->speciesPtr(s, k);
            sp.cellOut = o.cell[k];
            sp.posOut = o.pos[k];
            sp.momOut = o.mom[k];
            CUDA_TRY(launchDiffPush(d->prec, d->cfg.shape, sp, d->histE(i), d->histB(i), nullptr,
                                    d->gatheredPtr(gathered, k), d->g, st));
        }
        return PICGB_OK;
    }

    // Room for the fields of every step of an n-step forward, if it fits in a quarter of the
    // free device memory; false otherwise (the backward pass then replays whole steps).
    bool ensureFieldHistory(picgb_diff* d, size_t n)
    {
        if(d->fieldHist && d->histSteps >= n)
            return true;
        size_t const bytes = 2 * n * d->fieldStride();
        size_t freeB = 0, total = 0;
        if(cudaMemGetInfo(&freeB, &total) != cudaSuccess || bytes > freeB / 4)
            return false;
        if(d->fieldHist)
            cudaFree(d->fieldHist);
        d->fieldHist = nullptr;
        d->histSteps = 0;
        if(cudaMalloc(&d->fieldHist, bytes) != cudaSuccess)
        {
            cudaGetLastError();
            d->fieldHist = nullptr;
            return false;
        }
        d->histSteps = n;
        return true;
    }

    // Adjoint of the step that started in state s; lam holds dL/d(state after) on entry.
    // gathered: the particles' fields kept by the replay of this step, or null.
    int stepAdjoint(picgb_diff* d, StatePtrs const& s, StatePtrs const& lam, cudaStream_t st, void* gathered)
    {
        double const dt = d->g.dt, c2 = d->g.c * d->g.c;
        CUDA_TRY(launchDiffCurlAdd(d->prec, lam.E, lam.B, -0.5 * dt, false, d->g, st));
        CUDA_TRY(launchDiffCurlAdd(d->prec, lam.B, lam.E, c2 * dt, true, d->g, st));
        CUDA_TRY(cudaMemsetAsync(d->lamJ, 0, d->fieldBytes(), st));
        CUDA_TRY(launchDiffAxpby(d->prec, d->lamJ, -dt / d->g.eps0, lam.E, 0.0, 3 * d->nc, st));
        CUDA_TRY(launchDiffCurlAdd(d->prec, lam.E, lam.B, -0.5 * dt, false, d->g, st));
        for(size_t k = 0; k < d->species.size(); ++k)
            CUDA_TRY(launchDiffAdjoint(
                d->prec,
                d->cfg.shape,
                d->speciesPtr(s, k),
                s.E,
                s.B,
                d->lamJ,
                lam.E,
                lam.B,
                lam.pos[k],
                lam.mom[k],
                d->gatheredPtr(gathered, k),
                d->g,
                st));
        return PICGB_OK;
    }

    int ensureBlobs(picgb_diff* d, size_t nckpt)
    {
        while(d->ckpts.size() < nckpt)
        {
            void* p = nullptr;
            CUDA_TRY(cudaMalloc(&p, d->blobBytes));
            d->ckpts.push_back(p);
        }
        size_t const K = size_t(d->cfg.checkpoint_every);
        while(d->seg.size() < K)
        {
            void* p = nullptr;
            CUDA_TRY(cudaMalloc(&p, d->blobBytes));
            d->seg.push_back(p);
        }
        while(d->gathered.size() < K)
        {
            void* p = nullptr;
            CUDA_TRY(cudaMalloc(&p, d->gatheredBytes()));
            d->gathered.push_back(p);
        }
        return PICGB_OK;
    }

    int checkState(picgb_diff const* d, picgb_diff_state const* st, bool grad)
    {
        if(!st || !st->E || !st->B || st->nspecies != int32_t(d->species.size()))
            return fail(PICGB_ERR_INVALID, "state needs E, B and %zu species", d->species.size());
        for(size_t k = 0; k < d->species.size(); ++k)
            if(d->species[k].n && (!st->pos[k] || !st->mom[k] || (!grad && (!st->cell[k] || !st->w[k]))))
                return fail(PICGB_ERR_INVALID, "species %zu: null state array", k);
        return PICGB_OK;
    }
} // namespace

extern "C"
{
    int picgb_diff_create(
        const picgb_diff_config* cfg,
        int32_t nspecies,
        const picgb_diff_species* species,
        picgb_diff** out)
    {
        if(!cfg || !out || nspecies < 0 || nspecies > kMaxSpecies || (nspecies && !species))
            return fail(PICGB_ERR_INVALID, "invalid arguments (at most %d species)", kMaxSpecies);
        *out = nullptr;
        if(cfg->nx < 4 || cfg->ny < 4 || cfg->nz < 4 || double(cfg->nx) * cfg->ny * cfg->nz >= 4294967296.0)
            return fail(PICGB_ERR_INVALID, "grid needs at least 4 cells per axis and fewer than 2^32 cells");
        if(cfg->precision != 4 && cfg->precision != 8)
            return fail(PICGB_ERR_INVALID, "precision must be 4 (float) or 8 (double)");
        if(cfg->shape < PICGB_SHAPE_CIC || cfg->shape > PICGB_SHAPE_PQS)
            return fail(PICGB_ERR_UNSUPPORTED, "shape %d: CIC, TSC or PQS", int(cfg->shape));
        if(cfg->checkpoint_every < 1)
            return fail(PICGB_ERR_INVALID, "checkpoint_every must be >= 1");
        if(!(cfg->dx > 0 && cfg->dy > 0 && cfg->dz > 0 && cfg->dt > 0 && cfg->c > 0 && cfg->eps0 > 0))
            return fail(PICGB_ERR_INVALID, "cell sizes, dt, c and eps0 must be positive");
        double const cfl = cfg->c * cfg->c * cfg->dt * cfg->dt
            * (1.0 / (cfg->dx * cfg->dx) + 1.0 / (cfg->dy * cfg->dy) + 1.0 / (cfg->dz * cfg->dz));
        if(cfl > 1.0)
            return fail(PICGB_ERR_INVALID, "Courant-Friedrichs-Lewy condition violated (%g > 1)", cfl);
        int ndev = 0;
        CUDA_TRY(cudaGetDeviceCount(&ndev));
        if(cfg->device < 0 || cfg->device >= ndev)
            return fail(PICGB_ERR_INVALID, "CUDA device %d not present", int(cfg->device));
        CUDA_TRY(cudaSetDevice(cfg->device));
        auto* d = new picgb_diff();
        d->cfg = *cfg;
        d->g = DiffGridDesc{cfg->nx, cfg->ny, cfg->nz, cfg->dx, cfg->dy, cfg->dz, cfg->dt, cfg->c, cfg->eps0};
        d->prec = cfg->precision;
        d->esz = size_t(cfg->precision);
        d->nc = size_t(cfg->nx) * cfg->ny * cfg->nz;
        d->species.assign(species, species + nspecies);
        d->weights.assign(size_t(nspecies), nullptr);
        d->blobBytes = d->computeBlobBytes();
        if(cudaMalloc(&d->J, d->fieldBytes()) != cudaSuccess || cudaMalloc(&d->lamJ, d->fieldBytes()) != cudaSuccess)
        {
            picgb_diff_destroy(d);
            return fail(PICGB_ERR_CUDA, "allocation of the current buffers failed");
        }
        *out = d;
        return PICGB_OK;
    }

    int picgb_diff_destroy(picgb_diff* d)
    {
        if(!d)
            return PICGB_OK;
        cudaSetDevice(d->cfg.device);
        cudaDeviceSynchronize();
        for(void* p : d->ckpts)
            cudaFree(p);
        for(void* p : d->seg)
            cudaFree(p);
        for(void* p : d->gathered)
            cudaFree(p);
        if(d->fieldHist)
            cudaFree(d->fieldHist);
        if(d->J)
            cudaFree(d->J);
        if(d->lamJ)
            cudaFree(d->lamJ);
        delete d;
        return PICGB_OK;
    }

    int picgb_diff_forward(picgb_diff* d, picgb_diff_state* state, uint32_t nsteps, void* stream)
    {
        if(!d)
            return fail(PICGB_ERR_INVALID, "null handle");
        if(int r = checkState(d, state, false))
            return r;
        CUDA_TRY(cudaSetDevice(d->cfg.device));
        cudaStream_t const st = static_cast<cudaStream_t>(stream);
        for(size_t k = 0; k < d->species.size(); ++k)
            d->weights[k] = state->w[k];
        size_t const K = size_t(d->cfg.checkpoint_every);
        size_t const nckpt = nsteps == 0 ? 1 : (size_t(nsteps) + K - 1) / K;
        if(int r = ensureBlobs(d, nckpt))
            return r;
        StatePtrs const s = callerPtrs(d, state);
        d->denseFields = ensureFieldHistory(d, nsteps);
        for(uint32_t i = 0; i < nsteps; ++i)
        {
            if(i % K == 0)
                if(int r = copyState(d, d->blobPtrs(d->ckpts[i / K]), s, st))
                    return r;
            if(d->denseFields)
            {
                CUDA_TRY(cudaMemcpyAsync(d->histE(i), s.E, d->fieldBytes(), cudaMemcpyDeviceToDevice, st));
                CUDA_TRY(cudaMemcpyAsync(d->histB(i), s.B, d->fieldBytes(), cudaMemcpyDeviceToDevice, st));
            }
            if(int r = stepForward(d, s, s, st))
                return r;
        }
        d->nsteps = nsteps;
        d->haveForward = true;
        return PICGB_OK;
    }

    int picgb_diff_backward(picgb_diff* d, picgb_diff_state* grad, void* stream)
    {
        if(!d)
            return fail(PICGB_ERR_INVALID, "null handle");
        if(!d->haveForward)
            return fail(PICGB_ERR_INVALID, "backward needs a preceding forward");
        if(int r = checkState(d, grad, true))
            return r;
        CUDA_TRY(cudaSetDevice(d->cfg.device));
        cudaStream_t const st = static_cast<cudaStream_t>(stream);
        StatePtrs const lam = callerPtrs(d, grad);
        size_t const K = size_t(d->cfg.checkpoint_every);
        size_t const N = d->nsteps;
        if(N == 0)
            return PICGB_OK;
        for(size_t sidx = (N + K - 1) / K; sidx-- > 0;)
        {
            size_t const a = sidx * K, b = std::min(N, a + K);
            // replay the segment: each step reads the state of step i and writes that of step i + 1
            if(int r = copyState(d, d->blobPtrs(d->seg[0]), d->blobPtrs(d->ckpts[sidx]), st))
                return r;
            for(size_t i = a; i + 1 < b; ++i)
            {
                StatePtrs const in = d->blobPtrs(d->seg[i - a]), out = d->blobPtrs(d->seg[i - a + 1]);
                int const r = d->denseFields ? stepReplayParticles(d, i, in, out, st, d->gathered[i - a])
                                             : stepForward(d, in, out, st, d->gathered[i - a]);
                if(r)
                    return r;
            }
            // the last step of the segment was not replayed: its adjoint gathers the fields itself
            for(size_t i = b; i-- > a;)
            {
                StatePtrs s = d->blobPtrs(d->seg[i - a]);
                if(d->denseFields)
                {
                    s.E = d->histE(i);
                    s.B = d->histB(i);
                }
                if(int r = stepAdjoint(d, s, lam, st, i + 1 < b ? d->gathered[i - a] : nullptr))
                    return r;
            }
        }
        return PICGB_OK;
    }

    int picgb_diff_kinetic_energy(picgb_diff* d, const picgb_diff_state* state, int32_t species, double* out, void* stream)
    {
        if(!d || !out || species < 0 || species >= int32_t(d->species.size()))
            return fail(PICGB_ERR_INVALID, "invalid arguments");
        if(!state || !state->mom[species] || !state->w[species])
            return fail(PICGB_ERR_INVALID, "state needs mom and w of the species");
        cudaStream_t const st = static_cast<cudaStream_t>(stream);
        double* acc = nullptr;
        CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&acc), sizeof(double), st));
        CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(double), st));
        DiffSpeciesPtr const sp{
            nullptr,
            nullptr,
            state->mom[species],
            state->w[species],
            d->species[species].n,
            d->species[species].charge,
            d->species[species].mass};
        CUDA_TRY(launchDiffKinetic(d->prec, sp, d->g.c, acc, st));
        CUDA_TRY(cudaMemcpyAsync(out, acc, sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaFreeAsync(acc, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return PICGB_OK;
    }
}
