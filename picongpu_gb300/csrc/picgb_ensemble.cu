// Batched ensemble of independent periodic boxes (picgb_ensemble_* in picgb.h).
//
// Each box is an ordinary simulation handle: species upload/download, fields,
// diagnostics and the single-box step all go through the existing entry
// points.  The ensemble adds device tables that describe every box (fields,
// species storage, push parameters) and a batched step in which each kernel
// of the single-box step runs once over all boxes:
//   J = 0 (all boxes) -> one push launch over all (box, supercell) items per
//   species -> compaction per species -> B half, E (+J), B half (all boxes).
// The step is captured once as a CUDA graph and replayed; after every replay
// the status word is read so that an overflowing supercell is re-laid out
// before the next step, exactly as picgb_step does.
#include "picgb_batch.hpp"
#include "picgb_sim.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

using namespace picgb;
using namespace picgb::host;

struct picgb_ensemble
{
    picgb_ensemble_config cfg{};
    int threads = 256;
    std::vector<picgb_sim*> boxes;
    cudaStream_t stream = nullptr;
    // device tables (rebuilt before every run)
    BatchBox* dBoxes = nullptr;
    uint32_t* dBlockBox = nullptr;
    uint32_t nblocks = 0;
    BatchSpecies* dSpecies = nullptr; // [nspecies][nbox]
    size_t speciesSlots = 0;
    uint32_t* dItems = nullptr;
    uint32_t nitems = 0;
    uint32_t* dCounters = nullptr; // one work counter per species
    size_t counterSlots = 0;
    unsigned* dStatus = nullptr;
    unsigned* hStatus = nullptr;
    cudaGraphExec_t graph = nullptr;
    uint64_t kernelsPerStep = 0;
    std::vector<uint64_t> signature; // state of the boxes the tables and the graph were built from
    uint64_t launches = 0;
    uint32_t maxCap = 32; // largest slots per supercell of any box (shared memory of the reorder)
    std::vector<int> pushed; // species pushed in the batched step
    // interleaved order restored every sortInterval batched steps (0: never), as picgb_step does
    uint32_t sortInterval = 20;
    uint32_t stepsSinceSort = 0;
};

namespace
{
    int checkEns(picgb_ensemble* e)
    {
        if(!e)
            return fail(PICGB_ERR_INVALID, "null ensemble handle");
        return PICGB_OK;
    }

    void dropGraph(picgb_ensemble* e)
    {
        if(e->graph)
            cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
    }

    void freeTables(picgb_ensemble* e)
    {
        dfree(e->dBoxes);
        dfree(e->dBlockBox);
        dfree(e->dSpecies);
        dfree(e->dItems);
        dfree(e->dCounters);
        e->speciesSlots = e->counterSlots = 0;
    }

    int destroyEnsemble(picgb_ensemble* e)
    {
        cudaSetDevice(e->cfg.grid.device);
        if(e->stream)
            cudaStreamSynchronize(e->stream);
        dropGraph(e);
        freeTables(e);
        dfree(e->dStatus);
        if(e->hStatus)
            cudaFreeHost(e->hStatus);
        for(auto* b : e->boxes)
        {
            b->stream = nullptr; // the ensemble's stream, destroyed below
            b->ownStream = false;
            destroySim(b);
        }
        if(e->stream)
            cudaStreamDestroy(e->stream);
        delete e;
        return PICGB_OK;
    }

    size_t speciesCount(picgb_ensemble const* e) { return e->boxes.empty() ? 0 : e->boxes[0]->species.size(); }

    // What the device tables depend on: storage addresses, capacities and the
    // weighting bound (fixed-point J format) of every species of every box.
    std::vector<uint64_t> boxSignature(picgb_ensemble const* e)
    {
        std::vector<uint64_t> sig;
        for(auto const* b : e->boxes)
        {
            sig.push_back(b->species.size());
            for(auto const& sp : b->species)
            {
                uint32_t wbits = 0;
                std::memcpy(&wbits, &sp->wmax, sizeof(wbits));
                sig.push_back(uint64_t(reinterpret_cast<uintptr_t>(sp->dev.px)));
                sig.push_back((uint64_t(sp->dev.cap) << 33) | (uint64_t(wbits) << 1) | (sp->allocated ? 1u : 0u));
            }
        }
        return sig;
    }

    // Device tables of the current state of every box, and the step graph.
    int buildStep(picgb_ensemble* e)
    {
        size_t const nbox = e->boxes.size();
        size_t const nspec = speciesCount(e);
        for(auto* b : e->boxes)
            if(b->species.size() != nspec)
                return fail(PICGB_ERR_INVALID, "every box of an ensemble needs the same species");
        // fields: blocks of kBatchFieldThreads cells per box
        std::vector<BatchBox> hb(nbox);
        std::vector<uint32_t> blockBox;
        for(size_t i = 0; i < nbox; ++i)
        {
            picgb_sim* s = e->boxes[i];
            hb[i].g = s->g;
            hb[i].E = s->E;
            hb[i].B = s->B;
            hb[i].J = s->J;
            hb[i].coeffJ = s->coeffJ();
            hb[i].block0 = uint32_t(blockBox.size());
            size_t const nb = (s->ncell + kBatchFieldThreads - 1) / kBatchFieldThreads;
            blockBox.insert(blockBox.end(), nb, uint32_t(i));
        }
        // push work items: the boxes with the most particle slots per supercell first, so that
        // the blocks finish together
        std::vector<uint64_t> work(nbox, 0);
        uint32_t maxCap = 32;
        for(size_t i = 0; i < nbox; ++i)
            for(auto& sp : e->boxes[i]->species)
                if(sp->allocated)
                {
                    work[i] += sp->dev.cap;
                    maxCap = std::max(maxCap, sp->dev.cap);
                }
        std::vector<uint32_t> order(nbox);
        std::iota(order.begin(), order.end(), 0u);
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return work[a] > work[b]; });
        std::vector<uint32_t> items;
        for(uint32_t i : order)
            for(int sc = 0; sc < e->boxes[i]->nsc; ++sc)
                items.push_back(batchItem(i, uint32_t(sc)));
        // species tables; a species that is not allocated in a box has count = nullptr there and is skipped
        std::vector<BatchSpecies> hs(nspec * nbox);
        std::vector<int> pushed(nspec, 0);
        for(size_t k = 0; k < nspec; ++k)
        {
            bool allAllocated = true;
            for(size_t i = 0; i < nbox; ++i)
            {
                picgb_sim* s = e->boxes[i];
                Species& sp = *s->species[k];
                if(!sp.allocated)
                {
                    allAllocated = false;
                    continue;
                }
                BatchSpecies& t = hs[k * nbox + i];
                t.sp = sp.dev;
                t.pp = s->pushParams(sp, hasCurrent(sp));
                t.pp.kindCount = nullptr;
                t.g = s->g;
                t.E = s->E;
                t.B = s->B;
                t.J = s->J;
            }
            Species const& s0 = *e->boxes[0]->species[k];
            if(s0.cfg.pusher != PICGB_PUSHER_NONE)
            {
                if(!allAllocated)
                    return fail(PICGB_ERR_INVALID, "species '%s' has no particles in some box", s0.name.c_str());
                pushed[k] = 1;
            }
        }
        CUDA_TRY(cudaStreamSynchronize(e->stream));
        dropGraph(e);
        freeTables(e);
        CUDA_TRY(dalloc(e->dBoxes, nbox));
        CUDA_TRY(dalloc(e->dBlockBox, blockBox.size()));
        CUDA_TRY(dalloc(e->dSpecies, hs.size()));
        CUDA_TRY(dalloc(e->dItems, items.size()));
        CUDA_TRY(dalloc(e->dCounters, std::max<size_t>(nspec, 1)));
        e->speciesSlots = hs.size();
        e->counterSlots = std::max<size_t>(nspec, 1);
        e->nblocks = uint32_t(blockBox.size());
        e->nitems = uint32_t(items.size());
        CUDA_TRY(cudaMemcpyAsync(e->dBoxes, hb.data(), sizeof(BatchBox) * nbox, cudaMemcpyHostToDevice, e->stream));
        CUDA_TRY(cudaMemcpyAsync(
            e->dBlockBox,
            blockBox.data(),
            sizeof(uint32_t) * blockBox.size(),
            cudaMemcpyHostToDevice,
            e->stream));
        if(!hs.empty())
            CUDA_TRY(cudaMemcpyAsync(e->dSpecies, hs.data(), sizeof(BatchSpecies) * hs.size(), cudaMemcpyHostToDevice, e->stream));
        CUDA_TRY(cudaMemcpyAsync(e->dItems, items.data(), sizeof(uint32_t) * items.size(), cudaMemcpyHostToDevice, e->stream));
        CUDA_TRY(cudaStreamSynchronize(e->stream));

        // capture one step
        int const scId = e->cfg.grid.supercell;
        cudaGraph_t g = nullptr;
        // relaxed: the launchers query occupancy and set kernel attributes while capturing
        CUDA_TRY(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeRelaxed));
        uint64_t kernels = 0;
        cudaError_t err = cudaSuccess;
        auto launch = [&](cudaError_t r)
        {
            if(err == cudaSuccess)
                err = r;
        };
        launch(cudaMemsetAsync(e->dCounters, 0, sizeof(uint32_t) * e->counterSlots, e->stream));
        launch(launchZeroJBatch(e->dBoxes, e->dBlockBox, e->nblocks, e->stream));
        ++kernels;
        for(size_t k = 0; k < nspec; ++k)
            if(pushed[k])
            {
                picgb_sim const* b0 = e->boxes[0];
                auto const& cfg = b0->species[k]->cfg;
                // what every box shares, as kernel arguments; the table entries hold the rest
                PushParams const pp0 = hs[k * nbox].pp;
                launch(launchPushBatch(
                    cfg.shape,
                    scId,
                    e->threads,
                    cfg.pusher,
                    cfg.current,
                    e->dSpecies + k * nbox,
                    e->dItems,
                    e->nitems,
                    e->dCounters + k,
                    e->dStatus,
                    b0->g,
                    pp0,
                    e->stream));
                ++kernels;
            }
        for(size_t k = 0; k < nspec; ++k)
            if(pushed[k])
            {
                launch(launchCompactBatch(e->dSpecies + k * nbox, e->dItems, e->nitems, maxCap, e->stream));
                ++kernels;
            }
        // update_beforeCurrent with the fused J add, then update_afterCurrent (FDTD.hpp:69-110)
        launch(launchYeeBHalfBatch(e->dBoxes, e->dBlockBox, e->nblocks, e->stream));
        launch(launchYeeEBatch(e->dBoxes, e->dBlockBox, e->nblocks, e->stream));
        launch(launchYeeBHalfBatch(e->dBoxes, e->dBlockBox, e->nblocks, e->stream));
        kernels += 3;
        cudaError_t const endErr = cudaStreamEndCapture(e->stream, &g);
        if(err != cudaSuccess)
        {
            if(g)
                cudaGraphDestroy(g);
            return fail(PICGB_ERR_CUDA, "capturing the batched step failed: %s", cudaGetErrorString(err));
        }
        CUDA_TRY(endErr);
        cudaError_t const instErr = cudaGraphInstantiate(&e->graph, g, 0);
        cudaGraphDestroy(g);
        CUDA_TRY(instErr);
        e->kernelsPerStep = kernels;
        e->signature = boxSignature(e);
        e->maxCap = maxCap;
        e->pushed = pushed;
        return PICGB_OK;
    }

    // Every sortInterval batched steps: the interleaved order of every box's supercells.
    int reorderBatched(picgb_ensemble* e)
    {
        if(!e->sortInterval || ++e->stepsSinceSort < e->sortInterval)
            return PICGB_OK;
        e->stepsSinceSort = 0;
        int const* sc = e->boxes[0]->sc;
        int const vol = sc[0] * sc[1] * sc[2];
        if(reorderSmemBytes(vol, e->maxCap) > 200 * 1024)
            return PICGB_OK;
        size_t const nbox = e->boxes.size();
        for(size_t k = 0; k < e->pushed.size(); ++k)
            if(e->pushed[k])
            {
                CUDA_TRY(launchReorderBatch(e->dSpecies + k * nbox, e->dItems, e->nitems, vol, e->maxCap, e->stream));
                ++e->launches;
            }
        return PICGB_OK;
    }

    // After a batched step: route an overflow to the boxes whose spill buffers hold particles.
    int afterBatchedStep(picgb_ensemble* e)
    {
        CUDA_TRY(cudaMemcpyAsync(e->hStatus, e->dStatus, sizeof(unsigned), cudaMemcpyDeviceToHost, e->stream));
        CUDA_TRY(cudaStreamSynchronize(e->stream));
        unsigned const bits = *e->hStatus;
        if(bits == 0)
            return PICGB_OK;
        if(bits & ST_LOST)
            return fail(PICGB_ERR_LOST, "particles were lost: a spill buffer overflowed");
        if(bits & ST_BAD_CELL)
            return fail(PICGB_ERR_INVALID, "a particle had an out-of-range cell in the batched push");
        bool relaid = false;
        for(auto* b : e->boxes)
        {
            bool spilled = false;
            for(auto& sp : b->species)
            {
                if(!sp->allocated)
                    continue;
                uint32_t n = 0;
                CUDA_TRY(cudaMemcpy(&n, sp->dev.sp_count, sizeof(uint32_t), cudaMemcpyDeviceToHost));
                spilled = spilled || n > 0;
            }
            if(!spilled)
                continue;
            unsigned const ov = ST_OVERFLOW;
            CUDA_TRY(cudaMemcpyAsync(b->status, &ov, sizeof(unsigned), cudaMemcpyHostToDevice, e->stream));
            if(int r = afterStep(b))
                return r;
            relaid = true;
        }
        CUDA_TRY(cudaMemsetAsync(e->dStatus, 0, sizeof(unsigned), e->stream));
        CUDA_TRY(cudaStreamSynchronize(e->stream));
        if(relaid)
            return buildStep(e); // new storage pointers and capacities
        return PICGB_OK;
    }

    bool divides(int const* dims, int nbox, int scId)
    {
        int sc[3];
        if(!scSize(scId, sc))
            return false;
        for(int i = 0; i < nbox; ++i)
            for(int d = 0; d < 3; ++d)
                if(dims[3 * i + d] <= 0 || dims[3 * i + d] % sc[d])
                    return false;
        return true;
    }
} // namespace

extern "C"
{
    int picgb_ensemble_create(const picgb_ensemble_config* cfg, picgb_ensemble** out)
    {
        if(!cfg || !out)
            return fail(PICGB_ERR_INVALID, "null argument");
        *out = nullptr;
        if(cfg->nbox <= 0 || uint32_t(cfg->nbox) > kBatchMaxBoxes || !cfg->dims)
            return fail(PICGB_ERR_INVALID, "an ensemble needs 1 to %u boxes", kBatchMaxBoxes);
        int const threads = cfg->threads ? cfg->threads : 256;
        if(threads != 128 && threads != 256 && threads != 512)
            return fail(PICGB_ERR_INVALID, "threads per supercell must be 128, 256 or 512, not %d", threads);
        auto e = new picgb_ensemble();
        e->cfg = *cfg;
        e->cfg.dims = nullptr;
        e->threads = threads;
        auto bail = [&](int r)
        {
            destroyEnsemble(e);
            return r;
        };
        if(cudaSetDevice(cfg->grid.device) != cudaSuccess)
            return bail(fail(PICGB_ERR_INVALID, "CUDA device %d not present", int(cfg->grid.device)));
        if(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess
           || dalloc(e->dStatus, 1) != cudaSuccess
           || cudaMallocHost(reinterpret_cast<void**>(&e->hStatus), sizeof(unsigned)) != cudaSuccess
           || cudaMemsetAsync(e->dStatus, 0, sizeof(unsigned), e->stream) != cudaSuccess)
            return bail(fail(PICGB_ERR_CUDA, "ensemble set-up failed: %s", cudaGetErrorString(cudaGetLastError())));
        for(int i = 0; i < cfg->nbox; ++i)
        {
            picgb_grid_config g = cfg->grid;
            g.nx = cfg->dims[3 * i];
            g.ny = cfg->dims[3 * i + 1];
            g.nz = cfg->dims[3 * i + 2];
            g.fuse_deposit = 1; // the batched step deposits inside the push
            picgb_sim* s = nullptr;
            if(int r = picgb_create(&g, &s))
                return bail(r);
            if(s->nsc > int(kBatchMaxSc))
            {
                destroySim(s);
                return bail(fail(PICGB_ERR_INVALID, "box %d has more than %u supercells", i, kBatchMaxSc));
            }
            cudaStreamSynchronize(s->stream);
            cudaStreamDestroy(s->stream);
            s->stream = e->stream;
            s->ownStream = false;
            s->inEnsemble = true;
            e->boxes.push_back(s);
        }
        *out = e;
        return PICGB_OK;
    }

    int picgb_ensemble_destroy(picgb_ensemble* e)
    {
        if(!e)
            return PICGB_OK;
        return destroyEnsemble(e);
    }

    int picgb_ensemble_size(picgb_ensemble* e, int32_t* n)
    {
        if(int r = checkEns(e))
            return r;
        if(!n)
            return fail(PICGB_ERR_INVALID, "null argument");
        *n = int32_t(e->boxes.size());
        return PICGB_OK;
    }

    int picgb_ensemble_box(picgb_ensemble* e, int32_t box, picgb_sim** out)
    {
        if(int r = checkEns(e))
            return r;
        if(!out || box < 0 || box >= int32_t(e->boxes.size()))
            return fail(PICGB_ERR_INVALID, "box %d out of range", int(box));
        *out = e->boxes[box];
        return PICGB_OK;
    }

    int picgb_ensemble_add_species(picgb_ensemble* e, const picgb_species_config* cfg, int32_t* index)
    {
        if(int r = checkEns(e))
            return r;
        for(auto* b : e->boxes)
            if(int r = picgb_add_species(b, cfg, index))
                return r;
        dropGraph(e);
        return PICGB_OK;
    }

    int picgb_ensemble_init_plasma(picgb_ensemble* e, int32_t species, const picgb_plasma_init* perBox)
    {
        if(int r = checkEns(e))
            return r;
        if(!perBox)
            return fail(PICGB_ERR_INVALID, "null argument");
        for(size_t i = 0; i < e->boxes.size(); ++i)
            if(int r = picgb_species_init_plasma(e->boxes[i], species, perBox + i))
                return r;
        dropGraph(e);
        return PICGB_OK;
    }

    int picgb_ensemble_run(picgb_ensemble* e, uint32_t nsteps)
    {
        if(int r = checkEns(e))
            return r;
        CUDA_TRY(cudaSetDevice(e->cfg.grid.device));
        // the boxes may have been changed through their handles since the last run
        if(!e->graph || boxSignature(e) != e->signature)
            if(int r = buildStep(e))
                return r;
        for(uint32_t i = 0; i < nsteps; ++i)
        {
            CUDA_TRY(cudaGraphLaunch(e->graph, e->stream));
            e->launches += e->kernelsPerStep;
            if(int r = afterBatchedStep(e))
                return r;
            if(int r = reorderBatched(e))
                return r;
        }
        return PICGB_OK;
    }

    int picgb_ensemble_set_sort_interval(picgb_ensemble* e, uint32_t steps)
    {
        if(int r = checkEns(e))
            return r;
        e->sortInterval = steps;
        e->stepsSinceSort = 0;
        for(auto* b : e->boxes)
            if(int r = picgb_set_sort_interval(b, steps))
                return r;
        return PICGB_OK;
    }

    int picgb_ensemble_run_sequential(picgb_ensemble* e, uint32_t nsteps)
    {
        if(int r = checkEns(e))
            return r;
        for(auto* b : e->boxes)
            if(int r = picgb_run(b, 0, nsteps))
                return r;
        return PICGB_OK;
    }

    int picgb_ensemble_launch_count(picgb_ensemble* e, uint64_t* n)
    {
        if(int r = checkEns(e))
            return r;
        if(!n)
            return fail(PICGB_ERR_INVALID, "null argument");
        *n = e->launches;
        return PICGB_OK;
    }

    int picgb_ensemble_autotune(
        const picgb_ensemble_config* cfg,
        int32_t nspecies,
        const picgb_species_config* species,
        const picgb_plasma_init* inits,
        uint32_t warmup,
        uint32_t steps,
        int32_t* bestSupercell,
        int32_t* bestThreads,
        double* rates)
    {
        if(!cfg || !cfg->dims || cfg->nbox <= 0 || nspecies <= 0 || !species || !inits || !bestSupercell || !bestThreads
           || steps == 0)
            return fail(PICGB_ERR_INVALID, "autotune needs a config, species, their inits and steps > 0");
        static int const cand[PICGB_AUTOTUNE_CANDIDATES][2]
            = {{0, 128}, {0, 256}, {0, 512}, {1, 128}, {1, 256}, {1, 512}, {2, 128}, {2, 256}, {2, 512}};
        double best = -1.0;
        for(int c = 0; c < PICGB_AUTOTUNE_CANDIDATES; ++c)
        {
            if(rates)
                rates[c] = 0.0;
            if(!divides(cfg->dims, cfg->nbox, cand[c][0]))
                continue;
            picgb_ensemble_config tc = *cfg;
            tc.grid.supercell = cand[c][0];
            tc.threads = cand[c][1];
            picgb_ensemble* e = nullptr;
            if(int r = picgb_ensemble_create(&tc, &e))
                return r;
            int r = PICGB_OK;
            for(int32_t s = 0; s < nspecies && r == PICGB_OK; ++s)
            {
                int32_t idx = 0;
                r = picgb_ensemble_add_species(e, species + s, &idx);
                if(r == PICGB_OK)
                    r = picgb_ensemble_init_plasma(e, idx, inits + size_t(s) * cfg->nbox);
            }
            if(r == PICGB_OK && warmup)
                r = picgb_ensemble_run(e, warmup);
            double rate = 0.0;
            if(r == PICGB_OK)
            {
                uint64_t parts = 0;
                for(auto* b : e->boxes)
                    for(size_t s = 0; s < b->species.size(); ++s)
                    {
                        uint64_t n = 0;
                        if(b->species[s]->cfg.pusher != PICGB_PUSHER_NONE && picgb_species_count(b, int32_t(s), &n) == PICGB_OK)
                            parts += n;
                    }
                cudaEvent_t a = nullptr, z = nullptr;
                cudaEventCreate(&a);
                cudaEventCreate(&z);
                cudaEventRecord(a, e->stream);
                r = picgb_ensemble_run(e, steps);
                cudaEventRecord(z, e->stream);
                cudaEventSynchronize(z);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, a, z);
                cudaEventDestroy(a);
                cudaEventDestroy(z);
                if(r == PICGB_OK && ms > 0.0f)
                    rate = double(parts) * steps / (ms * 1e-3);
            }
            picgb_ensemble_destroy(e);
            if(r != PICGB_OK)
                return r;
            if(rates)
                rates[c] = rate;
            if(rate > best)
            {
                best = rate;
                *bestSupercell = cand[c][0];
                *bestThreads = cand[c][1];
            }
        }
        if(best <= 0.0)
            return fail(PICGB_ERR_INVALID, "no candidate supercell divides every box");
        return PICGB_OK;
    }
}
