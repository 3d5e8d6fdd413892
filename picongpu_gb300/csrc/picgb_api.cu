// Host runtime behind the C-ABI of include/picgb.h: the simulation handle,
// the DataConnector-style registry, species upload/download, the stage
// sequence of one PIC step and the diagnostics.
#include "picgb_sim.hpp"
#include "picgb_init.hpp"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

using namespace picgb;
using namespace picgb::host;

namespace picgb::host
{
    namespace
    {
        thread_local std::string g_lastError;
    }

    int fail(int code, char const* fmt, ...)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        g_lastError = buf;
        return code;
    }
} // namespace picgb::host

PushParams picgb_sim::pushParams(Species const& s, bool deposit) const
{
    PushParams p{};
    p.charge = s.cfg.charge;
    p.mass = s.cfg.mass;
    p.dt = cfg.dt;
    p.c2 = cfg.c * cfg.c;
    p.rc2 = 1.0f / (cfg.c * cfg.c);
    float const vdt = cellVolume() * cfg.dt;
    p.invVdt = 1.0f / vdt;
    p.c = cfg.c;
    p.pusher = s.cfg.pusher;
    p.current = s.cfg.current;
    p.deposit = deposit ? 1 : 0;
    p.kindCount = prof ? kindCount : nullptr;
    // Fixed-point format of the J tile (kernels built with PICGB_J_FIXED).  A
    // deposited value is a running sum acc_k = sum DS * tmp with
    // |tmp| <= |q w| d / (V dt) and sum |DS| <= 2, so |acc| <= 2 |q| wmax dmax / (V dt)
    // =: vmax.  A tile node receives at most one value per particle of its
    // supercell (at most 2^cb).  With k = min(31 - cb, 22) and
    // vmax * 2^s <= 2^min(61 - 2 cb, k + 21), a high part stays within 2^21 and a low
    // part within 2^(k - 1), and the sums of either over 2^cb values stay in int32.
    int cb = 1;
    while((1u << cb) < s.dev.cap)
        ++cb;
    double const dmax = std::max(std::max(double(cfg.dx), double(cfg.dy)), double(cfg.dz));
    double const vmax = 2.0 * std::fabs(double(s.cfg.charge)) * double(s.wmax) * dmax * double(p.invVdt);
    int e = 0;
    if(vmax > 0.0 && std::isfinite(vmax))
        std::frexp(vmax, &e); // vmax < 2^e
    int const k = std::min(31 - cb, 22);
    int const sExp = std::min(std::max(std::min(61 - 2 * cb, k + 21) - e, -126), 126);
    p.jf.k = k;
    p.jf.scale = std::ldexp(1.0f, sExp);
    p.jf.invScale = std::ldexp(1.0f, -sExp);
    p.jf.hiStep = std::ldexp(1.0f, -k);
    p.jf.hiUnit = std::ldexp(1.0f, k);
    return p;
}

namespace picgb::host
{
    int checkSim(picgb_sim* s)
    {
        if(!s)
            return fail(PICGB_ERR_INVALID, "null simulation handle");
        return PICGB_OK;
    }

    int checkSpecies(picgb_sim* s, int32_t i)
    {
        if(int r = checkSim(s))
            return r;
        if(i < 0 || i >= int32_t(s->species.size()))
            return fail(PICGB_ERR_INVALID, "species index %d out of range", int(i));
        return PICGB_OK;
    }

    cudaError_t takeEvent(picgb_sim* s, cudaEvent_t* e)
    {
        if(!s->eventPool.empty())
        {
            *e = s->eventPool.back();
            s->eventPool.pop_back();
            return cudaSuccess;
        }
        return cudaEventCreate(e);
    }

    // Launch one kernel through `launch`, bracketed by events when profiling is on.
    template<typename F>
    cudaError_t timedLaunch(picgb_sim* s, int cls, F&& launch)
    {
        ++s->launches;
        if(!s->prof)
            return launch();
        picgb_sim::Pending p{cls, nullptr, nullptr};
        cudaError_t e = takeEvent(s, &p.a);
        if(e == cudaSuccess)
            e = takeEvent(s, &p.b);
        if(e == cudaSuccess)
            e = cudaEventRecord(p.a, s->stream);
        if(e != cudaSuccess)
            return e;
        e = launch();
        if(e != cudaSuccess)
            return e;
        e = cudaEventRecord(p.b, s->stream);
        s->pending.push_back(p);
        return e;
    }

    // Transverse extent of an incident-field face: a periodic transverse axis in full, an open one
    // between its absorbers.  Along its own axis the surface must keep out of the absorber, as
    // incidentField::detail::checkRequirements demands (Solver.hpp:113-168: the offset of the
    // Huygens surface from an open boundary at least the absorber thickness).
    int incidentExtent(picgb_sim* s, IncidentParams& p)
    {
        int const cells[3] = {s->cfg.nx, s->cfg.ny, s->cfg.nz};
        int const a = p.axis;
        if((s->g.open >> a) & 1)
        {
            // low face: POSITION >= thickness, surface = POSITION + 1; high face: cells - POSITION
            // >= thickness, surface = POSITION - 1
            bool const inside = p.dir > 0 ? p.plane < s->absorberThick[a][0] + 1
                                          : p.plane > cells[a] - 1 - s->absorberThick[a][1];
            if(inside)
                return fail(PICGB_ERR_INVALID, "incident-field surface %d on axis %d lies in the absorber (%d + %d cells)",
                            p.plane, a, s->absorberThick[a][0], s->absorberThick[a][1]);
        }
        int const tr[2] = {a == 0 ? 1 : 0, a == 2 ? 1 : 2};
        for(int q = 0; q < 2; ++q)
        {
            int const d = tr[q];
            bool const open = (s->g.open >> d) & 1;
            p.lo[q] = open ? s->absorberThick[d][0] : 0;
            p.hi[q] = open ? cells[d] - s->absorberThick[d][1] : cells[d];
        }
        return PICGB_OK;
    }

    // The incident-field correction of every enabled face: the B planes on the scattered side
    // (bField) or the E planes on the total side.
    int launchIncident(picgb_sim* s, bool bField, float t)
    {
        for(auto const& face : s->inc)
        {
            if(!face.enabled)
                continue;
            IncidentParams p = face;
            if(int r = incidentExtent(s, p))
                return r;
            CUDA_TRY(bField ? launchIncidentB(s->B, s->g, p, t, s->stream) : launchIncidentE(s->E, s->g, p, t, s->stream));
        }
        return PICGB_OK;
    }

    // Accumulate the completed event pairs (call after a stream synchronisation).
    cudaError_t profFlush(picgb_sim* s)
    {
        for(auto& p : s->pending)
        {
            float ms = 0.0f;
            cudaError_t e = cudaEventElapsedTime(&ms, p.a, p.b);
            if(e != cudaSuccess)
                return e;
            s->profMs[p.cls] += ms;
            s->profN[p.cls] += 1;
            s->eventPool.push_back(p.a);
            s->eventPool.push_back(p.b);
        }
        s->pending.clear();
        return cudaSuccess;
    }

    void fieldDesc(picgb_sim const* s, float* base, int ncomp, picgb_buffer_desc* d)
    {
        std::memset(d, 0, sizeof(*d));
        d->kind = PICGB_BUFFER_FIELD;
        d->ncomp = ncomp;
        for(int c = 0; c < ncomp; ++c)
            d->ptr[c] = base + c * s->ncell;
        d->dims[0] = s->cfg.nx;
        d->dims[1] = s->cfg.ny;
        d->dims[2] = s->cfg.nz;
        d->stride[0] = 1;
        d->stride[1] = s->cfg.nx;
        d->stride[2] = int64_t(s->cfg.nx) * s->cfg.ny;
        d->elem_bytes = 4;
        d->layout = 0;
    }

    void speciesDesc(picgb_sim const* s, Species const& sp, picgb_buffer_desc* d)
    {
        std::memset(d, 0, sizeof(*d));
        d->kind = PICGB_BUFFER_SPECIES;
        d->ncomp = 10;
        void* p[10] = {sp.dev.px, sp.dev.py, sp.dev.pz, sp.dev.ux, sp.dev.uy, sp.dev.uz, sp.dev.w, sp.dev.lcell,
                       sp.dev.id, sp.dev.count};
        for(int i = 0; i < 10; ++i)
            d->ptr[i] = p[i];
        d->dims[0] = s->g.nscx;
        d->dims[1] = s->g.nscy;
        d->dims[2] = s->g.nscz;
        d->stride[0] = 1;
        d->stride[1] = s->g.nscx;
        d->stride[2] = int64_t(s->g.nscx) * s->g.nscy;
        d->elem_bytes = 4;
        d->capacity = sp.dev.cap;
        d->layout = 0;
    }

    int addEntry(picgb_sim* s, std::string const& name, Entry e)
    {
        if(s->registry.count(name))
            return fail(PICGB_ERR_DUPLICATE, "DataConnector: id '%s' is already registered", name.c_str());
        s->registry.emplace(name, e);
        return PICGB_OK;
    }

    // Allocate the supercell-major storage of a species with `cap` slots per supercell.
    int allocSpecies(picgb_sim* s, Species& sp, uint32_t cap)
    {
        sp.freeAll();
        size_t const n = size_t(s->nsc) * cap;
        SpeciesDev& d = sp.dev;
        d.cap = cap;
        CUDA_TRY(dalloc(d.px, n));
        CUDA_TRY(dalloc(d.py, n));
        CUDA_TRY(dalloc(d.pz, n));
        CUDA_TRY(dalloc(d.ux, n));
        CUDA_TRY(dalloc(d.uy, n));
        CUDA_TRY(dalloc(d.uz, n));
        CUDA_TRY(dalloc(d.w, n));
        CUDA_TRY(dalloc(d.lcell, n));
        if(sp.cfg.with_ids)
            CUDA_TRY(dalloc(d.id, n));
        CUDA_TRY(dalloc(d.count, size_t(s->nsc)));
        CUDA_TRY(dalloc(d.tail, size_t(s->nsc)));
        CUDA_TRY(dalloc(d.nhole, size_t(s->nsc)));
        CUDA_TRY(dalloc(d.holes, n));
        // spill buffer: 1/64 of the slots, at least 4096
        d.spill_cap = uint32_t(std::max<size_t>(4096, n / 64));
        CUDA_TRY(dalloc(d.sp_attr, size_t(7) * d.spill_cap));
        CUDA_TRY(dalloc(d.sp_sc, size_t(d.spill_cap)));
        CUDA_TRY(dalloc(d.sp_lcell, size_t(d.spill_cap)));
        CUDA_TRY(dalloc(d.sp_id, size_t(d.spill_cap)));
        CUDA_TRY(dalloc(d.sp_count, 1));
        CUDA_TRY(dalloc(sp.leaveCount, size_t(128)));
        CUDA_TRY(cudaMemsetAsync(sp.leaveCount, 0, sizeof(unsigned long long) * 128, s->stream));
        CUDA_TRY(cudaMemsetAsync(d.count, 0, sizeof(uint32_t) * s->nsc, s->stream));
        CUDA_TRY(cudaMemsetAsync(d.tail, 0, sizeof(uint32_t) * s->nsc, s->stream));
        CUDA_TRY(cudaMemsetAsync(d.nhole, 0, sizeof(uint32_t) * s->nsc, s->stream));
        CUDA_TRY(cudaMemsetAsync(d.sp_count, 0, sizeof(uint32_t), s->stream));
        sp.nsc = s->nsc;
        sp.allocated = true;
        return PICGB_OK;
    }

    // Contiguous device copy of particles in the host exchange format.
    // Device arrays of n particles in the host exchange format, carved out of the simulation's
    // staging buffer, which grows when needed and is kept for the next upload or download (a
    // fresh cudaMalloc and cudaFree of several GB per call cost more than the copies).
    struct Staging
    {
        float* a[7] = {};
        int32_t* sc = nullptr;
        uint16_t* lcell = nullptr;
        uint32_t* id = nullptr;
        uint64_t n = 0;

        cudaError_t alloc(picgb_sim* s, uint64_t count, bool ids)
        {
            n = count;
            auto part = [&](size_t bytes) { return (bytes + 255) / 256 * 256; };
            size_t const need = 7 * part(sizeof(float) * count) + part(sizeof(int32_t) * count)
                + part(sizeof(uint16_t) * count) + (ids ? part(sizeof(uint32_t) * count) : 0);
            if(need > s->ioBytes)
            {
                if(s->ioBuf)
                {
                    cudaError_t e = cudaStreamSynchronize(s->stream);
                    if(e != cudaSuccess)
                        return e;
                    cudaFree(s->ioBuf);
                }
                s->ioBuf = nullptr;
                s->ioBytes = 0;
                cudaError_t e = cudaMalloc(&s->ioBuf, need);
                if(e != cudaSuccess)
                {
                    s->ioBuf = nullptr;
                    return e;
                }
                s->ioBytes = need;
            }
            char* b = static_cast<char*>(s->ioBuf);
            for(auto& p : a)
            {
                p = reinterpret_cast<float*>(b);
                b += part(sizeof(float) * count);
            }
            sc = reinterpret_cast<int32_t*>(b);
            b += part(sizeof(int32_t) * count);
            lcell = reinterpret_cast<uint16_t*>(b);
            b += part(sizeof(uint16_t) * count);
            id = ids ? reinterpret_cast<uint32_t*>(b) : nullptr;
            return cudaSuccess;
        }
    };

    // Device address of host memory that kernels can write directly (page-locked memory
    // registered with CUDA, e.g. from cudaHostAlloc), or nullptr (pageable memory).
    template<typename T>
    T* deviceView(T* host)
    {
        if(!host)
            return nullptr;
        cudaPointerAttributes at{};
        if(cudaPointerGetAttributes(&at, host) != cudaSuccess)
        {
            cudaGetLastError();
            return nullptr;
        }
        return at.type == cudaMemoryTypeHost ? static_cast<T*>(at.devicePointer) : nullptr;
    }

    int readStatus(picgb_sim* s, unsigned* bits, bool reset)
    {
        CUDA_TRY(cudaMemcpyAsync(s->hostStatus, s->status, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        *bits = *s->hostStatus;
        if(reset && *bits)
            CUDA_TRY(cudaMemsetAsync(s->status, 0, sizeof(unsigned), s->stream));
        return PICGB_OK;
    }

    // Grow the per-supercell capacity and re-insert the particles parked in the
    // spill buffer (the reference would abort on an exhausted frame heap).
    int relayout(picgb_sim* s, Species& sp, double growth)
    {
        std::vector<uint32_t> cnt(s->nsc);
        uint32_t spill = 0;
        CUDA_TRY(cudaMemcpyAsync(cnt.data(), sp.dev.count, sizeof(uint32_t) * s->nsc, cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaMemcpyAsync(&spill, sp.dev.sp_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        spill = std::min(spill, sp.dev.spill_cap);
        std::vector<uint64_t> off(s->nsc);
        uint64_t total = 0;
        for(int i = 0; i < s->nsc; ++i)
        {
            off[i] = total;
            total += cnt[i];
        }
        Staging st;
        CUDA_TRY(st.alloc(s, total + spill, sp.cfg.with_ids != 0));
        uint64_t* doff = nullptr;
        CUDA_TRY(dalloc(doff, size_t(s->nsc)));
        CUDA_TRY(cudaMemcpyAsync(doff, off.data(), sizeof(uint64_t) * s->nsc, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(launchGatherOut(sp.dev, s->nsc, doff, total, st.a, st.sc, st.lcell, st.id, s->stream));
        ++s->launches;
        size_t const C = sp.dev.spill_cap;
        for(int k = 0; k < 7; ++k)
            CUDA_TRY(cudaMemcpyAsync(
                st.a[k] + total,
                sp.dev.sp_attr + k * C,
                sizeof(float) * spill,
                cudaMemcpyDeviceToDevice,
                s->stream));
        CUDA_TRY(cudaMemcpyAsync(st.sc + total, sp.dev.sp_sc, sizeof(int32_t) * spill, cudaMemcpyDeviceToDevice, s->stream));
        CUDA_TRY(cudaMemcpyAsync(
            st.lcell + total,
            sp.dev.sp_lcell,
            sizeof(uint16_t) * spill,
            cudaMemcpyDeviceToDevice,
            s->stream));
        if(st.id)
            CUDA_TRY(
                cudaMemcpyAsync(st.id + total, sp.dev.sp_id, sizeof(uint32_t) * spill, cudaMemcpyDeviceToDevice, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        dfree(doff);
        // histogram of the new occupancy
        uint32_t* hcount = nullptr;
        CUDA_TRY(dalloc(hcount, size_t(s->nsc)));
        CUDA_TRY(cudaMemsetAsync(hcount, 0, sizeof(uint32_t) * s->nsc, s->stream));
        CUDA_TRY(launchHistogram(
            s->cfg.supercell,
            total + spill,
            st.sc,
            st.lcell,
            nullptr,
            hcount,
            s->nsc,
            s->status,
            s->stream));
        ++s->launches;
        CUDA_TRY(cudaMemcpyAsync(cnt.data(), hcount, sizeof(uint32_t) * s->nsc, cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        dfree(hcount);
        uint32_t mx = *std::max_element(cnt.begin(), cnt.end());
        uint64_t want = std::max<uint64_t>(uint64_t(std::ceil(mx * growth)), sp.dev.cap + 32);
        want = (want + 31) / 32 * 32;
        if(want > 65504)
            return fail(PICGB_ERR_OVERFLOW, "species '%s': %u particles in one supercell exceed the slot limit",
                        sp.name.c_str(), mx);
        if(int r = allocSpecies(s, sp, uint32_t(want)))
            return r;
        float const* attr[7] = {st.a[0], st.a[1], st.a[2], st.a[3], st.a[4], st.a[5], st.a[6]};
        CUDA_TRY(launchScatter(total + spill, attr, st.sc, st.lcell, st.id, sp.dev, s->status, s->stream));
        ++s->launches;
        CUDA_TRY(cudaMemcpyAsync(sp.dev.tail, sp.dev.count, sizeof(uint32_t) * s->nsc, cudaMemcpyDeviceToDevice, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        return PICGB_OK;
    }

    // A set overflow bit in the status word `bits` means that arrivals were parked in the
    // spill buffer; they are re-inserted with a larger capacity before anything else reads
    // the particles.  ST_LOST is an error.
    int reinsertSpilled(picgb_sim* s, unsigned bits)
    {
        if(bits & ST_LOST)
            return fail(PICGB_ERR_LOST, "particles were lost: the spill buffer overflowed");
        if(bits & ST_OVERFLOW)
        {
            for(auto& sp : s->species)
            {
                uint32_t spill = 0;
                CUDA_TRY(cudaMemcpy(&spill, sp->dev.sp_count, sizeof(uint32_t), cudaMemcpyDeviceToHost));
                if(spill)
                    if(int r = relayout(s, *sp, 1.25))
                        return r;
            }
            CUDA_TRY(cudaMemsetAsync(s->status, 0, sizeof(unsigned), s->stream));
        }
        return PICGB_OK;
    }

    // Fraction of a species' particles that left their supercell in a step, above which the
    // step compacts it with the compacting reorder (kCompactReorder) every step instead of
    // hole filling (kCompact): hole filling moves each arrival with scattered 4-byte accesses,
    // and a sort that visits every particle once restores the interleaved order as well.
    constexpr double kHotLeaveFraction = 0.03;

    // The counters of the compacting reorders of the last step (the stream is synchronised):
    // the species' leave fraction decides whether the next steps sort it every step.
    int readLeaveCounts(picgb_sim* s)
    {
        for(auto& sp : s->species)
        {
            if(!sp->allocated || !sp->counted)
                continue;
            unsigned long long c[128];
            CUDA_TRY(cudaMemcpy(c, sp->leaveCount, sizeof(c), cudaMemcpyDeviceToHost));
            CUDA_TRY(cudaMemsetAsync(sp->leaveCount, 0, sizeof(c), s->stream));
            unsigned long long left = 0, kept = 0;
            for(int i = 0; i < 64; ++i)
            {
                left += c[2 * i];
                kept += c[2 * i + 1];
            }
            sp->hot = double(left) > kHotLeaveFraction * double(left + kept);
            sp->counted = false;
        }
        return PICGB_OK;
    }

    // After a step: the profiling events are read and spilled arrivals re-inserted.
    int afterStep(picgb_sim* s)
    {
        unsigned bits = 0;
        if(int r = readStatus(s, &bits, false))
            return r;
        CUDA_TRY(profFlush(s));
        if(int r = readLeaveCounts(s))
            return r;
        return reinsertSpilled(s, bits);
    }

    // The status word read and spilled arrivals re-inserted (synchronises the stream).
    int settleParticles(picgb_sim* s)
    {
        unsigned bits = 0;
        if(int r = readStatus(s, &bits, false))
            return r;
        if(int r = readLeaveCounts(s))
            return r;
        return reinsertSpilled(s, bits);
    }

    bool hasCurrent(Species const& sp)
    {
        return sp.cfg.current == PICGB_CURRENT_ESIRKEPOV || sp.cfg.current == PICGB_CURRENT_EMZ;
    }

    // The push kernel of every pushed species (with the fused deposit), then their compaction.
    int pushLaunches(picgb_sim* s)
    {
        bool const fuse = s->cfg.fuse_deposit != 0;
        for(auto& sp : s->species)
        {
            if(!sp->allocated || sp->cfg.pusher == PICGB_PUSHER_NONE)
                continue;
            PushParams const pp = s->pushParams(*sp, fuse && hasCurrent(*sp));
            Species& x = *sp;
            CUDA_TRY(timedLaunch(s, PICGB_KERNEL_PUSH, [&] {
                return launchPush(x.cfg.shape, s->cfg.supercell, x.dev, s->E, s->B, s->J, s->g, pp, s->status, s->stream);
            }));
        }
        // compaction: every sortInterval steps, every step for a species that leaves its
        // supercells often, and in the first step after a device plasma initialisation (to
        // measure that), by the compacting reorder (it also restores the interleaved order);
        // otherwise by hole filling
        bool const sortStep = s->sortInterval && ++s->stepsSinceSort >= s->sortInterval;
        if(sortStep)
            s->stepsSinceSort = 0;
        int const vol = s->sc[0] * s->sc[1] * s->sc[2];
        for(auto& sp : s->species)
        {
            if(!sp->allocated || sp->cfg.pusher == PICGB_PUSHER_NONE)
                continue;
            Species& x = *sp;
            bool const canSort = s->sortInterval && reorderSmemBytes(vol, x.dev.cap) <= 200 * 1024;
            if(canSort && (sortStep || x.hot || x.probe))
            {
                x.probe = false;
                CUDA_TRY(timedLaunch(s, PICGB_KERNEL_REORDER, [&] {
                    return launchCompactReorder(x.dev, s->nsc, vol, x.leaveCount, s->stream);
                }));
                x.counted = true;
            }
            else
                CUDA_TRY(timedLaunch(s, PICGB_KERNEL_COMPACT, [&] { return launchCompact(x.dev, s->nsc, s->stream); }));
        }
        return PICGB_OK;
    }
} // namespace

extern "C"
{
    int picgb_abi_version(void) { return PICGB_ABI_VERSION; }

    const char* picgb_last_error(void) { return g_lastError.c_str(); }

    int picgb_create(const picgb_grid_config* cfg, picgb_sim** out)
    {
        if(!cfg || !out)
            return fail(PICGB_ERR_INVALID, "null argument");
        *out = nullptr;
        int sc[3];
        if(!scSize(cfg->supercell, sc))
            return fail(PICGB_ERR_INVALID, "unknown supercell id %d", int(cfg->supercell));
        if(cfg->nx <= 0 || cfg->ny <= 0 || cfg->nz <= 0 || cfg->nx % sc[0] || cfg->ny % sc[1] || cfg->nz % sc[2])
            return fail(PICGB_ERR_INVALID, "grid %dx%dx%d is not a positive multiple of the supercell %dx%dx%d",
                        int(cfg->nx), int(cfg->ny), int(cfg->nz), sc[0], sc[1], sc[2]);
        if(cfg->field_solver != PICGB_SOLVER_YEE)
            return fail(PICGB_ERR_UNSUPPORTED, "field solver %d is not available", int(cfg->field_solver));
        if(!(cfg->dx > 0 && cfg->dy > 0 && cfg->dz > 0 && cfg->dt > 0 && cfg->c > 0 && cfg->eps0 > 0))
            return fail(PICGB_ERR_INVALID, "cell sizes, dt, c and eps0 must be positive");
        // Courant-Friedrichs-Lewy condition of the Yee solver (MaxwellSolver/Yee/Yee.hpp:57-63)
        double const cfl = double(cfg->c) * cfg->c * double(cfg->dt) * cfg->dt
            * (1.0 / (double(cfg->dx) * cfg->dx) + 1.0 / (double(cfg->dy) * cfg->dy) + 1.0 / (double(cfg->dz) * cfg->dz));
        if(cfl > 1.0)
            return fail(PICGB_ERR_INVALID, "Courant-Friedrichs-Lewy condition violated: c^2 dt^2 sum 1/d^2 = %g > 1", cfl);
        int ndev = 0;
        CUDA_TRY(cudaGetDeviceCount(&ndev));
        if(cfg->device < 0 || cfg->device >= ndev)
            return fail(PICGB_ERR_INVALID, "CUDA device %d not present (%d devices)", int(cfg->device), ndev);
        CUDA_TRY(cudaSetDevice(cfg->device));

        auto s = std::make_unique<picgb_sim>();
        s->cfg = *cfg;
        std::copy(sc, sc + 3, s->sc);
        s->g.nx = cfg->nx;
        s->g.ny = cfg->ny;
        s->g.nz = cfg->nz;
        s->g.nscx = cfg->nx / sc[0];
        s->g.nscy = cfg->ny / sc[1];
        s->g.nscz = cfg->nz / sc[2];
        s->g.dx = cfg->dx;
        s->g.dy = cfg->dy;
        s->g.dz = cfg->dz;
        s->g.dt = cfg->dt;
        s->g.c = cfg->c;
        s->g.eps0 = cfg->eps0;
        // cell sizes that are powers of two divide exactly as a multiplication by their reciprocal
        auto pow2 = [](float v)
        {
            int e = 0;
            return std::frexp(v, &e) == 0.5f;
        };
        s->g.rd[0] = 1.0f / cfg->dx;
        s->g.rd[1] = 1.0f / cfg->dy;
        s->g.rd[2] = 1.0f / cfg->dz;
        s->g.recipExact = (pow2(cfg->dx) && pow2(cfg->dy) && pow2(cfg->dz)) ? 1 : 0;
        s->nsc = s->g.nscx * s->g.nscy * s->g.nscz;
        s->ncell = size_t(cfg->nx) * cfg->ny * cfg->nz;
        CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->ownStream = true;
        CUDA_TRY(dalloc(s->E, 3 * s->ncell));
        CUDA_TRY(dalloc(s->B, 3 * s->ncell));
        CUDA_TRY(dalloc(s->J, 3 * s->ncell));
        CUDA_TRY(dalloc(s->rho, s->ncell));
        CUDA_TRY(dalloc(s->status, 1));
        CUDA_TRY(dalloc(s->energy, 64));
        CUDA_TRY(dalloc(s->maxBits, 2));
        CUDA_TRY(dalloc(s->kindCount, 2));
        CUDA_TRY(cudaMemsetAsync(s->kindCount, 0, 2 * sizeof(unsigned long long), s->stream));
        CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&s->hostStatus), sizeof(unsigned)));
        CUDA_TRY(cudaMemsetAsync(s->E, 0, sizeof(float) * 3 * s->ncell, s->stream));
        CUDA_TRY(cudaMemsetAsync(s->B, 0, sizeof(float) * 3 * s->ncell, s->stream));
        CUDA_TRY(cudaMemsetAsync(s->J, 0, sizeof(float) * 3 * s->ncell, s->stream));
        CUDA_TRY(cudaMemsetAsync(s->rho, 0, sizeof(float) * s->ncell, s->stream));
        CUDA_TRY(cudaMemsetAsync(s->status, 0, sizeof(unsigned), s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        // DataConnector registrations of Simulation::init (Simulation.hpp:324-339, 740-753)
        addEntry(s.get(), "E", Entry{Entry::FieldE});
        addEntry(s.get(), "B", Entry{Entry::FieldB});
        addEntry(s.get(), "J", Entry{Entry::FieldJ});
        addEntry(s.get(), "FieldTmp0", Entry{Entry::FieldTmp});
        addEntry(s.get(), "FieldSolverFDTD", Entry{Entry::Opaque});
        addEntry(s.get(), "CurrentInterpolationAndAdditionToEMF", Entry{Entry::Opaque});
        *out = s.release();
        return PICGB_OK;
    }

    int picgb_destroy(picgb_sim* s)
    {
        if(!s)
            return PICGB_OK;
        if(s->inEnsemble)
            return fail(PICGB_ERR_INVALID, "the handle belongs to an ensemble; destroy the ensemble instead");
        return destroySim(s);
    }
}

int picgb::host::destroySim(picgb_sim* s)
{
    cudaSetDevice(s->cfg.device);
    if(s->stream)
        cudaStreamSynchronize(s->stream);
    for(auto& sp : s->species)
        sp->freeAll();
    dfree(s->E);
    dfree(s->B);
    dfree(s->J);
    dfree(s->rho);
    dfree(s->status);
    dfree(s->energy);
    dfree(s->maxBits);
    dfree(s->kindCount);
    dfree(s->pml.psiE);
    dfree(s->pml.psiB);
    dfree(s->pmlTab);
    dfree(s->expDamp);
    if(s->ioBuf)
        cudaFree(s->ioBuf);
    if(s->hostStatus)
        cudaFreeHost(s->hostStatus);
    profFlush(s);
    for(auto e : s->eventPool)
        cudaEventDestroy(e);
    if(s->ownStream && s->stream)
        cudaStreamDestroy(s->stream);
    delete s;
    return PICGB_OK;
}

extern "C"
{
    int picgb_add_species(picgb_sim* s, const picgb_species_config* cfg, int32_t* index)
    {
        if(int r = checkSim(s))
            return r;
        if(!cfg || !cfg->name || !cfg->name[0])
            return fail(PICGB_ERR_INVALID, "species needs a name");
        if(cfg->pusher < PICGB_PUSHER_BORIS || cfg->pusher > PICGB_PUSHER_PHOTON)
            return fail(PICGB_ERR_INVALID, "unknown pusher %d", int(cfg->pusher));
        if(cfg->shape < PICGB_SHAPE_CIC || cfg->shape > PICGB_SHAPE_PCS)
            return fail(PICGB_ERR_UNSUPPORTED, "shape %d has no CUDA kernel (CIC, TSC, PQS, PCS are available)",
                        int(cfg->shape));
        if(cfg->current < PICGB_CURRENT_NONE || cfg->current > PICGB_CURRENT_EMZ)
            return fail(PICGB_ERR_INVALID, "unknown current solver %d", int(cfg->current));
        // massless species (photons, massRatio 0) only with a pusher that does not divide by the mass
        bool const massless = cfg->pusher == PICGB_PUSHER_PHOTON || cfg->pusher == PICGB_PUSHER_FREE
            || cfg->pusher == PICGB_PUSHER_NONE;
        if(!(cfg->mass > 0.0f) && !(massless && cfg->mass == 0.0f))
            return fail(PICGB_ERR_INVALID, "species mass must be positive (0 only with the Photon, Free or no pusher)");
        if(cfg->capacity > 65504)
            return fail(PICGB_ERR_INVALID, "capacity %u exceeds 65504 slots per supercell", cfg->capacity);
        auto sp = std::make_unique<Species>();
        sp->name = cfg->name;
        sp->cfg = *cfg;
        sp->cfg.name = nullptr;
        Entry e{Entry::SpeciesBuf};
        e.index = int(s->species.size());
        if(int r = addEntry(s, sp->name, e))
            return r;
        s->species.push_back(std::move(sp));
        if(index)
            *index = e.index;
        return PICGB_OK;
    }

    int picgb_species_set(picgb_sim* s, int32_t si, const picgb_particles* h)
    {
        if(int r = checkSpecies(s, si))
            return r;
        if(!h)
            return fail(PICGB_ERR_INVALID, "null particle descriptor");
        Species& sp = *s->species[si];
        uint64_t const n = h->n;
        if(n && (!h->pos[0] || !h->pos[1] || !h->pos[2] || !h->mom[0] || !h->mom[1] || !h->mom[2] || !h->w || !h->sc
                 || !h->lcell))
            return fail(PICGB_ERR_INVALID, "particle arrays must not be null");
        CUDA_TRY(cudaSetDevice(s->cfg.device));
        Staging st;
        CUDA_TRY(st.alloc(s, n, sp.cfg.with_ids != 0 && h->id));
        float const* src[7] = {h->pos[0], h->pos[1], h->pos[2], h->mom[0], h->mom[1], h->mom[2], h->w};
        // page-locked host arrays are read by a copy kernel over the host link (SM loads, as the
        // download writes); other host memory goes through cudaMemcpyAsync
        CopyJobs jobs{};
        bool zeroCopy = n > 0;
        auto add = [&](void* dst, void const* hostSrc, size_t bytes)
        {
            void* const dv = deviceView(const_cast<void*>(hostSrc));
            zeroCopy = zeroCopy && dv != nullptr;
            jobs.s[jobs.n++] = CopySeg{dst, dv, bytes};
        };
        for(int k = 0; k < 7; ++k)
            add(st.a[k], src[k], sizeof(float) * n);
        add(st.sc, h->sc, sizeof(int32_t) * n);
        add(st.lcell, h->lcell, sizeof(uint16_t) * n);
        if(st.id)
            add(st.id, h->id, sizeof(uint32_t) * n);
        if(zeroCopy)
        {
            CUDA_TRY(launchCopyIn(jobs, s->stream));
            ++s->launches;
        }
        else
        {
            for(int k = 0; k < 7; ++k)
                CUDA_TRY(cudaMemcpyAsync(st.a[k], src[k], sizeof(float) * n, cudaMemcpyHostToDevice, s->stream));
            CUDA_TRY(cudaMemcpyAsync(st.sc, h->sc, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s->stream));
            CUDA_TRY(cudaMemcpyAsync(st.lcell, h->lcell, sizeof(uint16_t) * n, cudaMemcpyHostToDevice, s->stream));
            if(st.id)
                CUDA_TRY(cudaMemcpyAsync(st.id, h->id, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s->stream));
        }
        // per-supercell counts, and in the last word the bits of the largest |w|
        uint32_t* hcount = nullptr;
        CUDA_TRY(dalloc(hcount, size_t(s->nsc) + 1));
        CUDA_TRY(cudaMemsetAsync(hcount, 0, sizeof(uint32_t) * (s->nsc + 1), s->stream));
        CUDA_TRY(cudaMemsetAsync(s->status, 0, sizeof(unsigned), s->stream));
        float const* pos3[3] = {st.a[0], st.a[1], st.a[2]};
        CUDA_TRY(launchHistogram(s->cfg.supercell, n, st.sc, st.lcell, pos3, hcount, s->nsc, s->status, s->stream));
        CUDA_TRY(launchMaxAbsBits(st.a[6], n, hcount + s->nsc, s->stream));
        s->launches += 2;
        std::vector<uint32_t> cnt(s->nsc + 1);
        CUDA_TRY(cudaMemcpyAsync(cnt.data(), hcount, sizeof(uint32_t) * (s->nsc + 1), cudaMemcpyDeviceToHost, s->stream));
        unsigned bits = 0;
        if(int r = readStatus(s, &bits, true))
        {
            dfree(hcount);
            return r;
        }
        dfree(hcount);
        if(bits & ST_BAD_CELL)
            return fail(PICGB_ERR_INVALID, "species '%s': a particle has an out-of-range supercell, cell index or in-cell position",
                        sp.name.c_str());
        unsigned const wbits = cnt[s->nsc];
        cnt.pop_back();
        uint32_t const mx = cnt.empty() ? 0u : *std::max_element(cnt.begin(), cnt.end());
        if(wbits >= 0x7F800000u) // infinity or NaN
            return fail(PICGB_ERR_INVALID, "species '%s': a weighting is not finite", sp.name.c_str());
        float wmax;
        std::memcpy(&wmax, &wbits, sizeof(wmax));
        sp.wmax = wmax;
        uint32_t cap = sp.cfg.capacity;
        if(cap == 0)
            cap = uint32_t(std::max<uint64_t>(32, uint64_t(std::ceil(1.25 * mx))));
        cap = (cap + 31) / 32 * 32;
        if(cap > 65504)
            return fail(PICGB_ERR_OVERFLOW, "species '%s': %u particles per supercell exceed the slot limit",
                        sp.name.c_str(), mx);
        if(mx > cap)
            return fail(PICGB_ERR_OVERFLOW, "species '%s': a supercell holds %u particles, capacity is %u",
                        sp.name.c_str(), mx, cap);
        if(!sp.allocated || sp.dev.cap != cap)
        {
            if(int r = allocSpecies(s, sp, cap))
                return r;
        }
        else
        {
            CUDA_TRY(cudaMemsetAsync(sp.dev.count, 0, sizeof(uint32_t) * s->nsc, s->stream));
            CUDA_TRY(cudaMemsetAsync(sp.dev.nhole, 0, sizeof(uint32_t) * s->nsc, s->stream));
            CUDA_TRY(cudaMemsetAsync(sp.dev.sp_count, 0, sizeof(uint32_t), s->stream));
        }
        float const* attr[7] = {st.a[0], st.a[1], st.a[2], st.a[3], st.a[4], st.a[5], st.a[6]};
        CUDA_TRY(launchScatter(n, attr, st.sc, st.lcell, st.id, sp.dev, s->status, s->stream));
        ++s->launches;
        CUDA_TRY(cudaMemcpyAsync(sp.dev.tail, sp.dev.count, sizeof(uint32_t) * s->nsc, cudaMemcpyDeviceToDevice, s->stream));
        // the scatter's slots follow the arrival of its atomics: give the particles the interleaved
        // cell order the push's tiles are laid out for, as the periodic reorder does
        int const vol = s->sc[0] * s->sc[1] * s->sc[2];
        if(s->sortInterval && sp.cfg.pusher != PICGB_PUSHER_NONE && reorderSmemBytes(vol, sp.dev.cap) <= 200 * 1024)
        {
            CUDA_TRY(launchReorder(sp.dev, s->nsc, vol, s->stream));
            ++s->launches;
        }
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        return PICGB_OK;
    }

    int picgb_species_init_plasma(picgb_sim* s, int32_t si, const picgb_plasma_init* init)
    {
        if(int r = checkSpecies(s, si))
            return r;
        if(!init)
            return fail(PICGB_ERR_INVALID, "null plasma init");
        bool const quiet = init->quiet[0] || init->quiet[1] || init->quiet[2];
        uint64_t const lattice = uint64_t(init->quiet[0]) * init->quiet[1] * init->quiet[2];
        if(quiet && (lattice == 0 || lattice > 65504 || (init->ppc != 0 && init->ppc != lattice)))
            return fail(PICGB_ERR_INVALID, "quiet start %ux%ux%u: every axis needs particles, and ppc must be 0 or "
                        "their product", unsigned(init->quiet[0]), unsigned(init->quiet[1]), unsigned(init->quiet[2]));
        uint32_t const ppc = quiet ? uint32_t(lattice) : init->ppc;
        if(ppc == 0)
            return fail(PICGB_ERR_INVALID, "plasma init needs ppc > 0");
        if(init->split_axis > 2 || !(init->u_th >= 0.0f) || !(init->density >= 0.0f))
            return fail(PICGB_ERR_INVALID, "invalid plasma init parameters");
        Species& sp = *s->species[si];
        CUDA_TRY(cudaSetDevice(s->cfg.device));
        uint64_t const perSc = uint64_t(ppc) * s->sc[0] * s->sc[1] * s->sc[2];
        uint64_t cap = sp.cfg.capacity ? sp.cfg.capacity : uint64_t(std::ceil(1.25 * perSc));
        cap = (std::max<uint64_t>(cap, 32) + 31) / 32 * 32;
        if(cap < perSc || cap > 65504)
            return fail(PICGB_ERR_OVERFLOW, "species '%s': %llu particles per supercell do not fit %llu slots (max 65504)",
                        sp.name.c_str(), (unsigned long long) perSc, (unsigned long long) cap);
        if(!sp.allocated || sp.dev.cap != cap)
        {
            if(int r = allocSpecies(s, sp, uint32_t(cap)))
                return r;
        }
        InitParams ip{};
        ip.ppc = ppc;
        ip.weight = init->density * s->cellVolume() / float(ppc);
        sp.wmax = std::fabs(ip.weight);
        ip.mass = sp.cfg.mass;
        ip.c = s->cfg.c;
        ip.u_th = init->u_th;
        for(int d = 0; d < 3; ++d)
        {
            ip.drift_lo[d] = init->drift_lo[d];
            ip.drift_hi[d] = init->drift_hi[d];
        }
        ip.split_axis = init->split_axis;
        ip.split_cell = init->split_cell;
        ip.seed = init->seed;
        ip.position_seed = init->position_seed;
        for(int d = 0; d < 3; ++d)
            ip.quiet[d] = quiet ? init->quiet[d] : 0u;
        CUDA_TRY(cudaMemsetAsync(sp.dev.sp_count, 0, sizeof(uint32_t), s->stream));
        CUDA_TRY(launchInitPlasma(sp.dev, s->g, ip, s->sc, s->stream));
        ++s->launches;
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        sp.probe = true; // a new plasma: its first step measures how fast it leaves its supercells
        sp.hot = false;
        return PICGB_OK;
    }

    int picgb_species_count(picgb_sim* s, int32_t si, uint64_t* n)
    {
        if(int r = checkSpecies(s, si))
            return r;
        Species& sp = *s->species[si];
        *n = 0;
        if(!sp.allocated)
            return PICGB_OK;
        std::vector<uint32_t> cnt(s->nsc);
        CUDA_TRY(cudaMemcpyAsync(cnt.data(), sp.dev.count, sizeof(uint32_t) * s->nsc, cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        uint64_t t = 0;
        for(auto c : cnt)
            t += c;
        *n = t;
        return PICGB_OK;
    }

    int picgb_species_get(picgb_sim* s, int32_t si, picgb_particles* h)
    {
        if(int r = checkSpecies(s, si))
            return r;
        Species& sp = *s->species[si];
        if(!sp.allocated)
        {
            h->n = 0;
            return PICGB_OK;
        }
        std::vector<uint32_t> cnt(s->nsc);
        CUDA_TRY(cudaMemcpyAsync(cnt.data(), sp.dev.count, sizeof(uint32_t) * s->nsc, cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        std::vector<uint64_t> off(s->nsc);
        uint64_t total = 0;
        for(int i = 0; i < s->nsc; ++i)
        {
            off[i] = total;
            total += cnt[i];
        }
        if(h->n < total)
            return fail(PICGB_ERR_INVALID, "host arrays hold %llu particles, %llu needed",
                        (unsigned long long) h->n, (unsigned long long) total);
        uint64_t* doff = nullptr;
        CUDA_TRY(dalloc(doff, size_t(s->nsc)));
        CUDA_TRY(cudaMemcpyAsync(doff, off.data(), sizeof(uint64_t) * s->nsc, cudaMemcpyHostToDevice, s->stream));
        float* dst[7] = {h->pos[0], h->pos[1], h->pos[2], h->mom[0], h->mom[1], h->mom[2], h->w};
        // page-locked host arrays: the gather kernel writes them directly over the host link
        float* direct[7];
        bool zeroCopy = true;
        for(int k = 0; k < 7; ++k)
            zeroCopy = zeroCopy && (direct[k] = deviceView(dst[k])) != nullptr;
        int32_t* dsc = deviceView(h->sc);
        uint16_t* dlc = deviceView(h->lcell);
        uint32_t* did = deviceView(h->id);
        zeroCopy = zeroCopy && dsc && dlc && (!h->id || did);
        if(zeroCopy)
        {
            CUDA_TRY(launchGatherOut(sp.dev, s->nsc, doff, total, direct, dsc, dlc, did, s->stream));
            ++s->launches;
        }
        else
        {
            Staging st;
            CUDA_TRY(st.alloc(s, total, h->id != nullptr));
            CUDA_TRY(launchGatherOut(sp.dev, s->nsc, doff, total, st.a, st.sc, st.lcell, st.id, s->stream));
            ++s->launches;
            for(int k = 0; k < 7; ++k)
                CUDA_TRY(cudaMemcpyAsync(dst[k], st.a[k], sizeof(float) * total, cudaMemcpyDeviceToHost, s->stream));
            CUDA_TRY(cudaMemcpyAsync(h->sc, st.sc, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, s->stream));
            CUDA_TRY(cudaMemcpyAsync(h->lcell, st.lcell, sizeof(uint16_t) * total, cudaMemcpyDeviceToHost, s->stream));
            if(h->id)
                CUDA_TRY(cudaMemcpyAsync(h->id, st.id, sizeof(uint32_t) * total, cudaMemcpyDeviceToHost, s->stream));
        }
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        dfree(doff);
        h->n = total;
        return PICGB_OK;
    }

    static int fieldPtr(picgb_sim* s, const char* name, float** p, int* ncomp)
    {
        if(!name)
            return fail(PICGB_ERR_INVALID, "null field name");
        std::string const n(name);
        if(n == "E")
            *p = s->E, *ncomp = 3;
        else if(n == "B")
            *p = s->B, *ncomp = 3;
        else if(n == "J")
            *p = s->J, *ncomp = 3;
        else if(n == "FieldTmp0")
            *p = s->rho, *ncomp = 1;
        else
            return fail(PICGB_ERR_NOT_FOUND, "DataConnector: unknown field id '%s'", name);
        return PICGB_OK;
    }

    int picgb_field_set(picgb_sim* s, const char* name, const float* const* host)
    {
        if(int r = checkSim(s))
            return r;
        float* p = nullptr;
        int nc = 0;
        if(int r = fieldPtr(s, name, &p, &nc))
            return r;
        for(int c = 0; c < nc; ++c)
            CUDA_TRY(cudaMemcpyAsync(p + c * s->ncell, host[c], sizeof(float) * s->ncell, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        return PICGB_OK;
    }

    int picgb_field_get(picgb_sim* s, const char* name, float* const* host)
    {
        if(int r = checkSim(s))
            return r;
        float* p = nullptr;
        int nc = 0;
        if(int r = fieldPtr(s, name, &p, &nc))
            return r;
        for(int c = 0; c < nc; ++c)
            CUDA_TRY(cudaMemcpyAsync(host[c], p + c * s->ncell, sizeof(float) * s->ncell, cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        return PICGB_OK;
    }

    // ------------------------------------------------------------ registry
    int picgb_get_buffer(picgb_sim* s, const char* name, picgb_buffer_desc* out)
    {
        if(int r = checkSim(s))
            return r;
        if(!name || !out)
            return fail(PICGB_ERR_INVALID, "null argument");
        auto it = s->registry.find(name);
        if(it == s->registry.end())
            return fail(PICGB_ERR_NOT_FOUND, "DataConnector: unknown id '%s'", name);
        Entry const& e = it->second;
        switch(e.kind)
        {
        case Entry::FieldE:
            fieldDesc(s, s->E, 3, out);
            break;
        case Entry::FieldB:
            fieldDesc(s, s->B, 3, out);
            break;
        case Entry::FieldJ:
            fieldDesc(s, s->J, 3, out);
            break;
        case Entry::FieldTmp:
            fieldDesc(s, s->rho, 1, out);
            break;
        case Entry::SpeciesBuf:
            speciesDesc(s, *s->species[e.index], out);
            break;
        case Entry::Opaque:
            std::memset(out, 0, sizeof(*out));
            out->kind = PICGB_BUFFER_OPAQUE;
            break;
        case Entry::External:
            *out = e.desc;
            break;
        }
        return PICGB_OK;
    }

    int picgb_share(picgb_sim* s, const char* name, const picgb_buffer_desc* desc)
    {
        if(int r = checkSim(s))
            return r;
        if(!name || !name[0] || !desc)
            return fail(PICGB_ERR_INVALID, "null argument");
        Entry e{Entry::External};
        e.desc = *desc;
        return addEntry(s, name, e);
    }

    int picgb_unshare(picgb_sim* s, const char* name)
    {
        if(int r = checkSim(s))
            return r;
        auto it = s->registry.find(name ? name : "");
        if(it == s->registry.end())
            return fail(PICGB_ERR_NOT_FOUND, "DataConnector: unknown id '%s'", name ? name : "(null)");
        if(it->second.kind != Entry::External)
            return fail(PICGB_ERR_INVALID, "DataConnector: '%s' is owned by the simulation", name);
        s->registry.erase(it);
        return PICGB_OK;
    }

    int picgb_registry_size(picgb_sim* s, int32_t* n)
    {
        if(int r = checkSim(s))
            return r;
        *n = int32_t(s->registry.size());
        return PICGB_OK;
    }

    int picgb_registry_name(picgb_sim* s, int32_t i, char* buf, size_t len)
    {
        if(int r = checkSim(s))
            return r;
        if(i < 0 || i >= int32_t(s->registry.size()) || !buf || len == 0)
            return fail(PICGB_ERR_INVALID, "registry index %d out of range", int(i));
        auto it = s->registry.begin();
        std::advance(it, i);
        std::snprintf(buf, len, "%s", it->first.c_str());
        return PICGB_OK;
    }

    // ------------------------------------------------------------ stages
    int picgb_stage_current_reset(picgb_sim* s)
    {
        if(int r = checkSim(s))
            return r;
        CUDA_TRY(cudaMemsetAsync(s->J, 0, sizeof(float) * 3 * s->ncell, s->stream));
        return PICGB_OK;
    }

    int picgb_stage_push(picgb_sim* s, uint32_t)
    {
        if(int r = checkSim(s))
            return r;
        if(int r = pushLaunches(s))
            return r;
        // arrivals parked in the spill buffer go back into the supercells before a
        // later stage or a download reads the particles
        return settleParticles(s);
    }

    int picgb_stage_field_before(picgb_sim* s, uint32_t step)
    {
        if(int r = checkSim(s))
            return r;
        float const t = float(double(step) * s->cfg.dt);
        // the second half of the B update (FDTDBase.hpp:166-226): PML convolution fields unchanged
        CUDA_TRY(timedLaunch(s, PICGB_KERNEL_YEE_B, [&] {
            return s->g.open ? launchYeeBHalfOpen(s->E, s->B, s->g, s->pml, false, s->stream)
                             : launchYeeBHalf(s->E, s->B, s->g, s->stream);
        }));
        if(int r = launchIncident(s, true, t)) // incident E at t (Solver.hpp:500-533)
            return r;
        // with the fused deposit J is complete here: E += curl B c^2 dt and E += coeff J in one pass
        float const* J = s->cfg.fuse_deposit ? s->J : nullptr;
        CUDA_TRY(timedLaunch(s, PICGB_KERNEL_YEE_E, [&] {
            return s->g.open ? launchYeeEOpen(s->B, s->E, J, s->coeffJ(), s->g, s->pml, s->stream)
                             : launchYeeE(s->B, s->E, J, s->coeffJ(), s->g, s->stream);
        }));
        if(int r = launchIncident(s, false, t + 0.5f * s->cfg.dt)) // incident B at t + dt/2
            return r;
        if(s->expDamp) // exponential absorber on E (FDTDBase.hpp:121-124)
            CUDA_TRY(launchAbsorbExponential(s->E, s->g, s->expDamp, s->pml.nmax, s->stream));
        return PICGB_OK;
    }

    int picgb_stage_deposit(picgb_sim* s, uint32_t)
    {
        if(int r = checkSim(s))
            return r;
        if(s->cfg.fuse_deposit)
            return PICGB_OK;
        for(auto& sp : s->species)
        {
            if(!sp->allocated || !hasCurrent(*sp))
                continue;
            PushParams const pp = s->pushParams(*sp, true);
            Species& x = *sp;
            CUDA_TRY(timedLaunch(s, PICGB_KERNEL_DEPOSIT, [&] {
                return launchDeposit(x.cfg.shape, s->cfg.supercell, x.dev, s->J, s->g, pp, s->status, s->stream);
            }));
        }
        return PICGB_OK;
    }

    int picgb_stage_add_current(picgb_sim* s)
    {
        if(int r = checkSim(s))
            return r;
        if(s->cfg.fuse_deposit)
            return PICGB_OK; // folded into the E update of picgb_stage_field_before
        CUDA_TRY(timedLaunch(
            s,
            PICGB_KERNEL_ADD_CURRENT,
            [&] { return launchAddCurrent(s->E, s->J, s->coeffJ(), s->ncell, s->stream); }));
        return PICGB_OK;
    }

    int picgb_stage_field_after(picgb_sim* s, uint32_t step)
    {
        if(int r = checkSim(s))
            return r;
        // the first half of the B update: the PML convolution fields advance (FDTDBase.hpp:199-208)
        CUDA_TRY(timedLaunch(s, PICGB_KERNEL_YEE_B, [&] {
            return s->g.open ? launchYeeBHalfOpen(s->E, s->B, s->g, s->pml, true, s->stream)
                             : launchYeeBHalf(s->E, s->B, s->g, s->stream);
        }));
        if(int r = launchIncident(s, true, float(double(step + 1) * s->cfg.dt))) // incident E at t + dt
            return r;
        if(s->expDamp) // exponential absorber on B (FDTDBase.hpp:178-182)
            CUDA_TRY(launchAbsorbExponential(s->B, s->g, s->expDamp, s->pml.nmax, s->stream));
        return PICGB_OK;
    }

    int picgb_set_boundaries(picgb_sim* s, const picgb_boundary_config* b)
    {
        if(int r = checkSim(s))
            return r;
        if(!b)
            return fail(PICGB_ERR_INVALID, "null boundary config");
        if(s->inEnsemble)
            return fail(PICGB_ERR_UNSUPPORTED, "the boxes of an ensemble are periodic");
        int const cells[3] = {s->cfg.nx, s->cfg.ny, s->cfg.nz};
        float const edge[3] = {s->cfg.dx, s->cfg.dy, s->cfg.dz};
        double const m = b->grading_order, ma = b->alpha_grading_order;
        PmlAxis ax[3];
        int open = 0;
        for(int a = 0; a < 3; ++a)
        {
            if(b->open[a] != 0 && b->open[a] != 1)
                return fail(PICGB_ERR_INVALID, "open[%d] must be 0 or 1", a);
            if(b->absorber != PICGB_ABSORBER_PML && b->absorber != PICGB_ABSORBER_EXPONENTIAL)
                return fail(PICGB_ERR_INVALID, "unknown absorber %d", int(b->absorber));
            if(!b->open[a])
                continue;
            int const neg = b->thickness[a][0], pos = b->thickness[a][1];
            if(neg < 0 || pos < 0 || neg + pos > cells[a])
                return fail(PICGB_ERR_INVALID, "absorber of %d + %d cells does not fit %d cells on axis %d", neg, pos,
                            cells[a], a);
            if(!(b->strength[a][0] >= 0.0f) || !(b->strength[a][1] >= 0.0f))
                return fail(PICGB_ERR_INVALID, "exponential absorber strengths must be >= 0");
            if(!(m >= 0.0) || !(ma >= 0.0) || !(b->kappa_max[a] >= 1.0f) || !(b->alpha_max[a] >= 0.0f))
                return fail(PICGB_ERR_INVALID, "PML needs grading orders >= 0, kappa_max >= 1 and alpha_max >= 0");
            ax[a].open = true;
            ax[a].cells = cells[a];
            bool const pml = b->absorber == PICGB_ABSORBER_PML;
            ax[a].neg = pml ? neg : 0; // without PML layers the open Yee update is the plain one
            ax[a].pos = pml ? pos : 0;
            // default sigma: SIGMA_OPT = 0.8 (m + 1) / (Z0 d), normalized by eps0: 0.8 (m + 1) c / d
            ax[a].sigmaMax = b->sigma_max[a] < 0.0f ? 0.8 * (m + 1.0) * double(s->cfg.c) / double(edge[a])
                                                     : double(b->sigma_max[a]);
            ax[a].kappaMax = b->kappa_max[a];
            ax[a].alphaMax = b->alpha_max[a];
            ax[a].order = m;
            ax[a].alphaOrder = ma;
            open |= 1 << a;
        }
        for(int a = 0; a < 3; ++a)
            for(int side = 0; side < 2; ++side)
                s->absorberThick[a][side] = b->open[a] ? int(b->thickness[a][side]) : 0;
        CUDA_TRY(cudaSetDevice(s->cfg.device));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        dfree(s->pml.psiE);
        dfree(s->pml.psiB);
        dfree(s->pmlTab);
        dfree(s->expDamp);
        s->pml = PmlDev{};
        s->g.open = 0; // set below once the PML state exists
        if(!open)
            return PICGB_OK;
        int const nmax = std::max(cells[0], std::max(cells[1], cells[2]));
        std::vector<float> const tab = pmlTables(ax, double(s->cfg.dt), nmax);
        CUDA_TRY(dalloc(s->pmlTab, tab.size()));
        CUDA_TRY(cudaMemcpy(s->pmlTab, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice));
        if(b->absorber == PICGB_ABSORBER_PML)
        {
            CUDA_TRY(dalloc(s->pml.psiE, 6 * s->ncell));
            CUDA_TRY(dalloc(s->pml.psiB, 6 * s->ncell));
            CUDA_TRY(cudaMemsetAsync(s->pml.psiE, 0, sizeof(float) * 6 * s->ncell, s->stream));
            CUDA_TRY(cudaMemsetAsync(s->pml.psiB, 0, sizeof(float) * 6 * s->ncell, s->stream));
        }
        else
        {
            std::vector<float> const damp = expDampTable(cells, b->thickness, b->strength, open, nmax);
            CUDA_TRY(dalloc(s->expDamp, damp.size()));
            CUDA_TRY(cudaMemcpy(s->expDamp, damp.data(), sizeof(float) * damp.size(), cudaMemcpyHostToDevice));
        }
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        s->pml.tab = s->pmlTab;
        s->pml.nmax = nmax;
        s->g.open = open;
        return PICGB_OK;
    }

    int picgb_set_incident_field(picgb_sim* s, const picgb_incident_field* f)
    {
        if(int r = checkSim(s))
            return r;
        if(!f)
        {
            for(auto& face : s->inc)
                face = IncidentParams{};
            return PICGB_OK;
        }
        int const dir = f->direction == 0 ? 1 : f->direction;
        if(f->axis < 0 || f->axis > 2 || (dir != 1 && dir != -1))
            return fail(PICGB_ERR_INVALID, "incident field: axis %d must be 0, 1 or 2 and direction %d +1 or -1",
                        int(f->axis), int(f->direction));
        int const face = 2 * f->axis + (dir < 0 ? 1 : 0);
        if(!f->enabled)
        {
            s->inc[face] = IncidentParams{};
            return PICGB_OK;
        }
        if(s->inEnsemble)
            return fail(PICGB_ERR_UNSUPPORTED, "the batched step of an ensemble has no incident field");
        int const cells[3] = {s->cfg.nx, s->cfg.ny, s->cfg.nz};
        int const n = cells[f->axis];
        int const lo = dir > 0 ? 1 : 0, hi = n - 1; // the scattered-side B plane exists: surface - 1 or surface
        if(f->surface < lo || f->surface > hi)
            return fail(PICGB_ERR_INVALID, "incident-field surface %d outside %d..%d on axis %d", int(f->surface), lo, hi,
                        int(f->axis));
        if(!(f->wavelength > 0.0f && f->waist > 0.0f && f->duration_fwhm > 0.0f) || (f->polarisation != 0 && f->polarisation != 1))
            return fail(PICGB_ERR_INVALID, "incident field needs positive wavelength, waist, duration and polarisation 0 or 1");
        if(!(f->focus == f->focus))
            return fail(PICGB_ERR_INVALID, "incident field: focus is not a number");
        IncidentParams p{};
        p.enabled = 1;
        p.axis = f->axis;
        p.dir = dir;
        p.plane = f->surface;
        double const edge[3] = {s->cfg.dx, s->cfg.dy, s->cfg.dz};
        double const da = edge[f->axis];
        int const t1 = f->axis == 0 ? 1 : 0, t2 = f->axis == 2 ? 1 : 2;
        // propagation direction and polarisation (BaseParam.def DIRECTION_*, POLARISATION_DIRECTION_*)
        double dv[3] = {0.0, 0.0, 0.0}, pv[3] = {0.0, 0.0, 0.0};
        bool const oblique = f->propagation[0] != 0.0f || f->propagation[1] != 0.0f || f->propagation[2] != 0.0f;
        bool const polGiven = f->polarisation_vector[0] != 0.0f || f->polarisation_vector[1] != 0.0f
            || f->polarisation_vector[2] != 0.0f;
        for(int a = 0; a < 3; ++a)
        {
            dv[a] = oblique ? double(f->propagation[a]) : (a == f->axis ? double(dir) : 0.0);
            pv[a] = polGiven ? double(f->polarisation_vector[a]) : (a == (f->polarisation == 0 ? t1 : t2) ? 1.0 : 0.0);
        }
        double const dn = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
        double const pn = pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2];
        double const dp = dv[0] * pv[0] + dv[1] * pv[1] + dv[2] * pv[2];
        if(!(std::fabs(dn - 1.0) < 1e-4) || !(std::fabs(pn - 1.0) < 1e-4))
            return fail(PICGB_ERR_INVALID, "incident field: propagation and polarisation vectors must be unit vectors");
        if(!(std::fabs(dp) < 1e-4))
            return fail(PICGB_ERR_INVALID, "incident field: the polarisation must be orthogonal to the propagation");
        if(!(dv[f->axis] * dir > 1e-3))
            return fail(PICGB_ERR_INVALID, "incident field: the propagation must enter the box through the face");
        if(f->circular != 0 && f->circular != 1)
            return fail(PICGB_ERR_INVALID, "incident field: circular must be 0 or 1");
        double const qv[3] = {dv[1] * pv[2] - dv[2] * pv[1], dv[2] * pv[0] - dv[0] * pv[2], dv[0] * pv[1] - dv[1] * pv[0]};
        p.circular = f->circular;
        for(int a = 0; a < 3; ++a)
        {
            p.d[a] = float(dv[a]);
            p.pol[a] = float(pv[a]);
            p.pol2[a] = float(qv[a]);
        }
        for(int a = 0; a < 3; ++a)
            p.pv1[a] = f->circular ? p.pol[a] / std::sqrt(2.0f) : p.pol[a];
        for(int a = 0; a < 3; ++a) // d x pv1 (getCircularPolarizationVector2)
        {
            int const b = (a + 1) % 3, c = (a + 2) % 3;
            p.pv2[a] = f->circular ? p.d[b] * p.pv1[c] - p.d[c] * p.pv1[b] : 0.0f;
        }
        double const omega = 2.0 * 3.14159265358979323846 * s->cfg.c / f->wavelength;
        // a0 = q E0 / (m c omega) with the species' units given by the caller through e_over_m = q / m
        p.E0 = float(f->a0 * omega * s->cfg.c / f->e_over_m);
        p.omega = float(omega);
        p.w0 = f->waist;
        // PULSE_DURATION: given, or from the intensity FWHM = 2 sqrt(2 ln 2) tau with tau the rms
        // duration of the intensity (GaussianPulseEnvelope: exp(-(t / (2 tau))^2) on the field)
        if(!(f->pulse_duration >= 0.0f))
            return fail(PICGB_ERR_INVALID, "incident field: pulse_duration must be >= 0");
        float const pulseTau = f->pulse_duration > 0.0f
            ? f->pulse_duration
            : float(f->duration_fwhm / (2.0 * std::sqrt(2.0 * std::log(2.0))));
        p.pulseDuration = pulseTau;
        p.tau2 = 2.0f * pulseTau;
        p.tc = f->t_center;
        p.phase = f->phase;
        // origin: the beam axis on the Huygens plane, 0.75 cells inside POSITION
        p.o[f->axis] = float((double(f->surface) - 0.25 * dir) * da);
        p.o[t1] = float(double(f->center_x) * edge[t1]);
        p.o[t2] = float(double(f->center_z) * edge[t2]);
        p.focusDist = float(double(f->focus) * da);
        // phase velocity of the Yee grid at omega along d (calculatePhaseVelocity.hpp with the Yee
        // dispersion relation): sum_a (sin(k d_a h_a / 2) / h_a)^2 = (sin(omega dt / 2) / (c dt))^2,
        // by bisection on the monotonic branch k max_a |d_a| h_a <= pi
        double const rhs = std::pow(std::sin(0.5 * omega * double(s->cfg.dt)) / (double(s->cfg.c) * double(s->cfg.dt)), 2);
        auto lhs = [&](double k)
        {
            double v = 0.0;
            for(int a = 0; a < 3; ++a)
                v += std::pow(std::sin(0.5 * k * dv[a] * edge[a]) / edge[a], 2);
            return v;
        };
        double kmax = 0.0;
        for(int a = 0; a < 3; ++a)
            kmax = std::max(kmax, std::fabs(dv[a]) * edge[a]);
        kmax = 3.14159265358979323846 / kmax;
        if(!(rhs > 0.0 && rhs < lhs(kmax)))
            return fail(PICGB_ERR_INVALID, "incident field: wavelength %g is not resolved by the grid", double(f->wavelength));
        double klo = 0.0, khi = kmax;
        for(int it = 0; it < 200; ++it)
        {
            double const km = 0.5 * (klo + khi);
            (lhs(km) < rhs ? klo : khi) = km;
        }
        p.invVph = float(0.5 * (klo + khi) / omega);
        p.zR = float(3.14159265358979323846 * double(f->waist) * double(f->waist) / double(f->wavelength));
        p.k = float(omega / s->cfg.c);
        if(!(f->time_delay >= 0.0f))
            return fail(PICGB_ERR_INVALID, "incident field: time_delay must be >= 0 (TIME_DELAY)");
        p.timeDelay = f->time_delay;
        if(f->laguerre_count < 0 || f->laguerre_count > 8)
            return fail(PICGB_ERR_INVALID, "incident field: laguerre_count %d outside 0..8", int(f->laguerre_count));
        p.nmodes = f->laguerre_count ? f->laguerre_count : 1;
        p.modeNorm = 0.0f;
        for(int m = 0; m < p.nmodes; ++m)
        {
            p.modes[m] = f->laguerre_count ? f->laguerre_modes[m] : 1.0f;
            p.modePhases[m] = f->laguerre_count ? f->laguerre_phases[m] : 0.0f;
            p.modeNorm += p.modes[m];
        }
        if(!(std::fabs(p.modeNorm) > 1.1920929e-7f)) // GaussianPulse: "Sum of laguerreModes can not be 0."
            return fail(PICGB_ERR_INVALID, "incident field: the sum of the Laguerre mode amplitudes is 0");
        if(f->profile < PICGB_PROFILE_GAUSSIAN_PULSE || f->profile > PICGB_PROFILE_POLYNOM)
            return fail(PICGB_ERR_INVALID, "incident field: unknown profile %d", int(f->profile));
        p.profile = f->profile;
        if(!(f->ramp_init >= 0.0f) || !(f->plateau >= 0.0f) || !(f->pulse_init >= 0.0f))
            return fail(PICGB_ERR_INVALID, "incident field: ramp_init, plateau and pulse_init must be >= 0");
        p.pwPlateau = f->plateau;
        if(p.profile == PICGB_PROFILE_PLANE_WAVE)
        {
            p.pwMu = 0.5f * f->ramp_init * pulseTau;
            p.pwTau = pulseTau * std::sqrt(2.0f);
        }
        p.wpMu = 0.5f * (f->pulse_init * pulseTau + f->plateau); // Wavepacket INIT_TIME / 2
        p.w01 = f->waist_axis[0] > 0.0f ? f->waist_axis[0] : f->waist;
        p.w02 = f->waist_axis[1] > 0.0f ? f->waist_axis[1] : f->waist;
        if(!(p.w01 > 0.0f && p.w02 > 0.0f))
            return fail(PICGB_ERR_INVALID, "incident field: the transverse waists must be > 0");
        if(int r = incidentExtent(s, p))
            return r;
        s->inc[face] = p;
        return PICGB_OK;
    }

    int picgb_step(picgb_sim* s, uint32_t step)
    {
        if(int r = checkSim(s))
            return r;
        if(int r = picgb_stage_current_reset(s))
            return r;
        if(int r = pushLaunches(s))
            return r;
        // with the deposit fused into the push every particle has deposited, and the spilled
        // arrivals can wait for the end of the step; the separate deposit stage reads them
        if(s->cfg.fuse_deposit == 0)
            if(int r = settleParticles(s))
                return r;
        if(int r = picgb_stage_field_before(s, step))
            return r;
        if(int r = picgb_stage_deposit(s, step))
            return r;
        if(int r = picgb_stage_add_current(s))
            return r;
        if(int r = picgb_stage_field_after(s, step))
            return r;
        return afterStep(s);
    }

    int picgb_run(picgb_sim* s, uint32_t step, uint32_t n)
    {
        for(uint32_t i = 0; i < n; ++i)
            if(int r = picgb_step(s, step + i))
                return r;
        return PICGB_OK;
    }

    // ------------------------------------------------------------ diagnostics
    int picgb_energies(picgb_sim* s, double* out, size_t len)
    {
        if(int r = checkSim(s))
            return r;
        size_t const need = 2 + s->species.size();
        if(!out || len < need)
            return fail(PICGB_ERR_INVALID, "energies need %zu entries", need);
        if(need + 4 > 64)
            return fail(PICGB_ERR_INVALID, "too many species for the energy reduction");
        CUDA_TRY(cudaMemsetAsync(s->energy, 0, sizeof(double) * 64, s->stream));
        CUDA_TRY(launchFieldEnergy(s->E, s->ncell, s->energy, s->stream));
        CUDA_TRY(launchFieldEnergy(s->B, s->ncell, s->energy + 3, s->stream));
        s->launches += 2;
        for(size_t i = 0; i < s->species.size(); ++i)
        {
            Species& sp = *s->species[i];
            if(!sp.allocated)
                continue;
            CUDA_TRY(launchKineticEnergy(sp.dev, s->nsc, sp.cfg.mass, s->cfg.c, s->energy + 6 + i, s->stream));
            ++s->launches;
        }
        double h[64];
        CUDA_TRY(cudaMemcpyAsync(h, s->energy, sizeof(double) * (6 + s->species.size()), cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        double const V = double(s->cfg.dx) * double(s->cfg.dy) * double(s->cfg.dz);
        double const mu0 = 1.0 / (double(s->cfg.eps0) * double(s->cfg.c) * double(s->cfg.c));
        out[0] = out[1] = 0.0;
        for(int d = 0; d < 3; ++d)
        {
            out[0] += h[d] * (double(s->cfg.eps0) * V * 0.5);
            out[1] += h[3 + d] * (0.5 / mu0 * V);
        }
        for(size_t i = 0; i < s->species.size(); ++i)
            out[2 + i] = h[6 + i];
        return PICGB_OK;
    }

    int picgb_charge_residual(picgb_sim* s, double* maxResidual, double* maxRho)
    {
        if(int r = checkSim(s))
            return r;
        CUDA_TRY(cudaMemsetAsync(s->rho, 0, sizeof(float) * s->ncell, s->stream));
        CUDA_TRY(cudaMemsetAsync(s->maxBits, 0, sizeof(unsigned) * 2, s->stream));
        float const V = s->cellVolume();
        for(auto& sp : s->species)
        {
            // every charged species, immobile ones included (their density is part of rho)
            if(!sp->allocated || sp->cfg.charge == 0.0f)
                continue;
            CUDA_TRY(launchChargeDensity(sp->cfg.shape, s->cfg.supercell, sp->dev, s->rho, s->g, sp->cfg.charge, V, s->stream));
            ++s->launches;
        }
        CUDA_TRY(launchChargeResidual(s->E, s->rho, s->g, nullptr, s->maxBits, s->maxBits + 1, s->stream));
        ++s->launches;
        unsigned bits[2];
        CUDA_TRY(cudaMemcpyAsync(bits, s->maxBits, sizeof(bits), cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        float f0, f1;
        std::memcpy(&f0, &bits[0], 4);
        std::memcpy(&f1, &bits[1], 4);
        if(maxResidual)
            *maxResidual = f0;
        if(maxRho)
            *maxRho = f1;
        return PICGB_OK;
    }

    // ------------------------------------------------------------ execution control
    int picgb_set_sort_interval(picgb_sim* s, uint32_t steps)
    {
        if(int r = checkSim(s))
            return r;
        s->sortInterval = steps;
        s->stepsSinceSort = 0;
        return PICGB_OK;
    }

    int picgb_set_stream(picgb_sim* s, void* stream)
    {
        if(int r = checkSim(s))
            return r;
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        if(s->ownStream)
            cudaStreamDestroy(s->stream);
        if(stream)
        {
            s->stream = static_cast<cudaStream_t>(stream);
            s->ownStream = false;
        }
        else
        {
            CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
            s->ownStream = true;
        }
        return PICGB_OK;
    }

    int picgb_synchronize(picgb_sim* s)
    {
        if(int r = checkSim(s))
            return r;
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        return PICGB_OK;
    }

    int picgb_launch_count(picgb_sim* s, uint64_t* n)
    {
        if(int r = checkSim(s))
            return r;
        *n = s->launches;
        return PICGB_OK;
    }

    int picgb_profile_enable(picgb_sim* s, int32_t on)
    {
        if(int r = checkSim(s))
            return r;
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        CUDA_TRY(profFlush(s));
        s->prof = on != 0;
        for(int i = 0; i < PICGB_KERNEL_CLASSES; ++i)
        {
            s->profMs[i] = 0.0;
            s->profN[i] = 0;
        }
        CUDA_TRY(cudaMemsetAsync(s->kindCount, 0, 2 * sizeof(unsigned long long), s->stream));
        return PICGB_OK;
    }

    int picgb_profile_read(picgb_sim* s, int32_t cls, double* ms, uint64_t* n)
    {
        if(int r = checkSim(s))
            return r;
        if(cls < 0 || cls >= PICGB_KERNEL_CLASSES)
            return fail(PICGB_ERR_INVALID, "kernel class %d out of range", int(cls));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        CUDA_TRY(profFlush(s));
        if(ms)
            *ms = s->profMs[cls];
        if(n)
            *n = s->profN[cls];
        return PICGB_OK;
    }

    int picgb_profile_deposit_kinds(picgb_sim* s, uint64_t* out)
    {
        if(int r = checkSim(s))
            return r;
        if(!out)
            return fail(PICGB_ERR_INVALID, "null argument");
        unsigned long long h[2];
        CUDA_TRY(cudaMemcpyAsync(h, s->kindCount, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        out[0] = h[0];
        out[1] = h[1];
        return PICGB_OK;
    }

    int picgb_device_status(picgb_sim* s, uint32_t* bits, int32_t reset)
    {
        if(int r = checkSim(s))
            return r;
        unsigned b = 0;
        if(int r = readStatus(s, &b, reset != 0))
            return r;
        *bits = b;
        return PICGB_OK;
    }
}
