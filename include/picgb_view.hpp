/* Reference-layout views of the buffers registered by libpicgb, for plugin code
 * written against PIConGPU's DataBox and ParticlesBox.  Header-only C++17; every
 * accessor works in host and device code (the pointers are device pointers, so
 * dereference them in device code).
 *
 *   FieldBox      a float3_X-valued view of "E", "B", "J" (three SoA component
 *                 arrays in the library) indexed like the reference's
 *                 GridBuffer<float3_X> DataBox (fields/EMFieldBase.hpp:60-70):
 *                 getDeviceDataBox() is indexed from the lower guard corner,
 *                 shift(guard) moves the origin to the first core cell
 *                 (plugins/EnergyFields.x.cpp:250-255).  The library keeps no guard
 *                 cells: the view reports a guard (one supercell, as
 *                 param/memory.param:73, or what the caller asks for) and maps
 *                 every guard index periodically onto the core, which is what the
 *                 reference's guard exchange fills them with on a periodic box.
 *   ParticlesBox  getFirstFrame / getNextFrame / getLastFrame / getPreviousFrame
 *                 over one species (pmacc/particles/memory/boxes/ParticlesBox.hpp:157-190).
 *                 A frame is a window of frameSize consecutive slots of a supercell
 *                 (frameSize = cells per supercell, the reference's frame size,
 *                 pmacc/particles/memory/frames/Frame.hpp:58-85); slot i of a frame
 *                 holds a particle when isParticle(i) (the reference's multiMask != 0).
 *                 Supercell indices are core indices: a periodic single box has no
 *                 guard supercells.
 *
 * makeFieldBox / makeParticlesBox read the descriptor with picgb_get_buffer, as a
 * plugin reads DataConnector::get<T>(name) (pmacc/dataManagement/DataConnector.hpp:109-114).
 */
#pragma once

#include "picgb.h"

#include <cstddef>
#include <cstdint>

#if defined(__CUDACC__)
#    define PICGB_HD __host__ __device__ __forceinline__
#else
#    define PICGB_HD inline
#endif

namespace picgb
{
    namespace view
    {
        /* pmacc::DataSpace<3> */
        struct DataSpace3
        {
            int x, y, z;

            PICGB_HD DataSpace3 operator+(DataSpace3 const& o) const { return {x + o.x, y + o.y, z + o.z}; }
            PICGB_HD DataSpace3 operator-(DataSpace3 const& o) const { return {x - o.x, y - o.y, z - o.z}; }
            PICGB_HD int64_t productOfComponents() const { return int64_t(x) * y * z; }
        };

        /* float3_X */
        struct Float3
        {
            float x, y, z;

            PICGB_HD float& operator[](int d) { return d == 0 ? x : (d == 1 ? y : z); }
            PICGB_HD float operator[](int d) const { return d == 0 ? x : (d == 1 ? y : z); }
        };

        PICGB_HD int wrapIndex(int i, int n)
        {
            int const r = i % n;
            return r < 0 ? r + n : r;
        }

        /* Proxy of one cell's float3_X in a FieldBox: reads and writes the three component arrays. */
        struct Float3Ref
        {
            float* c0;
            float* c1;
            float* c2;

            PICGB_HD operator Float3() const { return {*c0, *c1, *c2}; }
            PICGB_HD Float3Ref const& operator=(Float3 const& v) const
            {
                *c0 = v.x;
                *c1 = v.y;
                *c2 = v.z;
                return *this;
            }
            PICGB_HD float& operator[](int d) const { return d == 0 ? *c0 : (d == 1 ? *c1 : *c2); }
        };

        /* GridLayout of a field (sizeWithoutGuardND, guardSizeND, sizeND). */
        struct GridLayout
        {
            DataSpace3 core;
            DataSpace3 guard;

            PICGB_HD DataSpace3 sizeWithoutGuardND() const { return core; }
            PICGB_HD DataSpace3 guardSizeND() const { return guard; }
            PICGB_HD DataSpace3 sizeND() const
            {
                return {core.x + 2 * guard.x, core.y + 2 * guard.y, core.z + 2 * guard.z};
            }
        };

        class FieldBox
        {
        public:
            float* comp[3] = {nullptr, nullptr, nullptr};
            int64_t stride[3] = {1, 0, 0}; /* element strides of x, y, z */
            GridLayout layout{};
            DataSpace3 origin{0, 0, 0}; /* position of index (0,0,0) relative to the lower guard corner */

            /* the cell at index i, counted from this box's origin */
            PICGB_HD Float3Ref operator()(DataSpace3 const& i) const
            {
                int64_t const o = offset(i);
                return {comp[0] + o, comp[1] + o, comp[2] + o};
            }

            /* DataBox::shift: a box whose (0,0,0) is this box's d */
            PICGB_HD FieldBox shift(DataSpace3 const& d) const
            {
                FieldBox b = *this;
                b.origin = origin + d;
                return b;
            }

            PICGB_HD GridLayout getGridLayout() const { return layout; }

            /* element offset of index i: guard indices wrap periodically onto the core */
            PICGB_HD int64_t offset(DataSpace3 const& i) const
            {
                DataSpace3 const g = origin + i - layout.guard; /* core coordinates */
                return int64_t(wrapIndex(g.x, layout.core.x)) * stride[0]
                    + int64_t(wrapIndex(g.y, layout.core.y)) * stride[1]
                    + int64_t(wrapIndex(g.z, layout.core.z)) * stride[2];
            }
        };

        /* The DataBox of a registered three-component field (FieldE/FieldB/FieldJ::getDeviceDataBox()),
         * indexed from the lower guard corner of a guard of `guard` cells per side. */
        inline int makeFieldBox(picgb_sim* sim, char const* name, DataSpace3 guard, FieldBox* out)
        {
            picgb_buffer_desc d{};
            int const r = picgb_get_buffer(sim, name, &d);
            if(r != PICGB_OK)
                return r;
            if(d.kind != PICGB_BUFFER_FIELD || d.ncomp != 3 || d.elem_bytes != 4)
                return PICGB_ERR_INVALID;
            FieldBox b;
            for(int c = 0; c < 3; ++c)
            {
                b.comp[c] = static_cast<float*>(d.ptr[c]);
                b.stride[c] = d.stride[c];
            }
            b.layout.core = {int(d.dims[0]), int(d.dims[1]), int(d.dims[2])};
            b.layout.guard = guard;
            *out = b;
            return PICGB_OK;
        }

        class ParticlesBox;

        /* FramePtr: one frame of a supercell, or the invalid frame that ends a list. */
        struct FramePtr
        {
            ParticlesBox const* box = nullptr;
            int64_t sc = -1; /* linear core supercell index */
            uint32_t first = 0; /* first slot of the frame inside the supercell */
            uint32_t n = 0; /* particles in this frame: slots [0, n) */

            PICGB_HD bool isValid() const { return box != nullptr; }
            PICGB_HD bool isParticle(uint32_t i) const { return i < n; }
            PICGB_HD Float3 position(uint32_t i) const;
            PICGB_HD Float3 momentum(uint32_t i) const;
            PICGB_HD float weighting(uint32_t i) const;
            PICGB_HD uint16_t localCellIdx(uint32_t i) const;
        };

        class ParticlesBox
        {
        public:
            float* pos[3] = {nullptr, nullptr, nullptr};
            float* mom[3] = {nullptr, nullptr, nullptr};
            float* w = nullptr;
            uint16_t* lcell = nullptr;
            uint32_t* count = nullptr; /* particles per supercell (device) */
            uint32_t capacity = 0; /* slots per supercell */
            uint32_t frameSize = 256; /* cells per supercell */
            DataSpace3 superCells{0, 0, 0};

            PICGB_HD int64_t linear(DataSpace3 const& idx) const
            {
                return idx.x + int64_t(superCells.x) * (idx.y + int64_t(superCells.y) * idx.z);
            }

            /* SuperCell::getNumParticles */
            PICGB_HD uint32_t getNumParticles(DataSpace3 const& idx) const { return count[linear(idx)]; }

            PICGB_HD FramePtr frameAt(int64_t sc, uint32_t first) const
            {
                uint32_t const total = count[sc];
                if(first >= total)
                    return FramePtr{};
                uint32_t const left = total - first;
                return FramePtr{this, sc, first, left < frameSize ? left : frameSize};
            }

            PICGB_HD FramePtr getFirstFrame(DataSpace3 const& idx) const { return frameAt(linear(idx), 0u); }

            PICGB_HD FramePtr getNextFrame(FramePtr const& f) const
            {
                return f.isValid() ? frameAt(f.sc, f.first + frameSize) : FramePtr{};
            }

            PICGB_HD FramePtr getLastFrame(DataSpace3 const& idx) const
            {
                int64_t const sc = linear(idx);
                uint32_t const total = count[sc];
                if(total == 0)
                    return FramePtr{};
                return frameAt(sc, ((total - 1) / frameSize) * frameSize);
            }

            PICGB_HD FramePtr getPreviousFrame(FramePtr const& f) const
            {
                return (f.isValid() && f.first >= frameSize) ? frameAt(f.sc, f.first - frameSize) : FramePtr{};
            }

            PICGB_HD size_t slot(FramePtr const& f, uint32_t i) const
            {
                return size_t(f.sc) * capacity + f.first + i;
            }
        };

        PICGB_HD Float3 FramePtr::position(uint32_t i) const
        {
            size_t const s = box->slot(*this, i);
            return {box->pos[0][s], box->pos[1][s], box->pos[2][s]};
        }

        PICGB_HD Float3 FramePtr::momentum(uint32_t i) const
        {
            size_t const s = box->slot(*this, i);
            return {box->mom[0][s], box->mom[1][s], box->mom[2][s]};
        }

        PICGB_HD float FramePtr::weighting(uint32_t i) const { return box->w[box->slot(*this, i)]; }

        PICGB_HD uint16_t FramePtr::localCellIdx(uint32_t i) const { return box->lcell[box->slot(*this, i)]; }

        /* The ParticlesBox of a registered species (Particles::getDeviceParticlesBox()); superCell is
         * the supercell size of the simulation (its volume is the frame size). */
        inline int makeParticlesBox(picgb_sim* sim, char const* species, DataSpace3 superCell, ParticlesBox* out)
        {
            picgb_buffer_desc d{};
            int const r = picgb_get_buffer(sim, species, &d);
            if(r != PICGB_OK)
                return r;
            if(d.kind != PICGB_BUFFER_SPECIES || d.ncomp < 10)
                return PICGB_ERR_INVALID;
            ParticlesBox b;
            for(int c = 0; c < 3; ++c)
            {
                b.pos[c] = static_cast<float*>(d.ptr[c]);
                b.mom[c] = static_cast<float*>(d.ptr[3 + c]);
            }
            b.w = static_cast<float*>(d.ptr[6]);
            b.lcell = static_cast<uint16_t*>(d.ptr[7]);
            b.count = static_cast<uint32_t*>(d.ptr[9]);
            b.capacity = d.capacity;
            b.frameSize = uint32_t(superCell.productOfComponents());
            b.superCells = {int(d.dims[0]), int(d.dims[1]), int(d.dims[2])};
            *out = b;
            return PICGB_OK;
        }
    } // namespace view
} // namespace picgb
