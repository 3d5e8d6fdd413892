// C entry points of the CPU oracle (test infrastructure only; see pic_oracle.hpp).
// Loaded by tests/ and by bench.py's CPU-baseline leg through ctypes.
#ifdef _OPENMP
#    include <omp.h>
#endif
#include "pic_oracle.hpp"

#include <cstdint>

extern "C"
{
    struct orc_grid
    {
        int nx, ny, nz, sx, sy, sz;
        float dx, dy, dz, dt, c, eps0;
        int open; // bit a: axis a open
    };
    struct orc_pml
    {
        int cells[3][2];
        double sigma_max[3], kappa_max[3], alpha_max[3];
        double order, alpha_order;
    };
    struct orc_species
    {
        float charge, mass;
        int shape, pusher, current;
    };
    struct orc_field
    {
        float* c[3];
    };
    struct orc_particles
    {
        uint64_t n;
        float* pos[3];
        float* mom[3];
        float* w;
        int32_t* sc;
        uint16_t* lcell;
    };
    // one face of the incident field (orc::IncidentFace)
    struct orc_incident_face
    {
        int axis, dir, surface;
        float dirv[3], polv[3], focus[3];
        int circular;
        float amplitude, wavelength, w0, pulse_duration, time_shift, laser_phase, phase_velocity;
        float time_delay;
        int nmodes;
        float modes[8], mode_phases[8];
        int profile;
        float ramp_init, nofocus, pulse_init, w0_axis1, w0_axis2;
    };
    // the FP64 instantiation's exchange format (reference gradients of the differentiable run)
    struct orc_field64
    {
        double* c[3];
    };
    struct orc_particles64
    {
        uint64_t n;
        double* pos[3];
        double* mom[3];
        double* w;
        int32_t* sc;
        uint16_t* lcell;
    };
}

namespace
{
    orc::Grid toGrid(orc_grid const* g)
    {
        return orc::Grid{g->nx, g->ny, g->nz, g->sx, g->sy, g->sz, g->dx, g->dy, g->dz, g->dt, g->c, g->eps0, g->open};
    }
    orc::SpeciesParam toSp(orc_species const* s)
    {
        return orc::SpeciesParam{s->charge, s->mass, s->shape, s->pusher, s->current};
    }
    orc::Field3<float> toF(orc_field const* f)
    {
        return orc::Field3<float>{{f->c[0], f->c[1], f->c[2]}};
    }
    orc::Particles<float> toP(orc_particles const* p)
    {
        orc::Particles<float> r;
        r.n = p->n;
        for(int d = 0; d < 3; ++d)
        {
            r.pos[d] = p->pos[d];
            r.mom[d] = p->mom[d];
        }
        r.w = p->w;
        r.sc = p->sc;
        r.lcell = p->lcell;
        return r;
    }
} // namespace

extern "C"
{
    int orc_abi_version() { return 1; }

    void orc_set_threads(int n)
    {
#ifdef _OPENMP
        omp_set_num_threads(n > 0 ? n : 1);
#else
        (void) n;
#endif
    }

    int orc_max_threads()
    {
#ifdef _OPENMP
        return omp_get_max_threads();
#else
        return 1;
#endif
    }

    // piecewise assignment functions: onSupport=0 -> ChargeAssignment, 1 -> ChargeAssignmentOnSupport
    float orc_shape_value(int shape, int onSupport, float x)
    {
        return onSupport ? orc::ShapeFn<float>::os(shape, x) : orc::ShapeFn<float>::ca(shape, x);
    }

    // ChargeAssignment::shapeArray(pos, isOutOfRange): support+1 values
    void orc_shape_ca_array(int shape, float pos, int isOutOfRange, float* out)
    {
        orc::ShapeFn<float>::caArray(shape, pos, isOutOfRange != 0, out);
    }

    // ChargeAssignmentOnSupport::shapeArray(x): support values
    void orc_shape_os_array(int shape, float x, float* out)
    {
        float v[6] = {0, 0, 0, 0, 0, 0};
        orc::ShapeFn<float>::baseArray(shape, x, v);
        for(int i = 0; i < orc::support(shape); ++i)
            out[i] = v[i];
    }

    int orc_move_particle(orc_grid const* g, float* pos, uint16_t* lcell, int* dir)
    {
        orc::Grid G = toGrid(g);
        return orc::moveParticle(G, pos, *lcell, dir);
    }

    void orc_gather(
        orc_grid const* g,
        int shape,
        orc_field const* F,
        int isB,
        int const* cell,
        float const* pos,
        float* out)
    {
        orc::Grid G = toGrid(g);
        orc::gather(G, shape, toF(F), isB ? orc::kPosB : orc::kPosE, cell, pos, out);
    }

    // TF/SF correction of one incident-field face after a B half step (update_b = 1, incident E
    // at time t) or after the E step (update_b = 0, incident B at time t).
    void orc_incident_update(orc_grid const* g, orc_incident_face const* f, orc_field* F, int update_b, float t)
    {
        orc::IncidentFace face;
        face.axis = f->axis;
        face.dir = f->dir;
        face.surface = f->surface;
        for(int d = 0; d < 3; ++d)
        {
            face.dirv[d] = f->dirv[d];
            face.polv[d] = f->polv[d];
            face.focus[d] = f->focus[d];
        }
        face.circular = f->circular;
        face.amplitude = f->amplitude;
        face.wavelength = f->wavelength;
        face.w0 = f->w0;
        face.pulseDuration = f->pulse_duration;
        face.timeShift = f->time_shift;
        face.laserPhase = f->laser_phase;
        face.phaseVelocity = f->phase_velocity;
        face.timeDelay = f->time_delay;
        face.nmodes = f->nmodes;
        face.profile = f->profile;
        face.rampInit = f->ramp_init;
        face.nofocus = f->nofocus;
        face.pulseInit = f->pulse_init;
        face.w0Axis1 = f->w0_axis1;
        face.w0Axis2 = f->w0_axis2;
        for(int m = 0; m < 8; ++m)
        {
            face.modes[m] = f->modes[m];
            face.modePhases[m] = f->mode_phases[m];
        }
        auto Ff = toF(F);
        orc::incidentUpdate(toGrid(g), face, Ff, update_b != 0, t);
    }

    void orc_yee_b_half(orc_grid const* g, orc_field const* E, orc_field* B)
    {
        auto Bf = toF(B);
        orc::yeeBHalf(toGrid(g), toF(E), Bf);
    }

    void orc_yee_e(orc_grid const* g, orc_field const* B, orc_field* E)
    {
        auto Ef = toF(E);
        orc::yeeE(toGrid(g), toF(B), Ef);
    }

    void orc_add_current(orc_grid const* g, orc_field const* J, orc_field* E)
    {
        auto Ef = toF(E);
        orc::addCurrent(toGrid(g), toF(J), Ef);
    }

    void orc_push(orc_grid const* g, orc_species const* s, orc_particles* p, orc_field const* E, orc_field const* B)
    {
        auto P = toP(p);
        orc::push(toGrid(g), toSp(s), P, toF(E), toF(B));
    }

    void orc_deposit(orc_grid const* g, orc_species const* s, orc_particles const* p, orc_field* J, int nthreads)
    {
        auto Jf = toF(J);
        orc::depositThreaded(toGrid(g), toSp(s), toP(p), Jf, nthreads);
    }

    // Single-particle Esirkepov deposit at a given global cell / in-cell position / velocity.
    void orc_esirkepov_one(
        orc_grid const* g,
        int shape,
        int const* cell,
        float const* pos,
        float const* vel,
        float charge,
        orc_field* J)
    {
        orc::Grid G = toGrid(g);
        auto Jf = toF(J);
        orc::JAccess<float> acc{&G, &Jf};
        orc::esirkepov(G, shape, cell, pos, vel, charge, acc);
    }

    static orc::PmlConfig toPml(orc_pml const* p)
    {
        orc::PmlConfig c{};
        for(int a = 0; a < 3; ++a)
        {
            c.cells[a][0] = p->cells[a][0];
            c.cells[a][1] = p->cells[a][1];
            c.sigmaMax[a] = p->sigma_max[a];
            c.kappaMax[a] = p->kappa_max[a];
            c.alphaMax[a] = p->alpha_max[a];
        }
        c.order = p->order;
        c.alphaOrder = p->alpha_order;
        return c;
    }

    void orc_yee_b_half_open(orc_grid const* g, orc_pml const* p, orc_field const* E, orc_field* B, float* const* psi, int update)
    {
        auto Bf = toF(B);
        orc::yeeBHalfOpen(toGrid(g), toPml(p), toF(E), Bf, psi, update != 0);
    }

    void orc_yee_e_open(orc_grid const* g, orc_pml const* p, orc_field const* B, orc_field* E, float* const* psi)
    {
        auto Ef = toF(E);
        orc::yeeEOpen(toGrid(g), toPml(p), toF(B), Ef, psi);
    }

    void orc_emz_one(
        orc_grid const* g,
        int shape,
        int const* cell,
        float const* pos,
        float const* vel,
        float charge,
        orc_field* J)
    {
        orc::Grid G = toGrid(g);
        auto Jf = toF(J);
        orc::JAccess<float> acc{&G, &Jf};
        orc::emz(G, shape, cell, pos, vel, charge, acc);
    }

    void orc_step(
        orc_grid const* g,
        int nspecies,
        orc_species const* s,
        orc_particles* p,
        orc_field* E,
        orc_field* B,
        orc_field* J,
        int depositThreads)
    {
        std::vector<orc::SpeciesParam> sp(nspecies);
        std::vector<orc::Particles<float>> P(nspecies);
        for(int i = 0; i < nspecies; ++i)
        {
            sp[i] = toSp(&s[i]);
            P[i] = toP(&p[i]);
        }
        auto Ef = toF(E), Bf = toF(B), Jf = toF(J);
        orc::step(toGrid(g), nspecies, sp.data(), P.data(), Ef, Bf, Jf, depositThreads);
    }

    // One PIC step of the FP64 instantiation (every float_X operation in double; the grid's
    // cell sizes, dt, c and eps0 as given in orc_grid).
    void orc_step_f64(
        orc_grid const* g,
        int nspecies,
        orc_species const* s,
        orc_particles64* p,
        orc_field64* E,
        orc_field64* B,
        orc_field64* J,
        int depositThreads)
    {
        std::vector<orc::SpeciesParam> sp(nspecies);
        std::vector<orc::Particles<double>> P(nspecies);
        for(int i = 0; i < nspecies; ++i)
        {
            sp[i] = toSp(&s[i]);
            orc::Particles<double>& r = P[i];
            r.n = p[i].n;
            for(int d = 0; d < 3; ++d)
            {
                r.pos[d] = p[i].pos[d];
                r.mom[d] = p[i].mom[d];
            }
            r.w = p[i].w;
            r.sc = p[i].sc;
            r.lcell = p[i].lcell;
        }
        orc::Field3<double> Ef{{E->c[0], E->c[1], E->c[2]}}, Bf{{B->c[0], B->c[1], B->c[2]}},
            Jf{{J->c[0], J->c[1], J->c[2]}};
        orc::step(toGrid(g), nspecies, sp.data(), P.data(), Ef, Bf, Jf, depositThreads);
    }

    void orc_charge_density(orc_grid const* g, orc_species const* s, orc_particles const* p, float* rho)
    {
        orc::chargeDensity(toGrid(g), toSp(s), toP(p), rho);
    }

    double orc_charge_residual(orc_grid const* g, orc_field const* E, float const* rho, float* out)
    {
        return orc::chargeResidual(toGrid(g), toF(E), rho, out);
    }

    double orc_kinetic_energy(orc_grid const* g, orc_species const* s, orc_particles const* p)
    {
        return orc::kineticEnergy(toGrid(g), toSp(s), toP(p));
    }

    void orc_field_energy(orc_grid const* g, orc_field const* E, orc_field const* B, double* out)
    {
        orc::fieldEnergy(toGrid(g), toF(E), toF(B), out);
    }
}
