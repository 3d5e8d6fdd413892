/* picgb.h -- C-ABI of the GB300-native PIC cycle (Yee + Boris/gather + Esirkepov
 * + supercell bookkeeping).
 *
 * Plain C types only: opaque handles, pointers and sizes.  Every call returns
 * an int status (PICGB_OK = 0); no C++ exception crosses this boundary.  The
 * text of the last error of the calling thread is available from
 * picgb_last_error().  One host thread drives one simulation handle, which
 * enqueues all its work on one CUDA stream (the reference's single host
 * thread over its event-system queues, pmacc/eventSystem/queues/QueueController.hpp:42-81).
 *
 * Units are the caller's: the library takes cell sizes, dt, c and eps0 as
 * given (the reference converts SI to its own units in unitless/simulation.unitless).
 *
 * Reference interfaces replaced (paths inside the PIConGPU source tree):
 *   picgb_create / picgb_destroy        Simulation::init / MappingDesc setup (simulation/control/Simulation.hpp:320-418)
 *   picgb_add_species                   VectorAllSpecies + speciesDefinition.param flags (param/speciesDefinition.param:49-92)
 *   picgb_get_buffer / picgb_share      DataConnector::get / share (pmacc/dataManagement/DataConnector.hpp:48-136)
 *   picgb_step                          Simulation::runOneStep (simulation/control/Simulation.hpp:522-542)
 *   picgb_stage_*                       the stages inside runOneStep (see each declaration)
 *   picgb_energies                      EnergyFields / EnergyParticles plugins (plugins/EnergyFields.x.cpp:183-261,
 *                                       plugins/EnergyParticles.x.cpp:58-160)
 *   picgb_charge_residual               ChargeConservation plugin (plugins/ChargeConservation.tpp:181-260)
 */
#ifndef PICGB_H
#define PICGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

#define PICGB_ABI_VERSION 1

    /* ------------------------------------------------------------ status codes */
    enum picgb_status
    {
        PICGB_OK = 0,
        PICGB_ERR_INVALID = 1, /* bad argument or configuration (e.g. CFL violated, Yee.hpp:57-63) */
        PICGB_ERR_CUDA = 2, /* a CUDA runtime call failed; see picgb_last_error() */
        PICGB_ERR_OVERFLOW = 3, /* a supercell ran out of particle slots (the reference traps on heap
                                   exhaustion, pmacc/particles/memory/boxes/ParticlesBox.hpp:97-122) */
        PICGB_ERR_NOT_FOUND = 4, /* unknown DataConnector id (DataConnector.hpp:113-114 throws) */
        PICGB_ERR_DUPLICATE = 5, /* id already registered (DataConnector::share throws) */
        PICGB_ERR_TIMEOUT = 6, /* a bounded device wait gave up */
        PICGB_ERR_UNSUPPORTED = 7, /* policy combination without a kernel */
        PICGB_ERR_LOST = 8, /* particles were dropped: overflow beyond the spill buffer */
        PICGB_ERR_IO = 9 /* a checkpoint file could not be written or read, or its index is malformed */
    };

    /* ------------------------------------------------------------ policies
     * The .param type policies (param/species.param:49-90, param/fieldSolver.param:57)
     * as run-time enums; each combination maps to a compile-time-specialised kernel. */
    enum picgb_pusher
    {
        PICGB_PUSHER_BORIS = 0, /* particles/pusher/particlePusherBoris.hpp */
        PICGB_PUSHER_FREE = 1, /* particles/pusher/particlePusherFree.hpp */
        PICGB_PUSHER_NONE = 2, /* species without the particlePusher<> flag: not pushed (immobile) */
        PICGB_PUSHER_HIGUERA_CARY = 3, /* particles/pusher/particlePusherHigueraCary.hpp, square roots in double */
        PICGB_PUSHER_VAY = 4, /* particles/pusher/particlePusherVay.hpp, square roots in double */
        PICGB_PUSHER_PHOTON = 5 /* particles/pusher/particlePusherPhoton.hpp: |v| = c along the momentum */
    };
    enum picgb_shape
    {
        PICGB_SHAPE_NGP = 0, /* oracle only */
        PICGB_SHAPE_CIC = 1,
        PICGB_SHAPE_TSC = 2,
        PICGB_SHAPE_PQS = 3,
        PICGB_SHAPE_PCS = 4 /* particles/shapes/PCS.hpp; single-box path */
    };
    enum picgb_current
    {
        PICGB_CURRENT_NONE = 0, /* species without the current<> flag */
        PICGB_CURRENT_ESIRKEPOV = 1, /* fields/currentDeposition/Esirkepov/Esirkepov.hpp */
        PICGB_CURRENT_EMZ = 2 /* fields/currentDeposition/EmZ/EmZ.hpp (Esirkepov meets ZigZag); single-box path */
    };
    enum picgb_field_solver
    {
        PICGB_SOLVER_YEE = 0 /* fields/MaxwellSolver/Yee/Yee.def */
    };
    enum picgb_supercell
    {
        PICGB_SUPERCELL_8x8x4 = 0, /* param/memory.param:51 default */
        PICGB_SUPERCELL_4x4x4 = 1,
        PICGB_SUPERCELL_8x8x8 = 2
    };

    typedef struct picgb_grid_config
    {
        int32_t nx, ny, nz; /* cells of the periodic box; multiples of the supercell size */
        int32_t supercell; /* enum picgb_supercell */
        float dx, dy, dz; /* cell edge lengths */
        float dt; /* time step; c^2 dt^2 sum(1/d^2) <= 1 is enforced */
        float c; /* speed of light */
        float eps0; /* vacuum permittivity (mu0 = 1/(eps0 c^2)) */
        int32_t field_solver; /* enum picgb_field_solver */
        int32_t fuse_deposit; /* 1: deposit J inside the push kernel (default); 0: separate deposit stage */
        int32_t device; /* CUDA device ordinal */
    } picgb_grid_config;

    typedef struct picgb_species_config
    {
        const char* name; /* DataConnector id, e.g. "e", "i" (FrameType::getName()) */
        float charge; /* charge of one real particle (chargeRatio * base charge) */
        float mass; /* mass of one real particle (massRatio * base mass) */
        int32_t pusher; /* enum picgb_pusher */
        int32_t shape; /* enum picgb_shape */
        int32_t current; /* enum picgb_current */
        uint32_t capacity; /* particle slots per supercell; 0 = 1.25 x the largest initial count */
        int32_t with_ids; /* keep a per-particle uint32 id through the migration */
    } picgb_species_config;

    /* Host exchange format of one species: n particles as SoA arrays.
     * pos = in-cell position in [0,1), mom = macro-weighted momentum, w = weighting,
     * sc = supercell linear index (x fastest), lcell = cell inside the supercell
     * (x fastest), id optional (NULL). */
    typedef struct picgb_particles
    {
        uint64_t n;
        float* pos[3];
        float* mom[3];
        float* w;
        int32_t* sc;
        uint16_t* lcell;
        uint32_t* id;
    } picgb_particles;

    /* Device buffer descriptor handed out by the registry (the DataBox a plugin reads). */
    enum picgb_buffer_kind
    {
        PICGB_BUFFER_FIELD = 0, /* ptr[0..ncomp) = component arrays, dims = cells, guard = 0 (periodic wrap) */
        PICGB_BUFFER_SPECIES = 1, /* ptr = px,py,pz,ux,uy,uz,w,lcell,id,count; capacity slots per supercell */
        PICGB_BUFFER_OPAQUE = 2 /* non-array simulation data (e.g. "FieldSolverFDTD") */
    };
    typedef struct picgb_buffer_desc
    {
        int32_t kind; /* enum picgb_buffer_kind */
        int32_t ncomp; /* number of valid entries in ptr */
        void* ptr[10]; /* device pointers */
        int64_t dims[3]; /* cells (fields) or supercells (species) per axis */
        int64_t stride[3]; /* element strides of x, y, z */
        int32_t guard[3]; /* guard cells per side: 0, periodic neighbours by wrap */
        int32_t elem_bytes; /* bytes per element of ptr[0] */
        uint32_t capacity; /* species: slots per supercell */
        int32_t layout; /* 0 = SoA per component, x fastest */
    } picgb_buffer_desc;

    typedef struct picgb_sim picgb_sim;

    /* ------------------------------------------------------------ lifetime */
    int picgb_abi_version(void);
    const char* picgb_last_error(void);

    /* Simulation::init (simulation/control/Simulation.hpp:320-418): fields E, B, J
     * (FieldE/B/J, names "E","B","J") zeroed and registered; "FieldTmp0" and
     * "FieldSolverFDTD" registered. */
    int picgb_create(const picgb_grid_config* cfg, picgb_sim** out);
    int picgb_destroy(picgb_sim* sim);

    /* CreateSpecies (Simulation.hpp:385-386) with the species' flags
     * (param/speciesDefinition.param:49-92); registers the species under cfg->name. */
    int picgb_add_species(picgb_sim* sim, const picgb_species_config* cfg, int32_t* index);

    /* Particle initialisation from host arrays (replaces the InitPipeline of
     * param/speciesInitialization.param): copies in and sorts into supercells. */
    int picgb_species_set(picgb_sim* sim, int32_t species, const picgb_particles* host);
    int picgb_species_count(picgb_sim* sim, int32_t species, uint64_t* n);

    /* Seeded plasma on the device (startPosition::Random + manipulators Temperature/Drift,
     * particles/startPosition/RandomImpl.hpp, particles/manipulators/unary/Temperature.hpp:61-108):
     * ppc particles per cell at uniform random in-cell positions, momenta
     * u = drift + u_th * N(0,1) per component (u = gamma*beta, macro momentum = u m w c),
     * weighting w = density * cell volume / ppc.  Species given the same
     * position_seed get identical positions (a quasi-neutral start).
     * quiet[0..2] > 0 selects startPosition::Quiet instead (particles/startPosition/QuietImpl.hpp:40-110):
     * quiet[0] x quiet[1] x quiet[2] particles per cell on the in-cell lattice
     * i * s + s / 2, s = 1 / quiet[d] (float, two roundings, as the reference evaluates it);
     * ppc must then be 0 or that product.  The reference's MIN_WEIGHTING reduction of the
     * lattice works on SI real-particle counts and is left to the caller's choice of quiet. */
    typedef struct picgb_plasma_init
    {
        uint32_t ppc;
        float density;
        float u_th;
        float drift_lo[3]; /* mean u where cell[split_axis] < split_cell (everywhere if split_axis < 0) */
        float drift_hi[3]; /* mean u where cell[split_axis] >= split_cell */
        int32_t split_axis;
        int32_t split_cell;
        uint64_t seed;
        uint64_t position_seed;
        uint32_t quiet[3]; /* lattice per axis of the quiet start; all 0: random start */
    } picgb_plasma_init;
    int picgb_species_init_plasma(picgb_sim* sim, int32_t species, const picgb_plasma_init* init);
    /* Copies all particles out (supercell order; order inside a supercell is not defined). */
    int picgb_species_get(picgb_sim* sim, int32_t species, picgb_particles* host);

    /* Whole-field copies (host arrays of nx*ny*nz floats per component, x fastest);
     * name is "E", "B", "J" or "FieldTmp0" (one component). */
    int picgb_field_set(picgb_sim* sim, const char* name, const float* const* host);
    int picgb_field_get(picgb_sim* sim, const char* name, float* const* host);

    /* ------------------------------------------------------------ DataConnector */
    /* DataConnector::get (DataConnector.hpp:109-114): PICGB_ERR_NOT_FOUND on an unknown id. */
    int picgb_get_buffer(picgb_sim* sim, const char* name, picgb_buffer_desc* out);
    /* DataConnector::share: registers caller-owned device data; PICGB_ERR_DUPLICATE on an existing id. */
    int picgb_share(picgb_sim* sim, const char* name, const picgb_buffer_desc* desc);
    /* DataConnector::unshare */
    int picgb_unshare(picgb_sim* sim, const char* name);
    /* Number of registered ids and the i-th id (for listing). */
    int picgb_registry_size(picgb_sim* sim, int32_t* n);
    int picgb_registry_name(picgb_sim* sim, int32_t i, char* buf, size_t len);

    /* ------------------------------------------------------------ the PIC step */
    /* Simulation::runOneStep (Simulation.hpp:522-542): CurrentReset, ParticlePush (+shift),
     * update_beforeCurrent, CurrentDeposition, AddCurrent, update_afterCurrent. */
    int picgb_step(picgb_sim* sim, uint32_t step);
    /* runs n steps starting at step index `step` */
    int picgb_run(picgb_sim* sim, uint32_t step, uint32_t n);

    /* Stages (for callers that interleave their own work):
     * CurrentReset (simulation/stage/CurrentReset.hpp:45-51): J = 0 */
    int picgb_stage_current_reset(picgb_sim* sim);
    /* ParticlePush (simulation/stage/ParticlePush.x.cpp:141): gather + push + move of all species
     * with a pusher, then the supercell migration.  With fuse_deposit the current of species with
     * current<> is deposited in the same kernel (J complete after this stage).  Synchronises the
     * stream: arrivals that overflowed their supercell are re-inserted with a larger capacity
     * before it returns (PICGB_ERR_LOST if the spill buffer overflowed as well). */
    int picgb_stage_push(picgb_sim* sim, uint32_t step);
    /* fieldSolver.update_beforeCurrent (FDTD.hpp:69; FDTDBase.hpp:97-121): B half step, E step */
    int picgb_stage_field_before(picgb_sim* sim, uint32_t step);
    /* CurrentDeposition (simulation/stage/CurrentDeposition.x.cpp:105); no-op with fuse_deposit */
    int picgb_stage_deposit(picgb_sim* sim, uint32_t step);
    /* CurrentInterpolationAndAdditionToEMF (stage/CurrentInterpolationAndAdditionToEMF.hpp:99-148):
     * E += -(dt/eps0) J, currentInterpolation::None */
    int picgb_stage_add_current(picgb_sim* sim);
    /* fieldSolver.update_afterCurrent (FDTD.hpp:95; FDTDBase.hpp:151-183): B half step */
    int picgb_stage_field_after(picgb_sim* sim, uint32_t step);

    /* Incident field (fields/incidentField/Solver.hpp:500-533 with profiles/GaussianPulse.hpp):
     * a Gaussian pulse enters through one face of the total-field/scattered-field box and travels
     * along the face's normal: axis 0, 1 or 2; direction +1 enters through the low face and
     * travels +axis (the reference's XMin/YMin/ZMin profiles), -1 through the high face,
     * travelling -axis (XMax/YMax/ZMax).  `surface` is the first (direction +1) or last
     * (direction -1) E plane of the total-field region along the axis; the B plane just beyond it
     * is on the scattered side (the reference's Huygens surface 0.75 cells inside its POSITION:
     * surface = POSITION + 1 on a low face, POSITION - 1 on a high face).  The field solver stages
     * add the incident E (B half steps, at times step*dt and (step+1)*dt) and the incident B (E
     * step, at (step+1/2)*dt) on that surface.  The transverse axes are the two other axes in
     * increasing order (for axis 1: x, then z); polarisation 0 or 1 puts E along the first or the
     * second, and center_x, center_z are the beam centre on the first and the second.  The face
     * spans a periodic transverse axis in full and an open one between its absorbers; on an open
     * axis the surface must keep out of the absorber (Solver.hpp:113-168), which every field stage
     * checks (PICGB_ERR_INVALID).  The pulse is the focused Gaussian beam of
     * profiles/GaussianPulse.hpp:206-290 (fundamental mode, linear polarisation, B = direction x
     * E / c: incidentField::detail::ApproximateIncidentB), at a position u along the axis (in
     * cells) and time t:
     *   dist = direction (u - origin) d, origin = surface - direction / 4 (the Huygens surface),
     *   t_loc = t - dist / v_ph with v_ph the Yee grid's phase velocity at omega along the axis
     *     (calculatePhaseVelocity.hpp; sin(k d/2)/d = sin(omega dt/2)/(c dt)); E = 0 while t_loc < 0,
     *   time = t_loc - t_center, z_f = focus d - dist (distance to the focus),
     *   w = w0 sqrt(1 + (z_f/z_R)^2), z_R = pi w0^2 / wavelength, w0 = waist,
     *   r_c = r^2/2 * (-z_f / (z_R^2 + z_f^2)) with r the transverse distance from the centre,
     *   E = E0 (w0/w) exp(-r^2/w^2) cos(k z_f - k r_c + xi + omega (time - z_f/c) + phase)
     *       exp(-((time - r_c/c) / (2 tau))^2),
     *   xi = atan(-z_f / z_R) (Gouy phase), omega = 2 pi c / wavelength, k = omega / c,
     *   E0 = a0 omega c / e_over_m, tau = duration_fwhm / (2 sqrt(2 ln 2)) (the rms duration of the
     *   intensity; duration_fwhm its FWHM).
     * In the reference's terms: phase = LASER_PHASE, t_center = PULSE_INIT * PULSE_DURATION / 2,
     * PULSE_DURATION = tau, focus = the distance of FOCUS_POSITION beyond the Huygens surface (0:
     * on it), center_x/center_z = FOCUS_POSITION on the transverse axes.  Each of the six faces
     * holds its own pulse: setting a face replaces that face's pulse, enabled = 0 switches the face
     * (axis, direction) off, and a NULL field switches every face off.
     * Oblique incidence: `propagation` (DIRECTION_{X,Y,Z}, unit, entering through the face) and
     * `polarisation_vector` (POLARISATION_DIRECTION_{X,Y,Z}, unit, orthogonal to it) replace the
     * face normal and the axis `polarisation`; the pulse is then evaluated in the reference's
     * vector form: internal coordinates are the dot products of the offset from the origin with
     * the direction, the polarisation and their cross product (Functors.hpp
     * getInternalCoordinates); the origin is where the beam axis crosses the face's Huygens plane
     * at the transverse centre (center_x, center_z), the focus lies `focus` face-axis cells along
     * the direction from it, and v_ph solves the Yee dispersion relation along the direction,
     * sum_a (sin(k d_a h_a / 2) / h_a)^2 = (sin(omega dt / 2) / (c dt))^2.  circular = 1 gives
     * E = (p/sqrt 2) value(phase + pi/2) + (d x p / sqrt 2) value(phase)
     * (GaussianPulseFunctorIncidentE::operator()).  With laguerre_count > 0 the transverse profile
     * is the reference's sum of Laguerre-Gauss modes (GaussianPulse.hpp:260-289):
     *   E = E0 (w0/w) [sum_m a_m L_m(2 r^2/w^2) exp(-r^2/w^2) cos(... + (2m+1) xi + phase + phi_m)]
     *       exp(-((time - r_c/c) / (2 tau))^2) / sum_m a_m,
     * L_m the Laguerre polynomials; time_delay is TIME_DELAY (t_loc = t - dist / v_ph - time_delay).
     * Pulse-front tilt is not supported.
     * profile = PICGB_PROFILE_PLANE_WAVE is profiles/PlaneWave.hpp (a separable functor, transversal
     * factor 1, the waist, focus and Laguerre fields unused): with mu = ramp_init tau / 2 and
     * T = tau sqrt(2), E = E0 (sin(ph) + cos(ph) f) env, ph = omega (t_loc - mu) + phase, env =
     * exp(-(t_loc - mu)^2 / (2 T^2)) and f = (t_loc - mu) / (omega T^2) on the rising ramp (t_loc < mu),
     * the same with mu + plateau on the falling ramp (t_loc > mu + plateau), env = 1 and f = 0 on the
     * plateau.  PICGB_PROFILE_WAVEPACKET (profiles/Wavepacket.hpp) and PICGB_PROFILE_POLYNOM
     * (profiles/Polynom.hpp) are separable functors with the transversal factor
     * exp(-((x_1 / W0_1)^2 + (x_2 / W0_2)^2)), x_1 along the polarisation and x_2 along d x p: the
     * Wavepacket's carrier and ramp correction as PlaneWave's around a plateau centred at
     * (pulse_init tau + plateau) / 2; the Polynom's sin(omega (t_loc - tau/2) + phase) times E0
     * s(2 t_loc / tau), s(u) = u^3 (10 - 15 u + 6 u^2) on [0, 1] and (2 - u)^3 (4 - 9 u + 6 u^2) on
     * (1, 2].  tau is pulse_duration when > 0, else duration_fwhm / (2 sqrt(2 ln 2)). */
    typedef struct picgb_incident_field
    {
        int32_t enabled;
        int32_t axis;
        int32_t surface;
        int32_t polarisation;
        float a0, e_over_m, wavelength, waist, duration_fwhm, t_center, center_x, center_z, phase;
        float focus; /* distance of the focus beyond the Huygens surface along the propagation, in cells */
        int32_t direction; /* +1 (or 0): travels +axis from the low face; -1: travels -axis from the high face */
        float propagation[3]; /* unit DIRECTION_{X,Y,Z}; all zero: the face normal (direction * e_axis) */
        float polarisation_vector[3]; /* unit POLARISATION_DIRECTION_{X,Y,Z}, orthogonal to the propagation;
                                          all zero: the transverse axis `polarisation` */
        int32_t circular; /* 0: linear polarisation; 1: circular (PolarisationType::Circular) */
        float time_delay; /* TIME_DELAY: the local time starts this much later (>= 0) */
        int32_t laguerre_count; /* Laguerre-Gauss modes 0 .. count-1 (at most 8); 0: the fundamental mode */
        float laguerre_modes[8]; /* laguerreModes: mode amplitudes (their sum must not be 0) */
        float laguerre_phases[8]; /* laguerrePhases: mode phases */
        int32_t profile; /* PICGB_PROFILE_GAUSSIAN_PULSE (0) or PICGB_PROFILE_PLANE_WAVE */
        float ramp_init; /* PlaneWave RAMP_INIT: PULSE_DURATIONs of the rising ramp before the plateau */
        float plateau; /* PlaneWave, Wavepacket LASER_NOFOCUS_CONSTANT: duration of the plateau */
        float pulse_duration; /* PULSE_DURATION; > 0 replaces the one derived from duration_fwhm */
        float waist_axis[2]; /* Wavepacket, Polynom W0_AXIS_1, W0_AXIS_2; 0: waist */
        float pulse_init; /* Wavepacket PULSE_INIT */
    } picgb_incident_field;
    enum picgb_incident_profile
    {
        PICGB_PROFILE_GAUSSIAN_PULSE = 0, /* profiles/GaussianPulse.hpp */
        PICGB_PROFILE_PLANE_WAVE = 1, /* profiles/PlaneWave.hpp */
        PICGB_PROFILE_WAVEPACKET = 2, /* profiles/Wavepacket.hpp */
        PICGB_PROFILE_POLYNOM = 3 /* profiles/Polynom.hpp */
    };
    int picgb_set_incident_field(picgb_sim* sim, const picgb_incident_field* field);

    /* ------------------------------------------------------------ diagnostics */
    /* out[0] = field energy of E, out[1] = of B, out[2 + s] = kinetic energy of species s;
     * FP64 sums (EnergyFields.x.cpp:211-225, EnergyParticles.x.cpp:58-160, KinEnergy.hpp:43-66).
     * Synchronises the stream.  len = entries available in out. */
    int picgb_energies(picgb_sim* sim, double* out, size_t len);
    /* Charge conservation (ChargeConservation.tpp:181-260): deposits rho of all charged species
     * (immobile ones included) into "FieldTmp0", returns max|eps0 div E - rho| and max|rho|.
     * Synchronises. */
    int picgb_charge_residual(picgb_sim* sim, double* max_residual, double* max_rho);

    /* Charge-conservation residual without any device allocation.  No counterpart in the
     * reference: it exists for callers that cannot call cudaMalloc, e.g. a plugin inside a
     * host application that has already reserved nearly all device memory for itself (as a
     * PIC code does when it sizes its particle heap to the free memory at start-up).
     * Inputs are caller-owned device arrays: E as three component arrays of nx*ny*nz floats
     * (x fastest), and nspecies particle lists in the host exchange format but in device
     * memory (pos, w, sc, lcell are read; mom and id are not); charge[] and shape[] are host
     * arrays with each species' charge per real particle and shape (CIC, TSC, PQS).  Outputs
     * are host doubles: max|eps0 div E - rho| and max|rho|, the same quantities as
     * picgb_charge_residual.  The charge density is accumulated in a file-scope device array
     * of at most picgb_noalloc_max_cells() = 2^22 cells (16 MiB); larger grids are rejected
     * with PICGB_ERR_INVALID.  CUDA loads device code lazily by default, so that array is
     * reserved on a device by the first call there (which also looks up its device address
     * with cudaGetSymbolAddress) and held until the process exits: a host that reserves
     * device memory for itself should make one call per device before doing so, and the
     * first call should come before any stream capture.  The call makes grid->device
     * current while it works and gives the calling thread its previous current device
     * back.  All calls share the array (each call clears it first), so calls that overlap
     * on the GPU race.  Work is enqueued on `stream` (cudaStream_t, NULL = default stream)
     * and the call waits for it.  Errors are reported by picgb_noalloc_last_error(). */
    uint64_t picgb_noalloc_max_cells(void);
    const char* picgb_noalloc_last_error(void);
    int picgb_charge_residual_noalloc(
        const picgb_grid_config* grid,
        const float* const* E,
        int32_t nspecies,
        const picgb_particles* species,
        const float* charge,
        const int32_t* shape,
        void* stream,
        double* max_residual,
        double* max_rho);

    /* ------------------------------------------------------------ execution control */
    /* Enqueue on a caller's CUDA stream (cudaStream_t passed as void*); NULL = own stream. */
    int picgb_set_stream(picgb_sim* sim, void* stream);
    /* Every `steps` steps (default 20; 0 = never) the step restores each pushed species'
     * interleaved cell order inside every supercell after the compaction: round r holds the
     * r-th particle of every cell with more than r, cells in index order.  Particles keep their
     * slot while they move between cells, which spreads a warp's particles over the supercell and
     * raises the push kernel's shared-memory bank conflicts (two-stream 256^3: 6 % after 200
     * steps); the reorder moves every particle once (about 3 ms per species there).  The
     * reorder also compacts the slots the push vacated, in place of that step's hole filling.
     * A species that left its supercells at more than 3 % of its particles in a reordered step
     * (the first step after picgb_species_init_plasma is one) is reordered every step from
     * then on, as long as steps > 0.  The reference's particle order inside a supercell is not
     * specified either (pmacc/particles/ParticlesBase.kernel:183-359 fills gaps in arbitrary
     * order). */
    int picgb_set_sort_interval(picgb_sim* sim, uint32_t steps);
    int picgb_synchronize(picgb_sim* sim);
    /* Device-side kernel launches issued by this handle since creation (own kernels only). */
    int picgb_launch_count(picgb_sim* sim, uint64_t* n);
    /* Status word written by the kernels (bits: 1 overflow, 2 lost, 4 bad cell, 8 timeout); reading
     * synchronises, reset clears it. */
    int picgb_device_status(picgb_sim* sim, uint32_t* bits, int32_t reset);

    /* Per-kernel timing with CUDA events recorded around each launch on the launching stream
     * (the reference's TimeIntervall step timer, pmacc/simulationControl/SimulationHelper.cpp:143-170,
     * at kernel granularity).  Enabling resets the counters. */
    enum picgb_kernel_class
    {
        PICGB_KERNEL_PUSH = 0, /* fused gather/push/move(/deposit)/migration */
        PICGB_KERNEL_COMPACT = 1, /* hole filling after the migration (steps without a reorder) */
        PICGB_KERNEL_YEE_B = 2, /* B half step */
        PICGB_KERNEL_YEE_E = 3, /* E step (+ J) */
        PICGB_KERNEL_DEPOSIT = 4, /* separate deposit (fuse_deposit = 0) */
        PICGB_KERNEL_ADD_CURRENT = 5, /* separate J add (fuse_deposit = 0) */
        PICGB_KERNEL_REORDER = 6, /* compaction with the interleaved cell order restored (picgb_set_sort_interval) */
        PICGB_KERNEL_CLASSES = 7
    };
    int picgb_profile_enable(picgb_sim* sim, int32_t on);
    /* Total device milliseconds and launch count of one kernel class; synchronises. */
    int picgb_profile_read(picgb_sim* sim, int32_t kernel_class, double* total_ms, uint64_t* launches);
    /* Deposits done by the fused push while profiling: out[0] particles that stayed in their
     * assignment cell along every axis (short footprint), out[1] the others.  Synchronises. */
    int picgb_profile_deposit_kinds(picgb_sim* sim, uint64_t* out);

    /* ------------------------------------------------------------ batched ensemble */
    /* Many independent periodic boxes of uneven size stepped together.  The reference runs one
     * simulation per process (one Simulation, simulation/control/Simulation.hpp:522-542, per
     * MPI domain); this form has no counterpart there.  Every box is a complete simulation
     * handle (picgb_ensemble_box) that the single-box API reads and writes as usual; the
     * ensemble adds the batched step: each kernel of picgb_step runs once over all boxes (the
     * push as one launch per species over every supercell of every box), and the whole step
     * is one CUDA graph launch.  Results per box equal those of picgb_step on that box (the
     * same per-particle and per-cell arithmetic; J sums in another atomic order).  All boxes
     * enqueue on the ensemble's stream. */
    typedef struct picgb_ensemble picgb_ensemble;
    typedef struct picgb_ensemble_config
    {
        picgb_grid_config grid; /* settings shared by all boxes; grid.nx, ny, nz are ignored */
        int32_t nbox;
        const int32_t* dims; /* nbox * 3 cell counts (x, y, z), each a multiple of the supercell */
        int32_t threads; /* threads per supercell of the batched push: 128, 256 or 512 (0 = 256) */
    } picgb_ensemble_config;
    int picgb_ensemble_create(const picgb_ensemble_config* cfg, picgb_ensemble** out);
    int picgb_ensemble_destroy(picgb_ensemble* ens);
    int picgb_ensemble_size(picgb_ensemble* ens, int32_t* nbox);
    /* Borrowed handle of box `box` (valid until picgb_ensemble_destroy; picgb_destroy refuses it). */
    int picgb_ensemble_box(picgb_ensemble* ens, int32_t box, picgb_sim** out);
    /* Adds the species to every box (picgb_add_species on each). */
    int picgb_ensemble_add_species(picgb_ensemble* ens, const picgb_species_config* cfg, int32_t* index);
    /* picgb_species_init_plasma on every box with its own parameters: per_box[nbox]. */
    int picgb_ensemble_init_plasma(picgb_ensemble* ens, int32_t species, const picgb_plasma_init* per_box);
    /* nsteps batched steps; one graph launch per step, then a status check (an overflowing
     * supercell is re-laid out before the next step, as in picgb_step).  The boxes are
     * periodic and carry no incident field: picgb_set_boundaries and
     * picgb_set_incident_field refuse a box of an ensemble (PICGB_ERR_UNSUPPORTED). */
    int picgb_ensemble_run(picgb_ensemble* ens, uint32_t nsteps);
    /* picgb_set_sort_interval for every box and for the batched step (one batched reorder per
     * species after every `steps`-th batched step); default 20, 0 = never. */
    int picgb_ensemble_set_sort_interval(picgb_ensemble* ens, uint32_t steps);
    /* nsteps steps of the single-box path, box after box (picgb_run on each box). */
    int picgb_ensemble_run_sequential(picgb_ensemble* ens, uint32_t nsteps);
    /* Kernels launched by batched steps so far (nodes of the step graph times replays). */
    int picgb_ensemble_launch_count(picgb_ensemble* ens, uint64_t* n);
    /* Autotuner: builds the ensemble `cfg` once for each candidate supercell (8x8x4, 4x4x4,
     * 8x8x8) and threads per supercell (128, 256, 512), initialises the species (nspecies
     * configs, inits[s * nbox + box]), runs `warmup` + `steps` batched steps and measures
     * particle-steps/s with CUDA events.  rates[PICGB_AUTOTUNE_CANDIDATES] (may be NULL)
     * receives the rate of each candidate in the order (8x8x4,128), (8x8x4,256), (8x8x4,512),
     * (4x4x4,128), ... and 0 for candidates that do not divide every box; *supercell and
     * *threads receive the fastest. */
#define PICGB_AUTOTUNE_CANDIDATES 9
    int picgb_ensemble_autotune(
        const picgb_ensemble_config* cfg,
        int32_t nspecies,
        const picgb_species_config* species,
        const picgb_plasma_init* inits,
        uint32_t warmup,
        uint32_t steps,
        int32_t* supercell,
        int32_t* threads,
        double* rates);

    /* ------------------------------------------------------------ differentiable run */
    /* Forward steps of the PIC cycle on particles kept in a fixed order and the hand-written
     * adjoint of those steps (no counterpart in the reference, which has no gradients).  The
     * forward step is Simulation::runOneStep with the fused deposit: gather, Boris, move and
     * Esirkepov deposit per particle, then the Yee split.  The backward pass gives dL/d(initial
     * state) from dL/d(final state): transposed curls for the field update, the transposed
     * Jacobian of the Boris rotation and of Velocity for the push, a deposit of the adjoint
     * force for the gather and a gather of the adjoint current with the derivatives of the
     * Esirkepov weights for the deposit.  The forward keeps the particles every
     * checkpoint_every steps and the fields E, B of every step (when 2 x nsteps field copies
     * fit in a quarter of the free device memory); the backward replays each segment from its
     * checkpoint, moving only the particles through the stored fields (without the stored
     * fields it replays whole steps).  T = float (precision 4) or double (precision 8); all
     * arrays are device memory the caller owns. */
#define PICGB_DIFF_MAX_SPECIES 4
    typedef struct picgb_diff picgb_diff;
    typedef struct picgb_diff_config
    {
        int32_t nx, ny, nz;
        double dx, dy, dz, dt, c, eps0;
        int32_t shape; /* PICGB_SHAPE_CIC, _TSC or _PQS */
        int32_t precision; /* 4 or 8 */
        int32_t checkpoint_every;
        int32_t device;
    } picgb_diff_config;
    typedef struct picgb_diff_species
    {
        double charge, mass; /* per real particle */
        uint64_t n;
    } picgb_diff_species;
    /* E, B: [3][nz][ny][nx] of T; per species s: cell[s] [3][n] int32 (cell index per axis),
     * pos[s] [3][n] T (in-cell position in [0,1)), mom[s] [3][n] T (macro-weighted momentum),
     * w[s] [n] T (weighting; read by the forward and kept for the backward). */
    typedef struct picgb_diff_state
    {
        void* E;
        void* B;
        int32_t nspecies;
        int32_t* cell[PICGB_DIFF_MAX_SPECIES];
        void* pos[PICGB_DIFF_MAX_SPECIES];
        void* mom[PICGB_DIFF_MAX_SPECIES];
        const void* w[PICGB_DIFF_MAX_SPECIES];
    } picgb_diff_state;
    int picgb_diff_create(const picgb_diff_config* cfg, int32_t nspecies, const picgb_diff_species* species, picgb_diff** out);
    int picgb_diff_destroy(picgb_diff* d);
    /* Advances `state` in place by nsteps; work is enqueued on `stream` (cudaStream_t). */
    int picgb_diff_forward(picgb_diff* d, picgb_diff_state* state, uint32_t nsteps, void* stream);
    /* grad: dL/dE, dL/dB, dL/dpos, dL/dmom of the state after the last forward; overwritten in
     * place with the gradients with respect to the state before it (cell and w unused). */
    int picgb_diff_backward(picgb_diff* d, picgb_diff_state* grad, void* stream);
    /* Sum over the species' particles of (gamma - 1) m w c^2, in FP64 (KinEnergy.hpp:43-66
     * without the low-energy branch); synchronises the stream. */
    int picgb_diff_kinetic_energy(picgb_diff* d, const picgb_diff_state* state, int32_t species, double* out, void* stream);

    /* ------------------------------------------------------------ open boundaries and absorbers
     * The reference's non-periodic boundaries (`--periodic 0` on an axis): fields absorbed in
     * layers at the open faces, particles absorbed (deleted) when they leave the box.  Beyond
     * the box the fields are zero.  Absorbers (param/fieldAbsorber.param):
     *  - PICGB_ABSORBER_PML: the convolutional PML of fields/absorber/pml (Yee updates of
     *    Pml.kernel:400-590, coefficients :130-267); sigma and alpha are the reference's
     *    "normalized" values (divided by eps0), in 1/time of the simulation's units;
     *  - PICGB_ABSORBER_EXPONENTIAL: fields/absorber/exponential/Exponential.kernel, a cell at
     *    depth f (1 .. thickness - 1 cells from the layer's inner edge) is multiplied by
     *    exp(-strength f) after each E update and after the B half update that follows it. */
    enum picgb_absorber
    {
        PICGB_ABSORBER_PML = 0,
        PICGB_ABSORBER_EXPONENTIAL = 1
    };
    typedef struct picgb_boundary_config
    {
        int32_t open[3]; /* per axis: 0 periodic, 1 open (absorbing layers, absorbing particles) */
        int32_t absorber; /* enum picgb_absorber */
        int32_t thickness[3][2]; /* absorber thickness per face (negative, positive) of an open axis */
        float sigma_max[3]; /* PML: normalized sigma max; < 0: 0.8 (m + 1) c / cell edge */
        float kappa_max[3]; /* PML: >= 1 */
        float alpha_max[3]; /* PML: normalized alpha max, >= 0 */
        float grading_order; /* PML: sigma and kappa grading order m (fieldAbsorber.param: 4) */
        float alpha_grading_order; /* PML: alpha grading order (fieldAbsorber.param: 1) */
        float strength[3][2]; /* exponential: strength per face (fieldAbsorber.param: 1e-3) */
    } picgb_boundary_config;
    /* Sets the boundaries (all periodic at creation); resets the PML's convolution fields. Not
     * for ensemble boxes.  The charge-residual diagnostic stays periodic, so with an open axis
     * it is meaningful away from the box faces only. */
    int picgb_set_boundaries(picgb_sim* sim, const picgb_boundary_config* cfg);

    /* ------------------------------------------------------------ openPMD checkpoints
     * The reference's Checkpoint and openPMD plugins (plugins/Checkpoint.x.cpp,
     * plugins/openPMD/openPMDWriter.hpp) write E, B and every species in the openPMD 1.1.0
     * layout with the ED-PIC extension.  One iteration here is the directory
     * <dir>/simData_<step>/ holding the series index simData_<step>.json (the openPMD tree in
     * the attribute/dataset form of openPMD-api's JSON backend: small datasets inline under
     * "data", large ones as raw little-endian C-order files named by "external") and those
     * files.  Meshes: E, B (dataOrder C, axisLabels z,y,x, Yee staggering in "position").
     * Particles: position (in-cell, unitSI = cell edge), positionOffset (int32 cell index),
     * momentum (macro-weighted), weighting, id (when kept), constant charge and mass records,
     * one particle patch.  Values are in the simulation's own unit system (unitSI 1). */
    typedef struct picgb_openpmd_species
    {
        const char* name; /* DataConnector id; letters, digits, '_' and '-' only */
        float charge; /* per real particle */
        float mass; /* per real particle */
        int32_t pusher; /* enum picgb_pusher, recorded as the ED-PIC particlePush attribute */
        int32_t shape; /* enum picgb_shape, recorded as particleShape */
        int32_t current; /* enum picgb_current, recorded as currentDeposition */
        picgb_particles particles; /* host arrays in the exchange format (sc, lcell for grid->supercell) */
    } picgb_openpmd_species;

    /* Host-side writer (no device work): the iteration directory from host arrays.  E and B
     * are 3 host arrays of nx*ny*nz floats each, x fastest. */
    int picgb_openpmd_write(
        const char* dir,
        uint32_t step,
        const picgb_grid_config* grid,
        const float* const* E,
        const float* const* B,
        int32_t nspecies,
        const picgb_openpmd_species* species);
    /* Particle count of species `name` in iteration `step` (PICGB_ERR_NOT_FOUND if absent). */
    int picgb_openpmd_species_count(const char* dir, uint32_t step, const char* name, uint64_t* n);
    /* Reads species `name` into host arrays of at least `host->n` particles; sc and lcell are
     * computed for grid->supercell, so a restart may change the supercell size.  The id array
     * is filled when host->id is not NULL and the file holds ids (else PICGB_ERR_NOT_FOUND). */
    int picgb_openpmd_read_species(
        const char* dir,
        uint32_t step,
        const char* name,
        const picgb_grid_config* grid,
        picgb_particles* host);
    /* Reads mesh "E" or "B" (3 host arrays of nx*ny*nz floats). */
    int picgb_openpmd_read_mesh(
        const char* dir,
        uint32_t step,
        const char* name,
        const picgb_grid_config* grid,
        float* const* host);

    /* Checkpoint of a simulation (Checkpoint::notify): E, B and every species with a
     * particle array, as iteration `step` under `dir`.  Iteration s is the state after s
     * steps, at time s * dt. */
    int picgb_checkpoint_write(picgb_sim* sim, const char* dir, uint32_t step);
    /* Restart (Simulation::restart -> checkpoint read): E and B, and every species of the
     * simulation by name; J is zeroed.  The grid must match the file's; the caller's next
     * step index is `step`. */
    int picgb_checkpoint_read(picgb_sim* sim, const char* dir, uint32_t step);

#ifdef __cplusplus
}
#endif

#endif /* PICGB_H */
