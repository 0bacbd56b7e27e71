/*
 * mdgb.h -- C ABI of the GB300 molecular-dynamics step engine (libmdgb.so).
 *
 * Drop-in boundary for moldyn's force / neighbour / integration path.  The
 * reference (a Rust workspace) has no FFI of its own; its boundary is the
 * solver crate's Rust API, which these entry points replace one for one:
 *
 *   mdgb_set_potential        Potential::new_lennard_jones + PotentialsDatabase::set_potential
 *                             (solver/src/solver/potential.rs:27-55, :141-144)
 *   mdgb_set_potential_raw    PotentialsDatabase::load_potentials_from_file entries
 *                             (potential.rs:125-139: sigma, eps, r_cut, u_cut as stored)
 *   mdgb_upload_state         State / StateToSave -> device (core/src/particle.rs:27-32,
 *                             core/src/save_data.rs:129-151)
 *   mdgb_compute_forces       update_force(&PotentialsDatabase, &mut State)
 *                             (solver/src/solver/potential.rs:158-216)
 *   mdgb_step                 Integrator::VerletMethod.calculate(..) called nsteps times with
 *                             Option<(&mut Barostat, P0)>, Option<(&mut Thermostat, T0)>
 *                             (solver/src/solver/integrator.rs:14-59,
 *                              solver/src/initializer/thermostat.rs:24-72,
 *                              solver/src/initializer/barostat.rs:21-56)
 *   mdgb_download_state       device -> State (positions, velocities, force, potential, temp, box)
 *   mdgb_macro_parameters     get_center_of_mass_velocity, get_momentum_of_system,
 *                             get_kinetic_energy, get_thermal_energy, get_potential_energy,
 *                             get_pressure, get_temperature
 *                             (solver/src/macro_parameters/{mod,energy,pressure,temperature}.rs)
 *   mdgb_ensemble_*           no single counterpart: many independent States, each driven as
 *                             `solve` drives one (cli/src/commands.rs:82-191)
 *   mdgb_lj_new / mdgb_lj_eval   Potential::new_lennard_jones / get_potential_and_force
 *                             (potential.rs:27-75), host only
 *   mdgb_lattice              initialize_particles_position (solver/src/initializer/position.rs:
 *                             25-99, :155-174), host only
 *   mdgb_maxwell_boltzmann    initialize_velocities_maxwell_boltzmann
 *                             (solver/src/initializer/velocity.rs:6-29), host only, seeded
 *   mdgb_splat                the GUI viewer's particle + bounding-box render pass
 *                             (gui/src/visualizer/window.rs:940-990, shader.wgsl,
 *                             bounding_box.wgsl), headless
 *
 * Conventions: every call returns an int status (MDGB_OK == 0); no C++
 * exception crosses the ABI; mdgb_last_error() gives the message of the last
 * failure on a handle.  One handle per host thread: calls on a handle are not
 * thread-safe.  All device work of a handle runs on one CUDA stream owned by
 * the handle.  Host arrays passed in are copied; the caller keeps ownership.
 *
 * Atom order: atoms are passed as one flat array with a type id per atom.
 * The reference groups atoms by type (`Vec<Vec<Particle>>`); the k-th atom of
 * type t in the flat array is the reference's particles[t][k].  Every array
 * returned by the engine is in the caller's original flat order.
 *
 * Units are the reference's (nm, 1e-27 kg, 1e-21 J, ps, K for temperature,
 * MPa for pressure); the engine applies the reference's formulas literally,
 * so reduced LJ units work with sigma = eps = mass = 1 and temperatures given
 * as T* * 100 / K_B.
 */
#ifndef MDGB_H
#define MDGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define MDGB_API __declspec(dllexport)
#else
#define MDGB_API __attribute__((visibility("default")))
#endif

#define MDGB_ABI_VERSION 1

/* ---- status codes ---------------------------------------------------- */
#define MDGB_OK 0
#define MDGB_ERR_INVALID_ARGUMENT 1
#define MDGB_ERR_CUDA 2
#define MDGB_ERR_NO_STATE 3
#define MDGB_ERR_NEIGHBOR_OVERFLOW 4   /* list capacity exceeded and regrowth failed */
#define MDGB_ERR_FIXED_POINT_OVERFLOW 5 /* a force sum left the 64-bit fixed-point range */
#define MDGB_ERR_UNSUPPORTED 6
#define MDGB_ERR_DEVICE_TIMEOUT 7      /* a bounded device-side wait gave up */
#define MDGB_ERR_OUT_OF_MEMORY 8
#define MDGB_ERR_SKIN_VIOLATION 9      /* fixed rebuild interval too long for the motion */
#define MDGB_ERR_NOALLOC_TOO_LARGE 10  /* n above MDGB_NOALLOC_MAX_ATOMS (mdgb_forces_noalloc) */

/* ---- precision ------------------------------------------------------- */
#define MDGB_PRECISION_FP64 0  /* plain path: the reference's FP64 arithmetic */
#define MDGB_PRECISION_MIXED 1 /* FP32 pair maths, 64-bit fixed-point force sums, FP64 drift/reductions */
#define MDGB_PRECISION_FP32_NAIVE 2 /* precision-study variant: as MIXED but force sums in plain FP32 */

/* ---- flags ----------------------------------------------------------- */
/* FP64 only: reproduce the reference's summation order (neighbour lists in
 * atom order, serial thermostat/barostat/macro reductions) so forces and
 * trajectories are bit-identical to the reference's FP64 CPU results. */
#define MDGB_FLAG_REFERENCE_ORDER 1u
/* Record CUDA events around every kernel launch (per-kernel timing). */
#define MDGB_FLAG_PROFILE 2u
/* Drive the per-step force pass with the persistent work-queue kernel. */
#define MDGB_FLAG_PERSISTENT 4u
/* Record per-phase device time of the step kernel (mdgb_trace_phases). */
#define MDGB_FLAG_TRACE 8u
/* Build every neighbour list directly (each cell tests all 27 neighbour
 * cells) instead of testing each pair of neighbouring cells once; the lists
 * are the same.  The engine does this by itself for a rebuild in which a cell
 * holds more than 32 atoms. */
#define MDGB_FLAG_DIRECT_LIST 16u

typedef struct mdgb_engine mdgb_engine;

typedef struct {
    int precision;          /* MDGB_PRECISION_* */
    double skin;            /* Verlet skin (length); 0: 0.12 x the largest r_cut (0.3 sigma);
                               < 0: chosen per replica size class on the first step call among
                               0.08 .. 0.16 x the largest r_cut (0.2 .. 0.4 sigma) by timing a short
                               stretch of steps with each (state put back after).  The choice follows
                               the timings, so a tuned mixed-path run is not reproducible bit for bit
                               across runs; an untuned one is. */
    int rebuild_every;      /* 0: rebuild when displacement needs it; >0: fixed interval, checked */
    int threads_per_atom;   /* 0: autotune; else 1, 2, 4 or 8 */
    int graph_steps;        /* >1: capture that many steps into one CUDA graph launch */
    int neighbor_capacity;  /* 0: automatic (grows on overflow) */
    int device;             /* CUDA device ordinal */
    unsigned flags;         /* MDGB_FLAG_* */
} mdgb_config;

/* Thermostat (solver/src/initializer/thermostat.rs:4-20).  lambda and psi
 * are updated in place by mdgb_step, as the reference mutates its enum. */
#define MDGB_THERMOSTAT_BERENDSEN 0
#define MDGB_THERMOSTAT_NOSE_HOOVER 1
typedef struct {
    int kind;
    double tau;
    double target_temperature;  /* T0 passed beside the thermostat (K) */
    double lambda;
    double psi;
} mdgb_thermostat;

/* Barostat::Berendsen (solver/src/initializer/barostat.rs:4-16); myu in/out. */
typedef struct {
    double beta;
    double tau;
    double target_pressure;     /* P0 passed beside the barostat */
    double myu;
} mdgb_barostat;

/* Macro parameters of one particle type (solver/src/macro_parameters). */
typedef struct {
    double kinetic_energy;      /* get_kinetic_energy */
    double potential_energy;    /* get_potential_energy (sum of potential / 2) */
    double thermal_energy;      /* get_thermal_energy with the COM velocity */
    double temperature;         /* get_temperature(thermal_energy, count of this type) */
    double pressure;            /* get_pressure */
    double com_velocity[3];     /* get_center_of_mass_velocity */
    double momentum[3];         /* get_momentum_of_system */
    int64_t count;
} mdgb_macro;

/* Engine counters (host-side view, filled by mdgb_get_stats). */
typedef struct {
    int64_t steps;              /* integrator steps taken */
    int64_t rebuilds;           /* neighbour-list rebuilds (sum over replicas) */
    int64_t kernel_launches;    /* kernels launched by this handle */
    int64_t graph_launches;
    int neighbor_capacity;
    int max_neighbors;          /* largest list seen at the last rebuild */
    int threads_per_atom;
    int retries;                /* chunks re-run after an overflow */
    double force_ms;            /* with MDGB_FLAG_PROFILE: summed force-kernel time */
    int64_t force_launches;
    double integrate_ms;        /* summed integrate/rebuild-kernel time */
    int64_t integrate_launches;
    int class_threads_per_atom[3]; /* autotuned per replica size class: <2048, <32768, larger */
    int class_replicas[3];
    double class_skin[3];       /* Verlet skin per size class (tuned when mdgb_config.skin < 0) */
    int64_t direct_list_builds; /* list builds that took the direct path (MDGB_FLAG_DIRECT_LIST) */
} mdgb_stats;

/* ---- lifecycle ------------------------------------------------------- */
MDGB_API int mdgb_abi_version(void);
MDGB_API int mdgb_config_default(mdgb_config* cfg);
MDGB_API int mdgb_create(const mdgb_config* cfg, mdgb_engine** out);
MDGB_API int mdgb_destroy(mdgb_engine* e);
MDGB_API const char* mdgb_last_error(const mdgb_engine* e);
MDGB_API const char* mdgb_status_string(int status);
/* The CUDA stream (cudaStream_t) all work of the handle runs on. */
MDGB_API void* mdgb_stream(mdgb_engine* e);

/* ---- potentials ------------------------------------------------------ */
MDGB_API int mdgb_set_potential(mdgb_engine* e, uint16_t t0, uint16_t t1, double sigma, double eps);
MDGB_API int mdgb_set_potential_raw(mdgb_engine* e, uint16_t t0, uint16_t t1, double sigma,
                                    double eps, double r_cut, double u_cut);

/* ---- single system --------------------------------------------------- */
MDGB_API int mdgb_upload_state(mdgb_engine* e, int64_t n, const uint16_t* type, const double* pos,
                               const double* vel, const double* mass_per_type, int ntypes,
                               const double box[3]);
/* The reference's Particle carries force, potential and temp into the next
 * Integrator::calculate; upload them (caller order; any pointer may be NULL)
 * after mdgb_upload_state to resume exactly. */
MDGB_API int mdgb_upload_forces(mdgb_engine* e, const double* force, const double* potential,
                                const double* temp);
MDGB_API int mdgb_compute_forces(mdgb_engine* e);
MDGB_API int mdgb_step(mdgb_engine* e, int64_t nsteps, double dt, mdgb_thermostat* thermostat,
                       mdgb_barostat* barostat);
/* Capture, without taking a step, the CUDA graphs a later mdgb_step(nsteps,
 * dt, ...) with these coupling kinds replays (engines with graph_steps > 1;
 * otherwise a no-op), so the capture is not paid inside that call.  The
 * coupling structs are only read for their kind.  Graphs stay valid across
 * uploads of the same shape. */
MDGB_API int mdgb_prepare_step(mdgb_engine* e, int64_t nsteps, double dt, const mdgb_thermostat* thermostat,
                               const mdgb_barostat* barostat);
MDGB_API int mdgb_download_state(mdgb_engine* e, double* pos, double* vel, double* force,
                                 double* potential, double* temp, double box[3]);
MDGB_API int mdgb_macro_parameters(mdgb_engine* e, int type, mdgb_macro* out);

/* ---- ensembles of independent replicas ------------------------------ */
/* offsets[nrep+1]: replica r owns flat atoms [offsets[r], offsets[r+1]).
 * boxes[3*nrep].  Each replica is its own State; the type table is shared. */
MDGB_API int mdgb_ensemble_upload(mdgb_engine* e, int nrep, const int64_t* offsets,
                                  const uint16_t* type, const double* pos, const double* vel,
                                  const double* mass_per_type, int ntypes, const double* boxes);
/* Per-replica coupling; either array may be NULL (no coupling of that kind). */
MDGB_API int mdgb_ensemble_set_coupling(mdgb_engine* e, const mdgb_thermostat* thermostats,
                                        const mdgb_barostat* barostats);
MDGB_API int mdgb_ensemble_step(mdgb_engine* e, int64_t nsteps, double dt);
/* mdgb_prepare_step for ensembles, with the coupling set by mdgb_ensemble_set_coupling. */
MDGB_API int mdgb_ensemble_prepare(mdgb_engine* e, int64_t nsteps, double dt);
MDGB_API int mdgb_ensemble_get_coupling(mdgb_engine* e, mdgb_thermostat* thermostats,
                                        mdgb_barostat* barostats);
MDGB_API int mdgb_ensemble_download(mdgb_engine* e, double* pos, double* vel, double* force,
                                    double* potential, double* temp, double* boxes);
MDGB_API int mdgb_ensemble_macro(mdgb_engine* e, int type, mdgb_macro* out_per_replica);

/* ---- diagnostics ----------------------------------------------------- */
/* The set of interacting pairs of the last force evaluation: every (i, j),
 * caller indices, whose distance by the reference's FP64 rule is <= r_cut
 * (the pairs update_force sums, potential.rs:176-204), read from the
 * neighbour list.  Writes up to `capacity` pairs; *count receives the total. */
MDGB_API int mdgb_interacting_pairs(mdgb_engine* e, int64_t capacity, int32_t* out_i, int32_t* out_j,
                                    int64_t* count);
MDGB_API int mdgb_get_stats(mdgb_engine* e, mdgb_stats* out);
/* With MDGB_FLAG_TRACE: microseconds spent in each phase of the per-step
 * kernel since the last call (then reset), in this order: coupling
 * reductions, kick/drift, rebuild decision, then (rebuild launches only) zero
 * cells, bin, scan A, scan B, scan C, scatter, in-cell sort (0: the sort runs
 * inside the gather phase), gather, Verlet list; then the number of
 * step-kernel launches and of rebuild launches.
 * Writes min(n, 14) values. */
MDGB_API int mdgb_trace_phases(mdgb_engine* e, double* out, int n);
MDGB_API int mdgb_reset_stats(mdgb_engine* e);
/* Failure test of the step kernel's bounded grid barrier (no GPU fault): the
 * next step call's first chunk runs with block hold_block of the step kernel
 * entering its first barrier after 2 * wait_cycles clock cycles and every
 * barrier waiting at most wait_cycles.  The other blocks give up, the call
 * returns MDGB_ERR_DEVICE_TIMEOUT and the state is restored to where the
 * chunk began, so the engine stays usable. */
MDGB_API int mdgb_test_barrier_timeout(mdgb_engine* e, int hold_block, int64_t wait_cycles);
MDGB_API int mdgb_synchronize(mdgb_engine* e);

/* ---- allocation-free force evaluation -------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate GPU
 * memory themselves (a plugin whose host owns all device memory, a loop where
 * an allocation's implicit synchronisation is not allowed, a fixed memory
 * budget): Lennard-Jones forces, potential and temp for n atoms of one type,
 * using no memory beyond the caller's buffers and one static device array of
 * about 1.2 MB that every GPU loading the library holds until exit.  Each
 * pair is evaluated with the reference's FP64 arithmetic (update_force), but
 * the sums run cell by cell rather than in the reference's ascending-j order:
 * results are deterministic and agree with the reference to about 1e-12 of
 * the force scale, not bit for bit.
 *   d_pos      device, 3*n doubles, positions inside [0, box) (others are taken
 *              to their periodic image for binning)
 *   box        host, 3 positive finite doubles
 *   d_force    device, 3*n doubles (out); d_potential, d_temp device, n (out, nullable)
 *   stream     cudaStream_t (NULL: the default stream); the call only enqueues work
 * Limits: n <= MDGB_NOALLOC_MAX_ATOMS (else MDGB_ERR_NOALLOC_TOO_LARGE); at most
 * MDGB_NOALLOC_MAX_CELLS cells (larger boxes use coarser cells); an axis
 * shorter than three cut-off radii is one cell wide, and a box that is one
 * cell on every axis takes at most MDGB_NOALLOC_MAX_SMALL_BOX atoms.  The
 * first call on a device looks up the static array's device address: make it
 * before any stream capture.  Calls share the array: calls that overlap on the
 * GPU race.  The status covers this call's own launches only. */
#define MDGB_NOALLOC_MAX_ATOMS 65536
#define MDGB_NOALLOC_MAX_CELLS 32768
#define MDGB_NOALLOC_MAX_SMALL_BOX 4096
MDGB_API int mdgb_forces_noalloc(int64_t n, const double* d_pos, const double box[3], double sigma, double eps,
                                 double* d_force, double* d_potential, double* d_temp, void* stream);

/* ---- headless particle render ----------------------------------------- */
/* Replaces the GUI viewer's render pass (gui/src/visualizer/window.rs:940-990
 * with shader.wgsl:38-130 and bounding_box.wgsl:26-59) without a graphics
 * stack: spheres ray-cast into an RGBA float image, nearest sphere per pixel
 * (lower index on equal depth), shaded as the GUI's fragment shader, box
 * edges alpha-blended.  Camera fields are the GUI's CameraUniform
 * (window.rs:61-65, built by CameraUniform::from, window.rs:366-377):
 * column-major view (look_to_rh) and a symmetric perspective projection. */
typedef struct {
    float view_pos[4];          /* eye, w = 1 */
    float view[16];             /* column-major */
    float proj[16];             /* column-major cgmath::perspective */
    float gradient_min[4];      /* VisualizationParameter (shader.wgsl:7-13) */
    float gradient_mid[4];
    float gradient_max[4];
    float gradient_min_max[4];  /* speed range: [0] min, [1] max */
    uint32_t mode;              /* 0: colour by particle id % 6, 1: speed gradient, else black */
    int32_t draw_box;           /* blend the bounding-box edges */
    float box[4];               /* bounding box size (x, y, z); the box spans [0, size] */
} mdgb_splat_params;
/* particles: n x 12 floats per particle, the GUI's ParticleDataLite
 * (window.rs:53-57, :340-350): position xyz1, velocity xyz1, (mass, radius, id, 0).
 * out_rgba: height x width x 4 floats, row 0 at the top. */
MDGB_API int mdgb_splat(const float* particles, int64_t n, const mdgb_splat_params* params, int width,
                        int height, float* out_rgba);

/* ---- host-only helpers (no GPU) ------------------------------------- */
/* out = {sigma, eps, r_cut, u_cut} */
MDGB_API int mdgb_lj_new(double sigma, double eps, double out[4]);
MDGB_API int mdgb_lj_eval(const double pot[4], double r, double* u, double* dudr);
/* kind 0 = U (simple cubic), 1 = FCC; out has 3*n doubles, n = nx*ny*nz*(1 or 4) */
MDGB_API int mdgb_lattice(int kind, int64_t nx, int64_t ny, int64_t nz, double a,
                          const double start[3], double* out);
/* Maxwell-Boltzmann at temperature T (K) for mass m, seeded and portable:
 * sigma_v = sqrt(K_B * T * 0.01 / m); the first n/2 atoms get +v, the next
 * n/2 get -v (zero momentum); with odd n the last atom keeps v = 0. */
MDGB_API int mdgb_maxwell_boltzmann(int64_t n, double temperature, double mass, uint64_t seed,
                                    double* out_vel);

#ifdef __cplusplus
}
#endif
#endif /* MDGB_H */
