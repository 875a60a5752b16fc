/*
 * mdg.h -- C ABI of the GB300-native particle hot path (libmddem_gb300.so).
 *
 * The reference (SueHeir/MDDEM, Rust) runs this path as plain systems that
 * share resources inside its App/Scheduler.  This library replaces the systems
 * below with device-resident CUDA kernels for sm_103a; a host plugin (Rust
 * shim over FFI, the C++ host in mddem_gb300/host, or Python ctypes) calls
 * these entry points from the same schedule phases.  Replaced reference
 * interfaces (paths relative to the reference repository):
 *
 *   mdg_create / mdg_batch_create
 *       NeighborPlugin::build + neighbor_setup   crates/mddem_core/src/neighbor.rs:417-541
 *       DemAtomPlugin::build (MaterialTable)      crates/dem_atom/src/lib.rs:592-664, 389-515
 *       HertzMindlinContactPlugin::build          crates/dem_granular/src/contact.rs:52-91
 *       LJForcePlugin + build_lj_pair_table       crates/md_lj/src/lib.rs:290-384
 *       NoseHooverPlugin + setup_nose_hoover      crates/md_thermostat/src/lib.rs:166-243
 *   mdg_upload_state / mdg_download_state
 *       Atom SoA + DemAtom + ContactHistoryStore  crates/mddem_core/src/atom.rs:310-335,
 *                                                 crates/dem_atom/src/lib.rs:530-557,
 *                                                 crates/dem_granular/src/tangential.rs:54-133
 *   mdg_step (one call = nsteps full timesteps, schedule order of schedule.dot:45-153)
 *       initial_integration / final_integration   crates/mddem_verlet/src/lib.rs:97-154
 *       initial_rotation / final_rotation         crates/dem_granular/src/rotational.rs:59-100
 *       nh_pre_initial / nh_post_final            crates/md_thermostat/src/lib.rs:254-353
 *       decide_rebuild                            crates/mddem_core/src/neighbor.rs:639-674
 *       zero_all_forces / remove_ghost_atoms      crates/mddem_core/src/atom.rs:523-533
 *       pbc                                       crates/mddem_core/src/domain.rs:413-459
 *       forward_comm / borders / reverse_send_force
 *                                                 crates/mddem_core/src/comm.rs:367-656
 *                                                 (replaced by on-device periodic images)
 *       sort_atoms_by_bin / bin_neighbor_list     crates/mddem_core/src/neighbor.rs:686-1080
 *       hertz_mindlin_contact_force / hooke_contact_force
 *                                                 crates/dem_granular/src/contact.rs:103-990
 *       lj_force                                  crates/md_lj/src/lib.rs:488-633
 *       zero_virial_stress / VirialStress         crates/mddem_core/src/virial.rs:48-121
 *   mdg_force_only  (neighbor rebuild + force phase, no integration)
 *   mdg_get_pairs   Neighbor::pairs               crates/mddem_core/src/neighbor.rs:172-227
 *   mdg_get_history ContactHistoryStore.contacts  crates/dem_granular/src/tangential.rs:54-75
 *   mdg_thermo      compute_ke + print_granular_temperature + NoseHooverState
 *                                                 crates/mddem_core/src/atom.rs:489-502,
 *                                                 crates/dem_granular/src/granular_temp.rs:44-134
 *
 * Conventions: every call returns an int status (MDG_OK = 0); nothing in the
 * library aborts the process.  Host arrays are borrowed for the duration of a
 * call and copied; the context owns all device memory.  A context is used by
 * one host thread at a time (one CUDA stream per context); distinct contexts
 * may be used from different threads.  Vectors are interleaved per particle
 * (x0,y0,z0,x1,...).  Units are the caller's (SI for DEM, reduced for LJ).
 */
#ifndef MDG_H
#define MDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDG_ABI_VERSION 1

/* status codes */
enum {
    MDG_OK = 0,
    MDG_ERR_CONFIG = 1,        /* invalid configuration (reference: process::exit(1)) */
    MDG_ERR_CUDA = 2,          /* CUDA runtime error */
    MDG_ERR_OOM = 3,           /* device allocation failed */
    MDG_ERR_BUDGET = 4,        /* request exceeds the HBM budget */
    MDG_ERR_OVERLAP_LIMIT = 5, /* > 500 large overlaps in one step (reference panics) */
    MDG_ERR_NAN = 6,           /* non-finite value in the state */
    MDG_ERR_LIST_OVERFLOW = 7, /* neighbor or contact-history capacity exceeded */
    MDG_ERR_TIMEOUT = 8,       /* a bounded device wait gave up */
    MDG_ERR_ARG = 9,           /* bad argument (null pointer, index, size) */
    MDG_ERR_STATE = 10,        /* call out of order (e.g. step before upload) */
    MDG_ERR_NODEVICE = 11,     /* no CUDA device */
    MDG_ERR_LOST = 12          /* a particle left the box across a fixed boundary
                                  (the reference removes it, domain.rs:434-452) */
};

enum { MDG_KIND_DEM = 0, MDG_KIND_LJ = 1 };
enum { MDG_FP64 = 0, MDG_MIXED = 1 };
enum { MDG_CONTACT_HERTZ = 0, MDG_CONTACT_HOOKE = 1 };
enum { MDG_ADHESION_JKR = 0, MDG_ADHESION_DMT = 1 };
enum { MDG_MODEL_CONSTANT = 0, MDG_MODEL_SDS = 1 };
/* Rebuild policy.  REFERENCE: rebuild when any atom moved more than the skin
 * share or left the box (decide_rebuild, neighbor.rs:639-674); positions are
 * wrapped only on rebuild steps.  DISPLACEMENT: rebuild on displacement only;
 * positions stay unwrapped between rebuilds (periodic images are carried by
 * the list), which removes the per-crossing rebuilds of large boxes. */
enum { MDG_REBUILD_REFERENCE = 0, MDG_REBUILD_DISPLACEMENT = 1 };

/* One [[dem.materials]] entry (crates/dem_atom/src/lib.rs:78-121). */
typedef struct mdg_material {
    double youngs_mod, poisson_ratio, restitution, friction;
    double rolling_friction, twisting_friction, cohesion_energy, surface_energy;
    double kn, kt, rolling_stiffness, rolling_damping, twisting_stiffness, twisting_damping;
} mdg_material;

/* Plane wall ([[wall]] type = "plane", crates/dem_wall/src/lib.rs:171-347):
 * the plane through `point` with outward `normal` (normalised on use); active
 * for particles inside [bound_lo, bound_hi] (use +-HUGE_VAL for unbounded);
 * `velocity` a constant wall velocity (the plane moves by velocity * dt before
 * every step's force, wall_move, lib.rs:766-790); `material` an index into the
 * config's materials.  Sphere-wall Hertz normal force with damping and
 * adhesion and a twisting torque (wall_contact_force, lib.rs:848-990). */
typedef struct mdg_wall {
    double point[3], normal[3];
    double bound_lo[3], bound_hi[3];
    double velocity[3];
    int material;
} mdg_wall;
#define MDG_MAX_WALLS 6

/* One LJ type pair: well depth, length scale and the cutoff in units of
 * sigma (LJPairCoeffs::from_params, crates/md_lj/src/lib.rs:226-238). */
typedef struct mdg_lj_pair {
    double epsilon, sigma, cutoff;
} mdg_lj_pair;

/* One simulation (a "system"): the TOML sections the plugins read. */
typedef struct mdg_config {
    int kind;                    /* MDG_KIND_* */
    int precision;               /* MDG_FP64 or MDG_MIXED ([gpu] precision) */
    double box_lo[3], box_hi[3]; /* [domain]; periodic unless `fixed` below */
    double dt;                   /* [run] dt (> 0) */
    /* [neighbor] (crates/mddem_core/src/neighbor.rs:44-80) */
    double skin_fraction, bin_size;
    int every, check, sort_every, newton;
    /* [dem] */
    int n_materials;
    const mdg_material* materials;
    int contact_model, adhesion_model, rolling_model, twisting_model;
    /* [lj] single type (crates/md_lj/src/lib.rs:115-140) */
    double lj_epsilon, lj_sigma, lj_cutoff;
    /* [thermostat] Nose-Hoover (crates/md_thermostat/src/lib.rs:85-97) */
    int nose_hoover;
    double nh_temperature, nh_coupling;
    int virial;                  /* accumulate the 6-component virial each step */
    /* [gpu] */
    int rebuild_policy;          /* MDG_REBUILD_* */
    int threads_per_particle;    /* 0 = auto; 1,2,4,8,16,32 for the force kernels */
    int neighbor_capacity;       /* 0 = auto: max full-list entries per particle */
    int history_capacity;        /* 0 = auto: max stored contacts per particle */
    /* [langevin] (crates/md_thermostat/src/lib.rs:380-581): at PostForce
     * F += -gamma m v + sqrt(2 gamma m kT / dt) N(0,1) per component.  The
     * reference draws from one ChaCha8 stream in atom order; here N(0,1) comes
     * from a counter-based stream keyed by (seed, step, tag, component), so a
     * run is reproducible and independent of particle order and batching. */
    int langevin;
    double lv_temperature, lv_damping;
    uint64_t lv_seed;
    /* [domain] boundary_x/y/z = "fixed": no periodic images along that axis
     * (0 = periodic, the default); a particle found outside the box there at a
     * rebuild makes the step return MDG_ERR_LOST (the reference removes it). */
    int fixed[3];
    /* [[wall]] plane walls (DEM), at most MDG_MAX_WALLS */
    int n_walls;
    const mdg_wall* walls;
    /* [lj] multi-type mode (build_lj_pair_table, crates/md_lj/src/lib.rs:
     * 334-384): n_lj_types > 1 gives the n x n pair table `lj_pairs`
     * (row-major and symmetric, with the mixing rule and the pair_coeffs
     * overrides applied), and each particle's `type` (< n_lj_types) picks its
     * row and column; 0 or 1 = the single type of lj_epsilon/sigma/cutoff. */
    int n_lj_types;
    const mdg_lj_pair* lj_pairs;
} mdg_config;


/* SoA view of one system's particles (caller-owned, n particles). */
typedef struct mdg_state_view {
    size_t n;
    uint32_t* tag;
    uint32_t* type;          /* material index (DEM) or LJ type (< n_lj_types in
                                multi-type mode, else unused) */
    double* pos;             /* n*3 */
    double* vel;             /* n*3 */
    double* force;           /* n*3: initial force on upload (restart), NULL = zero */
    double* mass;            /* n */
    double* cutoff_radius;   /* n: neighbor cutoff radius (DEM: radius; LJ: lattice skin) */
    int32_t* image;          /* n*3 periodic image counters (may be NULL) */
    /* DEM only (NULL for LJ) */
    double* radius;          /* n */
    double* inv_inertia;     /* n */
    double* omega;           /* n*3 */
    double* torque;          /* n*3: initial torque on upload (restart), NULL = zero */
    double* quat;            /* n*4 [w,x,y,z] */
} mdg_state_view;

/* Thermo record (print_thermo / GranularTemp columns plus extended state). */
typedef struct mdg_thermo_t {
    double ke;               /* 0.5 sum m |v|^2 */
    double pe;               /* LJ 12-6 energy sum over pairs (unshifted) */
    double temp;             /* 2 KE / (3N - 3) */
    double p_xi;             /* Nose-Hoover thermostat momentum */
    double granular_temp;    /* sum m |v - vbar|^2 / (3 M) */
    double momentum;         /* |sum m v| */
    double virial[6];        /* xx yy zz xy xz yz of the last force evaluation */
    int64_t step;
    int64_t nbuilds;         /* neighbor-list builds so far */
    int64_t n;
    int32_t status;          /* sticky device status word for this system */
    int32_t max_neighbors;   /* largest full-list row seen at the last build */
    double e_tail, p_tail;   /* LJ long-range tail corrections (setup_lj_tails,
                                md_lj/src/lib.rs:397-445); 0 for DEM */
    double rot_temp;         /* DEM: sum 0.4 m r^2 |omega|^2 / (3 M)
                                (examples/bench_sphere_haff_cooling/main.rs:88-105) */
    double pressure;         /* rho T - tr(virial) / (3 V) + P_tail (compute_pressure,
                                md_measure/src/lib.rs:605-652; virial 0 unless enabled) */
} mdg_thermo_t;

typedef struct mdg_ctx mdg_ctx;

/* Library / device */
int  mdg_abi_version(void);
const char* mdg_status_string(int status);
int  mdg_device_count(int* count);

/* Context lifecycle.  mdg_create makes a context holding one system;
 * mdg_batch_create makes one context advancing nsys systems (replicas of
 * uneven sizes) with one launch per kernel per step.  capacity[k] is the
 * largest particle count system k will hold. */
int  mdg_create(const mdg_config* cfg, size_t capacity, mdg_ctx** out);
int  mdg_batch_create(const mdg_config* cfgs, const size_t* capacity, int nsys, mdg_ctx** out);
void mdg_destroy(mdg_ctx* ctx);
/* Replace the physics of system `sys` (a slot) with `cfg`: contact laws,
 * materials, LJ coefficients, timestep, [neighbor] settings.  The kind and
 * precision must match the slot; memory stays allocated; other systems are
 * untouched.  The slot is frozen until the next mdg_upload_state. */
int  mdg_configure_system(mdg_ctx* ctx, int sys, const mdg_config* cfg);
int  mdg_num_systems(const mdg_ctx* ctx);

/* State transfer for system `sys` (0 for single-system contexts).
 * Upload resets neighbor/rebuild state (next step performs a full rebuild,
 * like the reference's first step) and clears contact history. */
int  mdg_upload_state(mdg_ctx* ctx, int sys, const mdg_state_view* st);
int  mdg_download_state(mdg_ctx* ctx, int sys, mdg_state_view* st);

/* Contact history transfer: keys = (owner tag, partner tag) pairs, vals = 7
 * doubles per entry, in the reference's canonical (lower-tag) frame. */
int  mdg_set_history(mdg_ctx* ctx, int sys, size_t n, const uint32_t* keys, const double* vals);
int  mdg_get_history(mdg_ctx* ctx, int sys, uint32_t* keys, double* vals, size_t cap, size_t* n);

/* Advance every active system of the context by nsteps timesteps (graph
 * mode: one launch of a device-side loop).  Returns the first non-zero system
 * status, if any. */
int  mdg_step(mdg_ctx* ctx, int64_t nsteps);
/* mdg_step in two halves, for a caller that advances several contexts at
 * once (each on its own stream, so their launches overlap on the GPU):
 * mdg_step_async queues the nsteps on the context's stream and returns;
 * mdg_step_wait blocks until they are done and returns what mdg_step would.
 * No other call on the context between the two. */
int  mdg_step_async(mdg_ctx* ctx, int64_t nsteps);
int  mdg_step_wait(mdg_ctx* ctx);
/* Step budget of one system: it advances `steps` more timesteps and then
 * freezes (its kernels skip it) until given a new budget; -1 = unlimited (the
 * default after upload).  Used by batching and serving to stop finished jobs
 * inside one multi-step launch. */
int  mdg_set_remaining(mdg_ctx* ctx, int sys, int64_t steps);
int  mdg_get_remaining(mdg_ctx* ctx, int sys, int64_t* steps);
/* A copy of system sys's current config (its materials, walls and lj_pairs
 * pointers refer to the context's own copies, valid until the next
 * mdg_configure_system of sys; passing it back to mdg_configure_system is
 * fine).  Every array a config points at is copied by mdg_create /
 * mdg_batch_create / mdg_configure_system / mdg_server_submit. */
int  mdg_get_config(mdg_ctx* ctx, int sys, mdg_config* out);
/* Lanes per particle row of the LJ force kernel (1, 2, 4 or 8), for the whole
 * context; changes the per-particle summation order, not the physics. */
int  mdg_set_threads_per_particle(mdg_ctx* ctx, int tpp);
int  mdg_get_threads_per_particle(const mdg_ctx* ctx);
/* Work split of the neighbour-list build (bin_neighbor_list,
 * crates/mddem_core/src/neighbor.rs:810-1080) for every system of the
 * context: 0 = a warp per bin, 1 = a warp per particle, 2 = a thread per
 * particle, -1 = chosen per system from its particles per bin and bin count
 * (the default).  Every mode writes the same rows; the mode applies to the
 * systems uploaded so far and to later uploads. */
int  mdg_set_build_mode(mdg_ctx* ctx, int mode);

/* ---- autotuner -----------------------------------------------------------------
 * Picks, by timing short trial runs on the context's own systems, the LJ
 * force kernel's threads per particle, and per particle kind (DEM, LJ) the
 * skin fraction (the rebuild cadence: list cutoff 2 r skin, rebuild when a
 * particle moved (skin - 1) r_min) and the bin size (a multiple of the list
 * cutoff).  All three leave the physics unchanged: forces use the contact /
 * LJ cutoff, not the list cutoff.  Call after uploading and before the first
 * step: every trial restarts from the uploaded state (and contact history),
 * and the call ends with that state uploaded again under the chosen
 * parameters, so the simulation is exactly as uploaded.  Coordinate descent
 * over the candidates; a trial's cost is its mean step time over `steps`
 * graph-launched steps (extended until two rebuilds were seen, at most
 * 8 x steps), plus the measured full-rebuild time over the trial's steps
 * when no rebuild occurred in them. */
typedef struct mdg_tune_opts {
    int steps;              /* steps per trial (0 = 40) */
    int tune_tpp, tune_skin, tune_bin;  /* 0 = keep that parameter */
} mdg_tune_opts;
typedef struct mdg_tune_result {
    int tpp;
    double skin_fraction[2];    /* [DEM, LJ] chosen (0 = kind absent) */
    double bin_factor[2];       /* bin size / list cutoff chosen (>= 1: bins are
                                   never smaller than the list cutoff) */
    double ms_before, ms_after; /* modelled ms per step, first and chosen */
    int trials;
} mdg_tune_result;
int  mdg_autotune(mdg_ctx* ctx, const mdg_tune_opts* opts, mdg_tune_result* out);

/* ---- measurements (md_measure/src/lib.rs) ----------------------------------
 * mdg_rdf: pair counts per bin of width r_max / nbins over all pairs of one
 * system under the minimum image (accumulate_rdf's single-rank loop,
 * lib.rs:333-410, same fp64 arithmetic: the counts equal the reference's on
 * the same positions); counts (nbins <= 4096 entries, host) are overwritten.
 * g(r) = counts_k V / (N (N - 1) / 2 x 4/3 pi (r_{k+1}^3 - r_k^3)).
 * mdg_msd_reset records every particle's unwrapped position (x + image L) by
 * tag; mdg_msd returns the mean of |unwrapped - recorded|^2 (track_msd,
 * lib.rs:459-600). */
int  mdg_rdf(mdg_ctx* ctx, int sys, double r_max, int nbins, uint64_t* counts);
int  mdg_msd_reset(mdg_ctx* ctx, int sys);
int  mdg_msd(mdg_ctx* ctx, int sys, double* msd);

/* The context's CUDA stream (cudaStream_t): all of the context's device work
 * is ordered on it, so a caller may record events on it or make its own
 * streams wait for it. */
int  mdg_get_stream(mdg_ctx* ctx, void** stream);
/* Run the context's work on a new stream of CUDA priority `priority`
 * (lower numbers run first; clamped to the device's range; 0 = the default).
 * No counterpart in the reference: contexts launched side by side (several
 * batches, the server's slot groups) can put a latency-bound chain ahead of a
 * bandwidth-bound one.  Not while a launch is in flight (MDG_ERR_STATE). */
int  mdg_set_stream_priority(mdg_ctx* ctx, int priority);
/* Every system's step budget, status word and step counter in one device
 * read (arrays of mdg_num_systems entries; any may be NULL). */
int  mdg_get_progress(mdg_ctx* ctx, int64_t* remaining, int32_t* status, int64_t* steps);
/* Sticky device status word of one system (0 = healthy). */
int  mdg_get_status(mdg_ctx* ctx, int sys, int32_t* status);
/* Neighbor rebuild + force evaluation at the current state (no integration). */
int  mdg_force_only(mdg_ctx* ctx);
/* Half-list pairs at the last build as (owner tag, partner tag). */
int  mdg_get_pairs(mdg_ctx* ctx, int sys, uint32_t* pairs, size_t cap, size_t* n);
int  mdg_thermo(mdg_ctx* ctx, int sys, mdg_thermo_t* out);
/* Block until all device work of the context is complete. */
int  mdg_synchronize(mdg_ctx* ctx);
/* Device kernels launched by this context so far (for launch accounting). */
int64_t mdg_kernel_launches(const mdg_ctx* ctx);
/* Capture the per-step kernel sequence into a CUDA graph (1) or launch
 * kernels individually (0).  Default 1. */
int  mdg_set_graph_mode(mdg_ctx* ctx, int enabled);

/* Device timing of individual steps (tracing).  Each step runs as one
 * captured graph bracketed by CUDA events on the context's stream, with event
 * records between its phases; before each step, outside the events, the L2
 * cache is flushed by writing l2_flush_bytes of scratch memory (0 = no
 * flush).  per_step receives nsteps records. */
typedef struct mdg_step_timing {
    double step_ms;          /* whole step, first to last event */
    double phase_ms[4];      /* initial integration, rebuild pipeline, force, final */
    int32_t kernels;         /* kernels launched by the step */
    int32_t rebuilt;         /* 1 if any system rebuilt its list this step */
} mdg_step_timing;
int  mdg_timed_steps(mdg_ctx* ctx, int64_t nsteps, size_t l2_flush_bytes, mdg_step_timing* per_step);

/* Granular temperature without allocating.  No counterpart in the reference:
 * it is the mdg_thermo reduction (print_granular_temperature + compute_ke) for
 * callers that cannot call cudaMalloc -- e.g. a host that reserves all device
 * memory for its own pool, or a latency-critical loop that must not risk an
 * allocation's device synchronisation.  vel (n*3 interleaved) and mass (n) are
 * device pointers; out3 (device, 3 doubles) receives
 * [sum m|v-vbar|^2 / (3M), 0.5 sum m|v|^2, |sum m v|].  The only scratch is a
 * static device array inside the library (about 256 KB, held on every GPU that
 * loads the library until exit), which limits n to 1,048,576 particles
 * (larger n returns MDG_ERR_ARG).  The first call on a device looks up that
 * array's device address, so make the first call before any stream capture;
 * the address is kept for the life of the device's primary context, so do
 * not call this again after a cudaDeviceReset in the same process.
 * All calls share the array: calls that overlap on the GPU race.  Work is
 * queued on `stream` (NULL = default stream); the call does not synchronise. */
int  mdg_granular_temp_noalloc(const double* vel, const double* mass, size_t n, double* out3, void* stream);

/* ---- Serving: continuous batching of independent jobs --------------------
 * A server's slots (kind and particle capacity from slot_cfgs /
 * slot_capacity) are the systems of one batch context per particle kind, each
 * on its own stream.  Submitted jobs (config + initial state + step count)
 * queue on the host; mdg_server_pump admits queued jobs into free slots of
 * their kind while the resident jobs' estimated device footprint stays within
 * hbm_budget bytes, advances all resident jobs with one multi-step device
 * launch of at most max_steps steps per context (all launched before any is
 * waited for, so the kinds run side by side; each job freezes at its own step
 * count), and retires finished jobs (final state kept on the host until
 * fetched).  Times are seconds since server creation. */
typedef struct mdg_server mdg_server;
typedef struct mdg_job_info {
    int64_t id;
    int32_t status;          /* MDG_OK or the job's error */
    int32_t slot;
    int64_t steps;
    int64_t n;
    double submit_s, start_s, end_s;
} mdg_job_info;
int  mdg_server_create(const mdg_config* slot_cfgs, const size_t* slot_capacity, int nslots, size_t hbm_budget,
                       mdg_server** out);
/* As mdg_server_create, with the slots placed by slot_group: the slots that
 * share a group id (which must share a kind) make one batch context on its
 * own stream, so e.g. small and large jobs of one kind can also run side by
 * side.  mdg_server_create groups by kind. */
int  mdg_server_create_grouped(const mdg_config* slot_cfgs, const size_t* slot_capacity, const int* slot_group,
                               int nslots, size_t hbm_budget, mdg_server** out);
void mdg_server_destroy(mdg_server* srv);
int  mdg_server_submit(mdg_server* srv, const mdg_config* cfg, const mdg_state_view* st, int64_t steps, int64_t* id);
int  mdg_server_pump(mdg_server* srv, int64_t max_steps, int* active, int* pending);
int  mdg_server_poll(mdg_server* srv, mdg_job_info* out, int cap, int* n);
int  mdg_server_fetch(mdg_server* srv, int64_t id, mdg_state_view* out);
/* The context holding slot 0; mdg_server_slot_context gives the context
 * holding any slot and the slot's system index there (diagnostics: timed
 * steps, pairs, a resident job's state). */
int  mdg_server_context(mdg_server* srv, mdg_ctx** ctx);
int  mdg_server_slot_context(mdg_server* srv, int slot, mdg_ctx** ctx, int* sys);
/* Running totals: particle-steps advanced by all pumps, pumps that launched
 * work, jobs retired; resident and queued jobs and their estimated device
 * bytes now; seconds since creation; host seconds spent in admission
 * (configure + upload), in the multi-step launches (to completion) and in
 * retirement (progress read + download); kernels launched; contexts. */
typedef struct mdg_server_stats_t {
    double particle_steps;
    int64_t pumps, retired;
    int32_t resident, pending;
    size_t hbm_used;
    double time_s;
    double admit_s, step_s, retire_s;
    int64_t launches;        /* device kernels launched by all of the server's contexts */
    int32_t contexts;        /* batch contexts (one per particle kind among the slots) */
} mdg_server_stats_t;
int  mdg_server_stats(mdg_server* srv, mdg_server_stats_t* out);
/* The jobs resident in slots now (steps = steps done so far, end_s = -1);
 * *n receives the count, of which min(cap, count) are written. */
int  mdg_server_resident(mdg_server* srv, mdg_job_info* out, int cap, int* n);

/* ---- seeded initial conditions ---------------------------------------------
 * Random sequential addition of non-overlapping spheres in a periodic box:
 * replaces the rejection loop of insert.rs:523-571 (candidate centre uniform in
 * the box, inset by the largest radius when `inset`; radius uniform in
 * [rmin, rmax]; rejected when any placed sphere lies within
 * sep_factor * (r_i + r_j) under the minimum image) with a cell grid so that
 * 1e6 spheres place in seconds.  The random stream is xoshiro256** seeded by
 * splitmix64(seed): same seed, same spheres on every host.  pos_out (n*3) and
 * rad_out (n) are host buffers; *placed receives the count placed, and the
 * call returns MDG_ERR_ARG when fewer than n fit within max_attempts
 * (0 = 20000 n). */
int  mdg_rsa_spheres(size_t n, const double box_lo[3], const double box_hi[3], double rmin, double rmax,
                     double sep_factor, int inset, uint64_t seed, uint64_t max_attempts, double* pos_out,
                     double* rad_out, size_t* placed);

/* Generators on the device: they write system `sys` of a context directly
 * (no host state, no host->device copy), then arm it like mdg_upload_state.
 * Their random numbers are counter based -- mdg_counter_draw(seed, stream, i)
 * is the 64-bit draw i of a stream, a uniform takes its top 53 bits, a normal
 * comes from the Box-Muller transform of draws (2k, 2k+1) -- so the results do
 * not depend on the launch shape and are the same on every GPU. */
uint64_t mdg_counter_draw(uint64_t seed, uint32_t stream, uint64_t index);

/* FCC lattice of an LJ system, restating fcc_insert
 * (crates/md_lattice/src/lib.rs:232-454): lattice constant (4/density)^(1/3),
 * cells per axis floor(L / a) (MDG_ERR_CONFIG when 0 on an axis), cells
 * stretched to tile the box from box_lo, 4-atom basis in (ix, iy, iz, basis)
 * order, tags 0..N-1; atom k takes the first type whose cumulative fraction
 * exceeds (k + 0.5) / N (the last type past them); velocities N(0, sqrt(T/m))
 * per component from draws 4k..4k+3 of stream 2, the plain mean removed,
 * rescaled to exactly T with 3N - 3 degrees of freedom.  *n_out receives N
 * (MDG_ERR_ARG when above the system's capacity). */
#define MDG_GEN_MAX_TYPES 8
typedef struct mdg_fcc_spec {
    double density;          /* reduced number density rho */
    double temperature;      /* T (reduced units) */
    double mass;             /* atom mass (every type without its own) */
    double skin;             /* cutoff_radius of every atom (the lattice skin) */
    uint64_t seed;
    int32_t n_types;         /* 0 or 1: every atom type 0 */
    double type_fractions[MDG_GEN_MAX_TYPES];  /* cumulative thresholds */
    double type_masses[MDG_GEN_MAX_TYPES];     /* > 0: that type's mass */
} mdg_fcc_spec;
int  mdg_generate_fcc(mdg_ctx* ctx, int sys, const mdg_fcc_spec* spec, size_t* n_out);

/* Granular gas of a DEM system: the acceptance rule of insert.rs:523-571 over
 * the proposal stream g = 0, 1, ... (centre uniform in the box of the system's
 * config, inset by rmax when `inset`, from draws 4g..4g+2 of stream 1; radius
 * rmin + (rmax - rmin) u from draw 4g+3), placed by a grid-parallel random
 * sequential addition whose result equals the sequential one on that stream;
 * tags in acceptance order.  Velocities by velocity_mode from stream 2:
 * MDG_VEL_SPEED |v| = speed in an isotropic direction (z = 1 - 2 u_{4k},
 * azimuth 2 pi u_{4k+1}); MDG_VEL_MAXWELL_RMS Gaussian components of sigma
 * speed / sqrt(3); MDG_VEL_GAUSSIAN sigma = speed per component (the
 * reference's `velocity`, insert.rs:580-592).  omega 0, identity quaternions,
 * mass density 4/3 pi r^3 and 1 / (0.4 m r^2) as insert.rs:343-349,
 * cutoff_radius = r, type = material.  *placed receives the spheres placed;
 * MDG_ERR_ARG (and nothing written) when fewer than n fit within
 * max_proposals (0 = 20000 n). */
enum { MDG_VEL_SPEED = 0, MDG_VEL_MAXWELL_RMS = 1, MDG_VEL_GAUSSIAN = 2 };
typedef struct mdg_gas_spec {
    size_t n;
    double rmin, rmax;       /* radius uniform in [rmin, rmax] */
    double density;          /* kg/m^3 */
    double sep_factor;       /* rejection distance sep_factor (r_i + r_j); the reference uses 1.1 */
    int32_t inset;
    int32_t velocity_mode;   /* MDG_VEL_* */
    double speed;
    uint32_t material;
    uint64_t seed;
    uint64_t max_proposals;
} mdg_gas_spec;
int  mdg_generate_gas(mdg_ctx* ctx, int sys, const mdg_gas_spec* spec, size_t* placed);

#ifdef __cplusplus
}
#endif
#endif /* MDG_H */
