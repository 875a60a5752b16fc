/*
 * mdg_oracle.h -- C interface of the CPU FP64 oracle.
 *
 * TEST INFRASTRUCTURE ONLY. The oracle is a plain C++17 restatement of
 * MDDEM's single-rank CPU path for the particle hot path (periodic ghosts,
 * bin sort, half neighbor list, Hertz-Mindlin / Hooke contact with history,
 * LJ 12-6, velocity Verlet, rotational Verlet, Nose-Hoover, plane walls and
 * fixed boundaries, Langevin).  It is used by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU baseline leg as the
 * checker, never as the product path.
 *
 * Parity pin: the reference (Rust, un-vendored git dependency grass @ ea21ea36)
 * cannot be built here, so the oracle is pinned against the known-answer tests
 * held in the reference's own unit tests (analytic Hertz force, Verlet exact
 * values, rotational kick, beta(e) formula, bin list vs brute force), restated
 * in tests/test_kat.py and tests/golden/; walls by the reference's sphere-wall
 * rebound benchmark bounds (tests/test_walls.py).
 */
#ifndef MDG_ORACLE_H
#define MDG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_material {
    double youngs_mod, poisson_ratio, restitution, friction;
    double rolling_friction, twisting_friction, cohesion_energy, surface_energy;
    double kn, kt, rolling_stiffness, rolling_damping, twisting_stiffness, twisting_damping;
} orc_material;

/* One plane wall ([[wall]], dem_wall/src/lib.rs:160-260): a point, a normal
 * (normalised here, lib.rs:1259), the bounding region, a constant velocity and
 * a material index. */
typedef struct orc_wall {
    double point[3], normal[3], bound_lo[3], bound_hi[3], velocity[3];
    int material;
} orc_wall;

/* One LJ type pair: epsilon, sigma, cutoff in units of sigma
 * (LJPairCoeffs::from_params, md_lj/src/lib.rs:226-238). */
typedef struct orc_lj_pair {
    double epsilon, sigma, cutoff;
} orc_lj_pair;

typedef struct orc_config {
    int kind;                 /* 0 = DEM granular, 1 = LJ */
    double lo[3], hi[3];      /* [domain] */
    double dt;                /* [run] dt */
    double skin_fraction;     /* [neighbor] */
    double bin_size;
    int every, check, sort_every, newton;
    int n_materials;          /* [[dem.materials]] */
    const orc_material* materials;
    int contact_model;        /* 0 hertz, 1 hooke */
    int adhesion_model;       /* 0 jkr, 1 dmt */
    int rolling_model;        /* 0 constant, 1 sds */
    int twisting_model;       /* 0 constant, 1 sds */
    double lj_epsilon, lj_sigma, lj_cutoff;   /* [lj] single type */
    int nose_hoover;          /* 1 = NoseHooverPlugin present */
    double nh_temperature, nh_coupling;
    int virial;               /* VirialStress active each step */
    int fixed[3];             /* boundary_x/y/z = "fixed" (0 = periodic) */
    int n_walls;              /* plane walls (DEM) */
    const orc_wall* walls;
    /* [langevin] (md_thermostat/src/lib.rs:529-581); the N(0,1) draws come
     * from the counter-based stream the device uses, keyed by (seed, step,
     * tag, component), instead of the reference's ChaCha8 stream */
    int langevin;
    double lv_temperature, lv_damping;
    uint64_t lv_seed;
    /* [lj] multi-type mode: n_lj_types > 1 gives the n x n pair table
     * (row-major; build_lj_pair_table, md_lj/src/lib.rs:334-384) and
     * pair_table.get(type_i, type_j) picks each pair's coefficients */
    int n_lj_types;
    const orc_lj_pair* lj_pairs;
} orc_config;

enum {
    ORC_F_POS = 0, ORC_F_VEL = 1, ORC_F_FORCE = 2, ORC_F_OMEGA = 3, ORC_F_TORQUE = 4,
    ORC_F_QUAT = 5, ORC_F_MASS = 6, ORC_F_RADIUS = 7, ORC_F_LAST_BUILD_POS = 8
};

void*  orc_create(const orc_config* cfg);
void   orc_destroy(void* h);
/* Load nlocal particles (SoA, xyz interleaved per particle).  DEM arrays may be
 * NULL for LJ.  image may be NULL (zeros). */
int    orc_load(void* h, size_t n, const uint32_t* tag, const uint32_t* type,
                const double* pos, const double* vel, const double* mass,
                const double* cutoff_radius, const double* radius,
                const double* density, const double* inv_inertia,
                const double* omega, const double* quat);
/* Set the current force (and torque, DEM) of local atom i (restart state). */
int    orc_set_force(void* h, size_t i, const double* f3, const double* t3);
/* Advance nsteps full timesteps (reference schedule order). */
int    orc_step(void* h, long nsteps);
/* Ghost rebuild + bin list + force evaluation at the current state, no
 * integration (single-step force parity). */
int    orc_force_only(void* h);
size_t orc_nlocal(void* h);
/* Copy a per-local-atom field out (3 or 4 doubles per atom). */
int    orc_get_field(void* h, int field, double* out);
int    orc_get_tags(void* h, uint32_t* out);
/* Per local atom: sum over its pairs of |f_pair| and of |tau_pair| at the
 * last force evaluation (either array may be NULL); the normaliser of the
 * per-particle force and torque error metric. */
int    orc_get_scale(void* h, double* fs, double* ts);
/* Per-local-atom type index (material for DEM, LJ type for LJ). */
int    orc_get_types(void* h, uint32_t* out);
int    orc_get_image(void* h, int32_t* out);
/* Half-list pairs as (owner tag, partner tag); returns count, fills up to cap. */
size_t orc_get_pairs(void* h, uint32_t* out, size_t cap);
/* Contact history: (owner tag, partner tag) + 7 doubles per entry. */
size_t orc_get_history(void* h, uint32_t* keys, double* vals, size_t cap);
/* Inject history entries (owner tag, partner tag, 7 doubles). */
int    orc_set_history(void* h, size_t n, const uint32_t* keys, const double* vals);
/* thermo: [ke, pe, temp(3N-3), p_xi, granular_temp, |momentum|,
 *          vxx, vyy, vzz, vxy, vxz, vyz, nbuilds, step, ndof, q_mass] */
int    orc_thermo(void* h, double* out16);
long   orc_overlap_count(void* h);
/* LJ long-range tail corrections E_tail, P_tail (equimolar weights over the
 * type pairs, setup_lj_tails). */
int    orc_lj_tails(void* h, double* e_tail, double* p_tail);
/* Seeded random sequential addition of spheres, the same stream and
 * acceptance rule as the library's mdg_rsa_spheres (same seed, same spheres):
 * inputs for the CPU arm made without the library.  Returns 0 when all n fit. */
int    orc_rsa_spheres(size_t n, const double* box_lo, const double* box_hi, double rmin, double rmax,
                       double sep_factor, int inset, uint64_t seed, uint64_t max_attempts, double* pos,
                       double* rad, size_t* placed);

#ifdef __cplusplus
}
#endif
#endif
