/*
 * rdsim.h -- C ABI of the GB300 simulation-step engine for PyRDSim decks.
 *
 * The reference (PyRDSim, a single Cython class `system`) has no C FFI: its
 * step engine is the private methods of `system` (pyrdsim/pyrdsim.pyx).
 * Each entry point below replaces one of those methods, cited as
 * pyrdsim.pyx:<line>; the Python package `pyrdsim_gb300` binds them with
 * ctypes behind a `system(...).simulate()` class that mirrors the reference.
 *
 * Conventions
 *  - Every function returns an rdsim status code (0 = ok).  A failing call
 *    stores a message readable with rdsim_last_error().
 *  - All pointers are HOST pointers unless a flag says otherwise.  Particle
 *    arrays are in the caller's particle order (the order of the initial
 *    condition file), systems concatenated in the order given to
 *    rdsim_create().
 *  - One handle owns its device memory and one CUDA stream; calls on one
 *    handle are not re-entrant.  Host-visible results are synchronous.
 *  - Positions are float64 at the boundary.  On the device they are held as
 *    64-bit fixed point per dimension (exact periodic wrap); pair and bonded
 *    forces are float32; reaction propensities and draws are float64.
 */
#ifndef RDSIM_H
#define RDSIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RDSIM_MAX_DIM 3
#define RDSIM_MAX_TYPES 16
#define RDSIM_MAX_REACTIONS 8
#define RDSIM_MAX_INTERACTIONS 32
#define RDSIM_MAX_ATOMS 32

/* ---- status codes ------------------------------------------------------ */
enum {
  RDSIM_OK = 0,
  RDSIM_ERR_ARG = 1,          /* invalid argument / inconsistent deck        */
  RDSIM_ERR_CUDA = 2,         /* CUDA runtime error                          */
  RDSIM_ERR_NOMEM = 3,        /* device allocation failed                    */
  RDSIM_ERR_UNSUPPORTED = 4,  /* deck outside what the engine implements     */
  RDSIM_ERR_OUT_OF_BOUNDS = 16, /* particle outside the box (pyrdsim.pyx:2287) */
  RDSIM_ERR_ANGLE_DOMAIN = 17,  /* cos(angle) < -1.0000001 (pyrdsim.pyx:1365) */
  RDSIM_ERR_SKIN = 18,        /* a particle moved more than half the skin
                                 (Euclidean; dim = -1) between two rebuilds */
  RDSIM_ERR_NONFINITE = 19,   /* non-finite or larger-than-box displacement  */
  RDSIM_ERR_CAPACITY = 20,    /* a per-call buffer was too small             */
  RDSIM_ERR_SYNC = 21         /* a wait of the period kernel on the progress
                                 of neighbouring chunks ran out (no GPU hang:
                                 every CTA gives up and returns)           */
};

/* ---- model description (parsed decks) ---------------------------------- */

/* Nonbonded interaction laws, pyrdsim.pyx:1068-1145.  Each law returns the
 * force magnitude f = dU/dr applied as a_i += f * (x_j - x_i)/r
 * (pyrdsim.pyx:2025-2031); walls act on one coordinate, a_i[d] -= f.      */
enum {
  RDSIM_LAW_LJ = 1,               /* f = -2 n u0 / r * s (s - 1), s = (r0/r)^n */
  RDSIM_LAW_TANH = 2,             /* f = u0 (1 - tanh^2((r-r0)/a)) / (2a)      */
  RDSIM_LAW_YUKAWA = 3,           /* f = -u0 (1 + r0/r) exp(-r/r0) / (r r0)    */
  RDSIM_LAW_HARMONIC = 4,         /* f = u0 r                                  */
  RDSIM_LAW_PIECEWISE_LINEAR = 5, /* f = 0 if r < r0-dr else u0/dr; rc = r0    */
  RDSIM_LAW_WALL = 6,             /* tanh wall on x_d, no cutoff               */
  RDSIM_LAW_WALL93 = 7            /* 9-3 wall U = u0[(2/15)(r0/y)^9-(r0/y)^3],
                                     y = x_d, cut at rc (not in the reference) */
};

typedef struct {
  int32_t law;      /* RDSIM_LAW_*                                           */
  int32_t type_a;   /* pair types as listed (pair = a b); wall: particle type */
  int32_t type_b;   /* wall: direction (dimension index)                     */
  int32_t n;        /* LJ exponent                                           */
  double u0, r0, rc, a, dr;
} rdsim_interaction;

/* Reactions, pyrdsim.pyx:2070-2223. */
enum { RDSIM_RX_LINEAR = 1, RDSIM_RX_CATALYZED = 2, RDSIM_RX_INHIBITED = 3 };

typedef struct {
  int32_t kind;                 /* RDSIM_RX_*                                */
  int32_t reactant, product;
  int32_t catalyst;             /* -1 if unused                              */
  int32_t inhibitor, inhibitor2;/* -1 if unused                              */
  double rate, r0, rate_decrease;
} rdsim_reaction;

/* Bonded terms of one molecule template, pyrdsim.pyx:823-1034, 1268-1408. */
enum { RDSIM_TERM_BOND = 1, RDSIM_TERM_ANGLE = 2 };

typedef struct {
  int32_t kind;   /* RDSIM_TERM_*                                            */
  int32_t i, j, k;/* atom indices within the molecule (k unused for bonds)   */
  double p0;      /* bond: r0.  angle: theta0 in radians                     */
  double k0;      /* bond: U0.  angle: k * (180/pi)^2                        */
} rdsim_term;

typedef struct {
  int32_t molecule_id, n_atoms, first_term, n_terms;
} rdsim_template;

/* One independent system: the content of the four decks plus the initial
 * condition file (pyrdsim.pyx:406-587, 1790-1912). */
typedef struct {
  int32_t n_dim;                   /* 2 or 3                                  */
  int32_t n_types;                 /* len(tau_by_tauD)                        */
  int32_t n_particles;
  int32_t n_molecules;
  double L[RDSIM_MAX_DIM];
  double periodic[RDSIM_MAX_DIM];  /* > 0 periodic, < 0 reflecting            */
  double dt;
  double rs;                       /* neighbour-list radius (pyrdsim.pyx:578) */
  int32_t cell_length_ratio;       /* pyrdsim.pyx:327, 575                    */
  int32_t neighbor_list_update_frequency; /* pyrdsim.pyx:325, 584          */
  int32_t angle_is_pi;             /* +1 / -1: the theta0 == pi flag that every
                                      angle term reads (pyrdsim.pyx:1350-1401:
                                      the flag of the last angle defined);
                                      0: each angle term uses its own
                                      theta0 == pi test (no late binding)   */
  int32_t n_interactions, n_reactions, n_templates, n_terms;
  const double* tau_by_tauD;       /* [n_types]                               */
  const rdsim_interaction* interactions; /* file order                       */
  const rdsim_reaction* reactions; /* file order                             */
  const rdsim_template* templates;
  const rdsim_term* terms;
  const double* x;                 /* [n_particles][n_dim]                    */
  const int32_t* particle_types;   /* [n_particles]                           */
  const int32_t* molecule_ids;     /* [n_particles][3]: molecule number, index
                                      in molecule, molecule id (template)     */
  const int32_t* first_index_of_molecule; /* [n_molecules]                    */
  uint64_t seed;                   /* counter-based noise key                 */
} rdsim_system;

/* ---- engine ------------------------------------------------------------ */

typedef struct rdsim_handle rdsim_handle;

typedef struct {
  int32_t device;                 /* CUDA device ordinal                      */
  double skin;                    /* cell skin in length units; <= 0: auto    */
  int32_t threads_per_particle;   /* lanes sharing one particle's list: 1, 2,
                                     4 or 8; other values: 2                  */
  int32_t force_precision;        /* 0: float32 pair and bonded forces from
                                     the pair words (the default); 1: float64
                                     forces, drift and increments with the
                                     reference's formulas (the plain method) */
  int32_t use_graphs;             /* >= 0: replay whole rebuild periods as CUDA
                                     graphs (Philox noise); < 0: plain launches */
  int32_t list_width;             /* Verlet-list entries stored per particle;
                                     0: auto.  Longer rows are regenerated from
                                     the cells each step (same results)       */
  int32_t reaction_prefilter;     /* the drift kernel bounds each particle's
                                     next reaction draw; the reaction kernel
                                     then visits only the particles whose draw
                                     may succeed (same results).  0: when few
                                     draws are expected to pass the bound;
                                     > 0: whenever the rates allow; < 0: off  */
  int32_t period_kernel;          /* >= 0: graph-replayed rebuild periods run
                                     as one launch of the period kernel when
                                     every chunk of particles fits on the GPU
                                     at once (same results); < 0: one drift
                                     and one reaction launch per step        */
  int32_t sync_wait_ms;           /* limit of one wait of the period kernel on
                                     its neighbouring chunks; <= 0: 1000 ms   */
  int32_t list_period;            /* steps between the engine's neighbour-list
                                     rebuilds; <= 0: the deck's
                                     neighbor_list_update_frequency.  The
                                     automatic skin covers the diffusion of
                                     one period and the displacement check
                                     keeps every pair in range listed, so the
                                     forces do not depend on it (float32 sums
                                     in another order)                       */
  int32_t reserved[2];
} rdsim_options;

/* rdsim_step flags */
enum {
  RDSIM_STEP_NO_NOISE = 1,       /* random_force=False (pyrdsim.pyx:2341)    */
  RDSIM_STEP_INJECT_HOST = 2,    /* xi/u1/u2 are host arrays                 */
  RDSIM_STEP_INJECT_DEVICE = 4   /* xi/u1/u2 are device arrays               */
};

/* Replaces simulate()'s set-up: set_parameters (pyrdsim.pyx:406-587),
 * create_arrays (1658), set_up_neighbor_list_cells (1415),
 * create_bond_and_angle_force_functions (1268), and the initial
 * create_neighbor_list + update_drifts (2398-2401).  Several systems may be
 * batched into one handle; they are stepped together. */
int rdsim_create(const rdsim_system* systems, int32_t n_systems,
                 const rdsim_options* options, rdsim_handle** out);

/* Releases the handle's device memory and stream. */
int rdsim_destroy(rdsim_handle* h);

/* Replaces the loop body of simulate() (pyrdsim.pyx:2410-2426): n_steps calls
 * of integration_step (pyrdsim.pyx:2296-2322): Euler-Maruyama update
 * (2225-2250), boundary conditions (2253-2292), neighbour-list rebuild every
 * neighbor_list_update_frequency steps (1448-1587), reactions (2070-2223)
 * and drift (1941-2067).
 * Noise: by default counter-based Philox4x32-10 keyed by (seed, step,
 * particle).  With RDSIM_STEP_INJECT_*, xi[n_steps][N][n_dim] supplies the
 * standard normals and u1[n_steps][N], u2[n_steps][N] the reaction uniforms
 * (u2 is read only for particles that react), N = total particles. */
int rdsim_step(rdsim_handle* h, int32_t n_steps, int32_t flags,
               const double* xi, const double* u1, const double* u2);

/* Replaces the state load of simulate() (pyrdsim.pyx:1790-1912, 1703-1723):
 * sets positions [N][n_dim] and types [N] (either may be NULL to keep),
 * rebuilds the neighbour list and recomputes the drift. */
int rdsim_set_state(rdsim_handle* h, const double* x, const int32_t* types);

/* Current positions [N][n_dim] and types [N] (either may be NULL); the
 * dictionary entries 'x' and 'particle_types' of simulate() (2446-2456). */
int rdsim_get_state(rdsim_handle* h, double* x, int32_t* types);

/* Drift a = -grad U at the current state [N][n_dim] (self.a, 1941-2067). */
int rdsim_get_drift(rdsim_handle* h, double* a);

/* Total reaction propensity per particle [N] (total_reaction_rates,
 * pyrdsim.pyx:2070-2206) at the current positions and types. */
int rdsim_get_reaction_rates(rdsim_handle* h, double* total);

/* Neighbour list of system `sys` as if rebuilt now (create_neighbor_list,
 * 1448-1587): pairs (i<j), indices local to the system, written as
 * pairs[2*p], pairs[2*p+1], sorted.  *n_pairs receives the count; returns
 * RDSIM_ERR_CAPACITY if it exceeds cap (nothing is written then). */
int rdsim_get_pairs(rdsim_handle* h, int32_t sys, int32_t* pairs,
                    int64_t cap, int64_t* n_pairs);

/* No counterpart in the reference.  The same sorted pair list as
 * rdsim_get_pairs, for callers that cannot allocate device memory: processes
 * whose device memory is already committed (a preallocated pool, another
 * framework's cache), where cudaMalloc fails, and loops that must not pay the
 * device-wide synchronisation of cudaFree.  It calls no cudaMalloc/cudaFree:
 * its scratch is a static device array of RDSIM_STATIC_PAIRS_MAX pairs
 * (8 MiB, held by every GPU that loads the library until exit).  More pairs
 * than that return RDSIM_ERR_CAPACITY.  The first call on a device (and the
 * first after its context is recreated, e.g. by cudaDeviceReset) looks the
 * array up and loads the pair kernels of every dimension.  Concurrent calls
 * race on the shared array. */
#define RDSIM_STATIC_PAIRS_MAX (1LL << 20)
int rdsim_get_pairs_static(rdsim_handle* h, int32_t sys, int32_t* pairs,
                           int64_t cap, int64_t* n_pairs);

/* Cell indices floor(x_k / cl_k) [n][n_dim] of system `sys` in the
 * reference's cell geometry (pyrdsim.pyx:1415-1446, 1506-1508). */
int rdsim_get_cell_ids(rdsim_handle* h, int32_t sys, int32_t* cell_ids);

/* ---- observables (no reference counterpart except min_distance) --------
 * Float64 reductions over system `sys` at the current state, computed on the
 * device.  Energies are the potentials whose derivatives are the
 * reference's force laws (pyrdsim.pyx:1068-1145, 2037-2066), each truncated
 * (not shifted) where its force stops:
 *   lj                U = u0 [(r0/r)^2n - 2 (r0/r)^n]            r <= rc
 *   tanh              U = (u0/2) [tanh((r - r0)/a) - 1]          r <= rc
 *   yukawa            U = u0 exp(-r/r0) / r                      r <= rc
 *   harmonic          U = u0 r^2 / 2                             r <= rc
 *   piecewise_linear  U = (u0/dr) (r - r0) on [r0 - dr, r0], -u0 below
 *   tanh wall         U = (u0/2) [tanh((x_d - r0)/a) - 1]
 *   9-3 wall          U = u0 [(2/15)(r0/y)^9 - (r0/y)^3]         y <= rc
 *   bond              U = U0 (d - r0)^2 / 2
 *   angle             U = k (theta - theta0)^2 / 2  (k in the deck's
 *                                                    per-radian^2 units)
 * Pair terms run over the pairs whose forces the drift applies: listed
 * pairs of different molecules, each law of their (small, large) type pair
 * within its cutoff.  virial = sum over those pairs and the bonds of
 * -r dU/dr (angle terms contribute nothing, walls are external).
 * min_distance is the smallest distance between listed interaction or
 * reaction partners of different molecules: pairs within the Verlet-list
 * radius (interaction range + skin) at the last rebuild; +inf if there is
 * none.  At a rebuild it equals the reference's min_dist
 * (pyrdsim.pyx:1640-1652) whenever that is below the interaction range. */
typedef struct {
  double pair_energy, wall_energy, bond_energy, angle_energy;
  double virial;
  double min_distance;
  int64_t n_pairs;      /* particle pairs within the cutoff of one of their
                           pair laws                                        */
  int64_t n_particles;
  int64_t type_counts[RDSIM_MAX_TYPES];  /* particles of each current type */
} rdsim_observables;
int rdsim_get_observables(rdsim_handle* h, int32_t sys, rdsim_observables* out);

/* Pair-distance histogram of system `sys` (for g(r)): counts[b] += 1 for
 * every unordered particle pair of types {type_a, type_b} (-1: any type)
 * at float64 distance r < r_max (minimum image in periodic dimensions),
 * b = floor(r / (r_max / n_bins)).  With RDSIM_RDF_OTHER_MOLECULES only
 * pairs of different molecules count.  r_max must not exceed half of any
 * periodic box length; 1 <= n_bins <= 16384.  counts[n_bins] is
 * overwritten. */
enum { RDSIM_RDF_OTHER_MOLECULES = 1 };
int rdsim_get_rdf(rdsim_handle* h, int32_t sys, int32_t type_a, int32_t type_b,
                  double r_max, int32_t n_bins, int32_t flags, int64_t* counts);

/* Step counter (the reference's `step` argument of integration_step); the
 * next rdsim_step performs step counter+1.  Sets it for append mode. */
int rdsim_get_step(rdsim_handle* h, int64_t* step);
int rdsim_set_step(rdsim_handle* h, int64_t step);

/* Trajectory ring on the device (simulate(), pyrdsim.pyx:2429-2444): every
 * `stride`-th step stores positions and types in frame (step/stride-1) %
 * n_frames.  n_frames == 0 disables it. */
int rdsim_set_trajectory(rdsim_handle* h, int32_t stride, int32_t n_frames);
int rdsim_get_trajectory(rdsim_handle* h, double* x, int32_t* types);

/* First error recorded on the device since the last call: *code is an
 * RDSIM_ERR_* (0 if none); for RDSIM_ERR_OUT_OF_BOUNDS, particle index,
 * dimension and value are filled like the reference's message. */
int rdsim_get_error(rdsim_handle* h, int32_t* code, int64_t* particle,
                    int32_t* dim, double* value, int64_t* step);

/* CUDA stream (cudaStream_t) that all work of the handle runs on. */
int rdsim_get_stream(rdsim_handle* h, void** stream);

/* Engine geometry chosen at create time, for reports: cells, CTAs per step
 * kernel, lanes per particle, Verlet-list width, skin, cell size. */
typedef struct {
  int64_t n_particles, n_cells, n_blocks;
  int32_t threads_per_particle, list_width;
  double skin, cell_size_min, interaction_range;
  int64_t device_bytes;
  int32_t reaction_prefilter;     /* 1: on for this handle                    */
  int32_t force_precision;        /* as in rdsim_options                      */
  int32_t period_kernel;          /* 1: rebuild periods replay as one launch of
                                     the period kernel                       */
  int32_t list_period;            /* steps between Verlet-list rebuilds     */
} rdsim_info;
int rdsim_get_info(rdsim_handle* h, rdsim_info* info);

/* Kernel accounting (no reference counterpart; measurement only).  Launch
 * counts are always kept.  With bit 0 of `enable` every kernel launch is also
 * bracketed by CUDA events on the handle's stream and its device time summed
 * per class: 0 = drift (k_force_l), 1 = reactions (k_react_l,
 * k_react_listed), 2 = stand-alone Euler-Maruyama (k_em), 3 = cell-list and
 * Verlet-list rebuild (6 kernels), 4 = hooks and observables (the events
 * serialise launches and keep graphs from replaying).  With bit 1 the drift
 * kernel itself (the period kernel alone, when rdsim_get_info reports it)
 * records the global timer when each CTA starts its work (after waiting for
 * the previous kernel) and when each of its warps ends; drift_span_ms sums,
 * per launch, last end minus first start over the last drift_spans launches
 * (up to 32768 kept), without changing how the step runs (graphs replay). */
#define RDSIM_PROFILE_CLASSES 5
typedef struct {
  int64_t launches[RDSIM_PROFILE_CLASSES];
  double ms[RDSIM_PROFILE_CLASSES];
  int64_t timed[RDSIM_PROFILE_CLASSES];
  double drift_span_ms;
  int64_t drift_spans;
} rdsim_profile;
int rdsim_set_profiling(rdsim_handle* h, int32_t enable);
/* Fills *p and resets the counters (synchronises the stream). */
int rdsim_get_profile(rdsim_handle* h, rdsim_profile* p);

/* Test hook, no counterpart in the reference: chunk `chunk` (a CTA of the
 * period kernel) stops publishing its progress, so that the waits of its
 * neighbours run out after sync_wait_ms and the next rdsim_step returns
 * RDSIM_ERR_SYNC.  -1 restores normal operation. */
int rdsim_test_withhold(rdsim_handle* h, int32_t chunk);

/* Message of the last failing call on this thread. */
const char* rdsim_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* RDSIM_H */
