/* flygpu.h -- C ABI of the GB300 (sm_103a) saddle-search inner loop.
 *
 * The reference (openFLY) runs this path in C++ behind three interfaces:
 *   fly::neigh::List            include/libfly/neigh/list.hpp:71-211
 *   fly::potential::EAM/Generic include/libfly/potential/EAM/eam.hpp:42-120, potential/generic.hpp:50-140
 *   fly::saddle::Dimer / fly::minimise::LBFGS
 *                               include/libfly/saddle/dimer.hpp:51-170, minimise/LBFGS/lbfgs.hpp:48-128
 * Each entry point below names the reference member it replaces. Conventions:
 *   - every function returns an int status (FLYGPU_OK = 0); flygpu_last_error() gives detail;
 *   - host arrays use the reference's layout: positions, axes, deltas and gradients are interleaved
 *     xyz doubles, 3 per atom (system/adaptor.hpp:77); types are uint32 (TypeID, property.hpp:113);
 *     frozen flags are one byte per atom (Frozen, property.hpp:192);
 *   - "_device" variants take device pointers of the same layout and do not synchronise;
 *   - handles are not thread-safe: use one per host thread (the reference keeps one potential and one
 *     List per OpenMP thread, saddle/find.hpp:310-317). The server handle is internally synchronised.
 */
#ifndef FLYGPU_H
#define FLYGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum flygpu_status_code {
  FLYGPU_OK = 0,
  FLYGPU_INVALID_ARG = 1,     /* fly::RuntimeError from verify() (utility/core.hpp:89-137) */
  FLYGPU_SPLINE_OOB = 2,      /* Spline::OutOfBounds (utility/spline.hpp:46-51,141-143) */
  FLYGPU_GHOST_OVERFLOW = 3,  /* more than List::MAX_GHOST_RATIO * n ghosts (neigh/list.hpp:78) */
  FLYGPU_NLIST_OVERFLOW = 4,  /* neighbour capacity exceeded after one automatic regrow */
  FLYGPU_OOM = 5,             /* device or pinned allocation failed */
  FLYGPU_TIMEOUT = 6,         /* a search hit its device-side iteration budget */
  FLYGPU_CUDA_ERROR = 7       /* any other CUDA runtime error */
};

/* Arithmetic of the EAM passes. FP64: every operation in binary64 without contraction, the
 * reference's arithmetic. MIXED: spline lookups and pair terms in binary32, per-atom density,
 * energy and force accumulators in binary64. */
enum flygpu_precision { FLYGPU_FP64 = 0, FLYGPU_MIXED = 1 };

/* Dimer::Exit (saddle/dimer.hpp:123-129) */
enum flygpu_exit { FLYGPU_EXIT_SUCCESS = 0, FLYGPU_EXIT_CONVEX = -1, FLYGPU_EXIT_ITER_MAX = -2,
                   FLYGPU_EXIT_COLLISION = -3, FLYGPU_EXIT_UNINIT = -4 };

typedef struct flygpu_eam flygpu_eam;
typedef struct flygpu_list flygpu_list;
typedef struct flygpu_server flygpu_server;

const char* flygpu_status_string(int status);
/* Message of the last failing call on this host thread ("" if none). */
const char* flygpu_last_error(void);
/* Number of CUDA kernels this library has launched since it was loaded (all threads). No reference
 * counterpart: instrumentation for throughput accounting. */
int64_t flygpu_launch_count(void);

/* ---------------------------------------------------------------- EAM tables
 * Replaces DataEAM::DataEAM (potential/EAM/data.hpp:54, src/potential/EAM/data.cpp:67-153): parses a
 * LAMMPS eam/fs file, builds the natural cubic splines (utility/spline.hpp:66, spline.cpp:27-103)
 * on the host and uploads binary64 and binary32 coefficient tables. */
int flygpu_eam_load(const char* path, flygpu_eam** out);
void flygpu_eam_destroy(flygpu_eam* eam);
/* EAM::r_cut (potential/EAM/eam.hpp:71) */
double flygpu_eam_r_cut(const flygpu_eam* eam);
int flygpu_eam_n_types(const flygpu_eam* eam);
/* Host copy of one function's binary64 coefficients {a,b,c,d} per interval: kind 0 = F(type a),
 * 1 = phi(a, b), 2 = v(a, b). Returns the interval count; copies if cap >= 4 * count. */
int64_t flygpu_eam_table(const flygpu_eam* eam, int kind, int a, int b, double* out, int64_t cap);
/* Spline::Spline (src/utility/spline.cpp:27-103) on the host, the construction every EAM table goes
 * through: the natural cubic spline of n >= 2 samples y spaced dx, padded with 5 copies of the last
 * sample. Returns the interval count (n + 4); copies the binary64 {a,b,c,d} per interval if
 * cap >= 4 * count. Needs no GPU. */
int64_t flygpu_spline_build(const double* y, int64_t n, double dx, double* out, int64_t cap);

/* ---------------------------------------------------------------- neighbour list
 * Replaces neigh::List::List(box, r_cut) (neigh/list.hpp:86-90) for an orthorhombic box
 * (system/boxes/orthorhombic.hpp:115-118). stream may be NULL (the handle then owns one). */
int flygpu_list_create(const double extents[3], const int periodic[3], double r_cut, void* stream,
                       flygpu_list** out);
void flygpu_list_destroy(flygpu_list* list);
/* List::rebuild (neigh/list.hpp:98, src/neigh/list.cpp:53-95). pos: 3n doubles. */
int flygpu_list_rebuild(flygpu_list* list, const double* pos, int64_t n);
int flygpu_list_rebuild_device(flygpu_list* list, const double* d_pos, int64_t n);
/* List::update (neigh/list.hpp:118, src/neigh/list.cpp:37-51): r <- r - delta for real and ghost
 * atoms. delta: 3n doubles. The call returns once the update is queued on the list's stream; a delta in
 * pinned (page-locked) host memory is copied asynchronously, so keep it unchanged until the list's next
 * synchronising call (any EAM call that returns results to the host). */
int flygpu_list_update(flygpu_list* list, const double* delta);
int flygpu_list_update_device(flygpu_list* list, const double* d_delta);
/* List::size (neigh/list.hpp:161) */
int64_t flygpu_list_size(const flygpu_list* list);
int64_t flygpu_list_num_ghosts(const flygpu_list* list);
/* Every (atom, neighbour) pair that List::for_neighbours (neigh/list.hpp:139-154) visits within
 * r_cut, in its visiting order: counts[n] per atom, then CSR real indices idx[] and dr[3*] (neighbour
 * minus atom). total receives the pair count; idx/dr are filled when cap >= total. */
int flygpu_list_neighbours(flygpu_list* list, double r_cut, int32_t* counts, int32_t* idx, double* dr,
                           int64_t cap, int64_t* total);
/* Per-kernel CUDA-event timing on the list's stream (no reference counterpart; the reference's only
 * instrumentation is timeit(), utility/core.hpp:888-921). Enabling clears earlier records.
 * kernel_times fills ms[4] / counts[4] for {density pass, force pass, update, rebuild} since the last
 * call and clears them. */
int flygpu_list_set_timing(flygpu_list* list, int enable);
int flygpu_list_kernel_times(flygpu_list* list, double* ms, int64_t* counts);
/* Wait for the list's stream and report the first device-side error raised since the last call. */
int flygpu_list_sync(flygpu_list* list);

/* ---------------------------------------------------------------- EAM energy / gradient
 * types (n uint32) and frozen (n bytes) are uploaded when non-NULL and reused when NULL. */
/* EAM::energy (potential/EAM/eam.hpp:83, src/potential/EAM/eam.cpp:33-51) */
int flygpu_eam_energy(flygpu_eam* eam, flygpu_list* list, const uint32_t* types, const uint8_t* frozen,
                      int precision, double* energy);
/* EAM::gradient (potential/EAM/eam.hpp:95, src/potential/EAM/eam.cpp:53-120). grad: 3n doubles. */
int flygpu_eam_gradient(flygpu_eam* eam, flygpu_list* list, const uint32_t* types, const uint8_t* frozen,
                        int precision, double* grad);
/* Both in one density pass + one force pass (energy may be NULL). A grad buffer in pinned host memory
 * receives the force pass's stores directly (the transfer overlaps the pass); other memory receives a
 * copy after it. Either way the call returns with the results in place. */
int flygpu_eam_energy_gradient(flygpu_eam* eam, flygpu_list* list, const uint32_t* types,
                               const uint8_t* frozen, int precision, double* energy, double* grad);
/* Device-pointer form of the above: d_types / d_frozen may be NULL (reuse), d_energy may be NULL. */
int flygpu_eam_energy_gradient_device(flygpu_eam* eam, flygpu_list* list, const uint32_t* d_types,
                                      const uint8_t* d_frozen, int precision, double* d_energy,
                                      double* d_grad);

/* EAM::hessian (potential/EAM/eam.hpp:110, src/potential/EAM/eam.cpp:122-233): the dense 3n x 3n
 * Hessian of the list's atoms in binary64, row-major, the rows 3a..3a+2 belonging to atom a. As in the
 * reference only the lower 3x3 blocks (a >= z) are written, and the blocks of frozen atoms are zero;
 * the values are the reference's, bit for bit. types (n) and frozen (n) are required; hess: 9 n^2
 * doubles on the host. Neighbours are taken within the potential's cut-off from the list as built.
 * The list keeps the device scratch for the next call (the dense matrix only while it is at most 1 GiB). */
int flygpu_eam_hessian(flygpu_eam* eam, flygpu_list* list, const uint32_t* types, const uint8_t* frozen,
                       double* hess);
/* Hessian::mass_weight then Hessian::eigenvalues (system/hessian.hpp:86-93,136-143) of that Hessian,
 * built, weighted and diagonalised on the device (the prefactor step of find.cpp:838-871 and
 * Master::calc_minima_hess, find.cpp:1094-1144). masses: one per type (n_types doubles), NULL for the
 * potential file's masses. eig: 3n doubles, ascending. hess (may be NULL): 9 n^2 doubles receiving the
 * mass-weighted matrix. The active atoms' block is diagonalised (at most 9000 coordinates, with a
 * Gershgorin norm below 2^30; FLYGPU_INVALID_ARG otherwise); each frozen coordinate adds an exact zero. */
int flygpu_hessian_eigenvalues(flygpu_eam* eam, flygpu_list* list, const uint32_t* types, const uint8_t* frozen,
                               const double* masses, double* eig, double* hess);

/* For callers that cannot allocate device memory (a host framework that owns every device allocation,
 * a real-time loop that must not touch the allocator after start-up, a caller holding only borrowed
 * device pointers). No reference counterpart. Computes the same energy and gradient as
 * flygpu_eam_energy_gradient with FLYGPU_FP64 for one system of at most FLYGPU_NOALLOC_MAX_ATOMS atoms,
 * from device inputs into device outputs, and allocates nothing: its scratch is a fixed array inside
 * the library (about 33 KB per GPU, held until the process exits) and pairs are found by a minimum-image
 * scan without a neighbour list (periodic extents must exceed twice the cut-off). The first call on
 * each device looks up that array's device address (and may load the library's device code on that
 * device), so make the first call before any stream capture. The address is kept for the life of the
 * process: it does not survive cudaDeviceReset. Calls share the array, so calls that overlap on the GPU
 * race. Every call copies the kernels' error word back to a host variable and waits for its stream to
 * finish before returning, so it can report spline and type errors. Larger systems are rejected with
 * FLYGPU_INVALID_ARG. d_pos: 3n doubles; d_grad: 3n doubles; d_energy: 1 double. */
#define FLYGPU_NOALLOC_MAX_ATOMS 4096
int flygpu_eam_energy_gradient_noalloc(const flygpu_eam* eam, const double* d_pos, const uint32_t* d_types,
                                       const uint8_t* d_frozen, int64_t n, const double extents[3],
                                       const int periodic[3], double* d_energy, double* d_grad, void* stream);

/* ---------------------------------------------------------------- perturbations
 * The random stream of Master (saddle/find.hpp:314): xoshiro256** 1.0 (utility/random.hpp:42-162),
 * 256 bits of state. The reference seeds thread 0's generator from std::random_device and thread k's
 * k long jumps further (find.cpp:188-193). These calls need no GPU. */
typedef struct {
  uint64_t s[4];
} flygpu_xoshiro;
/* Xoshiro::Xoshiro(seed) (random.hpp:72-76): an all-zero seed is rejected (FLYGPU_INVALID_ARG). */
int flygpu_xoshiro_seed(flygpu_xoshiro* prng, const uint64_t seed[4]);
/* Xoshiro::operator() (random.hpp:94-109) */
uint64_t flygpu_xoshiro_next(flygpu_xoshiro* prng);
/* Xoshiro::long_jump (random.hpp:130-132): 2^192 outputs ahead. */
void flygpu_xoshiro_long_jump(flygpu_xoshiro* prng);
/* count draws of one std::normal_distribution<double>(mean, stddev) object from prng, as libstdc++
 * produces them (Marsaglia's polar method, the second value of each pair cached for the next draw).
 * The draws Master::perturb makes come from three such objects (find.cpp:1152-1164). */
int flygpu_normal_draws(flygpu_xoshiro* prng, double mean, double stddev, int64_t count, double* out);
/* Master::perturb (saddle/find.cpp:1147-1214): out_pos = in_pos with Gaussian noise of a stddev drawn
 * from N(stddev, stddev / 3) (redrawn while negative), scaled by 1 - r / r_pert, on every unfrozen
 * neighbour of `centre` within r_pert in nl_pert's List::for_neighbours order, and unscaled on the
 * centre; out_axis = Gaussian components on the same atoms, normalised over all 3n. nl_pert is a list
 * of cut-off >= r_pert rebuilt on in_pos (find.cpp:217-219). Draws from prng in the reference's order;
 * stddev_used (may be NULL) receives the stddev drawn. */
int flygpu_perturb(flygpu_list* nl_pert, int64_t centre, const double* in_pos, const uint8_t* frozen, int64_t n,
                   double stddev, double r_pert, flygpu_xoshiro* prng, double* out_pos, double* out_axis,
                   double* stddev_used);

/* ---------------------------------------------------------------- searches */

/* Dimer::Options (saddle/dimer.hpp:56-98) then Rotor::Options (saddle/rotor.hpp:47-60). */
typedef struct {
  int n, max_steps, hist_check_freq, use_history;
  double f2norm, skin_frac, proj_tol, max_trust, min_trust, grow_trust, shrink_trust, convex_max;
  int rot_n, iter_max_rot, relax_in_convex, pad_;
  double delta_r, theta_tol;
} flygpu_dimer_options;

/* LBFGS::Options (minimise/LBFGS/lbfgs.hpp:56-80). */
typedef struct {
  int n, iter_max;
  double f2norm, skin_frac, proj_tol, max_trust, min_trust, grow_trust, shrink_trust;
} flygpu_lbfgs_options;

/* The reference's defaults. */
void flygpu_dimer_options_default(flygpu_dimer_options* opt);
void flygpu_lbfgs_options_default(flygpu_lbfgs_options* opt);

enum flygpu_search_mode { FLYGPU_SEARCH_DIMER = 0, FLYGPU_SEARCH_MINIMISE = 1 };

/* One search: the arguments of Dimer::find_sp (saddle/dimer.hpp:148-155) or LBFGS::minimise
 * (minimise/LBFGS/lbfgs.hpp:115-118) for one system. Host arrays; copied by the call taking them. */
typedef struct {
  int64_t n;               /* atoms */
  const double* pos;       /* 3n Position */
  const double* axis;      /* 3n Axis (dimer); NULL for a minimisation */
  const uint32_t* types;   /* n TypeID */
  const uint8_t* frozen;   /* n Frozen */
  double extents[3];       /* orthorhombic box */
  int periodic[3];
  int mode;                /* flygpu_search_mode */
  int n_hist;              /* previously found saddle points (hist_sp, dimer.cpp:102-131) */
  const double* hist;      /* n_hist * 3n */
  const double* in_min;    /* 3n minimum the dimer climbs from; NULL = pos */
  double theta_tol;        /* collision angle in radians (find.cpp:692) */
} flygpu_search_desc;

typedef struct {
  int exit_code;     /* Dimer::Exit, or for a minimisation 0 = converged, 1 = not (lbfgs.cpp:114) */
  int status;        /* FLYGPU_* status of this search */
  int steps;         /* translation / minimiser steps taken */
  int pad_;
  int64_t grad_calls; /* EAM gradient evaluations */
  double curvature;  /* last dimer curvature (eV/A^2) */
  double energy;     /* EAM energy at the final positions (eV) */
} flygpu_search_result;

/* Launch shape of the batched search kernel: lanes per atom in the EAM passes (1, 2, 4, 8),
 * threads per CTA (multiple of 32), resident CTAs per SM of the persistent grid and the kernel
 * variant's register cap (0 = the compiler's allocation, 128 = at most 128 registers a thread).
 * Each CTA stages its search's vectors, positions and slot records in shared memory as far as its
 * budget allows; the budget is the largest that keeps blocks_per_sm CTAs resident, so a higher
 * residency trades staged state for more searches in flight. */
typedef struct {
  int lanes_per_atom, threads, blocks_per_sm, max_registers;
} flygpu_tuning;

typedef struct flygpu_batch flygpu_batch;

/* Master::find_batch's fan-out (saddle/find.cpp:684-732) as one persistent launch: every search of
 * the batch is resident in HBM; one CTA runs one search at a time, largest first. */
int flygpu_batch_create(flygpu_eam* eam, const flygpu_dimer_options* dimer, const flygpu_lbfgs_options* lbfgs,
                        int precision, const flygpu_search_desc* descs, int n_search, void* stream,
                        flygpu_batch** out);
void flygpu_batch_destroy(flygpu_batch* batch);
/* Runs every unfinished search to completion (asynchronous). tuning NULL = the autotuned shape. */
int flygpu_batch_run(flygpu_batch* batch, const flygpu_tuning* tuning);
/* Times candidate launch shapes on a sample of the batch's searches and returns the fastest; the
 * choice is cached per (device, atoms-per-search bucket). Leaves the batch reset. */
int flygpu_batch_autotune(flygpu_batch* batch, flygpu_tuning* best);
/* Restores every search's inputs so the batch can run again. */
int flygpu_batch_reset(flygpu_batch* batch);
/* Two-phase runs (the default: 100 steps, wide = {4, 512, 1, 128}): flygpu_batch_run first runs every
 * search for at most `steps` translation steps in the throughput shape, then the unfinished ones to
 * completion in the `wide` shape (one CTA per search with more threads: lower latency per step).
 * steps <= 0: one launch. wide NULL keeps the current wide shape. No reference counterpart (the
 * reference runs one search per OpenMP task, saddle/find.cpp:697-731). */
int flygpu_batch_set_stragglers(flygpu_batch* batch, int steps, const flygpu_tuning* wide);
/* Waits for the batch and copies results; pos_out / axis_out (sum of 3n) may be NULL. */
int flygpu_batch_results(flygpu_batch* batch, flygpu_search_result* results, double* pos_out, double* axis_out);
int64_t flygpu_batch_device_bytes(const flygpu_batch* batch);

/* Dimer::find_sp / LBFGS::minimise for one system the plain drop-in way: the search runs on the host
 * (the reference's algorithm) and every gradient goes through this library's List and EAM on the GPU,
 * one search at a time. */
int flygpu_search_plain(flygpu_eam* eam, const flygpu_dimer_options* dimer, const flygpu_lbfgs_options* lbfgs,
                        int precision, const flygpu_search_desc* desc, double* pos_out, double* axis_out,
                        flygpu_search_result* result);

/* ---------------------------------------------------------------- served searches
 * Continuous batching of search requests. The reference's Master::find_mechs runs each environment's
 * searches batch by batch (saddle/find.cpp:374-372 find_n, 684-755 find_batch); this server takes
 * searches as they are emitted, keeps every search's positions, axis and L-BFGS history resident on the
 * device, admits them while the sum of their device footprints stays under hbm_budget_bytes, and
 * advances all admitted searches together steps_per_tick translation steps at a time. Finished slots
 * are refilled at the next tick. The server handle is internally synchronised. */
typedef struct flygpu_server flygpu_server;

typedef struct {
  uint64_t id;
  flygpu_search_result result;
  double latency_ms;  /* submit to completion */
  double queue_ms;    /* submit to admission */
} flygpu_served;

typedef struct {
  int64_t pending, active, completed, ticks, hbm_used, hbm_budget;
} flygpu_server_stats;

int flygpu_server_create(flygpu_eam* eam, const flygpu_dimer_options* dimer, const flygpu_lbfgs_options* lbfgs,
                         int precision, int64_t hbm_budget_bytes, int max_active, int steps_per_tick,
                         const flygpu_tuning* tuning, flygpu_server** out);
void flygpu_server_destroy(flygpu_server* srv);
/* Queues one search (inputs are copied); id receives its request id. */
int flygpu_server_submit(flygpu_server* srv, const flygpu_search_desc* desc, uint64_t* id);
/* n searches in one call, all or none: every descriptor is checked first (an invalid one, reported with
 * its index, queues nothing), then they are queued in order with consecutive ids (ids: n entries). */
int flygpu_server_submit_many(flygpu_server* srv, const flygpu_search_desc* descs, int n, uint64_t* ids);
/* Returns up to max finished searches, waiting up to wait_ms for the first. */
int flygpu_server_poll(flygpu_server* srv, int max, int wait_ms, flygpu_served* out, int* n_out);
/* Copies a polled search's final positions / axis (3n each, may be NULL) and forgets it. */
int flygpu_server_take(flygpu_server* srv, uint64_t id, double* pos_out, double* axis_out);
int flygpu_server_get_stats(flygpu_server* srv, flygpu_server_stats* stats);

/* LBFGS::minimise (src/minimise/LBFGS/lbfgs.cpp:29-115) for one system of any size, every vector on the
 * device: the whole-system relaxation an SKMC step ends with (kinetic/skmc.hpp:297-307). pos, types,
 * frozen: host arrays (3n, n, n); pos_out (3n, may be NULL) receives the final positions. result:
 * exit_code = LBFGS::minimise's bool (0 converged), steps, grad_calls, energy at the final positions.
 * stream NULL: a private stream. */
int flygpu_minimise(flygpu_eam* eam, const flygpu_lbfgs_options* lbfgs, int precision, int64_t n,
                    const double* pos, const uint32_t* types, const uint8_t* frozen, const double extents[3],
                    const int periodic[3], void* stream, double* pos_out, flygpu_search_result* result);

/* The prefactor step for many systems in one call (the saddles, or minima, of one Master batch,
 * find.cpp:838-871): for each system EAM::hessian, Hessian::mass_weight and Hessian::eigenvalues as
 * flygpu_hessian_eigenvalues computes them, with each system's own list at the potential's cut-off.
 * systems: n, pos, types, frozen, extents and periodic of each descriptor are read (the search fields are
 * ignored). The systems run on `workers` host threads (<= 0: 8), each with its own stream and list, so
 * their eigensolves (each one thread-block cluster of 8 or 16 SMs) overlap on the GPU. eig: the 3 n_k ascending
 * eigenvalues of every system, concatenated in order. masses: per type, NULL for the file's. */
int flygpu_hessian_eigenvalues_batch(flygpu_eam* eam, const flygpu_search_desc* systems, int n_systems,
                                     const double* masses, int workers, double* eig);

/* ------------------------------------------------------------------ catalogue local environments */

typedef struct flygpu_env flygpu_env;

/* The local environment of every atom of the list, as Catalogue::rebuild_env builds them before the
 * graph hash (env/catalogue.cpp:66-78): the geometry of env/geometry.hpp:391-407 (rebuild_geo_from_nl:
 * the atom at the origin, then its neighbours within r_env in the list's order, colour 2 type + frozen,
 * shifted to the centroid) and the fingerprint of env/heuristics.hpp:93-110 (Fingerprint::rebuild:
 * sorted distances to the central atom and between the others), binary64 in the reference's operation
 * order. types (n entries, host) and frozen (n, host, 0/1) are by real-atom index; r_env <= the list's
 * cut-off. The graph hash (canon_hash, nauty) is the caller's. */
int flygpu_env_build(flygpu_list* list, double r_env, const uint32_t* types, const uint8_t* frozen,
                     flygpu_env** out);
/* Atoms, geometry entries (atoms + neighbours), r_0j values and r_ij values. */
int flygpu_env_sizes(const flygpu_env* env, int64_t* n_atoms, int64_t* n_geo, int64_t* n_r0j, int64_t* n_rij);
/* Host copies (each may be NULL): atom i's geometry is entries [geo_offsets[i], geo_offsets[i + 1]) of
 * geo_pos (xyz), geo_colour and geo_index (real-atom index, the atom itself first); its r_0j values are
 * [geo_offsets[i] - i, geo_offsets[i + 1] - i - 1) of r0j and its r_ij values [rij_offsets[i],
 * rij_offsets[i + 1]) of rij, both ascending. Offsets have n + 1 entries. */
int flygpu_env_get(const flygpu_env* env, int64_t* geo_offsets, double* geo_pos, int32_t* geo_colour,
                   int32_t* geo_index, int64_t* rij_offsets, double* r0j, double* rij);
void flygpu_env_destroy(flygpu_env* env);

#ifdef __cplusplus
}
#endif

#endif /* FLYGPU_H */
