/* lm_api.h - C ABI of liblmgb300: the GB300 hot path of lagrangian-microbes
 * (advect -> bin -> pair -> interact), callable from ctypes / cffi / any C FFI.
 *
 * Plain pointers and sizes only. Host pointers are borrowed for the duration of the call
 * (copy-in / copy-out); device memory is owned by the context. Every entry returns an int status
 * (LM_OK = 0); nothing aborts or throws across the boundary. lm_last_error() gives the message of
 * the last failing call on a context. One host thread per context; calls on a context are
 * serialised on its CUDA stream; contexts are independent.
 *
 * Reference interfaces replaced (paths within ali-ramadhan/lagrangian-microbes):
 *   particle_advecter.py:177-186  parcels RectilinearZGrid / Field / FieldSet / ParticleSet build
 *   particle_advecter.py:220-244  pset.execute(parcels.AdvectionRK4, runtime=dt, dt=dt) loop,
 *                                 position store loop and diffusion kick
 *   interactions.py:43-54         rock_paper_scissors(N, pRS, pPR, pSP) parameters and species
 *   interaction_simulator.py:93-98   cKDTree(X).query_pairs(r, p)
 *   interaction_simulator.py:104-105 sequential pair loop calling rock_paper_scissors_interaction
 *                                    (interactions.py:13-40)
 */
#ifndef LM_API_H
#define LM_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LM_API_VERSION 1

/* Status codes. */
#define LM_OK 0
#define LM_ERR_ARG 1            /* invalid argument */
#define LM_ERR_CUDA 2           /* CUDA runtime error (message in lm_last_error) */
#define LM_ERR_OOM 3            /* device allocation failed */
#define LM_ERR_STATE 4          /* call out of order (no field / no particles / no parameters) */
#define LM_ERR_OUT_OF_BOUNDS 5  /* particles left the field domain (they are frozen and excluded) */
#define LM_ERR_NAN 6            /* non-finite positions */
#define LM_ERR_ROUND_CAP 7      /* a microbe has more than 2^24 - 1 neighbours in one step */
#define LM_ERR_TIMEOUT 8        /* a bounded device wait gave up; the context stays usable */
#define LM_ERR_TIME 9           /* a stage time fell outside the field's time axis */
#define LM_ERR_GRID 10          /* field axes are not uniformly spaced / ascending */
#define LM_ERR_CAPACITY 11      /* caller buffer too small (the needed size is returned) */

/* Flags of lm_step / lm_graph_capture. */
#define LM_STEP_ADVECT 1u     /* RK4 advection (+ diffusion kick when Kh > 0) */
#define LM_STEP_INTERACT 2u   /* bin -> pair -> rock-paper-scissors rounds */
#define LM_STEP_CENSUS 4u     /* species counts after each step */
#define LM_STEP_LOG_PAIRS 8u  /* keep (i, j, round) of every pair applied in the last step */
#define LM_STEP_COUNT_PAIRS 16u /* bin -> count the pairs within the radius, no lists and no interaction
                                   (instead of LM_STEP_INTERACT; the counts land in lm_stats) */

/* Norm codes for lm_set_interaction (cKDTree's Minkowski p). */
#define LM_NORM_INF 0
#define LM_NORM_L1 1
#define LM_NORM_L2 2

typedef struct lm_ctx lm_ctx;

typedef struct lm_stats {
  int64_t n_particles;
  int64_t pairs;          /* unordered pairs found in the last interaction step */
  int64_t rounds;         /* interaction rounds of the last step */
  int64_t max_rounds;     /* max rounds over steps since the last lm_stats_reset */
  int64_t out_of_bounds;  /* particles flagged out of domain or non-finite (sticky) */
  int64_t step;           /* device step counter (next step index) */
  int64_t census[4];      /* species counts after the last step: [0]=other, [1]=rock, [2]=paper, [3]=scissors */
  int64_t adj_capacity;   /* capacity of the long neighbour-list area (entries) */
  int64_t regrows;        /* neighbour-list regrowths since creation */
  int64_t pairs_total;    /* unordered pairs summed over interaction steps since lm_stats_reset */
  int64_t steps_total;    /* interaction steps since lm_stats_reset */
  int64_t cells;          /* binning cells of the last step (all ensembles) */
  int64_t long_lists;     /* microbes of the last step with more than 8 neighbours */
  int64_t n_ensembles;
  int64_t rounds_total;   /* levels summed over interaction steps since lm_stats_reset */
} lm_stats;

int lm_version(void);
/* SM architecture of the library's kernels as the CUDA runtime reports it for the current device
 * (cudaFuncAttributes::binaryVersion: 103 for sm_103a). LM_ERR_CUDA when no GPU can load them. */
int lm_kernel_arch(int* sm);

/* Page-locked host memory (cudaHostAlloc, portable across contexts) for step records: device-to-host
 * copies into it run asynchronously on the context's copy stream, overlapping the next steps, where
 * copies into pageable memory hold the calling thread for each record. Free with lm_host_free. */
int lm_host_alloc(size_t bytes, void** ptr);
int lm_host_free(void* ptr);

/* Create a context on CUDA device `device` with its own non-blocking stream. */
int lm_ctx_create(int device, lm_ctx** out);
int lm_ctx_destroy(lm_ctx* ctx);
/* Copy the last error message of `ctx` (or of the last failed lm_ctx_create when ctx is NULL). */
int lm_last_error(const lm_ctx* ctx, char* buf, size_t len);
/* Run all further work of `ctx` on an external stream (a cudaStream_t passed as an integer); 0 restores
 * the context's own stream. */
int lm_ctx_set_stream(lm_ctx* ctx, uintptr_t stream);
/* Block until all queued work of the context finished; returns the sticky device status. */
int lm_sync(lm_ctx* ctx);

/* Velocity field: u, v float32 [nt][ny][nx] in m/s on a rectilinear lon/lat grid whose axes are
 * uniformly spaced and ascending (lon[nx], lat[ny] degrees, t_sec[nt] seconds, nt >= 2). u and v
 * may be host or device pointers (both are copied).
 * Replaces parcels RectilinearZGrid + Field(interp_method="linear") + FieldSet
 * (particle_advecter.py:177-184). */
int lm_field_upload(lm_ctx* ctx, const float* u, const float* v, int nt, int ny, int nx, const double* lon,
                    const double* lat, const double* t_sec);
/* n_fields fields on one shared grid: u, v float32 [n_fields][nt][ny][nx]. With several ensembles,
 * ensemble e reads field e (n_fields == number of ensembles) or all read field 0 (n_fields == 1).
 * Batched form of the per-tile field build of particle_advecter.py:177-184 (one field per
 * ensemble of the sweep in sandbox/slurm_rock_paper_scissors.py). */
int lm_field_upload_batch(lm_ctx* ctx, int n_fields, const float* u, const float* v, int nt, int ny, int nx,
                          const double* lon, const double* lat, const double* t_sec);

/* Particles: positions in degrees (float64, as uniform_particle_locations returns them) and species
 * (int8, ROCK=1 PAPER=2 SCISSORS=3; NULL keeps all species at 0). Requires the field (the state is
 * stored as float32 offsets from the field origin). Replaces ParticleSet.from_list
 * (particle_advecter.py:186) and the species array of rock_paper_scissors (interactions.py:45). */
int lm_particles_upload(lm_ctx* ctx, int64_t n, const double* lon, const double* lat, const int8_t* species);
/* n_ens independent ensembles in one context (counts[e] microbes each; positions and species
 * concatenated in ensemble order). Every per-step kernel then covers all ensembles in one launch;
 * microbes of different ensembles never pair. Replaces the per-job ensembles of
 * sandbox/slurm_rock_paper_scissors.py:77-134 and the joblib tiles of particle_advecter.py:143-148. */
int lm_ensembles_upload(lm_ctx* ctx, int n_ens, const int64_t* counts, const double* lon, const double* lat,
                        const int8_t* species);
/* Current state: absolute float32 lon/lat (after any diffusion kick), species, status (0 ok,
 * 1 out of domain, 2 non-finite). Any pointer may be NULL. */
int lm_particles_download(lm_ctx* ctx, float* lon, float* lat, int8_t* species, uint8_t* status);
/* Device snapshot of the state (positions, species, status, step counter) and its restoration, bit
 * for bit, e.g. to time candidates from one state (autotuning) or to rewind. The reference's
 * equivalent is its per-chunk pickle of positions (particle_advecter.py:246-249). */
int lm_snapshot_save(lm_ctx* ctx);
int lm_snapshot_restore(lm_ctx* ctx);
/* Exact state in caller order for checkpoint files: float32 offsets from the field's float32
 * origin (lon[0], lat[0] of the field axes), species, status and the step counter. Import needs
 * the same field and particle layout (lm_particles_upload / lm_ensembles_upload first); a run
 * resumed from an exported state continues bit-identically. */
int lm_state_export(lm_ctx* ctx, float* xo, float* yo, int8_t* species, uint8_t* status, int64_t* step);
int lm_state_import(lm_ctx* ctx, const float* xo, const float* yo, const int8_t* species, const uint8_t* status,
                    int64_t step);
/* Set the species array (int8[n]). With particles uploaded, n must match their count; without
 * (the two-phase workflow, where positions arrive per step through lm_interact) it sizes the
 * context for n microbes. */
int lm_species_upload(lm_ctx* ctx, int64_t n, const int8_t* species);

/* Interaction parameters: radius and norm of cKDTree.query_pairs (interaction_simulator.py:98),
 * forward-win probabilities of rock_paper_scissors (interactions.py:43-54), Philox seed of the
 * per-pair uniform (replaces np.random.rand at interactions.py:20). */
int lm_set_interaction(lm_ctx* ctx, double radius, int norm, double p_rs, double p_pr, double p_sp,
                       uint64_t seed);
/* Per-ensemble forward probabilities and seeds (arrays of n_ens; radius and norm stay those of
 * lm_set_interaction). Each ensemble draws from its own Philox stream keyed by its seed and its
 * local microbe indices, so it evolves exactly as it would alone in a context. */
int lm_set_ensemble_params(lm_ctx* ctx, int n_ens, const double* p_rs, const double* p_pr, const double* p_sp,
                           const uint64_t* seeds);
/* Binning cell size in units of the radius (default 1.004; any value >= 1.004 gives the same pairs). */
int lm_set_cell_factor(lm_ctx* ctx, double factor);
/* Launch shapes of the step kernels, chosen by an autotuner (Simulation.autotune): no knob changes
 * any result, only the speed. LM_TUNE_ROUNDS_THREADS: interaction blocks of 1024 threads owning two
 * vertices each (default) or 512 owning four; LM_TUNE_LONG_BLOCKS_PER_SM: blocks per SM of the
 * long-neighbour-list kernel (1..32, default 6); LM_TUNE_ADVECT_THREADS: advection threads per
 * block, 128 or 256 (default). Setting a knob forgets the captured graph (capture again). No
 * counterpart in the reference (its parallelism is joblib tiles, particle_advecter.py:143-148). */
#define LM_TUNE_ROUNDS_THREADS 1
#define LM_TUNE_LONG_BLOCKS_PER_SM 2
#define LM_TUNE_ADVECT_THREADS 3
int lm_set_tuning(lm_ctx* ctx, int knob, int value);
int lm_get_tuning(lm_ctx* ctx, int knob, int* value);

/* n_steps fused steps starting at field time t_sec with global step index step0. Each step:
 * advect (flags & LM_STEP_ADVECT), then bin + pair + interact (flags & LM_STEP_INTERACT) on the
 * advected positions. kh_deg2_s > 0 adds the diffusion kick of particle_advecter.py:239-244 after the
 * positions are recorded. Optional host outputs, each [n_steps][N] (NULL to skip): rec_lon/rec_lat
 * (positions before the kick, the reference's stored positions) and rec_species (species after the
 * step). rec_census may be NULL or int64[n_steps][4]. */
int lm_step(lm_ctx* ctx, double t_sec, double dt_sec, int n_steps, int64_t step0, uint32_t flags,
            double kh_deg2_s, float* rec_lon, float* rec_lat, int8_t* rec_species, int64_t* rec_census);

/* Pairs of externally supplied float32 positions: the unordered pairs (i < j) within radius/norm of
 * lm_set_interaction. Replaces cKDTree(X).query_pairs(r, p) (interaction_simulator.py:93-98). Pairs are
 * written in (i, j) ascending order when cap suffices; *n_pairs always receives the count
 * (LM_ERR_CAPACITY if cap was too small). */
int lm_query_pairs(lm_ctx* ctx, int64_t n, const float* lon, const float* lat, int32_t* pi, int32_t* pj,
                   int64_t cap, int64_t* n_pairs);

/* Number of unordered pairs within the radius of lm_set_interaction, the size of
 * cKDTree(X).query_pairs(r, p) (interaction_simulator.py:93-98), without listing them: for
 * positions whose pair set is too large to hold. Pair semantics are lm_query_pairs'. */
int lm_count_pairs(lm_ctx* ctx, int64_t n, const float* lon, const float* lat, int64_t* n_pairs);
/* One interaction step on externally supplied float32 positions (the interaction phase of the
 * reference, interaction_simulator.py:83-117: pairs + pair loop), updating the context's species in
 * place; step_index keys the Philox draws. n must equal the particle count of the species array. */
int lm_interact(lm_ctx* ctx, int64_t n, const float* lon, const float* lat, int64_t step_index,
                uint32_t flags);

/* Pairs applied by the last interaction step when LM_STEP_LOG_PAIRS was set, in an application
 * order equal in effect to the one used: by level (pairs of one level share no microbe), then
 * (i, j). i < j are particle indices in upload order. */
int lm_pairs_get(lm_ctx* ctx, int32_t* pi, int32_t* pj, int32_t* round, int64_t cap, int64_t* n);

/* Capture `steps_per_graph` fused steps (flags as lm_step, Kh as lm_step) into a CUDA graph. The
 * graph reads the step index from the device step counter, which lm_step / lm_graph_run advance,
 * so t = t_start + (step - step0) * dt. */
int lm_graph_capture(lm_ctx* ctx, double t_start, double dt_sec, int64_t step0, int steps_per_graph,
                     uint32_t flags, double kh_deg2_s);
/* Launch the captured graph n_launches times (n_launches * steps_per_graph steps). sync=1 waits and
 * checks device status (regrowing neighbour lists and recapturing if a step overflowed them);
 * sync=0 only enqueues. */
int lm_graph_run(lm_ctx* ctx, int n_launches, int sync);
/* Set the device step counter (the next step index). */
int lm_set_step(lm_ctx* ctx, int64_t step);

int lm_stats_get(lm_ctx* ctx, lm_stats* out);
int lm_stats_reset(lm_ctx* ctx);
/* Species counts of every ensemble after the last step run with LM_STEP_CENSUS:
 * out[4*e + s] for species s (0 = values outside 1..3); cap >= 4 * n_ens. Replaces the species
 * time series of analysis.py:20-35 computed from microbe_data.nc. */
int lm_census_get(lm_ctx* ctx, int64_t* out, int64_t cap);

/* Per-kernel CUDA-event timing of plain (non-graph) launches: enable (1) / disable (0) and reset the
 * accumulators; read kernel k (0 <= k < lm_profile_count()): its name, summed duration and launch
 * count. Used by the benchmark to time the dominant kernel; costs two event records per launch. */
int lm_profile_enable(lm_ctx* ctx, int on);
int lm_profile_get(lm_ctx* ctx, int kernel, char* name, size_t name_len, double* total_ms, int64_t* launches);
int lm_profile_count(void);

/* Pair counting for callers that cannot allocate device memory (no counterpart in the reference;
 * it has no GPU path). Some callers may not call cudaMalloc/cudaFree at all: hosts that give all
 * device memory to their own pool allocator, plugins whose process forbids device allocation after
 * start-up, latency-bound loops that cannot afford the device-wide synchronisation of cudaFree.
 * They pass device pointers: d_lon, d_lat (float32[n]) in, d_degree (int32[n], neighbours of each
 * point) and d_pairs (one uint64, the number of unordered pairs, the size of
 * cKDTree.query_pairs) out, all written on `stream` (a cudaStream_t as an integer, 0 = default
 * stream). Pair semantics are lm_query_pairs'.
 * Nothing is allocated: the scratch is a fixed ~1.8 MB array inside the library that every GPU
 * loading it keeps until the process exits, so n is limited to 65536 (larger n: LM_ERR_ARG).
 * The first call on a device, with that device current, looks up that array's device address and
 * loads the function's kernels; make that first call before any stream capture. The address is
 * kept for the life of the process and belongs to the device's primary context: after
 * cudaDeviceReset it is stale, so do not call this function again in that process. All calls
 * share the array and it keeps the last call's contents (each call clears what must start at
 * zero), so calls whose work overlaps on the GPU (other streams, other threads) race: serialise
 * them. Errors: lm_last_error(NULL, ...). */
int lm_count_pairs_noalloc(const float* d_lon, const float* d_lat, int64_t n, double radius, int norm,
                           int32_t* d_degree, unsigned long long* d_pairs, uintptr_t stream);

/* ---- Adjoint of the advection (no reference counterpart: the reference does not differentiate) ----
 * A tape records a forward RK4 run, with the arithmetic and freezing rules of lm_step's advection
 * (particle_advecter.py:220-223; no diffusion kick), and returns gradients of a loss on the final
 * positions w.r.t. the initial positions and the gridded u, v. The tape keeps its own copy of the
 * field and the state every `checkpoint_every` steps; the backward sweep recomputes each segment
 * from its checkpoint. The velocity gradient is a deterministic segmented reduction (bit-identical
 * from run to run, no float atomics). All arrays are DEVICE pointers (float32), on ctx's stream
 * (lm_ctx_set_stream); errors through lm_last_error(ctx). Destroy tapes before their context. */
typedef struct lm_adjoint lm_adjoint;
int lm_adjoint_create(lm_ctx* ctx, lm_adjoint** out);
int lm_adjoint_destroy(lm_adjoint* adj);
/* Working precision of the next lm_adjoint_forward. LM_ADJ_DS (default): double-float positions
 * (two float32 words each) with float32 velocities, Jacobians and adjoint state: the trajectory
 * does not pick up float32 position rounding every step, so on long chaotic runs (720 hourly
 * steps) its gradients stay within 1e-4 of FP64 finite differences at close to float32 cost.
 * LM_ADJ_F32: float32 state with the engine's arithmetic, final positions bit-identical to
 * lm_step's. LM_ADJ_F64: float64 state and arithmetic (the field stays float32). */
#define LM_ADJ_F32 0
#define LM_ADJ_F64 1
#define LM_ADJ_DS 2
int lm_adjoint_set_precision(lm_adjoint* adj, int precision);
/* u, v [nt][ny][nx] m/s and the axes as lm_field_upload (axes are host arrays); n microbes from
 * lon0/lat0 (absolute degrees) for n_steps steps of dt_sec from t_sec0; final positions into
 * lon_out/lat_out. Microbes leaving the domain are frozen (LM_ERR_OUT_OF_BOUNDS is returned, the tape is
 * still valid and their gradient passes through the frozen steps unchanged). */
int lm_adjoint_forward(lm_adjoint* adj, const float* u, const float* v, int nt, int ny, int nx, const double* lon,
                       const double* lat, const double* t_sec, int64_t n, const float* lon0, const float* lat0,
                       double t_sec0, double dt_sec, int n_steps, int checkpoint_every, float* lon_out,
                       float* lat_out);
/* dL/d(final lon, lat) [n] -> dL/d(initial lon, lat) [n] and dL/du, dL/dv [nt][ny][nx] (overwritten).
 * May be called several times after one forward. */
int lm_adjoint_backward(lm_adjoint* adj, const float* g_lon, const float* g_lat, float* g_lon0, float* g_lat0,
                        float* g_u, float* g_v);
/* Final positions of the recorded run in float64 (device double [n] each, absolute degrees): the
 * working state rounded only once, for losses that need more than float32 positions. */
int lm_adjoint_final_positions(lm_adjoint* adj, double* lon, double* lat);
/* Cell path of every microbe of the recorded run (device uint64 [n]): the grid cell j * nx + i of
 * every stage evaluation, folded in order as sig = (sig ^ cell) * 0x100000001B3. The forward map
 * is piecewise smooth (bilinear pieces meet at cell edges); two runs whose signatures agree
 * sampled the same pieces. Used to compare gradients with an FP64 run cell path by cell path. */
int lm_adjoint_cell_signature(lm_adjoint* adj, unsigned long long* sig);

/* ---- failure injection (tests; no reference counterpart) ----
 * The next lm_step call that interacts (plain launches only, never a captured graph) makes its
 * first step's interaction kernel wait on a device flag that nothing sets, as a stalled
 * dependency would, until `seconds` (0 < seconds <= 10) have passed: the kernel then records the
 * timeout and returns, no pair of that step is applied, and the call returns LM_ERR_TIMEOUT. The
 * context stays usable; later steps run normally. Failure detection is exercised this way without
 * any fault on the GPU. */
int lm_debug_inject_wait(lm_ctx* ctx, double seconds);

/* ---- pairwise distance histogram ----
 * Replaces pairwise_distance_histogram_parallel / pairwise_distance_histogram_1point
 * (sandbox/pairwise_distance_histogram_distributed.jl:56-76) and pairwise_dist_gpu
 * (sandbox/pairwise_distance_histogram_gpu.jl:45-77): for every unordered pair of points inside
 * each segment [seg[s], seg[s+1]) (the reference: one segment per species), the float32 haversine
 * distance d of haversine_distance32 (:35-46, latitude first, radius_m as `radius`) is counted in
 * bin round-half-even(10 log10(max(1, d))); bins >= `bins` are counted in the last column.
 * lat, lon: host float32 [n] (finite, else LM_ERR_NAN); seg: host int64 [n_seg + 1] from 0 to n
 * (NULL with n_seg = 1: one segment); counts: host uint64 [n_seg][bins + 1], overwritten.
 * 1 <= bins <= 256. */
int lm_distance_histogram(lm_ctx* ctx, const float* lat, const float* lon, int64_t n, const int64_t* seg, int n_seg,
                          int bins, double radius_m, uint64_t* counts);

#ifdef __cplusplus
}
#endif

#endif /* LM_API_H */
