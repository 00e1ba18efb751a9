// Internal declarations shared by the CUDA translation units of liblmgb300.
//
// One context holds E >= 1 independent ensembles. Particle arrays use a padded slot layout:
// ensemble e owns slots [base_e, base_e + n_e) and, when E > 1, base_e is a multiple of
// SLOT_BLOCK so that every 256-slot block belongs to one ensemble (block_ens[block]). Pad slots
// carry status PAD and never take part in anything.
//
// Data layout in HBM:
//   field      float2 uv[F][nt][ny][nx]   (u,v interleaved; ensemble e reads field_off_e)
//   state      float  xo[S], yo[S]        (lon/lat offsets from a float32 origin, slot order)
//              int8   species[S], uint8 status[S]
//   per step   float  plon[S], plat[S]    (absolute float32 lon/lat after advection, pre-kick)
//              uint32 key[S], rank[S]     (cell key, rank inside the cell from the counting pass)
//              uint32 ccount[C+1], cstart[C+1]  (cell counts / exclusive starts, C = cell capacity)
//              uint32 sid[S], skey[S], sens[S]; float2 spos[S]  (particles in cell order)
//              uint32 deg[S], slab[S][SLAB]     (neighbour lists up to SLAB, sorted by priority;
//                                                a longer list's overflow offset in slot 0)
//              uint32 ovf[cap]; uint64 oprio[cap]  (longer lists, allocated per step)
//              uint64 wstate[S] = species << 56 | list position << 32 | partner;
//              uint32 level[S] (pair-log runs only), act[S]   (interaction dataflow)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <utility>

struct lm_ctx;

namespace lm {

constexpr uint32_t NONE = 0xffffffffu;
constexpr uint32_t SLOT_BLOCK = 256;   // threads per block of every per-slot kernel
constexpr uint32_t SLAB = 8;           // neighbour-list entries kept in the per-vertex slab
constexpr uint8_t STATUS_OK = 0, STATUS_OOB = 1, STATUS_NAN = 2, STATUS_PAD = 3;
constexpr uint32_t MAX_DEGREE = (1u << 24) - 1;  // list positions take 24 bits of the state word

// Neighbour-list entry: the partner's cell-order index in bits 0-28 and, on the entries of the
// lower endpoint of a pair (the endpoint that applies it), the pair's three rock-paper-scissors
// outcomes in bits 29-31: bit 29 + c is set when the pair's Philox uniform lies below the
// forward-win threshold of matchup c (0 rock/scissors, 1 paper/rock, 2 scissors/paper). The draw
// is made once, in the sweep that builds the list, instead of in the interaction's dependency
// chain. Indices stay below ENTRY_ID_MASK, so an entry never equals NONE.
constexpr uint32_t ENTRY_ID_MASK = (1u << 29) - 1;
constexpr uint32_t ENTRY_WIN_SHIFT = 29;
constexpr uint64_t MAX_SLOTS = ENTRY_ID_MASK - 1;
__host__ __device__ inline uint32_t entry_id(uint32_t e) { return e & ENTRY_ID_MASK; }

// Interaction state word of a vertex: its current species, the position of its current pair in
// its list, and that pair's partner (NONE once the list is done).
__host__ __device__ inline unsigned long long pack_state(uint32_t partner, uint32_t pos, int species) {
  return ((unsigned long long)(uint8_t)species << 56) | ((unsigned long long)(pos & MAX_DEGREE) << 32) | partner;
}
__host__ __device__ inline uint32_t state_partner(unsigned long long w) { return (uint32_t)w; }
__host__ __device__ inline uint32_t state_pos(unsigned long long w) { return (uint32_t)(w >> 32) & MAX_DEGREE; }
__host__ __device__ inline int state_species(unsigned long long w) { return (int)(int8_t)(uint8_t)(w >> 56); }

// Sticky error bits in Ctrl::err (mirrored by the LM_ERR_* status codes of lm_api.h).
enum : uint32_t {
  ERRB_OOB = 1u << 0,        // a particle left the field domain (frozen, excluded from pairing)
  ERRB_NAN = 1u << 1,        // a non-finite position or velocity
  ERRB_OVERFLOW = 1u << 2,   // long-list capacity exceeded (step halted)
  ERRB_ROUNDCAP = 1u << 3,   // a microbe has more than MAX_DEGREE neighbours (step halted)
  ERRB_TIMEOUT = 1u << 4,    // a bounded device wait gave up
  ERRB_TIME = 1u << 5,       // a stage time fell outside the field's time axis
};

// Device control block: one per context, lives in device memory.
struct Ctrl {
  unsigned long long n_dir;     // directed neighbour entries of the current step (2 x pairs)
  unsigned long long ovf_cap;   // capacity of ovf/oprio
  unsigned long long ovf_used;  // long-list entries requested this step
  unsigned long long pairs_total;  // unordered pairs summed over completed steps since the last reset
  unsigned long long steps_total;  // interaction steps since the last reset
  uint32_t err;                 // sticky error bits
  uint32_t halt;                // nonzero: every later kernel of the step sequence returns at once
  uint32_t halt_step;           // step index at which halt was raised
  uint32_t step;                // device-side step counter (used by captured graphs)
  uint32_t oob;                 // particles flagged out of domain or non-finite (sticky count)
  uint32_t n_valid;             // particles binned this step
  uint32_t ncells;              // cells of this step's grids (sum over ensembles)
  uint32_t n_long;              // vertices whose list exceeds SLAB
  uint32_t rounds;              // longest dependency chain (levels) of the current step
  uint32_t max_rounds;          // max over steps since the last reset
  uint32_t plog_n;              // pair-log entries written this step
  uint32_t act_n;               // active vertices (with at least one pair)
  uint32_t census[4];           // species counts after the step, all ensembles ([0] = other values)
  unsigned long long rounds_total;  // sum of per-step levels since the last reset
  int stage_k[3];               // frame brackets of this step's stage times t, t+dt/2, t+dt
  float stage_w[3];
  int stage_ok;                 // 0 when a stage time left the field's time axis
  uint32_t never;               // a flag nothing sets: the injected failure of the tests waits on it
};

// Per-ensemble constants (device array, one entry per ensemble).
struct EnsInfo {
  unsigned long long t_rs, t_pr, t_sp;  // u53 < t  <=>  r < p (exact)
  unsigned long long field_off;         // element offset of this ensemble's frames in uv
  uint32_t seed_lo, seed_hi;            // Philox key of pair draws and diffusion kicks
  uint32_t base;                        // first slot
  uint32_t n;                           // microbes
};

// Per-step uniform cell grid of one ensemble: cell (cx, cy) covers
// [x0 + cx*c, x0 + (cx+1)*c) x [y0 + cy*c, ...), c >= radius; global key = cell_base + cy*ncx + cx.
struct EnsGrid {
  float x0, y0, inv_c, c;
  int ncx, ncy;
  uint32_t cell_base;
  uint32_t tshift;  // tiles of (1 << tshift) x (1 << tshift) cells
};

// Cell numbering inside an ensemble's key range is tile-major: T x T cells form a tile, tiles are
// numbered row by row, cells inside a tile row by row. Cell-ordered particles of one tile are
// then contiguous, so a contiguous range of them is a compact 2D patch (the interaction kernel
// gives such ranges, 2,048 vertices each, to its blocks). A grid's key range is padded to whole
// tiles. T is chosen per ensemble and step from its microbes per cell rho (tile_shift): the
// interaction's ranges come out nearest to square when a tile holds about as many microbes as a
// block owns, T ~ sqrt(2048 / rho), rounded down (rho is an average over the bounding box, and
// clustered microbes are denser than that where they are): T = 32 below 2 microbes per cell, 16
// below 8, else 8.
__host__ __device__ inline uint32_t tile_shift(float n, float cells) {
  const float rho = n / fmaxf(cells, 1.f);
  return rho < 2.f ? 5u : rho < 8.f ? 4u : 3u;
}
__host__ __device__ inline uint32_t tiles_x(const EnsGrid& g) {
  return ((uint32_t)g.ncx + (1u << g.tshift) - 1u) >> g.tshift;
}
__host__ __device__ inline uint32_t cell_index(const EnsGrid& g, uint32_t cx, uint32_t cy) {
  const uint32_t s = g.tshift, m = (1u << s) - 1u;
  return ((((cy >> s) * tiles_x(g) + (cx >> s)) << s) + (cy & m)) << s | (cx & m);
}
__host__ __device__ inline void cell_coords(const EnsGrid& g, uint32_t k, uint32_t* cx, uint32_t* cy) {
  const uint32_t s = g.tshift, m = (1u << s) - 1u;
  const uint32_t t = k >> (2u * s), ntx = tiles_x(g);
  *cx = ((t % ntx) << s) + (k & m);
  *cy = ((t / ntx) << s) + ((k >> s) & m);
}
// The keys of cells x0..x1 (at most three) of row ry: one contiguous run, or two when the cells
// straddle a tile edge. Fixed-size, so the callers' loops unroll with static indices.
struct RowRuns {
  uint32_t lo[2], hi[2];  // first and last key of each run
  int n;
};
__device__ __forceinline__ RowRuns row_runs(const EnsGrid& g, int x0, int x1, int ry) {
  RowRuns r;
  const int s = (int)g.tshift;
  const int split = (x0 >> s) != (x1 >> s) ? (((x0 >> s) + 1) << s) - 1 : x1;
  r.lo[0] = g.cell_base + cell_index(g, (uint32_t)x0, (uint32_t)ry);
  r.hi[0] = g.cell_base + cell_index(g, (uint32_t)split, (uint32_t)ry);
  r.n = 1;
  r.lo[1] = r.hi[1] = 0;
  if (split < x1) {
    r.lo[1] = g.cell_base + cell_index(g, (uint32_t)split + 1, (uint32_t)ry);
    r.hi[1] = g.cell_base + cell_index(g, (uint32_t)x1, (uint32_t)ry);
    r.n = 2;
  }
  return r;
}

// Velocity field geometry shared by all ensembles.
struct FieldView {
  const float2* uv;   // [F][nt][ny][nx]
  int nx, ny, nt;
  float gx0, gy0;     // grid origin minus the state origin (degrees, small)
  float inv_dx, inv_dy;
  float max_fx, max_fy;  // nx-1, ny-1
  float org_lon, org_lat;  // float32 origin of the offsets (absolute degrees)
  double t0, dT;      // frame 0 time and frame spacing (seconds)
  // the same geometry in float64 (the adjoint's FP64-trajectory mode)
  double gx0d, gy0d, inv_dxd, inv_dyd;
};

struct PairParams {
  double r;           // radius (degrees)
  double r2;          // fl(r*r)
  float r2f_lo, r2f_hi;  // float32 accept / reject thresholds around r^2 (p = 2)
  float rf_lo, rf_hi;    // float32 accept / reject thresholds around r   (p = 1, inf)
  float cell_factor;  // binning cell size = cell_factor * r (>= 1.004)
  int norm;           // 1, 2 or 0 (= infinity)
};

// Pair-test parameters of radius r and norm code `norm` (lm_api.h). A float32 pre-test decides
// every candidate whose distance lies outside a relative band of 2e-6 around r (float32 error
// < 3e-7 relative); candidates inside the band are re-decided in float64. Radii float32 cannot
// resolve get an empty float32 range: every candidate is then decided in float64. Shared by every
// entry point that tests pairs, so all of them draw the same boundary.
inline PairParams make_pair_params(double r, int norm, float cell_factor) {
  PairParams pp{};
  pp.r = r;
  pp.r2 = r * r;
  pp.norm = norm;
  const double band = 2e-6;
  if (r > 1e-15 && r < 1e15) {
    pp.r2f_lo = std::nextafter((float)(pp.r2 * (1 - band)), 0.f);
    pp.r2f_hi = std::nextafter((float)(pp.r2 * (1 + band)), INFINITY);
    pp.rf_lo = std::nextafter((float)(r * (1 - band)), 0.f);
    pp.rf_hi = std::nextafter((float)(r * (1 + band)), INFINITY);
  } else {
    pp.r2f_lo = pp.rf_lo = -1.f;
    pp.r2f_hi = pp.rf_hi = INFINITY;
  }
  pp.cell_factor = cell_factor;
  return pp;
}

struct StepArgs {
  double t_start;     // time of step step0 (seconds, field clock)
  double dt;          // step length (seconds)
  uint32_t step0;     // global step index of t_start
  int use_ctrl_step;  // 1: step index = ctrl->step (graph mode); 0: step index = step0
  float kick;         // sqrt(6 |dt| Kh) in degrees, 0 disables the diffusion kick
  // failure injection (lm_debug_inject_wait, plain steps only): when nonzero, k_rounds waits on
  // Ctrl::never, which nothing sets, until this many nanoseconds have passed, and reports a timeout
  unsigned long long test_wait_ns;
};

// Everything the per-step kernels need besides the field.
struct Bufs {
  const EnsInfo* ens;
  const uint32_t* block_ens;
  uint32_t n_ens;
  uint32_t nslots;
  uint32_t cells_cap;
  float* xo;
  float* yo;
  int8_t* species;
  uint8_t* status;
  float* plon;
  float* plat;
  uint32_t* ebox;     // [E][4] ordered-int encoded min x, min y, max x, max y
  EnsGrid* grids;     // [E]
  uint32_t* eord;     // [E] the ensembles in the order of their key ranges (cell order)
  uint32_t* key;
  uint32_t* rank;
  uint32_t* ccount;   // [cells_cap + 1]
  uint32_t* cstart;   // [cells_cap + 1]
  uint32_t* csum;     // [SCAN_BLOCKS]
  uint32_t* sid;
  uint32_t* skey;
  uint32_t* sens;
  float2* spos;
  uint32_t* deg;
  uint32_t* slab;     // [S][SLAB]; slot 0 of a list longer than SLAB holds its offset in ovf
  uint32_t* ovf;
  unsigned long long* oprio;
  uint32_t* longv;    // vertices with lists longer than SLAB
  unsigned long long* wstate;  // per vertex: species << 56 | current list position << 32 | partner
  uint32_t* level;
  uint32_t* act;
  uint32_t* census;   // [E][4]
  uint32_t* plog;     // 3 x uint32 per logged pair (slot i, slot j, level) or nullptr
  uint32_t plog_cap;
};

// ---- programmatic dependent launch ----
// Per-step kernels start with pdl_wait() and are launched with launch_dep() (plain launches and
// captured graphs alike). pdl_wait() holds the kernel's threads until the previous grid has
// completed and its memory is visible (griddepcontrol.wait), then lets the next kernel of the
// stream launch (griddepcontrol.launch_dependents): once every block of this grid has started, the
// next grid's blocks are placed on the SMs as they free up and wait there, so the launch and ramp
// of each step kernel overlap the tail of the one before. A kernel launched without the attribute
// passes the wait at once. The cooperative interaction kernel is launched without it (its blocks
// must all be resident together).
__device__ __forceinline__ void pdl_wait() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}
bool pdl_enabled();  // off when the environment sets LM_PDL=0

template <typename... KArgs, typename... Args>
inline void launch_dep(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// ---- launchers (each enqueues on `st`) ----
void launch_interleave(const float* u, const float* v, float2* uv, size_t n, cudaStream_t st);
void launch_particles_in(const double* lon, const double* lat, const int8_t* sp, const int32_t* map, uint32_t S,
                         double org_lon, double org_lat, float* xo, float* yo, int8_t* species, uint8_t* status,
                         cudaStream_t st);
// step_begin also brackets the stage times of the step in the field's frames when `f` is given.
void launch_step_begin(const Bufs& b, const FieldView* f, const StepArgs& a, Ctrl* ctrl, cudaStream_t st);
void launch_step_end(Ctrl* ctrl, bool interact, cudaStream_t st);
// End of a step and start of the next (arguments `an`) in one launch (steps of one call).
void launch_step_turn(const Bufs& b, const FieldView* f, const StepArgs& an, Ctrl* ctrl, bool interact,
                      cudaStream_t st);
// threads: 128 or 256 per block (tuning)
void launch_advect(const FieldView& f, const StepArgs& a, const Bufs& b, Ctrl* ctrl, int threads, cudaStream_t st);
void launch_bbox(const Bufs& b, Ctrl* ctrl, bool use_status, cudaStream_t st);

// K2 binning: per-ensemble grids, counting pass, cell scan, scatter into cell order.
constexpr int SCAN_BLOCKS = 304;
void launch_grid(const Bufs& b, const PairParams& pp, Ctrl* ctrl, cudaStream_t st);
// own_grid (one ensemble): k_keys computes the grid itself (no launch_grid before it).
void launch_keys(const Bufs& b, const PairParams& pp, Ctrl* ctrl, bool use_status, bool own_grid, cudaStream_t st);
void launch_cell_scan(const Bufs& b, Ctrl* ctrl, cudaStream_t st);
void launch_scatter(const Bufs& b, Ctrl* ctrl, cudaStream_t st);

// K3 neighbour lists.
void launch_sweep(const Bufs& b, const PairParams& pp, const StepArgs& a, Ctrl* ctrl, cudaStream_t st);
void launch_count_pairs(const Bufs& b, const PairParams& pp, Ctrl* ctrl, cudaStream_t st);
// blocks_per_sm: grid of sms x blocks_per_sm blocks of LONG_WARPS warps (tuning)
void launch_sweep_long(const Bufs& b, const PairParams& pp, const StepArgs& a, Ctrl* ctrl, int sms,
                       int blocks_per_sm, cudaStream_t st);

// K4/K5 interaction dataflow (cooperative persistent kernel).
// Grid of the cooperative launch with `threads` (512 or 1,024) per block; *block receives the block size.
int rounds_grid(int device, int threads, int* block);
cudaError_t launch_rounds(const Bufs& b, const StepArgs& a, Ctrl* ctrl, int grid, int block, cudaStream_t st);
void launch_census(const Bufs& b, Ctrl* ctrl, cudaStream_t st);
const void* lm_census_kernel();  // one kernel of the library, for attribute queries
void launch_unpad(const float* src, float* dst, const int32_t* map, uint32_t nslots, cudaStream_t st);
void launch_unpad8(const int8_t* src, int8_t* dst, const int32_t* map, uint32_t nslots, cudaStream_t st);

// ---- K6/K7 adjoint of the advection (k_adjoint.cu) ----
// Stage brackets of one step: frames k[g] and weights w[g] of the stage times t, t + dt/2, t + dt.
struct AdjStep {
  int k[3];
  float w[3];
  double wd[3];  // the weights in float64 (FP64-trajectory mode)
};
// Working precision of the adjoint tape: ADJ_F32 the engine's float32 arithmetic, ADJ_F64 float64
// state and arithmetic, ADJ_DS double-float positions with float32 velocities and adjoint state.
enum AdjPrecision { ADJ_F32 = 0, ADJ_F64 = 1, ADJ_DS = 2 };
// Bytes of one position coordinate / one adjoint coordinate in each precision.
inline size_t adj_state_bytes(int prec) { return prec == ADJ_F32 ? 4 : 8; }
inline size_t adj_lambda_bytes(int prec) { return prec == ADJ_F64 ? 8 : 4; }
constexpr int RS_BITS_MAX = 10;                      // digit width of one radix pass
constexpr uint32_t RS_RADIX_MAX = 1u << RS_BITS_MAX;

struct AdjSortBufs {
  const uint32_t* key;      // input keys (m)
  uint32_t *k1, *k2;        // ping-pong keys (m)
  uint32_t *v1, *v2;        // ping-pong record ids (m)
  uint32_t *hist, *hscan;   // adj_sort_hist_len(m)
  uint32_t* bsum;           // SCAN_BLOCKS
};

void launch_adj_stages(const FieldView& f, double t_start, double dt, int n_steps, AdjStep* table, uint32_t* err,
                       cudaStream_t st);
// Per-microbe kernels in precision `prec`: x, y point to position arrays of adj_state_bytes(prec)
// per element (float, double, or a double-float pair), lx, ly to adjoint arrays of
// adj_lambda_bytes(prec) (float, or double for ADJ_F64).
void launch_adj_init(const FieldView& f, int prec, uint32_t n, const float* lon, const float* lat, void* x, void* y,
                     uint8_t* status, cudaStream_t st);
void launch_adj_final(const FieldView& f, int prec, uint32_t n, const void* x, const void* y, float* lon, float* lat,
                      cudaStream_t st);
void launch_adj_final64(const FieldView& f, int prec, uint32_t n, const void* x, const void* y, double* lon,
                        double* lat, cudaStream_t st);
void launch_adj_seed(int prec, uint32_t n, const float* gx, const float* gy, void* lx, void* ly, cudaStream_t st);
void launch_adj_unseed(int prec, uint32_t n, const void* lx, const void* ly, float* gx, float* gy, cudaStream_t st);
void launch_adj_forward(const FieldView& f, int prec, const AdjStep* table, int m0, int m1, double dt, uint32_t n,
                        void* x, void* y, uint8_t* status, void* rec_x, void* rec_y, uint8_t* rec_st, uint32_t* err,
                        cudaStream_t st);
// mkey (or nullptr): gather form of the reduction. Per microbe, in mcode, 4 bits a stage: the slot
// (dj + 1) * 3 + (di + 1) of the stage's cell around the cell b where the step starts, and in mkey
// 2b + (1 when a stage leaves b), msent when frozen; a stage outside those 3 x 3 cells sets
// ADJ_WIDE. Without mkey the step writes the four record keys (cell * 4 + stage time, or `sent`).
constexpr uint32_t ADJ_WIDE = 1u << 8;
void launch_adj_step(const FieldView& f, int prec, const AdjStep& s, double dt, uint32_t n, const void* x,
                     const void* y, const uint8_t* status, void* lx, void* ly, float4* rec, uint32_t* key, uint32_t sent,
                     uint32_t* mkey, uint32_t* mcode, uint32_t msent, uint32_t* err, cudaStream_t st);
// After the sort of mkey: cell bounds, stage codes in sorted order, target cells listed once a step.
void launch_adj_cells(const uint32_t* skey, const uint32_t* sval, uint32_t m, uint32_t cw, uint32_t ch,
                      const uint32_t* mcode, uint32_t* scode, uint32_t* cst, uint32_t* cen, uint32_t* mark,
                      uint32_t stamp, uint32_t* tlist, uint32_t* tcnt, cudaStream_t st);
void launch_adj_gather(uint32_t cw, uint32_t ch, const uint32_t* tcnt, const uint32_t* tlist, const uint32_t* cst,
                       const uint32_t* cen, const uint32_t* scode, const uint32_t* sval, const float4* rec,
                       float* csum, int sms, cudaStream_t st);
void launch_adj_signature(const FieldView& f, int prec, const AdjStep* table, int n_steps, double dt, uint32_t n,
                          const void* x, const void* y, const uint8_t* status, unsigned long long* sig,
                          cudaStream_t st);
size_t adj_sort_hist_len(uint32_t m);
// Stable sort of m keys of key_bits bits; returns the sorted keys and the record ids (input index).
void adj_sort(const AdjSortBufs& sb, uint32_t m, int key_bits, cudaStream_t st, const uint32_t** skey,
              const uint32_t** sval);
void launch_adj_bounds(const uint32_t* skey, uint32_t m, uint32_t sent, uint32_t* cst, uint32_t* cen,
                       cudaStream_t st);
void launch_adj_reduce(uint32_t ncells, uint32_t* cst, uint32_t* cen, const uint32_t* sval, const float4* rec,
                       float* csum, int sms, cudaStream_t st);
// mark (or nullptr): only cells with mark[c] == stamp hold sums (the gather form's target list).
void launch_adj_nodes(int nx, int ny, const AdjStep& s, const float* csum, const uint32_t* mark, uint32_t stamp,
                      float* gu, float* gv, cudaStream_t st);

// Field geometry from uniform axes (shared by lm_field_upload_batch and the adjoint tape).
bool uniform_axis(const double* a, int n, double* d);
void fill_field_view(FieldView& f, float2* uv, int nt, int ny, int nx, const double* lon, const double* lat,
                     const double* t_sec, double dx, double dy, double dT);

// Message for lm_last_error(NULL, ...) from entry points that have no context.
void set_thread_error(const char* msg);
// Context accessors for translation units other than lm_api.cu.
int ctx_device(const lm_ctx* c);
int ctx_sms(const lm_ctx* c);
cudaStream_t ctx_stream(const lm_ctx* c);
void ctx_set_error(lm_ctx* c, const char* msg);

// Ordered-int encoding of floats for atomicMin/atomicMax.
__host__ __device__ inline uint32_t enc_f(float f) {
  uint32_t u;
#ifdef __CUDA_ARCH__
  u = __float_as_uint(f);
#else
  union { float f; uint32_t u; } x;
  x.f = f;
  u = x.u;
#endif
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float dec_f(uint32_t e) {
  uint32_t u = (e & 0x80000000u) ? (e & 0x7fffffffu) : ~e;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  union { float f; uint32_t u; } x;
  x.u = u;
  return x.f;
#endif
}

}  // namespace lm
