// Internal declarations shared by the CUDA translation units of liblmgb300.
//
// Data layout in HBM (one context = one GPU stream):
//   field      float2 uv[nt][ny][nx]      (u,v interleaved so one 8-byte load gives both)
//   state      float  xo[N], yo[N]        (lon/lat offsets from a float32 origin, id order)
//              int8   species[N]          (ROCK=1, PAPER=2, SCISSORS=3, id order)
//              uint8  status[N]           (bit0 out of domain, bit1 non-finite)
//   per step   float  plon[N], plat[N]    (absolute float32 lon/lat after advection, id order)
//              uint32 key[2][N], id[2][N] (radix-sort ping-pong of (cell key, particle id))
//              float2 spos[N]             (pos gathered into cell order)
//              uint32 cell_start[ncells]  (first sorted index of each occupied cell; never cleared,
//                                          an entry is trusted only if key[start] == cell)
//              uint32 deg[N], off[N]      (neighbour counts / CSR offsets, cell order)
//              uint32 adj[cap]            (neighbour lists in cell-order indices, each list sorted by
//                                          descending pair priority)
//              uint64 prio[cap]           (pair priorities while the lists are sorted)
//              uint32 want[N], head[N], level[N], act[N]  (interaction dataflow)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lm {

constexpr uint32_t NONE = 0xffffffffu;

// Sticky error bits in Ctrl::err (mirrored by the LM_ERR_* status codes of lm_api.h).
enum : uint32_t {
  ERRB_OOB = 1u << 0,        // a particle left the field domain (frozen, excluded from pairing)
  ERRB_NAN = 1u << 1,        // a non-finite position or velocity
  ERRB_OVERFLOW = 1u << 2,   // neighbour-list capacity exceeded (step halted)
  ERRB_ROUNDCAP = 1u << 3,   // interaction round cap reached
  ERRB_TIMEOUT = 1u << 4,    // a bounded device wait gave up
  ERRB_TIME = 1u << 5,       // a stage time fell outside the field's time axis
};

// Device control block: one per context, lives in device memory.
struct Ctrl {
  unsigned long long n_dir;   // directed neighbour entries of the current step (2 x pairs)
  unsigned long long cap;     // capacity of adj/prio
  uint32_t err;               // sticky error bits
  uint32_t halt;              // nonzero: every later kernel of the step sequence returns at once
  uint32_t halt_step;         // step index at which halt was raised
  uint32_t step;              // device-side step counter (used by captured graphs)
  uint32_t oob;               // particles flagged out of domain (sticky count)
  uint32_t n_valid;           // particles with a valid cell key this step
  uint32_t rounds;            // interaction rounds used by the current step
  uint32_t max_rounds;        // max over steps since the last reset
  uint32_t applied;           // pairs whose species differed (draws taken) this step
  uint32_t plog_n;            // pair-log entries written this step
  uint32_t bar_count;         // grid barrier arrival counter
  uint32_t bar_gen;           // grid barrier generation
  uint32_t act_n[3];          // active-vertex list sizes (rotating)
  uint32_t census[4];         // species counts after the current step (index = species)
  unsigned long long pairs_total;  // unordered pairs summed over steps since the last stats reset
  unsigned long long steps_total;  // interaction steps since the last stats reset
};

// Velocity field as the advection kernel sees it.
struct FieldView {
  const float2* uv;   // [nt][ny][nx]
  int nx, ny, nt;
  float gx0, gy0;     // grid origin minus the state origin (degrees, small)
  float inv_dx, inv_dy;
  float max_fx, max_fy;  // nx-1, ny-1
  float org_lon, org_lat;  // float32 origin of the offsets (absolute degrees)
  double t0, dT;      // frame 0 time and frame spacing (seconds)
};

// Uniform cell grid for binning: cell (cx, cy) covers
// [x0 + cx*c, x0 + (cx+1)*c) x [y0 + cy*c, y0 + (cy+1)*c) with c >= radius.
struct CellGrid {
  float x0, y0;       // absolute degrees
  float inv_c;
  int ncx, ncy;
  uint32_t ncells;    // ncx*ncy; key value ncells marks an invalid (excluded) particle
};

struct PairParams {
  double r;           // radius (degrees)
  double r2;          // fl(r*r)
  float r2f_lo, r2f_hi;  // float32 accept / reject thresholds around r^2 (p = 2)
  float rf_lo, rf_hi;    // float32 accept / reject thresholds around r   (p = 1, inf)
  int norm;           // 1, 2 or 0 (= infinity)
};

struct RpsParams {
  unsigned long long t_rs, t_pr, t_sp;  // u53 < t  <=>  u53 * 2^-53 < p
  uint32_t seed_lo, seed_hi;
};

struct StepArgs {
  double t_start;     // time of step 0 of this launch sequence (seconds, field clock)
  double dt;          // step length (seconds)
  uint32_t step0;     // global step index of t_start
  int use_ctrl_step;  // 1: step index = ctrl->step (graph mode); 0: step index = step0
  float kick;         // sqrt(6 |dt| Kh) in degrees, 0 disables the diffusion kick
  uint32_t seed_lo, seed_hi;
};

// ---- launchers (each enqueues on `st`) ----
void launch_interleave(const float* u, const float* v, float2* uv, size_t n, cudaStream_t st);
void launch_advect(const FieldView& f, const CellGrid& g, const StepArgs& a, Ctrl* ctrl, float* xo, float* yo,
                   uint8_t* status, float* plon, float* plat, uint32_t* key, uint32_t* id, uint32_t n,
                   cudaStream_t st);
void launch_keys_from_pos(const CellGrid& g, Ctrl* ctrl, const float* lon, const float* lat, uint32_t* key,
                          uint32_t* id, uint32_t n, cudaStream_t st);

// LSD radix sort of (key, id), 8-bit digits: per pass hist -> scan -> scatter (ping-pong buffers).
struct SortScratch {
  uint32_t* counts;      // [256 * ntiles]
  uint32_t* digit_total; // [256]
  uint32_t ntiles_cap;
};
int sort_tiles(uint32_t n);
int radix_passes(int bits);
void launch_radix_hist(const uint32_t* key, uint32_t n, int shift, SortScratch& s, uint32_t* digit_total, Ctrl* ctrl,
                       cudaStream_t st);
void launch_radix_scan(uint32_t n, SortScratch& s, const uint32_t* digit_total, Ctrl* ctrl, cudaStream_t st);
void launch_radix_scatter(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                          int shift, SortScratch& s, Ctrl* ctrl, cudaStream_t st);
void launch_cells(const uint32_t* key, const uint32_t* id, const float* plon, const float* plat, float2* spos,
                  uint32_t* cell_start, Ctrl* ctrl, uint32_t n, uint32_t invalid_key, cudaStream_t st);

// Pair sweep and neighbour lists.
int sweep_blocks(uint32_t n);
void launch_sweep_count(const CellGrid& g, const PairParams& pp, const uint32_t* key, const float2* spos,
                        const uint32_t* cell_start, Ctrl* ctrl, uint32_t* deg, uint32_t* block_sum, uint32_t n,
                        cudaStream_t st);
void launch_scan_blocks(uint32_t* block_sum, uint32_t nblocks, Ctrl* ctrl, cudaStream_t st);
void launch_sweep_fill(const CellGrid& g, const PairParams& pp, const RpsParams& rp, const StepArgs& a,
                       const uint32_t* key, const uint32_t* id, const float2* spos, const uint32_t* cell_start,
                       const uint32_t* block_sum, Ctrl* ctrl, const uint32_t* deg, uint32_t* off, uint32_t* adj,
                       unsigned long long* prio, uint32_t* want0, uint32_t* head, uint32_t* act0, uint32_t* level,
                       uint32_t n, cudaStream_t st);

// Interaction rounds (cooperative persistent kernel).
struct RoundBufs {
  const uint32_t* off;
  const uint32_t* deg;
  const uint32_t* adj;
  const uint32_t* id;
  int8_t* species;
  uint32_t* want[2];
  uint32_t* head;
  uint32_t* act[2];
  uint32_t* level;    // per vertex: level of its last applied pair
  uint32_t* plog;     // 3 x uint32 per logged pair (i, j, level) or nullptr
  uint32_t plog_cap;  // entries
};
int rounds_grid(int device, int* block);
cudaError_t launch_rounds(const RoundBufs& b, const RpsParams& rp, const StepArgs& a, Ctrl* ctrl, uint32_t n,
                          int grid, int block, uint32_t round_cap, cudaStream_t st);
void launch_census(const int8_t* species, Ctrl* ctrl, uint32_t n, cudaStream_t st);
void launch_step_end(Ctrl* ctrl, cudaStream_t st);
void launch_step_begin(Ctrl* ctrl, cudaStream_t st);

}  // namespace lm
