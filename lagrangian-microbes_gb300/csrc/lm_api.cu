// C-ABI of liblmgb300 (declared in include/lm_api.h): context, device buffers, step orchestration,
// neighbour-list regrowth and CUDA-graph capture. Kernels live in k_advect.cu (K1), k_bin.cu (K2),
// k_pairs.cu (K3) and k_rounds.cu (K4/K5).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lm_api.h"
#include "lm_internal.h"

using namespace lm;

namespace {

constexpr uint32_t ROUND_CAP = 1u << 22;
constexpr uint64_t MAX_CELLS = 1ull << 26;
thread_local std::string g_create_error;

}  // namespace

struct lm_ctx {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t st = nullptr;
  std::string err;

  // field
  float2* uv = nullptr;
  size_t uv_n = 0;
  FieldView fv{};
  bool has_field = false;
  double lon0 = 0, lat0 = 0, dlon = 0, dlat = 0, lon1 = 0, lat1 = 0, t_first = 0, t_last = 0;
  double org_lon = 0, org_lat = 0;

  // particles and per-particle scratch
  uint32_t n = 0;       // particles in the state
  uint32_t ncap = 0;    // capacity of per-particle buffers
  bool has_particles = false;  // positions + species (fused path)
  bool has_species = false;    // species only (two-phase interaction path)
  float *xo = nullptr, *yo = nullptr, *plon = nullptr, *plat = nullptr;
  int8_t* species = nullptr;
  uint8_t* status = nullptr;
  uint32_t *key[2] = {nullptr, nullptr}, *id[2] = {nullptr, nullptr};
  float2* spos = nullptr;
  uint32_t *deg = nullptr, *off = nullptr, *block_sum = nullptr, *head = nullptr, *level = nullptr;
  uint32_t *want[2] = {nullptr, nullptr}, *act[2] = {nullptr, nullptr};
  uint32_t* sort_counts = nullptr;
  uint32_t* digit_total = nullptr;
  size_t sort_counts_cap = 0;

  // neighbour lists
  uint32_t* adj = nullptr;
  unsigned long long* prio = nullptr;
  size_t adj_cap = 0;
  int64_t regrows = 0;

  // cells
  uint32_t* cell_start = nullptr;
  size_t cells_cap = 0;
  CellGrid grid{};
  int key_bits = 1;

  // interaction parameters
  bool has_params = false;
  PairParams pp{};
  RpsParams rp{};

  // control block
  Ctrl* ctrl = nullptr;
  Ctrl* hctrl = nullptr;  // pinned mirror
  uint32_t* hstage = nullptr;  // pinned staging (census)
  size_t hstage_n = 0;

  // pair log
  uint32_t* plog = nullptr;
  uint32_t plog_cap = 0;

  // rounds launch shape
  int rgrid = 0, rblock = 0;

  // graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  double g_t_start = 0, g_dt = 0, g_kh = 0;
  int64_t g_step0 = 0;
  int g_spg = 0;
  uint32_t g_flags = 0;
  int64_t next_step = 0;  // host mirror of the device step counter

  // per-kernel CUDA-event timing of plain launches (lm_profile_enable)
  bool prof_on = false;
  bool capturing = false;
  std::vector<cudaEvent_t> ev_pool;
  struct Pend {
    int id;
    cudaEvent_t a, b;
  };
  std::vector<Pend> pend;
  double prof_ms[32] = {};
  int64_t prof_n[32] = {};
};

namespace {

enum ProfId {
  P_ADVECT, P_KEYS, P_HIST, P_SCAN, P_SCATTER, P_CELLS, P_SWEEP_COUNT, P_SCAN_BLOCKS, P_SWEEP_FILL, P_ROUNDS,
  P_CENSUS, P_BOOKKEEPING, P_COUNT
};
const char* const kProfNames[P_COUNT] = {"k_advect",      "k_keys_from_pos", "k_radix_hist", "k_radix_scan",
                                         "k_radix_scatter", "k_cells",       "k_sweep_count", "k_scan_blocks",
                                         "k_sweep_fill",  "k_rounds",        "k_census",      "k_step_begin_end"};

cudaEvent_t prof_begin(lm_ctx* c) {
  if (!c->prof_on || c->capturing) return nullptr;
  cudaEvent_t e;
  if (!c->ev_pool.empty()) {
    e = c->ev_pool.back();
    c->ev_pool.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  cudaEventRecord(e, c->st);
  return e;
}

void prof_end(lm_ctx* c, int id, cudaEvent_t a) {
  if (!a) return;
  cudaEvent_t b;
  if (!c->ev_pool.empty()) {
    b = c->ev_pool.back();
    c->ev_pool.pop_back();
  } else if (cudaEventCreate(&b) != cudaSuccess) {
    cudaGetLastError();
    c->ev_pool.push_back(a);
    return;
  }
  cudaEventRecord(b, c->st);
  c->pend.push_back({id, a, b});
}

// Accumulate the timings of completed launches (call after a stream synchronisation).
void prof_collect(lm_ctx* c) {
  for (auto& p : c->pend) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      c->prof_ms[p.id] += ms;
      c->prof_n[p.id] += 1;
    } else {
      cudaGetLastError();
    }
    c->ev_pool.push_back(p.a);
    c->ev_pool.push_back(p.b);
  }
  c->pend.clear();
}

#define PROF(c, id, stmt)              \
  do {                                 \
    cudaEvent_t pa_ = prof_begin(c);   \
    stmt;                              \
    prof_end(c, id, pa_);              \
  } while (0)

int fail(lm_ctx* c, int code, const char* fmt, ...) __attribute__((format(printf, 3, 4)));
int fail(lm_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  else g_create_error = buf;
  return code;
}

#define CK(call)                                                                                 \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return fail(c, LM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int dalloc(lm_ctx* c, T** p, size_t count) {
  if (*p) {
    cudaFree(*p);
    *p = nullptr;
  }
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(c, LM_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
  }
  return LM_OK;
}

int ensure_particles(lm_ctx* c, uint32_t n) {
  if (n <= c->ncap && c->xo) return LM_OK;
  uint32_t cap = std::max<uint32_t>(n, 1024);
  int r = LM_OK;
  if ((r = dalloc(c, &c->xo, cap)) || (r = dalloc(c, &c->yo, cap)) || (r = dalloc(c, &c->plon, cap)) ||
      (r = dalloc(c, &c->plat, cap)) || (r = dalloc(c, &c->species, cap)) || (r = dalloc(c, &c->status, cap)) ||
      (r = dalloc(c, &c->key[0], cap)) || (r = dalloc(c, &c->key[1], cap)) || (r = dalloc(c, &c->id[0], cap)) ||
      (r = dalloc(c, &c->id[1], cap)) || (r = dalloc(c, &c->spos, cap)) || (r = dalloc(c, &c->deg, cap)) ||
      (r = dalloc(c, &c->off, cap)) || (r = dalloc(c, &c->head, cap)) || (r = dalloc(c, &c->level, cap)) || (r = dalloc(c, &c->want[0], cap)) ||
      (r = dalloc(c, &c->want[1], cap)) || (r = dalloc(c, &c->act[0], cap)) || (r = dalloc(c, &c->act[1], cap)) ||
      (r = dalloc(c, &c->block_sum, (size_t)sweep_blocks(cap) + 1)) ||
      (r = dalloc(c, &c->sort_counts, (size_t)256 * sort_tiles(cap))) ||
      (r = dalloc(c, &c->digit_total, (size_t)256 * 4)))
    return r;
  c->ncap = cap;
  return LM_OK;
}

int set_adj_capacity(lm_ctx* c, size_t cap) {
  int r;
  if (cap > 0xfffffff0ull) cap = 0xfffffff0ull;
  if ((r = dalloc(c, &c->adj, cap)) || (r = dalloc(c, &c->prio, cap))) return r;
  c->adj_cap = cap;
  unsigned long long cv = cap;
  CK(cudaMemcpyAsync(&c->ctrl->cap, &cv, sizeof(cv), cudaMemcpyHostToDevice, c->st));
  // the pair log holds at most one entry per unordered pair
  c->plog_cap = (uint32_t)std::min<size_t>(cap / 2 + 1, 0x7fffffffu);
  if ((r = dalloc(c, &c->plog, (size_t)3 * c->plog_cap))) return r;
  CK(cudaStreamSynchronize(c->st));
  return LM_OK;
}

int ensure_adj(lm_ctx* c, uint32_t n) {
  size_t want = std::max<size_t>((size_t)16 * n, (size_t)1 << 16);
  if (c->adj && c->adj_cap >= want) return LM_OK;
  return set_adj_capacity(c, want);
}

// Cell grid over [x0, x1] x [y0, y1] with one margin cell per side; cell size >= radius.
int set_grid(lm_ctx* c, double x0, double y0, double x1, double y1) {
  double r = c->pp.r;
  double cs = r * 1.004;
  double w = std::max(x1 - x0, 0.0), h = std::max(y1 - y0, 0.0);
  if (!(cs > 0) || !std::isfinite(cs)) cs = std::max(std::max(w, h), 1e-6);
  double ncx = std::floor(w / cs) + 3, ncy = std::floor(h / cs) + 3;
  if (ncx * ncy > (double)MAX_CELLS - 1) {
    cs = std::sqrt(std::max(w * h, 1e-300) / (double)(MAX_CELLS / 2));
    cs = std::max(cs, r * 1.004);
    ncx = std::floor(w / cs) + 3;
    ncy = std::floor(h / cs) + 3;
  }
  CellGrid g;
  g.x0 = (float)(x0 - cs);
  g.y0 = (float)(y0 - cs);
  g.inv_c = (float)(1.0 / cs);
  g.ncx = (int)ncx;
  g.ncy = (int)ncy;
  g.ncells = (uint32_t)(ncx * ncy);
  int bits = 1;
  while (bits < 32 && ((uint64_t)1 << bits) <= (uint64_t)g.ncells) ++bits;  // ncells itself = invalid key
  if (g.ncells + 1 > c->cells_cap) {
    int rr = dalloc(c, &c->cell_start, (size_t)g.ncells + 1);
    if (rr) return rr;
    c->cells_cap = (size_t)g.ncells + 1;
  }
  c->grid = g;
  c->key_bits = bits;
  return LM_OK;
}

int set_field_grid(lm_ctx* c) {
  // Cells are addressed in absolute degrees over the field domain.
  return set_grid(c, c->lon0, c->lat0, c->lon1, c->lat1);
}

int read_ctrl(lm_ctx* c) {
  CK(cudaMemcpyAsync(c->hctrl, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  prof_collect(c);
  return LM_OK;
}

int write_ctrl_step(lm_ctx* c, int64_t step) {
  uint32_t s = (uint32_t)step;
  CK(cudaMemcpyAsync(&c->ctrl->step, &s, sizeof(s), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->next_step = step;
  return LM_OK;
}

int clear_halt(lm_ctx* c) {
  // halt = 0 and the overflow bit cleared; other sticky bits are kept
  c->hctrl->halt = 0;
  c->hctrl->err &= ~(uint32_t)ERRB_OVERFLOW;
  CK(cudaMemcpyAsync(&c->ctrl->halt, &c->hctrl->halt, sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(&c->ctrl->err, &c->hctrl->err, sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return LM_OK;
}

// Map and clear the sticky device error bits.
int consume_errors(lm_ctx* c) {
  uint32_t e = c->hctrl->err;
  if (!e) return LM_OK;
  uint32_t zero = 0;
  CK(cudaMemcpyAsync(&c->ctrl->err, &zero, sizeof(zero), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->hctrl->err = 0;
  if (e & ERRB_TIMEOUT) return fail(c, LM_ERR_TIMEOUT, "a device barrier wait timed out");
  if (e & ERRB_ROUNDCAP) return fail(c, LM_ERR_ROUND_CAP, "interaction round cap (%u) reached", ROUND_CAP);
  if (e & ERRB_TIME) return fail(c, LM_ERR_TIME, "a stage time fell outside the field's time axis");
  if (e & ERRB_NAN) return fail(c, LM_ERR_NAN, "non-finite particle positions (%u flagged in total)", c->hctrl->oob);
  if (e & ERRB_OOB)
    return fail(c, LM_ERR_OUT_OF_BOUNDS, "particles left the field domain (%u flagged in total)", c->hctrl->oob);
  if (e & ERRB_OVERFLOW) return fail(c, LM_ERR_CAPACITY, "neighbour-list capacity exceeded");
  return LM_OK;
}

StepArgs step_args(const lm_ctx* c, double t, double dt, int64_t step, double kh, bool graph) {
  StepArgs a;
  a.t_start = t;
  a.dt = dt;
  a.step0 = (uint32_t)step;
  a.use_ctrl_step = graph ? 1 : 0;
  a.kick = kh > 0 ? (float)std::sqrt(6.0 * std::fabs(dt) * kh) : 0.f;
  a.seed_lo = c->rp.seed_lo;
  a.seed_hi = c->rp.seed_hi;
  return a;
}

cudaError_t enqueue_interaction(lm_ctx* c, const StepArgs& a, uint32_t flags, uint32_t n) {
  cudaStream_t st = c->st;
  SortScratch ss{c->sort_counts, c->digit_total, (uint32_t)sort_tiles(c->ncap)};
  const int passes = radix_passes(c->key_bits);
  cudaError_t e = cudaMemsetAsync(c->digit_total, 0, sizeof(uint32_t) * 256 * passes, st);
  if (e != cudaSuccess) return e;
  int r = 0;
  for (int p = 0; p < passes; ++p) {
    uint32_t* dt = c->digit_total + 256 * p;
    PROF(c, P_HIST, launch_radix_hist(c->key[r], n, 8 * p, ss, dt, c->ctrl, st));
    PROF(c, P_SCAN, launch_radix_scan(n, ss, dt, c->ctrl, st));
    PROF(c, P_SCATTER, launch_radix_scatter(c->key[r], c->id[r], c->key[r ^ 1], c->id[r ^ 1], n, 8 * p, ss, c->ctrl, st));
    r ^= 1;
  }
  PROF(c, P_CELLS,
       launch_cells(c->key[r], c->id[r], c->plon, c->plat, c->spos, c->cell_start, c->ctrl, n, c->grid.ncells, st));
  PROF(c, P_SWEEP_COUNT,
       launch_sweep_count(c->grid, c->pp, c->key[r], c->spos, c->cell_start, c->ctrl, c->deg, c->block_sum, n, st));
  PROF(c, P_SCAN_BLOCKS, launch_scan_blocks(c->block_sum, (uint32_t)sweep_blocks(n), c->ctrl, st));
  PROF(c, P_SWEEP_FILL,
       launch_sweep_fill(c->grid, c->pp, c->rp, a, c->key[r], c->id[r], c->spos, c->cell_start, c->block_sum, c->ctrl,
                         c->deg, c->off, c->adj, c->prio, c->want[0], c->head, c->act[0], c->level, n, st));
  if (flags & LM_STEP_INTERACT) {
    RoundBufs rb;
    rb.off = c->off;
    rb.deg = c->deg;
    rb.adj = c->adj;
    rb.id = c->id[r];
    rb.species = c->species;
    rb.want[0] = c->want[0];
    rb.want[1] = c->want[1];
    rb.head = c->head;
    rb.act[0] = c->act[0];
    rb.act[1] = c->act[1];
    rb.level = c->level;
    rb.plog = (flags & LM_STEP_LOG_PAIRS) ? c->plog : nullptr;
    rb.plog_cap = c->plog_cap;
    cudaEvent_t pa = prof_begin(c);
    e = launch_rounds(rb, c->rp, a, c->ctrl, n, c->rgrid, c->rblock, ROUND_CAP, st);
    prof_end(c, P_ROUNDS, pa);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

// One fused step; `advect` false re-runs only the interaction part (overflow recovery).
cudaError_t enqueue_step(lm_ctx* c, const StepArgs& a, uint32_t flags, bool advect) {
  PROF(c, P_BOOKKEEPING, launch_step_begin(c->ctrl, c->st));
  if (advect && (flags & LM_STEP_ADVECT))
    PROF(c, P_ADVECT, launch_advect(c->fv, c->grid, a, c->ctrl, c->xo, c->yo, c->status, c->plon, c->plat,
                                    c->key[0], c->id[0], c->n, c->st));
  if (flags & LM_STEP_INTERACT) {
    cudaError_t e = enqueue_interaction(c, a, flags, c->n);
    if (e != cudaSuccess) return e;
  }
  if (flags & LM_STEP_CENSUS) PROF(c, P_CENSUS, launch_census(c->species, c->ctrl, c->n, c->st));
  PROF(c, P_BOOKKEEPING, launch_step_end(c->ctrl, c->st));
  return cudaGetLastError();
}

int clear_err_bits(lm_ctx* c, uint32_t mask) {
  c->hctrl->err &= ~mask;
  CK(cudaMemcpyAsync(&c->ctrl->err, &c->hctrl->err, sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return LM_OK;
}

int ensure_hstage(lm_ctx* c, size_t n) {
  if (c->hstage_n >= n) return LM_OK;
  if (c->hstage) cudaFreeHost(c->hstage);
  c->hstage = nullptr;
  CK(cudaMallocHost((void**)&c->hstage, n * sizeof(uint32_t)));
  c->hstage_n = n;
  return LM_OK;
}

int regrow(lm_ctx* c) {
  size_t need = (size_t)c->hctrl->n_dir;
  size_t cap = std::max(need + need / 4 + 1024, c->adj_cap * 2);
  int r = set_adj_capacity(c, cap);
  if (r) return r;
  c->regrows++;
  return clear_halt(c);
}

int check_time(lm_ctx* c, double t, double dt, int n_steps) {
  double lo = std::min(t, t + dt * n_steps), hi = std::max(t, t + dt * n_steps);
  double tol = 1e-9 * std::fabs(c->fv.dT);
  if (lo < c->t_first - tol || hi > c->t_last + tol)
    return fail(c, LM_ERR_TIME, "time window [%.9g, %.9g] s is outside the field's [%.9g, %.9g] s", lo, hi,
                c->t_first, c->t_last);
  return LM_OK;
}

int set_pair_params(lm_ctx* c, double r, int norm) {
  PairParams& pp = c->pp;
  pp.r = r;
  pp.r2 = r * r;
  pp.norm = norm;
  const double band = 2e-6;
  if (r > 1e-15 && r < 1e15) {
    pp.r2f_lo = std::nextafter((float)(pp.r2 * (1 - band)), 0.f);
    pp.r2f_hi = std::nextafter((float)(pp.r2 * (1 + band)), INFINITY);
    pp.rf_lo = std::nextafter((float)(r * (1 - band)), 0.f);
    pp.rf_hi = std::nextafter((float)(r * (1 + band)), INFINITY);
  } else {  // float32 cannot represent the band: decide every candidate in float64
    pp.r2f_lo = pp.rf_lo = -1.f;
    pp.r2f_hi = pp.rf_hi = INFINITY;
  }
  return LM_OK;
}

unsigned long long prob_threshold(double p) {
  if (!(p > 0)) return 0ull;  // also NaN: r < NaN is false
  if (p >= 1.0) return 1ull << 53;
  return (unsigned long long)std::ceil(std::ldexp(p, 53));
}

bool uniform_axis(const double* a, int n, double* d) {
  if (n < 2) return false;
  double step = (a[n - 1] - a[0]) / (n - 1);
  if (!(step > 0) || !std::isfinite(step)) return false;
  for (int k = 0; k < n; ++k)
    if (std::fabs(a[k] - (a[0] + step * k)) > 1e-6 * step) return false;
  *d = step;
  return true;
}

}  // namespace

extern "C" {

int lm_version(void) { return LM_API_VERSION; }

int lm_ctx_create(int device, lm_ctx** out) {
  if (!out) return fail(nullptr, LM_ERR_ARG, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(nullptr, LM_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  if (device < 0 || device >= ndev) return fail(nullptr, LM_ERR_ARG, "device %d out of range [0, %d)", device, ndev);
  lm_ctx* c = new lm_ctx();
  c->device = device;
  auto bail = [&](int code) {
    g_create_error = c->err;
    lm_ctx_destroy(c);
    return code;
  };
  if ((e = cudaSetDevice(device)) != cudaSuccess) {
    fail(c, LM_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    return bail(LM_ERR_CUDA);
  }
  if ((e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking)) != cudaSuccess) {
    fail(c, LM_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    return bail(LM_ERR_CUDA);
  }
  c->st = c->own;
  int r = dalloc(c, &c->ctrl, 1);
  if (r) return bail(r);
  if ((e = cudaMallocHost((void**)&c->hctrl, sizeof(Ctrl))) != cudaSuccess) {
    fail(c, LM_ERR_CUDA, "cudaMallocHost: %s", cudaGetErrorString(e));
    return bail(LM_ERR_CUDA);
  }
  memset(c->hctrl, 0, sizeof(Ctrl));
  if ((e = cudaMemsetAsync(c->ctrl, 0, sizeof(Ctrl), c->st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->st)) != cudaSuccess) {
    fail(c, LM_ERR_CUDA, "ctrl init: %s", cudaGetErrorString(e));
    return bail(LM_ERR_CUDA);
  }
  c->rgrid = rounds_grid(device, &c->rblock);
  *out = c;
  return LM_OK;
}

int lm_ctx_destroy(lm_ctx* c) {
  if (!c) return LM_OK;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  void* bufs[] = {c->uv,          c->xo,      c->yo,      c->plon,   c->plat,      c->species,   c->status,
                  c->key[0],      c->key[1],  c->id[0],   c->id[1],  c->spos,      c->deg,       c->off,
                  c->block_sum,   c->head,    c->want[0], c->want[1], c->act[0],   c->act[1],    c->sort_counts, c->level,
                  c->digit_total, c->adj,     c->prio,    c->cell_start, c->ctrl,  c->plog};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (c->hctrl) cudaFreeHost(c->hctrl);
  if (c->hstage) cudaFreeHost(c->hstage);
  for (auto& p : c->pend) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return LM_OK;
}

int lm_last_error(const lm_ctx* c, char* buf, size_t len) {
  if (!buf || len == 0) return LM_ERR_ARG;
  const std::string& s = c ? c->err : g_create_error;
  snprintf(buf, len, "%s", s.c_str());
  return LM_OK;
}

int lm_ctx_set_stream(lm_ctx* c, uintptr_t stream) {
  if (!c) return LM_ERR_ARG;
  CK(cudaStreamSynchronize(c->st));
  c->st = stream ? (cudaStream_t)stream : c->own;
  return LM_OK;
}

int lm_sync(lm_ctx* c) {
  if (!c) return LM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  int r = read_ctrl(c);
  if (r) return r;
  return consume_errors(c);
}

int lm_field_upload(lm_ctx* c, const float* u, const float* v, int nt, int ny, int nx, const double* lon,
                    const double* lat, const double* t_sec) {
  if (!c || !u || !v || !lon || !lat || !t_sec) return fail(c, LM_ERR_ARG, "NULL argument");
  if (nt < 2 || ny < 2 || nx < 2) return fail(c, LM_ERR_ARG, "field needs nt, ny, nx >= 2 (got %d, %d, %d)", nt, ny, nx);
  double dx, dy, dT;
  if (!uniform_axis(lon, nx, &dx)) return fail(c, LM_ERR_GRID, "longitude axis is not uniform and ascending");
  if (!uniform_axis(lat, ny, &dy)) return fail(c, LM_ERR_GRID, "latitude axis is not uniform and ascending");
  if (!uniform_axis(t_sec, nt, &dT)) return fail(c, LM_ERR_GRID, "time axis is not uniform and ascending");
  CK(cudaSetDevice(c->device));
  size_t n = (size_t)nt * ny * nx;
  int r;
  if (n > c->uv_n || !c->uv) {
    if ((r = dalloc(c, &c->uv, n))) return r;
    c->uv_n = n;
  }
  // stage u and v through a temporary device buffer, then interleave
  float* tmp = nullptr;
  if ((r = dalloc(c, &tmp, 2 * n))) return r;
  CK(cudaMemcpyAsync(tmp, u, n * sizeof(float), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(tmp + n, v, n * sizeof(float), cudaMemcpyHostToDevice, c->st));
  launch_interleave(tmp, tmp + n, c->uv, n, c->st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  cudaFree(tmp);
  c->lon0 = lon[0];
  c->lat0 = lat[0];
  c->lon1 = lon[nx - 1];
  c->lat1 = lat[ny - 1];
  c->dlon = dx;
  c->dlat = dy;
  c->t_first = t_sec[0];
  c->t_last = t_sec[nt - 1];
  c->org_lon = (double)(float)lon[0];
  c->org_lat = (double)(float)lat[0];
  FieldView& f = c->fv;
  f.uv = c->uv;
  f.nx = nx;
  f.ny = ny;
  f.nt = nt;
  f.gx0 = (float)(lon[0] - c->org_lon);
  f.gy0 = (float)(lat[0] - c->org_lat);
  f.inv_dx = (float)(1.0 / dx);
  f.inv_dy = (float)(1.0 / dy);
  f.max_fx = (float)(nx - 1);
  f.max_fy = (float)(ny - 1);
  f.org_lon = (float)c->org_lon;
  f.org_lat = (float)c->org_lat;
  f.t0 = t_sec[0];
  f.dT = dT;
  c->has_field = true;
  if (c->has_particles) {  // offsets are relative to the field origin: positions must be re-uploaded
    c->has_particles = false;
    c->has_species = false;
  }
  return LM_OK;
}

int lm_particles_upload(lm_ctx* c, int64_t n, const double* lon, const double* lat, const int8_t* species) {
  if (!c || (n > 0 && (!lon || !lat))) return fail(c, LM_ERR_ARG, "NULL argument");
  if (n < 0 || n > 0x7fffffff) return fail(c, LM_ERR_ARG, "particle count %lld out of range", (long long)n);
  if (!c->has_field) return fail(c, LM_ERR_STATE, "upload the velocity field before the particles");
  CK(cudaSetDevice(c->device));
  int r;
  if ((r = ensure_particles(c, (uint32_t)n)) || (r = ensure_adj(c, (uint32_t)n))) return r;
  std::vector<float> xo(n), yo(n);
  for (int64_t k = 0; k < n; ++k) {
    xo[k] = (float)(lon[k] - c->org_lon);
    yo[k] = (float)(lat[k] - c->org_lat);
  }
  if (n > 0) {
    CK(cudaMemcpyAsync(c->xo, xo.data(), n * sizeof(float), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->yo, yo.data(), n * sizeof(float), cudaMemcpyHostToDevice, c->st));
    if (species) CK(cudaMemcpyAsync(c->species, species, n, cudaMemcpyHostToDevice, c->st));
    else CK(cudaMemsetAsync(c->species, 0, n, c->st));
    CK(cudaMemsetAsync(c->status, 0, n, c->st));
  }
  uint32_t zero = 0;
  CK(cudaMemcpyAsync(&c->ctrl->oob, &zero, sizeof(zero), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->n = (uint32_t)n;
  c->has_particles = true;
  c->has_species = true;
  return LM_OK;
}

int lm_species_upload(lm_ctx* c, int64_t n, const int8_t* species) {
  if (!c || (n > 0 && !species)) return fail(c, LM_ERR_ARG, "NULL argument");
  if (n < 0 || n > 0x7fffffff) return fail(c, LM_ERR_ARG, "species count out of range");
  if (c->has_particles && n != (int64_t)c->n)
    return fail(c, LM_ERR_ARG, "n = %lld but the context holds %u particles", (long long)n, c->n);
  CK(cudaSetDevice(c->device));
  int r;
  if (!c->has_particles) {
    if ((r = ensure_particles(c, (uint32_t)n)) || (r = ensure_adj(c, (uint32_t)n))) return r;
    c->n = (uint32_t)n;
  }
  if (n) CK(cudaMemcpyAsync(c->species, species, n, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->has_species = true;
  return LM_OK;
}

int lm_particles_download(lm_ctx* c, float* lon, float* lat, int8_t* species, uint8_t* status) {
  if (!c) return LM_ERR_ARG;
  if (!c->has_particles && (lon || lat || status || !c->has_species)) return fail(c, LM_ERR_STATE, "no particles");
  CK(cudaSetDevice(c->device));
  uint32_t n = c->n;
  std::vector<float> xo(lon ? n : 0), yo(lat ? n : 0);
  if (n) {
    if (lon) CK(cudaMemcpyAsync(xo.data(), c->xo, n * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    if (lat) CK(cudaMemcpyAsync(yo.data(), c->yo, n * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    if (species) CK(cudaMemcpyAsync(species, c->species, n, cudaMemcpyDeviceToHost, c->st));
    if (status) CK(cudaMemcpyAsync(status, c->status, n, cudaMemcpyDeviceToHost, c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  const float ox = (float)c->org_lon, oy = (float)c->org_lat;
  for (uint32_t k = 0; lon && k < n; ++k) lon[k] = ox + xo[k];  // same single rounding as the device
  for (uint32_t k = 0; lat && k < n; ++k) lat[k] = oy + yo[k];
  return LM_OK;
}

int lm_set_interaction(lm_ctx* c, double radius, int norm, double p_rs, double p_pr, double p_sp, uint64_t seed) {
  if (!c) return LM_ERR_ARG;
  if (!(radius >= 0) || !std::isfinite(radius)) return fail(c, LM_ERR_ARG, "radius must be finite and >= 0");
  if (norm != LM_NORM_INF && norm != LM_NORM_L1 && norm != LM_NORM_L2)
    return fail(c, LM_ERR_ARG, "norm must be 1, 2 or infinity (code 0); got %d", norm);
  set_pair_params(c, radius, norm);
  c->rp.t_rs = prob_threshold(p_rs);
  c->rp.t_pr = prob_threshold(p_pr);
  c->rp.t_sp = prob_threshold(p_sp);
  c->rp.seed_lo = (uint32_t)seed;
  c->rp.seed_hi = (uint32_t)(seed >> 32);
  c->has_params = true;
  return LM_OK;
}

static int run_steps(lm_ctx* c, double t, double dt, int n_steps, int64_t step0, uint32_t flags, double kh,
                     float* rec_lon, float* rec_lat, int8_t* rec_species, int64_t* rec_census) {
  const uint32_t n = c->n;
  int r;
  if ((r = write_ctrl_step(c, step0))) return r;
  if (rec_census && (r = ensure_hstage(c, (size_t)4 * n_steps))) return r;
  int64_t s = 0;
  bool redo_interaction_only = false;
  while (s < n_steps) {
    for (int64_t k = s; k < n_steps; ++k) {
      StepArgs a = step_args(c, t + dt * k, dt, step0 + k, kh, false);
      CK(enqueue_step(c, a, flags, !(redo_interaction_only && k == s)));
      if (n) {
        if (rec_lon) CK(cudaMemcpyAsync(rec_lon + k * n, c->plon, n * sizeof(float), cudaMemcpyDeviceToHost, c->st));
        if (rec_lat) CK(cudaMemcpyAsync(rec_lat + k * n, c->plat, n * sizeof(float), cudaMemcpyDeviceToHost, c->st));
        if (rec_species) CK(cudaMemcpyAsync(rec_species + k * n, c->species, n, cudaMemcpyDeviceToHost, c->st));
      }
      if (rec_census)
        CK(cudaMemcpyAsync(c->hstage + 4 * k, c->ctrl->census, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
    }
    CK(cudaGetLastError());
    if ((r = read_ctrl(c))) return r;
    if (c->hctrl->halt) {
      int64_t k = (int64_t)c->hctrl->halt_step - step0;
      if ((r = regrow(c))) return r;
      if ((r = write_ctrl_step(c, step0 + k))) return r;
      s = k;
      redo_interaction_only = true;  // the halted step was advected already
      continue;
    }
    break;
  }
  c->next_step = step0 + n_steps;
  if (rec_census)
    for (int64_t k = 0; k < 4 * (int64_t)n_steps; ++k) rec_census[k] = c->hstage[k];
  return consume_errors(c);
}

int lm_step(lm_ctx* c, double t_sec, double dt_sec, int n_steps, int64_t step0, uint32_t flags, double kh_deg2_s,
            float* rec_lon, float* rec_lat, int8_t* rec_species, int64_t* rec_census) {
  if (!c) return LM_ERR_ARG;
  if (n_steps < 0) return fail(c, LM_ERR_ARG, "n_steps < 0");
  if (!(flags & LM_STEP_ADVECT)) return fail(c, LM_ERR_ARG, "lm_step needs LM_STEP_ADVECT (use lm_interact)");
  if (!c->has_field || !c->has_particles) return fail(c, LM_ERR_STATE, "field and particles must be uploaded first");
  if ((flags & LM_STEP_INTERACT) && !c->has_params) return fail(c, LM_ERR_STATE, "call lm_set_interaction first");
  if (!(dt_sec != 0) || !std::isfinite(dt_sec)) return fail(c, LM_ERR_ARG, "dt must be finite and nonzero");
  if (!(kh_deg2_s >= 0)) return fail(c, LM_ERR_ARG, "Kh must be >= 0");
  CK(cudaSetDevice(c->device));
  int r;
  if ((r = check_time(c, t_sec, dt_sec, n_steps))) return r;
  if (!c->has_params) set_pair_params(c, 0.0, LM_NORM_L2);
  if ((r = set_field_grid(c))) return r;
  if (n_steps == 0) return LM_OK;
  return run_steps(c, t_sec, dt_sec, n_steps, step0, flags, kh_deg2_s, rec_lon, rec_lat, rec_species, rec_census);
}

// Bounding box of finite positions (host loop; the positions come from the host anyway).
static void bbox(const float* lon, const float* lat, int64_t n, double* x0, double* y0, double* x1, double* y1) {
  float a = INFINITY, b = INFINITY, cmax = -INFINITY, d = -INFINITY;
  for (int64_t k = 0; k < n; ++k) {
    float x = lon[k], y = lat[k];
    if (!std::isfinite(x) || !std::isfinite(y)) continue;
    a = std::min(a, x);
    cmax = std::max(cmax, x);
    b = std::min(b, y);
    d = std::max(d, y);
  }
  if (!(a <= cmax)) a = cmax = b = d = 0.f;
  *x0 = a;
  *y0 = b;
  *x1 = cmax;
  *y1 = d;
}

static int stage_positions(lm_ctx* c, int64_t n, const float* lon, const float* lat) {
  int r;
  if ((r = ensure_particles(c, (uint32_t)n)) || (r = ensure_adj(c, (uint32_t)n))) return r;
  double x0, y0, x1, y1;
  bbox(lon, lat, n, &x0, &y0, &x1, &y1);
  if ((r = set_grid(c, x0, y0, x1, y1))) return r;
  if (n) {
    CK(cudaMemcpyAsync(c->plon, lon, n * sizeof(float), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->plat, lat, n * sizeof(float), cudaMemcpyHostToDevice, c->st));
  }
  return LM_OK;
}

int lm_query_pairs(lm_ctx* c, int64_t n, const float* lon, const float* lat, int32_t* pi, int32_t* pj, int64_t cap,
                   int64_t* n_pairs) {
  if (!c || !n_pairs || (n > 0 && (!lon || !lat))) return fail(c, LM_ERR_ARG, "NULL argument");
  if (n < 0 || n > 0x7fffffff) return fail(c, LM_ERR_ARG, "particle count out of range");
  if (!c->has_params) return fail(c, LM_ERR_STATE, "call lm_set_interaction first");
  CK(cudaSetDevice(c->device));
  *n_pairs = 0;
  if (n == 0) return LM_OK;
  int r;
  if ((r = stage_positions(c, n, lon, lat))) return r;
  for (;;) {
    StepArgs a = step_args(c, 0.0, 1.0, 0, 0.0, false);
    launch_step_begin(c->ctrl, c->st);
    PROF(c, P_KEYS, launch_keys_from_pos(c->grid, c->ctrl, c->plon, c->plat, c->key[0], c->id[0], (uint32_t)n, c->st));
    CK(enqueue_interaction(c, a, 0u, (uint32_t)n));
    if ((r = read_ctrl(c))) return r;
    if (c->hctrl->halt) {
      if ((r = regrow(c))) return r;
      continue;
    }
    break;
  }
  if ((r = clear_err_bits(c, ERRB_NAN))) return r;  // non-finite query points are simply never paired
  uint32_t nv = c->hctrl->n_valid;
  size_t ndir = (size_t)c->hctrl->n_dir;
  int sorted = radix_passes(c->key_bits) & 1;
  std::vector<uint32_t> deg(nv), off(nv), ids(nv), adj(ndir);
  if (nv) {
    CK(cudaMemcpyAsync(deg.data(), c->deg, nv * 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(off.data(), c->off, nv * 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(ids.data(), c->id[sorted], nv * 4, cudaMemcpyDeviceToHost, c->st));
  }
  if (ndir) CK(cudaMemcpyAsync(adj.data(), c->adj, ndir * 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  std::vector<uint64_t> pairs;
  pairs.reserve(ndir / 2);
  for (uint32_t s = 0; s < nv; ++s)
    for (uint32_t x = off[s]; x < off[s] + deg[s]; ++x) {
      uint32_t a = ids[s], b = ids[adj[x]];
      if (a < b) pairs.push_back(((uint64_t)a << 32) | b);
    }
  std::sort(pairs.begin(), pairs.end());
  *n_pairs = (int64_t)pairs.size();
  if (!pi || !pj) return LM_OK;  // count query
  if ((int64_t)pairs.size() > cap)
    return fail(c, LM_ERR_CAPACITY, "pair buffer holds %lld pairs, %zu needed", (long long)cap, pairs.size());
  for (size_t k = 0; k < pairs.size(); ++k) {
    pi[k] = (int32_t)(pairs[k] >> 32);
    pj[k] = (int32_t)(pairs[k] & 0xffffffffu);
  }
  return LM_OK;
}

int lm_interact(lm_ctx* c, int64_t n, const float* lon, const float* lat, int64_t step_index, uint32_t flags) {
  if (!c || (n > 0 && (!lon || !lat))) return fail(c, LM_ERR_ARG, "NULL argument");
  if (!c->has_params) return fail(c, LM_ERR_STATE, "call lm_set_interaction first");
  if (!c->has_species) return fail(c, LM_ERR_STATE, "upload species (lm_particles_upload or lm_species_upload) first");
  if (n != (int64_t)c->n) return fail(c, LM_ERR_ARG, "n = %lld but the context holds %u species", (long long)n, c->n);
  CK(cudaSetDevice(c->device));
  if (n == 0) return LM_OK;
  int r;
  if ((r = stage_positions(c, n, lon, lat))) return r;
  if ((r = write_ctrl_step(c, step_index))) return r;
  for (;;) {
    StepArgs a = step_args(c, 0.0, 1.0, step_index, 0.0, false);
    launch_step_begin(c->ctrl, c->st);
    PROF(c, P_KEYS, launch_keys_from_pos(c->grid, c->ctrl, c->plon, c->plat, c->key[0], c->id[0], (uint32_t)n, c->st));
    CK(enqueue_interaction(c, a, flags | LM_STEP_INTERACT, (uint32_t)n));
    if (flags & LM_STEP_CENSUS) launch_census(c->species, c->ctrl, c->n, c->st);
    launch_step_end(c->ctrl, c->st);
    CK(cudaGetLastError());
    if ((r = read_ctrl(c))) return r;
    if (c->hctrl->halt) {  // halted before the rounds ran: species untouched, safe to redo
      if ((r = regrow(c))) return r;
      if ((r = write_ctrl_step(c, step_index))) return r;
      continue;
    }
    break;
  }
  if ((r = clear_err_bits(c, ERRB_NAN))) return r;  // non-finite positions are excluded from pairing
  c->next_step = step_index + 1;
  return consume_errors(c);
}

int lm_pairs_get(lm_ctx* c, int32_t* pi, int32_t* pj, int32_t* round, int64_t cap, int64_t* n) {
  if (!c || !n) return LM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  int r;
  if ((r = read_ctrl(c))) return r;
  uint32_t m = std::min(c->hctrl->plog_n, c->plog_cap);
  *n = m;
  if (m == 0) return LM_OK;
  if (!pi || !pj || !round) return LM_OK;  // count query
  if ((int64_t)m > cap) return fail(c, LM_ERR_CAPACITY, "pair log holds %u pairs", m);
  std::vector<uint32_t> h((size_t)3 * m);
  CK(cudaMemcpyAsync(h.data(), c->plog, h.size() * 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  std::vector<uint32_t> order(m);
  for (uint32_t k = 0; k < m; ++k) order[k] = k;
  std::sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
    const uint32_t* a = &h[3 * x];
    const uint32_t* b = &h[3 * y];
    if (a[2] != b[2]) return a[2] < b[2];
    if (a[0] != b[0]) return a[0] < b[0];
    return a[1] < b[1];
  });
  for (uint32_t k = 0; k < m; ++k) {
    const uint32_t* e = &h[3 * order[k]];
    pi[k] = (int32_t)e[0];
    pj[k] = (int32_t)e[1];
    round[k] = (int32_t)e[2];
  }
  return LM_OK;
}

static int capture(lm_ctx* c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->gexec = nullptr;
  c->graph = nullptr;
  CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
  c->capturing = true;
  for (int k = 0; k < c->g_spg; ++k) {
    StepArgs a = step_args(c, c->g_t_start, c->g_dt, c->g_step0, c->g_kh, true);
    cudaError_t le = enqueue_step(c, a, c->g_flags, true);
    if (le != cudaSuccess) {
      c->capturing = false;
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(c->st, &g);
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return fail(c, LM_ERR_CUDA, "launch during capture failed: %s", cudaGetErrorString(le));
    }
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->st, &g);
  c->capturing = false;
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, LM_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
  }
  c->graph = g;
  CK(cudaGraphInstantiate(&c->gexec, c->graph, 0));
  return LM_OK;
}

int lm_graph_capture(lm_ctx* c, double t_start, double dt_sec, int64_t step0, int steps_per_graph, uint32_t flags,
                     double kh_deg2_s) {
  if (!c) return LM_ERR_ARG;
  if (steps_per_graph < 1) return fail(c, LM_ERR_ARG, "steps_per_graph must be >= 1");
  if (!(flags & LM_STEP_ADVECT)) return fail(c, LM_ERR_ARG, "graph steps need LM_STEP_ADVECT");
  if (!c->has_field || !c->has_particles) return fail(c, LM_ERR_STATE, "field and particles must be uploaded first");
  if ((flags & LM_STEP_INTERACT) && !c->has_params) return fail(c, LM_ERR_STATE, "call lm_set_interaction first");
  if (!(dt_sec != 0) || !std::isfinite(dt_sec)) return fail(c, LM_ERR_ARG, "dt must be finite and nonzero");
  CK(cudaSetDevice(c->device));
  if (!c->has_params) set_pair_params(c, 0.0, LM_NORM_L2);
  int r;
  if ((r = set_field_grid(c))) return r;
  c->g_t_start = t_start;
  c->g_dt = dt_sec;
  c->g_step0 = step0;
  c->g_spg = steps_per_graph;
  c->g_flags = flags & ~(uint32_t)LM_STEP_LOG_PAIRS;
  c->g_kh = kh_deg2_s;
  if ((r = capture(c))) return r;
  return write_ctrl_step(c, step0);
}

int lm_graph_run(lm_ctx* c, int n_launches, int sync) {
  if (!c) return LM_ERR_ARG;
  if (!c->gexec) return fail(c, LM_ERR_STATE, "no captured graph");
  if (n_launches < 0) return fail(c, LM_ERR_ARG, "n_launches < 0");
  CK(cudaSetDevice(c->device));
  const int64_t first = c->next_step;
  const int64_t total = (int64_t)n_launches * c->g_spg;
  int r;
  if ((r = check_time(c, c->g_t_start + (first - c->g_step0) * c->g_dt, c->g_dt, (int)total))) return r;
  for (int k = 0; k < n_launches; ++k) CK(cudaGraphLaunch(c->gexec, c->st));
  c->next_step = first + total;
  if (!sync) return LM_OK;
  if ((r = read_ctrl(c))) return r;
  if (c->hctrl->halt) {
    // A step overflowed its neighbour lists: the graph halted at that step (already advected).
    // Regrow, finish that step and the rest with plain launches, then recapture for later runs.
    int64_t k = (int64_t)c->hctrl->halt_step;
    if ((r = regrow(c))) return r;
    if ((r = write_ctrl_step(c, k))) return r;
    StepArgs a = step_args(c, c->g_t_start + (k - c->g_step0) * c->g_dt, c->g_dt, k, c->g_kh, false);
    CK(enqueue_step(c, a, c->g_flags, false));
    if ((r = read_ctrl(c))) return r;
    if (c->hctrl->halt) return fail(c, LM_ERR_CAPACITY, "neighbour lists overflowed again after regrowth");
    int64_t rest = first + total - (k + 1);
    if (rest > 0) {
      r = run_steps(c, c->g_t_start + (k + 1 - c->g_step0) * c->g_dt, c->g_dt, (int)rest, k + 1, c->g_flags, c->g_kh,
                    nullptr, nullptr, nullptr, nullptr);
      if (r) return r;
    }
    if ((r = capture(c))) return r;
    if ((r = write_ctrl_step(c, first + total))) return r;
  }
  return consume_errors(c);
}

int lm_set_step(lm_ctx* c, int64_t step) {
  if (!c) return LM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  return write_ctrl_step(c, step);
}

int lm_stats_get(lm_ctx* c, lm_stats* out) {
  if (!c || !out) return LM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  int r;
  if ((r = read_ctrl(c))) return r;
  const Ctrl& h = *c->hctrl;
  out->n_particles = c->n;
  out->pairs = (int64_t)(h.n_dir / 2);
  out->rounds = h.rounds;
  out->max_rounds = h.max_rounds;
  out->out_of_bounds = h.oob;
  out->step = h.step;
  for (int k = 0; k < 4; ++k) out->census[k] = h.census[k];
  out->adj_capacity = (int64_t)c->adj_cap;
  out->regrows = c->regrows;
  out->pairs_total = (int64_t)h.pairs_total;
  out->steps_total = (int64_t)h.steps_total;
  return LM_OK;
}

int lm_stats_reset(lm_ctx* c) {
  if (!c) return LM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  uint32_t zero = 0;
  unsigned long long z64 = 0;
  CK(cudaMemcpyAsync(&c->ctrl->max_rounds, &zero, sizeof(zero), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(&c->ctrl->pairs_total, &z64, sizeof(z64), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(&c->ctrl->steps_total, &z64, sizeof(z64), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return LM_OK;
}

int lm_profile_enable(lm_ctx* c, int on) {
  if (!c) return LM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->st));
  prof_collect(c);
  for (int k = 0; k < P_COUNT; ++k) {
    c->prof_ms[k] = 0;
    c->prof_n[k] = 0;
  }
  c->prof_on = on != 0;
  return LM_OK;
}

int lm_profile_get(lm_ctx* c, int kernel, char* name, size_t name_len, double* total_ms, int64_t* launches) {
  if (!c) return LM_ERR_ARG;
  if (kernel < 0 || kernel >= P_COUNT) return fail(c, LM_ERR_ARG, "kernel index %d out of range [0, %d)", kernel, P_COUNT);
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->st));
  prof_collect(c);
  if (name && name_len) snprintf(name, name_len, "%s", kProfNames[kernel]);
  if (total_ms) *total_ms = c->prof_ms[kernel];
  if (launches) *launches = c->prof_n[kernel];
  return LM_OK;
}

int lm_profile_count(void) { return P_COUNT; }

}  // extern "C"
