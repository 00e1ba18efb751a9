// C-ABI of liblmgb300 (declared in include/lm_api.h): context, ensembles, device buffers, step
// orchestration, capacity regrowth and CUDA-graph capture. Kernels live in k_advect.cu (K1),
// k_bin.cu (K2), k_pairs.cu (K3) and k_rounds.cu (K4/K5).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lm_api.h"
#include "lm_internal.h"

using namespace lm;

namespace {
thread_local std::string g_create_error;

enum ProfId {
  P_ADVECT, P_BBOX, P_GRID, P_KEYS, P_CELL_SCAN, P_SCATTER, P_SWEEP, P_SWEEP_LONG, P_ROUNDS, P_CENSUS,
  P_BOOKKEEPING, P_COUNT, P_NUM
};
const char* const kProfNames[P_NUM] = {"k_advect", "k_bbox",   "k_grid",       "k_keys",   "k_cscan",
                                       "k_scatter", "k_sweep", "k_sweep_long", "k_rounds", "k_census",
                                       "k_step_begin_end", "k_count_pairs"};
}  // namespace

struct lm_ctx {
  int device = 0;
  int sms = 0;
  cudaStream_t own = nullptr;
  cudaStream_t st = nullptr;
  std::string err;

  // field
  float2* uv = nullptr;
  size_t uv_n = 0;
  float* stage_uv = nullptr;  // field upload staging: u and v chunks before interleaving
  size_t field_elems = 0;  // nt * ny * nx
  int n_fields = 0;
  FieldView fv{};
  bool has_field = false;
  double lon0 = 0, lat0 = 0, lon1 = 0, lat1 = 0, t_first = 0, t_last = 0, org_lon = 0, org_lat = 0;

  // ensembles and slots
  uint32_t n_ens = 0;
  std::vector<uint32_t> counts, base;
  uint32_t nslots = 0, ntotal = 0;
  std::vector<int32_t> hmap;  // slot -> caller index (or -1)
  std::vector<EnsInfo> ens_h;
  EnsInfo* ens_d = nullptr;
  uint32_t* block_ens = nullptr;
  int32_t* map_d = nullptr;
  bool has_particles = false;  // positions + species (fused path)
  bool has_species = false;    // species only (two-phase interaction path)

  // per-slot buffers
  uint32_t slot_cap = 0;
  float *xo = nullptr, *yo = nullptr, *plon = nullptr, *plat = nullptr;
  int8_t* species = nullptr;
  uint8_t* status = nullptr;
  uint32_t *key = nullptr, *rank = nullptr, *sid = nullptr, *skey = nullptr, *sens = nullptr, *deg = nullptr;
  uint32_t *slab = nullptr, *longv = nullptr, *level = nullptr;
  unsigned long long* wstate = nullptr;
  uint32_t* act = nullptr;
  float2* spos = nullptr;
  uint32_t ens_cap = 0;
  EnsGrid* grids = nullptr;
  uint32_t* eord = nullptr;
  uint32_t* ebox = nullptr;
  uint32_t* census = nullptr;

  // cells
  uint32_t cells_cap = 0;
  uint32_t *ccount = nullptr, *cstart = nullptr, *csum = nullptr;

  // long lists
  size_t ovf_cap = 0;
  uint32_t* ovf = nullptr;
  unsigned long long* oprio = nullptr;
  int64_t regrows = 0;

  // interaction parameters
  bool has_params = false;
  PairParams pp{};
  double cell_factor = 1.004;
  std::vector<double> p_rs, p_pr, p_sp;
  std::vector<uint64_t> seeds;

  // control block
  Ctrl* ctrl = nullptr;
  Ctrl* hctrl = nullptr;
  unsigned long long inject_wait_ns = 0;  // lm_debug_inject_wait: the next plain interaction step
  uint32_t* hstage = nullptr;
  size_t hstage_n = 0;

  // device snapshot of the state (lm_snapshot_save / lm_snapshot_restore)
  float *snap_xo = nullptr, *snap_yo = nullptr;
  int8_t* snap_sp = nullptr;
  uint8_t* snap_st = nullptr;
  uint32_t snap_slots = 0;
  int64_t snap_step = -1;

  // pair log
  uint32_t* plog = nullptr;
  uint32_t plog_cap = 0;

  // step records of lm_step (rec_lon / rec_lat / rec_species): every step's record is packed into
  // one slot of a device ring (caller order), and copied to the caller's arrays on the copy stream
  // rec_st REC_SLOTS - 1 steps later, so the copies of step k overlap the kernels of the next steps
  // instead of holding up the compute stream.
  static constexpr int REC_SLOTS = 3;
  cudaStream_t rec_st = nullptr;
  unsigned char* rec_ring = nullptr;
  size_t rec_slot = 0;  // bytes per slot: lon [n] float, lat [n] float, species [n] int8
  cudaEvent_t rec_done[REC_SLOTS] = {}, rec_copied[REC_SLOTS] = {};
  std::vector<int64_t> rec_pending;  // steps whose records wait in the ring, oldest first
  float *rec_lon = nullptr, *rec_lat = nullptr;
  int8_t* rec_sp = nullptr;

  int rgrid = 0, rblock = 0;
  // tuning knobs (lm_set_tuning): block sizes and grid shapes that change speed, never results
  int tune_rounds_threads = 1024;  // interaction blocks: 1,024 threads x 2 vertices or 512 x 4
  int tune_long_per_sm = 6;        // long-list blocks per SM
  int tune_advect_threads = 256;   // advection threads per block (128 or 256)

  // graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  double g_t_start = 0, g_dt = 0, g_kh = 0;
  int64_t g_step0 = 0;
  int g_spg = 0;
  uint32_t g_flags = 0;
  int64_t next_step = 0;

  // per-kernel CUDA-event timing of plain launches
  bool prof_on = false;
  bool capturing = false;
  std::vector<cudaEvent_t> ev_pool;
  struct Pend {
    int id;
    cudaEvent_t a, b;
  };
  std::vector<Pend> pend;
  double prof_ms[P_NUM] = {};
  int64_t prof_n[P_NUM] = {};
};

namespace {

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

#define PROF(c, id, stmt)            \
  do {                               \
    cudaEvent_t pa_ = prof_begin(c); \
    stmt;                            \
    prof_end(c, id, pa_);            \
  } while (0)

// Forget the captured graph: its kernels hold the buffers' addresses and the field geometry by
// value, so it is stale once a buffer is reallocated or a field is uploaded (capture again).
void drop_graph(lm_ctx* c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->gexec = nullptr;
  c->graph = nullptr;
}

template <class T>
int dalloc(lm_ctx* c, T** p, size_t count) {
  if (*p) {
    drop_graph(c);  // a captured graph holds the old address
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

uint32_t next_pow2(uint64_t x) {
  uint64_t p = 1;
  while (p < x) p <<= 1;
  return (uint32_t)std::min<uint64_t>(p, 1ull << 31);
}

int set_cells_capacity(lm_ctx* c, uint32_t cap) {
  int r;
  if ((r = dalloc(c, &c->ccount, (size_t)cap + 1)) || (r = dalloc(c, &c->cstart, (size_t)cap + 1))) return r;
  CK(cudaMemsetAsync(c->ccount, 0, ((size_t)cap + 1) * sizeof(uint32_t), c->st));
  CK(cudaStreamSynchronize(c->st));
  c->cells_cap = cap;
  return LM_OK;
}

int set_ovf_capacity(lm_ctx* c, size_t cap) {
  int r;
  cap = std::min<size_t>(cap, 0xfffffff0ull);
  if ((r = dalloc(c, &c->ovf, cap)) || (r = dalloc(c, &c->oprio, cap))) return r;
  c->ovf_cap = cap;
  unsigned long long cv = cap;
  CK(cudaMemcpyAsync(&c->ctrl->ovf_cap, &cv, sizeof(cv), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return LM_OK;
}

// Per-slot and per-ensemble buffers for `slots` slots and `n_ens` ensembles.
int ensure_slots(lm_ctx* c, uint32_t slots, uint32_t n_ens) {
  int r;
  if (slots > c->slot_cap || !c->xo) {
    const uint32_t cap = std::max<uint32_t>(slots, 1024);
    const size_t nblk = (cap + SLOT_BLOCK - 1) / SLOT_BLOCK + 1;
    if ((r = dalloc(c, &c->xo, cap)) || (r = dalloc(c, &c->yo, cap)) || (r = dalloc(c, &c->plon, cap)) ||
        (r = dalloc(c, &c->plat, cap)) || (r = dalloc(c, &c->species, cap)) || (r = dalloc(c, &c->status, cap)) ||
        (r = dalloc(c, &c->key, cap)) || (r = dalloc(c, &c->rank, cap)) || (r = dalloc(c, &c->sid, cap)) ||
        (r = dalloc(c, &c->skey, cap)) || (r = dalloc(c, &c->sens, cap)) || (r = dalloc(c, &c->deg, cap)) ||
        (r = dalloc(c, &c->slab, (size_t)cap * SLAB)) ||
        (r = dalloc(c, &c->longv, cap)) || (r = dalloc(c, &c->wstate, cap)) ||
        (r = dalloc(c, &c->level, cap)) || (r = dalloc(c, &c->act, cap)) || (r = dalloc(c, &c->spos, cap)) ||
        (r = dalloc(c, &c->map_d, cap)) || (r = dalloc(c, &c->block_ens, nblk)))
      return r;
    c->slot_cap = cap;
    if ((r = set_cells_capacity(c, std::max<uint32_t>(1u << 20, next_pow2((uint64_t)4 * cap)))) ||
        (r = set_ovf_capacity(c, std::max<size_t>((size_t)2 * cap, (size_t)1 << 16))))
      return r;
    if (!c->csum && (r = dalloc(c, &c->csum, SCAN_BLOCKS))) return r;
  }
  if (n_ens > c->ens_cap || !c->ens_d) {
    const uint32_t cap = std::max<uint32_t>(n_ens, 1);
    if ((r = dalloc(c, &c->ens_d, cap)) || (r = dalloc(c, &c->grids, cap)) || (r = dalloc(c, &c->eord, cap)) ||
        (r = dalloc(c, &c->ebox, (size_t)4 * cap)) ||
        (r = dalloc(c, &c->census, (size_t)4 * cap)))
      return r;
    CK(cudaMemsetAsync(c->census, 0, sizeof(uint32_t) * 4 * cap, c->st));
    c->ens_cap = cap;
  }
  if ((uint64_t)16 * n_ens > c->cells_cap && (r = set_cells_capacity(c, next_pow2((uint64_t)16 * n_ens)))) return r;
  return LM_OK;
}

// Ensemble layout: counts -> slot bases (padded to SLOT_BLOCK when n_ens > 1), maps, block table.
int layout(lm_ctx* c, uint32_t n_ens, const int64_t* counts) {
  std::vector<uint32_t> cnt(n_ens), base(n_ens);
  uint64_t slot = 0, total = 0;
  for (uint32_t e = 0; e < n_ens; ++e) {
    if (counts[e] < 0) return fail(c, LM_ERR_ARG, "negative count for ensemble %u", e);
    cnt[e] = (uint32_t)counts[e];
    if (n_ens > 1) slot = (slot + SLOT_BLOCK - 1) / SLOT_BLOCK * SLOT_BLOCK;
    base[e] = (uint32_t)slot;
    slot += cnt[e];
    total += cnt[e];
    if (slot > MAX_SLOTS)
      return fail(c, LM_ERR_ARG, "too many particles: a context holds at most %llu slots",
                  (unsigned long long)MAX_SLOTS);
  }
  int r;
  if ((r = ensure_slots(c, (uint32_t)slot, n_ens))) return r;
  c->n_ens = n_ens;
  c->counts = cnt;
  c->base = base;
  c->nslots = (uint32_t)slot;
  c->ntotal = (uint32_t)total;
  c->hmap.assign(slot, -1);
  std::vector<uint32_t> bens((slot + SLOT_BLOCK - 1) / SLOT_BLOCK + 1, 0);
  uint64_t idx = 0;
  for (uint32_t e = 0; e < n_ens; ++e) {
    for (uint32_t k = 0; k < cnt[e]; ++k) c->hmap[base[e] + k] = (int32_t)(idx + k);
    idx += cnt[e];
    if (cnt[e]) {
      const uint32_t b0 = base[e] / SLOT_BLOCK, b1 = (base[e] + cnt[e] - 1) / SLOT_BLOCK;
      for (uint32_t b = b0; b <= b1; ++b) bens[b] = e;
    }
  }
  if (slot) CK(cudaMemcpyAsync(c->map_d, c->hmap.data(), slot * sizeof(int32_t), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->block_ens, bens.data(), bens.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
  // key ranges in index order until the first k_grid (which may reorder them; one ensemble never is)
  std::vector<uint32_t> eord(n_ens);
  for (uint32_t e = 0; e < n_ens; ++e) eord[e] = e;
  CK(cudaMemcpyAsync(c->eord, eord.data(), n_ens * sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return LM_OK;
}

unsigned long long prob_threshold(double p) {
  if (!(p > 0)) return 0ull;  // also NaN: r < NaN is false
  if (p >= 1.0) return 1ull << 53;
  return (unsigned long long)std::ceil(std::ldexp(p, 53));
}

// Per-ensemble constants to the device (parameters default to the last lm_set_interaction).
int upload_ens(lm_ctx* c) {
  c->ens_h.assign(c->n_ens, EnsInfo{});
  for (uint32_t e = 0; e < c->n_ens; ++e) {
    EnsInfo& x = c->ens_h[e];
    const size_t k = e < c->p_rs.size() ? e : 0;
    x.t_rs = c->p_rs.empty() ? 0 : prob_threshold(c->p_rs[k]);
    x.t_pr = c->p_pr.empty() ? 0 : prob_threshold(c->p_pr[k]);
    x.t_sp = c->p_sp.empty() ? 0 : prob_threshold(c->p_sp[k]);
    const uint64_t seed = c->seeds.empty() ? 0 : c->seeds[e < c->seeds.size() ? e : 0];
    x.seed_lo = (uint32_t)seed;
    x.seed_hi = (uint32_t)(seed >> 32);
    x.base = c->base[e];
    x.n = c->counts[e];
    x.field_off = (c->n_fields > 1) ? (unsigned long long)e * c->field_elems : 0ull;
  }
  if (c->n_ens) CK(cudaMemcpyAsync(c->ens_d, c->ens_h.data(), c->n_ens * sizeof(EnsInfo), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return LM_OK;
}

Bufs bufs(const lm_ctx* c, bool log) {
  Bufs b;
  b.ens = c->ens_d;
  b.block_ens = c->block_ens;
  b.n_ens = c->n_ens;
  b.nslots = c->nslots;
  b.cells_cap = c->cells_cap;
  b.xo = c->xo;
  b.yo = c->yo;
  b.species = c->species;
  b.status = c->status;
  b.plon = c->plon;
  b.plat = c->plat;
  b.ebox = c->ebox;
  b.grids = c->grids;
  b.eord = c->eord;
  b.key = c->key;
  b.rank = c->rank;
  b.ccount = c->ccount;
  b.cstart = c->cstart;
  b.csum = c->csum;
  b.sid = c->sid;
  b.skey = c->skey;
  b.sens = c->sens;
  b.spos = c->spos;
  b.deg = c->deg;
  b.slab = c->slab;
  b.ovf = c->ovf;
  b.oprio = c->oprio;
  b.longv = c->longv;
  b.wstate = c->wstate;
  b.level = c->level;
  b.act = c->act;
  b.census = c->census;
  b.plog = log ? c->plog : nullptr;
  b.plog_cap = c->plog_cap;
  return b;
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

int write_err(lm_ctx* c, uint32_t err, uint32_t halt) {
  c->hctrl->err = err;
  c->hctrl->halt = halt;
  CK(cudaMemcpyAsync(&c->ctrl->err, &c->hctrl->err, sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(&c->ctrl->halt, &c->hctrl->halt, sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return LM_OK;
}

int clear_err_bits(lm_ctx* c, uint32_t mask) { return write_err(c, c->hctrl->err & ~mask, c->hctrl->halt); }

// Map and clear the sticky device error bits.
int consume_errors(lm_ctx* c) {
  const uint32_t e = c->hctrl->err;
  if (!e) return LM_OK;
  int r;
  if ((r = write_err(c, 0u, c->hctrl->halt))) return r;
  if (e & ERRB_TIMEOUT) return fail(c, LM_ERR_TIMEOUT, "a bounded device wait timed out");
  if (e & ERRB_TIME) return fail(c, LM_ERR_TIME, "a stage time fell outside the field's time axis");
  if (e & ERRB_NAN) return fail(c, LM_ERR_NAN, "non-finite particle positions (%u flagged in total)", c->hctrl->oob);
  if (e & ERRB_OOB)
    return fail(c, LM_ERR_OUT_OF_BOUNDS, "particles left the field domain (%u flagged in total)", c->hctrl->oob);
  if (e & ERRB_OVERFLOW) return fail(c, LM_ERR_CAPACITY, "neighbour-list capacity exceeded");
  return LM_OK;
}

// Regrow after a halted step: long-list area and/or cell capacity, then clear the halt.
int regrow(lm_ctx* c) {
  int r;
  const Ctrl& h = *c->hctrl;
  if (h.err & ERRB_ROUNDCAP) {
    write_err(c, 0u, 0u);
    return fail(c, LM_ERR_ROUND_CAP, "a microbe has more than %u neighbours", MAX_DEGREE);
  }
  if (h.ovf_used > c->ovf_cap) {
    size_t need = (size_t)h.ovf_used;
    if ((r = set_ovf_capacity(c, std::max(need + need / 4 + 4096, c->ovf_cap * 2)))) return r;
  }
  if (h.ncells >= c->cells_cap && h.halt) {
    if ((r = set_cells_capacity(c, (uint32_t)std::min<uint64_t>((uint64_t)c->cells_cap * 2, 1ull << 31)))) return r;
  }
  c->regrows++;
  return write_err(c, h.err & ~(uint32_t)ERRB_OVERFLOW, 0u);
}

StepArgs step_args(double t, double dt, int64_t step, double kh, bool graph) {
  StepArgs a;
  a.t_start = t;
  a.dt = dt;
  a.step0 = (uint32_t)step;
  a.use_ctrl_step = graph ? 1 : 0;
  a.kick = kh > 0 ? (float)std::sqrt(6.0 * std::fabs(dt) * kh) : 0.f;
  a.test_wait_ns = 0;
  return a;
}

// bin -> pair -> (interact). `positions_only`: the boxes come from plon/plat (no advection ran).
cudaError_t enqueue_interaction(lm_ctx* c, const StepArgs& a, uint32_t flags, bool positions_only, bool use_status) {
  cudaStream_t st = c->st;
  const Bufs b = bufs(c, (flags & LM_STEP_LOG_PAIRS) != 0);
  if (positions_only) PROF(c, P_BBOX, launch_bbox(b, c->ctrl, use_status, st));
  const bool own_grid = c->n_ens == 1;  // one ensemble: k_keys derives the grid itself
  if (!own_grid) PROF(c, P_GRID, launch_grid(b, c->pp, c->ctrl, st));
  PROF(c, P_KEYS, launch_keys(b, c->pp, c->ctrl, use_status, own_grid, st));
  PROF(c, P_CELL_SCAN, launch_cell_scan(b, c->ctrl, st));
  PROF(c, P_SCATTER, launch_scatter(b, c->ctrl, st));
  if (flags & LM_STEP_COUNT_PAIRS) {  // count-only: no lists, no interaction
    PROF(c, P_COUNT, launch_count_pairs(b, c->pp, c->ctrl, st));
    return cudaGetLastError();
  }
  PROF(c, P_SWEEP, launch_sweep(b, c->pp, a, c->ctrl, st));
  PROF(c, P_SWEEP_LONG, launch_sweep_long(b, c->pp, a, c->ctrl, c->sms, c->tune_long_per_sm, st));
  if (flags & LM_STEP_INTERACT) {
    cudaEvent_t pa = prof_begin(c);
    cudaError_t e = launch_rounds(b, a, c->ctrl, c->rgrid, c->rblock, st);
    prof_end(c, P_ROUNDS, pa);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

// One fused step; `advect` false re-runs only the interaction part of an advected step. `begun`:
// the previous step's end already started this one; `next` (the next step of the same call, which
// advects): this step's end also starts that one.
cudaError_t enqueue_step(lm_ctx* c, const StepArgs& a, uint32_t flags, bool advect, bool begun = false,
                         const StepArgs* next = nullptr) {
  const Bufs b = bufs(c, false);
  if (!begun) PROF(c, P_BOOKKEEPING, launch_step_begin(b, advect ? &c->fv : nullptr, a, c->ctrl, c->st));
  if (advect) PROF(c, P_ADVECT, launch_advect(c->fv, a, b, c->ctrl, c->tune_advect_threads, c->st));
  if (flags & (LM_STEP_INTERACT | LM_STEP_COUNT_PAIRS)) {
    cudaError_t e = enqueue_interaction(c, a, flags, !advect, true);
    if (e != cudaSuccess) return e;
  }
  if (flags & LM_STEP_CENSUS) PROF(c, P_CENSUS, launch_census(b, c->ctrl, c->st));
  const bool counted = (flags & (LM_STEP_INTERACT | LM_STEP_COUNT_PAIRS)) != 0;
  if (next)
    PROF(c, P_BOOKKEEPING, launch_step_turn(b, &c->fv, *next, c->ctrl, counted, c->st));
  else
    PROF(c, P_BOOKKEEPING, launch_step_end(c->ctrl, counted, c->st));
  return cudaGetLastError();
}

int ensure_hstage(lm_ctx* c, size_t n) {
  if (c->hstage_n >= n) return LM_OK;
  if (c->hstage) cudaFreeHost(c->hstage);
  c->hstage = nullptr;
  CK(cudaMallocHost((void**)&c->hstage, n * sizeof(uint32_t)));
  c->hstage_n = n;
  return LM_OK;
}

int check_time(lm_ctx* c, double t, double dt, int64_t n_steps) {
  const double lo = std::min(t, t + dt * n_steps), hi = std::max(t, t + dt * n_steps);
  const double tol = 1e-9 * std::fabs(c->fv.dT);
  if (lo < c->t_first - tol || hi > c->t_last + tol)
    return fail(c, LM_ERR_TIME, "time window [%.9g, %.9g] s is outside the field's [%.9g, %.9g] s", lo, hi,
                c->t_first, c->t_last);
  return LM_OK;
}

void set_pair_params(lm_ctx* c, double r, int norm) { c->pp = make_pair_params(r, norm, (float)c->cell_factor); }

// The record ring: slots sized for the current particle count, the copy stream and the events.
int ensure_rec_ring(lm_ctx* c) {
  const size_t n = c->ntotal;
  const size_t slot = (9 * n + 255) / 256 * 256;
  if (!c->rec_st) {
    CK(cudaStreamCreateWithFlags(&c->rec_st, cudaStreamNonBlocking));
    for (int q = 0; q < lm_ctx::REC_SLOTS; ++q) {
      CK(cudaEventCreateWithFlags(&c->rec_done[q], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&c->rec_copied[q], cudaEventDisableTiming));
    }
  }
  if (slot > c->rec_slot) {
    if (c->rec_ring) {
      CK(cudaStreamSynchronize(c->rec_st));
      cudaFree(c->rec_ring);
      c->rec_ring = nullptr;
      c->rec_slot = 0;
    }
    const cudaError_t e = cudaMalloc(&c->rec_ring, slot * lm_ctx::REC_SLOTS);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(c, LM_ERR_OOM, "cudaMalloc of the %zu-byte record ring failed: %s", slot * lm_ctx::REC_SLOTS,
                  cudaGetErrorString(e));
    }
    c->rec_slot = slot;
  }
  return LM_OK;
}

// Copy the oldest pending record from its ring slot to the caller's arrays (copy stream, after the
// step that packed it). Copies into pageable memory return once they are done; the compute stream
// keeps running the steps queued behind that record meanwhile.
int flush_record(lm_ctx* c) {
  const int64_t k = c->rec_pending.front();
  c->rec_pending.erase(c->rec_pending.begin());
  const int q = (int)(k % lm_ctx::REC_SLOTS);
  const size_t n = c->ntotal;
  unsigned char* slot = c->rec_ring + (size_t)q * c->rec_slot;
  CK(cudaStreamWaitEvent(c->rec_st, c->rec_done[q], 0));
  if (c->rec_lon) CK(cudaMemcpyAsync(c->rec_lon + k * n, slot, n * 4, cudaMemcpyDeviceToHost, c->rec_st));
  if (c->rec_lat) CK(cudaMemcpyAsync(c->rec_lat + k * n, slot + n * 4, n * 4, cudaMemcpyDeviceToHost, c->rec_st));
  if (c->rec_sp) CK(cudaMemcpyAsync(c->rec_sp + k * n, slot + n * 8, n, cudaMemcpyDeviceToHost, c->rec_st));
  CK(cudaEventRecord(c->rec_copied[q], c->rec_st));
  return LM_OK;
}

// Every pending record in the caller's arrays.
int flush_records(lm_ctx* c) {
  int r;
  while (!c->rec_pending.empty())
    if ((r = flush_record(c))) return r;
  if (c->rec_st) CK(cudaStreamSynchronize(c->rec_st));
  return LM_OK;
}

// One step's record (positions before the kick, species after the step) into a ring slot in
// caller order; its copy to the host follows REC_SLOTS - 1 steps later (flush_record).
int record_step(lm_ctx* c, int64_t k) {
  const uint32_t n = c->ntotal;
  if (!n || !(c->rec_lon || c->rec_lat || c->rec_sp)) return LM_OK;
  const int q = (int)(k % lm_ctx::REC_SLOTS);
  unsigned char* slot = c->rec_ring + (size_t)q * c->rec_slot;
  float* lon = reinterpret_cast<float*>(slot);
  float* lat = reinterpret_cast<float*>(slot + (size_t)n * 4);
  int8_t* sp = reinterpret_cast<int8_t*>(slot + (size_t)n * 8);
  CK(cudaStreamWaitEvent(c->st, c->rec_copied[q], 0));  // the slot's previous copy has read it
  const bool direct = (c->n_ens == 1);
  if (c->rec_lon) {
    if (direct) CK(cudaMemcpyAsync(lon, c->plon, n * 4, cudaMemcpyDeviceToDevice, c->st));
    else launch_unpad(c->plon, lon, c->map_d, c->nslots, c->st);
  }
  if (c->rec_lat) {
    if (direct) CK(cudaMemcpyAsync(lat, c->plat, n * 4, cudaMemcpyDeviceToDevice, c->st));
    else launch_unpad(c->plat, lat, c->map_d, c->nslots, c->st);
  }
  if (c->rec_sp) {
    if (direct) CK(cudaMemcpyAsync(sp, c->species, n, cudaMemcpyDeviceToDevice, c->st));
    else launch_unpad8(c->species, sp, c->map_d, c->nslots, c->st);
  }
  CK(cudaEventRecord(c->rec_done[q], c->st));
  c->rec_pending.push_back(k);
  int r;
  while ((int)c->rec_pending.size() >= lm_ctx::REC_SLOTS)
    if ((r = flush_record(c))) return r;
  return LM_OK;
}

int run_steps(lm_ctx* c, double t, double dt, int64_t n_steps, int64_t step0, uint32_t flags, double kh,
              float* rec_lon, float* rec_lat, int8_t* rec_species, int64_t* rec_census) {
  int r;
  if ((r = write_ctrl_step(c, step0))) return r;
  if (rec_census && (r = ensure_hstage(c, (size_t)4 * n_steps))) return r;
  c->rec_lon = rec_lon;
  c->rec_lat = rec_lat;
  c->rec_sp = rec_species;
  if ((rec_lon || rec_lat || rec_species) && (r = ensure_rec_ring(c))) return r;
  int64_t s = 0;
  bool redo = false;
  while (s < n_steps) {
    bool chained = false;  // the previous step's end started step k
    for (int64_t k = s; k < n_steps; ++k) {
      StepArgs a = step_args(t + dt * k, dt, step0 + k, kh, false);
      if (c->inject_wait_ns && (flags & LM_STEP_INTERACT)) {  // armed by lm_debug_inject_wait: this step only
        a.test_wait_ns = c->inject_wait_ns;
        c->inject_wait_ns = 0;
      }
      // the last step keeps its counters for lm_stats; a per-step census read keeps them per step
      const bool chain = k + 1 < n_steps && !rec_census;
      const StepArgs an = step_args(t + dt * (k + 1), dt, step0 + k + 1, kh, false);
      CK(enqueue_step(c, a, flags, !(redo && k == s), chained, chain ? &an : nullptr));
      chained = chain;
      if ((r = record_step(c, k))) return r;
      if (rec_census)
        CK(cudaMemcpyAsync(c->hstage + 4 * k, c->ctrl->census, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
    }
    CK(cudaGetLastError());
    if ((r = flush_records(c))) return r;  // (a halted step's record is written again by its redo)
    if ((r = read_ctrl(c))) return r;
    if (c->hctrl->halt) {
      const int64_t k = (int64_t)c->hctrl->halt_step - step0;
      if ((r = regrow(c))) return r;
      if ((r = write_ctrl_step(c, step0 + k))) return r;
      s = k;
      redo = true;  // the halted step was advected already
      continue;
    }
    break;
  }
  c->next_step = step0 + n_steps;
  if (rec_census)
    for (int64_t k = 0; k < 4 * n_steps; ++k) rec_census[k] = c->hstage[k];
  return consume_errors(c);
}

// Positions supplied by the caller (float32, E = 1): the two-phase interaction path.
int stage_positions(lm_ctx* c, int64_t n, const float* lon, const float* lat) {
  if (c->n_ens != 1 || c->ntotal != (uint32_t)n) {
    const int64_t cnt = n;
    int r = layout(c, 1, &cnt);
    if (r) return r;
    if ((r = upload_ens(c))) return r;
  }
  if (n) {
    CK(cudaMemcpyAsync(c->plon, lon, n * sizeof(float), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->plat, lat, n * sizeof(float), cudaMemcpyHostToDevice, c->st));
  }
  return LM_OK;
}

int capture(lm_ctx* c) {
  drop_graph(c);
  CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
  c->capturing = true;
  for (int k = 0; k < c->g_spg; ++k) {
    const StepArgs a = step_args(c->g_t_start, c->g_dt, c->g_step0, c->g_kh, true);  // step from the device counter
    const cudaError_t le = enqueue_step(c, a, c->g_flags, true, k > 0, k + 1 < c->g_spg ? &a : nullptr);
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
  const cudaError_t e = cudaStreamEndCapture(c->st, &g);
  c->capturing = false;
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, LM_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
  }
  c->graph = g;
  CK(cudaGraphInstantiate(&c->gexec, c->graph, 0));
  return LM_OK;
}

int check_ready(lm_ctx* c, uint32_t flags) {
  if (!(flags & LM_STEP_ADVECT)) return fail(c, LM_ERR_ARG, "steps need LM_STEP_ADVECT (use lm_interact)");
  if (!c->has_field || !c->has_particles) return fail(c, LM_ERR_STATE, "field and particles must be uploaded first");
  if ((flags & (LM_STEP_INTERACT | LM_STEP_COUNT_PAIRS)) && !c->has_params)
    return fail(c, LM_ERR_STATE, "call lm_set_interaction first");
  if ((flags & LM_STEP_INTERACT) && (flags & LM_STEP_COUNT_PAIRS))
    return fail(c, LM_ERR_ARG, "LM_STEP_COUNT_PAIRS replaces the interaction: pass one of the two");
  if (c->n_fields != 1 && c->n_fields != (int)c->n_ens)
    return fail(c, LM_ERR_STATE, "%d fields for %u ensembles (need 1 or one per ensemble)", c->n_fields, c->n_ens);
  return LM_OK;
}

}  // namespace

extern "C" {

int lm_version(void) { return LM_API_VERSION; }

int lm_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) {
    set_thread_error("NULL argument");
    return LM_ERR_ARG;
  }
  *ptr = nullptr;
  const cudaError_t e = cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocPortable);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    cudaGetLastError();
    set_thread_error(cudaGetErrorString(e));
    return LM_ERR_OOM;
  }
  return LM_OK;
}

int lm_host_free(void* ptr) {
  if (!ptr) return LM_OK;
  const cudaError_t e = cudaFreeHost(ptr);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_thread_error(cudaGetErrorString(e));
    return LM_ERR_CUDA;
  }
  return LM_OK;
}

int lm_kernel_arch(int* sm) {
  if (!sm) {
    set_thread_error("NULL argument");
    return LM_ERR_ARG;
  }
  cudaFuncAttributes fa;
  const cudaError_t e = cudaFuncGetAttributes(&fa, (const void*)lm_census_kernel());
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_thread_error(cudaGetErrorString(e));
    return LM_ERR_CUDA;
  }
  *sm = fa.binaryVersion;
  return LM_OK;
}

int lm_ctx_create(int device, lm_ctx** out) {
  if (!out) return fail(nullptr, LM_ERR_ARG, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(nullptr, LM_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  if (device < 0 || device >= ndev) return fail(nullptr, LM_ERR_ARG, "device %d out of range [0, %d)", device, ndev);
  lm_ctx* c = new lm_ctx();
  c->device = device;
  auto bail = [&](int code) {
    g_create_error = c->err;
    lm_ctx_destroy(c);
    return code;
  };
  if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(fail(c, LM_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e)));
  if ((e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(fail(c, LM_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)));
  c->st = c->own;
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  int r = dalloc(c, &c->ctrl, 1);
  if (r) return bail(r);
  if ((e = cudaMallocHost((void**)&c->hctrl, sizeof(Ctrl))) != cudaSuccess)
    return bail(fail(c, LM_ERR_CUDA, "cudaMallocHost: %s", cudaGetErrorString(e)));
  memset(c->hctrl, 0, sizeof(Ctrl));
  if ((e = cudaMemsetAsync(c->ctrl, 0, sizeof(Ctrl), c->st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->st)) != cudaSuccess)
    return bail(fail(c, LM_ERR_CUDA, "ctrl init: %s", cudaGetErrorString(e)));
  c->rgrid = rounds_grid(device, c->tune_rounds_threads, &c->rblock);
  set_pair_params(c, 0.0, LM_NORM_L2);
  *out = c;
  return LM_OK;
}

int lm_ctx_destroy(lm_ctx* c) {
  if (!c) return LM_OK;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  void* bufs_[] = {c->uv,     c->xo,    c->yo,     c->plon,   c->plat,   c->species, c->status, c->key,
                   c->rank,   c->sid,   c->skey,   c->sens,   c->deg,    c->slab,    c->longv,
                   c->wstate, c->level,  c->act,    c->spos,
                   c->map_d,  c->block_ens, c->ens_d, c->grids, c->eord, c->ebox, c->census,  c->ccount, c->cstart,
                   c->csum,   c->ovf,   c->oprio,  c->ctrl,   c->plog,  c->snap_xo, c->snap_yo, c->snap_sp,
                   c->snap_st};
  for (void* p : bufs_)
    if (p) cudaFree(p);
  if (c->hctrl) cudaFreeHost(c->hctrl);
  if (c->hstage) cudaFreeHost(c->hstage);
  if (c->rec_st) {
    cudaStreamSynchronize(c->rec_st);
    cudaStreamDestroy(c->rec_st);
  }
  if (c->rec_ring) cudaFree(c->rec_ring);
  if (c->stage_uv) cudaFree(c->stage_uv);
  for (int q = 0; q < lm_ctx::REC_SLOTS; ++q) {
    if (c->rec_done[q]) cudaEventDestroy(c->rec_done[q]);
    if (c->rec_copied[q]) cudaEventDestroy(c->rec_copied[q]);
  }
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

int lm_field_upload_batch(lm_ctx* c, int n_fields, const float* u, const float* v, int nt, int ny, int nx,
                          const double* lon, const double* lat, const double* t_sec) {
  if (!c || !u || !v || !lon || !lat || !t_sec) return fail(c, LM_ERR_ARG, "NULL argument");
  if (n_fields < 1) return fail(c, LM_ERR_ARG, "n_fields must be >= 1");
  if (nt < 2 || ny < 2 || nx < 2) return fail(c, LM_ERR_ARG, "field needs nt, ny, nx >= 2 (got %d, %d, %d)", nt, ny, nx);
  double dx, dy, dT;
  if (!uniform_axis(lon, nx, &dx)) return fail(c, LM_ERR_GRID, "longitude axis is not uniform and ascending");
  if (!uniform_axis(lat, ny, &dy)) return fail(c, LM_ERR_GRID, "latitude axis is not uniform and ascending");
  if (!uniform_axis(t_sec, nt, &dT)) return fail(c, LM_ERR_GRID, "time axis is not uniform and ascending");
  CK(cudaSetDevice(c->device));
  drop_graph(c);  // the graph's steps carry the old field geometry and time axis
  const size_t per = (size_t)nt * ny * nx;
  const size_t n = per * (size_t)n_fields;
  int r;
  if (n > c->uv_n || !c->uv) {
    if ((r = dalloc(c, &c->uv, n))) return r;
    c->uv_n = n;
  }
  // page-locked u and v (mapped into the device's address space): one kernel reads both over the
  // host link and writes the interleaved field, with no copies through a staging buffer
  cudaPointerAttributes pa_u, pa_v;
  const bool mapped = cudaPointerGetAttributes(&pa_u, u) == cudaSuccess &&
                      cudaPointerGetAttributes(&pa_v, v) == cudaSuccess && pa_u.type == cudaMemoryTypeHost &&
                      pa_v.type == cudaMemoryTypeHost && pa_u.devicePointer && pa_v.devicePointer;
  cudaGetLastError();  // an unregistered pointer is not an error here
  if (mapped) {
    launch_interleave(static_cast<const float*>(pa_u.devicePointer), static_cast<const float*>(pa_v.devicePointer),
                      c->uv, n, c->st);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
  }
  // otherwise stage u and v through the context's staging buffer (allocated once, 2 x 16M floats),
  // one chunk of values at a time: no field-sized temporary is allocated and freed per upload
  const size_t chunk = (size_t)16 << 20;
  if (!mapped && !c->stage_uv) {
    const cudaError_t e = cudaMalloc(&c->stage_uv, 2 * chunk * sizeof(float));
    if (e != cudaSuccess) {
      c->stage_uv = nullptr;
      cudaGetLastError();
      return fail(c, LM_ERR_OOM, "cudaMalloc of the field staging buffer failed: %s", cudaGetErrorString(e));
    }
  }
  for (size_t o = 0; !mapped && o < n; o += chunk) {
    const size_t m = std::min(chunk, n - o);
    CK(cudaMemcpyAsync(c->stage_uv, u + o, m * sizeof(float), cudaMemcpyDefault, c->st));
    CK(cudaMemcpyAsync(c->stage_uv + chunk, v + o, m * sizeof(float), cudaMemcpyDefault, c->st));
    launch_interleave(c->stage_uv, c->stage_uv + chunk, c->uv + o, m, c->st);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  c->n_fields = n_fields;
  c->field_elems = per;
  c->lon0 = lon[0];
  c->lat0 = lat[0];
  c->lon1 = lon[nx - 1];
  c->lat1 = lat[ny - 1];
  c->t_first = t_sec[0];
  c->t_last = t_sec[nt - 1];
  const double new_org_lon = (double)(float)lon[0], new_org_lat = (double)(float)lat[0];
  if (c->has_particles && (new_org_lon != c->org_lon || new_org_lat != c->org_lat)) {
    c->has_particles = false;  // offsets are relative to the field origin: positions must be re-uploaded
    c->has_species = false;
  }
  c->org_lon = new_org_lon;
  c->org_lat = new_org_lat;
  fill_field_view(c->fv, c->uv, nt, ny, nx, lon, lat, t_sec, dx, dy, dT);
  c->has_field = true;
  if (c->n_ens) return upload_ens(c);
  return LM_OK;
}

int lm_field_upload(lm_ctx* c, const float* u, const float* v, int nt, int ny, int nx, const double* lon,
                    const double* lat, const double* t_sec) {
  return lm_field_upload_batch(c, 1, u, v, nt, ny, nx, lon, lat, t_sec);
}

int lm_ensembles_upload(lm_ctx* c, int n_ens, const int64_t* counts, const double* lon, const double* lat,
                        const int8_t* species) {
  if (!c || n_ens < 1 || !counts) return fail(c, LM_ERR_ARG, "need n_ens >= 1 and counts");
  if (!c->has_field) return fail(c, LM_ERR_STATE, "upload the velocity field before the particles");
  int64_t total = 0;
  for (int e = 0; e < n_ens; ++e) total += counts[e];
  if (total > 0 && (!lon || !lat)) return fail(c, LM_ERR_ARG, "NULL positions");
  CK(cudaSetDevice(c->device));
  int r;
  if ((r = layout(c, (uint32_t)n_ens, counts))) return r;
  const uint32_t S = c->nslots;
  // page-locked caller arrays (mapped into the device's address space): one kernel converts them
  // into the slot layout; otherwise the conversion runs here and the slots are copied
  const void* dev_in[3] = {nullptr, nullptr, nullptr};
  const void* host_in[3] = {lon, lat, species};
  bool mapped = total > 0;
  for (int i = 0; i < 3 && mapped; ++i) {
    if (!host_in[i]) continue;
    cudaPointerAttributes pa;
    mapped = cudaPointerGetAttributes(&pa, host_in[i]) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
             pa.devicePointer;
    if (mapped) dev_in[i] = pa.devicePointer;
  }
  cudaGetLastError();  // an unregistered pointer is not an error here
  if (mapped) {
    launch_particles_in(static_cast<const double*>(dev_in[0]), static_cast<const double*>(dev_in[1]),
                        static_cast<const int8_t*>(dev_in[2]), c->map_d, S, c->org_lon, c->org_lat, c->xo, c->yo,
                        c->species, c->status, c->st);
    CK(cudaGetLastError());
  }
  std::vector<float> xo(mapped ? 0 : S, 0.f), yo(mapped ? 0 : S, 0.f);
  std::vector<int8_t> sp(mapped ? 0 : S, 0);
  std::vector<uint8_t> st(mapped ? 0 : S, STATUS_PAD);
  for (uint32_t k = 0; !mapped && k < S; ++k) {
    const int32_t q = c->hmap[k];
    if (q < 0) continue;
    xo[k] = (float)(lon[q] - c->org_lon);
    yo[k] = (float)(lat[q] - c->org_lat);
    sp[k] = species ? species[q] : 0;
    st[k] = STATUS_OK;
  }
  if (S && !mapped) {
    CK(cudaMemcpyAsync(c->xo, xo.data(), S * sizeof(float), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->yo, yo.data(), S * sizeof(float), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->species, sp.data(), S, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->status, st.data(), S, cudaMemcpyHostToDevice, c->st));
  }
  const uint32_t zero = 0;
  CK(cudaMemcpyAsync(&c->ctrl->oob, &zero, sizeof(zero), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  if ((r = upload_ens(c))) return r;
  c->has_particles = true;
  c->has_species = true;
  return LM_OK;
}

int lm_particles_upload(lm_ctx* c, int64_t n, const double* lon, const double* lat, const int8_t* species) {
  if (!c) return LM_ERR_ARG;
  if (n < 0 || n > 0x7fffff00) return fail(c, LM_ERR_ARG, "particle count %lld out of range", (long long)n);
  return lm_ensembles_upload(c, 1, &n, lon, lat, species);
}

int lm_species_upload(lm_ctx* c, int64_t n, const int8_t* species) {
  if (!c || (n > 0 && !species)) return fail(c, LM_ERR_ARG, "NULL argument");
  if (n < 0 || n > 0x7fffff00) return fail(c, LM_ERR_ARG, "species count out of range");
  CK(cudaSetDevice(c->device));
  int r;
  if (c->has_particles) {
    if (n != (int64_t)c->ntotal)
      return fail(c, LM_ERR_ARG, "n = %lld but the context holds %u particles", (long long)n, c->ntotal);
  } else if (c->n_ens != 1 || c->ntotal != (uint32_t)n) {
    if ((r = layout(c, 1, &n)) || (r = upload_ens(c))) return r;
  }
  std::vector<int8_t> sp(c->nslots, 0);
  for (uint32_t k = 0; k < c->nslots; ++k)
    if (c->hmap[k] >= 0) sp[k] = species[c->hmap[k]];
  if (c->nslots) CK(cudaMemcpyAsync(c->species, sp.data(), c->nslots, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->has_species = true;
  return LM_OK;
}

int lm_particles_download(lm_ctx* c, float* lon, float* lat, int8_t* species, uint8_t* status) {
  if (!c) return LM_ERR_ARG;
  if (!c->has_particles && (lon || lat || status || !c->has_species)) return fail(c, LM_ERR_STATE, "no particles");
  CK(cudaSetDevice(c->device));
  const uint32_t S = c->nslots;
  std::vector<float> xo(lon ? S : 0), yo(lat ? S : 0);
  std::vector<int8_t> sp(species ? S : 0);
  std::vector<uint8_t> st(status ? S : 0);
  if (S) {
    if (lon) CK(cudaMemcpyAsync(xo.data(), c->xo, S * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    if (lat) CK(cudaMemcpyAsync(yo.data(), c->yo, S * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    if (species) CK(cudaMemcpyAsync(sp.data(), c->species, S, cudaMemcpyDeviceToHost, c->st));
    if (status) CK(cudaMemcpyAsync(st.data(), c->status, S, cudaMemcpyDeviceToHost, c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  const float ox = (float)c->org_lon, oy = (float)c->org_lat;
  for (uint32_t k = 0; k < S; ++k) {
    const int32_t q = c->hmap[k];
    if (q < 0) continue;
    if (lon) lon[q] = ox + xo[k];  // same single rounding as the device
    if (lat) lat[q] = oy + yo[k];
    if (species) species[q] = sp[k];
    if (status) status[q] = st[k];
  }
  return LM_OK;
}

int lm_snapshot_save(lm_ctx* c) {
  if (!c) return LM_ERR_ARG;
  if (!c->has_particles) return fail(c, LM_ERR_STATE, "no particles");
  CK(cudaSetDevice(c->device));
  const uint32_t S = c->nslots;
  int r;
  if (S > c->snap_slots || !c->snap_xo) {
    if ((r = dalloc(c, &c->snap_xo, S)) || (r = dalloc(c, &c->snap_yo, S)) || (r = dalloc(c, &c->snap_sp, S)) ||
        (r = dalloc(c, &c->snap_st, S)))
      return r;
  }
  if (S) {
    CK(cudaMemcpyAsync(c->snap_xo, c->xo, S * sizeof(float), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->snap_yo, c->yo, S * sizeof(float), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->snap_sp, c->species, S, cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->snap_st, c->status, S, cudaMemcpyDeviceToDevice, c->st));
  }
  if ((r = read_ctrl(c))) return r;
  c->snap_slots = S;
  c->snap_step = c->hctrl->step;
  return LM_OK;
}

int lm_snapshot_restore(lm_ctx* c) {
  if (!c) return LM_ERR_ARG;
  if (c->snap_step < 0 || !c->has_particles || c->snap_slots != c->nslots)
    return fail(c, LM_ERR_STATE, "no snapshot of the current particle layout");
  CK(cudaSetDevice(c->device));
  const uint32_t S = c->nslots;
  if (S) {
    CK(cudaMemcpyAsync(c->xo, c->snap_xo, S * sizeof(float), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->yo, c->snap_yo, S * sizeof(float), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->species, c->snap_sp, S, cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->status, c->snap_st, S, cudaMemcpyDeviceToDevice, c->st));
  }
  return write_ctrl_step(c, c->snap_step);
}

int lm_state_export(lm_ctx* c, float* xo, float* yo, int8_t* species, uint8_t* status, int64_t* step) {
  if (!c || !xo || !yo || !species || !status || !step) return fail(c, LM_ERR_ARG, "NULL argument");
  if (!c->has_particles) return fail(c, LM_ERR_STATE, "no particles");
  CK(cudaSetDevice(c->device));
  const uint32_t S = c->nslots;
  std::vector<float> hx(S), hy(S);
  std::vector<int8_t> hs(S);
  std::vector<uint8_t> ht(S);
  if (S) {
    CK(cudaMemcpyAsync(hx.data(), c->xo, S * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(hy.data(), c->yo, S * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(hs.data(), c->species, S, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(ht.data(), c->status, S, cudaMemcpyDeviceToHost, c->st));
  }
  int r;
  if ((r = read_ctrl(c))) return r;
  for (uint32_t k = 0; k < S; ++k) {
    const int32_t q = c->hmap[k];
    if (q < 0) continue;
    xo[q] = hx[k];
    yo[q] = hy[k];
    species[q] = hs[k];
    status[q] = ht[k];
  }
  *step = c->hctrl->step;
  return LM_OK;
}

int lm_state_import(lm_ctx* c, const float* xo, const float* yo, const int8_t* species, const uint8_t* status,
                    int64_t step) {
  if (!c || !xo || !yo || !species || !status) return fail(c, LM_ERR_ARG, "NULL argument");
  if (!c->has_particles) return fail(c, LM_ERR_STATE, "upload particles (the layout) before importing a state");
  CK(cudaSetDevice(c->device));
  const uint32_t S = c->nslots;
  std::vector<float> hx(S, 0.f), hy(S, 0.f);
  std::vector<int8_t> hs(S, 0);
  std::vector<uint8_t> ht(S, STATUS_PAD);
  for (uint32_t k = 0; k < S; ++k) {
    const int32_t q = c->hmap[k];
    if (q < 0) continue;
    hx[k] = xo[q];
    hy[k] = yo[q];
    hs[k] = species[q];
    ht[k] = status[q] == STATUS_PAD ? STATUS_NAN : status[q];
  }
  if (S) {
    CK(cudaMemcpyAsync(c->xo, hx.data(), S * sizeof(float), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->yo, hy.data(), S * sizeof(float), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->species, hs.data(), S, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->status, ht.data(), S, cudaMemcpyHostToDevice, c->st));
  }
  return write_ctrl_step(c, step);
}

int lm_set_interaction(lm_ctx* c, double radius, int norm, double p_rs, double p_pr, double p_sp, uint64_t seed) {
  if (!c) return LM_ERR_ARG;
  if (!(radius >= 0) || !std::isfinite(radius)) return fail(c, LM_ERR_ARG, "radius must be finite and >= 0");
  if (norm != LM_NORM_INF && norm != LM_NORM_L1 && norm != LM_NORM_L2)
    return fail(c, LM_ERR_ARG, "norm must be 1, 2 or infinity (code 0); got %d", norm);
  CK(cudaSetDevice(c->device));
  set_pair_params(c, radius, norm);
  c->p_rs.assign(1, p_rs);
  c->p_pr.assign(1, p_pr);
  c->p_sp.assign(1, p_sp);
  c->seeds.assign(1, seed);
  c->has_params = true;
  if (c->n_ens) return upload_ens(c);
  return LM_OK;
}

int lm_set_ensemble_params(lm_ctx* c, int n_ens, const double* p_rs, const double* p_pr, const double* p_sp,
                           const uint64_t* seeds) {
  if (!c || !p_rs || !p_pr || !p_sp || !seeds) return fail(c, LM_ERR_ARG, "NULL argument");
  if (!c->has_params) return fail(c, LM_ERR_STATE, "call lm_set_interaction first (radius and norm)");
  if (n_ens != (int)c->n_ens) return fail(c, LM_ERR_ARG, "%d parameter sets for %u ensembles", n_ens, c->n_ens);
  CK(cudaSetDevice(c->device));
  c->p_rs.assign(p_rs, p_rs + n_ens);
  c->p_pr.assign(p_pr, p_pr + n_ens);
  c->p_sp.assign(p_sp, p_sp + n_ens);
  c->seeds.assign(seeds, seeds + n_ens);
  return upload_ens(c);
}

int lm_set_tuning(lm_ctx* c, int knob, int value) {
  if (!c) return LM_ERR_ARG;
  switch (knob) {
    case LM_TUNE_ROUNDS_THREADS:
      if (value != 512 && value != 1024) return fail(c, LM_ERR_ARG, "interaction block size must be 512 or 1024");
      c->tune_rounds_threads = value;
      CK(cudaSetDevice(c->device));
      c->rgrid = rounds_grid(c->device, value, &c->rblock);
      break;
    case LM_TUNE_LONG_BLOCKS_PER_SM:
      if (value < 1 || value > 32) return fail(c, LM_ERR_ARG, "long-list blocks per SM must be in [1, 32]");
      c->tune_long_per_sm = value;
      break;
    case LM_TUNE_ADVECT_THREADS:
      if (value != 128 && value != 256) return fail(c, LM_ERR_ARG, "advection block size must be 128 or 256");
      c->tune_advect_threads = value;
      break;
    default:
      return fail(c, LM_ERR_ARG, "unknown tuning knob %d", knob);
  }
  drop_graph(c);  // a captured graph keeps the launch shapes it was captured with
  return LM_OK;
}

int lm_get_tuning(lm_ctx* c, int knob, int* value) {
  if (!c || !value) return LM_ERR_ARG;
  switch (knob) {
    case LM_TUNE_ROUNDS_THREADS: *value = c->tune_rounds_threads; break;
    case LM_TUNE_LONG_BLOCKS_PER_SM: *value = c->tune_long_per_sm; break;
    case LM_TUNE_ADVECT_THREADS: *value = c->tune_advect_threads; break;
    default: return fail(c, LM_ERR_ARG, "unknown tuning knob %d", knob);
  }
  return LM_OK;
}

int lm_set_cell_factor(lm_ctx* c, double factor) {
  if (!c) return LM_ERR_ARG;
  if (!(factor >= 1.004) || !(factor <= 64.0)) return fail(c, LM_ERR_ARG, "cell factor must be in [1.004, 64]");
  c->cell_factor = factor;
  c->pp.cell_factor = (float)factor;
  return LM_OK;
}

int lm_step(lm_ctx* c, double t_sec, double dt_sec, int n_steps, int64_t step0, uint32_t flags, double kh_deg2_s,
            float* rec_lon, float* rec_lat, int8_t* rec_species, int64_t* rec_census) {
  if (!c) return LM_ERR_ARG;
  if (n_steps < 0) return fail(c, LM_ERR_ARG, "n_steps < 0");
  int r;
  if ((r = check_ready(c, flags))) return r;
  if (!(dt_sec != 0) || !std::isfinite(dt_sec)) return fail(c, LM_ERR_ARG, "dt must be finite and nonzero");
  if (!(kh_deg2_s >= 0)) return fail(c, LM_ERR_ARG, "Kh must be >= 0");
  CK(cudaSetDevice(c->device));
  if ((r = check_time(c, t_sec, dt_sec, n_steps))) return r;
  if (n_steps == 0) return LM_OK;
  if ((flags & LM_STEP_LOG_PAIRS) && c->plog_cap < (uint64_t)8 * c->nslots + 1024) {
    c->plog_cap = (uint32_t)std::min<uint64_t>((uint64_t)8 * c->nslots + 1024, 0x7fffffffull);
    if ((r = dalloc(c, &c->plog, (size_t)3 * c->plog_cap))) return r;
  }
  return run_steps(c, t_sec, dt_sec, n_steps, step0, flags, kh_deg2_s, rec_lon, rec_lat, rec_species, rec_census);
}

int lm_query_pairs(lm_ctx* c, int64_t n, const float* lon, const float* lat, int32_t* pi, int32_t* pj, int64_t cap,
                   int64_t* n_pairs) {
  if (!c || !n_pairs || (n > 0 && (!lon || !lat))) return fail(c, LM_ERR_ARG, "NULL argument");
  if (n < 0 || n > 0x7fffff00) return fail(c, LM_ERR_ARG, "particle count out of range");
  if (!c->has_params) return fail(c, LM_ERR_STATE, "call lm_set_interaction first");
  CK(cudaSetDevice(c->device));
  *n_pairs = 0;
  if (n == 0) return LM_OK;
  int r;
  if ((r = stage_positions(c, n, lon, lat))) return r;
  c->has_particles = false;  // positions now hold query points, not an advected state
  const StepArgs a = step_args(0.0, 1.0, 0, 0.0, false);
  for (;;) {
    PROF(c, P_BOOKKEEPING, launch_step_begin(bufs(c, false), nullptr, a, c->ctrl, c->st));
    CK(enqueue_interaction(c, a, 0u, true, false));
    if ((r = read_ctrl(c))) return r;
    if (c->hctrl->halt) {
      if ((r = regrow(c))) return r;
      continue;
    }
    break;
  }
  if ((r = clear_err_bits(c, ERRB_NAN))) return r;  // non-finite query points are never paired
  const uint32_t nv = c->hctrl->n_valid;
  const size_t novf = (size_t)c->hctrl->ovf_used;
  std::vector<uint32_t> deg(nv), ids(nv), slab((size_t)nv * SLAB), ovf(novf);
  if (nv) {
    CK(cudaMemcpyAsync(deg.data(), c->deg, nv * 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(ids.data(), c->sid, nv * 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(slab.data(), c->slab, (size_t)nv * SLAB * 4, cudaMemcpyDeviceToHost, c->st));
  }
  if (novf) CK(cudaMemcpyAsync(ovf.data(), c->ovf, novf * 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  std::vector<uint64_t> pairs;
  pairs.reserve((size_t)c->hctrl->n_dir / 2);
  for (uint32_t s = 0; s < nv; ++s)
    for (uint32_t h = 0; h < deg[s]; ++h) {
      const uint32_t t = entry_id(deg[s] <= SLAB ? slab[(size_t)s * SLAB + h] : ovf[(size_t)slab[(size_t)s * SLAB] + h]);
      const uint32_t a_ = ids[s], b_ = ids[t];
      if (a_ < b_) pairs.push_back(((uint64_t)a_ << 32) | b_);
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

int lm_debug_inject_wait(lm_ctx* c, double seconds) {
  if (!c) return LM_ERR_ARG;
  if (!(seconds > 0.0 && seconds <= 10.0)) return fail(c, LM_ERR_ARG, "seconds must be in (0, 10]");
  c->inject_wait_ns = std::max<unsigned long long>(1ull, (unsigned long long)(seconds * 1e9));
  return LM_OK;
}

int lm_count_pairs(lm_ctx* c, int64_t n, const float* lon, const float* lat, int64_t* n_pairs) {
  if (!c || !n_pairs || (n > 0 && (!lon || !lat))) return fail(c, LM_ERR_ARG, "NULL argument");
  if (n < 0 || n > 0x7fffff00) return fail(c, LM_ERR_ARG, "particle count out of range");
  if (!c->has_params) return fail(c, LM_ERR_STATE, "call lm_set_interaction first");
  CK(cudaSetDevice(c->device));
  *n_pairs = 0;
  if (n == 0) return LM_OK;
  int r;
  if ((r = stage_positions(c, n, lon, lat))) return r;
  c->has_particles = false;  // positions now hold query points, not an advected state
  const StepArgs a = step_args(0.0, 1.0, 0, 0.0, false);
  PROF(c, P_BOOKKEEPING, launch_step_begin(bufs(c, false), nullptr, a, c->ctrl, c->st));
  CK(enqueue_interaction(c, a, LM_STEP_COUNT_PAIRS, true, false));
  if ((r = read_ctrl(c))) return r;
  if ((r = clear_err_bits(c, ERRB_NAN))) return r;  // non-finite query points are never paired
  *n_pairs = (int64_t)(c->hctrl->n_dir / 2);
  return LM_OK;
}

int lm_interact(lm_ctx* c, int64_t n, const float* lon, const float* lat, int64_t step_index, uint32_t flags) {
  if (!c || (n > 0 && (!lon || !lat))) return fail(c, LM_ERR_ARG, "NULL argument");
  if (!c->has_params) return fail(c, LM_ERR_STATE, "call lm_set_interaction first");
  if (!c->has_species) return fail(c, LM_ERR_STATE, "upload species (lm_particles_upload or lm_species_upload) first");
  if (n != (int64_t)c->ntotal) return fail(c, LM_ERR_ARG, "n = %lld but the context holds %u species", (long long)n, c->ntotal);
  if (c->n_ens != 1) return fail(c, LM_ERR_STATE, "lm_interact works on a single ensemble");
  CK(cudaSetDevice(c->device));
  if (n == 0) return LM_OK;
  int r;
  if ((r = stage_positions(c, n, lon, lat))) return r;
  if ((flags & LM_STEP_LOG_PAIRS) && c->plog_cap < (uint64_t)8 * c->nslots + 1024) {
    c->plog_cap = (uint32_t)std::min<uint64_t>((uint64_t)8 * c->nslots + 1024, 0x7fffffffull);
    if ((r = dalloc(c, &c->plog, (size_t)3 * c->plog_cap))) return r;
  }
  if ((r = write_ctrl_step(c, step_index))) return r;
  const StepArgs a = step_args(0.0, 1.0, step_index, 0.0, false);
  const Bufs b = bufs(c, false);
  for (;;) {
    PROF(c, P_BOOKKEEPING, launch_step_begin(b, nullptr, a, c->ctrl, c->st));
    CK(enqueue_interaction(c, a, flags | LM_STEP_INTERACT, true, false));
    if (flags & LM_STEP_CENSUS) PROF(c, P_CENSUS, launch_census(b, c->ctrl, c->st));
    PROF(c, P_BOOKKEEPING, launch_step_end(c->ctrl, true, c->st));
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
  if (c->plog && c->hctrl->plog_n > c->plog_cap) return fail(c, LM_ERR_CAPACITY, "pair log truncated");
  return consume_errors(c);
}

int lm_pairs_get(lm_ctx* c, int32_t* pi, int32_t* pj, int32_t* round, int64_t cap, int64_t* n) {
  if (!c || !n) return LM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  int r;
  if ((r = read_ctrl(c))) return r;
  const uint32_t m = std::min(c->hctrl->plog_n, c->plog_cap);
  *n = m;
  if (m == 0 || !pi || !pj || !round) return LM_OK;  // count query
  if ((int64_t)m > cap) return fail(c, LM_ERR_CAPACITY, "pair log holds %u pairs", m);
  std::vector<uint32_t> h((size_t)3 * m);
  CK(cudaMemcpyAsync(h.data(), c->plog, h.size() * 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  std::vector<uint32_t> order(m);
  for (uint32_t k = 0; k < m; ++k) order[k] = k;
  std::sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
    const uint32_t* a = &h[3 * (size_t)x];
    const uint32_t* b = &h[3 * (size_t)y];
    if (a[2] != b[2]) return a[2] < b[2];
    if (a[0] != b[0]) return a[0] < b[0];
    return a[1] < b[1];
  });
  for (uint32_t k = 0; k < m; ++k) {
    const uint32_t* e = &h[3 * (size_t)order[k]];
    pi[k] = c->hmap[e[0]];  // slots -> caller indices
    pj[k] = c->hmap[e[1]];
    round[k] = (int32_t)e[2];
  }
  return LM_OK;
}

int lm_graph_capture(lm_ctx* c, double t_start, double dt_sec, int64_t step0, int steps_per_graph, uint32_t flags,
                     double kh_deg2_s) {
  if (!c) return LM_ERR_ARG;
  if (steps_per_graph < 1) return fail(c, LM_ERR_ARG, "steps_per_graph must be >= 1");
  int r;
  if ((r = check_ready(c, flags))) return r;
  if (!(dt_sec != 0) || !std::isfinite(dt_sec)) return fail(c, LM_ERR_ARG, "dt must be finite and nonzero");
  CK(cudaSetDevice(c->device));
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
  if (!c->gexec)
    return fail(c, LM_ERR_STATE, "no captured graph (capture again after a field upload or a change of capacity)");
  if (n_launches < 0) return fail(c, LM_ERR_ARG, "n_launches < 0");
  CK(cudaSetDevice(c->device));
  const int64_t first = c->next_step;
  const int64_t total = (int64_t)n_launches * c->g_spg;
  int r;
  if ((r = check_time(c, c->g_t_start + (first - c->g_step0) * c->g_dt, c->g_dt, total))) return r;
  for (int k = 0; k < n_launches; ++k) CK(cudaGraphLaunch(c->gexec, c->st));
  c->next_step = first + total;
  if (!sync) return LM_OK;
  if ((r = read_ctrl(c))) return r;
  if (c->hctrl->halt) {
    // A step overflowed a capacity: the graph halted at that step (already advected). Regrow,
    // finish that step and the rest with plain launches, then recapture for later runs.
    const int64_t k = (int64_t)c->hctrl->halt_step;
    if ((r = regrow(c))) return r;
    if ((r = write_ctrl_step(c, k))) return r;
    const StepArgs a = step_args(c->g_t_start + (k - c->g_step0) * c->g_dt, c->g_dt, k, c->g_kh, false);
    CK(enqueue_step(c, a, c->g_flags, false));
    if ((r = read_ctrl(c))) return r;
    if (c->hctrl->halt) return fail(c, LM_ERR_CAPACITY, "capacity exceeded again after regrowth");
    const int64_t rest = first + total - (k + 1);
    if (rest > 0) {
      r = run_steps(c, c->g_t_start + (k + 1 - c->g_step0) * c->g_dt, c->g_dt, rest, k + 1, c->g_flags, c->g_kh,
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
  out->n_particles = c->ntotal;
  out->pairs = (int64_t)(h.n_dir / 2);
  out->rounds = h.rounds;
  out->max_rounds = h.max_rounds;
  out->out_of_bounds = h.oob;
  out->step = h.step;
  for (int k = 0; k < 4; ++k) out->census[k] = h.census[k];
  out->adj_capacity = (int64_t)c->ovf_cap;
  out->regrows = c->regrows;
  out->pairs_total = (int64_t)h.pairs_total;
  out->steps_total = (int64_t)h.steps_total;
  out->cells = h.ncells;
  out->long_lists = h.n_long;
  out->n_ensembles = c->n_ens;
  out->rounds_total = (int64_t)h.rounds_total;
  return LM_OK;
}

int lm_stats_reset(lm_ctx* c) {
  if (!c) return LM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  const uint32_t zero = 0;
  const unsigned long long z64 = 0;
  CK(cudaMemcpyAsync(&c->ctrl->max_rounds, &zero, sizeof(zero), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(&c->ctrl->pairs_total, &z64, sizeof(z64), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(&c->ctrl->steps_total, &z64, sizeof(z64), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(&c->ctrl->rounds_total, &z64, sizeof(z64), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return LM_OK;
}

int lm_census_get(lm_ctx* c, int64_t* out, int64_t cap) {
  if (!c || !out) return LM_ERR_ARG;
  if (cap < 4 * (int64_t)c->n_ens) return fail(c, LM_ERR_CAPACITY, "need %u entries", 4 * c->n_ens);
  CK(cudaSetDevice(c->device));
  std::vector<uint32_t> h((size_t)4 * c->n_ens);
  if (!h.empty()) CK(cudaMemcpyAsync(h.data(), c->census, h.size() * 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (size_t k = 0; k < h.size(); ++k) out[k] = h[k];
  return LM_OK;
}

int lm_profile_enable(lm_ctx* c, int on) {
  if (!c) return LM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->st));
  prof_collect(c);
  for (int k = 0; k < P_NUM; ++k) {
    c->prof_ms[k] = 0;
    c->prof_n[k] = 0;
  }
  c->prof_on = on != 0;
  return LM_OK;
}

int lm_profile_get(lm_ctx* c, int kernel, char* name, size_t name_len, double* total_ms, int64_t* launches) {
  if (!c) return LM_ERR_ARG;
  if (kernel < 0 || kernel >= P_NUM) return fail(c, LM_ERR_ARG, "kernel index %d out of range [0, %d)", kernel, P_NUM);
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->st));
  prof_collect(c);
  if (name && name_len) snprintf(name, name_len, "%s", kProfNames[kernel]);
  if (total_ms) *total_ms = c->prof_ms[kernel];
  if (launches) *launches = c->prof_n[kernel];
  return LM_OK;
}

int lm_profile_count(void) { return P_NUM; }

}  // extern "C"

namespace lm {
void set_thread_error(const char* msg) { g_create_error = msg ? msg : ""; }
bool pdl_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("LM_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}
int ctx_device(const lm_ctx* c) { return c->device; }
int ctx_sms(const lm_ctx* c) { return c->sms; }
cudaStream_t ctx_stream(const lm_ctx* c) { return c->st; }
void ctx_set_error(lm_ctx* c, const char* msg) { c->err = msg ? msg : ""; }

bool uniform_axis(const double* a, int n, double* d) {
  if (n < 2) return false;
  const double step = (a[n - 1] - a[0]) / (n - 1);
  if (!(step > 0) || !std::isfinite(step)) return false;
  for (int k = 0; k < n; ++k)
    if (std::fabs(a[k] - (a[0] + step * k)) > 1e-6 * step) return false;
  *d = step;
  return true;
}

// Offsets are taken from the float32 origin (lon[0], lat[0]) of the grid.
void fill_field_view(FieldView& f, float2* uv, int nt, int ny, int nx, const double* lon, const double* lat,
                     const double* t_sec, double dx, double dy, double dT) {
  const double org_lon = (double)(float)lon[0], org_lat = (double)(float)lat[0];
  f.uv = uv;
  f.nx = nx;
  f.ny = ny;
  f.nt = nt;
  f.gx0 = (float)(lon[0] - org_lon);
  f.gy0 = (float)(lat[0] - org_lat);
  f.inv_dx = (float)(1.0 / dx);
  f.inv_dy = (float)(1.0 / dy);
  f.max_fx = (float)(nx - 1);
  f.max_fy = (float)(ny - 1);
  f.org_lon = (float)org_lon;
  f.org_lat = (float)org_lat;
  f.t0 = t_sec[0];
  f.dT = dT;
  f.gx0d = lon[0] - org_lon;
  f.gy0d = lat[0] - org_lat;
  f.inv_dxd = 1.0 / dx;
  f.inv_dyd = 1.0 / dy;
}
}  // namespace lm
