// K4 + K5: rock-paper-scissors species update over the step's pair set.
//
// The reference applies the pairs one after another, in place, in the iteration order of the
// Python set returned by query_pairs (interaction_simulator.py:104-105), calling
// rock_paper_scissors_interaction (interactions.py:13-40): if the two species differ, draw
// r ~ U[0,1); the cyclic winner (rock > scissors > paper > rock) wins with probability
// pRS / pSP / pPR of that matchup, and the loser takes the winner's species. Updates cascade to
// later pairs of the same step. The set order is an artifact of hashing, not a semantic.
//
// Here the order is fixed as descending pair priority (a Philox function of (seed, step, i, j)),
// which the CPU oracle replays with a restatement of the reference's pair function. Pairs that
// share no microbe commute, so any order that keeps the priority order at every microbe gives the
// same species: a pair may be applied as soon as it is the highest-priority unprocessed pair of
// both its microbes. r is drawn from the same Philox block (53-bit uniform), and r < p is
// evaluated exactly as the integer test u53 < ceil(p * 2^53).
//
// All pairs are applied by one persistent cooperative launch without grid barriers. Each vertex v
// publishes want[v], the partner of its highest-priority unprocessed pair (NONE when it has none).
// A pair (v, u) is ready exactly when want[v] == u and want[u] == v; the thread that polls the
// lower endpoint applies it and advances both heads. Only the applier of a vertex's current head
// pair ever writes that vertex's head/want, so every write has a single owner. Species and head
// writes are released before the want words that hand the vertices on; pollers read want with
// acquire loads. The globally highest-priority pending pair is always ready, so the loop always
// progresses; every wait is still bounded (error flag + return after a timeout).
//
// Each applied pair gets a level = 1 + max(level of the previous pair at either endpoint): pairs of
// one level share no microbe, and (level, i, j) is a deterministic sequential order equal in
// effect to the priority order. The pair log records it; the step's "rounds" is the max level.
#include "lm_internal.h"
#include "lm_philox.cuh"

namespace lm {

constexpr int RD_THREADS = 256;
constexpr unsigned long long ROUNDS_TIMEOUT_NS = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool beats(int x, int y) {
  // rock(1) > scissors(3), paper(2) > rock(1), scissors(3) > paper(2)
  return (x == 1 && y == 3) || (x == 2 && y == 1) || (x == 3 && y == 2);
}

// Apply pair (s, u), s < u in cell order, both heads pointing at it; returns its level.
__device__ __forceinline__ uint32_t apply_pair(const RoundBufs& b, const RpsParams& rp, uint32_t step, uint32_t s,
                                               uint32_t u, Ctrl* ctrl) {
  const uint32_t ia = b.id[s], ib = b.id[u];
  const uint32_t i = min(ia, ib), j = max(ia, ib);
  const int si = __ldcg(b.species + i), sj = __ldcg(b.species + j);
  if (si != sj) {
    unsigned long long t = 0;
    bool valid = true;
    if ((si == 1 && sj == 3) || (si == 3 && sj == 1)) t = rp.t_rs;
    else if ((si == 2 && sj == 1) || (si == 1 && sj == 2)) t = rp.t_pr;
    else if ((si == 3 && sj == 2) || (si == 2 && sj == 3)) t = rp.t_sp;
    else valid = false;  // species outside {1,2,3}: the reference's table has no case -> no change
    if (valid) {
      const PairDraw d = pair_draw(i, j, step, rp.seed_lo, rp.seed_hi);
      const bool fwd_wins = d.u53 < t;
      const bool i_wins = (beats(si, sj) == fwd_wins);  // particle i is the cyclic winner xor it lost the draw
      if (i_wins) __stcg(b.species + j, (int8_t)si);
      else __stcg(b.species + i, (int8_t)sj);
    }
  }
  const uint32_t level = max(__ldcg(b.level + s), __ldcg(b.level + u)) + 1u;
  __stcg(b.level + s, level);
  __stcg(b.level + u, level);
  if (b.plog) {
    const uint32_t k = atomicAdd(&ctrl->plog_n, 1u);
    if (k < b.plog_cap) {
      b.plog[3 * k + 0] = i;
      b.plog[3 * k + 1] = j;
      b.plog[3 * k + 2] = level - 1u;
    }
  }
  // hand both vertices on to their next pair
  const uint32_t hu = __ldcg(b.head + u) + 1u, hs = __ldcg(b.head + s) + 1u;
  __stcg(b.head + u, hu);
  __stcg(b.head + s, hs);
  const uint32_t nu = hu < b.deg[u] ? b.adj[b.off[u] + hu] : NONE;
  const uint32_t ns = hs < b.deg[s] ? b.adj[b.off[s] + hs] : NONE;
  __threadfence();
  st_release(b.want[0] + u, nu);
  st_release(b.want[0] + s, ns);
  return level;
}

__global__ void __launch_bounds__(RD_THREADS) k_rounds(RoundBufs b, RpsParams rp, StepArgs a, Ctrl* ctrl,
                                                       uint32_t round_cap) {
  (void)round_cap;
  if (((volatile uint32_t*)&ctrl->halt)[0]) return;
  const uint32_t step = a.use_ctrl_step ? ctrl->step : a.step0;
  const uint32_t cnt = ((volatile uint32_t*)ctrl->act_n)[0];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t* L = b.act[0];
  uint32_t* want = b.want[0];
  uint32_t max_level = 0;
  const unsigned long long t0 = globaltimer();
  bool pending = first < cnt;
  uint32_t polls = 0;
  while (pending) {
    pending = false;
    for (uint32_t x = first; x < cnt; x += stride) {
      const uint32_t s = L[x];
      const uint32_t u = ld_acquire(want + s);
      if (u == NONE) continue;
      pending = true;
      if (s < u && ld_acquire(want + u) == s) max_level = max(max_level, apply_pair(b, rp, step, s, u, ctrl));
    }
    if (pending && ((++polls & 63u) == 0u) && globaltimer() - t0 > ROUNDS_TIMEOUT_NS) {
      atomicOr(&ctrl->err, (uint32_t)ERRB_TIMEOUT);
      break;
    }
  }
  for (int o = 16; o > 0; o >>= 1) max_level = max(max_level, __shfl_xor_sync(0xffffffffu, max_level, o));
  if ((threadIdx.x & 31) == 0 && max_level) {
    atomicMax(&ctrl->rounds, max_level);
    atomicMax(&ctrl->max_rounds, max_level);
  }
}

int rounds_grid(int device, int* block) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rounds, RD_THREADS, 0);
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 4) per_sm = 4;
  *block = RD_THREADS;
  return sms * per_sm;
}

cudaError_t launch_rounds(const RoundBufs& b, const RpsParams& rp, const StepArgs& a, Ctrl* ctrl, uint32_t n,
                          int grid, int block, uint32_t round_cap, cudaStream_t st) {
  (void)n;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_rounds, b, rp, a, ctrl, round_cap);
}

// Per-step species census (counts of species 0..3 after the step; 0 collects anything else).
__global__ void k_census(const int8_t* __restrict__ species, Ctrl* ctrl, uint32_t n) {
  if (ctrl->halt) return;
  __shared__ uint32_t h[4];
  if (threadIdx.x < 4) h[threadIdx.x] = 0;
  __syncthreads();
  uint32_t c[4] = {0, 0, 0, 0};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int s = species[i];
    c[(s >= 1 && s <= 3) ? s : 0]++;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    uint32_t v = c[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&h[k], v);
  }
  __syncthreads();
  if (threadIdx.x < 4 && h[threadIdx.x]) atomicAdd(&ctrl->census[threadIdx.x], h[threadIdx.x]);
}

void launch_census(const int8_t* species, Ctrl* ctrl, uint32_t n, cudaStream_t st) {
  int grid = (int)((n + 255) / 256);
  if (grid > 152 * 8) grid = 152 * 8;
  if (grid < 1) grid = 1;
  k_census<<<grid, 256, 0, st>>>(species, ctrl, n);
}

// Per-step bookkeeping: reset per-step counters (start), advance the device step counter (end).
__global__ void k_step_begin(Ctrl* ctrl) {
  if (ctrl->halt) return;
  ctrl->act_n[0] = ctrl->act_n[1] = ctrl->act_n[2] = 0;
  ctrl->plog_n = 0;
  ctrl->rounds = 0;
  ctrl->applied = 0;
  ctrl->n_valid = 0;
  ctrl->n_dir = 0;
  ctrl->bar_count = 0;
  ctrl->census[0] = ctrl->census[1] = ctrl->census[2] = ctrl->census[3] = 0;
}

__global__ void k_step_end(Ctrl* ctrl) {
  if (ctrl->halt) return;
  ctrl->step += 1;
}

void launch_step_begin(Ctrl* ctrl, cudaStream_t st) { k_step_begin<<<1, 1, 0, st>>>(ctrl); }
void launch_step_end(Ctrl* ctrl, cudaStream_t st) { k_step_end<<<1, 1, 0, st>>>(ctrl); }

}  // namespace lm
