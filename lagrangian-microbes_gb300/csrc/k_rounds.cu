// K4 + K5: rock-paper-scissors species update over the step's pair set.
//
// The reference applies the pairs one after another, in place, in the iteration order of the
// Python set returned by query_pairs (interaction_simulator.py:104-105), calling
// rock_paper_scissors_interaction (interactions.py:13-40): if the two species differ, draw
// r ~ U[0,1); the cyclic winner (rock > scissors > paper > rock) wins with probability
// pRS / pSP / pPR of that matchup, and the loser takes the winner's species. Updates cascade to
// later pairs of the same step. The set order is an artifact of hashing, not a semantic.
//
// Here the order is fixed as descending pair priority (k_pairs.cu), which the CPU oracle replays
// with a restatement of the reference's pair function. Pairs that share no microbe commute, so
// any schedule that keeps the priority order at every microbe gives the same species: a pair may
// be applied as soon as it is the highest-priority unprocessed pair of both its microbes.
// r is drawn from a Philox block keyed by (ensemble seed, step, i, j) (53-bit uniform), and
// r < p is evaluated exactly as the integer test u53 < ceil(p * 2^53).
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

// Partner of vertex s at list position h (NONE past the end).
__device__ __forceinline__ uint32_t next_partner(const Bufs& b, uint32_t s, uint32_t h) {
  const uint32_t d = b.deg[s];
  if (h >= d) return NONE;
  return d <= SLAB ? b.slab[(size_t)s * SLAB + h] : b.ovf[(size_t)b.off[s] + h];
}

// Apply pair (s, u), s < u in cell order, both heads pointing at it; returns its level.
__device__ __forceinline__ uint32_t apply_pair(const Bufs& b, uint32_t step, uint32_t s, uint32_t u, Ctrl* ctrl) {
  const EnsInfo& info = b.ens[b.sens[s]];
  const uint32_t pa = b.sid[s], pb = b.sid[u];
  const uint32_t pi = min(pa, pb), pj = max(pa, pb);  // slots; local ids are slot - base
  const int si = __ldcg(b.species + pi), sj = __ldcg(b.species + pj);
  if (si != sj) {
    unsigned long long t = 0;
    bool valid = true;
    if ((si == 1 && sj == 3) || (si == 3 && sj == 1)) t = info.t_rs;
    else if ((si == 2 && sj == 1) || (si == 1 && sj == 2)) t = info.t_pr;
    else if ((si == 3 && sj == 2) || (si == 2 && sj == 3)) t = info.t_sp;
    else valid = false;  // species outside {1,2,3}: the reference's table has no case -> no change
    if (valid) {
      const PairDraw d = pair_draw(pi - info.base, pj - info.base, step, info.seed_lo, info.seed_hi);
      const bool fwd_wins = d.u53 < t;
      const bool i_wins = (beats(si, sj) == fwd_wins);  // i is the cyclic winner and won, or lost and won anyway
      if (i_wins) __stcg(b.species + pj, (int8_t)si);
      else __stcg(b.species + pi, (int8_t)sj);
    }
  }
  const uint32_t level = max(__ldcg(b.level + s), __ldcg(b.level + u)) + 1u;
  __stcg(b.level + s, level);
  __stcg(b.level + u, level);
  if (b.plog) {
    const uint32_t k = atomicAdd(&ctrl->plog_n, 1u);
    if (k < b.plog_cap) {
      b.plog[3 * k + 0] = pi;
      b.plog[3 * k + 1] = pj;
      b.plog[3 * k + 2] = level - 1u;
    }
  }
  // hand both vertices on to their next pair
  const uint32_t hu = __ldcg(b.head + u) + 1u, hs = __ldcg(b.head + s) + 1u;
  __stcg(b.head + u, hu);
  __stcg(b.head + s, hs);
  const uint32_t nu = next_partner(b, u, hu);
  const uint32_t ns = next_partner(b, s, hs);
  __threadfence();
  st_release(b.want + u, nu);
  st_release(b.want + s, ns);
  return level;
}

__global__ void __launch_bounds__(RD_THREADS) k_rounds(Bufs b, StepArgs a, Ctrl* ctrl) {
  if (((volatile uint32_t*)&ctrl->halt)[0]) return;
  const uint32_t step = a.use_ctrl_step ? ctrl->step : a.step0;
  const uint32_t cnt = ((volatile uint32_t*)&ctrl->act_n)[0];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t max_level = 0;
  const unsigned long long t0 = globaltimer();
  bool pending = first < cnt;
  uint32_t polls = 0;
  while (pending) {
    pending = false;
    for (uint32_t x = first; x < cnt; x += stride) {
      const uint32_t s = b.act[x];
      const uint32_t u = ld_acquire(b.want + s);
      if (u == NONE) continue;
      pending = true;
      if (s < u && ld_acquire(b.want + u) == s) max_level = max(max_level, apply_pair(b, step, s, u, ctrl));
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

cudaError_t launch_rounds(const Bufs& b, const StepArgs& a, Ctrl* ctrl, int grid, int block, cudaStream_t st) {
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
  return cudaLaunchKernelEx(&cfg, k_rounds, b, a, ctrl);
}

// Species counts after the step, per ensemble and in total ([0] collects values outside 1..3).
__global__ void __launch_bounds__(SLOT_BLOCK) k_census(Bufs b, Ctrl* ctrl) {
  if (ctrl->halt) return;
  __shared__ uint32_t h[4];
  if (threadIdx.x < 4) h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t p = blockIdx.x * SLOT_BLOCK + threadIdx.x;
  int s = -1;
  if (p < b.nslots && b.status[p] != STATUS_PAD) {
    s = b.species[p];
    s = (s >= 1 && s <= 3) ? s : 0;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    uint32_t v = __popc(__ballot_sync(0xffffffffu, s == k));
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&h[k], v);
  }
  __syncthreads();
  if (threadIdx.x < 4 && h[threadIdx.x]) {
    atomicAdd(&b.census[4 * b.block_ens[blockIdx.x] + threadIdx.x], h[threadIdx.x]);
    atomicAdd(&ctrl->census[threadIdx.x], h[threadIdx.x]);
  }
}

void launch_census(const Bufs& b, Ctrl* ctrl, cudaStream_t st) {
  if (b.nslots == 0) return;
  k_census<<<(b.nslots + SLOT_BLOCK - 1) / SLOT_BLOCK, SLOT_BLOCK, 0, st>>>(b, ctrl);
}

}  // namespace lm
