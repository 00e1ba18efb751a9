// K4 + K5: rock-paper-scissors species update over the step's pair set.
//
// The reference applies the pairs one after another, in place, in the iteration order of the
// Python set returned by query_pairs (interaction_simulator.py:104-105), calling
// rock_paper_scissors_interaction (interactions.py:13-40): if the two species differ, draw
// r ~ U[0,1); the cyclic winner (rock > scissors > paper > rock) wins with probability
// pRS / pSP / pPR of that matchup, and the loser takes the winner's species. Updates cascade to
// later pairs of the same step. The set order is an artifact of hashing, not a semantic.
//
// Here the order is fixed as descending pair priority (a Philox function of (seed, step, i, j)).
// That order is applied in parallel without changing its result: in round r every vertex looks at
// its highest-priority unprocessed pair; a pair whose two endpoints both look at it is the
// earliest unprocessed pair at both, so all such pairs form a matching that commutes with itself
// and precedes every pair it conflicts with. Applying rounds one after another is therefore the
// same as applying the whole list in priority order, which the CPU oracle replays with the
// reference's own pair function. r is drawn from the same Philox block (53-bit uniform), and
// r < p is evaluated exactly as the integer test u53 < ceil(p * 2^53).
//
// One persistent cooperative launch runs all rounds, separated by a grid barrier whose waits are
// bounded (error flag + return on timeout). When the active set drops below SOLO_VERTICES the
// remaining rounds run in block 0 alone with block barriers.
#include "lm_internal.h"
#include "lm_philox.cuh"

namespace lm {

constexpr int RD_THREADS = 512;
constexpr uint32_t SOLO_VERTICES = 2048;
constexpr unsigned long long BARRIER_TIMEOUT_NS = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t lanemask_lt_r() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Sense-by-generation grid barrier. Returns false if the wait timed out (error bit set).
__device__ bool grid_barrier(Ctrl* c, uint32_t nblocks) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* gen = &c->bar_gen;
    uint32_t g = *gen;
    __threadfence();
    uint32_t arrived = atomicAdd(&c->bar_count, 1u);
    int res = 1;
    if (arrived == nblocks - 1) {
      atomicExch(&c->bar_count, 0u);
      __threadfence();
      atomicAdd(&c->bar_gen, 1u);
    } else {
      unsigned long long t0 = globaltimer();
      while (*gen == g) {
        if (globaltimer() - t0 > BARRIER_TIMEOUT_NS) {
          atomicOr(&c->err, (uint32_t)ERRB_TIMEOUT);
          res = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (((volatile uint32_t*)&c->err)[0] & ERRB_TIMEOUT) res = 0;
    ok = res;
  }
  __syncthreads();
  return ok != 0;
}

__device__ __forceinline__ bool beats(int x, int y) {
  // rock(1) > scissors(3), paper(2) > rock(1), scissors(3) > paper(2)
  return (x == 1 && y == 3) || (x == 2 && y == 1) || (x == 3 && y == 2);
}

__device__ __forceinline__ void apply_pair(const RoundBufs& b, const RpsParams& rp, uint32_t step, uint32_t s,
                                           uint32_t u, uint32_t round, Ctrl* ctrl) {
  const uint32_t ia = b.id[s], ib = b.id[u];
  const uint32_t i = min(ia, ib), j = max(ia, ib);
  const int si = __ldcg(b.species + i), sj = __ldcg(b.species + j);
  if (si != sj) {
    PairDraw d = pair_draw(i, j, step, rp.seed_lo, rp.seed_hi);
    unsigned long long t = 0;
    bool valid = true;
    if ((si == 1 && sj == 3) || (si == 3 && sj == 1)) t = rp.t_rs;
    else if ((si == 2 && sj == 1) || (si == 1 && sj == 2)) t = rp.t_pr;
    else if ((si == 3 && sj == 2) || (si == 2 && sj == 3)) t = rp.t_sp;
    else valid = false;  // species outside {1,2,3}: the reference's table has no case -> no change
    if (valid) {
      const bool fwd_i = beats(si, sj);  // particle i is the cyclic (forward) winner
      const bool fwd_wins = d.u53 < t;
      const bool i_wins = (fwd_i == fwd_wins);
      if (i_wins) b.species[j] = (int8_t)si;
      else b.species[i] = (int8_t)sj;
    }
  }
  if (b.plog) {
    uint32_t k = atomicAdd(&ctrl->plog_n, 1u);
    if (k < b.plog_cap) {
      b.plog[3 * k + 0] = i;
      b.plog[3 * k + 1] = j;
      b.plog[3 * k + 2] = round;
    }
  }
}

__global__ void __launch_bounds__(RD_THREADS) k_rounds(RoundBufs b, RpsParams rp, StepArgs a, Ctrl* ctrl,
                                                       uint32_t round_cap) {
  if (((volatile uint32_t*)&ctrl->halt)[0]) return;
  const uint32_t step = a.use_ctrl_step ? ctrl->step : a.step0;
  const uint32_t nblocks = gridDim.x;
  const int lane = threadIdx.x & 31;
  bool solo = (nblocks == 1);
  uint32_t r = 0;
  uint32_t cnt = ((volatile uint32_t*)ctrl->act_n)[0];
  if (!solo && cnt <= SOLO_VERTICES) {
    if (blockIdx.x != 0) return;
    solo = true;
  }
  while (cnt > 0) {
    if (r >= round_cap) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&ctrl->err, (uint32_t)ERRB_ROUNDCAP);
      break;
    }
    const bool odd = (r & 1u) != 0;
    const uint32_t* L = odd ? b.act[1] : b.act[0];
    uint32_t* Ln = odd ? b.act[0] : b.act[1];
    const uint32_t* cur = odd ? b.want[1] : b.want[0];
    uint32_t* nxt = odd ? b.want[0] : b.want[1];
    const uint32_t r3 = r % 3u;
    uint32_t* ncnt = ctrl->act_n + (r3 == 2u ? 0u : r3 + 1u);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->act_n[r3 == 0u ? 2u : r3 - 1u] = 0;
    const uint32_t stride = solo ? blockDim.x : nblocks * blockDim.x;
    const uint32_t first = solo ? threadIdx.x : blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lim = (cnt + 31u) & ~31u;  // warp-uniform trip count
    for (uint32_t x = first - lane + 0; x < lim; x += stride) {
      const uint32_t xi = x + lane;
      bool keep = false;
      uint32_t s = 0;
      if (xi < cnt) {
        s = __ldcg(L + xi);
        const uint32_t u = __ldcg(cur + s);
        if (__ldcg(cur + u) == s) {
          if (s < u) apply_pair(b, rp, step, s, u, r, ctrl);
          const uint32_t h = b.head[s] + 1;
          b.head[s] = h;
          if (h < b.deg[s]) {
            nxt[s] = b.adj[b.off[s] + h];
            keep = true;
          }
        } else {
          nxt[s] = u;
          keep = true;
        }
      }
      const uint32_t m = __ballot_sync(0xffffffffu, keep);
      if (m) {
        const int leader = __ffs(m) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(ncnt, (uint32_t)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (keep) Ln[base + __popc(m & lanemask_lt_r())] = s;
      }
    }
    if (solo) {
      __threadfence_block();
      __syncthreads();
    } else if (!grid_barrier(ctrl, nblocks)) {
      return;
    }
    cnt = ((volatile uint32_t*)ncnt)[0];
    ++r;
    if (solo) __syncthreads();  // everyone has read cnt before thread 0 resets the next counter
    if (!solo && cnt <= SOLO_VERTICES) {
      if (blockIdx.x != 0) return;
      solo = true;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctrl->rounds = r;
    if (r > ctrl->max_rounds) ctrl->max_rounds = r;
  }
}

int rounds_grid(int device, int* block) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rounds, RD_THREADS, 0);
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 2) per_sm = 2;
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
