// K3: fixed-radius neighbour search over the cell-sorted particles, replacing
// cKDTree(X).query_pairs(r=interaction_radius, p=interaction_norm) (interaction_simulator.py:93-98).
//
// Distance semantics are the reference's: Minkowski-p on raw (lon, lat) degrees, inclusive
// (d <= r), on float32 positions promoted to float64. For p = 2 the decision is
// fl(fl(dx*dx) + fl(dy*dy)) <= fl(r*r) in float64 without FMA contraction; p = 1 uses |dx| + |dy| <= r
// and p = inf uses max(|dx|, |dy|) <= r. A float32 test accepts or rejects every candidate whose
// float32 distance lies outside a relative band of 2e-6 around the radius (its rounding error is
// below 3e-7 relative), and only candidates inside the band are decided in float64.
//
// Each particle scans the 3 rows of its 3x3 cell neighbourhood; the three cells of a row are
// consecutive keys, hence one contiguous run of the sorted array. Two passes: count (degree), then
// fill (neighbour list, sorted by descending pair priority, the order the interaction rounds use).
#include "lm_internal.h"
#include "lm_philox.cuh"

// the local insertion sort reads pr[y-1] / pid[y-1] only for y > 0, i.e. after they were written
#pragma nv_diag_suppress 549

namespace lm {

constexpr int SW_THREADS = 256;
constexpr uint32_t LOCAL_MAX = 16;  // neighbour lists up to this length are sorted in thread-local storage

int sweep_blocks(uint32_t n) { return (int)((n + SW_THREADS - 1) / SW_THREADS); }

__device__ __forceinline__ bool within(const PairParams& pp, float2 a, float2 b) {
  float dx = a.x - b.x, dy = a.y - b.y;
  if (pp.norm == 2) {
    float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    if (d2 < pp.r2f_lo) return true;
    if (d2 > pp.r2f_hi) return false;
    double ddx = __dsub_rn((double)a.x, (double)b.x), ddy = __dsub_rn((double)a.y, (double)b.y);
    double d = __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy));
    return d <= pp.r2;
  } else if (pp.norm == 1) {
    float d1 = fabsf(dx) + fabsf(dy);
    if (d1 < pp.rf_lo) return true;
    if (d1 > pp.rf_hi) return false;
    double ddx = __dsub_rn((double)a.x, (double)b.x), ddy = __dsub_rn((double)a.y, (double)b.y);
    return __dadd_rn(fabs(ddx), fabs(ddy)) <= pp.r;
  } else {
    float di = fmaxf(fabsf(dx), fabsf(dy));
    if (di < pp.rf_lo) return true;
    if (di > pp.rf_hi) return false;
    double ddx = __dsub_rn((double)a.x, (double)b.x), ddy = __dsub_rn((double)a.y, (double)b.y);
    return fmax(fabs(ddx), fabs(ddy)) <= pp.r;
  }
}

// Calls f(t) for every sorted index t != s within the radius of particle s (cell order).
template <class F>
__device__ __forceinline__ void for_neighbours(const CellGrid& g, const PairParams& pp,
                                               const uint32_t* __restrict__ key, const float2* __restrict__ spos,
                                               const uint32_t* __restrict__ cell_start, uint32_t n_valid, uint32_t s,
                                               F&& f) {
  const uint32_t k = key[s];
  const int cy = (int)(k / (uint32_t)g.ncx);
  const int cx = (int)(k - (uint32_t)cy * (uint32_t)g.ncx);
  const float2 ps = spos[s];
  for (int dy = -1; dy <= 1; ++dy) {
    const int ry = cy + dy;
    if (ry < 0 || ry >= g.ncy) continue;
    const uint32_t kl = (uint32_t)ry * g.ncx + (uint32_t)max(cx - 1, 0);
    const uint32_t kh = (uint32_t)ry * g.ncx + (uint32_t)min(cx + 1, g.ncx - 1);
    uint32_t start = NONE;
    for (uint32_t kk = kl; kk <= kh; ++kk) {
      uint32_t c = cell_start[kk];
      if (c < n_valid && key[c] == kk) {
        start = c;
        break;
      }
    }
    if (start == NONE) continue;
    for (uint32_t t = start; t < n_valid; ++t) {
      if (key[t] > kh) break;
      if (t != s && within(pp, ps, spos[t])) f(t);
    }
  }
}

__global__ void __launch_bounds__(SW_THREADS) k_sweep_count(CellGrid g, PairParams pp, const uint32_t* __restrict__ key,
                                                            const float2* __restrict__ spos,
                                                            const uint32_t* __restrict__ cell_start, Ctrl* ctrl,
                                                            uint32_t* __restrict__ deg,
                                                            uint32_t* __restrict__ block_sum, uint32_t n) {
  if (ctrl->halt) return;
  __shared__ uint32_t ws[SW_THREADS / 32];
  const uint32_t s = blockIdx.x * SW_THREADS + threadIdx.x;
  const uint32_t n_valid = ctrl->n_valid;
  uint32_t c = 0;
  if (s < n_valid) {
    for_neighbours(g, pp, key, spos, cell_start, n_valid, s, [&](uint32_t) { ++c; });
  }
  if (s < n) deg[s] = c;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < SW_THREADS / 32; ++w) t += ws[w];
    block_sum[blockIdx.x] = t;
  }
}

// Exclusive scan of the per-block degree sums (one block), total -> ctrl->n_dir, capacity check.
__global__ void __launch_bounds__(1024) k_scan_blocks(uint32_t* __restrict__ bs, uint32_t nb, Ctrl* ctrl) {
  if (ctrl->halt) return;
  __shared__ unsigned long long warp_sums[32];
  __shared__ unsigned long long carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t start = 0; start < nb; start += blockDim.x) {
    uint32_t i = start + threadIdx.x;
    unsigned long long x = (i < nb) ? bs[i] : 0ull;
    unsigned long long y = x;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long t = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += t;
    }
    if (lane == 31) warp_sums[wid] = y;
    __syncthreads();
    if (wid == 0) {
      unsigned long long w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0ull;
      for (int o = 1; o < 32; o <<= 1) {
        unsigned long long t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      warp_sums[lane] = w;
    }
    __syncthreads();
    unsigned long long c = carry + (wid ? warp_sums[wid - 1] : 0ull);
    unsigned long long excl = c + y - x;
    if (i < nb) bs[i] = (uint32_t)(excl > 0xffffffffull ? 0xffffffffull : excl);
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = c + y;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    unsigned long long total = carry;
    ctrl->n_dir = total;
    if (total > ctrl->cap) {  // the step is redone after the host regrows the lists
      ctrl->halt = 1;
      ctrl->halt_step = ctrl->step;
      atomicOr(&ctrl->err, (uint32_t)ERRB_OVERFLOW);
    } else {
      ctrl->pairs_total += total / 2;
      ctrl->steps_total += 1;
    }
  }
}

__device__ __forceinline__ uint32_t lanemask_lt_p() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Descending priority; ties (probability 2^-64 per pair) broken by ascending partner id, which is
// consistent with one global order on unordered pairs (prio desc, then (min id, max id) asc).
__device__ __forceinline__ bool before(unsigned long long pa, uint32_t ia, unsigned long long pb, uint32_t ib) {
  return pa > pb || (pa == pb && ia < ib);
}

__device__ void sort_segment(unsigned long long* __restrict__ pr, uint32_t* __restrict__ nb,
                             const uint32_t* __restrict__ id, uint32_t d) {
  if (d <= 64) {
    for (uint32_t x = 1; x < d; ++x) {
      unsigned long long p = pr[x];
      uint32_t t = nb[x], it = id[t];
      uint32_t y = x;
      while (y > 0) {
        unsigned long long q = pr[y - 1];
        uint32_t u = nb[y - 1];
        if (!before(p, it, q, id[u])) break;
        pr[y] = q;
        nb[y] = u;
        --y;
      }
      pr[y] = p;
      nb[y] = t;
    }
    return;
  }
  // Heap sort for long lists: build a heap whose root is the LAST element in the final order.
  auto sift = [&](uint32_t root, uint32_t len) {
    while (true) {
      uint32_t c = 2 * root + 1;
      if (c >= len) break;
      if (c + 1 < len && before(pr[c], id[nb[c]], pr[c + 1], id[nb[c + 1]])) ++c;
      if (!before(pr[root], id[nb[root]], pr[c], id[nb[c]])) break;
      unsigned long long tp = pr[root]; pr[root] = pr[c]; pr[c] = tp;
      uint32_t tn = nb[root]; nb[root] = nb[c]; nb[c] = tn;
      root = c;
    }
  };
  for (uint32_t r = d / 2; r-- > 0;) sift(r, d);
  for (uint32_t end = d - 1; end > 0; --end) {
    unsigned long long tp = pr[0]; pr[0] = pr[end]; pr[end] = tp;
    uint32_t tn = nb[0]; nb[0] = nb[end]; nb[end] = tn;
    sift(0, end);
  }
}

__global__ void __launch_bounds__(SW_THREADS) k_sweep_fill(CellGrid g, PairParams pp, RpsParams rp, StepArgs a,
                                                           const uint32_t* __restrict__ key,
                                                           const uint32_t* __restrict__ id,
                                                           const float2* __restrict__ spos,
                                                           const uint32_t* __restrict__ cell_start,
                                                           const uint32_t* __restrict__ block_sum, Ctrl* ctrl,
                                                           const uint32_t* __restrict__ deg, uint32_t* __restrict__ off,
                                                           uint32_t* __restrict__ adj, unsigned long long* __restrict__ prio,
                                                           uint32_t* __restrict__ want0, uint32_t* __restrict__ head,
                                                           uint32_t* __restrict__ act0, uint32_t* __restrict__ level,
                                                           uint32_t n) {
  if (ctrl->halt) return;
  __shared__ uint32_t ws[SW_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t s = blockIdx.x * SW_THREADS + threadIdx.x;
  const uint32_t step = a.use_ctrl_step ? ctrl->step : a.step0;
  const uint32_t d = (s < n) ? deg[s] : 0u;
  // block-exclusive scan of degrees
  uint32_t y = d;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, y, o);
    if (lane >= o) y += t;
  }
  if (lane == 31) ws[wid] = y;
  __syncthreads();
  uint32_t wp = 0;
  for (int w = 0; w < wid; ++w) wp += ws[w];
  const uint32_t o = block_sum[blockIdx.x] + wp + y - d;
  bool active = false;
  if (s < n) {
    off[s] = o;
    head[s] = 0;
    level[s] = 0;
    if (d > 0) {
      const uint32_t n_valid = ctrl->n_valid;
      const uint32_t ia = id[s];
      if (d <= LOCAL_MAX) {
        // short lists: collect and insertion-sort in thread-local storage, write the sorted list once
        unsigned long long pr[LOCAL_MAX];
        uint32_t nb[LOCAL_MAX], pid[LOCAL_MAX];
        uint32_t m = 0;
        for_neighbours(g, pp, key, spos, cell_start, n_valid, s, [&](uint32_t t) {
          if (m < LOCAL_MAX) {
            const uint32_t ib = id[t];
            const PairDraw pd = pair_draw(min(ia, ib), max(ia, ib), step, rp.seed_lo, rp.seed_hi);
            uint32_t y = m;
            while (y > 0 && before(pd.prio, ib, pr[y - 1], pid[y - 1])) {
              pr[y] = pr[y - 1];
              nb[y] = nb[y - 1];
              pid[y] = pid[y - 1];
              --y;
            }
            pr[y] = pd.prio;
            nb[y] = t;
            pid[y] = ib;
          }
          ++m;
        });
        for (uint32_t k = 0; k < d; ++k) adj[o + k] = nb[k];
        want0[s] = nb[0];
      } else {
        uint32_t m = 0;
        for_neighbours(g, pp, key, spos, cell_start, n_valid, s, [&](uint32_t t) {
          if (m < d) {
            const uint32_t ib = id[t];
            const PairDraw pd = pair_draw(min(ia, ib), max(ia, ib), step, rp.seed_lo, rp.seed_hi);
            adj[o + m] = t;
            prio[o + m] = pd.prio;
          }
          ++m;
        });
        sort_segment(prio + o, adj + o, id, d);
        want0[s] = adj[o];
      }
      active = true;
    }
  }
  // warp-aggregated append of active vertices to the round-0 list
  uint32_t mask = __ballot_sync(0xffffffffu, active);
  if (mask) {
    uint32_t base = 0;
    int leader = __ffs(mask) - 1;
    if (lane == leader) base = atomicAdd(&ctrl->act_n[0], (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (active) act0[base + __popc(mask & lanemask_lt_p())] = s;
  }
}

void launch_sweep_count(const CellGrid& g, const PairParams& pp, const uint32_t* key, const float2* spos,
                        const uint32_t* cell_start, Ctrl* ctrl, uint32_t* deg, uint32_t* block_sum, uint32_t n,
                        cudaStream_t st) {
  if (n == 0) return;
  k_sweep_count<<<sweep_blocks(n), SW_THREADS, 0, st>>>(g, pp, key, spos, cell_start, ctrl, deg, block_sum, n);
}

void launch_scan_blocks(uint32_t* block_sum, uint32_t nblocks, Ctrl* ctrl, cudaStream_t st) {
  k_scan_blocks<<<1, 1024, 0, st>>>(block_sum, nblocks, ctrl);
}

void launch_sweep_fill(const CellGrid& g, const PairParams& pp, const RpsParams& rp, const StepArgs& a,
                       const uint32_t* key, const uint32_t* id, const float2* spos, const uint32_t* cell_start,
                       const uint32_t* block_sum, Ctrl* ctrl, const uint32_t* deg, uint32_t* off, uint32_t* adj,
                       unsigned long long* prio, uint32_t* want0, uint32_t* head, uint32_t* act0, uint32_t* level,
                       uint32_t n, cudaStream_t st) {
  if (n == 0) return;
  k_sweep_fill<<<sweep_blocks(n), SW_THREADS, 0, st>>>(g, pp, rp, a, key, id, spos, cell_start, block_sum, ctrl, deg,
                                                        off, adj, prio, want0, head, act0, level, n);
}

}  // namespace lm
