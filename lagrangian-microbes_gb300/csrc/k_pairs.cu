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
// One thread per particle (cell order) scans the three rows of its 3x3 cell neighbourhood; the
// three cells of a row are consecutive keys, hence one contiguous run of the sorted array. Each
// neighbour list is kept sorted by descending pair priority, the order in which the interaction
// applies pairs: lists of up to SLAB entries are gathered in registers, sorted by a sorting network and stored in
// the per-vertex slab; longer lists are rebuilt by a second kernel into a per-step overflow
// area (allocated with an atomic cursor, regrown by the host on overflow) and sorted there.
//
// Pair priority: a 64-bit order hash of (seed, step, i, j) (the output function of SplitMix64, a
// bijection of its input, so no two pairs of a step share a priority). Any fixed order is a valid
// choice for the reference's unordered set iteration. A random order keeps the dependency chains
// of the interaction short: on the mixed lattice of the 490k workload its longest chain is
// 56-70 pairs against 80-91 for a 2x2 checkerboard-colour-major order (measured on the oracle),
// and degree-first orders are worse still (110-180).
#include "lm_internal.h"
#include "lm_philox.cuh"

namespace lm {

__device__ __forceinline__ bool within(const PairParams& pp, float2 a, float2 b) {
  const float dx = a.x - b.x, dy = a.y - b.y;
  if (pp.norm == 2) {
    const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    if (d2 < pp.r2f_lo) return true;
    if (d2 > pp.r2f_hi) return false;
    const double ddx = __dsub_rn((double)a.x, (double)b.x), ddy = __dsub_rn((double)a.y, (double)b.y);
    return __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)) <= pp.r2;
  } else if (pp.norm == 1) {
    const float d1 = fabsf(dx) + fabsf(dy);
    if (d1 < pp.rf_lo) return true;
    if (d1 > pp.rf_hi) return false;
    const double ddx = __dsub_rn((double)a.x, (double)b.x), ddy = __dsub_rn((double)a.y, (double)b.y);
    return __dadd_rn(fabs(ddx), fabs(ddy)) <= pp.r;
  } else {
    const float di = fmaxf(fabsf(dx), fabsf(dy));
    if (di < pp.rf_lo) return true;
    if (di > pp.rf_hi) return false;
    const double ddx = __dsub_rn((double)a.x, (double)b.x), ddy = __dsub_rn((double)a.y, (double)b.y);
    return fmax(fabs(ddx), fabs(ddy)) <= pp.r;
  }
}

__device__ __forceinline__ unsigned long long pair_prio(uint32_t i, uint32_t j, uint32_t step, uint32_t k0,
                                                        uint32_t k1) {
  return order_hash(i, j, step, ((unsigned long long)k1 << 32) | k0);
}

// The three rock-paper-scissors outcomes of pair (local ids la, lb) at `step`, as list-entry bits:
// the pair's Philox uniform (interactions.py:20's np.random.rand(), keyed by the pair) against the
// ensemble's forward-win threshold of each matchup (interactions.py:24-35), u53 < t exactly as
// r < p. Only the entry of the endpoint that applies the pair (the lower cell-order index) gets them.
__device__ __forceinline__ uint32_t win_bits(const EnsInfo& info, uint32_t la, uint32_t lb, uint32_t step) {
  const PairDraw d = pair_draw(min(la, lb), max(la, lb), step, info.seed_lo, info.seed_hi);
  return ((d.u53 < info.t_rs ? 1u : 0u) | (d.u53 < info.t_pr ? 2u : 0u) | (d.u53 < info.t_sp ? 4u : 0u))
         << ENTRY_WIN_SHIFT;
}

// a before b: higher priority first, ties by lower partner id (one global order on pairs).
__device__ __forceinline__ bool before(unsigned long long pa, uint32_t ia, unsigned long long pb, uint32_t ib) {
  return pa > pb || (pa == pb && ia < ib);
}

struct Vertex {
  uint32_t s, e, base, cx, cy;
  EnsGrid g;
  float2 ps;
};

__device__ __forceinline__ Vertex load_vertex(const Bufs& b, uint32_t s) {
  Vertex v;
  v.s = s;
  v.e = b.sens[s];
  v.g = b.grids[v.e];
  v.base = b.ens[v.e].base;
  cell_coords(v.g, b.skey[s] - v.g.cell_base, &v.cx, &v.cy);
  v.ps = b.spos[s];
  return v;
}

// Calls f(t) for every cell-order index t != s within the radius of vertex v (in no particular
// order). The key runs of the three rows (at most two each) are found first and all their cell
// starts loaded together, so a microbe waits for one round of those loads instead of one per row.
// (Walking the runs four candidates at a time as well needed 58 registers and was slower.)
// The cell-order ranges [t0[k], t1[k]) of the (at most six) key runs of v's 3x3 neighbourhood,
// all cell starts loaded together; missing runs are empty.
__device__ __forceinline__ void neighbour_runs(const Bufs& b, const Vertex& v, uint32_t* t0, uint32_t* t1) {
  uint32_t klo[6], khi[6];
  bool has[6];
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy) {
    const int ry = (int)v.cy + dy;
    const bool row = ry >= 0 && ry < v.g.ncy;
    const RowRuns rr = row_runs(v.g, max((int)v.cx - 1, 0), min((int)v.cx + 1, v.g.ncx - 1), row ? ry : (int)v.cy);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      has[(dy + 1) * 2 + q] = row && q < rr.n;
      klo[(dy + 1) * 2 + q] = rr.lo[q];
      khi[(dy + 1) * 2 + q] = rr.hi[q];
    }
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    t0[k] = has[k] ? b.cstart[klo[k]] : 0u;
    t1[k] = has[k] ? b.cstart[khi[k] + 1] : 0u;
  }
}

// The six runs are walked as one candidate range (candidate i lies in the run q with
// c[q] <= i < c[q + 1]), so a warp's loop lasts as long as its longest total, not the sum of its
// longest run of each row.
template <class F>
__device__ __forceinline__ void for_neighbours(const Bufs& b, const PairParams& pp, const Vertex& v, F&& f) {
  uint32_t t0[6], t1[6];
  neighbour_runs(b, v, t0, t1);
  uint32_t c[7];
  c[0] = 0;
#pragma unroll
  for (int q = 0; q < 6; ++q) c[q + 1] = c[q] + (t1[q] - t0[q]);
  for (uint32_t i = 0; i < c[6]; ++i) {
    uint32_t t = t0[0] + i;
#pragma unroll
    for (int q = 1; q < 6; ++q)
      if (i >= c[q]) t = t0[q] + (i - c[q]);  // the last run starting at or before i (empty runs never win)
    if (t != v.s && within(pp, v.ps, b.spos[t])) f(t);
  }
}

__device__ __forceinline__ uint32_t lanemask_lt_p() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ void append_active(const Bufs& b, Ctrl* ctrl, bool active, uint32_t s) {
  const uint32_t mask = __ballot_sync(0xffffffffu, active);
  if (mask) {
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&ctrl->act_n, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (active) b.act[base + __popc(mask & lanemask_lt_p())] = s;
  }
}

// The outcome draws of a warp's slab lists, spread evenly over its lanes: lane L needs the draws of
// the entries in `mask` (bit k: entry k), pair (la, lb[k]) of ensemble `ens`. Drawn one slot per
// lane in turn, at most 8 x 32 per warp, instead of each lane drawing its own (about half the slots
// of a lattice list need a draw, and the lanes need them at different slots). The bits are merged
// into e[k]. Every lane of the warp calls this.
__device__ __forceinline__ void sweep_draws(const Bufs& b, uint32_t step, uint32_t mask, uint32_t la,
                                            const uint32_t* lb, uint32_t ens, uint32_t* e) {
  __shared__ uint32_t q_lb[SLOT_BLOCK / 32][32 * SLAB];    // local id of the partner, per draw
  __shared__ uint16_t q_src[SLOT_BLOCK / 32][32 * SLAB];   // lane * SLAB + slot of the draw
  __shared__ uint8_t q_bits[SLOT_BLOCK / 32][32 * SLAB];   // outcome bits, by lane * SLAB + slot
  __shared__ uint32_t w_la[SLOT_BLOCK / 32][32], w_ens[SLOT_BLOCK / 32][32];
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  const uint32_t cnt = __popc(mask);
  uint32_t incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  if (total == 0) return;
  uint32_t pos = incl - cnt;
#pragma unroll
  for (int k = 0; k < (int)SLAB; ++k) {
    if ((mask >> k) & 1u) {
      q_lb[w][pos] = lb[k];
      q_src[w][pos] = (uint16_t)(lane * SLAB + k);
      ++pos;
    }
  }
  w_la[w][lane] = la;
  w_ens[w][lane] = ens;
  __syncwarp();
  for (uint32_t q = lane; q < total; q += 32) {
    const uint32_t src = q_src[w][q], owner = src / SLAB;
    const EnsInfo& info = b.ens[w_ens[w][owner]];
    q_bits[w][src] = (uint8_t)(win_bits(info, w_la[w][owner], q_lb[w][q], step) >> ENTRY_WIN_SHIFT);
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < (int)SLAB; ++k)
    if ((mask >> k) & 1u) e[k] |= (uint32_t)q_bits[w][lane * SLAB + k] << ENTRY_WIN_SHIFT;
}

__global__ void __launch_bounds__(SLOT_BLOCK, 5) k_sweep(Bufs b, PairParams pp, StepArgs a, Ctrl* ctrl) {
  pdl_wait();
  if (ctrl->halt) return;
  const uint32_t n_valid = ctrl->n_valid;
  const uint32_t step = a.use_ctrl_step ? ctrl->step : a.step0;
  const uint32_t s = blockIdx.x * SLOT_BLOCK + threadIdx.x;
  bool active = false, is_long = false;
  uint32_t m = 0;
  // slab lists awaiting their outcome draws: entries, which ones need a draw, local ids, ensemble
  uint32_t nbo[SLAB], draw_mask = 0, draw_la = 0, draw_lb[SLAB], draw_info = 0;
#pragma unroll
  for (int k = 0; k < (int)SLAB; ++k) nbo[k] = draw_lb[k] = 0;
  if (s < n_valid) {
    const Vertex v = load_vertex(b, s);
    const EnsInfo& info = b.ens[v.e];
    const uint32_t k0 = info.seed_lo, k1 = info.seed_hi;
    const uint32_t la = b.sid[s] - v.base;
    unsigned long long pr[SLAB];
    uint32_t nb[SLAB], pl[SLAB];
#pragma unroll
    for (int k = 0; k < (int)SLAB; ++k) {
      pr[k] = 0ull;
      nb[k] = NONE;
      pl[k] = NONE;
    }
    // phase 1: collect the neighbours (compile-time slots, predicated); the divergent candidate
    // loop does no more than the distance test
    for_neighbours(b, pp, v, [&](uint32_t t) {
      // shift register: the newest neighbour in slot 0 (the slots are sorted below; entries past
      // the eighth are collected again by the long-list kernel)
#pragma unroll
      for (int k = (int)SLAB - 1; k > 0; --k) nb[k] = nb[k - 1];
      nb[0] = t;
      ++m;
    });
    // phase 2: priorities over the slots, a loop whose trip count (the degree) is nearly the same
    // across the warp
    if (m <= SLAB) {
#pragma unroll
      for (int k = 0; k < (int)SLAB; ++k) {
        if ((uint32_t)k < m) {
          const uint32_t t = nb[k];
          const uint32_t lb = b.sid[t] - v.base;
          pr[k] = pair_prio(min(la, lb), max(la, lb), step, k0, k1);
          pl[k] = lb;
        }
      }
    }
    // sorting network; empty slots (priority 0, partner NONE) sort last. When no list of the warp
    // has more than 4 entries (most of a lattice), the 5-comparator network of 4 entries suffices.
#define LM_CX(x, y)                                         \
  if (before(pr[y], pl[y], pr[x], pl[x])) {                  \
    const unsigned long long tp = pr[x]; pr[x] = pr[y]; pr[y] = tp; \
    const uint32_t tn = nb[x]; nb[x] = nb[y]; nb[y] = tn;    \
    const uint32_t tl = pl[x]; pl[x] = pl[y]; pl[y] = tl;    \
  }
    if (__all_sync(__activemask(), m <= 4)) {
      if (m > 1) {
        LM_CX(0, 1) LM_CX(2, 3) LM_CX(0, 2) LM_CX(1, 3) LM_CX(1, 2)
      }
    } else if (m > 1 && m <= SLAB) {
      // 19-comparator network for 8 entries
      LM_CX(0, 2) LM_CX(1, 3) LM_CX(4, 6) LM_CX(5, 7)
      LM_CX(0, 4) LM_CX(1, 5) LM_CX(2, 6) LM_CX(3, 7)
      LM_CX(0, 1) LM_CX(2, 3) LM_CX(4, 5) LM_CX(6, 7)
      LM_CX(2, 4) LM_CX(3, 5) LM_CX(1, 4) LM_CX(3, 6)
      LM_CX(1, 2) LM_CX(3, 4) LM_CX(5, 6)
    }
#undef LM_CX
    b.deg[s] = m;
    b.level[s] = 0;
    if (m <= SLAB) {
      // the outcomes of the pairs this vertex applies (partner above it in cell order), drawn by
      // the whole warp (sweep_draws) and merged into the entries
      uint32_t need = 0;
#pragma unroll
      for (int k = 0; k < (int)SLAB; ++k)
        if ((uint32_t)k < m && nb[k] > s) need |= 1u << k;
      draw_mask = need;
      draw_la = la;
#pragma unroll
      for (int k = 0; k < (int)SLAB; ++k) {
        draw_lb[k] = pl[k];
        nbo[k] = nb[k];
      }
      draw_info = v.e;
      active = m > 0;
    } else {
      is_long = true;
      b.wstate[s] = pack_state(NONE, 0u, b.species[b.sid[s]]);  // set by k_sweep_long
    }
  }
  sweep_draws(b, step, draw_mask, draw_la, draw_lb, draw_info, nbo);
  if (s < n_valid && m <= SLAB) {
#pragma unroll
    for (int k = 0; k < (int)SLAB; ++k)
      if ((uint32_t)k < m) b.slab[(size_t)s * SLAB + k] = nbo[k];
    b.wstate[s] = pack_state(m ? nbo[0] : NONE, 0u, b.species[b.sid[s]]);  // entry 0 of the list
  }
  append_active(b, ctrl, active, s);
  // long lists are finished by k_sweep_long
  {
    const uint32_t mask = __ballot_sync(0xffffffffu, is_long);
    if (mask) {
      const int lane = threadIdx.x & 31;
      const int leader = __ffs(mask) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(&ctrl->n_long, (uint32_t)__popc(mask));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (is_long) b.longv[base + __popc(mask & lanemask_lt_p())] = s;
    }
  }
  // directed entries of the step
  __shared__ unsigned long long tot;
  if (threadIdx.x == 0) tot = 0;
  __syncthreads();
  unsigned long long mm = m;
  for (int o = 16; o > 0; o >>= 1) mm += __shfl_xor_sync(0xffffffffu, mm, o);
  if ((threadIdx.x & 31) == 0 && mm) atomicAdd(&tot, mm);
  __syncthreads();
  if (threadIdx.x == 0 && tot) atomicAdd(&ctrl->n_dir, tot);
}

void launch_sweep(const Bufs& b, const PairParams& pp, const StepArgs& a, Ctrl* ctrl, cudaStream_t st) {
  if (b.nslots == 0) return;
  launch_dep(k_sweep, dim3((b.nslots + SLOT_BLOCK - 1) / SLOT_BLOCK), dim3(SLOT_BLOCK), st, b, pp, a, ctrl);
}

// Count-only pair search (the clustered stress workload, whose 1e11+ pairs per step cannot be
// listed): every unordered pair within the radius is counted once, with the same cell grid and
// the same distance test as the sweep. Microbe a (cell order) tests the members of its own cell
// with a higher cell-order index and every member of its four "forward" cells: (cx+1, cy) and the
// three cells of row cy+1 (cx-1 .. cx+1, one contiguous run). A block whose 256 microbes all lie
// in one cell (cluster cores, thousands per cell) walks those runs through shared-memory tiles;
// any other block lets each thread walk its own runs. Counts are summed per block and added to
// the step's directed-entry counter (2 per pair) with one atomic.
constexpr uint32_t COUNT_THREADS = 256;
constexpr int COUNT_RUNS = 4;

__device__ __forceinline__ void count_runs(const Vertex& v, const Bufs& b, uint32_t* r0, uint32_t* r1) {
  // r[0] = the rest of the own cell, r[1] = (cx+1, cy), r[2..3] = row cy+1 from cx-1 to cx+1 (one
  // or two key runs: the row may cross a tile edge); unused runs are empty
  const uint32_t kc = v.g.cell_base + cell_index(v.g, v.cx, v.cy);
  r0[0] = v.s + 1;
  r1[0] = b.cstart[kc + 1];
  for (int q = 1; q < COUNT_RUNS; ++q) r0[q] = r1[q] = 0;
  if ((int)v.cx + 1 < v.g.ncx) {
    const uint32_t ke = v.g.cell_base + cell_index(v.g, v.cx + 1, v.cy);
    r0[1] = b.cstart[ke];
    r1[1] = b.cstart[ke + 1];
  }
  if ((int)v.cy + 1 < v.g.ncy) {
    const RowRuns rr = row_runs(v.g, max((int)v.cx - 1, 0), min((int)v.cx + 1, v.g.ncx - 1), (int)v.cy + 1);
    r0[2] = b.cstart[rr.lo[0]];
    r1[2] = b.cstart[rr.hi[0] + 1];
    if (rr.n == 2) {
      r0[3] = b.cstart[rr.lo[1]];
      r1[3] = b.cstart[rr.hi[1] + 1];
    }
  }
}

__global__ void __launch_bounds__(COUNT_THREADS) k_count_pairs(Bufs b, PairParams pp, Ctrl* ctrl) {
  pdl_wait();
  if (ctrl->halt) return;
  __shared__ __align__(16) float2 tile[COUNT_THREADS];
  __shared__ uint32_t first_key, last_key;
  __shared__ unsigned long long tot;
  const uint32_t n_valid = ctrl->n_valid;
  const uint32_t blk0 = blockIdx.x * COUNT_THREADS;
  if (blk0 >= n_valid) return;  // block-uniform
  const uint32_t s = blk0 + threadIdx.x;
  const uint32_t last = min(n_valid, blk0 + COUNT_THREADS) - 1;
  if (threadIdx.x == 0) {
    first_key = b.skey[blk0];
    last_key = b.skey[last];
    tot = 0;
  }
  __syncthreads();
  unsigned long long cnt = 0;
  const bool dense = first_key == last_key && last - blk0 + 1 == COUNT_THREADS;
  if (dense) {
    // all 256 microbes share one cell and hence the same forward runs; the own-cell run starts
    // after the block's first microbe, each thread keeps only partners with a higher index
    const Vertex v = load_vertex(b, blk0);
    uint32_t r0[COUNT_RUNS], r1[COUNT_RUNS];
    count_runs(v, b, r0, r1);
    const float2 me = b.spos[s];
    for (int q = 0; q < COUNT_RUNS; ++q) {
      for (uint32_t tb = r0[q]; tb < r1[q]; tb += COUNT_THREADS) {
        const uint32_t n_t = min(COUNT_THREADS, r1[q] - tb);
        if (threadIdx.x < n_t) tile[threadIdx.x] = b.spos[tb + threadIdx.x];
        __syncthreads();
        // own cell: partner index tb + k must exceed s
        const uint32_t k0 = q == 0 ? (s + 1 > tb ? min(s + 1 - tb, n_t) : 0u) : 0u;
        if (pp.norm == 2) {
          // branch-free float32 decision, two candidates per 16-byte shared load: clo counts the
          // candidates below the float32 band around r^2, chi those not above it; a tile where they
          // differ holds a candidate inside the band and is recounted with the exact test (the same
          // decision as within()). d2 is one fused multiply-add: its error is far inside the band.
          uint32_t clo = 0, chi = 0;
          const float lo = pp.r2f_lo, hi = pp.r2f_hi;
          uint32_t k = k0;
          if ((k & 1u) && k < n_t) {
            const float dx = me.x - tile[k].x, dy = me.y - tile[k].y;
            const float d2 = fmaf(dx, dx, dy * dy);
            clo += d2 < lo ? 1u : 0u;
            chi += d2 <= hi ? 1u : 0u;
            ++k;
          }
          const float4* t4 = reinterpret_cast<const float4*>(tile);
#pragma unroll 4
          for (; k + 1 < n_t; k += 2) {
            const float4 q = t4[k >> 1];
            const float ax = me.x - q.x, ay = me.y - q.y, bx = me.x - q.z, by = me.y - q.w;
            const float da = fmaf(ax, ax, ay * ay), db = fmaf(bx, bx, by * by);
            clo += (da < lo ? 1u : 0u) + (db < lo ? 1u : 0u);
            chi += (da <= hi ? 1u : 0u) + (db <= hi ? 1u : 0u);
          }
          if (k < n_t) {
            const float dx = me.x - tile[k].x, dy = me.y - tile[k].y;
            const float d2 = fmaf(dx, dx, dy * dy);
            clo += d2 < lo ? 1u : 0u;
            chi += d2 <= hi ? 1u : 0u;
          }
          if (clo != chi) {
            clo = 0;
            for (uint32_t kk = k0; kk < n_t; ++kk) clo += within(pp, me, tile[kk]) ? 1u : 0u;
          }
          cnt += clo;
        } else {
          for (uint32_t k = k0; k < n_t; ++k) cnt += within(pp, me, tile[k]) ? 1u : 0u;
        }
        __syncthreads();
      }
    }
  } else if (s < n_valid) {
    const Vertex v = load_vertex(b, s);
    uint32_t r0[COUNT_RUNS], r1[COUNT_RUNS];
    count_runs(v, b, r0, r1);
    for (int q = 0; q < COUNT_RUNS; ++q)
      for (uint32_t t = r0[q]; t < r1[q]; ++t) cnt += within(pp, v.ps, b.spos[t]) ? 1u : 0u;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&tot, cnt);
  __syncthreads();
  if (threadIdx.x == 0 && tot) atomicAdd(&ctrl->n_dir, 2ull * tot);
}

void launch_count_pairs(const Bufs& b, const PairParams& pp, Ctrl* ctrl, cudaStream_t st) {
  if (b.nslots == 0) return;
  launch_dep(k_count_pairs, dim3((b.nslots + COUNT_THREADS - 1) / COUNT_THREADS), dim3(COUNT_THREADS), st, b, pp,
             ctrl);
}

// In-place sort of one long list (priorities pr, list entries nb) into `before` order.
__device__ void sort_segment(unsigned long long* __restrict__ pr, uint32_t* __restrict__ nb,
                             const uint32_t* __restrict__ sid, uint32_t d) {
  if (d <= 64) {
    for (uint32_t x = 1; x < d; ++x) {
      const unsigned long long p = pr[x];
      const uint32_t t = nb[x], it = sid[entry_id(t)];
      uint32_t y = x;
      while (y > 0) {
        const unsigned long long q = pr[y - 1];
        const uint32_t u = nb[y - 1];
        if (!before(p, it, q, sid[entry_id(u)])) break;
        pr[y] = q;
        nb[y] = u;
        --y;
      }
      pr[y] = p;
      nb[y] = t;
    }
    return;
  }
  // heap sort for long lists: the heap's root is the element that comes last
  auto sift = [&](uint32_t root, uint32_t len) {
    while (true) {
      uint32_t c = 2 * root + 1;
      if (c >= len) break;
      if (c + 1 < len && before(pr[c], sid[entry_id(nb[c])], pr[c + 1], sid[entry_id(nb[c + 1])])) ++c;
      if (!before(pr[root], sid[entry_id(nb[root])], pr[c], sid[entry_id(nb[c])])) break;
      const unsigned long long tp = pr[root];
      pr[root] = pr[c];
      pr[c] = tp;
      const uint32_t tn = nb[root];
      nb[root] = nb[c];
      nb[c] = tn;
      root = c;
    }
  };
  for (uint32_t r = d / 2; r-- > 0;) sift(r, d);
  for (uint32_t end = d - 1; end > 0; --end) {
    const unsigned long long tp = pr[0];
    pr[0] = pr[end];
    pr[end] = tp;
    const uint32_t tn = nb[0];
    nb[0] = nb[end];
    nb[end] = tn;
    sift(0, end);
  }
}

// Long lists (more than SLAB neighbours): one warp per vertex. The warp reserves the overflow space
// of all its vertices with one atomic; for each batch of 32 vertices lane k loads vertex k's cell,
// position, key runs and ensemble constants, so the dependent loads happen once per batch. For
// each vertex the warp then walks its six key runs as one candidate range, 64 candidates a pass
// (position and id loaded together), and gathers the neighbours with ballots into shared memory.
// The order (priority descending, partner's local id ascending) comes from:
//   - up to 32 entries: a rank sort in registers, one entry per lane;
//   - up to LONG_SMEM_MAX: a bucket sort. The priorities are uniform 64-bit hashes, so 256 buckets
//     on their top 8 bits (descending) hold about d / 256 entries each, and an insertion sort
//     inside each bucket by the exact order finishes it;
//   - beyond: a sort in global memory by one lane.
// Only the sorted partners are kept (the priorities were needed for the order only).
constexpr int LONG_WARPS = 4;
constexpr uint32_t LONG_SMEM_MAX = 512;
constexpr uint32_t LONG_BUCKETS = 256;

struct LongSmem {
  unsigned long long p[LONG_SMEM_MAX];  // pair priority of entry i (gather order)
  uint32_t t[LONG_SMEM_MAX];            // list entry (partner's cell-order index + outcome bits)
  uint16_t ord[LONG_SMEM_MAX];          // entries in list order
  uint32_t start[LONG_BUCKETS], cur[LONG_BUCKETS];
};

// Does entry x come before entry y? Ties of the 64-bit priority (rare) go by the partner's local id.
__device__ __forceinline__ bool long_before(const Bufs& b, const LongSmem& sh, uint32_t base, uint32_t x, uint32_t y) {
  const unsigned long long px = sh.p[x], py = sh.p[y];
  if (px != py) return px > py;
  return b.sid[entry_id(sh.t[x])] - base < b.sid[entry_id(sh.t[y])] - base;
}

// The bucket sort of entries [0, d) of sh into sh.ord (one warp).
__device__ __forceinline__ void long_sort(const Bufs& b, LongSmem& sh, uint32_t base, uint32_t d, uint32_t lane) {
  for (uint32_t i = lane; i < LONG_BUCKETS; i += 32) sh.cur[i] = 0;
  __syncwarp();
  for (uint32_t i = lane; i < d; i += 32) atomicAdd(&sh.cur[255u - (uint32_t)(sh.p[i] >> 56)], 1u);
  __syncwarp();
  // exclusive scan of the bucket counts: lane holds buckets 8 lane .. 8 lane + 7
  uint32_t c[8], tot = 0;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    c[r] = sh.cur[8 * lane + r];
    tot += c[r];
  }
  uint32_t incl = tot;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  uint32_t run = incl - tot;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    sh.start[8 * lane + r] = run;
    sh.cur[8 * lane + r] = run;
    run += c[r];
  }
  __syncwarp();
  for (uint32_t i = lane; i < d; i += 32)
    sh.ord[atomicAdd(&sh.cur[255u - (uint32_t)(sh.p[i] >> 56)], 1u)] = (uint16_t)i;
  __syncwarp();
  for (uint32_t k = lane; k < LONG_BUCKETS; k += 32) {
    const uint32_t lo = sh.start[k], hi = sh.cur[k];
    for (uint32_t x = lo + 1; x < hi; ++x) {
      const uint16_t e = sh.ord[x];
      uint32_t y = x;
      while (y > lo && long_before(b, sh, base, e, sh.ord[y - 1])) {
        sh.ord[y] = sh.ord[y - 1];
        --y;
      }
      sh.ord[y] = e;
    }
  }
  __syncwarp();
}

__global__ void __launch_bounds__(LONG_WARPS * 32) k_sweep_long(Bufs b, PairParams pp, StepArgs a, Ctrl* ctrl) {
  pdl_wait();
  if (ctrl->halt) return;
  __shared__ LongSmem sh_all[LONG_WARPS];
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  LongSmem& sh = sh_all[w];
  const uint32_t n_long = ctrl->n_long;
  const uint32_t step = a.use_ctrl_step ? ctrl->step : a.step0;
  const unsigned long long cap = ctrl->ovf_cap;
  const uint32_t gw = blockIdx.x * LONG_WARPS + w, nw = gridDim.x * LONG_WARPS;
  // this warp's vertices: gw, gw + nw, gw + 2 nw, ...; one atomic reserves the space of all of them
  const uint32_t count = gw < n_long ? (n_long - gw + nw - 1) / nw : 0u;
  if (count == 0) return;
  unsigned long long sum = 0;
  bool too_many = false;
  for (uint32_t i = lane; i < count; i += 32) {
    const uint32_t d = b.deg[b.longv[gw + i * nw]];
    sum += d;
    too_many |= d > MAX_DEGREE;
  }
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  too_many = __any_sync(0xffffffffu, too_many);
  unsigned long long run = 0;
  if (lane == 0) run = atomicAdd(&ctrl->ovf_used, sum);
  run = __shfl_sync(0xffffffffu, run, 0);
  if (too_many || run + sum > cap) {  // positions would not fit the state word / the area is full
    if (lane == 0) {
      ctrl->halt = 1;
      ctrl->halt_step = ctrl->step;
      atomicOr(&ctrl->err, too_many ? (uint32_t)ERRB_ROUNDCAP : (uint32_t)ERRB_OVERFLOW);
    }
    return;
  }
  for (uint32_t ib = 0; ib < count; ib += 32) {
    // lane k holds vertex ib + k of this warp's list, and loads its cell, position, key runs and
    // ensemble constants, for all 32 vertices at once (a chain of dependent loads per batch
    // instead of one per vertex)
    const bool mine = ib + lane < count;
    const uint32_t s_l = mine ? b.longv[gw + (ib + lane) * nw] : 0u;
    const uint32_t d_l = mine ? b.deg[s_l] : 0u;
    unsigned long long incl = d_l;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    const unsigned long long o_l = run + incl - d_l;
    run += __shfl_sync(0xffffffffu, incl, 31);
    uint32_t r0[6], r1[6], la_l = 0, base_l = 0, k0_l = 0, k1_l = 0, e_l = 0;
    int sp_l = 0;
    float px_l = 0.f, py_l = 0.f;
#pragma unroll
    for (int q = 0; q < 6; ++q) r0[q] = r1[q] = 0u;
    if (mine) {
      const Vertex v = load_vertex(b, s_l);
      neighbour_runs(b, v, r0, r1);
      const EnsInfo& info = b.ens[v.e];
      k0_l = info.seed_lo;
      k1_l = info.seed_hi;
      e_l = v.e;
      base_l = v.base;
      const uint32_t id = b.sid[s_l];
      la_l = id - v.base;
      sp_l = b.species[id];
      px_l = v.ps.x;
      py_l = v.ps.y;
    }
    const uint32_t nk = min(32u, count - ib);
    for (uint32_t k = 0; k < nk; ++k) {
      const uint32_t s = __shfl_sync(0xffffffffu, s_l, k);
      const uint32_t d = __shfl_sync(0xffffffffu, d_l, k);
      const unsigned long long o = __shfl_sync(0xffffffffu, o_l, k);
      const uint32_t la = __shfl_sync(0xffffffffu, la_l, k), base = __shfl_sync(0xffffffffu, base_l, k);
      const uint32_t k0 = __shfl_sync(0xffffffffu, k0_l, k), k1 = __shfl_sync(0xffffffffu, k1_l, k);
      const float2 ps = make_float2(__shfl_sync(0xffffffffu, px_l, k), __shfl_sync(0xffffffffu, py_l, k));
      const int sp = __shfl_sync(0xffffffffu, sp_l, k);
      const EnsInfo& info = b.ens[__shfl_sync(0xffffffffu, e_l, k)];
      // the six runs as one candidate range: candidate i is in the run q with c[q] <= i < c[q + 1]
      uint32_t t0[6], c[7];
      c[0] = 0;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        t0[q] = __shfl_sync(0xffffffffu, r0[q], k);
        c[q + 1] = c[q] + (__shfl_sync(0xffffffffu, r1[q], k) - t0[q]);
      }
      const bool in_smem = d <= LONG_SMEM_MAX;
      uint32_t m = 0;
      // two slices of 32 candidates per pass, each candidate's position and id loaded together
      for (uint32_t tb = 0; tb < c[6]; tb += 64) {
        uint32_t t[2], id[2];
        float2 pt[2];
        bool in[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint32_t i = tb + 32u * h + lane;
          uint32_t x = t0[0] + i;
#pragma unroll
          for (int q = 1; q < 6; ++q)
            if (i >= c[q]) x = t0[q] + (i - c[q]);  // the last run starting at or before i (empty runs never win)
          t[h] = x;
          in[h] = i < c[6] && x != s;
          pt[h] = in[h] ? b.spos[x] : ps;
          id[h] = in[h] ? b.sid[x] : 0u;
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const bool ok = in[h] && within(pp, ps, pt[h]);
          const uint32_t mask = __ballot_sync(0xffffffffu, ok);
          if (ok) {
            const uint32_t pos = m + __popc(mask & lanemask_lt_p());
            if (pos < d) {  // the partner and its local id; priority and draw follow below
              if (in_smem) {
                sh.p[pos] = id[h] - base;
                sh.t[pos] = t[h];
              } else {
                b.ovf[o + pos] = t[h];
                b.oprio[o + pos] = id[h] - base;
              }
            }
          }
          m += __popc(mask);
        }
      }
      // priorities and outcome draws of the d entries, one entry per lane (in the gather only the
      // lanes that found a neighbour would work, about a third of them)
      __syncwarp();
      for (uint32_t i = lane; i < d; i += 32) {
        const uint32_t tt = in_smem ? sh.t[i] : b.ovf[o + i];
        const uint32_t lb = (uint32_t)(in_smem ? sh.p[i] : b.oprio[o + i]);
        const unsigned long long p = pair_prio(min(la, lb), max(la, lb), step, k0, k1);
        const uint32_t e = tt > s ? tt | win_bits(info, la, lb, step) : tt;
        if (in_smem) {
          sh.p[i] = p;
          sh.t[i] = e;
        } else {
          b.ovf[o + i] = e;
          b.oprio[o + i] = p;
        }
      }
      uint32_t first;
      if (d <= 32) {
        // one entry per lane, ranked by counting the entries that come before it
        __syncwarp();
        const bool has = lane < d;
        const unsigned long long pi = has ? sh.p[lane] : 0ull;
        const uint32_t ti = has ? sh.t[lane] : 0u;
        uint32_t rank = 0;
        bool tie = false;
        for (uint32_t j = 0; j < d; ++j) {
          const unsigned long long pj = __shfl_sync(0xffffffffu, pi, j);
          rank += pj > pi ? 1u : 0u;
          tie |= pj == pi && j != lane;
        }
        if (__any_sync(0xffffffffu, has && tie)) {
          // equal priorities go by the partner's local id (the order hash is a bijection of the
          // pair, so this is not expected within one list)
          const uint32_t li = has ? b.sid[entry_id(ti)] - base : 0u;
          for (uint32_t j = 0; j < d; ++j) {
            const unsigned long long pj = __shfl_sync(0xffffffffu, pi, j);
            const uint32_t lj = __shfl_sync(0xffffffffu, li, j);
            rank += (pj == pi && j != lane && lj < li) ? 1u : 0u;
          }
        }
        if (has) b.ovf[o + rank] = ti;
        const uint32_t r0m = __ballot_sync(0xffffffffu, has && rank == 0u);
        first = __shfl_sync(0xffffffffu, ti, __ffs(r0m) - 1);
        __syncwarp();  // the next vertex reuses the shared list
      } else if (in_smem) {
        __syncwarp();
        long_sort(b, sh, base, d, lane);
        for (uint32_t i = lane; i < d; i += 32) b.ovf[o + i] = sh.t[sh.ord[i]];
        first = sh.t[sh.ord[0]];
        __syncwarp();  // the next vertex reuses the shared list
      } else {
        __syncwarp();
        if (lane == 0) sort_segment(b.oprio + o, b.ovf + o, b.sid, d);
        __syncwarp();
        first = b.ovf[o];
      }
      if (lane == 0) {
        b.slab[(size_t)s * SLAB] = (uint32_t)o;  // a long list's overflow offset, in its unused slab row
        b.wstate[s] = pack_state(first, 0u, sp);  // entry 0 of the list
      }
    }
    // every vertex of the batch is active (it has > SLAB pairs): one atomic per batch
    uint32_t at = 0;
    if (lane == 0) at = atomicAdd(&ctrl->act_n, nk);
    at = __shfl_sync(0xffffffffu, at, 0);
    if (lane < nk) b.act[at + lane] = s_l;
  }
}

void launch_sweep_long(const Bufs& b, const PairParams& pp, const StepArgs& a, Ctrl* ctrl, int sms,
                       int blocks_per_sm, cudaStream_t st) {
  // at most 6 blocks of 36 KB fit an SM's shared memory; more queue behind them
  launch_dep(k_sweep_long, dim3(sms * blocks_per_sm), dim3(LONG_WARPS * 32), st, b, pp, a, ctrl);
}

}  // namespace lm
