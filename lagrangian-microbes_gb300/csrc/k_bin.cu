// K2: uniform-cell binning, replacing the KD-tree build of the reference, cKDTree(X)
// (interaction_simulator.py:93); the fixed-radius query that follows is K3 (k_pairs.cu).
//
// Each step builds, per ensemble, a cell grid over the bounding box of its advected positions
// (cell size = cell_factor * r >= r, so every pair within r lies in the 3x3 neighbourhood), then
// sorts the particles by cell with a single counting pass on the full cell key (a one-digit
// radix sort): a warp-aggregated atomic count gives each particle its rank inside its cell, an
// exclusive scan over the cells gives the cell starts, and a scatter writes particle id, key,
// ensemble and position into cell order. The order inside a cell follows the atomics and is not
// deterministic; nothing downstream depends on it (pair lists are re-sorted by pair priority and
// every pair-order tie is broken by particle ids).
#include "lm_internal.h"

namespace lm {

constexpr int GRID_THREADS = 1024;

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Cells of one ensemble's grid at cell size c (1 for an empty ensemble). Float32 throughout: the
// grid only has to be consistent within the step (any c >= r gives the same pairs), and float64 is
// slow on this GPU.
__device__ __forceinline__ float grid_dims(const uint32_t* box, float c, float n, float* ncx, float* ncy,
                                           uint32_t* tshift) {
  const float mnx = dec_f(box[0]), mny = dec_f(box[1]), mxx = dec_f(box[2]), mxy = dec_f(box[3]);
  if (!(mnx <= mxx && mny <= mxy)) {
    *ncx = *ncy = 1.f;
    *tshift = 3u;
    return 1.f;
  }
  *ncx = floorf((mxx - mnx) / c) + 3.f;
  *ncy = floorf((mxy - mny) / c) + 3.f;
  *tshift = tile_shift(n, *ncx * *ncy);
  // the key range covers whole tiles
  const float t = (float)(1u << *tshift);
  return ceilf(*ncx / t) * ceilf(*ncy / t) * (t * t);
}

// Key ranges in ensemble index order (batches of more ensembles than the block has threads).
__device__ __forceinline__ void grid_in_order(const Bufs& b, float c, unsigned long long* carry_sh, uint32_t* wsi) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint32_t e0 = 0; e0 < b.n_ens; e0 += GRID_THREADS) {
    const uint32_t e = e0 + threadIdx.x;
    float nx = 0.f, ny = 0.f;
    uint32_t cells = 0, ts = 3u;
    if (e < b.n_ens) cells = (uint32_t)fminf(grid_dims(b.ebox + 4 * e, c, (float)b.ens[e].n, &nx, &ny, &ts), 4.0e9f);
    uint32_t y = cells;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += t;
    }
    if (lane == 31) wsi[wid] = y;
    __syncthreads();
    unsigned long long wp = 0, tot = 0;
    for (int w = 0; w < GRID_THREADS / 32; ++w) {
      if (w < wid) wp += wsi[w];
      tot += wsi[w];
    }
    const unsigned long long base = (*carry_sh) + wp + y - cells;
    if (e < b.n_ens) {
      EnsGrid g;
      const uint32_t* box = b.ebox + 4 * e;
      const bool empty = !(dec_f(box[0]) <= dec_f(box[2]));
      g.c = c;
      g.inv_c = 1.f / c;
      g.x0 = empty ? 0.f : dec_f(box[0]) - c;
      g.y0 = empty ? 0.f : dec_f(box[1]) - c;
      g.ncx = (int)nx;
      g.ncy = (int)ny;
      g.cell_base = (uint32_t)(base > 0xffffffffull ? 0xffffffffull : base);
      g.tshift = ts;
      b.grids[e] = g;
    }
    __syncthreads();
    if (threadIdx.x == 0) (*carry_sh) += tot;
    __syncthreads();
  }
  for (uint32_t e = threadIdx.x; e < b.n_ens; e += GRID_THREADS) b.eord[e] = e;
}

// Key ranges ordered by density, densest ensemble first (microbes per bounding-box area, ties by
// index). The interaction applies batches larger than the blocks' shared memory in groups of
// ensembles consecutive in key order, and a group lasts as long as its longest dependency chains,
// which grow with the density: consecutive dense ensembles share groups instead of each slowing a
// group of sparse ones. Pairs do not depend on the order (every ensemble has its own key range).
__device__ __forceinline__ void grid_ranked(const Bufs& b, float c, unsigned long long* carry_sh) {
  __shared__ float dsh[GRID_THREADS];
  __shared__ uint32_t csh[GRID_THREADS];
  __shared__ unsigned long long bsh[GRID_THREADS];
  __shared__ unsigned long long wsum[GRID_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t E = b.n_ens, e = threadIdx.x;
  float nx = 0.f, ny = 0.f, dens = -1.f;
  uint32_t cells = 0, ts = 3u;
  if (e < E) {
    const uint32_t* box = b.ebox + 4 * e;
    cells = (uint32_t)fminf(grid_dims(box, c, (float)b.ens[e].n, &nx, &ny, &ts), 4.0e9f);
    const float w = dec_f(box[2]) - dec_f(box[0]), h = dec_f(box[3]) - dec_f(box[1]);
    dens = (w >= 0.f && h >= 0.f) ? (float)b.ens[e].n / ((w + c) * (h + c)) : 0.f;  // also NaN -> 0
  }
  dsh[e] = dens;
  __syncthreads();
  uint32_t rk = e;  // threads past E keep their index (no cells)
  if (e < E) {
    rk = 0;
    for (uint32_t f = 0; f < E; ++f) {
      const float d = dsh[f];
      rk += (d > dens || (d == dens && f < e)) ? 1u : 0u;
    }
    b.eord[rk] = e;
  }
  csh[rk] = cells;  // the ranks of [0, E) are a permutation of [0, E)
  __syncthreads();
  // exclusive scan of the cells in rank order (thread j holds rank j)
  const unsigned long long own = csh[threadIdx.x];
  unsigned long long y = own;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(0xffffffffu, y, o);
    if (lane >= o) y += t;
  }
  if (lane == 31) wsum[wid] = y;
  __syncthreads();
  unsigned long long wp = 0, tot = 0;
  for (int w = 0; w < GRID_THREADS / 32; ++w) {
    if (w < wid) wp += wsum[w];
    tot += wsum[w];
  }
  bsh[threadIdx.x] = wp + y - own;
  __syncthreads();
  if (e < E) {
    const unsigned long long base = bsh[rk];
    EnsGrid g;
    const uint32_t* box = b.ebox + 4 * e;
    const bool empty = !(dec_f(box[0]) <= dec_f(box[2]));
    g.c = c;
    g.inv_c = 1.f / c;
    g.x0 = empty ? 0.f : dec_f(box[0]) - c;
    g.y0 = empty ? 0.f : dec_f(box[1]) - c;
    g.ncx = (int)nx;
    g.ncy = (int)ny;
    g.cell_base = (uint32_t)(base > 0xffffffffull ? 0xffffffffull : base);
    g.tshift = ts;
    b.grids[e] = g;
  }
  if (threadIdx.x == 0) *carry_sh = tot;
  __syncthreads();
}

// One block: grid geometry of every ensemble and the global cell numbering. If the cells would
// exceed the capacity, the cell size grows (pairs stay exact because only c >= r matters).
__global__ void __launch_bounds__(GRID_THREADS) k_grid(Bufs b, PairParams pp, Ctrl* ctrl) {
  pdl_wait();
  if (ctrl->halt) return;
  __shared__ float ws[GRID_THREADS / 32];
  __shared__ float total_sh;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float c = pp.cell_factor * (float)pp.r;
  if (!(c > 0.f)) c = 1e-3f;
  const float cap = (float)b.cells_cap;
  // 1. cell size: total cells over all ensembles must fit the capacity
  for (int attempt = 0; attempt < 16; ++attempt) {
    float t = 0.f;
    for (uint32_t e = threadIdx.x; e < b.n_ens; e += GRID_THREADS) {
      float nx, ny;
      uint32_t ts;
      t += grid_dims(b.ebox + 4 * e, c, (float)b.ens[e].n, &nx, &ny, &ts);
    }
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) ws[wid] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      float sum = 0.f;
      for (int w = 0; w < GRID_THREADS / 32; ++w) sum += ws[w];
      total_sh = sum;
    }
    __syncthreads();
    const float total = total_sh;
    __syncthreads();
    if (total <= cap * 0.999f) break;  // margin for float rounding of the sum
    c = c * sqrtf(total / cap) * 1.02f;
  }
  // 2. per-ensemble geometry and exclusive cell offsets (integers, exact)
  __shared__ uint32_t wsi[GRID_THREADS / 32];
  __shared__ unsigned long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  if (b.n_ens <= GRID_THREADS) {
    grid_ranked(b, c, &carry);
  } else {
    grid_in_order(b, c, &carry, wsi);
  }
  if (threadIdx.x == 0) {
    const unsigned long long total = carry;
    if (total > b.cells_cap) {  // only when ensembles vastly outnumber the capacity
      ctrl->ncells = b.cells_cap;
      ctrl->halt = 1;
      ctrl->halt_step = ctrl->step;
      atomicOr(&ctrl->err, (uint32_t)ERRB_OVERFLOW);
    } else {
      ctrl->ncells = (uint32_t)total;
    }
  }
}

void launch_grid(const Bufs& b, const PairParams& pp, Ctrl* ctrl, cudaStream_t st) {
  launch_dep(k_grid, dim3(1), dim3(GRID_THREADS), st, b, pp, ctrl);
}

// The grid of a context with one ensemble, as k_grid computes it: the cell size grows until the
// cells fit the capacity; `fits` is false when they still do not (the step halts).
__device__ __forceinline__ EnsGrid single_grid(const Bufs& b, const PairParams& pp, bool* fits, uint32_t* cells) {
  float c = pp.cell_factor * (float)pp.r;
  if (!(c > 0.f)) c = 1e-3f;
  const float cap = (float)b.cells_cap;
  const float n = (float)b.ens[0].n;
  float nx, ny, total = 0.f;
  uint32_t ts = 3u;
  for (int attempt = 0; attempt < 16; ++attempt) {
    total = grid_dims(b.ebox, c, n, &nx, &ny, &ts);
    if (total <= cap * 0.999f) break;
    c = c * sqrtf(total / cap) * 1.02f;
  }
  total = grid_dims(b.ebox, c, n, &nx, &ny, &ts);
  EnsGrid g;
  const bool empty = !(dec_f(b.ebox[0]) <= dec_f(b.ebox[2]));
  g.c = c;
  g.inv_c = 1.f / c;
  g.x0 = empty ? 0.f : dec_f(b.ebox[0]) - c;
  g.y0 = empty ? 0.f : dec_f(b.ebox[1]) - c;
  g.ncx = (int)nx;
  g.ncy = (int)ny;
  g.cell_base = 0;
  g.tshift = ts;
  *cells = (uint32_t)fminf(total, 4.0e9f);
  *fits = *cells <= b.cells_cap;
  return g;
}

// Cell key of every valid particle + its rank inside the cell (warp-aggregated atomics). With
// `own_grid` (one ensemble) every block computes the grid itself and block 0 publishes it for the
// later kernels, in place of a k_grid launch.
__global__ void __launch_bounds__(SLOT_BLOCK) k_keys(Bufs b, PairParams pp, Ctrl* ctrl, int use_status,
                                                     int own_grid) {
  pdl_wait();
  if (ctrl->halt) return;
  __shared__ EnsGrid g;
  __shared__ EnsInfo info;
  __shared__ int fits;
  if (threadIdx.x == 0) {
    const uint32_t e = b.block_ens[blockIdx.x];
    info = b.ens[e];
    if (own_grid) {
      bool ok;
      uint32_t cells;
      g = single_grid(b, pp, &ok, &cells);
      fits = ok ? 1 : 0;
      if (blockIdx.x == 0) {
        b.grids[0] = g;
        if (ok) {
          ctrl->ncells = cells;
        } else {
          ctrl->ncells = b.cells_cap;
          ctrl->halt = 1;
          ctrl->halt_step = ctrl->step;
          atomicOr(&ctrl->err, (uint32_t)ERRB_OVERFLOW);
        }
      }
    } else {
      g = b.grids[e];
      fits = 1;
    }
  }
  __syncthreads();
  if (!fits) return;  // block-uniform
  const uint32_t p = blockIdx.x * SLOT_BLOCK + threadIdx.x;
  bool valid = p < b.nslots;
  float x = 0.f, y = 0.f;
  if (valid) {
    valid = use_status ? (b.status[p] == STATUS_OK) : (p - info.base < info.n);
    x = b.plon[p];
    y = b.plat[p];
    valid = valid && isfinite(x) && isfinite(y);
  }
  uint32_t key = NONE;
  if (valid) {
    const float fx = fminf(fmaxf((x - g.x0) * g.inv_c, 0.f), (float)(g.ncx - 1));
    const float fy = fminf(fmaxf((y - g.y0) * g.inv_c, 0.f), (float)(g.ncy - 1));
    key = g.cell_base + cell_index(g, (uint32_t)(int)fx, (uint32_t)(int)fy);
  }
  const uint32_t peers = __match_any_sync(0xffffffffu, key);
  uint32_t rank = 0;
  if (valid) {
    const int leader = __ffs(peers) - 1;
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(b.ccount + key, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    rank = base + __popc(peers & lanemask_lt());
  }
  if (p < b.nslots) {
    b.key[p] = key;
    b.rank[p] = rank;
  }
}

void launch_keys(const Bufs& b, const PairParams& pp, Ctrl* ctrl, bool use_status, bool own_grid, cudaStream_t st) {
  if (b.nslots == 0) {
    if (own_grid) launch_grid(b, pp, ctrl, st);  // the grid and cell count are still needed
    return;
  }
  launch_dep(k_keys, dim3((b.nslots + SLOT_BLOCK - 1) / SLOT_BLOCK), dim3(SLOT_BLOCK), st, b, pp, ctrl,
             use_status ? 1 : 0, own_grid ? 1 : 0);
}

// Exclusive scan of the cell counts in two launches over SCAN_BLOCKS fixed chunks:
// (1) chunk sums, (2) per-chunk scan with the prefix of the chunk sums. The counts are zeroed
// as they are consumed, ready for the next counting pass. Each thread takes 4 consecutive cells
// (one 16-byte word: chunks are whole multiples of 4 cells, and the count and start arrays are
// separate 256-byte aligned allocations), so a pass of a 1,024-thread block covers 4,096 cells and
// the scan of a sparse multi-ensemble grid (tens of millions of cells) is bound by bandwidth
// rather than by the block's barriers.
constexpr uint32_t SCAN_CPT = 4;

__device__ __forceinline__ void chunk_of(uint32_t ncells, uint32_t* c0, uint32_t* c1) {
  const uint32_t per = ((ncells + SCAN_BLOCKS - 1) / SCAN_BLOCKS + (SCAN_CPT - 1)) & ~(SCAN_CPT - 1);
  *c0 = min(ncells, blockIdx.x * per);
  *c1 = min(ncells, *c0 + per);
}

// Cells i .. i + 3 of [.., c1) (zero past c1); i is a multiple of 4.
__device__ __forceinline__ uint4 load_cells(const uint32_t* a, uint32_t i, uint32_t c1) {
  if (i + SCAN_CPT <= c1) return *reinterpret_cast<const uint4*>(a + i);
  return make_uint4(i < c1 ? a[i] : 0u, i + 1 < c1 ? a[i + 1] : 0u, i + 2 < c1 ? a[i + 2] : 0u, 0u);
}

__device__ __forceinline__ void store_cells(uint32_t* a, uint32_t i, uint32_t c1, uint4 v) {
  if (i + SCAN_CPT <= c1) {
    *reinterpret_cast<uint4*>(a + i) = v;
    return;
  }
  if (i < c1) a[i] = v.x;
  if (i + 1 < c1) a[i + 1] = v.y;
  if (i + 2 < c1) a[i + 2] = v.z;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v) {
  __shared__ uint32_t bs[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) bs[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t t = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += bs[w];
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(1024) k_cscan_reduce(Bufs b, Ctrl* ctrl) {
  pdl_wait();
  if (ctrl->halt) return;
  uint32_t c0, c1;
  chunk_of(ctrl->ncells, &c0, &c1);
  uint32_t s = 0;
  for (uint32_t i = c0 + threadIdx.x * SCAN_CPT; i < c1; i += blockDim.x * SCAN_CPT) {
    const uint4 x = load_cells(b.ccount, i, c1);
    s += x.x + x.y + x.z + x.w;
  }
  s = block_sum(s);
  if (threadIdx.x == 0) b.csum[blockIdx.x] = s;
}

__global__ void __launch_bounds__(1024) k_cscan_down(Bufs b, Ctrl* ctrl) {
  pdl_wait();
  if (ctrl->halt) return;
  __shared__ uint32_t ws[32];
  __shared__ uint32_t carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t ncells = ctrl->ncells;
  uint32_t c0, c1;
  chunk_of(ncells, &c0, &c1);
  uint32_t pre = 0;
  for (uint32_t k = threadIdx.x; k < blockIdx.x; k += blockDim.x) pre += b.csum[k];
  pre = block_sum(pre);
  if (threadIdx.x == 0) carry = pre;
  __syncthreads();
  for (uint32_t start = c0; start < c1; start += blockDim.x * SCAN_CPT) {
    const uint32_t i = start + threadIdx.x * SCAN_CPT;
    const uint4 x = load_cells(b.ccount, i, c1);
    store_cells(b.ccount, i, c1, make_uint4(0u, 0u, 0u, 0u));
    const uint32_t t1 = x.x, t2 = t1 + x.y, t3 = t2 + x.z, t4 = t3 + x.w;  // inclusive, in the thread
    uint32_t y = t4;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += t;
    }
    if (lane == 31) ws[wid] = y;
    __syncthreads();
    if (wid == 0) {
      uint32_t w = (lane < (int)(blockDim.x >> 5)) ? ws[lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      ws[lane] = w;
    }
    __syncthreads();
    const uint32_t c = carry + (wid ? ws[wid - 1] : 0u) + y - t4;  // start of the thread's first cell
    store_cells(b.cstart, i, c1, make_uint4(c, c + t1, c + t2, c + t3));
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = c + t4;
    __syncthreads();
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    // the last chunk ends the scan: its carry (the chunks before it plus its own) is the total
    b.cstart[ncells] = carry;
    ctrl->n_valid = carry;
  }
}

void launch_cell_scan(const Bufs& b, Ctrl* ctrl, cudaStream_t st) {
  launch_dep(k_cscan_reduce, dim3(SCAN_BLOCKS), dim3(1024), st, b, ctrl);
  launch_dep(k_cscan_down, dim3(SCAN_BLOCKS), dim3(1024), st, b, ctrl);
}

// Particles into cell order: id, key, ensemble, position.
__global__ void __launch_bounds__(SLOT_BLOCK) k_scatter(Bufs b, Ctrl* ctrl) {
  pdl_wait();
  if (ctrl->halt) return;
  const uint32_t p = blockIdx.x * SLOT_BLOCK + threadIdx.x;
  if (p >= b.nslots) return;
  const uint32_t key = b.key[p];
  if (key == NONE) return;
  const uint32_t s = b.cstart[key] + b.rank[p];
  b.sid[s] = p;
  b.skey[s] = key;
  b.sens[s] = b.block_ens[blockIdx.x];
  b.spos[s] = make_float2(b.plon[p], b.plat[p]);
}

void launch_scatter(const Bufs& b, Ctrl* ctrl, cudaStream_t st) {
  if (b.nslots == 0) return;
  launch_dep(k_scatter, dim3((b.nslots + SLOT_BLOCK - 1) / SLOT_BLOCK), dim3(SLOT_BLOCK), st, b, ctrl);
}

}  // namespace lm
