// K2: uniform-cell binning. A stable LSD radix sort of (cell key, particle id) with 8-bit digits,
// then a pass that records the first sorted index of every occupied cell and gathers positions
// into cell order. This replaces the KD-tree build of the reference, cKDTree(X)
// (interaction_simulator.py:93); the fixed-radius query that follows is K3 (k_pairs.cu).
//
// Each pass is three kernels: per-tile digit histograms, a per-digit scan over tiles (one block per
// digit, so the scan is parallel in the digit), and a stable scatter whose in-tile ranks come from
// warp-level __match_any_sync multisplit. Tiles are 256 threads x 8 keys, warp-striped so that
// loads are coalesced and the in-tile order equals the input order (stability).
#include "lm_internal.h"

namespace lm {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARPS = RS_THREADS / 32;

int sort_tiles(uint32_t n) { return (int)((n + RS_TILE - 1) / RS_TILE); }

int radix_passes(int bits) { return bits <= 8 ? 1 : (bits + 7) / 8; }

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__global__ void __launch_bounds__(RS_THREADS) k_radix_hist(const uint32_t* __restrict__ key, uint32_t n, int shift,
                                                           uint32_t* __restrict__ counts,
                                                           uint32_t* __restrict__ digit_total, uint32_t ntiles,
                                                           const Ctrl* ctrl) {
  if (ctrl->halt) return;
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * RS_TILE;
#pragma unroll
  for (int k = 0; k < RS_ITEMS; ++k) {
    uint32_t idx = base + k * RS_THREADS + threadIdx.x;
    if (idx < n) atomicAdd(&h[(key[idx] >> shift) & 255u], 1u);
  }
  __syncthreads();
  uint32_t c = h[threadIdx.x];
  counts[threadIdx.x * ntiles + blockIdx.x] = c;
  if (c) atomicAdd(&digit_total[threadIdx.x], c);
}

// Block d: global start of digit d for every tile = sum of totals of smaller digits + prefix over tiles.
__global__ void __launch_bounds__(1024) k_radix_scan(uint32_t* __restrict__ counts,
                                                     const uint32_t* __restrict__ digit_total, uint32_t ntiles,
                                                     const Ctrl* ctrl) {
  if (ctrl->halt) return;
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t carry;
  const int d = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // base = sum_{d' < d} digit_total[d']
  uint32_t v = (threadIdx.x < (unsigned)d) ? digit_total[threadIdx.x] : 0u;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) warp_sums[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += warp_sums[w];
    carry = s;
  }
  __syncthreads();
  uint32_t* row = counts + (size_t)d * ntiles;
  for (uint32_t start = 0; start < ntiles; start += blockDim.x) {
    uint32_t i = start + threadIdx.x;
    uint32_t x = (i < ntiles) ? row[i] : 0u;
    // inclusive warp scan
    uint32_t y = x;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += t;
    }
    __syncthreads();
    if (lane == 31) warp_sums[wid] = y;
    __syncthreads();
    if (wid == 0) {
      uint32_t w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      warp_sums[lane] = w;  // inclusive
    }
    __syncthreads();
    uint32_t warp_prefix = wid ? warp_sums[wid - 1] : 0u;
    uint32_t c = carry;
    if (i < ntiles) row[i] = c + warp_prefix + y - x;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = c + warp_prefix + y;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(RS_THREADS) k_radix_scatter(const uint32_t* __restrict__ kin,
                                                              const uint32_t* __restrict__ vin,
                                                              uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                              uint32_t n, int shift,
                                                              const uint32_t* __restrict__ offs, uint32_t ntiles,
                                                              const Ctrl* ctrl) {
  if (ctrl->halt) return;
  __shared__ uint32_t wc[RS_WARPS][256];
  __shared__ uint32_t toff[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < RS_WARPS; ++w) wc[w][threadIdx.x] = 0;
  toff[threadIdx.x] = offs[threadIdx.x * ntiles + blockIdx.x];
  __syncthreads();

  const uint32_t base = blockIdx.x * RS_TILE + warp * (32 * RS_ITEMS);
  uint32_t kk[RS_ITEMS], vv[RS_ITEMS], rk[RS_ITEMS];
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int k = 0; k < RS_ITEMS; ++k) {
    uint32_t idx = base + k * 32 + lane;
    bool valid = idx < n;
    kk[k] = valid ? kin[idx] : 0u;
    vv[k] = valid ? vin[idx] : 0u;
    uint32_t d = valid ? ((kk[k] >> shift) & 255u) : 256u;
    uint32_t peers = __match_any_sync(0xffffffffu, d);
    uint32_t prior = __popc(peers & lt);
    uint32_t cnt = valid ? wc[warp][d] : 0u;
    rk[k] = cnt + prior;
    __syncwarp();
    if (valid && prior == 0) wc[warp][d] = cnt + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
      uint32_t c = wc[w][threadIdx.x];
      wc[w][threadIdx.x] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < RS_ITEMS; ++k) {
    uint32_t idx = base + k * 32 + lane;
    if (idx < n) {
      uint32_t d = (kk[k] >> shift) & 255u;
      uint32_t dst = toff[d] + wc[warp][d] + rk[k];
      kout[dst] = kk[k];
      vout[dst] = vv[k];
    }
  }
}

void launch_radix_hist(const uint32_t* key, uint32_t n, int shift, SortScratch& s, uint32_t* digit_total, Ctrl* ctrl,
                       cudaStream_t st) {
  uint32_t ntiles = (uint32_t)sort_tiles(n);
  k_radix_hist<<<ntiles, RS_THREADS, 0, st>>>(key, n, shift, s.counts, digit_total, ntiles, ctrl);
}

void launch_radix_scan(uint32_t n, SortScratch& s, const uint32_t* digit_total, Ctrl* ctrl, cudaStream_t st) {
  k_radix_scan<<<256, 1024, 0, st>>>(s.counts, digit_total, (uint32_t)sort_tiles(n), ctrl);
}

void launch_radix_scatter(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                          int shift, SortScratch& s, Ctrl* ctrl, cudaStream_t st) {
  uint32_t ntiles = (uint32_t)sort_tiles(n);
  k_radix_scatter<<<ntiles, RS_THREADS, 0, st>>>(kin, vin, kout, vout, n, shift, s.counts, ntiles, ctrl);
}

// Cell starts + gather of positions into cell order + count of valid (binned) particles.
__global__ void k_cells(const uint32_t* __restrict__ key, const uint32_t* __restrict__ id,
                        const float* __restrict__ plon, const float* __restrict__ plat, float2* __restrict__ spos,
                        uint32_t* __restrict__ cell_start, Ctrl* ctrl, uint32_t n, uint32_t invalid) {
  if (ctrl->halt) return;
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  uint32_t k = key[s];
  uint32_t prev = s ? key[s - 1] : NONE;
  if (k != invalid) {
    if (k != prev) cell_start[k] = s;
    const uint32_t p = id[s];
    spos[s] = make_float2(plon[p], plat[p]);
    if (s == n - 1) ctrl->n_valid = n;
  } else if (prev != invalid) {
    ctrl->n_valid = s;
  }
}

void launch_cells(const uint32_t* key, const uint32_t* id, const float* plon, const float* plat, float2* spos,
                  uint32_t* cell_start, Ctrl* ctrl, uint32_t n, uint32_t invalid_key, cudaStream_t st) {
  if (n == 0) return;
  k_cells<<<(n + 255) / 256, 256, 0, st>>>(key, id, plon, plat, spos, cell_start, ctrl, n, invalid_key);
}

}  // namespace lm
