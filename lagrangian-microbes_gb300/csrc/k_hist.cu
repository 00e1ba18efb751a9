// Pairwise great-circle distance histogram (lm_distance_histogram, include/lm_api.h).
//
// The reference's sandbox computes, for the microbes of one species, the distance of every
// unordered pair with its float32 haversine formula and counts it in a log bin
// (sandbox/pairwise_distance_histogram_distributed.jl:35-46 haversine_distance32, :56-66 the
// per-point loop and the bin round(10 log10(max(1, d))), :68-76 the sum over points, :133-147 one
// histogram per species; sandbox/pairwise_distance_histogram_gpu.jl:14-43 a CUDA tiling of the
// same pairs whose histogram update was left unwritten). Here all pairs of every segment
// (species) are counted in one persistent launch:
//
//   * work items are the tiles (I, J), I <= J, of 256 x 256 points of a segment, enumerated
//     triangle by triangle; a block loads tile J (latitude, longitude, cos(latitude)) into shared
//     memory and thread t takes point I * 256 + t against it (on the diagonal only j > i);
//   * the distance follows haversine_distance32 operation by operation in float32 (divisions and
//     products rounded as written, no fused multiply-add), with CUDA's sinpif / cospif / asinf /
//     log10f for the functions;
//   * bin = round-half-even(10 log10(max(1, d))) (Julia's round); bins at or past `bins` go to an
//     overflow count (the reference indexes past its array there);
//   * counts go to four copies per warp of a shared-memory histogram (lanes l and l + 4 share a
//     copy, so same-bin lanes mostly hit different words) and are added to 64-bit global counts
//     at segment changes, every DH_FLUSH items and at the end.
//
// The kernel is bound by instruction issue (no memory traffic beyond the tile loads), so most
// pairs take a shorter route to the same bin: the distance from odd polynomials for sin and asin,
// a reciprocal square root and the hardware log2 (dh_fast), valid for 1.5 m <= d, asin argument
// <= 0.25 (d <= ~3,200 km) and |dlon| <= 180 degrees. Its 10 log10 d differs from the reference
// chain's by a few 1e-5 at most; only when it lies farther than DH_MARGIN = 1e-3 from a bin
// boundary is its rounding taken, otherwise (and outside that range) the reference chain decides,
// so every bin is the reference chain's. LM_HIST_EXACT=1 in the environment makes every pair take
// the reference chain (the tests compare the two).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "lm_api.h"
#include "lm_internal.h"

namespace lm {
namespace {

constexpr int DH_THREADS = 256;                // points per tile, threads per block
constexpr int DH_WARPS = DH_THREADS / 32;
constexpr int DH_COPIES = 4;                   // histogram copies per warp
constexpr int DH_BINS_MAX = 256;
constexpr uint32_t DH_FLUSH = 16384;           // items between flushes: < 2^32 counts per word

struct DhSeg {
  unsigned long long item0;  // first work item of the segment
  uint32_t start, n;         // first point, points
};

__global__ void k_dh_prep(const float* __restrict__ lat, uint32_t n, float* __restrict__ cs) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cs[i] = cospif(__fdiv_rn(lat[i], 180.0f));
}

// haversine_distance32 (lat, lon in degrees, c = cospi(lat / 180)), then the bin.
__device__ __forceinline__ int dh_bin(float la1, float lo1, float c1, float la2, float lo2, float c2, float R) {
  const float dlat = __fsub_rn(la2, la1), dlon = __fsub_rn(lo2, lo1);
  const float d1 = sinpif(__fdiv_rn(dlat, 360.0f));
  const float d2 = sinpif(__fdiv_rn(dlon, 360.0f));
  const float t = __fmul_rn(__fmul_rn(__fmul_rn(d2, d2), c1), c2);
  const float a = __fadd_rn(__fmul_rn(d1, d1), t);
  const float c = __fmul_rn(2.0f, asinf(fminf(1.0f, __fsqrt_rn(a))));
  const float d = __fmul_rn(R, c);
  return (int)rintf(__fmul_rn(10.0f, log10f(fmaxf(1.0f, d))));
}

constexpr float DH_MARGIN = 1e-3f;
constexpr float DH_PI_360 = 8.72664625997164788e-3f;  // pi / 360
constexpr float DH_TEN_LOG10_2 = 3.01029995663981195f;  // 10 log10(2)

// sin x for |x| <= pi / 2: Taylor series to x^11 (truncation below 6e-8 relative there).
__device__ __forceinline__ float dh_sin(float x) {
  const float z = x * x;
  float p = -2.50521083854417188e-8f;  // -1 / 11!
  p = fmaf(p, z, 2.75573192239858907e-6f);  // 1 / 9!
  p = fmaf(p, z, -1.98412698412698413e-4f);  // -1 / 7!
  p = fmaf(p, z, 8.33333333333333333e-3f);   // 1 / 5!
  p = fmaf(p, z, -1.66666666666666667e-1f);  // -1 / 3!
  return fmaf(x * z, p, x);
}

// asin s for 0 <= s <= 0.25: Taylor series to s^11 (truncation below 1e-9 relative there).
__device__ __forceinline__ float dh_asin(float s) {
  const float z = s * s;
  float p = 2.23721590909090909e-2f;  // 63 / 2816
  p = fmaf(p, z, 3.03819444444444444e-2f);  // 35 / 1152
  p = fmaf(p, z, 4.46428571428571429e-2f);  // 5 / 112
  p = fmaf(p, z, 7.5e-2f);                  // 3 / 40
  p = fmaf(p, z, 1.66666666666666667e-1f);  // 1 / 6
  return fmaf(s * z, p, s);
}

// 10 log10 d of the pair by the short route; false when the pair is outside its range.
__device__ __forceinline__ bool dh_fast(float la1, float lo1, float c1, float la2, float lo2, float c2, float R,
                                        float* x) {
  const float dlat = la2 - la1, dlon = lo2 - lo1;
  const float d1 = dh_sin(dlat * DH_PI_360), d2 = dh_sin(dlon * DH_PI_360);
  const float a = fmaf(d1, d1, d2 * d2 * c1 * c2);
  const float s = a * rsqrtf(a);  // NaN for a = 0: the reference chain takes it
  const float d = 2.0f * R * dh_asin(s);
  *x = DH_TEN_LOG10_2 * __log2f(d);
  return fabsf(dlon) <= 180.0f && s <= 0.25f && d >= 1.5f;
}

__device__ __forceinline__ int dh_pair_bin(float la1, float lo1, float c1, float la2, float lo2, float c2, float R,
                                           int exact) {
  float x;
  if (!exact && dh_fast(la1, lo1, c1, la2, lo2, c2, R, &x)) {
    const float k = rintf(x);
    if (fabsf(x - k) < 0.5f - DH_MARGIN) return (int)k;
  }
  return dh_bin(la1, lo1, c1, la2, lo2, c2, R);
}

__device__ void dh_flush(uint32_t* hist, int nb, unsigned long long* out) {
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += DH_THREADS) {
    unsigned long long s = 0;
    for (int w = 0; w < DH_WARPS; ++w)
      for (int q = 0; q < DH_COPIES; ++q) {
        uint32_t* p = hist + ((size_t)w * nb + b) * DH_COPIES + q;
        s += *p;
        *p = 0;
      }
    if (s) atomicAdd(out + b, s);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(DH_THREADS) k_dist_hist(const float* __restrict__ lat, const float* __restrict__ lon,
                                                          const float* __restrict__ cs,
                                                          const DhSeg* __restrict__ segs, int n_seg,
                                                          unsigned long long n_items, int bins, float R, int exact,
                                                          unsigned long long* __restrict__ counts) {
  __shared__ float tla[DH_THREADS], tlo[DH_THREADS], tc[DH_THREADS];
  extern __shared__ uint32_t hist[];  // [warp][bin][copy], bin = bins is the overflow
  const int nb = bins + 1;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  for (int q = threadIdx.x; q < DH_WARPS * nb * DH_COPIES; q += DH_THREADS) hist[q] = 0;
  __syncthreads();
  uint32_t* mine = hist + (size_t)warp * nb * DH_COPIES + (lane & (DH_COPIES - 1));
  int cur = -1;
  uint32_t since = 0;
  for (unsigned long long w = blockIdx.x; w < n_items; w += gridDim.x) {
    int sg = cur < 0 ? 0 : cur;  // items come in segment order
    while (sg + 1 < n_seg && w >= segs[sg + 1].item0) ++sg;
    if (sg != cur || since >= DH_FLUSH) {  // block-uniform
      if (cur >= 0) dh_flush(hist, nb, counts + (size_t)cur * nb);
      cur = sg;
      since = 0;
    }
    const DhSeg S = segs[sg];
    // item t of the segment is tile pair (I, J) with J (J + 1) / 2 <= t < (J + 1) (J + 2) / 2
    const unsigned long long t = w - S.item0;
    unsigned long long J = (unsigned long long)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (J * (J + 1) / 2 > t) --J;
    while ((J + 1) * (J + 2) / 2 <= t) ++J;
    const uint32_t I = (uint32_t)(t - J * (J + 1) / 2);
    const uint32_t j0 = (uint32_t)J * DH_THREADS;
    const uint32_t jn = min((uint32_t)DH_THREADS, S.n - j0);
    __syncthreads();  // the previous tile is no longer read
    if (threadIdx.x < jn) {
      const uint32_t g = S.start + j0 + threadIdx.x;
      tla[threadIdx.x] = lat[g];
      tlo[threadIdx.x] = lon[g];
      tc[threadIdx.x] = cs[g];
    }
    __syncthreads();
    const uint32_t i = I * DH_THREADS + threadIdx.x;
    if (i < S.n) {
      const uint32_t g = S.start + i;
      const float la = lat[g], lo = lon[g], c = cs[g];
      const uint32_t js = (I == (uint32_t)J) ? threadIdx.x + 1 : 0u;  // j > i on the diagonal
#pragma unroll 4
      for (uint32_t jj = js; jj < jn; ++jj) {
        const int b = min(dh_pair_bin(la, lo, c, tla[jj], tlo[jj], tc[jj], R, exact), bins);
        atomicAdd(mine + b * DH_COPIES, 1u);
      }
    }
    ++since;
  }
  if (cur >= 0) dh_flush(hist, nb, counts + (size_t)cur * nb);
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  cudaStream_t st = nullptr;
  ~DevBuf() {
    if (p) cudaFreeAsync(p, st);
  }
  cudaError_t alloc(size_t n, cudaStream_t s) {
    st = s;
    return cudaMallocAsync((void**)&p, n * sizeof(T) + 16, s);
  }
};

int dh_fail(lm_ctx* c, int code, const char* msg) {
  if (c) ctx_set_error(c, msg);
  return code;
}

int dh_cuda(lm_ctx* c, cudaError_t e) {
  if (e == cudaSuccess) return LM_OK;
  cudaGetLastError();
  return dh_fail(c, e == cudaErrorMemoryAllocation ? LM_ERR_OOM : LM_ERR_CUDA, cudaGetErrorString(e));
}

}  // namespace
}  // namespace lm

using namespace lm;

extern "C" int lm_distance_histogram(lm_ctx* c, const float* lat, const float* lon, int64_t n, const int64_t* seg,
                                     int n_seg, int bins, double radius_m, uint64_t* counts) {
  if (!c) return LM_ERR_ARG;
  if (!counts || (n > 0 && (!lat || !lon))) return dh_fail(c, LM_ERR_ARG, "NULL argument");
  if (n < 0 || n > 0x7fffff00) return dh_fail(c, LM_ERR_ARG, "point count out of range");
  if (bins < 1 || bins > DH_BINS_MAX) return dh_fail(c, LM_ERR_ARG, "bins must be in [1, 256]");
  if (!(radius_m > 0.0) || !std::isfinite(radius_m)) return dh_fail(c, LM_ERR_ARG, "radius must be finite and > 0");
  if (n_seg < 1 || (n_seg > 1 && !seg)) return dh_fail(c, LM_ERR_ARG, "n_seg >= 1 and seg offsets are required");
  std::vector<int64_t> off(n_seg + 1);
  if (seg) {
    for (int s = 0; s <= n_seg; ++s) off[s] = seg[s];
  } else {
    off[0] = 0;
    off[1] = n;
  }
  if (off[0] != 0 || off[n_seg] != n) return dh_fail(c, LM_ERR_ARG, "segments must start at 0 and end at n");
  for (int s = 0; s < n_seg; ++s)
    if (off[s + 1] < off[s]) return dh_fail(c, LM_ERR_ARG, "segment offsets must not decrease");
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(lat[i]) || !std::isfinite(lon[i])) return dh_fail(c, LM_ERR_NAN, "non-finite coordinates");
  const size_t nb = (size_t)bins + 1;
  for (size_t q = 0; q < nb * n_seg; ++q) counts[q] = 0;
  std::vector<DhSeg> hs(n_seg);
  unsigned long long items = 0;
  for (int s = 0; s < n_seg; ++s) {
    const uint64_t m = (uint64_t)(off[s + 1] - off[s]);
    const uint64_t nt = (m + DH_THREADS - 1) / DH_THREADS;
    hs[s].item0 = items;
    hs[s].start = (uint32_t)off[s];
    hs[s].n = (uint32_t)m;
    items += nt * (nt + 1) / 2;
  }
  if (items == 0) return LM_OK;
  int r;
  if ((r = dh_cuda(c, cudaSetDevice(ctx_device(c))))) return r;
  cudaStream_t st = ctx_stream(c);
  {
    DevBuf<float> dlat, dlon, dcs;
    DevBuf<DhSeg> dseg;
    DevBuf<unsigned long long> dcnt;
    if ((r = dh_cuda(c, dlat.alloc(n, st))) || (r = dh_cuda(c, dlon.alloc(n, st))) ||
        (r = dh_cuda(c, dcs.alloc(n, st))) || (r = dh_cuda(c, dseg.alloc(n_seg, st))) ||
        (r = dh_cuda(c, dcnt.alloc(nb * n_seg, st))))
      return r;
    if ((r = dh_cuda(c, cudaMemcpyAsync(dlat.p, lat, n * sizeof(float), cudaMemcpyHostToDevice, st))) ||
        (r = dh_cuda(c, cudaMemcpyAsync(dlon.p, lon, n * sizeof(float), cudaMemcpyHostToDevice, st))) ||
        (r = dh_cuda(c, cudaMemcpyAsync(dseg.p, hs.data(), n_seg * sizeof(DhSeg), cudaMemcpyHostToDevice, st))) ||
        (r = dh_cuda(c, cudaMemsetAsync(dcnt.p, 0, nb * n_seg * sizeof(unsigned long long), st))))
      return r;
    k_dh_prep<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dlat.p, (uint32_t)n, dcs.p);
    const size_t smem = (size_t)DH_WARPS * nb * DH_COPIES * sizeof(uint32_t);
    int per_sm = 0;
    if ((r = dh_cuda(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dist_hist, DH_THREADS, smem))))
      return r;
    const unsigned long long cap = (unsigned long long)std::max(per_sm, 1) * (unsigned long long)std::max(ctx_sms(c), 1);
    const unsigned blocks = (unsigned)std::min(items, cap);
    const char* ex = std::getenv("LM_HIST_EXACT");
    const int exact = (ex && ex[0] == '1') ? 1 : 0;
    k_dist_hist<<<blocks, DH_THREADS, smem, st>>>(dlat.p, dlon.p, dcs.p, dseg.p, n_seg, items, bins, (float)radius_m,
                                                   exact,
                                                   dcnt.p);
    if ((r = dh_cuda(c, cudaGetLastError()))) return r;
    if ((r = dh_cuda(c, cudaMemcpyAsync(counts, dcnt.p, nb * n_seg * sizeof(unsigned long long),
                                        cudaMemcpyDeviceToHost, st))))
      return r;
  }
  return dh_cuda(c, cudaStreamSynchronize(st));
}
