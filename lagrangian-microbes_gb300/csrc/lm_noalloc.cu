// Fixed-radius pair counting that allocates no memory: lm_count_pairs_noalloc (include/lm_api.h).
//
// Who needs it: callers that must not call cudaMalloc or cudaFree, for example a host that has
// handed all device memory to its own pool allocator, a plugin whose host process forbids device
// allocation after start-up, or a latency-bound loop that cannot afford the device-wide
// synchronisation cudaFree implies. They pass device pointers for inputs and outputs; everything
// else the kernels need lives in NA_SCRATCH below, a file-scope __device__ array that every GPU
// loading this library holds until the process exits.
//
// The counting follows the same pair semantics as lm_query_pairs (cKDTree.query_pairs, inclusive
// Minkowski-p on float32 lon/lat promoted to float64) in five small launches on the caller's
// stream: bounding box + grid + clearing, cell keys, cell scan, scatter into cell order, count.
#include <cmath>
#include <mutex>

#include "lm_api.h"
#include "lm_internal.h"

namespace lm {
namespace {

constexpr uint32_t NA_MAX_POINTS = 65536;  // largest n accepted
constexpr uint32_t NA_MAX_SIDE = 256;      // cells per axis at most
constexpr uint32_t NA_MAX_CELLS = NA_MAX_SIDE * NA_MAX_SIDE;
constexpr int NA_THREADS = 256;

struct NaHeader {
  float x0, y0, inv_c;
  int ncx, ncy;
  uint32_t ncells;
  uint32_t pad[2];
};

// Scratch layout (bytes): header | counts[C+1] | starts[C+1] | key[P] | rank[P] | sid[P] | spos[P]
constexpr size_t NA_OFF_COUNTS = 256;
constexpr size_t NA_OFF_STARTS = NA_OFF_COUNTS + 4 * (NA_MAX_CELLS + 64);
constexpr size_t NA_OFF_KEY = NA_OFF_STARTS + 4 * (NA_MAX_CELLS + 64);
constexpr size_t NA_OFF_RANK = NA_OFF_KEY + 4 * NA_MAX_POINTS;
constexpr size_t NA_OFF_SID = NA_OFF_RANK + 4 * NA_MAX_POINTS;
constexpr size_t NA_OFF_SPOS = NA_OFF_SID + 4 * NA_MAX_POINTS;
constexpr size_t NA_SCRATCH_BYTES = NA_OFF_SPOS + 8 * NA_MAX_POINTS;  // about 1.8 MB

__device__ __align__(256) unsigned char NA_SCRATCH[NA_SCRATCH_BYTES];

struct NaView {
  NaHeader* h;
  uint32_t* counts;
  uint32_t* starts;
  uint32_t* key;
  uint32_t* rank;
  uint32_t* sid;
  float2* spos;
};

NaView view_of(unsigned char* base) {
  NaView v;
  v.h = reinterpret_cast<NaHeader*>(base);
  v.counts = reinterpret_cast<uint32_t*>(base + NA_OFF_COUNTS);
  v.starts = reinterpret_cast<uint32_t*>(base + NA_OFF_STARTS);
  v.key = reinterpret_cast<uint32_t*>(base + NA_OFF_KEY);
  v.rank = reinterpret_cast<uint32_t*>(base + NA_OFF_RANK);
  v.sid = reinterpret_cast<uint32_t*>(base + NA_OFF_SID);
  v.spos = reinterpret_cast<float2*>(base + NA_OFF_SPOS);
  return v;
}

// Same decision as the pair search of k_pairs.cu: float32 test outside a 2e-6 relative band of the
// radius, float64 (no FMA) inside it.
__device__ __forceinline__ bool na_within(const PairParams& pp, float2 a, float2 b) {
  const float dx = a.x - b.x, dy = a.y - b.y;
  const double ddx = __dsub_rn((double)a.x, (double)b.x), ddy = __dsub_rn((double)a.y, (double)b.y);
  if (pp.norm == 2) {
    const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    if (d2 < pp.r2f_lo) return true;
    if (d2 > pp.r2f_hi) return false;
    return __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)) <= pp.r2;
  }
  if (pp.norm == 1) {
    const float d1 = fabsf(dx) + fabsf(dy);
    if (d1 < pp.rf_lo) return true;
    if (d1 > pp.rf_hi) return false;
    return __dadd_rn(fabs(ddx), fabs(ddy)) <= pp.r;
  }
  const float di = fmaxf(fabsf(dx), fabsf(dy));
  if (di < pp.rf_lo) return true;
  if (di > pp.rf_hi) return false;
  return fmax(fabs(ddx), fabs(ddy)) <= pp.r;
}

// One block: bounding box, grid (at most NA_MAX_SIDE cells per axis), counts and output cleared.
__global__ void __launch_bounds__(1024) k_na_prepare(NaView v, const float* __restrict__ lon,
                                                     const float* __restrict__ lat, uint32_t n, double r,
                                                     unsigned long long* pairs) {
  __shared__ float red[4][32];
  float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
  for (uint32_t p = threadIdx.x; p < n; p += blockDim.x) {
    const float x = lon[p], y = lat[p];
    if (isfinite(x) && isfinite(y)) {
      mnx = fminf(mnx, x);
      mny = fminf(mny, y);
      mxx = fmaxf(mxx, x);
      mxy = fmaxf(mxy, y);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = mnx;
    red[1][threadIdx.x >> 5] = mny;
    red[2][threadIdx.x >> 5] = mxx;
    red[3][threadIdx.x >> 5] = mxy;
  }
  __syncthreads();
  __shared__ NaHeader h;
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      mnx = fminf(mnx, red[0][w]);
      mny = fminf(mny, red[1][w]);
      mxx = fmaxf(mxx, red[2][w]);
      mxy = fmaxf(mxy, red[3][w]);
    }
    if (!(mnx <= mxx)) mnx = mxx = mny = mxy = 0.f;
    const double w = (double)mxx - mnx, hh = (double)mxy - mny;
    double c = fmax(r * 1.004, fmax(w, hh) / (double)(NA_MAX_SIDE - 3));
    if (!(c > 0.0)) c = 1.0;
    h.x0 = (float)((double)mnx - c);
    h.y0 = (float)((double)mny - c);
    h.inv_c = (float)(1.0 / c);
    h.ncx = (int)fmin(floor(w / c) + 3.0, (double)NA_MAX_SIDE);
    h.ncy = (int)fmin(floor(hh / c) + 3.0, (double)NA_MAX_SIDE);
    h.ncells = (uint32_t)(h.ncx * h.ncy);
    *v.h = h;
    *pairs = 0ull;
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k <= h.ncells; k += blockDim.x) v.counts[k] = 0u;
}

__global__ void __launch_bounds__(NA_THREADS) k_na_keys(NaView v, const float* __restrict__ lon,
                                                        const float* __restrict__ lat, uint32_t n,
                                                        int32_t* __restrict__ degree) {
  const uint32_t p = blockIdx.x * NA_THREADS + threadIdx.x;
  const NaHeader h = *v.h;
  uint32_t key = NONE;
  if (p < n) {
    const float x = lon[p], y = lat[p];
    if (isfinite(x) && isfinite(y)) {
      const float fx = fminf(fmaxf((x - h.x0) * h.inv_c, 0.f), (float)(h.ncx - 1));
      const float fy = fminf(fmaxf((y - h.y0) * h.inv_c, 0.f), (float)(h.ncy - 1));
      key = (uint32_t)(int)fy * (uint32_t)h.ncx + (uint32_t)(int)fx;
    } else {
      degree[p] = 0;  // never paired
    }
  }
  const uint32_t peers = __match_any_sync(0xffffffffu, key);
  uint32_t rank = 0;
  if (key != NONE) {
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(v.counts + key, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    rank = base + __popc(peers & ((1u << lane) - 1u));
  }
  if (p < n) {
    v.key[p] = key;
    v.rank[p] = rank;
  }
}

// One block: exclusive scan of at most NA_MAX_CELLS counts; starts[ncells] = points binned.
__global__ void __launch_bounds__(1024) k_na_scan(NaView v) {
  __shared__ uint32_t ws[32];
  __shared__ uint32_t carry;
  const uint32_t nc = v.h->ncells;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t start = 0; start < nc; start += blockDim.x) {
    const uint32_t i = start + threadIdx.x;
    const uint32_t x = i < nc ? v.counts[i] : 0u;
    uint32_t y = x;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += t;
    }
    if (lane == 31) ws[wid] = y;
    __syncthreads();
    if (wid == 0) {
      uint32_t w = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      ws[lane] = w;
    }
    __syncthreads();
    const uint32_t c = carry + (wid ? ws[wid - 1] : 0u);
    if (i < nc) v.starts[i] = c + y - x;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = c + y;
    __syncthreads();
  }
  if (threadIdx.x == 0) v.starts[nc] = carry;
}

__global__ void __launch_bounds__(NA_THREADS) k_na_scatter(NaView v, const float* __restrict__ lon,
                                                           const float* __restrict__ lat, uint32_t n) {
  const uint32_t p = blockIdx.x * NA_THREADS + threadIdx.x;
  if (p >= n) return;
  const uint32_t key = v.key[p];
  if (key == NONE) return;
  const uint32_t s = v.starts[key] + v.rank[p];
  v.sid[s] = p;
  v.spos[s] = make_float2(lon[p], lat[p]);
}

// Neighbour count of every binned point; each unordered pair is added to *pairs once.
__global__ void __launch_bounds__(NA_THREADS) k_na_count(NaView v, PairParams pp, uint32_t n,
                                                         int32_t* __restrict__ degree, unsigned long long* pairs) {
  __shared__ unsigned long long tot;
  if (threadIdx.x == 0) tot = 0;
  __syncthreads();
  const NaHeader h = *v.h;
  const uint32_t nb = v.starts[h.ncells];
  const uint32_t s = blockIdx.x * NA_THREADS + threadIdx.x;
  uint32_t upper = 0;
  if (s < nb) {
    const float2 ps = v.spos[s];
    const uint32_t me = v.sid[s];
    const float fx = fminf(fmaxf((ps.x - h.x0) * h.inv_c, 0.f), (float)(h.ncx - 1));
    const float fy = fminf(fmaxf((ps.y - h.y0) * h.inv_c, 0.f), (float)(h.ncy - 1));
    const int cx = (int)fx, cy = (int)fy;
    uint32_t deg = 0;
    for (int ry = max(cy - 1, 0); ry <= min(cy + 1, h.ncy - 1); ++ry) {
      const uint32_t kl = (uint32_t)ry * h.ncx + (uint32_t)max(cx - 1, 0);
      const uint32_t kh = (uint32_t)ry * h.ncx + (uint32_t)min(cx + 1, h.ncx - 1);
      for (uint32_t t = v.starts[kl]; t < v.starts[kh + 1]; ++t) {
        if (t == s || !na_within(pp, ps, v.spos[t])) continue;
        ++deg;
        upper += v.sid[t] > me ? 1u : 0u;
      }
    }
    degree[me] = (int32_t)deg;
  }
  unsigned long long u = upper;
  for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
  if ((threadIdx.x & 31) == 0 && u) atomicAdd(&tot, u);
  __syncthreads();
  if (threadIdx.x == 0 && tot) atomicAdd(pairs, tot);
}

}  // namespace
}  // namespace lm

namespace {

int na_fail(int code, const char* msg) {
  lm::set_thread_error(msg);
  return code;
}

// Device address of NA_SCRATCH, looked up once per device with that device current. In host code
// the symbol NA_SCRATCH is only a stand-in, never a device address, so kernels get this pointer.
// The same first call also loads all five kernels (with lazy module loading a kernel is otherwise
// loaded at its first launch, and a first call with n = 0 launches only one of them), so every
// later call only enqueues launches. The address is kept for the life of the process: it belongs
// to the device's primary context and is not valid after that context is reset (cudaDeviceReset).
unsigned char* na_scratch_for(int device, int* rc) {
  static std::mutex mu;
  static unsigned char* addr[64] = {};
  *rc = LM_OK;
  if (device < 0 || device >= 64) {
    *rc = na_fail(LM_ERR_ARG, "device index out of range for lm_count_pairs_noalloc");
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, lm::NA_SCRATCH);
    cudaFuncAttributes fa;
    const void* kernels[] = {(const void*)lm::k_na_prepare, (const void*)lm::k_na_keys, (const void*)lm::k_na_scan,
                             (const void*)lm::k_na_scatter, (const void*)lm::k_na_count};
    for (const void* k : kernels)
      if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k);
    if (e != cudaSuccess) {
      cudaGetLastError();
      *rc = na_fail(LM_ERR_CUDA, cudaGetErrorString(e));
      return nullptr;
    }
    addr[device] = static_cast<unsigned char*>(p);
  }
  return addr[device];
}

}  // namespace

extern "C" int lm_count_pairs_noalloc(const float* d_lon, const float* d_lat, int64_t n, double radius, int norm,
                                      int32_t* d_degree, unsigned long long* d_pairs, uintptr_t stream) {
  using namespace lm;
  if (n < 0 || (uint64_t)n > NA_MAX_POINTS)
    return na_fail(LM_ERR_ARG, "lm_count_pairs_noalloc accepts at most 65536 points");
  if (!d_pairs || (n > 0 && (!d_lon || !d_lat || !d_degree))) return na_fail(LM_ERR_ARG, "NULL argument");
  if (!(radius >= 0) || !std::isfinite(radius)) return na_fail(LM_ERR_ARG, "radius must be finite and >= 0");
  if (norm != LM_NORM_INF && norm != LM_NORM_L1 && norm != LM_NORM_L2)
    return na_fail(LM_ERR_ARG, "norm must be 1, 2 or infinity (code 0)");
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return na_fail(LM_ERR_CUDA, cudaGetErrorString(e));
  }
  int rc = LM_OK;
  unsigned char* base = na_scratch_for(device, &rc);
  if (!base) return rc;
  const PairParams pp = make_pair_params(radius, norm, 1.0f);
  const cudaStream_t st = (cudaStream_t)stream;
  const NaView v = view_of(base);
  const uint32_t un = (uint32_t)n;
  const uint32_t blocks = (un + NA_THREADS - 1) / NA_THREADS;
  k_na_prepare<<<1, 1024, 0, st>>>(v, d_lon, d_lat, un, radius, d_pairs);
  if (un) {
    k_na_keys<<<blocks, NA_THREADS, 0, st>>>(v, d_lon, d_lat, un, d_degree);
    k_na_scan<<<1, 1024, 0, st>>>(v);
    k_na_scatter<<<blocks, NA_THREADS, 0, st>>>(v, d_lon, d_lat, un);
    k_na_count<<<blocks, NA_THREADS, 0, st>>>(v, pp, un, d_degree, d_pairs);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(LM_ERR_CUDA, cudaGetErrorString(e));
  return LM_OK;
}
