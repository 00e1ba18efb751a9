// C-ABI of the adjoint tape (declared in include/lm_api.h): RK4 advection with checkpoints every K
// steps, then the backward sweep that recomputes each segment from its checkpoint and runs the
// K6/K7 kernels of k_adjoint.cu step by step from the last step to the first. The reference has
// no differentiation; the forward is the advection of particle_advecter.py:220-223 (as lm_step).
//
// Device memory of one tape (n microbes, S steps, checkpoint interval K, C = (nx-1)(ny-1) cells):
//   uv      float2 [nt][ny][nx]            own copy of the field the forward ran on
//   ck_*    T, T, uint8 [ceil(S/K)][n]     state at steps 0, K, 2K, ... (T = float or double)
//   seg_*   T, T, uint8 [K][n]             state before every step of the segment being reversed
//   lx, ly  T [n]                          the adjoint dL/dx_m
//   rec     float4 [4n], key/k1/k2/v1/v2 uint32 [4n]  stage records and the radix-sort ping-pong
//   mkey, mcode, scode  uint32 [n]         gather form: key 2 * (cell where the step starts) + (a stage
//                                          leaves it), slots of the stages around it (sorted: scode)
//   mark [C + 1], tlist [C], tcnt [S]      gather form: target cells listed per step (stamped in mark)
//   cst/cen uint32 [4C + 1], csum float [C][3][8]     segment bounds, per-cell corner sums
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <vector>

#include "lm_api.h"
#include "lm_internal.h"

using namespace lm;

namespace {

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t cap = 0;
};

}  // namespace

struct lm_adjoint {
  lm_ctx* ctx = nullptr;
  int device = 0;
  int sms = 0;
  // field
  DBuf<float2> uv;
  FieldView fv{};
  int nt = 0, ny = 0, nx = 0;
  // the recorded run
  bool done = false;
  uint32_t n = 0;
  int n_steps = 0, K = 0, n_ck = 0;
  double dt = 0.0;
  int prec = ADJ_DS;  // working precision of the recorded run
  int prec_next = ADJ_DS;
  DBuf<AdjStep> table;
  std::vector<AdjStep> table_h;
  // positions of adj_state_bytes(prec) per element; adjoint state lx, ly of adj_lambda_bytes(prec)
  DBuf<unsigned char> x, y, ck_x, ck_y, seg_x, seg_y, lx, ly, fin_x, fin_y;
  DBuf<float> csum;
  DBuf<uint8_t> st, ck_st, seg_st;
  DBuf<float4> rec;
  DBuf<uint32_t> key, k1, k2, v1, v2, hist, hscan, bsum, cst, cen, mkey, mcode, scode, mark, tlist, tcnt;
  uint32_t* err_d = nullptr;
  uint32_t* err_h = nullptr;
};

namespace {

int afail(lm_adjoint* a, int code, const char* fmt, ...) __attribute__((format(printf, 3, 4)));
int afail(lm_adjoint* a, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (a && a->ctx) ctx_set_error(a->ctx, buf);
  else set_thread_error(buf);
  return code;
}

#define ACK(call)                                                                                    \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return afail(a, LM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));    \
  } while (0)

template <class T>
int grow(lm_adjoint* a, DBuf<T>& b, size_t need, bool zero = false) {
  if (need == 0) need = 1;
  if (b.p && b.cap >= need) return LM_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  const cudaError_t e = cudaMalloc((void**)&b.p, need * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    return afail(a, LM_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", need * sizeof(T), cudaGetErrorString(e));
  }
  b.cap = need;
  if (zero) ACK(cudaMemset(b.p, 0, need * sizeof(T)));
  return LM_OK;
}

template <class T>
void release(DBuf<T>& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
}

bool on_device(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int key_bits_for(uint32_t sent) {
  int b = 1;
  while (b < 32 && (sent >> b) != 0) ++b;
  return b;
}

int read_err(lm_adjoint* a, cudaStream_t st, uint32_t* out) {
  ACK(cudaMemcpyAsync(a->err_h, a->err_d, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  ACK(cudaStreamSynchronize(st));
  *out = *a->err_h;
  return LM_OK;
}

}  // namespace

extern "C" {

int lm_adjoint_create(lm_ctx* ctx, lm_adjoint** out) {
  if (!ctx || !out) return LM_ERR_ARG;
  *out = nullptr;
  lm_adjoint* a = new lm_adjoint();
  a->ctx = ctx;
  a->device = ctx_device(ctx);
  a->sms = ctx_sms(ctx);
  cudaError_t e;
  if ((e = cudaSetDevice(a->device)) != cudaSuccess || (e = cudaMalloc((void**)&a->err_d, sizeof(uint32_t))) != cudaSuccess ||
      (e = cudaMallocHost((void**)&a->err_h, sizeof(uint32_t))) != cudaSuccess) {
    const int r = afail(a, LM_ERR_CUDA, "adjoint tape: %s", cudaGetErrorString(e));
    lm_adjoint_destroy(a);
    return r;
  }
  *out = a;
  return LM_OK;
}

int lm_adjoint_destroy(lm_adjoint* a) {
  if (!a) return LM_OK;
  cudaSetDevice(a->device);
  if (a->ctx) cudaStreamSynchronize(ctx_stream(a->ctx));
  release(a->uv);
  release(a->table);
  release(a->x), release(a->y), release(a->ck_x), release(a->ck_y), release(a->seg_x), release(a->seg_y);
  release(a->lx), release(a->ly), release(a->fin_x), release(a->fin_y), release(a->csum), release(a->st), release(a->ck_st), release(a->seg_st);
  release(a->rec), release(a->key), release(a->k1), release(a->k2), release(a->v1), release(a->v2);
  release(a->hist), release(a->hscan), release(a->bsum), release(a->cst), release(a->cen), release(a->mkey);
  if (a->err_d) cudaFree(a->err_d);
  if (a->err_h) cudaFreeHost(a->err_h);
  delete a;
  return LM_OK;
}

int lm_adjoint_set_precision(lm_adjoint* a, int precision) {
  if (!a) return LM_ERR_ARG;
  if (precision != LM_ADJ_F32 && precision != LM_ADJ_F64 && precision != LM_ADJ_DS)
    return afail(a, LM_ERR_ARG, "precision must be LM_ADJ_F32, LM_ADJ_F64 or LM_ADJ_DS (got %d)", precision);
  a->prec_next = precision == LM_ADJ_F64 ? ADJ_F64 : precision == LM_ADJ_DS ? ADJ_DS : ADJ_F32;
  return LM_OK;
}

int lm_adjoint_forward(lm_adjoint* a, const float* u, const float* v, int nt, int ny, int nx, const double* lon,
                       const double* lat, const double* t_sec, int64_t n, const float* lon0, const float* lat0,
                       double t_start, double dt_sec, int n_steps, int checkpoint_every, float* lon_out,
                       float* lat_out) {
  if (!a) return LM_ERR_ARG;
  a->done = false;
  if (!lon || !lat || !t_sec) return afail(a, LM_ERR_ARG, "NULL axis");
  if (nt < 2 || ny < 2 || nx < 2) return afail(a, LM_ERR_ARG, "field needs nt, ny, nx >= 2 (got %d, %d, %d)", nt, ny, nx);
  if (n < 0 || 4 * n >= (int64_t)0xffffffffu) return afail(a, LM_ERR_ARG, "n = %lld out of range", (long long)n);
  if (n_steps < 1 || checkpoint_every < 1) return afail(a, LM_ERR_ARG, "need n_steps >= 1 and checkpoint_every >= 1");
  if (!(dt_sec != 0.0) || !std::isfinite(dt_sec) || !std::isfinite(t_start)) return afail(a, LM_ERR_ARG, "bad t or dt");
  const uint64_t cells = (uint64_t)(nx - 1) * (uint64_t)(ny - 1);
  if (4 * cells + 1 >= 0xffffffffull) return afail(a, LM_ERR_ARG, "field grid too large for the adjoint");
  if (!on_device(u) || !on_device(v)) return afail(a, LM_ERR_ARG, "u and v must be device pointers");
  if (n > 0 && (!on_device(lon0) || !on_device(lat0) || !on_device(lon_out) || !on_device(lat_out)))
    return afail(a, LM_ERR_ARG, "positions must be device pointers");
  double dx, dy, dT;
  if (!uniform_axis(lon, nx, &dx)) return afail(a, LM_ERR_GRID, "longitude axis is not uniform and ascending");
  if (!uniform_axis(lat, ny, &dy)) return afail(a, LM_ERR_GRID, "latitude axis is not uniform and ascending");
  if (!uniform_axis(t_sec, nt, &dT)) return afail(a, LM_ERR_GRID, "time axis is not uniform and ascending");
  {
    const double t_end = t_start + dt_sec * n_steps;
    const double lo = std::min(t_start, t_end), hi = std::max(t_start, t_end), tol = 1e-9 * dT;
    if (lo < t_sec[0] - tol || hi > t_sec[nt - 1] + tol)
      return afail(a, LM_ERR_TIME, "time window [%.9g, %.9g] s is outside the field's [%.9g, %.9g] s", lo, hi,
                   t_sec[0], t_sec[nt - 1]);
  }
  ACK(cudaSetDevice(a->device));
  cudaStream_t st = ctx_stream(a->ctx);
  const size_t fe = (size_t)nt * ny * nx;
  const uint32_t N = (uint32_t)n;
  const int n_ck = (n_steps + checkpoint_every - 1) / checkpoint_every;
  const size_t M = (size_t)4 * N;
  const int prec = a->prec_next;
  const size_t es = adj_state_bytes(prec);  // lx, ly need no more (adj_lambda_bytes)
  int r;
  if ((r = grow(a, a->uv, fe)) || (r = grow(a, a->table, (size_t)n_steps)) || (r = grow(a, a->x, es * N)) ||
      (r = grow(a, a->y, es * N)) || (r = grow(a, a->st, N)) || (r = grow(a, a->ck_x, es * n_ck * N)) ||
      (r = grow(a, a->ck_y, es * n_ck * N)) || (r = grow(a, a->ck_st, (size_t)n_ck * N)) ||
      (r = grow(a, a->seg_x, es * checkpoint_every * N)) || (r = grow(a, a->seg_y, es * checkpoint_every * N)) ||
      (r = grow(a, a->seg_st, (size_t)checkpoint_every * N)) || (r = grow(a, a->lx, es * N)) ||
      (r = grow(a, a->ly, es * N)) || (r = grow(a, a->fin_x, es * N)) || (r = grow(a, a->fin_y, es * N)) ||
      (r = grow(a, a->rec, M)) || (r = grow(a, a->key, M)) || (r = grow(a, a->mkey, N)) ||
      (r = grow(a, a->mcode, N)) || (r = grow(a, a->scode, N)) || (r = grow(a, a->mark, cells + 1)) ||
      (r = grow(a, a->tlist, cells)) || (r = grow(a, a->tcnt, (size_t)n_steps)) ||
      (r = grow(a, a->k1, M)) || (r = grow(a, a->k2, M)) || (r = grow(a, a->v1, M)) || (r = grow(a, a->v2, M)) ||
      (r = grow(a, a->hist, adj_sort_hist_len((uint32_t)M))) || (r = grow(a, a->hscan, adj_sort_hist_len((uint32_t)M))) ||
      (r = grow(a, a->bsum, SCAN_BLOCKS)) || (r = grow(a, a->cst, 4 * cells + 1, true)) ||
      (r = grow(a, a->cen, 4 * cells + 1, true)) || (r = grow(a, a->csum, cells * 24)))
    return r;
  launch_interleave(u, v, a->uv.p, fe, st);
  fill_field_view(a->fv, a->uv.p, nt, ny, nx, lon, lat, t_sec, dx, dy, dT);
  a->nt = nt;
  a->ny = ny;
  a->nx = nx;
  a->n = N;
  a->n_steps = n_steps;
  a->K = checkpoint_every;
  a->n_ck = n_ck;
  a->prec = prec;
  a->dt = dt_sec;
  ACK(cudaMemsetAsync(a->err_d, 0, sizeof(uint32_t), st));
  launch_adj_stages(a->fv, t_start, dt_sec, n_steps, a->table.p, a->err_d, st);
  a->table_h.resize(n_steps);
  ACK(cudaMemcpyAsync(a->table_h.data(), a->table.p, sizeof(AdjStep) * n_steps, cudaMemcpyDeviceToHost, st));
  uint32_t err;
  if ((r = read_err(a, st, &err))) return r;
  if (err & ERRB_TIME) return afail(a, LM_ERR_TIME, "a stage time fell outside the field's time axis");
  launch_adj_init(a->fv, prec, N, lon0, lat0, a->x.p, a->y.p, a->st.p, st);
  for (int s = 0; s < n_ck; ++s) {
    const int m0 = s * checkpoint_every, m1 = std::min(m0 + checkpoint_every, n_steps);
    if (N) {
      ACK(cudaMemcpyAsync(a->ck_x.p + es * s * N, a->x.p, es * N, cudaMemcpyDeviceToDevice, st));
      ACK(cudaMemcpyAsync(a->ck_y.p + es * s * N, a->y.p, es * N, cudaMemcpyDeviceToDevice, st));
      ACK(cudaMemcpyAsync(a->ck_st.p + (size_t)s * N, a->st.p, N, cudaMemcpyDeviceToDevice, st));
    }
    launch_adj_forward(a->fv, prec, a->table.p, m0, m1, a->dt, N, a->x.p, a->y.p, a->st.p, nullptr, nullptr, nullptr,
                       a->err_d, st);
  }
  launch_adj_final(a->fv, prec, N, a->x.p, a->y.p, lon_out, lat_out, st);
  if (N) {
    ACK(cudaMemcpyAsync(a->fin_x.p, a->x.p, es * N, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(a->fin_y.p, a->y.p, es * N, cudaMemcpyDeviceToDevice, st));
  }
  ACK(cudaGetLastError());
  if ((r = read_err(a, st, &err))) return r;
  a->done = true;
  if (err & ERRB_NAN) return afail(a, LM_ERR_NAN, "non-finite positions (frozen; their gradient passes through)");
  if (err & ERRB_OOB)
    return afail(a, LM_ERR_OUT_OF_BOUNDS, "particles left the field domain (frozen; their gradient passes through)");
  return LM_OK;
}

int lm_adjoint_backward(lm_adjoint* a, const float* g_lon, const float* g_lat, float* g_lon0, float* g_lat0,
                        float* g_u, float* g_v) {
  if (!a) return LM_ERR_ARG;
  if (!a->done) return afail(a, LM_ERR_STATE, "run lm_adjoint_forward first");
  const uint32_t N = a->n;
  if (N && (!on_device(g_lon) || !on_device(g_lat) || !on_device(g_lon0) || !on_device(g_lat0)))
    return afail(a, LM_ERR_ARG, "gradients must be device pointers");
  if (!on_device(g_u) || !on_device(g_v)) return afail(a, LM_ERR_ARG, "g_u and g_v must be device pointers");
  ACK(cudaSetDevice(a->device));
  cudaStream_t st = ctx_stream(a->ctx);
  const size_t fe = (size_t)a->nt * a->ny * a->nx;
  const uint32_t cells = (uint32_t)(a->nx - 1) * (uint32_t)(a->ny - 1);
  const uint32_t sent = 4u * cells;
  const int kb = key_bits_for(sent);
  const uint32_t M = 4u * N;
  const size_t es = adj_state_bytes(a->prec);
  const uint32_t cw = (uint32_t)(a->nx - 1), ch = (uint32_t)(a->ny - 1);
  const int kbm = key_bits_for(2u * cells);
  int r;
  // Gather form first (microbes sorted by the cell where each step starts, records gathered from
  // the 3 x 3 cells around every cell); if a stage left that neighbourhood anywhere, the whole
  // sweep is redone with the records themselves sorted by cell.
  for (int form = 0; form < 2; ++form) {
    const bool gather = form == 0;
    ACK(cudaMemsetAsync(g_u, 0, fe * sizeof(float), st));
    ACK(cudaMemsetAsync(g_v, 0, fe * sizeof(float), st));
    ACK(cudaMemsetAsync(a->err_d, 0, sizeof(uint32_t), st));
    if (gather) {  // target lists start empty, stamps at 0 (step m stamps m + 1)
      ACK(cudaMemsetAsync(a->mark.p, 0, sizeof(uint32_t) * (cells + 1), st));
      ACK(cudaMemsetAsync(a->tcnt.p, 0, sizeof(uint32_t) * a->n_steps, st));
    } else {  // the record form needs every segment bound at zero
      ACK(cudaMemsetAsync(a->cst.p, 0, sizeof(uint32_t) * (4 * (size_t)cells + 1), st));
      ACK(cudaMemsetAsync(a->cen.p, 0, sizeof(uint32_t) * (4 * (size_t)cells + 1), st));
    }
    if (N) launch_adj_seed(a->prec, N, g_lon, g_lat, a->lx.p, a->ly.p, st);
    const AdjSortBufs sb{gather ? a->mkey.p : a->key.p, a->k1.p, a->k2.p, a->v1.p, a->v2.p,
                         a->hist.p, a->hscan.p, a->bsum.p};
    for (int s = a->n_ck - 1; s >= 0 && N; --s) {
      const int m0 = s * a->K, m1 = std::min(m0 + a->K, a->n_steps);
      ACK(cudaMemcpyAsync(a->x.p, a->ck_x.p + es * s * N, es * N, cudaMemcpyDeviceToDevice, st));
      ACK(cudaMemcpyAsync(a->y.p, a->ck_y.p + es * s * N, es * N, cudaMemcpyDeviceToDevice, st));
      ACK(cudaMemcpyAsync(a->st.p, a->ck_st.p + (size_t)s * N, N, cudaMemcpyDeviceToDevice, st));
      launch_adj_forward(a->fv, a->prec, a->table.p, m0, m1, a->dt, N, a->x.p, a->y.p, a->st.p, a->seg_x.p,
                         a->seg_y.p, a->seg_st.p, a->err_d, st);
      for (int m = m1 - 1; m >= m0; --m) {
        const size_t o = (size_t)(m - m0) * N;
        const AdjStep& sg = a->table_h[m];
        launch_adj_step(a->fv, a->prec, sg, a->dt, N, a->seg_x.p + es * o, a->seg_y.p + es * o, a->seg_st.p + o,
                        a->lx.p, a->ly.p, a->rec.p, a->key.p, sent, gather ? a->mkey.p : nullptr, a->mcode.p,
                        2u * cells, a->err_d, st);
        const uint32_t *skey, *sval;
        const uint32_t stamp = (uint32_t)m + 1u;
        if (gather) {
          ACK(cudaMemsetAsync(a->cen.p, 0, sizeof(uint32_t) * 2 * cells, st));
          adj_sort(sb, N, kbm, st, &skey, &sval);
          launch_adj_cells(skey, sval, N, cw, ch, a->mcode.p, a->scode.p, a->cst.p, a->cen.p, a->mark.p, stamp,
                           a->tlist.p, a->tcnt.p + m, st);
          launch_adj_gather(cw, ch, a->tcnt.p + m, a->tlist.p, a->cst.p, a->cen.p, a->scode.p, sval, a->rec.p,
                            a->csum.p, a->sms, st);
        } else {
          adj_sort(sb, M, kb, st, &skey, &sval);
          launch_adj_bounds(skey, M, sent, a->cst.p, a->cen.p, st);
          launch_adj_reduce(cells, a->cst.p, a->cen.p, sval, a->rec.p, a->csum.p, a->sms, st);
        }
        launch_adj_nodes(a->nx, a->ny, sg, a->csum.p, gather ? a->mark.p : nullptr, stamp, g_u, g_v, st);
      }
    }
    ACK(cudaGetLastError());
    uint32_t err = 0;
    if ((r = read_err(a, st, &err))) return r;
    if (!(gather && (err & ADJ_WIDE))) break;
  }
  if (N) launch_adj_unseed(a->prec, N, a->lx.p, a->ly.p, g_lon0, g_lat0, st);
  ACK(cudaGetLastError());
  ACK(cudaStreamSynchronize(st));
  return LM_OK;
}

int lm_adjoint_final_positions(lm_adjoint* a, double* lon, double* lat) {
  if (!a) return LM_ERR_ARG;
  if (!a->done) return afail(a, LM_ERR_STATE, "run lm_adjoint_forward first");
  if (a->n && (!on_device(lon) || !on_device(lat))) return afail(a, LM_ERR_ARG, "lon and lat must be device pointers");
  ACK(cudaSetDevice(a->device));
  cudaStream_t st = ctx_stream(a->ctx);
  launch_adj_final64(a->fv, a->prec, a->n, a->fin_x.p, a->fin_y.p, lon, lat, st);
  ACK(cudaGetLastError());
  ACK(cudaStreamSynchronize(st));
  return LM_OK;
}

int lm_adjoint_cell_signature(lm_adjoint* a, unsigned long long* sig) {
  if (!a) return LM_ERR_ARG;
  if (!a->done) return afail(a, LM_ERR_STATE, "run lm_adjoint_forward first");
  if (a->n && !on_device(sig)) return afail(a, LM_ERR_ARG, "sig must be a device pointer");
  ACK(cudaSetDevice(a->device));
  cudaStream_t st = ctx_stream(a->ctx);
  launch_adj_signature(a->fv, a->prec, a->table.p, a->n_steps, a->dt, a->n, a->ck_x.p, a->ck_y.p, a->ck_st.p, sig,
                       st);
  ACK(cudaGetLastError());
  ACK(cudaStreamSynchronize(st));
  return LM_OK;
}

}  // extern "C"
