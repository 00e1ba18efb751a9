// K6 + K7: adjoint of the RK4 advection. The reference has no differentiation; the forward scheme
// is the one of K1 (particle_advecter.py:177-187, 220-223), shared through lm_field.cuh so that
// recomputed trajectories are bit-identical to lm_step's.
//
// K6 k_adj_step: one thread per microbe takes x_m (recomputed from a checkpoint) and the adjoint
// lambda_{m+1} = dL/dx_{m+1}, and returns lambda_m by running the four RK4 stages forward and
// their Jacobians backward:
//   x' = x + dt/6 (k1 + 2 k2 + 2 k3 + k4),  k_s = f(t_s, x_s),  f = (U / (M cos lat), V / M),
//   with U, V bilinear in (lon, lat), linear in time, M = 1852 * 60 m per degree.
// For every stage it emits a record (a, b, dL/dU_s, dL/dV_s) keyed by (field cell, stage time):
// the stage's bilinear fractions inside its cell and its adjoint in field units.
//
// K7, the deterministic segmented reduction: the 4 N records of a step are put in (cell, stage
// time, record id) order by a stable LSD radix sort (block-local ranks from warp match masks, no
// atomics on positions); one warp per cell then sums each (cell, stage time) segment into the four
// corner weights (fixed lane order, Neumaier-compensated float32 lane sums, fixed-shape warp tree);
// a node pass adds, for every grid node, the four cells around it in a fixed order and spreads the
// three stage times onto the field's frames with the linear-in-time weights. No float atomics: the
// gradient is bit-identical from run to run.
#include <algorithm>

#include "lm_field.cuh"
#include "lm_internal.h"

namespace lm {

// ---------------------------------------------------------------- stage table, recompute

// Stage brackets of step m at t_m = t_start + m * dt (the arithmetic of k_step_begin).
__global__ void k_adj_stages(FieldView f, double t_start, double dt, int n_steps, AdjStep* table, uint32_t* err) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n_steps) return;
  const double t0 = t_start + (double)m * dt;
  const double ts[3] = {t0, t0 + 0.5 * dt, t0 + dt};
  AdjStep s;
  int ok = 1;
  for (int k = 0; k < 3; ++k) {
    const Stage sg = stage_at(f, ts[k]);
    s.k[k] = sg.k;
    s.w[k] = sg.w;
    // the float64 weight of the same bracket (stage_at rounds it to float32)
    const double fk = (ts[k] - f.t0) / f.dT;
    s.wd[k] = sg.w == 0.f ? 0.0 : fmin(fmax(fk - (double)sg.k, 0.0), 1.0);
    ok = ok && sg.ok;
  }
  table[m] = s;
  if (!ok) atomicOr(err, (uint32_t)ERRB_TIME);
}

// Geometry of the offset frame in the working precision T. The float32 instance is the forward
// engine's (FieldView's float fields); the float64 one is the same grid in float64.
template <class T>
struct Geo;
template <>
struct Geo<float> {
  float gx0, gy0, inv_dx, inv_dy, max_fx, max_fy, org_lat;
  __device__ explicit Geo(const FieldView& f)
      : gx0(f.gx0), gy0(f.gy0), inv_dx(f.inv_dx), inv_dy(f.inv_dy), max_fx(f.max_fx), max_fy(f.max_fy),
        org_lat(f.org_lat) {}
};
template <>
struct Geo<double> {
  double gx0, gy0, inv_dx, inv_dy, max_fx, max_fy, org_lat;
  __device__ explicit Geo(const FieldView& f)
      : gx0(f.gx0d), gy0(f.gy0d), inv_dx(f.inv_dxd), inv_dy(f.inv_dyd), max_fx(f.max_fx), max_fy(f.max_fy),
        org_lat((double)f.org_lat) {}
};
__device__ __forceinline__ float cospi_t(float x) { return cospif(x); }
__device__ __forceinline__ double cospi_t(double x) { return cospi(x); }
__device__ __forceinline__ float sinpi_t(float x) { return sinpif(x); }
__device__ __forceinline__ double sinpi_t(double x) { return sinpi(x); }
template <class T>
__device__ __forceinline__ T stage_w(const AdjStep& s, int g);
template <>
__device__ __forceinline__ float stage_w<float>(const AdjStep& s, int g) { return s.w[g]; }
template <>
__device__ __forceinline__ double stage_w<double>(const AdjStep& s, int g) { return s.wd[g]; }

// Absolute float32 positions -> offsets from the field's float32 origin (exact in float64), status.
template <class T>
__global__ void k_adj_init(FieldView f, uint32_t n, const float* __restrict__ lon, const float* __restrict__ lat,
                           T* __restrict__ x, T* __restrict__ y, uint8_t* __restrict__ st) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float a = lon[p], b = lat[p];
  x[p] = (T)((double)a - (double)f.org_lon);
  y[p] = (T)((double)b - (double)f.org_lat);
  st[p] = (isfinite(a) && isfinite(b)) ? STATUS_OK : STATUS_NAN;
}

template <class T>
__global__ void k_adj_final(FieldView f, uint32_t n, const T* __restrict__ x, const T* __restrict__ y,
                            float* __restrict__ lon, float* __restrict__ lat) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (sizeof(T) == sizeof(float)) {  // the engine's rounding of the recorded position
    lon[p] = __fadd_rn(f.org_lon, (float)x[p]);
    lat[p] = __fadd_rn(f.org_lat, (float)y[p]);
  } else {
    lon[p] = (float)((double)f.org_lon + (double)x[p]);
    lat[p] = (float)((double)f.org_lat + (double)y[p]);
  }
}

// Final positions in float64 (absolute degrees) from the T-typed state.
template <class T>
__global__ void k_adj_final64(FieldView f, uint32_t n, const T* __restrict__ x, const T* __restrict__ y,
                              double* __restrict__ lon, double* __restrict__ lat) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  lon[p] = (double)f.org_lon + (double)x[p];
  lat[p] = (double)f.org_lat + (double)y[p];
}

// dL/dx of the final positions (float32) into the T-typed adjoint state, and back out at the end.
template <class T>
__global__ void k_adj_convert_in(uint32_t n, const float* __restrict__ gx, const float* __restrict__ gy,
                                 T* __restrict__ lx, T* __restrict__ ly) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  lx[p] = (T)gx[p];
  ly[p] = (T)gy[p];
}
template <class T>
__global__ void k_adj_convert_out(uint32_t n, const T* __restrict__ lx, const T* __restrict__ ly,
                                  float* __restrict__ gx, float* __restrict__ gy) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  gx[p] = (float)lx[p];
  gy[p] = (float)ly[p];
}

// ---------------------------------------------------------------- K6: one backward step

// Velocity and its Jacobian w.r.t. the offset position. For T = float the value is computed with
// exactly the arithmetic of velocity() so that the recomputed stage positions are the forward's.
template <class T>
struct VelJac {
  T flon, flat;                          // deg/s
  T dlon_dx, dlon_dy, dlat_dx, dlat_dy;  // 1/s
  uint32_t cell;                         // j * (nx - 1) + i
  T a, b;                                // bilinear fractions
  T inv_mc;                              // d flon / d U = 1 / (M cos lat)
};

// Velocity and Jacobian in cell (i, j) at bilinear fractions (a, b); `lat` is the absolute latitude.
template <class T>
__device__ __forceinline__ void vel_jac_at(const FieldView& f, int k, T w, int i, int j, T a, T b, T lat, T inv_dx,
                                           T inv_dy, VelJac<T>& r) {
  const float2* p = f.uv + ((size_t)k * f.ny + j) * f.nx + i;
  float2 q00 = __ldg(p), q01 = __ldg(p + 1), q10 = __ldg(p + f.nx), q11 = __ldg(p + f.nx + 1);
  const T w00 = (T(1) - a) * (T(1) - b), w01 = a * (T(1) - b), w10 = (T(1) - a) * b, w11 = a * b;
  T u = w00 * (T)q00.x + w01 * (T)q01.x + w10 * (T)q10.x + w11 * (T)q11.x;
  T v = w00 * (T)q00.y + w01 * (T)q01.y + w10 * (T)q10.y + w11 * (T)q11.y;
  T ua = (T(1) - b) * ((T)q01.x - (T)q00.x) + b * ((T)q11.x - (T)q10.x);
  T ub = (T(1) - a) * ((T)q10.x - (T)q00.x) + a * ((T)q11.x - (T)q01.x);
  T va = (T(1) - b) * ((T)q01.y - (T)q00.y) + b * ((T)q11.y - (T)q10.y);
  T vb = (T(1) - a) * ((T)q10.y - (T)q00.y) + a * ((T)q11.y - (T)q01.y);
  if (w != T(0)) {
    p += (size_t)f.nx * f.ny;
    q00 = __ldg(p); q01 = __ldg(p + 1); q10 = __ldg(p + f.nx); q11 = __ldg(p + f.nx + 1);
    const T u1 = w00 * (T)q00.x + w01 * (T)q01.x + w10 * (T)q10.x + w11 * (T)q11.x;
    const T v1 = w00 * (T)q00.y + w01 * (T)q01.y + w10 * (T)q10.y + w11 * (T)q11.y;
    u = u + w * (u1 - u);
    v = v + w * (v1 - v);
    ua = ua + w * (((T(1) - b) * ((T)q01.x - (T)q00.x) + b * ((T)q11.x - (T)q10.x)) - ua);
    ub = ub + w * (((T(1) - a) * ((T)q10.x - (T)q00.x) + a * ((T)q11.x - (T)q01.x)) - ub);
    va = va + w * (((T(1) - b) * ((T)q01.y - (T)q00.y) + b * ((T)q11.y - (T)q10.y)) - va);
    vb = vb + w * (((T(1) - a) * ((T)q10.y - (T)q00.y) + a * ((T)q11.y - (T)q01.y)) - vb);
  }
  const T c = cospi_t(lat * (T(1) / T(180)));
  const T sn = sinpi_t(lat * (T(1) / T(180)));
  const T M = (T)M_PER_DEG;
  r.flon = u / (M * c);
  r.flat = v * (T(1) / M);
  r.inv_mc = T(1) / (M * c);
  // d/dlat (1 / cos(lat)) = tan(lat) / cos(lat) * pi / 180 per degree
  r.dlon_dx = ua * inv_dx * r.inv_mc;
  r.dlon_dy = ub * inv_dy * r.inv_mc + r.flon * (sn / c) * (T)0.017453292519943295;
  r.dlat_dx = va * inv_dx * (T(1) / M);
  r.dlat_dy = vb * inv_dy * (T(1) / M);
  r.cell = (uint32_t)j * (uint32_t)(f.nx - 1) + (uint32_t)i;
  r.a = a;
  r.b = b;
}

template <class T>
__device__ __forceinline__ bool vel_jac(const FieldView& f, const Geo<T>& g, int k, T w, T xo, T yo, VelJac<T>& r) {
  const T fx = (xo - g.gx0) * g.inv_dx;
  const T fy = (yo - g.gy0) * g.inv_dy;
  if (!(fx >= T(0) && fx <= g.max_fx && fy >= T(0) && fy <= g.max_fy)) return false;
  const int i = min((int)fx, f.nx - 2);
  const int j = min((int)fy, f.ny - 2);
  vel_jac_at<T>(f, k, w, i, j, fx - (T)i, fy - (T)j, g.org_lat + yo, g.inv_dx, g.inv_dy, r);
  return true;
}

// One RK4 step in precision T. For T = float it is rk4_step, the engine's own arithmetic.
template <class T>
__device__ __forceinline__ bool rk4_t(const FieldView& f, const Geo<T>& g, const AdjStep& s, T dt, T x, T y, T& nx,
                                      T& ny);
template <>
__device__ __forceinline__ bool rk4_t<float>(const FieldView& f, const Geo<float>&, const AdjStep& s, float dt, float x,
                                             float y, float& nx, float& ny) {
  const Stage sh[3] = {{s.k[0], s.w[0], 1}, {s.k[1], s.w[1], 1}, {s.k[2], s.w[2], 1}};
  return rk4_step(f, f.uv, sh, dt, x, y, nx, ny);
}
template <>
__device__ __forceinline__ bool rk4_t<double>(const FieldView& f, const Geo<double>& g, const AdjStep& s, double dt,
                                              double x, double y, double& nx, double& ny) {
  VelJac<double> J1, J2, J3, J4;
  bool ok = vel_jac(f, g, s.k[0], s.wd[0], x, y, J1);
  ok = ok && vel_jac(f, g, s.k[1], s.wd[1], x + 0.5 * dt * J1.flon, y + 0.5 * dt * J1.flat, J2);
  ok = ok && vel_jac(f, g, s.k[1], s.wd[1], x + 0.5 * dt * J2.flon, y + 0.5 * dt * J2.flat, J3);
  ok = ok && vel_jac(f, g, s.k[2], s.wd[2], x + dt * J3.flon, y + dt * J3.flat, J4);
  if (!ok) return false;
  nx = x + (J1.flon + 2.0 * J2.flon + 2.0 * J3.flon + J4.flon) * (dt * (1.0 / 6.0));
  ny = y + (J1.flat + 2.0 * J2.flat + 2.0 * J3.flat + J4.flat) * (dt * (1.0 / 6.0));
  return true;
}

// Steps [m0, m1) of every microbe in registers, the forward's freezing rules. With rec_* set, the
// state before every step is stored ([m - m0][n]) for the backward sweep.
template <class T>
__global__ void __launch_bounds__(256) k_adj_forward(FieldView f, const AdjStep* __restrict__ table, int m0, int m1,
                                                     T dt, uint32_t n, T* __restrict__ xs, T* __restrict__ ys,
                                                     uint8_t* __restrict__ sts, T* __restrict__ rec_x,
                                                     T* __restrict__ rec_y, uint8_t* __restrict__ rec_st,
                                                     uint32_t* err) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const Geo<T> g(f);
  T x = xs[p], y = ys[p];
  uint8_t st = sts[p];
  uint32_t bits = 0;
  for (int m = m0; m < m1; ++m) {
    if (rec_x) {
      const size_t o = (size_t)(m - m0) * n + p;
      rec_x[o] = x;
      rec_y[o] = y;
      rec_st[o] = st;
    }
    if (st != STATUS_OK) continue;
    const AdjStep s = table[m];
    T nx, ny;
    if (rk4_t<T>(f, g, s, dt, x, y, nx, ny)) {
      if (isfinite(nx) && isfinite(ny)) {
        x = nx;
        y = ny;
      } else {
        st = STATUS_NAN;
        bits |= ERRB_NAN;
      }
    } else {
      st = (isfinite(x) && isfinite(y)) ? STATUS_OOB : STATUS_NAN;
      bits |= st == STATUS_OOB ? (uint32_t)ERRB_OOB : (uint32_t)ERRB_NAN;
    }
  }
  xs[p] = x;
  ys[p] = y;
  sts[p] = st;
  if (bits) atomicOr(err, bits);
}

// The backward of one RK4 step of microbe p from its four stage Jacobians (every precision):
// lambda_{m+1} -> lambda_m in lx, ly, plus its 4 records and their keys. `ok` false: the step was
// frozen (a stage left the grid or the step was non-finite), x_{m+1} = x_m and the adjoint passes
// through.
template <class T>
__device__ __forceinline__ void adj_tail(const FieldView& f, uint32_t p, bool ok, const VelJac<T>& J1,
                                         const VelJac<T>& J2, const VelJac<T>& J3, const VelJac<T>& J4, T dt,
                                         T* __restrict__ lx, T* __restrict__ ly, float4* __restrict__ rec,
                                         uint32_t* __restrict__ key, uint32_t sent, uint32_t* __restrict__ mkey,
                                         uint32_t* __restrict__ mcode, uint32_t msent, uint32_t* err) {
  if (!ok) {  // frozen this step: x_{m+1} = x_m, the adjoint passes through
    if (mkey)
      mkey[p] = msent;
    else
      reinterpret_cast<uint4*>(key)[p] = make_uint4(sent, sent, sent, sent);
    return;
  }
  if (mkey) {
    // gather form: every stage is coded by the slot (dj + 1) * 3 + (di + 1) of its cell around the
    // cell where the step starts (stage 1), 4 bits a stage; the microbe is keyed by that cell * 2 +
    // (1 when a stage leaves the cell). A stage outside the 3 x 3 cells sets ADJ_WIDE and the
    // backward is redone with the record sort.
    const uint32_t cw = (uint32_t)(f.nx - 1);
    const int bi = (int)(J1.cell % cw), bj = (int)(J1.cell / cw);
    const uint32_t cs[3] = {J2.cell, J3.cell, J4.cell};
    uint32_t code = 4u;
    bool wide = false;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int di = (int)(cs[q] % cw) - bi, dj = (int)(cs[q] / cw) - bj;
      wide |= abs(di) > 1 || abs(dj) > 1;
      code |= (uint32_t)((dj + 1) * 3 + (di + 1)) << (4 * (q + 1));
    }
    mcode[p] = code;
    mkey[p] = 2u * J1.cell + (code != 0x4444u ? 1u : 0u);
    if (wide) atomicOr(err, ADJ_WIDE);
  }
  const T gx = lx[p], gy = ly[p];
  const T h6 = dt * (T(1) / T(6)), h3 = dt * (T(1) / T(3)), h2 = T(0.5) * dt;
  // dL/dk4, then back through x3 = x + dt k3, x2 = x + dt/2 k2, x1 = x + dt/2 k1
  const T g4x = h6 * gx, g4y = h6 * gy;
  const T x3x = J4.dlon_dx * g4x + J4.dlat_dx * g4y, x3y = J4.dlon_dy * g4x + J4.dlat_dy * g4y;
  const T g3x = h3 * gx + dt * x3x, g3y = h3 * gy + dt * x3y;
  const T x2x = J3.dlon_dx * g3x + J3.dlat_dx * g3y, x2y = J3.dlon_dy * g3x + J3.dlat_dy * g3y;
  const T g2x = h3 * gx + h2 * x2x, g2y = h3 * gy + h2 * x2y;
  const T x1x = J2.dlon_dx * g2x + J2.dlat_dx * g2y, x1y = J2.dlon_dy * g2x + J2.dlat_dy * g2y;
  const T g1x = h6 * gx + h2 * x1x, g1y = h6 * gy + h2 * x1y;
  const T x0x = J1.dlon_dx * g1x + J1.dlat_dx * g1y, x0y = J1.dlon_dy * g1x + J1.dlat_dy * g1y;
  lx[p] = gx + ((x0x + x1x) + (x2x + x3x));
  ly[p] = gy + ((x0y + x1y) + (x2y + x3y));
  // records: dL/dU_s = dL/dk_s,lon / (M cos lat_s), dL/dV_s = dL/dk_s,lat / M (float32 for the reduction)
  const T invM = T(1) / (T)M_PER_DEG;
  float4* rq = rec + 4 * (size_t)p;
  rq[0] = make_float4((float)J1.a, (float)J1.b, (float)(g1x * J1.inv_mc), (float)(g1y * invM));
  rq[1] = make_float4((float)J2.a, (float)J2.b, (float)(g2x * J2.inv_mc), (float)(g2y * invM));
  rq[2] = make_float4((float)J3.a, (float)J3.b, (float)(g3x * J3.inv_mc), (float)(g3y * invM));
  rq[3] = make_float4((float)J4.a, (float)J4.b, (float)(g4x * J4.inv_mc), (float)(g4y * invM));
  if (!mkey)
    reinterpret_cast<uint4*>(key)[p] =
        make_uint4(4u * J1.cell + 0u, 4u * J2.cell + 1u, 4u * J3.cell + 1u, 4u * J4.cell + 2u);
}

// lambda_{m+1} -> lambda_m, plus 4 records per microbe (key = cell * 4 + stage time, or `sent`).
template <class T>
__global__ void __launch_bounds__(256) k_adj_step(FieldView f, AdjStep s, T dt, uint32_t n, const T* __restrict__ xs,
                                                  const T* __restrict__ ys, const uint8_t* __restrict__ sts,
                                                  T* __restrict__ lx, T* __restrict__ ly, float4* __restrict__ rec,
                                                  uint32_t* __restrict__ key, uint32_t sent, uint32_t* __restrict__ mkey,
                                                  uint32_t* __restrict__ mcode, uint32_t msent, uint32_t* err) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const Geo<T> g(f);
  const T x = xs[p], y = ys[p];
  const T w0 = stage_w<T>(s, 0), w1 = stage_w<T>(s, 1), w2 = stage_w<T>(s, 2);
  VelJac<T> J1, J2, J3, J4;
  bool ok = sts[p] == STATUS_OK;
  ok = ok && vel_jac(f, g, s.k[0], w0, x, y, J1);
  ok = ok && vel_jac(f, g, s.k[1], w1, x + T(0.5) * dt * J1.flon, y + T(0.5) * dt * J1.flat, J2);
  ok = ok && vel_jac(f, g, s.k[1], w1, x + T(0.5) * dt * J2.flon, y + T(0.5) * dt * J2.flat, J3);
  ok = ok && vel_jac(f, g, s.k[2], w2, x + dt * J3.flon, y + dt * J3.flat, J4);
  if (ok) {  // a non-finite step was frozen by the forward: identity, like a stage off the grid
    const T nx = x + (J1.flon + T(2) * J2.flon + T(2) * J3.flon + J4.flon) * (dt * (T(1) / T(6)));
    const T ny = y + (J1.flat + T(2) * J2.flat + T(2) * J3.flat + J4.flat) * (dt * (T(1) / T(6)));
    ok = isfinite(nx) && isfinite(ny);
  }
  adj_tail<T>(f, p, ok, J1, J2, J3, J4, dt, lx, ly, rec, key, sent, mkey, mcode, msent, err);
}

// ---------------------------------------------------------------- double-float positions
//
// The default working precision of the tape (ADJ_DS): each offset is an unevaluated sum of two
// float32 words, hi + lo (about 48 significant bits), so a 720-step trajectory does not pick up the
// float32 rounding of the position every step (0.1 m at the field's scale) that the flow then
// amplifies. Only the position arithmetic is double-float: stage positions, the RK4 update and the
// position -> (cell, bilinear fraction) mapping. Velocities, Jacobians, the adjoint state and the
// records stay float32 with the f32 mode's arithmetic (vel_jac_at<float>). Error-free sums and
// products follow Dekker (1971) and Knuth's two-sum; every operation is rounded explicitly
// (__fadd_rn & co.) so that no contraction changes it between kernels.
struct DS {
  float hi, lo;
};

__device__ __forceinline__ DS ds_of(double d) {
  const float h = (float)d;
  return DS{h, (float)(d - (double)h)};
}
__device__ __forceinline__ double ds_value(DS a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ bool ds_finite(DS a) { return isfinite(a.hi) && isfinite(a.lo); }

// hi + lo of s + t where |s| >= |t| (fast two-sum)
__device__ __forceinline__ DS ds_renorm(float s, float t) {
  const float h = __fadd_rn(s, t);
  return DS{h, __fsub_rn(t, __fsub_rn(h, s))};
}
// a + b, b a float32 (two-sum of the high words, then the low word)
__device__ __forceinline__ DS ds_add(DS a, float b) {
  const float s = __fadd_rn(a.hi, b);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ds_renorm(s, __fadd_rn(e, a.lo));
}
// a + b for two double-float values
__device__ __forceinline__ DS ds_add(DS a, DS b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return ds_renorm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
// a * b (the product of the high words is exact through one fma)
__device__ __forceinline__ DS ds_mul(DS a, DS b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ds_renorm(p, e);
}

// The grid in double-float: fx = (x - gx0) / dx with 1/dx to double-float accuracy (a float32
// 1/dx alone would shift the sampling point by up to ~0.1 m at the far edge of the grid).
struct GeoDS {
  DS mgx0, mgy0, inv_dx, inv_dy;  // -gx0, -gy0 (grid origin minus state origin), 1/dx, 1/dy
  float max_fx, max_fy, org_lat, inv_dxf, inv_dyf;
  __device__ explicit GeoDS(const FieldView& f)
      : mgx0(ds_of(-f.gx0d)), mgy0(ds_of(-f.gy0d)), inv_dx(ds_of(f.inv_dxd)), inv_dy(ds_of(f.inv_dyd)),
        max_fx(f.max_fx), max_fy(f.max_fy), org_lat(f.org_lat), inv_dxf((float)f.inv_dxd), inv_dyf((float)f.inv_dyd) {}
};

// Cell index and bilinear fraction of a double-float grid coordinate u in [0, max]; false outside.
__device__ __forceinline__ bool ds_cell(DS u, float max_u, int n_cells, int& i, float& a) {
  const bool in = (u.hi > 0.f || (u.hi == 0.f && u.lo >= 0.f)) && (u.hi < max_u || (u.hi == max_u && u.lo <= 0.f));
  if (!in) return false;
  float fl = floorf(u.hi);
  if (fl == u.hi && u.lo < 0.f) fl = __fsub_rn(fl, 1.f);  // hi is an integer and the value lies just below it
  i = min((int)fl, n_cells - 1);
  a = __fadd_rn(__fsub_rn(u.hi, (float)i), u.lo);  // u.hi - i is exact (Sterbenz) for i >= 1, and for i = 0
  return true;
}

// Velocity and Jacobian at a double-float offset position (float32 arithmetic past the fractions).
__device__ __forceinline__ bool vel_jac_ds(const FieldView& f, const GeoDS& g, int k, float w, DS xo, DS yo,
                                           VelJac<float>& r) {
  int i, j;
  float a, b;
  if (!ds_cell(ds_mul(ds_add(xo, g.mgx0), g.inv_dx), g.max_fx, f.nx - 1, i, a)) return false;
  if (!ds_cell(ds_mul(ds_add(yo, g.mgy0), g.inv_dy), g.max_fy, f.ny - 1, j, b)) return false;
  vel_jac_at<float>(f, k, w, i, j, a, b, __fadd_rn(g.org_lat, yo.hi), g.inv_dxf, g.inv_dyf, r);
  return true;
}

// The increment (k1 + 2 k2 + 2 k3 + k4) dt / 6 of one coordinate, float32.
__device__ __forceinline__ float rk4_increment(float k1, float k2, float k3, float k4, float dt) {
  return __fmul_rn(__fadd_rn(__fadd_rn(k1, __fmul_rn(2.f, k2)), __fadd_rn(__fmul_rn(2.f, k3), k4)), dt * (1.0f / 6.0f));
}

// Stage q (0..3) of one RK4 step from (x, y): its velocity and Jacobian in J[q], given the earlier
// stages J[0..q-1] (stage positions x + dt/2 k1, x + dt/2 k2, x + dt k3). False outside the grid.
// The forward, the backward recomputation and the cell signature all evaluate stages through this.
__device__ __forceinline__ bool ds_stage(const FieldView& f, const GeoDS& g, const AdjStep& s, float dt, DS x, DS y,
                                         VelJac<float>* J, int q) {
  if (q == 0) return vel_jac_ds(f, g, s.k[0], s.w[0], x, y, J[0]);
  const float h = q == 3 ? dt : 0.5f * dt;
  const int g_ = q == 3 ? 2 : 1;
  return vel_jac_ds(f, g, s.k[g_], s.w[g_], ds_add(x, __fmul_rn(h, J[q - 1].flon)), ds_add(y, __fmul_rn(h, J[q - 1].flat)),
                    J[q]);
}

// One RK4 step from (x, y): the four stages and the new position. False when a stage leaves the grid.
__device__ __forceinline__ bool rk4_ds(const FieldView& f, const GeoDS& g, const AdjStep& s, float dt, DS x, DS y,
                                       VelJac<float>* J, DS& nx, DS& ny) {
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (!ds_stage(f, g, s, dt, x, y, J, q)) return false;
  nx = ds_add(x, rk4_increment(J[0].flon, J[1].flon, J[2].flon, J[3].flon, dt));
  ny = ds_add(y, rk4_increment(J[0].flat, J[1].flat, J[2].flat, J[3].flat, dt));
  return true;
}

__global__ void k_adj_init_ds(FieldView f, uint32_t n, const float* __restrict__ lon, const float* __restrict__ lat,
                              DS* __restrict__ x, DS* __restrict__ y, uint8_t* __restrict__ st) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float a = lon[p], b = lat[p];
  x[p] = ds_of((double)a - (double)f.org_lon);
  y[p] = ds_of((double)b - (double)f.org_lat);
  st[p] = (isfinite(a) && isfinite(b)) ? STATUS_OK : STATUS_NAN;
}

__global__ void k_adj_final_ds(FieldView f, uint32_t n, const DS* __restrict__ x, const DS* __restrict__ y,
                               float* __restrict__ lon, float* __restrict__ lat, double* __restrict__ lon64,
                               double* __restrict__ lat64) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const double a = (double)f.org_lon + ds_value(x[p]), b = (double)f.org_lat + ds_value(y[p]);
  if (lon) {
    lon[p] = (float)a;
    lat[p] = (float)b;
  } else {
    lon64[p] = a;
    lat64[p] = b;
  }
}

__global__ void __launch_bounds__(256) k_adj_forward_ds(FieldView f, const AdjStep* __restrict__ table, int m0, int m1,
                                                        float dt, uint32_t n, DS* __restrict__ xs, DS* __restrict__ ys,
                                                        uint8_t* __restrict__ sts, DS* __restrict__ rec_x,
                                                        DS* __restrict__ rec_y, uint8_t* __restrict__ rec_st,
                                                        uint32_t* err) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const GeoDS g(f);
  DS x = xs[p], y = ys[p];
  uint8_t st = sts[p];
  uint32_t bits = 0;
  for (int m = m0; m < m1; ++m) {
    if (rec_x) {
      const size_t o = (size_t)(m - m0) * n + p;
      rec_x[o] = x;
      rec_y[o] = y;
      rec_st[o] = st;
    }
    if (st != STATUS_OK) continue;
    VelJac<float> J[4];
    DS nx, ny;
    if (rk4_ds(f, g, table[m], dt, x, y, J, nx, ny)) {
      if (ds_finite(nx) && ds_finite(ny)) {
        x = nx;
        y = ny;
      } else {
        st = STATUS_NAN;
        bits |= ERRB_NAN;
      }
    } else {
      st = (ds_finite(x) && ds_finite(y)) ? STATUS_OOB : STATUS_NAN;
      bits |= st == STATUS_OOB ? (uint32_t)ERRB_OOB : (uint32_t)ERRB_NAN;
    }
  }
  xs[p] = x;
  ys[p] = y;
  sts[p] = st;
  if (bits) atomicOr(err, bits);
}

__global__ void __launch_bounds__(256) k_adj_step_ds(FieldView f, AdjStep s, float dt, uint32_t n,
                                                     const DS* __restrict__ xs, const DS* __restrict__ ys,
                                                     const uint8_t* __restrict__ sts, float* __restrict__ lx,
                                                     float* __restrict__ ly, float4* __restrict__ rec,
                                                     uint32_t* __restrict__ key, uint32_t sent,
                                                     uint32_t* __restrict__ mkey, uint32_t* __restrict__ mcode,
                                                     uint32_t msent, uint32_t* err) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const GeoDS g(f);
  VelJac<float> J[4];
  DS nx, ny;
  bool ok = sts[p] == STATUS_OK && rk4_ds(f, g, s, dt, xs[p], ys[p], J, nx, ny);
  ok = ok && ds_finite(nx) && ds_finite(ny);
  adj_tail<float>(f, p, ok, J[0], J[1], J[2], J[3], dt, lx, ly, rec, key, sent, mkey, mcode, msent, err);
}

__global__ void __launch_bounds__(256) k_adj_signature_ds(FieldView f, const AdjStep* __restrict__ table, int n_steps,
                                                          float dt, uint32_t n, const DS* __restrict__ xs,
                                                          const DS* __restrict__ ys, const uint8_t* __restrict__ sts,
                                                          unsigned long long* __restrict__ sig) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const GeoDS g(f);
  DS x = xs[p], y = ys[p];
  bool live = sts[p] == STATUS_OK;
  unsigned long long h = 0;
  const unsigned long long nx = (unsigned long long)f.nx, cw = (unsigned long long)(f.nx - 1);
  for (int m = 0; m < n_steps && live; ++m) {
    const AdjStep s = table[m];
    VelJac<float> J[4];
    int q = 0;
#pragma unroll
    for (; q < 4; ++q) {  // the stages evaluated, up to one that leaves the grid
      if (!ds_stage(f, g, s, dt, x, y, J, q)) break;
      h = (h ^ ((J[q].cell / cw) * nx + J[q].cell % cw)) * 0x100000001B3ull;
    }
    if (q < 4) break;
    const DS x1 = ds_add(x, rk4_increment(J[0].flon, J[1].flon, J[2].flon, J[3].flon, dt));
    const DS y1 = ds_add(y, rk4_increment(J[0].flat, J[1].flat, J[2].flat, J[3].flat, dt));
    if (!(ds_finite(x1) && ds_finite(y1))) break;
    x = x1;
    y = y1;
  }
  sig[p] = h;
}

// Cell path of every microbe over steps [0, n_steps): the grid cell (j * nx + i) of each stage that
// the forward evaluated, folded in order as sig = (sig ^ cell) * 0x100000001B3. The stage
// positions come from vel_jac, whose values are the forward's; two runs of one microbe with equal
// signatures sampled the same bilinear pieces, so the map between them is smooth.
template <class T>
__global__ void __launch_bounds__(256) k_adj_signature(FieldView f, const AdjStep* __restrict__ table, int n_steps,
                                                       T dt, uint32_t n, const T* __restrict__ xs,
                                                       const T* __restrict__ ys, const uint8_t* __restrict__ sts,
                                                       unsigned long long* __restrict__ sig) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const Geo<T> g(f);
  T x = xs[p], y = ys[p];
  bool live = sts[p] == STATUS_OK;
  unsigned long long h = 0;
  const unsigned long long nx = (unsigned long long)f.nx, cw = (unsigned long long)(f.nx - 1);
  for (int m = 0; m < n_steps && live; ++m) {
    const AdjStep s = table[m];
    const int ks[4] = {s.k[0], s.k[1], s.k[1], s.k[2]};
    const T ws[4] = {stage_w<T>(s, 0), stage_w<T>(s, 1), stage_w<T>(s, 1), stage_w<T>(s, 2)};
    const T hs[4] = {T(0), T(0.5), T(0.5), T(1)};
    T kx[4], ky[4];
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (!ok) break;
      VelJac<T> J;
      const T sx = q == 0 ? x : x + hs[q] * dt * kx[q - 1];
      const T sy = q == 0 ? y : y + hs[q] * dt * ky[q - 1];
      ok = vel_jac(f, g, ks[q], ws[q], sx, sy, J);
      if (ok) {
        h = (h ^ ((J.cell / cw) * nx + J.cell % cw)) * 0x100000001B3ull;
        kx[q] = J.flon;
        ky[q] = J.flat;
      }
    }
    if (!ok) break;
    const T nx_ = x + (kx[0] + T(2) * kx[1] + T(2) * kx[2] + kx[3]) * (dt * (T(1) / T(6)));
    const T ny_ = y + (ky[0] + T(2) * ky[1] + T(2) * ky[2] + ky[3]) * (dt * (T(1) / T(6)));
    if (!(isfinite(nx_) && isfinite(ny_))) break;
    x = nx_;
    y = ny_;
  }
  sig[p] = h;
}

// ---------------------------------------------------------------- K7a: stable LSD radix sort

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr uint32_t RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARPS = RS_THREADS / 32;

// Digit histogram of one tile, written digit-major: hist[d * tiles + tile].
__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const uint32_t* __restrict__ keys, uint32_t m, int shift,
                                                        int bits, uint32_t* __restrict__ hist, uint32_t tiles) {
  __shared__ uint32_t h[RS_RADIX_MAX];
  const uint32_t R = 1u << bits, mask = R - 1u;
  for (uint32_t d = threadIdx.x; d < R; d += RS_THREADS) h[d] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * RS_TILE;
  const uint32_t lane = threadIdx.x & 31u;
  for (int r = 0; r < RS_ITEMS; ++r) {
    const uint32_t i = base + (uint32_t)r * RS_THREADS + threadIdx.x;
    const bool valid = i < m;
    const uint32_t d = valid ? (keys[i] >> shift) & mask : R;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    if (valid && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(&h[d], (uint32_t)__popc(peers));
  }
  __syncthreads();
  for (uint32_t d = threadIdx.x; d < R; d += RS_THREADS) hist[(size_t)d * tiles + blockIdx.x] = h[d];
}

// Stable scatter of one tile. Warp w takes the tile's w-th run of RS_ITEMS * 32 consecutive items
// (RS_ITEMS rounds of 32) and ranks each item among the equal digits of its run with match masks and
// a per-warp digit counter, without block barriers; the block then turns the counters into per-warp
// digit offsets (the tile's offset of the digit plus the counts of the earlier warps), and each
// item goes to its warp's offset plus its rank: equal keys keep their order.
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint32_t* __restrict__ kin,
                                                           const uint32_t* __restrict__ vin,
                                                           uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t m, int shift, int bits,
                                                           const uint32_t* __restrict__ hscan, uint32_t tiles) {
  __shared__ uint32_t wcnt[RS_WARPS][RS_RADIX_MAX];
  const uint32_t R = 1u << bits, mask = R - 1u;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t d = threadIdx.x; d < R; d += RS_THREADS)
    for (int w = 0; w < RS_WARPS; ++w) wcnt[w][d] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * RS_TILE + warp * (RS_ITEMS * 32u);
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t kk[RS_ITEMS], rk[RS_ITEMS];
#pragma unroll
  for (int r = 0; r < RS_ITEMS; ++r) {
    const uint32_t i = base + (uint32_t)r * 32u + lane;
    const bool valid = i < m;
    const uint32_t k = valid ? kin[i] : 0u;
    const uint32_t d = valid ? (k >> shift) & mask : R;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t below = peers & lt;
    const uint32_t c = valid ? wcnt[warp][d] : 0u;  // every peer reads the count before the update
    __syncwarp();
    if (valid && below == 0) wcnt[warp][d] = c + (uint32_t)__popc(peers);
    __syncwarp();
    kk[r] = k;
    rk[r] = c + (uint32_t)__popc(below);
  }
  __syncthreads();
  for (uint32_t d = threadIdx.x; d < R; d += RS_THREADS) {
    uint32_t o = hscan[(size_t)d * tiles + blockIdx.x];
    for (int w = 0; w < RS_WARPS; ++w) {
      const uint32_t c = wcnt[w][d];
      wcnt[w][d] = o;
      o += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_ITEMS; ++r) {
    const uint32_t i = base + (uint32_t)r * 32u + lane;
    if (i < m) {
      const uint32_t o = wcnt[warp][(kk[r] >> shift) & mask] + rk[r];
      kout[o] = kk[r];
      vout[o] = vin ? vin[i] : i;
    }
  }
}

// Exclusive scan of n uint32 values (in -> out), in SCAN_BLOCKS contiguous chunks: block sums, then
// each block adds the sums of the blocks before it while scanning its chunk.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* sh, uint32_t* total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < blockDim.x / 32 ? sh[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= (uint32_t)o) s += y;
    }
    sh[lane] = s;  // inclusive warp totals
  }
  __syncthreads();
  const uint32_t before = warp ? sh[warp - 1] : 0u;
  *total = sh[blockDim.x / 32 - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(256) k_scan_sums(const uint32_t* __restrict__ in, size_t n, size_t chunk,
                                                   uint32_t* __restrict__ bsum) {
  __shared__ uint32_t red[8];
  const size_t lo = (size_t)blockIdx.x * chunk, hi = min(n, lo + chunk);
  uint32_t s = 0;
  for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += in[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < 8; ++w) t += red[w];
    bsum[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(256) k_scan_chunks(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                     size_t n, size_t chunk, const uint32_t* __restrict__ bsum) {
  __shared__ uint32_t sh[32];
  __shared__ uint32_t carry;
  if (threadIdx.x < 32) {
    uint32_t s = 0;
    for (uint32_t b = threadIdx.x; b < blockIdx.x; b += 32) s += bsum[b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) carry = s;
  }
  __syncthreads();
  const size_t lo = (size_t)blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (size_t t = lo; t < hi; t += blockDim.x) {
    const size_t i = t + threadIdx.x;
    const uint32_t v = i < hi ? in[i] : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(v, sh, &total);
    if (i < hi) out[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
}

// ---------------------------------------------------------------- K7b: segmented reduction

// Segment bounds of the sorted keys: cst[k] = first index, cen[k] = one past the last (both left at
// 0 for absent keys; the reduction resets the entries it read).
__global__ void k_adj_bounds(const uint32_t* __restrict__ skey, uint32_t m, uint32_t sent, uint32_t* __restrict__ cst,
                             uint32_t* __restrict__ cen) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint32_t k = skey[i];
  if (k >= sent) return;
  if (i == 0 || skey[i - 1] != k) cst[k] = i;
  if (i + 1 == m || skey[i + 1] != k) cen[k] = i + 1;
}

__device__ __forceinline__ void neumaier(float& s, float& c, float v) {
  const float t = s + v;
  c += (fabsf(s) >= fabsf(v)) ? ((s - t) + v) : ((v - t) + s);
  s = t;
}

// One warp per field cell: for each stage time g, the records of segment (cell, g) in sorted order,
// lane l taking entries l, l+32, ...; out csum[(cell * 3 + g) * 8 + q], q = corner (00, 01, 10, 11)
// of dL/dU, then of dL/dV.
__global__ void __launch_bounds__(256) k_adj_reduce(uint32_t ncells, uint32_t* __restrict__ cst,
                                                    uint32_t* __restrict__ cen, const uint32_t* __restrict__ sval,
                                                    const float4* __restrict__ rec, float* __restrict__ csum) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = wid; c < ncells; c += nw) {
    for (uint32_t g = 0; g < 3; ++g) {
      const uint32_t k = 4u * c + g;
      const uint32_t lo = cst[k], hi = cen[k];
      float* out = csum + ((size_t)c * 3 + g) * 8;
      if (lo == hi) {  // warp-uniform: an empty segment
        if (lane < 8) out[lane] = 0.f;
        continue;
      }
      float s[8], e[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) s[q] = e[q] = 0.f;
      for (uint32_t i = lo + lane; i < hi; i += 32) {
        const float4 r = rec[sval[i]];
        const float a = r.x, b = r.y;
        const float w[4] = {(1.f - a) * (1.f - b), a * (1.f - b), (1.f - a) * b, a * b};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          neumaier(s[q], e[q], w[q] * r.z);
          neumaier(s[4 + q], e[4 + q], w[q] * r.w);
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        float t = s[q] + e[q];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        s[q] = t;
      }
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < 8; ++q) out[q] = s[q];
        cst[k] = 0;
        cen[k] = 0;
      }
    }
  }
}

// Gather form, after the stable sort of the microbe keys (cell * 2 + leaves-the-cell, so in index
// order within a key): bounds of every key, the stage codes in sorted order, and the list of target
// cells: a cell with microbes, and the 3 x 3 cells around one whose microbes leave it, each listed
// once a step (mark[c] takes the step's stamp when c is listed; tcnt counts the list).
__global__ void k_adj_cells(const uint32_t* __restrict__ skey, const uint32_t* __restrict__ sval, uint32_t m,
                            uint32_t cw, uint32_t ch, const uint32_t* __restrict__ mcode,
                            uint32_t* __restrict__ scode, uint32_t* __restrict__ cst, uint32_t* __restrict__ cen,
                            uint32_t* __restrict__ mark, uint32_t stamp, uint32_t* __restrict__ tlist,
                            uint32_t* __restrict__ tcnt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint32_t k = skey[i];
  if (k >= 2u * cw * ch) return;  // frozen microbes sort last
  scode[i] = mcode[sval[i]];
  if (i + 1 == m || skey[i + 1] != k) cen[k] = i + 1;
  if (i != 0 && skey[i - 1] == k) return;
  cst[k] = i;
  const uint32_t b = k >> 1;
  if (!(k & 1u)) {
    if (atomicExch(&mark[b], stamp) != stamp) tlist[atomicAdd(tcnt, 1u)] = b;
    return;
  }
  const int bi = (int)(b % cw), bj = (int)(b / cw);
  const uint32_t cells = cw * ch;
  uint32_t tc[9], old[9], fresh = 0;
#pragma unroll
  for (int r = 0; r < 9; ++r) {  // no branch between the exchanges: they are issued together
    const int ti = bi + r % 3 - 1, tj = bj + r / 3 - 1;
    const bool in = ti >= 0 && tj >= 0 && ti < (int)cw && tj < (int)ch;
    tc[r] = in ? (uint32_t)tj * cw + (uint32_t)ti : cells;  // mark[cells]: a slot no target reads
    old[r] = atomicExch(&mark[tc[r]], stamp);
  }
#pragma unroll
  for (int r = 0; r < 9; ++r) fresh |= (tc[r] != cells && old[r] != stamp) ? 1u << r : 0u;
  if (!fresh) return;
  uint32_t o = atomicAdd(tcnt, (uint32_t)__popc(fresh));
#pragma unroll
  for (int r = 0; r < 9; ++r)
    if (fresh & (1u << r)) tlist[o++] = tc[r];
}

template <int G>
__device__ __forceinline__ void gather_add(const float4& rr, float (&acc)[3][8], float (&cmp)[3][8]) {
  const float a = rr.x, b = rr.y;
  const float w[4] = {(1.f - a) * (1.f - b), a * (1.f - b), (1.f - a) * b, a * b};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    neumaier(acc[G][q], cmp[G][q], w[q] * rr.z);
    neumaier(acc[G][4 + q], cmp[G][4 + q], w[q] * rr.w);
  }
}

// One warp per listed target cell c. Neighbour cell r = (dj + 1) * 3 + (di + 1) in turn: its whole
// run for r = 4 (c itself), else only its microbes that leave it; lane l takes entries l, l + 32,
// ... of each run, and a stage of a microbe of neighbour r lands in c when its slot is 8 - r. Stage
// times: stage 1 at t (group 0), stages 2 and 3 at t + dt/2 (group 1), stage 4 at t + dt (group 2).
// Sums as in k_adj_reduce (Neumaier float32 per lane, fixed warp tree), so the result does not
// depend on which warp took c.
__global__ void __launch_bounds__(256) k_adj_gather(uint32_t cw, uint32_t ch, const uint32_t* __restrict__ tcnt,
                                                    const uint32_t* __restrict__ tlist,
                                                    const uint32_t* __restrict__ cst,
                                                    const uint32_t* __restrict__ cen,
                                                    const uint32_t* __restrict__ scode,
                                                    const uint32_t* __restrict__ sval,
                                                    const float4* __restrict__ rec, float* __restrict__ csum) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t nt = *tcnt;
  const uint32_t stride = gridDim.x * (blockDim.x >> 5);
  for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += stride) {
    const uint32_t c = tlist[t];
    const int ci = (int)(c % cw), cj = (int)(c / cw);
    uint32_t lo = 0, hi = 0;
    if (lane < 9) {
      const int bi = ci + (int)(lane % 3) - 1, bj = cj + (int)(lane / 3) - 1;
      if (bi >= 0 && bj >= 0 && bi < (int)cw && bj < (int)ch) {
        const uint32_t k1 = 2u * ((uint32_t)bj * cw + (uint32_t)bi) + 1u;
        const uint32_t e1 = cen[k1];  // bounds of absent keys: cen = 0
        if (lane == 4) {              // keys 2b and 2b + 1 are adjacent in sorted order
          const uint32_t e0 = cen[k1 - 1];
          lo = e0 ? cst[k1 - 1] : (e1 ? cst[k1] : 0u);
          hi = e1 ? e1 : e0;
        } else if (e1) {
          lo = cst[k1];
          hi = e1;
        }
      }
    }
    float acc[3][8], cmp[3][8];
#pragma unroll
    for (int g = 0; g < 3; ++g)
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[g][q] = cmp[g][q] = 0.f;
    {  // c's own microbes: stage 1 always lands in c, the others mostly; two entries in flight
      const uint32_t rlo = __shfl_sync(0xffffffffu, lo, 4), rhi = __shfl_sync(0xffffffffu, hi, 4);
      for (uint32_t s = rlo + lane; s < rhi; s += 64) {
        const uint32_t s2 = s + 32;
        const bool two = s2 < rhi;
        const uint32_t code0 = scode[s], code1 = two ? scode[s2] : 0u;
        const float4* rp0 = rec + 4 * (size_t)sval[s];
        const float4* rp1 = rec + 4 * (size_t)(two ? sval[s2] : 0u);
        float4 r[2][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) r[0][q] = rp0[q];
        if (two) {
#pragma unroll
          for (int q = 0; q < 4; ++q) r[1][q] = rp1[q];
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (h == 1 && !two) break;
          const uint32_t code = h ? code1 : code0;
          gather_add<0>(r[h][0], acc, cmp);
          if (((code >> 4) & 15u) == 4u) gather_add<1>(r[h][1], acc, cmp);
          if (((code >> 8) & 15u) == 4u) gather_add<1>(r[h][2], acc, cmp);
          if (((code >> 12) & 15u) == 4u) gather_add<2>(r[h][3], acc, cmp);
        }
      }
    }
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
      if (r == 4) continue;
      const uint32_t rlo = __shfl_sync(0xffffffffu, lo, r), rhi = __shfl_sync(0xffffffffu, hi, r);
      const uint32_t slot = 8u - (uint32_t)r;
      for (uint32_t s = rlo + lane; s < rhi; s += 64) {
        const uint32_t s2 = s + 32;
        const uint32_t c0 = scode[s];
        const uint32_t c1 = s2 < rhi ? scode[s2] : 0xffffffffu;  // slot 15 matches nothing
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint32_t code = h ? c1 : c0;
          const bool m1 = ((code >> 4) & 15u) == slot, m2 = ((code >> 8) & 15u) == slot;
          const bool m3 = ((code >> 12) & 15u) == slot;  // stage 1 never leaves its cell
          if (!(m1 | m2 | m3)) continue;
          const float4* rp = rec + 4 * (size_t)sval[h ? s2 : s];
          if (m1) gather_add<1>(rp[1], acc, cmp);
          if (m2) gather_add<1>(rp[2], acc, cmp);
          if (m3) gather_add<2>(rp[3], acc, cmp);
        }
      }
    }
    float* out = csum + (size_t)c * 24;
#pragma unroll
    for (int g = 0; g < 3; ++g)
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        float v = acc[g][q] + cmp[g][q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == (uint32_t)(g * 8 + q)) out[g * 8 + q] = v;
      }
  }
}

// One thread per grid node: the four cells around it in a fixed order, then the three stage times
// spread onto frames k_g (weight 1 - w_g) and k_g + 1 (weight w_g), added to the gradient.
__global__ void __launch_bounds__(256) k_adj_nodes(int nx, int ny, AdjStep s, const float* __restrict__ csum,
                                                   const uint32_t* __restrict__ mark, uint32_t stamp,
                                                   float* __restrict__ gu, float* __restrict__ gv) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (uint32_t)nx * (uint32_t)ny) return;
  const int ni = (int)(q % (uint32_t)nx), nj = (int)(q / (uint32_t)nx);
  const int cw = nx - 1;
  float U[3] = {0.f, 0.f, 0.f}, V[3] = {0.f, 0.f, 0.f};
  // cell (ci, cj) sees this node as corner (nj - cj) * 2 + (ni - ci)
  const int ci_[4] = {ni - 1, ni, ni - 1, ni}, cj_[4] = {nj - 1, nj - 1, nj, nj}, corner[4] = {3, 2, 1, 0};
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int ci = ci_[t], cj = cj_[t];
    if (ci < 0 || cj < 0 || ci > nx - 2 || cj > ny - 2) continue;
    const size_t cell = (size_t)cj * cw + ci;
    if (mark && mark[cell] != stamp) continue;  // gather form: only listed cells were summed
    const float* cs = csum + cell * 24;
#pragma unroll
    for (int g = 0; g < 3; ++g) {
      U[g] += cs[g * 8 + corner[t]];
      V[g] += cs[g * 8 + 4 + corner[t]];
    }
  }
  if (U[0] == 0.f && U[1] == 0.f && U[2] == 0.f && V[0] == 0.f && V[1] == 0.f && V[2] == 0.f) return;
  int kmin = s.k[0], kmax = s.k[0];
#pragma unroll
  for (int g = 0; g < 3; ++g) {
    kmin = min(kmin, s.k[g]);
    kmax = max(kmax, s.k[g] + (s.w[g] != 0.f ? 1 : 0));
  }
  const size_t plane = (size_t)nx * ny;
  for (int fr = kmin; fr <= kmax; ++fr) {
    float du = 0.f, dv = 0.f;
    bool any = false;
#pragma unroll
    for (int g = 0; g < 3; ++g) {
      if (s.k[g] == fr) {
        du += (1.f - s.w[g]) * U[g];
        dv += (1.f - s.w[g]) * V[g];
        any = true;
      }
      if (s.w[g] != 0.f && s.k[g] + 1 == fr) {
        du += s.w[g] * U[g];
        dv += s.w[g] * V[g];
        any = true;
      }
    }
    if (any) {
      gu[(size_t)fr * plane + q] += du;
      gv[(size_t)fr * plane + q] += dv;
    }
  }
}

// ---------------------------------------------------------------- launchers

static inline unsigned grid_for(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

void launch_adj_stages(const FieldView& f, double t_start, double dt, int n_steps, AdjStep* table, uint32_t* err,
                       cudaStream_t st) {
  if (n_steps > 0) k_adj_stages<<<grid_for(n_steps, 128), 128, 0, st>>>(f, t_start, dt, n_steps, table, err);
}

void launch_adj_init(const FieldView& f, int prec, uint32_t n, const float* lon, const float* lat, void* x, void* y,
                     uint8_t* status, cudaStream_t st) {
  if (!n) return;
  if (prec == ADJ_F64)
    k_adj_init<double><<<grid_for(n, 256), 256, 0, st>>>(f, n, lon, lat, (double*)x, (double*)y, status);
  else if (prec == ADJ_DS)
    k_adj_init_ds<<<grid_for(n, 256), 256, 0, st>>>(f, n, lon, lat, (DS*)x, (DS*)y, status);
  else
    k_adj_init<float><<<grid_for(n, 256), 256, 0, st>>>(f, n, lon, lat, (float*)x, (float*)y, status);
}

void launch_adj_final(const FieldView& f, int prec, uint32_t n, const void* x, const void* y, float* lon, float* lat,
                      cudaStream_t st) {
  if (!n) return;
  if (prec == ADJ_F64)
    k_adj_final<double><<<grid_for(n, 256), 256, 0, st>>>(f, n, (const double*)x, (const double*)y, lon, lat);
  else if (prec == ADJ_DS)
    k_adj_final_ds<<<grid_for(n, 256), 256, 0, st>>>(f, n, (const DS*)x, (const DS*)y, lon, lat, nullptr, nullptr);
  else
    k_adj_final<float><<<grid_for(n, 256), 256, 0, st>>>(f, n, (const float*)x, (const float*)y, lon, lat);
}

void launch_adj_final64(const FieldView& f, int prec, uint32_t n, const void* x, const void* y, double* lon,
                        double* lat, cudaStream_t st) {
  if (!n) return;
  if (prec == ADJ_F64)
    k_adj_final64<double><<<grid_for(n, 256), 256, 0, st>>>(f, n, (const double*)x, (const double*)y, lon, lat);
  else if (prec == ADJ_DS)
    k_adj_final_ds<<<grid_for(n, 256), 256, 0, st>>>(f, n, (const DS*)x, (const DS*)y, nullptr, nullptr, lon, lat);
  else
    k_adj_final64<float><<<grid_for(n, 256), 256, 0, st>>>(f, n, (const float*)x, (const float*)y, lon, lat);
}

void launch_adj_seed(int prec, uint32_t n, const float* gx, const float* gy, void* lx, void* ly, cudaStream_t st) {
  if (!n) return;
  if (prec == ADJ_F64)
    k_adj_convert_in<double><<<grid_for(n, 256), 256, 0, st>>>(n, gx, gy, (double*)lx, (double*)ly);
  else
    k_adj_convert_in<float><<<grid_for(n, 256), 256, 0, st>>>(n, gx, gy, (float*)lx, (float*)ly);
}

void launch_adj_unseed(int prec, uint32_t n, const void* lx, const void* ly, float* gx, float* gy, cudaStream_t st) {
  if (!n) return;
  if (prec == ADJ_F64)
    k_adj_convert_out<double><<<grid_for(n, 256), 256, 0, st>>>(n, (const double*)lx, (const double*)ly, gx, gy);
  else
    k_adj_convert_out<float><<<grid_for(n, 256), 256, 0, st>>>(n, (const float*)lx, (const float*)ly, gx, gy);
}

void launch_adj_forward(const FieldView& f, int prec, const AdjStep* table, int m0, int m1, double dt, uint32_t n,
                        void* x, void* y, uint8_t* status, void* rec_x, void* rec_y, uint8_t* rec_st, uint32_t* err,
                        cudaStream_t st) {
  if (!n || m1 <= m0) return;
  if (prec == ADJ_F64)
    k_adj_forward<double><<<grid_for(n, 256), 256, 0, st>>>(f, table, m0, m1, dt, n, (double*)x, (double*)y, status,
                                                            (double*)rec_x, (double*)rec_y, rec_st, err);
  else if (prec == ADJ_DS)
    k_adj_forward_ds<<<grid_for(n, 256), 256, 0, st>>>(f, table, m0, m1, (float)dt, n, (DS*)x, (DS*)y, status,
                                                       (DS*)rec_x, (DS*)rec_y, rec_st, err);
  else
    k_adj_forward<float><<<grid_for(n, 256), 256, 0, st>>>(f, table, m0, m1, (float)dt, n, (float*)x, (float*)y, status,
                                                           (float*)rec_x, (float*)rec_y, rec_st, err);
}

void launch_adj_step(const FieldView& f, int prec, const AdjStep& s, double dt, uint32_t n, const void* x,
                     const void* y, const uint8_t* status, void* lx, void* ly, float4* rec, uint32_t* key, uint32_t sent,
                     uint32_t* mkey, uint32_t* mcode, uint32_t msent, uint32_t* err, cudaStream_t st) {
  if (!n) return;
  if (prec == ADJ_F64)
    k_adj_step<double><<<grid_for(n, 256), 256, 0, st>>>(f, s, dt, n, (const double*)x, (const double*)y, status,
                                                         (double*)lx, (double*)ly, rec, key, sent, mkey, mcode, msent,
                                                         err);
  else if (prec == ADJ_DS)
    k_adj_step_ds<<<grid_for(n, 256), 256, 0, st>>>(f, s, (float)dt, n, (const DS*)x, (const DS*)y, status,
                                                    (float*)lx, (float*)ly, rec, key, sent, mkey, mcode, msent, err);
  else
    k_adj_step<float><<<grid_for(n, 256), 256, 0, st>>>(f, s, (float)dt, n, (const float*)x, (const float*)y, status,
                                                        (float*)lx, (float*)ly, rec, key, sent, mkey, mcode, msent,
                                                        err);
}

void launch_adj_cells(const uint32_t* skey, const uint32_t* sval, uint32_t m, uint32_t cw, uint32_t ch,
                      const uint32_t* mcode, uint32_t* scode, uint32_t* cst, uint32_t* cen, uint32_t* mark,
                      uint32_t stamp, uint32_t* tlist, uint32_t* tcnt, cudaStream_t st) {
  if (m) k_adj_cells<<<grid_for(m, 256), 256, 0, st>>>(skey, sval, m, cw, ch, mcode, scode, cst, cen, mark, stamp,
                                                       tlist, tcnt);
}

void launch_adj_gather(uint32_t cw, uint32_t ch, const uint32_t* tcnt, const uint32_t* tlist, const uint32_t* cst,
                       const uint32_t* cen, const uint32_t* scode, const uint32_t* sval, const float4* rec,
                       float* csum, int sms, cudaStream_t st) {
  const size_t ncells = (size_t)cw * ch;
  unsigned blocks = grid_for(ncells * 32, 256);
  const unsigned cap = (unsigned)(sms > 0 ? sms : 152) * 8u;
  if (blocks > cap) blocks = cap;
  if (ncells) k_adj_gather<<<blocks, 256, 0, st>>>(cw, ch, tcnt, tlist, cst, cen, scode, sval, rec, csum);
}

void launch_adj_signature(const FieldView& f, int prec, const AdjStep* table, int n_steps, double dt, uint32_t n,
                          const void* x, const void* y, const uint8_t* status, unsigned long long* sig,
                          cudaStream_t st) {
  if (!n) return;
  if (prec == ADJ_F64)
    k_adj_signature<double><<<grid_for(n, 256), 256, 0, st>>>(f, table, n_steps, dt, n, (const double*)x,
                                                              (const double*)y, status, sig);
  else if (prec == ADJ_DS)
    k_adj_signature_ds<<<grid_for(n, 256), 256, 0, st>>>(f, table, n_steps, (float)dt, n, (const DS*)x, (const DS*)y,
                                                         status, sig);
  else
    k_adj_signature<float><<<grid_for(n, 256), 256, 0, st>>>(f, table, n_steps, (float)dt, n, (const float*)x,
                                                             (const float*)y, status, sig);
}

size_t adj_sort_hist_len(uint32_t m) { return (size_t)RS_RADIX_MAX * grid_for(m, RS_TILE); }

void adj_sort(const AdjSortBufs& sb, uint32_t m, int key_bits, cudaStream_t st, const uint32_t** skey,
              const uint32_t** sval) {
  const uint32_t tiles = grid_for(m, RS_TILE);
  const int passes = key_bits <= RS_BITS_MAX ? 1 : (key_bits + RS_BITS_MAX - 1) / RS_BITS_MAX;
  const int width = (key_bits + passes - 1) / passes;
  const uint32_t* kin = sb.key;
  const uint32_t* vin = nullptr;
  for (int p = 0; p < passes; ++p) {
    uint32_t* kout = (p & 1) ? sb.k2 : sb.k1;
    uint32_t* vout = (p & 1) ? sb.v2 : sb.v1;
    const int shift = p * width;
    const int bits = key_bits - shift < width ? key_bits - shift : width;
    k_rs_hist<<<tiles, RS_THREADS, 0, st>>>(kin, m, shift, bits, sb.hist, tiles);
    const size_t len = ((size_t)1 << bits) * tiles;
    const size_t chunk = (len + SCAN_BLOCKS - 1) / SCAN_BLOCKS;
    const unsigned nb = grid_for(len, chunk);
    k_scan_sums<<<nb, 256, 0, st>>>(sb.hist, len, chunk, sb.bsum);
    k_scan_chunks<<<nb, 256, 0, st>>>(sb.hist, sb.hscan, len, chunk, sb.bsum);
    k_rs_scatter<<<tiles, RS_THREADS, 0, st>>>(kin, vin, kout, vout, m, shift, bits, sb.hscan, tiles);
    kin = kout;
    vin = vout;
  }
  *skey = kin;
  *sval = vin;
}

void launch_adj_bounds(const uint32_t* skey, uint32_t m, uint32_t sent, uint32_t* cst, uint32_t* cen,
                       cudaStream_t st) {
  if (m) k_adj_bounds<<<grid_for(m, 256), 256, 0, st>>>(skey, m, sent, cst, cen);
}

void launch_adj_reduce(uint32_t ncells, uint32_t* cst, uint32_t* cen, const uint32_t* sval, const float4* rec,
                       float* csum, int sms, cudaStream_t st) {
  unsigned blocks = grid_for((size_t)ncells * 32, 256);
  const unsigned cap = (unsigned)(sms > 0 ? sms : 152) * 16u;
  if (blocks > cap) blocks = cap;
  if (ncells) k_adj_reduce<<<blocks, 256, 0, st>>>(ncells, cst, cen, sval, rec, csum);
}

void launch_adj_nodes(int nx, int ny, const AdjStep& s, const float* csum, const uint32_t* mark, uint32_t stamp,
                      float* gu, float* gv, cudaStream_t st) {
  k_adj_nodes<<<grid_for((size_t)nx * ny, 256), 256, 0, st>>>(nx, ny, s, csum, mark, stamp, gu, gv);
}

}  // namespace lm
