// Velocity sampling shared by the forward advection (k_advect.cu) and its adjoint (k_adjoint.cu):
// both must evaluate exactly the same float32 arithmetic so that the adjoint's recomputed
// trajectories are bit-identical to the forward's.
//
// Semantics follow the reference's advection call, pset.execute(parcels.AdvectionRK4, runtime=dt,
// dt=dt) on a RectilinearZGrid(mesh="spherical") with interp_method="linear"
// (particle_advecter.py:177-187, 220-223): bilinear in (lon, lat), linear in time between the two
// frames that bracket the stage time, converted to deg/s with u / (1852*60*cos(lat)) and v / (1852*60).
#pragma once
#include "lm_internal.h"

namespace lm {

struct Stage {
  int k;    // frame index
  float w;  // weight of frame k+1 (0 means frame k only)
  int ok;
};

// Frame bracket of time t on a uniform time axis t0 + k*dT, k in [0, nt).
__device__ __forceinline__ Stage stage_at(const FieldView& f, double t) {
  Stage s;
  double fk = (t - f.t0) / f.dT;
  s.ok = (fk >= -1e-9 && fk <= (double)(f.nt - 1) + 1e-9);
  double kf = floor(fk);
  int k = (int)fmin(fmax(kf, 0.0), (double)(f.nt - 2));
  double w = fmin(fmax(fk - (double)k, 0.0), 1.0);
  if (w >= 1.0) {  // exactly on frame k+1: read that frame alone
    k += 1;
    w = 0.0;
  }
  s.k = k;
  s.w = (float)w;
  return s;
}

// 1 degree of latitude = 1852 m * 60 (the nautical-mile convention of a spherical mesh).
constexpr float M_PER_DEG = 111120.0f;

// Velocity in deg/s at offset position (xo, yo). Returns false outside the grid or on NaN.
__device__ __forceinline__ bool velocity(const FieldView& f, const float2* __restrict__ uv, const Stage& s, float xo,
                                         float yo, float& dlon, float& dlat) {
  float fx = (xo - f.gx0) * f.inv_dx;
  float fy = (yo - f.gy0) * f.inv_dy;
  if (!(fx >= 0.f && fx <= f.max_fx && fy >= 0.f && fy <= f.max_fy)) return false;
  int i = min((int)fx, f.nx - 2);
  int j = min((int)fy, f.ny - 2);
  float a = fx - (float)i, b = fy - (float)j;
  const float2* p = uv + ((size_t)s.k * f.ny + j) * f.nx + i;
  float2 c00 = __ldg(p), c01 = __ldg(p + 1), c10 = __ldg(p + f.nx), c11 = __ldg(p + f.nx + 1);
  float w00 = (1.f - a) * (1.f - b), w01 = a * (1.f - b), w10 = (1.f - a) * b, w11 = a * b;
  float u = w00 * c00.x + w01 * c01.x + w10 * c10.x + w11 * c11.x;
  float v = w00 * c00.y + w01 * c01.y + w10 * c10.y + w11 * c11.y;
  if (s.w != 0.f) {
    p += (size_t)f.nx * f.ny;
    c00 = __ldg(p); c01 = __ldg(p + 1); c10 = __ldg(p + f.nx); c11 = __ldg(p + f.nx + 1);
    float u1 = w00 * c00.x + w01 * c01.x + w10 * c10.x + w11 * c11.x;
    float v1 = w00 * c00.y + w01 * c01.y + w10 * c10.y + w11 * c11.y;
    u = u + s.w * (u1 - u);
    v = v + s.w * (v1 - v);
  }
  float lat = f.org_lat + yo;
  float c = cospif(lat * (1.0f / 180.0f));
  dlon = u / (M_PER_DEG * c);
  dlat = v * (1.0f / M_PER_DEG);
  return true;
}

// One RK4 step of one microbe (x, y offsets), exactly the forward's arithmetic. Returns false when a
// stage leaves the grid (the caller freezes the microbe); the new position may be non-finite.
__device__ __forceinline__ bool rk4_step(const FieldView& f, const float2* __restrict__ uv, const Stage* sh, float dt,
                                         float x, float y, float& nx, float& ny) {
  float k1x, k1y, k2x, k2y, k3x, k3y, k4x, k4y;
  bool ok = velocity(f, uv, sh[0], x, y, k1x, k1y);
  ok = ok && velocity(f, uv, sh[1], x + 0.5f * dt * k1x, y + 0.5f * dt * k1y, k2x, k2y);
  ok = ok && velocity(f, uv, sh[1], x + 0.5f * dt * k2x, y + 0.5f * dt * k2y, k3x, k3y);
  ok = ok && velocity(f, uv, sh[2], x + dt * k3x, y + dt * k3y, k4x, k4y);
  if (!ok) return false;
  nx = x + (k1x + 2.f * k2x + 2.f * k3x + k4x) * (dt * (1.0f / 6.0f));
  ny = y + (k1y + 2.f * k2y + 2.f * k3y + k4y) * (dt * (1.0f / 6.0f));
  return true;
}

}  // namespace lm
