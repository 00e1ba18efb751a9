// K1: classical RK4 advection through a gridded, time-varying velocity field, bilinear in space,
// linear in time, with the m/s -> deg/s metric terms of a spherical lon/lat mesh done in-register.
//
// Semantics follow the reference's advection call, pset.execute(parcels.AdvectionRK4, runtime=dt,
// dt=dt) on a RectilinearZGrid(mesh="spherical") with interp_method="linear"
// (particle_advecter.py:177-187, 220-223): four velocity evaluations at t, t+dt/2, t+dt/2, t+dt,
// each converted with u / (1852*60*cos(lat)) and v / (1852*60), then
// x += dt/6 (k1 + 2 k2 + 2 k3 + k4). The optional diffusion kick of particle_advecter.py:239-244
// (lat first, then lon, uniform in (-1,1) times sqrt(6 |dt| Kh)) is fused and applied after the
// position is recorded, as in the reference.
//
// The same kernel writes the binning input of the pair search (cell key + particle id, absolute
// float32 position), so the advected positions never make a separate trip through HBM.
#include "lm_internal.h"
#include "lm_philox.cuh"

namespace lm {

__global__ void k_interleave(const float* __restrict__ u, const float* __restrict__ v, float2* __restrict__ uv,
                             size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    uv[i] = make_float2(u[i], v[i]);
}

void launch_interleave(const float* u, const float* v, float2* uv, size_t n, cudaStream_t st) {
  int grid = (int)((n + 255) / 256);
  if (grid > 152 * 32) grid = 152 * 32;
  if (grid < 1) grid = 1;
  k_interleave<<<grid, 256, 0, st>>>(u, v, uv, n);
}

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

// Velocity in deg/s at offset position (xo, yo). Returns false outside the grid or on NaN.
__device__ __forceinline__ bool velocity(const FieldView& f, const Stage& s, float xo, float yo, float& dlon,
                                         float& dlat) {
  float fx = (xo - f.gx0) * f.inv_dx;
  float fy = (yo - f.gy0) * f.inv_dy;
  if (!(fx >= 0.f && fx <= f.max_fx && fy >= 0.f && fy <= f.max_fy)) return false;
  int i = min((int)fx, f.nx - 2);
  int j = min((int)fy, f.ny - 2);
  float a = fx - (float)i, b = fy - (float)j;
  const float2* p = f.uv + ((size_t)s.k * f.ny + j) * f.nx + i;
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
  // 1 degree of latitude = 1852 m * 60 (the nautical-mile convention of a spherical mesh).
  float lat = f.org_lat + yo;
  float c = cospif(lat * (1.0f / 180.0f));
  dlon = u / (111120.0f * c);
  dlat = v * (1.0f / 111120.0f);
  return true;
}

__device__ __forceinline__ uint32_t cell_key(const CellGrid& g, float ax, float ay) {
  float fx = (ax - g.x0) * g.inv_c;
  float fy = (ay - g.y0) * g.inv_c;
  fx = fminf(fmaxf(fx, 0.f), (float)(g.ncx - 1));
  fy = fminf(fmaxf(fy, 0.f), (float)(g.ncy - 1));
  return (uint32_t)(int)fy * (uint32_t)g.ncx + (uint32_t)(int)fx;
}

__global__ void __launch_bounds__(256) k_advect(FieldView f, CellGrid g, StepArgs a, Ctrl* ctrl,
                                                float* __restrict__ xo, float* __restrict__ yo,
                                                uint8_t* __restrict__ status, float* __restrict__ plon,
                                                float* __restrict__ plat, uint32_t* __restrict__ key,
                                                uint32_t* __restrict__ id, uint32_t n) {
  __shared__ Stage sh[3];
  __shared__ uint32_t sh_step;
  __shared__ int sh_skip;
  if (threadIdx.x == 0) {
    uint32_t step = a.use_ctrl_step ? ctrl->step : a.step0;
    double t = a.t_start + (double)(int)(step - a.step0) * a.dt;
    sh[0] = stage_at(f, t);
    sh[1] = stage_at(f, t + 0.5 * a.dt);
    sh[2] = stage_at(f, t + a.dt);
    sh_step = step;
    int ok = sh[0].ok && sh[1].ok && sh[2].ok;
    sh_skip = ctrl->halt != 0 || !ok;
    if (!ok && blockIdx.x == 0) atomicOr(&ctrl->err, ERRB_TIME);
  }
  __syncthreads();
  if (sh_skip) return;
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;

  float x = xo[p], y = yo[p];
  uint32_t st = status[p];
  const float dt = (float)a.dt;
  if (st == 0) {
    float k1x, k1y, k2x, k2y, k3x, k3y, k4x, k4y;
    bool ok = velocity(f, sh[0], x, y, k1x, k1y);
    ok = ok && velocity(f, sh[1], x + 0.5f * dt * k1x, y + 0.5f * dt * k1y, k2x, k2y);
    ok = ok && velocity(f, sh[1], x + 0.5f * dt * k2x, y + 0.5f * dt * k2y, k3x, k3y);
    ok = ok && velocity(f, sh[2], x + dt * k3x, y + dt * k3y, k4x, k4y);
    if (ok) {
      float nx = x + (k1x + 2.f * k2x + 2.f * k3x + k4x) * (dt * (1.0f / 6.0f));
      float ny = y + (k1y + 2.f * k2y + 2.f * k3y + k4y) * (dt * (1.0f / 6.0f));
      if (isfinite(nx) && isfinite(ny)) {
        x = nx;
        y = ny;
      } else {
        st = 2u;
      }
    } else {
      st = (isfinite(x) && isfinite(y)) ? 1u : 2u;
    }
    if (st) {
      atomicAdd(&ctrl->oob, 1u);
      atomicOr(&ctrl->err, st == 1u ? (uint32_t)ERRB_OOB : (uint32_t)ERRB_NAN);
      status[p] = (uint8_t)st;
    }
  }
  // Recorded position (before the kick), absolute float32 as the reference stores it.
  float ax = __fadd_rn(f.org_lon, x), ay = __fadd_rn(f.org_lat, y);
  plon[p] = ax;
  plat[p] = ay;
  key[p] = st ? g.ncells : cell_key(g, ax, ay);
  id[p] = p;
  if (a.kick != 0.f && st == 0) {
    float ulat, ulon;
    diffusion_draw(p, sh_step, a.seed_lo, a.seed_hi, &ulat, &ulon);
    y = y + ulat * a.kick;
    x = x + ulon * a.kick;
    xo[p] = x;
    yo[p] = y;
  } else if (st == 0) {
    xo[p] = x;
    yo[p] = y;
  }
}

void launch_advect(const FieldView& f, const CellGrid& g, const StepArgs& a, Ctrl* ctrl, float* xo, float* yo,
                   uint8_t* status, float* plon, float* plat, uint32_t* key, uint32_t* id, uint32_t n,
                   cudaStream_t st) {
  if (n == 0) return;
  k_advect<<<(n + 255) / 256, 256, 0, st>>>(f, g, a, ctrl, xo, yo, status, plon, plat, key, id, n);
}

// Binning input from externally supplied positions (the interaction phase of the two-phase
// reference workflow, interaction_simulator.py:88-93, reads positions from particle_data.nc).
__global__ void k_keys_from_pos(CellGrid g, Ctrl* ctrl, const float* __restrict__ lon, const float* __restrict__ lat,
                                uint32_t* __restrict__ key, uint32_t* __restrict__ id, uint32_t n) {
  if (ctrl->halt) return;
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  float ax = lon[p], ay = lat[p];
  bool ok = isfinite(ax) && isfinite(ay);
  key[p] = ok ? cell_key(g, ax, ay) : g.ncells;
  id[p] = p;
  if (!ok) atomicOr(&ctrl->err, (uint32_t)ERRB_NAN);
}

void launch_keys_from_pos(const CellGrid& g, Ctrl* ctrl, const float* lon, const float* lat, uint32_t* key,
                          uint32_t* id, uint32_t n, cudaStream_t st) {
  if (n == 0) return;
  k_keys_from_pos<<<(n + 255) / 256, 256, 0, st>>>(g, ctrl, lon, lat, key, id, n);
}

}  // namespace lm
