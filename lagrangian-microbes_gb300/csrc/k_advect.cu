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
// One thread per particle slot; every 256-slot block belongs to one ensemble, whose field frames,
// seed and slot base are loaded once per block. The block also reduces the bounding box of its
// advected positions into its ensemble's box (ordered-int atomics), from which the binning grid
// of this step is built.
#include "lm_field.cuh"
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

// Caller-order particles (float64 positions, int8 species) into the padded slot layout: offsets
// from the float32 field origin with the same single rounding as the host path, status OK, and pad
// slots (map < 0) zeroed with status PAD. Reads the caller's page-locked arrays directly.
__global__ void k_particles_in(const double* __restrict__ lon, const double* __restrict__ lat,
                               const int8_t* __restrict__ sp, const int32_t* __restrict__ map, uint32_t S,
                               double org_lon, double org_lat, float* __restrict__ xo, float* __restrict__ yo,
                               int8_t* __restrict__ species, uint8_t* __restrict__ status) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < S; k += gridDim.x * blockDim.x) {
    const int32_t q = map[k];
    if (q < 0) {
      xo[k] = yo[k] = 0.f;
      species[k] = 0;
      status[k] = STATUS_PAD;
      continue;
    }
    xo[k] = (float)__dsub_rn(lon[q], org_lon);
    yo[k] = (float)__dsub_rn(lat[q], org_lat);
    species[k] = sp ? sp[q] : (int8_t)0;
    status[k] = STATUS_OK;
  }
}

void launch_particles_in(const double* lon, const double* lat, const int8_t* sp, const int32_t* map, uint32_t S,
                         double org_lon, double org_lat, float* xo, float* yo, int8_t* species, uint8_t* status,
                         cudaStream_t st) {
  int grid = (int)((S + 255) / 256);
  if (grid > 152 * 16) grid = 152 * 16;
  if (grid < 1) grid = 1;
  k_particles_in<<<grid, 256, 0, st>>>(lon, lat, sp, map, S, org_lon, org_lat, xo, yo, species, status);
}

// Block-level bounding box of valid positions, merged into the ensemble's box (blocks of B threads).
template <int B = SLOT_BLOCK>
__device__ __forceinline__ void block_bbox(bool valid, float x, float y, uint32_t* ebox_e) {
  __shared__ float red[4][B / 32];
  float mnx = valid ? x : INFINITY, mny = valid ? y : INFINITY;
  float mxx = valid ? x : -INFINITY, mxy = valid ? y : -INFINITY;
  for (int o = 16; o > 0; o >>= 1) {
    mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = mnx;
    red[1][w] = mny;
    red[2][w] = mxx;
    red[3][w] = mxy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < B / 32; ++k) {
      mnx = fminf(mnx, red[0][k]);
      mny = fminf(mny, red[1][k]);
      mxx = fmaxf(mxx, red[2][k]);
      mxy = fmaxf(mxy, red[3][k]);
    }
    if (mnx <= mxx) {
      atomicMin(ebox_e + 0, enc_f(mnx));
      atomicMin(ebox_e + 1, enc_f(mny));
      atomicMax(ebox_e + 2, enc_f(mxx));
      atomicMax(ebox_e + 3, enc_f(mxy));
    }
  }
}

// Blocks of B = 128 or 256 threads (a tuning knob, lm_set_tuning): B divides the 256-slot blocks of
// the slot layout, so every block still lies inside one ensemble.
template <int B>
__global__ void __launch_bounds__(B) k_advect(FieldView f, StepArgs a, Bufs b, Ctrl* ctrl) {
  pdl_wait();
  __shared__ Stage sh[3];
  __shared__ uint32_t sh_step;
  __shared__ int sh_skip;
  __shared__ EnsInfo sh_ens;
  __shared__ uint32_t sh_e;
  if (threadIdx.x == 0) {  // the step's stage brackets were computed once by k_step_begin
    for (int k = 0; k < 3; ++k) {
      sh[k].k = ctrl->stage_k[k];
      sh[k].w = ctrl->stage_w[k];
      sh[k].ok = 1;
    }
    sh_step = a.use_ctrl_step ? ctrl->step : a.step0;
    sh_skip = ctrl->halt != 0 || !ctrl->stage_ok;
    sh_e = b.block_ens[(blockIdx.x * (uint32_t)B) / SLOT_BLOCK];
    sh_ens = b.ens[sh_e];
  }
  __syncthreads();
  if (sh_skip) return;
  const uint32_t p = blockIdx.x * (uint32_t)B + threadIdx.x;
  const float2* uv = f.uv + sh_ens.field_off;

  uint32_t st = (p < b.nslots) ? b.status[p] : STATUS_PAD;
  float x = 0.f, y = 0.f;
  if (st != STATUS_PAD) {
    x = b.xo[p];
    y = b.yo[p];
  }
  const float dt = (float)a.dt;
  if (st == STATUS_OK) {
    float nx, ny;
    if (rk4_step(f, uv, sh, dt, x, y, nx, ny)) {
      if (isfinite(nx) && isfinite(ny)) {
        x = nx;
        y = ny;
      } else {
        st = STATUS_NAN;
      }
    } else {
      st = (isfinite(x) && isfinite(y)) ? STATUS_OOB : STATUS_NAN;
    }
    if (st != STATUS_OK) {
      atomicAdd(&ctrl->oob, 1u);
      atomicOr(&ctrl->err, st == STATUS_OOB ? (uint32_t)ERRB_OOB : (uint32_t)ERRB_NAN);
      b.status[p] = (uint8_t)st;
    }
  }
  // Recorded position (before the kick), absolute float32 as the reference stores it.
  const float ax = __fadd_rn(f.org_lon, x), ay = __fadd_rn(f.org_lat, y);
  if (st != STATUS_PAD) {
    b.plon[p] = ax;
    b.plat[p] = ay;
  }
  if (st == STATUS_OK) {
    if (a.kick != 0.f) {
      float ulat, ulon;
      diffusion_draw(p - sh_ens.base, sh_step, sh_ens.seed_lo, sh_ens.seed_hi, &ulat, &ulon);
      y = y + ulat * a.kick;
      x = x + ulon * a.kick;
    }
    b.xo[p] = x;
    b.yo[p] = y;
  }
  block_bbox<B>(st == STATUS_OK, ax, ay, b.ebox + 4 * sh_e);
}

void launch_advect(const FieldView& f, const StepArgs& a, const Bufs& b, Ctrl* ctrl, int threads, cudaStream_t st) {
  if (b.nslots == 0) return;
  if (threads == 128)
    launch_dep(k_advect<128>, dim3((b.nslots + 127) / 128), dim3(128), st, f, a, b, ctrl);
  else
    launch_dep(k_advect<SLOT_BLOCK>, dim3((b.nslots + SLOT_BLOCK - 1) / SLOT_BLOCK), dim3(SLOT_BLOCK), st, f, a, b, ctrl);
}

// Bounding boxes from the recorded positions (two-phase interaction path and step re-runs).
__global__ void __launch_bounds__(SLOT_BLOCK) k_bbox(Bufs b, Ctrl* ctrl, int use_status) {
  pdl_wait();
  if (ctrl->halt) return;
  const uint32_t p = blockIdx.x * SLOT_BLOCK + threadIdx.x;
  const uint32_t e = b.block_ens[blockIdx.x];
  bool valid = p < b.nslots;
  float x = 0.f, y = 0.f;
  if (valid) {
    valid = use_status ? (b.status[p] == STATUS_OK) : (p - b.ens[e].base < b.ens[e].n);
    x = b.plon[p];
    y = b.plat[p];
    valid = valid && isfinite(x) && isfinite(y);
  }
  block_bbox(valid, x, y, b.ebox + 4 * e);
}

void launch_bbox(const Bufs& b, Ctrl* ctrl, bool use_status, cudaStream_t st) {
  if (b.nslots == 0) return;
  launch_dep(k_bbox, dim3((b.nslots + SLOT_BLOCK - 1) / SLOT_BLOCK), dim3(SLOT_BLOCK), st, b, ctrl, use_status ? 1 : 0);
}

// Per-step bookkeeping: reset the per-step counters and the ensemble boxes (start), advance the
// device step counter (end). Within one call the end of a step also does the start of the next
// (k_step_end with `chain`), which saves a launch per step; the counters are reset by the same
// thread that has just accumulated them.
__device__ __forceinline__ void step_begin_body(const Bufs& b, const FieldView& f, const StepArgs& a, int bracket,
                                                Ctrl* ctrl) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t e = t; e < b.n_ens; e += gridDim.x * blockDim.x) {
    b.ebox[4 * e + 0] = 0xffffffffu;  // min: start at the largest encoding
    b.ebox[4 * e + 1] = 0xffffffffu;
    b.ebox[4 * e + 2] = 0u;           // max: start at the smallest encoding
    b.ebox[4 * e + 3] = 0u;
    b.census[4 * e + 0] = b.census[4 * e + 1] = b.census[4 * e + 2] = b.census[4 * e + 3] = 0u;
  }
  if (t == 0) {
    ctrl->act_n = 0;
    ctrl->plog_n = 0;
    ctrl->rounds = 0;
    ctrl->n_valid = 0;
    ctrl->n_dir = 0;
    ctrl->n_long = 0;
    ctrl->ovf_used = 0;
    ctrl->census[0] = ctrl->census[1] = ctrl->census[2] = ctrl->census[3] = 0;
    if (bracket) {  // float64 time arithmetic once per step, not once per advection block
      const uint32_t step = a.use_ctrl_step ? ctrl->step : a.step0;
      const double t0 = a.t_start + (double)(int)(step - a.step0) * a.dt;
      const double ts[3] = {t0, t0 + 0.5 * a.dt, t0 + a.dt};
      int ok = 1;
      for (int k = 0; k < 3; ++k) {
        const Stage sg = stage_at(f, ts[k]);
        ctrl->stage_k[k] = sg.k;
        ctrl->stage_w[k] = sg.w;
        ok = ok && sg.ok;
      }
      ctrl->stage_ok = ok;
      if (!ok) atomicOr(&ctrl->err, (uint32_t)ERRB_TIME);
    }
  }
}

__global__ void k_step_begin(Bufs b, FieldView f, StepArgs a, int bracket, Ctrl* ctrl) {
  pdl_wait();
  if (ctrl->halt) return;
  step_begin_body(b, f, a, bracket, ctrl);
}

// End of a step; with `chain`, also the start of the next one (`an` its arguments).
__global__ void k_step_end(Bufs b, FieldView f, StepArgs an, int bracket, Ctrl* ctrl, int interact, int chain) {
  pdl_wait();
  if (ctrl->halt) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (interact) {
      ctrl->pairs_total += ctrl->n_dir / 2;
      ctrl->steps_total += 1;
      ctrl->rounds_total += ctrl->rounds;
    }
    ctrl->step += 1;
  }
  if (chain) step_begin_body(b, f, an, bracket, ctrl);
}

static int bookkeeping_grid(const Bufs& b) {
  int grid = (int)((b.n_ens + 255) / 256);
  if (grid < 1) grid = 1;
  if (grid > 64) grid = 64;
  return grid;
}

void launch_step_begin(const Bufs& b, const FieldView* f, const StepArgs& a, Ctrl* ctrl, cudaStream_t st) {
  FieldView fv{};
  if (f) fv = *f;
  launch_dep(k_step_begin, dim3(bookkeeping_grid(b)), dim3(256), st, b, fv, a, f ? 1 : 0, ctrl);
}
void launch_step_end(Ctrl* ctrl, bool interact, cudaStream_t st) {
  launch_dep(k_step_end, dim3(1), dim3(1), st, Bufs{}, FieldView{}, StepArgs{}, 0, ctrl, interact ? 1 : 0, 0);
}
void launch_step_turn(const Bufs& b, const FieldView* f, const StepArgs& an, Ctrl* ctrl, bool interact,
                      cudaStream_t st) {
  FieldView fv{};
  if (f) fv = *f;
  launch_dep(k_step_end, dim3(bookkeeping_grid(b)), dim3(256), st, b, fv, an, f ? 1 : 0, ctrl, interact ? 1 : 0, 1);
}

// Gathers from the padded slot layout into caller order (map[slot] = caller index or -1).
template <class T>
__global__ void k_unpad(const T* __restrict__ src, T* __restrict__ dst, const int32_t* __restrict__ map, uint32_t n) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int32_t q = map[p];
  if (q >= 0) dst[q] = src[p];
}

void launch_unpad(const float* src, float* dst, const int32_t* map, uint32_t nslots, cudaStream_t st) {
  if (nslots) k_unpad<float><<<(nslots + 255) / 256, 256, 0, st>>>(src, dst, map, nslots);
}
void launch_unpad8(const int8_t* src, int8_t* dst, const int32_t* map, uint32_t nslots, cudaStream_t st) {
  if (nslots) k_unpad<int8_t><<<(nslots + 255) / 256, 256, 0, st>>>(src, dst, map, nslots);
}

}  // namespace lm
