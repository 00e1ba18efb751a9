/* CPU oracle of the lagrangian-microbes hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm as the
 * checker and the timed CPU restatement; never by the product path (liblmgb300.so).
 *
 * Restates, in plain C, the reference's algorithm for each piece of the path:
 *   orc_advect_f64 / orc_advect_f32 : RK4 of pset.execute(parcels.AdvectionRK4, runtime=dt, dt=dt)
 *       on a RectilinearZGrid(mesh="spherical") with interp_method="linear"
 *       (particle_advecter.py:177-187, 220-223): bilinear in lon/lat, linear in time, velocities
 *       converted with u / (1852*60*cos(lat)), v / (1852*60). Parcels itself (2.0.0beta2) is not
 *       vendored; the scheme is restated from its documented kernel and interpolation.
 *       f64 = accuracy oracle; f32 = the Parcels-JIT-like float32 loop used as the CPU baseline,
 *       split into contiguous tiles over threads like particle_advecter.py:38-66,146;
 *       orc_advect_f64d = the f64 scheme on a float64 field, the forward of the adjoint's central
 *       finite differences (no reference counterpart: the reference does not differentiate); it
 *       can fold the grid cells of every stage evaluation into a per-particle signature, so that a
 *       difference quotient whose two runs sample different cells (straddling an edge of the
 *       piecewise-bilinear field, where the derivative jumps) is recognised and left out;
 *       orc_advect_f64d_dir runs it on the field moved along an int8 direction, u + s du, without
 *       a field-sized float64 copy per difference.
 *   orc_pairs        : cKDTree(X).query_pairs(r, p) (interaction_simulator.py:93-98): all i < j with
 *       Minkowski-p distance <= r on float32 positions promoted to float64; for p = 2 the test is
 *       fl(fl(dx*dx) + fl(dy*dy)) <= fl(r*r) (no FMA; this file must be compiled with
 *       -ffp-contract=off), pinned against scipy's cKDTree by the golden fixtures.
 *   orc_rps_replay   : the sequential pair loop (interaction_simulator.py:104-105) calling
 *       rock_paper_scissors_interaction (interactions.py:13-40), with r drawn per pair from
 *       Philox4x32-10 (Salmon et al., SC'11) keyed by (seed, step, i, j) instead of MT19937.
 *   orc_priority_order / orc_interact_step : the pair order used by the GPU, then the sequential
 *       replay. The order key is a 64-bit order hash of (seed, step, i, j) (SplitMix64's output
 *       function, a bijection: no ties within a step), descending.
 */
#include "lm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u
#define TAG_PAIR 0x50414952u
#define TAG_DIFF 0x44494646u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
    uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += PHILOX_W0;
    k1 += PHILOX_W1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void orc_pair_draw(uint32_t i, uint32_t j, uint32_t step, uint64_t seed, uint64_t* u53, uint64_t* prio) {
  uint32_t ctr[4] = {i, j, step, TAG_PAIR};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  orc_philox4x32_10(ctr, key, o);
  if (u53) *u53 = ((uint64_t)o[0] << 21) | (o[1] >> 11);
  if (prio) *prio = ((uint64_t)o[2] << 32) | o[3];
}

void orc_diffusion_draw(uint32_t p, uint32_t step, uint64_t seed, float* ulat, float* ulon) {
  uint32_t ctr[4] = {p, step, 0u, TAG_DIFF};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  orc_philox4x32_10(ctr, key, o);
  *ulat = (float)(2u * (o[0] >> 9) + 1u) * (1.0f / 8388608.0f) - 1.0f;
  *ulon = (float)(2u * (o[1] >> 9) + 1u) * (1.0f / 8388608.0f) - 1.0f;
}

/* 64-bit order hash: the output function of SplitMix64 (Steele, Lea, Flood, OOPSLA 2014) applied to
 * (i << 32 | j) offset by Weyl multiples of seed and step. */
uint64_t orc_order_hash(uint32_t i, uint32_t j, uint32_t step, uint64_t seed) {
  uint64_t z = (((uint64_t)i << 32) | j) + seed * 0x9E3779B97F4A7C15ull + (uint64_t)step * 0xD1B54A32D192ED03ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Application order key of pair (i < j) at `step`: the order hash alone, descending. */
uint64_t orc_pair_prio(uint32_t i, uint32_t j, uint32_t step, uint64_t seed) { return orc_order_hash(i, j, step, seed); }

uint64_t orc_prob_threshold(double p) {
  if (!(p > 0)) return 0;
  if (p >= 1.0) return (uint64_t)1 << 53;
  return (uint64_t)ceil(ldexp(p, 53));
}

/* ---------------- advection ---------------- */

/* frame bracket on the uniform time axis; returns 0 outside [t0, t_last] */
static int bracket(const orc_field* f, double t, int* k, double* w) {
  double fk = (t - f->t0) / f->dT;
  if (!(fk >= -1e-9 && fk <= (double)(f->nt - 1) + 1e-9)) return 0;
  double kf = floor(fk);
  int kk = (int)fmin(fmax(kf, 0.0), (double)(f->nt - 2));
  double ww = fmin(fmax(fk - kk, 0.0), 1.0);
  if (ww >= 1.0) { kk += 1; ww = 0.0; }
  *k = kk;
  *w = ww;
  return 1;
}

/* 1: ok, 0: out of domain, -1: time outside the axis */
static int vel64(const orc_field* f, double t, double x, double y, double* dlon, double* dlat) {
  int k;
  double w;
  if (!bracket(f, t, &k, &w)) return -1;
  double fx = (x - f->lon0) / f->dlon, fy = (y - f->lat0) / f->dlat;
  if (!(fx >= 0 && fx <= f->nx - 1 && fy >= 0 && fy <= f->ny - 1)) return 0;
  int i = (int)fx, j = (int)fy;
  if (i > f->nx - 2) i = f->nx - 2;
  if (j > f->ny - 2) j = f->ny - 2;
  double a = fx - i, b = fy - j;
  double w00 = (1 - a) * (1 - b), w01 = a * (1 - b), w10 = (1 - a) * b, w11 = a * b;
  size_t base = ((size_t)k * f->ny + j) * f->nx + i;
  size_t nxny = (size_t)f->nx * f->ny;
  double u = 0, v = 0;
  for (int fr = 0; fr < 2; ++fr) {
    double wt = fr == 0 ? 1.0 - w : w;
    if (wt == 0.0) continue;
    size_t q = base + fr * nxny;
    double uu = w00 * f->u[q] + w01 * f->u[q + 1] + w10 * f->u[q + f->nx] + w11 * f->u[q + f->nx + 1];
    double vv = w00 * f->v[q] + w01 * f->v[q + 1] + w10 * f->v[q + f->nx] + w11 * f->v[q + f->nx + 1];
    u += wt * uu;
    v += wt * vv;
  }
  *dlon = u / (1852.0 * 60.0 * cos(y * M_PI / 180.0));
  *dlat = v / (1852.0 * 60.0);
  return 1;
}

int64_t orc_advect_f64(const orc_field* f, int64_t n, double* lon, double* lat, uint8_t* status, double t0,
                       double dt, int n_steps, double* rec_lon, double* rec_lat) {
  int64_t bad = 0;
  for (int s = 0; s < n_steps; ++s) {
    double t = t0 + dt * s;
    for (int64_t p = 0; p < n; ++p) {
      if (status[p] == 0) {
        double x = lon[p], y = lat[p];
        double k1x, k1y, k2x, k2y, k3x, k3y, k4x, k4y;
        int ok = vel64(f, t, x, y, &k1x, &k1y);
        if (ok == 1) ok = vel64(f, t + 0.5 * dt, x + 0.5 * dt * k1x, y + 0.5 * dt * k1y, &k2x, &k2y);
        if (ok == 1) ok = vel64(f, t + 0.5 * dt, x + 0.5 * dt * k2x, y + 0.5 * dt * k2y, &k3x, &k3y);
        if (ok == 1) ok = vel64(f, t + dt, x + dt * k3x, y + dt * k3y, &k4x, &k4y);
        if (ok == 1) {
          lon[p] = x + (k1x + 2 * k2x + 2 * k3x + k4x) * dt / 6.0;
          lat[p] = y + (k1y + 2 * k2y + 2 * k3y + k4y) * dt / 6.0;
        } else if (ok == 0) {
          status[p] = 1;
          ++bad;
        } else {
          return -1;
        }
      }
      if (rec_lon) rec_lon[(size_t)s * n + p] = lon[p];
      if (rec_lat) rec_lat[(size_t)s * n + p] = lat[p];
    }
  }
  return bad;
}

/* The same FP64 scheme on an FP64 field (finite differences along u, v directions need
 * perturbations far below float32 resolution). Stage brackets as bracket(); one thread per particle. */
static int vel64d(const orc_field64* f, const int8_t* du, const int8_t* dv, double s, int k, double w, double x,
                  double y, double* dlon, double* dlat, uint64_t* sig) {
  double fx = (x - f->lon0) / f->dlon, fy = (y - f->lat0) / f->dlat;
  if (!(fx >= 0 && fx <= f->nx - 1 && fy >= 0 && fy <= f->ny - 1)) return 0;
  int i = (int)fx, j = (int)fy;
  if (i > f->nx - 2) i = f->nx - 2;
  if (j > f->ny - 2) j = f->ny - 2;
  *sig = (*sig ^ (uint64_t)((int64_t)j * f->nx + i)) * 0x100000001B3ull; /* FNV-style fold of the cell path */
  double a = fx - i, b = fy - j;
  double w00 = (1 - a) * (1 - b), w01 = a * (1 - b), w10 = (1 - a) * b, w11 = a * b;
  size_t base = ((size_t)k * f->ny + j) * f->nx + i;
  size_t nxny = (size_t)f->nx * f->ny;
  double u = 0, v = 0;
  for (int fr = 0; fr < 2; ++fr) {
    double wt = fr == 0 ? 1.0 - w : w;
    if (wt == 0.0) continue;
    size_t q = base + fr * nxny;
    double u00 = f->u[q], u01 = f->u[q + 1], u10 = f->u[q + f->nx], u11 = f->u[q + f->nx + 1];
    double v00 = f->v[q], v01 = f->v[q + 1], v10 = f->v[q + f->nx], v11 = f->v[q + f->nx + 1];
    if (du) { /* the field moved along an int8 direction: u + s du (finite differences) */
      u00 += s * du[q], u01 += s * du[q + 1], u10 += s * du[q + f->nx], u11 += s * du[q + f->nx + 1];
      v00 += s * dv[q], v01 += s * dv[q + 1], v10 += s * dv[q + f->nx], v11 += s * dv[q + f->nx + 1];
    }
    u += wt * (w00 * u00 + w01 * u01 + w10 * u10 + w11 * u11);
    v += wt * (w00 * v00 + w01 * v01 + w10 * v10 + w11 * v11);
  }
  *dlon = u / (1852.0 * 60.0 * cos(y * M_PI / 180.0));
  *dlat = v / (1852.0 * 60.0);
  return 1;
}

int64_t orc_advect_f64d(const orc_field64* f, int64_t n, double* lon, double* lat, uint8_t* status, double t0,
                        double dt, int n_steps, int n_threads, uint64_t* cell_sig) {
  return orc_advect_f64d_dir(f, NULL, NULL, 0.0, n, lon, lat, status, t0, dt, n_steps, n_threads, cell_sig);
}

int64_t orc_advect_f64d_dir(const orc_field64* f, const int8_t* du, const int8_t* dv, double s_dir, int64_t n,
                            double* lon, double* lat, uint8_t* status, double t0, double dt, int n_steps, int n_threads,
                            uint64_t* cell_sig) {
  const orc_field fk = {NULL, NULL, f->nx, f->ny, f->nt, f->lon0, f->dlon, f->lat0, f->dlat, f->t0, f->dT};
  int64_t bad = 0;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
  for (int s = 0; s < n_steps; ++s) {
    double t = t0 + dt * s;
    int k[3];
    double w[3];
    if (!bracket(&fk, t, &k[0], &w[0]) || !bracket(&fk, t + 0.5 * dt, &k[1], &w[1]) ||
        !bracket(&fk, t + dt, &k[2], &w[2]))
      return -1;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int64_t p = 0; p < n; ++p) {
      if (status[p]) continue;
      double x = lon[p], y = lat[p];
      double k1x, k1y, k2x, k2y, k3x, k3y, k4x, k4y;
      uint64_t sg = cell_sig ? cell_sig[p] : 0;
      int ok = vel64d(f, du, dv, s_dir, k[0], w[0], x, y, &k1x, &k1y, &sg) &&
               vel64d(f, du, dv, s_dir, k[1], w[1], x + 0.5 * dt * k1x, y + 0.5 * dt * k1y, &k2x, &k2y, &sg) &&
               vel64d(f, du, dv, s_dir, k[1], w[1], x + 0.5 * dt * k2x, y + 0.5 * dt * k2y, &k3x, &k3y, &sg) &&
               vel64d(f, du, dv, s_dir, k[2], w[2], x + dt * k3x, y + dt * k3y, &k4x, &k4y, &sg);
      if (cell_sig) cell_sig[p] = sg;
      if (ok) {
        lon[p] = x + (k1x + 2 * k2x + 2 * k3x + k4x) * dt / 6.0;
        lat[p] = y + (k1y + 2 * k2y + 2 * k3y + k4y) * dt / 6.0;
      } else {
        status[p] = 1;
        bad += 1;
      }
    }
  }
  return bad;
}

static int vel32(const orc_field* f, int k, float w, float x, float y, float* dlon, float* dlat) {
  float fx = (x - (float)f->lon0) * (float)(1.0 / f->dlon), fy = (y - (float)f->lat0) * (float)(1.0 / f->dlat);
  if (!(fx >= 0.f && fx <= (float)(f->nx - 1) && fy >= 0.f && fy <= (float)(f->ny - 1))) return 0;
  int i = (int)fx, j = (int)fy;
  if (i > f->nx - 2) i = f->nx - 2;
  if (j > f->ny - 2) j = f->ny - 2;
  float a = fx - i, b = fy - j;
  float w00 = (1 - a) * (1 - b), w01 = a * (1 - b), w10 = (1 - a) * b, w11 = a * b;
  size_t q = ((size_t)k * f->ny + j) * f->nx + i;
  float u = w00 * f->u[q] + w01 * f->u[q + 1] + w10 * f->u[q + f->nx] + w11 * f->u[q + f->nx + 1];
  float v = w00 * f->v[q] + w01 * f->v[q + 1] + w10 * f->v[q + f->nx] + w11 * f->v[q + f->nx + 1];
  if (w != 0.f) {
    q += (size_t)f->nx * f->ny;
    float u1 = w00 * f->u[q] + w01 * f->u[q + 1] + w10 * f->u[q + f->nx] + w11 * f->u[q + f->nx + 1];
    float v1 = w00 * f->v[q] + w01 * f->v[q + 1] + w10 * f->v[q + f->nx] + w11 * f->v[q + f->nx + 1];
    u += w * (u1 - u);
    v += w * (v1 - v);
  }
  *dlon = u / (111120.0f * cosf(y * (float)(M_PI / 180.0)));
  *dlat = v * (1.0f / 111120.0f);
  return 1;
}

int64_t orc_advect_f32(const orc_field* f, int64_t n, float* lon, float* lat, uint8_t* status, double t0, double dt,
                       int n_steps, int n_threads) {
  int64_t bad = 0;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
  for (int s = 0; s < n_steps; ++s) {
    double t = t0 + dt * s;
    int k[3];
    double wd[3];
    if (!bracket(f, t, &k[0], &wd[0]) || !bracket(f, t + 0.5 * dt, &k[1], &wd[1]) || !bracket(f, t + dt, &k[2], &wd[2]))
      return -1;
    float w[3] = {(float)wd[0], (float)wd[1], (float)wd[2]};
    const float h = (float)dt;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int64_t p = 0; p < n; ++p) {
      if (status[p]) continue;
      float x = lon[p], y = lat[p];
      float k1x, k1y, k2x, k2y, k3x, k3y, k4x, k4y;
      int ok = vel32(f, k[0], w[0], x, y, &k1x, &k1y) &&
               vel32(f, k[1], w[1], x + 0.5f * h * k1x, y + 0.5f * h * k1y, &k2x, &k2y) &&
               vel32(f, k[1], w[1], x + 0.5f * h * k2x, y + 0.5f * h * k2y, &k3x, &k3y) &&
               vel32(f, k[2], w[2], x + h * k3x, y + h * k3y, &k4x, &k4y);
      if (ok) {
        lon[p] = x + (k1x + 2.f * k2x + 2.f * k3x + k4x) * (h / 6.f);
        lat[p] = y + (k1y + 2.f * k2y + 2.f * k3y + k4y) * (h / 6.f);
      } else {
        status[p] = 1;
        bad += 1;
      }
    }
  }
  return bad;
}

/* ---------------- pairs ---------------- */

static int within(double r, double r2, int norm, float ax, float ay, float bx, float by) {
  double dx = (double)ax - (double)bx, dy = (double)ay - (double)by;
  if (norm == 2) {
    double sx = dx * dx;
    double sy = dy * dy;
    double d = sx + sy;
    return d <= r2;
  }
  if (norm == 1) return fabs(dx) + fabs(dy) <= r;
  return fmax(fabs(dx), fabs(dy)) <= r;
}

typedef struct {
  uint64_t* v;
  size_t n, cap;
} vec64;

static int push(vec64* a, uint64_t x) {
  if (a->n == a->cap) {
    size_t nc = a->cap ? 2 * a->cap : 1024;
    uint64_t* nv = (uint64_t*)realloc(a->v, nc * sizeof(uint64_t));
    if (!nv) return -1;
    a->v = nv;
    a->cap = nc;
  }
  a->v[a->n++] = x;
  return 0;
}

static int cmp_u64(const void* a, const void* b) {
  uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : x > y;
}

/* All pairs as packed (i << 32 | j), i < j, sorted ascending. Returns count or -1 on failure. */
static int64_t pairs_packed(int64_t n, const float* lon, const float* lat, double r, int norm, int n_threads,
                            uint64_t** out) {
  *out = NULL;
  if (n <= 1) return 0;
  double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
  for (int64_t p = 0; p < n; ++p) {
    if (!isfinite(lon[p]) || !isfinite(lat[p])) continue;
    x0 = fmin(x0, lon[p]); x1 = fmax(x1, lon[p]);
    y0 = fmin(y0, lat[p]); y1 = fmax(y1, lat[p]);
  }
  if (!(x0 <= x1)) return 0;
  double c = r * 1.004;
  double w = x1 - x0, h = y1 - y0;
  if (!(c > 0)) c = fmax(fmax(w, h), 1e-6);
  double ncx_d = floor(w / c) + 3, ncy_d = floor(h / c) + 3;
  if (ncx_d * ncy_d > 1e7) {
    c = fmax(sqrt(fmax(w * h, 1e-300) / 5e6), c);
    ncx_d = floor(w / c) + 3;
    ncy_d = floor(h / c) + 3;
  }
  int64_t ncx = (int64_t)ncx_d, ncy = (int64_t)ncy_d, ncell = ncx * ncy;
  int64_t* cell = (int64_t*)malloc(sizeof(int64_t) * n);
  int64_t* start = (int64_t*)calloc(ncell + 1, sizeof(int64_t));
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * n);
  if (!cell || !start || !order) { free(cell); free(start); free(order); return -1; }
  for (int64_t p = 0; p < n; ++p) {
    if (!isfinite(lon[p]) || !isfinite(lat[p])) { cell[p] = -1; continue; }
    int64_t cx = (int64_t)floor(((double)lon[p] - (x0 - c)) / c), cy = (int64_t)floor(((double)lat[p] - (y0 - c)) / c);
    if (cx < 0) cx = 0;
    if (cx >= ncx) cx = ncx - 1;
    if (cy < 0) cy = 0;
    if (cy >= ncy) cy = ncy - 1;
    cell[p] = cy * ncx + cx;
    start[cell[p] + 1]++;
  }
  for (int64_t k = 0; k < ncell; ++k) start[k + 1] += start[k];
  {
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * ncell);
    if (!fill) { free(cell); free(start); free(order); return -1; }
    memcpy(fill, start, sizeof(int64_t) * ncell);
    for (int64_t p = 0; p < n; ++p)
      if (cell[p] >= 0) order[fill[cell[p]]++] = p;
    free(fill);
  }
  const double r2 = r * r;
  int nt = 1;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
  nt = n_threads > 0 ? n_threads : omp_get_max_threads();
#else
  (void)n_threads;
#endif
  vec64* parts = (vec64*)calloc(nt, sizeof(vec64));
  int failed = 0;
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nt)
  for (int64_t p = 0; p < n; ++p) {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    if (cell[p] < 0) continue;
    int64_t cy = cell[p] / ncx, cx = cell[p] % ncx;
    for (int64_t yy = cy - 1; yy <= cy + 1; ++yy) {
      if (yy < 0 || yy >= ncy) continue;
      for (int64_t xx = cx - 1; xx <= cx + 1; ++xx) {
        if (xx < 0 || xx >= ncx) continue;
        int64_t k = yy * ncx + xx;
        for (int64_t t = start[k]; t < start[k + 1]; ++t) {
          int64_t q = order[t];
          if (q <= p) continue;
          if (within(r, r2, norm, lon[p], lat[p], lon[q], lat[q]))
            if (push(&parts[tid], ((uint64_t)p << 32) | (uint64_t)q)) failed = 1;
        }
      }
    }
  }
  free(cell); free(start); free(order);
  size_t total = 0;
  for (int t = 0; t < nt; ++t) total += parts[t].n;
  uint64_t* all = (uint64_t*)malloc(sizeof(uint64_t) * (total ? total : 1));
  if (!all || failed) {
    for (int t = 0; t < nt; ++t) free(parts[t].v);
    free(parts); free(all);
    return -1;
  }
  size_t o = 0;
  for (int t = 0; t < nt; ++t) {
    if (parts[t].n) memcpy(all + o, parts[t].v, parts[t].n * sizeof(uint64_t));
    o += parts[t].n;
    free(parts[t].v);
  }
  free(parts);
  qsort(all, total, sizeof(uint64_t), cmp_u64);
  *out = all;
  return (int64_t)total;
}

/* The number of pairs of orc_pairs without storing them (the clustered stress workload): the same
 * cell list and distance test, summed per thread. */
int64_t orc_count_pairs(int64_t n, const float* lon, const float* lat, double r, int norm, int n_threads) {
  if (n <= 0) return 0;
  double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
  for (int64_t p = 0; p < n; ++p) {
    if (!(isfinite(lon[p]) && isfinite(lat[p]))) continue;
    if (lon[p] < x0) x0 = lon[p];
    if (lon[p] > x1) x1 = lon[p];
    if (lat[p] < y0) y0 = lat[p];
    if (lat[p] > y1) y1 = lat[p];
  }
  if (!(x0 <= x1)) return 0;
  double c = r > 0 ? r * 1.0001 : 1.0;
  int64_t ncx = (int64_t)((x1 - x0) / c) + 1, ncy = (int64_t)((y1 - y0) / c) + 1;
  while (ncx * ncy > ((int64_t)1 << 26)) {
    c *= 2;
    ncx = (int64_t)((x1 - x0) / c) + 1;
    ncy = (int64_t)((y1 - y0) / c) + 1;
  }
  const int64_t ncell = ncx * ncy;
  int64_t* cell = (int64_t*)malloc(sizeof(int64_t) * n);
  int64_t* start = (int64_t*)calloc(ncell + 1, sizeof(int64_t));
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * n);
  if (!cell || !start || !order) { free(cell); free(start); free(order); return -1; }
  for (int64_t p = 0; p < n; ++p) {
    if (!(isfinite(lon[p]) && isfinite(lat[p]))) { cell[p] = -1; continue; }
    int64_t cx = (int64_t)((lon[p] - x0) / c), cy = (int64_t)((lat[p] - y0) / c);
    if (cx >= ncx) cx = ncx - 1;
    if (cy >= ncy) cy = ncy - 1;
    cell[p] = cy * ncx + cx;
    start[cell[p] + 1]++;
  }
  for (int64_t k = 0; k < ncell; ++k) start[k + 1] += start[k];
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * ncell);
  if (!fill) { free(cell); free(start); free(order); return -1; }
  memcpy(fill, start, sizeof(int64_t) * ncell);
  for (int64_t p = 0; p < n; ++p)
    if (cell[p] >= 0) order[fill[cell[p]]++] = p;
  free(fill);
  const double r2 = r * r;
  int64_t total = 0;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : total)
  for (int64_t p = 0; p < n; ++p) {
    if (cell[p] < 0) continue;
    const int64_t cy = cell[p] / ncx, cx = cell[p] % ncx;
    for (int64_t yy = cy - 1; yy <= cy + 1; ++yy) {
      if (yy < 0 || yy >= ncy) continue;
      for (int64_t xx = cx - 1; xx <= cx + 1; ++xx) {
        if (xx < 0 || xx >= ncx) continue;
        const int64_t k = yy * ncx + xx;
        for (int64_t t = start[k]; t < start[k + 1]; ++t) {
          const int64_t q = order[t];
          if (q > p && within(r, r2, norm, lon[p], lat[p], lon[q], lat[q])) ++total;
        }
      }
    }
  }
  free(cell); free(start); free(order);
  return total;
}

int64_t orc_pairs(int64_t n, const float* lon, const float* lat, double r, int norm, int n_threads, int32_t* pi,
                  int32_t* pj, int64_t cap) {
  uint64_t* all = NULL;
  int64_t m = pairs_packed(n, lon, lat, r, norm, n_threads, &all);
  if (m < 0) return -1;
  if (pi && pj)
    for (int64_t k = 0; k < m && k < cap; ++k) {
      pi[k] = (int32_t)(all[k] >> 32);
      pj[k] = (int32_t)(all[k] & 0xffffffffu);
    }
  free(all);
  return m;
}

/* ---------------- interaction ---------------- */

static int beats(int x, int y) { return (x == 1 && y == 3) || (x == 2 && y == 1) || (x == 3 && y == 2); }

void orc_rps_apply(int8_t* species, int32_t p1, int32_t p2, uint64_t u53, uint64_t t_rs, uint64_t t_pr, uint64_t t_sp) {
  int s1 = species[p1], s2 = species[p2];
  if (s1 == s2) return;
  uint64_t t;
  if ((s1 == 1 && s2 == 3) || (s1 == 3 && s2 == 1)) t = t_rs;
  else if ((s1 == 2 && s2 == 1) || (s1 == 1 && s2 == 2)) t = t_pr;
  else if ((s1 == 3 && s2 == 2) || (s1 == 2 && s2 == 3)) t = t_sp;
  else return;
  int fwd_wins = u53 < t;
  int p1_wins = beats(s1, s2) ? fwd_wins : !fwd_wins;
  if (p1_wins) species[p2] = (int8_t)s1;
  else species[p1] = (int8_t)s2;
}

void orc_rps_replay(int8_t* species, int64_t m, const int32_t* pi, const int32_t* pj, uint32_t step, uint64_t seed,
                    uint64_t t_rs, uint64_t t_pr, uint64_t t_sp) {
  for (int64_t k = 0; k < m; ++k) {
    uint32_t a = (uint32_t)pi[k], b = (uint32_t)pj[k];
    uint64_t u53;
    orc_pair_draw(a < b ? a : b, a < b ? b : a, step, seed, &u53, NULL);
    orc_rps_apply(species, pi[k], pj[k], u53, t_rs, t_pr, t_sp);
  }
}

typedef struct {
  uint64_t prio;
  uint32_t i, j;
} prio_pair;

static int cmp_prio(const void* a, const void* b) {
  const prio_pair* x = (const prio_pair*)a;
  const prio_pair* y = (const prio_pair*)b;
  if (x->prio != y->prio) return x->prio > y->prio ? -1 : 1;  /* descending priority */
  if (x->i != y->i) return x->i < y->i ? -1 : 1;
  if (x->j != y->j) return x->j < y->j ? -1 : 1;
  return 0;
}

/* Reorder (pi, pj) in place into the GPU's application order: descending priority, ties by (i, j). */
void orc_priority_order(int64_t m, int32_t* pi, int32_t* pj, uint32_t step, uint64_t seed) {
  prio_pair* a = (prio_pair*)malloc(sizeof(prio_pair) * (m ? m : 1));
  for (int64_t k = 0; k < m; ++k) {
    uint32_t x = (uint32_t)pi[k], y = (uint32_t)pj[k];
    a[k].i = x < y ? x : y;
    a[k].j = x < y ? y : x;
    a[k].prio = orc_pair_prio(a[k].i, a[k].j, step, seed);
  }
  qsort(a, (size_t)m, sizeof(prio_pair), cmp_prio);
  for (int64_t k = 0; k < m; ++k) {
    pi[k] = (int32_t)a[k].i;
    pj[k] = (int32_t)a[k].j;
  }
  free(a);
}

int64_t orc_interact_step(int64_t n, const float* lon, const float* lat, int8_t* species, double r, int norm,
                          uint64_t t_rs, uint64_t t_pr, uint64_t t_sp, uint64_t seed, uint32_t step, int n_threads) {
  uint64_t* all = NULL;
  int64_t m = pairs_packed(n, lon, lat, r, norm, n_threads, &all);
  if (m < 0) return -1;
  prio_pair* a = (prio_pair*)malloc(sizeof(prio_pair) * (m ? m : 1));
#pragma omp parallel for schedule(static) num_threads(n_threads > 0 ? n_threads : 1) if (m > 100000)
  for (int64_t k = 0; k < m; ++k) {
    a[k].i = (uint32_t)(all[k] >> 32);
    a[k].j = (uint32_t)(all[k] & 0xffffffffu);
    a[k].prio = orc_pair_prio(a[k].i, a[k].j, step, seed);
  }
  free(all);
  qsort(a, (size_t)m, sizeof(prio_pair), cmp_prio);
  for (int64_t k = 0; k < m; ++k) {
    uint64_t u53;
    orc_pair_draw(a[k].i, a[k].j, step, seed, &u53, NULL);
    orc_rps_apply(species, (int32_t)a[k].i, (int32_t)a[k].j, u53, t_rs, t_pr, t_sp);
  }
  free(a);
  return m;
}

/* Fused CPU step sequence (float32 advection + pairs + interaction) for the CPU baseline. */
int64_t orc_run(const orc_field* f, int64_t n, float* lon, float* lat, uint8_t* status, int8_t* species, double t0,
                double dt, int n_steps, uint32_t step0, double r, int norm, uint64_t t_rs, uint64_t t_pr,
                uint64_t t_sp, uint64_t seed, int n_threads) {
  int64_t pairs = 0;
  for (int s = 0; s < n_steps; ++s) {
    if (orc_advect_f32(f, n, lon, lat, status, t0 + dt * s, dt, 1, n_threads) < 0) return -1;
    int64_t m = orc_interact_step(n, lon, lat, species, r, norm, t_rs, t_pr, t_sp, seed, step0 + (uint32_t)s, n_threads);
    if (m < 0) return -1;
    pairs += m;
  }
  return pairs;
}

/* ---- pairwise distance histogram (sandbox/pairwise_distance_histogram_distributed.jl) ----
 * haversine_distance32 (:35-46) evaluated in float64 on the float32 inputs:
 *   a = sin(pi dlat / 360)^2 + cos(pi lat1 / 180) cos(pi lat2 / 180) sin(pi dlon / 360)^2,
 *   d = radius * 2 asin(min(1, sqrt(a))),
 * and the bin of pairwise_distance_histogram_1point (:56-66): round(10 log10(max(1, d))). */
double orc_haversine(double lat1, double lon1, double lat2, double lon2, double radius) {
  const double c1 = cos(M_PI * (lat1 / 180.0)), c2 = cos(M_PI * (lat2 / 180.0));
  const double d1 = sin(M_PI * ((lat2 - lat1) / 360.0)), d2 = sin(M_PI * ((lon2 - lon1) / 360.0));
  const double a = d1 * d1 + d2 * d2 * c1 * c2;
  return radius * (2.0 * asin(fmin(1.0, sqrt(a))));
}

/* All pairs i < j: x = 10 log10(max(1, d)). A pair whose x lies within `delta` of a bin boundary
 * k + 1/2 is ambiguous between bins k and k + 1 (float32 rounding may put it on either side) and
 * counted in amb[min(k, bins)]; every other pair in def[min(round(x), bins)] (bins = overflow).
 * def, amb: uint64 [bins + 1], overwritten. */
void orc_distance_histogram(int64_t n, const float* lat, const float* lon, int bins, double radius, double delta,
                            int n_threads, uint64_t* def, uint64_t* amb) {
  const int nb = bins + 1;
  memset(def, 0, sizeof(uint64_t) * nb);
  memset(amb, 0, sizeof(uint64_t) * nb);
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
#pragma omp parallel
  {
    uint64_t* hd = (uint64_t*)calloc((size_t)nb, sizeof(uint64_t));
    uint64_t* ha = (uint64_t*)calloc((size_t)nb, sizeof(uint64_t));
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
      for (int64_t j = i + 1; j < n; ++j) {
        const double d = orc_haversine(lat[i], lon[i], lat[j], lon[j], radius);
        const double x = 10.0 * log10(fmax(1.0, d));
        const double k0 = floor(x);
        const int lo = k0 < bins ? (int)k0 : bins, hi = k0 + 1 < bins ? (int)k0 + 1 : bins;
        if (lo != hi && fabs(x - (k0 + 0.5)) < delta) {
          ha[lo]++;
        } else {
          const double kr = nearbyint(x);
          hd[kr < bins ? (int)kr : bins]++;
        }
      }
    }
#pragma omp critical
    for (int k = 0; k < nb; ++k) {
      def[k] += hd[k];
      amb[k] += ha[k];
    }
    free(hd);
    free(ha);
  }
}
