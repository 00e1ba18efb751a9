/* CPU oracle of the lagrangian-microbes hot path -- TEST INFRASTRUCTURE ONLY (see lm_oracle.c). */
#ifndef LM_ORACLE_H
#define LM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Velocity field on uniform axes: u, v float32 [nt][ny][nx] (m/s). */
typedef struct orc_field {
  const float* u;
  const float* v;
  int nx, ny, nt;
  double lon0, dlon, lat0, dlat, t0, dT;
} orc_field;

/* The same field with float64 u, v (finite differences of the adjoint). */
typedef struct orc_field64 {
  const double* u;
  const double* v;
  int nx, ny, nt;
  double lon0, dlon, lat0, dlat, t0, dT;
} orc_field64;

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_pair_draw(uint32_t i, uint32_t j, uint32_t step, uint64_t seed, uint64_t* u53, uint64_t* prio);
void orc_diffusion_draw(uint32_t p, uint32_t step, uint64_t seed, float* ulat, float* ulon);
uint64_t orc_prob_threshold(double p);

int64_t orc_advect_f64(const orc_field* f, int64_t n, double* lon, double* lat, uint8_t* status, double t0,
                       double dt, int n_steps, double* rec_lon, double* rec_lat);
int64_t orc_advect_f64d(const orc_field64* f, int64_t n, double* lon, double* lat, uint8_t* status, double t0,
                        double dt, int n_steps, int n_threads, uint64_t* cell_sig);
int64_t orc_advect_f64d_dir(const orc_field64* f, const int8_t* du, const int8_t* dv, double s, int64_t n, double* lon,
                            double* lat, uint8_t* status, double t0, double dt, int n_steps, int n_threads,
                            uint64_t* cell_sig);
int64_t orc_advect_f32(const orc_field* f, int64_t n, float* lon, float* lat, uint8_t* status, double t0, double dt,
                       int n_steps, int n_threads);

int64_t orc_pairs(int64_t n, const float* lon, const float* lat, double r, int norm, int n_threads, int32_t* pi,
                  int32_t* pj, int64_t cap);

int64_t orc_count_pairs(int64_t n, const float* lon, const float* lat, double r, int norm, int n_threads);

void orc_rps_apply(int8_t* species, int32_t p1, int32_t p2, uint64_t u53, uint64_t t_rs, uint64_t t_pr, uint64_t t_sp);
void orc_rps_replay(int8_t* species, int64_t m, const int32_t* pi, const int32_t* pj, uint32_t step, uint64_t seed,
                    uint64_t t_rs, uint64_t t_pr, uint64_t t_sp);
uint64_t orc_order_hash(uint32_t i, uint32_t j, uint32_t step, uint64_t seed);
uint64_t orc_pair_prio(uint32_t i, uint32_t j, uint32_t step, uint64_t seed);
void orc_priority_order(int64_t m, int32_t* pi, int32_t* pj, uint32_t step, uint64_t seed);
int64_t orc_interact_step(int64_t n, const float* lon, const float* lat, int8_t* species, double r, int norm,
                          uint64_t t_rs, uint64_t t_pr, uint64_t t_sp, uint64_t seed, uint32_t step, int n_threads);
int64_t orc_run(const orc_field* f, int64_t n, float* lon, float* lat, uint8_t* status, int8_t* species, double t0,
                double dt, int n_steps, uint32_t step0, double r, int norm, uint64_t t_rs, uint64_t t_pr,
                uint64_t t_sp, uint64_t seed, int n_threads);

double orc_haversine(double lat1, double lon1, double lat2, double lon2, double radius);
void orc_distance_histogram(int64_t n, const float* lat, const float* lon, int bins, double radius, double delta,
                            int n_threads, uint64_t* def, uint64_t* amb);

#ifdef __cplusplus
}
#endif

#endif
