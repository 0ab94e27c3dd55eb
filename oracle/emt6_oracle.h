/*
 * emt6_oracle.h -- CPU oracle for the EMT6-Ro batched simulation step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (banasraf/EMT6-Ro) used as the checker for the CUDA path.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * The product library never links or calls it.
 *
 * Parity anchors (reference files, paths relative to the reference project):
 *   cell model ........ src/emt6ro/cell/cell.cu:16-100, cell/cell.h:102-136
 *   site step ......... src/emt6ro/site/site.h:62-82
 *   division .......... src/emt6ro/simulation/cell-division.h:10-54
 *   occupied list ..... src/emt6ro/simulation/simulation.cu:41-64
 *   cell kernel ....... src/emt6ro/simulation/simulation.cu:30-39, 66-110
 *   cadence ........... src/emt6ro/simulation/simulation.cu:153-166
 *   ROI + mask ........ src/emt6ro/diffusion/diffusion.cu:16-100
 *   diffusion ......... src/emt6ro/diffusion/diffusion.cu:119-191
 *   living count ...... src/emt6ro/statistics/statistics.cu:9-26
 *   dose lookup ....... src/emt6ro/common/protocol.h:9-18
 * The pinning of this restatement against the reference itself is in
 * tests/golden/ (vectors generated from the reference's own host-compiled
 * cell functions by oracle/build_ref.sh + tests/golden/make_golden.py).
 */
#ifndef EMT6_ORACLE_H_
#define EMT6_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Flat parameter block, same field order as the reference's Parameters
 * (src/emt6ro/parameters/parameters.h:10-70) and as include/emt6ro_gb300.h. */
typedef struct {
  int32_t lattice_height, lattice_width; /* interior dims, border excluded */
  float time_step;                       /* seconds per step */
  float diffusion_coeffs[3];             /* cho, ox, gi */
  float diffusion_time_step;             /* seconds per diffusion substep */
  float metabolism[4][3];                /* aer.prolif, anaer.prolif, aer.quiesc, anaer.quiesc */
  float external_levels[3];
  float death_gi, quiescence_gi, death_gi_production;
  float cycle_times[5][2];               /* (mean, stddev) of g1, s, g2, m, d */
  float delay_time_coeff, delay_time_exp_coeff;
  float survival_prob_coeff, survival_prob_exp_coeff;
  float repair_half_time;
} orc_params;

/* One lattice site, array-of-structs form used at the API boundary. */
typedef struct {
  float cho, ox, gi;
  float time_in_repair, irradiation, repair_delay_time, proliferation_time;
  float cycle_times[5];
  uint8_t mode, phase, state, pad;
} orc_site;

typedef struct {
  float tir, irr, delay, prolif;
  float t[5];
  uint8_t mode, phase;
} orc_cell;

enum { ORC_VACANT = 0, ORC_OCCUPIED = 1, ORC_MOCKED = 2 };

/* Instrumentation counters (src/emt6ro/common/instr.h:33-58). */
typedef struct {
  unsigned long long repair_decisions, repair_kills, irradiation_events, divisions;
  double sum_death_prob;
} orc_instr;

/* ---- random numbers ---------------------------------------------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float orc_expf(float x);
double orc_log_core(double x);
void orc_sincos2pi(double u, double *s, double *c);
void orc_box_muller(uint32_t a, uint32_t b, float *z0, float *z1);
void orc_division_normals(uint64_t seed, uint32_t step, uint32_t sim, uint32_t epoch,
                          float z[5]);
float orc_uniform(uint64_t seed, uint32_t step, uint32_t sim, uint32_t site, uint32_t occ,
                  uint32_t purpose, uint32_t epoch);

/* ---- cell model, single-function hooks (for known-answer tests) --------- */
int orc_update_state(orc_cell *c, const float lv[3], const orc_params *p, uint32_t vac);
int orc_progress_clock(orc_cell *c, float time_step);
void orc_metabolise(const orc_cell *c, float lv[3], const orc_params *p);
void orc_irradiate(orc_cell *c, float dose, const orc_params *p);
float orc_calc_delay(float irr, const orc_params *p);
/* u: the uniform draw used if a repair decision fires.  Returns alive. *drew = 1 if used. */
int orc_try_repair(orc_cell *c, const orc_params *p, int cycle_changed, float u, int *drew);
/* neighbour choice for site (r, c) with uniform u; writes (rr, cc) */
void orc_choose_neighbour(int r, int c, float u, int *rr, int *cc);
void orc_divide_cell(orc_cell *parent, orc_cell *child, const float z[5], const orc_params *p);
/* Site::step on one AoS site with injected draws: u_repair used by tryRepair.
 * Returns 1 if ready to divide.  *drew = 1 if the repair draw was consumed. */
int orc_site_step(orc_site *s, const orc_params *p, uint32_t vac, float dose, float u_repair,
                  int *drew);

/* ---- batched simulator ------------------------------------------------- */
typedef struct orc_batch orc_batch;

/* H, W: full lattice dims including the border ring. */
orc_batch *orc_batch_create(const orc_params *p, int n_sims, uint64_t seed);
void orc_batch_destroy(orc_batch *b);
/* Load an initial state (H*W AoS sites) into simulation `i`; sim_index keys the
 * random stream; protocol is `bins` floats (dose per protocol_resolution steps). */
int orc_batch_set(orc_batch *b, int i, const orc_site *sites, const float *protocol,
                  uint32_t bins, uint32_t resolution, uint32_t length, uint32_t sim_index,
                  uint32_t epoch, uint32_t step0, uint32_t horizon);
/* Advance every simulation by nsteps (clamped at its horizon), nthreads workers. */
void orc_batch_run(orc_batch *b, uint32_t nsteps, int nthreads);
void orc_batch_get(const orc_batch *b, int i, orc_site *out);
void orc_batch_counts(const orc_batch *b, uint32_t *out);
void orc_batch_list(const orc_batch *b, int i, uint16_t *list, uint32_t *n);
void orc_batch_roi(const orc_batch *b, int i, int32_t out[5]);
void orc_batch_instr(const orc_batch *b, orc_instr *out, unsigned long long *hist /*600*/);
/* total free-site diffusion substeps executed (for the roofline count) */
unsigned long long orc_batch_diffused(const orc_batch *b);

/* ---- building blocks, exposed for the tests ---------------------------- */
/* occupied list in the reference's 32-column-stripe order; returns n */
uint32_t orc_rebuild_list(const uint8_t *st, int H, int W, uint16_t *list);
/* ROI {r0, c0, h, w, dist}; mask (h+2)x(w+2) bytes, 1 = fixed at external level */
void orc_find_roi(const uint8_t *st, int H, int W, int32_t roi[5], uint8_t *mask);
/* One step of diffusion on field arrays (3 x H*W) with the given ROI/mask.
 * f32: the project's FP32 formula (bit-exact with the CUDA kernel).
 * f64: the reference's formula evaluated in double (accuracy oracle). */
void orc_diffuse_f32(float *fld, int H, int W, const int32_t roi[5], const uint8_t *mask,
                     const orc_params *p);
void orc_diffuse_f64(double *fld, int H, int W, const int32_t roi[5], const uint8_t *mask,
                     const orc_params *p);
void orc_diffusion_coeffs(const orc_params *p, float k[3], float a[3], float b[3], float d[3],
                          int *nsub);

#ifdef __cplusplus
}
#endif
#endif /* EMT6_ORACLE_H_ */
