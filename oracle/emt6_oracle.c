/*
 * emt6_oracle.c -- CPU oracle for the EMT6-Ro batched simulation step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, never the product.
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fPIC -shared (see oracle/build.py).
 * -ffp-contract=off is part of the contract: every float expression below is
 * evaluated exactly as written (no fused multiply-add unless fmaf/fma is
 * called), which is also how the CUDA library is compiled (--fmad=false).
 *
 * Semantics restated from the reference (paths relative to its project root):
 *  - Cell model: src/emt6ro/cell/cell.cu:16-100 and cell/cell.h:102-136.
 *  - Site::step composition: src/emt6ro/site/site.h:62-82.
 *  - Division: src/emt6ro/simulation/cell-division.h:10-54.
 *  - Occupied list order: src/emt6ro/simulation/simulation.cu:41-64 (32 column
 *    stripes, each stripe row-major, stripes concatenated in order).
 *  - Cell kernel: simulation.cu:66-110.  Resolutions of the reference's data
 *    races, shared with the CUDA path:
 *      * the 8-neighbour vacancy snapshot is taken before any site is updated
 *        (as the reference does, simulation.cu:79-83);
 *      * a division target is valid if it is VACANT after all of this step's
 *        updates (the reference reads it while other threads write);
 *      * among valid candidates the lowest occupied-list index wins (equal to
 *        the reference's lowest-thread rule for lists of <= 512 entries);
 *      * a site listed k times (a dead entry revived before the next rebuild,
 *        simulation.cu:105 + :154) is stepped k times, in list order.
 *  - Cadence: list rebuild every 128 steps, ROI every 32 (simulation.cu:153-166).
 *  - ROI/mask: src/emt6ro/diffusion/diffusion.cu:16-100.
 *  - Diffusion: diffusion.cu:135-191 (23 substeps over free sites, one final
 *    substep over the whole ROI, write-back of the ROI).
 *  - Living count: src/emt6ro/statistics/statistics.cu:9-26.
 *  - Dose lookup: src/emt6ro/common/protocol.h:9-18.
 * Randomness: Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel Random
 * Numbers: As Easy as 1, 2, 3", SC'11) keyed by the seed, counter = (step,
 * simulation, site | occurrence<<16 | purpose<<24, epoch).  The reference uses
 * curand XORWOW per thread (random-engine.cu:8-39); parity at that boundary is
 * distributional.  Transcendentals that feed the state (exp for repair delay
 * and survival, log/sin/cos for normals) are evaluated by the double-precision
 * routines below, written from Cody-Waite reduction + Taylor/atanh series,
 * using only IEEE-exact basic operations and fma so the CPU and the GPU produce
 * identical bits.
 *
 * When compiled with -DORC_REF_CELL (oracle/build_ref.sh only) the per-site
 * model calls are routed to the reference's own host-compiled functions and
 * its std::mt19937 engine, and diffusion uses the reference's own summation
 * order in FP32; that build generates the distribution fixtures.
 */
#include "emt6_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================== */
/* Philox4x32-10                                                             */
/* ======================================================================== */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int i = 0; i < 10; ++i) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline void orc_draw(uint64_t seed, uint32_t step, uint32_t sim, uint32_t site,
                            uint32_t occ, uint32_t purpose, uint32_t epoch, uint32_t out[4]) {
  uint32_t ctr[4] = {step, sim, (site & 0xFFFFu) | ((occ & 0xFFu) << 16) | (purpose << 24),
                     epoch};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  orc_philox4x32_10(ctr, key, out);
}

/* uniform in (0, 1], like curand_uniform (random-engine.cu:33-35) */
static inline float orc_u01(uint32_t x) { return (float)((x >> 8) + 1u) * 0x1p-24f; }

float orc_uniform(uint64_t seed, uint32_t step, uint32_t sim, uint32_t site, uint32_t occ,
                  uint32_t purpose, uint32_t epoch) {
  uint32_t r[4];
  orc_draw(seed, step, sim, site, occ, purpose, epoch, r);
  return orc_u01(r[0]);
}

/* ======================================================================== */
/* double-precision kernels shared bit-for-bit with the CUDA path            */
/* ======================================================================== */
static inline double orc_bits2d(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static inline uint64_t orc_d2bits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }

/* exp(x) for |x| < 700: k = rint(x/ln2), r = x - k*ln2 (Cody-Waite, ln2 split
 * hi/lo, fused), exp(r) by its Taylor series to degree 13, times 2^k. */
static double orc_exp_core(double x) {
  double k = rint(x * 0x1.71547652b82fep+0);
  double r = fma(-k, 0x1.62e42fefa39efp-1, x);
  r = fma(-k, 0x1.abc9e3b39803fp-56, r);
  double q = 0x1.6124613a86d09p-33;
  q = fma(q, r, 0x1.1eed8eff8d898p-29);
  q = fma(q, r, 0x1.ae64567f544e4p-26);
  q = fma(q, r, 0x1.27e4fb7789f5cp-22);
  q = fma(q, r, 0x1.71de3a556c734p-19);
  q = fma(q, r, 0x1.a01a01a01a01ap-16);
  q = fma(q, r, 0x1.a01a01a01a01ap-13);
  q = fma(q, r, 0x1.6c16c16c16c17p-10);
  q = fma(q, r, 0x1.1111111111111p-7);
  q = fma(q, r, 0x1.5555555555555p-5);
  q = fma(q, r, 0x1.5555555555555p-3);
  q = fma(q, r, 0x1.0000000000000p-1);
  q = fma(q, r, 1.0);
  q = fma(q, r, 1.0);
  return q * orc_bits2d((uint64_t)((int64_t)k + 1023) << 52);
}

float orc_expf(float x) { return (float)orc_exp_core((double)x); }

/* log(x), x normal and positive: x = m 2^e, m in [sqrt(1/2), sqrt(2)),
 * log(m) = 2 atanh(s), s = (m-1)/(m+1), series to s^23. */
double orc_log_core(double x) {
  uint64_t b = orc_d2bits(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  double m = orc_bits2d((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  if (m > 0x1.6a09e667f3bcdp+0) { m *= 0.5; e += 1; }
  double s = (m - 1.0) / (m + 1.0);
  double s2 = s * s;
  double q = 0x1.642c8590b2164p-5;
  q = fma(q, s2, 0x1.8618618618618p-5);
  q = fma(q, s2, 0x1.af286bca1af28p-5);
  q = fma(q, s2, 0x1.e1e1e1e1e1e1ep-5);
  q = fma(q, s2, 0x1.1111111111111p-4);
  q = fma(q, s2, 0x1.3b13b13b13b14p-4);
  q = fma(q, s2, 0x1.745d1745d1746p-4);
  q = fma(q, s2, 0x1.c71c71c71c71cp-4);
  q = fma(q, s2, 0x1.2492492492492p-3);
  q = fma(q, s2, 0x1.999999999999ap-3);
  q = fma(q, s2, 0x1.5555555555555p-2);
  double s2x = 2.0 * s;
  double lm = fma(s2x * s2, q, s2x);
  double de = (double)e;
  return fma(de, 0x1.62e42fefa39efp-1, fma(de, 0x1.abc9e3b39803fp-56, lm));
}

/* sin/cos of 2*pi*u for u in [0, 1): exact quarter-turn reduction on u, then
 * Taylor series on |a| <= pi/4. */
void orc_sincos2pi(double u, double *s_out, double *c_out) {
  double q = floor(u * 4.0);
  double t = u - q * 0.25;
  if (t > 0.125) { t -= 0.25; q += 1.0; }
  double a = t * 0x1.921fb54442d18p+2;
  double a2 = a * a;
  double ps = 0x1.952c77030ad4ap-49;
  ps = fma(ps, a2, -0x1.ae7f3e733b81fp-41);
  ps = fma(ps, a2, 0x1.6124613a86d09p-33);
  ps = fma(ps, a2, -0x1.ae64567f544e4p-26);
  ps = fma(ps, a2, 0x1.71de3a556c734p-19);
  ps = fma(ps, a2, -0x1.a01a01a01a01ap-13);
  ps = fma(ps, a2, 0x1.1111111111111p-7);
  ps = fma(ps, a2, -0x1.5555555555555p-3);
  double sn = fma(a * a2, ps, a);
  double pc = -0x1.6827863b97d97p-53;
  pc = fma(pc, a2, 0x1.ae7f3e733b81fp-45);
  pc = fma(pc, a2, -0x1.93974a8c07c9dp-37);
  pc = fma(pc, a2, 0x1.1eed8eff8d898p-29);
  pc = fma(pc, a2, -0x1.27e4fb7789f5cp-22);
  pc = fma(pc, a2, 0x1.a01a01a01a01ap-16);
  pc = fma(pc, a2, -0x1.6c16c16c16c17p-10);
  pc = fma(pc, a2, 0x1.5555555555555p-5);
  pc = fma(pc, a2, -0x1.0000000000000p-1);
  double cs = fma(a2, pc, 1.0);
  int qi = ((int)q) & 3;
  switch (qi) {
    case 0: *s_out = sn; *c_out = cs; break;
    case 1: *s_out = cs; *c_out = -sn; break;
    case 2: *s_out = -sn; *c_out = -cs; break;
    default: *s_out = -cs; *c_out = sn; break;
  }
}

/* Box-Muller pair from two 32-bit words: u1 in (0,1], u2 in [0,1). */
void orc_box_muller(uint32_t a, uint32_t b, float *z0, float *z1) {
  float u1 = orc_u01(a);
  float u2 = (float)(b >> 8) * 0x1p-24f;
  double r = sqrt(-2.0 * orc_log_core((double)u1));
  double s, c;
  orc_sincos2pi((double)u2, &s, &c);
  *z0 = (float)(r * c);
  *z1 = (float)(r * s);
}

/* The five standard normals of one division (one per cycle phase). */
void orc_division_normals(uint64_t seed, uint32_t step, uint32_t sim, uint32_t epoch,
                          float z[5]) {
  uint32_t r1[4], r2[4];
  float unused;
  orc_draw(seed, step, sim, 0xFFFFu, 0, 2, epoch, r1);
  orc_draw(seed, step, sim, 0xFFFFu, 0, 3, epoch, r2);
  orc_box_muller(r1[0], r1[1], &z[0], &z[1]);
  orc_box_muller(r1[2], r1[3], &z[2], &z[3]);
  orc_box_muller(r2[0], r2[1], &z[4], &unused);
}

/* ======================================================================== */
/* cell model (src/emt6ro/cell/cell.cu, cell.h)                              */
/* ======================================================================== */
int orc_update_state(orc_cell *c, const float lv[3], const orc_params *p, uint32_t vac) {
  /* cell.cu:72-82 */
  if (c->prolif >= c->t[4] - p->time_step / 3600.f) return 0;
  /* enterG1SStopping, cell.cu:67-70 */
  int g1s = c->prolif > (c->t[0] - 2 * p->time_step / 3600.f) && c->phase == 0 && vac <= 1;
  if (!g1s) {
    /* tryProliferating, cell.cu:33-47 */
    if (lv[0] >= p->metabolism[0][0] && lv[1] >= p->metabolism[0][1] &&
        lv[2] < p->quiescence_gi) {
      c->mode = 0;
      return 1;
    } else if (lv[0] >= p->metabolism[1][0] && lv[1] >= p->metabolism[1][1] &&
               lv[2] < p->quiescence_gi) {
      c->mode = 1;
      return 1;
    }
  }
  /* tryQuiescence, cell.cu:49-65 */
  if (c->phase != 0 && c->phase != 2) return 0;
  if (lv[0] >= p->metabolism[2][0] && lv[1] >= p->metabolism[2][1] && lv[2] < p->death_gi) {
    c->mode = 2;
    return 1;
  } else if (lv[0] >= p->metabolism[3][0] && lv[1] >= p->metabolism[3][1] &&
             lv[2] < p->death_gi) {
    c->mode = 3;
    return 1;
  }
  return 0;
}

int orc_progress_clock(orc_cell *c, float time_step) {
  /* cell.cu:21-32 */
  if ((c->mode == 0 || c->mode == 1) && c->tir == 0) {
    c->prolif += time_step / 3600;
    uint8_t cur = c->phase;
    c->phase = (uint8_t)(cur + (uint8_t)(c->prolif > c->t[cur]));
    return c->phase != cur && c->phase != 4;
  }
  return 0;
}

void orc_metabolise(const orc_cell *c, float lv[3], const orc_params *p) {
  /* cell.cu:16-19 */
  lv[0] -= p->metabolism[c->mode][0];
  lv[1] -= p->metabolism[c->mode][1];
  lv[2] -= p->metabolism[c->mode][2];
}

float orc_calc_delay(float irr, const orc_params *p) {
  /* cell.cu:93-100 */
  return p->delay_time_coeff * orc_expf(p->delay_time_exp_coeff * irr);
}

void orc_irradiate(orc_cell *c, float dose, const orc_params *p) {
  /* cell.cu:84-91 */
  c->irr = c->irr / (1 + c->tir / p->repair_half_time) + dose;
  c->tir = 0;
  c->delay = orc_calc_delay(c->irr, p);
}

/* first half of tryRepair (cell.h:102-107): advance the repair clock and say
 * whether the survival decision fires this step */
static inline int orc_repair_pre(orc_cell *c, const orc_params *p, int cycle_changed) {
  if (c->tir > 0 || (c->irr > 0 && cycle_changed)) {
    c->tir += p->time_step / 3600.f;
    if (c->tir >= c->delay) return 1;
  }
  return 0;
}

static inline float orc_death_prob(const orc_cell *c, const orc_params *p) {
  /* cell.h:108-110 */
  return 1 - p->survival_prob_coeff * orc_expf(p->survival_prob_exp_coeff * c->irr);
}

/* second half (cell.h:124-133): returns alive */
static inline int orc_repair_post(orc_cell *c, float death_prob, float u) {
  if (u < death_prob) return 0;
  c->irr = 0.f;
  c->tir = 0.f;
  c->delay = 0.f;
  return 1;
}

int orc_try_repair(orc_cell *c, const orc_params *p, int cycle_changed, float u, int *drew) {
  *drew = 0;
  if (!orc_repair_pre(c, p, cycle_changed)) return 1;
  *drew = 1;
  return orc_repair_post(c, orc_death_prob(c, p), u);
}

void orc_choose_neighbour(int r, int c, float u, int *rr, int *cc) {
  /* cell-division.h:32-54 */
  const float diag_prob = 4.f;
  const float ortho_prob = (float)(4. * 1.41421356237309504880);
  float score = u * (diag_prob + ortho_prob);
  if (score < diag_prob) {
    uint8_t num = (uint8_t)score;
    int vert = (num & 1u) * 2 - 1;
    int hor = ((num & 2u) >> 1u) * 2 - 1;
    *rr = r + vert;
    *cc = c + hor;
  } else {
    uint8_t num = (uint8_t)((double)(score - diag_prob) / 1.41421356237309504880);
    int which = num & 1u;
    int diff = ((num & 2u) >> 1u) * 2 - 1;
    if (which) { *rr = r + diff; *cc = c; }
    else { *rr = r; *cc = c + diff; }
  }
}

void orc_divide_cell(orc_cell *parent, orc_cell *child, const float z[5], const orc_params *p) {
  /* cell-division.h:10-30 */
  parent->phase = 0;
  parent->prolif = 0;
  memset(child, 0, sizeof(*child));
  child->t[0] = p->cycle_times[0][1] * z[0] + p->cycle_times[0][0];
  for (int i = 1; i < 5; ++i)
    child->t[i] = child->t[i - 1] + (p->cycle_times[i][1] * z[i] + p->cycle_times[i][0]);
  child->irr = parent->irr;
  if (parent->irr > 0) child->delay = orc_calc_delay(child->irr, p);
}

static void orc_site_to_cell(const orc_site *s, orc_cell *c) {
  c->tir = s->time_in_repair;
  c->irr = s->irradiation;
  c->delay = s->repair_delay_time;
  c->prolif = s->proliferation_time;
  for (int i = 0; i < 5; ++i) c->t[i] = s->cycle_times[i];
  c->mode = s->mode;
  c->phase = s->phase;
}

static void orc_cell_to_site(const orc_cell *c, orc_site *s) {
  s->time_in_repair = c->tir;
  s->irradiation = c->irr;
  s->repair_delay_time = c->delay;
  s->proliferation_time = c->prolif;
  for (int i = 0; i < 5; ++i) s->cycle_times[i] = c->t[i];
  s->mode = c->mode;
  s->phase = c->phase;
}

int orc_site_step(orc_site *s, const orc_params *p, uint32_t vac, float dose, float u_repair,
                  int *drew) {
  /* site.h:62-82 */
  *drew = 0;
  if (s->state != ORC_OCCUPIED) return 0;
  orc_cell c;
  orc_site_to_cell(s, &c);
  float lv[3] = {s->cho, s->ox, s->gi};
  int ready = 0;
  if (orc_update_state(&c, lv, p, vac)) {
    if (dose > 0) orc_irradiate(&c, dose, p);
    orc_metabolise(&c, lv, p);
    int cc = orc_progress_clock(&c, p->time_step);
    if (orc_try_repair(&c, p, cc, u_repair, drew)) ready = c.phase == 4;
    else s->state = ORC_VACANT;
  } else {
    s->state = ORC_VACANT;
  }
  s->cho = lv[0]; s->ox = lv[1]; s->gi = lv[2];
  orc_cell_to_site(&c, s);
  return ready;
}

/* ======================================================================== */
/* occupied list, ROI, diffusion                                             */
/* ======================================================================== */
uint32_t orc_rebuild_list(const uint8_t *st, int H, int W, uint16_t *list) {
  /* simulation.cu:41-64: thread k of 32 walks rows 0..H-2, columns k, k+32, ...
   * < W-1; per-thread collections are concatenated in thread order. */
  uint32_t n = 0;
  for (int k = 0; k < 32; ++k)
    for (int r = 0; r < H - 1; ++r)
      for (int c = k; c < W - 1; c += 32)
        if (st[r * W + c] == ORC_OCCUPIED) list[n++] = (uint16_t)(r * W + c);
  return n;
}

void orc_find_roi(const uint8_t *st, int H, int W, int32_t roi[5], uint8_t *mask) {
  /* diffusion.cu:65-100 */
  int minr = H, minc = W, maxr = 0, maxc = 0;
  for (int r = 0; r < H; ++r)
    for (int c = 0; c < W; ++c)
      if (st[r * W + c] == ORC_OCCUPIED) {
        if (r < minr) minr = r;
        if (c < minc) minc = c;
        if (r > maxr) maxr = r;
        if (c > maxc) maxc = c;
      }
  if (maxr == 0 && maxc == 0) {
    roi[0] = roi[1] = roi[2] = roi[3] = roi[4] = 0;
    return;
  }
  int midr = minr + (maxr - minr + 1) / 2;
  int midc = minc + (maxc - minc + 1) / 2;
  int dist = 0;
  for (int r = minr; r <= maxr; ++r)
    for (int c = minc; c <= maxc; ++c)
      if (st[r * W + c] == ORC_OCCUPIED) {
        float d2 = (float)((midr - r) * (midr - r) + (midc - c) * (midc - c));
        int d = (int)ceilf(sqrtf(d2));
        if (d > dist) dist = d;
      }
  int sub_r = (midr <= dist) ? 1 : midr - dist;
  int sub_c = (midc <= dist) ? 1 : midc - dist;
  int sub_w = (midc + dist >= W - 1) ? W - 1 - sub_c : midc + dist - sub_c + 1;
  int sub_h = (midr + dist >= H - 1) ? H - 1 - sub_r : midr + dist - sub_r + 1;
  roi[0] = sub_r; roi[1] = sub_c; roi[2] = sub_h; roi[3] = sub_w; roi[4] = dist;
  /* fillBorderMask, diffusion.cu:16-30 */
  int mh = sub_h + 2, mw = sub_w + 2;
  float mr = mh / 2.f, mc = mw / 2.f;
  for (int i = 0; i < mh; ++i)
    for (int j = 0; j < mw; ++j) {
      float fr = (float)(i + 1), fc = (float)(j + 1);
      float d = sqrtf((fr - mr) * (fr - mr) + (fc - mc) * (fc - mc));
      mask[i * mw + j] = (d >= (float)dist) ? 1 : 0;
    }
}

void orc_diffusion_coeffs(const orc_params *p, float k[3], float a[3], float b[3], float d[3],
                          int *nsub) {
  /* diffusion.cu:119-120, 163; simulation.cu:170 */
  const float HS = (float)(2 * 1.41421356237309504880);
  const float F = (float)(4. + (double)HS);
  const float S2 = (float)0.70710678118654752440;
  for (int f = 0; f < 3; ++f) {
    k[f] = ((p->diffusion_coeffs[f] * p->diffusion_time_step) * HS) / F;
    a[f] = (float)(1.0 - (double)k[f] * (double)F);
    b[f] = k[f];
    d[f] = (float)((double)k[f] * (double)S2);
  }
  *nsub = (int16_t)(p->time_step / p->diffusion_time_step);
}

/* tile helpers: region rows i in [0, h+2), cols j in [0, w+2), lattice
 * (r0-1+i, c0-1+j); padded by one zero ring (the reference's outer ring). */
#define ORC_TILE(T, i, j) T[((i) + 1) * tw + ((j) + 1)]

/* a where m is all ones, b where m is zero (a bitwise blend, so the loops
 * using it have no branches and vectorise) */
static inline float orc_sel(int32_t m, float a, float b) {
  uint32_t ua, ub;
  memcpy(&ua, &a, 4);
  memcpy(&ub, &b, 4);
  const uint32_t r = (ua & (uint32_t)m) | (ub & ~(uint32_t)m);
  float f;
  memcpy(&f, &r, 4);
  return f;
}

/* Which tile sites a substep updates, as all-ones / zero words so the update
 * loops below are branch-free (and vectorise): free substeps update the
 * sites the mask leaves free, the final substep every ROI site (the interior
 * of the ring).  Positions outside the region stay zero. */
static void orc_update_masks(const uint8_t *mask, int h, int w, int tw, int tn, int32_t *ufree,
                             int32_t *ufin) {
  int nrow = h + 2, ncol = w + 2;
  memset(ufree, 0, sizeof(int32_t) * tn);
  memset(ufin, 0, sizeof(int32_t) * tn);
  for (int i = 0; i < nrow; ++i)
    for (int j = 0; j < ncol; ++j) {
      ORC_TILE(ufree, i, j) = mask[i * ncol + j] ? 0 : -1;
      ORC_TILE(ufin, i, j) = (i >= 1 && i <= h && j >= 1 && j <= w) ? -1 : 0;
    }
}

void orc_diffuse_f32(float *fld, int H, int W, const int32_t roi[5], const uint8_t *mask,
                     const orc_params *p) {
  int r0 = roi[0], c0 = roi[1], h = roi[2], w = roi[3];
  if (h == 0 || w == 0) return;
  float kk[3], a[3], b[3], d[3];
  int nsub;
  orc_diffusion_coeffs(p, kk, a, b, d, &nsub);
  /* rows of the tile are padded to a multiple of 8 columns (zero, never
   * updated) so the substep loops have no remainder iterations */
  int nrow = h + 2, ncol = w + 2, ncp = (ncol + 7) & ~7, tw = ncp + 2, tn = (nrow + 2) * tw;
  /* X, Y: the field tile with the zero outer ring; Hs, G per site; the rows
   * of G above and below the region stay zero (the ring's G) */
  float *X = (float *)calloc((size_t)tn, sizeof(float));
  float *Y = (float *)calloc((size_t)tn, sizeof(float));
  float *Hs = (float *)calloc((size_t)tn, sizeof(float));
  float *G = (float *)calloc((size_t)tn, sizeof(float));
  int32_t *ufree = (int32_t *)malloc(sizeof(int32_t) * (size_t)tn);
  int32_t *ufin = (int32_t *)malloc(sizeof(int32_t) * (size_t)tn);
  orc_update_masks(mask, h, w, tw, tn, ufree, ufin);
  int nfree = nsub - 1 > 0 ? nsub - 1 : 0;
  for (int f = 0; f < 3; ++f) {
    float *L = fld + (size_t)f * H * W;
    const float ext = p->external_levels[f], fa = a[f], fb = b[f], fd = d[f];
    memset(X, 0, sizeof(float) * tn);
    memset(Y, 0, sizeof(float) * tn);
    for (int i = 0; i < nrow; ++i)
      for (int j = 0; j < ncol; ++j)
        ORC_TILE(X, i, j) = mask[i * ncol + j] ? ext : L[(r0 - 1 + i) * W + (c0 - 1 + j)];
    for (int s = 0; s <= nfree; ++s) {
      const int32_t *U = (s == nfree) ? ufin : ufree;
      /* H = left + right, G = b*x + d*H (rounded as fmaf(d, H, b*x));
       * x' = a*x + b*(H + up + down) + d*(H_up + H_down)
       *    = fmaf(a, x, fmaf(b, H, G_up + G_down)) */
      for (int i = 0; i < nrow; ++i) {
        const float *restrict x = &ORC_TILE(X, i, 0);
        float *restrict hs = &ORC_TILE(Hs, i, 0), *restrict g = &ORC_TILE(G, i, 0);
        for (int j = 0; j < ncp; ++j) {
          const float hv = x[j - 1] + x[j + 1];
          hs[j] = hv;
          g[j] = fmaf(fd, hv, fb * x[j]);
        }
      }
      for (int i = 0; i < nrow; ++i) {
        const float *restrict x = &ORC_TILE(X, i, 0), *restrict hs = &ORC_TILE(Hs, i, 0);
        const float *restrict gu = &ORC_TILE(G, i - 1, 0), *restrict gd = &ORC_TILE(G, i + 1, 0);
        const int32_t *restrict u = &ORC_TILE(U, i, 0);
        float *restrict y = &ORC_TILE(Y, i, 0);
        for (int j = 0; j < ncp; ++j) {
          const float nv = fmaf(fa, x[j], fmaf(fb, hs[j], gu[j] + gd[j]));
          y[j] = orc_sel(u[j], nv, x[j]);
        }
      }
      float *tmp = X; X = Y; Y = tmp;
    }
    for (int i = 1; i <= h; ++i)
      for (int j = 1; j <= w; ++j) L[(r0 - 1 + i) * W + (c0 - 1 + j)] = ORC_TILE(X, i, j);
  }
  free(X); free(Y); free(Hs); free(G); free(ufree); free(ufin);
}

/* The reference's own expression (diffusion.cu:122-133) in FP32, used by the
 * ORC_REF_CELL build for the reference CPU path.  The increment of every
 * site is computed from the substep's old values, then added where the
 * substep updates (diffusion.cu:172-188). */
static void orc_diffuse_ref_f32(float *fld, int H, int W, const int32_t roi[5],
                                const uint8_t *mask, const orc_params *p) {
  int r0 = roi[0], c0 = roi[1], h = roi[2], w = roi[3];
  if (h == 0 || w == 0) return;
  float kk[3], a[3], b[3], d[3];
  int nsub;
  orc_diffusion_coeffs(p, kk, a, b, d, &nsub);
  const float S2 = (float)0.70710678118654752440;
  const float F = (float)(4. + (double)(float)(2 * 1.41421356237309504880));
  /* rows of the tile are padded to a multiple of 8 columns (zero, never
   * updated) so the substep loops have no remainder iterations */
  int nrow = h + 2, ncol = w + 2, ncp = (ncol + 7) & ~7, tw = ncp + 2, tn = (nrow + 2) * tw;
  float *X = (float *)calloc((size_t)tn, sizeof(float));
  float *D = (float *)calloc((size_t)tn, sizeof(float));
  int32_t *ufree = (int32_t *)malloc(sizeof(int32_t) * (size_t)tn);
  int32_t *ufin = (int32_t *)malloc(sizeof(int32_t) * (size_t)tn);
  orc_update_masks(mask, h, w, tw, tn, ufree, ufin);
  int nfree = nsub - 1 > 0 ? nsub - 1 : 0;
  for (int f = 0; f < 3; ++f) {
    float *L = fld + (size_t)f * H * W;
    const float k = kk[f];
    memset(X, 0, sizeof(float) * tn);
    for (int i = 0; i < nrow; ++i)
      for (int j = 0; j < ncol; ++j)
        ORC_TILE(X, i, j) =
            mask[i * ncol + j] ? p->external_levels[f] : L[(r0 - 1 + i) * W + (c0 - 1 + j)];
    for (int s = 0; s <= nfree; ++s) {
      const int32_t *U = (s == nfree) ? ufin : ufree;
      for (int i = 0; i < nrow; ++i) {
        const float *restrict xu = &ORC_TILE(X, i - 1, 0), *restrict x = &ORC_TILE(X, i, 0);
        const float *restrict xd = &ORC_TILE(X, i + 1, 0);
        float *restrict dd = &ORC_TILE(D, i, 0);
        for (int j = 0; j < ncp; ++j) {
          float res = xu[j] + x[j - 1] + xd[j] + x[j + 1];
          res += (xu[j - 1] + xu[j + 1] + xd[j - 1] + xd[j + 1]) * S2;
          res -= x[j] * F;
          res *= k;
          dd[j] = res;
        }
      }
      for (int i = 0; i < nrow; ++i) {
        float *restrict x = &ORC_TILE(X, i, 0);
        const float *restrict dd = &ORC_TILE(D, i, 0);
        const int32_t *restrict u = &ORC_TILE(U, i, 0);
        for (int j = 0; j < ncp; ++j) x[j] = orc_sel(u[j], x[j] + dd[j], x[j]);
      }
    }
    for (int i = 1; i <= h; ++i)
      for (int j = 1; j <= w; ++j) L[(r0 - 1 + i) * W + (c0 - 1 + j)] = ORC_TILE(X, i, j);
  }
  free(X); free(D); free(ufree); free(ufin);
}

void orc_diffuse_f64(double *fld, int H, int W, const int32_t roi[5], const uint8_t *mask,
                     const orc_params *p) {
  int r0 = roi[0], c0 = roi[1], h = roi[2], w = roi[3];
  if (h == 0 || w == 0) return;
  float kk[3], a[3], b[3], d[3];
  int nsub;
  orc_diffusion_coeffs(p, kk, a, b, d, &nsub);
  const double S2 = (double)(float)0.70710678118654752440;
  const double F = (double)(float)(4. + (double)(float)(2 * 1.41421356237309504880));
  int nrow = h + 2, ncol = w + 2, tw = ncol + 2, tn = (nrow + 2) * tw;
  double *X = (double *)calloc((size_t)tn, sizeof(double));
  double *D = (double *)calloc((size_t)tn, sizeof(double));
  int nfree = nsub - 1 > 0 ? nsub - 1 : 0;
  for (int f = 0; f < 3; ++f) {
    double *L = fld + (size_t)f * H * W;
    memset(X, 0, sizeof(double) * tn);
    for (int i = 0; i < nrow; ++i)
      for (int j = 0; j < ncol; ++j)
        ORC_TILE(X, i, j) = mask[i * ncol + j] ? (double)p->external_levels[f]
                                               : L[(r0 - 1 + i) * W + (c0 - 1 + j)];
    for (int s = 0; s <= nfree; ++s) {
      int final = (s == nfree);
      for (int i = 0; i < nrow; ++i)
        for (int j = 0; j < ncol; ++j) {
          int upd = final ? (i >= 1 && i <= h && j >= 1 && j <= w) : !mask[i * ncol + j];
          if (!upd) continue;
          double res = ORC_TILE(X, i - 1, j) + ORC_TILE(X, i, j - 1) + ORC_TILE(X, i + 1, j) +
                       ORC_TILE(X, i, j + 1);
          res += (ORC_TILE(X, i - 1, j - 1) + ORC_TILE(X, i - 1, j + 1) +
                  ORC_TILE(X, i + 1, j - 1) + ORC_TILE(X, i + 1, j + 1)) * S2;
          res -= ORC_TILE(X, i, j) * F;
          res *= (double)kk[f];
          ORC_TILE(D, i, j) = res;
        }
      for (int i = 0; i < nrow; ++i)
        for (int j = 0; j < ncol; ++j) {
          int upd = final ? (i >= 1 && i <= h && j >= 1 && j <= w) : !mask[i * ncol + j];
          if (upd) ORC_TILE(X, i, j) += ORC_TILE(D, i, j);
        }
    }
    for (int i = 1; i <= h; ++i)
      for (int j = 1; j <= w; ++j) L[(r0 - 1 + i) * W + (c0 - 1 + j)] = ORC_TILE(X, i, j);
  }
  free(X); free(D);
}
#undef ORC_TILE

/* ======================================================================== */
/* batched simulator                                                         */
/* ======================================================================== */
#ifdef ORC_REF_CELL
/* provided by oracle/ref_shim.cc: the reference's own functions */
void *orc_ref_rng_create(uint32_t seed);
void orc_ref_rng_destroy(void *rng);
int orc_ref_site_step(orc_site *s, const orc_params *p, uint32_t vac, float dose, void *rng);
void orc_ref_choose_neighbour(int r, int c, void *rng, int *rr, int *cc);
void orc_ref_divide_cell(orc_site *parent, orc_site *child, const orc_params *p, void *rng);
#endif

typedef struct {
  float *fld;  /* 3 * H * W */
  uint8_t *st;
  orc_cell *cell;
  uint16_t *list;
  uint32_t n;
  uint8_t *occ;
  int32_t roi[5];
  uint8_t *mask;
  float *prot;
  uint32_t bins, res, length, sim_index, epoch, step, horizon;
  orc_instr instr;
  unsigned long long hist[600];
  unsigned long long diffused;
  uint8_t *vac;
  int32_t *cand;
  uint8_t *seen;
  void *rng;
} orc_sim;

struct orc_batch {
  orc_params p;
  int H, W, n;
  uint32_t lcap;
  uint64_t seed;
  orc_sim *s;
  int next;
  pthread_mutex_t mu;
  uint32_t nsteps;
};

orc_batch *orc_batch_create(const orc_params *p, int n_sims, uint64_t seed) {
  orc_batch *b = (orc_batch *)calloc(1, sizeof(orc_batch));
  b->p = *p;
  b->H = p->lattice_height + 2;
  b->W = p->lattice_width + 2;
  b->n = n_sims;
  b->seed = seed;
  b->lcap = (uint32_t)(p->lattice_height * p->lattice_width) + 256u;
  b->s = (orc_sim *)calloc((size_t)n_sims, sizeof(orc_sim));
  size_t hw = (size_t)b->H * b->W;
  for (int i = 0; i < n_sims; ++i) {
    orc_sim *S = &b->s[i];
    S->fld = (float *)calloc(3 * hw, sizeof(float));
    S->st = (uint8_t *)calloc(hw, 1);
    S->cell = (orc_cell *)calloc(hw, sizeof(orc_cell));
    S->list = (uint16_t *)calloc(b->lcap, sizeof(uint16_t));
    S->occ = (uint8_t *)calloc(hw, 1);
    S->mask = (uint8_t *)calloc(hw, 1);
    S->vac = (uint8_t *)calloc(b->lcap, 1);
    S->cand = (int32_t *)calloc(b->lcap, sizeof(int32_t));
    S->seen = (uint8_t *)calloc(hw, 1);
  }
  pthread_mutex_init(&b->mu, NULL);
  return b;
}

void orc_batch_destroy(orc_batch *b) {
  if (!b) return;
  for (int i = 0; i < b->n; ++i) {
    orc_sim *S = &b->s[i];
    free(S->fld); free(S->st); free(S->cell); free(S->list); free(S->occ); free(S->mask);
    free(S->vac); free(S->cand); free(S->seen); free(S->prot);
#ifdef ORC_REF_CELL
    if (S->rng) orc_ref_rng_destroy(S->rng);
#endif
  }
  free(b->s);
  pthread_mutex_destroy(&b->mu);
  free(b);
}

int orc_batch_set(orc_batch *b, int i, const orc_site *sites, const float *protocol,
                  uint32_t bins, uint32_t resolution, uint32_t length, uint32_t sim_index,
                  uint32_t epoch, uint32_t step0, uint32_t horizon) {
  if (i < 0 || i >= b->n || resolution == 0) return -1;
  orc_sim *S = &b->s[i];
  size_t hw = (size_t)b->H * b->W;
  for (size_t k = 0; k < hw; ++k) {
    S->fld[k] = sites[k].cho;
    S->fld[hw + k] = sites[k].ox;
    S->fld[2 * hw + k] = sites[k].gi;
    S->st[k] = sites[k].state;
    orc_site_to_cell(&sites[k], &S->cell[k]);
  }
  free(S->prot);
  S->prot = (float *)calloc(bins ? bins : 1, sizeof(float));
  if (bins) memcpy(S->prot, protocol, bins * sizeof(float));
  S->bins = bins;
  S->res = resolution;
  S->length = length;
  S->sim_index = sim_index;
  S->epoch = epoch;
  S->step = step0;
  S->horizon = horizon;
  S->n = 0;
  memset(S->occ, 0, hw);
  memset(S->roi, 0, sizeof(S->roi));
  memset(&S->instr, 0, sizeof(S->instr));
  memset(S->hist, 0, sizeof(S->hist));
  S->diffused = 0;
#ifdef ORC_REF_CELL
  if (S->rng) orc_ref_rng_destroy(S->rng);
  S->rng = orc_ref_rng_create((uint32_t)(b->seed * 1000003ull + sim_index));
#endif
  return 0;
}

static inline float orc_dose(const orc_sim *S, uint32_t t) {
  /* protocol.h:9-14 */
  if (t < S->length && t % S->res == 0) {
    uint32_t bin = t / S->res;
    return bin < S->bins ? S->prot[bin] : 0.f;
  }
  return 0.f;
}

static inline int orc_hist_bin(float v) {
  int bi = (int)(v / 0.1f);
  if (bi < 0) bi = 0;
  if (bi >= 300) bi = 299;
  return bi;
}

#ifndef ORC_REF_CELL
/* Site::step on the batch's own storage with Philox draws keyed by
 * (step, sim, site, occurrence). */
static int orc_step_site(const orc_batch *b, orc_sim *S, int s, uint32_t vac, float dose,
                         uint32_t t, uint32_t occ) {
  const orc_params *p = &b->p;
  size_t hw = (size_t)b->H * b->W;
  orc_cell *c = &S->cell[s];
  float lv[3] = {S->fld[s], S->fld[hw + s], S->fld[2 * hw + s]};
  if (!orc_update_state(c, lv, p, vac)) {
    S->st[s] = ORC_VACANT;
    return 0;
  }
  if (dose > 0) {
    orc_irradiate(c, dose, p);
    S->instr.irradiation_events++;
  }
  orc_metabolise(c, lv, p);
  S->fld[s] = lv[0];
  S->fld[hw + s] = lv[1];
  S->fld[2 * hw + s] = lv[2];
  int cc = orc_progress_clock(c, p->time_step);
  if (orc_repair_pre(c, p, cc)) {
    float dp = orc_death_prob(c, p);
    S->instr.repair_decisions++;
    S->instr.sum_death_prob += (double)dp;
    S->hist[orc_hist_bin(c->irr)]++;
    S->hist[300 + orc_hist_bin(c->tir)]++;
    float u = orc_uniform(b->seed, t, S->sim_index, (uint32_t)s, occ, 1, S->epoch);
    if (!orc_repair_post(c, dp, u)) {
      S->instr.repair_kills++;
      S->st[s] = ORC_VACANT;
      return 0;
    }
  }
  return c->phase == 4;
}
#endif

static void orc_step(const orc_batch *b, orc_sim *S) {
  const int H = b->H, W = b->W;
  const uint32_t t = S->step;
  size_t hw = (size_t)H * W;
  if (t % 128 == 0) {
    S->n = orc_rebuild_list(S->st, H, W, S->list);
    memset(S->occ, 0, hw);
    for (uint32_t e = 0; e < S->n; ++e) S->occ[S->list[e]]++;
  }
  if (t % 32 == 0) orc_find_roi(S->st, H, W, S->roi, S->mask);
  if (S->roi[2] > 0 && S->roi[3] > 0) {
#ifdef ORC_REF_CELL
    orc_diffuse_ref_f32(S->fld, H, W, S->roi, S->mask, &b->p);
#else
    orc_diffuse_f32(S->fld, H, W, S->roi, S->mask, &b->p);
#endif
    /* count of free-site substeps (23 substeps x free sites + final ROI pass) */
    int nrow = S->roi[2] + 2, ncol = S->roi[3] + 2;
    unsigned long long nf = 0;
    for (int q = 0; q < nrow * ncol; ++q) nf += !S->mask[q];
    float kk[3], a[3], bb[3], d[3];
    int nsub;
    orc_diffusion_coeffs(&b->p, kk, a, bb, d, &nsub);
    int nfree = nsub - 1 > 0 ? nsub - 1 : 0;
    S->diffused += nf * (unsigned long long)nfree + (unsigned long long)S->roi[2] * S->roi[3];
  }
  /* cell kernel, simulation.cu:66-110 */
  float dose = orc_dose(S, t);
  for (uint32_t e = 0; e < S->n; ++e) {
    int s = S->list[e];
    const uint8_t *q = S->st;
    S->vac[e] = (uint8_t)((q[s - W - 1] == ORC_VACANT) + (q[s - W + 1] == ORC_VACANT) +
                          (q[s + W - 1] == ORC_VACANT) + (q[s + W + 1] == ORC_VACANT) +
                          (q[s - 1] == ORC_VACANT) + (q[s + 1] == ORC_VACANT) +
                          (q[s - W] == ORC_VACANT) + (q[s + W] == ORC_VACANT));
  }
  for (uint32_t e = 0; e < S->n; ++e) {
    int s = S->list[e];
    uint32_t occ = S->seen[s]++;
    S->cand[e] = -1;
    if (S->st[s] != ORC_OCCUPIED) continue;
#ifdef ORC_REF_CELL
    orc_site site;
    {
      site.cho = S->fld[s]; site.ox = S->fld[hw + s]; site.gi = S->fld[2 * hw + s];
      orc_cell_to_site(&S->cell[s], &site);
      site.state = S->st[s];
    }
    int ready = orc_ref_site_step(&site, &b->p, S->vac[e], dose, S->rng);
    S->fld[s] = site.cho; S->fld[hw + s] = site.ox; S->fld[2 * hw + s] = site.gi;
    orc_site_to_cell(&site, &S->cell[s]);
    S->st[s] = site.state;
    if (ready) {
      int rr, cc;
      orc_ref_choose_neighbour(s / W, s % W, S->rng, &rr, &cc);
      S->cand[e] = rr * W + cc;
    }
    (void)occ;
#else
    if (orc_step_site(b, S, s, S->vac[e], dose, t, occ)) {
      int rr, cc;
      float u = orc_uniform(b->seed, t, S->sim_index, (uint32_t)s, occ, 0, S->epoch);
      orc_choose_neighbour(s / W, s % W, u, &rr, &cc);
      S->cand[e] = rr * W + cc;
    }
#endif
  }
  for (uint32_t e = 0; e < S->n; ++e) S->seen[S->list[e]] = 0;
  int winner = -1;
  for (uint32_t e = 0; e < S->n; ++e)
    if (S->cand[e] >= 0 && S->st[S->cand[e]] == ORC_VACANT) {
      winner = (int)e;
      break;
    }
  if (winner >= 0) {
    int parent = S->list[winner], child = S->cand[winner];
    S->st[child] = ORC_OCCUPIED;
#ifdef ORC_REF_CELL
    orc_site ps, cs;
    orc_cell_to_site(&S->cell[parent], &ps);
    orc_ref_divide_cell(&ps, &cs, &b->p, S->rng);
    orc_site_to_cell(&ps, &S->cell[parent]);
    orc_site_to_cell(&cs, &S->cell[child]);
#else
    float z[5];
    orc_division_normals(b->seed, t, S->sim_index, S->epoch, z);
    orc_divide_cell(&S->cell[parent], &S->cell[child], z, &b->p);
#endif
    if (S->n < b->lcap) S->list[S->n++] = (uint16_t)child;
    S->occ[child]++;
    S->instr.divisions++;
  }
  S->step = t + 1;
}

static void *orc_worker(void *arg) {
  orc_batch *b = (orc_batch *)arg;
  for (;;) {
    pthread_mutex_lock(&b->mu);
    int i = b->next++;
    pthread_mutex_unlock(&b->mu);
    if (i >= b->n) break;
    orc_sim *S = &b->s[i];
    for (uint32_t k = 0; k < b->nsteps && S->step < S->horizon; ++k) orc_step(b, S);
  }
  return NULL;
}

void orc_batch_run(orc_batch *b, uint32_t nsteps, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > b->n) nthreads = b->n > 0 ? b->n : 1;
  b->next = 0;
  b->nsteps = nsteps;
  if (nthreads == 1) {
    orc_worker(b);
    return;
  }
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  for (int k = 0; k < nthreads; ++k) pthread_create(&th[k], NULL, orc_worker, b);
  for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
  free(th);
}

void orc_batch_get(const orc_batch *b, int i, orc_site *out) {
  const orc_sim *S = &b->s[i];
  size_t hw = (size_t)b->H * b->W;
  for (size_t k = 0; k < hw; ++k) {
    memset(&out[k], 0, sizeof(orc_site));
    out[k].cho = S->fld[k];
    out[k].ox = S->fld[hw + k];
    out[k].gi = S->fld[2 * hw + k];
    orc_cell_to_site(&S->cell[k], &out[k]);
    out[k].state = S->st[k];
  }
}

void orc_batch_counts(const orc_batch *b, uint32_t *out) {
  size_t hw = (size_t)b->H * b->W;
  for (int i = 0; i < b->n; ++i) {
    uint32_t c = 0;
    for (size_t k = 0; k < hw; ++k) c += b->s[i].st[k] == ORC_OCCUPIED;
    out[i] = c;
  }
}

void orc_batch_list(const orc_batch *b, int i, uint16_t *list, uint32_t *n) {
  *n = b->s[i].n;
  memcpy(list, b->s[i].list, b->s[i].n * sizeof(uint16_t));
}

void orc_batch_roi(const orc_batch *b, int i, int32_t out[5]) {
  memcpy(out, b->s[i].roi, sizeof(int32_t) * 5);
}

void orc_batch_instr(const orc_batch *b, orc_instr *out, unsigned long long *hist) {
  memset(out, 0, sizeof(*out));
  if (hist) memset(hist, 0, 600 * sizeof(unsigned long long));
  for (int i = 0; i < b->n; ++i) {
    const orc_sim *S = &b->s[i];
    out->repair_decisions += S->instr.repair_decisions;
    out->repair_kills += S->instr.repair_kills;
    out->irradiation_events += S->instr.irradiation_events;
    out->divisions += S->instr.divisions;
    out->sum_death_prob += S->instr.sum_death_prob;
    if (hist)
      for (int k = 0; k < 600; ++k) hist[k] += S->hist[k];
  }
}

unsigned long long orc_batch_diffused(const orc_batch *b) {
  unsigned long long t = 0;
  for (int i = 0; i < b->n; ++i) t += b->s[i].diffused;
  return t;
}
