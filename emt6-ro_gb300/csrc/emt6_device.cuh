// emt6_device.cuh -- device-side model of the EMT6-Ro simulation step.
//
// Compiled with --fmad=false: every float/double expression is evaluated as
// written, fused multiply-adds appear only where fmaf/fma is called.  This is
// what makes the library reproduce, bit for bit, a CPU evaluation of the same
// expressions (the parity tests' oracle is compiled with -ffp-contract=off).
//
// Model semantics follow the reference (paths relative to banasraf/EMT6-Ro):
//   Cell::updateState / tryProliferating / tryQuiescence  src/emt6ro/cell/cell.cu:33-82
//   Cell::irradiate / calcDelayTime                        cell.cu:84-100
//   Cell::metabolise / progressClock                       cell.cu:16-32
//   Cell::tryRepair                                        src/emt6ro/cell/cell.h:102-136
//   chooseNeighbour / divideCell / createCell              src/emt6ro/simulation/cell-division.h
//   Protocol::getDose                                      src/emt6ro/common/protocol.h:9-14
#pragma once
#include <cstdint>

namespace emt6 {

constexpr unsigned kFull = 0xffffffffu;

constexpr uint8_t kVacant = 0, kOccupied = 1, kMocked = 2;
// st byte: bits 0-1 site state, bit 2 listed at the last rebuild, bit 3 listed
// more than once, bit 4 appended since the last rebuild
constexpr uint8_t kStMask = 3, kStRebuilt = 4, kStMulti = 8, kStTail = 16;

// Model constants, precomputed on the host exactly as the reference's
// expressions evaluate them (see emt6_host.cpp: make_kparams).
struct KParams {
  int H, W, HW, lcap;
  float dt_h;   // time_step / 3600.f          (cell.cu:25, :73; cell.h:106)
  float dt2_h;  // 2 * time_step / 3600.f      (cell.cu:68)
  float met[4][3];
  float ext[3];
  float death_gi, quiescence_gi;
  float ct_mean[5], ct_sd[5];
  float dl_c, dl_e, sv_c, sv_e, rht;
  float da[3], db[3], dd[3];  // diffusion: x' = da*x + db*orth + dd*diag
  int nfree;                  // substeps over free sites before the final ROI pass
  uint32_t seed_lo, seed_hi;
  uint32_t res, length, bins;
  uint32_t sim_base;  // added to the simulation index of every random key
  // tile shapes the step kernels may use (kLayout*); results do not depend on it
  uint32_t layouts;
};

// kLayoutBands: eight-lane bands for narrow regions up to 23 columns;
// kLayoutWideBands: three-column half-warp bands for 41-48-row wide regions;
// kLayoutRing: the ring mapping of 35 x 35 regions on the narrow kernel
constexpr uint32_t kLayoutBands = 1u, kLayoutWideBands = 2u, kLayoutRing = 4u,
                   kLayoutAll = 7u;

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11), counter = (step, sim, site|occ<<16|
// purpose<<24, epoch), key = seed.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ uint4 draw(const KParams &p, uint32_t step, uint32_t sim,
                                      uint32_t site, uint32_t occ, uint32_t purpose,
                                      uint32_t epoch) {
  return philox4x32_10(
      make_uint4(step, sim + p.sim_base, (site & 0xFFFFu) | ((occ & 0xFFu) << 16) | (purpose << 24),
                 epoch),
      p.seed_lo, p.seed_hi);
}

// uniform in (0, 1], the range of curand_uniform (random-engine.cu:33-35)
__device__ __forceinline__ float u01(uint32_t x) {
  return __uint2float_rn((x >> 8) + 1u) * 0x1p-24f;
}

// ---------------------------------------------------------------------------
// Double-precision exp / log / sincos(2*pi*u) from IEEE basic operations and
// fma only (Cody-Waite reduction + Taylor / atanh series), so results are the
// same bits on any IEEE machine.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double exp_core(double x) {
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
  return q * __longlong_as_double(((long long)k + 1023) << 52);
}

__device__ __forceinline__ float dexpf(float x) { return (float)exp_core((double)x); }

__device__ __forceinline__ double log_core(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  double m = __longlong_as_double((long long)((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull));
  if (m > 0x1.6a09e667f3bcdp+0) {
    m *= 0.5;
    e += 1;
  }
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

__device__ __forceinline__ void sincos2pi(double u, double *s_out, double *c_out) {
  double q = floor(u * 4.0);
  double t = u - q * 0.25;
  if (t > 0.125) {
    t -= 0.25;
    q += 1.0;
  }
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
  switch (((int)q) & 3) {
    case 0: *s_out = sn; *c_out = cs; break;
    case 1: *s_out = cs; *c_out = -sn; break;
    case 2: *s_out = -sn; *c_out = -cs; break;
    default: *s_out = -cs; *c_out = sn; break;
  }
}

// Box-Muller pair: u1 in (0,1] from a, u2 in [0,1) from b
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float *z0, float *z1) {
  float u1 = u01(a);
  float u2 = __uint2float_rn(b >> 8) * 0x1p-24f;
  double r = sqrt(-2.0 * log_core((double)u1));
  double s, c;
  sincos2pi((double)u2, &s, &c);
  *z0 = (float)(r * c);
  *z1 = (float)(r * s);
}

// ---------------------------------------------------------------------------
// Cell model.  Registers hold one cell: A = (prolif, tir, irr, delay),
// B = (t_g1, t_s, t_g2, t_m), C = (t_d, mode | phase << 8, -, -).
// ---------------------------------------------------------------------------
struct DCell {
  float prolif, tir, irr, delay;
  float t0, t1, t2, t3, t4;
  uint32_t mode, phase;
};

__device__ __forceinline__ DCell load_cell(const float4 *c) {
  float4 A = c[0], B = c[1], C = c[2];
  DCell d;
  d.prolif = A.x; d.tir = A.y; d.irr = A.z; d.delay = A.w;
  d.t0 = B.x; d.t1 = B.y; d.t2 = B.z; d.t3 = B.w; d.t4 = C.x;
  uint32_t mp = __float_as_uint(C.y);
  d.mode = mp & 0xffu;
  d.phase = (mp >> 8) & 0xffu;
  return d;
}

__device__ __forceinline__ void store_cell(float4 *c, const DCell &d) {
  c[0] = make_float4(d.prolif, d.tir, d.irr, d.delay);
  c[1] = make_float4(d.t0, d.t1, d.t2, d.t3);
  c[2] = make_float4(d.t4, __uint_as_float(d.mode | (d.phase << 8)), 0.f, 0.f);
}

// cell.cu:72-82 (+ :33-70)
__device__ __forceinline__ bool update_state(DCell &c, float l0, float l1, float l2,
                                             const KParams &p, uint32_t vac) {
  if (c.prolif >= c.t4 - p.dt_h) return false;
  bool g1s = c.prolif > (c.t0 - p.dt2_h) && c.phase == 0 && vac <= 1;
  if (!g1s) {
    if (l0 >= p.met[0][0] && l1 >= p.met[0][1] && l2 < p.quiescence_gi) {
      c.mode = 0;
      return true;
    } else if (l0 >= p.met[1][0] && l1 >= p.met[1][1] && l2 < p.quiescence_gi) {
      c.mode = 1;
      return true;
    }
  }
  if (c.phase != 0 && c.phase != 2) return false;
  if (l0 >= p.met[2][0] && l1 >= p.met[2][1] && l2 < p.death_gi) {
    c.mode = 2;
    return true;
  } else if (l0 >= p.met[3][0] && l1 >= p.met[3][1] && l2 < p.death_gi) {
    c.mode = 3;
    return true;
  }
  return false;
}

// cell.cu:84-91, :93-100
__device__ __forceinline__ void irradiate(DCell &c, float dose, const KParams &p) {
  c.irr = c.irr / (1 + c.tir / p.rht) + dose;
  c.tir = 0;
  c.delay = p.dl_c * dexpf(p.dl_e * c.irr);
}

// cell.cu:21-32
__device__ __forceinline__ bool progress_clock(DCell &c, const KParams &p) {
  if ((c.mode == 0 || c.mode == 1) && c.tir == 0) {
    c.prolif += p.dt_h;
    uint32_t cur = c.phase;
    float tc = cur == 0 ? c.t0 : cur == 1 ? c.t1 : cur == 2 ? c.t2 : cur == 3 ? c.t3 : c.t4;
    c.phase = cur + (c.prolif > tc ? 1u : 0u);
    return c.phase != cur && c.phase != 4;
  }
  return false;
}

// cell.h:104-107: advance the repair clock; true if the survival decision fires
__device__ __forceinline__ bool repair_pre(DCell &c, const KParams &p, bool cycle_changed) {
  if (c.tir > 0 || (c.irr > 0 && cycle_changed)) {
    c.tir += p.dt_h;
    if (c.tir >= c.delay) return true;
  }
  return false;
}

__device__ __forceinline__ float death_prob(const DCell &c, const KParams &p) {
  return 1 - p.sv_c * dexpf(p.sv_e * c.irr);  // cell.h:108-110
}

// cell-division.h:32-54
__device__ __forceinline__ int choose_neighbour(int s, int W, float u) {
  const float diag_prob = 4.f;
  const float ortho_prob = (float)(4. * 1.41421356237309504880);
  float score = u * (diag_prob + ortho_prob);
  int r = s / W, c = s - (s / W) * W;
  if (score < diag_prob) {
    uint32_t num = (uint8_t)score;
    int vert = (int)(num & 1u) * 2 - 1;
    int hor = (int)((num & 2u) >> 1u) * 2 - 1;
    return (r + vert) * W + (c + hor);
  }
  uint32_t num = (uint8_t)((double)(score - diag_prob) / 1.41421356237309504880);
  int which = num & 1u;
  int diff = (int)((num & 2u) >> 1u) * 2 - 1;
  return which ? (r + diff) * W + c : r * W + (c + diff);
}

// createCell/divideCell, cell-division.h:10-30: child from five standard normals
__device__ __forceinline__ DCell make_child(const DCell &parent, const float z[5],
                                            const KParams &p) {
  DCell ch;
  ch.prolif = 0.f;
  ch.tir = 0.f;
  ch.t0 = p.ct_sd[0] * z[0] + p.ct_mean[0];
  ch.t1 = ch.t0 + (p.ct_sd[1] * z[1] + p.ct_mean[1]);
  ch.t2 = ch.t1 + (p.ct_sd[2] * z[2] + p.ct_mean[2]);
  ch.t3 = ch.t2 + (p.ct_sd[3] * z[3] + p.ct_mean[3]);
  ch.t4 = ch.t3 + (p.ct_sd[4] * z[4] + p.ct_mean[4]);
  ch.irr = parent.irr;
  ch.delay = parent.irr > 0 ? p.dl_c * dexpf(p.dl_e * ch.irr) : 0.f;
  ch.mode = 0;
  ch.phase = 0;
  return ch;
}

}  // namespace emt6
