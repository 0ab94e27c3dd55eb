// emt6_kernels.cu -- sm_103a kernels of the EMT6-Ro batched simulation step.
//
// One CTA owns one simulation for a whole launch of N steps: the three
// substrate fields (3 x 53 x 53 FP32), the site-state bytes and the occupied
// list live in shared memory for the launch; per-site cell records (48 B)
// stay in global memory, where the few hundred live cells of each resident
// simulation stay L2-resident.  Two kernels: run_kernel<false> (192 threads,
// 4 CTAs/SM) for regions up to 32 x 32 (33 x 33 with a fixed ring), and
// run_kernel<true> (384 threads, 2 CTAs/SM) for wider regions.  Per step
// (reference cadence, src/emt6ro/simulation/simulation.cu:153-166):
//   t % 128 == 0  rebuild the occupied list        (simulation.cu:41-64)
//   t % 32  == 0  ROI + circular fixed-value mask   (diffusion.cu:65-100)
//   diffusion: 23 substeps over free sites + 1 over the ROI (diffusion.cu:135-191).
//     Each field is held in registers, two columns per lane: in the narrow
//     kernel by a pair of warps whose half-warps hold four bands of rows
//     (diffuse_half), or, for regions up to 24 columns, whose eight-lane
//     groups hold eight bands of two or three columns per lane
//     (diffuse_band), in the wide kernel by four warps of one band each
//     (diffuse_part) or, for 41-48 rows, half-warp bands of three columns
//     per lane (diffuse_wband).  Horizontal neighbours come from warp shuffles,
//     vertical ones from the same thread's registers; bands swap one
//     boundary row per substep (a shuffle across half-warps, shared memory
//     between warps under 64- or 128-thread named barriers).
//   cell update: 8-neighbour vacancy snapshot, Site::step per list entry,
//     at most one division per simulation (simulation.cu:66-110).
// Randomness is Philox keyed by (step, simulation, site, occurrence), so the
// results do not depend on the launch shape, nor on the order in which CTAs
// take simulations: before every chunk of steps three small kernels sort the
// simulations by their region, largest first, so that the CTAs resident on
// an SM run the same tile code (launch_order).
#include <cuda_runtime.h>

#include <cstdint>

#include "emt6_device.cuh"
#include "emt6_kernels.h"

namespace emt6 {

__device__ unsigned long long g_instr_counts[4];  // decisions, kills, irradiations, divisions
__device__ double g_instr_sum_death_prob;
__device__ unsigned long long g_instr_hist[600];  // irradiation bins, then time-in-repair

struct Misc {
  int roi[5];  // r0, c0, h, w, dist
  uint32_t n, n0;
  int has_multi;
  int winner, target;
  int red[12][4];
  unsigned int ins[4];
  double ins_dp;
  unsigned long long diffused;
  unsigned long long nfs;  // free sites of the current mask
  int narrow_ok, roff, coff;  // region fits the narrow kernel; row/column offset
  int ring;  // 35 x 35 region with every free site in rows and columns 1..32
  int wblk;  // 49 x 49 region with every free site in rows and columns 1..46
};

__host__ __device__ inline uint32_t align_up(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }

struct SmemLayout {
  uint32_t fld, st, list, aux, colmask, xch, misc, total;
};

__host__ __device__ inline SmemLayout smem_layout(int HW, int lcap, int np) {
  SmemLayout L;
  uint32_t o = 0;
  // fld and st regions match the global per-simulation strides (3*HW padded
  // to 32 floats, HW padded to 128 bytes) so whole-stride copies stay inside
  L.fld = o; o += align_up(3u * (uint32_t)HW, 32) * 4u;
  L.st = o; o += align_up((uint32_t)HW, 128);
  L.list = o; o += align_up((uint32_t)lcap * 2u, 16);
  L.aux = o; o += align_up((uint32_t)lcap, 16);
  L.colmask = o; o += 64 * 8;
  // boundary-row exchange: per field, 2 parities x NP parts x (1 side when
  // NP == 2, else 2) x 32 lanes of float4
  L.xch = o; o += 3u * 2u * (uint32_t)np * (np == 2 ? 1u : 2u) * 32u * 16u;
  L.misc = o; o += align_up(sizeof(Misc), 16);
  L.total = o;
  return L;
}

size_t run_kernel_smem(int HW, int lcap, bool wide) {
  return smem_layout(HW, lcap, wide ? 4 : 2).total;
}

// ---------------------------------------------------------------------------
// x where bit i of u is clear, nv where it is set: the fixed-site select of
// the diffusion tiles.  Written as a bitwise blend with a mask made by
// shifting bit i into the sign and back, so it issues a shift pair and one
// three-input logic op instead of a bit test, a predicate and a select: the
// ALU pipe (the busiest of the step kernels) carries less, and the result is
// the same bits.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float sel_bit(uint32_t u, int i, float nv, float x) {
  const uint32_t m = (uint32_t)((int32_t)(u << (31 - i)) >> 31);
  return __uint_as_float((__float_as_uint(nv) & m) | (__float_as_uint(x) & ~m));
}

// ---------------------------------------------------------------------------
// block reductions
// ---------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ void block_minmax4(int v[4], Misc *m) {
  // v = (min r, min c, max r, max c)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    v[0] = min(v[0], __shfl_xor_sync(kFull, v[0], o));
    v[1] = min(v[1], __shfl_xor_sync(kFull, v[1], o));
    v[2] = max(v[2], __shfl_xor_sync(kFull, v[2], o));
    v[3] = max(v[3], __shfl_xor_sync(kFull, v[3], o));
  }
  if (lane == 0)
    for (int k = 0; k < 4; ++k) m->red[wid][k] = v[k];
  __syncthreads();
  v[0] = m->red[0][0]; v[1] = m->red[0][1]; v[2] = m->red[0][2]; v[3] = m->red[0][3];
  for (int w = 1; w < NT / 32; ++w) {
    v[0] = min(v[0], m->red[w][0]);
    v[1] = min(v[1], m->red[w][1]);
    v[2] = max(v[2], m->red[w][2]);
    v[3] = max(v[3], m->red[w][3]);
  }
  __syncthreads();
}

template <int NT>
__device__ __forceinline__ int block_max(int v, Misc *m) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
  if (lane == 0) m->red[wid][0] = v;
  __syncthreads();
  v = m->red[0][0];
  for (int w = 1; w < NT / 32; ++w) v = max(v, m->red[w][0]);
  __syncthreads();
  return v;
}

template <int NT>
__device__ __forceinline__ int block_min(int v, Misc *m) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(kFull, v, o));
  if (lane == 0) m->red[wid][0] = v;
  __syncthreads();
  v = m->red[0][0];
  for (int w = 1; w < NT / 32; ++w) v = min(v, m->red[w][0]);
  __syncthreads();
  return v;
}

// ---------------------------------------------------------------------------
// occupied list (simulation.cu:41-64): 32 column stripes, stripe k = columns
// k, k+32, ... < W-1 over rows 0..H-2, stripes concatenated in order.
// Called by all threads; warp 0 builds.
// ---------------------------------------------------------------------------
template <int NT>
__device__ void rebuild_list(uint8_t *st, uint16_t *list, Misc *m, int H, int W, int HW) {
  for (int q = threadIdx.x; q < HW; q += NT) st[q] &= kStMask;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int k = threadIdx.x;
    uint32_t cnt = 0;
    for (int r = 0; r < H - 1; ++r)
      for (int c = k; c < W - 1; c += 32) cnt += (st[r * W + c] & kStMask) == kOccupied;
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, incl, o);
      if (k >= o) incl += y;
    }
    uint32_t off = incl - cnt;
    for (int r = 0; r < H - 1; ++r)
      for (int c = k; c < W - 1; c += 32) {
        int q = r * W + c;
        if ((st[q] & kStMask) == kOccupied) {
          list[off++] = (uint16_t)q;
          st[q] |= kStRebuilt;
        }
      }
    if (k == 31) {
      m->n = incl;
      m->n0 = incl;
      m->has_multi = 0;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// ROI + mask (diffusion.cu:16-100).  colmask[j] bit i = site (i, j) of the
// (h+2) x (w+2) region is free (not held at the external level).
// ---------------------------------------------------------------------------
template <int NT>
__device__ void compute_roi(const uint8_t *st, uint64_t *colmask, Misc *m, int H, int W, int HW) {
  int v[4] = {H, W, 0, 0};
  for (int q = threadIdx.x; q < HW; q += NT)
    if ((st[q] & kStMask) == kOccupied) {
      int r = q / W, c = q - (q / W) * W;
      v[0] = min(v[0], r); v[1] = min(v[1], c);
      v[2] = max(v[2], r); v[3] = max(v[3], c);
    }
  block_minmax4<NT>(v, m);
  if (v[2] == 0 && v[3] == 0) {
    if (threadIdx.x == 0) m->roi[0] = m->roi[1] = m->roi[2] = m->roi[3] = m->roi[4] = 0;
    if (threadIdx.x < 64) colmask[threadIdx.x] = 0;
    __syncthreads();
    return;
  }
  const int midr = v[0] + (v[2] - v[0] + 1) / 2;
  const int midc = v[1] + (v[3] - v[1] + 1) / 2;
  int dist = 0;
  for (int q = threadIdx.x; q < HW; q += NT)
    if ((st[q] & kStMask) == kOccupied) {
      int r = q / W, c = q - (q / W) * W;
      float d2 = (float)((midr - r) * (midr - r) + (midc - c) * (midc - c));
      dist = max(dist, (int)ceilf(sqrtf(d2)));
    }
  dist = block_max<NT>(dist, m);
  const int sub_r = (midr <= dist) ? 1 : midr - dist;
  const int sub_c = (midc <= dist) ? 1 : midc - dist;
  const int sub_w = (midc + dist >= W - 1) ? W - 1 - sub_c : midc + dist - sub_c + 1;
  const int sub_h = (midr + dist >= H - 1) ? H - 1 - sub_r : midr + dist - sub_r + 1;
  if (threadIdx.x == 0) {
    m->roi[0] = sub_r; m->roi[1] = sub_c; m->roi[2] = sub_h; m->roi[3] = sub_w; m->roi[4] = dist;
  }
  const int mh = sub_h + 2, mw = sub_w + 2;
  const float mr = mh / 2.f, mc = mw / 2.f;
  if (threadIdx.x < 64) {
    const int j = threadIdx.x;
    uint64_t bits = 0;
    if (j < mw) {
      const float fc = (float)(j + 1);
      for (int i = 0; i < mh && i < 64; ++i) {
        const float fr = (float)(i + 1);
        const float d = sqrtf((fr - mr) * (fr - mr) + (fc - mc) * (fc - mc));
        if (!(d >= (float)dist)) bits |= 1ull << i;
      }
    }
    colmask[j] = bits;
  }
  __syncthreads();
}

// recompute the mask from a stored ROI (launch start between ROI updates)
__device__ void restore_colmask(uint64_t *colmask, const Misc *m) {
  if (threadIdx.x < 64) {
    const int j = threadIdx.x, h = m->roi[2], w = m->roi[3], dist = m->roi[4];
    uint64_t bits = 0;
    if (h > 0 && w > 0) {
      const int mh = h + 2, mw = w + 2;
      const float mr = mh / 2.f, mc = mw / 2.f;
      if (j < mw) {
        const float fc = (float)(j + 1);
        for (int i = 0; i < mh && i < 64; ++i) {
          const float fr = (float)(i + 1);
          const float d = sqrtf((fr - mr) * (fr - mr) + (fc - mc) * (fc - mc));
          if (!(d >= (float)dist)) bits |= 1ull << i;
        }
      }
    }
    colmask[j] = bits;
  }
}

// The narrow kernel maps lanes to 32 region columns and registers to at most
// 32 region rows.  A 33-wide region fits when its ring columns 0 and 32 are
// entirely fixed (an unclipped ROI): lanes then hold columns 1..32, and the
// rotating shuffle hands lane 0 the value of column 32, which equals that of
// column 0 (both fixed at the external level).  Likewise a region with an
// entirely fixed first row may hold rows 1.. only (row 0 becomes a constant):
// required for 33 rows, and taken for regions wider than 23 columns (those
// use the half-warp layout, whose bands it shortens when nrow % 4 == 1).
// The rotating shuffle also hands column 0 its left neighbour and the last
// column its right one: a column beyond the region (zero, like the ring
// outside the tile) while the region has fewer columns than the lanes hold,
// but the opposite ring column in a 32-wide region.  That is only right when
// both ring columns are fixed; a clipped ROI (against the lattice edge) can
// leave ring sites free, and such a 32-wide region goes to the wide kernel.
// A 35 x 35 region (an unclipped ROI of distance 16) fits when every free site
// lies in rows and columns 1..32 ("ring" mapping): the lanes hold that block,
// whose neighbours outside it are all fixed, and the final substep of the
// ROI's last row and column (33) runs as a separate pass (diffuse_half).
// Called by one thread.
__device__ void narrow_mapping(const uint64_t *colmask, Misc *m, uint32_t layouts) {
  const int nrow = m->roi[2] + 2, ncol = m->roi[3] + 2;
  int ok = 1, roff = 0, coff = 0, ring = 0;
  uint64_t rows_any = 0;  // rows holding a free site
  for (int j = 0; j < ncol && j < 64; ++j) rows_any |= colmask[j];
  if (m->roi[2] == 0 || m->roi[3] == 0) {
    ok = 1;
  } else if (nrow == 35 && ncol == 35 && (layouts & kLayoutRing)) {
    ok = (rows_any & 1ull) == 0 && (rows_any >> 33) == 0 && colmask[0] == 0 &&
         colmask[33] == 0 && colmask[34] == 0;
    roff = coff = ring = 1;
  } else if (ncol > 33 || nrow > 33) {
    ok = 0;
  } else {
    if (ncol == 33) {
      if (colmask[0] != 0 || colmask[32] != 0) ok = 0;
      coff = 1;
    }
    if (ncol == 32 && (colmask[0] != 0 || colmask[31] != 0)) ok = 0;
    if (nrow == 33) {
      if (rows_any & 1ull) ok = 0;
      roff = 1;
    } else if (ncol > 23 && !(rows_any & 1ull)) {
      roff = 1;
    }
  }
  m->narrow_ok = ok;
  m->roff = roff;
  m->coff = coff;
  m->ring = ok ? ring : 0;
  // an unclipped ROI of distance 23 (49 x 49 region): the wide kernel's
  // three-column bands hold its rows and columns 1..48 (wblk)
  int wblk = 0;
  if (nrow == 49 && ncol == 49 && (layouts & kLayoutWideBands) && (rows_any & 1ull) == 0 &&
      (rows_any >> 47) == 0 && colmask[0] == 0 && colmask[47] == 0 && colmask[48] == 0)
    wblk = 1;
  m->wblk = wblk;
}

// ---------------------------------------------------------------------------
// diffusion of one field by one warp of NP = 4 (wide kernel; part k = region
// rows [k*RH, (k+1)*RH) of the (h+2) x (w+2) region; lane = column for
// regions up to 31 columns, columns 2*lane, 2*lane+1 when WIDE).
// With H = x_left + x_right and G = b*x + d*H per site (fmaf(d, H, b*x)):
//   x' = a*x + b*(H + x_up + x_down) + d*(H_up + H_down)
//      = fmaf(a, x, fmaf(b, H, G_up + G_down))
// so a site needs its own x and H and the G of the rows above and below.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void named_barrier(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// producer side of a named barrier: marks arrival without waiting
__device__ __forceinline__ void named_arrive(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

template <int NP, int RH, bool WIDE>
__device__ __noinline__ void diffuse_part(float *__restrict__ f, const uint64_t *__restrict__ colmask,
                                          float4 *__restrict__ xch, int part, int r0, int c0,
                                          int h, int w, int nrow, int ncol, int W, float ext,
                                          float ca, float cb, float cd, int nfree, int bar_id,
                                          int roff, int coff) {
  const int lane = threadIdx.x & 31;
  const int base = part * RH + roff;  // region row of register row 0
  const int j0 = (WIDE ? 2 * lane : lane) + coff;
  const int j1 = 2 * lane + 1;
  const int left = (lane + 31) & 31, right = (lane + 1) & 31;
  const uint32_t rowsel = RH >= 32 ? 0xFFFFFFFFu : (1u << RH) - 1u;
  const uint32_t fm0 = (j0 < ncol) ? (uint32_t)(colmask[j0] >> base) & rowsel : 0u;
  const uint32_t fm1 = (WIDE && j1 < ncol) ? (uint32_t)(colmask[j1] >> base) & rowsel : 0u;
  const uint32_t roirows = (uint32_t)(((((1ull << h) - 1ull) << 1)) >> base) & rowsel;
  const uint32_t rm0 = (j0 >= 1 && j0 <= w) ? roirows : 0u;
  const uint32_t rm1 = (WIDE && j1 >= 1 && j1 <= w) ? roirows : 0u;
  const int lat0 = (r0 - 1) * W + (c0 - 1);
  // G of the row above part 0: the zero ring (G = 0), or region row 0 held at
  // the external level when the mapping starts at row 1
  auto top_g = [&]() -> float {
    if (!roff) return 0.f;
    const float tx = (j0 < ncol) ? ext : 0.f;
    const float th = ((j0 - 1 >= 0 && j0 - 1 < ncol) ? ext : 0.f) + ((j0 + 1 < ncol) ? ext : 0.f);
    return fmaf(cd, th, cb * tx);
  };

  float x0[RH], x1[WIDE ? RH : 1];
#pragma unroll
  for (int i = 0; i < RH; ++i) {
    const int gi = base + i;
    const bool inr = gi < nrow;
    x0[i] = (inr && j0 < ncol) ? (((fm0 >> i) & 1u) ? f[lat0 + gi * W + j0] : ext) : 0.f;
    if (WIDE) x1[i] = (inr && j1 < ncol) ? (((fm1 >> i) & 1u) ? f[lat0 + gi * W + j1] : ext) : 0.f;
  }

  // exchange slot of (parity, part, side); side 0 = the part's first row
  // (read by part - 1), side 1 = its last row (read by part + 1).  One G per
  // lane (two in the wide layout), packed so a warp's slot is 32 consecutive
  // words (64-bit words when wide): conflict-free shared-memory accesses.
  auto slot = [&](int par, int pt, int side) -> float * {
    return reinterpret_cast<float *>(xch) +
           ((NP == 2 ? (par * 2 + pt) : ((par * NP + pt) * 2 + side)) * 32 + lane) * (WIDE ? 2 : 1);
  };
  // two substeps per iteration: the loop-carried tile registers need no
  // copies at the back edge of every substep
#pragma unroll 2
  for (int s = 0; s <= nfree; ++s) {
    const bool fin = (s == nfree);
    const uint32_t u0 = fin ? rm0 : fm0;
    const uint32_t u1 = fin ? rm1 : fm1;
    const int par = s & 1;
    if constexpr (!WIDE) {
      // four warps per field, one column per lane: horizontal sums on the fly
      const float ht0 = __shfl_sync(kFull, x0[0], left) + __shfl_sync(kFull, x0[0], right);
      const float hb0 =
          __shfl_sync(kFull, x0[RH - 1], left) + __shfl_sync(kFull, x0[RH - 1], right);
      const float gt = fmaf(cd, ht0, cb * x0[0]);
      const float gb = fmaf(cd, hb0, cb * x0[RH - 1]);
      if (part > 0) *slot(par, part, 0) = gt;
      if (part < NP - 1) *slot(par, part, 1) = gb;
      named_barrier(bar_id, NP * 32);
      float gm = part > 0 ? *slot(par, part - 1, 1) : top_g();
      const float gx = part < NP - 1 ? *slot(par, part + 1, 0) : 0.f;
      float hc0 = ht0, gc = gt;
#pragma unroll
      for (int i = 0; i < RH; ++i) {
        float hn0 = 0.f, gn;
        if (i + 1 < RH) {
          const float xn0 = x0[i + 1];
          hn0 = (i + 1 == RH - 1) ? hb0
                                  : __shfl_sync(kFull, xn0, left) + __shfl_sync(kFull, xn0, right);
          gn = (i + 1 == RH - 1) ? gb : fmaf(cd, hn0, cb * xn0);
        } else {
          gn = gx;
        }
        const float nv0 = fmaf(ca, x0[i], fmaf(cb, hc0, gm + gn));
        x0[i] = sel_bit(u0, i, nv0, x0[i]);
        gm = gc;
        gc = gn;
        hc0 = hn0;
      }
    } else {
      const float ht0 = __shfl_sync(kFull, x1[0], left) + x1[0];
      const float ht1 = x0[0] + __shfl_sync(kFull, x0[0], right);
      const float hb0 = __shfl_sync(kFull, x1[RH - 1], left) + x1[RH - 1];
      const float hb1 = x0[RH - 1] + __shfl_sync(kFull, x0[RH - 1], right);
      const float gt0 = fmaf(cd, ht0, cb * x0[0]), gt1 = fmaf(cd, ht1, cb * x1[0]);
      const float gb0 = fmaf(cd, hb0, cb * x0[RH - 1]), gb1 = fmaf(cd, hb1, cb * x1[RH - 1]);
      if (part > 0) *reinterpret_cast<float2 *>(slot(par, part, 0)) = make_float2(gt0, gt1);
      if (part < NP - 1) *reinterpret_cast<float2 *>(slot(par, part, 1)) = make_float2(gb0, gb1);
      named_barrier(bar_id, NP * 32);
      float2 pv = make_float2(0.f, 0.f), nx = make_float2(0.f, 0.f);
      if (part > 0) pv = *reinterpret_cast<const float2 *>(slot(par, part - 1, 1));
      if (part < NP - 1) nx = *reinterpret_cast<const float2 *>(slot(par, part + 1, 0));
      float gm0 = pv.x, gm1 = pv.y, gc0 = gt0, gc1 = gt1, hc0 = ht0, hc1 = ht1;
#pragma unroll
      for (int i = 0; i < RH; ++i) {
        float hn0 = 0.f, hn1 = 0.f, gn0, gn1;
        if (i + 1 < RH) {
          const float xn0 = x0[i + 1], xn1 = x1[i + 1];
          if (i + 1 == RH - 1) {
            hn0 = hb0;
            hn1 = hb1;
            gn0 = gb0;
            gn1 = gb1;
          } else {
            hn0 = __shfl_sync(kFull, xn1, left) + xn1;
            hn1 = xn0 + __shfl_sync(kFull, xn0, right);
            gn0 = fmaf(cd, hn0, cb * xn0);
            gn1 = fmaf(cd, hn1, cb * xn1);
          }
        } else {
          gn0 = nx.x;
          gn1 = nx.y;
        }
        const float nv0 = fmaf(ca, x0[i], fmaf(cb, hc0, gm0 + gn0));
        const float nv1 = fmaf(ca, x1[i], fmaf(cb, hc1, gm1 + gn1));
        x0[i] = sel_bit(u0, i, nv0, x0[i]);
        x1[i] = sel_bit(u1, i, nv1, x1[i]);
        gm0 = gc0;
        gc0 = gn0;
        gm1 = gc1;
        gc1 = gn1;
        hc0 = hn0;
        hc1 = hn1;
      }
    }
  }
  // write back the ROI interior
#pragma unroll
  for (int i = 0; i < RH; ++i) {
    const int gi = base + i;
    if (gi >= 1 && gi <= h) {
      if (j0 >= 1 && j0 <= w) f[lat0 + gi * W + j0] = x0[i];
      if (WIDE && j1 >= 1 && j1 <= w) f[lat0 + gi * W + j1] = x1[i];
    }
  }
}

// Two-warp narrow layout with two columns per lane: the 16 lanes of each
// half-warp cover columns 2*hl + coff and 2*hl + 1 + coff (32 columns), the
// half-warps split the warp's rows, so the four half-warps of a field hold
// bands of R rows (band = 2 * part + half).  A horizontal sum costs one
// shuffle per site instead of two; the bands of one warp swap boundary G by
// a shuffle across the half-warps, the two warps through shared memory with
// the same producer/consumer barriers as diffuse_part.  Same sites, same
// expressions as diffuse_part, so the results are bit-identical.
//
// EDGE (the "ring" mapping of narrow_mapping, R = 8): the lanes hold rows and
// columns 1..32 of a 35 x 35 region whose free sites all lie in that block.
// Its left, right, top and bottom neighbours are fixed sites: the shuffles
// that would wrap to the opposite column take the external level instead,
// and the rows above and below are constants.  The final substep of the
// ROI's last row and column (33), outside the block, is computed after the
// loop from the block's last row and column as they were before that
// substep (kept in shared memory), with the same expressions.
template <int R, bool EDGE>
__device__ __noinline__ void diffuse_half(float *__restrict__ f, const uint64_t *__restrict__ colmask,
                                          float4 *__restrict__ xch, int part, int r0, int c0,
                                          int h, int w, int nrow, int ncol, int W, float ext,
                                          float ca, float cb, float cd, int nfree, int bar_id,
                                          int roff, int coff, int field) {
  const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
  const int band = part * 2 + half;
  const int base = band * R + roff;  // region row of register row 0
  const int j0 = 2 * hl + coff, j1 = j0 + 1;
  const int left = (lane & 16) | ((hl + 15) & 15), right = (lane & 16) | ((hl + 1) & 15);
  const uint32_t rowsel = (1u << R) - 1u;
  const uint32_t fm0 = (j0 < ncol) ? (uint32_t)(colmask[j0] >> base) & rowsel : 0u;
  const uint32_t fm1 = (j1 < ncol) ? (uint32_t)(colmask[j1] >> base) & rowsel : 0u;
  const uint32_t roirows = (uint32_t)(((((1ull << h) - 1ull) << 1)) >> base) & rowsel;
  const uint32_t rm0 = (j0 >= 1 && j0 <= w) ? roirows : 0u;
  const uint32_t rm1 = (j1 >= 1 && j1 <= w) ? roirows : 0u;
  const int lat0 = (r0 - 1) * W + (c0 - 1);
  // G of the row above band 0: the zero ring, or region row 0 held at the
  // external level when the mapping starts at row 1
  float top0 = 0.f, top1 = 0.f;
  if (roff) {
    const float tx0 = (j0 < ncol) ? ext : 0.f, tx1 = (j1 < ncol) ? ext : 0.f;
    const float th0 = ((j0 - 1 >= 0 && j0 - 1 < ncol) ? ext : 0.f) + tx1;
    const float th1 = tx0 + ((j1 + 1 < ncol) ? ext : 0.f);
    top0 = fmaf(cd, th0, cb * tx0);
    top1 = fmaf(cd, th1, cb * tx1);
  }
  // G of the row below band 3: the zero ring, or a fixed row (EDGE)
  const float bot = EDGE ? fmaf(cd, ext + ext, cb * ext) : 0.f;
  float *edge = reinterpret_cast<float *>(xch) + 256;  // EDGE: row 32 then column 32
  float x0[R], x1[R];
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int gi = base + i;
    const bool inr = gi < nrow;
    x0[i] = (inr && j0 < ncol) ? (((fm0 >> i) & 1u) ? f[lat0 + gi * W + j0] : ext) : 0.f;
    x1[i] = (inr && j1 < ncol) ? (((fm1 >> i) & 1u) ? f[lat0 + gi * W + j1] : ext) : 0.f;
  }
  // boundary G between the two warps: slot 0 = part 0's last row (written by
  // its second half-warp), slot 1 = part 1's first row (its first half-warp)
  float2 *xs = reinterpret_cast<float2 *>(xch);
  const bool writes = (part == 0) ? half == 1 : half == 0;
  // two substeps per iteration: the loop-carried tile registers need no
  // copies at the back edge of every substep
#pragma unroll 2
  for (int s = 0; s <= nfree; ++s) {
    const bool fin = (s == nfree);
    const uint32_t u0 = fin ? rm0 : fm0;
    const uint32_t u1 = fin ? rm1 : fm1;
    const int par = s & 1;
    if (EDGE && fin) {
      // the block's last row and column before the final substep
      if (band == 3) {
        edge[2 * hl] = x0[R - 1];
        edge[2 * hl + 1] = x1[R - 1];
      }
      if (hl == 15) {
#pragma unroll
        for (int i = 0; i < R; ++i) edge[32 + band * R + i] = x1[i];
      }
    }
    float h0[R], h1[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const float lv = __shfl_sync(kFull, x1[i], left), rv = __shfl_sync(kFull, x0[i], right);
      h0[i] = (EDGE && hl == 0 ? ext : lv) + x1[i];
      h1[i] = x0[i] + (EDGE && hl == 15 ? ext : rv);
    }
    const float gf0 = fmaf(cd, h0[0], cb * x0[0]), gf1 = fmaf(cd, h1[0], cb * x1[0]);
    const float gl0 = fmaf(cd, h0[R - 1], cb * x0[R - 1]);
    const float gl1 = fmaf(cd, h1[R - 1], cb * x1[R - 1]);
    // the first half-warp sends its last row's G, the second its first row's
    const float rc0 = __shfl_xor_sync(kFull, half ? gf0 : gl0, 16);
    const float rc1 = __shfl_xor_sync(kFull, half ? gf1 : gl1, 16);
    const int own = bar_id + par * 2 + part, other = bar_id + par * 2 + (1 - part);
    if (writes) xs[(par * 2 + part) * 16 + hl] = part == 0 ? make_float2(gl0, gl1)
                                                           : make_float2(gf0, gf1);
    named_arrive(own, 64);
    // rows 1 .. R-2 need only this band's G
    float gm0 = gf0, gm1 = gf1;
    float gc0 = R > 1 ? fmaf(cd, h0[R > 1 ? 1 : 0], cb * x0[R > 1 ? 1 : 0]) : 0.f;
    float gc1 = R > 1 ? fmaf(cd, h1[R > 1 ? 1 : 0], cb * x1[R > 1 ? 1 : 0]) : 0.f;
    const float g_second0 = gc0, g_second1 = gc1;
#pragma unroll
    for (int i = 1; i < R - 1; ++i) {
      const float gn0 = (i + 1 == R - 1) ? gl0 : fmaf(cd, h0[i + 1], cb * x0[i + 1]);
      const float gn1 = (i + 1 == R - 1) ? gl1 : fmaf(cd, h1[i + 1], cb * x1[i + 1]);
      const float nv0 = fmaf(ca, x0[i], fmaf(cb, h0[i], gm0 + gn0));
      const float nv1 = fmaf(ca, x1[i], fmaf(cb, h1[i], gm1 + gn1));
      x0[i] = sel_bit(u0, i, nv0, x0[i]);
      x1[i] = sel_bit(u1, i, nv1, x1[i]);
      gm0 = gc0;
      gm1 = gc1;
      gc0 = gn0;
      gc1 = gn1;
    }
    // G of the row before the last (rows 0 .. R-2 are not yet overwritten at
    // their G's computation): the loop leaves it in gm when R > 2
    const float g_penult0 = R > 2 ? gm0 : gf0, g_penult1 = R > 2 ? gm1 : gf1;
    named_barrier(other, 64);
    float2 pw = make_float2(0.f, 0.f);
    if (writes) pw = xs[(par * 2 + (1 - part)) * 16 + hl];
    // above the first row, below the last row
    const float ab0 = band == 0 ? top0 : (half ? rc0 : pw.x);
    const float ab1 = band == 0 ? top1 : (half ? rc1 : pw.y);
    const float be0 = band == 3 ? bot : (half ? pw.x : rc0);
    const float be1 = band == 3 ? bot : (half ? pw.y : rc1);
    if (R == 1) {
      const float nv0 = fmaf(ca, x0[0], fmaf(cb, h0[0], ab0 + be0));
      const float nv1 = fmaf(ca, x1[0], fmaf(cb, h1[0], ab1 + be1));
      x0[0] = sel_bit(u0, 0, nv0, x0[0]);
      x1[0] = sel_bit(u1, 0, nv1, x1[0]);
    } else {
      const float f0 = fmaf(ca, x0[0], fmaf(cb, h0[0], ab0 + g_second0));
      const float f1 = fmaf(ca, x1[0], fmaf(cb, h1[0], ab1 + g_second1));
      const float l0 = fmaf(ca, x0[R - 1], fmaf(cb, h0[R - 1], g_penult0 + be0));
      const float l1 = fmaf(ca, x1[R - 1], fmaf(cb, h1[R - 1], g_penult1 + be1));
      x0[0] = sel_bit(u0, 0, f0, x0[0]);
      x1[0] = sel_bit(u1, 0, f1, x1[0]);
      x0[R - 1] = sel_bit(u0, (R - 1), l0, x0[R - 1]);
      x1[R - 1] = sel_bit(u1, (R - 1), l1, x1[R - 1]);
    }
  }
  // write back the ROI interior
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int gi = base + i;
    if (gi >= 1 && gi <= h) {
      if (j0 >= 1 && j0 <= w) f[lat0 + gi * W + j0] = x0[i];
      if (j1 >= 1 && j1 <= w) f[lat0 + gi * W + j1] = x1[i];
    }
  }
  if (EDGE) {
    // final substep of the ROI's row 33 and column 33: every site there is
    // fixed (x = ext) and so are all its neighbours outside the block;
    // G = fmaf(cd, H, cb*x) and x' = fmaf(ca, x, fmaf(cb, H, G_up + G_down))
    // as in the register tiles, from the block's values before the substep
    named_barrier(13 + field, 64);
    const float gfix = fmaf(cd, ext + ext, cb * ext);  // G of an all-fixed row
    for (int k = part * 32 + lane; k < 65; k += 64) {
      float nv;
      int gi, gj;
      if (k < 33) {  // (33, j): above it row 32 of the block, below it row 34
        gj = k + 1;
        gi = 33;
        const float xl = gj >= 2 ? edge[gj - 2] : ext;
        const float xc = gj <= 32 ? edge[gj - 1] : ext;
        const float xr = gj <= 31 ? edge[gj] : ext;
        const float gu = fmaf(cd, xl + xr, cb * xc);
        nv = fmaf(ca, ext, fmaf(cb, ext + ext, gu + gfix));
      } else {  // (i, 33): left of it column 32 of the block, right of it 34
        gi = k - 32;
        gj = 33;
        const float xu = gi >= 2 ? edge[32 + gi - 2] : ext;
        const float xc = edge[32 + gi - 1];
        const float xd = gi <= 31 ? edge[32 + gi] : ext;
        const float gu = fmaf(cd, xu + ext, cb * ext);
        const float gd = fmaf(cd, xd + ext, cb * ext);
        nv = fmaf(ca, ext, fmaf(cb, xc + ext, gu + gd));
      }
      f[lat0 + gi * W + gj] = nv;
    }
  }
}

// Eight-lane bands for regions up to 8*C - 1 columns (no row or column
// offset; the spare lane column is the zero left neighbour of column 0):
// lane = 8*bw + bl holds columns C*bl .. C*bl + C - 1, a warp holds four bands
// of R rows (bw = 0..3), a field eight (band = 4*part + bw).  Horizontal
// neighbours cost two shuffles per lane and row (one per lane edge); band
// boundaries cross by shuffles up and down by 8 lanes inside a warp and
// through shared memory between the two warps, with the producer/consumer
// barriers of diffuse_half.  Same sites and expressions as diffuse_half, so
// bit-identical results, with C*R lane slots per lane (R = ceil(rows/8))
// instead of 2*ceil(rows/4), for regions up to 15 (C = 2) or 23 (C = 3)
// columns.
template <int C, int R>
__device__ __noinline__ void diffuse_band(float *__restrict__ f, const uint64_t *__restrict__ colmask,
                                          float4 *__restrict__ xch, int part, int r0, int c0,
                                          int h, int w, int nrow, int ncol, int W, float ext,
                                          float ca, float cb, float cd, int nfree, int bar_id) {
  constexpr int L = 8, K = 4;
  const int lane = threadIdx.x & 31, bw = lane >> 3, bl = lane & 7;
  const int band = part * K + bw;
  const int base = band * R;  // region row of register row 0
  const int left = (lane & ~7) | ((bl + 7) & 7), right = (lane & ~7) | ((bl + 1) & 7);
  const uint32_t rowsel = (1u << R) - 1u;
  const uint32_t roirows = (uint32_t)(((((1ull << h) - 1ull) << 1)) >> base) & rowsel;
  const int lat0 = (r0 - 1) * W + (c0 - 1);
  uint32_t fm[C], rm[C];
  float X[C][R];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int j = C * bl + c;
    fm[c] = (j < ncol) ? (uint32_t)(colmask[j] >> base) & rowsel : 0u;
    rm[c] = (j >= 1 && j <= w) ? roirows : 0u;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int gi = base + i;
      X[c][i] = (gi < nrow && j < ncol) ? (((fm[c] >> i) & 1u) ? f[lat0 + gi * W + j] : ext) : 0.f;
    }
  }
  // boundary G between the two warps, C per lane: slot (parity, part) holds
  // part 0's last row (its band 3) or part 1's first row (its band 0)
  float *xs = reinterpret_cast<float *>(xch);
  const bool writes = (part == 0) ? bw == K - 1 : bw == 0;
  // two substeps per iteration: the loop-carried tile registers need no
  // copies at the back edge of every substep
#pragma unroll 2
  for (int s = 0; s <= nfree; ++s) {
    const bool fin = (s == nfree);
    const int par = s & 1;
    float hs[C][R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const float lv = __shfl_sync(kFull, X[C - 1][i], left);
      const float rv = __shfl_sync(kFull, X[0][i], right);
#pragma unroll
      for (int c = 0; c < C; ++c)
        hs[c][i] = (c == 0 ? lv : X[c > 0 ? c - 1 : 0][i]) + (c == C - 1 ? rv : X[c < C - 1 ? c + 1 : 0][i]);
    }
    float gf[C], gl[C], up[C], dn[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      gf[c] = fmaf(cd, hs[c][0], cb * X[c][0]);
      gl[c] = fmaf(cd, hs[c][R - 1], cb * X[c][R - 1]);
      up[c] = __shfl_up_sync(kFull, gl[c], L);    // the band above: its last row
      dn[c] = __shfl_down_sync(kFull, gf[c], L);  // the band below: its first row
    }
    const int own = bar_id + par * 2 + part, other = bar_id + par * 2 + (1 - part);
    if (writes) {
#pragma unroll
      for (int c = 0; c < C; ++c) xs[((par * 2 + part) * L + bl) * C + c] = part == 0 ? gl[c] : gf[c];
    }
    named_arrive(own, 64);
    float g_second[C], g_penult[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const uint32_t u = fin ? rm[c] : fm[c];
      // rows 1 .. R-2 need only this band's G
      float gm = gf[c];
      float gc = R > 1 ? fmaf(cd, hs[c][R > 1 ? 1 : 0], cb * X[c][R > 1 ? 1 : 0]) : 0.f;
      g_second[c] = gc;
#pragma unroll
      for (int i = 1; i < R - 1; ++i) {
        const float gn = (i + 1 == R - 1) ? gl[c] : fmaf(cd, hs[c][i + 1], cb * X[c][i + 1]);
        const float nv = fmaf(ca, X[c][i], fmaf(cb, hs[c][i], gm + gn));
        X[c][i] = sel_bit(u, i, nv, X[c][i]);
        gm = gc;
        gc = gn;
      }
      g_penult[c] = R > 2 ? gm : gf[c];
    }
    named_barrier(other, 64);
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const uint32_t u = fin ? rm[c] : fm[c];
      const float pw = writes ? xs[((par * 2 + (1 - part)) * L + bl) * C + c] : 0.f;
      // above the first row, below the last row
      const float ab = band == 0 ? 0.f : (bw == 0 ? pw : up[c]);
      const float be = band == 2 * K - 1 ? 0.f : (bw == K - 1 ? pw : dn[c]);
      if (R == 1) {
        const float nv = fmaf(ca, X[c][0], fmaf(cb, hs[c][0], ab + be));
        X[c][0] = sel_bit(u, 0, nv, X[c][0]);
      } else {
        const float f0 = fmaf(ca, X[c][0], fmaf(cb, hs[c][0], ab + g_second[c]));
        const float l0 = fmaf(ca, X[c][R - 1], fmaf(cb, hs[c][R - 1], g_penult[c] + be));
        X[c][0] = sel_bit(u, 0, f0, X[c][0]);
        X[c][R - 1] = sel_bit(u, (R - 1), l0, X[c][R - 1]);
      }
    }
  }
  // write back the ROI interior
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int j = C * bl + c;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int gi = base + i;
      if (gi >= 1 && gi <= h && j >= 1 && j <= w) f[lat0 + gi * W + j] = X[c][i];
    }
  }
}

// Half-warp bands of three columns per lane for the wide kernel's regions of
// 32-47 columns and 41-48 rows: lane 16*half + hl holds columns 3*hl ..
// 3*hl + 2, each of the four warps of a field two bands of R rows
// (band = 2*part + half).  The two halves of a warp swap boundary G by a
// shuffle, neighbouring warps through shared-memory slots (double-buffered by
// substep parity) under one named barrier of the field's 128 threads per
// substep, as in diffuse_part.  Same sites and expressions as diffuse_part,
// so bit-identical results, with 18 lane slots per lane (R = 6) instead of 24
// (RH = 12).
//
// BLK (49 x 49 regions of unclipped ROIs, whose free sites all lie in rows and
// columns 1..46): the bands hold rows and columns 1..48 instead of 0..47, so
// the 49th column fits; row 0 above the first band is fixed (a constant G),
// and the wrap of column 1's left neighbour lands on column 48, which is
// fixed like column 0.
template <int R, bool BLK>
__device__ __noinline__ void diffuse_wband(float *__restrict__ f, const uint64_t *__restrict__ colmask,
                                           float4 *__restrict__ xch, int part, int r0, int c0,
                                           int h, int w, int nrow, int ncol, int W, float ext,
                                           float ca, float cb, float cd, int nfree, int bar_id) {
  constexpr int C = 3, NPW = 4, OFF = BLK ? 1 : 0;
  const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
  const int band = part * 2 + half;
  const int base = band * R + OFF;  // region row of register row 0
  const float top = BLK ? fmaf(cd, ext + ext, cb * ext) : 0.f;  // G of the row above band 0
  const int left = (lane & 16) | ((hl + 15) & 15), right = (lane & 16) | ((hl + 1) & 15);
  const uint32_t rowsel = (1u << R) - 1u;
  const uint32_t roirows = (uint32_t)(((((1ull << h) - 1ull) << 1)) >> base) & rowsel;
  const int lat0 = (r0 - 1) * W + (c0 - 1);
  uint32_t fm[C], rm[C];
  float X[C][R];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int j = C * hl + c + OFF;
    fm[c] = (j < ncol) ? (uint32_t)(colmask[j] >> base) & rowsel : 0u;
    rm[c] = (j >= 1 && j <= w) ? roirows : 0u;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int gi = base + i;
      X[c][i] = (gi < nrow && j < ncol) ? (((fm[c] >> i) & 1u) ? f[lat0 + gi * W + j] : ext) : 0.f;
    }
  }
  // exchange slot of (parity, warp, side): side 0 = the warp's first row (its
  // first half-warp's row 0, read by the warp above), side 1 = its last row
  // (read by the warp below); C floats per lane of a half-warp
  auto slot = [&](int par, int pt, int side) -> float * {
    return reinterpret_cast<float *>(xch) + (((par * NPW + pt) * 2 + side) * 16 + hl) * C;
  };
  // two substeps per iteration: the loop-carried tile registers need no
  // copies at the back edge of every substep
#pragma unroll 2
  for (int s = 0; s <= nfree; ++s) {
    const bool fin = (s == nfree);
    const int par = s & 1;
    float hs[C][R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const float lv = __shfl_sync(kFull, X[C - 1][i], left);
      const float rv = __shfl_sync(kFull, X[0][i], right);
#pragma unroll
      for (int c = 0; c < C; ++c)
        hs[c][i] = (c == 0 ? lv : X[c > 0 ? c - 1 : 0][i]) + (c == C - 1 ? rv : X[c < C - 1 ? c + 1 : 0][i]);
    }
    float gf[C], gl[C], rc[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      gf[c] = fmaf(cd, hs[c][0], cb * X[c][0]);
      gl[c] = fmaf(cd, hs[c][R - 1], cb * X[c][R - 1]);
      // the first half-warp sends its last row's G, the second its first row's
      rc[c] = __shfl_xor_sync(kFull, half ? gf[c] : gl[c], 16);
    }
    if (half == 0 && part > 0) {
#pragma unroll
      for (int c = 0; c < C; ++c) slot(par, part, 0)[c] = gf[c];
    }
    if (half == 1 && part < NPW - 1) {
#pragma unroll
      for (int c = 0; c < C; ++c) slot(par, part, 1)[c] = gl[c];
    }
    named_barrier(bar_id, NPW * 32);
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const uint32_t u = fin ? rm[c] : fm[c];
      // the warp above's last row (first half-warp) or the warp below's first
      // row (second half-warp); zero beyond the field's first and last band
      float pw = (half == 0 && part == 0) ? top : 0.f;
      if (half == 0 && part > 0) pw = slot(par, part - 1, 1)[c];
      if (half == 1 && part < NPW - 1) pw = slot(par, part + 1, 0)[c];
      const float ab = half ? rc[c] : pw;  // above the first row
      const float be = half ? pw : rc[c];  // below the last row
      if (R == 1) {
        const float nv = fmaf(ca, X[c][0], fmaf(cb, hs[c][0], ab + be));
        X[c][0] = sel_bit(u, 0, nv, X[c][0]);
      } else {
        // rows 1 .. R-2, then the first and last rows (their G taken before
        // any row of the band changes)
        float gm = gf[c];
        float gc = fmaf(cd, hs[c][R > 1 ? 1 : 0], cb * X[c][R > 1 ? 1 : 0]);
        const float g_second = gc;
#pragma unroll
        for (int i = 1; i < R - 1; ++i) {
          const float gn = (i + 1 == R - 1) ? gl[c] : fmaf(cd, hs[c][i + 1], cb * X[c][i + 1]);
          const float nv = fmaf(ca, X[c][i], fmaf(cb, hs[c][i], gm + gn));
          X[c][i] = sel_bit(u, i, nv, X[c][i]);
          gm = gc;
          gc = gn;
        }
        const float g_penult = R > 2 ? gm : gf[c];
        const float f0 = fmaf(ca, X[c][0], fmaf(cb, hs[c][0], ab + g_second));
        const float l0 = fmaf(ca, X[c][R - 1], fmaf(cb, hs[c][R - 1], g_penult + be));
        X[c][0] = sel_bit(u, 0, f0, X[c][0]);
        X[c][R - 1] = sel_bit(u, (R - 1), l0, X[c][R - 1]);
      }
    }
  }
  // write back the ROI interior
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int j = C * hl + c + OFF;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int gi = base + i;
      if (gi >= 1 && gi <= h && j >= 1 && j <= w) f[lat0 + gi * W + j] = X[c][i];
    }
  }
}

// NP warps per field; warp w diffuses field w / NP, part w % NP.
// The caller guarantees 2*NP*RH_max >= nrow and (WIDE_OK or ncol <= 31).
template <int NP, bool WIDE_OK>
__device__ __forceinline__ void diffuse_step(float *fld, const uint64_t *colmask, float4 *xch,
                                             const Misc *m, const KParams &p) {
  const int r0 = m->roi[0], c0 = m->roi[1], h = m->roi[2], w = m->roi[3];
  if (h == 0 || w == 0) return;
  const int nrow = h + 2, ncol = w + 2;
  const int wid = threadIdx.x >> 5;
  const int field = wid / NP, part = wid % NP;
  const int roff = NP == 2 ? m->roff : 0, coff = NP == 2 ? m->coff : 0;
  const int RH = (((nrow - roff + NP - 1) / NP) + 1) & ~1;  // four-warp path: even rows
  float *f = fld + field * p.HW;
  float4 *x = xch + field * 2 * NP * (NP == 2 ? 1 : 2) * 32;
  const float ext = p.ext[field], ca = p.da[field], cb = p.db[field], cd = p.dd[field];
  // named barriers: 4 ids per field in the two-warp path (2 parts x 2
  // parities), one id per field otherwise; id 0 is __syncthreads
  const int nf = p.nfree, bar = 1 + (NP == 2 ? 4 : 1) * field, W = p.W;
#define EMT6_CALL(R, WD)                                                                   \
  diffuse_part<NP, R, WD>(f, colmask, x, part, r0, c0, h, w, nrow, ncol, W, ext, ca, cb, cd, \
                          nf, bar, roff, coff)
#define EMT6_CASES(WD)               \
  switch (RH) {                      \
    case 2: EMT6_CALL(2, WD); break;   \
    case 4: EMT6_CALL(4, WD); break;   \
    case 6: EMT6_CALL(6, WD); break;   \
    case 8: EMT6_CALL(8, WD); break;   \
    case 10: EMT6_CALL(10, WD); break; \
    case 12: EMT6_CALL(12, WD); break; \
    case 14: EMT6_CALL(14, WD); break; \
    default: break;                    \
  }
  if constexpr (NP == 2) {
    // narrow kernel: two columns per lane, four bands of R rows per field,
    // or eight-lane bands when that takes fewer lane slots
    const int R = (nrow - roff + 3) / 4;
    // (a band layout needs a spare lane column: the shuffle that fetches
    // column 0's left neighbour then wraps to a zero column)
    if (roff == 0 && coff == 0 && ncol <= 23 && (p.layouts & kLayoutBands)) {
      const int R8 = (nrow + 7) / 8;  // nrow <= 32 without a row offset
      const bool two = ncol <= 15;
      if ((two ? 2 : 3) * R8 < 2 * R) {
#define EMT6_BAND(CC, RR) \
  diffuse_band<CC, RR>(f, colmask, x, part, r0, c0, h, w, nrow, ncol, W, ext, ca, cb, cd, nf, bar)
        switch (R8 * 2 + (two ? 0 : 1)) {
          case 2: EMT6_BAND(2, 1); break;
          case 3: EMT6_BAND(3, 1); break;
          case 4: EMT6_BAND(2, 2); break;
          case 5: EMT6_BAND(3, 2); break;
          case 6: EMT6_BAND(2, 3); break;
          case 7: EMT6_BAND(3, 3); break;
          case 8: EMT6_BAND(2, 4); break;
          case 9: EMT6_BAND(3, 4); break;
          default: break;
        }
#undef EMT6_BAND
        return;
      }
    }
#define EMT6_HALF(RR)                                                                         \
  diffuse_half<RR, false>(f, colmask, x, part, r0, c0, h, w, nrow, ncol, W, ext, ca, cb, cd, nf, \
                          bar, roff, coff, field)
    if (m->ring) {
      diffuse_half<8, true>(f, colmask, x, part, r0, c0, h, w, nrow, ncol, W, ext, ca, cb, cd, nf,
                            bar, roff, coff, field);
      return;
    }
    switch (R) {
      case 1: EMT6_HALF(1); break;
      case 2: EMT6_HALF(2); break;
      case 3: EMT6_HALF(3); break;
      case 4: EMT6_HALF(4); break;
      case 5: EMT6_HALF(5); break;
      case 6: EMT6_HALF(6); break;
      case 7: EMT6_HALF(7); break;
      case 8: EMT6_HALF(8); break;
      default: break;
    }
#undef EMT6_HALF
  } else if (!WIDE_OK || ncol <= 31) {
    EMT6_CASES(false)
  } else if ((p.layouts & kLayoutWideBands) && ncol <= 47 && nrow > 40 && nrow <= 48) {
    // 32-47 columns (a spare lane column for the wrap of column 0's left
    // neighbour) and 41-48 rows: half-warp bands of three columns per lane
    // (6 rows each) instead of 12-row tiles of two columns per lane.  Shorter
    // bands do not pay for their per-substep exchange: measured slower than
    // the 10-row tiles at 33-40 rows.
    diffuse_wband<6, false>(f, colmask, x, part, r0, c0, h, w, nrow, ncol, W, ext, ca, cb, cd, nf,
                            bar);
  } else if (m->wblk) {
    diffuse_wband<6, true>(f, colmask, x, part, r0, c0, h, w, nrow, ncol, W, ext, ca, cb, cd, nf,
                           bar);
  } else {
    EMT6_CASES(WIDE_OK)
  }
  (void)coff;
#undef EMT6_CASES
#undef EMT6_CALL
}

// ---------------------------------------------------------------------------
// Site::step (site/site.h:62-82) on the CTA's lattice; returns ready-to-divide.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool step_site(const KParams &p, float *fld, uint8_t *st,
                                          float4 *cells, int s, DCell c, uint32_t vac,
                                          float dose, uint32_t t, uint32_t sim, uint32_t occ,
                                          uint32_t epoch, Misc *m) {
  const int HW = p.HW;
  const uint32_t mp0 = c.mode | (c.phase << 8);
  float l0 = fld[s], l1 = fld[HW + s], l2 = fld[2 * HW + s];
  if (!update_state(c, l0, l1, l2, p, vac)) {
    st[s] = (st[s] & ~kStMask) | kVacant;
    return false;
  }
  if (dose > 0) {
    irradiate(c, dose, p);
    atomicAdd(&m->ins[2], 1u);
  }
  l0 -= p.met[c.mode][0];
  l1 -= p.met[c.mode][1];
  l2 -= p.met[c.mode][2];
  fld[s] = l0;
  fld[HW + s] = l1;
  fld[2 * HW + s] = l2;
  const bool cc = progress_clock(c, p);
  bool dead = false;
  if (repair_pre(c, p, cc)) {
    const float dp = death_prob(c, p);
    atomicAdd(&m->ins[0], 1u);
    atomicAdd(&m->ins_dp, (double)dp);
    int bi = (int)(c.irr / 0.1f);
    bi = bi < 0 ? 0 : (bi >= 300 ? 299 : bi);
    int bj = (int)(c.tir / 0.1f);
    bj = bj < 0 ? 0 : (bj >= 300 ? 299 : bj);
    atomicAdd(&g_instr_hist[bi], 1ull);
    atomicAdd(&g_instr_hist[300 + bj], 1ull);
    const float u = u01(draw(p, t, sim, (uint32_t)s, occ, 1, epoch).x);
    if (u < dp) {
      dead = true;
      atomicAdd(&m->ins[1], 1u);
    } else {
      c.irr = 0.f;
      c.tir = 0.f;
      c.delay = 0.f;
    }
  }
  // the cycle times (t0..t4) never change here: store the clocks and, when
  // they changed, mode and phase (same memory contents as a full store)
  cells[3 * s] = make_float4(c.prolif, c.tir, c.irr, c.delay);
  const uint32_t mp = c.mode | (c.phase << 8);
  if (mp != mp0) reinterpret_cast<float2 *>(cells + 3 * s + 2)[0] = make_float2(c.t4, __uint_as_float(mp));
  if (dead) {
    st[s] = (st[s] & ~kStMask) | kVacant;
    return false;
  }
  return c.phase == 4;
}

// occurrence index of list entry e of a multi-listed site (entries before e
// with the same site): 0 in the rebuilt part, else rebuilt-bit + tail count.
__device__ __forceinline__ uint32_t occurrence(const uint16_t *list, const uint8_t *st, uint32_t e,
                                               uint32_t n0) {
  const int lane = threadIdx.x & 31;
  const uint16_t s = list[e];
  if (e < n0) return 0;
  uint32_t k = (st[s] & kStRebuilt) ? 1u : 0u;
  for (uint32_t b = n0; b < e; b += 32) {
    const uint32_t q = b + lane;
    k += __popc(__ballot_sync(kFull, q < e && list[q] == s));
  }
  return k;
}

// ---------------------------------------------------------------------------
// the fused step kernel
// ---------------------------------------------------------------------------
// WIDE_OK = false: 192 threads, two warps per field, regions up to 32 x 31
// (4 CTAs/SM); a simulation whose region grows beyond that is parked at the
// start of that step for the WIDE_OK = true kernel: 384 threads, four warps
// per field, regions up to 56 x 62 (2 CTAs/SM).
template <bool WIDE_OK>
__global__ void __launch_bounds__(WIDE_OK ? 384 : 192, WIDE_OK ? 2 : 4)
    run_kernel(const RunArgs a, uint32_t t_end) {
  constexpr int NT = WIDE_OK ? 384 : 192;
  constexpr int NP = NT / 96;
  extern __shared__ __align__(16) uint8_t sm[];
  const KParams &p = a.p;
  const int H = p.H, W = p.W, HW = p.HW;
  const SmemLayout L = smem_layout(HW, p.lcap, NP);
  float *fld = reinterpret_cast<float *>(sm + L.fld);
  uint8_t *st = sm + L.st;
  uint16_t *list = reinterpret_cast<uint16_t *>(sm + L.list);
  uint8_t *aux = sm + L.aux;
  uint64_t *colmask = reinterpret_cast<uint64_t *>(sm + L.colmask);
  float4 *xch = reinterpret_cast<float4 *>(sm + L.xch);
  Misc *m = reinterpret_cast<Misc *>(sm + L.misc);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  for (int64_t item = blockIdx.x;; item += gridDim.x) {
    int64_t sim;
    if (a.queue) {
      // persistent CTAs: take the next simulation from the work queue
      __syncthreads();
      if (tid == 0) m->winner = (int)atomicAdd(a.ticket, 1u);
      __syncthreads();
      const int64_t ticket = m->winner;
      if (ticket >= a.nsims) break;
      sim = a.order[ticket];
    } else {
      if (item >= a.nsims) break;
      sim = a.order ? a.order[item] : item;
    }
    {
      // nothing to do for a simulation already at its target step
      const uint32_t hz = a.horizon ? a.horizon[sim] : 0xFFFFFFFFu;
      if (a.step[sim] >= (t_end < hz ? t_end : hz)) continue;
    }

    // ---- load the simulation into shared memory ----
    const float4 *gf = reinterpret_cast<const float4 *>(a.fld + sim * a.fstride);
    for (uint32_t q = tid; q < a.fstride / 4; q += NT)
      reinterpret_cast<float4 *>(fld)[q] = gf[q];
    const uint4 *gs = reinterpret_cast<const uint4 *>(a.st + sim * a.sstride);
    for (uint32_t q = tid; q < a.sstride / 16; q += NT)
      reinterpret_cast<uint4 *>(st)[q] = gs[q];
    const int4 meta = a.meta[sim];
    const uint16_t *gl = a.list + sim * a.lstride;
    for (int q = tid; q < meta.x; q += NT) list[q] = gl[q];
    if (tid == 0) {
      m->n = (uint32_t)meta.x;
      m->n0 = (uint32_t)meta.y;
      m->has_multi = meta.z;
      for (int k = 0; k < 5; ++k) m->roi[k] = a.roi[sim * 8 + k];
      m->ins[0] = m->ins[1] = m->ins[2] = m->ins[3] = 0;
      m->ins_dp = 0.0;
      m->diffused = 0;
    }
    __syncthreads();
    restore_colmask(colmask, m);
    __syncthreads();
    if (tid == 0) {
      unsigned long long nf = 0;
      for (int j = 0; j < 64; ++j) nf += __popcll(colmask[j]);
      m->nfs = nf;
      narrow_mapping(colmask, m, p.layouts);
    }
    float4 *cells = a.cell + sim * (int64_t)HW * 3;
    const uint32_t step0 = a.step[sim];
    const uint32_t horizon = a.horizon ? a.horizon[sim] : 0xFFFFFFFFu;
    const int32_t prot = a.sim_protocol[sim];
    const float *doses = a.doses + (int64_t)prot * p.bins;
    uint32_t t = step0;
    __syncthreads();

    const uint32_t t_stop = t_end < horizon ? t_end : horizon;
    for (; t < t_stop; ++t) {
      if (t % 128 == 0) rebuild_list<NT>(st, list, m, H, W, HW);
      if (t % 32 == 0) {
        compute_roi<NT>(st, colmask, m, H, W, HW);
        if (tid == 0) {
          unsigned long long nf = 0;
          for (int j = 0; j < 64; ++j) nf += __popcll(colmask[j]);
          m->nfs = nf;
          narrow_mapping(colmask, m, p.layouts);
        }
        __syncthreads();
      }
      // a region the narrow mapping cannot hold is left for the wide-capable
      // kernel; the state stored is the state at the start of step t (the list
      // rebuild and ROI above are recomputed identically there)
      if (!WIDE_OK && !m->narrow_ok) break;
      // vacancy snapshot (simulation.cu:79-83), before any site changes
      const uint32_t n = m->n;
      for (uint32_t e = tid; e < n; e += NT) {
        const int s = list[e];
        aux[e] = (uint8_t)(((st[s - W - 1] & kStMask) == kVacant) +
                           ((st[s - W + 1] & kStMask) == kVacant) +
                           ((st[s + W - 1] & kStMask) == kVacant) +
                           ((st[s + W + 1] & kStMask) == kVacant) +
                           ((st[s - 1] & kStMask) == kVacant) + ((st[s + 1] & kStMask) == kVacant) +
                           ((st[s - W] & kStMask) == kVacant) + ((st[s + W] & kStMask) == kVacant));
      }
      diffuse_step<NP, WIDE_OK>(fld, colmask, xch, m, p);
      // diffused site-substeps: free sites x free substeps + the final ROI pass
      if (tid == 0 && m->roi[2] > 0)
        m->diffused += m->nfs * (unsigned long long)p.nfree +
                       (unsigned long long)m->roi[2] * (unsigned long long)m->roi[3];
      __syncthreads();

      // ---- cell update (simulation.cu:84-96) ----
      // may_divide: some cell is ready and may find a vacant neighbour.  A
      // ready cell whose 8 neighbours were all taken at the vacancy snapshot
      // can only find one if a neighbour dies in this step (divisions fill
      // sites only after the arbitration), so the arbitration runs only when
      // a ready cell had a vacant neighbour or some cell died.
      bool may_divide = false;
      const float dose =
          (t < p.length && t % p.res == 0 && t / p.res < p.bins) ? doses[t / p.res] : 0.f;
      {
        // Software pipeline over this thread's entries: the next entry's cell
        // record is loaded from L2 before the current entry is stepped.  Entries
        // of sites listed once name distinct sites, so stepping the current
        // entry never writes the record or state the early load reads.
        uint32_t e = tid;
        DCell nc{};
        if (e < n) {
          const int s0 = list[e];
          if ((st[s0] & (kStMask | kStMulti)) == kOccupied) nc = load_cell(cells + 3 * s0);
        }
        for (; e < n; e += NT) {
          const DCell c = nc;
          const uint32_t en = e + NT;
          if (en < n) {
            const int s2 = list[en];
            if ((st[s2] & (kStMask | kStMulti)) == kOccupied) nc = load_cell(cells + 3 * s2);
          }
          const int s = list[e];
          const uint8_t sv = st[s];
          if ((sv & kStMask) != kOccupied) {
            if (!(sv & kStMulti)) aux[e] = 0;
            continue;
          }
          if (sv & kStMulti) continue;  // stepped in list order below
          const uint32_t vac = aux[e];
          const bool ready = step_site(p, fld, st, cells, s, c, vac, dose, t, (uint32_t)sim, 0,
                                       a.epoch, m);
          aux[e] = ready ? 0x80 : 0;
          may_divide |= (ready && vac != 0) || (st[s] & kStMask) == kVacant;
        }
      }
      if (m->has_multi && wid == 0) {
        // sites listed more than once: every entry steps the site, in list order
        const uint32_t n0 = m->n0;
        for (uint32_t b = 0; b < n; b += 32) {
          const uint32_t e = b + lane;
          const bool mult = e < n && (st[list[e]] & kStMulti);
          uint32_t bal = __ballot_sync(kFull, mult);
          while (bal) {
            const int bit = __ffs(bal) - 1;
            bal &= bal - 1;
            const uint32_t ee = b + bit;
            const uint32_t occ = occurrence(list, st, ee, n0);
            if (lane == 0) {
              const int s = list[ee];
              uint8_t res = 0;
              if ((st[s] & kStMask) == kOccupied) {
                const uint32_t vac = aux[ee] & 15u;
                const bool ready = step_site(p, fld, st, cells, s, load_cell(cells + 3 * s), vac,
                                             dose, t, (uint32_t)sim, occ, a.epoch, m);
                if (ready) {
                  if (occ > 127) atomicOr(a.err, 4u);
                  res = (uint8_t)(0x80 | (occ & 0x7f));
                }
                may_divide |= (ready && vac != 0) || (st[s] & kStMask) == kVacant;
              }
              aux[ee] = res;
            }
            __syncwarp();
          }
        }
      }
      // most steps have no cell that may divide: skip the arbitration then
      if (!__syncthreads_or(may_divide)) continue;

      // ---- division arbitration: lowest list index with a vacant target ----
      int best = 0x7fffffff, best_target = -1;
      for (uint32_t e = tid; e < n; e += NT) {
        const uint8_t av = aux[e];
        if (av & 0x80) {
          const int s = list[e];
          // a cell none of whose neighbours is vacant now cannot divide,
          // whatever the draw: skip the draw (interior cells stay ready)
          const bool open = ((st[s - W - 1] & kStMask) == kVacant) |
                            ((st[s - W] & kStMask) == kVacant) |
                            ((st[s - W + 1] & kStMask) == kVacant) |
                            ((st[s - 1] & kStMask) == kVacant) |
                            ((st[s + 1] & kStMask) == kVacant) |
                            ((st[s + W - 1] & kStMask) == kVacant) |
                            ((st[s + W] & kStMask) == kVacant) |
                            ((st[s + W + 1] & kStMask) == kVacant);
          if (!open) continue;
          const float u = u01(draw(p, t, (uint32_t)sim, (uint32_t)s, av & 0x7fu, 0, a.epoch).x);
          const int tg = choose_neighbour(s, W, u);
          if ((st[tg] & kStMask) == kVacant) {
            best = (int)e;
            best_target = tg;
            break;
          }
        }
      }
      const int win = block_min<NT>(best, m);
      if (win != 0x7fffffff && best == win) {
        m->winner = win;
        m->target = best_target;
      }
      __syncthreads();
      if (win != 0x7fffffff && wid == 0) {
        // divideCell (cell-division.h:10-30) with five Philox normals; lanes
        // 0..2 each evaluate one Box-Muller pair
        float za = 0.f, zb = 0.f;
        if (lane < 3) {
          const uint4 r = draw(p, t, (uint32_t)sim, 0xFFFFu, 0, lane == 2 ? 3 : 2, a.epoch);
          if (lane == 0) box_muller(r.x, r.y, &za, &zb);
          else if (lane == 1) box_muller(r.z, r.w, &za, &zb);
          else box_muller(r.x, r.y, &za, &zb);
        }
        float z[5];
        z[0] = __shfl_sync(kFull, za, 0);
        z[1] = __shfl_sync(kFull, zb, 0);
        z[2] = __shfl_sync(kFull, za, 1);
        z[3] = __shfl_sync(kFull, zb, 1);
        z[4] = __shfl_sync(kFull, za, 2);
        if (lane == 0) {
          const int parent = list[m->winner], child = m->target;
          DCell pc = load_cell(cells + 3 * parent);
          pc.phase = 0;
          pc.prolif = 0.f;
          store_cell(cells + 3 * parent, pc);
          const DCell cc = make_child(pc, z, p);
          store_cell(cells + 3 * child, cc);
          const uint8_t sv = st[child];
          const bool listed = (sv & (kStRebuilt | kStTail)) != 0;
          st[child] = (uint8_t)((sv & (kStRebuilt | kStTail | kStMulti)) | kStTail |
                                (listed ? kStMulti : 0) | kOccupied);
          if (listed) m->has_multi = 1;
          if (m->n < (uint32_t)p.lcap) list[m->n++] = (uint16_t)child;
          else atomicOr(a.err, 1u);
          m->ins[3] += 1;
        }
      }
      __syncthreads();
    }

    // ---- write the simulation back ----
    float4 *of = reinterpret_cast<float4 *>(a.fld + sim * a.fstride);
    for (uint32_t q = tid; q < a.fstride / 4; q += NT)
      of[q] = reinterpret_cast<const float4 *>(fld)[q];
    uint4 *os = reinterpret_cast<uint4 *>(a.st + sim * a.sstride);
    for (uint32_t q = tid; q < a.sstride / 16; q += NT)
      os[q] = reinterpret_cast<const uint4 *>(st)[q];
    uint16_t *ol = a.list + sim * a.lstride;
    for (uint32_t q = tid; q < m->n; q += NT) ol[q] = list[q];
    int live = 0;
    for (int q = tid; q < HW; q += NT) live += (st[q] & kStMask) == kOccupied;
#pragma unroll
    for (int o = 16; o; o >>= 1) live += __shfl_xor_sync(kFull, live, o);
    __syncthreads();
    if (lane == 0) m->red[wid][1] = live;
    __syncthreads();
    if (tid == 0) {
      int tot = 0;
      for (int w2 = 0; w2 < NT / 32; ++w2) tot += m->red[w2][1];
      a.counts[sim] = (uint32_t)tot;
      a.meta[sim] = make_int4((int)m->n, (int)m->n0, m->has_multi, 0);
      for (int k2 = 0; k2 < 5; ++k2) a.roi[sim * 8 + k2] = m->roi[k2];
      a.step[sim] = t;
      if (m->ins[0]) atomicAdd(&g_instr_counts[0], (unsigned long long)m->ins[0]);
      if (m->ins[1]) atomicAdd(&g_instr_counts[1], (unsigned long long)m->ins[1]);
      if (m->ins[2]) atomicAdd(&g_instr_counts[2], (unsigned long long)m->ins[2]);
      if (m->ins[3]) atomicAdd(&g_instr_counts[3], (unsigned long long)m->ins[3]);
      if (m->ins_dp != 0.0) atomicAdd(&g_instr_sum_death_prob, m->ins_dp);
      if (m->diffused) atomicAdd(a.diffused, m->diffused);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// launch order: simulations sorted by the region their next step diffuses
// (largest first), so the CTAs resident on an SM at once mostly run the same
// diffusion tile code and take similar times.  A counting sort over the
// region's (rows, columns) key: count, exclusive scan, scatter.  The order
// inside a key is whatever the atomics give; results do not depend on it
// (every draw is keyed by the simulation, not by the CTA).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t order_key(const RunArgs &a, int64_t sim, uint32_t t_end) {
  const uint32_t hz = a.horizon ? a.horizon[sim] : 0xFFFFFFFFu;
  if (a.step[sim] >= (t_end < hz ? t_end : hz)) return kOrderKeys - 1;  // nothing to do: last
  const int h = a.roi[sim * 8 + 2], w = a.roi[sim * 8 + 3];
  // regions are at most 56 x 62 (lattice limit); the clamps keep any key in
  // [0, kOrderKeys - 2] whatever the stored ROI holds
  const uint32_t nr = (uint32_t)min(max(h + 2, 0), 62), nc = (uint32_t)min(max(w + 2, 0), 63);
  return (kOrderKeys - 2) - (nr * 64u + nc);
}

__global__ void order_count_kernel(const RunArgs a, uint32_t t_end, uint32_t *hist) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.nsims;
       i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&hist[order_key(a, i, t_end)], 1u);
}

static_assert(kOrderKeys == 4 * 1024, "order_scan_kernel scans four counters per thread");

__global__ void __launch_bounds__(1024) order_scan_kernel(uint32_t *hist) {
  // kOrderKeys = 4 x 1024 counters: each thread scans four, then the block
  __shared__ uint32_t part[1024];
  const int t = threadIdx.x;
  uint32_t v[4], run = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = run;
    run += hist[4 * t + k];
  }
  part[t] = run;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const uint32_t add = t >= o ? part[t - o] : 0u;
    __syncthreads();
    part[t] += add;
    __syncthreads();
  }
  const uint32_t base = part[t] - run;
#pragma unroll
  for (int k = 0; k < 4; ++k) hist[4 * t + k] = base + v[k];
}

__global__ void order_scatter_kernel(const RunArgs a, uint32_t t_end, uint32_t *hist,
                                     int64_t *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.nsims;
       i += (int64_t)gridDim.x * blockDim.x)
    out[atomicAdd(&hist[order_key(a, i, t_end)], 1u)] = i;
}

// ---------------------------------------------------------------------------
// reset: expand the initial tumours into every simulation
// ---------------------------------------------------------------------------
__global__ void reset_kernel(const ResetArgs a) {
  for (int64_t sim = blockIdx.x; sim < a.nsims; sim += gridDim.x) {
    const int t = a.sim_tumor[sim];
    const float4 *sf = reinterpret_cast<const float4 *>(a.tpl_fld + (int64_t)t * a.fstride);
    float4 *df = reinterpret_cast<float4 *>(a.fld + sim * a.fstride);
    for (uint32_t q = threadIdx.x; q < a.fstride / 4; q += blockDim.x) df[q] = sf[q];
    const uint4 *ss = reinterpret_cast<const uint4 *>(a.tpl_st + (int64_t)t * a.sstride);
    uint4 *ds = reinterpret_cast<uint4 *>(a.st + sim * a.sstride);
    for (uint32_t q = threadIdx.x; q < a.sstride / 16; q += blockDim.x) ds[q] = ss[q];
    const float4 *sc = a.tpl_cell + (int64_t)t * a.HW * 3;
    float4 *dc = a.cell + sim * (int64_t)a.HW * 3;
    for (int q = threadIdx.x; q < a.HW * 3; q += blockDim.x) dc[q] = sc[q];
    if (threadIdx.x == 0) {
      a.meta[sim] = make_int4(0, 0, 0, 0);
      for (int k = 0; k < 8; ++k) a.roi[sim * 8 + k] = 0;
      a.step[sim] = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// unit hooks: run the device functions above on caller-provided inputs
// ---------------------------------------------------------------------------
__global__ void test_philox_kernel(const uint4 *ctr, const uint2 *key, uint4 *out, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = philox4x32_10(ctr[i], key[i].x, key[i].y);
}

__global__ void test_math_kernel(const float *x, float *ex, const double *u, double *lg, double *sn,
                                 double *cs, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    ex[i] = dexpf(x[i]);
    lg[i] = log_core(u[i] > 0 ? u[i] : 1.0);
    double s, c;
    double v = u[i] - floor(u[i]);
    sincos2pi(v, &s, &c);
    sn[i] = s;
    cs[i] = c;
  }
}

__global__ void test_site_step_kernel(const KParams p, float4 *cells, float *lv, uint8_t *state,
                                      const uint32_t *vac, const float *dose, const float *draws,
                                      int32_t *ready, int32_t *used, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  ready[i] = 0;
  used[i] = 0;
  if (state[i] != kOccupied) return;
  DCell c = load_cell(cells + 3 * i);
  float l0 = lv[3 * i], l1 = lv[3 * i + 1], l2 = lv[3 * i + 2];
  if (!update_state(c, l0, l1, l2, p, vac[i])) {
    state[i] = kVacant;
    store_cell(cells + 3 * i, c);
    return;
  }
  if (dose[i] > 0) irradiate(c, dose[i], p);
  l0 -= p.met[c.mode][0];
  l1 -= p.met[c.mode][1];
  l2 -= p.met[c.mode][2];
  lv[3 * i] = l0; lv[3 * i + 1] = l1; lv[3 * i + 2] = l2;
  const bool cc = progress_clock(c, p);
  bool dead = false;
  if (repair_pre(c, p, cc)) {
    used[i] = 1;
    if (draws[i] < death_prob(c, p)) dead = true;
    else { c.irr = 0.f; c.tir = 0.f; c.delay = 0.f; }
  }
  store_cell(cells + 3 * i, c);
  if (dead) state[i] = kVacant;
  else ready[i] = c.phase == 4;
}

__global__ void test_choose_kernel(const float *u, int r, int c, int W, int32_t *rc, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    int s = choose_neighbour(r * W + c, W, u[i]);
    rc[2 * i] = s / W;
    rc[2 * i + 1] = s % W;
  }
}

__global__ void test_divide_kernel(const KParams p, float4 *parents, const float *z,
                                   float4 *children, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  DCell pc = load_cell(parents + 3 * i);
  pc.phase = 0;
  pc.prolif = 0.f;
  store_cell(parents + 3 * i, pc);
  float zz[5] = {z[5 * i], z[5 * i + 1], z[5 * i + 2], z[5 * i + 3], z[5 * i + 4]};
  store_cell(children + 3 * i, make_child(pc, zz, p));
}

__global__ void test_normals_kernel(const KParams p, const uint32_t *step, const uint32_t *sim,
                                    uint32_t epoch, float *z, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 r1 = draw(p, step[i], sim[i], 0xFFFFu, 0, 2, epoch);
  const uint4 r2 = draw(p, step[i], sim[i], 0xFFFFu, 0, 3, epoch);
  float unused;
  box_muller(r1.x, r1.y, &z[5 * i], &z[5 * i + 1]);
  box_muller(r1.z, r1.w, &z[5 * i + 2], &z[5 * i + 3]);
  box_muller(r2.x, r2.y, &z[5 * i + 4], &unused);
}

// one CTA: list rebuild + ROI on a lattice, or one diffusion step with the
// narrow (WIDE_OK = false) or wide kernel's diffusion path
template <bool WIDE_OK>
__global__ void __launch_bounds__(WIDE_OK ? 384 : 192)
    test_block_kernel(const KParams p, int mode, float *gfld, const uint8_t *gst, int32_t *roi,
                      uint8_t *mask, uint16_t *glist, uint32_t *gn) {
  constexpr int NT = WIDE_OK ? 384 : 192;
  constexpr int NP = NT / 96;
  extern __shared__ __align__(16) uint8_t sm[];
  const int HW = p.HW;
  const SmemLayout L = smem_layout(HW, p.lcap, NP);
  float *fld = reinterpret_cast<float *>(sm + L.fld);
  uint8_t *st = sm + L.st;
  uint16_t *list = reinterpret_cast<uint16_t *>(sm + L.list);
  uint64_t *colmask = reinterpret_cast<uint64_t *>(sm + L.colmask);
  float4 *xch = reinterpret_cast<float4 *>(sm + L.xch);
  Misc *m = reinterpret_cast<Misc *>(sm + L.misc);
  for (int q = threadIdx.x; q < HW; q += NT) st[q] = gst ? gst[q] : 0;
  if (gfld)
    for (int q = threadIdx.x; q < 3 * HW; q += NT) fld[q] = gfld[q];
  __syncthreads();
  if (mode == 0) {
    rebuild_list<NT>(st, list, m, p.H, p.W, HW);
    for (uint32_t q = threadIdx.x; q < m->n; q += NT) glist[q] = list[q];
    if (threadIdx.x == 0) *gn = m->n;
  } else if (mode == 1) {
    compute_roi<NT>(st, colmask, m, p.H, p.W, HW);
    if (threadIdx.x == 0)
      for (int k = 0; k < 5; ++k) roi[k] = m->roi[k];
    const int mh = m->roi[2] + 2, mw = m->roi[3] + 2;
    if (m->roi[2] > 0)
      for (int q = threadIdx.x; q < mh * mw; q += NT) {
        int i = q / mw, j = q % mw;
        mask[q] = ((colmask[j] >> i) & 1ull) ? 0 : 1;
      }
  } else {
    if (threadIdx.x == 0)
      for (int k = 0; k < 5; ++k) m->roi[k] = roi[k];
    __syncthreads();
    restore_colmask(colmask, m);
    __syncthreads();
    if (threadIdx.x == 0) {
      narrow_mapping(colmask, m, p.layouts);
      if (WIDE_OK) m->roff = m->coff = m->ring = 0;
      if (!WIDE_OK) m->wblk = 0;
      *gn = (WIDE_OK || m->narrow_ok) ? 0u : 1u;
    }
    __syncthreads();
    if (!WIDE_OK && !m->narrow_ok) return;
    diffuse_step<NP, WIDE_OK>(fld, colmask, xch, m, p);
    __syncthreads();
    for (int q = threadIdx.x; q < 3 * HW; q += NT) gfld[q] = fld[q];
  }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
// the dynamic shared-memory limit is raised once per device and size (the
// attribute call is kept out of CUDA-graph captures)
static size_t g_smem_set[2][64];

static cudaError_t ensure_smem(bool wide, size_t smem) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) dev = 63;
  if (g_smem_set[wide][dev] >= smem) return cudaSuccess;
  e = wide ? cudaFuncSetAttribute(run_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem)
           : cudaFuncSetAttribute(run_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem);
  if (e == cudaSuccess) g_smem_set[wide][dev] = smem;
  return e;
}

cudaError_t launch_run(const RunArgs &a, uint32_t t_end, bool wide, int grid,
                       cudaStream_t stream) {
  const size_t smem = run_kernel_smem(a.p.HW, a.p.lcap, wide);
  cudaError_t e = ensure_smem(wide, smem);
  if (e != cudaSuccess) return e;
  if (wide)
    run_kernel<true><<<grid, 384, smem, stream>>>(a, t_end);
  else
    run_kernel<false><<<grid, 192, smem, stream>>>(a, t_end);
  return cudaGetLastError();
}

cudaError_t launch_order(const RunArgs &a, uint32_t t_end, uint32_t *hist, int64_t *out,
                         cudaStream_t stream) {
  if (a.nsims < 1) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(hist, 0, kOrderKeys * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  const int64_t blocks = (a.nsims + 255) / 256;
  const int grid = (int)(blocks < 4096 ? blocks : 4096);
  order_count_kernel<<<grid, 256, 0, stream>>>(a, t_end, hist);
  order_scan_kernel<<<1, 1024, 0, stream>>>(hist);
  order_scatter_kernel<<<grid, 256, 0, stream>>>(a, t_end, hist, out);
  return cudaGetLastError();
}

cudaError_t launch_reset(const ResetArgs &a, cudaStream_t stream) {
  int grid = (int)(a.nsims < 65535 * 8 ? a.nsims : 65535 * 8);
  if (grid < 1) return cudaSuccess;
  reset_kernel<<<grid, 256, 0, stream>>>(a);
  return cudaGetLastError();
}

int max_ctas_per_sm(const KParams &p, bool wide) {
  const size_t smem = run_kernel_smem(p.HW, p.lcap, wide);
  int n = 0;
  if (ensure_smem(wide, smem) != cudaSuccess) return 0;
  if (wide) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, run_kernel<true>, 384, smem) !=
        cudaSuccess)
      return 0;
  } else {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, run_kernel<false>, 192, smem) !=
        cudaSuccess)
      return 0;
  }
  return n;
}

cudaError_t instr_read(unsigned long long counts[4], double *sum_dp, unsigned long long *hist) {
  cudaError_t e = cudaMemcpyFromSymbol(counts, g_instr_counts, sizeof(unsigned long long) * 4);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyFromSymbol(sum_dp, g_instr_sum_death_prob, sizeof(double));
  if (e != cudaSuccess) return e;
  if (hist) e = cudaMemcpyFromSymbol(hist, g_instr_hist, sizeof(unsigned long long) * 600);
  return e;
}

cudaError_t instr_reset() {
  unsigned long long z[600] = {0};
  double zd = 0.0;
  cudaError_t e = cudaMemcpyToSymbol(g_instr_counts, z, sizeof(unsigned long long) * 4);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyToSymbol(g_instr_sum_death_prob, &zd, sizeof(double));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(g_instr_hist, z, sizeof(z));
}

// FP32 issue-rate probe: 8 independent FMA chains per thread, register only
__global__ void __launch_bounds__(256) fma_probe_kernel(float *out, float a, float b, int iters) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = a * (threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], b, a);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t fp32_peak(int device, double *tflops) {
  int sms = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  const int blocks = sms * 8, threads = 256, iters = 8192;
  float *out = nullptr;
  e = cudaMalloc(&out, sizeof(float) * blocks * threads);
  if (e != cudaSuccess) return e;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  double best = 0;
  for (int rep = 0; rep < 12; ++rep) {
    cudaEventRecord(t0);
    fma_probe_kernel<<<blocks, threads>>>(out, 1.0001f, 0.9999f, iters);
    cudaEventRecord(t1);
    e = cudaEventSynchronize(t1);
    if (e != cudaSuccess) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    const double flop = 2.0 * 8 * (double)iters * blocks * threads;
    if (rep >= 2 && ms > 0) best = fmax(best, flop / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  *tflops = best;
  return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t launch_test_philox(const uint4 *c, const uint2 *k, uint4 *o, int64_t n) {
  test_philox_kernel<<<(unsigned)((n + 127) / 128), 128>>>(c, k, o, n);
  return cudaGetLastError();
}
cudaError_t launch_test_math(const float *x, float *ex, const double *u, double *lg, double *sn,
                             double *cs, int64_t n) {
  test_math_kernel<<<(unsigned)((n + 127) / 128), 128>>>(x, ex, u, lg, sn, cs, n);
  return cudaGetLastError();
}
cudaError_t launch_test_site_step(const KParams &p, float4 *cells, float *lv, uint8_t *state,
                                  const uint32_t *vac, const float *dose, const float *draws,
                                  int32_t *ready, int32_t *used, int64_t n) {
  test_site_step_kernel<<<(unsigned)((n + 127) / 128), 128>>>(p, cells, lv, state, vac, dose,
                                                               draws, ready, used, n);
  return cudaGetLastError();
}
cudaError_t launch_test_choose(const float *u, int r, int c, int W, int32_t *rc, int64_t n) {
  test_choose_kernel<<<(unsigned)((n + 127) / 128), 128>>>(u, r, c, W, rc, n);
  return cudaGetLastError();
}
cudaError_t launch_test_divide(const KParams &p, float4 *parents, const float *z, float4 *children,
                               int64_t n) {
  test_divide_kernel<<<(unsigned)((n + 127) / 128), 128>>>(p, parents, z, children, n);
  return cudaGetLastError();
}
cudaError_t launch_test_normals(const KParams &p, const uint32_t *step, const uint32_t *sim,
                                uint32_t epoch, float *z, int64_t n) {
  test_normals_kernel<<<(unsigned)((n + 127) / 128), 128>>>(p, step, sim, epoch, z, n);
  return cudaGetLastError();
}
cudaError_t launch_test_block(const KParams &p, int mode, bool wide, float *fld,
                              const uint8_t *st, int32_t *roi, uint8_t *mask, uint16_t *list,
                              uint32_t *n) {
  const size_t smem = run_kernel_smem(p.HW, p.lcap, wide);
  cudaError_t e;
  if (wide) {
    e = cudaFuncSetAttribute(test_block_kernel<true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    test_block_kernel<true><<<1, 384, smem>>>(p, mode, fld, st, roi, mask, list, n);
  } else {
    e = cudaFuncSetAttribute(test_block_kernel<false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    test_block_kernel<false><<<1, 192, smem>>>(p, mode, fld, st, roi, mask, list, n);
  }
  return cudaGetLastError();
}

}  // namespace emt6
