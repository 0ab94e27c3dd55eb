// emt6_kernels.h -- interface between the host engine and the sm_103a kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "emt6_device.cuh"

namespace emt6 {

// Device-resident batch, simulation-major.  Per simulation: fields
// [3][H*W] FP32 (stride fstride floats), state bytes (sstride), cell records
// [H*W][3] float4, occupied list (lstride u16), meta = (n, n0, multi, -),
// roi[8] = (r0, c0, h, w, dist, -, -, -), step counter.
struct RunArgs {
  KParams p;
  float *fld;
  uint8_t *st;
  float4 *cell;
  uint16_t *list;
  int4 *meta;
  int32_t *roi;
  uint32_t *step;
  const uint32_t *horizon;
  const int32_t *sim_protocol;
  const float *doses;
  uint32_t *counts;
  uint32_t *err;
  unsigned long long *diffused;
  uint32_t fstride, sstride, lstride, epoch;
  int64_t nsims;
  int queue;  // 1: persistent CTAs take simulations from order[] via *ticket
  uint32_t *ticket;
  const int64_t *order;  // simulation of each CTA or ticket (null: the identity)
};

struct ResetArgs {
  float *fld;
  uint8_t *st;
  float4 *cell;
  int4 *meta;
  int32_t *roi;
  uint32_t *step;
  const float *tpl_fld;
  const uint8_t *tpl_st;
  const float4 *tpl_cell;
  const int32_t *sim_tumor;
  uint32_t fstride, sstride;
  int HW;
  int64_t nsims;
};

size_t run_kernel_smem(int HW, int lcap, bool wide);
int max_ctas_per_sm(const KParams &p, bool wide);
// Advance every simulation to step min(t_end, horizon).  wide = false runs the
// narrow-region kernel (4 CTAs/SM), which stops a simulation at the first step
// whose ROI is wider than 31 columns; wide = true finishes such simulations.
cudaError_t launch_run(const RunArgs &a, uint32_t t_end, bool wide, int grid,
                       cudaStream_t stream);
cudaError_t launch_reset(const ResetArgs &a, cudaStream_t stream);
// simulations sorted largest region first into out[0 .. a.nsims) for the
// launches of a chunk ending at t_end; hist holds kOrderKeys counters
constexpr uint32_t kOrderKeys = 4096;
cudaError_t launch_order(const RunArgs &a, uint32_t t_end, uint32_t *hist, int64_t *out,
                         cudaStream_t stream);
cudaError_t instr_read(unsigned long long counts[4], double *sum_dp, unsigned long long *hist);
cudaError_t instr_reset();
cudaError_t fp32_peak(int device, double *tflops);

cudaError_t launch_test_philox(const uint4 *c, const uint2 *k, uint4 *o, int64_t n);
cudaError_t launch_test_math(const float *x, float *ex, const double *u, double *lg, double *sn,
                             double *cs, int64_t n);
cudaError_t launch_test_site_step(const KParams &p, float4 *cells, float *lv, uint8_t *state,
                                  const uint32_t *vac, const float *dose, const float *draws,
                                  int32_t *ready, int32_t *used, int64_t n);
cudaError_t launch_test_choose(const float *u, int r, int c, int W, int32_t *rc, int64_t n);
cudaError_t launch_test_divide(const KParams &p, float4 *parents, const float *z,
                               float4 *children, int64_t n);
cudaError_t launch_test_normals(const KParams &p, const uint32_t *step, const uint32_t *sim,
                                uint32_t epoch, float *z, int64_t n);
cudaError_t launch_test_block(const KParams &p, int mode, bool wide, float *fld,
                              const uint8_t *st, int32_t *roi, uint8_t *mask, uint16_t *list,
                              uint32_t *n);

}  // namespace emt6
