// ref_cell_kernels.cu -- the reference's own cell model, compiled for the GPU.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build.py (build_ref_cell_cubin) compiles
// this file against the reference's headers where they lie, together with
// the reference's src/emt6ro/cell/cell.cu, for sm_103a with nvcc's defaults
// (FMA contraction on, CUDA's expf), and device-links both into
// oracle/_ref/emt6ro_ref_cell_sm103a.cubin.  oracle/ref_gpu_driver.cu loads
// it by the unmangled names below.  The kernels drive the reference's
// templated functions (Site::step<R>, site/site.h:62-82; divideCell<R> and
// chooseNeighbour<R>, simulation/cell-division.h:10-54) with injected draws,
// so the reference's device build can be compared with this project's
// kernels on identical inputs.
#include <cstdint>

#include "emt6ro/simulation/cell-division.h"
#include "emt6ro/site/site.h"

namespace {

// serves injected draws: uniform() returns the next value, normal(p) returns
// p.stddev * z + p.mean for the next z (the reference's RandEngine interface)
struct DeviceReplay {
  const float *v;
  int n;
  int i;
  __device__ float uniform() { return i < n ? v[i++] : 0.5f; }
  __device__ float normal(const emt6ro::Parameters::NormalDistribution &p) {
    const float z = i < n ? v[i++] : 0.f;
    return p.stddev * z + p.mean;
  }
};

}  // namespace

// Site::step on site i with vac[i] vacant neighbours, dose[i] and the draws
// draws[i * ndraw ..]; ready[i] = its return value, used[i] = draws consumed.
extern "C" __global__ void ref_site_step_kernel(emt6ro::Site *sites, emt6ro::Parameters params,
                                                const uint32_t *vac, const float *dose,
                                                const float *draws, int ndraw, int32_t *ready,
                                                int32_t *used, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  DeviceReplay rr{draws + i * ndraw, ndraw, 0};
  const bool r = sites[i].step(params, static_cast<uint8_t>(vac[i]), dose[i], rr);
  ready[i] = r ? 1 : 0;
  used[i] = rr.i;
}

// divideCell on parents[i] with the five standard normals z[5 i .. 5 i + 4];
// the child's cell goes to children[i].
extern "C" __global__ void ref_divide_kernel(emt6ro::Site *parents, emt6ro::Site *children,
                                             emt6ro::Parameters params, const float *z,
                                             int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  DeviceReplay rr{z + 5 * i, 5, 0};
  children[i].cell = emt6ro::divideCell(parents[i].cell, params, rr);
}

// chooseNeighbour of site (r, c) for the uniform u[i]: rc[2 i], rc[2 i + 1].
extern "C" __global__ void ref_choose_kernel(const float *u, int r, int c, int32_t *rc,
                                             int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  DeviceReplay rr{u + i, 1, 0};
  const emt6ro::Coords co =
      emt6ro::chooseNeighbour(static_cast<uint32_t>(r), static_cast<uint32_t>(c), rr);
  rc[2 * i] = co.r;
  rc[2 * i + 1] = co.c;
}
