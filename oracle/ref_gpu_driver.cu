// ref_gpu_driver.cu -- runs the reference's own CUDA kernels on the GPU.
//
// BENCHMARK INFRASTRUCTURE ONLY (bench.py's reference-kernel comparison).
// oracle/build.py compiles the reference's CUDA sources where they lie
// (src/emt6ro/{simulation,diffusion,statistics,cell,common}/*.cu) for sm_103a
// and device-links them into oracle/_ref/emt6ro_ref_sm103a.cubin; this file
// loads that cubin with the CUDA driver API and drives its kernels with a host
// loop that restates Simulation's constructor, step() and getResults()
// (src/emt6ro/simulation/simulation.cu:114-198, statistics/statistics.cu:30-38):
//   every 128 steps findOccupied<<<B, 32, 128 B>>>
//   every 32 steps  findROIsKernel<<<B, 16x16, 64 B>>>
//   every step      diffusionKernel<<<B, 32x32, 12 (H+4)(W+4) B>>>
//                   cellSimulationKernel<<<B, 512, 128 B>>>
// The kernel names are the Itanium manglings of the reference's signatures
// (obtained by compiling host declarations of them against its headers).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

extern "C" {
#include "emt6_oracle.h"
}

namespace {

// reference data layouts (parameters/parameters.h, site/site.h, common/grid.h,
// common/protocol.h)
struct RSubs { float cho, ox, gi; };
struct RDims { int16_t h, w; };
struct RParams {
  RDims dims;
  float time_step;
  RSubs dcoeffs;
  float dts;
  RSubs met[4];
  RSubs ext;
  float death_gi, quiescence_gi, death_gi_production;
  float ct[5][2];
  float dl_c, dl_e, sv_c, sv_e, rht;
};
static_assert(sizeof(RParams) == 156, "Parameters is 156 bytes");
struct RDiffusion { RSubs coeffs; float time_step; };
struct RSite {
  RSubs s;
  float tir, irr, delay, prolif;
  float times[5];
  uint8_t mode, phase, pad0[2];
  uint8_t state, pad1[3];
};
static_assert(sizeof(RSite) == 56, "Site is 56 bytes");
struct RGridView { RSite *data; RDims dims; int32_t pad; };
static_assert(sizeof(RGridView) == 16, "GridView<Site> is 16 bytes");
struct RProtocol { uint32_t res, length; float *data; };
static_assert(sizeof(RProtocol) == 16, "Protocol is 16 bytes");

const char *kPopulate =
    "_ZN6emt6ro6detail23populateGridViewsKernelEPNS_8GridViewINS_4SiteEEEjNS_4DimsEPS2_";
const char *kInitRng = "_ZN6emt6ro6detail15initializeStateEP17curandStateXORWOWjm";
const char *kFindOccupied = "_ZN6emt6ro6detail12findOccupiedEPNS_8GridViewINS_4SiteEEEPj";
const char *kFindRois =
    "_ZN6emt6ro14findROIsKernelEPNS_3ROIEPhPKNS_8GridViewINS_4SiteEEE";
const char *kDiffusion =
    "_ZN6emt6ro15diffusionKernelEPNS_8GridViewINS_4SiteEEEPKNS_3ROIEPKhNS_10Parameters9Diffusi"
    "onENS_10SubstratesEs";
const char *kCells =
    "_ZN6emt6ro6detail20cellSimulationKernelEPNS_8GridViewINS_4SiteEEEPjNS_10ParametersEP17cur"
    "andStateXORWOWPNS_8ProtocolEj";
const char *kCount = "_ZN6emt6ro6detail17countLivingKernelEPjPNS_4SiteEj";

// replicate tumour templates into every simulation (one block per simulation)
__global__ void expand_kernel(const RSite *tpl, const int32_t *sim_tumor, int hw, int64_t n,
                              RSite *data) {
  for (int64_t s = blockIdx.x; s < n; s += gridDim.x) {
    const RSite *src = tpl + (int64_t)sim_tumor[s] * hw;
    RSite *dst = data + s * hw;
    for (int q = threadIdx.x; q < hw; q += blockDim.x) dst[q] = src[q];
  }
}

struct Ref {
  CUmodule mod = nullptr;
  CUfunction k_populate, k_init, k_occ, k_rois, k_diff, k_cells, k_count;
  cudaStream_t stream = nullptr;
  RParams p;
  int H = 0, W = 0, HW = 0;
  int64_t n = 0;
  uint32_t step = 0;
  RSite *data = nullptr;
  RGridView *lattices = nullptr;
  RProtocol *protocols = nullptr;
  float *doses = nullptr;
  void *rois = nullptr;
  uint8_t *masks = nullptr;
  uint32_t *occupied = nullptr;
  void *rng = nullptr;
  uint32_t *results = nullptr;
  std::string err;
};

bool ok(Ref *r, CUresult e, const char *what) {
  if (e == CUDA_SUCCESS) return true;
  const char *s = nullptr;
  cuGetErrorString(e, &s);
  r->err = std::string(what) + ": " + (s ? s : "?");
  return false;
}

bool ok(Ref *r, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  r->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

bool launch(Ref *r, CUfunction f, unsigned gx, unsigned bx, unsigned by, unsigned smem,
            void **args, const char *what) {
  return ok(r, cuLaunchKernel(f, gx, 1, 1, bx, by, 1, smem, (CUstream)r->stream, args, nullptr),
            what);
}

}  // namespace

extern "C" {

const char *refgpu_error(void *h) { return h ? static_cast<Ref *>(h)->err.c_str() : "null"; }

// Returns a handle (check refgpu_error for failures: a non-empty message).
void *refgpu_create(const char *cubin, const orc_params *op, const orc_site *tumors, int n_tumors,
                    int H, int W, const int32_t *sim_tumor, const int32_t *sim_protocol,
                    const float *doses, int n_protocols, uint32_t bins, uint32_t res,
                    uint32_t length, int64_t n_sims, uint32_t seed) {
  Ref *r = new Ref();
  // the reference's kernels size their per-thread arrays for lattices of at
  // most 55 x 55 sites including the border (diffusion.cu:11-14)
  if (H < 3 || W < 3 || H > 53 || W > 53 || n_sims < 1 || n_tumors < 1 || n_protocols < 1 ||
      res == 0 || (uint64_t)bins * res < length) {
    r->err = "refgpu_create: unsupported sizes";
    return r;
  }
  for (int64_t i = 0; i < n_sims; ++i)
    if (sim_tumor[i] < 0 || sim_tumor[i] >= n_tumors || sim_protocol[i] < 0 ||
        sim_protocol[i] >= n_protocols) {
      r->err = "refgpu_create: simulation maps to a missing tumour or protocol";
      return r;
    }
  if (!ok(r, cudaFree(nullptr), "cudaFree(0)")) return r;
  if (!ok(r, cuModuleLoad(&r->mod, cubin), "cuModuleLoad")) return r;
  const char *names[7] = {kPopulate, kInitRng, kFindOccupied, kFindRois, kDiffusion, kCells, kCount};
  CUfunction *fns[7] = {&r->k_populate, &r->k_init,  &r->k_occ,  &r->k_rois,
                        &r->k_diff,     &r->k_cells, &r->k_count};
  for (int i = 0; i < 7; ++i)
    if (!ok(r, cuModuleGetFunction(fns[i], r->mod, names[i]), names[i])) return r;
  if (!ok(r, cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking), "stream")) return r;
  std::memset(&r->p, 0, sizeof(r->p));
  r->p.dims = {(int16_t)op->lattice_height, (int16_t)op->lattice_width};
  r->p.time_step = op->time_step;
  r->p.dcoeffs = {op->diffusion_coeffs[0], op->diffusion_coeffs[1], op->diffusion_coeffs[2]};
  r->p.dts = op->diffusion_time_step;
  for (int m = 0; m < 4; ++m)
    r->p.met[m] = {op->metabolism[m][0], op->metabolism[m][1], op->metabolism[m][2]};
  r->p.ext = {op->external_levels[0], op->external_levels[1], op->external_levels[2]};
  r->p.death_gi = op->death_gi;
  r->p.quiescence_gi = op->quiescence_gi;
  r->p.death_gi_production = op->death_gi_production;
  for (int i = 0; i < 5; ++i) {
    r->p.ct[i][0] = op->cycle_times[i][0];
    r->p.ct[i][1] = op->cycle_times[i][1];
  }
  r->p.dl_c = op->delay_time_coeff;
  r->p.dl_e = op->delay_time_exp_coeff;
  r->p.sv_c = op->survival_prob_coeff;
  r->p.sv_e = op->survival_prob_exp_coeff;
  r->p.rht = op->repair_half_time;
  r->H = H;
  r->W = W;
  r->HW = H * W;
  r->n = n_sims;
  const size_t hw = (size_t)r->HW, n = (size_t)n_sims;
  std::vector<RSite> tpl((size_t)n_tumors * hw);
  for (size_t k = 0; k < tpl.size(); ++k) {
    const orc_site &s = tumors[k];
    RSite &d = tpl[k];
    std::memset(&d, 0, sizeof(d));
    d.s = {s.cho, s.ox, s.gi};
    d.tir = s.time_in_repair;
    d.irr = s.irradiation;
    d.delay = s.repair_delay_time;
    d.prolif = s.proliferation_time;
    for (int i = 0; i < 5; ++i) d.times[i] = s.cycle_times[i];
    d.mode = s.mode;
    d.phase = s.phase;
    d.state = s.state;
  }
  RSite *dtpl = nullptr;
  int32_t *dst = nullptr;
  if (!ok(r, cudaMalloc(&dtpl, tpl.size() * sizeof(RSite)), "malloc tpl")) return r;
  if (!ok(r, cudaMalloc(&dst, n * 4), "malloc map")) return r;
  cudaMemcpy(dtpl, tpl.data(), tpl.size() * sizeof(RSite), cudaMemcpyHostToDevice);
  cudaMemcpy(dst, sim_tumor, n * 4, cudaMemcpyHostToDevice);
  if (!ok(r, cudaMalloc(&r->data, n * hw * sizeof(RSite)), "malloc data")) return r;
  expand_kernel<<<(unsigned)(n < 65535 ? n : 65535), 256, 0, r->stream>>>(dtpl, dst, r->HW, n_sims,
                                                                          r->data);
  if (!ok(r, cudaStreamSynchronize(r->stream), "expand")) return r;
  cudaFree(dtpl);
  cudaFree(dst);
  // buffers of Simulation's constructor (simulation.cu:123-137)
  if (!ok(r, cudaMalloc(&r->lattices, n * sizeof(RGridView)), "malloc lattices")) return r;
  if (!ok(r, cudaMalloc(&r->rois, n * 8), "malloc rois")) return r;
  if (!ok(r, cudaMalloc(&r->masks, n * hw), "malloc masks")) return r;
  if (!ok(r, cudaMalloc(&r->occupied, n * 1024 * 4), "malloc occupied")) return r;
  if (!ok(r, cudaMalloc(&r->rng, n * 512 * 48), "malloc rng")) return r;
  if (!ok(r, cudaMalloc(&r->results, n * 4), "malloc results")) return r;
  if (!ok(r, cudaMalloc(&r->doses, (size_t)n_protocols * bins * 4), "malloc doses")) return r;
  cudaMemcpy(r->doses, doses, (size_t)n_protocols * bins * 4, cudaMemcpyHostToDevice);
  std::vector<RProtocol> prots(n);
  for (size_t i = 0; i < n; ++i) prots[i] = {res, length, r->doses + (size_t)sim_protocol[i] * bins};
  if (!ok(r, cudaMalloc(&r->protocols, n * sizeof(RProtocol)), "malloc protocols")) return r;
  cudaMemcpy(r->protocols, prots.data(), n * sizeof(RProtocol), cudaMemcpyHostToDevice);
  {
    uint32_t bs = (uint32_t)n_sims;
    RDims dims = {(int16_t)H, (int16_t)W};
    void *args[] = {&r->lattices, &bs, &dims, &r->data};
    const unsigned blk = n_sims > 256 ? 256 : (unsigned)n_sims;
    if (!launch(r, r->k_populate, (unsigned)((n + 255) / 256), blk, 1, 0, args, "populate")) return r;
  }
  {
    size_t size = n * 512;
    void *args[] = {&r->rng, &seed, &size};
    if (!launch(r, r->k_init, (unsigned)((size + 255) / 256), 256, 1, 0, args, "init rng")) return r;
  }
  ok(r, cudaStreamSynchronize(r->stream), "init");
  return r;
}

void *refgpu_stream(void *h) { return static_cast<Ref *>(h)->stream; }

// Enqueues nsteps steps (Simulation::run); returns 0 or -1 (see refgpu_error).
int refgpu_run(void *h, uint32_t nsteps) {
  Ref *r = static_cast<Ref *>(h);
  const unsigned B = (unsigned)r->n;
  RDiffusion dp = {r->p.dcoeffs, r->p.dts};
  RSubs ext = r->p.ext;
  int16_t sub = (int16_t)(r->p.time_step / r->p.dts);
  const unsigned diff_smem = (unsigned)(12 * (r->H + 4) * (r->W + 4));
  for (uint32_t k = 0; k < nsteps; ++k) {
    if (r->step % 128 == 0) {
      void *a[] = {&r->lattices, &r->occupied};
      if (!launch(r, r->k_occ, B, 32, 1, 32 * 4, a, "findOccupied")) return -1;
    }
    if (r->step % 32 == 0) {
      void *a[] = {&r->rois, &r->masks, &r->lattices};
      if (!launch(r, r->k_rois, B, 16, 16, 64, a, "findROIs")) return -1;
    }
    {
      void *a[] = {&r->lattices, &r->rois, &r->masks, &dp, &ext, &sub};
      if (!launch(r, r->k_diff, B, 32, 32, diff_smem, a, "diffusion")) return -1;
    }
    {
      uint32_t step = r->step;
      void *a[] = {&r->lattices, &r->occupied, &r->p, &r->rng, &r->protocols, &step};
      if (!launch(r, r->k_cells, B, 512, 1, 128, a, "cellSimulation")) return -1;
    }
    r->step += 1;
  }
  return 0;
}

// Living counts (Simulation::getResults, simulation.cu:186-191).  Blocks.
int refgpu_counts(void *h, uint32_t *out) {
  Ref *r = static_cast<Ref *>(h);
  uint32_t vol = (uint32_t)r->HW;
  const unsigned blk = vol < 1024 ? vol : 1024;
  void *a[] = {&r->results, &r->data, &vol};
  if (!launch(r, r->k_count, (unsigned)r->n, blk, 1, blk * 4, a, "countLiving")) return -1;
  if (!ok(r, cudaMemcpyAsync(out, r->results, r->n * 4, cudaMemcpyDeviceToHost, r->stream),
          "copy")) return -1;
  return ok(r, cudaStreamSynchronize(r->stream), "sync") ? 0 : -1;
}

void refgpu_destroy(void *h) {
  Ref *r = static_cast<Ref *>(h);
  if (!r) return;
  if (r->stream) cudaStreamSynchronize(r->stream);
  cudaFree(r->data);
  cudaFree(r->lattices);
  cudaFree(r->protocols);
  cudaFree(r->doses);
  cudaFree(r->rois);
  cudaFree(r->masks);
  cudaFree(r->occupied);
  cudaFree(r->rng);
  cudaFree(r->results);
  if (r->stream) cudaStreamDestroy(r->stream);
  if (r->mod) cuModuleUnload(r->mod);
  delete r;
}

}  // extern "C"
