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
// refgpu_find_occupied / refgpu_find_rois / refgpu_diffuse launch one of
// those kernels alone on the current lattices, so tests can hold the oracle's
// restatement of each kernel to the reference's own output.
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

// One findOccupied launch (simulation.cu:41-64) on the current lattices.
// out: n x 1024 words per simulation, as the kernel leaves them: the count,
// then (row, column) int16 pairs in the kernel's order.  Blocks.
int refgpu_find_occupied(void *h, uint32_t *out) {
  Ref *r = static_cast<Ref *>(h);
  void *a[] = {&r->lattices, &r->occupied};
  if (!launch(r, r->k_occ, (unsigned)r->n, 32, 1, 32 * 4, a, "findOccupied")) return -1;
  if (!ok(r, cudaMemcpyAsync(out, r->occupied, (size_t)r->n * 1024 * 4, cudaMemcpyDeviceToHost,
                             r->stream), "copy occupied")) return -1;
  return ok(r, cudaStreamSynchronize(r->stream), "sync") ? 0 : -1;
}

// One findROIsKernel launch (diffusion.cu:101-108).  rois: n x 4 int16
// (origin row, origin column, height, width); masks: n x H*W bytes, the
// border mask of (height + 2) x (width + 2) at the start of each.  Blocks.
int refgpu_find_rois(void *h, int16_t *rois, uint8_t *masks) {
  Ref *r = static_cast<Ref *>(h);
  void *a[] = {&r->rois, &r->masks, &r->lattices};
  if (!launch(r, r->k_rois, (unsigned)r->n, 16, 16, 64, a, "findROIs")) return -1;
  if (!ok(r, cudaMemcpyAsync(rois, r->rois, (size_t)r->n * 8, cudaMemcpyDeviceToHost, r->stream),
          "copy rois")) return -1;
  if (!ok(r, cudaMemcpyAsync(masks, r->masks, (size_t)r->n * r->HW, cudaMemcpyDeviceToHost,
                             r->stream), "copy masks")) return -1;
  return ok(r, cudaStreamSynchronize(r->stream), "sync") ? 0 : -1;
}

// One diffusionKernel launch (diffusion.cu:135-191) with the ROIs and masks
// the last findROIsKernel left.  Blocks.
int refgpu_diffuse(void *h) {
  Ref *r = static_cast<Ref *>(h);
  RDiffusion dp = {r->p.dcoeffs, r->p.dts};
  RSubs ext = r->p.ext;
  int16_t sub = (int16_t)(r->p.time_step / r->p.dts);
  const unsigned diff_smem = (unsigned)(12 * (r->H + 4) * (r->W + 4));
  void *a[] = {&r->lattices, &r->rois, &r->masks, &dp, &ext, &sub};
  if (!launch(r, r->k_diff, (unsigned)r->n, 32, 32, diff_smem, a, "diffusion")) return -1;
  return ok(r, cudaStreamSynchronize(r->stream), "sync") ? 0 : -1;
}

// Substrate fields of every site: n x 3 x H*W floats (cho, ox, gi planes per
// simulation).  Blocks.
int refgpu_get_fields(void *h, float *out) {
  Ref *r = static_cast<Ref *>(h);
  const size_t hw = (size_t)r->HW;
  std::vector<RSite> host((size_t)r->n * hw);
  if (!ok(r, cudaMemcpyAsync(host.data(), r->data, host.size() * sizeof(RSite),
                             cudaMemcpyDeviceToHost, r->stream), "copy lattices")) return -1;
  if (!ok(r, cudaStreamSynchronize(r->stream), "sync")) return -1;
  for (size_t i = 0; i < (size_t)r->n; ++i)
    for (size_t q = 0; q < hw; ++q) {
      const RSite &x = host[i * hw + q];
      out[(i * 3 + 0) * hw + q] = x.s.cho;
      out[(i * 3 + 1) * hw + q] = x.s.ox;
      out[(i * 3 + 2) * hw + q] = x.s.gi;
    }
  return 0;
}

}  // extern "C"

// ---- the reference's cell model alone (emt6ro_ref_cell_sm103a.cubin) -------

namespace {

RSite to_rsite(const orc_site &s) {
  RSite d;
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
  return d;
}

void from_rsite(const RSite &d, orc_site *s) {
  s->cho = d.s.cho;
  s->ox = d.s.ox;
  s->gi = d.s.gi;
  s->time_in_repair = d.tir;
  s->irradiation = d.irr;
  s->repair_delay_time = d.delay;
  s->proliferation_time = d.prolif;
  for (int i = 0; i < 5; ++i) s->cycle_times[i] = d.times[i];
  s->mode = d.mode;
  s->phase = d.phase;
  s->state = d.state;
}

RParams to_rparams(const orc_params *op) {
  RParams p;
  std::memset(&p, 0, sizeof(p));
  p.dims = {(int16_t)op->lattice_height, (int16_t)op->lattice_width};
  p.time_step = op->time_step;
  p.dcoeffs = {op->diffusion_coeffs[0], op->diffusion_coeffs[1], op->diffusion_coeffs[2]};
  p.dts = op->diffusion_time_step;
  for (int m = 0; m < 4; ++m)
    p.met[m] = {op->metabolism[m][0], op->metabolism[m][1], op->metabolism[m][2]};
  p.ext = {op->external_levels[0], op->external_levels[1], op->external_levels[2]};
  p.death_gi = op->death_gi;
  p.quiescence_gi = op->quiescence_gi;
  p.death_gi_production = op->death_gi_production;
  for (int i = 0; i < 5; ++i) {
    p.ct[i][0] = op->cycle_times[i][0];
    p.ct[i][1] = op->cycle_times[i][1];
  }
  p.dl_c = op->delay_time_coeff;
  p.dl_e = op->delay_time_exp_coeff;
  p.sv_c = op->survival_prob_coeff;
  p.sv_e = op->survival_prob_exp_coeff;
  p.rht = op->repair_half_time;
  return p;
}

// device buffers of one call, freed on every exit path
struct Bufs {
  std::vector<void *> p;
  ~Bufs() {
    for (void *x : p) cudaFree(x);
  }
  template <typename T>
  T *get(size_t bytes, const void *src, std::string *err) {
    void *d = nullptr;
    cudaError_t e = cudaMalloc(&d, bytes ? bytes : 1);
    if (e == cudaSuccess && src) e = cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      *err = cudaGetErrorString(e);
      if (d) cudaFree(d);
      return nullptr;
    }
    p.push_back(d);
    return static_cast<T *>(d);
  }
};

thread_local std::string g_cell_err;

int cell_fail(const std::string &m) {
  g_cell_err = m;
  return -1;
}

bool cell_fn(const char *cubin, const char *name, CUmodule *mod, CUfunction *f) {
  if (cudaFree(nullptr) != cudaSuccess) return cell_fail("cudaFree(0)") == 0;
  if (cuModuleLoad(mod, cubin) != CUDA_SUCCESS) return cell_fail("cuModuleLoad") == 0;
  if (cuModuleGetFunction(f, *mod, name) != CUDA_SUCCESS) {
    cuModuleUnload(*mod);
    return cell_fail(name) == 0;
  }
  return true;
}

int cell_launch(CUmodule mod, CUfunction f, int64_t n, void **args) {
  const unsigned blocks = (unsigned)((n + 127) / 128);
  CUresult e = cuLaunchKernel(f, blocks, 1, 1, 128, 1, 1, 0, nullptr, args, nullptr);
  if (e == CUDA_SUCCESS) e = cuCtxSynchronize();
  if (e != CUDA_SUCCESS) {
    cuModuleUnload(mod);
    return cell_fail("launch");
  }
  return 0;
}

}  // namespace

extern "C" {

const char *refgpu_cell_error() { return g_cell_err.c_str(); }

// Site::step<R> of the reference's device build on n sites with injected
// draws (ndraw per site); sites are updated in place.  Returns 0 or -1.
int refgpu_site_step(const char *cubin, const orc_params *op, orc_site *sites,
                     const uint32_t *vac, const float *dose, const float *draws, int ndraw,
                     int32_t *ready, int32_t *used, int64_t n) {
  if (n < 1 || ndraw < 1) return cell_fail("bad sizes");
  CUmodule mod;
  CUfunction f;
  if (!cell_fn(cubin, "ref_site_step_kernel", &mod, &f)) return -1;
  std::vector<RSite> rs((size_t)n);
  for (int64_t i = 0; i < n; ++i) rs[i] = to_rsite(sites[i]);
  Bufs b;
  RSite *ds = b.get<RSite>(rs.size() * sizeof(RSite), rs.data(), &g_cell_err);
  uint32_t *dv = b.get<uint32_t>((size_t)n * 4, vac, &g_cell_err);
  float *dd = b.get<float>((size_t)n * 4, dose, &g_cell_err);
  float *dr = b.get<float>((size_t)n * ndraw * 4, draws, &g_cell_err);
  int32_t *dready = b.get<int32_t>((size_t)n * 4, nullptr, &g_cell_err);
  int32_t *dused = b.get<int32_t>((size_t)n * 4, nullptr, &g_cell_err);
  if (!ds || !dv || !dd || !dr || !dready || !dused) {
    cuModuleUnload(mod);
    return -1;
  }
  RParams p = to_rparams(op);
  void *args[] = {&ds, &p, &dv, &dd, &dr, &ndraw, &dready, &dused, &n};
  if (cell_launch(mod, f, n, args)) return -1;
  cudaMemcpy(rs.data(), ds, rs.size() * sizeof(RSite), cudaMemcpyDeviceToHost);
  cudaMemcpy(ready, dready, (size_t)n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(used, dused, (size_t)n * 4, cudaMemcpyDeviceToHost);
  for (int64_t i = 0; i < n; ++i) from_rsite(rs[i], &sites[i]);
  cuModuleUnload(mod);
  return 0;
}

// divideCell<R> of the reference's device build: parents updated in place,
// children's cells written (their substrates and state are zero).
int refgpu_divide(const char *cubin, const orc_params *op, orc_site *parents, const float *z,
                  orc_site *children, int64_t n) {
  if (n < 1) return cell_fail("bad sizes");
  CUmodule mod;
  CUfunction f;
  if (!cell_fn(cubin, "ref_divide_kernel", &mod, &f)) return -1;
  std::vector<RSite> rp((size_t)n), rc((size_t)n);
  for (int64_t i = 0; i < n; ++i) rp[i] = to_rsite(parents[i]);
  std::memset(rc.data(), 0, rc.size() * sizeof(RSite));
  Bufs b;
  RSite *dp = b.get<RSite>(rp.size() * sizeof(RSite), rp.data(), &g_cell_err);
  RSite *dc = b.get<RSite>(rc.size() * sizeof(RSite), rc.data(), &g_cell_err);
  float *dz = b.get<float>((size_t)n * 5 * 4, z, &g_cell_err);
  if (!dp || !dc || !dz) {
    cuModuleUnload(mod);
    return -1;
  }
  RParams p = to_rparams(op);
  void *args[] = {&dp, &dc, &p, &dz, &n};
  if (cell_launch(mod, f, n, args)) return -1;
  cudaMemcpy(rp.data(), dp, rp.size() * sizeof(RSite), cudaMemcpyDeviceToHost);
  cudaMemcpy(rc.data(), dc, rc.size() * sizeof(RSite), cudaMemcpyDeviceToHost);
  for (int64_t i = 0; i < n; ++i) {
    from_rsite(rp[i], &parents[i]);
    std::memset(&children[i], 0, sizeof(orc_site));
    from_rsite(rc[i], &children[i]);
  }
  cuModuleUnload(mod);
  return 0;
}

// chooseNeighbour<R> of the reference's device build for site (r, c).
int refgpu_choose(const char *cubin, const float *u, int r, int c, int32_t *rc, int64_t n) {
  if (n < 1) return cell_fail("bad sizes");
  CUmodule mod;
  CUfunction f;
  if (!cell_fn(cubin, "ref_choose_kernel", &mod, &f)) return -1;
  Bufs b;
  float *du = b.get<float>((size_t)n * 4, u, &g_cell_err);
  int32_t *drc = b.get<int32_t>((size_t)n * 8, nullptr, &g_cell_err);
  if (!du || !drc) {
    cuModuleUnload(mod);
    return -1;
  }
  void *args[] = {&du, &r, &c, &drc, &n};
  if (cell_launch(mod, f, n, args)) return -1;
  cudaMemcpy(rc, drc, (size_t)n * 8, cudaMemcpyDeviceToHost);
  cuModuleUnload(mod);
  return 0;
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
