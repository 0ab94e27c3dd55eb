// emt6_noalloc.cu -- a simulation entry point that allocates no device memory.
//
// emt6_simulate_noalloc serves callers that cannot call cudaMalloc: code
// embedded in a host application or framework whose allocator owns all device
// memory (a caching pool such as PyTorch's, where stray cudaMalloc calls
// fragment the pool or push it past its budget), or a plug-in whose host
// fixes every device allocation at start-up.  Such a caller hands over device
// buffers it already owns -- the initial lattices, the dose table, the
// simulation -> tumour/protocol maps and the output counts -- and the library
// keeps each simulation's working state (fields, site states, cell records,
// occupied list) in the file-scope array below, which every GPU that loads the
// library holds until the process exits.
//
// Limits and contract:
//   * kNoAllocBytes (8 MiB) of working state per device: a default 53 x 53
//     lattice takes about 177 KB per simulation, so one call runs at most 47
//     of them; larger requests are rejected with EMT6_ERR_LIMIT.
//   * The first call on a device (and the first one after the device's
//     context was re-created, e.g. by cudaDeviceReset) looks the array's
//     device address up with that device current; make that first call
//     before any stream capture.
//   * All calls share the one array and it keeps the last call's contents;
//     every call re-initialises the state it uses.  Calls that overlap on the
//     GPU (concurrent streams, or host threads racing on one device) race on
//     it: serialise them.
//   * The call enqueues its kernels on the given stream, then copies the
//     device error flag to the host and synchronises that stream, so it
//     returns only when the counts are written.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/emt6ro_gb300.h"
#include "emt6_kernels.h"

namespace {

constexpr size_t kNoAllocBytes = 8u << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_mu;
// per device: the scratch array's address and the id of the context it was
// looked up in (0 = not looked up yet)
void *g_scratch_addr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

int fail(int code, const std::string &msg);

// AoS sites of tumour sim_tumor[sim] -> the kernels' per-simulation layout;
// clears the per-simulation list, ROI and step counter
__global__ void noalloc_expand_kernel(const emt6_site *tumors, const int32_t *sim_tumor,
                                      int64_t n, int H, int W, uint32_t fstride, uint32_t sstride,
                                      float *fld, uint8_t *st, float4 *cell, int4 *meta,
                                      int32_t *roi, uint32_t *step, uint32_t *err) {
  for (int64_t sim = blockIdx.x; sim < n; sim += gridDim.x) {
    const int HW = H * W;
    const emt6_site *src = tumors + (int64_t)sim_tumor[sim] * HW;
    float *f = fld + sim * fstride;
    uint8_t *s = st + sim * sstride;
    float4 *c = cell + sim * (int64_t)HW * 3;
    for (int q = threadIdx.x; q < HW; q += blockDim.x) {
      const emt6_site x = src[q];
      const int r = q / W, col = q - (q / W) * W;
      uint8_t state = x.state & 3;
      if ((r == 0 || col == 0 || r == H - 1 || col == W - 1) && state == 1) {
        // a cell on the border ring would make the kernels read outside the
        // lattice: refuse it (the site is neutralised so nothing runs off it)
        atomicOr(err, 8u);
        state = 2;
      }
      f[q] = x.cho;
      f[HW + q] = x.ox;
      f[2 * HW + q] = x.gi;
      s[q] = state;
      c[3 * q] = make_float4(x.proliferation_time, x.time_in_repair, x.irradiation,
                             x.repair_delay_time);
      c[3 * q + 1] = make_float4(x.cycle_times[0], x.cycle_times[1], x.cycle_times[2],
                                 x.cycle_times[3]);
      c[3 * q + 2] = make_float4(x.cycle_times[4],
                                 __uint_as_float((uint32_t)x.mode | ((uint32_t)x.phase << 8)),
                                 0.f, 0.f);
    }
    for (uint32_t q = 3 * HW + threadIdx.x; q < fstride; q += blockDim.x) f[q] = 0.f;
    for (uint32_t q = HW + threadIdx.x; q < sstride; q += blockDim.x) s[q] = 0;
    if (threadIdx.x == 0) {
      meta[sim] = make_int4(0, 0, 0, 0);
      for (int k = 0; k < 8; ++k) roi[sim * 8 + k] = 0;
      step[sim] = 0;
    }
  }
}

__global__ void noalloc_count_kernel(const uint8_t *st, uint32_t sstride, int HW,
                                     uint32_t *counts, int64_t n) {
  for (int64_t sim = blockIdx.x; sim < n; sim += gridDim.x) {
    const uint8_t *s = st + sim * sstride;
    int c = 0;
    for (int q = threadIdx.x; q < HW; q += blockDim.x) c += (s[q] & 3) == 1;
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ int part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
      counts[sim] = (uint32_t)t;
    }
    __syncthreads();
  }
}

// Id of the context current on this thread (0 when there is none or the
// driver does not report ids).  Context ids are unique for the life of the
// process, so a re-created context never matches an old one.
unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the scratch array on the current device.  The set-up
// (cudaGetSymbolAddress with the device current) runs once per device and
// again whenever the device's context has been re-created since, because the
// module, and with it the array, may then sit at another address.
int scratch_address(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return fail(EMT6_ERR_INVALID, "device id too large");
  std::lock_guard<std::mutex> lk(g_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_scratch_addr[device] || ctx == 0 || ctx != g_scratch_ctx[device]) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(EMT6_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_addr[device] = ptr;
    // the lookup made the device's context current on this thread
    g_scratch_ctx[device] = current_context_id();
  }
  *out = static_cast<unsigned char *>(g_scratch_addr[device]);
  return EMT6_OK;
}

}  // namespace

namespace emt6 {
// defined in emt6_host.cu: the model constants and the emt6_last_error message
KParams make_kparams_public(const emt6_params &p, uint64_t seed, uint32_t res, uint32_t length,
                            uint32_t bins);
int set_error(int code, const std::string &msg);
}  // namespace emt6

namespace {
int fail(int code, const std::string &msg) { return emt6::set_error(code, msg); }
}  // namespace

extern "C" {

int emt6_simulate_noalloc(const emt6_params *p, const emt6_site *d_tumors, int32_t height,
                          int32_t width, const int32_t *d_sim_tumor,
                          const int32_t *d_sim_protocol, int64_t n_sims, const float *d_doses,
                          uint32_t protocol_bins, uint32_t protocol_resolution,
                          uint32_t protocol_length, uint32_t nsteps, uint64_t seed,
                          uint32_t *d_counts, void *stream) {
  if (!p || !d_tumors || !d_sim_tumor || !d_sim_protocol || !d_doses || !d_counts)
    return fail(EMT6_ERR_INVALID, "null argument");
  if (n_sims < 1) return fail(EMT6_ERR_INVALID, "n_sims must be positive");
  if (protocol_resolution == 0) return fail(EMT6_ERR_INVALID, "protocol_resolution must be > 0");
  if (p->lattice_height < 1 || p->lattice_width < 1 ||
      p->lattice_height > EMT6_MAX_INTERIOR_HEIGHT || p->lattice_width > EMT6_MAX_INTERIOR_WIDTH)
    return fail(EMT6_ERR_LIMIT, "lattice_dims outside 1..54 x 1..60");
  if (height != p->lattice_height + 2 || width != p->lattice_width + 2)
    return fail(EMT6_ERR_INVALID, "tumour dims do not match lattice_dims + 2");
  if (!(p->time_step > 0) || !(p->diffusion_time_step > 0))
    return fail(EMT6_ERR_INVALID, "time steps must be positive");
  const emt6::KParams kp =
      emt6::make_kparams_public(*p, seed, protocol_resolution, protocol_length, protocol_bins);
  const int HW = kp.HW;
  const uint32_t fstride = (uint32_t)((3 * HW + 31) / 32 * 32);
  const uint32_t sstride = (uint32_t)((HW + 127) / 128 * 128);
  const uint32_t lstride = (uint32_t)((kp.lcap + 63) / 64 * 64);
  const size_t n = (size_t)n_sims;
  // carve the scratch array: header (error flag, ticket, counter), then
  // per-simulation arrays
  size_t off = 0;
  const size_t o_err = off; off += 256;
  const size_t o_fld = off; off = align256(off + n * fstride * sizeof(float));
  const size_t o_st = off; off = align256(off + n * sstride);
  const size_t o_cell = off; off = align256(off + n * (size_t)HW * 3 * sizeof(float4));
  const size_t o_list = off; off = align256(off + n * lstride * sizeof(uint16_t));
  const size_t o_meta = off; off = align256(off + n * sizeof(int4));
  const size_t o_roi = off; off = align256(off + n * 8 * sizeof(int32_t));
  const size_t o_step = off; off = align256(off + n * sizeof(uint32_t));
  if (off > kNoAllocBytes) {
    const size_t per = (off - 256) / n;
    return fail(EMT6_ERR_LIMIT,
                std::to_string(n_sims) + " simulations need " + std::to_string(off) +
                    " bytes of working state; the allocation-free entry point holds " +
                    std::to_string(kNoAllocBytes) + " bytes (at most " +
                    std::to_string((kNoAllocBytes - 256) / per) +
                    " simulations of this lattice size per call)");
  }
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return fail(EMT6_ERR_CUDA, cudaGetErrorString(e));
  unsigned char *base = nullptr;
  int rc = scratch_address(device, &base);
  if (rc) return rc;
  uint32_t *err = reinterpret_cast<uint32_t *>(base + o_err);
  uint32_t *ticket = err + 1;
  unsigned long long *diffused = reinterpret_cast<unsigned long long *>(base + o_err + 8);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  emt6::RunArgs a;
  a.p = kp;
  a.fld = reinterpret_cast<float *>(base + o_fld);
  a.st = base + o_st;
  a.cell = reinterpret_cast<float4 *>(base + o_cell);
  a.list = reinterpret_cast<uint16_t *>(base + o_list);
  a.meta = reinterpret_cast<int4 *>(base + o_meta);
  a.roi = reinterpret_cast<int32_t *>(base + o_roi);
  a.step = reinterpret_cast<uint32_t *>(base + o_step);
  a.horizon = nullptr;
  a.sim_protocol = d_sim_protocol;
  a.doses = d_doses;
  a.counts = d_counts;
  a.err = err;
  a.diffused = diffused;
  a.fstride = fstride;
  a.sstride = sstride;
  a.lstride = lstride;
  a.epoch = 0;
  a.nsims = n_sims;
  a.queue = 0;
  a.ticket = ticket;
  a.order = nullptr;

  // the header (error flag, ticket, counter) must start at zero
  e = cudaMemsetAsync(base + o_err, 0, 256, s);
  if (e != cudaSuccess) return fail(EMT6_ERR_CUDA, cudaGetErrorString(e));
  const int grid = (int)(n_sims < 65535 ? n_sims : 65535);
  noalloc_expand_kernel<<<grid, 256, 0, s>>>(d_tumors, d_sim_tumor, n_sims, height, width,
                                              fstride, sstride,
                                              a.fld, a.st, a.cell, a.meta, a.roi, a.step, err);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(EMT6_ERR_CUDA, cudaGetErrorString(e));
  for (uint32_t t = 0; t < nsteps;) {
    const uint32_t end = nsteps - t > 1200 ? t + 1200 : nsteps;
    for (int wide = 0; wide < 2; ++wide) {
      e = emt6::launch_run(a, end, wide != 0, (int)n_sims, s);
      if (e != cudaSuccess) return fail(EMT6_ERR_CUDA, cudaGetErrorString(e));
    }
    t = end;
  }
  noalloc_count_kernel<<<grid, 256, 0, s>>>(a.st, sstride, HW, d_counts, n_sims);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(EMT6_ERR_CUDA, cudaGetErrorString(e));
  uint32_t herr = 0;
  e = cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(EMT6_ERR_CUDA, cudaGetErrorString(e));
  if (herr & 8u) return fail(EMT6_ERR_INVALID, "occupied site on the border ring of a tumour");
  if (herr) return fail(EMT6_ERR_DEVICE, "device error flag " + std::to_string(herr));
  return EMT6_OK;
}

}  // extern "C"
