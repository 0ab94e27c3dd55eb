// emt6_host.cu -- host engine and C ABI of the GB300 EMT6-Ro simulator.
//
// Replaces, on the host side, the reference's Simulation class
// (src/emt6ro/simulation/simulation.{h,cu}), its pybind11 Experiment
// (python/emt6ro/simulation/backend.cc:16-136), the JSON parameter loader
// (src/emt6ro/parameters/parameters.cc:66-80) and the tumour text format
// (src/emt6ro/state/state.cc).  All device memory is owned by the handles;
// work is issued on one CUDA stream per handle.  Compiled with
// -ffp-contract=off so the model constants derived here round exactly as the
// reference's expressions do.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/emt6ro_gb300.h"
#include "emt6_kernels.h"

using emt6::KParams;
using emt6::kLayoutAll;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

#define EMT6_CUDA(call)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(EMT6_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

// exp for the model constants derived on the host (same evaluation as the
// kernels' exp_core: Cody-Waite reduction + degree-13 Taylor, in double)
double host_exp_core(double x) {
  double k = std::rint(x * 0x1.71547652b82fep+0);
  double r = std::fma(-k, 0x1.62e42fefa39efp-1, x);
  r = std::fma(-k, 0x1.abc9e3b39803fp-56, r);
  static const double c[] = {0x1.6124613a86d09p-33, 0x1.1eed8eff8d898p-29, 0x1.ae64567f544e4p-26,
                             0x1.27e4fb7789f5cp-22, 0x1.71de3a556c734p-19, 0x1.a01a01a01a01ap-16,
                             0x1.a01a01a01a01ap-13, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7,
                             0x1.5555555555555p-5,  0x1.5555555555555p-3,  0x1.0000000000000p-1,
                             1.0,                   1.0};
  double q = c[0];
  for (int i = 1; i < 14; ++i) q = std::fma(q, r, c[i]);
  uint64_t bits = (uint64_t)((int64_t)k + 1023) << 52;
  double s;
  std::memcpy(&s, &bits, 8);
  return q * s;
}

float host_calc_delay(float irr, const emt6_params &p) {
  return p.delay_time_coeff * (float)host_exp_core((double)(p.delay_time_exp_coeff * irr));
}

int check_params(const emt6_params *p) {
  if (!p) return fail(EMT6_ERR_INVALID, "null parameters");
  if (p->lattice_height < 1 || p->lattice_width < 1)
    return fail(EMT6_ERR_INVALID, "lattice_dims must be positive");
  if (p->lattice_height > EMT6_MAX_INTERIOR_HEIGHT || p->lattice_width > EMT6_MAX_INTERIOR_WIDTH)
    return fail(EMT6_ERR_LIMIT, "lattice_dims " + std::to_string(p->lattice_height) + "x" +
                                    std::to_string(p->lattice_width) + " exceed the supported " +
                                    std::to_string(EMT6_MAX_INTERIOR_HEIGHT) + "x" +
                                    std::to_string(EMT6_MAX_INTERIOR_WIDTH));
  if (!(p->diffusion_time_step > 0) || !(p->time_step > 0))
    return fail(EMT6_ERR_INVALID, "time steps must be positive");
  return EMT6_OK;
}

KParams make_kparams(const emt6_params &p, uint64_t seed, uint32_t res, uint32_t length,
                     uint32_t bins) {
  KParams k;
  std::memset(&k, 0, sizeof(k));
  k.H = p.lattice_height + 2;
  k.W = p.lattice_width + 2;
  k.HW = k.H * k.W;
  k.lcap = p.lattice_height * p.lattice_width + 256;
  k.dt_h = p.time_step / 3600.f;          // cell.cu:25,73; cell.h:106
  k.dt2_h = (2 * p.time_step) / 3600.f;   // cell.cu:68
  for (int m = 0; m < 4; ++m)
    for (int f = 0; f < 3; ++f) k.met[m][f] = p.metabolism[m][f];
  for (int f = 0; f < 3; ++f) k.ext[f] = p.external_levels[f];
  k.death_gi = p.death_gi;
  k.quiescence_gi = p.quiescence_gi;
  for (int i = 0; i < 5; ++i) {
    k.ct_mean[i] = p.cycle_times[i][0];
    k.ct_sd[i] = p.cycle_times[i][1];
  }
  k.dl_c = p.delay_time_coeff;
  k.dl_e = p.delay_time_exp_coeff;
  k.sv_c = p.survival_prob_coeff;
  k.sv_e = p.survival_prob_exp_coeff;
  k.rht = p.repair_half_time;
  // diffusion.cu:119-120 and :163: k = coeffs * dt * 2sqrt2 / (4 + 2sqrt2)
  const float HS = (float)(2 * 1.41421356237309504880);
  const float F = (float)(4. + (double)HS);
  const float S2 = (float)0.70710678118654752440;
  for (int f = 0; f < 3; ++f) {
    const float kk = ((p.diffusion_coeffs[f] * p.diffusion_time_step) * HS) / F;
    k.da[f] = (float)(1.0 - (double)kk * (double)F);
    k.db[f] = kk;
    k.dd[f] = (float)((double)kk * (double)S2);
  }
  const int nsub = (int16_t)(p.time_step / p.diffusion_time_step);  // simulation.cu:170
  k.nfree = nsub - 1 > 0 ? nsub - 1 : 0;
  k.seed_lo = (uint32_t)seed;
  k.seed_hi = (uint32_t)(seed >> 32);
  k.res = res;
  k.length = length;
  k.bins = bins;
  k.layouts = kLayoutAll;
  return k;
}

// ---- minimal JSON reader (objects, numbers, strings, arrays, literals) ----
struct JVal {
  enum { NUM, STR, OBJ, ARR, LIT } kind = LIT;
  double num = 0;
  std::string str;
  std::map<std::string, JVal> obj;
  std::vector<JVal> arr;
};

struct JParser {
  const std::string &s;
  size_t i = 0;
  explicit JParser(const std::string &src) : s(src) {}
  void ws() {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
  }
  bool parse(JVal &v) {
    ws();
    if (i >= s.size()) return false;
    char c = s[i];
    if (c == '{') {
      v.kind = JVal::OBJ;
      ++i;
      ws();
      if (i < s.size() && s[i] == '}') { ++i; return true; }
      for (;;) {
        ws();
        JVal key;
        if (!parse(key) || key.kind != JVal::STR) return false;
        ws();
        if (i >= s.size() || s[i] != ':') return false;
        ++i;
        JVal val;
        if (!parse(val)) return false;
        v.obj[key.str] = std::move(val);
        ws();
        if (i < s.size() && s[i] == ',') { ++i; continue; }
        if (i < s.size() && s[i] == '}') { ++i; return true; }
        return false;
      }
    }
    if (c == '[') {
      v.kind = JVal::ARR;
      ++i;
      ws();
      if (i < s.size() && s[i] == ']') { ++i; return true; }
      for (;;) {
        JVal val;
        if (!parse(val)) return false;
        v.arr.push_back(std::move(val));
        ws();
        if (i < s.size() && s[i] == ',') { ++i; continue; }
        if (i < s.size() && s[i] == ']') { ++i; return true; }
        return false;
      }
    }
    if (c == '"') {
      v.kind = JVal::STR;
      ++i;
      while (i < s.size() && s[i] != '"') {
        if (s[i] == '\\' && i + 1 < s.size()) ++i;
        v.str += s[i++];
      }
      if (i >= s.size()) return false;
      ++i;
      return true;
    }
    if (c == '-' || c == '+' || c == '.' || std::isdigit((unsigned char)c)) {
      size_t j = i;
      while (j < s.size() && (std::isdigit((unsigned char)s[j]) || s[j] == '-' || s[j] == '+' ||
                              s[j] == '.' || s[j] == 'e' || s[j] == 'E'))
        ++j;
      v.kind = JVal::NUM;
      v.str = s.substr(i, j - i);
      char *end = nullptr;
      v.num = std::strtod(v.str.c_str(), &end);
      i = j;
      return true;
    }
    for (const char *lit : {"true", "false", "null"}) {
      size_t n = std::strlen(lit);
      if (s.compare(i, n, lit) == 0) {
        v.kind = JVal::LIT;
        v.str = lit;
        i += n;
        return true;
      }
    }
    return false;
  }
};

struct JsonMissing {
  std::string key;
};

const JVal &jget(const JVal &o, const char *key) {
  if (o.kind != JVal::OBJ) throw JsonMissing{key};
  auto it = o.obj.find(key);
  if (it == o.obj.end()) throw JsonMissing{key};
  return it->second;
}

// The reference reads every number with nlohmann's get<float>() (a double
// parsed from the text, then converted), parameters.cc:27-64.
float jf(const JVal &o, const char *key) {
  const JVal &v = jget(o, key);
  if (v.kind != JVal::NUM) throw JsonMissing{key};
  return (float)v.num;
}

void jsub(const JVal &o, float out[3]) {
  out[0] = jf(o, "cho");
  out[1] = jf(o, "ox");
  out[2] = jf(o, "gi");
}

// ---- engine ------------------------------------------------------------------
template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    n = count;
    return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

struct emt6_batch {
  std::mutex mu;
  int device = 0;
  cudaStream_t stream = nullptr;
  emt6_params params{};
  KParams kp{};
  int H = 0, W = 0, HW = 0;
  int64_t n = 0;
  int32_t T = 0, P = 0;
  uint32_t bins = 0, res = 0, length = 0;
  uint32_t fstride = 0, sstride = 0, lstride = 0;
  uint32_t epoch = 0;
  uint32_t t_host = 0;  // common step counter of the batch (simulations stop at their horizon)
  uint64_t seed = 0;
  int sched = 0;
  uint32_t chunk = 1200;
  unsigned long long launches = 0;  // kernels issued by this handle
  bool use_graph = false;
  bool occ_known = false;
  int per_sm_cache[2] = {1, 1};
  cudaGraphExec_t graph_exec = nullptr;
  uint64_t graph_key[5] = {0, 0, 0, 0, 0};
  unsigned long long graph_kernels = 0;
  bool has_horizon = false;
  uint32_t max_horizon = 0xFFFFFFFFu;
  DevBuf<float> fld, tpl_fld, doses;
  DevBuf<uint8_t> st, tpl_st;
  DevBuf<float4> cell, tpl_cell;
  DevBuf<uint16_t> list;
  DevBuf<int4> meta;
  DevBuf<int32_t> roi, sim_tumor, sim_protocol;
  DevBuf<uint32_t> step, horizon, counts, err, ticket, order_hist;
  DevBuf<int64_t> order;  // per chunk: simulations by region, largest first
  DevBuf<unsigned long long> diffused;
  std::vector<float> h_doses;

  ~emt6_batch() {
    if (stream) {
      DeviceGuard g(device);
      cudaStreamSynchronize(stream);
      if (graph_exec) cudaGraphExecDestroy(graph_exec);
      cudaStreamDestroy(stream);
    }
  }

  emt6::RunArgs run_args() {
    emt6::RunArgs a;
    a.p = kp;
    a.fld = fld.p;
    a.st = st.p;
    a.cell = cell.p;
    a.list = list.p;
    a.meta = meta.p;
    a.roi = roi.p;
    a.step = step.p;
    a.horizon = has_horizon ? horizon.p : nullptr;
    a.sim_protocol = sim_protocol.p;
    a.doses = doses.p;
    a.counts = counts.p;
    a.err = err.p;
    a.diffused = diffused.p;
    a.fstride = fstride;
    a.sstride = sstride;
    a.lstride = lstride;
    a.epoch = epoch;
    a.nsims = n;
    a.queue = 0;
    a.ticket = ticket.p;
    a.order = order.p;
    return a;
  }

  int check_err() {
    uint32_t e = 0;
    EMT6_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(e), cudaMemcpyDeviceToHost, stream));
    EMT6_CUDA(cudaStreamSynchronize(stream));
    if (e)
      return fail(EMT6_ERR_DEVICE,
                  "device error flag " + std::to_string(e) +
                      " (1: occupied-list overflow, 4: occurrence index overflow)");
    return EMT6_OK;
  }

  int upload_doses() {
    EMT6_CUDA(cudaMemcpyAsync(doses.p, h_doses.data(), h_doses.size() * sizeof(float),
                              cudaMemcpyHostToDevice, stream));
    // the host vector may change before the copy runs: wait for it
    EMT6_CUDA(cudaStreamSynchronize(stream));
    return EMT6_OK;
  }

  int reset() {
    emt6::ResetArgs r;
    r.fld = fld.p;
    r.st = st.p;
    r.cell = cell.p;
    r.meta = meta.p;
    r.roi = roi.p;
    r.step = step.p;
    r.tpl_fld = tpl_fld.p;
    r.tpl_st = tpl_st.p;
    r.tpl_cell = tpl_cell.p;
    r.sim_tumor = sim_tumor.p;
    r.fstride = fstride;
    r.sstride = sstride;
    r.HW = HW;
    r.nsims = n;
    EMT6_CUDA(emt6::launch_reset(r, stream));
    launches += 1;
    std::fill(h_doses.begin(), h_doses.end(), 0.f);
    int rc = upload_doses();
    if (rc) return rc;
    t_host = 0;
    epoch += 1;
    return EMT6_OK;
  }

  // launches of one run() call from t_host to target, on the handle's stream
  int issue(uint32_t target, unsigned long long *count) {
    emt6::RunArgs a = run_args();
    int sms = 0;
    EMT6_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    if (!occ_known) {
      for (int wide = 0; wide < 2; ++wide)
        per_sm_cache[wide] = std::max(emt6::max_ctas_per_sm(kp, wide != 0), 1);
      occ_known = true;
    }
    const int *per_sm = per_sm_cache;
    uint32_t t = t_host;
    while (t < target) {
      const uint32_t end = (uint32_t)std::min<uint64_t>(target, (uint64_t)t + chunk);
      if (has_horizon && t >= max_horizon) break;
      EMT6_CUDA(emt6::launch_order(a, end, order_hist.p, order.p, stream));
      *count += 3;
      for (int wide = 0; wide < 2; ++wide) {
        int grid = (int)std::min<int64_t>(n, 0x7fffffff);
        if (sched == 1) {
          grid = (int)std::min<int64_t>(n, (int64_t)per_sm[wide] * sms);
          EMT6_CUDA(cudaMemsetAsync(ticket.p, 0, sizeof(uint32_t), stream));
          a.queue = 1;
        }
        EMT6_CUDA(emt6::launch_run(a, end, wide != 0, grid, stream));
        *count += 1;
      }
      t = end;
    }
    return EMT6_OK;
  }

  int run(uint32_t nsteps) {
    const uint64_t target64 = (uint64_t)t_host + nsteps;
    const uint32_t target = target64 > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)target64;
    if (!use_graph) {
      int rc = issue(target, &launches);
      if (rc) return rc;
      t_host = target;
      return EMT6_OK;
    }
    // CUDA-graph mode: capture the whole chunk sequence once per
    // (start, target, schedule, chunk, epoch) and replay it
    const uint64_t key[5] = {t_host, target, (uint64_t)sched, chunk, epoch};
    if (!graph_exec || std::memcmp(key, graph_key, sizeof(key)) != 0) {
      if (graph_exec) {
        cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
      }
      // occupancy queries and attributes outside the capture
      if (!occ_known) {
        for (int wide = 0; wide < 2; ++wide)
          per_sm_cache[wide] = std::max(emt6::max_ctas_per_sm(kp, wide != 0), 1);
        occ_known = true;
      }
      EMT6_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      unsigned long long nodes = 0;
      int rc = issue(target, &nodes);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(stream, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (e != cudaSuccess) return fail(EMT6_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
      e = cudaGraphInstantiate(&graph_exec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return fail(EMT6_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
      std::memcpy(graph_key, key, sizeof(key));
      graph_kernels = nodes;
    }
    EMT6_CUDA(cudaGraphLaunch(graph_exec, stream));
    launches += graph_kernels;
    t_host = target;
    return EMT6_OK;
  }
};

struct emt6_experiment {
  emt6_batch *b = nullptr;
  int32_t runs = 0, protocols = 0, tumors = 0;
  bool running = false;
  ~emt6_experiment() { delete b; }
};

namespace {

__global__ void count_kernel(const uint8_t *st, uint32_t sstride, int HW, uint32_t *counts,
                             int64_t n) {
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

// Per simulation, 13 floats: cho, ox, gi at the centre site (H/2, W/2), the
// living count, occupied sites per metabolic mode (4) and per cycle phase (5)
// (the quantities example/timelapse.cc records, computed on the device).
__global__ void summary_kernel(const float *fld, uint32_t fstride, const uint8_t *st,
                               uint32_t sstride, const float4 *cell, int H, int W, float *out,
                               int64_t n) {
  __shared__ int part[8][10];
  const int HW = H * W, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t sim = blockIdx.x; sim < n; sim += gridDim.x) {
    const uint8_t *s = st + sim * sstride;
    const float4 *c = cell + sim * (int64_t)HW * 3;
    int cnt[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = threadIdx.x; q < HW; q += blockDim.x) {
      if ((s[q] & 3) != 1) continue;
      const uint32_t mp = __float_as_uint(c[3 * q + 2].y);
      cnt[0] += 1;
      cnt[1 + (mp & 3)] += 1;
      cnt[5 + min((int)((mp >> 8) & 0xff), 4)] += 1;
    }
#pragma unroll
    for (int k = 0; k < 10; ++k)
      for (int o = 16; o; o >>= 1) cnt[k] += __shfl_xor_sync(0xffffffffu, cnt[k], o);
    if (lane == 0)
      for (int k = 0; k < 10; ++k) part[wid][k] = cnt[k];
    __syncthreads();
    if (threadIdx.x < 10) {
      int t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w][threadIdx.x];
      out[sim * 13 + 3 + threadIdx.x] = (float)t;
    } else if (threadIdx.x < 13) {
      const int f = threadIdx.x - 10;
      out[sim * 13 + f] = fld[sim * fstride + (int64_t)f * HW + (H / 2) * W + W / 2];
    }
    __syncthreads();
  }
}

void site_to_records(const emt6_site &s, float *fld3, uint8_t *stv, float4 *cell3) {
  fld3[0] = s.cho;
  fld3[1] = s.ox;
  fld3[2] = s.gi;
  *stv = s.state & 3;
  uint32_t mp = (uint32_t)s.mode | ((uint32_t)s.phase << 8);
  float mpf;
  std::memcpy(&mpf, &mp, 4);
  cell3[0] = make_float4(s.proliferation_time, s.time_in_repair, s.irradiation,
                         s.repair_delay_time);
  cell3[1] = make_float4(s.cycle_times[0], s.cycle_times[1], s.cycle_times[2], s.cycle_times[3]);
  cell3[2] = make_float4(s.cycle_times[4], mpf, 0.f, 0.f);
}

void records_to_site(float cho, float ox, float gi, uint8_t stv, const float4 *c, emt6_site &s) {
  std::memset(&s, 0, sizeof(s));
  s.cho = cho;
  s.ox = ox;
  s.gi = gi;
  s.proliferation_time = c[0].x;
  s.time_in_repair = c[0].y;
  s.irradiation = c[0].z;
  s.repair_delay_time = c[0].w;
  s.cycle_times[0] = c[1].x;
  s.cycle_times[1] = c[1].y;
  s.cycle_times[2] = c[1].z;
  s.cycle_times[3] = c[1].w;
  s.cycle_times[4] = c[2].x;
  uint32_t mp;
  std::memcpy(&mp, &c[2].y, 4);
  s.mode = (uint8_t)(mp & 0xff);
  s.phase = (uint8_t)((mp >> 8) & 0xff);
  s.state = stv & 3;
}

}  // namespace

extern "C" {

const char *emt6_last_error(void) { return g_err.c_str(); }
int emt6_version(void) { return 1; }

// ---- file formats ----------------------------------------------------------------
int emt6_load_parameters(const char *path, emt6_params *out) {
  if (!path || !out) return fail(EMT6_ERR_INVALID, "null argument");
  std::ifstream f(path);
  if (!f.good()) return fail(EMT6_ERR_IO, std::string("Could not open the file: ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  std::string text = ss.str();
  JVal root;
  JParser jp(text);
  if (!jp.parse(root) || root.kind != JVal::OBJ)
    return fail(EMT6_ERR_IO, std::string("malformed JSON: ") + path);
  try {
    emt6_params p;
    std::memset(&p, 0, sizeof(p));
    const JVal &dims = jget(root, "lattice_dims");
    p.lattice_height = (int16_t)jget(dims, "height").num;  // parameters.cc:16-18 (int16_t)
    p.lattice_width = (int16_t)jget(dims, "width").num;
    p.time_step = jf(root, "time_step");
    const JVal &dp = jget(root, "diffusion_params");
    jsub(jget(dp, "coeffs"), p.diffusion_coeffs);
    p.diffusion_time_step = jf(dp, "time_step");
    const JVal &met = jget(root, "metabolism");
    jsub(jget(met, "aerobic_proliferation"), p.metabolism[0]);
    jsub(jget(met, "anaerobic_proliferation"), p.metabolism[1]);
    jsub(jget(met, "aerobic_quiescence"), p.metabolism[2]);
    jsub(jget(met, "anaerobic_quiescence"), p.metabolism[3]);
    jsub(jget(root, "external_levels"), p.external_levels);
    p.death_gi = jf(root, "death_gi");
    p.quiescence_gi = jf(root, "quiescence_gi");
    p.death_gi_production = jf(root, "death_gi_production");
    const JVal &ct = jget(root, "cycle_times");
    const char *names[5] = {"g1", "s", "g2", "m", "d"};
    for (int i = 0; i < 5; ++i) {
      p.cycle_times[i][0] = jf(jget(ct, names[i]), "mean");
      p.cycle_times[i][1] = jf(jget(ct, names[i]), "stddev");
    }
    const JVal &cr = jget(root, "cell_repair");
    p.delay_time_coeff = jf(jget(cr, "delay_time"), "coeff");
    p.delay_time_exp_coeff = jf(jget(cr, "delay_time"), "exp_coeff");
    p.survival_prob_coeff = jf(jget(cr, "survival_prob"), "coeff");
    p.survival_prob_exp_coeff = jf(jget(cr, "survival_prob"), "exp_coeff");
    p.repair_half_time = jf(cr, "repair_half_time");
    *out = p;
  } catch (const JsonMissing &m) {
    return fail(EMT6_ERR_IO, "missing or non-numeric key '" + m.key + "' in " + path);
  }
  return EMT6_OK;
}

int emt6_load_state(const char *path, const emt6_params *p, emt6_site *out, int32_t cap,
                    int32_t *height, int32_t *width) {
  if (!path || !p || !height || !width) return fail(EMT6_ERR_INVALID, "null argument");
  std::ifstream file(path);
  if (!file.good()) return fail(EMT6_ERR_IO, std::string("Could not open the file: ") + path);
  int16_t h = 0, w = 0;
  file >> h >> w;
  if (!file || h < 1 || w < 1) return fail(EMT6_ERR_IO, std::string("malformed state: ") + path);
  const int32_t H = h + 2, W = w + 2;
  *height = H;
  *width = W;
  if (!out) return EMT6_OK;  // size query
  if ((int64_t)H * W > cap)
    return fail(EMT6_ERR_LIMIT, "state has " + std::to_string(H * W) + " sites, buffer holds " +
                                    std::to_string(cap));
  for (int32_t r = 0; r < H; ++r)
    for (int32_t c = 0; c < W; ++c) {
      emt6_site &s = out[r * W + c];
      std::memset(&s, 0, sizeof(s));
      if (r == 0 || r == h + 1 || c == 0 || c == w + 1) {  // state.cc:19-22
        s.state = 2;
        s.cho = p->external_levels[0];
        s.ox = p->external_levels[1];
        s.gi = p->external_levels[2];
        continue;
      }
      int st = 0;
      file >> st >> s.cho >> s.ox >> s.gi;
      if (st) {
        s.state = 1;
        file >> s.time_in_repair >> s.irradiation;
        if (s.irradiation > 0) s.repair_delay_time = host_calc_delay(s.irradiation, *p);
        file >> s.proliferation_time;
        for (int i = 0; i < 5; ++i) file >> s.cycle_times[i];
        int mode = 0, phase = 0;
        file >> mode >> phase;
        s.mode = (uint8_t)mode;
        s.phase = (uint8_t)phase;
      } else {
        s.state = 0;
      }
      if (!file)
        return fail(EMT6_ERR_IO, std::string("truncated state file: ") + path);
    }
  return EMT6_OK;
}

int emt6_save_state(const char *path, const emt6_site *sites, int32_t height, int32_t width) {
  if (!path || !sites) return fail(EMT6_ERR_INVALID, "null argument");
  std::ofstream file(path);
  if (!file.good()) return fail(EMT6_ERR_IO, std::string("Could not open the file: ") + path);
  const int32_t h = height - 2, w = width - 2;
  file << h << "\n" << w << "\n";  // state.cc:55-82
  for (int32_t r = 1; r < h + 1; ++r)
    for (int32_t c = 1; c < w + 1; ++c) {
      const emt6_site &s = sites[r * width + c];
      const bool occ = s.state == 1;
      file << (int)occ << "\n";
      file << s.cho << "\n" << s.ox << "\n" << s.gi << "\n";
      if (occ) {
        file << s.time_in_repair << "\n" << s.irradiation << "\n" << s.proliferation_time << "\n";
        for (int i = 0; i < 5; ++i) file << s.cycle_times[i] << "\n";
        file << (int)s.mode << "\n" << (int)s.phase << "\n";
      }
    }
  return file.good() ? EMT6_OK : fail(EMT6_ERR_IO, std::string("write failed: ") + path);
}

// ---- batch ---------------------------------------------------------------------------
int emt6_batch_create(const emt6_params *p, const emt6_site *tumors, int32_t n_tumors,
                      int32_t height, int32_t width, int32_t n_protocols, uint32_t protocol_bins,
                      uint32_t protocol_resolution, uint32_t protocol_length, int64_t n_sims,
                      const int32_t *sim_tumor, const int32_t *sim_protocol,
                      const uint32_t *sim_horizon, int32_t device, uint64_t seed,
                      emt6_batch **out) {
  if (!out) return fail(EMT6_ERR_INVALID, "null output handle");
  *out = nullptr;
  int rc = check_params(p);
  if (rc) return rc;
  if (!tumors || n_tumors < 1 || n_sims < 1 || !sim_tumor || !sim_protocol || n_protocols < 1)
    return fail(EMT6_ERR_INVALID, "empty batch");
  if (height != p->lattice_height + 2 || width != p->lattice_width + 2)
    return fail(EMT6_ERR_INVALID, "tumour dims " + std::to_string(height) + "x" +
                                      std::to_string(width) + " do not match lattice_dims + 2");
  if (protocol_resolution == 0) return fail(EMT6_ERR_INVALID, "protocol_resolution must be > 0");
  for (int64_t i = 0; i < n_sims; ++i) {
    if (sim_tumor[i] < 0 || sim_tumor[i] >= n_tumors)
      return fail(EMT6_ERR_INVALID, "sim_tumor out of range at " + std::to_string(i));
    if (sim_protocol[i] < 0 || sim_protocol[i] >= n_protocols)
      return fail(EMT6_ERR_INVALID, "sim_protocol out of range at " + std::to_string(i));
  }
  // the border ring must not hold cells: the kernels read the 8 neighbours of
  // every occupied site without bounds checks
  for (int32_t t = 0; t < n_tumors; ++t)
    for (int32_t r = 0; r < height; ++r)
      for (int32_t c = 0; c < width; ++c) {
        const emt6_site &s = tumors[(size_t)t * height * width + (size_t)r * width + c];
        const bool border = r == 0 || c == 0 || r == height - 1 || c == width - 1;
        if (s.state > 2)
          return fail(EMT6_ERR_INVALID, "site state must be 0, 1 or 2");
        if (border && s.state == 1)
          return fail(EMT6_ERR_INVALID, "occupied site on the border ring of tumour " +
                                            std::to_string(t));
      }
  int ndev = 0;
  EMT6_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev)
    return fail(EMT6_ERR_INVALID, "device " + std::to_string(device) + " not available");
  DeviceGuard g(device);
  std::unique_ptr<emt6_batch> b(new emt6_batch());
  b->device = device;
  b->params = *p;
  b->H = height;
  b->W = width;
  b->HW = height * width;
  b->n = n_sims;
  b->T = n_tumors;
  b->P = n_protocols;
  b->bins = protocol_bins;
  b->res = protocol_resolution;
  b->length = protocol_length;
  b->seed = seed;
  b->kp = make_kparams(*p, seed, protocol_resolution, protocol_length, protocol_bins);
  b->fstride = (uint32_t)((3 * b->HW + 31) / 32 * 32);
  b->sstride = (uint32_t)((b->HW + 127) / 128 * 128);
  b->lstride = (uint32_t)((b->kp.lcap + 63) / 64 * 64);
  EMT6_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  const size_t HW = b->HW;
  EMT6_CUDA(b->fld.alloc((size_t)n_sims * b->fstride));
  EMT6_CUDA(b->st.alloc((size_t)n_sims * b->sstride));
  EMT6_CUDA(b->cell.alloc((size_t)n_sims * HW * 3));
  EMT6_CUDA(b->list.alloc((size_t)n_sims * b->lstride));
  EMT6_CUDA(b->meta.alloc((size_t)n_sims));
  EMT6_CUDA(b->roi.alloc((size_t)n_sims * 8));
  EMT6_CUDA(b->step.alloc((size_t)n_sims));
  EMT6_CUDA(b->counts.alloc((size_t)n_sims));
  EMT6_CUDA(b->sim_tumor.alloc((size_t)n_sims));
  EMT6_CUDA(b->sim_protocol.alloc((size_t)n_sims));
  EMT6_CUDA(b->err.alloc(1));
  EMT6_CUDA(b->ticket.alloc(1));
  EMT6_CUDA(b->diffused.alloc(1));
  EMT6_CUDA(b->doses.alloc((size_t)n_protocols * std::max<uint32_t>(protocol_bins, 1)));
  EMT6_CUDA(b->tpl_fld.alloc((size_t)n_tumors * b->fstride));
  EMT6_CUDA(b->tpl_st.alloc((size_t)n_tumors * b->sstride));
  EMT6_CUDA(b->tpl_cell.alloc((size_t)n_tumors * HW * 3));
  EMT6_CUDA(cudaMemsetAsync(b->err.p, 0, sizeof(uint32_t), b->stream));
  EMT6_CUDA(cudaMemsetAsync(b->diffused.p, 0, sizeof(unsigned long long), b->stream));
  EMT6_CUDA(cudaMemsetAsync(b->counts.p, 0, sizeof(uint32_t) * n_sims, b->stream));
  // tumour templates: field planes, state bytes, cell records
  {
    std::vector<float> hf((size_t)n_tumors * b->fstride, 0.f);
    std::vector<uint8_t> hs((size_t)n_tumors * b->sstride, 0);
    std::vector<float4> hc((size_t)n_tumors * HW * 3);
    for (int32_t t = 0; t < n_tumors; ++t)
      for (size_t q = 0; q < HW; ++q) {
        float f3[3];
        site_to_records(tumors[t * HW + q], f3, &hs[t * b->sstride + q], &hc[(t * HW + q) * 3]);
        for (int k = 0; k < 3; ++k) hf[t * b->fstride + k * HW + q] = f3[k];
      }
    EMT6_CUDA(cudaMemcpy(b->tpl_fld.p, hf.data(), hf.size() * 4, cudaMemcpyHostToDevice));
    EMT6_CUDA(cudaMemcpy(b->tpl_st.p, hs.data(), hs.size(), cudaMemcpyHostToDevice));
    EMT6_CUDA(cudaMemcpy(b->tpl_cell.p, hc.data(), hc.size() * 16, cudaMemcpyHostToDevice));
  }
  EMT6_CUDA(cudaMemcpy(b->sim_tumor.p, sim_tumor, n_sims * 4, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(b->sim_protocol.p, sim_protocol, n_sims * 4, cudaMemcpyHostToDevice));
  if (sim_horizon) {
    b->has_horizon = true;
    EMT6_CUDA(b->horizon.alloc((size_t)n_sims));
    EMT6_CUDA(cudaMemcpy(b->horizon.p, sim_horizon, n_sims * 4, cudaMemcpyHostToDevice));
    b->max_horizon = *std::max_element(sim_horizon, sim_horizon + n_sims);
  }
  // launch order, rebuilt on the device before every chunk (emt6::launch_order)
  EMT6_CUDA(b->order.alloc((size_t)n_sims));
  EMT6_CUDA(b->order_hist.alloc(emt6::kOrderKeys));
  b->h_doses.assign((size_t)n_protocols * std::max<uint32_t>(protocol_bins, 1), 0.f);
  b->epoch = 0;
  rc = b->reset();
  if (rc) return rc;
  b->epoch = 0;  // the first epoch after creation is 0
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  *out = b.release();
  return EMT6_OK;
}

int emt6_batch_destroy(emt6_batch *b) {
  delete b;
  return EMT6_OK;
}

int emt6_batch_reset(emt6_batch *b) {
  if (!b) return fail(EMT6_ERR_INVALID, "null handle");
  std::lock_guard<std::mutex> lk(b->mu);
  DeviceGuard g(b->device);
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  return b->reset();
}

int emt6_batch_add_irradiations(emt6_batch *b, const int32_t *protocol, const uint32_t *step,
                                const float *dose, int64_t n) {
  if (!b) return fail(EMT6_ERR_INVALID, "null handle");
  if (n > 0 && (!protocol || !step || !dose)) return fail(EMT6_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(b->mu);
  DeviceGuard g(b->device);
  const uint32_t nb = std::max<uint32_t>(b->bins, 1);
  for (int64_t i = 0; i < n; ++i) {
    if (protocol[i] < 0 || protocol[i] >= b->P)
      return fail(EMT6_ERR_INVALID, "protocol index out of range: " + std::to_string(protocol[i]));
    const uint32_t bin = step[i] / b->res;  // Protocol::closestDose, protocol.h:16-18
    if (bin >= nb)
      return fail(EMT6_ERR_INVALID, "irradiation step " + std::to_string(step[i]) +
                                        " is beyond the protocol length");
  }
  for (int64_t i = 0; i < n; ++i) b->h_doses[(size_t)protocol[i] * nb + step[i] / b->res] += dose[i];
  return b->upload_doses();
}

int emt6_batch_set_doses(emt6_batch *b, const float *doses) {
  if (!b || !doses) return fail(EMT6_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(b->mu);
  DeviceGuard g(b->device);
  std::memcpy(b->h_doses.data(), doses, b->h_doses.size() * sizeof(float));
  return b->upload_doses();
}

int emt6_batch_run(emt6_batch *b, uint32_t nsteps) {
  if (!b) return fail(EMT6_ERR_INVALID, "null handle");
  std::lock_guard<std::mutex> lk(b->mu);
  DeviceGuard g(b->device);
  return b->run(nsteps);
}

int emt6_batch_sync(emt6_batch *b) {
  if (!b) return fail(EMT6_ERR_INVALID, "null handle");
  DeviceGuard g(b->device);
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  return b->check_err();
}

int emt6_batch_counts(emt6_batch *b, uint32_t *out) {
  if (!b || !out) return fail(EMT6_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(b->mu);
  DeviceGuard g(b->device);
  const int grid = (int)std::min<int64_t>(b->n, 65535 * 4);
  count_kernel<<<grid, 256, 0, b->stream>>>(b->st.p, b->sstride, b->HW, b->counts.p, b->n);
  EMT6_CUDA(cudaGetLastError());
  b->launches += 1;
  EMT6_CUDA(cudaMemcpyAsync(out, b->counts.p, b->n * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            b->stream));
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  return b->check_err();
}

int emt6_batch_summary(emt6_batch *b, float *out) {
  if (!b || !out) return fail(EMT6_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(b->mu);
  DeviceGuard g(b->device);
  DevBuf<float> d;
  EMT6_CUDA(d.alloc((size_t)b->n * 13));
  const int grid = (int)std::min<int64_t>(b->n, 65535 * 4);
  summary_kernel<<<grid, 256, 0, b->stream>>>(b->fld.p, b->fstride, b->st.p, b->sstride,
                                              b->cell.p, b->H, b->W, d.p, b->n);
  EMT6_CUDA(cudaGetLastError());
  b->launches += 1;
  EMT6_CUDA(cudaMemcpyAsync(out, d.p, (size_t)b->n * 13 * sizeof(float), cudaMemcpyDeviceToHost,
                            b->stream));
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  return b->check_err();
}

int emt6_batch_get_state(emt6_batch *b, int64_t sim, emt6_site *out) {
  if (!b || !out) return fail(EMT6_ERR_INVALID, "null argument");
  if (sim < 0 || sim >= b->n)
    return fail(EMT6_ERR_INVALID, "Cannot read data from sample " + std::to_string(sim) +
                                      ". Batch size: " + std::to_string(b->n));
  std::lock_guard<std::mutex> lk(b->mu);
  DeviceGuard g(b->device);
  const size_t HW = b->HW;
  std::vector<float> f(b->fstride);
  std::vector<uint8_t> s(b->sstride);
  std::vector<float4> c(HW * 3);
  EMT6_CUDA(cudaMemcpyAsync(f.data(), b->fld.p + sim * b->fstride, b->fstride * 4,
                            cudaMemcpyDeviceToHost, b->stream));
  EMT6_CUDA(cudaMemcpyAsync(s.data(), b->st.p + sim * b->sstride, b->sstride,
                            cudaMemcpyDeviceToHost, b->stream));
  EMT6_CUDA(cudaMemcpyAsync(c.data(), b->cell.p + sim * HW * 3, HW * 3 * 16,
                            cudaMemcpyDeviceToHost, b->stream));
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  for (size_t q = 0; q < HW; ++q)
    records_to_site(f[q], f[HW + q], f[2 * HW + q], s[q], &c[q * 3], out[q]);
  return EMT6_OK;
}

int emt6_batch_step(emt6_batch *b, int64_t sim, uint32_t *out) {
  if (!b || !out || sim < 0 || sim >= b->n) return fail(EMT6_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(b->mu);
  DeviceGuard g(b->device);
  EMT6_CUDA(cudaMemcpyAsync(out, b->step.p + sim, 4, cudaMemcpyDeviceToHost, b->stream));
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  return EMT6_OK;
}

void *emt6_batch_stream(emt6_batch *b) { return b ? (void *)b->stream : nullptr; }

int emt6_batch_diffused(emt6_batch *b, unsigned long long *out) {
  if (!b || !out) return fail(EMT6_ERR_INVALID, "null argument");
  DeviceGuard g(b->device);
  EMT6_CUDA(cudaMemcpyAsync(out, b->diffused.p, 8, cudaMemcpyDeviceToHost, b->stream));
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  return EMT6_OK;
}

int emt6_batch_launches(emt6_batch *b, unsigned long long *out) {
  if (!b || !out) return fail(EMT6_ERR_INVALID, "null argument");
  *out = b->launches;
  return EMT6_OK;
}

int emt6_probe_fp32_peak(int32_t device, double *tflops) {
  if (!tflops) return fail(EMT6_ERR_INVALID, "null argument");
  DeviceGuard g(device);
  double best = 0;
  EMT6_CUDA(emt6::fp32_peak(device, &best));
  *tflops = best;
  return EMT6_OK;
}

int emt6_batch_set_schedule(emt6_batch *b, int32_t mode, uint32_t steps_per_launch) {
  if (!b || mode < 0 || mode > 3) return fail(EMT6_ERR_INVALID, "bad schedule");
  std::lock_guard<std::mutex> lk(b->mu);
  b->sched = mode & 1;
  b->use_graph = (mode & 2) != 0;
  if (steps_per_launch) b->chunk = steps_per_launch;
  return EMT6_OK;
}

int emt6_batch_set_layouts(emt6_batch *b, uint32_t layouts) {
  if (!b) return fail(EMT6_ERR_INVALID, "null handle");
  if (layouts & ~kLayoutAll) return fail(EMT6_ERR_INVALID, "unknown layout bits");
  std::lock_guard<std::mutex> lk(b->mu);
  DeviceGuard g(b->device);
  // a captured launch sequence holds the old parameters: drop it
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  if (b->graph_exec) {
    cudaGraphExecDestroy(b->graph_exec);
    b->graph_exec = nullptr;
  }
  b->kp.layouts = layouts;
  return EMT6_OK;
}

int emt6_batch_set_index_base(emt6_batch *b, uint32_t base) {
  if (!b) return fail(EMT6_ERR_INVALID, "null handle");
  std::lock_guard<std::mutex> lk(b->mu);
  if ((uint64_t)base + (uint64_t)b->n > 0x100000000ull)
    return fail(EMT6_ERR_INVALID, "simulation index base + n_sims exceeds 2^32");
  DeviceGuard g(b->device);
  // a captured launch sequence holds the old parameters: drop it
  EMT6_CUDA(cudaStreamSynchronize(b->stream));
  if (b->graph_exec) {
    cudaGraphExecDestroy(b->graph_exec);
    b->graph_exec = nullptr;
  }
  b->kp.sim_base = base;
  return EMT6_OK;
}

// ---- experiment ------------------------------------------------------------------------
int emt6_experiment_create(const emt6_params *p, const emt6_site *tumors, int32_t n_tumors,
                           int32_t height, int32_t width, int32_t runs, int32_t protocols_num,
                           uint32_t simulation_steps, uint32_t protocol_resolution,
                           int32_t device, uint64_t seed, emt6_experiment **out) {
  if (!out) return fail(EMT6_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (runs < 1 || protocols_num < 1 || n_tumors < 1)
    return fail(EMT6_ERR_INVALID, "runs, protocols_num and the tumour count must be positive");
  if (protocol_resolution == 0) return fail(EMT6_ERR_INVALID, "protocol_resolution must be > 0");
  const int64_t B = (int64_t)runs * protocols_num * n_tumors;
  std::vector<int32_t> st(B), sp(B);
  int64_t i = 0;
  for (int32_t pp = 0; pp < protocols_num; ++pp)  // backend.cc:58-66: (protocol, tumour, run)
    for (int32_t t = 0; t < n_tumors; ++t)
      for (int32_t r = 0; r < runs; ++r, ++i) {
        st[i] = t;
        sp[i] = pp;
      }
  const uint32_t bins = (simulation_steps + protocol_resolution - 1) / protocol_resolution;
  std::unique_ptr<emt6_experiment> e(new emt6_experiment());
  int rc = emt6_batch_create(p, tumors, n_tumors, height, width, protocols_num, bins,
                             protocol_resolution, simulation_steps, B, st.data(), sp.data(),
                             nullptr, device, seed, &e->b);
  if (rc) return rc;
  e->runs = runs;
  e->protocols = protocols_num;
  e->tumors = n_tumors;
  *out = e.release();
  return EMT6_OK;
}

int emt6_experiment_destroy(emt6_experiment *e) {
  delete e;
  return EMT6_OK;
}

int emt6_experiment_add_irradiations(emt6_experiment *e, const int32_t *protocol,
                                     const uint32_t *step, const float *dose, int64_t n) {
  if (!e) return fail(EMT6_ERR_INVALID, "null handle");
  return emt6_batch_add_irradiations(e->b, protocol, step, dose, n);
}

int emt6_experiment_run(emt6_experiment *e, uint32_t nsteps) {
  if (!e) return fail(EMT6_ERR_INVALID, "null handle");
  if (e->running) return fail(EMT6_ERR_STATE, "Check failed: !running; Experiment already running.");
  int rc = emt6_batch_run(e->b, nsteps);
  if (rc) return rc;
  e->running = true;
  return EMT6_OK;
}

int emt6_experiment_results(emt6_experiment *e, uint32_t *out) {
  if (!e) return fail(EMT6_ERR_INVALID, "null handle");
  if (!e->running) return fail(EMT6_ERR_STATE, "First you have to run the experiment.");
  e->running = false;
  return emt6_batch_counts(e->b, out);
}

int emt6_experiment_reset(emt6_experiment *e) {
  if (!e) return fail(EMT6_ERR_INVALID, "null handle");
  return emt6_batch_reset(e->b);
}

int emt6_experiment_state(emt6_experiment *e, int64_t sim, emt6_site *out) {
  if (!e) return fail(EMT6_ERR_INVALID, "null handle");
  return emt6_batch_get_state(e->b, sim, out);
}

emt6_batch *emt6_experiment_batch(emt6_experiment *e) { return e ? e->b : nullptr; }

// ---- instrumentation -------------------------------------------------------------------
int emt6_read_instr_counters(int32_t device, emt6_instr_counters *out) {
  if (!out) return fail(EMT6_ERR_INVALID, "null argument");
  DeviceGuard g(device);
  unsigned long long c[4];
  double dp = 0;
  EMT6_CUDA(emt6::instr_read(c, &dp, nullptr));
  out->repair_decisions = c[0];
  out->repair_kills = c[1];
  out->irradiation_events = c[2];
  out->divisions = c[3];
  out->sum_death_prob = dp;
  return EMT6_OK;
}

int emt6_reset_instr_counters(int32_t device) {
  DeviceGuard g(device);
  EMT6_CUDA(emt6::instr_reset());
  return EMT6_OK;
}

int emt6_read_instr_histograms(int32_t device, unsigned long long *out) {
  if (!out) return fail(EMT6_ERR_INVALID, "null argument");
  DeviceGuard g(device);
  unsigned long long c[4];
  double dp = 0;
  EMT6_CUDA(emt6::instr_read(c, &dp, out));
  return EMT6_OK;
}

}  // extern "C"

namespace {
template <typename T>
struct Tmp {
  T *p = nullptr;
  ~Tmp() {
    if (p) cudaFree(p);
  }
};
}  // namespace

extern "C" {

// ---- device unit hooks ---------------------------------------------------------------

#define EMT6_TMP(T, name, count)                                       \
  Tmp<T> name;                                                         \
  EMT6_CUDA(cudaMalloc(&name.p, std::max<size_t>((size_t)(count), 1) * sizeof(T)))

int emt6_test_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out, int64_t n,
                     int32_t device) {
  DeviceGuard g(device);
  EMT6_TMP(uint4, c, n);
  EMT6_TMP(uint2, k, n);
  EMT6_TMP(uint4, o, n);
  EMT6_CUDA(cudaMemcpy(c.p, ctr, n * 16, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(k.p, key, n * 8, cudaMemcpyHostToDevice));
  EMT6_CUDA(emt6::launch_test_philox(c.p, k.p, o.p, n));
  EMT6_CUDA(cudaMemcpy(out, o.p, n * 16, cudaMemcpyDeviceToHost));
  return EMT6_OK;
}

int emt6_test_math(const float *x, float *expf_out, const double *u, double *log_out,
                   double *sin_out, double *cos_out, int64_t n, int32_t device) {
  DeviceGuard g(device);
  EMT6_TMP(float, dx, n);
  EMT6_TMP(float, de, n);
  EMT6_TMP(double, du, n);
  EMT6_TMP(double, dl, n);
  EMT6_TMP(double, ds, n);
  EMT6_TMP(double, dc, n);
  EMT6_CUDA(cudaMemcpy(dx.p, x, n * 4, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(du.p, u, n * 8, cudaMemcpyHostToDevice));
  EMT6_CUDA(emt6::launch_test_math(dx.p, de.p, du.p, dl.p, ds.p, dc.p, n));
  EMT6_CUDA(cudaMemcpy(expf_out, de.p, n * 4, cudaMemcpyDeviceToHost));
  EMT6_CUDA(cudaMemcpy(log_out, dl.p, n * 8, cudaMemcpyDeviceToHost));
  EMT6_CUDA(cudaMemcpy(sin_out, ds.p, n * 8, cudaMemcpyDeviceToHost));
  EMT6_CUDA(cudaMemcpy(cos_out, dc.p, n * 8, cudaMemcpyDeviceToHost));
  return EMT6_OK;
}

int emt6_test_site_step(const emt6_params *p, emt6_site *sites, const uint32_t *vac,
                        const float *dose, const float *draws, int32_t *ready, int32_t *used,
                        int64_t n, int32_t device) {
  int rc = check_params(p);
  if (rc) return rc;
  DeviceGuard g(device);
  const KParams kp = make_kparams(*p, 0, 1, 0, 0);
  std::vector<float4> hc(n * 3);
  std::vector<float> hl(n * 3);
  std::vector<uint8_t> hs(n);
  for (int64_t i = 0; i < n; ++i) site_to_records(sites[i], &hl[3 * i], &hs[i], &hc[3 * i]);
  EMT6_TMP(float4, dc, n * 3);
  EMT6_TMP(float, dl, n * 3);
  EMT6_TMP(uint8_t, ds, n);
  EMT6_TMP(uint32_t, dv, n);
  EMT6_TMP(float, dd, n);
  EMT6_TMP(float, dr, n);
  EMT6_TMP(int32_t, dy, n);
  EMT6_TMP(int32_t, du, n);
  EMT6_CUDA(cudaMemcpy(dc.p, hc.data(), n * 48, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(dl.p, hl.data(), n * 12, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(ds.p, hs.data(), n, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(dv.p, vac, n * 4, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(dd.p, dose, n * 4, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(dr.p, draws, n * 4, cudaMemcpyHostToDevice));
  EMT6_CUDA(emt6::launch_test_site_step(kp, dc.p, dl.p, ds.p, dv.p, dd.p, dr.p, dy.p, du.p, n));
  EMT6_CUDA(cudaMemcpy(hc.data(), dc.p, n * 48, cudaMemcpyDeviceToHost));
  EMT6_CUDA(cudaMemcpy(hl.data(), dl.p, n * 12, cudaMemcpyDeviceToHost));
  EMT6_CUDA(cudaMemcpy(hs.data(), ds.p, n, cudaMemcpyDeviceToHost));
  EMT6_CUDA(cudaMemcpy(ready, dy.p, n * 4, cudaMemcpyDeviceToHost));
  EMT6_CUDA(cudaMemcpy(used, du.p, n * 4, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < n; ++i)
    records_to_site(hl[3 * i], hl[3 * i + 1], hl[3 * i + 2], hs[i], &hc[3 * i], sites[i]);
  return EMT6_OK;
}

int emt6_test_choose(const float *u, int32_t r, int32_t c, int32_t *rc_out, int64_t n,
                     int32_t device) {
  DeviceGuard g(device);
  const int W = c + 2 > 64 ? c + 2 : 64;
  EMT6_TMP(float, du, n);
  EMT6_TMP(int32_t, dr, n * 2);
  EMT6_CUDA(cudaMemcpy(du.p, u, n * 4, cudaMemcpyHostToDevice));
  EMT6_CUDA(emt6::launch_test_choose(du.p, r, c, W, dr.p, n));
  EMT6_CUDA(cudaMemcpy(rc_out, dr.p, n * 8, cudaMemcpyDeviceToHost));
  return EMT6_OK;
}

int emt6_test_divide(const emt6_params *p, emt6_site *parents, const float *z,
                     emt6_site *children, int64_t n, int32_t device) {
  int rc = check_params(p);
  if (rc) return rc;
  DeviceGuard g(device);
  const KParams kp = make_kparams(*p, 0, 1, 0, 0);
  std::vector<float4> hp(n * 3), hc(n * 3);
  std::vector<float> hl(n * 3);
  std::vector<uint8_t> hs(n);
  for (int64_t i = 0; i < n; ++i) site_to_records(parents[i], &hl[3 * i], &hs[i], &hp[3 * i]);
  EMT6_TMP(float4, dp, n * 3);
  EMT6_TMP(float4, dc, n * 3);
  EMT6_TMP(float, dz, n * 5);
  EMT6_CUDA(cudaMemcpy(dp.p, hp.data(), n * 48, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(dz.p, z, n * 20, cudaMemcpyHostToDevice));
  EMT6_CUDA(emt6::launch_test_divide(kp, dp.p, dz.p, dc.p, n));
  EMT6_CUDA(cudaMemcpy(hp.data(), dp.p, n * 48, cudaMemcpyDeviceToHost));
  EMT6_CUDA(cudaMemcpy(hc.data(), dc.p, n * 48, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < n; ++i) {
    records_to_site(parents[i].cho, parents[i].ox, parents[i].gi, parents[i].state, &hp[3 * i],
                    parents[i]);
    records_to_site(0.f, 0.f, 0.f, 0, &hc[3 * i], children[i]);
  }
  return EMT6_OK;
}

int emt6_test_normals(uint64_t seed, const uint32_t *step, const uint32_t *sim, uint32_t epoch,
                      float *z, int64_t n, int32_t device) {
  DeviceGuard g(device);
  KParams kp;
  std::memset(&kp, 0, sizeof(kp));
  kp.seed_lo = (uint32_t)seed;
  kp.seed_hi = (uint32_t)(seed >> 32);
  EMT6_TMP(uint32_t, ds, n);
  EMT6_TMP(uint32_t, dm, n);
  EMT6_TMP(float, dz, n * 5);
  EMT6_CUDA(cudaMemcpy(ds.p, step, n * 4, cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(dm.p, sim, n * 4, cudaMemcpyHostToDevice));
  EMT6_CUDA(emt6::launch_test_normals(kp, ds.p, dm.p, epoch, dz.p, n));
  EMT6_CUDA(cudaMemcpy(z, dz.p, n * 20, cudaMemcpyDeviceToHost));
  return EMT6_OK;
}

}  // extern "C"

static int test_block(int mode, int variant, const emt6_params *pp, float *fields,
                      const uint8_t *state, int32_t height, int32_t width, int32_t *roi,
                      uint8_t *mask, uint16_t *list, uint32_t *n, int32_t device) {
  emt6_params p;
  if (pp) {
    p = *pp;
  } else {
    std::memset(&p, 0, sizeof(p));
    p.time_step = 6.f;
    p.diffusion_time_step = 0.25f;
  }
  p.lattice_height = height - 2;
  p.lattice_width = width - 2;
  int rc = check_params(&p);
  if (rc) return rc;
  DeviceGuard g(device);
  const KParams kp = make_kparams(p, 0, 1, 0, 0);
  const int HW = height * width;
  EMT6_TMP(float, df, 3 * HW);
  EMT6_TMP(uint8_t, ds, HW);
  EMT6_TMP(int32_t, dr, 8);
  EMT6_TMP(uint8_t, dm, HW + 4 * (height + width) + 16);
  EMT6_TMP(uint16_t, dl, kp.lcap);
  EMT6_TMP(uint32_t, dn, 1);
  if (fields) EMT6_CUDA(cudaMemcpy(df.p, fields, 3 * HW * 4, cudaMemcpyHostToDevice));
  if (state) EMT6_CUDA(cudaMemcpy(ds.p, state, HW, cudaMemcpyHostToDevice));
  if (mode == 2) EMT6_CUDA(cudaMemcpy(dr.p, roi, 5 * 4, cudaMemcpyHostToDevice));
  EMT6_CUDA(emt6::launch_test_block(kp, mode, variant != 0, fields ? df.p : nullptr,
                                    state ? ds.p : nullptr, dr.p, dm.p, dl.p, dn.p));
  EMT6_CUDA(cudaDeviceSynchronize());
  if (mode == 0) {
    EMT6_CUDA(cudaMemcpy(n, dn.p, 4, cudaMemcpyDeviceToHost));
    EMT6_CUDA(cudaMemcpy(list, dl.p, *n * 2, cudaMemcpyDeviceToHost));
  } else if (mode == 1) {
    EMT6_CUDA(cudaMemcpy(roi, dr.p, 5 * 4, cudaMemcpyDeviceToHost));
    if (roi[2] > 0)
      EMT6_CUDA(cudaMemcpy(mask, dm.p, (roi[2] + 2) * (roi[3] + 2), cudaMemcpyDeviceToHost));
  } else {
    uint32_t refused = 0;
    EMT6_CUDA(cudaMemcpy(&refused, dn.p, 4, cudaMemcpyDeviceToHost));
    if (refused) return fail(EMT6_ERR_LIMIT, "region does not fit the narrow kernel path");
    EMT6_CUDA(cudaMemcpy(fields, df.p, 3 * HW * 4, cudaMemcpyDeviceToHost));
  }
  return EMT6_OK;
}

extern "C" {

int emt6_test_roi(const uint8_t *state, int32_t height, int32_t width, int32_t *roi,
                  uint8_t *mask, int32_t device) {
  return test_block(1, 0, nullptr, nullptr, state, height, width, roi, mask, nullptr, nullptr,
                    device);
}

int emt6_test_list(const uint8_t *state, int32_t height, int32_t width, uint16_t *list,
                   uint32_t *n, int32_t device) {
  return test_block(0, 0, nullptr, nullptr, state, height, width, nullptr, nullptr, list, n,
                    device);
}

int emt6_test_diffuse(const emt6_params *p, float *fields, int32_t height, int32_t width,
                      const int32_t *roi, int32_t variant, int32_t device) {
  if (!p || !fields || !roi) return fail(EMT6_ERR_INVALID, "null argument");
  int32_t r[8] = {roi[0], roi[1], roi[2], roi[3], roi[4], 0, 0, 0};
  return test_block(2, variant, p, fields, nullptr, height, width, r, nullptr, nullptr, nullptr,
                    device);
}

int emt6_test_order(const int32_t *roi, const uint32_t *step, const uint32_t *horizon,
                    int64_t nsims, uint32_t t_end, int64_t *order, int32_t device) {
  if (!roi || !step || !order || nsims < 1) return fail(EMT6_ERR_INVALID, "null argument");
  DeviceGuard g(device);
  EMT6_TMP(int32_t, r, nsims * 8);
  EMT6_TMP(uint32_t, st, nsims);
  EMT6_TMP(uint32_t, hz, nsims);
  EMT6_TMP(uint32_t, hist, emt6::kOrderKeys);
  EMT6_TMP(int64_t, out, nsims);
  EMT6_CUDA(cudaMemcpy(r.p, roi, nsims * 8 * sizeof(int32_t), cudaMemcpyHostToDevice));
  EMT6_CUDA(cudaMemcpy(st.p, step, nsims * sizeof(uint32_t), cudaMemcpyHostToDevice));
  if (horizon)
    EMT6_CUDA(cudaMemcpy(hz.p, horizon, nsims * sizeof(uint32_t), cudaMemcpyHostToDevice));
  emt6::RunArgs a{};
  a.roi = r.p;
  a.step = st.p;
  a.horizon = horizon ? hz.p : nullptr;
  a.nsims = nsims;
  EMT6_CUDA(emt6::launch_order(a, t_end, hist.p, out.p, 0));
  EMT6_CUDA(cudaMemcpy(order, out.p, nsims * sizeof(int64_t), cudaMemcpyDeviceToHost));
  return EMT6_OK;
}

}  // extern "C"

namespace emt6 {
// for the allocation-free entry point (emt6_noalloc.cu)
KParams make_kparams_public(const emt6_params &p, uint64_t seed, uint32_t res, uint32_t length,
                            uint32_t bins) {
  return make_kparams(p, seed, res, length, bins);
}
int set_error(int code, const std::string &msg) { return fail(code, msg); }
}  // namespace emt6
