// surrogate.cu -- the protocol-outcome surrogate: a 100 -> 512 -> 512 -> 512 -> 1
// GELU MLP trained and evaluated on the GPU with hand-written kernels.
//
// GEMMs run on the 5th-generation tensor cores: one CTA of 512 threads owns a
// 128 x 128 FP32 accumulator in tensor memory (TMEM, 128 columns); thread 0
// streams 128 x 64 BF16 tiles of both operands into a 4-stage shared-memory
// ring with TMA (128-byte swizzle), thread 32 issues tcgen05.mma (M = 128,
// N = 128, K = 16, BF16 in, FP32 accumulate) and frees each stage with
// tcgen05.commit; after the last k-block the 16 warps read the accumulator
// back with tcgen05.ld (warp w: TMEM lanes 32(w % 4)..+31 = tile rows,
// columns 32(w / 4)..+31) and run a fused epilogue:
//   EPI_STORE_F32  C = A B^T in FP32 (tests, gradient export)
//   EPI_BIAS_GELU  forward hidden layer: Z = acc + b, A = gelu(Z); stores Z, A
//                  and A^T (BF16) so every later GEMM reads K-major operands
//   EPI_GELU_BWD   dZ = acc * gelu'(Z) for the layer below; stores dZ, dZ^T
//   EPI_ADAM       the accumulator is dW: Adam update of the FP32 master
//                  weights, moments, and the BF16 copies W and W^T
// Both operands are K-major ("TN": C[M,N] = sum_k A[m,k] B[n,k]), so a layer
// keeps W [out, in] and W^T [in, out] in BF16 and activations in both
// orientations; no transposes run between GEMMs.
//
// Every wait on an mbarrier is bounded (kWaitLimitNs); a wait that runs out
// sets an error flag, the CTA stops issuing work, waits (bounded) for its own
// tensor-core work, frees its TMEM and returns; the host reports the flag.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <utility>
#include <vector>

#include "emt6ro_gb300.h"
#include "emt6ro_surrogate.h"

namespace emt6 {
int set_error(int code, const std::string &msg);
}

namespace {

// 16 warps: warp w reads TMEM lane quarter w % 4 (tile rows 32(w % 4)..+31)
// and runs the epilogue of column group w / 4 (32 columns), so the
// epilogue's transcendental work and stores spread over 4x more warps
constexpr int BM = 128, BN = 128, BK = 64, STAGES = 4, GEMM_THREADS = 512;
constexpr int TILE_BYTES = BM * BK * 2;  // 16 KB per operand per stage
constexpr int GEMM_SMEM = 1024 + STAGES * 2 * TILE_BYTES + 256;
constexpr uint64_t kWaitLimitNs = 1000000000ull;  // 1 s

enum { EPI_STORE_F32 = 0, EPI_BIAS_GELU = 1, EPI_GELU_BWD = 2, EPI_ADAM = 3 };

struct EpiArgs {
  int M, N;
  float *c_out;                 // STORE_F32: [M][N]
  const float *bias;            // BIAS_GELU: [N]
  __nv_bfloat16 *z_out;         // BIAS_GELU: [M][N]
  __nv_bfloat16 *a_out;         // BIAS_GELU: A [M][N]; GELU_BWD: dZ [M][N]
  __nv_bfloat16 *a_out_t;       // BIAS_GELU: A^T [N][M]; GELU_BWD: dZ^T [N][M]
  const __nv_bfloat16 *z_in;    // GELU_BWD: Z of the layer below [M][N]
  float *w, *m, *v;             // ADAM: master weights and moments [M][N]
  __nv_bfloat16 *w_bf, *w_bf_t; // ADAM: BF16 W [M][N] and W^T [N][M]
  float lr, beta1, beta2, eps, bc1, bc2;
  int *err;
  // test hook (emt6_test_mlp_gemm_timeout): when nonzero, the MMA issuer
  // first waits this many ns on a barrier nothing arrives on, so it gives up
  // exactly as a timed-out pipeline wait would
  uint32_t stall_ns;
};

// ---- PTX wrappers ----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase of `parity` to complete.  Gives up after
// limit_ns (default kWaitLimitNs), or early when another thread of the CTA
// raised `abort`.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, const volatile int *abort,
                          uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (abort && *abort) return false;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, uint32_t bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Programmatic dependent launch: the kernels of a training step are launched
// with programmatic stream serialisation, so each one's launch and prologue
// overlap the tail of the one before.  pdl_wait() blocks until the previous
// kernel in the stream has completed and its writes are visible (a no-op
// without the launch attribute); pdl_trigger(), issued after a CTA's last
// global write, lets the next kernel be scheduled.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, BF16 inputs, FP32 accumulator.
__device__ __forceinline__ void umma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane; the wait is in the
// same statement so no use of the registers can be scheduled before it.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: K-major tile written by TMA with the
// 128-byte swizzle (rows of 64 BF16 = 128 B, 8-row atoms of 1024 B).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) |
         (static_cast<uint64_t>(1) << 16) |            // leading offset (unused when swizzled)
         (static_cast<uint64_t>(1024 >> 4) << 32) |    // stride offset: next 8-row atom
         (static_cast<uint64_t>(1) << 46) |            // descriptor version
         (static_cast<uint64_t>(2) << 61);             // 128-byte swizzle
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 128, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                            (static_cast<uint32_t>(BN >> 3) << 17) |
                            (static_cast<uint32_t>(BM >> 4) << 24);

__device__ __forceinline__ float gelu(float z) {
  return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}

__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) +
         z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// ---- epilogues ---------------------------------------------------------------
template <int EPI>
__device__ __forceinline__ void epilogue(const EpiArgs &ep, int row, int col0, const float (&v)[32]) {
  const int M = ep.M, N = ep.N;
  if constexpr (EPI == EPI_STORE_F32) {
    float4 *dst = reinterpret_cast<float4 *>(ep.c_out + static_cast<size_t>(row) * N + col0);
#pragma unroll
    for (int i = 0; i < 8; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
  } else if constexpr (EPI == EPI_BIAS_GELU) {
    alignas(16) __nv_bfloat16 zb[32], ab[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const float z = v[i] + __ldg(ep.bias + col0 + i);
      zb[i] = __float2bfloat16_rn(z);
      ab[i] = __float2bfloat16_rn(gelu(z));
    }
    uint4 *zd = reinterpret_cast<uint4 *>(ep.z_out + static_cast<size_t>(row) * N + col0);
    uint4 *ad = reinterpret_cast<uint4 *>(ep.a_out + static_cast<size_t>(row) * N + col0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      zd[i] = reinterpret_cast<const uint4 *>(zb)[i];
      ad[i] = reinterpret_cast<const uint4 *>(ab)[i];
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) ep.a_out_t[static_cast<size_t>(col0 + i) * M + row] = ab[i];
  } else if constexpr (EPI == EPI_GELU_BWD) {
    alignas(16) __nv_bfloat16 zin[32], db[32];
    const uint4 *zs = reinterpret_cast<const uint4 *>(ep.z_in + static_cast<size_t>(row) * N + col0);
#pragma unroll
    for (int i = 0; i < 4; ++i) reinterpret_cast<uint4 *>(zin)[i] = zs[i];
#pragma unroll
    for (int i = 0; i < 32; ++i)
      db[i] = __float2bfloat16_rn(v[i] * gelu_grad(__bfloat162float(zin[i])));
    uint4 *dd = reinterpret_cast<uint4 *>(ep.a_out + static_cast<size_t>(row) * N + col0);
#pragma unroll
    for (int i = 0; i < 4; ++i) dd[i] = reinterpret_cast<const uint4 *>(db)[i];
#pragma unroll
    for (int i = 0; i < 32; ++i) ep.a_out_t[static_cast<size_t>(col0 + i) * M + row] = db[i];
  } else {  // EPI_ADAM
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const size_t k = static_cast<size_t>(row) * N + col0 + i;
      const float g = v[i];
      const float m = ep.beta1 * ep.m[k] + (1.0f - ep.beta1) * g;
      const float s = ep.beta2 * ep.v[k] + (1.0f - ep.beta2) * g * g;
      const float w = ep.w[k] - ep.lr * (m / ep.bc1) / (sqrtf(s / ep.bc2) + ep.eps);
      ep.m[k] = m;
      ep.v[k] = s;
      ep.w[k] = w;
      const __nv_bfloat16 wb = __float2bfloat16_rn(w);
      ep.w_bf[k] = wb;
      ep.w_bf_t[static_cast<size_t>(col0 + i) * M + row] = wb;
    }
  }
}

// C tile (blockIdx.y, blockIdx.x) of C[M,N] = A[M,K] B[N,K]^T over the
// k-blocks [blockIdx.z * nk, (blockIdx.z + 1) * nk) (split K: each z writes
// its own FP32 partial tile, EPI_STORE_F32 only).
template <int EPI>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    mlp_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    int nk, EpiArgs ep) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~static_cast<uintptr_t>(1023));
  uint8_t *sA = smem;
  uint8_t *sB = smem + STAGES * TILE_BYTES;
  // barriers: full[STAGES], empty[STAGES], done, never (nothing arrives on
  // it: the target of the test hook's stalled wait)
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * STAGES * TILE_BYTES);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * STAGES + 2);
  volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES),
                 done = smem_u32(bars + 2 * STAGES), never = smem_u32(bars + 2 * STAGES + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int kb0 = blockIdx.z * nk;
  if (EPI == EPI_STORE_F32 && blockIdx.z) ep.c_out += static_cast<size_t>(blockIdx.z) * ep.M * ep.N;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(done, 1);
    mbar_init(never, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
  }
  if (warp == 0) tmem_alloc(smem_u32(tmem_slot), BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  pdl_wait();  // operands and epilogue inputs come from the previous kernel

  bool failed = false;
  int issued = 0;  // k-blocks whose loads thread 0 issued
  if (threadIdx.x == 0) {
    // TMA producer
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait(empty0 + 8 * s, ((kb / STAGES) - 1) & 1, abort)) {
        failed = true;
        *abort = 1;
        break;
      }
      mbar_expect_tx(full0 + 8 * s, 2 * TILE_BYTES);
      tma_load_2d(smem_u32(sA + s * TILE_BYTES), &tmA, full0 + 8 * s, (kb0 + kb) * BK, m0);
      tma_load_2d(smem_u32(sB + s * TILE_BYTES), &tmB, full0 + 8 * s, (kb0 + kb) * BK, n0);
      ++issued;
    }
  } else if (threadIdx.x == 32) {
    // MMA issuer
    if (ep.stall_ns && !mbar_wait(never, 0, abort, ep.stall_ns)) {
      failed = true;
      *abort = 1;
      __threadfence_block();
    }
    for (int kb = 0; kb < nk && !failed; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait(full0 + 8 * s, (kb / STAGES) & 1, abort)) {
        failed = true;
        *abort = 1;
        __threadfence_block();
        break;
      }
      tc_fence_after();
      const uint32_t a = smem_u32(sA + s * TILE_BYTES), b = smem_u32(sB + s * TILE_BYTES);
#pragma unroll
      for (int k = 0; k < BK / 16; ++k)
        umma_bf16(tmem, sw128_desc(a + 32 * k), sw128_desc(b + 32 * k), kIdesc,
                  (kb | k) != 0 ? 1u : 0u);
      umma_commit(empty0 + 8 * s);
    }
    // arrives once every MMA issued above has completed, failed or not
    umma_commit(done);
  }
  __syncwarp();
  bool have = mbar_wait(done, 0, nullptr);
  if (threadIdx.x == 0 && *abort) {
    // a pipeline wait gave up: let the loads still in flight (at most the
    // last STAGES issued; older stages were consumed before being reused)
    // land before the CTA frees its shared memory
    for (int kb = issued - STAGES < 0 ? 0 : issued - STAGES; kb < issued; ++kb)
      mbar_wait(full0 + 8 * (kb % STAGES), (kb / STAGES) & 1, nullptr);
  }
  have = __all_sync(0xffffffffu, have && !*abort && !failed);
  tc_fence_after();
  if (have) {
    const int quarter = warp & 3, group = warp >> 2;
    float v[32];
    tmem_ld32(tmem + (static_cast<uint32_t>(quarter * 32) << 16) + group * 32, v);
    epilogue<EPI>(ep, m0 + quarter * 32 + lane, n0 + group * 32, v);
  } else if (lane == 0) {
    atomicOr(ep.err, 1);
  }
  pdl_trigger();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tmem_dealloc(tmem, BN);
  }
}

// ---- small kernels -------------------------------------------------------------
// fp32 features [B][in] -> BF16 X [B][in_pad] (zero padded) and X^T
// [in_pad][B]; one block per 32 rows, the transpose through shared memory.
__global__ void __launch_bounds__(256) pack_input_kernel(const float *x, int B, int in, int in_pad,
                                                         __nv_bfloat16 *X, __nv_bfloat16 *XT,
                                                         float *loss) {
  __shared__ __nv_bfloat16 tile[128][34];
  const int r0 = blockIdx.x * 32;
  pdl_wait();
  if (loss && blockIdx.x == 0 && threadIdx.x == 0) *loss = 0.0f;  // this step's loss sum
  for (int i = threadIdx.x; i < 32 * in_pad; i += 256) {
    const int rr = i / in_pad, c = i % in_pad;
    const __nv_bfloat16 v =
        __float2bfloat16_rn(c < in ? x[static_cast<size_t>(r0 + rr) * in + c] : 0.0f);
    X[static_cast<size_t>(r0 + rr) * in_pad + c] = v;
    tile[c][rr] = v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 32 * in_pad; i += 256) {
    const int c = i / 32, rr = i % 32;
    XT[static_cast<size_t>(c) * B + r0 + rr] = tile[c][rr];
  }
  pdl_trigger();
}

// Output layer and loss: y = A3 w4 + b4, one warp per row (8 BF16 per lane
// per load); with targets, dy = 2 (y - t) / B and sum (y - t)^2 into *loss.
__global__ void __launch_bounds__(256) head_y_kernel(const __nv_bfloat16 *A3, const float *w4,
                                                     const float *b4, int B, int H,
                                                     const float *target, float *y, float *dy,
                                                     float *loss) {
  __shared__ float s_loss[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // the grid covers B exactly
  const uint4 *row = reinterpret_cast<const uint4 *>(A3 + static_cast<size_t>(r) * H);
  pdl_wait();
  float acc = 0.0f;
  for (int j = lane; j < H / 8; j += 32) {
    const uint4 u = row[j];
    const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&u);
#pragma unroll
    for (int q = 0; q < 8; ++q) acc += __bfloat162float(h[q]) * w4[8 * j + q];
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    const float yr = acc + b4[0];
    y[r] = yr;
    float e2 = 0.0f;
    if (target) {
      const float e = yr - target[r];
      dy[r] = 2.0f * e / static_cast<float>(B);
      e2 = e * e;
    }
    s_loss[wid] = e2;
  }
  if (!target) return;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) t += s_loss[i];
    atomicAdd(loss, t);
  }
  pdl_trigger();
}

// dZ3 = dy w4 * gelu'(Z3) for a 32-row x 64-column tile per block, stored in
// both orientations (the transposed copy through shared memory).
__global__ void __launch_bounds__(256) head_dz_kernel(const __nv_bfloat16 *Z3, const float *w4,
                                                      const float *dy, int B, int H,
                                                      __nv_bfloat16 *dZ3, __nv_bfloat16 *dZ3T) {
  __shared__ __nv_bfloat16 tile[64][34];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 64;
  pdl_wait();
  for (int i = threadIdx.x; i < 32 * 64; i += 256) {
    const int rr = i / 64, cc = i % 64;
    const int r = r0 + rr, c = c0 + cc;
    const float z = __bfloat162float(Z3[static_cast<size_t>(r) * H + c]);
    const __nv_bfloat16 g = __float2bfloat16_rn(dy[r] * w4[c] * gelu_grad(z));
    dZ3[static_cast<size_t>(r) * H + c] = g;
    tile[cc][rr] = g;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 32 * 64; i += 256) {
    const int cc = i / 32, rr = i % 32;
    dZ3T[static_cast<size_t>(c0 + cc) * B + r0 + rr] = tile[cc][rr];
  }
  pdl_trigger();
}

struct VecAdam {
  float *w, *m, *v;
  const __nv_bfloat16 *rows;  // [n][B] rows to sum (bias: dZ^T), or A3^T for w4
  const float *dy;            // w4: weights of the row sum; null for biases
  float *grad_out;            // optional: export of the gradient
  int n;
};

// Gradients and Adam updates of the vectors: b1, b2, b3 (row sums of dZ^T),
// w4 (A3^T dy) and b4 (sum dy).  One warp per element.
__global__ void vec_adam_kernel(VecAdam p0, VecAdam p1, VecAdam p2, VecAdam p3, VecAdam p4, int B,
                                float lr, float beta1, float beta2, float eps, float bc1, float bc2,
                                int apply) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  pdl_wait();
  int idx = gw;
  VecAdam p;
  if (idx < p0.n) {
    p = p0;
  } else if ((idx -= p0.n) < p1.n) {
    p = p1;
  } else if ((idx -= p1.n) < p2.n) {
    p = p2;
  } else if ((idx -= p2.n) < p3.n) {
    p = p3;
  } else if ((idx -= p3.n) < p4.n) {
    p = p4;
  } else {
    return;
  }
  float g = 0.0f;
  if (p.rows) {
    // B is a multiple of 128: 8 BF16 (16 bytes) per lane per load
    const uint4 *row = reinterpret_cast<const uint4 *>(p.rows + static_cast<size_t>(idx) * B);
    for (int j = lane; j < B / 8; j += 32) {
      const uint4 u = row[j];
      const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&u);
      if (p.dy) {
        const float4 d0 = reinterpret_cast<const float4 *>(p.dy)[2 * j];
        const float4 d1 = reinterpret_cast<const float4 *>(p.dy)[2 * j + 1];
        g += __bfloat162float(h[0]) * d0.x + __bfloat162float(h[1]) * d0.y +
             __bfloat162float(h[2]) * d0.z + __bfloat162float(h[3]) * d0.w +
             __bfloat162float(h[4]) * d1.x + __bfloat162float(h[5]) * d1.y +
             __bfloat162float(h[6]) * d1.z + __bfloat162float(h[7]) * d1.w;
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) g += __bfloat162float(h[q]);
      }
    }
  } else {
    for (int j = lane; j < B; j += 32) g += p.dy[j];
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
  if (lane != 0) return;
  if (p.grad_out) p.grad_out[idx] = g;
  if (!apply) return;
  const float m = beta1 * p.m[idx] + (1.0f - beta1) * g;
  const float s = beta2 * p.v[idx] + (1.0f - beta2) * g * g;
  p.m[idx] = m;
  p.v[idx] = s;
  p.w[idx] -= lr * (m / bc1) / (sqrtf(s / bc2) + eps);
  pdl_trigger();
}

__global__ void to_bf16_kernel(const float *src, __nv_bfloat16 *dst, __nv_bfloat16 *dst_t, int rows,
                               int cols) {
  const int total = rows * cols;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int r = i / cols, c = i % cols;
    const __nv_bfloat16 b = __float2bfloat16_rn(src[i]);
    dst[i] = b;
    if (dst_t) dst_t[static_cast<size_t>(c) * rows + r] = b;
  }
}

// ---- host side -------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// K-major BF16 matrix [rows][cols] (cols = K contiguous), boxes of 128 rows x 64 columns.
bool make_map(CUtensorMap *map, const void *base, int rows, int cols) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
  cuuint64_t strides[1] = {static_cast<cuuint64_t>(cols) * 2};
  cuuint32_t box[2] = {BK, BM};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Launch with programmatic stream serialisation (see pdl_wait / pdl_trigger).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t st, Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <int EPI>
cudaError_t launch_gemm(const CUtensorMap &a, const CUtensorMap &b, int M, int N, int K,
                        const EpiArgs &ep, cudaStream_t st, int splits = 1) {
  static bool attr_set[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr_set[dev]) {
    cudaError_t e = cudaFuncSetAttribute(mlp_gemm_kernel<EPI>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_SMEM);
    if (e != cudaSuccess) return e;
    attr_set[dev] = true;
  }
  return launch_pdl(mlp_gemm_kernel<EPI>, dim3(N / BN, M / BM, splits), dim3(GEMM_THREADS),
                    GEMM_SMEM, st, a, b, K / BK / splits, ep);
}

// Sum of the split-K partial tiles of a weight gradient g[M][N] in a fixed
// order, then either the Adam update (FP32 master, moments, BF16 W and W^T)
// or, with grad_out, the gradient itself.  One element per thread, 32 x 32
// tiles of 1024 threads; W^T goes through shared memory so both stores are
// coalesced.
__global__ void __launch_bounds__(1024) adam_reduce_kernel(const float *__restrict__ part,
                                                           int splits, int M, int N, float *w,
                                                           float *m, float *v,
                                                           __nv_bfloat16 *w_bf,
                                                           __nv_bfloat16 *w_bf_t, float *grad_out,
                                                           float lr, float beta1, float beta2,
                                                           float eps, float bc1, float bc2) {
  __shared__ __nv_bfloat16 tile[32][34];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int r = blockIdx.y * 32 + ty, c = blockIdx.x * 32 + tx;
  const size_t MN = static_cast<size_t>(M) * N;
  const size_t k = static_cast<size_t>(r) * N + c;
  pdl_wait();
  float pz[8];
#pragma unroll
  for (int z = 0; z < 8; ++z) pz[z] = z < splits ? part[z * MN + k] : 0.0f;
  float g = pz[0];
#pragma unroll
  for (int z = 1; z < 8; ++z)
    if (z < splits) g += pz[z];
  if (grad_out) {
    grad_out[k] = g;
    return;
  }
  const float mm = beta1 * m[k] + (1.0f - beta1) * g;
  const float vv = beta2 * v[k] + (1.0f - beta2) * g * g;
  const float ww = w[k] - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
  m[k] = mm;
  v[k] = vv;
  w[k] = ww;
  const __nv_bfloat16 wb = __float2bfloat16_rn(ww);
  w_bf[k] = wb;
  tile[tx][ty] = wb;
  __syncthreads();
  w_bf_t[static_cast<size_t>(blockIdx.x * 32 + ty) * M + blockIdx.y * 32 + tx] = tile[ty][tx];
  pdl_trigger();
}

template <typename T>
struct DevArr {
  T *p = nullptr;
  size_t n = 0;
  bool alloc(size_t count) {
    n = count;
    return cudaMalloc(&p, count * sizeof(T)) == cudaSuccess;
  }
  ~DevArr() {
    if (p) cudaFree(p);
  }
};

}  // namespace

struct emt6_mlp {
  int device = 0, max_batch = 0;
  int in = EMT6_MLP_IN, in_pad = EMT6_MLP_IN_PAD, H = EMT6_MLP_HIDDEN;
  cudaStream_t stream = nullptr;
  int64_t step = 0;
  int cur_b = -1;
  float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  // parameters: FP32 masters, Adam moments, BF16 copies (W and W^T)
  DevArr<float> w[3], m[3], v[3], b[3], bm[3], bv[3], w4, m4, v4, b4, mb4, vb4;
  DevArr<__nv_bfloat16> wb[3], wbt[3];
  // activations for max_batch rows
  DevArr<__nv_bfloat16> X, XT, Z[3], A[3], AT[3], dZ[3], dZT[3];
  DevArr<float> y, dy, loss, gradw[3], gradv[5], work;
  int split_override = 0;  // 0: choose per batch size
  DevArr<int> err;
  CUtensorMap mX, mXT, mA[3], mAT[3], mW[3], mWT[3], mdZ[3], mdZT[3];
};

namespace {

int rows_of(int) { return EMT6_MLP_HIDDEN; }
int cols_of(int l) { return l == 0 ? EMT6_MLP_IN_PAD : EMT6_MLP_HIDDEN; }

int fail(const std::string &m, int code = EMT6_ERR_DEVICE) { return emt6::set_error(code, m); }

int cuda_fail(cudaError_t e, const char *what) {
  return fail(std::string(what) + ": " + cudaGetErrorString(e), EMT6_ERR_CUDA);
}

EpiArgs base_args(emt6_mlp *net, int M, int N) {
  EpiArgs ep;
  std::memset(&ep, 0, sizeof(ep));
  ep.M = M;
  ep.N = N;
  ep.err = net->err.p;
  return ep;
}

// forward hidden layers for B rows already packed into X / X^T
int forward_hidden(emt6_mlp *net, int B) {
  for (int l = 0; l < 3; ++l) {
    EpiArgs ep = base_args(net, B, net->H);
    ep.bias = net->b[l].p;
    ep.z_out = net->Z[l].p;
    ep.a_out = net->A[l].p;
    ep.a_out_t = net->AT[l].p;
    const CUtensorMap &a = l == 0 ? net->mX : net->mA[l - 1];
    cudaError_t e = launch_gemm<EPI_BIAS_GELU>(a, net->mW[l], B, net->H, cols_of(l), ep, net->stream);
    if (e != cudaSuccess) return cuda_fail(e, "surrogate forward GEMM");
  }
  return EMT6_OK;
}

int check_batch(emt6_mlp *net, int B) {
  if (B <= 0 || B > net->max_batch || B % 128 != 0)
    return fail("surrogate batch must be a positive multiple of 128 up to max_batch",
                EMT6_ERR_INVALID);
  return EMT6_OK;
}

int read_err(emt6_mlp *net) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, net->err.p, sizeof(int), cudaMemcpyDeviceToHost, net->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
  if (e != cudaSuccess) return cuda_fail(e, "surrogate");
  if (h) return fail("surrogate GEMM: a tensor-core pipeline wait timed out");
  return EMT6_OK;
}

// maps depend on the batch size through the activation shapes
bool build_maps(emt6_mlp *net, int B) {
  bool ok = make_map(&net->mX, net->X.p, B, net->in_pad) &&
            make_map(&net->mXT, net->XT.p, net->in_pad, B);
  for (int l = 0; l < 3 && ok; ++l) {
    ok = make_map(&net->mA[l], net->A[l].p, B, net->H) &&
         make_map(&net->mAT[l], net->AT[l].p, net->H, B) &&
         make_map(&net->mW[l], net->wb[l].p, rows_of(l), cols_of(l)) &&
         make_map(&net->mWT[l], net->wbt[l].p, cols_of(l), rows_of(l)) &&
         make_map(&net->mdZ[l], net->dZ[l].p, B, net->H) &&
         make_map(&net->mdZT[l], net->dZT[l].p, net->H, B);
  }
  return ok;
}

// Split of the weight-gradient GEMMs' K (= B) dimension: the most of 8, 4, 2
// that leaves every CTA at least 4 k-blocks of 64 rows.
int weight_splits(const emt6_mlp *net, int B) {
  const int nkb = B / BK;
  if (net->split_override > 0) return nkb % net->split_override == 0 ? net->split_override : 1;
  for (int sp : {8, 4, 2})
    if (nkb % sp == 0 && nkb / sp >= 4) return sp;
  return 1;
}

int backward(emt6_mlp *net, int B, const float *d_target, bool apply, float lr) {
  cudaStream_t st = net->stream;
  cudaError_t e;
  float *loss = net->loss.p;
  // the loss sum was zeroed by the input packing of this step
  e = launch_pdl(head_y_kernel, dim3(B / 8), dim3(256), 0, st, (const __nv_bfloat16 *)net->A[2].p,
                 (const float *)net->w4.p, (const float *)net->b4.p, B, net->H, d_target,
                 net->y.p, net->dy.p, loss);
  if (e == cudaSuccess)
    e = launch_pdl(head_dz_kernel, dim3(B / 32, net->H / 64), dim3(256), 0, st,
                   (const __nv_bfloat16 *)net->Z[2].p, (const float *)net->w4.p,
                   (const float *)net->dy.p, B, net->H, net->dZ[2].p, net->dZT[2].p);
  if (e != cudaSuccess) return cuda_fail(e, "surrogate head");
  ++net->step;
  const float bc1 = 1.0f - std::pow(net->beta1, static_cast<float>(net->step));
  const float bc2 = 1.0f - std::pow(net->beta2, static_cast<float>(net->step));
  for (int l = 2; l >= 0; --l) {
    // dA of the layer below (before W[l] changes), then dW[l]
    if (l > 0) {
      EpiArgs ep = base_args(net, B, net->H);
      ep.z_in = net->Z[l - 1].p;
      ep.a_out = net->dZ[l - 1].p;
      ep.a_out_t = net->dZT[l - 1].p;
      e = launch_gemm<EPI_GELU_BWD>(net->mdZ[l], net->mWT[l], B, net->H, net->H, ep, st);
      if (e != cudaSuccess) return cuda_fail(e, "surrogate backward GEMM");
    }
    const CUtensorMap &bmap = l == 0 ? net->mXT : net->mAT[l - 1];
    const int N = cols_of(l);
    const int splits = weight_splits(net, B);
    if (splits > 1) {
      // K = B is long and M x N small: split K over `splits` CTAs per tile,
      // then reduce the partial tiles in a fixed order (deterministic)
      EpiArgs ep = base_args(net, net->H, N);
      ep.c_out = net->work.p;
      e = launch_gemm<EPI_STORE_F32>(net->mdZT[l], bmap, net->H, N, B, ep, st, splits);
      if (e == cudaSuccess) {
        e = launch_pdl(adam_reduce_kernel, dim3(N / 32, net->H / 32), dim3(1024), 0, st,
                       (const float *)net->work.p, splits, net->H, N, net->w[l].p, net->m[l].p,
                       net->v[l].p, net->wb[l].p, net->wbt[l].p,
                       apply ? nullptr : net->gradw[l].p, lr, net->beta1, net->beta2, net->eps,
                       bc1, bc2);
      }
    } else if (apply) {
      EpiArgs ep = base_args(net, net->H, N);
      ep.w = net->w[l].p;
      ep.m = net->m[l].p;
      ep.v = net->v[l].p;
      ep.w_bf = net->wb[l].p;
      ep.w_bf_t = net->wbt[l].p;
      ep.lr = lr;
      ep.beta1 = net->beta1;
      ep.beta2 = net->beta2;
      ep.eps = net->eps;
      ep.bc1 = bc1;
      ep.bc2 = bc2;
      e = launch_gemm<EPI_ADAM>(net->mdZT[l], bmap, net->H, N, B, ep, st);
    } else {
      EpiArgs ep = base_args(net, net->H, N);
      ep.c_out = net->gradw[l].p;
      e = launch_gemm<EPI_STORE_F32>(net->mdZT[l], bmap, net->H, N, B, ep, st);
    }
    if (e != cudaSuccess) return cuda_fail(e, "surrogate weight-gradient GEMM");
  }
  VecAdam vp[5];
  for (int l = 0; l < 3; ++l)
    vp[l] = {net->b[l].p, net->bm[l].p, net->bv[l].p, net->dZT[l].p, nullptr,
             apply ? nullptr : net->gradv[l].p, net->H};
  vp[3] = {net->w4.p, net->m4.p, net->v4.p, net->AT[2].p, net->dy.p,
           apply ? nullptr : net->gradv[3].p, net->H};
  vp[4] = {net->b4.p, net->mb4.p, net->vb4.p, nullptr, net->dy.p,
           apply ? nullptr : net->gradv[4].p, 1};
  const int warps = 4 * net->H + 1;
  e = launch_pdl(vec_adam_kernel, dim3((warps * 32 + 255) / 256), dim3(256), 0, st, vp[0], vp[1],
                 vp[2], vp[3], vp[4], B, lr, net->beta1, net->beta2, net->eps, bc1, bc2,
                 apply ? 1 : 0);
  if (e != cudaSuccess) return cuda_fail(e, "surrogate vector Adam");
  if (!apply) --net->step;
  return EMT6_OK;
}

int pack(emt6_mlp *net, const float *d_x, int B) {
  cudaError_t e = launch_pdl(pack_input_kernel, dim3(B / 32), dim3(256), 0, net->stream, d_x, B,
                             net->in, net->in_pad, net->X.p, net->XT.p, net->loss.p);
  return e == cudaSuccess ? EMT6_OK : cuda_fail(e, "surrogate input");
}

int refresh_bf16(emt6_mlp *net) {
  for (int l = 0; l < 3; ++l) {
    to_bf16_kernel<<<304, 256, 0, net->stream>>>(net->w[l].p, net->wb[l].p, net->wbt[l].p,
                                                  rows_of(l), cols_of(l));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "surrogate weights");
  }
  return EMT6_OK;
}

// The 8 FP32 parameter arrays in the C ABI's order and their element counts.
void param_arrays(emt6_mlp *net, float *dev[8], size_t cnt[8]) {
  for (int l = 0; l < 3; ++l) {
    dev[2 * l] = net->w[l].p;
    cnt[2 * l] = static_cast<size_t>(rows_of(l)) * cols_of(l);
    dev[2 * l + 1] = net->b[l].p;
    cnt[2 * l + 1] = net->H;
  }
  dev[6] = net->w4.p;
  cnt[6] = net->H;
  dev[7] = net->b4.p;
  cnt[7] = 1;
}

// Batch-size-dependent maps are rebuilt when B changes.
int ensure_maps(emt6_mlp *net, int B) {
  if (net->cur_b == B) return EMT6_OK;
  if (!build_maps(net, B)) return fail("surrogate: cuTensorMapEncodeTiled failed");
  net->cur_b = B;
  return EMT6_OK;
}

}  // namespace

extern "C" {

int emt6_mlp_create(int max_batch, uint64_t seed, int device, emt6_mlp **out) {
  if (!out) return fail("emt6_mlp_create: null output", EMT6_ERR_INVALID);
  *out = nullptr;
  if (max_batch <= 0 || max_batch % 128 != 0)
    return fail("emt6_mlp_create: max_batch must be a positive multiple of 128", EMT6_ERR_INVALID);
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(e, "emt6_mlp_create");
  if (!encode_fn()) return fail("emt6_mlp_create: cuTensorMapEncodeTiled unavailable");
  auto *net = new emt6_mlp();
  net->device = device;
  net->max_batch = max_batch;
  const int H = net->H;
  bool ok = cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) == cudaSuccess;
  for (int l = 0; l < 3 && ok; ++l) {
    const size_t n = static_cast<size_t>(rows_of(l)) * cols_of(l);
    ok = net->w[l].alloc(n) && net->m[l].alloc(n) && net->v[l].alloc(n) && net->b[l].alloc(H) &&
         net->bm[l].alloc(H) && net->bv[l].alloc(H) && net->wb[l].alloc(n) &&
         net->wbt[l].alloc(n) && net->gradw[l].alloc(n);
  }
  const size_t BH = static_cast<size_t>(max_batch) * H;
  ok = ok && net->w4.alloc(H) && net->m4.alloc(H) && net->v4.alloc(H) && net->b4.alloc(1) &&
       net->mb4.alloc(1) && net->vb4.alloc(1) && net->X.alloc(static_cast<size_t>(max_batch) * net->in_pad) &&
       net->XT.alloc(static_cast<size_t>(max_batch) * net->in_pad) && net->y.alloc(max_batch) &&
       net->dy.alloc(max_batch) && net->loss.alloc(1) && net->err.alloc(1);
  for (int l = 0; l < 3 && ok; ++l)
    ok = net->Z[l].alloc(BH) && net->A[l].alloc(BH) && net->AT[l].alloc(BH) &&
         net->dZ[l].alloc(BH) && net->dZT[l].alloc(BH);
  for (int i = 0; i < 5 && ok; ++i) ok = net->gradv[i].alloc(i < 4 ? H : 1);
  ok = ok && net->work.alloc(static_cast<size_t>(8) * H * H);
  if (!ok) {
    if (net->stream) cudaStreamDestroy(net->stream);
    delete net;
    return fail("emt6_mlp_create: out of device memory");
  }
  // He-style initialisation from a seeded generator; biases and moments zero
  std::mt19937_64 rng(seed);
  std::vector<float> host;
  e = cudaSuccess;
  for (int l = 0; l < 4 && e == cudaSuccess; ++l) {
    const int rows = l < 3 ? rows_of(l) : 1, cols = l < 3 ? cols_of(l) : H;
    const int fan_in = l == 0 ? net->in : H;
    std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / static_cast<float>(fan_in)));
    host.assign(static_cast<size_t>(rows) * cols, 0.0f);
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c)
        if (l != 0 || c < net->in) host[static_cast<size_t>(r) * cols + c] = nd(rng);
    float *dst = l < 3 ? net->w[l].p : net->w4.p;
    e = cudaMemcpy(dst, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice);
  }
  float *zero[] = {net->m[0].p, net->v[0].p, net->m[1].p, net->v[1].p, net->m[2].p, net->v[2].p,
                   net->b[0].p, net->bm[0].p, net->bv[0].p, net->b[1].p, net->bm[1].p,
                   net->bv[1].p, net->b[2].p, net->bm[2].p, net->bv[2].p, net->m4.p, net->v4.p,
                   net->b4.p, net->mb4.p, net->vb4.p};
  const size_t zn[] = {net->m[0].n, net->v[0].n, net->m[1].n, net->v[1].n, net->m[2].n,
                       net->v[2].n, net->b[0].n, net->bm[0].n, net->bv[0].n, net->b[1].n,
                       net->bm[1].n, net->bv[1].n, net->b[2].n, net->bm[2].n, net->bv[2].n,
                       net->m4.n, net->v4.n, net->b4.n, net->mb4.n, net->vb4.n};
  for (size_t i = 0; i < sizeof(zero) / sizeof(zero[0]) && e == cudaSuccess; ++i)
    e = cudaMemset(zero[i], 0, zn[i] * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(net->err.p, 0, sizeof(int));
  if (e != cudaSuccess) {
    emt6_mlp_destroy(net);
    return cuda_fail(e, "emt6_mlp_create");
  }
  int rc = refresh_bf16(net);
  if (rc == EMT6_OK) {
    e = cudaStreamSynchronize(net->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "emt6_mlp_create");
  }
  if (rc != EMT6_OK) {
    emt6_mlp_destroy(net);
    return rc;
  }
  *out = net;
  return EMT6_OK;
}

void emt6_mlp_destroy(emt6_mlp *net) {
  if (!net) return;
  cudaSetDevice(net->device);
  if (net->stream) cudaStreamSynchronize(net->stream);
  if (net->stream) cudaStreamDestroy(net->stream);
  delete net;
}

void *emt6_mlp_stream(emt6_mlp *net) { return net ? net->stream : nullptr; }

int emt6_mlp_set_params(emt6_mlp *net, const float *const *host) {
  if (!net || !host) return fail("emt6_mlp_set_params: null argument", EMT6_ERR_INVALID);
  cudaSetDevice(net->device);
  float *dev[8];
  size_t cnt[8];
  param_arrays(net, dev, cnt);
  cudaError_t e = cudaStreamSynchronize(net->stream);
  for (int i = 0; i < 8 && e == cudaSuccess; ++i)
    e = cudaMemcpy(dev[i], host[i], cnt[i] * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "emt6_mlp_set_params");
  int rc = refresh_bf16(net);
  if (rc != EMT6_OK) return rc;
  e = cudaStreamSynchronize(net->stream);
  return e == cudaSuccess ? EMT6_OK : cuda_fail(e, "emt6_mlp_set_params");
}

int emt6_mlp_get_params(emt6_mlp *net, float *const *host) {
  if (!net || !host) return fail("emt6_mlp_get_params: null argument", EMT6_ERR_INVALID);
  cudaSetDevice(net->device);
  float *dev[8];
  size_t cnt[8];
  param_arrays(net, dev, cnt);
  cudaError_t e = cudaStreamSynchronize(net->stream);
  for (int i = 0; i < 8 && e == cudaSuccess; ++i)
    e = cudaMemcpy(host[i], dev[i], cnt[i] * sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? EMT6_OK : cuda_fail(e, "emt6_mlp_get_params");
}

int emt6_mlp_predict(emt6_mlp *net, const float *d_x, int B, float *d_y) {
  if (!net || !d_x || !d_y) return fail("emt6_mlp_predict: null argument", EMT6_ERR_INVALID);
  cudaSetDevice(net->device);
  int rc = check_batch(net, B);
  if (rc == EMT6_OK) rc = ensure_maps(net, B);
  if (rc == EMT6_OK) rc = pack(net, d_x, B);
  if (rc == EMT6_OK) rc = forward_hidden(net, B);
  if (rc != EMT6_OK) return rc;
  cudaError_t e = launch_pdl(head_y_kernel, dim3(B / 8), dim3(256), 0, net->stream,
                             (const __nv_bfloat16 *)net->A[2].p, (const float *)net->w4.p,
                             (const float *)net->b4.p, B, net->H, (const float *)nullptr, d_y,
                             (float *)nullptr, (float *)nullptr);
  return e == cudaSuccess ? EMT6_OK : cuda_fail(e, "emt6_mlp_predict");
}

int emt6_mlp_train_step(emt6_mlp *net, const float *d_x, const float *d_target, int B, float lr,
                        float *h_loss) {
  if (!net || !d_x || !d_target) return fail("emt6_mlp_train_step: null argument", EMT6_ERR_INVALID);
  cudaSetDevice(net->device);
  int rc = check_batch(net, B);
  if (rc == EMT6_OK) rc = ensure_maps(net, B);
  if (rc == EMT6_OK) rc = pack(net, d_x, B);
  if (rc == EMT6_OK) rc = forward_hidden(net, B);
  if (rc == EMT6_OK) rc = backward(net, B, d_target, true, lr);
  if (rc != EMT6_OK) return rc;
  if (h_loss) {
    float s = 0.0f;
    cudaError_t e = cudaMemcpyAsync(&s, net->loss.p, 4, cudaMemcpyDeviceToHost, net->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
    if (e != cudaSuccess) return cuda_fail(e, "emt6_mlp_train_step");
    *h_loss = s / static_cast<float>(B);
    return read_err(net);
  }
  return EMT6_OK;
}

int emt6_mlp_gradients(emt6_mlp *net, const float *d_x, const float *d_target, int B,
                       float *const *host_grads, float *h_loss) {
  if (!net || !d_x || !d_target || !host_grads)
    return fail("emt6_mlp_gradients: null argument", EMT6_ERR_INVALID);
  cudaSetDevice(net->device);
  int rc = check_batch(net, B);
  if (rc == EMT6_OK) rc = ensure_maps(net, B);
  if (rc == EMT6_OK) rc = pack(net, d_x, B);
  if (rc == EMT6_OK) rc = forward_hidden(net, B);
  if (rc == EMT6_OK) rc = backward(net, B, d_target, false, 0.0f);
  if (rc != EMT6_OK) return rc;
  if ((rc = read_err(net)) != EMT6_OK) return rc;
  const float *grad[8] = {net->gradw[0].p, net->gradv[0].p, net->gradw[1].p, net->gradv[1].p,
                          net->gradw[2].p, net->gradv[2].p, net->gradv[3].p, net->gradv[4].p};
  float *dev[8];
  size_t cnt[8];
  param_arrays(net, dev, cnt);
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 8 && e == cudaSuccess; ++i)
    e = cudaMemcpy(host_grads[i], grad[i], cnt[i] * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && h_loss) {
    float s = 0.0f;
    e = cudaMemcpy(&s, net->loss.p, 4, cudaMemcpyDeviceToHost);
    *h_loss = s / static_cast<float>(B);
  }
  return e == cudaSuccess ? EMT6_OK : cuda_fail(e, "emt6_mlp_gradients");
}

int emt6_mlp_set_splitk(emt6_mlp *net, int splits) {
  if (!net || (splits != 0 && splits != 1 && splits != 2 && splits != 4 && splits != 8))
    return fail("emt6_mlp_set_splitk: splits must be 0 (automatic), 1, 2, 4 or 8",
                EMT6_ERR_INVALID);
  net->split_override = splits;
  return EMT6_OK;
}

int emt6_mlp_sync(emt6_mlp *net) {
  if (!net) return fail("emt6_mlp_sync: null", EMT6_ERR_INVALID);
  cudaSetDevice(net->device);
  return read_err(net);
}

int emt6_test_mlp_gemm(const void *d_a, const void *d_b, float *d_c, int M, int N, int K,
                       void *stream) {
  if (!d_a || !d_b || !d_c) return fail("emt6_test_mlp_gemm: null argument", EMT6_ERR_INVALID);
  if (M <= 0 || N <= 0 || K <= 0 || M % BM || N % BN || K % BK)
    return fail("emt6_test_mlp_gemm: M, N multiples of 128 and K of 64 required", EMT6_ERR_INVALID);
  if (!encode_fn()) return fail("cuTensorMapEncodeTiled unavailable");
  CUtensorMap ma, mb;
  if (!make_map(&ma, d_a, M, K) || !make_map(&mb, d_b, N, K))
    return fail("emt6_test_mlp_gemm: cuTensorMapEncodeTiled failed");
  int *err = nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMallocAsync(&err, sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(e, "emt6_test_mlp_gemm");
  EpiArgs ep;
  std::memset(&ep, 0, sizeof(ep));
  ep.M = M;
  ep.N = N;
  ep.c_out = d_c;
  ep.err = err;
  e = launch_gemm<EPI_STORE_F32>(ma, mb, M, N, K, ep, st);
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(err, st);
  if (e != cudaSuccess) return cuda_fail(e, "emt6_test_mlp_gemm");
  if (h) return fail("emt6_test_mlp_gemm: a tensor-core pipeline wait timed out");
  return EMT6_OK;
}

int emt6_test_mlp_gemm_timeout(const void *d_a, const void *d_b, float *d_c, int M, int N,
                               int K, uint32_t stall_us, void *stream) {
  if (!d_a || !d_b || !d_c || stall_us == 0 || stall_us > 100000)
    return fail("emt6_test_mlp_gemm_timeout: null argument or stall outside 1..100000 us",
                EMT6_ERR_INVALID);
  if (M <= 0 || N <= 0 || K <= 0 || M % BM || N % BN || K % BK)
    return fail("emt6_test_mlp_gemm_timeout: M, N multiples of 128 and K of 64 required",
                EMT6_ERR_INVALID);
  if (!encode_fn()) return fail("cuTensorMapEncodeTiled unavailable");
  CUtensorMap ma, mb;
  if (!make_map(&ma, d_a, M, K) || !make_map(&mb, d_b, N, K))
    return fail("emt6_test_mlp_gemm_timeout: cuTensorMapEncodeTiled failed");
  int *err = nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMallocAsync(&err, sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(e, "emt6_test_mlp_gemm_timeout");
  EpiArgs ep;
  std::memset(&ep, 0, sizeof(ep));
  ep.M = M;
  ep.N = N;
  ep.c_out = d_c;
  ep.err = err;
  ep.stall_ns = stall_us * 1000u;
  e = launch_gemm<EPI_STORE_F32>(ma, mb, M, N, K, ep, st);
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(err, st);
  if (e != cudaSuccess) return cuda_fail(e, "emt6_test_mlp_gemm_timeout");
  if (h) return fail("emt6_test_mlp_gemm_timeout: a tensor-core pipeline wait timed out");
  return EMT6_OK;
}

}  // extern "C"
