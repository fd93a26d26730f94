// gemm_tc.cu -- tcgen05 GEMM for float32 matrices in BF16 or split-BF16
// precision: C[m][n] = act(sum_k op(A)[m][k] * op(B)[k][n] + bias[n]).
//
// This is the matrix product of Owl's FullyConnected neuron
// (owl_neural_neuron.ml:1907, (x *@ w) + b) and of the backward passes of its
// dot (x^T g, g w^T), so the operands arrive row-major with either the k or
// the m/n index contiguous.  Each operand is staged by producer warps from
// float32 into shared memory in whichever core-matrix layout keeps its global
// reads contiguous: K-major [k chunk][row][16 B] when k is contiguous,
// MN-major [row chunk][k][16 B] when rows are (the instruction descriptor
// carries the choice per operand).  One thread issues M = 128 x N = BN x
// K = 16 MMAs into TMEM; four warps drain it.
//
// Small-M products (a batch of 256 rows) have few output tiles, so the K
// reduction is split over CTAs: each split writes a float32 partial and a
// second kernel sums the partials in split order (deterministic) and applies
// the bias and activation.  Split-BF16 keeps the cross terms in their own
// TMEM accumulator (the tensor core rounds its accumulator toward zero after
// every MMA).  Every pipeline wait is bounded, as in the convolution kernels.
#include <cuda_bf16.h>

#include <algorithm>

#include "../../include/owlgpu.h"
#include "common.cuh"
#include "tc_ptx.cuh"
#include "tc_stage.cuh"

namespace owlgpu {
namespace {

using namespace ptx;

constexpr int kWarps = 16;
constexpr int kThreads = kWarps * 32;
constexpr int kMmaWarp = 0;
constexpr int kEpiWarp0 = 12;
constexpr int kProducerThreads = (kWarps - 1) * 32;
constexpr int kBM = 128;  // MMA M: rows of C per tile
constexpr int kBK = 64;   // k per pipeline stage (four K = 16 MMAs)
constexpr int kSmemMax = 232448;
constexpr long long kSpinLimit = 4000000000LL;

struct GemmParams {
  const float *a, *b;
  float *c;           // the result (splits == 1) or partials [split][M][N]
  const float *bias;  // per column, or null; applied when splits == 1
  int act;
  long long M, N, K;
  long long a_sm, a_sk;  // element strides of op(A) along m and along k
  long long b_sn, b_sk;  // element strides of op(B) along n and along k
  int a_kmaj, b_kmaj;    // 1: the operand's k stride is 1 (else its row stride is 1)
  int BN, NS, splits;
  long long kps;              // k per split, a multiple of kBK
  unsigned a_bytes, b_bytes;  // one stage of each operand, per precision part
  unsigned idesc, tmem_cols, small_off;
  int *status;
  long long spin_limit;
};

__device__ int g_gemm_status;

__device__ __forceinline__ bool wait_bar(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                         int *status, long long limit) {
  if (mbar_try_wait(bar, parity)) return true;
  long long t0 = clock64();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (clock64() - t0 > limit) {
      *abort_flag = 1;
      atomicExch(status, 1);
      return false;
    }
  }
}

__device__ __forceinline__ float apply_act(float v, int act) {
  return act == OWLGPU_ACT_RELU ? (v > 0.f ? v : 0.f) : v;
}

// Stage one operand's k block [k0, k0 + kBK) of rows [row0, row0 + R) into
// `dst` (bf16, or bf16 hi + lo planes lo_off apart), zero outside the
// matrix.  Element (row, k) is at src[row*s_row + k] when kmaj (k
// contiguous), else at src[k*s_k + row].  K-major layout: chunk c of row r at
// (c*R + r)*16; MN-major: k of row chunk j at (j*kBK + k)*16.  Consecutive threads take consecutive
// 16-byte destinations (no bank conflicts); each thread reads 8 contiguous
// floats.  Four slots per thread are loaded before any is converted.
template <int KIND>
__device__ __forceinline__ void stage_operand(uint8_t *dst, uint32_t lo_off, const float *src,
                                              long long s_row, long long s_k, int kmaj,
                                              long long row0, long long rows, int R, long long k0,
                                              long long kend, int tid) {
  constexpr int Q = 4;
  const int total = 8 * R;  // slots: R rows x 8 chunks, or R/8 row chunks x 64 k
  for (int base = tid; base < total; base += Q * kProducerThreads) {
    float v[Q][8];
    int off[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int sl = base + q * kProducerThreads;
#pragma unroll
      for (int e = 0; e < 8; ++e) v[q][e] = 0.f;
      off[q] = -1;
      if (sl < total) {
        if (kmaj) {
          const int c = sl / R, r = sl - c * R;
          off[q] = sl * 16;
          const long long row = row0 + r, k = k0 + 8 * c;
          if (row < rows && k < kend) {
            const float *p = src + row * s_row + k;
            if (k + 8 <= kend && ((uintptr_t)p & 15) == 0) {
              const float4 x0 = __ldg(reinterpret_cast<const float4 *>(p));
              const float4 x1 = __ldg(reinterpret_cast<const float4 *>(p) + 1);
              v[q][0] = x0.x; v[q][1] = x0.y; v[q][2] = x0.z; v[q][3] = x0.w;
              v[q][4] = x1.x; v[q][5] = x1.y; v[q][6] = x1.z; v[q][7] = x1.w;
            } else {
#pragma unroll
              for (int e = 0; e < 8; ++e)
                if (k + e < kend) v[q][e] = __ldg(p + e);
            }
          }
        } else {
          const int j = sl / kBK, kk = sl - j * kBK;
          off[q] = sl * 16;
          const long long k = k0 + kk, row = row0 + 8 * j;
          if (k < kend && row < rows) {
            const float *p = src + k * s_k + row;
            if (row + 8 <= rows && ((uintptr_t)p & 15) == 0) {
              const float4 x0 = __ldg(reinterpret_cast<const float4 *>(p));
              const float4 x1 = __ldg(reinterpret_cast<const float4 *>(p) + 1);
              v[q][0] = x0.x; v[q][1] = x0.y; v[q][2] = x0.z; v[q][3] = x0.w;
              v[q][4] = x1.x; v[q][5] = x1.y; v[q][6] = x1.z; v[q][7] = x1.w;
            } else {
#pragma unroll
              for (int e = 0; e < 8; ++e)
                if (row + e < rows) v[q][e] = __ldg(p + e);
            }
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q)
      if (off[q] >= 0) stage::put_chunk<KIND, 8>(dst + off[q], lo_off, v[q]);
  }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads, 1) gemm_tc_kernel(const __grid_constant__ GemmParams p) {
  constexpr int PARTS = (KIND == stage::K_BF16X3) ? 2 : 1;
  constexpr bool SEP = (KIND == stage::K_BF16X3);
  extern __shared__ __align__(1024) uint8_t smem[];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long m0 = (long long)blockIdx.x * kBM, n0 = (long long)blockIdx.y * p.BN;
  const long long k_begin = (long long)blockIdx.z * p.kps;
  const long long k_end = min(p.K, k_begin + p.kps);
  const int nkb = (int)((k_end - k_begin + kBK - 1) / kBK);
  const unsigned stage_bytes = PARTS * (p.a_bytes + p.b_bytes);

  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)p.NS * stage_bytes);
  uint64_t *full = bars;
  uint64_t *empty = full + p.NS;
  uint64_t *acc_full = empty + p.NS;
  uint64_t *drain = acc_full + 1;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  if (threadIdx.x == 0) {
    for (int i = 0; i < p.NS; ++i) {
      mbar_init(smem_u32(&full[i]), kProducerThreads);
      mbar_init(smem_u32(&empty[i]), 1);
    }
    mbar_init(smem_u32(acc_full), 1);
    mbar_init(smem_u32(drain), 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == kMmaWarp) {
    tmem_alloc(smem_u32(tmem_slot), p.tmem_cols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp != kMmaWarp) {
    // ===================== producers =====================
    const int tid = threadIdx.x - 32;
    bool staged = true;
    for (int i = 0; i < nkb; ++i) {
      const int st = i % p.NS;
      if (!wait_bar(smem_u32(&empty[st]), (uint32_t)(((i / p.NS) & 1) ^ 1), abort_flag, p.status,
                    p.spin_limit)) {
        staged = false;
        break;
      }
      uint8_t *sa = smem + (size_t)st * stage_bytes;
      uint8_t *sb = sa + PARTS * p.a_bytes;
      const long long k0 = k_begin + (long long)i * kBK;
      stage_operand<KIND>(sa, p.a_bytes, p.a, p.a_sm, p.a_sk, p.a_kmaj, m0, p.M, kBM, k0, k_end,
                          tid);
      stage_operand<KIND>(sb, p.b_bytes, p.b, p.b_sn, p.b_sk, p.b_kmaj, n0, p.N, p.BN, k0, k_end,
                          tid);
      fence_proxy_async();
      mbar_arrive(smem_u32(&full[st]));
    }
    if (staged && warp >= kEpiWarp0) {
      // ===================== epilogue: TMEM -> C =====================
      const int q = warp & 3;
      const long long m = m0 + q * 32 + lane;
      if (wait_bar(smem_u32(acc_full), 0, abort_flag, p.status, p.spin_limit)) {
        tc_fence_after();
        const bool final_ = p.splits == 1;
        float *crow = p.c + (final_ ? 0 : (long long)blockIdx.z * p.M * p.N) + m * p.N;
        const uint32_t tcol = tmem_base + ((uint32_t)(q * 32) << 16);
        for (int c0 = 0; c0 < p.BN; c0 += 16) {
          uint32_t r[16];
          tmem_ld16(tcol + (uint32_t)c0, r);
          if (SEP) {
            uint32_t r2[16];
            tmem_ld16(tcol + p.small_off + (uint32_t)c0, r2);
            tmem_ld_wait();
#pragma unroll
            for (int e = 0; e < 16; ++e)
              r[e] = __float_as_uint(__uint_as_float(r[e]) + __uint_as_float(r2[e]));
          } else {
            tmem_ld_wait();
          }
          if (m < p.M) {
            const long long n = n0 + c0;
            float v[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) {
              v[e] = __uint_as_float(r[e]);
              if (final_) {
                if (p.bias && n + e < p.N) v[e] += p.bias[n + e];
                v[e] = apply_act(v[e], p.act);
              }
            }
            if (n + 16 <= p.N && ((uintptr_t)(crow + n) & 15) == 0) {
#pragma unroll
              for (int e = 0; e < 16; e += 4)
                *reinterpret_cast<float4 *>(crow + n + e) = make_float4(v[e], v[e + 1], v[e + 2], v[e + 3]);
            } else {
#pragma unroll
              for (int e = 0; e < 16; ++e)
                if (n + e < p.N) crow[n + e] = v[e];
            }
          }
        }
        tc_fence_before();
      }
    }
  } else if (lane == 0) {
    // ===================== MMA issuer =====================
    const uint32_t s0 = smem_u32(smem);
    // K-major: core matrices along k are R*16 bytes apart, along rows 128;
    // MN-major: along k 128 bytes apart, along rows kBK*16.  One K = 16 step
    // is two k chunks (K-major) or 16 k rows (MN-major), in 16-byte units.
    const uint32_t a_lbo = p.a_kmaj ? kBM * 16 : 128, a_sbo = p.a_kmaj ? 128 : kBK * 16;
    const uint32_t b_lbo = p.b_kmaj ? (uint32_t)p.BN * 16 : 128, b_sbo = p.b_kmaj ? 128 : kBK * 16;
    const uint32_t a_step = p.a_kmaj ? 2 * kBM : 16, b_step = p.b_kmaj ? 2 * (uint32_t)p.BN : 16;
    const uint32_t alo = p.a_bytes >> 4, blo = p.b_bytes >> 4;
    const uint32_t d = tmem_base, ds = tmem_base + p.small_off;
    uint32_t acc = 0;
    bool ok = true;
    for (int i = 0; i < nkb; ++i) {
      const int st = i % p.NS;
      if (!wait_bar(smem_u32(&full[st]), (uint32_t)((i / p.NS) & 1), abort_flag, p.status,
                    p.spin_limit)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t sa = s0 + (uint32_t)st * stage_bytes, sb = sa + PARTS * p.a_bytes;
      const uint64_t ad0 = smem_desc(sa, a_lbo, a_sbo), bd0 = smem_desc(sb, b_lbo, b_sbo);
#pragma unroll
      for (int s = 0; s < kBK / 16; ++s) {
        const uint64_t ad = ad0 + (uint64_t)(s * a_step), bd = bd0 + (uint64_t)(s * b_step);
        mma_bf16(d, ad, bd, p.idesc, acc);
        if (SEP) {
          mma_bf16(ds, ad + (uint64_t)alo, bd, p.idesc, acc);
          mma_bf16(ds, ad, bd + (uint64_t)blo, p.idesc, 1);
        }
        acc = 1;
      }
      mma_commit(smem_u32(&empty[st]));
    }
    if (ok) mma_commit(smem_u32(acc_full));
    mma_commit(smem_u32(drain));
    long long t0 = clock64();
    while (!mbar_try_wait(smem_u32(drain), 0) && clock64() - t0 < kSpinLimit) {
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    tmem_dealloc(tmem_base, p.tmem_cols);
  }
}

// out[m][n] = act(sum over splits z = 0, 1, ... of part[z][m][n] + bias[n]),
// in split order.
__global__ void gemm_reduce(const float *__restrict__ part, float *__restrict__ out,
                            const float *__restrict__ bias, int act, long long M, long long N,
                            int splits) {
  const long long n_all = M * N;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_all;
       i += (long long)gridDim.x * blockDim.x) {
    float s = part[i];
    for (int z = 1; z < splits; ++z) s += part[(long long)z * n_all + i];
    if (bias) s += bias[i % N];
    out[i] = apply_act(s, act);
  }
}

int *gemm_status_word() {
  static int *p[64] = {nullptr};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return nullptr;
  if (!p[dev]) {
    void *q = nullptr;
    if (cudaGetSymbolAddress(&q, g_gemm_status) != cudaSuccess) return nullptr;
    p[dev] = static_cast<int *>(q);
  }
  return p[dev];
}

int num_sms() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 148;
}

template <int KIND>
int launch(const GemmParams &p, size_t smem, dim3 grid, cudaStream_t s) {
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    OWL_CUDA(cudaFuncSetAttribute(gemm_tc_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kSmemMax));
    attr[dev] = true;
  }
  gemm_tc_kernel<KIND><<<grid, kThreads, smem, s>>>(p);
  note_tc_launch();
  OWL_CHECK_LAUNCH("gemm_tc_kernel");
  return kOk;
}

}  // namespace

int *tc_gemm_status_word() { return gemm_status_word(); }

int tc_gemm(int prec, bool trans_a, bool trans_b, long long M, long long N, long long K,
            const float *a, const float *b, float *c, const float *bias, int act,
            cudaStream_t s) {
  if (prec != OWLGPU_PREC_BF16 && prec != OWLGPU_PREC_BF16X3) return kErrUnsupported;
  if (M == 0 || N == 0) return kOk;
  if (K == 0) return kErrUnsupported;  // the caller fills act(bias)
  const int kind = prec == OWLGPU_PREC_BF16X3 ? stage::K_BF16X3 : stage::K_BF16;
  const int parts = kind == stage::K_BF16X3 ? 2 : 1;
  GemmParams p{};
  p.a = a; p.b = b; p.bias = bias; p.act = act;
  p.M = M; p.N = N; p.K = K;
  // op(A) is M x K: stored [M][K] (k contiguous) or, transposed, [K][M]
  p.a_kmaj = trans_a ? 0 : 1;
  p.a_sm = trans_a ? 1 : K;
  p.a_sk = trans_a ? M : 1;
  // op(B) is K x N: stored [K][N] (n contiguous) or, transposed, [N][K]
  p.b_kmaj = trans_b ? 1 : 0;
  p.b_sn = trans_b ? K : 1;
  p.b_sk = trans_b ? 1 : N;
  p.BN = N >= 256 ? 256 : (int)std::max<long long>(16, (N + 15) / 16 * 16);
  p.a_bytes = (unsigned)(kBM * kBK * 2);
  p.b_bytes = (unsigned)(p.BN * kBK * 2);
  const size_t stage_bytes = (size_t)parts * (p.a_bytes + p.b_bytes);
  p.NS = (int)std::min<size_t>(4, (kSmemMax - 256) / stage_bytes);
  if (p.NS < 2) return kErrUnsupported;
  const long long mt = (M + kBM - 1) / kBM, nt = (N + p.BN - 1) / p.BN;
  const long long nkb = (K + kBK - 1) / kBK;
  // split the reduction so that about two waves of CTAs cover the GPU, each
  // split at least two k blocks deep
  long long splits = std::max<long long>(1, (2LL * num_sms() + mt * nt - 1) / (mt * nt));
  splits = std::min<long long>(splits, std::max<long long>(1, nkb / 2));
  splits = std::min<long long>(splits, 64);
  const long long kbs = (nkb + splits - 1) / splits;
  p.kps = kbs * kBK;
  p.splits = (int)((nkb + kbs - 1) / kbs);
  p.small_off = (unsigned)p.BN;
  p.tmem_cols = 32;
  while (p.tmem_cols < (unsigned)(parts * p.BN)) p.tmem_cols <<= 1;
  p.idesc = instr_desc(1u, (uint32_t)p.BN) | ((p.a_kmaj ? 0u : 1u) << 15) |
            ((p.b_kmaj ? 0u : 1u) << 16);
  p.spin_limit = wait_limit();
  p.status = gemm_status_word();
  if (!p.status) {
    set_error("gemm_tc: cannot locate device status word");
    return kErrCuda;
  }
  float *part = nullptr;
  if (p.splits > 1) {
    int rc = scratch_alloc((void **)&part, sizeof(float) * (size_t)p.splits * M * N, s);
    if (rc) return rc;
    p.c = part;
  } else {
    p.c = c;
  }
  const size_t smem = (size_t)p.NS * stage_bytes + (2 * p.NS + 2) * 8 + 16;
  const dim3 grid((unsigned)mt, (unsigned)nt, (unsigned)p.splits);
  int rc = kind == stage::K_BF16X3 ? launch<stage::K_BF16X3>(p, smem, grid, s)
                                   : launch<stage::K_BF16>(p, smem, grid, s);
  if (rc == kOk && p.splits > 1) {
    const long long n_all = M * N;
    const int blocks = (int)std::max<long long>(1, std::min<long long>((n_all + 255) / 256, 4 * 152));
    gemm_reduce<<<blocks, 256, 0, s>>>(part, c, bias, act, M, N, p.splits);
    cudaError_t e = cudaGetLastError();
    note_launch();
    if (e != cudaSuccess) rc = cuda_fail(e, "gemm_reduce");
  }
  if (part) scratch_free(part, s);
  return rc;
}

}  // namespace owlgpu
