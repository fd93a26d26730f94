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

// Operand A gathered from an array by non-overlapping windows (a
// convolution whose kernel equals its stride): the A element of pixel p and
// combined index tc = (tap, channel) is X[b][oc*KC + tcol][or*KR + tr]
// [od*KD + td][c], p = ((b*OC + oc)*OR + or)*OD + od over the window grid.
// Pixel counts and (tap, channel) counts are below 2^31 (checked on the
// host), so the decodes divide in 32 bits; the offset is formed in 64.
struct S2D {
  int on;
  unsigned C;            // channels of the array
  unsigned KC, KR, KD;   // window = stride
  unsigned OC, OR, OD;   // window grid
  long long IC, IR, ID;  // array extents
};

__device__ __forceinline__ long long s2d_off(const S2D &g, long long p, long long tc) {
  unsigned t = (unsigned)tc / g.C;
  const unsigned c = (unsigned)tc - t * g.C;
  const unsigned td = t % g.KD;
  t /= g.KD;
  const unsigned tr = t % g.KR, tcl = t / g.KR;
  unsigned q = (unsigned)p;
  const unsigned od = q % g.OD;
  q /= g.OD;
  const unsigned orr = q % g.OR;
  q /= g.OR;
  const unsigned oc = q % g.OC, b = q / g.OC;
  return ((((long long)b * g.IC + (long long)oc * g.KC + tcl) * g.IR +
           (long long)orr * g.KR + tr) * g.ID + (long long)od * g.KD + td) * g.C + c;
}

struct GemmParams {
  S2D s2d;  // operand A gathered by windows (s2d.on), else by its strides
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

// One operand's part of a stage: rows [row0, row0 + R) of k block
// [k0, k0 + kBK), zero outside the matrix.  Element (row, k) is at
// src[row*s_row + k] when kmaj (k contiguous), else at src[k*s_k + row], or
// where the window gather `g` puts it.  Slot sl (0 .. 8R-1) is one 16-byte
// destination and 8 contiguous source floats.
//   K-major: slot sl = chunk c (sl % 8) of row r (sl / 8), at
//   (c*(R+1) + r)*16: 8 consecutive lanes read one row's 256 contiguous
//   bytes, and the planes' stride of R+1 chunks (1 mod 8) puts the 8
//   chunks of a row in 8 different bank groups.
//   MN-major: slot sl = row chunk j (sl % (R/8)) at k (sl / (R/8)), at
//   (j*(kBK+1) + k)*16: consecutive lanes read consecutive row chunks of one
//   k (contiguous), the plane stride kBK+1 keeps them in distinct banks.
// Each warp-wide load therefore touches whole lines, not one line per lane.
struct Operand {
  const float *src;
  long long s_row, s_k, row0, rows;
  int kmaj, R;
  uint32_t dst;  // byte offset of the operand's hi part in the stage
};

__device__ __forceinline__ void load_slot(const Operand &o, int sl, long long k0, long long kend,
                                          const S2D &g, float (&v)[8], int &off) {
#pragma unroll
  for (int e = 0; e < 8; ++e) v[e] = 0.f;
  const float *p = nullptr;
  bool vec = false;
  if (o.kmaj) {
    const int c = sl & 7, r = sl >> 3;
    off = (int)o.dst + (c * (o.R + 1) + r) * 16;
    const long long row = o.row0 + r, k = k0 + 8 * c;
    if (row < o.rows && k < kend) {
      p = o.src + (g.on ? s2d_off(g, row, k) : row * o.s_row + k);
      vec = k + 8 <= kend;
      if (!vec)
        for (int e = 0; e < 8; ++e)
          if (k + e < kend) v[e] = __ldg(p + e);
    }
  } else {
    const int nj = o.R >> 3;
    const int kk = sl / nj, j = sl - kk * nj;
    off = (int)o.dst + (j * (kBK + 1) + kk) * 16;
    const long long k = k0 + kk, row = o.row0 + 8 * j;
    if (k < kend && row < o.rows) {
      p = o.src + (g.on ? s2d_off(g, k, row) : k * o.s_k + row);
      vec = row + 8 <= o.rows;
      if (!vec)
        for (int e = 0; e < 8; ++e)
          if (row + e < o.rows) v[e] = __ldg(p + e);
    }
  }
  if (vec) {
    if (((uintptr_t)p & 15) == 0) {
      const float4 x0 = __ldg(reinterpret_cast<const float4 *>(p));
      const float4 x1 = __ldg(reinterpret_cast<const float4 *>(p) + 1);
      v[0] = x0.x; v[1] = x0.y; v[2] = x0.z; v[3] = x0.w;
      v[4] = x1.x; v[5] = x1.y; v[6] = x1.z; v[7] = x1.w;
    } else {
#pragma unroll
      for (int e = 0; e < 8; ++e) v[e] = __ldg(p + e);
    }
  }
}

// A whole stage (both operands) in one round per thread: every load of the
// stage is issued first (up to kQ slots per thread, 2 x 16-byte loads
// each), then `ready()` waits for the stage's buffer to be free, then the
// values are converted and stored.  The loads' latency overlaps the wait.
// slots per thread per stage: (8*128 + 8*256) / 480 producer threads <= 7
constexpr int kQ = 7;
static_assert(kQ * kProducerThreads >= 8 * (kBM + 256), "a stage must fit one round");

// 8 floats in one 32-byte load (p 32-byte aligned), through the read-only
// path: one L1 wavefront per lane instead of two 16-byte loads' two.
__device__ __forceinline__ void ld8(const float *p, float (&v)[8]) {
  asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]),
                 "=f"(v[6]), "=f"(v[7])
               : "l"(p));
}

// A thread's slots, resolved once per tile: where slot q's 8 floats of the
// first k block are, how far they move per k block, and its destination.
// A slot whose row lies outside the matrix has base == nullptr (zeros).
struct Slots {
  const float *base[kQ];
  int off[kQ];
  long long step_a, step_b;  // per k block, operand A's slots and B's
};

__device__ __forceinline__ long long slot_step(const Operand &o) {
  return o.kmaj ? (long long)kBK : (long long)kBK * o.s_k;
}

__device__ __forceinline__ void slot_plan(const Operand &o, int sl, long long k_begin,
                                          const float *&base, int &off) {
  base = nullptr;
  if (o.kmaj) {
    const int c = sl & 7, r = sl >> 3;
    off = (int)o.dst + (c * (o.R + 1) + r) * 16;
    const long long row = o.row0 + r;
    if (row < o.rows) base = o.src + row * o.s_row + k_begin + 8 * c;
  } else {
    const int nj = o.R >> 3;
    const int kk = sl / nj, j = sl - kk * nj;
    off = (int)o.dst + (j * (kBK + 1) + kk) * 16;
    const long long row = o.row0 + 8 * j;
    if (row + 8 <= o.rows) base = o.src + (k_begin + kk) * o.s_k + row;
  }
}

// A whole stage (both operands) in one round per thread: every load of the
// stage is issued first (up to kQ slots per thread, 2 x 16-byte loads
// each), then `ready()` waits for the stage's buffer to be free, then the
// values are converted and stored.  The loads' latency overlaps the wait.
// `fast`: the k block lies wholly inside the matrix, the operands are read
// through their strides and every source is 16-byte aligned, so each slot
// is two vector loads at base + i*step; otherwise each slot is resolved in
// full (matrix edges, the window gather).
template <int KIND, class Ready>
__device__ __forceinline__ bool stage_round(uint8_t *stage, uint32_t lo_a, uint32_t lo_b,
                                            const Operand &A, const Operand &B, long long k0,
                                            long long kend, const S2D &g, int tid,
                                            const Slots &sp, bool fast, bool wide, long long i,
                                            Ready ready) {
  const int na = 8 * A.R, total = na + 8 * B.R;
  const S2D none{};
  float v[kQ][8];
  int off[kQ];
  if (fast) {
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
      const int sl = tid + q * kProducerThreads;
      off[q] = sl < total ? sp.off[q] : -1;
      if (off[q] >= 0 && sp.base[q]) {
        const float *src = sp.base[q] + i * (sl < na ? sp.step_a : sp.step_b);
        if (wide) {
          ld8(src, v[q]);
        } else {
          const float4 *p4 = reinterpret_cast<const float4 *>(src);
          const float4 x0 = __ldg(p4), x1 = __ldg(p4 + 1);
          v[q][0] = x0.x; v[q][1] = x0.y; v[q][2] = x0.z; v[q][3] = x0.w;
          v[q][4] = x1.x; v[q][5] = x1.y; v[q][6] = x1.z; v[q][7] = x1.w;
        }
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) v[q][e] = 0.f;
      }
    }
  } else {
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
      const int sl = tid + q * kProducerThreads;
      off[q] = -1;
      if (sl < na) {
        load_slot(A, sl, k0, kend, g, v[q], off[q]);
      } else if (sl < total) {
        load_slot(B, sl - na, k0, kend, none, v[q], off[q]);
      }
    }
  }
  if (!ready()) return false;
#pragma unroll
  for (int q = 0; q < kQ; ++q)
    if (off[q] >= 0) {
      const uint32_t lo = off[q] < (int)B.dst ? lo_a : lo_b;
      stage::put_chunk<KIND, 8>(stage + off[q], lo, v[q]);
    }
  return true;
}

template <int KIND>
__global__ void __launch_bounds__(kThreads, 1) gemm_tc_kernel(const __grid_constant__ GemmParams p) {
  constexpr int PARTS = (KIND == stage::K_BF16X3) ? 2 : 1;
  constexpr bool SEP = (KIND == stage::K_BF16X3);
  extern __shared__ __align__(1024) uint8_t smem[];
  // launched with launch_pdl: the operands may be the previous kernel's output
  asm volatile("griddepcontrol.wait;" ::: "memory");

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
    // the stage: A hi [, A lo], B hi [, B lo]
    const Operand A{p.a, p.a_sm, p.a_sk, m0, p.M, p.a_kmaj, kBM, 0u};
    const Operand B{p.b, p.b_sn, p.b_sk, n0, p.N, p.b_kmaj, p.BN, PARTS * p.a_bytes};
    Slots sp;
    const int na = 8 * kBM, total = na + 8 * p.BN;
    sp.step_a = slot_step(A);
    sp.step_b = slot_step(B);
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
      const int sl = tid + q * kProducerThreads;
      sp.base[q] = nullptr;
      sp.off[q] = -1;
      if (sl < na) slot_plan(A, sl, k_begin, sp.base[q], sp.off[q]);
      else if (sl < total) slot_plan(B, sl - na, k_begin, sp.base[q], sp.off[q]);
    }
    // plain strided operands whose rows start 16-byte aligned (the fast path)
    const bool aligned = !p.s2d.on && ((uintptr_t)p.a & 15) == 0 && ((uintptr_t)p.b & 15) == 0 &&
                         (p.a_kmaj ? p.a_sm % 4 == 0 : p.a_sk % 4 == 0) &&
                         (p.b_kmaj ? p.b_sn % 4 == 0 : p.b_sk % 4 == 0);
    // ... and 32-byte aligned: one 32-byte load per slot
    const bool wide = aligned && ((uintptr_t)p.a & 31) == 0 && ((uintptr_t)p.b & 31) == 0 &&
                      (p.a_kmaj ? p.a_sm % 8 == 0 : p.a_sk % 8 == 0) &&
                      (p.b_kmaj ? p.b_sn % 8 == 0 : p.b_sk % 8 == 0);
    for (int i = 0; i < nkb; ++i) {
      const int st = i % p.NS;
      uint8_t *stg = smem + (size_t)st * stage_bytes;
      const long long k0 = k_begin + (long long)i * kBK;
      const bool fast = aligned && k0 + kBK <= k_end;
      if (!stage_round<KIND>(stg, p.a_bytes, p.b_bytes, A, B, k0, k_end, p.s2d, tid, sp, fast,
                             wide, i,
                             [&] {
            return wait_bar(smem_u32(&empty[st]), (uint32_t)(((i / p.NS) & 1) ^ 1), abort_flag,
                            p.status, p.spin_limit);
          })) {
        staged = false;
        break;
      }
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
    // K-major: core matrices along k are (R+1)*16 bytes apart, along rows
    // 128; MN-major: along k 128 bytes apart, along rows (kBK+1)*16.  One
    // K = 16 step is two k chunks (K-major) or 16 k rows (MN-major), in
    // 16-byte units.
    const uint32_t a_lbo = p.a_kmaj ? (kBM + 1) * 16 : 128, a_sbo = p.a_kmaj ? 128 : (kBK + 1) * 16;
    const uint32_t b_lbo = p.b_kmaj ? (uint32_t)(p.BN + 1) * 16 : 128,
                   b_sbo = p.b_kmaj ? 128 : (kBK + 1) * 16;
    const uint32_t a_step = p.a_kmaj ? 2 * (kBM + 1) : 16,
                   b_step = p.b_kmaj ? 2 * (uint32_t)(p.BN + 1) : 16;
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
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
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
  cudaError_t e = launch_pdl(gemm_tc_kernel<KIND>, grid, dim3(kThreads), smem, s, p);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  note_tc_launch();
  return e == cudaSuccess ? kOk : cuda_fail(e, "gemm_tc_kernel");
}

}  // namespace

int *tc_gemm_status_word() { return gemm_status_word(); }

namespace {

// Tiles, pipeline depth and split of a GEMM whose operands `p` describes
// (a, b, strides, majorness, M, N, K, bias, act, s2d), then the launch and
// the fixed-order sum of the splits into c.
int gemm_run(int prec, GemmParams p, float *c, cudaStream_t s) {
  const long long M = p.M, N = p.N, K = p.K;
  const float *bias = p.bias;
  const int act = p.act;
  const int kind = prec == OWLGPU_PREC_BF16X3 ? stage::K_BF16X3 : stage::K_BF16;
  const int parts = kind == stage::K_BF16X3 ? 2 : 1;
  p.BN = N >= 256 ? 256 : (int)std::max<long long>(16, (N + 15) / 16 * 16);
  // one padded plane per k chunk (K-major) or per row chunk (MN-major)
  p.a_bytes = (unsigned)(p.a_kmaj ? 8 * (kBM + 1) * 16 : (kBM / 8) * (kBK + 1) * 16);
  p.b_bytes = (unsigned)(p.b_kmaj ? 8 * (p.BN + 1) * 16 : (p.BN / 8) * (kBK + 1) * 16);
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
    cudaError_t e = launch_pdl(gemm_reduce, dim3(blocks), dim3(256), 0, s, (const float *)part,
                               c, bias, act, M, N, p.splits);
    if (e == cudaSuccess) e = cudaGetLastError();
    note_launch();
    if (e != cudaSuccess) rc = cuda_fail(e, "gemm_reduce");
  }
  if (part) scratch_free(part, s);
  return rc;
}

}  // namespace

int tc_gemm(int prec, bool trans_a, bool trans_b, long long M, long long N, long long K,
            const float *a, const float *b, float *c, const float *bias, int act,
            cudaStream_t s) {
  if (prec != OWLGPU_PREC_BF16 && prec != OWLGPU_PREC_BF16X3) return kErrUnsupported;
  if (M == 0 || N == 0) return kOk;
  if (K == 0) return kErrUnsupported;  // the caller fills act(bias)
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
  return gemm_run(prec, p, c, s);
}

// A convolution whose kernel equals its stride, without dilation or
// padding, its windows tiling the input exactly (a transpose convolution's
// backward passes with kernel = stride, patchify layers): forward and
// backward_kernel are GEMMs over the windows, with operand A gathered from
// the activation window by window (no im2col copy).
//   forward:         y[p][co]        = sum_(t,ci) X[win(p) + t][ci] * W[t][ci][co]
//   backward_kernel: dW[(t,ci)][co]  = sum_p      X[win(p) + t][ci] * dY[p][co]
// Channel chunks of 8 must not straddle taps (Ci % 8 == 0).  TF32 runs the
// split-BF16 GEMM, which is at least as accurate.
int tc_conv_s2d(int prec, bool bwd_kernel, const ConvGeom &g, const float *x,
                const float *w_or_dy, float *out, const float *bias, int act, cudaStream_t s) {
  if (prec == OWLGPU_PREC_TF32) prec = OWLGPU_PREC_BF16X3;
  if (prec != OWLGPU_PREC_BF16 && prec != OWLGPU_PREC_BF16X3) return kErrUnsupported;
  const bool win = g.KC == g.sc && g.KR == g.sr && g.KD == g.sd && g.dc == 1 && g.dr == 1 &&
                   g.dd == 1 && g.pc == 0 && g.pr == 0 && g.pd == 0 && g.IC == g.OC * g.sc &&
                   g.IR == g.OR * g.sr && g.ID == g.OD * g.sd && g.taps() > 1 && g.Ci % 8 == 0;
  if (!win) return kErrUnsupported;
  if (g.out_pixels() == 0 || g.Ci == 0 || g.Co == 0) return kErrUnsupported;
  if (g.out_pixels() >= (1LL << 31) || g.taps() * g.Ci >= (1LL << 31)) return kErrUnsupported;
  GemmParams p{};
  p.s2d.on = 1;
  p.s2d.C = (unsigned)g.Ci;
  p.s2d.KC = (unsigned)g.KC; p.s2d.KR = (unsigned)g.KR; p.s2d.KD = (unsigned)g.KD;
  p.s2d.OC = (unsigned)g.OC; p.s2d.OR = (unsigned)g.OR; p.s2d.OD = (unsigned)g.OD;
  p.s2d.IC = g.IC; p.s2d.IR = g.IR; p.s2d.ID = g.ID;
  p.a = x;
  p.b = w_or_dy;
  p.N = g.Co;
  // B is [K][N] row-major in both: W[(t,ci)][co] or dY[p][co]
  p.b_kmaj = 0; p.b_sn = 1; p.b_sk = g.Co;
  if (!bwd_kernel) {
    p.M = g.out_pixels(); p.K = g.taps() * g.Ci;
    p.a_kmaj = 1;  // rows = pixels, k = (tap, channel), 8 channels contiguous
    p.bias = bias; p.act = act;
  } else {
    p.M = g.taps() * g.Ci; p.K = g.out_pixels();
    p.a_kmaj = 0;  // rows = (tap, channel), 8 contiguous; k = pixels
  }
  return gemm_run(prec, p, out, s);
}

}  // namespace owlgpu
