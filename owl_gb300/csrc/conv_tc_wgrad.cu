// conv_tc_wgrad.cu -- tcgen05 backward-kernel (weight gradient) for float32
// data in BF16 or split-BF16 precision (a TF32 request runs split-BF16),
// strides up to 8, any dilation, 2-D/3-D.
//
//   dW[t][ci][co] = sum over output pixels p of X[p + off(t)][ci] * dY[p][co]
//
// Per tap this is a GEMM with M = ci (128 per MMA), N = co (BN <= 256), and the
// reduction K running over output pixels.  Both operands are staged from the
// float32 activations by producer warps in the same [16-byte channel chunk]
// [pixel][16 B] layout as the forward kernel's halo.  Read MN-major, 8
// consecutive pixels x 8 channels of that layout form one core matrix, so
// every tap of a tap group reads the same X halo through a shifted descriptor
// and all of them share one staged dY tile.  Taps are grouped by phase
// (k*d mod s per dimension), so a strided convolution's halo holds only the
// input rows and columns its group reads: a quarter of the footprint at
// stride 2 in 2-D.
//
// Work split: a CTA owns (tap group, ci block, co block, pixel range).  It
// accumulates the group's taps in TMEM (TG * BN columns) over all the pixel
// tiles of its range, then writes the partial dW of its range.  A second
// kernel sums the ranges in a fixed order, so the result is deterministic.
// CTAs that share a pixel range are launched next to each other, so the
// activations they re-read come from L2.
#include <cuda_bf16.h>

#include <algorithm>

#include "../../include/owlgpu.h"
#include "common.cuh"
#include "tc_ptx.cuh"
#include "tc_stage.cuh"

namespace owlgpu {
namespace {

using namespace ptx;

// Warp roles.  The accumulator is drained once per CTA, after the last
// pixel tile, so every warp but the MMA issuer (warp 0) stages operands;
// warps 12-15, one per TMEM lane quadrant, then drain the accumulator.
// (Measured on GB300: 15 producer warps beat 9 or 12 here even though three
// of them share the MMA warp's scheduler.)
constexpr int kWarps = 16;
constexpr int kThreads = kWarps * 32;
constexpr int kMmaWarp = 0;
constexpr int kEpiWarp0 = 12;
constexpr int kProducerWarps = kWarps - 1;
constexpr int kProducerThreads = kProducerWarps * 32;
__device__ __forceinline__ int producer_index(int warp) { return warp - 1; }
constexpr int kSmemMax = 232448;
// Taps are grouped through a table in the launch parameters when the
// convolution is strided (and, up to this many taps, always).
constexpr int kMaxOrderedTaps = 256;
constexpr long long kSpinLimit = 4000000000LL;

enum Kind { K_BF16 = 0, K_TF32 = 1, K_BF16X3 = 2 };

struct WgParams {
  const float *x, *dy;
  float *out;
  int *status;
  int B, IW, IU, IV, OW, OU, OV, KW, KU, KV, dw, du, dv, pw, pu, pv, sw, su, sv;
  long long xsb, xsw, xsu, xsv, ysb, ysw, ysu, ysv;
  int Ci, Co, T, TG, n_tg, BN, n_nb, n_mb, R;
  int TU, TP;             // reduction tile: TU output rows (u) x 8 columns (v) = TP pixels
  int YPS;                // dY plane stride in pixels: TP + 1, so that the 16-byte chunks
                          // of one pixel fall in different shared-memory banks
  int u_tiles, v_tiles;
  long long total_tiles, tiles_per_range;
  int PS;                 // X halo plane stride in pixels (max over groups)
  unsigned x_bytes, y_bytes;  // per stage, per precision part
  int NS;
  unsigned idesc, tmem_cols;
  unsigned small_off;  // BF16X3: TMEM column of the cross-term accumulators (TG * BN)
  int vec_x, vec_y;
  // Tap groups.  ordered: group g holds taps tap_order[gstart[g] ..
  // gstart[g+1]); else group g holds taps g*TG .. min(T, (g+1)*TG) - 1.
  // Every group is phase-uniform: all its taps have the same k*d mod s in
  // each dimension, so its X halo needs only input rows and columns of
  // that phase (every s-th one).
  long long spin_limit;  // cycles a pipeline wait polls before the CTA gives up
  int ordered;
  unsigned short tap_order[kMaxOrderedTaps];
  unsigned short gstart[kMaxOrderedTaps + 1];
};

__device__ int g_tc_status_wg;

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

template <int KIND>
__global__ void __launch_bounds__(kThreads, 1) wgrad_tc_kernel(const __grid_constant__ WgParams p) {
  constexpr int EB = (KIND == K_TF32) ? 4 : 2;
  constexpr int EPC = 16 / EB;
  constexpr int PARTS = (KIND == K_BF16X3) ? 2 : 1;
  constexpr int XPL = 128 * EB / 16;  // planes for 128 input channels
  constexpr int KSTEP_PIX = 32 / EB;  // pixels per MMA (K = 16 bf16 / 8 tf32)
  // BF16X3: the cross terms (hi*lo + lo*hi) accumulate apart from the hi*hi
  // sums and are added in the epilogue.  The tensor core rounds its FP32
  // accumulator toward zero after every MMA; with all three MMAs of a K step
  // in one accumulator that rounding is three times that of the hi*hi sums.
  constexpr bool SEP = (KIND == K_BF16X3);
  extern __shared__ __align__(1024) uint8_t smem[];
  // a programmatic dependent of the work before it: wait for that work (X
  // and dY may be its output) before any global access
  asm volatile("griddepcontrol.wait;" ::: "memory");

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int YPL = p.BN * EB / 16;

  // ---- work unit of this CTA ----
  long long u = blockIdx.x;
  const int tg = (int)(u % p.n_tg); u /= p.n_tg;
  const int nb = (int)(u % p.n_nb); u /= p.n_nb;
  const int mb = (int)(u % p.n_mb);
  const int r = (int)(u / p.n_mb);
  const long long t_begin = (long long)r * p.tiles_per_range;
  const long long t_end = min(p.total_tiles, t_begin + p.tiles_per_range);
  const int gbeg = p.ordered ? (int)p.gstart[tg] : tg * p.TG;
  const int ntap = p.ordered ? (int)p.gstart[tg + 1] - gbeg : min(p.TG, p.T - gbeg);
  auto tap_of = [&](int i) { return p.ordered ? (int)p.tap_order[gbeg + i] : gbeg + i; };

  // bounding box of this group's tap offsets -> halo extents
  int minw = 1 << 30, minu = 1 << 30, minv = 1 << 30, maxw = -1, maxu = -1, maxv = -1;
  for (int i = 0; i < ntap; ++i) {
    const int t = tap_of(i);
    const int kv = t % p.KV, ku = (t / p.KV) % p.KU, kw = t / (p.KV * p.KU);
    minw = min(minw, kw * p.dw); maxw = max(maxw, kw * p.dw);
    minu = min(minu, ku * p.du); maxu = max(maxu, ku * p.du);
    minv = min(minv, kv * p.dv); maxv = max(maxv, kv * p.dv);
  }
  // X halo of a phase-uniform group: input rows and columns of the group's
  // phase only, so halo row (hw, hu) is input (minw + hw*sw, minu + hu*su)
  // relative to the tile origin, and its HVR pixels are every sv-th input
  // column: 8 consecutive output columns are 8 consecutive stored pixels.
  const int HW = (maxw - minw) / p.sw + 1, HU = p.TU + (maxu - minu) / p.su;
  const int HVR = 8 + (maxv - minv) / p.sv;
  // X halo rows; when both operand tiles have at most one row per producer
  // warp, each warp stages its X row and dY row together in a single pass
  const int xrows = HW * HU;
  const bool paired = xrows <= kProducerWarps && p.TU <= kProducerWarps &&
                      HVR * XPL <= 32 * 5 && 8 * YPL <= 32 * 4;

  uint8_t *xs = smem;
  uint8_t *ys = smem + (size_t)p.NS * PARTS * p.x_bytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(ys + (size_t)p.NS * PARTS * p.y_bytes);
  uint64_t *full = bars;
  uint64_t *empty = full + p.NS;
  uint64_t *acc_full = empty + p.NS;
  uint64_t *drain = acc_full + 1;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  uint32_t *tap_off = tmem_slot + 2;  // per-tap start pixel in the X halo (16-byte units)

  for (int i = threadIdx.x; i < ntap; i += blockDim.x) {
    const int tt = tap_of(i);
    const int kv = tt % p.KV, ku = (tt / p.KV) % p.KU, kw = tt / (p.KV * p.KU);
    tap_off[i] = (uint32_t)((((kw * p.dw - minw) / p.sw) * HU + (ku * p.du - minu) / p.su) * HVR +
                            (kv * p.dv - minv) / p.sv);
  }

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

  const int pidx = producer_index(warp);
  if (warp != kMmaWarp) {
    // ===================== producers: X halo + dY tile =====================
    bool staged = true;
    long long k = 0;
    for (long long t = t_begin; t < t_end; ++t, ++k) {
      long long q = t;
      const int v0 = (int)(q % p.v_tiles) * 8; q /= p.v_tiles;
      const int u0 = (int)(q % p.u_tiles) * p.TU; q /= p.u_tiles;
      const int ow = (int)(q % p.OW);
      const int b = (int)(q / p.OW);
      const int st = (int)(k % p.NS);
      if (!wait_bar(smem_u32(&empty[st]), (uint32_t)(((k / p.NS) & 1) ^ 1), abort_flag,
                    p.status, p.spin_limit)) {
        staged = false;
        break;
      }
      uint8_t *xd = xs + (size_t)st * PARTS * p.x_bytes;
      uint8_t *yd = ys + (size_t)st * PARTS * p.y_bytes;
      // X halo: rows (w, u) of HVR pixels x 128 channels of ci block mb;
      // dY tile: TU rows (u) of 8 output pixels x BN channels of co block nb.
      const int xcb = mb * 128, ycb = nb * p.BN;
      auto xrow = [&](int r) {
        const int hu = r % HU, hw = r / HU;
        const int iw = ow * p.sw - p.pw + minw + hw * p.sw;
        const int iu = u0 * p.su - p.pu + minu + hu * p.su;
        const int ivs = v0 * p.sv - p.pv + minv;
        stage::Row row;
        row.ok = iw >= 0 && iw < p.IW && iu >= 0 && iu < p.IU;
        row.rowp = p.x + ((long long)b * p.xsb + (long long)iw * p.xsw + (long long)iu * p.xsu +
                          (long long)ivs * p.xsv) * p.Ci + xcb;
        row.pstep = (long long)p.sv * p.xsv * p.Ci;
        row.vfirst = ivs;
        row.vstride = p.sv;
        row.vlim = p.IV;
        return row;
      };
      auto yrow = [&](int r) {
        const int ou = u0 + r;
        stage::Row row;
        row.ok = ou < p.OU;
        row.rowp = p.dy + ((long long)b * p.ysb + (long long)ow * p.ysw + (long long)ou * p.ysu +
                           (long long)v0 * p.ysv) * p.Co + ycb;
        row.pstep = p.ysv * p.Co;
        row.vfirst = v0;
        row.vstride = 1;
        row.vlim = p.OV;
        return row;
      };
      if (paired) {
        // at most one row of each per warp: both rows in one pass
        stage::RowSet sx{xd, p.x_bytes, (uint32_t)p.PS * 16, xrows, HVR, XPL, p.Ci - xcb};
        stage::RowSet sy{yd, p.y_bytes, (uint32_t)p.YPS * 16, p.TU, 8, YPL, p.Co - ycb};
        stage::stage_rows2<KIND, EPC, 5, 4>(sx, xrow, sy, yrow, min(p.vec_x, p.vec_y),
                                            pidx, kProducerWarps, lane);
      } else {
        stage::stage_rows<KIND, EPC, 6>(xd, p.x_bytes, (uint32_t)p.PS * 16, xrows, HVR, XPL,
                                        p.Ci - xcb, p.vec_x, pidx, kProducerWarps, lane,
                                        xrow);
        stage::stage_rows<KIND, EPC, 4>(yd, p.y_bytes, (uint32_t)p.YPS * 16, p.TU, 8, YPL,
                                        p.Co - ycb, p.vec_y, pidx, kProducerWarps, lane,
                                        yrow);
      }
      fence_proxy_async();
      mbar_arrive(smem_u32(&full[st]));
    }
    if (staged && warp >= kEpiWarp0) {
      // ===================== epilogue: TMEM -> partial dW =====================
      const int q = warp & 3;
      const int ci = mb * 128 + q * 32 + lane;
      if (wait_bar(smem_u32(acc_full), 0, abort_flag, p.status, p.spin_limit)) {
        tc_fence_after();
        for (int i = 0; i < ntap; ++i) {
          const int tt = tap_of(i);
          float *out = p.out + (((long long)r * p.T + tt) * p.Ci + ci) * p.Co + nb * p.BN;
          const uint32_t tcol = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(i * p.BN);
          for (int c0 = 0; c0 < p.BN; c0 += 16) {
            uint32_t rr[16];
            tmem_ld16(tcol + (uint32_t)c0, rr);
            if (SEP) {
              uint32_t r2[16];
              tmem_ld16(tcol + p.small_off + (uint32_t)c0, r2);
              tmem_ld_wait();
#pragma unroll
              for (int e = 0; e < 16; ++e)
                rr[e] = __float_as_uint(__uint_as_float(rr[e]) + __uint_as_float(r2[e]));
            } else {
              tmem_ld_wait();
            }
            if (ci < p.Ci) {
              const int n0 = nb * p.BN + c0;
              if (p.vec_y && n0 + 16 <= p.Co && ((uintptr_t)(out + c0) % 16 == 0)) {
#pragma unroll
                for (int e = 0; e < 16; e += 4)
                  *reinterpret_cast<float4 *>(out + c0 + e) =
                      make_float4(__uint_as_float(rr[e]), __uint_as_float(rr[e + 1]),
                                  __uint_as_float(rr[e + 2]), __uint_as_float(rr[e + 3]));
              } else {
#pragma unroll
                for (int e = 0; e < 16; ++e)
                  if (n0 + e < p.Co) out[c0 + e] = __uint_as_float(rr[e]);
              }
            }
          }
        }
        tc_fence_before();
      }
    }
  } else {
    // ===================== MMA issuer =====================
    if (lane == 0) {
      const uint32_t x0 = smem_u32(xs), y0 = smem_u32(ys);
      const uint32_t a_lbo = (uint32_t)HVR * 16, a_sbo = (uint32_t)p.PS * 16;
      const uint32_t b_lbo = 128, b_sbo = (uint32_t)p.YPS * 16;
      const uint32_t xlo16 = p.x_bytes >> 4, ylo16 = p.y_bytes >> 4;
      // per K step: 16 pixels = two halo rows further into the X halo, 16
      // pixels further into the dY tile (16-byte units)
      const uint32_t xk16 = (uint32_t)(KSTEP_PIX / 8) * (uint32_t)HVR;
      const int nks = p.TP / KSTEP_PIX;
      // up to four taps' A offsets in registers (the common tap groups)
      const bool few = ntap <= 4;
      uint32_t to[4], dc[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        to[i] = i < ntap ? tap_off[i] : 0u;
        dc[i] = tmem_base + (uint32_t)(i * p.BN);
      }
      int st = 0;
      uint32_t ph = 0;
      uint32_t acc = 0;
      bool ok = true;
      for (long long t = t_begin; t < t_end; ++t) {
        if (!wait_bar(smem_u32(&full[st]), ph, abort_flag, p.status, p.spin_limit)) {
          ok = false;
          break;
        }
        tc_fence_after();
        // descriptors advance by adds of 16-byte units (start-address field)
        const uint64_t xd_st = smem_desc(x0 + (uint32_t)st * PARTS * p.x_bytes, a_lbo, a_sbo);
        const uint64_t yd_st = smem_desc(y0 + (uint32_t)st * PARTS * p.y_bytes, b_lbo, b_sbo);
        for (int s = 0; s < nks; ++s) {
          const uint64_t bd = yd_st + (uint64_t)(s * KSTEP_PIX);
          const uint64_t xs_ = xd_st + (uint64_t)(s * xk16);
          if (few) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              if (i < ntap) {
                const uint64_t ad = xs_ + (uint64_t)to[i];
                if (KIND == K_TF32) {
                  mma_tf32(dc[i], ad, bd, p.idesc, acc);
                } else {
                  mma_bf16(dc[i], ad, bd, p.idesc, acc);
                  if (KIND == K_BF16X3) {
                    mma_bf16(dc[i] + p.small_off, ad, bd + (uint64_t)ylo16, p.idesc, acc);
                    mma_bf16(dc[i] + p.small_off, ad + (uint64_t)xlo16, bd, p.idesc, 1);
                  }
                }
              }
            }
          } else {
            for (int i = 0; i < ntap; ++i) {
              const uint64_t ad = xs_ + (uint64_t)tap_off[i];
              const uint32_t d = tmem_base + (uint32_t)(i * p.BN);
              if (KIND == K_TF32) {
                mma_tf32(d, ad, bd, p.idesc, acc);
              } else {
                mma_bf16(d, ad, bd, p.idesc, acc);
                if (KIND == K_BF16X3) {
                  mma_bf16(d + p.small_off, ad, bd + (uint64_t)ylo16, p.idesc, acc);
                  mma_bf16(d + p.small_off, ad + (uint64_t)xlo16, bd, p.idesc, 1);
                }
              }
            }
          }
          acc = 1;
        }
        mma_commit(smem_u32(&empty[st]));
        if (++st == p.NS) { st = 0; ph ^= 1; }
      }
      if (ok) mma_commit(smem_u32(acc_full));
      mma_commit(smem_u32(drain));
      long long t0 = clock64();
      while (!mbar_try_wait(smem_u32(drain), 0) && clock64() - t0 < kSpinLimit) {
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    tmem_dealloc(tmem_base, p.tmem_cols);
  }
}

// out[i] = sum_r part[r][i] in increasing r (deterministic).  Each thread
// sums four consecutive elements and issues the loads of 16 partials before
// adding them, in order, so the sum is the same as one add at a time while
// 16 loads are in flight.
__global__ void wgrad_reduce(const float *__restrict__ part, float *__restrict__ out, long long n,
                             int R, int vec) {
  // a programmatic dependent of the kernel that wrote the partials
  asm volatile("griddepcontrol.wait;" ::: "memory");
  // vec: n % 4 == 0 and `out` 16-byte aligned (the partials always are)
  const long long n4 = vec ? n / 4 : 0;
  const float4 *p4 = reinterpret_cast<const float4 *>(part);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
       i += (long long)gridDim.x * blockDim.x) {
    float4 s = __ldg(p4 + i);
    int r = 1;
    for (; r + 16 <= R; r += 16) {
      float4 v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = __ldg(p4 + (long long)(r + q) * n4 + i);
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        s.x += v[q].x; s.y += v[q].y; s.z += v[q].z; s.w += v[q].w;
      }
    }
    for (; r < R; ++r) {
      const float4 v = __ldg(p4 + (long long)r * n4 + i);
      s.x += v.x; s.y += v.y; s.z += v.z; s.w += v.w;
    }
    reinterpret_cast<float4 *>(out)[i] = s;
  }
  for (long long i = n4 * 4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float s = part[i];
    for (int r = 1; r < R; ++r) s += part[(long long)r * n + i];
    out[i] = s;
  }
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 148;
}

int *status_word() {
  static int *p[64] = {nullptr};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return nullptr;
  if (!p[dev]) {
    void *q = nullptr;
    if (cudaGetSymbolAddress(&q, g_tc_status_wg) != cudaSuccess) return nullptr;
    p[dev] = static_cast<int *>(q);
  }
  return p[dev];
}

template <int KIND>
int launch(const WgParams &p, size_t smem, int grid, cudaStream_t s) {
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    OWL_CUDA(cudaFuncSetAttribute(wgrad_tc_kernel<KIND>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemMax));
    attr[dev] = true;
  }
  cudaError_t e = launch_pdl(wgrad_tc_kernel<KIND>, dim3(grid), dim3(kThreads), smem, s, p);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  note_tc_launch();
  if (e != cudaSuccess) return cuda_fail(e, "wgrad_tc_kernel");
  return kOk;
}

}  // namespace

int *tc_wgrad_status_word() { return status_word(); }

// out[i] = sum_r part[r][i] for r = 0 .. R-1 in order (deterministic).
int sum_partials_f32(const float *part, float *out, long long n, int R, cudaStream_t s) {
  if (n <= 0) return kOk;
  const bool v4 = n % 4 == 0 && (uintptr_t)out % 16 == 0 && (uintptr_t)part % 16 == 0;
  const long long work = v4 ? n / 4 : n;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((work + 127) / 128, 8 * 152));
  cudaError_t e = launch_pdl(wgrad_reduce, dim3(blocks), dim3(128), 0, s, part, out, n, R,
                             v4 ? 1 : 0);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  if (e != cudaSuccess) return cuda_fail(e, "wgrad_reduce");
  return kOk;
}

int tc_conv_bwd_kernel(int prec, const ConvGeom &g, const float *x, float *dw, const float *dy,
                       cudaStream_t s) {
  if (g.sc > 8 || g.sr > 8 || g.sd > 8) return kErrUnsupported;
  // The weight gradient reads both operands MN-major, which the TF32 MMA
  // kind does not accept here; a TF32 request runs the split-BF16 kernel,
  // whose error (~1e-5) is below TF32's (~1e-3).
  const int kind = (prec == OWLGPU_PREC_TF32 || prec == OWLGPU_PREC_BF16X3) ? K_BF16X3 : K_BF16;
  const int EB = kind == K_TF32 ? 4 : 2;
  const int parts = kind == K_BF16X3 ? 2 : 1;
  if (g.Ci == 0 || g.Co == 0 || g.taps() == 0) return kErrUnsupported;
  if (g.out_pixels() == 0) return kErrUnsupported;
  WgParams p{};
  p.x = x; p.dy = dy;
  p.B = (int)g.B;
  p.Ci = (int)g.Ci; p.Co = (int)g.Co;
  const bool flat = (g.ID == 1 && g.OD == 1 && g.KD == 1);
  if (flat) {
    p.IW = 1; p.IU = (int)g.IC; p.IV = (int)g.IR; p.OW = 1; p.OU = (int)g.OC; p.OV = (int)g.OR;
    p.KW = 1; p.KU = (int)g.KC; p.KV = (int)g.KR; p.dw = 1; p.du = g.dc; p.dv = g.dr;
    p.pw = 0; p.pu = g.pc; p.pv = g.pr;
    p.sw = 1; p.su = g.sc; p.sv = g.sr;
    p.xsw = 1; p.xsu = g.IR; p.xsv = 1; p.ysw = 1; p.ysu = g.OR; p.ysv = 1;
  } else {
    p.IW = (int)g.IC; p.IU = (int)g.IR; p.IV = (int)g.ID;
    p.OW = (int)g.OC; p.OU = (int)g.OR; p.OV = (int)g.OD;
    p.KW = (int)g.KC; p.KU = (int)g.KR; p.KV = (int)g.KD;
    p.dw = g.dc; p.du = g.dr; p.dv = g.dd; p.pw = g.pc; p.pu = g.pr; p.pv = g.pd;
    p.sw = g.sc; p.su = g.sr; p.sv = g.sd;
    p.xsw = g.IR * g.ID; p.xsu = g.ID; p.xsv = 1;
    p.ysw = g.OR * g.OD; p.ysu = g.OD; p.ysv = 1;
  }
  p.xsb = g.IC * g.IR * g.ID;
  p.ysb = g.OC * g.OR * g.OD;
  p.T = (int)g.taps();
  p.n_mb = (p.Ci + 127) / 128;
  // Tap order: taps sorted by phase class (k*d mod s in each dimension), in
  // tap order within a class, so that every group of consecutive taps of a
  // class reads only input rows and columns of one phase.  Unstrided
  // convolutions have a single class (the identity order).
  const bool strided = p.sw > 1 || p.su > 1 || p.sv > 1;
  if (strided && p.T > kMaxOrderedTaps) return kErrUnsupported;
  p.ordered = p.T <= kMaxOrderedTaps;
  int order[kMaxOrderedTaps], cls_begin[kMaxOrderedTaps + 1], n_cls = 0;
  if (p.ordered) {
    auto phase = [&](int t) {
      const int kv = t % p.KV, ku = (t / p.KV) % p.KU, kw = t / (p.KV * p.KU);
      return ((kw * p.dw % p.sw) * p.su + ku * p.du % p.su) * p.sv + kv * p.dv % p.sv;
    };
    for (int t = 0; t < p.T; ++t) order[t] = t;
    std::stable_sort(order, order + p.T, [&](int a, int b) { return phase(a) < phase(b); });
    for (int i = 0; i < p.T; ++i)
      if (i == 0 || phase(order[i]) != phase(order[i - 1])) cls_begin[n_cls++] = i;
    cls_begin[n_cls] = p.T;
    for (int i = 0; i < p.T; ++i) p.tap_order[i] = (unsigned short)order[i];
  }
  // Groups of at most tg taps: each class split into the fewest groups,
  // sizes as even as possible.  Returns the number of groups and fills
  // gstart (ordered) or sets the contiguous split (unordered).
  auto make_groups = [&](int tg) {
    if (!p.ordered) {
      const int n = (p.T + tg - 1) / tg;
      p.TG = (p.T + n - 1) / n;
      return (p.T + p.TG - 1) / p.TG;
    }
    int n = 0, widest = 0;
    for (int c = 0; c < n_cls; ++c) {
      const int nc = cls_begin[c + 1] - cls_begin[c];
      const int ng = (nc + tg - 1) / tg;
      for (int g = 0, at = cls_begin[c]; g < ng; ++g) {
        const int sz = nc / ng + (g < nc % ng ? 1 : 0);
        p.gstart[n++] = (unsigned short)at;
        at += sz;
        widest = std::max(widest, sz);
      }
    }
    p.gstart[n] = (unsigned short)p.T;
    p.TG = widest;
    return n;
  };
  // Halo pixels of the largest group for tile height tu.
  auto max_halo = [&](int tu) {
    int maxHP = 0;
    for (int gi = 0; gi < p.n_tg; ++gi) {
      const int b0 = p.ordered ? p.gstart[gi] : gi * p.TG;
      const int b1 = p.ordered ? p.gstart[gi + 1] : std::min(p.T, b0 + p.TG);
      int mnw = 1 << 30, mnu = 1 << 30, mnv = 1 << 30, mxw = -1, mxu = -1, mxv = -1;
      for (int i = b0; i < b1; ++i) {
        const int t = p.ordered ? p.tap_order[i] : i;
        const int kv = t % p.KV, ku = (t / p.KV) % p.KU, kw = t / (p.KV * p.KU);
        mnw = std::min(mnw, kw * p.dw); mxw = std::max(mxw, kw * p.dw);
        mnu = std::min(mnu, ku * p.du); mxu = std::max(mxu, ku * p.du);
        mnv = std::min(mnv, kv * p.dv); mxv = std::max(mxv, kv * p.dv);
      }
      maxHP = std::max(maxHP, ((mxw - mnw) / p.sw + 1) * (tu + (mxu - mnu) / p.su) *
                                  (8 + (mxv - mnv) / p.sv));
    }
    return maxHP;
  };

  // Plan: BN (co block), TG (taps per CTA, TG*BN <= 512 TMEM columns, or
  // 2*TG*BN with split-BF16's separate cross-term accumulators), NS = 2.
  // Tile height TU (even, so that TU*8 pixels fill whole 16-pixel K steps),
  // tried in order of estimated cost: rows staged including padding plus a
  // fixed per-tile cost of about four rows; a tile taller than the number of
  // producer warps needs a second staging pass and ranks last.
  int tus[8], ntu = 0;
  {
    int cand[8] = {14, 12, 10, 16, 8, 6, 4, 2}, waste[8];
    for (int i = 0; i < 8; ++i) {
      waste[i] = (p.OU + cand[i] - 1) / cand[i] * (cand[i] + 4);
      if (cand[i] > kProducerWarps) waste[i] += 1 << 20;
    }
    bool used[8] = {false};
    for (int k = 0; k < 8; ++k) {
      int best = -1;
      for (int i = 0; i < 8; ++i)
        if (!used[i] && (best < 0 || waste[i] < waste[best] ||
                         (waste[i] == waste[best] && cand[i] > cand[best])))
          best = i;
      used[best] = true;
      tus[ntu++] = cand[best];
    }
  }
  // Widest output-channel block first (it is the MMA's N: narrow blocks waste
  // the tensor core), then the cheapest tile height, then the fewest tap
  // groups whose two stages of X halo + dY tile fit shared memory.
  bool planned = false;
  for (int bn : {256, 128, 64, 32, 16}) {
    if (planned) break;
    p.BN = std::min(bn, (p.Co + 15) / 16 * 16);
    const int tg_max = std::min(p.T, std::min(16, 512 / (parts * p.BN)));
    if (tg_max < 1) continue;
    for (int ti = 0; ti < ntu && !planned; ++ti) {
      const int tu = tus[ti];
      p.TU = tu;
      p.TP = tu * 8;
      p.YPS = p.TP + 1;
      int last_n = -1;
      for (int tg = tg_max; tg >= 1 && !planned; --tg) {
        p.n_tg = make_groups(tg);
        if (p.n_tg == last_n) continue;
        last_n = p.n_tg;
        const int maxHP = max_halo(tu);
        p.PS = maxHP + (((1 - maxHP) % 8) + 8) % 8;
        if (p.PS >= 16384) continue;
        p.x_bytes = (unsigned)(128 * EB / 16) * (unsigned)p.PS * 16u;
        p.y_bytes = (unsigned)(p.BN * EB / 16) * (unsigned)p.YPS * 16u;
        p.NS = 2;
        const size_t need = (size_t)p.NS * parts * (p.x_bytes + p.y_bytes) + 256;
        if (need <= (size_t)kSmemMax) planned = true;
      }
    }
  }
  if (!planned) return kErrUnsupported;
  p.u_tiles = (p.OU + p.TU - 1) / p.TU;
  p.v_tiles = (p.OV + 7) / 8;
  p.total_tiles = (long long)p.B * p.OW * p.u_tiles * p.v_tiles;
  p.n_nb = (p.Co + p.BN - 1) / p.BN;
  p.small_off = (unsigned)(p.TG * p.BN);
  p.tmem_cols = 32;
  while (p.tmem_cols < (unsigned)(parts * p.TG * p.BN)) p.tmem_cols <<= 1;
  // pixel ranges: enough CTAs to fill the GPU once
  const long long units = (long long)p.n_tg * p.n_nb * p.n_mb;
  const int sms = sm_count();
  long long R = std::max<long long>(1, sms / std::max<long long>(1, units));
  R = std::min<long long>(R, p.total_tiles);
  p.tiles_per_range = (p.total_tiles + R - 1) / R;
  R = (p.total_tiles + p.tiles_per_range - 1) / p.tiles_per_range;
  p.R = (int)R;
  uint32_t idesc = instr_desc(kind == K_TF32 ? 2u : 1u, (uint32_t)p.BN);
  idesc |= (1u << 15) | (1u << 16);  // A and B MN-major
  p.idesc = idesc;
  // 1: 16-byte vector loads; 2: 32-byte aligned chunks (one load per chunk)
  auto vec_of = [](const float *a, long long ch) {
    if ((uintptr_t)a % 32 == 0 && ch % 8 == 0) return 2;
    return ((uintptr_t)a % 16 == 0 && ch % 4 == 0) ? 1 : 0;
  };
  p.vec_x = vec_of(x, p.Ci);
  p.vec_y = vec_of(dy, p.Co);
  p.spin_limit = wait_limit();
  p.status = status_word();
  if (!p.status) {
    set_error("wgrad_tc: cannot locate device status word");
    return kErrCuda;
  }
  const long long welems = (long long)p.T * p.Ci * p.Co;
  float *part = nullptr;
  if (p.R > 1) {
    int rc = scratch_alloc((void **)&part, sizeof(float) * (size_t)welems * p.R, s);
    if (rc) return rc;
    p.out = part;
  } else {
    p.out = dw;
  }
  const size_t smem =
      (size_t)p.NS * parts * (p.x_bytes + p.y_bytes) + (2 * p.NS + 2) * 8 + 16 + 4 * (size_t)p.TG;
  const int grid = (int)(units * p.R);
  int rc;
  if (kind == K_BF16X3) rc = launch<K_BF16X3>(p, smem, grid, s);
  else rc = launch<K_BF16>(p, smem, grid, s);
  if (rc == kOk && p.R > 1) {
    // float4 path needs 16-byte aligned rows: welems % 4 == 0 and dw aligned
    const bool v4 = welems % 4 == 0 && (uintptr_t)dw % 16 == 0;
    const long long work = v4 ? welems / 4 : welems;
    const int blocks = (int)std::max<long long>(1, std::min<long long>((work + 127) / 128, 8 * 152));
    cudaError_t e = launch_pdl(wgrad_reduce, dim3(blocks), dim3(128), 0, s, (const float *)part,
                               dw, welems, p.R, v4 ? 1 : 0);
    if (e == cudaSuccess) e = cudaGetLastError();
    note_launch();
    if (e != cudaSuccess) rc = cuda_fail(e, "wgrad_reduce");
  }
  if (part) scratch_free(part, s);
  return rc;
}

}  // namespace owlgpu
