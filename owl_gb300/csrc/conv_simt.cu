// conv_simt.cu -- CUDA-core implicit-GEMM convolutions (float32 "plain",
// float64, complex32 and complex64), forward / backward-input /
// backward-kernel, 2-D, 3-D, strided, dilated.  No im2col matrix is ever
// materialised: every GEMM operand element is gathered from the NHWC-style
// Owl array while the tile is staged into
// shared memory.
//
// GEMM views (k = ((kc*KR + kr)*KD + kd)*Ci + ci, Owl's im2col column order,
// owl_ndarray_conv_impl.h:315-325):
//   forward      Y[m][co]  = sum_k  X[gather(m, k)]           * W[k][co]
//                m = output pixel (b, oc, or, od)
//   bwd input    dX[m][ci] = sum_{tap,co} dY[scatter^-1(m,tap)][co] * W[tap][ci][co]
//                m = input pixel; only taps with (i + p - t*d) % s == 0 hit
//   bwd kernel   dW[tap*Ci+ci][co] = sum_m X[gather(m, tap)][ci] * dY[m][co]
//                reduction over output pixels, split across CTAs and summed
//                by a second kernel in a fixed order (deterministic).
#include "common.cuh"

#include <algorithm>
#include <type_traits>

namespace owlgpu {
namespace {

enum Mode { FWD = 0, BWDI = 1, BWDK = 2 };

struct Dev {
  int64_t B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co;
  int sc, sr, sd, dc, dr, dd, pc, pr, pd;
  int64_t M, N, K;  // GEMM view sizes
  // FWD only, ystrided: output pixel (b, oc, or, od) is written at pixel
  // yoff + b*ysb + oc*ysc + or*ysr + od*ysd of the output array (one
  // residue class of a backward_input); otherwise the output is dense.
  int ystrided;
  int64_t yoff, ysb, ysc, ysr, ysd;
  // FWD, float32 vector kernel only, ystrided == 2 (window scatter): column
  // n = t*s2d_ci + ci of row m goes to output pixel (row pixel of m) +
  // tc*s2d_tc + tr*s2d_tr + td, channel ci, for tap t = (tc*s2d_kr + tr)*s2d_kd
  // + td (a backward_input whose kernel equals its stride: every input pixel
  // receives exactly one tap)
  int64_t s2d_ci, s2d_tc, s2d_tr;
  int s2d_kr, s2d_kd;
};

template <typename T, int MODE, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    conv_simt_kernel(Dev g, const T *__restrict__ A0, const T *__restrict__ B0,
                     T *__restrict__ C, int64_t k_per_split) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int A_PER = BM * BK / NT;
  constexpr int B_PER = BN * BK / NT;
  static_assert(BM * BK % NT == 0 && BN * BK % NT == 0, "tile/thread mismatch");

  __shared__ T As[2][BK][BM + 4];
  __shared__ T Bs[2][BK][BN + 4];
  // Per-row (FWD/BWDI) or per-k (BWDK) pixel decode cache.
  constexpr int PIX = (MODE == BWDK) ? BK : BM;
  __shared__ int64_t s_base[2][PIX];
  __shared__ int s_c[2][PIX], s_r[2][PIX], s_d[2][PIX];

  const int tid = threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  // BWDK: a thread's A elements all sit in row m0 + tid % BM (NT is a
  // multiple of BM), so its tap and channel are decoded once.
  static_assert(MODE != BWDK || NT % BM == 0, "BWDK row decode needs NT % BM == 0");
  int a_dc = 0, a_dr = 0, a_dd = 0, a_ci = 0;
  bool a_mval = false;
  if (MODE == BWDK) {
    const int64_t m = m0 + tid % BM;
    a_mval = m < g.M;
    if (a_mval) {
      int64_t tap = m / g.Ci;
      a_ci = (int)(m - tap * g.Ci);
      const int kd = (int)(tap % g.KD);
      tap /= g.KD;
      const int kr = (int)(tap % g.KR), kc = (int)(tap / g.KR);
      a_dc = kc * g.dc;
      a_dr = kr * g.dr;
      a_dd = kd * g.dd;
    }
  }
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  const int64_t k_begin = (int64_t)blockIdx.z * k_per_split;
  const int64_t k_end = min(g.K, k_begin + k_per_split);

  // ---- pixel decode helpers ------------------------------------------
  // FWD: row m is an output pixel; store batch base of X and window origin.
  // BWDI: row m is an input pixel; store batch base of dY and (i + pad).
  // BWDK: k index is an output pixel; store batch base of X and origin.
  auto decode_pixel = [&](int64_t p, int slot, int buf) {
    if (MODE == BWDI) {
      if (p < g.M) {
        int64_t id = p % g.ID, t = p / g.ID;
        int64_t ir = t % g.IR; t /= g.IR;
        int64_t ic = t % g.IC, b = t / g.IC;
        s_base[buf][slot] = b * g.OC * g.OR * g.OD;
        s_c[buf][slot] = (int)ic + g.pc;
        s_r[buf][slot] = (int)ir + g.pr;
        s_d[buf][slot] = (int)id + g.pd;
      } else {
        s_base[buf][slot] = -1;
      }
    } else {
      int64_t lim = (MODE == FWD) ? g.M : g.K;
      if (p < lim) {
        int64_t od = p % g.OD, t = p / g.OD;
        int64_t orr = t % g.OR; t /= g.OR;
        int64_t oc = t % g.OC, b = t / g.OC;
        s_base[buf][slot] = b * g.IC * g.IR * g.ID;
        s_c[buf][slot] = (int)(oc * g.sc) - g.pc;
        s_r[buf][slot] = (int)(orr * g.sr) - g.pr;
        s_d[buf][slot] = (int)(od * g.sd) - g.pd;
      } else {
        s_base[buf][slot] = -1;
      }
    }
  };

  if (MODE != BWDK) {
    for (int i = tid; i < BM; i += NT) decode_pixel(m0 + i, i, 0);
    for (int i = tid; i < BM; i += NT) {
      s_base[1][i] = s_base[0][i];
      s_c[1][i] = s_c[0][i]; s_r[1][i] = s_r[0][i]; s_d[1][i] = s_d[0][i];
    }
    __syncthreads();  // rows decoded by one thread are gathered by others
  }

  T a_reg[A_PER], b_reg[B_PER];

  // Gather one BK-slab of A and B into registers.
  auto load_tiles = [&](int64_t k0, int buf) {
    if (MODE == FWD) {
      // A[m][k]: thread owns a fixed k column, several rows.
      const int kk = tid % BK;
      const int64_t k = k0 + kk;
      int kc = 0, kr = 0, kd = 0, ci = 0;
      bool kval = k < k_end;
      if (kval) {
        int64_t tap = k / g.Ci;
        ci = (int)(k - tap * g.Ci);
        kd = (int)(tap % g.KD); tap /= g.KD;
        kr = (int)(tap % g.KR); kc = (int)(tap / g.KR);
      }
#pragma unroll
      for (int i = 0; i < A_PER; ++i) {
        int mm = tid / BK + i * (NT / BK);
        T v = T(0);
        int64_t base = s_base[buf][mm];
        if (kval && base >= 0) {
          int c = s_c[buf][mm] + kc * g.dc, r = s_r[buf][mm] + kr * g.dr,
              d = s_d[buf][mm] + kd * g.dd;
          if (c >= 0 && c < g.IC && r >= 0 && r < g.IR && d >= 0 && d < g.ID)
            v = A0[((base + ((int64_t)c * g.IR + r) * g.ID + d) * g.Ci) + ci];
        }
        a_reg[i] = v;
      }
      // B[k][n] = W[k][n], n fastest.
#pragma unroll
      for (int i = 0; i < B_PER; ++i) {
        int e = tid + i * NT;
        int kk2 = e / BN, nn = e % BN;
        int64_t kq = k0 + kk2, n = n0 + nn;
        b_reg[i] = (kq < k_end && n < g.N) ? B0[kq * g.N + n] : T(0);
      }
    } else if (MODE == BWDI) {
      // A[m][k], k = tap*Co + co: thread owns fixed k, several rows.
      const int kk = tid % BK;
      const int64_t k = k0 + kk;
      int kc = 0, kr = 0, kd = 0, co = 0;
      bool kval = k < k_end;
      if (kval) {
        int64_t tap = k / g.Co;
        co = (int)(k - tap * g.Co);
        kd = (int)(tap % g.KD); tap /= g.KD;
        kr = (int)(tap % g.KR); kc = (int)(tap / g.KR);
      }
#pragma unroll
      for (int i = 0; i < A_PER; ++i) {
        int mm = tid / BK + i * (NT / BK);
        T v = T(0);
        int64_t base = s_base[buf][mm];
        if (kval && base >= 0) {
          int tc = s_c[buf][mm] - kc * g.dc, tr = s_r[buf][mm] - kr * g.dr,
              td = s_d[buf][mm] - kd * g.dd;
          if (tc >= 0 && tr >= 0 && td >= 0 && tc % g.sc == 0 && tr % g.sr == 0 &&
              td % g.sd == 0) {
            int oc = tc / g.sc, orr = tr / g.sr, od = td / g.sd;
            if (oc < g.OC && orr < g.OR && od < g.OD)
              v = A0[((base + ((int64_t)oc * g.OR + orr) * g.OD + od) * g.Co) + co];
          }
        }
        a_reg[i] = v;
      }
      // B[k][n] = W[tap][n=ci][co]: co fastest across threads for coalescing.
#pragma unroll
      for (int i = 0; i < B_PER; ++i) {
        int e = tid + i * NT;
        int kk2 = e % BK, nn = e / BK;
        int64_t kq = k0 + kk2, n = n0 + nn;
        T v = T(0);
        if (kq < k_end && n < g.N) {
          int64_t tap = kq / g.Co, co = kq - tap * g.Co;
          v = B0[(tap * g.Ci + n) * g.Co + co];
        }
        b_reg[i] = v;
      }
    } else {
      // BWDK: A[m=(tap,ci)][k=pixel] = X[gather], m fastest across threads.
#pragma unroll
      for (int i = 0; i < A_PER; ++i) {
        const int kk = (tid + i * NT) / BM;
        T v = T(0);
        const int64_t base = s_base[buf][kk];
        if (a_mval && base >= 0) {
          const int c = s_c[buf][kk] + a_dc, r = s_r[buf][kk] + a_dr, d = s_d[buf][kk] + a_dd;
          if (c >= 0 && c < g.IC && r >= 0 && r < g.IR && d >= 0 && d < g.ID)
            v = A0[((base + ((int64_t)c * g.IR + r) * g.ID + d) * g.Ci) + a_ci];
        }
        a_reg[i] = v;
      }
      // B[k=pixel][n=co] = dY[pixel][co].
#pragma unroll
      for (int i = 0; i < B_PER; ++i) {
        int e = tid + i * NT;
        int kk2 = e / BN, nn = e % BN;
        int64_t kq = k0 + kk2, n = n0 + nn;
        b_reg[i] = (kq < k_end && n < g.N) ? B0[kq * g.N + n] : T(0);
      }
    }
  };

  auto store_tiles = [&](int buf) {
    if (MODE == BWDK) {
#pragma unroll
      for (int i = 0; i < A_PER; ++i) {
        int e = tid + i * NT;
        As[buf][e / BM][e % BM] = a_reg[i];
      }
    } else {
#pragma unroll
      for (int i = 0; i < A_PER; ++i) {
        int mm = tid / BK + i * (NT / BK);
        As[buf][tid % BK][mm] = a_reg[i];
      }
    }
    if (MODE == BWDI) {
#pragma unroll
      for (int i = 0; i < B_PER; ++i) {
        int e = tid + i * NT;
        Bs[buf][e % BK][e / BK] = b_reg[i];
      }
    } else {
#pragma unroll
      for (int i = 0; i < B_PER; ++i) {
        int e = tid + i * NT;
        Bs[buf][e / BN][e % BN] = b_reg[i];
      }
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

  const int tx = tid % (BN / TN), ty = tid / (BN / TN);

  if (k_begin < k_end) {
    int buf = 0;
    if (MODE == BWDK) {
      for (int i = tid; i < BK; i += NT) decode_pixel(k_begin + i, i, 0);
      __syncthreads();
    }
    load_tiles(k_begin, 0);
    store_tiles(0);
    __syncthreads();
    for (int64_t k0 = k_begin; k0 < k_end; k0 += BK) {
      const int64_t kn = k0 + BK;
      const bool more = kn < k_end;
      if (more) {
        if (MODE == BWDK) {
          for (int i = tid; i < BK; i += NT) decode_pixel(kn + i, i, buf ^ 1);
          __syncthreads();
        }
        load_tiles(kn, buf ^ 1);
      }
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        T a[TM], b[TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) a[i] = As[buf][kk][ty * TM + i];
#pragma unroll
        for (int j = 0; j < TN; ++j) b[j] = Bs[buf][kk][tx * TN + j];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      if (more) store_tiles(buf ^ 1);
      __syncthreads();
      buf ^= 1;
    }
  }

  // ---- epilogue --------------------------------------------------------
  // split z of a split-K launch writes its own partial (z = 0 otherwise)
  T *Cz = C + (int64_t)blockIdx.z * g.M * g.N;
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    int64_t m = m0 + ty * TM + i;
    if (m >= g.M) continue;
    int64_t row = m;
    if (MODE == FWD && g.ystrided) {
      int64_t t = m;
      const int64_t od = t % g.OD;
      t /= g.OD;
      const int64_t orr = t % g.OR;
      t /= g.OR;
      const int64_t oc = t % g.OC, b = t / g.OC;
      row = g.yoff + b * g.ysb + oc * g.ysc + orr * g.ysr + od * g.ysd;
    }
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int64_t n = n0 + tx * TN + j;
      if (n < g.N) Cz[row * g.N + n] = acc[i][j];
    }
  }
}

// Fixed-order sum of split-K partials: out[i] = ((p0 + p1) + p2) + ...
template <typename T>
__global__ void splitk_reduce_kernel(const T *__restrict__ part, T *__restrict__ out,
                                     int64_t n, int splits) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) {
    T s = part[i];
    for (int z = 1; z < splits; ++z) s += part[(int64_t)z * n + i];
    out[i] = s;
  }
}

// ---- float32 vector path ----------------------------------------------------
// The same GEMM views in float32 with 16-byte operand gathers: 128 x 128
// tiles (128 x 64 when N <= 64, 256 x 32 when N <= 32), 16-deep k slabs,
// 256 threads of 8 x 8 outputs (four 4 x 4 quadrants, rows ty*4 and
// 64 + ty*4, columns tx*4 and 64 + tx*4, so every shared-memory fragment is
// one 16-byte load without bank conflicts; 8 x 4 in the narrower tiles).
//   FWD : a slab is 16 consecutive input channels of one tap (Ci % 16 == 0);
//         four threads read one pixel's 64 bytes, and each thread's two
//         output pixels are decoded once per CTA.  A is stored k-major with
//         its row index XOR-swizzled by the channel quad (k / 4) * 8, so the
//         four threads of a pixel write four different bank groups.
//   BWDK: a slab is 16 consecutive output pixels; a thread reads four
//         consecutive (tap, ci) rows of one pixel (Ci % 4 == 0), a warp one
//         pixel's 128 rows; the slab's pixels are decoded by 16 threads into
//         shared memory one slab ahead.
// The k order of every output's sum is the same as the scalar kernel's
// (ascending, one fused multiply-add per k), so a float32 forward gives the
// same bits on either path.
constexpr int kVBK = 16, kVNT = 256;

__device__ __forceinline__ float4 ldg4(const float *p) {
  return __ldg(reinterpret_cast<const float4 *>(p));
}

// Tile shapes, by the GEMM's N:
//   CN = 2: 128 x 128, a thread 8 x 8 (rows ty*4 + {0, 64}, columns tx*4 + {0, 64})
//   CN = 1: 128 x 64,  a thread 8 x 4 (columns tx*4)
//   CN = 0: 256 x 32,  a thread 8 x 4 (rows ty*4 + {0, 128}, columns tx*4)
template <int CN>
struct F32vShape {
  static constexpr int BM = CN == 0 ? 256 : 128;
  static constexpr int BN = CN == 0 ? 32 : 64 * CN;
  static constexpr int RQ = BM / 64;    // FWD: A rows per thread (a 4-channel quad each)
  static constexpr int NJ = CN == 0 ? 1 : CN;  // column quads per thread
  static constexpr int RSTEP = BM / 2;  // a thread's second row quad
  static constexpr int BH = CN == 2 ? 2 : 1;  // B float4 loads per thread
};

template <int MODE, int CN>
__global__ void __launch_bounds__(kVNT, 1)
    conv_f32v_kernel(Dev g, const float *__restrict__ A0, const float *__restrict__ B0,
                     float *__restrict__ C, int64_t k_per_split) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  using S = F32vShape<CN>;
  constexpr int BM = S::BM, BN = S::BN, RQ = S::RQ, NJ = S::NJ;
  __shared__ __align__(16) float As[2][kVBK][BM];
  __shared__ __align__(16) float Bs[2][kVBK][BN];
  __shared__ int64_t s_base[2][kVBK];  // BWDK: slab pixels (batch image offset, -1 past the end)
  __shared__ int s_c[2][kVBK], s_r[2][kVBK], s_d[2][kVBK];

  const int tid = threadIdx.x;
  // A warp's 16-byte fragment loads touch one contiguous run of A and one of
  // B per k (one shared-memory wavefront each): 8 row groups x 4 column
  // groups in the 128-row tiles, 4 x 8 in the 256-row one.
  const int lane = tid & 31, warp = tid >> 5;
  const int ty = CN == 0 ? warp * 4 + (lane >> 3) : (warp >> 2) * 8 + (lane >> 2);
  const int tx = CN == 0 ? (lane & 7) : (warp & 3) * 4 + (lane & 3);
  const int64_t m0 = (int64_t)blockIdx.x * BM, n0 = (int64_t)blockIdx.y * BN;
  const int64_t k_begin = (int64_t)blockIdx.z * k_per_split;
  const int64_t k_end = min(g.K, k_begin + k_per_split);
  const int64_t img = g.IC * g.IR * g.ID;  // pixels per batch image of X

  // ---- FWD: this thread's RQ output pixels and its channel quad -----------
  const int aq = tid & 3;  // FWD: channel quad within the slab
  int64_t abase[RQ];
  int ac[RQ], ar[RQ], ad[RQ];
  // ---- BWDK: this thread's four (tap, ci) rows, its pixels ak + k*(256/(BM/4))
  constexpr int MQ = BM / 4;       // row quads per k row
  constexpr int AKS = kVNT / MQ;   // k rows per pass
  const int mq = (tid % MQ) * 4;
  const int ak = tid / MQ;
  bool mval = false;
  int t_dc = 0, t_dr = 0, t_dd = 0;
  int64_t mci = 0;
  if (MODE == FWD) {
#pragma unroll
    for (int h = 0; h < RQ; ++h) {
      const int64_t m = m0 + (tid >> 2) + 64 * h;
      abase[h] = -1;
      ac[h] = ar[h] = ad[h] = 0;
      if (m < g.M) {
        int64_t t = m;
        const int64_t od = t % g.OD;
        t /= g.OD;
        const int64_t orr = t % g.OR;
        t /= g.OR;
        const int64_t oc = t % g.OC, b = t / g.OC;
        abase[h] = b * img;
        ac[h] = (int)(oc * g.sc) - g.pc;
        ar[h] = (int)(orr * g.sr) - g.pr;
        ad[h] = (int)(od * g.sd) - g.pd;
      }
    }
  } else {
    const int64_t m = m0 + mq;
    if (m < g.M) {
      mval = true;
      int64_t tap = m / g.Ci;
      mci = m - tap * g.Ci;
      const int kd = (int)(tap % g.KD);
      tap /= g.KD;
      const int kr = (int)(tap % g.KR), kc = (int)(tap / g.KR);
      t_dc = kc * g.dc;
      t_dr = kr * g.dr;
      t_dd = kd * g.dd;
    }
  }
  // BWDK: decode pixel p into slot `slot` of buffer `buf` (-1 past k_end)
  auto decode = [&](int64_t p, int slot, int buf) {
    if (p < k_end) {
      int64_t t = p;
      const int64_t od = t % g.OD;
      t /= g.OD;
      const int64_t orr = t % g.OR;
      t /= g.OR;
      const int64_t oc = t % g.OC, b = t / g.OC;
      s_base[buf][slot] = b * img;
      s_c[buf][slot] = (int)(oc * g.sc) - g.pc;
      s_r[buf][slot] = (int)(orr * g.sr) - g.pr;
      s_d[buf][slot] = (int)(od * g.sd) - g.pd;
    } else {
      s_base[buf][slot] = -1;
    }
  };

  // BWDK: in the loop, decode thread tid (< 16) decodes pixel dp = (slab j +
  // 2)'s pixel tid, one slab further each step: (b, oc, orr*OD + od) advance
  // by adding 16 to the last with carries, no division per slab
  int64_t dp = 0, db = 0, doc = 0, dq = 0;
  const int64_t ORD = g.OR * g.OD;
  if (MODE == BWDK && tid < kVBK) {
    dp = k_begin + 2 * kVBK + tid;
    int64_t t = dp;
    dq = t % ORD;
    t /= ORD;
    doc = t % g.OC;
    db = t / g.OC;
  }
  auto decode_next = [&](int slot, int buf) {
    if (dp < k_end) {
      const int64_t orr = g.OD == 1 ? dq : dq / g.OD, od = dq - orr * g.OD;
      s_base[buf][slot] = db * img;
      s_c[buf][slot] = (int)(doc * g.sc) - g.pc;
      s_r[buf][slot] = (int)(orr * g.sr) - g.pr;
      s_d[buf][slot] = (int)(od * g.sd) - g.pd;
    } else {
      s_base[buf][slot] = -1;
    }
    dp += kVBK;
    dq += kVBK;
    while (dq >= ORD) {
      dq -= ORD;
      if (++doc == g.OC) {
        doc = 0;
        ++db;
      }
    }
  };

  // FWD slab position: tap (kc, kr, kd) and first channel ci0 of slab k0
  int kc = 0, kr = 0, kd = 0;
  int64_t ci0 = 0;
  if (MODE == FWD) {
    int64_t tap = k_begin / g.Ci;
    ci0 = k_begin - tap * g.Ci;
    kd = (int)(tap % g.KD);
    tap /= g.KD;
    kr = (int)(tap % g.KR);
    kc = (int)(tap / g.KR);
  }

  // A: FWD RQ float4 (pixels), BWDK 16/AKS float4 (k rows); B: BH float4
  constexpr int AH = MODE == FWD ? RQ : kVBK / AKS;
  float4 va[AH], vb[S::BH];
  // B: float4 column bcol of k rows bk (+ 8)
  constexpr int BQ = BN / 4;  // float4 per k row of B
  const int bcol = (tid % BQ) * 4;
  const int bk = tid / BQ;
  const bool bval = bk < kVBK && n0 + bcol < g.N;  // (256x32: threads past 128 load no B)

  // global -> registers for slab k0 (FWD: at tap kc/kr/kd, channels ci0..)
  auto load = [&](int64_t k0, int buf) {
    if (MODE == FWD) {
#pragma unroll
      for (int h = 0; h < AH; ++h) {
        const int c = ac[h] + kc * g.dc, r = ar[h] + kr * g.dr, d = ad[h] + kd * g.dd;
        va[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (abase[h] >= 0 && (unsigned)c < (unsigned)g.IC && (unsigned)r < (unsigned)g.IR &&
            (unsigned)d < (unsigned)g.ID)
          va[h] = ldg4(A0 + (abase[h] + ((int64_t)c * g.IR + r) * g.ID + d) * g.Ci + ci0 + aq * 4);
      }
    } else {
#pragma unroll
      for (int h = 0; h < AH; ++h) {
        const int kl = ak + AKS * h;
        const int64_t base = s_base[buf][kl];
        va[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (mval && base >= 0) {
          const int c = s_c[buf][kl] + t_dc, r = s_r[buf][kl] + t_dr, d = s_d[buf][kl] + t_dd;
          if ((unsigned)c < (unsigned)g.IC && (unsigned)r < (unsigned)g.IR &&
              (unsigned)d < (unsigned)g.ID)
            va[h] = ldg4(A0 + (base + ((int64_t)c * g.IR + r) * g.ID + d) * g.Ci + mci);
        }
      }
    }
#pragma unroll
    for (int h = 0; h < S::BH; ++h) {
      const int64_t kq = k0 + bk + 8 * h;
      vb[h] = (bval && kq < k_end) ? ldg4(B0 + kq * g.N + n0 + bcol)
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };
  auto store = [&](int buf) {
    if (MODE == FWD) {
#pragma unroll
      for (int h = 0; h < AH; ++h) {
        const int row = ((tid >> 2) + 64 * h) ^ (aq << 3);
        As[buf][aq * 4 + 0][row] = va[h].x;
        As[buf][aq * 4 + 1][row] = va[h].y;
        As[buf][aq * 4 + 2][row] = va[h].z;
        As[buf][aq * 4 + 3][row] = va[h].w;
      }
    } else {
#pragma unroll
      for (int h = 0; h < AH; ++h)
        *reinterpret_cast<float4 *>(&As[buf][ak + AKS * h][mq]) = va[h];
    }
    if (bk < kVBK) {
#pragma unroll
      for (int h = 0; h < S::BH; ++h)
        *reinterpret_cast<float4 *>(&Bs[buf][bk + 8 * h][bcol]) = vb[h];
    }
  };
  auto next_tap = [&]() {
    ci0 += kVBK;
    if (ci0 == g.Ci) {
      ci0 = 0;
      if (++kd == g.KD) {
        kd = 0;
        if (++kr == g.KR) {
          kr = 0;
          ++kc;
        }
      }
    }
  };

  float acc[8][4 * NJ];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4 * NJ; ++j) acc[i][j] = 0.f;

  if (k_begin < k_end) {
    if (MODE == BWDK) {
      if (tid < kVBK) decode(k_begin + tid, tid, 0);
      if (tid >= kVBK && tid < 2 * kVBK) decode(k_begin + kVBK + tid - kVBK, tid - kVBK, 1);
      __syncthreads();
    }
    load(k_begin, 0);
    store(0);
    if (MODE == FWD) next_tap();
    __syncthreads();
    int buf = 0;
    for (int64_t k0 = k_begin; k0 < k_end; k0 += kVBK) {
      const int64_t kn = k0 + kVBK;
      const bool more = kn < k_end;
      if (more) load(kn, buf ^ 1);  // BWDK: slab kn's pixels sit in buffer buf ^ 1
      // BWDK: decode slab kn + 16 into this slab's (now unused) buffer
      if (MODE == BWDK && tid < kVBK) decode_next(tid, buf);  // pixel kn + 16 + tid
#pragma unroll
      for (int k = 0; k < kVBK; ++k) {
        const int sw = MODE == FWD ? ((k >> 2) << 3) : 0;
        float a[8];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float4 f =
              *reinterpret_cast<const float4 *>(&As[buf][k][(S::RSTEP * q + ty * 4) ^ sw]);
          a[4 * q] = f.x; a[4 * q + 1] = f.y; a[4 * q + 2] = f.z; a[4 * q + 3] = f.w;
        }
        float b[4 * NJ];
#pragma unroll
        for (int q = 0; q < NJ; ++q) {
          const float4 f = *reinterpret_cast<const float4 *>(&Bs[buf][k][64 * q + tx * 4]);
          b[4 * q] = f.x; b[4 * q + 1] = f.y; b[4 * q + 2] = f.z; b[4 * q + 3] = f.w;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 4 * NJ; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
      }
      if (more) {
        store(buf ^ 1);
        if (MODE == FWD) next_tap();
      }
      __syncthreads();
      buf ^= 1;
    }
  }

  float *Cz = C + (int64_t)blockIdx.z * g.M * g.N;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int64_t m = m0 + S::RSTEP * (i >> 2) + ty * 4 + (i & 3);
    if (m >= g.M) continue;
    int64_t row = m;
    if (MODE == FWD && g.ystrided) {
      int64_t t = m;
      const int64_t od = t % g.OD;
      t /= g.OD;
      const int64_t orr = t % g.OR;
      t /= g.OR;
      const int64_t oc = t % g.OC, b = t / g.OC;
      row = g.yoff + b * g.ysb + oc * g.ysc + orr * g.ysr + od * g.ysd;
    }
#pragma unroll
    for (int q = 0; q < NJ; ++q) {
      const int64_t n = n0 + q * 64 + tx * 4;
      if (n >= g.N) continue;
      const float4 v =
          make_float4(acc[i][4 * q], acc[i][4 * q + 1], acc[i][4 * q + 2], acc[i][4 * q + 3]);
      if (MODE == FWD && g.ystrided == 2) {
        const int64_t t = n / g.s2d_ci, ci = n - t * g.s2d_ci;
        const int64_t tc = t / (g.s2d_kr * g.s2d_kd), tr = (t / g.s2d_kd) % g.s2d_kr,
                      td = t % g.s2d_kd;
        *reinterpret_cast<float4 *>(
            Cz + (row + tc * g.s2d_tc + tr * g.s2d_tr + td) * g.s2d_ci + ci) = v;
      } else {
        *reinterpret_cast<float4 *>(Cz + row * g.N + n) = v;
      }
    }
  }
}

// Whether the float32 vector path takes a launch: 16-byte aligned operands,
// N a multiple of 4 (128-, 64- or 32-wide tiles), FWD slabs inside one tap
// (Ci % 16, whole slabs per split), BWDK rows in quads of one tap (Ci % 4).
bool f32v_ok(int mode, const Dev &d, const void *A, const void *B, const void *C,
             int64_t kps) {
  auto al = [](const void *p) { return ((uintptr_t)p & 15) == 0; };
  if (!al(A) || !al(B) || !al(C) || d.N % 4 != 0 || d.N == 0) return false;
  if (d.IC >= (1 << 30) || d.IR >= (1 << 30) || d.ID >= (1 << 30)) return false;
  if (mode == FWD) return d.Ci % kVBK == 0 && kps % kVBK == 0;
  if (mode == BWDK) return d.Ci % 4 == 0;
  return false;
}

template <int MODE>
int launch_f32v(const Dev &d, const float *A, const float *B, float *C, int splits, int64_t kps,
                cudaStream_t s) {
  const int cn = d.N > 64 ? 2 : (d.N > 32 ? 1 : 0);
  const int bm = cn == 0 ? 256 : 128, bn = cn == 0 ? 32 : 64 * cn;
  dim3 grid((unsigned)ceil_div(d.M, bm), (unsigned)ceil_div(d.N, bn), (unsigned)splits);
  cudaError_t e;
  if (cn == 2)
    e = launch_pdl(conv_f32v_kernel<MODE, 2>, grid, dim3(kVNT), 0, s, d, A, B, C, kps);
  else if (cn == 1)
    e = launch_pdl(conv_f32v_kernel<MODE, 1>, grid, dim3(kVNT), 0, s, d, A, B, C, kps);
  else
    e = launch_pdl(conv_f32v_kernel<MODE, 0>, grid, dim3(kVNT), 0, s, d, A, B, C, kps);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  return e == cudaSuccess ? kOk : cuda_fail(e, "conv_f32v_kernel");
}

Dev make_dev(const ConvGeom &g, int mode) {
  Dev d{};
  d.B = g.B; d.IC = g.IC; d.IR = g.IR; d.ID = g.ID; d.Ci = g.Ci;
  d.KC = g.KC; d.KR = g.KR; d.KD = g.KD;
  d.OC = g.OC; d.OR = g.OR; d.OD = g.OD; d.Co = g.Co;
  d.sc = g.sc; d.sr = g.sr; d.sd = g.sd;
  d.dc = g.dc; d.dr = g.dr; d.dd = g.dd;
  d.pc = g.pc; d.pr = g.pr; d.pd = g.pd;
  d.ystrided = 0;
  d.yoff = 0;
  d.ysb = g.OC * g.OR * g.OD; d.ysc = g.OR * g.OD; d.ysr = g.OD; d.ysd = 1;
  if (mode == FWD) { d.M = g.out_pixels(); d.N = g.Co; d.K = g.taps() * g.Ci; }
  else if (mode == BWDI) { d.M = g.in_pixels(); d.N = g.Ci; d.K = g.taps() * g.Co; }
  else { d.M = g.taps() * g.Ci; d.N = g.Co; d.K = g.out_pixels(); }
  return d;
}

template <typename T, int MODE, int BM, int BN, int BK, int TM, int TN>
int launch_cfg(const Dev &d, const T *A, const T *B, T *C, int splits, int64_t kps,
               cudaStream_t s) {
  constexpr int NT = (BM / TM) * (BN / TN);
  dim3 grid((unsigned)ceil_div(d.M, BM), (unsigned)ceil_div(d.N, BN), (unsigned)splits);
  cudaError_t e = launch_pdl(conv_simt_kernel<T, MODE, BM, BN, BK, TM, TN>, grid, dim3(NT), 0, s,
                             d, A, B, C, kps);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  return e == cudaSuccess ? kOk : cuda_fail(e, "conv_simt_kernel");
}

// Tile choice by the GEMM's N (output channels for FWD, input channels for
// BWDI, Co for BWDK).
template <typename T, int MODE>
int launch_any(const Dev &d, const T *A, const T *B, T *C, int splits, int64_t kps,
               cudaStream_t s) {
  if constexpr (std::is_same_v<T, float>) {
    if ((MODE == FWD || MODE == BWDK) && f32v_ok(MODE, d, A, B, C, kps))
      return launch_f32v<MODE == BWDK ? BWDK : FWD>(d, A, B, C, splits, kps, s);
  }
  if constexpr (sizeof(T) == 4) {
    if (d.N > 64) return launch_cfg<T, MODE, 128, 128, 8, 8, 8>(d, A, B, C, splits, kps, s);
    if (d.N > 32) return launch_cfg<T, MODE, 128, 64, 8, 8, 4>(d, A, B, C, splits, kps, s);
    return launch_cfg<T, MODE, 128, 32, 8, 4, 4>(d, A, B, C, splits, kps, s);
  } else {
    if (d.N > 32) return launch_cfg<T, MODE, 64, 64, 8, 4, 4>(d, A, B, C, splits, kps, s);
    return launch_cfg<T, MODE, 64, 32, 8, 4, 2>(d, A, B, C, splits, kps, s);
  }
}

template <typename T>
int tile_m(const Dev &d) { return sizeof(T) == 4 ? (d.N <= 32 ? 256 : 128) : 64; }
template <typename T>
int tile_n(const Dev &d) {
  if (sizeof(T) == 4) return d.N > 64 ? 128 : (d.N > 32 ? 64 : 32);
  return d.N > 32 ? 64 : 32;
}

template <typename T>
int fwd_t(const ConvGeom &g, const T *x, const T *w, T *y, cudaStream_t s) {
  Dev d = make_dev(g, FWD);
  if (d.M == 0 || d.N == 0) return kOk;
  if (d.K == 0) {
    OWL_CUDA(cudaMemsetAsync(y, 0, sizeof(T) * d.M * d.N, s));
    return kOk;
  }
  return launch_any<T, FWD>(d, x, w, y, 1, d.K, s);
}

// The kernel of one residue class of backward_input, laid out as the kernel
// of a forward convolution of dY: w2[t'][co][ci] = w[orig(t')][ci][co], t' =
// (a, b, c) over the class's taps, orig = (base + mul * t') per axis.
template <typename T>
__global__ void bwdi_class_weights(const T *__restrict__ w, T *__restrict__ w2, int Ka, int Kb,
                                   int Kc, int base_a, int base_b, int base_c, int mul_a,
                                   int mul_b, int mul_c, int KR, int KD, int64_t Ci,
                                   int64_t Co) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  const int64_t total = (int64_t)Ka * Kb * Kc * Co * Ci;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ci = i % Ci;
    int64_t r = i / Ci;
    const int64_t co = r % Co;
    r /= Co;
    const int c = (int)(r % Kc), b = (int)((r / Kc) % Kb), a = (int)(r / ((int64_t)Kc * Kb));
    const int64_t orig = ((int64_t)(base_a + mul_a * a) * KR + (base_b + mul_b * b)) * KD +
                         (base_c + mul_c * c);
    w2[i] = w[(orig * Ci + ci) * Co + co];
  }
}

// The kernel of a kernel = stride backward_input as one GEMM operand:
// w2[co][t*Ci + ci] = w[t][ci][co].
__global__ void window_weights(const float *__restrict__ w, float *__restrict__ w2, int64_t T,
                               int64_t Ci, int64_t Co) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  const int64_t total = T * Ci * Co;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ci = i % Ci;
    const int64_t r = i / Ci;
    const int64_t t = r % T, co = r / T;
    w2[i] = w[(t * Ci + ci) * Co + co];
  }
}

// float32 backward_input of a convolution whose kernel equals its stride
// (no dilation, no padding, the windows tiling the input exactly): every
// input pixel takes exactly one tap of one output pixel, so dX is one GEMM,
// dY [pixels][Co] x w2 [Co][taps*Ci], scattered window by window
// (depth-to-space) in its epilogue.  One launch reads dY once, where the
// residue classes (one tap each) read it once per class.  Returns 1 when the
// geometry or the operands do not qualify.
int bwdi_window_f32(const ConvGeom &g, float *dx, const float *w, const float *dy,
                    cudaStream_t s) {
  const bool win = g.KC == g.sc && g.KR == g.sr && g.KD == g.sd && g.dc == 1 && g.dr == 1 &&
                   g.dd == 1 && g.pc == 0 && g.pr == 0 && g.pd == 0 &&
                   g.IC == g.OC * g.sc && g.IR == g.OR * g.sr && g.ID == g.OD * g.sd &&
                   g.taps() > 1;
  if (!win) return 1;
  ConvGeom gc{};
  gc.B = g.B;
  gc.IC = g.OC; gc.IR = g.OR; gc.ID = g.OD; gc.Ci = g.Co;
  gc.KC = gc.KR = gc.KD = 1;
  gc.OC = g.OC; gc.OR = g.OR; gc.OD = g.OD; gc.Co = g.taps() * g.Ci;
  gc.sc = gc.sr = gc.sd = 1;
  gc.dc = gc.dr = gc.dd = 1;
  Dev d = make_dev(gc, FWD);
  d.ystrided = 2;
  d.yoff = 0;
  d.ysb = g.IC * g.IR * g.ID;
  d.ysc = (int64_t)g.sc * g.IR * g.ID;
  d.ysr = (int64_t)g.sr * g.ID;
  d.ysd = g.sd;
  d.s2d_ci = g.Ci;
  d.s2d_tc = g.IR * g.ID;
  d.s2d_tr = g.ID;
  d.s2d_kr = (int)g.KR;
  d.s2d_kd = (int)g.KD;
  if (g.Ci % 4 != 0 || !f32v_ok(FWD, d, dy, dy, dx, d.K)) return 1;  // w2 is fresh scratch
  float *w2 = nullptr;
  int rc = scratch_alloc((void **)&w2, sizeof(float) * (size_t)g.w_elems(), s);
  if (rc) return rc;
  const int64_t nw = g.w_elems();
  const dim3 wgrid((unsigned)std::min<int64_t>(ceil_div(nw, 256), 1024));
  cudaError_t e = launch_pdl(window_weights, wgrid, dim3(256), 0, s, w, w2, (int64_t)g.taps(),
                             (int64_t)g.Ci, (int64_t)g.Co);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  if (e != cudaSuccess) rc = cuda_fail(e, "window_weights");
  if (rc == kOk) rc = launch_f32v<FWD>(d, dy, w2, dx, 1, d.K, s);
  scratch_free(w2, s);
  return rc;
}

// backward_input as forward convolutions over the residue classes of dX.
// With forward index s*o - p + t*d, element i = s*a + r of dX receives
// dY[o] W[t] for the taps with (r + p - t*d) divisible by s, at
// o = a + (r + p - t*d)/s.  Those taps, largest first, spaced s/g apart
// (g = gcd(s, d)), form a stride-1 convolution of dY with dilation d/g and
// leading pad -(r + p - tmax*d)/s, whose output is the sub-grid i = s*a + r
// of dX: every multiply-add is a useful one (no tap is tested and masked).
// Classes that no tap reaches are zero; dX is cleared first when there are
// any.  Stride 1 is one class: dY against the flipped, channel-exchanged
// kernel.
template <typename T>
int bwdi_t(const ConvGeom &g, T *dx, const T *w, const T *dy, cudaStream_t s) {
  if (g.in_pixels() == 0 || g.Ci == 0) return kOk;
  if constexpr (std::is_same_v<T, float>) {
    if (g.Co > 0 && g.out_pixels() > 0) {
      const int rc = bwdi_window_f32(g, dx, w, dy, s);
      if (rc != 1) return rc;
    }
  }
  const int S[3] = {g.sc, g.sr, g.sd}, D[3] = {g.dc, g.dr, g.dd}, P[3] = {g.pc, g.pr, g.pd};
  const int64_t K[3] = {g.KC, g.KR, g.KD}, I[3] = {g.IC, g.IR, g.ID};
  struct Axis {
    int n, base, mul, dil, pad;
    int64_t out;
  };
  auto axis_class = [&](int ax, int r) {
    Axis a{0, 0, 0, 1, 0, 0};
    int tmax = -1;
    for (int t = 0; t < (int)K[ax]; ++t)
      if ((((r + P[ax] - t * D[ax]) % S[ax]) + S[ax]) % S[ax] == 0) {
        tmax = t > tmax ? t : tmax;
        ++a.n;
      }
    int gg = S[ax], dd = D[ax];
    while (dd) { const int t = gg % dd; gg = dd; dd = t; }
    a.base = tmax;
    a.mul = -(S[ax] / gg);
    a.dil = D[ax] / gg;
    a.pad = a.n ? -((r + P[ax] - tmax * D[ax]) / S[ax]) : 0;
    a.out = I[ax] > r ? (I[ax] - r + S[ax] - 1) / S[ax] : 0;
    return a;
  };
  bool any_empty = g.Co == 0 || g.out_pixels() == 0;
  for (int ax = 0; ax < 3; ++ax)
    for (int r = 0; r < S[ax]; ++r) {
      const Axis a = axis_class(ax, r);
      if (a.n == 0 && a.out > 0) any_empty = true;
    }
  if (any_empty) OWL_CUDA(cudaMemsetAsync(dx, 0, sizeof(T) * (size_t)g.x_elems(), s));
  if (g.Co == 0 || g.out_pixels() == 0) return kOk;
  T *w2 = nullptr;
  int rc = scratch_alloc((void **)&w2, sizeof(T) * (size_t)g.w_elems(), s);
  if (rc) return rc;
  for (int r0 = 0; r0 < S[0] && rc == kOk; ++r0)
    for (int r1 = 0; r1 < S[1] && rc == kOk; ++r1)
      for (int r2 = 0; r2 < S[2] && rc == kOk; ++r2) {
        const Axis a = axis_class(0, r0), b = axis_class(1, r1), c = axis_class(2, r2);
        if (a.n == 0 || b.n == 0 || c.n == 0 || a.out * b.out * c.out == 0) continue;
        const int64_t nw = (int64_t)a.n * b.n * c.n * g.Co * g.Ci;
        cudaError_t e = launch_pdl(
            bwdi_class_weights<T>, dim3((unsigned)std::min<int64_t>(ceil_div(nw, 256), 1024)),
            dim3(256), 0, s, w, w2, a.n, b.n, c.n, a.base, b.base, c.base, a.mul, b.mul, c.mul,
            (int)g.KR, (int)g.KD, (int64_t)g.Ci, (int64_t)g.Co);
        if (e == cudaSuccess) e = cudaGetLastError();
        note_launch();
        if (e != cudaSuccess) {
          rc = cuda_fail(e, "bwdi_class_weights");
          break;
        }
        ConvGeom gc{};
        gc.B = g.B;
        gc.IC = g.OC; gc.IR = g.OR; gc.ID = g.OD; gc.Ci = g.Co;
        gc.KC = a.n; gc.KR = b.n; gc.KD = c.n;
        gc.OC = a.out; gc.OR = b.out; gc.OD = c.out; gc.Co = g.Ci;
        gc.sc = gc.sr = gc.sd = 1;
        gc.dc = a.dil; gc.dr = b.dil; gc.dd = c.dil;
        gc.pc = a.pad; gc.pr = b.pad; gc.pd = c.pad;
        Dev d = make_dev(gc, FWD);
        d.ystrided = 1;
        d.ysb = g.IC * g.IR * g.ID;
        d.ysc = (int64_t)S[0] * g.IR * g.ID;
        d.ysr = (int64_t)S[1] * g.ID;
        d.ysd = S[2];
        d.yoff = ((int64_t)r0 * g.IR + r1) * g.ID + r2;
        rc = launch_any<T, FWD>(d, dy, w2, dx, 1, d.K, s);
      }
  scratch_free(w2, s);
  return rc;
}

// The GEMM view of one pass with its reduction split across CTAs: each
// split writes a partial, summed in split order by a second kernel
// (deterministic).  A/B are the pass's operands in launch_any's order.
template <typename T, int MODE>
int splitk_t(const ConvGeom &g, const T *A, const T *B, T *C, cudaStream_t s) {
  Dev d = make_dev(g, MODE);
  if (d.M == 0 || d.N == 0) return kOk;
  if (d.K == 0) {
    OWL_CUDA(cudaMemsetAsync(C, 0, sizeof(T) * d.M * d.N, s));
    return kOk;
  }
  // Split the reduction so that ~4 waves of CTAs cover 152 SMs, with
  // each split at least 8 K-tiles deep.
  int64_t tiles = ceil_div(d.M, tile_m<T>(d)) * ceil_div(d.N, tile_n<T>(d));
  int64_t want = ceil_div(4 * 152, tiles);
  int64_t max_by_k = ceil_div(d.K, 64);
  int splits = (int)std::max<int64_t>(1, std::min<int64_t>(want, std::min<int64_t>(max_by_k, 256)));
  int64_t kps = ceil_div(ceil_div(d.K, splits), 16) * 16;
  splits = (int)ceil_div(d.K, kps);
  if (splits == 1) return launch_any<T, MODE>(d, A, B, C, 1, kps, s);
  void *ws = nullptr;
  size_t bytes = sizeof(T) * (size_t)splits * d.M * d.N;
  int rc = scratch_alloc(&ws, bytes, s);
  if (rc) return rc;
  rc = launch_any<T, MODE>(d, A, B, (T *)ws, splits, kps, s);
  if (rc == kOk) {
    int64_t n = d.M * d.N;
    int blocks = (int)std::min<int64_t>(ceil_div(n, 256), 4 * 152);
    cudaError_t e = launch_pdl(splitk_reduce_kernel<T>, dim3(blocks), dim3(256), 0, s,
                               (const T *)ws, C, (int64_t)n, splits);
    if (e == cudaSuccess) e = cudaGetLastError();
    note_launch();
    if (e != cudaSuccess) rc = cuda_fail(e, "splitk_reduce_kernel");
  }
  scratch_free(ws, s);
  return rc;
}

template <typename T>
int bwdk_t(const ConvGeom &g, const T *x, T *dw, const T *dy, cudaStream_t s) {
  return splitk_t<T, BWDK>(g, x, dy, dw, s);
}

// backward_kernel, float32, with the split-K partials written into a
// caller-provided workspace of `ws_elems` floats instead of an allocation.
// The split count is capped so that splits * |dW| fits the workspace; every
// partial element is written before it is read, so the workspace needs no
// clearing between calls.
int bwdk_f32_into(const ConvGeom &g, const float *x, float *dw, const float *dy, float *ws,
                  int64_t ws_elems, cudaStream_t s) {
  Dev d = make_dev(g, BWDK);
  if (d.M == 0 || d.N == 0) return kOk;
  if (d.K == 0) {
    OWL_CUDA(cudaMemsetAsync(dw, 0, sizeof(float) * d.M * d.N, s));
    return kOk;
  }
  int64_t tiles = ceil_div(d.M, tile_m<float>(d)) * ceil_div(d.N, tile_n<float>(d));
  int64_t want = ceil_div(4 * 152, tiles);
  int64_t max_by_k = ceil_div(d.K, 64);
  int64_t max_by_ws = ws_elems / (d.M * d.N);
  int splits = (int)std::max<int64_t>(
      1, std::min<int64_t>(std::min<int64_t>(want, max_by_ws), std::min<int64_t>(max_by_k, 256)));
  int64_t kps = ceil_div(ceil_div(d.K, splits), 16) * 16;
  splits = (int)ceil_div(d.K, kps);
  if (splits == 1) return launch_any<float, BWDK>(d, x, dy, dw, 1, kps, s);
  int rc = launch_any<float, BWDK>(d, x, dy, ws, splits, kps, s);
  if (rc != kOk) return rc;
  int64_t n = d.M * d.N;
  int blocks = (int)std::min<int64_t>(ceil_div(n, 256), 4 * 152);
  cudaError_t e = launch_pdl(splitk_reduce_kernel<float>, dim3(blocks), dim3(256), 0, s,
                             (const float *)ws, dw, (int64_t)n, splits);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  return e == cudaSuccess ? kOk : cuda_fail(e, "splitk_reduce_kernel");
}

}  // namespace

int simt_conv_bwd_kernel_f32_into(const ConvGeom &g, const float *x, float *dw,
                                  const float *dy, float *ws, int64_t ws_elems,
                                  cudaStream_t s) {
  return bwdk_f32_into(g, x, dw, dy, ws, ws_elems, s);
}

// Element type of each Dtype: float, double, and the complex pairs (whose
// tiles are those of double: 8- and 16-byte elements).
template <typename F>
static int by_dtype(Dtype dt, F f) {
  switch (dt) {
    case F32: return f((float *)nullptr);
    case F64: return f((double *)nullptr);
    case C32: return f((c32 *)nullptr);
    case C64: return f((c64 *)nullptr);
  }
  set_error("unknown element type");
  return kErrInvalid;
}

int simt_conv_fwd(Dtype dt, const ConvGeom &g, const void *x, const void *w, void *y,
                  cudaStream_t s) {
  return by_dtype(dt, [&](auto *tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    return fwd_t<T>(g, (const T *)x, (const T *)w, (T *)y, s);
  });
}

int simt_conv_bwd_input(Dtype dt, const ConvGeom &g, void *dx, const void *w, const void *dy,
                        cudaStream_t s) {
  return by_dtype(dt, [&](auto *tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    return bwdi_t<T>(g, (T *)dx, (const T *)w, (const T *)dy, s);
  });
}

// A pass of a 1x1 geometry as a split-K GEMM (the dense layer's products on
// the CUDA cores): mode 0 forward (a = x, b = w, c = y), 1 backward_input
// (a = dy, b = w, c = dx), 2 backward_kernel (a = x, b = dy, c = dw).
int simt_gemm(Dtype dt, int mode, const ConvGeom &g, const void *a, const void *b, void *c,
              cudaStream_t s) {
  if (dt != F32 && dt != F64) {
    set_error("simt_gemm: real element kinds only");
    return kErrInvalid;
  }
  return by_dtype(dt, [&](auto *tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    if (mode == FWD) return splitk_t<T, FWD>(g, (const T *)a, (const T *)b, (T *)c, s);
    if (mode == BWDI) return splitk_t<T, BWDI>(g, (const T *)a, (const T *)b, (T *)c, s);
    return splitk_t<T, BWDK>(g, (const T *)a, (const T *)b, (T *)c, s);
  });
}

int simt_conv_bwd_kernel(Dtype dt, const ConvGeom &g, const void *x, void *dw, const void *dy,
                         cudaStream_t s) {
  return by_dtype(dt, [&](auto *tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    return bwdk_t<T>(g, (const T *)x, (T *)dw, (const T *)dy, s);
  });
}

}  // namespace owlgpu
