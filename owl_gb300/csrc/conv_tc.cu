// conv_tc.cu -- tcgen05 tensor-core convolutions for float32 data
// (precisions BF16, TF32 and split BF16 "BF16X3"): forward at any stride and
// dilation, backward-input (stride 1 directly, larger strides as residue
// classes), 2-D and 3-D.
//
// Design: persistent, warp-specialised "halo" implicit GEMM.
//   * An output tile is TU positions along one spatial axis (u) by 8 along
//     another (v): N = 8*TU pixels (TU even, up to 32), each group of 8
//     v-positions one 8-row core-matrix band of the MMA's N dimension.  The
//     kernel tile (128 output channels) is the M = 128 operand.  tcgen05.mma
//     costs the same number of cycles for any N at M = 128, so the pixel
//     dimension goes on N, the tile is as tall as the fewest tiles along u
//     allow, and no taller (less halo).
//   * Producer warps load the input halo the tile needs for one block of
//     channels -- once -- from the float32 activation, convert it (bf16 RN,
//     tf32 RNA, or bf16 hi + lo) and store it in shared memory as
//     [16-byte channel chunk][halo pixel][16 B].  Any 8 consecutive v-pixels
//     then form a K-major core matrix, so the A operand for every tap is the
//     same halo seen through a shifted descriptor: each staged pixel feeds all
//     KC*KR*KD taps with no im2col copy anywhere.
//   * The kernel tensor is re-laid out once per call (prep_weights) into the
//     exact shared-memory image of each (channel block, tap) B tile, which one
//     thread streams with cp.async.bulk (TMA engine) into a ring of stages.
//   * One thread issues tcgen05.mma (M=128 channels, N=8*TU pixels, K=16/8
//     per instruction) into a TMEM accumulator, double-buffered when two fit
//     TMEM's 512 columns; four epilogue warps drain the finished buffer
//     (tcgen05.ld, one TMEM lane per output
//     channel) and write float32 results to HBM, 32 consecutive channels of a
//     pixel per warp store.
//   * Every wait is bounded: a stuck barrier sets an error word and the CTA
//     unwinds (waits for its in-flight copies and MMAs, frees TMEM, returns).
//
// Backward-input with stride 1 is the same computation on dY with the kernel
// flipped in every spatial axis and its channel axes exchanged:
//   dX[i] = sum_t dY[i + p - t*d] W[t]^T = sum_t' dY[i - ((K-1)d - p) + t'd] W[K-1-t']^T.
// With stride s it splits into s^d residue classes of dX, each such a
// stride-1 correlation over the taps that reach it (run_bwd_input_strided).
// The classes run as the segments of one persistent launch (up to eight per
// launch), so one class's epilogue overlaps the next tile's staging and MMAs
// and the GPU is filled by all classes' tiles together.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/owlgpu.h"
#include "common.cuh"
#include "tc_ptx.cuh"
#include "tc_stage.cuh"

namespace owlgpu {
namespace {

using namespace ptx;

// Warp roles.  A warp's scheduler (SM sub-partition) is warp_id % 4.  The
// MMA warp (0) shares scheduler 0 only with the weight loader (4), an idle
// warp (8) and one epilogue warp (12): every instruction another warp issues
// there would delay the next tcgen05.mma.  The nine producer warps sit on
// schedulers 1-3; the epilogue warps 12-15 cover TMEM lane quadrants 0-3.
constexpr int kWarps = 16;
constexpr int kThreads = kWarps * 32;
constexpr int kMmaWarp = 0;
constexpr int kLoadWarp = 4;
constexpr int kEpiWarp0 = 12;
constexpr int kProducerWarps = 9;
constexpr int kProducerThreads = kProducerWarps * 32;
// producer index of a warp (warps 1-3, 5-7, 9-11), or -1
__device__ __forceinline__ int producer_index(int warp) {
  return (warp & 3) != 0 && warp < 12 ? (warp >> 2) * 3 + (warp & 3) - 1 : -1;
}
constexpr int kSmemMax = 232448;  // 227 KB opt-in dynamic shared memory
constexpr long long kSpinLimit = 4000000000LL;  // cycles (~2 s) before a wait gives up

enum Kind { K_BF16 = 0, K_TF32 = 1, K_BF16X3 = 2 };

// A launch covers up to kMaxSeg segments: convolutions that share the input,
// the channels and the tile geometry but differ in output extents, output
// origin, pads and taps (the residue classes of a strided backward_input).
// Their tiles are numbered one segment after another.
constexpr int kMaxSeg = 8;
struct Seg {
  long long tile0;  // first tile of the segment
  long long yoff;   // output origin: element offset into y
  long long woff;   // byte offset of the segment's weight images (per part)
  int OW, OU, OV, u_tiles, v_tiles;
  int KW, KU, KV, dw, du, dv, pw, pu, pv;
  int T, NSL, toff;  // taps, weight slots per channel block, first tap_off entry
};

struct TcParams {
  const float *x;
  float *y;
  const uint8_t *wt_hi, *wt_lo;
  int *status;
  int B, IW, IU, IV;  // input extents (output extents, taps and pads per segment)
  long long xsb, xsw, xsu, xsv, ysb, ysw, ysu, ysv;  // pixel strides
  int Cin, Cout;
  int BN, CB, NCH, CPB, NCB;
  // Output tile: TU positions along u (even, <= 32) by 8 along v, TN = 8*TU
  // pixels = the MMA's N; TNA = TN rounded up to 32 TMEM columns (the
  // column stride of the accumulators of a tile's co tiles and buffers).
  int TU, TN, TNA;
  int T;  // plan: taps of the longest segment
  int sw, su, sv;          // strides along w, u, v
  int HW, HU, HV, HVR, HP, PS;  // halo rows along w, u; pixels per u-row (= sv * HVR)
  int n_tiles;
  int NCT, n_groups;  // output-channel tiles per CTA tile (1 or 2), and tile groups
  long long total_tiles;
  unsigned halo_bytes, b_bytes;  // one halo stage / one weight slot (TPS taps), per part
  unsigned tile_bytes;           // one tap's weight tile (BN x CB)
  int TPS, NSL;                  // taps per weight slot; plan: slots of the longest segment
  int NH, NB;
  unsigned idesc, tmem_cols;
  // Accumulator sets in TMEM: nbuf (1 or 2) buffers of acc_cols columns; a
  // BF16X3 set holds the hi*hi sums at column 0 and the cross terms (hi*lo +
  // lo*hi) at small_off, added in the epilogue.
  int nbuf;
  unsigned acc_cols, small_off;
  int vec_in;
  int nseg;
  Seg seg[kMaxSeg];
  // Output channels per pixel of y (Cout, or fuse_n).  fuse_n > 0: the
  // Cout = classes * fuse_n output channels are the residue classes of a
  // strided backward_input with one tap each, side by side: channel co
  // belongs to class co / fuse_n, whose outputs start at fuse_yoff[class]
  // (a depth-to-space epilogue; one staged input tile serves all classes).
  int ych, fuse_n;
  long long fuse_yoff[kMaxSeg];
  // forward only: y = act(conv + bias[co]) in the epilogue (bias may be
  // null; act OWLGPU_ACT_NONE or OWLGPU_ACT_RELU)
  const float *bias;
  int act;
  long long spin_limit;  // cycles a pipeline wait polls before the CTA gives up
  // 1: launched as a programmatic dependent of arbitrary earlier work (a
  // cached weight image, no prep_weights before it): every thread waits for
  // that work before any global access.  0: the dependent of prep_weights,
  // which itself waited for the earlier work; only the weight loader waits.
  int wait_all;
};

__device__ int g_tc_status;

// Bounded mbarrier wait.  Returns false when the CTA is aborting.
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

struct Tile {
  int nt, b, ow, u0, v0, c;  // c: segment
};

// Segment of tile t, advancing from segment c (tiles are visited in
// increasing order, so the search resumes where the last one ended).
__device__ __forceinline__ int seg_of(const TcParams &p, long long t, int c) {
  while (c + 1 < p.nseg && t >= p.seg[c + 1].tile0) ++c;
  return c;
}

__device__ __forceinline__ Tile decode_tile(const TcParams &p, long long t, int c) {
  Tile r;
  const Seg &sg = p.seg[c];
  r.c = c;
  t -= sg.tile0;
  r.nt = (int)(t % p.n_groups);  // co-tile group: tiles nt*NCT .. nt*NCT+NCT-1
  t /= p.n_groups;
  r.v0 = (int)(t % sg.v_tiles) * 8;
  t /= sg.v_tiles;
  r.u0 = (int)(t % sg.u_tiles) * p.TU;
  t /= sg.u_tiles;
  r.ow = (int)(t % sg.OW);
  r.b = (int)(t / sg.OW);
  return r;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&h);
}
__device__ __forceinline__ float bf16_round(float a) {
  return __bfloat162float(__float2bfloat16_rn(a));
}
__device__ __forceinline__ uint32_t to_tf32(float a) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(a));
  return r;
}

// MULTI: the launch has several segments (else segment 0 only, read at a
// constant offset of the parameters).
template <int KIND, bool MULTI>
__global__ void __launch_bounds__(kThreads, 1) conv_tc_kernel(const __grid_constant__ TcParams p) {
  if (p.wait_all) asm volatile("griddepcontrol.wait;" ::: "memory");
  constexpr int EPC = (KIND == K_TF32) ? 4 : 8;  // channels per 16-byte chunk
  constexpr int PARTS = (KIND == K_BF16X3) ? 2 : 1;
  // BF16X3 keeps the cross terms in an accumulator of their own: the tensor
  // core rounds its FP32 accumulator toward zero after every MMA, and three
  // MMAs per K step into one accumulator cost about three times the rounding
  // of the hi*hi sums alone (up to 2e-5 of max|y| at K = 3456); in their own
  // accumulator the cross terms, 2^-8 of the result, round at their own
  // small magnitude.
  constexpr bool SEP = (KIND == K_BF16X3);
  extern __shared__ __align__(1024) uint8_t smem[];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint8_t *halo = smem;
  uint8_t *bring = smem + (size_t)p.NH * PARTS * p.halo_bytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(bring + (size_t)p.NB * PARTS * p.b_bytes);
  uint64_t *halo_full = bars;
  uint64_t *halo_empty = halo_full + p.NH;
  uint64_t *b_full = halo_empty + p.NH;
  uint64_t *b_empty = b_full + p.NB;
  uint64_t *acc_full = b_empty + p.NB;
  uint64_t *acc_empty = acc_full + 2;
  uint64_t *drain = acc_empty + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  uint32_t *tap_off = tmem_slot + 2;  // per-tap start pixel in the halo (16-byte units)

  // tap offsets of every segment, segment c's at tap_off[seg[c].toff ..]
  for (int c = 0; c < (MULTI ? p.nseg : 1); ++c) {
    const Seg &sg = p.seg[c];
    for (int tap = threadIdx.x; tap < sg.T; tap += blockDim.x) {
      const int kv = tap % sg.KV, ku = (tap / sg.KV) % sg.KU, kw = tap / (sg.KV * sg.KU);
      const int qv = kv * sg.dv;
      tap_off[sg.toff + tap] = (uint32_t)((kw * sg.dw * p.HU + ku * sg.du) * p.HV +
                                          (qv % p.sv) * p.HVR + qv / p.sv);
    }
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < p.NH; ++i) {
      mbar_init(smem_u32(&halo_full[i]), kProducerThreads);
      mbar_init(smem_u32(&halo_empty[i]), 1);
    }
    for (int i = 0; i < p.NB; ++i) {
      mbar_init(smem_u32(&b_full[i]), 1);
      mbar_init(smem_u32(&b_empty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_u32(&acc_full[i]), 1);
      mbar_init(smem_u32(&acc_empty[i]), 128);
    }
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
  if (pidx >= 0) {
    // ===================== halo producers =====================
    // Each warp stages whole halo rows: a row is one (w, u, residue) line of
    // HVR pixels whose global addresses advance by a fixed step, so the row
    // bounds are checked once and each lane only adds offsets.  A pass takes
    // one or two rows and deals their chunk slots flat over the lanes, up to
    // six loads in flight per lane.
    const int nrows = p.HW * p.HU * p.sv;
    const int S = p.HVR * p.NCH;  // chunk slots per row
    // rows per producer pass: two when both rows' slots fit 6 per lane
    const int rpp = 2 * S <= 32 * 6 ? 2 : 1;
    const int nsh = (p.NCH & (p.NCH - 1)) == 0 ? __ffs(p.NCH) - 1 : -1;
    const long long vstep = (long long)p.sv * p.xsv * p.Cin;  // floats between row pixels
    long long k = 0;  // halo stage counter
    int sc = 0;       // segment of the current tile
    for (long long t = blockIdx.x; t < p.total_tiles; t += gridDim.x) {
      sc = MULTI ? seg_of(p, t, sc) : 0;
      const Tile tl = decode_tile(p, t, sc);
      const int pw = p.seg[sc].pw, pu = p.seg[sc].pu, pv = p.seg[sc].pv;
      for (int cb = 0; cb < p.NCB; ++cb, ++k) {
        const int hs = (int)(k % p.NH);
        const uint32_t ph = (uint32_t)((k / p.NH) & 1);
        if (!wait_bar(smem_u32(&halo_empty[hs]), ph ^ 1, abort_flag, p.status, p.spin_limit)) goto done;
        uint8_t *dst = halo + (size_t)hs * PARTS * p.halo_bytes;
        const int cbase = cb * p.CPB;
        for (int r0 = pidx * rpp; r0 < nrows; r0 += rpp * kProducerWarps) {
          // the pass's rpp rows: bounds checked and base addresses formed once
          // (two named rows, not an array: a slot picks its row by a select)
          const float *rowp0, *rowp1;
          bool ok0, ok1;
          int ivs0, ivs1;
          auto row_setup = [&](int rr, const float *&rp, bool &ok, int &ivs) {
            const int r = r0 + rr;
            // row -> (w row, u row, residue class)
            const int hr = r % p.sv, t3 = r / p.sv;
            const int hu = t3 % p.HU, hw = t3 / p.HU;
            const int iw = tl.ow * p.sw - pw + hw, iu = tl.u0 * p.su - pu + hu;
            ivs = tl.v0 * p.sv - pv + hr;  // global v of the row's pixel 0
            ok = rr < rpp && r < nrows && iw >= 0 && iw < p.IW && iu >= 0 && iu < p.IU;
            rp = p.x + ((long long)tl.b * p.xsb + (long long)iw * p.xsw + (long long)iu * p.xsu +
                        (long long)ivs * p.xsv) * p.Cin + cbase;
          };
          row_setup(0, rowp0, ok0, ivs0);
          row_setup(1, rowp1, ok1, ivs1);
          // the pass's rpp*S chunk slots dealt over the lanes, up to kSlots each
          constexpr int kSlots = 6;
          float v[kSlots][EPC];
          int off[kSlots];
#pragma unroll
          for (int q = 0; q < kSlots; ++q) {
            const int sl = lane + 32 * q;
#pragma unroll
            for (int e = 0; e < EPC; ++e) v[q][e] = 0.f;
            off[q] = -1;
            const int rr = sl >= S ? 1 : 0;
            const int s2 = sl - rr * S;
            const int r = r0 + rr;
            if (sl < rpp * S && s2 < S && r < nrows) {
              const int hc = nsh >= 0 ? (s2 >> nsh) : s2 / p.NCH;
              const int j = s2 - hc * p.NCH;
              off[q] = j * p.PS * 16 + (r * p.HVR + hc) * 16;
              const int iv = (rr ? ivs1 : ivs0) + hc * p.sv;
              const int c = cbase + j * EPC;
              if ((rr ? ok1 : ok0) && iv >= 0 && iv < p.IV && c < p.Cin) {
                const float *src = (rr ? rowp1 : rowp0) + hc * vstep + j * EPC;
                if (p.vec_in && c + EPC <= p.Cin) {
                  stage::load_vec<EPC>(src, p.vec_in, v[q]);
                } else {
#pragma unroll
                  for (int e = 0; e < EPC; ++e)
                    if (c + e < p.Cin) v[q][e] = __ldg(src + e);
                }
              }
            }
          }
#pragma unroll
          for (int q = 0; q < kSlots; ++q) {
            if (off[q] < 0) continue;
            uint4 hi;
            if (KIND == K_TF32) {
              hi = make_uint4(to_tf32(v[q][0]), to_tf32(v[q][1]), to_tf32(v[q][2]),
                              to_tf32(v[q][3]));
            } else {
              hi = make_uint4(pack_bf16(v[q][0], v[q][1]), pack_bf16(v[q][2], v[q][3]),
                              pack_bf16(v[q][4], v[q][5]), pack_bf16(v[q][6], v[q][7]));
            }
            *reinterpret_cast<uint4 *>(dst + off[q]) = hi;
            if (KIND == K_BF16X3) {
              float rs[8];
#pragma unroll
              for (int e = 0; e < 8; ++e) rs[e] = v[q][e] - bf16_round(v[q][e]);
              uint4 lo = make_uint4(pack_bf16(rs[0], rs[1]), pack_bf16(rs[2], rs[3]),
                                    pack_bf16(rs[4], rs[5]), pack_bf16(rs[6], rs[7]));
              *reinterpret_cast<uint4 *>(dst + p.halo_bytes + off[q]) = lo;
            }
          }
          // rows wider than 32*kSlots chunk slots (one row per pass then):
          // stage the remainder one slot at a time (large dilations / long
          // kernel rows only)
          for (int rr = 0; rr < rpp; ++rr) {
            const int r = r0 + rr;
            if (r >= nrows) break;
            for (int sl = lane + 32 * kSlots; sl < S; sl += 32) {
              const int hr = r % p.sv, t3 = r / p.sv;
              const int hu = t3 % p.HU, hw = t3 / p.HU;
              const int iw = tl.ow * p.sw - pw + hw, iu = tl.u0 * p.su - pu + hu;
              const int hc = sl / p.NCH, j = sl - hc * p.NCH;
              const int iv = tl.v0 * p.sv - pv + hr + hc * p.sv;
              const int c = cbase + j * EPC;
              float w8[EPC];
#pragma unroll
              for (int e = 0; e < EPC; ++e) w8[e] = 0.f;
              if (iw >= 0 && iw < p.IW && iu >= 0 && iu < p.IU && iv >= 0 && iv < p.IV) {
                const float *src = p.x + ((long long)tl.b * p.xsb + (long long)iw * p.xsw +
                                          (long long)iu * p.xsu + (long long)iv * p.xsv) *
                                             p.Cin + c;
#pragma unroll
                for (int e = 0; e < EPC; ++e)
                  if (c + e < p.Cin) w8[e] = __ldg(src + e);
              }
              const int o = j * p.PS * 16 + (r * p.HVR + hc) * 16;
              uint4 hi;
              if (KIND == K_TF32) {
                hi = make_uint4(to_tf32(w8[0]), to_tf32(w8[1]), to_tf32(w8[2]), to_tf32(w8[3]));
              } else {
                hi = make_uint4(pack_bf16(w8[0], w8[1]), pack_bf16(w8[2], w8[3]),
                                pack_bf16(w8[4], w8[5]), pack_bf16(w8[6], w8[7]));
              }
              *reinterpret_cast<uint4 *>(dst + o) = hi;
              if (KIND == K_BF16X3) {
                float rs[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) rs[e] = w8[e] - bf16_round(w8[e]);
                *reinterpret_cast<uint4 *>(dst + p.halo_bytes + o) =
                    make_uint4(pack_bf16(rs[0], rs[1]), pack_bf16(rs[2], rs[3]),
                               pack_bf16(rs[4], rs[5]), pack_bf16(rs[6], rs[7]));
              }
            }
          }
        }
        fence_proxy_async();
        mbar_arrive(smem_u32(&halo_full[hs]));
      }
    }
  } else if (warp == kMmaWarp) {
    // ===================== MMA issuer =====================
    if (lane == 0) {
      // ring positions and phases advance by counting (no division in the
      // issue loop: this thread's own work is on the critical path)
      int hs = 0, bs = 0;
      uint32_t hph = 0, bph = 0;
      int tc = 0;
      const uint32_t halo0 = smem_u32(halo), b0 = smem_u32(bring);
      const uint32_t a_lbo = (uint32_t)p.PS * 16, a_sbo = (uint32_t)(p.su * p.HV) * 16;
      const uint32_t b_lbo = (uint32_t)p.BN * 16;
      const int ksteps = p.NCH / 2;
      // descriptor increments in 16-byte units
      const uint64_t wd_ring = smem_desc(b0, b_lbo, 128);
      const uint32_t wslot16 = (PARTS * p.b_bytes) >> 4, wstep16 = (2 * b_lbo) >> 4;
      const uint32_t tile16 = p.tile_bytes >> 4;
      const uint32_t wlo16 = p.b_bytes >> 4, xstep16 = (2 * a_lbo) >> 4, xlo16 = p.halo_bytes >> 4;
      int sc = 0;
      for (long long t = blockIdx.x; t < p.total_tiles; t += gridDim.x, ++tc) {
        sc = MULTI ? seg_of(p, t, sc) : 0;
        const int nsl = p.seg[sc].NSL, ntap = p.seg[sc].T;
        const uint32_t *toffs = tap_off + p.seg[sc].toff;
        const int abuf = p.nbuf == 2 ? (tc & 1) : 0;
        const uint32_t aph = (uint32_t)((p.nbuf == 2 ? (tc >> 1) : tc) & 1);
        if (!wait_bar(smem_u32(&acc_empty[abuf]), aph ^ 1, abort_flag, p.status, p.spin_limit)) break;
        tc_fence_after();
        const uint32_t d0 = tmem_base + (uint32_t)abuf * p.acc_cols;
        const uint32_t so = p.small_off;  // cross-term accumulators (BF16X3)
        const int nct = min(p.NCT, p.n_tiles - (int)(t % p.n_groups) * p.NCT);
        uint32_t acc = 0;
        bool ok = true;
        for (int cb = 0; cb < p.NCB && ok; ++cb) {
          if (!wait_bar(smem_u32(&halo_full[hs]), hph, abort_flag, p.status, p.spin_limit)) {
            ok = false;
            break;
          }
          tc_fence_after();
          // Descriptors advance by plain adds: the start-address field is the
          // low 14 bits (16-byte units) and never carries out of them here.
          const uint64_t xd_stage =
              smem_desc(halo0 + (uint32_t)hs * PARTS * p.halo_bytes, a_lbo, a_sbo);
          for (int sl = 0; sl < nsl; ++sl) {
            if (!wait_bar(smem_u32(&b_full[bs]), bph, abort_flag, p.status, p.spin_limit)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const int t0 = sl * p.TPS, t1 = min(ntap, t0 + p.TPS);
            const uint64_t wslot = wd_ring + (uint64_t)(bs * wslot16);
            for (int tap = t0; tap < t1; ++tap) {
              const uint64_t wd0 = wslot + (uint64_t)((tap - t0) * tile16);
              const uint64_t xd0 = xd_stage + (uint64_t)toffs[tap];
              if (nct == 1) {
#pragma unroll 4
                for (int s = 0; s < ksteps; ++s) {
                  const uint64_t wd = wd0 + (uint64_t)(s * wstep16);  // A: 128 output channels
                  const uint64_t xd = xd0 + (uint64_t)(s * xstep16);  // B: TU pixel groups
                  if (KIND == K_TF32) {
                    mma_tf32(d0, wd, xd, p.idesc, acc);
                  } else {
                    mma_bf16(d0, wd, xd, p.idesc, acc);
                    if (KIND == K_BF16X3) {
                      mma_bf16(d0 + so, wd + (uint64_t)wlo16, xd, p.idesc, acc);
                      mma_bf16(d0 + so, wd, xd + (uint64_t)xlo16, p.idesc, 1);
                    }
                  }
                  acc = 1;
                }
              } else {
                // two co tiles share the pixel operand; alternating between
                // their accumulators keeps N = 128 MMAs at full rate
                const uint32_t d1 = d0 + (uint32_t)p.TNA;
                const uint64_t wd1 = wd0 + (uint64_t)(p.TPS * tile16);
#pragma unroll 2
                for (int s = 0; s < ksteps; ++s) {
                  const uint64_t xd = xd0 + (uint64_t)(s * xstep16);
                  const uint64_t wa = wd0 + (uint64_t)(s * wstep16);
                  const uint64_t wb = wd1 + (uint64_t)(s * wstep16);
                  if (KIND == K_TF32) {
                    mma_tf32(d0, wa, xd, p.idesc, acc);
                    mma_tf32(d1, wb, xd, p.idesc, acc);
                  } else {
                    mma_bf16(d0, wa, xd, p.idesc, acc);
                    mma_bf16(d1, wb, xd, p.idesc, acc);
                    if (KIND == K_BF16X3) {
                      mma_bf16(d0 + so, wa + (uint64_t)wlo16, xd, p.idesc, acc);
                      mma_bf16(d1 + so, wb + (uint64_t)wlo16, xd, p.idesc, acc);
                      mma_bf16(d0 + so, wa, xd + (uint64_t)xlo16, p.idesc, 1);
                      mma_bf16(d1 + so, wb, xd + (uint64_t)xlo16, p.idesc, 1);
                    }
                  }
                  acc = 1;
                }
              }
            }
            mma_commit(smem_u32(&b_empty[bs]));
            if (++bs == p.NB) { bs = 0; bph ^= 1; }
          }
          if (!ok) break;
          mma_commit(smem_u32(&halo_empty[hs]));
          if (++hs == p.NH) { hs = 0; hph ^= 1; }
        }
        if (!ok) break;
        mma_commit(smem_u32(&acc_full[abuf]));
      }
      // Drain: every MMA issued above has completed before TMEM is freed.
      mma_commit(smem_u32(drain));
      long long t0 = clock64();
      while (!mbar_try_wait(smem_u32(drain), 0) && clock64() - t0 < kSpinLimit) {
      }
    }
  } else if (warp == kLoadWarp) {
    // ===================== B (kernel) loader =====================
    if (lane == 0) {
      // The kernel is a programmatic dependent of prep_weights: wait for that
      // grid to finish (and its weight images to be visible) before copying.
      asm volatile("griddepcontrol.wait;" ::: "memory");
      long long kb = 0;
      const uint32_t b0 = smem_u32(bring);
      int sc = 0;
      for (long long t = blockIdx.x; t < p.total_tiles; t += gridDim.x) {
        sc = MULTI ? seg_of(p, t, sc) : 0;
        const Tile tl = decode_tile(p, t, sc);
        const int nsl = p.seg[sc].NSL, ntap = p.seg[sc].T;
        const uint8_t *whi = p.wt_hi + p.seg[sc].woff;
        const uint8_t *wlo = PARTS == 2 ? p.wt_lo + p.seg[sc].woff : nullptr;
        for (int cb = 0; cb < p.NCB; ++cb)
          for (int sl = 0; sl < nsl; ++sl, ++kb) {
            const int bs = (int)(kb % p.NB);
            if (!wait_bar(smem_u32(&b_empty[bs]), (uint32_t)(((kb / p.NB) & 1) ^ 1), abort_flag,
                          p.status, p.spin_limit))
              goto loader_done;
            const int t0 = sl * p.TPS, nt_ = min(ntap - t0, p.TPS);
            const uint32_t bytes = (uint32_t)nt_ * p.tile_bytes;
            const int nct = min(p.NCT, p.n_tiles - tl.nt * p.NCT);
            const uint32_t bar = smem_u32(&b_full[bs]);
            mbar_arrive_expect_tx(bar, PARTS * bytes * (uint32_t)nct);
            // slot layout: [co tile c][tap][...], co tile c at c * TPS tiles
            for (int c = 0; c < nct; ++c) {
              const size_t src =
                  ((size_t)((tl.nt * p.NCT + c) * p.NCB + cb) * ntap + t0) * p.tile_bytes;
              const uint32_t dst = b0 + (uint32_t)bs * PARTS * p.b_bytes +
                                   (uint32_t)(c * p.TPS) * p.tile_bytes;
              for (uint32_t o = 0; o < bytes; o += 32768u) {
                const uint32_t n = min(32768u, bytes - o);
                bulk_g2s(dst + o, whi + src + o, n, bar);
                if (PARTS == 2) bulk_g2s(dst + p.b_bytes + o, wlo + src + o, n, bar);
              }
            }
          }
      }
    loader_done:
      // Wait (bounded) for the copies still in flight before the CTA exits.
      if (*abort_flag) {
        const long long first = kb > p.NB ? kb - p.NB : 0;
        for (long long q = first; q < kb; ++q) {
          long long t0 = clock64();
          const int bs = (int)(q % p.NB);
          while (!mbar_try_wait(smem_u32(&b_full[bs]), (uint32_t)((q / p.NB) & 1)) &&
                 clock64() - t0 < kSpinLimit) {
          }
        }
      }
    }
  } else if (warp >= kEpiWarp0) {
    // ===================== epilogue =====================
    const int q = warp & 3;  // TMEM lane quadrant this warp may access
    int tc = 0, sc = 0;
    for (long long t = blockIdx.x; t < p.total_tiles; t += gridDim.x, ++tc) {
      sc = MULTI ? seg_of(p, t, sc) : 0;
      const Tile tl = decode_tile(p, t, sc);
      const Seg &sg = p.seg[sc];
      const int abuf = p.nbuf == 2 ? (tc & 1) : 0;
      if (!wait_bar(smem_u32(&acc_full[abuf]), (uint32_t)((p.nbuf == 2 ? (tc >> 1) : tc) & 1),
                    abort_flag, p.status, p.spin_limit))
        break;
      tc_fence_after();
      // TMEM lane = output channel, column = pixel (group g = col / 8, v = col % 8)
      const int nct = min(p.NCT, p.n_tiles - tl.nt * p.NCT);
      for (int ct = 0; ct < nct; ++ct) {
        const int co = (tl.nt * p.NCT + ct) * 128 + q * 32 + lane;
        const bool co_ok = co < p.Cout;
        const uint32_t tcol = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)abuf * p.acc_cols +
                              (uint32_t)(ct * p.TNA);
        // Few instructions per store: this warp (quadrant 0) shares a
        // scheduler with the MMA issuer.  Element (u, v) of the tile is at
        // ytile + (u - u0) * du + (v - v0) * dv.  Streaming stores: the
        // output is not read again here, so it should not displace the
        // input halo lines the producers still read from L2.
        const float bco = (p.bias && co_ok) ? __ldg(p.bias + co) : 0.f;
        const bool epi = p.bias != nullptr || p.act != 0;
        int cy = co;
        long long yo = sg.yoff;
        if (p.fuse_n > 0) {
          const int cls = min(co / p.fuse_n, kMaxSeg - 1);
          cy = co - cls * p.fuse_n;
          yo = p.fuse_yoff[cls];
        }
        float *ytile = p.y + yo +
                       ((long long)tl.b * p.ysb + (long long)tl.ow * p.ysw +
                        (long long)tl.u0 * p.ysu + (long long)tl.v0 * p.ysv) * p.ych + cy;
        const long long du = p.ysu * (long long)p.ych, dv = p.ysv * (long long)p.ych;
        const int urows = min(p.TU, sg.OU - tl.u0), vcols = min(8, sg.OV - tl.v0);
        // four 16-column loads per wait; BF16X3 loads two of the hi*hi sums
        // and the two matching cross-term sums, and adds them
        constexpr int LD = SEP ? 2 : 4;
        // (TN is a multiple of 16 columns: a load group may end early, the
        // same for every lane, so the warp-collective loads stay uniform)
        for (int c0 = 0; c0 < p.TN; c0 += 16 * LD) {
          uint32_t r[LD][16];
#pragma unroll
          for (int k = 0; k < LD; ++k)
            if (c0 + 16 * k < p.TN) tmem_ld16(tcol + (uint32_t)(c0 + 16 * k), r[k]);
          if (SEP) {
            uint32_t r2[LD][16];
#pragma unroll
            for (int k = 0; k < LD; ++k)
              if (c0 + 16 * k < p.TN) tmem_ld16(tcol + p.small_off + (uint32_t)(c0 + 16 * k), r2[k]);
            tmem_ld_wait();
#pragma unroll
            for (int k = 0; k < LD; ++k)
#pragma unroll
              for (int e = 0; e < 16; ++e)
                r[k][e] = __float_as_uint(__uint_as_float(r[k][e]) + __uint_as_float(r2[k][e]));
          } else {
            tmem_ld_wait();
          }
          if (epi) {
#pragma unroll
            for (int k = 0; k < LD; ++k)
#pragma unroll
              for (int e = 0; e < 16; ++e) {
                float v = __uint_as_float(r[k][e]) + bco;
                if (p.act == OWLGPU_ACT_RELU) v = v > 0.f ? v : 0.f;
                r[k][e] = __float_as_uint(v);
              }
          }
          // (the next tcgen05.ld is warp-collective: no lane leaves the loop)
          if (co_ok) {
#pragma unroll
            for (int k = 0; k < LD; ++k) {
#pragma unroll
              for (int h = 0; h < 2; ++h) {
                const int ur = (c0 + 16 * k + 8 * h) >> 3;  // u row within the tile
                if (ur < urows && c0 + 16 * k < p.TN) {
                  float *row = ytile + ur * du;
                  if (vcols == 8) {
#pragma unroll
                    for (int e = 0; e < 8; ++e) __stcs(row + e * dv, __uint_as_float(r[k][8 * h + e]));
                  } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                      if (e < vcols) __stcs(row + e * dv, __uint_as_float(r[k][8 * h + e]));
                  }
                }
              }
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(smem_u32(&acc_empty[abuf]));
    }
  }
done:
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    tmem_dealloc(tmem_base, p.tmem_cols);
  }
}

// Which kernel taps a convolution uses, per view axis (w, u, v): tap t' of
// the K[a] used along axis a is original tap base[a] + mul[a] * t' of the
// KO[a] the kernel tensor has.  Forward: base 0, mul 1.  Backward-input
// (flipped kernel): base K-1, mul -1.  One residue class of a strided
// backward-input: the taps that reach it, largest first.
struct TapMap {
  int K[3], base[3], mul[3], KO[3];
};

// The B-tile images of every segment of a launch: segment c (blockIdx.y)
// has T[c] taps chosen by tm[c], its images at byte off[c] of each part.
struct PrepSegs {
  int T[kMaxSeg];
  long long off[kMaxSeg];
  TapMap tm[kMaxSeg];
  int fuse_n;  // > 0: one segment whose output channel n is class n / fuse_n
};

// Re-lay the kernel tensor into B-tile images: [ntile][cblock][tap][chunk j]
// [n < BN][16 B], element (n, k) with k = cb*CPB + j*EPC + e.  FWD reads
// W[tap][k][n]; BWDI reads the channel-exchanged kernel W[tap][n][k] (kernel
// layout [tap][Ci][Co]), taps chosen by the segment's TapMap.
template <int KIND>
__global__ void prep_weights(const float *__restrict__ w, uint8_t *__restrict__ hi_base,
                             uint8_t *__restrict__ lo_base, int Ci, int Co, int K, int N,
                             int BN, int CPB, int NCB, int n_tiles, int bwd_input,
                             const __grid_constant__ PrepSegs ps) {
  // Launched as a programmatic dependent of whatever ran before it: wait
  // for that work (the kernel tensor may be its output), then let the
  // convolution launched next start its prologue and halo staging; its
  // weight loader waits for this grid (griddepcontrol.wait).
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;");
  const int T = ps.T[blockIdx.y];
  uint8_t *hi = hi_base + ps.off[blockIdx.y];
  uint8_t *lo = lo_base ? lo_base + ps.off[blockIdx.y] : nullptr;
  constexpr int EPC = (KIND == K_TF32) ? 4 : 8;
  const int NCH = CPB / EPC;
  const long long total = (long long)n_tiles * NCB * T * NCH * BN;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int n = (int)(r % BN); r /= BN;
    const int j = (int)(r % NCH); r /= NCH;
    const int tap = (int)(r % T); r /= T;
    const int cb = (int)(r % NCB);
    const int nt = (int)(r / NCB);
    const int nf = nt * BN + n;  // output channel of the launch
    int ng = nf, seg = blockIdx.y;
    if (ps.fuse_n > 0) {  // class-fused channels: class nf / fuse_n, its channel ng
      seg = min(nf / ps.fuse_n, kMaxSeg - 1);
      ng = nf - seg * ps.fuse_n;
    }
    const TapMap &tm = ps.tm[seg];
    const int ta = tap / (tm.K[1] * tm.K[2]), tb = tap / tm.K[2] % tm.K[1], tc = tap % tm.K[2];
    const long long orig =
        ((long long)(tm.base[0] + tm.mul[0] * ta) * tm.KO[1] + (tm.base[1] + tm.mul[1] * tb)) *
            tm.KO[2] + (tm.base[2] + tm.mul[2] * tc);
    float v[EPC];
#pragma unroll
    for (int e = 0; e < EPC; ++e) {
      const int k = cb * CPB + j * EPC + e;
      float val = 0.f;
      if (k < K && nf < N) {
        val = bwd_input ? w[(orig * Ci + ng) * Co + k] : w[(orig * Ci + k) * Co + ng];
      }
      v[e] = val;
    }
    uint4 h4, l4;
    if (KIND == K_TF32) {
      h4 = make_uint4(to_tf32(v[0]), to_tf32(v[1]), to_tf32(v[2]), to_tf32(v[3]));
    } else {
      h4 = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                      pack_bf16(v[6], v[7]));
      if (KIND == K_BF16X3) {
        float rr[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) rr[e] = v[e] - bf16_round(v[e]);
        l4 = make_uint4(pack_bf16(rr[0], rr[1]), pack_bf16(rr[2], rr[3]), pack_bf16(rr[4], rr[5]),
                        pack_bf16(rr[6], rr[7]));
      }
    }
    // byte offset of (nt, cb, tap) tile, then chunk j, row n
    const long long tile = ((long long)nt * NCB + cb) * T + tap;
    const long long off = tile * (long long)NCH * BN * 16 + ((long long)j * BN + n) * 16;
    *reinterpret_cast<uint4 *>(hi + off) = h4;
    if (KIND == K_BF16X3) *reinterpret_cast<uint4 *>(lo + off) = l4;
  }
}

// The same re-layout, BF16 kinds, when the kernel tensor's channel axes are
// multiples of 4 and 16-byte aligned and no classes are fused: a thread
// takes four consecutive output channels n of one (tile, block, tap, chunk)
// and reads the 32 floats with eight 16-byte loads (along n for the forward,
// along k for backward_input), then writes the four 16-byte chunks.
template <int KIND>
__global__ void prep_weights_v4(const float *__restrict__ w, uint8_t *__restrict__ hi_base,
                                uint8_t *__restrict__ lo_base, int Ci, int Co, int K, int N,
                                int BN, int CPB, int NCB, int n_tiles, int bwd_input,
                                const __grid_constant__ PrepSegs ps) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // as prep_weights
  asm volatile("griddepcontrol.launch_dependents;");
  static_assert(KIND != K_TF32, "8-channel chunks");
  const int T = ps.T[blockIdx.y];
  uint8_t *hi = hi_base + ps.off[blockIdx.y];
  uint8_t *lo = lo_base ? lo_base + ps.off[blockIdx.y] : nullptr;
  const int NCH = CPB / 8, BN4 = BN / 4;
  const TapMap &tm = ps.tm[blockIdx.y];
  const long long total = (long long)n_tiles * NCB * T * NCH * BN4;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int n0 = (int)(r % BN4) * 4; r /= BN4;
    const int j = (int)(r % NCH); r /= NCH;
    const int tap = (int)(r % T); r /= T;
    const int cb = (int)(r % NCB);
    const int nt = (int)(r / NCB);
    const int nf0 = nt * BN + n0;
    const int ta = tap / (tm.K[1] * tm.K[2]), tb = tap / tm.K[2] % tm.K[1], tc = tap % tm.K[2];
    const long long orig =
        ((long long)(tm.base[0] + tm.mul[0] * ta) * tm.KO[1] + (tm.base[1] + tm.mul[1] * tb)) *
            tm.KO[2] + (tm.base[2] + tm.mul[2] * tc);
    const int k0 = cb * CPB + j * 8;
    float v[4][8];
    if (!bwd_input) {  // W[tap][k][n]: 16 bytes along n
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k0 + e < K && nf0 < N)
          f = __ldg(reinterpret_cast<const float4 *>(w + (orig * Ci + k0 + e) * Co + nf0));
        v[0][e] = f.x; v[1][e] = f.y; v[2][e] = f.z; v[3][e] = f.w;
      }
    } else {  // channel-exchanged W[tap][n][k]: 16 bytes along k
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int e = 0; e < 8; e += 4) {
          float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
          if (k0 + e < K && nf0 + q < N)
            f = __ldg(reinterpret_cast<const float4 *>(w + (orig * Ci + nf0 + q) * Co + k0 + e));
          v[q][e] = f.x; v[q][e + 1] = f.y; v[q][e + 2] = f.z; v[q][e + 3] = f.w;
        }
    }
    const long long tile = ((long long)nt * NCB + cb) * T + tap;
    const long long off = tile * (long long)NCH * BN * 16 + ((long long)j * BN + n0) * 16;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      *reinterpret_cast<uint4 *>(hi + off + q * 16) =
          make_uint4(pack_bf16(v[q][0], v[q][1]), pack_bf16(v[q][2], v[q][3]),
                     pack_bf16(v[q][4], v[q][5]), pack_bf16(v[q][6], v[q][7]));
      if (KIND == K_BF16X3) {
        float rr[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) rr[e] = v[q][e] - bf16_round(v[q][e]);
        *reinterpret_cast<uint4 *>(lo + off + q * 16) =
            make_uint4(pack_bf16(rr[0], rr[1]), pack_bf16(rr[2], rr[3]), pack_bf16(rr[4], rr[5]),
                       pack_bf16(rr[6], rr[7]));
      }
    }
  }
}

// A convolution seen as (w, u, v) spatial axes plus channels.
struct View {
  int B, IW, IU, IV, OW, OU, OV, KW, KU, KV, dw, du, dv, pw, pu, pv, sw, su, sv;
  long long xsb, xsw, xsu, xsv, ysb, ysw, ysu, ysv;
  int Cin, Cout;
};

// Map Owl's (cols, rows, dpts) onto (w, u, v): the 8-wide core-matrix axis v
// is the innermost non-trivial spatial axis.
View make_view(const ConvGeom &g, bool bwd_input) {
  // "in" = the array the conv reads, "out" = the array it writes.
  const long long iC = bwd_input ? g.OC : g.IC, iR = bwd_input ? g.OR : g.IR,
                  iD = bwd_input ? g.OD : g.ID;
  const long long oC = bwd_input ? g.IC : g.OC, oR = bwd_input ? g.IR : g.OR,
                  oD = bwd_input ? g.ID : g.OD;
  auto pad = [](long long k, int d, int p, bool bi) {
    return bi ? (int)((k - 1) * d - p) : p;
  };
  View v;
  v.B = (int)g.B;
  v.Cin = (int)(bwd_input ? g.Co : g.Ci);
  v.Cout = (int)(bwd_input ? g.Ci : g.Co);
  const bool flat = (iD == 1 && oD == 1 && g.KD == 1);
  if (flat) {
    v.IW = 1; v.IU = (int)iC; v.IV = (int)iR;
    v.OW = 1; v.OU = (int)oC; v.OV = (int)oR;
    v.KW = 1; v.KU = (int)g.KC; v.KV = (int)g.KR;
    v.dw = 1; v.du = g.dc; v.dv = g.dr;
    v.sw = 1; v.su = bwd_input ? 1 : g.sc; v.sv = bwd_input ? 1 : g.sr;
    v.pw = 0; v.pu = pad(g.KC, g.dc, g.pc, bwd_input); v.pv = pad(g.KR, g.dr, g.pr, bwd_input);
    v.xsw = 1; v.xsu = iR; v.xsv = 1;
    v.ysw = 1; v.ysu = oR; v.ysv = 1;
  } else {
    v.IW = (int)iC; v.IU = (int)iR; v.IV = (int)iD;
    v.OW = (int)oC; v.OU = (int)oR; v.OV = (int)oD;
    v.KW = (int)g.KC; v.KU = (int)g.KR; v.KV = (int)g.KD;
    v.dw = g.dc; v.du = g.dr; v.dv = g.dd;
    v.sw = bwd_input ? 1 : g.sc; v.su = bwd_input ? 1 : g.sr; v.sv = bwd_input ? 1 : g.sd;
    v.pw = pad(g.KC, g.dc, g.pc, bwd_input); v.pu = pad(g.KR, g.dr, g.pr, bwd_input);
    v.pv = pad(g.KD, g.dd, g.pd, bwd_input);
    v.xsw = iR * iD; v.xsu = iD; v.xsv = 1;
    v.ysw = oR * oD; v.ysu = oD; v.ysv = 1;
  }
  v.xsb = iC * iR * iD;
  v.ysb = oC * oR * oD;
  return v;
}

int num_sms() {
  static int n[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (n[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    n[dev] = v > 0 ? v : 148;
  }
  return n[dev];
}

int *status_ptr() {
  static int *p[64] = {nullptr};
  static std::mutex mu;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!p[dev]) {
    void *q = nullptr;
    if (cudaGetSymbolAddress(&q, g_tc_status) != cudaSuccess) return nullptr;
    p[dev] = static_cast<int *>(q);
  }
  return p[dev];
}

// Choose tile and pipeline sizes; false if no configuration fits.
// Priorities: the fewest halo stagings, tiles along u times co-tile groups
// (an MMA costs the same whatever its N, so a tile's MMA count does not
// depend on its height, and a tile of up to 128 pixels stages its halo once
// for two co tiles); then the widest
// channel block (fewer, fuller halo stages for the producers: a whole
// 128-channel pixel per stage when two stages fit); then the most taps per
// weight slot (fewer barrier polls between MMAs); then the lowest tile (the
// least halo).  Tile heights are even (N = 8*TU a multiple of 16) up to 32.
// `v` holds the largest halo extents of the launch's segments; t_slot is the
// most taps of one segment (weight slots), t_table the taps of all segments
// (the shared-memory tap table).
bool plan(TcParams &p, const View &v, int kind, int t_slot, int t_table) {
  const int EB = (kind == K_TF32) ? 4 : 2;
  const int parts = (kind == K_BF16X3) ? 2 : 1;
  p.BN = 128;  // output channels per tile = the MMA's M
  p.n_tiles = (v.Cout + p.BN - 1) / p.BN;
  p.T = t_slot;
  const int cb0 = std::min(256, (int)((v.Cin * EB + 31) / 32 * 32));
  bool found = false;
  TcParams best = p;
  long long best_score = 0;
  // two halo stages (staging overlaps the MMAs); one only when two do not
  // fit shared memory (wide strided halos in split-BF16)
  for (int nh = 2; nh >= 1 && !found; --nh)
  for (int tu = 32; tu >= 2; tu -= 2) {
    const long long u_tiles = (v.OU + tu - 1) / tu;
    for (int cb = cb0; cb >= 32; cb -= 32) {
      // cb0 (all channels, up to 256 bytes), then 128, 64, 32: blocks that
      // divide the channels evenly (a ragged last block costs full MMAs)
      if (cb != cb0 && cb != 128 && cb != 64 && cb != 32) continue;
      TcParams q = p;
      q.NH = nh;
      q.TU = tu;
      q.TN = 8 * tu;
      q.TNA = (q.TN + 31) / 32 * 32;
      // tiles of up to 128 pixels take two co tiles when there are two: the
      // halo is staged once for both and their MMAs alternate accumulators
      q.NCT = (q.TN <= 128 && p.n_tiles >= 2) ? 2 : 1;
      q.n_groups = (p.n_tiles + q.NCT - 1) / q.NCT;
      q.CB = cb;
      q.CPB = q.CB / EB;
      q.NCH = q.CB / 16;
      q.NCB = (v.Cin + q.CPB - 1) / q.CPB;
      q.tile_bytes = (unsigned)(q.BN * q.CB);
      q.HW = (v.KW - 1) * v.dw + 1;
      q.HU = (tu - 1) * v.su + (v.KU - 1) * v.du + 1;
      q.HVR = 8 + ((v.KV - 1) * v.dv) / v.sv;
      q.HV = v.sv * q.HVR;
      q.HP = q.HW * q.HU * q.HV;
      q.PS = q.HP + (((1 - q.HP) % 8) + 8) % 8;  // plane stride = 1 (mod 8) pixels
      if (q.PS >= 16384 || q.HV >= 16384) continue;
      q.halo_bytes = (unsigned)q.PS * 16u * (unsigned)q.NCH;
      const long long fixed = (long long)q.NH * parts * q.halo_bytes + 512 + 4LL * t_table;
      const long long room = kSmemMax - fixed;
      if (room <= 0) continue;
      // at least two weight slots
      const long long tps =
          std::min<long long>(q.T, room / (2LL * parts * q.NCT * q.tile_bytes));
      if (tps < 1) continue;
      q.TPS = (int)tps;
      q.NSL = (q.T + q.TPS - 1) / q.TPS;
      q.TPS = (q.T + q.NSL - 1) / q.NSL;  // balance the slots
      q.b_bytes = (unsigned)(q.NCT * q.TPS) * q.tile_bytes;
      q.NB = (int)std::min<long long>(4, room / ((long long)parts * q.b_bytes));
      if (q.NB < 2) continue;
      // accumulator sets: double-buffered when they fit TMEM (the epilogue
      // of one tile overlaps the next tile's MMAs), else one set
      q.small_off = (unsigned)(q.NCT * q.TNA);
      q.acc_cols = q.small_off * (unsigned)parts;
      q.nbuf = q.acc_cols * 2 <= 512 ? 2 : 1;
      if (q.acc_cols > 512) continue;
      q.tmem_cols = 32;
      while (q.tmem_cols < q.acc_cols * (unsigned)q.nbuf) q.tmem_cols <<= 1;
      // halo stagings per output: tiles along u times co-tile groups
      const long long stagings = u_tiles * q.n_groups;
      const long long score = -stagings * 1000000000000LL + (long long)q.CB * 1000000LL +
                              (long long)q.TPS * (q.NCH / 2) * 1000LL - tu;
      if (!found || score > best_score) {
        best_score = score;
        best = q;
        found = true;
      }
    }
  }
  if (!found) return false;
  p = best;
  return true;
}

// ---- weight-image cache ------------------------------------------------------
// A caller that keeps a kernel tensor unchanged across calls declares its
// contents with a version (owlgpu_weights_declare); calls whose kernel
// pointer has a declared version reuse the B-tile images built for that
// version, one per layout (the plan and tap maps a geometry needs), instead
// of re-laying the tensor out on every call.

struct WeightKey {
  int dev, kind, bwd_input, BN, CB, NCB, n_tiles, nseg, Ci, Co;
  const float *w;
  PrepSegs ps;  // zero-initialised before it is filled: compared bytewise
};

struct WeightImage {
  WeightKey key;
  uint64_t version;
  uint8_t *buf;
  size_t bytes;
  bool ready;  // built and synchronised (calls meanwhile use per-call scratch)
};

std::mutex g_wmu;
std::vector<std::pair<std::pair<int, const void *>, uint64_t>> g_declared;
std::vector<WeightImage> g_images;

bool same_key(const WeightKey &a, const WeightKey &b) {
  return std::memcmp(&a, &b, sizeof(WeightKey)) == 0;
}

// The declared version of (device, pointer); false when none.
bool declared_version(int dev, const void *w, uint64_t *v) {
  for (const auto &d : g_declared)
    if (d.first.first == dev && d.first.second == w) {
      *v = d.second;
      return true;
    }
  return false;
}

// Free the images of (device, pointer), or all of them, after the device
// has finished every queued kernel (they may still be reading them).
// Caller holds g_wmu.
int drop_images(int dev, const void *w, bool all) {
  bool any = false;
  for (const auto &im : g_images)
    if (all || (im.key.dev == dev && im.key.w == w)) any = true;
  if (!any) return kOk;
  OWL_CUDA(cudaDeviceSynchronize());
  for (size_t i = 0; i < g_images.size();) {
    WeightImage &im = g_images[i];
    if (all || (im.key.dev == dev && im.key.w == w)) {
      cudaFree(im.buf);
      g_images[i] = g_images.back();
      g_images.pop_back();
    } else {
      ++i;
    }
  }
  return kOk;
}

template <int KIND, bool MULTI>
int launch(const TcParams &p, size_t smem, cudaStream_t s, bool after_prep) {
  static bool attr_set[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    OWL_CUDA(cudaFuncSetAttribute(conv_tc_kernel<KIND, MULTI>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemMax));
    attr_set[dev] = true;
  }
  int grid = (int)std::min<long long>(p.total_tiles, num_sms());
  // programmatic dependent launch (on prep_weights when it ran just before)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // a cached weight image has no prep_weights launch before the kernel:
  // then every thread waits for the earlier work (wait_all)
  TcParams q = p;
  q.wait_all = after_prep ? 0 : 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, conv_tc_kernel<KIND, MULTI>, q);
  note_launch();
  note_tc_launch();
  if (e != cudaSuccess) return cuda_fail(e, "conv_tc_kernel");
  return kOk;
}

// One launch over a view: `x` is read, `y` written, `tm` picks the taps of
// the kernel tensor `w` ([taps][Ci][Co]); bwd_input exchanges its channels.
// One segment of a launch: a view (output extents, pads, taps), the kernel
// taps it uses, and its output origin in y (elements).
struct SegSpec {
  View v;
  TapMap tm;
  long long yoff;
};

// One launch over up to kMaxSeg segments that share the input, the channels
// and the strides: x is read, y written, `w` ([taps][Ci][Co]) re-laid out
// per segment; bwd_input exchanges its channels.
//
// fuse > 0: the segments are residue classes with one tap each and the same
// extents and pads; they run as a single segment with fuse * nseg output
// channels and a depth-to-space epilogue (sp[0].v.Cout must be fuse).
int run_segs(int prec, int nseg_in, const SegSpec *sp, bool bwd_input, int Ci, int Co,
             const float *x, const float *w, float *y, cudaStream_t s, int fuse = 0,
             const float *bias = nullptr, int act = 0) {
  const int kind = prec == OWLGPU_PREC_TF32 ? K_TF32 : (prec == OWLGPU_PREC_BF16X3 ? K_BF16X3 : K_BF16);
  // segments with work, and the union of their halo extents
  int idx[kMaxSeg], nseg = 0, spw = 0, spu = 0, spv = 0, t_slot = 0, t_table = 0;
  for (int c = 0; c < nseg_in && c < kMaxSeg; ++c) {
    const View &v = sp[c].v;
    if (v.OW * (long long)v.OU * v.OV * v.B == 0 || v.Cout == 0) continue;
    idx[nseg++] = c;
    spw = std::max(spw, (v.KW - 1) * v.dw);
    spu = std::max(spu, (v.KU - 1) * v.du);
    spv = std::max(spv, (v.KV - 1) * v.dv);
    t_slot = std::max(t_slot, v.KW * v.KU * v.KV);
    t_table += v.KW * v.KU * v.KV;
  }
  if (nseg == 0) return kOk;
  int fuse_n = 0, nclass = 1;
  long long fuse_yoff[kMaxSeg] = {0};
  TapMap fuse_tm[kMaxSeg];
  if (fuse > 0 && nseg > 1) {
    fuse_n = fuse;
    nclass = nseg;
    for (int k = 0; k < nseg; ++k) {
      fuse_yoff[k] = sp[idx[k]].yoff;
      fuse_tm[k] = sp[idx[k]].tm;
    }
    nseg = 1;  // one launch segment; the classes are output channels
    t_table = t_slot;
  }
  View pv = sp[idx[0]].v;
  if (fuse_n) pv.Cout = fuse_n * nclass;
  pv.KW = spw + 1; pv.KU = spu + 1; pv.KV = spv + 1;
  pv.dw = pv.du = pv.dv = 1;
  TcParams p{};
  if (pv.Cin == 0 || !plan(p, pv, kind, t_slot, t_table)) return kErrUnsupported;
  p.x = x; p.y = y;
  p.B = pv.B; p.IW = pv.IW; p.IU = pv.IU; p.IV = pv.IV;
  p.sw = pv.sw; p.su = pv.su; p.sv = pv.sv;
  p.xsb = pv.xsb; p.xsw = pv.xsw; p.xsu = pv.xsu; p.xsv = pv.xsv;
  p.ysb = pv.ysb; p.ysw = pv.ysw; p.ysu = pv.ysu; p.ysv = pv.ysv;
  p.Cin = pv.Cin; p.Cout = pv.Cout;
  p.ych = fuse_n ? fuse_n : pv.Cout;
  p.fuse_n = fuse_n;
  p.bias = bias;
  p.act = act;
  for (int k = 0; k < kMaxSeg; ++k) p.fuse_yoff[k] = fuse_yoff[k];
  p.nseg = nseg;
  long long tiles = 0;
  size_t woff = 0;
  int toff = 0;
  for (int k = 0; k < nseg; ++k) {
    const View &v = sp[idx[k]].v;
    Seg &g = p.seg[k];
    g.tile0 = tiles;
    g.yoff = fuse_n ? 0 : sp[idx[k]].yoff;
    g.woff = (long long)woff;
    g.OW = v.OW; g.OU = v.OU; g.OV = v.OV;
    g.u_tiles = (v.OU + p.TU - 1) / p.TU;
    g.v_tiles = (v.OV + 7) / 8;
    g.KW = v.KW; g.KU = v.KU; g.KV = v.KV;
    g.dw = v.dw; g.du = v.du; g.dv = v.dv;
    g.pw = v.pw; g.pu = v.pu; g.pv = v.pv;
    g.T = v.KW * v.KU * v.KV;
    g.NSL = (g.T + p.TPS - 1) / p.TPS;
    g.toff = toff;
    tiles += (long long)v.B * v.OW * g.u_tiles * g.v_tiles * p.n_groups;
    toff += g.T;
    woff += (size_t)p.n_tiles * p.NCB * g.T * p.tile_bytes;
  }
  p.total_tiles = tiles;
  p.idesc = instr_desc(kind == K_TF32 ? 2u : 1u, (uint32_t)p.TN);
  // 1: 16-byte vector loads; 2: 32-byte aligned chunks (one load per chunk)
  p.vec_in = ((uintptr_t)x % 32 == 0 && pv.Cin % 8 == 0)
                 ? 2
                 : (((uintptr_t)x % 16 == 0) && (pv.Cin % 4 == 0) ? 1 : 0);
  p.spin_limit = wait_limit();
  p.status = status_ptr();
  if (!p.status) {
    set_error("conv_tc: cannot locate device status word");
    return kErrCuda;
  }
  const int parts = kind == K_BF16X3 ? 2 : 1;
  const size_t wt_bytes = woff;
  // the images of every segment (blockIdx.y of prep_weights = segment)
  PrepSegs ps;
  std::memset(&ps, 0, sizeof(ps));
  for (int k = 0; k < nseg; ++k) {
    ps.T[k] = p.seg[k].T;
    ps.off[k] = p.seg[k].woff;
    ps.tm[k] = sp[idx[k]].tm;
  }
  if (fuse_n) {
    ps.fuse_n = fuse_n;
    // channels past the last class (tile padding) read no weight; their
    // map entry is any valid one
    for (int k = 0; k < kMaxSeg; ++k) ps.tm[k] = fuse_tm[k < nclass ? k : 0];
  }
  // a declared kernel tensor: reuse (or build, outside stream capture) its
  // cached images; otherwise re-lay it out into per-call scratch
  WeightKey key;
  std::memset(&key, 0, sizeof(key));
  cudaGetDevice(&key.dev);
  key.kind = kind; key.bwd_input = bwd_input ? 1 : 0; key.BN = p.BN; key.CB = p.CB;
  key.NCB = p.NCB; key.n_tiles = p.n_tiles; key.nseg = nseg; key.Ci = Ci; key.Co = Co;
  key.w = w;
  key.ps = ps;
  uint8_t *cached = nullptr;
  bool build_cached = false;
  {
    std::lock_guard<std::mutex> lk(g_wmu);
    uint64_t ver = 0;
    if (declared_version(key.dev, w, &ver)) {
      bool present = false;
      for (const WeightImage &im : g_images)
        if (im.version == ver && same_key(im.key, key)) {
          present = true;
          if (im.ready) cached = im.buf;
        }
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (!present && cudaStreamIsCapturing(s, &cs) == cudaSuccess &&
          cs == cudaStreamCaptureStatusNone) {
        void *buf = nullptr;
        if (cudaMalloc(&buf, wt_bytes * parts) == cudaSuccess) {
          g_images.push_back({key, ver, (uint8_t *)buf, wt_bytes * parts, false});
          cached = (uint8_t *)buf;
          build_cached = true;
        } else {
          cudaGetLastError();  // no room for an image: per-call scratch instead
        }
      }
    }
  }
  void *wt = cached;
  int rc = kOk;
  if (!cached) {
    rc = scratch_alloc(&wt, wt_bytes * parts, s);
    if (rc) return rc;
  }
  p.wt_hi = (const uint8_t *)wt;
  p.wt_lo = parts == 2 ? (const uint8_t *)wt + wt_bytes : nullptr;
  const bool prep = !cached || build_cached;
  if (prep) {
    uint8_t *hi = (uint8_t *)wt;
    uint8_t *lo = parts == 2 ? (uint8_t *)wt + wt_bytes : nullptr;
    const long long n = (long long)p.n_tiles * p.NCB * t_slot * p.NCH * p.BN;
    const dim3 grid((unsigned)std::min<long long>((n + 255) / 256, 4096), (unsigned)nseg);
    const int K = pv.Cin, N = pv.Cout;
    // the vector re-layout: 16-byte loads along the kernel tensor's Co axis
    // (n for the forward, k for backward_input) and whole 4-channel groups
    const bool v4 = kind != K_TF32 && !fuse_n && (uintptr_t)w % 16 == 0 && Co % 4 == 0 &&
                    K % 4 == 0 && N % 4 == 0 && p.BN % 4 == 0;
    cudaError_t e;
    if (v4) {
      const dim3 g4((unsigned)std::min<long long>((n / 4 + 255) / 256, 4096), (unsigned)nseg);
      if (kind == K_BF16X3)
        e = launch_pdl(prep_weights_v4<K_BF16X3>, g4, dim3(256), 0, s, w, hi, lo, Ci, Co, K, N,
                       p.BN, p.CPB, p.NCB, p.n_tiles, (int)bwd_input, ps);
      else
        e = launch_pdl(prep_weights_v4<K_BF16>, g4, dim3(256), 0, s, w, hi, (uint8_t *)nullptr,
                       Ci, Co, K, N, p.BN, p.CPB, p.NCB, p.n_tiles, (int)bwd_input, ps);
    } else if (kind == K_TF32)
      e = launch_pdl(prep_weights<K_TF32>, grid, dim3(256), 0, s, w, hi, (uint8_t *)nullptr, Ci,
                     Co, K, N, p.BN, p.CPB, p.NCB, p.n_tiles, (int)bwd_input, ps);
    else if (kind == K_BF16X3)
      e = launch_pdl(prep_weights<K_BF16X3>, grid, dim3(256), 0, s, w, hi, lo, Ci, Co, K, N,
                     p.BN, p.CPB, p.NCB, p.n_tiles, (int)bwd_input, ps);
    else
      e = launch_pdl(prep_weights<K_BF16>, grid, dim3(256), 0, s, w, hi, (uint8_t *)nullptr, Ci,
                     Co, K, N, p.BN, p.CPB, p.NCB, p.n_tiles, (int)bwd_input, ps);
    if (e == cudaSuccess) e = cudaGetLastError();
    note_launch();
    if (e != cudaSuccess) {
      if (!cached) scratch_free(wt, s);
      return cuda_fail(e, "prep_weights");
    }
    if (build_cached) {
      // the image is complete before any call, on any stream, reads it
      OWL_CUDA(cudaStreamSynchronize(s));
      std::lock_guard<std::mutex> lk(g_wmu);
      for (WeightImage &im : g_images)
        if (im.buf == wt) im.ready = true;
    }
  }
  const size_t smem = (size_t)p.NH * parts * p.halo_bytes + (size_t)p.NB * parts * p.b_bytes +
                      (2 * p.NH + 2 * p.NB + 5) * 8 + 16 + 4 * (size_t)t_table;
  const bool multi = p.nseg > 1;
  const bool pdl = prep && !build_cached;
  if (kind == K_TF32)
    rc = multi ? launch<K_TF32, true>(p, smem, s, pdl) : launch<K_TF32, false>(p, smem, s, pdl);
  else if (kind == K_BF16X3)
    rc = multi ? launch<K_BF16X3, true>(p, smem, s, pdl) : launch<K_BF16X3, false>(p, smem, s, pdl);
  else rc = multi ? launch<K_BF16, true>(p, smem, s, pdl) : launch<K_BF16, false>(p, smem, s, pdl);
  if (!cached) scratch_free(wt, s);
  return rc;
}

int run_view(int prec, const View &v, const TapMap &tm, bool bwd_input, int Ci, int Co,
             const float *x, const float *w, float *y, cudaStream_t s,
             const float *bias = nullptr, int act = 0) {
  SegSpec sp{v, tm, 0};
  return run_segs(prec, 1, &sp, bwd_input, Ci, Co, x, w, y, s, 0, bias, act);
}

// The whole kernel over a geometry: forward, or stride-1 backward-input
// (a forward convolution of dY with the flipped, channel-exchanged kernel).
int run(int prec, const ConvGeom &g, bool bwd_input, const float *x, const float *w, float *y,
        cudaStream_t s, const float *bias = nullptr, int act = 0) {
  if (bwd_input && (g.sc != 1 || g.sr != 1 || g.sd != 1)) return kErrUnsupported;
  if (g.sc > 8 || g.sr > 8 || g.sd > 8) return kErrUnsupported;
  const View v = make_view(g, bwd_input);
  TapMap tm;
  const int KO[3] = {v.KW, v.KU, v.KV};
  for (int a = 0; a < 3; ++a) {
    tm.K[a] = KO[a];
    tm.KO[a] = KO[a];
    tm.base[a] = bwd_input ? KO[a] - 1 : 0;
    tm.mul[a] = bwd_input ? -1 : 1;
  }
  return run_view(prec, v, tm, bwd_input, (int)g.Ci, (int)g.Co, x, w, y, s, bias, act);
}

// Strided backward-input by residue classes.  With forward x index
// s*o - p + t*d, output element i = s*a + r of dX receives dY[o] W[t] for
// the taps with (r + p - t*d) divisible by s, at o = a + (r + p - t*d)/s.
// Those taps, largest first, form a stride-1 correlation of dY with
// dilation d/g (g = gcd(s, d)) and pad -min((r + p - t*d)/s); its output
// is the sub-grid i = s*a + r of dX.  The classes together do exactly the
// multiply-adds of the backward pass (no zero-stuffed dY).  Classes that no
// tap reaches are zero; dX is cleared first when there are any.
int run_bwd_input_strided(int prec, const ConvGeom &g, float *dx, const float *w,
                          const float *dy, cudaStream_t s) {
  const View full = make_view(g, true);  // dY -> dX extents and strides
  const bool flat = (g.ID == 1 && g.OD == 1 && g.KD == 1);
  // per view axis (w, u, v): stride, dilation, forward pad, kernel size
  int S[3], D[3], P[3], KO[3];
  if (flat) {
    S[0] = 1; D[0] = 1; P[0] = 0; KO[0] = 1;
    S[1] = g.sc; D[1] = g.dc; P[1] = g.pc; KO[1] = (int)g.KC;
    S[2] = g.sr; D[2] = g.dr; P[2] = g.pr; KO[2] = (int)g.KR;
  } else {
    S[0] = g.sc; D[0] = g.dc; P[0] = g.pc; KO[0] = (int)g.KC;
    S[1] = g.sr; D[1] = g.dr; P[1] = g.pr; KO[1] = (int)g.KR;
    S[2] = g.sd; D[2] = g.dd; P[2] = g.pd; KO[2] = (int)g.KD;
  }
  const int I[3] = {full.OW, full.OU, full.OV};  // dX extents
  const long long YS[3] = {full.ysw, full.ysu, full.ysv};
  struct Axis {
    int K, base, mul, dil, pad, out;
  };
  // classes of one axis
  auto axis_class = [&](int a, int r, Axis &ax) {
    int tmax = -1, n = 0;
    for (int t = 0; t < KO[a]; ++t)
      if ((((r + P[a] - t * D[a]) % S[a]) + S[a]) % S[a] == 0) {
        tmax = t > tmax ? t : tmax;
        ++n;
      }
    int gg = S[a], dd = D[a];
    while (dd) { const int t = gg % dd; gg = dd; dd = t; }  // gcd(s, d)
    ax.K = n;
    ax.base = tmax;
    ax.mul = -(S[a] / gg);
    ax.dil = D[a] / gg;
    ax.pad = n ? -((r + P[a] - tmax * D[a]) / S[a]) : 0;
    ax.out = I[a] > r ? (I[a] - r + S[a] - 1) / S[a] : 0;
    return n > 0;
  };
  bool any_empty = false;
  for (int a = 0; a < 3; ++a)
    for (int r = 0; r < S[a]; ++r) {
      Axis ax;
      if (!axis_class(a, r, ax) && ax.out > 0) any_empty = true;
    }
  if (any_empty)
    OWL_CUDA(cudaMemsetAsync(dx, 0, sizeof(float) * (size_t)g.x_elems(), s));
  // the classes that receive taps
  std::vector<SegSpec> segs;
  for (int r0 = 0; r0 < S[0]; ++r0)
    for (int r1 = 0; r1 < S[1]; ++r1)
      for (int r2 = 0; r2 < S[2]; ++r2) {
        Axis ax[3];
        const int rr[3] = {r0, r1, r2};
        bool ok = true;
        for (int a = 0; a < 3; ++a) ok = axis_class(a, rr[a], ax[a]) && ok;
        if (!ok || ax[0].out * ax[1].out * ax[2].out == 0) continue;
        View v = full;
        v.OW = ax[0].out; v.OU = ax[1].out; v.OV = ax[2].out;
        v.KW = ax[0].K; v.KU = ax[1].K; v.KV = ax[2].K;
        v.dw = ax[0].dil; v.du = ax[1].dil; v.dv = ax[2].dil;
        v.pw = ax[0].pad; v.pu = ax[1].pad; v.pv = ax[2].pad;
        v.sw = v.su = v.sv = 1;
        v.ysw = YS[0] * S[0]; v.ysu = YS[1] * S[1]; v.ysv = YS[2] * S[2];
        segs.emplace_back();
        SegSpec &sg = segs.back();
        sg.v = v;
        sg.yoff = (r0 * YS[0] + r1 * YS[1] + r2 * YS[2]) * (long long)g.Ci;
        for (int a = 0; a < 3; ++a) {
          sg.tm.K[a] = ax[a].K;
          sg.tm.base[a] = ax[a].base;
          sg.tm.mul[a] = ax[a].mul;
          sg.tm.KO[a] = KO[a];
        }
      }
  // One tap per class with common extents and pads (kernel <= stride, as in
  // a stride-s transpose convolution with kernel s): all classes read the
  // same dY pixel for an output tile, so they run as one 1x1 convolution
  // to classes * Ci channels with a depth-to-space epilogue.
  bool fuse = segs.size() > 1 && segs.size() <= (size_t)kMaxSeg;
  for (const SegSpec &sg : segs) {
    const View &a = sg.v, &b0 = segs[0].v;
    fuse = fuse && a.KW * a.KU * a.KV == 1 && a.OW == b0.OW && a.OU == b0.OU &&
           a.OV == b0.OV && a.pw == b0.pw && a.pu == b0.pu && a.pv == b0.pv;
  }
  if (fuse)
    return run_segs(prec, (int)segs.size(), segs.data(), true, (int)g.Ci, (int)g.Co, dy, w, dx,
                    s, (int)g.Ci);
  for (size_t k0 = 0; k0 < segs.size(); k0 += kMaxSeg) {
    const int n = (int)std::min<size_t>(kMaxSeg, segs.size() - k0);
    const int rc = run_segs(prec, n, segs.data() + k0, true, (int)g.Ci, (int)g.Co, dy, w, dx, s);
    if (rc) return rc;
  }
  return kOk;
}

}  // namespace

int weights_declare(const void *w, uint64_t version) {
  int dev = 0;
  OWL_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_wmu);
  for (auto &d : g_declared)
    if (d.first.first == dev && d.first.second == w) {
      if (d.second == version) return kOk;
      d.second = version;
      return drop_images(dev, w, false);
    }
  g_declared.push_back({{dev, w}, version});
  return kOk;
}

int weights_forget(const void *w) {
  int dev = 0;
  OWL_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_wmu);
  for (size_t i = 0; i < g_declared.size(); ++i)
    if (g_declared[i].first.first == dev && g_declared[i].first.second == w) {
      g_declared[i] = g_declared.back();
      g_declared.pop_back();
      break;
    }
  return drop_images(dev, w, false);
}

int weights_drop_all() {
  std::lock_guard<std::mutex> lk(g_wmu);
  return drop_images(0, nullptr, true);
}

int tc_conv_fwd(int prec, const ConvGeom &g, const float *x, const float *w, float *y,
                cudaStream_t s, const float *bias, int act) {
  return run(prec, g, false, x, w, y, s, bias, act);
}

int tc_conv_bwd_input(int prec, const ConvGeom &g, float *dx, const float *w, const float *dy,
                      cudaStream_t s) {
  if (g.sc == 1 && g.sr == 1 && g.sd == 1) return run(prec, g, true, dy, w, dx, s);
  if (g.sc > 8 || g.sr > 8 || g.sd > 8) return kErrUnsupported;
  return run_bwd_input_strided(prec, g, dx, w, dy, s);
}

// The tensor-core kernels' status words (convolution, weight gradient,
// GEMM), read with one synchronisation and cleared when set.
// The three status words are copied into page-locked host memory of the
// calling thread, so the copies are asynchronous and a host drop-in call can
// enqueue them before its final synchronisation instead of after it.
int *status_host() {
  static thread_local int *h = nullptr;
  if (!h) {
    void *q = nullptr;
    if (cudaHostAlloc(&q, 4 * sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    h = static_cast<int *>(q);
  }
  return h;
}

int tc_status_enqueue(cudaStream_t s) {
  int *w[3] = {status_ptr(), tc_wgrad_status_word(), tc_gemm_status_word()};
  int *h = status_host();
  if (!w[0] || !w[1] || !w[2] || !h) return kErrCuda;
  for (int i = 0; i < 3; ++i)
    OWL_CUDA(cudaMemcpyAsync(&h[i], w[i], sizeof(int), cudaMemcpyDeviceToHost, s));
  return kOk;
}

int tc_status_take(int *out, cudaStream_t s) {
  int *w[3] = {status_ptr(), tc_wgrad_status_word(), tc_gemm_status_word()};
  const int *h = status_host();
  if (!w[0] || !w[1] || !w[2] || !h) return kErrCuda;
  for (int i = 0; i < 3; ++i)
    if (h[i]) OWL_CUDA(cudaMemsetAsync(w[i], 0, sizeof(int), s));
  *out = h[0] | h[1] | h[2];
  return kOk;
}

int tc_read_status(int *out, cudaStream_t s) {
  int rc = tc_status_enqueue(s);
  if (rc) return rc;
  OWL_CUDA(cudaStreamSynchronize(s));
  return tc_status_take(out, s);
}

}  // namespace owlgpu
