// tc_stage.cuh -- producer-side staging of float32 activations into the
// tensor-core operand layout [16-byte channel chunk][pixel][16 B], converted
// to bf16 (round to nearest), tf32 (round to nearest, ties away) or bf16
// hi + lo (the lo part lo_off bytes after the hi part).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace owlgpu {
namespace stage {

enum Kind { K_BF16 = 0, K_TF32 = 1, K_BF16X3 = 2 };

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

// 8 floats in one 32-byte load through the read-only path (p 32-byte
// aligned): one L1 wavefront per lane where two 16-byte loads take two.
__device__ __forceinline__ void ld8(const float *p, float *v) {
  asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]),
                 "=f"(v[6]), "=f"(v[7])
               : "l"(p));
}

// EPC floats from src: vec 2 = 32-byte aligned (one 32-byte load when EPC
// is 8), else 16-byte vector loads.
template <int EPC>
__device__ __forceinline__ void load_vec(const float *src, int vec, float *v) {
  if (EPC == 8 && vec >= 2) {
    ld8(src, v);
  } else {
#pragma unroll
    for (int e = 0; e < EPC; e += 4) {
      float4 f = __ldg(reinterpret_cast<const float4 *>(src + e));
      v[e] = f.x; v[e + 1] = f.y; v[e + 2] = f.z; v[e + 3] = f.w;
    }
  }
}

template <int KIND, int EPC>
__device__ __forceinline__ void put_chunk(uint8_t *dst, uint32_t lo_off, const float (&v)[EPC]) {
  uint4 hi;
  if (KIND == K_TF32) {
    hi = make_uint4(to_tf32(v[0]), to_tf32(v[1]), to_tf32(v[2]), to_tf32(v[3]));
  } else {
    hi = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                    pack_bf16(v[6], v[7]));
  }
  *reinterpret_cast<uint4 *>(dst) = hi;
  if (KIND == K_BF16X3) {
    float r[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) r[e] = v[e] - bf16_round(v[e]);
    *reinterpret_cast<uint4 *>(dst + lo_off) = make_uint4(
        pack_bf16(r[0], r[1]), pack_bf16(r[2], r[3]), pack_bf16(r[4], r[5]), pack_bf16(r[6], r[7]));
  }
}

// One row of `npix` pixels: pixel i lives at rowp + i*pstep floats, is in
// range when 0 <= vfirst + i*vstride < vlim; whole row invalid when !ok.
struct Row {
  const float *rowp;
  long long pstep;
  int vfirst, vstride, vlim;
  bool ok;
};

// Stage nrows rows (this warp takes rows warp, warp + nwarps, ...), each
// npix pixels x nch chunks of EPC channels; chunk j of row pixel i goes to
// dst + j*plane_bytes + (r*npix + i)*16.  `clim` = channels available from
// the block start (chunks past it are zero).  Loads are issued BATCH slots
// per lane at a time before any conversion, so each lane keeps BATCH
// requests in flight.
template <int KIND, int EPC, int BATCH, class RowFn>
__device__ __forceinline__ void stage_rows(uint8_t *dst, uint32_t lo_off, uint32_t plane_bytes,
                                           int nrows, int npix, int nch, int clim, int vec,
                                           int warp, int nwarps, int lane, RowFn rowfn) {
  const int S = npix * nch;
  const int nsh = (nch & (nch - 1)) == 0 ? __ffs(nch) - 1 : -1;
  for (int r = warp; r < nrows; r += nwarps) {
    const Row row = rowfn(r);
    for (int s0 = 0; s0 < S; s0 += 32 * BATCH) {
      float v[BATCH][EPC];
      int off[BATCH];
#pragma unroll
      for (int q = 0; q < BATCH; ++q) {
        const int sl = s0 + lane + 32 * q;
#pragma unroll
        for (int e = 0; e < EPC; ++e) v[q][e] = 0.f;
        off[q] = -1;
        if (sl < S) {
          const int i = nsh >= 0 ? (sl >> nsh) : sl / nch;
          const int j = sl - i * nch;
          off[q] = (int)(j * plane_bytes) + (r * npix + i) * 16;
          const int vv = row.vfirst + i * row.vstride;
          const int c = j * EPC;
          if (row.ok && vv >= 0 && vv < row.vlim && c < clim) {
            const float *src = row.rowp + (long long)i * row.pstep + c;
            if (vec && c + EPC <= clim) {
load_vec<EPC>(src, vec, v[q]);
            } else {
#pragma unroll
              for (int e = 0; e < EPC; ++e)
                if (c + e < clim) v[q][e] = __ldg(src + e);
            }
          }
        }
      }
#pragma unroll
      for (int q = 0; q < BATCH; ++q)
        if (off[q] >= 0) put_chunk<KIND, EPC>(dst + off[q], lo_off, v[q]);
    }
  }
}

}  // namespace stage
}  // namespace owlgpu

namespace owlgpu {
namespace stage {

// One operand tile for stage_rows2: nrows rows of npix pixels x nch chunks,
// chunk j of row r pixel i at dst + j*plane_bytes + (r*npix + i)*16.
struct RowSet {
  uint8_t *dst;
  uint32_t lo_off, plane_bytes;
  int nrows, npix, nch, clim;
};

// Stage two row sets in the same passes: warp w takes row w (+ k*nwarps)
// of each set and issues the loads of both rows before converting either,
// so a tile whose two sets have at most nwarps rows each costs every warp a
// single round trip to memory.
template <int KIND, int EPC, int BA, int BB, class FnA, class FnB>
__device__ __forceinline__ void stage_rows2(const RowSet &A, FnA rowa, const RowSet &Bs,
                                            FnB rowb, int vec, int warp, int nwarps,
                                            int lane) {
  const int SA = A.npix * A.nch, SB = Bs.npix * Bs.nch;
  const int nshA = (A.nch & (A.nch - 1)) == 0 ? __ffs(A.nch) - 1 : -1;
  const int nshB = (Bs.nch & (Bs.nch - 1)) == 0 ? __ffs(Bs.nch) - 1 : -1;
  const int nr = max(A.nrows, Bs.nrows);
  for (int r = warp; r < nr; r += nwarps) {
    const bool hasA = r < A.nrows, hasB = r < Bs.nrows;
    Row ra, rb;
    ra.ok = rb.ok = false;
    if (hasA) ra = rowa(r);
    if (hasB) rb = rowb(r);
    const int passes = max(hasA ? (SA + 32 * BA - 1) / (32 * BA) : 0,
                           hasB ? (SB + 32 * BB - 1) / (32 * BB) : 0);
    for (int ps = 0; ps < passes; ++ps) {
      float va[BA][EPC], vb[BB][EPC];
      int oa[BA], ob[BB];
#pragma unroll
      for (int q = 0; q < BA; ++q) {
        const int sl = ps * 32 * BA + lane + 32 * q;
#pragma unroll
        for (int e = 0; e < EPC; ++e) va[q][e] = 0.f;
        oa[q] = -1;
        if (hasA && sl < SA) {
          const int i = nshA >= 0 ? (sl >> nshA) : sl / A.nch;
          const int j = sl - i * A.nch;
          oa[q] = (int)(j * A.plane_bytes) + (r * A.npix + i) * 16;
          const int vv = ra.vfirst + i * ra.vstride, c = j * EPC;
          if (ra.ok && vv >= 0 && vv < ra.vlim && c < A.clim) {
            const float *src = ra.rowp + (long long)i * ra.pstep + c;
            if (vec && c + EPC <= A.clim) {
load_vec<EPC>(src, vec, va[q]);
            } else {
#pragma unroll
              for (int e = 0; e < EPC; ++e)
                if (c + e < A.clim) va[q][e] = __ldg(src + e);
            }
          }
        }
      }
#pragma unroll
      for (int q = 0; q < BB; ++q) {
        const int sl = ps * 32 * BB + lane + 32 * q;
#pragma unroll
        for (int e = 0; e < EPC; ++e) vb[q][e] = 0.f;
        ob[q] = -1;
        if (hasB && sl < SB) {
          const int i = nshB >= 0 ? (sl >> nshB) : sl / Bs.nch;
          const int j = sl - i * Bs.nch;
          ob[q] = (int)(j * Bs.plane_bytes) + (r * Bs.npix + i) * 16;
          const int vv = rb.vfirst + i * rb.vstride, c = j * EPC;
          if (rb.ok && vv >= 0 && vv < rb.vlim && c < Bs.clim) {
            const float *src = rb.rowp + (long long)i * rb.pstep + c;
            if (vec && c + EPC <= Bs.clim) {
load_vec<EPC>(src, vec, vb[q]);
            } else {
#pragma unroll
              for (int e = 0; e < EPC; ++e)
                if (c + e < Bs.clim) vb[q][e] = __ldg(src + e);
            }
          }
        }
      }
#pragma unroll
      for (int q = 0; q < BA; ++q)
        if (oa[q] >= 0) put_chunk<KIND, EPC>(A.dst + oa[q], A.lo_off, va[q]);
#pragma unroll
      for (int q = 0; q < BB; ++q)
        if (ob[q] >= 0) put_chunk<KIND, EPC>(Bs.dst + ob[q], Bs.lo_off, vb[q]);
    }
  }
}

}  // namespace stage
}  // namespace owlgpu
