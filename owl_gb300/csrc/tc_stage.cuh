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
                                           int nrows, int npix, int nch, int clim, bool vec,
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
#pragma unroll
              for (int e = 0; e < EPC; e += 4) {
                float4 f = __ldg(reinterpret_cast<const float4 *>(src + e));
                v[q][e] = f.x; v[q][e + 1] = f.y; v[q][e + 2] = f.z; v[q][e + 3] = f.w;
              }
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
