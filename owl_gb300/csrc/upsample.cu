// upsample.cu -- nearest-neighbour 2-D upsampling (Owl's upsampling2d) and
// its backward, float32 and float64 (complex32 / complex64 as twice the
// channels of their real parts).
//
// Forward: Owl computes upsampling2d as `repeat x [|1; sc; sr; 1|]`
// (owl_dense_ndarray_generic.ml:8223-8233):
//   y[b][c][r][ch] = x[b][c / sc][r / sr][ch].
// Backward: stub_*_ndarray_upsampling_spatial_backward
// (owl_ndarray_upsampling_impl.h:9-58) zero-fills dx and, for every output
// position in order (col outer, row inner), adds dy into the input position
// (min(c / sc, IC - 1), min(r / sr, IR - 1)).  Here one thread owns one input
// vector and gathers its block in that same order, so the float sums are
// identical and no atomics are needed; the last input col/row also collects
// any output cols/rows past IC*sc / IR*sr, as the stub's clamp does.
//
// Both kernels stream HBM with one thread per 16-byte channel vector of the
// input when the channel count and pointers allow (else per element); a
// block row is one (batch, input col) line, so the index arithmetic inside
// is 32-bit.
#include <algorithm>

#include "../../include/owlgpu.h"
#include "common.cuh"

namespace owlgpu {
namespace {

__device__ __forceinline__ float4 vadd(float4 a, float4 b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ double2 vadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float vadd(float a, float b) { return a + b; }
__device__ __forceinline__ double vadd(double a, double b) { return a + b; }

template <typename V>
__device__ __forceinline__ V vzero() {
  V v;
  memset(&v, 0, sizeof(V));
  return v;
}

template <typename V>
__device__ __forceinline__ void st_stream(V *p, V v) {
  __stcs(p, v);
}

// One thread per input vector (rows = B * IC input lines of IR * nv
// vectors): read it once, write its sc x sr copies with streaming stores.
// Forward extents are exact (OC = IC * sc, OR = IR * sr).
template <typename V>
__global__ void upsample_fwd_kernel(const V *__restrict__ x, V *__restrict__ y, long long rows,
                                    int IC, int IR, int OC, int OR, int nv, int sc, int sr) {
  const int n = IR * nv;
  for (long long row = blockIdx.y; row < rows; row += gridDim.y) {
    const long long b = row / IC;
    const int ic = (int)(row - b * IC);
    const V *xl = x + row * (long long)n;
    V *yb = y + (b * OC + (long long)ic * sc) * (long long)OR * nv;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const int ir = i / nv, v = i - ir * nv;
      const V val = __ldg(xl + i);
      V *yp = yb + (long long)ir * sr * nv + v;
      for (int dc = 0; dc < sc; ++dc, yp += (long long)OR * nv)
        for (int dr = 0; dr < sr; ++dr) st_stream(yp + (long long)dr * nv, val);
    }
  }
}

// One thread per input vector: the dy vectors of its block are loaded eight
// at a time before they are added, in the stub's order (col outer, row
// inner), so the sum is the same as one add at a time.
template <typename V>
__global__ void upsample_bwd_kernel(V *__restrict__ dx, const V *__restrict__ dy,
                                    long long rows, int IC, int IR, int OC, int OR, int nv,
                                    int sc, int sr) {
  constexpr int kBatch = 8;
  const int n = IR * nv;
  for (long long row = blockIdx.y; row < rows; row += gridDim.y) {
    const long long b = row / IC;
    const int ic = (int)(row - b * IC);
    const int c0 = ic * sc, c1 = ic == IC - 1 ? OC : min(OC, c0 + sc);
    const V *dyb = dy + b * OC * (long long)OR * nv;
    V *dxl = dx + row * (long long)n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const int ir = i / nv, v = i - ir * nv;
      const int r0 = ir * sr, r1 = ir == IR - 1 ? OR : min(OR, r0 + sr);
      const int nr = max(r1 - r0, 0), total = max(c1 - c0, 0) * nr;
      V acc = vzero<V>();
      for (int k0 = 0; k0 < total; k0 += kBatch) {
        V t[kBatch];
#pragma unroll
        for (int q = 0; q < kBatch; ++q) {
          const int k = k0 + q;
          if (k < total) {
            const int c = c0 + k / nr, r = r0 + k - (k / nr) * nr;
            t[q] = __ldg(dyb + ((long long)c * OR + r) * nv + v);
          }
        }
#pragma unroll
        for (int q = 0; q < kBatch; ++q)
          if (k0 + q < total) acc = vadd(acc, t[q]);
      }
      dxl[i] = acc;
    }
  }
}

template <typename V>
int launch_up(bool fwd, const UpGeom &g, const void *x, void *y, int nv, cudaStream_t s) {
  const long long rows = g.B * g.IC;
  const long long n = (long long)g.IR * nv;
  if (rows == 0 || n == 0) return kOk;
  const int threads = 256;
  const dim3 grid((unsigned)std::min<long long>((n + threads - 1) / threads, 64),
                  (unsigned)std::min<long long>(rows, 65535));
  if (fwd)
    upsample_fwd_kernel<V><<<grid, threads, 0, s>>>((const V *)x, (V *)y, rows, (int)g.IC,
                                                    (int)g.IR, (int)g.OC, (int)g.OR, nv, g.sc,
                                                    g.sr);
  else
    upsample_bwd_kernel<V><<<grid, threads, 0, s>>>((V *)y, (const V *)x, rows, (int)g.IC,
                                                    (int)g.IR, (int)g.OC, (int)g.OR, nv, g.sc,
                                                    g.sr);
  OWL_CHECK_LAUNCH(fwd ? "upsample_fwd_kernel" : "upsample_bwd_kernel");
  return kOk;
}

// x: the array read, y: the array written (forward: input -> output;
// backward: dy -> dx).
int run_up(Dtype dt, bool fwd, const UpGeom &g, const void *x, void *y, cudaStream_t s) {
  // A complex element is two reals that are copied and summed independently:
  // the same pass over twice the channels, in the same order.
  if (dt == C32 || dt == C64) {
    UpGeom h = g;
    h.Ch *= 2;
    return run_up(dt == C32 ? F32 : F64, fwd, h, x, y, s);
  }
  const int64_t lim = 1LL << 31;
  if (std::max(g.OR, g.IR) * g.Ch >= lim || std::max(g.OC, g.OR) >= lim ||
      g.IC * g.sc >= lim || g.IR * g.sr >= lim) {
    set_error("upsampling: a (batch, col) line exceeds 2^31 elements");
    return kErrInvalid;
  }
  const bool al = (uintptr_t)x % 16 == 0 && (uintptr_t)y % 16 == 0;
  if (dt == F32) {
    if (al && g.Ch % 4 == 0) return launch_up<float4>(fwd, g, x, y, (int)(g.Ch / 4), s);
    return launch_up<float>(fwd, g, x, y, (int)g.Ch, s);
  }
  if (al && g.Ch % 2 == 0) return launch_up<double2>(fwd, g, x, y, (int)(g.Ch / 2), s);
  return launch_up<double>(fwd, g, x, y, (int)g.Ch, s);
}

}  // namespace

int upsample_fwd(Dtype dt, const UpGeom &g, const void *x, void *y, cudaStream_t s) {
  return run_up(dt, true, g, x, y, s);
}

int upsample_bwd(Dtype dt, const UpGeom &g, void *dx, const void *dy, cudaStream_t s) {
  return run_up(dt, false, g, dy, dx, s);
}

}  // namespace owlgpu
