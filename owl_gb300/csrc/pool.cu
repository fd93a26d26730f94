// pool.cu -- max / average pooling, forward and backward, 2-D and 3-D,
// float32 and float64, with Owl's exact semantics
// (src/owl/core/owl_ndarray_pool_impl.h):
//   * window scan order: cols outer, rows, dpts inner; out-of-range taps
//     skipped (:60-77, :282-300);
//   * max: accumulator starts at -inf, replaced only when `acc < t`, so the
//     first maximum in scan order wins and NaN is never selected (:20-23 of
//     owl_ndarray_pool_stub.c); argmax is the flat index into the whole input
//     (batch offset included), -1 when nothing was selected (:516-527);
//   * avg: sum in the element type, in scan order, divided by the in-range
//     count (:71-79);
//   * backward: max routes dY to the recomputed argmax with max_idx
//     starting at 0 (:167); avg adds dY / count to every in-range element
//     (:189-191); contributions accumulate with += in output (window) order.
//
// Layout: channels innermost, so every thread works on a vector of V
// consecutive channels (16-byte loads and stores when the channel count
// allows) and a warp covers a contiguous run of channels and pixels.
//
// The backward pass is written in gather form: one thread per input element
// (vector) visits the windows that contain it, in the same output order in
// which Owl's scatter loop adds their contributions, so the float result is
// identical to Owl's `+=` sequence without atomics.  A window in which no
// element beats -inf routes its gradient to flat element 0 in Owl; that case
// is detected (device flag) and element 0 is then rebuilt by an ordered
// fix-up pass.
#include "common.cuh"

#include <algorithm>

namespace owlgpu {
namespace {

struct PG {
  int64_t B, IC, IR, ID, Ch, KC, KR, KD, OC, OR, OD;
  int sc, sr, sd, pc, pr, pd;
};

PG to_pg(const PoolGeom &g) {
  PG p{g.B, g.IC, g.IR, g.ID, g.Ch, g.KC, g.KR, g.KD, g.OC, g.OR, g.OD,
       g.sc, g.sr, g.sd, g.pc, g.pr, g.pd};
  return p;
}

template <typename T, int V>
struct Vec;
template <>
struct Vec<float, 4> { using type = float4; };
template <>
struct Vec<float, 2> { using type = float2; };
template <>
struct Vec<float, 1> { using type = float; };
template <>
struct Vec<double, 2> { using type = double2; };
template <>
struct Vec<double, 1> { using type = double; };

template <typename T, int V>
__device__ __forceinline__ void load_vec(const T *p, T (&v)[V]) {
  using VT = typename Vec<T, V>::type;
  VT t = __ldg(reinterpret_cast<const VT *>(p));
  const T *e = reinterpret_cast<const T *>(&t);
#pragma unroll
  for (int i = 0; i < V; ++i) v[i] = e[i];
}

template <typename T, int V>
__device__ __forceinline__ void store_vec(T *p, const T (&v)[V]) {
  using VT = typename Vec<T, V>::type;
  VT t;
  T *e = reinterpret_cast<T *>(&t);
#pragma unroll
  for (int i = 0; i < V; ++i) e[i] = v[i];
  *reinterpret_cast<VT *>(p) = t;
}

// ---- forward --------------------------------------------------------------

template <typename T, int V, int MODE, bool ARG>
__global__ void __launch_bounds__(256) pool_fwd_kernel(PG g, const T *__restrict__ x,
                                                       T *__restrict__ y,
                                                       int64_t *__restrict__ argmax) {
  const int64_t CV = g.Ch / V;
  const int64_t total = g.B * g.OC * g.OR * g.OD * CV;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t cv = idx % CV, p = idx / CV;
    int64_t od = p % g.OD, t = p / g.OD;
    int64_t orr = t % g.OR; t /= g.OR;
    int64_t oc = t % g.OC, b = t / g.OC;
    const int64_t xbase = b * g.IC * g.IR * g.ID * g.Ch;
    const int cs = (int)(oc * g.sc) - g.pc, rs = (int)(orr * g.sr) - g.pr,
              ds = (int)(od * g.sd) - g.pd;
    T acc[V];
    int64_t mi[V];
#pragma unroll
    for (int i = 0; i < V; ++i) {
      acc[i] = MODE == POOL_MAX ? T(-INFINITY) : T(0);
      mi[i] = -1;
    }
    int cnt = 0;
    const int c0 = max(cs, 0), c1 = min(cs + (int)g.KC, (int)g.IC);
    const int r0 = max(rs, 0), r1 = min(rs + (int)g.KR, (int)g.IR);
    const int d0 = max(ds, 0), d1 = min(ds + (int)g.KD, (int)g.ID);
    for (int a = c0; a < c1; ++a)
      for (int bb = r0; bb < r1; ++bb)
        for (int c = d0; c < d1; ++c) {
          const int64_t off = xbase + (((int64_t)a * g.IR + bb) * g.ID + c) * g.Ch + cv * V;
          T v[V];
          load_vec<T, V>(x + off, v);
#pragma unroll
          for (int i = 0; i < V; ++i) {
            if (MODE == POOL_MAX) {
              if (acc[i] < v[i]) { acc[i] = v[i]; mi[i] = off + i; }
            } else {
              acc[i] += v[i];
            }
          }
          ++cnt;
        }
    T out[V];
#pragma unroll
    for (int i = 0; i < V; ++i) out[i] = MODE == POOL_MAX ? acc[i] : acc[i] / (T)cnt;
    store_vec<T, V>(y + p * g.Ch + cv * V, out);
    if (ARG) {
#pragma unroll
      for (int i = 0; i < V; ++i) argmax[p * g.Ch + cv * V + i] = mi[i];
    }
  }
}

// ---- backward (gather form) ---------------------------------------------

// Range of output positions o whose window [o*s - p, o*s - p + k) contains i.
__device__ __forceinline__ void win_range(int i, int s, int p, int k, int64_t O, int &lo,
                                          int &hi) {
  // o*s <= i + p  and  o*s > i + p - k
  int num = i + p - k + 1;  // o >= ceil(num / s)
  lo = num <= 0 ? 0 : (num + s - 1) / s;
  int top = i + p;  // o <= floor(top / s)
  hi = top < 0 ? -1 : top / s;
  if (hi > (int)O - 1) hi = (int)O - 1;
}

template <typename T, int V, int MODE>
__global__ void __launch_bounds__(256) pool_bwd_kernel(PG g, const T *__restrict__ x,
                                                       const T *__restrict__ dy,
                                                       T *__restrict__ dx,
                                                       int *__restrict__ degenerate) {
  const int64_t CV = g.Ch / V;
  const int64_t total = g.B * g.IC * g.IR * g.ID * CV;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t cv = idx % CV, p = idx / CV;
    int id = (int)(p % g.ID);
    int64_t t = p / g.ID;
    int ir = (int)(t % g.IR); t /= g.IR;
    int ic = (int)(t % g.IC);
    int64_t b = t / g.IC;
    const int64_t xbase = b * g.IC * g.IR * g.ID * g.Ch;
    const int64_t ybase = b * g.OC * g.OR * g.OD * g.Ch;
    const int64_t my_off = xbase + (((int64_t)ic * g.IR + ir) * g.ID + id) * g.Ch + cv * V;
    int oc0, oc1, or0, or1, od0, od1;
    win_range(ic, g.sc, g.pc, (int)g.KC, g.OC, oc0, oc1);
    win_range(ir, g.sr, g.pr, (int)g.KR, g.OR, or0, or1);
    win_range(id, g.sd, g.pd, (int)g.KD, g.OD, od0, od1);
    T acc[V];
#pragma unroll
    for (int i = 0; i < V; ++i) acc[i] = T(0);
    bool degen = false;
    for (int oc = oc0; oc <= oc1; ++oc)
      for (int orr = or0; orr <= or1; ++orr)
        for (int od = od0; od <= od1; ++od) {
          const int cs = oc * g.sc - g.pc, rs = orr * g.sr - g.pr, ds = od * g.sd - g.pd;
          const int c0 = max(cs, 0), c1 = min(cs + (int)g.KC, (int)g.IC);
          const int r0 = max(rs, 0), r1 = min(rs + (int)g.KR, (int)g.IR);
          const int d0 = max(ds, 0), d1 = min(ds + (int)g.KD, (int)g.ID);
          T gv[V];
          load_vec<T, V>(dy + ybase + (((int64_t)oc * g.OR + orr) * g.OD + od) * g.Ch + cv * V,
                         gv);
          if (MODE == POOL_AVG) {
            const int cnt = (c1 - c0) * (r1 - r0) * (d1 - d0);
#pragma unroll
            for (int i = 0; i < V; ++i) acc[i] += gv[i] / (T)cnt;
          } else {
            T best[V];
            int64_t bi[V];
#pragma unroll
            for (int i = 0; i < V; ++i) { best[i] = T(-INFINITY); bi[i] = -1; }
            for (int a = c0; a < c1; ++a)
              for (int bb = r0; bb < r1; ++bb)
                for (int c = d0; c < d1; ++c) {
                  const int64_t off =
                      xbase + (((int64_t)a * g.IR + bb) * g.ID + c) * g.Ch + cv * V;
                  T v[V];
                  load_vec<T, V>(x + off, v);
#pragma unroll
                  for (int i = 0; i < V; ++i)
                    if (best[i] < v[i]) { best[i] = v[i]; bi[i] = off; }
                }
#pragma unroll
            for (int i = 0; i < V; ++i) {
              if (bi[i] < 0) degen = true;
              else if (bi[i] == my_off) acc[i] += gv[i];
            }
          }
        }
    store_vec<T, V>(dx + my_off, acc);
    if (MODE == POOL_MAX && degen) atomicOr(degenerate, 1);
  }
}

// Ordered rebuild of dX[0] for max-pool backward when some window selected
// nothing (Owl routes those windows to flat element 0, owl_ndarray_pool_impl.h
// :167).  One block walks all windows in Owl's loop order (b, oc, or, od,
// ch), 1024 at a time; contributions are summed by one thread in order.
template <typename T>
__global__ void __launch_bounds__(1024) pool_max_fix0_kernel(PG g, const T *__restrict__ x,
                                                             const T *__restrict__ dy,
                                                             T *__restrict__ dx,
                                                             const int *__restrict__ flag) {
  if (*flag == 0) return;
  __shared__ T contrib[1024];
  __shared__ int hit[1024];
  const int64_t total = g.B * g.OC * g.OR * g.OD * g.Ch;
  T sum = T(0);
  for (int64_t base = 0; base < total; base += 1024) {
    int64_t w = base + threadIdx.x;
    hit[threadIdx.x] = 0;
    if (w < total) {
      int64_t ch = w % g.Ch, p = w / g.Ch;
      int64_t od = p % g.OD, t = p / g.OD;
      int64_t orr = t % g.OR; t /= g.OR;
      int64_t oc = t % g.OC, b = t / g.OC;
      const int64_t xbase = b * g.IC * g.IR * g.ID * g.Ch;
      const int cs = (int)(oc * g.sc) - g.pc, rs = (int)(orr * g.sr) - g.pr,
                ds = (int)(od * g.sd) - g.pd;
      T best = T(-INFINITY);
      int64_t bi = 0;
      for (int a = cs; a < cs + (int)g.KC; ++a)
        for (int bb = rs; bb < rs + (int)g.KR; ++bb)
          for (int c = ds; c < ds + (int)g.KD; ++c)
            if (a >= 0 && a < g.IC && bb >= 0 && bb < g.IR && c >= 0 && c < g.ID) {
              int64_t off = xbase + (((int64_t)a * g.IR + bb) * g.ID + c) * g.Ch + ch;
              T v = x[off];
              if (best < v) { best = v; bi = off; }
            }
      if (bi == 0) { hit[threadIdx.x] = 1; contrib[threadIdx.x] = dy[w]; }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t rem = total - base;
      int n = rem < 1024 ? (int)rem : 1024;
      for (int i = 0; i < n; ++i)
        if (hit[i]) sum += contrib[i];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) dx[0] = sum;
}

int grid_for(int64_t work) {
  int64_t blocks = ceil_div(work, 256);
  return (int)std::max<int64_t>(1, std::min<int64_t>(blocks, 152 * 16));
}

template <typename T>
int vec_width(int64_t ch, const void *a, const void *b, const void *c) {
  auto al = [](const void *p, int bytes) { return ((uintptr_t)p % bytes) == 0; };
  if (sizeof(T) == 4 && ch % 4 == 0 && al(a, 16) && al(b, 16) && al(c, 16)) return 4;
  if (ch % 2 == 0 && al(a, 2 * sizeof(T)) && al(b, 2 * sizeof(T)) && al(c, 2 * sizeof(T)))
    return 2;
  return 1;
}

template <typename T, int V>
int fwd_launch(const PG &g, PoolMode mode, const T *x, T *y, int64_t *arg, cudaStream_t s) {
  int grid = grid_for(g.B * g.OC * g.OR * g.OD * (g.Ch / V));
  if (mode == POOL_AVG)
    pool_fwd_kernel<T, V, POOL_AVG, false><<<grid, 256, 0, s>>>(g, x, y, nullptr);
  else if (arg)
    pool_fwd_kernel<T, V, POOL_MAX, true><<<grid, 256, 0, s>>>(g, x, y, arg);
  else
    pool_fwd_kernel<T, V, POOL_MAX, false><<<grid, 256, 0, s>>>(g, x, y, nullptr);
  OWL_CHECK_LAUNCH("pool_fwd_kernel");
  return kOk;
}

template <typename T>
int fwd_t(const PoolGeom &pg, PoolMode mode, const T *x, T *y, int64_t *arg, cudaStream_t s) {
  PG g = to_pg(pg);
  if (pg.y_elems() == 0) return kOk;
  int v = vec_width<T>(g.Ch, x, y, y);
  if (v == 4) return fwd_launch<T, (sizeof(T) == 4 ? 4 : 1)>(g, mode, x, y, arg, s);
  if (v == 2) return fwd_launch<T, 2>(g, mode, x, y, arg, s);
  return fwd_launch<T, 1>(g, mode, x, y, arg, s);
}

template <typename T, int V>
int bwd_launch(const PG &g, PoolMode mode, const T *x, const T *dy, T *dx, int *flag,
               cudaStream_t s) {
  int grid = grid_for(g.B * g.IC * g.IR * g.ID * (g.Ch / V));
  if (mode == POOL_AVG)
    pool_bwd_kernel<T, V, POOL_AVG><<<grid, 256, 0, s>>>(g, x, dy, dx, flag);
  else
    pool_bwd_kernel<T, V, POOL_MAX><<<grid, 256, 0, s>>>(g, x, dy, dx, flag);
  OWL_CHECK_LAUNCH("pool_bwd_kernel");
  return kOk;
}

// True when some window has no in-range element (possible only with
// inconsistent explicit pads); Owl then routes its max gradient to element 0.
bool has_empty_window(const PG &g) {
  auto dim_empty = [](int64_t I, int64_t K, int64_t O, int s, int p) {
    if (O <= 0) return false;
    int64_t first_end = -p + K;           // window 0 covers [-p, K - p)
    int64_t last_start = (O - 1) * s - p;  // last window start
    return first_end <= 0 || last_start >= I;
  };
  return dim_empty(g.IC, g.KC, g.OC, g.sc, g.pc) || dim_empty(g.IR, g.KR, g.OR, g.sr, g.pr) ||
         dim_empty(g.ID, g.KD, g.OD, g.sd, g.pd);
}

template <typename T>
int bwd_t(const PoolGeom &pg, PoolMode mode, const T *x, const T *dy, T *dx, cudaStream_t s) {
  PG g = to_pg(pg);
  if (pg.x_elems() == 0) return kOk;
  if (pg.y_elems() == 0) {
    OWL_CUDA(cudaMemsetAsync(dx, 0, sizeof(T) * pg.x_elems(), s));
    return kOk;
  }
  int *flag = nullptr;
  if (mode == POOL_MAX) {
    int rc = scratch_alloc((void **)&flag, sizeof(int), s);
    if (rc) return rc;
    int init = has_empty_window(g) ? 1 : 0;
    cudaError_t e = cudaMemsetAsync(flag, init, sizeof(int), s);
    if (e != cudaSuccess) { scratch_free(flag, s); return cuda_fail(e, "cudaMemsetAsync"); }
  }
  int v = vec_width<T>(g.Ch, x ? (const void *)x : (const void *)dy, dy, dx);
  int rc;
  if (v == 4) rc = bwd_launch<T, (sizeof(T) == 4 ? 4 : 1)>(g, mode, x, dy, dx, flag, s);
  else if (v == 2) rc = bwd_launch<T, 2>(g, mode, x, dy, dx, flag, s);
  else rc = bwd_launch<T, 1>(g, mode, x, dy, dx, flag, s);
  if (rc == kOk && mode == POOL_MAX) {
    pool_max_fix0_kernel<T><<<1, 1024, 0, s>>>(g, x, dy, dx, flag);
    cudaError_t e = cudaGetLastError();
    note_launch();
    if (e != cudaSuccess) rc = cuda_fail(e, "pool_max_fix0_kernel");
  }
  if (flag) scratch_free(flag, s);
  return rc;
}

}  // namespace

int pool_fwd(Dtype dt, PoolMode mode, const PoolGeom &g, const void *x, void *y,
             int64_t *argmax, cudaStream_t s) {
  return dt == F32 ? fwd_t<float>(g, mode, (const float *)x, (float *)y, argmax, s)
                   : fwd_t<double>(g, mode, (const double *)x, (double *)y, argmax, s);
}

int pool_bwd(Dtype dt, PoolMode mode, const PoolGeom &g, const void *x, const void *dy,
             void *dx, cudaStream_t s) {
  return dt == F32
             ? bwd_t<float>(g, mode, (const float *)x, (const float *)dy, (float *)dx, s)
             : bwd_t<double>(g, mode, (const double *)x, (const double *)dy, (double *)dx, s);
}

}  // namespace owlgpu
