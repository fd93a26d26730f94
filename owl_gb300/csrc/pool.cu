// pool.cu -- max / average pooling, forward and backward, 2-D and 3-D,
// float32, float64, complex32 and complex64, with Owl's exact semantics
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
// Every thread walks its window in chunks of eight taps, issuing the eight
// vector loads before reducing them in scan order, so each thread keeps
// several loads in flight (a pooling kernel is bound by HBM latency x
// parallelism, not by arithmetic).  The reduction axis is the window, not
// the contiguous channel axis, so no cross-lane shuffle is needed: a warp's
// loads of one tap are one contiguous run of channels.
//
// Backward has two forms, both equal to Owl's zero-initialised `+=` scatter
// bit for bit and without atomics:
//   * windows that do not overlap (stride >= kernel in every dimension):
//     one thread per window recomputes its winner and writes each element
//     of the window's cell once (read X and dY once, write dX once);
//   * overlapping windows: one thread per input element visits the windows
//     that contain it in output order, the order of Owl's `+=` sequence.
// A max window in which no element beats -inf routes its gradient to flat
// element 0 in Owl; such windows are detected on the device and element 0
// is then rebuilt by an ordered fix-up pass.
#include "common.cuh"

#include <algorithm>
#include <atomic>
#include <type_traits>

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

// Unsigned 32-bit division by a divisor fixed for the whole launch, by one
// multiply-high, an add and a shift (Granlund & Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994, round-up variant):
// with l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1,
// n / d = (umulhi(m, n) + n) >> l for every n < 2^31.
struct FastDiv {
  uint32_t d, m, l;
};

FastDiv make_fastdiv(uint32_t d) {
  uint32_t l = 0;
  while ((1ull << l) < d) ++l;
  const uint64_t m = (((1ull << l) - d) << 32) / d + 1;
  return FastDiv{d, (uint32_t)m, l};
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
  return (__umulhi(f.m, n) + n) >> f.l;
}

// Output index -> (b, oc, or, od, channel vector) with channel vectors
// innermost; valid while the output has fewer than 2^31 vectors.
struct OutDecode {
  FastDiv cv, od, orr, oc;
};

OutDecode make_out_decode(const PG &g, int64_t cv) {
  return OutDecode{make_fastdiv((uint32_t)cv), make_fastdiv((uint32_t)g.OD),
                   make_fastdiv((uint32_t)g.OR), make_fastdiv((uint32_t)g.OC)};
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
template <>
struct Vec<c32, 2> { using type = float4; };
template <>
struct Vec<c32, 1> { using type = float2; };
template <>
struct Vec<c64, 1> { using type = double2; };

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

// ---- window walking ------------------------------------------------------

// In-range part of one window: [c0,c1) x [r0,r1) x [d0,d1); n taps.
struct Box {
  int c0, c1, r0, r1, d0, d1, nr, nd, n;
};

__device__ __forceinline__ Box window_box(const PG &g, int oc, int orr, int od) {
  Box w;
  const int cs = oc * g.sc - g.pc, rs = orr * g.sr - g.pr, ds = od * g.sd - g.pd;
  w.c0 = max(cs, 0); w.c1 = min(cs + (int)g.KC, (int)g.IC);
  w.r0 = max(rs, 0); w.r1 = min(rs + (int)g.KR, (int)g.IR);
  w.d0 = max(ds, 0); w.d1 = min(ds + (int)g.KD, (int)g.ID);
  const int nc = max(w.c1 - w.c0, 0);
  w.nr = max(w.r1 - w.r0, 0);
  w.nd = max(w.d1 - w.d0, 0);
  w.n = nc * w.nr * w.nd;
  return w;
}

// Walks a window's taps in Owl's scan order (cols, rows, dpts) U at a time:
// all U loads of a chunk are issued before any is used, so a thread keeps U
// vector loads in flight instead of one.
struct Cursor {
  int a, b, c;
};

template <typename T, int V, int U>
__device__ __forceinline__ void load_chunk(const T *__restrict__ x, int64_t base, const PG &g,
                                           const Box &w, Cursor &cur, int left,
                                           T (&v)[U][V]) {
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if (u < left) {
      load_vec<T, V>(x + base + (((int64_t)cur.a * g.IR + cur.b) * g.ID + cur.c) * g.Ch, v[u]);
      if (++cur.c == w.d1) {
        cur.c = w.d0;
        if (++cur.b == w.r1) { cur.b = w.r0; ++cur.a; }
      }
    }
  }
}

// Max over the window with Owl's strict `<` (first maximum wins, NaN never
// selected); bt = tap index of the winner in scan order, -1 if none.
template <typename T, int V, int U>
__device__ __forceinline__ void window_max(const T *__restrict__ x, int64_t base, const PG &g,
                                           const Box &w, T (&best)[V], int (&bt)[V]) {
#pragma unroll
  for (int i = 0; i < V; ++i) { best[i] = T(-INFINITY); bt[i] = -1; }
  Cursor cur{w.c0, w.r0, w.d0};
  for (int t0 = 0; t0 < w.n; t0 += U) {
    T v[U][V];
    load_chunk<T, V, U>(x, base, g, w, cur, w.n - t0, v);
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (u < w.n - t0) {
#pragma unroll
        for (int i = 0; i < V; ++i)
          if (best[i] < v[u][i]) { best[i] = v[u][i]; bt[i] = t0 + u; }
      }
  }
}

// Sum over the window in scan order, in the element type.
template <typename T, int V, int U>
__device__ __forceinline__ void window_sum(const T *__restrict__ x, int64_t base, const PG &g,
                                           const Box &w, T (&acc)[V]) {
#pragma unroll
  for (int i = 0; i < V; ++i) acc[i] = T(0);
  Cursor cur{w.c0, w.r0, w.d0};
  for (int t0 = 0; t0 < w.n; t0 += U) {
    T v[U][V];
    load_chunk<T, V, U>(x, base, g, w, cur, w.n - t0, v);
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (u < w.n - t0) {
#pragma unroll
        for (int i = 0; i < V; ++i) acc[i] += v[u][i];
      }
  }
}

// Flat input offset (without the channel) of tap t of window w.
__device__ __forceinline__ int64_t tap_offset(const PG &g, int64_t xbase, const Box &w, int t) {
  const int per_c = w.nr * w.nd;
  const int a = w.c0 + t / per_c, rem = t % per_c;
  const int b = w.r0 + rem / w.nd, c = w.d0 + rem % w.nd;
  return xbase + (((int64_t)a * g.IR + b) * g.ID + c) * g.Ch;
}

constexpr int kChunk = 8;

// ---- forward --------------------------------------------------------------

template <typename T, int V, int MODE, bool ARG>
__global__ void __launch_bounds__(256) pool_fwd_kernel(PG g, const T *__restrict__ x,
                                                       T *__restrict__ y,
                                                       int64_t *__restrict__ argmax) {
  const int64_t CV = g.Ch / V;
  const int64_t total = g.B * g.OC * g.OR * g.OD * CV;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cv = idx % CV, p = idx / CV;
    const int od = (int)(p % g.OD);
    int64_t t = p / g.OD;
    const int orr = (int)(t % g.OR); t /= g.OR;
    const int oc = (int)(t % g.OC);
    const int64_t b = t / g.OC;
    const int64_t xbase = b * g.IC * g.IR * g.ID * g.Ch;
    const Box w = window_box(g, oc, orr, od);
    T out[V];
    if (MODE == POOL_MAX) {
      int bt[V];
      window_max<T, V, kChunk>(x, xbase + cv * V, g, w, out, bt);
      if (ARG) {
#pragma unroll
        for (int i = 0; i < V; ++i)
          argmax[p * g.Ch + cv * V + i] =
              bt[i] < 0 ? -1 : tap_offset(g, xbase, w, bt[i]) + cv * V + i;
      }
    } else {
      window_sum<T, V, kChunk>(x, xbase + cv * V, g, w, out);
#pragma unroll
      for (int i = 0; i < V; ++i) out[i] = div_count(out[i], w.n);
    }
    store_vec<T, V>(y + p * g.Ch + cv * V, out);
  }
}

// ---- degenerate max windows ------------------------------------------------

// A max window in which no element beats -inf (all -inf/NaN, or no in-range
// element) routes its gradient to flat element 0 in Owl.  Kernels that meet
// one raise this device-wide mark to their call's ticket with atomicMax; the
// fix-up kernel of a call runs when the mark is at or above its own ticket.
// Tickets grow monotonically, so a call never misses its own mark; a later
// call's mark can only make an earlier call redo the (always exact) ordered
// rebuild of dX[0].  No per-call memory is needed.
__device__ unsigned long long g_degenerate_mark = 0;
std::atomic<unsigned long long> g_ticket{0};

__device__ __forceinline__ void raise_mark(unsigned long long ticket) {
  atomicMax(&g_degenerate_mark, ticket);
}

// ---- backward, non-overlapping windows (scatter form) ---------------------

// Per-dimension part of the input owned by output position o when s >= k:
// [o*s - p, (o+1)*s - p) clipped to [0, I), the last position taking the
// tail up to I.  These ranges partition [0, I) and each contains its window.
__device__ __forceinline__ void cell_range(int o, int s, int p, int64_t O, int64_t I, int &lo,
                                           int &hi) {
  lo = min(max(o * s - p, 0), (int)I);
  hi = o == (int)O - 1 ? (int)I : min(max((o + 1) * s - p, 0), (int)I);
}

// One thread per (window, channel vector): recompute the window's maximum
// (or its count), then write every element of the window's cell exactly
// once: 0 + dY at the winner, 0 + dY/count for average, 0 elsewhere.  With
// s >= k every input element lies in at most one window, so this equals
// Owl's zero-initialised `+=` scatter bit for bit.
template <typename T, int V, int MODE>
__global__ void __launch_bounds__(256) pool_bwd_cell_kernel(PG g, const T *__restrict__ x,
                                                            const T *__restrict__ dy,
                                                            T *__restrict__ dx,
                                                            unsigned long long ticket) {
  asm volatile("griddepcontrol.launch_dependents;");
  const int64_t CV = g.Ch / V;
  const int64_t total = g.B * g.OC * g.OR * g.OD * CV;
  bool degen = false;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cv = idx % CV, p = idx / CV;
    const int od = (int)(p % g.OD);
    int64_t t = p / g.OD;
    const int orr = (int)(t % g.OR); t /= g.OR;
    const int oc = (int)(t % g.OC);
    const int64_t b = t / g.OC;
    const int64_t xbase = b * g.IC * g.IR * g.ID * g.Ch;
    const Box w = window_box(g, oc, orr, od);
    T gv[V];
    load_vec<T, V>(dy + p * g.Ch + cv * V, gv);
    int bt[V];
    if (MODE == POOL_MAX) {
      T best[V];
      window_max<T, V, kChunk>(x, xbase + cv * V, g, w, best, bt);
#pragma unroll
      for (int i = 0; i < V; ++i) degen |= bt[i] < 0;
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) gv[i] = div_count(gv[i], w.n);
    }
    int alo, ahi, blo, bhi, clo, chi;
    cell_range(oc, g.sc, g.pc, g.OC, g.IC, alo, ahi);
    cell_range(orr, g.sr, g.pr, g.OR, g.IR, blo, bhi);
    cell_range(od, g.sd, g.pd, g.OD, g.ID, clo, chi);
    for (int a = alo; a < ahi; ++a)
      for (int bb = blo; bb < bhi; ++bb)
        for (int c = clo; c < chi; ++c) {
          const bool in = a >= w.c0 && a < w.c1 && bb >= w.r0 && bb < w.r1 && c >= w.d0 &&
                          c < w.d1;
          const int tap = ((a - w.c0) * w.nr + (bb - w.r0)) * w.nd + (c - w.d0);
          T o[V];
#pragma unroll
          for (int i = 0; i < V; ++i) {
            if (MODE == POOL_MAX) o[i] = in && tap == bt[i] ? T(0) + gv[i] : T(0);
            else o[i] = in ? T(0) + gv[i] : T(0);
          }
          store_vec<T, V>(dx + xbase + (((int64_t)a * g.IR + bb) * g.ID + c) * g.Ch + cv * V, o);
        }
  }
  if (MODE == POOL_MAX && degen) raise_mark(ticket);
}

// ---- fixed-window fast paths ----------------------------------------------

// Windows of compile-time size KC x KR x KD that lie wholly inside the input
// (no padding, (O-1)*s + k <= I in every dimension): the taps are constant
// strides apart, every tap of a window is loaded before the reduction, and
// nothing is clipped.  Same scan order and comparisons as the general path.
template <typename T, int V, int KC, int KR, int KD, int MODE, bool ARG>
__global__ void __launch_bounds__(256) pool_fwd_fixed_kernel(PG g, OutDecode dec,
                                                             const T *__restrict__ x,
                                                             T *__restrict__ y,
                                                             int64_t *__restrict__ argmax) {
  constexpr int N = KC * KR * KD;
  const uint32_t total = (uint32_t)(g.B * g.OC * g.OR * g.OD * (g.Ch / V));
  const int64_t sd = g.Ch, sr = g.ID * g.Ch, sc = g.IR * g.ID * g.Ch;
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += gridDim.x * blockDim.x) {
    const uint32_t p32 = fdiv(idx, dec.cv);
    const int64_t cv = idx - p32 * dec.cv.d, p = p32;
    const uint32_t t1 = fdiv(p32, dec.od);
    const int od = (int)(p32 - t1 * dec.od.d);
    const uint32_t t2 = fdiv(t1, dec.orr);
    const int orr = (int)(t1 - t2 * dec.orr.d);
    const uint32_t t3 = fdiv(t2, dec.oc);
    const int oc = (int)(t2 - t3 * dec.oc.d);
    const int64_t b = t3;
    const int64_t base = b * g.IC * sc + (int64_t)oc * g.sc * sc + (int64_t)orr * g.sr * sr +
                         (int64_t)od * g.sd * sd + cv * V;
    T v[N][V];
#pragma unroll
    for (int a = 0; a < KC; ++a)
#pragma unroll
      for (int bb = 0; bb < KR; ++bb)
#pragma unroll
        for (int c = 0; c < KD; ++c)
          load_vec<T, V>(x + base + a * sc + bb * sr + c * sd, v[(a * KR + bb) * KD + c]);
    T out[V];
    if (MODE == POOL_MAX) {
      int bt[V];
#pragma unroll
      for (int i = 0; i < V; ++i) { out[i] = T(-INFINITY); bt[i] = -1; }
#pragma unroll
      for (int u = 0; u < N; ++u)
#pragma unroll
        for (int i = 0; i < V; ++i)
          if (out[i] < v[u][i]) { out[i] = v[u][i]; bt[i] = u; }
      if (ARG) {
#pragma unroll
        for (int i = 0; i < V; ++i) {
          const int a = bt[i] / (KR * KD), bb = bt[i] / KD % KR, c = bt[i] % KD;
          argmax[p * g.Ch + cv * V + i] = bt[i] < 0 ? -1 : base + a * sc + bb * sr + c * sd + i;
        }
      }
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) out[i] = T(0);
#pragma unroll
      for (int u = 0; u < N; ++u)
#pragma unroll
        for (int i = 0; i < V; ++i) out[i] += v[u][i];
#pragma unroll
      for (int i = 0; i < V; ++i) out[i] = div_count(out[i], N);
    }
    store_vec<T, V>(y + p * g.Ch + cv * V, out);
  }
}

// Backward for windows that tile the input exactly (stride = kernel, no
// padding, O*s = I): each window is its own cell.
template <typename T, int V, int KC, int KR, int KD, int MODE>
__global__ void __launch_bounds__(256) pool_bwd_tile_kernel(PG g, OutDecode dec,
                                                            const T *__restrict__ x,
                                                            const T *__restrict__ dy,
                                                            T *__restrict__ dx,
                                                            unsigned long long ticket) {
  asm volatile("griddepcontrol.launch_dependents;");
  constexpr int N = KC * KR * KD;
  const uint32_t total = (uint32_t)(g.B * g.OC * g.OR * g.OD * (g.Ch / V));
  const int64_t sd = g.Ch, sr = g.ID * g.Ch, sc = g.IR * g.ID * g.Ch;
  bool degen = false;
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += gridDim.x * blockDim.x) {
    const uint32_t p32 = fdiv(idx, dec.cv);
    const int64_t cv = idx - p32 * dec.cv.d, p = p32;
    const uint32_t t1 = fdiv(p32, dec.od);
    const int od = (int)(p32 - t1 * dec.od.d);
    const uint32_t t2 = fdiv(t1, dec.orr);
    const int orr = (int)(t1 - t2 * dec.orr.d);
    const uint32_t t3 = fdiv(t2, dec.oc);
    const int oc = (int)(t2 - t3 * dec.oc.d);
    const int64_t b = t3;
    const int64_t base = b * g.IC * sc + (int64_t)oc * KC * sc + (int64_t)orr * KR * sr +
                         (int64_t)od * KD * sd + cv * V;
    T gv[V];
    load_vec<T, V>(dy + p * g.Ch + cv * V, gv);
    int bt[V];
    if (MODE == POOL_MAX) {
      T v[N][V];
#pragma unroll
      for (int a = 0; a < KC; ++a)
#pragma unroll
        for (int bb = 0; bb < KR; ++bb)
#pragma unroll
          for (int c = 0; c < KD; ++c)
            load_vec<T, V>(x + base + a * sc + bb * sr + c * sd, v[(a * KR + bb) * KD + c]);
      T best[V];
#pragma unroll
      for (int i = 0; i < V; ++i) { best[i] = T(-INFINITY); bt[i] = -1; }
#pragma unroll
      for (int u = 0; u < N; ++u)
#pragma unroll
        for (int i = 0; i < V; ++i)
          if (best[i] < v[u][i]) { best[i] = v[u][i]; bt[i] = u; }
#pragma unroll
      for (int i = 0; i < V; ++i) degen |= bt[i] < 0;
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) gv[i] = div_count(gv[i], N);
    }
#pragma unroll
    for (int a = 0; a < KC; ++a)
#pragma unroll
      for (int bb = 0; bb < KR; ++bb)
#pragma unroll
        for (int c = 0; c < KD; ++c) {
          const int u = (a * KR + bb) * KD + c;
          T o[V];
#pragma unroll
          for (int i = 0; i < V; ++i) {
            if (MODE == POOL_MAX) o[i] = bt[i] == u ? T(0) + gv[i] : T(0);
            else o[i] = T(0) + gv[i];
          }
          store_vec<T, V>(dx + base + a * sc + bb * sr + c * sd, o);
        }
  }
  if (MODE == POOL_MAX && degen) raise_mark(ticket);
}

// ---- backward, overlapping windows (gather form) ---------------------------

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

// One thread per input element (vector): visit the windows that contain it
// in output order, the order in which Owl's scatter loop adds their
// contributions, so the float sum is Owl's `+=` sequence without atomics.
template <typename T, int V, int MODE>
__global__ void __launch_bounds__(256) pool_bwd_gather_kernel(PG g, const T *__restrict__ x,
                                                              const T *__restrict__ dy,
                                                              T *__restrict__ dx,
                                                              unsigned long long ticket) {
  asm volatile("griddepcontrol.launch_dependents;");
  const int64_t CV = g.Ch / V;
  const int64_t total = g.B * g.IC * g.IR * g.ID * CV;
  bool degen = false;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cv = idx % CV, p = idx / CV;
    const int id = (int)(p % g.ID);
    int64_t t = p / g.ID;
    const int ir = (int)(t % g.IR); t /= g.IR;
    const int ic = (int)(t % g.IC);
    const int64_t b = t / g.IC;
    const int64_t xbase = b * g.IC * g.IR * g.ID * g.Ch;
    const int64_t ybase = b * g.OC * g.OR * g.OD * g.Ch;
    int oc0, oc1, or0, or1, od0, od1;
    win_range(ic, g.sc, g.pc, (int)g.KC, g.OC, oc0, oc1);
    win_range(ir, g.sr, g.pr, (int)g.KR, g.OR, or0, or1);
    win_range(id, g.sd, g.pd, (int)g.KD, g.OD, od0, od1);
    T acc[V];
#pragma unroll
    for (int i = 0; i < V; ++i) acc[i] = T(0);
    for (int oc = oc0; oc <= oc1; ++oc)
      for (int orr = or0; orr <= or1; ++orr)
        for (int od = od0; od <= od1; ++od) {
          const Box w = window_box(g, oc, orr, od);
          T gv[V];
          load_vec<T, V>(dy + ybase + (((int64_t)oc * g.OR + orr) * g.OD + od) * g.Ch + cv * V,
                         gv);
          if (MODE == POOL_AVG) {
#pragma unroll
            for (int i = 0; i < V; ++i) acc[i] += div_count(gv[i], w.n);
          } else {
            T best[V];
            int bt[V];
            window_max<T, V, kChunk>(x, xbase + cv * V, g, w, best, bt);
            const int mine = ((ic - w.c0) * w.nr + (ir - w.r0)) * w.nd + (id - w.d0);
#pragma unroll
            for (int i = 0; i < V; ++i) {
              if (bt[i] < 0) degen = true;
              else if (bt[i] == mine) acc[i] += gv[i];
            }
          }
        }
    store_vec<T, V>(dx + xbase + (((int64_t)ic * g.IR + ir) * g.ID + id) * g.Ch + cv * V, acc);
  }
  if (MODE == POOL_MAX && degen) raise_mark(ticket);
}

// Ordered rebuild of dX[0] for max-pool backward when some window selected
// nothing (Owl routes those windows to flat element 0, owl_ndarray_pool_impl.h
// :167).  One block walks all windows in Owl's loop order (b, oc, or, od,
// ch), 1024 at a time; contributions are summed by one thread in order.
// Runs only when this call's ticket is marked (or `force`: some window has
// no in-range element, which the gather form never visits).
template <typename T>
__global__ void __launch_bounds__(1024) pool_max_fix0_kernel(PG g, const T *__restrict__ x,
                                                             const T *__restrict__ dy,
                                                             T *__restrict__ dx,
                                                             unsigned long long ticket,
                                                             int force) {
  // Launched as a programmatic dependent of the backward kernel: wait for
  // that grid to finish and its writes to become visible.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (!force && *(volatile unsigned long long *)&g_degenerate_mark < ticket) return;
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

// Elements per 16-byte vector: 4 floats, 2 doubles or complex32, 1 complex64.
template <typename T>
constexpr int kWide = (int)(16 / sizeof(T));

template <typename T>
int vec_width(int64_t ch, const void *a, const void *b, const void *c) {
  auto al = [](const void *p, int bytes) { return ((uintptr_t)p % bytes) == 0; };
  if (kWide<T> >= 4 && ch % 4 == 0 && al(a, 16) && al(b, 16) && al(c, 16)) return 4;
  if (kWide<T> >= 2 && ch % 2 == 0 && al(a, 2 * sizeof(T)) && al(b, 2 * sizeof(T)) &&
      al(c, 2 * sizeof(T)))
    return 2;
  return 1;
}

// Every window lies wholly inside the input: no padding and the last
// window ends at or before the input's end, in every dimension.
bool interior(const PG &g) {
  auto ok = [](int64_t I, int64_t K, int64_t O, int s, int p) {
    return p == 0 && (O - 1) * s + K <= I;
  };
  return ok(g.IC, g.KC, g.OC, g.sc, g.pc) && ok(g.IR, g.KR, g.OR, g.sr, g.pr) &&
         ok(g.ID, g.KD, g.OD, g.sd, g.pd);
}

// Windows tile the input exactly: stride = kernel, no padding, O*s = I.
bool exact_tiling(const PG &g) {
  auto ok = [](int64_t I, int64_t K, int64_t O, int s, int p) {
    return p == 0 && s == K && O * s == I;
  };
  return ok(g.IC, g.KC, g.OC, g.sc, g.pc) && ok(g.IR, g.KR, g.OR, g.sr, g.pr) &&
         ok(g.ID, g.KD, g.OD, g.sd, g.pd);
}

bool window_is(const PG &g, int kc, int kr, int kd) {
  return g.KC == kc && g.KR == kr && g.KD == kd;
}

template <typename T, int V, int KC, int KR, int KD>
void fwd_fixed(const PG &g, PoolMode mode, const T *x, T *y, int64_t *arg, int grid,
               cudaStream_t s) {
  const OutDecode d = make_out_decode(g, g.Ch / V);
  if (mode == POOL_AVG)
    pool_fwd_fixed_kernel<T, V, KC, KR, KD, POOL_AVG, false>
        <<<grid, 256, 0, s>>>(g, d, x, y, nullptr);
  else if (arg)
    pool_fwd_fixed_kernel<T, V, KC, KR, KD, POOL_MAX, true><<<grid, 256, 0, s>>>(g, d, x, y, arg);
  else
    pool_fwd_fixed_kernel<T, V, KC, KR, KD, POOL_MAX, false>
        <<<grid, 256, 0, s>>>(g, d, x, y, nullptr);
}

// The fixed-window kernels index outputs with 32-bit fast division.
bool small_output(const PG &g, int V) {
  return g.B * g.OC * g.OR * g.OD * (g.Ch / V) < (int64_t(1) << 31);
}

// Fixed-window kernels exist for the widest vector of each type (16 bytes)
// and the common window shapes 2x2, 3x3 and 2x2x2.

template <typename T, int V>
int fwd_launch(const PG &g, PoolMode mode, const T *x, T *y, int64_t *arg, cudaStream_t s) {
  int grid = grid_for(g.B * g.OC * g.OR * g.OD * (g.Ch / V));
  const bool fixed = V == kWide<T> && interior(g) && small_output(g, V);
  if (fixed && window_is(g, 2, 2, 1)) {
    fwd_fixed<T, V, 2, 2, 1>(g, mode, x, y, arg, grid, s);
  } else if (fixed && window_is(g, 3, 3, 1)) {
    fwd_fixed<T, V, 3, 3, 1>(g, mode, x, y, arg, grid, s);
  } else if (fixed && window_is(g, 2, 2, 2)) {
    fwd_fixed<T, V, 2, 2, 2>(g, mode, x, y, arg, grid, s);
  } else if (mode == POOL_AVG) {
    pool_fwd_kernel<T, V, POOL_AVG, false><<<grid, 256, 0, s>>>(g, x, y, nullptr);
  } else if (arg) {
    pool_fwd_kernel<T, V, POOL_MAX, true><<<grid, 256, 0, s>>>(g, x, y, arg);
  } else {
    pool_fwd_kernel<T, V, POOL_MAX, false><<<grid, 256, 0, s>>>(g, x, y, nullptr);
  }
  OWL_CHECK_LAUNCH("pool_fwd_kernel");
  return kOk;
}

template <typename T>
int fwd_t(const PoolGeom &pg, PoolMode mode, const T *x, T *y, int64_t *arg, cudaStream_t s) {
  PG g = to_pg(pg);
  if (pg.y_elems() == 0) return kOk;
  int v = vec_width<T>(g.Ch, x, y, y);
  if (v == 4) return fwd_launch<T, kWide<T>>(g, mode, x, y, arg, s);
  if constexpr (kWide<T> >= 2) {
    if (v == 2) return fwd_launch<T, 2>(g, mode, x, y, arg, s);
  }
  return fwd_launch<T, 1>(g, mode, x, y, arg, s);
}

// Windows overlap in no dimension: every input element lies in at most one.
bool non_overlapping(const PG &g) { return g.sc >= g.KC && g.sr >= g.KR && g.sd >= g.KD; }

template <typename T, int V, int KC, int KR, int KD>
void bwd_tile(const PG &g, PoolMode mode, const T *x, const T *dy, T *dx,
              unsigned long long ticket, int grid, cudaStream_t s) {
  const OutDecode d = make_out_decode(g, g.Ch / V);
  if (mode == POOL_AVG)
    pool_bwd_tile_kernel<T, V, KC, KR, KD, POOL_AVG>
        <<<grid, 256, 0, s>>>(g, d, x, dy, dx, ticket);
  else
    pool_bwd_tile_kernel<T, V, KC, KR, KD, POOL_MAX>
        <<<grid, 256, 0, s>>>(g, d, x, dy, dx, ticket);
}

template <typename T, int V>
int bwd_launch(const PG &g, PoolMode mode, const T *x, const T *dy, T *dx,
               unsigned long long ticket, cudaStream_t s) {
  if (non_overlapping(g)) {
    int grid = grid_for(g.B * g.OC * g.OR * g.OD * (g.Ch / V));
    const bool tile = V == kWide<T> && exact_tiling(g) && small_output(g, V);
    if (tile && window_is(g, 2, 2, 1))
      bwd_tile<T, V, 2, 2, 1>(g, mode, x, dy, dx, ticket, grid, s);
    else if (tile && window_is(g, 2, 2, 2))
      bwd_tile<T, V, 2, 2, 2>(g, mode, x, dy, dx, ticket, grid, s);
    else if (mode == POOL_AVG)
      pool_bwd_cell_kernel<T, V, POOL_AVG><<<grid, 256, 0, s>>>(g, x, dy, dx, ticket);
    else
      pool_bwd_cell_kernel<T, V, POOL_MAX><<<grid, 256, 0, s>>>(g, x, dy, dx, ticket);
    OWL_CHECK_LAUNCH("pool_bwd_cell_kernel");
  } else {
    int grid = grid_for(g.B * g.IC * g.IR * g.ID * (g.Ch / V));
    if (mode == POOL_AVG)
      pool_bwd_gather_kernel<T, V, POOL_AVG><<<grid, 256, 0, s>>>(g, x, dy, dx, ticket);
    else
      pool_bwd_gather_kernel<T, V, POOL_MAX><<<grid, 256, 0, s>>>(g, x, dy, dx, ticket);
    OWL_CHECK_LAUNCH("pool_bwd_gather_kernel");
  }
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
  const unsigned long long ticket = ++g_ticket;
  int v = vec_width<T>(g.Ch, x ? (const void *)x : (const void *)dy, dy, dx);
  int rc;
  if (v == 4) rc = bwd_launch<T, kWide<T>>(g, mode, x, dy, dx, ticket, s);
  else if (v == 2) rc = bwd_launch<T, kWide<T> >= 2 ? 2 : 1>(g, mode, x, dy, dx, ticket, s);
  else rc = bwd_launch<T, 1>(g, mode, x, dy, dx, ticket, s);
  if (rc == kOk && mode == POOL_MAX) {
    const int force = has_empty_window(g) ? 1 : 0;
    // Programmatic dependent launch: the fix-up grid is scheduled while the
    // backward grid drains and waits on it with griddepcontrol.wait.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(1024);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, pool_max_fix0_kernel<T>, g, x, dy, dx, ticket, force);
    note_launch();
    if (e != cudaSuccess) rc = cuda_fail(e, "pool_max_fix0_kernel");
  }
  return rc;
}

}  // namespace

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

int pool_fwd(Dtype dt, PoolMode mode, const PoolGeom &g, const void *x, void *y,
             int64_t *argmax, cudaStream_t s) {
  return by_dtype(dt, [&](auto *tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    return fwd_t<T>(g, mode, (const T *)x, (T *)y, argmax, s);
  });
}

int pool_bwd(Dtype dt, PoolMode mode, const PoolGeom &g, const void *x, const void *dy,
             void *dx, cudaStream_t s) {
  return by_dtype(dt, [&](auto *tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    return bwd_t<T>(g, mode, (const T *)x, (const T *)dy, (T *)dx, s);
  });
}

}  // namespace owlgpu
