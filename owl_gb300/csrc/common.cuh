// common.cuh -- shared definitions for libowlgpu (sm_103a).
//
// Geometry is always carried as a 3-D problem: a 2-D Owl array
// [batch][cols][rows][ch] is the 3-D array [batch][cols][rows][1][ch] with a
// unit depth axis, which keeps the flat element order (and therefore Owl's
// flat argmax indices and window scan order) unchanged.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

namespace owlgpu {

enum Dtype { F32 = 0, F64 = 1, C32 = 2, C64 = 3 };

// Complex elements of Owl's Complex32 / Complex64 arrays: two reals, real
// part first (the layout of C's `float _Complex` / `double _Complex`).
// Arithmetic follows Owl's complex stubs: products of the plain formula
// (cblas_cgemm / cblas_zgemm, no conjugation anywhere), sums componentwise,
// division by a count componentwise (C's complex / real), and ordering by
// magnitude then argument (CLTF / CLT, src/owl/core/owl_core.h:125, :133).
// Its own namespace, so that `fma` and the operators reach it only by
// argument-dependent lookup and never hide the real overloads.
namespace cx {
template <typename R>
struct __align__(2 * sizeof(R)) cplx {
  R re, im;
  cplx() = default;
  __host__ __device__ explicit constexpr cplx(R r) : re(r), im(0) {}
  __host__ __device__ constexpr cplx(R r, R i) : re(r), im(i) {}
  __host__ __device__ cplx &operator+=(const cplx &b) {
    re += b.re;
    im += b.im;
    return *this;
  }
};
template <typename R>
__host__ __device__ inline cplx<R> operator+(cplx<R> a, const cplx<R> &b) {
  a += b;
  return a;
}
// c + a*b, the real part as ((c.re + a.re*b.re) - a.im*b.im) with each step
// fused, the imaginary part likewise.
template <typename R>
__device__ inline cplx<R> fma(const cplx<R> &a, const cplx<R> &b, const cplx<R> &c) {
  cplx<R> r;
  r.re = ::fma(-a.im, b.im, ::fma(a.re, b.re, c.re));
  r.im = ::fma(a.im, b.re, ::fma(a.re, b.im, c.im));
  return r;
}
__device__ inline float mag(const cplx<float> &a) { return hypotf(a.re, a.im); }
__device__ inline double mag(const cplx<double> &a) { return hypot(a.re, a.im); }
__device__ inline float arg(const cplx<float> &a) { return atan2f(a.im, a.re); }
__device__ inline double arg(const cplx<double> &a) { return atan2(a.im, a.re); }
template <typename R>
__device__ inline bool operator<(const cplx<R> &a, const cplx<R> &b) {
  const R ma = mag(a), mb = mag(b);
  return ma < mb || (ma == mb && arg(a) < arg(b));
}
}  // namespace cx

using c32 = cx::cplx<float>;
using c64 = cx::cplx<double>;

// x / n for a window count n: the element type's division, componentwise for
// complex elements.
template <typename T>
__device__ __forceinline__ T div_count(const T &x, int n) { return x / (T)n; }
template <>
__device__ __forceinline__ c32 div_count<c32>(const c32 &x, int n) {
  return c32(x.re / (float)n, x.im / (float)n);
}
template <>
__device__ __forceinline__ c64 div_count<c64>(const c64 &x, int n) {
  return c64(x.re / (double)n, x.im / (double)n);
}

// Convolution geometry.  Leading pads are the values Owl's C stubs derive
// (owl_ndarray_conv_impl.h:288-294 forward, :502-505 backward); dilation is
// the "in stride" (owl_ndarray_conv_impl.h:3141-3142).
struct ConvGeom {
  int64_t B;
  int64_t IC, IR, ID, Ci;  // input cols, rows, dpts, channels
  int64_t KC, KR, KD;      // kernel extent
  int64_t OC, OR, OD, Co;  // output cols, rows, dpts, channels
  int sc, sr, sd;          // strides
  int dc, dr, dd;          // dilation rates
  int pc, pr, pd;          // leading padding
  int64_t in_pixels() const { return B * IC * IR * ID; }
  int64_t out_pixels() const { return B * OC * OR * OD; }
  int64_t taps() const { return KC * KR * KD; }
  int64_t x_elems() const { return in_pixels() * Ci; }
  int64_t y_elems() const { return out_pixels() * Co; }
  int64_t w_elems() const { return taps() * Ci * Co; }
};

// Pooling geometry (owl_ndarray_pool_impl.h:9-15, :212-219).
struct PoolGeom {
  int64_t B;
  int64_t IC, IR, ID, Ch;
  int64_t KC, KR, KD;
  int64_t OC, OR, OD;
  int sc, sr, sd;
  int pc, pr, pd;
  int64_t in_pixels() const { return B * IC * IR * ID; }
  int64_t out_pixels() const { return B * OC * OR * OD; }
  int64_t x_elems() const { return in_pixels() * Ch; }
  int64_t y_elems() const { return out_pixels() * Ch; }
};

enum PoolMode { POOL_MAX = 0, POOL_AVG = 1 };

// Nearest-neighbour 2-D upsampling geometry (owl_ndarray_upsampling_impl.h:
// 9-32): input [B][IC][IR][Ch], output [B][OC][OR][Ch], scales sc (cols) and
// sr (rows).
struct UpGeom {
  int64_t B, IC, IR, Ch, OC, OR;
  int sc, sr;
  int64_t x_elems() const { return B * IC * IR * Ch; }
  int64_t y_elems() const { return B * OC * OR * Ch; }
};

// Status codes (mirrors include/owlgpu.h).
constexpr int kOk = 0;
constexpr int kErrInvalid = -1;
constexpr int kErrCuda = -2;
constexpr int kErrNoMem = -3;
constexpr int kErrUnsupported = -4;
constexpr int kErrTimeout = -5;

// Thread-local error text, read back through owlgpu_last_error().
void set_error(const std::string &msg);
const char *get_error();
int cuda_fail(cudaError_t e, const char *where);

// Launch accounting: every kernel launch in the library goes through
// note_launch() so that a caller can count the GPU work it triggered.
extern std::atomic<uint64_t> g_launches;
inline void note_launch(int n = 1) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

// Launch kernel k as a programmatic dependent of the work before it on s: it
// may be scheduled while that work drains, so the launch gap overlaps the
// previous kernel's tail.  Every such kernel executes griddepcontrol.wait
// before it touches global memory, and so sees all earlier work complete.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, static_cast<Args &&>(args)...);
}

#define OWL_CHECK_LAUNCH(where)                                   \
  do {                                                            \
    owlgpu::note_launch();                                        \
    cudaError_t _e = cudaGetLastError();                          \
    if (_e != cudaSuccess) return owlgpu::cuda_fail(_e, where);   \
  } while (0)

#define OWL_CUDA(call)                                            \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) return owlgpu::cuda_fail(_e, #call);   \
  } while (0)

// Stream-ordered scratch allocation used by kernels that need workspace.
int scratch_alloc(void **p, size_t bytes, cudaStream_t s);
void scratch_free(void *p, cudaStream_t s);

// ---- compute entry points (device pointers, asynchronous) --------------
// Forward convolution; with `bias` (per output channel, or null) and `act`
// (OWLGPU_ACT_*), y = act(conv + bias): in the tensor-core epilogue, or by a
// second pass after the CUDA-core kernel.
int conv_fwd(Dtype dt, int prec, const ConvGeom &g, const void *x, const void *w, void *y,
             cudaStream_t s, const void *bias = nullptr, int act = 0);
// y[i] = act(y[i] + bias[i % C]) over n elements (real kinds).
int bias_act_inplace(Dtype dt, void *y, const void *bias, long long n, long long C, int act,
                     cudaStream_t s);
int conv_bwd_input(Dtype dt, int prec, const ConvGeom &g, void *dx, const void *w,
                   const void *dy, cudaStream_t s);
int conv_bwd_kernel(Dtype dt, int prec, const ConvGeom &g, const void *x, void *dw,
                    const void *dy, cudaStream_t s);

int pool_fwd(Dtype dt, PoolMode mode, const PoolGeom &g, const void *x, void *y,
             int64_t *argmax, cudaStream_t s);
int pool_bwd(Dtype dt, PoolMode mode, const PoolGeom &g, const void *x, const void *dy,
             void *dx, cudaStream_t s);

// y = x repeated sc times along cols and sr times along rows; dx = the sum of
// dy over each input element's block, in Owl's order.
int upsample_fwd(Dtype dt, const UpGeom &g, const void *x, void *y, cudaStream_t s);
int upsample_bwd(Dtype dt, const UpGeom &g, void *dx, const void *dy, cudaStream_t s);

// SIMT (CUDA-core) implementations: the plain FP32 path and the FP64 path.
int simt_conv_fwd(Dtype dt, const ConvGeom &g, const void *x, const void *w, void *y,
                  cudaStream_t s);
int simt_conv_bwd_input(Dtype dt, const ConvGeom &g, void *dx, const void *w, const void *dy,
                        cudaStream_t s);
int simt_conv_bwd_kernel(Dtype dt, const ConvGeom &g, const void *x, void *dw, const void *dy,
                         cudaStream_t s);

// A pass of a 1x1 geometry on the CUDA cores as a split-K GEMM (partials
// summed in order): mode 0 forward (a = x, b = w, c = y), 1 backward_input
// (a = dy, b = w, c = dx), 2 backward_kernel (a = x, b = dy, c = dw).
int simt_gemm(Dtype dt, int mode, const ConvGeom &g, const void *a, const void *b, void *c,
              cudaStream_t s);

// backward_kernel (float32, SIMT) with split-K partials in a caller-provided
// workspace of ws_elems floats; splits are capped to fit it.
// A ConvGeom from Owl stub arguments, with the argument checks every conv
// entry point applies (dimensions 0..2^30, strides and rates 1..2^20,
// padding 0 or 1 for forward) and the stubs' padding rules (`bwd` selects
// the backward rule).  Sets the error message and returns kErrInvalid on a
// bad argument.
int make_conv(const char *fn, ConvGeom &g, long B, long IC, long IR, long ID, long Ci, long KC,
              long KR, long KD, long OC, long OR, long OD, long Co, long sc, long sr, long sd,
              long dc, long dr, long dd, bool bwd, long padding);

int simt_conv_bwd_kernel_f32_into(const ConvGeom &g, const float *x, float *dw,
                                  const float *dy, float *ws, int64_t ws_elems,
                                  cudaStream_t s);

// Tensor-core (tcgen05) implementations for float32 data.  Return
// kErrUnsupported when a geometry is outside what the kernels handle, in
// which case the caller reports the error (there is no silent fallback).
int tc_conv_fwd(int prec, const ConvGeom &g, const float *x, const float *w, float *y,
                cudaStream_t s, const float *bias = nullptr, int act = 0);
int tc_conv_bwd_input(int prec, const ConvGeom &g, float *dx, const float *w, const float *dy,
                      cudaStream_t s);
int tc_conv_bwd_kernel(int prec, const ConvGeom &g, const float *x, float *dw, const float *dy,
                       cudaStream_t s);

// Weight-image cache of the tensor-core convolutions: declare a kernel
// tensor's contents version (its cached images are dropped when the version
// changes), forget a pointer, or drop every image.  Dropping synchronises
// the device first.
int weights_declare(const void *w, uint64_t version);
int weights_forget(const void *w);
int weights_drop_all();

// A convolution whose kernel equals its stride (no dilation or padding,
// windows tiling the input): forward (bwd_kernel false: x, w -> out = y) or
// backward_kernel (x, dy -> out = dw) as a tcgen05 GEMM over the windows.
// kErrUnsupported for any other geometry or precision.
int tc_conv_s2d(int prec, bool bwd_kernel, const ConvGeom &g, const float *x,
                const float *w_or_dy, float *out, const float *bias, int act, cudaStream_t s);

// Cycles a tensor-core pipeline wait polls before its CTA gives up and sets
// the device error word (default about 2 s; shorter for a watchdog or for
// exercising the give-up path).
long long wait_limit();
long long set_wait_limit(long long cycles);

// Read (and clear) the tensor-core kernels' device error word on stream s.
int tc_read_status(int *out, cudaStream_t s);
// The same in two steps around a synchronisation the caller makes anyway:
// enqueue the copies of the status words on s, then (after s has been
// synchronised) take their value and clear the words that were set.
int tc_status_enqueue(cudaStream_t s);
int tc_status_take(int *out, cudaStream_t s);
int *tc_wgrad_status_word();  // device address of the weight-gradient kernel's status word
int *tc_gemm_status_word();   // device address of the tensor-core GEMM's status word
// out[i] = sum over r = 0 .. R-1 of part[r * n + i], in that order.
int sum_partials_f32(const float *part, float *out, long long n, int R, cudaStream_t s);
// The calling thread launched a tensor-core kernel (whose watchdog status the
// host drop-in then reads); take_tc_launched() returns and clears the mark.
void note_tc_launch();
bool take_tc_launched();

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace owlgpu
