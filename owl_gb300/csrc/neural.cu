// neural.cu -- the layers around the convolutions in a training or serving
// step, as device kernels of this library: the dense layer's matrix product,
// the bias + activation backward, softmax cross-entropy and the gradient
// descent update.  In Owl these are OCaml compositions of ndarray operations
// (FullyConnected.run, owl_neural_neuron.ml:1907; Loss Cross_entropy,
// owl_optimise_generic.ml:172 with the batch mean of :646-649; softmax,
// owl_algodiff_ops.ml:918-922; cross_entropy, :1392).
//
// Every reduction here sums in a fixed order, so results are bit-identical
// from run to run.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../../include/owlgpu.h"
#include "common.cuh"

namespace owlgpu {

int tc_gemm(int prec, bool trans_a, bool trans_b, long long M, long long N, long long K,
            const float *a, const float *b, float *c, const float *bias, int act,
            cudaStream_t s);

namespace {

template <typename T>
__device__ __forceinline__ T act_fn(T v, int act) {
  return act == OWLGPU_ACT_RELU ? (v > T(0) ? v : T(0)) : v;
}

// y[p][c] = act(y[p][c] + bias[c]) in place (bias may be null).
template <typename T>
__global__ void bias_act_kernel(T *__restrict__ y, const T *__restrict__ bias, long long n,
                                long long C, int act) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    T v = y[i];
    if (bias) v += bias[i % C];
    y[i] = act_fn(v, act);
  }
}

// dz = dy * act'(from y); partial[chunk][c] = sum of dz over the chunk's
// pixels, in pixel order within each of the 8 row groups, the groups summed
// in order.  Block (32, 8): x = channel within a 32-channel tile, y = row
// group.
constexpr int kBiasRows = 8;
template <typename T>
__global__ void bias_act_bwd_kernel(const T *__restrict__ y, const T *__restrict__ dy,
                                    T *__restrict__ dz, T *__restrict__ partial, long long P,
                                    long long C, long long rows_per_chunk, int act) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  __shared__ T red[kBiasRows][33];
  const long long c = (long long)blockIdx.x * 32 + threadIdx.x;
  const long long p0 = (long long)blockIdx.y * rows_per_chunk;
  const long long p1 = min(P, p0 + rows_per_chunk);
  T acc = T(0);
  if (c < C) {
    for (long long p = p0 + threadIdx.y; p < p1; p += kBiasRows) {
      const long long i = p * C + c;
      T g = dy[i];
      if (act == OWLGPU_ACT_RELU && !(y[i] > T(0))) g = T(0);
      if (dz) dz[i] = g;
      acc += g;
    }
  }
  red[threadIdx.y][threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.y == 0 && c < C && partial) {
    T s = red[0][threadIdx.x];
#pragma unroll
    for (int r = 1; r < kBiasRows; ++r) s += red[r][threadIdx.x];
    partial[(long long)blockIdx.y * C + c] = s;
  }
}

// out[c] = sum over chunks of partial[chunk][c]: block (32, 32), x = channel
// of a 32-channel tile, y = one of 32 interleaved chunk sets (y, y + 32,
// ...) summed in order, then the 32 set sums added in order (a fixed order
// whatever the run).
template <typename T>
__global__ void sum_chunks_kernel(const T *__restrict__ partial, T *__restrict__ out, long long C,
                                  int chunks) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  __shared__ T red[32][33];
  const long long c = (long long)blockIdx.x * 32 + threadIdx.x;
  T s = T(0);
  if (c < C)
    for (int k = threadIdx.y; k < chunks; k += 32) s += partial[(long long)k * C + c];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && c < C) {
    T t = red[0][threadIdx.x];
#pragma unroll 8
    for (int r = 1; r < 32; ++r) t += red[r][threadIdx.x];
    out[c] = t;
  }
}

__device__ __forceinline__ float exp_t(float v) { return expf(v); }
__device__ __forceinline__ double exp_t(double v) { return exp(v); }
__device__ __forceinline__ float log_t(float v) { return logf(v); }
__device__ __forceinline__ double log_t(double v) { return log(v); }

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// Sum over the warp's lanes in a fixed tree order (the same on every run).
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One warp per row: m = max, lse = log(sum exp(x - m)), row loss
// -sum(label * (x - m - lse)), dlogits = (exp(x - m - lse) - label) * scale.
template <typename T>
__global__ void softmax_ce_rows(const T *__restrict__ logits, const T *__restrict__ labels,
                                T *__restrict__ row_loss, T *__restrict__ dlogits,
                                const T *__restrict__ dloss, long long R, long long C) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  const long long r = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (r >= R) return;
  const T *x = logits + r * C;
  const T *l = labels + r * C;
  T m = -INFINITY;
  for (long long c = lane; c < C; c += 32) m = max(m, x[c]);
  m = warp_max(m);
  T s = T(0);
  for (long long c = lane; c < C; c += 32) s += exp_t(x[c] - m);
  s = warp_sum(s);
  const T lse = log_t(s);
  T acc = T(0);
  for (long long c = lane; c < C; c += 32) acc += l[c] * (x[c] - m - lse);
  acc = warp_sum(acc);
  if (lane == 0) row_loss[r] = -acc;
  if (dlogits) {
    const T scale = (dloss ? *dloss : T(1)) / (T)R;
    for (long long c = lane; c < C; c += 32)
      dlogits[r * C + c] = (exp_t(x[c] - m - lse) - l[c]) * scale;
  }
}

// loss = (sum over rows of row_loss, in a fixed order) / R, one block of 256.
template <typename T>
__global__ void softmax_ce_total(const T *__restrict__ row_loss, T *__restrict__ loss, long long R) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  __shared__ T part[256];
  T s = T(0);
  const long long per = (R + 255) / 256;
  const long long a = threadIdx.x * per, b = min(R, a + per);
  for (long long i = a; i < b; ++i) s += row_loss[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = part[0] / (T)R;
}

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// w -= lr * g with the product rounded before the subtraction (no fused
// multiply-add), as the composition rate * g, then w - that, rounds.
template <typename T>
__global__ void sgd_kernel(T *__restrict__ w, const T *__restrict__ g, long long n, T lr) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // launched with launch_pdl
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    w[i] = w[i] - mul_rn(lr, g[i]);
}

int grid_for(long long n, int threads) {
  return (int)std::max<long long>(1, std::min<long long>((n + threads - 1) / threads, 8 * 152));
}

int bad(const char *fn, const char *what) {
  set_error(std::string(fn) + ": " + what);
  return kErrInvalid;
}

template <typename T>
int bias_act(T *y, const T *bias, long long n, long long C, int act, cudaStream_t s) {
  if (n == 0 || (!bias && act == OWLGPU_ACT_NONE)) return kOk;
  cudaError_t e = launch_pdl(bias_act_kernel<T>, dim3(grid_for(n, 256)), dim3(256), 0, s, y,
                             bias, n, C, act);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  return e == cudaSuccess ? kOk : cuda_fail(e, "bias_act_kernel");
}

// C = op(A) op(B) on the CUDA cores, as a 1x1 convolution with its
// reduction split across CTAs: NN is a forward convolution of A ([M] pixels
// x [K] channels) with B ([K][N]), NT a backward_input (dY = A, kernel = B
// read as [N][K]), TN a backward_kernel (X = A over K pixels, dY = B).
template <typename T>
int simt_dot(Dtype dt, bool ta, bool tb, long long M, long long N, long long K, const T *a,
             const T *b, T *c, cudaStream_t s) {
  ConvGeom g{};
  g.B = 1; g.IC = 1; g.ID = 1; g.OC = 1; g.OD = 1;
  g.KC = g.KR = g.KD = 1;
  g.sc = g.sr = g.sd = 1; g.dc = g.dr = g.dd = 1;
  g.pc = g.pr = g.pd = 0;
  if (!ta && !tb) {
    g.IR = g.OR = M; g.Ci = K; g.Co = N;
    return simt_gemm(dt, 0, g, a, b, c, s);
  }
  if (!ta && tb) {
    g.IR = g.OR = M; g.Ci = N; g.Co = K;
    return simt_gemm(dt, 1, g, a, b, c, s);
  }
  g.IR = g.OR = K; g.Ci = M; g.Co = N;
  return simt_gemm(dt, 2, g, a, b, c, s);
}

template <typename T>
int dot_t(Dtype dt, const char *fn, const T *a, const T *b, T *c, long m, long n, long k,
          int trans_a, int trans_b, const T *bias, int act, int prec, cudaStream_t s) {
  if (m < 0 || n < 0 || k < 0 || m > (1L << 31) || n > (1L << 31) || k > (1L << 31))
    return bad(fn, "negative or oversized dimension");
  if (trans_a && trans_b) return bad(fn, "op(a) and op(b) both transposed is not supported");
  if (act != OWLGPU_ACT_NONE && act != OWLGPU_ACT_RELU) return bad(fn, "unknown activation");
  if (prec < OWLGPU_PREC_FP32 || prec > OWLGPU_PREC_BF16X3) return bad(fn, "unknown precision");
  if (m == 0 || n == 0) return kOk;
  if (k == 0) {
    OWL_CUDA(cudaMemsetAsync(c, 0, sizeof(T) * (size_t)m * n, s));
    return bias_act<T>(c, bias, (long long)m * n, n, act, s);
  }
  if constexpr (sizeof(T) == 4) {
    if (prec == OWLGPU_PREC_BF16 || prec == OWLGPU_PREC_BF16X3) {
      int rc = tc_gemm(prec, trans_a != 0, trans_b != 0, m, n, k, (const float *)a,
                       (const float *)b, (float *)c, (const float *)bias, act, s);
      if (rc != kErrUnsupported) return rc;
    }
  }
  int rc = simt_dot<T>(dt, trans_a != 0, trans_b != 0, m, n, k, a, b, c, s);
  if (rc) return rc;
  return bias_act<T>(c, bias, (long long)m * n, n, act, s);
}

template <typename T>
int bias_act_bwd_t(const char *fn, const T *y, const T *dy, T *dz, T *db, long P, long C, int act,
                   cudaStream_t s) {
  if (P < 0 || C < 0 || P > (1L << 40) || C > (1L << 31))
    return bad(fn, "negative or oversized dimension");
  if (act != OWLGPU_ACT_NONE && act != OWLGPU_ACT_RELU) return bad(fn, "unknown activation");
  if (C == 0) return kOk;
  if (P == 0) {
    if (db) OWL_CUDA(cudaMemsetAsync(db, 0, sizeof(T) * (size_t)C, s));
    return kOk;
  }
  if (!db && !dz) return kOk;
  // pixel chunks: about four blocks per SM over all channel tiles
  const long long ctiles = (C + 31) / 32;
  long long chunks = std::max<long long>(1, std::min<long long>(4 * 152 / ctiles + 1, P / 64));
  chunks = std::min<long long>(chunks, 4096);
  const long long rows = (P + chunks - 1) / chunks;
  chunks = (P + rows - 1) / rows;
  T *part = nullptr;
  if (db) {
    int rc = scratch_alloc((void **)&part, sizeof(T) * (size_t)(chunks * C), s);
    if (rc) return rc;
  }
  cudaError_t e = launch_pdl(bias_act_bwd_kernel<T>, dim3((unsigned)ctiles, (unsigned)chunks),
                             dim3(32, kBiasRows), 0, s, y, dy, dz, part, P, C, rows, act);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  int rc = e == cudaSuccess ? kOk : cuda_fail(e, "bias_act_bwd_kernel");
  if (rc == kOk && db) {
    e = launch_pdl(sum_chunks_kernel<T>, dim3((unsigned)ctiles), dim3(32, 32), 0, s,
                   (const T *)part, db, C, (int)chunks);
    if (e == cudaSuccess) e = cudaGetLastError();
    note_launch();
    if (e != cudaSuccess) rc = cuda_fail(e, "sum_chunks_kernel");
  }
  if (part) scratch_free(part, s);
  return rc;
}

template <typename T>
int softmax_ce_t(const char *fn, const T *logits, const T *labels, T *loss, T *dlogits,
                 const T *dloss, long R, long C, cudaStream_t s) {
  if (R <= 0 || C <= 0 || R > (1L << 31) || C > (1L << 31))
    return bad(fn, "rows and classes must be positive");
  if (!loss && !dlogits) return kOk;
  T *row_loss = nullptr;
  int rc = scratch_alloc((void **)&row_loss, sizeof(T) * (size_t)R, s);
  if (rc) return rc;
  const int rows_per_block = 8;
  cudaError_t e = launch_pdl(softmax_ce_rows<T>,
                             dim3((unsigned)((R + rows_per_block - 1) / rows_per_block)),
                             dim3(32 * rows_per_block), 0, s, logits, labels, row_loss, dlogits,
                             dloss, R, C);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  rc = e == cudaSuccess ? kOk : cuda_fail(e, "softmax_ce_rows");
  if (rc == kOk && loss) {
    e = launch_pdl(softmax_ce_total<T>, dim3(1), dim3(256), 0, s, (const T *)row_loss, loss,
                   (long long)R);
    if (e == cudaSuccess) e = cudaGetLastError();
    note_launch();
    if (e != cudaSuccess) rc = cuda_fail(e, "softmax_ce_total");
  }
  scratch_free(row_loss, s);
  return rc;
}

template <typename T>
int sgd_t(const char *fn, T *w, const T *g, long n, T lr, cudaStream_t s) {
  if (n < 0) return bad(fn, "negative size");
  if (n == 0) return kOk;
  cudaError_t e = launch_pdl(sgd_kernel<T>, dim3(grid_for(n, 256)), dim3(256), 0, s, w, g,
                             (long long)n, lr);
  if (e == cudaSuccess) e = cudaGetLastError();
  note_launch();
  return e == cudaSuccess ? kOk : cuda_fail(e, "sgd_kernel");
}

}  // namespace

int bias_act_inplace(Dtype dt, void *y, const void *bias, long long n, long long C, int act,
                     cudaStream_t s) {
  if (dt == F32) return bias_act<float>((float *)y, (const float *)bias, n, C, act, s);
  if (dt == F64) return bias_act<double>((double *)y, (const double *)bias, n, C, act, s);
  set_error("bias/activation: real element kinds only");
  return kErrInvalid;
}

}  // namespace owlgpu

using namespace owlgpu;

#define S(x) static_cast<cudaStream_t>(x)

extern "C" {

int owlgpu_float32_dot(const float *a, const float *b, float *c, long m, long n, long k,
                       int trans_a, int trans_b, const float *bias, int act, int precision,
                       void *stream) {
  return dot_t<float>(F32, "float32_dot", a, b, c, m, n, k, trans_a, trans_b, bias, act,
                      precision, S(stream));
}
int owlgpu_float64_dot(const double *a, const double *b, double *c, long m, long n, long k,
                       int trans_a, int trans_b, const double *bias, int act, int precision,
                       void *stream) {
  (void)precision;
  return dot_t<double>(F64, "float64_dot", a, b, c, m, n, k, trans_a, trans_b, bias, act,
                       OWLGPU_PREC_FP32, S(stream));
}

int owlgpu_float32_bias_act_backward(const float *output, const float *output_grad,
                                     float *pre_grad, float *bias_grad, long pixels,
                                     long channels, int act, void *stream) {
  return bias_act_bwd_t<float>("float32_bias_act_backward", output, output_grad, pre_grad,
                               bias_grad, pixels, channels, act, S(stream));
}
int owlgpu_float64_bias_act_backward(const double *output, const double *output_grad,
                                     double *pre_grad, double *bias_grad, long pixels,
                                     long channels, int act, void *stream) {
  return bias_act_bwd_t<double>("float64_bias_act_backward", output, output_grad, pre_grad,
                                bias_grad, pixels, channels, act, S(stream));
}

int owlgpu_float32_softmax_cross_entropy(const float *logits, const float *labels, float *loss,
                                         float *dlogits, const float *dloss, long rows,
                                         long classes, void *stream) {
  return softmax_ce_t<float>("float32_softmax_cross_entropy", logits, labels, loss, dlogits,
                             dloss, rows, classes, S(stream));
}
int owlgpu_float64_softmax_cross_entropy(const double *logits, const double *labels,
                                         double *loss, double *dlogits, const double *dloss,
                                         long rows, long classes, void *stream) {
  return softmax_ce_t<double>("float64_softmax_cross_entropy", logits, labels, loss, dlogits,
                              dloss, rows, classes, S(stream));
}

int owlgpu_float32_sgd_update(float *weight, const float *grad, long n, double lr, void *stream) {
  return sgd_t<float>("float32_sgd_update", weight, grad, n, (float)lr, S(stream));
}
int owlgpu_float64_sgd_update(double *weight, const double *grad, long n, double lr,
                              void *stream) {
  return sgd_t<double>("float64_sgd_update", weight, grad, n, lr, S(stream));
}

}  // extern "C"
