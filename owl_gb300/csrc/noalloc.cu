// noalloc.cu -- a backward-kernel entry point that allocates no memory.
//
// Some callers cannot let a library allocate device memory during a call:
//   * a host program whose GPU memory is entirely owned by another allocator
//     (a serving engine or training framework that reserved HBM up front in
//     its own arena), where a fresh cudaMalloc/cudaMallocAsync either fails or
//     carves memory out from under that arena;
//   * latency-critical or budget-audited code (real-time inference loops,
//     certified deployments) that must not stall on the driver's allocator
//     or exceed a memory budget fixed before the program starts.
// For them, owlgpu_float32_ndarray_conv_spatial_backward_kernel_noalloc runs
// the same FP32 split-K backward-kernel kernels as the regular entry point,
// but its split-K partial sums live in one file-scope device array of
// kNoallocScratchFloats floats (16 MiB) instead of a per-call allocation.
//
// The array exists on every GPU on which this library's kernels are loaded
// and stays there until the process exits.  Its device address is obtained
// once per device with cudaGetSymbolAddress (the host-side name of a
// __device__ variable is only a stand-in, never a usable device pointer);
// that set-up happens inside the first call made on a device, with that
// device current, so the first call on each device should come before any
// stream capture.  All calls share the array: two calls whose kernels
// overlap on the GPU (different streams, or different host threads) race on
// it and produce wrong results; serialise them.  Each call writes every
// partial it later reads, so no clearing is needed between calls.  The
// array's address is kept per device for the life of the process, so
// cudaDeviceReset is not supported while this library is loaded (a reset
// reloads the module and may move the array).
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/owlgpu.h"
#include "common.cuh"

namespace owlgpu {
namespace {

constexpr int64_t kNoallocScratchFloats = int64_t(4) << 20;  // 16 MiB per device

static __device__ __align__(256) float g_noalloc_scratch[kNoallocScratchFloats];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
float *g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (set-up on the
// first call per device).
int noalloc_scratch(float **out) {
  int dev = 0;
  OWL_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("noalloc: device ordinal out of range");
    return kErrInvalid;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_ptr[dev] == nullptr) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[dev] = static_cast<float *>(p);
  }
  *out = g_noalloc_ptr[dev];
  return kOk;
}

}  // namespace
}  // namespace owlgpu

using namespace owlgpu;

extern "C" int owlgpu_float32_ndarray_conv_spatial_backward_kernel_noalloc(
    const float *input, float *kernel_grad, const float *output_grad, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride, long col_stride,
    long row_in_stride, long col_in_stride, void *stream) {
  // As in the regular backward-kernel stub, the in-strides are unused.
  (void)row_in_stride;
  (void)col_in_stride;
  const char *fn = "conv_spatial_backward_kernel_noalloc";
  // the same argument checks and padding rule as the regular entry point
  ConvGeom g;
  int rc = make_conv(fn, g, batches, input_cols, input_rows, 1, in_channel, kernel_cols,
                     kernel_rows, 1, output_cols, output_rows, 1, out_channel, col_stride,
                     row_stride, 1, 1, 1, 1, true, 0);
  if (rc) return rc;
  // kernel elements, multiplied out only while they stay within the limit
  // (each factor is at most 2^30, so the running product cannot overflow)
  int64_t kernel_elems = 1;
  for (long d : {kernel_cols, kernel_rows, in_channel, out_channel}) {
    kernel_elems *= d;
    if (kernel_elems > kNoallocScratchFloats) {
      set_error(std::string(fn) + ": the kernel has more than " +
                std::to_string(kNoallocScratchFloats) +
                " elements, the most this entry point handles (its fixed 16 MiB device "
                "scratch); use the allocating entry point");
      return kErrInvalid;
    }
    if (kernel_elems == 0) break;
  }
  float *ws = nullptr;
  rc = noalloc_scratch(&ws);
  if (rc) return rc;
  return simt_conv_bwd_kernel_f32_into(g, input, kernel_grad, output_grad, ws,
                                       kNoallocScratchFloats, (cudaStream_t)stream);
}
