/*
 * owlgpu.h -- C ABI of libowlgpu, a GB300 (sm_103a) implementation of Owl's
 * dense-ndarray convolution and pooling stubs.
 *
 * Two families of entry points replace the C stubs that Owl binds from
 * src/owl/core/owl_ndarray_conv.ml and src/owl/core/owl_ndarray_pool.ml:
 *
 *  1. Host drop-in, `owl_<kind>_ndarray_<op>`: the OCaml `external` name of
 *     the stub it replaces, the same argument order, meaning and units, with
 *     Bigarray values replaced by their data pointers (host memory) and OCaml
 *     ints by `long`.  The call copies the inputs to the GPU, runs, copies the
 *     outputs back and returns when the outputs are in host memory, exactly
 *     like the synchronous CPU stub.  Outputs are fully overwritten (the CPU
 *     stubs memset them first), so `_ ~out` callers see the same behaviour.
 *
 *  2. Device resident, `owlgpu_<kind>_ndarray_<op>`: the same arguments with
 *     device pointers, followed by `precision` (float32 only; ignored for
 *     float64) and a `cudaStream_t` passed as `void *` (NULL = the legacy
 *     default stream).  The call is asynchronous on that stream.
 *
 * Every entry point returns OWLGPU_OK (0) or a negative status; the reason is
 * available from owlgpu_last_error() on the calling thread.  Nothing aborts
 * the process.  The Owl stubs return unit and exit(1) on allocation failure
 * (owl_ndarray_conv_impl.h:300); the OCaml binding turns a negative status
 * into an exception instead.
 *
 * Layouts are Owl's row-major ones: input [batch][cols][rows]([dpts])[ch],
 * kernel [kcols][krows]([kdpts])[in_ch][out_ch].  "row_stride"/"col_stride"
 * follow the stub parameter names (col = dim 1, row = dim 2).
 */
#ifndef OWLGPU_H
#define OWLGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ---- status, precision, housekeeping ---------------------------------- */

#define OWLGPU_OK              0
#define OWLGPU_ERR_INVALID    -1 /* bad shape / argument                  */
#define OWLGPU_ERR_CUDA       -2 /* CUDA runtime error                    */
#define OWLGPU_ERR_NOMEM      -3 /* device or pinned allocation failed    */
#define OWLGPU_ERR_UNSUPPORTED -4
#define OWLGPU_ERR_TIMEOUT    -5 /* a bounded device-side wait gave up    */

/* Arithmetic used by float32 convolutions.  FP32 is the plain SIMT kernel
 * (results within 1e-4 relative of Owl's S.conv2d); TF32 and BF16 run on the
 * tcgen05 tensor cores with FP32 accumulation; BF16X3 splits each operand
 * into bf16 hi + lo parts and sums hi*hi + hi*lo + lo*hi on the tensor cores
 * (close to FP32 accuracy).  Float64 always runs FP64 SIMT kernels. */
#define OWLGPU_PREC_FP32   0
#define OWLGPU_PREC_TF32   1
#define OWLGPU_PREC_BF16   2
#define OWLGPU_PREC_BF16X3 3

/* Last error message of the calling thread ("" if none). */
const char *owlgpu_last_error(void);
/* Library version string. */
const char *owlgpu_version(void);
/* Process-wide precision used by the host drop-in float32 convolutions.
 * The initial value comes from the environment variable OWLGPU_PRECISION
 * (fp32 | tf32 | bf16 | bf16x3), default fp32. Returns the previous value. */
int owlgpu_set_precision(int precision);
int owlgpu_get_precision(void);
/* Number of kernel launches issued by this library since the process began
 * (all threads).  Lets a caller count GPU work inside a timed region. */
uint64_t owlgpu_launch_count(void);
/* Kernel family that ran the calling thread's last convolution:
 * 0 = CUDA cores (FP32 / FP64), 1 = tcgen05 tensor cores, -1 = none yet. */
int owlgpu_last_conv_path(void);
/* Synchronise the host drop-in stream and report OWLGPU_ERR_TIMEOUT if a
 * tensor-core kernel abandoned a bounded pipeline wait since the last check
 * (the host drop-in entry points check this themselves). */
int owlgpu_device_status(void);
/* Device ordinal used by the host drop-in entry points (default 0). */
int owlgpu_set_device(int device);
/* Release cached device/pinned staging memory held by the host drop-in,
 * and every cached weight image (below). */
int owlgpu_trim(void);
/* Weight-image cache (no counterpart in Owl, whose stubs re-pack their
 * kernel operand on every call too).  The tensor-core convolutions re-lay
 * the kernel tensor out into the image of its shared-memory tiles on every
 * call.  A caller whose kernel tensors stay unchanged across calls -- a
 * serving loop -- declares their contents with a version; later calls on
 * the current device whose kernel pointer has a declared version reuse the
 * images built for that version (one per layout the call's geometry needs),
 * so a captured forward pass launches no re-layout.  An image is built by
 * the first call that needs it outside stream capture, which synchronises
 * its stream once; calls made while their stream is capturing and finding
 * no image re-lay the tensor out per call as usual.  The caller declares a
 * new version whenever it changes the tensor's contents, and forgets the
 * pointer before freeing it (images are keyed by device address); both drop
 * the pointer's images after synchronising the device, and neither may race
 * with calls that use the pointer. */
int owlgpu_weights_declare(const void *kernel, uint64_t version);
int owlgpu_weights_forget(const void *kernel);

/* Device buffers and streams for a caller that does not link the CUDA
 * runtime itself -- the OCaml binding's custom blocks (owl_gb300/ocaml/
 * owlgpu_device_stubs.c), which hold the pointers the device-resident entry
 * points take.  No counterpart in Owl, whose arrays live in host memory.
 * Streams are created on the device of owlgpu_set_device, blocking with
 * respect to the legacy default stream (NULL).  Allocation and free are
 * stream-ordered: a buffer freed on the legacy default stream is released
 * after all earlier work on every such stream.  The copies return when the
 * bytes have arrived. */
int owlgpu_stream_create(void **stream);
int owlgpu_stream_destroy(void *stream);
int owlgpu_stream_synchronize(void *stream);
int owlgpu_device_alloc(void **ptr, uint64_t bytes, void *stream);
int owlgpu_device_free(void *ptr, void *stream);
int owlgpu_copy_to_device(void *dst, const void *src, uint64_t bytes, void *stream);
int owlgpu_copy_to_host(void *dst, const void *src, uint64_t bytes, void *stream);

/* ======================================================================
 * Convolution.  Owl kernel families: GEBP `spatial*` for 2-D
 * (owl_ndarray_conv.ml:257-282), `cuboid_*_im2col` for 3-D
 * (owl_ndarray_conv.ml:826-851), `dilated_*_im2col` (owl_ndarray_conv.ml:
 * 2540-2596).  All of them map onto the same GPU implementation.
 * ====================================================================== */

/* replaces stub_float32_ndarray_conv_spatial_native
 * (owl_ndarray_conv.ml:13, owl_ndarray_conv_impl.h:246-253).
 * padding: 0 = SAME, 1 = VALID. row/col_in_stride are ignored as in Owl. */
int owl_float32_ndarray_conv_spatial(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);
/* replaces stub_float64_ndarray_conv_spatial_native (owl_ndarray_conv.ml:34) */
int owl_float64_ndarray_conv_spatial(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);

/* replaces stub_float32_ndarray_conv_spatial_backward_input_native
 * (owl_ndarray_conv.ml:97, owl_ndarray_conv_impl.h:465-472).
 * First argument is dX (written); `output` is dY.  The padding is re-derived
 * from the shapes as in owl_ndarray_conv_impl.h:502-505. */
int owl_float32_ndarray_conv_spatial_backward_input(
    float *input_grad, const float *kernel, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
/* replaces stub_float64_ndarray_conv_spatial_backward_input_native (:117) */
int owl_float64_ndarray_conv_spatial_backward_input(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);

/* replaces stub_float32_ndarray_conv_spatial_backward_kernel_native
 * (owl_ndarray_conv.ml:177, owl_ndarray_conv_impl.h:675-682).
 * Second argument is dW (written). */
int owl_float32_ndarray_conv_spatial_backward_kernel(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
/* replaces stub_float64_ndarray_conv_spatial_backward_kernel_native (:197) */
int owl_float64_ndarray_conv_spatial_backward_kernel(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);

/* replace the im2col spelling of the same three 2-D stubs
 * (owl_ndarray_conv.ml:287, :308, :328 and float64 :415, :436, :456).
 * Identical semantics to the GEBP entry points above. */
int owl_float32_ndarray_conv_spatial_im2col(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_spatial_im2col(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);
int owl_float32_ndarray_conv_spatial_backward_input_im2col(
    float *input_grad, const float *kernel, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_spatial_backward_input_im2col(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
int owl_float32_ndarray_conv_spatial_backward_kernel_im2col(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_spatial_backward_kernel_im2col(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);

/* replaces stub_{float32,float64}_ndarray_conv_cuboid_im2col_native
 * (owl_ndarray_conv.ml:348/:476, owl_ndarray_conv_impl.h:1211-1219). */
int owl_float32_ndarray_conv_cuboid_im2col(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding);
int owl_float64_ndarray_conv_cuboid_im2col(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding);
/* replaces stub_*_ndarray_conv_cuboid_backward_input_im2col_native
 * (owl_ndarray_conv.ml:393/:521, owl_ndarray_conv_impl.h:1456-1463). */
int owl_float32_ndarray_conv_cuboid_backward_input_im2col(
    float *input_grad, const float *kernel, const float *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride);
int owl_float64_ndarray_conv_cuboid_backward_input_im2col(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride);
/* replaces stub_*_ndarray_conv_cuboid_backward_kernel_im2col_native
 * (owl_ndarray_conv.ml:371/:499, owl_ndarray_conv_impl.h:1331-1338). */
int owl_float32_ndarray_conv_cuboid_backward_kernel_im2col(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride);
int owl_float64_ndarray_conv_cuboid_backward_kernel_im2col(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride);

/* replaces stub_*_ndarray_conv_dilated_spatial_im2col_native
 * (owl_ndarray_conv.ml:1992, owl_ndarray_conv_impl.h:3097-3103):
 * row/col_in_stride are the dilation rates. */
int owl_float32_ndarray_conv_dilated_spatial_im2col(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_dilated_spatial_im2col(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);
/* replaces stub_*_ndarray_conv_dilated_spatial_backward_input_im2col_native
 * (owl_ndarray_conv.ml:2033, owl_ndarray_conv_impl.h:3317-3323). */
int owl_float32_ndarray_conv_dilated_spatial_backward_input_im2col(
    float *input_grad, const float *kernel, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_dilated_spatial_backward_input_im2col(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
/* replaces stub_*_ndarray_conv_dilated_spatial_backward_kernel_im2col_native
 * (owl_ndarray_conv.ml:2013, owl_ndarray_conv_impl.h:3203-3209). */
int owl_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);

/* replaces stub_*_ndarray_conv_dilated_cuboid_im2col_native
 * (owl_ndarray_conv.ml:2053, owl_ndarray_conv_impl.h:3417-3426). */
int owl_float32_ndarray_conv_dilated_cuboid_im2col(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long dpt_in_stride, long row_in_stride,
    long col_in_stride, long padding);
int owl_float64_ndarray_conv_dilated_cuboid_im2col(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long dpt_in_stride, long row_in_stride,
    long col_in_stride, long padding);
/* replaces stub_*_ndarray_conv_dilated_cuboid_backward_input_im2col_native
 * (owl_ndarray_conv.ml:2104, owl_ndarray_conv_impl.h:3678-3686). */
int owl_float32_ndarray_conv_dilated_cuboid_backward_input_im2col(
    float *input_grad, const float *kernel, const float *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride, long dpt_in_stride,
    long row_in_stride, long col_in_stride);
int owl_float64_ndarray_conv_dilated_cuboid_backward_input_im2col(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride, long dpt_in_stride,
    long row_in_stride, long col_in_stride);
/* replaces stub_*_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native
 * (owl_ndarray_conv.ml:2079, owl_ndarray_conv_impl.h:3545-3553). */
int owl_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride, long dpt_in_stride,
    long row_in_stride, long col_in_stride);
int owl_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride, long dpt_in_stride,
    long row_in_stride, long col_in_stride);

/* ======================================================================
 * Pooling (owl_ndarray_pool.ml:1042-1115 dispatch; owl_ndarray_pool_impl.h).
 * Max pooling keeps Owl's tie rule (first maximum in scan order wins, NaN is
 * never selected); average pooling divides by the in-range element count.
 * ====================================================================== */

/* replaces stub_*_ndarray_{max,avg}pool_spatial_native
 * (owl_ndarray_pool.ml:9/:28, owl_ndarray_pool_impl.h:9-15) */
int owl_float32_ndarray_maxpool_spatial(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_float64_ndarray_maxpool_spatial(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_float32_ndarray_avgpool_spatial(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_float64_ndarray_avgpool_spatial(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);

/* replaces stub_*_ndarray_{max,avg}pool_spatial_backward_native
 * (owl_ndarray_pool.ml:47/:66, owl_ndarray_pool_impl.h:102-108).
 * (input, output_grad, input_grad written); pads are explicit, negatives
 * clipped to 0.  Average pooling ignores `input` (Owl passes a dummy). */
int owl_float32_ndarray_maxpool_spatial_backward(
    const float *input, const float *output_grad, float *input_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows, long pad_cols);
int owl_float64_ndarray_maxpool_spatial_backward(
    const double *input, const double *output_grad, double *input_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows, long pad_cols);
int owl_float32_ndarray_avgpool_spatial_backward(
    const float *input, const float *output_grad, float *input_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows, long pad_cols);
int owl_float64_ndarray_avgpool_spatial_backward(
    const double *input, const double *output_grad, double *input_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows, long pad_cols);

/* replaces stub_*_ndarray_maxpool_spatial_arg_native
 * (owl_ndarray_pool.ml:121 `maxpool_argmax_spatial`,
 *  owl_ndarray_pool_impl.h:459-465): max value and int64 flat index into the
 * whole input (batch offset included), -1 for a window with no maximum. */
int owl_float32_ndarray_maxpool_argmax_spatial(
    const float *input, float *output, int64_t *argmax, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long pad_rows, long pad_cols);
int owl_float64_ndarray_maxpool_argmax_spatial(
    const double *input, double *output, int64_t *argmax, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long pad_rows, long pad_cols);

/* replaces stub_*_ndarray_{max,avg}pool_cuboid_native
 * (owl_ndarray_pool.ml:140/:161, owl_ndarray_pool_impl.h:212-219) */
int owl_float32_ndarray_maxpool_cuboid(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long dpt_stride, long row_stride, long col_stride,
    long padding);
int owl_float64_ndarray_maxpool_cuboid(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long dpt_stride, long row_stride, long col_stride,
    long padding);
int owl_float32_ndarray_avgpool_cuboid(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long dpt_stride, long row_stride, long col_stride,
    long padding);
int owl_float64_ndarray_avgpool_cuboid(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long dpt_stride, long row_stride, long col_stride,
    long padding);

/* replaces stub_*_ndarray_{max,avg}pool_cuboid_backward_native
 * (owl_ndarray_pool.ml:182, owl_ndarray_pool_impl.h:324-331).  Note the
 * stride order col, row, dpt -- reversed relative to the forward. */
int owl_float32_ndarray_maxpool_cuboid_backward(
    const float *input, const float *output_grad, float *input_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long col_stride,
    long row_stride, long dpt_stride, long padding);
int owl_float64_ndarray_maxpool_cuboid_backward(
    const double *input, const double *output_grad, double *input_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long col_stride,
    long row_stride, long dpt_stride, long padding);
int owl_float32_ndarray_avgpool_cuboid_backward(
    const float *input, const float *output_grad, float *input_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long col_stride,
    long row_stride, long dpt_stride, long padding);
int owl_float64_ndarray_avgpool_cuboid_backward(
    const double *input, const double *output_grad, double *input_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long col_stride,
    long row_stride, long dpt_stride, long padding);

/* ======================================================================
 * Device-resident entry points.  For every host drop-in `owl_<kind>_ndarray_
 * <op>(args...)` above (except the 2-D `_im2col` spellings, which are plain
 * aliases) there is an `owlgpu_<kind>_ndarray_<op>(args..., int precision,
 * void *stream)` taking device pointers, asynchronous on `stream`.
 * ====================================================================== */

#define OWLGPU_DEVICE_ARGS , int precision, void *stream

int owlgpu_float32_ndarray_conv_spatial(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_spatial(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_spatial_backward_input(
    float *input_grad, const float *kernel, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_spatial_backward_input(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_spatial_backward_kernel(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_spatial_backward_kernel(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_cuboid_im2col(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_cuboid_im2col(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_cuboid_backward_input_im2col(
    float *input_grad, const float *kernel, const float *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_cuboid_backward_input_im2col(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_cuboid_backward_kernel_im2col(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_cuboid_backward_kernel_im2col(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_dilated_spatial_im2col(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_dilated_spatial_im2col(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_dilated_spatial_backward_input_im2col(
    float *input_grad, const float *kernel, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_dilated_spatial_backward_input_im2col(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_dilated_cuboid_im2col(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long dpt_in_stride, long row_in_stride,
    long col_in_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_dilated_cuboid_im2col(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long dpt_in_stride, long row_in_stride,
    long col_in_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_dilated_cuboid_backward_input_im2col(
    float *input_grad, const float *kernel, const float *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride, long dpt_in_stride,
    long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_dilated_cuboid_backward_input_im2col(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride, long dpt_in_stride,
    long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride, long dpt_in_stride,
    long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride, long dpt_in_stride,
    long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);

int owlgpu_float32_ndarray_maxpool_spatial(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_maxpool_spatial(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_avgpool_spatial(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_avgpool_spatial(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_maxpool_spatial_backward(
    const float *input, const float *output_grad, float *input_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_maxpool_spatial_backward(
    const double *input, const double *output_grad, double *input_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_avgpool_spatial_backward(
    const float *input, const float *output_grad, float *input_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_avgpool_spatial_backward(
    const double *input, const double *output_grad, double *input_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_maxpool_argmax_spatial(
    const float *input, float *output, int64_t *argmax, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long pad_rows, long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_maxpool_argmax_spatial(
    const double *input, double *output, int64_t *argmax, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long pad_rows, long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_maxpool_cuboid(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long dpt_stride, long row_stride, long col_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_maxpool_cuboid(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long dpt_stride, long row_stride, long col_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_avgpool_cuboid(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long dpt_stride, long row_stride, long col_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_avgpool_cuboid(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long dpt_stride, long row_stride, long col_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_maxpool_cuboid_backward(
    const float *input, const float *output_grad, float *input_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long col_stride,
    long row_stride, long dpt_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_maxpool_cuboid_backward(
    const double *input, const double *output_grad, double *input_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long col_stride,
    long row_stride, long dpt_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_avgpool_cuboid_backward(
    const float *input, const float *output_grad, float *input_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long col_stride,
    long row_stride, long dpt_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_avgpool_cuboid_backward(
    const double *input, const double *output_grad, double *input_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long col_stride,
    long row_stride, long dpt_stride, long padding OWLGPU_DEVICE_ARGS);

/* Pipeline-wait watchdog of the tensor-core kernels: a wait that polls
 * longer than `cycles` SM clock cycles makes its CTA unwind (wait for its own
 * copies and MMAs, free tensor memory, return) and sets the device status
 * word (owlgpu_device_status; host drop-ins return OWLGPU_ERR_TIMEOUT).
 * cycles <= 0 restores the default (4e9, about 2 s).  Returns the previous
 * limit; applies to launches made after the call. */
long long owlgpu_set_wait_limit(long long cycles);

/* ======================================================================
 * Nearest-neighbour 2-D upsampling (Owl's upsampling2d), host drop-in
 * (owl_*) and device-resident (owlgpu_*) forms.
 *
 * replaces stub_*_ndarray_upsampling_spatial_backward_native
 * (owl_ndarray_upsampling.ml:9-35, owl_ndarray_upsampling_impl.h:9-58):
 * (input_grad written, output_grad, batches, input_cols, input_rows,
 * in_channel, output_cols, output_rows, col_scale, row_scale).
 * input_grad[b][ic][ir][ch] = sum of output_grad over the output positions
 * whose (min(c / col_scale, input_cols - 1), min(r / row_scale,
 * input_rows - 1)) is (ic, ir), added in the stub's order.
 *
 * upsampling_spatial is the forward, which Owl computes in OCaml as
 * repeat input [|1; col_scale; row_scale; 1|] (owl_dense_ndarray_generic.ml:
 * 8223-8233): output[b][c][r][ch] = input[b][c / col_scale][r / row_scale][ch];
 * output_cols/rows must equal input_cols/rows times the scales.
 * ====================================================================== */
int owl_float32_ndarray_upsampling_spatial_backward(
    float *input_grad, const float *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long output_cols, long output_rows,
    long col_scale, long row_scale);
int owl_float64_ndarray_upsampling_spatial_backward(
    double *input_grad, const double *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long output_cols, long output_rows,
    long col_scale, long row_scale);
int owl_float32_ndarray_upsampling_spatial(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long in_channel, long output_cols, long output_rows,
    long col_scale, long row_scale);
int owl_float64_ndarray_upsampling_spatial(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long in_channel, long output_cols, long output_rows,
    long col_scale, long row_scale);
int owlgpu_float32_ndarray_upsampling_spatial_backward(
    float *input_grad, const float *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long output_cols, long output_rows,
    long col_scale, long row_scale OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_upsampling_spatial_backward(
    double *input_grad, const double *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long output_cols, long output_rows,
    long col_scale, long row_scale OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_upsampling_spatial(
    const float *input, float *output, long batches, long input_cols,
    long input_rows, long in_channel, long output_cols, long output_rows,
    long col_scale, long row_scale OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_upsampling_spatial(
    const double *input, double *output, long batches, long input_cols,
    long input_rows, long in_channel, long output_cols, long output_rows,
    long col_scale, long row_scale OWLGPU_DEVICE_ARGS);

/* ======================================================================
 * Complex32 / Complex64: the same entry points for Owl's complex kinds
 * (elements are {re, im} pairs, the layout of C's float/double _Complex).
 * They replace the complex stubs Owl binds next to each real one:
 * conv owl_ndarray_conv.ml:55, :76 (spatial), :137, :157 (backward_input),
 * :217, :237 (backward_kernel), :543-777 (spatial/cuboid im2col families),
 * :2266-2515 (dilated); pool owl_ndarray_pool.ml:525-740 (complex32),
 * :783-1022 (complex64); upsampling owl_ndarray_upsampling.ml:37, :51.
 * Semantics are those of the complex stubs: conv products without
 * conjugation (cblas_cgemm / cblas_zgemm, owl_ndarray_conv_stub.c);
 * average pooling sums componentwise and divides by the count; max pooling
 * orders by magnitude then argument (CLTF / CLT, owl_core.h:125, :133)
 * starting from -INFINITY, i.e. (-inf, 0).  The upsampling forward, which
 * Owl computes with `repeat`, is provided for symmetry.  `precision` is
 * ignored: complex convolutions run on the CUDA cores in the element type.
 * ====================================================================== */

typedef struct { float re, im; } owlgpu_complex32;
typedef struct { double re, im; } owlgpu_complex64;

int owl_complex32_ndarray_conv_spatial(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_spatial_backward_input(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial_backward_input(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_spatial_backward_kernel(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial_backward_kernel(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_spatial_im2col(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial_im2col(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_spatial_backward_input_im2col(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial_backward_input_im2col(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_spatial_backward_kernel_im2col(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial_backward_kernel_im2col(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_cuboid_im2col(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long padding);
int owl_complex64_ndarray_conv_cuboid_im2col(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long padding);
int owl_complex32_ndarray_conv_cuboid_backward_input_im2col(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex64_ndarray_conv_cuboid_backward_input_im2col(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex32_ndarray_conv_cuboid_backward_kernel_im2col(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex64_ndarray_conv_cuboid_backward_kernel_im2col(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex32_ndarray_conv_dilated_spatial_im2col(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_dilated_spatial_im2col(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_dilated_spatial_backward_input_im2col(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_dilated_spatial_backward_input_im2col(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_dilated_cuboid_im2col(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long dpt_in_stride, long row_in_stride, long col_in_stride, long padding);
int owl_complex64_ndarray_conv_dilated_cuboid_im2col(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long dpt_in_stride, long row_in_stride, long col_in_stride, long padding);
int owl_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride, long dpt_in_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride, long dpt_in_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride, long dpt_in_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride, long dpt_in_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_maxpool_spatial(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long padding, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_maxpool_spatial(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long padding, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_avgpool_spatial(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long padding, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_avgpool_spatial(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long padding, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_maxpool_spatial_backward(
    const owlgpu_complex32 *input, const owlgpu_complex32 *output_grad,
    owlgpu_complex32 *input_grad, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long row_stride, long col_stride, long pad_rows,
    long pad_cols);
int owl_complex64_ndarray_maxpool_spatial_backward(
    const owlgpu_complex64 *input, const owlgpu_complex64 *output_grad,
    owlgpu_complex64 *input_grad, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long row_stride, long col_stride, long pad_rows,
    long pad_cols);
int owl_complex32_ndarray_avgpool_spatial_backward(
    const owlgpu_complex32 *input, const owlgpu_complex32 *output_grad,
    owlgpu_complex32 *input_grad, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long row_stride, long col_stride, long pad_rows,
    long pad_cols);
int owl_complex64_ndarray_avgpool_spatial_backward(
    const owlgpu_complex64 *input, const owlgpu_complex64 *output_grad,
    owlgpu_complex64 *input_grad, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long row_stride, long col_stride, long pad_rows,
    long pad_cols);
int owl_complex32_ndarray_maxpool_argmax_spatial(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, int64_t *argmax,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows, long pad_cols);
int owl_complex64_ndarray_maxpool_argmax_spatial(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, int64_t *argmax,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows, long pad_cols);
int owl_complex32_ndarray_maxpool_cuboid(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long dpt_stride, long row_stride,
    long col_stride, long padding);
int owl_complex64_ndarray_maxpool_cuboid(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long dpt_stride, long row_stride,
    long col_stride, long padding);
int owl_complex32_ndarray_avgpool_cuboid(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long dpt_stride, long row_stride,
    long col_stride, long padding);
int owl_complex64_ndarray_avgpool_cuboid(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long dpt_stride, long row_stride,
    long col_stride, long padding);
int owl_complex32_ndarray_maxpool_cuboid_backward(
    const owlgpu_complex32 *input, const owlgpu_complex32 *output_grad,
    owlgpu_complex32 *input_grad, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long col_stride, long row_stride, long dpt_stride, long padding);
int owl_complex64_ndarray_maxpool_cuboid_backward(
    const owlgpu_complex64 *input, const owlgpu_complex64 *output_grad,
    owlgpu_complex64 *input_grad, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long col_stride, long row_stride, long dpt_stride, long padding);
int owl_complex32_ndarray_avgpool_cuboid_backward(
    const owlgpu_complex32 *input, const owlgpu_complex32 *output_grad,
    owlgpu_complex32 *input_grad, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long col_stride, long row_stride, long dpt_stride, long padding);
int owl_complex64_ndarray_avgpool_cuboid_backward(
    const owlgpu_complex64 *input, const owlgpu_complex64 *output_grad,
    owlgpu_complex64 *input_grad, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long col_stride, long row_stride, long dpt_stride, long padding);
int owl_complex32_ndarray_upsampling_spatial_backward(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long output_cols, long output_rows, long col_scale, long row_scale);
int owl_complex64_ndarray_upsampling_spatial_backward(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long output_cols, long output_rows, long col_scale, long row_scale);
int owl_complex32_ndarray_upsampling_spatial(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long in_channel, long output_cols,
    long output_rows, long col_scale, long row_scale);
int owl_complex64_ndarray_upsampling_spatial(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long in_channel, long output_cols,
    long output_rows, long col_scale, long row_scale);

int owlgpu_complex32_ndarray_conv_spatial(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_spatial(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_spatial_backward_input(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_spatial_backward_input(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_spatial_backward_kernel(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_spatial_backward_kernel(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_cuboid_im2col(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_cuboid_im2col(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_cuboid_backward_input_im2col(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_cuboid_backward_input_im2col(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_cuboid_backward_kernel_im2col(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_cuboid_backward_kernel_im2col(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_dilated_spatial_im2col(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_dilated_spatial_im2col(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_dilated_spatial_backward_input_im2col(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_dilated_spatial_backward_input_im2col(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_dilated_cuboid_im2col(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long dpt_in_stride, long row_in_stride, long col_in_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_dilated_cuboid_im2col(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long dpt_in_stride, long row_in_stride, long col_in_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride, long dpt_in_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride, long dpt_in_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride, long dpt_in_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride, long dpt_in_stride, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_maxpool_spatial(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long padding, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_maxpool_spatial(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long padding, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_avgpool_spatial(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long padding, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_avgpool_spatial(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long row_stride,
    long col_stride, long padding, long row_in_stride,
    long col_in_stride OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_maxpool_spatial_backward(
    const owlgpu_complex32 *input, const owlgpu_complex32 *output_grad,
    owlgpu_complex32 *input_grad, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_maxpool_spatial_backward(
    const owlgpu_complex64 *input, const owlgpu_complex64 *output_grad,
    owlgpu_complex64 *input_grad, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_avgpool_spatial_backward(
    const owlgpu_complex32 *input, const owlgpu_complex32 *output_grad,
    owlgpu_complex32 *input_grad, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_avgpool_spatial_backward(
    const owlgpu_complex64 *input, const owlgpu_complex64 *output_grad,
    owlgpu_complex64 *input_grad, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_maxpool_argmax_spatial(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, int64_t *argmax,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_maxpool_argmax_spatial(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, int64_t *argmax,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long row_stride, long col_stride, long pad_rows,
    long pad_cols OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_maxpool_cuboid(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long dpt_stride, long row_stride,
    long col_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_maxpool_cuboid(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long dpt_stride, long row_stride,
    long col_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_avgpool_cuboid(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long dpt_stride, long row_stride,
    long col_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_avgpool_cuboid(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long dpt_stride, long row_stride,
    long col_stride, long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_maxpool_cuboid_backward(
    const owlgpu_complex32 *input, const owlgpu_complex32 *output_grad,
    owlgpu_complex32 *input_grad, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long col_stride, long row_stride, long dpt_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_maxpool_cuboid_backward(
    const owlgpu_complex64 *input, const owlgpu_complex64 *output_grad,
    owlgpu_complex64 *input_grad, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long col_stride, long row_stride, long dpt_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_avgpool_cuboid_backward(
    const owlgpu_complex32 *input, const owlgpu_complex32 *output_grad,
    owlgpu_complex32 *input_grad, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long col_stride, long row_stride, long dpt_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_avgpool_cuboid_backward(
    const owlgpu_complex64 *input, const owlgpu_complex64 *output_grad,
    owlgpu_complex64 *input_grad, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long col_stride, long row_stride, long dpt_stride,
    long padding OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_upsampling_spatial_backward(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long output_cols, long output_rows, long col_scale,
    long row_scale OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_upsampling_spatial_backward(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long output_cols, long output_rows, long col_scale,
    long row_scale OWLGPU_DEVICE_ARGS);
int owlgpu_complex32_ndarray_upsampling_spatial(
    const owlgpu_complex32 *input, owlgpu_complex32 *output, long batches,
    long input_cols, long input_rows, long in_channel, long output_cols,
    long output_rows, long col_scale, long row_scale OWLGPU_DEVICE_ARGS);
int owlgpu_complex64_ndarray_upsampling_spatial(
    const owlgpu_complex64 *input, owlgpu_complex64 *output, long batches,
    long input_cols, long input_rows, long in_channel, long output_cols,
    long output_rows, long col_scale, long row_scale OWLGPU_DEVICE_ARGS);

/* ======================================================================
 * MEC and naive spellings.  Owl binds its memory-efficient (MEC) and naive
 * CPU conv algorithms as separate stubs with the same arguments as the
 * GEBP / im2col ones (owl_ndarray_conv.ml:856-1346 MEC, :1424-1914 naive;
 * owl_ndarray_conv_impl.h:1570-3086); they compute the same functions, and
 * Owl's unit_conv_mec_naive.ml runs its conv2d / conv3d suites on them.
 * These host drop-ins are aliases of the entry points above:
 *   conv_spatial[_backward_input|_backward_kernel]_{mec,naive}
 *     = conv_spatial[_backward_input|_backward_kernel]
 *   conv_cuboid[_backward_input|_backward_kernel]_{mec,naive}
 *     = conv_cuboid[_backward_input|_backward_kernel]_im2col
 * ====================================================================== */

int owl_float32_ndarray_conv_spatial_mec(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);
int owl_float32_ndarray_conv_spatial_backward_input_mec(
    float *input_grad, const float *kernel, const float *output_grad, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long row_in_stride, long col_in_stride);
int owl_float32_ndarray_conv_spatial_backward_kernel_mec(
    const float *input, float *kernel_grad, const float *output_grad, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long row_in_stride, long col_in_stride);
int owl_float32_ndarray_conv_cuboid_mec(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding);
int owl_float32_ndarray_conv_cuboid_backward_input_mec(
    float *input_grad, const float *kernel, const float *output_grad, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride);
int owl_float32_ndarray_conv_cuboid_backward_kernel_mec(
    const float *input, float *kernel_grad, const float *output_grad, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride);
int owl_float64_ndarray_conv_spatial_mec(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_spatial_backward_input_mec(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_spatial_backward_kernel_mec(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_cuboid_mec(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding);
int owl_float64_ndarray_conv_cuboid_backward_input_mec(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride);
int owl_float64_ndarray_conv_cuboid_backward_kernel_mec(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride);
int owl_complex32_ndarray_conv_spatial_mec(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_spatial_backward_input_mec(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_spatial_backward_kernel_mec(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_cuboid_mec(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long padding);
int owl_complex32_ndarray_conv_cuboid_backward_input_mec(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex32_ndarray_conv_cuboid_backward_kernel_mec(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex64_ndarray_conv_spatial_mec(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial_backward_input_mec(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial_backward_kernel_mec(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_cuboid_mec(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long padding);
int owl_complex64_ndarray_conv_cuboid_backward_input_mec(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex64_ndarray_conv_cuboid_backward_kernel_mec(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_float32_ndarray_conv_spatial_naive(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);
int owl_float32_ndarray_conv_spatial_backward_input_naive(
    float *input_grad, const float *kernel, const float *output_grad, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long row_in_stride, long col_in_stride);
int owl_float32_ndarray_conv_spatial_backward_kernel_naive(
    const float *input, float *kernel_grad, const float *output_grad, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long row_in_stride, long col_in_stride);
int owl_float32_ndarray_conv_cuboid_naive(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding);
int owl_float32_ndarray_conv_cuboid_backward_input_naive(
    float *input_grad, const float *kernel, const float *output_grad, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride);
int owl_float32_ndarray_conv_cuboid_backward_kernel_naive(
    const float *input, float *kernel_grad, const float *output_grad, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride);
int owl_float64_ndarray_conv_spatial_naive(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_spatial_backward_input_naive(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_spatial_backward_kernel_naive(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride);
int owl_float64_ndarray_conv_cuboid_naive(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding);
int owl_float64_ndarray_conv_cuboid_backward_input_naive(
    double *input_grad, const double *kernel, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride);
int owl_float64_ndarray_conv_cuboid_backward_kernel_naive(
    const double *input, double *kernel_grad, const double *output_grad,
    long batches, long input_cols, long input_rows, long input_dpts,
    long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts,
    long output_cols, long output_rows, long output_dpts, long out_channel,
    long dpt_stride, long row_stride, long col_stride);
int owl_complex32_ndarray_conv_spatial_naive(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_spatial_backward_input_naive(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_spatial_backward_kernel_naive(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex32_ndarray_conv_cuboid_naive(
    const owlgpu_complex32 *input, const owlgpu_complex32 *kernel,
    owlgpu_complex32 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long padding);
int owl_complex32_ndarray_conv_cuboid_backward_input_naive(
    owlgpu_complex32 *input_grad, const owlgpu_complex32 *kernel,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex32_ndarray_conv_cuboid_backward_kernel_naive(
    const owlgpu_complex32 *input, owlgpu_complex32 *kernel_grad,
    const owlgpu_complex32 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex64_ndarray_conv_spatial_naive(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long in_channel, long kernel_cols, long kernel_rows, long output_cols,
    long output_rows, long out_channel, long row_stride, long col_stride,
    long padding, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial_backward_input_naive(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_spatial_backward_kernel_naive(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long in_channel, long kernel_cols, long kernel_rows,
    long output_cols, long output_rows, long out_channel, long row_stride,
    long col_stride, long row_in_stride, long col_in_stride);
int owl_complex64_ndarray_conv_cuboid_naive(
    const owlgpu_complex64 *input, const owlgpu_complex64 *kernel,
    owlgpu_complex64 *output, long batches, long input_cols, long input_rows,
    long input_dpts, long in_channel, long kernel_cols, long kernel_rows,
    long kernel_dpts, long output_cols, long output_rows, long output_dpts,
    long out_channel, long dpt_stride, long row_stride, long col_stride,
    long padding);
int owl_complex64_ndarray_conv_cuboid_backward_input_naive(
    owlgpu_complex64 *input_grad, const owlgpu_complex64 *kernel,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);
int owl_complex64_ndarray_conv_cuboid_backward_kernel_naive(
    const owlgpu_complex64 *input, owlgpu_complex64 *kernel_grad,
    const owlgpu_complex64 *output_grad, long batches, long input_cols,
    long input_rows, long input_dpts, long in_channel, long kernel_cols,
    long kernel_rows, long kernel_dpts, long output_cols, long output_rows,
    long output_dpts, long out_channel, long dpt_stride, long row_stride,
    long col_stride);

/* ======================================================================
 * Extensions: the layers around the convolutions.  No counterpart among
 * Owl's C stubs: in Owl these are OCaml compositions of ndarray operations
 * inside the neural-network layers (src/base/neural/owl_neural_neuron.ml)
 * and the optimiser (src/base/optimise/owl_optimise_generic.ml).  They let
 * a training or serving step stay on the device in this library's own
 * kernels.  Device pointers, asynchronous on `stream`; every reduction sums
 * in a fixed order, so results repeat bit for bit.
 * ====================================================================== */

#define OWLGPU_ACT_NONE 0
#define OWLGPU_ACT_RELU 1 /* x > 0 ? x : 0, Owl's Activation Relu */

/* Conv2D / Conv3D neuron forward with its bias and activation:
 * output = act(conv(input, kernel) + bias[out_channel]), as Conv2D.run
 * (owl_neural_neuron.ml:1253, conv2d x w s + b) followed by an Activation
 * neuron.  Arguments of owlgpu_<kind>_ndarray_conv_spatial /
 * _conv_cuboid_im2col, then `bias` (out_channel values, or NULL for none)
 * and `act`.  On the tensor cores the bias and activation are applied in
 * the convolution's epilogue; the CUDA-core kernels apply them in a second
 * pass. */
int owlgpu_float32_ndarray_conv_spatial_bias_act(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride, const float *bias, int act OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_spatial_bias_act(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long in_channel, long kernel_cols,
    long kernel_rows, long output_cols, long output_rows, long out_channel,
    long row_stride, long col_stride, long padding, long row_in_stride,
    long col_in_stride, const double *bias, int act OWLGPU_DEVICE_ARGS);
int owlgpu_float32_ndarray_conv_cuboid_bias_act(
    const float *input, const float *kernel, float *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding, const float *bias,
    int act OWLGPU_DEVICE_ARGS);
int owlgpu_float64_ndarray_conv_cuboid_bias_act(
    const double *input, const double *kernel, double *output, long batches,
    long input_cols, long input_rows, long input_dpts, long in_channel,
    long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols,
    long output_rows, long output_dpts, long out_channel, long dpt_stride,
    long row_stride, long col_stride, long padding, const double *bias,
    int act OWLGPU_DEVICE_ARGS);

/* Backward of output = act(z + bias): pre_grad = output_grad * act'(z),
 * read from the layer's output (for ReLU, output > 0 exactly where z > 0),
 * and bias_grad[c] = the sum over pixels of pre_grad[p][c].  Arrays are
 * [pixels][channels]; pre_grad may alias output_grad; pre_grad or bias_grad
 * may be NULL (not written).  The backward of Owl's bias add and Relu
 * (owl_algodiff_ops.ml: add's adjoint summed over the broadcast axes,
 * relu's adjoint masked by x > 0). */
int owlgpu_float32_bias_act_backward(const float *output, const float *output_grad,
                                     float *pre_grad, float *bias_grad, long pixels,
                                     long channels, int act, void *stream);
int owlgpu_float64_bias_act_backward(const double *output, const double *output_grad,
                                     double *pre_grad, double *bias_grad, long pixels,
                                     long channels, int act, void *stream);

/* The dense layer's matrix product and the two products of its backward
 * pass (FullyConnected.run, owl_neural_neuron.ml:1907: (x *@ w) + b; Owl's
 * `dot` is cblas_?gemm): c[m][n] = act(sum over k of op(a)[m][k] op(b)[k][n]
 * + bias[n]), row-major.  op(a) = a stored [m][k], or with trans_a its
 * transpose (a stored [k][m]); op(b) = b stored [k][n], or with trans_b its
 * transpose (b stored [n][k]).  Both transposed is rejected.  bias: n
 * values or NULL.  float32 at BF16 / BF16X3 runs the tcgen05 GEMM (split-K,
 * partials summed in order); FP32 / TF32 and float64 run the CUDA-core
 * kernels (precision is ignored for float64). */
int owlgpu_float32_dot(const float *a, const float *b, float *c, long m, long n, long k,
                       int trans_a, int trans_b, const float *bias,
                       int act OWLGPU_DEVICE_ARGS);
int owlgpu_float64_dot(const double *a, const double *b, double *c, long m, long n, long k,
                       int trans_a, int trans_b, const double *bias,
                       int act OWLGPU_DEVICE_ARGS);

/* Softmax cross-entropy of a classifier's training step: loss = -sum over
 * rows and classes of labels * log softmax(logits), divided by rows (Owl's
 * Loss Cross_entropy, owl_optimise_generic.ml:172, cross_entropy
 * owl_algodiff_ops.ml:1392, softmax :918-922, and the batch mean of
 * owl_optimise_generic.ml:646-649); dlogits = (softmax(logits) - labels) *
 * dloss / rows.  logits, labels, dlogits: [rows][classes]; loss: one value;
 * dloss: the loss's adjoint on the device (one value) or NULL for 1;
 * loss or dlogits may be NULL (not written). */
int owlgpu_float32_softmax_cross_entropy(const float *logits, const float *labels,
                                         float *loss, float *dlogits, const float *dloss,
                                         long rows, long classes, void *stream);
int owlgpu_float64_softmax_cross_entropy(const double *logits, const double *labels,
                                         double *loss, double *dlogits, const double *dloss,
                                         long rows, long classes, void *stream);

/* Gradient-descent update weight -= lr * grad over n elements (Owl's
 * optimiser with a constant learning rate and no momentum). */
int owlgpu_float32_sgd_update(float *weight, const float *grad, long n, double lr,
                              void *stream);
int owlgpu_float64_sgd_update(double *weight, const double *grad, long n, double lr,
                              void *stream);

/* ======================================================================
 * Allocation-free entry point.  No counterpart in the reference: Owl's C
 * stubs allocate their own scratch with malloc.  This is the float32 2-D
 * conv backward_kernel (same arguments and results as
 * owlgpu_float32_ndarray_conv_spatial_backward_kernel at FP32) for callers
 * that cannot let a library allocate GPU memory mid-call: programs whose HBM
 * is owned by another allocator's arena, and latency- or budget-bound code
 * that must not touch the driver allocator.  Its split-K scratch is a fixed
 * 16 MiB device array held by every GPU that loads the library until exit;
 * kernels with more than 4,194,304 elements (kernel_cols * kernel_rows *
 * in_channel * out_channel) are rejected with OWLGPU_ERR_INVALID.  The first
 * call on a device looks up the array's device address, so make it before
 * any stream capture; calls that overlap on the GPU share the array and
 * race, so serialise them.  Device pointers; asynchronous on `stream`.
 * ====================================================================== */
int owlgpu_float32_ndarray_conv_spatial_backward_kernel_noalloc(
    const float *input, float *kernel_grad, const float *output_grad,
    long batches, long input_cols, long input_rows, long in_channel,
    long kernel_cols, long kernel_rows, long output_cols, long output_rows,
    long out_channel, long row_stride, long col_stride, long row_in_stride,
    long col_in_stride, void *stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif
#endif /* OWLGPU_H */
