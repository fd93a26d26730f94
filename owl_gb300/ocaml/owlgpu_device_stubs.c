/* owlgpu_device_stubs.c -- device-resident Owl arrays for OCaml: device
 * buffers and CUDA streams held in custom blocks, and the stubs of
 * libowlgpu's device-resident entry points (include/owlgpu.h).  Generated
 * by make_stubs.py; link with -lowlgpu. */
#include <caml/alloc.h>
#include <caml/bigarray.h>
#include <caml/custom.h>
#include <caml/fail.h>
#include <caml/memory.h>
#include <caml/mlvalues.h>
#include <caml/signals.h>
#include <stddef.h>
#include <stdint.h>

#include "owlgpu.h"

/* ---- owlgpu.buf: device memory owned by the block ---------------------- */

typedef struct {
  void *ptr;
  uint64_t bytes;
} owlgpu_buf;

#define Buf_val(v) ((owlgpu_buf *)Data_custom_val(v))
#define Buf_ptr(v) (Buf_val(v)->ptr)

/* Released on the legacy default stream: after all earlier work on every
 * stream of the library (they are blocking streams), whichever stream the
 * buffer was used on. */
static void owlgpu_buf_finalize(value v) {
  owlgpu_buf *b = Buf_val(v);
  if (b->ptr) owlgpu_device_free(b->ptr, NULL);
  b->ptr = NULL;
  b->bytes = 0;
}

static struct custom_operations owlgpu_buf_ops = {
    "owlgpu.buf",           owlgpu_buf_finalize,         custom_compare_default,
    custom_hash_default,    custom_serialize_default,    custom_deserialize_default,
    custom_compare_ext_default, custom_fixed_length_default};

/* ---- owlgpu.stream: a CUDA stream owned by the block (NULL: the legacy
 * default stream, not destroyed) ----------------------------------------- */

typedef struct {
  void *s;
} owlgpu_stream;

#define Stream_val(v) (((owlgpu_stream *)Data_custom_val(v))->s)

static void owlgpu_stream_finalize(value v) {
  owlgpu_stream *st = (owlgpu_stream *)Data_custom_val(v);
  if (st->s) owlgpu_stream_destroy(st->s);
  st->s = NULL;
}

static struct custom_operations owlgpu_stream_ops = {
    "owlgpu.stream",        owlgpu_stream_finalize,      custom_compare_default,
    custom_hash_default,    custom_serialize_default,    custom_deserialize_default,
    custom_compare_ext_default, custom_fixed_length_default};

static value alloc_stream(void *s) {
  value v = caml_alloc_custom(&owlgpu_stream_ops, sizeof(owlgpu_stream), 0, 1);
  ((owlgpu_stream *)Data_custom_val(v))->s = s;
  return v;
}

CAMLprim value owlgpu_dstub_stream_create(value unit) {
  void *s = NULL;
  (void)unit;
  if (owlgpu_stream_create(&s) != 0) caml_failwith(owlgpu_last_error());
  return alloc_stream(s);
}

CAMLprim value owlgpu_dstub_stream_default(value unit) {
  (void)unit;
  return alloc_stream(NULL);
}

CAMLprim value owlgpu_dstub_stream_sync(value vs) {
  void *s = Stream_val(vs);
  int rc;
  caml_enter_blocking_section();
  rc = owlgpu_stream_synchronize(s);
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}

/* buf_create bytes stream: uninitialised device memory, allocated in order
 * on `stream`. */
CAMLprim value owlgpu_dstub_buf_create(value vbytes, value vs) {
  CAMLparam2(vbytes, vs);
  CAMLlocal1(v);
  void *p = NULL;
  intnat n = Long_val(vbytes);
  if (n < 0) caml_failwith("owlgpu buf_create: negative size");
  if (owlgpu_device_alloc(&p, (uint64_t)n, Stream_val(vs)) != 0)
    caml_failwith(owlgpu_last_error());
  v = caml_alloc_custom(&owlgpu_buf_ops, sizeof(owlgpu_buf), 0, 1);
  Buf_val(v)->ptr = p;
  Buf_val(v)->bytes = (uint64_t)n;
  CAMLreturn(v);
}

CAMLprim value owlgpu_dstub_buf_bytes(value vb) { return Val_long((intnat)Buf_val(vb)->bytes); }

/* buf_free b: release now (the finaliser then has nothing to do); later
 * calls on b see a buffer of 0 bytes. */
CAMLprim value owlgpu_dstub_buf_free(value vb) {
  owlgpu_buf_finalize(vb);
  return Val_unit;
}

/* buf_upload b a stream / buf_download b a stream: copy the Bigarray's
 * bytes into / out of the buffer; they return when the bytes have arrived. */
static value copy_ba(value vb, value va, value vs, int to_device) {
  CAMLparam3(vb, va, vs);
  owlgpu_buf *b = Buf_val(vb);
  void *host = Caml_ba_data_val(va);
  uint64_t n = (uint64_t)caml_ba_byte_size(Caml_ba_array_val(va));
  void *dev = b->ptr, *s = Stream_val(vs);
  int rc;
  if (n > b->bytes) caml_failwith("owlgpu buf copy: the array is larger than the buffer");
  caml_enter_blocking_section();
  rc = to_device ? owlgpu_copy_to_device(dev, host, n, s) : owlgpu_copy_to_host(host, dev, n, s);
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}

CAMLprim value owlgpu_dstub_buf_upload(value vb, value va, value vs) {
  return copy_ba(vb, va, vs, 1);
}

CAMLprim value owlgpu_dstub_buf_download(value vb, value va, value vs) {
  return copy_ba(vb, va, vs, 0);
}

/* ---- device-resident entry points ------------------------------------ */

CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_float32_ndarray_conv_spatial((float *)Buf_ptr(v0), (float *)Buf_ptr(v1),
      (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6),
      Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_float64_ndarray_conv_spatial((double *)Buf_ptr(v0), (double *)Buf_ptr(v1),
      (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6),
      Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_backward_input_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  int rc = owlgpu_float32_ndarray_conv_spatial_backward_input((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_backward_input_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_spatial_backward_input_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_spatial_backward_input_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  int rc = owlgpu_float64_ndarray_conv_spatial_backward_input((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_spatial_backward_input_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_spatial_backward_input_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  int rc = owlgpu_float32_ndarray_conv_spatial_backward_kernel((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_spatial_backward_kernel_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  int rc = owlgpu_float64_ndarray_conv_spatial_backward_kernel((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_spatial_backward_kernel_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_spatial_backward_kernel_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_cuboid_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18, value v19, value v20) {
  int rc = owlgpu_float32_ndarray_conv_cuboid_im2col((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Long_val(v19), Stream_val(v20));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_cuboid_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18], argv[19],
      argv[20]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_cuboid_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18, value v19, value v20) {
  int rc = owlgpu_float64_ndarray_conv_cuboid_im2col((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19), Stream_val(v20));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_cuboid_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18], argv[19],
      argv[20]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19) {
  int rc = owlgpu_float32_ndarray_conv_cuboid_backward_input_im2col((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_cuboid_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17],
      argv[18], argv[19]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19) {
  int rc = owlgpu_float64_ndarray_conv_cuboid_backward_input_im2col((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_cuboid_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17],
      argv[18], argv[19]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19) {
  int rc = owlgpu_float32_ndarray_conv_cuboid_backward_kernel_im2col((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_cuboid_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17],
      argv[18], argv[19]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19) {
  int rc = owlgpu_float64_ndarray_conv_cuboid_backward_kernel_im2col((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_cuboid_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17],
      argv[18], argv[19]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_spatial_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18) {
  int rc = owlgpu_float32_ndarray_conv_dilated_spatial_im2col((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_spatial_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_dilated_spatial_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_spatial_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18) {
  int rc = owlgpu_float64_ndarray_conv_dilated_spatial_im2col((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_spatial_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_dilated_spatial_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  int rc = owlgpu_float32_ndarray_conv_dilated_spatial_backward_input_im2col(
      (float *)Buf_ptr(v0), (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  int rc = owlgpu_float64_ndarray_conv_dilated_spatial_backward_input_im2col(
      (double *)Buf_ptr(v0), (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  int rc = owlgpu_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col(
      (float *)Buf_ptr(v0), (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  int rc = owlgpu_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col(
      (double *)Buf_ptr(v0), (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19, value v20, value v21, value v22, value v23) {
  int rc = owlgpu_float32_ndarray_conv_dilated_cuboid_im2col((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Long_val(v19), Long_val(v20), Long_val(v21),
      Long_val(v22), Stream_val(v23));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20], argv[21], argv[22], argv[23]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19, value v20, value v21, value v22, value v23) {
  int rc = owlgpu_float64_ndarray_conv_dilated_cuboid_im2col((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19), Long_val(v20),
      Long_val(v21), Long_val(v22), Stream_val(v23));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20], argv[21], argv[22], argv[23]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_float32_ndarray_conv_dilated_cuboid_backward_input_im2col(
      (float *)Buf_ptr(v0), (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Long_val(v20), Long_val(v21), Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_float64_ndarray_conv_dilated_cuboid_backward_input_im2col(
      (double *)Buf_ptr(v0), (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Long_val(v20), Long_val(v21), Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
      (float *)Buf_ptr(v0), (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Long_val(v20), Long_val(v21), Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
      (double *)Buf_ptr(v0), (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Long_val(v20), Long_val(v21), Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float32_ndarray_maxpool_spatial((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_maxpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float64_ndarray_maxpool_spatial((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_maxpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_avgpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float32_ndarray_avgpool_spatial((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_avgpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_avgpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_avgpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float64_ndarray_avgpool_spatial((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_avgpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_avgpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float32_ndarray_maxpool_spatial_backward((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_maxpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float64_ndarray_maxpool_spatial_backward((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_maxpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_avgpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float32_ndarray_avgpool_spatial_backward((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_avgpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_avgpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_avgpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float64_ndarray_avgpool_spatial_backward((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_avgpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_avgpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_argmax_spatial_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float32_ndarray_maxpool_argmax_spatial((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (int64_t *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_argmax_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_maxpool_argmax_spatial_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_argmax_spatial_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_float64_ndarray_maxpool_argmax_spatial((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (int64_t *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_argmax_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_maxpool_argmax_spatial_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_float32_ndarray_maxpool_cuboid((float *)Buf_ptr(v0), (float *)Buf_ptr(v1),
      Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_cuboid_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_maxpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_float64_ndarray_maxpool_cuboid((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_cuboid_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_maxpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_avgpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_float32_ndarray_avgpool_cuboid((float *)Buf_ptr(v0), (float *)Buf_ptr(v1),
      Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_avgpool_cuboid_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_avgpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_avgpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_float64_ndarray_avgpool_cuboid((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_avgpool_cuboid_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_avgpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19) {
  int rc = owlgpu_float32_ndarray_maxpool_cuboid_backward((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_maxpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_maxpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19) {
  int rc = owlgpu_float64_ndarray_maxpool_cuboid_backward((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_maxpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_maxpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_avgpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19) {
  int rc = owlgpu_float32_ndarray_avgpool_cuboid_backward((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_avgpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_avgpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_avgpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19) {
  int rc = owlgpu_float64_ndarray_avgpool_cuboid_backward((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_avgpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_avgpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_upsampling_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11) {
  int rc = owlgpu_float32_ndarray_upsampling_spatial_backward((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_upsampling_spatial_backward_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_upsampling_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_upsampling_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11) {
  int rc = owlgpu_float64_ndarray_upsampling_spatial_backward((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_upsampling_spatial_backward_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_upsampling_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_upsampling_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11) {
  int rc = owlgpu_float32_ndarray_upsampling_spatial((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_upsampling_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_upsampling_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_upsampling_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11) {
  int rc = owlgpu_float64_ndarray_upsampling_spatial((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_upsampling_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_upsampling_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_complex32_ndarray_conv_spatial((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_complex64_ndarray_conv_spatial((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_spatial_backward_input_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  int rc = owlgpu_complex32_ndarray_conv_spatial_backward_input(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_spatial_backward_input_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_spatial_backward_input_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_spatial_backward_input_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  int rc = owlgpu_complex64_ndarray_conv_spatial_backward_input(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_spatial_backward_input_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_spatial_backward_input_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_spatial_backward_kernel_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  int rc = owlgpu_complex32_ndarray_conv_spatial_backward_kernel(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_spatial_backward_kernel_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_spatial_backward_kernel_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_spatial_backward_kernel_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  int rc = owlgpu_complex64_ndarray_conv_spatial_backward_kernel(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_spatial_backward_kernel_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_spatial_backward_kernel_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_cuboid_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18, value v19, value v20) {
  int rc = owlgpu_complex32_ndarray_conv_cuboid_im2col((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Stream_val(v20));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_cuboid_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18], argv[19],
      argv[20]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_cuboid_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18, value v19, value v20) {
  int rc = owlgpu_complex64_ndarray_conv_cuboid_im2col((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Stream_val(v20));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_cuboid_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18], argv[19],
      argv[20]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19) {
  int rc = owlgpu_complex32_ndarray_conv_cuboid_backward_input_im2col(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17],
      argv[18], argv[19]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19) {
  int rc = owlgpu_complex64_ndarray_conv_cuboid_backward_input_im2col(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17],
      argv[18], argv[19]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19) {
  int rc = owlgpu_complex32_ndarray_conv_cuboid_backward_kernel_im2col(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17],
      argv[18], argv[19]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19) {
  int rc = owlgpu_complex64_ndarray_conv_cuboid_backward_kernel_im2col(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17],
      argv[18], argv[19]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18) {
  int rc = owlgpu_complex32_ndarray_conv_dilated_spatial_im2col(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18) {
  int rc = owlgpu_complex64_ndarray_conv_dilated_spatial_im2col(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  int rc = owlgpu_complex32_ndarray_conv_dilated_spatial_backward_input_im2col(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  int rc = owlgpu_complex64_ndarray_conv_dilated_spatial_backward_input_im2col(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  int rc = owlgpu_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  int rc = owlgpu_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Stream_val(v17));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19, value v20, value v21, value v22, value v23) {
  int rc = owlgpu_complex32_ndarray_conv_dilated_cuboid_im2col(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Long_val(v19), Long_val(v20), Long_val(v21),
      Long_val(v22), Stream_val(v23));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20], argv[21], argv[22], argv[23]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19, value v20, value v21, value v22, value v23) {
  int rc = owlgpu_complex64_ndarray_conv_dilated_cuboid_im2col(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Long_val(v19), Long_val(v20), Long_val(v21),
      Long_val(v22), Stream_val(v23));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20], argv[21], argv[22], argv[23]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Long_val(v19), Long_val(v20), Long_val(v21),
      Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Long_val(v19), Long_val(v20), Long_val(v21),
      Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Long_val(v19), Long_val(v20), Long_val(v21),
      Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18), Long_val(v19), Long_val(v20), Long_val(v21),
      Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex32_ndarray_maxpool_spatial((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_maxpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex64_ndarray_maxpool_spatial((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_maxpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_avgpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex32_ndarray_avgpool_spatial((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_avgpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_avgpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_avgpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex64_ndarray_avgpool_spatial((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_avgpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_avgpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex32_ndarray_maxpool_spatial_backward(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_maxpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex64_ndarray_maxpool_spatial_backward(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_maxpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_avgpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex32_ndarray_avgpool_spatial_backward(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1),
      (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_avgpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_avgpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_avgpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex64_ndarray_avgpool_spatial_backward(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1),
      (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_avgpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_avgpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_argmax_spatial_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex32_ndarray_maxpool_argmax_spatial((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), (int64_t *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_argmax_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_maxpool_argmax_spatial_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_argmax_spatial_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  int rc = owlgpu_complex64_ndarray_maxpool_argmax_spatial((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), (int64_t *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_argmax_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_maxpool_argmax_spatial_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_complex32_ndarray_maxpool_cuboid((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_cuboid_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_maxpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_complex64_ndarray_maxpool_cuboid((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_cuboid_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_maxpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_avgpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_complex32_ndarray_avgpool_cuboid((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_avgpool_cuboid_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_avgpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_avgpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  int rc = owlgpu_complex64_ndarray_avgpool_cuboid((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Stream_val(v18));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_avgpool_cuboid_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_avgpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19) {
  int rc = owlgpu_complex32_ndarray_maxpool_cuboid_backward((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_maxpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_maxpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19) {
  int rc = owlgpu_complex64_ndarray_maxpool_cuboid_backward((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_maxpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_maxpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_avgpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19) {
  int rc = owlgpu_complex32_ndarray_avgpool_cuboid_backward((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), (owlgpu_complex32 *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_avgpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_avgpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_avgpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19) {
  int rc = owlgpu_complex64_ndarray_avgpool_cuboid_backward((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), (owlgpu_complex64 *)Buf_ptr(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Stream_val(v19));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_avgpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_avgpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_upsampling_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11) {
  int rc = owlgpu_complex32_ndarray_upsampling_spatial_backward(
      (owlgpu_complex32 *)Buf_ptr(v0), (owlgpu_complex32 *)Buf_ptr(v1), Long_val(v2),
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_upsampling_spatial_backward_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_upsampling_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_upsampling_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11) {
  int rc = owlgpu_complex64_ndarray_upsampling_spatial_backward(
      (owlgpu_complex64 *)Buf_ptr(v0), (owlgpu_complex64 *)Buf_ptr(v1), Long_val(v2),
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_upsampling_spatial_backward_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_upsampling_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11]);
}

CAMLprim value owlgpu_dstub_complex32_ndarray_upsampling_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11) {
  int rc = owlgpu_complex32_ndarray_upsampling_spatial((owlgpu_complex32 *)Buf_ptr(v0),
      (owlgpu_complex32 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex32_ndarray_upsampling_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex32_ndarray_upsampling_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11]);
}

CAMLprim value owlgpu_dstub_complex64_ndarray_upsampling_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11) {
  int rc = owlgpu_complex64_ndarray_upsampling_spatial((owlgpu_complex64 *)Buf_ptr(v0),
      (owlgpu_complex64 *)Buf_ptr(v1), Long_val(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_complex64_ndarray_upsampling_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_complex64_ndarray_upsampling_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_bias_act_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18, value v19, value v20) {
  int rc = owlgpu_float32_ndarray_conv_spatial_bias_act((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      (float *)(Is_block(v17) ? Buf_ptr(Field(v17, 0)) : NULL), Long_val(v18),
      Long_val(v19), Stream_val(v20));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_bias_act_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_spatial_bias_act_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_spatial_bias_act_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18, value v19, value v20) {
  int rc = owlgpu_float64_ndarray_conv_spatial_bias_act((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), (double *)(Is_block(v17) ? Buf_ptr(Field(v17, 0)) : NULL),
      Long_val(v18), Long_val(v19), Stream_val(v20));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_spatial_bias_act_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_spatial_bias_act_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20]);
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_cuboid_bias_act_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_float32_ndarray_conv_cuboid_bias_act((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16),
      Long_val(v17), Long_val(v18),
      (float *)(Is_block(v19) ? Buf_ptr(Field(v19, 0)) : NULL), Long_val(v20),
      Long_val(v21), Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_cuboid_bias_act_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_cuboid_bias_act_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18], argv[19],
      argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_float64_ndarray_conv_cuboid_bias_act_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18, value v19, value v20, value v21, value v22) {
  int rc = owlgpu_float64_ndarray_conv_cuboid_bias_act((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16), Long_val(v17), Long_val(v18),
      (double *)(Is_block(v19) ? Buf_ptr(Field(v19, 0)) : NULL), Long_val(v20),
      Long_val(v21), Stream_val(v22));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_ndarray_conv_cuboid_bias_act_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_dstub_float64_ndarray_conv_cuboid_bias_act_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18], argv[19],
      argv[20], argv[21], argv[22]);
}

CAMLprim value owlgpu_dstub_float32_bias_act_backward_native(value v0, value v1, value v2,
    value v3, value v4, value v5, value v6, value v7) {
  int rc = owlgpu_float32_bias_act_backward((float *)Buf_ptr(v0), (float *)Buf_ptr(v1),
      (float *)(Is_block(v2) ? Buf_ptr(Field(v2, 0)) : NULL),
      (float *)(Is_block(v3) ? Buf_ptr(Field(v3, 0)) : NULL), Long_val(v4), Long_val(v5),
      Long_val(v6), Stream_val(v7));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_bias_act_backward_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_bias_act_backward_native(argv[0], argv[1], argv[2], argv[3],
      argv[4], argv[5], argv[6], argv[7]);
}

CAMLprim value owlgpu_dstub_float64_bias_act_backward_native(value v0, value v1, value v2,
    value v3, value v4, value v5, value v6, value v7) {
  int rc = owlgpu_float64_bias_act_backward((double *)Buf_ptr(v0), (double *)Buf_ptr(v1),
      (double *)(Is_block(v2) ? Buf_ptr(Field(v2, 0)) : NULL),
      (double *)(Is_block(v3) ? Buf_ptr(Field(v3, 0)) : NULL), Long_val(v4), Long_val(v5),
      Long_val(v6), Stream_val(v7));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_bias_act_backward_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_bias_act_backward_native(argv[0], argv[1], argv[2], argv[3],
      argv[4], argv[5], argv[6], argv[7]);
}

CAMLprim value owlgpu_dstub_float32_dot_native(value v0, value v1, value v2, value v3,
    value v4, value v5, value v6, value v7, value v8, value v9, value v10, value v11) {
  int rc = owlgpu_float32_dot((float *)Buf_ptr(v0), (float *)Buf_ptr(v1),
      (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6),
      Long_val(v7), (float *)(Is_block(v8) ? Buf_ptr(Field(v8, 0)) : NULL), Long_val(v9),
      Long_val(v10), Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_dot_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_dot_native(argv[0], argv[1], argv[2], argv[3], argv[4],
      argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11]);
}

CAMLprim value owlgpu_dstub_float64_dot_native(value v0, value v1, value v2, value v3,
    value v4, value v5, value v6, value v7, value v8, value v9, value v10, value v11) {
  int rc = owlgpu_float64_dot((double *)Buf_ptr(v0), (double *)Buf_ptr(v1),
      (double *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6),
      Long_val(v7), (double *)(Is_block(v8) ? Buf_ptr(Field(v8, 0)) : NULL), Long_val(v9),
      Long_val(v10), Stream_val(v11));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_dot_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_dot_native(argv[0], argv[1], argv[2], argv[3], argv[4],
      argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11]);
}

CAMLprim value owlgpu_dstub_float32_softmax_cross_entropy_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7) {
  int rc = owlgpu_float32_softmax_cross_entropy((float *)Buf_ptr(v0), (float *)Buf_ptr(v1),
      (float *)(Is_block(v2) ? Buf_ptr(Field(v2, 0)) : NULL),
      (float *)(Is_block(v3) ? Buf_ptr(Field(v3, 0)) : NULL),
      (float *)(Is_block(v4) ? Buf_ptr(Field(v4, 0)) : NULL), Long_val(v5), Long_val(v6),
      Stream_val(v7));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_softmax_cross_entropy_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_softmax_cross_entropy_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7]);
}

CAMLprim value owlgpu_dstub_float64_softmax_cross_entropy_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7) {
  int rc = owlgpu_float64_softmax_cross_entropy((double *)Buf_ptr(v0),
      (double *)Buf_ptr(v1), (double *)(Is_block(v2) ? Buf_ptr(Field(v2, 0)) : NULL),
      (double *)(Is_block(v3) ? Buf_ptr(Field(v3, 0)) : NULL),
      (double *)(Is_block(v4) ? Buf_ptr(Field(v4, 0)) : NULL), Long_val(v5), Long_val(v6),
      Stream_val(v7));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float64_softmax_cross_entropy_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float64_softmax_cross_entropy_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7]);
}

CAMLprim value owlgpu_dstub_float32_sgd_update_native(value v0, value v1, value v2,
    value v3, value v4) {
  int rc = owlgpu_float32_sgd_update((float *)Buf_ptr(v0), (float *)Buf_ptr(v1),
      Long_val(v2), Double_val(v3), Stream_val(v4));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}

CAMLprim value owlgpu_dstub_float64_sgd_update_native(value v0, value v1, value v2,
    value v3, value v4) {
  int rc = owlgpu_float64_sgd_update((double *)Buf_ptr(v0), (double *)Buf_ptr(v1),
      Long_val(v2), Double_val(v3), Stream_val(v4));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}

CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_noalloc_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16) {
  int rc = owlgpu_float32_ndarray_conv_spatial_backward_kernel_noalloc((float *)Buf_ptr(v0),
      (float *)Buf_ptr(v1), (float *)Buf_ptr(v2), Long_val(v3), Long_val(v4), Long_val(v5),
      Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11),
      Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15), Stream_val(v16));
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}
CAMLprim value owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_noalloc_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_noalloc_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}
