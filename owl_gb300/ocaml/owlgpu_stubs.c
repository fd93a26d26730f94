/* owlgpu_stubs.c -- OCaml C stubs binding Owl's conv / pool / upsampling
 * externals to libowlgpu's host drop-in entry points (include/owlgpu.h).
 * Generated by make_stubs.py; link with -lowlgpu. */
#include <caml/bigarray.h>
#include <caml/fail.h>
#include <caml/memory.h>
#include <caml/mlvalues.h>
#include <caml/signals.h>
#include <stdint.h>

#include "owlgpu.h"

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_native(value v0, value v1, value v2,
    value v3, value v4, value v5, value v6, value v7, value v8, value v9, value v10,
    value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial(input, kernel, output, Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_native(argv[0], argv[1], argv[2], argv[3],
      argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11], argv[12],
      argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_native(value v0, value v1, value v2,
    value v3, value v4, value v5, value v6, value v7, value v8, value v9, value v10,
    value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial(input, kernel, output, Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_native(argv[0], argv[1], argv[2], argv[3],
      argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11], argv[12],
      argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_input_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_backward_input(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_input_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_backward_input_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_input_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_backward_input(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_input_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_backward_input_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel_grad = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_backward_kernel(input, kernel_grad, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel_grad = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_backward_kernel(input, kernel_grad, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel_grad = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel_grad = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_cuboid_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_cuboid_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_cuboid_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_cuboid_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_cuboid_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_cuboid_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel_grad = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_cuboid_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel_grad = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_cuboid_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_spatial_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_dilated_spatial_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_spatial_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_dilated_spatial_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_spatial_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_dilated_spatial_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_spatial_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_dilated_spatial_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_dilated_spatial_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_dilated_spatial_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel_grad = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel_grad = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_cuboid_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19, value v20, value v21) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_dilated_cuboid_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Long_val(v20), Long_val(v21));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_dilated_cuboid_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20], argv[21]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_cuboid_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19, value v20, value v21) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_dilated_cuboid_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Long_val(v20), Long_val(v21));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_dilated_cuboid_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20], argv[21]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20) {
  CAMLparam3(v0, v1, v2);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_dilated_cuboid_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Long_val(v18), Long_val(v19), Long_val(v20));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20) {
  CAMLparam3(v0, v1, v2);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_dilated_cuboid_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Long_val(v18), Long_val(v19), Long_val(v20));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel_grad = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Long_val(v18), Long_val(v19), Long_val(v20));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel_grad = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Long_val(v18), Long_val(v19), Long_val(v20));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20]);
}

CAMLprim value owlgpu_stub_float32_ndarray_maxpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam2(v0, v1);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output = (float *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_maxpool_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_maxpool_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_maxpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float64_ndarray_maxpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam2(v0, v1);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output = (double *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_maxpool_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_maxpool_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_maxpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float32_ndarray_avgpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam2(v0, v1);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output = (float *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_avgpool_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_avgpool_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_avgpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float64_ndarray_avgpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam2(v0, v1);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output = (double *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_avgpool_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_avgpool_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_avgpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float32_ndarray_maxpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output_grad = (float *)Caml_ba_data_val(v1);
  float *input_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_maxpool_spatial_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_maxpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_maxpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float64_ndarray_maxpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output_grad = (double *)Caml_ba_data_val(v1);
  double *input_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_maxpool_spatial_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_maxpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_maxpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float32_ndarray_avgpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output_grad = (float *)Caml_ba_data_val(v1);
  float *input_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_avgpool_spatial_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_avgpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_avgpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float64_ndarray_avgpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output_grad = (double *)Caml_ba_data_val(v1);
  double *input_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_avgpool_spatial_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_avgpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_avgpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float32_ndarray_maxpool_argmax_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output = (float *)Caml_ba_data_val(v1);
  int64_t *argmax = (int64_t *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_maxpool_argmax_spatial(input, output, argmax, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_maxpool_argmax_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_maxpool_argmax_spatial_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float64_ndarray_maxpool_argmax_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output = (double *)Caml_ba_data_val(v1);
  int64_t *argmax = (int64_t *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_maxpool_argmax_spatial(input, output, argmax, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_maxpool_argmax_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_maxpool_argmax_spatial_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_float32_ndarray_maxpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam2(v0, v1);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output = (float *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_maxpool_cuboid(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_maxpool_cuboid_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_maxpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float64_ndarray_maxpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam2(v0, v1);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output = (double *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_maxpool_cuboid(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_maxpool_cuboid_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_maxpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float32_ndarray_avgpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam2(v0, v1);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output = (float *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_avgpool_cuboid(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_avgpool_cuboid_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_avgpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float64_ndarray_avgpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam2(v0, v1);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output = (double *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_avgpool_cuboid(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_avgpool_cuboid_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_avgpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float32_ndarray_maxpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output_grad = (float *)Caml_ba_data_val(v1);
  float *input_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_maxpool_cuboid_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_maxpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_maxpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float64_ndarray_maxpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output_grad = (double *)Caml_ba_data_val(v1);
  double *input_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_maxpool_cuboid_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_maxpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_maxpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float32_ndarray_avgpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output_grad = (float *)Caml_ba_data_val(v1);
  float *input_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_avgpool_cuboid_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_avgpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_avgpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float64_ndarray_avgpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output_grad = (double *)Caml_ba_data_val(v1);
  double *input_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_avgpool_cuboid_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_avgpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_avgpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float32_ndarray_upsampling_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9) {
  CAMLparam2(v0, v1);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *output_grad = (float *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_upsampling_spatial_backward(input_grad, output_grad,
      Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_upsampling_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_upsampling_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9]);
}

CAMLprim value owlgpu_stub_float64_ndarray_upsampling_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9) {
  CAMLparam2(v0, v1);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *output_grad = (double *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_upsampling_spatial_backward(input_grad, output_grad,
      Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_upsampling_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_upsampling_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9]);
}

CAMLprim value owlgpu_stub_float32_ndarray_upsampling_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9) {
  CAMLparam2(v0, v1);
  float *input = (float *)Caml_ba_data_val(v0);
  float *output = (float *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_upsampling_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_upsampling_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_upsampling_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9]);
}

CAMLprim value owlgpu_stub_float64_ndarray_upsampling_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9) {
  CAMLparam2(v0, v1);
  double *input = (double *)Caml_ba_data_val(v0);
  double *output = (double *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_upsampling_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_upsampling_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_upsampling_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial(input, kernel, output, Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial(input, kernel, output, Long_val(v3), Long_val(v4),
      Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9), Long_val(v10),
      Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14), Long_val(v15),
      Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_backward_input(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_backward_input(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_backward_kernel(input, kernel_grad, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_backward_kernel(input, kernel_grad, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_cuboid_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_cuboid_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_im2col_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_cuboid_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_im2col_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_cuboid_im2col_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_cuboid_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_cuboid_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_cuboid_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_cuboid_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_spatial_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_dilated_spatial_im2col(input, kernel, output,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_spatial_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_dilated_spatial_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_spatial_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_dilated_spatial_im2col(input, kernel, output,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_spatial_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_dilated_spatial_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_dilated_spatial_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_dilated_spatial_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19, value v20, value v21) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_dilated_cuboid_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Long_val(v20), Long_val(v21));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20], argv[21]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_im2col_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17, value v18, value v19, value v20, value v21) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_dilated_cuboid_im2col(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18), Long_val(v19),
      Long_val(v20), Long_val(v21));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_im2col_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18],
      argv[19], argv[20], argv[21]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Long_val(v18), Long_val(v19), Long_val(v20));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Long_val(v18), Long_val(v19), Long_val(v20));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Long_val(v18), Long_val(v19), Long_val(v20));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17, value v18, value v19, value v20) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17),
      Long_val(v18), Long_val(v19), Long_val(v20));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native(
      argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8],
      argv[9], argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16],
      argv[17], argv[18], argv[19], argv[20]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam2(v0, v1);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_maxpool_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_maxpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam2(v0, v1);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_maxpool_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_maxpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_avgpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam2(v0, v1);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_avgpool_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_avgpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_avgpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_avgpool_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14) {
  CAMLparam2(v0, v1);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_avgpool_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_avgpool_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_avgpool_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_maxpool_spatial_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_maxpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_maxpool_spatial_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_maxpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_avgpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_avgpool_spatial_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_avgpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_avgpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_avgpool_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_avgpool_spatial_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_avgpool_spatial_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_avgpool_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_argmax_spatial_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  int64_t *argmax = (int64_t *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_maxpool_argmax_spatial(input, output, argmax, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_argmax_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_maxpool_argmax_spatial_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_argmax_spatial_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  int64_t *argmax = (int64_t *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_maxpool_argmax_spatial(input, output, argmax, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_argmax_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_maxpool_argmax_spatial_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam2(v0, v1);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_maxpool_cuboid(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_cuboid_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_maxpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam2(v0, v1);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_maxpool_cuboid(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_cuboid_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_maxpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_avgpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam2(v0, v1);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_avgpool_cuboid(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_avgpool_cuboid_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_avgpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_avgpool_cuboid_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam2(v0, v1);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_avgpool_cuboid(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_avgpool_cuboid_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_avgpool_cuboid_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_maxpool_cuboid_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_maxpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_maxpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_maxpool_cuboid_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_maxpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_maxpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_avgpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_avgpool_cuboid_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_avgpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_avgpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_avgpool_cuboid_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_avgpool_cuboid_backward(input, output_grad, input_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_avgpool_cuboid_backward_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_avgpool_cuboid_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_upsampling_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9) {
  CAMLparam2(v0, v1);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_upsampling_spatial_backward(input_grad, output_grad,
      Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_upsampling_spatial_backward_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_upsampling_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_upsampling_spatial_backward_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9) {
  CAMLparam2(v0, v1);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_upsampling_spatial_backward(input_grad, output_grad,
      Long_val(v2), Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_upsampling_spatial_backward_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_upsampling_spatial_backward_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_upsampling_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9) {
  CAMLparam2(v0, v1);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_upsampling_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_upsampling_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_upsampling_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_upsampling_spatial_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9) {
  CAMLparam2(v0, v1);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_upsampling_spatial(input, output, Long_val(v2), Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_upsampling_spatial_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_upsampling_spatial_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_mec_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_mec(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_mec_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_mec_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_input_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_backward_input_mec(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_input_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_backward_input_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel_grad = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_backward_kernel_mec(input, kernel_grad, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_mec_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_cuboid_mec(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_mec_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_cuboid_mec_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_cuboid_backward_input_mec(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_mec_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel_grad = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_cuboid_backward_kernel_mec(input, kernel_grad, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_mec_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_mec(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_mec_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_mec_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_input_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_backward_input_mec(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_input_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_backward_input_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel_grad = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_backward_kernel_mec(input, kernel_grad, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_mec_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_cuboid_mec(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_mec_bytecode(value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_cuboid_mec_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_cuboid_backward_input_mec(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_mec_native(argv[0], argv[1],
      argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10],
      argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel_grad = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_cuboid_backward_kernel_mec(input, kernel_grad, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_mec_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_mec(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_mec_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_mec_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_mec_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_backward_input_mec(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_mec_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_backward_kernel_mec(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_mec_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_cuboid_mec(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_mec_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_cuboid_mec_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_cuboid_backward_input_mec(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_mec_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_cuboid_backward_kernel_mec(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_mec_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_mec(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_mec_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_mec_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_mec_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_backward_input_mec(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_mec_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_backward_kernel_mec(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_mec_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_cuboid_mec(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_mec_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_cuboid_mec_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_mec_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_cuboid_backward_input_mec(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_mec_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_cuboid_backward_kernel_mec(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_mec_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_mec_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_naive_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_naive(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_naive_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_naive_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_input_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_backward_input_naive(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_input_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_backward_input_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel_grad = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_spatial_backward_kernel_naive(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_naive_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_cuboid_naive(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_naive_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_cuboid_naive_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_naive_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  float *input_grad = (float *)Caml_ba_data_val(v0);
  float *kernel = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_cuboid_backward_input_naive(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  float *input = (float *)Caml_ba_data_val(v0);
  float *kernel_grad = (float *)Caml_ba_data_val(v1);
  float *output_grad = (float *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float32_ndarray_conv_cuboid_backward_kernel_naive(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_naive_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_naive(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_naive_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_naive_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_input_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_backward_input_naive(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_input_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_backward_input_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel_grad = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_spatial_backward_kernel_naive(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_naive_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_cuboid_naive(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_naive_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_cuboid_naive_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_naive_native(value v0,
    value v1, value v2, value v3, value v4, value v5, value v6, value v7, value v8,
    value v9, value v10, value v11, value v12, value v13, value v14, value v15, value v16,
    value v17) {
  CAMLparam3(v0, v1, v2);
  double *input_grad = (double *)Caml_ba_data_val(v0);
  double *kernel = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_cuboid_backward_input_naive(input_grad, kernel, output_grad,
      Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8),
      Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13),
      Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  double *input = (double *)Caml_ba_data_val(v0);
  double *kernel_grad = (double *)Caml_ba_data_val(v1);
  double *output_grad = (double *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_float64_ndarray_conv_cuboid_backward_kernel_naive(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_naive_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_naive(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_naive_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_naive_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_backward_input_naive(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_spatial_backward_kernel_naive(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_naive_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_cuboid_naive(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_naive_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_cuboid_naive_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input_grad = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_cuboid_backward_input_naive(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex32 *input = (owlgpu_complex32 *)Caml_ba_data_val(v0);
  owlgpu_complex32 *kernel_grad = (owlgpu_complex32 *)Caml_ba_data_val(v1);
  owlgpu_complex32 *output_grad = (owlgpu_complex32 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex32_ndarray_conv_cuboid_backward_kernel_naive(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_naive_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_naive(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_naive_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_naive_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_backward_input_naive(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_spatial_backward_kernel_naive(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_naive_native(value v0, value v1,
    value v2, value v3, value v4, value v5, value v6, value v7, value v8, value v9,
    value v10, value v11, value v12, value v13, value v14, value v15, value v16, value v17,
    value v18) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_cuboid_naive(input, kernel, output, Long_val(v3),
      Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7), Long_val(v8), Long_val(v9),
      Long_val(v10), Long_val(v11), Long_val(v12), Long_val(v13), Long_val(v14),
      Long_val(v15), Long_val(v16), Long_val(v17), Long_val(v18));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_naive_bytecode(value *argv,
    int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_cuboid_naive_native(argv[0], argv[1], argv[2],
      argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9], argv[10], argv[11],
      argv[12], argv[13], argv[14], argv[15], argv[16], argv[17], argv[18]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input_grad = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_cuboid_backward_input_naive(input_grad, kernel,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}

CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_naive_native(
    value v0, value v1, value v2, value v3, value v4, value v5, value v6, value v7,
    value v8, value v9, value v10, value v11, value v12, value v13, value v14, value v15,
    value v16, value v17) {
  CAMLparam3(v0, v1, v2);
  owlgpu_complex64 *input = (owlgpu_complex64 *)Caml_ba_data_val(v0);
  owlgpu_complex64 *kernel_grad = (owlgpu_complex64 *)Caml_ba_data_val(v1);
  owlgpu_complex64 *output_grad = (owlgpu_complex64 *)Caml_ba_data_val(v2);
  int rc;
  caml_enter_blocking_section();
  rc = owl_complex64_ndarray_conv_cuboid_backward_kernel_naive(input, kernel_grad,
      output_grad, Long_val(v3), Long_val(v4), Long_val(v5), Long_val(v6), Long_val(v7),
      Long_val(v8), Long_val(v9), Long_val(v10), Long_val(v11), Long_val(v12),
      Long_val(v13), Long_val(v14), Long_val(v15), Long_val(v16), Long_val(v17));
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}
CAMLprim value owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_naive_bytecode(
    value *argv, int argn) {
  (void)argn;
  return owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_naive_native(argv[0],
      argv[1], argv[2], argv[3], argv[4], argv[5], argv[6], argv[7], argv[8], argv[9],
      argv[10], argv[11], argv[12], argv[13], argv[14], argv[15], argv[16], argv[17]);
}
