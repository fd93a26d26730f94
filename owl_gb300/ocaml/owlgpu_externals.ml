(* owlgpu_externals.ml -- Owl's conv / pool / upsampling externals bound to
   libowlgpu through owlgpu_stubs.c.  Generated by make_stubs.py. *)

open Owl_core_types

external owl_float32_ndarray_conv_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_native"

external owl_float64_ndarray_conv_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_native"

external owl_float32_ndarray_conv_spatial_backward_input
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_backward_input_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_backward_input_native"

external owl_float64_ndarray_conv_spatial_backward_input
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_backward_input_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_backward_input_native"

external owl_float32_ndarray_conv_spatial_backward_kernel
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_native"

external owl_float64_ndarray_conv_spatial_backward_kernel
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_native"

external owl_float32_ndarray_conv_spatial_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_im2col_native"

external owl_float64_ndarray_conv_spatial_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_im2col_native"

external owl_float32_ndarray_conv_spatial_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_backward_input_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_backward_input_im2col_native"

external owl_float64_ndarray_conv_spatial_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_backward_input_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_backward_input_im2col_native"

external owl_float32_ndarray_conv_spatial_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_im2col_native"

external owl_float64_ndarray_conv_spatial_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_im2col_native"

external owl_float32_ndarray_conv_cuboid_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_cuboid_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_cuboid_im2col_native"

external owl_float64_ndarray_conv_cuboid_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_cuboid_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_cuboid_im2col_native"

external owl_float32_ndarray_conv_cuboid_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_im2col_native"

external owl_float64_ndarray_conv_cuboid_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_im2col_native"

external owl_float32_ndarray_conv_cuboid_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_im2col_native"

external owl_float64_ndarray_conv_cuboid_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_im2col_native"

external owl_float32_ndarray_conv_dilated_spatial_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_dilated_spatial_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_dilated_spatial_im2col_native"

external owl_float64_ndarray_conv_dilated_spatial_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_dilated_spatial_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_dilated_spatial_im2col_native"

external owl_float32_ndarray_conv_dilated_spatial_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_native"

external owl_float64_ndarray_conv_dilated_spatial_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_native"

external owl_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native"

external owl_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native"

external owl_float32_ndarray_conv_dilated_cuboid_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_dilated_cuboid_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_dilated_cuboid_im2col_native"

external owl_float64_ndarray_conv_dilated_cuboid_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_dilated_cuboid_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_dilated_cuboid_im2col_native"

external owl_float32_ndarray_conv_dilated_cuboid_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_native"

external owl_float64_ndarray_conv_dilated_cuboid_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_native"

external owl_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_stub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native"

external owl_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_stub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native"

external owl_float32_ndarray_maxpool_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_maxpool_spatial_bytecode"
    "owlgpu_stub_float32_ndarray_maxpool_spatial_native"

external owl_float64_ndarray_maxpool_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_maxpool_spatial_bytecode"
    "owlgpu_stub_float64_ndarray_maxpool_spatial_native"

external owl_float32_ndarray_avgpool_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_avgpool_spatial_bytecode"
    "owlgpu_stub_float32_ndarray_avgpool_spatial_native"

external owl_float64_ndarray_avgpool_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_avgpool_spatial_bytecode"
    "owlgpu_stub_float64_ndarray_avgpool_spatial_native"

external owl_float32_ndarray_maxpool_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_maxpool_spatial_backward_bytecode"
    "owlgpu_stub_float32_ndarray_maxpool_spatial_backward_native"

external owl_float64_ndarray_maxpool_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_maxpool_spatial_backward_bytecode"
    "owlgpu_stub_float64_ndarray_maxpool_spatial_backward_native"

external owl_float32_ndarray_avgpool_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_avgpool_spatial_backward_bytecode"
    "owlgpu_stub_float32_ndarray_avgpool_spatial_backward_native"

external owl_float64_ndarray_avgpool_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_avgpool_spatial_backward_bytecode"
    "owlgpu_stub_float64_ndarray_avgpool_spatial_backward_native"

external owl_float32_ndarray_maxpool_argmax_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> (int64, Bigarray.int64_elt) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_maxpool_argmax_spatial_bytecode"
    "owlgpu_stub_float32_ndarray_maxpool_argmax_spatial_native"

external owl_float64_ndarray_maxpool_argmax_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> (int64, Bigarray.int64_elt) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_maxpool_argmax_spatial_bytecode"
    "owlgpu_stub_float64_ndarray_maxpool_argmax_spatial_native"

external owl_float32_ndarray_maxpool_cuboid
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_maxpool_cuboid_bytecode"
    "owlgpu_stub_float32_ndarray_maxpool_cuboid_native"

external owl_float64_ndarray_maxpool_cuboid
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_maxpool_cuboid_bytecode"
    "owlgpu_stub_float64_ndarray_maxpool_cuboid_native"

external owl_float32_ndarray_avgpool_cuboid
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_avgpool_cuboid_bytecode"
    "owlgpu_stub_float32_ndarray_avgpool_cuboid_native"

external owl_float64_ndarray_avgpool_cuboid
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_avgpool_cuboid_bytecode"
    "owlgpu_stub_float64_ndarray_avgpool_cuboid_native"

external owl_float32_ndarray_maxpool_cuboid_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_maxpool_cuboid_backward_bytecode"
    "owlgpu_stub_float32_ndarray_maxpool_cuboid_backward_native"

external owl_float64_ndarray_maxpool_cuboid_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_maxpool_cuboid_backward_bytecode"
    "owlgpu_stub_float64_ndarray_maxpool_cuboid_backward_native"

external owl_float32_ndarray_avgpool_cuboid_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_avgpool_cuboid_backward_bytecode"
    "owlgpu_stub_float32_ndarray_avgpool_cuboid_backward_native"

external owl_float64_ndarray_avgpool_cuboid_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_avgpool_cuboid_backward_bytecode"
    "owlgpu_stub_float64_ndarray_avgpool_cuboid_backward_native"

external owl_float32_ndarray_upsampling_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_upsampling_spatial_backward_bytecode"
    "owlgpu_stub_float32_ndarray_upsampling_spatial_backward_native"

external owl_float64_ndarray_upsampling_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_upsampling_spatial_backward_bytecode"
    "owlgpu_stub_float64_ndarray_upsampling_spatial_backward_native"

external owl_float32_ndarray_upsampling_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_upsampling_spatial_bytecode"
    "owlgpu_stub_float32_ndarray_upsampling_spatial_native"

external owl_float64_ndarray_upsampling_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_upsampling_spatial_bytecode"
    "owlgpu_stub_float64_ndarray_upsampling_spatial_native"

external owl_complex32_ndarray_conv_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_native"

external owl_complex64_ndarray_conv_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_native"

external owl_complex32_ndarray_conv_spatial_backward_input
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_native"

external owl_complex64_ndarray_conv_spatial_backward_input
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_native"

external owl_complex32_ndarray_conv_spatial_backward_kernel
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_native"

external owl_complex64_ndarray_conv_spatial_backward_kernel
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_native"

external owl_complex32_ndarray_conv_spatial_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_im2col_native"

external owl_complex64_ndarray_conv_spatial_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_im2col_native"

external owl_complex32_ndarray_conv_spatial_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_im2col_native"

external owl_complex64_ndarray_conv_spatial_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_im2col_native"

external owl_complex32_ndarray_conv_spatial_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_im2col_native"

external owl_complex64_ndarray_conv_spatial_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_im2col_native"

external owl_complex32_ndarray_conv_cuboid_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_cuboid_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_cuboid_im2col_native"

external owl_complex64_ndarray_conv_cuboid_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_cuboid_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_cuboid_im2col_native"

external owl_complex32_ndarray_conv_cuboid_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_im2col_native"

external owl_complex64_ndarray_conv_cuboid_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_im2col_native"

external owl_complex32_ndarray_conv_cuboid_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_native"

external owl_complex64_ndarray_conv_cuboid_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_native"

external owl_complex32_ndarray_conv_dilated_spatial_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_dilated_spatial_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_dilated_spatial_im2col_native"

external owl_complex64_ndarray_conv_dilated_spatial_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_dilated_spatial_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_dilated_spatial_im2col_native"

external owl_complex32_ndarray_conv_dilated_spatial_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_native"

external owl_complex64_ndarray_conv_dilated_spatial_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_native"

external owl_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native"

external owl_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native"

external owl_complex32_ndarray_conv_dilated_cuboid_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_im2col_native"

external owl_complex64_ndarray_conv_dilated_cuboid_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_im2col_native"

external owl_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_native"

external owl_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_native"

external owl_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native"

external owl_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native"

external owl_complex32_ndarray_maxpool_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_maxpool_spatial_bytecode"
    "owlgpu_stub_complex32_ndarray_maxpool_spatial_native"

external owl_complex64_ndarray_maxpool_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_maxpool_spatial_bytecode"
    "owlgpu_stub_complex64_ndarray_maxpool_spatial_native"

external owl_complex32_ndarray_avgpool_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_avgpool_spatial_bytecode"
    "owlgpu_stub_complex32_ndarray_avgpool_spatial_native"

external owl_complex64_ndarray_avgpool_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_avgpool_spatial_bytecode"
    "owlgpu_stub_complex64_ndarray_avgpool_spatial_native"

external owl_complex32_ndarray_maxpool_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_maxpool_spatial_backward_bytecode"
    "owlgpu_stub_complex32_ndarray_maxpool_spatial_backward_native"

external owl_complex64_ndarray_maxpool_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_maxpool_spatial_backward_bytecode"
    "owlgpu_stub_complex64_ndarray_maxpool_spatial_backward_native"

external owl_complex32_ndarray_avgpool_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_avgpool_spatial_backward_bytecode"
    "owlgpu_stub_complex32_ndarray_avgpool_spatial_backward_native"

external owl_complex64_ndarray_avgpool_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_avgpool_spatial_backward_bytecode"
    "owlgpu_stub_complex64_ndarray_avgpool_spatial_backward_native"

external owl_complex32_ndarray_maxpool_argmax_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> (int64, Bigarray.int64_elt) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_maxpool_argmax_spatial_bytecode"
    "owlgpu_stub_complex32_ndarray_maxpool_argmax_spatial_native"

external owl_complex64_ndarray_maxpool_argmax_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> (int64, Bigarray.int64_elt) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_maxpool_argmax_spatial_bytecode"
    "owlgpu_stub_complex64_ndarray_maxpool_argmax_spatial_native"

external owl_complex32_ndarray_maxpool_cuboid
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_maxpool_cuboid_bytecode"
    "owlgpu_stub_complex32_ndarray_maxpool_cuboid_native"

external owl_complex64_ndarray_maxpool_cuboid
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_maxpool_cuboid_bytecode"
    "owlgpu_stub_complex64_ndarray_maxpool_cuboid_native"

external owl_complex32_ndarray_avgpool_cuboid
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_avgpool_cuboid_bytecode"
    "owlgpu_stub_complex32_ndarray_avgpool_cuboid_native"

external owl_complex64_ndarray_avgpool_cuboid
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_avgpool_cuboid_bytecode"
    "owlgpu_stub_complex64_ndarray_avgpool_cuboid_native"

external owl_complex32_ndarray_maxpool_cuboid_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_maxpool_cuboid_backward_bytecode"
    "owlgpu_stub_complex32_ndarray_maxpool_cuboid_backward_native"

external owl_complex64_ndarray_maxpool_cuboid_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_maxpool_cuboid_backward_bytecode"
    "owlgpu_stub_complex64_ndarray_maxpool_cuboid_backward_native"

external owl_complex32_ndarray_avgpool_cuboid_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_avgpool_cuboid_backward_bytecode"
    "owlgpu_stub_complex32_ndarray_avgpool_cuboid_backward_native"

external owl_complex64_ndarray_avgpool_cuboid_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_avgpool_cuboid_backward_bytecode"
    "owlgpu_stub_complex64_ndarray_avgpool_cuboid_backward_native"

external owl_complex32_ndarray_upsampling_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_upsampling_spatial_backward_bytecode"
    "owlgpu_stub_complex32_ndarray_upsampling_spatial_backward_native"

external owl_complex64_ndarray_upsampling_spatial_backward
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_upsampling_spatial_backward_bytecode"
    "owlgpu_stub_complex64_ndarray_upsampling_spatial_backward_native"

external owl_complex32_ndarray_upsampling_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_upsampling_spatial_bytecode"
    "owlgpu_stub_complex32_ndarray_upsampling_spatial_native"

external owl_complex64_ndarray_upsampling_spatial
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_upsampling_spatial_bytecode"
    "owlgpu_stub_complex64_ndarray_upsampling_spatial_native"

external owl_float32_ndarray_conv_spatial_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_mec_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_mec_native"

external owl_float32_ndarray_conv_spatial_backward_input_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_backward_input_mec_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_backward_input_mec_native"

external owl_float32_ndarray_conv_spatial_backward_kernel_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_mec_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_mec_native"

external owl_float32_ndarray_conv_cuboid_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_cuboid_mec_bytecode"
    "owlgpu_stub_float32_ndarray_conv_cuboid_mec_native"

external owl_float32_ndarray_conv_cuboid_backward_input_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_mec_bytecode"
    "owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_mec_native"

external owl_float32_ndarray_conv_cuboid_backward_kernel_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_mec_bytecode"
    "owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_mec_native"

external owl_float64_ndarray_conv_spatial_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_mec_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_mec_native"

external owl_float64_ndarray_conv_spatial_backward_input_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_backward_input_mec_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_backward_input_mec_native"

external owl_float64_ndarray_conv_spatial_backward_kernel_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_mec_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_mec_native"

external owl_float64_ndarray_conv_cuboid_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_cuboid_mec_bytecode"
    "owlgpu_stub_float64_ndarray_conv_cuboid_mec_native"

external owl_float64_ndarray_conv_cuboid_backward_input_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_mec_bytecode"
    "owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_mec_native"

external owl_float64_ndarray_conv_cuboid_backward_kernel_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_mec_bytecode"
    "owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_mec_native"

external owl_complex32_ndarray_conv_spatial_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_mec_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_mec_native"

external owl_complex32_ndarray_conv_spatial_backward_input_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_mec_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_mec_native"

external owl_complex32_ndarray_conv_spatial_backward_kernel_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_mec_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_mec_native"

external owl_complex32_ndarray_conv_cuboid_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_cuboid_mec_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_cuboid_mec_native"

external owl_complex32_ndarray_conv_cuboid_backward_input_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_mec_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_mec_native"

external owl_complex32_ndarray_conv_cuboid_backward_kernel_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_mec_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_mec_native"

external owl_complex64_ndarray_conv_spatial_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_mec_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_mec_native"

external owl_complex64_ndarray_conv_spatial_backward_input_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_mec_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_mec_native"

external owl_complex64_ndarray_conv_spatial_backward_kernel_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_mec_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_mec_native"

external owl_complex64_ndarray_conv_cuboid_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_cuboid_mec_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_cuboid_mec_native"

external owl_complex64_ndarray_conv_cuboid_backward_input_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_mec_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_mec_native"

external owl_complex64_ndarray_conv_cuboid_backward_kernel_mec
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_mec_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_mec_native"

external owl_float32_ndarray_conv_spatial_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_naive_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_naive_native"

external owl_float32_ndarray_conv_spatial_backward_input_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_backward_input_naive_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_backward_input_naive_native"

external owl_float32_ndarray_conv_spatial_backward_kernel_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_naive_bytecode"
    "owlgpu_stub_float32_ndarray_conv_spatial_backward_kernel_naive_native"

external owl_float32_ndarray_conv_cuboid_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_cuboid_naive_bytecode"
    "owlgpu_stub_float32_ndarray_conv_cuboid_naive_native"

external owl_float32_ndarray_conv_cuboid_backward_input_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_naive_bytecode"
    "owlgpu_stub_float32_ndarray_conv_cuboid_backward_input_naive_native"

external owl_float32_ndarray_conv_cuboid_backward_kernel_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_naive_bytecode"
    "owlgpu_stub_float32_ndarray_conv_cuboid_backward_kernel_naive_native"

external owl_float64_ndarray_conv_spatial_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_naive_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_naive_native"

external owl_float64_ndarray_conv_spatial_backward_input_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_backward_input_naive_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_backward_input_naive_native"

external owl_float64_ndarray_conv_spatial_backward_kernel_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_naive_bytecode"
    "owlgpu_stub_float64_ndarray_conv_spatial_backward_kernel_naive_native"

external owl_float64_ndarray_conv_cuboid_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_cuboid_naive_bytecode"
    "owlgpu_stub_float64_ndarray_conv_cuboid_naive_native"

external owl_float64_ndarray_conv_cuboid_backward_input_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_naive_bytecode"
    "owlgpu_stub_float64_ndarray_conv_cuboid_backward_input_naive_native"

external owl_float64_ndarray_conv_cuboid_backward_kernel_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_naive_bytecode"
    "owlgpu_stub_float64_ndarray_conv_cuboid_backward_kernel_naive_native"

external owl_complex32_ndarray_conv_spatial_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_naive_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_naive_native"

external owl_complex32_ndarray_conv_spatial_backward_input_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_naive_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_backward_input_naive_native"

external owl_complex32_ndarray_conv_spatial_backward_kernel_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_naive_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_spatial_backward_kernel_naive_native"

external owl_complex32_ndarray_conv_cuboid_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_cuboid_naive_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_cuboid_naive_native"

external owl_complex32_ndarray_conv_cuboid_backward_input_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_naive_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_input_naive_native"

external owl_complex32_ndarray_conv_cuboid_backward_kernel_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_naive_bytecode"
    "owlgpu_stub_complex32_ndarray_conv_cuboid_backward_kernel_naive_native"

external owl_complex64_ndarray_conv_spatial_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_naive_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_naive_native"

external owl_complex64_ndarray_conv_spatial_backward_input_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_naive_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_backward_input_naive_native"

external owl_complex64_ndarray_conv_spatial_backward_kernel_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_naive_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_spatial_backward_kernel_naive_native"

external owl_complex64_ndarray_conv_cuboid_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_cuboid_naive_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_cuboid_naive_native"

external owl_complex64_ndarray_conv_cuboid_backward_input_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_naive_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_input_naive_native"

external owl_complex64_ndarray_conv_cuboid_backward_kernel_naive
  :  ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> ('a, 'b) owl_arr
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> unit
  = "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_naive_bytecode"
    "owlgpu_stub_complex64_ndarray_conv_cuboid_backward_kernel_naive_native"
