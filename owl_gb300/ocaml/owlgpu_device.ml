(* owlgpu_device.ml -- device-resident Owl arrays for OCaml: libowlgpu's
   device-resident entry points over GPU buffers held in custom blocks.
   Generated by make_stubs.py.

   A [buf] is device memory, freed by its finaliser (or [buf_free]) after
   all earlier work on every stream.  A [stream] orders the calls made on
   it; the entry points only enqueue work, [stream_sync] waits for it.
   Shapes, strides and padding follow Owl's stub arguments, as for the host
   externals; each buffer must hold the bytes its argument covers. *)

type buf
type stream

external stream_create : unit -> stream = "owlgpu_dstub_stream_create"
external stream_default : unit -> stream = "owlgpu_dstub_stream_default"
external stream_sync : stream -> unit = "owlgpu_dstub_stream_sync"
external buf_create : int -> stream -> buf = "owlgpu_dstub_buf_create"
external buf_bytes : buf -> int = "owlgpu_dstub_buf_bytes"
external buf_free : buf -> unit = "owlgpu_dstub_buf_free"
external buf_upload
  :  buf -> ('a, 'b, Bigarray.c_layout) Bigarray.Genarray.t -> stream -> unit
  = "owlgpu_dstub_buf_upload"
external buf_download
  :  buf -> ('a, 'b, Bigarray.c_layout) Bigarray.Genarray.t -> stream -> unit
  = "owlgpu_dstub_buf_download"

external float32_ndarray_conv_spatial
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_spatial_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_spatial_native"

external float64_ndarray_conv_spatial
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_spatial_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_spatial_native"

external float32_ndarray_conv_spatial_backward_input
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_spatial_backward_input_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_spatial_backward_input_native"

external float64_ndarray_conv_spatial_backward_input
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_spatial_backward_input_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_spatial_backward_input_native"

external float32_ndarray_conv_spatial_backward_kernel
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_native"

external float64_ndarray_conv_spatial_backward_kernel
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_spatial_backward_kernel_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_spatial_backward_kernel_native"

external float32_ndarray_conv_cuboid_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_cuboid_im2col_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_cuboid_im2col_native"

external float64_ndarray_conv_cuboid_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_cuboid_im2col_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_cuboid_im2col_native"

external float32_ndarray_conv_cuboid_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_cuboid_backward_input_im2col_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_cuboid_backward_input_im2col_native"

external float64_ndarray_conv_cuboid_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_cuboid_backward_input_im2col_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_cuboid_backward_input_im2col_native"

external float32_ndarray_conv_cuboid_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_cuboid_backward_kernel_im2col_native"

external float64_ndarray_conv_cuboid_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_cuboid_backward_kernel_im2col_native"

external float32_ndarray_conv_dilated_spatial_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_dilated_spatial_im2col_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_dilated_spatial_im2col_native"

external float64_ndarray_conv_dilated_spatial_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_dilated_spatial_im2col_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_dilated_spatial_im2col_native"

external float32_ndarray_conv_dilated_spatial_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_input_im2col_native"

external float64_ndarray_conv_dilated_spatial_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_input_im2col_native"

external float32_ndarray_conv_dilated_spatial_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native"

external float64_ndarray_conv_dilated_spatial_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native"

external float32_ndarray_conv_dilated_cuboid_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_im2col_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_im2col_native"

external float64_ndarray_conv_dilated_cuboid_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_im2col_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_im2col_native"

external float32_ndarray_conv_dilated_cuboid_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_input_im2col_native"

external float64_ndarray_conv_dilated_cuboid_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_input_im2col_native"

external float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native"

external float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native"

external float32_ndarray_maxpool_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_maxpool_spatial_bytecode"
    "owlgpu_dstub_float32_ndarray_maxpool_spatial_native"

external float64_ndarray_maxpool_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_maxpool_spatial_bytecode"
    "owlgpu_dstub_float64_ndarray_maxpool_spatial_native"

external float32_ndarray_avgpool_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_avgpool_spatial_bytecode"
    "owlgpu_dstub_float32_ndarray_avgpool_spatial_native"

external float64_ndarray_avgpool_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_avgpool_spatial_bytecode"
    "owlgpu_dstub_float64_ndarray_avgpool_spatial_native"

external float32_ndarray_maxpool_spatial_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_maxpool_spatial_backward_bytecode"
    "owlgpu_dstub_float32_ndarray_maxpool_spatial_backward_native"

external float64_ndarray_maxpool_spatial_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_maxpool_spatial_backward_bytecode"
    "owlgpu_dstub_float64_ndarray_maxpool_spatial_backward_native"

external float32_ndarray_avgpool_spatial_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_avgpool_spatial_backward_bytecode"
    "owlgpu_dstub_float32_ndarray_avgpool_spatial_backward_native"

external float64_ndarray_avgpool_spatial_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_avgpool_spatial_backward_bytecode"
    "owlgpu_dstub_float64_ndarray_avgpool_spatial_backward_native"

external float32_ndarray_maxpool_argmax_spatial
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_maxpool_argmax_spatial_bytecode"
    "owlgpu_dstub_float32_ndarray_maxpool_argmax_spatial_native"

external float64_ndarray_maxpool_argmax_spatial
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_maxpool_argmax_spatial_bytecode"
    "owlgpu_dstub_float64_ndarray_maxpool_argmax_spatial_native"

external float32_ndarray_maxpool_cuboid
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_maxpool_cuboid_bytecode"
    "owlgpu_dstub_float32_ndarray_maxpool_cuboid_native"

external float64_ndarray_maxpool_cuboid
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_maxpool_cuboid_bytecode"
    "owlgpu_dstub_float64_ndarray_maxpool_cuboid_native"

external float32_ndarray_avgpool_cuboid
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_avgpool_cuboid_bytecode"
    "owlgpu_dstub_float32_ndarray_avgpool_cuboid_native"

external float64_ndarray_avgpool_cuboid
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_avgpool_cuboid_bytecode"
    "owlgpu_dstub_float64_ndarray_avgpool_cuboid_native"

external float32_ndarray_maxpool_cuboid_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_maxpool_cuboid_backward_bytecode"
    "owlgpu_dstub_float32_ndarray_maxpool_cuboid_backward_native"

external float64_ndarray_maxpool_cuboid_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_maxpool_cuboid_backward_bytecode"
    "owlgpu_dstub_float64_ndarray_maxpool_cuboid_backward_native"

external float32_ndarray_avgpool_cuboid_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_avgpool_cuboid_backward_bytecode"
    "owlgpu_dstub_float32_ndarray_avgpool_cuboid_backward_native"

external float64_ndarray_avgpool_cuboid_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_avgpool_cuboid_backward_bytecode"
    "owlgpu_dstub_float64_ndarray_avgpool_cuboid_backward_native"

external float32_ndarray_upsampling_spatial_backward
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_upsampling_spatial_backward_bytecode"
    "owlgpu_dstub_float32_ndarray_upsampling_spatial_backward_native"

external float64_ndarray_upsampling_spatial_backward
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_upsampling_spatial_backward_bytecode"
    "owlgpu_dstub_float64_ndarray_upsampling_spatial_backward_native"

external float32_ndarray_upsampling_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_upsampling_spatial_bytecode"
    "owlgpu_dstub_float32_ndarray_upsampling_spatial_native"

external float64_ndarray_upsampling_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_upsampling_spatial_bytecode"
    "owlgpu_dstub_float64_ndarray_upsampling_spatial_native"

external complex32_ndarray_conv_spatial
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_spatial_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_spatial_native"

external complex64_ndarray_conv_spatial
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_spatial_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_spatial_native"

external complex32_ndarray_conv_spatial_backward_input
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_spatial_backward_input_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_spatial_backward_input_native"

external complex64_ndarray_conv_spatial_backward_input
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_spatial_backward_input_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_spatial_backward_input_native"

external complex32_ndarray_conv_spatial_backward_kernel
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_spatial_backward_kernel_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_spatial_backward_kernel_native"

external complex64_ndarray_conv_spatial_backward_kernel
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_spatial_backward_kernel_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_spatial_backward_kernel_native"

external complex32_ndarray_conv_cuboid_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_cuboid_im2col_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_cuboid_im2col_native"

external complex64_ndarray_conv_cuboid_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_cuboid_im2col_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_cuboid_im2col_native"

external complex32_ndarray_conv_cuboid_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_input_im2col_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_input_im2col_native"

external complex64_ndarray_conv_cuboid_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_input_im2col_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_input_im2col_native"

external complex32_ndarray_conv_cuboid_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_cuboid_backward_kernel_im2col_native"

external complex64_ndarray_conv_cuboid_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_cuboid_backward_kernel_im2col_native"

external complex32_ndarray_conv_dilated_spatial_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_im2col_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_im2col_native"

external complex64_ndarray_conv_dilated_spatial_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_im2col_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_im2col_native"

external complex32_ndarray_conv_dilated_spatial_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_input_im2col_native"

external complex64_ndarray_conv_dilated_spatial_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_input_im2col_native"

external complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_dilated_spatial_backward_kernel_im2col_native"

external complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_dilated_spatial_backward_kernel_im2col_native"

external complex32_ndarray_conv_dilated_cuboid_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_im2col_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_im2col_native"

external complex64_ndarray_conv_dilated_cuboid_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_im2col_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_im2col_native"

external complex32_ndarray_conv_dilated_cuboid_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_input_im2col_native"

external complex64_ndarray_conv_dilated_cuboid_backward_input_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_input_im2col_native"

external complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_complex32_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native"

external complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_bytecode"
    "owlgpu_dstub_complex64_ndarray_conv_dilated_cuboid_backward_kernel_im2col_native"

external complex32_ndarray_maxpool_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_maxpool_spatial_bytecode"
    "owlgpu_dstub_complex32_ndarray_maxpool_spatial_native"

external complex64_ndarray_maxpool_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_maxpool_spatial_bytecode"
    "owlgpu_dstub_complex64_ndarray_maxpool_spatial_native"

external complex32_ndarray_avgpool_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_avgpool_spatial_bytecode"
    "owlgpu_dstub_complex32_ndarray_avgpool_spatial_native"

external complex64_ndarray_avgpool_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_avgpool_spatial_bytecode"
    "owlgpu_dstub_complex64_ndarray_avgpool_spatial_native"

external complex32_ndarray_maxpool_spatial_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_maxpool_spatial_backward_bytecode"
    "owlgpu_dstub_complex32_ndarray_maxpool_spatial_backward_native"

external complex64_ndarray_maxpool_spatial_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_maxpool_spatial_backward_bytecode"
    "owlgpu_dstub_complex64_ndarray_maxpool_spatial_backward_native"

external complex32_ndarray_avgpool_spatial_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_avgpool_spatial_backward_bytecode"
    "owlgpu_dstub_complex32_ndarray_avgpool_spatial_backward_native"

external complex64_ndarray_avgpool_spatial_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_avgpool_spatial_backward_bytecode"
    "owlgpu_dstub_complex64_ndarray_avgpool_spatial_backward_native"

external complex32_ndarray_maxpool_argmax_spatial
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_maxpool_argmax_spatial_bytecode"
    "owlgpu_dstub_complex32_ndarray_maxpool_argmax_spatial_native"

external complex64_ndarray_maxpool_argmax_spatial
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_maxpool_argmax_spatial_bytecode"
    "owlgpu_dstub_complex64_ndarray_maxpool_argmax_spatial_native"

external complex32_ndarray_maxpool_cuboid
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_maxpool_cuboid_bytecode"
    "owlgpu_dstub_complex32_ndarray_maxpool_cuboid_native"

external complex64_ndarray_maxpool_cuboid
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_maxpool_cuboid_bytecode"
    "owlgpu_dstub_complex64_ndarray_maxpool_cuboid_native"

external complex32_ndarray_avgpool_cuboid
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_avgpool_cuboid_bytecode"
    "owlgpu_dstub_complex32_ndarray_avgpool_cuboid_native"

external complex64_ndarray_avgpool_cuboid
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_avgpool_cuboid_bytecode"
    "owlgpu_dstub_complex64_ndarray_avgpool_cuboid_native"

external complex32_ndarray_maxpool_cuboid_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_maxpool_cuboid_backward_bytecode"
    "owlgpu_dstub_complex32_ndarray_maxpool_cuboid_backward_native"

external complex64_ndarray_maxpool_cuboid_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_maxpool_cuboid_backward_bytecode"
    "owlgpu_dstub_complex64_ndarray_maxpool_cuboid_backward_native"

external complex32_ndarray_avgpool_cuboid_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_avgpool_cuboid_backward_bytecode"
    "owlgpu_dstub_complex32_ndarray_avgpool_cuboid_backward_native"

external complex64_ndarray_avgpool_cuboid_backward
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_avgpool_cuboid_backward_bytecode"
    "owlgpu_dstub_complex64_ndarray_avgpool_cuboid_backward_native"

external complex32_ndarray_upsampling_spatial_backward
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_upsampling_spatial_backward_bytecode"
    "owlgpu_dstub_complex32_ndarray_upsampling_spatial_backward_native"

external complex64_ndarray_upsampling_spatial_backward
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_upsampling_spatial_backward_bytecode"
    "owlgpu_dstub_complex64_ndarray_upsampling_spatial_backward_native"

external complex32_ndarray_upsampling_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex32_ndarray_upsampling_spatial_bytecode"
    "owlgpu_dstub_complex32_ndarray_upsampling_spatial_native"

external complex64_ndarray_upsampling_spatial
  :  buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_complex64_ndarray_upsampling_spatial_bytecode"
    "owlgpu_dstub_complex64_ndarray_upsampling_spatial_native"

external float32_ndarray_conv_spatial_bias_act
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> buf option
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_spatial_bias_act_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_spatial_bias_act_native"

external float64_ndarray_conv_spatial_bias_act
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> buf option
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_spatial_bias_act_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_spatial_bias_act_native"

external float32_ndarray_conv_cuboid_bias_act
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> buf option
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_cuboid_bias_act_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_cuboid_bias_act_native"

external float64_ndarray_conv_cuboid_bias_act
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> buf option
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_ndarray_conv_cuboid_bias_act_bytecode"
    "owlgpu_dstub_float64_ndarray_conv_cuboid_bias_act_native"

external float32_bias_act_backward
  :  buf
  -> buf
  -> buf option
  -> buf option
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_bias_act_backward_bytecode"
    "owlgpu_dstub_float32_bias_act_backward_native"

external float64_bias_act_backward
  :  buf
  -> buf
  -> buf option
  -> buf option
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_bias_act_backward_bytecode"
    "owlgpu_dstub_float64_bias_act_backward_native"

external float32_dot
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> buf option
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_dot_bytecode"
    "owlgpu_dstub_float32_dot_native"

external float64_dot
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> buf option
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_dot_bytecode"
    "owlgpu_dstub_float64_dot_native"

external float32_softmax_cross_entropy
  :  buf
  -> buf
  -> buf option
  -> buf option
  -> buf option
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_softmax_cross_entropy_bytecode"
    "owlgpu_dstub_float32_softmax_cross_entropy_native"

external float64_softmax_cross_entropy
  :  buf
  -> buf
  -> buf option
  -> buf option
  -> buf option
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float64_softmax_cross_entropy_bytecode"
    "owlgpu_dstub_float64_softmax_cross_entropy_native"

external float32_sgd_update
  :  buf
  -> buf
  -> int
  -> float
  -> stream
  -> unit
  = "owlgpu_dstub_float32_sgd_update_native"

external float64_sgd_update
  :  buf
  -> buf
  -> int
  -> float
  -> stream
  -> unit
  = "owlgpu_dstub_float64_sgd_update_native"

external float32_ndarray_conv_spatial_backward_kernel_noalloc
  :  buf
  -> buf
  -> buf
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> int
  -> stream
  -> unit
  = "owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_noalloc_bytecode"
    "owlgpu_dstub_float32_ndarray_conv_spatial_backward_kernel_noalloc_native"
