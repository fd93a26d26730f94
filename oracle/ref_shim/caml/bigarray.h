/* Stand-in for <caml/bigarray.h>: only the array descriptor layout. */
#ifndef OWLREF_SHIM_BIGARRAY_H
#define OWLREF_SHIM_BIGARRAY_H
#include "mlvalues.h"
struct caml_ba_array {
  void *data;
  intnat num_dims;
  intnat flags;
  void *proxy;
  intnat dim[8];
};
#define Caml_ba_array_val(v) ((struct caml_ba_array *)(v))
#define Caml_ba_data_val(v) (Caml_ba_array_val(v)->data)
#define CAML_BA_KIND_MASK 0xFF
/* bytes of the array's data (element kind in flags & CAML_BA_KIND_MASK) */
uintnat caml_ba_byte_size(struct caml_ba_array *b);
#endif
