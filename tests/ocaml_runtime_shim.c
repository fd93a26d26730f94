/* Test stand-ins for the OCaml runtime calls the generated stubs make
 * (owl_gb300/ocaml/owlgpu_stubs.c, owlgpu_device_stubs.c): caml_failwith
 * records its message instead of raising, the blocking-section calls are
 * counted, custom blocks are malloc'd (operations pointer, then data) and
 * shim_finalize runs a block's finaliser as the collector would. */
#include <stdlib.h>
#include <string.h>

#include <caml/bigarray.h>
#include <caml/custom.h>

static char g_failure[512];
static int g_enter, g_leave;

/* OCaml's caml_failwith does not return; this one does, so the stub runs
 * on -- only the first failure after shim_reset is kept, the one OCaml
 * would have raised. */
void caml_failwith(const char *msg) {
  if (g_failure[0]) return;
  strncpy(g_failure, msg, sizeof g_failure - 1);
  g_failure[sizeof g_failure - 1] = 0;
}
void caml_enter_blocking_section(void) { ++g_enter; }
void caml_leave_blocking_section(void) { ++g_leave; }

value caml_alloc_custom(struct custom_operations *ops, uintnat size, mlsize_t mem, mlsize_t max) {
  (void)mem;
  (void)max;
  value *blk = calloc(1 + (size + sizeof(value) - 1) / sizeof(value), sizeof(value));
  *(struct custom_operations **)blk = ops;
  return (value)blk;
}

/* element sizes of Bigarray kinds, in OCaml's kind order (float32, float64,
 * int8, uint8, int16, uint16, int32, int64, caml_int, native_int,
 * complex32, complex64, char) */
static const int kind_size[] = {4, 8, 1, 1, 2, 2, 4, 8, 8, 8, 8, 16, 1};

uintnat caml_ba_byte_size(struct caml_ba_array *b) {
  uintnat n = (uintnat)kind_size[b->flags & CAML_BA_KIND_MASK];
  for (intnat i = 0; i < b->num_dims; ++i) n *= (uintnat)b->dim[i];
  return n;
}

const char *shim_last_failure(void) { return g_failure; }
int shim_entered(void) { return g_enter; }
int shim_left(void) { return g_leave; }
void shim_reset(void) {
  g_failure[0] = 0;
  g_enter = g_leave = 0;
}
/* the collector's view: run the block's finaliser, if it has one */
void shim_finalize(value v) {
  struct custom_operations *ops = Custom_ops_val(v);
  if (ops->finalize) ops->finalize(v);
}
const char *shim_custom_id(value v) { return Custom_ops_val(v)->identifier; }
void *shim_custom_data(value v) { return Data_custom_val(v); }
