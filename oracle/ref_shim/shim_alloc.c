/* Definitions behind the shim's alloc.h; the conv/pool stubs never call them. */
#include <stdlib.h>
#include "caml/alloc.h"
value caml_alloc_small(mlsize_t wosize, tag_t tag) { (void)tag; return (value)calloc(wosize + 1, sizeof(value)); }
value caml_copy_double(double d) { double *p = malloc(sizeof(double)); *p = d; return (value)p; }
