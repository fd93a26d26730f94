#ifndef OWLREF_SHIM_ALLOC_H
#define OWLREF_SHIM_ALLOC_H
#include "mlvalues.h"
/* Never called by the conv/pool stubs; declared for owl_core.h inlines. */
value caml_alloc_small(mlsize_t wosize, tag_t tag);
value caml_copy_double(double d);
#endif
