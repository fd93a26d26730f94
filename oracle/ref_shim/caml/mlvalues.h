/* Minimal stand-in for OCaml's <caml/mlvalues.h>, enough to compile Owl's
 * conv/pool C stubs as a plain shared library for use as a test oracle.
 * A `value` holding a Bigarray is a pointer to struct caml_ba_array; an
 * integer argument is tagged as OCaml does ((n << 1) | 1). */
#ifndef OWLREF_SHIM_MLVALUES_H
#define OWLREF_SHIM_MLVALUES_H
#include <stdint.h>
#include <stddef.h>
typedef intptr_t intnat;
typedef uintptr_t uintnat;
typedef intnat value;
typedef uintnat mlsize_t;
typedef unsigned int tag_t;
#define CAMLprim
#define CAMLextern extern
#define Long_val(x) ((intnat)(x) >> 1)
#define Int_val(x) ((int)Long_val(x))
#define Val_long(x) ((((intnat)(x)) << 1) + 1)
#define Val_int(x) Val_long(x)
#define Val_unit Val_long(0)
#define Val_bool(x) Val_long((x) != 0)
#define Bool_val(x) Int_val(x)
#define Double_val(v) (*(double *)(v))
#define Field(x, i) (((value *)(x))[i])
#define Double_wosize 1
#define Double_array_tag 254
#define Store_double_field(v, i, d) (((double *)(v))[i] = (d))
#define Double_field(v, i) (((double *)(v))[i])
#define Wosize_val(v) 0
#define Is_long(x) (((x) & 1) != 0)
#define Is_block(x) (((x) & 1) == 0)
#endif
