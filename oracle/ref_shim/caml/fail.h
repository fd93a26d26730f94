/* Stand-in for <caml/fail.h>; Owl's conv/pool stubs use nothing
 * from it; the OCaml binding in owl_gb300/ocaml/ uses what is declared here. */
#include "mlvalues.h"
void caml_failwith(const char *msg);
