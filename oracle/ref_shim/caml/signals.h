/* Stand-in for <caml/signals.h>; Owl's conv/pool stubs use nothing
 * from it; the OCaml binding in owl_gb300/ocaml/ uses what is declared here. */
#include "mlvalues.h"
void caml_enter_blocking_section(void);
void caml_leave_blocking_section(void);
