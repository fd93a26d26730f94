/* Stand-in for <caml/memory.h>; Owl's conv/pool stubs use nothing from it.
 * Local-root registration is a no-op here (there is no collector). */
#include "mlvalues.h"
#define CAMLparam0() do { } while (0)
#define CAMLparam1(a) (void)(a)
#define CAMLparam2(a, b) ((void)(a), (void)(b))
#define CAMLparam3(a, b, c) ((void)(a), (void)(b), (void)(c))
#define CAMLparam4(a, b, c, d) ((void)(a), (void)(b), (void)(c), (void)(d))
#define CAMLreturn(v) return (v)
#define CAMLlocal1(a) value a = 0
