/* Empty stand-in for <caml/fail.h>; the conv/pool stubs use nothing from it. */
#include "mlvalues.h"
