/* Empty stand-in for <caml/memory.h>; the conv/pool stubs use nothing from it. */
#include "mlvalues.h"
