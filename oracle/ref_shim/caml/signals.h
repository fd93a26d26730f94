/* Empty stand-in for <caml/signals.h>; the conv/pool stubs use nothing from it. */
#include "mlvalues.h"
