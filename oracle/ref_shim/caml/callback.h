/* Empty stand-in for <caml/callback.h>; the conv/pool stubs use nothing from it. */
#include "mlvalues.h"
