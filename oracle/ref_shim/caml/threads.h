/* Empty stand-in for <caml/threads.h>; the conv/pool stubs use nothing from it. */
#include "mlvalues.h"
