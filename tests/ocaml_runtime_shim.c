/* Test stand-ins for the three OCaml runtime calls the generated stubs make
 * (owl_gb300/ocaml/owlgpu_stubs.c): caml_failwith records its message
 * instead of raising, and the blocking-section calls are counted. */
#include <string.h>

static char g_failure[512];
static int g_enter, g_leave;

void caml_failwith(const char *msg) {
  strncpy(g_failure, msg, sizeof g_failure - 1);
  g_failure[sizeof g_failure - 1] = 0;
}
void caml_enter_blocking_section(void) { ++g_enter; }
void caml_leave_blocking_section(void) { ++g_leave; }

const char *shim_last_failure(void) { return g_failure; }
int shim_entered(void) { return g_enter; }
int shim_left(void) { return g_leave; }
void shim_reset(void) {
  g_failure[0] = 0;
  g_enter = g_leave = 0;
}
