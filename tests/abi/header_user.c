/* A C11 program against include/tara.h alone: the header compiles as C with
 * -Wall -Wextra -pedantic -Werror, the library links, and the entry points
 * validate their arguments and report through tara_last_error() without a
 * GPU.  Prints "ok" and exits 0, or prints the failing check and exits 1. */
#include <stdio.h>
#include <string.h>

#include "tara.h"

int fortran_style_calls(void);

#define CHECK(cond)                                   \
  do {                                                \
    if (!(cond)) {                                    \
      printf("failed: %s (line %d)\n", #cond, __LINE__); \
      return 1;                                       \
    }                                                 \
  } while (0)

int main(void) {
  const char* v = tara_version();
  CHECK(v != NULL && strstr(v, "sm_103a") != NULL);

  tara2d_config c;
  tara2d_default_config(&c, 64, 64);
  CHECK(c.nx == 64 && c.ny == 64);
  c.nx = 88; /* neither a power of two nor 2, 3, 5, 7-smooth (a factor 11) */
  tara2d* h = (tara2d*)&c; /* must be reset to NULL on failure */
  CHECK(tara2d_create(&c, &h) == TARA_ERR_ARGS);
  CHECK(h == NULL);
  CHECK(tara_last_error() == TARA_ERR_ARGS);
  CHECK(tara_last_error_message() != NULL && tara_last_error_message()[0] != '\0');
  tara_clear_error();
  CHECK(tara_last_error() == TARA_OK);
  CHECK(tara2d_create(NULL, &h) == TARA_ERR_ARGS);
  CHECK(tara2d_destroy(NULL) == TARA_OK);

  const int rc = fortran_style_calls();
  if (rc != 0) {
    printf("failed: fortran_style_calls check %d\n", rc);
    return 1;
  }
  printf("ok\n");
  return 0;
}
