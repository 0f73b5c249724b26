/* A C99 caller of the C ABI (include/pymoto_gb300.h) without Python: the header compiles as C, and the host-only
 * entry points and the argument checks work from C.  Built and run by tests/test_capi.py; needs no GPU. */
#include <stdio.h>

#include "pymoto_gb300.h"

int main(void) {
  double K0[24 * 24];
  int rc = pmg_element_stiffness(3, 1.0, 0.3, 0, 1.0, 1.0, 1.0, K0);
  if (rc != PMG_OK) return 10 + rc;
  printf("version %d\n", pmg_version());
  printf("status %s\n", pmg_status_string(PMG_BAD_ARG));
  printf("K0");
  for (int i = 0; i < 24 * 24; ++i) printf(" %.17g", K0[i]);
  printf("\n");
  /* invalid arguments are rejected before any launch: no device is touched */
  double dummy = 0.0;
  printf("bad_mode %d\n", pmg_scalar_apply(7, PMG_F64, 4, 4, 4, &dummy, &dummy, &dummy, &dummy, 0.0, &dummy + 1,
                                           NULL));
  printf("bad_grid %d\n", pmg_ebe_apply(PMG_APPLY_MATVEC, PMG_F64, 0, 4, 4, &dummy, K0, NULL, 1.0, &dummy, NULL,
                                        NULL, 0.0, &dummy + 1, NULL, NULL));
  return 0;
}
