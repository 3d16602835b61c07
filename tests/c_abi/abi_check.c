/* Plain-C client of the library's C ABI (include/qimpy_gb300.h): compiles as
 * C99 against the header, links libqimpy_gb300.so, and exercises entry points
 * that need no GPU: version, workspace sizing, and argument validation (every
 * call below must return an error status with a message, touching no device
 * memory).  Prints one line per check; exit status 0 when all pass. */
#include <stdio.h>
#include <string.h>

#include "qimpy_gb300.h"

static int failures = 0;

static void expect(int ok, const char* what) {
  printf("%s %s\n", ok ? "ok  " : "FAIL", what);
  if (!ok) ++failures;
}

int main(void) {
  expect(qgb_abi_version() == QGB_ABI_VERSION, "abi version matches the header");

  qgb_sphere s;
  memset(&s, 0, sizeof s);
  s.nk = 2;
  s.n_tot = 1200;
  s.N[0] = s.N[1] = s.N[2] = 36;
  s.L1[0] = s.L1[1] = s.L1[2] = 6;
  s.L2[0] = s.L2[1] = s.L2[2] = 6;
  s.max_slabs = 15;
  /* planes of one band: nk * max_slabs * N1 * N2 complex */
  expect(qgb_potential_workspace_bytes(&s, 1, QGB_F64) == (size_t)2 * 15 * 36 * 36 * 16,
         "FP64 plane workspace per band");
  expect(qgb_potential_workspace_bytes(&s, 4, QGB_F32) == (size_t)4 * 2 * 15 * 36 * 36 * 8,
         "FP32 plane workspace for 4 bands");
  expect(qgb_potential_workspace_bytes(NULL, 1, QGB_F64) == 0, "NULL sphere sizes to 0");

  /* The sphere's device tables are NULL: rejected before any launch. */
  int rc = qgb_apply_potential(&s, QGB_F64, NULL, NULL, 1, 0u, NULL, 0, NULL);
  expect(rc == QGB_ERR_INVALID && strlen(qgb_last_error()) > 0, "apply_potential rejects NULL tables");
  rc = qgb_apply_potential(NULL, QGB_F64, NULL, NULL, 1, 0u, NULL, 0, NULL);
  expect(rc == QGB_ERR_INVALID, "apply_potential rejects a NULL sphere");
  rc = qgb_apply_potential(&s, 7, NULL, NULL, 1, 0u, NULL, 0, NULL);
  expect(rc == QGB_ERR_INVALID, "apply_potential rejects an unknown dtype");
  s.L1[1] = 5; /* 5 * 6 != 36 */
  rc = qgb_collect_density(&s, QGB_F64, NULL, 1, NULL, NULL, 0u, NULL, 0, NULL);
  expect(rc == QGB_ERR_INVALID, "collect_density rejects a bad factorisation");
  rc = qgb_apply_nonlocal_tc_phase(NULL, NULL, 1, 4, NULL, NULL, NULL, 1, 1, 1, NULL, 0, NULL, 5, NULL);
  expect(rc == QGB_ERR_INVALID, "the store flag (4) needs phase 2");
  rc = qgb_apply_nonlocal_tc_phase(NULL, NULL, 1, 4, NULL, NULL, NULL, 1, 1, 1, NULL, 0, NULL, 8, NULL);
  expect(rc == QGB_ERR_INVALID, "nonlocal phases are 1, 2 or 3, plus 4 with 2");
  rc = qgb_apply_nonlocal_tc_phase(NULL, NULL, 1, 4, NULL, NULL, NULL, 1, 1, 1, NULL, 0, NULL, 6, NULL);
  expect(rc == QGB_ERR_INVALID && strstr(qgb_last_error(), "NULL") != NULL,
         "a valid store phase still rejects NULL pointers");
  return failures ? 1 : 0;
}
