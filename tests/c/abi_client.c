/* A plain C99 client of the sfx C ABI (include/sfx.h, sfx_solver.h,
 * sfx_learned.h): compiled with gcc as C, linked against libsfx_gb300.so, and
 * run without a GPU — it checks the version and the host-side argument
 * validation, and prints OK. */
#include <stdio.h>
#include <string.h>

#include "sfx.h"
#include "sfx_learned.h"
#include "sfx_solver.h"

int main(void) {
  sfx_mesh mesh = NULL;
  sfx_form form = NULL;
  int failures = 0;
  if (sfx_version() < 1) failures++;
  if (sfx_mesh_create_structured_hex(0, 1, 1, NULL, &mesh) != SFX_ERR_INVALID) failures++;
  if (strstr(sfx_last_error(), "dimensions") == NULL) failures++;
  if (sfx_form_create_from_table(3, 1, 1, 8, NULL, NULL, &form) != SFX_ERR_UNSUPPORTED) failures++;
  if (sfx_residual(NULL, 0.0, NULL, NULL, NULL) != SFX_ERR_INVALID) failures++;
  if (sfx_qoi_evaluate(NULL, 0.0, NULL, NULL, NULL) != SFX_ERR_INVALID) failures++;
  if (sfx_solver_solve(NULL, 0.0, NULL, NULL) != SFX_ERR_INVALID) failures++;
  if (failures) {
    printf("%d checks failed\n", failures);
    return 1;
  }
  printf("OK\n");
  return 0;
}
