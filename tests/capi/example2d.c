/* The reference's examples/example2d.py through the C-ABI alone: three
 * cells of type 1 grow to area 200 in a 256^2 box.  Prints the centroids,
 * one "x y" line per cell, and exits 0 when every call succeeded.
 *
 *   cc -I include tests/capi/example2d.c -L gpu-cpm_gb300 -lgpucpm_gb300 \
 *      -Wl,-rpath,gpu-cpm_gb300 -o example2d && ./example2d
 */
#include <stdio.h>

#include "gpucpm.h"

#define CHECK(call)                                                       \
  do {                                                                    \
    int rc_ = (call);                                                     \
    if (rc_ != CPM_OK) {                                                  \
      fprintf(stderr, "%s failed (%d): %s\n", #call, rc_,                 \
              cpm_last_error(h));                                         \
      return 1;                                                           \
    }                                                                     \
  } while (0)

int main(void) {
  cpm_handle* h = NULL;
  /* Cpm(dimension=256, dimensionality=2, number_of_cells=10, temperature=20) */
  if (cpm_create(256, 2, 10, 20.0f, 0, &h) != CPM_OK) {
    fprintf(stderr, "cpm_create failed: %s\n", cpm_last_error(NULL));
    return 1;
  }
  CHECK(cpm_set_seed(h, 7, 0));
  CHECK(cpm_add_cell(h, 1, 100, 100, 0));
  CHECK(cpm_add_cell(h, 1, 200, 200, 0));
  CHECK(cpm_add_cell(h, 1, 200, 100, 0));
  CHECK(cpm_set_area(h, 1, 200, 10.0f));        /* lambda_area=10, target_area=200 */
  CHECK(cpm_set_adhesion(h, 0, 1, 10.0f, 1));   /* medium-cell J = 10, symmetric */
  CHECK(cpm_push(h));
  CHECK(cpm_run(h, 2000));
  CHECK(cpm_synchronize(h));
  CHECK(cpm_pull(h));
  double c[3 * 2];
  int n = 0;
  CHECK(cpm_get_centroids(h, c, 3, &n));
  for (int i = 0; i < n; ++i) printf("%.6f %.6f\n", c[2 * i], c[2 * i + 1]);
  CHECK(cpm_destroy(h));
  return n == 3 ? 0 : 1;
}
