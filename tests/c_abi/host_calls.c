/* A C caller of the drop-in boundary (include/dgsw.h): host-only entry
 * points, as a reference-side binding would call them.  Prints what it gets
 * so the test can compare with the Python binding of the same library. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "dgsw.h"

int main(void) {
  double x[8], w[8], M[8 * 4];
  int rc = dgsw_lgl_points_weights(8, x, w);
  printf("abi %d\n", dgsw_abi_version());
  printf("lgl %d", rc);
  for (int i = 0; i < 8; ++i) printf(" %.17g %.17g", x[i], w[i]);
  printf("\n");
  rc = dgsw_amr_matrix(4, 8, 2, M);
  printf("amr %d", rc);
  for (int i = 0; i < 32; ++i) printf(" %.17g", M[i]);
  printf("\n");
  /* a 2 x 2 x 2 periodic brick: element ids and neighbours */
  DgswBrick brick = {{0.0, 0.0, 0.0}, {1.0, 1.0, 1.0}, {2, 2, 2}};
  DgswConfig cfg = {0};
  cfg.system = DGSW_SYSTEM_SCALAR_WAVE_3D;
  cfg.n_instances = 1;
  cfg.bricks = &brick;
  cfg.uniform_points = 6;
  int64_t n_elem = 0, n_doubles = 0;
  rc = dgsw_count_elements(&cfg, &n_elem, &n_doubles);
  printf("count %d %lld %lld\n", rc, (long long)n_elem, (long long)n_doubles);
  uint64_t ids[8];
  int32_t nbr[48], mortar[48];
  rc = dgsw_index_maps(&cfg, ids, nbr, mortar);
  printf("maps %d", rc);
  for (int e = 0; e < 8; ++e) printf(" %llu", (unsigned long long)ids[e]);
  for (int i = 0; i < 48; ++i) printf(" %d", nbr[i]);
  printf("\n");
  /* errors are status codes with a message, never an abort */
  rc = dgsw_amr_matrix(5, 4, 1, M);
  printf("error %d %s\n", rc, dgsw_last_error(NULL) ? "message" : "none");
  return 0;
}
