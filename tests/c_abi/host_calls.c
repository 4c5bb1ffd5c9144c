/* A plain C99 caller of the C ABI (the shape of a cgo / ctypes / JNI binding):
 * only host-side entry points, so it runs without a GPU.  Prints one line of
 * results that the test compares with the Python binding. */
#include <stdio.h>
#include <stdlib.h>

#include "qed3.h"

int main(void) {
  qed3_lattice* lat = NULL;
  int ns = 0, nl = 0, nf = 0, ft = 0, size = 0;
  if (qed3_lattice_create(4, &lat) != QED3_OK) return 1;
  if (qed3_lattice_sizes(lat, &ns, &nl, &nf, &ft) != QED3_OK) return 2;
  double* vert = (double*)malloc(sizeof(double) * 3 * (size_t)nf);
  int* tri = (int*)malloc(sizeof(int) * 3 * (size_t)ns);
  double* ell = (double*)malloc(sizeof(double) * (size_t)nl);
  if (qed3_lattice_mesh(lat, vert, tri) != QED3_OK) return 3;
  qed3_lattice* lat2 = NULL;
  if (qed3_lattice_from_mesh(nf, vert, ns, tri, NULL, &lat2) != QED3_OK) return 4;
  if (qed3_lattice_tables(lat2, NULL, NULL, NULL, NULL, NULL, NULL, ell, NULL, NULL, NULL, NULL, NULL) != QED3_OK)
    return 5;
  /* an invalid call reports an error code and a message, never aborts */
  qed3_lattice* bad = NULL;
  const int rc_bad = qed3_lattice_create(-1, &bad);
  double c[32], cp[32], A[32], scal[4];
  if (qed3_zolotarev(0.01, 21, c, cp, A, scal, &size) != QED3_OK) return 6;
  qed3_rng* rng = NULL;
  double g[3];
  if (qed3_rng_create(3, 1, 7, &rng) != QED3_OK || qed3_rng_gaussian_links(rng, 1.0, g) != QED3_OK) return 7;
  /* argument checks of the batched solver (no device work): no systems, unknown schedule */
  qed3_batch* bt = NULL;
  const int nr1 = 1;
  const int rc_b0 = qed3_batch_create2(0, NULL, &nr1, QED3_PREC_F32, 0, 0, 0, &bt);
  int sched = 0;
  const int rc_b1 = qed3_batch_schedule(NULL, &sched);
  printf("%d %d %d %d %.17g %d %d %.17g %.17g %d %d\n", ns, nl, nf, ft, ell[0], rc_bad, size, scal[3], g[0], rc_b0,
         rc_b1);
  printf("%s\n", qed3_last_error_string() ? "message" : "none");
  qed3_rng_destroy(rng);
  qed3_lattice_destroy(lat2);
  qed3_lattice_destroy(lat);
  free(vert);
  free(tri);
  free(ell);
  return 0;
}
