/* Golden-vector harness around the original Himeno benchmark's jacobi()
 * (examples/himeno/himenobmtxpa_original.c:297-346, set-up 86-116 and
 * 268-290).  Test infrastructure only: the reference source is #included
 * from where it lies (its main() renamed) so that jacobi() runs unmodified
 * for a fixed sweep count.  Writes
 *   <out>.p.f32     p after `nn` sweeps, rows x cols x deps with deps fastest
 *                   (= Physis x fastest), raw float32
 *   <out>.gosa.txt  the gosa of the last sweep (C99 hex float)
 * Usage: ref_himeno_harness <rows> <cols> <deps> <nn> <out-prefix> */
#define main himeno_original_main
#include HIMENO_SRC
#undef main

int main(int argc, char **argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: %s rows cols deps nn out-prefix\n", argv[0]);
    return 2;
  }
  int rows = atoi(argv[1]), cols = atoi(argv[2]), deps = atoi(argv[3]);
  int nn = atoi(argv[4]);
  char path[4096];
  newMat(&p, 1, rows, cols, deps);
  newMat(&bnd, 1, rows, cols, deps);
  newMat(&wrk1, 1, rows, cols, deps);
  newMat(&wrk2, 1, rows, cols, deps);
  newMat(&a, 4, rows, cols, deps);
  newMat(&b, 3, rows, cols, deps);
  newMat(&c, 3, rows, cols, deps);
  mat_set_init(&p);
  mat_set(&bnd, 0, 1.0);
  mat_set(&wrk1, 0, 0.0);
  mat_set(&wrk2, 0, 0.0);
  mat_set(&a, 0, 1.0);
  mat_set(&a, 1, 1.0);
  mat_set(&a, 2, 1.0);
  mat_set(&a, 3, 1.0 / 6.0);
  mat_set(&b, 0, 0.0);
  mat_set(&b, 1, 0.0);
  mat_set(&b, 2, 0.0);
  mat_set(&c, 0, 1.0);
  mat_set(&c, 1, 1.0);
  mat_set(&c, 2, 1.0);
  float gosa = jacobi(nn, &a, &b, &c, &p, &bnd, &wrk1, &wrk2);
  snprintf(path, sizeof(path), "%s.p.f32", argv[5]);
  FILE *f = fopen(path, "wb");
  fwrite(p.m, sizeof(float), (size_t)rows * cols * deps, f);
  fclose(f);
  snprintf(path, sizeof(path), "%s.gosa.txt", argv[5]);
  f = fopen(path, "w");
  fprintf(f, "%a\n", gosa);
  fclose(f);
  return 0;
}
