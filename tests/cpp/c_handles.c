/* The C handles (C_CPP_Matrix*_*, C_CPP_Vector_*) as a C caller such as the
 * YML components uses them, without products: fills, prints, files written,
 * read back at byte offsets and printed again, vector arithmetic, NULL
 * handling.  Built once against the drop-in headers and library and once
 * against the reference's own C headers and sources; the two runs must print
 * the same text and write the same files.
 *
 *   c_handles <directory for the files>
 */
#include <stdio.h>
#include <string.h>

#include <tbsla/cpp/MatrixCOO.h>
#include <tbsla/cpp/MatrixCSR.h>
#include <tbsla/cpp/MatrixDENSE.h>
#include <tbsla/cpp/MatrixELL.h>
#include <tbsla/cpp/MatrixSCOO.h>
#include <tbsla/cpp/Vector.h>

static char path[4096];

static char *file(const char *dir, const char *name) {
  snprintf(path, sizeof path, "%s/%s", dir, name);
  return path;
}

/* one format: two fills (the second a cdiag when `cd`; CSR and SCOO keep the
 * reference's nnz from before a cdiag fill, which this library does not),
 * written to two files, read back and printed */
#define EXERCISE(F, dir, cd)                                                              \
  do {                                                                                    \
    C_CPP_Matrix##F##_t *m = C_CPP_Matrix##F##_create();                                  \
    C_CPP_Matrix##F##_t *b = C_CPP_Matrix##F##_create();                                  \
    printf("== " #F "\n");                                                                \
    C_CPP_Matrix##F##_fill_cqmat(m, 12, 10, 4, 0.3, 2, 0, 0, 1, 1);                       \
    C_CPP_Matrix##F##_print(m);                                                           \
    printf("write %d\n", (int)C_CPP_Matrix##F##_write(m, file(dir, #F ".bin")));          \
    FILE *fh = fopen(path, "rb");                                                         \
    long first = 0;                                                                       \
    if (fh) { fseek(fh, 0, SEEK_END); first = ftell(fh); fclose(fh); }                    \
    if (cd) C_CPP_Matrix##F##_fill_cdiag(m, 9, 11, 2, 1, 0, 2, 1);                        \
    else C_CPP_Matrix##F##_fill_cqmat(m, 9, 11, 3, 0.5, 4, 1, 0, 2, 1);                    \
    C_CPP_Matrix##F##_print(m);                                                           \
    printf("write %d\n", (int)C_CPP_Matrix##F##_write(m, file(dir, #F "_2.bin")));        \
    printf("read %d\n", (int)C_CPP_Matrix##F##_read(b, file(dir, #F ".bin"), 0));          \
    C_CPP_Matrix##F##_print(b);                                                           \
    printf("first file %ld bytes\n", first);                                              \
    printf("read %d\n", (int)C_CPP_Matrix##F##_read(b, file(dir, #F "_2.bin"), 0));        \
    C_CPP_Matrix##F##_print(b);                                                           \
    printf("read missing %d\n", (int)C_CPP_Matrix##F##_read(b, file(dir, "none.bin"), 0)); \
    printf("read NULL %d\n", (int)C_CPP_Matrix##F##_read(NULL, file(dir, #F ".bin"), 0));  \
    printf("write NULL %d\n", (int)C_CPP_Matrix##F##_write(NULL, file(dir, "x.bin")));     \
    C_CPP_Matrix##F##_destroy(m);                                                         \
    C_CPP_Matrix##F##_destroy(b);                                                         \
    C_CPP_Matrix##F##_destroy(NULL);                                                      \
  } while (0)

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  const char *dir = argv[1];
  EXERCISE(COO, dir, 1);
  EXERCISE(SCOO, dir, 0);
  EXERCISE(CSR, dir, 0);
  EXERCISE(ELL, dir, 1);
  EXERCISE(DENSE, dir, 1);

  printf("== Vector\n");
  C_CPP_Vector_t *v = C_CPP_Vector_create(), *w = C_CPP_Vector_create(), *g = C_CPP_Vector_create();
  C_CPP_Vector_fill(v, 6, 3);
  C_CPP_Vector_fill(w, 9, -4);
  C_CPP_Vector_print(v);
  C_CPP_Vector_print(w);
  printf("add %d\n", (int)C_CPP_Vector_add(v, w));
  C_CPP_Vector_print(v);
  printf("add_incr %d\n", (int)C_CPP_Vector_add_incr(v, w, 3));
  C_CPP_Vector_print(v);
  printf("gather %d\n", (int)C_CPP_Vector_gather(g, v));
  printf("gather %d\n", (int)C_CPP_Vector_gather(g, w));
  C_CPP_Vector_print(g);
  printf("write %d\n", (int)C_CPP_Vector_write(v, file(dir, "vec.bin")));
  printf("write %d\n", (int)C_CPP_Vector_write(w, file(dir, "vec.bin")));  /* appends */
  C_CPP_Vector_t *r = C_CPP_Vector_create();
  printf("read %d\n", (int)C_CPP_Vector_read(r, file(dir, "vec.bin"), 0));
  C_CPP_Vector_print(r);
  printf("read %d\n", (int)C_CPP_Vector_read(r, file(dir, "vec.bin"), (int)(sizeof(size_t) + 6 * sizeof(double))));
  C_CPP_Vector_print(r);
  printf("read missing %d\n", (int)C_CPP_Vector_read(r, file(dir, "none.bin"), 0));
  C_CPP_Vector_copy(r, v->obj);
  C_CPP_Vector_print(r);
  printf("NULL: add %d add_incr %d gather %d read %d write %d\n", (int)C_CPP_Vector_add(NULL, v),
         (int)C_CPP_Vector_add_incr(v, NULL, 1), (int)C_CPP_Vector_gather(NULL, NULL),
         (int)C_CPP_Vector_read(NULL, file(dir, "vec.bin"), 0), (int)C_CPP_Vector_write(NULL, file(dir, "x.bin")));
  C_CPP_Vector_print(NULL);
  C_CPP_Vector_fill(NULL, 3, 1);
  C_CPP_Vector_copy(NULL, v->obj);
  C_CPP_Vector_destroy(v);
  C_CPP_Vector_destroy(w);
  C_CPP_Vector_destroy(g);
  C_CPP_Vector_destroy(r);
  C_CPP_Vector_destroy(NULL);
  fflush(stdout);
  return 0;
}
