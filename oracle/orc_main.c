/*
 * orc_main.c — whole-file CPU run of the oracle, the CPU counterpart of the
 * reference's main() (cuDebye-v15.cu:599-1004): read a .deb, histogram every
 * species pair in the order 00,01,..,0P,11,.. (:941-967), write
 * <prefix>x<row>x<col> when hist > 0 (:414-430), accumulate the FP64 Debye
 * sum and write <prefix>I when hist != 1 (:955-964, :988-1001).
 *
 * TEST INFRASTRUCTURE: used only to pin the oracle against the reference's
 * shipped outputs and as the CPU baseline.
 *
 * usage: orc_debye <file.deb> [output-prefix] [threads]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: orc_debye <file.deb> [output-prefix] [threads]\n");
    return 2;
  }
  const char *in = argv[1];
  const char *prefix = argc > 2 ? argv[2] : argv[1];
  int threads = argc > 3 ? atoi(argv[3]) : 0;
  orc_deb d;
  int rc = orc_deb_read(in, &d);
  if (rc == -1) {
    printf("\nERROR: >>%s<< does not exist\n", in);
    return 1;
  }
  if (rc == -3) {
    printf("\n\nERROR: Number of extracted Atoms doesn't match the number "
           "specified in the preamble!\n");
    return 1;
  }
  if (rc) {
    printf("ERROR: malformed .deb file (code %d)\n", rc);
    return 1;
  }
  const int64_t nb = orc_channels(d.rmax, d.rstep);
  const float inv = orc_inv_rstep(d.rstep);
  const int nq = orc_n_two_theta(d.tt_min, d.tt_max, d.tt_step);
  double *tt = (double *)malloc(sizeof(double) * nq);
  double *K = (double *)malloc(sizeof(double) * nq);
  double *ff = (double *)malloc(sizeof(double) * nq);
  double *I = (double *)calloc((size_t)nq, sizeof(double));
  int64_t *h = (int64_t *)malloc(sizeof(int64_t) * (size_t)nb);
  orc_k_grid(d.lambda, d.tt_min, d.tt_step, nq, tt, K);
  int64_t *start = (int64_t *)malloc(sizeof(int64_t) * d.nspecies);
  int64_t s0 = 0;
  for (int i = 0; i < d.nspecies; ++i) {
    start[i] = s0;
    s0 += d.sp[i].n;
  }
  char *path = (char *)malloc(strlen(prefix) + 64);
  for (int row = 0; row < d.nspecies; ++row) {
    for (int col = row; col < d.nspecies; ++col) {
      memset(h, 0, sizeof(int64_t) * (size_t)nb);
      int64_t bad = orc_block_histogram(d.x, d.y, d.z, start[row], d.sp[row].n,
                                        start[col], d.sp[col].n, row == col,
                                        inv, h, nb, threads, 1);
      if (bad) {
        printf("ERROR: %lld distances beyond rmax in block %d-%d\n",
               (long long)bad, row, col);
        return 1;
      }
      if (d.hist > 0) {
        sprintf(path, "%sx%dx%d", prefix, row, col);
        if (orc_write_debx(path, h, nb, d.rstep)) return 1;
      }
      if (d.hist != 1) {
        const orc_species *a = &d.sp[row], *b = &d.sp[col];
        orc_prefactor(K, nq, a->occ, a->beq, a->a, a->b, a->c, b->occ, b->beq,
                      b->a, b->b, b->c, ff);
        orc_debye_accumulate(K, nq, h, nb, d.rstep, ff, I, threads, 1);
      }
    }
  }
  if (d.hist != 1) {
    sprintf(path, "%sI", prefix);
    if (orc_write_debI(path, tt, I, nq)) return 1;
  }
  free(path);
  free(start);
  free(h);
  free(I);
  free(ff);
  free(K);
  free(tt);
  orc_deb_free(&d);
  return 0;
}
