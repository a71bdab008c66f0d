/*
 * oracle.c — CPU restatement of cuDebye v1.5's hot path (cuDebye-v15.cu).
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE: the checker for the CUDA engine and
 * the timed CPU baseline. Must be compiled with -ffp-contract=off (the
 * reference's distances are unfused FP32; a fused dz*dz+(dx*dx+dy*dy) gives
 * different bins on the shipped Gamma sample). Parity is pinned against the
 * reference's shipped outputs, see oracle.h.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846 /* cuDebye-v15.cu:46 */

float orc_inv_rstep(double rstep) { return (float)(1.0 / rstep); }

int64_t orc_channels(double rmax, double rstep) {
  return (int64_t)(int)(rmax / rstep) + 2;
}

/* cuDebye-v15.cu:101-107: dx = x[col]-x[row] etc., r = dx*dx+dy*dy+dz*dz
 * evaluated left to right without contraction, r = round(sqrt(r)*rp_rstep),
 * then int(r) at :115. The sign of dx does not matter (exact negation). */
static inline int64_t bin_of(float dx, float dy, float dz, float inv) {
  float s = dx * dx;
  s = s + dy * dy;
  s = s + dz * dz;
  float r = roundf(sqrtf(s) * inv);
  return (int64_t)r;
}

int64_t orc_pair_bin(float xi, float yi, float zi, float xj, float yj, float zj,
                     float inv_rstep) {
  return bin_of(xj - xi, yj - yi, zj - zi, inv_rstep);
}

int64_t orc_block_histogram(const float *x, const float *y, const float *z,
                            int64_t a0, int64_t na, int64_t b0, int64_t nb,
                            int diag, float inv, int64_t *hist, int64_t nbins,
                            int nthreads, int64_t row_stride) {
  int64_t bad = 0;
  if (row_stride < 1) row_stride = 1;
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nt = 1;
  (void)nthreads;
#endif
  /* One private int64 histogram per thread, merged at the end. */
  int64_t *priv = (int64_t *)calloc((size_t)nt * (size_t)nbins, sizeof(int64_t));
  if (!priv) return -1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt) reduction(+ : bad)
#endif
  {
#ifdef _OPENMP
    int t = omp_get_thread_num();
#else
    int t = 0;
#endif
    int64_t *h = priv + (size_t)t * (size_t)nbins;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int64_t ii = 0; ii < na; ii += row_stride) {
      const int64_t i = a0 + ii;
      const float xi = x[i], yi = y[i], zi = z[i];
      /* diag: the reference's kernel `dist` keeps col <= row, i.e. every
       * unordered pair once plus i == j (cuDebye-v15.cu:137). */
      const int64_t jend = diag ? (ii + 1) : nb;
      for (int64_t jj = 0; jj < jend; ++jj) {
        const int64_t j = b0 + jj;
        int64_t k = bin_of(x[j] - xi, y[j] - yi, z[j] - zi, inv);
        if (k >= 0 && k < nbins)
          h[k] += 1;
        else
          bad += 1;
      }
    }
  }
  for (int t = 0; t < nt; ++t) {
    const int64_t *h = priv + (size_t)t * (size_t)nbins;
    for (int64_t k = 0; k < nbins; ++k) hist[k] += h[k];
  }
  free(priv);
  return bad;
}

int orc_n_two_theta(double tt_min, double tt_max, double tt_step) {
  return (int)((tt_max - tt_min) / tt_step) + 1;
}

void orc_k_grid(double lambda, double tt_min, double tt_step, int n,
                double *two_theta, double *K) {
  for (int i = 0; i < n; ++i) {
    double tt = tt_min + (double)i * tt_step;
    if (two_theta) two_theta[i] = tt;
    K[i] = 4 * ORC_PI * sin(tt / 2 * ORC_PI / 180) / lambda;
  }
}

/* cuDebye-v15.cu:452-465, same constant and the same operation order. */
void orc_prefactor(const double *K, int nq, double occ1, double beq1,
                   const double *a1, const double *b1, double c1, double occ2,
                   double beq2, const double *a2, const double *b2, double c2,
                   double *ff) {
  const double rp16pi2 = -0.006332573977646;
  for (int q = 0; q < nq; ++q) {
    double nhs = K[q] * K[q] * rp16pi2;
    double v = occ1 * occ2;
    v = v * exp(nhs * (beq1 + beq2));
    double f1 = c1, f2 = c2;
    for (int i = 0; i < 5; ++i) {
      f1 += a1[i] * exp(b1[i] * nhs);
      f2 += a2[i] * exp(b2[i] * nhs);
    }
    ff[q] = v * f1 * f2;
  }
}

/* Compacted non-zero bins (cuDebye-v15.cu:309-346). */
static int64_t compact(const int64_t *hist, int64_t nbins, int64_t **idx) {
  int64_t nnz = 0;
  for (int64_t k = 0; k < nbins; ++k) nnz += hist[k] != 0;
  *idx = (int64_t *)malloc((size_t)(nnz ? nnz : 1) * sizeof(int64_t));
  int64_t p = 0;
  for (int64_t k = 0; k < nbins; ++k)
    if (hist[k] != 0) (*idx)[p++] = k;
  return nnz;
}

/* One row of debyeRowSum (cuDebye-v15.cu:508-522):
 * r > 0.0005: 2*nr*sin(K r)/(K r), else nr (self distance). */
static double rowsum(double Kq, const int64_t *hist, const int64_t *idx,
                     int64_t nnz, double rstep) {
  double s = 0.0;
  for (int64_t p = 0; p < nnz; ++p) {
    const int64_t k = idx[p];
    const double r = (double)k * rstep;
    const double n = (double)hist[k];
    if (r > 0.0005)
      s += 2 * n * sin(Kq * r) / (Kq * r);
    else
      s += n;
  }
  return s;
}

void orc_debye_accumulate(const double *K, int nq, const int64_t *hist,
                          int64_t nbins, double rstep, const double *ff,
                          double *Isum, int nthreads, int q_stride) {
  int64_t *idx;
  int64_t nnz = compact(hist, nbins, &idx);
  if (q_stride < 1) q_stride = 1;
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
#else
  (void)nthreads;
#endif
  for (int q = 0; q < nq; q += q_stride) {
    /* Sum = rowsum * ffoobb; Isum += Sum (cuDebye-v15.cu:534-536) */
    double s = rowsum(K[q], hist, idx, nnz, rstep);
    Isum[q] += s * ff[q];
  }
  free(idx);
}

void orc_debye_rowsum(const double *K, int nq, const int64_t *hist,
                      int64_t nbins, double rstep, double *S, int nthreads) {
  int64_t *idx;
  int64_t nnz = compact(hist, nbins, &idx);
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
#else
  (void)nthreads;
#endif
  for (int q = 0; q < nq; ++q) S[q] = rowsum(K[q], hist, idx, nnz, rstep);
  free(idx);
}

/* ------------------------------------------------------------------------ */
/* .deb reader (cuDebye-v15.cu:629-835). Lines are read whole; the header
 * lines are parsed with strtol/strtod like istringstream >> int/double; the
 * coordinates with strtof like >> float. A line holding only whitespace
 * (including a CR of a CRLF file) counts as empty and is skipped, as in the
 * reference's Windows text-mode build (:821). */

static char *read_line(FILE *f) {
  size_t cap = 256, len = 0;
  char *buf = (char *)malloc(cap);
  int c;
  while ((c = fgetc(f)) != EOF) {
    if (c == '\n') break;
    if (len + 1 >= cap) {
      cap *= 2;
      buf = (char *)realloc(buf, cap);
    }
    buf[len++] = (char)c;
  }
  if (c == EOF && len == 0) {
    free(buf);
    return NULL;
  }
  buf[len] = 0;
  return buf;
}

static int blank(const char *s) {
  for (; *s; ++s)
    if (*s != ' ' && *s != '\t' && *s != '\r' && *s != '\v' && *s != '\f')
      return 0;
  return 1;
}

int orc_deb_read(const char *path, orc_deb *d) {
  memset(d, 0, sizeof(*d));
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  char *l1 = read_line(f), *l2 = read_line(f), *l3 = read_line(f),
       *l4 = read_line(f);
  int rc = 0;
  if (!l1 || !l2 || !l3 || !l4) {
    rc = -2;
    goto done_hdr;
  }
  if (sscanf(l1, "%d %d %d", &d->device, &d->block, &d->grid) != 3 ||
      sscanf(l2, "%lf %lf %lf %lf", &d->lambda, &d->tt_min, &d->tt_max,
             &d->tt_step) != 4 ||
      sscanf(l3, "%lf %lf %d", &d->rmax, &d->rstep, &d->hist) != 3 ||
      sscanf(l4, "%d", &d->nspecies) != 1 || d->nspecies < 1) {
    rc = -2;
    goto done_hdr;
  }
  if (d->hist != 1 && d->hist != 2) d->hist = 0; /* :751-753 */
  d->sp = (orc_species *)calloc((size_t)d->nspecies, sizeof(orc_species));
  for (int i = 0; i < d->nspecies; ++i) {
    char *l = read_line(f);
    orc_species *s = &d->sp[i];
    long long n = 0;
    int got = l ? sscanf(l,
                         "%lld %31s %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf "
                         "%lf %lf %lf",
                         &n, s->name, &s->occ, &s->beq, &s->a[0], &s->a[1],
                         &s->a[2], &s->a[3], &s->a[4], &s->b[0], &s->b[1],
                         &s->b[2], &s->b[3], &s->b[4], &s->c)
                : 0;
    free(l);
    if (got != 15 || n < 0) {
      rc = -2;
      goto done_hdr;
    }
    s->n = n;
    d->natoms += n;
  }
  d->x = (float *)malloc((size_t)(d->natoms ? d->natoms : 1) * sizeof(float));
  d->y = (float *)malloc((size_t)(d->natoms ? d->natoms : 1) * sizeof(float));
  d->z = (float *)malloc((size_t)(d->natoms ? d->natoms : 1) * sizeof(float));
  {
    int64_t i = 0;
    char *l;
    while ((l = read_line(f)) != NULL) {
      if (!blank(l)) {
        if (i < d->natoms) {
          char *p = l, *e;
          float v[3];
          for (int c = 0; c < 3; ++c) {
            v[c] = strtof(p, &e);
            if (e == p) {
              rc = -4;
              break;
            }
            p = e;
          }
          if (rc == 0) {
            d->x[i] = v[0];
            d->y[i] = v[1];
            d->z[i] = v[2];
          }
        }
        ++i;
      }
      free(l);
      if (rc) break;
    }
    if (rc == 0 && i != d->natoms) rc = -3; /* :830-833 */
  }
done_hdr:
  free(l1);
  free(l2);
  free(l3);
  free(l4);
  fclose(f);
  if (rc) orc_deb_free(d);
  return rc;
}

void orc_deb_free(orc_deb *d) {
  free(d->sp);
  free(d->x);
  free(d->y);
  free(d->z);
  memset(d, 0, sizeof(*d));
}

int orc_write_debx(const char *path, const int64_t *hist, int64_t nbins,
                   double rstep) {
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  for (int64_t k = 0; k < nbins; ++k)
    if (hist[k] != 0)
      fprintf(f, "%.7g\t%lld\n", (double)k * rstep, (long long)hist[k]);
  return fclose(f) ? -1 : 0;
}

int orc_write_debI(const char *path, const double *two_theta, const double *I,
                   int n) {
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  for (int i = 0; i < n; ++i) fprintf(f, "%.6g\t%.6g\n", two_theta[i], I[i]);
  return fclose(f) ? -1 : 0;
}
