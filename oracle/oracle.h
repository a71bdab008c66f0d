/*
 * oracle.h — CPU restatement of cuDebye v1.5's hot path (cuDebye-v15.cu).
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE. Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference arm may load or run this code, and
 * only as the checker or as the timed CPU baseline. The engine never calls it.
 *
 * Parity status: pinned. The histogram reproduces the six shipped
 * Data/GammaAl2O3_10nm.debx* files of the reference bit for bit, and the
 * intensity reproduces the shipped .debI files (Gamma, UH3) to their
 * 6-significant-digit print precision (tests/test_oracle_golden.py).
 */
#ifndef CUDEBYE_ORACLE_H
#define CUDEBYE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* float(1/rstep) as the reference stores it (cuDebye-v15.cu:739). */
float orc_inv_rstep(double rstep);

/* Number of histogram channels int(rmax/rstep)+2 (cuDebye-v15.cu:732). */
int64_t orc_channels(double rmax, double rstep);

/* Bin of one atom pair, FP32 unfused, IEEE sqrtf and roundf
 * (cuDebye-v15.cu:101-107 and :115). */
int64_t orc_pair_bin(float xi, float yi, float zi, float xj, float yj, float zj,
                     float inv_rstep);

/* Distance histogram of one species block into int64 counts (added to hist).
 * diag != 0: block a==a, pairs j <= i including i == j (cuDebye-v15.cu:134-146);
 * diag == 0: all na*nb pairs (cuDebye-v15.cu:88-131).
 * Returns the number of pairs whose bin fell outside [0, nbins) (the reference
 * would write out of bounds there, README.md "Third Line"); those are not
 * counted. nthreads <= 0 uses all OpenMP threads. row_stride > 1 samples every
 * row_stride-th row atom (used only for bounded CPU-baseline timing). */
int64_t orc_block_histogram(const float *x, const float *y, const float *z,
                            int64_t a0, int64_t na, int64_t b0, int64_t nb,
                            int diag, float inv_rstep, int64_t *hist,
                            int64_t nbins, int nthreads, int64_t row_stride);

/* Number of 2theta points int((max-min)/step)+1 (cuDebye-v15.cu:690). */
int orc_n_two_theta(double tt_min, double tt_max, double tt_step);

/* 2theta_i = min + i*step and K_i = 4 pi sin(2theta_i/2 pi/180)/lambda
 * (cuDebye-v15.cu:695-698). */
void orc_k_grid(double lambda, double tt_min, double tt_step, int n,
                double *two_theta, double *K);

/* Per-q prefactor o_a o_b exp(-(B_a+B_b) K^2/16pi^2) f_a(K) f_b(K), FP64,
 * evaluation order of atomicScatter (cuDebye-v15.cu:447-467).
 * a1,b1,a2,b2 point at 5 coefficients each. */
void orc_prefactor(const double *K, int nq, double occ1, double beq1,
                   const double *a1, const double *b1, double c1, double occ2,
                   double beq2, const double *a2, const double *b2, double c2,
                   double *ff);

/* Isum[q] += ff[q] * sum_k m_k sin(K r_k)/(K r_k) over non-zero bins, with
 * r_k = k*rstep, m_k = 2 n_k for r_k > 0.0005 and m_k = n_k otherwise
 * (cuDebye-v15.cu:493-537 with the compaction of :283-346). FP64.
 * q_stride > 1 evaluates only every q_stride-th q (bounded CPU-baseline
 * timing); skipped entries are left untouched. */
void orc_debye_accumulate(const double *K, int nq, const int64_t *hist,
                          int64_t nbins, double rstep, const double *ff,
                          double *Isum, int nthreads, int q_stride);

/* Same sum without the prefactor: S[q] = sum_k m_k sinc(K r_k). */
void orc_debye_rowsum(const double *K, int nq, const int64_t *hist,
                      int64_t nbins, double rstep, double *S, int nthreads);

/* ------------------------------------------------------------------------ */
/* .deb model (cuDebye-v15.cu:635-833) */
typedef struct orc_species {
  int64_t n;
  char name[32];
  double occ, beq, a[5], b[5], c;
} orc_species;

typedef struct orc_deb {
  int device, block, grid;                      /* line 1 (:644) */
  double lambda, tt_min, tt_max, tt_step;       /* line 2 (:689) */
  double rmax, rstep;                           /* line 3 (:730) */
  int hist;                                     /* 0/1/2 (:745-754) */
  int nspecies;                                 /* line 4 (:761) */
  orc_species *sp;                              /* (:782-804) */
  int64_t natoms;
  float *x, *y, *z;                             /* (:819-827) */
} orc_deb;

/* Returns 0, or -1 file missing (:619-622), -2 malformed header,
 * -3 atom count mismatch (:830-833), -4 malformed coordinate line. */
int orc_deb_read(const char *path, orc_deb *out);
void orc_deb_free(orc_deb *d);

/* Writers, byte-compatible with the reference's ostream output on a POSIX
 * host ("\n" line ends). .debx: non-zero bins, "%.7g\t%llu" of k*rstep and
 * the count (:414-430). .debI: "%.6g\t%.6g" of 2theta and I (:988-1001). */
int orc_write_debx(const char *path, const int64_t *hist, int64_t nbins,
                   double rstep);
int orc_write_debI(const char *path, const double *two_theta, const double *I,
                   int n);

#ifdef __cplusplus
}
#endif
#endif
