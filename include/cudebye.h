/*
 * cudebye.h — C ABI of the GB300 Debye scattering engine.
 *
 * Drop-in for the hot path of cuDebye v1.5 (cuDebye-v15.cu). The reference
 * has no library interface: its path is the chain of host functions called
 * from main() for every species pair (cuDebye-v15.cu:941-967). Each entry
 * point below names the reference function it replaces. All entry points
 * are plain C: pointers, sizes and status codes; no CUDA or C++ types.
 *
 * Conventions
 *  - Every call returns DBX_OK (0) or a negative DBX_ERR_* code, and never
 *    exits the process (the reference calls exit() in gpuErrchk,
 *    cuDebye-v15.cu:58-66). dbx_last_error() gives the message of the last
 *    failed call on a context.
 *  - Host buffers belong to the caller; device memory belongs to the
 *    context. Calls are synchronous: on return the results are in the
 *    caller's host buffers.
 *  - One context per host thread (a context is not thread-safe).
 *  - Species pairs are numbered in the reference's loop order
 *    (cuDebye-v15.cu:941-942): for row = 0..P-1, for col = row..P-1.
 *    pair_index(row, col) = row*P - row*(row-1)/2 + (col - row).
 */
#ifndef CUDEBYE_H
#define CUDEBYE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DBX_OK 0
#define DBX_ERR_ARG (-1)      /* invalid argument */
#define DBX_ERR_CUDA (-2)     /* CUDA runtime error */
#define DBX_ERR_NOMEM (-3)    /* host or device allocation failed / HBM budget */
#define DBX_ERR_FILE (-4)     /* input file missing (cuDebye-v15.cu:619-622) */
#define DBX_ERR_PARSE (-5)    /* malformed .deb header or coordinate line */
#define DBX_ERR_COUNT (-6)    /* atom count != header total (:830-833) */
#define DBX_ERR_RANGE (-7)    /* a distance bins at or beyond rmax: the
                                 reference writes out of bounds there
                                 (README.md "Third Line") */
#define DBX_ERR_MODEL (-8)    /* unknown model id */
#define DBX_ERR_TIMEOUT (-9)  /* a bounded device-side wait ran out */
#define DBX_ERR_IO (-10)      /* output file could not be written */
#define DBX_ERR_LIMIT (-11)   /* request exceeds the fixed scratch of
                                 dbx_pair_histogram_noalloc */

typedef struct dbx_ctx dbx_ctx;

/* One species ("subgroup") of a .deb file (cuDebye-v15.cu:786): occupancy,
 * isotropic B (Beq) and the 11-parameter scattering factor
 * f = c + sum_i a_i exp(-b_i K^2/16 pi^2). */
typedef struct dbx_species {
  double occ, beq;
  double a[5], b[5], c;
} dbx_species;

/* Precision of the Debye sum. */
#define DBX_DEBYE_TC 0   /* tensor-core split contraction, FP64 chunk
                            reduction: max rel. error <= 1e-6 vs FP64 */
#define DBX_DEBYE_FP64 1 /* FP64 CUDA-core direct sum (the reference's
                            arithmetic, debyeRowSum cuDebye-v15.cu:493-538) */
#define DBX_DEBYE_FP32 2 /* plain FP32 direct sum (unbatched FP32 form) */
#define DBX_PLAIN 3      /* the plain unbatched FP32 GPU form of the whole
                            pattern: per model and pair one thread per atom
                            pair with a global atomic (the reference's dist /
                            dist2, cuDebye-v15.cu:88-146), then the FP32
                            direct Debye sum; comparison baseline only */
#define DBX_DEBYE_TC3 4  /* the tensor-core contraction with two 8-bit digits
                            per operand and three products (the BF16x3
                            scheme); not within 1e-6, for precision
                            comparisons only (dbx_intensity, dbx_pattern) */
#define DBX_DEBYE_TF32 5 /* the tensor-core contraction with each operand
                            split into tf32 hi/lo parts and three products
                            (the TF32-split scheme), FP32 accumulation per
                            256-bin chunk, FP64 chunk and q reduction; for
                            precision comparisons only (dbx_intensity,
                            dbx_pattern) */

/* ---- context ---------------------------------------------------------- */

/* Create a context on `device` (the reference's .deb line 1 device,
 * cudaSetDevice at cuDebye-v15.cu:646). hbm_budget_bytes = 0: no limit
 * beyond the device's free memory. */
int dbx_create(dbx_ctx **ctx, int device, size_t hbm_budget_bytes);
int dbx_destroy(dbx_ctx *ctx);
const char *dbx_strerror(int code);
const char *dbx_last_error(const dbx_ctx *ctx);
/* Bytes of device memory the context holds now. */
size_t dbx_device_bytes(const dbx_ctx *ctx);

/* ---- models ----------------------------------------------------------- */

/* Upload one atomistic model: FP32 SoA coordinates grouped by species in
 * species order (the reference's x/y/z arrays and start/end ranges,
 * cuDebye-v15.cu:770-833 and :887-909). species_counts[i] atoms belong to
 * species i. The model stays resident on the device until dbx_model_free
 * or dbx_destroy; the engine keeps its own spatially sorted copy. */
int dbx_model_upload(dbx_ctx *ctx, const float *x, const float *y,
                     const float *z, const int64_t *species_counts,
                     int nspecies, int64_t *model_id);
/* The same for coordinates interleaved as xyz[natoms][3] (x0 y0 z0 x1 ...),
 * the layout of .xyz files and of most host programs; no counterpart in the
 * reference, whose reader fills separate x, y, z arrays. Large models are
 * de-interleaved on the device, so the caller needs no transposed copy. */
int dbx_model_upload_xyz(dbx_ctx *ctx, const float *xyz,
                         const int64_t *species_counts, int nspecies,
                         int64_t *model_id);
int dbx_model_free(dbx_ctx *ctx, int64_t model_id);

/* ---- hot path 1: distance histogram ----------------------------------- */

/* Histogram of species pair (row, col), row <= col, into out_counts[nbins]
 * (int64, host). Replaces splitCalcDist + its kernels dist / dist2 /
 * care_dist2 (cuDebye-v15.cu:88-272): bin = (int)roundf(sqrtf((dx*dx +
 * dy*dy) + dz*dz) * float(1/rstep)) in unfused FP32, the diagonal block
 * counting i == j. Bit-exact with the reference. Returns DBX_ERR_RANGE if
 * any pair bins at k >= nbins. nbins is normally int(rmax/rstep)+2
 * (cuDebye-v15.cu:732; see dbx_channels). */
int dbx_pair_histogram(dbx_ctx *ctx, int64_t model_id, int row, int col,
                       double rstep, int64_t nbins, int64_t *out_counts);

/* The same histogram computed by the plain unbatched FP32 GPU form: one
 * thread per atom pair with one global 64-bit atomicAdd, in the
 * reference's launch shape (dist / dist2, cuDebye-v15.cu:88-146). The
 * comparison baseline only; bit-exact with dbx_pair_histogram. On
 * DBX_ERR_RANGE out_counts still holds the pairs binned below nbins. */
int dbx_pair_histogram_plain(dbx_ctx *ctx, int64_t model_id, int row, int col,
                             double rstep, int64_t nbins, int64_t *out_counts);

/* All P(P+1)/2 pair histograms in one device pass, out_counts
 * [npairs][nbins] in pair order (the pair loop cuDebye-v15.cu:941-967). */
int dbx_histogram(dbx_ctx *ctx, int64_t model_id, double rstep, int64_t nbins,
                  int64_t *out_counts);

/* Pair histogram for callers that cannot allocate device memory. No
 * counterpart in the reference (its splitCalcDist allocates with cudaMalloc
 * on every call, cuDebye-v15.cu:196-198).
 *
 * Who needs it: code running inside another framework's memory pool or a
 * fixed arena it must not grow, plugins in a host process that owns every
 * device allocation, and services that forbid device allocation once they
 * are up. This call allocates nothing: no cudaMalloc, no cudaFree, no
 * allocating library routine. All its scratch lives in one fixed 64 MiB
 * __device__ array that every GPU loading this library holds until the
 * process exits.
 *
 * Inputs are the reference's device arrays and index ranges: x, y, z
 * (float, device) and the atom ranges [a_start, a_start+a_count) and
 * [b_start, b_start+b_count). Equal starts mean a range paired with itself
 * (the reference's rule, cuDebye-v15.cu:241): it counts pairs j <= i
 * including i == j, like the reference's `dist` kernel, and needs equal
 * counts (else DBX_ERR_ARG). out (int64, device, nbins entries) receives
 * the histogram, bit-exact with dbx_pair_histogram; with DBX_ERR_RANGE it
 * still holds the pairs that binned below nbins. stream is a cudaStream_t
 * of the current device (NULL: the legacy default stream; a stream of
 * another device gives DBX_ERR_ARG). Every call waits for the stream to
 * finish its work before returning, so it blocks the calling thread.
 *
 * Limits: at most DBX_NOALLOC_MAX_ATOMS atoms (a_count + b_count, or a_count
 * for a range with itself; each count is checked alone first), else
 * DBX_ERR_LIMIT; nbins <= 4194304.
 * The first call on a device looks up the scratch array's device address
 * (with that device current), so make it before any stream capture. All
 * calls share the array and leave their data in it; each call clears what
 * must start at zero. Calls that overlap on the GPU race on the array: order
 * them (one stream, or events). */
#define DBX_NOALLOC_MAX_ATOMS 1834992
int dbx_pair_histogram_noalloc(const float *x, const float *y, const float *z,
                               int64_t a_start, int64_t a_count,
                               int64_t b_start, int64_t b_count, double rstep,
                               int64_t nbins, int64_t *out, void *stream);

/* int(rmax/rstep)+2 (cuDebye-v15.cu:732). */
int64_t dbx_channels(double rmax, double rstep);

/* Position of grid cell (x, y, z) (each < 2^bits, 1 <= bits <= 10) along
 * the Hilbert curve that orders each species' atoms into tiles (the
 * layout the upload builds; the reference keeps input order,
 * cuDebye-v15.cu:819-827). Host only; -1 for arguments out of range. */
int64_t dbx_curve_index(uint32_t x, uint32_t y, uint32_t z, int bits);

/* Self-checks of reduceCheck (cuDebye-v15.cu:360-410) on one pair
 * histogram: expected total n_a(n_a+1)/2 (diag) or n_a*n_b, bin 0 == n_a
 * (diag), and the count of distances below 0.25 A beyond the self pairs
 * ("possible atom collision"). Results in out[0..3] = {expected, observed,
 * zero-distance count (r <= 0.0005, diag) , collisions}. Returns DBX_OK;
 * the caller decides how to warn. */
int dbx_reduce_check(const int64_t *counts, int64_t nbins, double rstep,
                     int64_t n_row, int64_t n_col, int diag, int64_t out[4]);

/* Device self-check of the square root inside the histogram kernels (a
 * branch-free FMA-corrected form, not the library sqrtf): compares it bit
 * for bit with the IEEE square root for every float whose bits lie in
 * [lo_bits, hi_bits], 0 <= lo_bits <= hi_bits <= 0x7F800000 (+inf). Inputs
 * below 2^-75 only need a result below 2^-37 (every bin made from them is
 * 0), +inf only a non-finite one. out = {inputs checked, mismatches, bits of
 * the smallest mismatch or -1}. No counterpart in the reference, which
 * calls sqrtf (cuDebye-v15.cu:101-107). */
int dbx_check_sqrt(dbx_ctx *ctx, uint32_t lo_bits, uint32_t hi_bits,
                   int64_t out[3]);

/* ---- hot path 2: Debye sum -------------------------------------------- */

/* 2theta grid and K = 4 pi sin(theta)/lambda (cuDebye-v15.cu:690-698).
 * Returns the number of points int((max-min)/step)+1; fills the arrays when
 * they are non-NULL (they must hold that many doubles). */
int dbx_k_grid(double lambda, double tt_min, double tt_max, double tt_step,
               double *two_theta, double *K);

/* Prefactor o_a o_b exp(-(B_a+B_b)K^2/16pi^2) f_a(K) f_b(K) of one pair on
 * the device, FP64 (atomicProp/atomicScatter, cuDebye-v15.cu:447-479). */
int dbx_atomic_prop(dbx_ctx *ctx, const dbx_species *a, const dbx_species *b,
                    const double *K, int nq, double *out_ff);

/* Intensity of one model: I[q] = sum over pairs of ff_pair(q) *
 * sum_k m_k sin(K r_k)/(K r_k), r_k = k*rstep, m_k = 2 n_k (r_k > 0.0005),
 * n_k otherwise (intensity/debyeRowSum, cuDebye-v15.cu:493-577, summed over
 * the pair loop :941-967). Computes the histograms on the device first
 * (they are kept resident for re-scoring with new K or species). mode is
 * DBX_DEBYE_*. sp holds nspecies entries. out_I[nq] (host). */
int dbx_intensity(dbx_ctx *ctx, int64_t model_id, double rstep, int64_t nbins,
                  const dbx_species *sp, const double *K, int nq, int mode,
                  double *out_I);

/* One full pattern: recompute every pair histogram of the model (no cached
 * histograms are used) and the Debye sum, as one pass of the reference's
 * pair loop (cuDebye-v15.cu:941-967) does. Same arguments as
 * dbx_intensity. */
int dbx_pattern(dbx_ctx *ctx, int64_t model_id, double rstep, int64_t nbins,
                const dbx_species *sp, const double *K, int nq, int mode,
                double *out_I);

/* Full patterns of many resident models in one pass: one histogram launch
 * over every (model, pair) and one tensor-core contraction over every
 * column, replayed as a CUDA graph while the batch (models, binning, q grid)
 * stays the same; the histogram task granularity is autotuned on the first
 * pass of a batch. Replaces running the reference's main() once per model
 * (Matlab/multisim.m:19-65 runs cuDebye.exe file by file). All models share
 * rstep and the q grid K[nq]; model i has nbins[i] bins and its species are
 * the next nspecies(i) entries of sp (models in the order given). out_I is
 * [nmodels][nq]. mode: DBX_DEBYE_TC (batched), DBX_DEBYE_FP64 /
 * DBX_DEBYE_FP32 (per model, direct sums) or DBX_PLAIN (per model, the plain
 * form). */
int dbx_patterns(dbx_ctx *ctx, const int64_t *model_ids, int nmodels,
                 double rstep, const int64_t *nbins, const dbx_species *sp,
                 const double *K, int nq, int mode, double *out_I);

/* Max relative error of each pattern of a batch (I = out_I of dbx_patterns
 * with the same arguments, [nmodels][nq]) against the FP64 direct sum of
 * the models' resident histograms (the reference's debyeRowSum arithmetic,
 * cuDebye-v15.cu:493-538) at every q_stride-th q; q values where the FP64
 * sum is 0 or not finite are skipped. out_maxrel[nmodels]. No counterpart
 * in the reference, which has no error report. */
int dbx_pattern_errors(dbx_ctx *ctx, const int64_t *model_ids, int nmodels,
                       double rstep, const int64_t *nbins, const dbx_species *sp,
                       const double *K, int nq, const double *I, int q_stride,
                       double *out_maxrel);

/* The choices the batch autotuner made for the last dbx_patterns plan (no
 * counterpart in the reference, whose tiling is the user's .deb line 1,
 * cuDebye-v15.cu:644 and :152-224): out[0] histogram CTA tasks, out[1] tasks
 * per SM, out[2] 1 if the plan splits histograms into several bin windows,
 * out[3] the 32-row item factor chosen (0: 128-row items only), out[4] the
 * window geometry (0 chosen per species pair from sampled tile pairs, 1
 * disjoint windows), out[5] shapes timed, out[6] task counts timed, out[7]
 * the chosen histogram launch's device time in ms. DBX_ERR_ARG before the
 * first dbx_patterns call. */
int dbx_batch_tuning(const dbx_ctx *ctx, double out[8]);

/* CUDA-graph replay of dbx_patterns (default on). */
int dbx_set_graphs(dbx_ctx *ctx, int enable);

/* ---- streams and timing ----------------------------------------------- */

/* Launch on the caller's CUDA stream (a cudaStream_t passed as void*);
 * NULL returns to the context's own stream. The reference has no
 * counterpart (it runs on the legacy default stream). */
int dbx_set_stream(dbx_ctx *ctx, void *cuda_stream);

/* Device time of the phases of the last histogram / Debye call, measured
 * with CUDA events on the launching stream when enabled (timing adds one
 * event pair per launch). The reference printed clock() wall times
 * (cuDebye-v15.cu:928-971). */
#define DBX_T_HIST 0        /* tile-pair histogram kernel */
#define DBX_T_HIST_REDUCE 1 /* merge of the CTA windows */
#define DBX_T_PREFACTOR 2   /* atomicScatter equivalent */
#define DBX_T_DEBYE 3       /* Debye sum kernels */
#define DBX_T_PASS 4        /* a whole dbx_patterns graph replay */
#define DBX_NTIMERS 5
int dbx_set_timing(dbx_ctx *ctx, int enable);
int dbx_get_timing(const dbx_ctx *ctx, double out_ms[DBX_NTIMERS]);

/* Host<->device bytes the context has copied since it was created:
 * out[0] host to device, out[1] device to host. */
int dbx_get_traffic(const dbx_ctx *ctx, int64_t out[2]);

/* ---- serving ---------------------------------------------------------- */

/* A pattern server on one GPU: a worker thread admits pattern requests by
 * HBM footprint (idle resident models evicted least recently used first),
 * serves all admitted requests of a round together (the histograms of all
 * new models in one launch, then per request the contraction or, for new
 * species parameters on the same q grid, a weighted sum of the resident
 * per-pair row sums), and overlaps two rounds on two streams so requests
 * that arrive while others run are admitted as soon as a lane and memory
 * free up. No counterpart in the reference (one pattern per process run;
 * Matlab/multisim.m:19-65 loops over files). Thread-safe: any host thread
 * may submit and wait. */
typedef struct dbx_server dbx_server;

typedef struct dbx_request {
  int64_t model;                 /* 0: new model from x/y/z/species_counts;
                                    else a resident model returned by an
                                    earlier request (re-scoring) */
  const float *x, *y, *z;        /* new model: FP32 coordinates grouped by
                                    species */
  const int64_t *species_counts; /* new model: atoms per species */
  int nspecies;                  /* entries of sp (and species_counts) */
  const dbx_species *sp;         /* species parameters of this request */
  double rstep;                  /* bin width; re-scores repeat the model's */
  int64_t nbins;                 /* bins; re-scores repeat the model's */
  const double *K;               /* q grid of this request */
  int nq;
} dbx_request;

int dbx_server_create(dbx_server **srv, int device, size_t hbm_budget_bytes);
/* Copies the request and returns at once with a ticket. */
int dbx_server_submit(dbx_server *srv, const dbx_request *req, int64_t *ticket);
/* Blocks until the ticket's pattern is done: out_I[nq] (nq >= the request's
 * nq), the model id to re-score it later, and submit-to-done latency. */
int dbx_server_wait(dbx_server *srv, int64_t ticket, double *out_I, int nq,
                    int64_t *model_out, double *latency_ms);
/* out = {rounds, completed requests, resident models, device bytes held
 * (models and lane workspaces), evictions, bytes kept free for the lanes}. */
int dbx_server_stats(dbx_server *srv, int64_t out[6]);
int dbx_server_destroy(dbx_server *srv);

/* ---- .xyz -> .deb conversion (host only) -------------------------------- */

/* Header values of the written .deb (Matlab/xyz2deb.m:13-25 defaults via
 * dbx_xyz2deb_defaults: device 0, block 16, grid 2048, 1.5418 A, 2theta
 * 10-140 step 0.02, rstep 0.0001, intensity 1, distances 0). */
typedef struct dbx_xyz2deb_params {
  int device, block, grid;
  double lambda, tt_min, tt_max, tt_step, rstep;
  int intensity; /* write a .debI (hist 0 or 2) */
  int distances; /* write .debx files (hist 1 or 2) */
} dbx_xyz2deb_params;
void dbx_xyz2deb_defaults(dbx_xyz2deb_params *params);

/* The reference's Matlab converter xyz2deb (Matlab/xyz2deb.m:154-263):
 * "element x y z [occ [Beq]]" records -> species grouped by (element, occ,
 * Beq), coordinates centred, rmax = 2 ceil(1.025 max r), coefficients from a
 * Waasmaier-Kirfel table in the RIETAN layout (e.g. the reference's
 * Matlab/Tables/atomic_scattering_factors_RIETAN.txt). deb_path NULL = the
 * .xyz path with its last three characters replaced by "deb". params NULL =
 * the defaults. msg (may be NULL) receives an error text. Needs no GPU. */
int dbx_xyz2deb(const char *xyz_path, const char *table_path,
                const dbx_xyz2deb_params *params, const char *deb_path,
                char *msg, size_t msg_len);

/* The .deb content in binary form (the reference's wish list item "binary
 * file support", cuDebye-v15.cu:7): reads deb_path (text or binary) and
 * writes out_path as "DBXDEB1" + header values + species + float32 x[], y[],
 * z[] (layout in csrc/debio.cpp). dbx_run_deb and the command line take
 * either form. Needs no GPU. msg (may be NULL) receives an error text. */
int dbx_deb_pack(const char *deb_path, const char *out_path, char *msg,
                 size_t msg_len);

/* ---- whole-file drop-in ----------------------------------------------- */

/* The reference's main() (cuDebye-v15.cu:599-1004) on the GPU: read
 * `deb_path`, write <out_prefix>x<row>x<col> (hist 1/2) and <out_prefix>I
 * (hist 0/2), byte-compatible with the reference's outputs on a POSIX host.
 * out_prefix NULL = deb_path, as the reference does. verbose != 0 prints
 * the reference-style progress log to stdout. */
int dbx_run_deb(dbx_ctx *ctx, const char *deb_path, const char *out_prefix,
                int verbose);

/* The reference's Matlab batch driver multisim (Matlab/multisim.m:9-65)
 * without its plots: in directory `dir`, convert every .xyz that has no .deb
 * (dbx_xyz2deb with its defaults; skipped when table_path is NULL), then
 * compute every .deb that has no .debI, writing the same outputs as
 * dbx_run_deb would. Models sharing rstep and the 2theta grid run batched
 * (dbx_patterns, up to 64 per chunk); outputs are written on a host thread
 * while the next chunk runs. Every file is attempted; the first error is
 * returned. The device index on line 1 of the files is not used (ctx's
 * device is). */
int dbx_run_dir(dbx_ctx *ctx, const char *dir, const char *table_path,
                int verbose);

#ifdef __cplusplus
}
#endif
#endif
