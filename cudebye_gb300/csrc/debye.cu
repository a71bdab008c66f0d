// debye.cu — Debye sum kernels on sm_103a (hot path 2, direct forms).
//
//  * species_f_kernel + debye_prefactor_kernel / prefactor_cols_kernel: the
//    reference's atomicScatter (cuDebye-v15.cu:447-467) in FP64, the form
//    factor once per (species, q), the pair product once per (pair, q).
//  * debye_direct_kernel<T>: the reference's debyeRowSum arithmetic
//    (cuDebye-v15.cu:493-538) for all pairs of a model at once: one thread
//    per q, bins staged through shared memory, sinc evaluated once per
//    (q, bin) and shared by every pair. T = double is the FP64 form; T =
//    float is the plain unbatched FP32 GPU form used as the speed baseline.
//    Zero bins are skipped, as the reference's compaction does
//    (cuDebye-v15.cu:323-333).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "engine.h"

namespace dbx {

struct SpeciesDev {
  double occ, beq, a[5], b[5], c;
};

// f_s(q) = c + sum_i a_i exp(b_i nhs), nhs = -K^2/(16 pi^2): the form
// factor of atomicScatter (cuDebye-v15.cu:452-462), computed once per q and
// distinct coefficient set; the pair kernels read it instead of recomputing
// both factors for every pair (same operations, same values). Row u is
// species rep[u] (rep null: species u); rows with rep[u] < 0 are unused.
__global__ void species_f_kernel(const SpeciesDev *__restrict__ sp,
                                 const int *__restrict__ rep,
                                 const double *__restrict__ K, int nq,
                                 double *__restrict__ F) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int u = blockIdx.y;
  const int s = rep ? rep[u] : u;
  if (q >= nq || s < 0) return;
  const SpeciesDev &sd = sp[s];
  const double rp16pi2 = -0.006332573977646;  // cuDebye-v15.cu:452
  const double nhs = K[q] * K[q] * rp16pi2;
  double f = sd.c;
#pragma unroll
  for (int i = 0; i < 5; ++i) f += sd.a[i] * exp(sd.b[i] * nhs);
  F[(size_t)u * nq + q] = f;
}

// ff = (o1 o2) exp(nhs (B1 + B2)) f1 f2 in the reference's order
// (cuDebye-v15.cu:463-465).
__device__ __forceinline__ double pair_prefactor(const SpeciesDev &s1,
                                                 const SpeciesDev &s2,
                                                 double Kq, double f1,
                                                 double f2) {
  const double rp16pi2 = -0.006332573977646;  // cuDebye-v15.cu:452
  const double nhs = Kq * Kq * rp16pi2;
  double v = s1.occ * s2.occ;
  v = v * exp(nhs * (s1.beq + s2.beq));
  return v * f1 * f2;
}

__global__ void debye_prefactor_kernel(const SpeciesDev *__restrict__ sp,
                                       int nspecies,
                                       const double *__restrict__ K, int nq,
                                       const double *__restrict__ F,
                                       double *__restrict__ ff) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (q >= nq) return;
  // pair index -> (row, col) in the reference's loop order (:941-942)
  int row = 0, rem = p;
  while (rem >= nspecies - row) {
    rem -= nspecies - row;
    ++row;
  }
  const int col = row + rem;
  ff[(size_t)p * nq + q] = pair_prefactor(sp[row], sp[col], K[q],
                                          F[(size_t)row * nq + q],
                                          F[(size_t)col * nq + q]);
}

Error debye_prefactor(const dbx_species *sp, int nspecies, const double *d_K,
                      int nq, double *d_ff, cudaStream_t stream, PinArena *arena) {
  static_assert(sizeof(SpeciesDev) == sizeof(dbx_species), "layout");
  SpeciesDev *d_sp = nullptr;
  double *d_F = nullptr;
  DBX_CUDA_TRY(cudaMallocAsync((void **)&d_sp, sizeof(SpeciesDev) * nspecies,
                               stream));
  cudaError_t e = cudaMallocAsync((void **)&d_F,
                                  sizeof(double) * nq * (size_t)nspecies, stream);
  if (e == cudaSuccess) {
    const void *from = sp;
    if (arena)
      if (void *p = arena->take(sizeof(SpeciesDev) * nspecies)) {
        std::memcpy(p, sp, sizeof(SpeciesDev) * nspecies);
        from = p;
      }
    e = cudaMemcpyAsync(d_sp, from, sizeof(SpeciesDev) * nspecies,
                        cudaMemcpyHostToDevice, stream);
  }
  if (e == cudaSuccess) {
    species_f_kernel<<<dim3((nq + 127) / 128, nspecies), 128, 0, stream>>>(
        d_sp, nullptr, d_K, nq, d_F);
    dim3 grid((nq + 127) / 128, npairs_of(nspecies));
    debye_prefactor_kernel<<<grid, 128, 0, stream>>>(d_sp, nspecies, d_K, nq,
                                                     d_F, d_ff);
    e = cudaGetLastError();
  }
  if (d_F) cudaFreeAsync(d_F, stream);
  cudaFreeAsync(d_sp, stream);
  if (e != cudaSuccess)
    return fail(DBX_ERR_CUDA, std::string("prefactor: ") + cudaGetErrorString(e));
  return ok();
}

// Prefactor of many (model, pair) columns at once: column c uses species
// col_sp[c] = {a, b} of the concatenated species array, whose form factors
// are rows fid[a], fid[b] of F.
__global__ void prefactor_cols_kernel(const SpeciesDev *__restrict__ sp,
                                      const int2 *__restrict__ col_sp,
                                      const int *__restrict__ fid,
                                      const double *__restrict__ K, int nq,
                                      const double *__restrict__ F,
                                      double *__restrict__ ff) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (q >= nq) return;
  const int2 ab = col_sp[c];
  ff[(size_t)c * nq + q] = pair_prefactor(sp[ab.x], sp[ab.y], K[q],
                                          F[(size_t)fid[ab.x] * nq + q],
                                          F[(size_t)fid[ab.y] * nq + q]);
}

Error prefactor_upload(PrefState *st, const dbx_species *sp, int nsp,
                       const int2 *col_sp, int ncols, int nq,
                       cudaStream_t stream, size_t *delta) {
  const cudaStream_t as = st->alloc_stream;
  DBX_TRY(buf_grow(&st->sp, sizeof(SpeciesDev) * std::max(nsp, 1), delta, as));
  DBX_TRY(buf_grow(&st->colsp, sizeof(int2) * std::max(ncols, 1), delta, as));
  DBX_TRY(buf_grow(&st->f, sizeof(double) * std::max(nsp, 1) * (size_t)std::max(nq, 1),
                   delta, as));
  DBX_TRY(h2d_copy(st->sp.p, sp, sizeof(SpeciesDev) * nsp, stream, st->arena));
  DBX_TRY(h2d_copy(st->colsp.p, col_sp, sizeof(int2) * ncols, stream, st->arena));
  // species with equal form-factor coefficients (a, b, c) share one row of
  // F: a batch of many models holds few distinct elements
  std::vector<int> ids(2 * (size_t)std::max(nsp, 1), -1);  // fid, then rep
  int nu = 0;
  for (int i = 0; i < nsp; ++i) {
    int u = 0;
    for (; u < nu; ++u) {
      const dbx_species &r = sp[ids[nsp + u]];
      if (std::memcmp(r.a, sp[i].a, sizeof r.a) == 0 &&
          std::memcmp(r.b, sp[i].b, sizeof r.b) == 0 &&
          std::memcmp(&r.c, &sp[i].c, sizeof r.c) == 0)
        break;
    }
    if (u == nu) ids[nsp + nu++] = i;
    ids[i] = u;
  }
  DBX_TRY(buf_grow(&st->fid, sizeof(int) * ids.size(), delta, as));
  DBX_TRY(h2d_copy(st->fid.p, ids.data(), sizeof(int) * ids.size(), stream, st->arena));
  st->ncols = ncols;
  st->nsp = nsp;
  return ok();
}

Error prefactor_execute(const PrefState &st, const double *d_K, int nq,
                        double *d_ff, cudaStream_t stream) {
  if (st.f.bytes < sizeof(double) * std::max(st.nsp, 1) * (size_t)nq)
    return fail(DBX_ERR_ARG, "prefactor: q grid larger than prepared");
  // one block row per species; rows past the distinct sets return at once
  // (the launch shape does not depend on the coefficients, so a captured
  // graph stays valid when a re-score changes them)
  const int *fid = (const int *)st.fid.p;
  species_f_kernel<<<dim3((nq + 127) / 128, st.nsp), 128, 0, stream>>>(
      (const SpeciesDev *)st.sp.p, fid + st.nsp, d_K, nq, (double *)st.f.p);
  dim3 grid((nq + 127) / 128, st.ncols);
  prefactor_cols_kernel<<<grid, 128, 0, stream>>>(
      (const SpeciesDev *)st.sp.p, (const int2 *)st.colsp.p, fid, d_K, nq,
      (const double *)st.f.p, d_ff);
  DBX_CUDA_TRY(cudaGetLastError());
  return ok();
}

constexpr int kDirectThreads = 128;
constexpr int kDirectChunk = 128;  // bins staged per shared-memory round
constexpr int kDirectMaxPairs = 16;

template <typename T>
__device__ __forceinline__ T sinc_term(T kr);
template <>
__device__ __forceinline__ double sinc_term<double>(double kr) {
  return sin(kr) / kr;
}
template <>
__device__ __forceinline__ float sinc_term<float>(float kr) {
  return sinf(kr) / kr;
}

// I[q] += sum_{p < np} ff[p0+p][q] * sum_k m_kp sinc(K_q r_k).
template <typename T>
__global__ void __launch_bounds__(kDirectThreads)
    debye_direct_kernel(const unsigned long long *__restrict__ hist,
                        int p0, int np, long long pitch, int nbins,
                        double rstep, const double *__restrict__ K, int nq,
                        const double *__restrict__ ff, double *__restrict__ I) {
  __shared__ T s_m[kDirectMaxPairs][kDirectChunk];
  __shared__ T s_r[kDirectChunk];
  __shared__ int s_kind[kDirectChunk];  // 0 zero bin, 1 self (r<=0.0005), 2 sinc
  const int q = blockIdx.x * kDirectThreads + threadIdx.x;
  const T Kq = (T)K[q < nq ? q : nq - 1];
  T acc[kDirectMaxPairs];
#pragma unroll
  for (int p = 0; p < kDirectMaxPairs; ++p) acc[p] = 0;
  for (int k0 = 0; k0 < nbins; k0 += kDirectChunk) {
    __syncthreads();
    for (int i = threadIdx.x; i < kDirectChunk; i += kDirectThreads) {
      const int k = k0 + i;
      const double r = (double)k * rstep;  // r_reduced (cuDebye-v15.cu:735)
      int any = 0;
      for (int p = 0; p < np; ++p) {
        const unsigned long long n =
            k < nbins ? hist[(long long)(p0 + p) * pitch + k] : 0ull;
        any |= n != 0;
        // m = 2n off the self distance, n on it (cuDebye-v15.cu:508-514)
        s_m[p][i] = (T)(r > 0.0005 ? 2.0 * (double)n : (double)n);
      }
      s_r[i] = (T)r;
      s_kind[i] = any ? (r > 0.0005 ? 2 : 1) : 0;
    }
    __syncthreads();
    for (int i = 0; i < kDirectChunk; ++i) {
      const int kind = s_kind[i];
      if (kind == 0) continue;
      const T sc = kind == 2 ? sinc_term<T>(Kq * s_r[i]) : (T)1;
#pragma unroll
      for (int p = 0; p < kDirectMaxPairs; ++p)
        if (p < np) {
          const T m = s_m[p][i];
          if (m != (T)0) acc[p] += m * sc;
        }
    }
  }
  if (q < nq) {
    double s = I[q];
#pragma unroll
    for (int p = 0; p < kDirectMaxPairs; ++p)
      if (p < np) s += (double)acc[p] * ff[(size_t)(p0 + p) * nq + q];
    I[q] = s;
  }
}

Error debye_direct(int mode, const unsigned long long *d_hist, int npairs,
                   int64_t pitch, int64_t nbins, double rstep,
                   const double *d_K, int nq, const double *d_ff, double *d_I,
                   cudaStream_t stream) {
  DBX_CUDA_TRY(cudaMemsetAsync(d_I, 0, sizeof(double) * nq, stream));
  const int grid = (nq + kDirectThreads - 1) / kDirectThreads;
  for (int p0 = 0; p0 < npairs; p0 += kDirectMaxPairs) {
    const int np = std::min(kDirectMaxPairs, npairs - p0);
    if (mode == DBX_DEBYE_FP32)
      debye_direct_kernel<float><<<grid, kDirectThreads, 0, stream>>>(
          d_hist, p0, np, (long long)pitch, (int)nbins, rstep, d_K, nq, d_ff,
          d_I);
    else
      debye_direct_kernel<double><<<grid, kDirectThreads, 0, stream>>>(
          d_hist, p0, np, (long long)pitch, (int)nbins, rstep, d_K, nq, d_ff,
          d_I);
    DBX_CUDA_TRY(cudaGetLastError());
  }
  return ok();
}

}  // namespace dbx
