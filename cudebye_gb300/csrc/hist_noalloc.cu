// hist_noalloc.cu — the pair histogram for callers that cannot allocate
// device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs
// inside another framework's memory pool or a fixed arena it must not grow,
// plugins loaded into a host process that owns every device allocation,
// and deployments where allocating on the device is forbidden once the
// service is up. dbx_pair_histogram_noalloc serves them: the caller passes
// device coordinates and a device output histogram, and every piece of
// scratch the computation needs lives in one file-scope __device__ array of
// fixed size (kNoAllocBytes = 64 MiB), which every GPU that loads this
// library holds until the process exits. The entry point calls no
// cudaMalloc, cudaFree or allocating library routine.
//
// The scratch array holds: a header (the work counter and the
// out-of-range count), one packed shared-memory window per CTA, and a
// float4 copy of the atoms. Requests needing more atoms than fit
// (kNoAllocMaxAtoms) are rejected with DBX_ERR_LIMIT.
//
// Every call shares the one array and leaves its contents behind; each call
// clears the parts that must start at zero. Calls that overlap on the GPU
// (two host threads, or two streams without ordering between them) race on
// the array and give wrong results; the caller must order them.
//
// On the first call on a device, that device current, the entry point looks
// up the array's device address with cudaGetSymbolAddress (a host-side
// name of a __device__ array is not a device address). That first call
// should therefore come before any stream capture. Every call waits for its
// stream to finish the call's work before it returns (it reads back the
// out-of-range count), so it blocks the calling host thread.
//
// A range paired with itself is recognised by equal starts, as the
// reference's splitCalcDist does (cuDebye-v15.cu:241); equal starts with
// different counts name no species block and are rejected.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "../../include/cudebye.h"
#include "hist_device.cuh"

namespace dbx {
namespace {

constexpr size_t kNoAllocBytes = 64ull << 20;          // the whole array
constexpr size_t kHeaderBytes = 256;                   // counters
constexpr size_t kWindowRegion = 36ull << 20;          // CTA windows
constexpr size_t kAtomRegion = kNoAllocBytes - kHeaderBytes - kWindowRegion;
constexpr int64_t kNoAllocMaxAtoms = (int64_t)(kAtomRegion / sizeof(float4));
constexpr int kThreads = 512;
constexpr int kSmemBytes = 224 * 1024;
constexpr int kWindowBins = (kSmemBytes / 4) * 2;
constexpr int kTileAtoms = 128;

static __device__ __align__(256) unsigned char g_scratch[kNoAllocBytes];

struct Header {
  int next_item;
  int pad;
  unsigned long long oor;
};

// One slot per device: the array's device address, looked up once.
struct Slot {
  bool ready = false;
  unsigned char *ptr = nullptr;
};
constexpr int kMaxDevices = 64;
Slot g_slots[kMaxDevices];
std::mutex g_slots_mu;

__global__ void pack_kernel(const float *__restrict__ x,
                            const float *__restrict__ y,
                            const float *__restrict__ z, long long a0,
                            long long na, long long b0, long long nb,
                            float4 *__restrict__ atoms) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= na + nb) return;
  const long long src = i < na ? a0 + i : b0 + (i - na);
  atoms[i] = make_float4(x[src], y[src], z[src], 0.f);
}

// Tile pair of a flat item index: all (I, J) for two blocks, or I <= J
// (J-major triangle) for a block with itself.
__device__ __forceinline__ void item_tiles(int idx, int tI, int tJ, bool diag,
                                           int &I, int &J) {
  if (!diag) {
    I = idx / tJ;
    J = idx % tJ;
    return;
  }
  int j = (int)((sqrt(8.0 * idx + 1.0) - 1.0) * 0.5);
  while ((long long)j * (j + 1) / 2 > idx) --j;
  while ((long long)(j + 1) * (j + 2) / 2 <= idx) ++j;
  J = j;
  I = idx - j * (j + 1) / 2;
}

// wrap16 with the bins at or beyond `lim` skipped (the caller's histogram
// has no padding; a carry into the high half past its end is dropped with
// that half).
__device__ __forceinline__ void wrap16_lim(unsigned old, unsigned lk,
                                           unsigned lim,
                                           unsigned long long *gh) {
  const unsigned sh16 = (lk & 1u) << 4;
  if (((old >> sh16) & 0xFFFFu) == 0xFFFFu) {
    atomicAdd(&gh[lk], 65536ull);
    if (sh16 == 0 && lk + 1 < lim) {
      atomicAdd(&gh[lk + 1], ~0ull);
      if ((old >> 16) == 0xFFFFu) atomicAdd(&gh[lk + 1], 65536ull);
    }
  }
}

// One window [kb, kb+wl) of the histogram of atoms [0, na) against
// [na, na+nb) (or [0, na) with itself when diag). Warps take tile pairs from
// the work counter; each CTA keeps its window in shared memory and writes it
// to its slot in the windows region at the end.
__global__ void __launch_bounds__(kThreads, 1)
    noalloc_tiles_kernel(const float4 *__restrict__ atoms, int na, int nb,
                         bool diag, int kb, int wl, unsigned nbins, float inv,
                         Header *__restrict__ hdr,
                         unsigned *__restrict__ windows, int words,
                         unsigned long long *__restrict__ out) {
  extern __shared__ unsigned sh[];
  const int lane = threadIdx.x & 31;
  const int nw = (wl + 1) >> 1;
  for (int i = threadIdx.x; i < nw; i += kThreads) sh[i] = 0u;
  __syncthreads();
  const int tI = (na + kTileAtoms - 1) / kTileAtoms;
  const int tJ = diag ? tI : (nb + kTileAtoms - 1) / kTileAtoms;
  const int nitems = diag ? tI * (tI + 1) / 2 : tI * tJ;
  const float4 *bbase = diag ? atoms : atoms + na;
  const int nJ = diag ? na : nb;
  unsigned long long *gh = out + kb;
  const unsigned lim = nbins - (unsigned)kb;
  const unsigned base = 0x4B000000u + (unsigned)kb;
  const f2 ninv = pk(-2.0f * inv, -2.0f * inv);  // bins2 takes -2 inv
  unsigned my_oor = 0;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(&hdr->next_item, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= nitems) break;
    int I, J;
    item_tiles(idx, tI, tJ, diag, I, J);
    const int i0 = I * kTileAtoms, ni = min(kTileAtoms, na - i0);
    const int j0 = J * kTileAtoms, nj = min(kTileAtoms, nJ - j0);
    const bool dtile = diag && I == J;
    float x[4], y[4], z[4];
    int jlim[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int pi = lane + 32 * r;
      const bool act = pi < ni;
      const float4 a = atoms[i0 + (act ? pi : 0)];
      x[r] = a.x;
      y[r] = a.y;
      z[r] = a.z;
      jlim[r] = act ? (dtile ? pi : 0x7fffffff) : -1;
    }
    const float4 *bj = bbase + j0;
#pragma unroll 2
    for (int j = 0; j < nj; ++j) {
      const float4 b = bj[j];
      unsigned old[4], lk[4];
      bins2(x[0], x[1], y[0], y[1], z[0], z[1], b.x, b.x, b.y, b.y, b.z, b.z, ninv, base,
            lk[0], lk[1]);
      bins2(x[2], x[3], y[2], y[3], z[2], z[3], b.x, b.x, b.y, b.y, b.z, b.z, ninv, base,
            lk[2], lk[3]);
      bool hit[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const bool valid = j <= jlim[r];
        hit[r] = valid && lk[r] < (unsigned)wl;
        my_oor += (valid && !hit[r] && lk[r] + (unsigned)kb >= nbins) ? 1u : 0u;
        old[r] = hit[r] ? atomicAdd(&sh[lk[r] >> 1], (lk[r] & 1u) ? 0x10000u : 1u)
                        : 0u;
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
        if (hit[r]) wrap16_lim(old[r], lk[r], lim, gh);
    }
  }
  my_oor = __reduce_add_sync(0xffffffffu, my_oor);
  if (lane == 0 && my_oor) atomicAdd(&hdr->oor, (unsigned long long)my_oor);
  __syncthreads();
  unsigned *dst = windows + (size_t)blockIdx.x * words;
  for (int i = threadIdx.x; i < nw; i += kThreads) dst[i] = sh[i];
}

// out[kb + b] += sum over the CTA windows, for bins below nbins.
__global__ void noalloc_reduce_kernel(const unsigned *__restrict__ windows,
                                      int nslots, int words, int kb, int wl,
                                      long long nbins,
                                      unsigned long long *__restrict__ out) {
  const int nw = (wl + 1) >> 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw;
       i += gridDim.x * blockDim.x) {
    unsigned long long lo = 0, hi = 0;
    for (int s = 0; s < nslots; ++s) {
      const unsigned w = windows[(size_t)s * words + i];
      lo += w & 0xFFFFu;
      hi += w >> 16;
    }
    const long long b = (long long)kb + 2 * i;
    if (b < nbins) out[b] += lo;
    if (b + 1 < nbins) out[b + 1] += hi;
  }
}

int setup(int dev, unsigned char **ptr) {
  if (dev < 0 || dev >= kMaxDevices) return DBX_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_slots_mu);
  if (!g_slots[dev].ready) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p)
      return DBX_ERR_CUDA;
    g_slots[dev].ptr = static_cast<unsigned char *>(p);
    g_slots[dev].ready = true;
  }
  *ptr = g_slots[dev].ptr;
  return DBX_OK;
}

}  // namespace
}  // namespace dbx

static_assert(dbx::kNoAllocMaxAtoms == DBX_NOALLOC_MAX_ATOMS,
              "DBX_NOALLOC_MAX_ATOMS must match the scratch layout");

extern "C" int dbx_pair_histogram_noalloc(const float *x, const float *y,
                                          const float *z, int64_t a_start,
                                          int64_t a_count, int64_t b_start,
                                          int64_t b_count, double rstep,
                                          int64_t nbins, int64_t *out,
                                          void *stream) {
  using namespace dbx;
  if (!x || !y || !z || !out || a_start < 0 || b_start < 0 || a_count < 0 ||
      b_count < 0 || !(rstep > 0) || nbins < 1 || nbins > (int64_t(1) << 22))
    return DBX_ERR_ARG;
  // The reference's `dist` kernel serves a block paired with itself, chosen
  // by equal starts (cuDebye-v15.cu:241-243): pairs j <= i including i == j.
  const bool diag = a_start == b_start;
  if (diag && a_count != b_count) return DBX_ERR_ARG;
  // each count alone first, so that the sum below cannot overflow
  if (a_count > kNoAllocMaxAtoms || b_count > kNoAllocMaxAtoms) return DBX_ERR_LIMIT;
  const int64_t natoms = diag ? a_count : a_count + b_count;
  if (natoms > kNoAllocMaxAtoms) return DBX_ERR_LIMIT;
  // index ranges must fit the 64-bit arithmetic of pack_kernel
  if (a_start > INT64_MAX - a_count || b_start > INT64_MAX - b_count)
    return DBX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DBX_ERR_CUDA;
  // The scratch address below is the current device's; a stream of another
  // device is refused (the legacy default stream, NULL, is the current
  // device's).
  if (s) {
    int sdev = -1;
    if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) return DBX_ERR_CUDA;
    if (sdev != dev) return DBX_ERR_ARG;
  }
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) !=
      cudaSuccess)
    return DBX_ERR_CUDA;
  unsigned char *base = nullptr;
  int rc = setup(dev, &base);
  if (rc) return rc;
  Header *hdr = reinterpret_cast<Header *>(base);
  unsigned *windows = reinterpret_cast<unsigned *>(base + kHeaderBytes);
  float4 *atoms = reinterpret_cast<float4 *>(base + kHeaderBytes + kWindowRegion);
  if (cudaMemsetAsync(hdr, 0, sizeof(Header), s) != cudaSuccess ||
      cudaMemsetAsync(out, 0, sizeof(int64_t) * nbins, s) != cudaSuccess)
    return DBX_ERR_CUDA;
  if (a_count == 0 || b_count == 0) return cudaStreamSynchronize(s) ? DBX_ERR_CUDA : DBX_OK;
  pack_kernel<<<(unsigned)((natoms + 255) / 256), 256, 0, s>>>(
      x, y, z, a_start, a_count, b_start, diag ? 0 : b_count, atoms);
  if (cudaFuncSetAttribute(noalloc_tiles_kernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kSmemBytes) != cudaSuccess)
    return DBX_ERR_CUDA;
  const float inv = (float)(1.0 / rstep);  // cuDebye-v15.cu:739
  for (int64_t kb = 0; kb < nbins; kb += kWindowBins) {
    const int wl = (int)std::min<int64_t>(kWindowBins, nbins - kb);
    const int words = (wl + 1) / 2;
    const int grid = (int)std::max<int64_t>(
        1, std::min<int64_t>(nsm, kWindowRegion / ((size_t)words * 4)));
    if (cudaMemsetAsync(&hdr->next_item, 0, sizeof(int), s) != cudaSuccess)
      return DBX_ERR_CUDA;
    noalloc_tiles_kernel<<<grid, kThreads, words * 4, s>>>(
        atoms, (int)a_count, (int)(diag ? a_count : b_count), diag, (int)kb, wl,
        (unsigned)nbins, inv, hdr, windows, words,
        reinterpret_cast<unsigned long long *>(out));
    noalloc_reduce_kernel<<<(words + 255) / 256, 256, 0, s>>>(
        windows, grid, words, (int)kb, wl, nbins,
        reinterpret_cast<unsigned long long *>(out));
  }
  if (cudaGetLastError() != cudaSuccess) return DBX_ERR_CUDA;
  unsigned long long oor = 0;
  if (cudaMemcpyAsync(&oor, &hdr->oor, sizeof(oor), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return DBX_ERR_CUDA;
  return oor ? DBX_ERR_RANGE : DBX_OK;
}
