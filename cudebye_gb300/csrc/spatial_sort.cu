// spatial_sort.cu — the spatial sort of a model's atoms on the device.
//
// The same order as the host path (model_prepare): per species, Hilbert
// indices (curve.cuh) on a grid over the species' bounding cube with about 2 cells per
// atom, sorted stably (equal codes keep their input order), so a model
// uploaded either way has the same atoms, tiles and boxes. Used by
// dbx_model_upload for large models, where the host sort would dominate
// the upload: raw coordinates go to the device once and the codes, the
// radix sort (LSD, 8-bit digits, stable), the gather into float4 atoms and
// the tile bounding boxes run there.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "curve.cuh"
#include "engine.h"

namespace dbx {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortChunk = 4096;  // keys per block and pass (16 per thread)
constexpr int kRadix = 256;

// Species of global atom index i (species ranges start[0..ns]).
__device__ __forceinline__ int species_of(long long i, const long long *start,
                                          int ns) {
  int s = 0;
  while (s + 1 < ns && i >= start[s + 1]) ++s;
  return s;
}

// Per species, per block: min and max of x, y, z over the block's share;
// combined by atomics on order-preserving integer images of the floats
// (NaN coordinates are skipped, as std::min / std::max skip them on the
// host when the running value comes first).
__device__ __forceinline__ unsigned f2ord(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

__global__ void bbox_kernel(const float *__restrict__ xyz, long long n,
                            const long long *__restrict__ start, int ns,
                            unsigned *__restrict__ lohi /* [ns][6] */) {
  const int s = blockIdx.y;
  const long long b = start[s], e = start[s + 1];
  unsigned lo[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, hi[3] = {0u, 0u, 0u};
  for (long long i = b + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < e;
       i += (long long)gridDim.x * blockDim.x) {
    for (int d = 0; d < 3; ++d) {
      const float v = xyz[d * n + i];
      if (v != v) continue;  // NaN
      const unsigned o = f2ord(v);
      lo[d] = min(lo[d], o);
      hi[d] = max(hi[d], o);
    }
  }
  for (int d = 0; d < 3; ++d) {
    for (int off = 16; off > 0; off >>= 1) {
      lo[d] = min(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
      hi[d] = max(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&lohi[s * 6 + d], lo[d]);
      atomicMax(&lohi[s * 6 + 3 + d], hi[d]);
    }
  }
}

// Sort key of every atom: bits code_shift.. the species, bits below the
// code computed exactly as the host does (FP32, IEEE operations), so the
// radix passes cover the code's bits and the species' bits with no gap.
__global__ void keys_kernel(const float *__restrict__ xyz, long long n,
                            const long long *__restrict__ start, int ns,
                            const unsigned *__restrict__ lohi,
                            const int *__restrict__ bits, int code_shift,
                            unsigned long long *__restrict__ key,
                            int *__restrict__ idx) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = species_of(i, start, ns);
  float lo[3], ext = 0.f;
  for (int d = 0; d < 3; ++d) {
    const unsigned l = lohi[s * 6 + d], h = lohi[s * 6 + 3 + d];
    // an all-NaN axis has no extent (the host's running min stays +inf)
    lo[d] = l == 0xFFFFFFFFu ? INFINITY : ord2f(l);
    const float hv = h == 0u ? -INFINITY : ord2f(h);
    ext = fmaxf(ext, __fsub_rn(hv, lo[d]));
  }
  const float top = (float)((1u << bits[s]) - 1);
  const float scale = ext > 0 ? __fdiv_rn(top, ext) : 0.f;
  uint32_t q[3];
  for (int d = 0; d < 3; ++d) {
    float t = __fmul_rn(__fsub_rn(xyz[d * n + i], lo[d]), scale);
    t = t >= 0.f ? (t <= top ? t : top) : 0.f;  // NaN -> 0
    q[d] = (uint32_t)t;
  }
  const uint32_t code = hilbert3(q[0], q[1], q[2], bits[s]);
  key[i] = ((unsigned long long)s << code_shift) | code;
  idx[i] = (int)(i - start[s]);
}

// Digit counts of each block's chunk: cnt[digit * nblocks + block].
__global__ void radix_count_kernel(const unsigned long long *__restrict__ key,
                                   long long n, int shift,
                                   unsigned *__restrict__ cnt) {
  __shared__ unsigned h[kRadix];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kSortChunk;
  for (int k = threadIdx.x; k < kSortChunk; k += kSortThreads) {
    const long long i = base + k;
    if (i < n) atomicAdd(&h[(key[i] >> shift) & 0xFF], 1u);
  }
  __syncthreads();
  cnt[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive prefix sum of m counts in place (one block).
__global__ void radix_scan_kernel(unsigned *__restrict__ cnt, long long m) {
  __shared__ unsigned long long part[1024];
  const int t = threadIdx.x;
  const long long per = (m + blockDim.x - 1) / blockDim.x;
  const long long b = t * per, e = b + per < m ? b + per : m;
  unsigned long long s = 0;
  for (long long i = b; i < e; ++i) s += cnt[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < (int)blockDim.x; off <<= 1) {
    const unsigned long long v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  unsigned long long acc = part[t] - s;  // exclusive
  for (long long i = b; i < e; ++i) {
    const unsigned c = cnt[i];
    cnt[i] = (unsigned)acc;
    acc += c;
  }
}

// Stable scatter of each block's chunk: warp w takes its 512 keys in
// order, 32 at a time; lanes with equal digits are ranked by lane, and the
// warps' offsets per digit follow the warps' order.
__global__ void radix_scatter_kernel(const unsigned long long *__restrict__ key,
                                     const int *__restrict__ idx, long long n,
                                     int shift, const unsigned *__restrict__ cnt,
                                     unsigned long long *__restrict__ key2,
                                     int *__restrict__ idx2) {
  constexpr int kWarps = kSortThreads / 32;
  constexpr int kPerWarp = kSortChunk / kWarps;
  __shared__ unsigned wh[kWarps][kRadix];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < kWarps * kRadix; i += kSortThreads)
    (&wh[0][0])[i] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kSortChunk + warp * kPerWarp;
  for (int k = lane; k < kPerWarp; k += 32) {
    const long long i = base + k;
    if (i < n) atomicAdd(&wh[warp][(key[i] >> shift) & 0xFF], 1u);
  }
  __syncthreads();
  // offsets: global offset of (digit, block) + counts of earlier warps
  {
    const int d = threadIdx.x;  // kSortThreads == kRadix
    unsigned off = cnt[(size_t)d * gridDim.x + blockIdx.x];
    for (int w = 0; w < kWarps; ++w) {
      const unsigned c = wh[w][d];
      wh[w][d] = off;
      off += c;
    }
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  for (int k0 = 0; k0 < kPerWarp; k0 += 32) {
    const long long i = base + k0 + lane;
    const bool valid = i < n;
    // invalid lanes get a digit of their own (256 + lane): no peers
    const unsigned dig = valid ? (unsigned)((key[i] >> shift) & 0xFF) : 256u + lane;
    const unsigned peers = __match_any_sync(0xffffffffu, dig);
    const unsigned rank = __popc(peers & lt);
    unsigned pos = 0;
    if (valid) pos = wh[warp][dig] + rank;
    __syncwarp();
    if (valid) {
      key2[pos] = key[i];
      idx2[pos] = idx[i];
      if (rank == 0) wh[warp][dig] += __popc(peers);
    }
    __syncwarp();
  }
}

// atoms[j] = (x, y, z, 0) of the j-th sorted atom (idx: within species).
__global__ void gather_kernel(const float *__restrict__ xyz, long long n,
                              const long long *__restrict__ start, int ns,
                              const unsigned long long *__restrict__ key,
                              int code_shift, const int *__restrict__ idx,
                              float4 *__restrict__ atoms) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int s = (int)(key[j] >> code_shift);
  const long long src = start[s] + idx[j];
  atoms[j] = make_float4(xyz[src], xyz[n + src], xyz[2 * n + src], 0.f);
}

// Bounding box of every tile and of its column quarters (one warp per
// tile, one quarter of 32 atoms per pass; tiles {first, count}), as the
// host computes them.
__global__ void tile_boxes_kernel(const float4 *__restrict__ atoms,
                                  const int2 *__restrict__ tiles, int ntiles,
                                  TileBox *__restrict__ boxes) {
  const int t = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= ntiles) return;
  const int2 tl = tiles[t];
  TileBox b;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  bool nan = false;
  for (int q = 0; q < 4; ++q) {
    const int i = q * kQuarter + lane;
    float ql[3] = {INFINITY, INFINITY, INFINITY}, qh[3] = {-INFINITY, -INFINITY, -INFINITY};
    bool qn = false;
    if (i < tl.y) {
      const float4 a = atoms[tl.x + i];
      const float v[3] = {a.x, a.y, a.z};
      for (int d = 0; d < 3; ++d) {
        qn |= v[d] != v[d];
        ql[d] = fminf(ql[d], v[d]);
        qh[d] = fmaxf(qh[d], v[d]);
      }
    }
    qn = __any_sync(0xffffffffu, qn);
    for (int d = 0; d < 3; ++d) {
      for (int off = 16; off > 0; off >>= 1) {
        ql[d] = fminf(ql[d], __shfl_xor_sync(0xffffffffu, ql[d], off));
        qh[d] = fmaxf(qh[d], __shfl_xor_sync(0xffffffffu, qh[d], off));
      }
      b.qlo[q][d] = qn ? NAN : ql[d];  // a NaN atom gets a NaN box, as on the host
      b.qhi[q][d] = qn ? NAN : qh[d];
      lo[d] = fminf(lo[d], ql[d]);
      hi[d] = fmaxf(hi[d], qh[d]);
    }
    nan |= qn;
  }
  if (lane == 0) {
    for (int d = 0; d < 3; ++d) {
      b.lo[d] = nan ? NAN : lo[d];
      b.hi[d] = nan ? NAN : hi[d];
    }
    boxes[t] = b;
  }
}

}  // namespace

// Interleaved coordinates [n][3] to the SoA planes x[], y[], z[] the sort
// kernels read.
__global__ void deinterleave_kernel(const float *__restrict__ aos, long long n,
                                    float *__restrict__ soa) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  soa[i] = aos[3 * i];
  soa[n + i] = aos[3 * i + 1];
  soa[2 * n + i] = aos[3 * i + 2];
}

Error model_upload_sorted(Model *m, const float *x, const float *y, const float *z,
                          const float *xyz, const int64_t *counts, int nspecies,
                          float *pin, size_t pin_bytes, cudaStream_t st) {
  int64_t natoms = 0;
  for (int s = 0; s < nspecies; ++s) natoms += counts[s];
  const long long n = natoms;
  m->nspecies = nspecies;
  m->natoms = natoms;
  std::vector<long long> start(nspecies + 1, 0);
  std::vector<int> bits(nspecies);
  for (int s = 0; s < nspecies; ++s) {
    start[s + 1] = start[s] + counts[s];
    int b = 4;  // the host's grid: about 2 cells per atom, 16^3 to 1024^3
    while (b < 10 && (int64_t(1) << (3 * b)) < 2 * counts[s]) ++b;
    bits[s] = b;
  }
  m->tile_start.assign(1, 0);
  m->tiles.clear();
  m->boxes.clear();  // on the device; copied to the host when a plan needs them
  m->sp_start.clear();
  m->sp_count.clear();
  for (int s = 0; s < nspecies; ++s) {
    m->sp_start.push_back(start[s]);
    m->sp_count.push_back(counts[s]);
    for (int64_t t0 = 0; t0 < counts[s]; t0 += kTile)
      m->tiles.push_back(make_int2((int)(start[s] + t0),
                                   (int)std::min<int64_t>(kTile, counts[s] - t0)));
    m->tile_start.push_back((int)m->tiles.size());
  }
  const int ntiles = (int)m->tiles.size();
  const size_t abytes = sizeof(float4) * n, tbytes = sizeof(int2) * std::max(ntiles, 1),
               bbytes = sizeof(TileBox) * std::max(ntiles, 1);
  const long long nblk = (n + kSortChunk - 1) / kSortChunk;
  float *d_xyz = nullptr, *d_aos = nullptr;
  unsigned long long *k1 = nullptr, *k2 = nullptr;
  int *i1 = nullptr, *i2 = nullptr;
  unsigned *cnt = nullptr, *lohi = nullptr;
  long long *d_start = nullptr;
  int *d_bits = nullptr;
  auto cleanup = [&] {
    for (void *p : {(void *)d_xyz, (void *)d_aos, (void *)k1, (void *)k2, (void *)i1,
                    (void *)i2, (void *)cnt, (void *)lohi, (void *)d_start,
                    (void *)d_bits})
      if (p) cudaFreeAsync(p, st);
  };
  cudaError_t e = cudaSuccess;
  auto A = [&](void **p, size_t b) {
    if (e == cudaSuccess) e = cudaMallocAsync(p, b, st);
  };
  A((void **)&d_xyz, sizeof(float) * 3 * n);
  if (xyz) A((void **)&d_aos, sizeof(float) * 3 * n);
  A((void **)&k1, 8 * n);
  A((void **)&k2, 8 * n);
  A((void **)&i1, 4 * n);
  A((void **)&i2, 4 * n);
  A((void **)&cnt, sizeof(unsigned) * kRadix * nblk);
  A((void **)&lohi, sizeof(unsigned) * 6 * nspecies);
  A((void **)&d_start, sizeof(long long) * (nspecies + 1));
  A((void **)&d_bits, sizeof(int) * nspecies);
  // the model's arrays in the stream's order too (no device-wide wait)
  if (e == cudaSuccess && cudaMallocAsync(&m->d_atoms, abytes, st) != cudaSuccess)
    e = cudaErrorMemoryAllocation;
  if (e == cudaSuccess && cudaMallocAsync(&m->d_tiles, tbytes, st) != cudaSuccess)
    e = cudaErrorMemoryAllocation;
  if (e == cudaSuccess && cudaMallocAsync(&m->d_boxes, bbytes, st) != cudaSuccess)
    e = cudaErrorMemoryAllocation;
  if (e != cudaSuccess) {
    cleanup();
    return fail(DBX_ERR_NOMEM, "device allocation failed for model");
  }
  m->dev_bytes = abytes + tbytes + bbytes;
  std::vector<unsigned> lohi0(6 * nspecies);
  for (int s = 0; s < nspecies; ++s)
    for (int d = 0; d < 3; ++d) {
      lohi0[s * 6 + d] = 0xFFFFFFFFu;
      lohi0[s * 6 + 3 + d] = 0u;
    }
  // Raw coordinates through the pinned staging (3n floats), as given: SoA
  // planes, or one interleaved array de-interleaved on the device. They are
  // staged in pieces, each piece's copy queued as soon as it is staged, so
  // the transfer overlaps the staging of the rest.
  const long long nf = 3 * n;
  const long long piece = std::max<long long>(1 << 16, (nf + 3) / 4);
  float *dst = xyz ? d_aos : d_xyz;
  for (long long a = 0; a < nf && e == cudaSuccess; a += piece) {
    const long long b = std::min(nf, a + piece);
    if (xyz) {
      std::memcpy(pin + a, xyz + a, sizeof(float) * (b - a));
    } else {  // the planes end to end: x, y, z
      for (long long i = a; i < b;) {
        const int plane = (int)(i / n);
        const long long j = std::min(b, (long long)(plane + 1) * n);
        const float *src = plane == 0 ? x : (plane == 1 ? y : z);
        std::memcpy(pin + i, src + (i - plane * n), sizeof(float) * (j - i));
        i = j;
      }
    }
    e = cudaMemcpyAsync(dst + a, pin + a, sizeof(float) * (b - a),
                        cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess && xyz) {
    deinterleave_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_aos, n, d_xyz);
    e = cudaGetLastError();
  }
  // The small arrays through the rest of the staging, after the
  // coordinates, where they fit: a copy from pageable memory could wait for
  // the stream.
  {
    char *tail = reinterpret_cast<char *>(pin) + ((12 * n + 15) & ~15LL);
    char *const end = reinterpret_cast<char *>(pin) + pin_bytes;
    auto put = [&](void *d, const void *h, size_t bytes) {
      if (e != cudaSuccess || bytes == 0) return;
      const void *from = h;
      if (tail + bytes <= end) {
        std::memcpy(tail, h, bytes);
        from = tail;
        tail += (bytes + 15) & ~size_t(15);
      }
      e = cudaMemcpyAsync(d, from, bytes, cudaMemcpyHostToDevice, st);
    };
    put(lohi, lohi0.data(), sizeof(unsigned) * lohi0.size());
    put(d_start, start.data(), sizeof(long long) * start.size());
    put(d_bits, bits.data(), sizeof(int) * nspecies);
    put(m->d_tiles, m->tiles.data(), sizeof(int2) * ntiles);
  }
  if (e == cudaSuccess) {
    const unsigned g = (unsigned)((n + 255) / 256);
    bbox_kernel<<<dim3(std::min<unsigned>(g, 64u), nspecies), 256, 0, st>>>(
        d_xyz, n, d_start, nspecies, lohi);
    // digits over the code bits and the species bits above them (a stable
    // LSD sort: species-major, code order within, ties in input order);
    // the species share the code's last digit where it has room
    int code_bits = 0;
    for (int b : bits) code_bits = std::max(code_bits, 3 * b);
    int sp_bits = 0;
    while ((1 << sp_bits) < nspecies) ++sp_bits;
    keys_kernel<<<g, 256, 0, st>>>(d_xyz, n, d_start, nspecies, lohi, d_bits, code_bits,
                                   k1, i1);
    std::vector<int> shifts;
    for (int sh = 0; sh < code_bits + sp_bits; sh += 8) shifts.push_back(sh);
    for (int sh : shifts) {
      radix_count_kernel<<<(unsigned)nblk, kSortThreads, 0, st>>>(k1, n, sh, cnt);
      radix_scan_kernel<<<1, 1024, 0, st>>>(cnt, (long long)kRadix * nblk);
      radix_scatter_kernel<<<(unsigned)nblk, kSortThreads, 0, st>>>(k1, i1, n, sh, cnt,
                                                                  k2, i2);
      std::swap(k1, k2);
      std::swap(i1, i2);
    }
    gather_kernel<<<g, 256, 0, st>>>(d_xyz, n, d_start, nspecies, k1, code_bits, i1,
                                     m->d_atoms);
    tile_boxes_kernel<<<(unsigned)((ntiles * 32LL + 255) / 256), 256, 0, st>>>(
        m->d_atoms, m->d_tiles, ntiles, m->d_boxes);
    e = cudaGetLastError();
  }
  cleanup();
  if (e != cudaSuccess) return fail(DBX_ERR_CUDA, std::string("device sort: ") +
                                                      cudaGetErrorString(e));
  return ok();
}

Error model_host_boxes(Model *m, cudaStream_t st) {
  if (m->boxes.size() == m->tiles.size()) return ok();
  if (!m->d_boxes) return fail(DBX_ERR_ARG, "model has no tile boxes");
  m->boxes.resize(m->tiles.size());
  DBX_CUDA_TRY(cudaMemcpyAsync(m->boxes.data(), m->d_boxes,
                               sizeof(TileBox) * m->tiles.size(),
                               cudaMemcpyDeviceToHost, st));
  DBX_CUDA_TRY(cudaStreamSynchronize(st));
  return ok();
}

}  // namespace dbx
