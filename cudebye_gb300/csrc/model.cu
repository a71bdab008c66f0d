// model.cu — resident models: spatial sort, tiles and device upload.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "curve.cuh"
#include "engine.h"

namespace dbx {

// One species: Hilbert order (curve.cuh) of its atoms on a grid over the
// species' bounding cube with about 2 cells per atom (16^3 to 1024^3 cells; stable
// LSD radix sort in passes of up to 11 bits, so atoms with equal codes keep
// their input order), written to atoms[start..start+n), and the bounding
// boxes of its tiles of kTile atoms. Any order gives the same histograms; a
// compact one gives tile pairs narrow distance ranges.
static void sort_species(const float *const xyz[3], int64_t start, int64_t n,
                         float4 *atoms, std::vector<TileBox> *boxes) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int d = 0; d < 3; ++d) {
    const float *v = xyz[d] + start;
    for (int64_t i = 0; i < n; ++i) {
      lo[d] = std::min(lo[d], v[i]);
      hi[d] = std::max(hi[d], v[i]);
    }
  }
  float ext = 0;
  for (int d = 0; d < 3; ++d) ext = std::max(ext, hi[d] - lo[d]);
  int bits = 4;
  while (bits < 10 && (int64_t(1) << (3 * bits)) < 2 * n) ++bits;
  const float top = (float)((1u << bits) - 1);
  const float scale = ext > 0 ? top / ext : 0.f;  // NaN extent: scale NaN, t 0
  std::vector<uint32_t> code(n), code2(n);
  std::vector<int32_t> idx(n), idx2(n);
  for (int64_t i = 0; i < n; ++i) {
    uint32_t q[3];
    for (int d = 0; d < 3; ++d) {
      float t = (xyz[d][start + i] - lo[d]) * scale;
      t = t >= 0.f ? (t <= top ? t : top) : 0.f;  // NaN -> 0
      q[d] = (uint32_t)t;
    }
    code[i] = hilbert3(q[0], q[1], q[2], bits);
    idx[i] = (int32_t)i;
  }
  const int total = 3 * bits;
  const int passes = (total + 10) / 11;
  const int width = (total + passes - 1) / passes;
  std::vector<int64_t> hist((size_t(1) << width) + 1);
  for (int shift = 0; shift < total; shift += width) {
    const uint32_t mask = (1u << width) - 1u;
    std::fill(hist.begin(), hist.end(), 0);
    for (int64_t i = 0; i < n; ++i) ++hist[((code[i] >> shift) & mask) + 1];
    for (size_t k = 0; k + 1 < hist.size(); ++k) hist[k + 1] += hist[k];
    for (int64_t i = 0; i < n; ++i) {
      const int64_t o = hist[(code[i] >> shift) & mask]++;
      code2[o] = code[i];
      idx2[o] = idx[i];
    }
    code.swap(code2);
    idx.swap(idx2);
  }
  for (int64_t i = 0; i < n; ++i) {
    const int64_t src = start + idx[i];
    atoms[start + i] = make_float4(xyz[0][src], xyz[1][src], xyz[2][src], 0.f);
  }
  boxes->clear();
  for (int64_t t0 = 0; t0 < n; t0 += kTile) {
    const int cnt = (int)std::min<int64_t>(kTile, n - t0);
    TileBox bx;
    bool nan = false;
    for (int q = 0; q < 4; ++q) {
      bool qnan = false;
      for (int d = 0; d < 3; ++d) {
        bx.qlo[q][d] = INFINITY;
        bx.qhi[q][d] = -INFINITY;
      }
      for (int i = q * kQuarter; i < std::min(cnt, (q + 1) * kQuarter); ++i) {
        const float4 a = atoms[start + t0 + i];
        const float v[3] = {a.x, a.y, a.z};
        for (int d = 0; d < 3; ++d) {
          qnan |= v[d] != v[d];
          bx.qlo[q][d] = std::min(bx.qlo[q][d], v[d]);
          bx.qhi[q][d] = std::max(bx.qhi[q][d], v[d]);
        }
      }
      if (qnan)  // a NaN atom's distances are unknown: the box says so
        for (int d = 0; d < 3; ++d) bx.qlo[q][d] = bx.qhi[q][d] = NAN;
      nan |= qnan;
    }
    for (int d = 0; d < 3; ++d) {
      bx.lo[d] = nan ? NAN : std::min({bx.qlo[0][d], bx.qlo[1][d], bx.qlo[2][d], bx.qlo[3][d]});
      bx.hi[d] = nan ? NAN : std::max({bx.qhi[0][d], bx.qhi[1][d], bx.qhi[2][d], bx.qhi[3][d]});
    }
    boxes->push_back(bx);
  }
}

Error model_prepare(const float *x, const float *y, const float *z,
                    const int64_t *counts, int nspecies, Model *m,
                    float4 *atoms) {
  if (!counts || nspecies < 1) return fail(DBX_ERR_ARG, "need >= 1 species");
  int64_t natoms = 0;
  for (int s = 0; s < nspecies; ++s) {
    if (counts[s] < 0) return fail(DBX_ERR_ARG, "negative species count");
    natoms += counts[s];
  }
  if (natoms > 0 && (!x || !y || !z)) return fail(DBX_ERR_ARG, "null coordinate array");
  if (natoms >= (int64_t(1) << 31)) return fail(DBX_ERR_ARG, "more than 2^31 atoms");
  m->nspecies = nspecies;
  m->natoms = natoms;
  const float *xyz[3] = {x, y, z};
  atoms[0] = make_float4(0, 0, 0, 0);
  std::vector<int64_t> start(nspecies + 1, 0);
  for (int s = 0; s < nspecies; ++s) start[s + 1] = start[s] + counts[s];
  std::vector<std::vector<TileBox>> boxes(nspecies);
  // species sort independently: large models use one host thread each
  if (natoms >= 65536 && nspecies > 1) {
    std::vector<std::thread> th;
    for (int s = 0; s < nspecies; ++s)
      if (counts[s] > 0)
        th.emplace_back(sort_species, xyz, start[s], counts[s], atoms, &boxes[s]);
    for (std::thread &t : th) t.join();
  } else {
    for (int s = 0; s < nspecies; ++s)
      if (counts[s] > 0) sort_species(xyz, start[s], counts[s], atoms, &boxes[s]);
  }
  m->tile_start.assign(1, 0);
  m->tiles.clear();
  m->boxes.clear();
  m->sp_start.clear();
  m->sp_count.clear();
  for (int s = 0; s < nspecies; ++s) {
    const int64_t n = counts[s];
    m->sp_start.push_back(start[s]);
    m->sp_count.push_back(n);
    for (int64_t t0 = 0; t0 < n; t0 += kTile)
      m->tiles.push_back(make_int2((int)(start[s] + t0),
                                   (int)std::min<int64_t>(kTile, n - t0)));
    m->boxes.insert(m->boxes.end(), boxes[s].begin(), boxes[s].end());
    m->tile_start.push_back((int)m->tiles.size());
  }
  return ok();
}

void *PinArena::take(size_t n) {
  n = (n + 15) & ~size_t(15);
  if (!chunks.empty() && used + n <= chunks.back().second) {
    void *p = chunks.back().first + used;
    used += n;
    return p;
  }
  size_t total = 0;
  for (auto &c : chunks) total += c.second;
  const size_t cap = std::max(n, std::max<size_t>(total, size_t(8) << 20));
  char *p = nullptr;
  if (cudaMallocHost((void **)&p, cap) != cudaSuccess) return nullptr;
  chunks.emplace_back(p, cap);
  used = n;
  return p;
}

void PinArena::reset() {
  if (chunks.size() > 1) {
    size_t total = 0;
    for (auto &c : chunks) total += c.second;
    release();
    char *p = nullptr;
    if (cudaMallocHost((void **)&p, total) == cudaSuccess) chunks.emplace_back(p, total);
  }
  used = 0;
}

void PinArena::release() {
  for (auto &c : chunks) cudaFreeHost(c.first);
  chunks.clear();
  used = 0;
}

Error h2d_copy(void *dst, const void *src, size_t n, cudaStream_t stream,
               PinArena *arena) {
  if (n == 0) return ok();
  const void *from = src;
  if (arena) {
    if (void *p = arena->take(n)) {
      std::memcpy(p, src, n);
      from = p;
    }
  }
  DBX_CUDA_TRY(cudaMemcpyAsync(dst, from, n, cudaMemcpyHostToDevice, stream));
  return ok();
}

Error buf_grow(DevBuf *b, size_t bytes, size_t *delta, cudaStream_t stream) {
  if (b->bytes >= bytes) return ok();
  if (b->p) {
    if (stream)
      cudaFreeAsync(b->p, stream);
    else
      cudaFree(b->p);
    *delta -= b->bytes;
    b->p = nullptr;
    b->bytes = 0;
  }
  if (stream)
    DBX_CUDA_TRY(cudaMallocAsync(&b->p, bytes, stream));
  else
    DBX_CUDA_TRY(cudaMalloc(&b->p, bytes));
  b->bytes = bytes;
  *delta += bytes;
  return ok();
}

size_t model_upload_bytes(const Model &m) {
  return sizeof(float4) * std::max<int64_t>(m.natoms, 1) +
         (sizeof(int2) + sizeof(TileBox)) * std::max<size_t>(m.tiles.size(), 1);
}

Error model_to_device(Model *m, const float4 *atoms, cudaStream_t stream,
                      PinArena *arena) {
  const size_t abytes = sizeof(float4) * std::max<int64_t>(m->natoms, 1);
  const size_t tbytes = sizeof(int2) * std::max<size_t>(m->tiles.size(), 1);
  // the tile boxes go to the device too: the histogram kernel reads them to
  // skip the out-of-range clamp of tile pairs that cannot reach it
  const size_t bbytes = sizeof(TileBox) * std::max<size_t>(m->tiles.size(), 1);
  // the arrays are allocated in the stream's order, without waiting for
  // other work on the device
  if (cudaMallocAsync(&m->d_atoms, abytes, stream) != cudaSuccess ||
      cudaMallocAsync(&m->d_tiles, tbytes, stream) != cudaSuccess ||
      cudaMallocAsync(&m->d_boxes, bbytes, stream) != cudaSuccess)
    return fail(DBX_ERR_NOMEM, "device allocation failed for model");
  m->dev_bytes = abytes + tbytes + bbytes;
  DBX_CUDA_TRY(cudaMemcpyAsync(m->d_atoms, atoms, abytes,
                               cudaMemcpyHostToDevice, stream));
  if (!m->tiles.empty())
    DBX_TRY(h2d_copy(m->d_tiles, m->tiles.data(), sizeof(int2) * m->tiles.size(),
                     stream, arena));
  if (m->boxes.size() == m->tiles.size() && !m->boxes.empty())
    DBX_TRY(h2d_copy(m->d_boxes, m->boxes.data(), sizeof(TileBox) * m->boxes.size(),
                     stream, arena));
  return ok();
}

size_t model_device_bytes(const Model &m) {
  return m.dev_bytes + m.hist_bytes + m.plan_bytes;
}

void model_release_async(Model *m, cudaStream_t stream) {
  for (void *p : {(void *)m->d_atoms, (void *)m->d_tiles, (void *)m->d_boxes,
                  (void *)m->d_hist})
    if (p) cudaFreeAsync(p, stream);
  m->d_atoms = nullptr;
  m->d_tiles = nullptr;
  m->d_boxes = nullptr;
  m->d_hist = nullptr;
  if (m->plan_cache) {
    for (DevBuf *b : {&m->plan_cache->lists.items, &m->plan_cache->lists.segs,
                      &m->plan_cache->lists.tasks, &m->plan_cache->lists.rows})
      if (b->p) {
        cudaFreeAsync(b->p, stream);
        b->p = nullptr;
      }
  }
  model_release(m);  // the host part of the plan cache
}

void model_release(Model *m) {
  if (m->d_atoms) cudaFree(m->d_atoms);
  if (m->d_tiles) cudaFree(m->d_tiles);
  if (m->d_boxes) cudaFree(m->d_boxes);
  if (m->d_hist) cudaFree(m->d_hist);
  if (m->plan_cache) {
    for (DevBuf *b : {&m->plan_cache->lists.items, &m->plan_cache->lists.segs,
                      &m->plan_cache->lists.tasks, &m->plan_cache->lists.rows})
      if (b->p) cudaFree(b->p);
    delete m->plan_cache;
    m->plan_cache = nullptr;
  }
  m->d_atoms = nullptr;
  m->d_tiles = nullptr;
  m->d_boxes = nullptr;
  m->d_hist = nullptr;
  m->dev_bytes = m->hist_bytes = m->plan_bytes = 0;
}

}  // namespace dbx
