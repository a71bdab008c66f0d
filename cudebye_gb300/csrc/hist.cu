// hist.cu — all-pairs distance histogram on sm_103a (hot path 1).
//
// Replaces the reference's splitCalcDist and its kernels dist / dist2 /
// care_dist2 (cuDebye-v15.cu:88-272), which bin every pair with a global
// uint32 atomicAdd and synchronise the host after every 67M-pair launch.
//
// Design:
//  * Atoms of each species are sorted along a Hilbert curve and cut into
//    tiles of 128 (model.cu, spatial_sort.cu); a work item is one tile pair,
//    or one 32-row quarter of it (listed for multi-window histograms and
//    small plans).
//  * A CTA owns a window of up to ~114k bins held in shared memory as packed
//    16-bit counters (two bins per 32-bit word). A counter that wraps is
//    detected from the atomic's return value and compensated exactly in the
//    int64 global histogram (wrap_fix), so the counts stay exact.
//  * Tile pairs are grouped into (species pair, bin window) segments from
//    their bounding boxes, and split into equal CTA tasks. Each task writes
//    its packed window once to a scratch slot; a reduce kernel sums the slots
//    of a segment into the int64 histogram. No host round trip between tiles.
//  * The distance and bin are the reference's FP32 formula, unfused
//    (cuDebye-v15.cu:101-107): IEEE sqrt, explicit _rn intrinsics so that
//    nothing is contracted to FMA, and roundf computed exactly without a
//    float->int conversion (bin_rel).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>

#include "engine.h"
#include "hist_device.cuh"

namespace dbx {

constexpr int kHistThreads = 1024;
// Dynamic shared memory per CTA: the window (224 KB of packed counters) and
// 64 lane-private spare words; 1 CTA per SM.
constexpr int kWindowBins = (224 * 1024 / 4) * 2;  // 114688, even
constexpr int kSpareWords = 64;
constexpr int kHistSmemBytes = (kWindowBins / 2 + kSpareWords) * 4;

int hist_window_bins() { return kWindowBins; }

// Wrap compensation of one add whose 16-bit half went from 0xFFFF to 0.
// v is the add's virtual bin: v < wl a bin of the window; wl <= v < vend a
// half of an out-of-range counter (the spare words after the window, and
// bin wl itself when wl is odd); v >= vend an ignore word (not counted).
// The count of virtual bin v is its stored half + 65536 per wrap - 1 per
// carry received from the low half of its word; compensations of bins go
// to the global histogram, those of out-of-range counters to oor_total.
__device__ __forceinline__ void wrap_fix(unsigned old, unsigned v, unsigned wl,
                                         unsigned vend,
                                         unsigned long long *gh,
                                         unsigned long long *oor_total) {
  if (v >= vend) return;
  atomicAdd(v < wl ? &gh[v] : oor_total, 65536ull);
  if ((v & 1u) == 0u) {  // a low half carried 1 into the high half (v + 1)
    unsigned long long *hi = v + 1 < wl ? &gh[v + 1] : oor_total;
    atomicAdd(hi, ~0ull);
    if ((old >> 16) == 0xFFFFu) atomicAdd(hi, 65536ull);
  }
}

// How the pair loop treats bins outside its window (kMode):
//  kFull:     the window covers bins [0, nbins); a valid pair beyond it is
//             out of range (clamped to the lane's out-of-range counter);
//  kFullSafe: the same window, and the tile boxes show that no pair of the
//             item can bin beyond it: no clamp;
//  kMid:      a window that is not the histogram's last (the planner gives
//             it an unreachable nbins): pairs beyond it belong to other
//             windows, never to the range-error count, and are ignored;
//  kGeneral:  the last window of a wider histogram: bins beyond nbins are
//             range errors, other misses are ignored.
constexpr int kFull = 0, kFullSafe = 1, kMid = 2, kGeneral = 3;

// One pair's shared-memory add. Every pair makes exactly one shared
// atomic, with no branch: its virtual bin e is the window bin when it hits,
// else this lane's out-of-range counter vo (a valid pair beyond the
// histogram) or ignore word vi (a pair outside a diagonal or partial tile,
// or in another window). Lane-private spare words avoid same-address
// serialisation; adds to ignore words are 0. Bins are carried as the raw
// bits of the rounding float, u = e + base (base even, so u and e have the
// same parity), and the window's shared address is pre-offset by base:
// word address = sadj + 4 (u >> 1). Returns the word's old value (u is
// updated to the virtual bin actually added to).
template <int kMode>
__device__ __forceinline__ unsigned pair_add_bin(unsigned &u, bool valid, unsigned base,
                                                 unsigned sadj, unsigned wl, unsigned kb,
                                                 unsigned nbins, unsigned uo,
                                                 unsigned ui) {
  bool ignore = false;
  if (kMode == kFullSafe) {
    u = valid ? u : ui;
    ignore = !valid;
  } else if (kMode == kFull) {
    // bins >= wl all count as out of range: clamp them to vo
    u = valid ? min(u, uo) : ui;
    ignore = !valid;
  } else if (kMode == kMid) {
    const bool hit = valid && u - base < wl;
    u = hit ? u : ui;
    ignore = !hit;
  } else {
    const unsigned lk = u - base;
    const bool oor = valid && lk + kb >= nbins;
    const bool hit = valid && lk < wl;
    u = hit ? u : (oor ? uo : ui);
    ignore = !hit && !oor;
  }
  // 1 << (16 * (u & 1)): the shift count is taken mod 32
  unsigned inc = __funnelshift_l(0u, 1u, u << 4);
  if (ignore) inc = 0u;  // ignore words stay 0
  unsigned old;
  asm volatile("atom.shared.add.u32 %0, [%1], %2;"
               : "=r"(old)
               : "r"(sadj + ((u >> 1) << 2)), "r"(inc));
  return old;
}

// Whether an add wrapped its half (rotate the added half to the top: by 16
// for an even bin), and the compensation if it did.
__device__ __forceinline__ void wrap_check_bin(unsigned old, unsigned u, unsigned base,
                                               unsigned wl, unsigned vend,
                                               unsigned long long *gh,
                                               unsigned long long *oor_total) {
  const unsigned rot = u * 16u + 16u;
  if (__funnelshift_l(old, old, rot) >= 0xFFFF0000u)
    wrap_fix(old, u - base, wl, vend, gh, oor_total);
}

// The raw form skips forming the bin: a pair is carried as the raw bits w
// of its rounding float (bits2), w = bits(2^23) + 2 bin + r with r the
// rounding bit. Its counter word is bin >> 1 = (w - bits(2^23)) >> 2 and
// its half bin & 1 = bit 1 of w, so the shared address is sadjw + (w & ~3)
// with sadjw = sadj + bits(2^23) (4 (u >> 1) = (w & ~3) + bits(2^23) for u
// = bits(2^23) + bin), and a virtual bin v (a window bin or a spare word's
// half, as wrap_fix numbers them) is w = wbase + 2 v, wbase = 2 base -
// bits(2^23). Window tests hold on these values as on bins: for integers
// b, n and r in {0, 1}, 2 b + r < 2 n exactly when b < n; NaN and infinite
// distances have larger bits than any window value. One add, one mask and
// a shift pair per pair instead of the bin form's two more; which loops
// take which form was chosen by timing all combinations (the 128-row loop
// of one-window histograms and the 32-row loop of middle windows gained,
// the others did not).
struct WinRaw {
  unsigned wbase;  // w of the window's first bin (rounding bit 0)
  unsigned sadjw;  // sadj + bits(2^23)
  unsigned wl2;    // 2 wl
  unsigned wo, wi; // this lane's out-of-range and ignore words
};

__device__ __forceinline__ WinRaw win_raw(unsigned base, unsigned sadj, unsigned wl,
                                          unsigned vo, unsigned vi) {
  WinRaw q;
  q.wbase = 2u * base - 0x4B000000u;
  q.sadjw = sadj + 0x4B000000u;
  q.wl2 = 2u * wl;
  q.wo = q.wbase + 2u * vo;
  q.wi = q.wbase + 2u * vi;
  return q;
}

// The raw form of pair_add_bin for kFull, kFullSafe and kMid.
template <int kMode>
__device__ __forceinline__ unsigned pair_add_raw(unsigned &w, bool valid,
                                                 const WinRaw &q) {
  static_assert(kMode != kGeneral, "the last window keeps the bin form");
  bool ignore = !valid;
  if (kMode == kFullSafe) {
    w = valid ? w : q.wi;
  } else if (kMode == kFull) {
    // bins beyond the spare words all count as out of range: clamp to wo
    w = valid ? min(w, q.wo) : q.wi;
  } else {
    const bool hit = valid && w - q.wbase < q.wl2;
    w = hit ? w : q.wi;
    ignore = !hit;
  }
  // 1 << (16 * (bin & 1)), the bin's parity being bit 1 of w; as a select
  // on that bit (a logic op that sets a predicate, and a select) rather
  // than a computed shift: spinel_10nm histogram 4.20 -> 3.96 ms
  unsigned inc = (w & 2u) ? 0x10000u : 1u;
  if (ignore) inc = 0u;  // ignore words stay 0
  unsigned old;
  asm volatile("atom.shared.add.u32 %0, [%1], %2;"
               : "=r"(old)
               : "r"(q.sadjw + (w & ~3u)), "r"(inc));
  return old;
}

__device__ __forceinline__ void wrap_check_raw(unsigned old, unsigned w, const WinRaw &q,
                                               unsigned wl, unsigned vend,
                                               unsigned long long *gh,
                                               unsigned long long *oor_total) {
  const unsigned rot = ((w >> 1) << 4) + 16u;
  if (__funnelshift_l(old, old, rot) >= 0xFFFF0000u)
    wrap_fix(old, (w - q.wbase) >> 1, wl, vend, gh, oor_total);
}

// The column-atom loop of one tile pair for one warp: lanes hold four row
// atoms; each column atom is one warp-uniform 16-byte load serving four
// pairs. kAllValid: a full 128 x 128 off-diagonal tile pair (no per-pair
// validity test). Whether an add wrapped its half is read from the
// returned old value; one test of the four old words' sign bits guards the
// rare compensation.
template <bool kAllValid, int kMode>
__device__ __forceinline__ void pair_loop(const float4 *__restrict__ bj,
                                          int jend, const float (&x)[4],
                                          const float (&y)[4],
                                          const float (&z)[4],
                                          const int (&jlim)[4], float inv,
                                          unsigned base, unsigned sadj,
                                          unsigned wl, unsigned kb,
                                          unsigned nbins,
                                          unsigned long long *gh,
                                          unsigned vo, unsigned vi,
                                          unsigned vend,
                                          unsigned long long *oor_total) {
  constexpr bool kRaw = kMode == kFull || kMode == kFullSafe;
  const unsigned uo = vo + base, ui = vi + base;
  const WinRaw q = win_raw(base, sadj, wl, vo, vi);
  const f2 ninv = pk(-2.0f * inv, -2.0f * inv);  // bits2 / bins2 take -2 inv
#pragma unroll 4  // 2: 1-2% slower (spinel_10nm, Gamma sample, 256-model batch)
  for (int j = 0; j < jend; ++j) {
    const float4 b = __ldg(&bj[j]);  // warp-uniform: broadcast
    unsigned u[4], old[4];
#pragma unroll
    for (int h = 0; h < 4; h += 2) {
      if (kRaw)
        bits2(x[h], x[h + 1], y[h], y[h + 1], z[h], z[h + 1], b.x, b.x, b.y, b.y, b.z,
              b.z, ninv, u[h], u[h + 1]);
      else
        bins2(x[h], x[h + 1], y[h], y[h + 1], z[h], z[h + 1], b.x, b.x, b.y, b.y, b.z,
              b.z, ninv, 0u, u[h], u[h + 1]);
    }
    unsigned any = 0u;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const bool valid = kAllValid || j <= jlim[r];
      if constexpr (kRaw)
        old[r] = pair_add_raw<kMode>(u[r], valid, q);
      else
        old[r] = pair_add_bin<kMode>(u[r], valid, base, sadj, wl, kb, nbins, uo, ui);
      any |= old[r];
    }
    // A wrap returns a half at 0xFFFF, so its bit 15 is set: the filter
    // passes only when some counter of these words has reached 32768.
    if (any & 0x80008000u) {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        if (kRaw)
          wrap_check_raw(old[r], u[r], q, wl, vend, gh, oor_total);
        else
          wrap_check_bin(old[r], u[r], base, wl, vend, gh, oor_total);
      }
    }
  }
}

// The same for a 32-row item: each lane holds one row atom and pairs it
// with two column atoms per step (the packed arithmetic's two halves), so
// an item covers a quarter of the row tile's atoms. The last, odd column
// of an item is paired with a repeat of itself that counts nothing.
template <bool kAllValid, int kMode>
__device__ __forceinline__ void pair_loop32(const float4 *__restrict__ bj, int jend,
                                            float x, float y, float z, int jlim,
                                            float inv, unsigned base, unsigned sadj,
                                            unsigned wl, unsigned kb, unsigned nbins,
                                            unsigned long long *gh, unsigned vo,
                                            unsigned vi, unsigned vend,
                                            unsigned long long *oor_total) {
  constexpr bool kRaw = kMode == kMid;
  const unsigned uo = vo + base, ui = vi + base;
  const WinRaw q = win_raw(base, sadj, wl, vo, vi);
  const f2 ninv = pk(-2.0f * inv, -2.0f * inv);  // bits2 / bins2 take -2 inv
#pragma unroll 2
  for (int j = 0; j < jend; j += 2) {
    const float4 b0 = __ldg(&bj[j]);  // warp-uniform: broadcast
    const float4 b1 = __ldg(&bj[kAllValid ? j + 1 : min(j + 1, jend - 1)]);
    unsigned u[2], old[2];
    const bool v0 = kAllValid || j <= jlim;
    const bool v1 = kAllValid || (j + 1 <= jlim && j + 1 < jend);
    if constexpr (kRaw) {
      bits2(x, x, y, y, z, z, b0.x, b1.x, b0.y, b1.y, b0.z, b1.z, ninv, u[0], u[1]);
      old[0] = pair_add_raw<kMode>(u[0], v0, q);
      old[1] = pair_add_raw<kMode>(u[1], v1, q);
    } else {
      bins2(x, x, y, y, z, z, b0.x, b1.x, b0.y, b1.y, b0.z, b1.z, ninv, 0u, u[0],
            u[1]);
      old[0] = pair_add_bin<kMode>(u[0], v0, base, sadj, wl, kb, nbins, uo, ui);
      old[1] = pair_add_bin<kMode>(u[1], v1, base, sadj, wl, kb, nbins, uo, ui);
    }
    if ((old[0] | old[1]) & 0x80008000u) {
      for (int r = 0; r < 2; ++r) {
        if (kRaw)
          wrap_check_raw(old[r], u[r], q, wl, vend, gh, oor_total);
        else
          wrap_check_bin(old[r], u[r], base, wl, vend, gh, oor_total);
      }
    }
  }
}

// Item it_i of a segment: {tile I (rows), tile J (columns) | diag << 31}.
__device__ __forceinline__ int2 seg_item(const HistSeg &sg,
                                         const int2 *__restrict__ items,
                                         int it_i) {
  if (sg.shape == kSegList) return __ldg(&items[it_i]);
  if (sg.shape == kSegRect)
    return make_int2(sg.ti0 + it_i / sg.tnj, sg.tj0 + it_i % sg.tnj);
  // triangle row-major by J: item t = J (J + 1) / 2 + I, I <= J. The FP32
  // estimate of J is off by at most one for t < 2^31 and is corrected in
  // integers (an FP64 square root here would queue every warp of a CTA on
  // the slow FP64 pipe at each task start).
  int j = (int)((sqrtf(8.0f * (float)it_i + 1.0f) - 1.0f) * 0.5f);
  while ((long long)j * (j + 1) / 2 > it_i) --j;
  while ((long long)(j + 1) * (j + 2) / 2 <= it_i) ++j;
  const int i = it_i - j * (j + 1) / 2;
  return make_int2(sg.ti0 + i,
                   (sg.ti0 + j) | (i == j ? int(0x80000000u) : 0));
}

// One warp = one tile pair (128 x 128 atoms). CTAs pull tasks from a global
// counter in the order tasks[k].next (decreasing size, so the last tasks
// to start are the short ones), and warps pull the task's tile pairs from a
// shared counter (warps progress unevenly under the issue scheduler; a
// fixed round robin left the fast ones waiting at the task's end); task
// t's packed window goes to partial slot t.
__global__ void __launch_bounds__(kHistThreads, 1)
    hist_tiles_kernel(const int2 *__restrict__ items,
                      const HistTask *__restrict__ tasks, int ntasks,
                      const HistSeg *__restrict__ segs, float inv,
                      unsigned *__restrict__ partial, int words_per_task,
                      unsigned long long *__restrict__ oor_total,
                      int *__restrict__ task_counter) {
  extern __shared__ unsigned sh[];
  __shared__ int s_task, s_item;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) {  // tasks are pulled largest first
      const int k = atomicAdd(task_counter, 1);
      s_task = k < ntasks ? tasks[k].next : ntasks;
    }
    __syncthreads();
    const int t = s_task;
    if (t >= ntasks) break;
    const HistTask tk = tasks[t];
    const HistSeg sg = segs[tk.seg];
    const int nw = (sg.wl + 1) >> 1;
    if (threadIdx.x == 0) s_item = tk.item_begin;
    // window words, then 32 out-of-range words and 32 ignore words (one
    // each per lane), addressed as virtual bins 2 * word
    for (int i = threadIdx.x; i < nw + kSpareWords; i += kHistThreads)
      sh[i] = 0u;
    __syncthreads();
    const unsigned vo = 2u * ((unsigned)nw + lane), vi = vo + 64u;
    const unsigned vend = 2u * ((unsigned)nw + 32u);
    // shared address of word 0 minus 4 (base >> 1), mod 2^32
    const unsigned sadj = (unsigned)__cvta_generic_to_shared(sh) -
                          ((0x4B000000u + (unsigned)sg.kb) >> 1) * 4u;
    const float4 *atoms = sg.atoms;
    const int2 *tiles = sg.tiles;
    unsigned long long *gh = sg.out + sg.kb;
    const unsigned wl = (unsigned)sg.wl, kb = (unsigned)sg.kb;
    const unsigned nbins = sg.nbins;
    const unsigned base = 0x4B000000u + kb;
    const bool full_window = kb == 0 && wl >= nbins;
    // a window before the histogram's last: its misses are never range errors
    const bool mid_window = !full_window && nbins == 0xFFFFFFFFu;
    // The pairs this segment counts are its window's bins [own_lo, own_lo +
    // own_len) (the whole window unless overlapping windows share bins):
    // the pair loop sees that range as its window, by offsetting the base,
    // the histogram pointer and the spare counters' virtual bins (own_lo is
    // even, so bins keep their parity; the raw-bit addresses are unchanged).
    const unsigned olo = (unsigned)sg.own_lo;
    const unsigned pbase = base + olo, pwl = (unsigned)sg.own_len, pkb = kb + olo;
    unsigned long long *pgh = gh + olo;
    const unsigned pvo = vo - olo, pvi = vi - olo, pvend = vend - olo;
    for (;;) {
      int it_i = 0;
      if (lane == 0) it_i = atomicAdd(&s_item, 1);
      it_i = __shfl_sync(0xffffffffu, it_i, 0);
      if (it_i >= tk.item_end) break;
      const int2 it = seg_item(sg, items, it_i);
      const bool diag = it.y < 0;
      const unsigned ix = (unsigned)it.x;
      const int2 TI = __ldg(&tiles[ix & (unsigned)kItemTileMask]);
      const int2 TJ = __ldg(&tiles[it.y & 0x7fffffff]);
      // columns [jb, je): the item's quarters of tile J
      const int jb = kQuarter * (int)((ix >> kItemQ0Shift) & 3u);
      const int je = min(TJ.y, kQuarter * (4 - (int)((ix >> kItemQ1Shift) & 3u)));
      const float4 *bj = atoms + TJ.x + jb;
      if ((ix >> kItemRowQShift) & 1u) {
        // a 32-row item: rows [32 rq, 32 rq + 32) of tile I, one per lane
        // (listed by the planner in multi-window histograms only)
        const int pi = kQuarter * (int)(ix >> kItemRqShift) + lane;
        const bool act = pi < TI.y;
        const float4 a = __ldg(&atoms[TI.x + (act ? pi : 0)]);
        const int jl = act ? (diag ? pi - jb : 0x7fffffff) : -1;
        const bool av = !diag && pi - lane + kQuarter <= TI.y && ((je - jb) & 1) == 0;
#define DBX_PAIR_LOOP32(AV, MODE)                                                   \
  pair_loop32<AV, MODE>(bj, je - jb, a.x, a.y, a.z, jl, inv, pbase, sadj, pwl, pkb, \
                        nbins, pgh, pvo, pvi, pvend, oor_total)
        if (mid_window) {
          if (av) DBX_PAIR_LOOP32(true, kMid);
          else DBX_PAIR_LOOP32(false, kMid);
        } else {
          if (av) DBX_PAIR_LOOP32(true, kGeneral);
          else DBX_PAIR_LOOP32(false, kGeneral);
        }
#undef DBX_PAIR_LOOP32
        continue;
      }
      float x[4], y[4], z[4];
      int jlim[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int pi = lane + 32 * r;
        const bool act = pi < TI.y;
        const float4 a = __ldg(&atoms[TI.x + (act ? pi : 0)]);
        x[r] = a.x;
        y[r] = a.y;
        z[r] = a.z;
        // diag tile: pairs j <= i incl. i == j (cuDebye-v15.cu:137); the
        // loop counts columns from jb
        jlim[r] = act ? (diag ? pi - jb : 0x7fffffff) : -1;
      }
      const bool all_valid = !diag && TI.y == kTile;  // warp-uniform
      int mode = full_window ? kFull : (mid_window ? kMid : kGeneral);
      if (full_window) {
        // No pair of the item can bin at or beyond wl if the distance bound
        // of the tile boxes stays below it. The bound is computed in FP32
        // with a margin far above the rounding of both it and the pairs'
        // distances; NaN or infinite boxes fail the test.
        const TileBox *BI = sg.boxes + (ix & (unsigned)kItemTileMask);
        const TileBox *BJ = sg.boxes + (it.y & 0x7fffffff);
        float d2 = 0.f, all = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float g1 = fabsf(__ldg(&BJ->hi[c]) - __ldg(&BI->lo[c]));
          const float g2 = fabsf(__ldg(&BI->hi[c]) - __ldg(&BJ->lo[c]));
          const float g = fmaxf(g1, g2);
          d2 = fmaf(g, g, d2);
          all += g1 + g2;  // NaN or infinite if any box coordinate is
        }
        if (all - all == 0.f && sqrtf(d2) * inv * 1.000244f + 2.0f < (float)wl)
          mode = kFullSafe;
      }
#define DBX_PAIR_LOOP(AV, MODE)                                                   \
  pair_loop<AV, MODE>(bj, je - jb, x, y, z, jlim, inv, pbase, sadj, pwl, pkb, nbins, \
                      pgh, pvo, pvi, pvend, oor_total)
      if (all_valid) {
        if (mode == kFullSafe) DBX_PAIR_LOOP(true, kFullSafe);
        else if (mode == kFull) DBX_PAIR_LOOP(true, kFull);
        else if (mode == kMid) DBX_PAIR_LOOP(true, kMid);
        else DBX_PAIR_LOOP(true, kGeneral);
      } else {
        if (mode == kFullSafe) DBX_PAIR_LOOP(false, kFullSafe);
        else if (mode == kFull) DBX_PAIR_LOOP(false, kFull);
        else if (mode == kMid) DBX_PAIR_LOOP(false, kMid);
        else DBX_PAIR_LOOP(false, kGeneral);
      }
#undef DBX_PAIR_LOOP
    }
    __syncthreads();
    unsigned *dst = partial + (size_t)t * (size_t)words_per_task;
    for (int i = threadIdx.x; i < nw; i += kHistThreads) dst[i] = sh[i];
    if (warp == 0) {  // out-of-range counts: spare words and bin wl
      const unsigned w = sh[nw + lane];
      unsigned o = (w & 0xFFFFu) + (w >> 16);
      if (lane == 0 && (wl & 1u)) o += sh[nw - 1] >> 16;
      o = __reduce_add_sync(0xffffffffu, o);
      if (lane == 0 && o) atomicAdd(oor_total, (unsigned long long)o);
    }
    __syncthreads();
  }
}

// Sum the packed windows of each segment's tasks into the int64 histogram
// (bins a segment does not count hold 0 there). A histogram of one window
// has one segment owning every bin: plain read-modify-writes; the windows of
// a wider histogram overlap, so their sums are atomic. The wrap corrections
// of the tile kernel were made earlier on the same stream.
__global__ void hist_reduce_kernel(const unsigned *__restrict__ partial,
                                   int words_per_task,
                                   const HistSeg *__restrict__ segs) {
  const HistSeg sg = segs[blockIdx.y];
  const int nw = (sg.wl + 1) >> 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw;
       i += gridDim.x * blockDim.x) {
    unsigned long long lo = 0, hi = 0;
    for (int t = sg.task_begin; t < sg.task_end; ++t) {
      const unsigned w = partial[(size_t)t * (size_t)words_per_task + i];
      lo += w & 0xFFFFu;
      hi += w >> 16;
    }
    unsigned long long *g = sg.out + sg.kb + 2 * i;
    if (sg.kb == 0 && (unsigned)sg.wl >= sg.nbins) {  // one window: sole owner
      g[0] += lo;
      if (2 * i + 1 < sg.wl) g[1] += hi;  // bin wl (odd wl) counts range errors
    } else {  // windows of one histogram may overlap
      if (lo) atomicAdd(&g[0], lo);
      if (hi && 2 * i + 1 < sg.wl) atomicAdd(&g[1], hi);
    }
  }
}

// Zero the output histograms of a plan (row blockIdx.x, split over
// gridDim.y blocks).
__global__ void hist_zero_kernel(const HistRow *__restrict__ rows) {
  const HistRow r = rows[blockIdx.x];
  for (long long i = blockIdx.y * (long long)blockDim.x + threadIdx.x; i < r.len;
       i += (long long)gridDim.y * blockDim.x)
    r.out[i] = 0ull;
}

// One thread per pair (i of the row block, j of the column block), blocks of
// 16x16 pairs as in the reference's launch shape; diag keeps j <= i.
__global__ void plain_pairs_kernel(const float4 *__restrict__ atoms, long long a0,
                                   int na, long long b0, int nb, int diag,
                                   float inv, unsigned nbins,
                                   unsigned long long *__restrict__ out,
                                   unsigned long long *__restrict__ oor) {
  const int j = blockIdx.x * 16 + threadIdx.x;
  const int i = blockIdx.y * 16 + threadIdx.y;
  if (i >= na || j >= nb || (diag && j > i)) return;
  const float4 a = atoms[a0 + i], b = atoms[b0 + j];
  const unsigned k = bin_rel(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y),
                             __fsub_rn(b.z, a.z), inv, 0x4B000000u);
  if (k < nbins)
    atomicAdd(&out[k], 1ull);
  else
    atomicAdd(oor, 1ull);
}

// Self-check of the kernels' square roots against the IEEE one for the
// floats with bits in [lo, hi] (non-negative: hi <= bits of +inf): sqrt_rn,
// and nsqrt2 (the packed form the tile kernels use) on the neighbouring
// pair (u, u ^ 1) in its two lanes. res[0] counts mismatches, res[1] keeps
// the smallest mismatching bits. Inputs below 2^-75 only need a result
// below 2^-37 (they bin to 0 either way); +inf only a non-finite result.
__device__ __forceinline__ bool sqrt_ok(float s, float a) {
  const float b = __fsqrt_rn(s);
  if (!(s >= 0x1p-75f)) return a < 0x1p-37f;
  if (isinf(b)) return !isfinite(a);
  return __float_as_uint(a) == __float_as_uint(b);
}

__global__ void check_sqrt_kernel(unsigned lo, unsigned hi,
                                  unsigned long long *res) {
  const unsigned long long n = (unsigned long long)(hi - lo) + 1ull;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x +
                              threadIdx.x;
       i < n; i += stride) {
    const unsigned u = lo + (unsigned)i;
    const float s = __uint_as_float(u);
    // the packed form on (u, partner); lane 0 holds u
    const unsigned v = (u ^ 1u) <= 0x7F800000u ? (u ^ 1u) : u;
    const float sv = __uint_as_float(v);
    const f2 nc = sub2(pk(-0x1p-100f, -0x1p-100f), pk(s, sv));
    float m0, m1;
    upk(nsqrt2(nc), m0, m1);
    const float c0 = __fadd_rn(s, 0x1p-100f);
    const bool good = sqrt_ok(s, sqrt_rn(s)) && sqrt_ok(c0, -m0) &&
                      sqrt_ok(__fadd_rn(sv, 0x1p-100f), -m1);
    if (!good) {
      atomicAdd(&res[0], 1ull);
      atomicMin(&res[1], (unsigned long long)u);
    }
  }
}

Error check_sqrt(unsigned lo, unsigned hi, int num_sms, cudaStream_t stream,
                 int64_t out[3]) {
  if (lo > hi || hi > 0x7F800000u)
    return fail(DBX_ERR_ARG, "need lo <= hi <= 0x7F800000 (non-negative floats)");
  unsigned long long *res = nullptr;
  DBX_CUDA_TRY(cudaMallocAsync((void **)&res, 2 * sizeof(unsigned long long), stream));
  cudaMemsetAsync(res, 0, sizeof(unsigned long long), stream);
  cudaMemsetAsync(res + 1, 0xFF, sizeof(unsigned long long), stream);
  check_sqrt_kernel<<<num_sms * 8, 256, 0, stream>>>(lo, hi, res);
  cudaError_t e = cudaGetLastError();
  unsigned long long h[2] = {0, 0};
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, stream);
  cudaFreeAsync(res, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess)
    return fail(DBX_ERR_CUDA, std::string("check_sqrt: ") + cudaGetErrorString(e));
  out[0] = (int64_t)(hi - lo) + 1;
  out[1] = (int64_t)h[0];
  out[2] = h[0] ? (int64_t)h[1] : -1;
  return ok();
}

// ---------------------------------------------------------------------------
// Planner (host).

static void box_bins(const TileBox &A, const TileBox &B, double inv,
                     int64_t *kmin, int64_t *kmax) {
  double dmin2 = 0, dmax2 = 0;
  for (int c = 0; c < 3; ++c) {
    double g = std::max({0.0, (double)B.lo[c] - A.hi[c],
                         (double)A.lo[c] - B.hi[c]});
    double h = std::max(std::fabs((double)B.hi[c] - A.lo[c]),
                        std::fabs((double)A.hi[c] - B.lo[c]));
    dmin2 += g * g;
    dmax2 += h * h;
  }
  // FP32 distances carry a relative error of a few 1e-7; widen generously.
  // A box with a NaN or infinite coordinate may reach any bin (and beyond).
  if (!std::isfinite(dmax2) || !std::isfinite(dmin2)) {
    *kmin = 0;
    *kmax = INT64_MAX;
    return;
  }
  *kmin = (int64_t)std::floor(std::sqrt(dmin2) * inv * (1 - 1e-5)) - 2;
  *kmax = (int64_t)std::ceil(std::sqrt(dmax2) * inv * (1 + 1e-5)) + 2;
}

static int64_t item_pairs(int nI, int nJ, bool diag) {
  return diag ? (int64_t)nI * (nI + 1) / 2 : (int64_t)nI * nJ;
}

// Pairs (i, j) of rows [i0, i1) and columns [j0, j1) of a tile pair, with
// j <= i on a diagonal tile.
static int64_t sub_pairs(int i0, int i1, int j0, int j1, bool diag) {
  if (i1 <= i0 || j1 <= j0) return 0;
  if (!diag) return (int64_t)(i1 - i0) * (j1 - j0);
  int64_t n = 0;
  for (int i = i0; i < i1; ++i) n += std::max(0, std::min(j1, i + 1) - j0);
  return n;
}

// Cost of a pair in a 32-row item against one in a 128-row item (one more
// column load and the packing of two columns per two pairs, against one
// load and packing per four): 32-row items are listed where they cut the
// pairs of an item by more than this factor. Measured on the shipped Gamma
// sample (31 windows): factor 1.0 21.3 ms, 1.12 21.1, 1.25 20.9, 1.5 21.3,
// 2.0 22.1, 3.0 22.7, never 23.9. DBX_HIST_ROWQ sets it (0: never).
double hist_rowq_default() {
  static const double f = [] {
    const char *v = getenv("DBX_HIST_ROWQ");
    return v ? std::max(0.0, atof(v)) : 1.25;
  }();
  return f;
}

// Host threads for listing tile pairs (the machine's cores, at most 32).
static int plan_threads() {
  static const int n = [] {
    const unsigned h = std::thread::hardware_concurrency();
    return (int)std::min(32u, std::max(1u, h));
  }();
  return n;
}

// One thread's tile pairs per window: items, their pair counts and sums.
struct WinLists {
  std::vector<std::vector<int2>> items;
  std::vector<std::vector<int>> pairs;
  std::vector<int64_t> sum;
};

void hist_plan_clear(HistPlan *plan) {
  plan->items.clear();
  plan->item_pairs.clear();
  plan->segs.clear();
  plan->seg_items.clear();
  plan->seg_pairs.clear();
  plan->tasks.clear();
  plan->rows.clear();
  plan->pairs = 0;
  plan->nrows = 0;
  plan->window = 0;
  plan->quarters = -1;
}

Error hist_plan_add(const Model &m, const std::vector<int2> &pairs,
                    double rstep, int64_t nbins, unsigned long long *out,
                    int64_t pitch, HistPlan *plan) {
  if (nbins < 1 || nbins > (int64_t(1) << 22))
    return fail(DBX_ERR_ARG,
                "histogram needs 1 <= nbins <= 4194304 (got " +
                    std::to_string(nbins) + ")");
  const int W = kWindowBins;
  const double rowq = plan->rowq;
  plan->window = std::max(plan->window, (int)std::min<int64_t>(W, nbins));
  const int64_t nwin = (nbins + W - 1) / W;
  const double inv = 1.0 / rstep;
  for (size_t pi = 0; pi < pairs.size(); ++pi) {
    const int a = pairs[pi].x, b = pairs[pi].y;
    // integer arithmetic: `out` may be null (a plan made before upload)
    unsigned long long *row = reinterpret_cast<unsigned long long *>(
        reinterpret_cast<uintptr_t>(out) + (uintptr_t)pi * pitch * sizeof(*out));
    plan->rows.push_back(HistRow{row, pitch});
    const int64_t na = m.sp_count[a], nb = m.sp_count[b];
    const int64_t block_pairs = (a == b) ? na * (na + 1) / 2 : na * nb;
    if (nwin == 1) {
      // One window holds every bin: the segment's items are all its tile
      // pairs, enumerated by the kernel (no list, no bounding-box test).
      const int I0 = m.tile_start[a], nI = m.tile_start[a + 1] - I0;
      const int J0 = m.tile_start[b], nJ = m.tile_start[b + 1] - J0;
      const int64_t count = (a == b) ? (int64_t)nI * (nI + 1) / 2 : (int64_t)nI * nJ;
      if (count >= (int64_t(1) << 31))
        return fail(DBX_ERR_ARG, "too many tile pairs in one species pair");
      if (count > 0) {
        HistSeg s;
        s.atoms = m.d_atoms;
        s.tiles = m.d_tiles;
        s.boxes = m.d_boxes;
        s.out = row;
        s.kb = 0;
        s.wl = (int)nbins;
        s.task_begin = s.task_end = 0;
        s.nbins = (unsigned)nbins;
        s.shape = (a == b) ? kSegTri : kSegRect;
        s.own_lo = 0;
        s.own_len = s.wl;
        s.ti0 = I0;
        s.tni = nI;
        s.tj0 = J0;
        s.tnj = nJ;
        plan->segs.push_back(s);
        plan->seg_items.push_back(make_int2(0, (int)count));
        plan->seg_pairs.push_back(block_pairs);
      }
      plan->pairs += block_pairs;
      plan->nrows += 1;
      continue;
    }
    if (m.boxes.size() != m.tiles.size())
      return fail(DBX_ERR_ARG, "tile boxes are not on the host");
    if (m.tile_start[a + 1] > kItemTileMask + 1)
      return fail(DBX_ERR_ARG, "too many tiles in one model for a multi-window histogram");
    // Tile pairs listed per window from their bounding boxes, rows of tiles
    // split among host threads by item count; the lists are joined in row
    // order, so the plan does not depend on the thread count.
    const int I0 = m.tile_start[a], I1 = m.tile_start[a + 1];
    const int Jb0 = m.tile_start[b], Jb1 = m.tile_start[b + 1];
    auto row_items = [&](int I) -> int64_t {
      return Jb1 - ((a == b) ? I : Jb0);
    };
    int64_t nitems = 0;
    for (int I = I0; I < I1; ++I) nitems += row_items(I);
    const int nth = (int)std::max<int64_t>(
        1, std::min<int64_t>(plan_threads(), nitems / 4096));
    std::vector<int> row_cut(nth + 1, I1);
    row_cut[0] = I0;
    {
      int64_t acc = 0;
      int k = 1;
      for (int I = I0; I < I1 && k < nth; ++I) {
        acc += row_items(I);
        while (k < nth && acc * nth >= nitems * k) row_cut[k++] = I + 1;
      }
    }
    // Window geometry. Disjoint: window w covers [w W, (w + 1) W). Or
    // overlapping where nbins < nwin W: window w starts at an even kbw[w],
    // evenly spaced, the last ending at nbins. Window w owns the bins
    // [own[w], own[w + 1]) (boundaries even, inside both neighbours). A tile
    // pair whose bin range lies inside one window is listed there alone and
    // counts all its pairs in it ("whole" list); any other is listed in
    // every window whose owned bins its range reaches and counts only
    // those ("owned" list). Overlap saves the second pass of tile pairs
    // that straddle a boundary when windows are wide against the tile
    // pairs' ranges (a histogram slightly wider than one window), and costs
    // narrower owned ranges when they are not (fine bins): each species
    // pair takes the geometry under which evenly spaced sample tile pairs
    // list fewer pairs.
    struct Geom {
      std::vector<int64_t> kbw, wlw, own;
    };
    auto make_geom = [&](bool overlap) {
      Geom g;
      g.kbw.resize(nwin);
      g.wlw.resize(nwin);
      g.own.resize(nwin + 1);
      const int64_t last = std::max<int64_t>(0, (nbins - W + 1) & ~int64_t(1));
      for (int64_t w = 0; w < nwin; ++w) {
        g.kbw[w] = overlap ? ((w * last) / (nwin - 1)) & ~int64_t(1) : w * W;
        g.wlw[w] = std::min<int64_t>(W, nbins - g.kbw[w]);
      }
      g.own[0] = 0;
      g.own[nwin] = nbins;
      for (int64_t w = 1; w < nwin; ++w)  // middle of the overlap, even
        g.own[w] = overlap ? ((g.kbw[w] + g.kbw[w - 1] + g.wlw[w - 1]) / 2) & ~int64_t(1)
                           : g.kbw[w];
      return g;
    };
    // Lists of a tile pair with bin range [kmin, kmax]: emit(2 w) for the
    // whole list of window w, emit(2 w + 1) for its owned list.
    auto assign = [&](const Geom &g, int64_t kmin, int64_t kmax, auto &&emit) {
      kmin = std::max<int64_t>(kmin, 0);
      if (kmin >= nbins) {  // entirely beyond rmax: the last window reports
        emit(2 * (nwin - 1));  // them as range errors
        return;
      }
      // the last window starting at or below kmin, and the one before
      const int64_t wc = std::upper_bound(g.kbw.begin(), g.kbw.end(), kmin) - g.kbw.begin() - 1;
      int64_t whole = -1;
      for (int64_t w = std::max<int64_t>(0, wc - 1); w <= wc; ++w)
        if (g.kbw[w] <= kmin &&  // the last window counts bins >= nbins too
            (w == nwin - 1 || kmax < g.kbw[w] + g.wlw[w]))
          whole = w;
      if (whole >= 0) {
        emit(2 * whole);
        return;
      }
      const int64_t hi = std::min<int64_t>(kmax, nbins - 1);
      const int64_t w0 = std::upper_bound(g.own.begin(), g.own.end(), kmin) - g.own.begin() - 1;
      const int64_t w1 = std::upper_bound(g.own.begin(), g.own.end(), hi) - g.own.begin() - 1;
      for (int64_t w = w0; w <= std::min(w1, nwin - 1); ++w) emit(2 * w + 1);
    };
    const Geom gd = make_geom(false), go = make_geom(true);
    bool overlap = false;
    {
      double cd = 0, co = 0;
      const int nI = I1 - I0;
      for (int smp = 0; smp < 4096 && nitems > 0; ++smp) {  // nitems: both non-empty
        const int I = I0 + (int)((int64_t)smp * nI / 4096);
        const int Jlo = (a == b) ? I : Jb0;
        const int J = Jlo + (int)(((int64_t)smp * 7919) % std::max(1, Jb1 - Jlo));
        int64_t kmin, kmax;
        box_bins(m.boxes[I], m.boxes[J], inv, &kmin, &kmax);
        const double np = (double)item_pairs(m.tiles[I].y, m.tiles[J].y, a == b && I == J);
        assign(gd, kmin, kmax, [&](int64_t) { cd += np; });
        assign(go, kmin, kmax, [&](int64_t) { co += np; });
      }
      overlap = co < cd;
    }
    if (plan->geom == kGeomDisjoint) overlap = false;
    if (plan->geom == kGeomOverlap) overlap = true;
    const Geom &g = overlap ? go : gd;
    const std::vector<int64_t> &kbw = g.kbw, &wlw = g.wlw, &own = g.own;
    for (int64_t w = 1; w < nwin; ++w)
      if (own[w] < kbw[w] || own[w] > kbw[w - 1] + wlw[w - 1] || own[w] <= own[w - 1])
        return fail(DBX_ERR_ARG, "internal: histogram windows do not tile the bins");
    const int64_t nl = 2 * nwin;
    std::vector<WinLists> part(nth);
    auto list_rows = [&](int t) {
      WinLists &L = part[t];
      L.items.assign(nl, {});
      L.pairs.assign(nl, {});
      L.sum.assign(nl, 0);
      auto put = [&](int64_t l, int2 it, int np) {
        L.items[l].push_back(it);
        L.pairs[l].push_back(np);
        L.sum[l] += np;
      };
      for (int I = row_cut[t]; I < row_cut[t + 1]; ++I) {
        const int2 TI = m.tiles[I];
        const TileBox &BI = m.boxes[I];
        for (int J = (a == b) ? I : Jb0; J < Jb1; ++J) {
          const bool diag = (a == b) && (I == J);
          const int2 it = make_int2(I, J | (diag ? int(0x80000000u) : 0));
          const int nJ = m.tiles[J].y;
          const int np = (int)item_pairs(TI.y, nJ, diag);
          int64_t kmin, kmax;
          box_bins(BI, m.boxes[J], inv, &kmin, &kmax);
          // In an owned list the item runs only over the columns whose
          // quarters reach the window's owned bins (their bin ranges from
          // the quarter boxes, computed on first use), or is split into
          // 32-row items, each over the column quarters its row quarter
          // reaches, where that lists fewer pairs by more than the 32-row
          // loop's extra cost per pair.
          int64_t qk0[4], qk1[4];
          int nq = -1;
          int64_t rk0[4][4], rk1[4][4];  // row quarter x column quarter
          int nr = -1;
          assign(g, kmin, kmax, [&](int64_t l) {
            if (!(l & 1)) {
              put(l, it, np);
              return;
            }
            if (nq < 0) {
              nq = (nJ + kQuarter - 1) / kQuarter;
              for (int q = 0; q < nq; ++q) {
                TileBox Q;
                for (int d = 0; d < 3; ++d) {
                  Q.lo[d] = m.boxes[J].qlo[q][d];
                  Q.hi[d] = m.boxes[J].qhi[q][d];
                }
                box_bins(BI, Q, inv, &qk0[q], &qk1[q]);
              }
            }
            const int64_t w = l / 2, lo = own[w], hi = own[w + 1];
            // the last window counts bins >= nbins
            auto reach = [&](int64_t k0, int64_t k1) {
              return k1 >= lo && (w == nwin - 1 || std::max<int64_t>(k0, 0) < hi);
            };
            unsigned mask = 0;
            for (int q = 0; q < nq; ++q)
              if (reach(qk0[q], qk1[q])) mask |= 1u << q;
            if (!mask) return;
            const int q0 = __builtin_ctz(mask), q1 = 32 - __builtin_clz(mask);
            const int jb = q0 * kQuarter, je = std::min(nJ, q1 * kQuarter);
            const int npq = diag ? (je - jb) * TI.y - (jb + je - 1) * (je - jb) / 2
                                 : (je - jb) * TI.y;
            if (rowq > 0) {
              if (nr < 0) {
                nr = (TI.y + kQuarter - 1) / kQuarter;
                for (int r = 0; r < nr; ++r)
                  for (int q = 0; q < nq; ++q) {
                    TileBox R, Q;
                    for (int d = 0; d < 3; ++d) {
                      R.lo[d] = BI.qlo[r][d];
                      R.hi[d] = BI.qhi[r][d];
                      Q.lo[d] = m.boxes[J].qlo[q][d];
                      Q.hi[d] = m.boxes[J].qhi[q][d];
                    }
                    box_bins(R, Q, inv, &rk0[r][q], &rk1[r][q]);
                  }
              }
              int2 its[4];
              int nps[4];
              int nit = 0;
              int64_t sum = 0;
              for (int r = 0; r < nr; ++r) {
                unsigned rm = 0;
                for (int q = 0; q < nq; ++q)
                  if (reach(rk0[r][q], rk1[r][q])) rm |= 1u << q;
                if (!rm) continue;
                const int r0 = __builtin_ctz(rm), r1 = 32 - __builtin_clz(rm);
                const int cb = r0 * kQuarter, ce = std::min(nJ, r1 * kQuarter);
                const int np32 = (int)sub_pairs(r * kQuarter, std::min(TI.y, (r + 1) * kQuarter),
                                                  cb, ce, diag);
                if (np32 == 0) continue;
                its[nit] = make_int2(
                    (int)((unsigned)I | ((unsigned)r0 << kItemQ0Shift) |
                          ((unsigned)(4 - r1) << kItemQ1Shift) | (1u << kItemRowQShift) |
                          ((unsigned)r << kItemRqShift)),
                    it.y);
                nps[nit++] = np32;
                sum += np32;
              }
              if ((double)sum * rowq < (double)npq) {
                for (int k = 0; k < nit; ++k) put(l, its[k], nps[k]);
                return;
              }
            }
            const int2 itq = make_int2(I | (q0 << kItemQ0Shift) | ((4 - q1) << kItemQ1Shift), it.y);
            put(l, itq, npq);
          });
        }
      }
    };
    if (nth == 1) {
      list_rows(0);
    } else {
      std::vector<std::thread> th;
      for (int t = 1; t < nth; ++t) th.emplace_back(list_rows, t);
      list_rows(0);
      for (std::thread &x : th) x.join();
    }
    // Final positions of every (list, thread) part, then one resize of the
    // plan's arrays and a parallel copy into place.
    std::vector<int64_t> off((size_t)nl * nth);
    size_t at = plan->items.size();
    const size_t first_all = at;
    for (int64_t l = 0; l < nl; ++l)
      for (int t = 0; t < nth; ++t) {
        off[(size_t)l * nth + t] = (int64_t)at;
        at += part[t].items[l].size();
      }
    if (at > plan->items.capacity()) {  // grow geometrically across calls
      plan->items.reserve(std::max(at, 2 * plan->items.capacity()));
      plan->item_pairs.reserve(std::max(at, 2 * plan->item_pairs.capacity()));
    }
    plan->items.resize(at);
    plan->item_pairs.resize(at);
    auto place = [&](int t) {
      const WinLists &L = part[t];
      for (int64_t l = 0; l < nl; ++l) {
        const size_t o = (size_t)off[(size_t)l * nth + t];
        std::copy(L.items[l].begin(), L.items[l].end(), plan->items.begin() + o);
        std::copy(L.pairs[l].begin(), L.pairs[l].end(), plan->item_pairs.begin() + o);
      }
    };
    if (nth == 1) {
      place(0);
    } else {
      std::vector<std::thread> th;
      for (int t = 1; t < nth; ++t) th.emplace_back(place, t);
      place(0);
      for (std::thread &x : th) x.join();
    }
    size_t cur = first_all;
    for (int64_t l = 0; l < nl; ++l) {
      const int64_t w = l / 2;
      const bool owned = l & 1;
      int64_t sp = 0;
      size_t cnt = 0;
      for (const WinLists &L : part) {
        cnt += L.items[l].size();
        sp += L.sum[l];
      }
      if (cnt == 0) continue;
      HistSeg s;
      s.atoms = m.d_atoms;
      s.tiles = m.d_tiles;
      s.boxes = m.d_boxes;
      s.out = row;
      s.kb = (int)kbw[w];
      s.wl = (int)wlw[w];
      s.task_begin = s.task_end = 0;
      // out-of-range pairs are counted by the last window only: the others
      // get an unreachable bound (no bin reaches 2^32 - 1 in the test)
      s.nbins = w == nwin - 1 ? (unsigned)nbins : 0xFFFFFFFFu;
      s.shape = kSegList;
      s.own_lo = owned ? (int)(own[w] - kbw[w]) : 0;
      s.own_len = owned ? (int)(own[w + 1] - own[w]) : s.wl;
      s.ti0 = s.tni = s.tj0 = s.tnj = 0;
      plan->segs.push_back(s);
      plan->seg_items.push_back(make_int2((int)cur, (int)(cur + cnt)));
      plan->seg_pairs.push_back(sp);
      cur += cnt;
    }
    plan->pairs += block_pairs;
    plan->nrows += 1;
  }
  return ok();
}

void hist_plan_tasks(HistPlan *plan, int target_tasks) {
  // Split every segment into n_s tasks of about equal pair counts, n_s
  // from the segment's share of about target_tasks tasks in all. Listed
  // items are split by their pair counts; enumerated segments (nearly all
  // items full 128 x 128 tile pairs) by item count.
  plan->tasks.clear();
  int64_t total = 0;
  for (int64_t p : plan->seg_pairs) total += p;
  const size_t S = plan->segs.size();
  // A small plan of enumerated segments only (one window per histogram)
  // has too few tile pairs to give every warp of its CTAs one: a warp takes
  // one tile pair, so a plan of fewer than 8 per task left most warps idle
  // (a 5,000-atom model: 820 tile pairs over 304 tasks). Such a plan lists
  // each tile pair as four 32-row items (on a diagonal tile pair, row
  // quarter rq only over column quarters [0, rq]) and takes about 32 items
  // per task; the kernel runs them as the 32-row items of a last window,
  // whose test is exact for a window holding every bin. The decision is
  // kept for later splits of the plan.
  if (plan->quarters < 0) {
    int64_t enum_items = 0;
    bool all_enum = S > 0;
    for (size_t s = 0; s < S; ++s) {
      if (plan->segs[s].shape == kSegList) all_enum = false;
      else enum_items += plan->seg_items[s].y - plan->seg_items[s].x;
    }
    // 8: a 4,477-atom model's histogram 0.070 -> 0.045 ms with the 32-row
    // items, a 12,004-atom model's (15 tile pairs per task) 0.088 -> 0.096
    plan->quarters =
        !all_enum ? 0 : (enum_items < 8 * (int64_t)target_tasks ? 1 : 2);
    if (plan->quarters == 1) {
      for (size_t s = 0; s < S; ++s) {
        HistSeg &sg = plan->segs[s];
        const int begin = (int)plan->items.size();
        const int count = plan->seg_items[s].y - plan->seg_items[s].x;
        for (int p = 0; p < count; ++p) {
          int I, J;
          bool diag = false;
          if (sg.shape == kSegRect) {
            I = sg.ti0 + p / sg.tnj;
            J = sg.tj0 + p % sg.tnj;
          } else {  // p = j (j + 1) / 2 + i, i <= j
            int j = (int)((std::sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
            while ((int64_t)j * (j + 1) / 2 > p) --j;
            while ((int64_t)(j + 1) * (j + 2) / 2 <= p) ++j;
            const int i = p - j * (j + 1) / 2;
            I = sg.ti0 + i;
            J = sg.ti0 + j;
            diag = i == j;
          }
          for (int rq = 0; rq < 4; ++rq) {
            const unsigned q1 = diag ? (unsigned)rq + 1 : 4u;
            const unsigned x = (unsigned)I | ((4u - q1) << kItemQ1Shift) |
                               (1u << kItemRowQShift) | ((unsigned)rq << kItemRqShift);
            plan->items.push_back(
                make_int2((int)x, J | (diag ? int(0x80000000u) : 0)));
          }
        }
        // equal shares of the segment's pairs: its tasks split by item
        // count, as for an enumerated segment
        const int end = (int)plan->items.size();
        const int64_t share = std::max<int64_t>(1, plan->seg_pairs[s] / std::max(1, end - begin));
        plan->item_pairs.resize(end, (int)std::min<int64_t>(share, INT32_MAX));
        sg.shape = kSegList;
        plan->seg_items[s] = make_int2(begin, end);
      }
    }
  }
  // A plan of enumerated tile pairs (or their 32-row items) takes at least
  // 32 items per task where it has them: a CTA runs its task's items one
  // per warp, so two tasks of 15 items on one SM took two item times where
  // one task of 30 takes one (12,004 atoms: 4,560 tile pairs).
  if (plan->quarters > 0) {
    int64_t items = 0;
    for (size_t s = 0; s < S; ++s) items += plan->seg_items[s].y - plan->seg_items[s].x;
    target_tasks =
        (int)std::max<int64_t>(1, std::min<int64_t>(target_tasks, (items + 31) / 32));
  }
  // Task counts: each segment's share of target_tasks, rounded down, then
  // the largest remainders get one more until the counts sum to exactly
  // target_tasks (each count within [1, the segment's items]). The CTAs
  // (one per SM) pull equal tasks, so a count a little above a multiple
  // of the SM count would make a few CTAs run one task more than the rest:
  // on spinel_10nm 457 tasks for 152 SMs took 6.34 ms, 608 took 5.06 ms.
  std::vector<int64_t> ns(S);
  std::vector<std::pair<double, size_t>> rem;
  int64_t nsum = 0;
  for (size_t s = 0; s < S; ++s) {
    const int64_t items = plan->seg_items[s].y - plan->seg_items[s].x;
    const double q = total > 0 ? (double)plan->seg_pairs[s] * target_tasks / total : 1.0;
    ns[s] = std::max<int64_t>(1, std::min<int64_t>(items, (int64_t)std::floor(q)));
    nsum += ns[s];
    if (ns[s] < items) rem.emplace_back(q - (double)ns[s], s);
  }
  std::stable_sort(rem.begin(), rem.end(),
                   [](const auto &x, const auto &y) { return x.first > y.first; });
  for (size_t k = 0; k < rem.size() && nsum < target_tasks; ++k, ++nsum)
    ++ns[rem[k].second];
  for (size_t s = 0; s < S; ++s) {
    HistSeg &sg = plan->segs[s];
    sg.task_begin = (int)plan->tasks.size();
    const int i0 = plan->seg_items[s].x, i1 = plan->seg_items[s].y;
    const int64_t n_s = ns[s];
    if (sg.shape != kSegList) {
      for (int64_t k = 0; k < n_s; ++k) {
        const int b = (int)(i0 + (i1 - i0) * k / n_s);
        const int e = (int)(i0 + (i1 - i0) * (k + 1) / n_s);
        if (e > b) plan->tasks.push_back(HistTask{(int)s, b, e, 0});
      }
    } else {
      int64_t acc = 0, k = 1;
      int begin = i0;
      for (int i = i0; i < i1; ++i) {
        acc += plan->item_pairs[i];
        // close task k when the running sum reaches k/n_s of the segment
        if (i + 1 == i1 || (k < n_s && acc * n_s >= k * plan->seg_pairs[s])) {
          plan->tasks.push_back(HistTask{(int)s, begin, i + 1, 0});
          begin = i + 1;
          ++k;
        }
      }
    }
    sg.task_end = (int)plan->tasks.size();
  }
  // Pull order: decreasing binned pairs (longest task first), ties in task
  // order. Implicit segments' tasks are costed by their share of items.
  std::vector<double> cost(plan->tasks.size());
  for (size_t t = 0; t < plan->tasks.size(); ++t) {
    const HistTask &tk = plan->tasks[t];
    const int2 si = plan->seg_items[tk.seg];
    if (plan->segs[tk.seg].shape != kSegList) {
      cost[t] = (double)plan->seg_pairs[tk.seg] * (tk.item_end - tk.item_begin) /
                std::max(1, si.y - si.x);
    } else {
      double c = 0;
      for (int i = tk.item_begin; i < tk.item_end; ++i) c += plan->item_pairs[i];
      cost[t] = c;
    }
  }
  std::vector<int> order(plan->tasks.size());
  for (size_t t = 0; t < order.size(); ++t) order[t] = (int)t;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return cost[x] > cost[y]; });
  for (size_t k = 0; k < order.size(); ++k) plan->tasks[k].next = order[k];
}

void hist_plan_append(HistPlan *plan, const HistPlan &part, const float4 *atoms,
                      const int2 *tiles, const TileBox *boxes,
                      unsigned long long *out) {
  auto rebase = [&](unsigned long long *p) {
    return reinterpret_cast<unsigned long long *>(reinterpret_cast<uintptr_t>(out) +
                                                  reinterpret_cast<uintptr_t>(p));
  };
  const int ibase = (int)plan->items.size();
  plan->items.insert(plan->items.end(), part.items.begin(), part.items.end());
  plan->item_pairs.insert(plan->item_pairs.end(), part.item_pairs.begin(),
                          part.item_pairs.end());
  for (size_t i = 0; i < part.segs.size(); ++i) {
    HistSeg s = part.segs[i];
    s.atoms = atoms;
    s.tiles = tiles;
    s.boxes = boxes;
    s.out = rebase(s.out);
    plan->segs.push_back(s);
    int2 si = part.seg_items[i];
    if (s.shape == kSegList) si = make_int2(si.x + ibase, si.y + ibase);
    plan->seg_items.push_back(si);
    plan->seg_pairs.push_back(part.seg_pairs[i]);
  }
  for (const HistRow &r : part.rows) plan->rows.push_back(HistRow{rebase(r.out), r.len});
  plan->window = std::max(plan->window, part.window);
  plan->nrows += part.nrows;
  plan->pairs += part.pairs;
}

Error hist_plan(const Model &m, const std::vector<int2> &pairs, double rstep,
                int64_t nbins, unsigned long long *out, int64_t pitch,
                int target_tasks, HistPlan *plan) {
  hist_plan_clear(plan);
  DBX_TRY(hist_plan_add(m, pairs, rstep, nbins, out, pitch, plan));
  hist_plan_tasks(plan, target_tasks);
  return ok();
}

Error hist_upload(const HistPlan &plan, HistWorkspace *ws, cudaStream_t stream,
                  size_t *ws_bytes_delta) {
  const int ntasks = (int)plan.tasks.size();
  const int nsegs = (int)plan.segs.size();
  const cudaStream_t as = ws->alloc_stream;
  DBX_TRY(buf_grow(&ws->items, std::max<size_t>(plan.items.size(), 1) * sizeof(int2),
                   ws_bytes_delta, as));
  DBX_TRY(buf_grow(&ws->segs, std::max(nsegs, 1) * sizeof(HistSeg), ws_bytes_delta, as));
  DBX_TRY(buf_grow(&ws->tasks, std::max(ntasks, 1) * sizeof(HistTask), ws_bytes_delta, as));
  DBX_TRY(buf_grow(&ws->rows, std::max<size_t>(plan.rows.size(), 1) * sizeof(HistRow),
                   ws_bytes_delta, as));
  if (!plan.rows.empty())
    DBX_TRY(h2d_copy(ws->rows.p, plan.rows.data(), plan.rows.size() * sizeof(HistRow),
                     stream, ws->arena));
  if (ntasks == 0) return ok();
  if (!plan.items.empty())
    DBX_TRY(h2d_copy(ws->items.p, plan.items.data(), plan.items.size() * sizeof(int2),
                     stream, ws->arena));
  DBX_TRY(h2d_copy(ws->segs.p, plan.segs.data(), nsegs * sizeof(HistSeg), stream,
                   ws->arena));
  DBX_TRY(h2d_copy(ws->tasks.p, plan.tasks.data(), ntasks * sizeof(HistTask), stream,
                   ws->arena));
  return ok();
}

Error hist_scratch(const HistPlan &plan, HistWorkspace *ws,
                   size_t *ws_bytes_delta) {
  int max_wl = 0;
  for (const HistSeg &s : plan.segs) max_wl = std::max(max_wl, s.wl);
  const int words = (max_wl + 1) / 2;
  DBX_TRY(buf_grow(&ws->partial,
                   std::max<size_t>((size_t)plan.tasks.size() * words, 1) * 4,
                   ws_bytes_delta, ws->alloc_stream));
  DBX_TRY(buf_grow(&ws->oor, 2 * sizeof(unsigned long long), ws_bytes_delta,
                   ws->alloc_stream));
  // The tile kernel's shared-memory opt-in, once per device (kept out of
  // hist_launch so that a graph capture of it holds only stream work).
  static bool attr_done[64] = {false};
  int dev = 0;
  DBX_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64 || !attr_done[dev]) {
    DBX_CUDA_TRY(cudaFuncSetAttribute(hist_tiles_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kHistSmemBytes));
    if (dev >= 0 && dev < 64) attr_done[dev] = true;
  }
  return ok();
}

Error hist_launch(const HistPlan &plan, const HistWorkspace &lists,
                  HistWorkspace *ws, float inv_rstep, cudaStream_t stream,
                  int num_sms, size_t *ws_bytes_delta, Timers *tm) {
  const int ntasks = (int)plan.tasks.size();
  const int nsegs = (int)plan.segs.size();
  int max_wl = 0;
  for (const HistSeg &s : plan.segs) max_wl = std::max(max_wl, s.wl);
  const int words = (max_wl + 1) / 2;
  DBX_TRY(hist_scratch(plan, ws, ws_bytes_delta));
  if (!plan.rows.empty()) {  // a few rows (one model): several blocks each
    const unsigned per_row = plan.rows.size() < 64 ? 16u : 1u;
    hist_zero_kernel<<<dim3((unsigned)plan.rows.size(), per_row), 256, 0, stream>>>(
        (const HistRow *)lists.rows.p);
  }
  // oor counter and the task counter share one 16-byte buffer
  DBX_CUDA_TRY(cudaMemsetAsync(ws->oor.p, 0, 2 * sizeof(unsigned long long), stream));
  if (ntasks == 0) return ok();
  const int grid = std::min(ntasks, num_sms);
  tm->start(DBX_T_HIST, stream);
  hist_tiles_kernel<<<grid, kHistThreads, (words + kSpareWords) * 4,
                      stream>>>(
      (const int2 *)lists.items.p, (const HistTask *)lists.tasks.p, ntasks,
      (const HistSeg *)lists.segs.p, inv_rstep, (unsigned *)ws->partial.p,
      words, (unsigned long long *)ws->oor.p,
      (int *)((unsigned long long *)ws->oor.p + 1));
  DBX_CUDA_TRY(cudaGetLastError());
  tm->stop(DBX_T_HIST, stream);
  tm->start(DBX_T_HIST_REDUCE, stream);
  dim3 rgrid((words + 255) / 256, nsegs);
  hist_reduce_kernel<<<rgrid, 256, 0, stream>>>((const unsigned *)ws->partial.p,
                                                words,
                                                (const HistSeg *)lists.segs.p);
  DBX_CUDA_TRY(cudaGetLastError());
  tm->stop(DBX_T_HIST_REDUCE, stream);
  return ok();
}

Error hist_plain(const Model &m, int row, int col, float inv_rstep,
                 int64_t nbins, unsigned long long *out, HistWorkspace *ws,
                 cudaStream_t stream, size_t *ws_bytes_delta) {
  DBX_TRY(buf_grow(&ws->oor, 2 * sizeof(unsigned long long), ws_bytes_delta,
                   ws->alloc_stream));
  DBX_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(unsigned long long) * nbins, stream));
  DBX_CUDA_TRY(cudaMemsetAsync(ws->oor.p, 0, 2 * sizeof(unsigned long long), stream));
  const int na = (int)m.sp_count[row], nb = (int)m.sp_count[col];
  if (na == 0 || nb == 0) return ok();
  dim3 block(16, 16), grid((nb + 15) / 16, (na + 15) / 16);
  plain_pairs_kernel<<<grid, block, 0, stream>>>(
      m.d_atoms, m.sp_start[row], na, m.sp_start[col], nb, row == col, inv_rstep,
      (unsigned)nbins, out, (unsigned long long *)ws->oor.p);
  DBX_CUDA_TRY(cudaGetLastError());
  return ok();
}

Error hist_range_error(unsigned long long oor) {
  if (oor)
    return fail(DBX_ERR_RANGE, std::to_string(oor) +
                                   " distances bin at or beyond rmax; "
                                   "increase rmax");
  return ok();
}

Error hist_range_check(const HistWorkspace &ws, cudaStream_t stream) {
  unsigned long long oor = 0;
  if (ws.oor.p)
    DBX_CUDA_TRY(cudaMemcpyAsync(&oor, ws.oor.p, sizeof(oor),
                                 cudaMemcpyDeviceToHost, stream));
  DBX_CUDA_TRY(cudaStreamSynchronize(stream));
  return hist_range_error(oor);
}

Error hist_run(const HistPlan &plan, float inv_rstep, HistWorkspace *ws,
               cudaStream_t stream, int num_sms, size_t *ws_bytes_delta,
               Timers *tm) {
  DBX_TRY(hist_upload(plan, ws, stream, ws_bytes_delta));
  DBX_TRY(hist_launch(plan, *ws, ws, inv_rstep, stream, num_sms, ws_bytes_delta,
                      tm));
  return hist_range_check(*ws, stream);
}

}  // namespace dbx
