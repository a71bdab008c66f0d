// engine.h — internal declarations of the GB300 Debye engine (not part of
// the C ABI; see include/cudebye.h for that).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/cudebye.h"

namespace dbx {

// ---- error plumbing ------------------------------------------------------
struct Error {
  int code;
  std::string msg;
};

#define DBX_CUDA_TRY(expr)                                                   \
  do {                                                                       \
    cudaError_t e_ = (expr);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return ::dbx::Error{DBX_ERR_CUDA,                                      \
                          std::string(#expr) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

#define DBX_TRY(expr)                  \
  do {                                 \
    ::dbx::Error e_ = (expr);          \
    if (e_.code != DBX_OK) return e_;  \
  } while (0)

inline Error ok() { return Error{DBX_OK, std::string()}; }
inline Error fail(int code, const std::string &m) { return Error{code, m}; }

// ---- phase timers ----------------------------------------------------------
// CUDA-event timing of the phases of a call, on the launching stream.
struct Timers {
  bool on = false;
  bool created = false;
  cudaEvent_t ev[DBX_NTIMERS][2];
  bool recorded[DBX_NTIMERS] = {};
  void reset() {
    for (bool &r : recorded) r = false;
  }
  void start(int i, cudaStream_t s) {
    if (on) {
      cudaEventRecord(ev[i][0], s);
      recorded[i] = true;
    }
  }
  void stop(int i, cudaStream_t s) {
    if (on) cudaEventRecord(ev[i][1], s);
  }
};

// ---- device buffers -------------------------------------------------------
// Growable device buffer owned by a context; memory is accounted against the
// context's HBM budget by the owner.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

// Pinned host staging for host-to-device copies queued behind other work
// on a stream: a copy from pageable memory makes the host wait for the
// stream's earlier work, one from pinned memory does not. Space taken stays
// valid until reset(), which the owner calls once the stream's earlier
// copies are done (e.g. at the start of a server round on an idle lane).
struct PinArena {
  std::vector<std::pair<char *, size_t>> chunks;
  size_t used = 0;  // bytes used in the last chunk
  void *take(size_t n);  // n bytes, 16-byte aligned; nullptr if out of memory
  void reset();          // one chunk of the total size, empty
  void release();
  PinArena() = default;
  PinArena(const PinArena &) = delete;
  PinArena &operator=(const PinArena &) = delete;
  ~PinArena() { release(); }
};
// dst <- src (n bytes) on `stream`, through `arena` when it is not null.
Error h2d_copy(void *dst, const void *src, size_t n, cudaStream_t stream,
               PinArena *arena);
// Grow b to at least `bytes` (contents not kept; *delta tracks the bytes
// held). With `stream` the old buffer is freed and the new one allocated in
// stream order, without a device synchronisation (for buffers used on that
// stream only); without, cudaFree / cudaMalloc.
Error buf_grow(DevBuf *b, size_t bytes, size_t *delta, cudaStream_t stream);

// ---- resident model -------------------------------------------------------
// Atoms are stored per species, each species sorted along a Hilbert curve
// and cut into tiles of kTile atoms, so that a tile is spatially compact and
// a tile pair covers a narrow window of distances.
constexpr int kTile = 128;

// Bounding box of a tile, and of its column quarters (atoms [32 q, 32 q +
// 32), the columns one pass of a warp's lanes reads), for the planner of
// multi-window histograms. A box with a NaN coordinate is all NaN; an empty
// quarter is (+inf, -inf).
constexpr int kQuarter = 32;
struct TileBox {
  float lo[3], hi[3];
  float qlo[4][3], qhi[4][3];
};

struct Model {
  int64_t id = 0;
  int nspecies = 0;
  int64_t natoms = 0;
  std::vector<int64_t> sp_start, sp_count;  // in atoms (sorted layout)
  std::vector<int> tile_start;              // first tile of each species (+ end)
  std::vector<int2> tiles;                  // {first atom, count}
  std::vector<TileBox> boxes;               // per tile (host; for device-
                                            // sorted models filled on demand)
  float4 *d_atoms = nullptr;                // natoms x (x, y, z, 0)
  int2 *d_tiles = nullptr;
  TileBox *d_boxes = nullptr;               // per tile (device)
  size_t dev_bytes = 0;
  // Cached histogram plan of all pairs for (plan_rstep, plan_nbins): the
  // work lists depend only on the geometry and the binning.
  double plan_rstep = 0;
  int64_t plan_nbins = 0;
  struct HistPlanCache *plan_cache = nullptr;
  unsigned long long *plan_out = nullptr;   // d_hist the plan writes to
  size_t plan_bytes = 0;
  // Resident histograms (for re-scoring with new K or species).
  double hist_rstep = 0;
  int64_t hist_nbins = 0;
  int64_t hist_pitch = 0;                 // nbins padded, in int64
  unsigned long long *d_hist = nullptr;   // [npairs][pitch]
  size_t hist_bytes = 0;
};

// Model building (model.cu): host-side sort, tiles and boxes; device copy;
// release.
// atoms: room for max(natoms, 1) float4 (host memory, pinned or not).
Error model_prepare(const float *x, const float *y, const float *z,
                    const int64_t *counts, int nspecies, Model *m,
                    float4 *atoms);
size_t model_upload_bytes(const Model &m);
// Copies max(natoms, 1) atoms; from pinned memory the copy is asynchronous
// and `atoms` must stay untouched until it completes on `stream`.
Error model_to_device(Model *m, const float4 *atoms, cudaStream_t stream,
                      PinArena *arena = nullptr);
size_t model_device_bytes(const Model &m);  // atoms, tiles, hist, plan
// Sort and upload on the device (spatial_sort.cu): the same atoms, tiles and
// boxes as model_prepare + model_to_device; `pin` is pinned host memory
// of pin_bytes >= 12 natoms bytes (the coordinates; small arrays go
// through the rest where it fits); the tile boxes stay on the device
// (d_boxes) until model_host_boxes copies them for a multi-window plan.
// Coordinates as SoA planes x, y, z, or (xyz not null) one interleaved
// [natoms][3] array. For natoms > 0.
Error model_upload_sorted(Model *m, const float *x, const float *y, const float *z,
                          const float *xyz, const int64_t *counts, int nspecies,
                          float *pin, size_t pin_bytes, cudaStream_t stream);
Error model_host_boxes(Model *m, cudaStream_t stream);
void model_release(Model *m);
// The same, device arrays freed in `stream` order (no device-wide wait);
// for a model no queued or running work uses.
void model_release_async(Model *m, cudaStream_t stream);

inline int npairs_of(int p) { return p * (p + 1) / 2; }
inline int pair_index(int p, int row, int col) {
  return row * p - row * (row - 1) / 2 + (col - row);
}

// ---- histogram planner + kernels (hist.cu) --------------------------------
struct HistSeg {  // one (model, pair, bin window) accumulated in smem
  const float4 *atoms;      // the model's atoms
  const int2 *tiles;        // the model's tiles
  const TileBox *boxes;     // the model's tile boxes (device)
  unsigned long long *out;  // the pair's histogram, bin 0
  int kb;                   // first bin of the window
  int wl;                   // window length in bins
  int task_begin, task_end;
  unsigned nbins;           // bins of this histogram
  // Item source: kSegList reads {I | q0 << 25 | (4 - q1) << 27, J | diag
  // << 31} from the plan's item list (the item covers the columns of
  // quarters [q0, q1) of tile J: all of them when the bits are 0);
  // kSegRect enumerates tiles ti0 + [0, tni) x tj0 + [0, tnj) and kSegTri
  // the pairs I <= J of ti0 + [0, tni) (a species with itself), item index
  // = task-local position.
  int shape;
  int ti0, tni, tj0, tnj;
  // Bins of the window this segment counts, window-relative: [own_lo,
  // own_lo + own_len); the whole window (0, wl) unless overlapping windows
  // of a histogram share bins. own_lo is even, and own_lo + own_len is even
  // or the window's end.
  int own_lo, own_len;
};
constexpr int kSegList = 0, kSegRect = 1, kSegTri = 2;
constexpr int kItemQ0Shift = 25, kItemQ1Shift = 27;
// bit 29: a 32-row item (rows [32 rq, 32 rq + 32) of tile I, rq in bits
// 30-31), listed in multi-window histograms only
constexpr int kItemRowQShift = 29, kItemRqShift = 30;
constexpr int kItemTileMask = (1 << 25) - 1;
struct HistTask {  // one CTA-sized slice of a segment's tile pairs
  int seg;
  int item_begin, item_end;
  int next;  // the task that the k-th pull of the task counter runs (entry k)
};
struct HistRow {  // an output histogram to zero before a launch
  unsigned long long *out;
  long long len;
};

double hist_rowq_default();  // DBX_HIST_ROWQ, else the measured default
constexpr int kGeomSampled = 0, kGeomDisjoint = 1, kGeomOverlap = 2;

struct HistPlan {
  std::vector<int2> items;     // {tile I, tile J | (diag << 31)}
  std::vector<int> item_pairs; // pairs of each item (host only)
  std::vector<HistSeg> segs;
  std::vector<int2> seg_items; // item range of each segment (host only;
                               // [0, count) for enumerated segments)
  std::vector<int64_t> seg_pairs; // binned pairs of each segment (host only)
  std::vector<HistTask> tasks;
  std::vector<HistRow> rows;
  int window = 0;              // largest window in bins
  int nrows = 0;               // output histograms
  // 32-row items are listed in multi-window histograms where they cut an
  // item's pairs by more than this factor (0: never); not reset by
  // hist_plan_clear
  double rowq = hist_rowq_default();
  // window geometry of multi-window histograms: chosen per species pair
  // from sampled tile pairs (kGeomSampled), or forced; not reset by
  // hist_plan_clear
  int geom = 0;
  // a plan of enumerated segments only: 1 if they became lists of 32-row
  // items (a small plan), 2 if not; 0 for a plan with listed segments;
  // decided by hist_plan_tasks on its first split of the plan (-1 until
  // then); reset by hist_plan_clear
  int quarters = -1;
  int64_t pairs = 0;           // binned pairs (the reference's "Distances
                               // Expected" summed over the selected pairs)
  size_t upload_bytes() const {
    return items.size() * sizeof(int2) + segs.size() * sizeof(HistSeg) +
           tasks.size() * sizeof(HistTask) + rows.size() * sizeof(HistRow);
  }
};

// Plans: clear, add the pairs of one or more models (histogram of pairs[i]
// written to out + i*pitch; pitch >= nbins + 2: the two bins past the end
// absorb the carry bookkeeping of the packed counters), then split the
// segments into about target_tasks CTA tasks of equal pair counts.
void hist_plan_clear(HistPlan *plan);
Error hist_plan_add(const Model &m, const std::vector<int2> &pairs,
                    double rstep, int64_t nbins, unsigned long long *out,
                    int64_t pitch, HistPlan *plan);
void hist_plan_tasks(HistPlan *plan, int target_tasks);
// Append a plan made for a model whose device arrays did not exist yet
// (device pointers null, out = nullptr: output rows are byte offsets), with
// the model's atoms, tiles and histogram base filled in.
void hist_plan_append(HistPlan *plan, const HistPlan &part, const float4 *atoms,
                      const int2 *tiles, const TileBox *boxes,
                      unsigned long long *out);
// clear + add + tasks for one model
Error hist_plan(const Model &m, const std::vector<int2> &pairs, double rstep,
                int64_t nbins, unsigned long long *out, int64_t pitch,
                int target_tasks, HistPlan *plan);

struct HistWorkspace {  // device-side work lists and scratch
  DevBuf items, segs, tasks, rows, partial, oor;
  PinArena *arena = nullptr;          // staging of the list uploads
  cudaStream_t alloc_stream = nullptr;  // stream-ordered growth (buf_grow)
};

struct HistPlanCache {  // a plan and its uploaded work lists
  HistPlan plan;
  HistWorkspace lists;
};

// Copy a plan's work lists (items, segments, tasks, rows) to the device.
Error hist_upload(const HistPlan &plan, HistWorkspace *lists,
                  cudaStream_t stream, size_t *ws_bytes_delta);
// Allocate the scratch a plan needs (partial windows, counters).
Error hist_scratch(const HistPlan &plan, HistWorkspace *scratch,
                   size_t *ws_bytes_delta);
// Launch the histograms of an uploaded plan: outputs zeroed, tile kernel,
// reduce. Pairs binned at k >= nbins are counted in scratch->oor on the
// device; read them with hist_range_check. Asynchronous; only kernels and
// memsets, so it can be captured in a CUDA graph once hist_scratch has run.
Error hist_launch(const HistPlan &plan, const HistWorkspace &lists,
                  HistWorkspace *scratch, float inv_rstep, cudaStream_t stream,
                  int num_sms, size_t *ws_bytes_delta, Timers *tm);
// The plain form of the reference's kernels dist / dist2 (cuDebye-v15.cu:
// 88-146): one thread per pair of the species block (row, col) of model m,
// one global 64-bit atomicAdd per pair into out[nbins] (zeroed here).
// Pairs at k >= nbins are counted in scratch->oor. The comparison baseline
// of the "plain unbatched FP32 GPU form".
Error hist_plain(const Model &m, int row, int col, float inv_rstep,
                 int64_t nbins, unsigned long long *out, HistWorkspace *scratch,
                 cudaStream_t stream, size_t *ws_bytes_delta);

// Wait for the stream; DBX_ERR_RANGE if the last launch binned any pair at
// k >= nbins.
Error hist_range_check(const HistWorkspace &scratch, cudaStream_t stream);
// DBX_ERR_RANGE with the count when oor (out-of-range distances) is not 0.
Error hist_range_error(unsigned long long oor);
// upload + launch + range check
Error hist_run(const HistPlan &plan, float inv_rstep, HistWorkspace *ws,
               cudaStream_t stream, int num_sms, size_t *ws_bytes_delta,
               Timers *tm);

int hist_window_bins();  // shared-memory window capacity in bins
// Device check of the histogram kernels' square root (dbx_check_sqrt).
Error check_sqrt(unsigned lo, unsigned hi, int num_sms, cudaStream_t stream,
                 int64_t out[3]);

// ---- Debye kernels (debye.cu) ----------------------------------------------
struct PrefState {  // species and column descriptors of a batched prefactor
  DevBuf sp, colsp, f, fid;  // f: form factors [distinct set][q]; fid:
                             // species -> row of f, then row -> species
  int ncols = 0, nsp = 0;
  PinArena *arena = nullptr;            // staging of the uploads
  cudaStream_t alloc_stream = nullptr;  // stream-ordered growth (buf_grow)
};
// Upload species (concatenated) and per-column species pairs {a, b}; room
// for the form factors of nq q values.
Error prefactor_upload(PrefState *st, const dbx_species *sp, int nsp,
                       const int2 *col_sp, int ncols, int nq,
                       cudaStream_t stream, size_t *bytes_delta);
// ff[c][q] for every column (kernel only; capturable).
Error prefactor_execute(const PrefState &st, const double *d_K, int nq,
                        double *d_ff, cudaStream_t stream);
// out_ff[p][q] for every pair of the model's species.
// (the species go to the device through `arena` when it is not null)
Error debye_prefactor(const dbx_species *sp, int nspecies, const double *d_K,
                      int nq, double *d_ff, cudaStream_t stream,
                      PinArena *arena = nullptr);
// I[q] = sum_p ff[p][q] * sum_k m_k sinc(K r_k) over the model's histograms.
Error debye_direct(int mode, const unsigned long long *d_hist, int npairs,
                   int64_t pitch, int64_t nbins, double rstep,
                   const double *d_K, int nq, const double *d_ff, double *d_I,
                   cudaStream_t stream);

}  // namespace dbx
