// debye_tc.h — tensor-core Debye contraction (debye_tc.cu).
#pragma once
#include <vector>

#include "engine.h"

namespace dbx {

struct TcTile {  // 64 consecutive chunks of one column
  int col, ch0, pad0, pad1;
};

struct TcCol {  // one (model, species pair) column of the contraction
  const unsigned long long *hist;  // device counts [nbins]
  long long nbins;
  const double *ff;                // device prefactor [nq]
  int tile_begin, tile_end;        // filled by tc_prepare
  double self;                     // self-distance sum, filled on the device
};

struct TcState {  // cached plan data (basis, twiddles) and workspace
  DevBuf basis, twid, W, E, P, tiles, cols, mcb, nonself, err;
  std::vector<double> grid_K;
  double grid_rstep = 0;
  int grid_nch = 0;
  int64_t h2d = 0, d2h = 0;
  // shape of the prepared contraction
  int ncols = 0, nmodels = 0, ntiles = 0, nq = 0, Qp = 0;
  int num_sms = 0;  // persistent contraction: one CTA per SM
  // operand form: 0 = the exact split (4 bf16 digits, 10 products); 1 =
  // BF16x3 (2 digits, 3 products) and 2 = TF32x3 (2 tf32 parts, 3
  // products), used only to compare precisions
  int form = 0;
  bool grid_tf32 = false;  // the cached basis is in the tf32 layout
  // incremented by every tc_prepare: a caller that replays a prepared
  // contraction (a captured graph) checks that nobody prepared another one
  // on this state since
  uint64_t prep_gen = 0;
  double rstep = 0;
  double *S_out = nullptr;  // optional: per-column row sums S[c][q]
  PinArena *arena = nullptr;            // staging of the descriptor uploads
  cudaStream_t alloc_stream = nullptr;  // stream-ordered growth (buf_grow)
};

// Host part: column tiles, descriptors uploaded, basis and twiddles for a
// new q grid. The columns are grouped by model (model_col_begin has
// nmodels+1 offsets into cols, columns of a model in pair order).
Error tc_prepare(TcState *st, std::vector<TcCol> cols,
                 const std::vector<int> &model_col_begin, double rstep,
                 const double *h_K, const double *d_K, int nq,
                 cudaStream_t stream, size_t *bytes_delta);
// Device part: I[model][q] (kernels and memsets only; capturable).
Error tc_execute(TcState *st, const double *d_K, double *d_I,
                 cudaStream_t stream, Timers *tm);
// I[q] = sum_c ff[c][q] * S[c][q] (re-scoring resident row sums).
Error tc_combine(const double *d_ff, const double *d_S, int ncols, int nq,
                 double *d_I, cudaStream_t stream);
// Wait; DBX_ERR_TIMEOUT if a bounded device wait ran out.
Error tc_check(TcState *st, cudaStream_t stream);
// The status of a contraction from its error word read back by the caller.
Error tc_status(int herr);
void tc_release(TcState *st);
size_t tc_bytes(const TcState *st);

}  // namespace dbx
