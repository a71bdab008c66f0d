// capi.cu — context, resident models and the C ABI (include/cudebye.h).
#include <cuda_runtime.h>
#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#include <map>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "curve.cuh"
#include "debio.h"
#include "debye_tc.h"
#include "engine.h"

using dbx::Error;

// The prepared state of the last dbx_patterns batch.
struct BatchState {
  std::vector<int64_t> ids, nbins;
  std::vector<const void *> hist_ptrs;  // the models' histogram buffers
  double rstep = 0;
  std::vector<double> K;
  dbx::HistPlanCache hp;
  std::vector<int> model_col_begin;
  std::vector<int2> col_sp;
  int nsp = 0;
  dbx::PrefState pref;
  dbx::DevBuf ff, I, K_dev;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<const void *> graph_ptrs;  // buffers the graph was built on
  int tuned_tasks = 0;
  struct Tune {  // the autotuner's choice for this batch (dbx_batch_tuning)
    int tasks = 0, geom = 0, shapes = 0, task_counts = 0;
    double rowq = 0;
    bool multi = false;
    float ms = 0;
  } tune;
  uint64_t tc_gen = 0;  // the contraction state's preparation of this batch
  bool valid = false;
};

struct dbx_ctx {
  int device = 0;
  int num_sms = 0;
  int hist_tasks = 0;  // histogram CTA tasks per launch of a batch
  int hist_tasks_env = 0;  // DBX_HIST_TASKS, when set
  size_t budget = 0;  // 0 = no limit
  size_t used = 0;    // device bytes held
  cudaStream_t stream = nullptr;      // launch stream (own or caller's)
  cudaStream_t own_stream = nullptr;
  // a single pattern's prefactors run here beside a histogram that leaves
  // SMs free, joined back into `stream` by the event
  cudaStream_t side_stream = nullptr;
  cudaEvent_t join_ev = nullptr;
  float4 *pin = nullptr;              // pinned staging of model uploads
  size_t pin_cap = 0;                 // in atoms
  cudaEvent_t pin_ev = nullptr;       // the last upload's copy is done
  bool pin_used = false;
  dbx::Timers tm;
  int64_t h2d = 0, d2h = 0;           // bytes copied (dbx_get_traffic)
  std::map<int64_t, std::unique_ptr<dbx::Model>> models;
  int64_t next_id = 1;
  // Pinned staging of the host-to-device copies made while a call queues
  // its work (a copy from pageable memory would make the host wait for the
  // histogram just launched); reset at the start of the calls that use it,
  // all of which end synchronised.
  dbx::PinArena arena;
  dbx::HistWorkspace hws;
  dbx::TcState tc;
  dbx::DevBuf tmp_hist, K, ff, I;
  BatchState batch;
  bool graphs = true;
  std::string last_error;
};

namespace {

int set_err(dbx_ctx *c, const Error &e) {
  if (c && e.code != DBX_OK) c->last_error = e.msg;
  return e.code;
}

Error grow(dbx_ctx *c, dbx::DevBuf *b, size_t bytes) {
  if (b->bytes >= bytes) return dbx::ok();
  if (b->p) {
    cudaFree(b->p);
    c->used -= b->bytes;
    b->p = nullptr;
    b->bytes = 0;
  }
  if (c->budget && c->used + bytes > c->budget)
    return dbx::fail(DBX_ERR_NOMEM, "HBM budget exceeded (" +
                                        std::to_string(c->used + bytes) + " > " +
                                        std::to_string(c->budget) + " bytes)");
  DBX_CUDA_TRY(cudaMalloc(&b->p, bytes));
  b->bytes = bytes;
  c->used += bytes;
  return dbx::ok();
}

void release(dbx_ctx *c, dbx::DevBuf *b) {
  if (b->p) cudaFree(b->p);
  c->used -= b->bytes;
  b->p = nullptr;
  b->bytes = 0;
}

// The model's device arrays are freed in the context stream's order: work
// queued on it before (an upload still copying) finishes first, and no
// device-wide wait is made.
void free_model(dbx_ctx *c, dbx::Model *m) {
  c->used -= dbx::model_device_bytes(*m);
  dbx::model_release_async(m, c->stream);
}

dbx::Model *find_model(dbx_ctx *c, int64_t id) {
  auto it = c->models.find(id);
  return it == c->models.end() ? nullptr : it->second.get();
}

int64_t pitch_of(int64_t nbins) { return (nbins + 2 + 1) & ~int64_t(1); }

// Histogram CTA tasks of one model's plan: 2 per SM when one window holds
// the histogram (equal segments; every task boundary costs a window
// zeroing and write-out: spinel_10nm 5.02 ms vs 5.06 at 4 per SM), 8 per
// SM when several windows split it (segments of many sizes; finer tasks
// fill the largest-first tail: Gamma sample 26.3 vs 26.7 ms).
// DBX_HIST_TASKS overrides both.
int model_tasks(const dbx_ctx *c, int64_t nbins) {
  if (c->hist_tasks_env > 0) return c->hist_tasks_env;
  return (nbins > dbx::hist_window_bins() ? 8 : 2) * c->num_sms;
}

// Histograms of all pairs, kept resident in the model. The work lists are
// planned and uploaded once per (model, rstep, nbins) and reused. With
// `launched` non-null the range check is left to the caller (who must call
// hist_range_check on c->hws after the stream work it queues behind it);
// *launched tells whether kernels were queued.
Error ensure_hist(dbx_ctx *c, dbx::Model *m, double rstep, int64_t nbins,
                  bool *launched = nullptr) {
  if (launched) *launched = false;
  if (m->d_hist && m->hist_rstep == rstep && m->hist_nbins == nbins)
    return dbx::ok();
  const int np = dbx::npairs_of(m->nspecies);
  const int64_t pitch = pitch_of(nbins);
  const size_t bytes = sizeof(unsigned long long) * (size_t)pitch * np;
  if (m->hist_bytes < bytes) {
    if (m->d_hist) cudaFreeAsync(m->d_hist, c->stream);
    c->used -= m->hist_bytes;
    m->d_hist = nullptr;
    m->hist_bytes = 0;
    if (c->budget && c->used + bytes > c->budget)
      return dbx::fail(DBX_ERR_NOMEM, "HBM budget exceeded by histograms");
    DBX_CUDA_TRY(cudaMallocAsync(&m->d_hist, bytes, c->stream));
    m->hist_bytes = bytes;
    c->used += bytes;
  }
  size_t delta = 0;
  if (!m->plan_cache || m->plan_rstep != rstep || m->plan_nbins != nbins ||
      m->plan_out != m->d_hist) {
    if (!m->plan_cache) {
      m->plan_cache = new dbx::HistPlanCache();
      m->plan_cache->lists.arena = &c->arena;
    }
    // list buffers grow in the order of the stream the context uses now
    // (dbx_set_stream may have changed it since the cache was made)
    m->plan_cache->lists.alloc_stream = c->stream;
    std::vector<int2> pairs;
    for (int r = 0; r < m->nspecies; ++r)
      for (int q = r; q < m->nspecies; ++q) pairs.push_back(make_int2(r, q));
    m->plan_rstep = 0;
    m->plan_nbins = 0;
    if (nbins > dbx::hist_window_bins()) DBX_TRY(dbx::model_host_boxes(m, c->stream));
    DBX_TRY(dbx::hist_plan(*m, pairs, rstep, nbins, m->d_hist, pitch,
                           model_tasks(c, nbins), &m->plan_cache->plan));
    const size_t before = delta;
    Error e = dbx::hist_upload(m->plan_cache->plan, &m->plan_cache->lists,
                               c->stream, &delta);
    m->plan_bytes += delta - before;
    c->used += delta;
    delta = 0;
    if (e.code) return e;
    c->h2d += m->plan_cache->plan.upload_bytes();
    m->plan_rstep = rstep;
    m->plan_nbins = nbins;
    m->plan_out = m->d_hist;
  }
  m->hist_rstep = 0;
  m->hist_nbins = 0;
  Error e = dbx::hist_launch(m->plan_cache->plan, m->plan_cache->lists, &c->hws,
                             (float)(1.0 / rstep), c->stream, c->num_sms,
                             &delta, &c->tm);
  c->used += delta;
  if (e.code != DBX_OK) return e;
  if (launched) {
    *launched = true;
  } else {
    c->d2h += sizeof(unsigned long long);
    DBX_TRY(dbx::hist_range_check(c->hws, c->stream));
  }
  m->hist_rstep = rstep;
  m->hist_nbins = nbins;
  m->hist_pitch = pitch;
  return dbx::ok();
}

Error copy_rows(dbx_ctx *c, const unsigned long long *d, int64_t pitch,
                int64_t nbins, int rows, int64_t *out) {
  DBX_CUDA_TRY(cudaMemcpy2DAsync(out, nbins * 8, d, pitch * 8, nbins * 8, rows,
                                 cudaMemcpyDeviceToHost, c->stream));
  c->d2h += nbins * 8 * rows;
  DBX_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return dbx::ok();
}

Error intensity(dbx_ctx *c, dbx::Model *m, double rstep, int64_t nbins,
                const dbx_species *sp, const double *K, int nq, int mode,
                double *out_I) {
  if (nq < 1) return dbx::fail(DBX_ERR_ARG, "nq must be >= 1");
  c->arena.reset();  // the previous call ended synchronised
  if (mode != DBX_DEBYE_TC && mode != DBX_DEBYE_TC3 && mode != DBX_DEBYE_TF32 &&
      mode != DBX_DEBYE_FP64 && mode != DBX_DEBYE_FP32)
    return dbx::fail(DBX_ERR_ARG, "unknown Debye mode");
  bool launched = false;
  DBX_TRY(ensure_hist(c, m, rstep, nbins, &launched));
  const int np = dbx::npairs_of(m->nspecies);
  DBX_TRY(grow(c, &c->K, sizeof(double) * nq));
  DBX_TRY(grow(c, &c->ff, sizeof(double) * nq * (size_t)np));
  DBX_TRY(grow(c, &c->I, sizeof(double) * nq));
  // The prefactors depend on K and the species only (from the host). Beside
  // a histogram of fewer CTA tasks than SMs (a small model) they run on the
  // side stream on the SMs it leaves free, and the contraction waits for
  // them (5,000 atoms: 0.193 -> 0.165 ms per pattern); beside a histogram
  // that fills every SM, in stream order. K goes through the pinned arena:
  // a copy from pageable memory would hold the host.
  const bool side = launched && c->side_stream && m->plan_cache &&
                    (int)m->plan_cache->plan.tasks.size() < c->num_sms;
  const cudaStream_t ps = side ? c->side_stream : c->stream;
  Error pe = dbx::h2d_copy(c->K.p, K, sizeof(double) * nq, ps, &c->arena);
  c->h2d += sizeof(double) * nq + sizeof(dbx_species) * m->nspecies;
  if (!pe.code) {
    c->tm.start(DBX_T_PREFACTOR, ps);
    pe = dbx::debye_prefactor(sp, m->nspecies, (const double *)c->K.p, nq,
                              (double *)c->ff.p, ps, &c->arena);
    c->tm.stop(DBX_T_PREFACTOR, ps);
  }
  if (pe.code) {
    cudaStreamSynchronize(ps);
    return pe;
  }
  if (side) {
    DBX_CUDA_TRY(cudaEventRecord(c->join_ev, ps));
    DBX_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->join_ev, 0));
  }
  const bool tc_form =
      mode == DBX_DEBYE_TC || mode == DBX_DEBYE_TC3 || mode == DBX_DEBYE_TF32;
  if (tc_form) {
    std::vector<dbx::TcCol> cols(np);
    for (int p = 0; p < np; ++p) {
      cols[p].hist = m->d_hist + (size_t)p * m->hist_pitch;
      cols[p].nbins = nbins;
      cols[p].ff = (const double *)c->ff.p + (size_t)p * nq;
    }
    size_t delta = 0;
    const int64_t h0 = c->tc.h2d, d0 = c->tc.d2h;
    c->tc.form = mode == DBX_DEBYE_TC3 ? 1 : mode == DBX_DEBYE_TF32 ? 2 : 0;
    Error e = dbx::tc_prepare(&c->tc, cols, {0, np}, rstep, K, (const double *)c->K.p,
                              nq, c->stream, &delta);
    if (!e.code)
      e = dbx::tc_execute(&c->tc, (const double *)c->K.p, (double *)c->I.p, c->stream,
                          &c->tm);
    c->tc.form = 0;
    c->used += delta;
    c->h2d += c->tc.h2d - h0;
    c->d2h += c->tc.d2h - d0;
    if (e.code) return e;
  } else {
    c->tm.start(DBX_T_DEBYE, c->stream);
    DBX_TRY(dbx::debye_direct(mode, m->d_hist, np, m->hist_pitch, nbins, rstep,
                              (const double *)c->K.p, nq,
                              (const double *)c->ff.p, (double *)c->I.p,
                              c->stream));
    c->tm.stop(DBX_T_DEBYE, c->stream);
  }
  // What the host reads back — the contraction's wait-timeout word, the
  // histograms' out-of-range count (the range check deferred to here) and
  // the intensities — in one round trip through pinned staging, checked in
  // that order; without pinned memory, one synchronised copy each.
  const bool oor = launched && c->hws.oor.p;
  int *h_err = tc_form ? (int *)c->arena.take(sizeof(int)) : nullptr;
  unsigned long long *h_oor =
      oor ? (unsigned long long *)c->arena.take(sizeof(unsigned long long)) : nullptr;
  double *h_I = (double *)c->arena.take(sizeof(double) * nq);
  c->d2h += (tc_form ? sizeof(int) : 0) + (launched ? sizeof(unsigned long long) : 0) +
            sizeof(double) * nq;
  if ((tc_form && !h_err) || (oor && !h_oor) || !h_I) {
    if (tc_form) DBX_TRY(dbx::tc_check(&c->tc, c->stream));
    if (launched) {
      Error e = dbx::hist_range_check(c->hws, c->stream);
      if (e.code) {
        m->hist_nbins = 0;
        return e;
      }
    }
    DBX_CUDA_TRY(cudaMemcpyAsync(out_I, c->I.p, sizeof(double) * nq,
                                 cudaMemcpyDeviceToHost, c->stream));
    DBX_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return dbx::ok();
  }
  if (h_err)
    DBX_CUDA_TRY(cudaMemcpyAsync(h_err, c->tc.err.p, sizeof(int), cudaMemcpyDeviceToHost,
                                 c->stream));
  if (h_oor)
    DBX_CUDA_TRY(cudaMemcpyAsync(h_oor, c->hws.oor.p, sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, c->stream));
  DBX_CUDA_TRY(cudaMemcpyAsync(h_I, c->I.p, sizeof(double) * nq, cudaMemcpyDeviceToHost,
                               c->stream));
  DBX_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (h_err) DBX_TRY(dbx::tc_status(*h_err));
  if (h_oor && *h_oor) {
    m->hist_nbins = 0;
    return dbx::hist_range_error(*h_oor);
  }
  std::memcpy(out_I, h_I, sizeof(double) * nq);
  return dbx::ok();
}

// Histogram buffer of model m sized for nbins (resident afterwards).
Error alloc_hist(dbx_ctx *c, dbx::Model *m, int64_t nbins) {
  const int np = dbx::npairs_of(m->nspecies);
  const int64_t pitch = pitch_of(nbins);
  const size_t bytes = sizeof(unsigned long long) * (size_t)pitch * np;
  if (m->hist_bytes < bytes) {
    if (m->d_hist) cudaFreeAsync(m->d_hist, c->stream);
    c->used -= m->hist_bytes;
    m->d_hist = nullptr;
    m->hist_bytes = 0;
    if (c->budget && c->used + bytes > c->budget)
      return dbx::fail(DBX_ERR_NOMEM, "HBM budget exceeded by histograms");
    DBX_CUDA_TRY(cudaMallocAsync(&m->d_hist, bytes, c->stream));
    m->hist_bytes = bytes;
    c->used += bytes;
  }
  m->hist_pitch = pitch;
  return dbx::ok();
}

void drop_graph(BatchState *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->graph_ptrs.clear();
}

// The device work of one batch pass: histograms, prefactors, contraction.
Error batch_device_pass(dbx_ctx *c, dbx::Timers *tm) {
  BatchState &b = c->batch;
  size_t delta = 0;
  Error e = dbx::hist_launch(b.hp.plan, b.hp.lists, &c->hws, (float)(1.0 / b.rstep),
                             c->stream, c->num_sms, &delta, tm);
  c->used += delta;
  if (e.code) return e;
  DBX_TRY(dbx::prefactor_execute(b.pref, (const double *)b.K_dev.p, (int)b.K.size(),
                                 (double *)b.ff.p, c->stream));
  return dbx::tc_execute(&c->tc, (const double *)b.K_dev.p, (double *)b.I.p,
                         c->stream, tm);
}

// The histogram plan of a batch: every (model, species pair), with the
// plan's shape policy (window geometry, 32-row items) as set in b.hp.plan.
Error batch_plan(dbx_ctx *c, const std::vector<dbx::Model *> &ms, double rstep,
                 const int64_t *nbins, int tasks) {
  BatchState &b = c->batch;
  dbx::hist_plan_clear(&b.hp.plan);
  for (size_t i = 0; i < ms.size(); ++i) {
    dbx::Model *m = ms[i];
    std::vector<int2> pairs;
    for (int r = 0; r < m->nspecies; ++r)
      for (int q = r; q < m->nspecies; ++q) pairs.push_back(make_int2(r, q));
    if (nbins[i] > dbx::hist_window_bins()) DBX_TRY(dbx::model_host_boxes(m, c->stream));
    DBX_TRY(dbx::hist_plan_add(*m, pairs, rstep, nbins[i], m->d_hist, m->hist_pitch,
                               &b.hp.plan));
  }
  dbx::hist_plan_tasks(&b.hp.plan, tasks);
  size_t delta = 0;
  Error e = dbx::hist_upload(b.hp.plan, &b.hp.lists, c->stream, &delta);
  c->used += delta;
  return e;
}

// Device time of one histogram launch of the uploaded batch plan.
Error time_batch_hist(dbx_ctx *c, cudaEvent_t e0, cudaEvent_t e1, float *ms) {
  BatchState &b = c->batch;
  dbx::Timers off;
  size_t delta = 0;
  cudaEventRecord(e0, c->stream);
  Error e = dbx::hist_launch(b.hp.plan, b.hp.lists, &c->hws, (float)(1.0 / b.rstep),
                             c->stream, c->num_sms, &delta, &off);
  c->used += delta;
  if (e.code) return e;
  cudaEventRecord(e1, c->stream);
  DBX_CUDA_TRY(cudaEventSynchronize(e1));
  cudaEventElapsedTime(ms, e0, e1);
  return dbx::ok();
}

// The batch autotuner: times the histogram launch of the batch plan for
// each candidate shape and keeps the fastest. Candidates: when the plan
// splits histograms into several windows, the tile shape (32-row items
// where they list fewer pairs, or 128-row items only) and the window
// geometry (chosen per species pair from sampled tile pairs, or disjoint
// windows only); then the CTA task count ({4, 8, 16} x SMs) of the chosen
// shape. Every candidate gives the same histograms (integer sums).
Error autotune(dbx_ctx *c, const std::vector<dbx::Model *> &ms, double rstep,
               const int64_t *nbins) {
  BatchState &b = c->batch;
  dbx::HistPlan &plan = b.hp.plan;
  cudaEvent_t e0, e1;
  DBX_CUDA_TRY(cudaEventCreate(&e0));
  DBX_CUDA_TRY(cudaEventCreate(&e1));
  struct Ev {
    cudaEvent_t a, b;
    ~Ev() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } ev{e0, e1};
  // several windows per histogram: a segment's window does not start at
  // bin 0 or ends before the histogram's last bin (small one-window plans
  // list their items too)
  bool multi = false;
  for (const dbx::HistSeg &sg : plan.segs)
    multi |= sg.kb != 0 || (unsigned)sg.wl < sg.nbins;
  const int base_tasks = (multi ? 8 : 4) * c->num_sms;
  b.tune = BatchState::Tune{};
  float best = 1e30f;
  int best_geom = dbx::kGeomSampled;
  double best_rowq = dbx::hist_rowq_default();
  if (multi) {
    struct Shape {
      int geom;
      double rowq;
    };
    const double rq = dbx::hist_rowq_default();
    const Shape cand[3] = {{dbx::kGeomSampled, rq},
                           {dbx::kGeomSampled, 0.0},
                           {dbx::kGeomDisjoint, rq}};
    for (const Shape &sh : cand) {
      plan.geom = sh.geom;
      plan.rowq = sh.rowq;
      DBX_TRY(batch_plan(c, ms, rstep, nbins, base_tasks));
      float t0 = 0, t1 = 0;  // a warm launch, then the timed one
      DBX_TRY(time_batch_hist(c, e0, e1, &t0));
      DBX_TRY(time_batch_hist(c, e0, e1, &t1));
      ++b.tune.shapes;
      if (t1 < best) {
        best = t1;
        best_geom = sh.geom;
        best_rowq = sh.rowq;
      }
    }
    plan.geom = best_geom;
    plan.rowq = best_rowq;
    DBX_TRY(batch_plan(c, ms, rstep, nbins, base_tasks));
  } else {
    dbx::hist_plan_tasks(&plan, base_tasks);
  }
  best = 1e30f;
  int best_t = base_tasks;
  for (int t : {4, 8, 16}) {
    const int tasks = t * c->num_sms;
    dbx::hist_plan_tasks(&plan, tasks);
    size_t delta = 0;
    Error e = dbx::hist_upload(plan, &b.hp.lists, c->stream, &delta);
    c->used += delta;
    if (e.code) return e;
    float ms_t = 0;
    DBX_TRY(time_batch_hist(c, e0, e1, &ms_t));
    ++b.tune.task_counts;
    if (ms_t < best) {
      best = ms_t;
      best_t = tasks;
    }
  }
  b.tuned_tasks = best_t;
  b.tune.tasks = best_t;
  b.tune.geom = best_geom;
  b.tune.rowq = best_rowq;
  b.tune.multi = multi;
  b.tune.ms = best;
  dbx::hist_plan_tasks(&plan, best_t);
  size_t delta = 0;
  Error e = dbx::hist_upload(plan, &b.hp.lists, c->stream, &delta);
  c->used += delta;
  // later plans start from the default shape again
  plan.geom = dbx::kGeomSampled;
  plan.rowq = dbx::hist_rowq_default();
  return e;
}

Error patterns_tc(dbx_ctx *c, const std::vector<dbx::Model *> &ms,
                  const int64_t *ids, double rstep, const int64_t *nbins,
                  const dbx_species *sp, const double *K, int nq, double *out_I) {
  BatchState &b = c->batch;
  c->arena.reset();  // the previous call ended synchronised
  const int nm = (int)ms.size();
  for (int i = 0; i < nm; ++i) DBX_TRY(alloc_hist(c, ms[i], nbins[i]));
  std::vector<const void *> hist_ptrs(nm);
  for (int i = 0; i < nm; ++i) hist_ptrs[i] = ms[i]->d_hist;
  // (the contraction state is shared with single-pattern calls: a batch
  // is replayed only if no other call prepared a contraction since)
  const bool same = b.valid && b.tc_gen == c->tc.prep_gen && b.rstep == rstep &&
                    b.K.size() == (size_t)nq &&
                    b.ids == std::vector<int64_t>(ids, ids + nm) &&
                    b.nbins == std::vector<int64_t>(nbins, nbins + nm) &&
                    b.hist_ptrs == hist_ptrs &&
                    std::memcmp(b.K.data(), K, sizeof(double) * nq) == 0;
  size_t delta = 0;
  int nsp = 0;
  for (dbx::Model *m : ms) nsp += m->nspecies;
  if (!same) {
    b.valid = false;
    drop_graph(&b);
    b.ids.assign(ids, ids + nm);
    b.nbins.assign(nbins, nbins + nm);
    b.hist_ptrs = hist_ptrs;
    b.rstep = rstep;
    b.K.assign(K, K + nq);
    // one plan over every (model, pair), default shape; the autotuner
    // below may re-plan it with another
    b.hp.plan.geom = dbx::kGeomSampled;
    b.hp.plan.rowq = dbx::hist_rowq_default();
    DBX_TRY(batch_plan(c, ms, rstep, nbins, c->hist_tasks));
    // columns (model, pair) for the prefactor and the contraction
    b.model_col_begin.assign(1, 0);
    b.col_sp.clear();
    std::vector<dbx::TcCol> cols;
    int sp0 = 0;
    for (int i = 0; i < nm; ++i) {
      dbx::Model *m = ms[i];
      const int P = m->nspecies;
      int p = 0;
      for (int r = 0; r < P; ++r)
        for (int q = r; q < P; ++q, ++p) {
          dbx::TcCol col{};
          col.hist = m->d_hist + (size_t)p * m->hist_pitch;
          col.nbins = nbins[i];
          cols.push_back(col);
          b.col_sp.push_back(make_int2(sp0 + r, sp0 + q));
        }
      sp0 += P;
      b.model_col_begin.push_back((int)cols.size());
    }
    const int ncols = (int)cols.size();
    DBX_TRY(grow(c, &b.K_dev, sizeof(double) * nq));
    DBX_TRY(grow(c, &b.ff, sizeof(double) * nq * (size_t)ncols));
    DBX_TRY(grow(c, &b.I, sizeof(double) * nq * (size_t)nm));
    for (int i = 0; i < ncols; ++i) cols[i].ff = (const double *)b.ff.p + (size_t)i * nq;
    DBX_CUDA_TRY(cudaMemcpyAsync(b.K_dev.p, K, sizeof(double) * nq,
                                 cudaMemcpyHostToDevice, c->stream));
    c->h2d += sizeof(double) * nq;
    Error e = dbx::tc_prepare(&c->tc, cols, b.model_col_begin, rstep, K,
                              (const double *)b.K_dev.p, nq, c->stream, &delta);
    c->used += delta;
    delta = 0;
    if (e.code) return e;
    b.tc_gen = c->tc.prep_gen;
    e = dbx::hist_scratch(b.hp.plan, &c->hws, &delta);
    c->used += delta;
    delta = 0;
    if (e.code) return e;
    DBX_TRY(autotune(c, ms, rstep, nbins));
    DBX_TRY(dbx::hist_scratch(b.hp.plan, &c->hws, &delta));
    c->used += delta;
    delta = 0;
    c->h2d += b.hp.plan.upload_bytes();
    b.nsp = nsp;
    b.valid = true;
  }
  // species may change between passes (re-scoring): upload every pass
  Error e = dbx::prefactor_upload(&b.pref, sp, nsp, b.col_sp.data(),
                                  (int)b.col_sp.size(), (int)b.K.size(),
                                  c->stream, &delta);
  c->used += delta;
  c->h2d += sizeof(dbx_species) * nsp + sizeof(int2) * b.col_sp.size();
  if (e.code) return e;
  const std::vector<const void *> ptrs = {
      b.hp.lists.items.p, b.hp.lists.segs.p, b.hp.lists.tasks.p, b.hp.lists.rows.p,
      c->hws.partial.p,   c->hws.oor.p,      b.pref.sp.p,        b.pref.colsp.p,
      b.ff.p,             b.I.p,             b.K_dev.p,          c->tc.W.p,
      c->tc.E.p,          c->tc.P.p,         c->tc.tiles.p,      c->tc.cols.p,
      c->tc.basis.p,      c->tc.twid.p,      c->tc.nonself.p,    c->tc.err.p,
      b.pref.f.p,         b.pref.fid.p};
  if (c->graphs) {
    if (!b.exec || b.graph_ptrs != ptrs) {
      drop_graph(&b);
      dbx::Timers off;
      DBX_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      Error ce = batch_device_pass(c, &off);
      cudaGraph_t g = nullptr;
      cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
      if (ce.code) {
        if (g) cudaGraphDestroy(g);
        return ce;
      }
      if (ee != cudaSuccess) return dbx::fail(DBX_ERR_CUDA, cudaGetErrorString(ee));
      b.graph = g;
      DBX_CUDA_TRY(cudaGraphInstantiate(&b.exec, g, 0));
      b.graph_ptrs = ptrs;
    }
    c->tm.start(DBX_T_PASS, c->stream);
    DBX_CUDA_TRY(cudaGraphLaunch(b.exec, c->stream));
    c->tm.stop(DBX_T_PASS, c->stream);
  } else {
    DBX_TRY(batch_device_pass(c, &c->tm));
  }
  DBX_TRY(dbx::tc_check(&c->tc, c->stream));
  c->d2h += sizeof(int);
  Error re = dbx::hist_range_check(c->hws, c->stream);
  c->d2h += sizeof(unsigned long long);
  for (int i = 0; i < nm; ++i) {  // histograms stay resident for re-scoring
    ms[i]->hist_rstep = re.code ? 0 : rstep;
    ms[i]->hist_nbins = re.code ? 0 : nbins[i];
  }
  if (re.code) return re;
  DBX_CUDA_TRY(cudaMemcpyAsync(out_I, b.I.p, sizeof(double) * nq * nm,
                               cudaMemcpyDeviceToHost, c->stream));
  c->d2h += sizeof(double) * nq * nm;
  DBX_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return dbx::ok();
}

// The plain unbatched FP32 GPU form for one model: per pair a one-thread-
// per-pair global-atomic histogram, then the FP32 direct sum.
Error pattern_plain(dbx_ctx *c, dbx::Model *m, double rstep, int64_t nbins,
                    const dbx_species *sp, const double *K, int nq,
                    double *out_I) {
  DBX_TRY(alloc_hist(c, m, nbins));
  const float inv = (float)(1.0 / rstep);
  const int P = m->nspecies;
  int p = 0;
  for (int r = 0; r < P; ++r)
    for (int q = r; q < P; ++q, ++p) {
      size_t delta = 0;
      Error e = dbx::hist_plain(*m, r, q, inv, nbins,
                                m->d_hist + (size_t)p * m->hist_pitch, &c->hws,
                                c->stream, &delta);
      c->used += delta;
      if (e.code) return e;
      e = dbx::hist_range_check(c->hws, c->stream);  // per pair, as the reference syncs
      if (e.code) {
        m->hist_nbins = 0;
        return e;
      }
    }
  m->hist_rstep = rstep;
  m->hist_nbins = nbins;
  return intensity(c, m, rstep, nbins, sp, K, nq, DBX_DEBYE_FP32, out_I);
}

}  // namespace

extern "C" {

const char *dbx_strerror(int code) {
  switch (code) {
    case DBX_OK: return "ok";
    case DBX_ERR_ARG: return "invalid argument";
    case DBX_ERR_CUDA: return "CUDA error";
    case DBX_ERR_NOMEM: return "out of memory or HBM budget";
    case DBX_ERR_FILE: return "input file does not exist";
    case DBX_ERR_PARSE: return "malformed .deb file";
    case DBX_ERR_COUNT: return "atom count does not match the header";
    case DBX_ERR_RANGE: return "distance beyond rmax";
    case DBX_ERR_MODEL: return "unknown model id";
    case DBX_ERR_TIMEOUT: return "device wait timed out";
    case DBX_ERR_IO: return "output file could not be written";
    case DBX_ERR_LIMIT:
      return "request exceeds the fixed scratch of the no-allocation entry point";
    default: return "unknown error";
  }
}

const char *dbx_last_error(const dbx_ctx *c) {
  return c ? c->last_error.c_str() : "no context";
}

size_t dbx_device_bytes(const dbx_ctx *c) { return c ? c->used : 0; }

int dbx_create(dbx_ctx **out, int device, size_t budget) {
  if (!out) return DBX_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
    return DBX_ERR_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return DBX_ERR_CUDA;
  auto c = std::make_unique<dbx_ctx>();
  c->device = device;
  c->budget = budget;
  if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount,
                             device) != cudaSuccess)
    return DBX_ERR_CUDA;
  // Histogram tasks: a batch plan starts its autotuning from 4 per SM, a
  // single model's plan takes model_tasks(). DBX_HIST_TASKS fixes both
  // (tuning; fewer tasks also means more counts per task).
  c->hist_tasks = 4 * c->num_sms;
  if (const char *v = getenv("DBX_HIST_TASKS")) {
    const int t = atoi(v);
    if (t > 0) c->hist_tasks = c->hist_tasks_env = t;
  }
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) !=
          cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking) !=
          cudaSuccess ||
      cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming) != cudaSuccess)
    return DBX_ERR_CUDA;
  c->stream = c->own_stream;
  c->hws.arena = c->tc.arena = c->batch.pref.arena = c->batch.hp.lists.arena = &c->arena;
  *out = c.release();
  return DBX_OK;
}

int dbx_destroy(dbx_ctx *c) {
  if (!c) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto &kv : c->models) free_model(c, kv.second.get());
  c->models.clear();
  release(c, &c->hws.items);
  release(c, &c->hws.segs);
  release(c, &c->hws.tasks);
  release(c, &c->hws.rows);
  release(c, &c->hws.partial);
  release(c, &c->hws.oor);
  if (c->batch.exec) cudaGraphExecDestroy(c->batch.exec);
  if (c->batch.graph) cudaGraphDestroy(c->batch.graph);
  for (dbx::DevBuf *b : {&c->batch.hp.lists.items, &c->batch.hp.lists.segs,
                         &c->batch.hp.lists.tasks, &c->batch.hp.lists.rows,
                         &c->batch.pref.sp, &c->batch.pref.colsp,
                         &c->batch.pref.f, &c->batch.pref.fid, &c->batch.ff,
                         &c->batch.I, &c->batch.K_dev})
    release(c, b);
  dbx::tc_release(&c->tc);
  release(c, &c->tmp_hist);
  release(c, &c->K);
  release(c, &c->ff);
  release(c, &c->I);
  if (c->tm.created)
    for (auto &p : c->tm.ev) {
      cudaEventDestroy(p[0]);
      cudaEventDestroy(p[1]);
    }
  if (c->pin_ev) cudaEventDestroy(c->pin_ev);
  if (c->pin) cudaFreeHost(c->pin);
  if (c->side_stream) {
    cudaStreamSynchronize(c->side_stream);
    cudaStreamDestroy(c->side_stream);
  }
  if (c->join_ev) cudaEventDestroy(c->join_ev);
  cudaStreamDestroy(c->own_stream);
  delete c;
  return DBX_OK;
}

namespace {

// dbx_model_upload (x, y, z planes) and dbx_model_upload_xyz (xyz
// interleaved [natoms][3]): exactly one of the two forms is given.
int model_upload(dbx_ctx *c, const float *x, const float *y, const float *z,
                 const float *xyz, const int64_t *counts, int nspecies,
                 int64_t *model_id) {
  if (!c || !counts || nspecies < 1 || !model_id) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  auto m = std::make_unique<dbx::Model>();
  int64_t natoms = 0;
  for (int s = 0; s < nspecies; ++s) natoms += std::max<int64_t>(counts[s], 0);
  // The sorted atoms are staged in pinned memory owned by the context, so
  // the upload is an asynchronous copy; the staging buffer is reused only
  // once the previous upload's copy has completed.
  const size_t n = (size_t)std::max<int64_t>(natoms, 1);
  if (c->pin_used) {
    const cudaError_t ce = cudaEventSynchronize(c->pin_ev);
    if (ce != cudaSuccess)
      return set_err(c, dbx::fail(DBX_ERR_CUDA, cudaGetErrorString(ce)));
    c->pin_used = false;
  }
  if (c->pin_cap < n) {
    if (c->pin) cudaFreeHost(c->pin);
    c->pin = nullptr;
    c->pin_cap = 0;
    if (cudaMallocHost((void **)&c->pin, n * sizeof(float4)) != cudaSuccess) {
      c->pin = nullptr;
      return set_err(c, dbx::fail(DBX_ERR_NOMEM, "pinned staging buffer"));
    }
    c->pin_cap = n;
  }
  if (!c->pin_ev &&
      cudaEventCreateWithFlags(&c->pin_ev, cudaEventDisableTiming) != cudaSuccess)
    return set_err(c, dbx::fail(DBX_ERR_CUDA, "cudaEventCreate failed"));
  // Large models are sorted on the device (same order as the host sort,
  // which would dominate their upload); DBX_DEVICE_SORT_MIN sets the size.
  static const int64_t dev_min = [] {
    const char *v = getenv("DBX_DEVICE_SORT_MIN");
    return v ? std::max<int64_t>(1, atoll(v)) : int64_t(32768);
  }();
  Error e;
  for (int s = 0; s < nspecies; ++s)
    if (counts[s] < 0) return set_err(c, dbx::fail(DBX_ERR_ARG, "negative species count"));
  if (natoms > 0 && !xyz && (!x || !y || !z))
    return set_err(c, dbx::fail(DBX_ERR_ARG, "null coordinate array"));
  if (natoms >= (int64_t(1) << 31))
    return set_err(c, dbx::fail(DBX_ERR_ARG, "more than 2^31 atoms"));
  const int64_t ntiles_est = natoms / dbx::kTile + nspecies;
  const size_t need = sizeof(float4) * n + (sizeof(int2) + sizeof(dbx::TileBox)) *
                                               (size_t)std::max<int64_t>(ntiles_est, 1);
  if (c->budget && c->used + need > c->budget)
    return set_err(c, dbx::fail(DBX_ERR_NOMEM, "HBM budget exceeded by model"));
  if (natoms >= dev_min) {
    e = dbx::model_upload_sorted(m.get(), x, y, z, xyz, counts, nspecies,
                                 (float *)c->pin, c->pin_cap * sizeof(float4), c->stream);
  } else {
    std::vector<float> planes;  // small models: de-interleaved on the host
    if (xyz) {
      planes.resize(3 * (size_t)natoms);
      for (int64_t i = 0; i < natoms; ++i)
        for (int d = 0; d < 3; ++d) planes[d * natoms + i] = xyz[3 * i + d];
      x = planes.data();
      y = x + natoms;
      z = y + natoms;
    }
    e = dbx::model_prepare(x, y, z, counts, nspecies, m.get(), c->pin);
    if (e.code) return set_err(c, e);
    e = dbx::model_to_device(m.get(), c->pin, c->stream);
  }
  if (e.code) {
    dbx::model_release(m.get());
    return set_err(c, e);
  }
  if (cudaEventRecord(c->pin_ev, c->stream) != cudaSuccess)
    return set_err(c, dbx::fail(DBX_ERR_CUDA, "cudaEventRecord failed"));
  c->pin_used = true;
  c->used += m->dev_bytes;
  // bytes copied: sorted atoms, tiles (host sort) or raw coordinates,
  // tiles and the species descriptors (device sort)
  c->h2d += natoms >= dev_min
                ? (int64_t)(12 * natoms + sizeof(int2) * m->tiles.size() +
                            (6 * sizeof(unsigned) + sizeof(long long) + sizeof(int)) *
                                nspecies + sizeof(long long))
                : (int64_t)m->dev_bytes;
  m->id = c->next_id++;
  *model_id = m->id;
  c->models[m->id] = std::move(m);
  return DBX_OK;
}

}  // namespace

int dbx_model_upload(dbx_ctx *c, const float *x, const float *y,
                     const float *z, const int64_t *counts, int nspecies,
                     int64_t *model_id) {
  return model_upload(c, x, y, z, nullptr, counts, nspecies, model_id);
}

int dbx_model_upload_xyz(dbx_ctx *c, const float *xyz, const int64_t *counts,
                         int nspecies, int64_t *model_id) {
  int64_t natoms = 0;
  for (int s = 0; counts && s < nspecies; ++s) natoms += std::max<int64_t>(counts[s], 0);
  if (natoms > 0 && !xyz) return DBX_ERR_ARG;
  return model_upload(c, nullptr, nullptr, nullptr, xyz, counts, nspecies, model_id);
}

int dbx_model_free(dbx_ctx *c, int64_t id) {
  if (!c) return DBX_ERR_ARG;
  auto it = c->models.find(id);
  if (it == c->models.end()) return DBX_ERR_MODEL;
  cudaSetDevice(c->device);
  free_model(c, it->second.get());
  c->models.erase(it);
  return DBX_OK;
}

int64_t dbx_channels(double rmax, double rstep) {
  return (int64_t)(int)(rmax / rstep) + 2;  // cuDebye-v15.cu:732
}

int64_t dbx_curve_index(uint32_t x, uint32_t y, uint32_t z, int bits) {
  if (bits < 1 || bits > 10 || ((x | y | z) >> bits) != 0) return -1;
  return (int64_t)dbx::hilbert3(x, y, z, bits);
}

int dbx_pair_histogram(dbx_ctx *c, int64_t id, int row, int col, double rstep,
                       int64_t nbins, int64_t *out) {
  if (!c || !out || !(rstep > 0)) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  dbx::Model *m = find_model(c, id);
  if (!m) return set_err(c, dbx::fail(DBX_ERR_MODEL, "unknown model id"));
  if (row < 0 || col < row || col >= m->nspecies)
    return set_err(c, dbx::fail(DBX_ERR_ARG, "need 0 <= row <= col < nspecies"));
  const int64_t pitch = pitch_of(nbins);
  c->arena.reset();  // the previous call ended synchronised
  Error e = grow(c, &c->tmp_hist, sizeof(unsigned long long) * pitch);
  if (e.code) return set_err(c, e);
  dbx::HistPlan plan;
  if (nbins > dbx::hist_window_bins()) {
    e = dbx::model_host_boxes(m, c->stream);
    if (e.code) return set_err(c, e);
  }
  e = dbx::hist_plan(*m, {make_int2(row, col)}, rstep, nbins,
                     (unsigned long long *)c->tmp_hist.p, pitch,
                     model_tasks(c, nbins), &plan);
  if (e.code) return set_err(c, e);
  size_t delta = 0;
  c->tm.reset();
  e = dbx::hist_run(plan, (float)(1.0 / rstep), &c->hws, c->stream, c->num_sms,
                    &delta, &c->tm);
  c->used += delta;
  c->h2d += plan.upload_bytes();
  c->d2h += sizeof(unsigned long long);
  if (e.code) return set_err(c, e);
  return set_err(c, copy_rows(c, (const unsigned long long *)c->tmp_hist.p,
                              pitch, nbins, 1, out));
}

int dbx_pair_histogram_plain(dbx_ctx *c, int64_t id, int row, int col,
                             double rstep, int64_t nbins, int64_t *out) {
  if (!c || !out || !(rstep > 0) || nbins < 1) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  dbx::Model *m = find_model(c, id);
  if (!m) return set_err(c, dbx::fail(DBX_ERR_MODEL, "unknown model id"));
  if (row < 0 || col < row || col >= m->nspecies)
    return set_err(c, dbx::fail(DBX_ERR_ARG, "need 0 <= row <= col < nspecies"));
  c->arena.reset();  // the previous call ended synchronised
  Error e = grow(c, &c->tmp_hist, sizeof(unsigned long long) * (size_t)nbins);
  if (e.code) return set_err(c, e);
  size_t delta = 0;
  e = dbx::hist_plain(*m, row, col, (float)(1.0 / rstep), nbins,
                      (unsigned long long *)c->tmp_hist.p, &c->hws, c->stream,
                      &delta);
  c->used += delta;
  if (e.code) return set_err(c, e);
  c->d2h += sizeof(unsigned long long);
  // the counts below nbins are copied out before the range check reports
  const Error ce = copy_rows(c, (const unsigned long long *)c->tmp_hist.p,
                             nbins, nbins, 1, out);
  if (ce.code) return set_err(c, ce);
  return set_err(c, dbx::hist_range_check(c->hws, c->stream));
}

int dbx_histogram(dbx_ctx *c, int64_t id, double rstep, int64_t nbins,
                  int64_t *out) {
  if (!c || !out || !(rstep > 0)) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  dbx::Model *m = find_model(c, id);
  if (!m) return set_err(c, dbx::fail(DBX_ERR_MODEL, "unknown model id"));
  c->tm.reset();
  c->arena.reset();  // the previous call ended synchronised
  Error e = ensure_hist(c, m, rstep, nbins);
  if (e.code) return set_err(c, e);
  return set_err(c, copy_rows(c, m->d_hist, m->hist_pitch, nbins,
                              dbx::npairs_of(m->nspecies), out));
}

int dbx_check_sqrt(dbx_ctx *c, uint32_t lo_bits, uint32_t hi_bits,
                   int64_t out[3]) {
  if (!c || !out) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  return set_err(c, dbx::check_sqrt(lo_bits, hi_bits, c->num_sms, c->stream, out));
}

int dbx_reduce_check(const int64_t *counts, int64_t nbins, double rstep,
                     int64_t n_row, int64_t n_col, int diag, int64_t out[4]) {
  if (!counts || !out || nbins < 1) return DBX_ERR_ARG;
  // cuDebye-v15.cu:369-409
  int64_t expected = diag ? (n_col * n_row - n_row) / 2 + n_col : n_col * n_row;
  int64_t observed = 0, below = 0;
  for (int64_t k = 0; k < nbins; ++k) {
    observed += counts[k];
    if ((double)k * rstep < 0.25) below += counts[k];
  }
  out[0] = expected;
  out[1] = observed;
  out[2] = counts[0];
  out[3] = diag ? std::max<int64_t>(0, below - n_col) : below;
  return DBX_OK;
}

int dbx_k_grid(double lambda, double tt_min, double tt_max, double tt_step,
               double *two_theta, double *K) {
  if (!(tt_step > 0) || !(lambda > 0)) return DBX_ERR_ARG;
  const int n = (int)((tt_max - tt_min) / tt_step) + 1;  // cuDebye-v15.cu:690
  if (n < 1) return DBX_ERR_ARG;
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    const double tt = tt_min + (double)i * tt_step;
    if (two_theta) two_theta[i] = tt;
    if (K) K[i] = 4 * pi * sin(tt / 2 * pi / 180) / lambda;  // :697
  }
  return n;
}

int dbx_atomic_prop(dbx_ctx *c, const dbx_species *a, const dbx_species *b,
                    const double *K, int nq, double *out_ff) {
  if (!c || !a || !b || !K || !out_ff || nq < 1) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  dbx_species sp[2] = {*a, *b};
  // pair (0,1) of a 2-species list is index 1
  Error e = grow(c, &c->K, sizeof(double) * nq);
  if (!e.code) e = grow(c, &c->ff, sizeof(double) * nq * 3);
  if (e.code) return set_err(c, e);
  if (cudaMemcpyAsync(c->K.p, K, sizeof(double) * nq, cudaMemcpyHostToDevice,
                      c->stream) != cudaSuccess)
    return set_err(c, dbx::fail(DBX_ERR_CUDA, "copy K"));
  e = dbx::debye_prefactor(sp, 2, (const double *)c->K.p, nq,
                           (double *)c->ff.p, c->stream);
  if (e.code) return set_err(c, e);
  if (cudaMemcpyAsync(out_ff, (double *)c->ff.p + nq, sizeof(double) * nq,
                      cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return set_err(c, dbx::fail(DBX_ERR_CUDA, "copy ff"));
  return DBX_OK;
}

int dbx_intensity(dbx_ctx *c, int64_t id, double rstep, int64_t nbins,
                  const dbx_species *sp, const double *K, int nq, int mode,
                  double *out_I) {
  if (!c || !sp || !K || !out_I || !(rstep > 0)) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  dbx::Model *m = find_model(c, id);
  if (!m) return set_err(c, dbx::fail(DBX_ERR_MODEL, "unknown model id"));
  c->tm.reset();
  return set_err(c, intensity(c, m, rstep, nbins, sp, K, nq, mode, out_I));
}

int dbx_pattern(dbx_ctx *c, int64_t id, double rstep, int64_t nbins,
                const dbx_species *sp, const double *K, int nq, int mode,
                double *out_I) {
  if (!c || !sp || !K || !out_I || !(rstep > 0)) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  dbx::Model *m = find_model(c, id);
  if (!m) return set_err(c, dbx::fail(DBX_ERR_MODEL, "unknown model id"));
  c->tm.reset();
  m->hist_nbins = 0;  // recompute the histograms: one full pattern
  return set_err(c, intensity(c, m, rstep, nbins, sp, K, nq, mode, out_I));
}

int dbx_pattern_errors(dbx_ctx *c, const int64_t *ids, int nmodels, double rstep,
                       const int64_t *nbins, const dbx_species *sp, const double *K,
                       int nq, const double *I, int q_stride, double *out_maxrel) {
  if (!c || !ids || nmodels < 1 || !nbins || !sp || !K || nq < 1 || !I ||
      q_stride < 1 || !out_maxrel || !(rstep > 0))
    return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  std::vector<double> Ks, ref;
  for (int q = 0; q < nq; q += q_stride) Ks.push_back(K[q]);
  const int ns = (int)Ks.size();
  ref.resize(ns);
  int sp0 = 0;
  for (int i = 0; i < nmodels; ++i) {
    dbx::Model *m = find_model(c, ids[i]);
    if (!m) return set_err(c, dbx::fail(DBX_ERR_MODEL, "unknown model id"));
    c->tm.reset();
    Error e = intensity(c, m, rstep, nbins[i], sp + sp0, Ks.data(), ns,
                        DBX_DEBYE_FP64, ref.data());
    if (e.code) return set_err(c, e);
    double worst = 0.0;
    for (int j = 0; j < ns; ++j) {
      const double r = ref[j], v = I[(size_t)i * nq + (size_t)j * q_stride];
      if (r == 0.0 || !std::isfinite(r)) continue;
      worst = std::max(worst, std::fabs(v - r) / std::fabs(r));
    }
    out_maxrel[i] = worst;
    sp0 += m->nspecies;
  }
  return DBX_OK;
}

int dbx_batch_tuning(const dbx_ctx *c, double out[8]) {
  if (!c || !out) return DBX_ERR_ARG;
  const BatchState::Tune &t = c->batch.tune;
  out[0] = t.tasks;
  out[1] = c->num_sms ? (double)t.tasks / c->num_sms : 0.0;
  out[2] = t.multi ? 1.0 : 0.0;
  out[3] = t.rowq;
  out[4] = t.geom;
  out[5] = t.shapes;
  out[6] = t.task_counts;
  out[7] = t.ms;
  return c->batch.valid ? DBX_OK : DBX_ERR_ARG;
}

int dbx_set_graphs(dbx_ctx *c, int enable) {
  if (!c) return DBX_ERR_ARG;
  c->graphs = enable != 0;
  return DBX_OK;
}

int dbx_patterns(dbx_ctx *c, const int64_t *ids, int nmodels, double rstep,
                 const int64_t *nbins, const dbx_species *sp, const double *K,
                 int nq, int mode, double *out_I) {
  if (!c || !ids || nmodels < 1 || !nbins || !sp || !K || nq < 1 || !out_I ||
      !(rstep > 0))
    return DBX_ERR_ARG;
  if (mode != DBX_DEBYE_TC && mode != DBX_DEBYE_FP64 && mode != DBX_DEBYE_FP32 &&
      mode != DBX_PLAIN)
    return set_err(c, dbx::fail(DBX_ERR_ARG, "unknown mode"));
  cudaSetDevice(c->device);
  std::vector<dbx::Model *> ms(nmodels);
  for (int i = 0; i < nmodels; ++i) {
    ms[i] = find_model(c, ids[i]);
    if (!ms[i]) return set_err(c, dbx::fail(DBX_ERR_MODEL, "unknown model id"));
    for (int j = 0; j < i; ++j)
      if (ids[j] == ids[i])
        return set_err(c, dbx::fail(DBX_ERR_ARG, "a model appears twice in a batch"));
  }
  c->tm.reset();
  if (mode == DBX_DEBYE_TC)
    return set_err(c, patterns_tc(c, ms, ids, rstep, nbins, sp, K, nq, out_I));
  int sp0 = 0;
  for (int i = 0; i < nmodels; ++i) {
    Error e;
    if (mode == DBX_PLAIN) {
      e = pattern_plain(c, ms[i], rstep, nbins[i], sp + sp0, K, nq,
                        out_I + (size_t)i * nq);
    } else {
      ms[i]->hist_nbins = 0;
      e = intensity(c, ms[i], rstep, nbins[i], sp + sp0, K, nq, mode,
                    out_I + (size_t)i * nq);
    }
    if (e.code) return set_err(c, e);
    sp0 += ms[i]->nspecies;
  }
  return DBX_OK;
}

int dbx_set_stream(dbx_ctx *c, void *stream) {
  if (!c) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return DBX_OK;
}

int dbx_set_timing(dbx_ctx *c, int enable) {
  if (!c) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  if (enable && !c->tm.created) {
    for (auto &p : c->tm.ev)
      if (cudaEventCreate(&p[0]) != cudaSuccess ||
          cudaEventCreate(&p[1]) != cudaSuccess)
        return DBX_ERR_CUDA;
    c->tm.created = true;
  }
  c->tm.on = enable != 0;
  c->tm.reset();
  return DBX_OK;
}

int dbx_get_traffic(const dbx_ctx *c, int64_t out[2]) {
  if (!c || !out) return DBX_ERR_ARG;
  out[0] = c->h2d;
  out[1] = c->d2h;
  return DBX_OK;
}

int dbx_get_timing(const dbx_ctx *c, double out_ms[DBX_NTIMERS]) {
  if (!c || !out_ms) return DBX_ERR_ARG;
  for (int i = 0; i < DBX_NTIMERS; ++i) {
    out_ms[i] = 0.0;
    if (c->tm.created && c->tm.recorded[i]) {
      float ms = 0.f;
      if (cudaEventSynchronize(c->tm.ev[i][1]) != cudaSuccess ||
          cudaEventElapsedTime(&ms, c->tm.ev[i][0], c->tm.ev[i][1]) !=
              cudaSuccess)
        return DBX_ERR_CUDA;
      out_ms[i] = ms;
    }
  }
  return DBX_OK;
}

int dbx_run_deb(dbx_ctx *c, const char *deb_path, const char *out_prefix,
                int verbose) {
  if (!c || !deb_path) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  dbx::DebFile d;
  std::string msg;
  int rc = dbx::deb_read(deb_path, &d, &msg);
  if (rc) {
    c->last_error = msg;
    if (verbose) printf("\nERROR: %s\n", msg.c_str());
    return rc;
  }
  const std::string prefix = out_prefix ? out_prefix : deb_path;
  const int P = (int)d.species.size();
  std::vector<int64_t> counts(P);
  std::vector<dbx_species> sp(P);
  for (int i = 0; i < P; ++i) {
    counts[i] = d.species[i].n;
    sp[i] = d.species[i].p;
  }
  int64_t id = 0;
  rc = dbx_model_upload(c, d.x.data(), d.y.data(), d.z.data(), counts.data(), P,
                        &id);
  if (rc) return rc;
  struct Drop {
    dbx_ctx *c;
    int64_t id;
    ~Drop() { dbx_model_free(c, id); }
  } drop{c, id};
  const int64_t nbins = dbx_channels(d.rmax, d.rstep);
  dbx::Model *m = find_model(c, id);
  c->arena.reset();  // the previous call ended synchronised
  Error e = ensure_hist(c, m, d.rstep, nbins);
  if (e.code) {
    if (verbose) printf("\nERROR: %s\n", e.msg.c_str());
    return set_err(c, e);
  }
  // All pair histograms to the host at once; the .debx files are then
  // written by one thread each while the Debye sum runs on the device.
  const int np = dbx::npairs_of(P);
  std::vector<int64_t> h;
  std::vector<std::future<int>> writers;
  if (d.hist > 0 || verbose) {
    h.resize((size_t)np * nbins);
    e = copy_rows(c, m->d_hist, m->hist_pitch, nbins, np, h.data());
    if (e.code) return set_err(c, e);
    for (int row = 0; row < P; ++row)
      for (int col = row; col < P; ++col) {
        const int64_t *hp = h.data() + (size_t)dbx::pair_index(P, row, col) * nbins;
        if (verbose) {
          int64_t chk[4];
          dbx_reduce_check(hp, nbins, d.rstep, counts[row], counts[col],
                           row == col, chk);
          printf("\n>>>> Subgroup %d and %d\n", row, col);
          if (chk[0] != chk[1])
            printf("WARNING: %lld Distances Expected and %lld Observed!!!\n",
                   (long long)chk[0], (long long)chk[1]);
          if (row == col && chk[2] != counts[row])
            printf("WARNING: Number of Expected Zero Distances Missing or not "
                   "Correct!!!\n");
          if (chk[3] > 0)
            printf("WARNING: Possible Atom Collision!!! Found around %lld "
                   "interatomic Distances lower than the Radius of an Hydrogen "
                   "Atom.\n",
                   (long long)chk[3]);
          printf("Distances Expected: %lld - Distances Observed: %lld\n",
                 (long long)chk[0], (long long)chk[1]);
        }
        if (d.hist > 0) {
          const std::string path =
              prefix + "x" + std::to_string(row) + "x" + std::to_string(col);
          const double rstep = d.rstep;
          writers.push_back(std::async(std::launch::async, [=]() {
            return dbx::write_debx(path, hp, nbins, rstep);
          }));
        }
      }
  }
  Error out = dbx::ok();
  if (d.hist != 1) {
    const int nq = dbx_k_grid(d.lambda, d.tt_min, d.tt_max, d.tt_step, nullptr,
                              nullptr);
    if (nq < 1) {
      out = dbx::fail(DBX_ERR_PARSE, "empty 2theta grid");
    } else {
      std::vector<double> tt(nq), K(nq), I(nq);
      dbx_k_grid(d.lambda, d.tt_min, d.tt_max, d.tt_step, tt.data(), K.data());
      out = intensity(c, m, d.rstep, nbins, sp.data(), K.data(), nq,
                      DBX_DEBYE_TC, I.data());
      const std::string path = prefix + "I";
      if (!out.code && dbx::write_debI(path, tt.data(), I.data(), nq))
        out = dbx::fail(DBX_ERR_IO, "cannot write " + path);
      if (!out.code && verbose) printf("\nWrote %s (%d points)\n", path.c_str(), nq);
    }
  }
  for (auto &w : writers)
    if (w.get() != DBX_OK && !out.code)
      out = dbx::fail(DBX_ERR_IO, "cannot write a .debx file next to " + prefix);
  return set_err(c, out);
}

// ---- directory driver ------------------------------------------------------
// The reference's Matlab batch driver (Matlab/multisim.m:9-65) without its
// plots: every .xyz of `dir` without a .deb is converted first (when a
// scattering-factor table is given), then every .deb without a .debI is
// computed. Models that share rstep and the 2theta grid are batched
// (dbx_patterns: one histogram launch and one contraction per chunk of up to
// kDirChunk models); the outputs of a chunk are written on a host thread
// while the next chunk runs. A chunk that fails is redone file by file, so
// one bad file does not stop the others; the first error is returned.

namespace {
constexpr int kDirChunk = 64;

bool ends_with(const std::string &s, const char *t) {
  const size_t n = strlen(t);
  return s.size() >= n && s.compare(s.size() - n, n, t) == 0;
}

struct DirItem {
  std::string name, path;
  dbx::DebFile d;
};

// Writes the outputs of one model of a chunk: .debx (hist 1/2) and .debI
// (hist 0/2), from host copies.
int write_item(const DirItem &it, const std::vector<int64_t> &h, int64_t nbins,
               const std::vector<double> &tt, const double *I) {
  const int P = (int)it.d.species.size();
  if (it.d.hist > 0)
    for (int row = 0; row < P; ++row)
      for (int col = row; col < P; ++col) {
        const std::string path =
            it.path + "x" + std::to_string(row) + "x" + std::to_string(col);
        const int64_t *hp = h.data() + (size_t)dbx::pair_index(P, row, col) * nbins;
        if (dbx::write_debx(path, hp, nbins, it.d.rstep)) return DBX_ERR_IO;
      }
  if (it.d.hist != 1 && dbx::write_debI(it.path + "I", tt.data(), I, (int)tt.size()))
    return DBX_ERR_IO;
  return DBX_OK;
}
}  // namespace

extern "C" int dbx_run_dir(dbx_ctx *c, const char *dir, const char *table_path,
                           int verbose) {
  if (!c || !dir) return DBX_ERR_ARG;
  cudaSetDevice(c->device);
  auto list = [&](std::vector<std::string> *names) {
    names->clear();
    DIR *dp = opendir(dir);
    if (!dp) return false;
    while (dirent *de = readdir(dp)) {
      const std::string n = de->d_name;
      struct stat st;
      if (stat((std::string(dir) + "/" + n).c_str(), &st) == 0 && S_ISREG(st.st_mode))
        names->push_back(n);
    }
    closedir(dp);
    std::sort(names->begin(), names->end());
    return true;
  };
  std::vector<std::string> files;
  if (!list(&files))
    return set_err(c, dbx::fail(DBX_ERR_FILE, std::string("cannot open ") + dir));
  int first = DBX_OK;
  std::string first_msg;
  auto note = [&](int rc, const std::string &m) {
    if (rc && !first) {
      first = rc;
      first_msg = m;
    }
    if (rc && verbose) printf("ERROR: %s\n", m.c_str());
  };
  std::vector<std::string> xyz;
  for (const std::string &f : files)
    if (ends_with(f, ".xyz") &&
        !std::binary_search(files.begin(), files.end(), f.substr(0, f.size() - 3) + "deb"))
      xyz.push_back(f);
  for (size_t i = 0; i < xyz.size(); ++i) {
    const std::string path = std::string(dir) + "/" + xyz[i];
    if (!table_path) {
      if (verbose) printf("Skip %s: no scattering-factor table given\n", xyz[i].c_str());
      continue;
    }
    if (verbose)
      printf("Convert File %zu of %zu -- %s\n", i + 1, xyz.size(), xyz[i].c_str());
    char m[512] = {0};
    const int rc = dbx_xyz2deb(path.c_str(), table_path, nullptr, nullptr, m, sizeof m);
    note(rc, m);
  }
  if (!list(&files))
    return set_err(c, dbx::fail(DBX_ERR_FILE, std::string("cannot open ") + dir));
  std::vector<DirItem> items;
  for (const std::string &f : files)
    if (ends_with(f, ".deb") && !std::binary_search(files.begin(), files.end(), f + "I")) {
      DirItem it;
      it.name = f;
      it.path = std::string(dir) + "/" + f;
      std::string m;
      const int rc = dbx::deb_read(it.path, &it.d, &m);
      if (rc) {
        note(rc, f + ": " + m);
        continue;
      }
      items.push_back(std::move(it));
    }
  // groups: same rstep and 2theta grid, in file order
  std::vector<std::vector<int>> groups;
  for (int i = 0; i < (int)items.size(); ++i) {
    const dbx::DebFile &d = items[i].d;
    bool placed = false;
    for (auto &g : groups) {
      const dbx::DebFile &e = items[g[0]].d;
      if (e.rstep == d.rstep && e.lambda == d.lambda && e.tt_min == d.tt_min &&
          e.tt_max == d.tt_max && e.tt_step == d.tt_step &&
          (int)g.size() < kDirChunk) {
        g.push_back(i);
        placed = true;
        break;
      }
    }
    if (!placed) groups.push_back({i});
  }
  int done = 0;
  std::future<int> pending;
  for (const std::vector<int> &g : groups) {
    const dbx::DebFile &d0 = items[g[0]].d;
    const int nq = dbx_k_grid(d0.lambda, d0.tt_min, d0.tt_max, d0.tt_step, nullptr,
                              nullptr);
    std::vector<double> tt(std::max(nq, 1)), K(std::max(nq, 1));
    if (nq >= 1) dbx_k_grid(d0.lambda, d0.tt_min, d0.tt_max, d0.tt_step, tt.data(), K.data());
    std::vector<int64_t> ids, nb;
    std::vector<dbx_species> sp;
    int rc = nq >= 1 ? DBX_OK : DBX_ERR_PARSE;
    for (int i : g) {
      if (rc) break;
      const dbx::DebFile &d = items[i].d;
      std::vector<int64_t> counts;
      for (const dbx::DebSpecies &s : d.species) {
        counts.push_back(s.n);
        sp.push_back(s.p);
      }
      int64_t id = 0;
      rc = dbx_model_upload(c, d.x.data(), d.y.data(), d.z.data(), counts.data(),
                            (int)counts.size(), &id);
      if (!rc) {
        ids.push_back(id);
        nb.push_back(dbx_channels(d.rmax, d.rstep));
      }
    }
    std::vector<double> I;
    if (!rc) {
      I.resize((size_t)nq * g.size());
      rc = dbx_patterns(c, ids.data(), (int)ids.size(), d0.rstep, nb.data(), sp.data(),
                        K.data(), nq, DBX_DEBYE_TC, I.data());
    }
    // histograms of the chunk to the host (the writers need them)
    std::vector<std::vector<int64_t>> hs(g.size());
    for (size_t k = 0; !rc && k < g.size(); ++k) {
      dbx::Model *m = find_model(c, ids[k]);
      const int np = dbx::npairs_of(m->nspecies);
      hs[k].resize((size_t)np * nb[k]);
      Error e = copy_rows(c, m->d_hist, m->hist_pitch, nb[k], np, hs[k].data());
      rc = e.code;
    }
    for (int64_t id : ids) dbx_model_free(c, id);
    if (pending.valid()) note(pending.get(), "cannot write an output file");
    if (rc) {
      // isolate the failing file(s)
      for (int i : g) {
        if (verbose)
          printf("Calculate File %d of %zu -- %s\n", ++done, items.size(),
                 items[i].name.c_str());
        const int r1 = dbx_run_deb(c, items[i].path.c_str(), nullptr, 0);
        note(r1, items[i].name + ": " + dbx_last_error(c));
      }
      continue;
    }
    if (verbose)
      for (int i : g)
        printf("Calculate File %d of %zu -- %s\n", ++done, items.size(),
               items[i].name.c_str());
    std::vector<int> gi = g;
    pending = std::async(std::launch::async,
                         [&items, gi, hs = std::move(hs), nb, tt, I = std::move(I), nq]() {
                           for (size_t k = 0; k < gi.size(); ++k) {
                             const int r = write_item(items[gi[k]], hs[k], nb[k], tt,
                                                      I.data() + k * (size_t)nq);
                             if (r) return r;
                           }
                           return (int)DBX_OK;
                         });
  }
  if (pending.valid()) note(pending.get(), "cannot write an output file");
  if (first) c->last_error = first_msg;
  return first;
}

}  // extern "C"
