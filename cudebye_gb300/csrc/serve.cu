// serve.cu — a pattern server on one GPU: continuous batching of Debye
// pattern requests with admission by HBM footprint.
//
// The reference computes one pattern per process run; its only batching is
// the Matlab loop that runs cuDebye.exe file after file and skips files
// already done (Matlab/multisim.m:19-65). Here requests arrive at any time
// from any host thread (dbx_server_submit) and a worker thread owns the
// device:
//  * Admission: a request is admitted when its device footprint (atoms,
//    histograms, row sums) fits the HBM budget next to the resident models
//    and the two lanes' workspaces; idle resident models are evicted least
//    recently used first. Requests that do not fit wait in the queue.
//  * Rounds: every admitted request of a round is served together: the
//    histograms of all new models in one tile-pair launch, then per request
//    the prefactor and either the tensor-core contraction (new model or new
//    q grid) or, for new species parameters on the same grid, a weighted
//    sum of the resident per-pair row sums.
//  * Continuous batching: rounds alternate between two lanes (stream +
//    workspaces). The worker launches round r+1 while round r is still on
//    the GPU, so requests that arrive meanwhile are admitted as soon as a
//    lane and memory free up and their work overlaps on the device.
//  * Residency: histograms and row sums stay on the device for re-scoring;
//    a request names a resident model by the id an earlier request returned.
// Results do not depend on the mix: histograms are exact integers and each
// request's contraction is its own, with a fixed reduction order.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "debye_tc.h"
#include "engine.h"

namespace dbx {
namespace {

double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

enum Kind { kNew = 0, kSameGrid = 1, kNewGrid = 2 };

struct Req {
  int64_t ticket = 0;
  int64_t model = 0;  // resident model (0: new)
  std::vector<float> x, y, z;
  std::vector<int64_t> counts;
  std::vector<dbx_species> sp;
  double rstep = 0;
  int64_t nbins = 0;
  std::vector<double> K;
  int kind = kNew;
  int status = 1;  // 1 pending, 0 done, < 0 DBX_ERR_*
  std::string msg;
  std::vector<double> I;
  int64_t model_out = 0;
  double t_submit = 0, t_done = 0;
  size_t offset = 0;  // of I in the lane's result buffer
  bool solo = false;  // retried alone after its round failed
  // host preparation of a new model, done by a preparation thread before
  // the request is queued: its sorted atoms, its host part (tiles, boxes,
  // species ranges) and its histogram plan without device pointers
  std::unique_ptr<Model> hm;
  std::vector<float4> atoms;
  HistPlan part;
};

struct SModel {  // a resident model of the server
  std::unique_ptr<Model> m;
  double rstep = 0;
  int64_t nbins = 0;
  std::vector<double> K;  // q grid of the resident row sums
  DevBuf S;               // [npairs][nq]
  bool ready = false;     // histograms and row sums computed
  bool busy = false;      // a request on it is in flight
  double last_use = 0;
  size_t bytes() const { return model_device_bytes(*m) + S.bytes; }
};

struct Lane {
  cudaStream_t stream = nullptr;
  // pinned staging of the round's host-to-device copies, so that queueing
  // a request's work behind the histogram launch never waits for it
  PinArena arena;
  HistWorkspace hws;  // work lists and scratch of the round's histograms
  HistPlan plan;
  TcState tc;
  PrefState pref;
  DevBuf K, ff, I;
  double *hI = nullptr;  // the round's results (pinned, in the arena)
  std::vector<Req *> reqs;
  bool busy = false;
};

void release(DevBuf *b) {
  if (b->p) cudaFree(b->p);
  b->p = nullptr;
  b->bytes = 0;
}

int64_t pitch_of(int64_t nbins) { return (nbins + 2 + 1) & ~int64_t(1); }

size_t hist_bytes(int nspecies, int64_t nbins) {
  return sizeof(unsigned long long) * (size_t)pitch_of(nbins) * npairs_of(nspecies);
}

// Device bytes a lane may need for one request (contraction, prefactor).
size_t lane_need(const Req &r, int nspecies) {
  const size_t nq = r.K.size(), Qp = (nq + 127) / 128 * 128;
  const size_t np = npairs_of(nspecies);
  const size_t nch = (size_t)(r.nbins + 255) / 256, tiles = np * ((nch + 63) / 64);
  return tiles * 128 * 1024 + tiles * 2 * Qp * 8 + (2 * Qp / 128) * 256 * 1024 +
         ((nch + 63) / 64 * 64) * Qp * 16 + np * nq * 8 * 2 + nq * 8 +
         (size_t)nspecies * nq * 8;
}

}  // namespace
}  // namespace dbx

struct dbx_server {
  int device = 0;
  size_t budget = 0;
  int num_sms = 0;
  int hist_tasks = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<dbx::Req *> queue;     // ready for admission
  std::deque<dbx::Req *> prep_q;    // new models waiting for host preparation
  std::condition_variable cv_prep;
  int prepping = 0;                 // preparations in progress
  std::vector<std::thread> preps;
  std::map<int64_t, std::unique_ptr<dbx::Req>> reqs;  // by ticket
  std::map<int64_t, dbx::SModel> models;              // worker thread only
  int64_t next_ticket = 1, next_model = 1;
  dbx::Lane lanes[2];
  int next_lane = 0;
  std::thread worker;
  bool stop = false;
  size_t used = 0;  // device bytes: models + lane workspaces (worker only)
  int64_t rounds = 0, completed = 0, evicted = 0;
  size_t lane_reserve = 0;  // device bytes kept free for the lanes
};

namespace dbx {
namespace {

void complete(dbx_server *s, Req *r, int status, const std::string &msg) {
  r->status = status;
  r->msg = msg;
  r->t_done = now_ms();
}

// Evict least recently used idle models not named by a queued request until
// `need` more bytes fit. Worker thread, lock held.
bool make_room(dbx_server *s, size_t need) {
  if (!s->budget) return true;
  if (s->used + need + s->lane_reserve <= s->budget) return true;
  std::set<int64_t> named;  // models a queued request refers to
  for (Req *q : s->queue)
    if (q->model) named.insert(q->model);
  while (s->used + need + s->lane_reserve > s->budget) {
    int64_t victim = 0;
    double oldest = 1e300;
    for (auto &kv : s->models) {
      const SModel &sm = kv.second;
      if (!sm.ready || sm.busy || named.count(kv.first)) continue;
      if (sm.last_use < oldest) {
        oldest = sm.last_use;
        victim = kv.first;
      }
    }
    if (!victim) return false;
    SModel &sm = s->models[victim];
    s->used -= sm.bytes();
    // idle: no round in flight uses it; freed in stream order, without the
    // device-wide wait of cudaFree
    model_release_async(sm.m.get(), s->lanes[0].stream);
    if (sm.S.p) cudaFreeAsync(sm.S.p, s->lanes[0].stream);
    sm.S.p = nullptr;
    sm.S.bytes = 0;
    s->models.erase(victim);
    ++s->evicted;
  }
  return true;
}

// Take the admissible requests off the queue, FIFO. Worker thread, lock held.
std::vector<Req *> admit(dbx_server *s) {
  std::vector<Req *> out;
  int64_t round_pairs = 0;
  size_t pending = 0;                       // bytes of requests admitted now
  double round_rstep = 0;                   // new models of a round share it
  // binned pairs of new models per round: bounds a round's device time,
  // and so how long requests behind it wait (DBX_SERVE_ROUND_PAIRS)
  static const int64_t kMaxPairs = [] {
    const char *v = getenv("DBX_SERVE_ROUND_PAIRS");
    const long long p = v ? atoll(v) : 0;
    return p > 0 ? (int64_t)p : int64_t(40000000000LL);
  }();
  for (auto it = s->queue.begin(); it != s->queue.end() && out.size() < 64;) {
    Req *r = *it;
    if (r->solo && !out.empty()) break;  // a retried request runs alone
    size_t need = 0;
    int nspecies = (int)r->counts.size();
    if (r->model) {
      auto mit = s->models.find(r->model);
      if (mit == s->models.end()) {
        complete(s, r, DBX_ERR_MODEL, "unknown or evicted model");
        it = s->queue.erase(it);
        s->cv_done.notify_all();
        continue;
      }
      SModel &sm = mit->second;
      if (!sm.ready || sm.busy) {  // wait for its first pass / other request
        ++it;
        continue;
      }
      nspecies = sm.m->nspecies;
      if ((int)r->sp.size() != nspecies || r->rstep != sm.rstep ||
          r->nbins != sm.nbins) {
        complete(s, r, DBX_ERR_ARG,
                 "re-scoring must repeat the model's species count and binning");
        it = s->queue.erase(it);
        s->cv_done.notify_all();
        continue;
      }
      const bool same = sm.K == r->K;
      r->kind = same ? kSameGrid : kNewGrid;
      if (!same) need = npairs_of(nspecies) * r->K.size() * 8;
    } else {
      int64_t natoms = 0;
      for (int64_t c : r->counts) natoms += c;
      need = (size_t)natoms * 16 + ((size_t)natoms / 128 + nspecies + 1) * 8 +
             hist_bytes(nspecies, r->nbins) + npairs_of(nspecies) * r->K.size() * 8;
      int64_t pairs = 0;
      for (int a = 0; a < nspecies; ++a)
        for (int b = a; b < nspecies; ++b)
          pairs += a == b ? r->counts[a] * (r->counts[a] + 1) / 2
                          : r->counts[a] * r->counts[b];
      if (!out.empty() && round_pairs + pairs > kMaxPairs) break;
      if (round_rstep != 0 && r->rstep != round_rstep) {  // next round
        ++it;
        continue;
      }
      round_pairs += pairs;
      round_rstep = r->rstep;
      r->kind = kNew;
    }
    s->lane_reserve = std::max(s->lane_reserve, lane_need(*r, nspecies) + (160u << 20));
    if (!make_room(s, pending + need)) break;  // head of line waits for memory
    pending += need;
    if (r->model) s->models[r->model].busy = true;
    out.push_back(r);
    it = s->queue.erase(it);
    if (r->solo) break;
  }
  return out;
}

// Launch one round on a lane (asynchronous). Worker thread, no lock.
Error launch_round(dbx_server *s, Lane &L, const std::vector<Req *> &batch) {
  L.reqs = batch;
  L.busy = true;
  const cudaStream_t st = L.stream;
  size_t used_delta = 0;
  L.arena.reset();  // the lane is idle: its previous round's copies are done
  // 1. new models: sort + upload, histogram buffers
  std::vector<int64_t> new_ids;
  for (Req *r : batch) {
    if (r->kind != kNew) continue;
    // host part prepared by a preparation thread; atoms through the pinned
    // staging (pageable as a fallback)
    auto m = std::make_unique<Model>(*r->hm);
    const size_t abytes = sizeof(float4) * r->atoms.size();
    const float4 *atoms = r->atoms.data();
    if (void *p = L.arena.take(abytes)) {
      std::memcpy(p, atoms, abytes);
      atoms = (const float4 *)p;
    }
    DBX_TRY(model_to_device(m.get(), atoms, st, &L.arena));
    m->hist_pitch = pitch_of(r->nbins);
    m->hist_bytes = hist_bytes(m->nspecies, r->nbins);
    DBX_CUDA_TRY(cudaMallocAsync(&m->d_hist, m->hist_bytes, st));
    const int64_t id = s->next_model++;
    m->id = id;
    SModel sm;
    sm.m = std::move(m);
    sm.rstep = r->rstep;
    sm.nbins = r->nbins;
    sm.busy = true;
    s->used += sm.m->dev_bytes + sm.m->hist_bytes;
    r->model_out = id;
    s->models[id] = std::move(sm);
    new_ids.push_back(id);
  }
  // 2. histograms of all new models (one rstep per round): one plan, one
  //    launch
  Timers off;
  hist_plan_clear(&L.plan);
  double rstep = 0;
  for (Req *r : batch) {
    if (r->kind != kNew) continue;
    SModel &sm = s->models[r->model_out];
    hist_plan_append(&L.plan, r->part, sm.m->d_atoms, sm.m->d_tiles, sm.m->d_boxes,
                     sm.m->d_hist);
    rstep = sm.rstep;
  }
  hist_plan_tasks(&L.plan, s->hist_tasks);
  DBX_TRY(hist_upload(L.plan, &L.hws, st, &used_delta));
  if (!new_ids.empty()) {
    DBX_TRY(hist_launch(L.plan, L.hws, &L.hws, (float)(1.0 / rstep), st,
                        s->num_sms, &used_delta, &off));
  } else {
    DBX_TRY(hist_scratch(L.plan, &L.hws, &used_delta));
    DBX_CUDA_TRY(cudaMemsetAsync(L.hws.oor.p, 0, 16, st));
  }
  // 3. per request: prefactor, then contraction or weighted sum
  size_t total = 0;
  for (Req *r : batch) {
    r->offset = total;
    total += r->K.size();
  }
  DBX_TRY(buf_grow(&L.I, std::max<size_t>(total, 1) * 8, &s->used, st));
  L.hI = (double *)L.arena.take(std::max<size_t>(total, 1) * 8);
  if (!L.hI) return fail(DBX_ERR_NOMEM, "pinned host memory for results");
  for (Req *r : batch) {
    const int64_t id = r->model ? r->model : r->model_out;
    SModel &sm = s->models[id];
    const int P = sm.m->nspecies, np = npairs_of(P), nq = (int)r->K.size();
    DBX_TRY(buf_grow(&L.K, (size_t)nq * 8, &s->used, st));
    DBX_TRY(buf_grow(&L.ff, (size_t)np * nq * 8, &s->used, st));
    DBX_TRY(h2d_copy(L.K.p, r->K.data(), (size_t)nq * 8, st, &L.arena));
    std::vector<int2> col_sp;
    for (int a = 0; a < P; ++a)
      for (int b = a; b < P; ++b) col_sp.push_back(make_int2(a, b));
    DBX_TRY(prefactor_upload(&L.pref, r->sp.data(), P, col_sp.data(), np, nq,
                             st, &used_delta));
    DBX_TRY(prefactor_execute(L.pref, (const double *)L.K.p, nq, (double *)L.ff.p, st));
    double *dI = (double *)L.I.p + r->offset;
    if (r->kind == kSameGrid) {
      DBX_TRY(tc_combine((const double *)L.ff.p, (const double *)sm.S.p, np, nq, dI, st));
    } else {
      if (sm.S.bytes < (size_t)np * nq * 8) {
        s->used -= sm.S.bytes;
        release(&sm.S);
        DBX_CUDA_TRY(cudaMallocAsync(&sm.S.p, (size_t)np * nq * 8, st));
        sm.S.bytes = (size_t)np * nq * 8;
        s->used += sm.S.bytes;
      }
      sm.K = r->K;
      std::vector<TcCol> cols(np);
      for (int p = 0; p < np; ++p) {
        cols[p] = TcCol{};
        cols[p].hist = sm.m->d_hist + (size_t)p * sm.m->hist_pitch;
        cols[p].nbins = sm.nbins;
        cols[p].ff = (const double *)L.ff.p + (size_t)p * nq;
      }
      DBX_TRY(tc_prepare(&L.tc, cols, {0, np}, sm.rstep, r->K.data(),
                         (const double *)L.K.p, nq, st, &used_delta));
      L.tc.S_out = (double *)sm.S.p;
      DBX_TRY(tc_execute(&L.tc, (const double *)L.K.p, dI, st, &off));
      L.tc.S_out = nullptr;
    }
  }
  s->used += used_delta;
  // 4. results back (asynchronous)
  DBX_CUDA_TRY(cudaMemcpyAsync(L.hI, L.I.p, total * 8, cudaMemcpyDeviceToHost, st));
  return ok();
}

// Wait for a lane's round, publish its results. Worker thread.
void finish_round(dbx_server *s, Lane &L, const Error &launch_err) {
  Error e = launch_err;
  if (!e.code) {
    cudaError_t ce = cudaStreamSynchronize(L.stream);
    if (ce != cudaSuccess) e = fail(DBX_ERR_CUDA, cudaGetErrorString(ce));
  }
  if (!e.code && L.hws.oor.p) e = hist_range_check(L.hws, L.stream);
  if (!e.code && L.tc.err.p) e = tc_check(&L.tc, L.stream);
  std::lock_guard<std::mutex> lock(s->mu);
  // A failed round of several requests (one model with a distance beyond
  // its rmax fails the shared histogram launch) is retried request by
  // request, so that only the faulty one reports the error and the others'
  // results do not depend on what they were batched with. A CUDA error is
  // final for all.
  const bool retry = e.code && e.code != DBX_ERR_CUDA && L.reqs.size() > 1;
  for (auto it = L.reqs.rbegin(); retry && it != L.reqs.rend(); ++it) {
    Req *r = *it;
    const int64_t id = r->model ? r->model : r->model_out;
    auto mit = s->models.find(id);
    if (mit != s->models.end()) {
      SModel &sm = mit->second;
      sm.busy = false;
      if (r->kind == kNewGrid) sm.K.clear();  // its row sums are recomputed
      if (r->kind == kNew) {
        s->used -= sm.bytes();
        model_release(sm.m.get());
        release(&sm.S);
        s->models.erase(mit);
      }
    }
    r->model_out = 0;
    r->solo = true;
    s->queue.push_front(r);  // reverse walk: the round's order is kept
  }
  if (retry) {
    L.reqs.clear();
    L.busy = false;
    ++s->rounds;
    s->cv_work.notify_all();
    return;
  }
  for (Req *r : L.reqs) {
    const int64_t id = r->model ? r->model : r->model_out;
    auto mit = s->models.find(id);
    if (mit != s->models.end()) {
      SModel &sm = mit->second;
      sm.busy = false;
      sm.last_use = now_ms();
      if (!e.code) sm.ready = true;
      if (e.code && r->kind == kNew) {  // a failed new model is not kept
        s->used -= sm.bytes();
        model_release(sm.m.get());
        release(&sm.S);
        s->models.erase(mit);
        r->model_out = 0;
      }
    }
    if (!e.code) {
      r->I.assign(L.hI + r->offset, L.hI + r->offset + r->K.size());
      if (!r->model_out) r->model_out = r->model;
      complete(s, r, DBX_OK, "");
    } else {
      complete(s, r, e.code, e.msg);
    }
    ++s->completed;
  }
  L.reqs.clear();
  L.busy = false;
  ++s->rounds;
  s->cv_done.notify_all();
}

// Host preparation of a new model: spatial sort, tiles and the histogram
// plan (preparation thread, no lock).
Error prepare(Req *r) {
  const int P = (int)r->counts.size();
  int64_t natoms = 0;
  for (int64_t c : r->counts) natoms += c;
  r->hm = std::make_unique<Model>();
  r->atoms.resize(std::max<int64_t>(natoms, 1));
  DBX_TRY(model_prepare(r->x.data(), r->y.data(), r->z.data(), r->counts.data(), P,
                        r->hm.get(), r->atoms.data()));
  std::vector<int2> pairs;
  for (int a = 0; a < P; ++a)
    for (int b = a; b < P; ++b) pairs.push_back(make_int2(a, b));
  hist_plan_clear(&r->part);
  DBX_TRY(hist_plan_add(*r->hm, pairs, r->rstep, r->nbins, nullptr, pitch_of(r->nbins),
                        &r->part));
  // the coordinates are in r->atoms now
  std::vector<float>().swap(r->x);
  std::vector<float>().swap(r->y);
  std::vector<float>().swap(r->z);
  return ok();
}

void prep_main(dbx_server *s) {
  for (;;) {
    Req *r = nullptr;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      s->cv_prep.wait(lock, [&] { return s->stop || !s->prep_q.empty(); });
      if (s->prep_q.empty()) return;  // stopping, nothing left
      r = s->prep_q.front();
      s->prep_q.pop_front();
      ++s->prepping;
    }
    Error e = prepare(r);
    std::lock_guard<std::mutex> lock(s->mu);
    --s->prepping;
    if (e.code) {
      complete(s, r, e.code, e.msg);
      s->cv_done.notify_all();
    } else {
      s->queue.push_back(r);
    }
    s->cv_work.notify_all();
  }
}

void worker_main(dbx_server *s) {
  cudaSetDevice(s->device);
  int order[2] = {0, 1};  // lanes in launch order (oldest first)
  for (;;) {
    // retire lanes whose round has finished
    for (Lane &L : s->lanes)
      if (L.busy && cudaStreamQuery(L.stream) != cudaErrorNotReady)
        finish_round(s, L, ok());
    std::vector<Req *> batch;
    int free_lane = -1;
    bool any_busy;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      any_busy = s->lanes[0].busy || s->lanes[1].busy;
      const bool prep_idle = s->prep_q.empty() && s->prepping == 0;
      if (s->stop && s->queue.empty() && !any_busy && prep_idle) return;
      if (s->queue.empty() && !any_busy) {
        s->cv_work.wait(lock, [&] {
          return (s->stop && s->prep_q.empty() && s->prepping == 0) ||
                 !s->queue.empty();
        });
        continue;
      }
      for (int k = 0; k < 2; ++k)
        if (!s->lanes[order[k]].busy) {
          free_lane = order[k];
          break;
        }
      if (free_lane >= 0 && !s->queue.empty()) batch = admit(s);
      if (batch.empty() && !any_busy && !s->queue.empty()) {
        // nothing in flight and the head cannot be admitted: it never will
        Req *r = s->queue.front();
        s->queue.pop_front();
        complete(s, r, DBX_ERR_NOMEM, "request does not fit the HBM budget");
        s->cv_done.notify_all();
        continue;
      }
    }
    if (!batch.empty()) {
      Lane &L = s->lanes[free_lane];
      Error e = launch_round(s, L, batch);
      if (e.code) finish_round(s, L, e);
      if (order[0] == free_lane) std::swap(order[0], order[1]);  // newest last
    } else if (any_busy) {
      // nothing admissible now: wait for the oldest round in flight
      for (int k = 0; k < 2; ++k) {
        Lane &L = s->lanes[order[k]];
        if (L.busy) {
          finish_round(s, L, ok());
          break;
        }
      }
    }
  }
}

}  // namespace
}  // namespace dbx

extern "C" {

int dbx_server_create(dbx_server **out, int device, size_t budget) {
  if (!out) return DBX_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
    return DBX_ERR_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return DBX_ERR_CUDA;
  auto s = std::make_unique<dbx_server>();
  s->device = device;
  s->budget = budget;
  if (cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount,
                             device) != cudaSuccess)
    return DBX_ERR_CUDA;
  s->hist_tasks = 4 * s->num_sms;
  for (dbx::Lane &L : s->lanes) {
    if (cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess)
      return DBX_ERR_CUDA;
    // lane workspaces grow in the lane's stream order (no device-wide
    // synchronisation while the other lane computes)
    L.hws.arena = L.tc.arena = L.pref.arena = &L.arena;
    L.arena.take(size_t(64) << 20);  // initial capacity (grows when needed)
    L.arena.reset();
    L.hws.alloc_stream = L.tc.alloc_stream = L.pref.alloc_stream = L.stream;
  }
  dbx_server *raw = s.get();
  s->worker = std::thread(dbx::worker_main, raw);
  // host preparation (sort, plan) of new models runs beside the worker
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  for (unsigned i = 0; i < std::min(4u, std::max(1u, hw / 4)); ++i)
    s->preps.emplace_back(dbx::prep_main, raw);
  *out = s.release();
  return DBX_OK;
}

int dbx_server_submit(dbx_server *s, const dbx_request *q, int64_t *ticket) {
  if (!s || !q || !ticket || !q->K || q->nq < 1 || !q->sp || q->nspecies < 1 ||
      !(q->rstep > 0) || q->nbins < 1 || q->nbins > (int64_t(1) << 22))
    return DBX_ERR_ARG;
  auto r = std::make_unique<dbx::Req>();
  r->model = q->model;
  if (!q->model) {
    if (!q->species_counts) return DBX_ERR_ARG;
    int64_t natoms = 0;
    for (int i = 0; i < q->nspecies; ++i) {
      if (q->species_counts[i] < 0) return DBX_ERR_ARG;
      natoms += q->species_counts[i];
    }
    if (natoms > 0 && (!q->x || !q->y || !q->z)) return DBX_ERR_ARG;
    r->x.assign(q->x, q->x + natoms);
    r->y.assign(q->y, q->y + natoms);
    r->z.assign(q->z, q->z + natoms);
    r->counts.assign(q->species_counts, q->species_counts + q->nspecies);
  }
  r->sp.assign(q->sp, q->sp + q->nspecies);
  r->rstep = q->rstep;
  r->nbins = q->nbins;
  r->K.assign(q->K, q->K + q->nq);
  r->t_submit = dbx::now_ms();
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->stop) return DBX_ERR_ARG;
  r->ticket = s->next_ticket++;
  *ticket = r->ticket;
  if (r->model) {  // re-scoring: straight to admission
    s->queue.push_back(r.get());
    s->cv_work.notify_one();
  } else {
    s->prep_q.push_back(r.get());
    s->cv_prep.notify_one();
  }
  s->reqs[r->ticket] = std::move(r);
  return DBX_OK;
}

int dbx_server_wait(dbx_server *s, int64_t ticket, double *out_I, int nq,
                    int64_t *model_out, double *latency_ms) {
  if (!s) return DBX_ERR_ARG;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return DBX_ERR_ARG;
  dbx::Req *r = it->second.get();
  s->cv_done.wait(lock, [&] { return r->status != 1; });
  const int rc = r->status;
  if (rc == DBX_OK) {
    if (out_I) {
      if (nq < (int)r->I.size()) return DBX_ERR_ARG;
      std::memcpy(out_I, r->I.data(), r->I.size() * sizeof(double));
    }
  }
  if (model_out) *model_out = r->model_out;
  if (latency_ms) *latency_ms = r->t_done - r->t_submit;
  s->reqs.erase(it);
  return rc;
}

int dbx_server_stats(dbx_server *s, int64_t out[6]) {
  if (!s || !out) return DBX_ERR_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  out[0] = s->rounds;
  out[1] = s->completed;
  out[2] = (int64_t)s->models.size();
  out[3] = (int64_t)s->used;
  out[4] = s->evicted;
  out[5] = (int64_t)s->lane_reserve;
  return DBX_OK;
}

int dbx_server_destroy(dbx_server *s) {
  if (!s) return DBX_ERR_ARG;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_prep.notify_all();
  s->cv_work.notify_all();
  for (std::thread &t : s->preps)
    if (t.joinable()) t.join();
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(s->device);
  for (auto &kv : s->models) {
    dbx::model_release(kv.second.m.get());
    dbx::release(&kv.second.S);
  }
  for (dbx::Lane &L : s->lanes) {
    for (dbx::DevBuf *b : {&L.hws.items, &L.hws.segs, &L.hws.tasks, &L.hws.rows,
                           &L.hws.partial, &L.hws.oor, &L.pref.sp, &L.pref.colsp, &L.pref.f, &L.pref.fid,
                           &L.K, &L.ff, &L.I})
      dbx::release(b);
    dbx::tc_release(&L.tc);
    if (L.stream) cudaStreamDestroy(L.stream);
  }
  delete s;
  return DBX_OK;
}

}  // extern "C"
