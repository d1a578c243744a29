// Serving loop: intensity jobs of single block pairs, continuously batched
// over several device streams (include/gi.h, "Serving").
//
// The reference has no serving mode: it walks every initial level of one
// (J, J+1) run in a fixed order (cuda_host.cu:1174-1408).  Here an upstream
// eigensolver hands over (J, Gamma) blocks as it finishes them
// (gi_set_block / gi_set_block_device) and submits pair jobs
// (J, Gamma) -> (J', Gamma').  Each of `slots` worker threads owns a stream and
// the workspaces of one job in flight; the jobs share the context's dipole,
// bases, 3j table, dipole digits and blocks.  A job is admitted, in arrival
// order, when a slot is free and its blocks fit the device budget: blocks not
// resident are brought back from pinned host memory, after the least
// recently used blocks that no running job holds have been evicted there.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>

#include "engine.h"
#include "split.h"

namespace gi {

namespace {
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
}  // namespace

struct JobRec {
  uint64_t id = 0;
  int jI = 0, gI = 0, jF = 0, gF = 0;
  gi_params params{};
  double zpe = 0.0;
  int jmin = 0, jmax = 0;
  double qstat = 0.0;
  int state = GI_JOB_QUEUED;
  gi_status status = GI_OK;
  std::string err;
  std::vector<gi_line> lines;
  int64_t nlines_filtered = 0;
  double t_submit = 0, t_admit = 0, t_done = 0, seconds_gpu = 0;
};

// A cached half line strength (see zcache_acquire in engine.h).
struct ZEntry {
  uint64_t blk_uid = 0, blk_version = 0;
  int precision = 0, slices = 0;
  std::vector<int32_t> ivec;  // the initial records its columns hold
  DevArray<double> z;
  bool valid = false;         // written by a finished run
  int pins = 0;
  uint64_t last_use = 0;
  size_t bytes() const { return z.n * sizeof(double); }
};

struct Server {
  Ctx* owner = nullptr;
  int nslots = 0;
  size_t budget = 0, slot_ws = 0;
  std::vector<Ctx*> wctx;
  std::vector<std::thread> threads;
  std::deque<std::shared_ptr<JobRec>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<JobRec>> jobs;
  std::condition_variable cv_work, cv_done;
  bool stopping = false;
  uint64_t next_id = 1, clock = 0;
  int running = 0;
  int precision = GI_PREC_FP64, slices = 0;
  // statistics since the last reset
  std::vector<double> latency, queued;
  int64_t submitted = 0, completed = 0, failed = 0, lines = 0, lines_filtered = 0;
  int64_t evictions = 0, restores = 0;
  size_t peak_resident = 0;
  // cached half line strengths of initial blocks, shared by the jobs that
  // start from the same block (the same selection of its vectors)
  std::vector<std::unique_ptr<ZEntry>> zcache;
  bool zcache_on = true;
  int64_t z_hits = 0, z_misses = 0, z_evictions = 0;
};

// ------------------------------------------------------------------ residency
static size_t resident_bytes(Ctx* c) {
  size_t b = 0;
  for (auto& kv : c->blocks)
    if (kv.second->resident) b += kv.second->device_bytes();
  if (c->server)
    for (auto& e : c->server->zcache) b += e->bytes();
  return b;
}

static size_t block_budget(const Server* s) {
  const size_t ws = (size_t)s->nslots * s->slot_ws;
  return s->budget > ws ? s->budget - ws : 0;
}

// Moves a block's vectors to pinned host memory and frees its device arrays
// (the digits are recut when it comes back).  A host copy of the same
// version, kept from an earlier eviction, makes this free.
static gi_status evict(Ctx* c, Block& b) {
  if (!b.resident) return GI_OK;
  const size_t n = (size_t)b.nvec * b.nsize;
  if (n && !(b.h_vecs && b.h_version == b.version)) {
    if (!b.h_vecs)
      GI_CUDA(c, cudaMallocHost(reinterpret_cast<void**>(&b.h_vecs), sizeof(double) * n));
    GI_CUDA(c, cudaMemcpy2D(b.h_vecs, sizeof(double) * b.nsize, b.d_vecs.p, sizeof(double) * b.ld,
                            sizeof(double) * b.nsize, b.nvec, cudaMemcpyDeviceToHost));
    b.h_version = b.version;
  }
  b.d_vecs.reset();
  b.d_digits.reset();
  b.d_digit_exp.reset();
  b.digits_s = 0;
  b.resident = false;
  c->server->evictions++;
  return GI_OK;
}

static gi_status restore(Ctx* c, Block& b) {
  if (b.resident) return GI_OK;
  const size_t need = (size_t)std::max(b.nvec, 1) * b.ld;
  GI_CUDA(c, b.d_vecs.alloc(need));
  GI_CUDA(c, cudaMemset(b.d_vecs.p, 0, sizeof(double) * need));
  if (b.nvec)
    GI_CUDA(c, cudaMemcpy2D(b.d_vecs.p, sizeof(double) * b.ld, b.h_vecs, sizeof(double) * b.nsize,
                            sizeof(double) * b.nsize, b.nvec, cudaMemcpyHostToDevice));
  GI_CUDA(c, cudaStreamSynchronize(cudaStreamLegacy));
  b.resident = true;  // h_vecs stays: the next eviction of this version is free
  c->server->restores++;
  return GI_OK;
}

// Device bytes a block needs to run as the initial (vectors) or final
// (vectors and, in split precision, their digits) block of a job.
static size_t need_bytes(const Server* s, const Block& b, bool final_block) {
  size_t n = 0;
  if (!b.resident) n += (size_t)std::max(b.nvec, 1) * b.ld * sizeof(double);
  if (final_block && s->precision == GI_PREC_SPLIT && (!b.resident || b.digits_s == 0)) {
    const int s_digits = split_digits(s->owner);
    const size_t vpad = (size_t)round_up(std::max(b.nvec, 1), 128);
    n += (size_t)s_digits * vpad * b.ld * sizeof(uint16_t) + vpad * sizeof(int32_t);
  }
  return n;
}

gi_status server_make_room(Ctx* c, size_t bytes, Block* keep) {
  Server* s = c->server;
  if (!s) return GI_OK;
  const size_t cap = block_budget(s);
  size_t used = resident_bytes(c);
  while (used + bytes > cap) {
    // the least recently used of the unpinned blocks and cached Z (one clock
    // for both); a cached Z is dropped (recomputed when a job needs it), a
    // block moves to pinned host memory
    Block* victim = nullptr;
    for (auto& kv : c->blocks) {
      Block* b = kv.second.get();
      if (!b->resident || b->pins > 0 || b == keep || b->device_bytes() == 0) continue;
      if (!victim || b->last_use < victim->last_use) victim = b;
    }
    size_t zv = s->zcache.size();
    for (size_t k = 0; k < s->zcache.size(); k++) {
      const ZEntry& e = *s->zcache[k];
      if (e.pins > 0) continue;
      if (zv == s->zcache.size() || e.last_use < s->zcache[zv]->last_use) zv = k;
    }
    if (zv < s->zcache.size() && (!victim || s->zcache[zv]->last_use < victim->last_use)) {
      s->zcache.erase(s->zcache.begin() + zv);
      s->z_evictions++;
    } else if (victim) {
      gi_status st = evict(c, *victim);
      if (st != GI_OK) return st;
    } else {
      return fail(c, GI_ERR_BUDGET, "serving budget: %zu bytes more do not fit (%zu of %zu used)",
                  bytes, used, cap);
    }
    used = resident_bytes(c);
  }
  return GI_OK;
}

// ------------------------------------------------------------------ Z cache
gi_status zcache_acquire(Ctx* w, const Block* blk, const int32_t* ivec, int nI, size_t elems,
                         ZRef* out) {
  *out = ZRef{};
  Ctx* c = w->parent;
  Server* s = c ? c->server : nullptr;
  if (!s || !s->zcache_on || nI <= 0) return GI_OK;
  std::lock_guard<std::mutex> lk(c->model_mu);
  const int prec = w->params.precision, sl = w->params.split_slices;
  for (auto& ep : s->zcache) {
    ZEntry& e = *ep;
    if (e.blk_uid != blk->uid || e.blk_version != blk->version || e.precision != prec ||
        e.slices != sl || (int)e.ivec.size() != nI ||
        !std::equal(e.ivec.begin(), e.ivec.end(), ivec))
      continue;
    if (!e.valid) {  // another job is filling it: compute without the cache
      s->z_misses++;
      return GI_OK;
    }
    e.pins++;
    e.last_use = ++s->clock;
    s->z_hits++;
    *out = ZRef{&e, e.z.p, true};
    return GI_OK;
  }
  // a new entry, if it fits the budget beside everything the running jobs hold
  // and takes at most a quarter of it (one large entry would push out many
  // small ones that are asked for more often)
  s->z_misses++;
  const size_t bytes = elems * sizeof(double);
  if (bytes > block_budget(s) / 4) return GI_OK;
  if (server_make_room(c, bytes, nullptr) != GI_OK) {
    c->err.clear();
    return GI_OK;
  }
  auto e = std::make_unique<ZEntry>();
  e->blk_uid = blk->uid;
  e->blk_version = blk->version;
  e->precision = prec;
  e->slices = sl;
  e->ivec.assign(ivec, ivec + nI);
  if (e->z.alloc(elems) != cudaSuccess) {
    cudaGetLastError();
    return GI_OK;
  }
  e->pins = 1;
  e->last_use = ++s->clock;
  *out = ZRef{e.get(), e->z.p, false};
  s->zcache.push_back(std::move(e));
  s->peak_resident = std::max(s->peak_resident, resident_bytes(c));
  return GI_OK;
}

void zcache_release(Ctx* w, ZRef& r, bool ok) {
  if (!r.e) return;
  Ctx* c = w->parent;
  Server* s = c->server;
  std::lock_guard<std::mutex> lk(c->model_mu);
  for (size_t k = 0; k < s->zcache.size(); k++) {
    if (s->zcache[k].get() != r.e) continue;
    ZEntry& e = *s->zcache[k];
    e.pins--;
    if (!r.hit) {
      if (ok) {
        e.valid = true;
      } else if (e.pins == 0) {
        s->zcache.erase(s->zcache.begin() + k);
      }
    }
    break;
  }
  r = ZRef{};
}

// ------------------------------------------------------------------ workers
static void finish(Server* s, JobRec& j, gi_status st, const std::string& err) {
  j.status = st;
  j.err = err;
  j.state = st == GI_OK ? GI_JOB_DONE : GI_JOB_FAILED;
  j.t_done = now_s();
  if (st == GI_OK) {
    s->completed++;
    s->lines += (int64_t)j.lines.size();
    s->lines_filtered += j.nlines_filtered;
    s->latency.push_back(j.t_done - j.t_submit);
    s->queued.push_back(j.t_admit - j.t_submit);
  } else {
    s->failed++;
  }
}

static void worker_main(Server* s, int slot) {
  Ctx* c = s->owner;
  Ctx* w = s->wctx[slot];
  cudaSetDevice(c->device);
  std::unique_lock<std::mutex> lk(c->model_mu);
  for (;;) {
    s->cv_work.wait(lk, [&] { return s->stopping || !s->queue.empty(); });
    if (s->queue.empty()) break;  // stopping with nothing left
    std::shared_ptr<JobRec> j = s->queue.front();
    auto iI = c->blocks.find({j->jI, j->gI});
    auto iF = c->blocks.find({j->jF, j->gF});
    if (iI == c->blocks.end() || iF == c->blocks.end() || !c->bases.count(j->jI) ||
        !c->bases.count(j->jF)) {
      s->queue.pop_front();
      finish(s, *j, GI_ERR_NOTFOUND, "block or basis of the job is not loaded");
      s->cv_done.notify_all();
      continue;
    }
    std::shared_ptr<Block> bI = iI->second, bF = iF->second;
    size_t need = need_bytes(s, *bF, true);
    if (bI != bF) need += need_bytes(s, *bI, false);
    // admission: evict unpinned blocks (never this job's) until the job fits
    bI->pins++;
    bF->pins++;
    gi_status st = server_make_room(c, need, nullptr);
    if (st != GI_OK) {
      bI->pins--;
      bF->pins--;
      if (s->running > 0) {  // memory comes back when a running job ends
        s->cv_work.wait(lk);
        continue;
      }
      s->queue.pop_front();
      finish(s, *j, st, c->err);
      s->cv_done.notify_all();
      continue;
    }
    s->queue.pop_front();
    st = restore(c, *bI);
    if (st == GI_OK) st = restore(c, *bF);
    bI->last_use = bF->last_use = ++s->clock;
    s->peak_resident = std::max(s->peak_resident, resident_bytes(c) + need_bytes(s, *bF, true));
    j->state = GI_JOB_RUNNING;
    j->t_admit = now_s();
    s->running++;
    // the worker's view of the model: this pair's bases and blocks
    w->params = j->params;
    w->have_params = true;
    w->bases.clear();
    w->bases[j->jI] = c->bases[j->jI];
    w->bases[j->jF] = c->bases[j->jF];
    w->blocks.clear();
    w->blocks[{j->jI, j->gI}] = bI;
    w->blocks[{j->jF, j->gF}] = bF;
    w->threej = c->threej;
    w->threej_jmax = c->threej_jmax;
    w->threej_user = c->threej_user;
    w->job = JobSel{true, j->jI, j->gI, j->jF, j->gF, j->zpe, j->jmin, j->jmax, j->qstat};
    lk.unlock();
    int64_t n = 0;
    std::string err;
    if (st == GI_OK) {
      w->err.clear();
      st = run_job(w, 0, &n);
      if (st == GI_OK) {
        j->lines.assign(w->h_lines, w->h_lines + n);
        j->nlines_filtered = w->stats.nlines_filtered;
        j->seconds_gpu = w->stats.seconds_gpu;
      }
      err = w->err;
    } else {
      err = c->err;
    }
    w->blocks.clear();
    lk.lock();
    bI->pins--;
    bF->pins--;
    s->running--;
    finish(s, *j, st, err);
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

static Ctx* make_worker(Ctx* c, size_t slot_ws) {
  Ctx* w = new Ctx();
  w->parent = c;
  w->device = c->device;
  w->budget = 2 * slot_ws;  // the round planner keeps its workspaces within budget / 2
  w->nsm = c->nsm;
  if (cudaStreamCreateWithFlags(&w->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&w->ev0) != cudaSuccess || cudaEventCreate(&w->ev1) != cudaSuccess) {
    delete w;
    return nullptr;
  }
  w->stream = w->own_stream;
  w->sym_type = c->sym_type;
  w->nrep = c->nrep;
  w->degen = c->degen;
  w->N = c->N;
  w->Kp = c->Kp;
  w->tune_mode = c->tune_mode;
  w->tune_path = c->tune_path;
  return w;
}

static void destroy_worker(Ctx* w) { ctx_release(w); }

static double pct(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

gi_status server_stop(Ctx* c) {
  Server* s = c->server;
  if (!s) return GI_OK;
  {
    std::lock_guard<std::mutex> lk(c->model_mu);
    s->stopping = true;
    for (auto& j : s->queue) finish(s, *j, GI_ERR_STATE, "serving stopped before admission");
    s->queue.clear();
  }
  s->cv_work.notify_all();
  for (auto& t : s->threads) t.join();
  for (Ctx* w : s->wctx) destroy_worker(w);
  c->server = nullptr;
  delete s;
  return GI_OK;
}

}  // namespace gi

// ====================================================================== C ABI
using namespace gi;

extern "C" {

gi_status gi_serve_start(gi_ctx* h, const gi_serve_config* cfg) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return GI_ERR_ARG;
  if (c->server) return fail(c, GI_ERR_STATE, "serving already started");
  if (c->nrep == 0 || !c->have_params || c->N == 0 || c->bases.empty())
    return fail(c, GI_ERR_STATE, "symmetry, parameters, dipole and bases precede gi_serve_start");
  if (c->dstream) return fail(c, GI_ERR_STATE, "serving needs a resident dipole (gi_set_dipole)");
  cudaSetDevice(c->device);
  gi_serve_config cf{};
  if (cfg) cf = *cfg;
  const int slots = cf.slots > 0 ? cf.slots : 3;
  if (slots > 16) return fail(c, GI_ERR_ARG, "at most 16 serving slots");
  size_t budget = cf.hbm_budget_bytes ? cf.hbm_budget_bytes : c->budget;
  if (!budget) {
    size_t fr = 0, tot = 0;
    GI_CUDA(c, cudaMemGetInfo(&fr, &tot));
    budget = fr / 10 * 8;
  }
  const size_t slot_ws = cf.slot_workspace_bytes ? cf.slot_workspace_bytes : budget / (4 * slots);
  if ((size_t)slots * slot_ws >= budget)
    return fail(c, GI_ERR_ARG, "slot workspaces (%d x %zu bytes) leave no room for blocks", slots,
                slot_ws);
  // the dipole digits are cut once, before any worker runs
  if (c->params.precision == GI_PREC_SPLIT) {
    gi_status st = split_prepare(c);
    if (st != GI_OK) return st;
  }
  {
    std::lock_guard<std::mutex> lk(c->model_mu);
    for (auto& kv : c->bases) {
      gi_status st = ensure_ycsr(c, *kv.second);
      if (st != GI_OK) return st;
    }
    const int jmax = c->bases.rbegin()->first;
    if (c->threej_jmax < jmax) {
      precompute_threej(jmax, c->threej);
      c->threej_jmax = jmax;
      c->threej_user = false;
    }
  }
  Server* s = new Server();
  s->owner = c;
  s->nslots = slots;
  s->budget = budget;
  s->slot_ws = slot_ws;
  s->precision = c->params.precision;
  s->slices = c->params.split_slices;
  s->zcache_on = !(cf.flags & GI_SERVE_NO_ZCACHE);
  for (int i = 0; i < slots; i++) {
    Ctx* w = make_worker(c, slot_ws);
    if (!w) {
      for (Ctx* x : s->wctx) destroy_worker(x);
      delete s;
      return fail(c, GI_ERR_CUDA, "could not create serving stream %d", i);
    }
    s->wctx.push_back(w);
  }
  {
    std::lock_guard<std::mutex> lk(c->model_mu);
    c->server = s;
    // blocks loaded before serving count against the budget from now on
    gi_status st = server_make_room(c, 0, nullptr);
    if (st != GI_OK) {
      c->server = nullptr;
      for (Ctx* x : s->wctx) destroy_worker(x);
      delete s;
      return st;
    }
  }
  for (int i = 0; i < slots; i++) s->threads.emplace_back(worker_main, s, i);
  return GI_OK;
}

gi_status gi_serve_stop(gi_ctx* h) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return GI_ERR_ARG;
  return server_stop(c);
}

gi_status gi_submit(gi_ctx* h, int jI, int gammaI, int jF, int gammaF, uint64_t* id) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !id) return GI_ERR_ARG;
  Server* s = c->server;
  if (!s) return fail(c, GI_ERR_STATE, "gi_serve_start not called");
  if (gammaI < 0 || gammaI >= c->nrep || gammaF < 0 || gammaF >= c->nrep || std::abs(jI - jF) > 1)
    return fail(c, GI_ERR_ARG, "job (J=%d, gamma=%d) -> (J=%d, gamma=%d) is not a block pair", jI,
                gammaI, jF, gammaF);
  if (c->params.precision != s->precision || c->params.split_slices != s->slices)
    return fail(c, GI_ERR_STATE, "precision changed while serving");
  auto j = std::make_shared<JobRec>();
  j->jI = jI;
  j->gI = gammaI;
  j->jF = jF;
  j->gF = gammaF;
  j->params = c->params;
  j->t_submit = now_s();
  {
    std::lock_guard<std::mutex> lk(c->model_mu);
    // the filters of the whole loaded job: its J range and ZPE
    j->jmin = c->bases.begin()->first;
    j->jmax = c->bases.rbegin()->first;
    double zpe = c->params.ZPE;
    auto it = c->blocks.find({0, 0});
    if (zpe < 0 && c->bases.count(0) && c->params.gns[0] > 0.00000001 && it != c->blocks.end() &&
        !it->second->energies.empty())
      zpe = it->second->energies[0];
    j->zpe = zpe;
    j->qstat = c->params.q_stat > 0 ? c->params.q_stat
                                    : partition_sum(c, c->params.temperature, zpe);
    j->id = s->next_id++;
    s->jobs[j->id] = j;
    s->queue.push_back(j);
    s->submitted++;
  }
  s->cv_work.notify_one();
  *id = j->id;
  return GI_OK;
}

gi_status gi_job_wait(gi_ctx* h, uint64_t id, double timeout_s, gi_job_info* info) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return GI_ERR_ARG;
  Server* s = c->server;
  if (!s) return fail(c, GI_ERR_STATE, "gi_serve_start not called");
  std::unique_lock<std::mutex> lk(c->model_mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return fail(c, GI_ERR_NOTFOUND, "unknown job %llu", (unsigned long long)id);
  std::shared_ptr<JobRec> j = it->second;
  auto done = [&] { return j->state == GI_JOB_DONE || j->state == GI_JOB_FAILED; };
  if (timeout_s < 0)
    s->cv_done.wait(lk, done);
  else
    s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done);
  if (info) {
    gi_job_info r{};
    r.state = j->state;
    r.status = j->status;
    r.nlines = (int64_t)j->lines.size();
    r.nlines_filtered = j->nlines_filtered;
    r.seconds_queued = j->t_admit > 0 ? j->t_admit - j->t_submit : now_s() - j->t_submit;
    r.seconds_latency = done() ? j->t_done - j->t_submit : now_s() - j->t_submit;
    r.seconds_gpu = j->seconds_gpu;
    *info = r;
  }
  if (j->state == GI_JOB_FAILED) {
    c->err = j->err;
    return j->status;
  }
  return GI_OK;
}

gi_status gi_job_lines(gi_ctx* h, uint64_t id, int64_t offset, int64_t count, gi_line* out) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || offset < 0 || count < 0 || (count && !out)) return GI_ERR_ARG;
  Server* s = c->server;
  if (!s) return fail(c, GI_ERR_STATE, "gi_serve_start not called");
  std::lock_guard<std::mutex> lk(c->model_mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return fail(c, GI_ERR_NOTFOUND, "unknown job %llu", (unsigned long long)id);
  const JobRec& j = *it->second;
  if (j.state != GI_JOB_DONE) return fail(c, GI_ERR_STATE, "job %llu has not finished", (unsigned long long)id);
  if (offset + count > (int64_t)j.lines.size()) return fail(c, GI_ERR_ARG, "line range past the end");
  if (count) std::memcpy(out, j.lines.data() + offset, sizeof(gi_line) * count);
  return GI_OK;
}

gi_status gi_job_release(gi_ctx* h, uint64_t id) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return GI_ERR_ARG;
  Server* s = c->server;
  if (!s) return fail(c, GI_ERR_STATE, "gi_serve_start not called");
  std::lock_guard<std::mutex> lk(c->model_mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return fail(c, GI_ERR_NOTFOUND, "unknown job %llu", (unsigned long long)id);
  if (it->second->state != GI_JOB_DONE && it->second->state != GI_JOB_FAILED)
    return fail(c, GI_ERR_STATE, "job %llu is still in flight", (unsigned long long)id);
  s->jobs.erase(it);
  return GI_OK;
}

gi_status gi_serve_get_stats(gi_ctx* h, gi_serve_stats* out) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !out) return GI_ERR_ARG;
  Server* s = c->server;
  if (!s) return fail(c, GI_ERR_STATE, "gi_serve_start not called");
  std::lock_guard<std::mutex> lk(c->model_mu);
  gi_serve_stats r{};
  r.submitted = s->submitted;
  r.completed = s->completed;
  r.failed = s->failed;
  r.lines = s->lines;
  r.lines_filtered = s->lines_filtered;
  r.evictions = s->evictions;
  r.restores = s->restores;
  r.queued = (int32_t)s->queue.size();
  r.running = s->running;
  r.latency_p50 = pct(s->latency, 0.50);
  r.latency_p99 = pct(s->latency, 0.99);
  r.latency_max = pct(s->latency, 1.0);
  double sum = 0;
  for (double v : s->latency) sum += v;
  r.latency_mean = s->latency.empty() ? 0.0 : sum / (double)s->latency.size();
  r.queue_p50 = pct(s->queued, 0.50);
  r.queue_p99 = pct(s->queued, 0.99);
  r.resident_bytes = resident_bytes(c);
  r.peak_resident_bytes = s->peak_resident;
  r.budget_bytes = s->budget;
  r.slot_workspace_bytes = s->slot_ws;
  r.slots = s->nslots;
  r.zcache_hits = s->z_hits;
  r.zcache_misses = s->z_misses;
  r.zcache_evictions = s->z_evictions;
  for (auto& e : s->zcache) r.zcache_bytes += e->bytes();
  *out = r;
  return GI_OK;
}

gi_status gi_serve_reset_stats(gi_ctx* h) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return GI_ERR_ARG;
  Server* s = c->server;
  if (!s) return fail(c, GI_ERR_STATE, "gi_serve_start not called");
  std::lock_guard<std::mutex> lk(c->model_mu);
  s->latency.clear();
  s->queued.clear();
  s->submitted = s->completed = s->failed = s->lines = s->lines_filtered = 0;
  s->evictions = s->restores = 0;
  s->z_hits = s->z_misses = s->z_evictions = 0;
  s->peak_resident = resident_bytes(c);
  return GI_OK;
}

}  // extern "C"
