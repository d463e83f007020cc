// Batched render serving (gbpt_server_*): requests of uneven size, from any
// host thread, share one GPU.
//
// The reference renders one scene per process with synchronous calls and
// process-global device state (src/cudaRTBDPTStream.cu:134-169, 816-951).
// Here every worker thread owns renderers (each with its own CUDA stream) and
// runs one request at a time; with several workers the persistent walks of
// small requests run side by side on the SMs (a persistent grid whose ray
// queue is empty exits at once, so a concurrent request's CTAs take its
// place).  Scenes are shared and stay resident.
//
// Order: first come first served, or (default) shortest first with aging --
// the queued request with the least estimated run time minus time already
// waited starts next, so a burst of small requests is not stuck behind a
// large one and a large one is not passed over for long.
//
// Admission: a request starts when its renderer's device buffers fit in free
// HBM minus the reserve; otherwise the worker first frees its own idle
// renderers, then waits for running requests to finish, and fails the request
// with GBPT_ERR_OOM only when no other request is running.
//
// Autotuning: the walks' refill threshold, the bounce from which the tail
// kernel carries the remaining paths (fixed, or decided on the device below a
// live-path fraction), the bands a frame is split into and the persistent
// grids' CTAs per SM change scheduling and launch shape only -- every path
// executes the same operations in the same order -- so images are identical
// whichever values run.  Requests that leave them at their defaults
// (walk_refill 0, tail_from -1, bands 0, walk_ctas 0, tail_below the
// library's default) are assigned a candidate
// per class (mode,
// depth cap, image size rounded to a power of two); each candidate is timed
// on whole requests (device time per camera path) until it has kTrials
// samples, after which the class uses the fastest.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "gbpt_internal.h"

using namespace gbpt;

// the ctypes binding (cudapt_gb300/_native.py) mirrors these layouts
static_assert(sizeof(gbpt_request) == 80, "gbpt_request layout");
static_assert(sizeof(gbpt_request_status) == 56, "gbpt_request_status layout");

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Knobs {
  uint32_t refill;
  int32_t tail;    // -1: the library's rule
  uint32_t bands;  // wavefronts per frame
  uint32_t ctas;   // CTAs per SM of the persistent walk and tail grids (0: as many as fit)
  float below;     // live-path fraction below which the device switches to the tail kernel
  bool operator==(const Knobs& o) const {
    return refill == o.refill && tail == o.tail && bands == o.bands && ctas == o.ctas && below == o.below;
  }
};

// Candidates per class: the library default first (one band: concurrent
// requests already overlap each other's walks), then the refill thresholds
// and tail starts around it that measured within a few percent on the
// large workloads (small images favour earlier refills and earlier tails;
// a frame near the walk grid's size can go either way), then launch shapes:
// persistent grids of 2 or 3 CTAs per SM, which leave SMs to the requests
// running beside, and the tail switch decided on the device at two
// live-path fractions.  (Two bands, once a candidate for images of 512K
// pixels and more, measured 7-9 % slower than one band since walks are
// carried between launches.)
std::vector<Knobs> candidates(uint32_t depth, uint32_t sizeLog2, float below) {
  (void)sizeLog2;
  std::vector<Knobs> c;
  auto add = [&](Knobs k) {
    if (std::find(c.begin(), c.end(), k) == c.end()) c.push_back(k);
  };
  const uint32_t rf = walk_refill_for(0, false);  // the library's refill threshold
  add({rf, -1, 1, 0, below});
  add({4, -1, 1, 0, below});
  add({8, -1, 1, 0, below});
  if (depth > 3) add({rf, (int32_t)depth - 3, 1, 0, below});
  if (depth > 5) add({rf, (int32_t)depth - 5, 1, 0, below});
  if (depth > 6) add({rf, (int32_t)depth / 2 - 1, 1, 0, below});
  if (depth > 2) add({rf, 2, 1, 0, below});  // the default for frames smaller than the walk grid
  add({rf, (int32_t)depth, 1, 0, 0.f});  // no tail kernel but the carried walks'
  add({rf, -1, 1, 2, below});
  add({rf, -1, 1, 3, below});
  for (float f : {0.25f, 0.5f})
    if (f != below) add({rf, (int32_t)depth, 1, 0, f});
  return c;
}

constexpr uint32_t kTrials = 2;

// run-time estimate of the shortest-first order: camera paths per ms of one
// request alone (about the plain walk's rate on the benchmark scenes)
constexpr double kPathsPerMs = 1e5;

struct ClassKey {
  int32_t mode;
  uint32_t depth, size;  // size: ceil(log2(width * height))
  bool operator<(const ClassKey& o) const {
    return std::tie(mode, depth, size) < std::tie(o.mode, o.depth, o.size);
  }
};

struct Tuning {
  std::vector<Knobs> cand;
  std::vector<double> msPerPath;  // summed over trials
  std::vector<uint32_t> trials;
  uint32_t next = 0;              // round-robin cursor while exploring
};

struct Request {
  uint64_t id = 0;
  gbpt_request q{};
  gbpt_params p{};
  bool tuned = false;  // knobs come from the autotuner
  Knobs knobs{0, -1, 0, 0, 0.f};
  Clock::time_point tSubmit, tStart, tEnd;
  gbpt_status status = GBPT_OK;
  std::string err;
  bool done = false;
  uint64_t paths = 0;
  // the depth cap of the request's mode (its autotuning class)
  uint32_t depth() const { return q.mode == GBPT_MODE_PT_SC ? p.pt_depth_max : p.eye_depth_max; }
  uint32_t size() const {
    uint64_t n = (uint64_t)q.width * q.height, c = 0;
    while ((1ull << c) < n) c++;
    return (uint32_t)c;
  }
};

struct PoolKey {
  uint32_t w, h;
  int32_t mode;
  bool operator<(const PoolKey& o) const { return std::tie(w, h, mode) < std::tie(o.w, o.h, o.mode); }
};

}  // namespace

struct gbpt_server {
  std::mutex mu;
  std::condition_variable cvWork, cvDone, cvMem;
  std::deque<std::shared_ptr<Request>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> reqs;
  std::map<ClassKey, Tuning> tuning;
  std::vector<std::thread> workers;
  uint64_t nextId = 1;
  uint64_t reserve = 0;
  uint32_t running = 0;
  bool stop = false;
  int device = 0;
  int32_t policy = GBPT_SERVE_SHORTEST_FIRST;
  bool graphs = true;  // renderers issue plain / PTSC frames as CUDA graphs

  ~gbpt_server() {
    {
      std::lock_guard<std::mutex> lock(mu);
      stop = true;
    }
    cvWork.notify_all();
    cvMem.notify_all();
    for (auto& t : workers) t.join();
  }

  // knobs for a request of class k (called with mu held)
  Knobs assign(const ClassKey& k) {
    Tuning& t = tuning[k];
    if (t.cand.empty()) {
      gbpt_params dflt;
      gbpt_params_default(&dflt);
      t.cand = candidates(k.depth, k.size, dflt.tail_below);
      t.msPerPath.assign(t.cand.size(), 0.0);
      t.trials.assign(t.cand.size(), 0);
    }
    for (size_t i = 0; i < t.cand.size(); i++) {
      const size_t j = (t.next + i) % t.cand.size();
      if (t.trials[j] < kTrials) {
        t.next = (uint32_t)((j + 1) % t.cand.size());
        return t.cand[j];
      }
    }
    return t.cand[best(t)];
  }

  static size_t best(const Tuning& t) {
    size_t b = 0;
    double bv = 1e300;
    for (size_t i = 0; i < t.cand.size(); i++) {
      if (t.trials[i] == 0) continue;
      const double v = t.msPerPath[i] / t.trials[i];
      if (v < bv) {
        bv = v;
        b = i;
      }
    }
    return b;
  }

  void record(const ClassKey& k, const Knobs& kn, double msPerPath) {
    Tuning& t = tuning[k];
    for (size_t i = 0; i < t.cand.size(); i++)
      if (t.cand[i] == kn) {
        t.msPerPath[i] += msPerPath;
        t.trials[i]++;
      }
  }

  void worker_main();
};

namespace {

struct Pooled {
  gbpt_renderer* r = nullptr;
  uint64_t bytes = 0;
};

// the renderers of one worker thread, one per (size, mode); a worker runs one
// request at a time, so all of them are idle between requests
struct Pool {
  std::map<PoolKey, Pooled> m;
  ~Pool() {
    for (auto& kv : m) gbpt_renderer_destroy(kv.second.r);
  }
  bool drop_one_except(const PoolKey& keep) {
    for (auto it = m.begin(); it != m.end(); ++it)
      if (it->first < keep || keep < it->first) {
        gbpt_renderer_destroy(it->second.r);
        m.erase(it);
        return true;
      }
    return false;
  }
};

uint64_t free_hbm() {
  size_t f = 0, t = 0;
  if (cudaMemGetInfo(&f, &t) != cudaSuccess) return 0;
  return f;
}

// admission and allocation of the renderer for `k` are serialised over the
// workers, so two requests never count the same free bytes
std::mutex g_admit;

}  // namespace

static gbpt_status run_request(gbpt_server* srv, Pool& pool, Request& q, std::string& err) {
  const PoolKey key{q.q.width, q.q.height, q.q.mode};
  gbpt_params p = q.p;
  if (q.tuned) {
    p.walk_refill = q.knobs.refill;
    p.tail_from = q.knobs.tail;
    p.bands = q.knobs.bands;
    p.walk_ctas = q.knobs.ctas;
    p.tail_below = q.knobs.below;
  }
  gbpt_renderer* r = nullptr;
  {
    std::unique_lock<std::mutex> admit(g_admit);
    auto it = pool.m.find(key);
    if (it != pool.m.end()) {
      r = it->second.r;
    } else {
      const uint64_t need = renderer_bytes(q.q.width, q.q.height, p) + (64ull << 20);
      for (;;) {
        if (free_hbm() >= need + srv->reserve) break;
        if (pool.drop_one_except(key)) continue;
        std::unique_lock<std::mutex> lock(srv->mu);
        if (srv->running <= 1) {
          err = "request needs " + std::to_string(need) + " device bytes above the reserve; " +
                std::to_string(free_hbm()) + " free";
          return GBPT_ERR_OOM;
        }
        admit.unlock();
        srv->cvMem.wait_for(lock, std::chrono::milliseconds(50));
        lock.unlock();
        admit.lock();
      }
      gbpt_status st = gbpt_renderer_create(q.q.width, q.q.height, q.q.mode, &p, &r);
      if (st == GBPT_OK) st = gbpt_render_frames(r, q.q.scene, &q.q.camera, 0, nullptr);  // allocates
      if (st != GBPT_OK) {
        err = gbpt_last_error_string();
        if (r) gbpt_renderer_destroy(r);
        return st;
      }
      pool.m[key] = Pooled{r, need};
    }
  }
  gbpt_status st = gbpt_set_params(r, &p);
  if (st == GBPT_OK) st = gbpt_reset(r);
  if (st == GBPT_OK) st = gbpt_renderer_set_graphs(r, srv->graphs ? 1 : 0);
  gbpt_stats a{}, b{};
  if (st == GBPT_OK && q.q.frames > 1) st = gbpt_render_frames(r, q.q.scene, &q.q.camera, q.q.frames - 1, &a);
  if (st == GBPT_OK && q.q.frames > 0) st = gbpt_render(r, q.q.scene, &q.q.camera, q.q.out_rgb, 0, &b);
  if (st != GBPT_OK) {
    err = gbpt_last_error_string();
    return st;
  }
  q.paths = (uint64_t)q.q.width * q.q.height * q.q.frames;
  if (q.tuned && q.paths) {
    const double ms = (q.q.frames > 1 ? a.ms_total : 0.0) + b.ms_total;
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->record(ClassKey{q.q.mode, q.depth(), q.size()}, q.knobs, ms / q.paths);
  }
  return GBPT_OK;
}

void gbpt_server::worker_main() {
  cudaSetDevice(device);
  Pool pool;
  for (;;) {
    std::shared_ptr<Request> req;
    {
      std::unique_lock<std::mutex> lock(mu);
      cvWork.wait(lock, [&] { return stop || !queue.empty(); });
      if (queue.empty()) return;  // stopping, nothing left
      auto pick = queue.begin();
      if (policy == GBPT_SERVE_SHORTEST_FIRST) {  // least (estimated run time - time waited)
        const Clock::time_point now = Clock::now();
        double bestKey = 1e300;
        for (auto it = queue.begin(); it != queue.end(); ++it) {
          const double key = (double)(*it)->q.width * (*it)->q.height * (*it)->q.frames / kPathsPerMs -
                             ms_between((*it)->tSubmit, now);
          if (key < bestKey) {
            bestKey = key;
            pick = it;
          }
        }
      }
      req = *pick;
      queue.erase(pick);
      running++;
      if (req->tuned) req->knobs = assign(ClassKey{req->q.mode, req->depth(), req->size()});
    }
    req->tStart = Clock::now();
    std::string err;
    nvtxRangePushA("gbpt request");
    const gbpt_status st = run_request(this, pool, *req, err);
    nvtxRangePop();
    {
      std::lock_guard<std::mutex> lock(mu);
      req->tEnd = Clock::now();
      req->status = st;
      req->err = err;
      req->done = true;
      running--;
    }
    cvDone.notify_all();
    cvMem.notify_all();
  }
}

gbpt_status gbpt_server_create(uint32_t workers, uint64_t hbm_reserve_bytes, gbpt_server** out) {
  if (!out) return fail(GBPT_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (workers < 1 || workers > 64) return fail(GBPT_ERR_INVALID_ARG, "workers must be 1..64");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(GBPT_ERR_NO_DEVICE, "no CUDA device");
  gbpt_server* s = new (std::nothrow) gbpt_server();
  if (!s) return fail(GBPT_ERR_OOM, "host allocation failed");
  s->reserve = hbm_reserve_bytes;
  s->device = dev;
  for (uint32_t i = 0; i < workers; i++) s->workers.emplace_back([s] { s->worker_main(); });
  *out = s;
  return GBPT_OK;
}

gbpt_status gbpt_server_set_policy(gbpt_server* s, int32_t policy) {
  if (!s) return fail(GBPT_ERR_INVALID_ARG, "server is NULL");
  if (policy != GBPT_SERVE_FIFO && policy != GBPT_SERVE_SHORTEST_FIRST)
    return fail(GBPT_ERR_INVALID_ARG, "unknown queue policy");
  std::lock_guard<std::mutex> lock(s->mu);
  s->policy = policy;
  return GBPT_OK;
}

gbpt_status gbpt_server_set_graphs(gbpt_server* s, int32_t on) {
  if (!s) return fail(GBPT_ERR_INVALID_ARG, "server is NULL");
  std::lock_guard<std::mutex> lock(s->mu);
  s->graphs = on != 0;
  return GBPT_OK;
}

gbpt_status gbpt_server_destroy(gbpt_server* s) {
  delete s;
  return GBPT_OK;
}

gbpt_status gbpt_server_submit(gbpt_server* s, const gbpt_request* req, uint64_t* id) {
  if (!s || !req || !id) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (!req->scene) return fail(GBPT_ERR_INVALID_ARG, "request has no scene");
  if (req->width == 0 || req->height == 0 || (uint64_t)req->width * req->height > (1ull << 26))
    return fail(GBPT_ERR_INVALID_ARG, "image size must be 1..2^26 pixels");
  if (req->mode < GBPT_MODE_BDPT_SC || req->mode > GBPT_MODE_PT_SC)
    return fail(GBPT_ERR_INVALID_ARG, "unknown renderer mode");
  auto q = std::make_shared<Request>();
  q->q = *req;
  q->q.params = nullptr;
  if (req->params) {
    q->p = *req->params;
  } else {
    gbpt_params_default(&q->p);
  }
  gbpt_params dflt;
  gbpt_params_default(&dflt);
  q->tuned = q->p.walk_refill == 0 && q->p.tail_from == -1 && q->p.bands == 0 && q->p.walk_ctas == 0 &&
             q->p.tail_below == dflt.tail_below;
  q->knobs = Knobs{q->p.walk_refill, q->p.tail_from, q->p.bands, q->p.walk_ctas, q->p.tail_below};
  q->tSubmit = Clock::now();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return fail(GBPT_ERR_STATE, "server is stopping");
    q->id = s->nextId++;
    s->reqs[q->id] = q;
    s->queue.push_back(q);
  }
  s->cvWork.notify_one();
  *id = q->id;
  return GBPT_OK;
}

gbpt_status gbpt_server_wait(gbpt_server* s, uint64_t id, uint32_t timeout_ms, gbpt_request_status* out) {
  if (!s || !out) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(GBPT_ERR_INVALID_ARG, "unknown request id");
  std::shared_ptr<Request> q = it->second;
  s->cvDone.wait_for(lock, std::chrono::milliseconds(timeout_ms), [&] { return q->done; });
  std::memset(out, 0, sizeof(*out));
  out->id = id;
  out->done = q->done ? 1u : 0u;
  out->walk_refill = q->knobs.refill;
  out->tail_from = q->knobs.tail;
  if (!q->done) return fail(GBPT_ERR_TIMEOUT, "request still queued or running");
  out->status = q->status;
  out->queued_ms = ms_between(q->tSubmit, q->tStart);
  out->run_ms = ms_between(q->tStart, q->tEnd);
  out->latency_ms = ms_between(q->tSubmit, q->tEnd);
  out->paths = q->paths;
  if (q->status != GBPT_OK) set_error(q->err);
  return GBPT_OK;
}

gbpt_status gbpt_server_release(gbpt_server* s, uint64_t id) {
  if (!s) return fail(GBPT_ERR_INVALID_ARG, "server is NULL");
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(GBPT_ERR_INVALID_ARG, "unknown request id");
  if (!it->second->done) return fail(GBPT_ERR_STATE, "request still queued or running");
  s->reqs.erase(it);
  return GBPT_OK;
}

gbpt_status gbpt_server_tuned_params(gbpt_server* s, int32_t mode, uint32_t depth, uint32_t width, uint32_t height,
                                     gbpt_params* knobs, uint32_t* samples) {
  if (!s || !knobs || !samples) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  gbpt_params_default(knobs);
  Request probe;
  probe.q.width = width;
  probe.q.height = height;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->tuning.find(ClassKey{mode, depth, probe.size()});
  *samples = 0;
  if (it == s->tuning.end()) {
    const Knobs k = candidates(depth, probe.size(), knobs->tail_below)[0];
    knobs->walk_refill = k.refill;
    knobs->tail_from = k.tail;
    knobs->bands = k.bands;
    knobs->walk_ctas = k.ctas;
    knobs->tail_below = k.below;
    return GBPT_OK;
  }
  const Tuning& t = it->second;
  const Knobs& k = t.cand[gbpt_server::best(t)];
  knobs->walk_refill = k.refill;
  knobs->tail_from = k.tail;
  knobs->bands = k.bands;
  knobs->walk_ctas = k.ctas;
  knobs->tail_below = k.below;
  for (uint32_t n : t.trials) *samples += n;
  return GBPT_OK;
}

gbpt_status gbpt_server_tuned(gbpt_server* s, int32_t mode, uint32_t depth, uint32_t width, uint32_t height,
                              uint32_t* walk_refill, int32_t* tail_from, uint32_t* samples) {
  if (!s || !walk_refill || !tail_from || !samples) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  Request probe;
  probe.q.width = width;
  probe.q.height = height;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->tuning.find(ClassKey{mode, depth, probe.size()});
  if (it == s->tuning.end()) {
    *walk_refill = walk_refill_for(0, false);
    *tail_from = -1;
    *samples = 0;
    return GBPT_OK;
  }
  const Tuning& t = it->second;
  const size_t b = gbpt_server::best(t);
  *walk_refill = t.cand[b].refill;
  *tail_from = t.cand[b].tail;
  uint32_t n = 0;
  for (uint32_t k : t.trials) n += k;
  *samples = n;
  return GBPT_OK;
}
