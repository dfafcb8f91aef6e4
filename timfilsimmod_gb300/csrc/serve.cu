// serve.cu -- many independent swimmers on one GPU: a batch advanced one
// implicit step at a time, and a request server with admission by a device
// memory budget.
//
// Each swimmer is an instance (a tfs_solver with its tfs_stepper) on its own
// non-blocking stream. A pool of host worker threads runs the instances'
// step pipelines; the pipelines' kernels overlap on the GPU, so small
// swimmers that cannot fill the GPU alone fill it together. Work is handed to
// the workers largest first. The FP32C instances' inner GMRES solves run
// through a GMRES service (solve.cu): several solves share one cooperative
// launch of the persistent kernel, each on a fixed number of CTAs chosen from
// its own size; instances the kernel cannot take, and FP64 instances, use the
// kernel-sequence GMRES on their own streams. No instance's arithmetic
// depends on the others, so each result is the same as when the instance runs
// alone (a batch of one).
//
// The server keeps instances resident between requests (state, Krylov
// basis, Broyden matrices) in a pool keyed by the swimmer's geometry, admits
// a request when an idle instance of its geometry exists or a new one fits
// in the memory budget (evicting idle instances, least recently used
// first), and otherwise holds it until memory frees up. Requests are taken in
// arrival order.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "tfs_kernels.h"
#include "tfs_solver.h"

using tfs::fail;

namespace tfs {
tfs_solver *stepper_solver(tfs_stepper *st);
long stepper_segments(const tfs_stepper *st);
size_t stepper_bytes_estimate(int nfil, int nseg, int max_broyden_iter);
size_t solver_bytes_estimate(const tfs_config *cfg);
}  // namespace tfs

namespace {

// Persistent host threads that run job(i) for i in [0, n) and return when all
// are done.
class WorkerPool {
 public:
  explicit WorkerPool(int n, int device) : device_(device) {
    for (int i = 0; i < n; ++i) threads_.emplace_back([this] { loop(); });
  }
  ~WorkerPool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto &t : threads_) t.join();
  }
  void run(int n, std::function<void(int)> job) {
    std::unique_lock<std::mutex> g(m_);
    job_ = std::move(job);
    njobs_ = n;
    next_.store(0);
    busy_ = (int)threads_.size();
    ++gen_;
    cv_.notify_all();
    done_cv_.wait(g, [this] { return busy_ == 0; });
    job_ = nullptr;
  }

 private:
  void loop() {
    cudaSetDevice(device_);
    unsigned long long seen = 0;
    for (;;) {
      std::function<void(int)> job;
      int n;
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
        job = job_;
        n = njobs_;
      }
      for (int i = next_.fetch_add(1); i < n; i = next_.fetch_add(1)) job(i);
      std::lock_guard<std::mutex> g(m_);
      if (--busy_ == 0) done_cv_.notify_all();
    }
  }
  int device_;
  std::vector<std::thread> threads_;
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  std::function<void(int)> job_;
  int njobs_ = 0, busy_ = 0;
  unsigned long long gen_ = 0;
  bool stop_ = false;
  std::atomic<int> next_{0};
};

}  // namespace

struct tfs_batch {
  std::unique_ptr<WorkerPool> pool;
  std::vector<tfs_stepper *> inst;
  std::vector<char> shared;  // the instance's inner solves can go through the service
  std::vector<int> shared_ctas;  // CTAs of its solve in a shared launch
  tfs::GmresService *service = nullptr;
  int share_max_ctas = -1;  // -1: every solve the persistent kernel can take
  tfs::ProductService *pservice = nullptr;  // shared work-queue launches of the products
  bool share_products = true;
  ~tfs_batch() {
    tfs::service_destroy(service);
    tfs::product_service_destroy(pservice);
  }
};

extern "C" {

int tfs_batch_create(int num_workers, tfs_batch **out) {
  if (out == nullptr) return fail(TFS_EINVAL, "null output");
  *out = nullptr;
  if (num_workers < 1 || num_workers > 256) return fail(TFS_EINVAL, "num_workers must be in [1, 256]");
  int dev = 0;
  TFS_CUDA(cudaGetDevice(&dev), "device");
  tfs_batch *b = new (std::nothrow) tfs_batch();
  if (b == nullptr) return fail(TFS_ENOMEM, "host allocation");
  b->pool.reset(new WorkerPool(num_workers, dev));
  *out = b;
  return TFS_OK;
}

int tfs_batch_destroy(tfs_batch *b) {
  delete b;
  return TFS_OK;
}

// FP32C swimmers whose inner solve the persistent kernel can run share
// cooperative launches during tfs_batch_step (the service is attached to the
// solver only for the step); the others, and FP32C swimmers the kernel cannot
// run, solve alone with the kernel sequence.
int tfs_batch_add(tfs_batch *b, tfs_stepper *st, int *index) {
  if (b == nullptr || st == nullptr) return fail(TFS_EINVAL, "null handle");
  tfs_solver *s = tfs::stepper_solver(st);
  char shared = 0;
  if (s->cfg.precision == TFS_FP32C) {
    if (b->service == nullptr && (b->service = tfs::service_create()) == nullptr)
      return fail(TFS_ECUDA, "GMRES service creation failed");
    int rc = tfs::service_attach(b->service, s);
    s->service = nullptr;
    if (rc == TFS_OK) shared = 1;
    else if (rc != TFS_ESTATE) return rc;
    if ((rc = tfs_set_persistent_gmres(s, 0)) != TFS_OK) return rc;
  }
  if (b->pservice == nullptr && (b->pservice = tfs::product_service_create()) == nullptr)
    return fail(TFS_ECUDA, "product service creation failed");
  int prc = tfs::product_service_attach(b->pservice, s);
  if (prc != TFS_OK) return prc;
  b->inst.push_back(st);
  b->shared.push_back(shared);
  b->shared_ctas.push_back(shared ? s->pg_group.P : 0);
  if (index) *index = (int)b->inst.size() - 1;
  return TFS_OK;
}

int tfs_batch_size(tfs_batch *b, int *n) {
  if (b == nullptr || n == nullptr) return fail(TFS_EINVAL, "null argument");
  *n = (int)b->inst.size();
  return TFS_OK;
}

int tfs_batch_share_inner_solves(tfs_batch *b, int max_ctas) {
  if (b == nullptr) return fail(TFS_EINVAL, "null batch");
  b->share_max_ctas = max_ctas < 0 ? -1 : max_ctas;
  return TFS_OK;
}

int tfs_batch_share_products(tfs_batch *b, int enable) {
  if (b == nullptr) return fail(TFS_EINVAL, "null batch");
  b->share_products = enable != 0;
  return TFS_OK;
}

int tfs_batch_shared_products(tfs_batch *b, long long *launches, long long *products) {
  if (b == nullptr) return fail(TFS_EINVAL, "null batch");
  if (launches) *launches = 0;
  if (products) *products = 0;
  if (b->pservice) tfs::product_service_stats(b->pservice, launches, products);
  return TFS_OK;
}

int tfs_batch_shared_solves(tfs_batch *b, long long *launches, long long *solves) {
  if (b == nullptr) return fail(TFS_EINVAL, "null batch");
  if (launches) *launches = 0;
  if (solves) *solves = 0;
  if (b->service) tfs::service_stats(b->service, launches, solves);
  return TFS_OK;
}

int tfs_batch_step(tfs_batch *b, int nt, int *broyden_iters, int *gmres_iters, int *status) {
  if (b == nullptr) return fail(TFS_EINVAL, "null batch");
  const int n = (int)b->inst.size();
  std::vector<int> order(n), bi(n, 0), gi(n, 0), rc(n, TFS_OK);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return tfs::stepper_segments(b->inst[x]) > tfs::stepper_segments(b->inst[y]);
  });
  const int cap = b->share_max_ctas >= 0 ? b->share_max_ctas : tfs::num_sms();
  for (int i = 0; i < n; ++i) {
    if (b->shared[i] && b->shared_ctas[i] <= cap)
      tfs::stepper_solver(b->inst[i])->service = b->service;
    if (b->share_products) tfs::stepper_solver(b->inst[i])->product_service = b->pservice;
  }
  b->pool->run(n, [&](int k) {
    const int i = order[k];
    rc[i] = tfs_stepper_step(b->inst[i], nt, &bi[i], &gi[i]);
  });
  for (int i = 0; i < n; ++i) {
    tfs::stepper_solver(b->inst[i])->service = nullptr;
    tfs::stepper_solver(b->inst[i])->product_service = nullptr;
  }
  int first = TFS_OK;
  for (int i = 0; i < n; ++i) {
    if (broyden_iters) broyden_iters[i] = bi[i];
    if (gmres_iters) gmres_iters[i] = gi[i];
    if (status) status[i] = rc[i];
    if (first == TFS_OK && rc[i] != TFS_OK) first = rc[i];
  }
  if (first != TFS_OK) return fail(first, "%d of %d swimmers did not complete the step",
                                   (int)std::count_if(rc.begin(), rc.end(), [](int r) { return r != TFS_OK; }), n);
  return TFS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// request server
// ---------------------------------------------------------------------------

namespace {

using Clock = std::chrono::steady_clock;

struct Instance {
  unsigned long long key = 0;
  int nfil = 0, nseg = 0, nblob = 0;
  tfs_solver *s = nullptr;
  tfs_stepper *st = nullptr;
  size_t bytes = 0;
  bool busy = false;
  Clock::time_point last_used{};
};

struct Request {
  long long ticket = 0;
  tfs_request r{};
  unsigned long long key = 0;
  size_t bytes = 0;
  Clock::time_point arrival{}, done{};
  int status = 1;  // 1 = pending
  int broyden = 0, gmres = 0;
  std::string message;  // the failing call's message
};

unsigned long long fnv(unsigned long long h, const void *p, size_t n) {
  const unsigned char *c = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= c[i];
    h *= 1099511628211ULL;
  }
  return h;
}

unsigned long long geometry_key(const tfs_request &r) {
  unsigned long long h = 1469598103934665603ULL;
  const int sz[3] = {r.nfil, r.nseg, r.nblob};
  h = fnv(h, sz, sizeof sz);
  h = fnv(h, r.blob_refs, sizeof(double) * 3 * (size_t)r.nblob);
  h = fnv(h, r.fil_refs, sizeof(double) * 3 * (size_t)r.nfil);
  h = fnv(h, r.fil_dirs, sizeof(double) * 3 * (size_t)r.nfil);
  h = fnv(h, &r.body_radius, sizeof r.body_radius);
  return h;
}

void destroy_instance(Instance *in) {
  if (in->st) tfs_stepper_destroy(in->st);
  if (in->s) tfs_solver_destroy(in->s);
  delete in;
}

}  // namespace

struct tfs_server {
  tfs_server_config cfg{};
  int device = 0;
  std::mutex m;
  std::condition_variable cv;       // workers: new request or freed memory
  std::condition_variable done_cv;  // waiters: a request finished
  std::deque<Request *> queue;
  std::map<long long, std::unique_ptr<Request>> requests;
  std::vector<Instance *> pool;
  size_t bytes_in_use = 0;
  long long next_ticket = 1;
  long long inflight = 0;
  long long created = 0, evicted = 0, reused = 0, bypassed = 0;
  bool stop = false;
  std::vector<std::thread> workers;
  tfs::GmresService *service = nullptr;  // shared inner solves of FP32C instances
  tfs::ProductService *pservice = nullptr;  // shared work-queue launches of the products
  Clock::time_point t0 = Clock::now();

  void worker();
  bool can_admit(const Request *q) const;
  std::deque<Request *>::iterator pick();
  Instance *acquire(const Request *q, std::vector<Instance *> &victims, bool *fresh);
  int build(Instance *in, const tfs_request &r);
};

int tfs_server::build(Instance *in, const tfs_request &r) {
  tfs_config c;
  int rc = tfs_config_default(&c, 1, r.nfil, r.nseg, r.nblob);
  if (rc != TFS_OK) return rc;
  c.precision = cfg.precision;
  if ((rc = tfs_solver_create(&c, &in->s)) != TFS_OK) return rc;
  if ((rc = tfs_set_linear_solver(in->s, cfg.linear_tol, std::min(350, 3 * r.nblob + 6))) != TFS_OK)
    return rc;
  if (cfg.precision == TFS_FP32C) {
    rc = tfs::service_attach(service, in->s);
    if (rc != TFS_OK && rc != TFS_ESTATE) return rc;
    if ((rc = tfs_set_persistent_gmres(in->s, 0)) != TFS_OK) return rc;
  }
  if ((rc = tfs::product_service_attach(pservice, in->s)) != TFS_OK) return rc;
  in->s->product_service = pservice;
  if ((rc = tfs_set_blob_references(in->s, r.blob_refs)) != TFS_OK) return rc;
  tfs_step_config sc = cfg.step;
  sc.nfil = r.nfil;
  sc.nseg = r.nseg;
  if (r.body_radius > 0) sc.body_radius = r.body_radius;
  if ((rc = tfs_set_body_pose(in->s, sc.body_x, sc.body_q)) != TFS_OK) return rc;
  if ((rc = tfs_make_body_reference_matrices(in->s)) != TFS_OK) return rc;
  return tfs_stepper_create(in->s, &sc, r.fil_refs, r.fil_dirs, &in->st);
}

// With the lock held. can_admit: an idle instance of q's geometry exists, or
// a new one fits in the budget once idle instances are evicted.
bool tfs_server::can_admit(const Request *q) const {
  size_t idle = 0;
  for (const Instance *in : pool) {
    if (in->busy) continue;
    if (in->key == q->key) return true;
    idle += in->bytes;
  }
  return bytes_in_use - idle + q->bytes <= cfg.hbm_budget_bytes;
}

// With the lock held: the request to admit next, or queue.end(). The oldest
// request goes first when it can be admitted; while it waits for device
// memory held by running requests, a later one that fits now is admitted
// past it -- unless the oldest has waited max_bypass_ms or more, in which
// case nothing passes it, so that memory frees up for it (no starvation).
std::deque<Request *>::iterator tfs_server::pick() {
  if (queue.empty()) return queue.end();
  if (can_admit(queue.front())) return queue.begin();
  const double waited =
      std::chrono::duration<double, std::milli>(Clock::now() - queue.front()->arrival).count();
  if (waited >= cfg.max_bypass_ms) return queue.end();
  for (auto it = queue.begin() + 1; it != queue.end(); ++it)
    if (can_admit(*it)) return it;
  return queue.end();
}

// With the lock held, after can_admit(q): the idle instance of q's geometry,
// or a new (unbuilt) instance with its bytes accounted; idle instances
// evicted to make room (least recently used first) go to victims, to be
// destroyed without the lock.
Instance *tfs_server::acquire(const Request *q, std::vector<Instance *> &victims, bool *fresh) {
  for (Instance *in : pool)
    if (!in->busy && in->key == q->key) {
      in->busy = true;
      *fresh = false;
      ++reused;
      return in;
    }
  while (bytes_in_use + q->bytes > cfg.hbm_budget_bytes) {
    Instance *lru = nullptr;
    for (Instance *in : pool)
      if (!in->busy && (lru == nullptr || in->last_used < lru->last_used)) lru = in;
    if (lru == nullptr) break;  // cannot happen after can_admit
    pool.erase(std::find(pool.begin(), pool.end(), lru));
    bytes_in_use -= lru->bytes;
    ++evicted;
    victims.push_back(lru);
  }
  Instance *in = new Instance();
  in->key = q->key;
  in->nfil = q->r.nfil;
  in->nseg = q->r.nseg;
  in->nblob = q->r.nblob;
  in->bytes = q->bytes;
  in->busy = true;
  bytes_in_use += q->bytes;
  pool.push_back(in);
  *fresh = true;
  ++created;
  return in;
}

void tfs_server::worker() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> g(m);
  for (;;) {
    // a request held back only by the age bound needs a wake-up when the
    // bound runs out, so the wait is also bounded in time
    std::deque<Request *>::iterator it;
    for (;;) {
      if (stop) return;
      it = pick();
      if (it != queue.end()) break;
      cv.wait_for(g, std::chrono::milliseconds(20));
    }
    Request *q = *it;
    if (it != queue.begin()) ++bypassed;
    queue.erase(it);
    std::vector<Instance *> victims;
    bool fresh = false;
    Instance *in = acquire(q, victims, &fresh);
    g.unlock();
    for (Instance *v : victims) destroy_instance(v);
    int rc = TFS_OK;
    if (fresh) rc = build(in, q->r);
    if (rc == TFS_OK) rc = tfs_stepper_reset(in->st, q->r.seg_rotation);
    int bsum = 0, gsum = 0;
    for (int nt = 0; rc == TFS_OK && nt < q->r.num_steps; ++nt) {
      int b = 0, gm = 0;
      rc = tfs_stepper_step(in->st, nt, &b, &gm);
      bsum += b;
      gsum += gm;
    }
    // Broyden's method at its iteration cap ends the run, as the reference
    // stops there (cilia_sim_main.cu:542-557); the state so far is returned
    const bool unconverged = rc == TFS_ENOTCONV;
    if (rc == TFS_OK || unconverged) {
      const int rs = tfs_stepper_state(in->st, q->r.x_out, q->r.q_out, nullptr, nullptr, nullptr,
                                       nullptr, q->r.body_out,
                                       q->r.body_out ? q->r.body_out + 3 : nullptr, nullptr);
      if (rs != TFS_OK) rc = rs;
    }
    const bool drop = rc != TFS_OK && !(unconverged && rc == TFS_ENOTCONV);  // broken: not reused
    const std::string fail_msg = rc != TFS_OK ? std::string(tfs_last_error()) : std::string();
    if (drop) {
      g.lock();
      pool.erase(std::find(pool.begin(), pool.end(), in));
      bytes_in_use -= in->bytes;
      g.unlock();
      destroy_instance(in);
    }
    g.lock();
    q->message = fail_msg;
    if (!drop) {
      in->busy = false;
      in->last_used = Clock::now();
    }
    q->status = rc;
    q->broyden = bsum;
    q->gmres = gsum;
    q->done = Clock::now();
    --inflight;
    done_cv.notify_all();
    cv.notify_all();
  }
}

extern "C" {

int tfs_server_config_default(tfs_server_config *cfg) {
  if (cfg == nullptr) return fail(TFS_EINVAL, "null config");
  std::memset(cfg, 0, sizeof *cfg);
  cfg->num_workers = 16;
  cfg->hbm_budget_bytes = (size_t)160 << 30;
  cfg->precision = TFS_FP32C;
  cfg->linear_tol = 1e-8;
  cfg->max_bypass_ms = 1000.0;
  return tfs_step_config_default(&cfg->step, 1, 20);
}

int tfs_server_create(const tfs_server_config *cfg, tfs_server **out) {
  if (cfg == nullptr || out == nullptr) return fail(TFS_EINVAL, "null argument");
  *out = nullptr;
  if (cfg->num_workers < 1 || cfg->num_workers > 256) return fail(TFS_EINVAL, "num_workers must be in [1, 256]");
  if (cfg->precision != TFS_FP64 && cfg->precision != TFS_FP32C) return fail(TFS_EINVAL, "bad precision");
  if (!(cfg->linear_tol > 0) || cfg->hbm_budget_bytes == 0) return fail(TFS_EINVAL, "linear_tol and budget must be > 0");
  if (!(cfg->max_bypass_ms >= 0)) return fail(TFS_EINVAL, "max_bypass_ms must be >= 0");
  tfs_server *sv = new (std::nothrow) tfs_server();
  if (sv == nullptr) return fail(TFS_ENOMEM, "host allocation");
  sv->cfg = *cfg;
  cudaError_t e = cudaGetDevice(&sv->device);
  if (e != cudaSuccess) {
    delete sv;
    return tfs::cuda_fail(e, "device");
  }
  if (cfg->precision == TFS_FP32C && (sv->service = tfs::service_create()) == nullptr) {
    delete sv;
    return fail(TFS_ECUDA, "GMRES service creation failed");
  }
  if ((sv->pservice = tfs::product_service_create()) == nullptr) {
    tfs::service_destroy(sv->service);
    delete sv;
    return fail(TFS_ECUDA, "product service creation failed");
  }
  for (int i = 0; i < cfg->num_workers; ++i) sv->workers.emplace_back([sv] { sv->worker(); });
  *out = sv;
  return TFS_OK;
}

static bool malformed(const tfs_request *r) {
  return r->nfil < 1 || r->nseg < 3 || r->nblob < 1 || r->num_steps < 0 ||
         r->blob_refs == nullptr || r->fil_refs == nullptr || r->fil_dirs == nullptr;
}

static size_t request_bytes(const tfs_server *sv, const tfs_request *r) {
  tfs_config c;
  tfs_config_default(&c, 1, r->nfil, r->nseg, r->nblob);
  return tfs::solver_bytes_estimate(&c) +
         tfs::stepper_bytes_estimate(r->nfil, r->nseg, sv->cfg.step.max_broyden_iter);
}

int tfs_server_request_bytes(const tfs_server *sv, const tfs_request *r, size_t *bytes) {
  if (sv == nullptr || r == nullptr || bytes == nullptr) return fail(TFS_EINVAL, "null argument");
  if (malformed(r)) return fail(TFS_EINVAL, "malformed request");
  *bytes = request_bytes(sv, r);
  return TFS_OK;
}

int tfs_server_submit(tfs_server *sv, const tfs_request *r, long long *ticket) {
  if (sv == nullptr || r == nullptr || ticket == nullptr) return fail(TFS_EINVAL, "null argument");
  if (malformed(r)) return fail(TFS_EINVAL, "malformed request");
  std::unique_ptr<Request> q(new (std::nothrow) Request());
  if (!q) return fail(TFS_ENOMEM, "host allocation");
  q->r = *r;
  q->key = geometry_key(*r);
  q->bytes = request_bytes(sv, r);
  if (q->bytes > sv->cfg.hbm_budget_bytes)
    return fail(TFS_ENOMEM, "a swimmer of %d x %d segments and %d blobs needs ~%zu bytes, over the budget",
                r->nfil, r->nseg, r->nblob, q->bytes);
  std::lock_guard<std::mutex> g(sv->m);
  q->ticket = sv->next_ticket++;
  q->arrival = Clock::now();
  *ticket = q->ticket;
  sv->queue.push_back(q.get());
  sv->requests[q->ticket] = std::move(q);
  ++sv->inflight;
  sv->cv.notify_one();
  return TFS_OK;
}

int tfs_server_poll(tfs_server *sv, long long ticket, int wait, int *status, double *latency_ms,
                    int *broyden_iters, int *gmres_iters) {
  if (sv == nullptr || status == nullptr) return fail(TFS_EINVAL, "null argument");
  std::unique_lock<std::mutex> g(sv->m);
  auto it = sv->requests.find(ticket);
  if (it == sv->requests.end()) return fail(TFS_EINVAL, "unknown ticket %lld", ticket);
  Request *q = it->second.get();
  if (wait) sv->done_cv.wait(g, [&] { return q->status != 1; });
  *status = q->status;
  if (q->status == 1) return TFS_OK;
  if (q->status != TFS_OK)  // the request's message becomes this thread's last error
    fail(q->status, "request %lld: %s", ticket, q->message.c_str());
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(q->done - q->arrival).count();
  if (broyden_iters) *broyden_iters = q->broyden;
  if (gmres_iters) *gmres_iters = q->gmres;
  sv->requests.erase(it);
  return TFS_OK;
}

int tfs_server_drain(tfs_server *sv) {
  if (sv == nullptr) return fail(TFS_EINVAL, "null server");
  std::unique_lock<std::mutex> g(sv->m);
  sv->done_cv.wait(g, [&] { return sv->inflight == 0; });
  return TFS_OK;
}

int tfs_server_stats(tfs_server *sv, tfs_server_counters *out) {
  if (sv == nullptr || out == nullptr) return fail(TFS_EINVAL, "null argument");
  std::lock_guard<std::mutex> g(sv->m);
  out->resident_instances = (long long)sv->pool.size();
  out->bytes_in_use = sv->bytes_in_use;
  out->bypassed = sv->bypassed;
  out->created = sv->created;
  out->reused = sv->reused;
  out->evicted = sv->evicted;
  out->queued = (long long)sv->queue.size();
  out->inflight = sv->inflight;
  return TFS_OK;
}

int tfs_server_shared_solves(tfs_server *sv, long long *launches, long long *solves) {
  if (sv == nullptr) return fail(TFS_EINVAL, "null server");
  if (launches) *launches = 0;
  if (solves) *solves = 0;
  if (sv->service) tfs::service_stats(sv->service, launches, solves);
  return TFS_OK;
}

int tfs_server_shared_products(tfs_server *sv, long long *launches, long long *products) {
  if (sv == nullptr) return fail(TFS_EINVAL, "null server");
  if (launches) *launches = 0;
  if (products) *products = 0;
  if (sv->pservice) tfs::product_service_stats(sv->pservice, launches, products);
  return TFS_OK;
}

int tfs_server_destroy(tfs_server *sv) {
  if (sv == nullptr) return TFS_OK;
  {
    std::unique_lock<std::mutex> g(sv->m);
    sv->done_cv.wait(g, [&] { return sv->inflight == 0; });
    sv->stop = true;
  }
  sv->cv.notify_all();
  for (auto &t : sv->workers) t.join();
  for (Instance *in : sv->pool) destroy_instance(in);
  tfs::service_destroy(sv->service);
  tfs::product_service_destroy(sv->pservice);
  delete sv;
  return TFS_OK;
}

}  // extern "C"
