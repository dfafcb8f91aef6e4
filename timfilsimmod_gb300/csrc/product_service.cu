// product_service.cu -- the pair products of many swimmers in shared
// work-queue launches (the batch's and the request server's per-instance
// tile queue).
//
// Every swimmer of a batch or server runs its step on its own host thread
// and stream. When its solver is attached to a ProductService, each product
// (M_ss with M_bs, M_sb, the grand mobility, ...) is not launched on the
// swimmer's stream: the swimmer packs its source records there, marks them
// ready with an event and queues its job list. One waiting thread leads: it
// takes the pending requests of the same precision and source sets as the
// oldest (those that arrived while the previous launch was being issued), in
// arrival order, up to kQueueMaxJobs jobs, makes one of the service streams
// wait for each swimmer's records, copies the jobs (costliest units first)
// through a pinned slot to the device and issues one work-queue launch whose
// CTAs take the units of every swimmer's products from one counter. Each
// swimmer's stream then waits for the launch's completion event. Launches
// go round-robin over kStreams streams, so shared launches overlap one
// another as separate swimmers' launches would.
//
// A swimmer's jobs are the same descriptors its own launches use: the same
// chunking (a function of its sizes), its own partial buffers and arrival
// counters. So its result is the same, bit for bit, in a shared launch and
// alone, whatever else shares the launch and whatever launch variant runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <vector>

#include "tfs_kernels.h"
#include "tfs_solver.h"

namespace tfs {

struct ProductService {
  struct Req {
    tfs_solver *s;
    int kind, fp32, src, njobs;
    bool done;
    int rc;
  };
  static constexpr int kStreams = 4;  // shared launches in flight at once
  static constexpr int kSlots = 8;    // host staging of the job arrays (slot k on stream k % kStreams)
  struct Slot {
    QueueJob *jobs = nullptr;      // pinned host, kQueueMaxJobs
    QueueJob *dev_jobs = nullptr;  // device, kQueueMaxJobs
    cudaEvent_t copied = nullptr;
  };
  std::mutex m;
  std::condition_variable cv;
  std::deque<Req *> pending;
  bool busy = false;
  cudaStream_t stream[kStreams] = {};
  unsigned *counters = nullptr;  // [2 kStreams]: a pair per stream (its launches are serialised)
  Slot slot[kSlots];
  int next_slot = 0;
  long long launches = 0, products = 0;
  // Queues one launch of the products in batch (the leader, without the lock).
  int launch(std::vector<Req *> &batch) {
    const int k = next_slot;
    Slot &sl = slot[k];
    cudaStream_t stream = this->stream[k % kStreams];
    unsigned *cnt = counters + 2 * (k % kStreams);
    next_slot = (next_slot + 1) % kSlots;
    TFS_CUDA(cudaEventSynchronize(sl.copied), "product service: staging slot");
    int n = 0;
    for (Req *r : batch) {
      TFS_CUDA(cudaStreamWaitEvent(stream, r->s->pready_ev, 0), "product service: wait for inputs");
      for (int j = 0; j < r->njobs; ++j) sl.jobs[n++] = r->s->qjobs[r->kind][j];
    }
    // costliest units first: longer chunks, and 6-component targets before 3
    std::stable_sort(sl.jobs, sl.jobs + n, [](const QueueJob &a, const QueueJob &b) {
      return (long)a.chunk * (a.vd == 6 ? 2 : 1) > (long)b.chunk * (b.vd == 6 ? 2 : 1);
    });
    TFS_CUDA(cudaMemcpyAsync(sl.dev_jobs, sl.jobs, sizeof(QueueJob) * n, cudaMemcpyHostToDevice,
                             stream),
             "product service: jobs");
    TFS_CUDA(cudaEventRecord(sl.copied, stream), "product service: staging slot");
    cudaError_t e = launch_queue(batch.front()->fp32, 0, batch.front()->src, sl.dev_jobs, sl.jobs,
                                 n, cnt, stream);
    if (e != cudaSuccess) return cuda_fail(e, "product service: work-queue kernel");
    for (Req *r : batch)
      TFS_CUDA(cudaEventRecord(r->s->pdone_ev, stream), "product service: completion");
    return TFS_OK;
  }

  int run(tfs_solver *s, int kind, int fp32, int src) {
    Req r{s, kind, fp32, src, s->qjobs_n[kind], false, TFS_OK};
    if (r.njobs == 0) return TFS_OK;
    TFS_CUDA(cudaEventRecord(s->pready_ev, s->stream), "product service: inputs ready");
    std::unique_lock<std::mutex> g(m);
    pending.push_back(&r);
    cv.notify_all();
    while (!r.done) {
      if (busy) {
        cv.wait(g);
        continue;
      }
      busy = true;
      // the products waiting now go together; no launch waits for more
      std::vector<Req *> batch;
      int jobs = 0;
      const Req *head = pending.front();
      for (auto it = pending.begin(); it != pending.end();) {
        Req *q = *it;
        if (q->fp32 == head->fp32 && q->src == head->src && jobs + q->njobs <= kQueueMaxJobs) {
          jobs += q->njobs;
          batch.push_back(q);
          it = pending.erase(it);
        } else {
          ++it;
        }
      }
      g.unlock();
      const int lrc = launch(batch);
      g.lock();
      if (lrc == TFS_OK) {
        ++launches;
        products += (long long)batch.size();
      }
      for (Req *q : batch) {
        q->done = true;
        q->rc = lrc;
      }
      busy = false;
      cv.notify_all();
    }
    g.unlock();
    if (r.rc != TFS_OK) return r.rc;
    TFS_CUDA(cudaStreamWaitEvent(s->stream, s->pdone_ev, 0), "product service: wait for the product");
    return TFS_OK;
  }
};

ProductService *product_service_create() {
  ProductService *sv = new (std::nothrow) ProductService();
  if (sv == nullptr) return nullptr;
  bool ok = cudaMalloc(&sv->counters, 2 * ProductService::kStreams * sizeof(unsigned)) ==
                cudaSuccess &&
            cudaMemset(sv->counters, 0, 2 * ProductService::kStreams * sizeof(unsigned)) ==
                cudaSuccess;
  for (auto &st : sv->stream)
    ok = ok && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
  for (auto &sl : sv->slot)
    ok = ok &&
         cudaHostAlloc(&sl.jobs, sizeof(QueueJob) * kQueueMaxJobs, cudaHostAllocDefault) ==
             cudaSuccess &&
         cudaMalloc(&sl.dev_jobs, sizeof(QueueJob) * kQueueMaxJobs) == cudaSuccess &&
         cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    product_service_destroy(sv);
    return nullptr;
  }
  return sv;
}

void product_service_destroy(ProductService *sv) {
  if (sv == nullptr) return;
  for (auto st : sv->stream)
    if (st) cudaStreamSynchronize(st);
  for (auto &sl : sv->slot) {
    if (sl.jobs) cudaFreeHost(sl.jobs);
    if (sl.dev_jobs) cudaFree(sl.dev_jobs);
    if (sl.copied) cudaEventDestroy(sl.copied);
  }
  if (sv->counters) cudaFree(sv->counters);
  for (auto st : sv->stream)
    if (st) cudaStreamDestroy(st);
  delete sv;
}

int product_service_attach(ProductService *sv, tfs_solver *s) {
  if (sv == nullptr || s == nullptr) return fail(TFS_EINVAL, "null argument");
  for (cudaEvent_t *ev : {&s->pready_ev, &s->pdone_ev})
    if (*ev == nullptr && cudaEventCreateWithFlags(ev, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      return fail(TFS_ECUDA, "event creation failed");
    }
  return TFS_OK;
}

int product_service_run(ProductService *sv, tfs_solver *s, int kind, int fp32, int src) {
  return sv->run(s, kind, fp32, src);
}

void product_service_stats(ProductService *sv, long long *launches, long long *products) {
  std::lock_guard<std::mutex> g(sv->m);
  if (launches) *launches = sv->launches;
  if (products) *products = sv->products;
}

}  // namespace tfs
