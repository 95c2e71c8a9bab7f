// The batcher of the mixed form's refinement solves: one cooperative launch
// runs the Krylov solves of many model handles at once.
//
// Independent runs (an ensemble: uneven grids, viscosity models and
// iteration counts) each step on their own host thread and CUDA stream.  A
// handle in batched mode does not launch its persistent refinement engine
// itself: it records an event on its stream after the kernels that produce
// the solve's right-hand side and operators, queues the solve here, and
// waits for the solve's result block.  One launcher thread per device takes
// the queued solves -- as many as fit co-resident on the GPU -- and starts
// them in ONE cooperative launch of smc_refine_batch_kernel, each solve on
// its own range of CTAs with its own group barrier, so a solve that needs a
// few Arnoldi steps does not wait for one that needs hundreds.  Each solve's
// CTAs publish its results to host-mapped memory as soon as it ends, so its
// thread goes on with the rest of its step while the batch runs on.
//
// Refill: while a launch runs, the launcher publishes the solves queued since
// (once their inputs are complete) through a host-mapped feed; a slot whose
// solve has ended claims the next one and runs it on its own CTAs, so a
// launch does not idle down to its slowest solve.  A slot leaves when no
// solve arrives for `idle` microseconds, and none is claimed after `life`
// microseconds, so other cooperative kernels (ordered after the launch) are
// not held off for long; solves published but never claimed go back to the
// queue.
//
// Launch policy: the launcher starts a batch as soon as every handle that is
// stepping has a solve queued, or the oldest queued solve has waited `hold`
// microseconds, or the queued solves fill the GPU (or the cap set for it).  Batches do not overlap
// one another or any other cooperative kernel of the process (every
// cooperative launch is ordered on the GPU after the previous one, see
// CoopGuard): two partially resident grids whose CTAs wait for one another
// could otherwise never finish.  The launcher waits for a batch to finish
// before it starts the next; solves queued meanwhile go into the next one.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "smc_batch.cuh"

namespace smc {

namespace {

class Batcher {
 public:
  explicit Batcher(int dev) : dev_(dev) {
    SMC_CUDA(cudaSetDevice(dev_));
    SMC_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev_));
    SMC_CUDA(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
    SMC_CUDA(cudaMalloc(&d_err_, sizeof(int)));
    SMC_CUDA(cudaMemsetAsync(d_err_, 0, sizeof(int), s_));
    SMC_CUDA(cudaMalloc(&d_slot_bar_, 4 * ENGINE_BATCH_MAX * sizeof(unsigned int)));
    SMC_CUDA(cudaMemsetAsync(d_slot_bar_, 0, 4 * ENGINE_BATCH_MAX * sizeof(unsigned int), s_));
    SMC_CUDA(cudaMalloc(&d_claimed_, sizeof(int)));
    SMC_CUDA(cudaMalloc(&d_slot_ticket_, ENGINE_BATCH_MAX * sizeof(int)));
    SMC_CUDA(cudaHostAlloc((void**)&h_feed_, sizeof(BatchFeed), cudaHostAllocMapped));
    std::memset((void*)h_feed_, 0, sizeof(BatchFeed));
    SMC_CUDA(cudaHostGetDevicePointer((void**)&d_feed_, (void*)h_feed_, 0));
    SMC_CUDA(cudaStreamSynchronize(s_));
    th_ = std::thread([this] { loop(); });
  }

  void enter() {
    std::lock_guard<std::mutex> lk(mu_);
    ++participants_;
  }
  void leave() {
    std::lock_guard<std::mutex> lk(mu_);
    --participants_;
    cv_.notify_all();
  }
  void submit(BatchReq* r) {
    r->t = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(mu_);
    q_.push_back(r);
    cv_.notify_all();
  }
  void set_hold(double us) {
    std::lock_guard<std::mutex> lk(mu_);
    hold_us_ = std::max(0.0, us);
  }
  void set_refill(bool on, double idle_us, double life_us) {
    std::lock_guard<std::mutex> lk(mu_);
    refill_ = on;
    if (idle_us >= 0.0) idle_us_ = idle_us;
    if (life_us >= 0.0) life_us_ = life_us;
  }
  void set_cap(int ctas) {
    std::lock_guard<std::mutex> lk(mu_);
    cap_ctas_ = std::max(0, ctas);
  }
  void stats(long long* l, long long* s, long long* c) {
    std::lock_guard<std::mutex> lk(mu_);
    if (l) *l = launches_;
    if (s) *s = solves_;
    if (c) *c = ctas_;
  }
  long long refilled() {
    std::lock_guard<std::mutex> lk(mu_);
    return refilled_;
  }

 private:
  int capacity(size_t smem) {
    int c = -1;
    for (auto& p : caps_)
      if (p.first == smem) c = p.second;
    if (c < 0) {
      c = refine_batch_capacity(smem, sms_);
      caps_.push_back({smem, c});
    }
    // a cap leaves SM room for the ordinary kernels of the runs while a
    // refilling launch lives on
    return cap_ctas_ > 0 ? std::min(c, cap_ctas_) : c;
  }

  void fail_all(std::vector<BatchReq*>& take, int code) {
    for (BatchReq* r : take) {
      r->host->failed = code;
      std::atomic_thread_fence(std::memory_order_seq_cst);
      r->host->done = r->job.seq;
    }
  }

  void loop() {
    cudaSetDevice(dev_);
    std::unique_lock<std::mutex> lk(mu_);
    while (true) {
      cv_.wait(lk, [&] { return !q_.empty(); });
      // hold the batch open until every stepping handle has queued, the
      // queue fills the GPU, or the oldest solve has waited hold_us
      const auto deadline = q_.front()->t + std::chrono::nanoseconds((long long)(hold_us_ * 1e3));
      while ((int)q_.size() < participants_ && (int)q_.size() < ENGINE_BATCH_MAX) {
        int want = 0;
        size_t sm = 0;
        for (BatchReq* r : q_) { want += r->G; sm = std::max(sm, r->smem); }
        lk.unlock();
        const int cap = capacity(sm);
        lk.lock();
        if (want >= cap) break;
        if (cv_.wait_until(lk, deadline) == std::cv_status::timeout) break;
      }
      std::vector<BatchReq*> take;
      size_t smem = 0;
      int G = 0;
      while (!q_.empty() && (int)take.size() < ENGINE_BATCH_MAX) {
        BatchReq* r = q_.front();
        const size_t sm2 = std::max(smem, r->smem);
        lk.unlock();
        const int cap2 = capacity(sm2);
        lk.lock();
        if (cap2 < 1) {       // cannot be resident at all: report, do not launch
          q_.pop_front();
          std::vector<BatchReq*> one{r};
          fail_all(one, 3);
          continue;
        }
        if (G + std::min(r->G, cap2) > cap2) break;
        r->G = std::min(r->G, cap2);
        take.push_back(r);
        q_.pop_front();
        G += r->G;
        smem = sm2;
      }
      if (take.empty()) continue;
      lk.unlock();
      launch(take, smem, G);
      lk.lock();
    }
  }

  void launch(std::vector<BatchReq*>& take, size_t smem, int G) {
    RefineBatch B;
    B.njobs = (int)take.size();
    B.err = d_err_;
    B.slot_bar = d_slot_bar_;
    const bool refill = refill_;
    if (refill) {
      B.feed = d_feed_;
      B.claimed = d_claimed_;
      B.slot_ticket = d_slot_ticket_;
      B.idle_ns = (long long)(idle_us_ * 1e3);
      B.life_ns = (long long)(life_us_ * 1e3);
    }
    std::vector<BatchReq*> fed;          // fed[t]: the solve published as ticket t
    int c0 = 0;
    try {
      for (int j = 0; j < B.njobs; ++j) {
        SMC_CUDA(cudaStreamWaitEvent(s_, take[j]->ready, 0));
        B.job[j] = take[j]->job;
        B.job[j].cta0 = c0;
        B.job[j].G = take[j]->G;
        c0 += take[j]->G;
      }
      int gmin = c0;
      for (int j = 0; j < B.njobs; ++j) gmin = std::min(gmin, B.job[j].G);
      if (refill) {
        h_feed_->published = 0;
        SMC_CUDA(cudaMemsetAsync(d_claimed_, 0, sizeof(int), s_));
      }
      {
        CoopGuard guard(s_);           // ordered after every other cooperative grid
        refine_batch_launch(s_, B, smem);
      }
      // while the launch runs: publish the solves queued since, once their
      // inputs are complete, for the slots that free up
      while (refill) {
        const cudaError_t q = cudaStreamQuery(s_);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady)
          throw CudaError(std::string("batched engine: ") + cudaGetErrorString(q));
        std::unique_lock<std::mutex> lk(mu_);
        int pub = (int)fed.size();
        for (auto it = q_.begin(); it != q_.end() && pub < BATCH_FEED_CAP;) {
          BatchReq* r = *it;
          if (r->smem <= smem && cudaEventQuery(r->ready) == cudaSuccess) {
            h_feed_->ring[pub] = r->job;
            fed.push_back(r);
            ++pub;
            it = q_.erase(it);
          } else {
            ++it;
          }
        }
        if (pub != h_feed_->published) {
          std::atomic_thread_fence(std::memory_order_seq_cst);
          h_feed_->published = pub;
        }
        cv_.wait_for(lk, std::chrono::microseconds(20));
      }
      const cudaError_t e = cudaStreamSynchronize(s_);
      if (e != cudaSuccess) throw CudaError(std::string("batched engine: ") + cudaGetErrorString(e));
      int err = 0, claimed = 0;
      SMC_CUDA(cudaMemcpy(&err, d_err_, sizeof(int), cudaMemcpyDeviceToHost));
      if (refill) SMC_CUDA(cudaMemcpy(&claimed, d_claimed_, sizeof(int), cudaMemcpyDeviceToHost));
      if (err) {
        // a group barrier timed out: reset the slot words and the flag; the
        // groups that timed out reported failed results
        SMC_CUDA(cudaMemsetAsync(d_slot_bar_, 0, 4 * ENGINE_BATCH_MAX * sizeof(unsigned int), s_));
        SMC_CUDA(cudaMemsetAsync(d_err_, 0, sizeof(int), s_));
        SMC_CUDA(cudaStreamSynchronize(s_));
      }
      std::lock_guard<std::mutex> lk(mu_);
      // published solves no group claimed go back to the front of the queue
      for (int t = (int)fed.size() - 1; t >= claimed; --t) q_.push_front(fed[t]);
      ++launches_;
      solves_ += B.njobs + std::min(claimed, (int)fed.size());
      ctas_ += G;
      refilled_ += std::min(claimed, (int)fed.size());
    } catch (const std::exception&) {
      // nothing may be left waiting for a result that never comes
      std::vector<BatchReq*> pending;
      for (BatchReq* r : take)
        if (r->host->done != r->job.seq) pending.push_back(r);
      for (BatchReq* r : fed)
        if (r->host->done != r->job.seq) pending.push_back(r);
      fail_all(pending, 2);
    }
  }

  int dev_;
  int sms_ = 0;
  cudaStream_t s_ = nullptr;
  int* d_err_ = nullptr;
  unsigned int* d_slot_bar_ = nullptr;   // 4 words per slot (zero between launches)
  int* d_claimed_ = nullptr;
  int* d_slot_ticket_ = nullptr;
  BatchFeed* h_feed_ = nullptr;          // host-mapped
  BatchFeed* d_feed_ = nullptr;
  bool refill_ = true;
  double idle_us_ = 200.0, life_us_ = 20000.0;
  long long refilled_ = 0;
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<BatchReq*> q_;
  int participants_ = 0;
  double hold_us_ = 50.0;
  int cap_ctas_ = 0;
  long long launches_ = 0, solves_ = 0, ctas_ = 0;
  std::vector<std::pair<size_t, int>> caps_;
  std::thread th_;
};

// One batcher per device, created on first use and kept for the life of the
// process (its launcher thread waits on a condition variable when idle).
std::mutex g_batchers_mu;
Batcher* g_batchers[64] = {nullptr};

Batcher& batcher(int device) {
  if (device < 0 || device >= 64) throw std::runtime_error("batcher: device ordinal >= 64");
  std::lock_guard<std::mutex> lk(g_batchers_mu);
  if (!g_batchers[device]) g_batchers[device] = new Batcher(device);
  return *g_batchers[device];
}

}  // namespace

void batch_enter(int device) { batcher(device).enter(); }
void batch_leave(int device) { batcher(device).leave(); }
void batch_submit(int device, BatchReq* r) { batcher(device).submit(r); }
void batch_set_hold_us(int device, double us) { batcher(device).set_hold(us); }
void batch_set_refill(int device, int on, double idle_us, double life_us) {
  batcher(device).set_refill(on != 0, idle_us, life_us);
}
void batch_set_cap(int device, int ctas) { batcher(device).set_cap(ctas); }
void batch_stats(int device, long long* l, long long* s, long long* c) {
  batcher(device).stats(l, s, c);
}

void batch_wait(const BatchReq* r, double timeout_s) {
  const auto t0 = std::chrono::steady_clock::now();
  int spins = 0;
  while (r->host->done != r->job.seq) {
    if (++spins < 64) continue;
    std::this_thread::yield();
    if ((spins & 1023) == 0 &&
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > timeout_s)
      throw std::runtime_error("batched engine: no result after " + std::to_string(timeout_s) + " s");
  }
  std::atomic_thread_fence(std::memory_order_acquire);
}

}  // namespace smc
