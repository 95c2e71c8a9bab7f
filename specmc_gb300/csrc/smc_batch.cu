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
// Launch policy: the launcher starts a batch as soon as every handle that is
// stepping has a solve queued, or the oldest queued solve has waited `hold`
// microseconds, or the queued solves fill the GPU.  Batches do not overlap
// one another or any other cooperative kernel of the process (every
// cooperative launch is ordered on the GPU after the previous one, see
// CoopGuard): two partially resident grids whose CTAs wait for one another
// could otherwise never finish.  The launcher waits for a batch to finish
// before it starts the next; solves queued meanwhile go into the next one.
#include <algorithm>
#include <atomic>
#include <condition_variable>
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
  void stats(long long* l, long long* s, long long* c) {
    std::lock_guard<std::mutex> lk(mu_);
    if (l) *l = launches_;
    if (s) *s = solves_;
    if (c) *c = ctas_;
  }

 private:
  int capacity(size_t smem) {
    for (auto& p : caps_)
      if (p.first == smem) return p.second;
    const int c = refine_batch_capacity(smem, sms_);
    caps_.push_back({smem, c});
    return c;
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
    int c0 = 0;
    try {
      for (int j = 0; j < B.njobs; ++j) {
        SMC_CUDA(cudaStreamWaitEvent(s_, take[j]->ready, 0));
        B.job[j] = take[j]->job;
        B.job[j].cta0 = c0;
        B.job[j].G = take[j]->G;
        c0 += take[j]->G;
      }
      {
        CoopGuard guard(s_);           // ordered after every other cooperative grid
        refine_batch_launch(s_, B, smem);
      }
      const cudaError_t e = cudaStreamSynchronize(s_);
      if (e != cudaSuccess) throw CudaError(std::string("batched engine: ") + cudaGetErrorString(e));
      int err = 0;
      SMC_CUDA(cudaMemcpy(&err, d_err_, sizeof(int), cudaMemcpyDeviceToHost));
      if (err) {
        // a group barrier timed out: reset every barrier word of the batch
        // and the flag; the groups that timed out reported failed results
        for (int j = 0; j < B.njobs; ++j)
          SMC_CUDA(cudaMemsetAsync(B.job[j].bar, 0, 3 * sizeof(unsigned int), s_));
        SMC_CUDA(cudaMemsetAsync(d_err_, 0, sizeof(int), s_));
        SMC_CUDA(cudaStreamSynchronize(s_));
      }
      std::lock_guard<std::mutex> lk(mu_);
      ++launches_;
      solves_ += B.njobs;
      ctas_ += G;
    } catch (const std::exception&) {
      // nothing may be left waiting for a result that never comes
      std::vector<BatchReq*> pending;
      for (BatchReq* r : take)
        if (r->host->done != r->job.seq) pending.push_back(r);
      fail_all(pending, 2);
    }
  }

  int dev_;
  int sms_ = 0;
  cudaStream_t s_ = nullptr;
  int* d_err_ = nullptr;
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<BatchReq*> q_;
  int participants_ = 0;
  double hold_us_ = 50.0;
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
