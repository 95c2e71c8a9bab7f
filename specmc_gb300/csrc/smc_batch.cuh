// Batching of the mixed form's refinement solves across model handles
// (smc_batch.cu).
#pragma once
#include <chrono>

#include "smc_engine.cuh"

namespace smc {

// One solve handed to the device's batcher by the thread that owns its
// handle.  `ready` is recorded on the handle's stream after the work that
// produces the solve's inputs; `host` is the result block (host-mapped
// pinned memory; job.out is its device address).
struct BatchReq {
  RefineJob job;
  int G = 0;                  // CTAs wanted for this solve
  size_t smem = 0;            // its dynamic shared memory
  cudaEvent_t ready = nullptr;
  EngineJobResult* host = nullptr;
  std::chrono::steady_clock::time_point t;
};

// Handles in batched mode announce themselves while they step, so the
// batcher knows how many solves may still join the next launch.
void batch_enter(int device);
void batch_leave(int device);
// Queue one solve (returns at once); the caller then waits for
// host->done == job.seq (batch_wait).
void batch_submit(int device, BatchReq* r);
// Wait for the solve of `r` to finish (polling its result block); throws
// after `timeout_s` seconds.
void batch_wait(const BatchReq* r, double timeout_s);
// Batcher settings: how long the oldest queued solve may wait for others
// (microseconds) before a launch; refill on/off with the idle and life
// limits of a launch (microseconds; < 0 keeps the value); a cap on the CTAs
// of one launch (0: the co-resident maximum).
void batch_set_hold_us(int device, double us);
void batch_set_refill(int device, int on, double idle_us, double life_us);
void batch_set_cap(int device, int ctas);
// Statistics of the device's batcher: launches, solves, CTAs launched in all.
void batch_stats(int device, long long* launches, long long* solves, long long* ctas);

struct BatchScope {
  int device;
  bool on;
  BatchScope(int d, bool b) : device(d), on(b) { if (on) batch_enter(device); }
  ~BatchScope() { if (on) batch_leave(device); }
};

}  // namespace smc
