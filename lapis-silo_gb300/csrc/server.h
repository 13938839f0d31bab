// Serving loop: continuous batching of filter queries on one device partition.
//
// Requests (an expression and an action: Aggregated count, Mutations rows, Details ids) are
// submitted from any thread. A loop thread admits waiting requests into micro-batches as long as
// the in-flight queries fit the slot limit and their device buffers fit the memory budget, plans
// each micro-batch (with the learned planner when it is enabled) and launches it on one of several
// streams, so micro-batches admitted while others run overlap on the device. Completion is polled
// with events: the first phase ends with the counts, Details ids and the size of the Mutations
// rows on the host, the second (only with Mutations) with the rows. The partition and every
// in-flight query's buffers stay on the device; the host keeps only the results it returns.
// Results equal those of the same query run alone (nothing in the arithmetic depends on the batch).
#pragma once

#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

namespace rhygpu {

struct ServeRequest {
   uint64_t id = 0;
   std::string expr;
   int action = 0;  // 0 count, 1 mutations, 2 details
   int column = 0;
   double min_proportion = 0.05;
   uint32_t k = 1000;
   size_t bytes = 0;  // device bytes while in flight
   // results
   uint64_t count = 0;
   std::vector<DevMutationRow> rows;
   std::vector<uint32_t> ids;
   std::string error;
   double t_submit = 0, t_done = 0;  // seconds, steady clock
   bool done = false;
   bool cancelled = false;  // cancel() was called before the result was ready
};

struct ServerConfig {
   uint32_t max_batch = 512;      // queries per micro-batch
   uint32_t streams = 3;          // micro-batches in flight
   uint32_t max_inflight = 4096;  // admitted, unfinished queries
   uint64_t memory_budget = 0;    // device bytes of in-flight micro-batches; 0 = a quarter of free memory
   double max_wait_ms = 0.25;     // a partial micro-batch launches once its oldest request waited this long
   // Plain serving: every request runs alone through the single-query path (rhy_count /
   // rhy_mutations / rhy_eval), one after the other in arrival order; no batching.
   bool plain = false;
};

struct ServerStats {
   uint64_t submitted = 0, completed = 0, rejected = 0, batches = 0, cancelled = 0;
   double p50_ms = 0, p99_ms = 0, mean_batch = 0, qps = 0;
   uint64_t peak_bytes = 0, budget_bytes = 0;
   uint32_t peak_inflight = 0;
};

class Server {
  public:
   Server(Engine& engine, const ServerConfig& cfg);
   ~Server();
   Server(const Server&) = delete;
   Server& operator=(const Server&) = delete;

   // Validates the expression (user errors throw here) and queues the request; returns its id.
   uint64_t submit(const std::string& expr, int action, int column, double min_proportion, uint32_t k);
   // Blocks until the request is done (timeout_ms < 0: no limit); nullptr on timeout.
   std::shared_ptr<ServeRequest> wait(uint64_t id, double timeout_ms);
   void release(uint64_t id);
   // Cancels a request that is not done: a queued one is dropped before it is admitted, one already
   // on the device finishes there but its result is discarded. Either way its result reports
   // "request cancelled". Returns false when the request was already done.
   bool cancel(uint64_t id);
   ServerStats stats();
   void stop();
   // Open-loop replay of a request trace: every request is submitted at its arrival time (seconds
   // from the start) by a native thread, then all are awaited and released. Returns each request's
   // latency (ms, NaN if it failed) and the wall time from the first arrival to the last result.
   std::vector<double> replay(const std::vector<ServeRequest>& reqs, const std::vector<double>& arrival_s, double* wall_s);

  private:
   struct Slot {
      BatchState b;
      cudaStream_t stream = nullptr;
      cudaEvent_t event = nullptr;
      int phase = 0;  // 0 idle, 1 counts / ids / row sizes in flight, 2 rows in flight
      std::vector<std::shared_ptr<ServeRequest>> reqs;
      size_t bytes = 0;
      DevMutationRow* h_rows = nullptr;  // pinned
      size_t h_rows_cap = 0;
   };
   void loop();
   void launch(Slot& slot, std::vector<std::shared_ptr<ServeRequest>>&& reqs);
   void advance(Slot& slot);
   void finish(Slot& slot);
   void fail(Slot& slot, const std::string& what);
   void run_plain(ServeRequest& r, cudaStream_t stream);
   size_t request_bytes(const ServeRequest& r) const;

   Engine& engine_;
   ServerConfig cfg_;
   std::vector<Slot> slots_;
   std::thread thread_;
   std::mutex mu_;
   std::condition_variable cv_work_, cv_done_;
   std::deque<std::shared_ptr<ServeRequest>> pending_;
   std::map<uint64_t, std::shared_ptr<ServeRequest>> all_;
   uint64_t next_id_ = 1;
   bool stop_ = false;
   size_t inflight_bytes_ = 0;
   uint32_t inflight_ = 0;
   // statistics
   ServerStats st_;
   std::vector<double> latencies_ms_;
   double t_first_ = -1, t_last_ = 0;
   uint64_t batched_queries_ = 0;
};

}  // namespace rhygpu
