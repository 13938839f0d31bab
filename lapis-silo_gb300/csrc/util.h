// Small host utilities shared by the ingestion and planning code.
#pragma once

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <exception>
#include <functional>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace rhygpu {

// Runs fn(i) for i in [0, n) on up to `threads` worker threads (0 = all hardware threads).
// Exceptions thrown by fn are rethrown on the calling thread.
template <typename F>
void parallel_for(uint32_t n, uint32_t threads, F&& fn) {
   if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
   threads = std::min(threads, std::max(1u, n));
   std::atomic<uint32_t> next{0};
   std::exception_ptr error;
   std::atomic<bool> failed{false};
   auto body = [&]() {
      for (uint32_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
         if (failed.load()) return;
         try {
            fn(i);
         } catch (...) {
            if (!failed.exchange(true)) error = std::current_exception();
            return;
         }
      }
   };
   if (threads <= 1) {
      body();
   } else {
      std::vector<std::thread> pool;
      pool.reserve(threads);
      for (uint32_t t = 0; t < threads; ++t) pool.emplace_back(body);
      for (auto& th : pool) th.join();
   }
   if (error) std::rethrow_exception(error);
}

// Persistent workers for the per-call parallel loops of planning, where starting threads on every
// call would cost as much as the work. run(n, fn) calls fn(i) for i in [0, n) on the workers and
// the calling thread and returns when all calls are done; the first exception is rethrown on the
// caller. One run at a time (callers serialise, as the engine does under its mutex); a run from
// inside fn executes inline.
class WorkerPool {
  public:
   explicit WorkerPool(uint32_t threads = 0) {
      if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
      for (uint32_t t = 1; t < threads; ++t) workers_.emplace_back([this] { loop(); });
   }
   ~WorkerPool() {
      {
         std::lock_guard<std::mutex> lk(m_);
         stop_ = true;
      }
      cv_.notify_all();
      for (auto& w : workers_) w.join();
   }
   WorkerPool(const WorkerPool&) = delete;
   WorkerPool& operator=(const WorkerPool&) = delete;
   uint32_t size() const { return static_cast<uint32_t>(workers_.size()) + 1; }

   template <typename F>
   void run(uint32_t n, F&& fn) {
      if (n == 0) return;
      if (inside_ || workers_.empty() || n == 1) {
         for (uint32_t i = 0; i < n; ++i) fn(i);
         return;
      }
      std::atomic<uint32_t> next{0};
      std::atomic<bool> failed{false};
      std::exception_ptr error;
      std::mutex err_m;
      std::function<void()> body = [&] {
         for (uint32_t i = next.fetch_add(1); i < n && !failed.load(std::memory_order_relaxed); i = next.fetch_add(1)) {
            try {
               fn(i);
            } catch (...) {
               std::lock_guard<std::mutex> lk(err_m);
               if (!failed.exchange(true)) error = std::current_exception();
            }
         }
      };
      {
         std::lock_guard<std::mutex> lk(m_);
         job_ = &body;
         busy_ = static_cast<uint32_t>(workers_.size());
         ++gen_;
      }
      cv_.notify_all();
      inside_ = true;
      body();
      inside_ = false;
      {
         std::unique_lock<std::mutex> lk(m_);
         done_.wait(lk, [&] { return busy_ == 0; });
         job_ = nullptr;
      }
      if (error) std::rethrow_exception(error);
   }

  private:
   void loop() {
      uint64_t seen = 0;
      for (;;) {
         std::function<void()>* job;
         {
            std::unique_lock<std::mutex> lk(m_);
            cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
            if (stop_) return;
            seen = gen_;
            job = job_;
         }
         inside_ = true;
         (*job)();
         inside_ = false;
         std::lock_guard<std::mutex> lk(m_);
         if (--busy_ == 0) done_.notify_one();
      }
   }
   std::vector<std::thread> workers_;
   std::mutex m_;
   std::condition_variable cv_, done_;
   std::function<void()>* job_ = nullptr;
   uint64_t gen_ = 0;
   uint32_t busy_ = 0;
   bool stop_ = false;
   static inline thread_local bool inside_ = false;
};

// User-facing query errors (reference: IllegalQueryException via CHECK_SILO_QUERY).
struct IllegalQuery : std::runtime_error {
   using std::runtime_error::runtime_error;
};

// Internal planning errors (reference: QueryCompilationException).
struct CompilationError : std::runtime_error {
   using std::runtime_error::runtime_error;
};

}  // namespace rhygpu
