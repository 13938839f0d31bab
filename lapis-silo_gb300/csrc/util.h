// Small host utilities shared by the ingestion and planning code.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
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

// User-facing query errors (reference: IllegalQueryException via CHECK_SILO_QUERY).
struct IllegalQuery : std::runtime_error {
   using std::runtime_error::runtime_error;
};

// Internal planning errors (reference: QueryCompilationException).
struct CompilationError : std::runtime_error {
   using std::runtime_error::runtime_error;
};

}  // namespace rhygpu
