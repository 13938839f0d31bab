// Serving loop (see server.h).
#include "server.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>

namespace rhygpu {

namespace {

double now_s() {
   return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

Server::Server(Engine& engine, const ServerConfig& cfg) : engine_(engine), cfg_(cfg) {
   if (cfg_.max_batch == 0 || cfg_.streams == 0 || cfg_.max_inflight == 0)
      throw std::invalid_argument("server: max_batch, streams and max_inflight must be positive");
   cuda_check(cudaSetDevice(engine_.device()), "cudaSetDevice");
   if (cfg_.memory_budget == 0) {
      size_t free_b = 0, total_b = 0;
      cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
      cfg_.memory_budget = free_b / 4;
   }
   st_.budget_bytes = cfg_.memory_budget;
   slots_.resize(cfg_.streams);
   for (Slot& s : slots_) {
      cuda_check(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "cudaStreamCreate");
      cuda_check(cudaEventCreateWithFlags(&s.event, cudaEventDisableTiming), "cudaEventCreate");
   }
   thread_ = std::thread([this] { loop(); });
}

Server::~Server() {
   stop();
   cudaSetDevice(engine_.device());
   for (Slot& s : slots_) {
      if (s.stream) cudaStreamSynchronize(s.stream);
      engine_.batch_free(s.b);
      if (s.h_rows) cudaFreeHost(s.h_rows);
      if (s.event) cudaEventDestroy(s.event);
      if (s.stream) cudaStreamDestroy(s.stream);
   }
}

size_t Server::request_bytes(const ServeRequest& r) const {
   BatchQuery q;
   q.action = r.action;
   q.column = r.column;
   q.k = r.k;
   size_t b = engine_.batch_device_bytes({q});
   if (r.action == 1) b += static_cast<size_t>(engine_.nchunks()) * CHUNK_ROWS / 8;  // share of the query masks
   return b;
}

uint64_t Server::submit(const std::string& expr, int action, int column, double min_proportion, uint32_t k) {
   if (action < 0 || action > 2) throw std::invalid_argument("action must be 0 (count), 1 (mutations) or 2 (details)");
   if (action == 1 && (column < 0 || static_cast<size_t>(column) >= engine_.table().seq.size()))
      throw std::invalid_argument("no such sequence column");
   if (!(min_proportion >= 0.0 && min_proportion <= 1.0)) throw std::invalid_argument("min_proportion must lie in [0, 1]");
   compile_filter(expr, engine_.table());  // user errors surface here, before anything is queued
   auto r = std::make_shared<ServeRequest>();
   r->expr = expr;
   r->action = action;
   r->column = column;
   r->min_proportion = min_proportion;
   r->k = k;
   r->bytes = request_bytes(*r);
   if (r->bytes > cfg_.memory_budget)
      throw std::invalid_argument("request needs " + std::to_string(r->bytes) + " device bytes, the server's budget is " +
                                  std::to_string(cfg_.memory_budget));
   std::lock_guard<std::mutex> lock(mu_);
   if (stop_) throw std::logic_error("server stopped");
   r->id = next_id_++;
   r->t_submit = now_s();
   if (t_first_ < 0) t_first_ = r->t_submit;
   all_[r->id] = r;
   pending_.push_back(r);
   ++st_.submitted;
   cv_work_.notify_one();
   return r->id;
}

std::shared_ptr<ServeRequest> Server::wait(uint64_t id, double timeout_ms) {
   std::unique_lock<std::mutex> lock(mu_);
   auto it = all_.find(id);
   if (it == all_.end()) throw std::invalid_argument("no such request");
   std::shared_ptr<ServeRequest> r = it->second;
   auto ready = [&] { return r->done; };
   if (timeout_ms < 0) {
      cv_done_.wait(lock, ready);
   } else if (!cv_done_.wait_for(lock, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
      return nullptr;
   }
   return r;
}

void Server::release(uint64_t id) {
   std::lock_guard<std::mutex> lock(mu_);
   all_.erase(id);
}

bool Server::cancel(uint64_t id) {
   std::lock_guard<std::mutex> lock(mu_);
   auto it = all_.find(id);
   if (it == all_.end()) throw std::invalid_argument("no such request");
   ServeRequest& r = *it->second;
   if (r.done) return false;
   r.cancelled = true;
   const auto q = std::find(pending_.begin(), pending_.end(), it->second);
   if (q != pending_.end()) {  // not admitted yet: it never reaches the device
      pending_.erase(q);
      r.error = "request cancelled";
      r.t_done = now_s();
      r.done = true;
      ++st_.cancelled;
      cv_done_.notify_all();
   }
   return true;
}

void Server::run_plain(ServeRequest& r, cudaStream_t stream) {
   const Program p = engine_.plan(r.expr);
   if (r.action == 0) {
      r.count = engine_.count(p, stream);
   } else if (r.action == 1) {
      const SeqColumnImage& c = engine_.table().seq.at(static_cast<size_t>(r.column));
      std::vector<uint32_t> counts(static_cast<size_t>(alphabet(c.kind).count) * c.L);
      uint64_t n = 0;
      engine_.mutations(p, r.column, counts.data(), &n, stream);
      r.count = n;
      r.rows.resize(mutation_rows_host(c, counts.data(), r.min_proportion, nullptr, 0));
      mutation_rows_host(c, counts.data(), r.min_proportion, r.rows.data(), r.rows.size());
   } else {
      std::vector<uint32_t> bits(static_cast<size_t>(engine_.nchunks()) * CHUNK_WORDS);
      uint64_t n = 0;
      engine_.eval(p, bits.data(), &n, stream);
      r.count = n;
      for (size_t w = 0; w < bits.size() && r.ids.size() < r.k; ++w)
         for (uint32_t x = bits[w]; x && r.ids.size() < r.k; x &= x - 1)
            r.ids.push_back(static_cast<uint32_t>(w * 32 + static_cast<uint32_t>(__builtin_ctz(x))));
   }
}

ServerStats Server::stats() {
   std::lock_guard<std::mutex> lock(mu_);
   ServerStats s = st_;
   if (!latencies_ms_.empty()) {
      std::vector<double> v = latencies_ms_;
      std::sort(v.begin(), v.end());
      s.p50_ms = v[(v.size() - 1) / 2];
      s.p99_ms = v[static_cast<size_t>(0.99 * static_cast<double>(v.size() - 1))];
   }
   s.mean_batch = st_.batches ? static_cast<double>(batched_queries_) / static_cast<double>(st_.batches) : 0.0;
   if (t_first_ >= 0 && t_last_ > t_first_) s.qps = static_cast<double>(st_.completed) / (t_last_ - t_first_);
   return s;
}

void Server::stop() {
   {
      std::lock_guard<std::mutex> lock(mu_);
      if (stop_ && !thread_.joinable()) return;
      stop_ = true;
   }
   cv_work_.notify_all();
   if (thread_.joinable()) thread_.join();
}

void Server::loop() {
   cudaSetDevice(engine_.device());
   while (cfg_.plain) {  // one request at a time through the single-query path
      std::shared_ptr<ServeRequest> r;
      {
         std::unique_lock<std::mutex> lock(mu_);
         cv_work_.wait(lock, [&] { return stop_ || !pending_.empty(); });
         if (pending_.empty()) return;  // stopped and drained
         r = pending_.front();
         pending_.pop_front();
         ++inflight_;
         ++st_.batches;
         ++batched_queries_;
      }
      std::string error;
      try {
         run_plain(*r, slots_[0].stream);
      } catch (const std::exception& e) {
         error = e.what();
      }
      const double t = now_s();
      std::lock_guard<std::mutex> lock(mu_);
      --inflight_;
      r->t_done = t;
      t_last_ = t;
      if (r->cancelled) {
         r->error = "request cancelled";
         ++st_.cancelled;
      } else if (!error.empty()) {
         r->error = error;
         ++st_.rejected;
      } else {
         latencies_ms_.push_back(1000.0 * (r->t_done - r->t_submit));
         ++st_.completed;
      }
      r->done = true;
      cv_done_.notify_all();
   }
   for (;;) {
      bool progressed = false;
      for (Slot& s : slots_) {
         if (s.phase == 0) continue;
         const cudaError_t e = cudaEventQuery(s.event);
         if (e == cudaErrorNotReady) continue;
         if (e != cudaSuccess) {
            fail(s, std::string("device error: ") + cudaGetErrorString(e));
         } else {
            advance(s);
         }
         progressed = true;
      }
      Slot* idle = nullptr;
      bool busy = false;
      for (Slot& s : slots_) {
         if (s.phase == 0 && !idle) idle = &s;
         busy |= s.phase != 0;
      }
      std::vector<std::shared_ptr<ServeRequest>> take;
      {
         std::unique_lock<std::mutex> lock(mu_);
         if (stop_ && pending_.empty() && !busy) break;
         if (idle && !pending_.empty()) {
            const double waited_ms = 1000.0 * (now_s() - pending_.front()->t_submit);
            if (!busy || stop_ || pending_.size() >= cfg_.max_batch || waited_ms >= cfg_.max_wait_ms) {
               size_t bytes = 0;
               while (!pending_.empty() && take.size() < cfg_.max_batch && inflight_ + take.size() < cfg_.max_inflight) {
                  const auto& r = pending_.front();
                  if (inflight_bytes_ + bytes + r->bytes > cfg_.memory_budget) break;  // admission by device memory
                  bytes += r->bytes;
                  take.push_back(r);
                  pending_.pop_front();
               }
               if (!take.empty()) {
                  inflight_ += static_cast<uint32_t>(take.size());
                  inflight_bytes_ += bytes;
                  idle->bytes = bytes;
                  st_.peak_bytes = std::max<uint64_t>(st_.peak_bytes, inflight_bytes_);
                  st_.peak_inflight = std::max(st_.peak_inflight, inflight_);
                  ++st_.batches;
                  batched_queries_ += take.size();
               }
            }
         }
         if (take.empty() && !progressed) {
            // nothing to launch and nothing finished: sleep until a submit or a short poll period
            cv_work_.wait_for(lock, std::chrono::microseconds(busy ? 20 : 2000));
            continue;
         }
      }
      if (!take.empty()) launch(*idle, std::move(take));
   }
}

void Server::launch(Slot& slot, std::vector<std::shared_ptr<ServeRequest>>&& reqs) {
   slot.reqs = std::move(reqs);
   try {
      std::lock_guard<std::mutex> lock(engine_.mu);
      std::vector<std::string> texts;
      texts.reserve(slot.reqs.size());
      for (const auto& r : slot.reqs) texts.push_back(r->expr);
      std::vector<BatchQuery> qs = engine_.plan_batch(texts, 0);
      for (size_t i = 0; i < qs.size(); ++i) {
         qs[i].action = slot.reqs[i]->action;
         qs[i].column = slot.reqs[i]->column;
         qs[i].min_proportion = slot.reqs[i]->min_proportion;
         qs[i].k = slot.reqs[i]->k;
      }
      engine_.batch_prepare(slot.b, qs, 0);
      engine_.rows_phase1(slot.b, slot.stream);
      cuda_check(cudaEventRecord(slot.event, slot.stream), "event record");
      slot.phase = 1;
   } catch (const std::exception& e) {
      fail(slot, e.what());
   }
}

void Server::advance(Slot& slot) {
   if (slot.phase == 1 && slot.b.n_mut_slots > 0) {
      try {
         std::lock_guard<std::mutex> lock(engine_.mu);
         engine_.check_batch_error(slot.b);
         const size_t total = slot.b.h_rowblk[slot.b.n_blk];
         if (total > slot.h_rows_cap) {
            if (slot.h_rows) cudaFreeHost(slot.h_rows);
            slot.h_rows = nullptr;
            slot.h_rows_cap = 0;
            const size_t cap = total + total / 4 + 1024;
            cuda_check(cudaMallocHost(&slot.h_rows, cap * sizeof(DevMutationRow)), "cudaMallocHost (rows)");
            slot.h_rows_cap = cap;
         }
         engine_.rows_phase2(slot.b, slot.stream, slot.h_rows, slot.h_rows_cap);
         cuda_check(cudaEventRecord(slot.event, slot.stream), "event record");
         slot.phase = 2;
      } catch (const std::exception& e) {
         fail(slot, e.what());
      }
      return;
   }
   finish(slot);
}

void Server::finish(Slot& slot) {
   try {
      engine_.check_batch_error(slot.b);
   } catch (const std::exception& e) {
      fail(slot, e.what());
      return;
   }
   const double t = now_s();
   std::lock_guard<std::mutex> lock(mu_);
   for (size_t i = 0; i < slot.reqs.size(); ++i) {
      ServeRequest& r = *slot.reqs[i];
      const uint32_t q = static_cast<uint32_t>(i);
      if (r.cancelled) {  // ran on the device, the result is discarded
         r.error = "request cancelled";
         r.t_done = t;
         r.done = true;
         ++st_.cancelled;
         continue;
      }
      r.count = engine_.batch_state_count(slot.b, q);
      if (r.action == 1) {
         uint64_t begin;
         uint32_t n;
         engine_.row_range(slot.b, q, &begin, &n);
         r.rows.assign(slot.h_rows + begin, slot.h_rows + begin + n);
      } else if (r.action == 2) {
         uint32_t n;
         const uint32_t* ids = engine_.details_ids(slot.b, q, &n);
         if (ids) r.ids.assign(ids, ids + n);
      }
      r.t_done = t;
      r.done = true;
      latencies_ms_.push_back(1000.0 * (r.t_done - r.t_submit));
      ++st_.completed;
   }
   t_last_ = t;
   inflight_ -= static_cast<uint32_t>(slot.reqs.size());
   inflight_bytes_ -= slot.bytes;
   slot.reqs.clear();
   slot.bytes = 0;
   slot.phase = 0;
   cv_done_.notify_all();
}

void Server::fail(Slot& slot, const std::string& what) {
   if (slot.stream) cudaStreamSynchronize(slot.stream);
   const double t = now_s();
   std::lock_guard<std::mutex> lock(mu_);
   for (auto& r : slot.reqs) {
      r->error = what;
      r->t_done = t;
      r->done = true;
      ++st_.rejected;
   }
   inflight_ -= static_cast<uint32_t>(slot.reqs.size());
   inflight_bytes_ -= slot.bytes;
   slot.reqs.clear();
   slot.bytes = 0;
   slot.phase = 0;
   cv_done_.notify_all();
}

std::vector<double> Server::replay(const std::vector<ServeRequest>& reqs, const std::vector<double>& arrival_s,
                                   double* wall_s) {
   if (reqs.size() != arrival_s.size()) throw std::invalid_argument("replay: one arrival time per request");
   const size_t n = reqs.size();
   std::vector<uint64_t> ids(n, 0);
   std::vector<std::string> errors(n);
   const double t0 = now_s();
   std::thread producer([&] {
      for (size_t i = 0; i < n; ++i) {
         const double due = t0 + arrival_s[i];
         for (double t = now_s(); t < due; t = now_s()) {
            if (due - t > 200e-6) std::this_thread::sleep_for(std::chrono::microseconds(100));
         }
         try {
            ids[i] = submit(reqs[i].expr, reqs[i].action, reqs[i].column, reqs[i].min_proportion, reqs[i].k);
         } catch (const std::exception& e) {
            errors[i] = e.what();
         }
      }
   });
   producer.join();
   std::vector<double> lat(n, std::nan(""));
   double t_end = t0;
   for (size_t i = 0; i < n; ++i) {
      if (!ids[i]) continue;
      std::shared_ptr<ServeRequest> r = wait(ids[i], -1.0);
      if (r->error.empty()) lat[i] = 1000.0 * (r->t_done - r->t_submit);
      t_end = std::max(t_end, r->t_done);
      release(ids[i]);
   }
   if (wall_s) *wall_s = t_end - t0;
   return lat;
}

}  // namespace rhygpu
