// Upload of the table image to HBM and execution of the plain single-query path.
#include "engine.h"

#include <algorithm>
#include <cstring>

namespace rhygpu {

void cuda_check(cudaError_t e, const char* what) {
   if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

void* Engine::alloc(size_t bytes) {
   void* p = nullptr;
   bytes = std::max<size_t>(bytes, 16);
   cuda_check(cudaMalloc(&p, bytes), "cudaMalloc");
   allocs_.push_back(p);
   device_bytes_ += bytes;
   return p;
}

template <typename T>
T* Engine::upload(const std::vector<T>& v, size_t min_elems) {
   const size_t n = std::max(v.size(), min_elems);
   T* p = static_cast<T*>(alloc(n * sizeof(T)));
   if (!v.empty()) cuda_check(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
   return p;
}

Engine::Engine(const TableImage& t, int device) : table_(t), device_(device) {
   if (t.seq.size() > MAX_SEQ_COLS || t.dict.size() > MAX_DICT_COLS || t.date.size() > MAX_DATE_COLS)
      throw std::invalid_argument("too many columns for the device image");
   cuda_check(cudaSetDevice(device), "cudaSetDevice");
   try {
      cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
      const uint32_t nchunks = t.nchunks();
      view_.nchunks = nchunks;
      view_.n_rows = t.n_rows;
      view_.chunk_sizes = upload(t.chunk_sizes);
      uint32_t max_words = 1, max_L = 1;
      for (size_t c = 0; c < t.seq.size(); ++c) {
         const SeqColumnImage& s = t.seq[c];
         DevSeqCol& d = view_.seq[c];
         d.ctrs = upload(s.vertical.ctrs);
         d.payload = upload(s.vertical.payload, 8);
         d.off = upload(s.vertical.off);
         d.exc = upload(s.cov_exc);
         d.exc_off = upload(s.cov_exc_off);
         d.nblk = upload(s.nblk);
         d.nblk_off = upload(s.nblk_off);
         std::vector<uint32_t> nulls(static_cast<size_t>(nchunks) * CHUNK_WORDS, 0);
         for (uint32_t g : s.null_rows) nulls[g >> 5] |= 1u << (g & 31);
         d.null_tiles = upload(nulls);
         d.local_ref = upload(s.local_ref);
         d.L = s.L;
         d.nblocks = s.nblocks;
         d.nsym = alphabet(s.kind).count;
         d.nctrs = static_cast<uint32_t>(s.vertical.ctrs.size());
         max_words = std::max(max_words, d.nsym * s.L);
         max_L = std::max(max_L, s.L);
         // mutation partitions: containers of one chunk, ~64 KiB of work each
         std::vector<MutPart> parts;
         const auto& ctrs = s.vertical.ctrs;
         size_t i = 0;
         while (i < ctrs.size()) {
            MutPart p{ctrs[i].v, static_cast<uint32_t>(i), 0, 0};
            uint64_t cost = 0;
            while (i < ctrs.size() && ctrs[i].v == p.v && cost < 65536) {
               const CtrDesc& x = ctrs[i];
               cost += 48 + (x.type == CT_BITSET ? 8192u : x.type == CT_RUN ? 4u * x.nruns : 2u * (x.card_m1 + 1u));
               ++i;
            }
            p.end = static_cast<uint32_t>(i);
            parts.push_back(p);
         }
         nparts_.push_back(static_cast<uint32_t>(parts.size()));
         d_parts_.push_back(upload(parts));
      }
      for (size_t c = 0; c < t.dict.size(); ++c) {
         const DictColumnImage& s = t.dict[c];
         DevDictCol& d = view_.dict[c];
         d.ctrs = upload(s.inverted.ctrs);
         d.payload = upload(s.inverted.payload, 8);
         d.off = upload(s.inverted.off);
         d.nkeys = s.inverted.nkeys;
      }
      for (size_t c = 0; c < t.date.size(); ++c) view_.date[c].days = upload(t.date[c].days);
      d_table_ = static_cast<DevTable*>(alloc(sizeof(DevTable)));
      cuda_check(cudaMemcpy(d_table_, &view_, sizeof(DevTable), cudaMemcpyHostToDevice), "upload table view");

      d_filter = static_cast<uint32_t*>(alloc(static_cast<size_t>(nchunks) * CHUNK_WORDS * 4));
      d_count = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long)));
      counts_words = max_words;
      scratch_words = 3ull * (max_L + 1);
      d_counts = static_cast<uint32_t*>(alloc(counts_words * 4));
      d_scratch = static_cast<uint32_t*>(alloc(scratch_words * 4));
      d_code = static_cast<Instr*>(alloc(MAX_PROGRAM * sizeof(Instr)));
      d_err = static_cast<int*>(alloc(sizeof(int)));
      cuda_check(cudaMemset(d_err, 0, sizeof(int)), "memset");
      cuda_check(cudaMallocHost(&h_code_, MAX_PROGRAM * sizeof(Instr)), "cudaMallocHost");
      cuda_check(cudaMallocHost(&h_count_, sizeof(unsigned long long)), "cudaMallocHost");
      cuda_check(cudaMallocHost(&h_err_, sizeof(int)), "cudaMallocHost");
      cuda_check(cudaDeviceSynchronize(), "open");
   } catch (...) {
      for (void* p : allocs_) cudaFree(p);
      if (h_code_) cudaFreeHost(h_code_);
      if (h_count_) cudaFreeHost(h_count_);
      if (h_err_) cudaFreeHost(h_err_);
      if (stream_) cudaStreamDestroy(stream_);
      throw;
   }
}

Engine::~Engine() {
   cudaSetDevice(device_);
   if (stream_) cudaStreamSynchronize(stream_);
   for (void* p : allocs_) cudaFree(p);
   if (h_code_) cudaFreeHost(h_code_);
   if (h_count_) cudaFreeHost(h_count_);
   if (h_err_) cudaFreeHost(h_err_);
   if (stream_) cudaStreamDestroy(stream_);
}

uint64_t Engine::mutation_payload_bytes(int column) const { return table_.seq.at(column).vertical.payload_bytes(); }

Program Engine::plan(const std::string& expr, const LowerOptions& opt, std::string* tree) const {
   return plan_filter(expr, table_, nullptr, opt, tree);
}

void Engine::upload_program(const Program& p, Instr* dst, cudaStream_t stream) {
   if (p.code.size() > MAX_PROGRAM) throw std::invalid_argument("program too large");
   std::memcpy(h_code_, p.code.data(), p.code.size() * sizeof(Instr));
   cuda_check(cudaMemcpyAsync(dst, h_code_, p.code.size() * sizeof(Instr), cudaMemcpyHostToDevice, stream), "copy program");
}

void Engine::launch_count(const Instr* code, const Program& p, unsigned long long* count, uint32_t* tiles,
                          cudaStream_t stream) {
   uint32_t W = tile_bits;
   // shared memory: keep the stack under 200 KiB
   while (W > 4096 && static_cast<size_t>(p.max_depth) * (W / 8) > 200 * 1024) W >>= 1;
   if (static_cast<size_t>(p.max_depth) * (W / 8) > 200 * 1024) throw IllegalQuery("filter expression nests too deeply");
   rhygpu::launch_filter(d_table_, nchunks(), code, static_cast<uint32_t>(p.code.size()), W, p.max_depth, tiles, count,
                         d_err, stream);
   cuda_check(cudaGetLastError(), "filter kernel launch");
}

void Engine::launch_mutations(int column, const uint32_t* filter, const unsigned long long* count, uint32_t* counts,
                              uint32_t* scratch, cudaStream_t stream) {
   const DevSeqCol& c = view_.seq[column];
   rhygpu::launch_mutations(d_table_, c, static_cast<uint32_t>(column), nchunks(), d_parts_[column], nparts_[column],
                            filter, count, counts, scratch, stream);
   cuda_check(cudaGetLastError(), "mutations kernel launch");
}

void Engine::check_error_flag() {
   if (*h_err_ != 0) {
      const int e = *h_err_;
      *h_err_ = 0;
      cudaMemset(d_err, 0, sizeof(int));
      throw CompilationError("device program error " + std::to_string(e));
   }
}

uint64_t Engine::count(const Program& p, cudaStream_t stream) {
   std::lock_guard<std::mutex> lock(mu);
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   if (!stream) stream = stream_;
   upload_program(p, d_code, stream);
   cuda_check(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream), "memset");
   launch_count(d_code, p, d_count, nullptr, stream);
   cuda_check(cudaMemcpyAsync(h_count_, d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "copy count");
   cuda_check(cudaMemcpyAsync(h_err_, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "copy error flag");
   cuda_check(cudaStreamSynchronize(stream), "count");
   check_error_flag();
   return *h_count_;
}

void Engine::eval(const Program& p, uint32_t* host_bits, uint64_t* host_count, cudaStream_t stream) {
   std::lock_guard<std::mutex> lock(mu);
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   if (!stream) stream = stream_;
   upload_program(p, d_code, stream);
   cuda_check(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream), "memset");
   launch_count(d_code, p, d_count, d_filter, stream);
   if (host_bits)
      cuda_check(cudaMemcpyAsync(host_bits, d_filter, static_cast<size_t>(nchunks()) * CHUNK_WORDS * 4, cudaMemcpyDeviceToHost,
                                 stream),
                 "copy row set");
   cuda_check(cudaMemcpyAsync(h_count_, d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "copy count");
   cuda_check(cudaMemcpyAsync(h_err_, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "copy error flag");
   cuda_check(cudaStreamSynchronize(stream), "eval");
   check_error_flag();
   if (host_count) *host_count = *h_count_;
}

void Engine::mutations(const Program& p, int column, uint32_t* host_counts, uint64_t* filter_count, cudaStream_t stream) {
   if (column < 0 || static_cast<size_t>(column) >= table_.seq.size()) throw std::invalid_argument("no such sequence column");
   std::lock_guard<std::mutex> lock(mu);
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   if (!stream) stream = stream_;
   const DevSeqCol& c = view_.seq[column];
   const size_t words = static_cast<size_t>(c.nsym) * c.L;
   upload_program(p, d_code, stream);
   cuda_check(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream), "memset");
   cuda_check(cudaMemsetAsync(d_counts, 0, words * 4, stream), "memset");
   cuda_check(cudaMemsetAsync(d_scratch, 0, 3ull * (c.L + 1) * 4, stream), "memset");
   launch_count(d_code, p, d_count, d_filter, stream);
   launch_mutations(column, d_filter, d_count, d_counts, d_scratch, stream);
   cuda_check(cudaMemcpyAsync(h_count_, d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "copy count");
   cuda_check(cudaMemcpyAsync(host_counts, d_counts, words * 4, cudaMemcpyDeviceToHost, stream), "copy counts");
   cuda_check(cudaMemcpyAsync(h_err_, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "copy error flag");
   cuda_check(cudaStreamSynchronize(stream), "mutations");
   check_error_flag();
   if (filter_count) *filter_count = *h_count_;
}

}  // namespace rhygpu
