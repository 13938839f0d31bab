// Device-resident partition and the execution of filter / count / mutations queries on it.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "device.h"
#include "expr.h"
#include "table.h"

namespace rhygpu {

struct CudaError : std::runtime_error {
   using std::runtime_error::runtime_error;
};

void cuda_check(cudaError_t e, const char* what);

class Engine {
  public:
   Engine(const TableImage& table, int device);
   ~Engine();
   Engine(const Engine&) = delete;
   Engine& operator=(const Engine&) = delete;

   const TableImage& table() const { return table_; }
   int device() const { return device_; }
   uint32_t nchunks() const { return table_.nchunks(); }
   const DevTable* d_table() const { return d_table_; }
   const DevTable& host_view() const { return view_; }
   uint64_t device_bytes() const { return device_bytes_; }

   // Tile width of the filter kernel (rows per CTA). 4096 .. 65536, power of two.
   uint32_t tile_bits = 16384;

   Program plan(const std::string& expr, const LowerOptions& opt = {}, std::string* tree = nullptr) const;

   // Plain single-query path: host in, host out, synchronous on `stream` (nullptr = engine stream).
   uint64_t count(const Program& p, cudaStream_t stream);
   void eval(const Program& p, uint32_t* host_bits /* nchunks * 2048 */, uint64_t* host_count, cudaStream_t stream);
   void mutations(const Program& p, int column, uint32_t* host_counts /* nsym * L */, uint64_t* filter_count,
                  cudaStream_t stream);

   // Device-side building blocks (no host synchronisation); used by the timed benchmark legs.
   void upload_program(const Program& p, Instr* d_code, cudaStream_t stream);
   void launch_count(const Instr* d_code, const Program& p, unsigned long long* d_count, uint32_t* d_tiles,
                     cudaStream_t stream);
   void launch_mutations(int column, const uint32_t* d_filter, const unsigned long long* d_count, uint32_t* d_counts,
                         uint32_t* d_scratch, cudaStream_t stream);
   void check_error_flag();

   const MutPart* d_parts(int column) const { return d_parts_[column]; }
   uint32_t nparts(int column) const { return nparts_[column]; }
   uint64_t mutation_payload_bytes(int column) const;

   // scratch of the single-query path
   uint32_t* d_filter = nullptr;      // nchunks * CHUNK_WORDS
   unsigned long long* d_count = nullptr;
   uint32_t* d_counts = nullptr;      // max nsym * L
   uint32_t* d_scratch = nullptr;     // 3 * (max L + 1)
   Instr* d_code = nullptr;           // MAX_PROGRAM
   int* d_err = nullptr;
   size_t counts_words = 0, scratch_words = 0;
   std::mutex mu;

  private:
   template <typename T>
   T* upload(const std::vector<T>& v, size_t min_elems = 1);
   void* alloc(size_t bytes);

   const TableImage& table_;
   int device_;
   cudaStream_t stream_ = nullptr;
   DevTable view_{};
   DevTable* d_table_ = nullptr;
   std::vector<void*> allocs_;
   std::vector<MutPart*> d_parts_;
   std::vector<uint32_t> nparts_;
   Instr* h_code_ = nullptr;               // pinned staging
   unsigned long long* h_count_ = nullptr; // pinned
   int* h_err_ = nullptr;                  // pinned
   uint64_t device_bytes_ = 0;
};

}  // namespace rhygpu
