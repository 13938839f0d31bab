// Mutations pass without any device allocation.
//
// Some callers cannot let a library allocate device memory during a query: a serving process that
// hands all of its HBM to its own pool allocator at start-up (a cudaMalloc from inside the library
// would fail or fragment that pool), or a latency-critical thread that must not run into the
// implicit device synchronisation cudaMalloc / cudaFree can cause. rhy_mutations_noalloc serves
// them: the caller passes the filter row set, its cardinality, the output buffer and a status word,
// all in device memory it owns, and the only working memory is the fixed-size array below, which
// lives in the
// library's device image and is loaded with it on every GPU that uses the library (held until the
// process exits).
//
// Limits and sharing: the array holds the difference arrays of one pass for genomes of at most
// NOALLOC_MAX_POSITIONS positions; longer columns are rejected. Every call on a device uses the
// same array, so calls whose work overlaps on that GPU (other streams, other threads, other
// handles) race and must be serialised by the caller. The array keeps the last call's contents;
// each call clears the part it uses before its kernels run. A device error of the pass (a bounded
// wait of the container pass for its bulk copies that gave up: 7) goes to the caller's status word,
// never to the handle's own error flag, so it can neither pass unseen nor fall on a later call; a
// completed pass leaves it 0.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/rhydb_gpu.h"
#include "device.h"
#include "engine.h"

namespace rhygpu {

// Longest sequence column a no-allocation pass accepts (positions).
constexpr uint32_t NOALLOC_MAX_POSITIONS = 131072;
constexpr size_t NOALLOC_SCRATCH_WORDS = 3ull * (NOALLOC_MAX_POSITIONS + 1) + 3ull * ((NOALLOC_MAX_POSITIONS + MUT_SEG) / MUT_SEG);

// 1.5 MiB of working memory in the device image. In host code this name is only a stand-in for
// the symbol; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) uint32_t g_noalloc_scratch[NOALLOC_SCRATCH_WORDS];

namespace {

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
uint32_t* g_scratch_addr[MAX_DEVICES] = {};

// Device address of the array on the current device, looked up once per device.
uint32_t* scratch_address(int device) {
   if (device < 0 || device >= MAX_DEVICES) throw std::invalid_argument("device ordinal out of range");
   std::lock_guard<std::mutex> lock(g_setup_mu);
   if (g_scratch_addr[device] == nullptr) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) throw CudaError(std::string("cudaGetSymbolAddress of the no-allocation scratch: ") + cudaGetErrorString(e));
      g_scratch_addr[device] = static_cast<uint32_t*>(p);
   }
   return g_scratch_addr[device];
}

}  // namespace

void mutations_noalloc(Engine& engine, uint32_t column, const uint32_t* d_filter, const unsigned long long* d_filter_count,
                       uint32_t* d_counts, int* d_status, cudaStream_t stream) {
   if (column >= engine.table().seq.size()) throw std::invalid_argument("no such sequence column");
   const DevSeqCol& col = engine.host_view().seq[column];
   if (col.L > NOALLOC_MAX_POSITIONS)
      throw std::invalid_argument("rhy_mutations_noalloc: column has " + std::to_string(col.L) +
                                  " positions, the no-allocation pass supports at most " +
                                  std::to_string(NOALLOC_MAX_POSITIONS));
   if (d_filter == nullptr || d_filter_count == nullptr || d_counts == nullptr || d_status == nullptr)
      throw std::invalid_argument("rhy_mutations_noalloc: device buffers must not be NULL");
   // The handle's lock orders this enqueue against the handle's other calls (which share its
   // stream when `stream` is NULL); it allocates nothing.
   std::lock_guard<std::mutex> lock(engine.mu);
   cuda_check(cudaSetDevice(engine.device()), "cudaSetDevice");
   uint32_t* scratch = scratch_address(engine.device());
   cudaStream_t s = engine.stream_for(stream);
   // the pass accumulates into both buffers, so they start from zero; the status starts clear
   cuda_check(cudaMemsetAsync(scratch, 0, mut_scratch_words(col.L) * sizeof(uint32_t), s), "clear scratch");
   cuda_check(cudaMemsetAsync(d_counts, 0, static_cast<size_t>(col.nsym) * col.L * sizeof(uint32_t), s), "clear counts");
   cuda_check(cudaMemsetAsync(d_status, 0, sizeof(int), s), "clear status");
   cudaGetLastError();
   launch_mutations(engine.d_table(), col, column, engine.nchunks(), engine.d_ev(static_cast<int>(column)),
                    engine.n_ev(static_cast<int>(column)), d_filter, d_filter_count, d_counts, scratch, d_status, s,
                    MUT_PART_ALL | MUT_PART_SPARSE, engine.sparse_rows_plain);
   cuda_check(cudaGetLastError(), "mutations (no allocation) launch");
}

}  // namespace rhygpu
