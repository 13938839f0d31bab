// Upload of the table image to HBM and execution of the plain single-query path.
#include "engine.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <numeric>
#include <unordered_map>

#include "pass_plan.h"
#include "util.h"

namespace rhygpu {
namespace {
template <typename T>
void grow_device(T*& p, size_t& cap, size_t n) {
   if (n <= cap && p) return;
   if (p) cudaFree(p);
   p = nullptr;
   const size_t want = std::max<size_t>(n + n / 4, 16);
   cuda_check(cudaMalloc(&p, want * sizeof(T)), "cudaMalloc (batch)");
   cap = want;
}
template <typename T>
void grow_host(T*& p, size_t n, size_t& cap) {
   if (n <= cap && p) return;
   if (p) cudaFreeHost(p);
   p = nullptr;
   const size_t want = std::max<size_t>(n + n / 4, 16);
   cuda_check(cudaMallocHost(&p, want * sizeof(T)), "cudaMallocHost (batch)");
   cap = want;
}
// The profiles of a program as DevProfile entries whose arrays start at `base` (device memory of
// profile_words(aux) words, 8-byte aligned) and the words to copy there: per profile the
// interleaved (mask, diff) pairs of positions 0 .. L.
uint32_t profile_max_L(const std::vector<std::shared_ptr<const ProfileSpec>>& aux) {
   uint32_t L = 0;
   for (const auto& x : aux) L = std::max(L, static_cast<uint32_t>(x->mask.size()));
   return L;
}
size_t profile_words(const std::vector<std::shared_ptr<const ProfileSpec>>& aux) {
   size_t n = 0;
   for (const auto& x : aux) n += 2 * x->diff.size();
   return n;
}
void pack_profiles(const std::vector<std::shared_ptr<const ProfileSpec>>& aux, const uint32_t* base,
                   DevProfile* profs, uint32_t* data) {
   size_t off = 0;
   for (size_t k = 0; k < aux.size(); ++k) {
      const ProfileSpec& x = *aux[k];
      profs[k] = DevProfile{static_cast<uint32_t>(x.col), x.distance, x.base, 0,
                            reinterpret_cast<const uint2*>(base + off)};
      for (size_t p = 0; p < x.diff.size(); ++p) {
         data[off + 2 * p] = p < x.mask.size() ? x.mask[p] : 0u;
         data[off + 2 * p + 1] = x.diff[p];
      }
      off += 2 * x.diff.size();
   }
}
}  // namespace
}  // namespace rhygpu

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

// Work units of the batched container pass: per position, runs of consecutive chunks holding at
// most CTR_UNIT_ELEMENTS container elements (a heavier chunk forms a unit of its own) and at most
// CTR_UNIT_CHUNKS chunks; positions without containers have none. Sorted by element count,
// heaviest first, so the long units start in the first wave.
std::vector<CtrUnit> container_units(const SeqColumnImage& s, uint32_t nchunks) {
   const ContainerSet& cs = s.vertical;
   std::vector<std::pair<uint32_t, CtrUnit>> units;
   for (uint32_t p = 0; p < s.L; ++p) {
      uint32_t v0 = 0, acc = 0;
      for (uint32_t v = 0; v < nchunks; ++v) {
         uint32_t w = 0;
         for (uint32_t i = cs.off[static_cast<size_t>(v) * s.L + p]; i < cs.off[static_cast<size_t>(v) * s.L + p + 1]; ++i)
            w += cs.ctrs[i].card_m1 + 1u;
         if (v > v0 && (acc + w > CTR_UNIT_ELEMENTS || v - v0 == CTR_UNIT_CHUNKS)) {
            if (acc) units.push_back({acc, CtrUnit{p, static_cast<uint16_t>(v0), static_cast<uint16_t>(v)}});
            v0 = v;
            acc = 0;
         }
         acc += w;
      }
      if (acc) units.push_back({acc, CtrUnit{p, static_cast<uint16_t>(v0), static_cast<uint16_t>(nchunks)}});
   }
   std::stable_sort(units.begin(), units.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
   std::vector<CtrUnit> out(units.size());
   for (size_t i = 0; i < units.size(); ++i) out[i] = units[i].second;
   return out;
}

PassUnits pass_units(const SeqColumnImage& s, uint32_t nchunks) {
   const ContainerSet& cs = s.vertical;
   PassUnits P;
   P.afirst.assign(nchunks + 1, 0);
   P.ofirst.assign(nchunks + 1, 0);
   for (uint32_t v = 0; v < nchunks; ++v) {
      P.afirst[v] = static_cast<uint32_t>(P.au.size());
      P.ofirst[v] = static_cast<uint32_t>(P.ou.size());
      const uint32_t cb = cs.off[static_cast<size_t>(v) * s.L], ce = cs.off[static_cast<size_t>(v + 1) * s.L];
      std::vector<uint32_t> arr;
      for (uint32_t i = cb; i < ce; ++i)
         if (cs.ctrs[i].type == CT_ARRAY) arr.push_back(i);
      if (!arr.empty()) {
         auto start_of = [&](size_t k) { return cs.ctrs[arr[k]].payload; };
         auto end_of = [&](size_t k) { return cs.ctrs[arr[k]].payload + cs.ctrs[arr[k]].card_m1 + 1u; };
         const uint32_t A1 = end_of(arr.size() - 1);
         size_t lo = 0;  // first array ending after e0
         for (uint32_t e0 = start_of(0) & ~7u; e0 < A1;) {
            while (lo < arr.size() && end_of(lo) <= e0) ++lo;
            uint32_t e1 = std::min(e0 + WU, A1);
            size_t hi = lo;  // one past the last array starting before e1
            while (hi < arr.size() && start_of(hi) < e1) ++hi;
            if (arr[hi - 1] + 1 - arr[lo] > WU_DESC) {
               size_t h = lo + 1;  // arrays [lo, h) fit
               while (h < hi && arr[h] + 1 - arr[lo] <= WU_DESC) ++h;
               e1 = std::min(std::max(start_of(h) & ~7u, e0 + 8), A1);
               while (hi > lo + 1 && start_of(hi - 1) >= e1) --hi;
            }
            P.au.push_back(ArrUnit{e0, arr[lo], static_cast<uint16_t>(e1 - e0),
                                   static_cast<uint16_t>(arr[hi - 1] + 1 - arr[lo]), v});
            e0 = e1;
         }
      }
      for (uint32_t i = cb; i < ce; ++i) {
         const CtrDesc& d = cs.ctrs[i];
         if (d.type == CT_BITSET) P.ou.push_back(OtherUnit{SU_BITSET, v, d.payload, i});
         else if (d.type == CT_RUN) P.ou.push_back(OtherUnit{SU_RUN, v, 0, i});
      }
   }
   P.afirst[nchunks] = static_cast<uint32_t>(P.au.size());
   P.ofirst[nchunks] = static_cast<uint32_t>(P.ou.size());
   return P;
}

// The weights of the ranges are a consumer warp's cycles per unit, measured on the 2M-row
// benchmark table: an array unit costs a fixed part plus its elements and descriptors; a bitset,
// read by one warp straight from global memory, costs about one and a half array units.
std::vector<StreamRange> pass_ranges(const SeqColumnImage& s, const PassUnits& P, uint32_t nchunks, uint32_t ctas) {
   const ContainerSet& cs = s.vertical;
   auto aw = [&](const ArrUnit& u) -> uint64_t { return 2400ull + u.n + 20ull * u.nd; };
   auto ow = [&](const OtherUnit& u) -> uint64_t {
      return u.kind == SU_BITSET ? 6000ull : 600ull + 40ull * cs.ctrs[u.c].nruns;
   };
   uint64_t total = 0;
   for (const ArrUnit& u : P.au) total += aw(u);
   for (const OtherUnit& u : P.ou) total += ow(u);
   ctas = std::max(1u, ctas);
   std::vector<StreamRange> out;
   for (uint64_t per = std::max<uint64_t>(1, total / ctas);; per += per / 32 + 1) {
      out.clear();
      StreamRange cur{};
      bool open = false;
      uint64_t acc = 0;
      uint32_t ai = 0, oi = 0;
      auto close = [&]() {
         cur.a1 = ai;
         cur.o1 = oi;
         out.push_back(cur);
         open = false;
         acc = 0;
      };
      auto add = [&](uint32_t v, uint64_t w, bool array) {
         if (open && v != cur.v0 && v != cur.v1 && cur.v1 != cur.v0) close();  // a third chunk
         if (!open) {
            cur = StreamRange{ai, 0, oi, 0, v, v, {0, 0}};
            open = true;
         }
         cur.v1 = v;
         (array ? ai : oi)++;
         acc += w;
         if (acc >= per) close();
      };
      for (uint32_t v = 0; v < nchunks; ++v) {
         // merge the chunk's two lists so that other unit j follows array unit (j + 1/2) * na / no
         const uint64_t na = P.afirst[v + 1] - P.afirst[v], no = P.ofirst[v + 1] - P.ofirst[v];
         uint64_t ka = 0, ko = 0;
         while (ka < na || ko < no) {
            if (ko < no && (ka >= na || 2 * ka * no >= (2 * ko + 1) * na)) {
               add(v, ow(P.ou[P.ofirst[v] + ko]), false);
               ++ko;
            } else {
               add(v, aw(P.au[P.afirst[v] + ka]), true);
               ++ka;
            }
         }
      }
      if (open) close();
      // one wave; a table of more than 2 * ctas chunks needs more ranges than that (two chunks each)
      if (out.size() <= ctas || per >= total) break;
   }
   return out;
}

template <typename T>
T* Engine::upload(const std::vector<T>& v, size_t min_elems) {
   const size_t n = std::max(v.size(), min_elems);
   T* p = static_cast<T*>(alloc(n * sizeof(T)));
   if (!v.empty()) cuda_check(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
   return p;
}

// Bit-sliced date index: base = smallest date, nbits = bits of (largest - smallest), at least 1.
void Engine::upload_dates(const DateColumnImage& dc, uint32_t nchunks, DevDateCol& out) {
   const size_t words = static_cast<size_t>(nchunks) * CHUNK_WORDS;
   int64_t lo = INT64_MAX, hi = INT64_MIN;
   for (int32_t d : dc.days)
      if (d != INT32_MIN) lo = std::min<int64_t>(lo, d), hi = std::max<int64_t>(hi, d);
   if (lo > hi) lo = hi = 0;
   const uint64_t span = static_cast<uint64_t>(hi - lo);
   uint32_t nbits = 1;
   while (nbits < MAX_DATE_BITS && (span >> nbits) != 0) ++nbits;
   std::vector<uint32_t> planes(static_cast<size_t>(nbits) * words, 0), nulls(words, 0);
   for (size_t g = 0; g < dc.days.size() && g < words * 32; ++g) {
      const int32_t d = dc.days[g];
      if (d == INT32_MIN) {
         nulls[g >> 5] |= 1u << (g & 31);
         continue;
      }
      const uint64_t x = static_cast<uint64_t>(d - lo);
      for (uint32_t i = 0; i < nbits; ++i)
         if ((x >> i) & 1u) planes[i * words + (g >> 5)] |= 1u << (g & 31);
   }
   out.planes = upload(planes);
   out.nulls = upload(nulls);
   out.base = lo;
   out.nbits = nbits;
   out.pad = 0;
}

Engine::Engine(const TableImage& t, int device) : table_(t), device_(device), planner_(device) {
   if (t.seq.size() > MAX_SEQ_COLS || t.dict.size() > MAX_DICT_COLS || t.date.size() > MAX_DATE_COLS)
      throw std::invalid_argument("too many columns for the device image");
   sparse_rows_plain = t.n_rows / SPARSE_PLAIN_DIV;
   sparse_rows_batch = t.n_rows / SPARSE_BATCH_DIV;
   cuda_check(cudaSetDevice(device), "cudaSetDevice");
   try {
      cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
      mutations_setup();
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
         {
            const PassUnits P = pass_units(s, nchunks);
            d.au = upload(P.au);
            d.ou = upload(P.ou);
            d.nau = static_cast<uint32_t>(P.au.size());
            // one wave of the container pass's CTAs
            int sms = 0;
            cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_), "SM count");
            const std::vector<StreamRange> ranges =
               pass_ranges(s, P, nchunks, static_cast<uint32_t>(std::max(sms, 1)) * RING_CTAS_PER_SM);
            d.ranges = upload(ranges);
            d.nranges = static_cast<uint32_t>(ranges.size());
         }
         d.exc_toff = upload(s.exc_toff);
         d.nblk_toff = upload(s.nblk_toff);
         std::vector<uint32_t> nulls(static_cast<size_t>(nchunks) * CHUNK_WORDS, 0);
         for (uint32_t g : s.null_rows) nulls[g >> 5] |= 1u << (g & 31);
         d.null_tiles = upload(nulls);
         d.local_ref = upload(s.local_ref);
         d.global_ref = upload(s.global_ref);
         {
            const Alphabet& A = alphabet(s.kind);
            d.valid_mask = A.valid_mask;
            for (uint32_t k = 0; k < 32; ++k) d.chars[k] = k < A.count ? A.chars[k] : '?';
         }
         d.L = s.L;
         d.nblocks = s.nblocks;
         d.nsym = alphabet(s.kind).count;
         d.nctrs = static_cast<uint32_t>(s.vertical.ctrs.size());
         max_words = std::max(max_words, d.nsym * s.L);
         max_L = std::max(max_L, s.L);
         d.mstart = upload(s.mstart);
         d.mend = upload(s.mend);
         d.cstart = upload(s.cstart);
         d.cend = upload(s.cend);
         d.hrow_off = upload(s.hrow_off);
         d.hent = upload(s.hent, s.hent.size() + 8);  // 8 entries of tail: the profile pass reads whole uint4 pairs
         // coverage-pass work items: event ranges of at most EV_PER_CTA, never spanning two blocks
         std::vector<EvItem> items;
         auto split = [&](uint32_t list, uint32_t block, uint32_t b, uint32_t e) {
            for (uint32_t x = b; x < e; x += EV_PER_CTA) items.push_back({list, block, x, std::min(e, x + EV_PER_CTA)});
         };
         for (uint32_t b = 0; b < s.nblocks; ++b) {
            split(EV_MSTART, b, s.mstart_off[b], s.mstart_off[b + 1]);
            split(EV_MEND, b, s.mend_off[b], s.mend_off[b + 1]);
         }
         split(EV_CSTART, 0, 0, static_cast<uint32_t>(s.cstart.size()));
         split(EV_CEND, 0, 0, static_cast<uint32_t>(s.cend.size()));
         n_ev_.push_back(static_cast<uint32_t>(items.size()));
         d_ev_.push_back(upload(items));
         const std::vector<CtrUnit> units = container_units(s, nchunks);
         n_cu_.push_back(static_cast<uint32_t>(units.size()));
         d_cu_.push_back(upload(units));
      }
      for (size_t c = 0; c < t.dict.size(); ++c) {
         const DictColumnImage& s = t.dict[c];
         DevDictCol& d = view_.dict[c];
         d.ctrs = upload(s.inverted.ctrs);
         d.payload = upload(s.inverted.payload, 8);
         d.off = upload(s.inverted.off);
         d.nkeys = s.inverted.nkeys;
         // for aggregation: every row's value id (from the inverted index) and the string order
         std::vector<uint32_t> ids(static_cast<size_t>(nchunks) * CHUNK_ROWS, 0xFFFFFFFFu);
         for (const CtrDesc& x : s.inverted.ctrs) {
            const uint16_t* pl = s.inverted.payload.data() + x.payload;
            const size_t base = static_cast<size_t>(x.v) * CHUNK_ROWS;
            if (x.type == CT_ARRAY) {
               for (uint32_t k = 0; k <= x.card_m1; ++k) ids[base + pl[k]] = x.key;
            } else if (x.type == CT_BITSET) {
               for (uint32_t r = 0; r < CHUNK_ROWS; ++r)
                  if ((pl[r >> 4] >> (r & 15)) & 1u) ids[base + r] = x.key;
            } else {
               for (uint32_t k = 0; k < x.nruns; ++k)
                  for (uint32_t r = pl[2 * k]; r <= static_cast<uint32_t>(pl[2 * k]) + pl[2 * k + 1]; ++r) ids[base + r] = x.key;
            }
         }
         std::vector<uint32_t> by_rank(s.values.size());
         std::iota(by_rank.begin(), by_rank.end(), 0u);
         std::sort(by_rank.begin(), by_rank.end(), [&](uint32_t a, uint32_t b) { return s.values[a] < s.values[b]; });
         std::vector<uint32_t> rank(std::max<size_t>(1, s.values.size()));
         for (uint32_t r = 0; r < by_rank.size(); ++r) rank[by_rank[r]] = r;
         d_dict_ids_.push_back(upload(ids));
         d_dict_rank_.push_back(upload(rank));
         dict_by_rank_.push_back(std::move(by_rank));
      }
      for (size_t c = 0; c < t.date.size(); ++c) upload_dates(t.date[c], nchunks, view_.date[c]);
      d_table_ = static_cast<DevTable*>(alloc(sizeof(DevTable)));
      cuda_check(cudaMemcpy(d_table_, &view_, sizeof(DevTable), cudaMemcpyHostToDevice), "upload table view");

      d_filter = static_cast<uint32_t*>(alloc(static_cast<size_t>(nchunks) * CHUNK_WORDS * 4));
      d_count = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long)));
      counts_words = max_words;
      scratch_words = mut_scratch_words(max_L);
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
   cudaDeviceSynchronize();
   batch_free(batch_);
   for (auto& b : parts_) batch_free(*b);
   for (void* p : {static_cast<void*>(d_agg_dims_), static_cast<void*>(d_agg_counters_), static_cast<void*>(d_agg_blocks_),
                   static_cast<void*>(d_agg_out_), static_cast<void*>(d_prof_), static_cast<void*>(d_prof_data_),
                   static_cast<void*>(d_aux_)})
      if (p) cudaFree(p);
   for (void* p : allocs_) cudaFree(p);
   if (h_code_) cudaFreeHost(h_code_);
   if (h_count_) cudaFreeHost(h_count_);
   if (h_err_) cudaFreeHost(h_err_);
   if (stream_) cudaStreamDestroy(stream_);
}

size_t mutation_rows_host(const SeqColumnImage& c, const uint32_t* counts, double min_proportion, DevMutationRow* out,
                          size_t cap) {
   const Alphabet& A = alphabet(c.kind);
   size_t n = 0;
   for (uint32_t pos = 0; pos < c.L; ++pos) {
      uint32_t total = 0;
      for (uint32_t s = 0; s < A.count; ++s)
         if (A.valid_mask >> s & 1) total += counts[static_cast<size_t>(s) * c.L + pos];
      if (total == 0) continue;
      const uint32_t threshold =
         min_proportion == 0 ? 0 : static_cast<uint32_t>(std::ceil(static_cast<double>(total) * min_proportion) - 1);
      const uint32_t ref = c.global_ref[pos];
      for (uint32_t s = 0; s < A.count; ++s) {
         if (!(A.valid_mask >> s & 1) || s == ref) continue;
         const uint32_t count = counts[static_cast<size_t>(s) * c.L + pos];
         if (count <= threshold) continue;
         if (out && n < cap) {
            out[n].position = pos + 1;
            out[n].from = A.chars[ref];
            out[n].to = A.chars[s];
            out[n].pad = 0;
            out[n].count = count;
            out[n].coverage = total;
            out[n].proportion = static_cast<double>(count) / static_cast<double>(total);
         }
         ++n;
      }
   }
   return n;
}

uint64_t Engine::mutation_payload_bytes(int column) const { return table_.seq.at(column).vertical.payload_bytes(); }

namespace {
// Payload bytes of one container: array 2 * card, bitset 8 KiB, run 4 * nruns.
uint64_t container_bytes(const CtrDesc& d) {
   if (d.type == CT_BITSET) return CHUNK_ROWS / 8;
   if (d.type == CT_RUN) return 4ull * d.nruns;
   return 2ull * (d.card_m1 + 1u);
}
// Payload and descriptor bytes of the containers of one key whose symbol is in `mask`, over all chunks.
uint64_t key_bytes(const ContainerSet& cs, uint32_t nchunks, uint32_t key, uint32_t mask) {
   uint64_t b = 0;
   for (uint32_t v = 0; v < nchunks; ++v) {
      const size_t k = static_cast<size_t>(v) * cs.nkeys + key;
      for (uint32_t i = cs.off[k]; i < cs.off[k + 1]; ++i)
         if (mask >> cs.ctrs[i].sym & 1u) b += container_bytes(cs.ctrs[i]) + sizeof(CtrDesc);
   }
   return b;
}
}  // namespace

uint64_t Engine::instr_bytes(const Instr& in) const {
   const uint32_t nv = nchunks();
   const uint64_t set_bytes = static_cast<uint64_t>(nv) * (CHUNK_ROWS / 8);
   switch (in.op) {
      case OP_PUSH_SCAN: return key_bytes(table_.seq[in.col].vertical, nv, in.a, in.b);
      case OP_PUSH_DICT: return key_bytes(table_.dict[in.col].inverted, nv, in.a, 0xFFFFFFFFu);
      case OP_PUSH_NULLS:
      case OP_PUSH_AUX: return set_bytes;
      case OP_PUSH_COVERED: {
         const SeqColumnImage& c = table_.seq[in.col];
         const size_t blk = in.a / NBLOCK;
         return c.cov_exc.size() * sizeof(CovExc) +
                static_cast<uint64_t>(c.nblk_off[(blk + 1) * nv] - c.nblk_off[blk * nv]) * sizeof(NRunEntry);
      }
      case OP_PUSH_DATE: return static_cast<uint64_t>(view_.date[in.col].nbits + 1) * set_bytes;
      default: return 0;
   }
}

uint64_t Engine::program_bytes(const Program& p, bool writes_rows) const {
   uint64_t b = writes_rows ? static_cast<uint64_t>(nchunks()) * (CHUNK_ROWS / 8) : sizeof(unsigned long long);
   for (const Instr& in : p.code) b += instr_bytes(in);
   return b;
}

uint64_t Engine::batch_filter_bytes(const BatchState& b) const {
   uint64_t total = static_cast<uint64_t>(b.n_slots) * nchunks() * (CHUNK_ROWS / 8) +
                    static_cast<uint64_t>(b.n_queries - b.n_slots) * sizeof(unsigned long long);
   for (uint32_t i = 0; i < b.n_code; ++i) total += instr_bytes(b.h_code[i]);
   return total;
}

Program Engine::plan(const std::string& expr, const LowerOptions& opt, std::string* tree) const {
   LowerOptions o = opt;
   if (o.rows <= 0) o.rows = table_.n_rows;  // early-exit tests where the estimates say they can fire
   return plan_filter(expr, table_, nullptr, o, tree);
}

void Engine::upload_program(const Program& p, Instr* dst, cudaStream_t stream) {
   if (p.code.size() > MAX_PROGRAM) throw std::invalid_argument("program too large");
   std::memcpy(h_code_, p.code.data(), p.code.size() * sizeof(Instr));
   cuda_check(cudaMemcpyAsync(dst, h_code_, p.code.size() * sizeof(Instr), cudaMemcpyHostToDevice, stream), "copy program");
}

void Engine::launch_count(const Instr* code, const Program& p, unsigned long long* count, uint32_t* tiles,
                          cudaStream_t stream, const uint32_t* const* literals) {
   uint32_t W = tile_bits;
   // shared memory: keep the stack under 200 KiB
   while (W > 4096 && static_cast<size_t>(p.max_depth) * (W / 8) > 200 * 1024) W >>= 1;
   if (static_cast<size_t>(p.max_depth) * (W / 8) > 200 * 1024) throw IllegalQuery("filter expression nests too deeply");
   cudaGetLastError();  // an error left by an unrelated earlier call must not be reported here
   const uint32_t* aux = nullptr;
   if (p.n_literals > 0 && literals == nullptr) throw std::invalid_argument("the program reads caller row sets");
   const size_t set_words = static_cast<size_t>(nchunks()) * CHUNK_WORDS;
   if (!p.aux.empty() || p.n_literals > 0)
      grow_device(d_aux_, aux_cap_, (p.aux.size() + p.n_literals) * set_words);
   if (!p.aux.empty()) {  // MutationProfile row sets, before the program that reads them
      const uint32_t n = static_cast<uint32_t>(p.aux.size());
      const size_t nw = profile_words(p.aux);
      grow_device(d_prof_, prof_cap_, n);
      grow_device(d_prof_data_, prof_data_cap_, nw);
      std::vector<DevProfile> profs(n);
      std::vector<uint32_t> data(nw);
      pack_profiles(p.aux, d_prof_data_, profs.data(), data.data());
      cuda_check(cudaMemcpyAsync(d_prof_, profs.data(), n * sizeof(DevProfile), cudaMemcpyHostToDevice, stream), "H2D");
      cuda_check(cudaMemcpyAsync(d_prof_data_, data.data(), nw * 4, cudaMemcpyHostToDevice, stream), "H2D");
      cuda_check(cudaStreamSynchronize(stream), "profile upload");  // the host arrays go out of scope
      launch_profiles(d_table_, nchunks(), d_prof_, n, profile_max_L(p.aux), d_aux_, stream);
   }
   for (uint32_t k = 0; k < p.n_literals; ++k)  // the caller's row sets after the profiles' (the caller owns them)
      cuda_check(cudaMemcpyAsync(d_aux_ + (p.aux.size() + k) * set_words, literals[k], set_words * 4,
                                 cudaMemcpyHostToDevice, stream),
                 "copy caller row set");
   if (!p.aux.empty() || p.n_literals > 0) aux = d_aux_;
   const cudaError_t e = rhygpu::launch_filter(d_table_, nchunks(), code, static_cast<uint32_t>(p.code.size()),
                                               p.n_ctr_leaves | (p.n_cov_leaves << 16), W,
                                               p.max_depth, tiles, count, d_err, stream, nullptr, aux);
   if (e != cudaSuccess)
      throw CudaError("filter kernel launch (tile " + std::to_string(W) + " rows, stack " + std::to_string(p.max_depth) +
                      " tiles): " + cudaGetErrorString(e));
}

void Engine::launch_mutations(int column, const uint32_t* filter, const unsigned long long* count, uint32_t* counts,
                              uint32_t* scratch, cudaStream_t stream, uint32_t parts) {
   const DevSeqCol& c = view_.seq[column];
   rhygpu::launch_mutations(d_table_, c, static_cast<uint32_t>(column), nchunks(), d_ev_[column], n_ev_[column],
                            filter, count, counts, scratch, d_err, stream, parts, sparse_rows_plain);
   cuda_check(cudaGetLastError(), "mutations kernel launch");
}

void Engine::check_error_flag() {
   if (*h_err_ != 0) {
      const int e = *h_err_;
      *h_err_ = 0;
      cudaMemset(d_err, 0, sizeof(int));
      throw_device_error(e);
   }
}

void throw_device_error(int code) {
   if (code == DEVERR_WAIT_FILTER || code == DEVERR_WAIT_MUTATIONS)
      throw CudaError("a bounded device wait for bulk copies gave up (device error " + std::to_string(code) + ")");
   throw CompilationError("device program error " + std::to_string(code));
}

uint64_t Engine::count(const Program& p, cudaStream_t stream, const uint32_t* const* literals) {
   std::lock_guard<std::mutex> lock(mu);
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   if (!stream) stream = stream_;
   upload_program(p, d_code, stream);
   cuda_check(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream), "memset");
   launch_count(d_code, p, d_count, nullptr, stream, literals);
   cuda_check(cudaMemcpyAsync(h_count_, d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "copy count");
   cuda_check(cudaMemcpyAsync(h_err_, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "copy error flag");
   cuda_check(cudaStreamSynchronize(stream), "count");
   check_error_flag();
   return *h_count_;
}

void Engine::eval(const Program& p, uint32_t* host_bits, uint64_t* host_count, cudaStream_t stream,
                  const uint32_t* const* literals) {
   std::lock_guard<std::mutex> lock(mu);
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   if (!stream) stream = stream_;
   upload_program(p, d_code, stream);
   cuda_check(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream), "memset");
   launch_count(d_code, p, d_count, d_filter, stream, literals);
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

void Engine::mutations(const Program& p, int column, uint32_t* host_counts, uint64_t* filter_count, cudaStream_t stream,
                       const uint32_t* const* literals) {
   if (column < 0 || static_cast<size_t>(column) >= table_.seq.size()) throw std::invalid_argument("no such sequence column");
   std::lock_guard<std::mutex> lock(mu);
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   if (!stream) stream = stream_;
   const DevSeqCol& c = view_.seq[column];
   const size_t words = static_cast<size_t>(c.nsym) * c.L;
   upload_program(p, d_code, stream);
   cuda_check(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream), "memset");
   cuda_check(cudaMemsetAsync(d_counts, 0, words * 4, stream), "memset");
   cuda_check(cudaMemsetAsync(d_scratch, 0, mut_scratch_words(c.L) * 4, stream), "memset");
   launch_count(d_code, p, d_count, d_filter, stream, literals);
   launch_mutations(column, d_filter, d_count, d_counts, d_scratch, stream);
   cuda_check(cudaMemcpyAsync(h_count_, d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "copy count");
   cuda_check(cudaMemcpyAsync(host_counts, d_counts, words * 4, cudaMemcpyDeviceToHost, stream), "copy counts");
   cuda_check(cudaMemcpyAsync(h_err_, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "copy error flag");
   cuda_check(cudaStreamSynchronize(stream), "mutations");
   check_error_flag();
   if (filter_count) *filter_count = *h_count_;
}

}  // namespace rhygpu

// =================================================================================================
// Batched path

namespace rhygpu {

uint32_t Engine::fit_tile_bits(uint32_t requested, uint32_t depth, bool batch) const {
   uint32_t W = requested ? requested : batch ? batch_tile_bits : tile_bits;
   while (W > 4096 && static_cast<size_t>(depth) * (W / 8) > 200 * 1024) W >>= 1;
   if (static_cast<size_t>(depth) * (W / 8) > 200 * 1024) throw IllegalQuery("filter expression nests too deeply");
   return W;
}


void Engine::batch_free(BatchState& b) {
   if (b.graph) cudaGraphExecDestroy(b.graph);
   for (void* p : {static_cast<void*>(b.h_code), static_cast<void*>(b.h_q), static_cast<void*>(b.h_items),
                   static_cast<void*>(b.h_slot_query), static_cast<void*>(b.h_counts), static_cast<void*>(b.h_mcounts),
                   static_cast<void*>(b.h_minprop), static_cast<void*>(b.h_rowblk), static_cast<void*>(b.h_err),
                   static_cast<void*>(b.h_k), static_cast<void*>(b.h_ids), static_cast<void*>(b.h_nids),
                   static_cast<void*>(b.h_prof), static_cast<void*>(b.h_prof_data)})
      if (p) cudaFreeHost(p);
   for (void* p : {static_cast<void*>(b.d_code), static_cast<void*>(b.d_q), static_cast<void*>(b.d_items),
                   static_cast<void*>(b.d_slot_query), static_cast<void*>(b.d_counts), static_cast<void*>(b.d_next),
                   static_cast<void*>(b.d_tiles), static_cast<void*>(b.d_mcounts), static_cast<void*>(b.d_mscratch),
                   static_cast<void*>(b.d_masks), static_cast<void*>(b.d_minprop), static_cast<void*>(b.d_rowblk),
                   static_cast<void*>(b.d_rows), static_cast<void*>(b.d_err), static_cast<void*>(b.d_k),
                   static_cast<void*>(b.d_ids), static_cast<void*>(b.d_nids), static_cast<void*>(b.d_lists),
                   static_cast<void*>(b.d_prof), static_cast<void*>(b.d_prof_data), static_cast<void*>(b.d_aux)})
      if (p) cudaFree(p);
   b = BatchState{};
}

size_t Engine::batch_device_bytes(const std::vector<BatchQuery>& qs, uint32_t tile_bits) const {
   const uint32_t W = tile_bits ? tile_bits : batch_tile_bits;
   const size_t tiles = static_cast<size_t>(nchunks()) * (CHUNK_ROWS / W);
   const size_t tile_bytes = static_cast<size_t>(nchunks()) * CHUNK_WORDS * 4;
   size_t bytes = 0;
   std::vector<uint32_t> per_col(table_.seq.size(), 0);
   for (const auto& q : qs) {
      bytes += q.prog.code.size() * sizeof(Instr) + sizeof(QueryDesc) + tiles * sizeof(WorkItem) + 8;
      bytes += q.prog.aux.size() * (tile_bytes + sizeof(DevProfile)) + profile_words(q.prog.aux) * 4;
      if (q.action == 1 && q.column >= 0 && static_cast<size_t>(q.column) < per_col.size()) {
         const DevSeqCol& dc = view_.seq[q.column];
         bytes += tile_bytes + static_cast<size_t>(dc.nsym) * dc.L * 4 + mut_scratch_words(dc.L) * 4 + 16 + 8 +
                  (rows_blocks(dc.L) + 1) * 4 + static_cast<size_t>(dc.L) * 2 * sizeof(DevMutationRow);
         ++per_col[q.column];
      } else if (q.action == 2) {
         bytes += tile_bytes + static_cast<size_t>(q.k) * 4 + 16;
      }
   }
   for (size_t c = 0; c < per_col.size(); ++c)
      if (per_col[c]) bytes += mutations_batch_mask_bytes(per_col[c], nchunks());
   return bytes;
}

void Engine::batch_prepare(BatchState& b, const std::vector<BatchQuery>& qs, uint32_t requested_tile_bits) {
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   if (b.graph) {
      cudaGraphExecDestroy(b.graph);
      b.graph = nullptr;
   }
   const uint32_t n = static_cast<uint32_t>(qs.size());
   uint32_t depth = 1;
   size_t ncode = 0;
   for (const auto& q : qs) {
      if (q.prog.n_literals) throw std::invalid_argument("batched programs cannot read caller row sets");
      depth = std::max(depth, q.prog.max_depth);
      ncode += q.prog.code.size();
      if (q.action == 1 && (q.column < 0 || static_cast<size_t>(q.column) >= table_.seq.size()))
         throw std::invalid_argument("no such sequence column");
      if (q.action < 0 || q.action > 2) throw std::invalid_argument("action must be 0 (count), 1 (mutations) or 2 (details)");
   }
   // Filter classes: the stack of the deepest program sizes every CTA's shared memory, so programs
   // are grouped by tile width, chosen per program to keep the stack within the schedule's budget
   // (40 KiB by default: with the leaf cache, four CTAs per SM) while the tile stays as wide as the
   // schedule allows; one persistent launch per class.
   const BatchSchedule& sch = batch_schedule;
   auto class_w = [&](uint32_t d) {
      if (requested_tile_bits) return fit_tile_bits(requested_tile_bits, depth, true);
      uint32_t w = std::min(batch_tile_bits, std::max(sch.max_tile_bits, 4096u));
      while (w > 16384 && static_cast<size_t>(d) * (w / 8) > static_cast<size_t>(sch.stack_kb) * 1024) w >>= 1;
      return fit_tile_bits(w, d, true);
   };
   std::map<uint32_t, std::vector<uint32_t>, std::greater<uint32_t>> by_w;
   std::vector<uint32_t> width(n);
   for (uint32_t i = 0; i < n; ++i) {
      width[i] = class_w(qs[i].prog.max_depth);
      by_w[width[i]].push_back(i);
   }
   size_t nitems = 0;
   for (const auto& [w, v] : by_w) nitems += static_cast<size_t>(v.size()) * nchunks() * (CHUNK_ROWS / w);
   // slots (queries whose row set is kept): Mutations grouped by column, then Details
   std::vector<std::vector<uint32_t>> by_col(table_.seq.size());
   std::vector<uint32_t> details;
   for (uint32_t i = 0; i < n; ++i) {
      if (qs[i].action == 1) by_col[qs[i].column].push_back(i);
      if (qs[i].action == 2) details.push_back(i);
   }
   b.groups.clear();
   b.slot_of_query.assign(n, UINT32_MAX);
   std::vector<uint32_t> slot_query;
   size_t counts_words = 0, scratch_words = 0, mask_bytes = 0, lists_words = 0;
   uint32_t n_blk = 0;
   for (size_t c = 0; c < by_col.size(); ++c) {
      if (by_col[c].empty()) continue;
      BatchState::ColGroup g{static_cast<int>(c), static_cast<uint32_t>(slot_query.size()),
                             static_cast<uint32_t>(by_col[c].size()), counts_words, scratch_words, lists_words, n_blk};
      lists_words += 2 * static_cast<size_t>(g.n) + 2;
      n_blk += g.n * rows_blocks(view_.seq[c].L);
      for (uint32_t qi : by_col[c]) {
         b.slot_of_query[qi] = static_cast<uint32_t>(slot_query.size());
         slot_query.push_back(qi);
      }
      const DevSeqCol& dc = view_.seq[c];
      counts_words += static_cast<size_t>(g.n) * dc.nsym * dc.L;
      scratch_words += static_cast<size_t>(g.n) * mut_scratch_words(dc.L);
      mask_bytes = std::max(mask_bytes, mutations_batch_mask_bytes(g.n, nchunks()));
      b.groups.push_back(g);
   }
   const uint32_t n_mut = static_cast<uint32_t>(slot_query.size());
   for (uint32_t qi : details) {
      b.slot_of_query[qi] = static_cast<uint32_t>(slot_query.size());
      slot_query.push_back(qi);
   }
   const uint32_t nslots = static_cast<uint32_t>(slot_query.size());
   const uint32_t n_det = nslots - n_mut;
   if (nitems > 0xFFFFFFFFull) throw std::invalid_argument("batch too large");
   size_t n_ids = 0;
   for (uint32_t qi : details) n_ids += qs[qi].k;
   if (n_ids > 0xFFFFFFFFull) throw std::invalid_argument("details: too many row ids requested");
   size_t n_aux = 0, n_prof_data = 0;
   b.profile_max_L = 0;
   for (const auto& q : qs) {
      n_aux += q.prog.aux.size();
      n_prof_data += profile_words(q.prog.aux);
      b.profile_max_L = std::max(b.profile_max_L, profile_max_L(q.prog.aux));
   }
   grow_host(b.h_prof, n_aux, b.hc_prof);
   grow_device(b.d_prof, b.dc_prof, n_aux);
   grow_host(b.h_prof_data, n_prof_data, b.hc_prof_data);
   grow_device(b.d_prof_data, b.dc_prof_data, n_prof_data);
   grow_device(b.d_aux, b.dc_aux, n_aux * nchunks() * CHUNK_WORDS);
   b.n_aux = static_cast<uint32_t>(n_aux);
   b.n_prof_data = n_prof_data;
   grow_host(b.h_code, ncode, b.hc_code);
   grow_device(b.d_code, b.dc_code, ncode);
   grow_host(b.h_q, n, b.hc_q);
   grow_device(b.d_q, b.dc_q, n);
   grow_host(b.h_items, nitems, b.hc_items);
   grow_device(b.d_items, b.dc_items, nitems);
   grow_host(b.h_slot_query, nslots, b.hc_slot_query);
   grow_device(b.d_slot_query, b.dc_slot_query, nslots);
   grow_host(b.h_counts, n, b.hc_counts);
   grow_device(b.d_counts, b.dc_counts, n);
   grow_device(b.d_next, b.dc_next, by_w.size());
   grow_device(b.d_tiles, b.dc_tiles, static_cast<size_t>(nslots) * nchunks() * CHUNK_WORDS);
   grow_host(b.h_mcounts, counts_words, b.hc_mcounts);
   grow_device(b.d_mcounts, b.dc_mcounts, counts_words);
   grow_device(b.d_mscratch, b.dc_mscratch, scratch_words);
   grow_device(b.d_masks, b.dc_masks, mask_bytes / 2 + 8);
   grow_device(b.d_lists, b.dc_lists, lists_words + 2);
   grow_host(b.h_minprop, nslots, b.hc_minprop);
   grow_device(b.d_minprop, b.dc_minprop, nslots);
   grow_host(b.h_rowblk, static_cast<size_t>(n_blk) + 1, b.hc_rowblk);
   grow_device(b.d_rowblk, b.dc_rowblk, static_cast<size_t>(n_blk) + 1);
   grow_host(b.h_err, 1, b.hc_err);
   grow_device(b.d_err, b.dc_err, 1);
   grow_host(b.h_k, 2 * static_cast<size_t>(n_det), b.hc_k);
   grow_device(b.d_k, b.dc_k, 2 * static_cast<size_t>(n_det));
   grow_host(b.h_ids, n_ids, b.hc_ids);
   grow_device(b.d_ids, b.dc_ids, n_ids);
   grow_host(b.h_nids, n_det, b.hc_nids);
   grow_device(b.d_nids, b.dc_nids, n_det);
   for (uint32_t k = 0; k < nslots; ++k) {
      const double mp = qs[slot_query[k]].min_proportion;
      if (!(mp >= 0.0 && mp <= 1.0)) throw std::invalid_argument("min_proportion must lie in [0, 1]");
      b.h_minprop[k] = mp;
   }
   uint32_t koff = 0;
   for (uint32_t j = 0; j < n_det; ++j) {  // k of each Details slot, then its offset into the ids
      b.h_k[j] = qs[slot_query[n_mut + j]].k;
      b.h_k[n_det + j] = koff;
      koff += b.h_k[j];
   }
   *b.h_err = 0;
   b.n_blk = n_blk;
   b.n_rows = 0;
   b.n_mut_slots = n_mut;
   b.n_details = n_det;
   b.n_ids = static_cast<uint32_t>(n_ids);
   // programs, query descriptors, profile row sets, work items
   size_t off = 0, aux_off = 0, data_off = 0;
   for (uint32_t i = 0; i < n; ++i) {
      const Program& p = qs[i].prog;
      std::memcpy(b.h_code + off, p.code.data(), p.code.size() * sizeof(Instr));
      b.h_q[i] = QueryDesc{static_cast<uint32_t>(off), static_cast<uint32_t>(p.code.size()),
                           b.slot_of_query[i] == UINT32_MAX ? 0u : b.slot_of_query[i] + 1,
                           p.n_ctr_leaves | (p.n_cov_leaves << 16), std::max(p.max_depth, 1u),
                           static_cast<uint32_t>(aux_off), width[i]};
      off += p.code.size();
      if (!p.aux.empty()) {
         pack_profiles(p.aux, b.d_prof_data + data_off, b.h_prof + aux_off, b.h_prof_data + data_off);
         aux_off += p.aux.size();
         data_off += profile_words(p.aux);
      }
   }
   // items per class (widest tiles first), all in one persistent launch whose CTAs hold the stack
   // of any class: tile-major interleaving spreads the expensive queries over the launch; with
   // predicted costs (learned planner) the queries go heaviest first so the long ones do not end
   // their class alone
   int props = 0;
   cuda_check(cudaDeviceGetAttribute(&props, cudaDevAttrMultiProcessorCount, device_), "attribute");
   b.fgroups.clear();
   size_t k = 0;
   for (auto& [w, qv] : by_w) {
      bool costed = false;
      uint32_t gdepth = 1;
      for (uint32_t qi : qv) {
         costed |= qs[qi].cost > 0;
         gdepth = std::max(gdepth, qs[qi].prog.max_depth);
      }
      if (costed)
         std::stable_sort(qv.begin(), qv.end(), [&](uint32_t x, uint32_t y) { return qs[x].cost > qs[y].cost; });
      const uint32_t tiles = nchunks() * (CHUNK_ROWS / w);
      const size_t off = k;
      if (sch.query_major) {
         for (uint32_t qi : qv)
            for (uint32_t t = 0; t < tiles; ++t) b.h_items[k++] = WorkItem{qi, t};
      } else {
         for (uint32_t t = 0; t < tiles; ++t)
            for (uint32_t qi : qv) b.h_items[k++] = WorkItem{qi, t};
      }
      b.fgroups.push_back(BatchState::FilterGroup{static_cast<uint32_t>(off), static_cast<uint32_t>(k - off), w, gdepth});
   }
   size_t stack = 0;
   for (const auto& g : b.fgroups) stack = std::max(stack, static_cast<size_t>(g.max_depth) * (g.tile_bits / 8));
   uint32_t per_sm = static_cast<uint32_t>(filter_batch_blocks_per_sm(stack));
   if (sch.ctas_per_sm) per_sm = std::min(per_sm, sch.ctas_per_sm);
   b.stack_bytes = static_cast<uint32_t>(stack);
   b.grid = static_cast<uint32_t>(props) * per_sm;
   std::memcpy(b.h_slot_query, slot_query.data(), slot_query.size() * sizeof(uint32_t));
   b.n_queries = n;
   b.n_slots = nslots;
   b.n_items = static_cast<uint32_t>(nitems);
   b.n_code = static_cast<uint32_t>(ncode);
   b.max_depth = depth;
   // reported tile width: the class with the most items
   const auto big = std::max_element(b.fgroups.begin(), b.fgroups.end(),
                                     [](const auto& x, const auto& y) { return x.n_items < y.n_items; });
   b.tile_bits = big != b.fgroups.end() ? big->tile_bits : batch_tile_bits;
   b.counts_words = counts_words;
   b.scratch_words = scratch_words;
   b.mask_bytes = mask_bytes;
}

void Engine::batch_enqueue(BatchState& b, cudaStream_t s, bool copy_in, bool copy_out, uint32_t parts) {
   s = stream_for(s);
   if (b.n_queries == 0) return;
   if (copy_in) {
      cuda_check(cudaMemcpyAsync(b.d_code, b.h_code, b.n_code * sizeof(Instr), cudaMemcpyHostToDevice, s), "H2D");
      cuda_check(cudaMemcpyAsync(b.d_q, b.h_q, b.n_queries * sizeof(QueryDesc), cudaMemcpyHostToDevice, s), "H2D");
      cuda_check(cudaMemcpyAsync(b.d_items, b.h_items, static_cast<size_t>(b.n_items) * sizeof(WorkItem),
                                 cudaMemcpyHostToDevice, s),
                 "H2D");
      if (b.n_slots) {
         cuda_check(cudaMemcpyAsync(b.d_slot_query, b.h_slot_query, b.n_slots * sizeof(uint32_t), cudaMemcpyHostToDevice, s),
                    "H2D");
         cuda_check(cudaMemcpyAsync(b.d_minprop, b.h_minprop, b.n_slots * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
      }
      if (b.n_details)
         cuda_check(cudaMemcpyAsync(b.d_k, b.h_k, 2 * static_cast<size_t>(b.n_details) * sizeof(uint32_t),
                                    cudaMemcpyHostToDevice, s),
                    "H2D");
      if (b.n_aux) {
         cuda_check(cudaMemcpyAsync(b.d_prof, b.h_prof, b.n_aux * sizeof(DevProfile), cudaMemcpyHostToDevice, s), "H2D");
         cuda_check(cudaMemcpyAsync(b.d_prof_data, b.h_prof_data, b.n_prof_data * 4, cudaMemcpyHostToDevice, s), "H2D");
      }
      cuda_check(cudaMemsetAsync(b.d_err, 0, sizeof(int), s), "memset");
   }
   if ((parts & 1) && b.n_aux) {
      launch_profiles(d_table_, nchunks(), b.d_prof, b.n_aux, b.profile_max_L, b.d_aux, s);
      cuda_check(cudaGetLastError(), "profile launch");
   }
   if (parts & 1) {
      cuda_check(cudaMemsetAsync(b.d_counts, 0, b.n_queries * sizeof(unsigned long long), s), "memset");
      cuda_check(cudaMemsetAsync(b.d_next, 0, sizeof(uint32_t), s), "memset");
      if (b.counts_words) cuda_check(cudaMemsetAsync(b.d_mcounts, 0, b.counts_words * 4, s), "memset");
      if (b.scratch_words) cuda_check(cudaMemsetAsync(b.d_mscratch, 0, b.scratch_words * 4, s), "memset");
      if (b.n_items)
         cuda_check(launch_filter_batch(d_table_, nchunks(), b.d_code, b.d_q, b.d_items, b.n_items, b.stack_bytes, b.d_tiles,
                                        b.d_counts, b.d_next, b.grid, b.d_err, s, b.n_aux ? b.d_aux : nullptr),
                    "filter batch launch");
   }
   const size_t words = static_cast<size_t>(nchunks()) * CHUNK_WORDS;
   for (const auto& g : b.groups) {
      launch_mutations_batch(d_table_, view_.seq[g.column], static_cast<uint32_t>(g.column), nchunks(),
                             b.d_tiles + static_cast<size_t>(g.slot_begin) * words, g.n, b.d_counts,
                             b.d_slot_query + g.slot_begin, d_ev_[g.column], n_ev_[g.column], d_cu_[g.column],
                             n_cu_[g.column], b.d_masks, b.d_mcounts + g.counts_off, b.d_mscratch + g.scratch_off,
                             b.d_lists + g.lists_off, sparse_rows_batch, s,
                             (parts >> 1) & (BMUT_PART_ALL | BMUT_PART_SPARSE),
                             b.rows_in_final ? b.d_minprop + g.slot_begin : nullptr,
                             b.rows_in_final ? b.d_rowblk + g.blk_off : nullptr);
      cuda_check(cudaGetLastError(), "mutations batch launch");
   }
   if (b.n_details && (parts & 1)) {
      launch_first_k(b.d_tiles + static_cast<size_t>(b.n_mut_slots) * words, b.n_details, nchunks(), b.d_k,
                     b.d_k + b.n_details, b.d_ids, b.d_nids, s);
      cuda_check(cudaGetLastError(), "details launch");
   }
   if (copy_out) {
      cuda_check(cudaMemcpyAsync(b.h_counts, b.d_counts, b.n_queries * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s),
                 "D2H");
      if (b.counts_words)
         cuda_check(cudaMemcpyAsync(b.h_mcounts, b.d_mcounts, b.counts_words * 4, cudaMemcpyDeviceToHost, s), "D2H");
      copy_details(b, s);
      cuda_check(cudaMemcpyAsync(b.h_err, b.d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
   }
}

void Engine::copy_details(BatchState& b, cudaStream_t s) {
   if (!b.n_details) return;
   cuda_check(cudaMemcpyAsync(b.h_nids, b.d_nids, b.n_details * sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "D2H");
   if (b.n_ids) cuda_check(cudaMemcpyAsync(b.h_ids, b.d_ids, b.n_ids * sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "D2H");
}

void Engine::check_batch_error(BatchState& b) {
   if (b.h_err && *b.h_err != 0) {
      const int e = *b.h_err;
      *b.h_err = 0;
      throw_device_error(e);
   }
}

void Engine::rows_phase1(BatchState& b, cudaStream_t s) {
   s = stream_for(s);
   if (b.n_queries == 0) return;
   b.rows_in_final = true;  // the final pass counts the rows per block (no separate counting pass)
   try {
      batch_enqueue(b, s, true, false);
   } catch (...) {
      b.rows_in_final = false;
      throw;
   }
   b.rows_in_final = false;
   cuda_check(cudaMemcpyAsync(b.h_counts, b.d_counts, b.n_queries * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s),
              "D2H");
   copy_details(b, s);
   cuda_check(cudaMemcpyAsync(b.h_err, b.d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
   if (b.n_mut_slots) {
      launch_rows_scan(b.d_rowblk, b.n_blk, s);
      cuda_check(cudaMemcpyAsync(b.h_rowblk, b.d_rowblk, (static_cast<size_t>(b.n_blk) + 1) * sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, s),
                 "D2H");
   }
   cuda_check(cudaGetLastError(), "rows launch");
}

size_t Engine::rows_phase2(BatchState& b, cudaStream_t s, DevMutationRow* rows, size_t cap) {
   s = stream_for(s);
   check_batch_error(b);
   const size_t total = b.n_mut_slots ? b.h_rowblk[b.n_blk] : 0;
   b.n_rows = total;
   if (total) {
      grow_device(b.d_rows, b.dc_rows, total);
      for (const auto& g : b.groups)
         launch_rows_write(d_table_, view_.seq[g.column], static_cast<uint32_t>(g.column), b.d_mcounts + g.counts_off, g.n,
                           b.d_minprop + g.slot_begin, b.d_rowblk + g.blk_off, b.d_rows, s);
      cuda_check(cudaGetLastError(), "rows launch");
      if (rows && total <= cap)
         cuda_check(cudaMemcpyAsync(rows, b.d_rows, total * sizeof(DevMutationRow), cudaMemcpyDeviceToHost, s), "D2H");
   }
   return total;
}

void Engine::row_range(const BatchState& b, uint32_t i, uint64_t* begin, uint32_t* count) const {
   *begin = 0;
   *count = 0;
   const uint32_t slot = b.slot_of_query[i];
   if (slot == UINT32_MAX) return;
   for (const auto& g : b.groups) {
      if (slot < g.slot_begin || slot >= g.slot_begin + g.n) continue;
      const uint32_t nb = rows_blocks(view_.seq[g.column].L);
      const size_t k = g.blk_off + static_cast<size_t>(slot - g.slot_begin) * nb;
      *begin = b.h_rowblk[k];
      *count = b.h_rowblk[k + nb] - b.h_rowblk[k];
   }
}

const uint32_t* Engine::details_ids(const BatchState& b, uint32_t i, uint32_t* n) const {
   *n = 0;
   const uint32_t slot = b.slot_of_query[i];
   if (slot == UINT32_MAX || slot < b.n_mut_slots) return nullptr;
   const uint32_t j = slot - b.n_mut_slots;
   *n = b.h_nids[j];
   return b.h_ids + b.h_k[b.n_details + j];
}

size_t Engine::batch_rows(cudaStream_t s, DevMutationRow* rows, size_t cap, uint64_t* row_begin, uint32_t* row_count) {
   s = stream_for(s);
   BatchState& b = batch_;
   rows_parts_.assign(1, &batch_);
   if (b.n_queries == 0) return 0;
   const auto t0 = std::chrono::steady_clock::now();
   rows_phase1(b, s);
   cuda_check(cudaStreamSynchronize(s), "batch rows");
   const auto t1 = std::chrono::steady_clock::now();
   const size_t total = rows_phase2(b, s, rows, cap);
   cuda_check(cudaStreamSynchronize(s), "batch rows");
   batch_times.device_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
   batch_times.output_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
   for (uint32_t i = 0; i < b.n_queries; ++i) {
      uint64_t begin;
      uint32_t count;
      row_range(b, i, &begin, &count);
      if (row_begin) row_begin[i] = begin;
      if (row_count) row_count[i] = count;
   }
   return total;
}

void Engine::batch_rows_fetch(cudaStream_t s, DevMutationRow* rows, size_t cap) {
   s = stream_for(s);
   size_t total = 0;
   for (const BatchState* b : rows_parts_) total += b->n_rows;
   if (total > cap)
      throw std::invalid_argument("rows buffer holds " + std::to_string(cap) + " rows, " + std::to_string(total) +
                                  " needed");
   size_t off = 0;
   for (const BatchState* b : rows_parts_) {
      if (b->n_rows)
         cuda_check(cudaMemcpyAsync(rows + off, b->d_rows, b->n_rows * sizeof(DevMutationRow), cudaMemcpyDeviceToHost, s),
                    "D2H");
      off += b->n_rows;
   }
   cuda_check(cudaStreamSynchronize(s), "rows fetch");
}

size_t Engine::batch_rows_pipelined(const std::vector<std::string>& exprs, const int* actions, const uint32_t* columns,
                                    const double* min_proportions, uint32_t tile_bits, cudaStream_t s,
                                    DevMutationRow* rows, size_t cap, uint64_t* counts, uint64_t* row_begin,
                                    uint32_t* row_count) {
   using clk = std::chrono::steady_clock;
   auto ms = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
   s = stream_for(s);
   const uint32_t n = static_cast<uint32_t>(exprs.size());
   // first the Mutations and Details queries, in parts of at most PIPELINE_HEAVY (the device splits
   // a part's dense Mutations queries into passes of 256, and sparse ones take no pass, so one part
   // reads the containers as few times as the whole batch would), so that the device starts after
   // they are planned (without any: the first quarter of the counts); then the counts, in parts
   // planned while the parts before them run
   std::vector<std::vector<uint32_t>> parts(1);
   std::vector<uint32_t> light, heavy;
   for (uint32_t i = 0; i < n; ++i) {
      const int a = actions ? actions[i] : 0;
      if (a < 0 || a > 2) throw std::invalid_argument("action must be 0 (count), 1 (mutations) or 2 (details)");
      (a == 0 ? light : heavy).push_back(i);
   }
   {
      const size_t k = std::max<size_t>(1, (heavy.size() + PIPELINE_HEAVY - 1) / PIPELINE_HEAVY);  // heavy parts
      parts.assign(k, {});
      for (size_t j = 0; j < k; ++j)
         parts[j].assign(heavy.begin() + heavy.size() * j / k, heavy.begin() + heavy.size() * (j + 1) / k);
   }
   size_t first = 0;
   if (parts[0].empty()) {
      first = light.size() < 2 * PIPELINE_PART ? light.size() : light.size() / 4;
      parts[0].assign(light.begin(), light.begin() + first);
   }
   if (first < light.size()) {
      const size_t rest = light.size() - first;
      if (rest < PIPELINE_PART) {
         parts.back().insert(parts.back().end(), light.begin() + first, light.end());
      } else {
         // counts in parts of about PIPELINE_COUNTS, so that the planning of each overlaps the
         // device work of the part before it
         const size_t k = std::max<size_t>(1, (rest + PIPELINE_COUNTS / 2) / PIPELINE_COUNTS);
         for (size_t j = 0; j < k; ++j)
            parts.emplace_back(light.begin() + first + rest * j / k, light.begin() + first + rest * (j + 1) / k);
      }
   }
   while (parts_.size() + 1 < parts.size()) parts_.push_back(std::make_unique<BatchState>());
   std::vector<BatchState*> states(parts.size());
   for (size_t p = 0; p < parts.size(); ++p) states[p] = p == 0 ? &batch_ : parts_[p - 1].get();
   rows_parts_.assign(1, &batch_);
   for (BatchState* b : states) b->n_rows = 0;
   batch_times = BatchTimes{};
   double plan_ms = 0, prepare_ms = 0;
   clk::time_point launched;
   try {
      for (size_t p = 0; p < parts.size(); ++p) {
         const auto t0 = clk::now();
         std::vector<std::string> texts(parts[p].size());
         for (size_t j = 0; j < parts[p].size(); ++j) texts[j] = exprs[parts[p][j]];
         // the device is idle until the first part launches: that part is planned by the rule, the
         // later ones (learned planner on) with the network's inference while the device runs
         std::vector<BatchQuery> qs = plan_batch(texts, 0, p == 0);
         for (size_t j = 0; j < parts[p].size(); ++j) {
            const uint32_t i = parts[p][j];
            qs[j].action = actions ? actions[i] : 0;
            qs[j].column = columns ? static_cast<int>(columns[i]) : 0;
            if (min_proportions) qs[j].min_proportion = min_proportions[i];
         }
         const auto t1 = clk::now();
         batch_prepare(*states[p], qs, tile_bits);
         rows_phase1(*states[p], s);
         launched = clk::now();
         plan_ms += ms(t0, t1);
         prepare_ms += ms(t1, launched);
      }
      cuda_check(cudaStreamSynchronize(s), "batch rows");
   } catch (...) {
      cudaStreamSynchronize(s);  // parts already enqueued finish before their buffers are reused
      throw;
   }
   const auto t2 = clk::now();
   rows_parts_ = states;
   size_t total = 0;
   std::vector<size_t> off(parts.size());
   for (size_t p = 0; p < parts.size(); ++p) {
      off[p] = total;
      const bool fits = rows && total <= cap;
      total += rows_phase2(*states[p], s, fits ? rows + total : nullptr, fits ? cap - total : 0);
   }
   cuda_check(cudaStreamSynchronize(s), "batch rows");  // total > cap: the caller refetches every part
   for (size_t p = 0; p < parts.size(); ++p)
      for (size_t j = 0; j < parts[p].size(); ++j) {
         const uint32_t i = parts[p][j];
         uint64_t begin;
         uint32_t count;
         row_range(*states[p], static_cast<uint32_t>(j), &begin, &count);
         if (counts) counts[i] = states[p]->h_counts[j];
         if (row_begin) row_begin[i] = begin + off[p];
         if (row_count) row_count[i] = count;
      }
   batch_times.plan_ms = plan_ms;
   batch_times.prepare_ms = prepare_ms;
   batch_times.device_ms = ms(launched, t2);
   batch_times.output_ms = ms(t2, clk::now());
   return total;
}

std::vector<std::pair<BatchSchedule, double>> Engine::autotune_batch(const std::vector<BatchQuery>& qs, cudaStream_t s,
                                                                     uint32_t reps) {
   s = stream_for(s);
   reps = std::max(1u, reps);
   std::vector<BatchSchedule> cands;
   for (uint32_t w : {16384u, 32768u, 65536u})
      for (uint32_t kb : {24u, 40u, 64u})
         for (uint32_t cps : {0u, 2u})
            for (uint32_t qm : {0u, 1u}) cands.push_back(BatchSchedule{w, kb, cps, qm});
   const BatchSchedule saved = batch_schedule;
   BatchState b;
   cudaEvent_t e0 = nullptr, e1 = nullptr;
   std::vector<std::pair<BatchSchedule, double>> out;
   std::map<std::string, double> seen;  // candidates that lay the launches out alike are timed once
   try {
      cuda_check(cudaEventCreate(&e0), "event");
      cuda_check(cudaEventCreate(&e1), "event");
      for (const BatchSchedule& c : cands) {
         batch_schedule = c;
         batch_prepare(b, qs);
         std::string key = std::to_string(c.query_major);
         for (const auto& g : b.fgroups)
            key += "/" + std::to_string(g.tile_bits) + "x" + std::to_string(g.n_items);
         key += "@" + std::to_string(b.grid);
         if (const auto it = seen.find(key); it != seen.end()) {
            out.emplace_back(c, it->second);
            continue;
         }
         batch_enqueue(b, s, true, false, 1);  // copies the programs, warms the caches
         std::vector<float> t(reps);
         for (uint32_t r = 0; r < reps; ++r) {
            cuda_check(cudaEventRecord(e0, s), "event");
            batch_enqueue(b, s, false, false, 1);
            cuda_check(cudaEventRecord(e1, s), "event");
            cuda_check(cudaEventSynchronize(e1), "event");
            cuda_check(cudaEventElapsedTime(&t[r], e0, e1), "event");
         }
         cuda_check(cudaMemcpyAsync(b.h_err, b.d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
         cuda_check(cudaStreamSynchronize(s), "autotune");
         check_batch_error(b);
         std::nth_element(t.begin(), t.begin() + reps / 2, t.end());
         seen.emplace(key, t[reps / 2]);
         out.emplace_back(c, t[reps / 2]);
      }
   } catch (...) {
      cudaStreamSynchronize(s);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      batch_free(b);
      batch_schedule = saved;
      throw;
   }
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   batch_free(b);
   std::stable_sort(out.begin(), out.end(), [](const auto& x, const auto& y) { return x.second < y.second; });
   batch_schedule = out.empty() ? saved : out.front().first;
   return out;
}

void Engine::batch_capture(cudaStream_t s, bool copy_in, bool copy_out) {
   s = stream_for(s);
   BatchState& b = batch_;
   if (b.graph) {
      cudaGraphExecDestroy(b.graph);
      b.graph = nullptr;
   }
   cudaGraph_t g = nullptr;
   cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
   try {
      batch_enqueue(b, s, copy_in, copy_out);
   } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      throw;
   }
   cuda_check(cudaStreamEndCapture(s, &g), "end capture");
   cudaError_t e = cudaGraphInstantiate(&b.graph, g, 0);
   cudaGraphDestroy(g);
   cuda_check(e, "graph instantiate");
}

void Engine::batch_replay(cudaStream_t s) {
   s = stream_for(s);
   if (!batch_.graph) throw std::logic_error("no captured batch");
   cuda_check(cudaGraphLaunch(batch_.graph, s), "graph launch");
}

const uint32_t* Engine::batch_mutation_counts(uint32_t query) const {
   const BatchState& b = batch_;
   const uint32_t slot = b.slot_of_query.at(query);
   if (slot == UINT32_MAX || slot >= b.n_mut_slots) return nullptr;
   for (const auto& g : b.groups) {
      if (slot >= g.slot_begin && slot < g.slot_begin + g.n) {
         const DevSeqCol& dc = view_.seq[g.column];
         return b.h_mcounts + g.counts_off + static_cast<size_t>(slot - g.slot_begin) * dc.nsym * dc.L;
      }
   }
   return nullptr;
}

// =================================================================================================
// Learned planner

const FeatureContext& Engine::fctx() {
   if (!fctx_) fctx_ = std::make_unique<FeatureContext>(feature_context(table_));
   return *fctx_;
}

size_t Engine::planner_collect(const std::vector<std::string>& exprs) {
   std::lock_guard<std::mutex> lock(mu);
   return collect_traces(exprs, planner_.samples);
}

PlannerStats Engine::planner_evaluate(const std::vector<std::string>& exprs) {
   std::lock_guard<std::mutex> lock(mu);
   std::vector<PlannerSample> held_out;
   collect_traces(exprs, held_out);
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   const PlannerStats st = planner_.evaluate(held_out);
   planner_.accepted = st.accepted != 0;
   if (!planner_.accepted) use_learned_ = false;
   return st;
}

size_t Engine::collect_traces(const std::vector<std::string>& exprs, std::vector<PlannerSample>& out) {
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   const FeatureContext& ctx = fctx();
   const uint32_t W = tile_bits;
   const uint32_t ntiles = nchunks() * (CHUNK_ROWS / W);
   const double rows = std::max(1u, table_.n_rows);
   cudaStream_t s = stream_;
   uint32_t* d_trace = nullptr;
   size_t cap = 0;
   std::vector<uint32_t> trace;
   size_t added = 0;
   try {
      for (const std::string& text : exprs) {
         OpPtr op = compile_filter(text, table_);
         LowerOptions o;
         o.early_exit = false;
         o.record_spans = true;
         const Program p = lower(*op, ctx.rule, o);
         if (!p.aux.empty()) continue;  // MutationProfile row sets are not traced
         const uint32_t nc = static_cast<uint32_t>(p.code.size());
         const size_t words = static_cast<size_t>(ntiles) * nc * 2;
         if (words > cap) {
            if (d_trace) cudaFree(d_trace);
            d_trace = nullptr;
            cuda_check(cudaMalloc(&d_trace, words * sizeof(uint32_t)), "cudaMalloc (trace)");
            cap = words;
         }
         upload_program(p, d_code, s);
         cuda_check(cudaMemsetAsync(d_trace, 0, words * sizeof(uint32_t), s), "memset");
         cuda_check(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), s), "memset");
         const uint32_t Wf = fit_tile_bits(W, p.max_depth);
         if (Wf != W) continue;  // too deep for the trace tile width: skip
         cudaGetLastError();
         cuda_check(launch_filter(d_table_, nchunks(), d_code, nc, p.n_ctr_leaves | (p.n_cov_leaves << 16), W, p.max_depth,
                                  nullptr, d_count, d_err, s, d_trace),
                    "trace launch");
         trace.resize(words);
         cuda_check(cudaMemcpyAsync(trace.data(), d_trace, words * sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "D2H");
         cuda_check(cudaMemcpyAsync(h_err_, d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
         cuda_check(cudaStreamSynchronize(s), "trace");
         check_error_flag();
         for (const NodeSpan& sp : p.spans) {
            if (sp.op->t == OpT::EMPTY || sp.op->t == OpT::FULL) continue;
            double popc = 0, cyc = 0;
            uint32_t live = 0;
            for (uint32_t tl = 0; tl < ntiles; ++tl) {
               const uint32_t* tr = trace.data() + static_cast<size_t>(tl) * nc * 2;
               if (tr[2 * sp.last] == 0) continue;  // tile without rows
               ++live;
               popc += tr[2 * sp.last + 1];
               for (uint32_t pc = sp.first; pc <= sp.last; ++pc) cyc += tr[2 * pc];
            }
            if (!live) continue;
            PlannerSample smp;
            op_features(*sp.op, ctx, smp.x.data());
            smp.log_sel = static_cast<float>(std::log(std::max(popc / rows, 1e-7)));
            smp.log_cost = static_cast<float>(std::log(std::max(cyc / live, 1.0)));
            smp.rule_log_sel = static_cast<float>(std::log(std::max(std::min(1.0, ctx.rule(*sp.op) / rows), 1e-7)));
            out.push_back(smp);
            ++added;
         }
      }
   } catch (...) {
      if (d_trace) cudaFree(d_trace);
      throw;
   }
   if (d_trace) cudaFree(d_trace);
   return added;
}

PlannerStats Engine::planner_train(uint32_t epochs, uint32_t batch, float lr, uint64_t seed) {
   std::lock_guard<std::mutex> lock(mu);
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   return planner_.train(epochs, batch, lr, seed);
}

void Engine::set_planner_mode(int mode) {
   if (mode != 0 && mode != 1) throw std::invalid_argument("planner mode must be 0 (rule-based) or 1 (learned)");
   if (mode == 1 && !(planner_.trained && planner_.accepted))
      throw std::invalid_argument("the learned planner is not trained or was not accepted against the rule-based ordering");
   use_learned_ = mode == 1;
}

std::vector<BatchQuery> Engine::plan_batch(const std::vector<std::string>& exprs, uint32_t threads, bool rule_only) {
   const uint32_t n = static_cast<uint32_t>(exprs.size());
   // threads == 0: the engine's persistent workers; otherwise that many threads of their own
   auto each = [&](auto&& fn) {
      if (threads == 0) plan_pool_.run(n, fn);
      else parallel_for(n, threads, fn);
   };
   using clk = std::chrono::steady_clock;
   auto since = [](clk::time_point a) { return std::chrono::duration<double, std::milli>(clk::now() - a).count(); };
   auto t0 = clk::now();
   if (!use_learned_ || rule_only) {
      std::vector<BatchQuery> qs(n);
      const Estimator est = rule_estimator(table_);
      LowerOptions lo;
      lo.rows = table_.n_rows;
      each([&](uint32_t i) { qs[i].prog = plan_filter(exprs[i], table_, &est, lo, nullptr); });
      batch_times.compile_ms += since(t0);
      return qs;
   }
   LearnedPlans lp;
   learned_compile(exprs, threads, lp);
   std::vector<uint32_t> all(n);
   for (uint32_t i = 0; i < n; ++i) all[i] = i;
   return learned_lower(lp, all, threads);
}

// Learned planning, step 1: compile and featurise every expression, run the network once over every
// operator node (rows staged in pinned memory, each query's nodes at its own offset) and keep each
// query's estimates per node and its predicted cost.
void Engine::learned_compile(const std::vector<std::string>& exprs, uint32_t threads, LearnedPlans& lp) {
   const uint32_t n = static_cast<uint32_t>(exprs.size());
   auto each = [&](auto&& fn) {
      if (threads == 0) plan_pool_.run(n, fn);
      else parallel_for(n, threads, fn);
   };
   using clk = std::chrono::steady_clock;
   auto since = [](clk::time_point a) { return std::chrono::duration<double, std::milli>(clk::now() - a).count(); };
   auto t0 = clk::now();
   const FeatureContext& ctx = fctx();
   lp.ops.clear();
   lp.ops.resize(n);
   lp.est.assign(n, {});
   lp.cost.assign(n, 0.0);
   std::vector<std::vector<const Op*>> qnodes(n);
   std::vector<std::vector<std::array<float, PLAN_FEATURES>>> qx(n);
   each([&](uint32_t i) {
      lp.ops[i] = compile_filter(exprs[i], table_);
      tree_features(*lp.ops[i], ctx, qnodes[i], qx[i]);
   });
   batch_times.compile_ms += since(t0);
   t0 = clk::now();
   // network rows: every query's root (its predicted cost) and the nodes whose rule estimate is not
   // exact (index scans keep their exact rule estimate and need no inference)
   std::vector<uint32_t> base(n + 1, 0);  // query i's rows are base[i] .. base[i + 1]
   std::vector<std::vector<uint32_t>> row_of(n);
   each([&](uint32_t i) {
      row_of[i].assign(qnodes[i].size(), UINT32_MAX);
      uint32_t r = 0;
      for (uint32_t k = 0; k < qnodes[i].size(); ++k)
         if (k == 0 || !exact_by_rule(qx[i][k].data())) row_of[i][k] = r++;
      base[i + 1] = r;
   });
   for (uint32_t i = 0; i < n; ++i) base[i + 1] += base[i];
   const uint32_t total = base[n];
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   float* X = planner_.net.staged_input(total);
   each([&](uint32_t i) {
      for (uint32_t k = 0; k < qnodes[i].size(); ++k)
         if (row_of[i][k] != UINT32_MAX)
            planner_.normalize(qx[i][k].data(), X + static_cast<size_t>(base[i] + row_of[i][k]) * PLAN_FEATURES);
   });
   const float* Y = total ? planner_.net.predict_staged(total) : nullptr;
   batch_times.predict_ms += since(t0);
   t0 = clk::now();
   const double rows = std::max(1u, table_.n_rows);
   const float no_output[2] = {0.0f, 0.0f};  // exact nodes: the rule estimate, no network output read
   each([&](uint32_t i) {
      // (node, estimated rows) sorted by node for lookup while lowering
      auto& est = lp.est[i];
      est.resize(qnodes[i].size());
      for (uint32_t k = 0; k < qnodes[i].size(); ++k) {
         const float* y = row_of[i][k] != UINT32_MAX ? Y + 2 * static_cast<size_t>(base[i] + row_of[i][k]) : no_output;
         const double sel = planner_.selectivity_of(qx[i][k].data(), y);
         est[k] = {qnodes[i][k], std::isfinite(sel) ? sel * rows : -1.0};
      }
      const double c = qnodes[i].empty() ? 0.0 : planner_.cost_of(Y + 2 * static_cast<size_t>(base[i]));
      lp.cost[i] = std::isfinite(c) ? c : 0.0;
      std::sort(est.begin(), est.end());
      std::vector<const Op*>().swap(qnodes[i]);
      std::vector<std::array<float, PLAN_FEATURES>>().swap(qx[i]);
   });
   batch_times.lower_ms += since(t0);
}

// Learned planning, step 2: lowers the queries `idx` of a learned_compile with their estimates and
// frees their trees (in parallel: a serial teardown of every tree costs as much as the planning).
std::vector<BatchQuery> Engine::learned_lower(LearnedPlans& lp, const std::vector<uint32_t>& idx, uint32_t threads) {
   const uint32_t n = static_cast<uint32_t>(idx.size());
   std::vector<BatchQuery> qs(n);
   auto each = [&](auto&& fn) {
      if (threads == 0) plan_pool_.run(n, fn);
      else parallel_for(n, threads, fn);
   };
   using clk = std::chrono::steady_clock;
   const auto t0 = clk::now();
   const FeatureContext& ctx = fctx();
   each([&](uint32_t j) {
      const uint32_t i = idx[j];
      const auto& est = lp.est[i];
      const Estimator learned = [&](const Op& op) -> double {
         const auto it = std::lower_bound(est.begin(), est.end(), std::make_pair(&op, -2.0));
         if (it != est.end() && it->first == &op && it->second >= 0) return it->second;
         return ctx.rule(op);  // the rule where the network has no answer
      };
      LowerOptions lo;
      lo.rows = table_.n_rows;
      qs[j].prog = lower(*lp.ops[i], learned, lo);
      qs[j].cost = lp.cost[i];
      lp.ops[i].reset();
      std::vector<std::pair<const Op*, double>>().swap(lp.est[i]);
   });
   batch_times.lower_ms += std::chrono::duration<double, std::milli>(clk::now() - t0).count();
   return qs;
}

void Engine::aggregate(const Program& p, const std::vector<AggSpec>& spec, std::vector<int32_t>& groups,
                       std::vector<uint64_t>& counts, uint64_t* filter_count, cudaStream_t stream) {
   if (spec.empty() || spec.size() > 8) throw std::invalid_argument("aggregation needs 1 to 8 dimensions");
   std::vector<AggDim> dims(spec.size());
   for (size_t d = 0; d < spec.size(); ++d) {
      const AggSpec& x = spec[d];
      AggDim& a = dims[d];
      a.kind = x.kind;
      a.col = x.col;
      a.pos = x.pos;
      if (x.kind == AGG_SEQUENCE) {
         if (x.col >= table_.seq.size()) throw IllegalQuery("no such sequence column");
         if (x.pos >= table_.seq[x.col].L) throw IllegalQuery("position out of range for the sequence column");
         a.ngroups = view_.seq[x.col].nsym + 1;
         a.ids = a.rank = nullptr;
      } else if (x.kind == AGG_DICTIONARY) {
         if (x.col >= table_.dict.size()) throw IllegalQuery("no such dictionary column");
         a.ngroups = static_cast<uint32_t>(table_.dict[x.col].values.size()) + 1;
         a.ids = d_dict_ids_[x.col];
         a.rank = d_dict_rank_[x.col];
      } else {
         throw std::invalid_argument("dimension kind must be 0 (sequence position) or 1 (dictionary column)");
      }
   }
   uint64_t keys = 1;  // dimension 0 most significant: key order = the reference's depth-first order
   for (size_t d = dims.size(); d-- > 0;) {
      dims[d].stride = keys;
      keys *= dims[d].ngroups;
      if (keys > AGG_MAX_KEYS) throw std::invalid_argument("aggregation: more than 2^26 group combinations");
   }
   std::lock_guard<std::mutex> lock(mu);
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   if (!stream) stream = stream_;
   const uint64_t nblocks = (keys + AGG_BLOCK - 1) / AGG_BLOCK;
   grow_device(d_agg_dims_, agg_dims_cap_, 8);
   grow_device(d_agg_counters_, agg_counters_cap_, keys);
   grow_device(d_agg_blocks_, agg_blocks_cap_, nblocks);
   cuda_check(cudaMemcpyAsync(d_agg_dims_, dims.data(), dims.size() * sizeof(AggDim), cudaMemcpyHostToDevice, stream),
              "H2D");
   upload_program(p, d_code, stream);
   cuda_check(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream), "memset");
   cuda_check(cudaMemsetAsync(d_agg_counters_, 0, keys * sizeof(uint32_t), stream), "memset");
   launch_count(d_code, p, d_count, d_filter, stream);
   launch_agg_keys(d_table_, nchunks(), d_filter, d_agg_dims_, static_cast<uint32_t>(dims.size()), d_agg_counters_,
                   stream);
   launch_agg_nonzero(d_agg_counters_, keys, d_agg_blocks_, stream);
   cuda_check(cudaGetLastError(), "aggregation launch");
   std::vector<uint32_t> block(nblocks);
   cuda_check(cudaMemcpyAsync(block.data(), d_agg_blocks_, nblocks * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream),
              "D2H");
   cuda_check(cudaMemcpyAsync(h_count_, d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "D2H");
   cuda_check(cudaMemcpyAsync(h_err_, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "D2H");
   cuda_check(cudaStreamSynchronize(stream), "aggregation");
   check_error_flag();
   uint64_t total = 0;
   for (uint64_t b = 0; b < nblocks; ++b) {
      const uint32_t n = block[b];
      block[b] = static_cast<uint32_t>(total);
      total += n;
   }
   std::vector<AggCount> out(total);
   if (total) {
      grow_device(d_agg_out_, agg_out_cap_, total);
      cuda_check(cudaMemcpyAsync(d_agg_blocks_, block.data(), nblocks * sizeof(uint32_t), cudaMemcpyHostToDevice, stream),
                 "H2D");
      launch_agg_write(d_agg_counters_, keys, d_agg_blocks_, d_agg_out_, stream);
      cuda_check(cudaGetLastError(), "aggregation launch");
      cuda_check(cudaMemcpyAsync(out.data(), d_agg_out_, total * sizeof(AggCount), cudaMemcpyDeviceToHost, stream), "D2H");
      cuda_check(cudaStreamSynchronize(stream), "aggregation");
   }
   groups.resize(total * dims.size());
   counts.resize(total);
   for (uint64_t i = 0; i < total; ++i) {
      counts[i] = out[i].count;
      for (size_t d = 0; d < dims.size(); ++d) {
         const uint32_t g = static_cast<uint32_t>((out[i].key / dims[d].stride) % dims[d].ngroups);
         int32_t v = -1;  // the null group is the last one
         if (g + 1 < dims[d].ngroups) v = dims[d].kind == AGG_SEQUENCE ? static_cast<int32_t>(g)
                                                                       : static_cast<int32_t>(dict_by_rank_[dims[d].col][g]);
         groups[i * dims.size() + d] = v;
      }
   }
   if (filter_count) *filter_count = *h_count_;
}

}  // namespace rhygpu
