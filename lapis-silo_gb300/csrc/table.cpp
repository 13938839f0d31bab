// Ingestion of a raw table into the storage image (see table.h for the layout).
#include "table.h"
#include "table_build.h"

#include <algorithm>
#include <cstring>
#include <numeric>

#include "util.h"

namespace rhygpu {

uint64_t ContainerSet::payload_bytes() const {
   uint64_t b = 0;
   for (const auto& c : ctrs) {
      if (c.type == CT_BITSET) {
         b += 8192;
      } else if (c.type == CT_RUN) {
         b += 4ull * c.nruns;
      } else {
         b += 2ull * (c.card_m1 + 1u);
      }
   }
   return b;
}

int TableImage::find_seq(const std::string& name) const {
   for (size_t i = 0; i < seq.size(); ++i)
      if (seq[i].name == name) return static_cast<int>(i);
   return -1;
}
int TableImage::find_dict(const std::string& name) const {
   for (size_t i = 0; i < dict.size(); ++i)
      if (dict[i].name == name) return static_cast<int>(i);
   return -1;
}
int TableImage::find_date(const std::string& name) const {
   for (size_t i = 0; i < date.size(); ++i)
      if (date[i].name == name) return static_cast<int>(i);
   return -1;
}

namespace {

// key layout: key << 21 | sym << 16 | row_in_chunk
inline uint64_t pack(uint64_t key, uint32_t sym, uint32_t row) { return (key << 21) | (uint64_t(sym) << 16) | row; }
inline uint32_t key_of(uint64_t k) { return static_cast<uint32_t>(k >> 21); }
inline uint32_t sym_of(uint64_t k) { return static_cast<uint32_t>((k >> 16) & 31); }
inline uint32_t row_of(uint64_t k) { return static_cast<uint32_t>(k & 0xFFFF); }

struct ChunkContainers {
   std::vector<CtrDesc> ctrs;
   std::vector<uint16_t> payload;
};

// Encodes sorted (key, sym, row) entries of one chunk as containers. Array payloads come first and
// back to back in descriptor order (a warp can stream the arrays of consecutive descriptors as one
// contiguous range); bitsets (16-byte aligned) and runs follow them.
void encode_chunk(const std::vector<uint64_t>& keys, uint16_t v, ChunkContainers& out) {
   out.ctrs.clear();
   out.payload.clear();
   std::vector<uint16_t> other;            // bitset and run payloads
   std::vector<size_t> other_ctrs;         // descriptors whose payload offset is into `other`
   size_t i = 0;
   std::vector<uint16_t> rows;
   while (i < keys.size()) {
      const uint64_t group = keys[i] >> 16;
      rows.clear();
      size_t j = i;
      while (j < keys.size() && (keys[j] >> 16) == group) rows.push_back(static_cast<uint16_t>(row_of(keys[j++])));
      rows.erase(std::unique(rows.begin(), rows.end()), rows.end());
      const uint32_t card = static_cast<uint32_t>(rows.size());
      uint32_t nruns = 1;
      for (size_t k = 1; k < rows.size(); ++k) nruns += (rows[k] != rows[k - 1] + 1);
      const uint32_t base_bytes = card <= 4096 ? 2 + 2 * card : 8192;
      const uint32_t run_bytes = 2 + 4 * nruns;
      CtrDesc d{};
      d.key = key_of(keys[i]);
      d.v = v;
      d.sym = static_cast<uint8_t>(sym_of(keys[i]));
      d.card_m1 = static_cast<uint16_t>(card - 1);
      if (run_bytes < base_bytes) {
         d.type = CT_RUN;
         d.nruns = static_cast<uint16_t>(nruns);
         d.payload = static_cast<uint32_t>(other.size());
         size_t k = 0;
         while (k < rows.size()) {
            size_t e = k;
            while (e + 1 < rows.size() && rows[e + 1] == rows[e] + 1) ++e;
            other.push_back(rows[k]);
            other.push_back(static_cast<uint16_t>(e - k));
            k = e + 1;
         }
         other_ctrs.push_back(out.ctrs.size());
      } else if (card <= 4096) {
         d.type = CT_ARRAY;
         d.payload = static_cast<uint32_t>(out.payload.size());
         out.payload.insert(out.payload.end(), rows.begin(), rows.end());
      } else {
         d.type = CT_BITSET;
         while (other.size() % 8) other.push_back(0);
         d.payload = static_cast<uint32_t>(other.size());
         other.resize(other.size() + 4096, 0);
         uint16_t* bits = other.data() + d.payload;
         for (uint16_t r : rows) bits[r >> 4] |= static_cast<uint16_t>(1u << (r & 15));
         other_ctrs.push_back(out.ctrs.size());
      }
      out.ctrs.push_back(d);
      i = j;
   }
   while (out.payload.size() % 8) out.payload.push_back(0);
   const uint32_t base = static_cast<uint32_t>(out.payload.size());
   out.payload.insert(out.payload.end(), other.begin(), other.end());
   for (size_t k : other_ctrs) out.ctrs[k].payload += base;
}

// Concatenates per-chunk containers (chunk order) and builds the (v, key) offset table.
void assemble(std::vector<ChunkContainers>& chunks, uint32_t nkeys, ContainerSet& cs) {
   size_t nctr = 0, npay = 0;
   for (const auto& c : chunks) {
      nctr += c.ctrs.size();
      npay += c.payload.size() + 8;
   }
   cs.ctrs.reserve(nctr);
   cs.payload.reserve(npay);
   cs.nkeys = nkeys;
   for (auto& c : chunks) {
      while (cs.payload.size() % 8) cs.payload.push_back(0);
      const uint32_t base = static_cast<uint32_t>(cs.payload.size());
      if (cs.payload.size() + c.payload.size() > 0xFFFFFFFFull) throw std::runtime_error("payload arena exceeds 2^32 entries");
      cs.payload.insert(cs.payload.end(), c.payload.begin(), c.payload.end());
      for (auto d : c.ctrs) {
         d.payload += base;
         cs.ctrs.push_back(d);
      }
      c = ChunkContainers{};
   }
   // pad to whole 16-byte words plus one spare word: kernels read array payloads with aligned
   // 16-byte loads that may cover up to seven u16 past a container's last element
   while (cs.payload.size() % 8) cs.payload.push_back(0);
   cs.payload.insert(cs.payload.end(), 8, 0);
   finish_container_set(cs, static_cast<uint32_t>(chunks.size()));
}

}  // namespace

void finish_container_set(ContainerSet& cs, uint32_t nchunks) {
   const uint32_t nkeys = cs.nkeys;
   cs.stats.assign(static_cast<size_t>(nkeys) * STAT_SYMS, KeyStats{});
   for (const auto& d : cs.ctrs) {
      KeyStats& st = cs.stats[static_cast<size_t>(d.key) * STAT_SYMS + d.sym];
      st.card += d.card_m1 + 1u;
      ++st.nctr;
      st.nbits += d.type == CT_BITSET;
   }
   const uint64_t nslots = static_cast<uint64_t>(nchunks) * nkeys;
   cs.off.assign(nslots + 1, 0);
   for (const auto& d : cs.ctrs) cs.off[static_cast<uint64_t>(d.v) * nkeys + d.key + 1]++;
   for (uint64_t i = 0; i < nslots; ++i) cs.off[i + 1] += cs.off[i];
}

namespace {

void ingest_chunk(const RawSeqColumn& raw, const Alphabet& A, const std::vector<uint8_t>& ref_sym, uint32_t L,
                  uint32_t v, uint32_t size, ChunkRows& out) {
   out.nr_off.assign(1, 0);
   const uint32_t missing = A.missing;
   struct Run {
      uint32_t pos, len, sym;
   };
   std::vector<Run> runs;
   // intervals where the reference holds the missing symbol (empty for ordinary references)
   std::vector<std::pair<uint32_t, uint32_t>> ref_missing;
   for (uint32_t p = 0; p < L; ++p) {
      if (ref_sym[p] != missing) continue;
      if (!ref_missing.empty() && ref_missing.back().second == p) ref_missing.back().second = p + 1;
      else ref_missing.emplace_back(p, p + 1);
   }
   for (uint32_t r = 0; r < size; ++r) {
      const uint32_t row = v * CHUNK_ROWS + r;
      if (raw.is_null[row]) {
         out.nulls.push_back(row);
         out.exc.push_back({r, 0, 0, 0});
         out.nr_off.push_back(static_cast<uint32_t>(out.nr_s.size()));
         continue;
      }
      // The row's runs as (pos, len, symbol); positions where the reference itself holds the
      // missing symbol are missing in the row too unless a run overrides them.
      runs.clear();
      const uint64_t b = raw.row_off[row], e = raw.row_off[row + 1];
      size_t j = 0;
      // adds the reference-missing positions inside the gap [a, z) between runs
      auto fill_gap = [&](uint32_t a, uint32_t z) {
         while (j < ref_missing.size() && ref_missing[j].second <= a) ++j;
         for (size_t t = j; t < ref_missing.size() && ref_missing[t].first < z; ++t) {
            const uint32_t lo = std::max(a, ref_missing[t].first), hi = std::min(z, ref_missing[t].second);
            if (lo < hi) runs.push_back({lo, hi - lo, missing});
         }
      };
      uint32_t cursor = 0;
      for (uint64_t k = b; k < e; ++k) {
         const int s = A.sym(raw.run_char[k]);
         if (s < 0)  // the reference's message (aligned_sequence.cpp:38-41), then where
            throw std::invalid_argument(std::string("illegal character '") + raw.run_char[k] + "' at position " +
                                        std::to_string(raw.run_pos[k]) + " in the input sequence (column " + raw.name +
                                        ", row " + std::to_string(row) + ")");
         const uint32_t p0 = raw.run_pos[k], len = raw.run_len[k];
         if (len == 0 || p0 < cursor || static_cast<uint64_t>(p0) + len > L)
            throw std::invalid_argument("runs must be sorted, non-overlapping and inside the genome in column " + raw.name);
         if (!ref_missing.empty()) fill_gap(cursor, p0);
         runs.push_back({p0, len, static_cast<uint32_t>(s)});
         cursor = p0 + len;
      }
      if (!ref_missing.empty()) fill_gap(cursor, L);
      // Leading and trailing missing symbols are trimmed into the covered region
      // (reference: src/rhydb/common/aligned_sequence.cpp:89-120).
      uint32_t start = 0;
      size_t k = 0, kb = runs.size();
      while (k < kb && runs[k].pos == start && runs[k].sym == missing) {
         start = runs[k].pos + runs[k].len;
         ++k;
      }
      uint32_t end = L;
      while (kb > k && runs[kb - 1].pos + runs[kb - 1].len == end && runs[kb - 1].sym == missing) {
         end = runs[kb - 1].pos;
         --kb;
      }
      if (start >= end) {
         // Fully missing sequence: empty covered region, nothing recorded.
         out.exc.push_back({r, 0, 0, 0});
         out.nr_off.push_back(static_cast<uint32_t>(out.nr_s.size()));
         continue;
      }
      if (start != 0 || end != L) out.exc.push_back({r, start, end, 0});
      for (size_t q = k; q < kb; ++q) {
         const Run& run = runs[q];
         if (run.sym == missing) {
            if (!out.nr_s.empty() && out.nr_off.back() < out.nr_s.size() && out.nr_e.back() == run.pos) {
               out.nr_e.back() = run.pos + run.len;  // adjacent missing runs form one interval
            } else {
               out.nr_s.push_back(run.pos);
               out.nr_e.push_back(run.pos + run.len);
            }
            continue;
         }
         for (uint32_t p = run.pos; p < run.pos + run.len; ++p) {
            if (run.sym != ref_sym[p]) out.keys.push_back(pack(p, run.sym, r));
         }
      }
      out.nr_off.push_back(static_cast<uint32_t>(out.nr_s.size()));
   }
   std::sort(out.keys.begin(), out.keys.end());
}

// Start / end events of the missing intervals, counting-sorted by (block, position) with rows in
// increasing order inside each bucket, and the coverage boundary events. An interval [s, e)
// contributes +1 at s and -1 at e to the per-position difference array: its start event lives in
// block s / NBLOCK at offset s % NBLOCK, its end event in block (e - 1) / NBLOCK at offset 1..NBLOCK.
void build_mutation_events(SeqColumnImage& col, const std::vector<ChunkRows>& chunks,
                           const std::vector<uint32_t>& chunk_sizes) {
   const uint32_t nchunks = static_cast<uint32_t>(chunk_sizes.size());
   if (nchunks > MAX_EVENT_CHUNKS)
      throw std::invalid_argument("a partition holds at most " + std::to_string(MAX_EVENT_CHUNKS) + " chunks (" +
                                  std::to_string(MAX_EVENT_CHUNKS * CHUNK_ROWS) + " rows)");
   const uint32_t W = NBLOCK + 1;  // positions 0..NBLOCK inside a block
   const size_t nbuckets = static_cast<size_t>(col.nblocks) * W;
   std::vector<uint32_t> cs(nbuckets + 1, 0), ce(nbuckets + 1, 0);
   auto each = [&](auto&& fn) {
      for (uint32_t v = 0; v < nchunks; ++v) {
         const ChunkRows& c = chunks[v];
         for (uint32_t r = 0; r < chunk_sizes[v]; ++r) {
            for (uint32_t q = c.nr_off[r]; q < c.nr_off[r + 1]; ++q) {
               const uint32_t s = c.nr_s[q], e = c.nr_e[q];
               const uint32_t sb = s / NBLOCK, eb = (e - 1) / NBLOCK;
               fn((v << 16) | r, sb, s - sb * NBLOCK, eb, e - eb * NBLOCK);
            }
         }
      }
   };
   each([&](uint32_t, uint32_t sb, uint32_t lo, uint32_t eb, uint32_t hi) {
      cs[static_cast<size_t>(sb) * W + lo + 1]++;
      ce[static_cast<size_t>(eb) * W + hi + 1]++;
   });
   for (size_t i = 0; i < nbuckets; ++i) {
      cs[i + 1] += cs[i];
      ce[i + 1] += ce[i];
   }
   col.mstart.resize(cs[nbuckets]);
   col.mend.resize(ce[nbuckets]);
   col.mstart_off.resize(col.nblocks + 1);
   col.mend_off.resize(col.nblocks + 1);
   for (uint32_t b = 0; b <= col.nblocks; ++b) {
      col.mstart_off[b] = cs[static_cast<size_t>(b) * W];
      col.mend_off[b] = ce[static_cast<size_t>(b) * W];
   }
   each([&](uint32_t g, uint32_t sb, uint32_t lo, uint32_t eb, uint32_t hi) {
      col.mstart[cs[static_cast<size_t>(sb) * W + lo]++] = (g << 8) | lo;
      col.mend[ce[static_cast<size_t>(eb) * W + hi]++] = (g << 8) | hi;
   });
   // coverage boundaries
   for (uint32_t v = 0; v < nchunks; ++v) {
      for (const CovExc& x : chunks[v].exc) {
         const uint32_t g = (v << 16) | x.row;
         if (x.start > 0) col.cstart.push_back({g, x.start});
         if (x.end < col.L) col.cend.push_back({g, x.end});
      }
   }
   auto by_pos = [](const CovEvent& a, const CovEvent& b) { return a.pos != b.pos ? a.pos < b.pos : a.row < b.row; };
   std::sort(col.cstart.begin(), col.cstart.end(), by_pos);
   std::sort(col.cend.begin(), col.cend.end(), by_pos);
}

// The row index (see SeqColumnImage::hrow_off): every entry the dense passes would count for a row,
// from the same containers, coverage exceptions and missing intervals.
void build_row_index(SeqColumnImage& col, const std::vector<uint32_t>& chunk_sizes, uint32_t threads) {
   const uint32_t nchunks = static_cast<uint32_t>(chunk_sizes.size());
   const ContainerSet& V = col.vertical;
   const uint32_t nkeys = V.nkeys, L = col.L;
   if (alphabet(col.kind).count > ROW_COV_START) throw std::logic_error("row index: too many symbols");
   auto for_chunk = [&](uint32_t v, auto&& emit) {  // emit(row within chunk, entry)
      for (uint32_t i = V.off[static_cast<size_t>(v) * nkeys]; i < V.off[static_cast<size_t>(v + 1) * nkeys]; ++i) {
         const CtrDesc& d = V.ctrs[i];
         const uint32_t e = d.key << 5 | d.sym;
         const uint16_t* p = V.payload.data() + d.payload;
         if (d.type == CT_ARRAY) {
            for (uint32_t k = 0; k <= d.card_m1; ++k) emit(p[k], e);
         } else if (d.type == CT_BITSET) {
            for (uint32_t w = 0; w < CHUNK_WORDS; ++w) {
               uint32_t x = static_cast<uint32_t>(p[2 * w]) | static_cast<uint32_t>(p[2 * w + 1]) << 16;
               while (x) {
                  emit(32 * w + static_cast<uint32_t>(__builtin_ctz(x)), e);
                  x &= x - 1;
               }
            }
         } else {
            for (uint32_t k = 0; k < d.nruns; ++k)
               for (uint32_t r = p[2 * k]; r <= static_cast<uint32_t>(p[2 * k]) + p[2 * k + 1]; ++r) emit(r, e);
         }
      }
      for (uint32_t i = col.cov_exc_off[v]; i < col.cov_exc_off[v + 1]; ++i) {
         const CovExc& x = col.cov_exc[i];
         if (x.start > 0) emit(x.row, x.start << 5 | ROW_COV_START);
         if (x.end < L) emit(x.row, x.end << 5 | ROW_COV_END);
      }
      for (uint32_t r = 0; r < chunk_sizes[v]; ++r) {
         const size_t g = static_cast<size_t>(v) * CHUNK_ROWS + r;
         for (uint32_t q = col.nrow_off[g]; q < col.nrow_off[g + 1]; ++q) {
            emit(r, col.nrow_start[q] << 5 | ROW_MISS_START);
            emit(r, col.nrow_end[q] << 5 | ROW_MISS_END);
         }
      }
   };
   std::vector<uint32_t>& off = col.hrow_off;
   off.assign(static_cast<size_t>(nchunks) * CHUNK_ROWS + 1, 0);
   parallel_for(nchunks, threads, [&](uint32_t v) {
      uint32_t* o = off.data() + static_cast<size_t>(v) * CHUNK_ROWS + 1;
      for_chunk(v, [&](uint32_t r, uint32_t) { ++o[r]; });
   });
   uint64_t total = 0;
   for (size_t i = 1; i < off.size(); ++i) {
      total += off[i];
      if (total > 0xFFFFFFFFull) throw std::invalid_argument("row index: more than 2^32 entries in one column");
      off[i] = static_cast<uint32_t>(total);
   }
   col.hent.resize(total);
   parallel_for(nchunks, threads, [&](uint32_t v) {
      std::vector<uint32_t> at(off.begin() + static_cast<size_t>(v) * CHUNK_ROWS,
                               off.begin() + static_cast<size_t>(v + 1) * CHUNK_ROWS);
      for_chunk(v, [&](uint32_t r, uint32_t e) { col.hent[at[r]++] = e; });
   });
}

}  // namespace

void init_seq_column(const RawSeqColumn& raw, SeqColumnImage& col) {
   col.name = raw.name;
   col.kind = raw.kind;
   const Alphabet& A = alphabet(raw.kind);
   const uint32_t L = static_cast<uint32_t>(raw.reference.size());
   if (L == 0) throw std::invalid_argument("empty reference for column " + raw.name);
   col.L = L;
   col.reference = raw.reference;
   col.global_ref.resize(L);
   for (uint32_t p = 0; p < L; ++p) {
      const int s = A.sym(raw.reference[p]);
      if (s < 0) throw std::invalid_argument("illegal reference character in column " + raw.name);
      col.global_ref[p] = static_cast<uint8_t>(s);
   }
   col.local_ref = col.global_ref;
}

namespace {

SeqColumnImage build_seq_column(const RawSeqColumn& raw, const std::vector<uint32_t>& chunk_sizes, uint32_t threads) {
   SeqColumnImage col;
   init_seq_column(raw, col);
   const Alphabet& A = alphabet(raw.kind);
   const uint32_t L = col.L;
   const uint32_t nchunks = static_cast<uint32_t>(chunk_sizes.size());
   const uint32_t nsym = A.count;

   std::vector<ChunkRows> chunks(nchunks);
   parallel_for(nchunks, threads, [&](uint32_t v) { ingest_chunk(raw, A, col.global_ref, L, v, chunk_sizes[v], chunks[v]); });

   // ---- local reference adaptation (reference: sequence_column.cpp:158-195) ----
   std::vector<int64_t> diff(L + 1, 0);
   for (uint32_t v = 0; v < nchunks; ++v) {
      const ChunkRows& c = chunks[v];
      int64_t full_rows = chunk_sizes[v];
      for (const auto& x : c.exc) {
         --full_rows;
         if (x.start < x.end) {
            diff[x.start] += 1;
            diff[x.end] -= 1;
         }
      }
      diff[0] += full_rows;
      diff[L] -= full_rows;
      for (size_t i = 0; i < c.nr_s.size(); ++i) {
         diff[c.nr_s[i]] -= 1;
         diff[c.nr_e[i]] += 1;
      }
   }
   std::vector<uint64_t> coverage(L);
   int64_t run = 0;
   for (uint32_t p = 0; p < L; ++p) {
      run += diff[p];
      coverage[p] = static_cast<uint64_t>(run);
   }
   std::vector<uint32_t> counts(static_cast<size_t>(L) * nsym, 0);
   for (const auto& c : chunks) {
      for (uint64_t k : c.keys) counts[static_cast<size_t>(key_of(k)) * nsym + sym_of(k)]++;
   }
   struct Flip {
      uint32_t pos;
      uint8_t old_sym, new_sym;
   };
   std::vector<Flip> flips;
   for (uint32_t p = 0; p < L; ++p) {
      const uint32_t ref = col.local_ref[p];
      uint32_t ref_count = static_cast<uint32_t>(coverage[p]);
      for (uint32_t s = 0; s < nsym; ++s) ref_count -= counts[static_cast<size_t>(p) * nsym + s];
      uint32_t best = ref, best_count = ref_count;
      for (uint32_t s = 0; s < nsym; ++s) {
         if (s == ref) continue;
         const uint32_t c = counts[static_cast<size_t>(p) * nsym + s];
         if (c > best_count) {
            best = s;
            best_count = c;
         }
      }
      if (best != ref) flips.push_back({p, static_cast<uint8_t>(ref), static_cast<uint8_t>(best)});
   }
   counts.clear();
   counts.shrink_to_fit();
   col.flipped_positions = static_cast<uint32_t>(flips.size());
   if (!flips.empty()) {
      parallel_for(nchunks, threads, [&](uint32_t v) {
         ChunkRows& c = chunks[v];
         const uint32_t size = chunk_sizes[v];
         std::vector<uint8_t> covered(size);
         std::vector<uint64_t> added;
         std::vector<uint8_t> is_flip_pos_new;  // per key: drop?
         for (const Flip& f : flips) {
            // rows covered at f.pos
            std::fill(covered.begin(), covered.end(), 1);
            for (const auto& x : c.exc) covered[x.row] = (x.start <= f.pos && f.pos < x.end) ? 1 : 0;
            for (uint32_t r = 0; r < size; ++r) {
               if (!covered[r]) continue;
               for (uint32_t q = c.nr_off[r]; q < c.nr_off[r + 1]; ++q) {
                  if (c.nr_s[q] <= f.pos && f.pos < c.nr_e[q]) {
                     covered[r] = 0;
                     break;
                  }
               }
            }
            auto lo = std::lower_bound(c.keys.begin(), c.keys.end(), pack(f.pos, 0, 0));
            auto hi = std::lower_bound(c.keys.begin(), c.keys.end(), pack(f.pos + 1, 0, 0));
            for (auto it = lo; it != hi; ++it) covered[row_of(*it)] = 0;
            for (uint32_t r = 0; r < size; ++r)
               if (covered[r]) added.push_back(pack(f.pos, f.old_sym, r));
         }
         // drop the new reference symbol's entries at flipped positions
         std::vector<uint64_t> kept;
         kept.reserve(c.keys.size() + added.size());
         size_t fi = 0;
         for (uint64_t k : c.keys) {
            const uint32_t p = key_of(k);
            while (fi < flips.size() && flips[fi].pos < p) ++fi;
            if (fi < flips.size() && flips[fi].pos == p && sym_of(k) == flips[fi].new_sym) continue;
            kept.push_back(k);
         }
         kept.insert(kept.end(), added.begin(), added.end());
         std::sort(kept.begin(), kept.end());
         c.keys.swap(kept);
      });
      for (const Flip& f : flips) col.local_ref[f.pos] = f.new_sym;
   }

   // ---- containers ----
   std::vector<ChunkContainers> enc(nchunks);
   parallel_for(nchunks, threads, [&](uint32_t v) {
      encode_chunk(chunks[v].keys, static_cast<uint16_t>(v), enc[v]);
      std::vector<uint64_t>().swap(chunks[v].keys);
   });
   assemble(enc, L, col.vertical);
   finish_seq_column(col, chunks, chunk_sizes, threads);
   return col;
}

}  // namespace

void finish_seq_column(SeqColumnImage& col, const std::vector<ChunkRows>& chunks, const std::vector<uint32_t>& chunk_sizes,
                       uint32_t threads) {
   const uint32_t nchunks = static_cast<uint32_t>(chunk_sizes.size());
   const uint32_t L = col.L;
   // ---- coverage, nulls, missing intervals ----
   col.cov_exc_off.assign(1, 0);
   for (uint32_t v = 0; v < nchunks; ++v) {
      const ChunkRows& c = chunks[v];
      col.cov_exc.insert(col.cov_exc.end(), c.exc.begin(), c.exc.end());
      col.cov_exc_off.push_back(static_cast<uint32_t>(col.cov_exc.size()));
      col.null_rows.insert(col.null_rows.end(), c.nulls.begin(), c.nulls.end());
   }
   col.nrow_off.assign(static_cast<size_t>(nchunks) * CHUNK_ROWS + 1, 0);
   for (uint32_t v = 0; v < nchunks; ++v) {
      const ChunkRows& c = chunks[v];
      const uint32_t base = static_cast<uint32_t>(col.nrow_start.size());
      for (uint32_t r = 0; r < CHUNK_ROWS; ++r) {
         const uint32_t n = r < chunk_sizes[v] ? c.nr_off[r + 1] : c.nr_off[chunk_sizes[v]];
         col.nrow_off[static_cast<size_t>(v) * CHUNK_ROWS + r + 1] = base + n;
      }
      col.nrow_start.insert(col.nrow_start.end(), c.nr_s.begin(), c.nr_s.end());
      col.nrow_end.insert(col.nrow_end.end(), c.nr_e.begin(), c.nr_e.end());
   }
   col.nblocks = (L + NBLOCK - 1) / NBLOCK;
   const size_t nbuckets = static_cast<size_t>(col.nblocks) * nchunks;
   col.nblk_off.assign(nbuckets + 1, 0);
   for (uint32_t v = 0; v < nchunks; ++v) {
      const ChunkRows& c = chunks[v];
      for (size_t i = 0; i < c.nr_s.size(); ++i) {
         for (uint32_t b = c.nr_s[i] / NBLOCK; b <= (c.nr_e[i] - 1) / NBLOCK; ++b)
            col.nblk_off[static_cast<size_t>(b) * nchunks + v + 1]++;
      }
   }
   for (size_t i = 0; i < nbuckets; ++i) col.nblk_off[i + 1] += col.nblk_off[i];
   col.nblk.resize(col.nblk_off[nbuckets]);
   std::vector<uint32_t> fill(col.nblk_off.begin(), col.nblk_off.end() - 1);
   for (uint32_t v = 0; v < nchunks; ++v) {
      const ChunkRows& c = chunks[v];
      for (uint32_t r = 0; r < chunk_sizes[v]; ++r) {
         for (uint32_t q = c.nr_off[r]; q < c.nr_off[r + 1]; ++q) {
            const uint32_t s = c.nr_s[q], e = c.nr_e[q];
            for (uint32_t b = s / NBLOCK; b <= (e - 1) / NBLOCK; ++b) {
               const uint32_t bs = b * NBLOCK;
               NRunEntry en;
               en.row = (v << 16) | r;
               en.lo = static_cast<uint16_t>(std::max(s, bs) - bs);
               en.hi = static_cast<uint16_t>(std::min(e, bs + NBLOCK) - bs);
               col.nblk[fill[static_cast<size_t>(b) * nchunks + v]++] = en;
            }
         }
      }
   }
   // tile row-range offsets into both sorted lists
   auto toff = [](uint32_t* out, uint32_t b, uint32_t e, auto&& row_of) {
      uint32_t i = b;
      for (uint32_t k = 0; k < TOFF_N; ++k) {
         while (i < e && row_of(i) < k * TOFF_ROWS) ++i;
         out[k] = i;
      }
   };
   col.exc_toff.resize(static_cast<size_t>(nchunks) * TOFF_N);
   for (uint32_t v = 0; v < nchunks; ++v)
      toff(&col.exc_toff[static_cast<size_t>(v) * TOFF_N], col.cov_exc_off[v], col.cov_exc_off[v + 1],
           [&](uint32_t i) { return col.cov_exc[i].row; });
   col.nblk_toff.resize(nbuckets * TOFF_N);
   for (size_t bv = 0; bv < nbuckets; ++bv)
      toff(&col.nblk_toff[bv * TOFF_N], col.nblk_off[bv], col.nblk_off[bv + 1],
           [&](uint32_t i) { return col.nblk[i].row & 0xFFFFu; });
   build_mutation_events(col, chunks, chunk_sizes);
   build_row_index(col, chunk_sizes, threads);
}

namespace {

DictColumnImage build_dict_column(const RawDictColumn& raw, const std::vector<uint32_t>& chunk_sizes, uint32_t threads) {
   DictColumnImage col;
   col.name = raw.name;
   col.values = raw.values;
   for (uint32_t i = 0; i < raw.values.size(); ++i) col.index.emplace(raw.values[i], i);
   const uint32_t nchunks = static_cast<uint32_t>(chunk_sizes.size());
   const uint32_t nvalues = static_cast<uint32_t>(raw.values.size());
   std::vector<ChunkContainers> enc(nchunks);
   parallel_for(nchunks, threads, [&](uint32_t v) {
      std::vector<uint64_t> keys;
      for (uint32_t r = 0; r < chunk_sizes[v]; ++r) {
         const uint32_t id = raw.ids[v * CHUNK_ROWS + r];
         if (id == UINT32_MAX) continue;
         if (id >= nvalues) throw std::invalid_argument("dictionary id out of range in column " + raw.name);
         keys.push_back(pack(id, 0, r));
      }
      std::sort(keys.begin(), keys.end());
      encode_chunk(keys, static_cast<uint16_t>(v), enc[v]);
   });
   assemble(enc, std::max(1u, nvalues), col.inverted);
   return col;
}

}  // namespace

void build_table_frame(const RawTable& raw, TableImage& t) {
   t.n_rows = raw.n_rows;
   if (raw.n_rows == 0) throw std::invalid_argument("a partition needs at least one row");
   for (uint32_t left = raw.n_rows; left > 0;) {
      const uint32_t s = std::min(left, CHUNK_ROWS);
      t.chunk_sizes.push_back(s);
      left -= s;
   }
   if (t.chunk_sizes.size() >= 65535) throw std::invalid_argument("too many chunks");
   for (const auto& c : raw.seq)
      if (c.is_null.size() != raw.n_rows || c.row_off.size() != raw.n_rows + 1ull)
         throw std::invalid_argument("row count mismatch in column " + c.name);
}

void build_metadata_columns(const RawTable& raw, TableImage& t, uint32_t threads) {
   for (const auto& c : raw.dict) {
      if (c.ids.size() != raw.n_rows) throw std::invalid_argument("row count mismatch in column " + c.name);
      t.dict.push_back(build_dict_column(c, t.chunk_sizes, threads));
   }
   for (const auto& c : raw.date) {
      if (c.days.size() != raw.n_rows) throw std::invalid_argument("row count mismatch in column " + c.name);
      DateColumnImage d;
      d.name = c.name;
      d.days.assign(static_cast<size_t>(t.nchunks()) * CHUNK_ROWS, INT32_MIN);
      for (uint32_t i = 0; i < raw.n_rows; ++i) d.days[i] = c.days[i];  // full chunks: global id == row index
      t.date.push_back(std::move(d));
   }
}

TableImage build_table(const RawTable& raw, uint32_t threads) {
   TableImage t;
   build_table_frame(raw, t);
   for (const auto& c : raw.seq) t.seq.push_back(build_seq_column(c, t.chunk_sizes, threads));
   build_metadata_columns(raw, t, threads);
   return t;
}

}  // namespace rhygpu
