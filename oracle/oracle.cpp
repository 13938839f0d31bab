// CPU ORACLE — test infrastructure only.
//
// A plain C++ restatement of the reference's filter / count / mutations path, used by tests/ to
// check the CUDA path bit for bit, by __graft_entry__.smoke() and by bench.py's CPU baseline leg.
// Nothing in the product links or calls this file.
//
// Parity anchor: the reference (GenSpectrum/LAPIS-SILO, "RhyDB") cannot be compiled here — its
// set algebra lives in CRoaring roaring/4.5.0 (conanfile.py:24) and it needs Arrow, Boost, simdjson
// and more, none of which is present. This file therefore restates:
//   * the container set algebra (array <= 4096 / bitset containers keyed by the high 16 bits of the
//     row id, as in the published Roaring format; any correct set algebra yields the same sets),
//   * CopyOnWriteBitmap semantics (src/rhydb/query_engine/copy_on_write_bitmap.cpp),
//   * ingestion: extractCoverageAndMutationsFromSequence (src/rhydb/common/aligned_sequence.cpp:19-122),
//     HorizontalCoverageIndex::insertCoverage (storage/column/horizontal_coverage_index.cpp:17-46),
//     SequenceColumn::appendChunk / finalize (storage/column/sequence_column.cpp:100-212),
//     VerticalSequenceIndex (storage/column/vertical_sequence_index.cpp:17-283),
//   * expressions: SymbolEquals / HasMutation / SymbolInSet / And / Or / Negation / NOf / Maybe /
//     Exact / Equals (indexed string) / DateBetween rewrite + compile (query_engine/scalar_expressions/),
//     and MutationProfile's literal rewrite into Not(NOf(distance + 1, SymbolInSet per position))
//     with all three profile inputs (scalar_expressions/mutation_profile.cpp:62-257),
//   * operators: IndexScan, Intersection, Union, Complement, Threshold, Selection,
//     IsInCoveredRegion, CompareToValueSelection, Empty, Full (query_engine/filter/operators/),
//   * actions: CountFilterNode (operators/count_filter_node.cpp:35-71) and the Mutations action
//     (operators/mutations_node.cpp:39-366).
// The restatement is pinned against the reference's own known-answer tests, restated in
// tests/golden/reference_cases.py (file:line of each test cited there) and run by
// tests/test_golden_reference.py.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iterator>
#include <map>
#include <memory>
#include <mutex>
#include <optional>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace oracle {

// ================================================================================================
// Alphabets (reference: src/rhydb/common/nucleotide_symbols.{h,cpp}, aa_symbols.{h,cpp})

struct Alpha {
   int count;
   int missing;
   std::string chars;
   std::vector<int> valid;                  // VALID_MUTATION_SYMBOLS, in order
   std::vector<std::vector<int>> codes_for; // CODES_FOR
   std::vector<std::vector<int>> ambiguity; // AMBIGUITY_SYMBOLS
   int sym(char c) const {
      if (c >= 'a' && c <= 'z') c = static_cast<char>(c - 'a' + 'A');
      if (count == 16 && c == 'U') c = 'T';
      for (int i = 0; i < count; ++i)
         if (chars[i] == c) return i;
      return -1;
   }
   void derive() {
      ambiguity.assign(count, {});
      for (int s = 0; s < count; ++s) {
         for (int y = 0; y < count; ++y) {
            bool sup = true;
            for (int x : codes_for[s]) sup = sup && std::find(codes_for[y].begin(), codes_for[y].end(), x) != codes_for[y].end();
            if (sup) ambiguity[s].push_back(y);
         }
      }
   }
};

const Alpha& nuc() {
   static const Alpha a = [] {
      Alpha a;
      a.count = 16;
      a.chars = "-ACGTRYSWKMBDHVN";
      a.missing = 15;
      a.valid = {0, 1, 2, 3, 4};
      a.codes_for = {{0}, {1}, {2}, {3}, {4}, {1, 3}, {2, 4}, {3, 2}, {1, 4}, {3, 4}, {1, 2}, {2, 3, 4}, {1, 3, 4}, {1, 2, 4}, {1, 2, 3}, {}};
      for (int i = 0; i < 16; ++i) a.codes_for[15].push_back(i);
      a.derive();
      return a;
   }();
   return a;
}

const Alpha& aa() {
   static const Alpha a = [] {
      Alpha a;
      a.count = 28;
      a.chars = "-ACDEFGHIKLMNOPQRSTUVWYBJZ*X";
      a.missing = 27;
      for (int i = 0; i <= 22; ++i) a.valid.push_back(i);
      a.valid.push_back(26);
      a.codes_for.resize(28);
      for (int i = 0; i < 28; ++i) a.codes_for[i] = {i};
      a.codes_for[23] = {3, 12};   // B = D or N
      a.codes_for[24] = {10, 8};   // J = L or I
      a.codes_for[25] = {15, 4};   // Z = Q or E
      a.codes_for[27].clear();
      for (int i = 0; i < 28; ++i) a.codes_for[27].push_back(i);
      a.derive();
      return a;
   }();
   return a;
}

// ================================================================================================
// Containers and row sets

struct Ctr {
   bool is_bitset = false;
   std::vector<uint16_t> arr;
   std::vector<uint64_t> bits;  // 1024 words when is_bitset
   uint32_t card = 0;

   static Ctr from_sorted(std::vector<uint16_t> v) {
      Ctr c;
      c.card = static_cast<uint32_t>(v.size());
      if (v.size() > 4096) {
         c.is_bitset = true;
         c.bits.assign(1024, 0);
         for (uint16_t x : v) c.bits[x >> 6] |= 1ull << (x & 63);
      } else {
         c.arr = std::move(v);
      }
      return c;
   }
   static Ctr from_bits(std::vector<uint64_t> b) {
      uint32_t card = 0;
      for (uint64_t w : b) card += static_cast<uint32_t>(__builtin_popcountll(w));
      Ctr c;
      c.card = card;
      if (card > 4096) {
         c.is_bitset = true;
         c.bits = std::move(b);
      } else {
         c.arr.reserve(card);
         for (uint32_t i = 0; i < 1024; ++i) {
            uint64_t w = b[i];
            while (w) {
               c.arr.push_back(static_cast<uint16_t>(i * 64 + __builtin_ctzll(w)));
               w &= w - 1;
            }
         }
      }
      return c;
   }
   bool contains(uint16_t x) const {
      if (is_bitset) return bits[x >> 6] >> (x & 63) & 1;
      return std::binary_search(arr.begin(), arr.end(), x);
   }
   std::vector<uint64_t> to_bits() const {
      if (is_bitset) return bits;
      std::vector<uint64_t> b(1024, 0);
      for (uint16_t x : arr) b[x >> 6] |= 1ull << (x & 63);
      return b;
   }
   void add(uint16_t x) {  // appends in increasing order during ingestion
      if (is_bitset) {
         if (!(bits[x >> 6] >> (x & 63) & 1)) {
            bits[x >> 6] |= 1ull << (x & 63);
            ++card;
         }
         return;
      }
      if (!arr.empty() && arr.back() >= x) {
         auto it = std::lower_bound(arr.begin(), arr.end(), x);
         if (it != arr.end() && *it == x) return;
         arr.insert(it, x);
      } else {
         arr.push_back(x);
      }
      ++card;
      if (card > 4096) *this = from_bits(to_bits());
   }
};

Ctr ctr_and(const Ctr& a, const Ctr& b) {
   if (!a.is_bitset && !b.is_bitset) {
      std::vector<uint16_t> out;
      std::set_intersection(a.arr.begin(), a.arr.end(), b.arr.begin(), b.arr.end(), std::back_inserter(out));
      return Ctr::from_sorted(std::move(out));
   }
   if (!a.is_bitset || !b.is_bitset) {
      const Ctr& arr = a.is_bitset ? b : a;
      const Ctr& bs = a.is_bitset ? a : b;
      std::vector<uint16_t> out;
      for (uint16_t x : arr.arr)
         if (bs.contains(x)) out.push_back(x);
      return Ctr::from_sorted(std::move(out));
   }
   std::vector<uint64_t> o(1024);
   for (int i = 0; i < 1024; ++i) o[i] = a.bits[i] & b.bits[i];
   return Ctr::from_bits(std::move(o));
}

Ctr ctr_or(const Ctr& a, const Ctr& b) {
   if (!a.is_bitset && !b.is_bitset && a.card + b.card <= 4096) {
      std::vector<uint16_t> out;
      std::set_union(a.arr.begin(), a.arr.end(), b.arr.begin(), b.arr.end(), std::back_inserter(out));
      return Ctr::from_sorted(std::move(out));
   }
   std::vector<uint64_t> x = a.to_bits();
   if (b.is_bitset) {
      for (int i = 0; i < 1024; ++i) x[i] |= b.bits[i];
   } else {
      for (uint16_t v : b.arr) x[v >> 6] |= 1ull << (v & 63);
   }
   return Ctr::from_bits(std::move(x));
}

Ctr ctr_andnot(const Ctr& a, const Ctr& b) {
   if (!a.is_bitset) {
      std::vector<uint16_t> out;
      for (uint16_t x : a.arr)
         if (!b.contains(x)) out.push_back(x);
      return Ctr::from_sorted(std::move(out));
   }
   std::vector<uint64_t> x = a.bits;
   if (b.is_bitset) {
      for (int i = 0; i < 1024; ++i) x[i] &= ~b.bits[i];
   } else {
      for (uint16_t v : b.arr) x[v >> 6] &= ~(1ull << (v & 63));
   }
   return Ctr::from_bits(std::move(x));
}

uint32_t ctr_and_card(const Ctr& a, const Ctr& b) {
   if (!a.is_bitset && !b.is_bitset) {
      uint32_t n = 0;
      size_t i = 0, j = 0;
      while (i < a.arr.size() && j < b.arr.size()) {
         if (a.arr[i] < b.arr[j]) ++i;
         else if (a.arr[i] > b.arr[j]) ++j;
         else {
            ++n;
            ++i;
            ++j;
         }
      }
      return n;
   }
   if (!a.is_bitset || !b.is_bitset) {
      const Ctr& arr = a.is_bitset ? b : a;
      const Ctr& bs = a.is_bitset ? a : b;
      uint32_t n = 0;
      for (uint16_t x : arr.arr) n += bs.contains(x);
      return n;
   }
   uint32_t n = 0;
   for (int i = 0; i < 1024; ++i) n += static_cast<uint32_t>(__builtin_popcountll(a.bits[i] & b.bits[i]));
   return n;
}

// Complement within [0, size) of one chunk (reference: RowLayout::complementInPlace, row_layout.cpp:18-23).
Ctr ctr_flip(const Ctr& a, uint32_t size) {
   std::vector<uint64_t> x = a.to_bits();
   for (uint32_t r = 0; r < 65536; r += 64) {
      const uint32_t w = r >> 6;
      uint64_t m;
      if (r + 64 <= size) m = ~0ull;
      else if (r >= size) m = 0;
      else m = (1ull << (size - r)) - 1;
      x[w] ^= m;
   }
   return Ctr::from_bits(std::move(x));
}

struct Layout {
   std::vector<uint32_t> chunk_sizes;
   uint32_t num_rows = 0;
};

struct RowSet {
   std::vector<std::pair<uint16_t, Ctr>> c;  // sorted by key, no empty containers

   uint64_t cardinality() const {
      uint64_t n = 0;
      for (const auto& [k, x] : c) n += x.card;
      return n;
   }
   void push(uint16_t k, Ctr x) {
      if (x.card) c.emplace_back(k, std::move(x));
   }
   const Ctr* find(uint16_t k) const {
      auto it = std::lower_bound(c.begin(), c.end(), k, [](const auto& p, uint16_t key) { return p.first < key; });
      if (it != c.end() && it->first == k) return &it->second;
      return nullptr;
   }
   bool contains(uint32_t row) const {
      const Ctr* x = find(static_cast<uint16_t>(row >> 16));
      return x && x->contains(static_cast<uint16_t>(row & 0xFFFF));
   }
   bool empty() const { return c.empty(); }
};

RowSet rs_and(const RowSet& a, const RowSet& b) {  // copy_on_write_bitmap.cpp:145-176
   RowSet o;
   size_t i = 0, j = 0;
   while (i < a.c.size() && j < b.c.size()) {
      if (a.c[i].first < b.c[j].first) ++i;
      else if (a.c[i].first > b.c[j].first) ++j;
      else {
         o.push(a.c[i].first, ctr_and(a.c[i].second, b.c[j].second));
         ++i;
         ++j;
      }
   }
   return o;
}

RowSet rs_andnot(const RowSet& a, const RowSet& b) {  // copy_on_write_bitmap.cpp:178-211
   RowSet o;
   size_t j = 0;
   for (const auto& [k, x] : a.c) {
      while (j < b.c.size() && b.c[j].first < k) ++j;
      if (j < b.c.size() && b.c[j].first == k) {
         o.push(k, ctr_andnot(x, b.c[j].second));
      } else {
         o.push(k, x);
      }
   }
   return o;
}

RowSet rs_or(const RowSet& a, const RowSet& b) {  // copy_on_write_bitmap.cpp:213-284
   RowSet o;
   size_t i = 0, j = 0;
   while (i < a.c.size() || j < b.c.size()) {
      if (j >= b.c.size() || (i < a.c.size() && a.c[i].first < b.c[j].first)) {
         o.push(a.c[i].first, a.c[i].second);
         ++i;
      } else if (i >= a.c.size() || b.c[j].first < a.c[i].first) {
         o.push(b.c[j].first, b.c[j].second);
         ++j;
      } else {
         o.push(a.c[i].first, ctr_or(a.c[i].second, b.c[j].second));
         ++i;
         ++j;
      }
   }
   return o;
}

void rs_complement(RowSet& a, const Layout& L) {  // row_layout.cpp:18-23
   RowSet o;
   size_t j = 0;
   for (uint32_t k = 0; k < L.chunk_sizes.size(); ++k) {
      while (j < a.c.size() && a.c[j].first < k) ++j;
      if (j < a.c.size() && a.c[j].first == k) {
         o.push(static_cast<uint16_t>(k), ctr_flip(a.c[j].second, L.chunk_sizes[k]));
      } else {
         o.push(static_cast<uint16_t>(k), ctr_flip(Ctr{}, L.chunk_sizes[k]));
      }
   }
   a = std::move(o);
}

RowSet rs_full(const Layout& L) {  // RowLayout::fullBitmap, row_layout.cpp:9-16
   RowSet o;
   rs_complement(o, L);
   return o;
}

RowSet rs_from_sorted_rows(const std::vector<uint32_t>& rows) {
   RowSet o;
   size_t i = 0;
   while (i < rows.size()) {
      const uint16_t k = static_cast<uint16_t>(rows[i] >> 16);
      std::vector<uint16_t> v;
      while (i < rows.size() && (rows[i] >> 16) == k) v.push_back(static_cast<uint16_t>(rows[i++] & 0xFFFF));
      v.erase(std::unique(v.begin(), v.end()), v.end());
      o.push(k, Ctr::from_sorted(std::move(v)));
   }
   return o;
}

// ================================================================================================
// Raw input (same memory layout as the product's RhyRawTable)

extern "C" {
struct ORawSeqColumn {
   const char* name;
   int kind;
   const char* reference;
   uint32_t L;
   const uint8_t* is_null;
   const uint64_t* row_off;
   const uint32_t* run_pos;
   const uint32_t* run_len;
   const char* run_char;
};
struct ORawDictColumn {
   const char* name;
   uint32_t n_values;
   const char* const* values;
   const uint32_t* ids;
};
struct ORawDateColumn {
   const char* name;
   const int32_t* days;
};
struct ORawTable {
   uint32_t n_rows;
   uint32_t n_seq, n_dict, n_date;
   const ORawSeqColumn* seq;
   const ORawDictColumn* dict;
   const ORawDateColumn* date;
};
}

// ================================================================================================
// Storage

struct Interval {
   uint32_t s, e;
};

struct SeqColumn {
   std::string name;
   const Alpha* A;
   uint32_t L = 0;
   std::vector<int> reference;        // metadata->reference_sequence
   std::vector<int> local_reference;  // after adaptation
   struct Key {
      uint32_t position;
      uint16_t v_index;
      int symbol;
      bool operator<(const Key& o) const {
         if (position != o.position) return position < o.position;
         if (v_index != o.v_index) return v_index < o.v_index;
         return symbol < o.symbol;
      }
   };
   std::map<Key, Ctr> vertical;
   std::vector<std::vector<std::pair<uint32_t, uint32_t>>> start_end;  // per chunk per row
   std::vector<std::pair<uint32_t, uint32_t>> batch_start_ends;
   std::map<uint32_t, std::vector<Interval>> horizontal;  // missing positions inside coverage, as intervals
   RowSet null_bitmap;
   uint64_t sequence_count = 0;
   uint32_t flipped = 0;

   std::pair<uint32_t, uint32_t> coverage_range(uint32_t row) const { return start_end[row >> 16][row & 0xFFFF]; }
   bool horizontal_contains(uint32_t row, uint32_t pos) const {
      auto it = horizontal.find(row);
      if (it == horizontal.end()) return false;
      for (const auto& iv : it->second)
         if (iv.s <= pos && pos < iv.e) return true;
      return false;
   }
   // getCoverageBitmapForPositions<1> (horizontal_coverage_index.h:56-98)
   RowSet coverage_bitmap(uint32_t pos) const {
      std::vector<uint32_t> rows;
      for (size_t k = 0; k < start_end.size(); ++k) {
         auto [bs, be] = batch_start_ends[k];
         if (be <= pos || bs >= pos + 1) continue;
         for (size_t r = 0; r < start_end[k].size(); ++r) {
            auto [s, e] = start_end[k][r];
            if (s <= pos && pos < e) rows.push_back(static_cast<uint32_t>(k << 16 | r));
         }
      }
      // remove the rows whose missing positions contain pos, walking every per-row bitmap like the
      // reference does (horizontal_coverage_index.h:89-96)
      std::vector<uint32_t> drop;
      for (const auto& [row, ivs] : horizontal) {
         for (const auto& iv : ivs) {
            if (iv.s <= pos && pos < iv.e) {
               drop.push_back(row);
               break;
            }
         }
      }
      std::vector<uint32_t> keep;
      keep.reserve(rows.size());
      std::set_difference(rows.begin(), rows.end(), drop.begin(), drop.end(), std::back_inserter(keep));
      return rs_from_sorted_rows(keep);
   }
   // getMatchingContainersAsBitmap / fromContainerViews (vertical_sequence_index.cpp:206-227,297-322)
   RowSet matching(uint32_t pos, const std::vector<bool>& symbols) const {
      RowSet o;
      auto it = vertical.lower_bound(Key{pos, 0, 0});
      std::map<uint16_t, Ctr> acc;
      for (; it != vertical.end() && it->first.position == pos; ++it) {
         if (!symbols[it->first.symbol]) continue;
         auto f = acc.find(it->first.v_index);
         if (f == acc.end()) acc.emplace(it->first.v_index, it->second);
         else f->second = ctr_or(f->second, it->second);
      }
      for (auto& [k, x] : acc) o.push(k, std::move(x));
      return o;
   }
};

struct DictColumn {
   std::string name;
   std::map<std::string, RowSet> index;
};

struct DateColumn {
   std::string name;
   std::vector<int32_t> days;  // by global id (chunk stride), INT32_MIN null
   bool is_null(uint32_t row) const { return days[row] == INT32_MIN; }
};

struct Table {
   Layout layout;
   std::vector<SeqColumn> seq;
   std::vector<DictColumn> dict;
   std::vector<DateColumn> date;
   int primary_key = -1;  // dictionary column of the schema's primary key
   int find_seq(const std::string& n) const {
      for (size_t i = 0; i < seq.size(); ++i)
         if (seq[i].name == n) return static_cast<int>(i);
      return -1;
   }
   int find_dict(const std::string& n) const {
      for (size_t i = 0; i < dict.size(); ++i)
         if (dict[i].name == n) return static_cast<int>(i);
      return -1;
   }
   int find_date(const std::string& n) const {
      for (size_t i = 0; i < date.size(); ++i)
         if (date[i].name == n) return static_cast<int>(i);
      return -1;
   }
};

// extractCoverageAndMutationsFromSequence on an aligned sequence given as reference + runs.
struct Diff {
   uint32_t start = 0, end = 0;
   std::vector<uint32_t> missing;                 // positions
   std::vector<std::pair<uint32_t, int>> mutations;
};

// The reference's message for a character outside the alphabet (aligned_sequence.cpp:38-41).
std::string illegal_character(char c, size_t position) {
   return std::string("illegal character '") + c + "' at position " + std::to_string(position) + " in the input sequence";
}

Diff diff_runs(const ORawSeqColumn& raw, const Alpha& A, const std::vector<int>& ref, uint32_t row, bool ref_has_missing) {
   Diff d;
   const uint32_t L = raw.L;
   uint32_t cursor = 0;
   // Positions outside the runs hold the reference character; where that character is the
   // missing symbol the sequence is missing there (aligned_sequence.cpp:43-44 with
   // reference_is_missing_somewhere).
   auto reference_gap = [&](uint32_t a, uint32_t z) {
      for (uint32_t p = a; p < z; ++p)
         if (ref[p] == A.missing) d.missing.push_back(p);
   };
   for (uint64_t k = raw.row_off[row]; k < raw.row_off[row + 1]; ++k) {
      const int s = A.sym(raw.run_char[k]);
      if (s < 0) throw std::invalid_argument(illegal_character(raw.run_char[k], raw.run_pos[k]));
      if (ref_has_missing) reference_gap(cursor, raw.run_pos[k]);
      for (uint32_t p = raw.run_pos[k]; p < raw.run_pos[k] + raw.run_len[k]; ++p) {
         if (s == A.missing) d.missing.push_back(p);
         else if (s != ref[p]) d.mutations.emplace_back(p, s);
      }
      cursor = raw.run_pos[k] + raw.run_len[k];
   }
   if (ref_has_missing) reference_gap(cursor, L);
   // leading / trailing missing positions (aligned_sequence.cpp:89-120)
   size_t lead = 0;
   while (lead < d.missing.size() && d.missing[lead] == lead) ++lead;
   size_t trail = 0;
   while (trail < d.missing.size() - lead && d.missing[d.missing.size() - 1 - trail] == L - 1 - trail) ++trail;
   if (lead + trail == L) {
      d.missing.clear();
      d.start = d.end = 0;
   } else {
      d.start = static_cast<uint32_t>(lead);
      d.end = static_cast<uint32_t>(L - trail);
      d.missing.erase(d.missing.end() - static_cast<ptrdiff_t>(trail), d.missing.end());
      d.missing.erase(d.missing.begin(), d.missing.begin() + static_cast<ptrdiff_t>(lead));
   }
   return d;
}

// The reference's word-at-a-time string diff (aligned_sequence.cpp:19-122), for string inputs.
Diff diff_string(const std::string& seq, const std::string& refs, const Alpha& A) {
   Diff d;
   const size_t len = seq.size();
   const bool ref_missing = refs.find(A.chars[A.missing]) != std::string::npos;
   auto one = [&](size_t i) {
      const int s = A.sym(seq[i]);
      if (s < 0) throw std::invalid_argument(illegal_character(seq[i], i));
      if (s == A.missing) d.missing.push_back(static_cast<uint32_t>(i));
      else if (s != A.sym(refs[i])) d.mutations.emplace_back(static_cast<uint32_t>(i), s);
   };
   size_t i = 0;
   if (!ref_missing) {
      for (; i + 8 <= len; i += 8) {
         uint64_t a, b;
         std::memcpy(&a, seq.data() + i, 8);
         std::memcpy(&b, refs.data() + i, 8);
         uint64_t x = a ^ b;
         while (x) {
            const size_t byte = static_cast<size_t>(__builtin_ctzll(x)) / 8;
            one(i + byte);
            x &= ~(0xFFull << (byte * 8));
         }
      }
   }
   for (; i < len; ++i)
      if (ref_missing || seq[i] != refs[i]) one(i);
   size_t lead = 0;
   while (lead < d.missing.size() && d.missing[lead] == lead) ++lead;
   size_t trail = 0;
   while (trail < d.missing.size() - lead && d.missing[d.missing.size() - 1 - trail] == len - 1 - trail) ++trail;
   if (lead + trail == len) {
      d.missing.clear();
   } else {
      d.start = static_cast<uint32_t>(lead);
      d.end = static_cast<uint32_t>(len - trail);
      d.missing.erase(d.missing.end() - static_cast<ptrdiff_t>(trail), d.missing.end());
      d.missing.erase(d.missing.begin(), d.missing.begin() + static_cast<ptrdiff_t>(lead));
   }
   return d;
}

std::vector<Interval> to_intervals(const std::vector<uint32_t>& pos) {
   std::vector<Interval> v;
   for (uint32_t p : pos) {
      if (!v.empty() && v.back().e == p) v.back().e = p + 1;
      else v.push_back({p, p + 1});
   }
   return v;
}

SeqColumn build_seq(const ORawSeqColumn& raw, const Layout& layout) {
   SeqColumn col;
   col.name = raw.name;
   col.A = raw.kind == 0 ? &nuc() : &aa();
   const Alpha& A = *col.A;
   col.L = raw.L;
   col.reference.resize(raw.L);
   for (uint32_t p = 0; p < raw.L; ++p) {
      col.reference[p] = A.sym(raw.reference[p]);
      if (col.reference[p] < 0) throw std::invalid_argument("illegal reference character");
   }
   col.local_reference = col.reference;
   const bool ref_has_missing = std::find(col.reference.begin(), col.reference.end(), A.missing) != col.reference.end();
   // appendChunk per 2^16-row chunk; each chunk flushes the per-position mutation buffer
   std::vector<std::vector<std::vector<uint32_t>>> buffer(raw.L, std::vector<std::vector<uint32_t>>(A.count));
   uint32_t row = 0;
   for (uint32_t k = 0; k < layout.chunk_sizes.size(); ++k) {
      col.start_end.emplace_back();
      col.batch_start_ends.emplace_back(UINT32_MAX, 0);
      for (uint32_t r = 0; r < layout.chunk_sizes[k]; ++r, ++row) {
         const uint32_t g = k << 16 | r;
         col.sequence_count++;
         Diff d;
         if (raw.is_null[row]) {
            col.null_bitmap = rs_or(col.null_bitmap, rs_from_sorted_rows({g}));
         } else {
            d = diff_runs(raw, A, col.reference, row, ref_has_missing);
         }
         // insertCoverage (horizontal_coverage_index.cpp:17-46)
         col.start_end[k].emplace_back(d.start, d.end);
         auto& [bs, be] = col.batch_start_ends.back();
         bs = std::min(bs, d.start);
         be = std::max(be, d.end);
         std::vector<uint32_t> inside;
         for (uint32_t p : d.missing)
            if (p >= d.start && p < d.end) inside.push_back(p);
         if (!inside.empty()) col.horizontal.emplace(g, to_intervals(inside));
         for (const auto& [p, s] : d.mutations) buffer[p][s].push_back(g);
      }
      // flushBuffer -> addSymbolsToPositions (vertical_sequence_index.cpp:17-38)
      for (uint32_t p = 0; p < raw.L; ++p) {
         for (int s = 0; s < A.count; ++s) {
            auto& ids = buffer[p][s];
            if (ids.empty()) continue;
            // all ids of one flush share the chunk's v_index (splitIdsIntoBatches, vertical_sequence_index.cpp:419-446)
            Ctr& ctr = col.vertical[SeqColumn::Key{p, static_cast<uint16_t>(ids.front() >> 16), s}];
            for (uint32_t g : ids) ctr.add(static_cast<uint16_t>(g & 0xFFFF));
            ids.clear();
         }
      }
   }
   // finalize: local reference adaptation (sequence_column.cpp:158-195)
   std::vector<int64_t> changes(raw.L + 1, 0);
   for (const auto& chunk : col.start_end)
      for (auto [s, e] : chunk) {
         changes[s] += 1;
         changes[e] -= 1;
      }
   for (const auto& [g, ivs] : col.horizontal)
      for (const auto& iv : ivs) {
         changes[iv.s] -= 1;
         changes[iv.e] += 1;
      }
   std::vector<uint64_t> coverage(raw.L);
   int64_t acc = 0;
   for (uint32_t p = 0; p < raw.L; ++p) {
      acc += changes[p];
      coverage[p] = static_cast<uint64_t>(acc);
   }
   for (uint32_t p = 0; p < raw.L; ++p) {
      const int cur = col.local_reference[p];
      std::vector<uint32_t> counts(A.count, 0);
      counts[cur] = static_cast<uint32_t>(coverage[p]);
      for (auto it = col.vertical.lower_bound({p, 0, 0}); it != col.vertical.end() && it->first.position == p; ++it) {
         counts[it->first.symbol] += it->second.card;
         counts[cur] -= it->second.card;
      }
      int best = cur;
      uint32_t best_count = counts[cur];
      for (int s = 0; s < A.count; ++s) {
         if (s == cur) continue;
         if (counts[s] > best_count) {
            best = s;
            best_count = counts[s];
         }
      }
      if (best == cur) continue;
      // adaptLocalReference (vertical_sequence_index.cpp:237-283)
      std::vector<bool> all(A.count, true);
      RowSet old_ref = rs_andnot(col.coverage_bitmap(p), col.matching(p, all));
      for (auto& [v, x] : old_ref.c) col.vertical.emplace(SeqColumn::Key{p, v, cur}, x);
      for (auto it = col.vertical.lower_bound({p, 0, 0}); it != col.vertical.end() && it->first.position == p;) {
         if (it->first.symbol == best) it = col.vertical.erase(it);
         else ++it;
      }
      col.local_reference[p] = best;
      ++col.flipped;
   }
   return col;
}

Table build_table(const ORawTable& raw) {
   Table t;
   for (uint32_t left = raw.n_rows; left > 0;) {
      const uint32_t s = std::min<uint32_t>(left, 65536);
      t.layout.chunk_sizes.push_back(s);
      left -= s;
   }
   t.layout.num_rows = raw.n_rows;
   for (uint32_t c = 0; c < raw.n_seq; ++c) t.seq.push_back(build_seq(raw.seq[c], t.layout));
   for (uint32_t c = 0; c < raw.n_dict; ++c) {
      DictColumn d;
      d.name = raw.dict[c].name;
      std::vector<std::vector<uint32_t>> rows(raw.dict[c].n_values);
      for (uint32_t i = 0; i < raw.n_rows; ++i) {
         const uint32_t id = raw.dict[c].ids[i];
         if (id == UINT32_MAX) continue;
         rows.at(id).push_back((i >> 16) << 16 | (i & 0xFFFF));
      }
      for (uint32_t v = 0; v < raw.dict[c].n_values; ++v) {
         if (!rows[v].empty()) d.index.emplace(raw.dict[c].values[v], rs_from_sorted_rows(rows[v]));
      }
      t.dict.push_back(std::move(d));
   }
   for (uint32_t c = 0; c < raw.n_date; ++c) {
      DateColumn d;
      d.name = raw.date[c].name;
      d.days.assign(static_cast<size_t>(t.layout.chunk_sizes.size()) << 16, INT32_MIN);
      for (uint32_t i = 0; i < raw.n_rows; ++i) d.days[i] = raw.date[c].days[i];
      t.date.push_back(std::move(d));
   }
   return t;
}

// ================================================================================================
// Operators (query_engine/filter/operators/)

struct IllegalQuery : std::runtime_error {
   using std::runtime_error::runtime_error;
};
struct CompileError : std::runtime_error {
   using std::runtime_error::runtime_error;
};

enum class OT { EMPTY, FULL, INDEX_SCAN, INTERSECTION, UNION, COMPLEMENT, THRESHOLD, SELECTION };

struct Predicate {
   enum Kind { COVERED, DATE } kind;
   const SeqColumn* seq = nullptr;
   uint32_t pos = 0;
   bool is_covered = true;
   const DateColumn* date = nullptr;
   enum Cmp { EQ, NE, LT, GT, LE, GE } cmp = EQ;
   int32_t value = 0;
   bool with_nulls = false;

   bool match(uint32_t row) const {
      if (kind == COVERED) {  // is_in_covered_region.cpp:31-51
         auto [s, e] = seq->coverage_range(row);
         bool covered;
         if (pos < s || pos >= e) covered = false;
         else covered = !seq->horizontal_contains(row, pos);
         return covered == is_covered;
      }
      if (date->is_null(row)) return with_nulls;  // selection.h:112-130
      const int32_t d = date->days[row];
      switch (cmp) {
         case EQ: return d == value;
         case NE: return d != value;
         case LT: return d < value;
         case GE: return d >= value;
         case GT: return d > value;
         case LE: return d <= value;
      }
      return false;
   }
   RowSet make_bitmap(const Layout& L) const {
      if (kind == COVERED) {  // is_in_covered_region.cpp:53-62
         RowSet r = seq->coverage_bitmap(pos);
         if (!is_covered) rs_complement(r, L);
         return r;
      }
      std::vector<uint32_t> rows;  // Predicate::makeBitmap default: match every row
      for (uint32_t k = 0; k < L.chunk_sizes.size(); ++k)
         for (uint32_t r = 0; r < L.chunk_sizes[k]; ++r)
            if (match(k << 16 | r)) rows.push_back(k << 16 | r);
      return rs_from_sorted_rows(rows);
   }
   double selectivity() const { return kind == COVERED ? 0.1 : 0.5; }
   Predicate negate() const {
      Predicate p = *this;
      if (kind == COVERED) {
         p.is_covered = !is_covered;
         return p;
      }
      switch (cmp) {
         case EQ: p.cmp = NE; break;
         case NE: p.cmp = EQ; break;
         case LT: p.cmp = GE; break;
         case GE: p.cmp = LT; break;
         case GT: p.cmp = LE; break;
         case LE: p.cmp = GT; break;
      }
      p.with_nulls = !with_nulls;
      return p;
   }
};

struct Operator;
using OpP = std::unique_ptr<Operator>;

struct Operator {
   OT type;
   const Layout* layout;
   RowSet bitmap;                   // INDEX_SCAN
   std::vector<OpP> children;       // non-negated / union children / complement child / selection child
   std::vector<OpP> negated;
   std::vector<Predicate> preds;
   bool has_child = false;          // SELECTION
   uint32_t n = 0;
   bool exact = false;

   RowSet evaluate() const;
};

OpP mkop(OT t, const Layout& L) {
   auto o = std::make_unique<Operator>();
   o->type = t;
   o->layout = &L;
   return o;
}

OpP make_complement(OpP c, const Layout& L) {
   auto o = mkop(OT::COMPLEMENT, L);
   o->children.push_back(std::move(c));
   return o;
}

OpP make_intersection(std::vector<OpP> pos, std::vector<OpP> neg, const Layout& L) {
   if (pos.empty()) throw CompileError("Intersection without non-negated children");
   if (pos.size() + neg.size() < 2) throw CompileError("Intersection needs at least two children");
   auto o = mkop(OT::INTERSECTION, L);
   o->children = std::move(pos);
   o->negated = std::move(neg);
   return o;
}

OpP make_union(std::vector<OpP> c, const Layout& L) {
   auto o = mkop(OT::UNION, L);
   o->children = std::move(c);
   return o;
}

OpP make_scan(RowSet b, const Layout& L) {
   auto o = mkop(OT::INDEX_SCAN, L);
   o->bitmap = std::move(b);
   return o;
}

OpP make_selection(OpP child, std::vector<Predicate> preds, const Layout& L) {
   auto o = mkop(OT::SELECTION, L);
   if (child) {
      o->children.push_back(std::move(child));
      o->has_child = true;
   }
   std::stable_sort(preds.begin(), preds.end(),
                    [](const Predicate& a, const Predicate& b) { return a.selectivity() < b.selectivity(); });
   o->preds = std::move(preds);
   return o;
}

OpP make_threshold(std::vector<OpP> pos, std::vector<OpP> neg, uint32_t n, bool exact, const Layout& L) {
   if (n >= pos.size() + neg.size()) throw CompileError("number_of_matchers must be less than the number of children");
   if (n == 0) throw CompileError("number_of_matchers must be greater than zero");
   auto o = mkop(OT::THRESHOLD, L);
   o->children = std::move(pos);
   o->negated = std::move(neg);
   o->n = n;
   o->exact = exact;
   return o;
}

OpP negate_op(OpP op) {  // operator.cpp:23-66
   const Layout& L = *op->layout;
   switch (op->type) {
      case OT::EMPTY: return mkop(OT::FULL, L);
      case OT::FULL: return mkop(OT::EMPTY, L);
      case OT::COMPLEMENT: return std::move(op->children[0]);
      case OT::SELECTION:
         if (!op->has_child && op->preds.size() == 1) return make_selection(nullptr, {op->preds[0].negate()}, L);
         return make_complement(std::move(op), L);
      default: return make_complement(std::move(op), L);
   }
}

RowSet Operator::evaluate() const {
   const Layout& L = *layout;
   switch (type) {
      case OT::EMPTY: return RowSet{};
      case OT::FULL: return rs_full(L);
      case OT::INDEX_SCAN: return bitmap;
      case OT::COMPLEMENT: {  // complement.cpp:51-56
         RowSet r = children[0]->evaluate();
         rs_complement(r, L);
         return r;
      }
      case OT::UNION: {  // union.cpp:34-42, fastUnion = sequential |=
         RowSet r;
         for (const auto& c : children) r = rs_or(r, c->evaluate());
         return r;
      }
      case OT::INTERSECTION: {  // intersection.cpp:59-106
         std::vector<RowSet> pos, neg;
         for (const auto& c : children) pos.push_back(c->evaluate());
         for (const auto& c : negated) neg.push_back(c->evaluate());
         std::stable_sort(pos.begin(), pos.end(), [](const RowSet& a, const RowSet& b) { return a.cardinality() < b.cardinality(); });
         std::stable_sort(neg.begin(), neg.end(), [](const RowSet& a, const RowSet& b) { return a.cardinality() > b.cardinality(); });
         RowSet r = std::move(pos[0]);
         for (size_t i = 1; i < pos.size(); ++i) r = rs_and(r, pos[i]);
         for (const auto& x : neg) r = rs_andnot(r, x);
         return r;
      }
      case OT::SELECTION: {  // selection.cpp:94-141
         RowSet candidates;
         if (has_child) {
            RowSet child = children[0]->evaluate();
            if (child.cardinality() <= L.num_rows / 10) {
               std::vector<uint32_t> rows;
               for (const auto& [k, x] : child.c) {
                  auto visit = [&](uint16_t r) {
                     const uint32_t g = static_cast<uint32_t>(k) << 16 | r;
                     bool ok = true;
                     for (const auto& p : preds) ok = ok && p.match(g);
                     if (ok) rows.push_back(g);
                  };
                  if (x.is_bitset) {
                     for (uint32_t i = 0; i < 65536; ++i)
                        if (x.bits[i >> 6] >> (i & 63) & 1) visit(static_cast<uint16_t>(i));
                  } else {
                     for (uint16_t r : x.arr) visit(r);
                  }
               }
               return rs_from_sorted_rows(rows);
            }
            candidates = rs_and(child, preds.front().make_bitmap(L));
         } else {
            candidates = preds.front().make_bitmap(L);
         }
         if (preds.size() == 1) return candidates;
         std::vector<uint32_t> rows;
         for (const auto& [k, x] : candidates.c) {
            auto visit = [&](uint16_t r) {
               const uint32_t g = static_cast<uint32_t>(k) << 16 | r;
               bool ok = true;
               for (size_t i = 1; i < preds.size(); ++i) ok = ok && preds[i].match(g);
               if (ok) rows.push_back(g);
            };
            if (x.is_bitset) {
               for (uint32_t i = 0; i < 65536; ++i)
                  if (x.bits[i >> 6] >> (i & 63) & 1) visit(static_cast<uint16_t>(i));
            } else {
               for (uint16_t r : x.arr) visit(r);
            }
         }
         return rs_from_sorted_rows(rows);
      }
      case OT::THRESHOLD: {  // threshold.cpp:64-138
         const uint32_t size = exact ? n + 1 : n;
         std::vector<RowSet> bm(size);
         if (children.empty()) {
            bm[0] = negated[0]->evaluate();
            rs_complement(bm[0], L);
         } else {
            bm[0] = children[0]->evaluate();
         }
         const int max_idx = static_cast<int>(size) - 1;
         const int nn = static_cast<int>(children.size()), ng = static_cast<int>(negated.size());
         const int N = static_cast<int>(n), k = nn + ng;
         for (int i = 1; i < nn; ++i) {
            const RowSet b = children[i]->evaluate();
            for (int j = std::min(max_idx, i); j > std::max(0, N - k + i - 1); --j) bm[j] = rs_or(bm[j], rs_and(bm[j - 1], b));
            if (k - i > N - 1) bm[0] = rs_or(bm[0], b);
         }
         const int took_first = children.empty() ? 1 : 0;
         for (int li = took_first; li < ng; ++li) {
            RowSet b = negated[li]->evaluate();
            const int i = li + nn;
            for (int j = std::min(max_idx, i); j > std::max(0, N - k + i - 1); --j) bm[j] = rs_or(bm[j], rs_andnot(bm[j - 1], b));
            if (k - i > N - 1) {
               rs_complement(b, L);
               bm[0] = rs_or(bm[0], b);
            }
         }
         if (exact) return rs_andnot(bm[n - 1], bm[n]);
         return bm.back();
      }
   }
   return RowSet{};
}

// ================================================================================================
// Expressions (query_engine/scalar_expressions/)

enum class Mode { UPPER, LOWER, NONE };
Mode invert(Mode m) { return m == Mode::UPPER ? Mode::LOWER : m == Mode::LOWER ? Mode::UPPER : m; }

enum class EK { AND, OR, NOT, NOF, MAYBE, EXACT, SYM_EQ, HAS_MUT, SYM_IN_SET, STR_EQ, DATE_BETWEEN, BOOL, MUT_PROFILE };

struct Expr;
using EP = std::unique_ptr<Expr>;
struct Expr {
   EK k;
   std::vector<EP> ch;
   std::string column;
   uint32_t pos = 0;
   int sym = -1;  // -1 = '.'
   std::vector<int> symbols;  // SYM_IN_SET, may repeat; MUT_PROFILE: position << 8 | symbol
   int n = 0;
   bool exact = false;
   std::string value;
   std::optional<int32_t> from, to;
   bool truth = false;
   bool by_id = false;  // MUT_PROFILE: `value` is a primary key
   EP clone() const {
      auto e = std::make_unique<Expr>();
      e->k = k;
      for (const auto& c : ch) e->ch.push_back(c->clone());
      e->column = column;
      e->pos = pos;
      e->sym = sym;
      e->symbols = symbols;
      e->n = n;
      e->exact = exact;
      e->value = value;
      e->from = from;
      e->to = to;
      e->truth = truth;
      e->by_id = by_id;
      return e;
   }
};

struct Parser {
   const std::string& s;
   const Table& t;
   size_t i = 0;
   void ws() {
      while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n')) ++i;
   }
   bool eat(char c) {
      ws();
      if (i < s.size() && s[i] == c) {
         ++i;
         return true;
      }
      return false;
   }
   void expect(char c) {
      if (!eat(c)) throw IllegalQuery(std::string("expected ") + c);
   }
   std::string tok() {
      ws();
      size_t b = i;
      while (i < s.size() && s[i] != ',' && s[i] != '(' && s[i] != ')' && s[i] != ' ') ++i;
      if (b == i) throw IllegalQuery("expected token");
      return s.substr(b, i - b);
   }
   long long num() { return std::stoll(tok()); }
   EP node(EK k) {
      auto e = std::make_unique<Expr>();
      e->k = k;
      return e;
   }
   const Alpha& alpha_of(const std::string& col) {
      const int c = t.find_seq(col);
      if (c < 0) throw IllegalQuery("no such sequence column");
      return *t.seq[c].A;
   }
   EP parse() {
      const std::string name = tok();
      if (name == "True" || name == "False") {
         auto e = node(EK::BOOL);
         e->truth = name == "True";
         return e;
      }
      expect('(');
      EP e;
      if (name == "And" || name == "Or") {
         e = node(name == "And" ? EK::AND : EK::OR);
         if (eat(')')) return e;
         do e->ch.push_back(parse());
         while (eat(','));
      } else if (name == "Not" || name == "Maybe" || name == "Exact") {
         e = node(name == "Not" ? EK::NOT : name == "Maybe" ? EK::MAYBE : EK::EXACT);
         e->ch.push_back(parse());
      } else if (name == "NOf") {
         e = node(EK::NOF);
         e->n = static_cast<int>(num());
         expect(',');
         e->exact = tok() == "exactly";
         while (eat(',')) e->ch.push_back(parse());
      } else if (name == "SymEq") {
         e = node(EK::SYM_EQ);
         e->column = tok();
         expect(',');
         e->pos = static_cast<uint32_t>(num() - 1);
         expect(',');
         const std::string c = tok();
         e->sym = c == "." ? -1 : alpha_of(e->column).sym(c[0]);
         if (c != "." && e->sym < 0) throw IllegalQuery("illegal symbol");
      } else if (name == "HasMut") {
         e = node(EK::HAS_MUT);
         e->column = tok();
         expect(',');
         e->pos = static_cast<uint32_t>(num() - 1);
      } else if (name == "StrEq") {
         e = node(EK::STR_EQ);
         e->column = tok();
         expect(',');
         e->value = tok();
      } else if (name == "DateBetween") {
         e = node(EK::DATE_BETWEEN);
         e->column = tok();
         expect(',');
         if (!eat('*')) e->from = static_cast<int32_t>(num());
         expect(',');
         if (!eat('*')) e->to = static_cast<int32_t>(num());
      } else if (name == "MutProfile" || name == "MutProfileMutations" || name == "MutProfileSequenceId") {
         e = node(EK::MUT_PROFILE);
         e->column = tok();
         const Alpha& A = alpha_of(e->column);
         expect(',');
         e->n = static_cast<int>(num());
         if (e->n < 0) throw IllegalQuery("negative distance");
         if (name == "MutProfile" || name == "MutProfileSequenceId") {
            expect(',');
            e->value = tok();
            e->by_id = name == "MutProfileSequenceId";
         } else {
            while (eat(',')) {
               const std::string m = tok();
               const size_t colon = m.find(':');
               if (colon == std::string::npos || colon + 2 != m.size()) throw IllegalQuery("a mutation is position:symbol");
               const long long p = std::stoll(m.substr(0, colon));
               const int sy = A.sym(m[colon + 1]);
               if (p < 1 || sy < 0) throw IllegalQuery("bad mutation");
               e->symbols.push_back(static_cast<int>((p - 1) << 8 | sy));
            }
         }
      } else {
         throw IllegalQuery("unknown function " + name);
      }
      expect(')');
      return e;
   }
};

const SeqColumn& seq_of(const Table& t, const std::string& name) {
   const int c = t.find_seq(name);
   if (c < 0) throw IllegalQuery("no such sequence column");
   return t.seq[c];
}

EP sym_in_set(const std::string& col, uint32_t pos, std::vector<int> syms) {
   auto e = std::make_unique<Expr>();
   e->k = EK::SYM_IN_SET;
   e->column = col;
   e->pos = pos;
   e->symbols = std::move(syms);
   return e;
}

bool has(const std::vector<int>& v, int s) { return std::find(v.begin(), v.end(), s) != v.end(); }

// buildProfileFromSequenceId / reconstructSequenceAtRow (mutation_profile.cpp:95-150): the first
// row holding `id` in the primary-key dictionary column; the local reference overwritten by the
// row's vertical-index symbols, then the missing symbol outside its covered region and inside its
// missing intervals.
std::vector<int> sequence_at_primary_key(const Table& t, const SeqColumn& c, const std::string& id) {
   if (t.primary_key < 0) throw IllegalQuery("the table has no primary key column");
   const DictColumn& pk = t.dict[t.primary_key];
   const auto it = pk.index.find(id);
   if (it == pk.index.end() || it->second.empty()) throw IllegalQuery("No sequence found with primary key");
   const auto& [chunk, ctr] = it->second.c.front();
   uint32_t first = 0;
   if (ctr.is_bitset) {
      uint32_t w = 0;
      while (ctr.bits[w] == 0) ++w;
      first = 64 * w + static_cast<uint32_t>(__builtin_ctzll(ctr.bits[w]));
   } else {
      first = ctr.arr.front();
   }
   const uint32_t row = static_cast<uint32_t>(chunk) << 16 | first;
   std::vector<int> seq = c.local_reference;
   for (const auto& [key, x] : c.vertical)
      if (key.v_index == chunk && x.contains(static_cast<uint16_t>(first))) seq[key.position] = key.symbol;
   const auto [s, e] = c.coverage_range(row);
   for (uint32_t p = 0; p < c.L; ++p)
      if (p < s || p >= e || c.horizontal_contains(row, p)) seq[p] = c.A->missing;
   return seq;
}

EP rewrite(const Expr& e, const Table& t, Mode mode) {
   switch (e.k) {
      case EK::AND: {
         auto o = std::make_unique<Expr>();
         o->k = EK::AND;
         for (const auto& c : e.ch) o->ch.push_back(rewrite(*c, t, mode));
         return o;
      }
      case EK::OR: {  // or.cpp:173-192
         std::vector<const Expr*> collected, queue;
         for (const auto& c : e.ch) queue.push_back(c.get());
         while (!queue.empty()) {
            const Expr* cur = queue.back();
            queue.pop_back();
            if (cur->k == EK::OR) {
               for (const auto& c : cur->ch) queue.push_back(c.get());
            } else {
               collected.push_back(cur);
            }
         }
         std::vector<EP> rw;
         for (const Expr* c : collected) rw.push_back(rewrite(*c, t, mode));
         std::vector<EP> nt;
         bool short_true = false;
         while (!rw.empty()) {
            EP c = std::move(rw.back());
            rw.pop_back();
            if (c->k == EK::BOOL) {
               if (c->truth) {
                  short_true = true;
                  break;
               }
               continue;
            }
            if (c->k == EK::OR) {
               for (auto& g : c->ch) rw.push_back(std::move(g));
            } else {
               nt.push_back(std::move(c));
            }
         }
         if (short_true) {
            nt.clear();
            auto tr = std::make_unique<Expr>();
            tr->k = EK::BOOL;
            tr->truth = true;
            nt.push_back(std::move(tr));
         }
         for (int kind = 0; kind < 2; ++kind) {
            std::vector<EP> next;
            std::map<std::pair<std::string, uint32_t>, std::vector<int>> merged;
            for (auto& c : nt) {
               const bool match = c->k == EK::SYM_IN_SET && (t.seq[t.find_seq(c->column)].A == (kind == 0 ? &nuc() : &aa()));
               if (match) {
                  auto& v = merged[{c->column, c->pos}];
                  v.insert(v.end(), c->symbols.begin(), c->symbols.end());
               } else {
                  next.push_back(std::move(c));
               }
            }
            for (auto& [key, v] : merged) next.push_back(sym_in_set(key.first, key.second, v));
            nt = std::move(next);
         }
         if (nt.size() == 1) return std::move(nt[0]);
         auto o = std::make_unique<Expr>();
         o->k = EK::OR;
         o->ch = std::move(nt);
         return o;
      }
      case EK::NOT: {
         auto o = std::make_unique<Expr>();
         o->k = EK::NOT;
         o->ch.push_back(rewrite(*e.ch[0], t, invert(mode)));
         return o;
      }
      case EK::MAYBE: return rewrite(*e.ch[0], t, Mode::UPPER);
      case EK::EXACT: return rewrite(*e.ch[0], t, Mode::LOWER);
      case EK::NOF: {  // nof.cpp:217-257
         auto rc = [&]() {
            std::vector<EP> v;
            for (const auto& c : e.ch) v.push_back(rewrite(*c, t, mode));
            return v;
         };
         if (mode != Mode::NONE && e.exact && (e.n < 0 || static_cast<size_t>(e.n) < e.ch.size())) {
            auto a = std::make_unique<Expr>();
            a->k = EK::NOF;
            a->ch = rc();
            a->n = e.n;
            auto b = std::make_unique<Expr>();
            b->k = EK::NOF;
            b->ch = rc();
            b->n = e.n + 1;
            auto nb = std::make_unique<Expr>();
            nb->k = EK::NOT;
            nb->ch.push_back(std::move(b));
            auto o = std::make_unique<Expr>();
            o->k = EK::AND;
            o->ch.push_back(std::move(a));
            o->ch.push_back(std::move(nb));
            return o;
         }
         auto o = std::make_unique<Expr>();
         o->k = EK::NOF;
         o->n = e.n;
         o->exact = e.exact;
         o->ch = rc();
         return o;
      }
      case EK::SYM_EQ: {  // symbol_equals.cpp:65-93
         const SeqColumn& c = seq_of(t, e.column);
         if (e.pos >= c.reference.size()) throw IllegalQuery("position out of bounds");
         const int s = e.sym < 0 ? c.reference[e.pos] : e.sym;
         if (mode == Mode::UPPER) return sym_in_set(e.column, e.pos, c.A->ambiguity[s]);
         return sym_in_set(e.column, e.pos, {s});
      }
      case EK::HAS_MUT: {  // has_mutation.cpp:34-68
         const SeqColumn& c = seq_of(t, e.column);
         if (e.pos >= c.reference.size()) throw IllegalQuery("position out of bounds");
         const int ref = c.reference[e.pos];
         std::vector<int> syms;
         for (int s = 0; s < c.A->count; ++s) syms.push_back(s);
         if (mode == Mode::UPPER) {
            syms.erase(std::remove(syms.begin(), syms.end(), ref), syms.end());
         } else {
            for (int a : c.A->ambiguity[ref]) syms.erase(std::remove(syms.begin(), syms.end(), a), syms.end());
         }
         return sym_in_set(e.column, e.pos, syms);
      }
      case EK::MUT_PROFILE: {  // mutation_profile.cpp:172-257
         const SeqColumn& c = seq_of(t, e.column);
         const Alpha& A = *c.A;
         std::vector<int> profile(c.reference.begin(), c.reference.end());
         if (e.by_id) {
            profile = sequence_at_primary_key(t, c, e.value);
         } else if (!e.value.empty()) {
            if (e.value.size() != profile.size()) throw IllegalQuery("querySequence length does not match");
            for (size_t p = 0; p < profile.size(); ++p) {
               profile[p] = A.sym(e.value[p]);
               if (profile[p] < 0) throw IllegalQuery("Invalid symbol in querySequence");
            }
         } else {
            for (int m : e.symbols) {
               if (static_cast<size_t>(m >> 8) >= profile.size()) throw IllegalQuery("mutation position out of bounds");
               profile[m >> 8] = m & 0xFF;
            }
         }
         auto nof = std::make_unique<Expr>();
         nof->k = EK::NOF;
         nof->n = e.n + 1;
         for (size_t p = 0; p < profile.size(); ++p) {
            if (profile[p] == A.missing) continue;
            std::vector<int> diff;
            for (int y = 0; y < A.count; ++y)
               if (!has(A.ambiguity[profile[p]], y)) diff.push_back(y);
            if (diff.empty()) continue;
            nof->ch.push_back(sym_in_set(e.column, static_cast<uint32_t>(p), diff));
         }
         auto o = std::make_unique<Expr>();
         o->k = EK::NOT;
         o->ch.push_back(std::move(nof));
         return o;
      }
      case EK::SYM_IN_SET: throw CompileError("Cannot rewrite SymbolInSet");
      case EK::STR_EQ:
      case EK::DATE_BETWEEN:
      case EK::BOOL: return e.clone();
   }
   throw CompileError("unknown expression");
}

OpP compile(const Expr& e, const Table& t);

OpP compile_symbol_in_set(const Expr& e, const Table& t) {  // symbol_in_set.cpp:230-264
   const SeqColumn& c = seq_of(t, e.column);
   const Layout& L = t.layout;
   if (e.pos >= c.reference.size()) throw IllegalQuery("position out of bounds");
   const Alpha& A = *c.A;
   const int local_ref = c.local_reference[e.pos];
   const bool inc_ref = has(e.symbols, local_ref);
   const bool inc_missing = has(e.symbols, A.missing);
   auto scan = [&](const std::vector<int>& syms) {
      std::vector<bool> m(A.count, false);
      for (int s : syms) m[s] = true;
      return make_scan(c.matching(e.pos, m), L);
   };
   auto exclude_nulls = [&](OpP op) {  // symbol_in_set.cpp:110-126
      if (c.null_bitmap.empty()) return op;
      std::vector<OpP> pos, neg;
      pos.push_back(std::move(op));
      neg.push_back(make_scan(c.null_bitmap, L));
      return make_intersection(std::move(pos), std::move(neg), L);
   };
   Predicate cov;
   cov.kind = Predicate::COVERED;
   cov.seq = &c;
   cov.pos = e.pos;
   if (inc_ref && inc_missing) {
      std::vector<int> neg;
      for (int s = 0; s < A.count; ++s)
         if (!has(e.symbols, s)) neg.push_back(s);
      return exclude_nulls(make_complement(scan(neg), L));
   }
   if (inc_missing) {
      cov.is_covered = false;
      std::vector<OpP> u;
      u.push_back(make_selection(nullptr, {cov}, L));
      u.push_back(scan(e.symbols));
      return exclude_nulls(make_union(std::move(u), L));
   }
   if (inc_ref) {
      std::vector<int> neg;
      for (int s = 0; s < A.count; ++s)
         if (s != A.missing && !has(e.symbols, s)) neg.push_back(s);
      cov.is_covered = true;
      std::vector<OpP> pos, ng;
      pos.push_back(make_selection(nullptr, {cov}, L));
      ng.push_back(scan(neg));
      return make_intersection(std::move(pos), std::move(ng), L);
   }
   return scan(e.symbols);
}

OpP compile(const Expr& e, const Table& t) {
   const Layout& L = t.layout;
   switch (e.k) {
      case EK::AND: {  // and.cpp:91-219
         std::vector<OpP> un, pos, neg;
         std::vector<Predicate> preds;
         for (const auto& c : e.ch) un.push_back(compile(*c, t));
         while (!un.empty()) {
            OpP c = std::move(un.back());
            un.pop_back();
            if (c->type == OT::FULL) continue;
            if (c->type == OT::EMPTY) return mkop(OT::EMPTY, L);
            if (c->type == OT::INTERSECTION) {
               for (auto& g : c->children) pos.push_back(std::move(g));
               for (auto& g : c->negated) neg.push_back(std::move(g));
            } else if (c->type == OT::COMPLEMENT) {
               neg.push_back(negate_op(std::move(c)));
            } else if (c->type == OT::SELECTION) {
               for (const auto& p : c->preds) preds.push_back(p);
               if (c->has_child) un.push_back(std::move(c->children[0]));
            } else {
               pos.push_back(std::move(c));
            }
         }
         if (pos.empty() && neg.empty()) {
            if (preds.empty()) return mkop(OT::FULL, L);
            return make_selection(nullptr, std::move(preds), L);
         }
         OpP op;
         if (pos.size() == 1 && neg.empty()) op = std::move(pos[0]);
         else if (neg.size() == 1 && pos.empty()) op = make_complement(std::move(neg[0]), L);
         else if (pos.empty()) op = make_complement(make_union(std::move(neg), L), L);
         else op = make_intersection(std::move(pos), std::move(neg), L);
         if (preds.empty()) return op;
         return make_selection(std::move(op), std::move(preds), L);
      }
      case EK::OR: {  // or.cpp:194-241
         std::vector<OpP> f;
         for (const auto& c : e.ch) {
            OpP op = compile(*c, t);
            if (op->type == OT::EMPTY) continue;
            if (op->type == OT::FULL) return mkop(OT::FULL, L);
            if (op->type == OT::UNION) {
               for (auto& g : op->children) f.push_back(std::move(g));
            } else {
               f.push_back(std::move(op));
            }
         }
         if (f.empty()) return mkop(OT::EMPTY, L);
         if (f.size() == 1) return std::move(f[0]);
         bool any = false;
         for (const auto& c : f) any = any || c->type == OT::COMPLEMENT;
         if (any) {  // complement.cpp:23-39
            std::vector<OpP> pos, neg;
            for (auto& c : f) {
               if (c->type == OT::COMPLEMENT) neg.push_back(negate_op(std::move(c)));
               else pos.push_back(std::move(c));
            }
            return make_complement(make_intersection(std::move(neg), std::move(pos), L), L);
         }
         return make_union(std::move(f), L);
      }
      case EK::NOT: return negate_op(compile(*e.ch[0], t));
      case EK::NOF: {  // nof.cpp:183-215, 33-150, 259-277
         std::vector<OpP> pos, neg;
         int n = e.n;
         for (const auto& c : e.ch) {
            OpP op = compile(*c, t);
            if (op->type == OT::EMPTY) continue;
            if (op->type == OT::FULL) {
               --n;
               continue;
            }
            if (op->type == OT::COMPLEMENT) {
               neg.push_back(negate_op(std::move(op)));
               continue;
            }
            pos.push_back(std::move(op));
         }
         if (n < 0) return mkop(e.exact ? OT::EMPTY : OT::FULL, L);
         const int k = static_cast<int>(pos.size() + neg.size());
         // handleTrivialCases
         if (n > k) return mkop(OT::EMPTY, L);
         if (n == 0) {
            if (!e.exact) return mkop(OT::FULL, L);
            if (k == 0) return mkop(OT::FULL, L);
            if (k == 1) {
               if (pos.empty()) return std::move(neg[0]);
               return make_complement(std::move(pos[0]), L);
            }
            if (neg.empty()) return make_complement(make_union(std::move(pos), L), L);
            return make_intersection(std::move(neg), std::move(pos), L);
         }
         if (n == 1 && k == 1) {
            if (neg.empty()) return std::move(pos[0]);
            return make_complement(std::move(neg[0]), L);
         }
         if (n == k) {  // handleAndCase
            if (pos.empty()) return make_complement(make_union(std::move(neg), L), L);
            return make_intersection(std::move(pos), std::move(neg), L);
         }
         if (n == 1 && !e.exact) {  // handleOrCase
            if (neg.empty()) return make_union(std::move(pos), L);
            return make_complement(make_intersection(std::move(neg), std::move(pos), L), L);
         }
         return make_threshold(std::move(pos), std::move(neg), static_cast<uint32_t>(n), e.exact, L);
      }
      case EK::SYM_IN_SET: return compile_symbol_in_set(e, t);
      case EK::STR_EQ: {  // equals.cpp:174-187
         const int c = t.find_dict(e.column);
         if (c < 0) throw IllegalQuery("no such indexed string column");
         auto it = t.dict[c].index.find(e.value);
         if (it == t.dict[c].index.end() || it->second.empty()) return mkop(OT::EMPTY, L);
         return make_scan(it->second, L);
      }
      case EK::DATE_BETWEEN: {  // date_between.cpp:61-89
         const int c = t.find_date(e.column);
         if (c < 0) throw IllegalQuery("no such date column");
         Predicate lo, hi;
         lo.kind = hi.kind = Predicate::DATE;
         lo.date = hi.date = &t.date[c];
         lo.cmp = Predicate::GE;
         lo.value = e.from.value_or(INT32_MIN);
         hi.cmp = Predicate::LE;
         hi.value = e.to.value_or(INT32_MAX);
         return make_selection(nullptr, {lo, hi}, L);
      }
      case EK::BOOL: return mkop(e.truth ? OT::FULL : OT::EMPTY, L);
      default: throw CompileError("expression must be rewritten before compilation");
   }
}

RowSet compute_filter(const Table& t, const std::string& text) {  // compute_filter.cpp:14-21
   Parser p{text, t};
   EP e = p.parse();
   EP r = rewrite(*e, t, Mode::NONE);
   OpP op = compile(*r, t);
   return op->evaluate();
}

// ================================================================================================
// Mutations action (mutations_node.cpp:39-288)

std::vector<uint32_t> mutation_counts(const SeqColumn& c, const RowSet& filter, uint64_t sequence_count_in_column) {
   const uint32_t L = c.L;
   const int nsym = c.A->count;
   std::vector<uint32_t> counts(static_cast<size_t>(nsym) * L, 0);
   auto at = [&](int s, uint32_t p) -> uint32_t& { return counts[static_cast<size_t>(s) * L + p]; };
   const uint64_t fc = filter.cardinality();
   if (fc == 0) return counts;
   std::vector<uint32_t> ref(L, 0);
   auto subtract_cumulative = [&](const std::vector<size_t>& starts, const std::vector<size_t>& ends) {
      size_t run = starts.at(L);
      size_t p = L - 1;
      while (true) {
         ref.at(p) -= static_cast<uint32_t>(run);
         run += starts.at(p);
         if (p == 0) break;
         --p;
      }
      run = ends.at(0);
      p = 0;
      while (true) {
         ref.at(p) -= static_cast<uint32_t>(run);
         run += ends.at(p + 1);
         if (p == L - 1) break;
         ++p;
      }
   };
   if (fc == sequence_count_in_column) {  // addMutationCountsForFullBitmaps
      for (auto& x : ref) x += static_cast<uint32_t>(c.sequence_count);
      for (const auto& [g, ivs] : c.horizontal)
         for (const auto& iv : ivs)
            for (uint32_t p = iv.s; p < iv.e; ++p) ref[p] -= 1;
      std::vector<size_t> starts(L + 1), ends(L + 1);
      for (const auto& chunk : c.start_end)
         for (auto [s, e] : chunk) {
            starts.at(s) += 1;
            ends.at(e) += 1;
         }
      subtract_cumulative(starts, ends);
      for (const auto& [key, x] : c.vertical) {
         at(key.symbol, key.position) += x.card;
         ref[key.position] -= x.card;
      }
   } else {  // addMutationCountsForMixedBitmaps
      for (auto& x : ref) x += static_cast<uint32_t>(fc);
      std::vector<size_t> starts(L + 1), ends(L + 1);
      for (const auto& [k, x] : filter.c) {
         auto visit = [&](uint16_t r) {
            const uint32_t g = static_cast<uint32_t>(k) << 16 | r;
            auto it = c.horizontal.find(g);
            if (it != c.horizontal.end())
               for (const auto& iv : it->second)
                  for (uint32_t p = iv.s; p < iv.e; ++p) ref[p] -= 1;
            auto [s, e] = c.coverage_range(g);
            starts.at(s) += 1;
            ends.at(e) += 1;
         };
         if (x.is_bitset) {
            for (uint32_t i = 0; i < 65536; ++i)
               if (x.bits[i >> 6] >> (i & 63) & 1) visit(static_cast<uint16_t>(i));
         } else {
            for (uint16_t r : x.arr) visit(r);
         }
      }
      subtract_cumulative(starts, ends);
      for (const auto& [key, x] : c.vertical) {
         const Ctr* f = filter.find(key.v_index);
         if (!f) continue;
         const uint32_t n = ctr_and_card(*f, x);
         at(key.symbol, key.position) += n;
         ref[key.position] -= n;
      }
   }
   for (uint32_t p = 0; p < L; ++p) at(c.local_reference[p], p) += ref[p];  // accumulateFinalCounts
   return counts;
}

}  // namespace oracle

// ================================================================================================
// C API for the tests

using namespace oracle;

namespace {
thread_local std::string g_err;
template <typename F>
int guard(F&& f) {
   try {
      f();
      return 0;
   } catch (const IllegalQuery& e) {
      g_err = e.what();
      return 1;
   } catch (const CompileError& e) {
      g_err = e.what();
      return 2;
   } catch (const std::exception& e) {
      g_err = e.what();
      return 4;
   }
}
void rowset_to_bits(const RowSet& r, uint32_t* out, size_t nchunks) {
   std::memset(out, 0, nchunks * 2048 * 4);
   for (const auto& [k, x] : r.c) {
      const std::vector<uint64_t> b = x.to_bits();
      std::memcpy(out + static_cast<size_t>(k) * 2048, b.data(), 8192);
   }
}
}  // namespace

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

int oracle_build(const ORawTable* raw, void** out) {
   return guard([&] { *out = new Table(build_table(*raw)); });
}

void oracle_free(void* t) { delete static_cast<Table*>(t); }

int oracle_set_primary_key(void* t, const char* dict_column) {
   return guard([&] {
      Table& tab = *static_cast<Table*>(t);
      tab.primary_key = dict_column ? tab.find_dict(dict_column) : -1;
      if (dict_column && tab.primary_key < 0) throw IllegalQuery("no such dictionary column");
   });
}

int oracle_count(void* t, const char* expr, uint64_t* out) {
   return guard([&] { *out = compute_filter(*static_cast<Table*>(t), expr).cardinality(); });
}

int oracle_filter(void* t, const char* expr, uint32_t* bits, uint64_t* count) {
   return guard([&] {
      const Table& tab = *static_cast<Table*>(t);
      RowSet r = compute_filter(tab, expr);
      if (bits) rowset_to_bits(r, bits, tab.layout.chunk_sizes.size());
      if (count) *count = r.cardinality();
   });
}

int oracle_mutations(void* t, const char* expr, uint32_t column, uint32_t* counts, uint64_t* filter_count) {
   return guard([&] {
      const Table& tab = *static_cast<Table*>(t);
      const RowSet r = compute_filter(tab, expr);
      const auto c = mutation_counts(tab.seq.at(column), r, tab.layout.num_rows);
      std::memcpy(counts, c.data(), c.size() * 4);
      if (filter_count) *filter_count = r.cardinality();
   });
}

// addMutationsToOutput (mutations_node.cpp:292-366): rows as (position, from, to, count, coverage, proportion).
int oracle_mutation_rows(void* t, uint32_t column, const uint32_t* counts, double min_proportion, uint32_t* pos,
                         char* from, char* to, uint32_t* count, uint32_t* coverage, double* proportion, size_t cap,
                         size_t* n_rows) {
   return guard([&] {
      const SeqColumn& c = static_cast<Table*>(t)->seq.at(column);
      size_t n = 0;
      for (uint32_t p = 0; p < c.L; ++p) {
         uint32_t total = 0;
         for (int s : c.A->valid) total += counts[static_cast<size_t>(s) * c.L + p];
         if (total == 0) continue;
         const uint32_t thr =
            min_proportion == 0 ? 0 : static_cast<uint32_t>(std::ceil(static_cast<double>(total) * min_proportion) - 1);
         const int gref = c.reference[p];
         for (int s : c.A->valid) {
            if (s == gref) continue;
            const uint32_t k = counts[static_cast<size_t>(s) * c.L + p];
            if (k > thr) {
               if (n < cap) {
                  pos[n] = p + 1;
                  from[n] = c.A->chars[gref];
                  to[n] = c.A->chars[s];
                  count[n] = k;
                  coverage[n] = total;
                  proportion[n] = static_cast<double>(k) / static_cast<double>(total);
               }
               ++n;
            }
         }
      }
      *n_rows = n;
   });
}

int oracle_local_reference(void* t, uint32_t column, char* out) {
   return guard([&] {
      const SeqColumn& c = static_cast<Table*>(t)->seq.at(column);
      for (uint32_t p = 0; p < c.L; ++p) out[p] = c.A->chars[c.local_reference[p]];
   });
}

// Vertical index summary: per container (position, v_index, symbol, cardinality), in map order.
int oracle_vertical(void* t, uint32_t column, uint32_t* pos, uint16_t* v, uint8_t* sym, uint32_t* card, size_t cap,
                    size_t* n) {
   return guard([&] {
      const SeqColumn& c = static_cast<Table*>(t)->seq.at(column);
      size_t i = 0;
      for (const auto& [k, x] : c.vertical) {
         if (i < cap) {
            pos[i] = k.position;
            v[i] = k.v_index;
            sym[i] = static_cast<uint8_t>(k.symbol);
            card[i] = x.card;
         }
         ++i;
      }
      *n = i;
   });
}

// Coverage of one row: start, end and the missing intervals inside coverage.
int oracle_row_coverage(void* t, uint32_t column, uint32_t row, uint32_t* start, uint32_t* end, uint32_t* ivs,
                        size_t cap, size_t* n) {
   return guard([&] {
      const SeqColumn& c = static_cast<Table*>(t)->seq.at(column);
      auto [s, e] = c.coverage_range(row);
      *start = s;
      *end = e;
      auto it = c.horizontal.find(row);
      size_t i = 0;
      if (it != c.horizontal.end()) {
         for (const auto& iv : it->second) {
            if (2 * i + 1 < cap) {
               ivs[2 * i] = iv.s;
               ivs[2 * i + 1] = iv.e;
            }
            ++i;
         }
      }
      *n = i;
   });
}

// The reference's string diff, for comparing with the run-based ingestion on small inputs.
int oracle_diff_string(int kind, const char* seq, const char* ref, uint32_t* start, uint32_t* end, uint32_t* missing,
                       size_t* n_missing, uint32_t* mut_pos, uint8_t* mut_sym, size_t* n_mut, size_t cap) {
   return guard([&] {
      const Diff d = diff_string(seq, ref, kind == 0 ? nuc() : aa());
      *start = d.start;
      *end = d.end;
      *n_missing = d.missing.size();
      *n_mut = d.mutations.size();
      for (size_t i = 0; i < d.missing.size() && i < cap; ++i) missing[i] = d.missing[i];
      for (size_t i = 0; i < d.mutations.size() && i < cap; ++i) {
         mut_pos[i] = d.mutations[i].first;
         mut_sym[i] = static_cast<uint8_t>(d.mutations[i].second);
      }
   });
}

// Known-answer harness for the operators: evaluate an operator over explicit row sets.
// kind: 0 = Threshold(n, exact), 1 = Intersection, 2 = Union, 3 = Complement of sets[0].
// sets are given as concatenated sorted row lists with offsets.
int oracle_operator(int kind, const uint32_t* chunk_sizes, uint32_t n_chunks, const uint32_t* rows, const uint64_t* off,
                    uint32_t n_pos, uint32_t n_neg, uint32_t n, int exact, uint32_t* out, size_t cap, size_t* n_out) {
   return guard([&] {
      Layout L;
      for (uint32_t i = 0; i < n_chunks; ++i) {
         L.chunk_sizes.push_back(chunk_sizes[i]);
         L.num_rows += chunk_sizes[i];
      }
      std::vector<OpP> pos, neg;
      for (uint32_t i = 0; i < n_pos + n_neg; ++i) {
         std::vector<uint32_t> v(rows + off[i], rows + off[i + 1]);
         (i < n_pos ? pos : neg).push_back(make_scan(rs_from_sorted_rows(v), L));
      }
      OpP op;
      if (kind == 0) op = make_threshold(std::move(pos), std::move(neg), n, exact != 0, L);
      else if (kind == 1) op = make_intersection(std::move(pos), std::move(neg), L);
      else if (kind == 2) op = make_union(std::move(pos), L);
      else op = make_complement(std::move(pos[0]), L);
      const RowSet r = op->evaluate();
      size_t i = 0;
      for (const auto& [k, x] : r.c) {
         const std::vector<uint64_t> b = x.to_bits();
         for (uint32_t j = 0; j < 65536; ++j)
            if (b[j >> 6] >> (j & 63) & 1) {
               if (i < cap) out[i] = static_cast<uint32_t>(k) << 16 | j;
               ++i;
            }
      }
      *n_out = i;
   });
}

// CPU baseline: runs queries the way the reference serves them, one query per worker thread.
// action[i]: 0 = count, 1 = mutations of column `column[i]`. Returns wall seconds and per-query ms.
int oracle_run_batch(void* t, const char* const* exprs, const int* action, const uint32_t* column, uint32_t n,
                     uint32_t threads, uint64_t* counts, double* ms, double* seconds) {
   return guard([&] {
      const Table& tab = *static_cast<Table*>(t);
      std::atomic<uint32_t> next{0};
      std::atomic<int> failed{0};
      auto body = [&]() {
         for (uint32_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
            const auto t0 = std::chrono::steady_clock::now();
            try {
               const RowSet r = compute_filter(tab, exprs[i]);
               counts[i] = r.cardinality();
               if (action[i] == 1) {
                  const auto c = mutation_counts(tab.seq.at(column[i]), r, tab.layout.num_rows);
                  uint64_t sum = 0;
                  for (uint32_t x : c) sum += x;
                  counts[i] ^= sum << 1;
               }
            } catch (...) {
               failed = 1;
            }
            ms[i] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
         }
      };
      const auto t0 = std::chrono::steady_clock::now();
      std::vector<std::thread> pool;
      for (uint32_t k = 0; k < std::max(1u, threads); ++k) pool.emplace_back(body);
      for (auto& th : pool) th.join();
      *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (failed) throw std::runtime_error("a query failed in the batch");
   });
}

// Many queries on `threads` worker threads (the checker of large parity runs): counts[i] receives
// the filter cardinality of query i; for every i with tables[i] != NULL the Mutations counts of
// column[i] (n_symbols * L words, counts[symbol * L + position]) are written there.
int oracle_check_batch(void* t, const char* const* exprs, const uint32_t* column, uint32_t n, uint32_t threads,
                       uint64_t* counts, uint32_t* const* tables) {
   return guard([&] {
      const Table& tab = *static_cast<Table*>(t);
      std::atomic<uint32_t> next{0};
      std::atomic<int> failed{0};
      std::string first_error;
      std::mutex err_mu;
      auto body = [&]() {
         for (uint32_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
            try {
               const RowSet r = compute_filter(tab, exprs[i]);
               counts[i] = r.cardinality();
               if (tables && tables[i]) {
                  const auto c = mutation_counts(tab.seq.at(column[i]), r, tab.layout.num_rows);
                  std::copy(c.begin(), c.end(), tables[i]);
               }
            } catch (const std::exception& e) {
               std::lock_guard<std::mutex> lock(err_mu);
               if (!failed.exchange(1)) first_error = std::string(exprs[i]) + ": " + e.what();
            }
         }
      };
      std::vector<std::thread> pool;
      for (uint32_t k = 0; k < std::max(1u, threads); ++k) pool.emplace_back(body);
      for (auto& th : pool) th.join();
      if (failed) throw std::runtime_error("a query failed: " + first_error);
   });
}

}  // extern "C"
