// Seeded synthetic table generator and random filter-expression generator.
//
// Distribution (per row): Poisson(subs_mean) substitutions drawn Zipf(zipf_s) by rank from a pool of
// (position, symbol) sites, Poisson(gap_mean) gap runs of length U[gap_min, gap_max] and
// Poisson(nrun_mean) N-runs of length U[nrun_min, nrun_max] at uniform starts. Later layers
// overwrite earlier ones (substitutions < gaps < N). Amino-acid genes are the standard-code
// translation of the nucleotide sequence. Every draw comes from a per-row generator seeded from
// (seed, row), so the table is identical for any thread count.
#include "dataset.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <thread>

namespace rhygpu {
namespace {

struct Rng {
   uint64_t s[4];
   static uint64_t splitmix(uint64_t& x) {
      uint64_t z = (x += 0x9E3779B97F4A7C15ull);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      return z ^ (z >> 31);
   }
   explicit Rng(uint64_t seed) {
      uint64_t x = seed;
      for (auto& v : s) v = splitmix(x);
   }
   static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
   uint64_t next() {
      const uint64_t result = rotl(s[1] * 5, 7) * 9;
      const uint64_t t = s[1] << 17;
      s[2] ^= s[0];
      s[3] ^= s[1];
      s[1] ^= s[2];
      s[0] ^= s[3];
      s[2] ^= t;
      s[3] = rotl(s[3], 45);
      return result;
   }
   double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
   uint32_t below(uint32_t n) { return static_cast<uint32_t>((static_cast<unsigned __int128>(next()) * n) >> 64); }
   uint32_t range(uint32_t lo, uint32_t hi) { return lo + below(hi - lo + 1); }  // inclusive
   uint32_t poisson(double exp_neg_lambda) {
      // Knuth: count uniforms until their product drops below e^-lambda.
      uint32_t k = 0;
      double p = uniform();
      while (p > exp_neg_lambda) {
         ++k;
         p *= uniform();
      }
      return k;
   }
};

uint64_t row_seed(uint64_t seed, uint64_t stream, uint64_t row) {
   uint64_t x = seed * 0x100000001B3ull ^ (stream << 48) ^ row;
   return Rng::splitmix(x);
}

struct Zipf {
   std::vector<double> cdf;
   Zipf(uint32_t n, double s) : cdf(n) {
      double acc = 0;
      for (uint32_t k = 0; k < n; ++k) {
         acc += 1.0 / std::pow(static_cast<double>(k + 1), s);
         cdf[k] = acc;
      }
      for (auto& c : cdf) c /= acc;
   }
   uint32_t sample(Rng& r) const {
      const double u = r.uniform();
      auto it = std::upper_bound(cdf.begin(), cdf.end(), u);
      if (it == cdf.end()) --it;
      return static_cast<uint32_t>(it - cdf.begin());
   }
};

struct Interval {
   uint32_t s, e;  // [s, e)
};

void merge_intervals(std::vector<Interval>& v) {
   if (v.empty()) return;
   std::sort(v.begin(), v.end(), [](const Interval& a, const Interval& b) { return a.s < b.s; });
   size_t w = 0;
   for (size_t i = 1; i < v.size(); ++i) {
      if (v[i].s <= v[w].e) {
         v[w].e = std::max(v[w].e, v[i].e);
      } else {
         v[++w] = v[i];
      }
   }
   v.resize(w + 1);
}

// a \ b for sorted, merged interval lists.
std::vector<Interval> subtract_intervals(const std::vector<Interval>& a, const std::vector<Interval>& b) {
   std::vector<Interval> out;
   size_t j = 0;
   for (const auto& iv : a) {
      uint32_t cur = iv.s;
      while (j < b.size() && b[j].e <= cur) ++j;
      size_t k = j;
      while (k < b.size() && b[k].s < iv.e) {
         if (b[k].s > cur) out.push_back({cur, b[k].s});
         cur = std::max(cur, b[k].e);
         ++k;
      }
      if (cur < iv.e) out.push_back({cur, iv.e});
   }
   return out;
}

bool inside(const std::vector<Interval>& v, uint32_t p) {
   auto it = std::upper_bound(v.begin(), v.end(), p, [](uint32_t x, const Interval& iv) { return x < iv.s; });
   if (it == v.begin()) return false;
   --it;
   return p < it->e;
}

struct RowRuns {
   std::vector<uint32_t> pos, len;
   std::vector<char> ch;
   void clear() {
      pos.clear();
      len.clear();
      ch.clear();
   }
};

struct NucRowGen {
   const GenConfig& cfg;
   const std::vector<PoolSite>& pool;
   const Zipf& zipf;
   double e_subs, e_gap, e_n;

   // Produces the sorted, non-overlapping runs of one row.
   void make(Rng& r, RowRuns& out) const {
      out.clear();
      const uint32_t L = cfg.genome_len;
      const uint32_t nsubs = r.poisson(e_subs);
      std::vector<std::pair<uint32_t, char>> subs;
      subs.reserve(nsubs);
      for (uint32_t i = 0; i < nsubs; ++i) {
         const PoolSite& site = pool[zipf.sample(r)];
         subs.emplace_back(site.pos, site.ch);
      }
      std::vector<Interval> gaps, ns;
      const uint32_t ngap = r.poisson(e_gap);
      for (uint32_t i = 0; i < ngap; ++i) {
         const uint32_t s = r.below(L);
         const uint32_t l = r.range(cfg.gap_min, cfg.gap_max);
         gaps.push_back({s, std::min(L, s + l)});
      }
      const uint32_t nn = r.poisson(e_n);
      for (uint32_t i = 0; i < nn; ++i) {
         const uint32_t s = r.below(L);
         const uint32_t l = r.range(cfg.nrun_min, cfg.nrun_max);
         ns.push_back({s, std::min(L, s + l)});
      }
      merge_intervals(ns);
      merge_intervals(gaps);
      gaps = subtract_intervals(gaps, ns);
      // Later substitutions at the same position overwrite earlier ones.
      std::stable_sort(subs.begin(), subs.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
      std::vector<std::pair<uint32_t, char>> kept;
      for (size_t i = 0; i < subs.size(); ++i) {
         if (i + 1 < subs.size() && subs[i + 1].first == subs[i].first) continue;
         if (inside(ns, subs[i].first) || inside(gaps, subs[i].first)) continue;
         kept.push_back(subs[i]);
      }
      // Emit in position order.
      size_t a = 0, b = 0, c = 0;
      while (a < ns.size() || b < gaps.size() || c < kept.size()) {
         const uint32_t pa = a < ns.size() ? ns[a].s : UINT32_MAX;
         const uint32_t pb = b < gaps.size() ? gaps[b].s : UINT32_MAX;
         const uint32_t pc = c < kept.size() ? kept[c].first : UINT32_MAX;
         if (pa <= pb && pa <= pc) {
            out.pos.push_back(pa);
            out.len.push_back(ns[a].e - ns[a].s);
            out.ch.push_back('N');
            ++a;
         } else if (pb <= pc) {
            out.pos.push_back(pb);
            out.len.push_back(gaps[b].e - gaps[b].s);
            out.ch.push_back('-');
            ++b;
         } else {
            out.pos.push_back(pc);
            out.len.push_back(1);
            out.ch.push_back(kept[c].second);
            ++c;
         }
      }
   }
};

// Character of a row at nucleotide position q; `cursor` walks forward over the sorted runs.
struct RowCursor {
   const RowRuns& runs;
   const std::string& ref;
   size_t cursor = 0;
   char at(uint32_t q) {
      while (cursor < runs.pos.size() && runs.pos[cursor] + runs.len[cursor] <= q) ++cursor;
      if (cursor < runs.pos.size() && runs.pos[cursor] <= q) return runs.ch[cursor];
      return ref[q];
   }
};

void translate_row(const RowRuns& nuc, const std::string& nuc_ref, const Gene& g, const std::string& aa_ref,
                   RowRuns& out) {
   out.clear();
   const uint32_t gs = g.nuc_start, ge = g.nuc_start + 3 * g.aa_len;
   std::vector<Interval> codons;
   for (size_t i = 0; i < nuc.pos.size(); ++i) {
      const uint32_t s = std::max(nuc.pos[i], gs);
      const uint32_t e = std::min(nuc.pos[i] + nuc.len[i], ge);
      if (s >= e) continue;
      codons.push_back({(s - gs) / 3, (e - 1 - gs) / 3 + 1});
   }
   merge_intervals(codons);
   RowCursor cur{nuc, nuc_ref};
   for (const auto& iv : codons) {
      for (uint32_t c = iv.s; c < iv.e; ++c) {
         const uint32_t q = gs + 3 * c;
         const char x = cur.at(q), y = cur.at(q + 1), z = cur.at(q + 2);
         const char aa = translate_codon(x, y, z);
         if (aa == aa_ref[c]) continue;
         if (!out.pos.empty() && out.ch.back() == aa && out.pos.back() + out.len.back() == c) {
            out.len.back() += 1;
         } else {
            out.pos.push_back(c);
            out.len.push_back(1);
            out.ch.push_back(aa);
         }
      }
   }
}

std::vector<Gene> default_genes(uint32_t genome_len, uint32_t n_genes) {
   std::vector<Gene> genes;
   if (n_genes == 0) return genes;
   static const char* names[12] = {"ORF1a", "ORF1b", "S", "ORF3a", "E", "M",
                                   "ORF6", "ORF7a", "ORF7b", "ORF8", "N", "ORF9b"};
   static const uint32_t lens[12] = {4400, 2690, 1270, 275, 75, 222, 61, 121, 43, 121, 322, 100};  // 9,700 aa
   if (n_genes == 12 && genome_len >= 265 + 3 * 9700) {
      uint32_t start = 265;
      for (int i = 0; i < 12; ++i) {
         genes.push_back({names[i], start, lens[i]});
         start += 3 * lens[i];
      }
      return genes;
   }
   // Small genomes: split the genome evenly.
   const uint32_t usable = genome_len > 6 ? (genome_len - 6) / 3 : 0;
   const uint32_t per = usable / n_genes;
   if (per == 0) throw std::invalid_argument("genome too short for the requested genes");
   uint32_t start = 3;
   for (uint32_t i = 0; i < n_genes; ++i) {
      char buf[32];
      std::snprintf(buf, sizeof(buf), "%s", i < 12 ? names[i] : "G");
      std::string nm = buf;
      if (i >= 12) nm += std::to_string(i);
      genes.push_back({nm, start, per});
      start += 3 * per;
   }
   return genes;
}

template <typename F>
void parallel_blocks(uint32_t n_blocks, uint32_t threads, F&& fn) {
   if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
   threads = std::min(threads, std::max(1u, n_blocks));
   std::vector<std::thread> pool;
   std::atomic<uint32_t> next{0};
   for (uint32_t t = 0; t < threads; ++t) {
      pool.emplace_back([&]() {
         for (uint32_t b = next.fetch_add(1); b < n_blocks; b = next.fetch_add(1)) fn(b);
      });
   }
   for (auto& th : pool) th.join();
}

}  // namespace

GeneratedTable generate_table(const GenConfig& cfg) {
   if (cfg.genome_len == 0) throw std::invalid_argument("genome_len must be positive");
   GeneratedTable out;
   RawTable& t = out.table;
   t.n_rows = cfg.n_rows;
   Rng grng(row_seed(cfg.seed, 0xFFFF, 0));

   // Reference over ACGT.
   static const char acgt[4] = {'A', 'C', 'G', 'T'};
   std::string ref(cfg.genome_len, 'A');
   for (auto& c : ref) c = acgt[grng.below(4)];

   // Pool of (position, symbol) sites.
   static const char ambig[10] = {'R', 'Y', 'S', 'W', 'K', 'M', 'B', 'D', 'H', 'V'};
   out.pool.resize(cfg.pool_sites);
   for (auto& site : out.pool) {
      site.pos = grng.below(cfg.genome_len);
      if (grng.uniform() < cfg.pool_ambiguous_fraction) {
         site.ch = ambig[grng.below(10)];
      } else {
         char c;
         do {
            c = acgt[grng.below(4)];
         } while (c == ref[site.pos]);
         site.ch = c;
      }
   }
   out.genes = default_genes(cfg.genome_len, cfg.n_aa_genes);

   std::vector<std::string> aa_refs;
   for (const auto& g : out.genes) {
      std::string a(g.aa_len, 'X');
      for (uint32_t c = 0; c < g.aa_len; ++c) {
         const uint32_t q = g.nuc_start + 3 * c;
         a[c] = translate_codon(ref[q], ref[q + 1], ref[q + 2]);
      }
      aa_refs.push_back(std::move(a));
   }
   // Amino-acid sites reachable by one pool substitution.
   for (uint32_t gi = 0; gi < out.genes.size(); ++gi) {
      const Gene& g = out.genes[gi];
      for (const auto& site : out.pool) {
         if (site.pos < g.nuc_start || site.pos >= g.nuc_start + 3 * g.aa_len) continue;
         const uint32_t c = (site.pos - g.nuc_start) / 3;
         char cod[3] = {ref[g.nuc_start + 3 * c], ref[g.nuc_start + 3 * c + 1], ref[g.nuc_start + 3 * c + 2]};
         cod[(site.pos - g.nuc_start) % 3] = site.ch;
         const char aa = translate_codon(cod[0], cod[1], cod[2]);
         if (aa == aa_refs[gi][c] || aa == 'X') continue;
         out.aa_site_gene.push_back(gi);
         out.aa_site_pos.push_back(c);
         out.aa_site_char.push_back(aa);
      }
   }

   const Zipf zipf(std::max(1u, cfg.pool_sites), cfg.zipf_s);
   NucRowGen gen{cfg, out.pool, zipf, std::exp(-cfg.subs_mean), std::exp(-cfg.gap_mean), std::exp(-cfg.nrun_mean)};

   const uint32_t n_cols = 1 + static_cast<uint32_t>(out.genes.size());
   const uint32_t block = 1u << 14;
   const uint32_t n_blocks = (cfg.n_rows + block - 1) / block;
   struct BlockOut {
      std::vector<RowRuns> cols;             // concatenated runs of the block's rows
      std::vector<std::vector<uint32_t>> counts;  // runs per row per column
      std::vector<uint8_t> nulls;
   };
   std::vector<BlockOut> blocks(n_blocks);
   parallel_blocks(n_blocks, cfg.threads, [&](uint32_t b) {
      BlockOut& bo = blocks[b];
      bo.cols.resize(n_cols);
      bo.counts.assign(n_cols, {});
      const uint32_t r0 = b * block, r1 = std::min(cfg.n_rows, r0 + block);
      RowRuns nuc, aa;
      for (uint32_t row = r0; row < r1; ++row) {
         Rng r(row_seed(cfg.seed, 1, row));
         const bool is_null = cfg.null_fraction > 0 && r.uniform() < cfg.null_fraction;
         bo.nulls.push_back(is_null ? 1 : 0);
         if (is_null) {
            for (uint32_t c = 0; c < n_cols; ++c) bo.counts[c].push_back(0);
            continue;
         }
         gen.make(r, nuc);
         auto append = [&](uint32_t c, const RowRuns& rr) {
            RowRuns& dst = bo.cols[c];
            dst.pos.insert(dst.pos.end(), rr.pos.begin(), rr.pos.end());
            dst.len.insert(dst.len.end(), rr.len.begin(), rr.len.end());
            dst.ch.insert(dst.ch.end(), rr.ch.begin(), rr.ch.end());
            bo.counts[c].push_back(static_cast<uint32_t>(rr.pos.size()));
         };
         append(0, nuc);
         for (uint32_t gi = 0; gi < out.genes.size(); ++gi) {
            translate_row(nuc, ref, out.genes[gi], aa_refs[gi], aa);
            append(1 + gi, aa);
         }
      }
   });

   t.seq.resize(n_cols);
   for (uint32_t c = 0; c < n_cols; ++c) {
      RawSeqColumn& col = t.seq[c];
      if (c == 0) {
         col.name = "main";
         col.kind = SymKind::NUC;
         col.reference = ref;
      } else {
         col.name = out.genes[c - 1].name;
         col.kind = SymKind::AA;
         col.reference = aa_refs[c - 1];
      }
      col.is_null.reserve(cfg.n_rows);
      col.row_off.reserve(cfg.n_rows + 1);
      col.row_off.push_back(0);
      size_t total = 0;
      for (const auto& bo : blocks) total += bo.cols[c].pos.size();
      col.run_pos.reserve(total);
      col.run_len.reserve(total);
      col.run_char.reserve(total);
      for (const auto& bo : blocks) {
         col.is_null.insert(col.is_null.end(), bo.nulls.begin(), bo.nulls.end());
         col.run_pos.insert(col.run_pos.end(), bo.cols[c].pos.begin(), bo.cols[c].pos.end());
         col.run_len.insert(col.run_len.end(), bo.cols[c].len.begin(), bo.cols[c].len.end());
         col.run_char.insert(col.run_char.end(), bo.cols[c].ch.begin(), bo.cols[c].ch.end());
         for (uint32_t n : bo.counts[c]) col.row_off.push_back(col.row_off.back() + n);
      }
   }
   blocks.clear();

   // Metadata columns.
   RawDictColumn country{"country", {}, {}}, lineage{"lineage", {}, {}};
   for (uint32_t i = 0; i < cfg.n_countries; ++i) {
      char buf[32];
      std::snprintf(buf, sizeof(buf), "country_%03u", i);
      country.values.push_back(buf);
   }
   for (uint32_t i = 0; i < cfg.n_lineages; ++i) {
      char buf[32];
      std::snprintf(buf, sizeof(buf), "lineage_%04u", i);
      lineage.values.push_back(buf);
   }
   RawDateColumn date{"date", {}};
   country.ids.resize(cfg.n_rows);
   lineage.ids.resize(cfg.n_rows);
   date.days.resize(cfg.n_rows);
   const Zipf zc(std::max(1u, cfg.n_countries), 1.1), zl(std::max(1u, cfg.n_lineages), 1.0);
   parallel_blocks(n_blocks, cfg.threads, [&](uint32_t b) {
      const uint32_t r0 = b * block, r1 = std::min(cfg.n_rows, r0 + block);
      for (uint32_t row = r0; row < r1; ++row) {
         Rng r(row_seed(cfg.seed, 2, row));
         country.ids[row] = zc.sample(r);
         lineage.ids[row] = zl.sample(r);
         date.days[row] = cfg.date_base + static_cast<int32_t>(r.below(cfg.date_days));
      }
   });
   t.dict.push_back(std::move(country));
   t.dict.push_back(std::move(lineage));
   t.date.push_back(std::move(date));
   return out;
}

std::string materialize_row(const RawSeqColumn& col, uint32_t row) {
   std::string s = col.reference;
   if (col.is_null[row]) return std::string();
   for (uint64_t i = col.row_off[row]; i < col.row_off[row + 1]; ++i) {
      for (uint32_t k = 0; k < col.run_len[i]; ++k) s[col.run_pos[i] + k] = col.run_char[i];
   }
   return s;
}

// ------------------------------------------------------------------------------------------------
// Query generator

namespace {

struct QGen {
   const GeneratedTable& g;
   const QueryGenConfig& cfg;
   Rng r;

   std::string nuc_leaf() {
      const auto& pool = g.pool;
      const uint32_t L = static_cast<uint32_t>(g.table.seq[0].reference.size());
      // Bias towards frequent (low-rank) sites so that selectivities spread over many decades.
      auto pick_site = [&]() -> const PoolSite& {
         const uint32_t lim = r.uniform() < 0.6 ? std::min<uint32_t>(200, pool.size()) : pool.size();
         return pool[r.below(lim)];
      };
      const double u = r.uniform();
      char buf[96];
      if (u < 0.55) {
         const PoolSite& s = pick_site();
         std::snprintf(buf, sizeof(buf), "SymEq(main,%u,%c)", s.pos + 1, s.ch);
      } else if (u < 0.75) {
         const PoolSite& s = pick_site();
         std::snprintf(buf, sizeof(buf), "HasMut(main,%u)", s.pos + 1);
      } else if (u < 0.85) {
         const PoolSite& s = pick_site();
         std::snprintf(buf, sizeof(buf), "SymEq(main,%u,.)", s.pos + 1);
      } else if (u < 0.90) {
         std::snprintf(buf, sizeof(buf), "SymEq(main,%u,N)", r.below(L) + 1);
      } else if (u < 0.95) {
         const PoolSite& s = pick_site();
         static const char some[6] = {'A', 'C', 'G', 'T', '-', 'R'};
         std::snprintf(buf, sizeof(buf), "SymEq(main,%u,%c)", s.pos + 1, some[r.below(6)]);
      } else {
         std::snprintf(buf, sizeof(buf), "SymEq(main,%u,-)", r.below(L) + 1);
      }
      return buf;
   }

   std::string aa_leaf() {
      char buf[96];
      if (g.aa_site_pos.empty()) return nuc_leaf();
      const uint32_t i = r.below(static_cast<uint32_t>(g.aa_site_pos.size()));
      const std::string& gene = g.genes[g.aa_site_gene[i]].name;
      const double u = r.uniform();
      if (u < 0.6) {
         std::snprintf(buf, sizeof(buf), "SymEq(%s,%u,%c)", gene.c_str(), g.aa_site_pos[i] + 1, g.aa_site_char[i]);
      } else if (u < 0.85) {
         std::snprintf(buf, sizeof(buf), "HasMut(%s,%u)", gene.c_str(), g.aa_site_pos[i] + 1);
      } else if (u < 0.95) {
         std::snprintf(buf, sizeof(buf), "SymEq(%s,%u,.)", gene.c_str(), g.aa_site_pos[i] + 1);
      } else {
         std::snprintf(buf, sizeof(buf), "SymEq(%s,%u,X)", gene.c_str(), g.aa_site_pos[i] + 1);
      }
      return buf;
   }

   std::string meta_leaf() {
      const double u = r.uniform();
      char buf[96];
      if (u < 0.35) {
         const auto& c = g.table.dict[0];
         std::snprintf(buf, sizeof(buf), "StrEq(country,%s)", c.values[r.below(std::min<uint32_t>(40, c.values.size()))].c_str());
      } else if (u < 0.6) {
         const auto& c = g.table.dict[1];
         std::snprintf(buf, sizeof(buf), "StrEq(lineage,%s)", c.values[r.below(std::min<uint32_t>(300, c.values.size()))].c_str());
      } else {
         const int32_t base = 18262;
         const int32_t lo = base + static_cast<int32_t>(r.below(1096));
         const int32_t hi = lo + static_cast<int32_t>(r.below(400));
         const double v = r.uniform();
         if (v < 0.15) {
            std::snprintf(buf, sizeof(buf), "DateBetween(date,*,%d)", hi);
         } else if (v < 0.3) {
            std::snprintf(buf, sizeof(buf), "DateBetween(date,%d,*)", lo);
         } else {
            std::snprintf(buf, sizeof(buf), "DateBetween(date,%d,%d)", lo, hi);
         }
      }
      return buf;
   }

   std::string leaf() {
      const double u = r.uniform();
      std::string e;
      if (cfg.use_metadata && u < 0.2) {
         e = meta_leaf();
      } else if (cfg.use_aa && u < 0.45) {
         e = aa_leaf();
      } else {
         e = nuc_leaf();
      }
      if (cfg.use_ambiguity) {
         const double w = r.uniform();
         if (w < 0.04) return "Maybe(" + e + ")";
         if (w < 0.06) return "Exact(" + e + ")";
      }
      return e;
   }

   // A subtree using at most `budget` leaves (decremented by the leaves used); with no leaf limit
   // the budget never binds, so the random stream is the same as without one.
   std::string expr(uint32_t depth, uint32_t& budget) {
      if (depth >= cfg.max_depth || r.uniform() < 0.25 + 0.15 * depth || budget <= 1) {
         --budget;
         return leaf();
      }
      // children share the budget: each leaves one leaf for every later sibling
      auto child = [&](uint32_t i, uint32_t k) {
         uint32_t b = budget - (k - 1 - i);
         const uint32_t before = b;
         std::string c = expr(depth + 1, b);
         budget -= before - b;
         return c;
      };
      const double u = r.uniform();
      if (u < 0.15) return "Not(" + child(0, 1) + ")";
      if (u < 0.75) {
         const uint32_t k = std::min(2 + r.below(3), budget);
         std::string s = u < 0.45 ? "And(" : "Or(";
         for (uint32_t i = 0; i < k; ++i) {
            if (i) s += ",";
            s += child(i, k);
         }
         return s + ")";
      }
      const uint32_t k = std::min(1 + r.below(std::max(1u, cfg.max_nof_children)), budget);
      const uint32_t n = r.below(k + 2);  // 0..k+1 exercises the trivial cases
      const bool exact = r.uniform() < 0.3;
      std::string s = "NOf(" + std::to_string(n) + (exact ? ",exactly" : ",atleast");
      for (uint32_t i = 0; i < k; ++i) s += "," + child(i, k);
      s += ")";
      if (cfg.use_ambiguity && r.uniform() < 0.05) return "Maybe(" + s + ")";
      return s;
   }
};

}  // namespace

std::vector<std::string> generate_queries(const GeneratedTable& g, const QueryGenConfig& cfg) {
   QGen q{g, cfg, Rng(row_seed(cfg.seed, 3, 0))};
   std::vector<std::string> out;
   out.reserve(cfg.n_queries);
   for (uint32_t i = 0; i < cfg.n_queries; ++i) {
      uint32_t budget = cfg.max_leaves ? cfg.max_leaves : 0x40000000u;
      out.push_back(q.expr(0, budget));
   }
   return out;
}

}  // namespace rhygpu
