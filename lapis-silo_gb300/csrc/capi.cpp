// extern "C" boundary (include/rhydb_gpu.h). No exception crosses it: every entry point maps
// exceptions to a status code and a thread-local message.
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/rhydb_gpu.h"
#include "dataset.h"
#include "engine.h"
#include "expr.h"
#include "table.h"

struct RhyTable {
   rhygpu::GeneratedTable gen;  // raw input (generated or copied from the caller)
   rhygpu::TableImage image;
   std::vector<RhyRawSeqColumn> raw_seq;
   std::vector<RhyRawDictColumn> raw_dict;
   std::vector<RhyRawDateColumn> raw_date;
   std::vector<std::vector<const char*>> dict_values;
};

struct RhyDevice {
   const RhyTable* table;
   std::unique_ptr<rhygpu::Engine> engine;
};

namespace {

thread_local std::string g_last_error;

template <typename F>
int guarded(F&& fn) {
   try {
      fn();
      g_last_error.clear();
      return RHY_OK;
   } catch (const rhygpu::IllegalQuery& e) {
      g_last_error = e.what();
      return RHY_ILLEGAL_QUERY;
   } catch (const rhygpu::CompilationError& e) {
      g_last_error = e.what();
      return RHY_COMPILATION;
   } catch (const rhygpu::CudaError& e) {
      g_last_error = e.what();
      return RHY_CUDA;
   } catch (const std::invalid_argument& e) {
      g_last_error = e.what();
      return RHY_INVALID_ARGUMENT;
   } catch (const std::exception& e) {
      g_last_error = e.what();
      return RHY_INTERNAL;
   } catch (...) {
      g_last_error = "unknown error";
      return RHY_INTERNAL;
   }
}

void need(const void* p, const char* what) {
   if (p == nullptr) throw std::invalid_argument(std::string(what) + " must not be NULL");
}

void make_views(RhyTable& t) {
   const rhygpu::RawTable& r = t.gen.table;
   t.raw_seq.clear();
   t.raw_dict.clear();
   t.raw_date.clear();
   t.dict_values.clear();
   for (const auto& c : r.seq) {
      RhyRawSeqColumn v{};
      v.name = c.name.c_str();
      v.kind = c.kind == rhygpu::SymKind::NUC ? 0 : 1;
      v.reference = c.reference.c_str();
      v.L = static_cast<uint32_t>(c.reference.size());
      v.is_null = c.is_null.data();
      v.row_off = c.row_off.data();
      v.run_pos = c.run_pos.data();
      v.run_len = c.run_len.data();
      v.run_char = c.run_char.data();
      t.raw_seq.push_back(v);
   }
   for (const auto& c : r.dict) {
      std::vector<const char*> vals;
      for (const auto& s : c.values) vals.push_back(s.c_str());
      t.dict_values.push_back(std::move(vals));
   }
   for (size_t i = 0; i < r.dict.size(); ++i) {
      RhyRawDictColumn v{};
      v.name = r.dict[i].name.c_str();
      v.n_values = static_cast<uint32_t>(r.dict[i].values.size());
      v.values = t.dict_values[i].data();
      v.ids = r.dict[i].ids.data();
      t.raw_dict.push_back(v);
   }
   for (const auto& c : r.date) {
      RhyRawDateColumn v{};
      v.name = c.name.c_str();
      v.days = c.days.data();
      t.raw_date.push_back(v);
   }
}

}  // namespace

extern "C" {

const char* rhy_last_error(void) { return g_last_error.c_str(); }

int rhy_generate(const RhyGenConfig* cfg, RhyTable** out) {
   return guarded([&] {
      need(cfg, "cfg");
      need(out, "out");
      *out = nullptr;
      rhygpu::GenConfig g;
      g.seed = cfg->seed;
      g.n_rows = cfg->n_rows;
      if (cfg->genome_len) g.genome_len = cfg->genome_len;
      if (cfg->pool_sites) g.pool_sites = cfg->pool_sites;
      g.n_aa_genes = cfg->n_aa_genes;
      g.null_fraction = cfg->null_fraction;
      g.threads = cfg->threads;
      if (g.n_rows == 0) throw std::invalid_argument("n_rows must be positive");
      auto t = std::make_unique<RhyTable>();
      t->gen = rhygpu::generate_table(g);
      t->image = rhygpu::build_table(t->gen.table, g.threads);
      make_views(*t);
      *out = t.release();
   });
}

int rhy_table_from_raw(const RhyRawTable* raw, uint32_t threads, RhyTable** out) {
   return guarded([&] {
      need(raw, "raw");
      need(out, "out");
      *out = nullptr;
      if (raw->n_rows == 0) throw std::invalid_argument("n_rows must be positive");
      auto t = std::make_unique<RhyTable>();
      rhygpu::RawTable& r = t->gen.table;
      r.n_rows = raw->n_rows;
      for (uint32_t c = 0; c < raw->n_seq; ++c) {
         const RhyRawSeqColumn& s = raw->seq[c];
         need(s.name, "column name");
         need(s.reference, "reference");
         need(s.is_null, "is_null");
         need(s.row_off, "row_off");
         rhygpu::RawSeqColumn col;
         col.name = s.name;
         col.kind = s.kind == 0 ? rhygpu::SymKind::NUC : rhygpu::SymKind::AA;
         col.reference.assign(s.reference, s.L);
         col.is_null.assign(s.is_null, s.is_null + raw->n_rows);
         col.row_off.assign(s.row_off, s.row_off + raw->n_rows + 1);
         const uint64_t n = col.row_off.back();
         if (n > 0) {
            need(s.run_pos, "run_pos");
            need(s.run_len, "run_len");
            need(s.run_char, "run_char");
         }
         for (size_t i = 0; i + 1 < col.row_off.size(); ++i)
            if (col.row_off[i] > col.row_off[i + 1]) throw std::invalid_argument("row_off must be non-decreasing");
         col.run_pos.assign(s.run_pos, s.run_pos + n);
         col.run_len.assign(s.run_len, s.run_len + n);
         col.run_char.assign(s.run_char, s.run_char + n);
         for (uint32_t row = 0; row < raw->n_rows; ++row) {
            uint64_t prev_end = 0;
            for (uint64_t k = col.row_off[row]; k < col.row_off[row + 1]; ++k) {
               if (col.run_len[k] == 0 || col.run_pos[k] < prev_end || uint64_t(col.run_pos[k]) + col.run_len[k] > s.L)
                  throw std::invalid_argument("runs of a row must be sorted, non-overlapping and inside the genome");
               prev_end = uint64_t(col.run_pos[k]) + col.run_len[k];
            }
         }
         r.seq.push_back(std::move(col));
      }
      for (uint32_t c = 0; c < raw->n_dict; ++c) {
         const RhyRawDictColumn& s = raw->dict[c];
         rhygpu::RawDictColumn col;
         col.name = s.name;
         for (uint32_t i = 0; i < s.n_values; ++i) col.values.emplace_back(s.values[i]);
         col.ids.assign(s.ids, s.ids + raw->n_rows);
         r.dict.push_back(std::move(col));
      }
      for (uint32_t c = 0; c < raw->n_date; ++c) {
         const RhyRawDateColumn& s = raw->date[c];
         rhygpu::RawDateColumn col;
         col.name = s.name;
         col.days.assign(s.days, s.days + raw->n_rows);
         r.date.push_back(std::move(col));
      }
      t->image = rhygpu::build_table(r, threads);
      make_views(*t);
      *out = t.release();
   });
}

int rhy_table_info(const RhyTable* t, RhyTableInfo* out) {
   return guarded([&] {
      need(t, "table");
      need(out, "out");
      out->n_rows = t->image.n_rows;
      out->n_chunks = t->image.nchunks();
      out->n_seq = static_cast<uint32_t>(t->image.seq.size());
      out->n_dict = static_cast<uint32_t>(t->image.dict.size());
      out->n_date = static_cast<uint32_t>(t->image.date.size());
   });
}

int rhy_seq_column_info(const RhyTable* t, uint32_t column, RhySeqColumnInfo* out) {
   return guarded([&] {
      need(t, "table");
      need(out, "out");
      const auto& c = t->image.seq.at(column);
      std::memset(out, 0, sizeof(*out));
      out->L = c.L;
      out->n_symbols = rhygpu::alphabet(c.kind).count;
      out->kind = c.kind == rhygpu::SymKind::NUC ? 0 : 1;
      out->flipped_positions = c.flipped_positions;
      out->n_containers = c.vertical.ctrs.size();
      out->payload_bytes = c.vertical.payload_bytes();
      for (const auto& d : c.vertical.ctrs) {
         if (d.type == rhygpu::CT_ARRAY) ++out->n_array;
         else if (d.type == rhygpu::CT_BITSET) ++out->n_bitset;
         else ++out->n_run;
      }
      out->n_missing_intervals = c.nrow_start.size();
      out->n_coverage_exceptions = c.cov_exc.size();
      out->n_null_rows = c.null_rows.size();
   });
}

int rhy_seq_column_name(const RhyTable* t, uint32_t column, char* buf, size_t cap) {
   return guarded([&] {
      need(t, "table");
      need(buf, "buf");
      const std::string& n = t->image.seq.at(column).name;
      if (cap < n.size() + 1) throw std::invalid_argument("buffer too small");
      std::memcpy(buf, n.c_str(), n.size() + 1);
   });
}

int rhy_table_raw(const RhyTable* t, RhyRawTable* out) {
   return guarded([&] {
      need(t, "table");
      need(out, "out");
      out->n_rows = t->gen.table.n_rows;
      out->n_seq = static_cast<uint32_t>(t->raw_seq.size());
      out->n_dict = static_cast<uint32_t>(t->raw_dict.size());
      out->n_date = static_cast<uint32_t>(t->raw_date.size());
      out->seq = t->raw_seq.data();
      out->dict = t->raw_dict.data();
      out->date = t->raw_date.data();
   });
}

int rhy_local_reference(const RhyTable* t, uint32_t column, char* out, size_t cap) {
   return guarded([&] {
      need(t, "table");
      need(out, "out");
      const auto& c = t->image.seq.at(column);
      if (cap < c.L) throw std::invalid_argument("buffer too small");
      const rhygpu::Alphabet& A = rhygpu::alphabet(c.kind);
      for (uint32_t p = 0; p < c.L; ++p) out[p] = A.chars[c.local_ref[p]];
   });
}

int rhy_seq_containers(const RhyTable* t, uint32_t column, uint32_t* pos, uint16_t* chunk, uint8_t* sym, uint32_t* card,
                       uint8_t* type, size_t cap, size_t* n) {
   return guarded([&] {
      need(t, "table");
      need(n, "n");
      const auto& ctrs = t->image.seq.at(column).vertical.ctrs;
      *n = ctrs.size();
      if (cap == 0) return;
      if (cap < ctrs.size()) throw std::invalid_argument("buffer too small");
      need(pos, "pos");
      need(chunk, "chunk");
      need(sym, "sym");
      need(card, "card");
      need(type, "type");
      for (size_t i = 0; i < ctrs.size(); ++i) {
         pos[i] = ctrs[i].key;
         chunk[i] = ctrs[i].v;
         sym[i] = ctrs[i].sym;
         card[i] = ctrs[i].card_m1 + 1u;
         type[i] = ctrs[i].type;
      }
   });
}

int rhy_generate_queries(const RhyTable* t, uint64_t seed, uint32_t n, uint32_t max_depth, uint32_t max_nof_children,
                         int use_aa, int use_metadata, char* buf, size_t cap, size_t* needed) {
   return guarded([&] {
      need(t, "table");
      rhygpu::QueryGenConfig q;
      q.seed = seed;
      q.n_queries = n;
      q.max_depth = max_depth;
      q.max_nof_children = max_nof_children;
      q.use_aa = use_aa != 0;
      q.use_metadata = use_metadata != 0;
      if (t->gen.pool.empty()) throw std::invalid_argument("queries can only be generated for generated tables");
      const auto qs = rhygpu::generate_queries(t->gen, q);
      std::string all;
      for (const auto& s : qs) {
         all += s;
         all += '\n';
      }
      if (needed) *needed = all.size() + 1;
      if (buf) {
         if (cap < all.size() + 1) throw std::invalid_argument("buffer too small");
         std::memcpy(buf, all.c_str(), all.size() + 1);
      }
   });
}

void rhy_table_free(RhyTable* t) { delete t; }

int rhy_plan(const RhyTable* t, const char* expr, char* tree_buf, size_t cap, uint32_t* n_instr, uint32_t* depth) {
   return guarded([&] {
      need(t, "table");
      need(expr, "expr");
      std::string tree;
      const rhygpu::Program p = rhygpu::plan_filter(expr, t->image, nullptr, rhygpu::LowerOptions{}, &tree);
      if (tree_buf) {
         if (cap < tree.size() + 1) throw std::invalid_argument("buffer too small");
         std::memcpy(tree_buf, tree.c_str(), tree.size() + 1);
      }
      if (n_instr) *n_instr = static_cast<uint32_t>(p.code.size());
      if (depth) *depth = p.max_depth;
   });
}

int rhy_open(const RhyTable* t, int device, RhyDevice** out) {
   return guarded([&] {
      need(t, "table");
      need(out, "out");
      *out = nullptr;
      auto d = std::make_unique<RhyDevice>();
      d->table = t;
      d->engine = std::make_unique<rhygpu::Engine>(t->image, device);
      *out = d.release();
   });
}

int rhy_set_tile_bits(RhyDevice* d, uint32_t tile_bits) {
   return guarded([&] {
      need(d, "device");
      if (tile_bits < 4096 || tile_bits > 65536 || (tile_bits & (tile_bits - 1)))
         throw std::invalid_argument("tile_bits must be a power of two in [4096, 65536]");
      d->engine->tile_bits = tile_bits;
   });
}

int rhy_device_bytes(const RhyDevice* d, uint64_t* out) {
   return guarded([&] {
      need(d, "device");
      need(out, "out");
      *out = d->engine->device_bytes();
   });
}

int rhy_count(RhyDevice* d, const char* expr, void* stream, uint64_t* out) {
   return guarded([&] {
      need(d, "device");
      need(expr, "expr");
      need(out, "out");
      const rhygpu::Program p = d->engine->plan(expr);
      *out = d->engine->count(p, static_cast<cudaStream_t>(stream));
   });
}

int rhy_eval(RhyDevice* d, const char* expr, void* stream, uint32_t* out_bits, uint64_t* out_count) {
   return guarded([&] {
      need(d, "device");
      need(expr, "expr");
      const rhygpu::Program p = d->engine->plan(expr);
      d->engine->eval(p, out_bits, out_count, static_cast<cudaStream_t>(stream));
   });
}

int rhy_mutations(RhyDevice* d, const char* expr, uint32_t column, void* stream, uint32_t* counts, uint64_t* filter_count) {
   return guarded([&] {
      need(d, "device");
      need(expr, "expr");
      need(counts, "counts");
      if (column >= d->table->image.seq.size()) throw std::invalid_argument("no such sequence column");
      const rhygpu::Program p = d->engine->plan(expr);
      d->engine->mutations(p, static_cast<int>(column), counts, filter_count, static_cast<cudaStream_t>(stream));
   });
}

int rhy_mutation_rows(const RhyTable* t, uint32_t column, const uint32_t* counts, double min_proportion,
                      RhyMutationRow* rows, size_t cap, size_t* n_rows) {
   // reference: mutations_node.cpp:292-366
   return guarded([&] {
      need(t, "table");
      need(counts, "counts");
      need(n_rows, "n_rows");
      const auto& c = t->image.seq.at(column);
      const rhygpu::Alphabet& A = rhygpu::alphabet(c.kind);
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
            if (rows && n < cap) {
               rows[n].position = pos + 1;
               rows[n].from = A.chars[ref];
               rows[n].to = A.chars[s];
               rows[n].count = count;
               rows[n].coverage = total;
               rows[n].proportion = static_cast<double>(count) / static_cast<double>(total);
            }
            ++n;
         }
      }
      *n_rows = n;
   });
}

void rhy_close(RhyDevice* d) { delete d; }

}  // extern "C"
