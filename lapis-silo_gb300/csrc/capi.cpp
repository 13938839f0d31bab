// extern "C" boundary (include/rhydb_gpu.h). No exception crosses it: every entry point maps
// exceptions to a status code and a thread-local message.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rhydb_gpu.h"
#include "dataset.h"
#include "engine.h"
#include "server.h"
#include "expr.h"
#include "ingest.h"
#include "noalloc.h"
#include "op_program.h"
#include "pass_plan.h"
#include "table.h"

struct RhyTable {
   rhygpu::GeneratedTable gen;  // raw input (generated or copied from the caller)
   rhygpu::TableImage image;
   std::vector<RhyRawSeqColumn> raw_seq;
   std::vector<RhyRawDictColumn> raw_dict;
   std::vector<RhyRawDateColumn> raw_date;
   std::vector<std::vector<const char*>> dict_values;
   // planner features, built on first use
   std::unique_ptr<rhygpu::FeatureContext> fctx;
   std::mutex fctx_mu;
};

struct RhyDevice {
   const RhyTable* table;
   std::unique_ptr<rhygpu::Engine> engine;
   // plain path with device-resident programs
   struct PlainQuery {
      rhygpu::Program prog;
      size_t code_off;
      int action;
      uint32_t column;
   };
   std::vector<PlainQuery> plain;
   rhygpu::Instr* d_plain_code = nullptr;
   ~RhyDevice() {
      if (d_plain_code) cudaFree(d_plain_code);
   }
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

namespace {

// Copies and checks a caller's raw partition (the run order, dictionary ids, sequence kinds).
void import_raw(const RhyRawTable* raw, rhygpu::RawTable& r) {
   need(raw, "raw");
   if (raw->n_rows == 0) throw std::invalid_argument("n_rows must be positive");
   {
      r.n_rows = raw->n_rows;
      for (uint32_t c = 0; c < raw->n_seq; ++c) {
         const RhyRawSeqColumn& s = raw->seq[c];
         need(s.name, "column name");
         need(s.reference, "reference");
         need(s.is_null, "is_null");
         need(s.row_off, "row_off");
         if (s.kind != 0 && s.kind != 1)
            throw std::invalid_argument("column " + std::string(s.name) + ": kind must be 0 (nucleotide) or 1 (amino acid)");
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
         need(s.name, "column name");
         need(s.ids, "ids");
         if (s.n_values) need(s.values, "values");
         rhygpu::RawDictColumn col;
         col.name = s.name;
         for (uint32_t i = 0; i < s.n_values; ++i) {
            need(s.values[i], "dictionary value");
            col.values.emplace_back(s.values[i]);
         }
         col.ids.assign(s.ids, s.ids + raw->n_rows);
         for (uint32_t row = 0; row < raw->n_rows; ++row)
            if (col.ids[row] != UINT32_MAX && col.ids[row] >= s.n_values)
               throw std::invalid_argument("column " + col.name + ": row " + std::to_string(row) + " has value id " +
                                           std::to_string(col.ids[row]) + " of a dictionary of " +
                                           std::to_string(s.n_values) + " values");
         r.dict.push_back(std::move(col));
      }
      for (uint32_t c = 0; c < raw->n_date; ++c) {
         const RhyRawDateColumn& s = raw->date[c];
         rhygpu::RawDateColumn col;
         col.name = s.name;
         col.days.assign(s.days, s.days + raw->n_rows);
         r.date.push_back(std::move(col));
      }
   }
}

}  // namespace

int rhy_table_from_raw(const RhyRawTable* raw, uint32_t threads, RhyTable** out) {
   return guarded([&] {
      need(out, "out");
      *out = nullptr;
      auto t = std::make_unique<RhyTable>();
      import_raw(raw, t->gen.table);
      t->image = rhygpu::build_table(t->gen.table, threads);
      make_views(*t);
      *out = t.release();
   });
}

int rhy_table_from_raw_gpu(const RhyRawTable* raw, int device, uint32_t threads, RhyTable** out) {
   return guarded([&] {
      need(out, "out");
      *out = nullptr;
      auto t = std::make_unique<RhyTable>();
      import_raw(raw, t->gen.table);
      t->image = rhygpu::build_table_gpu(t->gen.table, device, threads);
      make_views(*t);
      *out = t.release();
   });
}

int rhy_seq_column_checksum(const RhyTable* t, uint32_t column, uint64_t* out) {
   return guarded([&] {
      need(t, "table");
      need(out, "out");
      const rhygpu::SeqColumnImage& c = t->image.seq.at(column);
      uint64_t h = 1469598103934665603ull;  // FNV-1a over every array of the column's image
      auto bytes = [&](const void* p, size_t n) {
         const auto* b = static_cast<const unsigned char*>(p);
         for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
      };
      auto vec = [&](const auto& v) {
         const uint64_t n = v.size();
         bytes(&n, sizeof n);
         if (n) bytes(v.data(), v.size() * sizeof(v[0]));
      };
      vec(c.local_ref);
      vec(c.vertical.ctrs);
      vec(c.vertical.payload);
      vec(c.vertical.off);
      vec(c.vertical.stats);
      vec(c.null_rows);
      vec(c.cov_exc);
      vec(c.cov_exc_off);
      vec(c.nrow_off);
      vec(c.nrow_start);
      vec(c.nrow_end);
      vec(c.nblk);
      vec(c.nblk_off);
      vec(c.exc_toff);
      vec(c.nblk_toff);
      vec(c.mstart);
      vec(c.mend);
      vec(c.mstart_off);
      vec(c.mend_off);
      vec(c.cstart);
      vec(c.cend);
      vec(c.hrow_off);
      vec(c.hent);
      bytes(&c.flipped_positions, sizeof c.flipped_positions);
      *out = h;
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

int rhy_table_set_primary_key(RhyTable* t, const char* dict_column) {
   return guarded([&] {
      need(t, "table");
      if (dict_column == nullptr) {
         t->image.primary_key = -1;
         return;
      }
      const int c = t->image.find_dict(dict_column);
      if (c < 0) throw rhygpu::IllegalQuery(std::string("no dictionary column '") + dict_column + "'");
      t->image.primary_key = c;
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
      out->n_row_index_entries = c.hent.size();
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

int rhy_container_pass_plan(const RhyTable* t, uint32_t column, uint32_t ctas, uint32_t* array_units, size_t array_cap,
                            size_t* n_array, uint32_t* other_units, size_t other_cap, size_t* n_other, uint32_t* ranges,
                            size_t range_cap, size_t* n_ranges) {
   return guarded([&] {
      need(t, "table");
      need(n_array, "n_array");
      need(n_other, "n_other");
      need(n_ranges, "n_ranges");
      const rhygpu::SeqColumnImage& col = t->image.seq.at(column);
      const uint32_t nchunks = t->image.nchunks();
      const rhygpu::PassUnits P = rhygpu::pass_units(col, nchunks);
      const std::vector<rhygpu::StreamRange> R = rhygpu::pass_ranges(col, P, nchunks, ctas);
      *n_array = P.au.size();
      *n_other = P.ou.size();
      *n_ranges = R.size();
      if (array_cap == 0 && other_cap == 0 && range_cap == 0) return;
      if (array_cap < P.au.size() || other_cap < P.ou.size() || range_cap < R.size())
         throw std::invalid_argument("buffer too small");
      need(array_units, "array_units");
      need(other_units, "other_units");
      need(ranges, "ranges");
      for (size_t i = 0; i < P.au.size(); ++i) {
         const rhygpu::ArrUnit& u = P.au[i];
         uint32_t* o = array_units + 5 * i;
         o[0] = u.e0;
         o[1] = u.n;
         o[2] = u.c0;
         o[3] = u.nd;
         o[4] = u.v;
      }
      for (size_t i = 0; i < P.ou.size(); ++i) {
         const rhygpu::OtherUnit& u = P.ou[i];
         uint32_t* o = other_units + 4 * i;
         o[0] = u.kind;
         o[1] = u.v;
         o[2] = u.e0;
         o[3] = u.c;
      }
      for (size_t i = 0; i < R.size(); ++i) {
         const rhygpu::StreamRange& r = R[i];
         uint32_t* o = ranges + 6 * i;
         o[0] = r.a0;
         o[1] = r.a1;
         o[2] = r.o0;
         o[3] = r.o1;
         o[4] = r.v0;
         o[5] = r.v1;
      }
   });
}

int rhy_generate_queries(const RhyTable* t, uint64_t seed, uint32_t n, uint32_t max_depth, uint32_t max_nof_children,
                         uint32_t max_leaves, int use_aa, int use_metadata, char* buf, size_t cap, size_t* needed) {
   return guarded([&] {
      need(t, "table");
      rhygpu::QueryGenConfig q;
      q.seed = seed;
      q.n_queries = n;
      q.max_depth = max_depth;
      q.max_nof_children = max_nof_children;
      q.max_leaves = max_leaves;
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
      d->engine->batch_tile_bits = tile_bits;
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

namespace {

// A caller's operator tree lowered to a device program, with its row sets (op_program.h).
struct ProgramCall {
   rhygpu::Program prog;
   std::vector<const uint32_t*> sets;
};

ProgramCall plan_program(const RhyTable& table, const RhyOpProgram* prog, std::string* tree = nullptr) {
   need(prog, "program");
   if (prog->n_nodes) need(prog->nodes, "program nodes");
   if (prog->n_row_sets) need(prog->row_sets, "program row sets");
   const rhygpu::TableImage& t = table.image;
   ProgramCall call;
   std::vector<double> cards(prog->n_row_sets);
   for (uint32_t k = 0; k < prog->n_row_sets; ++k) {
      const uint32_t* rs = prog->row_sets[k];
      need(rs, "row set");
      uint64_t c = 0;
      for (uint32_t v = 0; v < t.nchunks(); ++v) {
         const uint32_t* w = rs + static_cast<size_t>(v) * rhygpu::CHUNK_WORDS;
         const uint32_t rows = t.chunk_sizes[v];
         for (uint32_t i = rows / 32; i < rhygpu::CHUNK_WORDS; ++i) {
            const uint32_t keep = i == rows / 32 ? (rows % 32 ? (1u << (rows % 32)) - 1u : 0u) : 0u;
            if (w[i] & ~keep)
               throw std::invalid_argument("row set " + std::to_string(k) + " holds rows beyond chunk " + std::to_string(v) +
                                           "'s " + std::to_string(rows) + " rows");
         }
         for (uint32_t i = 0; i < rhygpu::CHUNK_WORDS; ++i) c += static_cast<uint64_t>(__builtin_popcount(w[i]));
      }
      cards[k] = static_cast<double>(c);
      call.sets.push_back(rs);
   }
   const rhygpu::OpPtr op = rhygpu::op_from_nodes(prog->nodes, prog->n_nodes, t, cards);
   if (tree) *tree = op->to_string();
   rhygpu::LowerOptions o;
   o.rows = t.n_rows;
   call.prog = rhygpu::lower(*op, rhygpu::rule_estimator(t), o);
   return call;
}

}  // namespace

int rhy_program_from_expr(const RhyTable* t, const char* expr, RhyOpNode* nodes, size_t cap, size_t* n) {
   return guarded([&] {
      need(t, "table");
      need(expr, "expr");
      need(n, "n");
      const rhygpu::OpPtr op = rhygpu::compile_filter(expr, t->image);
      std::vector<RhyOpNode> out;
      rhygpu::op_to_nodes(*op, out);
      *n = out.size();
      if (nodes) std::memcpy(nodes, out.data(), std::min(cap, out.size()) * sizeof(RhyOpNode));
   });
}

int rhy_program_plan(const RhyTable* t, const RhyOpProgram* prog, char* tree_buf, size_t cap, uint32_t* n_instr,
                     uint32_t* depth) {
   return guarded([&] {
      need(t, "table");
      std::string tree;
      const ProgramCall c = plan_program(*t, prog, &tree);
      if (tree_buf) {
         if (cap < tree.size() + 1) throw std::invalid_argument("buffer too small");
         std::memcpy(tree_buf, tree.c_str(), tree.size() + 1);
      }
      if (n_instr) *n_instr = static_cast<uint32_t>(c.prog.code.size());
      if (depth) *depth = c.prog.max_depth;
   });
}

int rhy_program_eval(RhyDevice* d, const RhyOpProgram* prog, void* stream, uint32_t* out_bits, uint64_t* out_count) {
   return guarded([&] {
      need(d, "device");
      const ProgramCall c = plan_program(*d->table, prog);
      d->engine->eval(c.prog, out_bits, out_count, static_cast<cudaStream_t>(stream), c.sets.data());
   });
}

int rhy_program_count(RhyDevice* d, const RhyOpProgram* prog, void* stream, uint64_t* out) {
   return guarded([&] {
      need(d, "device");
      need(out, "out");
      const ProgramCall c = plan_program(*d->table, prog);
      *out = d->engine->count(c.prog, static_cast<cudaStream_t>(stream), c.sets.data());
   });
}

int rhy_program_mutations(RhyDevice* d, const RhyOpProgram* prog, uint32_t column, void* stream, uint32_t* counts,
                          uint64_t* filter_count) {
   return guarded([&] {
      need(d, "device");
      need(counts, "counts");
      if (column >= d->table->image.seq.size()) throw std::invalid_argument("no such sequence column");
      const ProgramCall c = plan_program(*d->table, prog);
      d->engine->mutations(c.prog, static_cast<int>(column), counts, filter_count, static_cast<cudaStream_t>(stream),
                           c.sets.data());
   });
}

int rhy_aggregate(RhyDevice* d, const char* expr, const RhyAggDimension* dims, uint32_t n_dims, void* stream,
                  int32_t* groups, uint64_t* counts, size_t cap, size_t* n_out, uint64_t* filter_count) {
   return guarded([&] {
      need(d, "device");
      need(expr, "expr");
      need(n_out, "n_out");
      if (n_dims) need(dims, "dims");
      std::vector<rhygpu::Engine::AggSpec> spec(n_dims);
      for (uint32_t i = 0; i < n_dims; ++i) {
         if (dims[i].kind == 0 && dims[i].position == 0) throw rhygpu::IllegalQuery("positions are 1-based");
         spec[i] = {static_cast<uint32_t>(dims[i].kind), dims[i].column, dims[i].kind == 0 ? dims[i].position - 1 : 0u};
      }
      const rhygpu::Program p = d->engine->plan(expr);
      std::vector<int32_t> g;
      std::vector<uint64_t> c;
      d->engine->aggregate(p, spec, g, c, filter_count, static_cast<cudaStream_t>(stream));
      *n_out = c.size();
      const size_t m = std::min(cap, c.size());
      if (groups && m) std::copy(g.begin(), g.begin() + m * n_dims, groups);
      if (counts && m) std::copy(c.begin(), c.begin() + m, counts);
   });
}

namespace {

std::vector<rhygpu::BatchQuery> make_batch(RhyDevice* d, const char* const* exprs, const int* actions,
                                           const uint32_t* columns, uint32_t n, uint32_t plan_threads) {
   need(exprs, "exprs");
   std::vector<std::string> texts(n);
   for (uint32_t i = 0; i < n; ++i) {
      need(exprs[i], "expression");
      texts[i] = exprs[i];
   }
   std::vector<rhygpu::BatchQuery> qs = d->engine->plan_batch(texts, plan_threads);
   for (uint32_t i = 0; i < n; ++i) {
      qs[i].action = actions ? actions[i] : 0;
      qs[i].column = columns ? static_cast<int>(columns[i]) : 0;
      if (qs[i].action < 0 || qs[i].action > 2)
         throw std::invalid_argument("action must be 0 (count), 1 (mutations) or 2 (details)");
   }
   return qs;
}

void copy_batch_results(RhyDevice* d, uint32_t n, uint64_t* counts, uint32_t* const* mut_counts) {
   rhygpu::Engine& e = *d->engine;
   const auto& b = e.batch();
   if (n != b.n_queries) throw std::invalid_argument("result arrays do not match the prepared batch");
   e.check_batch_error(e.batch_state());
   for (uint32_t i = 0; i < n; ++i) {
      if (counts) counts[i] = e.batch_count(i);
      if (mut_counts && mut_counts[i]) {
         const uint32_t* src = e.batch_mutation_counts(i);
         if (!src) continue;
         uint32_t col = 0;
         for (const auto& g : b.groups) {
            const uint32_t slot = b.slot_of_query[i];
            if (slot >= g.slot_begin && slot < g.slot_begin + g.n) col = static_cast<uint32_t>(g.column);
         }
         const auto& dc = e.host_view().seq[col];
         std::memcpy(mut_counts[i], src, static_cast<size_t>(dc.nsym) * dc.L * 4);
      }
   }
}

}  // namespace

int rhy_batch(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns, uint32_t n,
              uint32_t tile_bits, void* stream, uint64_t* counts, uint32_t* const* mut_counts) {
   return guarded([&] {
      need(d, "device");
      if (n == 0) return;
      std::lock_guard<std::mutex> lock(d->engine->mu);
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      d->engine->batch_prepare(make_batch(d, exprs, actions, columns, n, 0), tile_bits);
      cudaStream_t s = d->engine->stream_for(static_cast<cudaStream_t>(stream));
      d->engine->batch_enqueue(s, true, true);
      rhygpu::cuda_check(cudaStreamSynchronize(s), "batch");
      copy_batch_results(d, n, counts, mut_counts);
   });
}

int rhy_batch_rows(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns,
                   const double* min_proportions, uint32_t n, uint32_t tile_bits, void* stream, uint64_t* counts,
                   RhyMutationRow* rows, size_t rows_cap, uint64_t* row_begin, uint32_t* row_count, size_t* n_rows) {
   static_assert(sizeof(RhyMutationRow) == sizeof(rhygpu::DevMutationRow), "row layout");
   static_assert(offsetof(RhyMutationRow, proportion) == offsetof(rhygpu::DevMutationRow, proportion), "row layout");
   return guarded([&] {
      need(d, "device");
      need(n_rows, "n_rows");
      *n_rows = 0;
      if (n == 0) return;
      need(exprs, "exprs");
      std::vector<std::string> texts(n);
      for (uint32_t i = 0; i < n; ++i) {
         need(exprs[i], "expression");
         texts[i] = exprs[i];
      }
      std::lock_guard<std::mutex> lock(d->engine->mu);
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      cudaStream_t s = d->engine->stream_for(static_cast<cudaStream_t>(stream));
      *n_rows = d->engine->batch_rows_pipelined(texts, actions, columns, min_proportions, tile_bits, s,
                                                reinterpret_cast<rhygpu::DevMutationRow*>(rows), rows ? rows_cap : 0,
                                                counts, row_begin, row_count);
   });
}

int rhy_batch_times(RhyDevice* d, RhyBatchTimes* out) {
   return guarded([&] {
      need(d, "device");
      need(out, "out");
      std::lock_guard<std::mutex> lock(d->engine->mu);
      const auto& t = d->engine->batch_times;
      *out = RhyBatchTimes{t.plan_ms, t.prepare_ms, t.device_ms, t.output_ms, t.compile_ms, t.predict_ms, t.lower_ms};
   });
}

int rhy_batch_rows_fetch(RhyDevice* d, void* stream, RhyMutationRow* rows, size_t rows_cap) {
   return guarded([&] {
      need(d, "device");
      need(rows, "rows");
      std::lock_guard<std::mutex> lock(d->engine->mu);
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      d->engine->batch_rows_fetch(static_cast<cudaStream_t>(stream), reinterpret_cast<rhygpu::DevMutationRow*>(rows),
                                  rows_cap);
   });
}

int rhy_batch_prepare(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns, uint32_t n,
                      uint32_t tile_bits, uint32_t plan_threads) {
   return guarded([&] {
      need(d, "device");
      std::lock_guard<std::mutex> lock(d->engine->mu);
      d->engine->batch_prepare(make_batch(d, exprs, actions, columns, n, plan_threads), tile_bits);
   });
}

int rhy_batch_launch(RhyDevice* d, void* stream, int copy_in, int copy_out) {
   return guarded([&] {
      need(d, "device");
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      d->engine->batch_enqueue(static_cast<cudaStream_t>(stream), copy_in != 0, copy_out != 0);
   });
}

int rhy_batch_capture(RhyDevice* d, void* stream) {
   return guarded([&] {
      need(d, "device");
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      d->engine->batch_capture(static_cast<cudaStream_t>(stream));
   });
}

int rhy_batch_replay(RhyDevice* d, void* stream) {
   return guarded([&] {
      need(d, "device");
      d->engine->batch_replay(static_cast<cudaStream_t>(stream));
   });
}

int rhy_batch_results(RhyDevice* d, uint64_t* counts, uint32_t* const* mut_counts) {
   return guarded([&] {
      need(d, "device");
      copy_batch_results(d, d->engine->batch().n_queries, counts, mut_counts);
   });
}

int rhy_batch_schedule(RhyDevice* d, const RhyBatchSchedule* set, RhyBatchSchedule* get) {
   return guarded([&] {
      need(d, "device");
      std::lock_guard<std::mutex> lock(d->engine->mu);
      rhygpu::BatchSchedule& b = d->engine->batch_schedule;
      if (set) {
         if (set->max_tile_bits < 4096 || set->max_tile_bits > 65536 || (set->max_tile_bits & (set->max_tile_bits - 1)))
            throw std::invalid_argument("max_tile_bits must be a power of two in [4096, 65536]");
         if (set->stack_kb < 8 || set->stack_kb > 200) throw std::invalid_argument("stack_kb must lie in [8, 200]");
         if (set->query_major > 1) throw std::invalid_argument("query_major must be 0 or 1");
         b = rhygpu::BatchSchedule{set->max_tile_bits, set->stack_kb, set->ctas_per_sm, set->query_major};
      }
      if (get) *get = RhyBatchSchedule{b.max_tile_bits, b.stack_kb, b.ctas_per_sm, b.query_major};
   });
}

int rhy_batch_autotune(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns, uint32_t n,
                       uint32_t reps, void* stream, RhyBatchSchedule* tried, double* tried_ms, size_t cap,
                       size_t* n_tried) {
   return guarded([&] {
      need(d, "device");
      if (n == 0) throw std::invalid_argument("autotune needs a batch");
      std::lock_guard<std::mutex> lock(d->engine->mu);
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      const std::vector<rhygpu::BatchQuery> qs = make_batch(d, exprs, actions, columns, n, 0);
      const auto res = d->engine->autotune_batch(qs, static_cast<cudaStream_t>(stream), reps);
      if (n_tried) *n_tried = res.size();
      for (size_t i = 0; i < res.size() && i < cap; ++i) {
         const auto& b = res[i].first;
         if (tried) tried[i] = RhyBatchSchedule{b.max_tile_bits, b.stack_kb, b.ctas_per_sm, b.query_major};
         if (tried_ms) tried_ms[i] = res[i].second;
      }
   });
}

int rhy_batch_info(RhyDevice* d, RhyBatchInfo* out) {
   return guarded([&] {
      need(d, "device");
      need(out, "out");
      const auto& b = d->engine->batch();
      out->n_queries = b.n_queries;
      out->n_mutation_slots = b.n_slots;
      out->n_items = b.n_items;
      out->n_instr = b.n_code;
      out->max_depth = b.max_depth;
      out->tile_bits = b.tile_bits;
      out->grid = b.grid;
      out->device_bytes = d->engine->device_bytes();
      out->n_filter_launches = b.n_items ? 1u : 0u;
      out->filter_bytes = d->engine->batch_filter_bytes(b);
   });
}

int rhy_plain_prepare(RhyDevice* d, const char* const* exprs, const int* actions, const uint32_t* columns, uint32_t n) {
   return guarded([&] {
      need(d, "device");
      auto qs = make_batch(d, exprs, actions, columns, n, 0);
      d->plain.clear();
      size_t off = 0;
      std::vector<rhygpu::Instr> code;
      for (auto& q : qs) {
         d->plain.push_back({std::move(q.prog), off, q.action, static_cast<uint32_t>(q.column)});
         const auto& p = d->plain.back().prog;
         code.insert(code.end(), p.code.begin(), p.code.end());
         off += p.code.size();
      }
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      if (d->d_plain_code) cudaFree(d->d_plain_code);
      d->d_plain_code = nullptr;
      rhygpu::cuda_check(cudaMalloc(&d->d_plain_code, std::max<size_t>(code.size(), 1) * sizeof(rhygpu::Instr)), "cudaMalloc");
      rhygpu::cuda_check(cudaMemcpy(d->d_plain_code, code.data(), code.size() * sizeof(rhygpu::Instr), cudaMemcpyHostToDevice),
                         "upload programs");
   });
}

int rhy_plain_launch_parts(RhyDevice* d, uint32_t i, void* stream, uint32_t parts) {
   return guarded([&] {
      need(d, "device");
      if (i >= d->plain.size()) throw std::invalid_argument("no such prepared query");
      rhygpu::Engine& e = *d->engine;
      const auto& q = d->plain[i];
      cudaStream_t s = e.stream_for(static_cast<cudaStream_t>(stream));
      if (parts & 1) rhygpu::cuda_check(cudaMemsetAsync(e.d_count, 0, sizeof(unsigned long long), s), "memset");
      if (q.action == 1) {
         const auto& dc = e.host_view().seq[q.column];
         if (parts & 1) {
            rhygpu::cuda_check(cudaMemsetAsync(e.d_counts, 0, static_cast<size_t>(dc.nsym) * dc.L * 4, s), "memset");
            rhygpu::cuda_check(cudaMemsetAsync(e.d_scratch, 0, rhygpu::mut_scratch_words(dc.L) * 4, s), "memset");
            e.launch_count(d->d_plain_code + q.code_off, q.prog, e.d_count, e.d_filter, s);
         }
         if (parts >> 1)
            e.launch_mutations(static_cast<int>(q.column), e.d_filter, e.d_count, e.d_counts, e.d_scratch, s,
                               (parts >> 1) & (rhygpu::MUT_PART_ALL | rhygpu::MUT_PART_SPARSE));
      } else if (parts & 1) {
         e.launch_count(d->d_plain_code + q.code_off, q.prog, e.d_count, nullptr, s);
      }
   });
}

int rhy_plain_launch(RhyDevice* d, uint32_t i, void* stream) { return rhy_plain_launch_parts(d, i, stream, 31); }

int rhy_sparse_rows(RhyDevice* d, const uint64_t* set, uint64_t* get) {
   return guarded([&] {
      need(d, "device");
      std::lock_guard<std::mutex> lock(d->engine->mu);
      if (set) {
         d->engine->sparse_rows_plain = set[0];
         d->engine->sparse_rows_batch = set[1];
      }
      if (get) {
         get[0] = d->engine->sparse_rows_plain;
         get[1] = d->engine->sparse_rows_batch;
      }
   });
}

int rhy_mutation_bytes(const RhyDevice* d, uint32_t column, uint64_t* payload_bytes, uint64_t* descriptor_bytes) {
   return guarded([&] {
      need(d, "device");
      const auto& c = d->table->image.seq.at(column);
      if (payload_bytes) *payload_bytes = c.vertical.payload_bytes();
      if (descriptor_bytes) *descriptor_bytes = c.vertical.ctrs.size() * sizeof(rhygpu::CtrDesc);
   });
}

int rhy_batch_capture_ex(RhyDevice* d, void* stream, int copy_in, int copy_out) {
   return guarded([&] {
      need(d, "device");
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      d->engine->batch_capture(static_cast<cudaStream_t>(stream), copy_in != 0, copy_out != 0);
   });
}

int rhy_batch_launch_parts(RhyDevice* d, void* stream, uint32_t parts) {
   return guarded([&] {
      need(d, "device");
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      d->engine->batch_enqueue(static_cast<cudaStream_t>(stream), false, false, parts);
   });
}

int rhy_mutations_noalloc(RhyDevice* d, uint32_t column, const uint32_t* d_filter, const uint64_t* d_filter_count,
                          uint32_t* d_counts, int* d_status, void* stream) {
   return guarded([&] {
      need(d, "device");
      rhygpu::mutations_noalloc(*d->engine, column, d_filter,
                                reinterpret_cast<const unsigned long long*>(d_filter_count), d_counts, d_status,
                                static_cast<cudaStream_t>(stream));
   });
}

int rhy_test_withhold_copies(RhyDevice* d, int on) {
   return guarded([&] {
      need(d, "device");
      std::lock_guard<std::mutex> lock(d->engine->mu);
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      rhygpu::cuda_check(cudaDeviceSynchronize(), "synchronise before switching copy withholding");
      rhygpu::set_copy_withholding((on & 1) != 0);
      rhygpu::set_ring_withholding((on & 2) != 0);
   });
}

int rhy_mutation_rows(const RhyTable* t, uint32_t column, const uint32_t* counts, double min_proportion,
                      RhyMutationRow* rows, size_t cap, size_t* n_rows) {
   // reference: mutations_node.cpp:292-366
   static_assert(sizeof(RhyMutationRow) == sizeof(rhygpu::DevMutationRow), "row layout");
   return guarded([&] {
      need(t, "table");
      need(counts, "counts");
      need(n_rows, "n_rows");
      *n_rows = rhygpu::mutation_rows_host(t->image.seq.at(column), counts, min_proportion,
                                           reinterpret_cast<rhygpu::DevMutationRow*>(rows), rows ? cap : 0);
   });
}

// ---- learned planner ----

static_assert(RHY_PLANNER_FEATURES == rhygpu::PLAN_FEATURES, "feature count");
static_assert(RHY_MLP_NPARAM == rhygpu::MLP_NPARAM, "parameter count");

int rhy_plan_features(const RhyTable* t, const char* expr, float* x, size_t cap, size_t* n) {
   return guarded([&] {
      need(t, "table");
      need(expr, "expression");
      need(n, "n");
      RhyTable* tt = const_cast<RhyTable*>(t);
      {
         std::lock_guard<std::mutex> lock(tt->fctx_mu);
         if (!tt->fctx) tt->fctx = std::make_unique<rhygpu::FeatureContext>(rhygpu::feature_context(t->image));
      }
      const rhygpu::FeatureContext& ctx = *tt->fctx;
      rhygpu::OpPtr op = rhygpu::compile_filter(expr, t->image);
      std::vector<const rhygpu::Op*> nodes;
      std::function<void(const rhygpu::Op&)> walk = [&](const rhygpu::Op& o) {
         nodes.push_back(&o);
         for (const auto& c : o.children) walk(*c);
         for (const auto& c : o.negated) walk(*c);
      };
      walk(*op);
      *n = nodes.size();
      for (size_t i = 0; i < nodes.size() && i < cap && x; ++i) rhygpu::op_features(*nodes[i], ctx, x + i * RHY_PLANNER_FEATURES);
   });
}

int rhy_planner_collect(RhyDevice* d, const char* const* exprs, uint32_t n, size_t* n_added) {
   return guarded([&] {
      need(d, "device");
      if (n) need(exprs, "exprs");
      std::vector<std::string> texts;
      for (uint32_t i = 0; i < n; ++i) {
         need(exprs[i], "expression");
         texts.emplace_back(exprs[i]);
      }
      const size_t k = d->engine->planner_collect(texts);
      if (n_added) *n_added = k;
   });
}

namespace {
void copy_stats(const rhygpu::PlannerStats& st, RhyPlannerStats* out) {
   if (!out) return;
   out->n_train = st.n_train;
   out->n_val = st.n_val;
   out->epochs = st.epochs;
   out->train_loss = st.train_loss;
   out->val_loss = st.val_loss;
   out->qerr_learned_median = st.qerr_learned_median;
   out->qerr_rule_median = st.qerr_rule_median;
   out->qerr_learned_p90 = st.qerr_learned_p90;
   out->qerr_rule_p90 = st.qerr_rule_p90;
   out->cost_err_median = st.cost_err_median;
   out->train_ms = st.train_ms;
   out->accepted = st.accepted;
}
}  // namespace

int rhy_planner_train(RhyDevice* d, uint32_t epochs, uint32_t batch, float lr, uint64_t seed, RhyPlannerStats* out) {
   return guarded([&] {
      need(d, "device");
      copy_stats(d->engine->planner_train(epochs, batch, lr, seed), out);
   });
}

int rhy_planner_evaluate(RhyDevice* d, const char* const* exprs, uint32_t n, RhyPlannerStats* out) {
   return guarded([&] {
      need(d, "device");
      if (n) need(exprs, "exprs");
      std::vector<std::string> texts;
      for (uint32_t i = 0; i < n; ++i) {
         need(exprs[i], "expression");
         texts.emplace_back(exprs[i]);
      }
      copy_stats(d->engine->planner_evaluate(texts), out);
   });
}

int rhy_planner_export(RhyDevice* d, RhyPlannerModel* out) {
   return guarded([&] {
      need(d, "device");
      need(out, "out");
      std::lock_guard<std::mutex> lock(d->engine->mu);
      rhygpu::Planner& p = d->engine->planner();
      if (!p.trained) throw std::invalid_argument("the planner network is not trained");
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      p.net.get_master(out->weights);
      std::copy(p.fmean.begin(), p.fmean.end(), out->feature_mean);
      std::copy(p.fstd.begin(), p.fstd.end(), out->feature_std);
      for (int k = 0; k < 2; ++k) {
         out->target_mean[k] = p.tmean[k];
         out->target_std[k] = p.tstd[k];
      }
      out->accepted = p.accepted ? 1 : 0;
   });
}

int rhy_planner_import(RhyDevice* d, const RhyPlannerModel* in) {
   return guarded([&] {
      need(d, "device");
      need(in, "model");
      for (int k = 0; k < RHY_PLANNER_FEATURES; ++k)
         if (!(std::isfinite(in->feature_mean[k]) && in->feature_std[k] > 0))
            throw std::invalid_argument("model: feature normalisation must be finite with positive deviations");
      for (int k = 0; k < 2; ++k)
         if (!(std::isfinite(in->target_mean[k]) && in->target_std[k] > 0))
            throw std::invalid_argument("model: target normalisation must be finite with positive deviations");
      std::lock_guard<std::mutex> lock(d->engine->mu);
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      rhygpu::Planner& p = d->engine->planner();
      p.net.set_master(in->weights);
      std::copy(in->feature_mean, in->feature_mean + RHY_PLANNER_FEATURES, p.fmean.begin());
      std::copy(in->feature_std, in->feature_std + RHY_PLANNER_FEATURES, p.fstd.begin());
      for (int k = 0; k < 2; ++k) {
         p.tmean[k] = in->target_mean[k];
         p.tstd[k] = in->target_std[k];
      }
      p.trained = true;
      p.accepted = in->accepted != 0;
      if (!p.accepted) d->engine->set_planner_mode(0);
   });
}

int rhy_planner_mode(RhyDevice* d, int mode) {
   return guarded([&] {
      need(d, "device");
      d->engine->set_planner_mode(mode);
   });
}

int rhy_planner_samples(RhyDevice* d, float* x, float* y, size_t cap, size_t* n) {
   return guarded([&] {
      need(d, "device");
      need(n, "n");
      const auto& sm = d->engine->planner().samples;
      *n = sm.size();
      for (size_t i = 0; i < sm.size() && i < cap; ++i) {
         if (x) std::copy(sm[i].x.begin(), sm[i].x.end(), x + i * RHY_PLANNER_FEATURES);
         if (y) {
            y[3 * i] = sm[i].log_sel;
            y[3 * i + 1] = sm[i].log_cost;
            y[3 * i + 2] = sm[i].rule_log_sel;
         }
      }
   });
}

int rhy_planner_predict(RhyDevice* d, const float* x, uint32_t n, double* sel, double* cost) {
   return guarded([&] {
      need(d, "device");
      if (n) need(x, "x");
      std::vector<std::array<float, rhygpu::PLAN_FEATURES>> rows(n);
      for (uint32_t i = 0; i < n; ++i) std::copy(x + static_cast<size_t>(i) * RHY_PLANNER_FEATURES,
                                                 x + static_cast<size_t>(i + 1) * RHY_PLANNER_FEATURES, rows[i].begin());
      std::vector<double> s, c;
      {
         std::lock_guard<std::mutex> lock(d->engine->mu);
         rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
         if (!d->engine->planner().trained) throw std::invalid_argument("the planner network is not trained");
         d->engine->planner().predict(rows, s, c);
      }
      for (uint32_t i = 0; i < n; ++i) {
         if (sel) sel[i] = s[i];
         if (cost) cost[i] = c[i];
      }
   });
}

int rhy_planner_weights(RhyDevice* d, float* w) {
   return guarded([&] {
      need(d, "device");
      need(w, "w");
      d->engine->planner().net.get_master(w);
   });
}

int rhy_mlp_gradient(RhyDevice* d, const float* w, const float* x, const float* t, uint32_t n, float* grad, float* loss,
                     float* y) {
   return guarded([&] {
      need(d, "device");
      need(w, "w");
      if (n) {
         need(x, "x");
         need(t, "t");
      }
      rhygpu::cuda_check(cudaSetDevice(d->engine->device()), "cudaSetDevice");
      rhygpu::PlannerNet net(d->engine->device());
      net.set_master(w);
      net.gradient(x, t, n, grad, loss, y);
   });
}

// ---- serving ----

struct RhyServer {
   std::unique_ptr<rhygpu::Server> server;
};

int rhy_server_start(RhyDevice* d, const RhyServerConfig* cfg, RhyServer** out) {
   return guarded([&] {
      need(d, "device");
      need(out, "out");
      *out = nullptr;
      rhygpu::ServerConfig c;
      if (cfg) {
         if (cfg->max_batch) c.max_batch = cfg->max_batch;
         if (cfg->streams) c.streams = cfg->streams;
         if (cfg->max_inflight) c.max_inflight = cfg->max_inflight;
         c.memory_budget = cfg->memory_budget;
         if (cfg->max_wait_ms >= 0) c.max_wait_ms = cfg->max_wait_ms;
         c.plain = cfg->plain != 0;
      }
      auto s = std::make_unique<RhyServer>();
      s->server = std::make_unique<rhygpu::Server>(*d->engine, c);
      *out = s.release();
   });
}

int rhy_server_submit(RhyServer* s, const char* expr, int action, uint32_t column, double min_proportion, uint32_t k,
                      uint64_t* id) {
   return guarded([&] {
      need(s, "server");
      need(expr, "expression");
      need(id, "id");
      *id = s->server->submit(expr, action, static_cast<int>(column), min_proportion, k);
   });
}

int rhy_server_result(RhyServer* s, uint64_t id, double timeout_ms, uint64_t* count, RhyMutationRow* rows,
                      size_t rows_cap, size_t* n_rows, uint32_t* ids, size_t ids_cap, size_t* n_ids, double* latency_ms) {
   int code = RHY_OK;
   const int rc = guarded([&] {
      need(s, "server");
      std::shared_ptr<rhygpu::ServeRequest> r = s->server->wait(id, timeout_ms);
      if (!r) {
         code = RHY_TIMEOUT;
         throw std::runtime_error("request " + std::to_string(id) + " not done within the timeout");
      }
      if (!r->error.empty()) {
         s->server->release(id);
         code = r->cancelled                                          ? RHY_CANCELLED
                : r->error.find("device program error") != std::string::npos ? RHY_COMPILATION
                                                                              : RHY_CUDA;
         throw std::runtime_error(r->error);
      }
      if (n_rows) *n_rows = r->rows.size();
      if (n_ids) *n_ids = r->ids.size();
      if (count) *count = r->count;
      if (latency_ms) *latency_ms = 1000.0 * (r->t_done - r->t_submit);
      if ((!r->rows.empty() && (!rows || rows_cap < r->rows.size())) || (!r->ids.empty() && (!ids || ids_cap < r->ids.size())))
         throw std::invalid_argument("result buffers too small: " + std::to_string(r->rows.size()) + " rows, " +
                                     std::to_string(r->ids.size()) + " ids");
      if (!r->rows.empty()) std::memcpy(rows, r->rows.data(), r->rows.size() * sizeof(RhyMutationRow));
      if (!r->ids.empty()) std::memcpy(ids, r->ids.data(), r->ids.size() * sizeof(uint32_t));
      s->server->release(id);
   });
   return rc == RHY_INTERNAL && code != RHY_OK ? code : rc;
}

int rhy_server_stats(RhyServer* s, RhyServerStats* out) {
   return guarded([&] {
      need(s, "server");
      need(out, "out");
      const rhygpu::ServerStats st = s->server->stats();
      out->submitted = st.submitted;
      out->completed = st.completed;
      out->rejected = st.rejected;
      out->batches = st.batches;
      out->p50_ms = st.p50_ms;
      out->p99_ms = st.p99_ms;
      out->mean_batch = st.mean_batch;
      out->qps = st.qps;
      out->peak_bytes = st.peak_bytes;
      out->budget_bytes = st.budget_bytes;
      out->peak_inflight = st.peak_inflight;
      out->cancelled = st.cancelled;
   });
}

int rhy_server_cancel(RhyServer* s, uint64_t id, int* was_pending) {
   return guarded([&] {
      need(s, "server");
      const bool c = s->server->cancel(id);
      if (was_pending) *was_pending = c ? 1 : 0;
   });
}

int rhy_server_replay(RhyServer* s, const char* const* exprs, const int* actions, const uint32_t* columns,
                      const double* min_proportions, const uint32_t* ks, const double* arrival_s, uint32_t n,
                      double* latency_ms, double* wall_s) {
   return guarded([&] {
      need(s, "server");
      if (n) {
         need(exprs, "exprs");
         need(arrival_s, "arrival_s");
      }
      std::vector<rhygpu::ServeRequest> reqs(n);
      std::vector<double> arr(arrival_s, arrival_s + n);
      for (uint32_t i = 0; i < n; ++i) {
         need(exprs[i], "expression");
         reqs[i].expr = exprs[i];
         reqs[i].action = actions ? actions[i] : 0;
         reqs[i].column = columns ? static_cast<int>(columns[i]) : 0;
         reqs[i].min_proportion = min_proportions ? min_proportions[i] : 0.05;
         reqs[i].k = ks ? ks[i] : 1000;
      }
      const std::vector<double> lat = s->server->replay(reqs, arr, wall_s);
      if (latency_ms) std::copy(lat.begin(), lat.end(), latency_ms);
   });
}

void rhy_server_stop(RhyServer* s) {
   if (!s) return;
   try {
      s->server->stop();
   } catch (...) {
   }
   delete s;
}

void rhy_close(RhyDevice* d) { delete d; }

}  // extern "C"
