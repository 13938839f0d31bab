// A C++ caller of include/rhydb_gpu.h, compiled with g++ against the header alone and linked to
// librhygpu.so, as RhyDB would bind it. tests/test_capi_client.py builds and runs it and checks its
// output against the oracle.
//
// Usage: capi_client host             table, planning and operator-tree calls (no GPU)
//        capi_client gpu              the same, then rhy_open / rhy_count / rhy_eval /
//                                     rhy_mutations / rhy_program_count / rhy_batch_rows /
//                                     rhy_close on GPU 0
// Output: one line per result, "<kind> <index> <values...>", for the checker to compare.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "rhydb_gpu.h"

namespace {

int fail(const char* what, int rc) {
   std::fprintf(stderr, "%s failed: %d %s\n", what, rc, rhy_last_error());
   return 1;
}

std::vector<std::string> split_lines(const std::vector<char>& buf) {
   std::vector<std::string> out;
   std::string cur;
   for (char c : buf) {
      if (c == '\0') break;
      if (c == '\n') {
         if (!cur.empty()) out.push_back(cur);
         cur.clear();
      } else {
         cur.push_back(c);
      }
   }
   if (!cur.empty()) out.push_back(cur);
   return out;
}

}  // namespace

int main(int argc, char** argv) {
   const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
   RhyGenConfig cfg{};
   cfg.seed = 7;
   cfg.n_rows = 70000;
   cfg.genome_len = 3000;
   cfg.pool_sites = 300;
   cfg.n_aa_genes = 0;
   cfg.null_fraction = 0.01;
   RhyTable* table = nullptr;
   int rc = rhy_generate(&cfg, &table);
   if (rc != RHY_OK) return fail("rhy_generate", rc);
   RhyTableInfo info{};
   if ((rc = rhy_table_info(table, &info)) != RHY_OK) return fail("rhy_table_info", rc);
   std::printf("info %u %u %u\n", info.n_rows, info.n_chunks, info.n_seq);

   size_t needed = 0;
   rhy_generate_queries(table, 11, 16, 4, 8, 0, 0, 1, nullptr, 0, &needed);
   std::vector<char> buf(needed);
   if ((rc = rhy_generate_queries(table, 11, 16, 4, 8, 0, 0, 1, buf.data(), buf.size(), &needed)) != RHY_OK)
      return fail("rhy_generate_queries", rc);
   const std::vector<std::string> queries = split_lines(buf);
   for (size_t i = 0; i < queries.size(); ++i) std::printf("query %zu %s\n", i, queries[i].c_str());

   // planning and operator trees on the host
   std::vector<std::vector<RhyOpNode>> programs;
   for (size_t i = 0; i < queries.size(); ++i) {
      uint32_t n_instr = 0, depth = 0;
      std::vector<char> tree(1 << 16);
      if ((rc = rhy_plan(table, queries[i].c_str(), tree.data(), tree.size(), &n_instr, &depth)) != RHY_OK)
         return fail("rhy_plan", rc);
      size_t n = 0;
      if ((rc = rhy_program_from_expr(table, queries[i].c_str(), nullptr, 0, &n)) != RHY_OK)
         return fail("rhy_program_from_expr", rc);
      std::vector<RhyOpNode> nodes(n);
      if ((rc = rhy_program_from_expr(table, queries[i].c_str(), nodes.data(), n, &n)) != RHY_OK)
         return fail("rhy_program_from_expr", rc);
      RhyOpProgram prog{nodes.data(), static_cast<uint32_t>(n), 0, nullptr};
      std::vector<char> tree2(1 << 16);
      if ((rc = rhy_program_plan(table, &prog, tree2.data(), tree2.size(), nullptr, nullptr)) != RHY_OK)
         return fail("rhy_program_plan", rc);
      std::printf("plan %zu %u %u %d\n", i, n_instr, depth, std::strcmp(tree.data(), tree2.data()) == 0 ? 1 : 0);
      programs.push_back(std::move(nodes));
   }
   // user errors come back as codes with a message, never as exceptions
   rc = rhy_plan(table, "SymEq(main,999999,A)", nullptr, 0, nullptr, nullptr);
   std::printf("error %d %d\n", rc, std::strlen(rhy_last_error()) > 0 ? 1 : 0);
   RhyOpNode bad{};
   bad.kind = RHY_NODE_INTERSECTION;
   bad.n_children = 2;
   RhyOpProgram bad_prog{&bad, 1, 0, nullptr};
   rc = rhy_program_plan(table, &bad_prog, nullptr, 0, nullptr, nullptr);
   std::printf("error %d %d\n", rc, std::strlen(rhy_last_error()) > 0 ? 1 : 0);

   if (gpu) {
      RhyDevice* dev = nullptr;
      if ((rc = rhy_open(table, 0, &dev)) != RHY_OK) return fail("rhy_open", rc);
      RhySeqColumnInfo col{};
      if ((rc = rhy_seq_column_info(table, 0, &col)) != RHY_OK) return fail("rhy_seq_column_info", rc);
      for (size_t i = 0; i < queries.size(); ++i) {
         uint64_t count = 0, eval_count = 0, prog_count = 0;
         if ((rc = rhy_count(dev, queries[i].c_str(), nullptr, &count)) != RHY_OK) return fail("rhy_count", rc);
         std::vector<uint32_t> bits(static_cast<size_t>(info.n_chunks) * 2048);
         if ((rc = rhy_eval(dev, queries[i].c_str(), nullptr, bits.data(), &eval_count)) != RHY_OK)
            return fail("rhy_eval", rc);
         uint64_t first = UINT64_MAX;
         for (size_t w = 0; w < bits.size() && first == UINT64_MAX; ++w)
            if (bits[w]) first = w * 32 + static_cast<uint64_t>(__builtin_ctz(bits[w]));
         RhyOpProgram prog{programs[i].data(), static_cast<uint32_t>(programs[i].size()), 0, nullptr};
         if ((rc = rhy_program_count(dev, &prog, nullptr, &prog_count)) != RHY_OK) return fail("rhy_program_count", rc);
         std::printf("count %zu %llu %llu %llu %lld\n", i, static_cast<unsigned long long>(count),
                     static_cast<unsigned long long>(eval_count), static_cast<unsigned long long>(prog_count),
                     first == UINT64_MAX ? -1LL : static_cast<long long>(first));
      }
      for (size_t i = 0; i < 4 && i < queries.size(); ++i) {
         std::vector<uint32_t> counts(static_cast<size_t>(col.n_symbols) * col.L);
         uint64_t fc = 0;
         if ((rc = rhy_mutations(dev, queries[i].c_str(), 0, nullptr, counts.data(), &fc)) != RHY_OK)
            return fail("rhy_mutations", rc);
         uint64_t sum = 0, weighted = 0;
         for (size_t k = 0; k < counts.size(); ++k) {
            sum += counts[k];
            weighted += counts[k] * (k % 9973 + 1);
         }
         std::printf("mutations %zu %llu %llu %llu\n", i, static_cast<unsigned long long>(fc),
                     static_cast<unsigned long long>(sum), static_cast<unsigned long long>(weighted));
      }
      // the batched call with rows built on the device
      std::vector<const char*> exprs;
      std::vector<int> actions;
      std::vector<uint32_t> columns;
      for (size_t i = 0; i < queries.size(); ++i) {
         exprs.push_back(queries[i].c_str());
         actions.push_back(i % 2);
         columns.push_back(0);
      }
      const uint32_t n = static_cast<uint32_t>(exprs.size());
      std::vector<uint64_t> counts(n), begin(n);
      std::vector<uint32_t> nrows(n);
      std::vector<RhyMutationRow> rows(1 << 16);
      size_t total = 0;
      if ((rc = rhy_batch_rows(dev, exprs.data(), actions.data(), columns.data(), nullptr, n, 0, nullptr, counts.data(),
                               rows.data(), rows.size(), begin.data(), nrows.data(), &total)) != RHY_OK)
         return fail("rhy_batch_rows", rc);
      for (uint32_t i = 0; i < n; ++i) {
         std::printf("batch %u %llu %u", i, static_cast<unsigned long long>(counts[i]), nrows[i]);
         for (uint32_t r = 0; r < nrows[i] && r < 3; ++r) {
            const RhyMutationRow& m = rows[begin[i] + r];
            std::printf(" %u:%c:%c:%u:%u:%.17g", m.position, m.from, m.to, m.count, m.coverage, m.proportion);
         }
         std::printf("\n");
      }
      rhy_close(dev);
   }
   rhy_table_free(table);
   std::printf("done\n");
   return 0;
}
