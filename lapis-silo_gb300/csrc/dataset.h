// Raw table input and the seeded synthetic generator.
//
// A raw sequence column stores each aligned sequence as the global reference with a sorted list of
// non-overlapping character runs (pos, len, char) applied on top. This is lossless: every position
// outside the runs holds the reference character. It is the input the ingestion step diffs against
// the reference (reference: src/rhydb/common/aligned_sequence.cpp:19-122); N-runs and gap runs stay
// intervals so a 2M-row column is a few hundred MB instead of 60 GB of text.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "alphabet.h"

namespace rhygpu {

struct RawSeqColumn {
   std::string name;
   SymKind kind = SymKind::NUC;
   std::string reference;           // global reference, one char per position
   std::vector<uint8_t> is_null;    // per row
   std::vector<uint64_t> row_off;   // n_rows + 1 offsets into the run arrays
   std::vector<uint32_t> run_pos;
   std::vector<uint32_t> run_len;
   std::vector<char> run_char;
};

struct RawDictColumn {
   std::string name;
   std::vector<std::string> values;  // dictionary
   std::vector<uint32_t> ids;        // per row, UINT32_MAX = null
};

struct RawDateColumn {
   std::string name;
   std::vector<int32_t> days;  // per row, INT32_MIN = null
};

struct RawTable {
   uint32_t n_rows = 0;
   std::vector<RawSeqColumn> seq;   // seq[0] is the nucleotide column, the rest amino-acid genes
   std::vector<RawDictColumn> dict;
   std::vector<RawDateColumn> date;
};

struct GenConfig {
   uint64_t seed = 42;
   uint32_t n_rows = 100000;
   uint32_t genome_len = 29903;
   uint32_t pool_sites = 5000;
   double pool_ambiguous_fraction = 0.03;  // share of pool sites whose symbol is an IUPAC ambiguity code
   double subs_mean = 30.0;
   double zipf_s = 1.1;
   double nrun_mean = 2.0;
   uint32_t nrun_min = 50, nrun_max = 500;
   double gap_mean = 0.5;
   uint32_t gap_min = 3, gap_max = 30;
   double null_fraction = 0.0;
   uint32_t n_countries = 200, n_lineages = 2000;
   int32_t date_base = 18262;  // 2020-01-01 as days since 1970-01-01
   uint32_t date_days = 1096;  // three years
   uint32_t n_aa_genes = 0;    // 0 = nucleotide column only; 12 = 9,700 aa over 12 genes
   uint32_t threads = 0;       // 0 = hardware concurrency
};

struct PoolSite {
   uint32_t pos;
   char ch;
};

struct Gene {
   std::string name;
   uint32_t nuc_start;
   uint32_t aa_len;
};

struct GeneratedTable {
   RawTable table;
   std::vector<PoolSite> pool;      // nucleotide pool, rank order (rank 1 first)
   std::vector<Gene> genes;
   // Amino-acid sites reachable from one pool substitution: (gene index, aa position, aa char).
   std::vector<uint32_t> aa_site_gene, aa_site_pos;
   std::vector<char> aa_site_char;
};

GeneratedTable generate_table(const GenConfig& cfg);

// Materialise one row of a raw column as a string (used by tests on small tables).
std::string materialize_row(const RawSeqColumn& col, uint32_t row);

struct QueryGenConfig {
   uint64_t seed = 43;
   uint32_t n_queries = 1000;
   uint32_t max_depth = 4;
   uint32_t max_nof_children = 8;
   bool use_aa = false;        // amino-acid leaves
   bool use_metadata = false;  // country/lineage equality, date ranges
   bool use_ambiguity = true;  // Maybe/Exact wrappers and ambiguity symbols
   uint32_t max_leaves = 0;    // leaves per tree at most (0 = no limit)
};

// Seeded random filter expressions in the textual expression syntax of expr.h.
std::vector<std::string> generate_queries(const GeneratedTable& gen, const QueryGenConfig& cfg);

}  // namespace rhygpu
