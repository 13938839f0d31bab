// Filter expressions, their rewrite and compile to operator trees, and the lowering of operator
// trees to device programs.
//
// Expression -> Operator mirrors the reference:
//   ScalarExpression::rewrite(table, AmbiguityMode) and ::compile(table)
//     (src/rhydb/query_engine/scalar_expressions/scalar_expression.h:81-90),
//   Operator::negate (src/rhydb/query_engine/filter/operators/operator.cpp:23-66).
// The operator tree keeps the reference's node kinds (Empty, Full, IndexScan, Intersection, Union,
// Complement, Threshold, Selection with IsInCoveredRegion / date predicates) and the same shapes,
// so the row set it denotes is the reference's. Only its evaluation differs: instead of merging
// roaring containers on the CPU, the tree is lowered to a postorder program (program.h) that the
// GPU evaluates tile by tile.
//
// Textual expression syntax (positions are 1-based as in the reference's query language):
//   And(e, ...)  Or(e, ...)  Not(e)  NOf(n, exactly|atleast, e, ...)  Maybe(e)  Exact(e)
//   SymEq(column, pos, c)  with c a symbol character or '.' for the reference symbol
//   HasMut(column, pos)    StrEq(column, value)    DateBetween(column, from|*, to|*)
//   True  False
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "program.h"
#include "table.h"
#include "util.h"

namespace rhygpu {

enum class Ambiguity : uint8_t { UPPER_BOUND, LOWER_BOUND, NONE };

enum class EK : uint8_t { AND, OR, NOT, NOF, MAYBE, EXACT, SYM_EQ, HAS_MUT, SYM_IN_SET, STR_EQ, DATE_BETWEEN, BOOL,
                          MUT_PROFILE };

struct Expr;
using ExprPtr = std::unique_ptr<Expr>;

struct Expr {
   EK kind;
   std::vector<ExprPtr> children;
   std::string column;
   uint32_t pos = 0;        // 0-based position
   int sym = -1;            // SYM_EQ: symbol, -1 = '.' (reference symbol)
   uint32_t symmask = 0;    // SYM_IN_SET
   int n = 0;               // NOF
   bool exact = false;      // NOF
   std::string value;       // STR_EQ
   bool has_from = false, has_to = false;
   int32_t from = 0, to = 0;  // DATE_BETWEEN
   bool truth = false;      // BOOL
   SymKind sym_kind = SymKind::NUC;
   // MUT_PROFILE: n = distance; the profile is the sequence of the row whose primary key is
   // `value` when `by_id`, else `value` (a query sequence) when not empty, else the reference with
   // `muts` applied (position << 8 | symbol)
   std::vector<uint32_t> muts;
   bool by_id = false;

   ExprPtr clone() const;
   std::string to_string() const;
};

ExprPtr parse_expression(const std::string& text, const TableImage& table);

// ---------------------------------------------------------------------------------------------
// Operator trees

// ROWS: an IndexScan over a row set the caller supplies with the operator tree (the reference's
// IndexScan over any CopyOnWriteBitmap, e.g. a column index the device does not hold).
enum class OpT : uint8_t { EMPTY, FULL, INDEX_SCAN, INTERSECTION, UNION, COMPLEMENT, THRESHOLD, SELECTION, PROFILE,
                           ROWS };

// A MutationProfile as one operator: the rows with at most `distance` positions whose symbol is
// not compatible with the profile's symbol there, which is the row set of the reference's rewrite
// Not(NOf(distance + 1, SymbolInSet(position, incompatible symbols) for every position))
// (reference: src/rhydb/query_engine/scalar_expressions/mutation_profile.cpp:198-257). Counted per
// row from the row index: `base` differences for a covered row holding the local reference
// everywhere, corrected by the row's own symbols and by the positions it does not cover.
struct ProfileSpec {
   int col = 0;
   uint32_t distance = 0;
   uint32_t base = 0;
   // L: bit s = symbol s counts as a difference at the position; bit 31 = the local reference
   // symbol does (alphabets have at most 28 symbols)
   std::vector<uint32_t> mask;
   // L + 1: diff[p] = (positions < p where the missing symbol is a difference) - (positions < p
   // where the local reference symbol is one), stored as two's complement
   std::vector<uint32_t> diff;
};

struct Pred {
   enum Kind : uint8_t { COVERED, DATE } kind = COVERED;
   int col = 0;
   uint32_t pos = 0;
   bool covered = true;         // COVERED: IS_COVERED vs IS_NOT_COVERED
   uint32_t cmp = CMP_EQ;       // DATE
   int32_t value = 0;
   bool with_nulls = false;
   Pred negated() const;
};

struct Leaf {
   enum Kind : uint8_t { SEQ, NULLS, DICT } kind = SEQ;
   int col = 0;
   uint32_t pos = 0;
   uint32_t symmask = 0;
   uint32_t value = 0;
};

struct Op;
using OpPtr = std::unique_ptr<Op>;

struct Op {
   OpT t = OpT::EMPTY;
   std::vector<OpPtr> children;  // INTERSECTION/UNION/THRESHOLD non-negated; COMPLEMENT/SELECTION child
   std::vector<OpPtr> negated;   // INTERSECTION/THRESHOLD negated children
   std::vector<Pred> preds;      // SELECTION
   Leaf leaf;                    // INDEX_SCAN
   int n = 0;                    // THRESHOLD
   bool exact = false;           // THRESHOLD
   std::shared_ptr<const ProfileSpec> profile;  // PROFILE
   uint32_t rows_index = 0;                     // ROWS: index of the caller's row set
   double rows_card = 0;                        // ROWS: its cardinality (estimates only)
   std::string to_string() const;
};

ExprPtr rewrite(const Expr& e, const TableImage& t, Ambiguity mode);
OpPtr compile(const Expr& e, const TableImage& t);
OpPtr negate(OpPtr op);

// Estimated number of rows of an operator's result; drives child ordering and early exits only,
// never the result.
using Estimator = std::function<double(const Op&)>;
Estimator rule_estimator(const TableImage& t);
// The rule estimate of one node given an estimator for its children (the children's estimates may
// come from a memo; rule_estimator recurses).
double rule_node_estimate(const Op& op, const TableImage& t, const std::function<double(const Op&)>& child);

// Instructions [first, last] of one operator node: its result is on top of the stack after `last`.
struct NodeSpan {
   const Op* op;
   uint32_t first, last;
};

struct Program {
   std::vector<Instr> code;
   std::vector<NodeSpan> spans;  // with LowerOptions::record_spans; the ops belong to the caller's tree
   uint32_t max_depth = 0;   // tiles of stack needed
   uint32_t n_leaves = 0;
   uint32_t n_ctr_leaves = 0;  // PUSH_SCAN / PUSH_DICT leaves, numbered 1.. in their c field
   uint32_t n_cov_leaves = 0;  // PUSH_COVERED leaves, numbered 1.. in their c field
   // row sets computed before the program runs (PUSH_AUX leaves, numbered 0.. in their a field)
   std::vector<std::shared_ptr<const ProfileSpec>> aux;
   // caller row sets read by ROWS leaves: PUSH_AUX leaves numbered aux.size() + the caller's index;
   // the program reads the caller's sets 0 .. n_literals - 1
   uint32_t n_literals = 0;
};

struct LowerOptions {
   bool early_exit = true;   // emit JZ/JFULL after partial intersections/unions
   bool reorder = true;      // order children by the estimator
   bool record_spans = false;  // fill Program::spans
   // With the table's rows (> 0), an early-exit test is emitted only where the estimates (children
   // independent) put the partial result within exit_sel of empty (JZ) or of every row (JFULL);
   // elsewhere a tile practically never exits there and the test would cost a barrier for nothing.
   double rows = 0;
   double exit_sel = 0.01;
};

// parse -> rewrite(NONE) -> compile, without lowering.
OpPtr compile_filter(const std::string& text, const TableImage& t);

Program lower(const Op& op, const Estimator& est, const LowerOptions& opt);

// rewrite(NONE) -> compile -> lower (reference: src/rhydb/query_engine/operators/compute_filter.cpp:14-21).
Program plan_filter(const std::string& text, const TableImage& t, const Estimator* est, const LowerOptions& opt,
                    std::string* operator_tree = nullptr);

}  // namespace rhygpu
