// Operator trees across the C-ABI (op_program.h).
#include "op_program.h"

#include <stdexcept>
#include <string>
#include <utility>

#include "alphabet.h"

namespace rhygpu {

namespace {

// One operand of the postorder evaluation: an operator, or a predicate waiting for its Selection.
struct Operand {
   OpPtr op;
   bool is_pred = false;
   Pred pred;
};

std::string where(uint32_t i) { return "operator node " + std::to_string(i) + ": "; }

OpPtr make(OpT t) {
   auto o = std::make_unique<Op>();
   o->t = t;
   return o;
}

}  // namespace

OpPtr op_from_nodes(const RhyOpNode* nodes, uint32_t n, const TableImage& t, const std::vector<double>& row_set_cards) {
   if (n == 0) throw CompilationError("empty operator program");
   std::vector<Operand> st;
   auto pop_ops = [&](uint32_t i, uint32_t k) {
      if (st.size() < k) throw CompilationError(where(i) + "needs " + std::to_string(k) + " operands, the stack holds " +
                                                std::to_string(st.size()));
      std::vector<Operand> v;
      for (size_t j = st.size() - k; j < st.size(); ++j) v.push_back(std::move(st[j]));
      st.resize(st.size() - k);
      return v;
   };
   auto only_ops = [&](uint32_t i, std::vector<Operand>& v) {
      std::vector<OpPtr> out;
      for (auto& x : v) {
         if (x.is_pred) throw CompilationError(where(i) + "a predicate is only an operand of a Selection");
         out.push_back(std::move(x.op));
      }
      return out;
   };
   auto seq_col = [&](uint32_t i, uint32_t c) -> const SeqColumnImage& {
      if (c >= t.seq.size()) throw IllegalQuery(where(i) + "no sequence column " + std::to_string(c));
      return t.seq[c];
   };
   for (uint32_t i = 0; i < n; ++i) {
      const RhyOpNode& nd = nodes[i];
      Operand out;
      switch (nd.kind) {
         case RHY_NODE_EMPTY: out.op = make(OpT::EMPTY); break;
         case RHY_NODE_FULL: out.op = make(OpT::FULL); break;
         case RHY_NODE_SCAN_SEQ: {
            const SeqColumnImage& c = seq_col(i, nd.column);
            if (nd.position >= c.L)
               throw IllegalQuery(where(i) + "position " + std::to_string(nd.position) + " is outside the column's " +
                                  std::to_string(c.L) + " positions");
            const Alphabet& A = alphabet(c.kind);
            if (nd.symbols & ~A.all_mask) throw IllegalQuery(where(i) + "symbol bit outside the column's alphabet");
            out.op = make(OpT::INDEX_SCAN);
            out.op->leaf.kind = Leaf::SEQ;
            out.op->leaf.col = static_cast<int>(nd.column);
            out.op->leaf.pos = nd.position;
            out.op->leaf.symmask = nd.symbols;
            break;
         }
         case RHY_NODE_SCAN_NULLS:
            seq_col(i, nd.column);
            out.op = make(OpT::INDEX_SCAN);
            out.op->leaf.kind = Leaf::NULLS;
            out.op->leaf.col = static_cast<int>(nd.column);
            break;
         case RHY_NODE_SCAN_DICT:
            if (nd.column >= t.dict.size()) throw IllegalQuery(where(i) + "no dictionary column " + std::to_string(nd.column));
            if (nd.value >= t.dict[nd.column].values.size())
               throw IllegalQuery(where(i) + "no value id " + std::to_string(nd.value));
            out.op = make(OpT::INDEX_SCAN);
            out.op->leaf.kind = Leaf::DICT;
            out.op->leaf.col = static_cast<int>(nd.column);
            out.op->leaf.value = nd.value;
            break;
         case RHY_NODE_SCAN_ROWS:
            if (nd.value >= row_set_cards.size())
               throw std::invalid_argument(where(i) + "row set " + std::to_string(nd.value) + " was not passed");
            out.op = make(OpT::ROWS);
            out.op->rows_index = nd.value;
            out.op->rows_card = row_set_cards[nd.value];
            break;
         case RHY_NODE_INTERSECTION: {
            // reference: intersection.cpp:18-40
            if (nd.n_negated >= nd.n_children)
               throw CompilationError(where(i) +
                                      "Intersection without non-negated children is not allowed. Should be compiled as a union.");
            if (nd.n_children < 2) throw CompilationError(where(i) + "Intersection needs at least two children.");
            auto v = pop_ops(i, nd.n_children);
            auto ops = only_ops(i, v);
            out.op = make(OpT::INTERSECTION);
            const uint32_t pos = nd.n_children - nd.n_negated;
            for (uint32_t j = 0; j < nd.n_children; ++j)
               (j < pos ? out.op->children : out.op->negated).push_back(std::move(ops[j]));
            break;
         }
         case RHY_NODE_UNION: {
            auto v = pop_ops(i, nd.n_children);
            out.op = make(OpT::UNION);
            out.op->children = only_ops(i, v);
            break;
         }
         case RHY_NODE_COMPLEMENT: {
            if (nd.n_children != 1) throw CompilationError(where(i) + "Complement has exactly one child");
            auto v = pop_ops(i, 1);
            out.op = make(OpT::COMPLEMENT);
            out.op->children = only_ops(i, v);
            break;
         }
         case RHY_NODE_THRESHOLD: {
            // reference: threshold.cpp:18-41
            if (nd.n_negated > nd.n_children) throw CompilationError(where(i) + "more negated children than children");
            if (nd.value >= nd.n_children)
               throw CompilationError(where(i) + "Compilation Error: number_of_matchers must be less than the number of "
                                                 "children of a threshold expression");
            if (nd.value == 0)
               throw CompilationError(where(i) + "Compilation Error: number_of_matchers must be greater than zero");
            auto v = pop_ops(i, nd.n_children);
            auto ops = only_ops(i, v);
            out.op = make(OpT::THRESHOLD);
            out.op->n = static_cast<int>(nd.value);
            out.op->exact = (nd.flags & 1u) != 0;
            const uint32_t pos = nd.n_children - nd.n_negated;
            for (uint32_t j = 0; j < nd.n_children; ++j)
               (j < pos ? out.op->children : out.op->negated).push_back(std::move(ops[j]));
            break;
         }
         case RHY_NODE_SELECTION: {
            // reference: selection.cpp (a child operator, or none, filtered by ANDed predicates)
            auto v = pop_ops(i, nd.n_children);
            out.op = make(OpT::SELECTION);
            for (auto& x : v) {
               if (x.is_pred) {
                  out.op->preds.push_back(x.pred);
               } else {
                  if (!out.op->children.empty()) throw CompilationError(where(i) + "Selection has at most one child operator");
                  out.op->children.push_back(std::move(x.op));
               }
            }
            if (out.op->preds.empty()) throw CompilationError(where(i) + "Selection without predicates");
            break;
         }
         case RHY_NODE_PRED_COVERED: {
            const SeqColumnImage& c = seq_col(i, nd.column);
            if (nd.position >= c.L) throw IllegalQuery(where(i) + "position outside the column");
            out.is_pred = true;
            out.pred.kind = Pred::COVERED;
            out.pred.col = static_cast<int>(nd.column);
            out.pred.pos = nd.position;
            out.pred.covered = (nd.flags & 1u) == 0;
            break;
         }
         case RHY_NODE_PRED_DATE: {
            if (nd.column >= t.date.size()) throw IllegalQuery(where(i) + "no date column " + std::to_string(nd.column));
            if ((nd.flags & 7u) > CMP_GE) throw CompilationError(where(i) + "unknown comparator");
            out.is_pred = true;
            out.pred.kind = Pred::DATE;
            out.pred.col = static_cast<int>(nd.column);
            out.pred.cmp = nd.flags & 7u;
            out.pred.with_nulls = (nd.flags & 8u) != 0;
            out.pred.value = nd.date;
            break;
         }
         default: throw CompilationError(where(i) + "unknown node kind " + std::to_string(nd.kind));
      }
      st.push_back(std::move(out));
   }
   if (st.size() != 1) throw CompilationError("operator program leaves " + std::to_string(st.size()) + " operands, not one");
   if (st[0].is_pred) throw CompilationError("operator program ends with a predicate");
   return std::move(st[0].op);
}

void op_to_nodes(const Op& op, std::vector<RhyOpNode>& out) {
   RhyOpNode nd{};
   switch (op.t) {
      case OpT::EMPTY: nd.kind = RHY_NODE_EMPTY; break;
      case OpT::FULL: nd.kind = RHY_NODE_FULL; break;
      case OpT::INDEX_SCAN:
         nd.column = static_cast<uint32_t>(op.leaf.col);
         if (op.leaf.kind == Leaf::SEQ) {
            nd.kind = RHY_NODE_SCAN_SEQ;
            nd.position = op.leaf.pos;
            nd.symbols = op.leaf.symmask;
         } else if (op.leaf.kind == Leaf::NULLS) {
            nd.kind = RHY_NODE_SCAN_NULLS;
         } else {
            nd.kind = RHY_NODE_SCAN_DICT;
            nd.value = op.leaf.value;
         }
         break;
      case OpT::ROWS:
         nd.kind = RHY_NODE_SCAN_ROWS;
         nd.value = op.rows_index;
         break;
      case OpT::INTERSECTION:
      case OpT::THRESHOLD:
         for (const auto& c : op.children) op_to_nodes(*c, out);
         for (const auto& c : op.negated) op_to_nodes(*c, out);
         nd.kind = op.t == OpT::INTERSECTION ? RHY_NODE_INTERSECTION : RHY_NODE_THRESHOLD;
         nd.n_children = static_cast<uint32_t>(op.children.size() + op.negated.size());
         nd.n_negated = static_cast<uint32_t>(op.negated.size());
         if (op.t == OpT::THRESHOLD) {
            nd.value = static_cast<uint32_t>(op.n);
            nd.flags = op.exact ? 1u : 0u;
         }
         break;
      case OpT::UNION:
      case OpT::COMPLEMENT:
         for (const auto& c : op.children) op_to_nodes(*c, out);
         nd.kind = op.t == OpT::UNION ? RHY_NODE_UNION : RHY_NODE_COMPLEMENT;
         nd.n_children = static_cast<uint32_t>(op.children.size());
         break;
      case OpT::SELECTION:
         for (const auto& c : op.children) op_to_nodes(*c, out);
         for (const Pred& p : op.preds) {
            RhyOpNode q{};
            q.column = static_cast<uint32_t>(p.col);
            if (p.kind == Pred::COVERED) {
               q.kind = RHY_NODE_PRED_COVERED;
               q.position = p.pos;
               q.flags = p.covered ? 0u : 1u;
            } else {
               q.kind = RHY_NODE_PRED_DATE;
               q.flags = p.cmp | (p.with_nulls ? 8u : 0u);
               q.date = p.value;
            }
            out.push_back(q);
         }
         nd.kind = RHY_NODE_SELECTION;
         nd.n_children = static_cast<uint32_t>(op.children.size() + op.preds.size());
         break;
      case OpT::PROFILE:
         throw std::invalid_argument("a MutationProfile leaf has no operator-node form");
   }
   out.push_back(nd);
}

}  // namespace rhygpu
