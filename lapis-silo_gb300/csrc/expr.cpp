// Expression parsing, rewrite, compile and lowering (see expr.h).
#include "expr.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <map>
#include <string_view>

namespace rhygpu {

// =============================================================================================
// Expression basics

ExprPtr Expr::clone() const {
   auto e = std::make_unique<Expr>();
   e->kind = kind;
   for (const auto& c : children) e->children.push_back(c->clone());
   e->column = column;
   e->pos = pos;
   e->sym = sym;
   e->symmask = symmask;
   e->n = n;
   e->exact = exact;
   e->value = value;
   e->has_from = has_from;
   e->has_to = has_to;
   e->from = from;
   e->to = to;
   e->truth = truth;
   e->sym_kind = sym_kind;
   e->muts = muts;
   e->by_id = by_id;
   return e;
}

std::string Expr::to_string() const {
   auto join = [&](const char* name) {
      std::string s = name;
      s += "(";
      for (size_t i = 0; i < children.size(); ++i) {
         if (i) s += ",";
         s += children[i]->to_string();
      }
      return s + ")";
   };
   const Alphabet& A = alphabet(sym_kind);
   switch (kind) {
      case EK::AND: return join("And");
      case EK::OR: return join("Or");
      case EK::NOT: return "Not(" + children[0]->to_string() + ")";
      case EK::MAYBE: return "Maybe(" + children[0]->to_string() + ")";
      case EK::EXACT: return "Exact(" + children[0]->to_string() + ")";
      case EK::NOF: {
         std::string s = "NOf(" + std::to_string(n) + (exact ? ",exactly" : ",atleast");
         for (const auto& c : children) s += "," + c->to_string();
         return s + ")";
      }
      case EK::SYM_EQ:
         return "SymEq(" + column + "," + std::to_string(pos + 1) + "," + (sym < 0 ? '.' : A.chars[sym]) + ")";
      case EK::HAS_MUT: return "HasMut(" + column + "," + std::to_string(pos + 1) + ")";
      case EK::SYM_IN_SET: {
         std::string s = "SymInSet(" + column + "," + std::to_string(pos + 1) + ",";
         for (uint32_t i = 0; i < A.count; ++i)
            if (symmask >> i & 1) s += A.chars[i];
         return s + ")";
      }
      case EK::STR_EQ: return "StrEq(" + column + "," + value + ")";
      case EK::DATE_BETWEEN:
         return "DateBetween(" + column + "," + (has_from ? std::to_string(from) : "*") + "," +
                (has_to ? std::to_string(to) : "*") + ")";
      case EK::BOOL: return truth ? "True" : "False";
      case EK::MUT_PROFILE: {
         if (by_id) return "MutProfileSequenceId(" + column + "," + std::to_string(n) + "," + value + ")";
         if (!value.empty()) return "MutProfile(" + column + "," + std::to_string(n) + "," + value + ")";
         std::string s = "MutProfileMutations(" + column + "," + std::to_string(n);
         for (uint32_t m : muts) s += "," + std::to_string((m >> 8) + 1) + ":" + A.chars[m & 0xFFu];
         return s + ")";
      }
   }
   return "?";
}

// =============================================================================================
// Parser

namespace {

struct Parser {
   const std::string& s;
   const TableImage& t;
   size_t i = 0;

   static bool space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }
   [[noreturn]] void fail(const std::string& msg) const {
      throw IllegalQuery("cannot parse expression at offset " + std::to_string(i) + ": " + msg);
   }
   void ws() {
      while (i < s.size() && space(s[i])) ++i;
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
      if (!eat(c)) fail(std::string("expected '") + c + "'");
   }
   // The next token, a view into the text (valid while the text is).
   std::string_view token() {
      ws();
      const size_t b = i;
      while (i < s.size() && s[i] != ',' && s[i] != '(' && s[i] != ')' && !space(s[i])) ++i;
      if (b == i) fail("expected a token");
      return std::string_view(s).substr(b, i - b);
   }
   // A base-10 integer with an optional sign, the whole token, within the range of long long.
   long long integer() {
      const std::string_view tok = token();
      size_t k = 0;
      const bool neg = tok[0] == '-';
      if (tok[0] == '-' || tok[0] == '+') k = 1;
      unsigned long long v = 0;
      const unsigned long long lim = neg ? 9223372036854775808ull : 9223372036854775807ull;
      bool ok = k < tok.size();
      for (; ok && k < tok.size(); ++k) {
         const char c = tok[k];
         if (c < '0' || c > '9') ok = false;
         else if (v > (lim - static_cast<unsigned long long>(c - '0')) / 10) ok = false;
         else v = v * 10 + static_cast<unsigned long long>(c - '0');
      }
      if (!ok) fail("expected an integer, got '" + std::string(tok) + "'");
      return neg ? static_cast<long long>(0ull - v) : static_cast<long long>(v);
   }
   uint32_t position() {
      const long long p = integer();
      if (p < 1 || p > 0xFFFFFFFFll) fail("positions are 1-based");
      return static_cast<uint32_t>(p - 1);
   }

   ExprPtr node(EK k) {
      auto e = std::make_unique<Expr>();
      e->kind = k;
      return e;
   }

   void seq_column(Expr& e) {
      e.column = std::string(token());
      const int c = t.find_seq(e.column);
      if (c < 0) throw IllegalQuery("the database does not contain the sequence column '" + e.column + "'");
      e.sym_kind = t.seq[c].kind;
   }

   ExprPtr parse() {
      const std::string_view name = token();
      if (name == "True" || name == "False") {
         auto e = node(EK::BOOL);
         e->truth = name == "True";
         return e;
      }
      expect('(');
      ExprPtr e;
      if (name == "And" || name == "Or") {
         e = node(name == "And" ? EK::AND : EK::OR);
         if (!eat(')')) {
            do {
               e->children.push_back(parse());
            } while (eat(','));
            expect(')');
         }
         return e;
      }
      if (name == "Not" || name == "Maybe" || name == "Exact") {
         e = node(name == "Not" ? EK::NOT : name == "Maybe" ? EK::MAYBE : EK::EXACT);
         e->children.push_back(parse());
      } else if (name == "NOf") {
         e = node(EK::NOF);
         const long long n = integer();
         if (n < -1000000 || n > 1000000) fail("NOf count out of range");
         e->n = static_cast<int>(n);
         expect(',');
         const std::string_view mode = token();
         if (mode != "exactly" && mode != "atleast") fail("NOf mode must be exactly or atleast");
         e->exact = mode == "exactly";
         while (eat(',')) e->children.push_back(parse());
      } else if (name == "SymEq") {
         e = node(EK::SYM_EQ);
         seq_column(*e);
         expect(',');
         e->pos = position();
         expect(',');
         const std::string_view c = token();
         if (c.size() != 1) fail("a symbol is a single character");
         if (c[0] == '.') {
            e->sym = -1;
         } else {
            e->sym = alphabet(e->sym_kind).sym(c[0]);
            if (e->sym < 0) throw IllegalQuery("illegal symbol '" + std::string(c) + "' for column " + e->column);
         }
      } else if (name == "HasMut") {
         e = node(EK::HAS_MUT);
         seq_column(*e);
         expect(',');
         e->pos = position();
      } else if (name == "StrEq") {
         e = node(EK::STR_EQ);
         e->column = std::string(token());
         expect(',');
         e->value = std::string(token());
      } else if (name == "DateBetween") {
         e = node(EK::DATE_BETWEEN);
         e->column = std::string(token());
         expect(',');
         if (eat('*')) {
            e->has_from = false;
         } else {
            e->has_from = true;
            e->from = static_cast<int32_t>(integer());
         }
         expect(',');
         if (eat('*')) {
            e->has_to = false;
         } else {
            e->has_to = true;
            e->to = static_cast<int32_t>(integer());
         }
      } else if (name == "MutProfile" || name == "MutProfileMutations" || name == "MutProfileSequenceId") {
         // MutProfile(column, distance, query sequence) / MutProfileMutations(column, distance,
         // position:symbol, ...) / MutProfileSequenceId(column, distance, primary key)
         // (reference: mutation_profile.cpp, querySequence, mutations and sequenceId input)
         e = node(EK::MUT_PROFILE);
         seq_column(*e);
         expect(',');
         const long long d = integer();
         if (d < 0 || d > 0x7FFFFFFFll) fail("the distance must not be negative");
         e->n = static_cast<int>(d);
         if (name == "MutProfile" || name == "MutProfileSequenceId") {
            expect(',');
            e->value = std::string(token());
            e->by_id = name == "MutProfileSequenceId";
         } else {
            while (eat(',')) {
               const std::string_view m = token();
               const size_t colon = m.find(':');
               if (colon == std::string_view::npos || colon + 2 != m.size()) fail("a mutation is position:symbol");
               uint64_t p = 0;
               for (size_t k = 0; k < colon; ++k) {
                  if (m[k] < '0' || m[k] > '9' || p > 0xFFFFFFull) fail("a mutation is position:symbol");
                  p = p * 10 + static_cast<uint64_t>(m[k] - '0');
               }
               if (p < 1) fail("positions are 1-based");
               const int sy = alphabet(e->sym_kind).sym(m[colon + 1]);
               if (sy < 0) throw IllegalQuery("illegal symbol '" + std::string(1, m[colon + 1]) + "' for column " + e->column);
               e->muts.push_back(static_cast<uint32_t>(p - 1) << 8 | static_cast<uint32_t>(sy));
            }
         }
      } else {
         fail("unknown function '" + std::string(name) + "'");
      }
      expect(')');
      return e;
   }
};

}  // namespace

ExprPtr parse_expression(const std::string& text, const TableImage& table) {
   Parser p{text, table};
   ExprPtr e = p.parse();
   p.ws();
   if (p.i != text.size()) p.fail("trailing characters");
   return e;
}

// =============================================================================================
// Rewrite (reference: and.cpp:154-162, or.cpp:173-192, negation.cpp:27-30, nof.cpp:217-257,
// maybe.cpp:28-33, exact.cpp:28-33, symbol_equals.cpp:65-93, has_mutation.cpp:34-68)

namespace {

Ambiguity invert(Ambiguity m) {
   if (m == Ambiguity::UPPER_BOUND) return Ambiguity::LOWER_BOUND;
   if (m == Ambiguity::LOWER_BOUND) return Ambiguity::UPPER_BOUND;
   return m;
}

const SeqColumnImage& seq_col(const TableImage& t, const std::string& name) {
   const int c = t.find_seq(name);
   if (c < 0) throw IllegalQuery("the database does not contain the sequence column '" + name + "'");
   return t.seq[c];
}

}  // namespace

ExprPtr rewrite(const Expr& e, const TableImage& t, Ambiguity mode) {
   switch (e.kind) {
      case EK::AND: {
         auto out = std::make_unique<Expr>();
         out->kind = EK::AND;
         for (const auto& c : e.children) out->children.push_back(rewrite(*c, t, mode));
         return out;
      }
      case EK::OR: {
         // collectChildren: flatten nested Or through a LIFO queue (or.cpp:26-57)
         std::vector<const Expr*> collected, queue;
         for (const auto& c : e.children) queue.push_back(c.get());
         while (!queue.empty()) {
            const Expr* cur = queue.back();
            queue.pop_back();
            if (cur->kind == EK::OR) {
               for (const auto& c : cur->children) queue.push_back(c.get());
            } else {
               collected.push_back(cur);
            }
         }
         std::vector<ExprPtr> rewritten;
         for (const Expr* c : collected) rewritten.push_back(rewrite(*c, t, mode));
         // algebraicSimplification (or.cpp:66-90)
         std::vector<ExprPtr> non_trivial;
         while (!rewritten.empty()) {
            ExprPtr child = std::move(rewritten.back());
            rewritten.pop_back();
            if (child->kind == EK::BOOL) {
               if (child->truth) {
                  std::vector<ExprPtr> only;
                  auto tr = std::make_unique<Expr>();
                  tr->kind = EK::BOOL;
                  tr->truth = true;
                  only.push_back(std::move(tr));
                  non_trivial = std::move(only);
                  break;
               }
               continue;
            }
            if (child->kind == EK::OR) {
               for (auto& g : child->children) rewritten.push_back(std::move(g));
            } else {
               non_trivial.push_back(std::move(child));
            }
         }
         // merge SymbolInSet children per (column, position), nucleotide then amino acid (or.cpp:92-116)
         for (SymKind kind : {SymKind::NUC, SymKind::AA}) {
            std::vector<ExprPtr> next;
            std::map<std::pair<std::string, uint32_t>, uint32_t> merged;
            for (auto& c : non_trivial) {
               if (c->kind == EK::SYM_IN_SET && c->sym_kind == kind) {
                  merged[{c->column, c->pos}] |= c->symmask;
               } else {
                  next.push_back(std::move(c));
               }
            }
            for (const auto& [key, mask] : merged) {
               auto s = std::make_unique<Expr>();
               s->kind = EK::SYM_IN_SET;
               s->column = key.first;
               s->pos = key.second;
               s->symmask = mask;
               s->sym_kind = kind;
               next.push_back(std::move(s));
            }
            non_trivial = std::move(next);
         }
         if (non_trivial.size() == 1) return std::move(non_trivial[0]);
         auto out = std::make_unique<Expr>();
         out->kind = EK::OR;
         out->children = std::move(non_trivial);
         return out;
      }
      case EK::NOT: {
         auto out = std::make_unique<Expr>();
         out->kind = EK::NOT;
         out->children.push_back(rewrite(*e.children[0], t, invert(mode)));
         return out;
      }
      case EK::MAYBE: return rewrite(*e.children[0], t, Ambiguity::UPPER_BOUND);
      case EK::EXACT: return rewrite(*e.children[0], t, Ambiguity::LOWER_BOUND);
      case EK::NOF: {
         auto rewrite_children = [&]() {
            std::vector<ExprPtr> v;
            for (const auto& c : e.children) v.push_back(rewrite(*c, t, mode));
            return v;
         };
         if (mode != Ambiguity::NONE && e.exact && (e.n < 0 || static_cast<size_t>(e.n) < e.children.size())) {
            auto at_least_k = std::make_unique<Expr>();
            at_least_k->kind = EK::NOF;
            at_least_k->children = rewrite_children();
            at_least_k->n = e.n;
            at_least_k->exact = false;
            auto at_least_k1 = std::make_unique<Expr>();
            at_least_k1->kind = EK::NOF;
            at_least_k1->children = rewrite_children();
            at_least_k1->n = e.n + 1;
            at_least_k1->exact = false;
            auto neg = std::make_unique<Expr>();
            neg->kind = EK::NOT;
            neg->children.push_back(std::move(at_least_k1));
            auto out = std::make_unique<Expr>();
            out->kind = EK::AND;
            out->children.push_back(std::move(at_least_k));
            out->children.push_back(std::move(neg));
            return out;
         }
         auto out = std::make_unique<Expr>();
         out->kind = EK::NOF;
         out->n = e.n;
         out->exact = e.exact;
         out->children = rewrite_children();
         return out;
      }
      case EK::SYM_EQ: {
         const SeqColumnImage& col = seq_col(t, e.column);
         if (e.pos >= col.L)
            throw IllegalQuery("SymbolEquals position is out of bounds " + std::to_string(e.pos + 1) + " > " + std::to_string(col.L));
         const uint32_t symbol = e.sym < 0 ? col.global_ref[e.pos] : static_cast<uint32_t>(e.sym);
         auto out = std::make_unique<Expr>();
         out->kind = EK::SYM_IN_SET;
         out->column = e.column;
         out->pos = e.pos;
         out->sym_kind = col.kind;
         out->symmask = mode == Ambiguity::UPPER_BOUND ? alphabet(col.kind).ambiguity[symbol] : (1u << symbol);
         return out;
      }
      case EK::HAS_MUT: {
         const SeqColumnImage& col = seq_col(t, e.column);
         if (e.pos >= col.L)
            throw IllegalQuery("HasMutation position is out of bounds " + std::to_string(e.pos + 1) + " > " + std::to_string(col.L));
         const Alphabet& A = alphabet(col.kind);
         const uint32_t ref = col.global_ref[e.pos];
         uint32_t mask = A.all_mask;
         if (mode == Ambiguity::UPPER_BOUND) {
            mask &= ~(1u << ref);
         } else {
            mask &= ~A.ambiguity[ref];
         }
         auto out = std::make_unique<Expr>();
         out->kind = EK::SYM_IN_SET;
         out->column = e.column;
         out->pos = e.pos;
         out->sym_kind = col.kind;
         out->symmask = mask;
         return out;
      }
      case EK::SYM_IN_SET:
         throw CompilationError("Cannot rewrite SymbolInSet - this expression should only be created during query rewrites");
      case EK::STR_EQ:
         if (t.find_dict(e.column) < 0) throw IllegalQuery("the database does not contain the indexed string column '" + e.column + "'");
         return e.clone();
      case EK::DATE_BETWEEN:
         if (t.find_date(e.column) < 0) throw IllegalQuery("the database does not contain the date column '" + e.column + "'");
         return e.clone();
      case EK::BOOL: return e.clone();
      case EK::MUT_PROFILE:
         // the ambiguity mode does not apply (mutation_profile.cpp:198-201)
         seq_col(t, e.column);
         return e.clone();
   }
   throw CompilationError("unknown expression kind");
}

// =============================================================================================
// Operators

Pred Pred::negated() const {
   Pred p = *this;
   if (kind == COVERED) {
      p.covered = !covered;
      return p;
   }
   // reference: selection.h:127-157 (the comparator flips and nulls flip)
   switch (cmp) {
      case CMP_EQ: p.cmp = CMP_NE; break;
      case CMP_NE: p.cmp = CMP_EQ; break;
      case CMP_LT: p.cmp = CMP_GE; break;
      case CMP_GE: p.cmp = CMP_LT; break;
      case CMP_GT: p.cmp = CMP_LE; break;
      case CMP_LE: p.cmp = CMP_GT; break;
   }
   p.with_nulls = !with_nulls;
   return p;
}

namespace {

OpPtr mk(OpT t) {
   auto o = std::make_unique<Op>();
   o->t = t;
   return o;
}
OpPtr complement_of(OpPtr c) {
   auto o = mk(OpT::COMPLEMENT);
   o->children.push_back(std::move(c));
   return o;
}
OpPtr intersection_of(std::vector<OpPtr> pos, std::vector<OpPtr> neg) {
   // reference: intersection.cpp:18-41
   if (pos.empty()) throw CompilationError("Compilation bug: Intersection without non-negated children is not allowed.");
   if (pos.size() + neg.size() < 2) throw CompilationError("Compilation bug: Intersection needs at least two children.");
   auto o = mk(OpT::INTERSECTION);
   o->children = std::move(pos);
   o->negated = std::move(neg);
   return o;
}
OpPtr union_of(std::vector<OpPtr> c) {
   auto o = mk(OpT::UNION);
   o->children = std::move(c);
   return o;
}
OpPtr scan_of(Leaf l) {
   auto o = mk(OpT::INDEX_SCAN);
   o->leaf = l;
   return o;
}
OpPtr selection_of(OpPtr child, std::vector<Pred> preds) {
   auto o = mk(OpT::SELECTION);
   if (child) o->children.push_back(std::move(child));
   o->preds = std::move(preds);
   return o;
}
OpPtr threshold_of(std::vector<OpPtr> pos, std::vector<OpPtr> neg, int n, bool exact) {
   // reference: threshold.cpp:18-41
   if (static_cast<size_t>(n) >= pos.size() + neg.size())
      throw CompilationError("Compilation Error: number_of_matchers must be less than the number of children of a threshold expression");
   if (n == 0) throw CompilationError("Compilation Error: number_of_matchers must be greater than zero");
   auto o = mk(OpT::THRESHOLD);
   o->children = std::move(pos);
   o->negated = std::move(neg);
   o->n = n;
   o->exact = exact;
   return o;
}

// reference: symbol_in_set.cpp:105-264
OpPtr compile_symbol_in_set(const TableImage& t, const Expr& e) {
   const int ci = t.find_seq(e.column);
   if (ci < 0) throw IllegalQuery("the database does not contain the sequence column '" + e.column + "'");
   const SeqColumnImage& col = t.seq[ci];
   if (e.pos >= col.L)
      throw IllegalQuery("SymbolInSet position is out of bounds " + std::to_string(e.pos + 1) + " > " + std::to_string(col.L));
   const Alphabet& A = alphabet(col.kind);
   const uint32_t local_ref = col.local_ref[e.pos];
   const bool has_ref = e.symmask >> local_ref & 1;
   const bool has_missing = e.symmask >> A.missing & 1;
   auto scan = [&](uint32_t mask) {
      Leaf l;
      l.kind = Leaf::SEQ;
      l.col = ci;
      l.pos = e.pos;
      l.symmask = mask & A.all_mask;
      return scan_of(l);
   };
   auto exclude_nulls = [&](OpPtr op) {
      if (col.null_rows.empty()) return op;
      Leaf l;
      l.kind = Leaf::NULLS;
      l.col = ci;
      std::vector<OpPtr> pos, neg;
      pos.push_back(std::move(op));
      neg.push_back(scan_of(l));
      return intersection_of(std::move(pos), std::move(neg));
   };
   Pred covered;
   covered.kind = Pred::COVERED;
   covered.col = ci;
   covered.pos = e.pos;
   if (has_ref && has_missing) {
      return exclude_nulls(complement_of(scan(A.all_mask & ~e.symmask)));
   }
   if (has_missing) {
      covered.covered = false;
      std::vector<OpPtr> u;
      u.push_back(selection_of(nullptr, {covered}));
      u.push_back(scan(e.symmask));
      return exclude_nulls(union_of(std::move(u)));
   }
   if (has_ref) {
      covered.covered = true;
      std::vector<OpPtr> pos, neg;
      pos.push_back(selection_of(nullptr, {covered}));
      neg.push_back(scan(A.all_mask & ~e.symmask & ~(1u << A.missing)));
      return intersection_of(std::move(pos), std::move(neg));
   }
   return scan(e.symmask);
}

// NOf helpers (reference: nof.cpp:33-150)
OpPtr nof_trivial(int n, std::vector<OpPtr>& pos, std::vector<OpPtr>& neg, bool exact) {
   const int k = static_cast<int>(pos.size() + neg.size());
   if (n > k) return mk(OpT::EMPTY);
   if (n < 0) return exact ? mk(OpT::EMPTY) : mk(OpT::FULL);
   if (n == 0) {
      if (!exact) return mk(OpT::FULL);
      if (k == 0) return mk(OpT::FULL);
      if (k == 1) {
         if (pos.empty()) return std::move(neg[0]);
         return complement_of(std::move(pos[0]));
      }
      if (neg.empty()) return complement_of(union_of(std::move(pos)));
      return intersection_of(std::move(neg), std::move(pos));
   }
   if (n == 1 && k == 1) {
      if (neg.empty()) return std::move(pos[0]);
      return complement_of(std::move(neg[0]));
   }
   return nullptr;
}

OpPtr nof_to_operator(int n, std::vector<OpPtr> pos, std::vector<OpPtr> neg, bool exact) {
   if (OpPtr tmp = nof_trivial(n, pos, neg, exact)) return tmp;
   const int k = static_cast<int>(pos.size() + neg.size());
   if (n == k) {
      if (pos.empty()) return complement_of(union_of(std::move(neg)));
      return intersection_of(std::move(pos), std::move(neg));
   }
   if (n == 1 && !exact) {
      if (neg.empty()) return union_of(std::move(pos));
      return complement_of(intersection_of(std::move(neg), std::move(pos)));
   }
   return threshold_of(std::move(pos), std::move(neg), n, exact);
}

}  // namespace

OpPtr negate(OpPtr op) {
   switch (op->t) {
      case OpT::EMPTY: return mk(OpT::FULL);
      case OpT::FULL: return mk(OpT::EMPTY);
      case OpT::COMPLEMENT: return std::move(op->children[0]);
      case OpT::SELECTION:
         if (op->children.empty() && op->preds.size() == 1) return selection_of(nullptr, {op->preds[0].negated()});
         return complement_of(std::move(op));
      default: return complement_of(std::move(op));
   }
}

namespace {

// The aligned sequence of the row whose primary key is `id`: the first row holding that value in
// the table's primary-key dictionary column. It is rebuilt from the row index: the local reference,
// overwritten by the row's own symbols, and the missing symbol wherever the row is not covered or
// lies in a missing interval, so a null row is missing everywhere (reference:
// mutation_profile.cpp:95-150, reconstructSequenceAtRow and buildProfileFromSequenceId).
std::vector<uint8_t> sequence_of_primary_key(const TableImage& t, const SeqColumnImage& col, const std::string& id) {
   const Alphabet& A = alphabet(col.kind);
   if (t.primary_key < 0 || static_cast<size_t>(t.primary_key) >= t.dict.size())
      throw IllegalQuery("MutationProfile sequenceId: the table has no primary key column");
   const DictColumnImage& pk = t.dict[t.primary_key];
   const auto it = pk.index.find(id);
   const ContainerSet& V = pk.inverted;
   uint32_t row = UINT32_MAX;
   if (it != pk.index.end() && it->second < V.nkeys) {
      for (uint32_t v = 0; v < t.nchunks() && row == UINT32_MAX; ++v) {
         const size_t k = static_cast<size_t>(v) * V.nkeys + it->second;
         uint32_t first = UINT32_MAX;
         for (uint32_t i = V.off[k]; i < V.off[k + 1]; ++i) {
            const CtrDesc& d = V.ctrs[i];
            const uint16_t* p = V.payload.data() + d.payload;
            uint32_t m = UINT32_MAX;
            if (d.type == CT_ARRAY || d.type == CT_RUN) {
               m = p[0];  // arrays ascend; runs are (start, length - 1) pairs in order
            } else {
               for (uint32_t w = 0; w < CHUNK_WORDS && m == UINT32_MAX; ++w) {
                  const uint32_t x = static_cast<uint32_t>(p[2 * w]) | static_cast<uint32_t>(p[2 * w + 1]) << 16;
                  if (x) m = 32 * w + static_cast<uint32_t>(__builtin_ctz(x));
               }
            }
            first = std::min(first, m);
         }
         if (first != UINT32_MAX) row = v * CHUNK_ROWS + first;
      }
   }
   if (row == UINT32_MAX)
      throw IllegalQuery("No sequence found with primary key '" + id + "' in " +
                         (col.kind == SymKind::NUC ? "Nucleotide" : "AminoAcid") + " MutationProfile");
   std::vector<uint8_t> seq = col.local_ref;
   std::vector<uint8_t> missing(col.L, 0);
   uint32_t start = 0, end = col.L, miss_a = 0;
   for (uint32_t i = col.hrow_off[row]; i < col.hrow_off[row + 1]; ++i) {
      const uint32_t code = col.hent[i] & 31u, p = col.hent[i] >> 5;
      if (code < ROW_COV_START) seq[p] = static_cast<uint8_t>(code);
      else if (code == ROW_COV_START) start = p;
      else if (code == ROW_COV_END) end = p;
      else if (code == ROW_MISS_START) miss_a = p;
      else std::fill(missing.begin() + miss_a, missing.begin() + p, 1);
   }
   for (uint32_t p = 0; p < col.L; ++p)
      if (p < start || p >= end || missing[p]) seq[p] = static_cast<uint8_t>(A.missing);
   return seq;
}

// The profile (query sequence, or the reference with the mutations applied), the symbols that
// differ from it at each position (every symbol not in AMBIGUITY_SYMBOLS of the profile's symbol;
// none where the profile holds the missing symbol) and the per-row counting terms
// (reference: mutation_profile.cpp:62-89, 160-196, 198-257).
OpPtr compile_profile(const TableImage& t, const Expr& e) {
   const int ci = t.find_seq(e.column);
   if (ci < 0) throw IllegalQuery("the database does not contain the sequence column '" + e.column + "'");
   const SeqColumnImage& col = t.seq[ci];
   const Alphabet& A = alphabet(col.kind);
   const uint32_t L = col.L;
   std::vector<uint8_t> profile;
   if (e.by_id) {
      profile = sequence_of_primary_key(t, col, e.value);
   } else if (!e.value.empty()) {
      if (e.value.size() != L)
         throw IllegalQuery("querySequence length " + std::to_string(e.value.size()) +
                            " does not match the reference sequence length " + std::to_string(L));
      profile.resize(L);
      for (uint32_t p = 0; p < L; ++p) {
         const int sy = A.sym(e.value[p]);
         if (sy < 0) throw IllegalQuery(std::string("Invalid symbol '") + e.value[p] + "' in querySequence for MutationProfile");
         profile[p] = static_cast<uint8_t>(sy);
      }
   } else {
      profile = col.global_ref;
      for (uint32_t m : e.muts) {
         if ((m >> 8) >= L)
            throw IllegalQuery("MutationProfile mutation position " + std::to_string((m >> 8) + 1) +
                               " is out of bounds (reference length " + std::to_string(L) + ")");
         profile[m >> 8] = static_cast<uint8_t>(m & 0xFFu);
      }
   }
   auto spec = std::make_shared<ProfileSpec>();
   spec->col = ci;
   spec->distance = static_cast<uint32_t>(e.n);
   spec->mask.resize(L);
   spec->diff.assign(L + 1, 0);
   uint32_t loc = 0;
   for (uint32_t p = 0; p < L; ++p) {
      const uint32_t m = profile[p] == A.missing ? 0u : A.all_mask & ~A.ambiguity[profile[p]];
      const uint32_t lbit = (m >> col.local_ref[p]) & 1u;
      spec->mask[p] = m | lbit << 31;
      spec->diff[p + 1] = spec->diff[p] + ((m >> A.missing) & 1u) - lbit;
      loc += lbit;
   }
   spec->base = loc;
   auto o = mk(OpT::PROFILE);
   o->profile = std::move(spec);
   return o;
}

}  // namespace

OpPtr compile(const Expr& e, const TableImage& t) {
   switch (e.kind) {
      case EK::AND: {
         // reference: and.cpp:91-219
         std::vector<OpPtr> unprocessed, pos, neg;
         std::vector<Pred> preds;
         for (const auto& c : e.children) unprocessed.push_back(compile(*c, t));
         while (!unprocessed.empty()) {
            OpPtr child = std::move(unprocessed.back());
            unprocessed.pop_back();
            if (child->t == OpT::FULL) continue;
            if (child->t == OpT::EMPTY) return mk(OpT::EMPTY);
            if (child->t == OpT::INTERSECTION) {
               for (auto& g : child->children) pos.push_back(std::move(g));
               for (auto& g : child->negated) neg.push_back(std::move(g));
            } else if (child->t == OpT::COMPLEMENT) {
               neg.push_back(negate(std::move(child)));
            } else if (child->t == OpT::SELECTION) {
               for (const auto& p : child->preds) preds.push_back(p);
               if (!child->children.empty()) unprocessed.push_back(std::move(child->children[0]));
            } else {
               pos.push_back(std::move(child));
            }
         }
         if (pos.empty() && neg.empty()) {
            if (preds.empty()) return mk(OpT::FULL);
            return selection_of(nullptr, std::move(preds));
         }
         OpPtr op;
         if (pos.size() == 1 && neg.empty()) {
            op = std::move(pos[0]);
         } else if (neg.size() == 1 && pos.empty()) {
            op = complement_of(std::move(neg[0]));
         } else if (pos.empty()) {
            op = complement_of(union_of(std::move(neg)));
         } else {
            op = intersection_of(std::move(pos), std::move(neg));
         }
         if (preds.empty()) return op;
         return selection_of(std::move(op), std::move(preds));
      }
      case EK::OR: {
         // reference: or.cpp:194-241
         std::vector<OpPtr> filtered;
         for (const auto& c : e.children) {
            OpPtr child = compile(*c, t);
            if (child->t == OpT::EMPTY) continue;
            if (child->t == OpT::FULL) return mk(OpT::FULL);
            if (child->t == OpT::UNION) {
               for (auto& g : child->children) filtered.push_back(std::move(g));
            } else {
               filtered.push_back(std::move(child));
            }
         }
         if (filtered.empty()) return mk(OpT::EMPTY);
         if (filtered.size() == 1) return std::move(filtered[0]);
         const bool any_complement =
            std::any_of(filtered.begin(), filtered.end(), [](const OpPtr& o) { return o->t == OpT::COMPLEMENT; });
         if (any_complement) {
            // Complement::fromDeMorgan (complement.cpp:23-39)
            std::vector<OpPtr> pos, neg;
            for (auto& c : filtered) {
               if (c->t == OpT::COMPLEMENT) {
                  neg.push_back(negate(std::move(c)));
               } else {
                  pos.push_back(std::move(c));
               }
            }
            return complement_of(intersection_of(std::move(neg), std::move(pos)));
         }
         return union_of(std::move(filtered));
      }
      case EK::NOT: return negate(compile(*e.children[0], t));
      case EK::NOF: {
         // reference: nof.cpp:183-215, 259-277
         std::vector<OpPtr> pos, neg;
         int n = e.n;
         for (const auto& c : e.children) {
            OpPtr child = compile(*c, t);
            if (child->t == OpT::EMPTY) continue;
            if (child->t == OpT::FULL) {
               --n;
               continue;
            }
            if (child->t == OpT::COMPLEMENT) {
               neg.push_back(negate(std::move(child)));
               continue;
            }
            pos.push_back(std::move(child));
         }
         if (n < 0) return e.exact ? mk(OpT::EMPTY) : mk(OpT::FULL);
         return nof_to_operator(n, std::move(pos), std::move(neg), e.exact);
      }
      case EK::SYM_IN_SET: return compile_symbol_in_set(t, e);
      case EK::STR_EQ: {
         // reference: equals.cpp:174-187 (indexed string column -> IndexScan of the inverted index)
         const int ci = t.find_dict(e.column);
         if (ci < 0) throw IllegalQuery("the database does not contain the indexed string column '" + e.column + "'");
         const DictColumnImage& d = t.dict[ci];
         auto it = d.index.find(e.value);
         if (it == d.index.end()) return mk(OpT::EMPTY);
         bool any = false;
         for (uint32_t v = 0; v < t.nchunks() && !any; ++v) {
            const size_t slot = static_cast<size_t>(v) * d.inverted.nkeys + it->second;
            any = d.inverted.off[slot + 1] > d.inverted.off[slot];
         }
         if (!any) return mk(OpT::EMPTY);
         Leaf l;
         l.kind = Leaf::DICT;
         l.col = ci;
         l.value = it->second;
         return scan_of(l);
      }
      case EK::DATE_BETWEEN: {
         // reference: date_between.cpp:61-89 (unsorted column -> Selection with two comparisons)
         const int ci = t.find_date(e.column);
         if (ci < 0) throw IllegalQuery("the database does not contain the date column '" + e.column + "'");
         Pred lo, hi;
         lo.kind = hi.kind = Pred::DATE;
         lo.col = hi.col = ci;
         lo.cmp = CMP_GE;
         lo.value = e.has_from ? e.from : INT32_MIN;
         hi.cmp = CMP_LE;
         hi.value = e.has_to ? e.to : INT32_MAX;
         return selection_of(nullptr, {lo, hi});
      }
      case EK::BOOL: return mk(e.truth ? OpT::FULL : OpT::EMPTY);
      case EK::MUT_PROFILE: return compile_profile(t, e);
      case EK::SYM_EQ: throw CompilationError("SymbolEquals should have been rewritten before compilation");
      case EK::HAS_MUT: throw CompilationError("HasMutation expression must be eliminated in query rewrite phase");
      case EK::MAYBE: throw CompilationError("Maybe expression must be elimitated in query rewrite phase");
      case EK::EXACT: throw CompilationError("Exact expression must be elimitated in query rewrite phase");
   }
   throw CompilationError("unknown expression kind");
}

std::string Op::to_string() const {
   auto list = [](const std::vector<OpPtr>& v) {
      std::string s;
      for (size_t i = 0; i < v.size(); ++i) {
         if (i) s += ",";
         s += v[i]->to_string();
      }
      return s;
   };
   switch (t) {
      case OpT::EMPTY: return "Empty";
      case OpT::FULL: return "Full";
      case OpT::INDEX_SCAN:
         if (leaf.kind == Leaf::SEQ) return "Scan(" + std::to_string(leaf.col) + "," + std::to_string(leaf.pos + 1) + ",0x" + [&] {
                   char b[16];
                   std::snprintf(b, sizeof b, "%x", leaf.symmask);
                   return std::string(b);
                }() + ")";
         if (leaf.kind == Leaf::NULLS) return "Nulls(" + std::to_string(leaf.col) + ")";
         return "Dict(" + std::to_string(leaf.col) + "," + std::to_string(leaf.value) + ")";
      case OpT::INTERSECTION: return "Intersection(" + list(children) + ";not:" + list(negated) + ")";
      case OpT::UNION: return "Union(" + list(children) + ")";
      case OpT::COMPLEMENT: return "!" + children[0]->to_string();
      case OpT::THRESHOLD:
         return std::string("Threshold(") + (exact ? "=" : ">=") + std::to_string(n) + ";" + list(children) + ";not:" + list(negated) + ")";
      case OpT::SELECTION: {
         std::string s = "Select[";
         for (size_t i = 0; i < preds.size(); ++i) {
            if (i) s += ",";
            const Pred& p = preds[i];
            if (p.kind == Pred::COVERED) {
               s += std::string(p.covered ? "" : "!") + "Covered(" + std::to_string(p.pos + 1) + ")";
            } else {
               s += "Date(" + std::to_string(p.cmp) + "," + std::to_string(p.value) + (p.with_nulls ? ",nulls" : "") + ")";
            }
         }
         return s + "](" + list(children) + ")";
      }
      case OpT::PROFILE:
         return "Profile(" + std::to_string(profile->col) + ",<=" + std::to_string(profile->distance) + ")";
      case OpT::ROWS: return "Rows(" + std::to_string(rows_index) + ")";
   }
   return "?";
}

// =============================================================================================
// Estimation (rule based): container cardinalities for leaves, independence for combinations.

double rule_node_estimate(const Op& op, const TableImage& t, const std::function<double(const Op&)>& child) {
   const double rows = std::max(1u, t.n_rows);
   auto frac = [rows](double x) { return std::min(1.0, std::max(0.0, x / rows)); };
   switch (op.t) {
      case OpT::EMPTY: return 0.0;
      case OpT::FULL: return rows;
      case OpT::INDEX_SCAN: {
         // exact: the containers of the symbols of one key are disjoint
         if (op.leaf.kind == Leaf::NULLS) return static_cast<double>(t.seq[op.leaf.col].null_rows.size());
         if (op.leaf.kind == Leaf::DICT) return t.dict[op.leaf.col].inverted.stat(op.leaf.value, 0).card;
         const ContainerSet& cs = t.seq[op.leaf.col].vertical;
         double s = 0;
         for (uint32_t m = op.leaf.symmask; m; m &= m - 1) s += cs.stat(op.leaf.pos, __builtin_ctz(m)).card;
         return s;
      }
      case OpT::COMPLEMENT: return rows - child(*op.children[0]);
      case OpT::INTERSECTION: {
         double f = 1;
         for (const auto& c : op.children) f *= frac(child(*c));
         for (const auto& c : op.negated) f *= 1 - frac(child(*c));
         return f * rows;
      }
      case OpT::UNION: {
         double f = 1;
         for (const auto& c : op.children) f *= 1 - frac(child(*c));
         return (1 - f) * rows;
      }
      case OpT::SELECTION: {
         double f = op.children.empty() ? 1.0 : frac(child(*op.children[0]));
         for (const auto& p : op.preds) {
            if (p.kind == Pred::COVERED) {
               f *= p.covered ? 0.97 : 0.03;
            } else {
               f *= 0.5;
            }
         }
         return f * rows;
      }
      case OpT::PROFILE:
         // no statistics of the profile distances: an even chance
         return 0.5 * rows;
      case OpT::ROWS: return op.rows_card;
      case OpT::THRESHOLD: {
         // Poisson-binomial distribution of the number of matching children.
         std::vector<double> dist(1, 1.0);
         auto add = [&](double p) {
            std::vector<double> nd(dist.size() + 1, 0.0);
            for (size_t i = 0; i < dist.size(); ++i) {
               nd[i] += dist[i] * (1 - p);
               nd[i + 1] += dist[i] * p;
            }
            dist.swap(nd);
         };
         for (const auto& c : op.children) add(frac(child(*c)));
         for (const auto& c : op.negated) add(1 - frac(child(*c)));
         double f = 0;
         if (op.exact) {
            f = static_cast<size_t>(op.n) < dist.size() ? dist[op.n] : 0.0;
         } else {
            for (size_t i = op.n; i < dist.size(); ++i) f += dist[i];
         }
         return f * rows;
      }
   }
   return rows;
}

Estimator rule_estimator(const TableImage& t) {
   std::shared_ptr<std::function<double(const Op&)>> self = std::make_shared<std::function<double(const Op&)>>();
   *self = [&t, self](const Op& op) -> double { return rule_node_estimate(op, t, *self); };
   return [self](const Op& op) { return (*self)(op); };
}

// =============================================================================================
// Lowering

namespace {

struct Lowerer {
   const Estimator& est;
   const LowerOptions& opt;
   Program prog;
   uint32_t depth = 0;

   void emit(uint8_t op, uint8_t col = 0, uint16_t flags = 0, uint32_t a = 0, uint32_t b = 0, uint32_t c = 0) {
      if (prog.code.size() >= MAX_PROGRAM) throw IllegalQuery("filter program too large");
      prog.code.push_back(Instr{op, col, flags, a, b, c});
   }
   void push() {
      ++depth;
      prog.max_depth = std::max(prog.max_depth, depth);
   }
   void pop(uint32_t n = 1) { depth -= n; }

   // Estimated fraction of the table's rows in an operator's result (1 without the row count).
   double sel(const Op& o) const {
      if (opt.rows <= 0) return 1.0;
      return std::min(1.0, std::max(0.0, est(o) / opt.rows));
   }

   std::vector<const Op*> order(const std::vector<OpPtr>& v, bool ascending) {
      std::vector<std::pair<double, const Op*>> e;
      for (const auto& c : v) e.emplace_back(opt.reorder ? est(*c) : 0.0, c.get());
      if (opt.reorder) {
         std::stable_sort(e.begin(), e.end(), [ascending](const auto& x, const auto& y) {
            return ascending ? x.first < y.first : x.first > y.first;
         });
      }
      std::vector<const Op*> out;
      for (auto& x : e) out.push_back(x.second);
      return out;
   }

   // A date comparison as "inside [lo, hi]" (or outside it) plus whether null dates match.
   struct DateLeaf {
      int col;
      int32_t lo, hi;
      bool invert, with_nulls;
   };
   static DateLeaf date_leaf(const Pred& p) {
      DateLeaf d{p.col, p.value, p.value, false, p.with_nulls};
      switch (p.cmp) {
         case CMP_EQ: break;
         case CMP_NE: d.invert = true; break;
         case CMP_LT:
            d.lo = INT32_MIN;
            if (p.value == INT32_MIN) d.lo = 1, d.hi = 0;  // empty
            else d.hi = p.value - 1;
            break;
         case CMP_LE: d.lo = INT32_MIN; break;
         case CMP_GT:
            d.hi = INT32_MAX;
            if (p.value == INT32_MAX) d.lo = 1, d.hi = 0;
            else d.lo = p.value + 1;
            break;
         default: d.hi = INT32_MAX; break;  // CMP_GE
      }
      return d;
   }
   void date(const DateLeaf& d) {
      emit(OP_PUSH_DATE, static_cast<uint8_t>(d.col), static_cast<uint16_t>((d.with_nulls ? 1 : 0) | (d.invert ? 2 : 0)),
           static_cast<uint32_t>(d.lo), static_cast<uint32_t>(d.hi));
      push();
      ++prog.n_leaves;
   }

   void pred(const Pred& p) {
      if (p.kind == Pred::DATE) {
         date(date_leaf(p));
         return;
      }
      emit(OP_PUSH_COVERED, static_cast<uint8_t>(p.col), p.covered ? 0 : 1, p.pos, 0, ++prog.n_cov_leaves);
      push();
      ++prog.n_leaves;
   }

   // Emits a conditional jump whose target is patched once the node is complete.
   size_t jump(uint8_t op) {
      emit(op);
      return prog.code.size() - 1;
   }
   void patch(const std::vector<size_t>& jumps) {
      for (size_t j : jumps) prog.code[j].a = static_cast<uint32_t>(prog.code.size());
   }

   void node(const Op& op) {
      const uint32_t first = static_cast<uint32_t>(prog.code.size());
      node_body(op);
      if (opt.record_spans && prog.code.size() > first)
         prog.spans.push_back(NodeSpan{&op, first, static_cast<uint32_t>(prog.code.size() - 1)});
   }

   void node_body(const Op& op) {
      switch (op.t) {
         case OpT::EMPTY:
            emit(OP_PUSH_EMPTY);
            push();
            return;
         case OpT::FULL:
            emit(OP_PUSH_FULL);
            push();
            return;
         case OpT::INDEX_SCAN:
            if (op.leaf.kind == Leaf::SEQ) {
               emit(OP_PUSH_SCAN, static_cast<uint8_t>(op.leaf.col), 0, op.leaf.pos, op.leaf.symmask,
                    ++prog.n_ctr_leaves);
            } else if (op.leaf.kind == Leaf::NULLS) {
               emit(OP_PUSH_NULLS, static_cast<uint8_t>(op.leaf.col));
            } else {
               emit(OP_PUSH_DICT, static_cast<uint8_t>(op.leaf.col), 0, op.leaf.value, 0, ++prog.n_ctr_leaves);
            }
            push();
            ++prog.n_leaves;
            return;
         case OpT::COMPLEMENT:
            node(*op.children[0]);
            emit(OP_NOT);
            return;
         case OpT::INTERSECTION: {
            auto pos = order(op.children, true);
            auto neg = order(op.negated, false);
            std::vector<size_t> jumps;
            node(*pos[0]);
            double part = sel(*pos[0]);  // estimated selectivity of the partial result
            for (size_t i = 1; i < pos.size(); ++i) {
               if (opt.early_exit && (opt.rows <= 0 || part <= opt.exit_sel)) jumps.push_back(jump(OP_JZ));
               node(*pos[i]);
               emit(OP_AND);
               pop();
               part *= sel(*pos[i]);
            }
            for (const Op* c : neg) {
               if (opt.early_exit && (opt.rows <= 0 || part <= opt.exit_sel)) jumps.push_back(jump(OP_JZ));
               node(*c);
               emit(OP_ANDNOT);
               pop();
               part *= 1.0 - sel(*c);
            }
            patch(jumps);
            return;
         }
         case OpT::UNION: {
            if (op.children.empty()) {
               emit(OP_PUSH_EMPTY);
               push();
               return;
            }
            auto ch = order(op.children, false);
            std::vector<size_t> jumps;
            node(*ch[0]);
            double miss = 1.0 - sel(*ch[0]);  // estimated fraction of rows the partial union misses
            for (size_t i = 1; i < ch.size(); ++i) {
               if (opt.early_exit && (opt.rows <= 0 || miss <= opt.exit_sel)) jumps.push_back(jump(OP_JFULL));
               node(*ch[i]);
               emit(OP_OR);
               pop();
               miss *= 1.0 - sel(*ch[i]);
            }
            patch(jumps);
            return;
         }
         case OpT::SELECTION: {
            // The predicates are ANDed; date comparisons on one column that drop null dates merge
            // into a single range leaf (DateBetween's two comparisons become one pass).
            std::vector<DateLeaf> leaves;
            for (const Pred& p : op.preds) {
               if (p.kind != Pred::DATE) continue;
               DateLeaf d = date_leaf(p);
               bool merged = false;
               for (DateLeaf& x : leaves) {
                  if (!d.invert && !d.with_nulls && !x.invert && !x.with_nulls && x.col == d.col) {
                     x.lo = std::max(x.lo, d.lo);
                     x.hi = std::min(x.hi, d.hi);
                     merged = true;
                     break;
                  }
               }
               if (!merged) leaves.push_back(d);
            }
            std::vector<std::function<void()>> parts;
            for (const Pred& p : op.preds)
               if (p.kind == Pred::COVERED) parts.push_back([this, p] { pred(p); });
            for (const DateLeaf& d : leaves) parts.push_back([this, d] { date(d); });
            std::vector<size_t> jumps;
            size_t first = 0;
            if (!op.children.empty()) {
               node(*op.children[0]);
            } else {
               parts[0]();
               first = 1;
            }
            for (size_t i = first; i < parts.size(); ++i) {
               // the predicates are not estimated one by one: keep every test
               if (opt.early_exit) jumps.push_back(jump(OP_JZ));
               parts[i]();
               emit(OP_AND);
               pop();
            }
            patch(jumps);
            return;
         }
         case OpT::THRESHOLD: {
            uint32_t planes = 1;
            while ((1u << planes) - 1 < static_cast<uint32_t>(op.n) + 1) ++planes;
            if (planes > MAX_THR_PLANES) throw IllegalQuery("NOf threshold too large");
            emit(OP_THR_BEGIN, 0, 0, planes);
            for (uint32_t i = 0; i < planes; ++i) push();
            for (const auto& c : op.children) {
               node(*c);
               emit(OP_THR_ADD, 0, 0, planes);
               pop();
            }
            for (const auto& c : op.negated) {
               node(*c);
               emit(OP_THR_ADD, 0, 1, planes);
               pop();
            }
            emit(OP_THR_END, 0, op.exact ? 1 : 0, planes, static_cast<uint32_t>(op.n));
            pop(planes);
            push();
            return;
         }
         case OpT::PROFILE:
            emit(OP_PUSH_AUX, static_cast<uint8_t>(op.profile->col), 0, static_cast<uint32_t>(prog.aux.size()));
            prog.aux.push_back(op.profile);
            push();
            ++prog.n_leaves;
            return;
         case OpT::ROWS:
            // numbered after the profiles once lowering is done (see lower)
            emit(OP_PUSH_AUX, 0, AUX_LITERAL, op.rows_index);
            prog.n_literals = std::max(prog.n_literals, op.rows_index + 1);
            push();
            ++prog.n_leaves;
            return;
      }
   }
};

}  // namespace

Program lower(const Op& op, const Estimator& est, const LowerOptions& opt) {
   Lowerer l{est, opt, {}, 0};
   l.node(op);
   if (l.depth != 1) throw CompilationError("internal error: unbalanced filter program");
   // caller row sets follow the MutationProfile row sets in the aux area
   for (Instr& in : l.prog.code)
      if (in.op == OP_PUSH_AUX && (in.flags & AUX_LITERAL)) in.a += static_cast<uint32_t>(l.prog.aux.size());
   return std::move(l.prog);
}

OpPtr compile_filter(const std::string& text, const TableImage& t) {
   ExprPtr e = parse_expression(text, t);
   ExprPtr r = rewrite(*e, t, Ambiguity::NONE);
   return compile(*r, t);
}

Program plan_filter(const std::string& text, const TableImage& t, const Estimator* est, const LowerOptions& opt,
                    std::string* operator_tree) {
   ExprPtr e = parse_expression(text, t);
   ExprPtr r = rewrite(*e, t, Ambiguity::NONE);
   OpPtr op = compile(*r, t);
   if (operator_tree) *operator_tree = op->to_string();
   if (est) return lower(*op, *est, opt);
   const Estimator rule = rule_estimator(t);
   return lower(*op, rule, opt);
}

}  // namespace rhygpu
