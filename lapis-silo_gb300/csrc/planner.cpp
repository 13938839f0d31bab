// Learned planner: features, training loop and the judge against the rule-based estimator.
#include "planner.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <unordered_map>

#include "alphabet.h"

namespace rhygpu {

void cuda_check(cudaError_t e, const char* what);  // engine.cu

namespace {

struct SubStats {
   uint32_t nodes = 0, depth = 0, leaves = 0;
};

SubStats subtree(const Op& op) {
   SubStats s{1, 1, 0};
   if (op.t == OpT::INDEX_SCAN || op.t == OpT::PROFILE) s.leaves = 1;
   if (op.t == OpT::SELECTION) s.leaves += static_cast<uint32_t>(op.preds.size());
   auto add = [&](const OpPtr& c) {
      const SubStats x = subtree(*c);
      s.nodes += x.nodes;
      s.leaves += x.leaves;
      s.depth = std::max(s.depth, x.depth + 1);
   };
   for (const auto& c : op.children) add(c);
   for (const auto& c : op.negated) add(c);
   return s;
}

float log2p(double x) { return static_cast<float>(std::log2(1.0 + x)); }

constexpr double MIN_SEL = 1e-7;

// The rule estimate's ln(selectivity) as encoded in feature 8.
double rule_log_sel_of(const float* x) { return static_cast<double>(x[8]) * -std::log(MIN_SEL); }

}  // namespace

bool exact_by_rule(const float* x) { return x[0] > 0.5f || x[1] > 0.5f; }

FeatureContext feature_context(const TableImage& t) {
   FeatureContext c;
   c.table = &t;
   c.rule = rule_estimator(t);
   for (const auto& d : t.date) {
      int32_t lo = INT32_MAX, hi = INT32_MIN;
      for (int32_t x : d.days)
         if (x != INT32_MIN) lo = std::min(lo, x), hi = std::max(hi, x);
      if (lo > hi) lo = hi = 0;
      c.date_range.emplace_back(lo, hi);
   }
   return c;
}

namespace {

void op_features_with(const Op& op, const FeatureContext& ctx, double rule_rows, const SubStats& ss, float* f) {
   const TableImage& t = *ctx.table;
   std::fill(f, f + PLAN_FEATURES, 0.0f);
   const double rows = std::max(1u, t.n_rows);
   switch (op.t) {
      case OpT::INDEX_SCAN: f[op.leaf.kind == Leaf::SEQ ? 0 : 1] = 1; break;
      case OpT::SELECTION: f[2] = 1; break;
      case OpT::INTERSECTION: f[3] = 1; break;
      case OpT::UNION: f[4] = 1; break;
      case OpT::COMPLEMENT: f[5] = 1; break;
      case OpT::THRESHOLD: f[6] = 1; break;
      default: f[7] = 1; break;
   }
   const double sel = std::min(1.0, std::max(0.0, rule_rows / rows));
   f[8] = static_cast<float>(std::log(std::max(sel, MIN_SEL)) / -std::log(MIN_SEL));
   f[9] = static_cast<float>(sel);
   const size_t nch = op.children.size() + op.negated.size();
   f[10] = log2p(static_cast<double>(nch)) / 6.0f;
   f[11] = nch ? static_cast<float>(op.negated.size()) / static_cast<float>(nch) : 0.0f;
   f[12] = log2p(ss.nodes) / 8.0f;
   f[13] = static_cast<float>(ss.depth) / 8.0f;
   f[14] = log2p(ss.leaves) / 8.0f;
   if (op.t == OpT::INDEX_SCAN && op.leaf.kind == Leaf::SEQ) {
      const SeqColumnImage& c = t.seq[op.leaf.col];
      const Alphabet& A = alphabet(c.kind);
      f[15] = static_cast<float>(__builtin_popcount(op.leaf.symmask)) / static_cast<float>(A.count);
      f[16] = static_cast<float>(op.leaf.pos) / static_cast<float>(std::max(1u, c.L));
      f[17] = c.kind == SymKind::AA ? 1.0f : 0.0f;
      uint32_t n = 0, nb = 0;
      for (uint32_t m = op.leaf.symmask; m; m &= m - 1) {
         const KeyStats& st = c.vertical.stat(op.leaf.pos, __builtin_ctz(m));
         n += st.nctr;
         nb += st.nbits;
      }
      f[18] = log2p(n) / 12.0f;
      f[19] = n ? static_cast<float>(nb) / static_cast<float>(n) : 0.0f;
   } else if (op.t == OpT::INDEX_SCAN && op.leaf.kind == Leaf::DICT) {
      const KeyStats& st = t.dict[op.leaf.col].inverted.stat(op.leaf.value, 0);
      f[18] = log2p(st.nctr) / 12.0f;
      f[19] = st.nctr ? static_cast<float>(st.nbits) / static_cast<float>(st.nctr) : 0.0f;
   } else if (op.t == OpT::SELECTION) {
      uint32_t ncov = 0;
      double width = 1.0;
      bool any_date = false;
      for (const Pred& p : op.preds) {
         if (p.kind == Pred::COVERED) {
            if (ncov == 0) {
               const SeqColumnImage& c = t.seq[p.col];
               f[16] = static_cast<float>(p.pos) / static_cast<float>(std::max(1u, c.L));
               f[17] = c.kind == SymKind::AA ? 1.0f : 0.0f;
            }
            ++ncov;
            continue;
         }
         any_date = true;
         const auto [lo, hi] = ctx.date_range[p.col];
         const double span = static_cast<double>(hi) - lo + 1.0;
         const double x = (static_cast<double>(p.value) - lo + 0.5) / span;  // position of the bound
         double w;
         switch (p.cmp) {
            case CMP_EQ: w = 1.0 / span; break;
            case CMP_NE: w = 1.0 - 1.0 / span; break;
            case CMP_LT:
            case CMP_LE: w = x; break;
            default: w = 1.0 - x; break;
         }
         width *= std::min(1.0, std::max(0.0, w));
      }
      f[20] = static_cast<float>(ncov) / 4.0f;
      f[21] = any_date ? static_cast<float>(width) : 1.0f;
      f[23] = op.children.empty() ? 0.0f : 1.0f;
   } else if (op.t == OpT::THRESHOLD) {
      f[22] = nch ? static_cast<float>(op.n) / static_cast<float>(nch) : 0.0f;
      f[23] = op.exact ? 1.0f : 0.0f;
   }
}

}  // namespace

void op_features(const Op& op, const FeatureContext& ctx, float* out) {
   op_features_with(op, ctx, ctx.rule(op), subtree(op), out);
}

void tree_features(const Op& root, const FeatureContext& ctx, std::vector<const Op*>& nodes,
                   std::vector<std::array<float, PLAN_FEATURES>>& x) {
   // rule estimates and subtree statistics once per node, bottom up
   std::unordered_map<const Op*, std::pair<double, SubStats>> memo;
   std::function<void(const Op&)> post = [&](const Op& op) {
      SubStats s{1, 1, 0};
      if (op.t == OpT::INDEX_SCAN || op.t == OpT::PROFILE) s.leaves = 1;
      if (op.t == OpT::SELECTION) s.leaves += static_cast<uint32_t>(op.preds.size());
      auto add = [&](const OpPtr& c) {
         post(*c);
         const SubStats& cs = memo.at(c.get()).second;
         s.nodes += cs.nodes;
         s.leaves += cs.leaves;
         s.depth = std::max(s.depth, cs.depth + 1);
      };
      for (const auto& c : op.children) add(c);
      for (const auto& c : op.negated) add(c);
      const double e = rule_node_estimate(op, *ctx.table, [&](const Op& c) { return memo.at(&c).first; });
      memo.emplace(&op, std::make_pair(e, s));
   };
   post(root);
   std::function<void(const Op&)> pre = [&](const Op& op) {
      const auto& m = memo.at(&op);
      nodes.push_back(&op);
      x.emplace_back();
      op_features_with(op, ctx, m.first, m.second, x.back().data());
      for (const auto& c : op.children) pre(*c);
      for (const auto& c : op.negated) pre(*c);
   };
   pre(root);
}

// ------------------------------------------------------------------------------------------------
// PlannerNet

PlannerNet::PlannerNet(int device) : device_(device) {}

PlannerNet::~PlannerNet() {
   cudaSetDevice(device_);
   for (void* p : {static_cast<void*>(d_master_), static_cast<void*>(d_m_), static_cast<void*>(d_v_),
                   static_cast<void*>(d_grad_), static_cast<void*>(d_loss_), static_cast<void*>(d_w_),
                   static_cast<void*>(d_X_), static_cast<void*>(d_T_), static_cast<void*>(d_Y_)})
      if (p) cudaFree(p);
   if (h_X_) cudaFreeHost(h_X_);
   if (h_Y_) cudaFreeHost(h_Y_);
   if (stream_) cudaStreamDestroy(stream_);
}

void PlannerNet::init(uint64_t seed) {
   std::mt19937_64 rng(seed);
   std::vector<float> w(MLP_NPARAM, 0.0f);
   auto fill = [&](uint32_t off, uint32_t out, uint32_t in) {
      std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / static_cast<float>(in)));
      for (uint32_t i = 0; i < out * in; ++i) w[off + i] = nd(rng);
   };
   fill(MLP_W1, MLP_H, MLP_IN);
   fill(MLP_W2, MLP_H, MLP_H);
   fill(MLP_W3, MLP_OUT, MLP_H);
   set_master(w.data());
}

void PlannerNet::reserve(uint32_t n) {
   cuda_check(cudaSetDevice(device_), "cudaSetDevice");
   if (!stream_) {  // high priority: inference during planning runs between the batch kernels' blocks
      int lo = 0, hi = 0;
      cuda_check(cudaDeviceGetStreamPriorityRange(&lo, &hi), "stream priorities");
      cuda_check(cudaStreamCreateWithPriority(&stream_, cudaStreamNonBlocking, hi), "stream");
   }
   if (!d_master_) {
      for (float** p : {&d_master_, &d_m_, &d_v_, &d_grad_})
         cuda_check(cudaMalloc(p, MLP_NPARAM * sizeof(float)), "cudaMalloc (planner)");
      cuda_check(cudaMalloc(&d_loss_, sizeof(float)), "cudaMalloc (planner)");
      cuda_check(cudaMalloc(&d_w_, MLP_NPARAM * sizeof(__nv_bfloat16)), "cudaMalloc (planner)");
   }
   if (n > cap_) {
      for (float* p : {d_X_, d_T_, d_Y_})
         if (p) cudaFree(p);
      const uint32_t c = std::max(n, 1024u);
      cuda_check(cudaMalloc(&d_X_, static_cast<size_t>(c) * MLP_IN * sizeof(float)), "cudaMalloc (planner)");
      cuda_check(cudaMalloc(&d_T_, static_cast<size_t>(c) * MLP_OUT * sizeof(float)), "cudaMalloc (planner)");
      cuda_check(cudaMalloc(&d_Y_, static_cast<size_t>(c) * MLP_OUT * sizeof(float)), "cudaMalloc (planner)");
      cap_ = c;
   }
}

void PlannerNet::set_master(const float* w) {
   reserve(0);
   cuda_check(cudaMemcpy(d_master_, w, MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice), "upload weights");
   cuda_check(cudaMemset(d_m_, 0, MLP_NPARAM * sizeof(float)), "memset");
   cuda_check(cudaMemset(d_v_, 0, MLP_NPARAM * sizeof(float)), "memset");
   cuda_check(cudaMemset(d_grad_, 0, MLP_NPARAM * sizeof(float)), "memset");
   cuda_check(mlp_cast(d_master_, d_w_, stream_), "cast weights");
   cuda_check(cudaStreamSynchronize(stream_), "cast weights");
   step_ = 0;
}

void PlannerNet::get_master(float* w) const {
   if (!d_master_) throw std::logic_error("planner network not initialised");
   cuda_check(cudaMemcpy(w, d_master_, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost), "download weights");
}

void PlannerNet::gradient(const float* X, const float* T, uint32_t n, float* grad, float* loss, float* Y) {
   if (!d_master_) throw std::logic_error("planner network not initialised");
   reserve(n);
   cudaStream_t s = stream_;
   cuda_check(cudaMemcpyAsync(d_X_, X, static_cast<size_t>(n) * MLP_IN * sizeof(float), cudaMemcpyHostToDevice, s), "H2D");
   cuda_check(cudaMemcpyAsync(d_T_, T, static_cast<size_t>(n) * MLP_OUT * sizeof(float), cudaMemcpyHostToDevice, s), "H2D");
   cuda_check(cudaMemsetAsync(d_grad_, 0, MLP_NPARAM * sizeof(float), s), "memset");
   cuda_check(cudaMemsetAsync(d_loss_, 0, sizeof(float), s), "memset");
   cuda_check(mlp_gradient(d_w_, d_X_, d_T_, n, d_grad_, d_loss_, s), "mlp gradient");
   if (Y) cuda_check(mlp_forward(d_w_, d_X_, n, d_Y_, s), "mlp forward");
   if (grad) cuda_check(cudaMemcpyAsync(grad, d_grad_, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
   if (loss) cuda_check(cudaMemcpyAsync(loss, d_loss_, sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
   if (Y) cuda_check(cudaMemcpyAsync(Y, d_Y_, static_cast<size_t>(n) * MLP_OUT * sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
   cuda_check(cudaStreamSynchronize(s), "mlp gradient");
   if (mlp_take_error() != 0) throw std::runtime_error("planner network: a bounded wait of the gradient kernel gave up");
   cuda_check(cudaMemsetAsync(d_grad_, 0, MLP_NPARAM * sizeof(float), s), "memset");
   cuda_check(cudaStreamSynchronize(s), "mlp gradient");
}

float PlannerNet::train(const std::vector<float>& X, const std::vector<float>& T, uint32_t n, uint32_t epochs,
                        uint32_t batch, float lr, uint64_t seed) {
   if (!d_master_) throw std::logic_error("planner network not initialised");
   if (n == 0) return 0.0f;
   batch = std::max(64u, std::min(batch, n));
   reserve(n);
   cudaStream_t s = stream_;
   // one shuffled copy per epoch, uploaded whole; minibatches are contiguous slices of it
   std::vector<uint32_t> perm(n);
   std::iota(perm.begin(), perm.end(), 0u);
   std::mt19937_64 rng(seed);
   std::vector<float> Xs(static_cast<size_t>(n) * MLP_IN), Ts(static_cast<size_t>(n) * MLP_OUT);
   float last = 0.0f;
   for (uint32_t e = 0; e < epochs; ++e) {
      std::shuffle(perm.begin(), perm.end(), rng);
      for (uint32_t i = 0; i < n; ++i) {
         std::copy_n(&X[static_cast<size_t>(perm[i]) * MLP_IN], MLP_IN, &Xs[static_cast<size_t>(i) * MLP_IN]);
         std::copy_n(&T[static_cast<size_t>(perm[i]) * MLP_OUT], MLP_OUT, &Ts[static_cast<size_t>(i) * MLP_OUT]);
      }
      cuda_check(cudaMemcpyAsync(d_X_, Xs.data(), Xs.size() * sizeof(float), cudaMemcpyHostToDevice, s), "H2D");
      cuda_check(cudaMemcpyAsync(d_T_, Ts.data(), Ts.size() * sizeof(float), cudaMemcpyHostToDevice, s), "H2D");
      cuda_check(cudaMemsetAsync(d_loss_, 0, sizeof(float), s), "memset");
      uint32_t nb = 0;
      for (uint32_t b = 0; b + batch <= n || (b < n && nb == 0); b += batch, ++nb) {
         const uint32_t m = std::min(batch, n - b);
         cuda_check(mlp_gradient(d_w_, d_X_ + static_cast<size_t>(b) * MLP_IN, d_T_ + static_cast<size_t>(b) * MLP_OUT, m,
                                 d_grad_, d_loss_, s),
                    "mlp gradient");
         cuda_check(mlp_adam(d_master_, d_w_, d_grad_, d_m_, d_v_, lr, ++step_, s), "adam");
      }
      float loss = 0.0f;
      cuda_check(cudaMemcpyAsync(&loss, d_loss_, sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
      cuda_check(cudaStreamSynchronize(s), "train epoch");
      if (mlp_take_error() != 0) throw std::runtime_error("planner network: a bounded wait of the gradient kernel gave up");
      last = loss / static_cast<float>(std::max(1u, nb));
   }
   return last;
}

void PlannerNet::predict(const float* X, uint32_t n, float* Y) {
   if (!d_master_) throw std::logic_error("planner network not initialised");
   if (n == 0) return;
   reserve(n);
   cudaStream_t s = stream_;
   cuda_check(cudaMemcpyAsync(d_X_, X, static_cast<size_t>(n) * MLP_IN * sizeof(float), cudaMemcpyHostToDevice, s), "H2D");
   cuda_check(mlp_forward(d_w_, d_X_, n, d_Y_, s), "mlp forward");
   cuda_check(cudaMemcpyAsync(Y, d_Y_, static_cast<size_t>(n) * MLP_OUT * sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
   cuda_check(cudaStreamSynchronize(s), "mlp forward");
}

float* PlannerNet::staged_input(uint32_t n) {
   reserve(n);
   if (n > hcap_) {
      if (h_X_) cudaFreeHost(h_X_);
      if (h_Y_) cudaFreeHost(h_Y_);
      h_X_ = h_Y_ = nullptr;
      hcap_ = 0;
      const uint32_t c = std::max(n + n / 4, 1024u);
      cuda_check(cudaMallocHost(&h_X_, static_cast<size_t>(c) * MLP_IN * sizeof(float)), "cudaMallocHost (planner)");
      cuda_check(cudaMallocHost(&h_Y_, static_cast<size_t>(c) * MLP_OUT * sizeof(float)), "cudaMallocHost (planner)");
      hcap_ = c;
   }
   return h_X_;
}

const float* PlannerNet::predict_staged(uint32_t n) {
   if (n > hcap_) throw std::logic_error("planner: staged rows exceed the staging buffer");
   predict(h_X_, n, h_Y_);
   return h_Y_;
}

// ------------------------------------------------------------------------------------------------
// Planner

namespace {
// output 0: residual of the rule estimate, ln(measured / rule); output 1: ln cycles per tile
double target_of(const PlannerSample& sm, int k) {
   return k ? sm.log_cost : static_cast<double>(sm.log_sel) - rule_log_sel_of(sm.x.data());
}
}  // namespace

void Planner::judge(const std::vector<const PlannerSample*>& set, const float* Y, PlannerStats& st) const {
   std::vector<float> ql, qr, ce;
   for (size_t i = 0; i < set.size(); ++i) {
      const PlannerSample& sm = *set[i];
      const double rl = rule_log_sel_of(sm.x.data());
      const double ls = exact_by_rule(sm.x.data()) ? rl : rl + static_cast<double>(Y[2 * i]) * tstd[0] + tmean[0];
      const double lc = static_cast<double>(Y[2 * i + 1]) * tstd[1] + tmean[1];
      const double truth = sm.log_sel;
      ql.push_back(static_cast<float>(std::exp(std::fabs(std::max(std::log(MIN_SEL), std::min(0.0, ls)) - truth))));
      qr.push_back(static_cast<float>(std::exp(std::fabs(sm.rule_log_sel - truth))));
      ce.push_back(static_cast<float>(std::fabs(lc - sm.log_cost)));
   }
   auto pct = [](std::vector<float> v, double q) {
      if (v.empty()) return std::nanf("");
      std::sort(v.begin(), v.end());
      return v[static_cast<size_t>(q * (v.size() - 1))];
   };
   st.qerr_learned_median = pct(ql, 0.5);
   st.qerr_rule_median = pct(qr, 0.5);
   st.qerr_learned_p90 = pct(ql, 0.9);
   st.qerr_rule_p90 = pct(qr, 0.9);
   st.cost_err_median = pct(ce, 0.5);
   // the judge: not worse than the rule at the median (index scans are exact for both, so ties
   // there are common) and not worse at the 90th percentile
   st.accepted = !set.empty() && std::isfinite(st.val_loss) &&
                       st.qerr_learned_median <= st.qerr_rule_median * (1.0f + 1e-4f) &&
                       st.qerr_learned_p90 <= st.qerr_rule_p90 * (1.0f + 1e-4f)
                    ? 1
                    : 0;
}

PlannerStats Planner::evaluate(const std::vector<PlannerSample>& set) {
   if (!trained) throw std::invalid_argument("the planner network is not trained");
   PlannerStats st{};
   st.n_val = static_cast<uint32_t>(set.size());
   const uint32_t n = st.n_val;
   std::vector<float> X(static_cast<size_t>(n) * PLAN_FEATURES), Y(static_cast<size_t>(n) * 2);
   std::vector<const PlannerSample*> ptrs(n);
   double loss = 0;
   for (uint32_t i = 0; i < n; ++i) {
      ptrs[i] = &set[i];
      normalize(set[i].x.data(), X.data() + static_cast<size_t>(i) * PLAN_FEATURES);
   }
   if (n) net.predict(X.data(), n, Y.data());
   for (uint32_t i = 0; i < n; ++i)
      for (int k = 0; k < 2; ++k) {
         const double t = (target_of(set[i], k) - tmean[k]) / tstd[k];
         loss += (Y[2 * i + k] - t) * (Y[2 * i + k] - t);
      }
   st.val_loss = n ? static_cast<float>(loss / n) : std::nanf("");
   judge(ptrs, Y.data(), st);
   return st;
}

PlannerStats Planner::train(uint32_t epochs, uint32_t batch, float lr, uint64_t seed) {
   const auto t0 = std::chrono::steady_clock::now();
   const uint32_t n = static_cast<uint32_t>(samples.size());
   if (n < 16) throw std::invalid_argument("planner: " + std::to_string(n) + " samples are too few to train on");
   std::vector<uint32_t> idx(n);
   std::iota(idx.begin(), idx.end(), 0u);
   std::mt19937_64 rng(seed ^ 0x9E3779B97F4A7C15ull);
   std::shuffle(idx.begin(), idx.end(), rng);
   const uint32_t n_val = std::max(1u, n / 5), n_tr = n - n_val;
   // normalisation from the training split
   for (uint32_t k = 0; k < PLAN_FEATURES; ++k) {
      double m = 0, v = 0;
      for (uint32_t i = 0; i < n_tr; ++i) m += samples[idx[i]].x[k];
      m /= n_tr;
      for (uint32_t i = 0; i < n_tr; ++i) v += (samples[idx[i]].x[k] - m) * (samples[idx[i]].x[k] - m);
      fmean[k] = static_cast<float>(m);
      fstd[k] = static_cast<float>(std::max(std::sqrt(v / n_tr), 1e-3));
   }
   auto target = target_of;
   for (int k = 0; k < 2; ++k) {
      double m = 0, v = 0;
      for (uint32_t i = 0; i < n_tr; ++i) m += target(samples[idx[i]], k);
      m /= n_tr;
      for (uint32_t i = 0; i < n_tr; ++i) {
         const double y = target(samples[idx[i]], k);
         v += (y - m) * (y - m);
      }
      tmean[k] = static_cast<float>(m);
      tstd[k] = static_cast<float>(std::max(std::sqrt(v / n_tr), 1e-3));
   }
   auto pack = [&](uint32_t b, uint32_t e, std::vector<float>& X, std::vector<float>& T) {
      X.resize(static_cast<size_t>(e - b) * PLAN_FEATURES);
      T.resize(static_cast<size_t>(e - b) * 2);
      for (uint32_t i = b; i < e; ++i) {
         const PlannerSample& sm = samples[idx[i]];
         for (uint32_t k = 0; k < PLAN_FEATURES; ++k)
            X[static_cast<size_t>(i - b) * PLAN_FEATURES + k] = (sm.x[k] - fmean[k]) / fstd[k];
         T[static_cast<size_t>(i - b) * 2] = static_cast<float>((target(sm, 0) - tmean[0]) / tstd[0]);
         T[static_cast<size_t>(i - b) * 2 + 1] = static_cast<float>((target(sm, 1) - tmean[1]) / tstd[1]);
      }
   };
   std::vector<float> Xtr, Ttr, Xva, Tva;
   pack(0, n_tr, Xtr, Ttr);
   pack(n_tr, n, Xva, Tva);
   net.init(seed);
   PlannerStats st{};
   st.n_train = n_tr;
   st.n_val = n_val;
   st.epochs = epochs;
   st.train_loss = net.train(Xtr, Ttr, n_tr, epochs, batch, lr, seed);
   // judge on the held-out split
   float vloss = 0.0f;
   std::vector<float> Y(static_cast<size_t>(n_val) * 2);
   net.gradient(Xva.data(), Tva.data(), n_val, nullptr, &vloss, Y.data());
   st.val_loss = vloss;
   std::vector<const PlannerSample*> val(n_val);
   for (uint32_t i = 0; i < n_val; ++i) val[i] = &samples[idx[n_tr + i]];
   judge(val, Y.data(), st);
   trained = true;
   accepted = st.accepted != 0;
   st.train_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
   return st;
}

void Planner::predict(const std::vector<std::array<float, PLAN_FEATURES>>& x, std::vector<double>& sel,
                      std::vector<double>& cost) {
   const uint32_t n = static_cast<uint32_t>(x.size());
   sel.assign(n, std::nan(""));
   cost.assign(n, std::nan(""));
   if (!trained || n == 0) return;
   std::vector<float> X(static_cast<size_t>(n) * PLAN_FEATURES), Y(static_cast<size_t>(n) * 2);
   for (uint32_t i = 0; i < n; ++i) normalize(x[i].data(), X.data() + static_cast<size_t>(i) * PLAN_FEATURES);
   net.predict(X.data(), n, Y.data());
   for (uint32_t i = 0; i < n; ++i) {
      sel[i] = selectivity_of(x[i].data(), Y.data() + 2 * i);
      cost[i] = cost_of(Y.data() + 2 * i);
   }
}

void Planner::normalize(const float* x, float* out) const {
   for (uint32_t k = 0; k < PLAN_FEATURES; ++k) out[k] = (x[k] - fmean[k]) / fstd[k];
}

double Planner::selectivity_of(const float* x, const float* y) const {
   const double rl = rule_log_sel_of(x);
   const double ls = exact_by_rule(x) ? rl : rl + static_cast<double>(y[0]) * tstd[0] + tmean[0];
   return std::exp(std::max(std::log(MIN_SEL), std::min(0.0, ls)));
}

double Planner::cost_of(const float* y) const { return std::exp(static_cast<double>(y[1]) * tstd[1] + tmean[1]); }

}  // namespace rhygpu
