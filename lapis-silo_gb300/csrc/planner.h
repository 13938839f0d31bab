// Learned planner: per-operator selectivity and cost predicted by a small network from the operator
// tree and the table's container statistics, trained on execution traces of the single-query path.
//
// A training sample is one operator node of a traced query: the node's features (op_features), the
// natural log of its result's fraction of the rows and of its subtree's cycles per tile, both
// measured by the trace mode of the filter kernel on a program lowered without early exits. The
// network (mlp.h) is trained on the GPU by the project's own kernels to predict the cost and the
// residual ln(measured / rule estimate) of the selectivity; index scans keep the rule estimate,
// which is their exact cardinality. A held-out split judges the result against the rule-based
// estimator (the planner is accepted only if neither its median nor its 90th-percentile q-error of
// the selectivity is worse), and every prediction that is not finite falls back to the rule.
// The planner orders And / Or / NOf children and the work items of a batch; it never changes a
// result.
#pragma once

#include <array>
#include <cstdint>
#include <vector>

#include <cuda_bf16.h>

#include "expr.h"
#include "mlp.h"
#include "table.h"

namespace rhygpu {

// Whether a node (by its features) is an index scan (features 0 / 1), whose rule estimate is its
// exact cardinality: the containers of the symbols of one position are disjoint, so their
// cardinalities add up to the rows. The network's selectivity is not used for such nodes.
bool exact_by_rule(const float* x);

constexpr uint32_t PLAN_FEATURES = MLP_IN;

// Table statistics the features are relative to.
struct FeatureContext {
   const TableImage* table = nullptr;
   Estimator rule;
   std::vector<std::pair<int32_t, int32_t>> date_range;  // per date column: smallest, largest date
};
FeatureContext feature_context(const TableImage& t);

// The 24 features of an operator node: kind (one-hot), the rule estimate, shape of the subtree,
// leaf statistics (symbols, position, container count and encodings), predicate and threshold
// parameters. Every value lies roughly in [-1, 1].
void op_features(const Op& op, const FeatureContext& ctx, float* out);
// Every node of a tree (preorder) with its features, each node's rule estimate and subtree
// statistics computed once.
void tree_features(const Op& root, const FeatureContext& ctx, std::vector<const Op*>& nodes,
                   std::vector<std::array<float, PLAN_FEATURES>>& x);

struct PlannerSample {
   std::array<float, PLAN_FEATURES> x;
   float log_sel;       // ln(max(|result| / rows, 1e-7))
   float log_cost;      // ln(cycles per tile of the node's subtree)
   float rule_log_sel;  // the rule estimate, same scale
};

struct PlannerStats {
   uint32_t n_train, n_val, epochs;
   float train_loss, val_loss;
   float qerr_learned_median, qerr_rule_median;  // q-error = exp(|ln(predicted) - ln(measured)|)
   float qerr_learned_p90, qerr_rule_p90;
   float cost_err_median;  // median |ln predicted - ln measured| of the cost
   float train_ms;
   int accepted;
};

// The network on one device: FP32 master weights, their BF16 copy, Adam state.
class PlannerNet {
  public:
   explicit PlannerNet(int device);
   ~PlannerNet();
   PlannerNet(const PlannerNet&) = delete;
   PlannerNet& operator=(const PlannerNet&) = delete;

   void init(uint64_t seed);             // He-normal weights, zero biases, fresh Adam state
   void set_master(const float* w);      // MLP_NPARAM host floats
   void get_master(float* w) const;
   // One forward + backward over (X, T) as given (n x 24, n x 2): the gradient with respect to the
   // BF16 weights, the loss and optionally the outputs.
   void gradient(const float* X, const float* T, uint32_t n, float* grad, float* loss, float* Y);
   // Minibatch Adam over shuffled (X, T); returns the final epoch's mean loss.
   float train(const std::vector<float>& X, const std::vector<float>& T, uint32_t n, uint32_t epochs, uint32_t batch,
               float lr, uint64_t seed);
   void predict(const float* X, uint32_t n, float* Y);
   // Pinned host rows (n x MLP_IN) to fill before predict_staged, which runs the network on them
   // and returns its outputs (n x MLP_OUT, pinned, valid until the next call).
   float* staged_input(uint32_t n);
   const float* predict_staged(uint32_t n);

  private:
   void reserve(uint32_t n);
   float* h_X_ = nullptr;  // pinned staging
   float* h_Y_ = nullptr;
   uint32_t hcap_ = 0;
   int device_;
   float* d_master_ = nullptr;
   float* d_m_ = nullptr;
   float* d_v_ = nullptr;
   float* d_grad_ = nullptr;
   float* d_loss_ = nullptr;
   __nv_bfloat16* d_w_ = nullptr;
   float* d_X_ = nullptr;
   float* d_T_ = nullptr;
   float* d_Y_ = nullptr;
   uint32_t cap_ = 0;
   uint32_t step_ = 0;
   cudaStream_t stream_ = nullptr;
};

class Planner {
  public:
   explicit Planner(int device) : net(device) {}
   std::vector<PlannerSample> samples;
   bool trained = false;
   bool accepted = false;
   std::array<float, PLAN_FEATURES> fmean{}, fstd{};
   double tmean[2] = {0, 0}, tstd[2] = {1, 1};
   PlannerNet net;

   // Trains on `samples` (a seeded 80/20 split) and judges the result on the held-out part.
   PlannerStats train(uint32_t epochs, uint32_t batch, float lr, uint64_t seed);
   // Judges the current network on another sample set (traces of held-out queries, possibly on
   // another table) with the statistics and the acceptance rule of train's held-out split; the
   // verdict is returned, not applied.
   PlannerStats evaluate(const std::vector<PlannerSample>& set);
   // Selectivity (fraction of rows) and cycles per tile for each feature row.
   void predict(const std::vector<std::array<float, PLAN_FEATURES>>& x, std::vector<double>& sel,
                std::vector<double>& cost);
   // The same one row at a time around the network: its normalised input, then the selectivity
   // and cost from the raw features and the network's two outputs.
   void normalize(const float* x, float* out) const;
   double selectivity_of(const float* x, const float* y) const;
   double cost_of(const float* y) const;

  private:
   // q-errors of the network's outputs Y (two per sample) and of the rule estimates against the
   // measured selectivities, the cost error, and the verdict (st.val_loss must be set).
   void judge(const std::vector<const PlannerSample*>& set, const float* Y, PlannerStats& st) const;
};

}  // namespace rhygpu
