// Operator trees across the C-ABI: a compiled operator tree as a postorder list of RhyOpNode
// (include/rhydb_gpu.h), to and from the engine's Op tree.
//
// A caller that has already compiled a filter into the reference's operator tree
// (src/rhydb/query_engine/filter/operators/operator.h:11-36: Empty, Full, IndexScan, Intersection,
// Complement, Selection, Threshold, Union) hands it over node by node, children before their
// parent. The checks of the reference's operator constructors apply and fail as they do there
// (QueryCompilationException: intersection.cpp:18-40, threshold.cpp:18-41).
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/rhydb_gpu.h"
#include "expr.h"
#include "table.h"

namespace rhygpu {

// Builds the Op tree of a postorder node list. row_set_cards[i] is the cardinality of the caller's
// row set i (RHY_NODE_SCAN_ROWS operands; used for estimates only). Malformed lists and operator
// invariants throw CompilationError; references to columns, positions, symbols or values that do
// not exist throw IllegalQuery.
OpPtr op_from_nodes(const RhyOpNode* nodes, uint32_t n, const TableImage& t, const std::vector<double>& row_set_cards);

// The postorder node list of an Op tree (its ROWS leaves keep their row-set indices). Trees holding
// a MutationProfile leaf have no node form and throw std::invalid_argument.
void op_to_nodes(const Op& op, std::vector<RhyOpNode>& out);

}  // namespace rhygpu
