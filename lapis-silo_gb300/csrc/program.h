// Device filter program: the postorder lowering of a compiled operator tree.
//
// Every filter operator of the reference is chunk-local (AND/OR/ANDNOT per roaring key, complement
// within each chunk's rows, NOf per row; reference: src/rhydb/query_engine/copy_on_write_bitmap.cpp:145-298,
// src/rhydb/storage/column/row_layout.cpp:18-23, src/rhydb/query_engine/filter/operators/threshold.cpp:64-138),
// so a program is evaluated independently for every tile of rows: one CTA runs the instruction
// list over a stack of dense bit tiles held in shared memory.
#pragma once

#include <cstdint>

namespace rhygpu {

enum OpCode : uint8_t {
   OP_PUSH_EMPTY = 0,
   OP_PUSH_FULL = 1,     // all rows of the tile that exist in the chunk
   OP_PUSH_SCAN = 2,     // col = sequence column, a = position, b = symbol mask: OR of the containers
                         // (c = ordinal among the program's PUSH_SCAN / PUSH_DICT leaves, from 1)
   OP_PUSH_NULLS = 3,    // col = sequence column: rows whose sequence is null
   OP_PUSH_DICT = 4,     // col = dictionary column, a = value id: inverted-index rows (c as for PUSH_SCAN)
   OP_PUSH_COVERED = 5,  // col = sequence column, a = position, flags&1: not covered instead of covered
                         // (c = ordinal among the program's PUSH_COVERED leaves, from 1)
   OP_PUSH_DATE = 6,     // col = date column; rows with lo <= date <= hi (a = lo, b = hi as int32),
                         // flags&2 = inverted (outside the range), flags&1 = null dates match
   OP_AND = 7,           // pop y, pop x, push x & y
   OP_ANDNOT = 8,        // pop y, pop x, push x & ~y
   OP_OR = 9,            // pop y, pop x, push x | y
   OP_NOT = 10,          // pop x, push valid & ~x
   OP_THR_BEGIN = 11,    // a = planes: push `a` zero counter planes
   OP_THR_ADD = 12,      // a = planes, flags&1 = negated child: pop x, saturating count += x (or ~x)
   OP_THR_END = 13,      // a = planes, b = n, flags&1 = exactly: pop planes, push count >= n (== n)
   OP_JZ = 14,           // a = target: jump if the top tile is all zero
   OP_JFULL = 15,        // a = target: jump if the top tile holds every valid row
   OP_PUSH_AUX = 16,     // a = index of a row set computed (a MutationProfile) or uploaded (a caller's row
                         // set, flags & AUX_LITERAL) before the program runs
};

constexpr uint16_t AUX_LITERAL = 1;  // PUSH_AUX of a caller's row set

// Comparators of the date predicate (reference: src/rhydb/query_engine/filter/operators/selection.h:40-72).
enum CmpCode : uint32_t { CMP_EQ = 0, CMP_NE = 1, CMP_LT = 2, CMP_LE = 3, CMP_GT = 4, CMP_GE = 5 };

struct Instr {
   uint8_t op;
   uint8_t col;
   uint16_t flags;
   uint32_t a;
   uint32_t b;
   uint32_t c;
};
static_assert(sizeof(Instr) == 16, "instruction layout");

constexpr uint32_t MAX_PROGRAM = 4096;   // instructions per program
constexpr uint32_t MAX_THR_PLANES = 16;  // counter planes (NOf up to 65,534 children)

}  // namespace rhygpu
