// The plan of the Mutations container pass of one sequence column (engine.cu): the units its
// consumer warps count and the ranges of units its CTAs take.
#pragma once

#include <cstdint>
#include <vector>

#include "device.h"
#include "table.h"

namespace rhygpu {

// Units of the Mutations container pass, chunk by chunk: the chunk's array payloads (back to back
// in descriptor order) cut into pieces of at most WU elements starting on 8-element (16-byte)
// boundaries, each with the descriptors that cover the arrays overlapping it, then one unit per
// bitset and run container. A piece ends early, before the first array whose descriptor would not
// fit, where more than WU_DESC descriptors would be needed. afirst[v] / ofirst[v]: the first array /
// other unit of chunk v (nchunks + 1 entries).
struct PassUnits {
   std::vector<ArrUnit> au;
   std::vector<OtherUnit> ou;
   std::vector<uint32_t> afirst, ofirst;
};
PassUnits pass_units(const SeqColumnImage& s, uint32_t nchunks);

// CTAs of the container pass: the units of each chunk, its bitset and run units spread evenly among
// its array units, cut into ranges of about the same counting time, none spanning more than two
// chunks; at most `ctas` ranges unless the table has more than 2 * ctas chunks.
std::vector<StreamRange> pass_ranges(const SeqColumnImage& s, const PassUnits& P, uint32_t nchunks, uint32_t ctas);

}  // namespace rhygpu
