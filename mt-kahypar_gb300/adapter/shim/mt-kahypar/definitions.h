// Minimal stand-in for Mt-KaHyPar's mt-kahypar/definitions.h, written for
// compiling the GPU refiner adapter without the reference tree: the id and
// weight types (32-bit, as the reference's) and the hypergraph aliases.
#pragma once

#include <cstddef>
#include <cstdint>
#include <limits>

namespace mt_kahypar {

using HypernodeID = uint32_t;
using HyperedgeID = uint32_t;
using PartitionID = int32_t;
using HypernodeWeight = int32_t;
using HyperedgeWeight = int32_t;
using Gain = int32_t;
using TaskGroupID = size_t;

constexpr PartitionID kInvalidPartition = -1;

namespace ds {
class StaticHypergraph;
class PartitionedHypergraph;
}  // namespace ds

using Hypergraph = ds::StaticHypergraph;
using PartitionedHypergraph = ds::PartitionedHypergraph;

}  // namespace mt_kahypar

#include "mt-kahypar/datastructures/partitioned_hypergraph.h"
