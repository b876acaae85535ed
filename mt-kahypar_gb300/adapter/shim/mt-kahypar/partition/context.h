// Minimal stand-in for the parts of Mt-KaHyPar's Context
// (mt-kahypar/partition/context.h) that the refiners read: the partition
// parameters and the label-propagation parameters, and setupPartWeights
// (perfect = ceil(W / k), max = (HypernodeWeight)((1 + eps) * perfect)).
#pragma once

#include <cmath>
#include <cstddef>
#include <limits>
#include <vector>

#include "kahypar/partition/metrics.h"
#include "mt-kahypar/definitions.h"

namespace mt_kahypar {

struct PartitioningParameters {
  kahypar::Mode mode = kahypar::Mode::direct_kway;
  kahypar::Objective objective = kahypar::Objective::km1;
  double epsilon = std::numeric_limits<double>::max();
  PartitionID k = std::numeric_limits<PartitionID>::max();
  std::vector<HypernodeWeight> perfect_balance_part_weights;
  std::vector<HypernodeWeight> max_part_weights;
};

struct LabelPropagationParameters {
  size_t maximum_iterations = 1;
  bool rebalancing = true;
  bool execute_sequential = false;
  size_t hyperedge_size_activation_threshold = std::numeric_limits<size_t>::max();
};

struct RefinementParameters {
  LabelPropagationParameters label_propagation;
};

class Context {
 public:
  PartitioningParameters partition{};
  RefinementParameters refinement{};

  void setupPartWeights(const HypernodeWeight total_hypergraph_weight) {
    const HypernodeWeight perfect =
        (HypernodeWeight)std::ceil(total_hypergraph_weight / static_cast<double>(partition.k));
    partition.perfect_balance_part_weights.assign(partition.k, perfect);
    partition.max_part_weights.assign(partition.k, (HypernodeWeight)((1.0 + partition.epsilon) * perfect));
  }
};

}  // namespace mt_kahypar
