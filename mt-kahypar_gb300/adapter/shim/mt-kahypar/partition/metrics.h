// Minimal stand-in for Mt-KaHyPar's metrics (mt-kahypar/partition/metrics.h):
// km1 = Σ_e (λ(e) - 1)·w(e) and the imbalance max_b c(V_b) / perfect_b - 1.
#pragma once

#include <algorithm>

#include "mt-kahypar/definitions.h"
#include "mt-kahypar/partition/context.h"

namespace mt_kahypar {
namespace metrics {

inline HyperedgeWeight km1(const PartitionedHypergraph& phg) {
  HyperedgeWeight s = 0;
  for (HyperedgeID e : phg.edges()) s += std::max(phg.connectivity(e) - 1, 0) * phg.edgeWeight(e);
  return s;
}

inline double imbalance(const PartitionedHypergraph& phg, const Context& context) {
  double worst = -1.0;
  for (PartitionID b = 0; b < context.partition.k; ++b)
    worst = std::max(worst, phg.partWeight(b) / static_cast<double>(context.partition.perfect_balance_part_weights[b]));
  return worst - 1.0;
}

}  // namespace metrics
}  // namespace mt_kahypar
