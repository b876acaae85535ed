// Minimal stand-in for Mt-KaHyPar's refiner interface
// (mt-kahypar/partition/refinement/i_refiner.h): initialize per level, refine
// in place, return whether the objective improved. The member signatures are
// the reference's so that an adapter compiles against either.
#pragma once

#include "kahypar/partition/metrics.h"
#include "mt-kahypar/definitions.h"
#include "mt-kahypar/parallel/stl/scalable_vector.h"

namespace mt_kahypar {

class IRefiner {
 public:
  IRefiner(const IRefiner&) = delete;
  IRefiner& operator=(const IRefiner&) = delete;
  virtual ~IRefiner() = default;

  void initialize(PartitionedHypergraph& hypergraph) { initializeImpl(hypergraph); }

  bool refine(PartitionedHypergraph& hypergraph, const parallel::scalable_vector<HypernodeID>& refinement_nodes,
              kahypar::Metrics& best_metrics, const double time_limit) {
    return refineImpl(hypergraph, refinement_nodes, best_metrics, time_limit);
  }

 protected:
  IRefiner() = default;

 private:
  virtual void initializeImpl(PartitionedHypergraph& hypergraph) = 0;
  virtual bool refineImpl(PartitionedHypergraph& hypergraph,
                          const parallel::scalable_vector<HypernodeID>& refinement_nodes,
                          kahypar::Metrics& best_metrics, const double time_limit) = 0;
};

}  // namespace mt_kahypar
