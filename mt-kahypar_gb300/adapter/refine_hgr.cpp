// Command-line driver of GpuLabelPropagationRefiner over the stand-in
// Mt-KaHyPar headers in shim/: reads an hMetis hypergraph and a partition
// file, refines with the device LP the way the multilevel driver calls a
// refiner (initialize, then refine with an empty node list), checks that the
// hypergraph's km1 equals the metrics the refiner reported, and writes the
// refined partition.
//
//   refine_hgr <graph.hgr> <k> <epsilon> <rounds> <partition_in> <partition_out>
//   refine_hgr --writeback-selftest       (no GPU needed)
//
// Exit codes: 0 ok, 1 usage or input error, 2 refiner error (for example no
// usable GPU), 3 inconsistent state after refinement.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "gpu_label_propagation_refiner.h"

using namespace mt_kahypar;

namespace {

Hypergraph make_hypergraph(int64_t n, int64_t m, const int64_t* off, const int32_t* pins, const int32_t* w_v,
                           const int32_t* w_e) {
  std::vector<size_t> o(off, off + m + 1);
  std::vector<HypernodeID> p(pins, pins + off[m]);
  std::vector<HypernodeWeight> wv(w_v ? w_v : nullptr, w_v ? w_v + n : nullptr);
  std::vector<HyperedgeWeight> we(w_e ? w_e : nullptr, w_e ? w_e + m : nullptr);
  if (!w_v) wv.assign(n, 1);
  if (!w_e) we.assign(m, 1);
  return Hypergraph((HypernodeID)n, (HyperedgeID)m, std::move(o), std::move(p), std::move(wv), std::move(we));
}

// The state phg holds equals a fresh initializePartition of its block ids.
bool consistent(const PartitionedHypergraph& phg) {
  PartitionedHypergraph fresh(phg.k(), phg.hypergraph());
  for (HypernodeID u = 0; u < phg.initialNumNodes(); ++u) fresh.setOnlyNodePart(u, phg.partID(u));
  fresh.initializePartition(0);
  for (PartitionID b = 0; b < phg.k(); ++b)
    if (fresh.partWeight(b) != phg.partWeight(b)) return false;
  for (HyperedgeID e = 0; e < phg.initialNumEdges(); ++e)
    for (PartitionID b = 0; b < phg.k(); ++b)
      if (fresh.pinCountInPart(e, b) != phg.pinCountInPart(e, b)) return false;
  return true;
}

int selftest() {
  // nets {0,1,2}, {1,3}, {2,4}, {0,4}, {3,4}: five vertices
  const int64_t off[] = {0, 3, 5, 7, 9, 11};
  const int32_t pins[] = {0, 1, 2, 1, 3, 2, 4, 0, 4, 3, 4};
  struct Case {
    PartitionID k;
    std::vector<int32_t> start, target;
    bool rebuilt;
  };
  const Case cases[] = {
      // block 0 holds only vertex 0, which leaves before vertex 3 arrives: retried
      {3, {0, 1, 1, 2, 2}, {1, 1, 1, 0, 2}, false},
      // the only vertices of blocks 0 and 1 swap: no order works, rebuilt
      {3, {0, 1, 2, 2, 2}, {1, 0, 2, 2, 2}, true},
      // plain moves
      {2, {0, 0, 1, 1, 1}, {0, 1, 1, 0, 1}, false},
  };
  for (const Case& c : cases) {
    Hypergraph hg = make_hypergraph(5, 5, off, pins, nullptr, nullptr);
    PartitionedHypergraph phg(c.k, hg);
    for (HypernodeID u = 0; u < 5; ++u) phg.setOnlyNodePart(u, c.start[u]);
    phg.initializePartition(0);
    const HyperedgeWeight before = metrics::km1(phg);
    const auto wb = GpuLabelPropagationRefiner::writeBack(phg, c.target, 0);
    for (HypernodeID u = 0; u < 5; ++u)
      if (phg.partID(u) != c.target[u]) return std::printf("selftest: block of %u\n", u), 3;
    if (!consistent(phg)) return std::printf("selftest: inconsistent pin counts\n"), 3;
    if (wb.delta != metrics::km1(phg) - before) return std::printf("selftest: delta\n"), 3;
    if (wb.rebuilt != c.rebuilt || (!c.rebuilt && c.k == 3 && wb.retried != 1))
      return std::printf("selftest: rebuilt %d retried %lld\n", (int)wb.rebuilt, (long long)wb.retried), 3;
  }
  std::printf("selftest ok\n");
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc == 2 && std::string(argv[1]) == "--writeback-selftest") return selftest();
  if (argc != 7) {
    std::fprintf(stderr, "usage: %s <graph.hgr> <k> <epsilon> <rounds> <partition_in> <partition_out>\n", argv[0]);
    return 1;
  }
  int64_t n = 0, m = 0, removed = 0;
  int64_t* off = nullptr;
  int32_t *pins = nullptr, *w_v = nullptr, *w_e = nullptr;
  if (lpgpu_read_hgr(argv[1], &n, &m, &off, &pins, &w_v, &w_e, &removed) != LPGPU_OK) {
    std::fprintf(stderr, "%s\n", lpgpu_last_error());
    return 1;
  }
  Hypergraph hg = make_hypergraph(n, m, off, pins, w_v, w_e);
  lpgpu_free(off);
  lpgpu_free(pins);
  lpgpu_free(w_v);
  lpgpu_free(w_e);
  Context context;
  context.partition.k = std::atoi(argv[2]);
  context.partition.epsilon = std::atof(argv[3]);
  context.partition.objective = kahypar::Objective::km1;
  context.setupPartWeights(hg.totalWeight());
  context.refinement.label_propagation.maximum_iterations = (size_t)std::atoi(argv[4]);
  context.refinement.label_propagation.rebalancing = true;
  context.refinement.label_propagation.hyperedge_size_activation_threshold = 100;
  std::vector<int32_t> part(n);
  if (lpgpu_read_partition(argv[5], n, part.data()) != LPGPU_OK) {
    std::fprintf(stderr, "%s\n", lpgpu_last_error());
    return 1;
  }
  PartitionedHypergraph phg(context.partition.k, hg);
  for (HypernodeID u = 0; u < (HypernodeID)n; ++u) phg.setOnlyNodePart(u, part[u]);
  phg.initializePartition(0);
  kahypar::Metrics best;
  best.km1 = metrics::km1(phg);
  best.imbalance = metrics::imbalance(phg, context);
  const HyperedgeWeight before = best.km1;
  bool improved = false;
  GpuLabelPropagationRefiner::WriteBack wb;
  try {
    GpuLabelPropagationRefiner refiner(hg, context, 0);
    refiner.initialize(phg);
    improved = refiner.refine(phg, {}, best, 0.0);
    wb = refiner.lastWriteBack();
  } catch (const std::exception& e) {
    std::fprintf(stderr, "refiner error: %s\n", e.what());
    return 2;
  }
  const HyperedgeWeight after = metrics::km1(phg);
  std::printf("km1_before %d km1_after %d reported %d improved %d imbalance %.6f moves %lld retried %lld rebuilt %d\n",
              before, after, best.km1, (int)improved, best.imbalance, (long long)wb.moves, (long long)wb.retried,
              (int)wb.rebuilt);
  if (after != best.km1 || !consistent(phg)) return 3;
  for (HypernodeID u = 0; u < (HypernodeID)n; ++u) part[u] = phg.partID(u);
  if (lpgpu_write_partition(argv[6], n, part.data()) != LPGPU_OK) {
    std::fprintf(stderr, "%s\n", lpgpu_last_error());
    return 1;
  }
  return 0;
}
