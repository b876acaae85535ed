// GpuLabelPropagationRefiner: the IRefiner of Mt-KaHyPar's label-propagation
// phase (mt-kahypar/partition/refinement/i_refiner.h:35-66), refining on one
// GB300 through liblpgpu's C ABI (include/lpgpu.h). A maintainer registers it
// next to the CPU refiner (register_refinement_algorithms.cpp:35-40) and the
// multilevel driver uses it unchanged: initialize() per uncoarsening level,
// refine() in place, returning whether km1 improved.
//
// What refine() does:
//   1. uploads the level's hypergraph once per initialize() (CSR of nets and
//      pins with vertex and net weights; the device builds the incident nets);
//   2. sets the current partition with the context's max and perfect block
//      weights (Context::setupPartWeights);
//   3. runs the synchronous device LP with the context's label-propagation
//      parameters (maximum_iterations, hyperedge_size_activation_threshold,
//      rebalancing) from `refinement_nodes` (empty: all vertices);
//   4. writes the refined partition back with changeNodePart, so that pin
//      counts, connectivity sets and block weights stay the hypergraph's own;
//   5. updates best_metrics (km1 and imbalance) as LabelPropagationRefiner
//      does (label_propagation_refiner.cpp:48-67).
//
// Write-back. The device only guarantees its final state (every block within
// its max weight and non-empty). Replaying its moves one by one can pass
// through a state the curried changeNodePart refuses: a block's last vertex
// leaving before another arrives (partitioned_hypergraph.h:551). Refused moves
// are retried after the others have been applied, until none is left or a
// pass makes no progress (vertices that swap the only vertices of two blocks);
// then the partition is rebuilt from the device's block ids (resetPartition,
// setOnlyNodePart, initializePartition). The km1 delta is summed from the
// delta function (km1Delta, hypergraph_common.h:133-140) over the applied
// moves, or taken as the difference of metrics::km1 after a rebuild, so
// best_metrics always ends at the hypergraph's km1.
//
// Errors: the reference stops the process on errors (ERROR, macros.h:108);
// this adapter throws std::runtime_error with the library's error text
// instead, and there is no CPU fallback: without a usable GPU, construction
// throws.
#pragma once

#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "lpgpu.h"
#include "mt-kahypar/definitions.h"
#include "mt-kahypar/partition/context.h"
#include "mt-kahypar/partition/metrics.h"
#include "mt-kahypar/partition/refinement/i_refiner.h"

namespace mt_kahypar {

class GpuLabelPropagationRefiner final : public IRefiner {
 public:
  // The factory signature of LabelPropagationFactory (factories.h:60-61).
  GpuLabelPropagationRefiner(Hypergraph&, const Context& context, const TaskGroupID task_group_id, int device = 0)
      : _context(context), _task_group_id(task_group_id) {
    check(lpgpu_session_create(device, &_session), "lpgpu_session_create");
  }

  ~GpuLabelPropagationRefiner() override { lpgpu_session_destroy(_session); }

  struct WriteBack {
    int64_t moves = 0;     // vertices whose block changed
    int64_t retried = 0;   // moves applied after a refused first try
    bool rebuilt = false;  // the partition was rebuilt from the block ids
    Gain delta = 0;        // km1 change
  };

  // Makes phg's partition equal `part` (see the file comment).
  static WriteBack writeBack(PartitionedHypergraph& phg, const std::vector<int32_t>& part, TaskGroupID task_group_id) {
    struct Move {
      HypernodeID u;
      PartitionID from, to;
    };
    WriteBack wb;
    std::vector<Move> pending;
    for (HypernodeID u = 0; u < phg.initialNumNodes(); ++u)
      if (phg.partID(u) != part[u]) pending.push_back({u, phg.partID(u), part[u]});
    wb.moves = (int64_t)pending.size();
    auto km1_delta = [&](const HyperedgeID, const HyperedgeWeight edge_weight, const HypernodeID,
                         const HypernodeID pin_count_in_from_part_after,
                         const HypernodeID pin_count_in_to_part_after) {
      wb.delta += (pin_count_in_to_part_after == 1 ? edge_weight : 0) +
                  (pin_count_in_from_part_after == 0 ? -edge_weight : 0);
    };
    bool first = true;
    while (!pending.empty()) {
      std::vector<Move> refused;
      for (const Move& m : pending) {
        if (phg.changeNodePart(m.u, m.from, m.to, km1_delta)) {
          if (!first) ++wb.retried;
        } else {
          refused.push_back(m);
        }
      }
      if (refused.size() == pending.size()) break;  // no progress: rebuild below
      pending.swap(refused);
      first = false;
    }
    if (!pending.empty()) {
      const HyperedgeWeight before = metrics::km1(phg) - wb.delta;  // km1 before any move
      phg.resetPartition();
      for (HypernodeID u = 0; u < phg.initialNumNodes(); ++u) phg.setOnlyNodePart(u, part[u]);
      phg.initializePartition(task_group_id);
      wb.delta = metrics::km1(phg) - before;
      wb.rebuilt = true;
    }
    return wb;
  }

  const WriteBack& lastWriteBack() const { return _last; }
  const lpgpu_result& lastResult() const { return _result; }

 private:
  static void check(lpgpu_status s, const char* what) {
    if (s != LPGPU_OK)
      throw std::runtime_error(std::string(what) + ": " + lpgpu_status_string(s) + ": " + lpgpu_last_error());
  }

  void initializeImpl(PartitionedHypergraph& phg) override {
    const HypernodeID n = phg.initialNumNodes();
    const HyperedgeID m = phg.initialNumEdges();
    std::vector<int64_t> net_off(m + 1, 0);
    std::vector<int32_t> pins;
    std::vector<int32_t> w_v(n), w_e(m);
    pins.reserve(phg.initialNumPins());
    for (HyperedgeID e = 0; e < m; ++e) {
      for (HypernodeID p : phg.pins(e)) pins.push_back((int32_t)p);
      net_off[e + 1] = (int64_t)pins.size();
      w_e[e] = phg.edgeWeight(e);
    }
    for (HypernodeID u = 0; u < n; ++u) w_v[u] = phg.nodeWeight(u);
    check(lpgpu_session_upload(_session, n, m, net_off.data(), pins.data(), w_v.data(), w_e.data()),
          "lpgpu_session_upload");
    _n = n;
    _m = m;
  }

  bool refineImpl(PartitionedHypergraph& phg, const parallel::scalable_vector<HypernodeID>& refinement_nodes,
                  kahypar::Metrics& best_metrics, const double) override {
    if (_n != phg.initialNumNodes() || _m != phg.initialNumEdges()) initializeImpl(phg);
    const PartitionID k = _context.partition.k;
    std::vector<int32_t> part(_n);
    for (HypernodeID u = 0; u < _n; ++u) part[u] = phg.partID(u);
    std::vector<int64_t> lmax(_context.partition.max_part_weights.begin(), _context.partition.max_part_weights.end());
    std::vector<int64_t> perfect(_context.partition.perfect_balance_part_weights.begin(),
                                 _context.partition.perfect_balance_part_weights.end());
    check(lpgpu_session_set_partition(_session, k, _context.partition.epsilon, part.data(), lmax.data(),
                                      perfect.data()),
          "lpgpu_session_set_partition");
    const LabelPropagationParameters& lp = _context.refinement.label_propagation;
    lpgpu_config cfg;
    lpgpu_config_default(&cfg);
    cfg.rounds = (int32_t)std::min<size_t>(lp.maximum_iterations, 1u << 20);
    cfg.rebalancing = lp.rebalancing ? 1 : 0;
    cfg.activation_threshold = lp.hyperedge_size_activation_threshold >= (size_t)std::numeric_limits<int32_t>::max()
                                   ? 0  // no limit
                                   : (int32_t)lp.hyperedge_size_activation_threshold;
    std::vector<int32_t> nodes(refinement_nodes.begin(), refinement_nodes.end());
    check(lpgpu_session_refine(_session, &cfg, nodes.empty() ? nullptr : nodes.data(), (int64_t)nodes.size(),
                               &_result),
          "lpgpu_session_refine");
    check(lpgpu_session_get_partition(_session, part.data()), "lpgpu_session_get_partition");
    _last = writeBack(phg, part, _task_group_id);
    if (_last.delta != _result.delta)
      throw std::runtime_error("write-back km1 change differs from the device's attributed delta");
    best_metrics.imbalance = metrics::imbalance(phg, _context);
    const HyperedgeWeight current = best_metrics.getMetric(kahypar::Mode::direct_kway, _context.partition.objective);
    best_metrics.updateMetric(current + _last.delta, kahypar::Mode::direct_kway, _context.partition.objective);
    return _last.delta < 0;
  }

  const Context& _context;
  TaskGroupID _task_group_id;
  lpgpu_session* _session = nullptr;
  HypernodeID _n = 0;
  HyperedgeID _m = 0;
  WriteBack _last;
  lpgpu_result _result{};
};

}  // namespace mt_kahypar
