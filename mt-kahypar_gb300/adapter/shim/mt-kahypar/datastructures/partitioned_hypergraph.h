// Minimal sequential stand-in for Mt-KaHyPar's StaticHypergraph and
// PartitionedHypergraph (mt-kahypar/datastructures/), enough to compile and
// test the GPU refiner adapter: CSR nets and incident nets, block ids, block
// weights and pin counts, with the reference's member names and semantics for
// setOnlyNodePart / initializePartition / resetPartition and the curried
// changeNodePart (refused when the source block would become empty,
// partitioned_hypergraph.h:539-572 of the reference; the delta function gets
// the pin counts after each net's update).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "mt-kahypar/definitions.h"

namespace mt_kahypar {
namespace ds {

template <typename T>
struct IdRange {  // [first, last) of consecutive ids
  struct It {
    T v;
    T operator*() const { return v; }
    It& operator++() {
      ++v;
      return *this;
    }
    bool operator!=(const It& o) const { return v != o.v; }
  };
  T first, last;
  It begin() const { return {first}; }
  It end() const { return {last}; }
};

template <typename T>
struct ArrayRange {  // a slice of an id array
  const T* first;
  const T* last;
  const T* begin() const { return first; }
  const T* end() const { return last; }
};

class StaticHypergraph {
 public:
  // Nets as CSR (net_offsets: m + 1 entries); the incident nets of every
  // vertex are built in increasing net id.
  StaticHypergraph(HypernodeID n, HyperedgeID m, std::vector<size_t> net_offsets, std::vector<HypernodeID> pins,
                   std::vector<HypernodeWeight> node_weights, std::vector<HyperedgeWeight> edge_weights)
      : _n(n), _m(m), _net_off(std::move(net_offsets)), _pins(std::move(pins)), _w_v(std::move(node_weights)),
        _w_e(std::move(edge_weights)), _vtx_off(n + 1, 0), _inets(_pins.size()) {
    for (HypernodeID p : _pins) ++_vtx_off[p + 1];
    for (HypernodeID v = 0; v < n; ++v) _vtx_off[v + 1] += _vtx_off[v];
    std::vector<size_t> cur(_vtx_off.begin(), _vtx_off.end() - 1);
    for (HyperedgeID e = 0; e < m; ++e)
      for (size_t i = _net_off[e]; i < _net_off[e + 1]; ++i) _inets[cur[_pins[i]]++] = e;
    for (HypernodeWeight w : _w_v) _total += w;
  }

  HypernodeID initialNumNodes() const { return _n; }
  HyperedgeID initialNumEdges() const { return _m; }
  size_t initialNumPins() const { return _pins.size(); }
  HypernodeWeight totalWeight() const { return _total; }
  HypernodeWeight nodeWeight(HypernodeID u) const { return _w_v[u]; }
  HyperedgeWeight edgeWeight(HyperedgeID e) const { return _w_e[e]; }
  HypernodeID edgeSize(HyperedgeID e) const { return (HypernodeID)(_net_off[e + 1] - _net_off[e]); }
  IdRange<HypernodeID> nodes() const { return {0, _n}; }
  IdRange<HyperedgeID> edges() const { return {0, _m}; }
  ArrayRange<HypernodeID> pins(HyperedgeID e) const { return {&_pins[_net_off[e]], &_pins[0] + _net_off[e + 1]}; }
  ArrayRange<HyperedgeID> incidentEdges(HypernodeID u) const {
    return {_inets.data() + _vtx_off[u], _inets.data() + _vtx_off[u + 1]};
  }

 private:
  HypernodeID _n;
  HyperedgeID _m;
  std::vector<size_t> _net_off;
  std::vector<HypernodeID> _pins;
  std::vector<HypernodeWeight> _w_v;
  std::vector<HyperedgeWeight> _w_e;
  std::vector<size_t> _vtx_off;
  std::vector<HyperedgeID> _inets;
  HypernodeWeight _total = 0;
};

class PartitionedHypergraph {
 public:
  PartitionedHypergraph(PartitionID k, StaticHypergraph& hypergraph)
      : _k(k), _hg(&hypergraph), _part(hypergraph.initialNumNodes(), kInvalidPartition), _part_w(k, 0),
        _phi((size_t)hypergraph.initialNumEdges() * k, 0) {}

  PartitionID k() const { return _k; }
  StaticHypergraph& hypergraph() const { return *_hg; }
  HypernodeID initialNumNodes() const { return _hg->initialNumNodes(); }
  HyperedgeID initialNumEdges() const { return _hg->initialNumEdges(); }
  size_t initialNumPins() const { return _hg->initialNumPins(); }
  HypernodeWeight totalWeight() const { return _hg->totalWeight(); }
  HypernodeWeight nodeWeight(HypernodeID u) const { return _hg->nodeWeight(u); }
  HyperedgeWeight edgeWeight(HyperedgeID e) const { return _hg->edgeWeight(e); }
  HypernodeID edgeSize(HyperedgeID e) const { return _hg->edgeSize(e); }
  IdRange<HypernodeID> nodes() const { return _hg->nodes(); }
  IdRange<HyperedgeID> edges() const { return _hg->edges(); }
  ArrayRange<HypernodeID> pins(HyperedgeID e) const { return _hg->pins(e); }
  ArrayRange<HyperedgeID> incidentEdges(HypernodeID u) const { return _hg->incidentEdges(u); }

  PartitionID partID(HypernodeID u) const { return _part[u]; }
  HypernodeWeight partWeight(PartitionID b) const { return _part_w[b]; }
  HypernodeID pinCountInPart(HyperedgeID e, PartitionID b) const { return _phi[(size_t)e * _k + b]; }
  PartitionID connectivity(HyperedgeID e) const {
    PartitionID c = 0;
    for (PartitionID b = 0; b < _k; ++b) c += _phi[(size_t)e * _k + b] > 0;
    return c;
  }

  // Block of a vertex without any other bookkeeping; the vertex must have none.
  void setOnlyNodePart(HypernodeID u, PartitionID p) { _part[u] = p; }

  // Block weights and pin counts from the block ids.
  void initializePartition(TaskGroupID) {
    std::fill(_part_w.begin(), _part_w.end(), 0);
    std::fill(_phi.begin(), _phi.end(), 0);
    for (HypernodeID u = 0; u < initialNumNodes(); ++u) _part_w[_part[u]] += nodeWeight(u);
    for (HyperedgeID e = 0; e < initialNumEdges(); ++e)
      for (HypernodeID p : pins(e)) ++_phi[(size_t)e * _k + _part[p]];
  }

  void resetPartition() {
    std::fill(_part.begin(), _part.end(), kInvalidPartition);
    std::fill(_part_w.begin(), _part_w.end(), 0);
    std::fill(_phi.begin(), _phi.end(), 0);
  }

  // Moves u from `from` to `to` unless `from` would become empty; calls
  // delta(e, w(e), |e|, pins of e left in from, pins of e now in to) per net.
  template <typename DeltaFunc>
  bool changeNodePart(HypernodeID u, PartitionID from, PartitionID to, DeltaFunc&& delta) {
    const HypernodeWeight wu = nodeWeight(u);
    if (_part_w[from] - wu <= 0) return false;
    _part_w[from] -= wu;
    _part_w[to] += wu;
    _part[u] = to;
    for (HyperedgeID e : incidentEdges(u)) {
      const HypernodeID from_after = --_phi[(size_t)e * _k + from];
      const HypernodeID to_after = ++_phi[(size_t)e * _k + to];
      delta(e, edgeWeight(e), edgeSize(e), from_after, to_after);
    }
    return true;
  }

 private:
  PartitionID _k;
  StaticHypergraph* _hg;
  std::vector<PartitionID> _part;
  std::vector<HypernodeWeight> _part_w;
  std::vector<HypernodeID> _phi;
};

}  // namespace ds
}  // namespace mt_kahypar
