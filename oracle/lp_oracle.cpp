// CPU oracle for the label-propagation (km1) refinement path.
//
// TEST INFRASTRUCTURE ONLY. This file is a plain C++17 restatement of the
// reference's algorithm, used as the checker by the test suite, by the smoke
// check and by the benchmark's CPU-baseline leg. Nothing in the product
// library links, loads or calls it.
//
// Reference files restated here (paths inside the Mt-KaHyPar source tree):
//   mt-kahypar/datastructures/static_hypergraph_factory.cpp:32-166 (stable incidence order)
//   mt-kahypar/datastructures/partitioned_hypergraph.h:539-563   (changeNodePart)
//   mt-kahypar/datastructures/partitioned_hypergraph.h:605-620   (isBorderNode)
//   mt-kahypar/datastructures/partitioned_hypergraph.h:647-688   (moveFromBenefit/moveToPenalty/km1Gain)
//   mt-kahypar/datastructures/partitioned_hypergraph.h:1067-1110 (initializeBlockWeights/PinCountInPart)
//   mt-kahypar/datastructures/partitioned_hypergraph.h:1133-1167 (updatePinCountOfHyperedge)
//   mt-kahypar/datastructures/hypergraph_common.h:133-140        (km1Delta)
//   mt-kahypar/partition/refinement/policies/gain_policy.h:108-177 (Km1Policy)
//   mt-kahypar/partition/refinement/label_propagation/label_propagation_refiner.h:76-165
//   mt-kahypar/partition/refinement/label_propagation/label_propagation_refiner.cpp:34-233
//   mt-kahypar/partition/metrics.cpp:29-65,114-128                (cut, km1, imbalance)
//   mt-kahypar/partition/context.cpp:237-250                      (perfect / max part weights)
//   mt-kahypar/utils/randomize.h:56-64,112-121                    (per-thread mt19937 coin flips)
//
// Parity status: pinned against the reference's own known-answer tests
// (gain_policy_test.cc, partitioned_hypergraph_test.cc, gain_updates_test.cc)
// in tests/test_oracle_pins.py. The reference itself cannot be built here
// (it needs TBB's legacy task API, hwloc, Boost and an un-vendored submodule).
//
// Layouts (shared with the device library):
//   net_off[m+1] int64, pins[P] int32, vtx_off[n+1] int64, inets[P] int32,
//   w_v[n] int32, w_e[m] int32, part[n] int32,
//   phi[m*k] int32 (pin count of net e in block b at e*k+b),
//   conn[m*W] uint32 with W = ceil(k/32) (bit b%32 of word b/32 = block b in Λ(e)).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

namespace {

constexpr int64_t kHighDegreeThreshold = 100000;  // partitioned_hypergraph.h:67

struct Hg {
  int64_t n, m;
  const int64_t* net_off;
  const int32_t* pins;
  const int64_t* vtx_off;
  const int32_t* inets;
  const int32_t* w_v;
  const int32_t* w_e;
};

inline int words_for(int k) { return (k + 31) / 32; }
inline bool bit_of(const uint32_t* conn, int W, int64_t e, int b) {
  return (conn[e * W + (b >> 5)] >> (b & 31)) & 1u;
}
inline void toggle(uint32_t* conn, int W, int64_t e, int b) {
  conn[e * W + (b >> 5)] ^= (1u << (b & 31));
}
inline int connectivity(const uint32_t* conn, int W, int64_t e) {
  int c = 0;
  for (int w = 0; w < W; ++w) c += __builtin_popcount(conn[e * W + w]);
  return c;
}

// Mutable partition state (PartitionedHypergraph without gain cache).
struct State {
  const Hg* hg;
  int k, W;
  std::vector<int32_t> part;
  std::vector<int32_t> phi;
  std::vector<uint32_t> conn;
  std::vector<int64_t> bw;

  // partitioned_hypergraph.h:1067-1110 (initializeBlockWeights + initializePinCountInPart)
  void init(const int32_t* p) {
    const int64_t n = hg->n, m = hg->m;
    part.assign(p, p + n);
    phi.assign(static_cast<size_t>(m) * k, 0);
    conn.assign(static_cast<size_t>(m) * W, 0u);
    bw.assign(k, 0);
    for (int64_t v = 0; v < n; ++v) bw[part[v]] += hg->w_v[v];
    for (int64_t e = 0; e < m; ++e) {
      for (int64_t i = hg->net_off[e]; i < hg->net_off[e + 1]; ++i) {
        const int b = part[hg->pins[i]];
        if (phi[e * k + b]++ == 0) toggle(conn.data(), W, e, b);
      }
    }
  }

  // partitioned_hypergraph.h:605-620
  bool is_border(int64_t v) const {
    const int64_t deg = hg->vtx_off[v + 1] - hg->vtx_off[v];
    if (deg > kHighDegreeThreshold) return false;
    for (int64_t i = hg->vtx_off[v]; i < hg->vtx_off[v + 1]; ++i)
      if (connectivity(conn.data(), W, hg->inets[i]) > 1) return true;
    return false;
  }

  // Km1Policy::computeMaxGainMoveImpl with disable_randomization = true
  // (gain_policy.h:108-167). Feasibility uses the block weights in `weights`.
  // Returns the target block (== from if none) and the objective delta
  // (negative = improvement) in *gain.
  int best_move(int64_t v, const int64_t* weights, const int64_t* lmax,
                std::vector<int64_t>& scores, int64_t* gain) const {
    const int from = part[v];
    int64_t internal = 0;
    for (int64_t i = hg->vtx_off[v]; i < hg->vtx_off[v + 1]; ++i) {
      const int64_t e = hg->inets[i];
      const int64_t we = hg->w_e[e];
      if (phi[e * k + from] > 1) internal += we;
      for (int w = 0; w < W; ++w) {
        uint32_t bits = conn[e * W + w];
        while (bits) {
          const int b = w * 32 + __builtin_ctz(bits);
          bits &= bits - 1;
          if (b != from) scores[b] -= we;
        }
      }
    }
    int to = from;
    int64_t best = 0;
    const int64_t wv = hg->w_v[v];
    for (int b = 0; b < k; ++b) {
      if (b != from) {
        const int64_t score = scores[b] + internal;
        if (score < best && weights[b] + wv <= lmax[b]) {
          to = b;
          best = score;
        }
      }
      scores[b] = 0;
    }
    *gain = best;
    return to;
  }

  // Objective delta of moving v (currently in `cur`) to `tgt`, no balance check.
  int64_t move_score(int64_t v, int cur, int tgt) const {
    int64_t internal = 0, pen = 0;
    for (int64_t i = hg->vtx_off[v]; i < hg->vtx_off[v + 1]; ++i) {
      const int64_t e = hg->inets[i];
      const int64_t we = hg->w_e[e];
      if (phi[e * k + cur] > 1) internal += we;
      if (bit_of(conn.data(), W, e, tgt)) pen += we;
    }
    return internal - pen;
  }

  // scores[b] = objective delta of moving v from `cur` to b, for every block
  // (no balance check); the all-blocks form of move_score.
  void move_scores(int64_t v, int cur, std::vector<int64_t>& scores) const {
    int64_t internal = 0;
    for (int64_t i = hg->vtx_off[v]; i < hg->vtx_off[v + 1]; ++i) {
      const int64_t e = hg->inets[i];
      const int64_t we = hg->w_e[e];
      if (phi[e * k + cur] > 1) internal += we;
      for (int w = 0; w < W; ++w) {
        uint32_t bits = conn[e * W + w];
        while (bits) {
          scores[w * 32 + __builtin_ctz(bits)] -= we;
          bits &= bits - 1;
        }
      }
    }
    for (int b = 0; b < k; ++b) scores[b] += internal;
  }

  // changeNodePart body after the weight check (partitioned_hypergraph.h:553-557)
  // with updatePinCountOfHyperedge (1133-1143) and km1Delta (hypergraph_common.h:133-140).
  int64_t apply_move(int64_t v, int from, int to) {
    int64_t delta = 0;
    const int64_t wv = hg->w_v[v];
    bw[to] += wv;
    bw[from] -= wv;
    part[v] = to;
    for (int64_t i = hg->vtx_off[v]; i < hg->vtx_off[v + 1]; ++i) {
      const int64_t e = hg->inets[i];
      const int64_t we = hg->w_e[e];
      const int32_t from_after = --phi[e * k + from];
      if (from_after == 0) toggle(conn.data(), W, e, from);
      const int32_t to_after = ++phi[e * k + to];
      if (to_after == 1) toggle(conn.data(), W, e, to);
      delta += (to_after == 1 ? we : 0) + (from_after == 0 ? -we : 0);
    }
    return delta;
  }

  int64_t km1() const {
    int64_t s = 0;
    for (int64_t e = 0; e < hg->m; ++e) {
      const int c = connectivity(conn.data(), W, e);
      s += static_cast<int64_t>(std::max(c - 1, 0)) * hg->w_e[e];
    }
    return s;
  }
};

Hg make_hg(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
           const int64_t* vtx_off, const int32_t* inets, const int32_t* w_v,
           const int32_t* w_e) {
  return Hg{n, m, net_off, pins, vtx_off, inets, w_v, w_e};
}

// body(i, scratch) for i in [0, count) on `threads` std::threads (contiguous
// chunks handed out dynamically); each thread owns a zeroed int64 scratch
// vector of `scratch_len` entries that body must leave zeroed.
template <typename Body>
void parallel_for(int threads, int64_t count, Body body, int scratch_len) {
  const int64_t chunk = 1024;
  if (threads <= 1 || count <= chunk) {
    std::vector<int64_t> scratch(scratch_len, 0);
    for (int64_t i = 0; i < count; ++i) body(i, scratch);
    return;
  }
  std::atomic<int64_t> next{0};
  auto worker = [&]() {
    std::vector<int64_t> scratch(scratch_len, 0);
    for (;;) {
      const int64_t b = next.fetch_add(chunk);
      if (b >= count) break;
      const int64_t e = std::min(count, b + chunk);
      for (int64_t i = b; i < e; ++i) body(i, scratch);
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
}

inline uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

}  // namespace

extern "C" {

// Run statistics, one record per executed LP round.
typedef struct {
  int64_t active;        // active vertices swept
  int64_t pins;          // Σ deg(v) over swept vertices (P_A)
  int64_t candidates;    // vertices with an improving feasible move
  int64_t moved;         // moves committed and kept
  int64_t reverted;      // moves undone by the hindsight check
  int64_t delta;         // Σ attributed objective deltas of the round
  int64_t km1_after;     // km1 recomputed after the round
  double seconds;        // wall-clock of the round
} orc_round_stats;

typedef struct {
  int32_t rounds;                // maximum LP rounds
  int32_t activation_threshold;  // nets with |e| <= threshold activate their pins (<= 0: all)
  int32_t subrounds;             // sub-rounds per round (>= 1)
  int32_t revert;                // 1: undo moves that turned out harmful
  int32_t rollback;              // 1: undo a whole sub-round whose delta is positive
  int32_t threads;               // worker threads (async mode; sync mode's per-vertex sweep)
  int32_t zero_gain;             // 1: deterministic zero-gain rebalancing moves (sync mode)
  int64_t seed;                  // async mode only
} orc_lp_cfg;

// Stable transpose of the pin lists (static_hypergraph_factory.cpp:51-156 with
// stable_construction: incident nets of a vertex in increasing net id).
void orc_transpose(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
                   int64_t* vtx_off, int32_t* inets) {
  std::memset(vtx_off, 0, sizeof(int64_t) * (n + 1));
  const int64_t P = net_off[m];
  for (int64_t i = 0; i < P; ++i) vtx_off[pins[i] + 1]++;
  for (int64_t v = 0; v < n; ++v) vtx_off[v + 1] += vtx_off[v];
  std::vector<int64_t> cur(vtx_off, vtx_off + n);
  for (int64_t e = 0; e < m; ++e)
    for (int64_t i = net_off[e]; i < net_off[e + 1]; ++i) inets[cur[pins[i]]++] = (int32_t)e;
}

// initializePartition (partitioned_hypergraph.h:693-698).
void orc_init_partition(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
                        const int32_t* w_v, int32_t k, const int32_t* part,
                        int32_t* phi, uint32_t* conn, int64_t* block_w) {
  Hg hg = make_hg(n, m, net_off, pins, nullptr, nullptr, w_v, nullptr);
  State s{&hg, k, words_for(k), {}, {}, {}, {}};
  s.init(part);
  std::memcpy(phi, s.phi.data(), sizeof(int32_t) * s.phi.size());
  std::memcpy(conn, s.conn.data(), sizeof(uint32_t) * s.conn.size());
  std::memcpy(block_w, s.bw.data(), sizeof(int64_t) * k);
}

// metrics::km1 and metrics::hyperedgeCut (metrics.cpp:29-65).
void orc_metrics(int64_t m, const int32_t* w_e, int32_t k, const uint32_t* conn,
                 int64_t* km1_out, int64_t* cut_out) {
  const int W = words_for(k);
  int64_t km1 = 0, cut = 0;
  for (int64_t e = 0; e < m; ++e) {
    const int c = connectivity(conn, W, e);
    km1 += static_cast<int64_t>(std::max(c - 1, 0)) * w_e[e];
    if (c > 1) cut += w_e[e];
  }
  *km1_out = km1;
  *cut_out = cut;
}

// Per-vertex best move under Km1Policy (disable_randomization) with the
// isBorderNode filter of moveVertex (label_propagation_refiner.h:82-85).
// to_out[v] = target block (== part[v] when no move), gain_out[v] = objective
// delta (0 when no move), border_out[v] = isBorderNode(v).
void orc_best_moves(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
                    const int64_t* vtx_off, const int32_t* inets, const int32_t* w_v,
                    const int32_t* w_e, int32_t k, const int32_t* part, const int64_t* lmax,
                    int32_t* to_out, int32_t* gain_out, uint8_t* border_out) {
  Hg hg = make_hg(n, m, net_off, pins, vtx_off, inets, w_v, w_e);
  State s{&hg, k, words_for(k), {}, {}, {}, {}};
  s.init(part);
  std::vector<int64_t> scores(k, 0);
  for (int64_t v = 0; v < n; ++v) {
    const bool border = s.is_border(v);
    border_out[v] = border;
    int64_t g = 0;
    int to = part[v];
    if (border) to = s.best_move(v, s.bw.data(), lmax, scores, &g);
    to_out[v] = to;
    gain_out[v] = (int32_t)g;
  }
}

// Gain cache (partitioned_hypergraph.h:647-688, 707-809): benefit[v] =
// moveFromBenefit(v); penalty[v*k+b] = moveToPenalty(v, b).
void orc_gain_cache(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
                    const int64_t* vtx_off, const int32_t* inets, const int32_t* w_v,
                    const int32_t* w_e, int32_t k, const int32_t* part,
                    int32_t* benefit, int32_t* penalty) {
  Hg hg = make_hg(n, m, net_off, pins, vtx_off, inets, w_v, w_e);
  State s{&hg, k, words_for(k), {}, {}, {}, {}};
  s.init(part);
  std::vector<int64_t> agg(k, 0);
  for (int64_t v = 0; v < n; ++v) {
    const int pv = part[v];
    int64_t b = 0, incident = 0;
    for (int64_t i = vtx_off[v]; i < vtx_off[v + 1]; ++i) {
      const int64_t e = inets[i];
      const int64_t we = w_e[e];
      if (s.phi[e * k + pv] == 1) b += we;
      for (int q = 0; q < k; ++q)
        if (bit_of(s.conn.data(), s.W, e, q)) agg[q] += we;
      incident += we;
    }
    benefit[v] = (int32_t)b;
    for (int q = 0; q < k; ++q) {
      penalty[v * k + q] = (int32_t)(incident - agg[q]);
      agg[q] = 0;
    }
  }
}

// Synchronous, snapshot-based LP refinement: the exact semantics of the
// device path. Per round (label_propagation_refiner.cpp:72-164 for the round
// loop and the active-set rules, label_propagation_refiner.h:76-143 per vertex):
//   * the active set is split into `subrounds` groups by a hash of (v >> 5, round);
//   * per group: every active border vertex computes its Km1Policy best move on
//     the current state (feasibility against the current block weights);
//   * moves with objective delta < 0 are candidates; per target block they are
//     ordered by (delta, vertex id) and the longest prefix that keeps the block
//     within its max weight is accepted; the accepted moves are then ordered the
//     same way per source block and the longest prefix that leaves the block
//     non-empty is kept;
//   * kept moves are committed with km1Delta attribution;
//   * with `revert`, every committed move whose reverse move now strictly
//     improves km1 is undone (all at once);
//   * with `rollback`, a group whose summed delta is positive is undone;
//   * moved vertices and the pins of their nets with |e| <= threshold become
//     active for the next round.
// Returns the number of rounds executed. `stats` holds up to cfg->rounds records.
int32_t orc_lp_sync(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
                    const int64_t* vtx_off, const int32_t* inets, const int32_t* w_v,
                    const int32_t* w_e, int32_t k, const int64_t* lmax, const int64_t* perfect,
                    int32_t* part_inout, const orc_lp_cfg* cfg, orc_round_stats* stats) {
  Hg hg = make_hg(n, m, net_off, pins, vtx_off, inets, w_v, w_e);
  State s{&hg, k, words_for(k), {}, {}, {}, {}};
  s.init(part_inout);
  // initializeActiveNodes (label_propagation_refiner.cpp:194-233): all vertices
  // with rebalancing, else the border vertices
  std::vector<int32_t> active;
  for (int64_t v = 0; v < n; ++v)
    if (cfg->zero_gain || s.is_border(v)) active.push_back((int32_t)v);
  std::vector<uint8_t> next_flag(n, 0);
  const int S = std::max(1, cfg->subrounds);
  const int64_t T = cfg->activation_threshold <= 0 ? INT64_MAX : cfg->activation_threshold;
  const int threads = std::max(1, cfg->threads);

  struct Cand { int32_t v, from, to; int64_t gain; int64_t w; };
  int32_t r = 0;
  for (; r < cfg->rounds; ++r) {
    if (active.empty()) break;
    auto t0 = std::chrono::steady_clock::now();
    orc_round_stats st{};
    std::fill(next_flag.begin(), next_flag.end(), 0);
    for (int sub = 0; sub < S; ++sub) {
      // the sub-round's vertices in active-list order, then their moves on the
      // snapshot (a pure function of the state, so worker threads give the
      // same candidates as one thread)
      std::vector<int32_t> group;
      for (int32_t v : active) {
        if (S > 1 && (int)(mix32((uint32_t)(v >> 5) ^ (0x9E3779B9u * (uint32_t)(r + 1))) % S) != sub)
          continue;
        group.push_back(v);
        st.active++;
        st.pins += vtx_off[v + 1] - vtx_off[v];
      }
      std::vector<Cand> found(group.size());
      std::vector<uint8_t> has(group.size(), 0);
      parallel_for(threads, (int64_t)group.size(), [&](int64_t i, std::vector<int64_t>& scores) {
        const int32_t v = group[i];
        if (!s.is_border(v)) return;
        int64_t g = 0;
        const int from = s.part[v];
        int to = s.best_move(v, s.bw.data(), lmax, scores, &g);
        if (to == from && cfg->zero_gain && perfect) {
          // lowest-id feasible block with score 0 under the rebalancing rule of
          // label_propagation_refiner.h:88-95
          s.move_scores(v, from, scores);
          for (int b = 0; b < k; ++b) {
            if (b == from || s.bw[b] + w_v[v] > lmax[b]) continue;
            if (scores[b] != 0) continue;
            if (s.bw[from] - 1 > s.bw[b] + 1 && s.bw[b] < perfect[b]) { to = b; g = 0; }
            break;
          }
          std::fill(scores.begin(), scores.end(), 0);
        }
        if (to != from && g <= 0) {
          found[i] = {v, from, to, g, w_v[v]};
          has[i] = 1;
        }
      }, k);
      std::vector<Cand> cands;
      for (size_t i = 0; i < group.size(); ++i)
        if (has[i]) cands.push_back(found[i]);
      st.candidates += (int64_t)cands.size();
      auto key_less = [](const Cand& a, const Cand& b) {
        return a.gain != b.gain ? a.gain < b.gain : a.v < b.v;
      };
      std::sort(cands.begin(), cands.end(), key_less);
      // target-side prefix
      std::vector<int64_t> in(k, 0);
      std::vector<uint8_t> stop_in(k, 0), ok(cands.size(), 0);
      for (size_t i = 0; i < cands.size(); ++i) {
        const Cand& c = cands[i];
        if (stop_in[c.to]) continue;
        if (s.bw[c.to] + in[c.to] + c.w <= lmax[c.to]) {
          in[c.to] += c.w;
          ok[i] = 1;
        } else {
          stop_in[c.to] = 1;
        }
      }
      // source-side prefix over the accepted moves
      std::vector<int64_t> out(k, 0);
      std::vector<uint8_t> stop_out(k, 0);
      for (size_t i = 0; i < cands.size(); ++i) {
        if (!ok[i]) continue;
        const Cand& c = cands[i];
        if (stop_out[c.from]) { ok[i] = 0; continue; }
        if (s.bw[c.from] - out[c.from] - c.w >= 1) {
          out[c.from] += c.w;
        } else {
          stop_out[c.from] = 1;
          ok[i] = 0;
        }
      }
      std::vector<Cand> moved;
      int64_t delta = 0;
      for (size_t i = 0; i < cands.size(); ++i) {
        if (!ok[i]) continue;
        delta += s.apply_move(cands[i].v, cands[i].from, cands[i].to);
        moved.push_back(cands[i]);
      }
      if (cfg->revert && !moved.empty()) {
        std::vector<uint8_t> back(moved.size(), 0);
        parallel_for(threads, (int64_t)moved.size(), [&](int64_t i, std::vector<int64_t>&) {
          back[i] = s.move_score(moved[i].v, moved[i].to, moved[i].from) < 0;
        }, 0);
        std::vector<Cand> kept;
        for (size_t i = 0; i < moved.size(); ++i) {
          if (back[i]) {
            delta += s.apply_move(moved[i].v, moved[i].to, moved[i].from);
            st.reverted++;
          } else {
            kept.push_back(moved[i]);
          }
        }
        moved.swap(kept);
      }
      if (cfg->rollback && delta > 0) {
        for (const Cand& c : moved) delta += s.apply_move(c.v, c.to, c.from);
        st.reverted += (int64_t)moved.size();
        moved.clear();
      }
      st.delta += delta;
      st.moved += (int64_t)moved.size();
      for (const Cand& c : moved) {
        next_flag[c.v] = 1;
        for (int64_t i = vtx_off[c.v]; i < vtx_off[c.v + 1]; ++i) {
          const int64_t e = inets[i];
          if (net_off[e + 1] - net_off[e] <= T)
            for (int64_t j = net_off[e]; j < net_off[e + 1]; ++j) next_flag[pins[j]] = 1;
        }
      }
    }
    active.clear();
    for (int64_t v = 0; v < n; ++v)
      if (next_flag[v]) active.push_back((int32_t)v);
    st.km1_after = s.km1();
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) stats[r] = st;
  }
  std::memcpy(part_inout, s.part.data(), sizeof(int32_t) * n);
  return r;
}

}  // extern "C"

namespace {

struct RepairMove {
  int32_t v, from, to, gain;
};

// Rebalancer::repairEmptyBlocks (rebalancing/rebalancer.cpp:169-269) as one
// worker thread computes it. For every empty block i (c(i) = 0), ascending:
//   * a vertex u in block p = part(u) is eligible when c(p) > w(u) and
//     w(u) <= L_max(i); its gain (positive = better, km1Gain) is
//     score(i) - unremovable(u), with score(i) = Σ w(e) over the incident nets
//     whose connectivity set holds i and unremovable(u) = Σ w(e) over the
//     incident nets with Φ(e, p) > 1 (rebalancer.cpp:190-201);
//   * the worker's bounded heap keeps the k eligible vertices of highest gain,
//     the earlier (lower) id on ties, as the heap of rebalancer.cpp:204-213
//     does for vertices scanned in id order;
//   * among them, ordered by gain, then c(part(u)), then u, all descending
//     (prefer_highest_gain, rebalancer.cpp:228-232), the first vertex not yet
//     chosen for an earlier block is the block's move (rebalancer.cpp:242-254).
// Block weights are those of the call (no move is applied here). A block
// without an eligible vertex stays empty: the reference's outer loop would
// repeat the same scan forever in that case, so one pass is the whole result.
std::vector<RepairMove> repair_empty_blocks(const State& s, const int64_t* lmax) {
  const Hg& hg = *s.hg;
  const int k = s.k;
  std::vector<RepairMove> moves;
  std::vector<uint8_t> used(hg.n, 0);
  std::vector<int64_t> unremovable(hg.n, 0);
  for (int64_t v = 0; v < hg.n; ++v)
    for (int64_t i = hg.vtx_off[v]; i < hg.vtx_off[v + 1]; ++i) {
      const int64_t e = hg.inets[i];
      if (s.phi[e * k + s.part[v]] > 1) unremovable[v] += hg.w_e[e];
    }
  struct C { int64_t gain; int32_t v; };
  for (int i = 0; i < k; ++i) {
    if (s.bw[i] != 0) continue;
    std::vector<C> top;
    for (int64_t v = 0; v < hg.n; ++v) {
      const int p = s.part[v];
      if (p == i || s.bw[p] <= hg.w_v[v] || hg.w_v[v] > lmax[i]) continue;
      int64_t score = 0;
      for (int64_t j = hg.vtx_off[v]; j < hg.vtx_off[v + 1]; ++j) {
        const int64_t e = hg.inets[j];
        if (bit_of(s.conn.data(), s.W, e, i)) score += hg.w_e[e];
      }
      top.push_back({score - unremovable[v], (int32_t)v});
    }
    auto heap_order = [](const C& a, const C& b) { return a.gain != b.gain ? a.gain > b.gain : a.v < b.v; };
    if ((int64_t)top.size() > k) {
      std::nth_element(top.begin(), top.begin() + k, top.end(), heap_order);
      top.resize(k);
    }
    std::sort(top.begin(), top.end(), [&](const C& a, const C& b) {
      const int64_t wa = s.bw[s.part[a.v]], wb = s.bw[s.part[b.v]];
      if (a.gain != b.gain) return a.gain > b.gain;
      if (wa != wb) return wa > wb;
      return a.v > b.v;
    });
    for (const C& c : top) {
      if (used[c.v]) continue;
      used[c.v] = 1;
      moves.push_back({c.v, s.part[c.v], i, (int32_t)c.gain});
      break;
    }
  }
  return moves;
}

}  // namespace

extern "C" {

// The moves of repairEmptyBlocks on `part_in` (see repair_empty_blocks), in
// empty-block order; returns their number (at most k), written to
// vertices/from/to/gain (each k entries).
int32_t orc_repair_empty_blocks(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
                                const int64_t* vtx_off, const int32_t* inets, const int32_t* w_v,
                                const int32_t* w_e, int32_t k, const int64_t* lmax, const int32_t* part_in,
                                int32_t* vertices, int32_t* from, int32_t* to, int32_t* gain) {
  Hg hg = make_hg(n, m, net_off, pins, vtx_off, inets, w_v, w_e);
  State s{&hg, k, words_for(k), {}, {}, {}, {}};
  s.init(part_in);
  const std::vector<RepairMove> mv = repair_empty_blocks(s, lmax);
  for (size_t i = 0; i < mv.size(); ++i) {
    vertices[i] = mv[i].v;
    from[i] = mv[i].from;
    to[i] = mv[i].to;
    gain[i] = mv[i].gain;
  }
  return (int32_t)mv.size();
}

// Deterministic rebalancer (the device's lpgpu_session_rebalance), a
// synchronous restatement of Rebalancer::rebalance (rebalancing/rebalancer.cpp:34-171,
// whose thread-local priority queues make the reference order-dependent).
// If some block is above its max weight and some block is empty, the moves of
// repairEmptyBlocks are applied first, in their order, each as moveVertex
// does (rebalancer.h:84-103: only if the target stays within L_max and the
// source keeps weight > 0); they form a first statistics record (active = n,
// pins = P, candidates = moves proposed, moved = moves applied).
// Then per round, while some block is above its max weight:
//   * every border vertex of an overloaded block computes its Km1Policy best
//     move with rebalance = true (gain_policy.h:108-167): the feasible block
//     (c(b) + w(v) <= L_max(b), b != from) of minimum score, any sign, lowest id
//     on ties; vertices without a feasible block are no candidates;
//   * per overloaded source block b with excess X = c(b) - L_max(b): every
//     candidate with score <= 0 is taken (the reference's first pass moves all
//     non-worsening moves); candidates with score > 0, ordered by (score,
//     vertex id), are taken while the weight taken so far is below X (the
//     second pass moves worsening moves only while the block is overloaded);
//   * the taken moves go through the LP selection: per target block the
//     longest (score, vertex id) prefix within L_max, then per source block the
//     longest prefix that leaves it non-empty; they are committed with km1Delta
//     attribution.
// Stops when no block is overloaded, after max_rounds, or when a round moves
// nothing. Returns the statistics records written (the repair record, if any,
// plus the rounds executed; `stats` holds max_rounds + 1 records).
int32_t orc_rebalance(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
                      const int64_t* vtx_off, const int32_t* inets, const int32_t* w_v,
                      const int32_t* w_e, int32_t k, const int64_t* lmax, int32_t* part_inout,
                      int32_t max_rounds, orc_round_stats* stats) {
  Hg hg = make_hg(n, m, net_off, pins, vtx_off, inets, w_v, w_e);
  State s{&hg, k, words_for(k), {}, {}, {}, {}};
  s.init(part_inout);
  std::vector<int64_t> scores(k, 0);
  struct Cand { int32_t v, from, to; int64_t gain; int64_t w; };
  auto key_less = [](const Cand& a, const Cand& b) { return a.gain != b.gain ? a.gain < b.gain : a.v < b.v; };
  int32_t rec = 0;  // statistics records written
  {
    bool over = false, empty = false;
    for (int b = 0; b < k; ++b) {
      over = over || s.bw[b] > lmax[b];
      empty = empty || s.bw[b] == 0;
    }
    if (over && empty) {
      // rebalancer.cpp:59-62: repairEmptyBlocks, then moveVertex per move
      orc_round_stats st{};
      st.active = n;
      st.pins = vtx_off[n];
      const std::vector<RepairMove> mv = repair_empty_blocks(s, lmax);
      st.candidates = (int64_t)mv.size();
      for (const RepairMove& x : mv) {
        const int64_t wv = w_v[x.v];
        if (s.bw[x.to] + wv <= lmax[x.to] && s.bw[x.from] - wv > 0) {
          st.delta += s.apply_move(x.v, x.from, x.to);
          st.moved++;
        }
      }
      st.km1_after = s.km1();
      if (stats) stats[rec] = st;
      ++rec;
    }
  }
  for (int32_t r = 0; r < max_rounds; ++r) {
    bool over = false;
    for (int b = 0; b < k; ++b) over = over || s.bw[b] > lmax[b];
    if (!over) break;
    orc_round_stats st{};
    std::vector<Cand> cands;
    for (int64_t v = 0; v < n; ++v) {
      const int from = s.part[v];
      if (s.bw[from] <= lmax[from]) continue;
      st.active++;
      st.pins += vtx_off[v + 1] - vtx_off[v];
      if (!s.is_border(v)) continue;
      // rebalance best move: minimum score over feasible blocks, any sign
      int64_t internal = 0;
      for (int64_t i = vtx_off[v]; i < vtx_off[v + 1]; ++i) {
        const int64_t e = inets[i];
        if (s.phi[e * k + from] > 1) internal += w_e[e];
        for (int b = 0; b < k; ++b)
          if (b != from && bit_of(s.conn.data(), s.W, e, b)) scores[b] -= w_e[e];
      }
      int to = from;
      int64_t best = 0;
      for (int b = 0; b < k; ++b) {
        if (b != from && s.bw[b] + w_v[v] <= lmax[b]) {
          const int64_t sc = scores[b] + internal;
          if (to == from || sc < best) {
            to = b;
            best = sc;
          }
        }
        scores[b] = 0;
      }
      if (to != from) cands.push_back({(int32_t)v, from, to, best, w_v[v]});
    }
    st.candidates = (int64_t)cands.size();
    std::sort(cands.begin(), cands.end(), key_less);
    // source side: non-worsening moves always, worsening ones while needed
    std::vector<int64_t> taken(k, 0);
    for (const Cand& c : cands)
      if (c.gain <= 0) taken[c.from] += c.w;
    std::vector<Cand> src;
    for (const Cand& c : cands) {
      if (c.gain <= 0) {
        src.push_back(c);
      } else if (taken[c.from] < s.bw[c.from] - lmax[c.from]) {
        taken[c.from] += c.w;
        src.push_back(c);
      }
    }
    // LP selection: target-side prefix, then source-side prefix keeping blocks non-empty
    std::vector<int64_t> in(k, 0), out(k, 0);
    std::vector<uint8_t> stop_in(k, 0), stop_out(k, 0), ok(src.size(), 0);
    for (size_t i = 0; i < src.size(); ++i) {
      const Cand& c = src[i];
      if (stop_in[c.to]) continue;
      if (s.bw[c.to] + in[c.to] + c.w <= lmax[c.to]) {
        in[c.to] += c.w;
        ok[i] = 1;
      } else {
        stop_in[c.to] = 1;
      }
    }
    for (size_t i = 0; i < src.size(); ++i) {
      if (!ok[i]) continue;
      const Cand& c = src[i];
      if (stop_out[c.from]) { ok[i] = 0; continue; }
      if (s.bw[c.from] - out[c.from] - c.w >= 1) {
        out[c.from] += c.w;
      } else {
        stop_out[c.from] = 1;
        ok[i] = 0;
      }
    }
    for (size_t i = 0; i < src.size(); ++i) {
      if (!ok[i]) continue;
      st.delta += s.apply_move(src[i].v, src[i].from, src[i].to);
      st.moved++;
    }
    st.km1_after = s.km1();
    if (stats) stats[rec] = st;
    ++rec;
    if (st.moved == 0) break;
  }
  std::memcpy(part_inout, s.part.data(), sizeof(int32_t) * n);
  return rec;
}

// Reference-style asynchronous LP (label_propagation_refiner.{h,cpp}):
// std::threads, shuffled active set, per-net spinlocks around pin-count
// updates, atomic block weights with rollback, per-thread precomputed coin
// flips for ties (randomize.h:56-64), zero-gain rebalancing moves, realised
// gain check with revert, and neighbour activation through small nets.
// `perfect` holds the perfect block weights (context.cpp:237-250).
int32_t orc_lp_async(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
                     const int64_t* vtx_off, const int32_t* inets, const int32_t* w_v,
                     const int32_t* w_e, int32_t k, const int64_t* lmax, const int64_t* perfect,
                     int32_t* part_inout, const orc_lp_cfg* cfg, orc_round_stats* stats) {
  const int W = words_for(k);
  const int nthreads = std::max(1, cfg->threads);
  const int64_t T = cfg->activation_threshold <= 0 ? INT64_MAX : cfg->activation_threshold;
  std::vector<std::atomic<int32_t>> part(n);
  std::vector<std::atomic<int32_t>> phi(static_cast<size_t>(m) * k);
  std::vector<std::atomic<uint32_t>> conn(static_cast<size_t>(m) * W);
  std::vector<std::atomic<int64_t>> bw(k);
  std::vector<std::atomic_flag> locks(m);
  for (auto& l : locks) l.clear();
  {
    Hg hg = make_hg(n, m, net_off, pins, vtx_off, inets, w_v, w_e);
    State s{&hg, k, W, {}, {}, {}, {}};
    s.init(part_inout);
    for (int64_t v = 0; v < n; ++v) part[v].store(s.part[v], std::memory_order_relaxed);
    for (size_t i = 0; i < s.phi.size(); ++i) phi[i].store(s.phi[i], std::memory_order_relaxed);
    for (size_t i = 0; i < s.conn.size(); ++i) conn[i].store(s.conn[i], std::memory_order_relaxed);
    for (int b = 0; b < k; ++b) bw[b].store(s.bw[b], std::memory_order_relaxed);
  }
  auto conn_of = [&](int64_t e) {
    int c = 0;
    for (int w = 0; w < W; ++w) c += __builtin_popcount(conn[e * W + w].load(std::memory_order_relaxed));
    return c;
  };
  // per-thread random state (randomize.h: mt19937 seeded seed+i, 128 precomputed coins)
  struct Rand {
    std::mt19937 gen;
    std::vector<uint8_t> coins;
    size_t next = 0;
    bool flip() { return coins[++next % coins.size()]; }
  };
  std::vector<Rand> rands(nthreads);
  for (int t = 0; t < nthreads; ++t) {
    rands[t].gen.seed((uint32_t)(cfg->seed + t));
    std::uniform_int_distribution<int> d(0, 1);
    rands[t].coins.resize(128);
    for (auto& c : rands[t].coins) c = (uint8_t)d(rands[t].gen);
  }
  std::vector<int32_t> active(n);
  for (int64_t v = 0; v < n; ++v) active[v] = (int32_t)v;
  std::vector<std::atomic<uint8_t>> next_flag(n);
  std::vector<uint8_t> visited(m, 0);
  int32_t r = 0;
  for (; r < cfg->rounds; ++r) {
    if (active.empty()) break;
    auto t0 = std::chrono::steady_clock::now();
    for (auto& f : next_flag) f.store(0, std::memory_order_relaxed);
    std::fill(visited.begin(), visited.end(), 0);
    std::shuffle(active.begin(), active.end(), rands[0].gen);
    std::atomic<int64_t> cursor{0};
    std::vector<std::vector<int32_t>> next_lists(nthreads);
    std::vector<orc_round_stats> tst(nthreads);
    auto worker = [&](int t) {
      std::vector<int64_t> scores(k, 0);
      Rand& rnd = rands[t];
      orc_round_stats& st = tst[t];
      int64_t local_delta = 0;
      auto change = [&](int64_t v, int from, int to) -> bool {
        const int64_t wv = w_v[v];
        const int64_t to_after = bw[to].fetch_add(wv, std::memory_order_relaxed) + wv;
        const int64_t from_after = bw[from].fetch_sub(wv, std::memory_order_relaxed) - wv;
        if (to_after <= lmax[to] && from_after > 0) {
          part[v].store(to, std::memory_order_relaxed);
          for (int64_t i = vtx_off[v]; i < vtx_off[v + 1]; ++i) {
            const int64_t e = inets[i];
            while (locks[e].test_and_set(std::memory_order_acquire)) {}
            const int32_t fa = phi[e * k + from].fetch_sub(1, std::memory_order_relaxed) - 1;
            if (fa == 0) conn[e * W + (from >> 5)].fetch_xor(1u << (from & 31), std::memory_order_relaxed);
            const int32_t ta = phi[e * k + to].fetch_add(1, std::memory_order_relaxed) + 1;
            if (ta == 1) conn[e * W + (to >> 5)].fetch_xor(1u << (to & 31), std::memory_order_relaxed);
            locks[e].clear(std::memory_order_release);
            local_delta += (ta == 1 ? w_e[e] : 0) + (fa == 0 ? -(int64_t)w_e[e] : 0);
          }
          return true;
        }
        bw[to].fetch_sub(wv, std::memory_order_relaxed);
        bw[from].fetch_add(wv, std::memory_order_relaxed);
        return false;
      };
      for (;;) {
        const int64_t begin = cursor.fetch_add(256);
        if (begin >= (int64_t)active.size()) break;
        const int64_t end = std::min<int64_t>(begin + 256, (int64_t)active.size());
        for (int64_t j = begin; j < end; ++j) {
          const int64_t v = active[j];
          st.active++;
          st.pins += vtx_off[v + 1] - vtx_off[v];
          // isBorderNode
          const int64_t deg = vtx_off[v + 1] - vtx_off[v];
          bool border = false;
          if (deg <= kHighDegreeThreshold)
            for (int64_t i = vtx_off[v]; i < vtx_off[v + 1] && !border; ++i)
              border = conn_of(inets[i]) > 1;
          if (!border) continue;
          // computeMaxGainMoveImpl with random tie-breaking
          const int from = part[v].load(std::memory_order_relaxed);
          int64_t internal = 0;
          for (int64_t i = vtx_off[v]; i < vtx_off[v + 1]; ++i) {
            const int64_t e = inets[i];
            const int64_t we = w_e[e];
            if (phi[e * k + from].load(std::memory_order_relaxed) > 1) internal += we;
            for (int w = 0; w < W; ++w) {
              uint32_t bits = conn[e * W + w].load(std::memory_order_relaxed);
              while (bits) {
                const int b = w * 32 + __builtin_ctz(bits);
                bits &= bits - 1;
                if (b != from) scores[b] -= we;
              }
            }
          }
          int to = from;
          int64_t best = 0;
          const int64_t wv = w_v[v];
          for (int b = 0; b < k; ++b) {
            if (b != from) {
              const int64_t score = scores[b] + internal;
              const bool nb = score < best || (score == best && rnd.flip());
              if (nb && bw[b].load(std::memory_order_relaxed) + wv <= lmax[b]) {
                to = b;
                best = score;
              }
            }
            scores[b] = 0;
          }
          const bool positive = best < 0;
          const bool zero_gain = best == 0 &&
              bw[from].load(std::memory_order_relaxed) - 1 > bw[to].load(std::memory_order_relaxed) + 1 &&
              bw[to].load(std::memory_order_relaxed) < perfect[to];
          if (to == from || !(positive || zero_gain)) continue;
          st.candidates++;
          const int64_t before = local_delta;
          if (!change(v, from, to)) continue;
          const int64_t realised = local_delta - before;
          if (realised == best || realised <= 0) {
            st.moved++;
            for (int64_t i = vtx_off[v]; i < vtx_off[v + 1]; ++i) {
              const int64_t e = inets[i];
              if (net_off[e + 1] - net_off[e] <= T && !visited[e]) {
                for (int64_t q = net_off[e]; q < net_off[e + 1]; ++q) {
                  uint8_t exp = 0;
                  if (next_flag[pins[q]].compare_exchange_strong(exp, 1)) next_lists[t].push_back(pins[q]);
                }
                visited[e] = 1;
              }
            }
            uint8_t exp = 0;
            if (next_flag[v].compare_exchange_strong(exp, 1)) next_lists[t].push_back((int32_t)v);
          } else {
            st.reverted++;
            change(v, to, from);
          }
        }
      }
      st.delta = local_delta;
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(worker, t);
    worker(0);
    for (auto& th : pool) th.join();
    orc_round_stats st{};
    active.clear();
    for (int t = 0; t < nthreads; ++t) {
      st.active += tst[t].active;
      st.pins += tst[t].pins;
      st.candidates += tst[t].candidates;
      st.moved += tst[t].moved;
      st.reverted += tst[t].reverted;
      st.delta += tst[t].delta;
      active.insert(active.end(), next_lists[t].begin(), next_lists[t].end());
    }
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    int64_t km1 = 0;
    for (int64_t e = 0; e < m; ++e) km1 += (int64_t)std::max(conn_of(e) - 1, 0) * w_e[e];
    st.km1_after = km1;
    if (stats) stats[r] = st;
  }
  for (int64_t v = 0; v < n; ++v) part_inout[v] = part[v].load(std::memory_order_relaxed);
  return r;
}

}  // extern "C"
