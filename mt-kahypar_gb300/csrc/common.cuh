// Internal declarations shared by the device translation units of liblpgpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "lpgpu.h"

namespace lpgpu {

// Thread-local last-error text (lpgpu_last_error).
void set_error(const std::string& msg);

// Vertices of degree above this threshold are never border vertices
// (PartitionedHypergraph::HIGH_DEGREE_THRESHOLD, partitioned_hypergraph.h:67).
constexpr int64_t kHighDegree = 100000;

// Sub-rounds are assigned per aligned chunk of 32 consecutive vertex ids.
constexpr int kChunkShift = 5;
constexpr int kMaxSubrounds = 64;
// Classes inside a sub-round's active list (see k_bin_count): heavy
// vertices, then LPGPU_DEG_CLASSES - 1 degree classes (at least one).
#ifndef LPGPU_DEG_CLASSES
#define LPGPU_DEG_CLASSES 3
#endif
constexpr int kDegClasses = LPGPU_DEG_CLASSES;
static_assert(kDegClasses >= 2, "the heavy class and at least one other");
// Log2 buckets of the upload-time degree histogram.
constexpr int kDegBuckets = 32;
// Above this degree the warp windows of the k > 128 sweep hand a vertex to a whole CTA.
constexpr int kHeavyDegree = 1024;

// Whether the sweep evaluates a vertex of degree d with a whole CTA (heavy)
// instead of its own lane (k <= 128: summed net weight reaches the 2^planes
// of the lane counters) or a warp window (k > 128). Vertices above
// kHighDegree are never border vertices and are not evaluated at all.
__host__ __device__ inline bool sweep_heavy(int64_t d, int W, int unit_nets, int max_we) {
  if (d <= 0 || d > kHighDegree) return false;
  return W <= 4 ? d * max_we >= (int64_t(1) << (unit_nets ? 6 : 8)) : d > kHeavyDegree;
}

// Sub-round of vertex v in round r: mix32((v >> 5) ^ (0x9E3779B9 * (r + 1))) % S.
__host__ __device__ inline uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
__host__ __device__ inline int subround_of(int64_t v, int round, int S) {
  if (S <= 1) return 0;
  return (int)(mix32((uint32_t)(v >> kChunkShift) ^ (0x9E3779B9u * (uint32_t)(round + 1))) %
               (uint32_t)S);
}

// Candidate ordering key: (gain, vertex) as one unsigned 64-bit integer. The
// gain maps to (gain - 1) XOR 2^31, which keeps the order of every gain above
// INT32_MIN (gains stay within +-INT32_MAX) and sends the non-positive gains of
// LP candidates (-d .. 0) to 0x7FFFFFFF - d .. 0x7FFFFFFF: a segment mixing
// improving and zero-gain moves then differs only in the gain's low byte(s),
// and the radix selection skips the constant ones.
__host__ __device__ inline uint64_t move_key(int32_t gain, int32_t v) {
  return ((uint64_t)((uint32_t)((int64_t)gain - 1) ^ 0x80000000u) << 32) | (uint32_t)v;
}

// Indices into the device scalar block.
enum Scalar : int {
  kDeltaSub = 0,   // summed attributed delta of the current sub-round
  kAnyOverTo = 1,  // some target block overflows
  kAnyOverFrom = 2,
  kKm1 = 3,        // km1 accumulator (metrics)
  kCut = 4,        // cut accumulator (metrics)
  kError = 5,      // device-side error flag
  kApplyDelta = 6, // apply_moves delta
  kDeltaRb = 7,    // delta of a sub-round rollback
  kEpoch = 8,      // activation stamp of the current round
  kDone = 9,       // arrival counter of the last-CTA pattern
  kOverCount = 10, // number of overflowing target blocks
  kHeavyCount = 11, // heavy vertices a per-vertex query deferred to k_sweep_heavy
  kRevCount = 12,  // moves marked for revert in the current sub-round
  kPxQueue = 13,   // work queue counter of a persistent round
  kScalars = 16
};

using ull = unsigned long long;

// Result words of the device-side input checks (validate.cu): the first
// failure code, the largest net weight, whether some net weight is not 1,
// then I per-instance sums of |e|·w(e) and I per-instance vertex weights.
enum ValidateWord : int { kVErr = 0, kVMaxWe = 1, kVNonUnit = 2, kVMaxSize = 3, kVSums = 4 };
enum ValidateCode : int {
  kVOk = 0,
  kVBadOffsets = 1,
  kVNegNetWeight = 2,
  kVPinRange = 3,
  kVNegVertexWeight = 4,
  kVBlockRange = 5
};

// Per-round statistics slots (lpgpu_round_stats order).
enum Stat : int {
  kStActive = 0,
  kStPins,
  kStCands,
  kStMoved,
  kStReverted,
  kStDelta,
  kStMovedPins,  // incidences of the moves k_commit applied (before reverts and rollbacks)
  kStToggles,    // Λ bits k_commit changed
  kStats = 8
};

// Device pointers of the round kernels.
struct RoundCtx {
  int64_t n, m;
  int32_t k, W;
  const int64_t* net_off;
  const int32_t* pins;
  const int64_t* vtx_off;
  const int32_t* inets;
  const int32_t* w_v;
  const int32_t* w_e;
  int32_t* part;
  int32_t* phi;          // Φ(e, b) at e * kmax + b: 16-bit entries when phi16, else 32-bit (phi_get / phi_add)
  uint32_t* conn;        // m x 2W words: Λ(e) (W words), then Λ1(e) (W words)
  int64_t* bw;
  const int64_t* lmax;
  const int64_t* perfect;
  // active lists
  int32_t* list;
  int64_t* sub_off;      // S + 1 offsets into list, then per sub-round the end of its heavy vertices
  uint8_t* next_flag;    // n
  int32_t* net_epoch;    // m: round stamp of nets to expand
  // per list position
  int4* rec;             // (to, gain, vertex, from), global blocks; to < 0: no candidate
  uint8_t* status;       // 0 none, 1 moved, 2 reverted, 3 rolled back
  // per block scratch
  int64_t* in_w;         // candidate weight by target block (sweep)
  int64_t* in_cnt;       // candidate count by target block (sweep)
  int64_t* cand_out;     // candidate weight by source block (sweep)
  int64_t* acc_w;        // target-accepted weight by source block
  int64_t* acc_cnt;      // target-accepted count by source block
  int64_t* seg_off;      // k + 1
  int64_t* cursor;
  uint64_t* thr_to;
  uint64_t* thr_from;
  uint8_t* over_to;
  uint8_t* over_from;
  uint64_t* seg_key;     // n
  int32_t* seg_w;        // n
  int64_t* scal;         // kScalars
  int64_t* stats;        // rounds x kStats
  // parameters
  int32_t zero_gain, revert, rollback;
  int32_t unit_nets;     // every net weight is 1
  int32_t phi16;         // every net has fewer than 2^16 pins: Φ entries are 16 bits
  int32_t max_we;        // largest net weight (0 without nets)
  int64_t act_threshold;
  int32_t heavy_share;   // per mille of the sweep's work in heavy vertices (0: none can exist)
  // batched sessions: many independent instances in one union hypergraph.
  // part[] holds global block ids (instance block offset + local id); Φ and
  // Λ are indexed by local ids. One instance: batched = 0, kmax = k.
  int32_t batched;
  int32_t kmax;           // Φ row stride and largest instance k
  int32_t num_inst;
  const int32_t* vinst;     // instance of each vertex
  const int64_t* inst_voff; // first vertex of each instance (num_inst + 1)
  const int32_t* inst_boff; // first global block of each instance
  const int32_t* inst_k;    // blocks of each instance
  int64_t* inst_delta;      // per-instance summed delta of the current sub-round
  int32_t* over_ids;        // target blocks that overflow (count in scal[kOverCount])
  int32_t* heavy;           // vertices a per-vertex query deferred (count in scal[kHeavyCount])
  int32_t* revl;            // list positions of moves marked for revert (count in scal[kRevCount])
};

#ifndef LPGPU_PHI16
#define LPGPU_PHI16 1  // 0: 32-bit Φ entries always
#endif

// Φ(e, b) at index i = e * kmax + b. With 16-bit entries two share a 32-bit
// word; an atomic add of d << 16 * (i & 1) changes one entry only, since an
// entry never leaves [0, 2^16): the counts stay at most |e| < 2^16 and only
// counts of at least 1 are decremented.
__device__ __forceinline__ int phi_get(const RoundCtx& c, int64_t i) {
  return c.phi16 ? (int)reinterpret_cast<const uint16_t*>(c.phi)[i] : c.phi[i];
}
__device__ __forceinline__ void phi_set(const RoundCtx& c, int64_t i, int v) {
  if (c.phi16)
    reinterpret_cast<uint16_t*>(c.phi)[i] = (uint16_t)v;
  else
    c.phi[i] = v;
}
// Adds d (+1 or -1) to Φ at i and returns the count before.
__device__ __forceinline__ int phi_add(const RoundCtx& c, int64_t i, int d) {
  if (c.phi16) {
    const int sh = (int)(i & 1) * 16;
    const uint32_t old = atomicAdd(reinterpret_cast<uint32_t*>(c.phi) + (i >> 1), (uint32_t)d << sh);
    return (int)((old >> sh) & 0xFFFFu);
  }
  return atomicAdd(&c.phi[i], d);
}

// Global block offset of vertex v's instance.
__device__ __forceinline__ int block_offset(const RoundCtx& c, int64_t v) {
  return c.batched ? c.inst_boff[c.vinst[v]] : 0;
}

// Kernels launched by this thread through the library so far.
int64_t kernel_launches();
// Adjusts the count (graph capture records kernels without running them;
// each graph replay runs them).
void add_kernel_launches(int64_t n);

// Launch helpers (lp_kernels.cu). All launch on `st`; none synchronizes.
struct Launch {
  cudaStream_t st;
  int num_sms;
};

cudaError_t scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t count, int64_t* tmp,
                               int64_t tmp_elems, cudaStream_t st);
int64_t scan_tmp_elems(int64_t count);

cudaError_t launch_build_incidence(const Launch& L, int64_t n, int64_t m, int64_t P, const int64_t* net_off,
                                   const int32_t* pins, int64_t* vtx_off, int32_t* inets,
                                   int32_t* rank, int64_t* scan_tmp, int64_t scan_tmp_elems,
                                   int64_t* deg_hist);
cudaError_t launch_init_partition(const Launch& L, const RoundCtx& c);
cudaError_t launch_metrics(const Launch& L, const RoundCtx& c);
cudaError_t launch_instance_metrics(const Launch& L, const RoundCtx& c, int64_t* km1_inst);
cudaError_t launch_best_moves(const Launch& L, const RoundCtx& c, int32_t* to, int32_t* gain,
                              uint8_t* border);
cudaError_t launch_gain_cache(const Launch& L, const RoundCtx& c, int32_t* benefit,
                              int32_t* penalty);
// Device-resident gain cache maintained by apply_moves (all null: none).
struct GainCache {
  int32_t* benefit;  // n: moveFromBenefit
  int32_t* penalty;  // n x k: moveToPenalty
  uint8_t* moved;    // n: zero outside apply_moves
};
cudaError_t launch_apply_moves(const Launch& L, const RoundCtx& c, int64_t count,
                               const int32_t* v, const int32_t* from, const int32_t* to, const GainCache& g);

// Device-side input checks (validate.cu). `out` holds kVSums + 2 I words;
// `inst_voff`, `inst_noff` and `inst_poff` (each instance's pin range,
// non-decreasing from 0 to P) are read when I > 1; `vinst` (batched
// sessions, null otherwise) receives every vertex's instance.
cudaError_t launch_validate_csr(const Launch& L, int64_t n, int64_t m, int64_t P, const int64_t* net_off,
                                const int32_t* pins, const int32_t* w_v, const int32_t* w_e, int I,
                                const int64_t* inst_voff, const int64_t* inst_noff, const int64_t* inst_poff,
                                int32_t* vinst, int64_t* out);
// Checks the partition ids in `part` (device) against k, or per instance when
// `vinst` is given, and turns local ids into global ones.
cudaError_t launch_check_partition(const Launch& L, int64_t n, int32_t* part, int k, const int32_t* vinst,
                                   const int32_t* inst_boff, const int32_t* inst_k, int64_t* out);

// Batches uploaded one instance at a time (validate.cu): instance i's local
// pins and net offsets, copied into place, are shifted to union ids.
// Instance-local vertex ids and pin offsets to union ones; with `staged`, the
// instances' offset arrays (m_i + 1 entries each, back to back) are moved into
// net_off first.
cudaError_t launch_rebase_instances(const Launch& L, int I, const int64_t* inst_voff, const int64_t* inst_noff,
                                    const int64_t* inst_poff, int64_t* net_off, int32_t* pins,
                                    const int64_t* staged);
cudaError_t launch_fill_ones(const Launch& L, int32_t* p, int64_t count);
// Multilevel projection: part[v] = coarse_part[map[v]]; *check != 0 when a
// map entry lies outside [0, nc).
cudaError_t launch_project(const Launch& L, int64_t n, const int32_t* map, const int32_t* coarse_part, int64_t nc,
                           int32_t* part, int64_t* check);
// Global block ids of a batch back to instance-local ids.
cudaError_t launch_local_blocks(const Launch& L, int64_t n, const int32_t* part, const int32_t* vinst,
                                const int32_t* inst_boff, int32_t* out);

// Round phases (the sub-round pipeline). `timer` may be null.
struct PhaseTimer;
cudaError_t launch_mark_all(const Launch& L, const RoundCtx& c, int rebalancing);
cudaError_t launch_mark_list(const Launch& L, const RoundCtx& c, const int32_t* nodes,
                             int64_t count);
// bin_cnt: 2 * kMaxSubrounds * kDegClasses entries, the first half zero
cudaError_t launch_bin_active(const Launch& L, const RoundCtx& c, int round, int S, int64_t* bin_cnt,
                              PhaseTimer* timer);
cudaError_t launch_subround(const Launch& L, const RoundCtx& c, int round, int sub, PhaseTimer* timer);
// End of a round that has a successor: activation of the kept moves
// (moveVertex, label_propagation_refiner.h:112-128) and expansion of the
// stamped nets into the next round's active set.
cudaError_t launch_expand_nets(const Launch& L, const RoundCtx& c, int S, PhaseTimer* timer);

// One round of the deterministic rebalancer on a single-instance session
// whose list is the identity over all vertices (sub_off = {0, n}). rb_to /
// rb_score: n-entry scratch; rb: 5k + 1 int64 scratch.
cudaError_t launch_rebalance_round(const Launch& L, const RoundCtx& c, int round, int32_t* rb_to,
                                   int32_t* rb_score, int64_t* rb);
// Empty-block repair candidates of block `blk` on a single-instance session:
// the (at most k) vertices the reference's bounded heap keeps, as (vertex,
// gain, block, weight) records in `out`; scratch[0] receives their number.
// keys / ws: n-entry scratch; scratch: 2 int64.
cudaError_t launch_repair_candidates(const Launch& L, const RoundCtx& c, int blk, uint64_t* keys, int32_t* ws,
                                     int4* out, int64_t* scratch);

// ---- persistent rounds (one launch per LP round of a batch of small instances)

// Largest k of an instance the persistent round kernel takes (Λ records of
// at most 2 words).
constexpr int kPxMaxK = 64;

// One instance of a persistent round. Arrays are indexed by the ids the
// instance's CSR stores (union ids in a batched session), so several
// instances may share one set of arrays; keys / kw / cand hold v1 - v0
// entries of per-instance scratch starting at their pointer.
struct PxInst {
  const int64_t* net_off;
  const int32_t* pins;
  const int64_t* vtx_off;
  const int32_t* inets;
  const int32_t* w_v;
  const int32_t* w_e;
  int32_t* part;        // global block ids: boff + local id
  int32_t* phi;
  uint32_t* conn;
  int64_t* bw;          // block weights at [boff, boff + k)
  const int64_t* lmax;
  const int64_t* perfect;
  uint8_t* flag;        // bit 0: active this round, bit 1: active next round
  int4* rec;            // per vertex: (to, gain, -, from) of its candidate move
  uint8_t* status;      // per vertex: 1 committed, 2 reverted, 3 rolled back
  uint64_t* keys;       // selection keys (scratch)
  int32_t* kw;          // selection weights (scratch)
  int32_t* cand;        // the sub-round's candidates as local ids (scratch)
  int32_t* net_epoch;   // round stamp of nets whose pins were activated
  int64_t* stats;       // kStats counters per round, round r at r * kStats (added to)
  int64_t v0, v1;
  int32_t boff, k;
  int32_t kstride;      // Φ row length
  int32_t W;            // Λ words per record half (1 or 2)
  int32_t unit_nets, phi16, max_we;
  int32_t round;        // round of this instance (when the launch does not set one)
};

struct PxParams {
  int32_t S, zero_gain, revert, rollback;
  int64_t act_threshold;
  int32_t round;        // >= 0: every instance runs this round; < 0: its own `round`
  int32_t unroll;       // incidences per lane step of the sweep (4 or 8)
};

// Runs one LP round of `count` instances, taken in `order` (null:
// 0..count-1) from the work queue counter `queue` (zeroed here). W: Λ words
// class of all instances (1 or 2); unit: every net weight is 1; ctas_per_sm:
// the 1- or 2-CTA-per-SM build of the kernel.
cudaError_t launch_px_round(const Launch& L, const PxInst* insts, const int32_t* order, int32_t count,
                            const PxParams& P, int W, bool unit, int ctas_per_sm, int64_t* queue);
// out[i]: active vertices of instance i's round `insts[i].round` (from its statistics).
cudaError_t launch_px_active(const Launch& L, const PxInst* insts, int32_t count, int64_t* out);

// Optional per-phase CUDA-event timing.
struct PhaseTimer {
  struct Rec {
    int phase;
    cudaEvent_t a, b;
  };
  std::vector<std::string> names;
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  cudaStream_t st = nullptr;
  int phase_id(const char* name);
  void begin(int phase, cudaEvent_t* a);
  void end(int phase, cudaEvent_t a);
  void reset();
  ~PhaseTimer();
};

}  // namespace lpgpu
