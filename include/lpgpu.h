/*
 * lpgpu.h -- C ABI of the GB300-native label-propagation (km1) refinement path.
 *
 * The reference (Mt-KaHyPar) exposes this phase only in C++, through
 *   IRefiner::initialize / IRefiner::refine
 *     (mt-kahypar/partition/refinement/i_refiner.h:45-53),
 *   created by LabelPropagationFactory
 *     (mt-kahypar/partition/factories.h:60-61,
 *      mt-kahypar/partition/registries/register_refinement_algorithms.cpp:35-40),
 * and operates on PartitionedHypergraph
 *     (mt-kahypar/datastructures/partitioned_hypergraph.h:44-1201).
 * Its public C API (include/libkahypar.h:58-86) has no refine-only entry point,
 * so the entry points below are what an FFI binding of that phase binds. Each
 * declaration names the reference interface it replaces.
 *
 * Conventions
 *   - All ids are int32 (vertices, nets, blocks); CSR offsets are int64.
 *   - A pin listed twice in one net counts twice (the reference's
 *     construction does not deduplicate either).
 *   - Host pointers are caller-owned and only read/written during the call.
 *   - Device state lives in an opaque session; every call returns a status.
 *   - There is no CPU fallback: without a usable CUDA device every call that
 *     needs one returns LPGPU_ERR_NO_DEVICE.
 *   - A session is not reentrant: calls on one session must not overlap.
 *     Distinct sessions may be used from distinct threads.
 */
#ifndef LPGPU_H_
#define LPGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define LPGPU_API __attribute__((visibility("default")))
#else
#define LPGPU_API
#endif

typedef enum {
  LPGPU_OK = 0,
  LPGPU_ERR_INVALID_ARG = 1,   /* malformed CSR, ids out of range, k too large ... */
  LPGPU_ERR_OOM = 2,           /* device allocation failed */
  LPGPU_ERR_ADMISSION = 3,     /* request does not fit the configured memory budget */
  LPGPU_ERR_TIMEOUT = 4,       /* a bounded device wait gave up */
  LPGPU_ERR_CUDA = 5,          /* any other CUDA runtime error */
  LPGPU_ERR_NO_DEVICE = 6,     /* no CUDA device, or the library was not built for it */
  LPGPU_ERR_STATE = 7          /* call order violated (e.g. refine before set_partition) */
} lpgpu_status;

/* Largest number of blocks the device path supports. */
#define LPGPU_MAX_K 1024

/* LP parameters. Mirrors Context::refinement.label_propagation
 * (mt-kahypar/partition/context.h:119-125) plus the synchronous-round knobs.
 * lpgpu_config_default() fills the fast_preset.ini values
 * (config/fast_preset.ini:57-61): 5 rounds, rebalancing on, activation
 * threshold 100. */
typedef struct {
  int32_t rounds;               /* maximum_iterations */
  int32_t activation_threshold; /* hyperedge_size_activation_threshold; <= 0 means no limit */
  int32_t rebalancing;          /* 1: all vertices start active and zero-gain rebalancing
                                   moves are allowed; 0: border vertices start active */
  int32_t subrounds;            /* sub-rounds per round (>= 1; default 7) */
  int32_t revert;               /* 1: undo moves whose reverse now strictly improves km1 */
  int32_t rollback;             /* 1: undo a sub-round whose summed delta is positive */
  int32_t flags;                /* LPGPU_FLAG_* */
  int32_t reserved1;
} lpgpu_config;

/* lpgpu_config.flags: launch the refine directly instead of capturing it once
 * as a CUDA graph and replaying it (useful when every call has new sizes). */
#define LPGPU_FLAG_NO_GRAPH 1
/* lpgpu_config.flags: run the refine as one persistent launch per round (every
 * CTA refines whole instances taken from a device work queue), or force the
 * multi-launch sub-round pipeline. Without either flag the session's tuning
 * decides (lpgpu_session_set_tuning, else the process-wide tuning table).
 * The persistent form needs every instance's k <= LPGPU_PERSISTENT_MAX_K and
 * no explicit refinement node list; otherwise the refine returns
 * LPGPU_ERR_INVALID_ARG when it is forced and takes the multi-launch form
 * when it is only tuned. Both forms give identical results. */
#define LPGPU_FLAG_PERSISTENT 2
#define LPGPU_FLAG_MULTI_LAUNCH 4
#define LPGPU_PERSISTENT_MAX_K 64

/* How a refine runs (the knobs the autotuner searches). */
typedef enum {
  LPGPU_MODE_MULTI_LAUNCH = 0, /* the sub-round pipeline over the whole (union) hypergraph */
  LPGPU_MODE_PERSISTENT = 1    /* one launch per round, instances as work items */
} lpgpu_mode;

typedef struct {
  int32_t mode;        /* lpgpu_mode */
  int32_t ctas_per_sm; /* persistent: resident CTAs per SM (1: up to 128 registers, 2: up to 64) */
  int32_t unroll;      /* persistent: incidences per lane step of the sweep (4 or 8) */
  int32_t order;       /* persistent: 0 largest instance first, 1 instance order */
} lpgpu_tuning;

/* One row of the tuning table: applies to a refine whose session holds at
 * least min_instances instances of at most max_mean_pins pins on average. */
typedef struct {
  int64_t max_mean_pins;
  int32_t min_instances;
  int32_t reserved;
  lpgpu_tuning tuning;
} lpgpu_tuning_entry;

/* Result of one refine call. Mirrors the kahypar::Metrics update done in
 * LabelPropagationRefiner::refineImpl (label_propagation_refiner.cpp:48-67). */
typedef struct {
  int64_t km1_before;
  int64_t km1_after;      /* recomputed from the device connectivity sets */
  int64_t delta;          /* sum of attributed objective deltas (km1_after - km1_before) */
  int64_t moves;          /* committed moves kept at the end */
  int64_t pins_processed; /* sum over rounds of sum of degrees of swept vertices */
  int32_t rounds;         /* rounds executed */
  int32_t improved;       /* IRefiner::refine return value: delta < 0 */
  double imbalance;       /* metrics::imbalance after refinement */
} lpgpu_result;

/* Per-round statistics. */
typedef struct {
  int64_t active;      /* vertices swept */
  int64_t pins;        /* sum of the degrees of the swept vertices */
  int64_t candidates;  /* vertices with a move to offer */
  int64_t moved;       /* moves kept at the end of the round */
  int64_t reverted;    /* moves undone (hindsight reverts and rolled-back sub-rounds) */
  int64_t delta;       /* summed attributed objective delta */
  int64_t moved_pins;  /* incidences of the committed moves, before reverts and rollbacks */
  int64_t toggles;     /* connectivity-set bits the commits changed */
} lpgpu_round_stats;

typedef struct lpgpu_session_s lpgpu_session;

/* ---------------------------------------------------------------- config */

/* Fills *cfg with the preset values (see lpgpu_config). */
LPGPU_API void lpgpu_config_default(lpgpu_config* cfg);

/* Human-readable name of a status code. */
LPGPU_API const char* lpgpu_status_string(lpgpu_status s);

/* Text of the last error on this thread (empty string if none). */
LPGPU_API const char* lpgpu_last_error(void);

/* ------------------------------------------------------------- one-shot */

/* Refine a partition in place: upload, initializePartition, LP rounds,
 * download. Replaces the pair LabelPropagationFactory::createObject +
 * IRefiner::refine on a PartitionedHypergraph built by
 * HypergraphFactory::construct (lib/libkahypar.cc:168-190) for this phase.
 * Max block weight follows Context::setupPartWeights (context.cpp:237-250):
 * perfect = ceil(W/k), max = (int)((1 + eps) * perfect). */
LPGPU_API lpgpu_status lpgpu_refine_km1(int64_t num_vertices, int64_t num_nets,
                                        const int64_t* net_offsets, const int32_t* pins,
                                        const int32_t* vertex_weights, /* NULL: unit */
                                        const int32_t* net_weights,    /* NULL: unit */
                                        int32_t k, double epsilon,
                                        int32_t* partition_inout,
                                        const lpgpu_config* cfg, /* NULL: defaults */
                                        lpgpu_result* result);

/* ----------------------------------------------------------- sessions */

/* Creates a session on CUDA device `device`. */
LPGPU_API lpgpu_status lpgpu_session_create(int32_t device, lpgpu_session** out);
LPGPU_API lpgpu_status lpgpu_session_destroy(lpgpu_session* s);

/* Uploads the hypergraph (net -> pins CSR) and builds the vertex -> incident
 * nets arrays on the device. Replaces StaticHypergraphFactory::construct
 * (static_hypergraph_factory.cpp:32-166). Incident-net order per vertex is
 * unspecified; nothing computed depends on it. Single-pin nets are kept. */
LPGPU_API lpgpu_status lpgpu_session_upload(lpgpu_session* s, int64_t num_vertices,
                                            int64_t num_nets, const int64_t* net_offsets,
                                            const int32_t* pins,
                                            const int32_t* vertex_weights, /* NULL: unit */
                                            const int32_t* net_weights);   /* NULL: unit */

/* Sets the block of every vertex and rebuilds block weights, pin counts and
 * connectivity sets. Replaces setOnlyNodePart for all vertices followed by
 * PartitionedHypergraph::initializePartition (partitioned_hypergraph.h:522-526,
 * 693-698, 1067-1110). max_part_weights / perfect_part_weights may be NULL, in
 * which case they are derived from epsilon as in lpgpu_refine_km1. */
LPGPU_API lpgpu_status lpgpu_session_set_partition(lpgpu_session* s, int32_t k, double epsilon,
                                                   const int32_t* partition,
                                                   const int64_t* max_part_weights,
                                                   const int64_t* perfect_part_weights);

/* ------------------------------------------------------------ batches
 *
 * A batched session holds many independent hypergraphs (instances) as one
 * union: instance i owns the vertices [instance_vertex_offsets[i],
 * instance_vertex_offsets[i+1]) and the nets [instance_net_offsets[i],
 * instance_net_offsets[i+1]) of the union CSR, and every net's pins lie inside
 * its instance. Each instance has its own k, epsilon, block weights and
 * bounds. One refine call refines all instances together in the same launches,
 * and every instance ends exactly as it would if refined alone: sub-rounds are
 * assigned from instance-local vertex ids and rollbacks are decided per
 * instance. Block ids passed in and returned are instance-local. This has no
 * counterpart in the reference, which partitions one hypergraph per call. */
LPGPU_API lpgpu_status lpgpu_session_upload_batch(lpgpu_session* s, int32_t num_instances,
                                                  const int64_t* instance_vertex_offsets,
                                                  const int64_t* instance_net_offsets,
                                                  const int64_t* net_offsets, const int32_t* pins,
                                                  const int32_t* vertex_weights,
                                                  const int32_t* net_weights);

/* Per-instance k (1..LPGPU_MAX_K) and epsilon, and the instance-local block of
 * every union vertex. Bounds follow Context::setupPartWeights per instance. */
LPGPU_API lpgpu_status lpgpu_session_set_partition_batch(lpgpu_session* s, const int32_t* instance_k,
                                                         const double* instance_eps,
                                                         const int32_t* partition);

/* km1 of every instance (num_instances values; one value for a plain session). */
LPGPU_API lpgpu_status lpgpu_session_instance_km1(lpgpu_session* s, int64_t* km1);

/* One instance of a batch in its own ids: pins in [0, num_vertices), net
 * offsets from 0 (num_nets + 1 entries). Weights may be NULL (unit). */
typedef struct lpgpu_instance {
  int64_t num_vertices;
  int64_t num_nets;
  const int64_t* net_offsets;
  const int32_t* pins;
  const int32_t* vertex_weights;
  const int32_t* net_weights;
} lpgpu_instance;

/* lpgpu_session_upload_batch from one buffer set per instance (for example
 * one per served request): no union is built on the host; every instance is
 * copied into place and shifted to union ids on the device. */
LPGPU_API lpgpu_status lpgpu_session_upload_instances(lpgpu_session* s, int32_t num_instances,
                                                      const lpgpu_instance* instances);

/* lpgpu_session_set_partition_batch with one instance-local partition array
 * per instance. */
LPGPU_API lpgpu_status lpgpu_session_set_partition_instances(lpgpu_session* s, const int32_t* instance_k,
                                                             const double* instance_eps,
                                                             const int32_t* const* partitions);

/* Instance-local blocks of every instance, one output array per instance. */
LPGPU_API lpgpu_status lpgpu_session_get_partition_instances(lpgpu_session* s, int32_t* const* partitions);

/* ------------------------------------------------------------ files
 *
 * hMetis hypergraph files, read as io::readHypergraphFile does
 * (mt-kahypar/io/hypergraph_io.cpp:95-333; mt_kahypar_read_hypergraph_from_file,
 * include/libkahypar.h:74-78): '%' comment lines, header "num_nets
 * num_vertices [type]" (type 1: net weights, 10: vertex weights, 11: both),
 * one net per line (weight first when present, pins 1-based), nets with fewer
 * than two pins dropped, then one weight per vertex when present. Returns
 * 0-based CSR arrays allocated with malloc (release with lpgpu_free) that
 * lpgpu_session_upload takes as they are; num_removed_single_pin_nets may be NULL. */
LPGPU_API lpgpu_status lpgpu_read_hgr(const char* path, int64_t* num_vertices, int64_t* num_nets,
                                      int64_t** net_offsets, int32_t** pins, int32_t** vertex_weights,
                                      int32_t** net_weights, int64_t* num_removed_single_pin_nets);
LPGPU_API void lpgpu_free(void* p);

/* Partition files: one block id per line (io::readPartitionFile /
 * io::writePartitionFile, hypergraph_io.cpp:336-365). */
LPGPU_API lpgpu_status lpgpu_read_partition(const char* path, int64_t num_vertices, int32_t* partition);
LPGPU_API lpgpu_status lpgpu_write_partition(const char* path, int64_t num_vertices, const int32_t* partition);

/* Runs the LP refinement on the device-resident state. Replaces
 * IRefiner::refine of LabelPropagationRefiner<Km1Policy>
 * (label_propagation_refiner.cpp:34-68). refinement_nodes (may be NULL with
 * count 0, meaning all vertices) restricts the initial active set
 * (label_propagation_refiner.cpp:200-230). */
LPGPU_API lpgpu_status lpgpu_session_refine(lpgpu_session* s, const lpgpu_config* cfg,
                                            const int32_t* refinement_nodes,
                                            int64_t num_refinement_nodes,
                                            lpgpu_result* result);

/* Process-wide tuning table (the autotuner's output, rows in priority order;
 * the first row that applies wins; count 0 clears it). Without a matching
 * row, and without a session tuning, refines use the multi-launch form. This
 * has no counterpart in the reference, which has no device code to tune. */
LPGPU_API lpgpu_status lpgpu_set_tuning_table(const lpgpu_tuning_entry* entries, int32_t count);

/* Tuning of one session (NULL: back to the table). lpgpu_session_tuning gives
 * the tuning the next refine of the session's current upload uses. */
LPGPU_API lpgpu_status lpgpu_session_set_tuning(lpgpu_session* s, const lpgpu_tuning* tuning);
LPGPU_API lpgpu_status lpgpu_session_tuning(lpgpu_session* s, lpgpu_tuning* out);

/* ------------------------------------------------------- stepped rounds
 *
 * Continuous batching at round granularity (no counterpart in the
 * reference, which refines one hypergraph per call): each request lives in
 * its own session; lpgpu_stepper_launch runs the next LP round of every
 * listed session in one persistent launch per group of equal round
 * parameters on the stepper's own stream, so sessions may join the list or
 * leave it between any two rounds, and each one ends exactly as
 * lpgpu_session_refine would leave it. The stepper's stream waits for the
 * work each session enqueued before the launch, and each session's stream
 * waits for the round, so uploads and downloads of other sessions overlap
 * with it. */
typedef struct lpgpu_stepper_s lpgpu_stepper;

LPGPU_API lpgpu_status lpgpu_stepper_create(int32_t device, lpgpu_stepper** out);
LPGPU_API lpgpu_status lpgpu_stepper_destroy(lpgpu_stepper* stepper);

/* Starts a stepped refinement of the session's partition with cfg (its
 * rounds are the session's round budget): the round-0 active set, cleared
 * statistics and km1 before. Every k must be <= LPGPU_PERSISTENT_MAX_K. */
LPGPU_API lpgpu_status lpgpu_session_begin_rounds(lpgpu_session* s, const lpgpu_config* cfg);

/* Enqueues the next round of every listed session (each begun and not done,
 * listed once) and returns without waiting. */
LPGPU_API lpgpu_status lpgpu_stepper_launch(lpgpu_stepper* stepper, lpgpu_session* const* sessions,
                                            int32_t count);

/* Waits for the launched round; done[i] = 1 when session i of the launch has
 * used its round budget or its last round found no active vertex. */
LPGPU_API lpgpu_status lpgpu_stepper_wait(lpgpu_stepper* stepper, int32_t* done);

/* Ends a stepped refinement: the refine result and per-round statistics
 * (lpgpu_session_round_stats) as lpgpu_session_refine gives them. */
LPGPU_API lpgpu_status lpgpu_session_end_rounds(lpgpu_session* s, lpgpu_result* result);

/* Statistics of the last refine: up to max_rounds records, returns the count in *rounds. */
LPGPU_API lpgpu_status lpgpu_session_round_stats(lpgpu_session* s, lpgpu_round_stats* out,
                                                 int32_t max_rounds, int32_t* rounds);

/* Downloads partID for all vertices (PartitionedHypergraph::partID, h:517);
 * instance-local block ids in a batched session. */
LPGPU_API lpgpu_status lpgpu_session_get_partition(lpgpu_session* s, int32_t* partition);

/* metrics::km1 and metrics::hyperedgeCut (metrics.cpp:29-65) on the device state,
 * plus metrics::imbalance (metrics.cpp:114-128). Any output pointer may be NULL. */
LPGPU_API lpgpu_status lpgpu_session_metrics(lpgpu_session* s, int64_t* km1, int64_t* cut,
                                             double* imbalance);

/* Block weights c(V_b) (partWeight, h:599), k values. */
LPGPU_API lpgpu_status lpgpu_session_get_block_weights(lpgpu_session* s, int64_t* weights);

/* Pin counts Φ(e,b) (pinCountInPart, h:640) as a dense num_nets x k int32 array
 * (num_nets x max instance k, local block ids, in a batched session). */
LPGPU_API lpgpu_status lpgpu_session_get_pin_counts(lpgpu_session* s, int32_t* pin_counts);

/* Connectivity sets Λ(e) (connectivitySet, connectivity_set.h:53-221) as
 * num_nets x ceil(k/32) uint32 words; bit b%32 of word b/32 is block b. */
LPGPU_API lpgpu_status lpgpu_session_get_connectivity(lpgpu_session* s, uint32_t* words);

/* Vertex -> incident nets arrays built by upload (vertex_offsets: n+1 int64,
 * incident_nets: P int32). */
LPGPU_API lpgpu_status lpgpu_session_get_incidence(lpgpu_session* s, int64_t* vertex_offsets,
                                                   int32_t* incident_nets);

/* Per-vertex best move under Km1Policy::computeMaxGainMoveImpl with
 * disable_randomization = true (gain_policy.h:108-167), guarded by
 * isBorderNode (partitioned_hypergraph.h:605-620). to[v] == partID(v) and
 * gain[v] == 0 when no strictly improving feasible move exists; border[v] is
 * isBorderNode(v). Any output may be NULL. */
LPGPU_API lpgpu_status lpgpu_session_best_moves(lpgpu_session* s, int32_t* to, int32_t* gain,
                                                uint8_t* border);

/* Gain cache (initializeGainCache, partitioned_hypergraph.h:707-809):
 * benefit[v] = moveFromBenefit(v), penalty[v*k+b] = moveToPenalty(v,b), so
 * km1Gain(v,from,to) = benefit[v] - penalty[v*k+to] (h:682-688). */
LPGPU_API lpgpu_status lpgpu_session_gain_cache(lpgpu_session* s, int32_t* benefit,
                                                int32_t* penalty);

/* Uncoarsening step (uncoarsening.cpp:111-122: setOnlyNodePart of every fine
 * vertex from its coarse representative, then initializePartition,
 * partitioned_hypergraph.h:522-526, 693-698), device to device: the partition
 * of `fine` becomes part[v] = part_coarse[fine_to_coarse[v]] with the coarse
 * session's k and block bounds, and its Φ, Λ and block weights are built. Both
 * sessions are single-instance and on the same device; `fine` holds the fine
 * hypergraph, `coarse` a partition. */
LPGPU_API lpgpu_status lpgpu_session_project_partition(lpgpu_session* fine, const lpgpu_session* coarse,
                                                       const int32_t* fine_to_coarse);

/* Rebalancer (Rebalancer::rebalance, rebalancing/rebalancer.cpp:34-171) in a
 * deterministic synchronous form. Per round, while some block is above its max
 * weight: every border vertex of an overloaded block takes its Km1Policy best
 * move with rebalance = true (the feasible block of minimum score, any sign,
 * lowest id on ties); per overloaded block all non-worsening candidates are
 * taken and worsening ones, in (score, vertex id) order, only while the weight
 * taken is below the block's excess; the taken moves then go through the LP
 * selection (target-side prefix within L_max, source blocks kept non-empty)
 * and are committed. Stops when balanced, after max_rounds, or when a round
 * moves nothing; lpgpu_session_round_stats gives the rounds (active =
 * vertices in overloaded blocks). As in the reference (rebalancer.cpp:59-62),
 * an imbalanced partition with empty blocks first gets the moves of
 * lpgpu_session_repair_empty_blocks, each applied only if its target stays
 * within its max weight and its source keeps weight > 0 (moveVertex,
 * rebalancer.h:84-103); they form a first statistics record (active = n,
 * pins = all pins, candidates = moves proposed, moved = moves applied). */
LPGPU_API lpgpu_status lpgpu_session_rebalance(lpgpu_session* s, int32_t max_rounds, lpgpu_result* result);

/* Rebalancer::repairEmptyBlocks (rebalancing/rebalancer.cpp:169-269) on the
 * current partition, computed on the device and not applied. For every empty
 * block b (weight 0), in increasing id: a vertex u in block p is eligible when
 * c(p) > w(u) and w(u) <= L_max(b); its gain (km1Gain, positive = better) is
 * Σ w(e) over its nets whose connectivity set holds b minus Σ w(e) over its
 * nets with Φ(e, p) > 1. The k eligible vertices of highest gain (lowest id on
 * ties: the bounded heap of rebalancer.cpp:204-213 on vertices in id order)
 * are ordered by gain, then c(p), then id, all descending
 * (rebalancer.cpp:228-232), and the first one no earlier block took is b's
 * move. A block without an eligible vertex stays empty. The arrays receive
 * up to k moves (each needs k entries); *count their number. Single-instance
 * sessions only. */
LPGPU_API lpgpu_status lpgpu_session_repair_empty_blocks(lpgpu_session* s, int32_t* vertices, int32_t* from,
                                                         int32_t* to, int32_t* gain, int32_t* count);

/* Device-resident gain cache (initializeGainCache, partitioned_hypergraph.h:707-809)
 * kept up to date by lpgpu_session_apply_moves with the transition rules of
 * gainCacheUpdate (h:1017-1047, as in changeNodePartWithGainCacheUpdate,
 * h:574-590): moveToPenalty of every pin changes when Φ(e, b) reaches or leaves
 * 0, moveFromBenefit of the non-moving pins in b when it reaches or leaves 1,
 * and the moved vertices' benefits are recounted on the final state. The
 * maintained cache equals a recomputation from scratch whatever the order of
 * the concurrent moves. lpgpu_session_gain_cache then copies it out; refine,
 * set_partition, restore_partition and upload drop it. */
LPGPU_API lpgpu_status lpgpu_session_init_gain_cache(lpgpu_session* s);
LPGPU_API lpgpu_status lpgpu_session_drop_gain_cache(lpgpu_session* s);

/* Applies `count` moves concurrently on the device without balance checks,
 * the curried PartitionedHypergraph::changeNodePart (h:566-572) with its
 * updatePinCountOfHyperedge / km1Delta attribution (h:1133-1167,
 * hypergraph_common.h:133-140). The vertices must be distinct and from[i]
 * must be the current block of vertices[i] (else LPGPU_ERR_INVALID_ARG and
 * nothing is applied). *delta receives the summed attributed objective delta. */
LPGPU_API lpgpu_status lpgpu_session_apply_moves(lpgpu_session* s, int64_t count,
                                                 const int32_t* vertices, const int32_t* from,
                                                 const int32_t* to, int64_t* delta);

/* Saves the current partition on the device / restores it and rebuilds
 * block weights, pin counts and connectivity sets from it
 * (PartitionedHypergraph::initializePartition, h:693-698). Lets a caller
 * repeat a refinement from the same start without host traffic. Restore is
 * asynchronous on the session stream. */
LPGPU_API lpgpu_status lpgpu_session_save_partition(lpgpu_session* s);
LPGPU_API lpgpu_status lpgpu_session_restore_partition(lpgpu_session* s);

/* Number of kernels this thread has launched through the library. */
LPGPU_API int64_t lpgpu_kernel_launches(void);

/* Device memory held by the session, in bytes. */
LPGPU_API lpgpu_status lpgpu_session_footprint(lpgpu_session* s, int64_t* bytes);

/* Device bytes a session would need for (n, m, pins, k): the admission
 * estimate used by the refine server. */
LPGPU_API int64_t lpgpu_estimate_footprint(int64_t num_vertices, int64_t num_nets,
                                           int64_t num_pins, int32_t k, int32_t subrounds);

/* Page-locked host buffers (cudaHostAlloc) so that uploads and downloads
 * run as DMA copies. Returns NULL on failure. */
LPGPU_API void* lpgpu_host_alloc(size_t bytes);
LPGPU_API void lpgpu_host_free(void* p);

/* ------------------------------------------------- allocation-free metrics */

/* Block weights c(V_b), km1 and cut of a partition, computed from device
 * buffers the caller already holds, without allocating any device memory.
 * This entry point has no counterpart in the reference; it exists for callers
 * that cannot let a library allocate: runtimes that own every byte of device
 * memory through their own pool or memory plan (a framework's caching
 * allocator that has reserved the device, a server with a fixed budget), and
 * latency-bound loops that must not block or fail in cudaMalloc, which can
 * synchronize the device.
 *
 *   - All array arguments are device pointers: net_offsets (int64, m+1),
 *     pins (int32), vertex_weights / net_weights (int32, NULL = unit),
 *     partition (int32, n) and the outputs block_weights (int64, k), km1 and
 *     cut (one int64 each).
 *   - The inputs are not validated the way lpgpu_session_upload validates
 *     them: net_offsets must start at 0, be non-decreasing and end at the
 *     number of entries of `pins`. Pins outside [0, n) and block ids outside
 *     [0, k) are skipped (the sums are then not meaningful), weights are
 *     summed as given (negative ones included), and nets with m > 0 but
 *     n == 0 are rejected with LPGPU_ERR_INVALID_ARG.
 *   - k must be in [1, LPGPU_MAX_K]; larger k is rejected with
 *     LPGPU_ERR_INVALID_ARG. The cross-block accumulators live in one fixed
 *     file-scope device array of LPGPU_MAX_K + 2 64-bit words (8 KB), which
 *     every GPU that loads the library holds until the process exits; no
 *     cudaMalloc, cudaFree or allocating library routine is called.
 *   - The work is enqueued on `stream` (a cudaStream_t, NULL = default
 *     stream) and the call returns without waiting; the outputs are valid once
 *     the stream reaches that point.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture. Later calls only enqueue kernels.
 *   - Every call on a device shares the one array: it is cleared at the start
 *     of each call, so calls in sequence are independent, but calls that
 *     overlap on the GPU (e.g. on two streams at once) race and give wrong
 *     results. */
LPGPU_API lpgpu_status lpgpu_partition_metrics_noalloc(int64_t num_vertices, int64_t num_nets,
                                                       const int64_t* net_offsets,
                                                       const int32_t* pins,
                                                       const int32_t* vertex_weights,
                                                       const int32_t* net_weights,
                                                       const int32_t* partition, int32_t k,
                                                       int64_t* block_weights, int64_t* km1,
                                                       int64_t* cut, void* stream);

/* ------------------------------------------------------------- timing */

/* CUDA events on the session stream: record into one of 16 slots, read the
 * elapsed device time between two recorded slots (waits for the later one). */
LPGPU_API lpgpu_status lpgpu_session_event_record(lpgpu_session* s, int32_t slot);
LPGPU_API lpgpu_status lpgpu_session_event_elapsed(lpgpu_session* s, int32_t a, int32_t b,
                                                   double* ms);
LPGPU_API lpgpu_status lpgpu_session_synchronize(lpgpu_session* s);

/* Kernel-phase timing with CUDA events on the session stream. When enabled,
 * every refine records, per named phase, the summed device time and launch
 * count; lpgpu_session_phase_times returns up to max entries. */
typedef struct {
  char name[24];
  int64_t launches;
  double ms;
} lpgpu_phase_time;

LPGPU_API lpgpu_status lpgpu_session_enable_timing(lpgpu_session* s, int32_t enable);
LPGPU_API lpgpu_status lpgpu_session_phase_times(lpgpu_session* s, lpgpu_phase_time* out,
                                                 int32_t max, int32_t* count);

#ifdef __cplusplus
}
#endif

#endif /* LPGPU_H_ */
