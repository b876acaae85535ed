// Session management and the C ABI of liblpgpu (declared in include/lpgpu.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "common.cuh"

namespace lpgpu {

static thread_local std::string g_error;
void set_error(const std::string& msg) { g_error = msg; }

// Device memory of a session: a session-owned pool, allocations and frees
// ordered on the session's stream (no device-wide synchronisation, as a
// cudaFree would impose on every other session), and the bytes held by the
// session's buffers.
struct Mem {
  cudaMemPool_t pool = nullptr;
  cudaStream_t st = nullptr;
  int64_t bytes = 0;
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t count = 0;
  cudaError_t alloc(size_t n, Mem* mem) {
    if (n == count && p) return cudaSuccess;
    release(mem);
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p), n * sizeof(T), mem->pool, mem->st);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    count = n;
    mem->bytes += (int64_t)(n * sizeof(T));
    return cudaSuccess;
  }
  void release(Mem* mem) {
    if (p) {
      cudaFreeAsync(p, mem->st);
      mem->bytes -= (int64_t)(count * sizeof(T));
    }
    p = nullptr;
    count = 0;
  }
};

// A temporary device buffer of one call, freed (stream-ordered) on every
// return path.
template <typename T>
struct TmpBuf {
  DevBuf<T> b;
  Mem m;
  TmpBuf(const Mem& owner) : m{owner.pool, owner.st, 0} {}
  ~TmpBuf() { b.release(&m); }
  cudaError_t alloc(size_t n) { return b.alloc(n, &m); }
  T* p() const { return b.p; }
};

// Copies of consecutive pieces in one direction: a piece whose host and
// device ranges both continue the previous piece's joins it, so buffers that
// callers keep back to back (arenas of many instances) go in one call.
struct CopyRun {
  cudaStream_t st;
  cudaMemcpyKind kind;
  char* dst = nullptr;
  const char* src = nullptr;
  size_t bytes = 0;
  cudaError_t add(void* d, const void* h, size_t b) {
    if (b == 0) return cudaSuccess;
    if (bytes && static_cast<char*>(d) == dst + bytes && static_cast<const char*>(h) == src + bytes) {
      bytes += b;
      return cudaSuccess;
    }
    const cudaError_t e = flush();
    dst = static_cast<char*>(d);
    src = static_cast<const char*>(h);
    bytes = b;
    return e;
  }
  cudaError_t flush() {
    if (!bytes) return cudaSuccess;
    const size_t b = bytes;
    bytes = 0;
    return cudaMemcpyAsync(dst, src, b, kind, st);
  }
};

static int word_count(int k) { return (k + 31) / 32; }
static int word_class_of(int k) {
  int w = 1;
  while (w < word_count(k)) w <<= 1;
  return w;
}

static lpgpu_status cuda_fail(cudaError_t e, const char* what) {
  // keep a more specific message set by a launch helper
  const std::string prev = g_error;
  const std::string here = std::string(what) + ": " + cudaGetErrorString(e);
  set_error(prev.empty() ? here : here + " [" + prev + "]");
  cudaGetLastError();  // clear sticky-free errors
  if (e == cudaErrorMemoryAllocation) return LPGPU_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ||
      e == cudaErrorNoKernelImageForDevice || e == cudaErrorInvalidDevice)
    return LPGPU_ERR_NO_DEVICE;
  return LPGPU_ERR_CUDA;
}

static lpgpu_status invalid(const std::string& msg) {
  set_error(msg);
  return LPGPU_ERR_INVALID_ARG;
}

}  // namespace lpgpu

using namespace lpgpu;

#define CK(expr)                                   \
  do {                                             \
    cudaError_t _e = (expr);                       \
    if (_e != cudaSuccess) return cuda_fail(_e, #expr); \
  } while (0)

struct lpgpu_session_s {
  int device = 0;
  cudaStream_t st = nullptr;
  int num_sms = 1;
  Mem mem;
  // hypergraph
  bool has_hg = false;
  int64_t n = 0, m = 0, P = 0;
  int64_t total_vw = 0;
  int64_t deg_inc[kDegBuckets] = {};  // incidences per log2 degree bucket
  bool unit_nets = true;
  int32_t max_we = 0;
  int64_t max_net_size = 0;
  DevBuf<int64_t> net_off, vtx_off;
  DevBuf<int32_t> pins, inets, w_v, w_e;
  // partition
  bool has_part = false;
  int32_t k = 0, W = 0;
  DevBuf<int32_t> part, phi;
  DevBuf<uint32_t> conn;
  DevBuf<int64_t> bw, lmax, perfect;
  std::vector<int64_t> h_perfect;
  // refine scratch
  DevBuf<int32_t> list, net_epoch, seg_w, heavy, revl;
  DevBuf<int64_t> sub_off, blk64, scal, stats, bin_cnt, scan_tmp;
  DevBuf<uint8_t> next_flag, status, over;
  DevBuf<int4> rec;
  DevBuf<uint64_t> seg_key, thr;
  DevBuf<int32_t> saved_part;
  // gain cache kept by apply_moves (lpgpu_session_init_gain_cache)
  bool gc_valid = false;
  DevBuf<int32_t> gc_benefit, gc_penalty;
  DevBuf<uint8_t> gc_moved;
  void drop_gain_cache() {
    gc_valid = false;
    gc_benefit.release(&mem);
    gc_penalty.release(&mem);
    gc_moved.release(&mem);
  }
  int64_t scan_tmp_n = 0;
  // batched sessions (lpgpu_session_upload_batch): instance ranges and blocks
  bool batched = false;
  int32_t num_inst = 0;
  int32_t kmax = 0;
  std::vector<int64_t> h_inst_voff, h_inst_noff, h_inst_weight;
  std::vector<int64_t> h_inst_pins;  // pins of every instance (work estimate of the persistent rounds)
  std::vector<int32_t> h_inst_boff, h_inst_k;
  // persistent rounds: instance descriptors, work order, what they were built from
  DevBuf<PxInst> px;
  DevBuf<int32_t> px_order;
  std::vector<int64_t> px_key;
  bool has_tuning = false;
  lpgpu_tuning tuning{};
  std::vector<PxInst> h_px;  // host copy of the descriptors
  // stepped refinement (lpgpu_session_begin_rounds, lpgpu_stepper_*)
  bool stepping = false, step_done = false;
  lpgpu_config step_cfg{};
  int32_t step_round = 0;
  int64_t step_km1_before = 0;
  cudaEvent_t step_ev = nullptr;
  DevBuf<int32_t> vinst, inst_boff, inst_k, over_ids;
  DevBuf<int64_t> inst_voff, inst_noff, inst_delta;
  DevBuf<int64_t> vout;  // result words of the device-side input checks
  // results of the last refine
  std::vector<lpgpu_round_stats> last_stats;
  // timing
  bool timing = false;
  PhaseTimer timer;
  std::vector<lpgpu_phase_time> phase_times;
  cudaEvent_t slots[16] = {};
  // cached CUDA graph of the refine sequence and the parameters baked into it
  cudaGraphExec_t graph = nullptr;
  std::vector<unsigned char> graph_key;
  int64_t graph_kernels = 0;  // kernel nodes in the cached graph

  Launch launch() const { return Launch{st, num_sms}; }

  // Per mille of the sweep's work in heavy vertices, from the degree
  // histogram: a bucket counts as heavy when its largest degree is; a heavy
  // incidence costs about twice a light one. 0 only when no vertex is heavy.
  int32_t heavy_share() const {
    double heavy = 0, light = 0;
    for (int j = 0; j < kDegBuckets; ++j) {
      const int64_t top = j >= 62 ? INT64_MAX : (int64_t(2) << j) - 1;
      if (sweep_heavy(top < kHighDegree ? top : kHighDegree, W, unit_nets ? 1 : 0, max_we))
        heavy += (double)deg_inc[j];
      else
        light += (double)deg_inc[j];
    }
    if (heavy == 0) return 0;
    const int x = (int)(1000.0 * 2.0 * heavy / (2.0 * heavy + light));
    return x < 1 ? 1 : x;
  }

  // Φ entries fit 16 bits when every net has fewer than 2^16 pins.
  bool phi16() const { return LPGPU_PHI16 && max_net_size < 65536; }
  size_t phi_words() const {
    const size_t entries = (size_t)m * kmax;
    return phi16() ? (entries + 1) / 2 : entries;
  }

  RoundCtx ctx(const lpgpu_config* cfg = nullptr) {
    RoundCtx c{};
    c.n = n;
    c.m = m;
    c.k = k;
    c.W = W;
    c.net_off = net_off.p;
    c.pins = pins.p;
    c.vtx_off = vtx_off.p;
    c.inets = inets.p;
    c.w_v = w_v.p;
    c.w_e = w_e.p;
    c.unit_nets = unit_nets ? 1 : 0;
    c.phi16 = phi16() ? 1 : 0;
    c.max_we = max_we;
    c.heavy_share = heavy_share();
    c.part = part.p;
    c.phi = phi.p;
    c.conn = conn.p;
    c.bw = bw.p;
    c.lmax = lmax.p;
    c.perfect = perfect.p;
    c.list = list.p;
    c.sub_off = sub_off.p;
    c.next_flag = next_flag.p;
    c.net_epoch = net_epoch.p;
    c.batched = batched ? 1 : 0;
    c.kmax = batched ? kmax : k;
    c.num_inst = num_inst;
    c.vinst = vinst.p;
    c.inst_voff = inst_voff.p;
    c.inst_boff = inst_boff.p;
    c.inst_k = inst_k.p;
    c.inst_delta = inst_delta.p;
    c.over_ids = over_ids.p;
    c.rec = rec.p;
    c.status = status.p;
    int64_t* b = blk64.p;
    if (b) {
      c.in_w = b;
      c.in_cnt = b + k;
      c.cand_out = b + 2 * k;
      c.acc_w = b + 3 * k;
      c.acc_cnt = b + 4 * k;
      c.seg_off = b + 5 * k;
      c.cursor = b + 6 * k + 1;
    }
    if (thr.p) {
      c.thr_to = thr.p;
      c.thr_from = thr.p + k;
    }
    if (over.p) {
      c.over_to = over.p;
      c.over_from = over.p + k;
    }
    c.seg_key = seg_key.p;
    c.seg_w = seg_w.p;
    c.heavy = heavy.p;
    c.revl = revl.p;
    c.scal = scal.p;
    c.stats = stats.p;
    if (cfg) {
      c.zero_gain = cfg->rebalancing ? 1 : 0;
      c.revert = cfg->revert;
      c.rollback = cfg->rollback;
      c.act_threshold = cfg->activation_threshold <= 0 ? INT64_MAX : cfg->activation_threshold;
    }
    return c;
  }

  void release_partition() {
    drop_gain_cache();
    part.release(&mem);
    phi.release(&mem);
    conn.release(&mem);
    bw.release(&mem);
    lmax.release(&mem);
    perfect.release(&mem);
    blk64.release(&mem);
    thr.release(&mem);
    over.release(&mem);
    over_ids.release(&mem);
    inst_boff.release(&mem);
    inst_k.release(&mem);
    inst_delta.release(&mem);
    has_part = false;
  }
  // Returns pooled memory beyond the buffers in use plus 1 GiB of slack
  // (call after a synchronisation: pending frees still count as in use).
  void trim() {
    uint64_t reserved = 0;
    if (cudaMemPoolGetAttribute(mem.pool, cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess) return;
    const uint64_t keep = (uint64_t)mem.bytes + (1ull << 30);
    if (reserved > keep) cudaMemPoolTrimTo(mem.pool, keep);
  }

  void release_all() {
    release_partition();
    DevBuf<int64_t>* b64[] = {&net_off, &vtx_off, &sub_off, &stats, &bin_cnt, &scan_tmp};
    for (auto* b : b64) b->release(&mem);
    DevBuf<int32_t>* b32[] = {&pins, &inets, &w_v, &w_e, &list, &net_epoch, &seg_w, &heavy, &revl};
    for (auto* b : b32) b->release(&mem);
    next_flag.release(&mem);
    saved_part.release(&mem);
    px.release(&mem);
    px_order.release(&mem);
    px_key.clear();
    vinst.release(&mem);
    inst_voff.release(&mem);
    inst_noff.release(&mem);
    vout.release(&mem);
    status.release(&mem);
    rec.release(&mem);
    seg_key.release(&mem);
    has_hg = false;
  }
};

namespace {

// Makes the session's device current for one API call and clears the
// thread's error text.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    g_error.clear();
    cudaGetLastError();  // drop a stale non-sticky error of an earlier unchecked call
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// Structural checks of the upload arguments on the host (O(instances)); the
// per-net, per-pin and per-vertex checks run on the device after the copy
// (launch_validate_csr) and are reported by upload_impl.
lpgpu_status check_shape(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins, int32_t num_inst,
                         const int64_t* inst_voff, const int64_t* inst_noff) {
  if (n < 0 || m < 0) return invalid("negative vertex or net count");
  if (n > INT32_MAX || m > INT32_MAX) return invalid("vertex and net ids must fit int32");
  if (!net_off || (m > 0 && net_off[m] > 0 && !pins)) return invalid("null CSR pointer");
  if (net_off[0] != 0) return invalid("net_offsets[0] must be 0");
  if (net_off[m] < 0) return invalid("net_offsets must be non-decreasing");
  if (inst_voff) {
    for (int32_t i = 0; i < num_inst; ++i) {
      const int64_t v0 = inst_voff[i], v1 = inst_voff[i + 1], e0 = inst_noff[i], e1 = inst_noff[i + 1];
      if (v0 < 0 || v1 < v0 || v1 > n || e0 < 0 || e1 < e0 || e1 > m)
        return invalid("instance offsets must be non-decreasing and within the union");
    }
    if (inst_voff[0] != 0 || inst_voff[num_inst] != n || inst_noff[0] != 0 || inst_noff[num_inst] != m)
      return invalid("instance offsets must cover the union exactly");
  }
  return LPGPU_OK;
}

}  // namespace

extern "C" {

void lpgpu_config_default(lpgpu_config* cfg) {
  if (!cfg) return;
  cfg->rounds = 5;
  cfg->activation_threshold = 100;
  cfg->rebalancing = 1;
  cfg->subrounds = 7;
  cfg->revert = 1;
  cfg->rollback = 1;
  cfg->flags = 0;
  cfg->reserved1 = 0;
}

const char* lpgpu_status_string(lpgpu_status s) {
  switch (s) {
    case LPGPU_OK: return "ok";
    case LPGPU_ERR_INVALID_ARG: return "invalid argument";
    case LPGPU_ERR_OOM: return "out of device memory";
    case LPGPU_ERR_ADMISSION: return "admission rejected";
    case LPGPU_ERR_TIMEOUT: return "device wait timed out";
    case LPGPU_ERR_CUDA: return "CUDA error";
    case LPGPU_ERR_NO_DEVICE: return "no usable CUDA device";
    case LPGPU_ERR_STATE: return "invalid call order";
  }
  return "unknown status";
}

const char* lpgpu_last_error(void) { return g_error.c_str(); }

lpgpu_status lpgpu_session_create(int32_t device, lpgpu_session** out) {
  if (!out) return invalid("null output pointer");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    set_error(std::string("no CUDA device: ") + cudaGetErrorString(e));
    cudaGetLastError();
    return LPGPU_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return invalid("device index out of range");
  DeviceGuard g(device);
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  auto* s = new lpgpu_session_s();
  s->device = device;
  s->num_sms = prop.multiProcessorCount;
  e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete s;
    return cuda_fail(e, "cudaStreamCreate");
  }
  s->timer.st = s->st;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  if ((e = cudaMemPoolCreate(&s->mem.pool, &props)) != cudaSuccess) {
    cudaStreamDestroy(s->st);
    delete s;
    return cuda_fail(e, "cudaMemPoolCreate");
  }
  // freed blocks stay in the pool for the next upload; trim() returns them
  uint64_t keep = UINT64_MAX;
  cudaMemPoolSetAttribute(s->mem.pool, cudaMemPoolAttrReleaseThreshold, &keep);
  s->mem.st = s->st;
  if ((e = s->scal.alloc(kScalars, &s->mem)) != cudaSuccess ||
      (e = cudaMemsetAsync(s->scal.p, 0, sizeof(int64_t) * kScalars, s->st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s->st)) != cudaSuccess) {
    s->scal.release(&s->mem);
    cudaStreamSynchronize(s->st);
    cudaMemPoolDestroy(s->mem.pool);
    cudaStreamDestroy(s->st);
    delete s;
    return cuda_fail(e, "alloc scalars");
  }
  *out = s;
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_destroy(lpgpu_session* s) {
  if (!s) return LPGPU_OK;
  {
    DeviceGuard g(s->device);
    cudaStreamSynchronize(s->st);
    s->release_all();
    s->scal.release(&s->mem);
    for (auto& ev : s->slots)
      if (ev) cudaEventDestroy(ev);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->step_ev) cudaEventDestroy(s->step_ev);
    cudaStreamSynchronize(s->st);
    cudaMemPoolDestroy(s->mem.pool);
    cudaStreamDestroy(s->st);
  }
  delete s;
  return LPGPU_OK;
}

// Upload of a union CSR (`insts` null) or of per-instance buffers (`insts`
// with the host-computed instance vertex / net / pin offsets). Shapes are
// checked by the caller.
static lpgpu_status upload_impl(lpgpu_session* s, int64_t n, int64_t m, int64_t P, const int64_t* net_off,
                                const int32_t* pins, const int32_t* w_v, const int32_t* w_e,
                                int32_t num_inst, const int64_t* inst_voff, const int64_t* inst_noff,
                                const lpgpu_instance* insts = nullptr, const int64_t* inst_poff = nullptr) {
  // each instance's pin range of a batch (host-computed for per-instance
  // buffers, from the union's offsets otherwise), checked before any copy
  const bool batch = inst_voff != nullptr;
  std::vector<int64_t> hpoff;
  if (batch) {
    hpoff.resize(num_inst + 1);
    for (int32_t i = 0; i < num_inst; ++i) hpoff[i] = insts ? inst_poff[i] : net_off[inst_noff[i]];
    hpoff[num_inst] = P;
    for (int32_t i = 0; i < num_inst; ++i)
      if (hpoff[i] < 0 || hpoff[i] > hpoff[i + 1])
        return invalid("net_offsets must be non-decreasing and within the pin array");
  }
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  // buffers of the same size are reused; the partition must be set again
  s->has_part = false;
  s->has_hg = false;
  s->drop_gain_cache();
  s->n = n;
  s->m = m;
  s->P = P;
  const int32_t I = inst_voff ? num_inst : 1;
  Mem* fp = &s->mem;
  TmpBuf<int64_t> staged(s->mem);  // per-instance offsets before the rebase
  CK(s->net_off.alloc(m + 1, fp));
  CK(s->vtx_off.alloc(n + 1, fp));
  CK(s->pins.alloc(P, fp));
  CK(s->inets.alloc(P, fp));
  CK(s->w_v.alloc(n, fp));
  CK(s->w_e.alloc(m, fp));
  CK(s->net_epoch.alloc(m, fp));
  CK(s->list.alloc(n, fp));
  CK(s->next_flag.alloc(n, fp));
  CK(s->status.alloc(n, fp));
  CK(s->rec.alloc(n, fp));
  CK(s->seg_key.alloc(n, fp));
  CK(s->seg_w.alloc(n, fp));
  CK(s->heavy.alloc(n, fp));
  CK(s->revl.alloc(n, fp));
  CK(s->vout.alloc(std::max<int64_t>(kVSums + 2 * (int64_t)I, kDegBuckets), fp));
  CK(s->sub_off.alloc(2 * kMaxSubrounds + 1, fp));
  CK(s->bin_cnt.alloc(2 * kMaxSubrounds * kDegClasses, fp));
  s->scan_tmp_n = std::max<int64_t>(1, scan_tmp_elems(n + 1));
  CK(s->scan_tmp.alloc(s->scan_tmp_n, fp));
  cudaStream_t st = s->st;
  const Launch L = s->launch();
  if (!insts) {
    CK(cudaMemcpyAsync(s->net_off.p, net_off, sizeof(int64_t) * (m + 1), cudaMemcpyHostToDevice, st));
    if (P > 0) CK(cudaMemcpyAsync(s->pins.p, pins, sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
    if (n > 0) {
      if (w_v) CK(cudaMemcpyAsync(s->w_v.p, w_v, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
      else CK(launch_fill_ones(L, s->w_v.p, n));
    }
    if (m > 0) {
      if (w_e) CK(cudaMemcpyAsync(s->w_e.p, w_e, sizeof(int32_t) * m, cudaMemcpyHostToDevice, st));
      else CK(launch_fill_ones(L, s->w_e.p, m));
    }
  } else {
    // unit weights first, then every instance's own buffers into place (stream order)
    bool unit_v = false, unit_e = false;
    for (int32_t i = 0; i < I; ++i) {
      unit_v = unit_v || !insts[i].vertex_weights;
      unit_e = unit_e || !insts[i].net_weights;
    }
    if (unit_v) CK(launch_fill_ones(L, s->w_v.p, n));
    if (unit_e) CK(launch_fill_ones(L, s->w_e.p, m));
    // offsets with their closing entry (m_i + 1 each) go back to back into a
    // staging buffer, instance i's at inst_noff[i] + i; the rebase moves them
    CK(staged.alloc((size_t)(m + I)));
    CopyRun c_off{st, cudaMemcpyHostToDevice}, c_pin{st, cudaMemcpyHostToDevice},
        c_wv{st, cudaMemcpyHostToDevice}, c_we{st, cudaMemcpyHostToDevice};
    for (int32_t i = 0; i < I; ++i) {
      const lpgpu_instance& x = insts[i];
      const int64_t ni = x.num_vertices, mi = x.num_nets, pi = inst_poff[i + 1] - inst_poff[i];
      if (mi > 0) CK(c_off.add(staged.p() + inst_noff[i] + i, x.net_offsets, sizeof(int64_t) * (mi + 1)));
      if (pi > 0) CK(c_pin.add(s->pins.p + inst_poff[i], x.pins, sizeof(int32_t) * pi));
      if (ni > 0 && x.vertex_weights) CK(c_wv.add(s->w_v.p + inst_voff[i], x.vertex_weights, sizeof(int32_t) * ni));
      if (mi > 0 && x.net_weights) CK(c_we.add(s->w_e.p + inst_noff[i], x.net_weights, sizeof(int32_t) * mi));
    }
    CK(c_off.flush());
    CK(c_pin.flush());
    CK(c_wv.flush());
    CK(c_we.flush());
    CK(cudaMemcpyAsync(s->net_off.p + m, &P, sizeof(int64_t), cudaMemcpyHostToDevice, st));  // synchronized below
  }
  if (n > 0) CK(cudaMemsetAsync(s->next_flag.p, 0, n, st));
  if (m > 0) CK(cudaMemsetAsync(s->net_epoch.p, 0, sizeof(int32_t) * m, st));
  // instance ranges of a batched session
  s->batched = inst_voff != nullptr;
  s->num_inst = I;
  s->h_inst_pins.assign(I, P);
  for (int32_t i = 0; inst_voff && i < I; ++i)
    s->h_inst_pins[i] = insts ? inst_poff[i + 1] - inst_poff[i] : net_off[inst_noff[i + 1]] - net_off[inst_noff[i]];
  s->h_inst_voff.assign(2, 0);
  s->h_inst_noff.assign(2, 0);
  s->h_inst_voff[1] = n;
  s->h_inst_noff[1] = m;
  TmpBuf<int64_t> poff(s->mem);  // hpoff on the device, alive through the checks
  if (s->batched) {
    s->h_inst_voff.assign(inst_voff, inst_voff + I + 1);
    s->h_inst_noff.assign(inst_noff, inst_noff + I + 1);
    CK(s->vinst.alloc(n, fp));
    CK(s->inst_voff.alloc(I + 1, fp));
    CK(s->inst_noff.alloc(I + 1, fp));
    CK(poff.alloc(I + 1));
    CK(cudaMemcpyAsync(s->inst_voff.p, inst_voff, sizeof(int64_t) * (I + 1), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->inst_noff.p, inst_noff, sizeof(int64_t) * (I + 1), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(poff.p(), hpoff.data(), sizeof(int64_t) * (I + 1), cudaMemcpyHostToDevice, st));
    if (insts) {  // local ids to union ids
      CK(launch_rebase_instances(L, I, s->inst_voff.p, s->inst_noff.p, poff.p(), s->net_off.p, s->pins.p,
                                 staged.p()));
      CK(cudaStreamSynchronize(st));
    }
  } else {
    s->vinst.release(fp);
    s->inst_voff.release(fp);
    s->inst_noff.release(fp);
  }
  // device-side checks; one copy back of the result words and the per-instance sums
  CK(launch_validate_csr(s->launch(), n, m, P, s->net_off.p, s->pins.p, s->w_v.p, s->w_e.p, I,
                         s->inst_voff.p, s->inst_noff.p, poff.p(), s->vinst.p, s->vout.p));
  std::vector<int64_t> h(kVSums + 2 * (size_t)I);
  CK(cudaMemcpyAsync(h.data(), s->vout.p, sizeof(int64_t) * h.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  switch (h[kVErr]) {
    case kVOk: break;
    case kVBadOffsets: return invalid("net_offsets must be non-decreasing and within the pin array");
    case kVNegNetWeight: return invalid("net weights must be >= 0");
    case kVPinRange:
      return invalid(I > 1 ? "pin id outside its instance's vertex range" : "pin id out of range");
    case kVNegVertexWeight: return invalid("vertex weights must be >= 0");
    default: return invalid("invalid hypergraph");
  }
  s->h_inst_weight.assign(I, 0);
  int64_t total = 0;
  for (int32_t i = 0; i < I; ++i) {
    if (h[kVSums + i] > INT32_MAX)
      return invalid("sum of |e| * w(e) exceeds int32: gains would overflow the reference's Gain type");
    const int64_t tw = h[kVSums + I + i];
    if (tw > INT32_MAX) return invalid("total vertex weight exceeds int32 (the reference's HypernodeWeight)");
    s->h_inst_weight[i] = tw;
    total += tw;
  }
  s->total_vw = total;
  s->max_we = (int32_t)h[kVMaxWe];
  s->max_net_size = h[kVMaxSize];
  s->unit_nets = h[kVNonUnit] == 0;
  TmpBuf<int32_t> rank(s->mem);  // each pin's slot in its vertex's incident-net list
  CK(rank.alloc((size_t)P));
  CK(launch_build_incidence(s->launch(), n, m, P, s->net_off.p, s->pins.p, s->vtx_off.p, s->inets.p, rank.p(),
                            s->scan_tmp.p, s->scan_tmp_n, s->vout.p));
  CK(cudaMemcpyAsync(s->deg_inc, s->vout.p, sizeof(s->deg_inc), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  s->has_hg = true;
  s->trim();
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_upload(lpgpu_session* s, int64_t n, int64_t m, const int64_t* net_off,
                                  const int32_t* pins, const int32_t* w_v, const int32_t* w_e) {
  if (!s) return invalid("null session");
  const lpgpu_status vs = check_shape(n, m, net_off, pins, 1, nullptr, nullptr);
  if (vs != LPGPU_OK) return vs;
  return upload_impl(s, n, m, net_off[m], net_off, pins, w_v, w_e, 1, nullptr, nullptr);
}

lpgpu_status lpgpu_session_upload_instances(lpgpu_session* s, int32_t num_instances,
                                            const lpgpu_instance* instances) {
  if (!s) return invalid("null session");
  if (num_instances < 1 || !instances) return invalid("a batch needs at least one instance");
  std::vector<int64_t> voff(num_instances + 1, 0), noff(num_instances + 1, 0), poff(num_instances + 1, 0);
  for (int32_t i = 0; i < num_instances; ++i) {
    const lpgpu_instance& x = instances[i];
    if (x.num_vertices < 0 || x.num_nets < 0) return invalid("negative vertex or net count");
    if (!x.net_offsets) return invalid("null CSR pointer");
    if (x.net_offsets[0] != 0) return invalid("net_offsets[0] must be 0");
    const int64_t pi = x.net_offsets[x.num_nets];
    if (pi < 0) return invalid("net_offsets must be non-decreasing");
    if (pi > 0 && !x.pins) return invalid("null CSR pointer");
    voff[i + 1] = voff[i] + x.num_vertices;
    noff[i + 1] = noff[i] + x.num_nets;
    poff[i + 1] = poff[i] + pi;
    if (voff[i + 1] > INT32_MAX || noff[i + 1] > INT32_MAX) return invalid("vertex and net ids must fit int32");
  }
  return upload_impl(s, voff[num_instances], noff[num_instances], poff[num_instances], nullptr, nullptr, nullptr,
                     nullptr, num_instances, voff.data(), noff.data(), instances, poff.data());
}

lpgpu_status lpgpu_session_upload_batch(lpgpu_session* s, int32_t num_instances,
                                        const int64_t* instance_vertex_offsets,
                                        const int64_t* instance_net_offsets, const int64_t* net_off,
                                        const int32_t* pins, const int32_t* w_v, const int32_t* w_e) {
  if (num_instances < 1 || !instance_vertex_offsets || !instance_net_offsets)
    return invalid("a batch needs at least one instance and its offsets");
  if (!s) return invalid("null session");
  const int64_t n = instance_vertex_offsets[num_instances], m = instance_net_offsets[num_instances];
  const lpgpu_status vs = check_shape(n, m, net_off, pins, num_instances, instance_vertex_offsets,
                                      instance_net_offsets);
  if (vs != LPGPU_OK) return vs;
  return upload_impl(s, n, m, net_off[m], net_off, pins, w_v, w_e, num_instances, instance_vertex_offsets,
                     instance_net_offsets);
}

// Allocates the partition state for K global blocks (Φ rows of kmax entries)
// and builds it from `part` (host): block ids in [0, K) for one instance, or
// local ids per instance for a batch (turned into global ids on the device).
static lpgpu_status set_partition_impl(lpgpu_session* s, int32_t K, int32_t kmax, const int32_t* part,
                                       const std::vector<int64_t>& hl, const std::vector<int64_t>& hp,
                                       const int32_t* const* parts = nullptr, const int32_t* part_dev = nullptr) {
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  s->has_part = false;
  s->drop_gain_cache();
  s->k = K;
  s->kmax = kmax;
  s->W = word_class_of(kmax);
  Mem* fp = &s->mem;
  // same-size buffers are kept from the previous partition
  CK(s->part.alloc(s->n, fp));
  CK(s->phi.alloc(s->phi_words(), fp));
  CK(s->conn.alloc((size_t)s->m * 2 * s->W, fp));
  CK(s->bw.alloc(K, fp));
  CK(s->lmax.alloc(K, fp));
  CK(s->perfect.alloc(K, fp));
  CK(s->blk64.alloc(7 * (size_t)K + 1, fp));
  CK(s->thr.alloc(2 * (size_t)K, fp));
  CK(s->over.alloc(2 * (size_t)K, fp));
  CK(s->over_ids.alloc(K, fp));
  cudaStream_t st = s->st;
  if (s->batched) {
    CK(s->inst_boff.alloc(s->num_inst, fp));
    CK(s->inst_k.alloc(s->num_inst, fp));
    CK(s->inst_delta.alloc(s->num_inst, fp));
    CK(cudaMemcpyAsync(s->inst_boff.p, s->h_inst_boff.data(), sizeof(int32_t) * s->num_inst, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->inst_k.p, s->h_inst_k.data(), sizeof(int32_t) * s->num_inst, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(s->inst_delta.p, 0, sizeof(int64_t) * s->num_inst, st));
  }
  if (part_dev) {
    if (s->n > 0) CK(cudaMemcpyAsync(s->part.p, part_dev, sizeof(int32_t) * s->n, cudaMemcpyDeviceToDevice, st));
  } else if (parts) {
    CopyRun run{st, cudaMemcpyHostToDevice};
    for (int32_t i = 0; i < s->num_inst; ++i) {
      const int64_t v0 = s->h_inst_voff[i], ni = s->h_inst_voff[i + 1] - v0;
      if (ni > 0) CK(run.add(s->part.p + v0, parts[i], sizeof(int32_t) * ni));
    }
    CK(run.flush());
  } else if (s->n > 0) {
    CK(cudaMemcpyAsync(s->part.p, part, sizeof(int32_t) * s->n, cudaMemcpyHostToDevice, st));
  }
  CK(launch_check_partition(s->launch(), s->n, s->part.p, K, s->batched ? s->vinst.p : nullptr,
                            s->inst_boff.p, s->inst_k.p, s->vout.p));
  int64_t check = 0;
  CK(cudaMemcpyAsync(&check, s->vout.p + kVErr, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(s->lmax.p, hl.data(), sizeof(int64_t) * K, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(s->perfect.p, hp.data(), sizeof(int64_t) * K, cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));
  if (check != kVOk) return invalid("block id out of range");
  CK(cudaMemsetAsync(s->blk64.p, 0, sizeof(int64_t) * (7 * (size_t)K + 1), st));
  RoundCtx c = s->ctx();
  CK(launch_init_partition(s->launch(), c));
  CK(cudaStreamSynchronize(st));
  s->h_perfect = hp;
  s->has_part = true;
  s->trim();
  return LPGPU_OK;
}

// Per-instance k / eps of a batch; the partition comes as one union array
// (`partition`) or one array per instance (`parts`).
static lpgpu_status set_partition_batch_impl(lpgpu_session* s, const int32_t* instance_k,
                                             const double* instance_eps, const int32_t* partition,
                                             const int32_t* const* parts) {
  if (!s) return invalid("null session");
  if (!s->has_hg || !s->batched) {
    set_error("set_partition_batch needs a batched upload");
    return LPGPU_ERR_STATE;
  }
  if (!instance_k || !instance_eps || (s->n > 0 && !partition && !parts)) return invalid("null argument");
  if (parts)
    for (int32_t i = 0; i < s->num_inst; ++i)
      if (!parts[i] && s->h_inst_voff[i + 1] > s->h_inst_voff[i]) return invalid("null argument");
  const int32_t I = s->num_inst;
  std::vector<int32_t> boff(I);
  int64_t K = 0;
  int32_t kmax = 1;
  for (int32_t i = 0; i < I; ++i) {
    if (instance_k[i] < 1 || instance_k[i] > LPGPU_MAX_K) return invalid("instance k must be in [1, 1024]");
    boff[i] = (int32_t)K;
    K += instance_k[i];
    kmax = std::max(kmax, instance_k[i]);
  }
  if (K > INT32_MAX / 8) return invalid("too many blocks in one batch");
  std::vector<int64_t> hl(K), hp(K);
  for (int32_t i = 0; i < I; ++i) {
    // total weight of the instance for Context::setupPartWeights (context.cpp:237-250)
    const int64_t tw = s->h_inst_weight[i];
    const int64_t perfect = std::max<int64_t>(1, (int64_t)std::ceil((double)tw / (double)instance_k[i]));
    const int64_t lmax = (int64_t)((1.0 + instance_eps[i]) * (double)perfect);
    for (int32_t b = 0; b < instance_k[i]; ++b) {
      hp[boff[i] + b] = perfect;
      hl[boff[i] + b] = lmax;
    }
  }
  s->h_inst_boff = boff;
  s->h_inst_k.assign(instance_k, instance_k + I);
  return set_partition_impl(s, (int32_t)K, kmax, partition, hl, hp, parts);
}

lpgpu_status lpgpu_session_set_partition_batch(lpgpu_session* s, const int32_t* instance_k,
                                               const double* instance_eps, const int32_t* partition) {
  return set_partition_batch_impl(s, instance_k, instance_eps, partition, nullptr);
}

lpgpu_status lpgpu_session_set_partition_instances(lpgpu_session* s, const int32_t* instance_k,
                                                   const double* instance_eps, const int32_t* const* partitions) {
  if (!partitions) return invalid("null argument");
  return set_partition_batch_impl(s, instance_k, instance_eps, nullptr, partitions);
}

lpgpu_status lpgpu_session_set_partition(lpgpu_session* s, int32_t k, double eps,
                                         const int32_t* partition, const int64_t* max_w,
                                         const int64_t* perfect_w) {
  if (!s) return invalid("null session");
  if (!s->has_hg) {
    set_error("set_partition before upload");
    return LPGPU_ERR_STATE;
  }
  if (s->batched) {
    set_error("batched session: use lpgpu_session_set_partition_batch");
    return LPGPU_ERR_STATE;
  }
  if (k < 1 || k > LPGPU_MAX_K) return invalid("k must be in [1, 1024]");
  if (s->n > 0 && !partition) return invalid("null partition");
  std::vector<int64_t> hp(k), hl(k);
  // Context::setupPartWeights (context.cpp:237-250)
  const int64_t perfect = (int64_t)std::ceil((double)s->total_vw / (double)k);
  const int64_t lmax = (int64_t)((1.0 + eps) * (double)perfect);
  for (int b = 0; b < k; ++b) {
    hp[b] = perfect_w ? perfect_w[b] : perfect;
    hl[b] = max_w ? max_w[b] : lmax;
    if (hp[b] < 1) hp[b] = 1;
  }
  return set_partition_impl(s, k, k, partition, hl, hp);
}

lpgpu_status lpgpu_session_project_partition(lpgpu_session* fine, const lpgpu_session* coarse,
                                             const int32_t* fine_to_coarse) {
  if (!fine || !coarse) return invalid("null session");
  if (!fine->has_hg || fine->batched) {
    set_error("project_partition needs a single-instance fine session with a hypergraph");
    return LPGPU_ERR_STATE;
  }
  if (!coarse->has_part || coarse->batched) {
    set_error("project_partition needs a single-instance coarse session with a partition");
    return LPGPU_ERR_STATE;
  }
  if (coarse->device != fine->device) return invalid("both sessions must live on the same device");
  if (fine->n > 0 && !fine_to_coarse) return invalid("null fine-to-coarse map");
  DeviceGuard g(fine->device);
  CK(cudaStreamSynchronize(coarse->st));
  TmpBuf<int32_t> map(fine->mem), proj(fine->mem);
  TmpBuf<int64_t> check(fine->mem);
  CK(map.alloc(fine->n));
  CK(proj.alloc(fine->n));
  CK(check.alloc(1));
  if (fine->n > 0)
    CK(cudaMemcpyAsync(map.p(), fine_to_coarse, sizeof(int32_t) * fine->n, cudaMemcpyHostToDevice, fine->st));
  CK(launch_project(fine->launch(), fine->n, map.p(), coarse->part.p, coarse->n, proj.p(), check.p()));
  int64_t bad = 0;
  std::vector<int64_t> hl(coarse->k);
  CK(cudaMemcpyAsync(&bad, check.p(), sizeof(int64_t), cudaMemcpyDeviceToHost, fine->st));
  CK(cudaMemcpyAsync(hl.data(), coarse->lmax.p, sizeof(int64_t) * coarse->k, cudaMemcpyDeviceToHost, fine->st));
  CK(cudaStreamSynchronize(fine->st));
  if (bad) return invalid("fine-to-coarse map entry outside the coarse vertices");
  const std::vector<int64_t> hp = coarse->h_perfect;
  return set_partition_impl(fine, coarse->k, coarse->k, nullptr, hl, hp, nullptr, proj.p());
}

static lpgpu_status read_metrics(lpgpu_session* s, int64_t* km1, int64_t* cut);
static lpgpu_status read_imbalance(lpgpu_session* s, double* imb);

static lpgpu_status read_metrics(lpgpu_session* s, int64_t* km1, int64_t* cut) {
  RoundCtx c = s->ctx();
  CK(launch_metrics(s->launch(), c));
  int64_t h[2];
  CK(cudaMemcpyAsync(h, s->scal.p + kKm1, sizeof(h), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (km1) *km1 = h[0];
  if (cut) *cut = h[1];
  return LPGPU_OK;
}

static lpgpu_status read_imbalance(lpgpu_session* s, double* imb) {
  std::vector<int64_t> w(s->k);
  CK(cudaMemcpyAsync(w.data(), s->bw.p, sizeof(int64_t) * s->k, cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  // metrics::imbalance (metrics.cpp:114-128)
  double mx = (double)w[0] / (double)s->h_perfect[0];
  for (int b = 1; b < s->k; ++b) mx = std::max(mx, (double)w[b] / (double)s->h_perfect[b]);
  *imb = mx - 1.0;
  return LPGPU_OK;
}

static lpgpu_status need_part(lpgpu_session* s) {
  if (!s) return invalid("null session");
  if (!s->has_part) {
    set_error("no partition set");
    return LPGPU_ERR_STATE;
  }
  return LPGPU_OK;
}

// ---- tuning (the autotuner's table and per-session choices)

static std::mutex g_tuning_mutex;
static std::vector<lpgpu_tuning_entry> g_tuning_table;

// The multi-launch form; when the persistent form is forced by the flag, its
// kernel parameters are the ones the autotuner picked on every size class
// where it won (2 CTAs per SM, unroll 8, largest instance first).
static lpgpu_tuning default_tuning() {
  lpgpu_tuning t{};
  t.mode = LPGPU_MODE_MULTI_LAUNCH;
  t.ctas_per_sm = 2;
  t.unroll = 8;
  t.order = 0;
  return t;
}

static bool valid_tuning(const lpgpu_tuning& t) {
  return (t.mode == LPGPU_MODE_MULTI_LAUNCH || t.mode == LPGPU_MODE_PERSISTENT) &&
         (t.ctas_per_sm == 1 || t.ctas_per_sm == 2) && (t.unroll == 4 || t.unroll == 8) &&
         (t.order == 0 || t.order == 1);
}

// The session's tuning, else the first table row whose instance count and
// mean instance size it meets, else the multi-launch form.
static lpgpu_tuning session_tuning(const lpgpu_session* s) {
  if (s->has_tuning) return s->tuning;
  const int64_t count = s->batched ? s->num_inst : 1;
  int64_t pins = 0;
  for (int64_t p : s->h_inst_pins) pins += p;
  const int64_t mean = count > 0 ? pins / count : 0;
  std::lock_guard<std::mutex> lock(g_tuning_mutex);
  for (const lpgpu_tuning_entry& e : g_tuning_table)
    if (count >= e.min_instances && mean <= e.max_mean_pins) return e.tuning;
  return default_tuning();
}

// Instance descriptors of the persistent rounds over the session's current
// buffers, and the work order (rebuilt when a buffer or the order changed).
static lpgpu_status build_px(lpgpu_session* s, int order) {
  const int32_t I = s->batched ? s->num_inst : 1;
  const std::vector<int64_t> key = {
      (int64_t)s->stats.p, (int64_t)s->part.p, (int64_t)s->phi.p,  (int64_t)s->conn.p,      (int64_t)s->bw.p,
      (int64_t)s->rec.p,   (int64_t)s->seg_key.p, (int64_t)s->revl.p, (int64_t)s->next_flag.p, (int64_t)s->net_off.p,
      (int64_t)s->inets.p, (int64_t)s->lmax.p, order, s->kmax, s->k, s->W, s->n, s->m, I, s->max_we,
      s->unit_nets ? 1 : 0};
  if (s->px.p && s->px_key == key) return LPGPU_OK;
  std::vector<PxInst> h(I);
  for (int32_t i = 0; i < I; ++i) {
    PxInst& x = h[i];
    x.net_off = s->net_off.p;
    x.pins = s->pins.p;
    x.vtx_off = s->vtx_off.p;
    x.inets = s->inets.p;
    x.w_v = s->w_v.p;
    x.w_e = s->w_e.p;
    x.part = s->part.p;
    x.phi = s->phi.p;
    x.conn = s->conn.p;
    x.bw = s->bw.p;
    x.lmax = s->lmax.p;
    x.perfect = s->perfect.p;
    x.flag = s->next_flag.p;
    x.rec = s->rec.p;
    x.status = s->status.p;
    x.v0 = s->h_inst_voff[i];
    x.v1 = s->h_inst_voff[i + 1];
    x.keys = s->seg_key.p + x.v0;
    x.kw = s->seg_w.p + x.v0;
    x.cand = s->revl.p + x.v0;
    x.net_epoch = s->net_epoch.p;
    x.stats = s->stats.p;
    x.boff = s->batched ? s->h_inst_boff[i] : 0;
    x.k = s->batched ? s->h_inst_k[i] : s->k;
    x.kstride = s->batched ? s->kmax : s->k;
    x.W = s->W;
    x.unit_nets = s->unit_nets ? 1 : 0;
    x.phi16 = s->phi16() ? 1 : 0;
    x.max_we = s->max_we;
    x.round = 0;
  }
  std::vector<int32_t> ord(I);
  for (int32_t i = 0; i < I; ++i) ord[i] = i;
  if (order == 0)  // largest instance first: the longest jobs start first on the work queue
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int32_t a, int32_t b) { return s->h_inst_pins[a] > s->h_inst_pins[b]; });
  Mem* fp = &s->mem;
  CK(s->px.alloc(I, fp));
  CK(s->px_order.alloc(I, fp));
  CK(cudaMemcpyAsync(s->px.p, h.data(), sizeof(PxInst) * I, cudaMemcpyHostToDevice, s->st));
  s->h_px = h;
  CK(cudaMemcpyAsync(s->px_order.p, ord.data(), sizeof(int32_t) * I, cudaMemcpyHostToDevice, s->st));
  CK(cudaStreamSynchronize(s->st));
  s->px_key = key;
  return LPGPU_OK;
}

lpgpu_status lpgpu_set_tuning_table(const lpgpu_tuning_entry* entries, int32_t count) {
  if (count < 0 || (count > 0 && !entries)) return invalid("bad tuning table");
  for (int32_t i = 0; i < count; ++i)
    if (!valid_tuning(entries[i].tuning)) return invalid("tuning row " + std::to_string(i) + " is out of range");
  std::lock_guard<std::mutex> lock(g_tuning_mutex);
  g_tuning_table.assign(entries, entries + count);
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_set_tuning(lpgpu_session* s, const lpgpu_tuning* t) {
  if (!s) return invalid("null session");
  if (t && !valid_tuning(*t)) return invalid("tuning out of range");
  s->has_tuning = t != nullptr;
  if (t) s->tuning = *t;
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_tuning(lpgpu_session* s, lpgpu_tuning* out) {
  if (!s || !out) return invalid("null argument");
  *out = session_tuning(s);
  return LPGPU_OK;
}

// Statistics of R rounds (hs: R x kStats, rounds after the first one without
// an active vertex did not run) into last_stats and the refine result
// (IRefiner::refine's metrics update, label_propagation_refiner.cpp:48-67).
static lpgpu_status book_rounds(lpgpu_session* s, const std::vector<int64_t>& hs, int R, int64_t km1_before,
                                lpgpu_result* result) {
  s->last_stats.clear();
  int executed = 0;
  bool stopped = false;
  int64_t delta = 0, moves = 0, pins = 0;
  for (int r = 0; r < R; ++r) {
    const int64_t* x = &hs[(size_t)r * kStats];
    if (x[kStActive] == 0) stopped = true;
    if (stopped) continue;
    lpgpu_round_stats rs{x[kStActive], x[kStPins],  x[kStCands],     x[kStMoved],
                         x[kStReverted], x[kStDelta], x[kStMovedPins], x[kStToggles]};
    s->last_stats.push_back(rs);
    ++executed;
    delta += rs.delta;
    moves += rs.moved;
    pins += rs.pins;
  }
  if (result) {
    int64_t km1_after = 0;
    lpgpu_status ms = read_metrics(s, &km1_after, nullptr);
    if (ms != LPGPU_OK) return ms;
    double imb = 0;
    ms = read_imbalance(s, &imb);
    if (ms != LPGPU_OK) return ms;
    result->km1_before = km1_before;
    result->km1_after = km1_after;
    result->delta = delta;
    result->moves = moves;
    result->pins_processed = pins;
    result->rounds = executed;
    result->improved = delta < 0;
    result->imbalance = imb;
  }
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_refine(lpgpu_session* s, const lpgpu_config* cfg_in,
                                  const int32_t* nodes, int64_t num_nodes, lpgpu_result* result) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  lpgpu_config cfg;
  if (cfg_in) cfg = *cfg_in; else lpgpu_config_default(&cfg);
  if (cfg.rounds < 0) return invalid("rounds must be >= 0");
  if (cfg.subrounds < 1 || cfg.subrounds > kMaxSubrounds) return invalid("subrounds must be in [1, 64]");
  if (num_nodes < 0 || (num_nodes > 0 && !nodes)) return invalid("bad refinement node list");
  if ((cfg.flags & LPGPU_FLAG_PERSISTENT) && (cfg.flags & LPGPU_FLAG_MULTI_LAUNCH))
    return invalid("LPGPU_FLAG_PERSISTENT and LPGPU_FLAG_MULTI_LAUNCH exclude each other");
  for (int64_t i = 0; i < num_nodes; ++i)
    if (nodes[i] < 0 || nodes[i] >= s->n) return invalid("refinement node out of range");
  // persistent rounds: forced by the flag, or chosen by the tuning when eligible
  const lpgpu_tuning tu = session_tuning(s);
  const bool px_ok = num_nodes == 0 && (s->batched ? s->kmax : s->k) <= kPxMaxK;
  bool use_px = tu.mode == LPGPU_MODE_PERSISTENT;
  if (cfg.flags & LPGPU_FLAG_PERSISTENT) {
    if (!px_ok) return invalid("persistent rounds need every k <= 64 and no refinement node list");
    use_px = true;
  }
  if (cfg.flags & LPGPU_FLAG_MULTI_LAUNCH) use_px = false;
  use_px = use_px && px_ok;
  DeviceGuard g(s->device);
  s->gc_valid = false;  // refinement moves without gain-cache maintenance
  const int R = cfg.rounds, S = cfg.subrounds;
  Mem* fp = &s->mem;
  CK(s->stats.alloc(std::max(1, R) * kStats, fp));
  if (use_px) {
    ps = build_px(s, tu.order);
    if (ps != LPGPU_OK) return ps;
  }
  PxParams pxp{};
  pxp.S = S;
  pxp.zero_gain = cfg.rebalancing ? 1 : 0;
  pxp.revert = cfg.revert;
  pxp.rollback = cfg.rollback;
  pxp.act_threshold = cfg.activation_threshold <= 0 ? INT64_MAX : cfg.activation_threshold;
  pxp.unroll = tu.unroll;
  const int32_t px_count = s->batched ? s->num_inst : 1;
  cudaStream_t st = s->st;
  int64_t km1_before = 0;
  lpgpu_status ms = read_metrics(s, &km1_before, nullptr);
  if (ms != LPGPU_OK) return ms;
  RoundCtx c = s->ctx(&cfg);
  const Launch L = s->launch();
  TmpBuf<int32_t> dnodes(s->mem);
  if (num_nodes > 0) {
    CK(dnodes.alloc(num_nodes));
    CK(cudaMemcpyAsync(dnodes.p(), nodes, sizeof(int32_t) * num_nodes, cudaMemcpyHostToDevice, st));
  }
  PhaseTimer* tm = s->timing ? &s->timer : nullptr;
  // The whole refine is a fixed sequence of launches whose element counts live
  // in device memory, so it is captured once as a CUDA graph and replayed.
  auto enqueue = [&]() -> cudaError_t {
    cudaError_t e;
    if ((e = cudaMemsetAsync(s->stats.p, 0, sizeof(int64_t) * std::max(1, R) * kStats, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s->blk64.p, 0, sizeof(int64_t) * (7 * s->k + 1), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s->scal.p, 0, sizeof(int64_t) * kScalars, st)) != cudaSuccess) return e;
    if (s->m > 0 && (e = cudaMemsetAsync(s->net_epoch.p, 0, sizeof(int32_t) * s->m, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s->bin_cnt.p, 0, sizeof(int64_t) * kMaxSubrounds * kDegClasses, st)) != cudaSuccess)
      return e;
    if (s->batched && (e = cudaMemsetAsync(s->inst_delta.p, 0, sizeof(int64_t) * s->num_inst, st)) != cudaSuccess)
      return e;
    if (num_nodes > 0) {
      if ((e = launch_mark_list(L, c, dnodes.p(), num_nodes)) != cudaSuccess) return e;
    } else {
      if (s->n > 0 && (e = cudaMemsetAsync(s->next_flag.p, 0, s->n, st)) != cudaSuccess) return e;
      if ((e = launch_mark_all(L, c, cfg.rebalancing)) != cudaSuccess) return e;
    }
    if (use_px) {  // one persistent launch per round
      for (int r = 0; r < R; ++r) {
        pxp.round = r;
        if ((e = launch_px_round(L, s->px.p, s->px_order.p, px_count, pxp, s->W, s->unit_nets, tu.ctas_per_sm,
                                 s->scal.p + kPxQueue)) != cudaSuccess)
          return e;
      }
      if (s->n > 0 && (e = cudaMemsetAsync(s->next_flag.p, 0, s->n, st)) != cudaSuccess) return e;
      return cudaSuccess;
    }
    for (int r = 0; r < R; ++r) {
      if ((e = launch_bin_active(L, c, r, S, s->bin_cnt.p, tm)) != cudaSuccess) return e;
      for (int sub = 0; sub < S; ++sub)
        if ((e = launch_subround(L, c, r, sub, tm)) != cudaSuccess) return e;
      if (r + 1 < R && (e = launch_expand_nets(L, c, S, tm)) != cudaSuccess) return e;
    }
    // drop flags left by the last round
    if (s->n > 0 && (e = cudaMemsetAsync(s->next_flag.p, 0, s->n, st)) != cudaSuccess) return e;
    return cudaSuccess;
  };
  if (num_nodes > 0 || tm || (cfg.flags & LPGPU_FLAG_NO_GRAPH)) {
    // direct launches: explicit node lists, and per-phase event timing
    if (tm) tm->reset();
    CK(enqueue());
  } else {
    // key: every pointer and parameter baked into the captured launches
    struct Key {
      RoundCtx c;
      int R, S, timing, px;
      int64_t* p[1];
      lpgpu_tuning tu;
      const void* px_ptr[2];
      int32_t px_count;
    } key;
    std::memset(&key, 0, sizeof(key));
    key.c = c;
    key.R = R;
    key.S = S;
    key.timing = 0;
    key.px = use_px ? 1 : 0;
    if (use_px) {
      key.tu = tu;
      key.px_ptr[0] = s->px.p;
      key.px_ptr[1] = s->px_order.p;
      key.px_count = px_count;
    }
    key.p[0] = s->bin_cnt.p;
    std::vector<unsigned char> kb(reinterpret_cast<unsigned char*>(&key),
                                  reinterpret_cast<unsigned char*>(&key) + sizeof(key));
    if (!s->graph || s->graph_key != kb) {
      if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
      }
      cudaGraph_t g0 = nullptr;
      const int64_t l0 = kernel_launches();
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
      const cudaError_t ce = enqueue();
      const cudaError_t ee = cudaStreamEndCapture(st, &g0);
      s->graph_kernels = kernel_launches() - l0;
      add_kernel_launches(-s->graph_kernels);  // recorded, not run
      if (ce != cudaSuccess) {
        if (g0) cudaGraphDestroy(g0);
        return cuda_fail(ce, "enqueue refine (capture)");
      }
      CK(ee);
      const cudaError_t ie = cudaGraphInstantiate(&s->graph, g0, 0);
      cudaGraphDestroy(g0);
      CK(ie);
      s->graph_key = kb;
    }
    CK(cudaGraphLaunch(s->graph, st));
    add_kernel_launches(s->graph_kernels);
  }
  std::vector<int64_t> hs(std::max(1, R) * kStats);
  CK(cudaMemcpyAsync(hs.data(), s->stats.p, sizeof(int64_t) * hs.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (tm) {
    std::map<int, lpgpu_phase_time> acc;
    for (auto& rec : tm->recs) {
      float ms_ = 0.f;
      CK(cudaEventElapsedTime(&ms_, rec.a, rec.b));
      auto& a = acc[rec.phase];
      a.launches += 1;
      a.ms += ms_;
    }
    s->phase_times.clear();
    for (auto& kv : acc) {
      lpgpu_phase_time t = kv.second;
      std::memset(t.name, 0, sizeof(t.name));
      std::strncpy(t.name, tm->names[kv.first].c_str(), sizeof(t.name) - 1);
      s->phase_times.push_back(t);
    }
  }
  return book_rounds(s, hs, R, km1_before, result);
}

// ---- stepped refinement: one persistent round of many sessions per launch

lpgpu_status lpgpu_session_begin_rounds(lpgpu_session* s, const lpgpu_config* cfg_in) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  lpgpu_config cfg;
  if (cfg_in) cfg = *cfg_in; else lpgpu_config_default(&cfg);
  if (cfg.rounds < 0) return invalid("rounds must be >= 0");
  if (cfg.subrounds < 1 || cfg.subrounds > kMaxSubrounds) return invalid("subrounds must be in [1, 64]");
  if ((s->batched ? s->kmax : s->k) > kPxMaxK) return invalid("stepped rounds need every k <= 64");
  DeviceGuard g(s->device);
  s->gc_valid = false;
  const int R = cfg.rounds;
  cudaStream_t st = s->st;
  CK(s->stats.alloc(std::max(1, R) * kStats, &s->mem));
  ps = build_px(s, 0);
  if (ps != LPGPU_OK) return ps;
  ps = read_metrics(s, &s->step_km1_before, nullptr);
  if (ps != LPGPU_OK) return ps;
  if (!s->step_ev) CK(cudaEventCreateWithFlags(&s->step_ev, cudaEventDisableTiming));
  RoundCtx c = s->ctx(&cfg);
  CK(cudaMemsetAsync(s->stats.p, 0, sizeof(int64_t) * std::max(1, R) * kStats, st));
  if (s->m > 0) CK(cudaMemsetAsync(s->net_epoch.p, 0, sizeof(int32_t) * s->m, st));
  if (s->n > 0) CK(cudaMemsetAsync(s->next_flag.p, 0, s->n, st));
  CK(launch_mark_all(s->launch(), c, cfg.rebalancing));
  s->step_cfg = cfg;
  s->step_round = 0;
  s->step_done = R == 0;
  s->stepping = true;
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_end_rounds(lpgpu_session* s, lpgpu_result* result) {
  if (!s) return invalid("null session");
  if (!s->stepping) {
    set_error("no stepped refinement was begun");
    return LPGPU_ERR_STATE;
  }
  DeviceGuard g(s->device);
  const int R = s->step_cfg.rounds;
  std::vector<int64_t> hs((size_t)std::max(1, R) * kStats);
  CK(cudaMemcpyAsync(hs.data(), s->stats.p, sizeof(int64_t) * hs.size(), cudaMemcpyDeviceToHost, s->st));
  if (s->n > 0) CK(cudaMemsetAsync(s->next_flag.p, 0, s->n, s->st));
  CK(cudaStreamSynchronize(s->st));
  s->stepping = false;
  return book_rounds(s, hs, R, s->step_km1_before, result);
}

}  // extern "C"

struct lpgpu_stepper_s {
  int device = 0;
  cudaStream_t st = nullptr;
  int num_sms = 1;
  Mem mem;
  DevBuf<PxInst> table;
  DevBuf<int64_t> active, queue;
  cudaEvent_t ev = nullptr;
  std::vector<lpgpu_session*> pending;  // sessions of the launched round
  std::vector<int32_t> first;           // their first row of the table
  std::vector<PxInst> h;
};

extern "C" {

lpgpu_status lpgpu_stepper_create(int32_t device, lpgpu_stepper** out) {
  if (!out) return invalid("null output pointer");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    set_error(std::string("no CUDA device: ") + cudaGetErrorString(e));
    cudaGetLastError();
    return LPGPU_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return invalid("device index out of range");
  DeviceGuard g(device);
  auto* t = new lpgpu_stepper_s();
  t->device = device;
  cudaDeviceProp prop;
  if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking)) != cudaSuccess) {
    delete t;
    return cuda_fail(e, "stepper stream");
  }
  t->num_sms = prop.multiProcessorCount;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  if ((e = cudaMemPoolCreate(&t->mem.pool, &props)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&t->ev, cudaEventDisableTiming)) != cudaSuccess) {
    if (t->mem.pool) cudaMemPoolDestroy(t->mem.pool);
    cudaStreamDestroy(t->st);
    delete t;
    return cuda_fail(e, "stepper pool");
  }
  t->mem.st = t->st;
  *out = t;
  return LPGPU_OK;
}

lpgpu_status lpgpu_stepper_destroy(lpgpu_stepper* t) {
  if (!t) return LPGPU_OK;
  {
    DeviceGuard g(t->device);
    cudaStreamSynchronize(t->st);
    t->table.release(&t->mem);
    t->active.release(&t->mem);
    t->queue.release(&t->mem);
    cudaStreamSynchronize(t->st);
    cudaEventDestroy(t->ev);
    cudaMemPoolDestroy(t->mem.pool);
    cudaStreamDestroy(t->st);
  }
  delete t;
  return LPGPU_OK;
}

lpgpu_status lpgpu_stepper_launch(lpgpu_stepper* t, lpgpu_session* const* sessions, int32_t count) {
  if (!t) return invalid("null stepper");
  if (count < 0 || (count > 0 && !sessions)) return invalid("bad session list");
  if (!t->pending.empty()) {
    set_error("the previous round was not waited for");
    return LPGPU_ERR_STATE;
  }
  for (int32_t i = 0; i < count; ++i) {
    const lpgpu_session* s = sessions[i];
    if (!s) return invalid("null session in the list");
    if (!s->stepping || s->step_done) {
      set_error("session " + std::to_string(i) + " has no round left to run");
      return LPGPU_ERR_STATE;
    }
    if (s->device != t->device) return invalid("session on another device");
    for (int32_t j = 0; j < i; ++j)
      if (sessions[j] == s) return invalid("session listed twice");
  }
  DeviceGuard g(t->device);
  // launches group the sessions whose round parameters agree
  struct Group {
    int W, unit, S, zero_gain, revert, rollback;
    int64_t act;
    bool operator<(const Group& o) const {
      return std::tie(W, unit, S, zero_gain, revert, rollback, act) <
             std::tie(o.W, o.unit, o.S, o.zero_gain, o.revert, o.rollback, o.act);
    }
  };
  std::map<Group, std::vector<int32_t>> groups;
  for (int32_t i = 0; i < count; ++i) {
    const lpgpu_session* s = sessions[i];
    const lpgpu_config& c = s->step_cfg;
    Group key{s->W, s->unit_nets ? 1 : 0, c.subrounds, c.rebalancing ? 1 : 0, c.revert, c.rollback,
              c.activation_threshold <= 0 ? INT64_MAX : (int64_t)c.activation_threshold};
    groups[key].push_back(i);
  }
  t->h.clear();
  t->first.assign(count, 0);
  std::vector<std::pair<Group, std::pair<int32_t, int32_t>>> ranges;  // group, (first row, rows)
  for (auto& kv : groups) {
    const int32_t beg = (int32_t)t->h.size();
    for (int32_t i : kv.second) {
      lpgpu_session* s = sessions[i];
      t->first[i] = (int32_t)t->h.size();
      for (PxInst x : s->h_px) {
        x.round = s->step_round;
        t->h.push_back(x);
      }
      // the stepper's stream waits for the session's own work (uploads, begin)
      CK(cudaEventRecord(s->step_ev, s->st));
      CK(cudaStreamWaitEvent(t->st, s->step_ev, 0));
    }
    ranges.push_back({kv.first, {beg, (int32_t)t->h.size() - beg}});
  }
  const size_t rows = t->h.size();
  if (rows > t->table.count) {
    CK(t->table.alloc(rows, &t->mem));
    CK(t->active.alloc(rows, &t->mem));
  }
  if (!t->queue.p) CK(t->queue.alloc(1, &t->mem));
  if (rows > 0)
    CK(cudaMemcpyAsync(t->table.p, t->h.data(), sizeof(PxInst) * rows, cudaMemcpyHostToDevice, t->st));
  const Launch L{t->st, t->num_sms};
  for (const auto& gr : ranges) {
    const Group& k = gr.first;
    // the kernel build of the group's first session's tuning when that is a
    // persistent one, else 2 CTAs per SM with unroll 8
    const lpgpu_tuning tu = session_tuning(sessions[groups[k].front()]);
    const bool tuned = tu.mode == LPGPU_MODE_PERSISTENT;
    PxParams P{};
    P.S = k.S;
    P.zero_gain = k.zero_gain;
    P.revert = k.revert;
    P.rollback = k.rollback;
    P.act_threshold = k.act;
    P.round = -1;  // every instance runs its own round
    P.unroll = tuned ? tu.unroll : 8;
    CK(launch_px_round(L, t->table.p + gr.second.first, nullptr, gr.second.second, P, k.W, k.unit != 0,
                       tuned ? tu.ctas_per_sm : 2, t->queue.p));
  }
  if (rows > 0) CK(launch_px_active(L, t->table.p, (int32_t)rows, t->active.p));
  // the sessions' later work (downloads, the next round's inputs) comes after this round
  CK(cudaEventRecord(t->ev, t->st));
  for (int32_t i = 0; i < count; ++i) CK(cudaStreamWaitEvent(sessions[i]->st, t->ev, 0));
  t->pending.assign(sessions, sessions + count);
  return LPGPU_OK;
}

lpgpu_status lpgpu_stepper_wait(lpgpu_stepper* t, int32_t* done) {
  if (!t) return invalid("null stepper");
  DeviceGuard g(t->device);
  const size_t rows = t->h.size();
  std::vector<int64_t> act(rows);
  if (rows > 0) CK(cudaMemcpyAsync(act.data(), t->active.p, sizeof(int64_t) * rows, cudaMemcpyDeviceToHost, t->st));
  CK(cudaStreamSynchronize(t->st));
  for (size_t i = 0; i < t->pending.size(); ++i) {
    lpgpu_session* s = t->pending[i];
    int64_t a = 0;
    for (size_t j = 0; j < s->h_px.size(); ++j) a += act[t->first[i] + j];
    s->step_round += 1;
    s->step_done = s->step_round >= s->step_cfg.rounds || a == 0;
    if (done) done[i] = s->step_done ? 1 : 0;
  }
  t->pending.clear();
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_round_stats(lpgpu_session* s, lpgpu_round_stats* out, int32_t max_rounds,
                                       int32_t* rounds) {
  if (!s) return invalid("null session");
  const int cnt = (int)std::min<size_t>(s->last_stats.size(), (size_t)std::max(0, max_rounds));
  for (int i = 0; i < cnt; ++i) out[i] = s->last_stats[i];
  if (rounds) *rounds = (int32_t)s->last_stats.size();
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_get_partition(lpgpu_session* s, int32_t* partition) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  DeviceGuard g(s->device);
  const int32_t* src = s->part.p;
  if (s->batched) {  // global block ids back to instance-local ids, staged in the selection scratch
    CK(launch_local_blocks(s->launch(), s->n, s->part.p, s->vinst.p, s->inst_boff.p, s->seg_w.p));
    src = s->seg_w.p;
  }
  if (s->n > 0) CK(cudaMemcpyAsync(partition, src, sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_get_partition_instances(lpgpu_session* s, int32_t* const* partitions) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  if (!s->batched) {
    set_error("get_partition_instances needs a batched session");
    return LPGPU_ERR_STATE;
  }
  if (!partitions) return invalid("null output");
  for (int32_t i = 0; i < s->num_inst; ++i)
    if (!partitions[i] && s->h_inst_voff[i + 1] > s->h_inst_voff[i]) return invalid("null output");
  DeviceGuard g(s->device);
  CK(launch_local_blocks(s->launch(), s->n, s->part.p, s->vinst.p, s->inst_boff.p, s->seg_w.p));
  CopyRun run{s->st, cudaMemcpyDeviceToHost};
  for (int32_t i = 0; i < s->num_inst; ++i) {
    const int64_t v0 = s->h_inst_voff[i], ni = s->h_inst_voff[i + 1] - v0;
    if (ni > 0) CK(run.add(partitions[i], s->seg_w.p + v0, sizeof(int32_t) * ni));
  }
  CK(run.flush());
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_instance_km1(lpgpu_session* s, int64_t* km1) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  if (!km1) return invalid("null output");
  DeviceGuard g(s->device);
  if (!s->batched) {
    return read_metrics(s, km1, nullptr);
  }
  TmpBuf<int64_t> d(s->mem);
  CK(d.alloc(s->num_inst));
  RoundCtx c = s->ctx();
  CK(launch_instance_metrics(s->launch(), c, d.p()));
  CK(cudaMemcpyAsync(km1, d.p(), sizeof(int64_t) * s->num_inst, cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_metrics(lpgpu_session* s, int64_t* km1, int64_t* cut, double* imbalance) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  DeviceGuard g(s->device);
  ps = read_metrics(s, km1, cut);
  if (ps != LPGPU_OK) return ps;
  if (imbalance) return read_imbalance(s, imbalance);
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_get_block_weights(lpgpu_session* s, int64_t* weights) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  DeviceGuard g(s->device);
  CK(cudaMemcpyAsync(weights, s->bw.p, sizeof(int64_t) * s->k, cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_get_pin_counts(lpgpu_session* s, int32_t* pc) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  DeviceGuard g(s->device);
  const size_t entries = (size_t)s->m * s->kmax;
  if (entries > 0 && !s->phi16()) {
    CK(cudaMemcpyAsync(pc, s->phi.p, sizeof(int32_t) * entries, cudaMemcpyDeviceToHost, s->st));
  } else if (entries > 0) {  // 16-bit entries: widened on the host
    std::vector<uint16_t> h(entries);
    CK(cudaMemcpyAsync(h.data(), s->phi.p, sizeof(uint16_t) * entries, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    for (size_t i = 0; i < entries; ++i) pc[i] = h[i];
  }
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_get_connectivity(lpgpu_session* s, uint32_t* words) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  DeviceGuard g(s->device);
  const int wc = word_count(s->kmax);
  if (s->m > 0) {
    // device rows hold 2W words (W >= wc words of Λ, then Λ1); copy the first wc of every row
    CK(cudaMemcpy2DAsync(words, sizeof(uint32_t) * wc, s->conn.p, sizeof(uint32_t) * 2 * s->W,
                         sizeof(uint32_t) * wc, s->m, cudaMemcpyDeviceToHost, s->st));
  }
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_get_incidence(lpgpu_session* s, int64_t* vtx_off, int32_t* inets) {
  if (!s) return invalid("null session");
  if (!s->has_hg) {
    set_error("no hypergraph uploaded");
    return LPGPU_ERR_STATE;
  }
  DeviceGuard g(s->device);
  if (vtx_off) CK(cudaMemcpyAsync(vtx_off, s->vtx_off.p, sizeof(int64_t) * (s->n + 1), cudaMemcpyDeviceToHost, s->st));
  if (inets && s->P > 0) CK(cudaMemcpyAsync(inets, s->inets.p, sizeof(int32_t) * s->P, cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_best_moves(lpgpu_session* s, int32_t* to, int32_t* gain, uint8_t* border) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  if (s->batched) {
    set_error("this query needs a single-instance session");
    return LPGPU_ERR_STATE;
  }
  DeviceGuard g(s->device);
  TmpBuf<int32_t> dto(s->mem), dgain(s->mem);
  TmpBuf<uint8_t> dborder(s->mem);
  CK(dto.alloc(s->n));
  CK(dgain.alloc(s->n));
  CK(dborder.alloc(s->n));
  RoundCtx c = s->ctx();
  CK(launch_best_moves(s->launch(), c, dto.p(), dgain.p(), dborder.p()));
  if (s->n > 0) {
    if (to) CK(cudaMemcpyAsync(to, dto.p(), sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost, s->st));
    if (gain) CK(cudaMemcpyAsync(gain, dgain.p(), sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost, s->st));
    if (border) CK(cudaMemcpyAsync(border, dborder.p(), s->n, cudaMemcpyDeviceToHost, s->st));
  }
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_gain_cache(lpgpu_session* s, int32_t* benefit, int32_t* penalty) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  if (s->batched) {
    set_error("this query needs a single-instance session");
    return LPGPU_ERR_STATE;
  }
  DeviceGuard g(s->device);
  TmpBuf<int32_t> db(s->mem), dp(s->mem);
  const int32_t *sb = s->gc_benefit.p, *sp = s->gc_penalty.p;
  if (!s->gc_valid) {  // computed for this call
    CK(db.alloc(s->n));
    CK(dp.alloc((size_t)s->n * s->k));
    RoundCtx c = s->ctx();
    CK(launch_gain_cache(s->launch(), c, db.p(), dp.p()));
    sb = db.p();
    sp = dp.p();
  }
  if (s->n > 0) {
    if (benefit) CK(cudaMemcpyAsync(benefit, sb, sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost, s->st));
    if (penalty) CK(cudaMemcpyAsync(penalty, sp, sizeof(int32_t) * s->n * s->k, cudaMemcpyDeviceToHost, s->st));
  }
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_init_gain_cache(lpgpu_session* s) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  if (s->batched) {
    set_error("this call needs a single-instance session");
    return LPGPU_ERR_STATE;
  }
  DeviceGuard g(s->device);
  Mem* fp = &s->mem;
  CK(s->gc_benefit.alloc(s->n, fp));
  CK(s->gc_penalty.alloc((size_t)s->n * s->k, fp));
  CK(s->gc_moved.alloc(s->n, fp));
  if (s->n > 0) CK(cudaMemsetAsync(s->gc_moved.p, 0, s->n, s->st));
  RoundCtx c = s->ctx();
  CK(launch_gain_cache(s->launch(), c, s->gc_benefit.p, s->gc_penalty.p));
  CK(cudaStreamSynchronize(s->st));
  s->gc_valid = true;
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_drop_gain_cache(lpgpu_session* s) {
  if (!s) return invalid("null session");
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  s->drop_gain_cache();
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_apply_moves(lpgpu_session* s, int64_t count, const int32_t* vs,
                                       const int32_t* fs, const int32_t* ts, int64_t* delta) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  if (s->batched) {
    set_error("this call needs a single-instance session");
    return LPGPU_ERR_STATE;
  }
  if (count < 0 || (count > 0 && (!vs || !fs || !ts))) return invalid("bad move list");
  DeviceGuard g(s->device);
  std::vector<int32_t> part(s->n);
  if (s->n > 0) {
    CK(cudaMemcpyAsync(part.data(), s->part.p, sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
  }
  std::vector<uint8_t> seen(s->n, 0);
  for (int64_t i = 0; i < count; ++i) {
    if (vs[i] < 0 || vs[i] >= s->n) return invalid("move vertex out of range");
    if (ts[i] < 0 || ts[i] >= s->k || fs[i] < 0 || fs[i] >= s->k) return invalid("move block out of range");
    if (fs[i] == ts[i]) return invalid("move with from == to");
    if (part[vs[i]] != fs[i]) return invalid("move source is not the vertex's current block");
    if (seen[vs[i]]) return invalid("vertex moved twice in one batch");
    seen[vs[i]] = 1;
  }
  TmpBuf<int32_t> dv(s->mem), df(s->mem), dt(s->mem);
  CK(dv.alloc(count));
  CK(df.alloc(count));
  CK(dt.alloc(count));
  if (count > 0) {
    CK(cudaMemcpyAsync(dv.p(), vs, sizeof(int32_t) * count, cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(df.p(), fs, sizeof(int32_t) * count, cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(dt.p(), ts, sizeof(int32_t) * count, cudaMemcpyHostToDevice, s->st));
  }
  RoundCtx c = s->ctx();
  GainCache gc{nullptr, nullptr, nullptr};
  if (s->gc_valid) gc = GainCache{s->gc_benefit.p, s->gc_penalty.p, s->gc_moved.p};
  CK(launch_apply_moves(s->launch(), c, count, dv.p(), df.p(), dt.p(), gc));
  int64_t d = 0;
  CK(cudaMemcpyAsync(&d, s->scal.p + kApplyDelta, sizeof(int64_t), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (delta) *delta = d;
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_footprint(lpgpu_session* s, int64_t* bytes) {
  if (!s || !bytes) return invalid("null pointer");
  *bytes = s->mem.bytes;
  return LPGPU_OK;
}

int64_t lpgpu_estimate_footprint(int64_t n, int64_t m, int64_t P, int32_t k, int32_t subrounds) {
  (void)subrounds;
  const int64_t W = word_class_of(std::max(1, k));
  int64_t b = 0;
  b += 8 * (m + 1) + 8 * (n + 1) + 4 * P * 2 + 4 * n + 4 * m;          // CSR + weights
  b += 4 * m + 4 * n + n + n + 16 * n + 8 * n + 4 * n + 8 * n;         // epoch, list, flags, status, rec, seg, queues
  b += 8 * (2 * kMaxSubrounds + 1) + 8 * 2 * kMaxSubrounds * kDegClasses;  // sub-round bins
  b += 8 * (scan_tmp_elems(n + 1) + 1);
  b += 4 * n + 4 * m * (int64_t)k + 8 * m * W;                         // part, Φ, Λ + Λ1
  b += 8 * (3 * k + 7 * k + 1 + 2 * k) + 2 * k + 8 * 64 + 8 * 8;       // per-block, stats, scalars
  return b;
}

lpgpu_status lpgpu_session_save_partition(lpgpu_session* s) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  DeviceGuard g(s->device);
  CK(s->saved_part.alloc(s->n, &s->mem));
  if (s->n > 0)
    CK(cudaMemcpyAsync(s->saved_part.p, s->part.p, sizeof(int32_t) * s->n, cudaMemcpyDeviceToDevice, s->st));
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_restore_partition(lpgpu_session* s) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  if (s->saved_part.count != (size_t)s->n || (s->n > 0 && !s->saved_part.p)) {
    set_error("no saved partition");
    return LPGPU_ERR_STATE;
  }
  DeviceGuard g(s->device);
  s->gc_valid = false;
  if (s->n > 0)
    CK(cudaMemcpyAsync(s->part.p, s->saved_part.p, sizeof(int32_t) * s->n, cudaMemcpyDeviceToDevice, s->st));
  RoundCtx c = s->ctx();
  CK(launch_init_partition(s->launch(), c));
  return LPGPU_OK;
}

// The moves of repairEmptyBlocks (rebalancer.cpp:169-269) on the current
// state, in empty-block order: per empty block the device keeps the k
// eligible vertices of highest gain (lowest id on ties), and the first of
// them in (gain, weight of its block, id) descending order that no earlier
// block took is the block's move. Block weights are read into *bw_out.
struct RepairMove {
  int32_t v, from, to, gain, w;
};
static lpgpu_status repair_moves(lpgpu_session* s, std::vector<RepairMove>* moves, std::vector<int64_t>* bw_out) {
  const int k = s->k;
  cudaStream_t st = s->st;
  std::vector<int64_t>& bw = *bw_out;
  bw.assign(k, 0);
  CK(cudaMemcpyAsync(bw.data(), s->bw.p, sizeof(int64_t) * k, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  moves->clear();
  std::vector<int> empty;
  for (int b = 0; b < k; ++b)
    if (bw[b] == 0) empty.push_back(b);
  if (empty.empty() || s->n == 0) return LPGPU_OK;
  TmpBuf<int4> cand(s->mem);
  TmpBuf<int64_t> scratch(s->mem);
  CK(cand.alloc(k));
  CK(scratch.alloc(2));
  RoundCtx c = s->ctx();
  std::vector<int4> h(k);
  std::vector<uint8_t> used(s->n, 0);
  for (int blk : empty) {
    CK(launch_repair_candidates(s->launch(), c, blk, s->seg_key.p, s->seg_w.p, cand.p(), scratch.p()));
    int64_t count = 0;
    CK(cudaMemcpyAsync(&count, scratch.p(), sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (count > k) return cuda_fail(cudaErrorUnknown, "repair candidate count above k");
    if (count == 0) continue;
    CK(cudaMemcpyAsync(h.data(), cand.p(), sizeof(int4) * count, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::sort(h.begin(), h.begin() + count, [&](const int4& a, const int4& b) {
      if (a.y != b.y) return a.y > b.y;
      if (bw[a.z] != bw[b.z]) return bw[a.z] > bw[b.z];
      return a.x > b.x;
    });
    for (int64_t i = 0; i < count; ++i) {
      if (used[h[i].x]) continue;
      used[h[i].x] = 1;
      moves->push_back(RepairMove{h[i].x, h[i].z, blk, h[i].y, h[i].w});
      break;
    }
  }
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_repair_empty_blocks(lpgpu_session* s, int32_t* vertices, int32_t* from, int32_t* to,
                                               int32_t* gain, int32_t* count) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  if (s->batched) {
    set_error("this call needs a single-instance session");
    return LPGPU_ERR_STATE;
  }
  if (!count) return invalid("null count pointer");
  DeviceGuard g(s->device);
  std::vector<RepairMove> mv;
  std::vector<int64_t> bw;
  ps = repair_moves(s, &mv, &bw);
  if (ps != LPGPU_OK) return ps;
  if (!mv.empty() && (!vertices || !from || !to || !gain)) return invalid("null move output array");
  for (size_t i = 0; i < mv.size(); ++i) {
    vertices[i] = mv[i].v;
    from[i] = mv[i].from;
    to[i] = mv[i].to;
    gain[i] = mv[i].gain;
  }
  *count = (int32_t)mv.size();
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_rebalance(lpgpu_session* s, int32_t max_rounds, lpgpu_result* result) {
  lpgpu_status ps = need_part(s);
  if (ps != LPGPU_OK) return ps;
  if (s->batched) {
    set_error("this call needs a single-instance session");
    return LPGPU_ERR_STATE;
  }
  if (max_rounds < 0) return invalid("max_rounds must be >= 0");
  DeviceGuard g(s->device);
  s->gc_valid = false;
  const int R = max_rounds, k = s->k;
  cudaStream_t st = s->st;
  Mem* fp = &s->mem;
  CK(s->stats.alloc(std::max(1, R) * kStats, fp));
  CK(cudaMemsetAsync(s->stats.p, 0, sizeof(int64_t) * std::max(1, R) * kStats, st));
  TmpBuf<int64_t> rb(s->mem);
  CK(rb.alloc(5 * (size_t)k + 1));
  int64_t km1_before = 0;
  ps = read_metrics(s, &km1_before, nullptr);
  if (ps != LPGPU_OK) return ps;
  std::vector<int64_t> hl(k), hb(k), hs(kStats);
  CK(cudaMemcpyAsync(hl.data(), s->lmax.p, sizeof(int64_t) * k, cudaMemcpyDeviceToHost, st));
  const int64_t sub[2] = {0, s->n};
  RoundCtx c = s->ctx();
  c.revert = 0;
  c.rollback = 0;
  s->last_stats.clear();
  int64_t delta = 0, moves = 0, pins = 0;
  {
    // rebalancer.cpp:59-62: on an imbalanced partition the moves of
    // repairEmptyBlocks come first, each applied as moveVertex does
    // (rebalancer.h:84-103: the target stays within L_max, the source keeps
    // weight > 0); they form the first statistics record
    CK(cudaMemcpyAsync(hb.data(), s->bw.p, sizeof(int64_t) * k, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    bool over = false, empty = false;
    for (int b = 0; b < k; ++b) {
      over = over || hb[b] > hl[b];
      empty = empty || hb[b] == 0;
    }
    if (over && empty) {
      std::vector<RepairMove> mv;
      std::vector<int64_t> bwr;
      ps = repair_moves(s, &mv, &bwr);
      if (ps != LPGPU_OK) return ps;
      std::vector<int32_t> av, af, at;
      for (const RepairMove& x : mv) {
        if (bwr[x.to] + x.w <= hl[x.to] && bwr[x.from] - x.w > 0) {
          bwr[x.to] += x.w;
          bwr[x.from] -= x.w;
          av.push_back(x.v);
          af.push_back(x.from);
          at.push_back(x.to);
        }
      }
      int64_t d = 0;
      if (!av.empty()) {
        const size_t cnt = av.size();
        TmpBuf<int32_t> dv(s->mem), df(s->mem), dt(s->mem);
        CK(dv.alloc(cnt));
        CK(df.alloc(cnt));
        CK(dt.alloc(cnt));
        CK(cudaMemcpyAsync(dv.p(), av.data(), sizeof(int32_t) * cnt, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(df.p(), af.data(), sizeof(int32_t) * cnt, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dt.p(), at.data(), sizeof(int32_t) * cnt, cudaMemcpyHostToDevice, st));
        CK(launch_apply_moves(s->launch(), c, (int64_t)cnt, dv.p(), df.p(), dt.p(), GainCache{nullptr, nullptr, nullptr}));
        CK(cudaMemcpyAsync(&d, s->scal.p + kApplyDelta, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
      }
      lpgpu_round_stats rs{s->n, s->P, (int64_t)mv.size(), (int64_t)av.size(), 0, d, 0, 0};
      s->last_stats.push_back(rs);
      delta += d;
      moves += rs.moved;
      pins += rs.pins;
    }
  }
  for (int r = 0; r < R; ++r) {
    CK(cudaMemcpyAsync(hb.data(), s->bw.p, sizeof(int64_t) * k, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    bool over = false;
    for (int b = 0; b < k; ++b) over = over || hb[b] > hl[b];
    if (!over) break;
    // one sub-round over all vertices (rec and status per vertex id)
    CK(cudaMemcpyAsync(s->sub_off.p, sub, sizeof(sub), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(s->blk64.p, 0, sizeof(int64_t) * 3 * k, st));  // in_w, in_cnt, cand_out
    CK(launch_rebalance_round(s->launch(), c, r, s->heavy.p, s->revl.p, rb.p()));
    CK(cudaMemcpyAsync(hs.data(), s->stats.p + (int64_t)r * kStats, sizeof(int64_t) * kStats,
                       cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    lpgpu_round_stats rs{hs[kStActive],   hs[kStPins],  hs[kStCands],     hs[kStMoved],
                         hs[kStReverted], hs[kStDelta], hs[kStMovedPins], hs[kStToggles]};
    s->last_stats.push_back(rs);
    delta += rs.delta;
    moves += rs.moved;
    pins += rs.pins;
    if (rs.moved == 0) break;
  }
  if (result) {
    int64_t km1_after = 0;
    ps = read_metrics(s, &km1_after, nullptr);
    if (ps != LPGPU_OK) return ps;
    double imb = 0;
    ps = read_imbalance(s, &imb);
    if (ps != LPGPU_OK) return ps;
    result->km1_before = km1_before;
    result->km1_after = km1_after;
    result->delta = delta;
    result->moves = moves;
    result->pins_processed = pins;
    result->rounds = (int32_t)s->last_stats.size();
    result->improved = delta < 0;
    result->imbalance = imb;
  }
  return LPGPU_OK;
}

int64_t lpgpu_kernel_launches(void) { return kernel_launches(); }

void* lpgpu_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

void lpgpu_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

lpgpu_status lpgpu_session_event_record(lpgpu_session* s, int32_t slot) {
  if (!s || slot < 0 || slot >= 16) return invalid("bad session or event slot");
  DeviceGuard g(s->device);
  if (!s->slots[slot]) CK(cudaEventCreate(&s->slots[slot]));
  CK(cudaEventRecord(s->slots[slot], s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_event_elapsed(lpgpu_session* s, int32_t a, int32_t b, double* ms) {
  if (!s || a < 0 || a >= 16 || b < 0 || b >= 16 || !ms) return invalid("bad event slots");
  if (!s->slots[a] || !s->slots[b]) {
    set_error("event slot never recorded");
    return LPGPU_ERR_STATE;
  }
  DeviceGuard g(s->device);
  CK(cudaEventSynchronize(s->slots[b]));
  float f = 0.f;
  CK(cudaEventElapsedTime(&f, s->slots[a], s->slots[b]));
  *ms = f;
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_synchronize(lpgpu_session* s) {
  if (!s) return invalid("null session");
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_enable_timing(lpgpu_session* s, int32_t enable) {
  if (!s) return invalid("null session");
  s->timing = enable != 0;
  return LPGPU_OK;
}

lpgpu_status lpgpu_session_phase_times(lpgpu_session* s, lpgpu_phase_time* out, int32_t max,
                                       int32_t* count) {
  if (!s) return invalid("null session");
  const int cnt = (int)std::min<size_t>(s->phase_times.size(), (size_t)std::max(0, max));
  for (int i = 0; i < cnt; ++i) out[i] = s->phase_times[i];
  if (count) *count = (int32_t)s->phase_times.size();
  return LPGPU_OK;
}

lpgpu_status lpgpu_refine_km1(int64_t n, int64_t m, const int64_t* net_off, const int32_t* pins,
                              const int32_t* w_v, const int32_t* w_e, int32_t k, double eps,
                              int32_t* part, const lpgpu_config* cfg, lpgpu_result* result) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = 0;
  }
  lpgpu_session* s = nullptr;
  lpgpu_status st = lpgpu_session_create(dev, &s);
  if (st != LPGPU_OK) return st;
  if ((st = lpgpu_session_upload(s, n, m, net_off, pins, w_v, w_e)) == LPGPU_OK &&
      (st = lpgpu_session_set_partition(s, k, eps, part, nullptr, nullptr)) == LPGPU_OK &&
      (st = lpgpu_session_refine(s, cfg, nullptr, 0, result)) == LPGPU_OK)
    st = lpgpu_session_get_partition(s, part);
  lpgpu_session_destroy(s);
  return st;
}

}  // extern "C"
