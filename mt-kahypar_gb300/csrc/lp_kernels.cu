// Device kernels of the label-propagation (km1) refinement path, sm_103a.
//
// All work is integer and memory bound; no tensor cores are involved. Kernels
// use grid-stride loops over persistent grids sized to the SM count, read their
// element counts from device memory (so a whole refine needs no host sync),
// and privatize per-block accumulators in shared memory.
#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"

namespace lpgpu {

#define FULLMASK 0xffffffffu


__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
  return v;
}

// Block-wide sum of an int64 (any blockDim multiple of 32, <= 1024). All threads get the total.
__device__ int64_t block_sum_i64(int64_t v) {
  __shared__ int64_t ws[32];
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane_id() == 0) ws[w] = v;
  __syncthreads();
  int64_t t = lane_id() < nw ? ws[lane_id()] : 0;
  t = warp_sum(t);
  return t;
}

// Block-wide exclusive scan of an int64 (blockDim multiple of 32, <= 1024).
__device__ int64_t block_scan_excl_i64(int64_t v, int64_t* total) {
  __shared__ int64_t ws[32];
  const int lane = lane_id(), w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(FULLMASK, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    int64_t s = lane < nw ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(FULLMASK, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) ws[lane] = s;
  }
  __syncthreads();
  const int64_t prefix = w > 0 ? ws[w - 1] : 0;
  *total = ws[nw - 1];
  return prefix + x - v;
}

static int blocks_per_sm_hint = 4;

static int grid_for(const Launch& L, int64_t work_items, int threads, int per_sm = 0) {
  const int64_t cap = (int64_t)L.num_sms * (per_sm > 0 ? per_sm : blocks_per_sm_hint);
  const int64_t need = (work_items + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(cap, need));
}

// Raises a kernel's dynamic shared memory limit on the current device to at
// least `bytes`. The limit belongs to the kernel, not to the launch, and
// sessions driven from several host threads launch the same kernel with
// different sizes: it only ever grows, under a lock, so that no thread lowers
// it below the size another thread is about to launch with.
template <typename Kernel>
static void allow_dyn_smem(Kernel kern_fn, size_t bytes) {
  const void* kern = (const void*)kern_fn;
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> limits;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = limits[{dev, kern}];
  if (bytes > cur && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess)
    cur = bytes;
}

// Resident CTAs per SM of `kern` (at least 1).
static int occupancy(const void* kern, int threads, size_t smem) {
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, threads, smem) != cudaSuccess ||
      blocks < 1)
    blocks = 1;
  return blocks;
}

// Reports the kernel that failed to launch (and a sticky error left by an
// earlier call) through the library's error text.
static thread_local int64_t t_launches = 0;
int64_t kernel_launches() { return t_launches; }
void add_kernel_launches(int64_t n) { t_launches += n; }

static cudaError_t launched(const char* name) {
  ++t_launches;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) set_error(std::string(name) + ": " + cudaGetErrorString(e));
  return e;
}
#define LAUNCHED(name)                          \
  do {                                          \
    const cudaError_t _e = launched(name);      \
    if (_e != cudaSuccess) return _e;           \
  } while (0)

// =================================================================== scan

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int64_t kScanTile = kScanThreads * kScanItems;

__global__ void k_tile_sums(const int64_t* __restrict__ in, int64_t count, int64_t* __restrict__ sums) {
  const int64_t base = blockIdx.x * kScanTile;
  int64_t s = 0;
  for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
    const int64_t g = base + i;
    if (g < count) s += in[g];
  }
  s = block_sum_i64(s);
  if (threadIdx.x == 0) sums[blockIdx.x] = s;
}

__global__ void k_scan_tiles(const int64_t* in, int64_t* out, int64_t count,
                             const int64_t* __restrict__ tile_prefix) {
  const int64_t base = blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    v[j] = (base + j < count) ? in[base + j] : 0;
    s += v[j];
  }
  int64_t total;
  int64_t run = block_scan_excl_i64(s, &total) + (tile_prefix ? tile_prefix[blockIdx.x] : 0);
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    if (base + j < count) out[base + j] = run;
    run += v[j];
  }
}

int64_t scan_tmp_elems(int64_t count) {
  const int64_t tiles = (count + kScanTile - 1) / kScanTile;
  if (tiles <= 1) return 0;
  return tiles + scan_tmp_elems(tiles);
}

cudaError_t scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t count, int64_t* tmp,
                               int64_t tmp_elems, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  const int64_t tiles = (count + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    k_scan_tiles<<<1, kScanThreads, 0, st>>>(in, out, count, nullptr);
    LAUNCHED("k_scan_tiles");
    return cudaGetLastError();
  }
  if (tmp_elems < scan_tmp_elems(count)) return cudaErrorInvalidValue;
  int64_t* sums = tmp;
  k_tile_sums<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, count, sums);
  LAUNCHED("k_tile_sums");
  cudaError_t e = scan_exclusive_i64(sums, sums, tiles, tmp + tiles, tmp_elems - tiles, st);
  if (e != cudaSuccess) return e;
  k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, count, sums);
  LAUNCHED("k_scan_tiles");
  return cudaGetLastError();
}

// Incidence packing shared by the kernels that walk the incidences of a set
// of vertices (one per lane). Vertices of degree 1..32 are packed greedily
// into groups of <= 32 incidences (lane = incidence, contiguous per vertex);
// longer vertices are walked alone in 32-incidence chunks. For every group
// `body(has, ow, j, seg_end)` runs on all lanes: lane `has` holds incidence j
// (index into inets) of the vertex held by lane `ow`. The return value is, on
// each selected lane, the sum over its vertex's incidences of the ints
// returned by body (segmented sums inside a group).
template <typename Body>
__device__ __forceinline__ int packed_incidences(bool sel, int64_t o0, int deg,
                                                 unsigned char* __restrict__ s_owner, Body&& body) {
  const int lane = lane_id();
  int my_total = 0;
  const bool small = sel && deg >= 1 && deg <= 32;
  const int dsm = small ? deg : 0;
  int incl = dsm;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(FULLMASK, incl, o);
    if (lane >= o) incl += y;
  }
  const int excl = incl - dsm;
  unsigned rem = __ballot_sync(FULLMASK, small);
  while (rem) {
    const int q = __ffs(rem) - 1;
    const int start = __shfl_sync(FULLMASK, excl, q);
    const bool inpack = ((rem >> lane) & 1u) && incl - start <= 32;
    const unsigned pmask = __ballot_sync(FULLMASK, inpack);
    const int D = __shfl_sync(FULLMASK, incl, 31 - __clz(pmask)) - start;
    const int st = excl - start;
    __syncwarp();
    if (inpack) s_owner[__popc(pmask & lanemask_lt())] = (unsigned char)lane;
    const unsigned starts = __reduce_or_sync(FULLMASK, inpack ? (1u << st) : 0u);
    __syncwarp();
    const bool has = lane < D;
    const int ow = has ? s_owner[__popc(starts & ((2u << lane) - 1u)) - 1] : lane;
    const int64_t o_ow = __shfl_sync(FULLMASK, o0, ow);
    const int st_ow = __shfl_sync(FULLMASK, st, ow);
    const int d_ow = __shfl_sync(FULLMASK, deg, ow);
    const int seg_end = has ? st_ow + d_ow : lane + 1;
    int x = body(has, ow, has ? o_ow + lane - st_ow : (int64_t)0);
    // segmented suffix sums: the first lane of every vertex gets its total
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_down_sync(FULLMASK, x, o);
      if (lane + o < seg_end) x += y;
    }
    const int tot = __shfl_sync(FULLMASK, x, inpack ? st : 0);
    if (inpack) my_total = tot;
    rem &= ~pmask;
  }
  unsigned bigm = __ballot_sync(FULLMASK, sel && deg > 32);
  while (bigm) {
    const int j = __ffs(bigm) - 1;
    bigm &= bigm - 1;
    const int64_t oj = __shfl_sync(FULLMASK, o0, j);
    const int dj = __shfl_sync(FULLMASK, deg, j);
    int acc = 0;
    for (int base = 0; base < dj; base += 32) {
      const bool has = base + lane < dj;
      acc += body(has, j, has ? oj + base + lane : (int64_t)0);
    }
    acc = warp_sum(acc);
    if (lane == j) my_total = acc;
  }
  return my_total;
}

// ============================================================ incidence

// Degrees by one atomic per pin; the count returned is the pin's rank among its
// vertex's incidences, i.e. its slot in the vertex's incident-net list.
__global__ void k_count_pins(const int32_t* __restrict__ pins, int64_t P, int64_t* __restrict__ cnt,
                             int32_t* __restrict__ rank) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P;
       i += (int64_t)gridDim.x * blockDim.x)
    rank[i] = (int32_t)atomicAdd(reinterpret_cast<ull*>(&cnt[pins[i]]), 1ull);
}

// Incidences per log2 degree bucket (bucket j: degree in [2^j, 2^(j+1))),
// from the per-vertex counts before the scan; sizes the sweep's heavy share.
__global__ void k_degree_hist(int64_t n, const int64_t* __restrict__ cnt, int64_t* __restrict__ hist) {
  __shared__ ull s_h[kDegBuckets];
  if (threadIdx.x < kDegBuckets) s_h[threadIdx.x] = 0;
  __syncthreads();
  // most vertices share a few buckets: lanes of one bucket add once
  const int lane = lane_id();
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = base + lane;
    const int64_t d = v < n ? cnt[v] : 0;  // 16-bit halves: exact below 2^43 incidences per vertex
    const int j = d > 0 ? min(63 - __clzll(d), kDegBuckets - 1) : -1;
    const unsigned peers = __match_any_sync(FULLMASK, j);
    const unsigned lo = __reduce_add_sync(peers, (unsigned)d & 0xFFFFu);
    const unsigned hi = __reduce_add_sync(peers, (unsigned)(d >> 16));
    if (j >= 0 && __ffs(peers) - 1 == lane) atomicAdd(&s_h[j], (ull)lo + ((ull)hi << 16));
  }
  __syncthreads();
  if (threadIdx.x < kDegBuckets && s_h[threadIdx.x])
    atomicAdd(reinterpret_cast<ull*>(&hist[threadIdx.x]), s_h[threadIdx.x]);
}

// Every pin writes its net id into its slot of its vertex's incident-net list
// (list start + the rank k_count_pins returned). A warp takes the next 32 nets
// from a counter and walks their pins in packed 32-pin groups (nets of more
// than 32 pins alone, 32 pins at a time), so small nets keep every lane busy.
// Taking nets in order keeps the nets in flight close together, so where a
// hypergraph's pins are local, the partly written 32-byte sectors of their
// vertices' lists stay in L2 until they are complete (a grid-stride loop lets
// warps drift apart over nets of uneven size).
__global__ void __launch_bounds__(256) k_scatter_incidence(int64_t m, const int64_t* __restrict__ net_off,
                                                           const int32_t* __restrict__ pins,
                                                           const int64_t* __restrict__ vtx_off,
                                                           const int32_t* __restrict__ rank,
                                                           int32_t* __restrict__ inets, ull* next_net) {
  __shared__ unsigned char s_own[256];
  const int lane = lane_id();
  unsigned char* own = s_own + (threadIdx.x & ~31);
  for (;;) {
    ull b = 0;
    if (lane == 0) b = atomicAdd(next_net, 32ull);
    const int64_t base = (int64_t)__shfl_sync(FULLMASK, b, 0);
    if (base >= m) break;
    const int64_t e = base + lane;
    const bool sel = e < m;
    const int64_t o0 = sel ? net_off[e] : 0;
    const int deg = sel ? (int)(net_off[e + 1] - o0) : 0;
    packed_incidences(sel, o0, deg, own, [&](bool has, int ow, int64_t j) -> int {
      if (has) inets[vtx_off[pins[j]] + rank[j]] = (int32_t)(base + ow);
      return 0;
    });
  }
}

cudaError_t launch_build_incidence(const Launch& L, int64_t n, int64_t m, int64_t P, const int64_t* net_off,
                                   const int32_t* pins, int64_t* vtx_off, int32_t* inets,
                                   int32_t* rank, int64_t* scan_tmp, int64_t scan_tmp_elems,
                                   int64_t* deg_hist) {
  cudaError_t e = cudaMemsetAsync(vtx_off, 0, sizeof(int64_t) * (n + 1), L.st);
  if (e != cudaSuccess) return e;
  if (P > 0) {
    k_count_pins<<<grid_for(L, P, 256, 8), 256, 0, L.st>>>(pins, P, vtx_off, rank);
    LAUNCHED("k_count_pins");
  }
  if (deg_hist) {
    if ((e = cudaMemsetAsync(deg_hist, 0, sizeof(int64_t) * kDegBuckets, L.st)) != cudaSuccess) return e;
    if (n > 0) {
      k_degree_hist<<<grid_for(L, n, 256, 4), 256, 0, L.st>>>(n, vtx_off, deg_hist);
      LAUNCHED("k_degree_hist");
    }
  }
  if ((e = scan_exclusive_i64(vtx_off, vtx_off, n + 1, scan_tmp, scan_tmp_elems, L.st)) != cudaSuccess)
    return e;
  if (m > 0) {
    ull* next_net = reinterpret_cast<ull*>(scan_tmp);  // free again after the scan
    if ((e = cudaMemsetAsync(next_net, 0, sizeof(ull), L.st)) != cudaSuccess) return e;
    k_scatter_incidence<<<grid_for(L, m, 256, 8), 256, 0, L.st>>>(m, net_off, pins, vtx_off, rank, inets, next_net);
    LAUNCHED("k_scatter_incidence");
  }
  return cudaGetLastError();
}

// ======================================================== partition init

// c(V_b) = sum of w(v) over v in block b (initializeBlockWeights, h:1067-1084).
// Batched sessions have too many blocks for shared memory: global atomics.
__global__ void k_block_weights(RoundCtx c) {
  extern __shared__ ull s_w[];
  const bool priv = !c.batched;
  if (priv) {
    for (int b = threadIdx.x; b < c.k; b += blockDim.x) s_w[b] = 0;
    __syncthreads();
  }
  // lanes of a warp whose vertices share a block (contiguous partitions) add once
  const int lane = lane_id();
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; base < c.n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = base + lane;
    const bool has = v < c.n;
    const int b = has ? c.part[v] : -1;
    const unsigned wv = has ? (unsigned)c.w_v[v] : 0u;  // vertex weights are >= 0
    const unsigned peers = __match_any_sync(FULLMASK, b);
    // sum over the lanes of the same block, in 16-bit halves (no 32-bit overflow)
    const unsigned lo = __reduce_add_sync(peers, wv & 0xFFFFu);
    const unsigned hi = __reduce_add_sync(peers, wv >> 16);
    const ull w = (ull)lo + ((ull)hi << 16);
    if (has && __ffs(peers) - 1 == lane) {
      if (priv)
        atomicAdd(&s_w[b], w);
      else
        atomicAdd(reinterpret_cast<ull*>(&c.bw[b]), w);
    }
  }
  if (priv) {
    __syncthreads();
    for (int b = threadIdx.x; b < c.k; b += blockDim.x)
      if (s_w[b]) atomicAdd(reinterpret_cast<ull*>(&c.bw[b]), s_w[b]);
  }
}


// Φ, Λ and Λ1 (blocks holding exactly one pin of the net) from scratch
// (initializePinCountInPart, h:1086-1110), fused with the km1 / cut sums. A
// warp takes 32 nets and zeroes their Φ rows and records before filling them. Nets of up to 32 pins are packed
// into 32-pin groups (lane = pin): lanes with the same (net, block) find each
// other with a match, and the lowest writes Φ(e, b) and sets the Λ / Λ1 bits;
// λ(e) is the number of such lanes. Larger nets are counted one at a time in a
// per-warp shared k-bin histogram. Net e's record is conn[e * 2W .. e * 2W + 2W):
// W words of Λ(e), then W words of Λ1(e).
__global__ void __launch_bounds__(256) k_pin_counts(RoundCtx c) {
  extern __shared__ int s_hist[];
  __shared__ unsigned char s_own[256];
  const int k = c.kmax, W = c.W;
  int* hist = s_hist + (threadIdx.x >> 5) * k;
  unsigned char* own = s_own + (threadIdx.x & ~31);
  const int lane = lane_id();
  for (int b = lane; b < k; b += 32) hist[b] = 0;
  __syncwarp();
  int64_t km1 = 0, cut = 0;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; base < c.m;
       base += (int64_t)gridDim.x * blockDim.x) {
    // The warp first zeroes the Φ rows and Λ records of its 32 nets (one
    // contiguous range each), so every sector it then changes is complete in
    // L2 and no partly written sector is read back from DRAM.
    {
      const int64_t e_end = base + 32 < c.m ? base + 32 : c.m;
      const int esz = c.phi16 ? 2 : 4;
      unsigned char* p0 = reinterpret_cast<unsigned char*>(c.phi) + base * k * esz;
      const int64_t bytes = ((e_end - base) * k * esz + 3) & ~(int64_t)3;  // Φ is allocated in whole words
      const int64_t n16 = bytes >> 4;
      for (int64_t i = lane; i < n16; i += 32) reinterpret_cast<uint4*>(p0)[i] = make_uint4(0, 0, 0, 0);
      for (int64_t i = (n16 << 2) + lane; i < (bytes >> 2); i += 32) reinterpret_cast<uint32_t*>(p0)[i] = 0;
      for (int64_t i = base * 2 * W + lane; i < e_end * 2 * W; i += 32) c.conn[i] = 0;
      __syncwarp();
    }
    const int64_t e = base + lane;
    int64_t b0 = 0;
    int deg = 0, bo = 0;
    if (e < c.m) {
      b0 = c.net_off[e];
      const int64_t d = c.net_off[e + 1] - b0;
      deg = d > INT32_MAX ? INT32_MAX : (int)d;
      if (c.batched && d > 0) bo = block_offset(c, c.pins[b0]);
    }
    const bool small = deg >= 1 && deg <= 32;
    const int lam = packed_incidences(small, b0, deg, own, [&](bool has, int ow, int64_t j) -> int {
      const int64_t e_ow = __shfl_sync(FULLMASK, e, ow);
      const int bo_ow = __shfl_sync(FULLMASK, bo, ow);
      int b = 0;
      unsigned key = 0x80000000u | (unsigned)lane;  // lanes without a pin match nobody
      if (has) {
        b = c.part[c.pins[j]] - bo_ow;
        key = ((unsigned)ow << 11) | (unsigned)b;
      }
      const unsigned peers = __match_any_sync(FULLMASK, key);
      const bool leader = has && __ffs(peers) - 1 == lane;
      if (leader) {
        const int cnt = __popc(peers);
        phi_set(c, e_ow * k + b, cnt);
        uint32_t* rec = c.conn + e_ow * 2 * W;
        atomicOr(&rec[b >> 5], 1u << (b & 31));
        if (cnt == 1) atomicOr(&rec[W + (b >> 5)], 1u << (b & 31));
      }
      return leader ? 1 : 0;
    });
    if (small) {
      const int64_t we = c.w_e[e];
      km1 += (int64_t)(lam > 1 ? lam - 1 : 0) * we;
      cut += lam > 1 ? we : 0;
    }
    unsigned bigm = __ballot_sync(FULLMASK, deg > 32);
    while (bigm) {
      const int q = __ffs(bigm) - 1;
      bigm &= bigm - 1;
      const int64_t eq = __shfl_sync(FULLMASK, e, q);
      const int64_t bq = __shfl_sync(FULLMASK, b0, q);
      const int dq = __shfl_sync(FULLMASK, deg, q);
      const int boq = __shfl_sync(FULLMASK, bo, q);
      for (int64_t i = bq + lane; i < bq + dq; i += 32) atomicAdd(&hist[c.part[c.pins[i]] - boq], 1);
      __syncwarp();
      int lq = 0;
      for (int w = 0; w < W; ++w) {
        const int b = w * 32 + lane;
        int cnt = 0;
        if (b < k) {
          cnt = hist[b];
          hist[b] = 0;
          if (cnt) phi_set(c, eq * k + b, cnt);
        }
        const unsigned bits = __ballot_sync(FULLMASK, cnt > 0);
        const unsigned ones = __ballot_sync(FULLMASK, cnt == 1);
        if (lane == 0) {
          c.conn[eq * 2 * W + w] = bits;
          c.conn[eq * 2 * W + W + w] = ones;
        }
        lq += __popc(bits);
      }
      __syncwarp();
      if (lane == 0) {
        const int64_t we = c.w_e[eq];
        km1 += (int64_t)(lq > 1 ? lq - 1 : 0) * we;
        cut += lq > 1 ? we : 0;
      }
    }
  }
  km1 = block_sum_i64(km1);
  cut = block_sum_i64(cut);
  if (threadIdx.x == 0) {
    atomicAdd(reinterpret_cast<ull*>(&c.scal[kKm1]), (ull)km1);
    atomicAdd(reinterpret_cast<ull*>(&c.scal[kCut]), (ull)cut);
  }
}

cudaError_t launch_init_partition(const Launch& L, const RoundCtx& c) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(c.bw, 0, sizeof(int64_t) * c.k, L.st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(c.scal + kKm1, 0, sizeof(int64_t) * 2, L.st)) != cudaSuccess) return e;
  if (c.n > 0) {
    k_block_weights<<<grid_for(L, c.n, 256), 256, c.batched ? 0 : sizeof(ull) * c.k, L.st>>>(c);
    LAUNCHED("k_block_weights");
  }
  if (c.m > 0) {
    // k_pin_counts writes all of Φ and the Λ records, zeros included
    const size_t smem = sizeof(int) * c.kmax * 8;
    k_pin_counts<<<grid_for(L, c.m, 256, occupancy((const void*)k_pin_counts, 256, smem)), 256, smem, L.st>>>(c);
    LAUNCHED("k_pin_counts");
  }
  return cudaSuccess;
}

// metrics::km1 / hyperedgeCut (metrics.cpp:29-65): thread per net.
__global__ void k_metrics(RoundCtx c) {
  int64_t km1 = 0, cut = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < c.m;
       e += (int64_t)gridDim.x * blockDim.x) {
    int lam = 0;
    for (int w = 0; w < c.W; ++w) lam += __popc(c.conn[e * 2 * c.W + w]);
    const int64_t we = c.w_e[e];
    km1 += (int64_t)(lam > 1 ? lam - 1 : 0) * we;
    cut += lam > 1 ? we : 0;
  }
  km1 = block_sum_i64(km1);
  cut = block_sum_i64(cut);
  if (threadIdx.x == 0) {
    atomicAdd(reinterpret_cast<ull*>(&c.scal[kKm1]), (ull)km1);
    atomicAdd(reinterpret_cast<ull*>(&c.scal[kCut]), (ull)cut);
  }
}

// km1 of every instance of a batched session (net instance = instance of its first pin).
__global__ void k_instance_metrics(RoundCtx c, int64_t* km1_inst) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < c.m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = c.net_off[e];
    if (b0 == c.net_off[e + 1]) continue;
    int lam = 0;
    for (int w = 0; w < c.W; ++w) lam += __popc(c.conn[e * 2 * c.W + w]);
    if (lam > 1)
      atomicAdd(reinterpret_cast<ull*>(&km1_inst[c.vinst[c.pins[b0]]]), (ull)((int64_t)(lam - 1) * c.w_e[e]));
  }
}

cudaError_t launch_instance_metrics(const Launch& L, const RoundCtx& c, int64_t* km1_inst) {
  cudaError_t e = cudaMemsetAsync(km1_inst, 0, sizeof(int64_t) * c.num_inst, L.st);
  if (e != cudaSuccess) return e;
  if (c.m > 0) {
    k_instance_metrics<<<grid_for(L, c.m, 256), 256, 0, L.st>>>(c, km1_inst);
    LAUNCHED("k_instance_metrics");
  }
  return cudaSuccess;
}

cudaError_t launch_metrics(const Launch& L, const RoundCtx& c) {
  cudaError_t e = cudaMemsetAsync(c.scal + kKm1, 0, sizeof(int64_t) * 2, L.st);
  if (e != cudaSuccess) return e;
  if (c.m > 0) {
    k_metrics<<<grid_for(L, c.m, 256), 256, 0, L.st>>>(c);
    LAUNCHED("k_metrics");
  }
  return cudaGetLastError();
}

// ====================================================== sweep / best move

// 32 x 32 bit transpose across a warp (recursive block swap with shuffles):
// on return lane j holds the word whose bit i is bit j of lane i's input.
__device__ __forceinline__ uint32_t transpose32(uint32_t x) {
  const int lane = lane_id();
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const uint32_t m = s == 16 ? 0x0000FFFFu : s == 8 ? 0x00FF00FFu : s == 4 ? 0x0F0F0F0Fu
                     : s == 2 ? 0x33333333u : 0x55555555u;
    const uint32_t y = __shfl_xor_sync(FULLMASK, x, s);
    x = (lane & s) ? ((x & ~m) | ((y >> s) & m)) : ((x & m) | ((y << s) & ~m));
  }
  return x;
}

// W words of a Λ record. NC: through the read-only data path (records that
// no thread of the running kernel changes); otherwise plain coherent loads.
template <int W, bool NC = true>
__device__ __forceinline__ void load_words(const uint32_t* __restrict__ p, uint32_t (&w)[W]) {
  if constexpr (W % 4 == 0) {
#pragma unroll
    for (int i = 0; i < W / 4; ++i) {
      const uint4 q = NC ? __ldg(reinterpret_cast<const uint4*>(p) + i) : reinterpret_cast<const uint4*>(p)[i];
      w[4 * i] = q.x; w[4 * i + 1] = q.y; w[4 * i + 2] = q.z; w[4 * i + 3] = q.w;
    }
  } else if constexpr (W == 2) {
    const uint2 q = NC ? __ldg(reinterpret_cast<const uint2*>(p)) : *reinterpret_cast<const uint2*>(p);
    w[0] = q.x; w[1] = q.y;
  } else {
#pragma unroll
    for (int i = 0; i < W; ++i) w[i] = NC ? __ldg(p + i) : p[i];
  }
}

// Weighted sum over the lanes in `mask` from weight bit-planes:
// sum_p popc(bits[p] & mask) << p (planes beyond kPlanes recomputed by the caller).
constexpr int kPlanes = 4;

struct Planes {
  uint32_t b[kPlanes];
  int n;  // number of planes in use (<= 31)
};

// Bit-planes of a per-lane non-negative weight `w` (all lanes participate).
__device__ __forceinline__ Planes make_planes(int w, int nplanes) {
  Planes p;
  p.n = nplanes;
#pragma unroll
  for (int i = 0; i < kPlanes; ++i) p.b[i] = i < nplanes ? __ballot_sync(FULLMASK, (w >> i) & 1) : 0u;
  return p;
}

// sum over lanes in mask of w; warp-uniform call (extra planes via ballot).
__device__ __forceinline__ int plane_sum(const Planes& p, uint32_t mask, int w) {
  int s = 0;
#pragma unroll
  for (int i = 0; i < kPlanes; ++i) s += __popc(p.b[i] & mask) << i;
  for (int i = kPlanes; i < p.n; ++i) s += __popc(__ballot_sync(FULLMASK, (w >> i) & 1) & mask) << i;
  return s;
}

// Decision of Km1Policy::computeMaxGainMoveImpl (gain_policy.h:147-166,
// disable_randomization) from penalties held by block-owning lanes: lane l
// owns blocks l + 32 t and pen[t] = sum of w(e) over incident nets with that
// block in Λ(e). score(b) = internal - pen(b); the move goes to the feasible
// block (slack(b) >= w(v), b != from) of minimum score < 0, lowest id on ties.
// Without one, and with zero_gain, the lowest feasible block of score 0 is
// taken if the rebalancing rule of label_propagation_refiner.h:88-95 holds.
template <int W, bool PACKED>
__device__ __forceinline__ void decide(int k, int from, int wv, int internal, int zero_gain,
                                       const int (&pen)[W], const int (&slack)[W],
                                       const int64_t* __restrict__ s_bw,
                                       const int64_t* __restrict__ s_perf, int& to, int& gain) {
  const int lane = lane_id();
  // quick reject: neither an improving move (pen > internal) nor a zero-gain
  // candidate (pen == internal) exists when every other block's penalty is
  // below the internal weight
  int any = -1;
#pragma unroll
  for (int t = 0; t < W; ++t) {
    const int blk = 32 * t + lane;
    if (blk != from && pen[t] > any) any = pen[t];
  }
  if (__reduce_max_sync(FULLMASK, any) < internal) return;
  int zb = INT_MAX;
  if constexpr (PACKED) {
    // penalties below 2^20: one max over (pen << 11 | 2047 - blk) gives the
    // largest penalty and, on ties, the lowest block; 0 = no feasible block
    unsigned key = 0;
#pragma unroll
    for (int t = 0; t < W; ++t) {
      const int blk = 32 * t + lane;
      if (blk < k && blk != from && slack[t] >= wv) {
        const unsigned kk = ((unsigned)pen[t] << 11) | (unsigned)(2047 - blk);
        key = kk > key ? kk : key;
        if (zb == INT_MAX && pen[t] == internal) zb = blk;
      }
    }
    const unsigned mk = __reduce_max_sync(FULLMASK, key);
    if (mk != 0 && (int)(mk >> 11) > internal) {
      to = 2047 - (int)(mk & 2047u);
      gain = internal - (int)(mk >> 11);
      return;
    }
  } else {
    int bp = -1, bb = INT_MAX;
#pragma unroll
    for (int t = 0; t < W; ++t) {
      const int blk = 32 * t + lane;
      if (blk < k && blk != from && slack[t] >= wv) {
        if (pen[t] > bp) { bp = pen[t]; bb = blk; }
        if (zb == INT_MAX && pen[t] == internal) zb = blk;
      }
    }
    const int mp = __reduce_max_sync(FULLMASK, bp);
    if (mp > internal) {
      to = __reduce_min_sync(FULLMASK, bp == mp ? bb : INT_MAX);
      gain = internal - mp;
      return;
    }
  }
  if (zero_gain) {
    const int z = __reduce_min_sync(FULLMASK, zb);
    if (z != INT_MAX && s_bw[from] - 1 > s_bw[z] + 1 && s_bw[z] < s_perf[z]) {
      to = z;
      gain = 0;
    }
  }
}

constexpr int kSweepThreads = 256;

__device__ bool last_cta(int64_t* counter);
__device__ void plan_to(const RoundCtx& c);

// ---- lane-per-vertex sweep (k <= 128)
//
// A lane evaluates its own vertex: it walks the vertex's incident nets and adds
// each net's Λ(e) bit vector (times w(e)) into bit-sliced counters, one
// 32-block word t and plane p per register cnt[t][p], so that bit l of plane p
// is bit p of the penalty of block 32 t + l. The best target then comes from a
// bit-sliced maximum over the feasible blocks. Vertices whose summed incident
// net weight stays below 2^PL take this path; the others take the
// warp-cooperative windows below.
constexpr int kLvWeights = 16;  // vertex weights 1..16 have precomputed feasibility masks
// Incidences per lane whose gathers are issued together (a multiple of 4), and
// resident CTAs per SM the k <= 128 sweep is compiled for.
#ifndef LPGPU_LV_UNROLL
#define LPGPU_LV_UNROLL 4
#endif
#ifndef LPGPU_SWEEP_MIN_BLOCKS
#define LPGPU_SWEEP_MIN_BLOCKS 3
#endif
static_assert(LPGPU_LV_UNROLL % 4 == 0, "the carry-save adder takes four vectors at a time");

// cnt += s0 + 2 s1 + 4 s2 (bit-sliced, ripple carry).
template <int PL>
__device__ __forceinline__ void lv_add3(uint32_t (&cnt)[PL], uint32_t s0, uint32_t s1, uint32_t s2) {
  uint32_t cy = cnt[0] & s0;
  cnt[0] ^= s0;
  uint32_t t = cnt[1];
  cnt[1] = t ^ s1 ^ cy;
  cy = (t & s1) | (cy & (t ^ s1));
  t = cnt[2];
  cnt[2] = t ^ s2 ^ cy;
  cy = (t & s2) | (cy & (t ^ s2));
#pragma unroll
  for (int p = 3; p < PL; ++p) {
    const uint32_t c2 = cnt[p] & cy;
    cnt[p] ^= cy;
    cy = c2;
  }
}

// cnt += w * x (bit-sliced; w < 2^PL).
template <int PL>
__device__ __forceinline__ void lv_add_weighted(uint32_t (&cnt)[PL], uint32_t x, int w) {
  uint32_t cy = 0;
#pragma unroll
  for (int p = 0; p < PL; ++p) {
    const uint32_t a = ((w >> p) & 1) ? x : 0u;
    const uint32_t t = cnt[p];
    cnt[p] = t ^ a ^ cy;
    cy = (t & a) | (cy & (t ^ a));
  }
}

// One step of a lane's vertex: the next U incidences (from index j) of the
// vertex with incidences [o0, o0 + d) and source block `from` (local) are
// added into the bit-sliced counters and the internal weight.
template <int W, bool UNIT, int PL, int U, bool NC = true>
__device__ __forceinline__ void lv_accumulate(const RoundCtx& c, int64_t o0, int d, int j, int from,
                                              uint32_t (&cnt)[W][PL], int& internal) {
  constexpr int W2 = 2 * W;
  const int fw = from >> 5;
  const uint32_t fbit = 1u << (from & 31);
  int32_t ee[U];
#pragma unroll
  for (int u = 0; u < U; ++u) ee[u] = j + u < d ? __ldg(&c.inets[o0 + j + u]) : -1;
  uint32_t wd[U][W], l1[U];
  int we[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
#pragma unroll
    for (int t = 0; t < W; ++t) wd[u][t] = 0;
    l1[u] = fbit;
    we[u] = 0;
    if (ee[u] >= 0) {
      const uint32_t* rec = c.conn + (int64_t)ee[u] * W2;
      load_words<W, NC>(rec, wd[u]);
      l1[u] = NC ? __ldg(rec + W + fw) : rec[W + fw];
      we[u] = UNIT ? 1 : __ldg(&c.w_e[ee[u]]);
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) internal += (l1[u] & fbit) ? 0 : we[u];
  if constexpr (UNIT) {
    // carry-save sum of each four vectors, then one 3-bit ripple add
#pragma unroll
    for (int g = 0; g < U; g += 4)
#pragma unroll
      for (int t = 0; t < W; ++t) {
        const uint32_t a = wd[g][t], b = wd[g + 1][t], e = wd[g + 2][t], f = wd[g + 3][t];
        const uint32_t s = a ^ b ^ e;
        const uint32_t c1 = (a & b) | (e & (a ^ b));
        const uint32_t c2 = s & f;
        lv_add3<PL>(cnt[t], s ^ f, c1 ^ c2, c1 & c2);
      }
  } else {
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int t = 0; t < W; ++t) lv_add_weighted<PL>(cnt[t], wd[u][t], we[u]);
  }
}

// Best move of one vertex from its counters: the same decision as `decide`
// (Km1Policy::computeMaxGainMoveImpl with disable_randomization, plus the
// zero-gain rebalancing rule of label_propagation_refiner.h:88-95). `from`,
// `to` are local block ids; `bo` is the instance's first global block.
template <int W, int PL>
__device__ __forceinline__ void lv_decide(const RoundCtx& c, const uint32_t (&cnt)[W][PL], int internal, int from,
                                          int wv, int bo, int inst, bool batched, int zero_gain,
                                          const uint32_t* __restrict__ s_fmask, const int* __restrict__ s_slack,
                                          const int64_t* __restrict__ s_bw, const int64_t* __restrict__ s_perf,
                                          int& to, int& gain, bool& border) {
  const int fw = from >> 5;
  const uint32_t fbit = 1u << (from & 31);
  // feasible targets: c(V_b) + w(v) <= L_max(b)
  uint32_t cand[W];
  if (!batched && wv >= 1 && wv <= kLvWeights) {
#pragma unroll
    for (int t = 0; t < W; ++t) cand[t] = s_fmask[(wv - 1) * W + t];
  } else {
    const int kk = batched ? c.inst_k[inst] : c.k;
#pragma unroll
    for (int t = 0; t < W; ++t) {
      uint32_t msk = 0;
      for (int l = 0; l < 32; ++l) {
        const int b = 32 * t + l;
        if (b < kk) {
          const int64_t sl = batched ? c.lmax[bo + b] - c.bw[bo + b] : (int64_t)s_slack[b];
          if (sl >= wv) msk |= 1u << l;
        }
      }
      cand[t] = msk;
    }
  }
  // isBorderNode: some incident net holds a block other than `from`
  uint32_t other = 0, anyc = 0;
#pragma unroll
  for (int t = 0; t < W; ++t) {
    const uint32_t fm = t == fw ? ~fbit : ~0u;
    uint32_t o = 0;
#pragma unroll
    for (int p = 0; p < PL; ++p) o |= cnt[t][p];
    other |= o & fm;
    cand[t] &= fm;
    anyc |= cand[t];
  }
  if (!other) return;
  border = true;
  if (!anyc) return;
  // maximum penalty over the candidates, plane by plane from the top
  int val = 0;
#pragma unroll
  for (int p = PL - 1; p >= 0; --p) {
    uint32_t tt[W], o = 0;
#pragma unroll
    for (int t = 0; t < W; ++t) {
      tt[t] = cand[t] & cnt[t][p];
      o |= tt[t];
    }
    if (o) {
#pragma unroll
      for (int t = 0; t < W; ++t) cand[t] = tt[t];
      val |= 1 << p;
    }
  }
  if (val < internal || (val == internal && !zero_gain)) return;
  int b = 0;  // lowest block of maximum penalty
#pragma unroll
  for (int t = W - 1; t >= 0; --t)
    if (cand[t]) b = 32 * t + __ffs(cand[t]) - 1;
  if (val > internal) {
    to = b;
    gain = internal - val;
    return;
  }
  const int64_t* bwp = batched ? c.bw + bo : s_bw;
  const int64_t* pfp = batched ? c.perfect + bo : s_perf;
  if (bwp[from] - 1 > bwp[b] + 1 && bwp[b] < pfp[b]) {
    to = b;
    gain = 0;
  }
}

// Best move of one vertex by its own lane (accumulate all incidences, decide);
// U incidences per step have their gathers in flight together; NC as in
// load_words.
template <int W, bool UNIT, int PL, int U = LPGPU_LV_UNROLL, bool NC = true>
__device__ __forceinline__ void lv_vertex(const RoundCtx& c, int64_t o0, int d, int from, int wv, int bo,
                                          int inst, bool batched, int zero_gain,
                                          const uint32_t* __restrict__ s_fmask, const int* __restrict__ s_slack,
                                          const int64_t* __restrict__ s_bw, const int64_t* __restrict__ s_perf,
                                          int& to, int& gain, bool& border) {
  static_assert(U % 4 == 0, "the carry-save adder takes four vectors at a time");
  uint32_t cnt[W][PL];
#pragma unroll
  for (int t = 0; t < W; ++t)
#pragma unroll
    for (int p = 0; p < PL; ++p) cnt[t][p] = 0;
  int internal = 0;  // Σ w(e) over incident nets with Φ(e, from) > 1
  for (int j = 0; j < d; j += U) lv_accumulate<W, UNIT, PL, U, NC>(c, o0, d, j, from, cnt, internal);
  lv_decide<W, PL>(c, cnt, internal, from, wv, bo, inst, batched, zero_gain, s_fmask, s_slack, s_bw, s_perf, to,
                   gain, border);
}


// One heavy vertex (sweep_heavy: summed net weight too large for the lane
// counters, or more than kHeavyDegree incidences) evaluated by the whole CTA:
// its warps split the incidence windows (lane = incidence, Λ words transposed
// so that lane l counts block l + 32 t), sum their per-block penalties in
// shared memory, and warp 0 decides. Query mode (dbg_to != null) writes
// to / gain / border of v; otherwise rec[pos] and the per-block candidate
// totals, counting the candidate in `cands` (thread 0 of warp 0).
template <int W, bool UNIT>
__device__ void heavy_vertex(const RoundCtx& c, int64_t pos, int64_t v, int zero_gain, int32_t* dbg_to,
                             int32_t* dbg_gain, uint8_t* dbg_border, int64_t& cands) {
  constexpr int B = W <= 4 ? 4 : (W <= 8 ? 2 : 1);  // windows per warp whose gathers are issued together
  constexpr int W2 = 2 * W;
  __shared__ int s_pen[32 * W];
  __shared__ ull s_int;
  __shared__ int s_border;
  const bool query = dbg_to != nullptr;
  const bool batched = c.batched != 0;
  const int lane = lane_id(), wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int64_t o0 = c.vtx_off[v];
  const int d = (int)(c.vtx_off[v + 1] - o0);  // 0 < d <= kHighDegree for heavy vertices
  const int inst = batched ? c.vinst[v] : 0;
  const int bo = batched ? c.inst_boff[inst] : 0;
  const int kk = batched ? c.inst_k[inst] : c.k;
  const int from = c.part[v] - bo;
  const int wv = c.w_v[v];
  for (int b = threadIdx.x; b < 32 * W; b += blockDim.x) s_pen[b] = 0;
  if (threadIdx.x == 0) {
    s_int = 0;
    s_border = 0;
  }
  __syncthreads();
  int pen[W];
#pragma unroll
  for (int t = 0; t < W; ++t) pen[t] = 0;
  long long internal = 0;
  bool border = false;
  for (int wb0 = 32 * B * wid; wb0 < d; wb0 += 32 * B * nw) {
    uint32_t wd[B][W];
    int we[B], lam[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const int j = wb0 + 32 * u + lane;
#pragma unroll
      for (int t = 0; t < W; ++t) wd[u][t] = 0;
      we[u] = 0;
      lam[u] = 0;
      if (j < d) {
        const int64_t e = c.inets[o0 + j];
        const int w = UNIT ? 1 : __ldg(&c.w_e[e]);
        const uint32_t* rec = c.conn + e * W2;
        load_words<W>(rec, wd[u]);
        const uint32_t l1 = __ldg(rec + W + (from >> 5));
        internal += ((l1 >> (from & 31)) & 1u) ? 0 : w;  // Φ(e, from) > 1
        we[u] = w;
#pragma unroll
        for (int t = 0; t < W; ++t) lam[u] += __popc(wd[u][t]);
      }
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      if (wb0 + 32 * u >= d) break;  // warp-uniform
      border = border || __ballot_sync(FULLMASK, lam[u] > 1) != 0;
      if constexpr (UNIT) {
#pragma unroll
        for (int t = 0; t < W; ++t) pen[t] += __popc(transpose32(wd[u][t]));
      } else {
        const int np = 32 - __clz(__reduce_or_sync(FULLMASK, (unsigned)we[u]));
        const Planes wp = make_planes(we[u], np);
#pragma unroll
        for (int t = 0; t < W; ++t) pen[t] += plane_sum(wp, transpose32(wd[u][t]), we[u]);
      }
    }
  }
  internal = warp_sum(internal);
  if (lane == 0 && internal) atomicAdd(&s_int, (ull)internal);
  if (lane == 0 && border) s_border = 1;
#pragma unroll
  for (int t = 0; t < W; ++t)
    if (pen[t]) atomicAdd(&s_pen[32 * t + lane], pen[t]);
  __syncthreads();
  if (wid == 0) {
    int to = from, gain = 0;
    const bool bd = s_border != 0;
    if (bd) {
      int p[W], slack[W];
#pragma unroll
      for (int t = 0; t < W; ++t) {
        const int b = 32 * t + lane;
        p[t] = s_pen[b];
        int sl = -1;
        if (b < kk) {
          const int64_t x = c.lmax[bo + b] - c.bw[bo + b];
          sl = x < 0 ? -1 : (x > INT_MAX ? INT_MAX : (int)x);
        }
        slack[t] = sl;
      }
      decide<W, UNIT>(kk, from, wv, (int)s_int, zero_gain, p, slack, c.bw + bo, c.perfect + bo, to, gain);
    }
    if (lane == 0) {
      if (query) {
        dbg_to[v] = to;
        if (dbg_gain) dbg_gain[v] = gain;
        if (dbg_border) dbg_border[v] = bd;
      } else {
        int4 r = make_int4(-1, 0, (int)v, from + bo);
        if (to != from) {
          r.x = to + bo;
          r.y = gain;
          atomicAdd(reinterpret_cast<ull*>(&c.in_w[to + bo]), (ull)(int64_t)wv);
          atomicAdd(reinterpret_cast<ull*>(&c.in_cnt[to + bo]), 1ull);
          atomicAdd(reinterpret_cast<ull*>(&c.cand_out[from + bo]), (ull)(int64_t)wv);
          ++cands;
        }
        c.rec[pos] = r;
      }
    }
  }
  __syncthreads();  // s_pen is cleared for the next vertex
}

// Sweep: the best move of every active vertex (moveVertex's isBorderNode +
// computeMaxGainMove, label_propagation_refiner.h:82-95) on the current state.
//
// Heavy vertices (sweep_heavy) lead a sub-round's list; the first `nheavy`
// CTAs take them one per CTA (heavy_vertex) while the other CTAs walk the
// rest. For k <= 128 a lane evaluates its own vertex (lv_vertex, bit-sliced
// counters). For k > 128 a warp takes a tile of 32 list entries (lane =
// vertex) and walks the tile's concatenated incidence lists in windows of 32
// incidences (lane = incidence); the gathers of B windows are issued before
// any is consumed.
// Each incidence lane loads its net's record {Λ(e), Λ1(e)} (one 32-byte
// sector for k <= 128) and, for weighted nets, w(e); Λ words are transposed
// across the warp so that lane l holds, per 32-block word t, the mask of
// incidences whose net contains block l + 32 t. A vertex's penalty for that
// block is the popcount of the mask restricted to its incidence lanes
// (through bit-planes of w(e) for weighted nets); its internal weight (nets
// with Φ(e, from) > 1, i.e. from not in Λ1(e)) and the border test come from
// ballots. A vertex that straddles windows carries its partial sums. Cost per
// incidence is independent of |Λ(e)|.
//
// Outputs: sub-round mode writes rec[pos] = (to, gain, v, from) (to = -1: none) and the
// per-block candidate totals, and its last CTA plans the selection; query
// mode (dbg_to != null) writes to / gain / border for every vertex (list =
// all vertices, no zero-gain moves).
template <int W, bool UNIT>
__global__ void __launch_bounds__(kSweepThreads, (W >= 8 ? 2 : (W == 4 ? LPGPU_SWEEP_MIN_BLOCKS : 3))) k_sweep(RoundCtx c, int round, int sub, int nheavy,
                                                             int32_t* dbg_to, int32_t* dbg_gain,
                                                             uint8_t* dbg_border) {
  constexpr int B = W <= 8 ? 2 : 1;  // windows whose gathers are issued together (k > 128)
  extern __shared__ unsigned char smem_raw[];
  const bool batched = c.batched != 0;
  const int k = batched ? 0 : c.k;  // blocks kept in shared memory (none when batched)
  const bool query = dbg_to != nullptr;
  int64_t* s_bw = reinterpret_cast<int64_t*>(smem_raw);
  int64_t* s_perf = s_bw + k;
  ull* s_in_w = reinterpret_cast<ull*>(s_perf + k);
  ull* s_out_w = s_in_w + k;
  int* s_slack = reinterpret_cast<int*>(s_out_w + k);
  unsigned* s_in_cnt = reinterpret_cast<unsigned*>(s_slack + k);
  // feasibility masks of the lane-per-vertex path: word t of weight w at (w - 1) W + t
  constexpr bool kLv = W <= 4;
  constexpr int PL = UNIT ? 6 : 8;  // lane-per-vertex counter planes
  const int nfm = (kLv && !batched) ? kLvWeights * W : 0;
  uint32_t* s_fmask = reinterpret_cast<uint32_t*>(s_in_cnt + k);
  unsigned char* s_owner = reinterpret_cast<unsigned char*>(s_fmask + nfm) + (threadIdx.x >> 5) * 32;
  for (int b = threadIdx.x; b < k; b += blockDim.x) {
    const int64_t bw = c.bw[b];
    const int64_t sl = c.lmax[b] - bw;
    s_bw[b] = bw;
    s_perf[b] = query ? 0 : c.perfect[b];
    s_slack[b] = sl < 0 ? -1 : (sl > INT_MAX ? INT_MAX : (int)sl);
    s_in_w[b] = 0;
    s_out_w[b] = 0;
    s_in_cnt[b] = 0;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nfm; i += blockDim.x) {
    const int w = i / W + 1, t = i % W;
    uint32_t msk = 0;
    for (int l = 0; l < 32; ++l) {
      const int b = 32 * t + l;
      if (b < k && s_slack[b] >= w) msk |= 1u << l;
    }
    s_fmask[i] = msk;
  }
  if (nfm) __syncthreads();
  const int lane = lane_id();
  int slack[W];
#pragma unroll
  for (int t = 0; t < W; ++t) slack[t] = (32 * t + lane < k) ? s_slack[32 * t + lane] : -1;
  int slack_inst = -1;  // batched: instance whose block slack is in `slack`
  const int zero_gain = query ? 0 : c.zero_gain;
  const int64_t sbeg = query ? 0 : c.sub_off[sub];
  const int64_t total = query ? c.n : c.sub_off[sub + 1] - sbeg;
  const int W2 = 2 * W;
  int64_t pins = 0, cands = 0;
  // sub-round mode: the sub-round's heavy vertices lead its list; the first
  // `nheavy` CTAs take them one at a time while the others walk the rest
  const int H = query ? 0 : nheavy;
  const int64_t hcnt = H ? c.sub_off[kMaxSubrounds + 1 + sub] - sbeg : 0;
  const int lb = (int)blockIdx.x - H;  // index among the lane-per-vertex CTAs (< 0: heavy CTA)
  if (lb < 0) {
    for (int64_t i = blockIdx.x; i < hcnt; i += H) {
      const int64_t v = c.list[sbeg + i];
      if (threadIdx.x == 0) pins += c.vtx_off[v + 1] - c.vtx_off[v];
      heavy_vertex<W, UNIT>(c, sbeg + i, v, zero_gain, nullptr, nullptr, nullptr, cands);
    }
  }
  const int64_t beg = sbeg + hcnt;
  const int64_t cnt = lb < 0 ? 0 : total - hcnt;
  const int64_t wstride = (int64_t)(gridDim.x - H) * blockDim.x;
  for (int64_t tile = (int64_t)(lb < 0 ? 0 : lb) * blockDim.x + threadIdx.x - lane; tile < cnt; tile += wstride) {
    // ---- one vertex per lane
    const int64_t pos = beg + tile + lane;
    const bool valid = tile + lane < cnt;
    const int64_t v = valid ? (query ? pos : (int64_t)c.list[pos]) : 0;
    int64_t o0 = 0;
    int d = 0, from = 0, wv = 0, bo = 0, inst = 0;
    if (valid) {
      o0 = c.vtx_off[v];
      const int64_t dd = c.vtx_off[v + 1] - o0;
      pins += dd;
      d = dd > kHighDegree ? 0 : (int)dd;  // isBorderNode is false above the threshold
      if (batched) {
        inst = c.vinst[v];
        bo = c.inst_boff[inst];
      }
      from = c.part[v] - bo;  // local block id
      wv = c.w_v[v];
    }
    int my_to = from, my_gain = 0;
    bool my_border = false;
    // light vertices are evaluated here; in query mode heavy ones are deferred
    // to k_sweep_heavy (sub-round lists keep them in the heavy CTAs' range)
    const bool heavy = sweep_heavy(d, W, UNIT, c.max_we);
    const bool defer = heavy && query;
    if constexpr (kLv) {
      if (d > 0 && !heavy)
        lv_vertex<W, UNIT, PL>(c, o0, d, from, wv, bo, inst, batched, zero_gain, s_fmask, s_slack, s_bw, s_perf,
                               my_to, my_gain, my_border);
      d = 0;
    } else if (heavy) {
      d = 0;
    }
    const unsigned dm = __ballot_sync(FULLMASK, defer);
    if (dm) {
      const int leader = __ffs(dm) - 1;
      ull base = 0;
      if (lane == leader) base = atomicAdd(reinterpret_cast<ull*>(&c.scal[kHeavyCount]), (ull)__popc(dm));
      base = __shfl_sync(FULLMASK, base, leader);
      if (defer) c.heavy[base + __popc(dm & lanemask_lt())] = (int32_t)pos;
    }
    if constexpr (!kLv) {  // k > 128: the tile's remaining vertices in warp windows
      int incl = d;
  #pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULLMASK, incl, o);
        if (lane >= o) incl += y;
      }
      const int excl = incl - d, eend = incl;
      const int R = __shfl_sync(FULLMASK, incl, 31);  // incidences of the tile
      const unsigned nz = __ballot_sync(FULLMASK, d > 0);
      __syncwarp();
      if (d > 0) s_owner[__popc(nz & lanemask_lt())] = (unsigned char)lane;
      __syncwarp();
      // partial sums of the vertex that continues past the current window
      int carry[W];
  #pragma unroll
      for (int t = 0; t < W; ++t) carry[t] = 0;
      int carry_int = 0;
      bool carry_border = false;

      // ---- the tile's incidences in windows of 32 (lane = incidence)
      for (int wb0 = 0; wb0 < R; wb0 += 32 * B) {
        uint32_t wd[B][W];
        int icv[B], lamv[B], wev[B];
  #pragma unroll
        for (int u = 0; u < B; ++u) {
          const int wb = wb0 + 32 * u;
          const int i = wb + lane;
          const bool has = i < R;
          const unsigned starts =
              __reduce_or_sync(FULLMASK, (d > 0 && excl >= wb && excl < wb + 32) ? (1u << (excl - wb)) : 0u);
          const int cb = __popc(__ballot_sync(FULLMASK, d > 0 && excl < wb));
          const int ow = has ? s_owner[cb + __popc(starts & ((2u << lane) - 1u)) - 1] : 0;
          const int64_t o_ow = __shfl_sync(FULLMASK, o0, ow);
          const int ex_ow = __shfl_sync(FULLMASK, excl, ow);
          const int f_ow = __shfl_sync(FULLMASK, from, ow);
  #pragma unroll
          for (int t = 0; t < W; ++t) wd[u][t] = 0;
          icv[u] = 0;
          lamv[u] = 0;
          wev[u] = 0;
          if (has) {
            const int64_t e = __ldcs(&c.inets[o_ow + i - ex_ow]);
            const int we = UNIT ? 1 : __ldg(&c.w_e[e]);
            const uint32_t* rec = c.conn + e * W2;
            load_words<W>(rec, wd[u]);
            const uint32_t l1 = __ldg(rec + W + (f_ow >> 5));
            icv[u] = ((l1 >> (f_ow & 31)) & 1u) ? 0 : we;  // Φ(e, from) > 1
            wev[u] = we;
            int lam = 0;
  #pragma unroll
            for (int t = 0; t < W; ++t) lam += __popc(wd[u][t]);
            lamv[u] = lam;
          }
        }
  #pragma unroll
        for (int u = 0; u < B; ++u) {
          const int wb = wb0 + 32 * u;
          if (wb >= R) break;
          uint32_t col[W];
  #pragma unroll
          for (int t = 0; t < W; ++t) col[t] = transpose32(wd[u][t]);
          const unsigned bm = __ballot_sync(FULLMASK, lamv[u] > 1);
          const unsigned icb = __ballot_sync(FULLMASK, icv[u] != 0);
          Planes wp, ip;
          if constexpr (!UNIT) {
            const int np = 32 - __clz(__reduce_or_sync(FULLMASK, (unsigned)wev[u]));
            wp = make_planes(wev[u], np);
            ip = make_planes(icv[u], np);
          }
          // vertices whose last incidence lies in this window
          unsigned endm = __ballot_sync(FULLMASK, d > 0 && eend > wb && eend <= wb + 32);
          while (endm) {
            const int j = __ffs(endm) - 1;
            endm &= endm - 1;
            const int exj = __shfl_sync(FULLMASK, excl, j);
            const int hi = __shfl_sync(FULLMASK, eend, j) - wb;
            const int lo = exj > wb ? exj - wb : 0;
            const unsigned mask = (hi == 32 ? FULLMASK : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
            const bool cont = exj < wb;
            if ((bm & mask) == 0 && !(cont && carry_border)) continue;  // not a border vertex
            int internal;
            int pen[W];
            if constexpr (UNIT) {
              internal = __popc(icb & mask);
  #pragma unroll
              for (int t = 0; t < W; ++t) pen[t] = __popc(col[t] & mask);
            } else {
              internal = plane_sum(ip, mask, icv[u]);
  #pragma unroll
              for (int t = 0; t < W; ++t) pen[t] = plane_sum(wp, col[t] & mask, wev[u]);
            }
            if (cont) {
              internal += carry_int;
  #pragma unroll
              for (int t = 0; t < W; ++t) pen[t] += carry[t];
            }
            const int fromj = __shfl_sync(FULLMASK, from, j);
            const int wvj = __shfl_sync(FULLMASK, wv, j);
            int to = fromj, gain = 0;
            if (batched) {
              const int ij = __shfl_sync(FULLMASK, inst, j);
              const int boj = c.inst_boff[ij];
              const int kj = c.inst_k[ij];
              if (ij != slack_inst) {  // warp-uniform: reload the instance's block slack
                slack_inst = ij;
  #pragma unroll
                for (int t = 0; t < W; ++t) {
                  const int b = 32 * t + lane;
                  int sl = -1;
                  if (b < kj) {
                    const int64_t x = c.lmax[boj + b] - c.bw[boj + b];
                    sl = x < 0 ? -1 : (x > INT_MAX ? INT_MAX : (int)x);
                  }
                  slack[t] = sl;
                }
              }
              decide<W, UNIT>(kj, fromj, wvj, internal, zero_gain, pen, slack, c.bw + boj, c.perfect + boj, to,
                              gain);
            } else {
              decide<W, UNIT>(k, fromj, wvj, internal, zero_gain, pen, slack, s_bw, s_perf, to, gain);
            }
            if (lane == j) {
              my_to = to;
              my_gain = gain;
              my_border = true;
            }
          }
          // the vertex that continues into the next window (at most one)
          const unsigned openm = __ballot_sync(FULLMASK, d > 0 && excl < wb + 32 && eend > wb + 32);
          if (openm) {
            const int j = __ffs(openm) - 1;
            const int exj = __shfl_sync(FULLMASK, excl, j);
            const int lo = exj > wb ? exj - wb : 0;
            const unsigned mask = FULLMASK & ~((1u << lo) - 1u);
            const bool cont = exj < wb;
            int pint;
            if constexpr (UNIT) {
              pint = __popc(icb & mask);
            } else {
              pint = plane_sum(ip, mask, icv[u]);
            }
            const bool pb = (bm & mask) != 0;
  #pragma unroll
            for (int t = 0; t < W; ++t) {
              int p;
              if constexpr (UNIT) {
                p = __popc(col[t] & mask);
              } else {
                p = plane_sum(wp, col[t] & mask, wev[u]);
              }
              carry[t] = cont ? carry[t] + p : p;
            }
            carry_int = cont ? carry_int + pint : pint;
            carry_border = cont ? (carry_border || pb) : pb;
          }
        }
      }
    }

    if (valid && !defer) {
      if (query) {
        dbg_to[v] = my_to;
        if (dbg_gain) dbg_gain[v] = my_gain;
        if (dbg_border) dbg_border[v] = my_border;
      } else {
        int4 r = make_int4(-1, 0, (int)v, from + bo);
        if (my_to != from) {
          r.x = my_to + bo;  // global target block
          r.y = my_gain;
          if (batched) {
            atomicAdd(reinterpret_cast<ull*>(&c.in_w[my_to + bo]), (ull)(int64_t)wv);
            atomicAdd(reinterpret_cast<ull*>(&c.in_cnt[my_to + bo]), 1ull);
            atomicAdd(reinterpret_cast<ull*>(&c.cand_out[from + bo]), (ull)(int64_t)wv);
          } else {
            atomicAdd(&s_in_w[my_to], (ull)(int64_t)wv);
            atomicAdd(&s_in_cnt[my_to], 1u);
            atomicAdd(&s_out_w[from], (ull)(int64_t)wv);
          }
          ++cands;
        }
        c.rec[pos] = r;
      }
    }
  }
  if (query) return;
  pins = block_sum_i64(pins);
  cands = block_sum_i64(cands);
  if (threadIdx.x == 0) {
    int64_t* st = c.stats + (int64_t)round * kStats;
    atomicAdd(reinterpret_cast<ull*>(&st[kStPins]), (ull)pins);
    atomicAdd(reinterpret_cast<ull*>(&st[kStCands]), (ull)cands);
    if (blockIdx.x == 0) atomicAdd(reinterpret_cast<ull*>(&st[kStActive]), (ull)total);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < k; b += blockDim.x) {
    if (s_in_cnt[b]) {
      atomicAdd(reinterpret_cast<ull*>(&c.in_w[b]), s_in_w[b]);
      atomicAdd(reinterpret_cast<ull*>(&c.in_cnt[b]), (ull)s_in_cnt[b]);
    }
    if (s_out_w[b]) atomicAdd(reinterpret_cast<ull*>(&c.cand_out[b]), s_out_w[b]);
  }
  if (last_cta(&c.scal[kDone])) plan_to(c);
}

// Per-vertex queries: the heavy vertices k_sweep deferred (list = all
// vertices, positions in c.heavy), one CTA each; clears the deferred count.
template <int W, bool UNIT>
__global__ void __launch_bounds__(kSweepThreads) k_sweep_heavy(RoundCtx c, int32_t* dbg_to, int32_t* dbg_gain,
                                                               uint8_t* dbg_border) {
  const int64_t nh = *(volatile int64_t*)&c.scal[kHeavyCount];
  if (nh == 0) return;
  int64_t cands = 0;
  for (int64_t i = blockIdx.x; i < nh; i += gridDim.x) {
    const int32_t v = c.heavy[i];
    heavy_vertex<W, UNIT>(c, v, v, 0, dbg_to, dbg_gain, dbg_border, cands);
  }
  if (last_cta(&c.scal[kDone]) && threadIdx.x == 0) c.scal[kHeavyCount] = 0;
}

#define LPGPU_DISPATCH_W(W, ...)          \
  switch (W) {                            \
    case 1: { constexpr int kW = 1; __VA_ARGS__; } break;   \
    case 2: { constexpr int kW = 2; __VA_ARGS__; } break;   \
    case 4: { constexpr int kW = 4; __VA_ARGS__; } break;   \
    case 8: { constexpr int kW = 8; __VA_ARGS__; } break;   \
    case 16: { constexpr int kW = 16; __VA_ARGS__; } break; \
    case 32: { constexpr int kW = 32; __VA_ARGS__; } break; \
    default: return cudaErrorInvalidValue;                  \
  }

// Words per net rounded up to a template instance.
static int word_class(int W) {
  int w = 1;
  while (w < W) w <<= 1;
  return w;
}


static size_t sweep_smem(int k, int W, bool batched) {
  const size_t fm = (W <= 4 && !batched) ? sizeof(uint32_t) * kLvWeights * W : 0;
  return sizeof(int64_t) * 4 * k + sizeof(int) * k + sizeof(unsigned) * k + fm + 32 * (kSweepThreads / 32);
}

static cudaError_t launch_sweep(const Launch& L, const RoundCtx& c, int round, int sub,
                                int32_t* to, int32_t* gain, uint8_t* border) {
  if (word_class(c.W) != c.W) return cudaErrorInvalidValue;
  const size_t smem = sweep_smem(c.batched ? 0 : c.k, c.W, c.batched != 0);
  LPGPU_DISPATCH_W(c.W, {
    auto kern = c.unit_nets ? k_sweep<kW, true> : k_sweep<kW, false>;
    allow_dyn_smem(kern, smem);
    const int per_sm = occupancy((const void*)kern, kSweepThreads, smem);
    int grid = grid_for(L, c.n * 4, kSweepThreads, per_sm);
    // CTAs for the heavy vertices: their share of the work, at least two
    int H = 0;
    if (!to && c.heavy_share > 0) {
      H = std::max(2, (int)((int64_t)grid * c.heavy_share / 1000));
      H = std::min(H, std::max(1, grid - 1));
      grid = std::max(grid, H + 1);
    }
    kern<<<grid, kSweepThreads, smem, L.st>>>(c, round, sub, H, to, gain, border);
    LAUNCHED("k_sweep");
    if (to) {
      auto heavy = c.unit_nets ? k_sweep_heavy<kW, true> : k_sweep_heavy<kW, false>;
      heavy<<<grid_for(L, c.n, kSweepThreads, 2), kSweepThreads, 0, L.st>>>(c, to, gain, border);
      LAUNCHED("k_sweep_heavy");
    }
  });
  return cudaSuccess;
}

cudaError_t launch_best_moves(const Launch& L, const RoundCtx& c, int32_t* to, int32_t* gain,
                              uint8_t* border) {
  if (c.n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(c.scal + kHeavyCount, 0, sizeof(int64_t), L.st);
  if (e != cudaSuccess) return e;
  return launch_sweep(L, c, 0, 0, to, gain, border);
}

// ============================================================ gain cache

// moveFromBenefit / moveToPenalty for every vertex (initializeGainCache,
// h:707-809): warp per vertex with a per-warp k-bin shared aggregator.
__global__ void __launch_bounds__(256) k_gain_cache(RoundCtx c, int32_t* benefit, int32_t* penalty) {
  extern __shared__ int s_agg[];
  int* agg = s_agg + (threadIdx.x >> 5) * c.k;
  const int lane = lane_id();
  for (int b = lane; b < c.k; b += 32) agg[b] = 0;
  __syncwarp();
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; v < c.n; v += warps) {
    const int pv = c.part[v];
    int ben = 0, inc = 0;
    for (int64_t j = c.vtx_off[v] + lane; j < c.vtx_off[v + 1]; j += 32) {
      const int e = c.inets[j];
      const int we = c.w_e[e];
      if (phi_get(c, (int64_t)e * c.k + pv) == 1) ben += we;
      inc += we;
      for (int w = 0; w < c.W; ++w) {
        uint32_t bits = c.conn[(int64_t)e * 2 * c.W + w];
        while (bits) {
          const int t = __ffs(bits) - 1;
          bits &= bits - 1;
          atomicAdd(&agg[w * 32 + t], we);
        }
      }
    }
    ben = warp_sum(ben);
    inc = warp_sum(inc);
    __syncwarp();
    for (int b = lane; b < c.k; b += 32) {
      penalty[v * c.k + b] = inc - agg[b];
      agg[b] = 0;
    }
    if (lane == 0) benefit[v] = ben;
    __syncwarp();
  }
}

cudaError_t launch_gain_cache(const Launch& L, const RoundCtx& c, int32_t* benefit, int32_t* penalty) {
  if (c.n == 0) return cudaSuccess;
  const size_t smem = sizeof(int) * c.k * 8;
  allow_dyn_smem(k_gain_cache, smem);
  k_gain_cache<<<grid_for(L, c.n * 32, 256), 256, smem, L.st>>>(c, benefit, penalty);
  LAUNCHED("k_gain_cache");
  return cudaGetLastError();
}

// ================================================================ commit

// Moves v from `f` to `t` on Φ, Λ and Λ1: per incident net one atomic
// decrement of Φ(e,f) and one atomic increment of Φ(e,t)
// (updatePinCountOfHyperedge, h:1133-1167). Each atomic returns the old count,
// so every transition is seen exactly once: Λ bits toggle on 1->0 / 0->1 and
// Λ1 bits toggle whenever the count enters or leaves 1. Concurrent moves on
// one net therefore leave Λ and Λ1 consistent with the final counts. Returns
// this lane's share of the attributed delta (km1Delta,
// hypergraph_common.h:133-140): -w(e) when Φ(e,f) drops to 0, +w(e) when
// Φ(e,t) rises to 1. The per-move split depends on interleaving; the sum over
// all concurrent moves is exactly the km1 change.
// Gain-cache maintenance for one flip of net e in block b (gainCacheUpdate,
// partitioned_hypergraph.h:1017-1047, stated on the transitions an atomic
// observed): `one` = +1 / -1 when Φ(e, b) reaches / leaves 1, `zero` = +1 / -1
// when Φ(e, b) reaches / leaves 0. moveToPenalty(u, b) (the weight of u's nets
// without b) changes with `zero` for every pin; moveFromBenefit(u) changes with
// `one` for the pins in block b that are not moving in this batch (moving
// vertices are recomputed afterwards).
__device__ __forceinline__ void gc_flip(const RoundCtx& c, const GainCache& g, int64_t e, int b, int one, int zero,
                                        int we) {
  if (!one && !zero) return;
  for (int64_t q = c.net_off[e]; q < c.net_off[e + 1]; ++q) {
    const int u = c.pins[q];
    if (zero) atomicAdd(&g.penalty[(int64_t)u * c.k + b], zero * we);
    if (one && !g.moved[u] && c.part[u] == b) atomicAdd(&g.benefit[u], one * we);
  }
}

__device__ __forceinline__ int64_t warp_commit_vertex(const RoundCtx& c, int64_t v, int f, int t, const GainCache& g) {
  int64_t att = 0;
  const int k = c.kmax, W = c.W;
  const uint32_t fbit = 1u << (f & 31), tbit = 1u << (t & 31);
  for (int64_t j = c.vtx_off[v] + lane_id(); j < c.vtx_off[v + 1]; j += 32) {
    const int64_t e = c.inets[j];
    const int we = c.w_e[e];
    uint32_t* rec = c.conn + e * 2 * W;
    const int of = phi_add(c, e * k + f, -1);
    if (of == 1) {
      atomicXor(&rec[f >> 5], fbit);
      att -= we;
    }
    if (of == 1 || of == 2) atomicXor(&rec[W + (f >> 5)], fbit);
    const int ot = phi_add(c, e * k + t, 1);
    if (ot == 0) {
      atomicXor(&rec[t >> 5], tbit);
      att += we;
    }
    if (ot == 0 || ot == 1) atomicXor(&rec[W + (t >> 5)], tbit);
    if (g.benefit) {
      // f: of -> of - 1; t: ot -> ot + 1
      gc_flip(c, g, e, f, of == 2 ? 1 : (of == 1 ? -1 : 0), of == 1 ? 1 : 0, we);
      gc_flip(c, g, e, t, ot == 0 ? 1 : (ot == 1 ? -1 : 0), ot == 0 ? -1 : 0, we);
    }
  }
  return att;
}

// Concurrent application of an explicit move list (lpgpu_session_apply_moves).
__global__ void k_apply_moves(RoundCtx c, int64_t count, const int32_t* __restrict__ vs,
                              const int32_t* __restrict__ fs, const int32_t* __restrict__ ts, GainCache g) {
  int64_t att = 0;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < count; i += warps) {
    const int64_t v = vs[i];
    const int f = fs[i], t = ts[i];
    att += warp_commit_vertex(c, v, f, t, g);
    if (lane_id() == 0) {
      c.part[v] = t;
      const int64_t wv = c.w_v[v];
      atomicAdd(reinterpret_cast<ull*>(&c.bw[t]), (ull)wv);
      atomicAdd(reinterpret_cast<ull*>(&c.bw[f]), (ull)(-wv));
    }
  }
  att = block_sum_i64(att);
  if (threadIdx.x == 0) atomicAdd(reinterpret_cast<ull*>(&c.scal[kApplyDelta]), (ull)att);
}

__global__ void k_mark_moved(int64_t count, const int32_t* __restrict__ vs, uint8_t* moved, uint8_t value) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    moved[vs[i]] = value;
}

// moveFromBenefit of the moved vertices on the final state: Σ w(e) over
// their nets with Φ(e, part(v)) = 1 (warp per vertex).
__global__ void k_gc_moved_benefit(RoundCtx c, int64_t count, const int32_t* __restrict__ vs, int32_t* benefit) {
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < count; i += warps) {
    const int64_t v = vs[i];
    const int pv = c.part[v];
    int ben = 0;
    for (int64_t j = c.vtx_off[v] + lane_id(); j < c.vtx_off[v + 1]; j += 32) {
      const int64_t e = c.inets[j];
      if (phi_get(c, e * c.kmax + pv) == 1) ben += c.w_e[e];
    }
    ben = warp_sum(ben);
    if (lane_id() == 0) benefit[v] = ben;
  }
}

cudaError_t launch_apply_moves(const Launch& L, const RoundCtx& c, int64_t count, const int32_t* v,
                               const int32_t* from, const int32_t* to, const GainCache& g) {
  cudaError_t e = cudaMemsetAsync(c.scal + kApplyDelta, 0, sizeof(int64_t), L.st);
  if (e != cudaSuccess) return e;
  if (count > 0) {
    const int gm = grid_for(L, count, 256);
    if (g.benefit) {
      k_mark_moved<<<gm, 256, 0, L.st>>>(count, v, g.moved, 1);
      LAUNCHED("k_mark_moved");
    }
    k_apply_moves<<<grid_for(L, count * 32, 256), 256, 0, L.st>>>(c, count, v, from, to, g);
    LAUNCHED("k_apply_moves");
    if (g.benefit) {
      k_gc_moved_benefit<<<grid_for(L, count * 32, 256), 256, 0, L.st>>>(c, count, v, g.benefit);
      LAUNCHED("k_gc_moved_benefit");
      k_mark_moved<<<gm, 256, 0, L.st>>>(count, v, g.moved, 0);
      LAUNCHED("k_mark_moved");
    }
  }
  return cudaGetLastError();
}

// ========================================================= active lists


__global__ void k_mark_all(uint8_t* flag, int64_t n) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    flag[v] = 1;
}

// initializeActiveNodes without rebalancing: border vertices only.
__global__ void k_mark_border(RoundCtx c) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < c.n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = c.vtx_off[v], e = c.vtx_off[v + 1];
    uint8_t f = 0;
    if (e - b <= kHighDegree) {
      for (int64_t j = b; j < e && !f; ++j) {
        int lam = 0;
        for (int w = 0; w < c.W; ++w) lam += __popc(c.conn[(int64_t)c.inets[j] * 2 * c.W + w]);
        f = lam > 1;
      }
    }
    c.next_flag[v] = f;
  }
}

__global__ void k_mark_list(uint8_t* flag, const int32_t* nodes, int64_t count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    flag[nodes[i]] = 1;
}

cudaError_t launch_mark_all(const Launch& L, const RoundCtx& c, int rebalancing) {
  if (c.n == 0) return cudaSuccess;
  if (rebalancing) {
    k_mark_all<<<grid_for(L, c.n, 256), 256, 0, L.st>>>(c.next_flag, c.n);
    LAUNCHED("k_mark_all");
  } else {
    k_mark_border<<<grid_for(L, c.n, 256), 256, 0, L.st>>>(c);
    LAUNCHED("k_mark_border");
  }
  return cudaGetLastError();
}

cudaError_t launch_mark_list(const Launch& L, const RoundCtx& c, const int32_t* nodes, int64_t count) {
  if (c.n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(c.next_flag, 0, c.n, L.st);
  if (e != cudaSuccess) return e;
  if (count > 0) {
    k_mark_list<<<grid_for(L, count, 256), 256, 0, L.st>>>(c.next_flag, nodes, count);
    LAUNCHED("k_mark_list");
  }
  return cudaGetLastError();
}

// Active-list binning. Each round's active vertices are grouped by sub-round
// and, inside a sub-round, by class (vertex_class): the heavy vertices first,
// which the sweep gives to whole CTAs, then the degree classes, since the
// lane-per-vertex sweep runs a warp until its longest incidence list is done.
// Bin b = sub-round * kDegClasses + class. k_bin_count adds each CTA's
// flagged vertices per bin to cnt[b] and keeps each flagged vertex's class in
// its flag (1 + class); k_bin_offsets turns the counts into the bins' start
// positions (cursors) and clears the counts for the next round; k_bin_scatter
// places batches of 32-vertex chunks with one cursor atomic per bin and batch
// and clears the flags. A warp's vertices of one bin stay together in id
// order; the order of the batches inside a bin is the order of their atomics,
// and which position a vertex takes inside its sub-round changes no result.
//
// All 32 vertices of an aligned chunk share one sub-round. Batched sessions
// hash instance-local ids (so that an instance gets the same sub-rounds alone
// and in a batch): then a chunk may straddle two instances and every vertex
// computes its own sub-round.
__device__ __forceinline__ int vertex_subround(const int32_t* vinst, const int64_t* inst_voff, int64_t v,
                                               int round, int S) {
  return subround_of(vinst ? v - inst_voff[vinst[v]] : v, round, S);
}

// Heavy vertices (sweep_heavy) -> 0; the others by the groups of four
// incidences a sweep lane walks: 0-4 incidences -> 1, 5-8 -> 2, ..., capped
// at the last class.
struct ClassRule {
  const int64_t* vtx_off;
  int W, unit_nets, max_we;
};
__device__ __forceinline__ int vertex_class(const ClassRule& r, int64_t v) {
  const int64_t d = r.vtx_off[v + 1] - r.vtx_off[v];
  if (sweep_heavy(d, r.W, r.unit_nets, r.max_we)) return 0;
  const int64_t g = (d + 3) >> 2;
  return g <= 1 ? 1 : (g >= kDegClasses - 1 ? kDegClasses - 1 : (int)g);  // D = 2: always 1
}

constexpr int kListBins = kMaxSubrounds * kDegClasses;  // (sub-round, class) bins
constexpr int kListBinThreads = 1024;                     // binning CTAs
constexpr int kListBinBatch = 4;  // chunks per warp and batch (independent loads in flight)
constexpr int kListBinChunks = (kListBinThreads / 32) * kListBinBatch;

__global__ void __launch_bounds__(kListBinThreads) k_bin_count(uint8_t* __restrict__ flag, int64_t n, int round,
                                                               int S, int64_t* __restrict__ cnt, ClassRule rule,
                                                               const int32_t* __restrict__ vinst,
                                                               const int64_t* __restrict__ inst_voff) {
  __shared__ int s_cnt[kListBins];
  const int bins = S * kDegClasses;
  const int w = threadIdx.x >> 5, lane = lane_id();
  for (int i = threadIdx.x; i < bins; i += blockDim.x) s_cnt[i] = 0;
  __syncthreads();
  const int64_t chunks = (n + 31) >> 5;
  for (int64_t c0 = (int64_t)blockIdx.x * kListBinChunks; c0 < chunks; c0 += (int64_t)gridDim.x * kListBinChunks) {
    bool f[kListBinBatch];
#pragma unroll
    for (int j = 0; j < kListBinBatch; ++j) {
      const int64_t v = ((c0 + j * 32 + w) << 5) + lane;
      f[j] = v < n && flag[v];
    }
    int cls[kListBinBatch];
#pragma unroll
    for (int j = 0; j < kListBinBatch; ++j) cls[j] = f[j] ? vertex_class(rule, ((c0 + j * 32 + w) << 5) + lane) : 0;
#pragma unroll
    for (int j = 0; j < kListBinBatch; ++j) {
      const int64_t v = ((c0 + j * 32 + w) << 5) + lane;
      if (f[j]) flag[v] = (uint8_t)(1 + cls[j]);
      if (vinst) {
        if (f[j]) atomicAdd(&s_cnt[vertex_subround(vinst, inst_voff, v, round, S) * kDegClasses + cls[j]], 1);
      } else {
        const int sub = subround_of(v, round, S);
#pragma unroll
        for (int q = 0; q < kDegClasses; ++q) {
          const unsigned bal = __ballot_sync(FULLMASK, f[j] && cls[j] == q);
          if (lane == 0 && bal) atomicAdd(&s_cnt[sub * kDegClasses + q], __popc(bal));
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < bins; i += blockDim.x)
    if (s_cnt[i]) atomicAdd(reinterpret_cast<ull*>(&cnt[i]), (ull)s_cnt[i]);
}

// One CTA: the bins' start positions (cnt[kListBins + b]) from their counts,
// which are cleared for the next round; the sub-round offsets (sub-round s
// occupies list[sub_off[s] .. sub_off[s + 1]), its heavy vertices the first
// sub_off[kMaxSubrounds + 1 + s] - sub_off[s]) and the round's activation
// epoch.
constexpr int kListOffThreads = (kListBins + 31) / 32 * 32;
__global__ void __launch_bounds__(kListOffThreads) k_bin_offsets(int64_t* __restrict__ cnt, int S,
                                                                 int64_t* __restrict__ sub_off, int64_t* scal) {
  __shared__ int64_t s_off[kListBins];
  const int bins = S * kDegClasses, i = threadIdx.x;
  const int64_t x = i < bins ? cnt[i] : 0;
  int64_t total;
  const int64_t off = block_scan_excl_i64(x, &total);
  if (i < bins) {
    cnt[kListBins + i] = off;
    cnt[i] = 0;
    s_off[i] = off;
  }
  __syncthreads();
  if (i < S) {
    sub_off[i] = s_off[i * kDegClasses];
    sub_off[kMaxSubrounds + 1 + i] = s_off[i * kDegClasses + 1];  // end of the heavy class
  }
  if (i == 0) {
    sub_off[S] = total;
    scal[kEpoch] += 1;  // new round: fresh activation stamp
  }
}

__global__ void __launch_bounds__(kListBinThreads) k_bin_scatter(uint8_t* __restrict__ flag, int64_t n, int round,
                                                                 int S, int64_t* __restrict__ cnt,
                                                                 int32_t* __restrict__ list,
                                                                 const int32_t* __restrict__ vinst,
                                                                 const int64_t* __restrict__ inst_voff) {
  __shared__ int s_cnt[kListBins];
  __shared__ int64_t s_base[kListBins];
  int64_t* cursor = cnt + kListBins;
  const int bins = S * kDegClasses;
  const int w = threadIdx.x >> 5, lane = lane_id();
  for (int i = threadIdx.x; i < bins; i += blockDim.x) s_cnt[i] = 0;
  __syncthreads();
  const int64_t chunks = (n + 31) >> 5;
  for (int64_t c0 = (int64_t)blockIdx.x * kListBinChunks; c0 < chunks; c0 += (int64_t)gridDim.x * kListBinChunks) {
    int fl[kListBinBatch];
#pragma unroll
    for (int j = 0; j < kListBinBatch; ++j) {
      const int64_t v = ((c0 + j * 32 + w) << 5) + lane;
      fl[j] = v < n ? flag[v] : 0;
    }
    // each vertex's bin and its place among the batch's vertices of that bin
    int bin[kListBinBatch], at[kListBinBatch];
#pragma unroll
    for (int j = 0; j < kListBinBatch; ++j) {
      const int64_t v = ((c0 + j * 32 + w) << 5) + lane;
      const bool f = fl[j] != 0;
      const int cls = f ? fl[j] - 1 : 0;
      bin[j] = -1;
      at[j] = 0;
      if (vinst) {
        if (f) {
          bin[j] = vertex_subround(vinst, inst_voff, v, round, S) * kDegClasses + cls;
          at[j] = atomicAdd(&s_cnt[bin[j]], 1);
        }
      } else {
        const int sub = subround_of(v, round, S);
#pragma unroll
        for (int q = 0; q < kDegClasses; ++q) {
          const unsigned bal = __ballot_sync(FULLMASK, f && cls == q);
          int o = 0;
          if (lane == 0 && bal) o = atomicAdd(&s_cnt[sub * kDegClasses + q], __popc(bal));
          o = __shfl_sync(FULLMASK, o, 0);
          if (f && cls == q) {
            bin[j] = sub * kDegClasses + q;
            at[j] = o + __popc(bal & lanemask_lt());
          }
        }
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < bins; i += blockDim.x) {
      const int c = s_cnt[i];
      if (c) s_base[i] = (int64_t)atomicAdd(reinterpret_cast<ull*>(&cursor[i]), (ull)c);
      s_cnt[i] = 0;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kListBinBatch; ++j) {
      if (bin[j] >= 0) {
        const int64_t v = ((c0 + j * 32 + w) << 5) + lane;
        list[s_base[bin[j]] + at[j]] = (int32_t)v;
        flag[v] = 0;
      }
    }
  }
}

// ================================================================= timer

int PhaseTimer::phase_id(const char* name) {
  for (size_t i = 0; i < names.size(); ++i)
    if (names[i] == name) return (int)i;
  names.emplace_back(name);
  return (int)names.size() - 1;
}
void PhaseTimer::begin(int phase, cudaEvent_t* a) {
  (void)phase;
  if (used + 2 > pool.size()) {
    for (int i = 0; i < 64; ++i) {
      cudaEvent_t ev;
      cudaEventCreate(&ev);
      pool.push_back(ev);
    }
  }
  *a = pool[used++];
  cudaEventRecord(*a, st);
}
void PhaseTimer::end(int phase, cudaEvent_t a) {
  cudaEvent_t b = pool[used++];
  cudaEventRecord(b, st);
  recs.push_back({phase, a, b});
}
void PhaseTimer::reset() {
  recs.clear();
  used = 0;
}
PhaseTimer::~PhaseTimer() {
  for (auto ev : pool) cudaEventDestroy(ev);
}

struct Scope {
  PhaseTimer* t;
  int id;
  cudaEvent_t a{};
  Scope(PhaseTimer* tm, const char* name) : t(tm), id(tm ? tm->phase_id(name) : -1) {
    if (t) t->begin(id, &a);
  }
  ~Scope() {
    if (t) t->end(id, a);
  }
};

// CTAs of the binning kernels: two resident per SM, at most one per batch of chunks
static int bin_ctas(int64_t n, int num_sms) {
  const int64_t batches = std::max<int64_t>(1, ((n + 31) / 32 + kListBinChunks - 1) / kListBinChunks);
  return (int)std::max<int64_t>(1, std::min<int64_t>(batches, 2 * (int64_t)std::max(1, num_sms)));
}

cudaError_t launch_bin_active(const Launch& L, const RoundCtx& c, int round, int S, int64_t* bin_cnt,
                              PhaseTimer* timer) {
  Scope sc(timer, "bin_active");
  const int G = bin_ctas(c.n, L.num_sms);
  const int32_t* vinst = c.batched ? c.vinst : nullptr;
  const ClassRule rule{c.vtx_off, c.W, c.unit_nets, c.max_we};
  k_bin_count<<<G, kListBinThreads, 0, L.st>>>(c.next_flag, c.n, round, S, bin_cnt, rule, vinst, c.inst_voff);
  LAUNCHED("k_bin_count");
  k_bin_offsets<<<1, kListOffThreads, 0, L.st>>>(bin_cnt, S, c.sub_off, c.scal);
  LAUNCHED("k_bin_offsets");
  k_bin_scatter<<<G, kListBinThreads, 0, L.st>>>(c.next_flag, c.n, round, S, bin_cnt, c.list, vinst, c.inst_voff);
  LAUNCHED("k_bin_scatter");
  return cudaGetLastError();
}

// ============================================================= sub-round

// Last-CTA detection: every CTA calls this once at its end (after its global
// writes); the CTA that arrives last gets true and resets the counter.
__device__ bool last_cta(int64_t* counter) {
  __shared__ bool s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const ull prev = atomicAdd(reinterpret_cast<ull*>(counter), 1ull);
    s_last = prev == (ull)(gridDim.x - 1);
    if (s_last) {
      *counter = 0;
      __threadfence();
    }
  }
  __syncthreads();
  return s_last;
}

// Plan of the target-side selection, run by the last CTA of the sweep: a block
// overflows when the candidates into it weigh more than its slack;
// overflowing blocks get a segment for their candidates. The source-side
// check is armed only if, for some block, all candidates leaving it weigh at
// least its weight (otherwise no block can become empty).
__device__ void plan_to(const RoundCtx& c) {
  const int k = c.k;
  __shared__ int64_t s_run, s_nover;
  __shared__ int s_any_over, s_any_from;
  if (threadIdx.x == 0) {
    s_run = 0;
    s_nover = 0;
    s_any_over = 0;
    s_any_from = 0;
  }
  __syncthreads();
  for (int b0 = 0; b0 < k; b0 += blockDim.x) {
    const int b = b0 + threadIdx.x;
    bool over = false, maybe_from = false;
    int64_t cnt = 0;
    if (b < k) {
      // atomics of the other CTAs are visible: they fenced before arriving
      const int64_t in_w = *(volatile int64_t*)&c.in_w[b];
      const int64_t out_w = *(volatile int64_t*)&c.cand_out[b];
      over = in_w > c.lmax[b] - c.bw[b];
      maybe_from = out_w >= c.bw[b];
      cnt = over ? *(volatile int64_t*)&c.in_cnt[b] : 0;
      c.over_to[b] = over;
      c.thr_to[b] = ~0ull;
      c.thr_from[b] = ~0ull;
      c.over_from[b] = 0;
      c.acc_w[b] = 0;  // source-side sums of this sub-round start from zero
      c.acc_cnt[b] = 0;
    }
    int64_t total;
    const int64_t off = block_scan_excl_i64(cnt, &total) + s_run;
    if (b < k) {
      c.seg_off[b] = off;
      c.cursor[b] = off;
    }
    int64_t novers;
    const int64_t oi = block_scan_excl_i64(over ? 1 : 0, &novers) + s_nover;
    if (over) c.over_ids[oi] = b;
    if (over) s_any_over = 1;
    if (maybe_from) s_any_from = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
      s_run += total;
      s_nover += novers;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    c.scal[kOverCount] = s_nover;
    c.scal[kAnyOverTo] = s_any_over;
    c.scal[kAnyOverFrom] = s_any_from;
    c.scal[kDeltaSub] = 0;
    c.scal[kDeltaRb] = 0;
    c.scal[kRevCount] = 0;
  }
}

// Places the candidates of overflowing target blocks into per-block segments.
// One instance (k <= kBinSmemBlocks): a CTA counts its candidates per block in
// shared memory and reserves each block's range with one global atomic, so the
// per-block cursors see one atomic per CTA instead of one per warp. Batches
// (many blocks) use warp-aggregated atomics.
#ifndef LPGPU_BIN_THREADS
#define LPGPU_BIN_THREADS 512
#endif
#ifndef LPGPU_BIN_PER
#define LPGPU_BIN_PER 4
#endif
constexpr int kBinThreads = LPGPU_BIN_THREADS;
constexpr int kBinPer = LPGPU_BIN_PER;  // list positions per thread
constexpr int kBinSmemBlocks = 2048;

__global__ void __launch_bounds__(kBinThreads) k_bin_moves(RoundCtx c, int sub) {
  if (c.scal[kAnyOverTo] == 0) return;
  const int64_t beg = c.sub_off[sub], end = c.sub_off[sub + 1];
  const bool cta = !c.batched && c.k <= kBinSmemBlocks;
  __shared__ unsigned s_cnt[kBinSmemBlocks];
  __shared__ unsigned long long s_base[kBinSmemBlocks];
  const int lane = lane_id();
  if (cta) {
    const int k = c.k;
    for (int64_t r0 = beg + (int64_t)blockIdx.x * kBinThreads * kBinPer; r0 < end;
         r0 += (int64_t)gridDim.x * kBinThreads * kBinPer) {
      for (int b = threadIdx.x; b < k; b += blockDim.x) s_cnt[b] = 0;
      __syncthreads();
      int grp[kBinPer];
      unsigned rank[kBinPer];
      uint64_t key[kBinPer];
      int w[kBinPer];
      int4 rv[kBinPer];
#pragma unroll
      for (int q = 0; q < kBinPer; ++q) {
        const int64_t pos = r0 + q * kBinThreads + threadIdx.x;
        rv[q] = pos < end ? c.rec[pos] : make_int4(-1, 0, 0, 0);
      }
#pragma unroll
      for (int q = 0; q < kBinPer; ++q) {
        grp[q] = -1;
        if (rv[q].x >= 0 && c.over_to[rv[q].x]) {
          grp[q] = rv[q].x;
          key[q] = move_key(rv[q].y, rv[q].z);
          w[q] = c.w_v[rv[q].z];
          rank[q] = atomicAdd(&s_cnt[grp[q]], 1u);
        }
      }
      __syncthreads();
      for (int b = threadIdx.x; b < k; b += blockDim.x)
        if (s_cnt[b]) s_base[b] = atomicAdd(reinterpret_cast<ull*>(&c.cursor[b]), (ull)s_cnt[b]);
      __syncthreads();
#pragma unroll
      for (int q = 0; q < kBinPer; ++q)
        if (grp[q] >= 0) {
          const int64_t slot = (int64_t)s_base[grp[q]] + rank[q];
          c.seg_key[slot] = key[q];
          c.seg_w[slot] = w[q];
        }
      __syncthreads();
    }
    return;
  }
  for (int64_t base = beg + (blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane); base < end;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pos = base + lane;
    int grp = -1;
    uint64_t key = 0;
    int w = 0;
    if (pos < end) {
      const int4 r = c.rec[pos];
      if (r.x >= 0 && c.over_to[r.x]) {
        key = move_key(r.y, r.z);
        grp = r.x;
        w = c.w_v[r.z];
      }
    }
    // warp-aggregated segment allocation per group
    const unsigned active = __ballot_sync(FULLMASK, grp >= 0);
    if (grp >= 0) {
      const unsigned peers = __match_any_sync(active, grp);
      const int leader = __ffs(peers) - 1;
      int64_t slot0 = 0;
      if (lane == leader) slot0 = (int64_t)atomicAdd(reinterpret_cast<ull*>(&c.cursor[grp]), (ull)__popc(peers));
      slot0 = __shfl_sync(peers, slot0, leader);
      const int64_t slot = slot0 + __popc(peers & lanemask_lt());
      c.seg_key[slot] = key;
      c.seg_w[slot] = w;
    }
  }
}

// Gain-sorted prefix without sorting, by one CTA: radix selection (8 bits per
// pass, most significant byte first) of the first key whose inclusive
// weighted prefix exceeds `budget`; keys below it are accepted. Bytes equal in
// all keys need no pass (bitwise AND == OR). Segments of up to kSelStage keys
// are staged in shared memory once; each warp keeps a private 256-bin
// histogram (32-bit: vertex weights total at most INT32_MAX) and the whole CTA
// folds them before one warp scans the bins. Returns the threshold to every
// thread.
#ifndef LPGPU_SEL_THREADS
#define LPGPU_SEL_THREADS 1024
#endif
#ifndef LPGPU_SEL_STAGE
#define LPGPU_SEL_STAGE 8192
#endif
#ifndef LPGPU_SEL_ONEHIST
#define LPGPU_SEL_ONEHIST 4096  // segments of at most this many keys share one histogram
#endif
constexpr int kSelThreads = LPGPU_SEL_THREADS;
constexpr int kSelStage = LPGPU_SEL_STAGE;  // keys (8 B) + weights (4 B) staged in shared memory
constexpr size_t kSelSmem = (size_t)kSelStage * 12;

// One histogram pass: the weights of the keys matching `prefix` under `mask`,
// binned by the byte at `shift`, into this warp's 256 bins. Trips are
// warp-uniform; U keys per lane are loaded before any is binned. On gain
// bytes (few distinct digits) lanes with the same digit add once.
template <int U>
__device__ __forceinline__ void sel_hist(const uint64_t* __restrict__ keys, const int32_t* __restrict__ ws,
                                         int64_t cnt, uint64_t mask, uint64_t prefix, int shift,
                                         unsigned* __restrict__ h) {
  const int lane = lane_id();
  const bool agg = shift >= 32;
  for (int64_t base = threadIdx.x - lane; base < cnt; base += (int64_t)U * blockDim.x) {
    uint64_t kv[U];
    int32_t wv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + (int64_t)u * blockDim.x + lane;
      kv[u] = i < cnt ? keys[i] : ~prefix;
      wv[u] = i < cnt ? ws[i] : 0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + (int64_t)u * blockDim.x + lane;
      const bool in = i < cnt && (kv[u] & mask) == prefix;
      const unsigned dig = (unsigned)(kv[u] >> shift) & 255u;
      if (agg) {
        const unsigned act = __ballot_sync(FULLMASK, in);
        if (in) {
          const unsigned peers = __match_any_sync(act, dig);
          const unsigned sum = __reduce_add_sync(peers, (unsigned)wv[u]);
          if (lane == __ffs(peers) - 1) atomicAdd(&h[dig], sum);
        }
      } else if (in) {
        atomicAdd(&h[dig], (unsigned)wv[u]);
      }
    }
  }
}

__device__ uint64_t cta_radix_select(const uint64_t* __restrict__ gkeys, const int32_t* __restrict__ gws,
                                     int64_t cnt, int64_t budget0, unsigned char* stage = nullptr,
                                     int stage_cap = kSelStage) {
  constexpr int NW = kSelThreads / 32;
  extern __shared__ __align__(16) unsigned char sel_smem[];
  __shared__ unsigned hist[NW][256];
  __shared__ unsigned tot[256];
  __shared__ uint64_t s_and[NW], s_or[NW];
  __shared__ int64_t s_budget;
  __shared__ int s_sel;
  const int lane = lane_id(), wid = threadIdx.x >> 5;
  // segments of up to stage_cap keys are staged in `stage` (default: the
  // kernel's dynamic shared memory, kSelStage keys)
  const bool staged = cnt <= stage_cap;
  uint64_t* skeys = reinterpret_cast<uint64_t*>(stage ? stage : sel_smem);
  int32_t* sws = reinterpret_cast<int32_t*>(skeys + stage_cap);
  uint64_t ka = ~0ull, ko = 0;
#pragma unroll 4
  for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x) {
    const uint64_t key = gkeys[i];
    if (staged) {
      skeys[i] = key;
      sws[i] = gws[i];
    }
    ka &= key;
    ko |= key;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ka &= __shfl_xor_sync(FULLMASK, ka, o);
    ko |= __shfl_xor_sync(FULLMASK, ko, o);
  }
  __syncthreads();
  if (lane == 0) { s_and[wid] = ka; s_or[wid] = ko; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {  // any CTA width up to kSelThreads
      ka &= s_and[w];
      ko |= s_or[w];
    }
    s_and[0] = ka;
    s_or[0] = ko;
    s_budget = budget0;
  }
  __syncthreads();
  ka = s_and[0];
  ko = s_or[0];
  uint64_t prefix = 0, mask = 0;
  // small segments bin into one shared histogram (atomics rarely collide),
  // large ones into a private histogram per warp folded afterwards
  const bool one = cnt <= LPGPU_SEL_ONEHIST;
  const int rows = one ? 1 : NW;
  for (int byte = 7; byte >= 0; --byte) {
    const int shift = 8 * byte;
    if ((((ka ^ ko) >> shift) & 255) == 0) {  // every key has this byte
      prefix |= ka & (255ull << shift);
      mask |= 255ull << shift;
      continue;
    }
    for (int i = threadIdx.x; i < rows * 256; i += blockDim.x) (&hist[0][0])[i] = 0;
    __syncthreads();
    if (staged)
      sel_hist<1>(skeys, sws, cnt, mask, prefix, shift, hist[one ? 0 : wid]);
    else
      sel_hist<8>(gkeys, gws, cnt, mask, prefix, shift, hist[one ? 0 : wid]);
    __syncthreads();
    for (int bin = threadIdx.x; bin < 256; bin += blockDim.x) {
      unsigned t = 0;
      for (int w = 0; w < rows; ++w) t += hist[w][bin];
      tot[bin] = t;
    }
    __syncthreads();
    if (wid == 0) {
      // lane l owns bins 8l .. 8l+7: first bin whose running sum exceeds the budget
      int64_t h[8], sum = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        h[j] = tot[8 * lane + j];
        sum += h[j];
      }
      int64_t run = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(FULLMASK, run, o);
        if (lane >= o) run += y;
      }
      const int64_t budget = s_budget;
      int sel = -1;
      int64_t below = 0, acc = run - sum;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (sel < 0 && acc + h[j] > budget) { sel = 8 * lane + j; below = acc; }
        acc += h[j];
      }
      const unsigned found = __ballot_sync(FULLMASK, sel >= 0);
      const int first = found ? __ffs(found) - 1 : 31;
      if (lane == first) {
        s_sel = found ? sel : 255;
        s_budget = budget - (found ? below : acc);
      }
    }
    __syncthreads();
    prefix |= (uint64_t)s_sel << shift;
    mask |= 255ull << shift;
  }
  return prefix;
}

// Warp-wide radix selection over the cnt keys at `keys` (written earlier in
// this kernel, so read through plain loads): the same threshold as
// cta_radix_select (the first key whose weighted prefix exceeds `budget`, all
// ones when the total stays within it), with only warp barriers between the
// byte passes. `hist`: 256 words of this warp's shared scratch.
__device__ uint64_t warp_radix_select(const uint64_t* keys, const int32_t* ws, int cnt, int64_t budget,
                                      unsigned* hist) {
  const int lane = lane_id();
  uint64_t ka = ~0ull, ko = 0;
  for (int i = lane; i < cnt; i += 32) {
    const uint64_t key = keys[i];
    ka &= key;
    ko |= key;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ka &= __shfl_xor_sync(FULLMASK, ka, o);
    ko |= __shfl_xor_sync(FULLMASK, ko, o);
  }
  uint64_t prefix = 0, mask = 0;
  for (int byte = 7; byte >= 0; --byte) {
    const int shift = 8 * byte;
    if ((((ka ^ ko) >> shift) & 255) == 0) {  // every key has this byte
      prefix |= ka & (255ull << shift);
      mask |= 255ull << shift;
      continue;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) hist[32 * j + lane] = 0;
    __syncwarp();
    for (int i = lane; i < cnt; i += 32) {
      const uint64_t key = keys[i];
      if ((key & mask) == prefix) atomicAdd(&hist[(unsigned)(key >> shift) & 255u], (unsigned)ws[i]);
    }
    __syncwarp();
    // lane l owns bins 8l .. 8l+7: first bin whose running sum exceeds the budget
    int64_t h[8], sum = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      h[j] = hist[8 * lane + j];
      sum += h[j];
    }
    int64_t run = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(FULLMASK, run, o);
      if (lane >= o) run += y;
    }
    int sel = -1;
    int64_t below = 0, acc = run - sum;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (sel < 0 && acc + h[j] > budget) {
        sel = 8 * lane + j;
        below = acc;
      }
      acc += h[j];
    }
    const unsigned found = __ballot_sync(FULLMASK, sel >= 0);
    const int first = found ? __ffs(found) - 1 : 31;
    const int pick = __shfl_sync(FULLMASK, found ? sel : 255, first);
    budget = __shfl_sync(FULLMASK, budget - (found ? below : acc), first);
    prefix |= (uint64_t)pick << shift;
    mask |= 255ull << shift;
    __syncwarp();  // the histogram is cleared by the next pass
  }
  return prefix;
}

#ifndef LPGPU_SEL_WARP
#define LPGPU_SEL_WARP 512  // segments of at most this many keys are selected by one warp
#endif
constexpr int kSelWarpKeys = LPGPU_SEL_WARP;
static_assert(kSelSmem >= (size_t)(kSelThreads / 32) * 256 * sizeof(unsigned),
              "every warp's selection histogram fits the staging area");

// Target-side selection. With more overflowing blocks than CTAs, warps
// first stride over the blocks with small segments (histograms in the staging
// area, not in use then), which CTAs would otherwise take one after another;
// CTAs take the others (all blocks when each gets a CTA of its own).
__device__ void from_side(const RoundCtx& c, int sub);

// Its last CTA then runs the source-side selection (from_side).
__global__ void __launch_bounds__(kSelThreads) k_select(RoundCtx c, int sub) {
  extern __shared__ __align__(16) unsigned char sel_smem[];
  const int64_t nover = c.scal[kOverCount];
  const int64_t warp_keys = nover > gridDim.x ? kSelWarpKeys : -1;
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned* whist = reinterpret_cast<unsigned*>(sel_smem) + 256 * wid;
  for (int64_t i = (int64_t)blockIdx.x * nw + wid; warp_keys >= 0 && i < nover; i += (int64_t)gridDim.x * nw) {
    const int b = c.over_ids[i];
    const int64_t cnt = c.in_cnt[b];
    if (cnt > warp_keys) continue;
    const int64_t off = c.seg_off[b];
    const uint64_t thr = warp_radix_select(c.seg_key + off, c.seg_w + off, (int)cnt, c.lmax[b] - c.bw[b], whist);
    if (lane_id() == 0) c.thr_to[b] = thr;
  }
  __syncthreads();
  for (int64_t i = blockIdx.x; i < nover; i += gridDim.x) {
    const int b = c.over_ids[i];
    if (c.in_cnt[b] <= warp_keys) continue;  // the same for the whole CTA
    const int64_t off = c.seg_off[b];
    const uint64_t thr = cta_radix_select(c.seg_key + off, c.seg_w + off, c.in_cnt[b],
                                          c.lmax[b] - c.bw[b]);
    if (threadIdx.x == 0) c.thr_to[b] = thr;
    __syncthreads();
  }
  if (last_cta(&c.scal[kDone])) from_side(c, sub);
}

// Source-side selection (changeNodePart's from_weight_after > 0,
// partitioned_hypergraph.h:551), only when armed by the plan: one CTA sums
// the target-accepted weight leaving each block; blocks that would become
// empty get their accepted moves ordered the same way and keep the longest
// prefix that leaves weight >= 1.
__device__ void from_side(const RoundCtx& c, int sub) {
  if (c.scal[kAnyOverFrom] == 0) return;
  const int k = c.k;
  __shared__ int s_any;
  __shared__ int64_t s_run;
  if (threadIdx.x == 0) {
    s_any = 0;
    s_run = 0;
  }
  __syncthreads();
  const int64_t beg = c.sub_off[sub], end = c.sub_off[sub + 1];
  // target-accepted weight and count per source block (acc_w / acc_cnt are cleared by the plan)
  for (int64_t pos = beg + threadIdx.x; pos < end; pos += blockDim.x) {
    const int4 r = c.rec[pos];
    if (r.x < 0) continue;
    if (move_key(r.y, r.z) < c.thr_to[r.x]) {
      atomicAdd(reinterpret_cast<ull*>(&c.acc_w[r.w]), (ull)(int64_t)c.w_v[r.z]);
      atomicAdd(reinterpret_cast<ull*>(&c.acc_cnt[r.w]), 1ull);
    }
  }
  __syncthreads();
  for (int b0 = 0; b0 < k; b0 += blockDim.x) {
    const int b = b0 + threadIdx.x;
    bool over = false;
    int64_t n = 0;
    if (b < k) {
      n = c.acc_cnt[b];
      over = n > 0 && c.bw[b] - c.acc_w[b] < 1;
    }
    int64_t total;
    const int64_t off = block_scan_excl_i64(over ? n : 0, &total) + s_run;
    if (b < k) {
      c.over_from[b] = over;
      c.seg_off[b] = off;
      c.cursor[b] = off;
    }
    if (over) s_any = 1;
    __syncthreads();
    if (threadIdx.x == 0) s_run += total;
    __syncthreads();
  }
  if (!s_any) return;
  for (int64_t pos = beg + threadIdx.x; pos < end; pos += blockDim.x) {
    const int4 r = c.rec[pos];
    if (r.x < 0) continue;
    const uint64_t key = move_key(r.y, r.z);
    const int f = r.w;
    if (key < c.thr_to[r.x] && c.over_from[f]) {
      const ull slot = atomicAdd(reinterpret_cast<ull*>(&c.cursor[f]), 1ull);
      c.seg_key[slot] = key;
      c.seg_w[slot] = c.w_v[r.z];
    }
  }
  __syncthreads();
  // several blocks: small segments one warp each, all at once (histograms in
  // the staging area); the others the whole CTA, one after another
  int nof = 0;
  for (int b0 = 0; b0 < k; b0 += blockDim.x)
    nof += __syncthreads_count(b0 + (int)threadIdx.x < k && c.over_from[b0 + threadIdx.x]);
  const int64_t warp_keys = nof > 1 ? kSelWarpKeys : -1;
  extern __shared__ __align__(16) unsigned char sel_smem[];
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned* whist = reinterpret_cast<unsigned*>(sel_smem) + 256 * wid;
  for (int b = wid; b < k; b += nw) {
    if (!c.over_from[b] || c.acc_cnt[b] > warp_keys) continue;
    const int64_t off = c.seg_off[b];
    const uint64_t thr = warp_radix_select(c.seg_key + off, c.seg_w + off, (int)c.acc_cnt[b], c.bw[b] - 1, whist);
    if (lane_id() == 0) c.thr_from[b] = thr;
  }
  __syncthreads();
  for (int b = 0; b < k; ++b) {
    if (!c.over_from[b] || c.acc_cnt[b] <= warp_keys) continue;  // uniform across the CTA
    const int64_t off = c.seg_off[b];
    const uint64_t thr = cta_radix_select(c.seg_key + off, c.seg_w + off, c.acc_cnt[b], c.bw[b] - 1);
    if (threadIdx.x == 0) c.thr_from[b] = thr;
    __syncthreads();
  }
}

// Books the sub-round's delta into the round statistics and clears the
// sweep accumulators for the next sub-round (last CTA of the last kernel).
__device__ void close_subround(const RoundCtx& c, int round) {
  if (threadIdx.x == 0) {
    c.stats[(int64_t)round * kStats + kStDelta] += c.scal[kDeltaSub] + c.scal[kDeltaRb];
  }
  for (int b = threadIdx.x; b < c.k; b += blockDim.x) {
    c.in_w[b] = 0;
    c.in_cnt[b] = 0;
    c.cand_out[b] = 0;
  }
  if (c.batched)
    for (int i = threadIdx.x; i < c.num_inst; i += blockDim.x) c.inst_delta[i] = 0;
}

// Activation stamp of one incident net of a kept move (see k_expand_nets).
__device__ __forceinline__ void activate_incidence(const RoundCtx& c, int64_t e, int epoch) {
  if (c.net_off[e + 1] - c.net_off[e] <= c.act_threshold) c.net_epoch[e] = epoch;
}


// ---- CTA-flat incidence walks
//
// A CTA collects the selected vertices of a range of list positions in shared
// memory (first incidence and degree), scans the degrees, and then spreads
// every incidence of every collected vertex over all its threads: thread t
// takes incidences t, t + blockDim, ... and finds its vertex by binary search
// in the scanned degrees. Hub vertices are split across the whole CTA, and the
// gathers and atomics of different vertices are in flight together.
#ifndef LPGPU_FLAT_THREADS
#define LPGPU_FLAT_THREADS 512
#endif
constexpr int kFlatThreads = LPGPU_FLAT_THREADS;
constexpr int kFlatItems = 1024;  // list positions (and so at most this many vertices) per CTA pass
static_assert(kFlatItems % kFlatThreads == 0, "whole items per thread");

struct FlatSmem {
  int64_t o0[kFlatItems];    // first incidence
  int pre[kFlatItems + 1];   // degrees, then their exclusive prefix sums
  int ft[kFlatItems];        // local from | local to << 16
  int att[kFlatItems];       // per-vertex sums (attributed delta, or the reverse move's gain)
  int inst[kFlatItems];      // instance (batched)
  int pos[kFlatItems];       // list position
  int wsum[kFlatThreads / 32];
  int n;
};

// Warp-aggregated append to a shared counter; returns each selected lane's slot.
__device__ __forceinline__ int flat_append_to(int* counter, bool sel) {
  const unsigned m = __ballot_sync(FULLMASK, sel);
  if (!m) return -1;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane_id() == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(FULLMASK, base, leader);
  return sel ? base + __popc(m & lanemask_lt()) : -1;
}

// Appends the lanes with `sel` to the CTA's item list; returns each lane's slot.
__device__ __forceinline__ int flat_append(FlatSmem& f, bool sel) { return flat_append_to(&f.n, sel); }

// In-place exclusive scan of f.pre[0 .. n) (n <= kFlatItems); f.pre[n] = total.
__device__ __forceinline__ int flat_scan(FlatSmem& f, int n) {
  constexpr int PER = kFlatItems / kFlatThreads;
  const int t = threadIdx.x, lane = lane_id(), wid = t >> 5;
  int v[PER], sum = 0;
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int i = t * PER + q;
    v[q] = i < n ? f.pre[i] : 0;
    sum += v[q];
  }
  int incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(FULLMASK, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) f.wsum[wid] = incl;
  __syncthreads();
  int wbase = 0, total = 0;
#pragma unroll
  for (int w = 0; w < kFlatThreads / 32; ++w) {
    const int x = f.wsum[w];
    if (w < wid) wbase += x;
    total += x;
  }
  int run = wbase + incl - sum;
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int i = t * PER + q;
    if (i < n) f.pre[i] = run;
    run += v[q];
  }
  if (t == 0) f.pre[n] = total;
  __syncthreads();
  return total;
}

// Vertex of flat incidence index x: the largest i with pre[i] <= x.
__device__ __forceinline__ int flat_find(const FlatSmem& f, int n, int x) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (f.pre[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Commit of Q incidences (e[q], from f[q], to t[q]; h[q]: present): all 2Q Φ
// atomics are issued before any result is used, then per incidence the
// decrement of Φ(e, f) and increment of Φ(e, t) toggle Λ when Φ(e, f) reaches
// 0 or Φ(e, t) leaves 0, and Λ1 when either passes through 1. The attributed
// delta (km1Delta, hypergraph_common.h:133-140) is -w(e) when Φ(e, f) reaches
// 0 and +w(e) when Φ(e, t) reaches 1; a[q] is each incidence's part.
template <int Q>
__device__ __forceinline__ void commit_group(const RoundCtx& c, const bool (&h)[Q], const int64_t (&e)[Q],
                                             const int (&f)[Q], const int (&t)[Q], int (&a)[Q], int& toggles) {
  const int W = c.W;
  const int64_t k = c.kmax;
  int of[Q], ot[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    of[q] = ot[q] = 0;
    if (h[q]) {
      of[q] = phi_add(c, e[q] * k + f[q], -1);
      ot[q] = phi_add(c, e[q] * k + t[q], 1);
    }
  }
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    a[q] = 0;
    if (!h[q]) continue;
    const int we = c.unit_nets ? 1 : c.w_e[e[q]];
    uint32_t* rec = c.conn + e[q] * 2 * W;
    const uint32_t fb = 1u << (f[q] & 31), tb = 1u << (t[q] & 31);
    if (of[q] == 1) { atomicXor(&rec[f[q] >> 5], fb); a[q] -= we; ++toggles; }
    if (of[q] == 1 || of[q] == 2) atomicXor(&rec[W + (f[q] >> 5)], fb);
    if (ot[q] == 0) { atomicXor(&rec[t[q] >> 5], tb); a[q] += we; ++toggles; }
    if (ot[q] == 0 || ot[q] == 1) atomicXor(&rec[W + (t[q] >> 5)], tb);
  }
}

// Incidences a thread of the CTA-flat commit handles per step.
#ifndef LPGPU_COMMIT_GROUP
#define LPGPU_COMMIT_GROUP 2  // 4 and 8 measured slower on rownet
#endif

// Moves every incidence of the CTA's collected vertices from their `from` to
// their `to` block (flat over the CTA). Returns this thread's summed delta;
// per-vertex sums go to f.att when `per_item`; *toggles counts this thread's
// Λ bit changes.
__device__ __forceinline__ int64_t flat_commit(const RoundCtx& c, FlatSmem& f, int n, int total, bool per_item,
                                               int64_t* toggles = nullptr) {
  constexpr int Q = LPGPU_COMMIT_GROUP;
  int64_t att = 0;
  int tg = 0;
  for (int x0 = threadIdx.x; x0 < total; x0 += Q * kFlatThreads) {
    bool h[Q];
    int64_t e[Q];
    int fr[Q], to[Q], it[Q], a[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int x = x0 + q * kFlatThreads;
      h[q] = x < total;
      it[q] = h[q] ? flat_find(f, n, x) : 0;
      e[q] = h[q] ? c.inets[f.o0[it[q]] + (x - f.pre[it[q]])] : 0;
      const int ft = h[q] ? f.ft[it[q]] : 0;
      fr[q] = ft & 0xffff;
      to[q] = ft >> 16;
    }
    commit_group<Q>(c, h, e, fr, to, a, tg);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      att += a[q];
      if (per_item && a[q]) atomicAdd(&f.att[it[q]], a[q]);
    }
  }
  if (toggles) *toggles += tg;
  return att;
}

// Commit of the accepted moves (changeNodePart, h:539-563, without the
// per-move weight check: the selection already guarantees both bounds).
// Marks status[pos] = 1 for committed moves. CTA-flat over ranges of
// kFlatItems list positions. With `last`, the moves are final and the
// sub-round is closed; kept moves are activated at the end of the round
// (k_activate_round).
__global__ void __launch_bounds__(kFlatThreads) k_commit(RoundCtx c, int round, int sub, int last) {
  extern __shared__ ull s_dw[];
  __shared__ FlatSmem f;
  // block-weight deltas: shared memory for one instance, global atomics for a batch
  const bool batched = c.batched != 0;
  ull* dw = batched ? reinterpret_cast<ull*>(c.bw) : s_dw;
  const int kdw = batched ? 0 : c.k;
  for (int b = threadIdx.x; b < kdw; b += blockDim.x) s_dw[b] = 0;
  const int64_t beg = c.sub_off[sub], end = c.sub_off[sub + 1];
  constexpr int PER = kFlatItems / kFlatThreads;
  int64_t att = 0, moved = 0, moved_pins = 0, toggles = 0;
  for (int64_t r0 = beg + (int64_t)blockIdx.x * kFlatItems; r0 < end; r0 += (int64_t)gridDim.x * kFlatItems) {
    if (threadIdx.x == 0) f.n = 0;
    __syncthreads();
    int4 rv[PER];
    bool acc[PER];
    int64_t o0[PER], o1[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int64_t pos = r0 + q * kFlatThreads + threadIdx.x;
      rv[q] = pos < end ? c.rec[pos] : make_int4(-1, 0, 0, 0);
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      acc[q] = false;
      o0[q] = o1[q] = 0;
      if (rv[q].x >= 0) {
        const uint64_t key = move_key(rv[q].y, rv[q].z);
        acc[q] = key < c.thr_to[rv[q].x] && key < c.thr_from[rv[q].w];
        o0[q] = c.vtx_off[rv[q].z];
        o1[q] = c.vtx_off[rv[q].z + 1];
      }
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int64_t pos = r0 + q * kFlatThreads + threadIdx.x;
      if (pos < end) c.status[pos] = acc[q] ? 1 : 0;
      const int slot = flat_append(f, acc[q]);
      if (acc[q]) {
        const int v = rv[q].z;
        int bo = 0;
        if (batched) {
          const int i = c.vinst[v];
          bo = c.inst_boff[i];
          f.inst[slot] = i;
          f.att[slot] = 0;
        }
        f.o0[slot] = o0[q];
        f.pre[slot] = (int)(o1[q] - o0[q]);
        f.ft[slot] = (rv[q].w - bo) | ((rv[q].x - bo) << 16);
        c.part[v] = rv[q].x;
        const int64_t wv = c.w_v[v];
        atomicAdd(&dw[rv[q].x], (ull)wv);
        atomicAdd(&dw[rv[q].w], (ull)(-wv));
        ++moved;
      }
    }
    __syncthreads();
    const int n = f.n;
    const int total = flat_scan(f, n);
    if (threadIdx.x == 0) moved_pins += total;
    att += flat_commit(c, f, n, total, batched, &toggles);
    __syncthreads();
    if (batched)
      for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (f.att[i]) atomicAdd(reinterpret_cast<ull*>(&c.inst_delta[f.inst[i]]), (ull)(int64_t)f.att[i]);
  }
  att = block_sum_i64(att);
  moved = block_sum_i64(moved);
  toggles = block_sum_i64(toggles);
  if (threadIdx.x == 0) {
    int64_t* st = c.stats + (int64_t)round * kStats;
    atomicAdd(reinterpret_cast<ull*>(&c.scal[kDeltaSub]), (ull)att);
    atomicAdd(reinterpret_cast<ull*>(&st[kStMoved]), (ull)moved);
    if (moved_pins) atomicAdd(reinterpret_cast<ull*>(&st[kStMovedPins]), (ull)moved_pins);
    if (toggles) atomicAdd(reinterpret_cast<ull*>(&st[kStToggles]), (ull)toggles);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kdw; b += blockDim.x)
    if (s_dw[b]) atomicAdd(reinterpret_cast<ull*>(&c.bw[b]), s_dw[b]);
  if (last && last_cta(&c.scal[kDone])) close_subround(c, round);
}

// Hindsight check, evaluated for all committed moves on the post-commit state
// before any is undone: a move from f to t is marked for revert (status 2)
// when moving the vertex back to f now strictly improves km1. This is the
// deterministic counterpart of the realised-gain check of moveVertex
// (label_propagation_refiner.h:100-137). CTA-flat over ranges of list
// positions; the marked positions are appended to the revert list with one
// global atomic per range.
__global__ void __launch_bounds__(kFlatThreads) k_revert_eval(RoundCtx c, int sub) {
  __shared__ FlatSmem f;
  __shared__ int s_rev, s_base;
  const bool batched = c.batched != 0;
  const int W = c.W;
  const int lane = lane_id();
  const int64_t beg = c.sub_off[sub], end = c.sub_off[sub + 1];
  constexpr int PER = kFlatItems / kFlatThreads;
  for (int64_t r0 = beg + (int64_t)blockIdx.x * kFlatItems; r0 < end; r0 += (int64_t)gridDim.x * kFlatItems) {
    if (threadIdx.x == 0) {
      f.n = 0;
      s_rev = 0;
    }
    __syncthreads();
    uint8_t st[PER];
    int4 rv[PER];
    int64_t o0[PER], o1[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int64_t pos = r0 + q * kFlatThreads + threadIdx.x;
      st[q] = pos < end ? c.status[pos] : 0;
      rv[q] = pos < end ? c.rec[pos] : make_int4(0, 0, 0, 0);
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      o0[q] = o1[q] = 0;
      if (st[q] == 1) {
        o0[q] = c.vtx_off[rv[q].z];
        o1[q] = c.vtx_off[rv[q].z + 1];
      }
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int slot = flat_append(f, st[q] == 1);
      if (slot >= 0) {
        const int bo = batched ? c.inst_boff[c.vinst[rv[q].z]] : 0;
        f.o0[slot] = o0[q];
        f.pre[slot] = (int)(o1[q] - o0[q]);
        f.ft[slot] = (rv[q].w - bo) | ((rv[q].x - bo) << 16);
        f.att[slot] = 0;
        f.pos[slot] = (int)(r0 + q * kFlatThreads + threadIdx.x);
      }
    }
    __syncthreads();
    const int n = f.n;
    const int total = flat_scan(f, n);
    // gain of moving back: + w(e) if Φ(e, t) > 1, - w(e) if f in Λ(e)
    for (int x0 = threadIdx.x; x0 < total; x0 += 2 * kFlatThreads) {
      const int x1 = x0 + kFlatThreads;
      const bool h1 = x1 < total;
      const int i0 = flat_find(f, n, x0), i1 = h1 ? flat_find(f, n, x1) : i0;
      const int64_t e0 = c.inets[f.o0[i0] + (x0 - f.pre[i0])];
      const int64_t e1 = h1 ? c.inets[f.o0[i1] + (x1 - f.pre[i1])] : 0;
      const int ft0 = f.ft[i0], ft1 = f.ft[i1];
      const int fa = ft0 & 0xffff, ta = ft0 >> 16, fb = ft1 & 0xffff, tb = ft1 >> 16;
      const uint32_t* ra = c.conn + e0 * 2 * W;
      const uint32_t* rb = c.conn + e1 * 2 * W;
      const uint32_t l1a = ra[W + (ta >> 5)], lfa = ra[fa >> 5];
      uint32_t l1b = 0, lfb = 0;
      if (h1) {
        l1b = rb[W + (tb >> 5)];
        lfb = rb[fb >> 5];
      }
      const int wa = c.unit_nets ? 1 : c.w_e[e0];
      const int wb = h1 ? (c.unit_nets ? 1 : c.w_e[e1]) : 0;
      const int xa = (((l1a >> (ta & 31)) & 1u) ? 0 : wa) - (((lfa >> (fa & 31)) & 1u) ? wa : 0);
      const int xb = h1 ? (((l1b >> (tb & 31)) & 1u) ? 0 : wb) - (((lfb >> (fb & 31)) & 1u) ? wb : 0) : 0;
      if (xa) atomicAdd(&f.att[i0], xa);
      if (xb) atomicAdd(&f.att[i1], xb);
    }
    __syncthreads();
    // mark, collect locally (in f.pre, no longer needed), then one global append
    for (int base = threadIdx.x - lane; base < n; base += blockDim.x) {
      const int i = base + lane;
      const bool rev = i < n && f.att[i] < 0;
      const int slot = flat_append_to(&s_rev, rev);
      if (rev) {
        c.status[f.pos[i]] = 2;
        f.pre[slot] = f.pos[i];
      }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_rev)
      s_base = (int)atomicAdd(reinterpret_cast<ull*>(&c.scal[kRevCount]), (ull)s_rev);
    __syncthreads();
    for (int i = threadIdx.x; i < s_rev; i += blockDim.x) c.revl[s_base + i] = f.pre[i];
    __syncthreads();
  }
}

// Collects undo items: vertex v moved from global block `from` to `to`; the
// item moves it back (its Φ / Λ / Λ1 from `to` to `from`), and part and the
// CTA's block-weight deltas are restored right away.
__device__ __forceinline__ void flat_undo_item(const RoundCtx& c, FlatSmem& f, int slot, int v, int to, int from,
                                               int64_t o0, int64_t o1, ull* dw, bool per_item) {
  int bo = 0;
  if (c.batched) {
    const int i = c.vinst[v];
    bo = c.inst_boff[i];
    f.inst[slot] = i;
  }
  f.att[slot] = 0;
  f.o0[slot] = o0;
  f.pre[slot] = (int)(o1 - o0);
  f.ft[slot] = (to - bo) | ((from - bo) << 16);
  (void)per_item;
  c.part[v] = from;
  const int64_t wv = c.w_v[v];
  atomicAdd(&dw[from], (ull)wv);
  atomicAdd(&dw[to], (ull)(-wv));
}

// Books undone moves into the sub-round's delta and statistics and flushes
// the CTA's block-weight deltas.
__device__ __forceinline__ void undo_epilogue(const RoundCtx& c, int round, int64_t att, int64_t undone,
                                              int slot, ull* s_dw, int kdw) {
  if (!__syncthreads_or(undone != 0)) return;  // this CTA undid nothing: no sums, no weight deltas
  att = block_sum_i64(att);
  undone = block_sum_i64(undone);
  if (threadIdx.x == 0 && undone) {
    atomicAdd(reinterpret_cast<ull*>(&c.scal[slot]), (ull)att);
    int64_t* stt = c.stats + (int64_t)round * kStats;
    atomicAdd(reinterpret_cast<ull*>(&stt[kStMoved]), (ull)(-undone));
    atomicAdd(reinterpret_cast<ull*>(&stt[kStReverted]), (ull)undone);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kdw; b += blockDim.x)
    if (s_dw[b]) atomicAdd(reinterpret_cast<ull*>(&c.bw[b]), s_dw[b]);
}

// Undo of the moves the hindsight check marked (status 2), from the compact
// list k_revert_eval wrote, spread over all CTAs (each takes a short range and
// walks its moves' incidences flat). With `last` the sub-round is closed.
__device__ void rollback_ranges(const RoundCtx& c, int round, int sub, bool roll, FlatSmem& f, ull* s_dw,
                                int64_t first, int64_t stride);

// With `roll_tail` (one instance), the last CTA also performs the sub-round's
// rollback when its delta is positive (rare), so no rollback kernel runs.
__global__ void __launch_bounds__(kFlatThreads) k_undo_reverts(RoundCtx c, int round, int sub, int last,
                                                                int roll_tail) {
  extern __shared__ ull s_dw[];
  __shared__ FlatSmem f;
  const bool batched = c.batched != 0;
  ull* dw = batched ? reinterpret_cast<ull*>(c.bw) : s_dw;
  const int kdw = batched ? 0 : c.k;
  for (int b = threadIdx.x; b < kdw; b += blockDim.x) s_dw[b] = 0;
  constexpr int PER = kFlatItems / kFlatThreads;
  const int64_t cnt = c.scal[kRevCount];
  const int64_t want = (cnt + gridDim.x - 1) / gridDim.x;
  const int per = want < 32 ? 32 : (want > kFlatItems ? kFlatItems : (int)want);
  int64_t att = 0, undone = 0;
  for (int64_t r0 = (int64_t)blockIdx.x * per; r0 < cnt; r0 += (int64_t)gridDim.x * per) {
    if (threadIdx.x == 0) f.n = 0;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int off = q * kFlatThreads + threadIdx.x;
      const bool sel = off < per && r0 + off < cnt;
      int4 rv = make_int4(0, 0, 0, 0);
      int64_t o0 = 0, o1 = 0;
      if (sel) {
        rv = c.rec[c.revl[r0 + off]];
        o0 = c.vtx_off[rv.z];
        o1 = c.vtx_off[rv.z + 1];
      }
      const int slot = flat_append(f, sel);
      if (sel) {
        flat_undo_item(c, f, slot, rv.z, rv.x, rv.w, o0, o1, dw, batched);
        ++undone;
      }
    }
    __syncthreads();
    const int n = f.n;
    const int total = flat_scan(f, n);
    att += flat_commit(c, f, n, total, batched);
    __syncthreads();
    if (batched)
      for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (f.att[i]) atomicAdd(reinterpret_cast<ull*>(&c.inst_delta[f.inst[i]]), (ull)(int64_t)f.att[i]);
  }
  undo_epilogue(c, round, att, undone, kDeltaSub, s_dw, kdw);
  if ((last || roll_tail) && last_cta(&c.scal[kDone])) {
    if (roll_tail) {
      const bool roll = *(volatile int64_t*)&c.scal[kDeltaSub] > 0;
      __syncthreads();
      if (roll) rollback_ranges(c, round, sub, true, f, s_dw, 0, 1);  // otherwise nothing to undo or book
    }
    close_subround(c, round);
  }
}

// Rollback: when the sub-round's delta is positive, undo of every move still
// marked 1 (status 3); decided per instance when batched (kDeltaSub and
// inst_delta are not written here). Closes the sub-round.
// Rollback of the sub-round's moves still marked 1 (status 3) over the list
// ranges first, first + stride, ... (CTA-flat); returns nothing, books into
// kDeltaRb and the statistics.
__device__ void rollback_ranges(const RoundCtx& c, int round, int sub, bool roll, FlatSmem& f, ull* s_dw,
                                int64_t first, int64_t stride) {
  const bool batched = c.batched != 0;
  ull* dw = batched ? reinterpret_cast<ull*>(c.bw) : s_dw;
  const int kdw = batched ? 0 : c.k;
  for (int b = threadIdx.x; b < kdw; b += blockDim.x) s_dw[b] = 0;
  constexpr int PER = kFlatItems / kFlatThreads;
  const int64_t beg = c.sub_off[sub], end = roll ? c.sub_off[sub + 1] : beg;
  int64_t att = 0, undone = 0;
  for (int64_t r0 = beg + first * kFlatItems; r0 < end; r0 += stride * kFlatItems) {
    if (threadIdx.x == 0) f.n = 0;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int64_t pos = r0 + q * kFlatThreads + threadIdx.x;
      bool sel = pos < end && c.status[pos] == 1;
      int4 rv = make_int4(0, 0, 0, 0);
      int64_t o0 = 0, o1 = 0;
      if (sel) {
        rv = c.rec[pos];
        if (batched) sel = c.inst_delta[c.vinst[rv.z]] > 0;  // rollback is decided per instance
      }
      if (sel) {
        o0 = c.vtx_off[rv.z];
        o1 = c.vtx_off[rv.z + 1];
      }
      const int slot = flat_append(f, sel);
      if (sel) {
        flat_undo_item(c, f, slot, rv.z, rv.x, rv.w, o0, o1, dw, false);
        c.status[pos] = 3;
        ++undone;
      }
    }
    __syncthreads();
    const int n = f.n;
    const int total = flat_scan(f, n);
    att += flat_commit(c, f, n, total, false);
    __syncthreads();
  }
  undo_epilogue(c, round, att, undone, kDeltaRb, s_dw, kdw);
}

__global__ void __launch_bounds__(kFlatThreads) k_rollback(RoundCtx c, int round, int sub) {
  extern __shared__ ull s_dw[];
  __shared__ FlatSmem f;
  rollback_ranges(c, round, sub, c.batched || c.scal[kDeltaSub] > 0, f, s_dw, blockIdx.x, gridDim.x);
  if (last_cta(&c.scal[kDone])) close_subround(c, round);
}

// Activation of the round's kept moves (status 1): the moved vertex and the
// pins of its incident nets with |e| <= activation threshold become active in
// the next round (moveVertex, label_propagation_refiner.h:112-128). Nets are
// stamped with the round's epoch and expanded by k_expand_nets.
#ifndef LPGPU_ACT_THREADS
#define LPGPU_ACT_THREADS 256
#endif
constexpr int kActThreads = LPGPU_ACT_THREADS;  // activation and expansion CTAs

__global__ void __launch_bounds__(kActThreads) k_activate_round(RoundCtx c, int S) {
  __shared__ unsigned char s_own[kActThreads];
  const int lane = lane_id();
  unsigned char* own = s_own + (threadIdx.x & ~31);
  const int epoch = (int)c.scal[kEpoch];
  const int64_t end = c.sub_off[S];
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; base < end;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pos = base + lane;
    const bool keep = pos < end && c.status[pos] == 1;
    int64_t v = 0, o0 = 0;
    int deg = 0;
    if (keep) {
      v = c.list[pos];
      o0 = c.vtx_off[v];
      deg = (int)(c.vtx_off[v + 1] - o0);
      c.next_flag[v] = 1;
    }
    packed_incidences(keep, o0, deg, own, [&](bool has, int, int64_t j) -> int {
      if (has) activate_incidence(c, c.inets[j], epoch);
      return 0;
    });
  }
}


// End of a round: the pins of every net stamped with the round's epoch
// become active for the next round. A warp takes 32 nets and walks the pins
// of the stamped ones in packed 32-pin groups.
__global__ void __launch_bounds__(kActThreads) k_expand_nets(RoundCtx c) {
  __shared__ unsigned char s_own[kActThreads];
  const int epoch = (int)c.scal[kEpoch];
  const int lane = lane_id();
  unsigned char* own = s_own + (threadIdx.x & ~31);
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; base < c.m;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = base + lane;
    const bool hit = e < c.m && c.net_epoch[e] == epoch;
    int64_t o0 = 0;
    int deg = 0;
    if (hit) {
      o0 = c.net_off[e];
      deg = (int)(c.net_off[e + 1] - o0);  // stamped nets have at most the activation threshold of pins
    }
    packed_incidences(hit, o0, deg, own, [&](bool has, int, int64_t j) -> int {
      if (has) c.next_flag[c.pins[j]] = 1;
      return 0;
    });
  }
}

cudaError_t launch_expand_nets(const Launch& L, const RoundCtx& c, int S, PhaseTimer* timer) {
  {
    Scope sc(timer, "activate");
    k_activate_round<<<grid_for(L, c.n, kActThreads, occupancy((const void*)k_activate_round, kActThreads, 0)),
                       kActThreads, 0, L.st>>>(c, S);
    LAUNCHED("k_activate_round");
  }
  if (c.m == 0) return cudaSuccess;
  Scope sc(timer, "expand");
  k_expand_nets<<<grid_for(L, c.m, kActThreads, occupancy((const void*)k_expand_nets, kActThreads, 0)),
                  kActThreads, 0, L.st>>>(c);
  LAUNCHED("k_expand_nets");
  return cudaSuccess;
}

// ============================================================= rebalancer
//
// One round of the deterministic rebalancer (lpgpu_session_rebalance, the
// synchronous restatement of Rebalancer::rebalance,
// rebalancing/rebalancer.cpp:34-171). The list is the identity over all
// vertices and the LP selection and commit run unchanged after it.
// Per-block scratch rb: W0 [0, k) (weight of non-worsening candidates), count
// of worsening ones [k, 2k), need [2k, 3k), segment offsets [3k, 4k + 1),
// thresholds [4k + 1, 5k + 1).

// Best move with rebalance = true of every border vertex of an overloaded
// block (Km1Policy::computeMaxGainMoveImpl, gain_policy.h:108-167): minimum
// score over feasible blocks, any sign, lowest id on ties. Warp per vertex,
// penalties summed per block in shared memory.
__global__ void __launch_bounds__(256) k_rb_candidates(RoundCtx c, int round, int32_t* __restrict__ rb_to,
                                                       int32_t* __restrict__ rb_score, int64_t* __restrict__ rb) {
  extern __shared__ int s_rbagg[];
  const int k = c.k, W = c.W, lane = lane_id();
  int* agg = s_rbagg + (threadIdx.x >> 5) * k;
  for (int b = lane; b < k; b += 32) agg[b] = 0;
  __syncwarp();
  int64_t active = 0, pins = 0, cands = 0;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; v < c.n; v += warps) {
    const int from = c.part[v];
    if (c.bw[from] <= c.lmax[from]) {
      if (lane == 0) rb_to[v] = -1;
      continue;
    }
    const int64_t o0 = c.vtx_off[v], o1 = c.vtx_off[v + 1];
    ++active;
    pins += o1 - o0;
    int internal = 0;
    bool border = false;
    if (o1 - o0 <= kHighDegree) {  // isBorderNode is false above the threshold
      for (int64_t j = o0 + lane; j < o1; j += 32) {
        const int64_t e = c.inets[j];
        const int we = c.w_e[e];
        const uint32_t* rec = c.conn + e * 2 * W;
        if (!((rec[W + (from >> 5)] >> (from & 31)) & 1u)) internal += we;  // Φ(e, from) > 1
        int lam = 0;
        for (int w = 0; w < W; ++w) {
          uint32_t bits = rec[w];
          lam += __popc(bits);
          while (bits) {
            const int b = 32 * w + __ffs(bits) - 1;
            bits &= bits - 1;
            if (b != from) atomicAdd(&agg[b], we);
          }
        }
        border = border || lam > 1;
      }
    }
    internal = warp_sum(internal);
    border = __any_sync(FULLMASK, border);
    __syncwarp();
    const int64_t wv = c.w_v[v];
    unsigned long long best = ~0ull;
    for (int b = lane; b < k; b += 32) {
      if (border && b != from && c.bw[b] + wv <= c.lmax[b]) {
        const int sc = internal - agg[b];
        const unsigned long long key = ((unsigned long long)((uint32_t)sc ^ 0x80000000u) << 32) | (uint32_t)b;
        best = key < best ? key : best;
      }
      agg[b] = 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long y = __shfl_xor_sync(FULLMASK, best, o);
      best = y < best ? y : best;
    }
    __syncwarp();
    if (lane == 0) {
      if (best == ~0ull) {
        rb_to[v] = -1;
      } else {
        const int sc = (int)((uint32_t)(best >> 32) ^ 0x80000000u);
        rb_to[v] = (int)(best & 0xffffffffu);
        rb_score[v] = sc;
        if (sc <= 0)
          atomicAdd(reinterpret_cast<ull*>(&rb[from]), (ull)wv);
        else
          atomicAdd(reinterpret_cast<ull*>(&rb[k + from]), 1ull);
        ++cands;
      }
    }
  }
  if (lane == 0) {
    int64_t* st = c.stats + (int64_t)round * kStats;
    if (active) atomicAdd(reinterpret_cast<ull*>(&st[kStActive]), (ull)active);
    if (pins) atomicAdd(reinterpret_cast<ull*>(&st[kStPins]), (ull)pins);
    if (cands) atomicAdd(reinterpret_cast<ull*>(&st[kStCands]), (ull)cands);
  }
}

// Need of every overloaded block beyond its non-worsening candidates, and
// segments for its worsening candidates (one CTA).
__global__ void k_rb_src_plan(RoundCtx c, int64_t* rb) {
  const int k = c.k;
  __shared__ int64_t s_run;
  if (threadIdx.x == 0) s_run = 0;
  __syncthreads();
  for (int b0 = 0; b0 < k; b0 += blockDim.x) {
    const int b = b0 + threadIdx.x;
    int64_t cnt = 0;
    if (b < k) {
      const int64_t x = c.bw[b] - c.lmax[b];
      const int64_t need = x > 0 ? x - rb[b] : 0;
      rb[2 * k + b] = need;
      cnt = need > 0 ? rb[k + b] : 0;
    }
    int64_t total;
    const int64_t off = block_scan_excl_i64(cnt, &total) + s_run;
    if (b < k) {
      rb[3 * k + b] = off;
      c.cursor[b] = off;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_run += total;
    __syncthreads();
  }
}

__global__ void k_rb_src_bin(RoundCtx c, const int32_t* __restrict__ rb_to, const int32_t* __restrict__ rb_score,
                             const int64_t* __restrict__ rb) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < c.n; v += (int64_t)gridDim.x * blockDim.x) {
    if (rb_to[v] < 0 || rb_score[v] <= 0) continue;
    const int from = c.part[v];
    if (rb[2 * c.k + from] <= 0) continue;
    const ull slot = atomicAdd(reinterpret_cast<ull*>(&c.cursor[from]), 1ull);
    c.seg_key[slot] = move_key(rb_score[v], (int32_t)v);
    c.seg_w[slot] = c.w_v[v];
  }
}

// Per block with a need: the first worsening key whose weighted prefix
// reaches the need (keys up to it are taken).
__global__ void __launch_bounds__(kSelThreads) k_rb_src_select(RoundCtx c, int64_t* rb) {
  const int k = c.k;
  uint64_t* thr = reinterpret_cast<uint64_t*>(rb + 4 * k + 1);
  for (int b = blockIdx.x; b < k; b += gridDim.x) {
    const int64_t need = rb[2 * k + b], cnt = need > 0 ? rb[k + b] : 0;
    uint64_t t = 0;
    if (cnt > 0) t = cta_radix_select(c.seg_key + rb[3 * k + b], c.seg_w + rb[3 * k + b], cnt, need - 1);
    if (threadIdx.x == 0) thr[b] = t;
    __syncthreads();
  }
}

// Candidates the source side takes become the LP candidates (rec, per-block
// totals); the last CTA plans the target-side selection.
__global__ void k_rb_emit(RoundCtx c, const int32_t* __restrict__ rb_to, const int32_t* __restrict__ rb_score,
                          const int64_t* __restrict__ rb) {
  const int k = c.k;
  const uint64_t* thr = reinterpret_cast<const uint64_t*>(rb + 4 * k + 1);
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < c.n; v += (int64_t)gridDim.x * blockDim.x) {
    const int from = c.part[v];
    int4 r = make_int4(-1, 0, (int)v, from);
    const int to = rb_to[v];
    if (to >= 0) {
      const int sc = rb_score[v];
      const bool take = sc <= 0 || (rb[2 * k + from] > 0 && rb[k + from] > 0 &&
                                    move_key(sc, (int32_t)v) <= thr[from]);
      if (take) {
        r.x = to;
        r.y = sc;
        const int64_t wv = c.w_v[v];
        atomicAdd(reinterpret_cast<ull*>(&c.in_w[to]), (ull)wv);
        atomicAdd(reinterpret_cast<ull*>(&c.in_cnt[to]), 1ull);
        atomicAdd(reinterpret_cast<ull*>(&c.cand_out[from]), (ull)wv);
      }
    }
    c.rec[v] = r;
  }
  if (last_cta(&c.scal[kDone])) plan_to(c);
}

// ---- empty-block repair (Rebalancer::repairEmptyBlocks, rebalancer.cpp:169-269)
//
// For one empty block `blk`: every vertex u eligible for it (c(part(u)) >
// w(u), w(u) <= L_max(blk)) gets its gain score(blk) - unremovable(u)
// (rebalancer.cpp:190-201; score = Σ w(e) of incident nets with blk in Λ(e),
// unremovable = Σ w(e) of incident nets with Φ(e, part(u)) > 1, read as
// part(u) not in Λ1(e)) and the key (gain descending, vertex ascending) with
// weight 1; ineligible vertices get key ~0 and weight 0. A radix selection
// then finds the k-th smallest key: the keys up to it are the k vertices the
// reference's bounded per-thread heap keeps (rebalancer.cpp:204-213).
__global__ void k_repair_keys(RoundCtx c, int blk, uint64_t* __restrict__ keys, int32_t* __restrict__ ws) {
  const int W = c.W;
  const int64_t cap = c.lmax[blk];
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < c.n; v += (int64_t)gridDim.x * blockDim.x) {
    const int p = c.part[v];
    const int64_t wv = c.w_v[v];
    uint64_t key = ~0ull;
    if (p != blk && c.bw[p] > wv && wv <= cap) {
      int64_t score = 0, unremovable = 0;
      for (int64_t j = c.vtx_off[v]; j < c.vtx_off[v + 1]; ++j) {
        const int64_t e = c.inets[j];
        const int we = c.w_e[e];
        const uint32_t* rec = c.conn + e * 2 * W;
        if ((rec[blk >> 5] >> (blk & 31)) & 1u) score += we;
        if (!((rec[W + (p >> 5)] >> (p & 31)) & 1u)) unremovable += we;
      }
      const int32_t gain = (int32_t)(score - unremovable);
      key = ((uint64_t)(~((uint32_t)gain ^ 0x80000000u)) << 32) | (uint32_t)v;
    }
    keys[v] = key;
    ws[v] = key == ~0ull ? 0 : 1;
  }
}

// One CTA: the k-th smallest key (budget k - 1 over unit weights), or ~0
// when fewer than k vertices are eligible.
__global__ void __launch_bounds__(kSelThreads) k_repair_select(const uint64_t* __restrict__ keys,
                                                               const int32_t* __restrict__ ws, int64_t n, int k,
                                                               uint64_t* thr) {
  const uint64_t t = cta_radix_select(keys, ws, n, (int64_t)k - 1);
  if (threadIdx.x == 0) *thr = t;
}

// The kept vertices (key <= threshold) as (vertex, gain, block, weight);
// *count receives their number (at most k).
__global__ void k_repair_collect(RoundCtx c, const uint64_t* __restrict__ keys, const uint64_t* __restrict__ thr,
                                 int4* __restrict__ out, int64_t* count) {
  const uint64_t t = *thr;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < c.n; v += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t key = keys[v];
    if (key == ~0ull || key > t) continue;
    const int32_t gain = (int32_t)((~(uint32_t)(key >> 32)) ^ 0x80000000u);
    const ull slot = atomicAdd(reinterpret_cast<ull*>(count), 1ull);
    out[slot] = make_int4((int)v, gain, c.part[v], c.w_v[v]);
  }
}

cudaError_t launch_repair_candidates(const Launch& L, const RoundCtx& c, int blk, uint64_t* keys, int32_t* ws,
                                     int4* out, int64_t* scratch) {
  if (c.n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(int64_t) * 2, L.st);
  if (e != cudaSuccess) return e;
  const int g = grid_for(L, c.n, 256);
  k_repair_keys<<<g, 256, 0, L.st>>>(c, blk, keys, ws);
  LAUNCHED("k_repair_keys");
  allow_dyn_smem(k_repair_select, kSelSmem);
  k_repair_select<<<1, kSelThreads, kSelSmem, L.st>>>(keys, ws, c.n, c.k,
                                                      reinterpret_cast<uint64_t*>(scratch + 1));
  LAUNCHED("k_repair_select");
  k_repair_collect<<<g, 256, 0, L.st>>>(c, keys, reinterpret_cast<const uint64_t*>(scratch + 1), out, scratch);
  LAUNCHED("k_repair_collect");
  return cudaGetLastError();
}

cudaError_t launch_rebalance_round(const Launch& L, const RoundCtx& c, int round, int32_t* rb_to,
                                   int32_t* rb_score, int64_t* rb) {
  if (c.n == 0) return cudaSuccess;
  const int k = c.k;
  cudaError_t e = cudaMemsetAsync(rb, 0, sizeof(int64_t) * 2 * k, L.st);
  if (e != cudaSuccess) return e;
  const size_t smem = sizeof(int) * k * 8;
  allow_dyn_smem(k_rb_candidates, smem);
  k_rb_candidates<<<grid_for(L, c.n * 32, 256), 256, smem, L.st>>>(c, round, rb_to, rb_score, rb);
  LAUNCHED("k_rb_candidates");
  k_rb_src_plan<<<1, 1024, 0, L.st>>>(c, rb);
  LAUNCHED("k_rb_src_plan");
  const int g = grid_for(L, c.n, 256);
  k_rb_src_bin<<<g, 256, 0, L.st>>>(c, rb_to, rb_score, rb);
  LAUNCHED("k_rb_src_bin");
  allow_dyn_smem(k_rb_src_select, kSelSmem);
  k_rb_src_select<<<(unsigned)std::min<int64_t>(k, 4 * (int64_t)L.num_sms), kSelThreads, kSelSmem, L.st>>>(c, rb);
  LAUNCHED("k_rb_src_select");
  k_rb_emit<<<g, 256, 0, L.st>>>(c, rb_to, rb_score, rb);
  LAUNCHED("k_rb_emit");
  // the LP target-side selection, source floor and commit of one sub-round
  k_bin_moves<<<grid_for(L, c.n, kBinThreads), kBinThreads, 0, L.st>>>(c, 0);
  LAUNCHED("k_bin_moves");
  allow_dyn_smem(k_select, kSelSmem);
  k_select<<<(unsigned)std::min<int64_t>(k, 4 * (int64_t)L.num_sms), kSelThreads, kSelSmem, L.st>>>(c, 0);
  LAUNCHED("k_select");
  const size_t dw_smem = sizeof(ull) * k;
  k_commit<<<grid_for(L, c.n, kFlatItems, occupancy((const void*)k_commit, kFlatThreads, dw_smem)), kFlatThreads,
             dw_smem, L.st>>>(c, round, 0, 1);
  LAUNCHED("k_commit");
  return cudaGetLastError();
}

cudaError_t launch_subround(const Launch& L, const RoundCtx& c, int round, int sub, PhaseTimer* timer) {
  const int k = c.k;
  const size_t dw_smem = c.batched ? 0 : sizeof(ull) * k;  // shared block-weight deltas
  const int64_t n = c.n;
  {
    Scope sc(timer, "sweep");
    cudaError_t e = launch_sweep(L, c, round, sub, nullptr, nullptr, nullptr);
    if (e != cudaSuccess) return e;
  }
  const int g = grid_for(L, n, 256, 8);
  // incidence kernels: one wave of resident CTAs striding over the sub-round
  const int g_commit = grid_for(L, n, kFlatItems, occupancy((const void*)k_commit, kFlatThreads, dw_smem));
  const int g_eval = grid_for(L, n, kFlatItems, occupancy((const void*)k_revert_eval, kFlatThreads, 0));
  // undo kernels usually have little to do: one CTA per SM
  const int g_undo = (int)std::max<int64_t>(1, std::min<int64_t>((n + kFlatItems - 1) / kFlatItems, L.num_sms));
  const int g_unrev = (int)std::max<int64_t>(1, std::min<int64_t>((n + 31) / 32, L.num_sms));
  const int g_bin = grid_for(L, n, kBinThreads * (c.batched ? 1 : kBinPer),
                             occupancy((const void*)k_bin_moves, kBinThreads, 0));
  {
    Scope sc(timer, "select");
    k_bin_moves<<<g_bin, kBinThreads, 0, L.st>>>(c, sub);
    LAUNCHED("k_bin_moves");
    allow_dyn_smem(k_select, kSelSmem);
    k_select<<<(unsigned)std::min<int64_t>(k, 4 * (int64_t)L.num_sms), kSelThreads, kSelSmem, L.st>>>(c, sub);
    LAUNCHED("k_select");
  }
  const int last_commit = !c.revert && !c.rollback;
  {
    Scope sc(timer, "commit");
    k_commit<<<g_commit, kFlatThreads, dw_smem, L.st>>>(c, round, sub, last_commit);
    LAUNCHED("k_commit");
  }
  // one instance with reverts: the rollback check runs in the undo kernel's last CTA
  const int roll_tail = c.revert && c.rollback && !c.batched;
  if (c.revert) {
    Scope sc(timer, "revert");
    k_revert_eval<<<g_eval, kFlatThreads, 0, L.st>>>(c, sub);
    LAUNCHED("k_revert_eval");
    k_undo_reverts<<<g_unrev, kFlatThreads, dw_smem, L.st>>>(c, round, sub, !c.rollback, roll_tail);
    LAUNCHED("k_undo_reverts");
  }
  if (c.rollback && !roll_tail) {
    Scope sc(timer, "rollback");
    k_rollback<<<g_undo, kFlatThreads, dw_smem, L.st>>>(c, round, sub);
    LAUNCHED("k_rollback");
  }
  return cudaSuccess;
}

// ======================================================= persistent rounds
//
// A batch of many small instances runs one launch per LP round. Every CTA
// takes whole instances from a device work queue (largest first unless the
// tuning says otherwise) and runs all S sub-rounds of that instance's round
// itself: sweep, target- and source-side selection, commit, hindsight
// reverts, rollback and activation, separated by CTA barriers instead of
// grid-wide launch boundaries. Instances are independent, so no CTA ever
// waits for another, and a CTA that finishes a small instance takes the next
// one while others are still on large ones. Each phase follows the same rule
// as the multi-launch pipeline (the same lane-per-vertex sweep, selection
// thresholds and CTA-flat commit), so every instance ends exactly as when it
// is refined alone. The sweep reads the Λ records that the same kernel's
// commits change, so it loads them through the coherent path, not __ldg.

constexpr int kPxThreads = kFlatThreads;  // the CTA-flat helpers are written for this width
constexpr int kPxWarps = kPxThreads / 32;
static_assert(kPxThreads <= kSelThreads, "the radix selection's histograms cover the CTA");

struct PxShared {
  int64_t bw[kPxMaxK], lmax[kPxMaxK], perf[kPxMaxK];
  int slack[kPxMaxK];
  uint32_t fmask[kLvWeights * 2];
  ull in_w[kPxMaxK], acc_w[kPxMaxK];
  unsigned in_cnt[kPxMaxK], acc_cnt[kPxMaxK];
  int64_t seg[kPxMaxK + 1];
  unsigned cursor[kPxMaxK];
  uint64_t thr_to[kPxMaxK], thr_from[kPxMaxK];
  int pen[kPxWarps][kPxMaxK];
  int ncand, nrev, item;
  long long st[kStats];
};

__device__ __forceinline__ RoundCtx px_ctx(const PxInst& I) {
  RoundCtx c{};
  c.vtx_off = I.vtx_off;
  c.inets = I.inets;
  c.w_v = I.w_v;
  c.w_e = I.w_e;
  c.part = I.part;
  c.phi = I.phi;
  c.conn = I.conn;
  c.k = I.k;
  c.W = I.W;
  c.kmax = I.kstride;
  c.unit_nets = I.unit_nets;
  c.phi16 = I.phi16;
  c.max_we = I.max_we;
  return c;
}

// A candidate move of local vertex lv: its record, the per-block totals and
// the sub-round's candidate list.
__device__ __forceinline__ void px_candidate(const PxInst& I, PxShared& s, int64_t lv, int from, int to, int gain,
                                             int wv) {
  I.rec[I.v0 + lv] = make_int4(to, gain, 0, from);
  atomicAdd(&s.in_w[to], (ull)(int64_t)wv);
  atomicAdd(&s.in_cnt[to], 1u);
  I.cand[atomicAdd(&s.ncand, 1)] = (int32_t)lv;
}

// A heavy vertex (summed net weight beyond the lane counters), evaluated by
// the warp that found it: lanes split its incidences, penalties are summed per
// block in the warp's shared row, then the block-owning lanes decide (decide:
// the rule of Km1Policy::computeMaxGainMoveImpl).
template <int W, bool UNIT>
__device__ void px_heavy(const PxInst& I, const PxParams& P, PxShared& s, int64_t lv) {
  const int lane = lane_id(), wid = threadIdx.x >> 5, k = I.k;
  int* pen = s.pen[wid];
  const int64_t v = I.v0 + lv;
  const int64_t o0 = I.vtx_off[v];
  const int d = (int)(I.vtx_off[v + 1] - o0);
  const int from = I.part[v] - I.boff, wv = I.w_v[v];
  for (int b = lane; b < k; b += 32) pen[b] = 0;
  __syncwarp();
  const int fw = from >> 5;
  const uint32_t fbit = 1u << (from & 31);
  int internal = 0;
  bool border = false;
  for (int j = lane; j < d; j += 32) {
    const int64_t e = I.inets[o0 + j];
    const int we = UNIT ? 1 : I.w_e[e];
    const uint32_t* rec = I.conn + e * 2 * W;
    if (!(rec[W + fw] & fbit)) internal += we;  // Φ(e, from) > 1
#pragma unroll
    for (int t = 0; t < W; ++t) {
      uint32_t bits = rec[t] & (t == fw ? ~fbit : ~0u);
      border = border || bits != 0;
      while (bits) {
        atomicAdd(&pen[32 * t + __ffs(bits) - 1], we);
        bits &= bits - 1;
      }
    }
  }
  internal = warp_sum(internal);
  border = __any_sync(FULLMASK, border);
  __syncwarp();
  if (border) {
    int pn[W], sl[W];
#pragma unroll
    for (int t = 0; t < W; ++t) {
      const int b = 32 * t + lane;
      pn[t] = b < k ? pen[b] : 0;
      sl[t] = b < k ? s.slack[b] : -1;
    }
    int to = from, gain = 0;
    decide<W, false>(k, from, wv, internal, P.zero_gain, pn, sl, s.bw, s.perf, to, gain);
    if (lane == 0 && to != from) px_candidate(I, s, lv, from, to, gain, wv);
  }
  __syncwarp();
}

constexpr int kPxStage = 2048;  // selection keys staged in the CTA-flat area (not in use then)
static_assert(sizeof(FlatSmem) >= (size_t)kPxStage * 12, "staged keys and weights fit the CTA-flat area");

#ifndef LPGPU_PX_WARP_SEL
#define LPGPU_PX_WARP_SEL 512  // segments of at most this many keys get one warp each
#endif
constexpr int kPxWarpSelKeys = LPGPU_PX_WARP_SEL;
static_assert(sizeof(FlatSmem) >= (size_t)(kPxThreads / 32) * 256 * sizeof(unsigned),
              "every warp's selection histogram fits the CTA-flat area");

// Thresholds of the blocks flagged in `over` (bit b): the first key of the
// block's segment whose weighted prefix exceeds budget(b). The segments are
// filled from the candidate list by member(rec, lv) (the block a candidate
// belongs to, or -1); cnt[b] is the size of block b's segment.
template <typename Member, typename Budget>
__device__ void px_select(const PxInst& I, PxShared& s, FlatSmem& f, uint64_t over, const unsigned* cnt,
                          uint64_t* thr, Member member, Budget budget) {
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (int b = 0; b < I.k; ++b) {
      s.seg[b] = run;
      s.cursor[b] = (unsigned)run;
      if ((over >> b) & 1) run += cnt[b];
    }
    s.seg[I.k] = run;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < s.ncand; i += blockDim.x) {
    const int lv = I.cand[i];
    const int4 r = I.rec[I.v0 + lv];
    const int b = member(r, lv);
    if (b >= 0 && ((over >> b) & 1)) {
      const unsigned slot = atomicAdd(&s.cursor[b], 1u);
      I.keys[slot] = move_key(r.y, lv);
      I.kw[slot] = I.w_v[I.v0 + lv];
    }
  }
  __syncthreads();
  // with several blocks to select, small segments get one warp each, all at
  // once (histograms in the CTA-flat area, not in use here); the others take
  // the whole CTA, one after another
  const int64_t warp_keys = __popcll(over) > 1 ? kPxWarpSelKeys : -1;
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned* whist = reinterpret_cast<unsigned*>(&f) + 256 * wid;
  for (int b = wid; b < I.k; b += nw) {
    const int64_t nb = s.seg[b + 1] - s.seg[b];
    if (((over >> b) & 1) && nb <= warp_keys) {
      const uint64_t t = warp_radix_select(I.keys + s.seg[b], I.kw + s.seg[b], (int)nb, budget(b), whist);
      if (lane_id() == 0) thr[b] = t;
    }
  }
  __syncthreads();
  for (int b = 0; b < I.k; ++b) {
    if (!((over >> b) & 1) || s.seg[b + 1] - s.seg[b] <= warp_keys) continue;
    const uint64_t t = cta_radix_select(I.keys + s.seg[b], I.kw + s.seg[b], s.seg[b + 1] - s.seg[b], budget(b),
                                        reinterpret_cast<unsigned char*>(&f), kPxStage);
    if (threadIdx.x == 0) thr[b] = t;
    __syncthreads();
  }
}

// Moves the collected items of f (local vertex ids in f.pos, local
// from | to << 16 in f.ft) between their blocks: part, block weights and,
// CTA-flat, Φ / Λ / Λ1 with km1Delta attribution. Returns this thread's
// attributed delta.
__device__ __forceinline__ int64_t px_move_items(const RoundCtx& c, const PxInst& I, PxShared& s, FlatSmem& f,
                                                 int64_t* moved_pins, int64_t* toggles) {
  __syncthreads();
  const int n = f.n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int64_t v = I.v0 + f.pos[i];
    const int from = f.ft[i] & 0xffff, to = f.ft[i] >> 16;
    const int64_t wv = I.w_v[v];
    I.part[v] = I.boff + to;
    atomicAdd(reinterpret_cast<ull*>(&s.bw[to]), (ull)wv);
    atomicAdd(reinterpret_cast<ull*>(&s.bw[from]), (ull)(-wv));
  }
  const int total = flat_scan(f, n);
  if (moved_pins && threadIdx.x == 0) *moved_pins += total;
  const int64_t att = flat_commit(c, f, n, total, false, toggles);
  __syncthreads();
  return att;
}

// Collects into f the candidates [c0, c0 + kFlatItems) of the sub-round list
// with status `want` (0: the accepted ones), as moves from `from` to `to`
// (back: the reverse), and sets their status to `set` (0: unchanged).
// Returns this thread's number of collected items.
template <bool ACCEPT>
__device__ __forceinline__ int px_gather(const PxInst& I, PxShared& s, FlatSmem& f, int c0, int ncand, int want,
                                         bool back, int set) {
  constexpr int PER = kFlatItems / kPxThreads;
  if (threadIdx.x == 0) f.n = 0;
  __syncthreads();
  int got = 0;
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int i = c0 + q * kPxThreads + threadIdx.x;
    bool take = false;
    int lv = 0;
    int4 r = make_int4(0, 0, 0, 0);
    if (i < ncand) {
      lv = I.cand[i];
      r = I.rec[I.v0 + lv];
      if constexpr (ACCEPT) {
        const uint64_t key = move_key(r.y, lv);
        take = key < s.thr_to[r.x] && key < s.thr_from[r.w];
      } else {
        take = I.status[I.v0 + lv] == want;
      }
    }
    const int slot = flat_append(f, take);
    if (take) {
      const int64_t v = I.v0 + lv;
      f.o0[slot] = I.vtx_off[v];
      f.pre[slot] = (int)(I.vtx_off[v + 1] - f.o0[slot]);
      f.ft[slot] = back ? (r.x | (r.w << 16)) : (r.w | (r.x << 16));
      f.att[slot] = 0;
      f.pos[slot] = lv;
      if (set) I.status[v] = (uint8_t)set;
      ++got;
    }
  }
  return got;
}

template <int W, bool UNIT, int U>
__device__ void px_instance_round(const PxInst& I, const PxParams& P, PxShared& s, FlatSmem& f) {
  constexpr int PL = UNIT ? 6 : 8;
  const RoundCtx c = px_ctx(I);
  const int k = I.k, S = P.S;
  const int round = P.round >= 0 ? P.round : I.round;
  const int64_t ni = I.v1 - I.v0;
  for (int b = threadIdx.x; b < k; b += blockDim.x) {
    s.bw[b] = I.bw[I.boff + b];
    s.lmax[b] = I.lmax[I.boff + b];
    s.perf[b] = I.perfect[I.boff + b];
  }
  if (threadIdx.x < kStats) s.st[threadIdx.x] = 0;
  int64_t t_active = 0, t_pins = 0, t_moved_pins = 0, t_toggles = 0;
  __syncthreads();
  for (int sub = 0; sub < S; ++sub) {
    // ---- slack, feasibility masks, per-block totals
    for (int b = threadIdx.x; b < k; b += blockDim.x) {
      const int64_t sl = s.lmax[b] - s.bw[b];
      s.slack[b] = sl < 0 ? -1 : (sl > INT_MAX ? INT_MAX : (int)sl);
      s.in_w[b] = s.acc_w[b] = 0;
      s.in_cnt[b] = s.acc_cnt[b] = 0;
      s.thr_to[b] = s.thr_from[b] = ~0ull;
    }
    if (threadIdx.x == 0) {
      s.ncand = 0;
      s.nrev = 0;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kLvWeights * W; i += blockDim.x) {
      const int w = i / W + 1, t = i % W;
      uint32_t msk = 0;
      for (int l = 0; l < 32; ++l) {
        const int b = 32 * t + l;
        if (b < k && s.slack[b] >= w) msk |= 1u << l;
      }
      s.fmask[i] = msk;
    }
    __syncthreads();
    // ---- sweep: a sub-round holds whole 32-vertex chunks; warps take the
    // sub-round's chunks independently (no CTA barrier), a lane evaluates its
    // own vertex, and the warp evaluates the chunk's heavy vertices together
    {
      const int lane = lane_id(), wid = threadIdx.x >> 5;
      const int64_t nch = (ni + 31) >> kChunkShift;
      for (int64_t ch = wid; ch < nch; ch += kPxWarps) {
        if (subround_of(ch << kChunkShift, round, S) != sub) continue;
        const int64_t lv = (ch << kChunkShift) + lane, v = I.v0 + lv;
        bool heavy = false;
        if (lv < ni && (I.flag[v] & 1)) {
          I.status[v] = 0;
          const int64_t o0 = I.vtx_off[v], dd = I.vtx_off[v + 1] - o0;
          ++t_active;
          t_pins += dd;
          const int d = dd > kHighDegree ? 0 : (int)dd;  // isBorderNode is false above the threshold
          heavy = sweep_heavy(d, W, UNIT, I.max_we);
          if (!heavy && d > 0) {
            const int from = I.part[v] - I.boff, wv = I.w_v[v];
            int to = from, gain = 0;
            bool border = false;
            lv_vertex<W, UNIT, PL, U, false>(c, o0, d, from, wv, 0, 0, false, P.zero_gain, s.fmask, s.slack, s.bw,
                                             s.perf, to, gain, border);
            if (to != from) px_candidate(I, s, lv, from, to, gain, wv);
          }
        }
        for (unsigned hm = __ballot_sync(FULLMASK, heavy); hm; hm &= hm - 1)
          px_heavy<W, UNIT>(I, P, s, (ch << kChunkShift) + __ffs(hm) - 1);
      }
    }
    __syncthreads();
    const int ncand = s.ncand;
    // ---- target side (the atomic weight check of changeNodePart, h:548-562):
    // per block the longest (gain, vertex) prefix within L_max
    uint64_t over = 0;
    for (int b = 0; b < k; ++b)
      if ((int64_t)s.in_w[b] > s.lmax[b] - s.bw[b]) over |= 1ull << b;
    if (over)
      px_select(I, s, f, over, s.in_cnt, s.thr_to, [](const int4& r, int) { return r.x; },
                [&](int b) { return s.lmax[b] - s.bw[b]; });
    // ---- source side (from_weight_after > 0, h:551): per block the longest
    // prefix of its target-accepted moves that leaves weight >= 1
    for (int i = threadIdx.x; i < ncand; i += blockDim.x) {
      const int lv = I.cand[i];
      const int4 r = I.rec[I.v0 + lv];
      if (move_key(r.y, lv) < s.thr_to[r.x]) {
        atomicAdd(&s.acc_w[r.w], (ull)(int64_t)I.w_v[I.v0 + lv]);
        atomicAdd(&s.acc_cnt[r.w], 1u);
      }
    }
    __syncthreads();
    uint64_t over_from = 0;
    for (int b = 0; b < k; ++b)
      if (s.bw[b] - (int64_t)s.acc_w[b] < 1) over_from |= 1ull << b;
    if (over_from)
      px_select(I, s, f, over_from, s.acc_cnt, s.thr_from,
                [&](const int4& r, int lv) { return move_key(r.y, lv) < s.thr_to[r.x] ? r.w : -1; },
                [&](int b) { return s.bw[b] - 1; });
    // ---- commit of the accepted moves
    int64_t att = 0;
    for (int c0 = 0; c0 < ncand; c0 += kFlatItems) {
      px_gather<true>(I, s, f, c0, ncand, 0, false, 1);
      att += px_move_items(c, I, s, f, &t_moved_pins, &t_toggles);
    }
    // ---- hindsight reverts: every committed move is evaluated on the
    // post-commit state before any is undone (moveVertex,
    // label_propagation_refiner.h:100-137, made deterministic)
    if (P.revert) {
      for (int c0 = 0; c0 < ncand; c0 += kFlatItems) {
        px_gather<false>(I, s, f, c0, ncand, 1, false, 0);
        __syncthreads();
        const int n = f.n;
        const int total = flat_scan(f, n);
        // gain of moving back: + w(e) if Φ(e, to) > 1, - w(e) if from is in Λ(e)
        for (int x = threadIdx.x; x < total; x += kPxThreads) {
          const int it = flat_find(f, n, x);
          const int64_t e = I.inets[f.o0[it] + (x - f.pre[it])];
          const int fa = f.ft[it] & 0xffff, ta = f.ft[it] >> 16;
          const uint32_t* rec = I.conn + e * 2 * W;
          const int we = UNIT ? 1 : I.w_e[e];
          const int xa = (((rec[W + (ta >> 5)] >> (ta & 31)) & 1u) ? 0 : we) -
                         (((rec[fa >> 5] >> (fa & 31)) & 1u) ? we : 0);
          if (xa) atomicAdd(&f.att[it], xa);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x)
          if (f.att[i] < 0) {
            I.status[I.v0 + f.pos[i]] = 2;
            atomicAdd(&s.nrev, 1);
          }
        __syncthreads();
      }
      if (s.nrev)
        for (int c0 = 0; c0 < ncand; c0 += kFlatItems) {
          px_gather<false>(I, s, f, c0, ncand, 2, true, 0);
          att += px_move_items(c, I, s, f, nullptr, nullptr);
        }
    }
    // ---- rollback of a sub-round whose summed delta is positive
    att = block_sum_i64(att);
    int64_t rolled = 0;
    if (P.rollback && att > 0) {
      for (int c0 = 0; c0 < ncand; c0 += kFlatItems) {
        rolled += px_gather<false>(I, s, f, c0, ncand, 1, true, 3);
        att += block_sum_i64(px_move_items(c, I, s, f, nullptr, nullptr));
      }
      rolled = block_sum_i64(rolled);
    }
    // ---- activation of the kept moves (label_propagation_refiner.h:112-128):
    // the vertex and the pins of its nets with |e| <= threshold, once per net
    int64_t kept = 0;
    const int stamp = round + 1;
    for (int c0 = 0; c0 < ncand; c0 += kFlatItems) {
      kept += px_gather<false>(I, s, f, c0, ncand, 1, false, 0);
      __syncthreads();
      const int n = f.n;
      for (int i = threadIdx.x; i < n; i += blockDim.x) I.flag[I.v0 + f.pos[i]] |= 2;
      const int total = flat_scan(f, n);
      for (int x = threadIdx.x; x < total; x += kPxThreads) {
        const int it = flat_find(f, n, x);
        const int64_t e = I.inets[f.o0[it] + (x - f.pre[it])];
        const int64_t p0 = I.net_off[e], p1 = I.net_off[e + 1];
        if (p1 - p0 <= P.act_threshold && atomicExch(&I.net_epoch[e], stamp) != stamp)
          for (int64_t j = p0; j < p1; ++j) I.flag[I.pins[j]] |= 2;
      }
      __syncthreads();
    }
    kept = block_sum_i64(kept);
    if (threadIdx.x == 0) {
      s.st[kStCands] += ncand;
      s.st[kStMoved] += kept;
      s.st[kStReverted] += s.nrev + rolled;
      s.st[kStDelta] += att;
    }
    __syncthreads();
  }
  // ---- end of the instance's round: next round's flags, weights, statistics
  for (int64_t lv = threadIdx.x; lv < ni; lv += blockDim.x) I.flag[I.v0 + lv] >>= 1;
  for (int b = threadIdx.x; b < k; b += blockDim.x) I.bw[I.boff + b] = s.bw[b];
  t_active = block_sum_i64(t_active);
  t_pins = block_sum_i64(t_pins);
  t_moved_pins = block_sum_i64(t_moved_pins);
  t_toggles = block_sum_i64(t_toggles);
  if (threadIdx.x == 0) {
    int64_t* st = I.stats + (int64_t)round * kStats;
    s.st[kStActive] = t_active;
    s.st[kStPins] = t_pins;
    s.st[kStMovedPins] = t_moved_pins;
    s.st[kStToggles] = t_toggles;
    for (int j = 0; j < kStats; ++j)
      if (s.st[j]) atomicAdd(reinterpret_cast<ull*>(&st[j]), (ull)s.st[j]);
  }
  __syncthreads();
}

template <int W, bool UNIT, int U, int MINB>
__global__ void __launch_bounds__(kPxThreads, MINB) k_px_round(const PxInst* __restrict__ insts,
                                                               const int32_t* __restrict__ order, int32_t count,
                                                               PxParams P, int64_t* queue) {
  extern __shared__ __align__(16) unsigned char px_smem[];
  FlatSmem& f = *reinterpret_cast<FlatSmem*>(px_smem);
  PxShared& s = *reinterpret_cast<PxShared*>(px_smem + ((sizeof(FlatSmem) + 15) & ~size_t(15)));
  for (;;) {
    if (threadIdx.x == 0) s.item = (int)atomicAdd(reinterpret_cast<ull*>(queue), 1ull);
    __syncthreads();
    const int it = s.item;
    __syncthreads();
    if (it >= count) break;
    px_instance_round<W, UNIT, U>(insts[order ? order[it] : it], P, s, f);
  }
}

constexpr size_t kPxSmem = ((sizeof(FlatSmem) + 15) & ~size_t(15)) + sizeof(PxShared);

// Kernel variant: W words, unit net weights, sweep unroll 4 or 8, compiled for
// 1 resident CTA per SM (up to 128 registers) or 2 (64 registers).
template <int W, bool UNIT>
static const void* px_kernel_wu(int unroll, int minb) {
  if (minb >= 2) return unroll == 8 ? (const void*)k_px_round<W, UNIT, 8, 2> : (const void*)k_px_round<W, UNIT, 4, 2>;
  return unroll == 8 ? (const void*)k_px_round<W, UNIT, 8, 1> : (const void*)k_px_round<W, UNIT, 4, 1>;
}

static const void* px_kernel_for(int W, bool unit, int unroll, int minb) {
  if (W == 1) return unit ? px_kernel_wu<1, true>(unroll, minb) : px_kernel_wu<1, false>(unroll, minb);
  return unit ? px_kernel_wu<2, true>(unroll, minb) : px_kernel_wu<2, false>(unroll, minb);
}

// Active vertices of every instance's last persistent round (its round's
// statistics), for the host's stop rule.
__global__ void k_px_active(const PxInst* __restrict__ insts, int32_t count, int64_t* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const PxInst& I = insts[i];
    out[i] = I.stats[(int64_t)I.round * kStats + kStActive];
  }
}

cudaError_t launch_px_active(const Launch& L, const PxInst* insts, int32_t count, int64_t* out) {
  if (count <= 0) return cudaSuccess;
  k_px_active<<<(count + 255) / 256, 256, 0, L.st>>>(insts, count, out);
  return launched("k_px_active");
}

cudaError_t launch_px_round(const Launch& L, const PxInst* insts, const int32_t* order, int32_t count,
                            const PxParams& P, int W, bool unit, int ctas_per_sm, int64_t* queue) {
  if (count <= 0) return cudaSuccess;
  if (W != 1 && W != 2) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(int64_t), L.st);
  if (e != cudaSuccess) return e;
  const int minb = ctas_per_sm >= 2 ? 2 : 1;
  const void* kern = px_kernel_for(W, unit, P.unroll, minb);
  allow_dyn_smem(kern, kPxSmem);
  const int occ = std::max(1, occupancy(kern, kPxThreads, kPxSmem));
  const int per_sm = std::min(minb, occ);
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(count, (int64_t)per_sm * L.num_sms));
  void* args[] = {(void*)&insts, (void*)&order, (void*)&count, (void*)&P, (void*)&queue};
  e = cudaLaunchKernel(kern, dim3(grid), dim3(kPxThreads), args, kPxSmem, L.st);
  if (e != cudaSuccess) return e;
  return launched("k_px_round");
}

}  // namespace lpgpu
