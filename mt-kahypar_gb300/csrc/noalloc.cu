// Allocation-free partition metrics (lpgpu_partition_metrics_noalloc).
//
// Some callers cannot let a library allocate device memory: runtimes that
// hand out every byte of device memory from their own pool or budget (a
// framework's caching allocator that has reserved the device, or a serving
// process with a fixed memory plan), and real-time loops where a cudaMalloc
// may synchronize the device or fail at the wrong moment. This entry point
// serves them: the caller passes device-resident inputs and outputs, and the
// only other device memory it uses is the file-scope array below, a fixed
// 8 KB that every GPU loading the library holds until the process exits.
#include <algorithm>
#include <mutex>
#include <string>

#include "common.cuh"

namespace lpgpu {

namespace {

// Cross-CTA accumulators: block weights [0, k), km1 at [k], cut at [k + 1].
constexpr int kNoAllocWords = LPGPU_MAX_K + 2;
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned long long* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array for the current device, looked up once
// per device (cudaGetSymbolAddress with that device current).
cudaError_t scratch_for_current_device(unsigned long long** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<unsigned long long*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

__global__ void k_noalloc_clear(unsigned long long* scratch, int words) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < words; i += gridDim.x * blockDim.x) scratch[i] = 0;
}

// c(V_b): shared-memory per-block sums, then one atomic per block and CTA.
__global__ void k_noalloc_block_weights(int64_t n, const int32_t* __restrict__ part,
                                        const int32_t* __restrict__ w_v, int k,
                                        unsigned long long* scratch) {
  extern __shared__ unsigned long long s_w[];
  for (int b = threadIdx.x; b < k; b += blockDim.x) s_w[b] = 0;
  __syncthreads();
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int b = part[v];
    if (b >= 0 && b < k) atomicAdd(&s_w[b], (unsigned long long)(int64_t)(w_v ? w_v[v] : 1));
  }
  __syncthreads();
  for (int b = threadIdx.x; b < k; b += blockDim.x)
    if (s_w[b]) atomicAdd(&scratch[b], s_w[b]);
}

// λ(e) per net from a per-warp k-bit shared set, summed into km1 and cut.
// Pins outside [0, n) and nets with a negative first offset are skipped, so
// a malformed CSR gives wrong sums instead of reads outside the partition.
__global__ void k_noalloc_connectivity(int64_t n, int64_t m, const int64_t* __restrict__ net_off,
                                       const int32_t* __restrict__ pins, const int32_t* __restrict__ w_e,
                                       const int32_t* __restrict__ part, int k,
                                       unsigned long long* scratch) {
  extern __shared__ unsigned s_bits[];
  const int words = (k + 31) / 32;
  const int lane = threadIdx.x & 31;
  unsigned* bits = s_bits + (threadIdx.x >> 5) * words;
  for (int w = lane; w < words; w += 32) bits[w] = 0;
  __syncwarp();
  long long km1 = 0, cut = 0;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; e < m; e += warps) {
    const int64_t lo = net_off[e], hi = net_off[e + 1];
    for (int64_t i = lo >= 0 ? lo + lane : hi; i < hi; i += 32) {
      const int32_t p = pins[i];
      if ((uint64_t)(int64_t)p >= (uint64_t)n) continue;
      const int b = part[p];
      if (b >= 0 && b < k) atomicOr(&bits[b >> 5], 1u << (b & 31));
    }
    __syncwarp();
    int lam = 0;
    for (int w = lane; w < words; w += 32) {
      lam += __popc(bits[w]);
      bits[w] = 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lam += __shfl_xor_sync(0xffffffffu, lam, o);
    __syncwarp();
    if (lane == 0) {
      const long long we = w_e ? w_e[e] : 1;
      km1 += (long long)(lam > 1 ? lam - 1 : 0) * we;
      cut += lam > 1 ? we : 0;
    }
  }
  if (lane == 0) {
    if (km1) atomicAdd(&scratch[k], (unsigned long long)km1);
    if (cut) atomicAdd(&scratch[k + 1], (unsigned long long)cut);
  }
}

__global__ void k_noalloc_finish(const unsigned long long* scratch, int k, int64_t* block_weights,
                                 int64_t* km1, int64_t* cut) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < k; b += gridDim.x * blockDim.x)
    block_weights[b] = (int64_t)scratch[b];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *km1 = (int64_t)scratch[k];
    *cut = (int64_t)scratch[k + 1];
  }
}

}  // namespace
}  // namespace lpgpu

using namespace lpgpu;

extern "C" lpgpu_status lpgpu_partition_metrics_noalloc(
    int64_t num_vertices, int64_t num_nets, const int64_t* net_offsets, const int32_t* pins,
    const int32_t* vertex_weights, const int32_t* net_weights, const int32_t* partition, int32_t k,
    int64_t* block_weights, int64_t* km1, int64_t* cut, void* stream) {
  if (k < 1 || k > LPGPU_MAX_K) {
    set_error("k = " + std::to_string(k) + " is outside [1, 1024]: the allocation-free metrics keep " +
              "their accumulators in a fixed " + std::to_string(kNoAllocWords) + "-word device array");
    return LPGPU_ERR_INVALID_ARG;
  }
  if (num_vertices < 0 || num_nets < 0) {
    set_error("negative vertex or net count");
    return LPGPU_ERR_INVALID_ARG;
  }
  if (!block_weights || !km1 || !cut || (num_vertices > 0 && !partition) ||
      (num_nets > 0 && (!net_offsets || !pins))) {
    set_error("null device pointer");
    return LPGPU_ERR_INVALID_ARG;
  }
  if (num_nets > 0 && num_vertices == 0) {
    set_error("nets without vertices: every pin must name a vertex in [0, num_vertices)");
    return LPGPU_ERR_INVALID_ARG;
  }
  cudaGetLastError();
  unsigned long long* scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess) {
    set_error(std::string("scratch lookup (cudaGetSymbolAddress): ") + cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice
               ? LPGPU_ERR_NO_DEVICE
               : LPGPU_ERR_CUDA;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_noalloc_clear<<<1, 1024, 0, st>>>(scratch, k + 2);
  if (num_vertices > 0) {
    const int blocks = (int)std::min<int64_t>(1024, num_vertices / 256 + 1);
    k_noalloc_block_weights<<<blocks, 256, sizeof(unsigned long long) * k, st>>>(
        num_vertices, partition, vertex_weights, k, scratch);
  }
  if (num_nets > 0) {
    // a warp per net, 8 warps per CTA, at most 2,048 CTAs striding over the nets
    const int blocks = (int)std::min<int64_t>(2048, num_nets / 8 + 1);
    k_noalloc_connectivity<<<blocks, 256, sizeof(unsigned) * 8 * ((k + 31) / 32), st>>>(
        num_vertices, num_nets, net_offsets, pins, net_weights, partition, k, scratch);
  }
  k_noalloc_finish<<<(k + 255) / 256, 256, 0, st>>>(scratch, k, block_weights, km1, cut);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("allocation-free metrics launch: ") + cudaGetErrorString(e));
    return LPGPU_ERR_CUDA;
  }
  return LPGPU_OK;
}
