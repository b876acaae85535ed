// Input checks of lpgpu_session_upload / _upload_batch and
// lpgpu_session_set_partition(_batch), run on the device over the copied
// buffers so that the host does no per-pin or per-vertex work.
//
// Every check sets the first failure code in out[kVErr]; the per-instance
// sums the int32 bounds need (Σ_e |e|·w(e), the Gain bound, and Σ_v w(v),
// the HypernodeWeight bound) are accumulated in out[kVSums + ...] and checked
// by the host after one copy back.
#include "common.cuh"

namespace lpgpu {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ void fail(int64_t* out, int code) {
  atomicCAS(reinterpret_cast<ull*>(&out[kVErr]), 0ull, (ull)code);
}

// Instance of element x given the instance start offsets off[0..I].
__device__ __forceinline__ int find_instance(const int64_t* __restrict__ off, int I, int64_t x) {
  int lo = 0, hi = I - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Batches: one CTA per instance. Its nets, thread per net: offsets inside
// [0, P] and non-decreasing, w(e) >= 0; its pins (the instance's pin range
// inst_poff[i] .. inst_poff[i + 1], non-decreasing and inside [0, P] by a
// host check), thread per pin: inside the instance's vertex range. Then the
// instance's Σ |e|·w(e), the largest net weight and size, and whether some
// weight differs from 1. With the offsets non-decreasing over all nets, the
// pins of instance i's nets are exactly its pin range, so this is the
// per-net pin check.
__global__ void __launch_bounds__(256) k_check_instances(int64_t P, const int64_t* __restrict__ net_off,
                                                         const int32_t* __restrict__ pins,
                                                         const int32_t* __restrict__ w_e,
                                                         const int64_t* __restrict__ inst_voff,
                                                         const int64_t* __restrict__ inst_noff,
                                                         const int64_t* __restrict__ inst_poff, int64_t* out) {
  __shared__ int64_t s_sum[8], s_maxs[8];
  __shared__ int s_maxw[8], s_flags[8];
  const int i = blockIdx.x;
  const int64_t e1 = inst_noff[i + 1];
  int64_t gsum = 0, maxs = 0;
  int maxw = 0, flags = 0;  // bit 0: non-unit weight, 1: bad offsets, 2: negative weight, 3: pin range
  for (int64_t e = inst_noff[i] + threadIdx.x; e < e1; e += blockDim.x) {
    const int64_t a = net_off[e], b = net_off[e + 1];
    if (a < 0 || b < a || b > P) {
      flags |= 2;
      continue;
    }
    const int we = w_e ? w_e[e] : 1;
    if (we < 0) {
      flags |= 4;
      continue;
    }
    maxw = max(maxw, we);
    maxs = max(maxs, b - a);
    flags |= we != 1;
    gsum += (b - a) * (int64_t)we;
  }
  const int64_t v0 = inst_voff[i], v1 = inst_voff[i + 1], q1 = inst_poff[i + 1];
  for (int64_t q = inst_poff[i] + threadIdx.x; q < q1; q += blockDim.x) {
    const int32_t p = pins[q];
    if (p < v0 || p >= v1) flags |= 8;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gsum += __shfl_xor_sync(FULL, gsum, o);
    maxw = max(maxw, __shfl_xor_sync(FULL, maxw, o));
    maxs = max(maxs, __shfl_xor_sync(FULL, maxs, o));
    flags |= __shfl_xor_sync(FULL, flags, o);
  }
  if (lane == 0) {
    s_sum[w] = gsum;
    s_maxw[w] = maxw;
    s_maxs[w] = maxs;
    s_flags[w] = flags;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int x = 1; x < (int)(blockDim.x >> 5); ++x) {
      gsum += s_sum[x];
      maxw = max(maxw, s_maxw[x]);
      maxs = max(maxs, s_maxs[x]);
      flags |= s_flags[x];
    }
    if (flags & 2) fail(out, kVBadOffsets);
    if (flags & 4) fail(out, kVNegNetWeight);
    if (flags & 8) fail(out, kVPinRange);
    if (gsum) atomicAdd(reinterpret_cast<ull*>(&out[kVSums + i]), (ull)gsum);
    if (maxw) atomicMax(reinterpret_cast<unsigned long long*>(&out[kVMaxWe]), (ull)maxw);
    if (maxs) atomicMax(reinterpret_cast<unsigned long long*>(&out[kVMaxSize]), (ull)maxs);
    if (flags & 1) atomicOr(reinterpret_cast<ull*>(&out[kVNonUnit]), 1ull);
  }
}

// One instance: thread per net (offsets, weights, Σ |e|·w(e)) ...
__global__ void k_check_nets_flat(int64_t m, int64_t P, const int64_t* __restrict__ net_off,
                                  const int32_t* __restrict__ w_e, int64_t* out) {
  int64_t gsum = 0, maxs = 0;
  int maxw = 0, nonunit = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = net_off[e], b = net_off[e + 1];
    if (a < 0 || b < a || b > P) {
      fail(out, kVBadOffsets);
      continue;
    }
    const int we = w_e ? w_e[e] : 1;
    if (we < 0) {
      fail(out, kVNegNetWeight);
      continue;
    }
    maxw = max(maxw, we);
    maxs = max(maxs, b - a);
    nonunit |= we != 1;
    gsum += (b - a) * (int64_t)we;
  }
  // one set of atomics per CTA: the sums meet in shared memory
  __shared__ int64_t s_sum[32], s_maxs[32];
  __shared__ int s_maxw[32], s_nonunit[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gsum += __shfl_xor_sync(FULL, gsum, o);
    maxw = max(maxw, __shfl_xor_sync(FULL, maxw, o));
    maxs = max(maxs, __shfl_xor_sync(FULL, maxs, o));
    nonunit |= __shfl_xor_sync(FULL, nonunit, o);
  }
  if (lane == 0) {
    s_sum[w] = gsum;
    s_maxw[w] = maxw;
    s_maxs[w] = maxs;
    s_nonunit[w] = nonunit;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int x = 1; x < (int)(blockDim.x >> 5); ++x) {
      gsum += s_sum[x];
      maxw = max(maxw, s_maxw[x]);
      maxs = max(maxs, s_maxs[x]);
      nonunit |= s_nonunit[x];
    }
    if (gsum) atomicAdd(reinterpret_cast<ull*>(&out[kVSums]), (ull)gsum);
    if (maxw) atomicMax(reinterpret_cast<unsigned long long*>(&out[kVMaxWe]), (ull)maxw);
    if (maxs) atomicMax(reinterpret_cast<unsigned long long*>(&out[kVMaxSize]), (ull)maxs);
    if (nonunit) atomicOr(reinterpret_cast<ull*>(&out[kVNonUnit]), 1ull);
  }
}

// ... and thread per pin (id in [0, n)): no pin read depends on the offsets.
__global__ void k_check_pins_flat(int64_t P, const int32_t* __restrict__ pins, int64_t n, int64_t* out) {
  bool bad = false;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < P; q += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = pins[q];
    bad |= p < 0 || p >= n;
  }
  if (bad) fail(out, kVPinRange);
}

// Thread per vertex: w(v) >= 0, the vertex's instance (written to vinst when
// given, i.e. for every batched session), Σ w(v) per instance (one instance:
// per-thread sums, one atomic per warp at the end; several: warp sums when
// the warp's vertices share an instance).
__global__ void k_check_vertices(int64_t n, const int32_t* __restrict__ w_v, int I,
                                 const int64_t* __restrict__ inst_voff, int32_t* __restrict__ vinst,
                                 int64_t* out) {
  const int lane = threadIdx.x & 31;
  if (I <= 1) {
    int64_t acc = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
      const int64_t w = w_v ? w_v[v] : 1;
      if (w < 0) fail(out, kVNegVertexWeight);
      if (vinst) vinst[v] = 0;
      acc += w;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
    if (lane == 0 && acc) atomicAdd(reinterpret_cast<ull*>(&out[kVSums + I]), (ull)acc);
    return;
  }
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = base + lane;
    const bool ok = v < n;
    int64_t w = 0;
    int inst = 0;
    if (ok) {
      w = w_v ? w_v[v] : 1;
      if (w < 0) fail(out, kVNegVertexWeight);
      if (vinst) {  // batched session (also with a single instance)
        inst = I > 1 ? find_instance(inst_voff, I, v) : 0;
        vinst[v] = inst;
      }
    }
    const int i0 = __shfl_sync(FULL, inst, 0);
    if (__all_sync(FULL, !ok || inst == i0)) {
      int64_t s = w;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
      if (lane == 0 && s) atomicAdd(reinterpret_cast<ull*>(&out[kVSums + I + i0]), (ull)s);
    } else if (ok && w) {
      atomicAdd(reinterpret_cast<ull*>(&out[kVSums + I + inst]), (ull)w);
    }
  }
}

// Partition ids: local id p of vertex v must lie in [0, k of v's instance);
// the stored id is the global block boff(instance) + p.
__global__ void k_check_partition(int64_t n, int32_t* __restrict__ part, int k, const int32_t* __restrict__ vinst,
                                  const int32_t* __restrict__ inst_boff, const int32_t* __restrict__ inst_k,
                                  int64_t* out) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = part[v];
    if (vinst) {
      const int i = vinst[v];
      if (p < 0 || p >= inst_k[i]) {
        fail(out, kVBlockRange);
        part[v] = 0;  // keeps later indexing in range; the call fails anyway
      } else {
        part[v] = p + inst_boff[i];
      }
    } else if (p < 0 || p >= k) {
      fail(out, kVBlockRange);
      part[v] = 0;
    }
  }
}

// CTA i shifts instance i's pins by its first vertex and its net offsets by
// its first pin (the ranges come from the host, so no access depends on the
// unchecked input).
// Instance-local ids to union ids, one CTA per instance. With `staged`, the
// instances' offset arrays (m_i + 1 entries each) lie back to back there,
// instance i's starting at inst_noff[i] + i, and are moved into place.
__global__ void k_rebase_instances(const int64_t* __restrict__ inst_voff, const int64_t* __restrict__ inst_noff,
                                   const int64_t* __restrict__ inst_poff, int64_t* __restrict__ net_off,
                                   int32_t* __restrict__ pins, const int64_t* __restrict__ staged) {
  const int i = blockIdx.x;
  const int32_t v0 = (int32_t)inst_voff[i];
  const int64_t p0 = inst_poff[i];
  if (v0)
    for (int64_t q = p0 + threadIdx.x; q < inst_poff[i + 1]; q += blockDim.x)
      pins[q] = (int32_t)((uint32_t)pins[q] + (uint32_t)v0);  // wraps: out-of-range ids stay out of range
  if (staged)
    for (int64_t e = inst_noff[i] + threadIdx.x; e < inst_noff[i + 1]; e += blockDim.x) net_off[e] = staged[e + i] + p0;
  else if (p0)
    for (int64_t e = inst_noff[i] + threadIdx.x; e < inst_noff[i + 1]; e += blockDim.x) net_off[e] += p0;
}

__global__ void k_fill_ones(int32_t* __restrict__ p, int64_t count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = 1;
}

__global__ void k_local_blocks(int64_t n, const int32_t* __restrict__ part, const int32_t* __restrict__ vinst,
                               const int32_t* __restrict__ inst_boff, int32_t* __restrict__ out) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    out[v] = part[v] - inst_boff[vinst[v]];
}

// part[v] = coarse_part[map[v]]; map entries outside [0, nc) set the check.
__global__ void k_project(int64_t n, const int32_t* __restrict__ map, const int32_t* __restrict__ coarse_part,
                          int64_t nc, int32_t* __restrict__ part, int64_t* check) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = map[v];
    if (u < 0 || u >= nc) {
      atomicCAS(reinterpret_cast<ull*>(check), 0ull, 1ull);
      part[v] = 0;
    } else {
      part[v] = coarse_part[u];
    }
  }
}

int grid(const Launch& L, int64_t items, int threads) {
  const int64_t need = (items + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)L.num_sms * 8));
}

}  // namespace

cudaError_t launch_validate_csr(const Launch& L, int64_t n, int64_t m, int64_t P, const int64_t* net_off,
                                const int32_t* pins, const int32_t* w_v, const int32_t* w_e, int I,
                                const int64_t* inst_voff, const int64_t* inst_noff, const int64_t* inst_poff,
                                int32_t* vinst, int64_t* out) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int64_t) * (kVSums + 2 * (int64_t)I), L.st);
  if (e != cudaSuccess) return e;
  if (I > 1) {
    if (m > 0 || P > 0)
      k_check_instances<<<I, 256, 0, L.st>>>(P, net_off, pins, w_e, inst_voff, inst_noff, inst_poff, out);
  } else {
    if (m > 0) k_check_nets_flat<<<grid(L, m, 256), 256, 0, L.st>>>(m, P, net_off, w_e, out);
    if (P > 0) k_check_pins_flat<<<grid(L, P, 256), 256, 0, L.st>>>(P, pins, n, out);
  }
  if (n > 0) k_check_vertices<<<grid(L, n, 256), 256, 0, L.st>>>(n, w_v, I, inst_voff, vinst, out);
  add_kernel_launches((I > 1 ? (m > 0 || P > 0) : (m > 0) + (P > 0)) + (n > 0));
  return cudaGetLastError();
}

cudaError_t launch_check_partition(const Launch& L, int64_t n, int32_t* part, int k, const int32_t* vinst,
                                   const int32_t* inst_boff, const int32_t* inst_k, int64_t* out) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int64_t) * kVSums, L.st);
  if (e != cudaSuccess) return e;
  if (n > 0) {
    k_check_partition<<<grid(L, n, 256), 256, 0, L.st>>>(n, part, k, vinst, inst_boff, inst_k, out);
    add_kernel_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t launch_rebase_instances(const Launch& L, int I, const int64_t* inst_voff, const int64_t* inst_noff,
                                    const int64_t* inst_poff, int64_t* net_off, int32_t* pins,
                                    const int64_t* staged) {
  if (I > 0) {
    k_rebase_instances<<<I, 256, 0, L.st>>>(inst_voff, inst_noff, inst_poff, net_off, pins, staged);
    add_kernel_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t launch_fill_ones(const Launch& L, int32_t* p, int64_t count) {
  if (count > 0) {
    k_fill_ones<<<grid(L, count, 256), 256, 0, L.st>>>(p, count);
    add_kernel_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t launch_local_blocks(const Launch& L, int64_t n, const int32_t* part, const int32_t* vinst,
                                const int32_t* inst_boff, int32_t* out) {
  if (n > 0) {
    k_local_blocks<<<grid(L, n, 256), 256, 0, L.st>>>(n, part, vinst, inst_boff, out);
    add_kernel_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t launch_project(const Launch& L, int64_t n, const int32_t* map, const int32_t* coarse_part, int64_t nc,
                           int32_t* part, int64_t* check) {
  cudaError_t e = cudaMemsetAsync(check, 0, sizeof(int64_t), L.st);
  if (e != cudaSuccess) return e;
  if (n > 0) {
    k_project<<<grid(L, n, 256), 256, 0, L.st>>>(n, map, coarse_part, nc, part, check);
    add_kernel_launches(1);
  }
  return cudaGetLastError();
}

}  // namespace lpgpu
