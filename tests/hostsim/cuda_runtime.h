// Stand-in for <cuda_runtime.h> that lets the solver headers compile with a
// host C++ compiler, so the float64 instantiations of a kernel body can run
// on the CPU, one "thread" at a time, under AddressSanitizer.  Test
// infrastructure only: the qualifiers become no-ops, the read-only-cache
// load is a plain load, warp primitives act on a single lane, and the CUDA
// runtime calls used by the launch helpers are inert.  Kernels whose warps
// cooperate run with a warp width of one lane, each warp as a host thread
// (named barriers and __syncthreads below).
#pragma once
#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#define PDQ_HOST_SIM 1

// Named barriers of a kernel whose warps run as host threads: a phase
// completes when `expected` threads have arrived; `sync` waits for the phase
// it arrived in, `arrive` does not wait.
struct PdqHostBarrier {
  std::mutex mu;
  std::condition_variable cv;
  int expected = 2, count = 0;
  long phase = 0;
  void arrive() {
    std::lock_guard<std::mutex> lk(mu);
    if (++count == expected) {
      count = 0;
      ++phase;
      cv.notify_all();
    }
  }
  void sync() {
    std::unique_lock<std::mutex> lk(mu);
    const long ph = phase;
    if (++count == expected) {
      count = 0;
      ++phase;
      cv.notify_all();
      return;
    }
    cv.wait(lk, [&] { return phase != ph; });
  }
};
// the named barriers (indexed by id; 0 is __syncthreads') of the block the
// calling thread runs in, when its threads run concurrently (else null)
inline thread_local PdqHostBarrier* pdq_host_barriers = nullptr;
inline void pdq_host_named_arrive(int id) { pdq_host_barriers[id].arrive(); }
inline void pdq_host_named_sync(int id) { pdq_host_barriers[id].sync(); }

// A warp whose 32 lanes run as host threads: __syncwarp(mask) waits for the
// lanes of mask, __any_sync(mask, p) also ORs their predicates.  One barrier
// per mask value; the lanes of a mask meet its barriers in the same order.
struct PdqHostWarp {
  struct Bar {
    int count = 0;
    long gen = 0;
    bool acc = false, result = false;
  };
  std::mutex mu;
  std::condition_variable cv;
  Bar bars[33];  // by the mask's lowest lane: masks are contiguous lane groups here
  // values published for a shuffle, by barrier generation parity (a lane is
  // at most one generation ahead of the slowest lane of its mask)
  unsigned char slots[2][32][8];
  static int key(unsigned mask) { return mask == 0xffffffffu ? 32 : __builtin_ctz(mask); }
  // every lane of mask arrives; returns the OR of their predicates and, for a
  // shuffle, copies lane src's published value into out
  bool meet(unsigned mask, bool p, int lane = -1, const void* in = nullptr, int src = -1, void* out = nullptr,
            size_t bytes = 0) {
    std::unique_lock<std::mutex> lk(mu);
    Bar& b = bars[key(mask)];
    const long gen = b.gen;
    if (in) std::memcpy(slots[gen & 1][lane], in, bytes);
    b.acc = b.acc || p;
    if (++b.count == __builtin_popcount(mask)) {
      b.result = b.acc;
      b.acc = false;
      b.count = 0;
      ++b.gen;
      cv.notify_all();
    } else {
      cv.wait(lk, [&] { return b.gen != gen; });
    }
    if (out) std::memcpy(out, slots[gen & 1][src], bytes);
    return b.result;
  }
};
// the warp the calling thread runs in, when its lanes run concurrently (else null)
inline thread_local PdqHostWarp* pdq_host_warp = nullptr;

// A thread-block cluster whose blocks' threads run as host threads: block r
// of the cluster has its shared memory at base + r * region (the dynamic
// part first, then the fixed arrays at offsets common to all blocks), and a
// cluster barrier with separate arrive and wait.
struct PdqHostCluster {
  int dim = 1;
  unsigned char* base = nullptr;
  size_t region = 0, dynamic_bytes = 0;
  int expected = 1, count = 0;
  long phase = 0;
  std::mutex mu;
  std::condition_variable cv;
  size_t next_fixed = 0;
  std::vector<std::pair<std::string, size_t>> fixed;  // name -> offset past the dynamic part
  long arrive() {
    std::lock_guard<std::mutex> lk(mu);
    const long ph = phase;
    if (++count == expected) {
      count = 0;
      ++phase;
      cv.notify_all();
    }
    return ph;
  }
  void wait(long ph) {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return phase != ph; });
  }
  // the offset of a fixed shared array (the same in every block)
  size_t fixed_offset(const char* name, size_t bytes) {
    std::lock_guard<std::mutex> lk(mu);
    for (auto& f : fixed)
      if (f.first == name) return f.second;
    const size_t off = dynamic_bytes + next_fixed;
    next_fixed += (bytes + 15) / 16 * 16;
    if (off + bytes > region) std::abort();  // the harness sized the region too small
    fixed.emplace_back(name, off);
    return off;
  }
};
// the cluster the calling thread's block belongs to (else null)
inline thread_local PdqHostCluster* pdq_host_cluster = nullptr;
inline thread_local long pdq_host_cluster_phase = 0;

#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __shared__ static
#define __align__(n) __attribute__((aligned(n)))
#define __launch_bounds__(...)
#define __restrict__

struct pdq_host_uint3 {
  unsigned x, y, z;
};
extern thread_local pdq_host_uint3 threadIdx, blockIdx, blockDim;

struct float4 {
  float x, y, z, w;
};
struct double2 {
  double x, y;
};

template <typename T>
inline T __ldg(const T* p) {
  return *p;
}
// Shuffles: with the warp's lanes as host threads the value of the source
// lane (within width-wide segments); a lane alone gets its own value.
template <typename T>
inline T __shfl_sync(unsigned mask, T v, int src, int width = 32);
template <typename T>
inline T __shfl_xor_sync(unsigned mask, T v, int lane_mask, int width = 32);
template <typename T>
inline T __shfl_sync(unsigned mask, T v, int src, int width) {
  static_assert(sizeof(T) <= 8, "one word per lane");
  if (!pdq_host_warp) return v;
  const int lane = int(threadIdx.x & 31u);
  T r;
  pdq_host_warp->meet(mask, false, lane, &v, (lane & ~(width - 1)) + (src % width), &r, sizeof(T));
  return r;
}
template <typename T>
inline T __shfl_xor_sync(unsigned mask, T v, int lane_mask, int width) {
  static_assert(sizeof(T) <= 8, "one word per lane");
  if (!pdq_host_warp) return v;
  const int lane = int(threadIdx.x & 31u);
  (void)width;
  T r;
  pdq_host_warp->meet(mask, false, lane, &v, lane ^ lane_mask, &r, sizeof(T));
  return r;
}
inline void __syncwarp(unsigned mask = 0xffffffffu) {
  if (pdq_host_warp) pdq_host_warp->meet(mask, false);
}
inline bool __any_sync(unsigned mask, bool p) {  // one lane: its own predicate
  return pdq_host_warp ? pdq_host_warp->meet(mask, p) : p;
}
inline unsigned __clusterRelativeBlockRank() {
  return pdq_host_cluster ? unsigned(blockIdx.x % unsigned(pdq_host_cluster->dim)) : 0u;
}
inline void __cluster_barrier_arrive() {
  if (pdq_host_cluster) pdq_host_cluster_phase = pdq_host_cluster->arrive();
}
inline void __cluster_barrier_wait() {
  if (pdq_host_cluster) pdq_host_cluster->wait(pdq_host_cluster_phase);
}
inline void* __cluster_map_shared_rank(void* p, unsigned rank) {
  PdqHostCluster* c = pdq_host_cluster;
  if (!c) return p;
  const size_t off = size_t(static_cast<unsigned char*>(p) - c->base) % c->region;
  return c->base + size_t(rank) * c->region + off;
}
// this block's shared memory
inline unsigned char* pdq_host_block_smem() {
  return pdq_host_cluster->base + size_t(__clusterRelativeBlockRank()) * pdq_host_cluster->region;
}
inline void __syncthreads() {
  if (pdq_host_barriers) pdq_host_barriers[0].sync();
}
inline void __threadfence() {}
inline double __longlong_as_double(long long v) {
  double d;
  std::memcpy(&d, &v, 8);
  return d;
}
inline long long __double_as_longlong(double v) {
  long long d;
  std::memcpy(&d, &v, 8);
  return d;
}
inline float __fdividef(float a, float b) { return a / b; }
inline float __frcp_rn(float a) { return 1.0f / a; }
inline float __powf(float a, float b) { return std::pow(a, b); }
inline float rsqrtf(float a) { return 1.0f / std::sqrt(a); }
inline double rsqrt(double a) { return 1.0 / std::sqrt(a); }
using std::fabs;
using std::fmax;
using std::isfinite;
using std::isinf;
using std::isnan;
using std::max;
using std::min;
using std::pow;
using std::sqrt;

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorInvalidDevice = 101, cudaLimitStackSize = 0 };
typedef void* cudaStream_t;
struct cudaFuncAttributes {
  size_t localSizeBytes;
};
template <typename K>
inline cudaError_t cudaFuncGetAttributes(cudaFuncAttributes* a, K) {
  a->localSizeBytes = 0;
  return cudaSuccess;
}
inline cudaError_t cudaDeviceGetLimit(size_t* v, int) {
  *v = size_t(1) << 20;
  return cudaSuccess;
}
inline cudaError_t cudaDeviceSetLimit(int, size_t) { return cudaSuccess; }
inline cudaError_t cudaGetDevice(int* d) {
  *d = 0;
  return cudaSuccess;
}
