// Shared device/host helpers: error reporting, launch geometry, deterministic
// FP64 reductions and padded-vector access.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/simkit_gb300.h"

namespace skg {

// gpu-scope acquire / release accesses of the grid barriers
__device__ __forceinline__ unsigned atom_add_acqrel_gpu(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_gpu(unsigned* p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}


// ---------------------------------------------------------------- errors --
int fail(int status, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define SKG_CUDA(call)                                                         \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) return ::skg::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)
#define SKG_LAUNCHED() SKG_CUDA(cudaGetLastError())
#define SKG_TRY(expr)          \
  do {                         \
    int s_ = (expr);           \
    if (s_ != SKG_OK) return s_; \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// ----------------------------------------------------------- geometry ----
constexpr int kBlock = 256;
// reductions run on a fixed grid so partial arrays are small and the
// summation order (hence the result) is fixed for a given size
constexpr int kReduceBlocks = 608;  // 152 SMs x 4

inline int blocks_for(int64_t n, int block = kBlock) {
  int64_t b = (n + block - 1) / block;
  return (int)(b < 1 ? 1 : b);
}

// ---------------------------------------------------------- reductions ---
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block of NV values per thread; result valid in thread 0.
template <int NV, int BLOCK>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double sh[NV][BLOCK / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = warp_sum(v[k]);
    if (lane == 0) sh[k][wid] = s;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = lane < BLOCK / 32 ? sh[k][lane] : 0.0;
      v[k] = warp_sum(s);
    }
  }
  __syncthreads();
}

// Deterministic grid reduction: every block stores its NV partials; the last
// block to arrive sums all partials in index order and writes out[0..NV-1].
// `counter` must be zero on entry and is reset to zero by the last block.
template <int NV, int BLOCK>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double* partials, unsigned* counter, double* out) {
  block_sum<NV, BLOCK>(v);
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    s[k] = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK)
      s[k] += *((volatile double*)&partials[k * gridDim.x + i]);
  }
  block_sum<NV, BLOCK>(s);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = s[k];
    *counter = 0u;
  }
  return true;
}

// ------------------------------------------------------- padded vectors --
// Per-vertex 3-vectors stored with stride 4 (x, y, z, pad) so that one
// vector load moves a vertex: float4 for FP32, two double2 for FP64.
template <typename R> struct Vec3 { R x, y, z; };

__device__ __forceinline__ Vec3<float> ld3(const float* p, int64_t v) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p) + v);
  return {a.x, a.y, a.z};
}
__device__ __forceinline__ Vec3<double> ld3(const double* p, int64_t v) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p) + 2 * v);
  const double b = __ldg(p + 4 * v + 2);
  return {a.x, a.y, b};
}
__device__ __forceinline__ void st3(float* p, int64_t v, Vec3<float> a) {
  reinterpret_cast<float4*>(p)[v] = make_float4(a.x, a.y, a.z, 0.f);
}
__device__ __forceinline__ void st3(double* p, int64_t v, Vec3<double> a) {
  reinterpret_cast<double2*>(p)[2 * v] = make_double2(a.x, a.y);
  reinterpret_cast<double2*>(p)[2 * v + 1] = make_double2(a.z, 0.0);
}
// plain (coherent) load for vectors written earlier in the same kernel
__device__ __forceinline__ Vec3<float> ld3c(const float* p, int64_t v) {
  const float4 a = reinterpret_cast<const float4*>(p)[v];
  return {a.x, a.y, a.z};
}
__device__ __forceinline__ Vec3<double> ld3c(const double* p, int64_t v) {
  const double2 a = reinterpret_cast<const double2*>(p)[2 * v];
  return {a.x, a.y, p[4 * v + 2]};
}

// 256-byte aligned bump allocator over a caller-provided workspace
struct Carve {
  char* base;
  int64_t off = 0;
  explicit Carve(void* b) : base(static_cast<char*>(b)) {}
  template <typename T> T* take(int64_t count) {
    off = (off + 255) & ~int64_t(255);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += count * (int64_t)sizeof(T);
    return p;
  }
};

}  // namespace skg
