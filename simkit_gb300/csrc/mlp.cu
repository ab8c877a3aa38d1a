// Tensor-core (tcgen05) BF16 GEMM and the elementwise kernels of the
// warm-start MLP.
//
// GEMM: C[R x Nc] = A[R x L] . B[Nc x L]^T, both operands BF16 with the
// reduction dimension L contiguous ("K-major"), FP32 accumulation in tensor
// memory.  One CTA of 128 threads computes one 128-row tile over a range of
// reduction blocks (split-K along gridDim.y):
//   * thread 0 loads every 64-wide reduction block of the A tile (128 x 64)
//     and of B (Nc x 64) with TMA (cp.async.bulk.tensor.2d, 128-byte swizzle)
//     into shared memory, completing on one mbarrier;
//   * thread 0 issues tcgen05.mma (kind::f16, BF16 in, FP32 out, M = 128,
//     N = Nc, K = 16 per instruction) into a TMEM accumulator allocated by
//     warp 0, and commits to a second mbarrier;
//   * the four warps read the accumulator back with tcgen05.ld (warp w owns
//     TMEM lanes 32w..32w+31, i.e. rows 32w..32w+31 of the tile) and apply
//     the epilogue (bias, GELU, BF16 / FP32 stores).
// All mbarrier waits are bounded; on a timeout the kernel records an error,
// waits (bounded) for its in-flight work, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <math.h>
#include <string.h>

#include "common.cuh"

namespace skg {

constexpr int kTileM = 128;
constexpr int kBlkK = 64;  // reduction block: 64 BF16 = one 128-byte swizzle row
// dynamic shared memory cap: the 227 KB per-block opt-in minus room for the static variables
constexpr size_t kGemmSmemMax = 226 * 1024;

// ------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t sa(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(sa(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait (about a second); false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  for (long long i = 0; i < (1ll << 24); ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          sa(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(sa(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sa(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void umma_bf16(uint32_t d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(sa(bar))
               : "memory");
}
// 32 TMEM lanes x 32 fp32 columns: thread t of the warp gets its lane's 32 columns
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor of tcgen05: K-major operand tile whose rows
// are 128 bytes with the 128-byte swizzle; groups of 8 rows are 1024 bytes
// apart (stride byte offset), the leading byte offset is unused for this
// layout; bits 46-48 hold the fixed value 0b001, bits 61-63 the swizzle
// mode (2 = 128-byte).
__device__ __forceinline__ uint64_t sdesc_kmajor_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float gelu_tanh(float x) {
  // 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  return 0.5f * x * (1.f + tanhf(k0 * (x + k1 * x * x * x)));
}
__device__ __forceinline__ float gelu_tanh_grad(float x) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float u = k0 * (x + k1 * x * x * x);
  const float t = tanhf(u);
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * k0 * (1.f + 3.f * k1 * x * x);
}

enum GemmEpilogue : int {
  EPI_F32 = 0,        // out_f32[r][c] = acc (+ bias[c])  (split-K partials: partial slice per split)
  EPI_BIAS_GELU = 1,  // z = acc + bias[c]: out_z (bf16) = z, out_h (bf16) = gelu(z)
  EPI_BF16 = 2,       // out_h (bf16) = acc (+ bias[c])
};

struct GemmArgs {
  int R;           // rows of C (tile rows beyond R are dropped)
  int Nc;          // columns of C computed (multiple of 16, <= 256)
  int Nstore;      // columns stored (<= Nc)
  int kblocks;     // reduction blocks of 64 in total
  int kb_per_split;
  int epi;
  const float* bias;
  float* out_f32;        // [splits][R][ld_out] for EPI_F32
  __nv_bfloat16* out_z;  // [R][ld_out]
  __nv_bfloat16* out_h;  // [R][ld_out]
  int ld_out;
  int* err;
};

// dynamic shared memory: A blocks (kb x 16 KB) then B blocks (kb x Nc x 128 B), 1024-aligned
__global__ void __launch_bounds__(256, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem_dyn[];
  __shared__ __align__(8) uint64_t bar_load;
  __shared__ __align__(8) uint64_t bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int ok_load, ok_mma;
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * kTileM;
  const int split = blockIdx.y;
  const int kb0 = split * g.kb_per_split;
  int kb1 = kb0 + g.kb_per_split;
  if (kb1 > g.kblocks) kb1 = g.kblocks;
  const int nkb = kb1 > kb0 ? kb1 - kb0 : 0;
  uint32_t ncols = 32;
  while ((int)ncols < g.Nc) ncols <<= 1;
  const uint32_t a_bytes = kTileM * 128, b_bytes = (uint32_t)g.Nc * 128;
  unsigned char* sA = smem;
  unsigned char* sB = smem + (size_t)nkb * a_bytes;

  if (tid == 0) {
    mbar_init(&bar_load, 1);
    mbar_init(&bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    ok_load = ok_mma = 1;
  }
  if (warp == 0) {
    tmem_alloc(&tmem_base, ncols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (tid == 0 && nkb > 0) {
    mbar_expect_tx(&bar_load, nkb * (a_bytes + b_bytes));
    for (int k = 0; k < nkb; ++k) {
      tma_load_2d(sA + (size_t)k * a_bytes, &mapA, (kb0 + k) * kBlkK, row0, &bar_load);
      tma_load_2d(sB + (size_t)k * b_bytes, &mapB, (kb0 + k) * kBlkK, 0, &bar_load);
    }
    if (!mbar_wait(&bar_load, 0)) {
      ok_load = 0;
      atomicExch(g.err, SKG_ERR_TIMEOUT);
      mbar_wait(&bar_load, 0);  // let in-flight copies land before the CTA can exit
    } else {
      tc_fence_after();
      const uint32_t idesc = idesc_bf16_f32(kTileM, g.Nc);
      for (int k = 0; k < nkb; ++k) {
        const uint32_t a0 = sa(sA + (size_t)k * a_bytes), b0 = sa(sB + (size_t)k * b_bytes);
#pragma unroll
        for (int j = 0; j < kBlkK / 16; ++j)
          umma_bf16(tmem, sdesc_kmajor_sw128(a0 + 32 * j), sdesc_kmajor_sw128(b0 + 32 * j), idesc,
                    (k | j) != 0 ? 1u : 0u);
      }
      umma_commit(&bar_mma);
    }
  }
  __syncthreads();
  if (nkb > 0 && ok_load) {
    if (!mbar_wait(&bar_mma, 0)) {
      if (lane == 0) {
        atomicExch(g.err, SKG_ERR_TIMEOUT);
        ok_mma = 0;
      }
      mbar_wait(&bar_mma, 0);
    }
  }
  tc_fence_after();
  __syncthreads();

  // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows of the tile; the lane quarter a
  // warp may access) and every other 32-column chunk starting at chunk w / 4
  const int quarter = warp & 3;
  const int r = row0 + quarter * 32 + lane;
  const bool live = ok_load && ok_mma;
  for (int c0 = (warp >> 2) * 32; c0 < g.Nc; c0 += 64) {
    float v[32];
    if (nkb > 0 && live) {
      tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0, v);
    } else {
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = 0.f;
    }
    if (r >= g.R) continue;
    // each thread writes its own row: 16-byte vector stores where the whole 32-column chunk is
    // stored and the row stride keeps them aligned, scalar stores otherwise
    const bool vec16 = c0 + 32 <= g.Nstore;
    if (g.epi == EPI_F32) {
      float* o = g.out_f32 + ((size_t)split * g.R + r) * g.ld_out;
      if (vec16 && (g.ld_out % 4) == 0) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float4 t;
          t.x = v[4 * q] + (g.bias ? g.bias[c0 + 4 * q] : 0.f);
          t.y = v[4 * q + 1] + (g.bias ? g.bias[c0 + 4 * q + 1] : 0.f);
          t.z = v[4 * q + 2] + (g.bias ? g.bias[c0 + 4 * q + 2] : 0.f);
          t.w = v[4 * q + 3] + (g.bias ? g.bias[c0 + 4 * q + 3] : 0.f);
          reinterpret_cast<float4*>(o + c0)[q] = t;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int c = c0 + i;
          if (c < g.Nstore) o[c] = v[i] + (g.bias ? g.bias[c] : 0.f);
        }
      }
    } else if (g.epi == EPI_BIAS_GELU) {
      __nv_bfloat16* oz = g.out_z + (size_t)r * g.ld_out;
      __nv_bfloat16* oh = g.out_h + (size_t)r * g.ld_out;
      if (vec16 && (g.ld_out % 8) == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint4 zz, hh;
          uint32_t* zw = reinterpret_cast<uint32_t*>(&zz);
          uint32_t* hw = reinterpret_cast<uint32_t*>(&hh);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int c = 8 * q + 2 * i;
            const float z0 = v[c] + g.bias[c0 + c], z1 = v[c + 1] + g.bias[c0 + c + 1];
            const __nv_bfloat162 zb = __floats2bfloat162_rn(z0, z1);
            const __nv_bfloat162 hb = __floats2bfloat162_rn(gelu_tanh(z0), gelu_tanh(z1));
            zw[i] = *reinterpret_cast<const uint32_t*>(&zb);
            hw[i] = *reinterpret_cast<const uint32_t*>(&hb);
          }
          reinterpret_cast<uint4*>(oz + c0)[q] = zz;
          reinterpret_cast<uint4*>(oh + c0)[q] = hh;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int c = c0 + i;
          if (c < g.Nstore) {
            const float z = v[i] + g.bias[c];
            oz[c] = __float2bfloat16(z);
            oh[c] = __float2bfloat16(gelu_tanh(z));
          }
        }
      }
    } else {
      __nv_bfloat16* oh = g.out_h + (size_t)r * g.ld_out;
      if (vec16 && (g.ld_out % 8) == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint4 hh;
          uint32_t* hw = reinterpret_cast<uint32_t*>(&hh);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int c = 8 * q + 2 * i;
            const __nv_bfloat162 hb = __floats2bfloat162_rn(v[c] + (g.bias ? g.bias[c0 + c] : 0.f),
                                                            v[c + 1] + (g.bias ? g.bias[c0 + c + 1] : 0.f));
            hw[i] = *reinterpret_cast<const uint32_t*>(&hb);
          }
          reinterpret_cast<uint4*>(oh + c0)[q] = hh;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int c = c0 + i;
          if (c < g.Nstore) oh[c] = __float2bfloat16(v[i] + (g.bias ? g.bias[c] : 0.f));
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

// ------------------------------------------------------ elementwise kernels
// dZ = dH * gelu'(Z), BF16 in/out, FP32 math
__global__ void k_gelu_backward(const __nv_bfloat16* __restrict__ dH, const __nv_bfloat16* __restrict__ Z, int64_t n,
                                __nv_bfloat16* __restrict__ dZ) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  dZ[i] = __float2bfloat16(__bfloat162float(dH[i]) * gelu_tanh_grad(__bfloat162float(Z[i])));
}

// out[c][r] = in[r][c] for a rows x cols BF16 matrix (32 x 32 tiles)
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ in, int rows, int cols, int ld_in,
                                 __nv_bfloat16* __restrict__ out, int ld_out) {
  __shared__ __nv_bfloat16 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + j, c = bx + threadIdx.x;
    tile[j][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * ld_in + c] : __float2bfloat16(0.f);
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = bx + j, r = by + threadIdx.x;
    if (c < cols && r < rows) out[(size_t)c * ld_out + r] = tile[threadIdx.x][j];
  }
}

// out[r][c] = sum_s part[s][r][c] in split order (deterministic split-K reduction)
__global__ void k_reduce_splits(const float* __restrict__ part, int splits, int64_t n, float* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.f;
  for (int k = 0; k < splits; ++k) s += part[(size_t)k * n + i];
  out[i] = s;
}

// db[c] = sum_r dZ[r][c] (one CTA per column, fixed order)
__global__ void __launch_bounds__(256) k_colsum_bf16(const __nv_bfloat16* __restrict__ dZ, int rows, int cols, int ld,
                                                     float* __restrict__ db) {
  const int c = blockIdx.x;
  double acc[1] = {0.0};
  for (int r = threadIdx.x; r < rows; r += blockDim.x) acc[0] += __bfloat162float(dZ[(size_t)r * ld + c]);
  block_sum<1, 256>(acc);
  if (threadIdx.x == 0) db[c] = (float)acc[0];
}

// MSE loss and its gradient: y, t [rows][cols]; dY (bf16, ld) = 2 (y - t) / (rows cols); loss partial sums
__global__ void __launch_bounds__(256) k_mse(const float* __restrict__ y, int ld_y, const float* __restrict__ t,
                                             int rows, int cols, __nv_bfloat16* __restrict__ dy, int ld_dy,
                                             double* partials, unsigned* counter, double* out) {
  double acc[1] = {0.0};
  const double scale = 2.0 / ((double)rows * cols);
  const int64_t n = (int64_t)rows * cols;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t r = i / cols, c = i % cols;
    const double d = (double)y[r * ld_y + c] - (double)t[i];
    acc[0] += d * d;
    dy[r * ld_dy + c] = __float2bfloat16((float)(scale * d));
  }
  grid_sum<1, 256>(acc, partials, counter, out);
}

// Adam (Kingma & Ba 2015) on FP32 master weights; refreshes the BF16 copy
// w16 [rows][ld16] and its transpose wt16 [cols][ldt] (optional).
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ grad, float* __restrict__ m1,
                       float* __restrict__ m2, int rows, int cols, float lr, float b1, float b2, float eps, float bc1,
                       float bc2, __nv_bfloat16* __restrict__ w16, int ld16, __nv_bfloat16* __restrict__ wt16,
                       int ldt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)rows * cols) return;
  const float gr = grad[i];
  const float a = b1 * m1[i] + (1.f - b1) * gr;
  const float b = b2 * m2[i] + (1.f - b2) * gr * gr;
  m1[i] = a;
  m2[i] = b;
  const float v = w[i] - lr * (a / bc1) / (sqrtf(b / bc2) + eps);
  w[i] = v;
  const int r = (int)(i / cols), c = (int)(i % cols);
  if (w16) w16[(size_t)r * ld16 + c] = __float2bfloat16(v);
  if (wt16) wt16[(size_t)c * ldt + r] = __float2bfloat16(v);
}

// ------------------------------------------------------------ host side
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static int get_encode() {
  if (g_encode) return SKG_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  SKG_CUDA(cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q));
  if (!fn || q != cudaDriverEntryPointSuccess) return fail(SKG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return SKG_OK;
}

// 2-D BF16 map over a [rows][ld] row-major matrix (cols valid), boxes of 64 x box_rows, 128-byte swizzle
static int make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
  SKG_TRY(get_encode());
  if ((reinterpret_cast<uintptr_t>(base) & 15) || ((ld * 2) & 15))
    return fail(SKG_ERR_ARG, "GEMM operand must be 16-byte aligned with a row pitch multiple of 16 bytes");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)kBlkK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(SKG_ERR_ARG, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return SKG_OK;
}

}  // namespace skg

using namespace skg;

extern "C" {

// C[R x Nc] = A[R x L] B[Nc x L]^T on tcgen05 (see the file comment); A, B BF16 with
// row pitches lda, ldb (elements); L a multiple of 64; Nc a multiple of 16 <= 256.
// splits > 1 writes per-split FP32 partials [splits][R][ld_out] (EPI_F32 only).
int skg_mlp_gemm(const void* A, int64_t R, int64_t lda, const void* B, int Nc, int64_t ldb, int64_t L, int splits,
                 int epi, const float* bias, float* out_f32, void* out_z, void* out_h, int Nstore, int ld_out,
                 int* err, void* stream) {
  if (R <= 0 || Nc < 16 || Nc > 256 || (Nc % 16) || L <= 0 || (L % kBlkK) || splits < 1 || Nstore > Nc || !err)
    return fail(SKG_ERR_ARG, "mlp_gemm: bad shape R=%lld Nc=%d L=%lld splits=%d", (long long)R, Nc, (long long)L,
                splits);
  if (splits > 1 && epi != EPI_F32) return fail(SKG_ERR_ARG, "mlp_gemm: split-K needs the FP32 epilogue");
  const int kblocks = (int)(L / kBlkK);
  const int kbps = (kblocks + splits - 1) / splits;
  const size_t smem = 1024 + (size_t)kbps * (kTileM * 128 + (size_t)Nc * 128);
  if (smem > kGemmSmemMax)
    return fail(SKG_ERR_CAPACITY, "mlp_gemm: %d reduction blocks per CTA need %zu bytes of shared memory", kbps, smem);
  CUtensorMap mA, mB;
  SKG_TRY(make_map(&mA, A, R, L, lda, kTileM));
  SKG_TRY(make_map(&mB, B, Nc, L, ldb, Nc));
  static bool attr = false;
  if (!attr) {
    SKG_CUDA(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmemMax));
    attr = true;
  }
  GemmArgs g{};
  g.R = (int)R; g.Nc = Nc; g.Nstore = Nstore; g.kblocks = kblocks; g.kb_per_split = kbps; g.epi = epi;
  g.bias = bias; g.out_f32 = out_f32; g.out_z = (__nv_bfloat16*)out_z; g.out_h = (__nv_bfloat16*)out_h;
  g.ld_out = ld_out; g.err = err;
  dim3 grid((unsigned)((R + kTileM - 1) / kTileM), (unsigned)splits);
  k_gemm_tc<<<grid, 256, smem, as_stream(stream)>>>(mA, mB, g);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_mlp_gelu_backward(const void* dH, const void* Z, int64_t n, void* dZ, void* stream) {
  if (n <= 0) return SKG_OK;
  k_gelu_backward<<<blocks_for(n), kBlock, 0, as_stream(stream)>>>((const __nv_bfloat16*)dH, (const __nv_bfloat16*)Z,
                                                                    n, (__nv_bfloat16*)dZ);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_mlp_transpose(const void* in, int rows, int cols, int ld_in, void* out, int ld_out, void* stream) {
  if (rows <= 0 || cols <= 0) return SKG_OK;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  k_transpose_bf16<<<grid, block, 0, as_stream(stream)>>>((const __nv_bfloat16*)in, rows, cols, ld_in,
                                                          (__nv_bfloat16*)out, ld_out);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_mlp_reduce_splits(const float* part, int splits, int64_t n, float* out, void* stream) {
  if (n <= 0) return SKG_OK;
  k_reduce_splits<<<blocks_for(n), kBlock, 0, as_stream(stream)>>>(part, splits, n, out);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_mlp_colsum(const void* dZ, int rows, int cols, int ld, float* db, void* stream) {
  if (cols <= 0) return SKG_OK;
  k_colsum_bf16<<<cols, 256, 0, as_stream(stream)>>>((const __nv_bfloat16*)dZ, rows, cols, ld, db);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_mlp_mse(const float* y, int ld_y, const float* t, int rows, int cols, void* dy, int ld_dy, double* scratch,
                double* loss_h, void* stream) {
  // scratch: 2048 partial doubles, then a counter word and the result
  double* partials = scratch;
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + 2048);
  double* out = scratch + 2050;
  cudaStream_t s = as_stream(stream);
  SKG_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), s));
  int64_t n = (int64_t)rows * cols;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  if (blocks < 1) blocks = 1;
  k_mse<<<blocks, 256, 0, s>>>(y, ld_y, t, rows, cols, (__nv_bfloat16*)dy, ld_dy, partials, counter, out);
  SKG_LAUNCHED();
  if (loss_h) {
    SKG_CUDA(cudaMemcpyAsync(loss_h, out, sizeof(double), cudaMemcpyDeviceToHost, s));
    SKG_CUDA(cudaStreamSynchronize(s));
    *loss_h /= (double)n;
  }
  return SKG_OK;
}

int skg_mlp_adam(float* w, const float* grad, float* m1, float* m2, int rows, int cols, float lr, float b1, float b2,
                 float eps, int step, void* w16, int ld16, void* wt16, int ldt, void* stream) {
  if (rows <= 0 || cols <= 0 || step < 1) return fail(SKG_ERR_ARG, "mlp_adam: bad arguments");
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  const int64_t n = (int64_t)rows * cols;
  k_adam<<<blocks_for(n), kBlock, 0, as_stream(stream)>>>(w, grad, m1, m2, rows, cols, lr, b1, b2, eps, bc1, bc2,
                                                          (__nv_bfloat16*)w16, ld16, (__nv_bfloat16*)wt16, ldt);
  SKG_LAUNCHED();
  return SKG_OK;
}

}  // extern "C"

// ------------------------------------------------------- warm-start features
namespace skg {

constexpr int kFeatCols = 64;   // 15 per-vertex features + 32 context + zero pad
constexpr int kVertFeat = 15;
constexpr int kCtxFeat = 32;

// per-vertex features (rows of [n][64], BF16), in units that keep them O(1):
//   X / 1 m, u / 0.1 m, (u - u_prev) / s, corr / s, f_ext / (m * 9.8)
// with s = 9.8 dt^2 and corr the previous step's Newton correction u_t - u_tilde_t.
__global__ void k_vertex_features(const double* __restrict__ X, const double* __restrict__ u,
                                  const double* __restrict__ u_prev, const double* __restrict__ corr,
                                  const double* __restrict__ f_ext, const double* __restrict__ mass, double dt,
                                  int64_t n, float* __restrict__ vf) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  const double s = 9.8 * dt * dt;
  float* o = vf + (size_t)v * 16;
  const double m = mass[v] > 0.0 ? mass[v] : 1.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int64_t k = 3 * v + c;
    o[c] = (float)X[k];
    o[3 + c] = (float)(u[k] * 10.0);
    o[6 + c] = (float)((u[k] - u_prev[k]) / s);
    o[9 + c] = (float)(corr ? corr[k] / s : 0.0);
    o[12 + c] = (float)(f_ext[k] / (m * 9.8));
  }
  o[15] = 0.f;
}

// per-instance context: mean of the vertex features (15), log10 E - 6, (nu - 0.4) * 10,
// size in cells (3, scaled), zero pad to 32.  One CTA per instance, fixed order.
__global__ void __launch_bounds__(256) k_instance_context(const float* __restrict__ vf, const int32_t* __restrict__ rows,
                                                          const float* __restrict__ inst_scalars,
                                                          float* __restrict__ ctx) {
  const int inst = blockIdx.x;
  double acc[kVertFeat];
#pragma unroll
  for (int k = 0; k < kVertFeat; ++k) acc[k] = 0.0;
  const int r0 = rows[inst], r1 = rows[inst + 1];
  for (int v = r0 + threadIdx.x; v < r1; v += blockDim.x)
#pragma unroll
    for (int k = 0; k < kVertFeat; ++k) acc[k] += vf[(size_t)v * 16 + k];
  block_sum<kVertFeat, 256>(acc);
  if (threadIdx.x == 0) {
    float* o = ctx + (size_t)inst * kCtxFeat;
    const double inv = r1 > r0 ? 1.0 / (r1 - r0) : 0.0;
    for (int k = 0; k < kVertFeat; ++k) o[k] = (float)(acc[k] * inv);
    for (int k = 0; k < 5; ++k) o[kVertFeat + k] = inst_scalars[inst * 5 + k];
    for (int k = kVertFeat + 5; k < kCtxFeat; ++k) o[k] = 0.f;
  }
}

// rows of the MLP input: [vertex features | instance context | 0], BF16
__global__ void k_assemble_features(const float* __restrict__ vf, const float* __restrict__ ctx,
                                    const int32_t* __restrict__ vert_inst, int64_t n,
                                    __nv_bfloat16* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * kFeatCols) return;
  const int64_t v = i / kFeatCols;
  const int c = (int)(i % kFeatCols);
  float x = 0.f;
  if (c < kVertFeat) x = vf[(size_t)v * 16 + c];
  else if (c < kVertFeat + kCtxFeat) x = ctx[(size_t)vert_inst[v] * kCtxFeat + (c - kVertFeat)];
  out[i] = __float2bfloat16(x);
}

// u_warm = u_tilde + corr + s * pred (pinned DOFs stay at rest), s = 9.8 dt^2: the network
// refines the second-order extrapolation u_tilde + corr (corr = previous Newton correction)
__global__ void k_apply_prediction(const double* __restrict__ u_tilde, const double* __restrict__ corr,
                                   const float* __restrict__ pred, int ld_pred, const uint8_t* __restrict__ pinned,
                                   double dt, int64_t n, double* __restrict__ uw) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  const double s = 9.8 * dt * dt;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int64_t k = 3 * v + c;
    const double base = u_tilde[k] + (corr ? corr[k] : 0.0);
    uw[k] = (pinned && pinned[k]) ? u_tilde[k] : base + (pred ? s * (double)pred[(size_t)v * ld_pred + c] : 0.0);
  }
}

// target rows: (u_next - u_tilde - corr) / s, FP32 [n][3]
__global__ void k_targets(const double* __restrict__ u_next, const double* __restrict__ u_tilde,
                          const double* __restrict__ corr, double dt, int64_t n, float* __restrict__ t) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  const double s = 9.8 * dt * dt;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int64_t k = 3 * v + c;
    t[(size_t)v * 3 + c] = (float)((u_next[k] - u_tilde[k] - (corr ? corr[k] : 0.0)) / s);
  }
}

}  // namespace skg

extern "C" {

// MLP input rows [n][64] (BF16) for one frame of a batch of instances; vf (n x 16 f32),
// ctx (n_inst x 32 f32) are scratch; inst_scalars (n_inst x 5): log10 E - 6, (nu - 0.4) 10, size x3.
int skg_warmstart_features(const double* X, const double* u, const double* u_prev, const double* corr,
                           const double* f_ext, const double* mass, double dt, int64_t n, const int32_t* inst_rows,
                           const int32_t* vert_inst, int n_inst, const float* inst_scalars, float* vf, float* ctx,
                           void* out, void* stream) {
  if (n <= 0 || n_inst <= 0) return fail(SKG_ERR_ARG, "warmstart_features: empty");
  cudaStream_t s = as_stream(stream);
  k_vertex_features<<<blocks_for(n), kBlock, 0, s>>>(X, u, u_prev, corr, f_ext, mass, dt, n, vf);
  k_instance_context<<<n_inst, 256, 0, s>>>(vf, inst_rows, inst_scalars, ctx);
  k_assemble_features<<<blocks_for(n * kFeatCols), kBlock, 0, s>>>(vf, ctx, vert_inst, n, (__nv_bfloat16*)out);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_warmstart_apply(const double* u_tilde, const double* corr, const float* pred, int ld_pred,
                        const uint8_t* pinned, double dt, int64_t n, double* u_warm, void* stream) {
  if (n <= 0) return SKG_OK;
  k_apply_prediction<<<blocks_for(n), kBlock, 0, as_stream(stream)>>>(u_tilde, corr, pred, ld_pred, pinned, dt, n,
                                                                       u_warm);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_warmstart_targets(const double* u_next, const double* u_tilde, const double* corr, double dt, int64_t n,
                          float* t, void* stream) {
  if (n <= 0) return SKG_OK;
  k_targets<<<blocks_for(n), kBlock, 0, as_stream(stream)>>>(u_next, u_tilde, corr, dt, n, t);
  SKG_LAUNCHED();
  return SKG_OK;
}

}  // extern "C"
