// PCG on thread-block clusters, for systems small enough that grid-wide
// synchronisation and L2 round trips dominate a PCG iteration (on the
// 12,288-tet beam the grid-persistent kernel spends 24 of 43 cycles per
// instruction at grid barriers and moves its whole working set through L2).
//
// Layout: the cluster's CTAs split the block rows into contiguous ranges.
// Each CTA keeps the PCG vectors of its own rows in shared memory: z and two
// buffers of the search direction p interleaved per row (so one address
// reaches all three), x, r, q = A p and the 3x3 block-Jacobi inverses.  The
// SpMV gathers neighbouring rows' z and previous p from the owning CTA through
// distributed shared memory (ld.shared::cluster), or from its own shared
// memory for its own rows.  When a CTA's rows fit, their block values are
// staged in shared memory once per solve (the matrix is constant during a
// solve) with the column index replaced by the shared::cluster address of the
// column's z|p row (mapa), so an iteration touches no global memory.
//
// One iteration has two cluster barriers, one per dependent reduction
// (p.q, then r.z and r.r): the direction p_k = z_k + beta_k p_{k-1} is never
// published before the SpMV that uses it; every CTA rebuilds the p_j it
// gathers from z_j and p_{k-1, j} with the same rounding as the owner, which
// writes p_k into the other buffer.  This is the standard PCG recurrence, not
// a reformulation, so the iterates equal the three-barrier form's.
//
// Dot products: FP64 for FP64 systems.  For FP32 systems each thread
// accumulates the exact FP32 products (fma splits each product into two
// floats) in a double-float pair with Knuth's TwoSum, and pairs are combined
// by TwoSum: a 48-bit significand, far beyond the FP32 vectors, at FP32
// instruction rates (the FP64 pipe of this part has 64-cycle dependent
// latency and 1/71 of the FP32 throughput).  Reductions run in a fixed order
// and every CTA sums all partials itself, so all CTAs hold bitwise the same
// scalars and take the same branches.
#pragma once

#include <cooperative_groups.h>

namespace skg {

namespace cgx = cooperative_groups;

constexpr int kClusterThreads = 512;
constexpr int kClusterWarps = kClusterThreads / 32;
constexpr int kClusterMax = 16;                 // non-portable cluster size
constexpr int kClusterSmemBudget = 220 * 1024;  // dynamic shared memory per CTA
// batched PCG defaults (measured on 512 beams of 324 to 13,056 block rows): the cluster size is
// the smallest of at least kClusterMinDefault CTAs whose per-CTA vectors take at most
// kClusterVecTarget bytes, the rest of the shared memory holding block records
constexpr int kClusterVecTarget = 170 * 1024;
constexpr int kClusterMinDefault = 4;
// shared-memory values per block row: z|p0|p1 (12), x (4), r (4), q (4), Jacobi inverse (9)
constexpr int kClusterVals = 33;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint32_t cluster_map(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ Vec3<float> ld_cluster3(uint32_t addr, float) {
  float a, b, c;
  [[maybe_unused]] float d;   // the record's fourth lane: padding
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(a), "=f"(b), "=f"(c), "=f"(d) : "r"(addr) : "memory");
  return {a, b, c};
}
__device__ __forceinline__ Vec3<double> ld_cluster3(uint32_t addr, double) {
  double a, b, c;
  [[maybe_unused]] double d;   // padding
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(a), "=d"(b) : "r"(addr) : "memory");
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(c), "=d"(d) : "r"(addr + 16) : "memory");
  return {a, b, c};
}
__device__ __forceinline__ Vec3<float> lds3(const unsigned char* p, float) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  return {a.x, a.y, a.z};
}
__device__ __forceinline__ Vec3<double> lds3(const unsigned char* p, double) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double b = reinterpret_cast<const double*>(p)[2];
  return {a.x, a.y, b};
}

// ---- dot-product accumulators ----------------------------------------------

template <typename R> struct Dacc;
template <> struct __align__(8) Dacc<double> { double v; };
template <> struct __align__(8) Dacc<float> { float hi, lo; };

__device__ __forceinline__ void dacc_zero(Dacc<double>& a) { a.v = 0.0; }
__device__ __forceinline__ void dacc_zero(Dacc<float>& a) { a.hi = 0.f; a.lo = 0.f; }

// Knuth's TwoSum: s + e == a + b exactly (explicit rounding: never contracted or reordered)
__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bv = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bv)), __fsub_rn(b, bv));
  return make_float2(s, e);
}
// (hi, lo) pairs: hi carries the running FP32 sum, lo the exact rounding errors of
// every addition into hi (Neumaier-style compensation), so hi + lo is the sum to
// about 2^-48 of the magnitudes summed
__device__ __forceinline__ Dacc<float> dacc_add(Dacc<float> a, Dacc<float> b) {
  const float2 s = two_sum(a.hi, b.hi);
  return {s.x, __fadd_rn(s.y, __fadd_rn(a.lo, b.lo))};
}
__device__ __forceinline__ Dacc<double> dacc_add(Dacc<double> a, Dacc<double> b) { return {a.v + b.v}; }

// a += x . y over three components; each product is split exactly by fma
__device__ __forceinline__ void dacc_dot3(Dacc<float>& a, Vec3<float> x, Vec3<float> y) {
  const float p0 = __fmul_rn(x.x, y.x), p1 = __fmul_rn(x.y, y.y), p2 = __fmul_rn(x.z, y.z);
  const float e0 = __fmaf_rn(x.x, y.x, -p0), e1 = __fmaf_rn(x.y, y.y, -p1), e2 = __fmaf_rn(x.z, y.z, -p2);
  const float2 s0 = two_sum(a.hi, p0);
  const float2 s1 = two_sum(s0.x, p1);
  const float2 s2 = two_sum(s1.x, p2);
  a.hi = s2.x;
  a.lo = __fadd_rn(a.lo, __fadd_rn(__fadd_rn(e0, __fadd_rn(e1, e2)), __fadd_rn(s0.y, __fadd_rn(s1.y, s2.y))));
}
__device__ __forceinline__ void dacc_dot3(Dacc<double>& a, Vec3<double> x, Vec3<double> y) {
  a.v = fma(x.z, y.z, fma(x.y, y.y, fma(x.x, y.x, a.v)));
}

__device__ __forceinline__ Dacc<float> dacc_shfl_down(Dacc<float> a, int o) {
  return {__shfl_down_sync(0xffffffffu, a.hi, o), __shfl_down_sync(0xffffffffu, a.lo, o)};
}
__device__ __forceinline__ Dacc<double> dacc_shfl_down(Dacc<double> a, int o) {
  return {__shfl_down_sync(0xffffffffu, a.v, o)};
}
__device__ __forceinline__ Dacc<float> dacc_bcast(Dacc<float> a) {
  return {__shfl_sync(0xffffffffu, a.hi, 0), __shfl_sync(0xffffffffu, a.lo, 0)};
}
__device__ __forceinline__ Dacc<double> dacc_bcast(Dacc<double> a) { return {__shfl_sync(0xffffffffu, a.v, 0)}; }

__device__ __forceinline__ void dacc_poison(Dacc<float>& a) { a.hi = __int_as_float(0x7fc00000); }
__device__ __forceinline__ void dacc_poison(Dacc<double>& a) { a.v = __longlong_as_double(0x7ff8000000000000ll); }
__device__ __forceinline__ double dacc_value(Dacc<float> a) { return double(a.hi) + double(a.lo); }
__device__ __forceinline__ double dacc_value(Dacc<double> a) { return a.v; }
// rounded to the working precision
__device__ __forceinline__ float dacc_r(Dacc<float> a) { return __fadd_rn(a.hi, a.lo); }
__device__ __forceinline__ double dacc_r(Dacc<double> a) { return a.v; }

__device__ __forceinline__ Dacc<float> ld_cluster_dacc(uint32_t addr, float) {
  float a, b;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(a), "=f"(b) : "r"(addr) : "memory");
  return {a, b};
}
__device__ __forceinline__ Dacc<double> ld_cluster_dacc(uint32_t addr, double) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return {v};
}

// tree sum over the first `width` lanes (a power of two) in a fixed order, result in lane 0
template <typename R, int W> __device__ __forceinline__ Dacc<R> dacc_tree(Dacc<R> a) {
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) a = dacc_add(a, dacc_shfl_down(a, o));
  return a;
}

// barrier over the cluster (a single-CTA "cluster" needs only the CTA barrier)
__device__ __forceinline__ void csync(cgx::cluster_group& cl, int csize) {
  if (csize > 1)
    cl.sync();
  else
    __syncthreads();
}

// ---- bulk copies into shared memory (TMA, non-tensor form) -------------------

constexpr int kRingMax = 8;                   // ring slots for streamed block records
// blocks per lane in flight in the SpMV (fewer for FP64 records, which take twice the registers)
template <typename R> constexpr int kUof = sizeof(R) == 4 ? 4 : 2;
constexpr int kWaitTries = 1 << 20;           // bound on mbarrier polls (each try_wait also blocks a while)

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// bounded wait for phase `parity` of the barrier to complete; false if it never did
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int tries = kWaitTries) {
  const uint32_t a = smem_addr(bar);
  for (int i = 0; i < tries; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok) : "r"(a), "r"(parity) : "memory");
    if (ok) return true;
  }
  return false;
}
// global -> this CTA's shared memory, completion counted on `bar` (16-byte aligned, size multiple of 16)
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// generic-proxy writes to global memory become visible to later bulk copies
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// ---- block records ------------------------------------------------------------

// Record slot 10 (a pad slot the assembly leaves zero) receives, at the start of
// each solve, the shared::cluster address of the z|p row of the block's column;
// slot 9 (the column) is left intact; slot 11 carries the column's two-level
// coarse word (aux1) when the per-instance coarse data is attached.
__device__ __forceinline__ Blk<float> ld_srec(const float* srec, int64_t i) {
  const float4* p = reinterpret_cast<const float4*>(srec) + 3 * i;
  const float4 a = p[0], b = p[1], c = p[2];
  return {{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x}, __float_as_int(c.z), 0u, __float_as_uint(c.w)};
}
__device__ __forceinline__ Blk<double> ld_srec(const double* srec, int64_t i) {
  const double2* p = reinterpret_cast<const double2*>(srec) + 6 * i;
  const double2 a = p[0], b = p[1], c = p[2], d = p[3], e = p[4], f = p[5];
  return {{a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, e.x}, (int)__double_as_longlong(f.x), 0u,
          (unsigned)__double_as_longlong(f.y)};
}
// the same from global memory with plain loads (the address slot was written in this kernel,
// so not through the read-only path)
__device__ __forceinline__ Blk<float> ld_grec(const float* rec, int64_t i) {
  const float4* p = reinterpret_cast<const float4*>(rec) + 3 * i;
  const float4 a = p[0], b = p[1], c = p[2];
  return {{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x}, __float_as_int(c.z), 0u, __float_as_uint(c.w)};
}
__device__ __forceinline__ Blk<double> ld_grec(const double* rec, int64_t i) {
  const double2* p = reinterpret_cast<const double2*>(rec) + 6 * i;
  const double2 a = p[0], b = p[1], c = p[2], d = p[3], e = p[4], f = p[5];
  return {{a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, e.x}, (int)__double_as_longlong(f.x), 0u,
          (unsigned)__double_as_longlong(f.y)};
}

// Shared memory the kernel needs for its vectors and local row offsets, per CTA.
__host__ __device__ inline int64_t cluster_vec_bytes(int64_t nbr, int csize, int rsize) {
  const int64_t rows_cap = (nbr + csize - 1) / csize;
  return ((rows_cap * kClusterVals * rsize + 15) & ~int64_t(15)) + ((4 * (rows_cap + 1) + 127) & ~int64_t(127));
}

struct ClusterPcgOut {
  int iters;
  int status;
  double rr, rz, bb;
};

// Static shared memory of a cluster PCG kernel.
template <typename R> struct ClusterShared {
  Dacc<R> pub[3][2];                  // CTA totals: [0] p.q, [1] r.z and r.r, [2] coarse (P^T r).e
  Dacc<R> wsum[2][kClusterWarps];     // warp totals
  uint64_t mbar[kRingMax];            // record ring (slot 0 alone when the records are resident)
  uint32_t zbase[kClusterMax];        // shared::cluster address of each rank's z|p rows
  int32_t rowb[kClusterMax + 1];      // first local row of each rank
  int32_t maxblk;                     // most blocks in one chunk of rows
  int32_t err;                        // a bounded wait gave up
};

// Totals over every thread of the cluster of NV accumulators, returned to every
// thread, in a fixed order (all CTAs get bitwise the same values): warp trees,
// the CTA's warp totals by warp 0, then each CTA's total read by every warp
// after the cluster barrier.  The barrier also orders the shared-memory writes
// of the phase before the call before everything after it.  A pub slot is
// rewritten only after the next cluster barrier.
template <typename R, int NV>
__device__ __forceinline__ void cluster_total(cgx::cluster_group& cl, int csize, Dacc<R> (&v)[NV], Dacc<R>* pub,
                                              Dacc<R> (*wsum)[kClusterWarps]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const Dacc<R> w = dacc_tree<R, 32>(v[k]);
    if (lane == 0) wsum[k][wid] = w;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      Dacc<R> x;
      dacc_zero(x);
      if (lane < kClusterWarps) x = wsum[k][lane];
      x = dacc_tree<R, kClusterWarps>(x);
      if (lane == 0) pub[k] = x;
    }
  }
  csync(cl, csize);
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    Dacc<R> y;
    dacc_zero(y);
    if (lane < csize) y = csize > 1 ? ld_cluster_dacc(cluster_map(smem_addr(pub + k), lane), R(0)) : pub[k];
    v[k] = dacc_bcast(dacc_tree<R, kClusterMax>(y));
  }
}

// the search direction p = z + beta p_prev, rounded identically wherever it is formed
__device__ __forceinline__ float pdir(float z, float pp, float beta) { return __fmaf_rn(beta, pp, z); }
__device__ __forceinline__ double pdir(double z, double pp, double beta) { return __fma_rn(beta, pp, z); }
template <typename R> __device__ __forceinline__ Vec3<R> pdir3(Vec3<R> z, Vec3<R> pp, R beta) {
  return {pdir(z.x, pp.x, beta), pdir(z.y, pp.y, beta), pdir(z.z, pp.z, beta)};
}

// owner rank of local row c (rowb: first row of each rank)
__device__ __forceinline__ int cl_owner(int c, const int32_t* rowb, int csize, float inv) {
  int o = min(csize - 1, (int)((float)c * inv));
  while (o > 0 && c < rowb[o]) --o;
  while (o < csize - 1 && c >= rowb[o + 1]) ++o;
  return o;
}

// Coarse correction of one instance on the calling cluster: e = A_c^-1 P^T r
// (the instance's dense block Mi, np x np), one row per warp over the cluster's
// warps.  Every CTA stages P^T r (fixed point -> float) into srcf; each row of e
// is stored into every CTA's copy sce over DSMEM (visible after the next
// cluster barrier); pc += (P^T r).e over the rows this CTA computed.
template <typename R>
__device__ __forceinline__ void coarse_product_cluster(int crank, int csize, const float* Mi, int nc, int np,
                                                       const unsigned long long* rc, float inv_scale, float* sce,
                                                       float* srcf, Dacc<R>& pc) {
  const int tid = threadIdx.x, lane = tid & 31, wpb = blockDim.x >> 5;
#pragma unroll 4
  for (int i = tid; i < np; i += blockDim.x)
    srcf[i] = i < nc ? __ll2float_rn((long long)__ldcg(rc + i)) * inv_scale : 0.f;
  __syncthreads();
  const float4* r4 = reinterpret_cast<const float4*>(srcf);
  for (int row = crank * wpb + (tid >> 5); row < nc; row += csize * wpb) {
    const float4* Mr = reinterpret_cast<const float4*>(Mi + (int64_t)row * np);
    float sacc = 0.f;
#pragma unroll 4
    for (int j = lane; j < (np >> 2); j += 32) {
      const float4 m = __ldcg(Mr + j), x = r4[j];
      sacc = fmaf(m.x, x.x, fmaf(m.y, x.y, fmaf(m.z, x.z, fmaf(m.w, x.w, sacc))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
    if (csize == 1) {
      if (lane == 0) sce[row] = sacc;
    } else if (lane < csize) {
      const uint32_t a = cluster_map(smem_addr(sce + row), lane);
      asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(sacc) : "memory");
    }
    if (lane == 0) dacc_dot3(pc, Vec3<R>{R(srcf[row]), R(0), R(0)}, Vec3<R>{R(sacc), R(0), R(0)});
  }
}

// Solve the system of block rows [gbase, gbase + nbr) (its columns lie in the
// same range) on the calling cluster.  b: right-hand side (3n, simkit layout,
// FP64) scaled by bsign, pinned DOFs forced to zero; x written to xout
// (padded, global rows).  rec: the block records of A (slot 10 of the own rows'
// records is written).  Every thread of every CTA of the cluster must call it;
// it ends with a cluster barrier, so shared memory may be reused after.
//
// Block records reach shared memory by bulk copies in chunks of one pass of
// rows: all at once when the CTA's records fit beside its vectors (then an
// iteration reads no global memory), else through a ring of kRingMax slots at
// most, refilled while later chunks (and, at the end of an iteration, the
// reductions and vector updates) are processed.  Without room for two slots
// the records are read from global memory.
template <typename R, int G, bool CO>
__device__ __forceinline__ ClusterPcgOut cluster_pcg_range(
    cgx::cluster_group& cl, const Bsr<R>& A, R* rec, int64_t gbase, int64_t nbr, const double* __restrict__ b,
    double bsign, const uint8_t* __restrict__ pinned, R* __restrict__ xout, double rtol, int max_iter,
    int smem_bytes, unsigned char* smem_raw, ClusterShared<R>& sh, const CoarseDev& cd, int inst) {
  const int crank = (int)cl.block_rank();
  const int csize = (int)cl.num_blocks();
  const int64_t r0 = gbase + nbr * crank / csize;
  const int64_t r1 = gbase + nbr * (crank + 1) / csize;
  const int64_t rows_cap = (nbr + csize - 1) / csize;
  const int nr = (int)(r1 - r0);
  constexpr int ZP = 12;  // z | p0 | p1, 4 values each
  constexpr uint32_t kRowBytes = ZP * sizeof(R);
  constexpr uint32_t kRecBytes = kRec * sizeof(R);
  R* szp = reinterpret_cast<R*>(smem_raw);
  R* sx = szp + ZP * rows_cap;
  R* sr = sx + 4 * rows_cap;
  R* sq = sr + 4 * rows_cap;
  R* sj = sq + 4 * rows_cap;
  int32_t* srp = reinterpret_cast<int32_t*>(smem_raw + ((rows_cap * kClusterVals * (int64_t)sizeof(R) + 15) & ~int64_t(15)));
  const int64_t vec_bytes = cluster_vec_bytes(nbr, csize, (int)sizeof(R));
  R* srec = reinterpret_cast<R*>(smem_raw + vec_bytes);
  const unsigned char* zp_local = smem_raw;
  const uint32_t my_cbase = csize > 1 ? cluster_map(smem_addr(szp), crank) : smem_addr(szp);
  const uint32_t my_span = (uint32_t)(nr * kRowBytes);
  const int tid = threadIdx.x;
  const int rows_per_pass = blockDim.x / G;
  // two-level coarse data of this instance (per-instance form); the instance's e and
  // P^T r live past the smem_bytes the vectors and records may use
  int cnc = 0, cnp = 0;
  const float* cM = nullptr;
  unsigned long long* crc = nullptr;
  bool con = false;
  float* sce = nullptr;
  float* srcf = nullptr;
  if constexpr (CO) {
    const int ag0 = cd.inst_agg[inst];
    cnc = 6 * (cd.inst_agg[inst + 1] - ag0);
    cnp = ((cnc + 31) / 32) * 32;
    cM = cd.M + cd.inst_moff[inst];
    crc = cd.rc + 6 * (int64_t)ag0;
    con = cd.ok[inst] != 0;
    sce = reinterpret_cast<float*>(smem_raw + smem_bytes);
    srcf = sce + kCoarseInstMax;
  }

  if (tid < csize) sh.zbase[tid] = csize > 1 ? cluster_map(smem_addr(szp), tid) : smem_addr(szp);
  if (tid <= csize) sh.rowb[tid] = (int32_t)(nbr * tid / csize);
  if (tid == 0) {
    sh.maxblk = 0;
    sh.err = 0;
  }
  const float inv = (float)csize / (float)nbr;
  const int b0 = __ldg(A.rowptr + r0);
  const int nblk = __ldg(A.rowptr + r1) - b0;
  for (int i = tid; i <= nr; i += blockDim.x) srp[i] = __ldg(A.rowptr + r0 + i) - b0;
  __syncthreads();
  // gather addresses into slot 10 of the own rows' records; chunk sizes
  for (int i = tid; i < nblk; i += blockDim.x) {
    R* rc = rec + (int64_t)kRec * (b0 + i);
    const int lc = bits_col(rc[9]) - (int)gbase;
    const int o = cl_owner(lc, sh.rowb, csize, inv);
    rc[10] = col_bits((int)(sh.zbase[o] + (uint32_t)(lc - sh.rowb[o]) * kRowBytes), R(0));
  }
  const int nchunks = (nr + rows_per_pass - 1) / rows_per_pass;
  {
    int mb = 0;
    for (int c = tid; c < nchunks; c += blockDim.x)
      mb = max(mb, srp[min(nr, (c + 1) * rows_per_pass)] - srp[c * rows_per_pass]);
    if (mb > 0) atomicMax(&sh.maxblk, mb);
  }
  fence_proxy_async();
  __syncthreads();
  const int64_t avail = (int64_t)smem_bytes - vec_bytes;
  const bool resident = (int64_t)nblk * kRecBytes <= avail;
  const uint32_t slot_bytes = (uint32_t)(((int64_t)sh.maxblk * kRecBytes + 127) & ~int64_t(127));
  int ring = 0;
  if (!resident && nchunks > 0) {
    const int64_t d = avail / (slot_bytes > 0 ? slot_bytes : 1);
    ring = (int)(d > kRingMax ? kRingMax : d);
    if (ring < 2) ring = 0;
  }
  auto chunk_rows = [&](int c, int& lo, int& hi) {
    lo = c * rows_per_pass;
    hi = min(nr, lo + rows_per_pass);
  };
  // issue j-th ring fill: chunk j mod nchunks into slot j mod ring
  auto issue = [&](int j) {
    const int c = j % nchunks, sl = j % ring;
    int lo, hi;
    chunk_rows(c, lo, hi);
    const uint32_t bytes = (uint32_t)(srp[hi] - srp[lo]) * kRecBytes;
    unsigned char* dst = reinterpret_cast<unsigned char*>(srec) + (int64_t)sl * slot_bytes;
    mbar_expect_tx(&sh.mbar[sl], bytes);
    bulk_copy(dst, rec + (int64_t)kRec * (b0 + srp[lo]), bytes, &sh.mbar[sl]);
  };
  if (tid == 0) {
    if (resident && nblk > 0) {
      mbar_init(&sh.mbar[0], 1);
      fence_mbar_init();
      mbar_expect_tx(&sh.mbar[0], (uint32_t)nblk * kRecBytes);
      for (int c = 0; c < nchunks; ++c) {
        int lo, hi;
        chunk_rows(c, lo, hi);
        bulk_copy(reinterpret_cast<unsigned char*>(srec) + (int64_t)srp[lo] * kRecBytes,
                  rec + (int64_t)kRec * (b0 + srp[lo]), (uint32_t)(srp[hi] - srp[lo]) * kRecBytes, &sh.mbar[0]);
      }
    } else if (ring) {
      for (int k = 0; k < ring; ++k) mbar_init(&sh.mbar[k], 1);
      fence_mbar_init();
      for (int j = 0; j < ring; ++j) issue(j);
    }
  }
  // init: x = 0, r = bsign * b (pinned -> 0), z = Jinv r, p_{-1} = 0
  Dacc<R> s2[2];
  dacc_zero(s2[0]);
  dacc_zero(s2[1]);
  for (int i = tid; i < nr; i += blockDim.x) {
    const int64_t g = r0 + i;
    R rv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double bb = bsign * b[3 * g + c];
      if (pinned && pinned[3 * g + c]) bb = 0.0;
      rv[c] = R(bb);
    }
    R jl[9];
#pragma unroll
    for (int m = 0; m < 9; ++m) {
      jl[m] = A.jinv[9 * g + m];
      sj[9 * i + m] = jl[m];
    }
    const Vec3<R> z{jl[0] * rv[0] + jl[1] * rv[1] + jl[2] * rv[2], jl[3] * rv[0] + jl[4] * rv[1] + jl[5] * rv[2],
                    jl[6] * rv[0] + jl[7] * rv[1] + jl[8] * rv[2]};
    R* zr = szp + ZP * i;
    zr[0] = z.x; zr[1] = z.y; zr[2] = z.z; zr[3] = R(0);
    zr[8] = R(0); zr[9] = R(0); zr[10] = R(0); zr[11] = R(0);
    R* pr = sr + 4 * i;
    pr[0] = rv[0]; pr[1] = rv[1]; pr[2] = rv[2]; pr[3] = R(0);
    R* px = sx + 4 * i;
    px[0] = px[1] = px[2] = px[3] = R(0);
    const Vec3<R> r3{rv[0], rv[1], rv[2]};
    dacc_dot3(s2[0], r3, z);
    dacc_dot3(s2[1], r3, r3);
  }
  cluster_total<R, 2>(cl, csize, s2, sh.pub[1], sh.wsum);
  Dacc<R> rz = s2[0];
  double rr = dacc_value(s2[1]);
  const double bb = rr;
  double rr_prev = rr;
  if (CO && con && bb > 0.0) {
    // coarse part of z_0 = D^-1 r_0 + P e_0
    const float sc = coarse_scale(rr_prev);
    for (int base = tid & ~31; base < nr; base += blockDim.x) {
      const int i = base + (tid & 31);
      const bool ok = i < nr;
      const R* rp = sr + 4 * (ok ? i : 0);
      coarse_restrict(cd, ok, r0 + i, float(rp[0]), float(rp[1]), float(rp[2]), sc);
    }
    csync(cl, csize);
    Dacc<R> pc[1];
    dacc_zero(pc[0]);
    coarse_product_cluster<R>(crank, csize, cM, cnc, cnp, crc, 1.f / sc, sce, srcf, pc[0]);
    cluster_total<R, 1>(cl, csize, pc, sh.pub[2], sh.wsum);
    rz = dacc_add(rz, pc[0]);
    if (crank == 0)
      for (int i = tid; i < cnc; i += blockDim.x) crc[i] = 0ull;
  }
  const double tol2 = rtol * rtol * bb;
  bool done = rr <= tol2 || bb == 0.0 || max_iter <= 0;
  // the per-iteration stop test in the working precision (FP64 compares cost a 64-cycle
  // dependent latency each on this part); a threshold below the FP32 range keeps its sign
  R tol2r = R(tol2);
  if (tol2 > 0.0 && !(tol2r > R(0))) tol2r = R(1e-45f);
  Dacc<R> rr_acc = s2[1];
  int it = 0, status = 0;
  const int lane = tid & (G - 1);
  const int row_off = (tid >> 5) * (32 / G) + ((tid & 31) / G);
  R beta = R(0);
  int cur = 0;        // p_k goes to buffer cur, p_{k-1} is in buffer cur ^ 1
  int consumed = 0;   // ring fills consumed so far
  bool waited_resident = false;
  while (!done) {
    const uint32_t po = (uint32_t)(4 * (1 + (cur ^ 1)) * sizeof(R));  // byte offset of p_{k-1} in a z|p row
    const int pn = 4 * (1 + cur);
    auto gather = [&](uint32_t caddr, uint32_t cword) -> Vec3<R> {
      const uint32_t d = caddr - my_cbase;
      Vec3<R> z, pp;
      if (d < my_span) {
        z = lds3(zp_local + d, R(0));
        pp = lds3(zp_local + d + po, R(0));
      } else {
        z = ld_cluster3(caddr, R(0));
        pp = ld_cluster3(caddr + po, R(0));
      }
      if (CO && con) {
        const Vec3<float> pe = prolong_word(sce, cword);
        z = {z.x + R(pe.x), z.y + R(pe.y), z.z + R(pe.z)};
      }
      return pdir3(z, pp, beta);
    };
    // q = A p_k on own rows; p_k written for own rows; partial p.q
    Dacc<R> pq[1];
    dacc_zero(pq[0]);
    bool lost = false;
    if (resident && nblk > 0 && !waited_resident) {
      lost = !mbar_wait(&sh.mbar[0], 0);
      waited_resident = true;
    }
    for (int c = 0; c < nchunks; ++c) {
      const R* base = srec;  // records of the chunk, indexed by block offset within the CTA
      if (ring) {
        const int sl = consumed % ring;
        if (!mbar_wait(&sh.mbar[sl], (uint32_t)((consumed / ring) & 1))) lost = true;
        int lo, hi;
        chunk_rows(c, lo, hi);
        base = reinterpret_cast<const R*>(reinterpret_cast<const unsigned char*>(srec) + (int64_t)sl * slot_bytes) -
               (int64_t)kRec * srp[lo];
      }
      const int li = c * rows_per_pass + row_off;
      const bool valid = li < nr;
      int rp = 0, K = 0;
      if (valid) {
        rp = srp[li];
        K = srp[li + 1] - rp;
      }
      // kU blocks per lane per round, all loads issued before the products
      constexpr int kU = kUof<R>;
      R a0 = 0, a1 = 0, a2 = 0;
      for (int k0 = lane; k0 < K; k0 += kU * G) {
        Blk<R> bk[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int k = k0 + u * G;
          if (k < K) bk[u] = (resident || ring) ? ld_srec(base, rp + k) : ld_grec(rec, b0 + rp + k);
        }
        Vec3<R> v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u)
          if (k0 + u * G < K) v[u] = gather((uint32_t)bk[u].col, bk[u].aux1);
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          if (k0 + u * G < K) {
            a0 += bk[u].m[0] * v[u].x + bk[u].m[1] * v[u].y + bk[u].m[2] * v[u].z;
            a1 += bk[u].m[3] * v[u].x + bk[u].m[4] * v[u].y + bk[u].m[5] * v[u].z;
            a2 += bk[u].m[6] * v[u].x + bk[u].m[7] * v[u].y + bk[u].m[8] * v[u].z;
          }
        }
      }
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o, G);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o, G);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o, G);
      }
      if (lane == 0 && valid) {
        R* zr = szp + ZP * li;
        const int pold = 12 - pn;  // the other p buffer
        Vec3<R> zo{zr[0], zr[1], zr[2]};
        if (CO && con) {
          const Vec3<float> pe = prolong_word(sce, __ldg(cd.colpack + r0 + li));
          zo = {zo.x + R(pe.x), zo.y + R(pe.y), zo.z + R(pe.z)};
        }
        const Vec3<R> p = pdir3(zo, Vec3<R>{zr[pold], zr[pold + 1], zr[pold + 2]}, beta);
        zr[pn] = p.x; zr[pn + 1] = p.y; zr[pn + 2] = p.z; zr[pn + 3] = R(0);
        R* q = sq + 4 * li;
        q[0] = a0; q[1] = a1; q[2] = a2;
        dacc_dot3(pq[0], p, Vec3<R>{a0, a1, a2});
      }
      if (ring) {
        __syncthreads();  // every thread is done with the slot
        if (tid == 0) issue(consumed + ring);
        ++consumed;
      }
    }
    if (lost) {  // a copy never landed: poison the reduction so every CTA stops here
      sh.err = 1;
      dacc_poison(pq[0]);
    }
    cluster_total<R, 1>(cl, csize, pq, sh.pub[0], sh.wsum);
    const R pqr = dacc_r(pq[0]);
    if (!(pqr > R(0)) || !isfinite(pqr)) {
      status = isfinite(pqr) ? 0 : SKG_ERR_NONFINITE;
      break;
    }
    const R a = dacc_r(rz) / pqr;
    Dacc<R> u2[2];
    dacc_zero(u2[0]);
    dacc_zero(u2[1]);
    const float csc = CO ? coarse_scale(rr_prev) : 1.f;
    for (int base = tid & ~31; base < nr; base += blockDim.x) {   // warp-uniform trip count
      const int i = base + (tid & 31);
      Vec3<R> rn{R(0), R(0), R(0)};
      if (i < nr) {
        R* x = sx + 4 * i;
        R* r = sr + 4 * i;
        R* zr = szp + ZP * i;
        const R* p = zr + pn;
        const R* q = sq + 4 * i;
        const R* J = sj + 9 * i;
        x[0] += a * p[0];
        x[1] += a * p[1];
        x[2] += a * p[2];
        rn = Vec3<R>{r[0] - a * q[0], r[1] - a * q[1], r[2] - a * q[2]};
        r[0] = rn.x; r[1] = rn.y; r[2] = rn.z;
        const Vec3<R> z{J[0] * rn.x + J[1] * rn.y + J[2] * rn.z, J[3] * rn.x + J[4] * rn.y + J[5] * rn.z,
                        J[6] * rn.x + J[7] * rn.y + J[8] * rn.z};
        zr[0] = z.x; zr[1] = z.y; zr[2] = z.z;
        dacc_dot3(u2[0], rn, z);
        dacc_dot3(u2[1], rn, rn);
      }
      if (CO && con) coarse_restrict(cd, i < nr, r0 + i, float(rn.x), float(rn.y), float(rn.z), csc);
    }
    cluster_total<R, 2>(cl, csize, u2, sh.pub[1], sh.wsum);
    ++it;
    rr_acc = u2[1];
    const R rrr = dacc_r(u2[1]);
    const Dacc<R> rz_old = rz;
    rz = u2[0];
    if (!isfinite(rrr)) {
      status = SKG_ERR_NONFINITE;
      break;
    }
    rr_prev = dacc_value(u2[1]);
    if (rrr <= tol2r || it >= max_iter) break;
    if (CO && con) {
      Dacc<R> pc[1];
      dacc_zero(pc[0]);
      coarse_product_cluster<R>(crank, csize, cM, cnc, cnp, crc, 1.f / csc, sce, srcf, pc[0]);
      cluster_total<R, 1>(cl, csize, pc, sh.pub[2], sh.wsum);
      rz = dacc_add(rz, pc[0]);
      // read by every CTA before that barrier; next accumulated after the next one
      if (crank == 0)
        for (int i = tid; i < cnc; i += blockDim.x) crc[i] = 0ull;
    }
    beta = dacc_r(rz) / dacc_r(rz_old);
    cur ^= 1;
  }
  if (CO && con) {
    // the last restriction is never used: leave the instance's residual at zero for the next solve
    csync(cl, csize);
    if (crank == 0)
      for (int i = tid; i < cnc; i += blockDim.x) crc[i] = 0ull;
  }
  // solution to global memory (padded, the layout the line search reads)
  for (int i = tid; i < nr; i += blockDim.x) {
    const R* x = sx + 4 * i;
    st3(xout, r0 + i, Vec3<R>{x[0], x[1], x[2]});
  }
  // let the copies still in flight land before the shared memory is reused
  if (tid == 0) {
    bool ok = true;
    if (ring) {
      for (int j = consumed; j < consumed + ring; ++j) ok = mbar_wait(&sh.mbar[j % ring], (uint32_t)((j / ring) & 1)) && ok;
      for (int k = 0; k < ring; ++k) mbar_inval(&sh.mbar[k]);
    } else if (resident && nblk > 0) {
      if (!waited_resident) ok = mbar_wait(&sh.mbar[0], 0);
      mbar_inval(&sh.mbar[0]);
    }
    if (!ok) sh.err = 1;
  }
  __syncthreads();
  if (sh.err) status = SKG_ERR_TIMEOUT;
  // no CTA may leave (or reuse its shared memory) while another still reads it
  csync(cl, csize);
  return ClusterPcgOut{it, status, dacc_value(rr_acc), dacc_value(rz), bb};
}

// one system on one cluster (pcg_mode 2); CO: two-level with the per-instance
// coarse data of instance 0 (e and P^T r past smem_bytes in dynamic shared memory)
template <typename R, int G, bool CO>
__global__ void __launch_bounds__(kClusterThreads, 1)
    k_pcg_cluster(Bsr<R> A, const double* __restrict__ b, double bsign, const uint8_t* __restrict__ pinned,
                  R* __restrict__ xout, double rtol, int max_iter, double* scal, int smem_bytes, CoarseDev cd) {
  cgx::cluster_group cl = cgx::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ClusterShared<R> sh;
  const ClusterPcgOut o = cluster_pcg_range<R, G, CO>(cl, A, const_cast<R*>(A.rec), 0, A.nbr, b, bsign, pinned,
                                                      xout, rtol, max_iter, smem_bytes, smem_raw, sh, cd, 0);
  if (cl.block_rank() == 0 && threadIdx.x == 0) {
    scal[S_ITERS] = o.iters;
    scal[S_RR] = o.rr;
    scal[S_RZ] = o.rz;
    scal[S_BB] = o.bb;
    scal[S_DONE] = 1.0;
    scal[S_STATUS] = o.status;
  }
}

// Many independent systems (instances), one per cluster at a time: each
// cluster takes the next instance from a queue ordered largest first and
// solves it to that instance's tolerance.  inst_rows (n_inst + 1) are the
// instances' block-row offsets; order lists the n instances this launch
// serves; inactive instances are skipped.
template <typename R, int G, bool CO>
__global__ void __launch_bounds__(kClusterThreads, 1)
    k_pcg_cluster_queue(Bsr<R> A, const int32_t* __restrict__ inst_rows, const int32_t* __restrict__ order,
                        int n, const uint8_t* __restrict__ active, const double* __restrict__ eta,
                        const double* __restrict__ b, double bsign, const uint8_t* __restrict__ pinned,
                        R* __restrict__ xout, int max_iter, int32_t* iters_out, int32_t* status_out,
                        unsigned* queue, int smem_bytes, CoarseDev cd) {
  cgx::cluster_group cl = cgx::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ClusterShared<R> sh;
  __shared__ int next_inst;
  __shared__ int inst_sh;
  const int csize = (int)cl.num_blocks();
  for (;;) {
    if (cl.block_rank() == 0 && threadIdx.x == 0) {
      const unsigned idx = atomicAdd(queue, 1u);
      next_inst = idx < (unsigned)n ? order[idx] : -1;
    }
    csync(cl, csize);
    if (threadIdx.x == 0) inst_sh = csize > 1 ? *cl.map_shared_rank(&next_inst, 0) : next_inst;
    __syncthreads();
    const int inst = inst_sh;
    csync(cl, csize);  // rank 0 may overwrite next_inst only after every CTA has read it
    if (inst < 0) break;
    if (!active[inst]) continue;
    const int64_t gbase = inst_rows[inst];
    const int64_t nbr = inst_rows[inst + 1] - gbase;
    if (cluster_vec_bytes(nbr, csize, (int)sizeof(R)) > smem_bytes) {
      if (cl.block_rank() == 0 && threadIdx.x == 0) {
        iters_out[inst] = 0;
        status_out[inst] = SKG_ERR_CAPACITY;
      }
      continue;
    }
    const ClusterPcgOut o = cluster_pcg_range<R, G, CO>(cl, A, const_cast<R*>(A.rec), gbase, nbr, b, bsign, pinned,
                                                        xout, eta[inst], max_iter, smem_bytes, smem_raw, sh, cd, inst);
    if (cl.block_rank() == 0 && threadIdx.x == 0) {
      iters_out[inst] = o.iters;
      status_out[inst] = o.status;
    }
  }
}

}  // namespace skg
