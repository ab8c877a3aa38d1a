// Block-Jacobi preconditioned CG on the assembled 3x3-block matrix, and the
// Newton / backward-Euler driver that replaces simkit's spsolve-based Newton
// (simkit/solvers/newton.py:46-69, simkit/integrators/backward_euler.py:76-91).
//
// PCG: FP32 (mixed) or FP64 vectors padded to 4 per vertex, FP64 dot
// products reduced deterministically.  Two execution modes:
//   mode 0: one kernel per phase (SpMV+dot, update+dots, direction update),
//           a device-side done flag turns later launches into no-ops and the
//           host checks it every few iterations;
//   mode 1: one persistent cooperative kernel for the whole solve, phases
//           separated by a grid barrier whose waits are bounded.
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "assembly.cuh"
#include "snh_math.cuh"

namespace skg {

enum ScalarSlot {
  S_RZ = 0, S_PQ = 1, S_RR = 2, S_BB = 3, S_BETA = 4, S_TOL2 = 5, S_ITERS = 6, S_DONE = 7, S_STATUS = 8,
  S_MAXIT = 9, S_GG = 10, S_E = 12,      /* 12: energy, 13: magnitude */
  S_SLOPE = 14, S_TMP = 16,               /* 16..19 scratch reduction outputs */
  S_BAR_ERR = 24, S_CERR = 26
};

constexpr double kKeepFrac = 0.2;   // fraction of the grid PCG's block records read with normal L2 priority

template <typename R> struct Bsr {
  int64_t nbr;
  const int32_t* rowptr;
  const int32_t* col;
  const R* val;    // entry-major values (used when rec is null)
  const R* jinv;
  const R* rec;    // 12-wide block records (values + column), preferred
  // grid PCG: records from slot `keep` on are read evict-first, so that the records
  // before it stay in L2 from one iteration to the next (all records do not fit)
  int64_t keep = INT64_MAX;
};

// one 3x3 block and its column from a record (three / five 16-byte loads);
// aux: the two spare slots (the column's packed coarse data), loaded for FP64
// records only when asked for (one more load)
template <typename R> struct Blk { R m[9]; int col; unsigned aux0, aux1; };

template <bool AUX = false>
__device__ __forceinline__ Blk<float> ld_rec(const float* __restrict__ rec, int64_t s, bool stream = false) {
  const float4* p = reinterpret_cast<const float4*>(rec) + 3 * s;
  float4 a, b, c;
  if (stream) {
    a = __ldcs(p); b = __ldcs(p + 1); c = __ldcs(p + 2);
  } else {
    a = __ldg(p); b = __ldg(p + 1); c = __ldg(p + 2);
  }
  return {{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x}, __float_as_int(c.y), __float_as_uint(c.z),
          __float_as_uint(c.w)};
}
template <bool AUX = false>
__device__ __forceinline__ Blk<double> ld_rec(const double* __restrict__ rec, int64_t s, bool stream = false) {
  (void)stream;
  const double2* p = reinterpret_cast<const double2*>(rec) + 6 * s;
  const double2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3), e = __ldg(p + 4);
  unsigned long long x = 0;
  if constexpr (AUX) x = (unsigned long long)__double_as_longlong(__ldg(reinterpret_cast<const double*>(p + 5)));
  return {{a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, e.x}, (int)__double_as_longlong(e.y), (unsigned)x,
          (unsigned)(x >> 32)};
}

// 3-term dot in the working precision, widened once
template <typename R> __device__ __forceinline__ double dot3w(Vec3<R> a, Vec3<R> b) {
  return double(a.x * b.x + a.y * b.y + a.z * b.z);
}
template <> __device__ __forceinline__ double dot3w<double>(Vec3<double> a, Vec3<double> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

template <typename R> struct PcgVecs {
  R* x;
  R* r;
  R* z;   // preconditioned residual (u in the Chronopoulos-Gear form)
  R* p;
  R* q;   // A p (w = A u in the Chronopoulos-Gear form)
  R* s;   // A p recurrence of the Chronopoulos-Gear form
};

template <typename R>
__device__ __forceinline__ Vec3<R> jacobi_apply(const R* __restrict__ jinv, int64_t v, Vec3<R> r) {
  const R* J = jinv + 9 * v;
  return {J[0] * r.x + J[1] * r.y + J[2] * r.z, J[3] * r.x + J[4] * r.y + J[5] * r.z,
          J[6] * r.x + J[7] * r.y + J[8] * r.z};
}

// y_v = sum_k A_vk x_{col_k} for one block row, G lanes per row; returns
// the row result in every lane of the group.
// Every lane of the warp must call this (the shuffles use a full mask);
// lanes whose row is out of range pass valid = false and contribute nothing.
template <typename R, int G>
__device__ __forceinline__ Vec3<R> spmv_row(const Bsr<R>& A, const R* __restrict__ xin, int64_t row, int lane,
                                            bool valid) {
  const int rp = valid ? __ldg(A.rowptr + row) : 0;
  int K = valid ? __ldg(A.rowptr + row + 1) - rp : 0;
  const R* vals = A.val + 9 * (int64_t)rp;
  R a0 = 0, a1 = 0, a2 = 0;
  if (A.rec) {
    for (int k = lane; k < K; k += G) {
      const Blk<R> b = ld_rec(A.rec, rp + k);
      const Vec3<R> xv = ld3c(xin, b.col);
      a0 += b.m[0] * xv.x + b.m[1] * xv.y + b.m[2] * xv.z;
      a1 += b.m[3] * xv.x + b.m[4] * xv.y + b.m[5] * xv.z;
      a2 += b.m[6] * xv.x + b.m[7] * xv.y + b.m[8] * xv.z;
    }
    K = 0;
  }
  for (int k = lane; k < K; k += G) {
    const int c = __ldg(A.col + rp + k);
    const Vec3<R> xv = ld3c(xin, c);
    const R m0 = vals[k], m1 = vals[K + k], m2 = vals[2 * K + k];
    const R m3 = vals[3 * K + k], m4 = vals[4 * K + k], m5 = vals[5 * K + k];
    const R m6 = vals[6 * K + k], m7 = vals[7 * K + k], m8 = vals[8 * K + k];
    a0 += m0 * xv.x + m1 * xv.y + m2 * xv.z;
    a1 += m3 * xv.x + m4 * xv.y + m5 * xv.z;
    a2 += m6 * xv.x + m7 * xv.y + m8 * xv.z;
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    a0 += __shfl_xor_sync(0xffffffffu, a0, o, G);
    a1 += __shfl_xor_sync(0xffffffffu, a1, o, G);
    a2 += __shfl_xor_sync(0xffffffffu, a2, o, G);
  }
  return {a0, a1, a2};
}

// U block rows per lane group at once (records only): all U rows' record
// loads are issued before any row's gathers, so each lane keeps U independent
// load chains in flight.
template <typename R, int G, int U>
__device__ __forceinline__ void spmv_rowsU(const Bsr<R>& A, const R* __restrict__ xin, const int64_t (&row)[U],
                                           const bool (&valid)[U], int lane, Vec3<R> (&y)[U]) {
  int p[U], K[U];
  int kmax = 0;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    p[u] = valid[u] ? __ldg(A.rowptr + row[u]) : 0;
    K[u] = valid[u] ? __ldg(A.rowptr + row[u] + 1) - p[u] : 0;
    kmax = K[u] > kmax ? K[u] : kmax;
  }
  R acc[U][3];
#pragma unroll
  for (int u = 0; u < U; ++u) acc[u][0] = acc[u][1] = acc[u][2] = R(0);
  for (int k = lane; k < kmax; k += G) {
    Blk<R> bk[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      bk[u] = Blk<R>{};
      if (k < K[u]) bk[u] = ld_rec(A.rec, p[u] + k);
    }
    Vec3<R> xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      xv[u] = Vec3<R>{R(0), R(0), R(0)};
      if (k < K[u]) xv[u] = ld3c(xin, bk[u].col);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      acc[u][0] += bk[u].m[0] * xv[u].x + bk[u].m[1] * xv[u].y + bk[u].m[2] * xv[u].z;
      acc[u][1] += bk[u].m[3] * xv[u].x + bk[u].m[4] * xv[u].y + bk[u].m[5] * xv[u].z;
      acc[u][2] += bk[u].m[6] * xv[u].x + bk[u].m[7] * xv[u].y + bk[u].m[8] * xv[u].z;
    }
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[u][c] += __shfl_xor_sync(0xffffffffu, acc[u][c], o, G);
#pragma unroll
  for (int u = 0; u < U; ++u) y[u] = Vec3<R>{acc[u][0], acc[u][1], acc[u][2]};
}

// ------------------------------------------------------ mode 0 kernels ---
template <typename R>
__global__ void __launch_bounds__(kBlock) k_pcg_init(Bsr<R> A, const double* __restrict__ b, double bsign,
                                                     const uint8_t* __restrict__ pinned, PcgVecs<R> v,
                                                     double rtol, int max_iter, double* partials,
                                                     unsigned* counter, double* scal,
                                                     const double* __restrict__ rtol_dev = nullptr) {
  double acc[3] = {0.0, 0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < A.nbr; i += stride) {
    double bb[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      bb[c] = bsign * b[3 * i + c];
      if (pinned && pinned[3 * i + c]) bb[c] = 0.0;
    }
    const Vec3<R> r = {R(bb[0]), R(bb[1]), R(bb[2])};
    const Vec3<R> z = jacobi_apply(A.jinv, i, r);
    st3(v.r, i, r);
    st3(v.z, i, z);
    st3(v.p, i, z);
    st3(v.x, i, Vec3<R>{R(0), R(0), R(0)});
    acc[0] += dot3w(r, z);
    acc[1] += dot3w(r, r);
  }
  acc[2] = acc[1];
  if (grid_sum<3, kBlock>(acc, partials, counter, scal + S_TMP) && threadIdx.x == 0) {
    const double rz = scal[S_TMP], rr = scal[S_TMP + 1], bb = scal[S_TMP + 2];
    if (rtol_dev) rtol = *rtol_dev;   // the forcing term decided on the device
    scal[S_RZ] = rz;
    scal[S_RR] = rr;
    scal[S_BB] = bb;
    scal[S_TOL2] = rtol * rtol * bb;
    scal[S_ITERS] = 0.0;
    scal[S_MAXIT] = max_iter;
    scal[S_STATUS] = 0.0;
    scal[S_DONE] = (rr <= rtol * rtol * bb || bb == 0.0 || max_iter <= 0) ? 1.0 : 0.0;
  }
}

template <typename R, int G>
__global__ void __launch_bounds__(kBlock) k_pcg_spmv(Bsr<R> A, PcgVecs<R> v, double* partials, unsigned* counter,
                                                     double* scal) {
  if (*((volatile double*)(scal + S_DONE)) != 0.0) return;
  double acc[1] = {0.0};
  const int lane = threadIdx.x & (G - 1);
  // warp-uniform trip count: each warp covers 32/G consecutive rows per pass
  const int64_t warp_rows = 32 / G;
  const int64_t stride = (int64_t)gridDim.x * (blockDim.x / G);
  const int64_t row0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * warp_rows;
  for (int64_t base = row0; base < A.nbr; base += stride) {
    const int64_t row = base + ((threadIdx.x & 31) / G);
    const bool valid = row < A.nbr;
    const Vec3<R> y = spmv_row<R, G>(A, v.p, row, lane, valid);
    if (lane == 0 && valid) {
      st3(v.q, row, y);
      acc[0] += dot3w(ld3c(v.p, row), y);
    }
  }
  if (grid_sum<1, kBlock>(acc, partials, counter, scal + S_PQ) && threadIdx.x == 0) {
    const double pq = scal[S_PQ];
    if (!(pq > 0.0) || !isfinite(pq)) {
      scal[S_DONE] = 1.0;
      scal[S_STATUS] = isfinite(pq) ? 0.0 : (double)SKG_ERR_NONFINITE;
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_pcg_update(Bsr<R> A, PcgVecs<R> v, double* partials, unsigned* counter,
                                                       double* scal) {
  if (*((volatile double*)(scal + S_DONE)) != 0.0) return;
  const double alpha = scal[S_RZ] / scal[S_PQ];
  const R a = R(alpha);
  double acc[2] = {0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < A.nbr; i += stride) {
    Vec3<R> x = ld3c(v.x, i), r = ld3c(v.r, i);
    const Vec3<R> p = ld3c(v.p, i), q = ld3c(v.q, i);
    x = {x.x + a * p.x, x.y + a * p.y, x.z + a * p.z};
    r = {r.x - a * q.x, r.y - a * q.y, r.z - a * q.z};
    const Vec3<R> z = jacobi_apply(A.jinv, i, r);
    st3(v.x, i, x);
    st3(v.r, i, r);
    st3(v.z, i, z);
    acc[0] += dot3w(r, z);
    acc[1] += dot3w(r, r);
  }
  if (grid_sum<2, kBlock>(acc, partials, counter, scal + S_TMP) && threadIdx.x == 0) {
    const double rz = scal[S_TMP], rr = scal[S_TMP + 1];
    scal[S_BETA] = rz / scal[S_RZ];
    scal[S_RZ] = rz;
    scal[S_RR] = rr;
    const double it = scal[S_ITERS] + 1.0;
    scal[S_ITERS] = it;
    if (!isfinite(rr)) {
      scal[S_STATUS] = (double)SKG_ERR_NONFINITE;
      scal[S_DONE] = 1.0;
    } else if (rr <= scal[S_TOL2] || it >= scal[S_MAXIT]) {
      scal[S_DONE] = 1.0;
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_pcg_direction(int64_t nbr, PcgVecs<R> v, const double* scal) {
  if (*((volatile const double*)(scal + S_DONE)) != 0.0) return;
  const R beta = R(scal[S_BETA]);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nbr; i += stride) {
    const Vec3<R> z = ld3c(v.z, i), p = ld3c(v.p, i);
    st3(v.p, i, Vec3<R>{z.x + beta * p.x, z.y + beta * p.y, z.z + beta * p.z});
  }
}

// ------------------------------------------------------ mode 1 kernel ----
// Sense-reversing grid barrier.  Every wait is bounded: after kSpinLimit
// polls the block records SKG_ERR_TIMEOUT and all blocks leave the solve at
// their next barrier.  The kernel is launched cooperatively, so all blocks
// are resident and the barrier completes in normal operation.
constexpr long long kSpinLimit = 1ll << 24;

// Arrive-and-wait grid barrier.  Thread 0 of each block arrives with an acq_rel
// atomic (releasing the block's writes, ordered before it by __syncthreads); the
// last arrival resets the count and publishes the next generation with a
// release store; the others poll the generation with acquire loads.  Bounded
// spin (at most `limit` polls): on timeout err is set and false returned.
__device__ __forceinline__ bool grid_barrier(unsigned* count, volatile unsigned* gen, volatile double* err,
                                             long long limit = kSpinLimit) {
  __syncthreads();
  __shared__ int ok_s;
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned g = *gen;
    if (atom_add_acqrel_gpu(count, 1u) == gridDim.x - 1) {
      st_relaxed_gpu(count, 0u);
      st_release_gpu((unsigned*)gen, g + 1u);
    } else {
      long long spins = 0;
      while (ld_acquire_gpu((const unsigned*)gen) == g) {
        if (++spins > limit) {
          *err = (double)SKG_ERR_TIMEOUT;
          ok = 0;
          break;
        }
        if (spins > 256) __nanosleep(32);
      }
    }
    if (*err != 0.0) ok = 0;
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// sum of NV per-block partials in index order, computed redundantly by
// every block (same order -> same value everywhere)
template <int NV>
__device__ __forceinline__ void all_sum(const double* partials, double (&out)[NV]) {
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    s[k] = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
      s[k] += *((volatile const double*)&partials[k * gridDim.x + i]);
  }
  block_sum<NV, kBlock>(s);
  __shared__ double res[NV];
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) res[k] = s[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = res[k];
  __syncthreads();
}

template <typename R, int G, int U>
__global__ void __launch_bounds__(kBlock, 3) k_pcg_persistent(Bsr<R> A, PcgVecs<R> v, double* partials,
                                                           unsigned* bar, double* scal) {
  // partials: 3 buffers of 2*gridDim doubles (pq | rz, rr | spare)
  double* P1 = partials;
  double* P2 = partials + 2 * gridDim.x;
  unsigned* count = bar;
  volatile unsigned* gen = bar + 1;
  volatile double* err = scal + S_BAR_ERR;
  double rz = scal[S_RZ];
  const double tol2 = scal[S_TOL2];
  const int max_iter = (int)scal[S_MAXIT];
  int it = 0;
  bool done = scal[S_DONE] != 0.0;
  int status = 0;
  const int lane = threadIdx.x & (G - 1);
  const int64_t groups = (int64_t)gridDim.x * (blockDim.x / G);
  const int64_t row0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * (32 / G);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double rr = scal[S_RR];
  while (!done) {
    // q = A p, pq
    double acc[2] = {0.0, 0.0};
    if (U > 1 && A.rec) {
      for (int64_t base = row0; base < A.nbr; base += U * groups) {
        int64_t rows[U];
        bool val[U];
        Vec3<R> ys[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          rows[u] = base + u * groups + ((threadIdx.x & 31) / G);
          val[u] = rows[u] < A.nbr;
        }
        spmv_rowsU<R, G, U>(A, v.p, rows, val, lane, ys);
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (lane == 0 && val[u]) {
            st3(v.q, rows[u], ys[u]);
            acc[0] += dot3w(ld3c(v.p, rows[u]), ys[u]);
          }
      }
    } else {
      for (int64_t base = row0; base < A.nbr; base += groups) {
        const int64_t row = base + ((threadIdx.x & 31) / G);
        const bool valid = row < A.nbr;
        const Vec3<R> y = spmv_row<R, G>(A, v.p, row, lane, valid);
        if (lane == 0 && valid) {
          st3(v.q, row, y);
          acc[0] += dot3w(ld3c(v.p, row), y);
        }
      }
    }
    double a1[1] = {acc[0]};
    block_sum<1, kBlock>(a1);
    if (threadIdx.x == 0) P1[blockIdx.x] = a1[0];
    if (!grid_barrier(count, gen, err)) { status = SKG_ERR_TIMEOUT; break; }
    double pq[1];
    all_sum<1>(P1, pq);
    if (!(pq[0] > 0.0) || !isfinite(pq[0])) {
      status = isfinite(pq[0]) ? 0 : SKG_ERR_NONFINITE;
      break;
    }
    const double alpha = rz / pq[0];
    const R a = R(alpha);
    acc[0] = acc[1] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < A.nbr; i += stride) {
      Vec3<R> x = ld3c(v.x, i), r = ld3c(v.r, i);
      const Vec3<R> p = ld3c(v.p, i), q = ld3c(v.q, i);
      x = {x.x + a * p.x, x.y + a * p.y, x.z + a * p.z};
      r = {r.x - a * q.x, r.y - a * q.y, r.z - a * q.z};
      const Vec3<R> z = jacobi_apply(A.jinv, i, r);
      st3(v.x, i, x);
      st3(v.r, i, r);
      st3(v.z, i, z);
      acc[0] += dot3w(r, z);
      acc[1] += dot3w(r, r);
    }
    block_sum<2, kBlock>(acc);
    if (threadIdx.x == 0) {
      P2[blockIdx.x] = acc[0];
      P2[gridDim.x + blockIdx.x] = acc[1];
    }
    if (!grid_barrier(count, gen, err)) { status = SKG_ERR_TIMEOUT; break; }
    double s2[2];
    all_sum<2>(P2, s2);
    ++it;
    rr = s2[1];
    const double beta = s2[0] / rz;
    rz = s2[0];
    if (!isfinite(rr)) { status = SKG_ERR_NONFINITE; break; }
    if (rr <= tol2 || it >= max_iter) break;
    const R b = R(beta);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < A.nbr; i += stride) {
      const Vec3<R> z = ld3c(v.z, i), p = ld3c(v.p, i);
      st3(v.p, i, Vec3<R>{z.x + b * p.x, z.y + b * p.y, z.z + b * p.z});
    }
    if (!grid_barrier(count, gen, err)) { status = SKG_ERR_TIMEOUT; break; }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_ITERS] = it;
    scal[S_RR] = rr;
    scal[S_RZ] = rz;
    scal[S_DONE] = 1.0;
    if (status != 0) scal[S_STATUS] = status;
    if (*err != 0.0) scal[S_STATUS] = *err;
  }
}


// ------------------------------------------------ mode 4: Chronopoulos-Gear
// Preconditioned CG in the Chronopoulos-Gear arrangement: the three dot
// products of an iteration are taken in the same phase as the SpMV, so an
// iteration has one elementwise phase and one SpMV+dots phase separated by
// two grid barriers (standard PCG needs three).  Recurrences, with u = M r
// and w = A u:
//   p = u + beta p;  s = w + beta s;  x += alpha p;  r -= alpha s;  u = M r
//   w = A u;  gamma = (r,u), delta = (w,u), rho = (r,r)
//   beta = gamma / gamma_old;  alpha = gamma / (delta - beta gamma / alpha_old)
// One CTA of kCgThreads per SM keeps the number of blocks arriving at each
// barrier at the SM count.
constexpr int kCgThreads = 768;

template <int NV, int BLOCK>
__device__ __forceinline__ void all_sum_b(const double* partials, double (&out)[NV]) {
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    s[k] = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK)
      s[k] += *((volatile const double*)&partials[k * gridDim.x + i]);
  }
  block_sum<NV, BLOCK>(s);
  __shared__ double res[NV];
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) res[k] = s[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = res[k];
  __syncthreads();
}

template <typename R, int G>
__device__ __forceinline__ void cg2_spmv_dots(const Bsr<R>& A, const PcgVecs<R>& v, int64_t row0, int64_t stride_rows,
                                              int lane, double (&acc)[3]) {
  for (int64_t base = row0; base < A.nbr; base += stride_rows) {
    const int64_t row = base + ((threadIdx.x & 31) / G);
    const bool valid = row < A.nbr;
    const Vec3<R> w = spmv_row<R, G>(A, v.z, row, lane, valid);
    if (lane == 0 && valid) {
      st3(v.q, row, w);
      const Vec3<R> r = ld3c(v.r, row), u = ld3c(v.z, row);
      acc[0] += dot3w(r, u);
      acc[1] += dot3w(w, u);
      acc[2] += dot3w(r, r);
    }
  }
}

template <typename R, int G>
__global__ void __launch_bounds__(kCgThreads, 1) k_pcg_cg2(Bsr<R> A, PcgVecs<R> v, double* partials, unsigned* bar,
                                                         double* scal) {
  unsigned* count = bar;
  volatile unsigned* gen = bar + 1;
  volatile double* err = scal + S_BAR_ERR;
  const double tol2 = scal[S_TOL2];
  const int max_iter = (int)scal[S_MAXIT];
  const int lane = threadIdx.x & (G - 1);
  const int64_t stride_rows = (int64_t)gridDim.x * (blockDim.x / G);
  const int64_t row0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * (32 / G);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int status = 0, it = 0;
  double rr = scal[S_RR], gamma = scal[S_RZ];
  if (scal[S_DONE] == 0.0) {
    // prologue: w = A u (u = z = M r from the init kernel), gamma, delta
    double acc[3] = {0.0, 0.0, 0.0};
    cg2_spmv_dots<R, G>(A, v, row0, stride_rows, lane, acc);
    block_sum<3, kCgThreads>(acc);
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < 3; ++k) partials[k * gridDim.x + blockIdx.x] = acc[k];
    bool ok = grid_barrier(count, gen, err);
    double sm[3] = {0.0, 0.0, 0.0};
    if (ok) all_sum_b<3, kCgThreads>(partials, sm);
    gamma = sm[0];
    double delta = sm[1];
    double alpha = gamma / delta;
    double beta = 0.0;
    if (!ok) status = SKG_ERR_TIMEOUT;
    else if (!(delta > 0.0) || !isfinite(delta)) status = isfinite(delta) ? 0 : SKG_ERR_NONFINITE;
    while (ok && status == 0 && (delta > 0.0)) {
      // p = u + beta p; s = w + beta s; x += alpha p; r -= alpha s; u = M r
      const R a = R(alpha), b = R(beta);
      for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < A.nbr; i += stride) {
        const Vec3<R> u = ld3c(v.z, i), w = ld3c(v.q, i);
        Vec3<R> p = ld3c(v.p, i), s = ld3c(v.s, i), x = ld3c(v.x, i), r = ld3c(v.r, i);
        if (it == 0) {
          p = u;
          s = w;
        } else {
          p = {u.x + b * p.x, u.y + b * p.y, u.z + b * p.z};
          s = {w.x + b * s.x, w.y + b * s.y, w.z + b * s.z};
        }
        x = {x.x + a * p.x, x.y + a * p.y, x.z + a * p.z};
        r = {r.x - a * s.x, r.y - a * s.y, r.z - a * s.z};
        st3(v.p, i, p);
        st3(v.s, i, s);
        st3(v.x, i, x);
        st3(v.r, i, r);
        st3(v.z, i, jacobi_apply(A.jinv, i, r));
      }
      ++it;
      if (!grid_barrier(count, gen, err)) { status = SKG_ERR_TIMEOUT; break; }
      double acc2[3] = {0.0, 0.0, 0.0};
      cg2_spmv_dots<R, G>(A, v, row0, stride_rows, lane, acc2);
      block_sum<3, kCgThreads>(acc2);
      if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 3; ++k) partials[k * gridDim.x + blockIdx.x] = acc2[k];
      if (!grid_barrier(count, gen, err)) { status = SKG_ERR_TIMEOUT; break; }
      all_sum_b<3, kCgThreads>(partials, sm);
      const double g_new = sm[0];
      delta = sm[1];
      rr = sm[2];
      if (!isfinite(rr) || !isfinite(g_new)) { status = SKG_ERR_NONFINITE; break; }
      if (rr <= tol2 || it >= max_iter) { gamma = g_new; break; }
      beta = g_new / gamma;
      const double den = delta - beta * g_new / alpha;
      if (!(den > 0.0)) { gamma = g_new; break; }   // loss of positive definiteness: stop with current x
      alpha = g_new / den;
      gamma = g_new;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_ITERS] = it;
    scal[S_RR] = rr;
    scal[S_RZ] = gamma;
    scal[S_DONE] = 1.0;
    if (status != 0) scal[S_STATUS] = status;
    if (*err != 0.0) scal[S_STATUS] = *err;
  }
}

}  // namespace skg

#include "coarse_common.cuh"
#include "pcg_cluster.cuh"
#include "pcg_grid.cuh"
#include "coarse.cuh"

namespace skg {

// ------------------------------------------------------ small kernels ----
// u_tilde = 2 u_curr - u_prev (simkit/energies/kinetic.py:87-90), u = u_tilde
__global__ void k_be_init(const double* __restrict__ uc, const double* __restrict__ up, int64_t m,
                          double* __restrict__ ut, double* __restrict__ u) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  const double x = uc[i] + (uc[i] - up[i]);
  ut[i] = x;
  u[i] = x;
}

// BDF2 target from four displacement levels, in the order of simkit/energies/kinetic.py:63-101
// (velocities by the second-order backward difference), u = u_tilde
__global__ void k_bdf2_init(const double* __restrict__ uc, const double* __restrict__ up,
                            const double* __restrict__ up2, const double* __restrict__ up3, double h, int64_t m,
                            double* __restrict__ ut, double* __restrict__ u) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  const double vc = (3.0 * uc[i] - 4.0 * up[i] + up2[i]) / (2.0 * h);
  const double vp = (3.0 * up[i] - 4.0 * up2[i] + up3[i]) / (2.0 * h);
  const double x = (4.0 / 3.0) * uc[i] - (1.0 / 3.0) * up[i] + (8.0 * h / 9.0) * vc - (2.0 * h / 9.0) * vp;
  ut[i] = x;
  u[i] = x;
}

// contact planes of the potential, from the parameters
static int make_contact(const skg_be_params* prm, const skg_be_state* st, Contact* c) {
  *c = Contact{};
  if (prm->n_planes <= 0) return SKG_OK;
  if (prm->n_planes > SKG_MAX_PLANES || !prm->planes)
    return fail(SKG_ERR_ARG, "contact planes: 1..%d planes and their array", SKG_MAX_PLANES);
  if (!st->x_rest) return fail(SKG_ERR_ARG, "contact planes need the rest positions");
  c->n = prm->n_planes;
  c->X = st->x_rest;
  c->w = prm->contact_mass_weighted ? st->mass : nullptr;
  for (int q = 0; q < c->n; ++q) {
    for (int i = 0; i < 3; ++i) {
      c->p[q][i] = prm->planes[q].p[i];
      c->nrm[q][i] = prm->planes[q].n[i];
    }
    c->k[q] = prm->planes[q].k;
  }
  return SKG_OK;
}

static int check_integrator(const skg_be_params* prm, const skg_be_state* st) {
  if (prm->integrator != 0 && prm->integrator != 1) return fail(SKG_ERR_ARG, "integrator must be 0 (BE) or 1 (BDF2)");
  if (prm->integrator == 1 && (!st->u_prev2 || !st->u_prev3))
    return fail(SKG_ERR_ARG, "BDF2 needs the displacements at steps k-2 and k-3");
  return SKG_OK;
}

// inertial target and Newton start of the chosen integrator; returns the kinetic factor c / h^2
static int launch_target(const skg_be_params* prm, const skg_be_state* st, int64_t nd, double* ut, cudaStream_t s,
                         double* inv_h2) {
  const double h = prm->dt;
  if (prm->integrator == 1) {
    k_bdf2_init<<<blocks_for(nd), kBlock, 0, s>>>(st->u_curr, st->u_prev, st->u_prev2, st->u_prev3, h, nd, ut,
                                                   st->u);
    *inv_h2 = (9.0 / 4.0) / (h * h);
  } else {
    k_be_init<<<blocks_for(nd), kBlock, 0, s>>>(st->u_curr, st->u_prev, nd, ut, st->u);
    *inv_h2 = 1.0 / (h * h);
  }
  SKG_LAUNCHED();
  return SKG_OK;
}

// u += step * dx on free DOFs
template <typename R>
__global__ void k_apply_step(double* __restrict__ u, const R* __restrict__ dx, double step, int64_t n,
                             const uint8_t* __restrict__ pinned) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  const Vec3<R> d = ld3c(dx, v);
  const double dd[3] = {double(d.x), double(d.y), double(d.z)};
#pragma unroll
  for (int c = 0; c < 3; ++c)
    if (!(pinned && pinned[3 * v + c])) u[3 * v + c] += step * dd[c];
}

// g . dx and dx . dx (FP64): the Armijo slope and the step norm of simkit's stop rule
template <typename R>
__global__ void __launch_bounds__(kBlock) k_dot_g(const double* __restrict__ g, const R* __restrict__ dx, int64_t n,
                                                  double* partials, unsigned* counter, double* out) {
  double acc[2] = {0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += stride) {
    const Vec3<R> d = ld3c(dx, v);
    const double x = double(d.x), y = double(d.y), z = double(d.z);
    acc[0] += g[3 * v] * x + g[3 * v + 1] * y + g[3 * v + 2] * z;
    acc[1] += x * x + y * y + z * z;
  }
  grid_sum<2, kBlock>(acc, partials, counter, out);
}

// padded vector -> simkit layout (3n), FP64
template <typename R>
__global__ void k_unpad(const R* __restrict__ x, int64_t n, double* __restrict__ out) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  const Vec3<R> a = ld3c(x, v);
  out[3 * v] = a.x;
  out[3 * v + 1] = a.y;
  out[3 * v + 2] = a.z;
}

// ---------------------------------------------------------- PCG driver ----
struct PcgResult {
  int iters;
  int status;
  int launches;
  double rr, bb;
};

// Phase timer on the launching stream (CUDA events; only when profiling).
struct PhaseTimer {
  bool on = false;
  cudaStream_t s = 0;
  cudaEvent_t a = nullptr, b = nullptr;
  void init(bool enable, cudaStream_t st) {
    on = enable;
    s = st;
    if (on) {
      static thread_local cudaEvent_t ea = nullptr, eb = nullptr;
      if (!ea) {
        cudaEventCreate(&ea);
        cudaEventCreate(&eb);
      }
      a = ea;
      b = eb;
    }
  }
  void begin() {
    if (on) cudaEventRecord(a, s);
  }
  double end() {
    if (!on) return 0.0;
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
};

static int g_num_sms = 0;

static int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

constexpr int kG = 8;   // lanes per block row in the grid SpMV
constexpr int kGc = 4;  // lanes per block row in the cluster SpMV
// systems up to this many block rows run PCG on one thread-block cluster
constexpr int64_t kClusterAutoRows = 24576;

// ------------------------------------------------- two-level coarse -----
static CoarseDev make_coarse_dev(const skg_tet_mesh* m, const Workspace& w) {
  CoarseDev c{};
  const skg_coarse* h = m->coarse;
  c.n_agg = h->n_agg;
  c.nc = 6 * h->n_agg;
  c.np = (int)coarse_padded(m);
  c.n_cb = h->n_cblocks;
  c.mode = reinterpret_cast<const float4*>(h->mode);
  c.cb_ptr = h->cb_ptr;
  c.cb_slot = h->cb_slot;
  c.cb_rc = h->cb_rc;
  c.bsr_row = m->bsr_row;
  c.M = w.cM;
  c.rowp = w.crowp;
  c.rc = w.crc;
  c.rq = w.crq;
  c.rcg = w.crcg;
  c.e = w.ce;
  c.ok = w.cok;
  c.bar = w.cbar;
  c.m_floats = (int64_t)c.np * c.np;
  if (h->inst_agg) {
    c.m_floats = h->m_floats;
    c.n_inst = h->n_inst;
    c.max_np = h->max_np;
    c.inst_agg = h->inst_agg;
    c.agg_inst = h->agg_inst;
    c.inst_moff = h->inst_moff;
    c.colpack = h->colpack;
  }
  return c;
}

// A_c = P^T A P from the assembled records, then its inverse in place; on a
// non-positive pivot (or a barrier timeout) c.ok stays 0 and the PCG runs
// one-level.  Two launches.
template <typename R>
static int coarse_refresh(const Bsr<R>& A, const CoarseDev& c, double* scal, cudaStream_t s,
                          const int32_t* order = nullptr) {
  SKG_CUDA(cudaMemsetAsync(c.M, 0, sizeof(float) * (size_t)c.m_floats, s));
  SKG_CUDA(cudaMemsetAsync(c.ok, 0, sizeof(int) * (size_t)(c.inst_agg ? c.n_inst : 1), s));
  SKG_CUDA(cudaMemsetAsync(c.bar, 0, 2 * sizeof(unsigned), s));
  SKG_CUDA(cudaMemsetAsync(scal + S_CERR, 0, sizeof(double), s));
  const int64_t gal_threads = 32 * (int64_t)c.n_cb;
  k_coarse_galerkin<R><<<(int)((gal_threads + kBlock - 1) / kBlock), kBlock, 0, s>>>(A, c);
  SKG_LAUNCHED();
  if (c.inst_agg && c.n_inst > 1) {
    // batches: one cluster of kGjCluster CTAs per instance, largest first
    int nclu = kCoarseInvCtas / kGjCluster;
    if (nclu > c.n_inst) nclu = c.n_inst;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kGjCluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(nclu * kGjCluster, 1, 1);
    cfg.blockDim = dim3(kGjCols, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SKG_CUDA(cudaLaunchKernelEx(&cfg, k_coarse_invert_inst, c, order));
    return SKG_OK;
  }
  static int per_sm = 0;
  if (per_sm == 0) {
    SKG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_coarse_invert, kGjCols, 0));
    if (per_sm < 1) return fail(SKG_ERR_CUDA, "the coarse inversion kernel does not fit on an SM");
  }
  // work units of the upper block triangle (as enumerated by the kernel)
  int units = 0;
  for (int ib = 0, ncu = (c.np + kGjCols - 1) / kGjCols; ib < c.np / kGjB; ++ib) units += ncu - (ib * kGjB) / kGjCols;
  int grid = per_sm * num_sms();
  if (grid > units) grid = units;
  if (grid < 1) grid = 1;
  CoarseDev c2 = c;
  volatile double* err = scal + S_CERR;
  void* args[] = {&c2, &err};
  SKG_CUDA(cudaLaunchCooperativeKernel((const void*)k_coarse_invert, dim3(grid), dim3(kGjCols), args, 0, s));
  return SKG_OK;
}

// cd (per-instance form, instance 0): the two-level kernel, which keeps the
// instance's coarse vectors in the last kCoarseSmem bytes of dynamic shared memory
template <typename R>
static int launch_pcg_cluster(const Bsr<R>& A, const double* b, double bsign, const uint8_t* pinned, R* xout,
                              double rtol, int max_iter, double* scal, cudaStream_t s, const CoarseDev* cd = nullptr,
                              int variant = 0) {
  const void* kern = cd ? (const void*)k_pcg_cluster<R, kGc, true> : (const void*)k_pcg_cluster<R, kGc, false>;
  static thread_local bool configured[2] = {false, false};
  if (!configured[cd ? 1 : 0]) {
    SKG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    SKG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kClusterSmemBudget));
    configured[cd ? 1 : 0] = true;
  }
  const int budget = cd ? kClusterSmemBudget - kCoarseSmem : kClusterSmemBudget;
  // cluster size: variant 0 by size, 1..4 = 16, 8, 4, 2 CTAs (picked by the autotuner), never
  // smaller than what holds the vectors
  int csize = A.nbr >= 2048 ? kClusterMax : 8;
  if (variant >= 1 && variant <= 4) csize = kClusterMax >> (variant - 1);
  while (csize < kClusterMax && cluster_vec_bytes(A.nbr, csize, (int)sizeof(R)) > budget) csize *= 2;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  cfg.blockDim = dim3(kClusterThreads, 1, 1);
  cfg.dynamicSmemBytes = kClusterSmemBudget;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  for (;;) {
    attr[0].val.clusterDim.x = csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(csize, 1, 1);
    int nclusters = 0;
    cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg);
    if (e == cudaSuccess && nclusters >= 1) break;
    (void)cudaGetLastError();
    if (csize <= 2) return fail(SKG_ERR_CUDA, "no thread-block cluster of the PCG kernel fits on this device");
    csize /= 2;
  }
  if (cluster_vec_bytes(A.nbr, csize, (int)sizeof(R)) > budget)
    return fail(SKG_ERR_CAPACITY, "system too large for one cluster");
  Bsr<R> a2 = A;
  int smem = budget;
  CoarseDev c2 = cd ? *cd : CoarseDev{};
  if (cd) SKG_CUDA(cudaMemsetAsync(cd->rc, 0, sizeof(unsigned long long) * 6 * (size_t)cd->n_agg, s));
  void* args[] = {&a2, (void*)&b, &bsign, (void*)&pinned, &xout, &rtol, &max_iter, &scal, &smem, &c2};
  SKG_CUDA(cudaLaunchKernelExC(&cfg, kern, args));
  return SKG_OK;
}

// largest system (block rows) the cluster PCG holds in shared memory
template <typename R> static int64_t cluster_rows_limit() {
  return (int64_t)kClusterMax * (kClusterSmemBudget / (kClusterVals * (int64_t)sizeof(R)));
}

// the PCG form a solve of nbr block rows runs in: 3 (auto) becomes the cluster form (2) up to
// kClusterAutoRows, above it the two-level grid form (7) with whole-mesh coarse data, else the
// one-level grid form (5); the cluster form falls back to 5 past what one cluster holds
template <typename R>
static int resolve_pcg_mode(int mode, int64_t nbr, bool grid_form) {
  if (mode == 7 && !grid_form) mode = 5;
  if (mode == 3) mode = nbr <= kClusterAutoRows ? 2 : (grid_form ? 7 : 5);
  if (mode == 2 && nbr > cluster_rows_limit<R>()) mode = 5;
  return mode;
}

// read = false: the solve is enqueued and its scalars (iterations, status, residual) are left in scal
// for the caller to read with its next host round trip.  rtol_dev: the relative tolerance is read
// from device memory when the solve starts (rtol is then ignored)
template <typename R>
static int pcg_solve(const Bsr<R>& A, const double* b, double bsign, const uint8_t* pinned, PcgVecs<R> v,
                     double rtol, int max_iter, int mode, double* partials, unsigned* counter, double* scal,
                     cudaStream_t s, PcgResult* res, int variant = 0, const CoarseDev* cd = nullptr,
                     bool read = true, const double* rtol_dev = nullptr) {
  const int rb = reduce_blocks(A.nbr);
  const bool grid_form = cd && !cd->inst_agg;
  mode = resolve_pcg_mode<R>(mode, A.nbr, grid_form);
  if (rtol_dev && (mode == 0 || mode == 2)) return fail(SKG_ERR_ARG, "pcg: a device tolerance needs a grid form");
  res->launches = 0;
  if (mode != 2) {
    k_pcg_init<R><<<rb, kBlock, 0, s>>>(A, b, bsign, pinned, v, rtol, max_iter, partials, counter, scal, rtol_dev);
    SKG_LAUNCHED();
    res->launches = 1;
  }
  if (mode == 2) {
    const CoarseDev* cc = cd && cd->inst_agg ? cd : nullptr;
    SKG_TRY(launch_pcg_cluster<R>(A, b, bsign, pinned, v.x, rtol, max_iter, scal, s, cc, variant));
    res->launches += 1;
  } else if (mode == 4) {
    int per_sm = 0;
    SKG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_cg2<R, kG>, kCgThreads, 0));
    if (per_sm < 1) return fail(SKG_ERR_CUDA, "the PCG kernel does not fit on an SM");
    int64_t want = (A.nbr * kG + kCgThreads - 1) / kCgThreads;
    int64_t cap = num_sms();
    int grid = (int)(want < cap ? want : cap);
    if (grid < 1) grid = 1;
    unsigned* bar = counter + 4;
    SKG_CUDA(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s));
    SKG_CUDA(cudaMemsetAsync(scal + S_BAR_ERR, 0, sizeof(double), s));
    Bsr<R> a2 = A;
    PcgVecs<R> v2 = v;
    double* p2 = partials;
    double* sc2 = scal;
    void* args[] = {&a2, &v2, &p2, &bar, &sc2};
    SKG_CUDA(cudaLaunchCooperativeKernel((const void*)k_pcg_cg2<R, kG>, dim3(grid), dim3(kCgThreads), args, 0, s));
    res->launches += 1;
  } else if (mode == 1 || mode == 5 || mode == 7) {
    // kernel variant: lanes per row G and rows in flight U (picked by the autotuner);
    // mode 5 is the two-barrier form (pcg_grid.cuh), mode 7 its two-level form (coarse.cuh)
    // mode 7 variants 9..17: the shapes of 0..8 with 768-thread blocks (one per SM); 18..20: the
    // two-barrier form (coarse residual by recurrence) with 768-thread blocks, shapes (4, 2), (8, 2), (2, 2)
    const bool two_barrier = mode == 7 && variant >= 18 && variant <= 20;
    const bool wide = mode == 7 && (variant >= 9 || two_barrier);
#define SKG_PCG_KERN(G_, U_)                                                                              \
  (mode == 7   ? (wide ? (const void*)k_pcg_grid2c<R, G_, U_, 768> : (const void*)k_pcg_grid2c<R, G_, U_>) \
   : mode == 5 ? (const void*)k_pcg_grid2<R, G_, U_>                                                      \
               : (const void*)k_pcg_persistent<R, G_, U_>)
    const void* kern = SKG_PCG_KERN(8, 1);
    int G = 8;
    if (two_barrier) {
      switch (variant) {
        case 18: kern = (const void*)k_pcg_grid2c<R, 4, 2, 768, true>; G = 4; break;
        case 19: kern = (const void*)k_pcg_grid2c<R, 8, 2, 768, true>; G = 8; break;
        default: kern = (const void*)k_pcg_grid2c<R, 2, 2, 768, true>; G = 2; break;
      }
      variant = -1;
    } else if (wide) {
      variant -= 9;
    }
    switch (variant) {
      case 1: kern = SKG_PCG_KERN(16, 1); G = 16; break;
      case 2: kern = SKG_PCG_KERN(8, 2); G = 8; break;
      case 3: kern = SKG_PCG_KERN(16, 2); G = 16; break;
      case 4: kern = SKG_PCG_KERN(4, 2); G = 4; break;
      case 5: kern = SKG_PCG_KERN(4, 4); G = 4; break;
      case 6: kern = SKG_PCG_KERN(2, 4); G = 2; break;
      case 7: kern = SKG_PCG_KERN(8, 4); G = 8; break;
      case 8: kern = SKG_PCG_KERN(2, 2); G = 2; break;
      default: break;
    }
#undef SKG_PCG_KERN
    const int nt = wide ? 768 : kBlock;
    int per_sm = 0;
    SKG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, 0));
    int64_t want = (A.nbr * G + nt - 1) / nt;
    int64_t cap = (int64_t)per_sm * num_sms();
    if (cap > kMaxGrid / 2) cap = kMaxGrid / 2;
    int grid = (int)(want < cap ? want : cap);
    if (grid < 1) grid = 1;
    unsigned* bar = counter + 4;
    SKG_CUDA(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s));
    SKG_CUDA(cudaMemsetAsync(scal + S_BAR_ERR, 0, sizeof(double), s));
    Bsr<R> a2 = A;
    PcgVecs<R> v2 = v;
    double* p2 = partials;
    double* sc2 = scal;
    if (mode == 7) {
      SKG_CUDA(cudaMemsetAsync(cd->rc, 0, sizeof(unsigned long long) * (size_t)cd->np, s));
      CoarseDev c2 = *cd;
      void* args[] = {&a2, &v2, &c2, &p2, &bar, &sc2};
      SKG_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(nt), args, 0, s));
    } else {
      void* args[] = {&a2, &v2, &p2, &bar, &sc2};
      SKG_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(kBlock), args, 0, s));
    }
    res->launches += 1;
  } else {
    const int sb = (int)((A.nbr * kG + kBlock - 1) / kBlock);
    const int spmv_blocks = sb < 4 * num_sms() * 4 ? sb : 4 * num_sms() * 4;
    const int chunk = A.nbr > 20000 ? 8 : 16;
    double hs[2];
    for (int it = 0; it < max_iter; it += chunk) {
      for (int c = 0; c < chunk; ++c) {
        k_pcg_spmv<R, kG><<<spmv_blocks < kMaxGrid ? spmv_blocks : kMaxGrid, kBlock, 0, s>>>(A, v, partials,
                                                                                          counter, scal);
        k_pcg_update<R><<<rb, kBlock, 0, s>>>(A, v, partials, counter, scal);
        k_pcg_direction<R><<<rb, kBlock, 0, s>>>(A.nbr, v, scal);
      }
      res->launches += 3 * chunk;
      SKG_LAUNCHED();
      SKG_CUDA(cudaMemcpyAsync(hs, scal + S_ITERS, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
      SKG_CUDA(cudaStreamSynchronize(s));
      if (hs[1] != 0.0) break;
    }
  }
  if (!read) return SKG_OK;
  double h[10];
  SKG_CUDA(cudaMemcpyAsync(h, scal, 10 * sizeof(double), cudaMemcpyDeviceToHost, s));
  SKG_CUDA(cudaStreamSynchronize(s));
  res->iters = (int)h[S_ITERS];
  res->status = (int)h[S_STATUS];
  res->rr = h[S_RR];
  res->bb = h[S_BB];
  return SKG_OK;
}

// ------------------------------------------------------- Newton / BE ------
static int read_scalars(const double* dev, double* host, int count, cudaStream_t s) {
  SKG_CUDA(cudaMemcpyAsync(host, dev, count * sizeof(double), cudaMemcpyDeviceToHost, s));
  SKG_CUDA(cudaStreamSynchronize(s));
  return SKG_OK;
}

// Eisenstat-Walker choice 2 after the first iteration: eta = gamma (r_k / r_{k-1})^alpha, raised to
// the safeguard gamma eta_{k-1}^alpha when that is above 0.1.  Exponents in quarter steps over [1, 2]
// are evaluated by square roots and products (correctly rounded on the host and the device alike, so
// the host loops and the control kernels take the same decisions); others by pow.
__host__ __device__ inline double ew_pow(double q, double a) {
  if (a == 2.0) return q * q;
  if (a == 1.0) return q;
  const double r2 = sqrt(q), r4 = sqrt(r2);
  if (a == 1.5) return q * r2;
  if (a == 1.25) return q * r4;
  if (a == 1.75) return q * r2 * r4;
  return pow(q, a);
}

__host__ __device__ inline double ew_forcing(double q, double eta_prev, double gamma, double alpha) {
  double e = gamma * ew_pow(q, alpha);
  const double safe = gamma * ew_pow(eta_prev, alpha);
  if (safe > 0.1 && safe > e) e = safe;
  return e;
}

static inline double ew_gamma(const skg_be_params* p) { return p->ew_gamma > 0.0 ? p->ew_gamma : 0.9; }
static inline double ew_alpha(const skg_be_params* p) { return p->ew_alpha > 0.0 ? p->ew_alpha : 2.0; }

// whether a single-mesh step runs the two-level PCG: the whole-mesh form with the grid kernel (mode 7,
// or mode 3 above the cluster size), the per-instance form with the cluster kernel (mode 2, or mode 3 up
// to the cluster size)
template <typename R>
static bool single_two_level(const skg_tet_mesh* m, const skg_be_params* prm) {
  const int64_t n = m->n_verts;
  const bool inst_form = m->coarse && m->coarse->inst_agg;
  const bool small = n <= kClusterAutoRows && n <= cluster_rows_limit<R>();
  return m->coarse && (inst_form ? (prm->pcg_mode == 2 || prm->pcg_mode == 3) && small && m->coarse->n_inst == 1
                                 : prm->pcg_mode == 7 || (prm->pcg_mode == 3 && n > kClusterAutoRows));
}

template <typename R>
static int be_step(const skg_tet_mesh* m, const skg_be_params* prm, const skg_be_state* st, Workspace& w,
                   skg_step_info* info, cudaStream_t s) {
  const int64_t n = m->n_verts, nd = 3 * n;
  const bool mixed = sizeof(R) == 4;
  double inv_h2 = 0.0;  // kinetic factor c / h^2, set with the target
  R* hbuf = mixed ? (R*)w.hbuf32 : (R*)w.hbuf64;
  R* rec = mixed ? (R*)w.rec32 : (R*)w.rec64;
  R* jinv = mixed ? (R*)w.jinv32 : (R*)w.jinv64;
  PcgVecs<R> pv;
  R** vv = mixed ? (R**)w.vec32 : (R**)w.vec64;
  pv.x = vv[0]; pv.r = vv[1]; pv.z = vv[2]; pv.p = vv[3]; pv.q = vv[4]; pv.s = vv[5];
  Bsr<R> A{n, m->bsr_rowptr, m->bsr_col, nullptr, jinv, rec};
  // the first 20% of the block records stay in L2 across PCG iterations, the rest is read
  // evict-first (measured on the 786,432-tet beam: 55.9 -> 52.0 us per two-level iteration with
  // 40% kept; 49.7 us with 20% kept and the dense coarse inverse read with normal priority)
  A.keep = (int64_t)(kKeepFrac * (double)m->n_blocks);

  PhaseTimer pt;
  pt.init(prm->profile != 0, s);
  info->launches = 0;
  info->t_hessian_ms = info->t_assemble_ms = info->t_pcg_ms = info->t_gradient_ms = info->t_energy_ms = 0.0;
  SKG_CUDA(cudaMemsetAsync(w.counter, 0, 16 * sizeof(unsigned), s));
  SKG_TRY(launch_target(prm, st, nd, w.ut, s, &inv_h2));
  info->launches++;

  GradArgs ga{};
  ga.n = n; ga.v2t_ptr = m->v2t_ptr; ga.v2t = m->v2t; ga.fbuf = w.fbuf; ga.mass = st->mass; ga.inv_h2 = inv_h2;
  ga.u = st->u; ga.ut = w.ut; ga.f_ext = st->f_ext; ga.pinned = st->pinned; ga.g = w.g;
  ga.partials = w.partials; ga.counter = w.counter; ga.out = w.scal + S_GG;
  Contact contact;
  SKG_TRY(make_contact(prm, st, &contact));
  ga.contact = contact;

  EnergyArgs<R> ea{};
  if constexpr (sizeof(R) == 4) ea.tet = make_tet_args32(m, st->u, w.uh, w.ul);
  else ea.tet = make_tet_args64(m, st->u);
  ea.n = n; ea.mass = st->mass; ea.inv_h2 = inv_h2; ea.ut = w.ut; ea.f_ext = st->f_ext; ea.pinned = st->pinned;
  ea.contact = contact;
  ea.partials = w.partials; ea.counter = w.counter; ea.out = w.scal + S_E;

  // mixed precision, neo-Hookean materials: forces in double-float from the hi/lo split
  // (the FP64 units of GB300 are the bottleneck of the FP64 force kernel)
  const bool dff = sizeof(R) == 4 && (m->material == kMatSNH || m->material == kMatMMNH || m->material == kMatLE);
  if (dff) {
    SKG_TRY(launch_dinv_lo(m, w.dinv_lo, s));
    info->launches++;
  }
  auto gradient = [&](double* gg) -> int {
    pt.begin();
    if (dff) {
      SKG_TRY(launch_split(st->u, n, w.uh, w.ul, s));
      SKG_TRY(launch_forces_df(make_tet_args64(m, st->u), m->dinv32, w.dinv_lo, w.uh, w.ul, w.fbuf, s));
      info->launches++;
    } else {
      SKG_TRY(launch_forces(make_tet_args64(m, st->u), 1, w.fbuf, s));
    }
    SKG_TRY(launch_vertex_gradient(ga, s, dff));
    info->launches += 2;
    info->t_gradient_ms += pt.end();
    return read_scalars(w.scal + S_GG, gg, 1, s);
  };
  auto energy_launch = [&](const R* dx, double step) -> int {
    ea.dx = dx;
    ea.step = step;
    pt.begin();
    SKG_TRY(launch_energy<R>(ea, false, s));
    info->launches++;
    info->t_energy_ms += pt.end();
    return SKG_OK;
  };
  auto energy = [&](const R* dx, double step, double* e2) -> int {
    SKG_TRY(energy_launch(dx, step));
    return read_scalars(w.scal + S_E, e2, 2, s);
  };
  auto split = [&]() -> int {
    if (!mixed) return SKG_OK;
    info->launches++;
    return launch_split(st->u, n, w.uh, w.ul, s);
  };

  info->newton_iters = 0; info->pcg_iters = 0; info->ls_trials = 0; info->status = SKG_OK;
  info->min_alpha = 1.0;
  // two-level PCG when the mesh has coarse data
  const bool inst_form = m->coarse && m->coarse->inst_agg;
  const bool two_level = single_two_level<R>(m, prm);
  CoarseDev cdev{};
  if (two_level) cdev = make_coarse_dev(m, w);
  double gg;
  SKG_TRY(gradient(&gg));
  const double r0 = sqrt(gg);
  info->residual0 = r0;
  info->residual = r0 > 0.0 ? 1.0 : 0.0;
  if (!isfinite(r0)) {
    info->status = SKG_ERR_NONFINITE;
    return SKG_OK;
  }
  SKG_TRY(split());
  double ecur[2];
  SKG_TRY(energy(nullptr, 0.0, ecur));
  const double eps_r = mixed ? 5.96e-8 : 1.11e-16;
  double res_prev = 1.0, eta_prev = 0.0;
  // stop_rule 1 is simkit's newton_solver (solvers/newton.py:43-75): at least one iteration, then
  // stop once ||alpha dx|| < tol, at most max_newton iterations, no convergence status
  const bool simkit_stop = prm->stop_rule == 1;
  skg_newton_record* nrec = prm->record;
  for (int it = 0; it < prm->max_newton && (r0 > 0.0 || simkit_stop); ++it) {
    const double res = r0 > 0.0 ? sqrt(gg) / r0 : 0.0;
    info->residual = res;
    if (!simkit_stop && res < prm->tol) break;
    const bool record = nrec && it < nrec->capacity;
    if (record) {
      SKG_CUDA(cudaMemcpyAsync(nrec->g + (int64_t)it * nd, w.g, nd * sizeof(double), cudaMemcpyDeviceToDevice, s));
      nrec->residual_h[it] = res;
      nrec->alpha_h[it] = 0.0;
      nrec->pcg_iters_h[it] = 0;
    }
    // PCG forcing term: fixed (pcg_rtol > 0) or Eisenstat-Walker choice 2
    // (gamma 0.9, exponent 2, safeguarded) capped at |pcg_rtol|, never
    // tighter than what brings the residual to a quarter of tol; the first
    // one is |pcg_rtol| times the start's relative residual (1 here)
    double eta = prm->pcg_rtol;
    if (prm->pcg_rtol < 0.0) {
      const double eta_max = -prm->pcg_rtol;
      if (it == 0) {
        eta = eta_max * (res < 1.0 ? res : 1.0);   // 1 from x_tilde; a closer start gets a tighter first solve
      } else {
        eta = ew_forcing(res / res_prev, eta_prev, ew_gamma(prm), ew_alpha(prm));
      }
      const double reach = 0.25 * prm->tol / res;
      if (eta < reach) eta = reach;
      if (eta > eta_max) eta = eta_max;
      if (eta < 1e-8) eta = 1e-8;
    }
    res_prev = res;
    eta_prev = eta;
    // H(u) + M/h^2 with pinned rows/columns, block-Jacobi inverses
    pt.begin();
    if constexpr (sizeof(R) == 4) {
      int hl = 1;
      SKG_TRY(launch_tet_hessian<float>(make_tet_args32(m, st->u, w.uh, w.ul), 1, 1, (float*)hbuf, s,
                                        HessLate{w.hlate, w.hlate_n, &hl}));
      info->launches += hl - 1;
    } else {
      SKG_TRY(launch_tet_hessian<double>(make_tet_args64(m, st->u), 1, 1, (double*)hbuf, s));
    }
    info->t_hessian_ms += pt.end();
    AsmArgs<R> aa = make_asm_args<R>(m, hbuf, nullptr, jinv);
    aa.rec = rec;
    aa.mass = st->mass;
    aa.inv_h2 = inv_h2;
    aa.contact = contact;
    aa.u = st->u;
    aa.pinned = st->pinned;
    aa.cmode = two_level && !inst_form ? cdev.mode : nullptr;
    aa.colpack = two_level && inst_form ? cdev.colpack : nullptr;
    pt.begin();
    SKG_TRY(launch_assemble<R>(aa, s));
    info->launches += 2;
    // coarse operator of the two-level preconditioner (timed with the assembly)
    if (two_level && ((it == 0 && prm->coarse_refresh >= 0) || prm->coarse_refresh > 0)) {
      SKG_TRY(coarse_refresh<R>(A, cdev, w.scal, s));
      info->launches += 2;
    }
    info->t_assemble_ms += pt.end();
    // dx = -H^-1 g
    PcgResult pr{};
    pt.begin();
    SKG_TRY(pcg_solve<R>(A, w.g, -1.0, st->pinned, pv, eta, prm->pcg_max_iter, prm->pcg_mode, w.partials,
                         w.counter, w.scal, s, &pr, prm->pcg_variant, two_level ? &cdev : nullptr, false));
    info->t_pcg_ms += pt.end();
    info->launches += pr.launches;
    if (record) {
      k_unpad<R><<<blocks_for(n), kBlock, 0, s>>>(pv.x, n, nrec->dx + (int64_t)it * nd);
      SKG_LAUNCHED();
      info->launches++;
    }
    // Armijo backtracking (simkit/backtracking_line_search.py:56-67).  The slope g.dx and the first
    // trial (step 1) are enqueued behind the PCG, and one host round trip reads the PCG's scalars,
    // the slope and that trial's energy (a failed solve discards the two)
    k_dot_g<R><<<reduce_blocks(n), kBlock, 0, s>>>(w.g, pv.x, n, w.partials, w.counter, w.scal + S_SLOPE);
    SKG_LAUNCHED();
    info->launches++;
    if (prm->do_line_search && prm->ls_max_iter > 0) SKG_TRY(energy_launch(pv.x, 1.0));
    double hs[S_SLOPE + 2];
    SKG_TRY(read_scalars(w.scal, hs, S_SLOPE + 2, s));
    pr.iters = (int)hs[S_ITERS];
    pr.status = (int)hs[S_STATUS];
    info->pcg_iters += pr.iters;
    info->newton_iters = it + 1;   // a failed solve counts as the iteration it ended
    if (record) nrec->pcg_iters_h[it] = pr.iters;
    if (pr.status != 0) {
      info->status = pr.status;
      break;
    }
    const double slope_dd[2] = {hs[S_SLOPE], hs[S_SLOPE + 1]};
    const double slope = slope_dd[0];
    double step = 1.0, enew[2] = {ecur[0], ecur[1]};
    bool accepted = !prm->do_line_search;
    if (prm->do_line_search) {
      const double thr = prm->ls_threshold >= 0.0 ? prm->ls_threshold : 1e-12 + 16.0 * eps_r * ecur[1];
      for (int k = 0; k < prm->ls_max_iter; ++k) {
        if (k == 0) {
          enew[0] = hs[S_E];
          enew[1] = hs[S_E + 1];
        } else {
          SKG_TRY(energy(pv.x, step, enew));
        }
        info->ls_trials++;
        if (enew[0] <= ecur[0] + prm->ls_alpha * step * slope + thr) {
          accepted = true;
          break;
        }
        step *= prm->ls_beta;
      }
    }
    info->newton_iters = it + 1;
    if (record) nrec->alpha_h[it] = accepted ? step : 0.0;
    if (!accepted) {
      // simkit returns t = 0 (backtracking_line_search.py:66-67) and Newton
      // stops because ||0 * dx|| < tol (newton.py:69)
      info->status = SKG_ERR_LINESEARCH;
      break;
    }
    k_apply_step<R><<<blocks_for(n), kBlock, 0, s>>>(st->u, pv.x, step, n, st->pinned);
    SKG_LAUNCHED();
    info->launches++;
    if (step < info->min_alpha) info->min_alpha = step;
    SKG_TRY(split());
    if (prm->do_line_search) {
      ecur[0] = enew[0];
      ecur[1] = enew[1];
    } else {
      SKG_TRY(energy(nullptr, 0.0, ecur));
    }
    SKG_TRY(gradient(&gg));
    if (!isfinite(gg)) {
      info->status = SKG_ERR_NONFINITE;
      break;
    }
    info->residual = r0 > 0.0 ? sqrt(gg) / r0 : 0.0;
    if (simkit_stop && step * sqrt(slope_dd[1]) < prm->tol) break;
  }
  if (!simkit_stop && info->status == SKG_OK && info->residual >= prm->tol && r0 > 0.0)
    info->status = SKG_ERR_NOT_CONVERGED;
  info->energy = ecur[0];
  return SKG_OK;
}


// ---------------------------------------------------------------- batched --
// Many independent meshes (instances) concatenated into one mesh with
// disjoint vertex and tet ranges.  The element, assembly and gradient kernels
// run over the concatenation (masked per instance); per-instance sums are one
// CTA per instance in a fixed order; each instance's PCG runs on a
// thread-block cluster taken from a largest-first queue; Newton, the forcing
// term and the line search are per instance.

__global__ void __launch_bounds__(kBlock) k_inst_sumsq(const double* __restrict__ g, const int32_t* __restrict__ rows,
                                                       double* __restrict__ out) {
  const int inst = blockIdx.x;
  double acc[1] = {0.0};
  for (int64_t d = 3 * (int64_t)rows[inst] + threadIdx.x; d < 3 * (int64_t)rows[inst + 1]; d += blockDim.x)
    acc[0] += g[d] * g[d];
  block_sum<1, kBlock>(acc);
  if (threadIdx.x == 0) out[inst] = acc[0];
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_inst_dot(const double* __restrict__ g, const R* __restrict__ dx,
                                                     const int32_t* __restrict__ rows, const uint8_t* __restrict__ mask,
                                                     double* __restrict__ out) {
  const int inst = blockIdx.x;
  if (mask && !mask[inst]) return;
  double acc[1] = {0.0};
  for (int64_t v = rows[inst] + threadIdx.x; v < rows[inst + 1]; v += blockDim.x) {
    const Vec3<R> d = ld3c(dx, v);
    acc[0] += g[3 * v] * double(d.x) + g[3 * v + 1] * double(d.y) + g[3 * v + 2] * double(d.z);
  }
  block_sum<1, kBlock>(acc);
  if (threadIdx.x == 0) out[inst] = acc[0];
}

template <typename R>
__global__ void k_apply_step_batched(double* __restrict__ u, const R* __restrict__ dx, const double* __restrict__ steps,
                                     const uint8_t* __restrict__ accept, const int32_t* __restrict__ vert_inst, int64_t n,
                                     const uint8_t* __restrict__ pinned) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  const int inst = vert_inst[v];
  if (!accept[inst]) return;
  const double step = steps[inst];
  const Vec3<R> d = ld3c(dx, v);
  const double dd[3] = {double(d.x), double(d.y), double(d.z)};
#pragma unroll
  for (int c = 0; c < 3; ++c)
    if (!(pinned && pinned[3 * v + c])) u[3 * v + c] += step * dd[c];
}

// u = use[inst] ? u_warm : u_tilde per vertex
__global__ void k_choose_start(double* __restrict__ u, const double* __restrict__ uw, const double* __restrict__ ut,
                               const uint8_t* __restrict__ use, const int32_t* __restrict__ vert_inst, int64_t n) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  const double* src = use[vert_inst[v]] ? uw : ut;
#pragma unroll
  for (int c = 0; c < 3; ++c) u[3 * v + c] = src[3 * v + c];
}

struct BatchWs {
  uint8_t* active;
  uint8_t* mask;
  double* eta;
  double* steps;
  double* gg;
  double* slope;
  double* e2;
  int32_t* pcg_it;
  int32_t* pcg_st;
  unsigned* queue;
  // device-resident Newton loop (batch plans): per-instance control state
  uint8_t* accept;
  double* g0;
  double* fnorm;
  double* res_prev;
  double* eta_prev;
  double* ecur;           // 2 per instance: incremental potential and its magnitude
  skg_step_info* info;    // n_inst per-instance records, then the total
  int32_t* ctr;           // loop counters (see BatchCtl)
  int64_t bytes;
};

static BatchWs carve_batch(const skg_tet_mesh* m, const skg_batch* b, int precision, void* base) {
  Workspace w0 = carve_workspace(m, precision, nullptr);
  Carve c(base ? static_cast<char*>(base) + w0.bytes : nullptr);
  const int64_t ni = b->n_inst;
  BatchWs w{};
  w.active = c.take<uint8_t>(ni);
  w.mask = c.take<uint8_t>(ni);
  w.eta = c.take<double>(ni);
  w.steps = c.take<double>(ni);
  w.gg = c.take<double>(ni);
  w.slope = c.take<double>(ni);
  w.e2 = c.take<double>(2 * ni);
  w.pcg_it = c.take<int32_t>(ni);
  w.pcg_st = c.take<int32_t>(ni);
  w.queue = c.take<unsigned>(8);
  w.accept = c.take<uint8_t>(ni);
  w.g0 = c.take<double>(ni);
  w.fnorm = c.take<double>(ni);
  w.res_prev = c.take<double>(ni);
  w.eta_prev = c.take<double>(ni);
  w.ecur = c.take<double>(2 * ni);
  w.info = c.take<skg_step_info>(ni + 1);
  w.ctr = c.take<int32_t>(8);
  w.bytes = w0.bytes + c.off + 256;
  return w;
}

// Streams the batched PCG forks its size classes onto (created once per thread).
struct ClassStreams {
  cudaStream_t s[5] = {};
  cudaEvent_t fork = nullptr, join[5] = {};
  bool ready = false;
};

// All active instances' PCG solves.  Each instance gets the smallest cluster
// (a power of two, at least min_cluster) whose CTAs hold its vectors in shared
// memory; instances are ordered largest first, so the instances of one cluster
// size are a contiguous range of the order and each range is one launch of the
// queue kernel.  The launches run concurrently on their own streams, each with
// a number of clusters proportional to the block rows of its active instances,
// so the classes finish together; within a launch, clusters take instances
// from the range largest first.  plan_pcg_classes does the host-side part (class
// ranges, cluster counts, kernel attributes, the class streams); launch_pcg_classes
// only enqueues, so a graph capture can record it.
struct PcgClassPlan {
  int n = 0;
  int begin[5], end[5], size[5], nclusters[5];
  bool two_level = false;
};

template <typename R>
static const void* pcg_queue_kernel(bool two_level) {
  return two_level ? (const void*)k_pcg_cluster_queue<R, kGc, true> : (const void*)k_pcg_cluster_queue<R, kGc, false>;
}

static ClassStreams& class_streams() {
  static thread_local ClassStreams cs;
  return cs;
}

template <typename R>
static int plan_pcg_classes(const skg_batch* bt, const int32_t* rows_h, const int32_t* order_h,
                            const uint8_t* active_h, int min_cluster, int vec_kb, bool two_level, PcgClassPlan* p) {
  const void* kern = pcg_queue_kernel<R>(two_level);
  static thread_local bool configured[2] = {false, false};
  if (!configured[two_level ? 1 : 0]) {
    SKG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    SKG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kClusterSmemBudget));
    configured[two_level ? 1 : 0] = true;
  }
  ClassStreams& cs = class_streams();
  if (!cs.ready) {
    for (int c = 0; c < 5; ++c) {
      SKG_CUDA(cudaStreamCreateWithFlags(&cs.s[c], cudaStreamNonBlocking));
      SKG_CUDA(cudaEventCreateWithFlags(&cs.join[c], cudaEventDisableTiming));
    }
    SKG_CUDA(cudaEventCreateWithFlags(&cs.fork, cudaEventDisableTiming));
    cs.ready = true;
  }
  // with the two-level data the instance's coarse vectors take the last kCoarseSmem bytes
  const int64_t budget = two_level ? kClusterSmemBudget - kCoarseSmem : kClusterSmemBudget;
  const int ni = bt->n_inst;
  if (min_cluster <= 0) min_cluster = kClusterMinDefault;
  int cmin = 1;
  while (cmin < min_cluster && cmin < kClusterMax) cmin *= 2;
  // smallest cluster of at least cmin CTAs whose per-CTA vectors take at most `target`
  // bytes (the rest holds block records), else the smallest that holds the vectors at all
  int64_t target = vec_kb > 0 ? (int64_t)vec_kb * 1024 : (int64_t)kClusterVecTarget;
  if (target > budget) target = budget;
  auto need = [&](int inst) {
    const int64_t rows = rows_h[inst + 1] - rows_h[inst];
    int c = cmin;
    while (c < kClusterMax && cluster_vec_bytes(rows, c, (int)sizeof(R)) > target) c *= 2;
    if (cluster_vec_bytes(rows, c, (int)sizeof(R)) > target) {
      c = cmin;
      while (c < kClusterMax && cluster_vec_bytes(rows, c, (int)sizeof(R)) > budget) c *= 2;
    }
    return c;
  };
  // the cluster size never grows along the order (a smaller instance fits wherever a larger
  // one does), so the classes are at most five contiguous ranges
  double cls_rows[5];
  double total_rows = 0.0;
  std::vector<int> csz(ni);
  for (int k = 0; k < ni; ++k) csz[k] = k == 0 ? need(order_h[0]) : std::min(need(order_h[k]), csz[k - 1]);
  p->n = 0;
  p->two_level = two_level;
  for (int k = 0; k < ni;) {
    const int c = csz[k];
    int e = k;
    double w = 0.0;
    while (e < ni && csz[e] == c) {
      const int inst = order_h[e];
      if (active_h[inst]) w += rows_h[inst + 1] - rows_h[inst];
      ++e;
    }
    if (p->n == 5) return fail(SKG_ERR_ARG, "batched PCG: more than five cluster sizes");
    p->begin[p->n] = k;
    p->end[p->n] = e;
    p->size[p->n] = c;
    cls_rows[p->n] = w;
    total_rows += w;
    ++p->n;
    k = e;
  }
  const int sms = num_sms();
  for (int c = 0; c < p->n; ++c) {
    p->nclusters[c] = 0;
    if (cls_rows[c] <= 0.0) continue;
    const int csize = p->size[c];
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kClusterThreads, 1, 1);
    cfg.dynamicSmemBytes = kClusterSmemBudget;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(csize, 1, 1);
    int fit = 0;
    SKG_CUDA(cudaOccupancyMaxActiveClusters(&fit, kern, &cfg));
    if (fit < 1) return fail(SKG_ERR_CUDA, "batched PCG: no cluster of %d CTAs fits", csize);
    int nclusters = (int)(sms * cls_rows[c] / total_rows / csize + 0.5);
    if (nclusters < 1) nclusters = 1;
    if (nclusters > fit) nclusters = fit;
    if (nclusters > p->end[c] - p->begin[c]) nclusters = p->end[c] - p->begin[c];
    p->nclusters[c] = nclusters;
  }
  return SKG_OK;
}

template <typename R>
static int launch_pcg_classes(const PcgClassPlan& p, const Bsr<R>& A, const skg_batch* bt, const uint8_t* active,
                              const double* eta, const double* b, const uint8_t* pinned, R* xout, int max_iter,
                              int32_t* it_out, int32_t* st_out, unsigned* queue, cudaStream_t s, int* launches,
                              const CoarseDev* cd = nullptr) {
  int any = 0;
  for (int c = 0; c < p.n; ++c) any += p.nclusters[c];
  if (any == 0) return SKG_OK;
  const void* kern = pcg_queue_kernel<R>(p.two_level);
  const int64_t budget = p.two_level ? kClusterSmemBudget - kCoarseSmem : kClusterSmemBudget;
  ClassStreams& cs = class_streams();
  SKG_CUDA(cudaMemsetAsync(queue, 0, 8 * sizeof(unsigned), s));
  if (cd) SKG_CUDA(cudaMemsetAsync(cd->rc, 0, sizeof(unsigned long long) * 6 * (size_t)cd->n_agg, s));
  CoarseDev c2 = cd ? *cd : CoarseDev{};
  SKG_CUDA(cudaEventRecord(cs.fork, s));
  for (int c = 0; c < p.n; ++c) {
    if (p.nclusters[c] <= 0) continue;
    const int csize = p.size[c];
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kClusterThreads, 1, 1);
    cfg.dynamicSmemBytes = kClusterSmemBudget;
    cfg.stream = cs.s[c];
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(csize * p.nclusters[c], 1, 1);
    SKG_CUDA(cudaStreamWaitEvent(cs.s[c], cs.fork, 0));
    Bsr<R> a2 = A;
    const int32_t* ord = bt->order + p.begin[c];
    int ncls_inst = p.end[c] - p.begin[c];
    double bs = -1.0;
    unsigned* qc = queue + c;
    int smem = (int)budget;
    void* args[] = {&a2, (void*)&bt->inst_rows, (void*)&ord, &ncls_inst, (void*)&active, (void*)&eta, (void*)&b, &bs,
                    (void*)&pinned, &xout, &max_iter, &it_out, &st_out, &qc, &smem, &c2};
    SKG_CUDA(cudaLaunchKernelExC(&cfg, kern, args));
    SKG_CUDA(cudaEventRecord(cs.join[c], cs.s[c]));
    SKG_CUDA(cudaStreamWaitEvent(s, cs.join[c], 0));
    ++*launches;
  }
  return SKG_OK;
}

template <typename R>
static int be_step_batched(const skg_tet_mesh* m, const skg_batch* bt, const skg_be_params* prm,
                           const skg_be_state* st, void* wsbase, skg_step_info* infos, skg_step_info* total,
                           cudaStream_t s) {
  const int64_t n = m->n_verts, nd = 3 * n;
  const int ni = bt->n_inst;
  const bool mixed = sizeof(R) == 4;
  double inv_h2 = 0.0;  // kinetic factor c / h^2, set with the target
  Workspace w = carve_workspace(m, prm->precision, wsbase);
  BatchWs bw = carve_batch(m, bt, prm->precision, wsbase);
  R* hbuf = mixed ? (R*)w.hbuf32 : (R*)w.hbuf64;
  R* rec = mixed ? (R*)w.rec32 : (R*)w.rec64;
  R* jinv = mixed ? (R*)w.jinv32 : (R*)w.jinv64;
  R** vv = mixed ? (R**)w.vec32 : (R**)w.vec64;
  R* dx = vv[0];
  Bsr<R> A{n, m->bsr_rowptr, m->bsr_col, nullptr, jinv, rec};
  PhaseTimer pt;
  pt.init(prm->profile != 0, s);
  *total = skg_step_info{};

  std::vector<uint8_t> active(ni, 0), mask(ni, 0);
  std::vector<double> g0(ni), gg(ni), eta(ni, 0.0), res_prev(ni, 1.0), eta_prev(ni, 0.0), steps(ni, 1.0),
      slope(ni), ecur(2 * ni), etry(2 * ni);
  std::vector<int32_t> pit(ni), pst(ni);
  for (int i = 0; i < ni; ++i) {
    infos[i] = skg_step_info{};
    infos[i].min_alpha = 1.0;
  }

  // instance offsets and order on the host (the size classes of the PCG launch)
  std::vector<int32_t> rows_h(ni + 1), order_h(ni);
  SKG_CUDA(cudaMemcpyAsync(rows_h.data(), bt->inst_rows, (ni + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  SKG_CUDA(cudaMemcpyAsync(order_h.data(), bt->order, ni * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  SKG_CUDA(cudaMemsetAsync(w.counter, 0, 16 * sizeof(unsigned), s));
  SKG_TRY(launch_target(prm, st, nd, w.ut, s, &inv_h2));
  GradArgs ga{};
  ga.n = n; ga.v2t_ptr = m->v2t_ptr; ga.v2t = m->v2t; ga.fbuf = w.fbuf; ga.mass = st->mass; ga.inv_h2 = inv_h2;
  ga.u = st->u; ga.ut = w.ut; ga.f_ext = st->f_ext; ga.pinned = st->pinned; ga.g = w.g;
  ga.partials = w.partials; ga.counter = w.counter; ga.out = w.scal + S_GG;
  Contact contact;
  SKG_TRY(make_contact(prm, st, &contact));
  ga.contact = contact;
  EnergyArgs<R> ea{};
  if constexpr (sizeof(R) == 4) ea.tet = make_tet_args32(m, st->u, w.uh, w.ul);
  else ea.tet = make_tet_args64(m, st->u);
  ea.n = n; ea.mass = st->mass; ea.inv_h2 = inv_h2; ea.ut = w.ut; ea.f_ext = st->f_ext; ea.pinned = st->pinned;
  ea.contact = contact;
  int launches = 1;

  const bool dff = sizeof(R) == 4 && (m->material == kMatSNH || m->material == kMatMMNH || m->material == kMatLE);
  if (dff) {
    SKG_TRY(launch_dinv_lo(m, w.dinv_lo, s));
    launches++;
  }
  auto gradient = [&]() -> int {
    pt.begin();
    if (dff) {
      SKG_TRY(launch_split(st->u, n, w.uh, w.ul, s));
      SKG_TRY(launch_forces_df(make_tet_args64(m, st->u), m->dinv32, w.dinv_lo, w.uh, w.ul, w.fbuf, s));
      launches++;
    } else {
      SKG_TRY(launch_forces(make_tet_args64(m, st->u), 1, w.fbuf, s));
    }
    SKG_TRY(launch_vertex_gradient(ga, s, dff));
    k_inst_sumsq<<<ni, kBlock, 0, s>>>(w.g, bt->inst_rows, bw.gg);
    SKG_LAUNCHED();
    launches += 3;
    total->t_gradient_ms += pt.end();
    SKG_CUDA(cudaMemcpyAsync(gg.data(), bw.gg, ni * sizeof(double), cudaMemcpyDeviceToHost, s));
    SKG_CUDA(cudaStreamSynchronize(s));
    return SKG_OK;
  };
  auto energy = [&](const R* d, const double* steps_dev, const uint8_t* mask_dev, double* out_h) -> int {
    ea.dx = d;
    pt.begin();
    SKG_TRY(launch_inst_energy<R>(ea, ni, bt->inst_rows, bt->inst_tets, mask_dev, steps_dev, bw.e2, s));
    launches++;
    total->t_energy_ms += pt.end();
    SKG_CUDA(cudaMemcpyAsync(out_h, bw.e2, 2 * ni * sizeof(double), cudaMemcpyDeviceToHost, s));
    SKG_CUDA(cudaStreamSynchronize(s));
    return SKG_OK;
  };
  auto split = [&]() -> int {
    if (!mixed) return SKG_OK;
    launches++;
    return launch_split(st->u, n, w.uh, w.ul, s);
  };

  // per-instance |f_ext|: the absolute residual floor 1e-10 |f_ext| (far below any physical
  // force, far above FP64 force-evaluation noise) ends instances that settle at rest, where
  // 1e-6 of ||g(x_tilde)|| is below the noise of the gradient itself
  std::vector<double> fnorm(ni);
  k_inst_sumsq<<<ni, kBlock, 0, s>>>(st->f_ext ? st->f_ext : w.g, bt->inst_rows, bw.gg);
  SKG_LAUNCHED();
  SKG_CUDA(cudaMemcpyAsync(fnorm.data(), bw.gg, ni * sizeof(double), cudaMemcpyDeviceToHost, s));
  SKG_TRY(gradient());
  int n_active = 0;
  for (int i = 0; i < ni; ++i) {
    fnorm[i] = st->f_ext ? sqrt(fnorm[i]) : 0.0;
    g0[i] = sqrt(gg[i]);
    infos[i].residual0 = g0[i];
    infos[i].residual = g0[i] > 0.0 ? 1.0 : 0.0;
    if (!isfinite(g0[i])) infos[i].status = SKG_ERR_NONFINITE;
  }
  SKG_TRY(split());
  SKG_TRY(energy(nullptr, nullptr, nullptr, ecur.data()));
  if (st->u_warm) {
    // residual-judged warm start: keep it per instance only where its gradient norm is below the
    // one at x_tilde (the start then begins Newton at a relative residual below 1)
    SKG_CUDA(cudaMemcpyAsync(st->u, st->u_warm, nd * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SKG_TRY(gradient());
    for (int i = 0; i < ni; ++i) {
      mask[i] = (isfinite(gg[i]) && sqrt(gg[i]) < g0[i]) ? 1 : 0;
      infos[i].warm_used = mask[i];
    }
    SKG_CUDA(cudaMemcpyAsync(bw.mask, mask.data(), ni, cudaMemcpyHostToDevice, s));
    k_choose_start<<<blocks_for(n), kBlock, 0, s>>>(st->u, st->u_warm, w.ut, bw.mask, bt->vert_inst, n);
    SKG_LAUNCHED();
    launches++;
    SKG_TRY(split());
    SKG_TRY(energy(nullptr, nullptr, nullptr, ecur.data()));
    SKG_TRY(gradient());
  }
  const double eps_r = mixed ? 5.96e-8 : 1.11e-16;
  // two-level PCG with the per-instance coarse data, when attached (one instance per mesh of the batch)
  const bool two_level = m->coarse && m->coarse->inst_agg && m->coarse->n_inst == bt->n_inst;
  CoarseDev cdev{};
  if (two_level) cdev = make_coarse_dev(m, w);
  for (int it = 0; it < prm->max_newton; ++it) {
    n_active = 0;
    for (int i = 0; i < ni; ++i) {
      active[i] = 0;
      if (infos[i].status != SKG_OK || !(g0[i] > 0.0)) continue;
      const double res = sqrt(gg[i]) / g0[i];
      infos[i].residual = res;
      if (res < prm->tol || sqrt(gg[i]) < 1e-10 * fnorm[i]) continue;
      double e = prm->pcg_rtol;
      if (prm->pcg_rtol < 0.0) {
        const double emax = -prm->pcg_rtol;
        if (it == 0) {
          e = emax * (res < 1.0 ? res : 1.0);   // a start closer than x_tilde gets a tighter first solve
        } else {
          e = ew_forcing(res / res_prev[i], eta_prev[i], ew_gamma(prm), ew_alpha(prm));
        }
        const double reach = 0.25 * prm->tol / res;
        if (e < reach) e = reach;
        if (e > emax) e = emax;
        if (e < 1e-8) e = 1e-8;
      }
      res_prev[i] = res;
      eta_prev[i] = e;
      eta[i] = e;
      active[i] = 1;
      ++n_active;
    }
    if (n_active == 0) break;
    SKG_CUDA(cudaMemcpyAsync(bw.active, active.data(), ni, cudaMemcpyHostToDevice, s));
    SKG_CUDA(cudaMemcpyAsync(bw.eta, eta.data(), ni * sizeof(double), cudaMemcpyHostToDevice, s));
    // Hessians and assembly of the active instances
    pt.begin();
    if constexpr (sizeof(R) == 4) {
      TetArgs<float> ta = make_tet_args32(m, st->u, w.uh, w.ul);
      ta.tet_inst = bt->tet_inst;
      ta.inst_active = bw.active;
      int hl = 1;
      SKG_TRY(launch_tet_hessian<float>(ta, 1, 1, (float*)hbuf, s, HessLate{w.hlate, w.hlate_n, &hl}));
      launches += hl - 1;
    } else {
      TetArgs<double> ta = make_tet_args64(m, st->u);
      ta.tet_inst = bt->tet_inst;
      ta.inst_active = bw.active;
      SKG_TRY(launch_tet_hessian<double>(ta, 1, 1, (double*)hbuf, s));
    }
    total->t_hessian_ms += pt.end();
    AsmArgs<R> aa = make_asm_args<R>(m, hbuf, nullptr, jinv);
    aa.rec = rec;
    aa.mass = st->mass;
    aa.inv_h2 = inv_h2;
    aa.contact = contact;
    aa.u = st->u;
    aa.pinned = st->pinned;
    aa.vert_inst = bt->vert_inst;
    aa.inst_active = bw.active;
    aa.colpack = two_level ? cdev.colpack : nullptr;
    pt.begin();
    SKG_TRY(launch_assemble<R>(aa, s));
    // per-instance coarse operators of the two-level PCG (every instance is active at the first
    // Newton iteration of the step)
    if (two_level && ((it == 0 && prm->coarse_refresh >= 0) || prm->coarse_refresh > 0)) {
      SKG_TRY(coarse_refresh<R>(A, cdev, w.scal, s, bt->order));
      launches += 2;
    }
    total->t_assemble_ms += pt.end();
    // all active instances' PCG solves, one cluster per instance at a time
    pt.begin();
    PcgClassPlan cp;
    SKG_TRY(plan_pcg_classes<R>(bt, rows_h.data(), order_h.data(), active.data(), prm->batch_min_cluster,
                                prm->batch_vec_kb, two_level, &cp));
    SKG_TRY(launch_pcg_classes<R>(cp, A, bt, bw.active, bw.eta, w.g, st->pinned, dx, prm->pcg_max_iter, bw.pcg_it,
                                  bw.pcg_st, bw.queue, s, &launches, two_level ? &cdev : nullptr));
    total->t_pcg_ms += pt.end();
    launches += 2;
    SKG_CUDA(cudaMemcpyAsync(pit.data(), bw.pcg_it, ni * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    SKG_CUDA(cudaMemcpyAsync(pst.data(), bw.pcg_st, ni * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    k_inst_dot<R><<<ni, kBlock, 0, s>>>(w.g, dx, bt->inst_rows, bw.active, bw.slope);
    SKG_LAUNCHED();
    launches++;
    SKG_CUDA(cudaMemcpyAsync(slope.data(), bw.slope, ni * sizeof(double), cudaMemcpyDeviceToHost, s));
    SKG_CUDA(cudaStreamSynchronize(s));
    // line search per instance (simkit/backtracking_line_search.py:56-67)
    int searching = 0;
    for (int i = 0; i < ni; ++i) {
      mask[i] = 0;
      if (!active[i]) continue;
      infos[i].pcg_iters += pit[i];
      infos[i].newton_iters = it + 1;
      if (pst[i] != 0) {
        infos[i].status = pst[i];
        active[i] = 0;
        continue;
      }
      steps[i] = 1.0;
      mask[i] = 1;
      ++searching;
    }
    std::vector<uint8_t> accept(ni, 0);
    for (int k = 0; k < prm->ls_max_iter && searching > 0; ++k) {
      SKG_CUDA(cudaMemcpyAsync(bw.mask, mask.data(), ni, cudaMemcpyHostToDevice, s));
      SKG_CUDA(cudaMemcpyAsync(bw.steps, steps.data(), ni * sizeof(double), cudaMemcpyHostToDevice, s));
      SKG_TRY(energy(dx, bw.steps, bw.mask, etry.data()));
      searching = 0;
      for (int i = 0; i < ni; ++i) {
        if (!mask[i]) continue;
        infos[i].ls_trials++;
        const double thr =
            prm->ls_threshold >= 0.0 ? prm->ls_threshold : 1e-12 + 16.0 * eps_r * ecur[2 * i + 1];
        if (!prm->do_line_search || etry[2 * i] <= ecur[2 * i] + prm->ls_alpha * steps[i] * slope[i] + thr) {
          accept[i] = 1;
          mask[i] = 0;
          ecur[2 * i] = etry[2 * i];
          ecur[2 * i + 1] = etry[2 * i + 1];
          if (steps[i] < infos[i].min_alpha) infos[i].min_alpha = steps[i];
        } else {
          steps[i] *= prm->ls_beta;
          ++searching;
        }
      }
    }
    for (int i = 0; i < ni; ++i)
      if (mask[i]) {  // exhausted: simkit returns t = 0 and its Newton loop stops
        infos[i].status = SKG_ERR_LINESEARCH;
        active[i] = 0;
      }
    SKG_CUDA(cudaMemcpyAsync(bw.mask, accept.data(), ni, cudaMemcpyHostToDevice, s));
    SKG_CUDA(cudaMemcpyAsync(bw.steps, steps.data(), ni * sizeof(double), cudaMemcpyHostToDevice, s));
    k_apply_step_batched<R><<<blocks_for(n), kBlock, 0, s>>>(st->u, dx, bw.steps, bw.mask, bt->vert_inst, n,
                                                             st->pinned);
    SKG_LAUNCHED();
    launches++;
    SKG_TRY(split());
    SKG_TRY(gradient());
  }
  for (int i = 0; i < ni; ++i) {
    if (infos[i].status == SKG_OK && g0[i] > 0.0) {
      infos[i].residual = sqrt(gg[i]) / g0[i];
      if (!(infos[i].residual < prm->tol) && !(sqrt(gg[i]) < 1e-10 * fnorm[i]))
        infos[i].status = SKG_ERR_NOT_CONVERGED;
    }
    infos[i].energy = ecur[2 * i];
    total->newton_iters += infos[i].newton_iters;
    total->pcg_iters += infos[i].pcg_iters;
    total->ls_trials += infos[i].ls_trials;
    if (infos[i].status != SKG_OK && total->status == SKG_OK) total->status = infos[i].status;
  }
  total->launches = launches;
  return SKG_OK;
}

// ------------------------------------------- device-resident batched loop --
// The batched step of be_step_batched with every per-instance decision made on the device and
// the whole step recorded once into a CUDA graph (skg_batch_plan).  Newton's relative-residual
// test, the Eisenstat-Walker forcing, the Armijo search and the stop are small control kernels
// between the solver's kernels; the Newton iterations and the line-search trials are
// conditional WHILE nodes whose conditions those kernels set (cudaGraphSetConditional), and the
// coarse refresh of the first iteration is a conditional IF node.  One graph launch runs the
// step; the host reads the per-instance records once at the end.  Every decision uses the
// arithmetic of be_step_batched's host loop, in the same order.

constexpr int kCtlThreads = 512;
enum { kCtrIter = 0, kCtrTrial = 1, kCtrTrials = 2, kCtrRefresh = 3 };

struct CtlParams {
  double tol, pcg_rtol, ls_alpha, ls_beta, ls_threshold, eps_r, ew_gamma, ew_alpha;
  int max_newton, ls_max_iter, do_line_search, coarse_refresh, has_fext, two_level;
};

struct BatchCtl {
  int ni;
  uint8_t *active, *mask, *accept;
  double *eta, *steps, *gg, *slope, *e2, *g0, *fnorm, *res_prev, *eta_prev, *ecur;
  int32_t *pit, *pst, *ctr;
  skg_step_info* info;
  const double* pscal = nullptr;   // one-instance plans: the PCG's iterations and status read from its scalars
};

static BatchCtl make_ctl(const BatchWs& bw, int ni) {
  BatchCtl c{};
  c.ni = ni;
  c.active = bw.active; c.mask = bw.mask; c.accept = bw.accept;
  c.eta = bw.eta; c.steps = bw.steps; c.gg = bw.gg; c.slope = bw.slope; c.e2 = bw.e2; c.g0 = bw.g0;
  c.fnorm = bw.fnorm; c.res_prev = bw.res_prev; c.eta_prev = bw.eta_prev; c.ecur = bw.ecur;
  c.pit = bw.pcg_it; c.pst = bw.pcg_st; c.ctr = bw.ctr; c.info = bw.info;
  return c;
}

// sum of v over the block (one control block of kCtlThreads)
__device__ __forceinline__ int ctl_block_sum(int v) {
  __shared__ int tot;
  if (threadIdx.x == 0) tot = 0;
  __syncthreads();
  if (v) atomicAdd(&tot, v);
  __syncthreads();
  const int r = tot;
  __syncthreads();
  return r;
}

// after the first gradient (gg at x_tilde, f_ext's squared norm in fnorm) and energy (e2)
__global__ void __launch_bounds__(kCtlThreads) k_bctl_begin(BatchCtl c, CtlParams p) {
  for (int i = threadIdx.x; i < c.ni; i += blockDim.x) {
    skg_step_info f{};
    f.min_alpha = 1.0;
    c.g0[i] = sqrt(c.gg[i]);
    c.fnorm[i] = p.has_fext ? sqrt(c.fnorm[i]) : 0.0;
    f.residual0 = c.g0[i];
    f.residual = c.g0[i] > 0.0 ? 1.0 : 0.0;
    if (!isfinite(c.g0[i])) f.status = SKG_ERR_NONFINITE;
    c.info[i] = f;
    c.res_prev[i] = 1.0;
    c.eta_prev[i] = 0.0;
    c.ecur[2 * i] = c.e2[2 * i];
    c.ecur[2 * i + 1] = c.e2[2 * i + 1];
  }
  if (threadIdx.x < 8) c.ctr[threadIdx.x] = 0;
}

// residual-judged warm start: kept per instance where its gradient norm is below the one at x_tilde (g0)
__global__ void __launch_bounds__(kCtlThreads) k_bctl_warm(BatchCtl c) {
  for (int i = threadIdx.x; i < c.ni; i += blockDim.x) {
    const bool keep = isfinite(c.gg[i]) && sqrt(c.gg[i]) < c.g0[i];
    c.mask[i] = keep ? 1 : 0;
    c.info[i].warm_used = keep ? 1 : 0;
  }
}

__global__ void __launch_bounds__(kCtlThreads) k_bctl_take_energy(BatchCtl c) {
  for (int i = threadIdx.x; i < 2 * c.ni; i += blockDim.x) c.ecur[i] = c.e2[i];
}

// top of a Newton iteration: convergence test and forcing term per instance; the loop goes on
// while an instance is active and fewer than max_newton iterations ran
__global__ void __launch_bounds__(kCtlThreads) k_bctl_newton(BatchCtl c, CtlParams p,
                                                             cudaGraphConditionalHandle loop) {
  const int it = c.ctr[kCtrIter];
  int na = 0;
  for (int i = threadIdx.x; i < c.ni; i += blockDim.x) {
    c.active[i] = 0;
    skg_step_info& f = c.info[i];
    if (f.status != SKG_OK) continue;
    if (!isfinite(c.gg[i])) {   // as the host loop: a non-finite gradient ends the step
      f.status = SKG_ERR_NONFINITE;
      continue;
    }
    if (it >= p.max_newton || !(c.g0[i] > 0.0)) continue;
    const double res = sqrt(c.gg[i]) / c.g0[i];
    f.residual = res;
    if (res < p.tol || sqrt(c.gg[i]) < 1e-10 * c.fnorm[i]) continue;
    double e = p.pcg_rtol;
    if (p.pcg_rtol < 0.0) {
      const double emax = -p.pcg_rtol;
      if (it == 0) {
        e = emax * (res < 1.0 ? res : 1.0);   // as the host loop: the first forcing scales with the start's residual
      } else {
        e = ew_forcing(res / c.res_prev[i], c.eta_prev[i], p.ew_gamma, p.ew_alpha);
      }
      const double reach = 0.25 * p.tol / res;
      if (e < reach) e = reach;
      if (e > emax) e = emax;
      if (e < 1e-8) e = 1e-8;
    }
    c.res_prev[i] = res;
    c.eta_prev[i] = e;
    c.eta[i] = e;
    c.active[i] = 1;
    ++na;
  }
  const int tot = ctl_block_sum(na);
  if (threadIdx.x == 0) cudaGraphSetConditional(loop, tot > 0 ? 1u : 0u);
}

// whether this iteration rebuilds the per-instance coarse operators
__global__ void k_bctl_refresh(BatchCtl c, CtlParams p, cudaGraphConditionalHandle refresh) {
  const int it = c.ctr[kCtrIter];
  const bool r = p.two_level && ((it == 0 && p.coarse_refresh >= 0) || p.coarse_refresh > 0);
  if (r) c.ctr[kCtrRefresh] += 1;
  cudaGraphSetConditional(refresh, r ? 1u : 0u);
}

// after the solves: per-instance PCG results, search start (step 1) for the instances that solved
__global__ void __launch_bounds__(kCtlThreads) k_bctl_search(BatchCtl c, CtlParams p, cudaGraphConditionalHandle ls) {
  const int it = c.ctr[kCtrIter];
  int ns = 0;
  for (int i = threadIdx.x; i < c.ni; i += blockDim.x) {
    c.mask[i] = 0;
    c.accept[i] = 0;
    if (!c.active[i]) continue;
    skg_step_info& f = c.info[i];
    const int32_t pit = c.pscal ? (int32_t)c.pscal[S_ITERS] : c.pit[i];
    const int32_t pst = c.pscal ? (int32_t)c.pscal[S_STATUS] : c.pst[i];
    f.pcg_iters += pit;
    f.newton_iters = it + 1;
    if (pst != 0) {
      f.status = pst;
      c.active[i] = 0;
      continue;
    }
    c.steps[i] = 1.0;
    c.mask[i] = 1;
    ++ns;
  }
  const int tot = ctl_block_sum(ns);
  if (threadIdx.x == 0) {
    c.ctr[kCtrTrial] = 0;
    cudaGraphSetConditional(ls, tot > 0 && p.ls_max_iter > 0 ? 1u : 0u);
  }
}

// one Armijo trial (simkit/backtracking_line_search.py:56-67) for the instances still searching
__global__ void __launch_bounds__(kCtlThreads) k_bctl_trial(BatchCtl c, CtlParams p, cudaGraphConditionalHandle ls) {
  int ns = 0;
  for (int i = threadIdx.x; i < c.ni; i += blockDim.x) {
    if (!c.mask[i]) continue;
    skg_step_info& f = c.info[i];
    f.ls_trials++;
    const double thr = p.ls_threshold >= 0.0 ? p.ls_threshold : 1e-12 + 16.0 * p.eps_r * c.ecur[2 * i + 1];
    if (!p.do_line_search || c.e2[2 * i] <= c.ecur[2 * i] + p.ls_alpha * c.steps[i] * c.slope[i] + thr) {
      c.accept[i] = 1;
      c.mask[i] = 0;
      c.ecur[2 * i] = c.e2[2 * i];
      c.ecur[2 * i + 1] = c.e2[2 * i + 1];
      if (c.steps[i] < f.min_alpha) f.min_alpha = c.steps[i];
    } else {
      c.steps[i] *= p.ls_beta;
      ++ns;
    }
  }
  const int tot = ctl_block_sum(ns);
  if (threadIdx.x == 0) {
    const int k = ++c.ctr[kCtrTrial];
    c.ctr[kCtrTrials] += 1;
    cudaGraphSetConditional(ls, tot > 0 && k < p.ls_max_iter ? 1u : 0u);
  }
}

// exhausted searches: simkit returns t = 0 and its Newton loop stops
__global__ void __launch_bounds__(kCtlThreads) k_bctl_searched(BatchCtl c) {
  for (int i = threadIdx.x; i < c.ni; i += blockDim.x)
    if (c.mask[i]) {
      c.info[i].status = SKG_ERR_LINESEARCH;
      c.active[i] = 0;
    }
  if (threadIdx.x == 0) c.ctr[kCtrIter] += 1;
}

// final residuals, statuses and energies; the total record after the instances
__global__ void __launch_bounds__(kCtlThreads) k_bctl_final(BatchCtl c, CtlParams p) {
  __shared__ int sn, sp, sl, sfirst;
  if (threadIdx.x == 0) {
    sn = sp = sl = 0;
    sfirst = c.ni;
  }
  __syncthreads();
  int n = 0, pc = 0, l = 0, first = c.ni;
  for (int i = threadIdx.x; i < c.ni; i += blockDim.x) {
    skg_step_info& f = c.info[i];
    if (f.status == SKG_OK && c.g0[i] > 0.0) {
      f.residual = sqrt(c.gg[i]) / c.g0[i];
      if (!(f.residual < p.tol) && !(sqrt(c.gg[i]) < 1e-10 * c.fnorm[i])) f.status = SKG_ERR_NOT_CONVERGED;
    }
    f.energy = c.ecur[2 * i];
    n += f.newton_iters;
    pc += f.pcg_iters;
    l += f.ls_trials;
    if (f.status != SKG_OK && i < first) first = i;
  }
  atomicAdd(&sn, n);
  atomicAdd(&sp, pc);
  atomicAdd(&sl, l);
  atomicMin(&sfirst, first);
  __syncthreads();
  if (threadIdx.x == 0) {
    skg_step_info t{};
    t.newton_iters = sn;
    t.pcg_iters = sp;
    t.ls_trials = sl;
    t.status = sfirst < c.ni ? c.info[sfirst].status : SKG_OK;
    c.info[c.ni] = t;
  }
}

}  // namespace skg

// One batched step recorded as an executable CUDA graph for fixed buffers.
struct skg_batch_plan {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap[3] = {nullptr, nullptr, nullptr};
  void* own = nullptr;            // device control state the plan allocated (single-mesh plans)
  skg_step_info* info = nullptr;  // device: n_inst records, then the total
  int32_t* ctr = nullptr;         // device loop counters
  int ni = 0;
  // kernel launches: before the loop, per Newton iteration, per search trial, per coarse refresh, after
  int l_pre = 0, l_iter = 0, l_trial = 0, l_refresh = 0, l_post = 0;
};

namespace skg {

// a conditional node of `type` at the capture position of `s`, its body graph returned; the
// capture of `s` continues after the node
static int add_conditional(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                           cudaGraph_t* body) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  SKG_CUDA(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
  if (st != cudaStreamCaptureStatusActive) return fail(SKG_ERR_CUDA, "batch plan: stream is not capturing");
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = type;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  SKG_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &np));
  *body = np.conditional.phGraph_out[0];
  SKG_CUDA(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return SKG_OK;
}

// a condition handle of the graph `s` is capturing into
static int capture_handle(cudaStream_t s, cudaGraphConditionalHandle* h) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  SKG_CUDA(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr));
  if (st != cudaStreamCaptureStatusActive) return fail(SKG_ERR_CUDA, "batch plan: stream is not capturing");
  SKG_CUDA(cudaGraphConditionalHandleCreate(h, g, 0, cudaGraphCondAssignDefault));
  return SKG_OK;
}

// Records the batched step into plan->graph with the plan's three capture streams.
template <typename R>
static int capture_batch_step(const skg_tet_mesh* m, const skg_batch* bt, const skg_be_params* prm,
                              const skg_be_state* st, void* wsbase, skg_batch_plan* plan) {
  const int64_t n = m->n_verts, nd = 3 * n;
  const int ni = bt->n_inst;
  const bool mixed = sizeof(R) == 4;
  Workspace w = carve_workspace(m, prm->precision, wsbase);
  BatchWs bw = carve_batch(m, bt, prm->precision, wsbase);
  R* hbuf = mixed ? (R*)w.hbuf32 : (R*)w.hbuf64;
  R* rec = mixed ? (R*)w.rec32 : (R*)w.rec64;
  R* jinv = mixed ? (R*)w.jinv32 : (R*)w.jinv64;
  R** vv = mixed ? (R**)w.vec32 : (R**)w.vec64;
  R* dx = vv[0];
  Bsr<R> A{n, m->bsr_rowptr, m->bsr_col, nullptr, jinv, rec};
  const BatchCtl ctl = make_ctl(bw, ni);
  plan->info = bw.info;
  plan->ctr = bw.ctr;
  plan->ni = ni;
  const bool two_level = m->coarse && m->coarse->inst_agg && m->coarse->n_inst == bt->n_inst;
  CoarseDev cdev{};
  if (two_level) cdev = make_coarse_dev(m, w);

  // host-side preparation: instance offsets and order, the PCG size classes (every instance
  // counted: the queue kernel skips the inactive ones), the contact planes
  std::vector<int32_t> rows_h(ni + 1), order_h(ni);
  SKG_CUDA(cudaMemcpy(rows_h.data(), bt->inst_rows, (ni + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost));
  SKG_CUDA(cudaMemcpy(order_h.data(), bt->order, ni * sizeof(int32_t), cudaMemcpyDeviceToHost));
  std::vector<uint8_t> all(ni, 1);
  PcgClassPlan cp;
  SKG_TRY(plan_pcg_classes<R>(bt, rows_h.data(), order_h.data(), all.data(), prm->batch_min_cluster,
                              prm->batch_vec_kb, two_level, &cp));
  Contact contact;
  SKG_TRY(make_contact(prm, st, &contact));
  CtlParams cpar{};
  cpar.tol = prm->tol; cpar.pcg_rtol = prm->pcg_rtol; cpar.ew_gamma = ew_gamma(prm); cpar.ew_alpha = ew_alpha(prm); cpar.ls_alpha = prm->ls_alpha; cpar.ls_beta = prm->ls_beta;
  cpar.ls_threshold = prm->ls_threshold; cpar.eps_r = mixed ? 5.96e-8 : 1.11e-16;
  cpar.max_newton = prm->max_newton; cpar.ls_max_iter = prm->ls_max_iter; cpar.do_line_search = prm->do_line_search;
  cpar.coarse_refresh = prm->coarse_refresh; cpar.has_fext = st->f_ext != nullptr; cpar.two_level = two_level;

  cudaStream_t s0 = plan->cap[0], s1 = plan->cap[1], s2 = plan->cap[2];
  double inv_h2 = 0.0;
  int launches = 0;
  SKG_CUDA(cudaGraphCreate(&plan->graph, 0));
  SKG_CUDA(cudaStreamBeginCaptureToGraph(s0, plan->graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));

  // ---- before the loop: target, first gradient and energy, optional warm start
  SKG_CUDA(cudaMemsetAsync(w.counter, 0, 16 * sizeof(unsigned), s0));
  SKG_TRY(launch_target(prm, st, nd, w.ut, s0, &inv_h2));
  launches++;
  GradArgs ga{};
  ga.n = n; ga.v2t_ptr = m->v2t_ptr; ga.v2t = m->v2t; ga.fbuf = w.fbuf; ga.mass = st->mass; ga.inv_h2 = inv_h2;
  ga.u = st->u; ga.ut = w.ut; ga.f_ext = st->f_ext; ga.pinned = st->pinned; ga.g = w.g;
  ga.partials = w.partials; ga.counter = w.counter; ga.out = w.scal + S_GG;
  ga.contact = contact;
  EnergyArgs<R> ea{};
  if constexpr (sizeof(R) == 4) ea.tet = make_tet_args32(m, st->u, w.uh, w.ul);
  else ea.tet = make_tet_args64(m, st->u);
  ea.n = n; ea.mass = st->mass; ea.inv_h2 = inv_h2; ea.ut = w.ut; ea.f_ext = st->f_ext; ea.pinned = st->pinned;
  ea.contact = contact;
  const bool dff = mixed && (m->material == kMatSNH || m->material == kMatMMNH || m->material == kMatLE);
  if (dff) {
    SKG_TRY(launch_dinv_lo(m, w.dinv_lo, s0));
    launches++;
  }
  auto gradient = [&](cudaStream_t s) -> int {
    if (dff) {
      SKG_TRY(launch_split(st->u, n, w.uh, w.ul, s));
      SKG_TRY(launch_forces_df(make_tet_args64(m, st->u), m->dinv32, w.dinv_lo, w.uh, w.ul, w.fbuf, s));
      launches++;
    } else {
      SKG_TRY(launch_forces(make_tet_args64(m, st->u), 1, w.fbuf, s));
    }
    SKG_TRY(launch_vertex_gradient(ga, s, dff));
    k_inst_sumsq<<<ni, kBlock, 0, s>>>(w.g, bt->inst_rows, bw.gg);
    SKG_LAUNCHED();
    launches += 3;
    return SKG_OK;
  };
  auto energy = [&](const R* d, const double* steps_dev, const uint8_t* mask_dev, cudaStream_t s) -> int {
    ea.dx = d;
    SKG_TRY(launch_inst_energy<R>(ea, ni, bt->inst_rows, bt->inst_tets, mask_dev, steps_dev, bw.e2, s));
    launches++;
    return SKG_OK;
  };
  auto split = [&](cudaStream_t s) -> int {
    if (!mixed) return SKG_OK;
    launches++;
    return launch_split(st->u, n, w.uh, w.ul, s);
  };
  if (st->f_ext) {
    k_inst_sumsq<<<ni, kBlock, 0, s0>>>(st->f_ext, bt->inst_rows, bw.fnorm);
    SKG_LAUNCHED();
    launches++;
  }
  SKG_TRY(gradient(s0));
  SKG_TRY(split(s0));
  SKG_TRY(energy(nullptr, nullptr, nullptr, s0));
  k_bctl_begin<<<1, kCtlThreads, 0, s0>>>(ctl, cpar);
  SKG_LAUNCHED();
  launches++;
  if (st->u_warm) {
    SKG_CUDA(cudaMemcpyAsync(st->u, st->u_warm, nd * sizeof(double), cudaMemcpyDeviceToDevice, s0));
    SKG_TRY(gradient(s0));
    k_bctl_warm<<<1, kCtlThreads, 0, s0>>>(ctl);
    SKG_LAUNCHED();
    k_choose_start<<<blocks_for(n), kBlock, 0, s0>>>(st->u, st->u_warm, w.ut, bw.mask, bt->vert_inst, n);
    SKG_LAUNCHED();
    launches += 2;
    SKG_TRY(split(s0));
    SKG_TRY(energy(nullptr, nullptr, nullptr, s0));
    k_bctl_take_energy<<<1, kCtlThreads, 0, s0>>>(ctl);
    SKG_LAUNCHED();
    launches++;
    SKG_TRY(gradient(s0));
  }
  cudaGraphConditionalHandle h_loop;
  SKG_TRY(capture_handle(s0, &h_loop));
  k_bctl_newton<<<1, kCtlThreads, 0, s0>>>(ctl, cpar, h_loop);
  SKG_LAUNCHED();
  launches++;
  plan->l_pre = launches;

  // ---- the Newton loop
  cudaGraph_t body = nullptr;
  SKG_TRY(add_conditional(s0, h_loop, cudaGraphCondTypeWhile, &body));
  SKG_CUDA(cudaStreamBeginCaptureToGraph(s1, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  launches = 0;
  if constexpr (sizeof(R) == 4) {
    TetArgs<float> ta = make_tet_args32(m, st->u, w.uh, w.ul);
    ta.tet_inst = bt->tet_inst;
    ta.inst_active = bw.active;
    int hl = 1;
    SKG_TRY(launch_tet_hessian<float>(ta, 1, 1, (float*)hbuf, s1, HessLate{w.hlate, w.hlate_n, &hl}));
    launches += hl - 1;
  } else {
    TetArgs<double> ta = make_tet_args64(m, st->u);
    ta.tet_inst = bt->tet_inst;
    ta.inst_active = bw.active;
    SKG_TRY(launch_tet_hessian<double>(ta, 1, 1, (double*)hbuf, s1));
  }
  AsmArgs<R> aa = make_asm_args<R>(m, hbuf, nullptr, jinv);
  aa.rec = rec;
  aa.mass = st->mass;
  aa.inv_h2 = inv_h2;
  aa.contact = contact;
  aa.u = st->u;
  aa.pinned = st->pinned;
  aa.vert_inst = bt->vert_inst;
  aa.inst_active = bw.active;
  aa.colpack = two_level ? cdev.colpack : nullptr;
  SKG_TRY(launch_assemble<R>(aa, s1));
  launches += 2;
  if (two_level) {
    cudaGraphConditionalHandle h_ref;
    SKG_TRY(capture_handle(s1, &h_ref));
    k_bctl_refresh<<<1, 1, 0, s1>>>(ctl, cpar, h_ref);
    SKG_LAUNCHED();
    launches++;
    cudaGraph_t rbody = nullptr;
    SKG_TRY(add_conditional(s1, h_ref, cudaGraphCondTypeIf, &rbody));
    SKG_CUDA(cudaStreamBeginCaptureToGraph(s2, rbody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    SKG_TRY(coarse_refresh<R>(A, cdev, w.scal, s2, bt->order));
    SKG_CUDA(cudaStreamEndCapture(s2, &rbody));
    plan->l_refresh = 2;
  }
  SKG_TRY(launch_pcg_classes<R>(cp, A, bt, bw.active, bw.eta, w.g, st->pinned, dx, prm->pcg_max_iter, bw.pcg_it,
                                bw.pcg_st, bw.queue, s1, &launches, two_level ? &cdev : nullptr));
  k_inst_dot<R><<<ni, kBlock, 0, s1>>>(w.g, dx, bt->inst_rows, bw.active, bw.slope);
  SKG_LAUNCHED();
  cudaGraphConditionalHandle h_ls;
  SKG_TRY(capture_handle(s1, &h_ls));
  k_bctl_search<<<1, kCtlThreads, 0, s1>>>(ctl, cpar, h_ls);
  SKG_LAUNCHED();
  launches += 2;
  {
    cudaGraph_t lbody = nullptr;
    SKG_TRY(add_conditional(s1, h_ls, cudaGraphCondTypeWhile, &lbody));
    SKG_CUDA(cudaStreamBeginCaptureToGraph(s2, lbody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const int before = launches;
    SKG_TRY(energy(dx, bw.steps, bw.mask, s2));
    k_bctl_trial<<<1, kCtlThreads, 0, s2>>>(ctl, cpar, h_ls);
    SKG_LAUNCHED();
    launches++;
    plan->l_trial = launches - before;
    launches = before;
    SKG_CUDA(cudaStreamEndCapture(s2, &lbody));
  }
  k_bctl_searched<<<1, kCtlThreads, 0, s1>>>(ctl);
  SKG_LAUNCHED();
  k_apply_step_batched<R><<<blocks_for(n), kBlock, 0, s1>>>(st->u, dx, bw.steps, bw.accept, bt->vert_inst, n,
                                                            st->pinned);
  SKG_LAUNCHED();
  launches += 2;
  SKG_TRY(split(s1));
  SKG_TRY(gradient(s1));
  k_bctl_newton<<<1, kCtlThreads, 0, s1>>>(ctl, cpar, h_loop);
  SKG_LAUNCHED();
  launches++;
  SKG_CUDA(cudaStreamEndCapture(s1, &body));
  plan->l_iter = launches;

  // ---- after the loop
  k_bctl_final<<<1, kCtlThreads, 0, s0>>>(ctl, cpar);
  SKG_LAUNCHED();
  plan->l_post = 1;
  SKG_CUDA(cudaStreamEndCapture(s0, &plan->graph));
  SKG_CUDA(cudaGraphInstantiate(&plan->exec, plan->graph, 0));
  return SKG_OK;
}

// ---------------------------------------------- single mesh, device loop --
// One skg_be_step recorded as a graph: the Newton loop and the line search are conditional WHILE
// nodes decided by the batch control kernels over one instance, the reductions are the whole-mesh
// ones of the host loop (gradient norm, energy, slope) writing into the control state, and the PCG
// reads its forcing term from it.  The same kernels in the same order with the same arithmetic as
// be_step: the two take bitwise the same steps.

// The end of a Newton iteration of the one-instance device loop: the search bookkeeping of
// k_bctl_searched (an exhausted search sets the status; the iteration counter), u += steps[0] dx on
// free DOFs when the search accepted a step (k_apply_step's arithmetic), and with SPLIT the hi/lo
// split of u for the FP32 kernels (k_split's)
template <typename R, bool SPLIT>
__global__ void k_sctl_apply(BatchCtl c, double* __restrict__ u, const R* __restrict__ dx, int64_t n,
                             const uint8_t* __restrict__ pinned, float* __restrict__ uh, float* __restrict__ ul) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v == 0) {
    if (c.mask[0]) {
      c.info[0].status = SKG_ERR_LINESEARCH;
      c.active[0] = 0;
    }
    c.ctr[kCtrIter] += 1;
  }
  if (v >= n) return;
  if (c.accept[0]) {
    const double step = c.steps[0];
    const Vec3<R> d = ld3c(dx, v);
    const double dd[3] = {double(d.x), double(d.y), double(d.z)};
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (!(pinned && pinned[3 * v + k])) u[3 * v + k] += step * dd[k];
  }
  if constexpr (SPLIT) {
    float h[3], l[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double x = u[3 * v + k];
      h[k] = float(x);
      l[k] = float(x - double(h[k]));
    }
    reinterpret_cast<float4*>(uh)[v] = make_float4(h[0], h[1], h[2], 0.f);
    reinterpret_cast<float4*>(ul)[v] = make_float4(l[0], l[1], l[2], 0.f);
  }
}

// control state of one instance: flags, per-instance scalars (two slots each: the slope buffer takes
// g.dx and dx.dx), counters and two step records (the instance's, then the total); base null: sizes only
static BatchCtl carve_single_ctl(void* base, int64_t* bytes) {
  Carve cv(base);
  BatchCtl c{};
  c.ni = 1;
  c.active = cv.take<uint8_t>(16); c.mask = cv.take<uint8_t>(16); c.accept = cv.take<uint8_t>(16);
  c.eta = cv.take<double>(2); c.steps = cv.take<double>(2); c.gg = cv.take<double>(2);
  c.slope = cv.take<double>(2); c.e2 = cv.take<double>(2); c.g0 = cv.take<double>(2);
  c.fnorm = cv.take<double>(2); c.res_prev = cv.take<double>(2); c.eta_prev = cv.take<double>(2);
  c.ecur = cv.take<double>(2);
  c.pit = cv.take<int32_t>(2); c.pst = cv.take<int32_t>(2); c.ctr = cv.take<int32_t>(8);
  c.info = cv.take<skg_step_info>(2);
  *bytes = cv.off;
  return c;
}

// whether skg_be_step with these parameters can be recorded: no profiling, no Newton record,
// the relative-residual stop rule, and a PCG form that takes its tolerance from the device
template <typename R>
static bool single_plan_eligible(const skg_tet_mesh* m, const skg_be_params* prm) {
  if (prm->profile || prm->record || prm->stop_rule != 0) return false;
  const bool two_level = single_two_level<R>(m, prm);
  const bool grid_form = two_level && !m->coarse->inst_agg;
  const int mode = resolve_pcg_mode<R>(prm->pcg_mode, m->n_verts, grid_form);
  return mode == 1 || mode == 4 || mode == 5 || mode == 7;
}

template <typename R>
static int capture_single_step(const skg_tet_mesh* m, const skg_be_params* prm, const skg_be_state* st,
                               void* wsbase, skg_batch_plan* plan) {
  const int64_t n = m->n_verts, nd = 3 * n;
  const bool mixed = sizeof(R) == 4;
  Workspace w = carve_workspace(m, prm->precision, wsbase);
  R* hbuf = mixed ? (R*)w.hbuf32 : (R*)w.hbuf64;
  R* rec = mixed ? (R*)w.rec32 : (R*)w.rec64;
  R* jinv = mixed ? (R*)w.jinv32 : (R*)w.jinv64;
  PcgVecs<R> pv;
  R** vv = mixed ? (R**)w.vec32 : (R**)w.vec64;
  pv.x = vv[0]; pv.r = vv[1]; pv.z = vv[2]; pv.p = vv[3]; pv.q = vv[4]; pv.s = vv[5];
  Bsr<R> A{n, m->bsr_rowptr, m->bsr_col, nullptr, jinv, rec};
  A.keep = (int64_t)(kKeepFrac * (double)m->n_blocks);
  int64_t ctl_bytes = 0;
  carve_single_ctl(nullptr, &ctl_bytes);
  SKG_CUDA(cudaMalloc(&plan->own, ctl_bytes));
  SKG_CUDA(cudaMemset(plan->own, 0, ctl_bytes));
  BatchCtl c = carve_single_ctl(plan->own, &ctl_bytes);
  c.pscal = w.scal;
  plan->info = c.info;
  plan->ctr = c.ctr;
  plan->ni = 1;
  const bool inst_form = m->coarse && m->coarse->inst_agg;
  const bool two_level = single_two_level<R>(m, prm);
  CoarseDev cdev{};
  if (two_level) cdev = make_coarse_dev(m, w);
  Contact contact;
  SKG_TRY(make_contact(prm, st, &contact));
  CtlParams cpar{};
  cpar.tol = prm->tol; cpar.pcg_rtol = prm->pcg_rtol; cpar.ew_gamma = ew_gamma(prm); cpar.ew_alpha = ew_alpha(prm); cpar.ls_alpha = prm->ls_alpha; cpar.ls_beta = prm->ls_beta;
  cpar.ls_threshold = prm->ls_threshold; cpar.eps_r = mixed ? 5.96e-8 : 1.11e-16;
  cpar.max_newton = prm->max_newton; cpar.ls_max_iter = prm->ls_max_iter; cpar.do_line_search = prm->do_line_search;
  cpar.coarse_refresh = prm->coarse_refresh; cpar.two_level = two_level;
  cpar.has_fext = 0;   // the host loop's stop rule: the relative residual alone

  cudaStream_t s0 = plan->cap[0], s1 = plan->cap[1], s2 = plan->cap[2];
  double inv_h2 = 0.0;
  int launches = 0;
  SKG_CUDA(cudaGraphCreate(&plan->graph, 0));
  SKG_CUDA(cudaStreamBeginCaptureToGraph(s0, plan->graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));

  // ---- before the loop: target, first gradient and energy
  SKG_CUDA(cudaMemsetAsync(w.counter, 0, 16 * sizeof(unsigned), s0));
  SKG_TRY(launch_target(prm, st, nd, w.ut, s0, &inv_h2));
  launches++;
  GradArgs ga{};
  ga.n = n; ga.v2t_ptr = m->v2t_ptr; ga.v2t = m->v2t; ga.fbuf = w.fbuf; ga.mass = st->mass; ga.inv_h2 = inv_h2;
  ga.u = st->u; ga.ut = w.ut; ga.f_ext = st->f_ext; ga.pinned = st->pinned; ga.g = w.g;
  ga.partials = w.partials; ga.counter = w.counter; ga.out = c.gg;
  ga.contact = contact;
  EnergyArgs<R> ea{};
  if constexpr (sizeof(R) == 4) ea.tet = make_tet_args32(m, st->u, w.uh, w.ul);
  else ea.tet = make_tet_args64(m, st->u);
  ea.n = n; ea.mass = st->mass; ea.inv_h2 = inv_h2; ea.ut = w.ut; ea.f_ext = st->f_ext; ea.pinned = st->pinned;
  ea.contact = contact;
  ea.partials = w.partials; ea.counter = w.counter; ea.out = c.e2;
  const bool dff = mixed && (m->material == kMatSNH || m->material == kMatMMNH || m->material == kMatLE);
  if (dff) {
    SKG_TRY(launch_dinv_lo(m, w.dinv_lo, s0));
    launches++;
  }
  auto gradient = [&](cudaStream_t s, bool split_done) -> int {   // split_done: uh, ul already hold u
    if (dff) {
      if (!split_done) SKG_TRY(launch_split(st->u, n, w.uh, w.ul, s));
      SKG_TRY(launch_forces_df(make_tet_args64(m, st->u), m->dinv32, w.dinv_lo, w.uh, w.ul, w.fbuf, s));
      launches += split_done ? 0 : 1;
    } else {
      SKG_TRY(launch_forces(make_tet_args64(m, st->u), 1, w.fbuf, s));
    }
    SKG_TRY(launch_vertex_gradient(ga, s, dff));
    launches += 2;
    return SKG_OK;
  };
  auto energy = [&](const R* dx, const double* step_dev, cudaStream_t s) -> int {
    ea.dx = dx;
    ea.step = 0.0;
    ea.step_dev = step_dev;
    SKG_TRY(launch_energy<R>(ea, false, s));
    launches++;
    return SKG_OK;
  };
  auto split = [&](cudaStream_t s) -> int {
    if (!mixed) return SKG_OK;
    launches++;
    return launch_split(st->u, n, w.uh, w.ul, s);
  };
  SKG_TRY(gradient(s0, false));
  SKG_TRY(split(s0));
  SKG_TRY(energy(nullptr, nullptr, s0));
  k_bctl_begin<<<1, kCtlThreads, 0, s0>>>(c, cpar);
  SKG_LAUNCHED();
  cudaGraphConditionalHandle h_loop;
  SKG_TRY(capture_handle(s0, &h_loop));
  k_bctl_newton<<<1, kCtlThreads, 0, s0>>>(c, cpar, h_loop);
  SKG_LAUNCHED();
  launches += 2;
  plan->l_pre = launches;

  // ---- the Newton loop
  cudaGraph_t body = nullptr;
  SKG_TRY(add_conditional(s0, h_loop, cudaGraphCondTypeWhile, &body));
  SKG_CUDA(cudaStreamBeginCaptureToGraph(s1, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  launches = 0;
  if constexpr (sizeof(R) == 4) {
    int hl = 1;
    SKG_TRY(launch_tet_hessian<float>(make_tet_args32(m, st->u, w.uh, w.ul), 1, 1, (float*)hbuf, s1,
                                      HessLate{w.hlate, w.hlate_n, &hl}));
    launches += hl;
  } else {
    SKG_TRY(launch_tet_hessian<double>(make_tet_args64(m, st->u), 1, 1, (double*)hbuf, s1));
    launches++;
  }
  AsmArgs<R> aa = make_asm_args<R>(m, hbuf, nullptr, jinv);
  aa.rec = rec;
  aa.mass = st->mass;
  aa.inv_h2 = inv_h2;
  aa.contact = contact;
  aa.u = st->u;
  aa.pinned = st->pinned;
  aa.cmode = two_level && !inst_form ? cdev.mode : nullptr;
  aa.colpack = two_level && inst_form ? cdev.colpack : nullptr;
  SKG_TRY(launch_assemble<R>(aa, s1));
  launches++;
  if (two_level) {
    cudaGraphConditionalHandle h_ref;
    SKG_TRY(capture_handle(s1, &h_ref));
    k_bctl_refresh<<<1, 1, 0, s1>>>(c, cpar, h_ref);
    SKG_LAUNCHED();
    launches++;
    cudaGraph_t rbody = nullptr;
    SKG_TRY(add_conditional(s1, h_ref, cudaGraphCondTypeIf, &rbody));
    SKG_CUDA(cudaStreamBeginCaptureToGraph(s2, rbody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    SKG_TRY(coarse_refresh<R>(A, cdev, w.scal, s2));
    SKG_CUDA(cudaStreamEndCapture(s2, &rbody));
    plan->l_refresh = 2;
  }
  // dx = -H^-1 g to the forcing term k_bctl_newton left in c.eta
  PcgResult pr{};
  SKG_TRY(pcg_solve<R>(A, w.g, -1.0, st->pinned, pv, 0.0, prm->pcg_max_iter, prm->pcg_mode, w.partials, w.counter,
                       w.scal, s1, &pr, prm->pcg_variant, two_level ? &cdev : nullptr, false, c.eta));
  launches += pr.launches;
  k_dot_g<R><<<reduce_blocks(n), kBlock, 0, s1>>>(w.g, pv.x, n, w.partials, w.counter, c.slope);
  SKG_LAUNCHED();
  cudaGraphConditionalHandle h_ls;
  SKG_TRY(capture_handle(s1, &h_ls));
  k_bctl_search<<<1, kCtlThreads, 0, s1>>>(c, cpar, h_ls);
  SKG_LAUNCHED();
  launches += 2;
  {
    cudaGraph_t lbody = nullptr;
    SKG_TRY(add_conditional(s1, h_ls, cudaGraphCondTypeWhile, &lbody));
    SKG_CUDA(cudaStreamBeginCaptureToGraph(s2, lbody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const int before = launches;
    SKG_TRY(energy(pv.x, c.steps, s2));
    k_bctl_trial<<<1, kCtlThreads, 0, s2>>>(c, cpar, h_ls);
    SKG_LAUNCHED();
    launches++;
    plan->l_trial = launches - before;
    launches = before;
    SKG_CUDA(cudaStreamEndCapture(s2, &lbody));
  }
  k_sctl_apply<R, sizeof(R) == 4><<<blocks_for(n), kBlock, 0, s1>>>(c, st->u, pv.x, n, st->pinned, w.uh, w.ul);
  SKG_LAUNCHED();
  launches++;
  SKG_TRY(gradient(s1, mixed));
  k_bctl_newton<<<1, kCtlThreads, 0, s1>>>(c, cpar, h_loop);
  SKG_LAUNCHED();
  launches++;
  SKG_CUDA(cudaStreamEndCapture(s1, &body));
  plan->l_iter = launches;

  // ---- after the loop
  k_bctl_final<<<1, kCtlThreads, 0, s0>>>(c, cpar);
  SKG_LAUNCHED();
  plan->l_post = 1;
  SKG_CUDA(cudaStreamEndCapture(s0, &plan->graph));
  SKG_CUDA(cudaGraphInstantiate(&plan->exec, plan->graph, 0));
  return SKG_OK;
}

// ends any capture still open on the plan's streams (after a failure part-way through)
static void abandon_capture(skg_batch_plan* plan) {
  for (int k = 2; k >= 0; --k) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (plan->cap[k] && cudaStreamIsCapturing(plan->cap[k], &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(plan->cap[k], &g);
    }
  }
  (void)cudaGetLastError();
}

static void release_plan(skg_batch_plan* plan) {
  if (!plan) return;
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->graph) cudaGraphDestroy(plan->graph);
  for (int k = 0; k < 3; ++k)
    if (plan->cap[k]) cudaStreamDestroy(plan->cap[k]);
  if (plan->own) cudaFree(plan->own);
  delete plan;
}

}  // namespace skg

using namespace skg;

extern "C" {

int64_t skg_be_workspace_size(const skg_tet_mesh* mesh, int precision) {
  return skg_assembly_workspace_size(mesh, precision);
}

int skg_be_step(const skg_tet_mesh* mesh, const skg_be_params* params, const skg_be_state* state, void* workspace,
                skg_step_info* info_h, void* stream) {
  if (!params || !state || !workspace || !info_h) return fail(SKG_ERR_ARG, "be_step: null argument");
  SKG_TRY(check_mesh(mesh, params->precision));
  if (!(params->dt > 0.0)) return fail(SKG_ERR_ARG, "be_step: dt must be positive");
  if (!state->u || !state->u_curr || !state->u_prev || !state->mass) return fail(SKG_ERR_ARG, "be_step: null state");
  SKG_TRY(check_integrator(params, state));
  if (params->do_line_search && !(params->ls_alpha > 0.0 && params->ls_alpha <= 0.5))
    return fail(SKG_ERR_ARG, "line search alpha must lie in (0, 0.5]");
  if (params->do_line_search && !(params->ls_beta > 0.0 && params->ls_beta < 1.0))
    return fail(SKG_ERR_ARG, "line search beta must lie in (0, 1)");
  const skg_newton_record* rec = params->record;
  if (rec && (rec->capacity < 0 || (rec->capacity > 0 && (!rec->g || !rec->dx || !rec->alpha_h || !rec->residual_h ||
                                                          !rec->pcg_iters_h))))
    return fail(SKG_ERR_ARG, "be_step: a Newton record needs capacity >= 0 and all five arrays");
  cudaStream_t s = as_stream(stream);
  Workspace w = carve_workspace(mesh, params->precision, workspace);
  if (params->precision == SKG_MIXED) return be_step<float>(mesh, params, state, w, info_h, s);
  return be_step<double>(mesh, params, state, w, info_h, s);
}

int64_t skg_batch_workspace_size(const skg_tet_mesh* mesh, const skg_batch* batch, int precision) {
  if (check_mesh(mesh, precision) != SKG_OK || !batch || batch->n_inst <= 0) return -1;
  return carve_batch(mesh, batch, precision, nullptr).bytes;
}

int skg_be_step_batched(const skg_tet_mesh* mesh, const skg_batch* batch, const skg_be_params* params,
                        const skg_be_state* state, void* workspace, skg_step_info* infos_h, skg_step_info* total_h,
                        void* stream) {
  if (!batch || !params || !state || !workspace || !infos_h || !total_h)
    return fail(SKG_ERR_ARG, "be_step_batched: null argument");
  SKG_TRY(check_mesh(mesh, params->precision));
  if (batch->n_inst <= 0 || !batch->inst_rows || !batch->inst_tets || !batch->vert_inst || !batch->tet_inst ||
      !batch->order)
    return fail(SKG_ERR_ARG, "be_step_batched: incomplete batch description");
  if (!(params->dt > 0.0)) return fail(SKG_ERR_ARG, "be_step_batched: dt must be positive");
  if (!state->u || !state->u_curr || !state->u_prev || !state->mass)
    return fail(SKG_ERR_ARG, "be_step_batched: null state");
  SKG_TRY(check_integrator(params, state));
  cudaStream_t s = as_stream(stream);
  if (params->precision == SKG_MIXED)
    return be_step_batched<float>(mesh, batch, params, state, workspace, infos_h, total_h, s);
  return be_step_batched<double>(mesh, batch, params, state, workspace, infos_h, total_h, s);
}

static int check_batch_args(const skg_tet_mesh* mesh, const skg_batch* batch, const skg_be_params* params,
                            const skg_be_state* state, const void* workspace) {
  if (!batch || !params || !state || !workspace) return fail(SKG_ERR_ARG, "batch plan: null argument");
  SKG_TRY(check_mesh(mesh, params->precision));
  if (batch->n_inst <= 0 || !batch->inst_rows || !batch->inst_tets || !batch->vert_inst || !batch->tet_inst ||
      !batch->order)
    return fail(SKG_ERR_ARG, "batch plan: incomplete batch description");
  if (!(params->dt > 0.0)) return fail(SKG_ERR_ARG, "batch plan: dt must be positive");
  if (!state->u || !state->u_curr || !state->u_prev || !state->mass) return fail(SKG_ERR_ARG, "batch plan: null state");
  SKG_TRY(check_integrator(params, state));
  return SKG_OK;
}

int skg_be_batch_plan_create(const skg_tet_mesh* mesh, const skg_batch* batch, const skg_be_params* params,
                             const skg_be_state* state, void* workspace, skg_batch_plan** plan_h) {
  if (!plan_h) return fail(SKG_ERR_ARG, "batch plan: null plan pointer");
  *plan_h = nullptr;
  SKG_TRY(check_batch_args(mesh, batch, params, state, workspace));
  skg_batch_plan* plan = new skg_batch_plan();
  for (int k = 0; k < 3; ++k) {
    if (cudaStreamCreateWithFlags(&plan->cap[k], cudaStreamNonBlocking) != cudaSuccess) {
      release_plan(plan);
      return fail(SKG_ERR_CUDA, "batch plan: stream creation failed");
    }
  }
  const int r = params->precision == SKG_MIXED
                    ? capture_batch_step<float>(mesh, batch, params, state, workspace, plan)
                    : capture_batch_step<double>(mesh, batch, params, state, workspace, plan);
  if (r != SKG_OK) {
    abandon_capture(plan);
    release_plan(plan);
    return r;
  }
  *plan_h = plan;
  return SKG_OK;
}

int skg_be_batch_plan_step(skg_batch_plan* plan, skg_step_info* infos_h, skg_step_info* total_h, void* stream) {
  if (!plan || !plan->exec || !infos_h || !total_h) return fail(SKG_ERR_ARG, "batch plan step: null argument");
  cudaStream_t s = as_stream(stream);
  SKG_CUDA(cudaGraphLaunch(plan->exec, s));
  int32_t ctr[8];
  SKG_CUDA(cudaMemcpyAsync(infos_h, plan->info, plan->ni * sizeof(skg_step_info), cudaMemcpyDeviceToHost, s));
  SKG_CUDA(cudaMemcpyAsync(total_h, plan->info + plan->ni, sizeof(skg_step_info), cudaMemcpyDeviceToHost, s));
  SKG_CUDA(cudaMemcpyAsync(ctr, plan->ctr, sizeof(ctr), cudaMemcpyDeviceToHost, s));
  SKG_CUDA(cudaStreamSynchronize(s));
  total_h->launches = plan->l_pre + ctr[kCtrIter] * plan->l_iter + ctr[kCtrTrials] * plan->l_trial +
                      ctr[kCtrRefresh] * plan->l_refresh + plan->l_post;
  return SKG_OK;
}

int skg_be_batch_plan_destroy(skg_batch_plan* plan) {
  release_plan(plan);
  return SKG_OK;
}

int skg_be_plan_eligible(const skg_tet_mesh* mesh, const skg_be_params* params) {
  if (!params || check_mesh(mesh, params->precision) != SKG_OK) return 0;
  return (params->precision == SKG_MIXED ? single_plan_eligible<float>(mesh, params)
                                         : single_plan_eligible<double>(mesh, params)) ? 1 : 0;
}

int skg_be_plan_create(const skg_tet_mesh* mesh, const skg_be_params* params, const skg_be_state* state,
                       void* workspace, skg_batch_plan** plan_h) {
  if (!plan_h) return fail(SKG_ERR_ARG, "be plan: null plan pointer");
  *plan_h = nullptr;
  if (!params || !state || !workspace) return fail(SKG_ERR_ARG, "be plan: null argument");
  SKG_TRY(check_mesh(mesh, params->precision));
  if (!(params->dt > 0.0)) return fail(SKG_ERR_ARG, "be plan: dt must be positive");
  if (!state->u || !state->u_curr || !state->u_prev || !state->mass) return fail(SKG_ERR_ARG, "be plan: null state");
  SKG_TRY(check_integrator(params, state));
  if (params->do_line_search && !(params->ls_alpha > 0.0 && params->ls_alpha <= 0.5))
    return fail(SKG_ERR_ARG, "line search alpha must lie in (0, 0.5]");
  if (params->do_line_search && !(params->ls_beta > 0.0 && params->ls_beta < 1.0))
    return fail(SKG_ERR_ARG, "line search beta must lie in (0, 1)");
  if (!skg_be_plan_eligible(mesh, params))
    return fail(SKG_ERR_ARG, "be plan: these parameters need the host loop (profiling, a Newton record, "
                             "stop_rule 1 or a PCG form without a device tolerance)");
  skg_batch_plan* plan = new skg_batch_plan();
  for (int k = 0; k < 3; ++k) {
    if (cudaStreamCreateWithFlags(&plan->cap[k], cudaStreamNonBlocking) != cudaSuccess) {
      release_plan(plan);
      return fail(SKG_ERR_CUDA, "be plan: stream creation failed");
    }
  }
  const int r = params->precision == SKG_MIXED ? capture_single_step<float>(mesh, params, state, workspace, plan)
                                               : capture_single_step<double>(mesh, params, state, workspace, plan);
  if (r != SKG_OK) {
    abandon_capture(plan);
    release_plan(plan);
    return r;
  }
  *plan_h = plan;
  return SKG_OK;
}

int skg_be_plan_step(skg_batch_plan* plan, skg_step_info* info_h, void* stream) {
  if (!plan || !plan->exec || !info_h || plan->ni != 1) return fail(SKG_ERR_ARG, "be plan step: bad argument");
  skg_step_info total;
  SKG_TRY(skg_be_batch_plan_step(plan, info_h, &total, stream));
  info_h->launches = total.launches;
  return SKG_OK;
}

int skg_be_plan_destroy(skg_batch_plan* plan) {
  release_plan(plan);
  return SKG_OK;
}

}  // extern "C"

namespace skg {

// Scratch of the generic block-Jacobi PCG for nbr block rows, carved from base (sizes only
// when base is null): five padded vectors, the 3x3 inverses, reduction partials, counters and
// scalars.  Shared by skg_pcg_bsr64 (caller workspace) and skg_pcg_bsr64_noalloc (fixed array).
struct PcgScratch {
  PcgVecs<double> v;
  double* jinv;
  double* partials;
  unsigned* counter;
  double* scal;
  int64_t bytes;
};

static PcgScratch carve_pcg_scratch(void* base, int64_t nbr) {
  Carve c(base);
  PcgScratch w{};
  w.v.x = c.take<double>(4 * nbr); w.v.r = c.take<double>(4 * nbr); w.v.z = c.take<double>(4 * nbr);
  w.v.p = c.take<double>(4 * nbr); w.v.q = c.take<double>(4 * nbr);
  w.jinv = c.take<double>(9 * nbr);
  w.partials = c.take<double>(8 * kMaxGrid);
  w.counter = c.take<unsigned>(16);
  w.scal = c.take<double>(64);
  w.bytes = c.off;
  return w;
}

// Generic symmetric solve for newton_solver's spsolve (newton.py:52): FP64
// block-Jacobi PCG on a block matrix in the entry-major layout.
__global__ void k_diag_inverse(int64_t nbr, const int32_t* rowptr, const int32_t* col, const double* val,
                               double* jinv) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= nbr) return;
  const int rp = rowptr[v], K = rowptr[v + 1] - rp;
  double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < K; ++k)
    if (col[rp + k] == v)
      for (int m = 0; m < 9; ++m) a[m] = val[9 * (int64_t)rp + (int64_t)m * K + k];
  double C[9];
  cof3(a, C);
  const double det = a[0] * C[0] + a[1] * C[1] + a[2] * C[2];
  double* ji = jinv + 9 * v;
  if (det != 0.0 && isfinite(det)) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) ji[3 * i + j] = C[3 * j + i] / det;
  } else {
    for (int m = 0; m < 9; ++m) ji[m] = (m % 4 == 0 && a[m] != 0.0) ? 1.0 / a[m] : 0.0;
  }
}

// The solve: block-Jacobi inverses, the grid-persistent PCG, x unpadded, then a stream
// synchronize to read the status and the convergence test.
static int pcg_bsr64_run(const PcgScratch& w, int64_t nbr, const int32_t* rowptr, const int32_t* col,
                         const double* val, const double* b, double* x, double rtol, int32_t max_iter,
                         int32_t* iters_h, cudaStream_t s) {
  // the scratch may hold an earlier call's contents: the reduction counters start at zero
  SKG_CUDA(cudaMemsetAsync(w.counter, 0, 16 * sizeof(unsigned), s));
  k_diag_inverse<<<blocks_for(nbr), kBlock, 0, s>>>(nbr, rowptr, col, val, w.jinv);
  SKG_LAUNCHED();
  Bsr<double> A{nbr, rowptr, col, val, w.jinv};
  PcgResult pr{};
  SKG_TRY(pcg_solve<double>(A, b, 1.0, nullptr, w.v, rtol, max_iter, 1, w.partials, w.counter, w.scal, s, &pr));
  k_unpad<double><<<blocks_for(nbr), kBlock, 0, s>>>(w.v.x, nbr, x);
  SKG_LAUNCHED();
  SKG_CUDA(cudaStreamSynchronize(s));
  if (iters_h) *iters_h = pr.iters;
  if (pr.status != 0) return fail(pr.status, "pcg failed with status %d", pr.status);
  if (!(pr.rr <= rtol * rtol * pr.bb) && pr.bb > 0.0)
    return fail(SKG_ERR_NOT_CONVERGED, "pcg reached %d iterations at relative residual %.3e", pr.iters,
                sqrt(pr.rr / pr.bb));
  return SKG_OK;
}

}  // namespace skg

extern "C" {

int64_t skg_pcg_workspace_size(int64_t nbr) { return carve_pcg_scratch(nullptr, nbr).bytes + 256; }

int skg_pcg_bsr64(int64_t nbr, const int32_t* rowptr, const int32_t* col, const double* val, const double* b,
                  double* x, double rtol, int32_t max_iter, int32_t* iters_h, void* workspace, void* stream) {
  if (nbr <= 0 || !rowptr || !col || !val || !b || !x || !workspace) return fail(SKG_ERR_ARG, "pcg: bad arguments");
  return pcg_bsr64_run(carve_pcg_scratch(workspace, nbr), nbr, rowptr, col, val, b, x, rtol, max_iter, iters_h,
                       as_stream(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free variant of skg_pcg_bsr64.
//
// Some callers cannot allocate device memory when they solve: a real-time
// loop (an interactive simulation frame, a control loop) that must not stall
// on cudaMalloc, or a host program that owns every device buffer itself and
// gives this library only its inputs and outputs.  For them the scratch of
// the solve (five padded PCG vectors, the 3x3 block-Jacobi inverses, the
// reduction partials, counters and scalars) lives in one file-scope device
// array sized for at most kNoAllocMaxRows block rows (12,288 unknowns), about
// 1 MB that every GPU which loads the library holds until the process exits.
//
// Host code cannot pass the array's name to a kernel (on the host it is only
// a stand-in for the device symbol), so every call looks the address up with
// cudaGetSymbolAddress on the current device; the first call on a device also
// loads the library's module there, so make it before any stream capture.
// Each call synchronizes its stream to read the solve's status.  All calls
// share the one array: two calls that overlap on the GPU (other streams, other
// host threads) race on it and must be serialised by the caller.
// ---------------------------------------------------------------------------
namespace skg {

constexpr int64_t kNoAllocMaxRows = 4096;
constexpr int64_t al256(int64_t x) { return (x + 255) & ~int64_t(255); }
constexpr int64_t kNoAllocBytes = 5 * al256(4 * kNoAllocMaxRows * (int64_t)sizeof(double)) +
                                  al256(9 * kNoAllocMaxRows * (int64_t)sizeof(double)) +
                                  al256(8 * (int64_t)kMaxGrid * (int64_t)sizeof(double)) +
                                  al256(16 * (int64_t)sizeof(unsigned)) + al256(64 * (int64_t)sizeof(double));

static __device__ __align__(256) unsigned char g_pcg_noalloc_scratch[kNoAllocBytes];

// device address of the scratch array on the current device, looked up on every call (a host-side
// lookup; a cached address would go stale if the device's context were torn down and re-created)
static int noalloc_scratch(void** out) {
  void* p = nullptr;
  SKG_CUDA(cudaGetSymbolAddress(&p, g_pcg_noalloc_scratch));
  *out = p;
  return SKG_OK;
}

}  // namespace skg

extern "C" {

int64_t skg_pcg_noalloc_max_rows(void) { return kNoAllocMaxRows; }

int skg_pcg_bsr64_noalloc(int64_t nbr, const int32_t* rowptr, const int32_t* col, const double* val, const double* b,
                          double* x, double rtol, int32_t max_iter, int32_t* iters_h, void* stream) {
  if (nbr <= 0 || !rowptr || !col || !val || !b || !x) return fail(SKG_ERR_ARG, "pcg_noalloc: bad arguments");
  if (nbr > kNoAllocMaxRows)
    return fail(SKG_ERR_CAPACITY,
                "pcg_noalloc: %lld block rows exceed the fixed scratch capacity of %lld block rows; "
                "use skg_pcg_bsr64 with a caller-provided workspace",
                (long long)nbr, (long long)kNoAllocMaxRows);
  void* scratch = nullptr;
  SKG_TRY(noalloc_scratch(&scratch));
  const PcgScratch w = carve_pcg_scratch(scratch, nbr);
  if (w.bytes > kNoAllocBytes)
    return fail(SKG_ERR_CAPACITY, "pcg_noalloc: %lld scratch bytes exceed the fixed array of %lld", (long long)w.bytes,
                (long long)kNoAllocBytes);
  return pcg_bsr64_run(w, nbr, rowptr, col, val, b, x, rtol, max_iter, iters_h, as_stream(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Self-test of the bounded waits.  Each kernel below runs one production wait
// helper (grid_barrier of the grid-persistent PCG forms, mbar_wait of the
// cluster PCG's bulk-copy pipeline) on a condition that nothing ever meets: a
// grid barrier whose second block never arrives, an mbarrier phase that waits
// for a second arrival that never comes.  The wait gives up after `limit`
// polls and the kernel returns SKG_ERR_TIMEOUT through device memory, so a
// caller can check that a stuck wait ends with a status and leaves the CUDA
// context usable.  No copy is ever in flight and no other block waits.
// ---------------------------------------------------------------------------
namespace skg {

__global__ void k_wait_selftest_grid(unsigned* count, unsigned* gen, double* err, int* status, long long limit) {
  if (blockIdx.x != 0) return;  // the second block never arrives at the barrier
  const bool ok = grid_barrier(count, gen, err, limit);
  if (threadIdx.x == 0) *status = ok ? SKG_OK : SKG_ERR_TIMEOUT;
}

__global__ void k_wait_selftest_mbar(int* status, int tries) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 2);
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&bar)) : "memory");
    const bool ok = mbar_wait(&bar, 0, tries);  // the phase needs a second arrival
    // complete the phase and retire the barrier before the block exits
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&bar)) : "memory");
    mbar_inval(&bar);
    *status = ok ? SKG_OK : SKG_ERR_TIMEOUT;
  }
}

// barrier words, error flag and status of the self-test, carved as the solvers carve theirs
struct WaitSelftestWs {
  unsigned* bar;
  double* err;
  int* status;
  int64_t bytes;
};
static WaitSelftestWs carve_wait_selftest(void* base) {
  Carve c(base);
  WaitSelftestWs w{};
  w.bar = c.take<unsigned>(2);
  w.err = c.take<double>(1);
  w.status = c.take<int>(1);
  w.bytes = c.off;
  return w;
}

}  // namespace skg

extern "C" {

int64_t skg_wait_selftest_workspace_size(void) { return carve_wait_selftest(nullptr).bytes; }

int skg_wait_selftest(int kind, int64_t limit, int32_t* status_h, void* workspace, void* stream) {
  if (!status_h || !workspace || limit < 1 || limit > (int64_t)kSpinLimit || (kind != 0 && kind != 1))
    return fail(SKG_ERR_ARG, "wait_selftest: kind 0 or 1, 1 <= limit <= %lld, status and workspace needed",
                (long long)kSpinLimit);
  cudaStream_t s = as_stream(stream);
  const WaitSelftestWs w = carve_wait_selftest(workspace);
  unsigned* bar = w.bar;
  double* err = w.err;
  int* st = w.status;
  SKG_CUDA(cudaMemsetAsync(workspace, 0, (size_t)w.bytes, s));
  if (kind == 0) {
    k_wait_selftest_grid<<<2, 32, 0, s>>>(bar, bar + 1, err, st, (long long)limit);
  } else {
    k_wait_selftest_mbar<<<1, 32, 0, s>>>(st, (int)(limit < (1 << 30) ? limit : (1 << 30)));
  }
  SKG_LAUNCHED();
  int h = 0;
  SKG_CUDA(cudaMemcpyAsync(&h, st, sizeof(int), cudaMemcpyDeviceToHost, s));
  SKG_CUDA(cudaStreamSynchronize(s));
  *status_h = h;
  return SKG_OK;
}

}  // extern "C"
