// Grid-persistent PCG with two grid barriers per iteration, for systems too
// large for one thread-block cluster.
//
// The same recurrence as the cluster kernel (pcg_cluster.cuh): the search
// direction p_k = z_k + beta_k p_{k-1} is never published before the SpMV
// that uses it.  Each lane group gathers z_j and p_{k-1, j} of its columns and
// forms p_k,j with the owner's rounding; the lane group of row i writes p_k,i
// into the buffer that held p_{k-2}.  So an iteration has one barrier per
// dependent reduction (p.q, then r.z and r.r) and no separate direction pass.
//
// Reductions: each block reduces its double-float (FP32 systems) or FP64
// partials with a fixed tree and stores them; after the barrier every block
// sums all partials in index order with the same tree.  The order of the sums
// does not depend on which block arrives last, so the scalars are the same in
// every block and on every run.
#pragma once

namespace skg {

// block total of NV accumulators by a fixed tree; valid in thread 0
template <typename R, int NV, int NT = kBlock>
__device__ __forceinline__ void block_total(Dacc<R> (&v)[NV], Dacc<R> (*wsum)[NT / 32]) {
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
      if (lane < NT / 32) x = wsum[k][lane];
      v[k] = dacc_tree<R, 32>(x);
    }
  }
}

__device__ __forceinline__ void st_dacc(Dacc<float>* p, Dacc<float> v) {
  __stcg(reinterpret_cast<float2*>(p), make_float2(v.hi, v.lo));
}
__device__ __forceinline__ void st_dacc(Dacc<double>* p, Dacc<double> v) { __stcg(&p->v, v.v); }
__device__ __forceinline__ Dacc<float> ld_dacc(const Dacc<float>* p) {
  const float2 a = __ldcg(reinterpret_cast<const float2*>(p));
  return {a.x, a.y};
}
__device__ __forceinline__ Dacc<double> ld_dacc(const Dacc<double>* p) { return {__ldcg(&p->v)}; }

// Grid barrier followed by the totals of the NV x gridDim partials
// (part[k * gridDim + b]): every block sums them itself in index order with the
// same tree, so all blocks hold bitwise the same totals and no block works
// between the last arrival and the release.  Returns false on a barrier timeout.
template <typename R, int NV, int NT = kBlock>
__device__ __forceinline__ bool grid_barrier_total(unsigned* count, volatile unsigned* gen, volatile double* err,
                                                   const Dacc<R>* part, Dacc<R> (&out)[NV],
                                                   Dacc<R> (*wsum)[NT / 32]) {
  __shared__ Dacc<R> bc[NV];
  const bool ok = grid_barrier(count, gen, err);
  Dacc<R> s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    dacc_zero(s[k]);
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s[k] = dacc_add(s[k], ld_dacc(part + k * gridDim.x + i));
  }
  block_total<R, NV, NT>(s, wsum);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) bc[k] = s[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = bc[k];
  return ok;
}

// preconditioned residual of a column as stored (one-level preconditioner)
template <typename R> struct ZPlain {
  static constexpr bool kAux = false;
  const R* z;
  __device__ __forceinline__ Vec3<R> operator()(const Blk<R>& b) const { return ld3c(z, b.col); }
};

// U block rows per lane group: y = A p_k with p_k = z + beta p_prev gathered per column
// (p_prev skipped on the first iteration, where p_0 = z); zf(block) gives z of the block's column
template <typename R, int G, int U, class Zf>
__device__ __forceinline__ void spmv_rows_dir(const Bsr<R>& A, const Zf& zf, const R* __restrict__ pp,
                                              R beta, bool first, const int64_t (&row)[U], const bool (&valid)[U],
                                              int lane, Vec3<R> (&y)[U]) {
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
      if (k < K[u]) bk[u] = ld_rec<Zf::kAux>(A.rec, p[u] + k, p[u] + k >= A.keep);
    }
    Vec3<R> xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      xv[u] = Vec3<R>{R(0), R(0), R(0)};
      if (k < K[u]) {
        const Vec3<R> zc = zf(bk[u]);
        xv[u] = first ? zc : pdir3(zc, ld3c(pp, bk[u].col), beta);
      }
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

// Solve after k_pcg_init (x = 0, r, z, p = z, rz, rr, bb, tol2 in scal).  Direction
// buffers: v.p and v.s alternate.  partials: >= 3 gridDim accumulators of scratch.
template <typename R, int G, int U>
__global__ void __launch_bounds__(kBlock, 3) k_pcg_grid2(Bsr<R> A, PcgVecs<R> v, double* partials, unsigned* bar,
                                                      double* scal) {
  __shared__ Dacc<R> wsum[2][kBlock / 32];
  Dacc<R>* PA = reinterpret_cast<Dacc<R>*>(partials);     // p.q per block
  Dacc<R>* PB = PA + gridDim.x;                            // r.z, r.r per block
  unsigned* count = bar;
  volatile unsigned* gen = bar + 1;
  volatile double* err = scal + S_BAR_ERR;
  const double rz0 = scal[S_RZ];
  Dacc<R> rz;
  if constexpr (sizeof(R) == 4) {
    const float h = float(rz0);
    rz = Dacc<R>{h, float(rz0 - double(h))};
  } else {
    rz = Dacc<R>{R(rz0)};
  }
  const double tol2 = scal[S_TOL2];
  R tol2r = R(tol2);
  if (tol2 > 0.0 && !(tol2r > R(0))) tol2r = R(1e-45f);
  const int max_iter = (int)scal[S_MAXIT];
  int it = 0;
  bool done = scal[S_DONE] != 0.0;
  int status = 0;
  const int lane = threadIdx.x & (G - 1);
  const int64_t groups = (int64_t)gridDim.x * (blockDim.x / G);
  const int64_t row0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * (32 / G);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  Dacc<R> rr_acc;
  dacc_zero(rr_acc);
  double rr_final = scal[S_RR];
  R beta = R(0);
  int cur = 0;  // p_k in v.p (cur 0) or v.s (cur 1), p_{k-1} in the other
  while (!done) {
    const bool first = it == 0;
    R* pk = cur ? v.s : v.p;
    const R* pprev = cur ? v.p : v.s;
    // q = A p_k; p_k written for the rows of this lane group; partial p.q
    Dacc<R> pq[1];
    dacc_zero(pq[0]);
    for (int64_t base = row0; base < A.nbr; base += U * groups) {
      int64_t rows[U];
      bool val[U];
      Vec3<R> ys[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        rows[u] = base + u * groups + ((threadIdx.x & 31) / G);
        val[u] = rows[u] < A.nbr;
      }
      spmv_rows_dir<R, G, U>(A, ZPlain<R>{v.z}, pprev, beta, first, rows, val, lane, ys);
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (lane == 0 && val[u]) {
          const Vec3<R> zi = ld3c(v.z, rows[u]);
          const Vec3<R> p = first ? zi : pdir3(zi, ld3c(pprev, rows[u]), beta);
          if (!first) st3(pk, rows[u], p);   // on the first iteration p_0 = z is already in buf[0]
          st3(v.q, rows[u], ys[u]);
          dacc_dot3(pq[0], p, ys[u]);
        }
    }
    block_total<R, 1>(pq, wsum);
    if (threadIdx.x == 0) st_dacc(PA + blockIdx.x, pq[0]);
    Dacc<R> t1[1];
    if (!grid_barrier_total<R, 1>(count, gen, err, PA, t1, wsum)) { status = SKG_ERR_TIMEOUT; break; }
    const R pqr = dacc_r(t1[0]);
    if (!(pqr > R(0)) || !isfinite(pqr)) {
      status = isfinite(pqr) ? 0 : SKG_ERR_NONFINITE;
      break;
    }
    const R a = dacc_r(rz) / pqr;
    Dacc<R> acc[2];
    dacc_zero(acc[0]);
    dacc_zero(acc[1]);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < A.nbr; i += stride) {
      Vec3<R> x = ld3c(v.x, i), r = ld3c(v.r, i);
      const Vec3<R> p = ld3c(pk, i), q = ld3c(v.q, i);
      x = {x.x + a * p.x, x.y + a * p.y, x.z + a * p.z};
      r = {r.x - a * q.x, r.y - a * q.y, r.z - a * q.z};
      const Vec3<R> z = jacobi_apply(A.jinv, i, r);
      st3(v.x, i, x);
      st3(v.r, i, r);
      st3(v.z, i, z);
      dacc_dot3(acc[0], r, z);
      dacc_dot3(acc[1], r, r);
    }
    block_total<R, 2>(acc, wsum);
    if (threadIdx.x == 0) {
      st_dacc(PB + blockIdx.x, acc[0]);
      st_dacc(PB + gridDim.x + blockIdx.x, acc[1]);
    }
    Dacc<R> t2[2];
    if (!grid_barrier_total<R, 2>(count, gen, err, PB, t2, wsum)) { status = SKG_ERR_TIMEOUT; break; }
    ++it;
    rr_acc = t2[1];
    const R rrr = dacc_r(t2[1]);
    const Dacc<R> rz_old = rz;
    rz = t2[0];
    if (!isfinite(rrr)) { status = SKG_ERR_NONFINITE; break; }
    if (rrr <= tol2r || it >= max_iter) break;
    beta = dacc_r(rz) / dacc_r(rz_old);
    cur ^= 1;
  }
  if (it > 0) rr_final = dacc_value(rr_acc);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[S_ITERS] = it;
    scal[S_RR] = rr_final;
    scal[S_RZ] = dacc_value(rz);
    scal[S_DONE] = 1.0;
    if (status != 0) scal[S_STATUS] = status;
    if (*err != 0.0) scal[S_STATUS] = *err;
  }
}

}  // namespace skg
