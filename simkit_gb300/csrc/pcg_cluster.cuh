// PCG on one thread-block cluster, for systems small enough that grid-wide
// synchronisation and L2 round trips dominate a PCG iteration (on the
// 12,288-tet beam the grid-persistent kernel spends 24 of 43 cycles per
// instruction at grid barriers and moves its whole working set through L2).
//
// Layout: the cluster's CTAs split the block rows into contiguous ranges.
// Each CTA keeps the PCG vectors of its own rows (x, r, z, p, q and the 3x3
// block-Jacobi inverses) in shared memory; the SpMV gathers p of
// neighbouring rows from the owning CTA through distributed shared memory
// (ld.shared::cluster).  When a CTA's rows fit, their block values are staged
// in shared memory once per solve (the matrix is constant during a solve) and
// their column indices are replaced by the shared::cluster addresses of the
// p entries they multiply (mapa), so an iteration touches no global memory.
//
// Synchronisation: the hardware cluster barrier (barrier.cluster arrive /
// wait with release / acquire semantics) separates phases.  Dot products are
// reduced per CTA, published in shared memory and summed by every CTA over
// all ranks with a fixed shuffle tree, so all CTAs hold bitwise the same
// scalars and take the same branches.
#pragma once

#include <cooperative_groups.h>

namespace skg {

namespace cgx = cooperative_groups;

constexpr int kClusterThreads = 512;
constexpr int kClusterMax = 16;                 // non-portable cluster size
constexpr int kClusterSmemBudget = 200 * 1024;  // dynamic shared memory per CTA

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint32_t cluster_map(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ Vec3<float> ld_cluster3(uint32_t addr, float) {
  float a, b, c, d;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(a), "=f"(b), "=f"(c), "=f"(d) : "r"(addr) : "memory");
  return {a, b, c};
}
__device__ __forceinline__ Vec3<double> ld_cluster3(uint32_t addr, double) {
  double a, b, c, d;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(a), "=d"(b) : "r"(addr) : "memory");
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(c), "=d"(d) : "r"(addr + 16) : "memory");
  return {a, b, c};
}
__device__ __forceinline__ double ld_cluster_f64(uint32_t addr) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}

// Sum of NV values published by every CTA of the cluster (pub[k] in each
// CTA's shared memory), computed in a fixed order; result in out[] for every
// thread of the CTA.  Caller guarantees a cluster barrier since publication.
template <int NV>
__device__ __forceinline__ void cluster_allsum(const double* pub, int csize, double* bcast, double (&out)[NV]) {
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double v = 0.0;
      if ((int)threadIdx.x < csize) v = ld_cluster_f64(cluster_map(smem_addr(pub + k), threadIdx.x));
      v = warp_sum(v);
      if (threadIdx.x == 0) bcast[k] = v;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = bcast[k];
}

// staged record from shared memory (three / six 16-byte loads)
__device__ __forceinline__ Blk<float> ld_srec(const float* srec, int64_t i) {
  const float4* p = reinterpret_cast<const float4*>(srec) + 3 * i;
  const float4 a = p[0], b = p[1], c = p[2];
  return {{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x}, __float_as_int(c.y)};
}
__device__ __forceinline__ Blk<double> ld_srec(const double* srec, int64_t i) {
  const double2* p = reinterpret_cast<const double2*>(srec) + 6 * i;
  const double2 a = p[0], b = p[1], c = p[2], d = p[3], e = p[4];
  return {{a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, e.x}, (int)__double_as_longlong(e.y)};
}

// first row owned by cluster rank j, and the owner of row c
__device__ __forceinline__ int64_t cl_row0(int64_t nbr, int j, int csize) { return nbr * j / csize; }
__device__ __forceinline__ int cl_owner(int64_t c, int64_t nbr, int csize) {
  return (int)(((c + 1) * csize + nbr - 1) / nbr) - 1;
}

// Shared memory the kernel needs for its vectors, per CTA.
inline int64_t cluster_vec_bytes(int64_t nbr, int csize, int rsize) {
  const int64_t rows_cap = (nbr + csize - 1) / csize;
  return rows_cap * (5 * 4 + 9) * rsize + 16;
}

struct ClusterPcgOut {
  int iters;
  int status;
  double rr, rz, bb;
};

// Solve the system of block rows [gbase, gbase + nbr) (its columns lie in the
// same range) on the calling cluster.  b: right-hand side (3n, simkit layout,
// FP64) scaled by bsign, pinned DOFs forced to zero; x written to xout
// (padded, global rows).  Every thread of every CTA of the cluster must call
// it; it ends with a cluster barrier, so shared memory may be reused after.
template <typename R, int G>
__device__ __forceinline__ ClusterPcgOut cluster_pcg_range(
    cgx::cluster_group& cl, const Bsr<R>& A, int64_t gbase, int64_t nbr, const double* __restrict__ b, double bsign,
    const uint8_t* __restrict__ pinned, R* __restrict__ xout, double rtol, int max_iter, int smem_bytes,
    unsigned char* smem_raw, double* pub, double* bcast, uint32_t* pbase) {
  const int crank = (int)cl.block_rank();
  const int csize = (int)cl.num_blocks();
  const int64_t r0 = gbase + cl_row0(nbr, crank, csize);
  const int64_t r1 = gbase + cl_row0(nbr, crank + 1, csize);
  const int64_t rows_cap = (nbr + csize - 1) / csize;
  const int nr = (int)(r1 - r0);
  // vectors of own rows, stride 4 per row; Jacobi inverses 9 per row
  R* sp = reinterpret_cast<R*>(smem_raw);
  R* sx = sp + 4 * rows_cap;
  R* sr = sx + 4 * rows_cap;
  R* sz = sr + 4 * rows_cap;
  R* sq = sz + 4 * rows_cap;
  R* sj = sq + 4 * rows_cap;
  // block records of own rows (column field replaced by the cluster address of p[col])
  const int64_t vec_bytes = ((int64_t)(reinterpret_cast<unsigned char*>(sj + 9 * rows_cap) - smem_raw) + 15) & ~int64_t(15);
  R* srec = reinterpret_cast<R*>(smem_raw + vec_bytes);

  if ((int)threadIdx.x < csize) pbase[threadIdx.x] = cluster_map(smem_addr(sp), threadIdx.x);
  const int b0 = __ldg(A.rowptr + r0);
  const int b1 = __ldg(A.rowptr + r1);
  const int64_t nblk = b1 - b0;
  const bool stage = vec_bytes + nblk * (int64_t)(kRec * sizeof(R)) <= (int64_t)smem_bytes;
  __syncthreads();
  if (stage) {
    for (int64_t i = threadIdx.x; i < nblk; i += blockDim.x) {
      const Blk<R> bk = ld_rec(A.rec, b0 + i);
      R* d = srec + kRec * i;
#pragma unroll
      for (int m = 0; m < 9; ++m) d[m] = bk.m[m];
      const int64_t lc = bk.col - gbase;
      const int o = cl_owner(lc, nbr, csize);
      d[9] = col_bits((int)(pbase[o] + (uint32_t)((lc - cl_row0(nbr, o, csize)) * 4 * (int64_t)sizeof(R))), R(0));
      d[10] = R(0);
      d[11] = R(0);
    }
  }
  // init: x = 0, r = bsign * b (pinned -> 0), z = p = Jinv r
  double acc[2] = {0.0, 0.0};
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
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
    const R z0 = jl[0] * rv[0] + jl[1] * rv[1] + jl[2] * rv[2];
    const R z1 = jl[3] * rv[0] + jl[4] * rv[1] + jl[5] * rv[2];
    const R z2 = jl[6] * rv[0] + jl[7] * rv[1] + jl[8] * rv[2];
    R* pr = sr + 4 * i;
    pr[0] = rv[0]; pr[1] = rv[1]; pr[2] = rv[2]; pr[3] = R(0);
    R* pz = sz + 4 * i;
    pz[0] = z0; pz[1] = z1; pz[2] = z2; pz[3] = R(0);
    R* pp = sp + 4 * i;
    pp[0] = z0; pp[1] = z1; pp[2] = z2; pp[3] = R(0);
    R* px = sx + 4 * i;
    px[0] = px[1] = px[2] = px[3] = R(0);
    acc[0] += double(rv[0]) * z0 + double(rv[1]) * z1 + double(rv[2]) * z2;
    acc[1] += double(rv[0]) * rv[0] + double(rv[1]) * rv[1] + double(rv[2]) * rv[2];
  }
  block_sum<2, kClusterThreads>(acc);
  if (threadIdx.x == 0) {
    pub[0] = acc[0];
    pub[1] = acc[1];
  }
  cl.sync();
  double s2[2];
  cluster_allsum<2>(pub, csize, bcast, s2);
  double rz = s2[0], rr = s2[1];
  const double bb = rr;
  const double tol2 = rtol * rtol * bb;
  bool done = rr <= tol2 || bb == 0.0 || max_iter <= 0;
  int it = 0, status = 0;
  const int lane = threadIdx.x & (G - 1);
  const int rows_per_pass = blockDim.x / G;
  const int row_off = (threadIdx.x >> 5) * (32 / G) + ((threadIdx.x & 31) / G);
  cl.sync();  // every CTA has read pub[0..1] before it is rewritten
  while (!done) {
    // q = A p on own rows; partial p.q
    acc[0] = 0.0;
    for (int pass = 0; pass < nr; pass += rows_per_pass) {
      const int li = pass + row_off;
      const bool valid = li < nr;
      const int64_t row = r0 + li;
      int rp = b0, K = 0;
      if (valid) {
        rp = __ldg(A.rowptr + row);
        K = __ldg(A.rowptr + row + 1) - rp;
      }
      R a0 = 0, a1 = 0, a2 = 0;
      if (stage) {
        for (int k = lane; k < K; k += G) {
          const Blk<R> bk = ld_srec(srec, rp - b0 + k);
          const Vec3<R> xv = ld_cluster3((uint32_t)bk.col, R(0));
          a0 += bk.m[0] * xv.x + bk.m[1] * xv.y + bk.m[2] * xv.z;
          a1 += bk.m[3] * xv.x + bk.m[4] * xv.y + bk.m[5] * xv.z;
          a2 += bk.m[6] * xv.x + bk.m[7] * xv.y + bk.m[8] * xv.z;
        }
      } else {
        for (int k = lane; k < K; k += G) {
          const Blk<R> bk = ld_rec(A.rec, rp + k);
          const int64_t lc = bk.col - gbase;
          const int o = cl_owner(lc, nbr, csize);
          const uint32_t ad = pbase[o] + (uint32_t)((lc - cl_row0(nbr, o, csize)) * 4 * (int64_t)sizeof(R));
          const Vec3<R> xv = ld_cluster3(ad, R(0));
          a0 += bk.m[0] * xv.x + bk.m[1] * xv.y + bk.m[2] * xv.z;
          a1 += bk.m[3] * xv.x + bk.m[4] * xv.y + bk.m[5] * xv.z;
          a2 += bk.m[6] * xv.x + bk.m[7] * xv.y + bk.m[8] * xv.z;
        }
      }
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o, G);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o, G);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o, G);
      }
      if (lane == 0 && valid) {
        R* q = sq + 4 * li;
        q[0] = a0; q[1] = a1; q[2] = a2;
        const R* p = sp + 4 * li;
        acc[0] += dot3w(Vec3<R>{p[0], p[1], p[2]}, Vec3<R>{a0, a1, a2});
      }
    }
    double a1v[1] = {acc[0]};
    block_sum<1, kClusterThreads>(a1v);
    if (threadIdx.x == 0) pub[2] = a1v[0];
    cl.sync();
    double pqv[1];
    cluster_allsum<1>(pub + 2, csize, bcast, pqv);
    const double pq = pqv[0];
    if (!(pq > 0.0) || !isfinite(pq)) {
      status = isfinite(pq) ? 0 : SKG_ERR_NONFINITE;
      break;
    }
    const R a = R(rz / pq);
    acc[0] = acc[1] = 0.0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      R* x = sx + 4 * i;
      R* r = sr + 4 * i;
      const R* p = sp + 4 * i;
      const R* q = sq + 4 * i;
      const R* J = sj + 9 * i;
      x[0] += a * p[0];
      x[1] += a * p[1];
      x[2] += a * p[2];
      const R ra = r[0] - a * q[0], rb = r[1] - a * q[1], rc = r[2] - a * q[2];
      r[0] = ra; r[1] = rb; r[2] = rc;
      const R z0 = J[0] * ra + J[1] * rb + J[2] * rc;
      const R z1 = J[3] * ra + J[4] * rb + J[5] * rc;
      const R z2 = J[6] * ra + J[7] * rb + J[8] * rc;
      R* z = sz + 4 * i;
      z[0] = z0; z[1] = z1; z[2] = z2;
      acc[0] += dot3w(Vec3<R>{ra, rb, rc}, Vec3<R>{z0, z1, z2});
      acc[1] += dot3w(Vec3<R>{ra, rb, rc}, Vec3<R>{ra, rb, rc});
    }
    block_sum<2, kClusterThreads>(acc);
    if (threadIdx.x == 0) {
      pub[0] = acc[0];
      pub[1] = acc[1];
    }
    cl.sync();
    cluster_allsum<2>(pub, csize, bcast, s2);
    ++it;
    rr = s2[1];
    const double beta = s2[0] / rz;
    rz = s2[0];
    if (!isfinite(rr)) {
      status = SKG_ERR_NONFINITE;
      break;
    }
    if (rr <= tol2 || it >= max_iter) break;
    const R bt = R(beta);
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      R* p = sp + 4 * i;
      const R* z = sz + 4 * i;
      p[0] = z[0] + bt * p[0];
      p[1] = z[1] + bt * p[1];
      p[2] = z[2] + bt * p[2];
    }
    cl.sync();
  }
  // solution to global memory (padded, the layout the line search reads)
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    const R* x = sx + 4 * i;
    st3(xout, r0 + i, Vec3<R>{x[0], x[1], x[2]});
  }
  // no CTA may leave (or reuse its shared memory) while another still reads it
  cl.sync();
  return ClusterPcgOut{it, status, rr, rz, bb};
}

// one system on one cluster (pcg_mode 2)
template <typename R, int G>
__global__ void __launch_bounds__(kClusterThreads, 1)
    k_pcg_cluster(Bsr<R> A, const double* __restrict__ b, double bsign, const uint8_t* __restrict__ pinned,
                  R* __restrict__ xout, double rtol, int max_iter, double* scal, int smem_bytes) {
  cgx::cluster_group cl = cgx::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double pub[4];
  __shared__ double bcast[4];
  __shared__ uint32_t pbase[kClusterMax];
  const ClusterPcgOut o = cluster_pcg_range<R, G>(cl, A, 0, A.nbr, b, bsign, pinned, xout, rtol, max_iter,
                                                  smem_bytes, smem_raw, pub, bcast, pbase);
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
// instances' block-row offsets; inactive instances are skipped.
template <typename R, int G>
__global__ void __launch_bounds__(kClusterThreads, 1)
    k_pcg_cluster_queue(Bsr<R> A, const int32_t* __restrict__ inst_rows, const int32_t* __restrict__ order,
                        int n_inst, const uint8_t* __restrict__ active, const double* __restrict__ eta,
                        const double* __restrict__ b, double bsign, const uint8_t* __restrict__ pinned,
                        R* __restrict__ xout, int max_iter, int32_t* iters_out, int32_t* status_out,
                        unsigned* queue, int smem_bytes) {
  cgx::cluster_group cl = cgx::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double pub[4];
  __shared__ double bcast[4];
  __shared__ uint32_t pbase[kClusterMax];
  __shared__ int next_inst;
  const int csize = (int)cl.num_blocks();
  for (;;) {
    if (cl.block_rank() == 0 && threadIdx.x == 0) {
      const unsigned idx = atomicAdd(queue, 1u);
      next_inst = idx < (unsigned)n_inst ? order[idx] : -1;
    }
    cl.sync();
    __shared__ int inst_sh;
    if (threadIdx.x == 0) inst_sh = *cl.map_shared_rank(&next_inst, 0);
    __syncthreads();
    const int inst = inst_sh;
    cl.sync();  // rank 0 may overwrite next_inst only after every CTA has read it
    if (inst < 0) break;
    if (!active[inst]) continue;
    const int64_t gbase = inst_rows[inst];
    const int64_t nbr = inst_rows[inst + 1] - gbase;
    const int64_t rows_cap = (nbr + csize - 1) / csize;
    if (rows_cap * (5 * 4 + 9) * (int64_t)sizeof(R) + 16 > smem_bytes) {
      if (cl.block_rank() == 0 && threadIdx.x == 0) {
        iters_out[inst] = 0;
        status_out[inst] = SKG_ERR_CAPACITY;
      }
      continue;
    }
    const ClusterPcgOut o = cluster_pcg_range<R, G>(cl, A, gbase, nbr, b, bsign, pinned, xout, eta[inst], max_iter,
                                                    smem_bytes, smem_raw, pub, bcast, pbase);
    if (cl.block_rank() == 0 && threadIdx.x == 0) {
      iters_out[inst] = o.iters;
      status_out[inst] = o.status;
    }
  }
}

}  // namespace skg
