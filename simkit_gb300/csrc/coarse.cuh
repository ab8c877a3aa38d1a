// Two-level additive preconditioner for the grid PCG:
//
//   M^-1 r = D^-1 r + P (P^T A P)^-1 P^T r
//
// D^-1 is the 3x3 block-Jacobi inverse the one-level solver uses.  P maps a
// coarse vector (6 unknowns per aggregate of vertices: 3 translations t and 3
// rotations w about the aggregate centroid) to the vertices,
//   (P e)_v = m_v * (t_a + w_a x d_v),   a = aggregate of v,
// with d_v the vertex offset from the centroid divided by the aggregate's RMS
// offset and m_v the free-DOF mask (pinned DOFs get nothing).  Both terms are
// symmetric positive (semi)definite, so M stays SPD and CG applies unchanged.
//
// Per refresh (first Newton iteration of a step, or every iteration):
//   k_coarse_galerkin  A_c = P^T A P from the assembled blocks, one warp per
//                      nonzero 6x6 coarse block, FP32 sums in a fixed
//                      order (bitwise reproducible), small diagonal shift;
//   k_coarse_invert    A_c^-1 in place by a blocked symmetric sweep (SPD, no
//                      pivoting, FP32), cooperative grid, one barrier per
//                      32-wide pivot block (k_coarse_invert_inst: one CTA per
//                      instance of a batch).  A non-positive pivot clears the
//                      valid flag and the PCG runs one-level.
// Per PCG iteration (k_pcg_grid2c): the coarse residual P^T r accumulated in
// 64-bit fixed point (order-independent, so reproducible), e = A_c^-1 P^T r by
// a dense row-per-warp product, and P e added where the SpMV gathers form the
// search direction.
#pragma once

namespace skg {

// ------------------------------------------------------------ Galerkin ----
// C = P_v^T A'_vw P_w for one fine block, P_v = [I | -S(d_v)], S(d) = [d]x,
// A' = diag(m_v) A diag(m_w):  C = [[A', -A' S_w], [S_v A', -S_v A' S_w]]
__device__ __forceinline__ void skew(const float4 d, float (&S)[9]) {
  S[0] = 0.f;   S[1] = -d.z; S[2] = d.y;
  S[3] = d.z;   S[4] = 0.f;  S[5] = -d.x;
  S[6] = -d.y;  S[7] = d.x;  S[8] = 0.f;
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_coarse_galerkin(Bsr<R> A, CoarseDev c) {
  const int cb = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (cb >= c.n_cb) return;   // warp-uniform
  float acc[36];
#pragma unroll
  for (int q = 0; q < 36; ++q) acc[q] = 0.f;
  const int k0 = c.cb_ptr[cb], k1 = c.cb_ptr[cb + 1];
  for (int k = k0 + lane; k < k1; k += 32) {
    const int s = c.cb_slot[k];
    const Blk<R> blk = ld_rec(A.rec, s);
    const int v = c.bsr_row[s], w = blk.col;
    const float4 mv = c.mode[v], mw = c.mode[w];
    const unsigned fv = mode_mask(mv), fw = mode_mask(mw);
    float a[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) a[3 * i + j] = (((fv >> i) & 1u) && ((fw >> j) & 1u)) ? float(blk.m[3 * i + j]) : 0.f;
    float Sv[9], Sw[9], B[9], SA[9];
    skew(mv, Sv);
    skew(mw, Sw);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        B[3 * i + j] = a[3 * i] * Sw[j] + a[3 * i + 1] * Sw[3 + j] + a[3 * i + 2] * Sw[6 + j];     // A' S_w
        SA[3 * i + j] = Sv[3 * i] * a[j] + Sv[3 * i + 1] * a[3 + j] + Sv[3 * i + 2] * a[6 + j];    // S_v A'
      }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        acc[6 * i + j] += a[3 * i + j];
        acc[6 * i + 3 + j] -= B[3 * i + j];
        acc[6 * (3 + i) + j] += SA[3 * i + j];
        acc[6 * (3 + i) + 3 + j] -= Sv[3 * i] * B[j] + Sv[3 * i + 1] * B[3 + j] + Sv[3 * i + 2] * B[6 + j];
      }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < 36; ++q) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
  if (lane != 0) return;
  int ra = c.cb_rc[2 * cb], ca = c.cb_rc[2 * cb + 1];
  const bool diag = ra == ca;
  float* Mb = c.M;
  int np = c.np;
  if (c.inst_agg) {   // per-instance dense blocks
    const int inst = c.agg_inst[ra];
    const int a0 = c.inst_agg[inst];
    np = ((6 * (c.inst_agg[inst + 1] - a0) + kGjB - 1) / kGjB) * kGjB;
    Mb = c.M + c.inst_moff[inst];
    ra -= a0;
    ca -= a0;
  }
  if (diag) {
    // shift the diagonal by a small fraction of the aggregate's largest one, so
    // rank-deficient aggregates (one vertex, collinear vertices) stay definite;
    // an aggregate with no free DOF gets the identity
    float dmax = 0.f;
#pragma unroll
    for (int i = 0; i < 6; ++i) dmax = fmaxf(dmax, acc[7 * i]);
#pragma unroll
    for (int i = 0; i < 6; ++i) acc[7 * i] = dmax > 0.f ? acc[7 * i] + float(kCoarseShift) * dmax : 1.f;
  }
  float* out = Mb + (int64_t)(6 * ra) * np + 6 * ca;
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) out[(int64_t)i * np + j] = acc[6 * i + j];
}

// ------------------------------------------------------- Gauss-Jordan ----
// Inverse of one SPD 32 x 32 block (row-major at src, leading dimension ld) by
// Gauss-Jordan in one warp: lane j keeps column j in registers, column p of
// each pivot step is broadcast by shuffles, no block barrier.  The result goes
// to out (shared).  False if a pivot is not positive.
__device__ __forceinline__ bool gj_inverse32_warp(const float* src, int64_t ld, float (*out)[kGjB + 1]) {
  const int lane = threadIdx.x & 31;
  float a[kGjB];
#pragma unroll
  for (int i = 0; i < kGjB; ++i) a[i] = src[(int64_t)i * ld + lane];
  bool good = true;
#pragma unroll
  for (int p = 0; p < kGjB; ++p) {
    const float d = __shfl_sync(0xffffffffu, a[p], p);
    good = good && d > 0.f && isfinite(d);
    const float inv = 1.f / d;
    const float f = a[p] * inv;   // new row-p entry of this lane's column
#pragma unroll
    for (int i = 0; i < kGjB; ++i) {
      if (i == p) continue;
      const float aip = __shfl_sync(0xffffffffu, a[i], p);   // row i of column p
      a[i] = lane == p ? -aip * inv : fmaf(-aip, f, a[i]);
    }
    a[p] = lane == p ? inv : f;
  }
#pragma unroll
  for (int i = 0; i < kGjB; ++i) out[i][lane] = a[i];
  return good;
}

// Symmetric sweep inverse of an SPD np x np matrix M (np a multiple of 32;
// rows nc..np-1 are padding set to the identity): pivot blocks K of 32 in
// order, with Pinv = (M_KK)^-1, the step's old row panel R = M[K, :] and C = R^T,
//   M_KK <- -Pinv,  M_Kj <- Pinv R_j,  M_iK <- C_i Pinv,  M_ij <- M_ij - C_i Pinv R_j,
// which keeps M symmetric, so only the upper triangle of 32-row blocks is
// updated; after the last step M = -A^-1 there, and a mirror pass writes the
// full A^-1.  Work unit: 32 rows (one block row) x 256 columns from the
// diagonal block on, one column per thread and the 32 rows in registers.  R
// comes from a double-buffered copy the previous step wrote (row K+1 from its
// own block row, the part left of the diagonal from column block K+1 of the
// rows above, transposed), so no unit reads what another unit of the same step
// writes and a step needs one barrier.
struct GjShared {
  float piv[kGjB][kGjB + 1];
  float rs[kGjB][kGjB + 1];
  __align__(16) float vt[kGjB][kGjB];
  int ustart[kCoarseMax / kGjB + 1];   // first unit of each block row (upper triangle)
};

// unit table of an np x np sweep; all threads of the block call it
__device__ __forceinline__ int gj_units(GjShared& g, int np) {
  const int nbk = np / kGjB, ncu = (np + kGjCols - 1) / kGjCols;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int ib = 0; ib < nbk; ++ib) {
      g.ustart[ib] = acc;
      acc += ncu - (ib * kGjB) / kGjCols;
    }
    g.ustart[nbk] = acc;
  }
  __syncthreads();
  return g.ustart[nbk];
}

// units u0, u0 + us, ... of sweep step kb (Pinv already in g.piv)
__device__ __forceinline__ void gj_step_units(GjShared& g, float* M, int np, int kb, const float* Rw, float* Rn, int u0,
                                              int us) {
  const int nbk = np / kGjB;
  const int units = g.ustart[nbk];
  const int K0 = kb * kGjB, K1 = K0 + kGjB;
  const int tid = threadIdx.x;
  int ib = 0;
  for (int u = u0; u < units; u += us) {
    while (g.ustart[ib + 1] <= u) ++ib;   // units are visited in increasing order
    const int I0 = ib * kGjB;
    const int cu = I0 / kGjCols + (u - g.ustart[ib]);
    const bool pivrow = ib == kb;
    __syncthreads();
    if (!pivrow)
      for (int q = tid; q < kGjB * kGjB; q += blockDim.x) g.rs[q >> 5][q & 31] = Rw[(int64_t)(q >> 5) * np + I0 + (q & 31)];
    __syncthreads();
    for (int q = tid; q < kGjB * kGjB; q += blockDim.x) {
      const int k = q >> 5, i = q & 31;
      float sacc;
      if (pivrow) {
        sacc = g.piv[i][k];
      } else {
        // V = C_I Pinv with C_I[i][l] = R[l][I0 + i]
        sacc = 0.f;
#pragma unroll 8
        for (int l = 0; l < kGjB; ++l) sacc = fmaf(g.rs[l][i], g.piv[l][k], sacc);
      }
      g.vt[k][i] = sacc;
    }
    __syncthreads();
    const int j = cu * kGjCols + tid;
    if (j < I0 || j >= np) continue;
    float a[kGjB];
    if (j >= K0 && j < K1) {
#pragma unroll
      for (int i = 0; i < kGjB; ++i) a[i] = pivrow ? -g.piv[i][j - K0] : g.vt[j - K0][i];
    } else {
#pragma unroll
      for (int i = 0; i < kGjB; ++i) a[i] = pivrow ? 0.f : M[(int64_t)(I0 + i) * np + j];
      const float sg = pivrow ? 1.f : -1.f;
      float rv[kGjB];
#pragma unroll
      for (int k = 0; k < kGjB; ++k) rv[k] = Rw[(int64_t)k * np + j];
#pragma unroll
      for (int k = 0; k < kGjB; ++k) {
        const float r = sg * rv[k];
        const float4* vk = reinterpret_cast<const float4*>(&g.vt[k][0]);
#pragma unroll
        for (int i4 = 0; i4 < kGjB / 4; ++i4) {
          const float4 t = vk[i4];
          a[4 * i4] = fmaf(t.x, r, a[4 * i4]);
          a[4 * i4 + 1] = fmaf(t.y, r, a[4 * i4 + 1]);
          a[4 * i4 + 2] = fmaf(t.z, r, a[4 * i4 + 2]);
          a[4 * i4 + 3] = fmaf(t.w, r, a[4 * i4 + 3]);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < kGjB; ++i) M[(int64_t)(I0 + i) * np + j] = a[i];
    if (kb + 1 < nbk) {
      if (ib == kb + 1) {
#pragma unroll
        for (int i = 0; i < kGjB; ++i) Rn[(int64_t)i * np + j] = a[i];
      } else if (ib < kb + 1 && j >= K1 && j < K1 + kGjB) {
        float4* dst = reinterpret_cast<float4*>(Rn + (int64_t)(j - K1) * np + I0);
#pragma unroll
        for (int i4 = 0; i4 < kGjB / 4; ++i4)
          dst[i4] = make_float4(a[4 * i4], a[4 * i4 + 1], a[4 * i4 + 2], a[4 * i4 + 3]);
      }
    }
  }
}

// tiles t0, t0 + ts, ... of the mirror pass: A^-1 = -M on the upper block triangle, transposed below
__device__ __forceinline__ void gj_mirror(GjShared& g, float* M, int np, int t0, int ts) {
  const int nbk = np / kGjB;
  for (int t = t0; t < nbk * nbk; t += ts) {
    const int ib = t / nbk, jb = t - ib * nbk;
    if (jb < ib) continue;   // block-uniform
    __syncthreads();
    for (int q = threadIdx.x; q < kGjB * kGjB; q += blockDim.x) {
      const int i = q >> 5, j = q & 31;
      float* m = M + (int64_t)(ib * kGjB + i) * np + jb * kGjB + j;
      const float v = -*m;
      *m = v;
      g.rs[i][j] = v;
    }
    __syncthreads();
    if (jb > ib)
      for (int q = threadIdx.x; q < kGjB * kGjB; q += blockDim.x) {
        const int i = q >> 5, j = q & 31;
        M[(int64_t)(jb * kGjB + i) * np + ib * kGjB + j] = g.rs[j][i];
      }
  }
}

// The whole-mesh form (and a one-instance cluster form): the sweep on the
// grid, launched cooperatively with kGjCols threads, one grid barrier per
// step.  Every CTA inverts the pivot block itself (one warp, same inputs and
// order: the same Pinv everywhere).  c.ok[0] is set to 1 only if every pivot
// was positive.
__global__ void __launch_bounds__(kGjCols, 3) k_coarse_invert(CoarseDev c, volatile double* err) {
  __shared__ GjShared g;
  const int np = c.np, nbk = np / kGjB;
  const int tid = threadIdx.x;
  gj_units(g, np);
  const int64_t gsz = (int64_t)gridDim.x * blockDim.x, g0 = blockIdx.x * (int64_t)blockDim.x + tid;
  unsigned* count = c.bar;
  volatile unsigned* gen = c.bar + 1;
  bool good = true;
  for (int64_t i = c.nc + g0; i < np; i += gsz) c.M[i * np + i] = 1.f;
  if (!grid_barrier(count, gen, err)) return;
  for (int64_t q = g0; q < (int64_t)np * kGjB; q += gsz) c.rowp[q] = c.M[q];   // rows 0..31
  if (!grid_barrier(count, gen, err)) return;
  for (int kb = 0; kb < nbk; ++kb) {
    const float* Rw = c.rowp + (int64_t)(kb & 1) * kGjB * np;
    float* Rn = c.rowp + (int64_t)((kb + 1) & 1) * kGjB * np;
    __syncthreads();   // piv of the previous step is no longer read
    if (tid < 32) good = gj_inverse32_warp(Rw + kb * kGjB, np, g.piv) && good;   // thread 0 keeps the flag
    __syncthreads();
    gj_step_units(g, c.M, np, kb, Rw, Rn, blockIdx.x, gridDim.x);
    if (!grid_barrier(count, gen, err)) return;
  }
  gj_mirror(g, c.M, np, blockIdx.x, gridDim.x);
  if (blockIdx.x == 0 && tid == 0) *c.ok = good ? 1 : 0;
}

// The per-instance form for batches: one thread-block cluster of kGjCluster
// CTAs per instance (instances largest first by `order`, clusters striding
// over them), the units of a sweep step spread over the cluster's CTAs and a
// cluster barrier per step; row panels in a per-cluster scratch of
// 2 x 32 x max_np floats.  c.ok[inst] = 1 only if every pivot was positive.
constexpr int kGjCluster = 4;
__global__ void __launch_bounds__(kGjCols, 3) k_coarse_invert_inst(CoarseDev c, const int32_t* __restrict__ order) {
  __shared__ GjShared g;
  cgx::cluster_group cl = cgx::this_cluster();
  const int crank = (int)cl.block_rank(), csize = (int)cl.num_blocks();
  const int cid = blockIdx.x / csize, ncl = gridDim.x / csize;
  const int tid = threadIdx.x;
  const int ct = crank * blockDim.x + tid, cstride = csize * blockDim.x;
  float* rowp = c.rowp + (int64_t)cid * 2 * kGjB * c.max_np;
  for (int idx = cid; idx < c.n_inst; idx += ncl) {
    const int inst = order ? order[idx] : idx;
    const int nc = 6 * (c.inst_agg[inst + 1] - c.inst_agg[inst]);
    const int np = ((nc + kGjB - 1) / kGjB) * kGjB;
    float* M = c.M + c.inst_moff[inst];
    const int nbk = np / kGjB;
    gj_units(g, np);
    for (int i = nc + ct; i < np; i += cstride) M[(int64_t)i * np + i] = 1.f;
    cl.sync();
    for (int q = ct; q < np * kGjB; q += cstride) rowp[q] = M[q];
    cl.sync();
    bool good = true;
    for (int kb = 0; kb < nbk; ++kb) {
      const float* Rw = rowp + (int64_t)(kb & 1) * kGjB * np;
      float* Rn = rowp + (int64_t)((kb + 1) & 1) * kGjB * np;
      __syncthreads();
      if (tid < 32) good = gj_inverse32_warp(Rw + kb * kGjB, np, g.piv) && good;
      __syncthreads();
      gj_step_units(g, M, np, kb, Rw, Rn, crank, csize);
      cl.sync();
    }
    gj_mirror(g, M, np, crank, csize);
    if (crank == 0 && tid == 0) c.ok[inst] = good ? 1 : 0;
    cl.sync();   // the scratch and the table are reused by the next instance
  }
}

// ---------------------------------------------------------------- PCG ----
// z_j = D^-1 r_j (stored) + (P e)_j, rounded the same wherever it is formed: in
// the gathers from the block record, for the own row from the mode array
template <typename R> struct ZCoarse {
  static constexpr bool kAux = true;
  const R* z;
  CoarseDev c;
  bool on;
  __device__ __forceinline__ Vec3<R> operator()(const Blk<R>& b) const {
    Vec3<R> a = ld3c(z, b.col);
    if (on) {
      const Vec3<float> p = prolong_rec(c.e, b.aux0, b.aux1);
      a = {a.x + R(p.x), a.y + R(p.y), a.z + R(p.z)};
    }
    return a;
  }
  __device__ __forceinline__ Vec3<R> own(int64_t v) const {
    Vec3<R> a = ld3c(z, v);
    if (on) {
      const Vec3<float> p = prolong(c, v);
      a = {a.x + R(p.x), a.y + R(p.y), a.z + R(p.z)};
    }
    return a;
  }
};

#ifndef SKG_ROW_LOADS
#define SKG_ROW_LOADS 12
#endif
constexpr int kRowLoads = SKG_ROW_LOADS;

// e = A_c^-1 (P^T r) for the rows of this CTA's warps (one row per warp, rows dealt to the blocks
// in turn so that every block gets nc / gridDim of them), pc += (P^T r) . e over those rows, from
// P^T r staged in shared memory (rcf: np floats)
template <typename R>
__device__ __forceinline__ void coarse_rows_product(const CoarseDev& c, const float* rcf, Dacc<R>& pc) {
  const int wpb = blockDim.x >> 5;
  const int lane = threadIdx.x & 31;
  const float4* r4 = reinterpret_cast<const float4*>(rcf);
  for (int row = blockIdx.x + (threadIdx.x >> 5) * gridDim.x; row < c.nc; row += gridDim.x * wpb) {
    // A_c^-1 is read with normal L2 priority: with the block records past 20% read evict-first
    // it stays in L2 beside the kept records and the vectors
    const float4* Mr = reinterpret_cast<const float4*>(c.M + (int64_t)row * c.np);
    float s = 0.f;
    // kRowLoads loads of the row in flight per lane before the first is used (the row is ~23 float4
    // per lane at 2,850 coarse unknowns: two rounds of L2 latency), summed in the order of j
    const int n4 = c.np >> 2;
    for (int j0 = lane; j0 < n4; j0 += 32 * kRowLoads) {
      float4 m[kRowLoads];
#pragma unroll
      for (int u = 0; u < kRowLoads; ++u)
        m[u] = j0 + 32 * u < n4 ? __ldcg(Mr + j0 + 32 * u) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int u = 0; u < kRowLoads; ++u)
        if (j0 + 32 * u < n4) {
          const float4 x = r4[j0 + 32 * u];
          s = fmaf(m[u].x, x.x, fmaf(m[u].y, x.y, fmaf(m[u].z, x.z, fmaf(m[u].w, x.w, s))));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      c.e[8 * (row / 6) + row % 6] = s;
      dacc_dot3(pc, Vec3<R>{R(rcf[row]), R(0), R(0)}, Vec3<R>{R(s), R(0), R(0)});
    }
  }
}

// The coarse product from the fixed-point restriction c.rc (scaled back by inv_scale).  keep: the
// two-barrier form also stores P^T r in double there, entry i by block i mod gridDim.
template <typename R>
__device__ __forceinline__ void coarse_product(const CoarseDev& c, float* rcf, float inv_scale, Dacc<R>& pc,
                                               double* keep = nullptr) {
  if ((int)blockIdx.x >= c.nc) return;   // block-uniform
#pragma unroll 4
  for (int i = threadIdx.x; i < c.np; i += blockDim.x) {
    const long long q = i < c.nc ? (long long)__ldcg(c.rc + i) : 0ll;
    rcf[i] = i < c.nc ? __ll2float_rn(q) * inv_scale : 0.f;
    if (keep && i < c.nc && i % (int)gridDim.x == (int)blockIdx.x) keep[i] = (double)q * (double)inv_scale;
  }
  __syncthreads();
  coarse_rows_product<R>(c, rcf, pc);
}

// Two-barrier form: P^T r_{k+1} = P^T r_k - alpha_k P^T q_k, with P^T r_k carried in double (cur)
// and P^T q_k in fixed point (rq, scale 1 / a_inv_sq times alpha_k).  Every block forms all entries
// with the same operations (so all hold the same bits) into rcf, and block i mod gridDim stores entry
// i for the next iteration (next); then the coarse product.
template <typename R>
__device__ __forceinline__ void coarse_product_recur(const CoarseDev& c, float* rcf, const double* cur,
                                                     const unsigned long long* rq, double a_inv_sq, double* next,
                                                     Dacc<R>& pc) {
  if ((int)blockIdx.x >= c.nc) return;   // block-uniform
#pragma unroll 4
  for (int i = threadIdx.x; i < c.np; i += blockDim.x) {
    double x = 0.0;
    if (i < c.nc) {
      x = __ldcg(cur + i) - a_inv_sq * (double)(long long)__ldcg(rq + i);
      if (i % (int)gridDim.x == (int)blockIdx.x) next[i] = x;
    }
    rcf[i] = (float)x;
  }
  __syncthreads();
  coarse_rows_product<R>(c, rcf, pc);
}

// iterations of the two-barrier form that restrict r itself (the recurrence restarts from the exact
// restriction; the first iteration has no alpha_{k-1} for the scale of P^T q)
constexpr int kRecurExact = 8;
// block rows whose q the two-barrier form stages in shared memory (larger ranges: three barriers)
constexpr int kStageRows = 2048;

// Two-level PCG, grid-persistent.  Solve after k_pcg_init (x = 0, r, z = D^-1 r,
// r.z in scal).  Per iteration three grid barriers:
//   A  q = A p with p = (D^-1 r + P e) + beta p_prev formed in the gathers;
//      p.q                                                     -> barrier 1
//   B  x += alpha p, r -= alpha q, z = D^-1 r; r.z, r.r; P^T r -> barrier 2
//   C  e = A_c^-1 P^T r; (P^T r).e                             -> barrier 3
// with r.M^-1 r = r.D^-1 r + (P^T r).e.  When the coarse inverse is not valid
// (c.ok == 0) phases C and the restriction are skipped: the one-level method.
// TB (two barriers): phase A also restricts q (staged in shared memory; P^T q in fixed point, scaled
// by the previous iteration's alpha), and phase B forms P^T r_{k+1} = P^T r_k - alpha P^T q and runs the coarse
// product beside the update, so barrier 3 goes.  Every kRecurExact-th iteration (and one whose
// scaled P^T q leaves the exact range, counted in the p.q reduction) takes the three-barrier path
// with the restriction of r itself, which restarts the recurrence.
// partials: >= 6 gridDim accumulators of scratch.  Each block owns an equal
// contiguous range of block rows (the SpMV lane groups and the per-row update
// both work inside it), so the phases end at about the same time in every block.
// NT threads per block: 256 (three blocks per SM) or 768 (one per SM: a third of the
// barrier arrivals and block partials, the same threads in flight)
template <typename R, int G, int U, int NT = kBlock, bool TB = false>
__global__ void __launch_bounds__(NT, NT == kBlock ? 3 : 1) k_pcg_grid2c(Bsr<R> A, PcgVecs<R> v, CoarseDev c,
                                                                      double* partials, unsigned* bar, double* scal) {
  constexpr int NA = TB ? 2 : 1;   // phase A totals: p.q (and the out-of-range count)
  constexpr int NB = TB ? 3 : 2;   // phase B totals: r.z, r.r (and (P^T r).e)
  __shared__ Dacc<R> wsum[3][NT / 32];
  __shared__ __align__(16) float rcf[kCoarseMax];
  __shared__ float qs[TB ? 3 * kStageRows : 1];   // q of the block's rows (two-barrier form)
  Dacc<R>* PA = reinterpret_cast<Dacc<R>*>(partials);     // p.q per block
  Dacc<R>* PB = PA + NA * gridDim.x;                       // r.z, r.r per block
  Dacc<R>* PC = PB + NB * gridDim.x;                       // (P^T r).e per block
  unsigned* count = bar;
  volatile unsigned* gen = bar + 1;
  volatile double* err = scal + S_BAR_ERR;
  const bool con = *c.ok != 0;
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
  const int64_t chunk = (A.nbr + gridDim.x - 1) / gridDim.x;
  const int64_t rbeg = min((int64_t)blockIdx.x * chunk, A.nbr), rend = min(rbeg + chunk, A.nbr);
  const int64_t groups = NT / G;                                  // lane groups per block
  const int64_t row0 = rbeg + (threadIdx.x >> 5) * (32 / G);      // warp-uniform loop bounds
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t wbase0 = rbeg + (threadIdx.x & ~31);
  Dacc<R> rr_acc;
  dacc_zero(rr_acc);
  double rr_final = scal[S_RR];
  double rr_prev = scal[S_RR];
  R beta = R(0);
  R a_prev = R(0);
  int cur = 0;  // p_k in v.p (cur 0) or v.s (cur 1), p_{k-1} in the other
  const ZCoarse<R> zf{v.z, c, con};
  if (!done && con) {
    // coarse part of z_0 = D^-1 r_0 + P e_0
    const float sc = coarse_scale(rr_prev);
    for (int64_t base = wbase0; base < rend; base += NT) {
      const int64_t i = base + (threadIdx.x & 31);
      const bool ok = i < rend;
      const Vec3<R> r = ok ? ld3c(v.r, i) : Vec3<R>{R(0), R(0), R(0)};
      coarse_restrict(c, ok, i, float(r.x), float(r.y), float(r.z), sc);
    }
    if (!grid_barrier(count, gen, err)) {
      status = SKG_ERR_TIMEOUT;
      done = true;
    } else {
      Dacc<R> pc[1];
      dacc_zero(pc[0]);
      coarse_product<R>(c, rcf, 1.f / sc, pc[0]);
      block_total<R, 1, NT>(pc, wsum);
      if (threadIdx.x == 0) st_dacc(PC + blockIdx.x, pc[0]);
      Dacc<R> t3[1];
      if (!grid_barrier_total<R, 1, NT>(count, gen, err, PC, t3, wsum)) {
        status = SKG_ERR_TIMEOUT;
        done = true;
      } else {
        rz = dacc_add(rz, t3[0]);
      }
    }
  }
  while (!done) {
    const bool first = it == 0;
    R* pk = cur ? v.s : v.p;
    const R* pprev = cur ? v.p : v.s;
    // two-barrier iterations restrict q here, at a power-of-two scale from |r_k| and alpha_{k-1}
    // (alpha_k P^T q_k is about the change of P^T r), 2^8 below the scale of r's restriction: room for
    // alpha_{k-1} |q| up to ~2^16 |r| per row, at a resolution of ~1e-8 |r|
    const bool rec = TB && con && !first && (it % kRecurExact) != 0 && chunk <= kStageRows;
    unsigned long long* rqk = TB && con ? c.rq + (int64_t)(it & 1) * c.np : nullptr;
    float sq = 0.f;
    if (rec) {
      int ea = 0;
      frexpf(float(a_prev), &ea);
      sq = ldexpf(coarse_scale(rr_prev), -ea - 8);
    }
    // the coarse residual was last read in phase C and is next written in phase B
    if (con)
      for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < c.np; i += stride) c.rc[i] = 0ull;
    Dacc<R> pq[NA];
#pragma unroll
    for (int k = 0; k < NA; ++k) dacc_zero(pq[k]);
    bool out_of_range = rec && !(sq > 0.f && sq < INFINITY);
    for (int64_t base = row0; base < rend; base += U * groups) {
      int64_t rows[U];
      bool val[U];
      Vec3<R> ys[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        rows[u] = base + u * groups + ((threadIdx.x & 31) / G);
        val[u] = rows[u] < rend;
      }
      spmv_rows_dir<R, G, U>(A, zf, pprev, beta, first, rows, val, lane, ys);
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (lane == 0 && val[u]) {
          const Vec3<R> zi = zf.own(rows[u]);
          const Vec3<R> p = first ? zi : pdir3(zi, ld3c(pprev, rows[u]), beta);
          st3(pk, rows[u], p);
          st3(v.q, rows[u], ys[u]);
          dacc_dot3(pq[0], p, ys[u]);
          if (TB && rec) {
            float* qq = qs + 3 * (rows[u] - rbeg);
            qq[0] = float(ys[u].x);
            qq[1] = float(ys[u].y);
            qq[2] = float(ys[u].z);
          }
        }
    }
    if constexpr (TB) {
      if (rec) {   // block-uniform: P^T q over the block's rows, 32 consecutive rows per warp pass
        __syncthreads();
#pragma unroll 2
        for (int64_t base = wbase0; base < rend; base += NT) {
          const int64_t i = base + (threadIdx.x & 31);
          const bool ok = i < rend;
          const float* qq = qs + 3 * (ok ? i - rbeg : 0);
          out_of_range |= coarse_restrict_groups<1>(c, rqk, ok, i, ok ? qq[0] : 0.f, ok ? qq[1] : 0.f,
                                                    ok ? qq[2] : 0.f, sq);
        }
      }
    }
    if constexpr (TB) {
      if (out_of_range) pq[NA - 1] = dacc_add(pq[NA - 1], Dacc<R>{R(1)});
    }
    block_total<R, NA, NT>(pq, wsum);
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NA; ++k) st_dacc(PA + k * gridDim.x + blockIdx.x, pq[k]);
    Dacc<R> t1[NA];
    if (!grid_barrier_total<R, NA, NT>(count, gen, err, PA, t1, wsum)) { status = SKG_ERR_TIMEOUT; break; }
    const R pqr = dacc_r(t1[0]);
    if (!(pqr > R(0)) || !isfinite(pqr)) {
      status = isfinite(pqr) ? 0 : SKG_ERR_NONFINITE;
      break;
    }
    const R a = dacc_r(rz) / pqr;
    bool use_rec = false;
    if constexpr (TB) use_rec = rec && dacc_value(t1[NA - 1]) == 0.0;
    const float sc = coarse_scale(rr_prev);
    Dacc<R> acc[NB];
#pragma unroll
    for (int k = 0; k < NB; ++k) dacc_zero(acc[k]);
    if constexpr (TB) {
      if (con) {
        // the P^T q buffer of the next iteration was last read in the previous iteration's phase B
        unsigned long long* rqn = c.rq + (int64_t)((it + 1) & 1) * c.np;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < c.np; i += stride) rqn[i] = 0ull;
      }
      if (use_rec)
        coarse_product_recur<R>(c, rcf, c.rcg + (int64_t)(it & 1) * c.np, rqk, double(a) / double(sq),
                                c.rcg + (int64_t)((it + 1) & 1) * c.np, acc[2]);
    }
    for (int64_t base = wbase0; base < rend; base += NT) {
      const int64_t i = base + (threadIdx.x & 31);
      const bool ok = i < rend;
      Vec3<R> r{R(0), R(0), R(0)};
      if (ok) {
        Vec3<R> x = ld3c(v.x, i);
        r = ld3c(v.r, i);
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
      if (con && !use_rec) coarse_restrict(c, ok, i, float(r.x), float(r.y), float(r.z), sc);
    }
    block_total<R, NB, NT>(acc, wsum);
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NB; ++k) st_dacc(PB + k * gridDim.x + blockIdx.x, acc[k]);
    Dacc<R> t2[NB];
    if (!grid_barrier_total<R, NB, NT>(count, gen, err, PB, t2, wsum)) { status = SKG_ERR_TIMEOUT; break; }
    ++it;
    a_prev = a;
    rr_acc = t2[1];
    rr_prev = dacc_value(t2[1]);
    const R rrr = dacc_r(t2[1]);
    const Dacc<R> rz_old = rz;
    rz = t2[0];
    if constexpr (TB) {
      if (use_rec) rz = dacc_add(rz, t2[2]);
    }
    if (!isfinite(rrr)) { status = SKG_ERR_NONFINITE; break; }
    if (rrr <= tol2r || it >= max_iter) break;
    if (con && !use_rec) {
      Dacc<R> pc[1];
      dacc_zero(pc[0]);
      coarse_product<R>(c, rcf, 1.f / sc, pc[0], TB ? c.rcg + (int64_t)(it & 1) * c.np : nullptr);
      block_total<R, 1, NT>(pc, wsum);
      if (threadIdx.x == 0) st_dacc(PC + blockIdx.x, pc[0]);
      Dacc<R> t3[1];
      if (!grid_barrier_total<R, 1, NT>(count, gen, err, PC, t3, wsum)) { status = SKG_ERR_TIMEOUT; break; }
      rz = dacc_add(rz, t3[0]);
    }
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
