// Assembled tier of the FEM path: per-tet Hessians with the analytic PSD
// floor, deterministic gather-assembly into the block pattern, FP64 vertex
// forces and the line-search energy.
//
// Data layout in HBM (t tets, n vertices, nb 3x3 blocks):
//   tets        int4[t]
//   dinv        R[9][t]   SoA, row c of the 3x3 = grad N_{c+1}
//   vol/mu/lam  R[t]      (FP32 copies packed as mat32[3][t])
//   hbuf        R[t][80]  per-tet lifted Hessian, 78 packed values + 2 pad
//   fbuf        f64[t][12] per-tet vertex forces
//   val         R[9 nb]   block values, entry-major inside each block row
//   u           f64[3n]   displacement from rest (or absolute positions)
//   uh, ul      f32[n][4] hi/lo split of u for FP32 kernels
#include "assembly.cuh"
#include "dfloat.cuh"
#include "snh_math.cuh"

namespace skg {

// --------------------------------------------------------- tet gathers ---
// edge displacement differences du[3(a-1)+i] = u_a,i - u_0,i
__device__ __forceinline__ void tet_du(const double* __restrict__ u, int4 v, double* du) {
  const int vv[3] = {v.y, v.z, v.w};
  const double u0 = u[3 * (int64_t)v.x], u1 = u[3 * (int64_t)v.x + 1], u2 = u[3 * (int64_t)v.x + 2];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    du[3 * a + 0] = u[3 * (int64_t)vv[a] + 0] - u0;
    du[3 * a + 1] = u[3 * (int64_t)vv[a] + 1] - u1;
    du[3 * a + 2] = u[3 * (int64_t)vv[a] + 2] - u2;
  }
}

// FP32 differences from the hi/lo split: (h_a - h_0) + (l_a - l_0) is
// accurate to FP32 relative precision of the difference itself.
__device__ __forceinline__ void tet_du(const float* __restrict__ uh, const float* __restrict__ ul, int4 v,
                                       float* du) {
  const Vec3<float> h0 = ld3(uh, v.x), l0 = ld3(ul, v.x);
  const int vv[3] = {v.y, v.z, v.w};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const Vec3<float> h = ld3(uh, vv[a]), l = ld3(ul, vv[a]);
    du[3 * a + 0] = (h.x - h0.x) + (l.x - l0.x);
    du[3 * a + 1] = (h.y - h0.y) + (l.y - l0.y);
    du[3 * a + 2] = (h.z - h0.z) + (l.z - l0.z);
  }
}

template <typename R>
__device__ __forceinline__ void load_dinv(const R* __restrict__ dinv, int64_t t, int64_t e, R* D) {
#pragma unroll
  for (int k = 0; k < 9; ++k) D[k] = __ldg(dinv + k * t + e);
}

// -------------------------------------------------------- tet Hessians ---
constexpr float kFallbackJ = 0.1f;   // det F below which the eigensystem's SVD runs in FP64

// F of tet e (G) and its shape operator (D)
template <typename R>
__device__ __forceinline__ void tet_F(const TetArgs<R>& a, int64_t e, int disp, R (&D)[9], R (&G)[9]) {
  const int4 v = __ldg(a.tets + e);
  R du[9];
  if constexpr (sizeof(R) == 8) {
    tet_du(a.u, v, du);
  } else {
    tet_du(a.uh, a.ul, v, du);
  }
  load_dinv(a.dinv, a.t, e, D);
  disp_grad(du, D, G);
  if (disp) {
    G[0] += R(1);
    G[4] += R(1);
    G[8] += R(1);
  }
  add_fbar(a, e, G);
}

// the 78 packed values of tet e's lifted Hessian from its F
template <typename R, bool LE, bool FP64_SVD = true>
__device__ __forceinline__ void tet_hessian_from_F(const TetArgs<R>& a, int64_t e, int project, const R (&D)[9],
                                                   const R (&G)[9], R (&out)[kTetHessVals]) {
  R gN[12];
  shape_grads(D, gN);
  const R vol = __ldg(a.vol + e), mu = __ldg(a.mu + e), lam = __ldg(a.lam + e);
  if constexpr (LE)
    le_tet_hessian<R>(mu, lam, vol, gN, out);
  else
    nh_tet_hessian<R, FP64_SVD>(G, mu, lam, vol, gN, out, R(kFallbackJ), project != 0, a.material);
}

template <typename R, bool LE>
__device__ __forceinline__ void tet_hessian_values(const TetArgs<R>& a, int64_t e, int disp, int project,
                                                   R (&out)[kTetHessVals]) {
  R D[9], G[9];
  tet_F(a, e, disp, D, G);
  tet_hessian_from_F<R, LE>(a, e, project, D, G, out);
}

// float pairs of a record (78 values)
__device__ __forceinline__ void store_hess_record(float* dst, const float (&out)[kTetHessVals]) {
#pragma unroll
  for (int k = 0; k < kTetHessVals / 2; ++k)
    reinterpret_cast<float2*>(dst)[k] = make_float2(out[2 * k], out[2 * k + 1]);
}

// One thread per tet.  FP32: at most 168 registers so that 3 blocks fit an SM (measured 1.60 ->
// 1.32 ms of Hessian evaluation per step on the 786,432-tet beam, despite ~140 bytes of spills; the
// split form below: 128 registers at 4 blocks), and the block's records leave through shared
// memory: every thread stores its 78 values as pairs at a conflict-free stride, then the block
// writes its tets' contiguous kHStride records with consecutive lanes on consecutive words - one
// thread storing its own record would touch 32 different records with every warp store (ncu:
// LSU-throttle stalls).  FP64 stores directly.
// LE: the instantiation for linear-elasticity meshes (constant stiffness, no eigensystem).
constexpr int kHessThreads = 128;
constexpr int kHessStage = kTetHessVals + 4;  // staging row stride (82 words: 41 pairs, odd, so the
                                              // 8-byte stores of a half-warp hit distinct bank pairs)

// SPLIT (FP32, non-linear materials): tets with det F < kFallbackJ are appended to late / late_n
// instead (their record is written by k_tet_hessian_late, with the eigensystem's SVD in FP64); without
// the FP64 path the kernel has no spills at 3 blocks per SM and fits 4 (measured on the 786,432-tet
// beam: 163 us with the FP64 path at 3 blocks, 155 us split at 3, ~144 us split at 4).
template <typename R, bool LE = false, bool SPLIT = false>
__global__ void __launch_bounds__(kHessThreads, sizeof(R) == 4 ? (SPLIT ? 4 : 3) : 1)
    k_tet_hessian(TetArgs<R> a, int disp, int project, R* __restrict__ hbuf, int32_t* late, unsigned* late_n) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool valid = e < a.t && !(a.inst_active && !a.inst_active[__ldg(a.tet_inst + e)]);
  if constexpr (sizeof(R) == 8) {
    if (!valid) return;
    R out[kTetHessVals];
    tet_hessian_values<R, LE>(a, e, disp, project, out);
    R* o = hbuf + (int64_t)kHStride * e;
#pragma unroll
    for (int k = 0; k < kTetHessVals / 2; ++k) reinterpret_cast<double2*>(o)[k] = make_double2(out[2 * k], out[2 * k + 1]);
  } else {
    __shared__ __align__(16) float stage[kHessThreads * kHessStage];
    __shared__ unsigned char keep[kHessThreads];
    keep[threadIdx.x] = valid ? 1 : 0;
    if (valid) {
      float D[9], G[9];
      tet_F(a, e, disp, D, G);
      if (SPLIT && det3(G) < kFallbackJ) {   // nearly inverted: the FP64-SVD kernel takes it
        late[atomicAdd(late_n, 1u)] = (int32_t)e;
        keep[threadIdx.x] = 0;
      } else {
        float out[kTetHessVals];
        tet_hessian_from_F<float, LE, !SPLIT>(a, e, project, D, G, out);
        store_hess_record(stage + threadIdx.x * kHessStage, out);
      }
    }
    __syncthreads();
    // each warp writes whole records: 39 pairs per tet (the 78 values), lanes on consecutive pairs
    const int64_t e0 = (int64_t)blockIdx.x * blockDim.x;
    const int nt = (int)min((int64_t)blockDim.x, a.t - e0);
    const int lane = threadIdx.x & 31;
    for (int tt = threadIdx.x >> 5; tt < nt; tt += blockDim.x >> 5) {
      if (!keep[tt]) continue;  // warp-uniform
      const float2* src = reinterpret_cast<const float2*>(stage + tt * kHessStage);
      float2* dst = reinterpret_cast<float2*>(hbuf + (int64_t)kHStride * (e0 + tt));
      dst[lane] = src[lane];
      if (lane < kTetHessVals / 2 - 32) dst[32 + lane] = src[32 + lane];
    }
  }
}

// The tets k_tet_hessian set aside (det F < kFallbackJ), with the FP64 SVD; grid-stride over the list
// (usually empty or a few tets: a small fixed grid).
constexpr int kLateBlocks = 256;
template <typename R, bool LE = false>
__global__ void __launch_bounds__(kHessThreads) k_tet_hessian_late(TetArgs<R> a, int disp, int project,
                                                                   R* __restrict__ hbuf, const int32_t* late,
                                                                   const unsigned* late_n) {
  const unsigned n = *late_n;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int64_t e = late[i];
    float out[kTetHessVals];
    tet_hessian_values<float, LE>(a, e, disp, project, out);
    store_hess_record(hbuf + (int64_t)kHStride * e, out);
  }
}

// ------------------------------------------------------------ assembly ---
// Terms every slot gets after its per-tet blocks are summed: lumped mass / h^2 and contact
// springs on diagonal blocks, then pinned rows / columns (identity on the diagonal).
template <typename R>
__device__ __forceinline__ void finish_slot(const AsmArgs<R>& a, int v, int w, R (&acc)[9]) {
  if (v == w && a.mass) {
    const R m = R(a.mass[v] * a.inv_h2);
    acc[0] += m; acc[4] += m; acc[8] += m;
  }
  if (v == w && a.contact.n > 0) {
    double x[3], hc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 3; ++i) x[i] = a.contact.X[3 * v + i] + a.u[3 * v + i];
    contact_terms(a.contact, v, x, nullptr, hc);
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] += R(hc[k]);
  }
  if (a.pinned) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        if (a.pinned[3 * v + i] | a.pinned[3 * w + j]) acc[3 * i + j] = (v == w && i == j) ? R(1) : R(0);
  }
}

// the 3x3 inverse of a diagonal block for the block-Jacobi preconditioner
template <typename R>
__device__ __forceinline__ void write_jinv(const AsmArgs<R>& a, int v, const R (&acc)[9]) {
  R C[9];
  cof3(acc, C);
  const R det = acc[0] * C[0] + acc[1] * C[1] + acc[2] * C[2];
  R* ji = a.jinv + 9 * (int64_t)v;
  if (det != R(0)) {
    const R id = R(1) / det;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) ji[3 * i + j] = C[3 * j + i] * id;
  } else {
#pragma unroll
    for (int m = 0; m < 9; ++m) ji[m] = (m % 4 == 0 && acc[m] != R(0)) ? R(1) / acc[m] : R(0);
  }
}

// the solver's block record of slot s (column w) at r
template <typename R>
__device__ __forceinline__ void fill_record(const AsmArgs<R>& a, int w, const R (&acc)[9], R* r) {
#pragma unroll
  for (int m = 0; m < 9; ++m) r[m] = acc[m];
  r[9] = col_bits(w, R(0));
  rec_aux_store(r, a.cmode ? coarse_pack(__ldg(a.cmode + w)) : make_uint2(0u, 0u));
  if (a.colpack) rec_word_store(r, __ldg(a.colpack + w));
}

// offset of a contribution's 9 values inside its tet's kHStride record: diagonal block cd < 4
// (6 stored values, read as 9: the 3 after them are not used and stay inside the record),
// off-diagonal pair cd - 4 (cd < 10) or its transpose (cd - 10)
__device__ __forceinline__ int contribution_offset(int cd) {
  return cd < 4 ? 6 * cd : 24 + 9 * (cd < 10 ? cd - 4 : cd - 10);
}

// Deterministic gather assembly.  Every block slot is the sum of its per-tet blocks (the
// hc_src list of the slot, in tet order) plus the lumped mass / h^2 and contact terms on
// diagonal blocks; pinned rows / columns become identity / zero; diagonal slots also give the
// 3x3 inverse for the block-Jacobi preconditioner.  Output: the solver's block records (rec)
// and / or the entry-major block values of the assembled tier (val).
// SYM: the work items are the upper-triangle slots (up_slot, with the lists hcu_ptr / hcu_src);
// each lane writes its block's record and the transposed block's record in the mirror slot, so the
// matrix is exactly symmetric and the lower triangle's contributions are not gathered again.
//
// A warp owns 32 consecutive slots, whose contributions are one contiguous range of hc_src.
// The range goes through shared memory kAsmChunk contributions at a time: the warp loads each
// contribution's 9 values with 9 consecutive lanes (one or two sectors per contribution, all
// nine loads of a lane in flight) - one lane per slot issuing 9 scalar loads would touch 32
// different tet records per instruction - and stores them already in the slot's orientation
// (diagonal blocks expanded from their 6 packed values, transposed pairs transposed).  Lane p
// then takes contribution p of the chunk; a segmented warp scan (segments = slots, whose
// contributions are contiguous) forms each slot's chunk sum, and the segment's last lane adds
// it to the slot's accumulator in shared memory.  Every sum's order is fixed by the mesh (chunk
// boundaries, scan tree), so the records are bitwise repeatable.  The warp writes its 32
// records with 16-byte stores.
constexpr int kAsmWarps = 8;
constexpr int kAsmChunk = 32;

// index, among a contribution's stored values, of entry m (row-major 3x3) of the slot's block
__device__ __forceinline__ int contribution_entry(int cd, int m) {
  const int i = m / 3, k = m - 3 * i;
  if (cd < 4) {  // symmetric diagonal block packed (xx, xy, xz, yy, yz, zz)
    const int lo = i < k ? i : k, hi = i < k ? k : i;
    return 3 * lo - (lo * (lo - 1)) / 2 + (hi - lo);
  }
  return cd < 10 ? m : 3 * k + i;
}

// a lane's record (staged in shared memory at r) to slot s, in 16-byte pieces
template <typename R>
__device__ __forceinline__ void store_record(const AsmArgs<R>& a, const R* r, int64_t s) {
  constexpr int kPer = kRec * (int)sizeof(R) / 16;
  const int4* src = reinterpret_cast<const int4*>(r);
  int4* dst = reinterpret_cast<int4*>(a.rec + kRec * s);
#pragma unroll
  for (int t = 0; t < kPer; ++t) dst[t] = src[t];
}

template <typename R, bool SYM>
__global__ void __launch_bounds__(32 * kAsmWarps) k_assemble(AsmArgs<R> a) {
  __shared__ __align__(16) R stage[kAsmWarps][9 * kAsmChunk];
  __shared__ __align__(16) R srec[kAsmWarps][kRec * 32];  // the slots' accumulators, then their records
  __shared__ unsigned char sown[kAsmWarps][kAsmChunk];
  __shared__ int sentry[16 * 9];  // [pair code][entry]: offset in the tet record, in the slot's orientation
  for (int i = threadIdx.x; i < 16 * 9; i += blockDim.x)
    sentry[i] = contribution_offset(i / 9) + contribution_entry(i / 9, i - 9 * (i / 9));
  __syncthreads();
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t items = SYM ? a.n_up : a.nb;              // slots, or upper-triangle slots
  const int32_t* hcp = SYM ? a.hcu_ptr : a.hc_ptr;
  const int32_t* hcs = SYM ? a.hcu_src : a.hc_src;
  const int64_t s0 = ((int64_t)blockIdx.x * kAsmWarps + wid) * 32;
  if (s0 >= items) return;  // warp-uniform
  const int64_t j = s0 + lane;
  const bool has = j < items;
  int64_t s = j, mir = j;
  int v = 0, w = 0, cb = 0, ce = 0;
  bool active = has;
  if (has) {
    if constexpr (SYM) {
      s = __ldg(a.up_slot + j);
      mir = __ldg(a.up_mirror + j);
    }
    v = __ldg(a.bsr_row + s);
    w = __ldg(a.bsr_col + s);
    cb = __ldg(hcp + j);
    ce = __ldg(hcp + j + 1);
    if (a.inst_active && !a.inst_active[__ldg(a.vert_inst + v)]) active = false;
  }
  const unsigned act = __ballot_sync(0xffffffffu, active);
  if (act == 0u) return;  // every slot of the warp belongs to an instance that is not stepping
  const int last = (int)min((int64_t)31, items - 1 - s0);
  const int wb = __shfl_sync(0xffffffffu, cb, 0);
  const int we = __shfl_sync(0xffffffffu, ce, last);
  R* st = stage[wid];
  R* accs = srec[wid];  // 9 per slot while summing
  unsigned char* own = sown[wid];
#pragma unroll
  for (int m = 0; m < 9; ++m) accs[9 * lane + m] = R(0);
  for (int k0 = wb; k0 < we; k0 += kAsmChunk) {
    const int nk = min(kAsmChunk, we - k0);
    const int code = lane < nk ? __ldg(hcs + k0 + lane) : 0;
    // segment heads and their owner slots: a slot's contributions start at cb - k0, and the slot
    // whose range holds k0 owns position 0 (exactly one lane meets each condition per position)
    const bool starts = has && cb > k0 && cb < k0 + nk;
    if (starts) own[cb - k0] = (unsigned char)lane;
    if (has && cb <= k0 && k0 < ce) own[0] = (unsigned char)lane;
    const unsigned heads = __reduce_or_sync(0xffffffffu, starts ? 1u << (cb - k0) : 0u) | 1u;
    R vals[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int j = lane + 32 * t;  // element j of the chunk: contribution j / 9, entry j % 9
      const int cj = j / 9;
      const int cc = __shfl_sync(0xffffffffu, code, cj);
      vals[t] = R(0);
      if (cj < nk) vals[t] = __ldg(a.hbuf + (int64_t)kHStride * (cc >> 4) + sentry[9 * (cc & 15) + (j - 9 * cj)]);
    }
#pragma unroll
    for (int t = 0; t < 9; ++t) st[lane + 32 * t] = vals[t];
    __syncwarp();
    // lane = position p: inclusive segmented scan over [head(p), p]
    const int hp = lane < nk ? 31 - __clz(heads & (0xffffffffu >> (31 - lane))) : lane;
    R x[9];
#pragma unroll
    for (int m = 0; m < 9; ++m) x[m] = lane < nk ? st[9 * lane + m] : R(0);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
      for (int m = 0; m < 9; ++m) {
        const R y = __shfl_up_sync(0xffffffffu, x[m], d);
        if (lane - d >= hp) x[m] += y;
      }
    }
    const bool tail = lane < nk && (lane == nk - 1 || ((heads >> (lane + 1)) & 1u));
    if (tail) {
      R* acc = accs + 9 * own[hp];
#pragma unroll
      for (int m = 0; m < 9; ++m) acc[m] += x[m];
    }
    __syncwarp();
  }
  R acc[9];
#pragma unroll
  for (int m = 0; m < 9; ++m) acc[m] = accs[9 * lane + m];
  __syncwarp();  // every accumulator is read before the records overwrite the area
  R* my = srec[wid] + kRec * lane;
  if (active) {
    finish_slot(a, v, w, acc);
    if (a.rec) {
      fill_record(a, w, acc, my);
      if constexpr (SYM) {   // this lane's record, then the transposed block's (own staging area only)
        store_record(a, my, s);
        if (mir != s) {
          R t[9];
#pragma unroll
          for (int m = 0; m < 9; ++m) t[m] = acc[3 * (m % 3) + m / 3];
          fill_record(a, v, t, my);
          store_record(a, my, mir);
        }
      }
    }
    if (a.val) {
      const int rp = __ldg(a.rowptr + v);
      const int K = __ldg(a.rowptr + v + 1) - rp;
      R* dst = a.val + 9 * (int64_t)rp + (s - rp);
#pragma unroll
      for (int m = 0; m < 9; ++m) dst[(int64_t)m * K] = acc[m];
      if (SYM && mir != s) {
        const int rq = __ldg(a.rowptr + w);
        const int Kq = __ldg(a.rowptr + w + 1) - rq;
        R* dq = a.val + 9 * (int64_t)rq + (mir - rq);
#pragma unroll
        for (int m = 0; m < 9; ++m) dq[(int64_t)m * Kq] = acc[3 * (m % 3) + m / 3];
      }
    }
    if (v == w && a.jinv) write_jinv(a, v, acc);
  }
  if (SYM || !a.rec) return;  // warp-uniform
  __syncwarp();
  // 32 records of kRec values: 16-byte pieces, each inside one record
  constexpr int kPer = kRec * (int)sizeof(R) / 16;  // pieces per record
  const int4* src = reinterpret_cast<const int4*>(srec[wid]);
  int4* dst = reinterpret_cast<int4*>(a.rec + kRec * s0);
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int q = lane + 32 * t;
    if ((act >> (q / kPer)) & 1u) dst[q] = src[q];
  }
}

// --------------------------------------------------------- FP64 forces ---
// f_a = vol P(F) grad N_a per tet, in FP64 (the Newton residual is formed
// from these; FP32 cannot resolve 1e-6 relative residuals of stiff beams).
// The mixed-precision stepper uses the double-float kernel below for the
// neo-Hookean and linear materials.
// COROT: the instantiation for ARAP / fixed-corotated meshes (its SVD would cost the
// neo-Hookean instantiation registers and occupancy).
template <bool COROT>
__global__ void __launch_bounds__(128) k_tet_forces(TetArgs<double> a, int disp, double* __restrict__ fbuf) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= a.t) return;
  const int4 v = __ldg(a.tets + e);
  double du[9], D[9], G[9], P[9], gN[12];
  tet_du(a.u, v, du);
  load_dinv(a.dinv, a.t, e, D);
  disp_grad(du, D, G);
  add_fbar(a, e, G);
  const double vol = a.vol[e], mu = a.mu[e], lam = a.lam[e];
  const int mat = COROT ? a.material : (a.material == kMatMMNH || a.material == kMatLE ? a.material : kMatSNH);
  if (COROT ? mat == kMatARAP : false) {
    if (disp) arap_pk1_disp<double>(G, mu, P);
    else arap_pk1<double>(G, mu, P);
  } else if (COROT) {
    if (disp) fcr_pk1_disp<double>(G, mu, lam, P);
    else fcr_pk1<double>(G, mu, lam, P);
  } else if (mat == kMatMMNH) {
    if (disp) mmnh_pk1_disp<double>(G, mu, lam, P);
    else mmnh_pk1<double>(G, mu, lam, P);
  } else if (mat == kMatLE) {
    if (disp) le_pk1_disp_d<double, 3>(G, mu, lam, P);
    else le_pk1_d<double, 3>(G, mu, lam, P);
  } else {
    if (disp) snh_pk1_disp<double>(G, mu, lam, P);
    else snh_pk1<double>(G, mu, lam, P);
  }
  shape_grads(D, gN);
  double* f = fbuf + 12 * e;
#pragma unroll
  for (int b = 0; b < 4; ++b)
#pragma unroll
    for (int i = 0; i < 3; ++i)
      f[3 * b + i] = vol * (P[3 * i] * gN[3 * b] + P[3 * i + 1] * gN[3 * b + 1] + P[3 * i + 2] * gN[3 * b + 2]);
}

// Double-float forces of the mixed-precision stepper (neo-Hookean and linear materials,
// displacement form): the f_a of k_tet_forces evaluated in double-float
// arithmetic (dfloat.cuh) from the FP32 hi/lo splits of u (uh, ul) and of Dinv
// (dinv_hi = dinv32, dinv_lo), so that only the three material loads touch the
// FP64 units.  Written as (hi, lo) pairs for k_vertex_gradient<true>.  This function: the 12
// components of tet e (vertex-major: f[3 b + i]) into f.
__device__ __forceinline__ void tet_forces_df(const TetArgs<double>& a, const float* __restrict__ dinv_hi,
                                              const float* __restrict__ dinv_lo, const float* __restrict__ uh,
                                              const float* __restrict__ ul, int64_t e, float2* f) {
  const int4 v = __ldg(a.tets + e);
  DF du[9], D[9], G[9], P[9], gN[12];
  {
    const Vec3<float> h0 = ld3(uh, v.x), l0 = ld3(ul, v.x);
    const DF x0 = DF(h0.x, l0.x), y0 = DF(h0.y, l0.y), z0 = DF(h0.z, l0.z);
    const int vv[3] = {v.y, v.z, v.w};
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const Vec3<float> h = ld3(uh, vv[b]), l = ld3(ul, vv[b]);
      du[3 * b + 0] = DF(h.x, l.x) - x0;
      du[3 * b + 1] = DF(h.y, l.y) - y0;
      du[3 * b + 2] = DF(h.z, l.z) - z0;
    }
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) D[k] = DF(__ldg(dinv_hi + k * a.t + e), __ldg(dinv_lo + k * a.t + e));
  disp_grad(du, D, G);
  const DF vol(a.vol[e]), mu(a.mu[e]), lam(a.lam[e]);
  if (a.material == kMatMMNH)
    mmnh_pk1_disp<DF>(G, mu, lam, P);
  else if (a.material == kMatLE)
    le_pk1_disp_d<DF, 3>(G, mu, lam, P);
  else
    snh_pk1_disp<DF>(G, mu, lam, P);
  shape_grads(D, gN);
#pragma unroll
  for (int b = 0; b < 4; ++b)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const DF s = vol * (P[3 * i] * gN[3 * b] + P[3 * i + 1] * gN[3 * b + 1] + P[3 * i + 2] * gN[3 * b + 2]);
      f[3 * b + i] = make_float2(s.hi, s.lo);
    }
}

__global__ void __launch_bounds__(128) k_tet_forces_df(TetArgs<double> a, const float* __restrict__ dinv_hi,
                                                       const float* __restrict__ dinv_lo,
                                                       const float* __restrict__ uh, const float* __restrict__ ul,
                                                       float2* __restrict__ fbuf) {
  // the block's 128 tets' forces are staged here and written out as one contiguous span (per-thread
  // stores of a tet's 12 pairs at a 96-byte stride made every warp store touch 32 sectors)
  __shared__ __align__(16) float2 stage[128 * 12];
  const int64_t e0 = blockIdx.x * (int64_t)blockDim.x;
  const int64_t e = e0 + threadIdx.x;
  if (e < a.t) tet_forces_df(a, dinv_hi, dinv_lo, uh, ul, e, stage + 12 * threadIdx.x);
  __syncthreads();
  const int nt = (int)min((int64_t)blockDim.x, a.t - e0);
  float4* dst = reinterpret_cast<float4*>(fbuf + 12 * e0);
  const float4* src = reinterpret_cast<const float4*>(stage);
  for (int k = threadIdx.x; k < 6 * nt; k += blockDim.x) dst[k] = src[k];
}

// low parts of Dinv for the double-float forces: dinv = dinv32 + dinv_lo to ~48 bits
__global__ void k_dinv_lo(const double* __restrict__ dinv, const float* __restrict__ dinv32, int64_t n,
                          float* __restrict__ lo) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) lo[i] = float(dinv[i] - double(dinv32[i]));
}

// Vertex gather of the forces in list (tet) order, plus the backward-Euler
// terms M/h^2 (u - u_tilde) - f_ext when `mass` is set; pinned DOFs are
// zeroed.  Grid-stride over a fixed grid; ||g||^2 reduced deterministically.
// DFB: the forces are double-float pairs (k_tet_forces_df), summed in double-float.
template <bool DFB>
__global__ void __launch_bounds__(kBlock) k_vertex_gradient(GradArgs a) {
  double gg[1] = {0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < a.n; v += stride) {
    double acc[3] = {0.0, 0.0, 0.0};
    if constexpr (DFB) {
      DF s[3] = {DF(0.f, 0.f), DF(0.f, 0.f), DF(0.f, 0.f)};
      const int kb = __ldg(a.v2t_ptr + v), ke = __ldg(a.v2t_ptr + v + 1);
#pragma unroll 4
      for (int k = kb; k < ke; ++k) {
        const int code = __ldg(a.v2t + k);
        const float2* f = reinterpret_cast<const float2*>(a.fbuf) + 12 * (int64_t)(code >> 2) + 3 * (code & 3);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float2 x = f[c];
          s[c] += DF(x.x, x.y);
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] = s[c].to_double();
    } else {
      for (int k = __ldg(a.v2t_ptr + v); k < __ldg(a.v2t_ptr + v + 1); ++k) {
        const int code = __ldg(a.v2t + k);
        const double* f = a.fbuf + 12 * (int64_t)(code >> 2) + 3 * (code & 3);
        acc[0] += f[0];
        acc[1] += f[1];
        acc[2] += f[2];
      }
    }
    if (a.contact.n > 0) {
      double x[3];
      for (int i = 0; i < 3; ++i) x[i] = a.contact.X[3 * v + i] + a.u[3 * v + i];
      contact_terms(a.contact, v, x, acc, nullptr);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int64_t d = 3 * v + i;
      double g = acc[i];
      if (a.mass) g += a.mass[v] * a.inv_h2 * (a.u[d] - a.ut[d]);
      if (a.f_ext) g -= a.f_ext[d];
      if (a.pinned && a.pinned[d]) g = 0.0;
      a.g[d] = g;
      gg[0] += g * g;
    }
  }
  grid_sum<1, kBlock>(gg, a.partials, a.counter, a.out);
}

// ----------------------------------------------------------- energies ----
// Solver energy relative to rest at u + step * dx:
//   sum_e vol_e (psi(F_e) - psi(I)) + sum_free [m/2h^2 (u+s dx-u~)^2 - f (u+s dx)]
// plus its magnitude sum |terms| (the FP32 noise scale of the value).
// Mode DIRECT instead sums vol_e psi(F_e) from absolute positions in FP64
// (simkit's stable_neo_hookean_energy_x, snh.py:449-474).
// vol * (psi - psi(I)) of tet e at u + step dx (DIRECT: vol * psi from absolute positions)
template <typename R, bool DIRECT>
__device__ __forceinline__ double tet_energy_term(const EnergyArgs<R>& a, int64_t e, R step) {
  const int4 v = __ldg(a.tet.tets + e);
  R du[9], D[9], G[9];
  if constexpr (sizeof(R) == 8) {
    tet_du(a.tet.u, v, du);
  } else {
    tet_du(a.tet.uh, a.tet.ul, v, du);
  }
  if (a.dx && step != R(0)) {
    const Vec3<R> d0 = ld3(a.dx, v.x);
    const int vv[3] = {v.y, v.z, v.w};
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const Vec3<R> db = ld3(a.dx, vv[b]);
      du[3 * b + 0] += step * (db.x - d0.x);
      du[3 * b + 1] += step * (db.y - d0.y);
      du[3 * b + 2] += step * (db.z - d0.z);
    }
  }
  load_dinv(a.tet.dinv, a.tet.t, e, D);
  disp_grad(du, D, G);
  if (DIRECT) add_fbar(a.tet, e, G);
  const R vol = __ldg(a.tet.vol + e), mu = __ldg(a.tet.mu + e), lam = __ldg(a.tet.lam + e);
  if (DIRECT) return double(vol) * double(mat_psi<R>(a.tet.material, G, mu, lam));
  return double(vol * mat_dpsi<R>(a.tet.material, G, mu, lam));
}

// kinetic + gravity terms of vertex v's free DOFs at u + step dx; acc[1] gets magnitudes
template <typename R>
__device__ __forceinline__ void vertex_energy_terms(const EnergyArgs<R>& a, int64_t v, double step, double (&acc)[2]) {
  Vec3<R> d = {R(0), R(0), R(0)};
  if (a.dx && step != 0.0) d = ld3(a.dx, v);
  const double dd[3] = {double(d.x), double(d.y), double(d.z)};
  const double mh = a.mass[v] * a.inv_h2;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int64_t k = 3 * v + c;
    if (a.pinned && a.pinned[k]) continue;
    const double x = a.tet.u[k] + step * dd[c];
    const double r = x - a.ut[k];
    const double kin = 0.5 * mh * r * r;
    const double pot = a.f_ext ? -a.f_ext[k] * x : 0.0;
    acc[0] += kin + pot;
    acc[1] += kin + fabs(pot);
  }
  if (a.contact.n > 0) {
    double x[3];
    for (int c = 0; c < 3; ++c) x[c] = a.contact.X[3 * v + c] + a.tet.u[3 * v + c] + step * dd[c];
    const double ec = contact_terms(a.contact, v, x, nullptr, nullptr);
    acc[0] += ec;
    acc[1] += ec;
  }
}

// standalone contact springs (simkit/energies/contact_springs_plane.py:44-200), one plane
__global__ void k_contact_plane(const double* __restrict__ x, int64_t n, Contact c, double* __restrict__ ev,
                                double* __restrict__ grad, double* __restrict__ hdiag, uint8_t* __restrict__ under) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  const double xv[3] = {x[3 * v], x[3 * v + 1], x[3 * v + 2]};
  double g[3] = {0.0, 0.0, 0.0}, h[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const double e = contact_terms(c, v, xv, g, h);
  const double d = (xv[0] - c.p[0][0]) * c.nrm[0][0] + (xv[1] - c.p[0][1]) * c.nrm[0][1] +
                   (xv[2] - c.p[0][2]) * c.nrm[0][2];
  if (ev) ev[v] = e;
  if (grad)
    for (int i = 0; i < 3; ++i) grad[3 * v + i] = g[i];
  if (hdiag)
    for (int k = 0; k < 9; ++k) hdiag[9 * v + k] = h[k];
  if (under) under[v] = d < 0.0 ? 1 : 0;
}

template <typename R, bool DIRECT>
__global__ void __launch_bounds__(kBlock) k_energy(EnergyArgs<R> a) {
  double acc[2] = {0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t total = a.tet.t + (DIRECT ? 0 : a.n);
  const double stepd = a.step_dev ? *a.step_dev : a.step;
  const R step = R(stepd);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += stride) {
    if (i < a.tet.t) {
      const double val = tet_energy_term<R, DIRECT>(a, i, step);
      acc[0] += val;
      acc[1] += fabs(val);
    } else {
      vertex_energy_terms<R>(a, i - a.tet.t, stepd, acc);
    }
  }
  grid_sum<2, kBlock>(acc, a.partials, a.counter, a.out);
}

// Per-instance energy of a batch: one CTA per instance sums its tets and
// vertices in a fixed order (deterministic); instances with mask 0 skip.
// steps[inst] is the trial step of that instance's line search.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_inst_energy(EnergyArgs<R> a, const int32_t* __restrict__ inst_rows,
                                                        const int32_t* __restrict__ inst_tets,
                                                        const uint8_t* __restrict__ mask,
                                                        const double* __restrict__ steps, double* __restrict__ out2) {
  const int inst = blockIdx.x;
  if (mask && !mask[inst]) return;
  const double stepd = steps ? steps[inst] : 0.0;
  const R step = R(stepd);
  double acc[2] = {0.0, 0.0};
  for (int64_t e = inst_tets[inst] + threadIdx.x; e < inst_tets[inst + 1]; e += blockDim.x) {
    const double val = tet_energy_term<R, false>(a, e, step);
    acc[0] += val;
    acc[1] += fabs(val);
  }
  for (int64_t v = inst_rows[inst] + threadIdx.x; v < inst_rows[inst + 1]; v += blockDim.x)
    vertex_energy_terms<R>(a, v, stepd, acc);
  block_sum<2, kBlock>(acc);
  if (threadIdx.x == 0) {
    out2[2 * inst] = acc[0];
    out2[2 * inst + 1] = acc[1];
  }
}

// hi/lo split of FP64 positions for the FP32 kernels, padded to 4
__global__ void k_split(const double* __restrict__ u, int64_t n, float* __restrict__ uh, float* __restrict__ ul) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  float h[3], l[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double x = u[3 * v + c];
    h[c] = float(x);
    l[c] = float(x - double(h[c]));
  }
  reinterpret_cast<float4*>(uh)[v] = make_float4(h[0], h[1], h[2], 0.f);
  reinterpret_cast<float4*>(ul)[v] = make_float4(l[0], l[1], l[2], 0.f);
}

// ------------------------------------------------------------ launchers --
template <typename R>
int launch_tet_hessian(const TetArgs<R>& a, int disp, int project, R* hbuf, cudaStream_t s, HessLate late) {
  if (late.launches) *late.launches = 1;
  if (a.t == 0) return SKG_OK;
  const int blocks = blocks_for(a.t, kHessThreads);
  bool launched = false;
  if (a.material == kMatLE) {
    k_tet_hessian<R, true><<<blocks, kHessThreads, 0, s>>>(a, disp, project, hbuf, nullptr, nullptr);
    launched = true;
  }
  if constexpr (sizeof(R) == 4) {
    if (!launched && late.list && late.n) {
      SKG_CUDA(cudaMemsetAsync(late.n, 0, sizeof(unsigned), s));
      k_tet_hessian<R, false, true><<<blocks, kHessThreads, 0, s>>>(a, disp, project, hbuf, late.list, late.n);
      SKG_LAUNCHED();
      k_tet_hessian_late<R, false><<<kLateBlocks, kHessThreads, 0, s>>>(a, disp, project, hbuf, late.list, late.n);
      if (late.launches) *late.launches = 2;
      launched = true;
    }
  }
  if (!launched) k_tet_hessian<R, false><<<blocks, kHessThreads, 0, s>>>(a, disp, project, hbuf, nullptr, nullptr);
  SKG_LAUNCHED();
  return SKG_OK;
}

template <typename R>
int launch_assemble(const AsmArgs<R>& a, cudaStream_t s) {
  if (a.nb == 0) return SKG_OK;
  const bool sym = a.up_slot != nullptr;
  const int64_t warps = ((sym ? a.n_up : a.nb) + 31) / 32;
  const int blocks = (int)((warps + kAsmWarps - 1) / kAsmWarps);
  if (sym)
    k_assemble<R, true><<<blocks, 32 * kAsmWarps, 0, s>>>(a);
  else
    k_assemble<R, false><<<blocks, 32 * kAsmWarps, 0, s>>>(a);
  SKG_LAUNCHED();
  return SKG_OK;
}

int launch_forces(const TetArgs<double>& a, int disp, double* fbuf, cudaStream_t s) {
  if (a.t == 0) return SKG_OK;
  if (a.material == kMatARAP || a.material == kMatFCR)
    k_tet_forces<true><<<blocks_for(a.t, 128), 128, 0, s>>>(a, disp, fbuf);
  else
    k_tet_forces<false><<<blocks_for(a.t, 128), 128, 0, s>>>(a, disp, fbuf);
  SKG_LAUNCHED();
  return SKG_OK;
}

int launch_vertex_gradient(const GradArgs& a, cudaStream_t s, bool df) {
  if (df)
    k_vertex_gradient<true><<<reduce_blocks(a.n), kBlock, 0, s>>>(a);
  else
    k_vertex_gradient<false><<<reduce_blocks(a.n), kBlock, 0, s>>>(a);
  SKG_LAUNCHED();
  return SKG_OK;
}

int launch_forces_df(const TetArgs<double>& a, const float* dinv32, const float* dinv_lo, const float* uh,
                     const float* ul, double* fbuf, cudaStream_t s) {
  if (a.t == 0) return SKG_OK;
  k_tet_forces_df<<<blocks_for(a.t, 128), 128, 0, s>>>(a, dinv32, dinv_lo, uh, ul, reinterpret_cast<float2*>(fbuf));
  SKG_LAUNCHED();
  return SKG_OK;
}

int launch_dinv_lo(const skg_tet_mesh* m, float* lo, cudaStream_t s) {
  const int64_t n = 9 * m->n_tets;
  if (n == 0) return SKG_OK;
  k_dinv_lo<<<blocks_for(n), kBlock, 0, s>>>(m->dinv, m->dinv32, n, lo);
  SKG_LAUNCHED();
  return SKG_OK;
}

template <typename R>
int launch_energy(const EnergyArgs<R>& a, bool direct, cudaStream_t s) {
  const int64_t total = a.tet.t + (direct ? 0 : a.n);
  if (direct)
    k_energy<R, true><<<reduce_blocks(total), kBlock, 0, s>>>(a);
  else
    k_energy<R, false><<<reduce_blocks(total), kBlock, 0, s>>>(a);
  SKG_LAUNCHED();
  return SKG_OK;
}

template <typename R>
int launch_inst_energy(const EnergyArgs<R>& a, int n_inst, const int32_t* inst_rows, const int32_t* inst_tets,
                       const uint8_t* mask, const double* steps, double* out2, cudaStream_t s) {
  if (n_inst <= 0) return SKG_OK;
  k_inst_energy<R><<<n_inst, kBlock, 0, s>>>(a, inst_rows, inst_tets, mask, steps, out2);
  SKG_LAUNCHED();
  return SKG_OK;
}
template int launch_inst_energy<float>(const EnergyArgs<float>&, int, const int32_t*, const int32_t*,
                                       const uint8_t*, const double*, double*, cudaStream_t);
template int launch_inst_energy<double>(const EnergyArgs<double>&, int, const int32_t*, const int32_t*,
                                        const uint8_t*, const double*, double*, cudaStream_t);

int launch_split(const double* u, int64_t n, float* uh, float* ul, cudaStream_t s) {
  k_split<<<blocks_for(n), kBlock, 0, s>>>(u, n, uh, ul);
  SKG_LAUNCHED();
  return SKG_OK;
}

template int launch_tet_hessian<float>(const TetArgs<float>&, int, int, float*, cudaStream_t, HessLate);
template int launch_tet_hessian<double>(const TetArgs<double>&, int, int, double*, cudaStream_t, HessLate);
template int launch_assemble<float>(const AsmArgs<float>&, cudaStream_t);
template int launch_assemble<double>(const AsmArgs<double>&, cudaStream_t);
template int launch_energy<float>(const EnergyArgs<float>&, bool, cudaStream_t);
template int launch_energy<double>(const EnergyArgs<double>&, bool, cudaStream_t);

// --------------------------------------------------- workspace layout ----
Workspace carve_workspace(const skg_tet_mesh* m, int precision, void* base) {
  Carve c(base);
  Workspace w{};
  const int64_t t = m->n_tets, n = m->n_verts, nb = m->n_blocks;
  const bool mixed = precision == SKG_MIXED;
  w.hbuf32 = mixed ? c.take<float>(kHStride * t) : nullptr;
  w.hlate = mixed ? c.take<int32_t>(t) : nullptr;
  w.hlate_n = mixed ? c.take<unsigned>(4) : nullptr;
  w.hbuf64 = mixed ? nullptr : c.take<double>(kHStride * t);
  w.fbuf = c.take<double>(12 * t);
  w.val32 = mixed ? c.take<float>(9 * nb) : nullptr;
  w.val64 = mixed ? nullptr : c.take<double>(9 * nb);
  w.rec32 = mixed ? c.take<float>(kRec * nb) : nullptr;
  w.rec64 = mixed ? nullptr : c.take<double>(kRec * nb);
  w.jinv32 = mixed ? c.take<float>(9 * n) : nullptr;
  w.jinv64 = mixed ? nullptr : c.take<double>(9 * n);
  w.g = c.take<double>(3 * n);
  w.ut = c.take<double>(3 * n);
  w.uh = c.take<float>(4 * n);
  w.ul = c.take<float>(4 * n);
  w.dinv_lo = mixed ? c.take<float>(9 * t) : nullptr;
  for (int k = 0; k < 6; ++k) {
    w.vec32[k] = mixed ? c.take<float>(4 * n) : nullptr;
    w.vec64[k] = mixed ? nullptr : c.take<double>(4 * n);
  }
  w.partials = c.take<double>(8 * kMaxGrid);
  w.counter = c.take<unsigned>(16);
  w.scal = c.take<double>(64);
  if (m->coarse && !m->coarse->inst_agg) {
    const int64_t np = coarse_padded(m);
    w.cM = c.take<float>(np * np);
    w.crowp = c.take<float>(2 * 32 * np);
    w.crc = c.take<unsigned long long>(np);
    w.crq = c.take<unsigned long long>(2 * np);
    w.crcg = c.take<double>(2 * np);
    w.ce = c.take<float>(8 * (int64_t)m->coarse->n_agg);
    w.cok = c.take<int>(4);
    w.cbar = c.take<unsigned>(4);
  } else if (m->coarse) {
    // per-instance form: dense blocks of every instance, row panels per inversion CTA
    const skg_coarse* h = m->coarse;
    w.cM = c.take<float>(h->m_floats);
    w.crowp = c.take<float>((int64_t)kCoarseInvCtas * 2 * 32 * h->max_np);
    w.crc = c.take<unsigned long long>(6 * (int64_t)h->n_agg + 32);
    w.ce = c.take<float>(8 * (int64_t)h->n_agg);
    w.cok = c.take<int>(h->n_inst + 4);
    w.cbar = c.take<unsigned>(4);
  }
  w.bytes = c.off + 256;
  return w;
}

}  // namespace skg

using namespace skg;

static TetArgs<double> tet_args64(const skg_tet_mesh* m, const double* u) {
  TetArgs<double> a{};
  a.t = m->n_tets;
  a.tets = reinterpret_cast<const int4*>(m->tets);
  a.dinv = m->dinv;
  a.vol = m->vol;
  a.mu = m->mu;
  a.lam = m->lam;
  a.u = u;
  a.material = m->material;
  return a;
}

namespace skg {
TetArgs<double> make_tet_args64(const skg_tet_mesh* m, const double* u) { return tet_args64(m, u); }
TetArgs<float> make_tet_args32(const skg_tet_mesh* m, const double* u, const float* uh, const float* ul) {
  TetArgs<float> a{};
  a.t = m->n_tets;
  a.tets = reinterpret_cast<const int4*>(m->tets);
  a.dinv = m->dinv32;
  a.vol = m->mat32;
  a.mu = m->mat32 + m->n_tets;
  a.lam = m->mat32 + 2 * m->n_tets;
  a.u = u;
  a.uh = uh;
  a.ul = ul;
  a.material = m->material;
  return a;
}
int check_mesh(const skg_tet_mesh* m, int precision) {
  if (!m) return fail(SKG_ERR_ARG, "mesh is null");
  if (m->n_verts <= 0 || m->n_tets < 0 || m->n_blocks < m->n_verts)
    return fail(SKG_ERR_ARG, "mesh sizes are inconsistent");
  if (!m->tets || !m->dinv || !m->vol || !m->mu || !m->lam || !m->bsr_rowptr || !m->bsr_col || !m->bsr_row ||
      !m->bsr_diag || !m->hc_ptr || !m->hc_src || !m->v2t_ptr || !m->v2t)
    return fail(SKG_ERR_ARG, "mesh has a null array");
  if (precision == SKG_MIXED && (!m->dinv32 || !m->mat32))
    return fail(SKG_ERR_ARG, "mixed precision needs the FP32 mesh copies");
  if (precision != SKG_MIXED && precision != SKG_FP64) return fail(SKG_ERR_ARG, "unknown precision %d", precision);
  if (m->material < SKG_MAT_STABLE_NEO_HOOKEAN || m->material > SKG_MAT_LINEAR_ELASTICITY)
    return fail(SKG_ERR_ARG, "unknown material %d", m->material);
  if (m->coarse) {
    const skg_coarse* c = m->coarse;
    if (!c->mode || !c->cb_ptr || !c->cb_slot || !c->cb_rc) return fail(SKG_ERR_ARG, "coarse has a null array");
    if (!c->inst_agg) {
      if (c->n_agg <= 0 || 6 * (int64_t)c->n_agg > 4096 || c->n_cblocks < c->n_agg)
        return fail(SKG_ERR_ARG, "coarse: %d aggregates (1..682 allowed), %d coarse blocks", c->n_agg, c->n_cblocks);
    } else {
      if (c->n_inst <= 0 || c->n_agg < c->n_inst || c->max_np <= 0 || c->max_np > 768 || c->max_np % 32 ||
          c->m_floats <= 0 || !c->agg_inst || !c->inst_moff || !c->colpack)
        return fail(SKG_ERR_ARG, "coarse (per instance): %d instances, %d aggregates, largest block %d", c->n_inst,
                    c->n_agg, c->max_np);
    }
  }
  return SKG_OK;
}
}  // namespace skg

extern "C" {

int64_t skg_assembly_workspace_size(const skg_tet_mesh* mesh, int precision) {
  if (check_mesh(mesh, precision) != SKG_OK) return -1;
  return carve_workspace(mesh, precision, nullptr).bytes;
}

int skg_contact_plane_terms(const double* x, int64_t n, const skg_contact_plane* plane_h, const double* mass,
                            double* energy_v, double* grad, double* hdiag, uint8_t* under, void* stream) {
  if (!x || !plane_h || n < 0) return fail(SKG_ERR_ARG, "contact_plane_terms: bad arguments");
  if (n == 0) return SKG_OK;
  Contact c{};
  c.n = 1;
  c.w = mass;
  for (int i = 0; i < 3; ++i) {
    c.p[0][i] = plane_h->p[i];
    c.nrm[0][i] = plane_h->n[i];
  }
  c.k[0] = plane_h->k;
  k_contact_plane<<<blocks_for(n), kBlock, 0, as_stream(stream)>>>(x, n, c, energy_v, grad, hdiag, under);
  SKG_LAUNCHED();
  return SKG_OK;
}

}  // extern "C"

// The _x tier (fbar = null: x are positions) and the _u tier (x are displacements u,
// F = J u + fbar) share these bodies.
static int energy_xu(const skg_tet_mesh* mesh, const double* x, const double* fbar, double* energy_h, void* ws,
                     void* stream) {
  SKG_TRY(check_mesh(mesh, SKG_FP64));
  if (!x || !ws || !energy_h) return fail(SKG_ERR_ARG, "energy: null pointer");
  cudaStream_t s = as_stream(stream);
  Workspace w = carve_workspace(mesh, SKG_FP64, ws);
  SKG_CUDA(cudaMemsetAsync(w.counter, 0, 16 * sizeof(unsigned), s));
  EnergyArgs<double> a{};
  a.tet = tet_args64(mesh, x);
  a.tet.fbar = fbar;
  a.n = mesh->n_verts;
  a.partials = w.partials;
  a.counter = w.counter;
  a.out = w.scal;
  SKG_TRY(launch_energy<double>(a, true, s));
  SKG_CUDA(cudaMemcpyAsync(energy_h, w.scal, sizeof(double), cudaMemcpyDeviceToHost, s));
  SKG_CUDA(cudaStreamSynchronize(s));
  return SKG_OK;
}

static int gradient_xu(const skg_tet_mesh* mesh, const double* x, const double* fbar, double* g, void* ws,
                       void* stream) {
  SKG_TRY(check_mesh(mesh, SKG_FP64));
  if (!x || !g || !ws) return fail(SKG_ERR_ARG, "gradient: null pointer");
  cudaStream_t s = as_stream(stream);
  Workspace w = carve_workspace(mesh, SKG_FP64, ws);
  SKG_CUDA(cudaMemsetAsync(w.counter, 0, 16 * sizeof(unsigned), s));
  TetArgs<double> ta = tet_args64(mesh, x);
  ta.fbar = fbar;
  SKG_TRY(launch_forces(ta, 0, w.fbuf, s));
  GradArgs ga{};
  ga.n = mesh->n_verts;
  ga.v2t_ptr = mesh->v2t_ptr;
  ga.v2t = mesh->v2t;
  ga.fbuf = w.fbuf;
  ga.g = g;
  ga.partials = w.partials;
  ga.counter = w.counter;
  ga.out = w.scal;
  return launch_vertex_gradient(ga, s);
}

static int hessian_xu(const skg_tet_mesh* mesh, const double* x, const double* fbar, int precision, int psd,
                      double* val64, float* val32, void* ws, void* stream) {
  SKG_TRY(check_mesh(mesh, precision));
  if (!x || !ws) return fail(SKG_ERR_ARG, "hessian: null pointer");
  cudaStream_t s = as_stream(stream);
  Workspace w = carve_workspace(mesh, precision, ws);
  if (precision == SKG_FP64) {
    if (!val64) return fail(SKG_ERR_ARG, "hessian: FP64 needs val64");
    TetArgs<double> ta = tet_args64(mesh, x);
    ta.fbar = fbar;
    SKG_TRY(launch_tet_hessian<double>(ta, 0, psd, w.hbuf64, s));
    AsmArgs<double> aa = make_asm_args<double>(mesh, w.hbuf64, val64, nullptr);
    return launch_assemble<double>(aa, s);
  }
  if (!val32) return fail(SKG_ERR_ARG, "hessian: mixed precision needs val32");
  SKG_TRY(launch_split(x, mesh->n_verts, w.uh, w.ul, s));
  TetArgs<float> ta = make_tet_args32(mesh, x, w.uh, w.ul);
  ta.fbar = fbar;
  SKG_TRY(launch_tet_hessian<float>(ta, 0, psd, w.hbuf32, s, HessLate{w.hlate, w.hlate_n, nullptr}));
  AsmArgs<float> aa = make_asm_args<float>(mesh, w.hbuf32, val32, nullptr);
  return launch_assemble<float>(aa, s);
}

extern "C" {

int skg_snh_energy_x(const skg_tet_mesh* mesh, const double* x, double* energy_h, void* ws, void* stream) {
  return energy_xu(mesh, x, nullptr, energy_h, ws, stream);
}

int skg_snh_gradient_x(const skg_tet_mesh* mesh, const double* x, double* g, void* ws, void* stream) {
  return gradient_xu(mesh, x, nullptr, g, ws, stream);
}

int skg_snh_hessian_x(const skg_tet_mesh* mesh, const double* x, int precision, int psd, double* val64,
                      float* val32, void* ws, void* stream) {
  return hessian_xu(mesh, x, nullptr, precision, psd, val64, val32, ws, stream);
}

int skg_snh_energy_u(const skg_tet_mesh* mesh, const double* u, const double* Jx_bar, double* energy_h, void* ws,
                     void* stream) {
  if (!Jx_bar) return fail(SKG_ERR_ARG, "energy_u: Jx_bar is null");
  return energy_xu(mesh, u, Jx_bar, energy_h, ws, stream);
}

int skg_snh_gradient_u(const skg_tet_mesh* mesh, const double* u, const double* Jx_bar, double* g, void* ws,
                       void* stream) {
  if (!Jx_bar) return fail(SKG_ERR_ARG, "gradient_u: Jx_bar is null");
  return gradient_xu(mesh, u, Jx_bar, g, ws, stream);
}

int skg_snh_hessian_u(const skg_tet_mesh* mesh, const double* u, const double* Jx_bar, int precision, int psd,
                      double* val64, float* val32, void* ws, void* stream) {
  if (!Jx_bar) return fail(SKG_ERR_ARG, "hessian_u: Jx_bar is null");
  return hessian_xu(mesh, u, Jx_bar, precision, psd, val64, val32, ws, stream);
}

}  // extern "C"
