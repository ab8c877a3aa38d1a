// Kernel argument bundles and launchers shared by the assembled tier and the
// Newton solver.
#pragma once
#include <cuda_fp16.h>

#include "common.cuh"

namespace skg {

constexpr int kHStride = 80;     // per-tet Hessian record: 78 values + 2 pad
constexpr int kMaxGrid = 2048;   // upper bound on grid-stride reduction grids

inline int reduce_blocks(int64_t n) {
  int64_t b = (n + kBlock - 1) / kBlock;
  if (b > kReduceBlocks) b = kReduceBlocks;
  return (int)(b < 1 ? 1 : b);
}

template <typename R> struct TetArgs {
  int64_t t;
  const int4* tets;
  const R* dinv;
  const R* vol;
  const R* mu;
  const R* lam;
  const double* u;   // FP64 displacement (or positions), 3n
  const float* uh;   // FP32 hi/lo split (FP32 kernels only)
  const float* ul;
  const int32_t* tet_inst;     // optional: instance of each tet (batched solves)
  const uint8_t* inst_active;  // optional: skip tets of inactive instances
  const double* fbar;          // optional: per-tet F offset, 9 row-major values per tet:
                               // F = (J u) + fbar, simkit's _u tier with fbar = J x_bar
  int material;                // kMatSNH, kMatMMNH, kMatARAP or kMatFCR
};

template <typename R>
__device__ __forceinline__ void add_fbar(const TetArgs<R>& a, int64_t e, R* G) {
  if (a.fbar) {
#pragma unroll
    for (int k = 0; k < 9; ++k) G[k] += R(a.fbar[9 * e + k]);
  }
}

// Contact springs against up to SKG_MAX_PLANES planes (simkit/energies/contact_springs_plane.py):
// vertex v at x = X + u with d = (x - p) . n < 0 adds k w d^2 / 2, w = mass[v] or 1.
struct Contact {
  int n = 0;
  const double* X = nullptr;      // rest positions (3n)
  const double* w = nullptr;      // per-vertex weights (lumped masses) or null for 1
  double p[SKG_MAX_PLANES][3];
  double nrm[SKG_MAX_PLANES][3];
  double k[SKG_MAX_PLANES];
};

// energy, gradient and Hessian (3x3, row-major) of the contact springs at vertex v, position x
__device__ __forceinline__ double contact_terms(const Contact& c, int64_t v, const double* x, double* g,
                                                double* h) {
  double e = 0.0;
  const double w = c.w ? c.w[v] : 1.0;
  for (int q = 0; q < c.n; ++q) {
    const double d = (x[0] - c.p[q][0]) * c.nrm[q][0] + (x[1] - c.p[q][1]) * c.nrm[q][1] +
                     (x[2] - c.p[q][2]) * c.nrm[q][2];
    if (!(d < 0.0)) continue;
    const double kw = c.k[q] * w;
    e += 0.5 * kw * d * d;
    if (g)
      for (int i = 0; i < 3; ++i) g[i] += kw * d * c.nrm[q][i];
    if (h)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) h[3 * i + j] += kw * c.nrm[q][i] * c.nrm[q][j];
  }
  return e;
}

template <typename R> struct AsmArgs {
  int64_t nb;
  const int32_t* bsr_row;
  const int32_t* bsr_col;
  const int32_t* rowptr;
  const int32_t* hc_ptr;
  const int32_t* hc_src;
  const R* hbuf;
  const double* mass;    // optional: adds mass/h^2 on diagonal blocks
  double inv_h2;
  const uint8_t* pinned; // optional: 3n DOF mask
  R* val;                // entry-major block values (9 nb), or null
  R* rec;                // 12-wide block records (9 values, column bits, 2 pad), or null
  R* jinv;               // optional: block-Jacobi inverses (9n)
  const int32_t* vert_inst;    // optional: instance of each block row (batched solves)
  const uint8_t* inst_active;  // optional: skip rows of inactive instances
  Contact contact;             // contact springs on diagonal blocks (positions from u)
  const double* u;             // displacement (needed with contact)
  const float4* cmode;         // optional: two-level coarse data per vertex, packed into record slots 10-11
  const uint32_t* colpack;     // optional (cluster PCG): the column's 32-bit coarse word into record slot 11
  // optional: the upper-triangle lists (symmetric assembly: each block summed once, its transpose
  // written into the mirror slot)
  int64_t n_up;
  const int32_t* up_slot;
  const int32_t* up_mirror;
  const int32_t* hcu_ptr;
  const int32_t* hcu_src;
};

// A column's two-level coarse data in the two spare record slots (64 bits):
// fp16 d_x | fp16 d_y << 16,  fp16 d_z | aggregate << 16 (13 bits) | free mask << 29.
// The host rounds d to fp16 precision, so the packing is exact and every user
// of d (coarse operator, restriction, prolongation) sees the same values.
__device__ __forceinline__ uint2 coarse_pack(float4 m) {
  const unsigned bits = __float_as_uint(m.w);
  const unsigned hx = __half_as_ushort(__float2half_rn(m.x));
  const unsigned hy = __half_as_ushort(__float2half_rn(m.y));
  const unsigned hz = __half_as_ushort(__float2half_rn(m.z));
  return make_uint2(hx | (hy << 16), hz | ((bits & 0x1fffu) << 16) | ((bits >> 29) << 29));
}
__device__ __forceinline__ void rec_aux_store(float* r, uint2 a) {
  r[10] = __uint_as_float(a.x);
  r[11] = __uint_as_float(a.y);
}
__device__ __forceinline__ void rec_aux_store(double* r, uint2 a) {
  r[10] = __longlong_as_double((long long)(((unsigned long long)a.y << 32) | a.x));
  r[11] = 0.0;
}
__device__ __forceinline__ void rec_word_store(float* r, uint32_t w) { r[11] = __uint_as_float(w); }
__device__ __forceinline__ void rec_word_store(double* r, uint32_t w) { r[11] = __longlong_as_double((long long)w); }

// Block record of the solver's SpMV: the 9 row-major entries of a 3x3 block,
// the block column stored in the bits of entry 9, entries 10-11 zero, so one
// block is three 16-byte loads (FP32) instead of ten scalar loads.
constexpr int kRec = 12;
__device__ __forceinline__ float col_bits(int c, float) { return __int_as_float(c); }
__device__ __forceinline__ double col_bits(int c, double) { return __longlong_as_double((long long)c); }
__device__ __forceinline__ int bits_col(float v) { return __float_as_int(v); }
__device__ __forceinline__ int bits_col(double v) { return (int)__double_as_longlong(v); }

struct GradArgs {
  int64_t n;
  const int32_t* v2t_ptr;
  const int32_t* v2t;
  const double* fbuf;
  const double* mass;   // optional backward-Euler terms
  double inv_h2;
  const double* u;
  const double* ut;
  const double* f_ext;
  const uint8_t* pinned;
  double* g;
  double* partials;
  unsigned* counter;
  double* out;          // out[0] = ||g||^2
  Contact contact;
};

template <typename R> struct EnergyArgs {
  TetArgs<R> tet;
  int64_t n;
  const R* dx;          // optional padded step direction
  double step;
  const double* mass;
  double inv_h2;
  const double* ut;
  const double* f_ext;
  const uint8_t* pinned;
  double* partials;
  unsigned* counter;
  double* out;          // out[0] = energy, out[1] = magnitude
  Contact contact;
  const double* step_dev = nullptr;   // when set, the step is read here (device-decided line search)
};

struct Workspace {
  float* hbuf32;
  double* hbuf64;
  double* fbuf;
  float* val32;
  double* val64;
  float* rec32;      // solver block records (kRec per block)
  double* rec64;
  float* jinv32;
  double* jinv64;
  double* g;
  double* ut;
  float* uh;
  float* ul;
  float* dinv_lo;    // mixed: low parts of Dinv for the double-float forces (9 t)
  int32_t* hlate;    // mixed: tets whose Hessian takes the FP64-SVD kernel (t)
  unsigned* hlate_n; // their count
  float* vec32[6];   // PCG x, r, z, p, q, s (padded)
  double* vec64[6];
  double* partials;
  unsigned* counter;
  double* scal;
  // two-level preconditioner (only with mesh->coarse)
  float* cM;                 // np x np coarse operator / its inverse
  float* crowp;              // 2 x 32 x np row panels
  unsigned long long* crc;   // np fixed-point coarse residual
  unsigned long long* crq;   // 2 np fixed-point P^T q (two-barrier PCG), by iteration parity
  double* crcg;              // 2 np coarse residual kept between iterations (two-barrier PCG)
  float* ce;                 // 8 per aggregate: coarse correction
  int* cok;                  // coarse inverse valid
  unsigned* cbar;            // grid barrier of the inversion
  int64_t bytes;
};

// coarse unknowns padded to the Gauss-Jordan block (32); the largest instance in the per-instance form
inline int64_t coarse_padded(const skg_tet_mesh* m) {
  if (!m->coarse) return 0;
  if (m->coarse->inst_agg) return m->coarse->max_np;
  return ((6 * (int64_t)m->coarse->n_agg + 31) / 32) * 32;
}
constexpr int kCoarseInvCtas = 456;   // CTAs of the per-instance coarse inversion (3 per SM on 152 SMs)
// (its row-panel scratch is sized per CTA, which covers one panel pair per cluster of CTAs)

Workspace carve_workspace(const skg_tet_mesh* m, int precision, void* base);
int check_mesh(const skg_tet_mesh* m, int precision);
TetArgs<double> make_tet_args64(const skg_tet_mesh* m, const double* u);
TetArgs<float> make_tet_args32(const skg_tet_mesh* m, const double* u, const float* uh, const float* ul);

template <typename R>
inline AsmArgs<R> make_asm_args(const skg_tet_mesh* m, const R* hbuf, R* val, R* jinv) {
  AsmArgs<R> a{};
  a.nb = m->n_blocks;
  a.bsr_row = m->bsr_row;
  a.bsr_col = m->bsr_col;
  a.rowptr = m->bsr_rowptr;
  a.hc_ptr = m->hc_ptr;
  a.hc_src = m->hc_src;
  if (m->up_slot && m->up_mirror && m->hcu_ptr && m->hcu_src) {
    a.n_up = m->n_upper;
    a.up_slot = m->up_slot;
    a.up_mirror = m->up_mirror;
    a.hcu_ptr = m->hcu_ptr;
    a.hcu_src = m->hcu_src;
  }
  a.hbuf = hbuf;
  a.val = val;
  a.jinv = jinv;
  return a;
}

// optional FP32 split of the Hessian kernel: the list (t entries) and counter for the nearly inverted
// tets, and where to return the number of kernels launched (1 or 2)
struct HessLate {
  int32_t* list = nullptr;
  unsigned* n = nullptr;
  int* launches = nullptr;
};
template <typename R>
int launch_tet_hessian(const TetArgs<R>& a, int disp, int project, R* hbuf, cudaStream_t s, HessLate late = {});
template <typename R> int launch_assemble(const AsmArgs<R>& a, cudaStream_t s);
int launch_forces(const TetArgs<double>& a, int disp, double* fbuf, cudaStream_t s);
// double-float forces (mixed precision, neo-Hookean materials, displacement form); fbuf holds
// 12 (hi, lo) float pairs per tet, summed by launch_vertex_gradient(..., df = true)
int launch_forces_df(const TetArgs<double>& a, const float* dinv32, const float* dinv_lo, const float* uh,
                     const float* ul, double* fbuf, cudaStream_t s);
int launch_dinv_lo(const skg_tet_mesh* m, float* lo, cudaStream_t s);
int launch_vertex_gradient(const GradArgs& a, cudaStream_t s, bool df = false);
template <typename R> int launch_energy(const EnergyArgs<R>& a, bool direct, cudaStream_t s);
int launch_split(const double* u, int64_t n, float* uh, float* ul, cudaStream_t s);
template <typename R>
int launch_inst_energy(const EnergyArgs<R>& a, int n_inst, const int32_t* inst_rows, const int32_t* inst_tets,
                       const uint8_t* mask, const double* steps, double* out2, cudaStream_t s);

}  // namespace skg
