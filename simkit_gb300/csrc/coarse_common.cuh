// Types and per-vertex helpers of the two-level preconditioner shared by the
// grid PCG (coarse.cuh) and the thread-block-cluster PCG (pcg_cluster.cuh).
#pragma once

namespace skg {

constexpr int kCoarseMax = 4096;   // coarse unknowns the PCG stages in shared memory
constexpr int kGjB = 32;           // Gauss-Jordan pivot block
constexpr int kGjCols = 256;       // columns per Gauss-Jordan work unit (one per thread)
constexpr double kCoarseShift = 1e-5;  // diagonal shift relative to the aggregate's largest diagonal
constexpr int kCoarseInstMax = 768;    // per-instance coarse unknowns of the cluster PCG (127 aggregates)
constexpr int kCoarseSmem = 2 * kCoarseInstMax * 4;   // cluster PCG: e and P^T r of the instance per CTA

struct CoarseDev {
  int n_agg;                   // aggregates
  int nc;                      // coarse unknowns, 6 n_agg
  int np;                      // nc padded to a multiple of kGjB (identity in the padding)
  int n_cb;                    // nonzero 6x6 coarse blocks
  const float4* mode;          // (n): d_v (x, y, z); w bits: aggregate | free mask << 29
  const int32_t* cb_ptr;       // (n_cb + 1)
  const int32_t* cb_slot;      // fine block slots grouped by coarse block
  const int32_t* cb_rc;        // (2 n_cb) aggregate row, column
  const int32_t* bsr_row;      // block row of each fine slot
  float* M;                    // np x np: A_c, inverted in place
  float* rowp;                 // 2 x kGjB x np row panels
  unsigned long long* rc;      // np: coarse residual in fixed point
  unsigned long long* rq;      // 2 np: P^T q in fixed point by iteration parity (two-barrier whole-mesh PCG)
  double* rcg;                 // 2 np: the coarse residual carried between iterations (two-barrier PCG)
  float* e;                    // 8 n_agg: (t, w) per aggregate, padded to 8
  int* ok;                     // 1 when M holds a valid inverse (per instance in the per-instance form)
  unsigned* bar;               // 2: grid barrier of the inversion
  // per-instance form (cluster PCG); inst_agg == nullptr in the whole-mesh form
  int n_inst;
  int max_np;
  const int32_t* inst_agg;     // (n_inst + 1) first aggregate of each instance
  const int32_t* agg_inst;     // (n_agg) instance of each aggregate
  const int64_t* inst_moff;    // (n_inst + 1) dense block offsets (floats)
  const uint32_t* colpack;     // (n) packed column word of each vertex
  int64_t m_floats;            // dense coarse storage (np^2, or the per-instance sum)
};

__device__ __forceinline__ int mode_agg(float4 m) { return (int)(__float_as_uint(m.w) & 0x1fffffffu); }
__device__ __forceinline__ unsigned mode_mask(float4 m) { return __float_as_uint(m.w) >> 29; }

// (P e) at a vertex with scaled offset d, aggregate a and free mask f, for the
// coarse correction e of the current iteration (plain loads: e is written
// earlier in the same kernel)
__device__ __forceinline__ Vec3<float> prolong_at(const float* e, float dx, float dy, float dz, int a, unsigned f) {
  const float4 e0 = reinterpret_cast<const float4*>(e)[2 * a];
  const float4 e1 = reinterpret_cast<const float4*>(e)[2 * a + 1];
  // t = (e0.x, e0.y, e0.z), w = (e0.w, e1.x, e1.y): t + w x d
  const float px = e0.x + (e1.x * dz - e1.y * dy);
  const float py = e0.y + (e1.y * dx - e0.w * dz);
  const float pz = e0.z + (e0.w * dy - e1.x * dx);
  return {(f & 1u) ? px : 0.f, (f & 2u) ? py : 0.f, (f & 4u) ? pz : 0.f};
}
// ... from the per-vertex mode array
__device__ __forceinline__ Vec3<float> prolong(const CoarseDev& c, int64_t v) {
  const float4 m = __ldg(c.mode + v);
  return prolong_at(c.e, m.x, m.y, m.z, mode_agg(m), mode_mask(m));
}
// ... from the column data packed into a block record (same values: d is fp16-exact)
__device__ __forceinline__ Vec3<float> prolong_rec(const float* e, unsigned a0, unsigned a1) {
  const float dx = __half2float(__ushort_as_half((unsigned short)(a0 & 0xffffu)));
  const float dy = __half2float(__ushort_as_half((unsigned short)(a0 >> 16)));
  const float dz = __half2float(__ushort_as_half((unsigned short)(a1 & 0xffffu)));
  return prolong_at(e, dx, dy, dz, (int)((a1 >> 16) & 0x1fffu), a1 >> 29);
}

// ... from the 32-bit column word of the per-instance form (offset k/64, local
// aggregate, free mask); e: the instance's coarse correction, 6 per aggregate
__device__ __forceinline__ Vec3<float> prolong_word(const float* e, uint32_t w) {
  const float dx = float((int)(w & 127u) - 64) * (1.f / 64.f);
  const float dy = float((int)((w >> 7) & 127u) - 64) * (1.f / 64.f);
  const float dz = float((int)((w >> 14) & 127u) - 64) * (1.f / 64.f);
  const float* ea = e + 6 * ((w >> 21) & 127u);
  const unsigned f = w >> 28;
  const float px = ea[0] + (ea[4] * dz - ea[5] * dy);
  const float py = ea[1] + (ea[5] * dx - ea[3] * dz);
  const float pz = ea[2] + (ea[3] * dy - ea[4] * dx);
  return {(f & 1u) ? px : 0.f, (f & 2u) ? py : 0.f, (f & 4u) ? pz : 0.f};
}

// Fixed-point scale of an iteration's coarse residual: a power of two putting
// 64 ||r|| at 2^50 (|P^T r| of an aggregate is far below 2^12 ||r||, so sums
// stay inside 64 bits with room for a residual that grows between iterations)
__device__ __forceinline__ float coarse_scale(double rr) {
  int ex;
  frexp(64.0 * sqrt(fmax(rr, 1e-300)), &ex);
  return ldexpf(1.f, max(-126, min(127, 50 - ex)));
}

// c.rc += P^T r over the calling warp's rows (every lane calls; consecutive
// rows of one aggregate are summed first by a segmented shuffle reduction, then
// one 64-bit atomic per segment and component: integer sums do not depend on
// the order of the atomics)
__device__ __forceinline__ void coarse_restrict(const CoarseDev& c, bool valid, int64_t row, float rx, float ry,
                                                float rz, float scale) {
  int key = -1;
  long long q[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) q[k] = 0;
  if (valid) {
    const float4 m = __ldg(c.mode + row);
    key = mode_agg(m);
    const unsigned f = mode_mask(m);
    const float x = (f & 1u) ? rx : 0.f, y = (f & 2u) ? ry : 0.f, z = (f & 4u) ? rz : 0.f;
    // P_v^T r = (r, d x r)
    const float v6[6] = {x, y, z, m.y * z - m.z * y, m.z * x - m.x * z, m.x * y - m.y * x};
#pragma unroll
    for (int k = 0; k < 6; ++k) q[k] = __float2ll_rn(v6[k] * scale);   // power-of-two scale: exact
  }
  const int lane = threadIdx.x & 31;
  const int prev = __shfl_up_sync(0xffffffffu, key, 1);
  const bool head = lane == 0 || prev != key;
  const unsigned heads = __ballot_sync(0xffffffffu, head);
  const int seg = __popc(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int so = __shfl_down_sync(0xffffffffu, seg, o);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const long long t = __shfl_down_sync(0xffffffffu, q[k], o);
      if (lane + o < 32 && so == seg) q[k] += t;
    }
  }
  if (head && key >= 0)
#pragma unroll
    for (int k = 0; k < 6; ++k) atomicAdd(c.rc + 6 * key + k, (unsigned long long)q[k]);
}

// dst += P^T y over the rows of the calling warp's lane groups (G lanes per block row, every lane
// of a group holding its row's y, as the SpMV leaves it): the first lane of each group contributes
// its row, runs of rows of one aggregate are summed by a segmented shuffle reduction over those
// lanes, then one 64-bit atomic per run and component.  The scaled values must stay within 2^52
// so that the sums of up to 2^10 rows of an aggregate cannot overflow; a value outside that range
// (or not finite) is left out and the return value is true, and the caller then does not use dst.
template <int G>
__device__ __forceinline__ bool coarse_restrict_groups(const CoarseDev& c, unsigned long long* dst, bool valid,
                                                      int64_t row, float yx, float yy, float yz, float scale) {
  const int lane = threadIdx.x & 31;
  const bool leader = (lane & (G - 1)) == 0;
  int key = -1;
  bool bad = false;
  long long q[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) q[k] = 0;
  if (valid) {
    const float4 m = __ldg(c.mode + row);
    key = mode_agg(m);
    if (leader) {
      const unsigned f = mode_mask(m);
      const float x = (f & 1u) ? yx : 0.f, y = (f & 2u) ? yy : 0.f, z = (f & 4u) ? yz : 0.f;
      const float v6[6] = {x, y, z, m.y * z - m.z * y, m.z * x - m.x * z, m.x * y - m.y * x};
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const float t = v6[k] * scale;   // power-of-two scale: exact
        if (fabsf(t) <= 0x1p52f) q[k] = __float2ll_rn(t);
        else bad = true;
      }
    }
  }
  const int prev = __shfl_up_sync(0xffffffffu, key, G);
  const bool head = leader && (lane == 0 || prev != key);
  const unsigned heads = __ballot_sync(0xffffffffu, head);
  const int seg = __popc(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
  for (int o = G; o < 32; o <<= 1) {
    const int so = __shfl_down_sync(0xffffffffu, seg, o);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const long long t = __shfl_down_sync(0xffffffffu, q[k], o);
      if (lane + o < 32 && so == seg) q[k] += t;
    }
  }
  if (head && key >= 0)
#pragma unroll
    for (int k = 0; k < 6; ++k) atomicAdd(dst + 6 * key + k, (unsigned long long)q[k]);
  return bad;
}

}  // namespace skg
