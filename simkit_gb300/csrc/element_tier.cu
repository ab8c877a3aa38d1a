// Element tier of the stable neo-Hookean and Macklin-Mueller neo-Hookean energies over arbitrary F arrays,
// simkit's generic psd_project, per-tet rest-shape setup, the F = J x gather
// and the J^T P vertex gather.  Also the error plumbing of the C ABI.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "common.cuh"
#include "snh_math.cuh"

namespace skg {

static thread_local char g_err[1024] = "";

int fail(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return status;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  return fail(SKG_ERR_CUDA, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

// ------------------------------------------------------------ element F --
// MAT: kMatSNH (stable_neo_hookean.py), kMatMMNH (macklin_mueller_neo_hookean.py),
// kMatARAP (arap.py), kMatFCR (fcr.py) or kMatLE (linear_elasticity.py)
template <typename R, int D, int MAT>
__global__ void k_elem_energy(const double* __restrict__ F, const double* __restrict__ mu,
                              const double* __restrict__ lam, double* __restrict__ psi, int64_t t) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= t) return;
  R f[D * D];
#pragma unroll
  for (int k = 0; k < D * D; ++k) f[k] = R(F[D * D * e + k]);
  psi[e] = double(elem_psi<R, D>(MAT, f, R(mu[e]), R(lam[e])));
}

template <typename R, int D, int MAT>
__global__ void k_elem_pk1(const double* __restrict__ F, const double* __restrict__ mu,
                           const double* __restrict__ lam, double* __restrict__ P, int64_t t) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= t) return;
  R f[D * D], p[D * D];
#pragma unroll
  for (int k = 0; k < D * D; ++k) f[k] = R(F[D * D * e + k]);
  elem_pk1<R, D>(MAT, f, R(mu[e]), R(lam[e]), p);
#pragma unroll
  for (int k = 0; k < D * D; ++k) P[D * D * e + k] = double(p[k]);
}

template <typename R, int D, int MAT>
__global__ void k_elem_hessian(const double* __restrict__ F, const double* __restrict__ mu,
                               const double* __restrict__ lam, double* __restrict__ H, int64_t t) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= t) return;
  R f[D * D], h[D * D * D * D];
#pragma unroll
  for (int k = 0; k < D * D; ++k) f[k] = R(F[D * D * e + k]);
  elem_hessian<R, D>(MAT, f, R(mu[e]), R(lam[e]), h);
  for (int k = 0; k < D * D * D * D; ++k) H[(int64_t)D * D * D * D * e + k] = double(h[k]);
}

typedef void (*ElemKernel)(const double*, const double*, const double*, double*, int64_t);

static int launch_elem(int dim, int precision, const double* F, const double* mu, const double* lam, double* out,
                       int64_t t, void* stream, ElemKernel k33, ElemKernel k32, ElemKernel k23, ElemKernel k22) {
  if (dim != 2 && dim != 3) return fail(SKG_ERR_ARG, "the element tier supports dim=2 or dim=3");
  if (t < 0) return fail(SKG_ERR_ARG, "negative element count");
  if (t == 0) return SKG_OK;
  auto kern = dim == 3 ? (precision == SKG_FP64 ? k33 : k32) : (precision == SKG_FP64 ? k23 : k22);
  kern<<<blocks_for(t, 128), 128, 0, as_stream(stream)>>>(F, mu, lam, out, t);
  SKG_LAUNCHED();
  return SKG_OK;
}

// --------------------------------------------------------- psd_project ---
// Cyclic Jacobi on one d x d symmetric block per thread (d <= 12), then
// eigenvalue floor (method 0: max(s, 1e-6), simkit/psd_project.py:37) or
// magnitude (method 1, :35), then U diag(s) U^T (:46).
template <int DMAX>
__global__ void k_psd_project(const double* __restrict__ H, double* __restrict__ out, int64_t n, int d,
                              int method) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  double A[DMAX * DMAX], V[DMAX * DMAX];
  const double* h = H + (int64_t)d * d * e;
  double scale = 0.0;
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      A[i * DMAX + j] = 0.5 * (h[i * d + j] + h[j * d + i]);
      V[i * DMAX + j] = (i == j) ? 1.0 : 0.0;
      scale += fabs(A[i * DMAX + j]);
    }
  for (int sweep = 0; sweep < 40; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < d; ++p)
      for (int q = p + 1; q < d; ++q) off += fabs(A[p * DMAX + q]);
    if (!(off > 1e-17 * scale)) break;
    for (int p = 0; p < d; ++p)
      for (int q = p + 1; q < d; ++q) {
        const double apq = A[p * DMAX + q];
        if (apq == 0.0) continue;
        const double theta = (A[q * DMAX + q] - A[p * DMAX + p]) / (2.0 * apq);
        const double at = fabs(theta);
        double tt = at > 1e150 ? 0.5 / theta : 1.0 / (at + sqrt(at * at + 1.0));
        if (theta < 0.0 && at <= 1e150) tt = -tt;
        const double c = 1.0 / sqrt(tt * tt + 1.0), s = tt * c;
        for (int r = 0; r < d; ++r) {  // A <- A J (columns p, q)
          const double arp = A[r * DMAX + p], arq = A[r * DMAX + q];
          A[r * DMAX + p] = c * arp - s * arq;
          A[r * DMAX + q] = s * arp + c * arq;
        }
        for (int r = 0; r < d; ++r) {  // A <- J^T A (rows p, q)
          const double apr = A[p * DMAX + r], aqr = A[q * DMAX + r];
          A[p * DMAX + r] = c * apr - s * aqr;
          A[q * DMAX + r] = s * apr + c * aqr;
        }
        A[p * DMAX + q] = A[q * DMAX + p] = 0.0;
        for (int r = 0; r < d; ++r) {
          const double vp = V[r * DMAX + p], vq = V[r * DMAX + q];
          V[r * DMAX + p] = c * vp - s * vq;
          V[r * DMAX + q] = s * vp + c * vq;
        }
      }
  }
  double s[DMAX];
  for (int k = 0; k < d; ++k) {
    double v = A[k * DMAX + k];
    s[k] = method == 1 ? fabs(v) : (v < kPsdFloor ? kPsdFloor : v);
  }
  double* o = out + (int64_t)d * d * e;
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      double acc = 0.0;
      for (int k = 0; k < d; ++k) acc += V[i * DMAX + k] * s[k] * V[j * DMAX + k];
      o[i * d + j] = acc;
    }
}

// ------------------------------------------------------------- tet setup --
__global__ void k_tet_setup(const double* __restrict__ X, const int4* __restrict__ T, int64_t n, int64_t t,
                            double* __restrict__ dinv, double* __restrict__ vol) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= t) return;
  const int4 v = T[e];
  // a vertex index outside [0, n) is not read: the tet gets NaN volume and shape operator
  const auto out = [n](int i) { return i < 0 || (int64_t)i >= n; };
  if (out(v.x) || out(v.y) || out(v.z) || out(v.w)) {
#pragma unroll
    for (int k = 0; k < 9; ++k) dinv[k * t + e] = nan("");
    vol[e] = nan("");
    return;
  }
  const double* x0 = X + 3 * (int64_t)v.x;
  double E[9];  // columns: X1 - X0, X2 - X0, X3 - X0
  const int vv[3] = {v.y, v.z, v.w};
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int i = 0; i < 3; ++i) E[3 * i + c] = X[3 * (int64_t)vv[c] + i] - x0[i];
  const double det = det3(E);
  double C[9];
  cof3(E, C);
  // E^-1 = cof(E)^T / det
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) dinv[(3 * i + j) * t + e] = C[3 * j + i] / det;
  vol[e] = det / 6.0;
}

// F = sum_a x_a (x) gN_a from absolute positions (simkit's J @ x)
__global__ void k_tet_F(const int4* __restrict__ T, const double* __restrict__ dinv, const double* __restrict__ x,
                        int64_t t, double* __restrict__ F) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= t) return;
  const int4 v = T[e];
  double Dv[9], du[9], G[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Dv[k] = dinv[k * t + e];
  const int vv[3] = {v.y, v.z, v.w};
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int i = 0; i < 3; ++i) du[3 * a + i] = x[3 * (int64_t)vv[a] + i] - x[3 * (int64_t)v.x + i];
  disp_grad(du, Dv, G);
#pragma unroll
  for (int k = 0; k < 9; ++k) F[9 * e + k] = G[k];
}

// y = J^T vec(P): per vertex, sum over incident (tet, corner) in list order
__global__ void k_tet_scatter(const double* __restrict__ dinv, const double* __restrict__ P,
                              const int32_t* __restrict__ v2t_ptr, const int32_t* __restrict__ v2t, int64_t n,
                              int64_t t, double* __restrict__ y) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= n) return;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int k = v2t_ptr[v]; k < v2t_ptr[v + 1]; ++k) {
    const int code = v2t[k];
    const int64_t e = code >> 2;
    const int a = code & 3;
    double g[3];
    if (a == 0) {
#pragma unroll
      for (int j = 0; j < 3; ++j) g[j] = -(dinv[j * t + e] + dinv[(3 + j) * t + e] + dinv[(6 + j) * t + e]);
    } else {
#pragma unroll
      for (int j = 0; j < 3; ++j) g[j] = dinv[(3 * (a - 1) + j) * t + e];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
      acc[i] += P[9 * e + 3 * i] * g[0] + P[9 * e + 3 * i + 1] * g[1] + P[9 * e + 3 * i + 2] * g[2];
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) y[3 * v + i] = acc[i];
}

}  // namespace skg

using namespace skg;

extern "C" {

int skg_version(void) { return 100; }

int skg_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return SKG_ERR_ARG;
  strncpy(buf, g_err, len - 1);
  buf[len - 1] = '\0';
  return SKG_OK;
}

#define SKG_ELEM(kern, M) kern<double, 3, M>, kern<float, 3, M>, kern<double, 2, M>, kern<float, 2, M>

int skg_snh_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                             double* psi, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, psi, t, stream, SKG_ELEM(k_elem_energy, kMatSNH));
}

int skg_snh_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                               double* P, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, P, t, stream, SKG_ELEM(k_elem_pk1, kMatSNH));
}

int skg_snh_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* H, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, H, t, stream, SKG_ELEM(k_elem_hessian, kMatSNH));
}

int skg_mmnh_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* psi, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, psi, t, stream, SKG_ELEM(k_elem_energy, kMatMMNH));
}

int skg_mmnh_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                                double* P, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, P, t, stream, SKG_ELEM(k_elem_pk1, kMatMMNH));
}

int skg_mmnh_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                               double* H, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, H, t, stream, SKG_ELEM(k_elem_hessian, kMatMMNH));
}

int skg_arap_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* psi, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, psi, t, stream, SKG_ELEM(k_elem_energy, kMatARAP));
}

int skg_arap_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                                double* P, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, P, t, stream, SKG_ELEM(k_elem_pk1, kMatARAP));
}

int skg_arap_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                               double* H, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, H, t, stream, SKG_ELEM(k_elem_hessian, kMatARAP));
}

int skg_fcr_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                             double* psi, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, psi, t, stream, SKG_ELEM(k_elem_energy, kMatFCR));
}

int skg_fcr_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                               double* P, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, P, t, stream, SKG_ELEM(k_elem_pk1, kMatFCR));
}

int skg_fcr_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* H, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, H, t, stream, SKG_ELEM(k_elem_hessian, kMatFCR));
}

int skg_le_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                            double* psi, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, psi, t, stream, SKG_ELEM(k_elem_energy, kMatLE));
}

int skg_le_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* P, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, P, t, stream, SKG_ELEM(k_elem_pk1, kMatLE));
}

int skg_le_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                             double* H, int64_t t, void* stream) {
  return launch_elem(dim, precision, F, mu, lam, H, t, stream, SKG_ELEM(k_elem_hessian, kMatLE));
}
#undef SKG_ELEM

int skg_psd_project(const double* H, double* out, int64_t n, int d, int method, void* stream) {
  if (d < 1 || d > 12) return fail(SKG_ERR_ARG, "psd_project supports block sizes 1..12, got %d", d);
  if (method != 0 && method != 1) return fail(SKG_ERR_ARG, "psd_project method must be 'proj' or 'abs'");
  if (n <= 0) return SKG_OK;
  if (d <= 4)
    k_psd_project<4><<<blocks_for(n, 64), 64, 0, as_stream(stream)>>>(H, out, n, d, method);
  else if (d <= 9)
    k_psd_project<9><<<blocks_for(n, 64), 64, 0, as_stream(stream)>>>(H, out, n, d, method);
  else
    k_psd_project<12><<<blocks_for(n, 64), 64, 0, as_stream(stream)>>>(H, out, n, d, method);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_tet_setup(const double* X, const int32_t* T, int64_t n, int64_t t, double* dinv, double* vol, void* stream) {
  if (n <= 0 || t < 0) return fail(SKG_ERR_ARG, "bad mesh sizes n=%lld t=%lld", (long long)n, (long long)t);
  if (t == 0) return SKG_OK;
  k_tet_setup<<<blocks_for(t), kBlock, 0, as_stream(stream)>>>(X, reinterpret_cast<const int4*>(T), n, t, dinv, vol);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_tet_deformation_gradient(const int32_t* T, const double* dinv, const double* x, int64_t t, double* F,
                                 void* stream) {
  if (t <= 0) return t == 0 ? SKG_OK : fail(SKG_ERR_ARG, "negative tet count");
  k_tet_F<<<blocks_for(t), kBlock, 0, as_stream(stream)>>>(reinterpret_cast<const int4*>(T), dinv, x, t, F);
  SKG_LAUNCHED();
  return SKG_OK;
}

int skg_tet_gradient_scatter(const int32_t* T, const double* dinv, const double* P, const int32_t* v2t_ptr,
                             const int32_t* v2t, int64_t n, int64_t t, double* y, void* stream) {
  (void)T;
  if (n <= 0) return SKG_OK;
  k_tet_scatter<<<blocks_for(n), kBlock, 0, as_stream(stream)>>>(dinv, P, v2t_ptr, v2t, n, t, y);
  SKG_LAUNCHED();
  return SKG_OK;
}

}  // extern "C"
