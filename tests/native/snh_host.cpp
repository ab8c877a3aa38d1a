// Host build of the device element math (simkit_gb300/csrc/snh_math.cuh).
// Test infrastructure: lets the CPU test suite compare the exact functions
// the kernels run against the FP64 oracle, without a GPU.
#include "../../simkit_gb300/csrc/snh_math.cuh"

using namespace skg;

template <typename R>
static void tet_hessian_batch(int64_t t, const double* F, const double* mu, const double* lam,
                              const double* vol, const double* gN, double* out, double fb, int mat = kMatSNH) {
  for (int64_t e = 0; e < t; ++e) {
    R f[9], g[12], o[kTetHessVals];
    for (int k = 0; k < 9; ++k) f[k] = R(F[9 * e + k]);
    for (int k = 0; k < 12; ++k) g[k] = R(gN[12 * e + k]);
    snh_tet_hessian<R>(f, R(mu[e]), R(lam[e]), R(vol[e]), g, o, R(fb), true, mat);
    for (int k = 0; k < kTetHessVals; ++k) out[kTetHessVals * e + k] = double(o[k]);
  }
}

template <typename R>
static void elem_batch(int64_t t, const double* F, const double* mu, const double* lam,
                       double* psi, double* dpsi, double* P, double* Pd, double* H) {
  for (int64_t e = 0; e < t; ++e) {
    R f[9], g[9], p[9], h[81];
    for (int k = 0; k < 9; ++k) { f[k] = R(F[9 * e + k]); g[k] = f[k] - ((k % 4 == 0) ? R(1) : R(0)); }
    // G computed from F here; callers that care pass F = I + G exactly representable
    psi[e] = double(snh_psi<R>(f, R(mu[e]), R(lam[e])));
    dpsi[e] = double(snh_dpsi<R>(g, R(mu[e]), R(lam[e])));
    snh_pk1<R>(f, R(mu[e]), R(lam[e]), p);
    for (int k = 0; k < 9; ++k) P[9 * e + k] = double(p[k]);
    snh_pk1_disp<R>(g, R(mu[e]), R(lam[e]), p);
    for (int k = 0; k < 9; ++k) Pd[9 * e + k] = double(p[k]);
    snh_hessian9<R>(f, R(mu[e]), R(lam[e]), h);
    for (int k = 0; k < 81; ++k) H[81 * e + k] = double(h[k]);
  }
}

template <typename R>
static void disp_batch(int64_t t, const double* G, const double* mu, const double* lam, double* dpsi, double* Pd) {
  for (int64_t e = 0; e < t; ++e) {
    R g[9], p[9];
    for (int k = 0; k < 9; ++k) g[k] = R(G[9 * e + k]);
    dpsi[e] = double(snh_dpsi<R>(g, R(mu[e]), R(lam[e])));
    snh_pk1_disp<R>(g, R(mu[e]), R(lam[e]), p);
    for (int k = 0; k < 9; ++k) Pd[9 * e + k] = double(p[k]);
  }
}

// any material: direct and displacement forms (3D), Hessian
template <typename R>
static void mat_batch(int mat, int64_t t, const double* F, const double* G, const double* mu, const double* lam,
                      double* psi, double* dpsi, double* P, double* Pd, double* H) {
  for (int64_t e = 0; e < t; ++e) {
    R f[9], g[9], p[9], h[81];
    for (int k = 0; k < 9; ++k) { f[k] = R(F[9 * e + k]); g[k] = R(G[9 * e + k]); }
    psi[e] = double(mat_psi<R>(mat, f, R(mu[e]), R(lam[e])));
    dpsi[e] = double(mat_dpsi<R>(mat, g, R(mu[e]), R(lam[e])));
    mat_pk1<R>(mat, f, R(mu[e]), R(lam[e]), p);
    for (int k = 0; k < 9; ++k) P[9 * e + k] = double(p[k]);
    mat_pk1_disp<R>(mat, g, R(mu[e]), R(lam[e]), p);
    for (int k = 0; k < 9; ++k) Pd[9 * e + k] = double(p[k]);
    elem_hessian<R, 3>(mat, f, R(mu[e]), R(lam[e]), h);
    for (int k = 0; k < 81; ++k) H[81 * e + k] = double(h[k]);
  }
}

// any material, 2D element tier
template <typename R>
static void mat_batch2(int mat, int64_t t, const double* F, const double* mu, const double* lam, double* psi,
                       double* P, double* H) {
  for (int64_t e = 0; e < t; ++e) {
    R f[4], p[4], h[16];
    for (int k = 0; k < 4; ++k) f[k] = R(F[4 * e + k]);
    psi[e] = double(elem_psi<R, 2>(mat, f, R(mu[e]), R(lam[e])));
    elem_pk1<R, 2>(mat, f, R(mu[e]), R(lam[e]), p);
    for (int k = 0; k < 4; ++k) P[4 * e + k] = double(p[k]);
    elem_hessian<R, 2>(mat, f, R(mu[e]), R(lam[e]), h);
    for (int k = 0; k < 16; ++k) H[16 * e + k] = double(h[k]);
  }
}

template <typename R>
static void svd_batch(int64_t t, const double* F, double* U, double* s, double* V) {
  for (int64_t e = 0; e < t; ++e) {
    R f[9], u[9], ss[3], v[9];
    for (int k = 0; k < 9; ++k) f[k] = R(F[9 * e + k]);
    svd3_rv<R>(f, u, ss, v);
    for (int k = 0; k < 9; ++k) { U[9 * e + k] = double(u[k]); V[9 * e + k] = double(v[k]); }
    for (int k = 0; k < 3; ++k) s[3 * e + k] = double(ss[k]);
  }
}

extern "C" {
void h_tet_hessian(int prec, int64_t t, const double* F, const double* mu, const double* lam, const double* vol,
                   const double* gN, double* out, double fallback_J) {
  if (prec == 64) tet_hessian_batch<double>(t, F, mu, lam, vol, gN, out, fallback_J);
  else tet_hessian_batch<float>(t, F, mu, lam, vol, gN, out, fallback_J);
}
void h_elem(int prec, int64_t t, const double* F, const double* mu, const double* lam, double* psi, double* dpsi,
            double* P, double* Pd, double* H) {
  if (prec == 64) elem_batch<double>(t, F, mu, lam, psi, dpsi, P, Pd, H);
  else elem_batch<float>(t, F, mu, lam, psi, dpsi, P, Pd, H);
}
void h_disp(int prec, int64_t t, const double* G, const double* mu, const double* lam, double* dpsi, double* Pd) {
  if (prec == 64) disp_batch<double>(t, G, mu, lam, dpsi, Pd);
  else disp_batch<float>(t, G, mu, lam, dpsi, Pd);
}
void h_tet_hessian_mat(int prec, int mat, int64_t t, const double* F, const double* mu, const double* lam,
                       const double* vol, const double* gN, double* out, double fallback_J) {
  if (prec == 64) tet_hessian_batch<double>(t, F, mu, lam, vol, gN, out, fallback_J, mat);
  else tet_hessian_batch<float>(t, F, mu, lam, vol, gN, out, fallback_J, mat);
}
void h_mm(int prec, int64_t t, const double* F, const double* G, const double* mu, const double* lam, double* psi,
          double* dpsi, double* P, double* Pd, double* H) {
  if (prec == 64) mat_batch<double>(kMatMMNH, t, F, G, mu, lam, psi, dpsi, P, Pd, H);
  else mat_batch<float>(kMatMMNH, t, F, G, mu, lam, psi, dpsi, P, Pd, H);
}
void h_mat(int prec, int mat, int64_t t, const double* F, const double* G, const double* mu, const double* lam,
           double* psi, double* dpsi, double* P, double* Pd, double* H) {
  if (prec == 64) mat_batch<double>(mat, t, F, G, mu, lam, psi, dpsi, P, Pd, H);
  else mat_batch<float>(mat, t, F, G, mu, lam, psi, dpsi, P, Pd, H);
}
void h_mat2(int prec, int mat, int64_t t, const double* F, const double* mu, const double* lam, double* psi,
            double* P, double* H) {
  if (prec == 64) mat_batch2<double>(mat, t, F, mu, lam, psi, P, H);
  else mat_batch2<float>(mat, t, F, mu, lam, psi, P, H);
}
void h_svd(int prec, int64_t t, const double* F, double* U, double* s, double* V) {
  if (prec == 64) svd_batch<double>(t, F, U, s, V);
  else svd_batch<float>(t, F, U, s, V);
}
double h_phi(double z) { return phi_log1p<double>(z); }
float h_phi_f(float z) { return phi_log1p<float>(z); }
}

// double-float stress of the mixed-precision force kernel (simkit_gb300/csrc/dfloat.cuh)
#include "../../simkit_gb300/csrc/dfloat.cuh"
extern "C" void h_pk1_disp_df(int mat, int64_t t, const double* G, const double* mu, const double* lam, double* P) {
  for (int64_t e = 0; e < t; ++e) {
    DF g[9], p[9];
    for (int k = 0; k < 9; ++k) g[k] = DF(G[9 * e + k]);
    if (mat == kMatMMNH) mmnh_pk1_disp<DF>(g, DF(mu[e]), DF(lam[e]), p);
    else snh_pk1_disp<DF>(g, DF(mu[e]), DF(lam[e]), p);
    for (int k = 0; k < 9; ++k) P[9 * e + k] = p[k].to_double();
  }
}
