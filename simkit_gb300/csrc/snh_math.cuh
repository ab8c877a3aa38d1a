// Element math shared by every kernel of the FEM path: the stable neo-Hookean
// energy and the Macklin-Mueller neo-Hookean energy (same I_C / J Hessian form).
//
// All routines are plain functions of registers, compiled for the device by
// nvcc and for the host by g++ (the host build is what the CPU unit tests
// exercise against the FP64 oracle).  Storage conventions:
//   * F, G, P, U, V: 3x3 row-major, a[3*i + j] = M_ij.
//   * F = I + G, where G is the displacement gradient.
//   * gN[3*a + j] = d N_a / d X_j, the rest-shape gradient of barycentric
//     coordinate a (a = 0..3), so that F_ij = sum_a x_{a,i} gN[a][j].
//
// Energy density (simkit/energies/stable_neo_hookean.py:65-129):
//   psi = mu/2 (I_C - 3) - mu/2 log(I_C + 1) + lam/2 (J - alpha)^2,
//   alpha = 1 + 3 mu / (4 lam).
// PK1 (:132-218): P = A F + D cof F, A = mu I_C/(I_C+1), D = lam (J - alpha).
// F-Hessian (:221-443): A I + B f f^T + lam c c^T + D d2J/dF2, B = 2 mu/(I_C+1)^2.
//
// The displacement forms below rewrite psi - psi(I) and P so that the terms
// that cancel at rest (A + D = 0 at F = I) are combined symbolically; in
// FP32 this keeps relative accuracy near rest where the direct forms lose
// digits to cancellation.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SK_HD __host__ __device__ __forceinline__
#else
#define SK_HD inline
#endif

namespace skg {

template <typename R> SK_HD R sk_sqrt(R x) { return sqrt(x); }
template <typename R> SK_HD R sk_abs(R x) { return x < R(0) ? -x : x; }
template <typename R> SK_HD R sk_log1p(R x) { return log1p(x); }
template <typename R> SK_HD R sk_log(R x) { return log(x); }
template <typename R> SK_HD R sk_max(R a, R b) { return a > b ? a : b; }
template <typename R> SK_HD R sk_min(R a, R b) { return a < b ? a : b; }
#if defined(__CUDACC__)
template <> SK_HD float sk_sqrt<float>(float x) { return sqrtf(x); }
template <> SK_HD float sk_log1p<float>(float x) { return log1pf(x); }
template <> SK_HD float sk_log<float>(float x) { return logf(x); }
#endif

template <typename R> struct Eps;
template <> struct Eps<float> { static constexpr float v = 1.1920929e-07f; static constexpr int sweeps = 6; };
template <> struct Eps<double> { static constexpr double v = 2.220446049250313e-16; static constexpr int sweeps = 10; };

// eigenvalue floor of simkit's psd_project 'proj' (simkit/psd_project.py:37)
constexpr double kPsdFloor = 1e-6;

// --------------------------------------------------------------------------
// small linear algebra
// --------------------------------------------------------------------------
template <typename R> SK_HD R det3(const R* F) {
  return F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) +
         F[2] * (F[3] * F[7] - F[4] * F[6]);
}

// cof(F)_ij = dJ/dF_ij
template <typename R> SK_HD void cof3(const R* F, R* C) {
  C[0] = F[4] * F[8] - F[5] * F[7];
  C[1] = F[5] * F[6] - F[3] * F[8];
  C[2] = F[3] * F[7] - F[4] * F[6];
  C[3] = F[2] * F[7] - F[1] * F[8];
  C[4] = F[0] * F[8] - F[2] * F[6];
  C[5] = F[1] * F[6] - F[0] * F[7];
  C[6] = F[1] * F[5] - F[2] * F[4];
  C[7] = F[2] * F[3] - F[0] * F[5];
  C[8] = F[0] * F[4] - F[1] * F[3];
}

// sum of principal 2x2 minors
template <typename R> SK_HD R minors2(const R* G) {
  return (G[0] * G[4] - G[1] * G[3]) + (G[0] * G[8] - G[2] * G[6]) + (G[4] * G[8] - G[5] * G[7]);
}

// phi(z) = z - log(1 + z) >= 0, accurate for small |z|.
// With w = z / (2 + z): log(1+z) = 2 atanh(w) = 2 (w + w^3/3 + w^5/5 + ...),
// and z - 2w = z w, so phi = z w - 2 w^3 (1/3 + w^2/5 + w^4/7 + ...), a
// series with no cancellation; |z| <= 1/2 gives |w| <= 1/3.
template <typename R> SK_HD R phi_log1p(R z) {
  if (sk_abs(z) <= R(0.5)) {
    const R w = z / (R(2) + z);
    const R w2 = w * w;
    R s = R(1) / R(23);
    s = s * w2 + R(1) / R(21);
    s = s * w2 + R(1) / R(19);
    s = s * w2 + R(1) / R(17);
    s = s * w2 + R(1) / R(15);
    s = s * w2 + R(1) / R(13);
    s = s * w2 + R(1) / R(11);
    s = s * w2 + R(1) / R(9);
    s = s * w2 + R(1) / R(7);
    s = s * w2 + R(1) / R(5);
    s = s * w2 + R(1) / R(3);
    return z * w - R(2) * w * w2 * s;
  }
  return z - sk_log1p(z);
}

// --------------------------------------------------------------------------
// energy density
// --------------------------------------------------------------------------
// direct form, exactly simkit's expression (snh.py:116-126)
template <typename R> SK_HD R snh_psi(const R* F, R mu, R lam) {
  R IC = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) IC += F[k] * F[k];
  const R J = det3(F);
  const R alpha = R(1) + R(3) * mu / (R(4) * lam);
  const R d = J - alpha;
  return R(0.5) * mu * (IC - R(3)) - R(0.5) * mu * sk_log(IC + R(1)) + R(0.5) * lam * d * d;
}

// psi(I + G) - psi(I)
//   = 3mu/8 (|G|^2 - 2 I2(G) - 2 det G) + mu/2 phi(x/4) + lam/2 y^2,
// with x = I_C - 3 = 2 tr G + |G|^2 and y = J - 1 = tr G + I2(G) + det G.
template <typename R> SK_HD R snh_dpsi(const R* G, R mu, R lam) {
  R g2 = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) g2 += G[k] * G[k];
  const R tr = G[0] + G[4] + G[8];
  const R i2 = minors2(G);
  const R dg = det3(G);
  const R x = R(2) * tr + g2;
  const R y = tr + i2 + dg;
  return R(0.375) * mu * (g2 - R(2) * i2 - R(2) * dg) + R(0.5) * mu * phi_log1p(R(0.25) * x) +
         R(0.5) * lam * y * y;
}

// psi(I) = -mu/2 log 4 + lam/2 (1 - alpha)^2, the rest energy density
template <typename R> SK_HD R snh_psi_rest(R mu, R lam) {
  const R a1 = R(3) * mu / (R(4) * lam);
  return R(-0.5) * mu * sk_log(R(4)) + R(0.5) * lam * a1 * a1;
}

// --------------------------------------------------------------------------
// first Piola-Kirchhoff stress
// --------------------------------------------------------------------------
template <typename R> SK_HD void snh_pk1(const R* F, R mu, R lam, R* P) {
  R IC = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) IC += F[k] * F[k];
  const R J = det3(F);
  const R alpha = R(1) + R(3) * mu / (R(4) * lam);
  const R A = mu * IC / (IC + R(1));
  const R D = lam * (J - alpha);
  R C[9];
  cof3(F, C);
#pragma unroll
  for (int k = 0; k < 9; ++k) P[k] = A * F[k] + D * C[k];
}

// P(I + G) with cof(I + G) = (1 + tr G) I - G^T + cof G and
// A + D = mu x / (4 (4 + x)) + lam y, D = lam y - 3 mu / 4:
//   P = (A + D) I + A G + D (tr G I - G^T + cof G).
template <typename R> SK_HD void snh_pk1_disp(const R* G, R mu, R lam, R* P) {
  R g2 = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) g2 += G[k] * G[k];
  const R tr = G[0] + G[4] + G[8];
  const R x = R(2) * tr + g2;
  const R y = tr + minors2(G) + det3(G);
  const R q = mu * x / (R(4) * (R(4) + x));
  const R ApD = q + lam * y;
  const R A = R(0.75) * mu + q;
  const R D = lam * y - R(0.75) * mu;
  R C[9];
  cof3(G, C);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int k = 3 * i + j;
      R v = A * G[k] + D * (C[k] - G[3 * j + i]);
      if (i == j) v += ApD + D * tr;
      P[k] = v;
    }
}

// --------------------------------------------------------------------------
// explicit 9x9 F-Hessian, row-major vec(F) (the element tier)
// --------------------------------------------------------------------------
// A I + B f f^T + L c c^T + D d2J/dF2 for any energy of I_C and J
template <typename R> SK_HD void hessian9_coef(const R* F, R A, R B, R L, R D, R* H) {
  R C[9];
  cof3(F, C);
  for (int p = 0; p < 9; ++p)
    for (int q = 0; q < 9; ++q) H[9 * p + q] = B * F[p] * F[q] + L * C[p] * C[q] + (p == q ? A : R(0));
  // D * d2J/dF_ij dF_kl = D * eps_ikm eps_jln F_mn: nonzero only for i != k, j != l
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) {
      if (i == k) continue;
      const int m = 3 - i - k;
      const R sik = ((k - i + 3) % 3 == 1) ? R(1) : R(-1);  // eps_ikm
      for (int j = 0; j < 3; ++j)
        for (int l = 0; l < 3; ++l) {
          if (j == l) continue;
          const int n = 3 - j - l;
          const R sjl = ((l - j + 3) % 3 == 1) ? R(1) : R(-1);
          H[9 * (3 * i + j) + (3 * k + l)] += D * sik * sjl * F[3 * m + n];
        }
    }
}

template <typename R> SK_HD void snh_hessian9(const R* F, R mu, R lam, R* H) {
  R IC = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) IC += F[k] * F[k];
  const R J = det3(F);
  const R alpha = R(1) + R(3) * mu / (R(4) * lam);
  const R den = IC + R(1);
  hessian9_coef(F, mu * IC / den, R(2) * mu / (den * den), lam, lam * (J - alpha), H);
}

// 2D element tier (simkit/energies/stable_neo_hookean.py, dim == 2 branches)
template <typename R> SK_HD R snh_psi2(const R* F, R mu, R lam) {
  const R IC = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
  const R J = F[0] * F[3] - F[1] * F[2];
  const R alpha = R(1) + R(2) * mu / (R(3) * lam);
  const R d = J - alpha;
  return R(0.5) * mu * (IC - R(2)) - R(0.5) * mu * sk_log(IC + R(1)) + R(0.5) * lam * d * d;
}

template <typename R> SK_HD void snh_pk1_2(const R* F, R mu, R lam, R* P) {
  const R IC = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
  const R J = F[0] * F[3] - F[1] * F[2];
  const R alpha = R(1) + R(2) * mu / (R(3) * lam);
  const R A = mu * IC / (IC + R(1));
  const R D = lam * (J - alpha);
  const R C[4] = {F[3], -F[2], -F[1], F[0]};
  for (int k = 0; k < 4; ++k) P[k] = A * F[k] + D * C[k];
}

template <typename R> SK_HD void hessian4_coef(const R* F, R A, R B, R L, R D, R* H) {
  const R C[4] = {F[3], -F[2], -F[1], F[0]};
  for (int p = 0; p < 4; ++p)
    for (int q = 0; q < 4; ++q) H[4 * p + q] = B * F[p] * F[q] + L * C[p] * C[q] + (p == q ? A : R(0));
  // d2J: (00,11) = (11,00) = +1, (01,10) = (10,01) = -1
  H[4 * 0 + 3] += D;
  H[4 * 3 + 0] += D;
  H[4 * 1 + 2] -= D;
  H[4 * 2 + 1] -= D;
}

template <typename R> SK_HD void snh_hessian4(const R* F, R mu, R lam, R* H) {
  const R IC = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
  const R J = F[0] * F[3] - F[1] * F[2];
  const R alpha = R(1) + R(2) * mu / (R(3) * lam);
  const R den = IC + R(1);
  hessian4_coef(F, mu * IC / den, R(2) * mu / (den * den), lam, lam * (J - alpha), H);
}

// --------------------------------------------------------------------------
// Macklin-Mueller neo-Hookean (simkit/energies/macklin_mueller_neo_hookean.py:66-443):
//   psi = mu (1 - J) + lam/2 (1 - J)^2 + mu/2 (I_C - dim),
//   P = mu F + D cof F with D = lam (J - 1) - mu,
//   F-Hessian mu I + lam c c^T + D d2J/dF2 (the I_C/J form above with A = mu, B = 0).
// psi(I) = 0, and the displacement forms combine the terms that cancel at rest
// (A + D = lam (J - 1)).
// --------------------------------------------------------------------------
template <typename R> SK_HD R mmnh_psi(const R* F, R mu, R lam) {
  // simkit's expression order (macklin_mueller_neo_hookean.py:108-121), d = 1 - J
  const R d = -F[0] * F[4] * F[8] + F[0] * F[5] * F[7] + F[1] * F[3] * F[8] - F[1] * F[5] * F[6] -
              F[2] * F[3] * F[7] + F[2] * F[4] * F[6] + R(1);
  R IC = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) IC += F[k] * F[k];
  return mu * d + (lam * d * d) / R(2) + (mu * (IC - R(3))) / R(2);
}

// psi(I + G) = mu (|G|^2/2 - I2(G) - det G) + lam/2 y^2, y = J - 1 = tr G + I2(G) + det G
template <typename R> SK_HD R mmnh_dpsi(const R* G, R mu, R lam) {
  R g2 = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) g2 += G[k] * G[k];
  const R i2 = minors2(G);
  const R dg = det3(G);
  const R y = G[0] + G[4] + G[8] + i2 + dg;
  return mu * (R(0.5) * g2 - i2 - dg) + R(0.5) * lam * y * y;
}

template <typename R> SK_HD void mmnh_pk1(const R* F, R mu, R lam, R* P) {
  const R D = lam * (det3(F) - R(1)) - mu;
  R C[9];
  cof3(F, C);
#pragma unroll
  for (int k = 0; k < 9; ++k) P[k] = mu * F[k] + D * C[k];
}

// P(I + G) = lam y I + mu G + D (tr G I - G^T + cof G)
template <typename R> SK_HD void mmnh_pk1_disp(const R* G, R mu, R lam, R* P) {
  const R tr = G[0] + G[4] + G[8];
  const R y = tr + minors2(G) + det3(G);
  const R D = lam * y - mu;
  R C[9];
  cof3(G, C);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int k = 3 * i + j;
      R v = mu * G[k] + D * (C[k] - G[3 * j + i]);
      if (i == j) v += lam * y + D * tr;
      P[k] = v;
    }
}

template <typename R> SK_HD void mmnh_hessian9(const R* F, R mu, R lam, R* H) {
  hessian9_coef(F, mu, R(0), lam, lam * (det3(F) - R(1)) - mu, H);
}

template <typename R> SK_HD R mmnh_psi2(const R* F, R mu, R lam) {
  const R d = -F[0] * F[3] + F[1] * F[2] + R(1);
  const R IC = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
  return mu * d + (lam * d * d) / R(2) + (mu * (IC - R(2))) / R(2);
}

template <typename R> SK_HD void mmnh_pk1_2(const R* F, R mu, R lam, R* P) {
  const R D = lam * (F[0] * F[3] - F[1] * F[2] - R(1)) - mu;
  const R C[4] = {F[3], -F[2], -F[1], F[0]};
  for (int k = 0; k < 4; ++k) P[k] = mu * F[k] + D * C[k];
}

template <typename R> SK_HD void mmnh_hessian4(const R* F, R mu, R lam, R* H) {
  hessian4_coef(F, mu, R(0), lam, lam * (F[0] * F[3] - F[1] * F[2] - R(1)) - mu, H);
}

// materials of the per-tet kernels
enum : int { kMatSNH = 0, kMatMMNH = 1, kMatARAP = 2, kMatFCR = 3, kMatLE = 4 };

// --------------------------------------------------------------------------
// symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations
// (Golub & Van Loan, Matrix Computations, sec. 8.5).  S = {s00,s01,s02,s11,s12,s22};
// on return ev[k] are eigenvalues and column k of W (W[3*i+k]) the eigenvector.
// --------------------------------------------------------------------------
template <typename R> SK_HD void jacobi_rotate(R& app, R& aqq, R& apq, R& arp, R& arq, R* W, int p, int q) {
  if (apq == R(0)) return;
  R t, c;
  bool fast = false;
#if defined(__CUDA_ARCH__)
  // FP32 on the device: the rotation only has to be orthogonal to working precision (c = 1/sqrt(1+t^2),
  // s = t c), not correctly rounded, so the approximate divide and reciprocal square root serve
  if constexpr (sizeof(R) == 4) {
    const float theta = __fdividef(aqq - app, 2.f * apq);
    const float at = fabsf(theta);
    if (at > 1e18f) {
      t = __fdividef(0.5f, theta);
    } else {
      const float s2 = fmaf(at, at, 1.f);
      t = __fdividef(1.f, at + s2 * rsqrtf(s2));
      if (theta < 0.f) t = -t;
    }
    c = rsqrtf(fmaf(t, t, 1.f));
    fast = true;
  }
#endif
  if (!fast) {
    const R theta = (aqq - app) / (R(2) * apq);
    const R at = sk_abs(theta);
    t = (at > R(1e18)) ? R(0.5) / theta : R(1) / (at + sk_sqrt(at * at + R(1)));
    if (theta < R(0) && at <= R(1e18)) t = -t;
    c = R(1) / sk_sqrt(t * t + R(1));
  }
  const R s = t * c;
  app -= t * apq;
  aqq += t * apq;
  apq = R(0);
  const R g = arp, h = arq;
  arp = c * g - s * h;
  arq = s * g + c * h;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const R vp = W[3 * i + p], vq = W[3 * i + q];
    W[3 * i + p] = c * vp - s * vq;
    W[3 * i + q] = s * vp + c * vq;
  }
}

template <typename R> SK_HD void sym3_eig(const R* S, R* ev, R* W) {
  R a00 = S[0], a01 = S[1], a02 = S[2], a11 = S[3], a12 = S[4], a22 = S[5];
#pragma unroll
  for (int k = 0; k < 9; ++k) W[k] = (k % 4 == 0) ? R(1) : R(0);
  const R scale = sk_abs(a00) + sk_abs(a11) + sk_abs(a22) + sk_abs(a01) + sk_abs(a02) + sk_abs(a12);
  for (int sweep = 0; sweep < Eps<R>::sweeps; ++sweep) {
    const R off = sk_abs(a01) + sk_abs(a02) + sk_abs(a12);
    if (!(off > Eps<R>::v * R(0.25) * scale)) break;
    jacobi_rotate(a00, a11, a01, a02, a12, W, 0, 1);  // r = 2: a20, a21
    jacobi_rotate(a00, a22, a02, a01, a12, W, 0, 2);  // r = 1: a10, a12
    jacobi_rotate(a11, a22, a12, a01, a02, W, 1, 2);  // r = 0: a01, a02
  }
  ev[0] = a00;
  ev[1] = a11;
  ev[2] = a22;
}

// --------------------------------------------------------------------------
// rotation-variant SVD: F = U diag(s) V^T with U, V in SO(3), s0 >= s1 >= |s2|,
// s2 carrying the sign of det F.  V from the eigenvectors of F^T F, U by
// Gram-Schmidt on the columns of F V (u2 = u0 x u1 keeps det U = +1).
// --------------------------------------------------------------------------
template <typename R> SK_HD void any_perp(const R* a, R* out) {
  R e[3] = {R(0), R(0), R(0)};
  e[(sk_abs(a[0]) < R(0.6)) ? 0 : 1] = R(1);
  R v[3] = {a[1] * e[2] - a[2] * e[1], a[2] * e[0] - a[0] * e[2], a[0] * e[1] - a[1] * e[0]};
  const R n = sk_sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  out[0] = v[0] / n;
  out[1] = v[1] / n;
  out[2] = v[2] / n;
}

// norm n = sqrt(q) and its reciprocal i (i unused when n is 0); FP32 on the device from the
// approximate reciprocal square root, otherwise the correctly rounded square root and divide
template <typename R> SK_HD void unit_scale(R q, R& n, R& i) {
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(R) == 4) {
    i = q > 0.f ? rsqrtf(q) : 0.f;
    n = q * i;
    return;
  }
#endif
  n = sk_sqrt(q);
  i = n > R(0) ? R(1) / n : R(0);
}

template <typename R> SK_HD void svd3_rv(const R* F, R* U, R* s, R* V) {
  R S[6];
  S[0] = F[0] * F[0] + F[3] * F[3] + F[6] * F[6];
  S[1] = F[0] * F[1] + F[3] * F[4] + F[6] * F[7];
  S[2] = F[0] * F[2] + F[3] * F[5] + F[6] * F[8];
  S[3] = F[1] * F[1] + F[4] * F[4] + F[7] * F[7];
  S[4] = F[1] * F[2] + F[4] * F[5] + F[7] * F[8];
  S[5] = F[2] * F[2] + F[5] * F[5] + F[8] * F[8];
  R ev[3];
  sym3_eig(S, ev, V);
  // sort descending; each swap negates one column so det V stays +1
#define SK_SWAPCOL(a, b)                                          \
  {                                                               \
    R t_ = ev[a]; ev[a] = ev[b]; ev[b] = t_;                      \
    for (int i_ = 0; i_ < 3; ++i_) {                              \
      R v_ = V[3 * i_ + a];                                       \
      V[3 * i_ + a] = -V[3 * i_ + b];                             \
      V[3 * i_ + b] = v_;                                         \
    }                                                             \
  }
  if (ev[0] < ev[1]) SK_SWAPCOL(0, 1);
  if (ev[0] < ev[2]) SK_SWAPCOL(0, 2);
  if (ev[1] < ev[2]) SK_SWAPCOL(1, 2);
#undef SK_SWAPCOL
  R b[9];  // B = F V, column k = b[3*i + k]
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) b[3 * i + k] = F[3 * i] * V[k] + F[3 * i + 1] * V[3 + k] + F[3 * i + 2] * V[6 + k];
  R u0[3] = {b[0], b[3], b[6]};
  R fscale = R(0);
  for (int k = 0; k < 9; ++k) fscale = sk_max(fscale, sk_abs(F[k]));
  const R tiny = Eps<R>::v * Eps<R>::v * (fscale > R(0) ? fscale : R(1));
  R n0, i0;
  unit_scale(u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2], n0, i0);
  if (n0 > tiny) {
    u0[0] *= i0; u0[1] *= i0; u0[2] *= i0;
  } else {
    n0 = R(0); u0[0] = R(1); u0[1] = R(0); u0[2] = R(0);
  }
  R u1[3] = {b[1], b[4], b[7]};
  const R d01 = u0[0] * u1[0] + u0[1] * u1[1] + u0[2] * u1[2];
  u1[0] -= d01 * u0[0]; u1[1] -= d01 * u0[1]; u1[2] -= d01 * u0[2];
  R n1, i1;
  unit_scale(u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2], n1, i1);
  if (n1 > tiny) {
    u1[0] *= i1; u1[1] *= i1; u1[2] *= i1;
  } else {
    n1 = R(0);
    any_perp(u0, u1);
  }
  const R u2[3] = {u0[1] * u1[2] - u0[2] * u1[1], u0[2] * u1[0] - u0[0] * u1[2], u0[0] * u1[1] - u0[1] * u1[0]};
  s[0] = n0;
  s[1] = n1;
  s[2] = u2[0] * b[2] + u2[1] * b[5] + u2[2] * b[8];
  for (int i = 0; i < 3; ++i) {
    U[3 * i + 0] = u0[i];
    U[3 * i + 1] = u1[i];
    U[3 * i + 2] = u2[i];
  }
}

// --------------------------------------------------------------------------
// Corotational energies (simkit/energies/arap.py:71-145, fcr.py:40-190):
//   ARAP: psi = mu/2 |F - R|^2,                  P = mu (F - R),
//         H = mu (I - dR/dF)
//   FCR:  psi = mu |F - R|^2 + lam/2 (J - 1)^2,   P = 2 mu (F - R) + lam (J - 1) cof F,
//         H = 2 mu (I - dR/dF) + lam c c^T + lam (J - 1) d2J/dF2
// with R = U V^T of the rotation-variant SVD and, as simkit/rotation_gradient.py
// forms it,
//   dR/dF = sum over the pairs (i,j) of 2 / max(s_i + s_j, 1e-8) t t^T,
//   t = vec(U (e_i e_j^T - e_j e_i^T) V^T) / sqrt2
// (one pair and 1e-12 in 2D).  In 2D the polar factor is closed form:
// R = [[c, -s], [s, c]] with (c, s) the unit vector along (F00 + F11, F10 - F01),
// s_0 + s_1 = |(F00 + F11, F10 - F01)| and t = vec(J R) / sqrt2, J the quarter turn.
// --------------------------------------------------------------------------
template <typename R> SK_HD void polar3(const R* F, R* Rm) {
  R U[9], s[3], V[9];
  svd3_rv(F, U, s, V);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Rm[3 * i + j] = U[3 * i] * V[3 * j] + U[3 * i + 1] * V[3 * j + 1] + U[3 * i + 2] * V[3 * j + 2];
}
template <typename R> SK_HD R corot_shear3(const R* F) {   // |F - R|^2
  R Rm[9];
  polar3(F, Rm);
  R a = 0;
  for (int k = 0; k < 9; ++k) a += (F[k] - Rm[k]) * (F[k] - Rm[k]);
  return a;
}
// H -= coef dR/dF (9x9, row-major vec(F))
template <typename R> SK_HD void corot_twist9(const R* F, R coef, R* H) {
  R U[9], s[3], V[9];
  svd3_rv(F, U, s, V);
  const R rs2 = R(0.70710678118654752440);
  const int pi[3] = {0, 1, 0}, pj[3] = {1, 2, 2};
  for (int p = 0; p < 3; ++p) {
    const int i = pi[p], j = pj[p];
    const R w = coef * R(2) / sk_max(s[i] + s[j], R(1e-8));
    R t[9];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) t[3 * a + b] = rs2 * (U[3 * a + i] * V[3 * b + j] - U[3 * a + j] * V[3 * b + i]);
    for (int q = 0; q < 9; ++q)
      for (int r = 0; r < 9; ++r) H[9 * q + r] -= w * t[q] * t[r];
  }
}
template <typename R> SK_HD R arap_psi(const R* F, R mu) { return R(0.5) * mu * corot_shear3(F); }
template <typename R> SK_HD R fcr_psi(const R* F, R mu, R lam) {
  const R y = det3(F) - R(1);
  return mu * corot_shear3(F) + R(0.5) * lam * y * y;
}
// Displacement forms psi(I + G), accurate relative to psi near rest.
// |F - R|^2 = sum_k (s_k - 1)^2 with s_k^2 = 1 + l_k, l_k the eigenvalues of
// E = F^T F - I = G + G^T + G^T G, so s_k - 1 = l_k / (sqrt(1 + l_k) + 1) has no
// cancellation; for det F < 0 the smallest singular value is negative
// (s - 1 = -(sqrt(1 + l) + 1)).  J - 1 = tr G + I2(G) + det G likewise.
template <typename R> SK_HD R corot_dshear3(const R* G, R Jm1) {
  R E[6];
  E[0] = R(2) * G[0] + G[0] * G[0] + G[3] * G[3] + G[6] * G[6];
  E[1] = G[1] + G[3] + G[0] * G[1] + G[3] * G[4] + G[6] * G[7];
  E[2] = G[2] + G[6] + G[0] * G[2] + G[3] * G[5] + G[6] * G[8];
  E[3] = R(2) * G[4] + G[1] * G[1] + G[4] * G[4] + G[7] * G[7];
  E[4] = G[5] + G[7] + G[1] * G[2] + G[4] * G[5] + G[7] * G[8];
  E[5] = R(2) * G[8] + G[2] * G[2] + G[5] * G[5] + G[8] * G[8];
  R l[3], W[9];
  sym3_eig(E, l, W);
  const int kmin = l[0] <= l[1] ? (l[0] <= l[2] ? 0 : 2) : (l[1] <= l[2] ? 1 : 2);
  R a = R(0);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const R r = sk_sqrt(sk_max(R(1) + l[k], R(0)));
    const R d = (Jm1 < R(-1) && k == kmin) ? -(r + R(1)) : l[k] / (r + R(1));
    a += d * d;
  }
  return a;
}
template <typename R> SK_HD R arap_dpsi(const R* G, R mu) {
  const R Jm1 = G[0] + G[4] + G[8] + minors2(G) + det3(G);
  return R(0.5) * mu * corot_dshear3(G, Jm1);
}
template <typename R> SK_HD R fcr_dpsi(const R* G, R mu, R lam) {
  const R y = G[0] + G[4] + G[8] + minors2(G) + det3(G);
  return mu * corot_dshear3(G, y) + R(0.5) * lam * y * y;
}
template <typename R> SK_HD void corot_pk1(const R* F, R two_mu_or_mu, R vol_coef, R* P) {
  // P = a (F - R) + vol_coef cof F
  R Rm[9], C[9];
  polar3(F, Rm);
  cof3(F, C);
  for (int k = 0; k < 9; ++k) P[k] = two_mu_or_mu * (F[k] - Rm[k]) + vol_coef * C[k];
}
template <typename R> SK_HD void arap_pk1(const R* F, R mu, R* P) { corot_pk1(F, mu, R(0), P); }
template <typename R> SK_HD void fcr_pk1(const R* F, R mu, R lam, R* P) {
  corot_pk1(F, R(2) * mu, lam * (det3(F) - R(1)), P);
}
template <typename R> SK_HD void arap_pk1_disp(const R* G, R mu, R* P) {
  R F[9];
  for (int k = 0; k < 9; ++k) F[k] = G[k] + ((k % 4 == 0) ? R(1) : R(0));
  corot_pk1(F, mu, R(0), P);
}
template <typename R> SK_HD void fcr_pk1_disp(const R* G, R mu, R lam, R* P) {
  R F[9];
  for (int k = 0; k < 9; ++k) F[k] = G[k] + ((k % 4 == 0) ? R(1) : R(0));
  const R y = G[0] + G[4] + G[8] + minors2(G) + det3(G);
  corot_pk1(F, R(2) * mu, lam * y, P);
}
template <typename R> SK_HD void arap_hessian9(const R* F, R mu, R* H) {
  hessian9_coef(F, mu, R(0), R(0), R(0), H);
  corot_twist9(F, mu, H);
}
template <typename R> SK_HD void fcr_hessian9(const R* F, R mu, R lam, R* H) {
  hessian9_coef(F, R(2) * mu, R(0), lam, lam * (det3(F) - R(1)), H);
  corot_twist9(F, R(2) * mu, H);
}
// 2D (row-major F = [F00, F01, F10, F11])
template <typename R> SK_HD R polar2(const R* F, R* Rm) {   // returns s_0 + s_1
  const R a = F[0] + F[3], b = F[2] - F[1];
  const R n = sk_sqrt(a * a + b * b);
  R c = R(1), sn = R(0);
  if (n > R(0)) {
    c = a / n;
    sn = b / n;
  }
  Rm[0] = c; Rm[1] = -sn; Rm[2] = sn; Rm[3] = c;
  return n;
}
template <typename R> SK_HD R corot_shear2(const R* F) {
  R Rm[4];
  polar2(F, Rm);
  R a = 0;
  for (int k = 0; k < 4; ++k) a += (F[k] - Rm[k]) * (F[k] - Rm[k]);
  return a;
}
template <typename R> SK_HD R arap_psi2(const R* F, R mu) { return R(0.5) * mu * corot_shear2(F); }
template <typename R> SK_HD R fcr_psi2(const R* F, R mu, R lam) {
  const R y = F[0] * F[3] - F[1] * F[2] - R(1);
  return mu * corot_shear2(F) + R(0.5) * lam * y * y;
}
template <typename R> SK_HD void corot_pk1_2(const R* F, R a, R vol_coef, R* P) {
  R Rm[4];
  polar2(F, Rm);
  const R C[4] = {F[3], -F[2], -F[1], F[0]};
  for (int k = 0; k < 4; ++k) P[k] = a * (F[k] - Rm[k]) + vol_coef * C[k];
}
template <typename R> SK_HD void arap_pk1_2(const R* F, R mu, R* P) { corot_pk1_2(F, mu, R(0), P); }
template <typename R> SK_HD void fcr_pk1_2(const R* F, R mu, R lam, R* P) {
  corot_pk1_2(F, R(2) * mu, lam * (F[0] * F[3] - F[1] * F[2] - R(1)), P);
}
template <typename R> SK_HD void corot_twist4(const R* F, R coef, R* H) {
  R Rm[4];
  const R n = polar2(F, Rm);
  const R c = Rm[0], sn = Rm[2];
  const R rs2 = R(0.70710678118654752440);
  const R t[4] = {-rs2 * sn, -rs2 * c, rs2 * c, -rs2 * sn};
  const R w = coef * R(2) / sk_max(n, R(1e-12));
  for (int q = 0; q < 4; ++q)
    for (int r = 0; r < 4; ++r) H[4 * q + r] -= w * t[q] * t[r];
}
template <typename R> SK_HD void arap_hessian4(const R* F, R mu, R* H) {
  hessian4_coef(F, mu, R(0), R(0), R(0), H);
  corot_twist4(F, mu, H);
}
template <typename R> SK_HD void fcr_hessian4(const R* F, R mu, R lam, R* H) {
  hessian4_coef(F, R(2) * mu, R(0), lam, lam * (F[0] * F[3] - F[1] * F[2] - R(1)), H);
  corot_twist4(F, R(2) * mu, H);
}

// --------------------------------------------------------------------------
// Linear (small-strain) elasticity (simkit/energies/linear_elasticity.py:43-136):
//   psi = mu |eps|^2 + lam/2 tr(eps)^2,  eps = (F + F^T)/2 - I
//   P   = mu (F + F^T - 2 I) + lam tr(F - I) I
//   H   = mu (I + T) + lam vec(I) vec(I)^T   (T: vec(X) -> vec(X^T)), constant and PSD;
// simkit applies no PSD projection to it.  In displacement form eps = sym(G) exactly.
// --------------------------------------------------------------------------
template <typename R, int D> SK_HD R le_dpsi_d(const R* G, R mu, R lam) {
  R e2 = 0, tr = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    tr += G[(D + 1) * i];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      const R e = R(0.5) * (G[D * i + j] + G[D * j + i]);
      e2 += e * e;
    }
  }
  return mu * e2 + R(0.5) * lam * tr * tr;
}
template <typename R, int D> SK_HD void le_pk1_disp_d(const R* G, R mu, R lam, R* P) {
  R tr = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) tr += G[(D + 1) * i];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) P[D * i + j] = mu * (G[D * i + j] + G[D * j + i]) + (i == j ? lam * tr : R(0));
}
template <typename R, int D> SK_HD void le_grad_of(const R* F, R* G) {
#pragma unroll
  for (int k = 0; k < D * D; ++k) G[k] = F[k] - ((k % (D + 1) == 0) ? R(1) : R(0));
}
template <typename R, int D> SK_HD R le_psi_d(const R* F, R mu, R lam) {
  R G[D * D];
  le_grad_of<R, D>(F, G);
  return le_dpsi_d<R, D>(G, mu, lam);
}
template <typename R, int D> SK_HD void le_pk1_d(const R* F, R mu, R lam, R* P) {
  R G[D * D];
  le_grad_of<R, D>(F, G);
  le_pk1_disp_d<R, D>(G, mu, lam, P);
}
template <typename R, int D> SK_HD void le_hessian_d(R mu, R lam, R* H) {
  constexpr int N = D * D;
#pragma unroll
  for (int p = 0; p < N; ++p)
#pragma unroll
    for (int q = 0; q < N; ++q) {
      const int i = p / D, j = p % D, k = q / D, l = q % D;
      H[N * p + q] = mu * (R(i == k && j == l) + R(i == l && j == k)) + lam * R(i == j && k == l);
    }
}

// element-tier dispatch over material and dimension (F is row-major D x D)
template <typename R, int D> SK_HD R elem_psi(int mat, const R* F, R mu, R lam) {
  if (mat == kMatLE) return le_psi_d<R, D>(F, mu, lam);
  if (D == 3) return mat == kMatMMNH ? mmnh_psi(F, mu, lam)
                   : mat == kMatARAP ? arap_psi(F, mu)
                   : mat == kMatFCR  ? fcr_psi(F, mu, lam) : snh_psi(F, mu, lam);
  return mat == kMatMMNH ? mmnh_psi2(F, mu, lam)
       : mat == kMatARAP ? arap_psi2(F, mu)
       : mat == kMatFCR  ? fcr_psi2(F, mu, lam) : snh_psi2(F, mu, lam);
}
template <typename R, int D> SK_HD void elem_pk1(int mat, const R* F, R mu, R lam, R* P) {
  if (mat == kMatLE) {
    le_pk1_d<R, D>(F, mu, lam, P);
  } else if (D == 3) {
    if (mat == kMatMMNH) mmnh_pk1(F, mu, lam, P);
    else if (mat == kMatARAP) arap_pk1(F, mu, P);
    else if (mat == kMatFCR) fcr_pk1(F, mu, lam, P);
    else snh_pk1(F, mu, lam, P);
  } else {
    if (mat == kMatMMNH) mmnh_pk1_2(F, mu, lam, P);
    else if (mat == kMatARAP) arap_pk1_2(F, mu, P);
    else if (mat == kMatFCR) fcr_pk1_2(F, mu, lam, P);
    else snh_pk1_2(F, mu, lam, P);
  }
}
template <typename R, int D> SK_HD void elem_hessian(int mat, const R* F, R mu, R lam, R* H) {
  if (mat == kMatLE) {
    le_hessian_d<R, D>(mu, lam, H);
  } else if (D == 3) {
    if (mat == kMatMMNH) mmnh_hessian9(F, mu, lam, H);
    else if (mat == kMatARAP) arap_hessian9(F, mu, H);
    else if (mat == kMatFCR) fcr_hessian9(F, mu, lam, H);
    else snh_hessian9(F, mu, lam, H);
  } else {
    if (mat == kMatMMNH) mmnh_hessian4(F, mu, lam, H);
    else if (mat == kMatARAP) arap_hessian4(F, mu, H);
    else if (mat == kMatFCR) fcr_hessian4(F, mu, lam, H);
    else snh_hessian4(F, mu, lam, H);
  }
}

// material dispatch of the per-tet kernels (3D)
template <typename R> SK_HD R mat_dpsi(int mat, const R* G, R mu, R lam) {
  if (mat == kMatLE) return le_dpsi_d<R, 3>(G, mu, lam);
  if (mat == kMatMMNH) return mmnh_dpsi(G, mu, lam);
  if (mat == kMatARAP) return arap_dpsi(G, mu);
  if (mat == kMatFCR) return fcr_dpsi(G, mu, lam);
  return snh_dpsi(G, mu, lam);
}
template <typename R> SK_HD R mat_psi(int mat, const R* F, R mu, R lam) {
  if (mat == kMatLE) return le_psi_d<R, 3>(F, mu, lam);
  if (mat == kMatMMNH) return mmnh_psi(F, mu, lam);
  if (mat == kMatARAP) return arap_psi(F, mu);
  if (mat == kMatFCR) return fcr_psi(F, mu, lam);
  return snh_psi(F, mu, lam);
}
template <typename R> SK_HD void mat_pk1_disp(int mat, const R* G, R mu, R lam, R* P) {
  if (mat == kMatLE) le_pk1_disp_d<R, 3>(G, mu, lam, P);
  else if (mat == kMatMMNH) mmnh_pk1_disp(G, mu, lam, P);
  else if (mat == kMatARAP) arap_pk1_disp(G, mu, P);
  else if (mat == kMatFCR) fcr_pk1_disp(G, mu, lam, P);
  else snh_pk1_disp(G, mu, lam, P);
}
template <typename R> SK_HD void mat_pk1(int mat, const R* F, R mu, R lam, R* P) {
  if (mat == kMatLE) le_pk1_d<R, 3>(F, mu, lam, P);
  else if (mat == kMatMMNH) mmnh_pk1(F, mu, lam, P);
  else if (mat == kMatARAP) arap_pk1(F, mu, P);
  else if (mat == kMatFCR) fcr_pk1(F, mu, lam, P);
  else snh_pk1(F, mu, lam, P);
}

// --------------------------------------------------------------------------
// Per-tet Hessian w.r.t. the 12 vertex coordinates:
//   K = L^T psd(vol * H_F) L, L the lift dF/dx,
// with psd() the eigenvalue floor of simkit's psd_project applied to the
// vol-weighted 9x9 block (simkit/energies/stable_neo_hookean.py:531-537).
//
// The 9x9 block's eigensystem is analytic in the rotation-variant SVD of F:
//   twist (i,j):  U (e_i e_j^T - e_j e_i^T) V^T / sqrt2, eigenvalue A + D s_k
//   flip  (i,j):  U (e_i e_j^T + e_j e_i^T) V^T / sqrt2, eigenvalue A - D s_k
//   scaling m:    U diag(w_m) V^T, w_m the eigenvectors of the 3x3
//                 A I + B s s^T + lam c c^T + D [[0,s2,s1],[s2,0,s0],[s1,s0,0]],
//                 c = (s1 s2, s0 s2, s0 s1)
// ({i,j,k} = {0,1,2}).  Flooring eigenvalue l at f adds (f - vol l) q q^T,
// so the projected block is the analytic one plus those rank-1 terms.
//
// Lifted, each term is per vertex pair (a,b):
//   vol A (gN_a . gN_b) I + vol B p_a p_b^T + vol lam c_a c_b^T
//   + vol D skew(F (gN_a x gN_b)) + sum_m kappa_m r_ma r_mb^T,
// with p_a = F gN_a, c_a = cof(F) gN_a, r_ma = Q_m gN_a.
//
// Output (78 values): diagonal blocks (a,a) a = 0..3 packed upper
// (xx,xy,xz,yy,yz,zz) at 6a; off-diagonal blocks (a,b), a < b in the order
// (0,1),(0,2),(0,3),(1,2),(1,3),(2,3), row-major at 24 + 9k.
// --------------------------------------------------------------------------
constexpr int kTetHessVals = 78;

SK_HD int offdiag_index(int a, int b) {  // a < b
  return a == 0 ? (b - 1) : (a == 1 ? (b + 1) : 5);
}

// Tw: coefficient of the corotational term -Tw dR/dF (0 for the neo-Hookean
// materials); it lowers each twist eigenvalue by Tw 2 / max(s_i + s_j, 1e-8).
template <typename R, typename RS>
SK_HD void snh_eigensystem(const R* F, R mu, R lam, R vol, R A, R D, R B,
                           R* U, R* s, R* V, R* W, R* lam9, R Tw = R(0)) {
  // SVD in precision RS (double for nearly inverted elements)
  RS Fs[9], Us[9], ss[3], Vs[9];
  for (int k = 0; k < 9; ++k) Fs[k] = RS(F[k]);
  svd3_rv(Fs, Us, ss, Vs);
  for (int k = 0; k < 9; ++k) { U[k] = R(Us[k]); V[k] = R(Vs[k]); }
  for (int k = 0; k < 3; ++k) s[k] = R(ss[k]);
  // twist/flip eigenvalues, pair order (0,1)->k=2, (0,2)->k=1, (1,2)->k=0
  lam9[0] = A + D * s[2]; lam9[1] = A - D * s[2];
  lam9[2] = A + D * s[1]; lam9[3] = A - D * s[1];
  lam9[4] = A + D * s[0]; lam9[5] = A - D * s[0];
  if (Tw != R(0)) {
    lam9[0] -= Tw * R(2) / sk_max(s[0] + s[1], R(1e-8));
    lam9[2] -= Tw * R(2) / sk_max(s[0] + s[2], R(1e-8));
    lam9[4] -= Tw * R(2) / sk_max(s[1] + s[2], R(1e-8));
  }
  // scaling block
  const R c0 = s[1] * s[2], c1 = s[0] * s[2], c2 = s[0] * s[1];
  RS S3[6];
  S3[0] = RS(A + B * s[0] * s[0] + lam * c0 * c0);
  S3[1] = RS(B * s[0] * s[1] + lam * c0 * c1 + D * s[2]);
  S3[2] = RS(B * s[0] * s[2] + lam * c0 * c2 + D * s[1]);
  S3[3] = RS(A + B * s[1] * s[1] + lam * c1 * c1);
  S3[4] = RS(B * s[1] * s[2] + lam * c1 * c2 + D * s[0]);
  S3[5] = RS(A + B * s[2] * s[2] + lam * c2 * c2);
  RS evs[3], Ws[9];
  sym3_eig(S3, evs, Ws);
  for (int k = 0; k < 3; ++k) lam9[6 + k] = R(evs[k]);
  for (int k = 0; k < 9; ++k) W[k] = R(Ws[k]);
  (void)mu; (void)vol;
}

// F: deformation gradient; gN: 4x3 shape gradients; out: 78 packed values.
// fallback_J: elements with det F below it run the SVD in FP64.
// floor_v: eigenvalue floor (simkit's 1e-6); project = false skips the
// projection (simkit's psd=False, snh.py:534).
// material: kMatSNH, kMatMMNH, kMatARAP or kMatFCR.  Every material's F-space
// Hessian has the form A I + B f f^T + Lc c c^T + D d2J/dF2 - Tw dR/dF
// (f = vec F, c = vec cof F); the first four terms are lifted analytically, the
// corotational term as its three rank-1 twist directions.
// linear elasticity: K_ab = vol (mu (g_a . g_b) I + mu g_b g_a^T + lam g_a g_b^T), constant in F
// and never projected (simkit/energies/linear_elasticity.py:199-230)
template <typename R> SK_HD void le_tet_hessian(R mu, R lam, R vol, const R* gN, R* out) {
  const R vm = vol * mu, vl = vol * lam;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const R* g = gN + 3 * a;
    const R gg = vm * (g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    R* o = out + 6 * a;
    o[0] = gg + (vm + vl) * g[0] * g[0];
    o[1] = (vm + vl) * g[0] * g[1];
    o[2] = (vm + vl) * g[0] * g[2];
    o[3] = gg + (vm + vl) * g[1] * g[1];
    o[4] = (vm + vl) * g[1] * g[2];
    o[5] = gg + (vm + vl) * g[2] * g[2];
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a + 1; b < 4; ++b) {
      R* o = out + 24 + 9 * offdiag_index(a, b);
      const R* ga = gN + 3 * a;
      const R* gb = gN + 3 * b;
      const R gg = vm * (ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2]);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) o[3 * i + k] = (i == k ? gg : R(0)) + vm * ga[k] * gb[i] + vl * ga[i] * gb[k];
    }
}

// FP64_SVD: nearly inverted elements (J < fallback_J) take the SVD in FP64; without it the caller has
// set those elements aside (the FP32 Hessian kernel hands them to a second kernel, so that the FP64
// path's registers do not limit the occupancy of the common one)
template <typename R, bool FP64_SVD = true>
SK_HD void nh_tet_hessian(const R* F, R mu, R lam, R vol, const R* gN, R* out, R fallback_J, bool project,
                          int material);

// any material (the kernels call le_tet_hessian / nh_tet_hessian from separate instantiations)
template <typename R>
SK_HD void snh_tet_hessian(const R* F, R mu, R lam, R vol, const R* gN, R* out, R fallback_J = R(0.1),
                           bool project = true, int material = kMatSNH) {
  if (material == kMatLE)
    le_tet_hessian(mu, lam, vol, gN, out);
  else
    nh_tet_hessian(F, mu, lam, vol, gN, out, fallback_J, project, material);
}

// the neo-Hookean and corotational materials
template <typename R, bool FP64_SVD>
SK_HD void nh_tet_hessian(const R* F, R mu, R lam, R vol, const R* gN, R* out, R fallback_J, bool project,
                          int material) {
  R IC = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) IC += F[k] * F[k];
  const R J = det3(F);
  R A, B, D, Lc = lam, Tw = R(0);
  if (material == kMatMMNH) {
    A = mu;
    B = R(0);
    D = lam * (J - R(1)) - mu;
  } else if (material == kMatARAP) {
    A = mu; B = R(0); Lc = R(0); D = R(0); Tw = mu;
  } else if (material == kMatFCR) {
    A = R(2) * mu; B = R(0); D = lam * (J - R(1)); Tw = R(2) * mu;
  } else {
    const R alpha = R(1) + R(3) * mu / (R(4) * lam);
    const R den = IC + R(1);
    A = mu * IC / den;
    B = R(2) * mu / (den * den);
    D = lam * (J - alpha);
  }
  R C[9];
  cof3(F, C);

  // per-vertex lifted vectors
  R p[12], c[12];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      p[3 * a + i] = F[3 * i] * gN[3 * a] + F[3 * i + 1] * gN[3 * a + 1] + F[3 * i + 2] * gN[3 * a + 2];
      c[3 * a + i] = C[3 * i] * gN[3 * a] + C[3 * i + 1] * gN[3 * a + 1] + C[3 * i + 2] * gN[3 * a + 2];
    }
  const R vA = vol * A, vB = vol * B, vL = vol * Lc, vD = vol * D;

  // analytic terms
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const R gg = vA * (gN[3 * a] * gN[3 * a] + gN[3 * a + 1] * gN[3 * a + 1] + gN[3 * a + 2] * gN[3 * a + 2]);
    R* o = out + 6 * a;
    o[0] = gg + vB * p[3 * a] * p[3 * a] + vL * c[3 * a] * c[3 * a];
    o[1] = vB * p[3 * a] * p[3 * a + 1] + vL * c[3 * a] * c[3 * a + 1];
    o[2] = vB * p[3 * a] * p[3 * a + 2] + vL * c[3 * a] * c[3 * a + 2];
    o[3] = gg + vB * p[3 * a + 1] * p[3 * a + 1] + vL * c[3 * a + 1] * c[3 * a + 1];
    o[4] = vB * p[3 * a + 1] * p[3 * a + 2] + vL * c[3 * a + 1] * c[3 * a + 2];
    o[5] = gg + vB * p[3 * a + 2] * p[3 * a + 2] + vL * c[3 * a + 2] * c[3 * a + 2];
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a + 1; b < 4; ++b) {
      R* o = out + 24 + 9 * offdiag_index(a, b);
      const R* ga = gN + 3 * a;
      const R* gb = gN + 3 * b;
      const R gg = vA * (ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2]);
      const R n[3] = {ga[1] * gb[2] - ga[2] * gb[1], ga[2] * gb[0] - ga[0] * gb[2], ga[0] * gb[1] - ga[1] * gb[0]};
      R w[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) w[i] = vD * (F[3 * i] * n[0] + F[3 * i + 1] * n[1] + F[3 * i + 2] * n[2]);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k)
          o[3 * i + k] = vB * p[3 * a + i] * p[3 * b + k] + vL * c[3 * a + i] * c[3 * b + k] + (i == k ? gg : R(0));
      // skew(w): (0,1)=w2 (0,2)=-w1 (1,0)=-w2 (1,2)=w0 (2,0)=w1 (2,1)=-w0
      o[1] += w[2]; o[2] -= w[1];
      o[3] -= w[2]; o[5] += w[0];
      o[6] += w[1]; o[7] -= w[0];
    }

  if (!project && Tw == R(0)) return;
  // eigenvalue floor
  R U[9], s[3], V[9], W[9], lam9[9];
  if constexpr (FP64_SVD) {
    if (J < fallback_J)
      snh_eigensystem<R, double>(F, mu, Lc, vol, A, D, B, U, s, V, W, lam9, Tw);
    else
      snh_eigensystem<R, R>(F, mu, Lc, vol, A, D, B, U, s, V, W, lam9, Tw);
  } else {
    snh_eigensystem<R, R>(F, mu, Lc, vol, A, D, B, U, s, V, W, lam9, Tw);
  }
  const R floor_v = R(kPsdFloor);
  R beta[12];  // beta[3a + n] = v_n . gN_a
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int n = 0; n < 3; ++n)
      beta[3 * a + n] = V[n] * gN[3 * a] + V[3 + n] * gN[3 * a + 1] + V[6 + n] * gN[3 * a + 2];
  const R rs2 = R(0.70710678118654752440);
#pragma unroll
  for (int m = 0; m < 9; ++m) {
    // Correction along eigenvector m on top of the analytic terms.  Twist
    // directions (even m < 6) of a corotational material carry -Tw dR/dF; when
    // the full eigenvalue falls below the floor the correction is taken from the
    // analytic eigenvalue A + D s_k, so the floor is met without cancelling two
    // large terms (s_i + s_j -> 0).
    const bool floored = project && floor_v - vol * lam9[m] > R(0);
    R kappa = floored ? floor_v - vol * lam9[m] : R(0);
    if (Tw != R(0) && m < 6 && !(m & 1)) {
      const int pr = m >> 1;
      const R ssum = pr == 0 ? s[0] + s[1] : (pr == 1 ? s[0] + s[2] : s[1] + s[2]);
      kappa = floored ? floor_v - vol * (A + D * s[2 - pr]) : -vol * Tw * R(2) / sk_max(ssum, R(1e-8));
    }
    if (kappa == R(0)) continue;
    R r[12];
    if (m < 6) {
      const int pr = m >> 1;
      const int i = pr == 2 ? 1 : 0;
      const int j = pr == 0 ? 1 : 2;
      const R sg = (m & 1) ? R(1) : R(-1);  // twist: u_i b_j - u_j b_i ; flip: +
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d)
          r[3 * a + d] = rs2 * (U[3 * d + i] * beta[3 * a + j] + sg * U[3 * d + j] * beta[3 * a + i]);
    } else {
      const int mm = m - 6;
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d)
          r[3 * a + d] = W[mm] * beta[3 * a] * U[3 * d] + W[3 + mm] * beta[3 * a + 1] * U[3 * d + 1] +
                         W[6 + mm] * beta[3 * a + 2] * U[3 * d + 2];
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      R* o = out + 6 * a;
      const R* ra = r + 3 * a;
      o[0] += kappa * ra[0] * ra[0]; o[1] += kappa * ra[0] * ra[1]; o[2] += kappa * ra[0] * ra[2];
      o[3] += kappa * ra[1] * ra[1]; o[4] += kappa * ra[1] * ra[2]; o[5] += kappa * ra[2] * ra[2];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = a + 1; b < 4; ++b) {
        R* o = out + 24 + 9 * offdiag_index(a, b);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int k = 0; k < 3; ++k) o[3 * i + k] += kappa * r[3 * a + i] * r[3 * b + k];
      }
  }
}

// shape gradients from the inverse rest edge matrix: rows of Dinv are
// gN_1..gN_3 and gN_0 = -(gN_1 + gN_2 + gN_3)
template <typename R> SK_HD void shape_grads(const R* Dinv, R* gN) {
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    gN[3 + j] = Dinv[j];
    gN[6 + j] = Dinv[3 + j];
    gN[9 + j] = Dinv[6 + j];
    gN[j] = -(Dinv[j] + Dinv[3 + j] + Dinv[6 + j]);
  }
}

// G = [du1 du2 du3] Dinv, du_a = u_a - u_0 (edge displacement differences)
template <typename R> SK_HD void disp_grad(const R* du, const R* Dinv, R* G) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      G[3 * i + j] = du[i] * Dinv[j] + du[3 + i] * Dinv[3 + j] + du[6 + i] * Dinv[6 + j];
}

}  // namespace skg
