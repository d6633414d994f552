// basis.cuh -- hierarchical H1 basis on the GPU (host+device templates).
//
// The polynomial recursions and shape definitions follow NGSolve:
//   IntLegNoBubble              fem/recursive_pol.hpp:1344-1377
//   JacobiPolynomialFix<1,1>    fem/recursive_pol.hpp:1641-1676
//   IntegratedJacobiPolynomialAlpha  fem/recursive_pol.hpp:1857-1917,
//                               coefficients fem/recursive_pol.cpp:126-155
//   DubinerBasisOrthoBub        fem/recursive_pol.hpp:2819-2860
//   DubinerBasis3DOrthoBub      fem/recursive_pol.hpp:2968-3008
//   tet shapes                  fem/h1hofe_impl.hpp:509-577
//   hex shapes                  fem/h1hofe_impl.hpp:821-890 (tensor form below)
// Forward-mode derivatives (value + 3 partials) play the role of AutoDiff<3>
// in CalcDShape (fem/tscalarfe_impl.hpp:24-32).
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"

namespace gh1 {

#define GH1_HD __host__ __device__ __forceinline__

struct Dual3 {
  double v, dx, dy, dz;
  GH1_HD Dual3() : v(0), dx(0), dy(0), dz(0) {}
  GH1_HD Dual3(double a) : v(a), dx(0), dy(0), dz(0) {}
  GH1_HD Dual3(double a, double b, double c, double d) : v(a), dx(b), dy(c), dz(d) {}
};
GH1_HD Dual3 operator+(Dual3 a, Dual3 b) { return Dual3(a.v + b.v, a.dx + b.dx, a.dy + b.dy, a.dz + b.dz); }
GH1_HD Dual3 operator-(Dual3 a, Dual3 b) { return Dual3(a.v - b.v, a.dx - b.dx, a.dy - b.dy, a.dz - b.dz); }
GH1_HD Dual3 operator*(Dual3 a, Dual3 b) {
  return Dual3(a.v * b.v, a.dx * b.v + a.v * b.dx, a.dy * b.v + a.v * b.dy, a.dz * b.v + a.v * b.dz);
}
GH1_HD Dual3 operator*(double s, Dual3 a) { return Dual3(s * a.v, s * a.dx, s * a.dy, s * a.dz); }
GH1_HD Dual3 operator*(Dual3 a, double s) { return s * a; }
GH1_HD Dual3 operator+(double s, Dual3 a) { return Dual3(s + a.v, a.dx, a.dy, a.dz); }
GH1_HD Dual3 operator+(Dual3 a, double s) { return s + a; }
GH1_HD Dual3 operator-(double s, Dual3 a) { return Dual3(s - a.v, -a.dx, -a.dy, -a.dz); }
GH1_HD Dual3 operator-(Dual3 a, double s) { return Dual3(a.v - s, a.dx, a.dy, a.dz); }

// ---- 1D: integrated Legendre divided by the bubble --------------------------
// P0 = -1/2, P1 = -x/2, P_k = A_k x P_{k-1} + C_k y^2 P_{k-2},
// A_k = (2k+1)/(k+2), C_k = -(k-1)/(k+2)  (index shift i -> i+2 of CalcA/CalcC)
template <class T>
GH1_HD void ilnb_scaled(int n, T x, T y, T c, T* out) {
  if (n < 0) return;
  T p0 = c * (-0.5);
  T p1 = (c * (-0.5)) * x;
  out[0] = p0;
  if (n >= 1) out[1] = p1;
  T yy = y * y;
  for (int k = 2; k <= n; k++) {
    double A = (2.0 * k + 1.0) / (k + 2.0), C = -(k - 1.0) / (k + 2.0);
    T pn = (A * x) * p1 + (C * yy) * p0;
    p0 = p1;
    p1 = pn;
    out[k] = pn;
  }
}

// ---- Jacobi(1,1), scaled, "1Assign" ordering ----------------------------------
GH1_HD double jac11_A(int i) { i--; return (2.0 * i + 2) * (2.0 * i + 3) * (2.0 * i + 4) / (2.0 * (i + 1) * (i + 3) * (2.0 * i + 2)); }
GH1_HD double jac11_C(int i) { i--; return -2.0 * (i + 1) * (i + 1) * (2.0 * i + 4) / (2.0 * (i + 1) * (i + 3) * (2.0 * i + 2)); }
template <class T>
GH1_HD void jac11_scaled(int n, T x, T y, T c, T* out) {
  T p2 = c, p1 = c * (2.0 * x);
  T yy = y * y;
  for (int i = 0; i <= n; i++) {
    out[i] = p2;
    int k = i + 2;
    T pn = (jac11_A(k) * x) * p1 + (jac11_C(k) * yy) * p2;
    p2 = p1;
    p1 = pn;
  }
}

// ---- integrated Jacobi with parameter alpha --------------------------------------
GH1_HD void ija_coef(double al, int n, double& A, double& B, double& C) {
  if (n == 1) { A = 0.25 * (al + 2); B = 0.25 * (al - 2); C = 0; return; }
  double den = (2.0 * n + 2) * (n + al) * (2.0 * n + al - 2);
  A = (2.0 * n + al - 1) * (2.0 * n + al - 2) * (2.0 * n + al) / den;
  B = (2.0 * n + al - 1) * al * (al - 2) / den;
  C = -2.0 * (n - 1) * (n + al - 2) * (2.0 * n + al) / den;
}
template <class T>
GH1_HD void ija_scaled(double al, int n, T x, T y, T c, T* out) {
  double A, B, C;
  ija_coef(al, 1, A, B, C);
  T p1 = c * (A * x + B * y), p2 = c;
  T yy = y * y;
  for (int i = 0; i <= n; i++) {
    out[i] = p2;
    ija_coef(al, i + 2, A, B, C);
    T pn = (A * x + B * y) * p1 + (C * yy) * p2;
    p2 = p1;
    p1 = pn;
  }
}
template <class T>
GH1_HD void ija_plain(double al, int n, T x, T c, T* out) {
  double A, B, C;
  ija_coef(al, 1, A, B, C);
  T p1 = c * (A * x + B), p2 = c;
  for (int i = 0; i <= n; i++) {
    out[i] = p2;
    ija_coef(al, i + 2, A, B, C);
    T pn = (A * x + B) * p1 + C * p2;
    p2 = p1;
    p1 = pn;
  }
}

// ---- triangle / tet bubble bases ---------------------------------------------------
template <class T>
GH1_HD int dubiner2d_bub(int n, T x, T y, T t, T c, T* out) {
  T leg[MAX_TET_ORDER + 1];
  jac11_scaled<T>(n, y - (t - x - y), t - x, c, leg);
  int ii = 0;
  for (int i = 0; i <= n; i++) {
    ija_scaled<T>(4.0 + 2 * i, n - i, 2.0 * x - t, t, leg[i], out + ii);
    ii += n - i + 1;
  }
  return ii;
}
template <class T>
GH1_HD int dubiner3d_bub(int n, T x, T y, T z, T c, T* out) {
  T lam4 = 1.0 - x - y - z;
  T polz[MAX_TET_ORDER + 1], polsy[MAX_TET_ORDER + 1];
  jac11_scaled<T>(n, z - lam4, z + lam4, c, polz);
  int ii = 0;
  for (int k = 0; k <= n; k++) {
    ija_scaled<T>(4.0 + 2 * k, n - k, y - z - lam4, 1.0 - x, polz[k], polsy);
    for (int j = 0; j <= n - k; j++) {
      ija_plain<T>(6.0 + 2 * k + 2 * j, n - k - j, 2.0 * x - 1.0, polsy[j], out + ii);
      ii += n - k - j + 1;
    }
  }
  return ii;
}

// ---- reference topology (fem/elementtopology.hpp:1177-1265, :1610-1700) ------------
struct TetTopo {
  static GH1_HD int edge(int i, int j) {
    const int E[6][2] = {{3, 0}, {3, 1}, {3, 2}, {0, 1}, {0, 2}, {1, 2}};
    return E[i][j];
  }
  static GH1_HD int face(int i, int j) {
    const int F[4][3] = {{3, 1, 2}, {3, 2, 0}, {3, 0, 1}, {0, 2, 1}};
    return F[i][j];
  }
};
struct HexTopo {
  static GH1_HD int edge(int i, int j) {
    const int E[12][2] = {{0, 1}, {2, 3}, {3, 0}, {1, 2}, {4, 5}, {6, 7}, {7, 4}, {5, 6}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    return E[i][j];
  }
  static GH1_HD int face(int i, int j) {
    const int F[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
    return F[i][j];
  }
  // reference coordinates of the hex vertices (fem/elementtopology.cpp:112-119)
  static GH1_HD int coord(int v, int axis) {
    const int P[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    return P[v][axis];
  }
};

// tet shapes (H1HighOrderFE_Shape<ET_TET>::T_CalcShape) for vertex ranks vn[4]
template <class T>
GH1_HD int tet_shapes(int p, const int* vn, T x, T y, T z, T* sh) {
  T lam[4] = {x, y, z, 1.0 - x - y - z};
  for (int i = 0; i < 4; i++) sh[i] = lam[i];
  int ii = 4;
  if (p >= 2)
    for (int i = 0; i < 6; i++) {
      int e0 = TetTopo::edge(i, 0), e1 = TetTopo::edge(i, 1);
      if (vn[e0] > vn[e1]) { int t = e0; e0 = e1; e1 = t; }
      ilnb_scaled<T>(p - 2, lam[e1] - lam[e0], lam[e0] + lam[e1], lam[e0] * lam[e1], sh + ii);
      ii += p - 1;
    }
  if (p >= 3)
    for (int i = 0; i < 4; i++) {
      int f0 = TetTopo::face(i, 0), f1 = TetTopo::face(i, 1), f2 = TetTopo::face(i, 2), t;
      if (vn[f0] > vn[f1]) { t = f0; f0 = f1; f1 = t; }
      if (vn[f1] > vn[f2]) { t = f1; f1 = f2; f2 = t; }
      if (vn[f0] > vn[f1]) { t = f0; f0 = f1; f1 = t; }
      int vop = 6 - f0 - f1 - f2;
      dubiner2d_bub<T>(p - 3, lam[f0], lam[f1], 1.0 - lam[vop], lam[f0] * lam[f1] * lam[f2], sh + ii);
      ii += (p - 2) * (p - 1) / 2;
    }
  if (p >= 4) {
    dubiner3d_bub<T>(p - 4, lam[0], lam[1], lam[2], lam[0] * lam[1] * lam[2] * lam[3], sh + ii);
    ii += (p - 1) * (p - 2) * (p - 3) / 6;
  }
  return ii;
}

// 1D hex factor functions on [0,1]:  psi_0 = 1-x, psi_1 = x,
// psi_{k+2} = x(1-x) P_k(2x-1)   (P_k = IntLegNoBubble).
// Every hex shape of h1hofe_impl.hpp:821-890 is +-psi_a(x) psi_b(y) psi_c(z).
template <class T>
GH1_HD void hex_psi(int p, T x, T* out) {
  out[0] = 1.0 - x;
  out[1] = x;
  if (p >= 2) ilnb_scaled<T>(p - 2, 2.0 * x - 1.0, T(1.0), x * (1.0 - x), out + 2);
}

// Full hex shape set in reference order (used for element-level checks):
template <class T>
GH1_HD int hex_shapes(int p, const int* vn, T x, T y, T z, T* sh) {
  T lam[8] = {(1.0 - x) * (1.0 - y) * (1.0 - z), x * (1.0 - y) * (1.0 - z), x * y * (1.0 - z), (1.0 - x) * y * (1.0 - z),
              (1.0 - x) * (1.0 - y) * z, x * (1.0 - y) * z, x * y * z, (1.0 - x) * y * z};
  T sigma[8] = {(1.0 - x) + (1.0 - y) + (1.0 - z), x + (1.0 - y) + (1.0 - z), x + y + (1.0 - z), (1.0 - x) + y + (1.0 - z),
                (1.0 - x) + (1.0 - y) + z, x + (1.0 - y) + z, x + y + z, (1.0 - x) + y + z};
  for (int i = 0; i < 8; i++) sh[i] = lam[i];
  int ii = 8;
  if (p < 2) return ii;
  T polx[MAX_HEX_ORDER + 1], poly[MAX_HEX_ORDER + 1], polz[MAX_HEX_ORDER + 1];
  for (int i = 0; i < 12; i++) {
    int e0 = HexTopo::edge(i, 0), e1 = HexTopo::edge(i, 1);
    if (vn[e0] > vn[e1]) { int t = e0; e0 = e1; e1 = t; }
    T xi = sigma[e1] - sigma[e0];
    T lam_e = lam[e0] + lam[e1];
    T bub = 0.25 * lam_e * (1.0 - xi * xi);
    ilnb_scaled<T>(p - 2, xi, T(1.0), bub, sh + ii);
    ii += p - 1;
  }
  for (int i = 0; i < 6; i++) {
    int f[4] = {HexTopo::face(i, 0), HexTopo::face(i, 1), HexTopo::face(i, 2), HexTopo::face(i, 3)};
    int fmin = 0;
    for (int j = 1; j < 4; j++) if (vn[f[j]] < vn[f[fmin]]) fmin = j;
    int j1 = (fmin + 3) % 4, j2 = (fmin + 1) % 4, jop = (fmin + 2) % 4;
    if (vn[f[j2]] < vn[f[j1]]) { int t = j1; j1 = j2; j2 = t; }
    int g0 = f[fmin], g1 = f[j1], g2 = f[jop], g3 = f[j2];
    T lam_f = lam[g0] + lam[g1] + lam[g2] + lam[g3];
    T xi = sigma[g0] - sigma[g1];
    T eta = sigma[g0] - sigma[g3];
    T bub = (1.0 / 16) * (1.0 - xi * xi) * (1.0 - eta * eta) * lam_f;
    ilnb_scaled<T>(p - 2, xi, T(1.0), bub, polx);
    ilnb_scaled<T>(p - 2, eta, T(1.0), T(1.0), poly);
    for (int k = 0; k < p - 1; k++)
      for (int j = 0; j < p - 1; j++) sh[ii++] = polx[k] * poly[j];
  }
  ilnb_scaled<T>(p - 2, 2.0 * x - 1.0, T(1.0), x * (1.0 - x), polx);
  ilnb_scaled<T>(p - 2, 2.0 * y - 1.0, T(1.0), y * (1.0 - y), poly);
  ilnb_scaled<T>(p - 2, 2.0 * z - 1.0, T(1.0), z * (1.0 - z), polz);
  for (int i = 0; i < p - 1; i++)
    for (int j = 0; j < p - 1; j++) {
      T pxy = polx[i] * poly[j];
      for (int k = 0; k < p - 1; k++) sh[ii++] = pxy * polz[k];
    }
  return ii;
}

}  // namespace gh1
