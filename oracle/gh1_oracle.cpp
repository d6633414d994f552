// gh1_oracle.cpp -- CPU restatement (FP64, OpenMP) of NGSolve's high-order H1
// Poisson path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check
// and the CPU-baseline leg of the benchmark load this library to compare with.
// Nothing in the GPU product links or calls it.
//
// Every routine names the reference file:line whose algorithm it restates
// (paths are relative to the NGSolve source tree).
//
// Parity pins: P1 tet mass entry of tests/pytest/test_matrix.py:57-93 on the
// tests/pytest/cube.vol.gz mesh (see tests/golden), p-exactness (Q_p on hexes,
// P_p on tets), orthogonality norms of the Dubiner bubble bases
// (fem/recursive_pol.hpp:2864-2874, :3011-3023).  Global edge/face numbering
// comes from netgen in the reference; here it is the documented rule
// "edges/faces sorted by their sorted global vertex tuples", which the GPU
// library follows as well.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <array>
#include <algorithm>
#include <numeric>
#include <omp.h>

namespace {

// ---------------------------------------------------------------------------
// forward-mode AD with 3 directional derivatives (role of ngcore AutoDiff<3>)
struct AD {
  double v, d[3];
  AD() : v(0), d{0, 0, 0} {}
  AD(double a) : v(a), d{0, 0, 0} {}
  static AD var(double a, int k) { AD r(a); r.d[k] = 1; return r; }
};
inline AD operator+(const AD& a, const AD& b) { AD r; r.v = a.v + b.v; for (int k = 0; k < 3; k++) r.d[k] = a.d[k] + b.d[k]; return r; }
inline AD operator-(const AD& a, const AD& b) { AD r; r.v = a.v - b.v; for (int k = 0; k < 3; k++) r.d[k] = a.d[k] - b.d[k]; return r; }
inline AD operator*(const AD& a, const AD& b) { AD r; r.v = a.v * b.v; for (int k = 0; k < 3; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r; }
inline AD operator+(const AD& a, double b) { AD r = a; r.v += b; return r; }
inline AD operator+(double b, const AD& a) { return a + b; }
inline AD operator-(const AD& a, double b) { AD r = a; r.v -= b; return r; }
inline AD operator-(double b, const AD& a) { AD r; r.v = b - a.v; for (int k = 0; k < 3; k++) r.d[k] = -a.d[k]; return r; }
inline AD operator*(const AD& a, double b) { AD r; r.v = a.v * b; for (int k = 0; k < 3; k++) r.d[k] = a.d[k] * b; return r; }
inline AD operator*(double b, const AD& a) { return a * b; }

// ---------------------------------------------------------------------------
// Recursive polynomials (fem/recursive_pol.hpp)

// IntLegNoBubble: P0=-1/2, P1=-x/2, P_k = A_k x P_{k-1} + C_k y^2 P_{k-2},
// A_k=(2(k+2)-3)/(k+2), C_k=-((k+2)-3)/(k+2)   (recursive_pol.hpp:1344-1377,
// evaluation loops :477-495 and :603-620; coefficient table recursive_pol.cpp:40-62)
template <class T>
void intleg_nobub_scaled_mult(int n, T x, T y, T c, T* out) {
  if (n < 0) return;
  T p0 = c * (-0.5), p1 = c * (-0.5) * x;
  out[0] = p0;
  if (n >= 1) out[1] = p1;
  T yy = y * y;
  for (int k = 2; k <= n; k++) {
    double A = (2.0 * (k + 2) - 3) / (k + 2), C = -((k + 2) - 3.0) / (k + 2);
    T pn = A * x * p1 + C * yy * p0;
    p0 = p1; p1 = pn; out[k] = pn;
  }
}
template <class T>
void intleg_nobub_mult(int n, T x, T c, T* out) { intleg_nobub_scaled_mult<T>(n, x, T(1.0), c, out); }

// JacobiPolynomialFix<1,1> (recursive_pol.hpp:1641-1676), scaled, "1Assign" loop (:648-660):
// P0=1, P1(x,y)=2x, P_k = (A_k x + B_k y) P_{k-1} + C_k y^2 P_{k-2}, B_k = 0 for al=be.
inline double jac11_A(int i) { i--; const double al = 1, be = 1; return (2.0 * i + al + be) * (2 * i + al + be + 1) * (2 * i + al + be + 2) / (2 * (i + 1) * (i + al + be + 1) * (2 * i + al + be)); }
inline double jac11_C(int i) { i--; const double al = 1, be = 1; return -2.0 * (i + al) * (i + be) * (2 * i + al + be + 2) / (2 * (i + 1) * (i + al + be + 1) * (2 * i + al + be)); }
template <class T>
void jac11_scaled_mult(int n, T x, T y, T c, T* out) {
  T p2 = c, p1 = c * (2.0 * x);
  T yy = y * y;
  for (int i = 0; i <= n; i++) {
    out[i] = p2;
    int k = i + 2;
    T pn = jac11_A(k) * x * p1 + jac11_C(k) * yy * p2;
    p2 = p1; p1 = pn;
  }
}

// IntegratedJacobiPolynomialAlpha (recursive_pol.hpp:1857-1917, coefficients
// recursive_pol.cpp:126-155): index-1 coefficients are 0.25(a+2), 0.25(a-2), 0.
struct IntJacAlpha {
  double al;
  explicit IntJacAlpha(int a) : al(a) {}
  double A(int n) const { if (n == 1) return 0.25 * (al + 2); return (2.0 * n + al - 1) * (2 * n + al - 2) * (2 * n + al) / ((2 * n + 2) * (n + al) * (2 * n + al - 2)); }
  double B(int n) const { if (n == 1) return 0.25 * (al - 2); return (2.0 * n + al - 1) * al * (al - 2) / ((2 * n + 2) * (n + al) * (2 * n + al - 2)); }
  double C(int n) const { if (n == 1) return 0.0; return -2.0 * (n - 1) * (n + al - 2) * (2 * n + al) / ((2 * n + 2) * (n + al) * (2 * n + al - 2)); }
  // EvalScaledMult1Assign (recursive_pol.hpp:1196-1212 with EvalScaledNext2 :903-922)
  template <class T> void scaled_mult(int n, T x, T y, T c, T* out) const {
    T p1 = c * (A(1) * x + B(1) * y), p2 = c;
    T yy = y * y;
    for (int i = 0; i <= n; i++) {
      out[i] = p2;
      int k = i + 2;
      T pn = (A(k) * x + B(k) * y) * p1 + C(k) * yy * p2;
      p2 = p1; p1 = pn;
    }
  }
  // EvalMult1Assign (recursive_pol.hpp:1120-1134 with EvalNext2 :763-781)
  template <class T> void mult(int n, T x, T c, T* out) const {
    T p1 = c * (A(1) * x + B(1)), p2 = c;
    for (int i = 0; i <= n; i++) {
      out[i] = p2;
      int k = i + 2;
      T pn = (A(k) * x + B(k)) * p1 + C(k) * p2;
      p2 = p1; p1 = pn;
    }
  }
};

// DubinerBasisOrthoBub::EvalScaledMult (recursive_pol.hpp:2847-2860)
template <class T>
int dubiner_orthobub_scaled_mult(int n, T x, T y, T t, T c, T* out) {
  std::vector<T> leg(n + 1);
  jac11_scaled_mult<T>(n, y - (t - x - y), t - x, c, leg.data());
  int ii = 0;
  for (int i = 0; i <= n; i++) {
    IntJacAlpha jac(4 + 2 * i);
    jac.scaled_mult<T>(n - i, 2.0 * x - t, t, leg[i], out + ii);
    ii += n - i + 1;
  }
  return ii;
}

// DubinerBasis3DOrthoBub::EvalMult (recursive_pol.hpp:2979-3008)
template <class T>
int dubiner3d_orthobub_mult(int n, T x, T y, T z, T c, T* out) {
  T lam4 = 1.0 - x - y - z;
  std::vector<T> polz(n + 1), polsy(n + 1);
  jac11_scaled_mult<T>(n, z - lam4, z + lam4, c, polz.data());
  int ii = 0;
  for (int k = 0; k <= n; k++) {
    IntJacAlpha jac1(4 + 2 * k);
    jac1.scaled_mult<T>(n - k, y - z - lam4, 1.0 - x, polz[k], polsy.data());
    for (int j = 0; j <= n - k; j++) {
      IntJacAlpha jac2(6 + 2 * k + 2 * j);
      jac2.mult<T>(n - k - j, 2.0 * x - 1.0, polsy[j], out + ii);
      ii += n - k - j + 1;
    }
  }
  return ii;
}

// ---------------------------------------------------------------------------
// Reference topology (fem/elementtopology.hpp:1177-1265 tet, :1610-1700 hex)
const int TET_EDGES[6][2] = {{3, 0}, {3, 1}, {3, 2}, {0, 1}, {0, 2}, {1, 2}};
const int TET_FACES[4][3] = {{3, 1, 2}, {3, 2, 0}, {3, 0, 1}, {0, 2, 1}};
const int HEX_EDGES[12][2] = {{0, 1}, {2, 3}, {3, 0}, {1, 2}, {4, 5}, {6, 7}, {7, 4}, {5, 6}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int HEX_FACES[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};

// GetEdgeSort (elementtopology.hpp:1208-1214 / :1645-1650)
inline void edge_sort(const int* e, const int* vn, int* out) {
  out[0] = e[0]; out[1] = e[1];
  if (vn[out[0]] > vn[out[1]]) std::swap(out[0], out[1]);
}
// tet GetFaceSort (elementtopology.hpp:1228-1236)
inline void tet_face_sort(const int* f, const int* vn, int* o) {
  o[0] = f[0]; o[1] = f[1]; o[2] = f[2];
  if (vn[o[0]] > vn[o[1]]) std::swap(o[0], o[1]);
  if (vn[o[1]] > vn[o[2]]) std::swap(o[1], o[2]);
  if (vn[o[0]] > vn[o[1]]) std::swap(o[0], o[1]);
}
// hex GetFaceSort (elementtopology.hpp:1674-1689)
inline void hex_face_sort(const int* f, const int* vn, int* o) {
  int fmin = 0;
  for (int j = 1; j < 4; j++) if (vn[f[j]] < vn[f[fmin]]) fmin = j;
  int f1 = (fmin + 3) % 4, f2 = (fmin + 1) % 4, fop = (fmin + 2) % 4;
  if (vn[f[f2]] < vn[f[f1]]) std::swap(f1, f2);
  o[0] = f[fmin]; o[1] = f[f1]; o[2] = f[fop]; o[3] = f[f2];
}

// ---------------------------------------------------------------------------
// Shapes.  H1HighOrderFE_Shape<ET_TET>::T_CalcShape (fem/h1hofe_impl.hpp:509-577)
template <class T>
int tet_shape(int p, const int* vn, T x, T y, T z, T* sh) {
  T lam[4] = {x, y, z, 1.0 - x - y - z};
  for (int i = 0; i < 4; i++) sh[i] = lam[i];
  int ii = 4;
  if (p >= 2)
    for (int i = 0; i < 6; i++) {
      int e[2]; edge_sort(TET_EDGES[i], vn, e);
      intleg_nobub_scaled_mult<T>(p - 2, lam[e[1]] - lam[e[0]], lam[e[0]] + lam[e[1]], lam[e[0]] * lam[e[1]], sh + ii);
      ii += p - 1;
    }
  if (p >= 3)
    for (int i = 0; i < 4; i++) {
      int f[3]; tet_face_sort(TET_FACES[i], vn, f);
      int vop = 6 - f[0] - f[1] - f[2];
      dubiner_orthobub_scaled_mult<T>(p - 3, lam[f[0]], lam[f[1]], 1.0 - lam[vop], lam[f[0]] * lam[f[1]] * lam[f[2]], sh + ii);
      ii += (p - 2) * (p - 1) / 2;
    }
  if (p >= 4) {
    dubiner3d_orthobub_mult<T>(p - 4, lam[0], lam[1], lam[2], lam[0] * lam[1] * lam[2] * lam[3], sh + ii);
    ii += (p - 1) * (p - 2) * (p - 3) / 6;
  }
  return ii;
}

// H1HighOrderFE_Shape<ET_HEX>::T_CalcShape (fem/h1hofe_impl.hpp:821-890)
template <class T>
int hex_shape(int p, const int* vn, T x, T y, T z, T* sh) {
  T lam[8] = {(1.0 - x) * (1.0 - y) * (1.0 - z), x * (1.0 - y) * (1.0 - z), x * y * (1.0 - z), (1.0 - x) * y * (1.0 - z),
              (1.0 - x) * (1.0 - y) * z, x * (1.0 - y) * z, x * y * z, (1.0 - x) * y * z};
  T sigma[8] = {(1.0 - x) + (1.0 - y) + (1.0 - z), x + (1.0 - y) + (1.0 - z), x + y + (1.0 - z), (1.0 - x) + y + (1.0 - z),
                (1.0 - x) + (1.0 - y) + z, x + (1.0 - y) + z, x + y + z, (1.0 - x) + y + z};
  for (int i = 0; i < 8; i++) sh[i] = lam[i];
  int ii = 8;
  if (p < 2) return ii;
  std::vector<T> polx(p + 1), poly(p + 1), polz(p + 1);
  for (int i = 0; i < 12; i++) {
    int e[2]; edge_sort(HEX_EDGES[i], vn, e);
    T xi = sigma[e[1]] - sigma[e[0]];
    T lam_e = lam[e[0]] + lam[e[1]];
    T bub = 0.25 * lam_e * (1.0 - xi * xi);
    intleg_nobub_mult<T>(p - 2, xi, bub, sh + ii);
    ii += p - 1;
  }
  for (int i = 0; i < 6; i++) {
    int f[4]; hex_face_sort(HEX_FACES[i], vn, f);
    T lam_f(0.0);
    for (int j = 0; j < 4; j++) lam_f = lam_f + lam[f[j]];
    T xi = sigma[f[0]] - sigma[f[1]];
    T eta = sigma[f[0]] - sigma[f[3]];
    T bub = (1.0 / 16) * (1.0 - xi * xi) * (1.0 - eta * eta) * lam_f;
    intleg_nobub_mult<T>(p - 2, xi, bub, polx.data());
    intleg_nobub_mult<T>(p - 2, eta, T(1.0), poly.data());
    for (int k = 0; k < p - 1; k++)
      for (int j = 0; j < p - 1; j++) sh[ii++] = polx[k] * poly[j];
  }
  intleg_nobub_mult<T>(p - 2, 2.0 * x - 1.0, x * (1.0 - x), polx.data());
  intleg_nobub_mult<T>(p - 2, 2.0 * y - 1.0, y * (1.0 - y), poly.data());
  intleg_nobub_mult<T>(p - 2, 2.0 * z - 1.0, z * (1.0 - z), polz.data());
  for (int i = 0; i < p - 1; i++)
    for (int j = 0; j < p - 1; j++) {
      T pxy = polx[i] * poly[j];
      for (int k = 0; k < p - 1; k++) sh[ii++] = pxy * polz[k];
    }
  return ii;
}

inline int nloc_of(int et, int p) {
  if (et == 4) return (p + 1) * (p + 2) * (p + 3) / 6;
  return (p + 1) * (p + 1) * (p + 1);
}

// ---------------------------------------------------------------------------
// Integration rules
// ComputeGaussRule (fem/intrule.cpp:700-740): Gauss-Legendre on (0,1), Newton on P_n
void gauss_rule(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0); w.assign(n, 0);
  int m = (n + 1) / 2;
  for (int i = 1; i <= m; i++) {
    double z = std::cos(M_PI * (i - 0.25) / (n + 0.5)), z1, pp, p1, p2, p3;
    for (int it = 0; it < 100; it++) {
      p1 = 1; p2 = 0;
      for (int j = 1; j <= n; j++) { p3 = p2; p2 = p1; p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j; }
      pp = n * (z * p1 - p2) / (z * z - 1);
      z1 = z; z = z1 - p1 / pp;
      if (std::fabs(z - z1) < 1e-15) break;
    }
    p1 = 1; p2 = 0;
    for (int j = 1; j <= n; j++) { p3 = p2; p2 = p1; p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j; }
    pp = n * (z * p1 - p2) / (z * z - 1);
    x[i - 1] = 0.5 * (1 - z); x[n - i] = 0.5 * (1 + z);
    w[i - 1] = w[n - i] = 1.0 / ((1 - z * z) * pp * pp);
  }
}

struct Rule { std::vector<double> x, y, z, w; int size() const { return (int)w.size(); } };

// hex: tensor Gauss with order/2+1 points (fem/intrule.cpp:3118-3132, :3234-3263)
Rule hex_rule(int order) {
  std::vector<double> g, gw; gauss_rule(order / 2 + 1, g, gw);
  Rule r; int n = (int)g.size();
  for (int i = 0; i < n; i++) for (int j = 0; j < n; j++) for (int l = 0; l < n; l++) {
    r.x.push_back(g[i]); r.y.push_back(g[j]); r.z.push_back(g[l]); r.w.push_back(gw[i] * gw[j] * gw[l]);
  }
  return r;
}
// tet: collapsed (Duffy) tensor rule (the construction of fem/intrule.cpp:3190-3226),
// here with Gauss-Legendre factors and the collapse Jacobian (1-x)^2(1-y) in the
// weights; n = order/2+2 points per direction integrates degree `order` exactly.
// The reference tabulates symmetric rules for order <= 6; on affine tets every rule
// that is exact for the integrand's degree gives the same element matrices.
Rule tet_rule(int order) {
  int n = order / 2 + 2;
  std::vector<double> g, gw; gauss_rule(n, g, gw);
  Rule r;
  for (int k = 0; k < n; k++) for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
    double xx = g[i], yy = g[j], zz = g[k];
    r.x.push_back(xx); r.y.push_back(yy * (1 - xx)); r.z.push_back(zz * (1 - xx) * (1 - yy));
    r.w.push_back(gw[i] * gw[j] * gw[k] * (1 - xx) * (1 - xx) * (1 - yy));
  }
  return r;
}

// ---------------------------------------------------------------------------
// Space: topology + DOF tables
struct Space {
  int et = 8, nvert = 8, nedge = 12, nface = 6;  // per element
  int p = 1, nv = 0, ne = 0, ned = 0, nfa = 0, nloc = 0;
  long ndof = 0;
  std::vector<double> X;       // nv*3
  std::vector<int> el;         // ne*nvert
  std::vector<int> el_edges, el_faces;  // global ids per element (local order)
  std::vector<std::array<int, 2>> edges;  // vertex pair of each global edge
  // deformation (MeshAccess::SetDeformation): a field in the H1 space `def` of
  // the same mesh, [3][def->ndof] component-major
  const struct Space* def = nullptr;
  std::vector<double> defvec;
  std::vector<long> edofs;     // ne*nloc (as long for safety)
  std::vector<unsigned char> freedof;
  // Dirichlet on these boundary faces only (sorted vertex numbers, padded with
  // INT32_MAX) when dir_select; dir_bad set if one is not a boundary face
  bool dir_select = false, dir_bad = false;
  std::vector<std::array<int, 4>> dir_faces;
  int n_edge_dofs = 0, n_face_dofs = 0, n_cell_dofs = 0;
  long first_edge = 0, first_face = 0, first_cell = 0;
  // CSR
  std::vector<long> rowptr; std::vector<int> colind;
};

void build_space(Space& S) {
  const bool tet = S.et == 4;
  S.nvert = tet ? 4 : 8; S.nedge = tet ? 6 : 12; S.nface = tet ? 4 : 6;
  const int fv = tet ? 3 : 4;
  // edges: unique sorted (min,max) pairs, numbered in lexicographic order
  std::vector<std::array<int, 2>> E; E.reserve((size_t)S.ne * S.nedge);
  for (int e = 0; e < S.ne; e++)
    for (int i = 0; i < S.nedge; i++) {
      int a = S.el[(size_t)e * S.nvert + (tet ? TET_EDGES[i][0] : HEX_EDGES[i][0])];
      int b = S.el[(size_t)e * S.nvert + (tet ? TET_EDGES[i][1] : HEX_EDGES[i][1])];
      E.push_back({std::min(a, b), std::max(a, b)});
    }
  std::vector<std::array<int, 2>> Eu = E;
  std::sort(Eu.begin(), Eu.end()); Eu.erase(std::unique(Eu.begin(), Eu.end()), Eu.end());
  S.ned = (int)Eu.size();
  S.edges = Eu;
  S.el_edges.resize(E.size());
  for (size_t k = 0; k < E.size(); k++) S.el_edges[k] = int(std::lower_bound(Eu.begin(), Eu.end(), E[k]) - Eu.begin());
  // faces: unique sorted vertex tuples, numbered in lexicographic order
  std::vector<std::array<int, 4>> F; F.reserve((size_t)S.ne * S.nface);
  for (int e = 0; e < S.ne; e++)
    for (int i = 0; i < S.nface; i++) {
      std::array<int, 4> t{INT32_MAX, INT32_MAX, INT32_MAX, INT32_MAX};
      for (int j = 0; j < fv; j++) t[j] = S.el[(size_t)e * S.nvert + (tet ? TET_FACES[i][j] : HEX_FACES[i][j])];
      std::sort(t.begin(), t.begin() + fv);
      F.push_back(t);
    }
  std::vector<std::array<int, 4>> Fu = F;
  std::sort(Fu.begin(), Fu.end()); Fu.erase(std::unique(Fu.begin(), Fu.end()), Fu.end());
  S.nfa = (int)Fu.size();
  S.el_faces.resize(F.size());
  std::vector<int> face_count(S.nfa, 0);
  for (size_t k = 0; k < F.size(); k++) { S.el_faces[k] = int(std::lower_bound(Fu.begin(), Fu.end(), F[k]) - Fu.begin()); face_count[S.el_faces[k]]++; }
  // DOF counts (comp/h1hofespace.cpp:823-950, uniform order p)
  const int p = S.p;
  S.n_edge_dofs = p > 1 ? p - 1 : 0;
  S.n_face_dofs = tet ? (p > 2 ? (p - 1) * (p - 2) / 2 : 0) : (p > 1 ? (p - 1) * (p - 1) : 0);
  S.n_cell_dofs = tet ? (p > 3 ? (p - 1) * (p - 2) * (p - 3) / 6 : 0) : (p > 1 ? (p - 1) * (p - 1) * (p - 1) : 0);
  S.first_edge = S.nv;
  S.first_face = S.first_edge + (long)S.ned * S.n_edge_dofs;
  S.first_cell = S.first_face + (long)S.nfa * S.n_face_dofs;
  S.ndof = S.first_cell + (long)S.ne * S.n_cell_dofs;
  S.nloc = nloc_of(S.et, p);
  // element DOFs (GetDofNrs, comp/h1hofespace.cpp:1389-1420)
  S.edofs.assign((size_t)S.ne * S.nloc, 0);
  for (int e = 0; e < S.ne; e++) {
    long* d = &S.edofs[(size_t)e * S.nloc]; int ii = 0;
    for (int i = 0; i < S.nvert; i++) d[ii++] = S.el[(size_t)e * S.nvert + i];
    for (int i = 0; i < S.nedge; i++) for (int k = 0; k < S.n_edge_dofs; k++) d[ii++] = S.first_edge + (long)S.el_edges[(size_t)e * S.nedge + i] * S.n_edge_dofs + k;
    for (int i = 0; i < S.nface; i++) for (int k = 0; k < S.n_face_dofs; k++) d[ii++] = S.first_face + (long)S.el_faces[(size_t)e * S.nface + i] * S.n_face_dofs + k;
    for (int k = 0; k < S.n_cell_dofs; k++) d[ii++] = S.first_cell + (long)e * S.n_cell_dofs + k;
  }
  // Dirichlet boundary (comp/fespace.cpp:440-516, :765-830): the boundary
  // faces (one adjacent element), or those of them the dirichlet regex
  // selected; DOFs of these faces and of their edges and vertices are not free.
  std::vector<char> dir(S.nfa, 0);
  for (int f = 0; f < S.nfa; f++) dir[f] = !S.dir_select && face_count[f] == 1;
  for (const auto& t : S.dir_faces) {
    auto it = std::lower_bound(Fu.begin(), Fu.end(), t);
    if (it == Fu.end() || *it != t || face_count[it - Fu.begin()] != 1) { S.dir_bad = true; continue; }
    dir[it - Fu.begin()] = 1;
  }
  S.freedof.assign(S.ndof, 1);
  for (int e = 0; e < S.ne; e++)
    for (int i = 0; i < S.nface; i++) {
      int f = S.el_faces[(size_t)e * S.nface + i];
      if (!dir[f]) continue;
      for (int k = 0; k < S.n_face_dofs; k++) S.freedof[S.first_face + (long)f * S.n_face_dofs + k] = 0;
      const int* lf = tet ? TET_FACES[i] : HEX_FACES[i];
      for (int j = 0; j < fv; j++) S.freedof[S.el[(size_t)e * S.nvert + lf[j]]] = 0;
      for (int j = 0; j < fv; j++) {
        int a = S.el[(size_t)e * S.nvert + lf[j]], b = S.el[(size_t)e * S.nvert + lf[(j + 1) % fv]];
        // the local edge with these two vertices
        for (int ie = 0; ie < S.nedge; ie++) {
          int ea = S.el[(size_t)e * S.nvert + (tet ? TET_EDGES[ie][0] : HEX_EDGES[ie][0])];
          int eb = S.el[(size_t)e * S.nvert + (tet ? TET_EDGES[ie][1] : HEX_EDGES[ie][1])];
          if ((ea == a && eb == b) || (ea == b && eb == a)) {
            int ge = S.el_edges[(size_t)e * S.nedge + ie];
            for (int k = 0; k < S.n_edge_dofs; k++) S.freedof[S.first_edge + (long)ge * S.n_edge_dofs + k] = 0;
          }
        }
      }
    }
}

// ---------------------------------------------------------------------------
// Element geometry
struct Geo { double J[9], Jinv[9], det; };
inline void invert3(const double* J, double* Ji, double& det) {
  det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) + J[2] * (J[3] * J[7] - J[4] * J[6]);
  double id = 1.0 / det;
  Ji[0] = (J[4] * J[8] - J[5] * J[7]) * id; Ji[1] = (J[2] * J[7] - J[1] * J[8]) * id; Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
  Ji[3] = (J[5] * J[6] - J[3] * J[8]) * id; Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id; Ji[5] = (J[2] * J[3] - J[0] * J[5]) * id;
  Ji[6] = (J[3] * J[7] - J[4] * J[6]) * id; Ji[7] = (J[1] * J[6] - J[0] * J[7]) * id; Ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
}
// tet: x = v3 + sum_j (v_j - v3) xi_j  (comp/meshaccess.cpp:541-552)
// hex: trilinear map from the 8 vertices with the hex vertex functions of
// h1hofe_impl.hpp:826-827 (netgen's own element map is not in the tree).
void add_deformation(const Space& S, int e, double x, double y, double z, double* J);
Geo geometry(const Space& S, int e, double x, double y, double z) {
  Geo g; const int* v = &S.el[(size_t)e * S.nvert];
  if (S.et == 4) {
    const double* p3 = &S.X[3 * (size_t)v[3]];
    for (int j = 0; j < 3; j++) { const double* pj = &S.X[3 * (size_t)v[j]]; for (int k = 0; k < 3; k++) g.J[3 * k + j] = pj[k] - p3[k]; }
  } else {
    double dl[8][3] = {
      {-(1 - y) * (1 - z), -(1 - x) * (1 - z), -(1 - x) * (1 - y)}, {(1 - y) * (1 - z), -x * (1 - z), -x * (1 - y)},
      {y * (1 - z), x * (1 - z), -x * y}, {-y * (1 - z), (1 - x) * (1 - z), -(1 - x) * y},
      {-(1 - y) * z, -(1 - x) * z, (1 - x) * (1 - y)}, {(1 - y) * z, -x * z, x * (1 - y)},
      {y * z, x * z, x * y}, {-y * z, (1 - x) * z, (1 - x) * y}};
    for (int i = 0; i < 9; i++) g.J[i] = 0;
    for (int a = 0; a < 8; a++) { const double* pa = &S.X[3 * (size_t)v[a]]; for (int k = 0; k < 3; k++) for (int j = 0; j < 3; j++) g.J[3 * k + j] += pa[k] * dl[a][j]; }
  }
  add_deformation(S, e, x, y, z, g.J);
  invert3(g.J, g.Jinv, g.det);
  return g;
}

int shape_ad(const Space& S, int e, double x, double y, double z, AD* sh) {
  const int* vn = &S.el[(size_t)e * S.nvert];
  AD X = AD::var(x, 0), Y = AD::var(y, 1), Z = AD::var(z, 2);
  return S.et == 4 ? tet_shape<AD>(S.p, vn, X, Y, Z, sh) : hex_shape<AD>(S.p, vn, X, Y, Z, sh);
}

// ALE_ElementTransformation::CalcJacobian (comp/meshaccess.cpp:318-330): the
// mesh Jacobian plus the reference gradient of the deformation field
void add_deformation(const Space& S, int e, double x, double y, double z, double* J) {
  if (!S.def) return;
  const Space& D = *S.def;
  std::vector<AD> sh(D.nloc);
  shape_ad(D, e, x, y, z, sh.data());
  const long* dn = &D.edofs[(size_t)e * D.nloc];
  for (int i = 0; i < D.nloc; i++)
    for (int r = 0; r < 3; r++) {
      const double dr = S.defvec[(size_t)r * D.ndof + dn[i]];
      for (int c = 0; c < 3; c++) J[3 * r + c] += dr * sh[i].d[c];
    }
}

Rule bilinear_rule(const Space& S) {
  // SymbolicBFI::GetIntegrationRule (fem/symbolicintegrator.cpp:1433-1455)
  return S.et == 4 ? tet_rule(2 * S.p - 2 > 0 ? 2 * S.p - 2 : 0) : hex_rule(2 * S.p);
}
Rule mass_rule(const Space& S) { return S.et == 4 ? tet_rule(2 * S.p) : hex_rule(2 * S.p); }

// Symmetric 3x3 tensor from its components (xx yy zz xy xz yz), row-major.
inline void tensor33(const double* k6, double* k) {
  k[0] = k6[0]; k[1] = k6[3]; k[2] = k6[4];
  k[3] = k6[3]; k[4] = k6[1]; k[5] = k6[5];
  k[6] = k6[4]; k[7] = k6[5]; k[8] = k6[2];
}

// element matrix of  kappa grad u.grad v + mu u v
// (T_CalcElementMatrixAdd, fem/symbolicintegrator.cpp:1548-1830: B^T diag(w|detJ| c) B)
// reverse != 0 sums the quadrature points in the opposite order: the difference
// between the two orders measures the rounding noise of the algorithm itself.
// k6 != NULL: the diffusion term is (K grad u).grad v with the element's
// symmetric tensor K = k6 (xx yy zz xy xz yz) in place of kappa (the D matrix
// of B^T D B is then w|detJ| K instead of w|detJ| kappa I).
void element_matrix(const Space& S, int e, double kappa, double mu, std::vector<double>& K, int reverse = 0,
                    const double* k6 = nullptr) {
  const int n = S.nloc;
  K.assign((size_t)n * n, 0.0);
  std::vector<AD> sh(n);
  std::vector<double> gx(n), gy(n), gz(n);
  if (k6) {
    double kt[9];
    tensor33(k6, kt);
    Rule r = bilinear_rule(S);
    std::vector<double> fx(n), fy(n), fz(n);
    for (int qq = 0; qq < r.size(); qq++) {
      const int q = reverse ? r.size() - 1 - qq : qq;
      shape_ad(S, e, r.x[q], r.y[q], r.z[q], sh.data());
      Geo g = geometry(S, e, r.x[q], r.y[q], r.z[q]);
      double fac = r.w[q] * std::fabs(g.det);
      for (int i = 0; i < n; i++) {  // mapped gradient J^{-T} grad_ref, and the flux K * it
        gx[i] = g.Jinv[0] * sh[i].d[0] + g.Jinv[3] * sh[i].d[1] + g.Jinv[6] * sh[i].d[2];
        gy[i] = g.Jinv[1] * sh[i].d[0] + g.Jinv[4] * sh[i].d[1] + g.Jinv[7] * sh[i].d[2];
        gz[i] = g.Jinv[2] * sh[i].d[0] + g.Jinv[5] * sh[i].d[1] + g.Jinv[8] * sh[i].d[2];
        fx[i] = kt[0] * gx[i] + kt[1] * gy[i] + kt[2] * gz[i];
        fy[i] = kt[3] * gx[i] + kt[4] * gy[i] + kt[5] * gz[i];
        fz[i] = kt[6] * gx[i] + kt[7] * gy[i] + kt[8] * gz[i];
      }
      for (int i = 0; i < n; i++) for (int j = 0; j < n; j++)
        K[(size_t)i * n + j] += fac * (gx[i] * fx[j] + gy[i] * fy[j] + gz[i] * fz[j]);
    }
  } else if (kappa != 0.0) {
    Rule r = bilinear_rule(S);
    for (int qq = 0; qq < r.size(); qq++) {
      const int q = reverse ? r.size() - 1 - qq : qq;
      shape_ad(S, e, r.x[q], r.y[q], r.z[q], sh.data());
      Geo g = geometry(S, e, r.x[q], r.y[q], r.z[q]);
      double fac = kappa * r.w[q] * std::fabs(g.det);
      for (int i = 0; i < n; i++) {  // mapped gradient J^{-T} grad_ref
        gx[i] = g.Jinv[0] * sh[i].d[0] + g.Jinv[3] * sh[i].d[1] + g.Jinv[6] * sh[i].d[2];
        gy[i] = g.Jinv[1] * sh[i].d[0] + g.Jinv[4] * sh[i].d[1] + g.Jinv[7] * sh[i].d[2];
        gz[i] = g.Jinv[2] * sh[i].d[0] + g.Jinv[5] * sh[i].d[1] + g.Jinv[8] * sh[i].d[2];
      }
      for (int i = 0; i < n; i++) for (int j = 0; j < n; j++)
        K[(size_t)i * n + j] += fac * (gx[i] * gx[j] + gy[i] * gy[j] + gz[i] * gz[j]);
    }
  }
  if (mu != 0.0) {
    Rule r = mass_rule(S);
    for (int qq = 0; qq < r.size(); qq++) {
      const int q = reverse ? r.size() - 1 - qq : qq;
      shape_ad(S, e, r.x[q], r.y[q], r.z[q], sh.data());
      Geo g = geometry(S, e, r.x[q], r.y[q], r.z[q]);
      double fac = mu * r.w[q] * std::fabs(g.det);
      for (int i = 0; i < n; i++) for (int j = 0; j < n; j++) K[(size_t)i * n + j] += fac * sh[i].v * sh[j].v;
    }
  }
}

// MatrixGraph (linalg/sparsematrix.cpp:450-900): row = sorted union of the DOFs
// of all elements touching the row DOF; full (non-symmetric) storage.
void build_graph(Space& S) {
  std::vector<long> cnt(S.ndof + 1, 0);
  for (size_t k = 0; k < S.edofs.size(); k++) cnt[S.edofs[k] + 1]++;
  for (long i = 0; i < S.ndof; i++) cnt[i + 1] += cnt[i];
  std::vector<int> dof2el(cnt[S.ndof]);
  std::vector<long> fill(cnt.begin(), cnt.end() - 1);
  for (int e = 0; e < S.ne; e++) for (int i = 0; i < S.nloc; i++) dof2el[fill[S.edofs[(size_t)e * S.nloc + i]]++] = e;
  std::vector<std::vector<int>> rows(S.ndof);
#pragma omp parallel for schedule(dynamic, 256)
  for (long r = 0; r < S.ndof; r++) {
    std::vector<int>& c = rows[r];
    for (long k = cnt[r]; k < cnt[r + 1]; k++) { int e = dof2el[k]; for (int i = 0; i < S.nloc; i++) c.push_back((int)S.edofs[(size_t)e * S.nloc + i]); }
    std::sort(c.begin(), c.end()); c.erase(std::unique(c.begin(), c.end()), c.end());
  }
  S.rowptr.assign(S.ndof + 1, 0);
  for (long r = 0; r < S.ndof; r++) S.rowptr[r + 1] = S.rowptr[r] + (long)rows[r].size();
  S.colind.resize(S.rowptr[S.ndof]);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < S.ndof; r++) std::copy(rows[r].begin(), rows[r].end(), S.colind.begin() + S.rowptr[r]);
}

// AddElementMatrix (linalg/sparsematrix_impl.hpp:148-190): sorted merge walk per row
bool add_element_matrix(const Space& S, const long* dn, const std::vector<double>& K, double* vals) {
  const int n = S.nloc;
  std::vector<int> map(n); std::iota(map.begin(), map.end(), 0);
  std::sort(map.begin(), map.end(), [&](int a, int b) { return dn[a] < dn[b]; });
  for (int i = 0; i < n; i++) {
    long r = dn[i]; long k = S.rowptr[r], kend = S.rowptr[r + 1];
    for (int j1 = 0; j1 < n; j1++) {
      int j = map[j1];
      while (S.colind[k] != dn[j]) { k++; if (k >= kend) return false; }
#pragma omp atomic
      vals[k] += K[(size_t)i * n + j];
    }
  }
  return true;
}

}  // namespace

// ===========================================================================
// C interface (loaded with ctypes by the tests and the CPU-baseline leg)
extern "C" {

void* orc_space_create(int et, int nv, const double* X, int ne, const int* el, int p) {
  Space* S = new Space();
  S->et = et; S->nv = nv; S->ne = ne; S->p = p;
  S->X.assign(X, X + 3 * (size_t)nv);
  S->el.assign(el, el + (size_t)ne * (et == 4 ? 4 : 8));
  build_space(*S);
  return S;
}
// a space with Dirichlet conditions on nbf given boundary faces (fv = 3 or 4
// vertex numbers each); NULL if one of them is not a boundary face
void* orc_space_create_bnd(int et, int nv, const double* X, int ne, const int* el, int p, long nbf, const int* faces) {
  Space* S = new Space();
  S->et = et; S->nv = nv; S->ne = ne; S->p = p;
  S->X.assign(X, X + 3 * (size_t)nv);
  S->el.assign(el, el + (size_t)ne * (et == 4 ? 4 : 8));
  const int fv = et == 4 ? 3 : 4;
  S->dir_select = true;
  for (long k = 0; k < nbf; k++) {
    std::array<int, 4> t{INT32_MAX, INT32_MAX, INT32_MAX, INT32_MAX};
    for (int j = 0; j < fv; j++) t[j] = faces[k * fv + j];
    std::sort(t.begin(), t.begin() + fv);
    S->dir_faces.push_back(t);
  }
  build_space(*S);
  if (S->dir_bad) { delete S; return nullptr; }
  return S;
}
void orc_space_destroy(void* h) { delete (Space*)h; }
void orc_space_info(void* h, long* out) {  // ndof, nloc, ned, nfa, first_edge, first_face, first_cell
  Space* S = (Space*)h;
  out[0] = S->ndof; out[1] = S->nloc; out[2] = S->ned; out[3] = S->nfa;
  out[4] = S->first_edge; out[5] = S->first_face; out[6] = S->first_cell;
}
void orc_space_dofs(void* h, int* out) { Space* S = (Space*)h; for (size_t k = 0; k < S->edofs.size(); k++) out[k] = (int)S->edofs[k]; }
void orc_space_freedofs(void* h, unsigned char* out) { Space* S = (Space*)h; std::memcpy(out, S->freedof.data(), S->ndof); }
void orc_space_topology(void* h, int* el_edges, int* el_faces) {
  Space* S = (Space*)h;
  std::memcpy(el_edges, S->el_edges.data(), S->el_edges.size() * sizeof(int));
  std::memcpy(el_faces, S->el_faces.data(), S->el_faces.size() * sizeof(int));
}

long orc_graph(void* h) { Space* S = (Space*)h; if (S->rowptr.empty()) build_graph(*S); return S->rowptr[S->ndof]; }
void orc_graph_get(void* h, long* rowptr, int* colind) {
  Space* S = (Space*)h;
  std::memcpy(rowptr, S->rowptr.data(), (S->ndof + 1) * sizeof(long));
  std::memcpy(colind, S->colind.data(), S->colind.size() * sizeof(int));
}
// Assemble (comp/bilinearform.cpp:1562-2200): vals of kappa_e grad.grad + mu_e u v
static int assemble_impl(void* h, const double* kappa, const double* k6, const double* mu, double* vals, int reverse) {
  Space* S = (Space*)h;
  if (S->rowptr.empty()) build_graph(*S);
  std::memset(vals, 0, S->colind.size() * sizeof(double));
  int bad = 0;
#pragma omp parallel
  {
    std::vector<double> K;
#pragma omp for schedule(dynamic, 16)
    for (int e = 0; e < S->ne; e++) {
      element_matrix(*S, e, kappa ? kappa[e] : 1.0, mu ? mu[e] : 0.0, K, reverse, k6 ? k6 + 6 * (size_t)e : nullptr);
      if (!add_element_matrix(*S, &S->edofs[(size_t)e * S->nloc], K, vals)) {
#pragma omp atomic write
        bad = 1;
      }
    }
  }
  return bad ? -1 : 0;
}
int orc_assemble(void* h, const double* kappa, const double* mu, double* vals, int reverse) {
  return assemble_impl(h, kappa, nullptr, mu, vals, reverse);
}
// anisotropic diffusion: k6[e*6 .. e*6+5] = (xx yy zz xy xz yz) of element e's tensor
int orc_assemble_k6(void* h, const double* k6, const double* mu, double* vals, int reverse) {
  return assemble_impl(h, nullptr, k6, mu, vals, reverse);
}
void orc_element_matrix(void* h, int e, double kappa, double mu, double* K) {
  std::vector<double> Kv; element_matrix(*(Space*)h, e, kappa, mu, Kv);
  std::memcpy(K, Kv.data(), Kv.size() * sizeof(double));
}

// SparseMatrix::MultAdd (linalg/sparsematrix_impl.hpp:264-290): y = s*A*x (+y)
void orc_spmv(long n, const long* rowptr, const int* colind, const double* vals, double s, const double* x, double* y, int accumulate) {
#pragma omp parallel for schedule(static)
  for (long r = 0; r < n; r++) {
    double sum = 0;
    for (long k = rowptr[r]; k < rowptr[r + 1]; k++) sum += vals[k] * x[colind[k]];
    y[r] = accumulate ? y[r] + s * sum : s * sum;
  }
}

// Matrix-free apply, element by element with shape recomputation
// (S_BilinearForm::AddMatrix1 comp/bilinearform.cpp:4668-4760 with
// SymbolicBFI::ApplyElementMatrix fem/symbolicintegrator.cpp:2959-3040):
// y = A x over elements [e0,e1) (whole mesh when e1<0), no element matrix formed.
static void apply_mf_impl(void* h, const double* kappa, const double* k6, const double* mu, const double* x, double* y,
                          int e0, int e1) {
  Space* S = (Space*)h;
  if (e1 < 0) e1 = S->ne;
  // a partial range (a timing sample) expects a zeroed y from the caller
  if (e0 == 0 && e1 == S->ne) std::memset(y, 0, S->ndof * sizeof(double));
  const int n = S->nloc;
  Rule r = bilinear_rule(*S);
  Rule rm = mass_rule(*S);
#pragma omp parallel
  {
    std::vector<AD> sh(n);
    std::vector<double> xe(n), ye(n);
#pragma omp for schedule(dynamic, 16)
    for (int e = e0; e < e1; e++) {
      const long* dn = &S->edofs[(size_t)e * n];
      for (int i = 0; i < n; i++) { xe[i] = x[dn[i]]; ye[i] = 0; }
      double ka = kappa ? kappa[e] : 1.0, m = mu ? mu[e] : 0.0;
      double kt[9];
      if (k6) tensor33(k6 + 6 * (size_t)e, kt);
      if (k6 || ka != 0.0)
        for (int q = 0; q < r.size(); q++) {
          shape_ad(*S, e, r.x[q], r.y[q], r.z[q], sh.data());
          Geo g = geometry(*S, e, r.x[q], r.y[q], r.z[q]);
          double gr[3] = {0, 0, 0};
          for (int i = 0; i < n; i++) for (int k = 0; k < 3; k++) gr[k] += sh[i].d[k] * xe[i];
          double gp[3];  // physical gradient J^{-T} gr
          for (int k = 0; k < 3; k++) gp[k] = g.Jinv[0 * 3 + k] * gr[0] + g.Jinv[1 * 3 + k] * gr[1] + g.Jinv[2 * 3 + k] * gr[2];
          double fac = ka * r.w[q] * std::fabs(g.det);
          if (k6) {  // flux K gp; the weight carries no kappa
            const double g0 = gp[0], g1 = gp[1], g2 = gp[2];
            for (int k = 0; k < 3; k++) gp[k] = kt[3 * k] * g0 + kt[3 * k + 1] * g1 + kt[3 * k + 2] * g2;
            fac = r.w[q] * std::fabs(g.det);
          }
          double fl[3];   // flux back to reference: J^{-1} (fac*gp)
          for (int k = 0; k < 3; k++) fl[k] = fac * (g.Jinv[3 * k + 0] * gp[0] + g.Jinv[3 * k + 1] * gp[1] + g.Jinv[3 * k + 2] * gp[2]);
          for (int i = 0; i < n; i++) ye[i] += sh[i].d[0] * fl[0] + sh[i].d[1] * fl[1] + sh[i].d[2] * fl[2];
        }
      if (m != 0.0)
        for (int q = 0; q < rm.size(); q++) {
          shape_ad(*S, e, rm.x[q], rm.y[q], rm.z[q], sh.data());
          Geo g = geometry(*S, e, rm.x[q], rm.y[q], rm.z[q]);
          double u = 0; for (int i = 0; i < n; i++) u += sh[i].v * xe[i];
          double fac = m * rm.w[q] * std::fabs(g.det) * u;
          for (int i = 0; i < n; i++) ye[i] += sh[i].v * fac;
        }
      for (int i = 0; i < n; i++) {
#pragma omp atomic
        y[dn[i]] += ye[i];
      }
    }
  }
}

void orc_apply_mf(void* h, const double* kappa, const double* mu, const double* x, double* y, int e0, int e1) {
  apply_mf_impl(h, kappa, nullptr, mu, x, y, e0, e1);
}
void orc_apply_mf_k6(void* h, const double* k6, const double* mu, const double* x, double* y, int e0, int e1) {
  apply_mf_impl(h, nullptr, k6, mu, x, y, e0, e1);
}

// Generic B^T D B: the reference's fused symbolic operator for an arbitrary
// bilinear integrand (comp/matrixfree.cpp:1090-1330 AssembleBDBFused: D from
// the integrand per trial/test component pair, then B^T D B per point with the
// element Jacobian), applied element by element as ApplyElementMatrix does
// (fem/symbolicintegrator.cpp:2959-3040):
//   y_e = sum_q w_q |det J_q| B_q^T D_q B_q x_e,  B_q x = (u, grad u) at point q
// in physical coordinates, D row = test component, column = trial component.
// per_point = 0: D[e][16]; 1: D[e][q][16] at the nq points of `rule` (reference
// x, y, z, w).  rule = NULL: the oracle's own rule of order 2p (D per element).
// diag != NULL: the diagonal of the operator instead of y (x unused).
static void bdb_impl(void* h, const double* D, int per_point, int nq, const double* rule, const double* x, double* y,
                     double* diag) {
  Space* S = (Space*)h;
  Rule r;
  if (rule) {
    for (int q = 0; q < nq; q++) {
      r.x.push_back(rule[4 * q]); r.y.push_back(rule[4 * q + 1]); r.z.push_back(rule[4 * q + 2]); r.w.push_back(rule[4 * q + 3]);
    }
  } else {
    r = mass_rule(*S);
  }
  double* out = diag ? diag : y;
  std::memset(out, 0, S->ndof * sizeof(double));
  const int n = S->nloc;
#pragma omp parallel
  {
    std::vector<AD> sh(n);
    std::vector<double> xe(n), ye(n);
#pragma omp for schedule(dynamic, 16)
    for (int e = 0; e < S->ne; e++) {
      const long* dn = &S->edofs[(size_t)e * n];
      for (int i = 0; i < n; i++) { xe[i] = diag ? 0.0 : x[dn[i]]; ye[i] = 0; }
      for (int q = 0; q < r.size(); q++) {
        shape_ad(*S, e, r.x[q], r.y[q], r.z[q], sh.data());
        Geo g = geometry(*S, e, r.x[q], r.y[q], r.z[q]);
        const double* De = per_point ? D + ((size_t)e * r.size() + q) * 16 : D + (size_t)e * 16;
        const double s = r.w[q] * std::fabs(g.det);
        if (diag) {
          for (int i = 0; i < n; i++) {
            double b[4] = {sh[i].v, 0, 0, 0};
            for (int k = 0; k < 3; k++) b[1 + k] = g.Jinv[k] * sh[i].d[0] + g.Jinv[3 + k] * sh[i].d[1] + g.Jinv[6 + k] * sh[i].d[2];
            double t = 0;
            for (int a = 0; a < 4; a++) for (int c = 0; c < 4; c++) t += b[a] * De[4 * a + c] * b[c];
            ye[i] += s * t;
          }
          continue;
        }
        double in[4] = {0, 0, 0, 0}, gr[3] = {0, 0, 0};
        for (int i = 0; i < n; i++) {
          in[0] += sh[i].v * xe[i];
          for (int k = 0; k < 3; k++) gr[k] += sh[i].d[k] * xe[i];
        }
        for (int k = 0; k < 3; k++) in[1 + k] = g.Jinv[k] * gr[0] + g.Jinv[3 + k] * gr[1] + g.Jinv[6 + k] * gr[2];
        double o[4];
        for (int a = 0; a < 4; a++) o[a] = s * (De[4 * a] * in[0] + De[4 * a + 1] * in[1] + De[4 * a + 2] * in[2] + De[4 * a + 3] * in[3]);
        double ref[3];  // J^{-1} (o_x, o_y, o_z): the test gradient's coefficients in reference coordinates
        for (int j = 0; j < 3; j++) ref[j] = g.Jinv[3 * j] * o[1] + g.Jinv[3 * j + 1] * o[2] + g.Jinv[3 * j + 2] * o[3];
        for (int i = 0; i < n; i++) ye[i] += sh[i].v * o[0] + sh[i].d[0] * ref[0] + sh[i].d[1] * ref[1] + sh[i].d[2] * ref[2];
      }
      for (int i = 0; i < n; i++) {
#pragma omp atomic
        out[dn[i]] += ye[i];
      }
    }
  }
}
void orc_apply_bdb(void* h, const double* D, int per_point, int nq, const double* rule, const double* x, double* y) {
  bdb_impl(h, D, per_point, nq, rule, x, y, nullptr);
}
void orc_diag_bdb(void* h, const double* D, int per_point, int nq, const double* rule, double* diag) {
  bdb_impl(h, D, per_point, nq, rule, nullptr, nullptr, diag);
}

// H1HighOrderFESpace::CreateSmoothingBlocks (comp/h1hofespace.cpp:1477-1600)
// through a FilteredTableCreator (only free DOFs enter): blocktype 4 "VE + F + I"
// -- row v holds vertex v and the DOFs of every edge at v, then one row per
// face, one per element interior; 3 "V + E + F + I".  Empty rows are dropped
// and each row is sorted (the block's matrix and inverse do not depend on the
// order).  Returns the number of rows; offsets / dofs may be NULL (sizes only:
// *nentries gets the total).
long orc_smoothing_blocks(void* h, int blocktype, long* nentries, long* offsets, int* dofs) {
  Space* S = (Space*)h;
  std::vector<std::vector<int>> rows;
  const int ned = S->n_edge_dofs;
  if (blocktype == 4) {
    std::vector<std::vector<int>> vb(S->nv);
    for (int v = 0; v < S->nv; v++) vb[v].push_back(v);
    for (int g = 0; g < S->ned; g++)
      for (int k = 0; k < ned; k++) {
        const int d = (int)(S->first_edge + (long)g * ned + k);
        vb[S->edges[g][0]].push_back(d);
        vb[S->edges[g][1]].push_back(d);
      }
    for (auto& r : vb) rows.push_back(r);
  } else {
    for (int v = 0; v < S->nv; v++) rows.push_back({v});
    for (int g = 0; g < S->ned; g++) {
      std::vector<int> r;
      for (int k = 0; k < ned; k++) r.push_back((int)(S->first_edge + (long)g * ned + k));
      rows.push_back(r);
    }
  }
  for (int f = 0; f < S->nfa; f++) {
    std::vector<int> r;
    for (int k = 0; k < S->n_face_dofs; k++) r.push_back((int)(S->first_face + (long)f * S->n_face_dofs + k));
    rows.push_back(r);
  }
  for (int e = 0; e < S->ne; e++) {
    std::vector<int> r;
    for (int k = 0; k < S->n_cell_dofs; k++) r.push_back((int)(S->first_cell + (long)e * S->n_cell_dofs + k));
    rows.push_back(r);
  }
  long nb = 0, nt = 0;
  if (offsets) offsets[0] = 0;
  for (auto& r : rows) {
    std::vector<int> f;
    for (int d : r) if (S->freedof[d]) f.push_back(d);
    if (f.empty()) continue;
    std::sort(f.begin(), f.end());
    for (int d : f) { if (dofs) dofs[nt] = d; nt++; }
    nb++;
    if (offsets) offsets[nb] = nt;
  }
  if (nentries) *nentries = nt;
  return nb;
}

// LinearForm f*v with f piecewise constant per element, integration order 2p
// (SymbolicLFI, fem/symbolicintegrator.cpp:1109)
// deformation: d[3][ndof of hdef] on the space hdef (same mesh); d = NULL removes it
void orc_space_set_deformation(void* h, void* hdef, const double* d) {
  Space* S = (Space*)h;
  if (!d) { S->def = nullptr; S->defvec.clear(); return; }
  S->def = (Space*)hdef;
  S->defvec.assign(d, d + 3 * (size_t)S->def->ndof);
}

static void rhs_impl(Space* S, const Rule& r, const double* f, double* b);
void orc_rhs(void* h, const double* f, double* b) {
  Space* S = (Space*)h;
  rhs_impl(S, mass_rule(*S), f, b);
}
// the same at a caller's rule (nq points: reference x, y, z, weight)
void orc_rhs_rule(void* h, const double* f, int nq, const double* rule, double* b) {
  Rule r;
  for (int q = 0; q < nq; q++) {
    r.x.push_back(rule[4 * q]); r.y.push_back(rule[4 * q + 1]); r.z.push_back(rule[4 * q + 2]); r.w.push_back(rule[4 * q + 3]);
  }
  rhs_impl((Space*)h, r, f, b);
}
static void rhs_impl(Space* S, const Rule& r, const double* f, double* b) {
  std::memset(b, 0, S->ndof * sizeof(double));
  const int n = S->nloc;
#pragma omp parallel
  {
    std::vector<AD> sh(n); std::vector<double> be(n);
#pragma omp for schedule(dynamic, 16)
    for (int e = 0; e < S->ne; e++) {
      std::fill(be.begin(), be.end(), 0.0);
      for (int q = 0; q < r.size(); q++) {
        shape_ad(*S, e, r.x[q], r.y[q], r.z[q], sh.data());
        Geo g = geometry(*S, e, r.x[q], r.y[q], r.z[q]);
        double fac = f[e] * r.w[q] * std::fabs(g.det);
        for (int i = 0; i < n; i++) be[i] += fac * sh[i].v;
      }
      const long* dn = &S->edofs[(size_t)e * n];
      for (int i = 0; i < n; i++) {
#pragma omp atomic
        b[dn[i]] += be[i];
      }
    }
  }
}

// element-wise integral of grad u . grad w  (Integrate(..., element_wise=True),
// comp/python_comp.cpp:3703-3948): the dJ/dkappa_e contraction
void orc_elem_grad_dot(void* h, const double* u, const double* w, double* out) {
  Space* S = (Space*)h;
  Rule r = bilinear_rule(*S);
  const int n = S->nloc;
#pragma omp parallel
  {
    std::vector<AD> sh(n);
#pragma omp for schedule(dynamic, 16)
    for (int e = 0; e < S->ne; e++) {
      const long* dn = &S->edofs[(size_t)e * n];
      double acc = 0;
      for (int q = 0; q < r.size(); q++) {
        shape_ad(*S, e, r.x[q], r.y[q], r.z[q], sh.data());
        Geo g = geometry(*S, e, r.x[q], r.y[q], r.z[q]);
        double gu[3] = {0, 0, 0}, gw[3] = {0, 0, 0};
        for (int i = 0; i < n; i++) for (int k = 0; k < 3; k++) { gu[k] += sh[i].d[k] * u[dn[i]]; gw[k] += sh[i].d[k] * w[dn[i]]; }
        double pu[3], pw[3];
        for (int k = 0; k < 3; k++) {
          pu[k] = g.Jinv[k] * gu[0] + g.Jinv[3 + k] * gu[1] + g.Jinv[6 + k] * gu[2];
          pw[k] = g.Jinv[k] * gw[0] + g.Jinv[3 + k] * gw[1] + g.Jinv[6 + k] * gw[2];
        }
        acc += r.w[q] * std::fabs(g.det) * (pu[0] * pw[0] + pu[1] * pw[1] + pu[2] * pw[2]);
      }
      out[e] = acc;
    }
  }
}

// shape values and reference gradients of one element at points (for table checks)
int orc_shapes(int et, int p, const int* vnums, int npts, const double* pts, double* val, double* grad) {
  int n = nloc_of(et, p);
  std::vector<AD> sh(n);
  for (int q = 0; q < npts; q++) {
    AD X = AD::var(pts[3 * q], 0), Y = AD::var(pts[3 * q + 1], 1), Z = AD::var(pts[3 * q + 2], 2);
    int m = et == 4 ? tet_shape<AD>(p, vnums, X, Y, Z, sh.data()) : hex_shape<AD>(p, vnums, X, Y, Z, sh.data());
    if (m != n) return -1;
    for (int i = 0; i < n; i++) {
      val[(size_t)q * n + i] = sh[i].v;
      for (int k = 0; k < 3; k++) grad[((size_t)q * n + i) * 3 + k] = sh[i].d[k];
    }
  }
  return n;
}
// 2D/3D Dubiner bubble bases alone (orthogonality checks)
int orc_dubiner2d(int n, double x, double y, double* out) { return dubiner_orthobub_scaled_mult<double>(n, x, y, 1.0, 1.0, out); }
int orc_dubiner3d(int n, double x, double y, double z, double* out) { return dubiner3d_orthobub_mult<double>(n, x, y, z, 1.0, out); }
int orc_rule(int et, int order, double* pts, double* w) {
  Rule r = et == 4 ? tet_rule(order) : hex_rule(order);
  if (pts) for (int q = 0; q < r.size(); q++) { pts[3 * q] = r.x[q]; pts[3 * q + 1] = r.y[q]; pts[3 * q + 2] = r.z[q]; w[q] = r.w[q]; }
  return r.size();
}

// Jacobi-preconditioned CG, the algorithm of CGSolver._SolveImpl
// (python/krylovspace.py:263-291) with CheckResidual (:129-219): residual =
// sqrt|w.d| (preconditioned), stop when <= tol*first or after maxit.
// Operator: assembled CSR (rowptr != NULL) or matrix-free (space handle).
// Preconditioner: invdiag on free DOFs, 0 elsewhere (linalg/jacobi.cpp:40-110).
int orc_cg(void* h, long n, const long* rowptr, const int* colind, const double* vals,
           const double* kappa, const double* mu, const double* invdiag,
           const double* b, double* x, double tol, int maxit, double* res_hist, int* iters) {
  std::vector<double> d(n), w(n), s(n), tmp(n);
  auto A = [&](const double* in, double* out) {
    if (rowptr) orc_spmv(n, rowptr, colind, vals, 1.0, in, out, 0);
    else orc_apply_mf(h, kappa, mu, in, out, 0, -1);
  };
  auto dot = [&](const std::vector<double>& a, const std::vector<double>& c) {
    double sum = 0;
#pragma omp parallel for reduction(+ : sum) schedule(static)
    for (long i = 0; i < n; i++) sum += a[i] * c[i];
    return sum;
  };
  A(x, tmp.data());
  for (long i = 0; i < n; i++) d[i] = b[i] - tmp[i];
  for (long i = 0; i < n; i++) w[i] = invdiag[i] * d[i];
  s = w;
  double wdn = dot(w, d);
  int it = 0;
  double first = std::sqrt(std::fabs(wdn));
  if (res_hist) res_hist[0] = first;
  it = 1;
  double stop = first * tol;
  if (first <= stop || maxit <= 1) { *iters = it; return 0; }
  while (true) {
    A(s.data(), w.data());
    double wd = wdn;
    double as_s = dot(s, w);
    if (as_s == 0 || wd == 0) break;
    double alpha = wd / as_s;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) { x[i] += alpha * s[i]; d[i] -= alpha * w[i]; w[i] = invdiag[i] * d[i]; }
    wdn = dot(w, d);
    double res = std::sqrt(std::fabs(wdn));
    if (res_hist) res_hist[it] = res;
    it++;
    if (it >= maxit || res <= stop) break;
    double beta = wdn / wd;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) s[i] = w[i] + beta * s[i];
  }
  *iters = it;
  return 0;
}

int orc_max_threads() { return omp_get_max_threads(); }

}  // extern "C"
