// Host construction of the DFR element operators in FP64.  See dfr_element.hpp
// for the reference functions each piece follows.
#include "dfr_element.hpp"

#include <cmath>
#include <stdexcept>
#include <string>

#include "wsj_table.h"

namespace gcfd {

DMat matmul(const DMat& a, const DMat& b) {
  if (a.cols != b.rows) throw std::runtime_error("matmul: shape mismatch");
  DMat c(a.rows, b.cols);
  for (int i = 0; i < a.rows; ++i)
    for (int k = 0; k < a.cols; ++k) {
      const double aik = a(i, k);
      if (aik == 0.0) continue;
      for (int j = 0; j < b.cols; ++j) c(i, j) += aik * b(k, j);
    }
  return c;
}

DMat inverse(const DMat& a) {
  if (a.rows != a.cols) throw std::runtime_error("inverse: matrix not square");
  const int n = a.rows;
  DMat lu = a, inv(n, n);
  std::vector<int> piv(n);
  for (int i = 0; i < n; ++i) piv[i] = i;
  for (int c = 0; c < n; ++c) {
    int p = c;
    double best = std::fabs(lu(c, c));
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(lu(r, c)) > best) { best = std::fabs(lu(r, c)); p = r; }
    if (best < 1e-300) throw std::runtime_error("inverse: singular matrix");
    if (p != c) {
      for (int j = 0; j < n; ++j) std::swap(lu(p, j), lu(c, j));
      std::swap(piv[p], piv[c]);
    }
    for (int r = c + 1; r < n; ++r) {
      const double f = lu(r, c) / lu(c, c);
      lu(r, c) = f;
      for (int j = c + 1; j < n; ++j) lu(r, j) -= f * lu(c, j);
    }
  }
  // Solve LU x = P e_j for every column j.
  std::vector<double> x(n);
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) x[i] = (piv[i] == j) ? 1.0 : 0.0;
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < i; ++k) x[i] -= lu(i, k) * x[k];
    for (int i = n - 1; i >= 0; --i) {
      for (int k = i + 1; k < n; ++k) x[i] -= lu(i, k) * x[k];
      x[i] /= lu(i, i);
    }
    for (int i = 0; i < n; ++i) inv(i, j) = x[i];
  }
  return inv;
}

// Gamma-function normalisation of the Jacobi polynomials (Hesthaven & Warburton,
// "Nodal DG Methods", JacobiP), as used by DG1D/elements.go:257-315.
double jacobi_p(double x, double alpha, double beta, int n) {
  const double g0 = std::pow(2.0, alpha + beta + 1.0) / (alpha + beta + 1.0) *
                    std::tgamma(alpha + 1.0) * std::tgamma(beta + 1.0) /
                    std::tgamma(alpha + beta + 1.0);
  double p0 = 1.0 / std::sqrt(g0);
  if (n == 0) return p0;
  const double g1 = (alpha + 1.0) * (beta + 1.0) / (alpha + beta + 3.0) * g0;
  double p1 = ((alpha + beta + 2.0) * x / 2.0 + (alpha - beta) / 2.0) / std::sqrt(g1);
  if (n == 1) return p1;
  double aold = 2.0 / (2.0 + alpha + beta) *
                std::sqrt((alpha + 1.0) * (beta + 1.0) / (alpha + beta + 3.0));
  for (int i = 1; i <= n - 1; ++i) {
    const double h1 = 2.0 * i + alpha + beta;
    const double anew = 2.0 / (h1 + 2.0) *
                        std::sqrt((i + 1.0) * (i + 1.0 + alpha + beta) * (i + 1.0 + alpha) *
                                  (i + 1.0 + beta) / (h1 + 1.0) / (h1 + 3.0));
    const double bnew = -(alpha * alpha - beta * beta) / h1 / (h1 + 2.0);
    const double p2 = (-aold * p0 + (x - bnew) * p1) / anew;
    p0 = p1;
    p1 = p2;
    aold = anew;
  }
  return p1;
}

double grad_jacobi_p(double x, double alpha, double beta, int n) {
  if (n == 0) return 0.0;
  return std::sqrt(n * (n + alpha + beta + 1.0)) * jacobi_p(x, alpha + 1.0, beta + 1.0, n - 1);
}

static void rs_to_ab(double r, double s, double* a, double* b) {
  *a = (s != 1.0) ? 2.0 * (1.0 + r) / (1.0 - s) - 1.0 : -1.0;
  *b = s;
}

double simplex2d_p(double r, double s, int i, int j) {
  double a, b;
  rs_to_ab(r, s, &a, &b);
  const double h1 = jacobi_p(a, 0.0, 0.0, i);
  const double h2 = jacobi_p(b, 2.0 * i + 1.0, 0.0, j);
  return std::sqrt(2.0) * h1 * h2 * std::pow(1.0 - b, i);
}

void grad_simplex2d_p(double r, double s, int id, int jd, double* ddr, double* dds) {
  double a, b;
  rs_to_ab(r, s, &a, &b);
  const double fa = jacobi_p(a, 0, 0, id), dfa = grad_jacobi_p(a, 0, 0, id);
  const double gb = jacobi_p(b, 2.0 * id + 1.0, 0, jd);
  const double dgb = grad_jacobi_p(b, 2.0 * id + 1.0, 0, jd);
  double dr = dfa * gb;
  if (id > 0) dr *= std::pow(0.5 * (1.0 - b), id - 1);
  double ds = 0.5 * dfa * gb * (1.0 + a);
  if (id > 0) ds *= std::pow(0.5 * (1.0 - b), id - 1);
  double tmp = dgb * std::pow(0.5 * (1.0 - b), id);
  if (id > 0) tmp -= 0.5 * id * gb * std::pow(0.5 * (1.0 - b), id - 1);
  ds += fa * tmp;
  const double norm = std::pow(2.0, id + 0.5);
  *ddr = dr * norm;
  *dds = ds * norm;
}

// Edge-point parameters, RT order P = 1..8 (raviart_thomas_element.go:377-400).
static const double kEdgeP1[] = {-0.38490018, 0.38490018};
static const double kEdgeP2[] = {-0.028, 0.000, 0.028};
static const double kEdgeP3[] = {-0.482, -0.161, 0.161, 0.482};
static const double kEdgeP4[] = {-0.586, -0.293, 0.000, 0.293, 0.586};
static const double kEdgeP5[] = {-0.634, -0.381, -0.127, 0.127, 0.381, 0.634};
static const double kEdgeP6[] = {-0.671, -0.452, -0.219, 0.000, 0.219, 0.452, 0.671};
static const double kEdgeP7[] = {-0.808, -0.578, -0.343, -0.113, 0.113, 0.343, 0.578, 0.808};
static const double kEdgeP8[] = {-0.692, -0.523, -0.350, -0.176, 0.000,
                                 0.176,  0.350,  0.523,  0.692};

const double* optimized_edge_points(int P) {
  switch (P) {
    case 1: return kEdgeP1;
    case 2: return kEdgeP2;
    case 3: return kEdgeP3;
    case 4: return kEdgeP4;
    case 5: return kEdgeP5;
    case 6: return kEdgeP6;
    case 7: return kEdgeP7;
    case 8: return kEdgeP8;
    default: return nullptr;
  }
}

static DMat vandermonde2d(int N, const std::vector<double>& r, const std::vector<double>& s) {
  const int np = (N + 1) * (N + 2) / 2;
  DMat V(static_cast<int>(r.size()), np);
  int sk = 0;
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N - i; ++j, ++sk)
      for (size_t p = 0; p < r.size(); ++p) V(static_cast<int>(p), sk) = simplex2d_p(r[p], s[p], i, j);
  return V;
}

// Raviart-Thomas divergence of order P at the given points.  The space RT_P is
// spanned here by (phi,0), (0,phi) for every orthonormal mode phi of degree <= P,
// plus x * r^(P-m) s^m for m = 0..P (x = (r,s)); the degrees of freedom are the
// point values dotted with the DOF directions of raviart_thomas_element.go:224-234.
// The resulting matrix depends only on the space and the DOFs, not on the basis.
static DMat rt_divergence(int P, const std::vector<double>& R, const std::vector<double>& S,
                          const std::vector<double>& bx, const std::vector<double>& by) {
  const int n = static_cast<int>(R.size());
  const int nmodes = (P + 1) * (P + 2) / 2;
  if (n != 2 * nmodes + P + 1) throw std::runtime_error("rt_divergence: dimension mismatch");
  DMat V(n, n), DivB(n, n);
  for (int p = 0; p < n; ++p) {
    const double r = R[p], s = S[p];
    int col = 0;
    for (int i = 0; i <= P; ++i)
      for (int j = 0; j <= P - i; ++j) {
        const double phi = simplex2d_p(r, s, i, j);
        double dr, ds;
        grad_simplex2d_p(r, s, i, j, &dr, &ds);
        V(p, col) = phi * bx[p];          // (phi, 0)
        DivB(p, col) = dr;
        V(p, col + nmodes) = phi * by[p];  // (0, phi)
        DivB(p, col + nmodes) = ds;
        ++col;
      }
    for (int m = 0; m <= P; ++m) {
      const double q = std::pow(r, P - m) * std::pow(s, m);
      const int c = 2 * nmodes + m;
      V(p, c) = r * q * bx[p] + s * q * by[p];
      DivB(p, c) = (P + 2.0) * q;  // div(x q) = 2q + x.grad q = (2+P) q
    }
  }
  return matmul(DivB, inverse(V));
}

static void recommended_filter(int P, double* alpha, int* s) {
  if (P <= 2) { *alpha = 4.0; *s = 4; }
  else if (P == 3) { *alpha = 6.0; *s = 4; }
  else if (P == 4) { *alpha = 8.0; *s = 5; }
  else if (P == 5) { *alpha = 10.0; *s = 6; }
  else if (P == 6) { *alpha = 14.0; *s = 6; }
  else if (P == 7) { *alpha = 18.0; *s = 7; }
  else if (P == 8) { *alpha = 24.0; *s = 8; }
  else { *alpha = 30.0 + 2.0 * (P - 9); *s = 8 + (P - 9) / 2; }
}

DFRElement build_dfr_element(int N) {
  if (N < 0 || N > gcfd_tables::kWSJMaxOrder)
    throw std::runtime_error("unsupported polynomial order N=" + std::to_string(N) + " (0..7)");
  DFRElement e;
  e.N = N;
  e.Np = (N + 1) * (N + 2) / 2;
  e.NpEdge = N + 2;
  e.NpFlux = (N + 2) * (N + 4);
  const int P = N + 1;
  const int np = e.Np, ne = e.NpEdge;

  // Solution points: barycentric -> (r,s) on (-1,-1),(1,-1),(-1,1).
  for (int i = gcfd_tables::kWSJOffset[N]; i < gcfd_tables::kWSJOffset[N + 1]; ++i) {
    const double* t = gcfd_tables::kWSJ[i];
    e.r.push_back(-t[0] + t[1] - t[2]);
    e.s.push_back(-t[0] - t[1] + t[2]);
    e.w.push_back(t[3]);
  }
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N - i; ++j) e.modeDegree.push_back(i + j);

  // Flux points: interior twice, then bottom, hypotenuse, left edges (CCW).
  const double* gp = optimized_edge_points(P);
  std::vector<double> bx, by;
  for (int c = 0; c < 2; ++c)
    for (int i = 0; i < np; ++i) {
      e.rFlux.push_back(e.r[i]);
      e.sFlux.push_back(e.s[i]);
      bx.push_back(c == 0 ? 1.0 : 0.0);
      by.push_back(c == 0 ? 0.0 : 1.0);
    }
  const double oosr2 = 0.5 * std::sqrt(2.0);
  for (int ed = 0; ed < 3; ++ed)
    for (int i = 0; i < ne; ++i) {
      const double g = gp[i];
      double rr, ss, nx, ny;
      if (ed == 0) { rr = g; ss = -1.0; nx = 0.0; ny = -1.0; }
      else if (ed == 1) { const double t = 0.5 * (g + 1.0); rr = 1.0 - 2.0 * t; ss = -1.0 + 2.0 * t; nx = oosr2; ny = oosr2; }
      else { rr = -1.0; ss = -g; nx = -1.0; ny = 0.0; }
      e.rFlux.push_back(rr);
      e.sFlux.push_back(ss);
      bx.push_back(nx);
      by.push_back(ny);
    }

  e.V = vandermonde2d(N, e.r, e.s);
  e.Vinv = inverse(e.V);
  std::vector<double> re(e.rFlux.begin() + 2 * np, e.rFlux.end());
  std::vector<double> se(e.sFlux.begin() + 2 * np, e.sFlux.end());
  e.FluxEdgeInterp = matmul(vandermonde2d(N, re, se), e.Vinv);

  e.Div = rt_divergence(P, e.rFlux, e.sFlux, bx, by);
  e.DivInt = DMat(np, e.NpFlux);
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < e.NpFlux; ++j) e.DivInt(i, j) = e.Div(i, j);

  // Shock sensor matrices (dfr_shock_capturing.go:71-107).
  DMat W(np, np);
  for (int i = 0; i < np; ++i) W(i, i) = e.w[i];
  DMat Vt(np, np);
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) Vt(i, j) = e.V(j, i);
  e.MassMatrix = matmul(matmul(Vt, W), e.V);
  DMat cut(np, np);
  for (int m = 0; m < np; ++m) cut(m, m) = (e.modeDegree[m] >= N) ? 0.0 : 1.0;
  e.Clipper = matmul(matmul(e.V, cut), e.Vinv);
  e.SensD = DMat(np, np);
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) e.SensD(i, j) = (i == j ? 1.0 : 0.0) - e.Clipper(i, j);
  e.SensP = matmul(e.MassMatrix, e.SensD);

  double alpha;
  int sexp;
  recommended_filter(N, &alpha, &sexp);
  e.ModeFilter.assign(np, 1.0);
  if (N > 1)
    for (int m = 0; m < np; ++m) {
      const int p = e.modeDegree[m];
      e.ModeFilter[m] = (p == 0) ? 1.0 : std::exp(-alpha * std::pow(double(p) / N, sexp));
    }

  // Barycentric coordinates of every flux point w.r.t. the reference vertices.
  e.Bary = DMat(e.NpFlux, 3);
  for (int i = 0; i < e.NpFlux; ++i) {
    const double r = e.rFlux[i], s = e.sFlux[i];
    e.Bary(i, 0) = -0.5 * (r + s);
    e.Bary(i, 1) = 0.5 * (1.0 + r);
    e.Bary(i, 2) = 0.5 * (1.0 + s);
  }
  return e;
}

}  // namespace gcfd
