// Host-side (FP64, set-up time) construction of the Direct Flux Reconstruction
// element: solution points, modal basis, the Raviart-Thomas flux element and
// every shared operator matrix that the device kernels multiply by.
//
// Reference behaviour followed (gocfd):
//   DG2D/dfr_startup.go:43-65        NewDFR2D: solution element of order N,
//                                    RT flux element of order N+1, FluxEdgeInterp
//   DG2D/lagrange_element.go:54-92   WSJ nodes, orthonormal Vandermonde, mass matrix
//   DG2D/basis_polynomials.go:19-153 Simplex2DP / GradSimplex2DP modal basis
//   DG2D/raviart_thomas_element.go:192-297,377-496  RT DOFs, edge points, Div/DivInt
//   DG2D/dfr_shock_capturing.go:43-140 ModalFilter, Clipper, sensor matrices
//   model_problems/Euler2D/dissipation.go:414-449 barycentric stencil
#pragma once
#include <cstddef>
#include <vector>

namespace gcfd {

struct DMat {
  int rows = 0, cols = 0;
  std::vector<double> v;
  DMat() = default;
  DMat(int r, int c) : rows(r), cols(c), v(static_cast<size_t>(r) * c, 0.0) {}
  double& operator()(int i, int j) { return v[static_cast<size_t>(i) * cols + j]; }
  double operator()(int i, int j) const { return v[static_cast<size_t>(i) * cols + j]; }
};

DMat matmul(const DMat& a, const DMat& b);
// Inverse by LU with partial pivoting; throws std::runtime_error when singular.
DMat inverse(const DMat& a);

// Normalised Jacobi polynomial P_n^(alpha,beta)(x) (orthonormal on [-1,1]
// with weight (1-x)^alpha (1+x)^beta), and its derivative.
double jacobi_p(double x, double alpha, double beta, int n);
double grad_jacobi_p(double x, double alpha, double beta, int n);
// Orthonormal simplex mode (i,j) on the reference triangle (-1,-1),(1,-1),(-1,1).
double simplex2d_p(double r, double s, int i, int j);
void grad_simplex2d_p(double r, double s, int i, int j, double* dr, double* ds);

// Optimised edge-point parameters for an RT element of order P (P = N+1).
const double* optimized_edge_points(int P);

struct DFRElement {
  int N = 0;       // solution polynomial order
  int Np = 0;      // (N+1)(N+2)/2 solution points (= RT interior points)
  int NpEdge = 0;  // N+2 points per edge
  int NpFlux = 0;  // (N+2)(N+4) RT degrees of freedom
  std::vector<double> r, s, w;          // solution points and WSJ weights
  std::vector<double> rFlux, sFlux;     // all NpFlux RT points (interior twice, then 3 edges)
  std::vector<int> modeDegree;          // total degree of each modal basis function
  DMat V, Vinv;                         // Np x Np modal Vandermonde and inverse
  DMat FluxEdgeInterp;                  // 3*NpEdge x Np, solution points -> edge points
  DMat Div;                             // NpFlux x NpFlux, RT divergence (r,s)
  DMat DivInt;                          // Np x NpFlux, first Np rows of Div
  DMat MassMatrix;                      // V^T W V
  DMat Clipper;                         // V diag(cutoff) Vinv, top modes removed
  DMat SensD;                           // I - Clipper
  DMat SensP;                           // MassMatrix * SensD
  std::vector<double> ModeFilter;       // exponential modal filter, Np
  DMat Bary;                            // NpFlux x 3 vertex -> flux-point interpolation
};

// Throws std::runtime_error for unsupported N (valid: 0..7).
DFRElement build_dfr_element(int N);

}  // namespace gcfd
