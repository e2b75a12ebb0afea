// Adjoint of the PerssonC0 shock capturing on the FP64 path (gcfd_diss.cuh):
// the transpose of, in forward order,
//   sensor      Se = log10(num / den), num = (D rho).(P rho), den = rho.(M rho);
//               sigma = ramp(Se); eps = Eps0 hK sigma           (dissipation.go:397-518)
//   vertex max  sigV, epsV = max over the elements at a vertex    (euler.go:1048-1065)
//   limiter     rkStep 2: Q <- V diag(1, mf (1 - a)) Vinv Q, a = sin(pi sigma_bar / 2),
//               sigma_bar = mean of the element's vertex sigV      (dissipation.go:606-622)
//   gradient    DissX/Y = eps_r grad(Q) at Np + 3 NpEdge flux points (dissipation.go:244-272)
//   viscous     VF = average of the two sides' n.(DissX, DissY) - Omega lambda / len (qa - qb),
//   edges       viscSpeed = max_p eps / hK^2                        (edges.go:151-286)
//   update      RHS = F(a) (RHS_Euler + DivInt DOF(DissX, DissY, VF) / |J|); dt with the viscous
//               limit (global: min(CFL / gmax, Cdiff / gvisc); local: the DTVisc running max that
//               persists across stages and steps)                   (dissipation.go:274-346, euler.go:945-1002)
// The max operations take their adjoint at the element / edge / point that
// set the max (the lowest index among exact ties; where sigma sits on a flat
// part of the ramp every tie has zero derivative anyway).
#pragma once
#include "gcfd_adjoint.cuh"
#include "gcfd_diss.cuh"

namespace gcfd {

struct AdjDissArgs {
  int nverts;
  const double* Qsens;      // state the sensor saw (before the rkStep-2 limiter)
  const double* rhsPre;     // taped RHS before the modal filter [n][i][k]
  double* RbE;              // out: adjoint of the Euler RHS [n][i][k]
  double* alphaBar;         // [K] adjoint of a = sin(pi sigma_bar / 2)
  double* sigVbar;          // [nverts]
  double* epsVbar;
  double* VFbar;            // [edge][4][NpEdge]
  double* DissXbar;         // [4][NR][K]
  double* DissYbar;
  double* QFb;              // [4][3 NpEdge][K] face adjoints
  double* vsBar;            // [edge] adjoint of the viscous speed
  const int* sigArg;        // [nverts] element that set sigV / epsV
  const int* epsArg;
  const double* sigE;       // [K] element sigma, eps, Se of this stage
  const double* SeE;
  const double* Q2pre;      // rkStep-2 state before the limiter
  double* Qlim;             // the stage-2 state adjoint, transposed through the limiter in place
};

__device__ __forceinline__ double vert_sigma_mean(const DissArgs& d, int k, size_t sK) {
  double acc = 0.0;
#pragma unroll
  for (int v = 0; v < 3; ++v) acc = acc + vdouble(d.sigV, d.etov[v * sK + k]);
  return acc / 3.0;
}

// Vertex argmax of the element sigma and eps of this stage (lowest element index).
static __global__ void k_diss_argmax(DissArgs d, const double* sigE, const double* epsE, int* sigArg, int* epsArg) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.K) return;
  const size_t sK = static_cast<size_t>(d.K);
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const int vert = d.etov[v * sK + k];
    if (sigE[k] == vdouble(d.sigV, vert)) atomicMin(&sigArg[vert], k);
    if (epsE[k] == vdouble(d.epsV, vert)) atomicMin(&epsArg[vert], k);
  }
}

// Stage update, modal filter and AddDissipation in reverse (k_diss_update).
// The SSP part is the same as k_adj_div's; the Euler RHS adjoint goes to RbE
// for k_adj_div (stage -1 form) to transpose.
template <int N>
__global__ void __launch_bounds__(128) k_adj_diss_update(DissArgs d, AdjArgs<double> a, AdjDissArgs x) {
  constexpr int NP = DissDims<N>::NP, NE = DissDims<N>::NE, NF = DissDims<N>::NF, NR = DissDims<N>::NR;
  __shared__ double sD[NP * NF], sV[NP * NP], sVi[NP * NP], smf[NP];
  stage_operator(sD, a.DivInt, NP * NF);
  stage_operator(sV, d.V, NP * NP);
  stage_operator(sVi, d.Vinv, NP * NP);
  stage_operator(smf, d.mf, NP);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = k < a.K;
  const size_t sK = static_cast<size_t>(a.K);
  const int s = a.stage;
  double dtb = 0.0;
  if (active) {
    const double Jd = a.Jdet[k], oojd = 1.0 / Jd;
    const double J0 = a.Jinv[k], J1 = a.Jinv[sK + k], J2 = a.Jinv[2 * sK + k], J3 = a.Jinv[3 * sK + k];
    const double alpha = sin(0.5 * 3.14159265358979323846 * vert_sigma_mean(d, k, sK));
    int eg[3];
    double esg[3];
    bool own[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      eg[e] = d.elemEdge[e * sK + k];
      own[e] = d.ekL[eg[e]] == k && (d.eLR[eg[e]] & 3) == e;
      esg[e] = (own[e] ? 1.0 : -1.0) * d.IIE[e * sK + k];
    }
    double al = 0.0, be = 0.0, ga = 0.0;
    if (s >= 0 && s < 4) stage_coeffs(s, al, be, ga);
    const double dt = s < 0 ? 0.0 : (a.localDT ? a.dtK[k] : a.dtS[s]);
    double abar = 0.0;
#pragma unroll 1
    for (int n = 0; n < 4; ++n) {
      double rb[NP];
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        const size_t ind = (n * NP + r) * sK + k;
        const double qb = a.Qbn[ind];
        if (s < 0) {
          rb[r] = qb;
        } else if (s == 4) {
          rb[r] = kSSP[4][4] * dt * qb;
          a.Rb3[ind] = kSSP[4][3] * dt * qb;
          dtb += qb * (kSSP[4][3] * a.rhs3[ind] + kSSP[4][4] * a.rhs[ind]);
          a.Qb2[ind] = kSSP[4][0] * qb;
          a.Qb3[ind] = kSSP[4][1] * qb;
          a.Qbs[ind] = kSSP[4][2] * qb;
        } else {
          rb[r] = ga * dt * qb + (s == 3 ? a.Rb3[ind] : 0.0);
          dtb += ga * qb * a.rhs[ind];
          if (s == 3) a.Qb0[ind] = al * qb;
          else a.Qb0[ind] += al * qb;
          if (s == 1) a.Qbs[ind] = be * qb;
          else if (be != 0.0) a.Qbs[ind] += be * qb;
        }
      }
      // filter u = V diag(1, mf (1 - a)) Vinv u_pre:  u_pre_bar = Vinv^T diag(..) V^T rb
      double m[NP], w[NP];
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        double acc = 0.0, acc2 = 0.0;
#pragma unroll
        for (int r = 0; r < NP; ++r) {
          acc += sV[r * NP + i] * rb[r];
          acc2 += sVi[i * NP + r] * x.rhsPre[(n * NP + r) * sK + k];
        }
        m[i] = acc;
        w[i] = acc2;
      }
#pragma unroll
      for (int i = 1; i < NP; ++i) {
        abar -= m[i] * smf[i] * w[i];
        m[i] *= smf[i] * (1.0 - alpha);
      }
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        double acc = 0.0;
#pragma unroll
        for (int i = 0; i < NP; ++i) acc += sVi[i * NP + r] * m[i];
        rb[r] = acc;
        x.RbE[(n * NP + r) * sK + k] = acc;
      }
      // u_pre = RHS_E + DivInt DOF / |J|:  DOF_bar = DivInt^T u_pre_bar / |J|
#pragma unroll 1
      for (int j = 0; j < NP; ++j) {
        double fr = 0.0, fs = 0.0;
#pragma unroll
        for (int r = 0; r < NP; ++r) {
          fr += sD[r * NF + j] * rb[r];
          fs += sD[r * NF + NP + j] * rb[r];
        }
        fr *= oojd;
        fs *= oojd;
        const size_t ind = (n * NR + j) * sK + k;
        x.DissXbar[ind] = Jd * (J0 * fr + J2 * fs);
        x.DissYbar[ind] = Jd * (J1 * fr + J3 * fs);
      }
#pragma unroll 1
      for (int e = 0; e < 3; ++e) {
        double* vfb = x.VFbar + (static_cast<size_t>(eg[e]) * 4 + n) * NE;
#pragma unroll
        for (int p = 0; p < NE; ++p) {
          double dd = 0.0;
#pragma unroll
          for (int r = 0; r < NP; ++r) dd += sD[r * NF + 2 * NP + e * NE + p] * rb[r];
          atomicAdd(&vfb[own[e] ? p : NE - 1 - p], oojd * dd * esg[e]);
        }
      }
    }
    x.alphaBar[k] = abar;
    if (s >= 0 && a.localDT) a.dtOwnK[k] = dtb;
  }
  if (s >= 0 && !a.localDT) {
    const double t = warp_sum(active ? dtb : 0.0);
    if ((threadIdx.x & 31) == 0) atomicAdd(&a.dtbarG[s], t);
  }
}

// Viscous edge flux and viscous speed in reverse (k_diss_edge).
template <int N>
__global__ void __launch_bounds__(128) k_adj_diss_edge(DissArgs d, AdjDissArgs x) {
  constexpr int NP = DissDims<N>::NP, NE = DissDims<N>::NE, NE3 = DissDims<N>::NE3;
  constexpr int NF = DissDims<N>::NF, NR = DissDims<N>::NR;
  __shared__ double sB[NF * 3];
  stage_operator(sB, d.Bary, NF * 3);
  __syncthreads();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= d.nInt + d.nBC) return;
  const size_t sK = static_cast<size_t>(d.K);
  const int kL = d.ekL[g], eL = d.eLR[g] & 3;
  const double nx = d.enx[g], ny = d.eny[g];
  const double oohK = d.eoohK[g];
  double evL[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) evL[v] = vdouble(d.epsV, d.etov[v * sK + kL]);
  double epsL[NE], ebL[NE];
#pragma unroll
  for (int p = 0; p < NE; ++p) {
    const int r = 2 * NP + eL * NE + p;
    epsL[p] = sB[r * 3] * evL[0] + sB[r * 3 + 1] * evL[1] + sB[r * 3 + 2] * evL[2];
    ebL[p] = 0.0;
  }
  // viscSpeed = max_p oohK^2 eps_L[p]: the adjoint goes to the point that set it
  const double vsb = x.vsBar[g];
  if (vsb != 0.0) {
    double vm = -1.7976931348623157e308;
    int pm = 0;
#pragma unroll
    for (int p = 0; p < NE; ++p) {
      const double w = oohK * oohK * epsL[p];
      if (w > vm) { vm = w; pm = p; }
    }
#pragma unroll
    for (int p = 0; p < NE; ++p)
      if (p == pm) ebL[p] += oohK * oohK * vsb;
  }
  const double* vfb = x.VFbar + static_cast<size_t>(g) * 4 * NE;
  if (g >= d.nInt) {
#pragma unroll 1
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const size_t ind = (n * NR + NP + eL * NE + p) * sK + kL;
        x.DissXbar[ind] = nx * vfb[n * NE + p];
        x.DissYbar[ind] = ny * vfb[n * NE + p];
      }
  } else {
    const int kR = d.ekR[g], eR = d.eLR[g] >> 2;
    double evR[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) evR[v] = vdouble(d.epsV, d.etov[v * sK + kR]);
    const double len = (eL == 1) ? 2.0 * sqrt(2.0) * d.eIIL[g] : 2.0 * d.eIIL[g];
    const double c = d.omega / len;
    double epsR[NE], ebR[NE];
#pragma unroll
    for (int q = 0; q < NE; ++q) {
      const int r = 2 * NP + eR * NE + q;
      epsR[q] = sB[r * 3] * evR[0] + sB[r * 3 + 1] * evR[1] + sB[r * 3 + 2] * evR[2];
      ebR[q] = 0.0;
    }
#pragma unroll 1
    for (int n = 0; n < 4; ++n) {
      double qfb[NE];
#pragma unroll
      for (int p = 0; p < NE; ++p) qfb[p] = 0.0;
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const double vb = vfb[n * NE + p];
        const size_t indL = (n * NR + NP + eL * NE + p) * sK + kL;
        const size_t indR = (n * NR + NP + eR * NE + (NE - 1 - p)) * sK + kR;
        x.DissXbar[indL] = 0.5 * nx * vb;
        x.DissYbar[indL] = 0.5 * ny * vb;
        x.DissXbar[indR] = 0.5 * nx * vb;
        x.DissYbar[indR] = 0.5 * ny * vb;
        const double lam = 0.5 * (epsL[p] + epsR[NE - 1 - p]);
        const double qa = d.QF[(n * NE3 + eL * NE + p) * sK + kL];
        const double qb = d.QF[(n * NE3 + eL * NE + (NE - 1 - p)) * sK + kL];
        const double lamb = -c * (qa - qb) * vb;
        ebL[p] += 0.5 * lamb;
        ebR[NE - 1 - p] += 0.5 * lamb;
        qfb[p] -= c * lam * vb;
        qfb[NE - 1 - p] += c * lam * vb;
      }
#pragma unroll
      for (int p = 0; p < NE; ++p) x.QFb[(n * NE3 + eL * NE + p) * sK + kL] += qfb[p];
    }
    double wR[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < NE; ++q) {
      const int r = 2 * NP + eR * NE + q;
#pragma unroll
      for (int v = 0; v < 3; ++v) wR[v] += sB[r * 3 + v] * ebR[q];
    }
#pragma unroll
    for (int v = 0; v < 3; ++v)
      if (wR[v] != 0.0) atomicAdd(&x.epsVbar[d.etov[v * sK + kR]], wR[v]);
  }
  double wL[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int p = 0; p < NE; ++p) {
    const int r = 2 * NP + eL * NE + p;
#pragma unroll
    for (int v = 0; v < 3; ++v) wL[v] += sB[r * 3 + v] * ebL[p];
  }
#pragma unroll
  for (int v = 0; v < 3; ++v)
    if (wL[v] != 0.0) atomicAdd(&x.epsVbar[d.etov[v * sK + kL]], wL[v]);
}

// eps * grad(Q) in reverse (k_diss_grad): the interior state, the stored left
// face states and the vertex eps.
template <int N>
__global__ void __launch_bounds__(128) k_adj_diss_grad(DissArgs d, AdjDissArgs x, double* Qbs) {
  constexpr int NP = DissDims<N>::NP, NE = DissDims<N>::NE, NE3 = DissDims<N>::NE3;
  constexpr int NF = DissDims<N>::NF, NR = DissDims<N>::NR;
  extern __shared__ double smem[];
  double* sDiv = smem;                 // NF x NF
  double* sB = smem + NF * NF;         // NF x 3
  stage_operator(sDiv, d.Div, NF * NF);
  stage_operator(sB, d.Bary, NF * 3);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.K) return;
  const size_t sK = static_cast<size_t>(d.K);
  const double J0 = d.Jinv[k], J1 = d.Jinv[sK + k], J2 = d.Jinv[2 * sK + k], J3 = d.Jinv[3 * sK + k];
  const double ooJd = 1.0 / d.Jdet[k];
  double ev[3], mx[3], my[3];
  int eg[3], eLn[3], kl[3];
  bool own[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) ev[v] = vdouble(d.epsV, d.etov[v * sK + k]);
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    eg[e] = d.elemEdge[e * sK + k];
    own[e] = d.ekL[eg[e]] == k && (d.eLR[eg[e]] & 3) == e;
    eLn[e] = d.eLR[eg[e]] & 3;
    kl[e] = d.ekL[eg[e]];
    const double ii = d.IIE[e * sK + k];
    mx[e] = ooJd * d.nxE[e * sK + k] * ii;
    my[e] = ooJd * d.nyE[e * sK + k] * ii;
  }
  double evb[3] = {0.0, 0.0, 0.0};
#pragma unroll 1
  for (int n = 0; n < 4; ++n) {
    double U[NP], Ue[NE3], Ub[NP], Ueb[NE3];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      U[i] = d.Qs[(n * NP + i) * sK + k];
      Ub[i] = 0.0;
    }
#pragma unroll
    for (int e = 0; e < 3; ++e)
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const int ii = own[e] ? p : NE - 1 - p;
        Ue[e * NE + p] = d.QF[(n * NE3 + eLn[e] * NE + ii) * sK + kl[e]];
        Ueb[e * NE + p] = 0.0;
      }
#pragma unroll 1
    for (int rr = 0; rr < NR; ++rr) {
      const int r = rr < NP ? rr : 2 * NP + (rr - NP);
      const double* row = sDiv + r * NF;
      double A = 0.0, B = 0.0, C[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int j = 0; j < NP; ++j) {
        A += row[j] * U[j];
        B += row[NP + j] * U[j];
      }
#pragma unroll
      for (int e = 0; e < 3; ++e)
#pragma unroll
        for (int p = 0; p < NE; ++p) C[e] += row[2 * NP + e * NE + p] * Ue[e * NE + p];
      const double gx = J0 * A + J2 * B + mx[0] * C[0] + mx[1] * C[1] + mx[2] * C[2];
      const double gy = J1 * A + J3 * B + my[0] * C[0] + my[1] * C[1] + my[2] * C[2];
      const double epsr = sB[r * 3] * ev[0] + sB[r * 3 + 1] * ev[1] + sB[r * 3 + 2] * ev[2];
      const double xb = x.DissXbar[(n * NR + rr) * sK + k], yb = x.DissYbar[(n * NR + rr) * sK + k];
      const double eb = gx * xb + gy * yb;
#pragma unroll
      for (int v = 0; v < 3; ++v) evb[v] += sB[r * 3 + v] * eb;
      const double gxb = epsr * xb, gyb = epsr * yb;
      const double Ab = J0 * gxb + J1 * gyb, Bb = J2 * gxb + J3 * gyb;
#pragma unroll
      for (int j = 0; j < NP; ++j) Ub[j] += row[j] * Ab + row[NP + j] * Bb;
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        const double Cb = mx[e] * gxb + my[e] * gyb;
#pragma unroll
        for (int p = 0; p < NE; ++p) Ueb[e * NE + p] += row[2 * NP + e * NE + p] * Cb;
      }
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) Qbs[(n * NP + i) * sK + k] += Ub[i];
#pragma unroll
    for (int e = 0; e < 3; ++e)
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const int ii = own[e] ? p : NE - 1 - p;
        atomicAdd(&x.QFb[(n * NE3 + eLn[e] * NE + ii) * sK + kl[e]], Ueb[e * NE + p]);
      }
  }
#pragma unroll
  for (int v = 0; v < 3; ++v)
    if (evb[v] != 0.0) atomicAdd(&x.epsVbar[d.etov[v * sK + k]], evb[v]);
}

// The rkStep-2 limiter in reverse, one thread per (variable, element): the
// stage-2 state adjoint moves through V diag(1, mf (1 - a)) Vinv transposed,
// and the limiter's share of the a-adjoint is added.
template <int N>
__global__ void __launch_bounds__(128) k_adj_diss_limit(DissArgs d, AdjDissArgs x) {
  constexpr int NP = DissDims<N>::NP;
  __shared__ double sV[NP * NP], sVi[NP * NP], smf[NP];
  stage_operator(sV, d.V, NP * NP);
  stage_operator(sVi, d.Vinv, NP * NP);
  stage_operator(smf, d.mf, NP);
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * d.K) return;
  const int n = t / d.K, k = t - n * d.K;
  const size_t sK = static_cast<size_t>(d.K);
  const double alpha = sin(0.5 * 3.14159265358979323846 * vert_sigma_mean(d, k, sK));
  double qb[NP], q[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    qb[i] = x.Qlim[(n * NP + i) * sK + k];
    q[i] = x.Q2pre[(n * NP + i) * sK + k];
  }
  double m[NP], w[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    double acc = 0.0, acc2 = 0.0;
#pragma unroll
    for (int r = 0; r < NP; ++r) {
      acc += sV[r * NP + i] * qb[r];
      acc2 += sVi[i * NP + r] * q[r];
    }
    m[i] = acc;
    w[i] = acc2;
  }
  double abar = 0.0;
#pragma unroll
  for (int i = 1; i < NP; ++i) {
    abar -= m[i] * smf[i] * w[i];
    m[i] *= smf[i] * (1.0 - alpha);
  }
#pragma unroll
  for (int r = 0; r < NP; ++r) {
    double acc = 0.0;
#pragma unroll
    for (int i = 0; i < NP; ++i) acc += sVi[i * NP + r] * m[i];
    x.Qlim[(n * NP + r) * sK + k] = acc;
  }
  atomicAdd(&x.alphaBar[k], abar);
}

// a = sin(pi sigma_bar / 2), sigma_bar = mean of the vertex sigV: to the vertices.
static __global__ void k_adj_diss_alpha(DissArgs d, AdjDissArgs x) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.K) return;
  const size_t sK = static_cast<size_t>(d.K);
  const double ab = x.alphaBar[k];
  if (ab == 0.0) return;
  const double pi = 3.14159265358979323846;
  const double sb = ab * 0.5 * pi * cos(0.5 * pi * vert_sigma_mean(d, k, sK)) / 3.0;
#pragma unroll
  for (int v = 0; v < 3; ++v) atomicAdd(&x.sigVbar[d.etov[v * sK + k]], sb);
}

// Sensor in reverse (k_diss_sensor): vertex adjoints to the element that set
// the max, eps = Eps0 hK sigma, the sine ramp, log10(num / den), the three
// modal products, into the density adjoint.
template <int N>
__global__ void __launch_bounds__(128) k_adj_diss_sensor(DissArgs d, AdjDissArgs x, double* Qbsens) {
  constexpr int NP = DissDims<N>::NP;
  __shared__ double sP[NP * NP], sM[NP * NP], sDq[NP * NP];
  stage_operator(sP, d.SensP, NP * NP);
  stage_operator(sM, d.Mass, NP * NP);
  stage_operator(sDq, d.SensD, NP * NP);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.K) return;
  const size_t sK = static_cast<size_t>(d.K);
  double sb = 0.0, eb = 0.0;
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const int vert = d.etov[v * sK + k];
    if (x.sigArg[vert] == k) sb += x.sigVbar[vert];
    if (x.epsArg[vert] == k) eb += x.epsVbar[vert];
  }
  sb += d.eps0 * d.hK[k] * eb;
  const double se = x.SeE[k];
  const double left = d.S0 - d.kappa, right = d.S0 + d.kappa;
  if (sb == 0.0 || !(se >= left && se <= right)) return;  // flat parts of the ramp, or a NaN moment
  const double w = 3.14159265358979323846 * (0.5 / d.kappa);
  const double seb = sb * 0.5 * cos(w * (se - d.S0)) * w;
  double rho[NP], xv[NP], yv[NP], dq[NP];
#pragma unroll
  for (int j = 0; j < NP; ++j) rho[j] = x.Qsens[j * sK + k];
  double num = 0.0, den = 0.0;
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    double a = 0.0, b = 0.0, c = 0.0;
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      a += sP[i * NP + j] * rho[j];
      b += sM[i * NP + j] * rho[j];
      c += sDq[i * NP + j] * rho[j];
    }
    xv[i] = a;
    yv[i] = b;
    dq[i] = c;
    num += c * a;
    den += rho[i] * b;
  }
  const double ln10 = 2.302585092994045684;
  const double numb = seb / (ln10 * num), denb = -seb / (ln10 * den);
#pragma unroll
  for (int j = 0; j < NP; ++j) {
    double r = denb * yv[j];
#pragma unroll
    for (int i = 0; i < NP; ++i)
      r += sDq[i * NP + j] * numb * xv[i] + sP[i * NP + j] * numb * dq[i] + sM[i * NP + j] * denb * rho[i];
    Qbsens[j * sK + k] += r;
  }
}

}  // namespace gcfd
