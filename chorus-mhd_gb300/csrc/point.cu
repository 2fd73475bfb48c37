// point.cu -- device evaluation of the reference's point routines over n points
// (getrusanovflux, getIfluxvectors, getVfluxvectors) and the deterministic
// diagnostic reduction.
#include <cuda_runtime.h>

#include "chorus_internal.h"
#include "physics.cuh"

namespace chorus {

// getrusanovflux (getrusanov.f90:1-109) with the reference's argument list
__global__ void k_point_rusanov(int n, double gam, const double* Qfl, const double* Qfr, double* Fnl, double* Fnr,
                                double* Az, const double* normf, const int* sl, const int* sr, double* ev) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double n1 = normf[2 * i], n2 = normf[2 * i + 1];
  const double mag = sqrt(n1 * n1 + n2 * n2);
  const int sign_l = sl[i], sign_r = sr[i];
  const double ux = n1 / mag * sign_l, uy = n2 / mag * sign_l;
  double ql[9], qr[9], Fh[8], vnl, e;
  for (int k = 0; k < 9; k++) { ql[k] = Qfl[9 * i + k]; qr[k] = Qfr[9 * i + k]; }
  const double msl = mag * sign_l, ss = (double)(sign_l * sign_r);
  rusanov_core(ql, qr, ux, uy, gam, 0.5 * msl, Fh, vnl, e);
  for (int k = 0; k < 8; k++) {
    Fnl[8 * i + k] = Fh[k];
    Fnr[8 * i + k] = times_sign(Fh[k], ss);
  }
  Az[i] = vnl > 0.0 ? ql[8] : qr[8];
  ev[i] = e;
}

// getIfluxvectors (getrusanov.f90:111-153): F and G are the contravariant flux with
// metric rows (1,0) and (0,1)
__global__ void k_point_iflux(int n, double gam, const double* Qi, double* Fi, double* Gi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double q[8];
  for (int k = 0; k < 8; k++) q[k] = Qi[8 * i + k];
  iflux_contra(q, 1.0, 0.0, gam - 1.0, Fi + 8 * i);
  iflux_contra(q, 0.0, 1.0, gam - 1.0, Gi + 8 * i);
}

// getVfluxvectors (getrusanov.f90:157-249), physical F and G
__global__ void k_point_vflux(int n, double gam, double mu, double eta0, const double* Qv, const double* nQ,
                              double* Fv, double* Gv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double q[9], g[18], F[8], G[8];
  for (int k = 0; k < 9; k++) q[k] = Qv[9 * i + k];
  for (int k = 0; k < 18; k++) g[k] = nQ[18 * i + k];
  vflux_contra(q, g, mu, eta0, gam, 1.0, 0.0, F);
  vflux_contra(q, g, mu, eta0, gam, 0.0, 1.0, G);
  for (int k = 0; k < 8; k++) { Fv[9 * i + k] = F[k]; Gv[9 * i + k] = G[k]; }
  Fv[9 * i + 8] = 0.0;
  Gv[9 * i + 8] = 0.0;
}

// getVfluxvectors_AV (getrusanov.f90:251-360): the viscous flux with mu_art linear in
// the flux-point coordinate between the cell's two face viscosities of the family
// (:273-281), eta_art = 0; physical F and G.  Indices are 1-based as in the reference
// and were range-checked on the host.  muf[4c + side-1] holds the face viscosity of
// local face side (1..4) of cell c.
__global__ void k_point_vflux_av(int n, double gam, PointAxes ax, const double* muf, const int* fam,
                                 const int* ifp, const int* jfp, const int* ic, const double* Qv, const double* nQ,
                                 double* Fv, double* Gv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* mf = muf + 4 * (size_t)(ic[i] - 1);
  double mu_art;
  if (fam[i] == 1) {
    const double xsi = ax.Xf[ifp[i] - 1];
    mu_art = mf[3] * (1.0 - xsi) + mf[1] * xsi;  // muAVfi(1,1,ic), muAVfi(1,2,ic)
  } else {
    const double eta = ax.Xf[jfp[i] - 1];
    mu_art = mf[0] * (1.0 - eta) + mf[2] * eta;  // muAVfj(1,1,ic), muAVfj(1,2,ic)
  }
  double q[9], g[18], F[8], G[8];
  for (int k = 0; k < 9; k++) q[k] = Qv[9 * i + k];
  for (int k = 0; k < 18; k++) g[k] = nQ[18 * i + k];
  vflux_contra(q, g, mu_art, 0.0, gam, 1.0, 0.0, F);
  vflux_contra(q, g, mu_art, 0.0, gam, 0.0, 1.0, G);
  for (int k = 0; k < 8; k++) { Fv[9 * i + k] = F[k]; Gv[9 * i + k] = G[k]; }
  Fv[9 * i + 8] = 0.0;
  Gv[9 * i + 8] = 0.0;
}

// sum of diag[e][0] and diag[e][1] over cells in a fixed order (one block)
__global__ void __launch_bounds__(1024) k_reduce_diag(const double* diag, int nc, double* out) {
  __shared__ double s0[1024], s1[1024];
  double a = 0.0, b = 0.0;
  for (int e = threadIdx.x; e < nc; e += blockDim.x) {
    a += diag[2 * e];
    b += diag[2 * e + 1];
  }
  s0[threadIdx.x] = a;
  s1[threadIdx.x] = b;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s0[threadIdx.x] += s0[threadIdx.x + w];
      s1[threadIdx.x] += s1[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s0[0];
    out[1] = s1[0];
  }
}

void launch_point_rusanov(int n, double gam, const double* Qfl, const double* Qfr, double* Fnl, double* Fnr,
                          double* Az, const double* normf, const int* sl, const int* sr, double* ev, cudaStream_t st) {
  if (n > 0) k_point_rusanov<<<(n + 127) / 128, 128, 0, st>>>(n, gam, Qfl, Qfr, Fnl, Fnr, Az, normf, sl, sr, ev);
}
void launch_point_iflux(int n, double gam, const double* Qi, double* Fi, double* Gi, cudaStream_t st) {
  if (n > 0) k_point_iflux<<<(n + 127) / 128, 128, 0, st>>>(n, gam, Qi, Fi, Gi);
}
void launch_point_vflux(int n, double gam, double mu, double eta0, const double* Qv, const double* nQ, double* Fv,
                        double* Gv, cudaStream_t st) {
  if (n > 0) k_point_vflux<<<(n + 127) / 128, 128, 0, st>>>(n, gam, mu, eta0, Qv, nQ, Fv, Gv);
}
void launch_point_vflux_av(int n, double gam, const PointAxes& ax, const double* muf, const int* fam, const int* ifp,
                           const int* jfp, const int* ic, const double* Qv, const double* nQ, double* Fv, double* Gv,
                           cudaStream_t st) {
  if (n > 0)
    k_point_vflux_av<<<(n + 127) / 128, 128, 0, st>>>(n, gam, ax, muf, fam, ifp, jfp, ic, Qv, nQ, Fv, Gv);
}
// Qvf variable 9 (the reference's Qvfi(9)/Qvfj(9)) from the compact A_z traces
__global__ void k_qvf9(const double* Azf, double* Qvf, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) Qvf[i * 9 + 8] = Azf[i];
}

void launch_qvf9(const SolveDev& s, cudaStream_t st) {
  const size_t n = (size_t)s.NC * 2 * (s.N + 1) * s.N;
  if (n > 0) k_qvf9<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s.Azf, s.Qvf, n);
}

void launch_reduce_diag(const double* diag, int NC, double* out2, cudaStream_t st) {
  k_reduce_diag<<<1, 1024, 0, st>>>(diag, NC, out2);
}

}  // namespace chorus
