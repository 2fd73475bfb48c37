// physics.cuh -- FP64 point physics shared by the stage kernels and the point
// entry points.  Each function states the reference routine it computes; the algebra
// is regrouped to spend fewer FP64 instructions (one reciprocal of rho per point,
// contravariant fluxes formed directly, viscous and AV fluxes fused), so results
// agree with the reference to rounding, not bit for bit.
#pragma once
#include <cuda_runtime.h>

namespace chorus {

constexpr double kLambda = -2.0 / 3.0;  // setup2d.f90:70
constexpr double kPrandt = 0.72;        // setup2d.f90:71

// 1/x for the positive, normal densities of the path: the hardware approximation
// r (PTX rcp.approx.ftz.f64, relative error e = 1 - x r below 2^-19.9 over 2^28 sampled
// normal x) refined by one third-order step of the series 1/x = r/(1 - e) =
// r(1 + e + e^2 + ...): r <- r + r(e + e^2), leaving a relative error of about e^3
// (2^-60) below the rounding of the last FMA.  Measured on the same sample: within one
// ulp of the IEEE quotient 1.0/x (0.03% of values one ulp off), in 3 FP64 FMAs against
// the longer IEEE-rounded division sequence.
__host__ __device__ __forceinline__ double rcp_pos(double x) {
#ifdef __CUDA_ARCH__
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
#else
  return 1.0 / x;
#endif
}

// x/2 without an FP64 instruction: decrement the exponent field (exact for normal
// numbers, the same value as 0.5*x); zeros, subnormals, infinities and NaNs take the
// multiply.  0.5*a + 0.5*b == half(a + b) bit for bit for normal operands.
__host__ __device__ __forceinline__ double half(double x) {
#ifdef __CUDA_ARCH__
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  return (ex > 1 && ex < 0x7FF) ? __longlong_as_double(b - (1LL << 52)) : 0.5 * x;
#else
  return 0.5 * x;
#endif
}

// -x as a sign-bit flip: a negation that no add or multiply absorbs would otherwise
// take an FP64 instruction
__host__ __device__ __forceinline__ double negate(double x) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ULL);
#else
  return -x;
#endif
}

// x * s for s = +-1 as a sign-bit flip (integer pipe, exact)
__host__ __device__ __forceinline__ double times_sign(double x, double s) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(__double_as_longlong(x) ^ (__double_as_longlong(s) & (long long)0x8000000000000000ULL));
#else
  return x * s;
#endif
}

// Contravariant ideal-MHD flux F*sx + G*sy of getIfluxvectors (getrusanov.f90:111-153)
// as used by inviscid_flux_interior (compflux.f90:77-78, 96-97).  Written in the
// momenta: with m = (ru, rv, rw), the mass flux m.s, the normal velocity (m.s)/rho and
// the normal field over rho, Bn/rho, give every term without forming u, v, w
// (u*Bn = ru*(Bn/rho), u.B = (m.B)/rho, rho|u|^2 = |m|^2/rho), 40 FP64 operations.
__host__ __device__ __forceinline__ void iflux_contra(const double* q, double sx, double sy, double gm1,
                                                      double* F) {
  const double rho = q[0], ru = q[1], rv = q[2], rw = q[3], E = q[4], Bx = q[5], By = q[6], Bz = q[7];
  const double ri = rcp_pos(rho);
  const double F0 = ru * sx + rv * sy;  // rho * Un
  const double Un = F0 * ri;
  const double Bn = Bx * sx + By * sy;
  const double bn = Bn * ri;            // Bn / rho
  const double B2 = Bx * Bx + By * By + Bz * Bz;
  const double m2 = ru * ru + rv * rv + rw * rw;
  const double hB2 = half(B2);
  const double pg = gm1 * (E - half(m2) * ri - hB2);
  const double pt = pg + hB2;
  const double mB = ru * Bx + rv * By + rw * Bz;
  F[0] = F0;
  F[1] = ru * Un + pt * sx - Bx * Bn;
  F[2] = rv * Un + pt * sy - By * Bn;
  F[3] = rw * Un - Bz * Bn;
  F[4] = (E + pt) * Un - mB * bn;
  F[5] = Bx * Un - ru * bn;
  F[6] = By * Un - rv * bn;
  F[7] = Bz * Un - rw * bn;
}

// Rusanov flux of getrusanovflux (getrusanov.f90:1-109) along the unit normal (ux,uy),
// times `scale`: Fh = scale*(Fl + Fr - eigv*(qr - ql)); with scale = magnorm*sign_l/2
// this is the reference's Fnl in the left cell's computational frame (:90-93).  Returns
// the left normal velocity (for the A_z upwinding, :99-103) and the wave-speed bound
// eigv (:87).
__host__ __device__ __forceinline__ void rusanov_core(const double* ql, const double* qr, double ux, double uy,
                                                      double gam, double scale, double* Fh, double& vnl,
                                                      double& eigv) {
  const double gm1 = gam - 1.0;
  double Fl[8], Fr[8], pgl, pgr, vn[2];
  const double* qs[2] = {ql, qr};
  double* Fs[2] = {Fl, Fr};
  double* pg[2] = {&pgl, &pgr};
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const double* q = qs[side];
    double* F = Fs[side];
    const double ri = rcp_pos(q[0]);
    const double u = ri * q[1], v = ri * q[2], w = ri * q[3];
    const double Bx = q[5], By = q[6], Bz = q[7];
    const double B2 = Bx * Bx + By * By + Bz * Bz;
    const double p = gm1 * (q[4] - 0.5 * q[0] * (u * u + v * v + w * w) - B2 * 0.5);
    const double pt = p + 0.5 * B2;
    const double Vn = u * ux + v * uy;
    const double Bn = Bx * ux + By * uy;
    F[0] = q[0] * Vn;
    F[1] = q[1] * Vn + pt * ux - Bx * Bn;
    F[2] = q[2] * Vn + pt * uy - By * Bn;
    F[3] = q[3] * Vn - Bz * Bn;
    F[4] = (q[4] + pt) * Vn - Bn * (u * Bx + v * By + w * Bz);
    F[5] = (v * Bx - u * By) * uy;
    F[6] = (u * By - v * Bx) * ux;
    F[7] = Bz * Vn - w * Bn;
    *pg[side] = p;
    vn[side] = Vn;
  }
  const double Bx = 0.5 * (ql[5] + qr[5]), By = 0.5 * (ql[6] + qr[6]), Bz = 0.5 * (ql[7] + qr[7]);
  const double irs = rcp_pos(ql[0] + qr[0]);
  const double ca = gam * (pgl + pgr) * irs;
  const double cd = (Bx * Bx + By * By + Bz * Bz) * (2.0 * irs);
  const double bn = Bx * ux + By * uy;
  const double cn = bn * bn * (2.0 * irs);
  const double cad = ca + cd;
  const double ctmp = sqrt(cad * cad - 4.0 * ca * cn);
  const double cf = sqrt(0.5 * (cad + ctmp));
  eigv = 0.5 * fabs(vn[0] + vn[1]) + cf;
#pragma unroll
  for (int k = 0; k < 8; k++) Fh[k] = scale * fma(-eigv, qr[k] - ql[k], Fl[k] + Fr[k]);
  vnl = vn[0];
}

// Contravariant viscous + resistive + artificial-viscosity flux at one flux point:
// getVfluxvectors (getrusanov.f90:157-249) with (mu, eta0) plus getVfluxvectors_AV
// (:251-360) with (mu_art, 0), summed (the hydrodynamic terms are linear in the
// viscosity) and contracted with the metric row (sx, sy) as in comp_viscous_flux
// (compflux.f90:216-225, 241-250).  g is nablaQ(9,2) in Fortran order; only
// components 1..7 of the result are nonzero (Fv(1) = Fv(9) = 0).
__host__ __device__ __forceinline__ void vflux_contra(const double* q, const double* g, double mut, double eta0,
                                                      double gam, double sx, double sy, double* Fc) {
  const double rho = q[0], Bx = q[5], By = q[6], Bz = q[7];
  const double ri = rcp_pos(rho);
  const double u = q[1] * ri, v = q[2] * ri, w = q[3] * ri;
  const double NU = u * u + v * v + w * w;
  const double B2 = Bx * Bx + By * By + Bz * Bz;
  const double inte = (q[4] - 0.5 * NU * rho - 0.5 * B2) * ri;
  double du[2], dv[2], dw[2], de[2];
#pragma unroll
  for (int d = 0; d < 2; d++) {
    const double* gd = g + 9 * d;
    const double dr = gd[0];
    du[d] = (gd[1] - dr * u) * ri;
    dv[d] = (gd[2] - dr * v) * ri;
    dw[d] = (gd[3] - dr * w) * ri;
    const double dke = 0.5 * NU * dr + rho * (u * du[d] + v * dv[d] + w * dw[d]);
    const double dpb = Bx * gd[5] + By * gd[6] + Bz * gd[7];
    de[d] = (gd[4] - dke - dpb - dr * inte) * ri;
  }
  const double ux = du[0], uy = du[1], vx = dv[0], vy = dv[1];
  const double div = ux + vy;
  const double kq = mut * gam / kPrandt;
  const double f1 = mut * (2.0 * ux + kLambda * div);
  const double f2 = mut * (vx + uy);
  const double f3 = mut * dw[0];
  const double g2 = mut * (2.0 * vy + kLambda * div);
  const double g3 = mut * dw[1];
  double f4 = u * f1 + v * f2 + w * f3 + kq * de[0];
  double g4 = f2 * u + g2 * v + g3 * w + kq * de[1];
  // resistive terms (eta0 only; the AV form has eta_art = 0)
  const double Jx = g[9 + 7], Jy = -g[7], Jz = g[6] - g[9 + 5];
  const double f6 = eta0 * Jz, f7 = -eta0 * Jy;
  const double g5 = -eta0 * Jz, g7 = eta0 * Jx;
  f4 = f4 + f6 * By + f7 * Bz;
  g4 = g4 + g5 * Bx + g7 * Bz;
  Fc[0] = 0.0;
  Fc[1] = f1 * sx + f2 * sy;
  Fc[2] = f2 * sx + g2 * sy;
  Fc[3] = f3 * sx + g3 * sy;
  Fc[4] = f4 * sx + g4 * sy;
  Fc[5] = g5 * sy;
  Fc[6] = f6 * sx;
  Fc[7] = f7 * sx + g7 * sy;
}

// muAV of variable 1 (AV.f90:157-172 with se_low=-6, se_high=-1) from the sensor sum
// ssum = sum ((Qsm-rho)/rho)^2 of a cell, Se = log10(ssum): zero below 1e-6, epsilon0
// above 0.1 (the ramp is continuous at both ends), the sine ramp in between.
__host__ __device__ __forceinline__ double av_mu(double ssum, double eps0) {
  if (ssum < 1e-6) return 0.0;
  if (ssum > 0.1) return eps0;
  const double se = log10(ssum);
  const double s0 = -3.5, kr = 2.5, pi = 3.14159265358979323846;
  return eps0 / 2.0 * (1.0 + sin(pi * (se - s0) / 2.0 / kr));
}

}  // namespace chorus
