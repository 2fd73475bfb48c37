// kernels.cuh -- stage kernels of the residual-and-time-step path, templated on N.
//
// One RK stage (compresid.f90:1-67 + the stage update of iterations.f90:162-217) is
// four launches, one per grid-wide dependency level of the reference's compflux:
//   E1  cell pass  Q -> flux-point values (all 2N(N+1) points), interior inviscid
//                  flux, interior A_z, AV sensor           inviscid_flux_interior,
//                                                          comp_artificial_viscosity
//   F1  face pass  Rusanov flux on every face point, upwinded A_z, face-averaged Q,
//                  max wave speed                          interfaceflux, CYCLOCFLUX,
//                                                          BCFLUX, getrusanovflux
//   E2  cell pass  face AV viscosities; grad Q (vars 1-8) at the solution and flux
//                  points of the cells that carry viscous work
//                                                          compAVflux, nablaQsp,
//                                                          nablaQ_interior_FP
//   E3  cell pass  viscous + AV flux with the face-averaged grad Q traces, divergence,
//                  grad A_z, A_z advection, RK update      interfaceVISflux,
//                                                          comp_viscous_flux, nablaAsp,
//                                                          compresid, RK_S5P3
// (k_f2 stores the face-averaged grad Q traces only when they are downloaded.)
// Cell passes stage a block of `epb` cells in shared memory; face passes run one
// thread per face point.  Values are IEEE doubles throughout; the fixed line operators
// (Lmat interpolation, Mmat differentiation, which carry no data-dependent
// coefficients) run as exact integer dot products on the integer pipes (fixdot.cuh),
// all other arithmetic is FP64.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "chorus_internal.h"
#include "fixdot.cuh"
#include "physics.cuh"

namespace chorus {

constexpr int kHalfF = kMaxN / 2 + 1;  // flux points up to the middle of a line
constexpr int kHalfS = kMaxN / 2;      // mirrored pairs of solution points

// wait for the predecessor grid of a programmatic (PDL) launch: its completion and its
// memory; a no-op for a launch without the attribute
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch with programmatic stream serialization: the kernel may be scheduled while its
// predecessor on the stream drains, and waits (griddepcontrol.wait, at its entry) for
// the predecessor's completion and memory before touching any of its data.  Hides the
// launch gap between dependent passes; the wait is hardware-managed.
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}


struct OpsN {
  double L[(kMaxN + 1) * kMaxN];  // Lmat(N+1,N) column-major
  double M[(kMaxN + 1) * kMaxN];  // Mmat(N+1,N)
  double A[kMaxN * kMaxN];        // AV smoothing operator A[i*N+m] (projection to N-1 points and back)
  double Xf[kMaxN + 1];
  double Xs[kMaxN];
  // Lmat split by the mirror symmetry of the points (Xs and Xf symmetric about 1/2):
  // for flux point f <= N/2 and solution pair (j, N-1-j),
  //   CE[f][j] = (L(f,j) + L(f,N-1-j))/2,  CO[f][j] = (L(f,j) - L(f,N-1-j))/2,
  // LMID[f] = L(f,(N-1)/2) for odd N; then with e_j = q_j + q_{N-1-j},
  // o_j = q_j - q_{N-1-j}: Qf(f) = E + O and Qf(N-f) = E - O,
  // E = sum CE e + LMID q_mid, O = sum CO o.
  double CE[kHalfF * kHalfS];
  double CO[kHalfF * kHalfS];
  double LMID[kHalfF];
  // the integer form of Lmat (fixdot.cuh) in mirror form (fix_mirror_coefs, sigma = +1,
  // C(f, j) = L(f, j): rows f <= N/2 of N limbs) at scale 2^LS
  int LH[(kMaxN + 1) * kMaxN];
  int LL[(kMaxN + 1) * kMaxN];
  int LS;
  // and of Mmat (sigma = -1, C(i, r) = M(r, i), the weight of flux point r in the
  // derivative at solution point i: rows i < (N+1)/2 of N+1 limbs) at scale 2^MS
  int MH[(kMaxN + 1) * kMaxN];
  int ML[(kMaxN + 1) * kMaxN];
  int MS;
};

// one copy per translation unit; upload_ops_n<N>() fills it
static __constant__ OpsN c_ops;

// operator accessors: the per-N kernels read their translation unit's single table,
// the multi-solve kernels one table per N
struct OpsTU {
  __device__ static const OpsN& ops() { return c_ops; }
};

template <int N>
struct D {
  static constexpr int NS = N * N;
  static constexpr int NF1 = (N + 1) * N;
  static constexpr int NFP = 2 * NF1;
};

// element-local flux-point index of face point nfp (0-based) of local face lf (1..4),
// from face2fpconnec (initsetup.f90:343-379)
template <int N>
__device__ __forceinline__ int face_fp(int lf, int nfp) {
  constexpr int NF1 = D<N>::NF1;
  switch (lf) {
    case 1: return NF1 + nfp;                   // family 2, ifp = nfp,     jfp = 1
    case 2: return nfp * (N + 1) + N;           // family 1, ifp = N+1,     jfp = nfp
    case 3: return NF1 + N * N + (N - 1 - nfp); // family 2, ifp = N-nfp+1, jfp = N+1
    default: return (N - 1 - nfp) * (N + 1);    // family 1, ifp = 1,       jfp = N-nfp+1
  }
}

// the inverse of face_fp: the local face (1..4) of element flux point fp and its
// position nfp along that face; 0 for an interior flux point
template <int N>
__device__ __forceinline__ int fp_face(int fp, int& nfp) {
  constexpr int NF1 = D<N>::NF1;
  if (fp < NF1) {
    const int ifp = fp % (N + 1), jfp = fp / (N + 1);
    if (ifp == 0) { nfp = N - 1 - jfp; return 4; }
    if (ifp == N) { nfp = jfp; return 2; }
    return 0;
  }
  const int r = fp - NF1, ifp = r % N, jfp = r / N;
  if (jfp == 0) { nfp = ifp; return 1; }
  if (jfp == N) { nfp = N - 1 - ifp; return 3; }
  return 0;
}

__device__ __forceinline__ unsigned long long ev_bits(double ev, unsigned int* err) {
  if (!(ev >= 0.0) || ev > 1.0e300) {  // NaN or inf wave speed: non-physical state
    atomicOr(err, 1u);
    return 0ull;
  }
  return (unsigned long long)__double_as_longlong(ev);
}

__device__ __forceinline__ void block_max_ull(unsigned long long v, unsigned long long* out) {
  __shared__ unsigned long long red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? red[lane] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
      v = w > v ? w : v;
    }
    if (lane == 0 && v) atomicMax(out, v);
  }
}

// ---------------------------------------------------------------------------
// E1: flux-point values, interior inviscid flux, AV sensor
// ---------------------------------------------------------------------------
// sum of v over the lanes of a warp (all lanes must call)
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// dst[0..n) = src[0..n) by the whole CTA, in 16-byte pieces when both are 16-byte
// aligned (the branch is uniform over the CTA)
__device__ __forceinline__ void block_copy(double* dst, const double* src, int n) {
  if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
    const double2* s2 = reinterpret_cast<const double2*>(src);
    double2* d2 = reinterpret_cast<double2*>(dst);
#pragma unroll 4
    for (int i = threadIdx.x; i < (n >> 1); i += blockDim.x) d2[i] = s2[i];
    if ((n & 1) && threadIdx.x == 0) dst[n - 1] = src[n - 1];
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
  }
}

// element-local flux-point index of the i-th interior flux point (i < 2N(N-1)):
// family 1 with ifp = 1..N-1, then family 2 with jfp = 1..N-1
template <int N>
__device__ __forceinline__ int interior_fp(int i) {
  constexpr int H = N * (N - 1);
  if (i < H) {
    const int jfp = i / (N - 1), ifp = 1 + i % (N - 1);
    return jfp * (N + 1) + ifp;
  }
  const int r = i - H, jfp = 1 + r / N, ifp = r % N;
  return D<N>::NF1 + jfp * N + ifp;
}

// interpolation along one line from the N solution values to the N+1 flux points,
// y_f = sum_j L(f,j) v_j: the integer form (fixdot.cuh), or FP64 for a line with
// non-finite or huge values, where the mirror symmetry of the points halves the
// multiplications (see OpsN::CE)
template <int N, class O>
__device__ __forceinline__ void interp_line(const double (&v)[N], double (&y)[N + 1]) {
  const int emax = fix_emax(v);
  if (emax <= kFixEmaxFast) {
    fix_apply_mirror<N + 1, N, 1>(v, emax, O::ops().LH, O::ops().LL, emax - 1017 - kFixG - O::ops().LS, y);
    return;
  }
  double ev[N / 2 > 0 ? N / 2 : 1], od[N / 2 > 0 ? N / 2 : 1];
#pragma unroll
  for (int j = 0; j < N / 2; j++) {
    ev[j] = v[j] + v[N - 1 - j];
    od[j] = v[j] - v[N - 1 - j];
  }
#pragma unroll
  for (int f = 0; f <= N / 2; f++) {
    double E = (N & 1) ? O::ops().LMID[f] * v[(N - 1) / 2] : 0.0;
    double Od = 0.0;
#pragma unroll
    for (int j = 0; j < N / 2; j++) {
      E += O::ops().CE[f * kHalfS + j] * ev[j];
      Od += O::ops().CO[f * kHalfS + j] * od[j];
    }
    y[f] = E + Od;
    if (f != N - f) y[N - f] = E - Od;
  }
}

// the derivative along one line, y_i = sum_r M(r,i) x_r (i < N) from the N+1 flux values
// x_r = x[r*xs]: the integer form (fixdot.cuh), or FP64 for a line with non-finite or
// huge values
template <int N, class O>
__device__ __forceinline__ void deriv_line(const double* x, int xs, double (&y)[N]) {
  double v[N + 1];
#pragma unroll
  for (int r = 0; r <= N; r++) v[r] = x[r * xs];
  const int emax = fix_emax(v);
  if (emax <= kFixEmaxFast) {
    fix_apply_mirror<N, N + 1, -1>(v, emax, O::ops().MH, O::ops().ML, emax - 1017 - kFixG - O::ops().MS, y);
  } else {
#pragma unroll
    for (int i = 0; i < N; i++) {
      double a = 0.0;
#pragma unroll
      for (int r = 0; r <= N; r++) a += O::ops().M[r + (N + 1) * i] * v[r];
      y[i] = a;
    }
  }
}

// ---------------------------------------------------------------------------
// E3: viscous + AV flux, divergence, A_z advection, RK update
// ---------------------------------------------------------------------------
template <int N, class O>
__device__ __forceinline__ void e1_body(const SolveDev& s, int e0, int cnt, int epb, int sensor, double* sm) {
  constexpr int NS = D<N>::NS, NF1 = D<N>::NF1, NFP = D<N>::NFP, NINT = 2 * N * (N - 1);
  double* sQ = sm;                    // [epb][NS][9]   cell states (16-byte aligned)
  double* sT = sQ + epb * NS * 9;     // [epb][NS]      sensor scratch
  double* sU = sT + epb * NS;         // [epb][NS]
  double* sV = sU + epb * NS;         // [epb][NFP][9]  flux-point values
  double* sA = sV + epb * NFP * 9;    // AV smoothing operator (N, N)
  // all global traffic of the pass is contiguous block copies (coalesced)
  block_copy(sQ, s.Q + (size_t)e0 * NS * 9, cnt * NS * 9);
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) sA[i] = O::ops().A[i];
  __syncthreads();
  // interpolation to every flux point, one (cell, line, variable) per thread so that
  // every lane of every warp does work; the line operator runs on the integer pipes,
  // which the FP64 work of the pass leaves idle
  for (int t = threadIdx.x; t < cnt * 2 * N * 9; t += blockDim.x) {
    const int k = t % 9, el = t / 9, e = el / (2 * N), line = el - e * 2 * N;
    const double* q = sQ + e * NS * 9 + k;
    const bool fam1 = line < N;
    const int ln = fam1 ? line : line - N;
    // solution values along the line and where the line's flux values go
    const double* qb = fam1 ? q + ln * N * 9 : q + ln * 9;
    const int qs = fam1 ? 9 : N * 9;
    double* ob = sV + (e * NFP + (fam1 ? ln * (N + 1) : NF1 + ln)) * 9 + k;
    const int os = fam1 ? 9 : N * 9;
    double v[N], y[N + 1];
#pragma unroll
    for (int sp = 0; sp < N; sp++) v[sp] = qb[sp * qs];
    interp_line<N, O>(v, y);
#pragma unroll
    for (int f = 0; f <= N; f++) ob[f * os] = y[f];
  }
  __syncthreads();
  // contravariant inviscid flux at the interior flux points only (face points of Fc and
  // Azf belong to the face pass), written straight out: consecutive threads take
  // consecutive interior points, whose 64-byte flux records mostly adjoin
  const double gm1 = s.gam - 1.0;
  for (int t = threadIdx.x; t < cnt * NINT; t += blockDim.x) {
    const int e = t / NINT, fp = interior_fp<N>(t - e * NINT);
    const double* qf = sV + (e * NFP + fp) * 9;
    const size_t g = (size_t)(e0 + e) * NFP + fp;
    const double2 m = reinterpret_cast<const double2*>(s.met)[g];  // 16-byte metric pair
    double F[8];
    iflux_contra(qf, m.x, m.y, gm1, F);
    double2* fo = reinterpret_cast<double2*>(s.Fc + g * 8);  // 64-byte flux record
#pragma unroll
    for (int k = 0; k < 4; k++) fo[k] = make_double2(F[2 * k], F[2 * k + 1]);
    s.Azf[g] = qf[8];
  }
  {
    block_copy(s.Qvf + (size_t)e0 * NFP * 9, sV, cnt * NFP * 9);
  }
  if (!sensor) {
    if (s.skip)
      for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
        s.act[e0 + e] = 0;
        s.nv[e0 + e] = 0;
      }
    return;
  }
  // AV sensor of variable 1 (AV.f90:15-82): Qsm = A rho A^T, sum ((Qsm-rho)/rho)^2.
  // Se = log10(sum) is compared with -6 and -1 only; the sum itself is kept (Se < -6
  // exactly when sum < 1e-6) and the logarithm is taken where the ramp needs it.
  for (int t = threadIdx.x; t < cnt * NS; t += blockDim.x) {
    const int e = t / NS, p = t - e * NS, is = p % N, n = p / N;
    const double* q = sQ + e * NS * 9;
    double a = 0.0;
#pragma unroll
    for (int m = 0; m < N; m++) a += sA[is * N + m] * q[(n * N + m) * 9];
    sT[e * NS + p] = a;  // T(is, n)
  }
  __syncthreads();
  for (int t = threadIdx.x; t < cnt * NS; t += blockDim.x) {
    const int e = t / NS, p = t - e * NS, is = p % N, js = p / N;
    double a = 0.0;
#pragma unroll
    for (int n = 0; n < N; n++) a += sA[js * N + n] * sT[e * NS + n * N + is];
    const double rho = sQ[(e * NS + p) * 9];
    const double d = (a - rho) * rcp_pos(rho);
    sU[e * NS + p] = d * d;
  }
  __syncthreads();
  // one warp per cell sums its points
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int e = warp; e < cnt; e += nwarp) {
    double acc = 0.0;
    for (int p = lane; p < NS; p += 32) acc += sU[e * NS + p];
    acc = warp_sum(acc);
    if (lane == 0) {
      s.Se[e0 + e] = acc;
      if (s.skip) {
        const int a = (acc < 1e-6) ? 0 : 1;  // NaN counts as active
        s.act[e0 + e] = a;
        s.nv[e0 + e] = a;
      }
    }
  }
  if (!(sensor & 2)) return;
  // the same sensor of variable 6 (B_x), whose muAV(6) only the plot output reads
  // (tecplotter.f90:39 from AV.f90:60-73); in the reference's division form, so a zero
  // B_x gives the reference's inf or NaN
  __syncthreads();
  for (int t = threadIdx.x; t < cnt * NS; t += blockDim.x) {
    const int e = t / NS, p = t - e * NS, is = p % N, n = p / N;
    const double* q = sQ + e * NS * 9 + 5;
    double a = 0.0;
#pragma unroll
    for (int m = 0; m < N; m++) a += sA[is * N + m] * q[(n * N + m) * 9];
    sT[e * NS + p] = a;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < cnt * NS; t += blockDim.x) {
    const int e = t / NS, p = t - e * NS, is = p % N, js = p / N;
    double a = 0.0;
#pragma unroll
    for (int n = 0; n < N; n++) a += sA[js * N + n] * sT[e * NS + n * N + is];
    const double b = sQ[(e * NS + p) * 9 + 5];
    sU[e * NS + p] = ((a - b) * (a - b)) / (b * b);
  }
  __syncthreads();
  for (int e = warp; e < cnt; e += nwarp) {
    double acc = 0.0;
    for (int p = lane; p < NS; p += 32) acc += sU[e * NS + p];
    acc = warp_sum(acc);
    if (lane == 0) s.Se6[e0 + e] = acc;
  }
}

// cells [c0, c1) of the solve, epb per CTA
template <int N>
__global__ void __launch_bounds__(512, 2) k_e1(SolveDev s, int epb, int sensor, int c0, int c1) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  // bit 4: the first pass of a stage, which starts the stage's wave-speed maximum
  if ((sensor & 4) && c0 == 0 && blockIdx.x == 0 && threadIdx.x == 0) *s.eig = 0ull;
  sensor &= 3;
  const int e0 = c0 + blockIdx.x * epb;
  const int cnt = min(epb, c1 - e0);
  if (cnt <= 0) return;
  if ((sensor & 2) && !*s.plot_flag) sensor &= 1;  // the plot's sensor only when asked for
  e1_body<N, OpsTU>(s, e0, cnt, epb, sensor, sm);
}

// cells of this CTA whose gradients (mode 0) or viscous fluxes (mode 1) are needed,
// compacted into a shared list; returns the count
__device__ __forceinline__ int active_cells(const SolveDev& s, int e0, int cnt, int mode, int* list) {
  // the first warp tests 32 cells at a time (their flag loads in flight together) and
  // compacts them in cell order with a ballot
  __shared__ int n_act;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    int n = 0;
    for (int base = 0; base < cnt; base += 32) {
      const int e = base + lane;
      int need = 0;
      if (e < cnt) {
        const int c = e0 + e;
        need = 1;
        if (s.skip) {
          need = s.nv[c];
          if (mode == 0) {
            const int4 b = s.nbr[c];
            const int nx = b.x >= 0 ? s.nv[b.x] : 0, ny = b.y >= 0 ? s.nv[b.y] : 0;
            const int nz = b.z >= 0 ? s.nv[b.z] : 0, nw = b.w >= 0 ? s.nv[b.w] : 0;
            need |= nx | ny | nz | nw;
          }
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, need != 0);
      if (need) list[n + __popc(m & ((1u << lane) - 1u))] = e;
      n += __popc(m);
    }
    if (lane == 0) n_act = n;
  }
  __syncthreads();
  return n_act;
}

// ---------------------------------------------------------------------------
// F1: Rusanov flux on every face point (interfaceflux / CYCLOCFLUX / BCFLUX)
// ---------------------------------------------------------------------------
// one face point t of the solve's two-sided (t < nface2*N) then FREE face points;
// returns the bit pattern of its wave speed for the block max
template <int N>
__device__ __forceinline__ unsigned long long f1_point(const SolveDev& s, int t) {
  constexpr int NFP = D<N>::NFP;
  const int n2 = s.nface2 * N, n1 = s.nface1 * N;
  unsigned long long evb = 0ull;
  if (t < n2 + n1) {
    const bool two = t < n2;
    const int tt = two ? t : t - n2;
    const int f = tt / N, nfp = tt - f * N;
    size_t gl, gr = 0;
    FaceNorm fn;
    if (two) {
      const int4 fc = s.face2[f];
      gl = (size_t)fc.x * NFP + face_fp<N>(fc.y, nfp);
      gr = (size_t)fc.z * NFP + face_fp<N>(fc.w, N - 1 - nfp);
      fn = s.fn2[tt];
    } else {
      const int2 fc = s.face1[f];
      gl = (size_t)fc.x * NFP + face_fp<N>(fc.y, nfp);
      fn = s.fn1[tt];
    }
    double ql[9], qr[9];
    const double* pl = s.Qvf + gl * 9;
#pragma unroll
    for (int k = 0; k < 9; k++) ql[k] = pl[k];
    if (two) {
      const double* pr = s.Qvf + gr * 9;
#pragma unroll
      for (int k = 0; k < 9; k++) qr[k] = pr[k];
    } else {
#pragma unroll
      for (int k = 0; k < 9; k++) qr[k] = ql[k];
    }
    double Fh[8], vnl, ev;
    rusanov_core(ql, qr, fn.ux, fn.uy, s.gam, fn.msl, Fh, vnl, ev);
    evb = ev_bits(ev, s.err);
    const double az = vnl > 0.0 ? ql[8] : qr[8];
    double2* fl = reinterpret_cast<double2*>(s.Fc + gl * 8);  // 64-byte flux records
#pragma unroll
    for (int k = 0; k < 4; k++) fl[k] = make_double2(Fh[2 * k], Fh[2 * k + 1]);
    s.Azf[gl] = az;
    if (two && s.skip && nfp == 0) {
      const int4 fc = s.face2[f];
      if (s.act[fc.x] | s.act[fc.z]) {
        s.nv[fc.x] = 1;
        s.nv[fc.z] = 1;
      }
    }
    if (two) {
      double2* fr = reinterpret_cast<double2*>(s.Fc + gr * 8);
#pragma unroll
      for (int k = 0; k < 4; k++) fr[k] = make_double2(times_sign(Fh[2 * k], fn.ss), times_sign(Fh[2 * k + 1], fn.ss));
      s.Azf[gr] = az;
      double* al = s.Qvf + gl * 9;
      double* ar = s.Qvf + gr * 9;
#pragma unroll
      for (int k = 0; k < 9; k++) {
        const double a = half(ql[k] + qr[k]);
        al[k] = a;
        ar[k] = a;
      }
    }
  }
  return evb;
}

// face points [t2, t2 + n2) of the two-sided list, then [t1, t1 + n - n2) of the FREE list
// (f1_point numbering: the FREE faces follow the two-sided ones)
template <int N>
__global__ void __launch_bounds__(256, 3) k_f1(SolveDev s, int t2, int n2, int t1, int n) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long evb = 0ull;
  if (i < n) evb = f1_point<N>(s, i < n2 ? t2 + i : t1 + (i - n2));
  block_max_ull(evb, s.eig);
}

// ---------------------------------------------------------------------------
// E2: gradients at solution points and their values at every flux point
// ---------------------------------------------------------------------------
// the AV viscosity on the four faces of cell c (compAVflux / interfaceAVflux /
// cyclocAVflux, AV.f90:199-303, 494-564): the mean of the two cells' muAV(1) on a
// two-sided face (the same bits from either side: the sum commutes), the cell's own on a
// FREE face; muAV(1) from the stage's sensor and epsilon0 = eigvmax h/(N-1) (AV.f90:147)
template <int N>
__device__ __forceinline__ void cell_face_mu(const SolveDev& s, int c) {
  double m[4] = {0.0, 0.0, 0.0, 0.0};
  if (s.artiv) {
    const double eps0 = __longlong_as_double((long long)*s.eig) * s.hmsh / (double)(N - 1) * 1.0;
    const double mc = av_mu(s.Se[c], eps0);
    const int4 b = s.nbr[c];
    const int o[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
    for (int k = 0; k < 4; k++) m[k] = o[k] >= 0 ? 0.5 * (mc + av_mu(s.Se[o[k]], eps0)) : mc;
  }
#pragma unroll
  for (int k = 0; k < 4; k++) s.muf[4 * c + k] = m[k];
}

template <int N, class O>
__device__ __forceinline__ void e2_cells(const SolveDev& s, const int* cells, int n, double* sm) {
  // gradients of the n (<= epb) listed cells; grad A_z (nablaAsp) is computed with the
  // divergence in the last pass.  nablaQsp (compflux.f90:107-157) in its conservative
  // form: grad_x Q = (1/J) [d/dxi (S1(1,1) Q) + d/deta (S2(2,1) Q)], grad_y the same with
  // the second metric entries, i.e. the divergence of the products of the face-corrected
  // flux-point states with the metric terms, differentiated along the lines on the
  // integer pipes as in E3.
  constexpr int NS = D<N>::NS, NF1 = D<N>::NF1, NFP = D<N>::NFP;
  double* sP = sm;                // [n][NFP][16] Q_k * (S_x, S_y): k + 8 d
  double* sG = sP + n * NFP * 16;  // [n][NS][16] grad Q (d*8 + k)
  double* sJ = sG + n * NS * 16;   // [n][NS] 1/J
  for (int i = threadIdx.x; i < n * NFP * 8; i += blockDim.x) {
    const int le = i / (NFP * 8), r = i - le * (NFP * 8), fp = r >> 3, k = r & 7;
    const size_t g = (size_t)cells[le] * NFP + fp;
    const double q = s.Qvf[g * 9 + k];
    sP[(le * NFP + fp) * 16 + k] = q * s.met[2 * g];
    sP[(le * NFP + fp) * 16 + 8 + k] = q * s.met[2 * g + 1];
  }
  for (int i = threadIdx.x; i < n * NS; i += blockDim.x) {
    const int le = i / NS, p = i - le * NS;
    sJ[i] = s.invJ[(size_t)cells[le] * NS + p];
  }
  __syncthreads();
  // grad Q (variables 1-8) at the solution points: one (cell, line, quantity) per thread,
  // the xi lines first, then the eta lines adding to them and scaling by 1/J
#pragma unroll 1
  for (int fam = 0; fam < 2; fam++) {
    for (int t = threadIdx.x; t < n * N * 16; t += blockDim.x) {
      const int c = t & 15, el = t >> 4, le = el / N, ln = el - le * N;
      const int fp0 = fam ? NF1 + ln : ln * (N + 1), fps = fam ? N : 1;
      double y[N];
      deriv_line<N, O>(sP + (le * NFP + fp0) * 16 + c, fps * 16, y);
      const int p0 = fam ? ln : ln * N, ps = fam ? N : 1;
      double* g = sG + (le * NS + p0) * 16 + c;
      if (!fam) {
#pragma unroll
        for (int i = 0; i < N; i++) g[i * ps * 16] = y[i];
      } else {
        double* out = s.nQs + ((size_t)cells[le] * NS + p0) * 18 + (c < 8 ? c : c + 1);
#pragma unroll
        for (int i = 0; i < N; i++) {
          const double a = (g[i * ps * 16] + y[i]) * sJ[le * NS + p0 + i * ps];
          g[i * ps * 16] = a;
          out[(size_t)i * ps * 18] = a;
        }
      }
    }
    __syncthreads();
  }
  // grad Q at every flux point (nablaQ_interior_FP + face traces): one (cell, line,
  // component) per thread, the line operator on the integer pipes as in E1
  for (int t = threadIdx.x; t < n * 2 * N * 16; t += blockDim.x) {
    const int c = t & 15, el = t >> 4, le = el / (2 * N), line = el - le * 2 * N;
    const bool fam1 = line < N;
    const int ln = fam1 ? line : line - N;
    const double* gb = sG + (le * NS + (fam1 ? ln * N : ln)) * 16 + c;
    const int gs = fam1 ? 16 : N * 16;
    const int f0 = fam1 ? ln * (N + 1) : NF1 + ln, fs = fam1 ? 1 : N;
    double* ob = s.nQvf + ((size_t)cells[le] * NFP + f0) * 18 + (c < 8 ? c : c + 1);
    double v[N], y[N + 1];
#pragma unroll
    for (int sp = 0; sp < N; sp++) v[sp] = gb[sp * gs];
    interp_line<N, O>(v, y);
#pragma unroll
    for (int f = 0; f <= N; f++) ob[(size_t)f * fs * 18] = y[f];
  }
}

// tile form (batched kernels): the cells of [e0, e0+cnt) whose gradients are needed
template <int N, class O>
__device__ __forceinline__ void e2_body(const SolveDev& s, int e0, int cnt, int epb, double* sm) {
  __shared__ int list[64];
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) cell_face_mu<N>(s, e0 + e);
  const int nact = active_cells(s, e0, cnt, 0, list);
  if (nact == 0) return;
  for (int i = threadIdx.x; i < nact; i += blockDim.x) list[i] += e0;
  __syncthreads();
  e2_cells<N, O>(s, list, nact, sm);
}

// does cell c need its gradients (itself or a face neighbour has viscous work)?
__device__ __forceinline__ bool needs_gradients(const SolveDev& s, int c) {
  if (!s.skip || s.nv[c]) return true;
  const int4 b = s.nbr[c];
  return (b.x >= 0 && s.nv[b.x]) || (b.y >= 0 && s.nv[b.y]) || (b.z >= 0 && s.nv[b.z]) || (b.w >= 0 && s.nv[b.w]);
}

// E2 over a chunk of `chunk` (<= blockDim.x) cells starting at c0: every thread tests
// one cell, the CTA compacts the cells that need gradients into an ordered list and runs
// them in groups of epb, so chunks without viscous work cost one coalesced test
template <int N, class O>
__device__ __forceinline__ void e2_chunk(const SolveDev& s, int c0, int chunk, int epb, double* sm) {
  __shared__ int list[512];
  __shared__ int woff[17];
  const int c = c0 + threadIdx.x;
  const bool mine = (int)threadIdx.x < chunk && c < s.NC;
  if (mine) cell_face_mu<N>(s, c);
  const bool need = mine && needs_gradients(s, c);
  const unsigned m = __ballot_sync(0xffffffffu, need);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) woff[w + 1] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    woff[0] = 0;
    for (int i = 1; i <= (int)(blockDim.x >> 5); i++) woff[i] += woff[i - 1];
  }
  __syncthreads();
  if (need) list[woff[w] + __popc(m & ((1u << lane) - 1u))] = c;
  const int n = woff[blockDim.x >> 5];
  __syncthreads();
  for (int g = 0; g < n; g += epb) {
    e2_cells<N, O>(s, list + g, min(epb, n - g), sm);
    __syncthreads();
  }
}

template <int N>
__global__ void __launch_bounds__(512) k_e2(SolveDev s, int epb, int chunk) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  e2_chunk<N, OpsTU>(s, blockIdx.x * chunk, chunk, epb, sm);
}
// ---------------------------------------------------------------------------
// F2: face-averaged gradients and face AV viscosity
// ---------------------------------------------------------------------------
// face averages of the grad Q traces in place (interfaceVISflux, CYCLOCVISFLUX).  The
// stage itself averages them where the viscous flux reads them (E3); this pass makes the
// stored traces equal to the reference's nablaQvfi/nablaQvfj when they are downloaded.
template <int N>
__device__ __forceinline__ void f2_point(const SolveDev& s, int t) {
  constexpr int NFP = D<N>::NFP;
  if (t >= s.nface2 * N) return;
  const int f = t / N, nfp = t - f * N;
  const int4 fc = s.face2[f];
  double* a = s.nQvf + ((size_t)fc.x * NFP + face_fp<N>(fc.y, nfp)) * 18;
  double* b = s.nQvf + ((size_t)fc.z * NFP + face_fp<N>(fc.w, N - 1 - nfp)) * 18;
#pragma unroll
  for (int d = 0; d < 2; d++)
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const double v = half(a[9 * d + k] + b[9 * d + k]);
      a[9 * d + k] = v;
      b[9 * d + k] = v;
    }
}

template <int N>
__global__ void __launch_bounds__(256) k_f2(SolveDev s) {
  f2_point<N>(s, blockIdx.x * blockDim.x + threadIdx.x);
}

template <int N, class O>
__device__ __forceinline__ void e3_body(const SolveDev& s, int e0, int cnt, int epb, const RKStage& rk, int update, double* sm) {
  constexpr int NS = D<N>::NS, NF1 = D<N>::NF1, NFP = D<N>::NFP;

  double* sF = sm;                  // [epb][NFP][8] F - Fv, the negated total flux
  double* sD = sF + epb * NFP * 8;  // [epb][NS] diagnostic partial sums
  double* sR = sD + epb * NS;       // [epb][NS][9] residual
  double* sJ = sR + epb * NS * 9;   // [epb][NS] 1/J
  double* sZ = sJ + epb * NS;       // [epb][NFP][2] A_z * (S_x, S_y) at the flux points
  double* sN = sZ + epb * NFP * 2;  // [epb][NS][2] grad A_z
  __shared__ int list[64];
  const int nact = active_cells(s, e0, cnt, 1, list);
  {
    // contiguous block copies (coalesced), issued together so their latencies overlap;
    // the state itself is read where it is used (the update is elementwise over the
    // block's contiguous state)
    // (16-byte loads: Fc's per-cell block and each metric pair are 16-byte aligned)
    const double2* fi = reinterpret_cast<const double2*>(s.Fc + (size_t)e0 * NFP * 8);
    double2* sF2 = reinterpret_cast<double2*>(sF);
#pragma unroll 4
    for (int i = threadIdx.x; i < cnt * NFP * 4; i += blockDim.x) sF2[i] = fi[i];
    for (int i = threadIdx.x; i < cnt * NS; i += blockDim.x) sJ[i] = s.invJ[(size_t)e0 * NS + i];
    const double2* met2 = reinterpret_cast<const double2*>(s.met);
    for (int i = threadIdx.x; i < cnt * NFP; i += blockDim.x) {
      const size_t g = (size_t)e0 * NFP + i;
      const double z = s.Azf[g];
      const double2 m = met2[g];
      sZ[2 * i] = z * m.x;
      sZ[2 * i + 1] = z * m.y;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nact * NFP; t += blockDim.x) {
    const int le = t / NFP, fp = t - le * NFP, e = list[le], c = e0 + e;
    const size_t g = (size_t)c * NFP + fp;
    double mut = s.mu;
    if (s.artiv) {
      const double* mf = s.muf + 4 * c;
      if (fp < NF1) {
        const double x = O::ops().Xf[fp % (N + 1)];
        mut += mf[3] * (1.0 - x) + mf[1] * x;
      } else {
        const double x = O::ops().Xf[(fp - NF1) / N];
        mut += mf[0] * (1.0 - x) + mf[2] * x;
      }
    }
    if (mut != 0.0 || s.eta0 != 0.0) {
      double q[9], gq[18], Fv[8];
      const double* pq = s.Qvf + g * 9;
      const double* pg = s.nQvf + g * 18;
#pragma unroll
      for (int k = 0; k < 8; k++) q[k] = pq[k];
      q[8] = 0.0;
      // on a two-sided face the trace of grad Q is the mean of both sides'
      // (interfaceVISflux / CYCLOCVISFLUX, interfaceflux_all.f90:118-199,
      // cyclocflux_all.f90:118-208); a FREE face keeps its own (BCVISFLUX)
      int nfp = 0;
      const int lf = fp_face<N>(fp, nfp);
      const int o = lf ? (&s.nbr[c].x)[lf - 1] : -1;
      if (o >= 0) {
        const int olf = (&s.nbrlf[c].x)[lf - 1];
        const double* po = s.nQvf + ((size_t)o * NFP + face_fp<N>(olf, N - 1 - nfp)) * 18;
#pragma unroll
        for (int k = 0; k < 8; k++) {
          gq[k] = half(pg[k] + po[k]);
          gq[9 + k] = half(pg[9 + k] + po[9 + k]);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 8; k++) {
          gq[k] = pg[k];
          gq[9 + k] = pg[9 + k];
        }
      }
      gq[8] = 0.0;
      gq[17] = 0.0;
      vflux_contra(q, gq, mut, s.eta0, s.gam, s.met[2 * g], s.met[2 * g + 1], Fv);
      double* d = sF + (e * NFP + fp) * 8;
#pragma unroll
      for (int k = 1; k < 8; k++) d[k] -= Fv[k];
    }
  }
  __syncthreads();
  // divergence of the total flux and grad A_z in the conservative form of nablaAsp
  // (magnetic_potential.f90:1-42), (1/J) sum_r Mmat (A_z S): ten line quantities per
  // cell (eight flux components, two A_z S components), each differentiated along its
  // lines on the integer pipes, one (cell, line, quantity) per thread; first the
  // family-1 lines (xi), then the family-2 lines (eta), which add to them and scale by
  // 1/J
  constexpr int NQ = 10;
#pragma unroll 1
  for (int fam = 0; fam < 2; fam++) {
    for (int t = threadIdx.x; t < cnt * N * NQ; t += blockDim.x) {
      const int k = t % NQ, el = t / NQ, e = el / N, ln = el - e * N;
      const bool fl = k < 8;
      // flux point r of line ln: family 1 at ln*(N+1) + r, family 2 at NF1 + r*N + ln
      const int fp0 = fam ? NF1 + ln : ln * (N + 1), fps = fam ? N : 1;
      const double* x = fl ? sF + (e * NFP + fp0) * 8 + k : sZ + (e * NFP + fp0) * 2 + (k - 8);
      double y[N];
      deriv_line<N, O>(x, fl ? fps * 8 : fps * 2, y);
      // solution point i of line ln: family 1 at ln*N + i, family 2 at i*N + ln
      const int p0 = e * NS + (fam ? ln : ln * N), ps = fam ? N : 1;
      double* out = fl ? sR + p0 * 9 + k : sN + p0 * 2 + (k - 8);
      const int os = fl ? ps * 9 : ps * 2;
      if (!fam) {
#pragma unroll
        for (int i = 0; i < N; i++) out[i * os] = fl ? negate(y[i]) : y[i];  // the flux enters negated
      } else {
#pragma unroll
        for (int i = 0; i < N; i++) {
          const double a = (fl ? out[i * os] - y[i] : out[i * os] + y[i]) * sJ[p0 + i * ps];
          out[i * os] = a;
          if (!fl) s.nAs[((size_t)e0 * NS + p0 + i * ps) * 2 + (k - 8)] = a;
        }
      }
    }
    __syncthreads();
  }
  // A_z advection (resid(9), compresid.f90:45-47) at every solution point
  for (int t = threadIdx.x; t < cnt * NS; t += blockDim.x) {
    const double* q = s.Q + ((size_t)e0 * NS + t) * 9;
    const double ri = rcp_pos(q[0]);
    const double ax = sN[2 * t] - s.B0y, ay = sN[2 * t + 1] + s.B0x;
    sR[t * 9 + 8] = negate(q[1] * ri * ax + q[2] * ri * ay);
  }
  if (rk.diag) {
    __syncthreads();
    for (int t = threadIdx.x; t < cnt * NS; t += blockDim.x) {
      const double* r = sR + t * 9;
      double acc = 0.0;
#pragma unroll
      for (int k = 0; k < 9; k++) acc += r[k] * r[k];
      sD[t] = acc;
    }
  }
  __syncthreads();
  // stage update, elementwise over the block's contiguous state (RK_S5P3 / FiveStageRk):
  // a streaming loop whose few FP64 operations hide under its memory traffic (the
  // integer form of fixdot.cuh measured slower here)
  {
    const size_t g0 = (size_t)e0 * NS * 9;
    const int n = cnt * NS * 9;
#pragma unroll 4
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const size_t g = g0 + i;
      const double q = s.Q[g], r = sR[i];
      if (rk.write_resid) s.resid[g] = r;
      if (!update) continue;
      double qn = rk.cQ * q + rk.cR * r;
      for (int j = 0; j < rk.nsrc; j++) qn += rk.c[j] * rk.src[j][g];
      if (rk.R0) qn += rk.cR0 * rk.R0[g];
      s.Q[g] = qn;
      if (rk.save_old) rk.save_old[g] = q;
      if (rk.save_new) rk.save_new[g] = qn;
      if (rk.save_R) rk.save_R[g] = r;
    }
  }
  if (rk.diag) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int e = warp; e < cnt; e += nwarp) {
      double acc = 0.0;
      for (int p = lane; p < NS; p += 32) acc += sD[e * NS + p];
      acc = warp_sum(acc);
      if (lane == 0) s.diag[2 * (e0 + e)] = acc;
    }
  }
}

template <int N>
__global__ void __launch_bounds__(512) k_e3(SolveDev s, RKStage rk, int epb, int update, int c0, int c1) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  const int e0 = c0 + blockIdx.x * epb;
  const int cnt = min(epb, c1 - e0);
  if (cnt <= 0) return;
  e3_body<N, OpsTU>(s, e0, cnt, epb, rk, update, sm);
}

// ---------------------------------------------------------------------------
// CT projection (correct_B_via_curl_Az, setinitialcond.f90:82-91)
//   mode 0: A_z at every flux point (into Qvf variable 9)
//   mode 2: grad A_z from the face-averaged values, B <- B0 + curl A_z
// (mode 1, the face average, is k_ctface)
// ---------------------------------------------------------------------------
template <int N, class O>
__device__ __forceinline__ void ct_elem_body(const SolveDev& s, int e0, int cnt, int epb, int mode, double* sm) {
  constexpr int NS = D<N>::NS, NF1 = D<N>::NF1, NFP = D<N>::NFP;
  // the A_z traces go to Azf only, which the gradient below reads coalesced; the
  // reference's Qvfi(9)/Qvfj(9) are filled from Azf where they are read (downloads,
  // nablaQsp(9,9)), so the pass makes no strided writes into Qvf
  if (mode == 0) {
    double* sA = sm;  // [epb][NS] A_z at the solution points
    for (int i = threadIdx.x; i < cnt * NS; i += blockDim.x) sA[i] = s.Q[((size_t)e0 * NS + i) * 9 + 8];
    __syncthreads();
    // one (cell, line) per thread, the line operator on the integer pipes as in E1
    for (int t = threadIdx.x; t < cnt * 2 * N; t += blockDim.x) {
      const int e = t / (2 * N), line = t - e * 2 * N;
      const bool fam1 = line < N;
      const int ln = fam1 ? line : line - N;
      const double* qb = sA + e * NS + (fam1 ? ln * N : ln);
      const int qs = fam1 ? 1 : N;
      const int f0 = fam1 ? ln * (N + 1) : NF1 + ln, fs = fam1 ? 1 : N;
      double v[N], y[N + 1];
#pragma unroll
      for (int sp = 0; sp < N; sp++) v[sp] = qb[sp * qs];
      interp_line<N, O>(v, y);
      double* az = s.Azf + (size_t)(e0 + e) * NFP + f0;
#pragma unroll
      for (int f = 0; f <= N; f++) az[f * fs] = y[f];
    }
  } else {
    // nablaQsp(9,9) (compflux.f90:107-157): (1/J) sum_r Mmat (A_z S) over both line
    // families, each component differentiated along its lines on the integer pipes, one
    // (cell, line, component) per thread, the xi lines first; then update_B
    // (magnetic_potential.f90:44-67): B = B0 + curl A_z
    double* sZ = sm;                  // [epb][NFP][2] A_z * (S_x, S_y)
    double* sP = sZ + epb * NFP * 2;  // [epb][NS][2]  the xi-line part of the gradient
    for (int i = threadIdx.x; i < cnt * NFP; i += blockDim.x) {
      const size_t g = (size_t)e0 * NFP + i;
      const double z = s.Azf[g];
      const double2 m = reinterpret_cast<const double2*>(s.met)[g];
      sZ[2 * i] = z * m.x;
      sZ[2 * i + 1] = z * m.y;
    }
    __syncthreads();
#pragma unroll 1
    for (int fam = 0; fam < 2; fam++) {
      for (int t = threadIdx.x; t < cnt * N * 2; t += blockDim.x) {
        const int c = t & 1, el = t >> 1, e = el / N, ln = el - e * N;
        const int fp0 = fam ? NF1 + ln : ln * (N + 1), fps = fam ? N : 1;
        double y[N];
        deriv_line<N, O>(sZ + (e * NFP + fp0) * 2 + c, fps * 2, y);
        const int p0 = e * NS + (fam ? ln : ln * N), ps = fam ? N : 1;
        if (!fam) {
#pragma unroll
          for (int i = 0; i < N; i++) sP[(p0 + i * ps) * 2 + c] = y[i];
        } else {
#pragma unroll
          for (int i = 0; i < N; i++) {
            const size_t gs = (size_t)e0 * NS + p0 + i * ps;
            const double a = (sP[(p0 + i * ps) * 2 + c] + y[i]) * s.invJ[gs];
            s.nQs9[gs * 2 + c] = a;
            if (c) s.Q[gs * 9 + 5] = a + s.B0x;  // Bx = dA/dy
            else s.Q[gs * 9 + 6] = s.B0y - a;    // By = -dA/dx
          }
        }
      }
      __syncthreads();
    }
  }
}

template <int N>
__global__ void __launch_bounds__(256) k_ct_elem(SolveDev s, int epb, int mode, int c0, int c1) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  const int e0 = c0 + blockIdx.x * epb;
  const int cnt = min(epb, c1 - e0);
  if (cnt <= 0) return;
  ct_elem_body<N, OpsTU>(s, e0, cnt, epb, mode, sm);
}

template <int N>
__device__ __forceinline__ void ctface_point(const SolveDev& s, int t) {
  constexpr int NFP = D<N>::NFP;
  if (t >= s.nface2 * N) return;
  const int f = t / N, nfp = t - f * N;
  const int4 fc = s.face2[f];
  const size_t gl = (size_t)fc.x * NFP + face_fp<N>(fc.y, nfp);
  const size_t gr = (size_t)fc.z * NFP + face_fp<N>(fc.w, N - 1 - nfp);
  const double v = half(s.Azf[gl] + s.Azf[gr]);
  s.Azf[gl] = v;
  s.Azf[gr] = v;
}

// the points of two-sided faces [f0, f1)
template <int N>
__global__ void __launch_bounds__(256) k_ct_face(SolveDev s, int f0, int f1) {
  pdl_wait();
  const int t = f0 * N + blockIdx.x * blockDim.x + threadIdx.x;
  if (t < f1 * N) ctface_point<N>(s, t);
}

// The diagnostic of iterations.f90:35-36 (comp_inviscid_flux, then nablaQsp(6,7) for
// div B) reads only B_x and B_y at the flux points: interpolate those two variables of
// the CT-corrected state (mode 0, one (cell, line, variable) per thread, the mirror
// symmetry of the points as in E1) and average them across the two-sided faces (the face
// pass below), as interfaceflux/CYCLOCFLUX do (interfaceflux_all.f90:79-91); a FREE face
// keeps its interior trace (bcflux.f90).
template <int N, class O>
__device__ __forceinline__ void diag_interp_body(const SolveDev& s, int e0, int cnt, double* sm) {
  constexpr int NS = D<N>::NS, NF1 = D<N>::NF1, NFP = D<N>::NFP;
  double* sB = sm;  // [cnt][NS][2] B_x, B_y
  for (int i = threadIdx.x; i < cnt * NS * 2; i += blockDim.x)
    sB[i] = s.Q[((size_t)e0 * NS + (i >> 1)) * 9 + 5 + (i & 1)];
  __syncthreads();
  for (int t = threadIdx.x; t < cnt * 2 * N * 2; t += blockDim.x) {
    const int v = t & 1, el = t >> 1, e = el / (2 * N), line = el - e * 2 * N;
    const bool fam1 = line < N;
    const int ln = fam1 ? line : line - N;
    const double* qb = sB + (e * NS + (fam1 ? ln * N : ln)) * 2 + v;
    const int qs = fam1 ? 2 : 2 * N;
    const int f0 = fam1 ? ln * (N + 1) : NF1 + ln, fs = fam1 ? 1 : N;
    double* ob = s.Qvf + ((size_t)(e0 + e) * NFP + f0) * 9 + 5 + v;
    double w[N], y[N + 1];
#pragma unroll
    for (int sp = 0; sp < N; sp++) w[sp] = qb[sp * qs];
    interp_line<N, O>(w, y);
#pragma unroll
    for (int f = 0; f <= N; f++) ob[(size_t)f * fs * 9] = y[f];
  }
}

template <int N>
__global__ void __launch_bounds__(256) k_diag_interp(SolveDev s, int epb) {
  extern __shared__ __align__(16) double sm[];
  const int e0 = blockIdx.x * epb;
  const int cnt = min(epb, s.NC - e0);
  if (cnt <= 0) return;
  diag_interp_body<N, OpsTU>(s, e0, cnt, sm);
}

template <int N>
__global__ void __launch_bounds__(256) k_diag_face(SolveDev s) {
  constexpr int NFP = D<N>::NFP;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= s.nface2 * N) return;
  const int f = t / N, nfp = t - f * N;
  const int4 fc = s.face2[f];
  double* a = s.Qvf + ((size_t)fc.x * NFP + face_fp<N>(fc.y, nfp)) * 9 + 5;
  double* b = s.Qvf + ((size_t)fc.z * NFP + face_fp<N>(fc.w, N - 1 - nfp)) * 9 + 5;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const double v = half(a[k] + b[k]);
    a[k] = v;
    b[k] = v;
  }
}

// nablaQsp(v0..v1) (compflux.f90:107-157) from the current Qvf, 0-based variables, for
// cells [e0, e0+cnt): the conservative form of E2 (metric-state products differentiated
// along the lines on the integer pipes), 2 (v1-v0+1) line quantities per cell
template <int N, class O>
__device__ __forceinline__ void nqsp_cells(const SolveDev& s, int e0, int cnt, int v0, int v1, double* sm) {
  constexpr int NS = D<N>::NS, NF1 = D<N>::NF1, NFP = D<N>::NFP;
  const int nv = v1 - v0 + 1, NQ = 2 * nv;
  double* sP = sm;                  // [cnt][NFP][NQ] Q_k * S_x (k < nv), Q_k * S_y
  double* sG = sP + cnt * NFP * NQ;  // [cnt][NS][NQ] the xi-line part
  for (int i = threadIdx.x; i < cnt * NFP * nv; i += blockDim.x) {
    const int kk = i % nv, lf = i / nv;
    const size_t g = (size_t)e0 * NFP + lf;
    const double q = s.Qvf[g * 9 + v0 + kk];
    sP[lf * NQ + kk] = q * s.met[2 * g];
    sP[lf * NQ + nv + kk] = q * s.met[2 * g + 1];
  }
  __syncthreads();
#pragma unroll 1
  for (int fam = 0; fam < 2; fam++) {
    for (int t = threadIdx.x; t < cnt * N * NQ; t += blockDim.x) {
      const int c = t % NQ, el = t / NQ, le = el / N, ln = el - le * N;
      const int fp0 = fam ? NF1 + ln : ln * (N + 1), fps = fam ? N : 1;
      double y[N];
      deriv_line<N, O>(sP + (le * NFP + fp0) * NQ + c, fps * NQ, y);
      const int p0 = fam ? ln : ln * N, ps = fam ? N : 1;
      double* g = sG + (le * NS + p0) * NQ + c;
      if (!fam) {
#pragma unroll
        for (int i = 0; i < N; i++) g[i * ps * NQ] = y[i];
      } else {
        const int k = v0 + c % nv, d = c / nv;
#pragma unroll
        for (int i = 0; i < N; i++) {
          const size_t gs = (size_t)(e0 + le) * NS + p0 + i * ps;
          const double a = (g[i * ps * NQ] + y[i]) * s.invJ[gs];
          if (k < 8) s.nQs[gs * 18 + 9 * d + k] = a;
          else s.nQs9[gs * 2 + d] = a;  // variable 9 is kept in its own array
        }
      }
    }
    __syncthreads();
  }
}

template <int N>
__global__ void __launch_bounds__(256) k_nqsp(SolveDev s, int epb, int v0, int v1) {
  extern __shared__ __align__(16) double sm[];
  const int e0 = blockIdx.x * epb;
  const int cnt = min(epb, s.NC - e0);
  if (cnt <= 0) return;
  nqsp_cells<N, OpsTU>(s, e0, cnt, v0, v1, sm);
}

// per-cell sum of (dBx/dx + dBy/dy)^2 (iterations.f90:48) into diag[e][1]
template <int N>
__global__ void __launch_bounds__(256) k_divb(SolveDev s) {
  constexpr int NS = D<N>::NS;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= s.NC) return;
  double acc = 0.0;
  for (int p = 0; p < NS; p++) {
    const double* g = s.nQs + ((size_t)c * NS + p) * 18;
    const double d = g[5] + g[9 + 6];
    acc += d * d;
  }
  s.diag[2 * c + 1] = acc;
}

}  // namespace chorus
