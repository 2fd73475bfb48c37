// fixdot.cuh -- the fixed line operators (Lmat interpolation, Mmat differentiation)
// applied in integer arithmetic.
//
// GB300 executes FP64 at 2 operations per clock per SM, while its integer pipes take
// 64 lane-operations per clock each and sit nearly idle in these FP64-bound passes.  A
// line operator y_k = sum_j C_kj x_j with fixed coefficients is therefore cheaper as an
// integer dot product:
//   * the inputs of one line are aligned to the largest exponent among them and held as
//     57-bit signed integers X_j = x_j * 2^(1075 + G - emax) (G = 4 guard bits below the
//     53-bit significand of the largest input; smaller inputs lose only bits below
//     2^-58 of the largest, by rounding),
//   * the coefficients as 59-bit signed integers c = round(C * 2^S), S per operator,
//   * both split at bit 29 (X = h 2^29 + l, c = ch 2^29 + cl, 0 <= l, cl < 2^29), so the
//     product sum is four 32x32->64 multiply-adds per term, exact in three 64-bit
//     accumulators:  sum c X = 2^58 sum h ch + 2^29 sum (h cl + l ch) + sum l cl,
//   * the sum, truncated to a multiple of 2^58 (at most 2^-55 of the largest term), is
//     rounded once, to nearest-even, into a double.
// The error stays below one unit in the last place of the line's largest term, as with a
// chain of FP64 fused multiply-adds, whose rounding errors are of that size too.
//
// The stage kernels apply the operators in mirror form (fix_apply_mirror): the solution
// and flux points are symmetric about the cell centre, so the operators satisfy
// C(NO-1-k, NI-1-j) = sigma C(k, j) (sigma = +1 for the interpolation Lmat, -1 for the
// derivative Mmat) up to the rounding of their construction (1e-16 to 2e-15 of the
// largest coefficient for N = 2..8).  With E_j = X_j + X_{NI-1-j} and O_j = X_j - X_{NI-1-j}
// (exact integers) each pair of mirror outputs k, NO-1-k shares one sum over the NI/2
// input pairs, U + W and sigma (U - W), so a line takes half the multiply-adds.  The
// coefficients are those of the operator averaged with its mirror image, each within one
// unit of 2^-S of both rows, and the error bound above holds for that operator.  The
// caller keeps the FP64 form for lines with NaN, infinite or huge (above 2^876) inputs,
// so non-finite states propagate as before.  Zero results are +0; results below the
// normal range (only from inputs below 2^-960) are flushed to zero.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define FIX_HD __host__ __device__ __forceinline__
#else
#define FIX_HD inline
#endif

namespace chorus {

constexpr int kFixG = 4;       // guard bits of the aligned inputs
constexpr int kFixSplit = 29;  // limb split of inputs and coefficients
constexpr int kFixEmaxFast = 1900;  // largest biased input exponent of the integer form

FIX_HD uint64_t fix_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  __builtin_memcpy(&u, &x, 8);
  return u;
#endif
}

FIX_HD double fix_double(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  __builtin_memcpy(&x, &u, 8);
  return x;
#endif
}

FIX_HD int fix_clz64(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)u);
#else
  return u ? __builtin_clzll(u) : 64;
#endif
}

// biased exponent field of x
FIX_HD int fix_exp(double x) { return (int)((fix_bits(x) >> 52) & 0x7ff); }

// the largest biased exponent over a line of NI values (at least 1, the exponent of
// the subnormals)
template <int NI>
FIX_HD int fix_emax(const double (&v)[NI]) {
  int e = 1;
#pragma unroll
  for (int j = 0; j < NI; j++) {
    const int ej = fix_exp(v[j]);
    e = ej > e ? ej : e;
  }
  return e;
}

// aligned integers of a line: X_j = x_j 2^(1075 + G - emax), rounded to the nearest
// integer (ties away from zero in magnitude); |X_j| < 2^57
template <int NI>
FIX_HD void fix_align_x(const double (&v)[NI], int emax, int64_t (&X)[NI]) {
#pragma unroll
  for (int j = 0; j < NI; j++) {
    const uint64_t u = fix_bits(v[j]);
    const int e = (int)((u >> 52) & 0x7ff);
    int d = emax - (e ? e : 1);  // zeros and subnormals have exponent 1, no hidden bit
    d = d < 63 ? d : 63;         // inputs 2^-59 below the largest vanish
    const uint64_t m = ((u & 0xfffffffffffffull) | (e ? 0x10000000000000ull : 0ull)) << kFixG;
    const int64_t x = (int64_t)((m + ((1ull << d) >> 1)) >> d);  // rounded to the nearest unit
    X[j] = (u >> 63) ? -x : x;
  }
}

// limbs x = h 2^29 + l, 0 <= l < 2^29 (h keeps the sign)
FIX_HD void fix_split(int64_t x, int& h, int& l) {
  h = (int)(x >> kFixSplit);
  l = (int)(x & ((1 << kFixSplit) - 1));
}

// aligned limbs of a line: X_j = h_j 2^29 + l_j
template <int NI>
FIX_HD void fix_align(const double (&v)[NI], int emax, int (&h)[NI], int (&l)[NI]) {
  int64_t X[NI];
  fix_align_x(v, emax, X);
#pragma unroll
  for (int j = 0; j < NI; j++) fix_split(X[j], h[j], l[j]);
}

// one term of a dot product in limbs: 2^58 h ch + 2^29 (h cl + l ch) + l cl
FIX_HD void fix_mac(int h, int l, int ch, int cl, int64_t& A, int64_t& B, int64_t& D) {
  A += (int64_t)h * ch;
  B += (int64_t)h * cl;
  B += (int64_t)l * ch;
  D += (int64_t)l * cl;
}

// the sum A 2^58 + B 2^29 + D rounded into a double scaled by 2^k (k = emax - 1017 - G - S:
// the sum is V 2^58 in units of 2^(emax - 1075 - G - S)); the shifts are arithmetic, so D
// may be negative (a difference of two sums)
FIX_HD double fix_round(int64_t A, int64_t B, int64_t D, int k) {
  B += D >> kFixSplit;
  const int64_t V = A + (B >> kFixSplit);  // floor(sum c X / 2^58)
  const uint64_t sgn = (uint64_t)V & 0x8000000000000000ull;
  const uint64_t u = V < 0 ? (uint64_t)(-V) : (uint64_t)V;
  if (u == 0) return 0.0;
  const int lz = fix_clz64(u);
  const uint64_t top = u << lz;
  uint64_t mant = top >> 11;
  const uint64_t rem = top & 0x7ff;
  mant += (rem > 0x400 || (rem == 0x400 && (mant & 1))) ? 1 : 0;
  const int E = k + 1086 - lz;  // biased exponent of mant * 2^(11 - lz + k)
  if (E < 1) return fix_double(sgn);  // below the normal range: flushed to zero
  return fix_double(sgn | (((uint64_t)(E - 1) << 52) + mant));
}

// sum of ch, cl against the aligned limbs, rounded into a double scaled by 2^k
template <int NI>
FIX_HD double fix_dot(const int (&h)[NI], const int (&l)[NI], const int* ch, const int* cl, int k) {
  int64_t A = 0, B = 0, D = 0;  // |A| < 2^61.2, |B| < 2^62.5, 0 <= D < 2^61.2 for NI <= 9
#pragma unroll
  for (int j = 0; j < NI; j++) fix_mac(h[j], l[j], ch[j], cl[j], A, B, D);
  return fix_round(A, B, D, k);
}

// y = C v for C (NO x NI) in mirror form (fix_mirror_coefs: per row k < (NO+1)/2 the
// coefficients [P(0..NI/2) | Q(0..NI/2) | R]), scaled by 2^k as fix_dot.  With
// E_j = X_j + X_{NI-1-j}, O_j = X_j - X_{NI-1-j} (|E|, |O| < 2^58), U = sum P E (+ R X_m for
// odd NI) and W = sum Q O: y_k = U + W, y_{NO-1-k} = sigma (U - W).  The middle row of an
// odd NO has only U (sigma = +1) or only W (sigma = -1): the other half is exactly zero.
// Bounds for NI <= 9 (|P|, |Q|, |R| < 2^59, so |ch| < 2^30): |A| < 9 2^59 = 2^62.2,
// |B| < 9 1.5 2^59 = 2^62.8, |D| < 9 2^58 = 2^61.2, for sums and differences alike.
template <int NO, int NI, int SIGMA>
FIX_HD void fix_apply_mirror(const double (&v)[NI], int emax, const int* ch, const int* cl, int k, double (&y)[NO]) {
  constexpr int NP = NI / 2;
  int64_t X[NI];
  fix_align_x(v, emax, X);
  int eh[NP > 0 ? NP : 1], el[NP > 0 ? NP : 1], oh[NP > 0 ? NP : 1], ol[NP > 0 ? NP : 1];
#pragma unroll
  for (int j = 0; j < NP; j++) {
    fix_split(X[j] + X[NI - 1 - j], eh[j], el[j]);
    fix_split(X[j] - X[NI - 1 - j], oh[j], ol[j]);
  }
  int mh = 0, ml = 0;
  if (NI & 1) fix_split(X[NP], mh, ml);
#pragma unroll
  for (int r = 0; r < (NO + 1) / 2; r++) {
    const int* rh = ch + r * NI;
    const int* rl = cl + r * NI;
    const bool mid = (NO & 1) && r == NO / 2;
    int64_t Au = 0, Bu = 0, Du = 0, Aw = 0, Bw = 0, Dw = 0;
    if (!mid || SIGMA > 0) {
#pragma unroll
      for (int j = 0; j < NP; j++) fix_mac(eh[j], el[j], rh[j], rl[j], Au, Bu, Du);
      if (NI & 1) fix_mac(mh, ml, rh[2 * NP], rl[2 * NP], Au, Bu, Du);
    }
    if (!mid || SIGMA < 0) {
#pragma unroll
      for (int j = 0; j < NP; j++) fix_mac(oh[j], ol[j], rh[NP + j], rl[NP + j], Aw, Bw, Dw);
    }
    y[r] = fix_round(Au + Aw, Bu + Bw, Du + Dw, k);
    if (!mid)
      y[NO - 1 - r] = SIGMA > 0 ? fix_round(Au - Aw, Bu - Bw, Du - Dw, k) : fix_round(Aw - Au, Bw - Bu, Dw - Du, k);
  }
}

// integer form of coefficients (host side): c = round(C 2^S), S the largest shift that
// keeps every |c| below 2^59 (S = 59 - e for max |C| in [2^(e-1), 2^e))
inline int fix_shift_for(const double* C, int n) {
  double mx = 0.0;
  for (int i = 0; i < n; i++) mx = C[i] > mx ? C[i] : (-C[i] > mx ? -C[i] : mx);
  if (mx == 0.0) return 59;
  int e;
  __builtin_frexp(mx, &e);
  return 59 - e;
}

// round(C 2^S) (ties away from zero), exact: |C 2^S| < 2^59
inline int64_t fix_coef(double C, int S) {
  double t = C;
  for (int i = 0; i < S; i++) t *= 2.0;  // exact scaling by 2^S
  const double r = t < 0 ? -__builtin_floor(-t + 0.5) : __builtin_floor(t + 0.5);
  return (int64_t)r;
}

// split c = ch 2^29 + cl with 0 <= cl < 2^29
inline void fix_split_coef(double C, int S, int* ch, int* cl) {
  const int64_t c = fix_coef(C, S);
  *ch = (int)(c >> kFixSplit);
  *cl = (int)(c & ((1 << kFixSplit) - 1));
}

// the mirror form of C (NO x NI, row-major C[k NI + j], C(NO-1-k, NI-1-j) = sigma C(k, j)
// up to rounding) for fix_apply_mirror: for each row k < (NO+1)/2, k' = NO-1-k, and input
// pair j < NI/2, j' = NI-1-j, from the integers c = round(C 2^S),
//   P(k,j) = (c(k,j) + c(k,j') + sigma c(k',j') + sigma c(k',j)) / 4
//   Q(k,j) = (c(k,j) - c(k,j') + sigma c(k',j') - sigma c(k',j)) / 4
//   R(k)   = (c(k,m) + sigma c(k',m)) / 2          (middle input m of an odd NI)
// each an exact 64-bit sum rounded once (half up), stored in limbs per row as
// [P(0..NI/2) | Q(0..NI/2) | R].  P + Q and P - Q, the coefficients of inputs j and j' in
// row k, lie within one unit of the average of row k and the mirror image of row k'.
inline void fix_mirror_coefs(const double* C, int NO, int NI, int sigma, int S, int* ch, int* cl) {
  const int NP = NI / 2;
  for (int k = 0; k < (NO + 1) / 2; k++) {
    const int kk = NO - 1 - k;
    auto c = [&](int row, int j) { return fix_coef(C[row * NI + j], S); };
    for (int j = 0; j < NP; j++) {
      const int jj = NI - 1 - j;
      const int64_t p = (c(k, j) + c(k, jj) + sigma * (c(kk, jj) + c(kk, j)) + 2) >> 2;
      const int64_t q = (c(k, j) - c(k, jj) + sigma * (c(kk, jj) - c(kk, j)) + 2) >> 2;
      ch[k * NI + j] = (int)(p >> kFixSplit);
      cl[k * NI + j] = (int)(p & ((1 << kFixSplit) - 1));
      ch[k * NI + NP + j] = (int)(q >> kFixSplit);
      cl[k * NI + NP + j] = (int)(q & ((1 << kFixSplit) - 1));
    }
    if (NI & 1) {
      const int64_t r = (c(k, NP) + sigma * c(kk, NP) + 1) >> 1;
      ch[k * NI + 2 * NP] = (int)(r >> kFixSplit);
      cl[k * NI + 2 * NP] = (int)(r & ((1 << kFixSplit) - 1));
    }
  }
}

}  // namespace chorus
