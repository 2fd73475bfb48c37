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
// chain of FP64 fused multiply-adds, whose rounding errors are of that size too.  The
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

// aligned limbs of a line: X_j = h_j 2^29 + l_j = x_j 2^(1075 + G - emax), rounded to
// the nearest integer (ties away from zero in magnitude)
template <int NI>
FIX_HD void fix_align(const double (&v)[NI], int emax, int (&h)[NI], int (&l)[NI]) {
#pragma unroll
  for (int j = 0; j < NI; j++) {
    const uint64_t u = fix_bits(v[j]);
    const int e = (int)((u >> 52) & 0x7ff);
    int d = emax - (e ? e : 1);  // zeros and subnormals have exponent 1, no hidden bit
    d = d < 63 ? d : 63;         // inputs 2^-59 below the largest vanish
    const uint64_t m = ((u & 0xfffffffffffffull) | (e ? 0x10000000000000ull : 0ull)) << kFixG;
    int64_t x = (int64_t)((m + ((1ull << d) >> 1)) >> d);  // rounded to the nearest unit
    x = (u >> 63) ? -x : x;
    h[j] = (int)(x >> kFixSplit);
    l[j] = (int)(x & ((1 << kFixSplit) - 1));
  }
}

// sum of ch, cl against the aligned limbs, rounded into a double scaled by 2^k
// (k = emax - 1017 - G - S: the sum is V 2^58 in units of 2^(emax - 1075 - G - S))
template <int NI>
FIX_HD double fix_dot(const int (&h)[NI], const int (&l)[NI], const int* ch, const int* cl, int k) {
  int64_t A = 0, B = 0, D = 0;  // |A| < 2^61.2, |B| < 2^62.5, 0 <= D < 2^61.2 for NI <= 9
#pragma unroll
  for (int j = 0; j < NI; j++) {
    A += (int64_t)h[j] * ch[j];
    B += (int64_t)h[j] * cl[j];
    B += (int64_t)l[j] * ch[j];
    D += (int64_t)l[j] * cl[j];
  }
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

// split c = ch 2^29 + cl with 0 <= cl < 2^29
inline void fix_split_coef(double C, int S, int* ch, int* cl) {
  double t = C;
  for (int i = 0; i < S; i++) t *= 2.0;  // exact scaling by 2^S
  const double r = t < 0 ? -__builtin_floor(-t + 0.5) : __builtin_floor(t + 0.5);
  const int64_t c = (int64_t)r;
  *ch = (int)(c >> kFixSplit);
  *cl = (int)(c & ((1 << kFixSplit) - 1));
}

}  // namespace chorus
