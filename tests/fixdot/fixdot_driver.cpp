// Host driver of the integer line operators (chorus-mhd_gb300/csrc/fixdot.cuh), the same
// code the stage kernels run: reads  int NO, NI, nlines; double C[NO][NI];
// double x[nlines][NI]  from argv[1] and writes  double y[nlines][NO]  to argv[2].
// Lines whose inputs are outside the integer form are written as NaN.
// With argv[3] = sigma (+1 or -1) and argv[4], the operator is applied in mirror form
// (fix_mirror_coefs / fix_apply_mirror, as the stage kernels do), and argv[4] receives
// int S and the effective integer operator  int64 c[NO][NI]  (y = 2^-S c x before rounding).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fixdot.cuh"

using namespace chorus;

template <int NI>
static void run(int NO, const std::vector<double>& C, const std::vector<double>& x, int nlines, std::vector<double>& y) {
  const int S = fix_shift_for(C.data(), NO * NI);
  std::vector<int> ch(NO * NI), cl(NO * NI);
  for (int i = 0; i < NO * NI; i++) fix_split_coef(C[i], S, &ch[i], &cl[i]);
  for (int n = 0; n < nlines; n++) {
    double v[NI];
    for (int j = 0; j < NI; j++) v[j] = x[(size_t)n * NI + j];
    const int emax = fix_emax(v);
    if (emax > kFixEmaxFast) {
      for (int k = 0; k < NO; k++) y[(size_t)n * NO + k] = NAN;
      continue;
    }
    int h[NI], l[NI];
    fix_align(v, emax, h, l);
    for (int k = 0; k < NO; k++)
      y[(size_t)n * NO + k] = fix_dot(h, l, &ch[k * NI], &cl[k * NI], emax - 1017 - kFixG - S);
  }
}

template <int NO, int NI, int SIGMA>
static void run_mirror(const std::vector<double>& C, const std::vector<double>& x, int nlines, std::vector<double>& y,
                       const char* opfile) {
  const int S = fix_shift_for(C.data(), NO * NI);
  std::vector<int> ch(NO * NI, 0), cl(NO * NI, 0);
  fix_mirror_coefs(C.data(), NO, NI, SIGMA, S, ch.data(), cl.data());
  // the effective operator: row k < (NO+1)/2 from P, Q, R; row NO-1-k its mirror image
  constexpr int NP = NI / 2;
  std::vector<int64_t> ce(NO * NI, 0);
  auto coef = [&](int k, int c) { return (int64_t)ch[k * NI + c] * ((int64_t)1 << kFixSplit) + cl[k * NI + c]; };
  for (int k = 0; k < (NO + 1) / 2; k++) {
    const int kk = NO - 1 - k;
    for (int j = 0; j < NP; j++) {
      const int64_t p = coef(k, j), q = coef(k, NP + j);
      ce[k * NI + j] = p + q;
      ce[k * NI + NI - 1 - j] = p - q;
      if (kk != k) {
        ce[kk * NI + j] = SIGMA * (p - q);
        ce[kk * NI + NI - 1 - j] = SIGMA * (p + q);
      }
    }
    if (NI & 1) {
      ce[k * NI + NP] = coef(k, 2 * NP);
      if (kk != k) ce[kk * NI + NP] = SIGMA * coef(k, 2 * NP);
    }
  }
  FILE* g = std::fopen(opfile, "wb");
  if (g) {
    std::fwrite(&S, sizeof(int), 1, g);
    std::fwrite(ce.data(), sizeof(int64_t), ce.size(), g);
    std::fclose(g);
  }
  for (int n = 0; n < nlines; n++) {
    double v[NI], out[NO];
    for (int j = 0; j < NI; j++) v[j] = x[(size_t)n * NI + j];
    const int emax = fix_emax(v);
    if (emax > kFixEmaxFast) {
      for (int k = 0; k < NO; k++) y[(size_t)n * NO + k] = NAN;
      continue;
    }
    fix_apply_mirror<NO, NI, SIGMA>(v, emax, ch.data(), cl.data(), emax - 1017 - kFixG - S, out);
    for (int k = 0; k < NO; k++) y[(size_t)n * NO + k] = out[k];
  }
}

// the shapes of the solver's operators: Lmat (N+1) x N with sigma = +1, Mmat N x (N+1) with
// sigma = -1, N = 2..8
template <int N>
static bool mirror_n(int NO, int NI, int sigma, const std::vector<double>& C, const std::vector<double>& x, int nlines,
                     std::vector<double>& y, const char* opfile) {
  if (sigma > 0 && NO == N + 1 && NI == N) return run_mirror<N + 1, N, 1>(C, x, nlines, y, opfile), true;
  if (sigma < 0 && NO == N && NI == N + 1) return run_mirror<N, N + 1, -1>(C, x, nlines, y, opfile), true;
  return false;
}

int main(int argc, char** argv) {
  if (argc != 3 && argc != 5) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int hdr[3];
  if (std::fread(hdr, sizeof(int), 3, f) != 3) return 2;
  const int NO = hdr[0], NI = hdr[1], nlines = hdr[2];
  if (NO < 1 || NO > 9 || NI < 2 || NI > 9 || nlines < 0) return 2;
  std::vector<double> C((size_t)NO * NI), x((size_t)nlines * NI), y((size_t)nlines * NO);
  if (std::fread(C.data(), sizeof(double), C.size(), f) != C.size()) return 2;
  if (std::fread(x.data(), sizeof(double), x.size(), f) != x.size()) return 2;
  std::fclose(f);
  if (argc == 5) {
    const int sigma = std::atoi(argv[3]);
    const bool ok = mirror_n<2>(NO, NI, sigma, C, x, nlines, y, argv[4]) ||
                    mirror_n<3>(NO, NI, sigma, C, x, nlines, y, argv[4]) ||
                    mirror_n<4>(NO, NI, sigma, C, x, nlines, y, argv[4]) ||
                    mirror_n<5>(NO, NI, sigma, C, x, nlines, y, argv[4]) ||
                    mirror_n<6>(NO, NI, sigma, C, x, nlines, y, argv[4]) ||
                    mirror_n<7>(NO, NI, sigma, C, x, nlines, y, argv[4]) ||
                    mirror_n<8>(NO, NI, sigma, C, x, nlines, y, argv[4]);
    if (!ok) return 2;
  } else {
    switch (NI) {
      case 2: run<2>(NO, C, x, nlines, y); break;
      case 3: run<3>(NO, C, x, nlines, y); break;
      case 4: run<4>(NO, C, x, nlines, y); break;
      case 5: run<5>(NO, C, x, nlines, y); break;
      case 6: run<6>(NO, C, x, nlines, y); break;
      case 7: run<7>(NO, C, x, nlines, y); break;
      case 8: run<8>(NO, C, x, nlines, y); break;
      default: run<9>(NO, C, x, nlines, y); break;
    }
  }
  FILE* g = std::fopen(argv[2], "wb");
  if (!g) return 2;
  std::fwrite(y.data(), sizeof(double), y.size(), g);
  std::fclose(g);
  return 0;
}
