// Host driver of the integer line operators (chorus-mhd_gb300/csrc/fixdot.cuh), the same
// code the stage kernels run: reads  int NO, NI, nlines; double C[NO][NI];
// double x[nlines][NI]  from argv[1] and writes  double y[nlines][NO]  to argv[2].
// Lines whose inputs are outside the integer form are written as NaN.
#include <cmath>
#include <cstdio>
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

int main(int argc, char** argv) {
  if (argc != 3) return 2;
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
  FILE* g = std::fopen(argv[2], "wb");
  if (!g) return 2;
  std::fwrite(y.data(), sizeof(double), y.size(), g);
  std::fclose(g);
  return 0;
}
