// plot.cu -- the plot output of iterations.f90:80-84 for one partition:
//   tecplotter2dsetup (tecplotter2dsetup.f90:1-177): plot nodes, their multiplicity
//     and the plot cells, built on the host once per solve;
//   tecplotter2d (tecplotter.f90:1-86): the conservative state interpolated to the
//     nodes of every cell, summed over the cells that share a node, averaged and
//     converted to primitive variables, on the device;
//   tecpost_parallel (tecplotter.f90:92-418): the Tecplot binary file.
// smooth_procint_plot (smooth_procint_plot.f90) only adds contributions across
// processor interfaces, of which one partition has none.
//
// The node kernel gathers each node's contributions through a node -> (cell, ii, jj)
// list kept in the reference's loop order (cells ascending, then jj, then ii) and does
// its arithmetic with explicitly rounded operations (no contraction), so the node
// values are those of the reference's loops bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "chorus_gpu.h"
#include "chorus_internal.h"
#include "physics.cuh"

namespace chorus {
int set_err(int code, const char* fmt, ...);
const SolveDev& ctx_solve(const ChorusCtx* c);
int ctx_device_of(const ChorusCtx* c);
bool ctx_plot_ready(const ChorusCtx* c);
}  // namespace chorus

using namespace chorus;

struct ChorusPlot {
  ChorusCtx* ctx = nullptr;
  int N = 0, NC = 0, Np = 0;
  int nodes = 0, cells = 0;
  double gam = 0.0;
  bool warned = false;             // the reference's 'something wrong' checks fired
  std::vector<double> plotX;       // (2, nodes)
  std::vector<int32_t> connec;     // (4, cells), 1-based
  std::vector<int32_t> gnumnode;   // (Np+1, Np+1, NCELL), 1-based
  std::vector<int32_t> factor;     // (nodes)
  // device
  int* d_row = nullptr;            // [nodes+1] into d_con
  int2* d_con = nullptr;           // (cell, ii | jj << 16), 0-based
  int* d_factor = nullptr;
  double* d_H = nullptr;           // [Np+1][N] Lagrange basis at the plot abscissae
  double* d_mu = nullptr;          // [NC][2] muAV(1), muAV(6)
  double* d_val = nullptr;         // [11][nodes] rho u v w p Bx By Bz Az muAV etaAV
  float* d_f32 = nullptr;          // [11][nodes]
  unsigned long long* d_mm = nullptr;  // [11] min keys, [11] max keys
};

namespace {

// xyCoor_atGps (mapder.f90:255-273) with the bilinear MapBaseFunc (:79-87)
void xy_coor(const double xs[2][4], double xi, double eta, double xx[2]) {
  const double f[4] = {(1.0 - xi) * (1.0 - eta), (1.0 - eta) * xi, xi * eta, (1.0 - xi) * eta};
  for (int i = 0; i < 2; i++) {
    xx[i] = 0.0;
    for (int nb = 0; nb < 4; nb++) xx[i] = xx[i] + xs[i][nb] * f[nb];
  }
}

// tecplotter2dsetup.f90:1-177 (CURVE_WALL = 0): vertices first (node id = vertex id),
// then per cell the edge nodes, matched by distance (<= 1e-5) against the nodes the
// neighbour across the face already created, then the interior nodes, then the
// Np x Np plot cells
void plot_topology(ChorusPlot& P, const int32_t* IVCELL, const int32_t* IC2F, const double* XV, const double* YV,
                   int NVERT, int NFACE) {
  const int Np = P.Np, NC = P.NC;
  const size_t nn = (size_t)(Np + 1) * (Np + 1) * NC;
  P.gnumnode.assign(nn, 0);
  std::vector<int32_t> factor(nn, 0);
  std::vector<double> X(2 * nn, 0.0);
  P.connec.assign(4 * (size_t)Np * Np * NC, 0);
  const int ne = std::max(Np - 1, 1);
  std::vector<int> isfacenod(NFACE, 0), gfacenode((size_t)ne * NFACE, 0);
  auto gnum = [&](int ii, int jj, int ic) -> int32_t& {
    return P.gnumnode[(ii - 1) + (size_t)(Np + 1) * ((jj - 1) + (size_t)(Np + 1) * ic)];
  };
  int nodes = 0, cells = 0;
  bool bad = false;
  for (int ic = 0; ic < NC; ic++) {
    int v[4];
    for (int k = 0; k < 4; k++) v[k] = IVCELL[ic + (size_t)NC * k];
    gnum(1, 1, ic) = v[0];
    gnum(Np + 1, 1, ic) = v[1];
    gnum(Np + 1, Np + 1, ic) = v[2];
    gnum(1, Np + 1, ic) = v[3];
    for (int k = 0; k < 4; k++) {
      const int g = v[k];
      if (factor[g - 1] == 0) {
        nodes++;
        X[2 * (g - 1)] = XV[g - 1];
        X[2 * (g - 1) + 1] = YV[g - 1];
      }
      factor[g - 1]++;
    }
  }
  if (nodes != NVERT) bad = true;
  for (int ic = 0; ic < NC; ic++) {
    double xs[2][4];
    for (int j = 0; j < 4; j++) {
      xs[0][j] = XV[IVCELL[ic + (size_t)NC * j] - 1];
      xs[1][j] = YV[IVCELL[ic + (size_t)NC * j] - 1];
    }
    for (int k = 1; k <= 4; k++) {
      const int iface = IC2F[ic + (size_t)NC * (k - 1)];
      for (int en = 1; en <= Np - 1; en++) {
        int ii, jj;
        switch (k) {
          case 1: ii = en + 1; jj = 1; break;
          case 2: ii = Np + 1; jj = en + 1; break;
          case 3: ii = Np + 1 - en; jj = Np + 1; break;
          default: ii = 1; jj = Np + 1 - en; break;
        }
        double rx[2];
        xy_coor(xs, (double)(ii - 1) / (double)Np, (double)(jj - 1) / (double)Np, rx);
        if (isfacenod[iface - 1] == 1) {
          bool match = false;
          for (int ex = 1; ex <= Np - 1; ex++) {  // every match counts, as in :88-97
            const int g = gfacenode[(ex - 1) + (size_t)ne * (iface - 1)];
            const double dx = rx[0] - X[2 * (g - 1)], dy = rx[1] - X[2 * (g - 1) + 1];
            if (std::fabs(std::sqrt(dx * dx + dy * dy)) <= 1e-5) {
              gnum(ii, jj, ic) = g;
              factor[g - 1]++;
              match = true;
            }
          }
          if (!match) bad = true;
        } else {
          nodes++;
          X[2 * (nodes - 1)] = rx[0];
          X[2 * (nodes - 1) + 1] = rx[1];
          gnum(ii, jj, ic) = nodes;
          gfacenode[(en - 1) + (size_t)ne * (iface - 1)] = nodes;
          factor[nodes - 1]++;
        }
      }
      if (isfacenod[iface - 1] == 0) isfacenod[iface - 1] = 1;
    }
    for (int ii = 2; ii <= Np; ii++)
      for (int jj = 2; jj <= Np; jj++) {
        double rx[2];
        xy_coor(xs, (double)(ii - 1) / (double)Np, (double)(jj - 1) / (double)Np, rx);
        nodes++;
        X[2 * (nodes - 1)] = rx[0];
        X[2 * (nodes - 1) + 1] = rx[1];
        gnum(ii, jj, ic) = nodes;
        factor[nodes - 1]++;
      }
    for (int ii = 1; ii <= Np; ii++)
      for (int jj = 1; jj <= Np; jj++) {
        int32_t* c = &P.connec[4 * (size_t)cells++];
        c[0] = gnum(ii, jj, ic);
        c[1] = gnum(ii + 1, jj, ic);
        c[2] = gnum(ii + 1, jj + 1, ic);
        c[3] = gnum(ii, jj + 1, ic);
      }
  }
  P.nodes = nodes;
  P.cells = cells;
  P.warned = bad;
  P.plotX.assign(X.begin(), X.begin() + 2 * (size_t)nodes);
  P.factor.assign(factor.begin(), factor.begin() + nodes);
}

// hval (tecplotter.f90:62-82)
double hval(const double* Xs, int np, int i, double xval) {
  double hn = 1.0, hd = 1.0;
  for (int s = 1; s <= np; s++)
    if (s != i) {
      hn = hn * (xval - Xs[s - 1]);
      hd = hd * (Xs[i - 1] - Xs[s - 1]);
    }
  return hn / hd;
}

__device__ __forceinline__ unsigned long long order_key(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
double key_value(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
}

// muAV(1) and muAV(6) of every cell (AV.f90:157-172) from the last stage's sensor sums
// and that stage's epsilon0 (:147-148)
__global__ void k_plot_cells(int NC, int N, int artiv, const unsigned long long* eig, double hmsh, const double* Se,
                             const double* Se6, double* mu) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= NC) return;
  const double eps0 = __longlong_as_double((long long)*eig) * hmsh / (double)(N - 1) * 1.0;
  mu[2 * c] = artiv ? av_mu(Se[c], eps0) : 0.0;
  mu[2 * c + 1] = artiv ? av_mu(Se6[c], eps0) : 0.0;
}

// tecplotter2d (tecplotter.f90:19-59) per plot node, in the reference's order
__global__ void __launch_bounds__(256) k_plot_nodes(int nodes, int N, double gm1, const int* row, const int2* con,
                                                    const double* H, const double* Q, const double* mu,
                                                    const int* factor, double* val, float* f32,
                                                    unsigned long long* mm) {
  const int nd = blockIdx.x * blockDim.x + threadIdx.x;
  double out[11];
  bool live = nd < nodes;
  if (live) {
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, a0 = 0.0, a1 = 0.0;
    const int NS = N * N;
    for (int r = row[nd]; r < row[nd + 1]; r++) {
      const int2 cc = con[r];
      const int ii = cc.y & 0xFFFF, jj = cc.y >> 16;
      const double* q = Q + (size_t)cc.x * NS * 9;
      double Qs[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int js = 0; js < N; js++)
        for (int is = 0; is < N; is++) {
          const double hx = H[ii * N + is], hy = H[jj * N + js];
          const double* qp = q + (js * N + is) * 9;
#pragma unroll
          for (int k = 0; k < 9; k++) Qs[k] = __dadd_rn(Qs[k], __dmul_rn(__dmul_rn(qp[k], hx), hy));
        }
#pragma unroll
      for (int k = 0; k < 9; k++) acc[k] = __dadd_rn(acc[k], Qs[k]);
      a0 = __dadd_rn(a0, mu[2 * cc.x]);
      a1 = __dadd_rn(a1, mu[2 * cc.x + 1]);
    }
    const double f = (double)factor[nd];
    double Qs[9];
#pragma unroll
    for (int k = 0; k < 9; k++) Qs[k] = __ddiv_rn(acc[k], f);
    out[0] = Qs[0];
    out[1] = __ddiv_rn(Qs[1], Qs[0]);
    out[2] = __ddiv_rn(Qs[2], Qs[0]);
    out[3] = __ddiv_rn(Qs[3], Qs[0]);
    for (int k = 5; k < 9; k++) out[k] = Qs[k];
    const double nu = __dadd_rn(__dadd_rn(__dmul_rn(out[1], out[1]), __dmul_rn(out[2], out[2])), __dmul_rn(out[3], out[3]));
    const double nb = __dadd_rn(__dadd_rn(__dmul_rn(out[5], out[5]), __dmul_rn(out[6], out[6])), __dmul_rn(out[7], out[7]));
    out[4] = __dmul_rn(__dsub_rn(__dsub_rn(Qs[4], __dmul_rn(__dmul_rn(0.5, Qs[0]), nu)), __dmul_rn(0.5, nb)), gm1);
    out[9] = __ddiv_rn(a0, f);
    out[10] = __ddiv_rn(a1, f);
#pragma unroll
    for (int v = 0; v < 11; v++) {
      val[(size_t)v * nodes + nd] = out[v];
      f32[(size_t)v * nodes + nd] = __double2float_rn(out[v]);
    }
  }
  // minval / maxval of every variable (exact: an order-independent reduction)
  __shared__ unsigned long long smin[11][8], smax[11][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < 11; v++) {
    unsigned long long lo = live ? order_key(out[v]) : ~0ull, hi = live ? order_key(out[v]) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, o), b = __shfl_xor_sync(0xffffffffu, hi, o);
      lo = a < lo ? a : lo;
      hi = b > hi ? b : hi;
    }
    if (lane == 0) {
      smin[v][w] = lo;
      smax[v][w] = hi;
    }
  }
  __syncthreads();
  if (threadIdx.x < 11) {
    const int v = threadIdx.x, nw = blockDim.x >> 5;
    unsigned long long lo = ~0ull, hi = 0ull;
    for (int i = 0; i < nw; i++) {
      lo = smin[v][i] < lo ? smin[v][i] : lo;
      hi = smax[v][i] > hi ? smax[v][i] : hi;
    }
    atomicMin(&mm[v], lo);
    atomicMax(&mm[11 + v], hi);
  }
}

void plot_release(ChorusPlot* P) {
  cudaFree(P->d_row);
  cudaFree(P->d_con);
  cudaFree(P->d_factor);
  cudaFree(P->d_H);
  cudaFree(P->d_mu);
  cudaFree(P->d_val);
  cudaFree(P->d_f32);
  cudaFree(P->d_mm);
}

#define PCK(x)                                                                                  \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) return set_err(CHORUS_ECUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
  } while (0)

int plot_upload(ChorusPlot* P, const double* Xs) {
  const int Np = P->Np, N = P->N, NC = P->NC;
  // node -> contributions in the loop order of tecplotter.f90:21-42
  std::vector<int> row(P->nodes + 1, 0);
  for (int32_t g : P->gnumnode) row[g]++;
  for (int i = 0; i < P->nodes; i++) row[i + 1] += row[i];
  if ((long long)row[P->nodes] != (long long)P->gnumnode.size())
    return set_err(CHORUS_EMESH, "plot node numbering is inconsistent");
  std::vector<int> fill(row.begin(), row.end() - 1);
  std::vector<int2> con(P->gnumnode.size());
  for (int ic = 0; ic < NC; ic++)
    for (int jj = 0; jj <= Np; jj++)
      for (int ii = 0; ii <= Np; ii++) {
        const int g = P->gnumnode[ii + (size_t)(Np + 1) * (jj + (size_t)(Np + 1) * ic)];
        con[fill[g - 1]++] = make_int2(ic, ii | (jj << 16));
      }
  std::vector<double> H((size_t)(Np + 1) * N);
  for (int ii = 0; ii <= Np; ii++)
    for (int is = 0; is < N; is++) H[(size_t)ii * N + is] = hval(Xs, N, is + 1, (double)ii / (double)Np);
  PCK(cudaMalloc(&P->d_row, sizeof(int) * row.size()));
  PCK(cudaMalloc(&P->d_con, sizeof(int2) * std::max<size_t>(con.size(), 1)));
  PCK(cudaMalloc(&P->d_factor, sizeof(int) * std::max(P->nodes, 1)));
  PCK(cudaMalloc(&P->d_H, sizeof(double) * H.size()));
  PCK(cudaMalloc(&P->d_mu, sizeof(double) * 2 * std::max(NC, 1)));
  PCK(cudaMalloc(&P->d_val, sizeof(double) * 11 * std::max(P->nodes, 1)));
  PCK(cudaMalloc(&P->d_f32, sizeof(float) * 11 * std::max(P->nodes, 1)));
  PCK(cudaMalloc(&P->d_mm, sizeof(unsigned long long) * 22));
  PCK(cudaMemcpy(P->d_row, row.data(), sizeof(int) * row.size(), cudaMemcpyHostToDevice));
  PCK(cudaMemcpy(P->d_con, con.data(), sizeof(int2) * con.size(), cudaMemcpyHostToDevice));
  PCK(cudaMemcpy(P->d_factor, P->factor.data(), sizeof(int) * P->nodes, cudaMemcpyHostToDevice));
  PCK(cudaMemcpy(P->d_H, H.data(), sizeof(double) * H.size(), cudaMemcpyHostToDevice));
  return CHORUS_OK;
}

// run the node kernels on the solve's stream and wait for them
int plot_eval(ChorusPlot* P) {
  const SolveDev& s = ctx_solve(P->ctx);
  if (!ctx_plot_ready(P->ctx))
    return set_err(CHORUS_ESTATE,
                   "etaAV needs the variable-6 sensor of the last stage: set the plot_sensor option before the "
                   "step (or compresid) that precedes the plot");
  PCK(cudaSetDevice(ctx_device_of(P->ctx)));
  cudaStream_t st = (cudaStream_t)chorus_gpu_stream(P->ctx);
  PCK(cudaMemsetAsync(P->d_mm, 0xFF, sizeof(unsigned long long) * 11, st));
  PCK(cudaMemsetAsync(P->d_mm + 11, 0, sizeof(unsigned long long) * 11, st));
  k_plot_cells<<<(P->NC + 255) / 256, 256, 0, st>>>(P->NC, P->N, s.artiv, s.eig, s.hmsh, s.Se, s.Se6, P->d_mu);
  if (P->nodes > 0)
    k_plot_nodes<<<(P->nodes + 255) / 256, 256, 0, st>>>(P->nodes, P->N, P->gam - 1.0, P->d_row, P->d_con, P->d_H,
                                                         s.Q, P->d_mu, P->d_factor, P->d_val, P->d_f32, P->d_mm);
  PCK(cudaGetLastError());
  PCK(cudaStreamSynchronize(st));
  return CHORUS_OK;
}

void put_i32(FILE* f, int32_t v) { std::fwrite(&v, 4, 1, f); }
void put_str(FILE* f, const char* s) {  // write_tecplot_string, tecplotter.f90:399-416
  for (; *s; s++) put_i32(f, (unsigned char)*s);
  put_i32(f, 0);
}

}  // namespace

extern "C" {

int chorus_plot_create(ChorusCtx* ctx, const int32_t* IVCELL, const int32_t* IC2F, const double* XV,
                       const double* YV, int32_t NVERT, int32_t NFACE, const double* Xs, int32_t NRE,
                       ChorusPlot** out) {
  if (!ctx || !IVCELL || !IC2F || !XV || !YV || !Xs || !out) return set_err(CHORUS_EINVAL, "null argument");
  *out = nullptr;
  const SolveDev& s = ctx_solve(ctx);
  if (NRE < 1 || NRE > 0x7FFF) return set_err(CHORUS_EINVAL, "NRE = %d out of range", NRE);
  if ((double)(NRE + 1) * (NRE + 1) * s.NC > 2.0e9) return set_err(CHORUS_EINVAL, "plot too large");
  for (size_t i = 0; i < 4 * (size_t)s.NC; i++)
    if (IVCELL[i] < 1 || IVCELL[i] > NVERT || IC2F[i] < 1 || IC2F[i] > NFACE)
      return set_err(CHORUS_EMESH, "IVCELL / IC2F entry %zu out of range", i);
  ChorusPlot* P = new ChorusPlot();
  P->ctx = ctx;
  P->N = s.N;
  P->NC = s.NC;
  P->Np = NRE;
  P->gam = s.gam;
  plot_topology(*P, IVCELL, IC2F, XV, YV, NVERT, NFACE);
  int rc = cudaSetDevice(ctx_device_of(ctx)) == cudaSuccess ? plot_upload(P, Xs)
                                                              : set_err(CHORUS_ECUDA, "cudaSetDevice failed");
  if (rc) {
    plot_release(P);
    delete P;
    return rc;
  }
  *out = P;
  return CHORUS_OK;
}

int chorus_plot_free(ChorusPlot* P) {
  if (!P) return CHORUS_OK;
  cudaSetDevice(ctx_device_of(P->ctx));
  plot_release(P);
  delete P;
  return CHORUS_OK;
}

int chorus_plot_info(const ChorusPlot* P, int64_t* nodes, int64_t* cells, int32_t* warned) {
  if (!P) return set_err(CHORUS_EINVAL, "null plot");
  if (nodes) *nodes = P->nodes;
  if (cells) *cells = P->cells;
  if (warned) *warned = P->warned ? 1 : 0;
  return CHORUS_OK;
}

int chorus_plot_values(ChorusPlot* P, double* plotX, double* plotQ, double* plotAV, int32_t* connec,
                       int32_t* gnode_factor) {
  if (!P) return set_err(CHORUS_EINVAL, "null plot");
  int rc = plot_eval(P);
  if (rc) return rc;
  const size_t n = (size_t)P->nodes;
  if (plotX) std::memcpy(plotX, P->plotX.data(), sizeof(double) * 2 * n);
  if (connec) std::memcpy(connec, P->connec.data(), sizeof(int32_t) * 4 * (size_t)P->cells);
  if (gnode_factor) std::memcpy(gnode_factor, P->factor.data(), sizeof(int32_t) * n);
  if (plotQ || plotAV) {
    std::vector<double> v(11 * n);
    PCK(cudaMemcpy(v.data(), P->d_val, sizeof(double) * v.size(), cudaMemcpyDeviceToHost));
    for (size_t nd = 0; nd < n; nd++) {
      if (plotQ)
        for (int k = 0; k < 9; k++) plotQ[9 * nd + k] = v[(size_t)k * n + nd];
      if (plotAV)
        for (int k = 0; k < 2; k++) plotAV[2 * nd + k] = v[(size_t)(9 + k) * n + nd];
    }
  }
  return CHORUS_OK;
}

int chorus_plot_filename(double ctime, char* buf, int32_t n) {
  if (!buf || n < 20) return set_err(CHORUS_EINVAL, "buffer too small");
  char dec[64];
  std::snprintf(dec, sizeof dec, "%6.3f", ctime - (double)(int)ctime);
  std::snprintf(buf, (size_t)n, "TEC%07d%.4s.plt", (int)ctime, dec + 2);
  return CHORUS_OK;
}

int chorus_plot_write(ChorusPlot* P, double ctime, const char* dir, char* path_out, int32_t path_len) {
  if (!P || !dir) return set_err(CHORUS_EINVAL, "null argument");
  int rc = plot_eval(P);
  if (rc) return rc;
  const size_t n = (size_t)P->nodes;
  const int nvar = 13;
  std::vector<float> f((size_t)11 * n);
  unsigned long long mm[22];
  PCK(cudaMemcpy(f.data(), P->d_f32, sizeof(float) * f.size(), cudaMemcpyDeviceToHost));
  PCK(cudaMemcpy(mm, P->d_mm, sizeof mm, cudaMemcpyDeviceToHost));
  double minmax[2 * 13];
  for (int v = 0; v < 2; v++) {
    double lo = 0.0, hi = 0.0;
    for (size_t nd = 0; nd < n; nd++) {
      const double x = P->plotX[2 * nd + v];
      if (nd == 0 || x < lo) lo = x;
      if (nd == 0 || x > hi) hi = x;
    }
    minmax[2 * v] = lo;
    minmax[2 * v + 1] = hi;
  }
  for (int v = 0; v < 11; v++) {
    minmax[2 * (v + 2)] = n ? key_value(mm[v]) : 0.0;
    minmax[2 * (v + 2) + 1] = n ? key_value(mm[11 + v]) : 0.0;
  }
  char name[64];
  chorus_plot_filename(ctime, name, sizeof name);
  std::string path = std::string(dir) + "/" + name;
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) return set_err(CHORUS_EIO, "cannot open %s", path.c_str());
  // header, tecplotter.f90:186-303
  std::fwrite("#!TDV111", 1, 8, fp);
  put_i32(fp, 1);
  put_i32(fp, 0);
  put_str(fp, "step data");
  put_i32(fp, nvar);
  const char* names[13] = {"X", "Y", "RHO", "U", "V", "W", "P", "Bx", "By", "Bz", "Az", "muAV", "etaAV"};
  for (auto nm : names) put_str(fp, nm);
  const float zone = 299.0f, eoh = 357.0f;
  std::fwrite(&zone, 4, 1, fp);
  put_str(fp, "ZONE 001");
  put_i32(fp, -1);
  put_i32(fp, 0);
  std::fwrite(&ctime, 8, 1, fp);
  const int32_t zh[12] = {-1, 3, 0, 0, 0, 0, P->nodes, P->cells, 0, 0, 0, 0};
  std::fwrite(zh, 4, 12, fp);
  std::fwrite(&eoh, 4, 1, fp);
  std::fwrite(&zone, 4, 1, fp);
  for (int v = 0; v < nvar; v++) put_i32(fp, 1);
  put_i32(fp, 0);
  put_i32(fp, 0);
  put_i32(fp, -1);
  std::fwrite(minmax, 8, 2 * nvar, fp);
  // data, block packed, :305-388
  std::vector<float> xy(n);
  for (int v = 0; v < 2; v++) {
    for (size_t nd = 0; nd < n; nd++) xy[nd] = (float)P->plotX[2 * nd + v];
    std::fwrite(xy.data(), 4, n, fp);
  }
  std::fwrite(f.data(), 4, f.size(), fp);
  // connectivity, 0-based, :390-395
  std::vector<int32_t> c0(P->connec.size());
  for (size_t i = 0; i < c0.size(); i++) c0[i] = P->connec[i] - 1;
  std::fwrite(c0.data(), 4, c0.size(), fp);
  const bool bad = std::ferror(fp) != 0;
  std::fclose(fp);
  if (bad) return set_err(CHORUS_EIO, "write failed: %s", path.c_str());
  if (path_out && path_len > 0) std::snprintf(path_out, (size_t)path_len, "%s", path.c_str());
  return CHORUS_OK;
}

}  // extern "C"
