// capi.cu -- the C-ABI of libchorus_gpu.so: context binding, resident state, the
// drop-in entry points for the reference routines, CUDA-graph step replay, parity
// downloads and the host-side setup entry points.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "chorus_internal.h"
#include "kernels.cuh"

namespace chorus {

// upload functions defined in kernels_n*.cu (each TU owns its constant operators)
void upload_ops_n2(const OpsN&);
void upload_ops_n3(const OpsN&);
void upload_ops_n4(const OpsN&);
void upload_ops_n5(const OpsN&);
void upload_ops_n6(const OpsN&);
void upload_ops_n7(const OpsN&);
void upload_ops_n8(const OpsN&);
void launch_e1_nosensor_n2(const SolveDev&, const Launch&, cudaStream_t);
void launch_e1_nosensor_n3(const SolveDev&, const Launch&, cudaStream_t);
void launch_e1_nosensor_n4(const SolveDev&, const Launch&, cudaStream_t);
void launch_e1_nosensor_n5(const SolveDev&, const Launch&, cudaStream_t);
void launch_e1_nosensor_n6(const SolveDev&, const Launch&, cudaStream_t);
void launch_e1_nosensor_n7(const SolveDev&, const Launch&, cudaStream_t);
void launch_e1_nosensor_n8(const SolveDev&, const Launch&, cudaStream_t);

static thread_local std::string g_err;

int set_err(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                               \
  do {                                                                                         \
    cudaError_t _e = (call);                                                                   \
    if (_e != cudaSuccess)                                                                     \
      return set_err(CHORUS_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__); \
  } while (0)

// ---------------------------------------------------------------------------
// operators in constant memory, once per (device, N)
// ---------------------------------------------------------------------------
static std::mutex g_ops_mu;
static bool g_ops_done[64][kMaxN + 1];

static void make_ops(int N, const double* Lmat, const double* Mmat, const double* Xs, const double* Xf, OpsN& o) {
  std::memset(&o, 0, sizeof o);
  for (int i = 0; i < (N + 1) * N; i++) { o.L[i] = Lmat[i]; o.M[i] = Mmat[i]; }
  for (int i = 0; i <= N; i++) o.Xf[i] = Xf[i];
  for (int i = 0; i < N; i++) o.Xs[i] = Xs[i];
  for (int f = 0; f <= N / 2; f++) {
    for (int j = 0; j < N / 2; j++) {
      const double a = Lmat[f + (N + 1) * j], b = Lmat[f + (N + 1) * (N - 1 - j)];
      o.CE[f * kHalfS + j] = 0.5 * (a + b);
      o.CO[f * kHalfS + j] = 0.5 * (a - b);
    }
    o.LMID[f] = (N & 1) ? Lmat[f + (N + 1) * ((N - 1) / 2)] : 0.0;
  }
  // the integer line operators in mirror form: Lmat as the row-major (N+1) x N operator
  // L(f, j), Mmat (column-major (N+1, N)) is already the row-major N x (N+1) operator
  // M(r, i) indexed [i][r]
  double Lrow[(kMaxN + 1) * kMaxN];
  for (int f = 0; f <= N; f++)
    for (int j = 0; j < N; j++) Lrow[f * N + j] = Lmat[f + (N + 1) * j];
  o.LS = fix_shift_for(Lmat, (N + 1) * N);
  fix_mirror_coefs(Lrow, N + 1, N, 1, o.LS, o.LH, o.LL);
  o.MS = fix_shift_for(Mmat, (N + 1) * N);
  fix_mirror_coefs(Mmat, N, N + 1, -1, o.MS, o.MH, o.ML);
  // AV smoothing A = Hlow * H: project N points onto the N-1 low-order points
  // (hhval at Xs_low, AV.f90:19-35) and evaluate back (hhval_low at Xs, :41-58)
  double xsl[kMaxN], xfl[kMaxN + 1];
  setsandpoints(N - 1, xsl, xfl);
  for (int i = 0; i < N; i++)
    for (int m = 0; m < N; m++) {
      double a = 0.0;
      for (int l = 0; l < N - 1; l++) a += lagrange(xsl, N - 1, l, Xs[i]) * lagrange(Xs, N, m, xsl[l]);
      o.A[i * N + m] = a;
    }
}

static int ensure_ops(int dev, int N, const double* Lmat, const double* Mmat, const double* Xs, const double* Xf) {
  std::lock_guard<std::mutex> lk(g_ops_mu);
  if (dev >= 0 && dev < 64 && g_ops_done[dev][N]) return CHORUS_OK;
  OpsN o;
  make_ops(N, Lmat, Mmat, Xs, Xf, o);
  switch (N) {
    case 2: upload_ops_n2(o); break;
    case 3: upload_ops_n3(o); break;
    case 4: upload_ops_n4(o); break;
    case 5: upload_ops_n5(o); break;
    case 6: upload_ops_n6(o); break;
    case 7: upload_ops_n7(o); break;
    case 8: upload_ops_n8(o); break;
    default: return set_err(CHORUS_EINVAL, "N=%d not supported", N);
  }
  CK(cudaGetLastError());
  if (dev >= 0 && dev < 64) g_ops_done[dev][N] = true;
  return CHORUS_OK;
}

// ---------------------------------------------------------------------------
// per-N dispatch of the stage launches
// ---------------------------------------------------------------------------
struct Dispatch {
  void (*e1)(const SolveDev&, const Launch&, cudaStream_t, int, int, int);
  void (*e1ns)(const SolveDev&, const Launch&, cudaStream_t);
  void (*f1)(const SolveDev&, cudaStream_t, int, int, int, int);
  void (*e2)(const SolveDev&, const Launch&, cudaStream_t);
  void (*f2)(const SolveDev&, cudaStream_t);
  void (*e3)(const SolveDev&, const RKStage&, const Launch&, cudaStream_t, int, int);
  void (*ct)(const SolveDev&, const Launch&, cudaStream_t, int, int, int);
  void (*nqsp)(const SolveDev&, int, int, cudaStream_t);
  void (*divb)(const SolveDev&, cudaStream_t);
  void (*diag)(const SolveDev&, const Launch&, cudaStream_t, int);
};
#define DISPATCH(n) \
  Dispatch{launch_e1<n>, launch_e1_nosensor_n##n, launch_f1<n>, launch_e2<n>, launch_f2<n>, launch_e3<n>, launch_ct<n>, launch_nqsp<n>, launch_divb<n>, \
           launch_diag<n>}
static const Dispatch* dispatch_for(int N) {
  static const Dispatch d[kMaxN + 1] = {Dispatch{}, Dispatch{}, DISPATCH(2), DISPATCH(3), DISPATCH(4),
                                        DISPATCH(5), DISPATCH(6), DISPATCH(7), DISPATCH(8)};
  return (N >= kMinN && N <= kMaxN) ? &d[N] : nullptr;
}

// default launch shapes per N (cells per CTA, threads per CTA)
Launch default_launch(int N, int which) {
  // which: 0 = E1, 1 = E2, 2 = E3, 3 = CT; cells per CTA and threads per CTA as the
  // autotuner picked them on GB300 for N = 3..6 (for N = 6 the shapes of an earlier tuning,
  // which the batched form runs faster); the CT passes take about 128/(2N) cells
  // so that their (cell, line) loop fills the 128 threads
  static const int epb[kMaxN + 1][4] = {{0}, {0}, {16, 16, 16, 32}, {16, 4, 2, 21}, {4, 4, 4, 16},
                                        {4, 2, 5, 12}, {3, 2, 2, 10}, {2, 2, 2, 9}, {2, 2, 2, 8}};
  static const int thr[kMaxN + 1][4] = {{0}, {0}, {128, 128, 128, 128}, {224, 128, 32, 128}, {128, 128, 96, 128},
                                        {128, 128, 160, 128}, {96, 192, 128, 128}, {128, 128, 128, 128},
                                        {128, 128, 128, 128}};
  return Launch{epb[N][which], thr[N][which]};
}

}  // namespace chorus

using namespace chorus;

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
constexpr int kMaxHostChunks = 32;  // chunks of a host-state upload / download

constexpr int kMaxHostSegs = 2 * kMaxHostChunks + 2;

// The chunks of a host-state step: cells [cut[k], cut[k+1]) (smaller towards both ends);
// two-sided faces [f2[k], f2[k+1])
// (those whose larger cell is in chunk k) and FREE faces [f1[k], f1[k+1]) (cell in chunk
// k).  The download goes by segments of cells [sb[i], se[i]) whose cells and face
// neighbours all lie in chunks 0..sk[i]: the maximal runs of cells that complete with the
// same chunk (with a structured numbering about one per chunk, shifted by a row), or the
// chunks themselves when the runs are more than kMaxHostSegs.
struct HostChunks {
  int K = 0;
  int cut[kMaxHostChunks + 1];
  int f2[kMaxHostChunks + 1];
  int f1[kMaxHostChunks + 1];
  int nseg = 0;
  int sb[kMaxHostSegs], se[kMaxHostSegs], sk[kMaxHostSegs];
};

// A host-state step captured as a CUDA graph for one pair of pinned host buffers (its
// copies address them) and one kind of step (with or without the diagnostic), so that a
// step is one launch however busy the host thread is
struct HostGraph {
  const double* qin = nullptr;
  double* qout = nullptr;
  int diag = 0;
  cudaGraphExec_t ex = nullptr;
};
constexpr int kHostGraphs = 4;
constexpr int kEvJoin = kMaxHostChunks + kMaxHostSegs + 1;  // the copy stream's join event

struct ChorusCtx {
  int device = 0;
  ChorusDims dims{};
  ChorusParams p{};
  int nface2 = 0, nface1 = 0;
  cudaStream_t st = nullptr;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  SolveDev sd{};
  double* red = nullptr;       // [4]: diag sums, eig as double
  double* h_pinned = nullptr;  // pinned staging for diag records
  Launch L[4];
  cudaGraphExec_t g_step = nullptr, g_diag = nullptr;
  double graph_dt = NAN;
  int graph_k = -1;
  const Dispatch* D = nullptr;
  int skip_option = 1;  // skip viscous work where it is exactly zero (mu = eta0 = 0, no AV)
  int diagnostics = 1;  // norms every tenth step in iterations_gpu
  int plot_sensor = 0;  // the last stage records the variable-6 sensor (plot etaAV)
  int se6_valid = 0;    // ... and did so in the latest residual evaluation
  // the CT projection leaves the A_z traces in Azf only: Qvf variable 9 (the reference's
  // Qvfi(9)/Qvfj(9)) is filled from Azf when it is next read, unless an E1 pass (which
  // rewrites every Qvf variable) comes first
  bool qvf9_pending = false;
  std::vector<double> Lmat, Mmat, Xs, Xf;
  // host-state steps: a copy stream and events that chain chunked copies to kernels
  cudaStream_t cp = nullptr;
  cudaEvent_t ev[kMaxHostChunks + kMaxHostSegs + 2] = {};
  int host_chunks = 16;  // option "host_chunks"
  // the larger cell of each two-sided face and the cell of each FREE face, in list order
  // (ascending), and per cell the largest index among itself and its face neighbours
  std::vector<int> f2max, f1cell, cellrel;
  HostChunks hc;  // built on first use for host_chunks (hc.K == 0: not built)
  HostGraph hg[kHostGraphs];
  int hg_next = 0;
};

static void drop_host_graphs(ChorusCtx* c) {
  for (HostGraph& g : c->hg) {
    if (g.ex) cudaGraphExecDestroy(g.ex);
    g = HostGraph{};
  }
}

namespace chorus {
void upload_ops_all(int N, const OpsN& o);
const SolveDev& ctx_solve(const ChorusCtx* c) { return c->sd; }
int ctx_device_of(const ChorusCtx* c) { return c->device; }
double ctx_dt(const ChorusCtx* c) { return c->p.dt; }
int ctx_kstage(const ChorusCtx* c) { return c->p.k_stage; }
int ctx_epb(const ChorusCtx* c, int pass) { return c->L[pass].epb; }
int ctx_threads(const ChorusCtx* c, int pass) { return c->L[pass].threads; }
bool ctx_plot_ready(const ChorusCtx* c) { return c->se6_valid != 0 || !c->sd.artiv; }
void ctx_mark_ct(ChorusCtx* c) { c->qvf9_pending = true; }
static bool g_ops_all_done[64][kMaxN + 1];
void ensure_ops_all(int dev, int N, const ChorusCtx* c) {
  std::lock_guard<std::mutex> lk(g_ops_mu);
  if (dev >= 0 && dev < 64 && g_ops_all_done[dev][N]) return;
  OpsN o;
  make_ops(N, c->Lmat.data(), c->Mmat.data(), c->Xs.data(), c->Xf.data(), o);
  upload_ops_all(N, o);
  if (dev >= 0 && dev < 64) g_ops_all_done[dev][N] = true;
}
}  // namespace chorus

static int ctx_device(ChorusCtx* c) {
  CK(cudaSetDevice(c->device));
  return CHORUS_OK;
}

struct ArenaPlan {
  size_t off = 0;
  template <typename T>
  size_t take(size_t count) {
    size_t o = off;
    off += ((count * sizeof(T) + 255) / 256) * 256;
    return o;
  }
};

// bytes of one solve's device arena (the same allocation sequence as chorus_gpu_bind)
static size_t arena_plan_bytes(int N, int NC, int nface2, int nface1, int k_stage) {
  const int NS = N * N, NFP = 2 * (N + 1) * N;
  const size_t nq = (size_t)NC * NS * 9, nfp = (size_t)NC * NFP;
  ArenaPlan P;
  P.take<double>(nq); P.take<double>(nq); P.take<double>(nq);
  if (k_stage == 5) { P.take<double>(nq); P.take<double>(nq); P.take<double>(nq); }
  P.take<double>(nq); P.take<double>(nfp * 9); P.take<double>(nfp * 8); P.take<double>(nfp);
  P.take<double>((size_t)NC * NS * 18); P.take<double>(nfp * 18); P.take<double>((size_t)NC * NS * 2);
  P.take<double>(nfp * 2); P.take<double>((size_t)NC * NS);
  P.take<double>((size_t)NC * 2); P.take<double>((size_t)NC * 4); P.take<double>((size_t)NC * 2);
  P.take<int4>(nface2 + 1); P.take<int2>(nface1 + 1); P.take<FaceNorm>((size_t)nface2 * N + 1);
  P.take<FaceNorm>((size_t)nface1 * N + 1); P.take<unsigned long long>(4); P.take<unsigned int>(4);
  P.take<double>(8); P.take<int>(NC); P.take<int>(NC); P.take<int4>(NC); P.take<int4>(NC);
  P.take<double>((size_t)NC * NS * 2);
  return P.off;
}

extern "C" {

const char* chorus_gpu_last_error(void) { return g_err.c_str(); }
const char* chorus_gpu_version(void) { return "chorus-gb300 0.1 (sm_103a, FP64)"; }

int chorus_gpu_device_name(int32_t device, char* buf, int32_t n) {
  if (!buf || n <= 0) return set_err(CHORUS_EINVAL, "null buffer");
  cudaDeviceProp p;
  CK(cudaGetDeviceProperties(&p, device));
  std::snprintf(buf, (size_t)n, "%s", p.name);
  return CHORUS_OK;
}

int chorus_gpu_bind(const ChorusDims* dims, const int32_t* IF2C, const int32_t* IBFINTER, const int32_t* IBFREE,
                    const int32_t* CYC2FPAIR, const int32_t* iface2fp, const int32_t* jface2fp, const double* Xs,
                    const double* Xf, const double* Lmat, const double* Mmat, const double* S1, const double* S2,
                    const double* Jac, const ChorusParams* params, int32_t device, ChorusCtx** out) {
  if (!dims || !params || !out || !Xs || !Xf || !Lmat || !Mmat || !S1 || !S2 || !Jac || !IF2C)
    return set_err(CHORUS_EINVAL, "chorus_gpu_bind: null argument");
  *out = nullptr;
  const int N = dims->N, NC = dims->NCELL, NF = dims->NFACE;
  if (N < kMinN || N > kMaxN) return set_err(CHORUS_EINVAL, "N=%d outside %d..%d", N, kMinN, kMaxN);
  if (NC <= 0 || NF <= 0 || dims->NINTER < 0 || dims->NFREE < 0 || dims->NPAIR < 0)
    return set_err(CHORUS_EINVAL, "bad dims (NCELL=%d NFACE=%d)", NC, NF);
  if ((dims->NINTER && !IBFINTER) || (dims->NFREE && !IBFREE) || (dims->NPAIR && !CYC2FPAIR))
    return set_err(CHORUS_EINVAL, "face list pointer is null");
  if (params->vismode != 1)
    return set_err(CHORUS_EINVAL, "vismode must be 1 (Qvfi/Azfi are written only when vismode==1)");
  if (params->k_stage != 3 && params->k_stage != 5)
    return set_err(CHORUS_EINVAL, "k_stage can be only 3 or 5");
  if ((int64_t)NC * 2 * (N + 1) * N * 18 > ((int64_t)1 << 40))
    return set_err(CHORUS_EINVAL, "mesh too large");
  // face2fpconnec must be the reference's (initsetup.f90:343-379); the kernels
  // hard-code it
  if (iface2fp && jface2fp)
    for (int nfp = 1; nfp <= N; nfp++) {
      const int ei[4] = {nfp, N + 1, N - nfp + 1, 1}, ej[4] = {1, nfp, N + 1, N - nfp + 1};
      for (int f = 0; f < 4; f++)
        if (iface2fp[nfp - 1 + N * f] != ei[f] || jface2fp[nfp - 1 + N * f] != ej[f])
          return set_err(CHORUS_EINVAL, "iface2fp/jface2fp differ from face2fpconnec");
    }
  ChorusCtx* c = new ChorusCtx();
  c->device = device;
  c->dims = *dims;
  c->p = *params;
  c->Lmat.assign(Lmat, Lmat + (N + 1) * N);
  c->Mmat.assign(Mmat, Mmat + (N + 1) * N);
  c->Xs.assign(Xs, Xs + N);
  c->Xf.assign(Xf, Xf + N + 1);
  c->D = dispatch_for(N);
  for (int w = 0; w < 4; w++) c->L[w] = default_launch(N, w);
  auto fail = [&](int code) {
    if (c->arena) cudaFree(c->arena);
    if (c->st) cudaStreamDestroy(c->st);
    if (c->cp) cudaStreamDestroy(c->cp);
    for (auto& ev : c->ev)
      if (ev) cudaEventDestroy(ev);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    delete c;
    return code;
  };
  if (cudaSetDevice(device) != cudaSuccess) return fail(set_err(CHORUS_ECUDA, "cudaSetDevice(%d) failed", device));

  // ---- faces: interior + periodic pairs are two-sided, FREE faces one-sided
  const int NI = dims->NINTER, NP = dims->NPAIR, NB = dims->NFREE;
  std::vector<int4> f2;
  std::vector<int2> f1;
  f2.reserve(NI + NP);
  auto cell_ok = [&](int ic) { return ic >= 1 && ic <= NC; };
  auto lf_ok = [&](int l) { return l >= 1 && l <= 4; };
  for (int i = 0; i < NI; i++) {
    const int f = IBFINTER[i] - 1;
    if (f < 0 || f >= NF) return fail(set_err(CHORUS_EMESH, "IBFINTER(%d)=%d out of range", i + 1, f + 1));
    const int cl = IF2C[f], cr = IF2C[f + NF], ll = IF2C[f + 2 * NF], lr = IF2C[f + 3 * NF];
    if (!cell_ok(cl) || !cell_ok(cr) || !lf_ok(ll) || !lf_ok(lr))
      return fail(set_err(CHORUS_EMESH, "IF2C row %d inconsistent", f + 1));
    f2.push_back(make_int4(cl - 1, ll, cr - 1, lr));
  }
  for (int i = 0; i < NP; i++) {
    const int k1 = CYC2FPAIR[i] - 1, k2 = CYC2FPAIR[i + NP] - 1;
    if (k1 < 0 || k1 >= NF || k2 < 0 || k2 >= NF) return fail(set_err(CHORUS_EMESH, "CYC2FPAIR(%d) out of range", i + 1));
    const int cl = IF2C[k1], cr = IF2C[k2], ll = IF2C[k1 + 2 * NF], lr = IF2C[k2 + 2 * NF];
    if (!cell_ok(cl) || !cell_ok(cr) || !lf_ok(ll) || !lf_ok(lr))
      return fail(set_err(CHORUS_EMESH, "periodic pair %d inconsistent", i + 1));
    f2.push_back(make_int4(cl - 1, ll, cr - 1, lr));
  }
  for (int i = 0; i < NB; i++) {
    const int f = IBFREE[i] - 1;
    if (f < 0 || f >= NF) return fail(set_err(CHORUS_EMESH, "IBFREE(%d) out of range", i + 1));
    const int cl = IF2C[f], ll = IF2C[f + 2 * NF];
    if (!cell_ok(cl) || !lf_ok(ll)) return fail(set_err(CHORUS_EMESH, "IF2C row %d inconsistent", f + 1));
    f1.push_back(make_int2(cl - 1, ll));
  }
  // two-sided faces in the order of their larger cell, FREE faces in cell order, so that
  // the faces whose cells all lie below a cell bound are a prefix of each list (a
  // host-state step runs the face passes chunk by chunk behind its copies); every face
  // pass writes per-cell slots and the wave speed is a maximum, so no result depends on
  // the order
  std::stable_sort(f2.begin(), f2.end(),
                   [](const int4& a, const int4& b) { return std::max(a.x, a.z) < std::max(b.x, b.z); });
  std::stable_sort(f1.begin(), f1.end(), [](const int2& a, const int2& b) { return a.x < b.x; });
  c->nface2 = (int)f2.size();
  c->nface1 = (int)f1.size();
  c->f2max.resize(f2.size());
  for (size_t i = 0; i < f2.size(); i++) c->f2max[i] = std::max(f2[i].x, f2[i].z);
  c->f1cell.resize(f1.size());
  for (size_t i = 0; i < f1.size(); i++) c->f1cell[i] = f1[i].x;
  c->hc.K = 0;
  // face neighbours per cell (local face 1..4 -> cell across it, -1 at FREE faces)
  std::vector<int4> nbr(NC, make_int4(-1, -1, -1, -1)), nbrlf(NC, make_int4(0, 0, 0, 0));
  auto setn = [&](int cell, int lf, int other, int olf) {
    reinterpret_cast<int*>(&nbr[cell])[lf - 1] = other;
    reinterpret_cast<int*>(&nbrlf[cell])[lf - 1] = olf;
  };
  for (const int4& f : f2) {
    setn(f.x, f.y, f.z, f.w);
    setn(f.z, f.w, f.x, f.y);
  }
  c->cellrel.resize(NC);
  for (int ic = 0; ic < NC; ic++) {
    const int4 b = nbr[ic];
    c->cellrel[ic] = std::max(std::max(ic, b.x), std::max(b.y, std::max(b.z, b.w)));
  }

  // ---- derived geometry
  const int NS = N * N, NF1 = (N + 1) * N, NFP = 2 * NF1;
  auto S1at = [&](int a, int b, int ifp, int jfp, int ic) {
    return S1[a + 2 * (b + 2 * (ifp + (N + 1) * (jfp + (size_t)N * ic)))];
  };
  auto S2at = [&](int a, int b, int ifp, int jfp, int ic) {
    return S2[a + 2 * (b + 2 * (ifp + N * (jfp + (size_t)(N + 1) * ic)))];
  };
  auto Jat = [&](int is, int js, int ic) { return Jac[is + N * (js + (size_t)N * ic)]; };
  std::vector<double> met((size_t)NC * NFP * 2), invJ((size_t)NC * NS);
  for (int ic = 0; ic < NC; ic++) {
    for (int jfp = 0; jfp < N; jfp++)
      for (int ifp = 0; ifp <= N; ifp++) {
        size_t g = ((size_t)ic * NFP + jfp * (N + 1) + ifp) * 2;
        met[g] = S1at(0, 0, ifp, jfp, ic);
        met[g + 1] = S1at(0, 1, ifp, jfp, ic);
      }
    for (int jfp = 0; jfp <= N; jfp++)
      for (int ifp = 0; ifp < N; ifp++) {
        size_t g = ((size_t)ic * NFP + NF1 + jfp * N + ifp) * 2;
        met[g] = S2at(1, 0, ifp, jfp, ic);
        met[g + 1] = S2at(1, 1, ifp, jfp, ic);
      }
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        const double J = Jat(is, js, ic);
        if (!(J > 0.0)) {
          int code = set_err(CHORUS_EMESH, "Jacobian %g <= 0 in cell %d", J, ic + 1);
          return fail(code);
        }
        invJ[(size_t)ic * NS + js * N + is] = 1.0 / J;
      }
  }
  // face normals from the left cell, getrusanov.f90:12-17 and interfaceflux_all.f90:46-76
  auto normal = [&](int cl, int lf, int nfp, double& n1, double& n2) {
    int ifp, jfp;
    switch (lf) {
      case 1: ifp = nfp; jfp = 0; n1 = S2at(1, 0, ifp, jfp, cl); n2 = S2at(1, 1, ifp, jfp, cl); break;
      case 2: ifp = N; jfp = nfp; n1 = S1at(0, 0, ifp, jfp, cl); n2 = S1at(0, 1, ifp, jfp, cl); break;
      case 3: ifp = N - 1 - nfp; jfp = N; n1 = S2at(1, 0, ifp, jfp, cl); n2 = S2at(1, 1, ifp, jfp, cl); break;
      default: ifp = 0; jfp = N - 1 - nfp; n1 = S1at(0, 0, ifp, jfp, cl); n2 = S1at(0, 1, ifp, jfp, cl); break;
    }
  };
  std::vector<FaceNorm> fn2((size_t)c->nface2 * N), fn1((size_t)c->nface1 * N);
  auto fill = [&](int cl, int ll, int lr, int nfp, FaceNorm& o) {
    double n1, n2;
    normal(cl, ll, nfp, n1, n2);
    const int sign_l = (ll == 1 || ll == 4) ? -1 : 1;
    const int sign_r = (lr == 2 || lr == 3) ? -1 : 1;
    const double mag = std::sqrt(n1 * n1 + n2 * n2);
    o.ux = n1 / mag * sign_l;
    o.uy = n2 / mag * sign_l;
    o.msl = 0.5 * (mag * sign_l);  // the 1/2 of the Rusanov average folded in
    o.ss = (double)(sign_l * sign_r);
  };
  for (int f = 0; f < c->nface2; f++)
    for (int nfp = 0; nfp < N; nfp++) fill(f2[f].x, f2[f].y, f2[f].w, nfp, fn2[(size_t)f * N + nfp]);
  for (int f = 0; f < c->nface1; f++)
    for (int nfp = 0; nfp < N; nfp++) fill(f1[f].x, f1[f].y, 1, nfp, fn1[(size_t)f * N + nfp]);

  // ---- device arena (arena_plan_bytes below must follow the same sequence)
  const size_t nq = (size_t)NC * NS * 9, nfp = (size_t)NC * NFP;
  ArenaPlan P;
  size_t oQ = P.take<double>(nq), oQk0 = P.take<double>(nq), oQka = P.take<double>(nq);
  const bool five = params->k_stage == 5;
  size_t oQr2 = five ? P.take<double>(nq) : 0, oQr3 = five ? P.take<double>(nq) : 0, oR0 = five ? P.take<double>(nq) : 0;
  size_t oRes = P.take<double>(nq), oQvf = P.take<double>(nfp * 9), oFc = P.take<double>(nfp * 8),
         oAzf = P.take<double>(nfp), onQs = P.take<double>((size_t)NC * NS * 18), onQvf = P.take<double>(nfp * 18),
         onAs = P.take<double>((size_t)NC * NS * 2), omet = P.take<double>(nfp * 2),
         oinvJ = P.take<double>((size_t)NC * NS),
         oSe = P.take<double>((size_t)NC * 2), omuf = P.take<double>((size_t)NC * 4), odiag = P.take<double>((size_t)NC * 2),
         of2 = P.take<int4>(f2.size() + 1), of1 = P.take<int2>(f1.size() + 1),
         ofn2 = P.take<FaceNorm>(fn2.size() + 1), ofn1 = P.take<FaceNorm>(fn1.size() + 1),
         oeig = P.take<unsigned long long>(4), oerr = P.take<unsigned int>(4), ored = P.take<double>(8),
         oact = P.take<int>(NC), onv = P.take<int>(NC), onbr = P.take<int4>(NC), onbrlf = P.take<int4>(NC),
         onQs9 = P.take<double>((size_t)NC * NS * 2);
  c->arena_bytes = P.off;
  if (P.off != arena_plan_bytes(N, NC, c->nface2, c->nface1, params->k_stage))
    return fail(set_err(CHORUS_EINVAL, "internal: arena plan mismatch"));
  cudaError_t e = cudaMalloc(&c->arena, P.off);
  if (e != cudaSuccess)
    return fail(set_err(CHORUS_ENOMEM, "cudaMalloc(%zu bytes) failed: %s", P.off, cudaGetErrorString(e)));
  char* A = (char*)c->arena;
  SolveDev& s = c->sd;
  s.N = N;
  s.NC = NC;
  s.nface2 = c->nface2;
  s.nface1 = c->nface1;
  s.artiv = params->ARTIV == 1;
  s.gam = params->gam;
  s.mu = params->mu;
  s.eta0 = params->eta0;
  s.B0x = params->B0x;
  s.B0y = params->B0y;
  s.hmsh = std::sqrt(params->DXCYCL * params->DYCYCL / (double)params->NCELLGLOB);
  s.Q = (double*)(A + oQ);
  s.Qk0 = (double*)(A + oQk0);
  s.Qka = (double*)(A + oQka);
  s.Qr2 = five ? (double*)(A + oQr2) : nullptr;
  s.Qr3 = five ? (double*)(A + oQr3) : nullptr;
  s.R0 = five ? (double*)(A + oR0) : nullptr;
  s.resid = (double*)(A + oRes);
  s.Qvf = (double*)(A + oQvf);
  s.Fc = (double*)(A + oFc);
  s.Azf = (double*)(A + oAzf);
  s.nQs = (double*)(A + onQs);
  s.nQvf = (double*)(A + onQvf);
  s.nAs = (double*)(A + onAs);
  s.met = (const double*)(A + omet);
  s.invJ = (const double*)(A + oinvJ);
  s.Se = (double*)(A + oSe);
  s.Se6 = s.Se + NC;
  s.muf = (double*)(A + omuf);
  s.diag = (double*)(A + odiag);
  s.face2 = (const int4*)(A + of2);
  s.face1 = (const int2*)(A + of1);
  s.fn2 = (const FaceNorm*)(A + ofn2);
  s.fn1 = (const FaceNorm*)(A + ofn1);
  s.act = (int*)(A + oact);
  s.nv = (int*)(A + onv);
  s.nbr = (const int4*)(A + onbr);
  s.nbrlf = (const int4*)(A + onbrlf);
  s.nQs9 = (double*)(A + onQs9);
  c->skip_option = 1;
  s.skip = (params->mu == 0.0 && params->eta0 == 0.0) ? 1 : 0;
  s.eig = (unsigned long long*)(A + oeig);
  s.err = (unsigned int*)(A + oerr);
  s.plot_flag = (const int*)(s.err + 1);  // zeroed with the arena
  c->red = (double*)(A + ored);
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->cp, cudaStreamNonBlocking) != cudaSuccess)
    return fail(set_err(CHORUS_ECUDA, "stream creation failed"));
  for (auto& ev : c->ev)
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
      return fail(set_err(CHORUS_ECUDA, "event creation failed"));
  if (cudaMallocHost(&c->h_pinned, 64 * sizeof(double)) != cudaSuccess)
    return fail(set_err(CHORUS_ECUDA, "pinned allocation failed"));
  e = cudaMemsetAsync(c->arena, 0, P.off, c->st);
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->st);
  };
  up((void*)s.met, met.data(), met.size() * sizeof(double));
  up((void*)s.invJ, invJ.data(), invJ.size() * sizeof(double));
  up((void*)s.face2, f2.data(), f2.size() * sizeof(int4));
  up((void*)s.face1, f1.data(), f1.size() * sizeof(int2));
  up((void*)s.fn2, fn2.data(), fn2.size() * sizeof(FaceNorm));
  up((void*)s.fn1, fn1.data(), fn1.size() * sizeof(FaceNorm));
  up((void*)s.nbr, nbr.data(), nbr.size() * sizeof(int4));
  up((void*)s.nbrlf, nbrlf.data(), nbrlf.size() * sizeof(int4));
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return fail(set_err(CHORUS_ECUDA, "upload failed: %s", cudaGetErrorString(e)));
  int rc = ensure_ops(device, N, Lmat, Mmat, Xs, Xf);
  if (rc) return fail(rc);
  *out = c;
  return CHORUS_OK;
}

int chorus_gpu_free(ChorusCtx* c) {
  if (!c) return CHORUS_OK;
  cudaSetDevice(c->device);
  if (c->g_step) cudaGraphExecDestroy(c->g_step);
  if (c->g_diag) cudaGraphExecDestroy(c->g_diag);
  drop_host_graphs(c);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->arena) cudaFree(c->arena);
  if (c->h_pinned) cudaFreeHost(c->h_pinned);
  if (c->cp) cudaStreamSynchronize(c->cp);
  if (c->st) cudaStreamDestroy(c->st);
  if (c->cp) cudaStreamDestroy(c->cp);
  for (auto& ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  delete c;
  return CHORUS_OK;
}

static void drop_graphs(ChorusCtx* c) {
  if (c->g_step) cudaGraphExecDestroy(c->g_step);
  if (c->g_diag) cudaGraphExecDestroy(c->g_diag);
  c->g_step = c->g_diag = nullptr;
  drop_host_graphs(c);
}

int chorus_gpu_set_params(ChorusCtx* c, const ChorusParams* p) {
  if (!c || !p) return set_err(CHORUS_EINVAL, "null argument");
  if (p->k_stage != c->p.k_stage) return set_err(CHORUS_EINVAL, "k_stage is fixed at bind time");
  c->p.dt = p->dt;
  c->p.mu = p->mu;
  c->p.eta0 = p->eta0;
  c->p.ARTIV = p->ARTIV;
  c->sd.mu = p->mu;
  c->sd.eta0 = p->eta0;
  c->sd.artiv = p->ARTIV == 1;
  c->sd.skip = (c->skip_option && p->mu == 0.0 && p->eta0 == 0.0) ? 1 : 0;
  drop_graphs(c);
  return CHORUS_OK;
}

int chorus_gpu_set_option(ChorusCtx* c, const char* name, int64_t value) {
  if (!c || !name) return set_err(CHORUS_EINVAL, "null argument");
  std::string n(name);
  if (n == "diagnostics") {
    c->diagnostics = value ? 1 : 0;
  } else if (n == "plot_sensor") {
    c->plot_sensor = value ? 1 : 0;
    CK(cudaMemsetAsync((void*)c->sd.plot_flag, c->plot_sensor, sizeof(int), c->st));
    return CHORUS_OK;  // read by the kernels at run time: the graphs stay valid
  } else if (n == "host_chunks") {
    if (value < 1 || value > kMaxHostChunks)
      return set_err(CHORUS_EINVAL, "host_chunks=%lld outside 1..%d", (long long)value, kMaxHostChunks);
    c->host_chunks = (int)value;
    c->hc.K = 0;
    drop_host_graphs(c);
    return CHORUS_OK;  // the step graphs do not use it
  } else if (n == "skip_inactive_viscous") {
    c->skip_option = value ? 1 : 0;
    c->sd.skip = (c->skip_option && c->p.mu == 0.0 && c->p.eta0 == 0.0) ? 1 : 0;
  } else if (n.rfind("epb_", 0) == 0 || n.rfind("threads_", 0) == 0) {
    const char* pass[4] = {"e1", "e2", "e3", "ct"};
    const bool epb = n[0] == 'e';
    const std::string which = n.substr(epb ? 4 : 8);
    int w = -1;
    for (int i = 0; i < 4; i++)
      if (which == pass[i]) w = i;
    if (w < 0) return set_err(CHORUS_EINVAL, "unknown option %s", name);
    if (epb) {
      if (value < 1 || value > 64) return set_err(CHORUS_EINVAL, "%s=%lld outside 1..64", name, (long long)value);
      c->L[w].epb = (int)value;
    } else {
      const int lim = w == 3 ? 256 : 512;  // the kernels' launch bounds
      if (value < 32 || value > lim || value % 32)
        return set_err(CHORUS_EINVAL, "%s=%lld must be 32..%d, a multiple of 32", name, (long long)value, lim);
      c->L[w].threads = (int)value;
    }
  } else {
    return set_err(CHORUS_EINVAL, "unknown option %s", name);
  }
  drop_graphs(c);
  return CHORUS_OK;
}

int64_t chorus_gpu_get_option(ChorusCtx* c, const char* name) {
  if (!c || !name) return -1;
  std::string n(name);
  if (n == "skip_inactive_viscous") return c->skip_option;
  if (n == "diagnostics") return c->diagnostics;
  if (n == "plot_sensor") return c->plot_sensor;
  if (n == "host_chunks") return c->host_chunks;
  if (n == "skip_active") return c->sd.skip;
  const char* pass[4] = {"e1", "e2", "e3", "ct"};
  for (int i = 0; i < 4; i++) {
    if (n == std::string("epb_") + pass[i]) return c->L[i].epb;
    if (n == std::string("threads_") + pass[i]) return c->L[i].threads;
  }
  return -1;
}

int chorus_gpu_upload_state(ChorusCtx* c, const double* Q) {
  if (!c || !Q) return set_err(CHORUS_EINVAL, "null argument");
  if (ctx_device(c)) return CHORUS_ECUDA;
  const size_t n = (size_t)c->dims.NCELL * c->dims.N * c->dims.N * 9;
  CK(cudaMemcpyAsync(c->sd.Q, Q, n * sizeof(double), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(c->sd.err, 0, sizeof(unsigned int), c->st));  // a new state: clear its error flags
  CK(cudaStreamSynchronize(c->st));
  return CHORUS_OK;
}

int chorus_gpu_download_state(ChorusCtx* c, double* Q) {
  if (!c || !Q) return set_err(CHORUS_EINVAL, "null argument");
  if (ctx_device(c)) return CHORUS_ECUDA;
  const size_t n = (size_t)c->dims.NCELL * c->dims.N * c->dims.N * 9;
  CK(cudaMemcpyAsync(Q, c->sd.Q, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return CHORUS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// stage sequences
// ---------------------------------------------------------------------------
namespace {

// one residual evaluation and stage update; `last` marks the last stage of a step (or a
// single compresid), whose E1 also records the variable-6 sensor the plot output reads
void enqueue_stage(ChorusCtx* c, const RKStage& rk, bool last) {
  const SolveDev& s = c->sd;
  c->D->e1(s, c->L[0], c->st, last ? 1 : 0, 0, -1);  // also zeroes the stage's wave speed
  c->qvf9_pending = false;
  c->D->f1(s, c->st, 0, -1, 0, -1);
  c->D->e2(s, c->L[1], c->st);  // also the face AV viscosities
  c->D->e3(s, rk, c->L[2], c->st, 0, -1);  // averages the grad Q traces where it reads them
}

void enqueue_ct(ChorusCtx* c) {
  c->D->ct(c->sd, c->L[3], c->st, 0, 0, -1);
  c->D->ct(c->sd, c->L[3], c->st, 1, 0, -1);
  c->D->ct(c->sd, c->L[3], c->st, 2, 0, -1);
  c->qvf9_pending = true;
}

// Qvf variable 9 from Azf, if a CT projection left it pending
void fill_qvf9(ChorusCtx* c) {
  if (!c->qvf9_pending) return;
  launch_qvf9(c->sd, c->st);
  c->qvf9_pending = false;
}

RKStage rk_blank() {
  RKStage r;
  std::memset(&r, 0, sizeof r);
  return r;
}

}  // namespace

// the records of the five stages of RK_S5P3 (iterations.f90:162-217) or FiveStageRk
// (:92-160) of one solve; `diag` marks the last stage to accumulate the residual norm
void chorus::rk_stage_records(const SolveDev& s, double dt, int k_stage, bool diag, RKStage* r) {
  for (int k = 0; k < 5; k++) std::memset(&r[k], 0, sizeof(RKStage));
  if (k_stage == 5) {
    const double a11 = 0.39175222700392, a21 = 0.44437049406734, a22 = 0.55562950593266, a23 = 0.36841059262959,
                 a31 = 0.6201018513854, a32 = 0.3798981486146, a33 = 0.25189177424738, a41 = 0.17807995410773,
                 a42 = 0.82192004589227, a43 = 0.54497475021237, a51 = 0.00683325884039, a52 = 0.51723167208978,
                 a53 = 0.12759831133288, a54 = 0.34833675773694, a55 = 0.08460416338212, a56 = 0.22600748319395;
    r[0].cQ = 1.0; r[0].cR = dt * a11; r[0].save_old = s.Qk0;
    r[1].nsrc = 1; r[1].src[0] = s.Qk0; r[1].c[0] = a21; r[1].cQ = a22; r[1].cR = a23 * dt; r[1].save_new = s.Qr2;
    r[2].nsrc = 1; r[2].src[0] = s.Qk0; r[2].c[0] = a31; r[2].cQ = a32; r[2].cR = a33 * dt; r[2].save_new = s.Qr3;
    r[3].nsrc = 1; r[3].src[0] = s.Qk0; r[3].c[0] = a41; r[3].cQ = a42; r[3].cR = a43 * dt; r[3].save_R = s.R0;
    r[4].nsrc = 3; r[4].src[0] = s.Qk0; r[4].src[1] = s.Qr2; r[4].src[2] = s.Qr3;
    r[4].c[0] = a51; r[4].c[1] = a52; r[4].c[2] = a53; r[4].cQ = a54; r[4].cR = a56 * dt;
    r[4].R0 = s.R0; r[4].cR0 = a55 * dt;
  } else {
    const double a30 = 0.355909775063327, a32 = 0.644090224936674, a40 = 0.367933791638137,
                 a43 = 0.632066208361863, a52 = 0.237593836598569, a54 = 0.762406163401431,
                 b10 = 0.377268915331368, b21 = 0.377268915331368, b32 = 0.242995220537396,
                 b43 = 0.238458932846290, b54 = 0.287632146308408;
    r[0].cQ = 1.0; r[0].cR = b10 * dt; r[0].save_old = s.Qk0;
    r[1].cQ = 1.0; r[1].cR = b21 * dt; r[1].save_new = s.Qka;
    r[2].nsrc = 1; r[2].src[0] = s.Qk0; r[2].c[0] = a30; r[2].cQ = a32; r[2].cR = b32 * dt;
    r[3].nsrc = 1; r[3].src[0] = s.Qk0; r[3].c[0] = a40; r[3].cQ = a43; r[3].cR = b43 * dt;
    r[4].nsrc = 1; r[4].src[0] = s.Qka; r[4].c[0] = a52; r[4].cQ = a54; r[4].cR = b54 * dt;
  }
  r[4].diag = diag ? 1 : 0;
  r[4].write_resid = 1;  // the last stage's residual stays available like the reference's resid
}

namespace {

void make_rk(ChorusCtx* c, bool diag, RKStage* r) { rk_stage_records(c->sd, c->p.dt, c->p.k_stage, diag, r); }

void enqueue_rk(ChorusCtx* c, bool diag) {
  RKStage r[5];
  make_rk(c, diag, r);
  for (int k = 0; k < 5; k++) enqueue_stage(c, r[k], k == 4);
}

__global__ void k_store_record(const double* red2, const unsigned long long* eig, double* rec) {
  rec[0] = red2[0];
  rec[1] = red2[1];
  rec[2] = __longlong_as_double((long long)eig[0]);
}

// diagnostic of iterations.f90:35-76 on the CT-corrected state
void enqueue_diag(ChorusCtx* c) {
  const SolveDev& s = c->sd;
  // comp_inviscid_flux + nablaQsp(6,7) (iterations.f90:35-36) of which the norms read
  // only the face-averaged B_x, B_y traces; the record keeps the last stage's wave speed
  c->D->diag(s, c->L[3], c->st, 0);
  c->D->diag(s, c->L[3], c->st, 1);
  c->D->nqsp(s, 5, 6, c->st);
  c->D->divb(s, c->st);
  launch_reduce_diag(s.diag, s.NC, c->red, c->st);
  k_store_record<<<1, 1, 0, c->st>>>(c->red, c->sd.eig, c->red + 4);
}

// the chunk plan of a host-state step from the keys of the face lists: the larger cell of
// each two-sided face and the cell of each FREE face (both ascending), and per cell the
// largest index among itself and its face neighbours
void plan_host_chunks(int NC, int chunks, const std::vector<int>& f2max, const std::vector<int>& f1cell,
                      const std::vector<int>& cellrel, HostChunks& h) {
  h.K = std::max(1, std::min(chunks, NC / 1024));
  // chunk sizes taper towards both ends (weights min(k+1, K-k, 4)): the first upload chunk
  // is all the compute waits for, the last download run all that follows it
  long long wsum[kMaxHostChunks + 1] = {0};
  for (int k = 0; k < h.K; k++) wsum[k + 1] = wsum[k] + std::min(std::min(k + 1, h.K - k), 4);
  for (int k = 0; k <= h.K; k++) {
    h.cut[k] = (int)((long long)NC * wsum[k] / wsum[h.K]);
    h.f2[k] = (int)(std::lower_bound(f2max.begin(), f2max.end(), h.cut[k]) - f2max.begin());
    h.f1[k] = (int)(std::lower_bound(f1cell.begin(), f1cell.end(), h.cut[k]) - f1cell.begin());
  }
  // the chunk that completes each cell's neighbourhood (cellrel >= the cell itself)
  auto chunk_of = [&](int ic) {
    return (int)(std::upper_bound(h.cut + 1, h.cut + h.K + 1, ic) - (h.cut + 1));
  };
  h.nseg = 0;
  for (int ic = 0; ic < NC;) {
    const int k = chunk_of(cellrel[ic]);
    int e = ic + 1;
    while (e < NC && chunk_of(cellrel[e]) == k) e++;
    if (h.nseg == kMaxHostSegs) {
      h.nseg = -1;
      break;
    }
    h.sb[h.nseg] = ic;
    h.se[h.nseg] = e;
    h.sk[h.nseg] = k;
    h.nseg++;
    ic = e;
  }
  if (h.nseg < 0) {  // fragmented: whole chunks, each when its last neighbour is through
    h.nseg = h.K;
    for (int j = 0; j < h.K; j++) {
      int r = h.cut[j + 1] - 1;
      for (int ic = h.cut[j]; ic < h.cut[j + 1]; ic++) r = std::max(r, cellrel[ic]);
      h.sb[j] = h.cut[j];
      h.se[j] = h.cut[j + 1];
      h.sk[j] = chunk_of(r);
    }
  }
}

const HostChunks& host_chunks(ChorusCtx* c) {
  if (!c->hc.K) plan_host_chunks(c->sd.NC, c->host_chunks, c->f2max, c->f1cell, c->cellrel, c->hc);
  return c->hc;
}

// One step whose state comes from / goes to host memory, the copies (on the copy stream,
// in chunks of cells) overlapped with the passes that can run chunk by chunk:
//  - the first stage's E1 on each chunk as soon as its cells have arrived, and F1 on the
//    faces whose cells have all been through E1 (E2 waits for every face: it reads the
//    stage's maximum wave speed);
//  - the last stage's E3 chunk by chunk, each chunk followed by the A_z traces of the CT
//    projection and their average on the faces whose cells are all updated; a run of
//    cells whose cells and face neighbours are all through that gets its B (the last CT
//    pass) and its download.
// Every pass runs on every cell and face exactly once, as in the step graph, so the
// results are the graph's bit for bit.
void enqueue_step_host(ChorusCtx* c, bool diag, const double* Qin, double* Qout) {
  const SolveDev& s = c->sd;
  const HostChunks& h = host_chunks(c);
  const int K = h.K;
  const size_t per = (size_t)s.N * s.N * 9;
  auto off = [&](int j) { return (size_t)h.cut[j] * per; };
  auto bytes = [&](int j) { return (size_t)(h.cut[j + 1] - h.cut[j]) * per * sizeof(double); };
  auto off_s = [&](int i) { return (size_t)h.sb[i] * per; };
  auto bytes_s = [&](int i) { return (size_t)(h.se[i] - h.sb[i]) * per * sizeof(double); };
  RKStage r[5];
  make_rk(c, diag, r);
  if (Qin) {
    cudaEventRecord(c->ev[kMaxHostChunks + kMaxHostSegs], c->st);  // earlier work on the state is done
    cudaStreamWaitEvent(c->cp, c->ev[kMaxHostChunks + kMaxHostSegs], 0);
    for (int k = 0; k < K; k++) {
      cudaMemcpyAsync(s.Q + off(k), Qin + off(k), bytes(k), cudaMemcpyHostToDevice, c->cp);
      cudaEventRecord(c->ev[k], c->cp);
      cudaStreamWaitEvent(c->st, c->ev[k], 0);
      c->D->e1(s, c->L[0], c->st, 0, h.cut[k], h.cut[k + 1]);  // the first chunk zeroes the wave speed
      c->D->f1(s, c->st, h.f2[k], h.f2[k + 1], h.f1[k], h.f1[k + 1]);
    }
  } else {
    c->D->e1(s, c->L[0], c->st, 0, 0, -1);
    c->D->f1(s, c->st, 0, -1, 0, -1);
  }
  c->D->e2(s, c->L[1], c->st);
  c->D->e3(s, r[0], c->L[2], c->st, 0, -1);
  for (int k = 1; k < 4; k++) enqueue_stage(c, r[k], false);
  c->D->e1(s, c->L[0], c->st, 1, 0, -1);
  c->D->f1(s, c->st, 0, -1, 0, -1);
  c->D->e2(s, c->L[1], c->st);
  if (Qout) {
    for (int k = 0; k < K; k++) {
      c->D->e3(s, r[4], c->L[2], c->st, h.cut[k], h.cut[k + 1]);
      c->D->ct(s, c->L[3], c->st, 0, h.cut[k], h.cut[k + 1]);
      c->D->ct(s, c->L[3], c->st, 1, h.f2[k], h.f2[k + 1]);
      for (int i = 0; i < h.nseg; i++) {
        if (h.sk[i] != k) continue;
        c->D->ct(s, c->L[3], c->st, 2, h.sb[i], h.se[i]);
        cudaEventRecord(c->ev[kMaxHostChunks + i], c->st);
        cudaStreamWaitEvent(c->cp, c->ev[kMaxHostChunks + i], 0);
        cudaMemcpyAsync(Qout + off_s(i), s.Q + off_s(i), bytes_s(i), cudaMemcpyDeviceToHost, c->cp);
      }
    }
  } else {
    c->D->e3(s, r[4], c->L[2], c->st, 0, -1);
    c->D->ct(s, c->L[3], c->st, 0, 0, -1);
    c->D->ct(s, c->L[3], c->st, 1, 0, -1);
    c->D->ct(s, c->L[3], c->st, 2, 0, -1);
  }
  c->qvf9_pending = true;
  if (diag) enqueue_diag(c);  // reads Q only: it may overlap the download
}

// page-locked host memory (cudaHostAlloc / cudaHostRegister), which a captured copy may
// address; null counts as such (no copy)
bool pinned_host(const void* p) {
  if (!p) return true;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// the captured host-state step for (qin, qout, diag), captured on first use; the copy
// stream joins the main stream at its end, so the graph's completion covers the download
cudaGraphExec_t host_graph(ChorusCtx* c, bool diag, const double* qin, double* qout) {
  for (const HostGraph& g : c->hg)
    if (g.ex && g.qin == qin && g.qout == qout && g.diag == (int)diag) return g.ex;
  HostGraph& g = c->hg[c->hg_next];
  c->hg_next = (c->hg_next + 1) % kHostGraphs;
  if (g.ex) cudaGraphExecDestroy(g.ex);
  g = HostGraph{};
  if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return nullptr;
  enqueue_step_host(c, diag, qin, qout);
  cudaEventRecord(c->ev[kEvJoin], c->cp);
  cudaStreamWaitEvent(c->st, c->ev[kEvJoin], 0);
  cudaGraph_t gr = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->st, &gr);
  if (e != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    return nullptr;
  }
  e = cudaGraphInstantiate(&g.ex, gr, 0);
  cudaGraphDestroy(gr);
  if (e != cudaSuccess) {
    g.ex = nullptr;
    return nullptr;
  }
  g.qin = qin;
  g.qout = qout;
  g.diag = diag ? 1 : 0;
  return g.ex;
}

int build_graphs(ChorusCtx* c) {
  drop_graphs(c);
  for (int which = 0; which < 2; which++) {
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    enqueue_rk(c, which == 1);
    enqueue_ct(c);
    if (which == 1) enqueue_diag(c);
    CK(cudaStreamEndCapture(c->st, &g));
    cudaGraphExec_t ex;
    cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
    (which ? c->g_diag : c->g_step) = ex;
  }
  c->graph_dt = c->p.dt;
  c->graph_k = c->p.k_stage;
  return CHORUS_OK;
}

int check_err_flag(ChorusCtx* c) {
  unsigned int h = 0;
  CK(cudaMemcpyAsync(&h, c->sd.err, sizeof h, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (h) return set_err(CHORUS_ESTATE, "kernels flagged a non-finite wave speed (state is not physical)");
  return CHORUS_OK;
}

void advance_ctime(int k_stage, double dt, double* ctime) {
  if (!ctime) return;
  // ctime bookkeeping of RK_S5P3 / FiveStageRk: the step ends at ctime0 + dt
  (void)k_stage;
  *ctime = *ctime + dt;
}

}  // namespace

extern "C" {

int compresid_gpu(ChorusCtx* c) {
  if (!c) return set_err(CHORUS_EINVAL, "null context");
  if (ctx_device(c)) return CHORUS_ECUDA;
  RKStage r = rk_blank();
  r.write_resid = 1;
  enqueue_stage(c, r, true);
  c->se6_valid = c->plot_sensor;
  CK(cudaGetLastError());
  return check_err_flag(c);
}

int comp_inviscid_flux_gpu(ChorusCtx* c) {
  if (!c) return set_err(CHORUS_EINVAL, "null context");
  if (ctx_device(c)) return CHORUS_ECUDA;
  c->D->e1ns(c->sd, c->L[0], c->st);
  c->qvf9_pending = false;
  c->D->f1(c->sd, c->st, 0, -1, 0, -1);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  return CHORUS_OK;
}

int nablaqsp_gpu(ChorusCtx* c, const int32_t* v_sta, const int32_t* v_end) {
  if (!c || !v_sta || !v_end) return set_err(CHORUS_EINVAL, "null argument");
  if (*v_sta < 1 || *v_end > 9 || *v_sta > *v_end) return set_err(CHORUS_EINVAL, "variable range %d..%d", *v_sta, *v_end);
  if (ctx_device(c)) return CHORUS_ECUDA;
  if (*v_end == 9) fill_qvf9(c);  // nablaQsp(9,9) reads the A_z traces
  c->D->nqsp(c->sd, *v_sta - 1, *v_end - 1, c->st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  return CHORUS_OK;
}

int correct_b_via_curl_az_gpu(ChorusCtx* c) {
  if (!c) return set_err(CHORUS_EINVAL, "null context");
  if (ctx_device(c)) return CHORUS_ECUDA;
  enqueue_ct(c);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  return CHORUS_OK;
}

static int one_step(ChorusCtx* c, double* ctime, int k_stage) {
  if (!c) return set_err(CHORUS_EINVAL, "null context");
  if (c->p.k_stage != k_stage) return set_err(CHORUS_EINVAL, "context was bound with k_stage=%d", c->p.k_stage);
  if (ctx_device(c)) return CHORUS_ECUDA;
  enqueue_rk(c, false);
  c->se6_valid = c->plot_sensor;
  CK(cudaGetLastError());
  advance_ctime(k_stage, c->p.dt, ctime);
  return check_err_flag(c);
}

int rk_s5p3_gpu(ChorusCtx* c, double* ctime) { return one_step(c, ctime, 3); }
int fivestagerk_gpu(ChorusCtx* c, double* ctime) { return one_step(c, ctime, 5); }

static int run_steps(ChorusCtx* c, int32_t nsteps, int32_t* iter, double* ctime, ChorusDiag* diag, int32_t max_diag,
                     int32_t* n_diag, const double* Qin, double* Qout);

int iterations_gpu(ChorusCtx* c, int32_t nsteps, int32_t* iter, double* ctime, ChorusDiag* diag, int32_t max_diag,
                   int32_t* n_diag) {
  return run_steps(c, nsteps, iter, ctime, diag, max_diag, n_diag, nullptr, nullptr);
}

int chorus_gpu_step_host(ChorusCtx* c, const double* Qin, double* Qout, int32_t nsteps, int32_t* iter, double* ctime,
                         ChorusDiag* diag, int32_t max_diag, int32_t* n_diag) {
  if (nsteps < 1) return set_err(CHORUS_EINVAL, "nsteps must be at least 1");
  return run_steps(c, nsteps, iter, ctime, diag, max_diag, n_diag, Qin, Qout);
}

static int run_steps(ChorusCtx* c, int32_t nsteps, int32_t* iter, double* ctime, ChorusDiag* diag, int32_t max_diag,
                     int32_t* n_diag, const double* Qin, double* Qout) {
  if (!c || !iter || nsteps < 0) return set_err(CHORUS_EINVAL, "bad argument");
  if (ctx_device(c)) return CHORUS_ECUDA;
  if (!c->g_step || c->graph_dt != c->p.dt || c->graph_k != c->p.k_stage) {
    int rc = build_graphs(c);
    if (rc) return rc;
  }
  int nd = 0;
  std::vector<int> diag_iters;
  std::vector<double> diag_times;
  const int N = c->dims.N;
  double* recs = c->h_pinned;  // up to 16 records of 3 doubles per sync window
  int pending = 0;
  auto flush = [&]() -> int {
    if (!pending) return CHORUS_OK;
    CK(cudaStreamSynchronize(c->st));
    for (int i = 0; i < pending; i++) {
      if (diag && nd < max_diag) {
        ChorusDiag& d = diag[nd];
        std::memset(&d, 0, sizeof d);
        d.iter = diag_iters[i];
        d.ctime = diag_times[i];
        const double nglob = (double)c->p.NCELLGLOB;
        d.residglob = std::sqrt(recs[3 * i] / (double)(c->p.NCELLGLOB * N * N * 5));
        d.divBglob = std::sqrt(recs[3 * i + 1] / (nglob * N * N));
        d.eigvmax_g = recs[3 * i + 2];
        d.epsilon0 = d.eigvmax_g * c->sd.hmsh / (N - 1) * 1.0;
      }
      nd++;
    }
    pending = 0;
    diag_iters.clear();
    diag_times.clear();
    return CHORUS_OK;
  };
  if (Qin) CK(cudaMemsetAsync(c->sd.err, 0, sizeof(unsigned int), c->st));  // a new state: clear its error flags
  for (int s = 0; s < nsteps; s++) {
    *iter = *iter + 1;
    const bool d = c->diagnostics && (*iter % 10) == 1;
    const double* qin = s == 0 ? Qin : nullptr;
    double* qout = s == nsteps - 1 ? Qout : nullptr;
    const size_t qbytes = (size_t)c->dims.NCELL * N * N * 9 * sizeof(double);
    if ((qin || qout) && qbytes >= ((size_t)64 << 20)) {
      // large states: copies in chunks, overlapped with the passes that can run chunk by
      // chunk; one graph launch for pinned buffers, the calls one by one for pageable
      // ones (a copy from pageable memory cannot be captured)
      if (pinned_host(qin) && pinned_host(qout)) {
        cudaGraphExec_t ex = host_graph(c, d, qin, qout);
        if (!ex) {
          cudaGetLastError();
          return set_err(CHORUS_ECUDA, "capturing the host-state step failed");
        }
        CK(cudaGraphLaunch(ex, c->st));
      } else {
        enqueue_step_host(c, d, qin, qout);
        CK(cudaGetLastError());
      }
    } else {
      // small states: the copies take less than the launches a chunked step would add
      if (qin) CK(cudaMemcpyAsync(c->sd.Q, qin, qbytes, cudaMemcpyHostToDevice, c->st));
      CK(cudaGraphLaunch(d ? c->g_diag : c->g_step, c->st));
      if (qout) CK(cudaMemcpyAsync(qout, c->sd.Q, qbytes, cudaMemcpyDeviceToHost, c->st));
    }
    if (ctime) *ctime = *ctime + c->p.dt;
    if (d) {
      CK(cudaMemcpyAsync(recs + 3 * pending, c->red + 4, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
      diag_iters.push_back(*iter);
      diag_times.push_back(ctime ? *ctime : 0.0);
      pending++;
      if (pending == 16) {
        int rc = flush();
        if (rc) return rc;
      }
    }
  }
  int rc = flush();
  if (rc) return rc;
  if (n_diag) *n_diag = nd;
  if (nsteps > 0) {
    c->se6_valid = c->plot_sensor;
    c->qvf9_pending = true;  // every step ends with the CT projection
  }
  if (Qout) CK(cudaStreamSynchronize(c->cp));
  return check_err_flag(c);
}

void* chorus_gpu_stream(ChorusCtx* c) { return c ? (void*)c->st : nullptr; }

int64_t chorus_gpu_device_bytes(ChorusCtx* c) { return c ? (int64_t)c->arena_bytes : 0; }

int chorus_gpu_launch_counts(ChorusCtx* c, int32_t* per_step, int32_t* per_diag) {
  if (!c) return set_err(CHORUS_EINVAL, "null context");
  const int nf = (c->nface2 + c->nface1) > 0 ? 1 : 0;
  const int stage = 3 + nf;             // E1 E2 E3 (+ F1)
  const int ct = 2 + (c->nface2 > 0);   // element passes + face average
  if (per_step) *per_step = 5 * stage + ct;
  if (per_diag) *per_diag = 1 + (c->nface2 > 0) + 4;  // B traces, face average, nablaQsp, divB, reduce, record
  return CHORUS_OK;
}

int chorus_gpu_profile_stage(ChorusCtx* c, int32_t reps, double* ms) {
  if (!c || !ms || reps <= 0) return set_err(CHORUS_EINVAL, "bad argument");
  if (ctx_device(c)) return CHORUS_ECUDA;
  cudaEvent_t ev[6];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  double acc[6] = {0, 0, 0, 0, 0, 0};
  RKStage r = rk_blank();
  r.cQ = 1.0;
  r.cR = 0.377268915331368 * c->p.dt;
  const SolveDev& s = c->sd;
  for (int it = 0; it < reps; it++) {
    CK(cudaMemsetAsync(s.eig, 0, sizeof(unsigned long long), c->st));
    CK(cudaEventRecord(ev[0], c->st));
    c->D->e1(s, c->L[0], c->st, 0, 0, -1);
    c->qvf9_pending = false;
    CK(cudaEventRecord(ev[1], c->st));
    c->D->f1(s, c->st, 0, -1, 0, -1);
    CK(cudaEventRecord(ev[2], c->st));
    c->D->e2(s, c->L[1], c->st);
    CK(cudaEventRecord(ev[3], c->st));
    CK(cudaEventRecord(ev[4], c->st));  // the former F2 pass lives in E2 and E3
    c->D->e3(s, r, c->L[2], c->st, 0, -1);
    CK(cudaEventRecord(ev[5], c->st));
    CK(cudaEventSynchronize(ev[5]));
    float t;
    for (int k = 0; k < 5; k++) {
      CK(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
      acc[k] += t;
    }
    CK(cudaEventElapsedTime(&t, ev[0], ev[5]));
    acc[5] += t;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  for (int k = 0; k < 6; k++) ms[k] = acc[k] / reps;
  return check_err_flag(c);
}

int chorus_gpu_get_eigvmax(ChorusCtx* c, double* eigvmax_g, double* epsilon0) {
  if (!c) return set_err(CHORUS_EINVAL, "null context");
  if (ctx_device(c)) return CHORUS_ECUDA;
  unsigned long long b = 0;
  CK(cudaMemcpyAsync(&b, c->sd.eig, sizeof b, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  double ev;
  std::memcpy(&ev, &b, sizeof ev);
  if (eigvmax_g) *eigvmax_g = ev;
  if (epsilon0) *epsilon0 = ev * c->sd.hmsh / (c->dims.N - 1) * 1.0;
  return CHORUS_OK;
}

int chorus_gpu_download_array(ChorusCtx* c, const char* name, double* out, int64_t count) {
  if (!c || !name || !out) return set_err(CHORUS_EINVAL, "null argument");
  if (ctx_device(c)) return CHORUS_ECUDA;
  const int N = c->dims.N, NC = c->dims.NCELL, NS = N * N, NF1 = (N + 1) * N, NFP = 2 * NF1;
  const SolveDev& s = c->sd;
  std::string n(name);
  auto pull = [&](const double* src, size_t cnt, std::vector<double>& h) -> int {
    h.resize(cnt);
    CK(cudaMemcpyAsync(h.data(), src, cnt * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return CHORUS_OK;
  };
  std::vector<double> h;
  // same layout as the reference
  struct Same { const char* nm; const double* p; size_t cnt; } same[] = {
      {"resid", s.resid, (size_t)NC * NS * 9}, {"nablaQs", s.nQs, (size_t)NC * NS * 18},
      {"nablaAs", s.nAs, (size_t)NC * NS * 2}, {"Q", s.Q, (size_t)NC * NS * 9}, {"SM_IND1", s.Se, (size_t)NC}};
  for (auto& x : same)
    if (n == x.nm) {
      if ((size_t)count != x.cnt) return set_err(CHORUS_EINVAL, "%s has %zu elements, not %lld", name, x.cnt, (long long)count);
      CK(cudaMemcpyAsync(out, x.p, x.cnt * sizeof(double), cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      if (x.p == s.nQs) {  // variable 9 lives in its own array
        int rc = pull(s.nQs9, (size_t)NC * NS * 2, h);
        if (rc) return rc;
        for (size_t pt = 0; pt < (size_t)NC * NS; pt++) {
          out[pt * 18 + 8] = h[2 * pt];
          out[pt * 18 + 17] = h[2 * pt + 1];
        }
      }
      if (n == "SM_IND1")  // the device keeps the sensor sum; Se = log10(sum) (AV.f90:79)
        for (size_t i = 0; i < x.cnt; i++) out[i] = std::log10(out[i]);
      return CHORUS_OK;
    }
  // per-cell flux-point blocks split into the family-1 / family-2 arrays
  struct Split { const char* nm; const double* p; int w; int fam; } split[] = {
      {"Qvfi", s.Qvf, 9, 0}, {"Qvfj", s.Qvf, 9, 1}, {"F1", s.Fc, 8, 0}, {"G2", s.Fc, 8, 1},
      {"Azfi", s.Azf, 1, 0}, {"Azfj", s.Azf, 1, 1}, {"nablaQvfi", s.nQvf, 18, 0}, {"nablaQvfj", s.nQvf, 18, 1}};
  for (auto& x : split)
    if (n == x.nm) {
      // the stage averages the grad Q traces where it reads them: store the averages
      // (idempotent) so that the arrays equal the reference's nablaQvfi / nablaQvfj
      if (x.p == s.nQvf) c->D->f2(s, c->st);
      if (x.p == s.Qvf) fill_qvf9(c);
      const size_t per = (size_t)NF1 * x.w;
      if ((size_t)count != per * NC) return set_err(CHORUS_EINVAL, "%s has %zu elements", name, per * NC);
      int rc = pull(x.p, (size_t)NC * NFP * x.w, h);
      if (rc) return rc;
      for (int e = 0; e < NC; e++)
        std::memcpy(out + per * e, h.data() + ((size_t)e * NFP + (size_t)x.fam * NF1) * x.w, per * sizeof(double));
      return CHORUS_OK;
    }
  if (n == "av_active" || n == "viscous_cells") {
    if ((size_t)count != (size_t)NC) return set_err(CHORUS_EINVAL, "%s has %d elements", name, NC);
    std::vector<int> hi(NC);
    CK(cudaMemcpyAsync(hi.data(), n == "av_active" ? s.act : s.nv, NC * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (int e = 0; e < NC; e++) out[e] = hi[e];
    return CHORUS_OK;
  }
  if (n == "muAVfi" || n == "muAVfj") {
    if ((size_t)count != (size_t)NC * 18) return set_err(CHORUS_EINVAL, "%s has %d elements", name, NC * 18);
    int rc = pull(s.muf, (size_t)NC * 4, h);
    if (rc) return rc;
    std::memset(out, 0, sizeof(double) * NC * 18);
    const bool fi = n == "muAVfi";
    for (int e = 0; e < NC; e++) {
      out[0 + 9 * (0 + 2 * e)] = fi ? h[4 * e + 3] : h[4 * e + 0];
      out[0 + 9 * (1 + 2 * e)] = fi ? h[4 * e + 1] : h[4 * e + 2];
    }
    return CHORUS_OK;
  }
  return set_err(CHORUS_EINVAL, "unknown array %s", name);
}

// ---------------------------------------------------------------------------
// point functions over n points (host arrays)
// ---------------------------------------------------------------------------
}  // extern "C"
template <typename T>
static int dev_copy(T** d, const T* h, size_t n, cudaStream_t st) {
  CK(cudaMalloc(d, std::max<size_t>(n, 1) * sizeof(T)));
  if (h) CK(cudaMemcpyAsync(*d, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
  return CHORUS_OK;
}
// device scratch of one point-function call: every buffer it hands out is freed when the
// call returns, on every path
struct DevScratch {
  std::vector<void*> bufs;
  template <typename T>
  int copy(T** d, const T* h, size_t n, cudaStream_t st) {
    *d = nullptr;
    const int rc = dev_copy(d, h, n, st);
    if (*d) bufs.push_back((void*)*d);
    return rc;
  }
  ~DevScratch() {
    for (void* b : bufs) cudaFree(b);
  }
};
extern "C" {

int getrusanovflux_gpu(int32_t n, double gam, const double* Qfl, const double* Qfr, double* Fnl, double* Fnr,
                       double* Az, const double* normf, const int32_t* sign_l, const int32_t* sign_r, double* eigv) {
  if (n < 0 || (n > 0 && (!Qfl || !Qfr || !Fnl || !Fnr || !Az || !normf || !sign_l || !sign_r || !eigv)))
    return set_err(CHORUS_EINVAL, "bad argument");
  if (n == 0) return CHORUS_OK;
  DevScratch S;
  double *a, *b, *fl, *fr, *az, *nf, *ev;
  int *sl, *sr;
  cudaStream_t st = 0;
  int rc = S.copy(&a, Qfl, 9 * (size_t)n, st) || S.copy(&b, Qfr, 9 * (size_t)n, st) ||
           S.copy<double>(&fl, nullptr, 8 * (size_t)n, st) || S.copy<double>(&fr, nullptr, 8 * (size_t)n, st) ||
           S.copy<double>(&az, nullptr, n, st) || S.copy(&nf, normf, 2 * (size_t)n, st) ||
           S.copy<double>(&ev, nullptr, n, st) || S.copy(&sl, (const int*)sign_l, n, st) ||
           S.copy(&sr, (const int*)sign_r, n, st);
  if (rc) return CHORUS_ECUDA;
  launch_point_rusanov(n, gam, a, b, fl, fr, az, nf, sl, sr, ev, st);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(Fnl, fl, 8 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(Fnr, fr, 8 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(Az, az, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(eigv, ev, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "getrusanovflux_gpu: %s", cudaGetErrorString(e));
  return CHORUS_OK;
}

int getifluxvectors_gpu(int32_t n, double gam, const double* Qi, double* Fi, double* Gi) {
  if (n < 0 || (n > 0 && (!Qi || !Fi || !Gi))) return set_err(CHORUS_EINVAL, "bad argument");
  if (n == 0) return CHORUS_OK;
  DevScratch S;
  double *q, *f, *g;
  if (S.copy(&q, Qi, 8 * (size_t)n, 0) || S.copy<double>(&f, nullptr, 8 * (size_t)n, 0) ||
      S.copy<double>(&g, nullptr, 8 * (size_t)n, 0))
    return CHORUS_ECUDA;
  launch_point_iflux(n, gam, q, f, g, 0);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(Fi, f, 8 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(Gi, g, 8 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "getifluxvectors_gpu: %s", cudaGetErrorString(e));
  return CHORUS_OK;
}

int getvfluxvectors_gpu(int32_t n, double gam, double mu, double eta0, const double* Qv, const double* nablaQ,
                        double* Fv, double* Gv) {
  if (n < 0 || (n > 0 && (!Qv || !nablaQ || !Fv || !Gv))) return set_err(CHORUS_EINVAL, "bad argument");
  if (n == 0) return CHORUS_OK;
  DevScratch S;
  double *q, *g, *f, *h;
  if (S.copy(&q, Qv, 9 * (size_t)n, 0) || S.copy(&g, nablaQ, 18 * (size_t)n, 0) ||
      S.copy<double>(&f, nullptr, 9 * (size_t)n, 0) || S.copy<double>(&h, nullptr, 9 * (size_t)n, 0))
    return CHORUS_ECUDA;
  launch_point_vflux(n, gam, mu, eta0, q, g, f, h, 0);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(Fv, f, 9 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(Gv, h, 9 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "getvfluxvectors_gpu: %s", cudaGetErrorString(e));
  return CHORUS_OK;
}

int getvfluxvectors_av_gpu(ChorusCtx* c, int32_t n, const double* Qv, const double* nablaQ, double* Fv, double* Gv,
                           const int32_t* fam, const int32_t* ifp, const int32_t* jfp, const int32_t* ic) {
  if (!c) return set_err(CHORUS_EINVAL, "null context");
  if (n < 0 || (n > 0 && (!Qv || !nablaQ || !Fv || !Gv || !fam || !ifp || !jfp || !ic)))
    return set_err(CHORUS_EINVAL, "bad argument");
  if (n == 0) return CHORUS_OK;
  DevScratch S;
  const int N = c->dims.N, NC = c->dims.NCELL;
  for (int i = 0; i < n; i++) {
    const int f = fam[i], ni = f == 1 ? N + 1 : N, nj = f == 1 ? N : N + 1;
    if ((f != 1 && f != 2) || ifp[i] < 1 || ifp[i] > ni || jfp[i] < 1 || jfp[i] > nj || ic[i] < 1 || ic[i] > NC)
      return set_err(CHORUS_EINVAL, "point %d: (fam, ifp, jfp, ic) = (%d, %d, %d, %d) out of range", i, f, ifp[i],
                     jfp[i], ic[i]);
  }
  int rc = ctx_device(c);
  if (rc) return rc;
  PointAxes ax{};
  for (int k = 0; k <= N; k++) ax.Xf[k] = c->Xf[k];
  double *q, *g, *f, *h;
  int *dfam, *di, *dj, *dc;
  cudaStream_t st = c->st;  // ordered after the context's own work (muf of the last stage)
  if (S.copy(&q, Qv, 9 * (size_t)n, st) || S.copy(&g, nablaQ, 18 * (size_t)n, st) ||
      S.copy<double>(&f, nullptr, 9 * (size_t)n, st) || S.copy<double>(&h, nullptr, 9 * (size_t)n, st) ||
      S.copy(&dfam, fam, (size_t)n, st) || S.copy(&di, ifp, (size_t)n, st) || S.copy(&dj, jfp, (size_t)n, st) ||
      S.copy(&dc, ic, (size_t)n, st))
    return CHORUS_ECUDA;
  launch_point_vflux_av(n, c->p.gam, ax, c->sd.muf, dfam, di, dj, dc, q, g, f, h, st);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpy(Fv, f, 9 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(Gv, h, 9 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "getvfluxvectors_av_gpu: %s", cudaGetErrorString(e));
  return CHORUS_OK;
}

// single-point forms with the reference's argument lists; the physical constants that
// the reference reads from module state (gam, mu, eta0: setup2d.f90:68,72,77) come from
// chorus_point_set_params.  Each evaluates on the device through the n-point entries.
static std::mutex g_point_mu;
static double g_point_gam = 5.0 / 3.0, g_point_mu_v = 0.0, g_point_eta0 = 0.0;

int chorus_point_set_params(double gam, double mu, double eta0) {
  if (!(gam > 1.0) || !(mu >= 0.0) || !(eta0 >= 0.0)) return set_err(CHORUS_EINVAL, "bad point parameters");
  std::lock_guard<std::mutex> lk(g_point_mu);
  g_point_gam = gam;
  g_point_mu_v = mu;
  g_point_eta0 = eta0;
  return CHORUS_OK;
}

static void point_params(double* gam, double* mu, double* eta0) {
  std::lock_guard<std::mutex> lk(g_point_mu);
  *gam = g_point_gam;
  if (mu) *mu = g_point_mu_v;
  if (eta0) *eta0 = g_point_eta0;
}

int getrusanovflux_c(const double* Qfl, const double* Qfr, double* Fnl, double* Fnr, double* Az, const double* normf,
                     const int32_t* sign_l, const int32_t* sign_r, double* eigv, double* eigvmax) {
  if (!Qfl || !Qfr || !Fnl || !Fnr || !Az || !normf || !sign_l || !sign_r || !eigv || !eigvmax)
    return set_err(CHORUS_EINVAL, "null argument");
  double gam;
  point_params(&gam, nullptr, nullptr);
  int rc = getrusanovflux_gpu(1, gam, Qfl, Qfr, Fnl, Fnr, Az, normf, sign_l, sign_r, eigv);
  if (rc) return rc;
  if (*eigv > *eigvmax) *eigvmax = *eigv;  // getrusanov.f90:105-107
  return CHORUS_OK;
}

int getifluxvectors_c(const double* Qi, double* Fi, double* Gi) {
  double gam;
  point_params(&gam, nullptr, nullptr);
  return getifluxvectors_gpu(1, gam, Qi, Fi, Gi);
}

int getvfluxvectors_c(const double* Qv, const double* nablaQ, double* Fv, double* Gv) {
  double gam, mu, eta0;
  point_params(&gam, &mu, &eta0);
  return getvfluxvectors_gpu(1, gam, mu, eta0, Qv, nablaQ, Fv, Gv);
}

int getvfluxvectors_av_c(ChorusCtx* ctx, const double* Qv, const double* nablaQ, double* Fv, double* Gv,
                         const int32_t* fam, const int32_t* ifp, const int32_t* jfp, const int32_t* ic) {
  return getvfluxvectors_av_gpu(ctx, 1, Qv, nablaQ, Fv, Gv, fam, ifp, jfp, ic);
}

// ---------------------------------------------------------------------------
// host-side setup
// ---------------------------------------------------------------------------
struct ChorusMesh {
  Mesh m;
};

int chorus_mesh_load(const char* dir, ChorusMesh** out) {
  if (!dir || !out) return set_err(CHORUS_EINVAL, "null argument");
  *out = nullptr;
  ChorusMesh* mh = new ChorusMesh();
  std::string err;
  int rc = mesh_load(dir, mh->m, err);
  if (rc) {
    delete mh;
    return set_err(rc, "%s", err.c_str());
  }
  *out = mh;
  return CHORUS_OK;
}

int chorus_mesh_load_gpu(const char* dir, int32_t device, ChorusMesh** out) {
  if (!dir || !out) return set_err(CHORUS_EINVAL, "null argument");
  *out = nullptr;
  ChorusMesh* mh = new ChorusMesh();
  std::string err;
  int rc = mesh_load_gpu(dir, device, mh->m, err);
  if (rc) {
    delete mh;
    return set_err(rc, "%s", err.c_str());
  }
  *out = mh;
  return CHORUS_OK;
}

int chorus_mesh_output_info(const ChorusMesh* mh, int32_t* nre, int32_t* nwrite) {
  if (!mh) return set_err(CHORUS_EINVAL, "null mesh");
  if (nre) *nre = mh->m.nre;
  if (nwrite) *nwrite = mh->m.nwrite;
  return CHORUS_OK;
}

int chorus_plot_create_mesh(ChorusCtx* ctx, const ChorusMesh* mh, int32_t NRE, ChorusPlot** plot) {
  if (!mh) return set_err(CHORUS_EINVAL, "null mesh");
  const Mesh& m = mh->m;
  if (!ctx || ctx->dims.NCELL != m.NCELL || ctx->dims.N != m.N)
    return set_err(CHORUS_EINVAL, "context and mesh differ");
  return chorus_plot_create(ctx, m.IVCELL.data(), m.IC2F.data(), m.XV.data(), m.YV.data(), m.NVERT, m.NFACE,
                            m.Xs.data(), NRE > 0 ? NRE : m.nre, plot);
}

int chorus_mesh_free(ChorusMesh* mh) {
  delete mh;
  return CHORUS_OK;
}

int chorus_mesh_info(const ChorusMesh* mh, ChorusDims* dims, ChorusParams* params, int32_t* maxiter, int32_t* problem) {
  if (!mh) return set_err(CHORUS_EINVAL, "null mesh");
  const Mesh& m = mh->m;
  if (dims) {
    dims->N = m.N;
    dims->NCELL = m.NCELL;
    dims->NFACE = m.NFACE;
    dims->NINTER = (int)m.IBFINTER.size();
    dims->NFREE = (int)m.IBFREE.size();
    dims->NPAIR = m.NPAIR;
  }
  if (params) *params = m.params;
  if (maxiter) *maxiter = m.maxiter;
  if (problem) *problem = m.problem;
  return CHORUS_OK;
}

const int32_t* chorus_mesh_iarray(const ChorusMesh* mh, const char* name, int64_t* count) {
  if (!mh || !name) return nullptr;
  const Mesh& m = mh->m;
  struct { const char* n; const std::vector<int32_t>* v; } t[] = {
      {"IF2C", &m.IF2C}, {"IC2F", &m.IC2F}, {"IF2V", &m.IF2V}, {"IVCELL", &m.IVCELL}, {"IBFINTER", &m.IBFINTER},
      {"IBFREE", &m.IBFREE}, {"IBFCYC", &m.IBFCYC}, {"IBFCYCLOC", &m.IBFCYCLOC}, {"CYC2FPAIR", &m.CYC2FPAIR},
      {"iface2fp", &m.iface2fp}, {"jface2fp", &m.jface2fp}};
  static const int32_t empty = 0;
  for (auto& x : t)
    if (!std::strcmp(name, x.n)) {
      if (count) *count = (int64_t)x.v->size();
      return x.v->empty() ? &empty : x.v->data();
    }
  if (count) *count = 0;
  return nullptr;
}

const double* chorus_mesh_darray(const ChorusMesh* mh, const char* name, int64_t* count) {
  if (!mh || !name) return nullptr;
  const Mesh& m = mh->m;
  struct { const char* n; const std::vector<double>* v; } t[] = {
      {"XV", &m.XV}, {"YV", &m.YV}, {"Xs", &m.Xs}, {"Xf", &m.Xf}, {"Lmat", &m.Lmat}, {"Mmat", &m.Mmat},
      {"S1", &m.S1}, {"S2", &m.S2}, {"Jac", &m.Jac}, {"XXsolu", &m.XXsolu}};
  static const double empty = 0.0;
  for (auto& x : t)
    if (!std::strcmp(name, x.n)) {
      if (count) *count = (int64_t)x.v->size();
      return x.v->empty() ? &empty : x.v->data();
    }
  if (count) *count = 0;
  return nullptr;
}

int64_t chorus_mesh_device_bytes(const ChorusMesh* mh) {
  if (!mh) return -1;
  const Mesh& m = mh->m;
  const int nface2 = (int)m.IBFINTER.size() + m.NPAIR, nface1 = (int)m.IBFREE.size();
  return (int64_t)arena_plan_bytes(m.N, m.NCELL, nface2, nface1, m.params.k_stage);
}

int chorus_mesh_host_chunks(const ChorusMesh* mh, int32_t chunks, int32_t* K, int32_t* cut, int32_t* f2cut,
                            int32_t* f1cut, int32_t* nseg, int32_t* seg) {
  if (!mh || !K || !cut || !f2cut || !f1cut || !nseg || !seg) return set_err(CHORUS_EINVAL, "null argument");
  if (chunks < 1 || chunks > kMaxHostChunks)
    return set_err(CHORUS_EINVAL, "chunks=%d outside 1..%d", (int)chunks, kMaxHostChunks);
  const Mesh& m = mh->m;
  const int NC = m.NCELL, NF = m.NFACE;
  // the keys the bound context computes from its face lists (chorus_gpu_bind)
  std::vector<int> f2max, f1cell, rel(NC);
  for (int ic = 0; ic < NC; ic++) rel[ic] = ic;
  auto two = [&](int cl, int cr) {
    f2max.push_back(std::max(cl, cr));
    rel[cl] = std::max(rel[cl], cr);
    rel[cr] = std::max(rel[cr], cl);
  };
  for (int32_t f1 : m.IBFINTER) two(m.IF2C[f1 - 1] - 1, m.IF2C[f1 - 1 + NF] - 1);
  for (int i = 0; i < m.NPAIR; i++) two(m.IF2C[m.CYC2FPAIR[i] - 1] - 1, m.IF2C[m.CYC2FPAIR[i + m.NPAIR] - 1] - 1);
  for (int32_t f1 : m.IBFREE) f1cell.push_back(m.IF2C[f1 - 1] - 1);
  std::sort(f2max.begin(), f2max.end());
  std::sort(f1cell.begin(), f1cell.end());
  HostChunks h;
  plan_host_chunks(NC, chunks, f2max, f1cell, rel, h);
  *K = h.K;
  for (int k = 0; k <= h.K; k++) {
    cut[k] = h.cut[k];
    f2cut[k] = h.f2[k];
    f1cut[k] = h.f1[k];
  }
  *nseg = h.nseg;
  for (int i = 0; i < h.nseg; i++) {
    seg[3 * i] = h.sb[i];
    seg[3 * i + 1] = h.se[i];
    seg[3 * i + 2] = h.sk[i];
  }
  return CHORUS_OK;
}

int chorus_gpu_bind_mesh(const ChorusMesh* mh, int32_t device, ChorusCtx** ctx) {
  if (!mh) return set_err(CHORUS_EINVAL, "null mesh");
  const Mesh& m = mh->m;
  ChorusDims d;
  chorus_mesh_info(mh, &d, nullptr, nullptr, nullptr);
  return chorus_gpu_bind(&d, m.IF2C.data(), m.IBFINTER.data(), m.IBFREE.data(), m.CYC2FPAIR.data(), m.iface2fp.data(),
                         m.jface2fp.data(), m.Xs.data(), m.Xf.data(), m.Lmat.data(), m.Mmat.data(), m.S1.data(),
                         m.S2.data(), m.Jac.data(), &m.params, device, ctx);
}

int chorus_initial_state(const ChorusMesh* mh, ChorusCtx* c, double* Qout) {
  if (!mh || !c) return set_err(CHORUS_EINVAL, "null argument");
  const Mesh& m = mh->m;
  const int N = m.N, NC = m.NCELL;
  if (c->dims.N != N || c->dims.NCELL != NC) return set_err(CHORUS_EINVAL, "mesh and context differ");
  const size_t np = (size_t)NC * N * N;
  std::vector<double> Q(np * 9);
  for (size_t p = 0; p < np; p++) initial_point(m.problem, m.params.gam, m.XXsolu[2 * p], m.XXsolu[2 * p + 1], nullptr, &Q[9 * p]);
  int rc = chorus_gpu_upload_state(c, Q.data());
  if (!rc) rc = correct_b_via_curl_az_gpu(c);
  if (!rc) rc = chorus_gpu_download_state(c, Q.data());
  if (rc) return rc;
  for (size_t p = 0; p < np; p++) {
    double B[3] = {Q[9 * p + 5], Q[9 * p + 6], Q[9 * p + 7]};
    initial_point(m.problem, m.params.gam, m.XXsolu[2 * p], m.XXsolu[2 * p + 1], B, &Q[9 * p]);
  }
  rc = chorus_gpu_upload_state(c, Q.data());
  if (rc) return rc;
  if (Qout) std::memcpy(Qout, Q.data(), Q.size() * sizeof(double));
  return CHORUS_OK;
}

int chorus_write_restart(ChorusCtx* c, const char* path, int32_t iter, double ctime) {
  if (!c || !path) return set_err(CHORUS_EINVAL, "null argument");
  const int N = c->dims.N, NC = c->dims.NCELL, nq = 9 * N * N;
  std::vector<double> Q((size_t)NC * nq);
  int rc = chorus_gpu_download_state(c, Q.data());
  if (rc) return rc;
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_err(CHORUS_EIO, "cannot open %s", path);
  bool ok = std::fwrite(&iter, 4, 1, f) == 1 && std::fwrite(&ctime, 8, 1, f) == 1;
  for (int e = 0; e < NC && ok; e++) {
    int32_t g = e + 1;
    ok = std::fwrite(&g, 4, 1, f) == 1 && std::fwrite(&Q[(size_t)e * nq], 8, nq, f) == (size_t)nq;
  }
  std::fclose(f);
  return ok ? CHORUS_OK : set_err(CHORUS_EIO, "short write to %s", path);
}

int chorus_read_restart(ChorusCtx* c, const char* path, int32_t* iter, double* ctime) {
  if (!c || !path) return set_err(CHORUS_EINVAL, "null argument");
  const int N = c->dims.N, NC = c->dims.NCELL, nq = 9 * N * N;
  // a cell the stream does not name keeps its current state, as in READ_ALL_DATA_BINARY
  // (read_data_restart.f90:55-56 assigns only the cells it reads)
  std::vector<double> Q((size_t)NC * nq, 0.0);
  int rc0 = chorus_gpu_download_state(c, Q.data());
  if (rc0) return rc0;
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_err(CHORUS_EIO, "cannot open %s", path);
  int32_t it = 0;
  double t = 0;
  bool ok = std::fread(&it, 4, 1, f) == 1 && std::fread(&t, 8, 1, f) == 1;
  for (int e = 0; e < NC && ok; e++) {
    int32_t g = 0;
    ok = std::fread(&g, 4, 1, f) == 1 && g >= 1 && g <= NC;
    if (ok) ok = std::fread(&Q[(size_t)(g - 1) * nq], 8, nq, f) == (size_t)nq;
  }
  std::fclose(f);
  if (!ok) return set_err(CHORUS_EIO, "bad restart file %s", path);
  if (iter) *iter = it;
  if (ctime) *ctime = t;
  return chorus_gpu_upload_state(c, Q.data());
}

}  // extern "C"
