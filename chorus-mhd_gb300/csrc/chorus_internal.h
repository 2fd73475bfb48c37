// chorus_internal.h -- types shared by the host runtime and the CUDA kernels.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>
#include <vector>

#include "../../include/chorus_gpu.h"

namespace chorus {

constexpr int kMaxN = 8;   // kernels are instantiated for N = 2..kMaxN
constexpr int kMinN = 2;

// ---------------------------------------------------------------------------
// Host-side mesh (what the reference's setup chain leaves in module setup2d)
// ---------------------------------------------------------------------------
struct Mesh {
  int N = 0, NCELL = 0, NVERT = 0, NFACE = 0, NPAIR = 0;
  int maxiter = 0, problem = 0, restart = 0;
  int nre = 1, nwrite = 0;  // plot sub-intervals per cell edge, output interval
  ChorusParams params{};
  std::vector<int32_t> IVCELL, IC2F, IF2C, IF2V, IBFINTER, IBFREE, IBFCYC, IBFCYCLOC, CYC2FPAIR;
  std::vector<int32_t> iface2fp, jface2fp;
  std::vector<double> XV, YV, Xs, Xf, Lmat, Mmat, S1, S2, Jac, XXsolu;
};

int mesh_load(const std::string& dir, Mesh& m, std::string& err);
// the same with the map building and the geometry on a GPU (meshgpu.cu): bit-identical
// results; a mesh the device path finds invalid is rebuilt on the host for the error
int mesh_load_gpu(const std::string& dir, int device, Mesh& m, std::string& err);

// stages of the setup chain shared by both paths (mesh.cpp)
struct BndRecord {      // one record of the .BND file whose vertices are on this partition
  int line;             // 1-based record number
  int a, b;             // local vertex ids of the edge
  int kind;             // 1 CYCL, 2 FREE, 0 anything else (rejected when its face is found)
  std::string type;
};
int mesh_parse(const std::string& dir, Mesh& m, std::vector<BndRecord>& bnd, std::string& err);
int mesh_maps_host(Mesh& m, const std::vector<BndRecord>& bnd, std::string& err);
int boundary_face(Mesh& m, const BndRecord& r, int K, std::vector<char>& bflag, std::string& err);
int mesh_periodic(Mesh& m, std::string& err);
void mesh_operators(Mesh& m);
void mesh_geometry_host(Mesh& m);
void setsandpoints(int np, double* xs, double* xf);
double lagrange(const double* x, int n, int i, double xv);
void compute_L_M(int N, const double* Xs, const double* Xf, double* L, double* M);
void initial_point(int problem, double gam, double x, double y, const double* B, double* q);

// ---------------------------------------------------------------------------
// Device-side view of one solve.  Element-blocked layouts (e = cell, 0-based):
//   Q, Qk0..   [e][js][is][9]              (the reference's Q(9,N,N,NC))
//   resid      [e][js][is][9]
//   Qvf        [e][fp][9]    fp = family-1 points (jfp*(N+1)+ifp), then family-2
//                            points ((N+1)N + jfp*N+ifp): one block per cell
//   Fc         [e][fp][8]    inviscid contravariant flux (F1 / G2)
//   Azf        [e][fp]       A_z at the flux points (upwinded on faces after a stage,
//                            face-averaged after the CT projection)
//   nQs        [e][js][is][2][9]   (variable 9 is not stored here: see nQs9)
//   nQs9       [e][js][is][2]      grad A_z of the CT projection / nablaQsp(9,9)
//   nQvf       [e][fp][2][9]
//   nAs        [e][js][is][2]
//   met        [e][fp][2]    (S1(1,1),S1(1,2)) on family 1, (S2(2,1),S2(2,2)) on 2
//   invJ       [e][js][is]
//   Se         [e]           AV sensor sum of variable 1 (the reference's SM_IND(1) is log10 of it)
//   muf        [e][4]        face-averaged AV viscosity per local face 1..4
// ---------------------------------------------------------------------------
struct FaceNorm {  // per face point: unit normal, magnorm*sign_l/2, sign_l*sign_r (+-1)
  double ux, uy, msl, ss;
};

struct SolveDev {
  int N, NC;
  int nface2, nface1;           // two-sided faces (interior + periodic), FREE faces
  int artiv;
  int pad0;
  double gam, mu, eta0, B0x, B0y, hmsh;
  double* Q;
  double* Qk0;
  double* Qka;
  double* Qr2;                  // extra registers for FiveStageRk (qj2, qj3, resid0)
  double* Qr3;
  double* R0;
  double* resid;
  double* Qvf;
  double* Fc;
  double* Azf;
  double* nQs;
  double* nQvf;
  double* nAs;
  const double* met;
  const double* invJ;
  double* Se;
  double* Se6;                  // the same sum for variable 6 (last stage, when plot_flag is set)
  double* muf;
  const int4* face2;            // (cL, lfL, cR, lfR): cells 0-based, local faces 1..4
  const FaceNorm* fn2;          // [face][nfp]
  const int2* face1;            // (c, lf)
  const FaceNorm* fn1;          // [face][nfp] (ss unused)
  // AV activity (used only when skip != 0, i.e. mu == 0 and eta0 == 0): act[e] = the
  // cell's sensor is not below se_low; nv[e] = the cell or a face neighbour is active
  // (the cell's viscous flux can be nonzero); nbr[e] = face neighbours (-1: none)
  int skip;
  int pad1;
  int* act;
  int* nv;
  const int4* nbr;
  const int4* nbrlf;            // the neighbour's local face (1..4) across each face, 0 at FREE faces
  unsigned long long* eig;      // bit pattern of the stage's max wave speed (>= 0)
  unsigned int* err;            // error flags (bit 0: non-finite wave speed)
  double* diag;                 // per-cell diagnostic partial sums [e][2]
  const int* plot_flag;         // nonzero: the last stage records Se6 (read by E1 at run time)
  double* nQs9;                 // [e][sp][2] grad A_z of variable 9 (nablaQs(9,:,...)), kept apart from nQs
  void* pad3;                   // keeps the size a multiple of 16 bytes
};

// One RK stage update: Qnew = sum_j c[j]*src[j] + cQ*Q + cR*R (+ cR0*R0), with
// optional copies of the old state, the new state and the residual.
struct RKStage {
  const double* src[3];
  double c[3];
  int nsrc;
  int pad;
  double cQ, cR, cR0;
  const double* R0;
  double* save_old;
  double* save_new;
  double* save_R;
  int write_resid;  // also store the residual in SolveDev::resid
  int diag;         // accumulate sum(resid^2) per cell into diag[e][0]
};

// the five stage records of RK_S5P3 / FiveStageRk for one solve (capi.cu)
void rk_stage_records(const SolveDev& s, double dt, int k_stage, bool diag, RKStage* r);

// launch helpers implemented in kernels_*.cu (one translation unit per N)
struct Launch {
  int epb;    // cells per CTA in element kernels
  int threads;
};

// plot != 0: also record the variable-6 sensor (Se6) when AV is on
// cells [c0, c1) (c1 < 0: to the end)
template <int N> void launch_e1(const SolveDev& s, const Launch& L, cudaStream_t st, int plot, int c0 = 0, int c1 = -1);
// two-sided faces [a2, b2) and FREE faces [a1, b1) (b < 0: to the end of the list)
template <int N> void launch_f1(const SolveDev& s, cudaStream_t st, int a2 = 0, int b2 = -1, int a1 = 0, int b1 = -1);
template <int N> void launch_e2(const SolveDev& s, const Launch& L, cudaStream_t st);
template <int N> void launch_f2(const SolveDev& s, cudaStream_t st);
template <int N> void launch_e3(const SolveDev& s, const RKStage& rk, const Launch& L, cudaStream_t st, int c0 = 0,
                                int c1 = -1);
// modes 0 and 2: cells [c0, c1); mode 1 (the face average): two-sided faces [c0, c1)
template <int N> void launch_ct(const SolveDev& s, const Launch& L, cudaStream_t st, int mode, int c0 = 0, int c1 = -1);
// the diagnostic's B_x, B_y traces: mode 0 interpolation, mode 1 face average
template <int N> void launch_diag(const SolveDev& s, const Launch& L, cudaStream_t st, int mode);
template <int N> void launch_nqsp(const SolveDev& s, int v0, int v1, cudaStream_t st);
template <int N> void launch_divb(const SolveDev& s, cudaStream_t st);

void upload_operators(int N, const double* Lmat, const double* Mmat, const double* Xs, const double* Xf,
                      const double* Aav);
void launch_point_rusanov(int n, double gam, const double* Qfl, const double* Qfr, double* Fnl, double* Fnr,
                          double* Az, const double* normf, const int* sl, const int* sr, double* ev,
                          cudaStream_t st);
void launch_point_iflux(int n, double gam, const double* Qi, double* Fi, double* Gi, cudaStream_t st);
void launch_point_vflux(int n, double gam, double mu, double eta0, const double* Qv, const double* nQ, double* Fv,
                        double* Gv, cudaStream_t st);
struct PointAxes {  // flux-point coordinates Xf(1..N+1) of a bound solve, by value
  double Xf[kMaxN + 1];
};
void launch_point_vflux_av(int n, double gam, const PointAxes& ax, const double* muf, const int* fam, const int* ifp,
                           const int* jfp, const int* ic, const double* Qv, const double* nQ, double* Fv, double* Gv,
                           cudaStream_t st);
void launch_reduce_diag(const double* diag, int NC, double* out2, cudaStream_t st);
void launch_qvf9(const SolveDev& s, cudaStream_t st);  // Qvf variable 9 from Azf (point.cu)

}  // namespace chorus
