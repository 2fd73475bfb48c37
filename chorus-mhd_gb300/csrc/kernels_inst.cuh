// kernels_inst.cuh -- explicit instantiation of the stage kernels for N = CHORUS_N.
// Each translation unit holds its own constant-memory copy of the N-point operators.
#include "kernels.cuh"

#ifndef CHORUS_N
#error "define CHORUS_N before including kernels_inst.cuh"
#endif
#define CHORUS_CAT2(a, b) a##b
#define CHORUS_CAT(a, b) CHORUS_CAT2(a, b)

namespace chorus {

namespace {
constexpr int kN = CHORUS_N;
inline size_t smem_e1(int epb) {
  return sizeof(double) * ((size_t)epb * (D<kN>::NS * 9 + 2 * D<kN>::NS + D<kN>::NFP * 9) + kN * kN);
}
inline size_t smem_e2(int epb) {
  return sizeof(double) * ((size_t)epb * (D<kN>::NFP * 16 + D<kN>::NS * 17));
}
inline size_t smem_e3(int epb) {
  return sizeof(double) * ((size_t)epb * (D<kN>::NFP * 8 + D<kN>::NS * (1 + 9 + 1 + 2) + D<kN>::NFP * 2));
}
inline size_t smem_ct(int epb) { return sizeof(double) * epb * (D<kN>::NFP * 2 + D<kN>::NS * 2); }
inline int grid_cells(int nc, int epb) { return (nc + epb - 1) / epb; }

// threads per CTA of a face-point pass: 256, or 64 when that leaves fewer than about
// eight CTAs per SM (small meshes), so that the points spread over every SM
inline int face_threads(int n) { return n >= 152 * 8 * 256 ? 256 : 64; }

void set_smem_limits() {
  static bool done[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && done[dev]) return;
  const int lim = 200 * 1024;
  cudaFuncSetAttribute(k_e1<kN>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(k_e2<kN>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(k_e3<kN>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(k_ct_elem<kN>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(k_diag_interp<kN>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(k_nqsp<kN>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  if (dev < 64) done[dev] = true;
}
}  // namespace

void CHORUS_CAT(upload_ops_n, CHORUS_N)(const OpsN& o) {
  set_smem_limits();
  cudaMemcpyToSymbol(c_ops, &o, sizeof(OpsN));
}

template <>
void launch_e1<kN>(const SolveDev& s, const Launch& L, cudaStream_t st, int plot, int c0, int c1) {
  const int sensor = (s.artiv ? (plot ? 3 : 1) : 0) | 4;  // 4: also reset the stage's wave speed
  if (c1 < 0) c1 = s.NC;
  if (c1 > c0) launch_pdl(k_e1<kN>, grid_cells(c1 - c0, L.epb), L.threads, smem_e1(L.epb), st, s, L.epb, sensor, c0, c1);
}
void CHORUS_CAT(launch_e1_nosensor_n, CHORUS_N)(const SolveDev& s, const Launch& L, cudaStream_t st) {
  launch_pdl(k_e1<kN>, grid_cells(s.NC, L.epb), L.threads, smem_e1(L.epb), st, s, L.epb, 0, 0, s.NC);
}
template <>
void launch_f1<kN>(const SolveDev& s, cudaStream_t st, int a2, int b2, int a1, int b1) {
  if (b2 < 0) b2 = s.nface2;
  if (b1 < 0) b1 = s.nface1;
  const int n2 = (b2 - a2) * kN, n = n2 + (b1 - a1) * kN;
  if (n > 0)
    launch_pdl(k_f1<kN>, (n + face_threads(n) - 1) / face_threads(n), face_threads(n), 0, st, s, a2 * kN, n2,
               (s.nface2 + a1) * kN, n);
}
template <>
void launch_e2<kN>(const SolveDev& s, const Launch& L, cudaStream_t st) {
  // chunks of up to one cell per thread, but small enough for about 16 CTAs per SM
  static int nsm_of[64];  // SM count per device, looked up once
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64) {
    if (!nsm_of[dev] && (cudaDeviceGetAttribute(&nsm_of[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
                         nsm_of[dev] <= 0))
      nsm_of[dev] = 152;
    nsm = nsm_of[dev];
  }
  int chunk = s.NC / (16 * nsm);
  chunk = chunk < L.epb ? L.epb : (chunk > L.threads ? L.threads : chunk);
  chunk -= chunk % L.epb;
  if (!s.skip) chunk = L.epb;  // every cell needs its gradients: one group per CTA
  launch_pdl(k_e2<kN>, grid_cells(s.NC, chunk), L.threads, smem_e2(L.epb), st, s, L.epb, chunk);
}
template <>
void launch_f2<kN>(const SolveDev& s, cudaStream_t st) {
  const int n = (s.nface2 + s.nface1) * kN;
  if (n > 0) k_f2<kN><<<(n + face_threads(n) - 1) / face_threads(n), face_threads(n), 0, st>>>(s);
}
template <>
void launch_e3<kN>(const SolveDev& s, const RKStage& rk, const Launch& L, cudaStream_t st, int c0, int c1) {
  const int update = (rk.cQ != 0.0 || rk.cR != 0.0 || rk.nsrc > 0) ? 1 : 0;
  if (c1 < 0) c1 = s.NC;
  if (c1 > c0)
    launch_pdl(k_e3<kN>, grid_cells(c1 - c0, L.epb), L.threads, smem_e3(L.epb), st, s, rk, L.epb, update, c0, c1);
}
template <>
void launch_ct<kN>(const SolveDev& s, const Launch& L, cudaStream_t st, int mode, int c0, int c1) {
  if (mode == 1) {
    if (c1 < 0) c1 = s.nface2;
    const int n = (c1 - c0) * kN;
    if (n > 0)
      launch_pdl(k_ct_face<kN>, (n + face_threads(n) - 1) / face_threads(n), face_threads(n), 0, st, s, c0, c1);
  } else {
    if (c1 < 0) c1 = s.NC;
    if (c1 > c0)
      launch_pdl(k_ct_elem<kN>, grid_cells(c1 - c0, L.epb), L.threads, smem_ct(L.epb), st, s, L.epb, mode, c0, c1);
  }
}
template <>
void launch_diag<kN>(const SolveDev& s, const Launch& L, cudaStream_t st, int mode) {
  if (mode == 0) {
    k_diag_interp<kN><<<grid_cells(s.NC, L.epb), L.threads, sizeof(double) * L.epb * D<kN>::NS * 2, st>>>(s, L.epb);
  } else {
    const int n = s.nface2 * kN;
    if (n > 0) k_diag_face<kN><<<(n + face_threads(n) - 1) / face_threads(n), face_threads(n), 0, st>>>(s);
  }
}
template <>
void launch_nqsp<kN>(const SolveDev& s, int v0, int v1, cudaStream_t st) {
  // 4 cells per 128 threads; 12 kB of shared memory per cell for all nine variables
  const int epb = 4, nq = 2 * (v1 - v0 + 1);
  const size_t smem = sizeof(double) * epb * (size_t)(D<kN>::NFP + D<kN>::NS) * nq;
  k_nqsp<kN><<<grid_cells(s.NC, epb), 128, smem, st>>>(s, epb, v0, v1);
}
template <>
void launch_divb<kN>(const SolveDev& s, cudaStream_t st) {
  k_divb<kN><<<(s.NC + 255) / 256, 256, 0, st>>>(s);
}

}  // namespace chorus
