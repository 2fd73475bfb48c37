// meshgpu.cu -- the setup chain's map building and geometry on the GPU.
//
// The host setup (mesh.cpp) takes about a second for a 512x512 mesh, most of it in
// CONNECTIVITY and the metrics; a serving process admitting large meshes pays that per
// request.  Here the text files are still parsed on the host (with GLOB2LOCAL), and the
// rest runs as kernels:
//   * CHECK_MESH (connectivity.f90:236-283): the corner cross products per cell;
//   * CONNECTIVITY (connectivity.f90:1-233): every (cell, local face) inserts its edge
//     into an open-addressing hash table (keys claimed with atomicCAS); an edge's two
//     sides are partners.  The reference numbers a face when the first of its two sides
//     is visited in cell-major, local-face order, so a face belongs to the smaller of its
//     two (4*cell + face) codes and its number is the count of owned codes before it: an
//     exclusive scan of the ownership flags;
//   * CONNECT_BDRY (connect_bdry.f90:1-354): each boundary record's edge is looked up in
//     the same table; the host walks the records in file order (the lists and the error
//     order of the reference), and IBFINTER is a scan-compaction of the two-sided faces;
//   * mapder + calcjacob (mapder.f90:1-76, calcjacob.f90:1-86) and xyCoor_atGps
//     (mapder.f90:255-273): one thread per point, every product and sum rounded
//     separately (__dmul_rn / __dadd_rn), the host's order of operations, so the metrics
//     are bit-identical to the host path compiled with -ffp-contract=off.
// MAPCYCLOC stays on the host (its faces are the domain's perimeter).  A mesh the device
// path finds invalid (a cell turned the wrong way, a non-manifold edge, a face pair that
// does not run opposite ways, a full table) is rebuilt by the host path, which reports
// the reference's error for it.  Temporary device memory is allocated and freed here.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "chorus_internal.h"

namespace chorus {

int set_err(int code, const char* fmt, ...);

namespace {

constexpr unsigned long long kEmptyKey = ~0ull;
constexpr int kScanBlock = 1024;
enum { kErrCheck = 1, kErrTable = 2, kErrManifold = 4, kErrOrient = 8 };

__constant__ int c_ivface[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};  // connectivity.f90:73-83

__device__ __forceinline__ unsigned long long edge_key(int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return ((unsigned long long)(unsigned)lo << 32) | (unsigned)hi;
}

__device__ __forceinline__ unsigned slot_hash(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return (unsigned)k;
}

// CHECK_MESH: cross products of consecutive corner edges (connectivity.f90:249-272)
__global__ void k_check_cells(int NC, const int* __restrict__ iv, const double* __restrict__ XV,
                              const double* __restrict__ YV, unsigned* err) {
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic >= NC) return;
  double x[4], y[4];
  for (int k = 0; k < 4; k++) {
    const int v = iv[ic + (size_t)NC * k] - 1;
    x[k] = XV[v];
    y[k] = YV[v];
  }
  const double v12x = __dsub_rn(x[1], x[0]), v12y = __dsub_rn(y[1], y[0]);
  const double v23x = __dsub_rn(x[2], x[1]), v23y = __dsub_rn(y[2], y[1]);
  const double v34x = __dsub_rn(x[3], x[2]), v34y = __dsub_rn(y[3], y[2]);
  const double c123 = __dsub_rn(__dmul_rn(v12x, v23y), __dmul_rn(v12y, v23x));
  const double c234 = __dsub_rn(__dmul_rn(v23x, v34y), __dmul_rn(v23y, v34x));
  if (__dmul_rn(c123, c234) < 0 || c123 < 0) atomicOr(err, (unsigned)kErrCheck);
}

// probe for key; returns its slot, or -1 when an empty slot ends the search
__device__ __forceinline__ int find_slot(const unsigned long long* keys, unsigned mask, unsigned long long key) {
  unsigned h = slot_hash(key) & mask;
  for (unsigned probe = 0; probe <= mask; probe++) {
    const unsigned long long k = keys[h];
    if (k == key) return (int)h;
    if (k == kEmptyKey) return -1;
    h = (h + 1) & mask;
  }
  return -1;
}

// every (cell, local face) code = 4*ic + f inserts its edge; the first two codes of an
// edge are kept (a third makes the edge non-manifold)
__global__ void k_edge_insert(int NC, const int* __restrict__ iv, unsigned long long* keys, int* cnt, int* side0,
                              int* side1, int* slot_of, unsigned mask, unsigned* err) {
  const int code = blockIdx.x * blockDim.x + threadIdx.x;
  if (code >= 4 * NC) return;
  const int ic = code >> 2, f = code & 3;
  const unsigned long long key =
      edge_key(iv[ic + (size_t)NC * c_ivface[f][0]], iv[ic + (size_t)NC * c_ivface[f][1]]);
  unsigned h = slot_hash(key) & mask;
  bool placed = false;
  for (unsigned probe = 0; probe <= mask; probe++) {
    const unsigned long long prev = atomicCAS(keys + h, kEmptyKey, key);
    if (prev == kEmptyKey || prev == key) {
      placed = true;
      break;
    }
    h = (h + 1) & mask;
  }
  if (!placed) {
    atomicOr(err, (unsigned)kErrTable);
    slot_of[code] = -1;
    return;
  }
  const int c = atomicAdd(cnt + h, 1);
  if (c == 0) side0[h] = code;
  else if (c == 1) side1[h] = code;
  else atomicOr(err, (unsigned)kErrManifold);
  slot_of[code] = (int)h;
}

// the other side of each code's edge (-1 on a boundary) and whether the code owns the face
__global__ void k_partner(int n4, const int* __restrict__ slot_of, const int* __restrict__ cnt,
                          const int* __restrict__ side0, const int* __restrict__ side1, int* other, int* owned) {
  const int code = blockIdx.x * blockDim.x + threadIdx.x;
  if (code >= n4) return;
  const int h = slot_of[code];
  int o = -1;
  if (h >= 0 && cnt[h] >= 2) o = side0[h] == code ? side1[h] : side0[h];
  other[code] = o;
  owned[code] = (o < 0 || code < o) ? 1 : 0;
}

// exclusive scan, stage 1: each block scans kScanBlock entries and leaves its total
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(int n, const int* __restrict__ in, int* out, int* sums) {
  __shared__ int warp_tot[kScanBlock / 32];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int v = i < n ? in[i] : 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;  // inclusive over warps
  }
  __syncthreads();
  const int before = w ? warp_tot[w - 1] : 0;
  if (i < n) out[i] = before + x - v;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = warp_tot[kScanBlock / 32 - 1];
}

// stage 2: one block turns the block totals into exclusive offsets, kScanBlock at a time
__global__ void __launch_bounds__(kScanBlock) k_scan_sums(int nb, int* sums) {
  __shared__ int warp_tot[kScanBlock / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int base = 0; base < nb; base += kScanBlock) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? sums[i] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_tot[lane] = t;
    }
    __syncthreads();
    const int before = (w ? warp_tot[w - 1] : 0) + carry;
    if (i < nb) sums[i] = before + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_tot[kScanBlock / 32 - 1];
    __syncthreads();
  }
}

// stage 3: add each block's offset
__global__ void k_scan_add(int n, int* out, const int* __restrict__ sums) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

// the face tables from the owned codes: IC2F(NC,4), IF2C(NF,4), IF2V(NF,2); a face's
// second side must run the other way round (both cells counter-clockwise)
__global__ void k_faces(int NC, int NF, const int* __restrict__ iv, const int* __restrict__ other,
                        const int* __restrict__ owned, const int* __restrict__ pos, int* IC2F, int* IF2C, int* IF2V,
                        unsigned* err) {
  const int code = blockIdx.x * blockDim.x + threadIdx.x;
  if (code >= 4 * NC || !owned[code]) return;
  const int ic = code >> 2, f = code & 3, id = pos[code] + 1;
  const int va = iv[ic + (size_t)NC * c_ivface[f][0]], vb = iv[ic + (size_t)NC * c_ivface[f][1]];
  const int o = other[code];
  IC2F[ic + (size_t)NC * f] = id;
  IF2C[id - 1] = ic + 1;
  IF2C[id - 1 + (size_t)2 * NF] = f + 1;
  IF2V[id - 1] = va;
  IF2V[id - 1 + (size_t)NF] = vb;
  if (o >= 0) {
    const int oc = o >> 2, of = o & 3;
    IC2F[oc + (size_t)NC * of] = id;
    IF2C[id - 1 + (size_t)NF] = oc + 1;
    IF2C[id - 1 + (size_t)3 * NF] = of + 1;
    if (iv[oc + (size_t)NC * c_ivface[of][0]] != vb || iv[oc + (size_t)NC * c_ivface[of][1]] != va)
      atomicOr(err, (unsigned)kErrOrient);
  } else {
    IF2C[id - 1 + (size_t)NF] = 0;
    IF2C[id - 1 + (size_t)3 * NF] = 0;
  }
}

// boundary records: the face of each edge (st 0), an edge that is no cell face (st 1) or
// an interior face (st 2)
__global__ void k_bnd_lookup(int nb, const int2* __restrict__ ab, const unsigned long long* __restrict__ keys,
                             const int* __restrict__ cnt, const int* __restrict__ side0, unsigned mask,
                             const int* __restrict__ IC2F, int NC, int* K, int* st) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb) return;
  const int h = find_slot(keys, mask, edge_key(ab[r].x, ab[r].y));
  if (h < 0) { st[r] = 1; K[r] = 0; return; }
  if (cnt[h] >= 2) { st[r] = 2; K[r] = 0; return; }
  const int code = side0[h];
  st[r] = 0;
  K[r] = IC2F[(code >> 2) + (size_t)NC * (code & 3)];
}

// two-sided faces (IBFINTER's flags) and the first one-sided face no record names
__global__ void k_inter_flags(int NF, const int* __restrict__ IF2C, const unsigned char* __restrict__ bflag,
                              int* flags, int* missing) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= NF) return;
  const int two = IF2C[f + (size_t)NF] != 0;
  flags[f] = two;
  if (!two && !bflag[f]) atomicMin(missing, f + 1);
}

__global__ void k_compact(int NF, const int* __restrict__ flags, const int* __restrict__ pos, int* out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < NF && flags[f]) out[pos[f]] = f + 1;
}

struct Axes {
  double Xs[kMaxN];
  double Xf[kMaxN + 1];
};

// x_psi, y_psi, x_eta, y_eta of the bilinear map at (psi, eta) (mapder.f90:1-76), in the
// host's order: a sum over the four corners, each product rounded
__device__ __forceinline__ void bilinear_metrics(const double* x, const double* y, double psi, double eta,
                                                 double& xpsi, double& ypsi, double& xeta, double& yeta) {
  const double dm[4][2] = {{__dsub_rn(eta, 1.0), __dsub_rn(psi, 1.0)},
                           {__dsub_rn(1.0, eta), -psi},
                           {eta, psi},
                           {-eta, __dsub_rn(1.0, psi)}};
  xpsi = 0.0;
  xeta = 0.0;
  ypsi = 0.0;
  yeta = 0.0;
  for (int k = 0; k < 4; k++) {
    xpsi = __dadd_rn(xpsi, __dmul_rn(dm[k][0], x[k]));
    ypsi = __dadd_rn(ypsi, __dmul_rn(dm[k][0], y[k]));
    xeta = __dadd_rn(xeta, __dmul_rn(dm[k][1], x[k]));
    yeta = __dadd_rn(yeta, __dmul_rn(dm[k][1], y[k]));
  }
}

// one thread per point of a cell: N^2 solution points (Jac, XXsolu), then the (N+1)N
// family-1 and N(N+1) family-2 flux points (S1, S2)
__global__ void k_geometry(int NC, int N, Axes ax, const int* __restrict__ iv, const double* __restrict__ XV,
                           const double* __restrict__ YV, double* Jac, double* S1, double* S2, double* XX) {
  const int per = N * N + 2 * N * (N + 1);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)NC * per) return;
  const int ic = (int)(t / per), p = (int)(t - (long long)ic * per);
  double x[4], y[4];
  for (int k = 0; k < 4; k++) {
    const int v = iv[ic + (size_t)NC * k] - 1;
    x[k] = XV[v];
    y[k] = YV[v];
  }
  double xpsi, ypsi, xeta, yeta;
  if (p < N * N) {
    const int is = p % N, js = p / N;
    bilinear_metrics(x, y, ax.Xs[is], ax.Xs[js], xpsi, ypsi, xeta, yeta);
    const size_t g = is + (size_t)N * (js + (size_t)N * ic);
    Jac[g] = __dsub_rn(__dmul_rn(xpsi, yeta), __dmul_rn(xeta, ypsi));
    // xyCoor_atGps: the bilinear shape functions at the solution point
    const double xi = ax.Xs[is], et = ax.Xs[js];
    const double fsh[4] = {__dmul_rn(__dsub_rn(1.0, xi), __dsub_rn(1.0, et)), __dmul_rn(__dsub_rn(1.0, et), xi),
                           __dmul_rn(xi, et), __dmul_rn(__dsub_rn(1.0, xi), et)};
    double ax_ = 0.0, ay_ = 0.0;
    for (int nb = 0; nb < 4; nb++) {
      ax_ = __dadd_rn(ax_, __dmul_rn(x[nb], fsh[nb]));
      ay_ = __dadd_rn(ay_, __dmul_rn(y[nb], fsh[nb]));
    }
    XX[2 * g] = ax_;
    XX[2 * g + 1] = ay_;
  } else if (p < N * N + N * (N + 1)) {
    const int q = p - N * N, ifp = q % (N + 1), jfp = q / (N + 1);
    bilinear_metrics(x, y, ax.Xf[ifp], ax.Xs[jfp], xpsi, ypsi, xeta, yeta);
    double* b = S1 + 4 * (ifp + (size_t)(N + 1) * (jfp + (size_t)N * ic));
    b[0] = yeta;
    b[2] = -xeta;
    b[1] = -ypsi;
    b[3] = xpsi;
  } else {
    const int q = p - N * N - N * (N + 1), ifp = q % N, jfp = q / N;
    bilinear_metrics(x, y, ax.Xs[ifp], ax.Xf[jfp], xpsi, ypsi, xeta, yeta);
    double* b = S2 + 4 * (ifp + (size_t)N * (jfp + (size_t)(N + 1) * ic));
    b[0] = yeta;
    b[2] = -xeta;
    b[1] = -ypsi;
    b[3] = xpsi;
  }
}

// device buffers of one setup, freed on destruction
struct Scratch {
  std::vector<void*> ptrs;
  cudaError_t e = cudaSuccess;
  template <class T>
  T* alloc(size_t n) {
    void* p = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&p, n * sizeof(T) + 16);
    if (e == cudaSuccess) ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
};

// exclusive scan of n ints in place of out (out may not alias in); returns the total
int scan_exclusive(int n, const int* in, int* out, int* sums, cudaStream_t st, cudaError_t& e) {
  if (n <= 0 || e != cudaSuccess) return 0;
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  k_scan_blocks<<<nb, kScanBlock, 0, st>>>(n, in, out, sums);
  k_scan_sums<<<1, kScanBlock, 0, st>>>(nb, sums);
  k_scan_add<<<nb, kScanBlock, 0, st>>>(n, out, sums);
  int last_out = 0, last_in = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&last_out, out + n - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&last_in, in + n - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return last_out + last_in;
}

inline unsigned grid_of(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// maps and geometry of a parsed mesh on the device; 0 = done, 1 = the mesh needs the
// host path (invalid somewhere), <0 = CUDA failure
int build_on_device(Mesh& m, const std::vector<BndRecord>& bnd, std::string& err, int& rc_out) {
  rc_out = CHORUS_OK;
  const int NC = m.NCELL, N = m.N, n4 = 4 * NC;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return -1;
  Scratch s;
  unsigned tsize = 1;
  while (tsize < (unsigned)(2 * n4)) tsize <<= 1;  // at most about a quarter full (one key per edge)
  const unsigned mask = tsize - 1;
  int* d_iv = s.alloc<int>(n4);
  double* d_x = s.alloc<double>(m.NVERT);
  double* d_y = s.alloc<double>(m.NVERT);
  unsigned long long* d_keys = s.alloc<unsigned long long>(tsize);
  int* d_cnt = s.alloc<int>(tsize);
  int* d_s0 = s.alloc<int>(tsize);
  int* d_s1 = s.alloc<int>(tsize);
  int* d_slot = s.alloc<int>(n4);
  int* d_other = s.alloc<int>(n4);
  int* d_owned = s.alloc<int>(n4);
  int* d_pos = s.alloc<int>(n4);
  int* d_sums = s.alloc<int>(n4 / kScanBlock + 2);
  int* d_ic2f = s.alloc<int>(n4);
  unsigned* d_err = s.alloc<unsigned>(1);
  cudaError_t& e = s.e;
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_iv, m.IVCELL.data(), sizeof(int) * n4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_x, m.XV.data(), sizeof(double) * m.NVERT, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_y, m.YV.data(), sizeof(double) * m.NVERT, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_keys, 0xff, sizeof(unsigned long long) * tsize, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_cnt, 0, sizeof(int) * tsize, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) { cudaStreamDestroy(st); return -1; }
  k_check_cells<<<grid_of(NC, 256), 256, 0, st>>>(NC, d_iv, d_x, d_y, d_err);
  k_edge_insert<<<grid_of(n4, 256), 256, 0, st>>>(NC, d_iv, d_keys, d_cnt, d_s0, d_s1, d_slot, mask, d_err);
  k_partner<<<grid_of(n4, 256), 256, 0, st>>>(n4, d_slot, d_cnt, d_s0, d_s1, d_other, d_owned);
  e = cudaGetLastError();
  const int NF = scan_exclusive(n4, d_owned, d_pos, d_sums, st, e);
  unsigned herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&herr, d_err, sizeof herr, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) { cudaStreamDestroy(st); return -1; }
  if (herr) { cudaStreamDestroy(st); return 1; }
  int* d_if2c = s.alloc<int>((size_t)4 * NF);
  int* d_if2v = s.alloc<int>((size_t)2 * NF);
  if (e == cudaSuccess)
    k_faces<<<grid_of(n4, 256), 256, 0, st>>>(NC, NF, d_iv, d_other, d_owned, d_pos, d_ic2f, d_if2c, d_if2v, d_err);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, d_err, sizeof herr, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { cudaStreamDestroy(st); return -1; }
  if (herr) { cudaStreamDestroy(st); return 1; }
  m.NFACE = NF;
  m.IC2F.resize(n4);
  m.IF2C.resize((size_t)4 * NF);
  m.IF2V.resize((size_t)2 * NF);
  e = cudaMemcpyAsync(m.IC2F.data(), d_ic2f, sizeof(int) * n4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m.IF2C.data(), d_if2c, sizeof(int) * 4 * (size_t)NF, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m.IF2V.data(), d_if2v, sizeof(int) * 2 * (size_t)NF, cudaMemcpyDeviceToHost, st);
  // boundary records: lookups on the device, lists and errors in record order on the host
  const int nb = (int)bnd.size();
  std::vector<int2> ab(nb);
  for (int r = 0; r < nb; r++) ab[r] = make_int2(bnd[r].a, bnd[r].b);
  std::vector<int> K(nb), stt(nb);
  if (nb) {
    int2* d_ab = s.alloc<int2>(nb);
    int* d_K = s.alloc<int>(nb);
    int* d_st = s.alloc<int>(nb);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_ab, ab.data(), sizeof(int2) * nb, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) k_bnd_lookup<<<grid_of(nb, 128), 128, 0, st>>>(nb, d_ab, d_keys, d_cnt, d_s0, mask, d_ic2f, NC, d_K, d_st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(K.data(), d_K, sizeof(int) * nb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(stt.data(), d_st, sizeof(int) * nb, cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { cudaStreamDestroy(st); return -1; }
  std::vector<char> bflag(NF, 0);
  m.IBFCYC.clear();
  m.IBFREE.clear();
  for (int r = 0; r < nb; r++) {
    int rc = CHORUS_OK;
    if (stt[r] == 1) { err = "boundary edge " + std::to_string(bnd[r].line) + " is not a cell face"; rc = CHORUS_EMESH; }
    else if (stt[r] == 2) { err = "boundary edge " + std::to_string(bnd[r].line) + " is an interior face"; rc = CHORUS_EMESH; }
    else rc = boundary_face(m, bnd[r], K[r], bflag, err);
    if (rc) { rc_out = rc; cudaStreamDestroy(st); return 0; }
  }
  // IBFINTER (two-sided faces in face order) and the missing-boundary check
  unsigned char* d_bflag = s.alloc<unsigned char>(NF);
  int* d_flags = s.alloc<int>(NF);
  int* d_fpos = s.alloc<int>(NF);
  int* d_missing = s.alloc<int>(1);
  const int big = 0x7fffffff;
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_bflag, bflag.data(), NF, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_missing, &big, sizeof(int), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) k_inter_flags<<<grid_of(NF, 256), 256, 0, st>>>(NF, d_if2c, d_bflag, d_flags, d_missing);
  if (e == cudaSuccess) e = cudaGetLastError();
  const int ninter = scan_exclusive(NF, d_flags, d_fpos, d_sums, st, e);
  int missing = big;
  if (e == cudaSuccess) e = cudaMemcpy(&missing, d_missing, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) { cudaStreamDestroy(st); return -1; }
  if (missing != big) {
    err = "boundary face " + std::to_string(missing) + " is missing from the BND file";
    rc_out = CHORUS_EMESH;
    cudaStreamDestroy(st);
    return 0;
  }
  int* d_inter = s.alloc<int>(ninter > 0 ? ninter : 1);
  if (e == cudaSuccess) k_compact<<<grid_of(NF, 256), 256, 0, st>>>(NF, d_flags, d_fpos, d_inter);
  m.IBFINTER.resize(ninter);
  if (e == cudaSuccess && ninter)
    e = cudaMemcpyAsync(m.IBFINTER.data(), d_inter, sizeof(int) * ninter, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { cudaStreamDestroy(st); return -1; }
  // periodic partners on the host, then the operators and the geometry on the device
  int rc = mesh_periodic(m, err);
  if (rc) { rc_out = rc; cudaStreamDestroy(st); return 0; }
  mesh_operators(m);
  Axes axes{};
  for (int i = 0; i < N; i++) axes.Xs[i] = m.Xs[i];
  for (int i = 0; i <= N; i++) axes.Xf[i] = m.Xf[i];
  const size_t ns = (size_t)N * N * NC, nf1 = (size_t)(N + 1) * N * NC;
  double* d_jac = s.alloc<double>(ns);
  double* d_s1m = s.alloc<double>(4 * nf1);
  double* d_s2m = s.alloc<double>(4 * nf1);
  double* d_xx = s.alloc<double>(2 * ns);
  if (e != cudaSuccess) { cudaStreamDestroy(st); return -1; }
  const long long npts = (long long)NC * (N * N + 2 * N * (N + 1));
  k_geometry<<<grid_of(npts, 256), 256, 0, st>>>(NC, N, axes, d_iv, d_x, d_y, d_jac, d_s1m, d_s2m, d_xx);
  e = cudaGetLastError();
  m.Jac.resize(ns);
  m.S1.resize(4 * nf1);
  m.S2.resize(4 * nf1);
  m.XXsolu.resize(2 * ns);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m.Jac.data(), d_jac, sizeof(double) * ns, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m.S1.data(), d_s1m, sizeof(double) * 4 * nf1, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m.S2.data(), d_s2m, sizeof(double) * 4 * nf1, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m.XXsolu.data(), d_xx, sizeof(double) * 2 * ns, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  return e == cudaSuccess ? 0 : -1;
}

}  // namespace

int mesh_load_gpu(const std::string& dir, int device, Mesh& m, std::string& err) {
  std::vector<BndRecord> bnd;
  int rc = mesh_parse(dir, m, bnd, err);
  if (rc) return rc;
  if (cudaSetDevice(device) != cudaSuccess) {
    err = "cudaSetDevice(" + std::to_string(device) + ") failed";
    return CHORUS_ECUDA;
  }
  int rc_dev = CHORUS_OK;
  const int r = build_on_device(m, bnd, err, rc_dev);
  if (r < 0) {
    err = std::string("device mesh setup: ") + cudaGetErrorString(cudaGetLastError());
    return CHORUS_ECUDA;
  }
  if (r == 1) {
    // an invalid mesh: the host path finds the reference's error for it
    rc = mesh_maps_host(m, bnd, err);
    if (!rc) rc = mesh_periodic(m, err);
    if (!rc) {
      mesh_operators(m);
      mesh_geometry_host(m);
    }
    if (rc) return rc;
  } else if (rc_dev) {
    return rc_dev;
  }
  m.params.NCELLGLOB = m.NCELL;
  return CHORUS_OK;
}

}  // namespace chorus
