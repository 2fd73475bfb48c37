// batch.cu -- many independent solves of mixed size and order advanced together:
// one launch per pass for the whole ensemble.
//
// Each pass is one launch per order N present in the batch: a persistent kernel (a grid
// of CTAs sized by occupancy to fill the GPU) specialised for N, with the launch shape
// tuned for N, walking that order's tiles with a static stride.  A cell tile is
// (solve, first cell, cells), a face tile (solve, first face point, points); the kernel
// copies the tile's solve descriptor to shared memory and runs the same per-N pass body
// as the single-solve kernels, so a solve gives the same bits alone and in a batch.
// Tables, counts and per-solve RK coefficients live in device memory and are rewritten
// between steps, so one captured CUDA graph serves any composition whose orders it
// already launches and that fits the table capacities (the serving loop changes the mix
// every step).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "chorus_internal.h"
#include "kernels.cuh"

namespace chorus {

int set_err(int code, const char* fmt, ...);

static __constant__ OpsN c_ops_all[kMaxN + 1];

template <int N>
struct OpsAll {
  __device__ static const OpsN& ops() { return c_ops_all[N]; }
};

void upload_ops_all(int N, const OpsN& o) {
  cudaMemcpyToSymbol(c_ops_all, &o, sizeof(OpsN), sizeof(OpsN) * N);
}

// passes of a step, in the order of the tile tables
enum { PE1 = 0, PF1, PE2, PE3, PCT, PCTF, kPasses };
constexpr int kGroups = kPasses * (kMaxN + 1);
__host__ __device__ constexpr int gidx(int pass, int N) { return pass * (kMaxN + 1) + N; }

struct BatchDev {
  const SolveDev* solves;  // per slot (eig/err point into the batch's own arrays)
  const int4* ctiles;      // cell tiles (slot, first cell, cells, 0) of every cell pass and order
  const int4* ftiles;      // face tiles (slot, first face point, points, 0)
  const int* gcount;       // [pass][N] tiles of that pass and order
  const int* goff;         // [pass][N] their first entry in ctiles / ftiles
  const RKStage* rk;       // [5][cap]
  int cap;
  int pad;
};

namespace {

__device__ __forceinline__ const SolveDev& load_solve(const SolveDev* src) {
  __shared__ __align__(16) SolveDev ss;
  constexpr int n4 = sizeof(SolveDev) / 16;
  static_assert(sizeof(SolveDev) % 16 == 0, "SolveDev must be a multiple of 16 bytes");
  const int4* a = reinterpret_cast<const int4*>(src);
  int4* d = reinterpret_cast<int4*>(&ss);
  for (int i = threadIdx.x; i < n4; i += blockDim.x) d[i] = a[i];
  __syncthreads();
  return ss;
}

// A CTA of a pass kernel for order N walks the pass's tiles of that order with a static
// stride (tile blockIdx.x, then + gridDim.x, ...): consecutive tiles of one solve go to
// consecutive CTAs, and the solve descriptor is copied to shared memory only when the
// solve changes.  body(T, s) runs with the whole CTA; a barrier separates tiles.
template <class Body>
__device__ __forceinline__ void for_tiles(const BatchDev& b, int g, const int4* tiles, Body&& body) {
  const int cnt = b.gcount[g];
  const int4* t = tiles + b.goff[g];
  int slot = -1;
  const SolveDev* s = nullptr;
  for (int ti = blockIdx.x; ti < cnt; ti += gridDim.x) {
    const int4 T = t[ti];
    if (T.x != slot) {
      s = &load_solve(b.solves + T.x);  // ends with a barrier
      slot = T.x;
    }
    body(T, *s);
    __syncthreads();  // every thread is done with this tile's shared memory
  }
}

// One kernel per pass and order N, launched only for the orders present in the batch,
// each with the launch shape tuned for its order and the register budget of its own
// body, running the same per-N bodies as the single-solve kernels (so a solve gives the
// same bits alone and in a batch).
template <int N>
__global__ void __launch_bounds__(512, 2) kg_e1(BatchDev b, int sensor_on) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  for_tiles(b, gidx(PE1, N), b.ctiles, [&](const int4& T, const SolveDev& s) {
    if (T.y == 0 && threadIdx.x == 0) *s.eig = 0ull;  // the solve's stage starts its wave-speed maximum
    // 1: variable-1 sensor; 3: also variable 6 when the solve's plot flag is set
    const int sensor = s.artiv ? ((sensor_on & 2) && !*s.plot_flag ? 1 : sensor_on) : 0;
    e1_body<N, OpsAll<N>>(s, T.y, T.z, T.z, sensor, sm);
  });
}

template <int N>
__global__ void __launch_bounds__(256) kg_f1(BatchDev b) {
  pdl_wait();
  for_tiles(b, gidx(PF1, N), b.ftiles, [&](const int4& T, const SolveDev& s) {
    unsigned long long evb = 0ull;
    if ((int)threadIdx.x < T.z) evb = f1_point<N>(s, T.y + threadIdx.x);
    block_max_ull(evb, s.eig);
  });
}

// E2 tiles are chunks of up to blockDim.x cells, compacted to the cells that need
// gradients and run in groups of epb (as k_e2)
template <int N>
__global__ void __launch_bounds__(512) kg_e2(BatchDev b, int epb) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  for_tiles(b, gidx(PE2, N), b.ctiles, [&](const int4& T, const SolveDev& s) {
    e2_chunk<N, OpsAll<N>>(s, T.y, T.z, epb, sm);
  });
}

template <int N>
__global__ void __launch_bounds__(512, 2) kg_e3(BatchDev b, int stage) {
  extern __shared__ __align__(16) double sm[];
  __shared__ __align__(16) RKStage srk;
  pdl_wait();
  for_tiles(b, gidx(PE3, N), b.ctiles, [&](const int4& T, const SolveDev& s) {
    if (threadIdx.x == 0) srk = b.rk[stage * b.cap + T.x];
    __syncthreads();
    e3_body<N, OpsAll<N>>(s, T.y, T.z, T.z, srk, 1, sm);
  });
}

template <int N>
__global__ void __launch_bounds__(256) kg_ct(BatchDev b, int mode) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  for_tiles(b, gidx(PCT, N), b.ctiles, [&](const int4& T, const SolveDev& s) {
    ct_elem_body<N, OpsAll<N>>(s, T.y, T.z, T.z, mode, sm);
  });
}

template <int N>
__global__ void __launch_bounds__(256) kg_ctface(BatchDev b) {
  pdl_wait();
  for_tiles(b, gidx(PCTF, N), b.ftiles, [&](const int4& T, const SolveDev& s) {
    if ((int)threadIdx.x < T.z) ctface_point<N>(s, T.y + threadIdx.x);
  });
}

// dynamic shared memory of a cell pass (0 E1, 1 E2, 2 E3, 3 CT) on tiles of epb cells
size_t cell_smem_bytes(int N, int epb, int pass) {
  const int NS = N * N, NFP = 2 * (N + 1) * N;
  size_t d = 0;
  switch (pass) {
    case 0: d = (size_t)epb * (NS * 9 + 2 * NS + NFP * 9) + N * N; break;
    case 1: d = (size_t)epb * (NFP * 16 + NS * 17); break;
    case 2: d = (size_t)epb * (NFP * 8 + NS * (1 + 9 + 1 + 2) + NFP * 2); break;
    default: d = (size_t)epb * (NFP * 2 + NS * 2); break;
  }
  return sizeof(double) * d;
}

}  // namespace

// launch shape of one pass kernel of one order
struct PassShape {
  int threads = 0, grid = 0, epb = 0;
  size_t smem = 0;
};

// the launches of order N: shapes filled on first use (occupancy-sized persistent grids)
template <int N>
static void pass_shapes(int nsm, const int (&epb)[4], const int (&threads)[4], PassShape (&sh)[kPasses]) {
  const int lim = 200 * 1024;
  cudaFuncSetAttribute(kg_e1<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(kg_e2<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(kg_e3<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(kg_ct<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  // every pass kernel asks for the same shared-memory carveout, so that CTAs of the
  // concurrent order chains share an SM without reconfiguring it
  const void* fns[6] = {(const void*)kg_e1<N>, (const void*)kg_f1<N>, (const void*)kg_e2<N>,
                        (const void*)kg_e3<N>, (const void*)kg_ct<N>, (const void*)kg_ctface<N>};
  for (const void* f : fns)
    cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  auto fill = [&](PassShape& p, const void* fn, int thr, int e, size_t smem) {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, thr, smem) != cudaSuccess || occ < 1) occ = 1;
    p.threads = thr;
    p.epb = e;
    p.smem = smem;
    p.grid = nsm * occ;
  };
  fill(sh[PE1], (const void*)kg_e1<N>, threads[0], epb[0], cell_smem_bytes(N, epb[0], 0));
  fill(sh[PF1], (const void*)kg_f1<N>, 256, 0, 0);
  fill(sh[PE2], (const void*)kg_e2<N>, threads[1], epb[1], cell_smem_bytes(N, epb[1], 1));
  fill(sh[PE3], (const void*)kg_e3<N>, threads[2], epb[2], cell_smem_bytes(N, epb[2], 2));
  fill(sh[PCT], (const void*)kg_ct<N>, threads[3], epb[3], cell_smem_bytes(N, epb[3], 3));
  fill(sh[PCTF], (const void*)kg_ctface<N>, 256, 0, 0);
}

template <int N>
static void launch_pass(const BatchDev& a, int pass, const PassShape& p, cudaStream_t st, int arg) {
  switch (pass) {
    case PE1: launch_pdl(kg_e1<N>, p.grid, p.threads, p.smem, st, a, arg); break;
    case PF1: launch_pdl(kg_f1<N>, p.grid, p.threads, 0, st, a); break;
    case PE2: launch_pdl(kg_e2<N>, p.grid, p.threads, p.smem, st, a, p.epb); break;
    case PE3: launch_pdl(kg_e3<N>, p.grid, p.threads, p.smem, st, a, arg); break;
    case PCT: launch_pdl(kg_ct<N>, p.grid, p.threads, p.smem, st, a, arg); break;
    default: launch_pdl(kg_ctface<N>, p.grid, p.threads, 0, st, a); break;
  }
}

#define CHORUS_BATCH_SWITCH(NV, CALL) \
  switch (NV) {                       \
    case 2: CALL(2); break;           \
    case 3: CALL(3); break;           \
    case 4: CALL(4); break;           \
    case 5: CALL(5); break;           \
    case 6: CALL(6); break;           \
    case 7: CALL(7); break;           \
    case 8: CALL(8); break;           \
    default: break;                   \
  }

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BatchSlot {
  ChorusCtx* ctx = nullptr;
  SolveDev sd{};
  int N = 0, NC = 0, nfp_faces = 0, nfp_two = 0;
  double dt = 0.0;
  int k_stage = 3;
  int64_t steps = 0;
  bool active = false;
};

// launch shapes of one order: cells per tile and threads per CTA of E1, E2, E3, CT
struct OrderShape {
  bool used = false;
  int epb[4] = {0, 0, 0, 0}, threads[4] = {0, 0, 0, 0};
  PassShape pass[kPasses];
};

}  // namespace chorus

using namespace chorus;

// accessors of ChorusCtx implemented in capi.cu
namespace chorus {
const SolveDev& ctx_solve(const ChorusCtx* c);
int ctx_device_of(const ChorusCtx* c);
double ctx_dt(const ChorusCtx* c);
int ctx_kstage(const ChorusCtx* c);
int ctx_epb(const ChorusCtx* c, int pass);
int ctx_threads(const ChorusCtx* c, int pass);
void ctx_mark_ct(ChorusCtx* c);
void ensure_ops_all(int dev, int N, const ChorusCtx* c);
}  // namespace chorus

struct ChorusBatch {
  int device = 0;
  int nsm = 152;
  cudaStream_t st = nullptr;
  int cap_solves = 0, cap_ctiles = 0, cap_ftiles = 0;
  std::vector<BatchSlot> slots;
  // device tables
  SolveDev* d_solves = nullptr;
  int4* d_ctiles = nullptr;
  int4* d_ftiles = nullptr;
  int* d_gcount = nullptr;  // [kGroups] then d_goff [kGroups]
  RKStage* d_rk = nullptr;
  unsigned long long* d_eig = nullptr;
  unsigned int* d_err = nullptr;
  OrderShape shape[kMaxN + 1];
  cudaStream_t side[kMaxN + 1] = {};       // one stream per order: the orders' steps are independent chains
  cudaEvent_t fork = nullptr, join[kMaxN + 1] = {};
  int cnt[kGroups] = {};                   // tiles per (pass, order) in the tables
  bool dirty = true;
  cudaGraphExec_t graph = nullptr;
  int graph_grid[kGroups] = {};            // CTAs per launch in the graph (one per tile when captured)
  int ctiles = 0, ftiles = 0;
};

static constexpr int kFaceTile = 256;  // face points per tile (one per thread)

static int batch_alloc(ChorusBatch* b, int cap_solves, int cap_ctiles, int cap_ftiles) {
  auto fr = [](void* p) { if (p) cudaFree(p); };
  cudaStreamSynchronize(b->st);
  fr(b->d_solves); fr(b->d_ctiles); fr(b->d_ftiles); fr(b->d_rk); fr(b->d_eig); fr(b->d_err);
  b->d_solves = nullptr; b->d_ctiles = nullptr; b->d_ftiles = nullptr; b->d_rk = nullptr;
  b->d_eig = nullptr; b->d_err = nullptr;
  cudaError_t e = cudaMalloc(&b->d_solves, sizeof(SolveDev) * std::max(cap_solves, 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_ctiles, sizeof(int4) * std::max(cap_ctiles, 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_ftiles, sizeof(int4) * std::max(cap_ftiles, 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_rk, sizeof(RKStage) * 5 * std::max(cap_solves, 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_eig, sizeof(unsigned long long) * 2 * std::max(cap_solves, 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_err, sizeof(unsigned int) * std::max(cap_solves, 1));
  if (e != cudaSuccess) return set_err(CHORUS_ENOMEM, "batch tables: %s", cudaGetErrorString(e));
  cudaMemsetAsync(b->d_err, 0, sizeof(unsigned int) * std::max(cap_solves, 1), b->st);
  b->cap_solves = cap_solves;
  b->cap_ctiles = cap_ctiles;
  b->cap_ftiles = cap_ftiles;
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  return CHORUS_OK;
}

// the launch shapes of order N, from the first solve of that order (the autotuned shapes
// of its context); every solve of the order is cut into tiles of those shapes
static void order_shape(ChorusBatch* b, const BatchSlot& sl) {
  OrderShape& o = b->shape[sl.N];
  if (o.used) return;
  for (int p = 0; p < 4; p++) {
    o.epb[p] = std::max(1, std::min(ctx_epb(sl.ctx, p), 64));
    o.threads[p] = std::max(32, std::min(ctx_threads(sl.ctx, p), 512));
  }
  // an E2 tile tests up to one cell per thread: a multiple of the group size
  o.epb[1] = std::min(o.epb[1], o.threads[1]);
#define CALL(n) pass_shapes<n>(b->nsm, o.epb, o.threads, o.pass)
  CHORUS_BATCH_SWITCH(sl.N, CALL)
#undef CALL
  o.used = true;
}

static int batch_rebuild(ChorusBatch* b) {
  // tiles per (pass, order); within an order, larger solves first
  std::vector<int> order;
  for (int i = 0; i < (int)b->slots.size(); i++)
    if (b->slots[i].active) order.push_back(i);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->slots[a].NC > b->slots[c].NC; });
  std::vector<int4> grp[kGroups];
  unsigned orders = 0;
  // E2 chunks as the single-solve launch sizes them: up to one cell per thread, but small
  // enough for about 16 CTAs per SM over all the order's cells, so that small solves whose
  // cells all need gradients spread over the GPU
  long long order_cells[kMaxN + 1] = {0};
  for (int i : order) order_cells[b->slots[i].N] += b->slots[i].NC;
  for (int i : order) {
    const BatchSlot& sl = b->slots[i];
    order_shape(b, sl);
    const OrderShape& o = b->shape[sl.N];
    orders |= 1u << sl.N;
    auto cut = [&](int pass, int n, int step) {
      for (int a = 0; a < n; a += step) grp[gidx(pass, sl.N)].push_back(make_int4(i, a, std::min(step, n - a), 0));
    };
    cut(PE1, sl.NC, o.epb[0]);
    cut(PF1, sl.nfp_faces, kFaceTile);
    long long chunk = order_cells[sl.N] / (16LL * b->nsm);
    chunk = std::max<long long>(o.epb[1], std::min<long long>(chunk, o.threads[1]));
    chunk -= chunk % o.epb[1];
    if (!sl.sd.skip) chunk = o.epb[1];
    cut(PE2, sl.NC, (int)std::max<long long>(chunk, 1));
    cut(PE3, sl.NC, o.epb[2]);
    cut(PCT, sl.NC, o.epb[3]);
    cut(PCTF, sl.nfp_two, kFaceTile);
  }
  std::vector<int4> ct, ft;
  int cnt[kGroups], off[kGroups];
  for (int g = 0; g < kGroups; g++) {
    const int pass = g / (kMaxN + 1);
    std::vector<int4>& dst = (pass == PF1 || pass == PCTF) ? ft : ct;
    off[g] = (int)dst.size();
    cnt[g] = (int)grp[g].size();
    dst.insert(dst.end(), grp[g].begin(), grp[g].end());
  }
  const int ns = (int)b->slots.size();
  if (ns > b->cap_solves || (int)ct.size() > b->cap_ctiles || (int)ft.size() > b->cap_ftiles) {
    int rc = batch_alloc(b, std::max(ns * 2, 16), std::max((int)ct.size() * 2, 1024), std::max((int)ft.size() * 2, 1024));
    if (rc) return rc;
  }
  std::vector<SolveDev> sd(ns);
  std::vector<RKStage> rk((size_t)5 * b->cap_solves);
  for (int i = 0; i < ns; i++) {
    sd[i] = b->slots[i].sd;
    sd[i].eig = b->d_eig + 2 * i;
    sd[i].err = b->d_err + i;
    RKStage r[5];
    rk_stage_records(sd[i], b->slots[i].dt, b->slots[i].k_stage, false, r);
    for (int k = 0; k < 5; k++) rk[(size_t)k * b->cap_solves + i] = r[k];
  }
  std::vector<int> counts(cnt, cnt + kGroups);
  counts.insert(counts.end(), off, off + kGroups);
  cudaError_t e = cudaSuccess;
  if (ns) e = cudaMemcpyAsync(b->d_solves, sd.data(), sizeof(SolveDev) * ns, cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess && !ct.empty())
    e = cudaMemcpyAsync(b->d_ctiles, ct.data(), sizeof(int4) * ct.size(), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess && !ft.empty())
    e = cudaMemcpyAsync(b->d_ftiles, ft.data(), sizeof(int4) * ft.size(), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_rk, rk.data(), sizeof(RKStage) * rk.size(), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_gcount, counts.data(), sizeof(int) * counts.size(), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "batch tables upload: %s", cudaGetErrorString(e));
  int n3 = 0;
  for (int N = kMinN; N <= kMaxN; N++) n3 += cnt[gidx(PE3, N)];
  b->ctiles = n3;
  b->ftiles = 0;
  for (int N = kMinN; N <= kMaxN; N++) b->ftiles += cnt[gidx(PF1, N)];
  // the graph launches one CTA per tile as captured; more tiles than that (a new order, or
  // a larger composition) need a new capture, fewer leave CTAs that find no tile
  bool grew = false;
  for (int g = 0; g < kGroups; g++) {
    b->cnt[g] = cnt[g];
    grew = grew || cnt[g] > b->graph_grid[g];
  }
  if (b->graph && grew) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  (void)orders;
  b->dirty = false;
  return CHORUS_OK;
}

// one step: for every order present, its own chain on its own stream -- five stages of
// E1, F1, E2, E3, then the CT projection -- forked from and joined to the batch stream.
// The orders' solves share nothing, so the chains run concurrently and the block
// scheduler mixes their CTAs (FP64-bound flux passes of one order beside the integer
// line operators of another); within a chain every launch is programmatic (scheduled
// while its predecessor drains, waiting for it at entry).  Each launch has one CTA per
// tile of the composition it was captured for.
static void batch_enqueue_step(ChorusBatch* b) {
  BatchDev a;
  a.solves = b->d_solves;
  a.ctiles = b->d_ctiles;
  a.ftiles = b->d_ftiles;
  a.gcount = b->d_gcount;
  a.goff = b->d_gcount + kGroups;
  a.rk = b->d_rk;
  a.cap = b->cap_solves;
  a.pad = 0;
  cudaEventRecord(b->fork, b->st);
  for (int N = kMaxN; N >= kMinN; N--) {
    if (!b->shape[N].used) continue;
    int any = 0;
    for (int p = 0; p < kPasses; p++) any += b->cnt[gidx(p, N)];
    if (!any) continue;
    cudaStream_t st = b->side[N];
    cudaStreamWaitEvent(st, b->fork, 0);
    auto pass = [&](int p, int arg) {
      const int g = gidx(p, N);
      if (!b->cnt[g]) return;
      PassShape ps = b->shape[N].pass[p];
      ps.grid = b->cnt[g];
      b->graph_grid[g] = ps.grid;
#define CALL(n) launch_pass<n>(a, p, ps, st, arg)
      CHORUS_BATCH_SWITCH(N, CALL)
#undef CALL
    };
    for (int stage = 0; stage < 5; stage++) {
      pass(PE1, stage == 4 ? 3 : 1);
      pass(PF1, 0);
      pass(PE2, 0);  // also the face AV viscosities
      pass(PE3, stage);
    }
    pass(PCT, 0);
    pass(PCTF, 0);
    pass(PCT, 2);
    cudaEventRecord(b->join[N], st);
    cudaStreamWaitEvent(b->st, b->join[N], 0);
  }
}

extern "C" {

int chorus_batch_create(int32_t device, ChorusBatch** out) {
  if (!out) return set_err(CHORUS_EINVAL, "null argument");
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return set_err(CHORUS_ECUDA, "cudaSetDevice(%d)", device);
  ChorusBatch* b = new ChorusBatch();
  b->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  for (int N = kMinN; N <= kMaxN && e == cudaSuccess; N++) {
    e = cudaStreamCreateWithFlags(&b->side[N], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[N], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_gcount, sizeof(int) * 2 * kGroups);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_gcount, 0, sizeof(int) * 2 * kGroups, b->st);
  if (e != cudaSuccess) {
    delete b;
    return set_err(CHORUS_ECUDA, "batch create: %s", cudaGetErrorString(e));
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && sms > 0) b->nsm = sms;
  int rc = batch_alloc(b, 16, 4096, 4096);
  if (rc) {
    delete b;
    return rc;
  }
  *out = b;
  return CHORUS_OK;
}

int chorus_batch_free(ChorusBatch* b) {
  if (!b) return CHORUS_OK;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->st);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  void* ptrs[] = {b->d_solves, b->d_ctiles, b->d_ftiles, b->d_gcount, b->d_rk, b->d_eig, b->d_err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (int N = kMinN; N <= kMaxN; N++) {
    if (b->side[N]) cudaStreamDestroy(b->side[N]);
    if (b->join[N]) cudaEventDestroy(b->join[N]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  cudaStreamDestroy(b->st);
  delete b;
  return CHORUS_OK;
}

int chorus_batch_add(ChorusBatch* b, ChorusCtx* ctx, int32_t* slot) {
  if (!b || !ctx) return set_err(CHORUS_EINVAL, "null argument");
  if (ctx_device_of(ctx) != b->device) return set_err(CHORUS_EINVAL, "context and batch are on different devices");
  BatchSlot sl;
  sl.ctx = ctx;
  sl.sd = ctx_solve(ctx);
  sl.N = sl.sd.N;
  sl.NC = sl.sd.NC;
  sl.nfp_faces = (sl.sd.nface2 + sl.sd.nface1) * sl.N;
  sl.nfp_two = sl.sd.nface2 * sl.N;
  sl.dt = ctx_dt(ctx);
  sl.k_stage = ctx_kstage(ctx);
  sl.active = true;
  ensure_ops_all(b->device, sl.N, ctx);
  int idx = -1;
  for (int i = 0; i < (int)b->slots.size(); i++)
    if (!b->slots[i].ctx) { idx = i; break; }
  if (idx < 0) {
    idx = (int)b->slots.size();
    b->slots.push_back(sl);
  } else {
    b->slots[idx] = sl;
  }
  // a reused slot starts without the error flag a previous solve in it may have raised
  // (a slot beyond the tables' capacity gets cleared flags when they grow)
  if (idx < b->cap_solves) {
    cudaError_t e = cudaMemsetAsync(b->d_err + idx, 0, sizeof(unsigned int), b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "batch add: %s", cudaGetErrorString(e));
  }
  b->dirty = true;
  if (slot) *slot = idx;
  return CHORUS_OK;
}

int chorus_batch_remove(ChorusBatch* b, int32_t slot) {
  if (!b || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].ctx)
    return set_err(CHORUS_EINVAL, "bad batch slot %d", slot);
  cudaStreamSynchronize(b->st);
  b->slots[slot] = BatchSlot();
  b->dirty = true;
  return CHORUS_OK;
}

int chorus_batch_step(ChorusBatch* b, int32_t nsteps) {
  if (!b || nsteps < 0) return set_err(CHORUS_EINVAL, "bad argument");
  if (cudaSetDevice(b->device) != cudaSuccess) return set_err(CHORUS_ECUDA, "cudaSetDevice");
  if (b->dirty) {
    int rc = batch_rebuild(b);
    if (rc) return rc;
  }
  if (b->ctiles == 0) return CHORUS_OK;
  if (!b->graph) {
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "capture: %s", cudaGetErrorString(e));
    for (int i = 0; i < kGroups; i++) b->graph_grid[i] = 0;
    batch_enqueue_step(b);
    e = cudaStreamEndCapture(b->st, &g);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (e == cudaSuccess) cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "batch graph: %s", cudaGetErrorString(e));
  }
  for (int s = 0; s < nsteps; s++) {
    cudaError_t e = cudaGraphLaunch(b->graph, b->st);
    if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "batch step: %s", cudaGetErrorString(e));
  }
  for (auto& sl : b->slots)
    if (sl.ctx && sl.active) {
      sl.steps += nsteps;
      if (nsteps > 0) ctx_mark_ct(sl.ctx);  // each step ends with the CT projection
    }
  return CHORUS_OK;
}

int chorus_batch_sync(ChorusBatch* b, int32_t* err_slot) {
  if (!b) return set_err(CHORUS_EINVAL, "null batch");
  cudaError_t e = cudaStreamSynchronize(b->st);
  if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "batch sync: %s", cudaGetErrorString(e));
  const int ns = (int)b->slots.size();
  if (err_slot) *err_slot = -1;
  if (ns) {
    std::vector<unsigned int> h(ns);
    e = cudaMemcpy(h.data(), b->d_err, sizeof(unsigned int) * ns, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "batch err read: %s", cudaGetErrorString(e));
    for (int i = 0; i < ns; i++)
      if (h[i] && b->slots[i].ctx) {
        if (err_slot) *err_slot = i;
        return set_err(CHORUS_ESTATE, "solve in batch slot %d flagged a non-finite wave speed", i);
      }
  }
  return CHORUS_OK;
}

int chorus_batch_stream(ChorusBatch* b, void** stream) {
  if (!b || !stream) return set_err(CHORUS_EINVAL, "null argument");
  *stream = (void*)b->st;
  return CHORUS_OK;
}

int chorus_batch_info(ChorusBatch* b, int32_t* n_solves, int32_t* cell_tiles, int32_t* face_tiles, int64_t* dofs) {
  if (!b) return set_err(CHORUS_EINVAL, "null batch");
  if (b->dirty) {
    int rc = batch_rebuild(b);
    if (rc) return rc;
  }
  int n = 0;
  int64_t d = 0;
  for (auto& sl : b->slots)
    if (sl.ctx && sl.active) {
      n++;
      d += (int64_t)sl.NC * sl.N * sl.N;
    }
  if (n_solves) *n_solves = n;
  if (cell_tiles) *cell_tiles = b->ctiles;
  if (face_tiles) *face_tiles = b->ftiles;
  if (dofs) *dofs = d;
  return CHORUS_OK;
}

}  // extern "C"
