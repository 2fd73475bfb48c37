// batch.cu -- many independent solves of mixed size and order advanced together:
// one launch per pass for the whole ensemble.
//
// Each pass is a persistent kernel (a fixed grid of CTAs sized to the GPU) that pulls
// tiles from a device work table with an atomic counter.  A cell tile is
// (solve, first cell, cells, N), a face tile (solve, first face point, points, N); the
// kernel copies the tile's solve descriptor to shared memory and runs the same
// per-N pass body as the single-solve kernels, so a solve gives the same bits alone and
// in a batch.  Tables, counts and per-solve RK coefficients live in device memory and
// are rewritten between steps, so one captured CUDA graph serves any composition that
// fits the table capacities (the serving loop changes the mix every step).
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

struct BatchDev {
  const SolveDev* solves;   // per slot (eig/err point into the batch's own arrays)
  const int4* ctiles;       // (slot, e0, cnt, N): the E1, E2, E3 and CT tile lists, one after another
  const int4* ftiles;       // (slot, t0, cnt, N)
  const int* ntiles;        // [0] E1 tiles, [1] face tiles, [2] E2 tiles, [3] E3 tiles, [4] CT tiles
  int* counters;            // per-launch tile counters, zeroed at the start of each stage
  const RKStage* rk;        // [5][cap]
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

// Walks a tile list with a persistent CTA: thread 0 claims the next tile with an atomic
// issued before the current tile's work (its latency overlaps the work), and the solve
// descriptor is copied to shared memory only when the solve changes.  body(T, s) runs
// with the whole CTA.
template <class Body>
__device__ __forceinline__ void for_each_tile(int* counter, int nt, const int4* tiles, const SolveDev* solves,
                                              Body&& body) {
  __shared__ int cur;
  if (threadIdx.x == 0) cur = atomicAdd(counter, 1);
  __syncthreads();
  int ti = cur, slot = -1;
  const SolveDev* s = nullptr;
  while (ti < nt) {
    int nxt = 0;
    if (threadIdx.x == 0) nxt = atomicAdd(counter, 1);  // consumed after the tile
    const int4 T = tiles[ti];
    if (T.x != slot) {
      s = &load_solve(solves + T.x);  // ends with a barrier
      slot = T.x;
    }
    body(T, *s);
    __syncthreads();  // every thread is done with this tile
    if (threadIdx.x == 0) cur = nxt;
    __syncthreads();
    ti = cur;
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

// each cell pass walks its own tile list, cut with that pass's cells per CTA.  The
// multi-order bodies need more registers than any single order; E1 and E3 are held to
// 64 (4 and 8 CTAs per SM), which measured faster than fewer CTAs without spills
__global__ void __launch_bounds__(256, 4) kb_e1(BatchDev b, int slot, int sensor_on) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  for_each_tile(b.counters + slot, b.ntiles[0], b.ctiles, b.solves, [&](const int4& T, const SolveDev& s) {
    if (T.y == 0 && threadIdx.x == 0) *s.eig = 0ull;  // the solve's stage starts its wave-speed maximum
    // 1: variable-1 sensor; 3: also variable 6 when the solve's plot flag is set
    const int sensor = s.artiv ? ((sensor_on & 2) && !*s.plot_flag ? 1 : sensor_on) : 0;
#define CALL(n) e1_body<n, OpsAll<n>>(s, T.y, T.z, T.z, sensor, sm)
    CHORUS_BATCH_SWITCH(T.w, CALL)
#undef CALL
  });
}

__global__ void __launch_bounds__(256) kb_e2(BatchDev b, int slot) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  for_each_tile(b.counters + slot, b.ntiles[2], b.ctiles + b.ntiles[0], b.solves,
                [&](const int4& T, const SolveDev& s) {
#define CALL(n) e2_body<n, OpsAll<n>>(s, T.y, T.z, T.z, sm)
                  CHORUS_BATCH_SWITCH(T.w, CALL)
#undef CALL
                });
}

__global__ void __launch_bounds__(128, 8) kb_e3(BatchDev b, int slot, int stage) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  for_each_tile(b.counters + slot, b.ntiles[3], b.ctiles + b.ntiles[0] + b.ntiles[2], b.solves,
                [&](const int4& T, const SolveDev& s) {
                  const RKStage& rk = b.rk[stage * b.cap + T.x];
#define CALL(n) e3_body<n, OpsAll<n>>(s, T.y, T.z, T.z, rk, 1, sm)
                  CHORUS_BATCH_SWITCH(T.w, CALL)
#undef CALL
                });
}

__global__ void __launch_bounds__(128) kb_ct(BatchDev b, int slot, int mode) {
  extern __shared__ __align__(16) double sm[];
  pdl_wait();
  for_each_tile(b.counters + slot, b.ntiles[4], b.ctiles + b.ntiles[0] + b.ntiles[2] + b.ntiles[3], b.solves,
                [&](const int4& T, const SolveDev& s) {
#define CALL(n) ct_elem_body<n, OpsAll<n>>(s, T.y, T.z, T.z, mode, sm)
                  CHORUS_BATCH_SWITCH(T.w, CALL)
#undef CALL
                });
}

// face passes: which = 0 Rusanov (F1), 1 grad Q trace averages (not part of a step), 2 CT average
__global__ void __launch_bounds__(128) kb_face(BatchDev b, int slot, int which) {
  pdl_wait();
  for_each_tile(b.counters + slot, b.ntiles[1], b.ftiles, b.solves, [&](const int4& T, const SolveDev& s) {
    // a tile holds 128 to kFaceTileMax points, taken blockDim.x at a time
    unsigned long long evb = 0ull;
    for (int base = 0; base < T.z; base += blockDim.x) {
      const int t = T.y + base + threadIdx.x;
      if (base + (int)threadIdx.x >= T.z) continue;
      if (which == 0) {
        unsigned long long v = 0ull;
#define CALL(n) v = f1_point<n>(s, t)
        CHORUS_BATCH_SWITCH(T.w, CALL)
#undef CALL
        evb = v > evb ? v : evb;
      } else if (which == 1) {
#define CALL(n) f2_point<n>(s, t)
        CHORUS_BATCH_SWITCH(T.w, CALL)
#undef CALL
      } else {
#define CALL(n) ctface_point<n>(s, t)
        CHORUS_BATCH_SWITCH(T.w, CALL)
#undef CALL
      }
    }
    if (which == 0) block_max_ull(evb, s.eig);
  });
}

// dynamic shared memory of a cell pass (0 E1, 1 E2, 2 E3, 3 CT) on tiles of epb cells:
// each pass is launched with its own maximum over the batch, so that one pass's large
// tiles do not cost the others occupancy
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

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BatchSlot {
  ChorusCtx* ctx = nullptr;
  SolveDev sd{};
  int N = 0, NC = 0, nfp_faces = 0;
  int epb = 4;             // cells per tile of E3 and the CT passes
  int epb1 = 4, epb2 = 4;  // ... of E1 and E2
  int epbct = 4;           // ... of the CT element passes
  double dt = 0.0;
  int k_stage = 3;
  int64_t steps = 0;
  bool active = false;
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
  cudaStream_t st = nullptr;
  int cap_solves = 0, cap_ctiles = 0, cap_ftiles = 0;
  std::vector<BatchSlot> slots;
  // device tables
  SolveDev* d_solves = nullptr;
  int4* d_ctiles = nullptr;
  int4* d_ftiles = nullptr;
  int* d_ntiles = nullptr;
  int* d_counters = nullptr;
  RKStage* d_rk = nullptr;
  unsigned long long* d_eig = nullptr;
  unsigned int* d_err = nullptr;
  int grid_cells = 0, grid_faces = 0;
  size_t smem[4] = {0, 0, 0, 0};  // per cell pass: E1, E2, E3, CT
  bool dirty = true;
  cudaGraphExec_t graph = nullptr;
  size_t graph_smem[4] = {0, 0, 0, 0};
  int ctiles = 0, ftiles = 0;
};

static constexpr int kCounterSlots = 32;  // one tile counter per launch of a step (5 x 4 + 3)
static constexpr int kFaceTileMax = 1024;  // face points per tile of the face passes, at most

static int batch_alloc(ChorusBatch* b, int cap_solves, int cap_ctiles, int cap_ftiles) {
  auto fr = [](void* p) { if (p) cudaFree(p); };
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

static int batch_rebuild(ChorusBatch* b) {
  std::vector<int> act;
  for (int i = 0; i < (int)b->slots.size(); i++)
    if (b->slots[i].active) act.push_back(i);
  // tiles: largest N first so the slowest tiles start early
  std::vector<int4> ct, ft;
  std::vector<int> order(act);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->slots[a].N > b->slots[c].N; });
  size_t smem[4] = {0, 0, 0, 0};
  std::vector<int4> ct2, ct3, ct4;
  // face tiles: 128 points (one per thread) while the batch is small, up to
  // kFaceTileMax when there are enough points for about four tiles per CTA
  long long total_fp = 0;
  for (int i : order) total_fp += b->slots[i].nfp_faces;
  int face_tile = (int)std::min<long long>(kFaceTileMax, std::max<long long>(128, total_fp / (4LL * b->grid_faces)));
  face_tile -= face_tile % 128;
  for (int i : order) {
    const BatchSlot& sl = b->slots[i];
    for (int e0 = 0; e0 < sl.NC; e0 += sl.epb1) ct.push_back(make_int4(i, e0, std::min(sl.epb1, sl.NC - e0), sl.N));
    for (int e0 = 0; e0 < sl.NC; e0 += sl.epb2) ct2.push_back(make_int4(i, e0, std::min(sl.epb2, sl.NC - e0), sl.N));
    for (int e0 = 0; e0 < sl.NC; e0 += sl.epb) ct3.push_back(make_int4(i, e0, std::min(sl.epb, sl.NC - e0), sl.N));
    for (int e0 = 0; e0 < sl.NC; e0 += sl.epbct) ct4.push_back(make_int4(i, e0, std::min(sl.epbct, sl.NC - e0), sl.N));
    for (int t0 = 0; t0 < sl.nfp_faces; t0 += face_tile)
      ft.push_back(make_int4(i, t0, std::min(face_tile, sl.nfp_faces - t0), sl.N));
    smem[0] = std::max(smem[0], cell_smem_bytes(sl.N, sl.epb1, 0));
    smem[1] = std::max(smem[1], cell_smem_bytes(sl.N, sl.epb2, 1));
    smem[2] = std::max(smem[2], cell_smem_bytes(sl.N, sl.epb, 2));
    smem[3] = std::max(smem[3], cell_smem_bytes(sl.N, sl.epbct, 3));
  }
  const int n_e1 = (int)ct.size(), n_e2 = (int)ct2.size(), n_e3 = (int)ct3.size(), n_ct = (int)ct4.size();
  ct.insert(ct.end(), ct2.begin(), ct2.end());
  ct.insert(ct.end(), ct3.begin(), ct3.end());
  ct.insert(ct.end(), ct4.begin(), ct4.end());
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
  cudaError_t e = cudaSuccess;
  if (ns) e = cudaMemcpyAsync(b->d_solves, sd.data(), sizeof(SolveDev) * ns, cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess && !ct.empty())
    e = cudaMemcpyAsync(b->d_ctiles, ct.data(), sizeof(int4) * ct.size(), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess && !ft.empty())
    e = cudaMemcpyAsync(b->d_ftiles, ft.data(), sizeof(int4) * ft.size(), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_rk, rk.data(), sizeof(RKStage) * rk.size(), cudaMemcpyHostToDevice, b->st);
  int nt[5] = {n_e1, (int)ft.size(), n_e2, n_e3, n_ct};
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_ntiles, nt, sizeof nt, cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "batch tables upload: %s", cudaGetErrorString(e));
  b->ctiles = nt[3];
  b->ftiles = nt[1];
  bool grew = false;
  for (int p = 0; p < 4; p++) {
    grew = grew || smem[p] > b->graph_smem[p];
    b->smem[p] = std::max(b->smem[p], smem[p]);
  }
  if (grew && b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  b->dirty = false;
  return CHORUS_OK;
}

static void batch_enqueue_step(ChorusBatch* b) {
  BatchDev a;
  a.solves = b->d_solves;
  a.ctiles = b->d_ctiles;
  a.ftiles = b->d_ftiles;
  a.ntiles = b->d_ntiles;
  a.counters = b->d_counters;
  a.rk = b->d_rk;
  a.cap = b->cap_solves;
  a.pad = 0;
  const size_t* sm = b->smem;
  // every launch of the step has its own tile counter, so one memset per step clears
  // them all; E1 starts each solve's wave-speed maximum; the launches are programmatic
  // (each is scheduled while its predecessor drains and waits for it at entry)
  cudaMemsetAsync(b->d_counters, 0, sizeof(int) * kCounterSlots, b->st);
  for (int stage = 0; stage < 5; stage++) {
    const int c0 = 4 * stage;
    launch_pdl(kb_e1, b->grid_cells, 256, sm[0], b->st, a, c0, stage == 4 ? 3 : 1);
    launch_pdl(kb_face, b->grid_faces, 128, 0, b->st, a, c0 + 1, 0);
    launch_pdl(kb_e2, b->grid_cells, 256, sm[1], b->st, a, c0 + 2);  // also the face AV viscosities
    launch_pdl(kb_e3, b->grid_cells, 128, sm[2], b->st, a, c0 + 3, stage);
  }
  launch_pdl(kb_ct, b->grid_cells, 128, sm[3], b->st, a, 20, 0);
  launch_pdl(kb_face, b->grid_faces, 128, 0, b->st, a, 21, 2);
  launch_pdl(kb_ct, b->grid_cells, 128, sm[3], b->st, a, 22, 2);
}

extern "C" {

int chorus_batch_create(int32_t device, ChorusBatch** out) {
  if (!out) return set_err(CHORUS_EINVAL, "null argument");
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return set_err(CHORUS_ECUDA, "cudaSetDevice(%d)", device);
  ChorusBatch* b = new ChorusBatch();
  b->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_ntiles, sizeof(int) * 5);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_counters, sizeof(int) * kCounterSlots);
  if (e != cudaSuccess) {
    delete b;
    return set_err(CHORUS_ECUDA, "batch create: %s", cudaGetErrorString(e));
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  b->grid_cells = sms * 8;  // persistent CTAs: 8 per SM (occupancy is not what bounds FP64)
  b->grid_faces = sms * 8;
  const int lim = 200 * 1024;
  cudaFuncSetAttribute(kb_e1, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(kb_e2, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(kb_e3, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  cudaFuncSetAttribute(kb_ct, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
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
  void* ptrs[] = {b->d_solves, b->d_ctiles, b->d_ftiles, b->d_ntiles, b->d_counters, b->d_rk, b->d_eig, b->d_err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
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
  // tiles keep the cells-per-thread ratio of the solve's tuned shapes at the batched
  // kernels' fixed CTA sizes (E1, E2 256 threads, E3 128); E1 and E2 tiles of at most 8
  // cells keep their shared memory (and occupancy) in the range the shapes were tuned for
  auto scaled = [&](int pass, int threads, int cap) {
    const int e = ctx_epb(ctx, pass) * threads / std::max(ctx_threads(ctx, pass), 1);
    return std::max(1, std::min(e, cap));
  };
  sl.epb = scaled(2, 128, 64);
  sl.epb1 = scaled(0, 256, 8);
  sl.epb2 = scaled(1, 256, 8);
  sl.epbct = std::max(1, std::min(ctx_epb(ctx, 3), 64));
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
    batch_enqueue_step(b);
    e = cudaStreamEndCapture(b->st, &g);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (e == cudaSuccess) cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_err(CHORUS_ECUDA, "batch graph: %s", cudaGetErrorString(e));
    for (int p = 0; p < 4; p++) b->graph_smem[p] = b->smem[p];
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
