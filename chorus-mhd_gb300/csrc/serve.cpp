// serve.cpp -- the serving form: a request loop with continuous batching.
//
// Requests (a case directory, an arrival time, a physical end time) arrive over time.
// At every step boundary the loop admits the requests that have arrived, in arrival
// order, while their device memory fits the HBM budget; an admitted solve is set up
// (mesh maps, binding, initial state with its CT projection) while the previous batch
// step is still running on the GPU, then joins the batch; every step advances all
// admitted solves with one launch per pass; a solve leaves the batch, and its memory
// returns to the budget, after its last step.  Mode 1 is the plain sequential loop the
// batched form is compared with: requests run one at a time, first come first served,
// each with its own single-solve CUDA graph.
//
// A retiring solve hands back its result before its memory is released: the final Q in
// the reference layout into the request's Q_out and/or the restart stream of
// write_data.f90:44-74 at restart_path.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <string>
#include <thread>
#include <vector>

#include "chorus_internal.h"

namespace chorus {
int set_err(int code, const char* fmt, ...);
}

namespace {

struct Live {
  int req = -1;
  ChorusMesh* mesh = nullptr;
  ChorusCtx* ctx = nullptr;
  int slot = -1;
  int64_t steps_left = 0;
  int64_t bytes = 0;
};

double now_s(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void wait_until(std::chrono::steady_clock::time_point t0, double t) {
  double d = t - now_s(t0);
  if (d > 0) std::this_thread::sleep_for(std::chrono::duration<double>(d));
}

int open_request(const ChorusServeRequest& r, int device, int gpu_setup, Live& L, int64_t* dof, int32_t* steps,
                 double* ctime) {
  int rc = gpu_setup ? chorus_mesh_load_gpu(r.case_dir, device, &L.mesh) : chorus_mesh_load(r.case_dir, &L.mesh);
  if (rc) return rc;
  ChorusDims d;
  ChorusParams p;
  chorus_mesh_info(L.mesh, &d, &p, nullptr, nullptr);
  L.bytes = chorus_mesh_device_bytes(L.mesh);
  L.steps_left = (int64_t)std::ceil(r.end_time / p.dt - 1e-9);
  if (L.steps_left < 1) L.steps_left = 1;
  *dof = (int64_t)d.NCELL * d.N * d.N;
  *steps = (int32_t)L.steps_left;
  // ctime of the reference's bookkeeping: dt added once per step (iterations.f90:162-217)
  double t = 0.0;
  for (int64_t k = 0; k < L.steps_left; k++) t = t + p.dt;
  *ctime = t;
  if (r.Q_out && r.Q_out_count != (int64_t)9 * d.N * d.N * d.NCELL)
    return chorus::set_err(CHORUS_EINVAL, "request %s: Q_out_count %lld, the state has %lld doubles", r.case_dir,
                           (long long)r.Q_out_count, (long long)9 * d.N * d.N * d.NCELL);
  return CHORUS_OK;
}

// hand back a finished solve's state (before its context is freed)
int deliver(const ChorusServeRequest& r, const ChorusServeResult& res, ChorusCtx* ctx) {
  int rc = CHORUS_OK;
  if (r.Q_out) rc = chorus_gpu_download_state(ctx, r.Q_out);
  if (!rc && r.restart_path) rc = chorus_write_restart(ctx, r.restart_path, res.steps, res.ctime);
  return rc;
}

void close_live(Live& L) {
  if (L.ctx) chorus_gpu_free(L.ctx);
  if (L.mesh) chorus_mesh_free(L.mesh);
  L.ctx = nullptr;
  L.mesh = nullptr;
}

}  // namespace

extern "C" int chorus_serve_run(const ChorusServeRequest* reqs, int32_t n, const ChorusServeConfig* cfg,
                                ChorusServeResult* out, double* makespan_s) {
  if (!reqs || n < 0 || !cfg || !out) return chorus::set_err(CHORUS_EINVAL, "chorus_serve_run: bad argument");
  for (int i = 0; i < n; i++) {
    std::memset(&out[i], 0, sizeof(ChorusServeResult));
    out[i].status = -1;
    if (i && reqs[i].arrival_s < reqs[i - 1].arrival_s)
      return chorus::set_err(CHORUS_EINVAL, "requests must be sorted by arrival time");
  }
  const auto t0 = std::chrono::steady_clock::now();
  const int dev = cfg->device;
  if (cfg->mode == 1) {
    // plain sequential loop: one solve at a time, first come first served
    for (int i = 0; i < n; i++) {
      wait_until(t0, reqs[i].arrival_s);
      Live L;
      int64_t dof = 0;
      int32_t steps = 0;
      double ctime_end = 0.0;
      out[i].admit_s = now_s(t0);
      int rc = open_request(reqs[i], dev, cfg->gpu_setup, L, &dof, &steps, &ctime_end);
      if (!rc) rc = chorus_gpu_bind_mesh(L.mesh, dev, &L.ctx);
      if (!rc) rc = chorus_initial_state(L.mesh, L.ctx, nullptr);
      if (!rc) rc = chorus_gpu_set_option(L.ctx, "diagnostics", 0);
      int32_t it = 0;
      double ct = 0.0;
      if (!rc) rc = iterations_gpu(L.ctx, steps, &it, &ct, nullptr, 0, nullptr);
      out[i].steps = steps;
      out[i].dof = dof;
      out[i].ctime = ctime_end;
      if (!rc) rc = deliver(reqs[i], out[i], L.ctx);
      out[i].finish_s = now_s(t0);
      out[i].latency_s = out[i].finish_s - reqs[i].arrival_s;
      out[i].status = rc;
      close_live(L);
    }
    if (makespan_s) *makespan_s = now_s(t0);
    return CHORUS_OK;
  }
  // continuous batching
  ChorusBatch* batch = nullptr;
  int rc = chorus_batch_create(dev, &batch);
  if (rc) return rc;
  std::vector<Live> live, ready;
  int next = 0, done = 0;
  int64_t used = 0;  // bytes of ready + live solves
  const int64_t budget = cfg->hbm_budget_bytes > 0 ? cfg->hbm_budget_bytes : INT64_MAX;
  bool running = false;  // a batch step is in flight
  Live pending;          // read (mesh maps built) but waiting for device memory
  bool have_pending = false;
  double blocked_since = -1.0;  // when the pending request was first refused for memory
  auto finish = [&](Live& L, int status) {
    if (status == CHORUS_OK && L.ctx) status = deliver(reqs[L.req], out[L.req], L.ctx);
    out[L.req].finish_s = now_s(t0);
    out[L.req].latency_s = out[L.req].finish_s - reqs[L.req].arrival_s;
    out[L.req].status = status;
    close_live(L);
    done++;
  };
  while (done < n) {
    // 1. set up arrived requests (host work, overlapping the step in flight)
    while (next < n || have_pending) {
      if (!have_pending) {
        if (reqs[next].arrival_s > now_s(t0)) break;
        int64_t dof = 0;
        int32_t steps = 0;
        double ctime_end = 0.0;
        pending = Live();
        pending.req = next;
        rc = open_request(reqs[next], dev, cfg->gpu_setup, pending, &dof, &steps, &ctime_end);
        out[next].dof = dof;
        out[next].steps = steps;
        out[next].ctime = ctime_end;
        next++;
        if (rc) { finish(pending, rc); continue; }
        if (pending.bytes > budget) { finish(pending, CHORUS_ENOMEM); continue; }
        have_pending = true;
      }
      if (used + pending.bytes > budget ||
          (cfg->max_active > 0 && (int)(live.size() + ready.size()) >= cfg->max_active)) {
        if (blocked_since < 0) blocked_since = now_s(t0);  // wait until memory returns
        break;
      }
      Live L = pending;
      have_pending = false;
      out[L.req].admit_s = now_s(t0);
      out[L.req].wait_s = blocked_since < 0 ? 0.0 : out[L.req].admit_s - blocked_since;
      blocked_since = -1.0;
      rc = chorus_gpu_bind_mesh(L.mesh, dev, &L.ctx);
      if (!rc) rc = chorus_initial_state(L.mesh, L.ctx, nullptr);
      if (rc) { finish(L, rc); continue; }
      used += L.bytes;
      ready.push_back(L);
    }
    // 2. finish the step in flight and retire completed (or failed) solves
    if (running) {
      int bad = -1;
      const int src = chorus_batch_sync(batch, &bad);
      running = false;
      if (src && bad < 0) { rc = src; break; }
      for (size_t i = 0; i < live.size();) {
        Live& L = live[i];
        const bool failed = src && bad == L.slot;
        if (L.steps_left <= 0 || failed) {
          chorus_batch_remove(batch, L.slot);
          used -= L.bytes;
          finish(L, failed ? CHORUS_ESTATE : CHORUS_OK);
          live.erase(live.begin() + i);
        } else {
          i++;
        }
      }
      continue;  // memory may have returned: admit before the next step
    }
    // 3. newly set-up solves join the batch between steps
    for (Live& L : ready) {
      rc = chorus_batch_add(batch, L.ctx, &L.slot);
      if (rc) { used -= L.bytes; finish(L, rc); continue; }
      live.push_back(L);
    }
    ready.clear();
    // 4. one step of every admitted solve
    if (live.empty()) {
      if (next < n && !have_pending) wait_until(t0, reqs[next].arrival_s);
      continue;
    }
    rc = chorus_batch_step(batch, 1);
    if (rc) break;
    running = true;
    for (auto& L : live) L.steps_left--;
  }
  if (running) chorus_batch_sync(batch, nullptr);
  for (auto& L : live) close_live(L);
  for (auto& L : ready) close_live(L);
  if (have_pending) close_live(pending);
  chorus_batch_free(batch);
  if (makespan_s) *makespan_s = now_s(t0);
  return rc;
}
