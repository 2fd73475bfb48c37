/*
 * chorus_gpu.h -- C-ABI of libchorus_gpu.so, the GB300 (sm_103a) implementation of
 * CHORUS-MHD's residual-and-time-step hot path.
 *
 * The reference's hot-path routines are external Fortran subroutines that talk
 * through module `setup2d` globals.  A Fortran host binds its setup2d arrays once
 * (chorus_gpu_bind), then calls the `_gpu` drop-ins where it used to CALL the CPU
 * routines; each drop-in keeps the routine's name and argument meaning, with the
 * module state replaced by an explicit context.  Every function returns 0 on success
 * and a nonzero CHORUS_E* code on failure; chorus_gpu_last_error() gives the message
 * (the reference prints and STOPs instead).
 *
 * Layout contract: every array is passed exactly as the Fortran host holds it --
 * column-major, first index fastest, integer maps with 1-based values, INTEGER =
 * int32, DOUBLE PRECISION = double.  The caller keeps ownership of its arrays.
 */
#ifndef CHORUS_GPU_H
#define CHORUS_GPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum {
  CHORUS_OK = 0,
  CHORUS_EINVAL = 1,   /* bad argument / size out of range */
  CHORUS_ECUDA = 2,    /* CUDA runtime error */
  CHORUS_EMESH = 3,    /* mesh/connectivity inconsistency (connectivity.f90 STOP paths) */
  CHORUS_EIO = 4,      /* file I/O */
  CHORUS_ESTATE = 5,   /* non-finite or non-physical state flagged by a kernel */
  CHORUS_ENOMEM = 6,   /* device memory budget exceeded */
};

/* Sizes of one single-partition solve (setup2d.f90:19-21). */
typedef struct ChorusDims {
  int32_t N;      /* solution points per direction, 2..8 (setup2d.f90:47) */
  int32_t NCELL;  /* cells */
  int32_t NFACE;  /* faces (rows of IF2C) */
  int32_t NINTER; /* interior faces (IBFINTER) */
  int32_t NFREE;  /* FREE boundary faces (IBFREE) */
  int32_t NPAIR;  /* local periodic face pairs (CYC2FPAIR) */
} ChorusDims;

/* Physical and run parameters (setup2d.f90:63-81, readinput.f90:17-30).  gam is a
 * compile-time parameter in the reference (5/3, setup2d.f90:68); here it is runtime.
 * B0x/B0y: uniform background field with A_z = A_bg + dA_z, B = B0 + curl(dA_z);
 * zero reproduces the reference exactly. */
typedef struct ChorusParams {
  double gam, mu, eta0;
  double DXCYCL, DYCYCL;  /* used only for the AV length scale (AV.f90:147) */
  double dt;
  double B0x, B0y;
  int32_t NCELLGLOB;
  int32_t vismode;  /* must be 1 (the reference reads Qvfi/Azfi only when vismode==1) */
  int32_t ARTIV;    /* 1: artificial viscosity on */
  int32_t k_stage;  /* 3: RK_S5P3, 5: FiveStageRk */
} ChorusParams;

/* Diagnostics of iterations.f90:39-76, produced when mod(iter,10)==1. */
typedef struct ChorusDiag {
  int32_t iter;
  int32_t pad;
  double ctime;
  double residglob; /* sqrt(sum resid^2 / (NCELLGLOB*N*N*5)) */
  double divBglob;  /* sqrt(sum (dBx/dx+dBy/dy)^2 / (NCELLGLOB*N*N)) */
  double eigvmax_g; /* global max Rusanov wave speed of the last stage (AV.f90:145) */
  double epsilon0;  /* AV amplitude of the last stage (AV.f90:148) */
} ChorusDiag;

typedef struct ChorusCtx ChorusCtx;
typedef struct ChorusMesh ChorusMesh;
typedef struct ChorusBatch ChorusBatch;

/* Thread-local message of the last failing call. */
const char* chorus_gpu_last_error(void);
/* Library version string. */
const char* chorus_gpu_version(void);
/* Name of a CUDA device (the key of the autotuned launch-shape tables). */
int chorus_gpu_device_name(int32_t device, char* buf, int32_t n);

/* ------------------------------------------------------------------------------
 * Binding (replaces the module state set up by INIT_SETUP, initsetup.f90:1-165)
 * --------------------------------------------------------------------------- */
/* Copy maps, operators and metrics to `device` and allocate the resident state and
 * work arrays.  Arrays (Fortran layout):
 *   IF2C(NFACE,4), IBFINTER(NINTER), IBFREE(NFREE), CYC2FPAIR(NPAIR,2),
 *   iface2fp(N,4), jface2fp(N,4)               -- connectivity.f90, connect_bdry.f90,
 *                                                 map_cyc_loc.f90, initsetup.f90:343
 *   Xs(N), Xf(N+1), Lmat(N+1,N), Mmat(N+1,N)   -- initsetup.f90:167-315
 *   S1(2,2,N+1,N,NCELL), S2(2,2,N,N+1,NCELL), Jac(N,N,NCELL) -- calcjacob.f90:1-86 */
int chorus_gpu_bind(const ChorusDims* dims, const int32_t* IF2C, const int32_t* IBFINTER,
                    const int32_t* IBFREE, const int32_t* CYC2FPAIR, const int32_t* iface2fp,
                    const int32_t* jface2fp, const double* Xs, const double* Xf, const double* Lmat,
                    const double* Mmat, const double* S1, const double* S2, const double* Jac,
                    const ChorusParams* params, int32_t device, ChorusCtx** ctx);
int chorus_gpu_free(ChorusCtx* ctx);
/* Change dt / mu / eta0 / ARTIV of a bound context (setup2d.f90:72,77,81). */
int chorus_gpu_set_params(ChorusCtx* ctx, const ChorusParams* params);

/* Resident state Q(9,N,N,NCELL) (setup2d.f90:54). */
int chorus_gpu_upload_state(ChorusCtx* ctx, const double* Q);
int chorus_gpu_download_state(ChorusCtx* ctx, double* Q);
/* Copy a named work array back in the reference layout, for parity checks:
 * "resid" (9,N,N,NC), "F1" (8,N+1,N,NC), "G2" (8,N,N+1,NC), "Qvfi"/"Qvfj" (9,..),
 * "Azfi"/"Azfj", "nablaQs" (9,2,N,N,NC), "nablaQvfi"/"nablaQvfj" (9,2,..),
 * "nablaAs" (2,N,N,NC), "muAVfi"/"muAVfj" (9,2,NC; only variable 1 is carried),
 * "SM_IND1" (NC; sensor of variable 1), "av_active" / "viscous_cells" (NC; 0/1 flags of
 * the last stage when skip_inactive_viscous is in effect).  `count` must equal the array
 * size. */
int chorus_gpu_download_array(ChorusCtx* ctx, const char* name, double* out, int64_t count);
/* eigvmax of the last stage (AV.f90:145) and epsilon0 (AV.f90:148). */
int chorus_gpu_get_eigvmax(ChorusCtx* ctx, double* eigvmax_g, double* epsilon0);

/* ------------------------------------------------------------------------------
 * Drop-ins (reference routine -> GPU entry point)
 * --------------------------------------------------------------------------- */
/* compresid.f90:1-67 (calls compflux.f90:1-31 and everything below it); the result
 * stays on the device in "resid". */
int compresid_gpu(ChorusCtx* ctx);
/* compflux.f90:33-49 comp_inviscid_flux (F1/G2, Qvfi/Qvfj, Azfi/Azfj, eigvmax).  The
 * reference's routine raises the module's eigvmax, which compflux zeroes before calling
 * it; here every evaluation starts it from zero, so chorus_gpu_get_eigvmax afterwards
 * gives the maximum wave speed over this evaluation's faces. */
int comp_inviscid_flux_gpu(ChorusCtx* ctx);
/* compflux.f90:107-157 nablaQsp(v_sta,v_end) on the current Qvfi/Qvfj (1-based
 * variable range, by reference like the Fortran call). */
int nablaqsp_gpu(ChorusCtx* ctx, const int32_t* v_sta, const int32_t* v_end);
/* setinitialcond.f90:82-91 correct_B_via_curl_Az (CT projection B <- curl A_z).  Afterwards
 * Q's B_x, B_y, the face-averaged A_z traces Qvfi(9)/Qvfj(9) (also in "Azfi"/"Azfj") and
 * nablaQs(9,:) hold the projection's values; the other work arrays keep their contents
 * (the reference's inner comp_inviscid_flux also refreshes F1/G2, Qvfi(1:8) and the upwinded
 * Azfi/Azfj: call comp_inviscid_flux_gpu for those). */
int correct_b_via_curl_az_gpu(ChorusCtx* ctx);
/* iterations.f90:162-217 RK_S5P3 and :92-160 FiveStageRk: one 5-stage step with the
 * bound dt; *ctime is advanced exactly as the reference does. */
int rk_s5p3_gpu(ChorusCtx* ctx, double* ctime);
int fivestagerk_gpu(ChorusCtx* ctx, double* ctime);
/* iterations.f90:19-87 without output: nsteps x (RK step by k_stage, CT projection,
 * norms when mod(iter,10)==1).  *iter and *ctime are advanced; up to max_diag
 * diagnostic records are written to diag (may be NULL) and their number to *n_diag.
 * The whole step is replayed from a CUDA graph. */
int iterations_gpu(ChorusCtx* ctx, int32_t nsteps, int32_t* iter, double* ctime, ChorusDiag* diag,
                   int32_t max_diag, int32_t* n_diag);
/* iterations_gpu on a state that lives in host memory, as the reference's own Q does
 * (setup2d.f90:54): Q(9,N,N,NCELL) is read from Qin before the first step and written to
 * Qout after the last one (either may be NULL; they may be the same buffer).  A state of
 * 64 MB or more is copied in chunks of cells on a second stream (option "host_chunks"):
 * the first stage's interior and face flux passes run on each chunk as soon as its cells
 * (and their face neighbours) have arrived, and the last stage's update and the CT
 * projection run chunk by chunk, each chunk's download starting once its cells and their
 * face neighbours are final.  With pinned host memory the copies overlap the kernels and
 * the step is captured as a CUDA graph on first use for each (Qin, Qout) pair and replayed
 * after; pageable memory is accepted and copied synchronously.  The results are those of
 * iterations_gpu bit for bit.  No counterpart in the reference (its Q never leaves the
 * host). */
int chorus_gpu_step_host(ChorusCtx* ctx, const double* Qin, double* Qout, int32_t nsteps, int32_t* iter,
                         double* ctime, ChorusDiag* diag, int32_t max_diag, int32_t* n_diag);

/* Point functions with the reference argument lists, evaluated on the device over n
 * points (host arrays, row i at offset i*stride): getrusanov.f90:1-109, :111-153,
 * :157-249 and :251-360 (the AV form is getvfluxvectors with mu=mu_art, eta0=0). */
int getrusanovflux_gpu(int32_t n, double gam, const double* Qfl /*n x 9*/, const double* Qfr /*n x 9*/,
                       double* Fnl /*n x 8*/, double* Fnr /*n x 8*/, double* Az /*n*/,
                       const double* normf /*n x 2*/, const int32_t* sign_l, const int32_t* sign_r,
                       double* eigv /*n*/);
int getifluxvectors_gpu(int32_t n, double gam, const double* Qi /*n x 8*/, double* Fi /*n x 8*/,
                        double* Gi /*n x 8*/);
int getvfluxvectors_gpu(int32_t n, double gam, double mu, double eta0, const double* Qv /*n x 9*/,
                        const double* nablaQ /*n x 18, (9,2) per point*/, double* Fv /*n x 9*/,
                        double* Gv /*n x 9*/);
/* getVfluxvectors_AV(Qv,nablaQ,Fv,Gv,fam,ifp,jfp,ic) (getrusanov.f90:251-360) over n
 * points of a bound solve: mu_art interpolated at flux point (ifp,jfp) of family fam
 * (1 or 2) of cell ic, all 1-based as in the reference, from the face AV viscosities
 * muAVfi/muAVfj that the context's last residual evaluation left (:273-281);
 * eta_art = 0.  Out-of-range indices return CHORUS_EINVAL before any device work. */
int getvfluxvectors_av_gpu(ChorusCtx* ctx, int32_t n, const double* Qv /*n x 9*/,
                           const double* nablaQ /*n x 18*/, double* Fv /*n x 9*/, double* Gv /*n x 9*/,
                           const int32_t* fam, const int32_t* ifp, const int32_t* jfp, const int32_t* ic);
/* Single-point forms with the reference's own argument lists (all by reference, as a
 * Fortran CALL passes them), for unit tests written against the reference routines:
 * getrusanovflux(Qfl,Qfr,Fnl,Fnr,Az,normf,sign_l,sign_r,eigv) plus the module variable
 * eigvmax it raises (getrusanov.f90:1-109), getIfluxvectors(Qi,Fi,Gi) (:111-153),
 * getVfluxvectors(Qv,nablaQ,Fv,Gv) (:157-249), getVfluxvectors_AV(...,fam,ifp,jfp,ic)
 * (:251-360, with the bound solve standing in for the module's muAVfi/muAVfj).  gam, mu
 * and eta0, module state in the reference (setup2d.f90:68,72,77), are set process-wide by
 * chorus_point_set_params (defaults 5/3, 0, 0).  They evaluate on the device. */
int chorus_point_set_params(double gam, double mu, double eta0);
int getrusanovflux_c(const double* Qfl, const double* Qfr, double* Fnl, double* Fnr, double* Az,
                     const double* normf, const int32_t* sign_l, const int32_t* sign_r, double* eigv,
                     double* eigvmax);
int getifluxvectors_c(const double* Qi, double* Fi, double* Gi);
int getvfluxvectors_c(const double* Qv, const double* nablaQ, double* Fv, double* Gv);
int getvfluxvectors_av_c(ChorusCtx* ctx, const double* Qv, const double* nablaQ, double* Fv, double* Gv,
                         const int32_t* fam, const int32_t* ifp, const int32_t* jfp, const int32_t* ic);
/* getrusanovflux_gpu for callers that cannot allocate device memory (no counterpart in
 * the reference): a host whose device memory is all held by its own pool, or one with
 * work in flight that a cudaFree would stall.  Same arguments and results; the device
 * staging lives in a fixed 10 MiB array inside the library, so n is limited to 32768
 * points per call (larger n returns CHORUS_EINVAL) and no cudaMalloc/cudaFree is made.
 * The first call on a device does its set-up: it looks up the array's address and
 * creates the non-blocking stream the copies and the kernel run on, and under CUDA's
 * lazy module loading that is also when the 10 MiB are reserved -- so it needs that much
 * free device memory.  A call with n = 0 does the set-up alone: a host that hands all
 * its device memory to a pool makes it first; make it before any stream capture.  A
 * CUDA error drops the set-up (the next call redoes it); calls after cudaDeviceReset
 * without such an error are not supported.  All calls share the array: calls that
 * overlap on the GPU race. */
int getrusanovflux_noalloc_gpu(int32_t n, double gam, const double* Qfl, const double* Qfr, double* Fnl,
                               double* Fnr, double* Az, const double* normf, const int32_t* sign_l,
                               const int32_t* sign_r, double* eigv);

/* ------------------------------------------------------------------------------
 * Runtime helpers (no reference counterpart)
 * --------------------------------------------------------------------------- */
/* The CUDA stream (cudaStream_t) all of ctx's work is enqueued on, so callers can
 * record events on it or order their own work after it. */
void* chorus_gpu_stream(ChorusCtx* ctx);
/* Run `reps` RK stages (stage 1 of RK_S5P3, state updated) launching each stage
 * kernel with CUDA events around it; ms[0..4] = mean duration of E1, F1, E2, F2, E3
 * and ms[5] = mean duration of a whole stage. */
int chorus_gpu_profile_stage(ChorusCtx* ctx, int32_t reps, double* ms);
/* Runtime options of a context:
 *   "diagnostics" (default 1): compute the norms of every tenth step in iterations_gpu;
 *   "skip_inactive_viscous" (default 1): with mu = eta0 = 0 the viscous flux at a flux
 *       point is exactly zero unless an adjacent face carries AV viscosity, and a cell's
 *       gradients are needed only within two face rings of an AV-active cell; skip that
 *       work (results are unchanged).  0 computes every cell (and fills every gradient
 *       array for inspection).
 *   "plot_sensor" (default 0): the last stage of each step also records the AV sensor
 *       of variable 6, which only the plot output reads (about 1% of a step); takes
 *       effect on the stream in order, without rebuilding the step graphs;
 *   "host_chunks" (1..32, default 16): chunks of cells in which chorus_gpu_step_host
 *       copies a state of 64 MB or more, each chunk's copy overlapped with the passes
 *       that can run on it (fewer for meshes under 1024 cells per chunk);
 *   "epb_e1" / "epb_e2" / "epb_e3" / "epb_ct" (1..64): cells per CTA of a cell pass;
 *   "threads_e1" / "threads_e2" / "threads_e3" (32..512) and "threads_ct" (32..256), multiples of 32:
 *       threads per CTA.
 * chorus_gpu_get_option returns the current value (-1 for an unknown name); the extra
 * read-only name "skip_active" tells whether skipping is in effect. */
int chorus_gpu_set_option(ChorusCtx* ctx, const char* name, int64_t value);
int64_t chorus_gpu_get_option(ChorusCtx* ctx, const char* name);
/* Kernel launches enqueued by one time step (5 stages + CT projection) and by the
 * extra diagnostic of every tenth step. */
int chorus_gpu_launch_counts(ChorusCtx* ctx, int32_t* per_step, int32_t* per_diag);
/* Device bytes held by ctx (state, work arrays, geometry). */
int64_t chorus_gpu_device_bytes(ChorusCtx* ctx);
/* The FP64 pipe's measured fused multiply-add rate on `device` (FMA per second; each FMA
 * is two flops): independent fma chains over 64 warps per SM, timed with CUDA events
 * after a warm-up launch.  *ms = the timed launches' duration (may be NULL).  The
 * residual path's FP64 instruction rate is reported against it. */
int chorus_gpu_fp64_fma_peak(int32_t device, double* fma_per_s, double* ms);

/* ------------------------------------------------------------------------------
 * Batched form: many independent solves (any N, size, problem, dt) advanced together,
 * one persistent launch per pass over a per-cell work table.  A solve's results are
 * the same alone and in a batch.  No reference counterpart (the reference runs one
 * solve per MPI job).
 * --------------------------------------------------------------------------- */
int chorus_batch_create(int32_t device, ChorusBatch** batch);
int chorus_batch_free(ChorusBatch* batch);
/* Add a bound context (its state stays where it is; the caller keeps ownership and
 * must not free it while it is in the batch).  *slot receives the solve's slot. */
int chorus_batch_add(ChorusBatch* batch, ChorusCtx* ctx, int32_t* slot);
int chorus_batch_remove(ChorusBatch* batch, int32_t slot);
/* Enqueue nsteps time steps (5 RK stages + CT projection, no norms) of every solve in
 * the batch, replayed from one CUDA graph; returns without waiting. */
int chorus_batch_step(ChorusBatch* batch, int32_t nsteps);
/* Wait for the batch and check the per-solve error flags (*err_slot = failing slot). */
int chorus_batch_sync(ChorusBatch* batch, int32_t* err_slot);
int chorus_batch_stream(ChorusBatch* batch, void** stream);
int chorus_batch_info(ChorusBatch* batch, int32_t* n_solves, int32_t* cell_tiles, int32_t* face_tiles,
                      int64_t* dofs);

/* ------------------------------------------------------------------------------
 * Serving form: a request loop with continuous batching (no reference counterpart).
 * Requests arrive over time; at every step boundary the loop admits arrived requests
 * in order while their device memory fits hbm_budget_bytes, sets each up (mesh maps,
 * binding, initial state) while the previous step runs, packs all admitted solves into
 * one batch step, and retires a solve after ceil(end_time/dt) steps.  mode 1 runs the
 * plain sequential loop instead (one solve at a time, first come first served).
 * --------------------------------------------------------------------------- */
typedef struct ChorusServeRequest {
  const char* case_dir; /* QUAD.INP + mesh files */
  double arrival_s;     /* seconds after the start of the run (sorted ascending) */
  double end_time;      /* physical end time of the solve */
  /* Results of the solve (each may be NULL):
   *   Q_out        receives the final state Q(9,N,N,NCELL) in the reference layout when the
   *                solve retires; Q_out_count must then equal 9*N*N*NCELL (else the request
   *                fails with CHORUS_EINVAL before any device work);
   *   restart_path receives the final state as the restart stream of write_data.f90:44-74
   *                (iter = steps run, ctime = their sum of dt), readable by
   *                chorus_read_restart and by the reference's READ_ALL_DATA_BINARY. */
  double* Q_out;
  int64_t Q_out_count;
  const char* restart_path;
} ChorusServeRequest;
typedef struct ChorusServeConfig {
  int32_t device;
  int32_t mode;              /* 0 continuous batching, 1 plain sequential */
  int64_t hbm_budget_bytes;  /* 0 = no limit */
  int32_t max_active;        /* 0 = no limit */
  int32_t gpu_setup;         /* 1: build each request's maps and geometry on the device
                                (chorus_mesh_load_gpu), 0: on the host */
} ChorusServeConfig;
typedef struct ChorusServeResult {
  double admit_s, finish_s, latency_s; /* seconds since start; latency = finish - arrival */
  double wait_s;  /* time an arrived request waited for device memory (admission control) */
  double ctime;   /* physical time reached: steps x dt, accumulated as the reference does */
  int64_t dof;
  int32_t steps;
  int32_t status; /* CHORUS_OK or the error of that request */
} ChorusServeResult;
int chorus_serve_run(const ChorusServeRequest* reqs, int32_t n, const ChorusServeConfig* cfg,
                     ChorusServeResult* results, double* makespan_s);
/* Device bytes chorus_gpu_bind_mesh would allocate for this mesh (admission control). */
int64_t chorus_mesh_device_bytes(const ChorusMesh* mesh);
/* The chunk plan chorus_gpu_step_host follows for this mesh with the option host_chunks =
 * chunks (host only; for inspection and tests): *K chunks of cells [cut[k], cut[k+1])
 * (K+1 entries, at most 33); the two-sided faces [f2cut[k], f2cut[k+1]) of the face list in
 * the order of its larger cell, i.e. those whose larger cell is in chunk k, and the FREE
 * faces [f1cut[k], f1cut[k+1]) in cell order; *nseg download runs (at most 66) as
 * seg[3i], seg[3i+1], seg[3i+2] = first cell, end cell, and the chunk after whose last-stage
 * passes all of the run's cells and their face neighbours are final. */
int chorus_mesh_host_chunks(const ChorusMesh* mesh, int32_t chunks, int32_t* K, int32_t* cut, int32_t* f2cut,
                            int32_t* f1cut, int32_t* nseg, int32_t* seg);

/* ------------------------------------------------------------------------------
 * Host-side setup for callers without the Fortran setup chain: reads QUAD.INP and
 * the .CEL/.VRT/.BND files and rebuilds the reference's maps (readinput.f90,
 * readGRIDinfo.f90, CHECK_MESH/CONNECTIVITY connectivity.f90, CONNECT_BDRY
 * connect_bdry.f90, MAPCYCLOC map_cyc_loc.f90) and geometry (initsetup.f90,
 * mapder.f90, calcjacob.f90).  The integer maps are bit-identical to the
 * reference's; the geometry follows its evaluation order.
 * --------------------------------------------------------------------------- */
int chorus_mesh_load(const char* case_dir, ChorusMesh** mesh);
/* chorus_mesh_load with the map building and the geometry on `device`: the files are
 * parsed on the host; CHECK_MESH, CONNECTIVITY (an edge hash table and a scan give the
 * reference's face numbering), the boundary lookups, IBFINTER and mapder/calcjacob run
 * as kernels, MAPCYCLOC on the host.  Every array is bit-identical to chorus_mesh_load's;
 * a mesh the kernels find invalid is rebuilt on the host, which returns the reference's
 * error for it.  Allocates and frees temporary device memory. */
int chorus_mesh_load_gpu(const char* case_dir, int32_t device, ChorusMesh** mesh);
int chorus_mesh_free(ChorusMesh* mesh);
/* dims/params as read; *maxiter = MAXITER, *problem = 0 OT, 1 rotor, 2 Alfven. */
int chorus_mesh_info(const ChorusMesh* mesh, ChorusDims* dims, ChorusParams* params, int32_t* maxiter,
                     int32_t* problem);
/* Named arrays: int -- IF2C IC2F IF2V IVCELL IBFINTER IBFREE IBFCYC IBFCYCLOC CYC2FPAIR
 * iface2fp jface2fp; double -- XV YV Xs Xf Lmat Mmat S1 S2 Jac XXsolu. */
const int32_t* chorus_mesh_iarray(const ChorusMesh* mesh, const char* name, int64_t* count);
const double* chorus_mesh_darray(const ChorusMesh* mesh, const char* name, int64_t* count);
/* Bind a loaded mesh (chorus_gpu_bind with the mesh's arrays). */
int chorus_gpu_bind_mesh(const ChorusMesh* mesh, int32_t device, ChorusCtx** ctx);
/* SETINITIALCOND (setinitialcond.f90:1-80): analytic data at the solution points,
 * CT projection on the device, energy rebuilt from the projected B; the state is
 * left resident in ctx and also returned in Q (may be NULL). */
int chorus_initial_state(const ChorusMesh* mesh, ChorusCtx* ctx, double* Q);

/* Restart stream of write_data.f90:5-83 / read_data_restart.f90:35-67: int32 iter,
 * float64 ctime, then per cell int32 global id + Q(9,N,N). */
int chorus_write_restart(ChorusCtx* ctx, const char* path, int32_t iter, double ctime);
int chorus_read_restart(ChorusCtx* ctx, const char* path, int32_t* iter, double* ctime);

/* ------------------------------------------------------------------------------
 * Plot output (iterations.f90:80-84 for one partition): tecplotter2dsetup
 * (tecplotter2dsetup.f90:1-177) on the host at create, tecplotter2d
 * (tecplotter.f90:1-86) on the device at every evaluation, tecpost_parallel
 * (tecplotter.f90:92-418) as a headless file write.  The node values use the Q of the
 * bound solve and the muAV(1), muAV(6) of its last stage.  muAV(6) needs the sensor of
 * variable 6, which only the plot reads: the last stage of a step (and compresid_gpu)
 * records it while the context option "plot_sensor" is 1, so set it before the step that
 * precedes an output; evaluating a plot otherwise returns CHORUS_ESTATE.  With ARTIV = 0
 * the reference never allocates muAV; the muAV/etaAV fields are zeros here.
 * --------------------------------------------------------------------------- */
typedef struct ChorusPlot ChorusPlot;
/* IVCELL(NCELL,4), IC2F(NCELL,4) 1-based, XV/YV(NVERT), Xs(N) as in the reference;
 * NRE sub-intervals per cell edge (readinput.f90:32). */
int chorus_plot_create(ChorusCtx* ctx, const int32_t* IVCELL, const int32_t* IC2F, const double* XV,
                       const double* YV, int32_t NVERT, int32_t NFACE, const double* Xs, int32_t NRE,
                       ChorusPlot** plot);
/* the same from a loaded case; NRE <= 0 takes the case file's NRE.  A plot refers to
 * its context: free the plot before the context. */
int chorus_plot_create_mesh(ChorusCtx* ctx, const ChorusMesh* mesh, int32_t NRE, ChorusPlot** plot);
int chorus_plot_free(ChorusPlot* plot);
/* plotnodes, plotcells; warned = 1 where the reference prints its 'something wrong'
 * checks (tecplotter2dsetup.f90:54-56, :99-106) */
int chorus_plot_info(const ChorusPlot* plot, int64_t* nodes, int64_t* cells, int32_t* warned);
/* evaluate on the device and copy out (any pointer may be NULL): plotX(2,nodes),
 * plotQ(9,nodes) = rho u v w p Bx By Bz Az, plotAV(2,nodes) = muAV etaAV,
 * connec(4,cells) 1-based, gnode_factor(nodes) */
int chorus_plot_values(ChorusPlot* plot, double* plotX, double* plotQ, double* plotAV, int32_t* connec,
                       int32_t* gnode_factor);
/* 'TEC' // i7.7 int(ctime) // the f6.3 fraction without its integer digit // '.plt' */
int chorus_plot_filename(double ctime, char* buf, int32_t n);
/* evaluate and write dir/<chorus_plot_filename(ctime)>: #!TDV111, one
 * FEQUADRILATERAL zone, 13 float32 variables in block packing, 0-based connectivity;
 * the written path goes to path_out when given */
int chorus_plot_write(ChorusPlot* plot, double ctime, const char* dir, char* path_out, int32_t path_len);
/* NRE and nwrite of a loaded case (readinput.f90:32-33) */
int chorus_mesh_output_info(const ChorusMesh* mesh, int32_t* nre, int32_t* nwrite);

#ifdef __cplusplus
}
#endif
#endif
