/*
 * chorus_oracle.h -- CPU oracle for the CHORUS-MHD residual-and-time-step path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, loop-for-loop restatement of the
 * reference's Fortran (setup2d module state, mesh/map setup, compresid/compflux,
 * Rusanov/BC/cyclic fluxes, artificial viscosity, magnetic potential, SSP-RK),
 * used as the checker for the CUDA path and as the timed CPU baseline.  Nothing
 * in the product library links or calls it.
 *
 * Parity status: the reference ships no golden vectors, tests or fixtures and no
 * Fortran compiler exists on either build machine, so the restatement is pinned
 * only by analytic known answers (Chebyshev/Legendre point formulas, Lagrange
 * operator identities, free-stream preservation, exact Orszag-Tang data) --
 * parity against the reference binary itself is UNPINNED.
 *
 * Arrays keep the reference's Fortran layout (column-major, first index fastest)
 * and integer maps keep its 1-based values, so they can be compared element by
 * element with the CUDA path and passed straight to the C-ABI.
 */
#ifndef CHORUS_ORACLE_H
#define CHORUS_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc orc_t;

/* Load QUAD.INP + mesh files from `dir` and run the reference's setup sequence
 * (main.f90:16-44).  Returns NULL and fills err on failure. */
orc_t* orc_load(const char* dir, char* err, int errlen);
void orc_free(orc_t* o);

/* Scalars: N, NCELL, NFACE, NINTER, NFREE, NPAIR, NCYCL, NVERT, k_stage, MAXITER,
 * vismode, ARTIV, iter, problem. */
int orc_geti(const orc_t* o, const char* name);
/* Scalars: dt, ctime, mu, eta0, gam, DXCYCL, DYCYCL, eigvmax, eigvmax_g, epsilon0,
 * B0x, B0y. */
double orc_getd(const orc_t* o, const char* name);
int orc_setd(orc_t* o, const char* name, double v);
int orc_seti(orc_t* o, const char* name, int v);

/* Raw pointer + element count of a named array (Fortran layout).
 * double arrays: Q resid F1 G2 Fv1 Gv2 Qvfi Qvfj nablaQs nablaQvfi nablaQvfj Azfi
 *   Azfj nablaAs S1 S2 Jac Lmat Mmat Xs Xf XV YV muAV muAVfi muAVfj SM_IND XXsolu
 * int arrays: IF2C IC2F IF2V IVCELL IBFINTER IBFREE IBFCYC IBFCYCLOC CYC2FPAIR
 *   iface2fp jface2fp */
double* orc_darray(orc_t* o, const char* name, int64_t* count);
int32_t* orc_iarray(orc_t* o, const char* name, int64_t* count);

/* Hot-path entry points (names follow the reference routines). */
void orc_compresid(orc_t* o);                /* compresid.f90:1 */
void orc_compflux(orc_t* o);                 /* compflux.f90:1 */
void orc_comp_inviscid_flux(orc_t* o);       /* compflux.f90:33 */
void orc_nablaQsp(orc_t* o, int v_sta, int v_end); /* compflux.f90:107 (1-based) */
void orc_correct_B_via_curl_Az(orc_t* o);    /* setinitialcond.f90:82 */
void orc_rk_s5p3(orc_t* o);                  /* iterations.f90:162 */
void orc_fivestagerk(orc_t* o);              /* iterations.f90:92 */

/* One iteration of iterations.f90:19-87 (RK step, CT correction, diagnostic
 * flux+gradient, norms when mod(iter,10)==1).  Returns 1 if norms were computed and
 * stores them in *residglob / *divBglob. */
int orc_step(orc_t* o, double* residglob, double* divBglob);
/* n steps; returns number of steps run. */
int orc_run(orc_t* o, int nsteps);

/* Restart stream (write_data.f90:5-83, read_data_restart.f90:35-67). */
int orc_write_restart(const orc_t* o, const char* path);
int orc_read_restart(orc_t* o, const char* path);

/* Plot output for one rank (tecplotter2dsetup.f90:1-177, tecplotter.f90:1-418):
 * plot nodes with NRE sub-intervals per cell edge (0 = ok, 1 = the reference's
 * 'something wrong' warnings fired), node values from the current Q and muAV, the
 * reference's file name for ctime, and the Tecplot binary file.  Arrays afterwards:
 * plotX(2,n) plotQ(9,n) plotAV(2,n), gnumnode(NRE+1,NRE+1,NCELL) gnode_factor(n)
 * connec_c2n(4,cells) (1-based). */
int orc_plot_setup(orc_t* o, int nre);
int orc_plot_eval(orc_t* o);
int orc_plot_filename(double ctime, char* out, int n);
int orc_plot_write(const orc_t* o, double ctime, const char* path);

/* Number of OpenMP threads used by cell/face loops (1 when built without OpenMP). */
int orc_set_threads(int n);

/* Point functions with the reference argument lists (getrusanov.f90). */
void orc_getrusanovflux(double gam, const double Qfl[9], const double Qfr[9],
                        double Fnl[8], double Fnr[8], double* Az, const double normf[2],
                        int sign_l, int sign_r, double* eigv, double* eigvmax);
void orc_getifluxvectors(double gam, const double Qi[8], double Fi[8], double Gi[8]);
void orc_getvfluxvectors(double gam, double mu, double eta0, const double Qv[9],
                         const double nablaQ[18], double Fv[9], double Gv[9]);

#ifdef __cplusplus
}
#endif
#endif
