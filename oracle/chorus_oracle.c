/*
 * chorus_oracle.c -- CPU oracle: plain-C restatement of CHORUS-MHD's setup and
 * residual-and-time-step path, loop for loop and in the reference's evaluation
 * order (built with -O2 -ffp-contract=off, no fast-math, glibc libm).
 *
 * TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
 * checker, and by bench.py's CPU-baseline leg.  The product library never links it.
 *
 * Parity status: pinned by analytic known answers only; UNPINNED against the
 * reference binary (no Fortran compiler on either machine, no golden data in the
 * reference).
 *
 * Each function cites the reference routine it restates (file:line, paths within
 * the reference project).  Extensions beyond the reference are marked EXTENSION:
 * runtime gamma (setup2d.f90:68 has it as a compile-time parameter), the rotor and
 * Alfven-wave initial conditions, and a uniform background field B0 for A_z
 * (B = B0 + curl dA_z); with the defaults (gamma=5/3, Orszag-Tang, B0=0) every
 * operation reduces to the reference's exactly.
 */
#include "chorus_oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NV 9
static const double PI = 3.14159265358979323846; /* atan(1.d0)*4.d0, setup2d.f90:67 */
static const double LAMBDA = -2.0 / 3.0;        /* setup2d.f90:70 */
static const double PRANDT = 0.72;              /* setup2d.f90:71 */
static const double TOLCYC = 1e-5;              /* setup2d.f90:64 */

struct orc {
  /* input (readinput.f90:6-36) */
  char namecel[1400], namevrt[1400], namebnd[1400], namerestart[1400];
  int N, CURVE_WALL, vismode, k_stage, MAXITER, ARTIV, NRE, nwrite, restart, restart_ord;
  double mu, eta0, dt, DXCYCL, DYCYCL;
  /* EXTENSION parameters */
  double gam, B0x, B0y;
  int problem; /* 0 Orszag-Tang (reference), 1 rotor, 2 Alfven wave */
  /* mesh */
  int NCELLGLOB, NVERTGLOB, NBOUNDEFINED, NCELL, NVERT, NFACE;
  int NINTER, NFREE, NCYCL, NCYCLOC, NCYCREM, NPAIR, NPROCINT, NINLET, NOUTLET, NSYMP, NWALL;
  int *IVCELL;       /* (NCELL,4) */
  double *XV, *YV;   /* local vertices */
  int *IVGBOUN;      /* (NBOUNDEFINED,2) global vertex ids */
  char (*IBOUNTYPE)[9];
  int *IVG2IV;
  int *ICVSTA, *ICVERT;
  int *IC2F, *IF2C, *IF2V; /* (NCELL,4) (NFACE,4) (NFACE,2) */
  int *IBFINTER, *IBFREE, *IBFCYC, *IBFCYCLOC, *CYC2FPAIR;
  int iface2fp[4 * 16], jface2fp[4 * 16]; /* (N,4) with N<=16 */
  /* SD operators */
  double *Xs, *Xf, *Lmat, *Mmat, *Xs_low, *Xf_low;
  double *dmdxs, *dmdxf1, *dmdxf2;
  double *Jac, *S1, *S2, *XXsolu;
  /* state and work arrays */
  double *Q, *F1, *G2, *Fv1, *Gv2, *resid, *Qvfi, *Qvfj;
  double *nablaQs, *nablaQvfi, *nablaQvfj, *Azfi, *Azfj, *nablaAs;
  double *muAV, *muAVfi, *muAVfj, *SM_IND;
  double *Qk0, *Qka, *qj2, *qj3, *resid0;
  double ctime, eigvmax, eigvmax_g, epsilon0;
  int iter;
  /* plot output (tecplotter2dsetup.f90, tecplotter.f90) */
  int plot_nre, plotnodes, plotcells;
  int *gnumnode, *gnode_factor, *connec_c2n;
  double *plotX, *plotQ, *plotAV;
};

/* ---------- index helpers (0-based, Fortran column-major) ---------- */
#define IDX_Q(o, k, is, js, ic) ((k) + NV * ((is) + (o)->N * ((js) + (o)->N * (int64_t)(ic))))
#define IDX_FI(o, nv, k, ifp, jfp, ic) ((k) + (nv) * ((ifp) + ((o)->N + 1) * ((jfp) + (o)->N * (int64_t)(ic))))
#define IDX_FJ(o, nv, k, ifp, jfp, ic) ((k) + (nv) * ((ifp) + (o)->N * ((jfp) + ((o)->N + 1) * (int64_t)(ic))))
#define IDX_NQS(o, k, d, is, js, ic) ((k) + NV * ((d) + 2 * ((is) + (o)->N * ((js) + (o)->N * (int64_t)(ic)))))
#define IDX_NQI(o, k, d, ifp, jfp, ic) ((k) + NV * ((d) + 2 * ((ifp) + ((o)->N + 1) * ((jfp) + (o)->N * (int64_t)(ic)))))
#define IDX_NQJ(o, k, d, ifp, jfp, ic) ((k) + NV * ((d) + 2 * ((ifp) + (o)->N * ((jfp) + ((o)->N + 1) * (int64_t)(ic)))))
#define IDX_S1(o, a, b, ifp, jfp, ic) ((a) + 2 * ((b) + 2 * ((ifp) + ((o)->N + 1) * ((jfp) + (o)->N * (int64_t)(ic)))))
#define IDX_S2(o, a, b, ifp, jfp, ic) ((a) + 2 * ((b) + 2 * ((ifp) + (o)->N * ((jfp) + ((o)->N + 1) * (int64_t)(ic)))))
#define IDX_J(o, is, js, ic) ((is) + (o)->N * ((js) + (o)->N * (int64_t)(ic)))
#define IDX_AI(o, ifp, jfp, ic) ((ifp) + ((o)->N + 1) * ((jfp) + (o)->N * (int64_t)(ic)))
#define IDX_AJ(o, ifp, jfp, ic) ((ifp) + (o)->N * ((jfp) + ((o)->N + 1) * (int64_t)(ic)))
#define LM(o, ifp, is) ((ifp) + ((o)->N + 1) * (is))
/* integer maps stored column-major with 1-based values */
#define IVCELL_(o, ic, k) ((o)->IVCELL[(ic) + (o)->NCELL * (k)])
#define IC2F_(o, ic, k) ((o)->IC2F[(ic) + (o)->NCELL * (k)])
#define IF2C_(o, f, k) ((o)->IF2C[(f) + (o)->NFACE * (k)])
#define IF2V_(o, f, k) ((o)->IF2V[(f) + (o)->NFACE * (k)])
#define IFACE2FP(o, nfp, f) ((o)->iface2fp[(nfp) + (o)->N * (f)])
#define JFACE2FP(o, nfp, f) ((o)->jface2fp[(nfp) + (o)->N * (f)])

static double* dalloc(int64_t n) { double* p = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); return p; }
static int* ialloc(int64_t n) { int* p = (int*)calloc((size_t)(n > 0 ? n : 1), sizeof(int)); return p; }

static int g_threads = 1;
int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n < 1) n = omp_get_max_threads();
  g_threads = n;
  return n;
#else
  (void)n;
  g_threads = 1;
  return 1;
#endif
}

/* =====================================================================
 * Input (readinput.f90:1-41, readGRIDinfo.f90:1-259)
 * ===================================================================== */
static int read_line(FILE* f, char* buf, int n) {
  if (!fgets(buf, n, f)) return 0;
  return 1;
}
static void first_token(const char* line, char* out, int n) {
  while (*line && isspace((unsigned char)*line)) line++;
  int i = 0;
  if (*line == '\'' || *line == '"') {
    char q = *line++;
    while (*line && *line != q && i < n - 1) out[i++] = *line++;
  } else {
    while (*line && !isspace((unsigned char)*line) && *line != ',' && i < n - 1) out[i++] = *line++;
  }
  out[i] = 0;
}
/* Fortran list-directed real: accept D/d exponents. */
static double fortran_real(const char* s) {
  char tmp[128];
  int i = 0;
  while (*s && isspace((unsigned char)*s)) s++;
  while (*s && !isspace((unsigned char)*s) && *s != ',' && i < 127) {
    char c = *s++;
    tmp[i++] = (c == 'D' || c == 'd') ? 'E' : c;
  }
  tmp[i] = 0;
  return strtod(tmp, NULL);
}

static int readinput(orc_t* o, const char* dir, char* err, int errlen) {
  char path[1100], line[1024], tok[256];
  snprintf(path, sizeof path, "%s/QUAD.INP", dir);
  FILE* f = fopen(path, "r");
  if (!f) { snprintf(err, errlen, "cannot open %s", path); return -1; }
  char lines[40][1024];
  int nl = 0;
  while (nl < 40 && read_line(f, line, sizeof line)) { strcpy(lines[nl++], line); }
  fclose(f);
  if (nl < 29) { snprintf(err, errlen, "QUAD.INP has %d lines, need 29", nl); return -1; }
  first_token(lines[2], tok, sizeof tok); snprintf(o->namecel, sizeof o->namecel, "%s/%s", dir, tok);
  first_token(lines[3], tok, sizeof tok); snprintf(o->namevrt, sizeof o->namevrt, "%s/%s", dir, tok);
  first_token(lines[5], tok, sizeof tok); snprintf(o->namebnd, sizeof o->namebnd, "%s/%s", dir, tok);
  first_token(lines[7], tok, sizeof tok); snprintf(o->namerestart, sizeof o->namerestart, "%s/%s", dir, tok);
  o->N = atoi(lines[9]);
  o->CURVE_WALL = atoi(lines[10]);
  o->vismode = atoi(lines[11]);
  o->mu = fortran_real(lines[12]);
  o->eta0 = fortran_real(lines[13]);
  o->k_stage = atoi(lines[15]);
  o->dt = fortran_real(lines[16]);
  o->MAXITER = atoi(lines[17]);
  o->DXCYCL = fortran_real(lines[19]);
  o->DYCYCL = fortran_real(lines[20]);
  o->ARTIV = atoi(lines[22]);
  o->NRE = atoi(lines[24]);
  o->nwrite = atoi(lines[25]);
  o->restart = atoi(lines[27]);
  o->restart_ord = atoi(lines[28]);
  /* EXTENSION block (lines 31-34): gamma, problem id, B0x, B0y */
  o->gam = 5.0 / 3;
  o->problem = 0;
  o->B0x = 0.0;
  o->B0y = 0.0;
  if (nl >= 31) o->gam = fortran_real(lines[30]);
  if (nl >= 32) o->problem = atoi(lines[31]);
  if (nl >= 33) o->B0x = fortran_real(lines[32]);
  if (nl >= 34) o->B0y = fortran_real(lines[33]);
  if (o->N < 2 || o->N > 10) { snprintf(err, errlen, "N=%d outside 2..10", o->N); return -1; }
  if (o->CURVE_WALL != 0) { snprintf(err, errlen, "CURVE_WALL=1 is unfinished in the reference"); return -1; }
  return 0;
}

static int count_lines(const char* path) {
  FILE* f = fopen(path, "r");
  if (!f) return -1;
  int n = 0, c, last = '\n';
  while ((c = fgetc(f)) != EOF) { if (c == '\n') n++; last = c; }
  if (last != '\n') n++;
  fclose(f);
  return n;
}

/* READ_CELL_DATA readGRIDinfo.f90:1-37, READ_VRT_DATA :40-85, READ_METIS :87-121
 * (one rank: NCELL=NCELLGLOB), GLOB2LOCAL :124-199, READ_BND_DATA :201-259 */
static int read_grid(orc_t* o, char* err, int errlen) {
  int n = count_lines(o->namecel);
  if (n <= 0) { snprintf(err, errlen, "cannot read %s", o->namecel); return -1; }
  o->NCELLGLOB = n;
  int* IVGCELLG = ialloc((int64_t)n * 4);
  FILE* f = fopen(o->namecel, "r");
  for (int i = 0; i < n; i++) {
    int ic, v[4], t, k;
    if (fscanf(f, "%d %d %d %d %d %d %d", &ic, &v[0], &v[1], &v[2], &v[3], &t, &k) != 7) {
      snprintf(err, errlen, "bad cell line %d", i + 1); fclose(f); free(IVGCELLG); return -1;
    }
    for (int q = 0; q < 4; q++) IVGCELLG[i + n * q] = v[q];
  }
  fclose(f);
  int nv = count_lines(o->namevrt);
  if (nv <= 0) { snprintf(err, errlen, "cannot read %s", o->namevrt); free(IVGCELLG); return -1; }
  o->NVERTGLOB = nv;
  double *XVG = dalloc(nv), *YVG = dalloc(nv);
  f = fopen(o->namevrt, "r");
  char line[512];
  for (int i = 0; i < nv; i++) {
    if (!fgets(line, sizeof line, f)) { snprintf(err, errlen, "short vrt file"); fclose(f); return -1; }
    /* FORMAT(I9,6X,3(D20.12,1X)) readGRIDinfo.f90:79-80 */
    char fx[21], fy[21];
    size_t L = strlen(line);
    if (L < 15 + 20 + 1 + 20) { snprintf(err, errlen, "short vrt line %d", i + 1); fclose(f); return -1; }
    memcpy(fx, line + 15, 20); fx[20] = 0;
    memcpy(fy, line + 36, 20); fy[20] = 0;
    for (int q = 0; q < 20; q++) { if (fx[q] == 'D' || fx[q] == 'd') fx[q] = 'E'; if (fy[q] == 'D' || fy[q] == 'd') fy[q] = 'E'; }
    XVG[i] = strtod(fx, NULL);
    YVG[i] = strtod(fy, NULL);
  }
  fclose(f);
  /* GLOB2LOCAL: local vertex ids in order of first appearance (cell-major). */
  o->NCELL = o->NCELLGLOB;
  o->IVCELL = ialloc((int64_t)o->NCELL * 4);
  o->IVG2IV = ialloc(nv + 1);
  double *XVt = dalloc(4 * (int64_t)o->NCELL), *YVt = dalloc(4 * (int64_t)o->NCELL);
  int ivnew = 0;
  for (int ic = 0; ic < o->NCELLGLOB; ic++) {
    for (int iv = 0; iv < 4; iv++) {
      int ivg = IVGCELLG[ic + n * iv];
      if (ivg < 1 || ivg > nv) { snprintf(err, errlen, "vertex id %d out of range", ivg); return -1; }
      int ivl;
      if (o->IVG2IV[ivg] == 0) {
        ivl = ++ivnew;
        o->IVG2IV[ivg] = ivl;
        XVt[ivl - 1] = XVG[ivg - 1];
        YVt[ivl - 1] = YVG[ivg - 1];
      } else {
        ivl = o->IVG2IV[ivg];
      }
      IVCELL_(o, ic, iv) = ivl;
    }
  }
  o->NVERT = ivnew;
  o->XV = dalloc(ivnew);
  o->YV = dalloc(ivnew);
  memcpy(o->XV, XVt, sizeof(double) * ivnew);
  memcpy(o->YV, YVt, sizeof(double) * ivnew);
  free(XVt); free(YVt); free(XVG); free(YVG); free(IVGCELLG);
  /* READ_BND_DATA */
  int nb = count_lines(o->namebnd);
  if (nb < 0) nb = 0;
  o->NBOUNDEFINED = nb;
  o->IVGBOUN = ialloc((int64_t)nb * 2);
  o->IBOUNTYPE = (char(*)[9])calloc(nb > 0 ? nb : 1, 9);
  f = fopen(o->namebnd, "r");
  for (int i = 0; i < nb && f; i++) {
    int ib, a, b, reg, pat;
    char ty[64];
    if (fscanf(f, "%d %d %d %d %d %63s", &ib, &a, &b, &reg, &pat, ty) != 6) {
      snprintf(err, errlen, "bad bnd line %d", i + 1); fclose(f); return -1;
    }
    o->IVGBOUN[i] = a;
    o->IVGBOUN[i + nb] = b;
    char* t = ty;
    if (*t == '\'' || *t == '"') t++;
    snprintf(o->IBOUNTYPE[i], 9, "%.8s", t);
    o->IBOUNTYPE[i][8] = 0;
    for (int q = 0; q < 8; q++) if (o->IBOUNTYPE[i][q] == '\'' || o->IBOUNTYPE[i][q] == '"') o->IBOUNTYPE[i][q] = 0;
  }
  if (f) fclose(f);
  return 0;
}

/* CHECK_MESH connectivity.f90:236-283 (the orientation "fix" is a no-op). */
static int check_mesh(orc_t* o, char* err, int errlen) {
  for (int ic = 0; ic < o->NCELL; ic++) {
    double xs[2][4];
    for (int k = 0; k < 4; k++) {
      int iv = IVCELL_(o, ic, k) - 1;
      xs[0][k] = o->XV[iv];
      xs[1][k] = o->YV[iv];
    }
    double v12[2] = {xs[0][1] - xs[0][0], xs[1][1] - xs[1][0]};
    double v23[2] = {xs[0][2] - xs[0][1], xs[1][2] - xs[1][1]};
    double v34[2] = {xs[0][3] - xs[0][2], xs[1][3] - xs[1][2]};
    double c123 = v12[0] * v23[1] - v12[1] * v23[0];
    double c234 = v23[0] * v34[1] - v23[1] * v34[0];
    if (c123 * c234 < 0) { snprintf(err, errlen, "Problems in the mesh! cell %d", ic + 1); return -1; }
  }
  return 0;
}

static const int IVFACE[4][2] = {{1, 2}, {2, 3}, {3, 4}, {4, 1}}; /* connectivity.f90:73-83 */

/* CONNECTIVITY connectivity.f90:1-233 */
static int connectivity(orc_t* o, char* err, int errlen) {
  int NC = o->NCELL, NVt = o->NVERT, MAXFACE = NC * 4;
  o->IC2F = ialloc((int64_t)NC * 4);
  int *IF2Ct = ialloc((int64_t)MAXFACE * 2), *IF2Vt = ialloc((int64_t)MAXFACE * 2);
  int *IFILL = ialloc(NVt + 1), *IDUMMY = ialloc(NVt + 1);
  o->ICVSTA = ialloc(NVt + 2);
  for (int ic = 0; ic < NC; ic++)
    for (int k = 0; k < 4; k++) IFILL[IVCELL_(o, ic, k)]++;
  for (int iv = 1; iv <= NVt; iv++)
    if (IFILL[iv] == 0) { snprintf(err, errlen, "IFILL = 0 at vertex %d", iv); return -1; }
  int K = 1;
  for (int iv = 1; iv <= NVt; iv++) { o->ICVSTA[iv] = K; IDUMMY[iv] = K; K += IFILL[iv]; }
  o->ICVSTA[NVt + 1] = o->ICVSTA[NVt] + IFILL[NVt];
  o->ICVERT = ialloc(o->ICVSTA[NVt + 1]);
  for (int ic = 0; ic < NC; ic++)
    for (int k = 0; k < 4; k++) {
      int iv = IVCELL_(o, ic, k);
      o->ICVERT[IDUMMY[iv]] = ic + 1;
      IDUMMY[iv]++;
    }
#define IF2CT(f, c) IF2Ct[(f) + MAXFACE * (c)]
#define IF2VT(f, c) IF2Vt[(f) + MAXFACE * (c)]
  int IFACE = 0;
  for (int ic = 1; ic <= NC; ic++) {
    for (int ifa = 1; ifa <= 4; ifa++) {
      int IFACEOLD = IFACE;
      if (IC2F_(o, ic - 1, ifa - 1) != 0) continue;
      int IVBASE = IVCELL_(o, ic - 1, IVFACE[ifa - 1][0] - 1);
      int IV1 = IVCELL_(o, ic - 1, IVFACE[ifa - 1][1] - 1);
      int found = 0;
      for (int k = o->ICVSTA[IVBASE]; k <= o->ICVSTA[IVBASE + 1] - 1 && !found; k++) {
        int ICC = o->ICVERT[k];
        if (ICC == ic) continue;
        for (int iffa = 1; iffa <= 4; iffa++) {
          int IVV1 = IVCELL_(o, ICC - 1, IVFACE[iffa - 1][0] - 1);
          int IVV2 = IVCELL_(o, ICC - 1, IVFACE[iffa - 1][1] - 1);
          int p11 = IVBASE - IVV1, p12 = IVBASE - IVV2, p21 = IV1 - IVV1, p22 = IV1 - IVV2;
          if ((p11 == 0 && p22 == 0) || (p12 == 0 && p21 == 0)) {
            IFACE++;
            IC2F_(o, ICC - 1, iffa - 1) = IFACE;
            IF2VT(IFACE - 1, 0) = IVBASE;
            IF2VT(IFACE - 1, 1) = IV1;
            IF2CT(IFACE - 1, 0) = ic;
            IF2CT(IFACE - 1, 1) = ICC;
            found = 1;
            break;
          }
        }
      }
      if (!found) {
        if (IF2CT(IFACEOLD, 0) == 0) {
          IF2CT(IFACEOLD, 0) = ic;
          IF2CT(IFACEOLD, 1) = 0;
          IFACE = IFACEOLD + 1;
          IF2VT(IFACE - 1, 0) = IVBASE;
          IF2VT(IFACE - 1, 1) = IV1;
        }
      }
      IC2F_(o, ic - 1, ifa - 1) = IFACE;
    }
  }
  o->NFACE = IFACE;
  int NF = IFACE;
  o->IF2C = ialloc((int64_t)NF * 4);
  o->IF2V = ialloc((int64_t)NF * 2);
  for (int f = 0; f < NF; f++) {
    IF2C_(o, f, 0) = IF2CT(f, 0);
    IF2C_(o, f, 1) = IF2CT(f, 1);
    IF2V_(o, f, 0) = IF2VT(f, 0);
    IF2V_(o, f, 1) = IF2VT(f, 1);
  }
  free(IF2Ct); free(IF2Vt); free(IFILL); free(IDUMMY);
#undef IF2CT
#undef IF2VT
  for (int f = 0; f < NF; f++) {
    int ic1 = IF2C_(o, f, 0), ic2 = IF2C_(o, f, 1);
    int iv1 = IF2V_(o, f, 0), iv2 = IF2V_(o, f, 1);
    int a1 = IVCELL_(o, ic1 - 1, 0), a2 = IVCELL_(o, ic1 - 1, 1), a3 = IVCELL_(o, ic1 - 1, 2), a4 = IVCELL_(o, ic1 - 1, 3);
    if (a1 == iv1 && a2 == iv2) IF2C_(o, f, 2) = 1;
    else if (a2 == iv1 && a3 == iv2) IF2C_(o, f, 2) = 2;
    else if (a3 == iv1 && a4 == iv2) IF2C_(o, f, 2) = 3;
    else if (a4 == iv1 && a1 == iv2) IF2C_(o, f, 2) = 4;
    else { snprintf(err, errlen, "Something wrong in connectivity! NF=%d", f + 1); return -1; }
    if (ic2 != 0) {
      int b1 = IVCELL_(o, ic2 - 1, 0), b2 = IVCELL_(o, ic2 - 1, 1), b3 = IVCELL_(o, ic2 - 1, 2), b4 = IVCELL_(o, ic2 - 1, 3);
      if (b2 == iv1 && b1 == iv2) IF2C_(o, f, 3) = 1;
      else if (b3 == iv1 && b2 == iv2) IF2C_(o, f, 3) = 2;
      else if (b4 == iv1 && b3 == iv2) IF2C_(o, f, 3) = 3;
      else if (b1 == iv1 && b4 == iv2) IF2C_(o, f, 3) = 4;
      else { snprintf(err, errlen, "Something wrong in connectivity (right cell)! NF=%d", f + 1); return -1; }
    }
  }
  return 0;
}

/* CONNECT_BDRY connect_bdry.f90:1-354 (single partition). */
static int connect_bdry(orc_t* o, char* err, int errlen) {
  int NF = o->NFACE, NB = o->NBOUNDEFINED;
  int* BOUNFACEINDEX = ialloc(NF);
  int* bface = ialloc(NB > 0 ? NB : 1);
  int cnt[6] = {0, 0, 0, 0, 0, 0};
  static const char* names[6] = {"INLE", "OUTL", "SYMP", "WALL", "CYCL", "FREE"};
  for (int ib = 0; ib < NB; ib++) {
    bface[ib] = 0;
    int ivb1 = o->IVG2IV[o->IVGBOUN[ib]], ivb3 = o->IVG2IV[o->IVGBOUN[ib + NB]];
    if (ivb1 == 0 || ivb3 == 0) continue;
    int icc = 0;
    for (int k1 = o->ICVSTA[ivb1]; k1 <= o->ICVSTA[ivb1 + 1] - 1; k1++)
      for (int k3 = o->ICVSTA[ivb3]; k3 <= o->ICVSTA[ivb3 + 1] - 1; k3++)
        if (o->ICVERT[k1] == o->ICVERT[k3]) icc = o->ICVERT[k1];
    if (icc == 0) continue;
    int ifa;
    for (ifa = 1; ifa <= 4; ifa++) {
      int iv1 = IVCELL_(o, icc - 1, IVFACE[ifa - 1][0] - 1);
      int iv2 = IVCELL_(o, icc - 1, IVFACE[ifa - 1][1] - 1);
      if ((iv1 == ivb1 || iv2 == ivb1) && (iv1 == ivb3 || iv2 == ivb3)) break;
    }
    if (ifa > 4) { snprintf(err, errlen, "boundary face %d not on cell %d", ib + 1, icc); return -1; }
    int K = IC2F_(o, icc - 1, ifa - 1);
    BOUNFACEINDEX[K - 1] = 1;
    bface[ib] = K;
    for (int t = 0; t < 6; t++)
      if (strcmp(o->IBOUNTYPE[ib], names[t]) == 0) cnt[t]++;
  }
  o->NINLET = cnt[0]; o->NOUTLET = cnt[1]; o->NSYMP = cnt[2]; o->NWALL = cnt[3];
  o->NCYCL = cnt[4]; o->NFREE = cnt[5];
  o->IBFCYC = ialloc(o->NCYCL);
  o->IBFREE = ialloc(o->NFREE);
  int nc = 0, nfr = 0;
  for (int ib = 0; ib < NB; ib++) {
    if (bface[ib] == 0) continue;
    if (strcmp(o->IBOUNTYPE[ib], "CYCL") == 0) o->IBFCYC[nc++] = bface[ib];
    if (strcmp(o->IBOUNTYPE[ib], "FREE") == 0) o->IBFREE[nfr++] = bface[ib];
  }
  /* interior faces :228-244 */
  o->NINTER = 0;
  for (int k = 0; k < NF; k++) if (IF2C_(o, k, 1) != 0) o->NINTER++;
  o->IBFINTER = ialloc(o->NINTER);
  int ni = 0;
  for (int k = 0; k < NF; k++) if (IF2C_(o, k, 1) != 0) o->IBFINTER[ni++] = k + 1;
  /* processor faces :248-272 -- must be empty for one partition */
  o->NPROCINT = 0;
  for (int k = 0; k < NF; k++) if (IF2C_(o, k, 1) == 0 && BOUNFACEINDEX[k] == 0) o->NPROCINT++;
  if (o->NPROCINT != 0) { snprintf(err, errlen, "%d boundary faces are missing from the BND file", o->NPROCINT); return -1; }
  /* local vs remote cyclic faces :275-314 */
  o->IBFCYCLOC = ialloc(o->NCYCL);
  o->NCYCLOC = 0;
  o->NCYCREM = 0;
  for (int ib = 0; ib < o->NCYCL; ib++) {
    int K = o->IBFCYC[ib];
    double XFIN = (o->XV[IF2V_(o, K - 1, 0) - 1] + o->XV[IF2V_(o, K - 1, 1) - 1]) / 2;
    double YFIN = (o->YV[IF2V_(o, K - 1, 0) - 1] + o->YV[IF2V_(o, K - 1, 1) - 1]) / 2;
    int local = 0;
    for (int ib2 = 0; ib2 < o->NCYCL; ib2++) {
      int K2 = o->IBFCYC[ib2];
      double XFOU = (o->XV[IF2V_(o, K2 - 1, 0) - 1] + o->XV[IF2V_(o, K2 - 1, 1) - 1]) / 2;
      double YFOU = (o->YV[IF2V_(o, K2 - 1, 0) - 1] + o->YV[IF2V_(o, K2 - 1, 1) - 1]) / 2;
      double epsX = fabs(fabs(XFIN - XFOU) - o->DXCYCL);
      double epsY = fabs(fabs(YFIN - YFOU) - o->DYCYCL);
      if ((fabs(XFIN - XFOU) < TOLCYC && epsY < TOLCYC) || (fabs(YFIN - YFOU) < TOLCYC && epsX < TOLCYC)) { local = 1; break; }
    }
    if (local) o->IBFCYCLOC[o->NCYCLOC++] = K;
    else o->NCYCREM++;
  }
  if (o->NCYCREM != 0) { snprintf(err, errlen, "%d cyclic faces have no partner", o->NCYCREM); return -1; }
  free(BOUNFACEINDEX);
  free(bface);
  return 0;
}

/* MAPCYCLOC map_cyc_loc.f90:1-42 */
static int mapcycloc(orc_t* o, char* err, int errlen) {
  int np = o->NCYCLOC / 2;
  o->CYC2FPAIR = ialloc((int64_t)np * 2);
  o->NPAIR = 0;
  for (int nf = 0; nf < o->NCYCLOC; nf++) {
    int K = o->IBFCYCLOC[nf];
    double XFIN = (o->XV[IF2V_(o, K - 1, 0) - 1] + o->XV[IF2V_(o, K - 1, 1) - 1]) / 2;
    double YFIN = (o->YV[IF2V_(o, K - 1, 0) - 1] + o->YV[IF2V_(o, K - 1, 1) - 1]) / 2;
    for (int nf2 = nf + 1; nf2 < o->NCYCLOC; nf2++) {
      int K2 = o->IBFCYCLOC[nf2];
      double XFOU = (o->XV[IF2V_(o, K2 - 1, 0) - 1] + o->XV[IF2V_(o, K2 - 1, 1) - 1]) / 2;
      double YFOU = (o->YV[IF2V_(o, K2 - 1, 0) - 1] + o->YV[IF2V_(o, K2 - 1, 1) - 1]) / 2;
      double epsX = fabs(fabs(XFIN - XFOU) - o->DXCYCL);
      double epsY = fabs(fabs(YFIN - YFOU) - o->DYCYCL);
      if ((epsX < TOLCYC && fabs(YFIN - YFOU) < TOLCYC) || (epsY < TOLCYC && fabs(XFIN - XFOU) < TOLCYC)) {
        if (o->NPAIR >= np) { snprintf(err, errlen, "error in matching CYCLOC faces !!!"); return -1; }
        o->CYC2FPAIR[o->NPAIR] = K;
        o->CYC2FPAIR[o->NPAIR + np] = K2;
        o->NPAIR++;
      }
    }
  }
  if (o->NPAIR != np) { snprintf(err, errlen, "error in matching CYCLOC faces !!!"); return -1; }
  return 0;
}

/* =====================================================================
 * SD operators and geometry (initsetup.f90, mapder.f90, calcjacob.f90)
 * ===================================================================== */
/* setsandpoints initsetup.f90:167-255 */
static void setsandpoints(int np, double* xs, double* xf) {
  for (int i = 1; i <= np; i++) xs[i - 1] = 0.5 * (1.0 - cos((double)(2 * i - 1) * PI / (2 * (double)np)));
  switch (np) {
    case 1: xf[0] = 0.0; xf[1] = 1.0; break;
    case 2: xf[0] = 0.0; xf[1] = 0.5; xf[2] = 1.0; break;
    case 3: xf[0] = 0.0; xf[1] = (1.0 - sqrt(3.0) / 3.0) / 2.0; xf[2] = (1.0 + sqrt(3.0) / 3.0) / 2.0; xf[3] = 1.0; break;
    case 4: xf[0] = 0.0; xf[1] = (1.0 - sqrt(15.0) / 5.0) / 2.0; xf[2] = 0.5; xf[3] = (1.0 + sqrt(15.0) / 5.0) / 2.0; xf[4] = 1.0; break;
    case 5:
      xf[0] = 0.0;
      xf[1] = (1.0 - sqrt(525.0 + 70.0 * sqrt(30.0)) / 35.0) / 2.0;
      xf[2] = (1.0 - sqrt(525.0 - 70.0 * sqrt(30.0)) / 35.0) / 2.0;
      xf[3] = (1.0 + sqrt(525.0 - 70.0 * sqrt(30.0)) / 35.0) / 2.0;
      xf[4] = (1.0 + sqrt(525.0 + 70.0 * sqrt(30.0)) / 35.0) / 2.0;
      xf[5] = 1.0;
      break;
    case 6:
      xf[0] = 0.0;
      xf[1] = (1. - sqrt(245.0 + 14.0 * sqrt(70.0)) / 21.0) / 2.0;
      xf[2] = (1. - sqrt(245.0 - 14.0 * sqrt(70.0)) / 21.0) / 2.0;
      xf[3] = 0.5;
      xf[4] = (1. + sqrt(245.0 - 14.0 * sqrt(70.0)) / 21.0) / 2.0;
      xf[5] = (1. + sqrt(245.0 + 14.0 * sqrt(70.0)) / 21.0) / 2.0;
      xf[6] = 1.0;
      break;
    case 7: {
      const double g[3] = {0.932469514203, 0.661209386466, 0.238619186083};
      xf[0] = 0.0; xf[1] = (1.0 - g[0]) / 2.0; xf[2] = (1.0 - g[1]) / 2.0; xf[3] = (1.0 - g[2]) / 2.0;
      xf[4] = (1.0 + g[2]) / 2.0; xf[5] = (1.0 + g[1]) / 2.0; xf[6] = (1.0 + g[0]) / 2.0; xf[7] = 1.0;
      break;
    }
    case 8: {
      const double g[3] = {0.949107912343, 0.741531185599, 0.405845151377};
      xf[0] = 0.0; xf[1] = (1.0 - g[0]) / 2.0; xf[2] = (1.0 - g[1]) / 2.0; xf[3] = (1.0 - g[2]) / 2.0; xf[4] = 0.5;
      xf[5] = (1.0 + g[2]) / 2.0; xf[6] = (1.0 + g[1]) / 2.0; xf[7] = (1.0 + g[0]) / 2.0; xf[8] = 1.0;
      break;
    }
    case 9: {
      const double g[4] = {0.960289856498, 0.796666477414, 0.525532409916, 0.183434642496};
      xf[0] = 0.0;
      for (int q = 0; q < 4; q++) xf[1 + q] = (1.0 - g[q]) / 2.0;
      for (int q = 0; q < 4; q++) xf[5 + q] = (1.0 + g[3 - q]) / 2.0;
      xf[9] = 1.0;
      break;
    }
    case 10: {
      const double g[4] = {0.968160239508, 0.836031107327, 0.613371432701, 0.324253423404};
      xf[0] = 0.0;
      for (int q = 0; q < 4; q++) xf[1 + q] = (1.0 - g[q]) / 2.0;
      xf[5] = 0.5;
      for (int q = 0; q < 4; q++) xf[6 + q] = (1.0 + g[3 - q]) / 2.0;
      xf[10] = 1.0;
      break;
    }
    default: break;
  }
}

/* hhval initsetup.f90:318-340 (i is 1-based) */
static double hhval(const orc_t* o, int i, double xval) {
  double n = 1.0, d = 1.0;
  for (int s = 1; s <= o->N; s++)
    if (s != i) { n = n * (xval - o->Xs[s - 1]); d = d * (o->Xs[i - 1] - o->Xs[s - 1]); }
  return n / d;
}
/* hhval_low AV.f90:176-197 */
static double hhval_low(const orc_t* o, int i, double xval) {
  double n = 1.0, d = 1.0;
  for (int s = 1; s <= o->N - 1; s++)
    if (s != i) { n = n * (xval - o->Xs_low[s - 1]); d = d * (o->Xs_low[i - 1] - o->Xs_low[s - 1]); }
  return n / d;
}

/* computeLandM initsetup.f90:258-315 */
static void computeLandM(orc_t* o) {
  int np = o->N;
  for (int ifp = 1; ifp <= np + 1; ifp++)
    for (int is = 1; is <= np; is++) o->Lmat[LM(o, ifp - 1, is - 1)] = hhval(o, is, o->Xf[ifp - 1]);
  for (int ifp = 1; ifp <= np + 1; ifp++)
    for (int is = 1; is <= np; is++) {
      double xval = o->Xs[is - 1], sum = 0.0;
      for (int k = 1; k <= np + 1; k++) {
        if (k == ifp) continue;
        double num = 1.0, den = 1.0;
        for (int s = 1; s <= np + 1; s++) {
          if (s != ifp && s != k) num = num * (xval - o->Xf[s - 1]);
          if (s != ifp) den = den * (o->Xf[ifp - 1] - o->Xf[s - 1]);
        }
        sum = sum + num / den;
      }
      o->Mmat[LM(o, ifp - 1, is - 1)] = sum;
    }
}

/* face2fpconnec initsetup.f90:343-379 (values 1-based) */
static void face2fpconnec(orc_t* o) {
  int N = o->N;
  for (int nfp = 1; nfp <= N; nfp++) {
    IFACE2FP(o, nfp - 1, 0) = nfp;         JFACE2FP(o, nfp - 1, 0) = 1;
    IFACE2FP(o, nfp - 1, 1) = N + 1;       JFACE2FP(o, nfp - 1, 1) = nfp;
    IFACE2FP(o, nfp - 1, 2) = N - nfp + 1; JFACE2FP(o, nfp - 1, 2) = N + 1;
    IFACE2FP(o, nfp - 1, 3) = 1;           JFACE2FP(o, nfp - 1, 3) = N - nfp + 1;
  }
}

/* mapder mapder.f90:1-76: dm(k,d) shape-function derivatives */
static void dm4(double psi, double eta, double dm[4][2]) {
  dm[0][0] = eta - 1.0; dm[0][1] = psi - 1.0;
  dm[1][0] = 1.0 - eta; dm[1][1] = -psi;
  dm[2][0] = eta;       dm[2][1] = psi;
  dm[3][0] = -eta;      dm[3][1] = 1.0 - psi;
}

/* calcjacob calcjacob.f90:1-86 */
static void calcjacob(orc_t* o) {
  int N = o->N;
  for (int ic = 0; ic < o->NCELL; ic++) {
    int v[4];
    for (int k = 0; k < 4; k++) v[k] = IVCELL_(o, ic, k) - 1;
    double dm[4][2];
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        dm4(o->Xs[is], o->Xs[js], dm);
        double xpsi = 0.0, xeta = 0.0, ypsi = 0.0, yeta = 0.0;
        for (int k = 0; k < 4; k++) {
          xpsi = xpsi + dm[k][0] * o->XV[v[k]];
          ypsi = ypsi + dm[k][0] * o->YV[v[k]];
          xeta = xeta + dm[k][1] * o->XV[v[k]];
          yeta = yeta + dm[k][1] * o->YV[v[k]];
        }
        o->Jac[IDX_J(o, is, js, ic)] = xpsi * yeta - xeta * ypsi;
      }
    for (int jfp = 0; jfp < N; jfp++)
      for (int ifp = 0; ifp < N + 1; ifp++) {
        dm4(o->Xf[ifp], o->Xs[jfp], dm);
        double xpsi = 0.0, xeta = 0.0, ypsi = 0.0, yeta = 0.0;
        for (int k = 0; k < 4; k++) {
          xpsi = xpsi + dm[k][0] * o->XV[v[k]];
          ypsi = ypsi + dm[k][0] * o->YV[v[k]];
          xeta = xeta + dm[k][1] * o->XV[v[k]];
          yeta = yeta + dm[k][1] * o->YV[v[k]];
        }
        o->S1[IDX_S1(o, 0, 0, ifp, jfp, ic)] = yeta;
        o->S1[IDX_S1(o, 0, 1, ifp, jfp, ic)] = -xeta;
        o->S1[IDX_S1(o, 1, 0, ifp, jfp, ic)] = -ypsi;
        o->S1[IDX_S1(o, 1, 1, ifp, jfp, ic)] = xpsi;
      }
    for (int jfp = 0; jfp < N + 1; jfp++)
      for (int ifp = 0; ifp < N; ifp++) {
        dm4(o->Xs[ifp], o->Xf[jfp], dm);
        double xpsi = 0.0, xeta = 0.0, ypsi = 0.0, yeta = 0.0;
        for (int k = 0; k < 4; k++) {
          xpsi = xpsi + dm[k][0] * o->XV[v[k]];
          ypsi = ypsi + dm[k][0] * o->YV[v[k]];
          xeta = xeta + dm[k][1] * o->XV[v[k]];
          yeta = yeta + dm[k][1] * o->YV[v[k]];
        }
        o->S2[IDX_S2(o, 0, 0, ifp, jfp, ic)] = yeta;
        o->S2[IDX_S2(o, 0, 1, ifp, jfp, ic)] = -xeta;
        o->S2[IDX_S2(o, 1, 0, ifp, jfp, ic)] = -ypsi;
        o->S2[IDX_S2(o, 1, 1, ifp, jfp, ic)] = xpsi;
      }
  }
}

/* xyCoor_atGps mapder.f90:255-273 with MapBaseFunc :79-87 */
static void xycoor(const double xs[2][4], double xi, double eta, double xx[2]) {
  double f[4];
  f[0] = (1.0 - xi) * (1.0 - eta);
  f[1] = (1.0 - eta) * xi;
  f[2] = xi * eta;
  f[3] = (1.0 - xi) * eta;
  for (int i = 0; i < 2; i++) {
    xx[i] = 0.0;
    for (int nb = 0; nb < 4; nb++) xx[i] = xx[i] + xs[i][nb] * f[nb];
  }
}

/* =====================================================================
 * Physics point functions (getrusanov.f90)
 * ===================================================================== */
/* getrusanovflux getrusanov.f90:1-109 */
void orc_getrusanovflux(double gam, const double Qfl[9], const double Qfr[9], double Fnl[8], double Fnr[8],
                        double* Az, const double normf[2], int sign_l, int sign_r, double* eigv, double* eigvmax) {
  double magnorm = sqrt(normf[0] * normf[0] + normf[1] * normf[1]);
  double unit_x = normf[0] / magnorm * sign_l;
  double unit_y = normf[1] / magnorm * sign_l;
  double rhoi = 1.0 / Qfl[0];
  double ul = rhoi * Qfl[1], vl = rhoi * Qfl[2], wl = rhoi * Qfl[3];
  double Bxl = Qfl[5], Byl = Qfl[6], Bzl = Qfl[7];
  double NORM_Bl = Bxl * Bxl + Byl * Byl + Bzl * Bzl;
  double pl = (gam - 1.0) * (Qfl[4] - 0.5 * Qfl[0] * (ul * ul + vl * vl + wl * wl) - NORM_Bl * 0.5);
  pl = pl + 0.5 * NORM_Bl;
  double Vn_l = ul * unit_x + vl * unit_y;
  double Bn_l = Bxl * unit_x + Byl * unit_y;
  rhoi = 1.0 / Qfr[0];
  double ur = rhoi * Qfr[1], vr = rhoi * Qfr[2], wr = rhoi * Qfr[3];
  double Bxr = Qfr[5], Byr = Qfr[6], Bzr = Qfr[7];
  double NORM_Br = Bxr * Bxr + Byr * Byr + Bzr * Bzr;
  double pr = (gam - 1.0) * (Qfr[4] - 0.5 * Qfr[0] * (ur * ur + vr * vr + wr * wr) - NORM_Br * 0.5);
  pr = pr + NORM_Br * 0.5;
  double Vn_r = ur * unit_x + vr * unit_y;
  double Bn_r = Bxr * unit_x + Byr * unit_y;
  Fnl[0] = Qfl[0] * Vn_l;
  Fnl[1] = Qfl[1] * Vn_l + pl * unit_x - Bxl * Bn_l;
  Fnl[2] = Qfl[2] * Vn_l + pl * unit_y - Byl * Bn_l;
  Fnl[3] = Qfl[3] * Vn_l - Bzl * Bn_l;
  Fnl[4] = (Qfl[4] + pl) * Vn_l - Bn_l * (ul * Bxl + vl * Byl + wl * Bzl);
  Fnl[5] = (vl * Bxl - ul * Byl) * unit_y;
  Fnl[6] = (ul * Byl - vl * Bxl) * unit_x;
  Fnl[7] = Bzl * Vn_l - wl * Bn_l;
  Fnr[0] = Qfr[0] * Vn_r;
  Fnr[1] = Qfr[1] * Vn_r + pr * unit_x - Bxr * Bn_r;
  Fnr[2] = Qfr[2] * Vn_r + pr * unit_y - Byr * Bn_r;
  Fnr[3] = Qfr[3] * Vn_r - Bzr * Bn_r;
  Fnr[4] = (Qfr[4] + pr) * Vn_r - Bn_r * (ur * Bxr + vr * Byr + wr * Bzr);
  Fnr[5] = (vr * Bxr - ur * Byr) * unit_y;
  Fnr[6] = (ur * Byr - vr * Bxr) * unit_x;
  Fnr[7] = Bzr * Vn_r - wr * Bn_r;
  pl = pl - 0.5 * NORM_Bl;
  pr = pr - 0.5 * NORM_Br;
  double Bx = 0.5 * (Bxl + Bxr), By = 0.5 * (Byl + Byr), Bz = 0.5 * (Bzl + Bzr);
  double c_a = gam * (pl + pr) / (Qfl[0] + Qfr[0]);
  double c_d = (Bx * Bx + By * By + Bz * Bz) / (0.5 * (Qfl[0] + Qfr[0]));
  double bn = Bx * unit_x + By * unit_y;
  double c_n = bn * bn / (0.5 * (Qfl[0] + Qfr[0]));
  double cad = c_a + c_d;
  double c_tmp = sqrt(cad * cad - 4.0 * c_a * c_n);
  double c_f = sqrt(0.5 * (c_a + c_d + c_tmp));
  double ev = 0.5 * fabs(Vn_l + Vn_r) + c_f;
  for (int k = 0; k < 8; k++) Fnl[k] = 0.5 * (Fnl[k] + Fnr[k] - ev * (Qfr[k] - Qfl[k]));
  double ms = magnorm * sign_l;
  for (int k = 0; k < 8; k++) Fnl[k] = ms * Fnl[k];
  double ss = (double)(sign_l * sign_r);
  for (int k = 0; k < 8; k++) Fnr[k] = ss * Fnl[k];
  *Az = (Vn_l > 0.0) ? Qfl[8] : Qfr[8];
  *eigv = ev;
  if (ev > *eigvmax) *eigvmax = ev;
}

/* getIfluxvectors getrusanov.f90:111-153 */
void orc_getifluxvectors(double gam, const double Qi[8], double Fi[8], double Gi[8]) {
  double rho = Qi[0], rhou = Qi[1], rhov = Qi[2], rhow = Qi[3], rhoE = Qi[4];
  double Bx = Qi[5], By = Qi[6], Bz = Qi[7];
  double NORM_B = Bx * Bx + By * By + Bz * Bz;
  double pr = (gam - 1.0) * (rhoE - 0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) / rho - 0.5 * NORM_B);
  Fi[0] = rhou;
  Fi[1] = (rhou * rhou) / rho + pr + (0.5 * NORM_B - Bx * Bx);
  Fi[2] = rhou * rhov / rho - Bx * By;
  Fi[3] = rhou * rhow / rho - Bx * Bz;
  Fi[4] = (rhou / rho) * (rhoE + pr + 0.5 * NORM_B) - (rhou / rho * Bx + rhov / rho * By + rhow / rho * Bz) * Bx;
  Fi[5] = 0.0;
  Fi[6] = rhou / rho * By - rhov / rho * Bx;
  Fi[7] = rhou / rho * Bz - rhow / rho * Bx;
  Gi[0] = rhov;
  Gi[1] = rhou * rhov / rho - Bx * By;
  Gi[2] = (rhov * rhov) / rho + pr + (0.5 * NORM_B - By * By);
  Gi[3] = rhow * rhov / rho - By * Bz;
  Gi[4] = (rhov / rho) * (rhoE + pr + 0.5 * NORM_B) - (rhou / rho * Bx + rhov / rho * By + rhow / rho * Bz) * By;
  Gi[5] = rhov / rho * Bx - rhou / rho * By;
  Gi[6] = 0.0;
  Gi[7] = rhov / rho * Bz - rhow / rho * By;
}

/* getVfluxvectors getrusanov.f90:157-249 (nablaQ is (9,2) column-major) and
 * getVfluxvectors_AV :251-360 (same algebra with mu -> mu_art, eta0 -> 0). */
void orc_getvfluxvectors(double gam, double mu, double eta0, const double Qv[9], const double nQ[18],
                         double Fv[9], double Gv[9]) {
  double rho = Qv[0], rhou = Qv[1], rhov = Qv[2], rhow = Qv[3], rhoE = Qv[4];
  double Bx = Qv[5], By = Qv[6], Bz = Qv[7];
  double u = rhou / rho, v = rhov / rho, w = rhow / rho;
  double NORM_U = u * u + v * v + w * w;
  double NORM_B = Bx * Bx + By * By + Bz * Bz;
  double inte = (rhoE - 0.5 * NORM_U * rho - 0.5 * NORM_B) / rho;
  double drho[2], du[2], dv[2], dw[2], dBx[2], dBy[2], dBz[2], de[2], dKE[2], dpB[2];
  for (int d = 0; d < 2; d++) {
    drho[d] = nQ[0 + 9 * d];
    du[d] = (nQ[1 + 9 * d] - drho[d] * u) / rho;
    dv[d] = (nQ[2 + 9 * d] - drho[d] * v) / rho;
    dw[d] = (nQ[3 + 9 * d] - drho[d] * w) / rho;
    dBx[d] = nQ[5 + 9 * d];
    dBy[d] = nQ[6 + 9 * d];
    dBz[d] = nQ[7 + 9 * d];
  }
  for (int d = 0; d < 2; d++) {
    dKE[d] = 0.5 * NORM_U * drho[d] + rho * (u * du[d] + v * dv[d] + w * dw[d]);
    dpB[d] = Bx * dBx[d] + By * dBy[d] + Bz * dBz[d];
  }
  for (int d = 0; d < 2; d++) de[d] = (nQ[4 + 9 * d] - dKE[d] - dpB[d] - drho[d] * inte) / rho;
  double ux = du[0], uy = du[1], vx = dv[0], vy = dv[1], wx = dw[0], wy = dw[1], ex = de[0], ey = de[1];
  double Bxy = dBx[1], Byx = dBy[0], Bzx = dBz[0], Bzy = dBz[1];
  Fv[0] = 0.0;
  Fv[1] = mu * (2.0 * ux + LAMBDA * (ux + vy));
  Fv[2] = mu * (vx + uy);
  Fv[3] = mu * wx;
  Fv[4] = u * Fv[1] + v * Fv[2] + w * Fv[3] + mu * gam * ex / PRANDT;
  Gv[0] = 0.0;
  Gv[1] = mu * (vx + uy);
  Gv[2] = mu * (2.0 * vy + LAMBDA * (ux + vy));
  Gv[3] = mu * wy;
  Gv[4] = Gv[1] * u + Gv[2] * v + Gv[3] * w + mu * gam * ey / PRANDT;
  double Jx = Bzy - 0.0, Jy = 0.0 - Bzx, Jz = Byx - Bxy;
  Fv[5] = 0.0;
  Fv[6] = eta0 * Jz;
  Fv[7] = -eta0 * Jy;
  Fv[4] = Fv[4] + Fv[6] * By + Fv[7] * Bz;
  Gv[5] = -eta0 * Jz;
  Gv[6] = 0.0;
  Gv[7] = eta0 * Jx;
  Gv[4] = Gv[4] + Gv[5] * Bx + Gv[7] * Bz;
  Fv[8] = 0.0;
  Gv[8] = 0.0;
}

/* =====================================================================
 * Hot path (compflux.f90, interfaceflux_all.f90, cyclocflux_all.f90, bcflux.f90,
 * magnetic_potential.f90, AV.f90, compresid.f90)
 * ===================================================================== */
/* left/right trace of Q at face point nfp of local face lf (1-based) of cell ic
 * (0-based); interfaceflux_all.f90:35-55 */
static void face_trace_Q(const orc_t* o, int ic, int lf, int ifp, int jfp, double Qf[9]) {
  int N = o->N, fam = lf % 2 + 1;
  for (int k = 0; k < 9; k++) Qf[k] = 0.0;
  if (fam == 1) {
    for (int sp = 0; sp < N; sp++)
      for (int k = 0; k < 9; k++) Qf[k] = Qf[k] + o->Q[IDX_Q(o, k, sp, jfp - 1, ic)] * o->Lmat[LM(o, ifp - 1, sp)];
  } else {
    for (int sp = 0; sp < N; sp++)
      for (int k = 0; k < 9; k++) Qf[k] = Qf[k] + o->Q[IDX_Q(o, k, ifp - 1, sp, ic)] * o->Lmat[LM(o, jfp - 1, sp)];
  }
}

/* inviscid_flux_interior compflux.f90:51-104 */
static void inviscid_flux_interior(orc_t* o) {
  int N = o->N;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int ic = 0; ic < o->NCELL; ic++) {
    double Qf[9], F[8], G[8];
    for (int jfp = 0; jfp < N; jfp++)
      for (int ifp = 1; ifp < N; ifp++) {
        for (int k = 0; k < 9; k++) Qf[k] = 0.0;
        for (int sp = 0; sp < N; sp++)
          for (int k = 0; k < 9; k++) Qf[k] = Qf[k] + o->Q[IDX_Q(o, k, sp, jfp, ic)] * o->Lmat[LM(o, ifp, sp)];
        if (o->vismode == 1) {
          for (int k = 0; k < 9; k++) o->Qvfi[IDX_FI(o, 9, k, ifp, jfp, ic)] = Qf[k];
          o->Azfi[IDX_AI(o, ifp, jfp, ic)] = Qf[8];
        }
        orc_getifluxvectors(o->gam, Qf, F, G);
        double s11 = o->S1[IDX_S1(o, 0, 0, ifp, jfp, ic)], s12 = o->S1[IDX_S1(o, 0, 1, ifp, jfp, ic)];
        for (int k = 0; k < 8; k++) o->F1[IDX_FI(o, 8, k, ifp, jfp, ic)] = F[k] * s11 + G[k] * s12;
      }
    for (int jfp = 1; jfp < N; jfp++)
      for (int ifp = 0; ifp < N; ifp++) {
        for (int k = 0; k < 9; k++) Qf[k] = 0.0;
        for (int sp = 0; sp < N; sp++)
          for (int k = 0; k < 9; k++) Qf[k] = Qf[k] + o->Q[IDX_Q(o, k, ifp, sp, ic)] * o->Lmat[LM(o, jfp, sp)];
        if (o->vismode == 1) {
          for (int k = 0; k < 9; k++) o->Qvfj[IDX_FJ(o, 9, k, ifp, jfp, ic)] = Qf[k];
          o->Azfj[IDX_AJ(o, ifp, jfp, ic)] = Qf[8];
        }
        orc_getifluxvectors(o->gam, Qf, F, G);
        double s21 = o->S2[IDX_S2(o, 1, 0, ifp, jfp, ic)], s22 = o->S2[IDX_S2(o, 1, 1, ifp, jfp, ic)];
        for (int k = 0; k < 8; k++) o->G2[IDX_FJ(o, 8, k, ifp, jfp, ic)] = F[k] * s21 + G[k] * s22;
      }
  }
}

/* Shared body of interfaceflux (interfaceflux_all.f90:1-116) and CYCLOCFLUX
 * (cyclocflux_all.f90:1-116): left cell icl/local face lfl, right cell icr/lfr. */
static void two_sided_flux(orc_t* o, int icl, int lfl, int icr, int lfr, double* emax) {
  int N = o->N;
  int faml = lfl % 2 + 1, famr = lfr % 2 + 1;
  double Qfl[9], Qfr[9], Fnl[8], Fnr[8], normf[2], eigv, Az;
  for (int nfp = 1; nfp <= N; nfp++) {
    int ifpl = IFACE2FP(o, nfp - 1, lfl - 1), jfpl = JFACE2FP(o, nfp - 1, lfl - 1);
    int sign_l = 1;
    face_trace_Q(o, icl, lfl, ifpl, jfpl, Qfl);
    if (faml == 1) {
      if (ifpl == 1) sign_l = -1;
      normf[0] = o->S1[IDX_S1(o, 0, 0, ifpl - 1, jfpl - 1, icl)];
      normf[1] = o->S1[IDX_S1(o, 0, 1, ifpl - 1, jfpl - 1, icl)];
    } else {
      if (jfpl == 1) sign_l = -1;
      normf[0] = o->S2[IDX_S2(o, 1, 0, ifpl - 1, jfpl - 1, icl)];
      normf[1] = o->S2[IDX_S2(o, 1, 1, ifpl - 1, jfpl - 1, icl)];
    }
    int ifpr = IFACE2FP(o, N - nfp, lfr - 1), jfpr = JFACE2FP(o, N - nfp, lfr - 1);
    int sign_r = 1;
    face_trace_Q(o, icr, lfr, ifpr, jfpr, Qfr);
    if (famr == 1) { if (ifpr == N + 1) sign_r = -1; }
    else { if (jfpr == N + 1) sign_r = -1; }
    if (o->vismode == 1) {
      for (int k = 0; k < 9; k++) {
        double a = 0.5 * Qfl[k] + 0.5 * Qfr[k];
        if (faml == 1) o->Qvfi[IDX_FI(o, 9, k, ifpl - 1, jfpl - 1, icl)] = a;
        else o->Qvfj[IDX_FJ(o, 9, k, ifpl - 1, jfpl - 1, icl)] = a;
        if (famr == 1) o->Qvfi[IDX_FI(o, 9, k, ifpr - 1, jfpr - 1, icr)] = a;
        else o->Qvfj[IDX_FJ(o, 9, k, ifpr - 1, jfpr - 1, icr)] = a;
      }
    }
    orc_getrusanovflux(o->gam, Qfl, Qfr, Fnl, Fnr, &Az, normf, sign_l, sign_r, &eigv, emax);
    if (faml == 1) {
      for (int k = 0; k < 8; k++) o->F1[IDX_FI(o, 8, k, ifpl - 1, jfpl - 1, icl)] = Fnl[k];
      o->Azfi[IDX_AI(o, ifpl - 1, jfpl - 1, icl)] = Az;
    } else {
      for (int k = 0; k < 8; k++) o->G2[IDX_FJ(o, 8, k, ifpl - 1, jfpl - 1, icl)] = Fnl[k];
      o->Azfj[IDX_AJ(o, ifpl - 1, jfpl - 1, icl)] = Az;
    }
    if (famr == 1) {
      for (int k = 0; k < 8; k++) o->F1[IDX_FI(o, 8, k, ifpr - 1, jfpr - 1, icr)] = Fnr[k];
      o->Azfi[IDX_AI(o, ifpr - 1, jfpr - 1, icr)] = Az;
    } else {
      for (int k = 0; k < 8; k++) o->G2[IDX_FJ(o, 8, k, ifpr - 1, jfpr - 1, icr)] = Fnr[k];
      o->Azfj[IDX_AJ(o, ifpr - 1, jfpr - 1, icr)] = Az;
    }
  }
}

static void interfaceflux(orc_t* o, double* emax) {
  double m = *emax;
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(max : m)
  for (int fi = 0; fi < o->NINTER; fi++) {
    int f = o->IBFINTER[fi] - 1;
    double lm = m;
    two_sided_flux(o, IF2C_(o, f, 0) - 1, IF2C_(o, f, 2), IF2C_(o, f, 1) - 1, IF2C_(o, f, 3), &lm);
    if (lm > m) m = lm;
  }
  *emax = m;
}

static void cyclocflux(orc_t* o, double* emax) {
  double m = *emax;
  int np = o->NPAIR;
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(max : m)
  for (int p = 0; p < np; p++) {
    int K1 = o->CYC2FPAIR[p] - 1, K2 = o->CYC2FPAIR[p + np] - 1;
    double lm = m;
    two_sided_flux(o, IF2C_(o, K1, 0) - 1, IF2C_(o, K1, 2), IF2C_(o, K2, 0) - 1, IF2C_(o, K2, 2), &lm);
    if (lm > m) m = lm;
  }
  *emax = m;
}

/* BCFLUX bcflux.f90:1-70 */
static void bcflux(orc_t* o, double* emax) {
  int N = o->N;
  double m = *emax;
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(max : m)
  for (int fn = 0; fn < o->NFREE; fn++) {
    int f = o->IBFREE[fn] - 1;
    int icl = IF2C_(o, f, 0) - 1, lfl = IF2C_(o, f, 2), faml = lfl % 2 + 1;
    double Qfl[9], Qfr[9], Fnl[8], Fnr[8], normf[2], eigv, Az, lm = m;
    for (int nfp = 1; nfp <= N; nfp++) {
      int ifpl = IFACE2FP(o, nfp - 1, lfl - 1), jfpl = JFACE2FP(o, nfp - 1, lfl - 1);
      int sign_l = 1, sign_r = 1;
      face_trace_Q(o, icl, lfl, ifpl, jfpl, Qfl);
      if (faml == 1) {
        if (ifpl == 1) sign_l = -1;
        normf[0] = o->S1[IDX_S1(o, 0, 0, ifpl - 1, jfpl - 1, icl)];
        normf[1] = o->S1[IDX_S1(o, 0, 1, ifpl - 1, jfpl - 1, icl)];
      } else {
        if (jfpl == 1) sign_l = -1;
        normf[0] = o->S2[IDX_S2(o, 1, 0, ifpl - 1, jfpl - 1, icl)];
        normf[1] = o->S2[IDX_S2(o, 1, 1, ifpl - 1, jfpl - 1, icl)];
      }
      for (int k = 0; k < 9; k++) Qfr[k] = Qfl[k];
      if (o->vismode == 1)
        for (int k = 0; k < 9; k++) {
          double a = 0.5 * Qfl[k] + 0.5 * Qfr[k];
          if (faml == 1) o->Qvfi[IDX_FI(o, 9, k, ifpl - 1, jfpl - 1, icl)] = a;
          else o->Qvfj[IDX_FJ(o, 9, k, ifpl - 1, jfpl - 1, icl)] = a;
        }
      /* sign_r is left uninitialised in the reference; BCFLUX never reads Fnr */
      orc_getrusanovflux(o->gam, Qfl, Qfr, Fnl, Fnr, &Az, normf, sign_l, sign_r, &eigv, &lm);
      if (faml == 1) {
        for (int k = 0; k < 8; k++) o->F1[IDX_FI(o, 8, k, ifpl - 1, jfpl - 1, icl)] = Fnl[k];
        o->Azfi[IDX_AI(o, ifpl - 1, jfpl - 1, icl)] = Az;
      } else {
        for (int k = 0; k < 8; k++) o->G2[IDX_FJ(o, 8, k, ifpl - 1, jfpl - 1, icl)] = Fnl[k];
        o->Azfj[IDX_AJ(o, ifpl - 1, jfpl - 1, icl)] = Az;
      }
    }
    if (lm > m) m = lm;
  }
  *emax = m;
}

/* comp_inviscid_flux compflux.f90:33-49 (PROCINTFLUX/CYCREMFLUX are empty at one
 * partition) */
void orc_comp_inviscid_flux(orc_t* o) {
  inviscid_flux_interior(o);
  double m = o->eigvmax;
  interfaceflux(o, &m);
  cyclocflux(o, &m);
  bcflux(o, &m);
  o->eigvmax = m;
}

/* nablaAsp magnetic_potential.f90:1-42 */
static void nablaAsp(orc_t* o) {
  int N = o->N;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int ic = 0; ic < o->NCELL; ic++)
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        double dApsi = 0.0, dAeta = 0.0;
        for (int r = 0; r < N + 1; r++)
          dApsi = dApsi + o->Azfi[IDX_AI(o, r, js, ic)] * o->Mmat[LM(o, r, is)] * o->S1[IDX_S1(o, 0, 0, r, js, ic)];
        for (int r = 0; r < N + 1; r++)
          dAeta = dAeta + o->Azfj[IDX_AJ(o, is, r, ic)] * o->Mmat[LM(o, r, js)] * o->S2[IDX_S2(o, 1, 0, is, r, ic)];
        o->nablaAs[0 + 2 * IDX_J(o, is, js, ic)] = (dApsi + dAeta) / o->Jac[IDX_J(o, is, js, ic)];
        dApsi = 0.0;
        for (int r = 0; r < N + 1; r++)
          dApsi = dApsi + o->Azfi[IDX_AI(o, r, js, ic)] * o->Mmat[LM(o, r, is)] * o->S1[IDX_S1(o, 0, 1, r, js, ic)];
        dAeta = 0.0;
        for (int r = 0; r < N + 1; r++)
          dAeta = dAeta + o->Azfj[IDX_AJ(o, is, r, ic)] * o->Mmat[LM(o, r, js)] * o->S2[IDX_S2(o, 1, 1, is, r, ic)];
        o->nablaAs[1 + 2 * IDX_J(o, is, js, ic)] = (dApsi + dAeta) / o->Jac[IDX_J(o, is, js, ic)];
      }
}

/* nablaQsp compflux.f90:107-157 (v_sta/v_end 1-based) */
void orc_nablaQsp(orc_t* o, int v_sta, int v_end) {
  int N = o->N;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int ic = 0; ic < o->NCELL; ic++)
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        double dp[9], de[9];
        double J = o->Jac[IDX_J(o, is, js, ic)];
        for (int c = 0; c < 2; c++) {
          for (int k = v_sta - 1; k < v_end; k++) dp[k] = 0.0;
          for (int r = 0; r < N + 1; r++) {
            double mm = o->Mmat[LM(o, r, is)], s = o->S1[IDX_S1(o, 0, c, r, js, ic)];
            for (int k = v_sta - 1; k < v_end; k++) dp[k] = dp[k] + o->Qvfi[IDX_FI(o, 9, k, r, js, ic)] * mm * s;
          }
          for (int k = v_sta - 1; k < v_end; k++) de[k] = 0.0;
          for (int r = 0; r < N + 1; r++) {
            double mm = o->Mmat[LM(o, r, js)], s = o->S2[IDX_S2(o, 1, c, is, r, ic)];
            for (int k = v_sta - 1; k < v_end; k++) de[k] = de[k] + o->Qvfj[IDX_FJ(o, 9, k, is, r, ic)] * mm * s;
          }
          for (int k = v_sta - 1; k < v_end; k++) o->nablaQs[IDX_NQS(o, k, c, is, js, ic)] = (dp[k] + de[k]) / J;
        }
      }
}

/* nablaQ_interior_FP compflux.f90:159-196 */
static void nablaQ_interior_FP(orc_t* o) {
  int N = o->N;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int ic = 0; ic < o->NCELL; ic++) {
    double a[9], b[9];
    for (int jfp = 0; jfp < N; jfp++)
      for (int ifp = 1; ifp < N; ifp++) {
        for (int k = 0; k < 9; k++) { a[k] = 0.0; b[k] = 0.0; }
        for (int sp = 0; sp < N; sp++) {
          double l = o->Lmat[LM(o, ifp, sp)];
          for (int k = 0; k < 9; k++) a[k] = a[k] + o->nablaQs[IDX_NQS(o, k, 0, sp, jfp, ic)] * l;
          for (int k = 0; k < 9; k++) b[k] = b[k] + o->nablaQs[IDX_NQS(o, k, 1, sp, jfp, ic)] * l;
        }
        for (int k = 0; k < 9; k++) {
          o->nablaQvfi[IDX_NQI(o, k, 0, ifp, jfp, ic)] = a[k];
          o->nablaQvfi[IDX_NQI(o, k, 1, ifp, jfp, ic)] = b[k];
        }
      }
    for (int jfp = 1; jfp < N; jfp++)
      for (int ifp = 0; ifp < N; ifp++) {
        for (int k = 0; k < 9; k++) { a[k] = 0.0; b[k] = 0.0; }
        for (int sp = 0; sp < N; sp++) {
          double l = o->Lmat[LM(o, jfp, sp)];
          for (int k = 0; k < 9; k++) a[k] = a[k] + o->nablaQs[IDX_NQS(o, k, 0, ifp, sp, ic)] * l;
          for (int k = 0; k < 9; k++) b[k] = b[k] + o->nablaQs[IDX_NQS(o, k, 1, ifp, sp, ic)] * l;
        }
        for (int k = 0; k < 9; k++) {
          o->nablaQvfj[IDX_NQJ(o, k, 0, ifp, jfp, ic)] = a[k];
          o->nablaQvfj[IDX_NQJ(o, k, 1, ifp, jfp, ic)] = b[k];
        }
      }
  }
}

/* trace of nablaQs (both components) at a face point; interfaceflux_all.f90:139-176 */
static void face_trace_nQ(const orc_t* o, int ic, int lf, int ifp, int jfp, double a[9], double b[9]) {
  int N = o->N, fam = lf % 2 + 1;
  for (int k = 0; k < 9; k++) { a[k] = 0.0; b[k] = 0.0; }
  if (fam == 1) {
    for (int sp = 0; sp < N; sp++) {
      double l = o->Lmat[LM(o, ifp - 1, sp)];
      for (int k = 0; k < 9; k++) {
        a[k] = a[k] + o->nablaQs[IDX_NQS(o, k, 0, sp, jfp - 1, ic)] * l;
        b[k] = b[k] + o->nablaQs[IDX_NQS(o, k, 1, sp, jfp - 1, ic)] * l;
      }
    }
  } else {
    for (int sp = 0; sp < N; sp++) {
      double l = o->Lmat[LM(o, jfp - 1, sp)];
      for (int k = 0; k < 9; k++) {
        a[k] = a[k] + o->nablaQs[IDX_NQS(o, k, 0, ifp - 1, sp, ic)] * l;
        b[k] = b[k] + o->nablaQs[IDX_NQS(o, k, 1, ifp - 1, sp, ic)] * l;
      }
    }
  }
}

static void store_nQ(orc_t* o, int ic, int lf, int ifp, int jfp, const double a[9], const double b[9]) {
  if (lf % 2 + 1 == 1)
    for (int k = 0; k < 9; k++) {
      o->nablaQvfi[IDX_NQI(o, k, 0, ifp - 1, jfp - 1, ic)] = a[k];
      o->nablaQvfi[IDX_NQI(o, k, 1, ifp - 1, jfp - 1, ic)] = b[k];
    }
  else
    for (int k = 0; k < 9; k++) {
      o->nablaQvfj[IDX_NQJ(o, k, 0, ifp - 1, jfp - 1, ic)] = a[k];
      o->nablaQvfj[IDX_NQJ(o, k, 1, ifp - 1, jfp - 1, ic)] = b[k];
    }
}

/* interfaceVISflux interfaceflux_all.f90:118-199 / CYCLOCVISFLUX cyclocflux_all.f90:118-208 */
static void two_sided_visflux(orc_t* o, int icl, int lfl, int icr, int lfr) {
  int N = o->N;
  double Qfl[9], Qfl2[9], Qfr[9], Qfr2[9], a[9], b[9];
  for (int nfp = 1; nfp <= N; nfp++) {
    int ifpl = IFACE2FP(o, nfp - 1, lfl - 1), jfpl = JFACE2FP(o, nfp - 1, lfl - 1);
    face_trace_nQ(o, icl, lfl, ifpl, jfpl, Qfl, Qfl2);
    int ifpr = IFACE2FP(o, N - nfp, lfr - 1), jfpr = JFACE2FP(o, N - nfp, lfr - 1);
    face_trace_nQ(o, icr, lfr, ifpr, jfpr, Qfr, Qfr2);
    for (int k = 0; k < 9; k++) { a[k] = 0.5 * Qfl[k] + 0.5 * Qfr[k]; b[k] = 0.5 * Qfl2[k] + 0.5 * Qfr2[k]; }
    store_nQ(o, icl, lfl, ifpl, jfpl, a, b);
    store_nQ(o, icr, lfr, ifpr, jfpr, a, b);
  }
}

static void vis_faces(orc_t* o) {
  int N = o->N;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int fi = 0; fi < o->NINTER; fi++) {
    int f = o->IBFINTER[fi] - 1;
    two_sided_visflux(o, IF2C_(o, f, 0) - 1, IF2C_(o, f, 2), IF2C_(o, f, 1) - 1, IF2C_(o, f, 3));
  }
  /* BCVISFLUX bcflux.f90:73-121 */
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int fn = 0; fn < o->NFREE; fn++) {
    int f = o->IBFREE[fn] - 1;
    int icl = IF2C_(o, f, 0) - 1, lfl = IF2C_(o, f, 2);
    double Qfl[9], Qfl2[9], a[9], b[9];
    for (int nfp = 1; nfp <= N; nfp++) {
      int ifpl = IFACE2FP(o, nfp - 1, lfl - 1), jfpl = JFACE2FP(o, nfp - 1, lfl - 1);
      face_trace_nQ(o, icl, lfl, ifpl, jfpl, Qfl, Qfl2);
      for (int k = 0; k < 9; k++) { a[k] = 0.5 * Qfl[k] + 0.5 * Qfl[k]; b[k] = 0.5 * Qfl2[k] + 0.5 * Qfl2[k]; }
      store_nQ(o, icl, lfl, ifpl, jfpl, a, b);
    }
  }
  int np = o->NPAIR;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int p = 0; p < np; p++) {
    int K1 = o->CYC2FPAIR[p] - 1, K2 = o->CYC2FPAIR[p + np] - 1;
    two_sided_visflux(o, IF2C_(o, K1, 0) - 1, IF2C_(o, K1, 2), IF2C_(o, K2, 0) - 1, IF2C_(o, K2, 2));
  }
}

/* comp_artificial_viscosity AV.f90:1-174 (the Se min/max allreduces are unused) */
static void comp_artificial_viscosity(orc_t* o) {
  int N = o->N, nl = N - 1;
#pragma omp parallel num_threads(g_threads)
  {
    double* Ql = dalloc((int64_t)9 * nl * nl);
    double* Qs = dalloc((int64_t)9 * N * N);
#pragma omp for schedule(static)
    for (int ic = 0; ic < o->NCELL; ic++) {
      for (int q = 0; q < 9 * nl * nl; q++) Ql[q] = 0.0;
      for (int jsl = 1; jsl <= nl; jsl++)
        for (int isl = 1; isl <= nl; isl++) {
          double xsi = o->Xs_low[isl - 1], eta = o->Xs_low[jsl - 1];
          for (int js = 1; js <= N; js++)
            for (int is = 1; is <= N; is++) {
              double h1 = hhval(o, is, xsi), h2 = hhval(o, js, eta);
              for (int k = 0; k < 9; k++)
                Ql[k + 9 * ((isl - 1) + nl * (jsl - 1))] =
                    Ql[k + 9 * ((isl - 1) + nl * (jsl - 1))] + o->Q[IDX_Q(o, k, is - 1, js - 1, ic)] * h1 * h2;
            }
        }
      for (int q = 0; q < 9 * N * N; q++) Qs[q] = 0.0;
      for (int js = 1; js <= N; js++)
        for (int is = 1; is <= N; is++) {
          double xsi = o->Xs[is - 1], eta = o->Xs[js - 1];
          for (int jsl = 1; jsl <= nl; jsl++)
            for (int isl = 1; isl <= nl; isl++) {
              double h1 = hhval_low(o, isl, xsi), h2 = hhval_low(o, jsl, eta);
              for (int k = 0; k < 9; k++)
                Qs[k + 9 * ((is - 1) + N * (js - 1))] =
                    Qs[k + 9 * ((is - 1) + N * (js - 1))] + Ql[k + 9 * ((isl - 1) + nl * (jsl - 1))] * h1 * h2;
            }
        }
      double Se[9];
      for (int k = 0; k < 9; k++) Se[k] = 0.0;
      for (int js = 0; js < N; js++)
        for (int is = 0; is < N; is++)
          for (int k = 0; k < 9; k++) {
            if (k == 3 || k == 7) continue;
            double q = o->Q[IDX_Q(o, k, is, js, ic)];
            double d = Qs[k + 9 * (is + N * js)] - q;
            Se[k] = Se[k] + d * d / (q * q);
          }
      Se[3] = 1.0;
      Se[7] = 1.0;
      for (int k = 0; k < 9; k++) Se[k] = log10(Se[k]);
      for (int k = 0; k < 9; k++) o->SM_IND[k + 9 * ic] = Se[k];
    }
    free(Ql);
    free(Qs);
  }
  double se_low[9], se_high[9], k_range[9], s0[9];
  for (int k = 0; k < 9; k++) { se_low[k] = -6.0; se_high[k] = -1.0; }
  se_low[3] = se_high[3] = 0.0;
  se_low[6] = se_high[6] = 0.0;
  se_low[7] = se_high[7] = 0.0;
  se_low[8] = se_high[8] = 0.0;
  for (int k = 0; k < 9; k++) { k_range[k] = (se_high[k] - se_low[k]) * 0.5; s0[k] = (se_high[k] + se_low[k]) * 0.5; }
  o->eigvmax_g = o->eigvmax;
  double h_msh = sqrt(o->DXCYCL * o->DYCYCL / (double)o->NCELL);
  o->epsilon0 = o->eigvmax_g * h_msh / (N - 1) * 1.0;
  double e0 = o->epsilon0;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int ic = 0; ic < o->NCELL; ic++)
    for (int k = 0; k < 9; k++) {
      double mv;
      if (k == 3 || k == 6 || k == 7 || k == 8) mv = 0.0;
      else {
        double s = o->SM_IND[k + 9 * ic];
        if (s < se_low[k]) mv = 0.0;
        else if (s > se_high[k]) mv = e0;
        else mv = e0 / 2.0 * (1.0 + sin(PI * (s - s0[k]) / 2.0 / k_range[k]));
      }
      o->muAV[k + 9 * ic] = mv;
    }
}

/* muAVfi/muAVfj slot of (cell, local face): AV.f90:245-254 */
static double* mu_slot(orc_t* o, int ic, int lf) {
  switch (lf) {
    case 1: return &o->muAVfj[9 * (0 + 2 * ic)];
    case 2: return &o->muAVfi[9 * (1 + 2 * ic)];
    case 3: return &o->muAVfj[9 * (1 + 2 * ic)];
    default: return &o->muAVfi[9 * (0 + 2 * ic)];
  }
}
static void av_face(orc_t* o, int icl, int lfl, int icr, int lfr) {
  double* l = mu_slot(o, icl, lfl);
  double* r = mu_slot(o, icr, lfr);
  double ml[9], mr[9];
  for (int k = 0; k < 9; k++) { ml[k] = l[k]; mr[k] = r[k]; }
  for (int k = 0; k < 9; k++) l[k] = 0.5 * (ml[k] + mr[k]);
  for (int k = 0; k < 9; k++) r[k] = 0.5 * (ml[k] + mr[k]);
}
/* compAVflux AV.f90:199-223, interfaceAVflux :226-303, cyclocAVflux :494-564 */
static void compAVflux(orc_t* o) {
  for (int ic = 0; ic < o->NCELL; ic++)
    for (int f = 0; f < 2; f++)
      for (int k = 0; k < 9; k++) {
        o->muAVfi[k + 9 * (f + 2 * ic)] = o->muAV[k + 9 * ic];
        o->muAVfj[k + 9 * (f + 2 * ic)] = o->muAV[k + 9 * ic];
      }
  for (int fi = 0; fi < o->NINTER; fi++) {
    int f = o->IBFINTER[fi] - 1;
    av_face(o, IF2C_(o, f, 0) - 1, IF2C_(o, f, 2), IF2C_(o, f, 1) - 1, IF2C_(o, f, 3));
  }
  int np = o->NPAIR;
  for (int p = 0; p < np; p++) {
    int K1 = o->CYC2FPAIR[p] - 1, K2 = o->CYC2FPAIR[p + np] - 1;
    av_face(o, IF2C_(o, K1, 0) - 1, IF2C_(o, K1, 2), IF2C_(o, K2, 0) - 1, IF2C_(o, K2, 2));
  }
}

/* comp_viscous_flux compflux.f90:198-258 with getVfluxvectors_AV getrusanov.f90:251-360 */
static void comp_viscous_flux(orc_t* o) {
  int N = o->N;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int ic = 0; ic < o->NCELL; ic++) {
    double Qs[9], nQ[18], Fv[9], Gv[9], Fa[9], Ga[9];
    for (int jfp = 0; jfp < N; jfp++)
      for (int ifp = 0; ifp < N + 1; ifp++) {
        for (int k = 0; k < 9; k++) {
          Qs[k] = o->Qvfi[IDX_FI(o, 9, k, ifp, jfp, ic)];
          nQ[k] = o->nablaQvfi[IDX_NQI(o, k, 0, ifp, jfp, ic)];
          nQ[9 + k] = o->nablaQvfi[IDX_NQI(o, k, 1, ifp, jfp, ic)];
        }
        orc_getvfluxvectors(o->gam, o->mu, o->eta0, Qs, nQ, Fv, Gv);
        double s11 = o->S1[IDX_S1(o, 0, 0, ifp, jfp, ic)], s12 = o->S1[IDX_S1(o, 0, 1, ifp, jfp, ic)];
        for (int k = 0; k < 9; k++) o->Fv1[IDX_FI(o, 9, k, ifp, jfp, ic)] = Fv[k] * s11 + Gv[k] * s12;
        if (o->ARTIV == 1) {
          double xsi = o->Xf[ifp];
          double mu_art = o->muAVfi[0 + 9 * (0 + 2 * ic)] * (1.0 - xsi) + o->muAVfi[0 + 9 * (1 + 2 * ic)] * xsi;
          orc_getvfluxvectors(o->gam, mu_art, 0.0, Qs, nQ, Fa, Ga);
          for (int k = 0; k < 9; k++)
            o->Fv1[IDX_FI(o, 9, k, ifp, jfp, ic)] = o->Fv1[IDX_FI(o, 9, k, ifp, jfp, ic)] + Fa[k] * s11 + Ga[k] * s12;
        }
      }
    for (int jfp = 0; jfp < N + 1; jfp++)
      for (int ifp = 0; ifp < N; ifp++) {
        for (int k = 0; k < 9; k++) {
          Qs[k] = o->Qvfj[IDX_FJ(o, 9, k, ifp, jfp, ic)];
          nQ[k] = o->nablaQvfj[IDX_NQJ(o, k, 0, ifp, jfp, ic)];
          nQ[9 + k] = o->nablaQvfj[IDX_NQJ(o, k, 1, ifp, jfp, ic)];
        }
        orc_getvfluxvectors(o->gam, o->mu, o->eta0, Qs, nQ, Fv, Gv);
        double s21 = o->S2[IDX_S2(o, 1, 0, ifp, jfp, ic)], s22 = o->S2[IDX_S2(o, 1, 1, ifp, jfp, ic)];
        for (int k = 0; k < 9; k++) o->Gv2[IDX_FJ(o, 9, k, ifp, jfp, ic)] = Fv[k] * s21 + Gv[k] * s22;
        if (o->ARTIV == 1) {
          double eta = o->Xf[jfp];
          double mu_art = o->muAVfj[0 + 9 * (0 + 2 * ic)] * (1.0 - eta) + o->muAVfj[0 + 9 * (1 + 2 * ic)] * eta;
          orc_getvfluxvectors(o->gam, mu_art, 0.0, Qs, nQ, Fa, Ga);
          for (int k = 0; k < 9; k++)
            o->Gv2[IDX_FJ(o, 9, k, ifp, jfp, ic)] = o->Gv2[IDX_FJ(o, 9, k, ifp, jfp, ic)] + Fa[k] * s21 + Ga[k] * s22;
        }
      }
  }
}

/* compflux compflux.f90:1-31 */
void orc_compflux(orc_t* o) {
  o->eigvmax = 0.0;
  orc_comp_inviscid_flux(o);
  nablaAsp(o);
  if (o->vismode == 1) {
    orc_nablaQsp(o, 1, 9);
    nablaQ_interior_FP(o);
    vis_faces(o);
    if (o->ARTIV == 1) {
      comp_artificial_viscosity(o);
      compAVflux(o);
    }
    comp_viscous_flux(o);
  }
}

/* compresid compresid.f90:1-67 (EXTENSION: the background field B0 enters the A_z
 * advection through grad(A_bg) = (-B0y, B0x); with B0=0 this is the reference). */
void orc_compresid(orc_t* o) {
  int N = o->N;
  orc_compflux(o);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int ic = 0; ic < o->NCELL; ic++)
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        double Qs[9], dF[8], dG[8], dFv[9], dGv[9];
        for (int k = 0; k < 9; k++) Qs[k] = o->Q[IDX_Q(o, k, is, js, ic)];
        double au = Qs[1] / Qs[0], av = Qs[2] / Qs[0];
        for (int k = 0; k < 8; k++) dF[k] = 0.0;
        for (int k = 0; k < 9; k++) dFv[k] = 0.0;
        for (int r = 0; r < N + 1; r++) {
          double m = o->Mmat[LM(o, r, is)];
          for (int k = 0; k < 8; k++) dF[k] = dF[k] + o->F1[IDX_FI(o, 8, k, r, js, ic)] * m;
          if (o->vismode == 1)
            for (int k = 0; k < 9; k++) dFv[k] = dFv[k] + o->Fv1[IDX_FI(o, 9, k, r, js, ic)] * m;
        }
        for (int k = 0; k < 8; k++) dG[k] = 0.0;
        for (int k = 0; k < 9; k++) dGv[k] = 0.0;
        for (int r = 0; r < N + 1; r++) {
          double m = o->Mmat[LM(o, r, js)];
          for (int k = 0; k < 8; k++) dG[k] = dG[k] + o->G2[IDX_FJ(o, 8, k, is, r, ic)] * m;
          if (o->vismode == 1)
            for (int k = 0; k < 9; k++) dGv[k] = dGv[k] + o->Gv2[IDX_FJ(o, 9, k, is, r, ic)] * m;
        }
        double* R = &o->resid[IDX_Q(o, 0, is, js, ic)];
        for (int k = 0; k < 8; k++) R[k] = -(dF[k] + dG[k]);
        double ax = o->nablaAs[0 + 2 * IDX_J(o, is, js, ic)] - o->B0y;
        double ay = o->nablaAs[1 + 2 * IDX_J(o, is, js, ic)] + o->B0x;
        R[8] = -au * ax - av * ay;
        R[8] = R[8] * o->Jac[IDX_J(o, is, js, ic)];
        if (o->vismode == 1)
          for (int k = 0; k < 9; k++) R[k] = R[k] + (dFv[k] + dGv[k]);
      }
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int ic = 0; ic < o->NCELL; ic++)
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        double J = o->Jac[IDX_J(o, is, js, ic)];
        for (int k = 0; k < 9; k++) o->resid[IDX_Q(o, k, is, js, ic)] = o->resid[IDX_Q(o, k, is, js, ic)] / J;
      }
}

/* update_B magnetic_potential.f90:44-67 (EXTENSION: + B0) */
static void update_B(orc_t* o) {
  int64_t np = (int64_t)o->N * o->N * o->NCELL;
  for (int64_t p = 0; p < np; p++) {
    double Bx = o->nablaQs[8 + NV * (1 + 2 * p)] + o->B0x;
    double By = -o->nablaQs[8 + NV * (0 + 2 * p)] + o->B0y;
    double Bz = o->Q[7 + NV * p];
    o->Q[5 + NV * p] = Bx;
    o->Q[6 + NV * p] = By;
    o->Q[7 + NV * p] = Bz;
  }
}

/* correct_B_via_curl_Az setinitialcond.f90:82-91 */
void orc_correct_B_via_curl_Az(orc_t* o) {
  orc_comp_inviscid_flux(o);
  orc_nablaQsp(o, 9, 9);
  update_B(o);
}

/* RK_S5P3 iterations.f90:162-217 */
void orc_rk_s5p3(orc_t* o) {
  const double a30 = 0.355909775063327, a32 = 0.644090224936674, a40 = 0.367933791638137,
               a43 = 0.632066208361863, a52 = 0.237593836598569, a54 = 0.762406163401431,
               b10 = 0.377268915331368, b21 = 0.377268915331368, b32 = 0.242995220537396,
               b43 = 0.238458932846290, b54 = 0.287632146308408;
  int64_t n = (int64_t)NV * o->N * o->N * o->NCELL;
  double dt = o->dt, *Q = o->Q, *R = o->resid, *Qk0 = o->Qk0, *Qka = o->Qka;
  memcpy(Qk0, Q, sizeof(double) * n);
  double ctime0 = o->ctime;
  orc_compresid(o);
  for (int64_t i = 0; i < n; i++) Q[i] = Q[i] + b10 * dt * R[i];
  double dt1 = b10 * dt;
  o->ctime = ctime0 + dt1;
  orc_compresid(o);
  for (int64_t i = 0; i < n; i++) Q[i] = Q[i] + b21 * dt * R[i];
  double dt2 = dt1 + b21 * dt;
  o->ctime = ctime0 + dt2;
  memcpy(Qka, Q, sizeof(double) * n);
  orc_compresid(o);
  for (int64_t i = 0; i < n; i++) Q[i] = a30 * Qk0[i] + a32 * Q[i] + b32 * dt * R[i];
  double dt3 = a32 * dt2 + b32 * dt;
  o->ctime = ctime0 + dt3;
  orc_compresid(o);
  for (int64_t i = 0; i < n; i++) Q[i] = a40 * Qk0[i] + a43 * Q[i] + b43 * dt * R[i];
  o->ctime = ctime0 + (a43 * dt3 + b43 * dt);
  orc_compresid(o);
  for (int64_t i = 0; i < n; i++) Q[i] = a52 * Qka[i] + a54 * Q[i] + b54 * dt * R[i];
  o->ctime = ctime0 + dt;
}

/* FiveStageRk iterations.f90:92-160 */
void orc_fivestagerk(orc_t* o) {
  int64_t n = (int64_t)NV * o->N * o->N * o->NCELL;
  double dt = o->dt, *Q = o->Q, *R = o->resid, *qj0 = o->Qk0;
  double old_time = o->ctime, rdt;
  memcpy(qj0, Q, sizeof(double) * n);
  orc_compresid(o);
  double a11 = 0.39175222700392;
  rdt = dt * a11;
  for (int64_t i = 0; i < n; i++) Q[i] = qj0[i] + rdt * R[i];
  o->ctime = old_time + rdt;
  orc_compresid(o);
  double a21 = 0.44437049406734, a22 = 0.55562950593266, a23 = 0.36841059262959;
  for (int64_t i = 0; i < n; i++) Q[i] = a21 * qj0[i] + a22 * Q[i] + a23 * R[i] * dt;
  memcpy(o->qj2, Q, sizeof(double) * n);
  rdt = rdt * a22 + a23 * dt;
  o->ctime = old_time + rdt;
  orc_compresid(o);
  double a31 = 0.6201018513854, a32 = 0.3798981486146, a33 = 0.25189177424738;
  for (int64_t i = 0; i < n; i++) Q[i] = a31 * qj0[i] + a32 * Q[i] + a33 * dt * R[i];
  memcpy(o->qj3, Q, sizeof(double) * n);
  rdt = rdt * a32 + a33 * dt;
  o->ctime = old_time + rdt;
  orc_compresid(o);
  double a41 = 0.17807995410773, a42 = 0.82192004589227, a43 = 0.54497475021237;
  for (int64_t i = 0; i < n; i++) Q[i] = a41 * qj0[i] + a42 * Q[i] + a43 * dt * R[i];
  memcpy(o->resid0, R, sizeof(double) * n);
  rdt = rdt * a42 + a43 * dt;
  o->ctime = old_time + rdt;
  orc_compresid(o);
  double a51 = 0.00683325884039, a52 = 0.51723167208978, a53 = 0.12759831133288, a54 = 0.34833675773694,
         a55 = 0.08460416338212, a56 = 0.22600748319395;
  for (int64_t i = 0; i < n; i++)
    Q[i] = a51 * qj0[i] + a52 * o->qj2[i] + a53 * o->qj3[i] + a54 * Q[i] + a55 * dt * o->resid0[i] + a56 * dt * R[i];
  o->ctime = old_time + dt;
}

/* one pass of the loop body in iterations.f90:19-87 */
int orc_step(orc_t* o, double* residglob, double* divBglob) {
  o->iter = o->iter + 1;
  if (o->k_stage == 5) orc_fivestagerk(o);
  else orc_rk_s5p3(o);
  orc_correct_B_via_curl_Az(o);
  if (o->iter % 10 == 1) {
    orc_comp_inviscid_flux(o);
    orc_nablaQsp(o, 1, 9);
    int N = o->N;
    double rn = 0.0, db = 0.0;
    for (int ic = 0; ic < o->NCELL; ic++)
      for (int js = 0; js < N; js++)
        for (int is = 0; is < N; is++) {
          for (int k = 0; k < 9; k++) { double r = o->resid[IDX_Q(o, k, is, js, ic)]; rn = rn + r * r; }
          double d = o->nablaQs[IDX_NQS(o, 5, 0, is, js, ic)] + o->nablaQs[IDX_NQS(o, 6, 1, is, js, ic)];
          db = db + d * d;
        }
    double rg = 0.0 + rn, dg = 0.0 + db;
    if (residglob) *residglob = sqrt(rg / (o->NCELLGLOB * N * N * 5));
    if (divBglob) *divBglob = sqrt(dg / (o->NCELLGLOB * N * N));
    return 1;
  }
  return 0;
}

int orc_run(orc_t* o, int nsteps) {
  for (int s = 0; s < nsteps; s++) orc_step(o, NULL, NULL);
  return nsteps;
}

/* =====================================================================
 * Initial conditions (setinitialcond.f90:1-80 and EXTENSION problems)
 * ===================================================================== */
static void ic_point(const orc_t* o, double x, double y, const double* Bproj, double Qv[9]) {
  double gam = o->gam, rho, u, v, w, pr, Bx, By, Bz, Az;
  if (o->problem == 1) {
    /* EXTENSION: MHD rotor (Balsara & Spicer 1999) on [0,1]^2 */
    const double r0 = 0.1, r1 = 0.115, u0 = 2.0;
    double dx = x - 0.5, dy = y - 0.5, r = sqrt(dx * dx + dy * dy);
    if (r < r0) { rho = 10.0; u = -u0 * dy / r0; v = u0 * dx / r0; }
    else if (r < r1) { double f = (r1 - r) / (r1 - r0); rho = 1.0 + 9.0 * f; u = -f * u0 * dy / r; v = f * u0 * dx / r; }
    else { rho = 1.0; u = 0.0; v = 0.0; }
    w = 0.0;
    pr = 1.0;
    double bx0 = 5.0 / sqrt(4.0 * PI);
    Bx = bx0; By = 0.0; Bz = 0.0;
    Az = bx0 * y;
  } else if (o->problem == 2) {
    /* EXTENSION: circularly polarised Alfven wave (Toth 2000), angle 30 deg,
     * amplitude 0.1; A_z stores only the periodic part dA (B = B0 + curl dA). */
    const double ca = sqrt(3.0) / 2.0, sa = 0.5, amp = 0.1, tp = 2.0 * PI;
    double xp = x * ca + y * sa;
    double vperp = amp * sin(tp * xp), vz = amp * cos(tp * xp);
    rho = 1.0; pr = 0.1;
    u = -vperp * sa; v = vperp * ca; w = vz;
    double bpar = 1.0, bperp = amp * sin(tp * xp);
    Bx = bpar * ca - bperp * sa; By = bpar * sa + bperp * ca; Bz = amp * cos(tp * xp);
    Az = amp * cos(tp * xp) / tp;
  } else {
    /* Orszag-Tang setinitialcond.f90:16-35 */
    rho = gam * gam;
    u = -sin(y);
    v = sin(x);
    w = 0.0;
    pr = gam;
    Bx = -sin(y);
    By = sin(x * 2);
    Bz = 0.0;
    Az = 0.5 * cos(x * 2) + cos(y);
  }
  if (Bproj) { Bx = Bproj[0]; By = Bproj[1]; Bz = Bproj[2]; }
  double NORM_U = u * u + v * v + w * w, NORM_B = Bx * Bx + By * By + Bz * Bz;
  Qv[0] = rho;
  Qv[1] = rho * u;
  Qv[2] = rho * v;
  Qv[3] = rho * w;
  Qv[4] = pr / (gam - 1) + 0.5 * rho * NORM_U + 0.5 * NORM_B;
  Qv[5] = Bx;
  Qv[6] = By;
  Qv[7] = Bz;
  Qv[8] = Az;
}

/* SETINITIALCOND setinitialcond.f90:1-80 */
static void setinitialcond(orc_t* o) {
  int N = o->N;
  for (int ic = 0; ic < o->NCELL; ic++)
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        double x = o->XXsolu[0 + 2 * IDX_J(o, is, js, ic)], y = o->XXsolu[1 + 2 * IDX_J(o, is, js, ic)];
        ic_point(o, x, y, NULL, &o->Q[IDX_Q(o, 0, is, js, ic)]);
      }
  o->ctime = 0.0;
  o->iter = 0;
  orc_correct_B_via_curl_Az(o);
  for (int ic = 0; ic < o->NCELL; ic++)
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        double x = o->XXsolu[0 + 2 * IDX_J(o, is, js, ic)], y = o->XXsolu[1 + 2 * IDX_J(o, is, js, ic)];
        double* q = &o->Q[IDX_Q(o, 0, is, js, ic)];
        double B[3] = {q[5], q[6], q[7]};
        ic_point(o, x, y, B, q);
      }
}

/* INIT_SETUP initsetup.f90:1-165 */
static int init_setup(orc_t* o, char* err, int errlen) {
  int N = o->N, NC = o->NCELL;
  o->Xs = dalloc(N);
  o->Xf = dalloc(N + 1);
  o->Lmat = dalloc((int64_t)(N + 1) * N);
  o->Mmat = dalloc((int64_t)(N + 1) * N);
  setsandpoints(N, o->Xs, o->Xf);
  computeLandM(o);
  int64_t ns = (int64_t)N * N * NC, nf = (int64_t)(N + 1) * N * NC;
  o->XXsolu = dalloc(2 * ns);
  o->Jac = dalloc(ns);
  o->S1 = dalloc(4 * nf);
  o->S2 = dalloc(4 * nf);
  o->Q = dalloc(9 * ns);
  o->Qvfi = dalloc(9 * nf);
  o->Qvfj = dalloc(9 * nf);
  o->F1 = dalloc(8 * nf);
  o->G2 = dalloc(8 * nf);
  o->resid = dalloc(9 * ns);
  o->Fv1 = dalloc(9 * nf);
  o->Gv2 = dalloc(9 * nf);
  o->SM_IND = dalloc(9 * (int64_t)NC);
  o->muAV = dalloc(9 * (int64_t)NC);
  o->muAVfi = dalloc(18 * (int64_t)NC);
  o->muAVfj = dalloc(18 * (int64_t)NC);
  o->Xs_low = dalloc(N - 1 > 0 ? N - 1 : 1);
  o->Xf_low = dalloc(N);
  setsandpoints(N - 1, o->Xs_low, o->Xf_low);
  o->nablaQs = dalloc(18 * ns);
  o->nablaQvfi = dalloc(18 * nf);
  o->nablaQvfj = dalloc(18 * nf);
  o->nablaAs = dalloc(2 * ns);
  o->Azfi = dalloc(nf);
  o->Azfj = dalloc(nf);
  o->Qk0 = dalloc(9 * ns);
  o->Qka = dalloc(9 * ns);
  o->qj2 = dalloc(9 * ns);
  o->qj3 = dalloc(9 * ns);
  o->resid0 = dalloc(9 * ns);
  if (!o->resid0) { snprintf(err, errlen, "out of memory"); return -1; }
  calcjacob(o);
  for (int ic = 0; ic < NC; ic++) {
    double xs[2][4];
    for (int iv = 0; iv < 4; iv++) {
      xs[0][iv] = o->XV[IVCELL_(o, ic, iv) - 1];
      xs[1][iv] = o->YV[IVCELL_(o, ic, iv) - 1];
    }
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        double xx[2];
        xycoor(xs, o->Xs[is], o->Xs[js], xx);
        o->XXsolu[0 + 2 * IDX_J(o, is, js, ic)] = xx[0];
        o->XXsolu[1 + 2 * IDX_J(o, is, js, ic)] = xx[1];
      }
  }
  face2fpconnec(o);
  if (o->restart == 0) setinitialcond(o);
  else if (o->restart == 1 && o->restart_ord == N) {
    if (orc_read_restart(o, o->namerestart) != 0) { snprintf(err, errlen, "cannot read restart %s", o->namerestart); return -1; }
  }
  return 0;
}

orc_t* orc_load(const char* dir, char* err, int errlen) {
  orc_t* o = (orc_t*)calloc(1, sizeof(orc_t));
  if (!o) return NULL;
  if (readinput(o, dir, err, errlen) || read_grid(o, err, errlen) || check_mesh(o, err, errlen) ||
      connectivity(o, err, errlen) || connect_bdry(o, err, errlen) || mapcycloc(o, err, errlen) ||
      init_setup(o, err, errlen)) {
    orc_free(o);
    return NULL;
  }
  return o;
}

void orc_free(orc_t* o) {
  if (!o) return;
  void* ptrs[] = {o->IVCELL, o->XV, o->YV, o->IVGBOUN, o->IBOUNTYPE, o->IVG2IV, o->ICVSTA, o->ICVERT,
                  o->IC2F, o->IF2C, o->IF2V, o->IBFINTER, o->IBFREE, o->IBFCYC, o->IBFCYCLOC, o->CYC2FPAIR,
                  o->Xs, o->Xf, o->Lmat, o->Mmat, o->Xs_low, o->Xf_low, o->dmdxs, o->dmdxf1, o->dmdxf2,
                  o->Jac, o->S1, o->S2, o->XXsolu, o->Q, o->F1, o->G2, o->Fv1, o->Gv2, o->resid, o->Qvfi,
                  o->Qvfj, o->nablaQs, o->nablaQvfi, o->nablaQvfj, o->Azfi, o->Azfj, o->nablaAs, o->muAV,
                  o->muAVfi, o->muAVfj, o->SM_IND, o->Qk0, o->Qka, o->qj2, o->qj3, o->resid0,
                  o->gnumnode, o->gnode_factor, o->connec_c2n, o->plotX, o->plotQ, o->plotAV};
  for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++) free(ptrs[i]);
  free(o);
}

/* =====================================================================
 * Plot output for one rank: tecplotter2dsetup (tecplotter2dsetup.f90:1-177),
 * tecplotter2d (tecplotter.f90:1-86), tecpost_parallel (tecplotter.f90:92-418).
 * smooth_procint_plot (smooth_procint_plot.f90) only adds the contributions of nodes
 * on processor interfaces; with one partition there are none.
 * ===================================================================== */
/* distcalc tecplotter2dsetup.f90:160-172 */
static double plot_dist(const orc_t* o, const double xx[2], int gnid) {
  double d = sqrt((xx[0] - o->plotX[2 * (gnid - 1)]) * (xx[0] - o->plotX[2 * (gnid - 1)]) +
                  (xx[1] - o->plotX[2 * (gnid - 1) + 1]) * (xx[1] - o->plotX[2 * (gnid - 1) + 1]));
  return fabs(d);
}

/* tecplotter2dsetup.f90:1-177 (CURVE_WALL = 0); gnumnode(ii,jj,icell) 1-based values */
int orc_plot_setup(orc_t* o, int nre) {
  const int Np = nre, NC = o->NCELL;
  if (Np < 1) return -1;
  free(o->gnumnode); free(o->gnode_factor); free(o->connec_c2n); free(o->plotX);
  free(o->plotQ); free(o->plotAV);
  o->plotQ = o->plotAV = NULL;
  const int64_t nn = (int64_t)(Np + 1) * (Np + 1) * NC;
  o->gnumnode = ialloc(nn);
  o->gnode_factor = ialloc(nn);
  o->plotX = dalloc(2 * nn);
  o->connec_c2n = ialloc(4 * (int64_t)Np * Np * NC);
  int* isfacenod = ialloc(o->NFACE);
  const int ne = Np - 1 > 0 ? Np - 1 : 1;
  int* gfacenode = ialloc((int64_t)ne * o->NFACE);
  int plotnodes = 0, plotcells = 0, bad = 0;
  const double tolplot = 1e-5;
#define GNUM(ii, jj, ic) o->gnumnode[((ii) - 1) + (Np + 1) * (((jj) - 1) + (Np + 1) * (int64_t)(ic))]
  /* the 4 vertices of each cell are global nodes :30-52 */
  for (int ic = 0; ic < NC; ic++) {
    int v[4];
    for (int k = 0; k < 4; k++) v[k] = IVCELL_(o, ic, k);
    GNUM(1, 1, ic) = v[0];
    GNUM(Np + 1, 1, ic) = v[1];
    GNUM(Np + 1, Np + 1, ic) = v[2];
    GNUM(1, Np + 1, ic) = v[3];
    for (int k = 0; k < 4; k++) {
      int gnid = v[k];
      if (o->gnode_factor[gnid - 1] == 0) {
        plotnodes++;
        o->plotX[2 * (gnid - 1)] = o->XV[gnid - 1];
        o->plotX[2 * (gnid - 1) + 1] = o->YV[gnid - 1];
      }
      o->gnode_factor[gnid - 1]++;
    }
  }
  if (plotnodes != o->NVERT) bad = 1; /* :54-56 */
  for (int ic = 0; ic < NC; ic++) {
    double xs[2][4];
    for (int j = 0; j < 4; j++) {
      xs[0][j] = o->XV[IVCELL_(o, ic, j) - 1];
      xs[1][j] = o->YV[IVCELL_(o, ic, j) - 1];
    }
    /* nodes on the 4 faces, shared with the neighbour through the face :67-123 */
    for (int k = 1; k <= 4; k++) {
      int iface = IC2F_(o, ic, k - 1);
      for (int enode = 1; enode <= Np - 1; enode++) {
        int ii, jj;
        switch (k) {
          case 1: ii = enode + 1; jj = 1; break;
          case 2: ii = Np + 1; jj = enode + 1; break;
          case 3: ii = Np + 1 - enode; jj = Np + 1; break;
          default: ii = 1; jj = Np + 1 - enode; break;
        }
        double xsi = (double)(ii - 1) / (double)Np, eta = (double)(jj - 1) / (double)Np, rx[2];
        xycoor(xs, xsi, eta, rx);
        if (isfacenod[iface - 1] == 1) {
          int checkmatch = 0;
          for (int existnode = 1; existnode <= Np - 1; existnode++) {
            int gnid = gfacenode[(existnode - 1) + (int64_t)ne * (iface - 1)];
            if (plot_dist(o, rx, gnid) <= tolplot) {
              GNUM(ii, jj, ic) = gnid;
              o->gnode_factor[gnid - 1]++;
              checkmatch = 1;
            }
          }
          if (!checkmatch) bad = 1;
        } else {
          plotnodes++;
          o->plotX[2 * (plotnodes - 1)] = rx[0];
          o->plotX[2 * (plotnodes - 1) + 1] = rx[1];
          GNUM(ii, jj, ic) = plotnodes;
          gfacenode[(enode - 1) + (int64_t)ne * (iface - 1)] = plotnodes;
          o->gnode_factor[plotnodes - 1]++;
        }
      }
      if (isfacenod[iface - 1] == 0) isfacenod[iface - 1] = 1;
    }
    /* interior nodes :127-137 */
    for (int ii = 2; ii <= Np; ii++)
      for (int jj = 2; jj <= Np; jj++) {
        double xsi = (double)(ii - 1) / (double)Np, eta = (double)(jj - 1) / (double)Np, rx[2];
        xycoor(xs, xsi, eta, rx);
        plotnodes++;
        o->plotX[2 * (plotnodes - 1)] = rx[0];
        o->plotX[2 * (plotnodes - 1) + 1] = rx[1];
        GNUM(ii, jj, ic) = plotnodes;
        o->gnode_factor[plotnodes - 1]++;
      }
    /* plot cells :139-148 */
    for (int ii = 1; ii <= Np; ii++)
      for (int jj = 1; jj <= Np; jj++) {
        plotcells++;
        int* c = o->connec_c2n + 4 * (int64_t)(plotcells - 1);
        c[0] = GNUM(ii, jj, ic);
        c[1] = GNUM(ii + 1, jj, ic);
        c[2] = GNUM(ii + 1, jj + 1, ic);
        c[3] = GNUM(ii, jj + 1, ic);
      }
  }
#undef GNUM
  free(isfacenod);
  free(gfacenode);
  o->plot_nre = Np;
  o->plotnodes = plotnodes;
  o->plotcells = plotcells;
  return bad ? 1 : 0;
}

/* hval tecplotter.f90:62-82: Lagrange basis i (1-based) through Xs at xval */
static double plot_hval(const orc_t* o, int np, int i, double xval) {
  double hvaln = 1.0, hvald = 1.0;
  for (int s = 1; s <= np; s++)
    if (s != i) {
      hvaln = hvaln * (xval - o->Xs[s - 1]);
      hvald = hvald * (o->Xs[i - 1] - o->Xs[s - 1]);
    }
  return hvaln / hvald;
}

/* tecplotter2d tecplotter.f90:1-59: conservative state summed over the cells sharing a
 * node, averaged, converted to (rho,u,v,w,p,Bx,By,Bz,Az); muAV(1) and muAV(6) likewise.
 * With ARTIV = 0 the reference never allocates muAV; the plot carries zeros there. */
int orc_plot_eval(orc_t* o) {
  if (!o->gnumnode) return -1;
  const int Np = o->plot_nre, N = o->N;
  free(o->plotQ); free(o->plotAV);
  o->plotQ = dalloc(9 * (int64_t)o->plotnodes);
  o->plotAV = dalloc(2 * (int64_t)o->plotnodes);
  for (int ic = 0; ic < o->NCELL; ic++)
    for (int jj = 1; jj <= Np + 1; jj++)
      for (int ii = 1; ii <= Np + 1; ii++) {
        double xsi = (double)(ii - 1) / (double)Np, eta = (double)(jj - 1) / (double)Np;
        int gnid = o->gnumnode[(ii - 1) + (Np + 1) * ((jj - 1) + (Np + 1) * (int64_t)ic)];
        double Qs[NV] = {0};
        for (int js = 1; js <= N; js++)
          for (int is = 1; is <= N; is++)
            for (int k = 0; k < NV; k++)
              Qs[k] = Qs[k] + o->Q[IDX_Q(o, k, is - 1, js - 1, ic)] * plot_hval(o, N, is, xsi) * plot_hval(o, N, js, eta);
        for (int k = 0; k < NV; k++) o->plotQ[k + 9 * (int64_t)(gnid - 1)] += Qs[k];
        if (o->ARTIV == 1) {
          o->plotAV[2 * (int64_t)(gnid - 1)] += o->muAV[0 + 9 * ic];
          o->plotAV[2 * (int64_t)(gnid - 1) + 1] += o->muAV[5 + 9 * ic];
        }
      }
  const double gam = o->gam;
  for (int nd = 0; nd < o->plotnodes; nd++) {
    double* pq = o->plotQ + 9 * (int64_t)nd;
    double Qs[NV];
    for (int k = 0; k < NV; k++) Qs[k] = pq[k] / (double)o->gnode_factor[nd];
    pq[0] = Qs[0];
    pq[1] = Qs[1] / Qs[0];
    pq[2] = Qs[2] / Qs[0];
    pq[3] = Qs[3] / Qs[0];
    for (int k = 5; k < 9; k++) pq[k] = Qs[k];
    double NORM_U = pq[1] * pq[1] + pq[2] * pq[2] + pq[3] * pq[3];
    double NORM_B = pq[5] * pq[5] + pq[6] * pq[6] + pq[7] * pq[7];
    pq[4] = (Qs[4] - 0.5 * Qs[0] * NORM_U - 0.5 * NORM_B) * (gam - 1);
    o->plotAV[2 * (int64_t)nd] = o->plotAV[2 * (int64_t)nd] / (double)o->gnode_factor[nd];
    o->plotAV[2 * (int64_t)nd + 1] = o->plotAV[2 * (int64_t)nd + 1] / (double)o->gnode_factor[nd];
  }
  return 0;
}

/* write_tecplot_string tecplotter.f90:399-416: characters as int32, then a zero */
static void tec_string(FILE* f, const char* s) {
  int32_t v;
  for (; *s; s++) { v = (unsigned char)*s; fwrite(&v, 4, 1, f); }
  v = 0;
  fwrite(&v, 4, 1, f);
}

/* file name tecplotter.f90:179-180: 'TEC', int(ctime) as i7.7, the fraction written
 * with f6.3 minus its leading blank and integer digit, '.plt' */
int orc_plot_filename(double ctime, char* out, int n) {
  char dec[32];
  snprintf(dec, sizeof dec, "%6.3f", ctime - (double)(int)ctime);
  return snprintf(out, (size_t)n, "TEC%07d%.4s.plt", (int)ctime, dec + 2);
}

/* tecpost_parallel tecplotter.f90:92-418 for one rank: Tecplot binary (#!TDV111), one
 * FEQUADRILATERAL zone, block packing, float32 fields, 0-based connectivity */
int orc_plot_write(const orc_t* o, double ctime, const char* path) {
  if (!o->plotQ) return -1;
  FILE* f = fopen(path, "wb");
  if (!f) return -1;
  const int nvar = 13, n = o->plotnodes;
  double minmax[2 * 13];
  for (int v = 0; v < nvar; v++) {
    double lo = 0, hi = 0;
    for (int nd = 0; nd < n; nd++) {
      double x = v < 2 ? o->plotX[2 * (int64_t)nd + v] : v < 11 ? o->plotQ[9 * (int64_t)nd + (v - 2)]
                                                                 : o->plotAV[2 * (int64_t)nd + (v - 11)];
      if (nd == 0 || x < lo) lo = x;
      if (nd == 0 || x > hi) hi = x;
    }
    minmax[2 * v] = lo;
    minmax[2 * v + 1] = hi;
  }
  const float ZONEMARKER = 299.0f, EOHMARKER = 357.0f;
  fwrite("#!TDV111", 1, 8, f);
  int32_t it[16] = {1, 0};
  fwrite(it, 4, 2, f);
  tec_string(f, "step data");
  int32_t nv = nvar;
  fwrite(&nv, 4, 1, f);
  const char* names[13] = {"X", "Y", "RHO", "U", "V", "W", "P", "Bx", "By", "Bz", "Az", "muAV", "etaAV"};
  for (int v = 0; v < nvar; v++) tec_string(f, names[v]);
  fwrite(&ZONEMARKER, 4, 1, f);
  tec_string(f, "ZONE 001");
  int32_t pz[2] = {-1, 0};
  fwrite(pz, 4, 2, f);
  fwrite(&ctime, 8, 1, f);
  int32_t zh[12] = {-1, 3, 0, 0, 0, 0, n, o->plotcells, 0, 0, 0, 0};
  fwrite(zh, 4, 12, f);
  fwrite(&EOHMARKER, 4, 1, f);
  fwrite(&ZONEMARKER, 4, 1, f);
  for (int v = 0; v < nvar; v++) it[v] = 1;
  it[nvar] = 0;
  it[nvar + 1] = 0;
  it[nvar + 2] = -1;
  fwrite(it, 4, nvar + 3, f);
  fwrite(minmax, 8, 2 * nvar, f);
  float* buf = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
  for (int v = 0; v < nvar; v++) {
    for (int nd = 0; nd < n; nd++)
      buf[nd] = (float)(v < 2 ? o->plotX[2 * (int64_t)nd + v] : v < 11 ? o->plotQ[9 * (int64_t)nd + (v - 2)]
                                                                        : o->plotAV[2 * (int64_t)nd + (v - 11)]);
    fwrite(buf, 4, (size_t)n, f);
  }
  free(buf);
  for (int64_t i = 0; i < 4 * (int64_t)o->plotcells; i++) {
    int32_t c = o->connec_c2n[i] - 1;
    fwrite(&c, 4, 1, f);
  }
  int rc = ferror(f) ? -1 : 0;
  fclose(f);
  return rc;
}

/* =====================================================================
 * Restart stream: int32 iter, float64 ctime, then per cell int32 global id and
 * Q(9,N,N) (write_data.f90:44-74, read_data_restart.f90:35-67).
 * ===================================================================== */
int orc_write_restart(const orc_t* o, const char* path) {
  FILE* f = fopen(path, "wb");
  if (!f) return -1;
  int32_t it = o->iter;
  fwrite(&it, 4, 1, f);
  fwrite(&o->ctime, 8, 1, f);
  int nq = 9 * o->N * o->N;
  for (int ic = 0; ic < o->NCELL; ic++) {
    int32_t g = ic + 1;
    fwrite(&g, 4, 1, f);
    fwrite(&o->Q[(int64_t)nq * ic], 8, nq, f);
  }
  fclose(f);
  return 0;
}

int orc_read_restart(orc_t* o, const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  int32_t it;
  int nq = 9 * o->N * o->N;
  if (fread(&it, 4, 1, f) != 1 || fread(&o->ctime, 8, 1, f) != 1) { fclose(f); return -1; }
  o->iter = it;
  for (int i = 0; i < o->NCELLGLOB; i++) {
    int32_t g;
    if (fread(&g, 4, 1, f) != 1) { fclose(f); return -1; }
    if (g < 1 || g > o->NCELL) { fclose(f); return -1; }
    if (fread(&o->Q[(int64_t)nq * (g - 1)], 8, nq, f) != (size_t)nq) { fclose(f); return -1; }
  }
  fclose(f);
  return 0;
}

/* =====================================================================
 * Accessors
 * ===================================================================== */
int orc_geti(const orc_t* o, const char* n) {
  if (!strcmp(n, "N")) return o->N;
  if (!strcmp(n, "NCELL")) return o->NCELL;
  if (!strcmp(n, "NFACE")) return o->NFACE;
  if (!strcmp(n, "NINTER")) return o->NINTER;
  if (!strcmp(n, "NFREE")) return o->NFREE;
  if (!strcmp(n, "NPAIR")) return o->NPAIR;
  if (!strcmp(n, "NCYCL")) return o->NCYCL;
  if (!strcmp(n, "NCYCLOC")) return o->NCYCLOC;
  if (!strcmp(n, "NVERT")) return o->NVERT;
  if (!strcmp(n, "k_stage")) return o->k_stage;
  if (!strcmp(n, "MAXITER")) return o->MAXITER;
  if (!strcmp(n, "vismode")) return o->vismode;
  if (!strcmp(n, "ARTIV")) return o->ARTIV;
  if (!strcmp(n, "iter")) return o->iter;
  if (!strcmp(n, "problem")) return o->problem;
  if (!strcmp(n, "nwrite")) return o->nwrite;
  if (!strcmp(n, "NRE")) return o->NRE;
  if (!strcmp(n, "plotnodes")) return o->plotnodes;
  if (!strcmp(n, "plotcells")) return o->plotcells;
  return -1;
}
double orc_getd(const orc_t* o, const char* n) {
  if (!strcmp(n, "dt")) return o->dt;
  if (!strcmp(n, "ctime")) return o->ctime;
  if (!strcmp(n, "mu")) return o->mu;
  if (!strcmp(n, "eta0")) return o->eta0;
  if (!strcmp(n, "gam")) return o->gam;
  if (!strcmp(n, "DXCYCL")) return o->DXCYCL;
  if (!strcmp(n, "DYCYCL")) return o->DYCYCL;
  if (!strcmp(n, "eigvmax")) return o->eigvmax;
  if (!strcmp(n, "eigvmax_g")) return o->eigvmax_g;
  if (!strcmp(n, "epsilon0")) return o->epsilon0;
  if (!strcmp(n, "B0x")) return o->B0x;
  if (!strcmp(n, "B0y")) return o->B0y;
  return NAN;
}
int orc_setd(orc_t* o, const char* n, double v) {
  if (!strcmp(n, "dt")) o->dt = v;
  else if (!strcmp(n, "ctime")) o->ctime = v;
  else if (!strcmp(n, "mu")) o->mu = v;
  else if (!strcmp(n, "eta0")) o->eta0 = v;
  else if (!strcmp(n, "eigvmax")) o->eigvmax = v;
  else return -1;
  return 0;
}
int orc_seti(orc_t* o, const char* n, int v) {
  if (!strcmp(n, "ARTIV")) o->ARTIV = v;
  else if (!strcmp(n, "vismode")) o->vismode = v;
  else if (!strcmp(n, "k_stage")) o->k_stage = v;
  else if (!strcmp(n, "iter")) o->iter = v;
  else return -1;
  return 0;
}

double* orc_darray(orc_t* o, const char* n, int64_t* count) {
  int64_t N = o->N, NC = o->NCELL, ns = N * N * NC, nf = (N + 1) * N * NC;
  struct { const char* name; double* p; int64_t c; } t[] = {
      {"Q", o->Q, 9 * ns},           {"resid", o->resid, 9 * ns},      {"F1", o->F1, 8 * nf},
      {"G2", o->G2, 8 * nf},         {"Fv1", o->Fv1, 9 * nf},          {"Gv2", o->Gv2, 9 * nf},
      {"Qvfi", o->Qvfi, 9 * nf},     {"Qvfj", o->Qvfj, 9 * nf},        {"nablaQs", o->nablaQs, 18 * ns},
      {"nablaQvfi", o->nablaQvfi, 18 * nf}, {"nablaQvfj", o->nablaQvfj, 18 * nf},
      {"Azfi", o->Azfi, nf},         {"Azfj", o->Azfj, nf},            {"nablaAs", o->nablaAs, 2 * ns},
      {"S1", o->S1, 4 * nf},         {"S2", o->S2, 4 * nf},            {"Jac", o->Jac, ns},
      {"Lmat", o->Lmat, (N + 1) * N}, {"Mmat", o->Mmat, (N + 1) * N},  {"Xs", o->Xs, N},
      {"Xf", o->Xf, N + 1},          {"XV", o->XV, o->NVERT},          {"YV", o->YV, o->NVERT},
      {"muAV", o->muAV, 9 * NC},     {"muAVfi", o->muAVfi, 18 * NC},   {"muAVfj", o->muAVfj, 18 * NC},
      {"SM_IND", o->SM_IND, 9 * NC}, {"XXsolu", o->XXsolu, 2 * ns},    {"Qk0", o->Qk0, 9 * ns},
      {"Xs_low", o->Xs_low, N - 1},  {"plotX", o->plotX, 2 * (int64_t)o->plotnodes},
      {"plotQ", o->plotQ, 9 * (int64_t)o->plotnodes}, {"plotAV", o->plotAV, 2 * (int64_t)o->plotnodes},
  };
  for (size_t i = 0; i < sizeof t / sizeof t[0]; i++)
    if (!strcmp(n, t[i].name)) { if (count) *count = t[i].c; return t[i].p; }
  if (count) *count = 0;
  return NULL;
}

int32_t* orc_iarray(orc_t* o, const char* n, int64_t* count) {
  struct { const char* name; int* p; int64_t c; } t[] = {
      {"IF2C", o->IF2C, 4 * (int64_t)o->NFACE},   {"IC2F", o->IC2F, 4 * (int64_t)o->NCELL},
      {"IF2V", o->IF2V, 2 * (int64_t)o->NFACE},   {"IVCELL", o->IVCELL, 4 * (int64_t)o->NCELL},
      {"IBFINTER", o->IBFINTER, o->NINTER},       {"IBFREE", o->IBFREE, o->NFREE},
      {"IBFCYC", o->IBFCYC, o->NCYCL},            {"IBFCYCLOC", o->IBFCYCLOC, o->NCYCLOC},
      {"CYC2FPAIR", o->CYC2FPAIR, 2 * (int64_t)o->NPAIR},
      {"iface2fp", o->iface2fp, 4 * (int64_t)o->N}, {"jface2fp", o->jface2fp, 4 * (int64_t)o->N},
      {"gnumnode", o->gnumnode, (int64_t)(o->plot_nre + 1) * (o->plot_nre + 1) * o->NCELL},
      {"gnode_factor", o->gnode_factor, o->plotnodes}, {"connec_c2n", o->connec_c2n, 4 * (int64_t)o->plotcells},
  };
  for (size_t i = 0; i < sizeof t / sizeof t[0]; i++)
    if (!strcmp(n, t[i].name)) { if (count) *count = t[i].c; return (int32_t*)t[i].p; }
  if (count) *count = 0;
  return NULL;
}
