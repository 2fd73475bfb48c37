// mesh.cpp -- host-side setup for callers without the Fortran setup chain.
//
// Reads QUAD.INP (readinput.f90:6-36) and the .CEL/.VRT/.BND files
// (readGRIDinfo.f90:1-259) and rebuilds the reference's integer maps and geometry:
//   * CHECK_MESH (connectivity.f90:236-283): reject cells whose corner cross products
//     change sign (the reference's orientation "fix" is a no-op, so cells must be ccw);
//   * CONNECTIVITY (connectivity.f90:1-233): faces are numbered in the order the
//     reference discovers them -- cell-major, local faces 1..4, a face taking the next
//     id when its first owner is visited.  The reference searches the vertex->cell
//     lists for the partner; here an edge hash map gives it in O(1), and the result is
//     identical for every conforming mesh (a non-manifold edge is rejected);
//   * CONNECT_BDRY (connect_bdry.f90:1-354): boundary faces in .BND order, the
//     interior-face list in face order; every boundary face must be listed;
//   * MAPCYCLOC (map_cyc_loc.f90:1-42): periodic partners by face-midpoint match with
//     the reference's tolerance test, found through a bucket grid instead of the
//     O(n^2) double loop, pairs emitted in the same order;
//   * setsandpoints / computeLandM / face2fpconnec (initsetup.f90:167-379),
//     mapder + calcjacob (mapder.f90:1-76, calcjacob.f90:1-86) and the solution-point
//     coordinates (initsetup.f90:88-112), in the reference's evaluation order (this
//     file is compiled with -ffp-contract=off so the metrics match bit for bit).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>
#include <algorithm>

#include "chorus_internal.h"

namespace chorus {

static const double kPi = 3.14159265358979323846;  // atan(1.d0)*4.d0
static const double kTolCyc = 1e-5;                 // setup2d.f90:64

static std::string trim_token(const std::string& line) {
  std::istringstream is(line);
  std::string t;
  is >> t;
  if (!t.empty() && (t[0] == '\'' || t[0] == '"')) {
    char q = t[0];
    t = t.substr(1);
    size_t p = t.find(q);
    if (p != std::string::npos) t = t.substr(0, p);
  }
  return t;
}

static double fortran_real(const std::string& s) {
  std::string t = trim_token(s);
  for (auto& c : t)
    if (c == 'D' || c == 'd') c = 'E';
  return std::strtod(t.c_str(), nullptr);
}

static int read_lines(const std::string& path, std::vector<std::string>& out) {
  std::ifstream f(path);
  if (!f) return -1;
  std::string l;
  while (std::getline(f, l)) out.push_back(l);
  // a file without a trailing newline still counts its last record
  return 0;
}

// setsandpoints initsetup.f90:167-255
void setsandpoints(int np, double* xs, double* xf) {
  for (int i = 1; i <= np; i++) xs[i - 1] = 0.5 * (1.0 - std::cos((double)(2 * i - 1) * kPi / (2 * (double)np)));
  auto sym = [&](const double* g, int ng, bool mid) {
    xf[0] = 0.0;
    for (int q = 0; q < ng; q++) xf[1 + q] = (1.0 - g[q]) / 2.0;
    int o = 1 + ng;
    if (mid) xf[o++] = 0.5;
    for (int q = 0; q < ng; q++) xf[o + q] = (1.0 + g[ng - 1 - q]) / 2.0;
    xf[np] = 1.0;
  };
  switch (np) {
    case 1: xf[0] = 0.0; xf[1] = 1.0; break;
    case 2: xf[0] = 0.0; xf[1] = 0.5; xf[2] = 1.0; break;
    case 3: { double g[1] = {std::sqrt(3.0) / 3.0}; sym(g, 1, false); break; }
    case 4: { double g[1] = {std::sqrt(15.0) / 5.0}; sym(g, 1, true); break; }
    case 5: {
      double g[2] = {std::sqrt(525.0 + 70.0 * std::sqrt(30.0)) / 35.0, std::sqrt(525.0 - 70.0 * std::sqrt(30.0)) / 35.0};
      sym(g, 2, false);
      break;
    }
    case 6: {
      double g[2] = {std::sqrt(245.0 + 14.0 * std::sqrt(70.0)) / 21.0, std::sqrt(245.0 - 14.0 * std::sqrt(70.0)) / 21.0};
      sym(g, 2, true);
      break;
    }
    case 7: { double g[3] = {0.932469514203, 0.661209386466, 0.238619186083}; sym(g, 3, false); break; }
    case 8: { double g[3] = {0.949107912343, 0.741531185599, 0.405845151377}; sym(g, 3, true); break; }
    case 9: { double g[4] = {0.960289856498, 0.796666477414, 0.525532409916, 0.183434642496}; sym(g, 4, false); break; }
    case 10: { double g[4] = {0.968160239508, 0.836031107327, 0.613371432701, 0.324253423404}; sym(g, 4, true); break; }
    default: break;
  }
}

// Lagrange basis i (0-based) on nodes x[0..n) at xv: initsetup.f90:318-340 / AV.f90:176-197
double lagrange(const double* x, int n, int i, double xv) {
  double num = 1.0, den = 1.0;
  for (int s = 0; s < n; s++)
    if (s != i) { num = num * (xv - x[s]); den = den * (x[i] - x[s]); }
  return num / den;
}

// computeLandM initsetup.f90:258-315 (column-major (N+1,N))
void compute_L_M(int N, const double* Xs, const double* Xf, double* L, double* M) {
  for (int ifp = 0; ifp <= N; ifp++)
    for (int is = 0; is < N; is++) L[ifp + (N + 1) * is] = lagrange(Xs, N, is, Xf[ifp]);
  for (int ifp = 0; ifp <= N; ifp++)
    for (int is = 0; is < N; is++) {
      double xv = Xs[is], sum = 0.0;
      for (int k = 0; k <= N; k++) {
        if (k == ifp) continue;
        double num = 1.0, den = 1.0;
        for (int s = 0; s <= N; s++) {
          if (s != ifp && s != k) num = num * (xv - Xf[s]);
          if (s != ifp) den = den * (Xf[ifp] - Xf[s]);
        }
        sum = sum + num / den;
      }
      M[ifp + (N + 1) * is] = sum;
    }
}

namespace {

struct EdgeKey {
  int64_t k;
  bool operator==(const EdgeKey& o) const { return k == o.k; }
};
struct EdgeHash {
  size_t operator()(const EdgeKey& e) const { return std::hash<int64_t>()(e.k * 0x9E3779B97F4A7C15LL); }
};
inline EdgeKey edge_key(int a, int b) {
  int lo = a < b ? a : b, hi = a < b ? b : a;
  return EdgeKey{((int64_t)lo << 32) | (uint32_t)hi};
}

const int kIVFACE[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};  // connectivity.f90:73-83

}  // namespace

// QUAD.INP, the cell and vertex files with GLOB2LOCAL, and the boundary file's records
// (readinput.f90:6-36, readGRIDinfo.f90:1-259)
int mesh_parse(const std::string& dir, Mesh& m, std::vector<BndRecord>& bnd, std::string& err) {
  // ---- QUAD.INP (readinput.f90:6-36) + extension block
  std::vector<std::string> L;
  if (read_lines(dir + "/QUAD.INP", L) || L.size() < 29) {
    err = "cannot read 29 lines of " + dir + "/QUAD.INP";
    return CHORUS_EIO;
  }
  std::string ncel = trim_token(L[2]), nvrt = trim_token(L[3]), nbnd = trim_token(L[5]);
  m.N = std::atoi(L[9].c_str());
  int curve = std::atoi(L[10].c_str());
  m.params.vismode = std::atoi(L[11].c_str());
  m.params.mu = fortran_real(L[12]);
  m.params.eta0 = fortran_real(L[13]);
  m.params.k_stage = std::atoi(L[15].c_str());
  m.params.dt = fortran_real(L[16]);
  m.maxiter = std::atoi(L[17].c_str());
  m.params.DXCYCL = fortran_real(L[19]);
  m.params.DYCYCL = fortran_real(L[20]);
  m.params.ARTIV = std::atoi(L[22].c_str());
  m.nre = std::atoi(L[24].c_str());
  m.nwrite = std::atoi(L[25].c_str());
  m.restart = std::atoi(L[27].c_str());
  m.params.gam = 5.0 / 3;
  m.problem = 0;
  m.params.B0x = 0.0;
  m.params.B0y = 0.0;
  if (L.size() >= 31) m.params.gam = fortran_real(L[30]);
  if (L.size() >= 32) m.problem = std::atoi(L[31].c_str());
  if (L.size() >= 33) m.params.B0x = fortran_real(L[32]);
  if (L.size() >= 34) m.params.B0y = fortran_real(L[33]);
  if (m.N < 2 || m.N > kMaxN) { err = "N must be in 2.." + std::to_string(kMaxN); return CHORUS_EINVAL; }
  if (curve != 0) { err = "CURVE_WALL=1 is unfinished in the reference (initsetup.f90:71-78)"; return CHORUS_EINVAL; }
  if (m.params.vismode != 1) { err = "vismode must be 1: Qvfi/Azfi are only written when vismode==1"; return CHORUS_EINVAL; }
  if (m.params.k_stage != 3 && m.params.k_stage != 5) { err = "k_stage can be only 3 or 5"; return CHORUS_EINVAL; }

  // ---- cells (readGRIDinfo.f90:1-37)
  std::vector<std::string> C;
  if (read_lines(dir + "/" + ncel, C) || C.empty()) { err = "cannot read cell file " + ncel; return CHORUS_EIO; }
  int nglob = (int)C.size();
  std::vector<int> ivg(4 * (size_t)nglob);
  for (int i = 0; i < nglob; i++) {
    int ic, a, b, c, d;
    if (std::sscanf(C[i].c_str(), "%d %d %d %d %d", &ic, &a, &b, &c, &d) != 5) {
      err = "bad cell line " + std::to_string(i + 1);
      return CHORUS_EIO;
    }
    ivg[4 * i] = a; ivg[4 * i + 1] = b; ivg[4 * i + 2] = c; ivg[4 * i + 3] = d;
  }
  // ---- vertices FORMAT(I9,6X,3(D20.12,1X)) readGRIDinfo.f90:79-80
  std::vector<std::string> V;
  if (read_lines(dir + "/" + nvrt, V) || V.empty()) { err = "cannot read vertex file " + nvrt; return CHORUS_EIO; }
  int nvg = (int)V.size();
  std::vector<double> xg(nvg), yg(nvg);
  for (int i = 0; i < nvg; i++) {
    const std::string& s = V[i];
    if (s.size() < 56) { err = "short vertex line " + std::to_string(i + 1); return CHORUS_EIO; }
    std::string fx = s.substr(15, 20), fy = s.substr(36, 20);
    for (auto& c : fx) if (c == 'D' || c == 'd') c = 'E';
    for (auto& c : fy) if (c == 'D' || c == 'd') c = 'E';
    xg[i] = std::strtod(fx.c_str(), nullptr);
    yg[i] = std::strtod(fy.c_str(), nullptr);
  }
  // ---- GLOB2LOCAL (readGRIDinfo.f90:124-199): local ids by first appearance
  m.NCELL = nglob;
  m.IVCELL.assign(4 * (size_t)nglob, 0);
  std::vector<int> g2l(nvg + 1, 0);
  m.XV.clear();
  m.YV.clear();
  for (int ic = 0; ic < nglob; ic++)
    for (int k = 0; k < 4; k++) {
      int g = ivg[4 * ic + k];
      if (g < 1 || g > nvg) { err = "vertex id out of range in cell " + std::to_string(ic + 1); return CHORUS_EMESH; }
      if (!g2l[g]) {
        m.XV.push_back(xg[g - 1]);
        m.YV.push_back(yg[g - 1]);
        g2l[g] = (int)m.XV.size();
      }
      m.IVCELL[ic + (size_t)nglob * k] = g2l[g];
    }
  m.NVERT = (int)m.XV.size();
  // ---- boundary file (readGRIDinfo.f90:201-259): records on this partition, in order
  std::vector<std::string> B;
  read_lines(dir + "/" + nbnd, B);
  bnd.clear();
  for (size_t i = 0; i < B.size(); i++) {
    int ib, a, b, reg, pat;
    char ty[64] = {0};
    if (std::sscanf(B[i].c_str(), "%d %d %d %d %d %63s", &ib, &a, &b, &reg, &pat, ty) != 6) {
      err = "bad boundary line " + std::to_string(i + 1);
      return CHORUS_EIO;
    }
    std::string t(ty);
    t.erase(std::remove(t.begin(), t.end(), '\''), t.end());
    t.erase(std::remove(t.begin(), t.end(), '"'), t.end());
    if (a < 1 || a > nvg || b < 1 || b > nvg || !g2l[a] || !g2l[b]) continue;  // not on this partition
    bnd.push_back(BndRecord{(int)i + 1, g2l[a], g2l[b], t == "CYCL" ? 1 : (t == "FREE" ? 2 : 0), t});
  }
  return CHORUS_OK;
}

// CHECK_MESH, CONNECTIVITY and CONNECT_BDRY's boundary lists on the host
int mesh_maps_host(Mesh& m, const std::vector<BndRecord>& bnd, std::string& err) {
  const int NC = m.NCELL;
  auto ivcell = [&](int ic, int k) { return m.IVCELL[ic + (size_t)NC * k]; };

  // ---- CHECK_MESH
  for (int ic = 0; ic < NC; ic++) {
    double x[4], y[4];
    for (int k = 0; k < 4; k++) { x[k] = m.XV[ivcell(ic, k) - 1]; y[k] = m.YV[ivcell(ic, k) - 1]; }
    double v12x = x[1] - x[0], v12y = y[1] - y[0], v23x = x[2] - x[1], v23y = y[2] - y[1];
    double v34x = x[3] - x[2], v34y = y[3] - y[2];
    double c123 = v12x * v23y - v12y * v23x, c234 = v23x * v34y - v23y * v34x;
    if (c123 * c234 < 0) { err = "Problems in the mesh! cell " + std::to_string(ic + 1); return CHORUS_EMESH; }
    if (c123 < 0) { err = "cell " + std::to_string(ic + 1) + " is clockwise; the reference needs ccw cells"; return CHORUS_EMESH; }
  }

  // ---- CONNECTIVITY via an edge map: edge -> up to two (cell, local face)
  std::unordered_map<EdgeKey, std::pair<int, int>, EdgeHash> edges;
  edges.reserve((size_t)NC * 3);
  for (int ic = 0; ic < NC; ic++)
    for (int f = 0; f < 4; f++) {
      EdgeKey k = edge_key(ivcell(ic, kIVFACE[f][0]), ivcell(ic, kIVFACE[f][1]));
      auto it = edges.find(k);
      int code = ic * 4 + f;
      if (it == edges.end()) edges.emplace(k, std::make_pair(code, -1));
      else if (it->second.second < 0) it->second.second = code;
      else { err = "non-manifold edge at cell " + std::to_string(ic + 1); return CHORUS_EMESH; }
    }
  m.IC2F.assign(4 * (size_t)NC, 0);
  std::vector<int> f_c1, f_c2, f_v1, f_v2, f_l1, f_l2;
  f_c1.reserve(2 * (size_t)NC + 64);
  for (int ic = 0; ic < NC; ic++)
    for (int f = 0; f < 4; f++) {
      if (m.IC2F[ic + (size_t)NC * f]) continue;
      int va = ivcell(ic, kIVFACE[f][0]), vb = ivcell(ic, kIVFACE[f][1]);
      auto& e = edges[edge_key(va, vb)];
      int other = (e.first == ic * 4 + f) ? e.second : e.first;
      int id = (int)f_c1.size() + 1;
      m.IC2F[ic + (size_t)NC * f] = id;
      f_c1.push_back(ic + 1);
      f_v1.push_back(va);
      f_v2.push_back(vb);
      f_l1.push_back(f + 1);
      if (other >= 0) {
        int oc = other / 4, of = other % 4;
        // the partner face must run the other way round (both cells ccw)
        if (ivcell(oc, kIVFACE[of][0]) != vb || ivcell(oc, kIVFACE[of][1]) != va) {
          err = "Something wrong in connectivity! face " + std::to_string(id);
          return CHORUS_EMESH;
        }
        m.IC2F[oc + (size_t)NC * of] = id;
        f_c2.push_back(oc + 1);
        f_l2.push_back(of + 1);
      } else {
        f_c2.push_back(0);
        f_l2.push_back(0);
      }
    }
  const int NF = (int)f_c1.size();
  m.NFACE = NF;
  m.IF2C.assign(4 * (size_t)NF, 0);
  m.IF2V.assign(2 * (size_t)NF, 0);
  for (int f = 0; f < NF; f++) {
    m.IF2C[f] = f_c1[f];
    m.IF2C[f + (size_t)NF] = f_c2[f];
    m.IF2C[f + 2 * (size_t)NF] = f_l1[f];
    m.IF2C[f + 3 * (size_t)NF] = f_l2[f];
    m.IF2V[f] = f_v1[f];
    m.IF2V[f + (size_t)NF] = f_v2[f];
  }

  // ---- CONNECT_BDRY: boundary faces in .BND order
  std::vector<char> bflag(NF, 0);
  m.IBFCYC.clear();
  m.IBFREE.clear();
  for (const BndRecord& r : bnd) {
    auto it = edges.find(edge_key(r.a, r.b));
    if (it == edges.end()) { err = "boundary edge " + std::to_string(r.line) + " is not a cell face"; return CHORUS_EMESH; }
    if (it->second.second >= 0) { err = "boundary edge " + std::to_string(r.line) + " is an interior face"; return CHORUS_EMESH; }
    int code = it->second.first;
    int K = m.IC2F[(code / 4) + (size_t)NC * (code % 4)];
    int rc = boundary_face(m, r, K, bflag, err);
    if (rc) return rc;
  }
  m.IBFINTER.clear();
  for (int f = 0; f < NF; f++) {
    if (m.IF2C[f + (size_t)NF]) m.IBFINTER.push_back(f + 1);
    else if (!bflag[f]) { err = "boundary face " + std::to_string(f + 1) + " is missing from the BND file"; return CHORUS_EMESH; }
  }
  return CHORUS_OK;
}

// one boundary record whose face K (1-based) was found: its list by type (shared by the
// host and device setup paths, so both report the same errors in the same order)
int boundary_face(Mesh& m, const BndRecord& r, int K, std::vector<char>& bflag, std::string& err) {
  bflag[K - 1] = 1;
  if (r.kind == 1) m.IBFCYC.push_back(K);
  else if (r.kind == 2) m.IBFREE.push_back(K);
  else {
    err = "boundary type " + r.type + " has no flux routine in the reference (bcflux.f90 handles FREE only)";
    return CHORUS_EMESH;
  }
  return CHORUS_OK;
}

// MAPCYCLOC: periodic partners on the host (the list is the domain's perimeter)
int mesh_periodic(Mesh& m, std::string& err) {
  const int NF = m.NFACE;
  // ---- periodic faces: midpoint matching (connect_bdry.f90:275-314, map_cyc_loc.f90:1-42)
  const int NCY = (int)m.IBFCYC.size();
  std::vector<double> mx(NCY), my(NCY);
  for (int i = 0; i < NCY; i++) {
    int K = m.IBFCYC[i] - 1;
    mx[i] = (m.XV[m.IF2V[K] - 1] + m.XV[m.IF2V[K + (size_t)NF] - 1]) / 2;
    my[i] = (m.YV[m.IF2V[K] - 1] + m.YV[m.IF2V[K + (size_t)NF] - 1]) / 2;
  }
  const double DX = m.params.DXCYCL, DY = m.params.DYCYCL;
  auto match = [&](int i, int j) {
    double epsX = std::fabs(std::fabs(mx[i] - mx[j]) - DX);
    double epsY = std::fabs(std::fabs(my[i] - my[j]) - DY);
    return (epsX < kTolCyc && std::fabs(my[i] - my[j]) < kTolCyc) || (epsY < kTolCyc && std::fabs(mx[i] - mx[j]) < kTolCyc);
  };
  // bucket grid with cell size 4*tol; a partner lies at (x +- DX, y) or (x, y +- DY)
  const double cell = 4 * kTolCyc;
  std::unordered_map<int64_t, std::vector<int>> grid;
  auto gkey = [&](int64_t gx, int64_t gy) {  // unsigned shift: the bucket coordinates can be negative
    return (int64_t)(((uint64_t)gx << 32) ^ ((uint64_t)gy & 0xffffffffULL));
  };
  for (int i = 0; i < NCY; i++) grid[gkey((int64_t)std::floor(mx[i] / cell), (int64_t)std::floor(my[i] / cell))].push_back(i);
  std::vector<std::vector<int>> partners(NCY);
  const double shifts[4][2] = {{DX, 0}, {-DX, 0}, {0, DY}, {0, -DY}};
  for (int i = 0; i < NCY; i++) {
    for (auto& sh : shifts) {
      double qx = mx[i] + sh[0], qy = my[i] + sh[1];
      int64_t gx = (int64_t)std::floor(qx / cell), gy = (int64_t)std::floor(qy / cell);
      for (int64_t a = gx - 1; a <= gx + 1; a++)
        for (int64_t b = gy - 1; b <= gy + 1; b++) {
          auto it = grid.find(gkey(a, b));
          if (it == grid.end()) continue;
          for (int j : it->second)
            if (j != i && match(i, j)) partners[i].push_back(j);
        }
    }
    std::sort(partners[i].begin(), partners[i].end());
    partners[i].erase(std::unique(partners[i].begin(), partners[i].end()), partners[i].end());
    if (partners[i].empty()) {
      err = "periodic face " + std::to_string(m.IBFCYC[i]) + " has no partner (remote cyclic faces need MPI)";
      return CHORUS_EMESH;
    }
  }
  // every CYCL face is local here, so IBFCYCLOC is IBFCYC in order
  m.IBFCYCLOC = m.IBFCYC;
  m.CYC2FPAIR.clear();
  std::vector<int> p1, p2;
  for (int i = 0; i < NCY; i++)
    for (int j : partners[i])
      if (j > i) { p1.push_back(m.IBFCYC[i]); p2.push_back(m.IBFCYC[j]); }
  if ((int)p1.size() != NCY / 2) { err = "error in matching CYCLOC faces !!!"; return CHORUS_EMESH; }
  m.NPAIR = (int)p1.size();
  m.CYC2FPAIR.resize(2 * (size_t)m.NPAIR);
  for (int p = 0; p < m.NPAIR; p++) { m.CYC2FPAIR[p] = p1[p]; m.CYC2FPAIR[p + m.NPAIR] = p2[p]; }

  return CHORUS_OK;
}

// setsandpoints, computeLandM and face2fpconnec (initsetup.f90:167-379)
void mesh_operators(Mesh& m) {
  const int N = m.N;
  m.Xs.assign(N, 0.0);
  m.Xf.assign(N + 1, 0.0);
  setsandpoints(N, m.Xs.data(), m.Xf.data());
  m.Lmat.assign((N + 1) * N, 0.0);
  m.Mmat.assign((N + 1) * N, 0.0);
  compute_L_M(N, m.Xs.data(), m.Xf.data(), m.Lmat.data(), m.Mmat.data());
  m.iface2fp.assign(4 * N, 0);
  m.jface2fp.assign(4 * N, 0);
  for (int nfp = 1; nfp <= N; nfp++) {  // face2fpconnec initsetup.f90:343-379
    m.iface2fp[nfp - 1] = nfp;               m.jface2fp[nfp - 1] = 1;
    m.iface2fp[nfp - 1 + N] = N + 1;         m.jface2fp[nfp - 1 + N] = nfp;
    m.iface2fp[nfp - 1 + 2 * N] = N - nfp + 1; m.jface2fp[nfp - 1 + 2 * N] = N + 1;
    m.iface2fp[nfp - 1 + 3 * N] = 1;         m.jface2fp[nfp - 1 + 3 * N] = N - nfp + 1;
  }
}

// mapder + calcjacob (mapder.f90:1-76, calcjacob.f90:1-86) and xyCoor_atGps
// (mapder.f90:255-273) on the host
void mesh_geometry_host(Mesh& m) {
  const int N = m.N, NC = m.NCELL;
  auto ivcell = [&](int ic, int k) { return m.IVCELL[ic + (size_t)NC * k]; };
  const size_t ns = (size_t)N * N * NC, nf1 = (size_t)(N + 1) * N * NC;
  m.Jac.assign(ns, 0.0);
  m.S1.assign(4 * nf1, 0.0);
  m.S2.assign(4 * nf1, 0.0);
  m.XXsolu.assign(2 * ns, 0.0);
  auto metrics = [&](int ic, double psi, double eta, double& xpsi, double& ypsi, double& xeta, double& yeta) {
    const double dm[4][2] = {{eta - 1.0, psi - 1.0}, {1.0 - eta, -psi}, {eta, psi}, {-eta, 1.0 - psi}};
    xpsi = 0.0; xeta = 0.0; ypsi = 0.0; yeta = 0.0;
    for (int k = 0; k < 4; k++) {
      double xv = m.XV[ivcell(ic, k) - 1], yv = m.YV[ivcell(ic, k) - 1];
      xpsi = xpsi + dm[k][0] * xv;
      ypsi = ypsi + dm[k][0] * yv;
      xeta = xeta + dm[k][1] * xv;
      yeta = yeta + dm[k][1] * yv;
    }
  };
  for (int ic = 0; ic < NC; ic++) {
    double xpsi, ypsi, xeta, yeta;
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {
        metrics(ic, m.Xs[is], m.Xs[js], xpsi, ypsi, xeta, yeta);
        m.Jac[is + N * (js + (size_t)N * ic)] = xpsi * yeta - xeta * ypsi;
      }
    for (int jfp = 0; jfp < N; jfp++)
      for (int ifp = 0; ifp <= N; ifp++) {
        metrics(ic, m.Xf[ifp], m.Xs[jfp], xpsi, ypsi, xeta, yeta);
        size_t b = 4 * (ifp + (N + 1) * (jfp + (size_t)N * ic));
        m.S1[b] = yeta; m.S1[b + 2] = -xeta; m.S1[b + 1] = -ypsi; m.S1[b + 3] = xpsi;
      }
    for (int jfp = 0; jfp <= N; jfp++)
      for (int ifp = 0; ifp < N; ifp++) {
        metrics(ic, m.Xs[ifp], m.Xf[jfp], xpsi, ypsi, xeta, yeta);
        size_t b = 4 * (ifp + N * (jfp + (size_t)(N + 1) * ic));
        m.S2[b] = yeta; m.S2[b + 2] = -xeta; m.S2[b + 1] = -ypsi; m.S2[b + 3] = xpsi;
      }
    double xs[2][4];
    for (int k = 0; k < 4; k++) { xs[0][k] = m.XV[ivcell(ic, k) - 1]; xs[1][k] = m.YV[ivcell(ic, k) - 1]; }
    for (int js = 0; js < N; js++)
      for (int is = 0; is < N; is++) {  // xyCoor_atGps mapder.f90:255-273
        double xi = m.Xs[is], et = m.Xs[js];
        double f[4] = {(1.0 - xi) * (1.0 - et), (1.0 - et) * xi, xi * et, (1.0 - xi) * et};
        for (int d = 0; d < 2; d++) {
          double acc = 0.0;
          for (int nb = 0; nb < 4; nb++) acc = acc + xs[d][nb] * f[nb];
          m.XXsolu[d + 2 * (is + N * (js + (size_t)N * ic))] = acc;
        }
      }
  }
}

int mesh_load(const std::string& dir, Mesh& m, std::string& err) {
  std::vector<BndRecord> bnd;
  int rc = mesh_parse(dir, m, bnd, err);
  if (!rc) rc = mesh_maps_host(m, bnd, err);
  if (!rc) rc = mesh_periodic(m, err);
  if (rc) return rc;
  mesh_operators(m);
  mesh_geometry_host(m);
  m.params.NCELLGLOB = m.NCELL;
  return CHORUS_OK;
}

// Analytic initial data at one point (setinitialcond.f90:16-35 for Orszag-Tang; the
// rotor and the circularly polarised Alfven wave are additions).  When B is given it
// replaces the analytic field (second pass, setinitialcond.f90:46-78).
void initial_point(int problem, double gam, double x, double y, const double* B, double* q) {
  double rho, u, v, w, pr, Bx, By, Bz, Az;
  if (problem == 1) {
    const double r0 = 0.1, r1 = 0.115, u0 = 2.0;
    double dx = x - 0.5, dy = y - 0.5, r = std::sqrt(dx * dx + dy * dy);
    if (r < r0) { rho = 10.0; u = -u0 * dy / r0; v = u0 * dx / r0; }
    else if (r < r1) { double f = (r1 - r) / (r1 - r0); rho = 1.0 + 9.0 * f; u = -f * u0 * dy / r; v = f * u0 * dx / r; }
    else { rho = 1.0; u = 0.0; v = 0.0; }
    w = 0.0; pr = 1.0;
    double bx0 = 5.0 / std::sqrt(4.0 * kPi);
    Bx = bx0; By = 0.0; Bz = 0.0; Az = bx0 * y;
  } else if (problem == 2) {
    const double ca = std::sqrt(3.0) / 2.0, sa = 0.5, amp = 0.1, tp = 2.0 * kPi;
    double xp = x * ca + y * sa;
    double vperp = amp * std::sin(tp * xp), vz = amp * std::cos(tp * xp);
    rho = 1.0; pr = 0.1;
    u = -vperp * sa; v = vperp * ca; w = vz;
    double bpar = 1.0, bperp = amp * std::sin(tp * xp);
    Bx = bpar * ca - bperp * sa; By = bpar * sa + bperp * ca; Bz = amp * std::cos(tp * xp);
    Az = amp * std::cos(tp * xp) / tp;
  } else {
    rho = gam * gam;
    u = -std::sin(y);
    v = std::sin(x);
    w = 0.0;
    pr = gam;
    Bx = -std::sin(y);
    By = std::sin(x * 2);
    Bz = 0.0;
    Az = 0.5 * std::cos(x * 2) + std::cos(y);
  }
  if (B) { Bx = B[0]; By = B[1]; Bz = B[2]; }
  double nu = u * u + v * v + w * w, nb = Bx * Bx + By * By + Bz * Bz;
  q[0] = rho;
  q[1] = rho * u;
  q[2] = rho * v;
  q[3] = rho * w;
  q[4] = pr / (gam - 1) + 0.5 * rho * nu + 0.5 * nb;
  q[5] = Bx;
  q[6] = By;
  q[7] = Bz;
  q[8] = Az;
}

}  // namespace chorus
