// shaw_oracle.cpp -- CPU oracle for the SHAW hot paths (TEST INFRASTRUCTURE ONLY).
//
// This file is the checker, never the product: only tests/, the smoke check and
// bench.py's CPU-baseline leg load it.  It restates, in plain C++ with the same
// arithmetic order, the reference computation for:
//   * mesh files          src/shared/mesh_helpers/{mesh_info,read_graph_file,read_vpcoeff_file}.hpp
//   * material models     src/shared/material_models/material_model_{unilayer,bilayer,prem}.hpp
//   * operator assembly   src/kokkos/shwavepp.hpp:246-466 (CRS Jvp / Jsp)
//   * grid mappers        src/shared/nominal_to_grid_mappers/*.hpp
//   * source signals      src/shared/various/signal.hpp:86-128
//   * FOM leapfrog        src/kokkos/fom_update_kernels.hpp:60-181, src/kokkos/fom_run.hpp:76-149
//   * observers           src/kokkos/state_observer.hpp:175-203, src/kokkos/seismogram.hpp:193-214
//   * ROM operators       src/kokkos/rom_compute_jacobians.hpp:83-102
//   * ROM leapfrog        src/kokkos/rom_run_rank_one.hpp:112-151,
//                         src/kokkos/torevise/run_rom_rank_two_forcing.hpp:149-188
//   * checkers            src/shared/checkers/check_cfl.hpp, check_dispersion_criterion.hpp
//   * full-mesh files     meshing/helpers/full_mesh_utils.py:8-89, build_graph_impl.py:7-172,
//                         write_files.py:10-119, create_single_mesh.py:24-60 (two variable groups)
// The sparse products follow Kokkos-Kernels 3.5.00's CRS row kernel: per row,
// sum = sum_k val[k]*x[ind[k]] in entry order, then y = y + alpha*sum.
// Parity: pinned against the reference's golden vectors (tests/golden).
// Built with -ffp-contract=off so the arithmetic is the same on x86_64 and aarch64.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

struct Mesh {
  std::string dir;
  double bounds[4] = {0, 0, 0, 0};  // thL deg, thR deg, rCmb m, rSurf m
  double dth = 0, drr = 0, dthInv = 0, drrInv = 0;
  uint64_t nvp = 0, nsp = 0, nth = 0, nr = 0;
  std::vector<int64_t> gvp;    // nvp x 5: gid, W, N, E, S
  std::vector<int64_t> gsp;    // nsp x 3: gid, a, b
  std::vector<int32_t> labels; // nsp
  std::vector<double> cvp;     // nvp x 2: theta, 1/r
  std::vector<double> csp;     // nsp x 2
  std::vector<double> cotvp, cotsp;
  std::vector<double> coeffvp; // nvp x 4
  // material
  std::vector<double> rhoInvVp, shearSp;
  double minVs = std::numeric_limits<double>::max();
  double maxVs = std::numeric_limits<double>::min();
  // CRS
  std::vector<uint64_t> ptrVp, indVp, ptrSp, indSp;
  std::vector<double> valVp, valSp;
  bool assembled = false;
};

bool essentiallyEqual(double a, double b) {
  const double eps = std::numeric_limits<double>::epsilon();
  return std::abs(a - b) <= ((std::abs(a) > std::abs(b) ? std::abs(b) : std::abs(a)) * eps);
}

double cotangent(double th) {
  const double c = std::cos(th), s = std::sin(th);
  if (essentiallyEqual(s, 0.0)) return 0.0;
  return c / s;
}

double degToRad(double v) { return v * (M_PI / 180.0); }

double polarDistance(double r1, double th1, double r2, double th2) {
  return std::sqrt((r1 * r1) + (r2 * r2) - 2.0 * r1 * r2 * std::cos(th2 - th1));
}

bool readMeshInfo(Mesh& m) {
  std::ifstream f(m.dir + "/mesh_info.dat");
  if (!f) { g_err = "mesh_info.dat not found in " + m.dir; return false; }
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string k, v;
    ss >> k;
    if (!(ss >> v)) continue;
    if (k == "thL") m.bounds[0] = std::stod(v);
    else if (k == "thR") m.bounds[1] = std::stod(v);
    else if (k == "rCmb") m.bounds[2] = std::stod(v) * 1000.0;
    else if (k == "rSurf") m.bounds[3] = std::stod(v) * 1000.0;
    else if (k == "dth") { m.dth = std::stod(v); m.dthInv = 1.0 / m.dth; }
    else if (k == "dr") { m.drr = std::stod(v) * 1000.0; m.drrInv = 1.0 / m.drr; }
    else if (k == "numPtsVp") m.nvp = std::stoull(v);
    else if (k == "numPtsSp") m.nsp = std::stoull(v);
    else if (k == "nth") m.nth = std::stoull(v);
    else if (k == "nr") m.nr = std::stoull(v);
  }
  return true;
}

// graph_{vp,sp}.dat: gid [label] onSym theta r_km neighbours...
bool readGraph(Mesh& m, bool sp) {
  const std::string path = m.dir + (sp ? "/graph_sp.dat" : "/graph_vp.dat");
  std::ifstream f(path);
  if (!f) { g_err = "graph file: " + path + " not found"; return false; }
  const uint64_t n = sp ? m.nsp : m.nvp;
  const int nnb = sp ? 2 : 4;
  auto& g = sp ? m.gsp : m.gvp;
  auto& c = sp ? m.csp : m.cvp;
  auto& cot = sp ? m.cotsp : m.cotvp;
  g.assign(n * (nnb + 1), 0);
  c.assign(n * 2, 0.0);
  cot.assign(n, 0.0);
  if (sp) m.labels.assign(n, 0);
  std::string line, col;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    if (!(ss >> col)) continue;
    const long gid = std::stol(col);
    if (gid < 0 || (uint64_t)gid >= n) { g_err = "gid out of range in " + path; return false; }
    g[gid * (nnb + 1)] = gid;
    if (sp) { ss >> col; m.labels[gid] = std::stoi(col); }
    ss >> col; const int onSym = std::stoi(col);
    ss >> col; c[gid * 2] = std::stod(col);
    ss >> col; c[gid * 2 + 1] = 1.0 / (std::stod(col) * 1000.0);
    cot[gid] = (onSym == 1) ? 0.0 : cotangent(c[gid * 2]);
    for (int i = 1; i <= nnb; ++i) { ss >> col; g[gid * (nnb + 1) + i] = std::stol(col); }
  }
  return true;
}

bool readCoeff(Mesh& m) {
  const std::string path = m.dir + "/coeff_vp.dat";
  std::ifstream f(path);
  if (!f) { g_err = " file: " + path + "not found"; return false; }
  m.coeffvp.assign(m.nvp * 4, 0.0);
  std::string line, col;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    if (!(ss >> col)) continue;
    const long gid = std::stol(col);
    if (gid < 0 || (uint64_t)gid >= m.nvp) { g_err = "gid out of range in coeff file"; return false; }
    for (int i = 0; i < 4; ++i) { ss >> col; m.coeffvp[gid * 4 + i] = std::stod(col); }
  }
  return true;
}

// material_model_*.hpp computeAt(radius [m], theta) -> rho [kg/m^3], vs [m/s]
struct Material {
  int kind = 0;  // 0 unilayer, 1 bilayer, 2 prem
  double rho[2][3] = {{0}}, vs[2][3] = {{0}};
  double discKm = 0;
  double surfM = 0;
  void at(double rM, double& rho_, double& vs_) const {
    if (kind == 0) {
      const double dM = surfM - rM;
      rho_ = rho[0][0] + rho[0][1] * dM + rho[0][2] * dM * dM;
      vs_ = vs[0][0] + vs[0][1] * dM + vs[0][2] * dM * dM;
    } else if (kind == 1) {
      const double d = surfM - rM;
      if (d < discKm * 1000.0) {
        rho_ = rho[0][0] + rho[0][1] * d + rho[0][2] * d * d;
        vs_ = vs[0][0] + vs[0][1] * d + vs[0][2] * d * d;
      } else {
        const double dM = d - (discKm * 1000.0);
        rho_ = rho[1][0] + rho[1][1] * dM + rho[1][2] * dM * dM;
        vs_ = vs[1][0] + vs[1][1] * dM + vs[1][2] * dM * dM;
      }
    } else {
      const double rKm = rM / 1000.0;
      const double x = rKm / 6371.0, xSq = x * x, xCu = x * x * x;
      double r = 0, v = 0;
      if (rKm >= 6356.0) { r = 2.6; v = 3.2; }
      else if (rKm >= 6346.6 && rKm < 6356.0) { r = 2.9; v = 3.9; }
      else if (rKm >= 6291.0 && rKm < 6346.6) { r = 2.691 + 0.6924 * x; v = 2.1519 + 2.3481 * x; }
      else if (rKm >= 6151.0 && rKm < 6291.0) { r = 2.691 + 0.6924 * x; v = 2.1519 + 2.3481 * x; }
      else if (rKm >= 5971.0 && rKm < 6151.0) { r = 7.1089 - 3.8045 * x; v = 8.9496 - 4.4597 * x; }
      else if (rKm >= 5771.0 && rKm < 5971.0) { r = 11.2494 - 8.0298 * x; v = 22.3512 - 18.5856 * x; }
      else if (rKm >= 5701.0 && rKm < 5771.0) { r = 5.3197 - 1.4836 * x; v = 9.9839 - 4.9324 * x; }
      else if (rKm >= 5600.0 && rKm < 5701.0) {
        r = 7.9565 - 6.4761 * x + 5.5283 * xSq - 3.0807 * xCu;
        v = 22.3459 - 17.2473 * x - 2.0834 * xSq + 0.9783 * xCu;
      } else if (rKm >= 3630.0 && rKm < 5600.0) {
        r = 7.9565 - 6.4761 * x + 5.5283 * xSq - 3.0807 * xCu;
        v = 11.1671 - 13.7818 * x + 17.4575 * xSq - 9.2777 * xCu;
      } else if (rKm >= 3480.0 && rKm < 3630.0) {
        r = 7.9565 - 6.4761 * x + 5.5283 * xSq - 3.0807 * xCu;
        v = 6.9254 + 1.4672 * x - 2.0834 * xSq + 0.9783 * xCu;
      } else if (rKm >= 1221.5 && rKm < 3480.0) {
        r = 12.5815 - 1.2638 * x - 3.6426 * xSq - 5.5281 * xCu; v = 0.0;
      } else { r = 13.0885 - 8.8381 * xSq; v = 3.6678 - 4.4475 * xSq; }
      v *= 1000.0;
      r *= 1000.0;
      rho_ = r; vs_ = v;
    }
  }
};

// shwavepp.hpp:319-400
void assembleVp(Mesh& m) {
  const uint64_t n = m.nvp;
  m.ptrVp.assign(n + 1, 0);
  m.indVp.clear(); m.valVp.clear();
  m.indVp.reserve(4 * n); m.valVp.reserve(4 * n);
  const double three = 3.0, oneHalf = 1.0 / 2.0;
  for (uint64_t p = 0; p < n; ++p) {
    const int64_t* g = &m.gvp[p * 5];
    const int64_t gid = g[0], w = g[1], no = g[2], e = g[3], s = g[4];
    const double rInv = m.cvp[gid * 2 + 1];
    const double cot = m.cotvp[gid];
    const double rhoInv = m.rhoInvVp[p];
    const double* c = &m.coeffvp[p * 4];
    const double cW = (-rInv * m.dthInv + rInv * cot) * c[0] * rhoInv;
    const double cN = (m.drrInv + three * oneHalf * rInv) * c[1] * rhoInv;
    const double cE = (rInv * m.dthInv + rInv * cot) * c[2] * rhoInv;
    const double cS = (-m.drrInv + three * oneHalf * rInv) * c[3] * rhoInv;
    uint64_t shift = 0;
    if (no == s) { m.indVp.push_back(no); m.valVp.push_back(cN + cS); shift += 1; }
    else { m.indVp.push_back(no); m.valVp.push_back(cN); m.indVp.push_back(s); m.valVp.push_back(cS); shift += 2; }
    if (w == e) { m.indVp.push_back(w); m.valVp.push_back(cW + cE); shift += 1; }
    else { m.indVp.push_back(w); m.valVp.push_back(cW); m.indVp.push_back(e); m.valVp.push_back(cE); shift += 2; }
    m.ptrVp[p + 1] = m.ptrVp[p] + shift;
  }
}

// shwavepp.hpp:402-466
void assembleSp(Mesh& m) {
  const uint64_t n = m.nsp;
  m.ptrSp.assign(n + 1, 0);
  for (uint64_t i = 0; i < n; ++i) m.ptrSp[i + 1] = m.ptrSp[i] + 2;
  m.indSp.assign(2 * n, 0); m.valSp.assign(2 * n, 0.0);
  const double oneHalf = 1.0 / 2.0;
  uint64_t k = 0;
  for (uint64_t p = 0; p < n; ++p) {
    const int64_t* g = &m.gsp[p * 3];
    const int64_t gid = g[0];
    const double rInv = m.csp[gid * 2 + 1];
    const int lab = m.labels[p];
    const double G = m.shearSp[p];
    if (lab == 1) {
      m.indSp[k] = g[1]; m.valSp[k++] = (m.drrInv - rInv * oneHalf) * G;
      m.indSp[k] = g[2]; m.valSp[k++] = (-m.drrInv - rInv * oneHalf) * G;
    }
    if (lab == 2) {
      m.indSp[k] = g[1]; m.valSp[k++] = (-m.dthInv - oneHalf * m.cotsp[gid]) * rInv * G;
      m.indSp[k] = g[2]; m.valSp[k++] = (m.dthInv - oneHalf * m.cotsp[gid]) * rInv * G;
    }
  }
}

// src/shared/various/signal.hpp:86-128; kind 0 ricker, 1 sinusoid, 2 gaussDer
double signal(int kind, double delay, double period, double t) {
  const double freq = 1.0 / period, freqSq = freq * freq;
  const double piSq = M_PI * M_PI;
  if (kind == 0) {
    const double tDiffSq = (t - delay) * (t - delay);
    const double expTerm = std::exp(-piSq * freqSq * tDiffSq);
    return (1.0 - 2.0 * piSq * tDiffSq * freqSq) * expTerm;
  } else if (kind == 1) {
    const double rn = 0.001;
    const double term2 = rn / (rn + 2.0);
    if (t < period) {
      const double term1 = std::sin(rn * M_PI * t / period);
      const double term3 = std::sin((rn + 2.0) * M_PI * t / period);
      return term1 - term2 * term3;
    }
    const double term1 = std::sin(rn * M_PI);
    const double term3 = std::sin((rn + 2.0) * M_PI);
    return term1 - term2 * term3;
  } else {
    const double tDiff = (t - delay);
    const double tDiffSq = tDiff * tDiff;
    const double expTerm = std::exp(-freqSq * tDiffSq);
    return -2.0 * tDiff * freqSq * expTerm;
  }
}

// CRS product on a row-major multivector: y[r,:] = y[r,:] + alpha * (A x)[r,:]
void crsUpdate(const std::vector<uint64_t>& ptr, const std::vector<uint64_t>& ind,
               const std::vector<double>& val, uint64_t nrows, int M, double alpha,
               const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < (int64_t)nrows; ++r) {
    for (int j = 0; j < M; ++j) {
      double sum = 0.0;
      for (uint64_t k = ptr[r]; k < ptr[r + 1]; ++k) sum += val[k] * x[ind[k] * M + j];
      sum *= alpha;
      y[(uint64_t)r * M + j] = 1.0 * y[(uint64_t)r * M + j] + sum;
    }
  }
}

int setThreads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  return omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

}  // namespace

extern "C" {

const char* orc_error(void) { return g_err.c_str(); }

void* orc_mesh_load(const char* dir) {
  Mesh* m = new Mesh();
  m->dir = dir;
  if (!readMeshInfo(*m) || !readGraph(*m, false) || !readGraph(*m, true) || !readCoeff(*m)) {
    delete m;
    return nullptr;
  }
  return m;
}

void orc_mesh_free(void* h) { delete static_cast<Mesh*>(h); }

// out: thL, thR, rCmb[m], rSurf[m], dth, drr, dthInv, drrInv, nvp, nsp, nth, nr, minArc, maxArc
void orc_mesh_info(const void* h, double* out) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  for (int i = 0; i < 4; ++i) out[i] = m.bounds[i];
  out[4] = m.dth; out[5] = m.drr; out[6] = m.dthInv; out[7] = m.drrInv;
  out[8] = (double)m.nvp; out[9] = (double)m.nsp; out[10] = (double)m.nth; out[11] = (double)m.nr;
  out[12] = m.dth * m.bounds[2]; out[13] = m.dth * m.bounds[3];
}

void orc_mesh_graph(const void* h, int64_t* gvp, int64_t* gsp, int32_t* labels,
                    double* cvp, double* csp, double* coeffvp) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  if (gvp) std::memcpy(gvp, m.gvp.data(), m.gvp.size() * sizeof(int64_t));
  if (gsp) std::memcpy(gsp, m.gsp.data(), m.gsp.size() * sizeof(int64_t));
  if (labels) std::memcpy(labels, m.labels.data(), m.labels.size() * sizeof(int32_t));
  if (cvp) std::memcpy(cvp, m.cvp.data(), m.cvp.size() * sizeof(double));
  if (csp) std::memcpy(csp, m.csp.data(), m.csp.size() * sizeof(double));
  if (coeffvp) std::memcpy(coeffvp, m.coeffvp.data(), m.coeffvp.size() * sizeof(double));
}

// kind 0 unilayer (params: rho[3], vs[3]); 1 bilayer (rho1[3], vs1[3], discKm, rho2[3], vs2[3]); 2 prem
int orc_set_material(void* h, int kind, const double* params) {
  Mesh& m = *static_cast<Mesh*>(h);
  Material mat;
  mat.kind = kind;
  mat.surfM = m.bounds[3];
  if (kind == 0 || kind == 1) {
    for (int i = 0; i < 3; ++i) { mat.rho[0][i] = params[i]; mat.vs[0][i] = params[3 + i]; }
  }
  if (kind == 1) {
    mat.discKm = params[6];
    for (int i = 0; i < 3; ++i) { mat.rho[1][i] = params[7 + i]; mat.vs[1][i] = params[10 + i]; }
  }
  if (kind == 2) {
    if (std::abs(m.bounds[3] / 1000.0 - 6371.0) > 1e-13 || std::abs(m.bounds[2] / 1000.0 - 3480.0) > 1e-13) {
      g_err = "PREM needs r_cmb=3480 km and r_surface=6371 km";
      return 1;
    }
  }
  m.rhoInvVp.assign(m.nvp, 0.0);
  m.shearSp.assign(m.nsp, 0.0);
  m.minVs = std::numeric_limits<double>::max();
  m.maxVs = std::numeric_limits<double>::min();
  double rho, vs;
  for (uint64_t p = 0; p < m.nvp; ++p) {
    const int64_t gid = m.gvp[p * 5];
    mat.at(1.0 / m.cvp[gid * 2 + 1], rho, vs);
    m.rhoInvVp[p] = 1.0 / rho;
  }
  for (uint64_t p = 0; p < m.nsp; ++p) {
    const int64_t gid = m.gsp[p * 3];
    mat.at(1.0 / m.csp[gid * 2 + 1], rho, vs);
    m.shearSp[p] = rho * vs * vs;
    if (vs != 0.) m.minVs = std::min(m.minVs, vs);
    m.maxVs = std::max(m.maxVs, vs);
  }
  assembleVp(m);
  assembleSp(m);
  m.assembled = true;
  return 0;
}

void orc_material_get(const void* h, double* rhoInvVp, double* shearSp, double* minmax) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  if (rhoInvVp) std::memcpy(rhoInvVp, m.rhoInvVp.data(), m.nvp * sizeof(double));
  if (shearSp) std::memcpy(shearSp, m.shearSp.data(), m.nsp * sizeof(double));
  if (minmax) { minmax[0] = m.minVs; minmax[1] = m.maxVs; }
}

// which 0 = Jvp, 1 = Jsp; sizes[0..2] = nrows, ncols, nnz
void orc_crs_sizes(const void* h, int which, uint64_t* sizes) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  sizes[0] = which == 0 ? m.nvp : m.nsp;
  sizes[1] = which == 0 ? m.nsp : m.nvp;
  sizes[2] = which == 0 ? m.indVp.size() : m.indSp.size();
}

void orc_crs_get(const void* h, int which, uint64_t* ptr, uint64_t* ind, double* val) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  const auto& P = which == 0 ? m.ptrVp : m.ptrSp;
  const auto& I = which == 0 ? m.indVp : m.indSp;
  const auto& V = which == 0 ? m.valVp : m.valSp;
  std::memcpy(ptr, P.data(), P.size() * sizeof(uint64_t));
  std::memcpy(ind, I.data(), I.size() * sizeof(uint64_t));
  std::memcpy(val, V.data(), V.size() * sizeof(double));
}

// map_point_source_to_velocity_grid_point.hpp:61-133 (last equal-distance point wins)
int orc_map_source(const void* h, double depthKm, double angleDeg, uint64_t* gid) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  const double radiusKm = m.bounds[3] / 1000.0 - depthKm;
  if (angleDeg < m.bounds[0] || angleDeg > m.bounds[1]) { g_err = "Source angle is outside theta axis"; return 1; }
  if (radiusKm * 1000.0 < m.bounds[2] || radiusKm * 1000.0 > m.bounds[3]) { g_err = "Source angle is outside radius axis"; return 1; }
  double angRad = degToRad(angleDeg);
  if (essentiallyEqual(angleDeg, m.bounds[0])) angRad = degToRad(m.bounds[0]) + m.dth;
  if (essentiallyEqual(angleDeg, m.bounds[1])) angRad = degToRad(m.bounds[1]) - m.dth;
  double best = std::numeric_limits<double>::max();
  uint64_t res = 0;
  for (uint64_t p = 0; p < m.nvp; ++p) {
    const int64_t g = m.gvp[p * 5];
    const double th = m.cvp[g * 2], r = 1.0 / m.cvp[g * 2 + 1];
    const double d = polarDistance(r, th, radiusKm * 1000.0, angRad);
    if (d <= best) { best = d; res = (uint64_t)g; }
  }
  *gid = res;
  return 0;
}

// map_nominal_location_to_velocity_grid_point.hpp:57-117 (receivers at r = rSurf)
int orc_map_receiver(const void* h, double angleDeg, uint64_t* gid) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  const double rM = m.bounds[3];
  if (angleDeg < m.bounds[0] || angleDeg > m.bounds[1]) { g_err = "Target angle is outside theta axis"; return 1; }
  const double angRad = degToRad(angleDeg);
  double best = std::numeric_limits<double>::max();
  uint64_t res = 0;
  for (uint64_t p = 0; p < m.nvp; ++p) {
    const int64_t g = m.gvp[p * 5];
    const double th = m.cvp[g * 2], r = 1.0 / m.cvp[g * 2 + 1];
    const double d = polarDistance(r, th, rM, angRad);
    if (d <= best) { best = d; res = (uint64_t)g; }
  }
  *gid = res;
  return 0;
}

double orc_signal(int kind, double delay, double period, double t) { return signal(kind, delay, period, t); }

// check_cfl.hpp:53-75 ; returns 0 ok, 1 violated; *value = the cfl number
int orc_check_cfl(const void* h, double dt, double* value) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  const double hRef = std::min(m.drr, std::min(m.dth * m.bounds[3], m.dth * m.bounds[2]));
  *value = (dt * std::sqrt(2.0) * m.maxVs) / hRef;
  return (*value <= 0.28) ? 0 : 1;
}

// check_dispersion_criterion.hpp:53-84 ; returns 0 ok, 1 radial violation, 2 angular violation
int orc_check_dispersion(const void* h, double maxfreq) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  const double ratio = m.minVs / (10.0 * maxfreq);
  if (!(m.drr <= ratio)) return 1;
  if (!(m.dth * m.bounds[3] <= ratio)) return 2;
  return 0;
}

// FOM leapfrog, fom_run.hpp:76-149.
//   rank 1: M == 1, forcing through KokkosBlas::mult  (x = 1*x + (dt*rhoInv)*f)
//   rank 2: forcing through AddForcingRank2            (x += (rhoInv*f)*dt)
// Signals: kind/period/delay per column; source vp gid per column.
// Outputs (any may be null), all LayoutLeft:
//   seis   [R x (nsteps/seisFreq) x M]
//   snapVp [nvp x (nsteps/freqVp) x M], snapSp [nsp x (nsteps/freqSp) x M]
//   finalVp [nvp x M], finalSp [nsp x M]
int orc_fom_run(const void* h, int rank, int M, uint64_t nsteps, double dt,
                const uint64_t* srcGid, const int32_t* kind, const double* period, const double* delay,
                int R, const uint64_t* rcvGid, uint64_t seisFreq, double* seis,
                uint64_t freqVp, uint64_t freqSp, double* snapVp, double* snapSp,
                double* finalVp, double* finalSp, int nthreads) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  if (!m.assembled) { g_err = "material not set"; return 1; }
  if (rank == 1 && M != 1) { g_err = "rank-1 needs M == 1"; return 1; }
  setThreads(nthreads);
  std::vector<double> xv(m.nvp * (uint64_t)M, 0.0), xs(m.nsp * (uint64_t)M, 0.0);
  std::vector<double> ftab;
  if (rank == 1) {  // forcing_rank_one.hpp:169-178: full signal table precomputed
    ftab.assign(nsteps, 0.0);
    double time = 0.0;
    for (uint64_t s = 1; s <= nsteps; ++s) { ftab[s - 1] = signal(kind[0], delay[0], period[0], time); time = s * dt; }
  }
  const uint64_t Tseis = seisFreq ? nsteps / seisFreq : 0;
  const uint64_t Tvp = freqVp ? nsteps / freqVp : 0, Tsp = freqSp ? nsteps / freqSp : 0;
  uint64_t cSeis = 0, cVp = 0, cSp = 0;
  std::vector<double> f(M, 0.0);
  double timeVp = 0.0;
  for (uint64_t step = 1; step <= nsteps; ++step) {
    // forcing evaluate
    if (rank == 2) for (int j = 0; j < M; ++j) f[j] = signal(kind[j], delay[j], period[j], timeVp);
    // velocity
    crsUpdate(m.ptrVp, m.indVp, m.valVp, m.nvp, M, dt, xs.data(), xv.data());
    if (rank == 1) {
      // KokkosBlas::mult over the whole vector: only the source entry is non-zero in f
      const uint64_t g = srcGid[0];
      xv[g] = 1.0 * xv[g] + dt * m.rhoInvVp[g] * ftab[step - 1];
    } else {
      for (int j = 0; j < M; ++j) {
        const uint64_t g = srcGid[j];
        xv[g * M + j] += m.rhoInvVp[g] * f[j] * dt;
      }
    }
    if (snapVp && freqVp && step % freqVp == 0) {
      for (int j = 0; j < M; ++j)
        for (uint64_t i = 0; i < m.nvp; ++i) snapVp[i + m.nvp * (cVp + Tvp * j)] = xv[i * M + j];
      ++cVp;
    }
    if (seis && seisFreq && step % seisFreq == 0) {
      for (int r = 0; r < R; ++r)
        for (int j = 0; j < M; ++j) seis[r + (uint64_t)R * (cSeis + Tseis * j)] = xv[rcvGid[r] * M + j];
      ++cSeis;
    }
    timeVp = step * dt;
    // stress
    crsUpdate(m.ptrSp, m.indSp, m.valSp, m.nsp, M, dt, xv.data(), xs.data());
    if (snapSp && freqSp && step % freqSp == 0) {
      for (int j = 0; j < M; ++j)
        for (uint64_t i = 0; i < m.nsp; ++i) snapSp[i + m.nsp * (cSp + Tsp * j)] = xs[i * M + j];
      ++cSp;
    }
  }
  // LayoutLeft copies of the final states (rows split over the threads)
  if (finalVp) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)m.nvp; ++i)
      for (int j = 0; j < M; ++j) finalVp[i + m.nvp * j] = xv[i * M + j];
  }
  if (finalSp) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)m.nsp; ++i)
      for (int j = 0; j < M; ++j) finalSp[i + m.nsp * j] = xs[i * M + j];
  }
  return 0;
}

// Advance a row-major state (nvp x M, nsp x M) by nsteps with no forcing and no
// observers: the bounded CPU-baseline workload of the FOM.  step0 is unused by the
// math (signals are off) and kept for symmetry with the GPU call.
int orc_fom_advance(const void* h, int M, uint64_t nsteps, double dt, double* xv, double* xs, int nthreads) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  if (!m.assembled) { g_err = "material not set"; return 1; }
  setThreads(nthreads);
  for (uint64_t s = 0; s < nsteps; ++s) {
    crsUpdate(m.ptrVp, m.indVp, m.valVp, m.nvp, M, dt, xs, xv);
    crsUpdate(m.ptrSp, m.indSp, m.valSp, m.nsp, M, dt, xv, xs);
  }
  return 0;
}

// The rank-2 leapfrog of orc_fom_run continued from a row-major state after step0
// completed steps: forcing of every column (AddForcingRank2 order), and the receiver
// gather of every step into seisRow (R x M, overwritten each step; may be null): the
// whole per-step work of the FOM benchmark, for the CPU timing of the reference path.
int orc_fom_advance_forced(const void* h, int M, uint64_t step0, uint64_t nsteps, double dt, const uint64_t* srcGid,
                           const int32_t* kind, const double* period, const double* delay, int R,
                           const uint64_t* rcvGid, double* seisRow, double* xv, double* xs, int nthreads) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  if (!m.assembled) { g_err = "material not set"; return 1; }
  setThreads(nthreads);
  std::vector<double> f(M, 0.0);
  for (uint64_t s = 0; s < nsteps; ++s) {
    const double t = (double)(step0 + s) * dt;
    for (int j = 0; j < M; ++j) f[j] = signal(kind[j], delay[j], period[j], t);
    crsUpdate(m.ptrVp, m.indVp, m.valVp, m.nvp, M, dt, xs, xv);
    for (int j = 0; j < M; ++j) {
      const uint64_t g = srcGid[j];
      xv[g * M + j] += m.rhoInvVp[g] * f[j] * dt;
    }
    if (seisRow)
      for (int r = 0; r < R; ++r)
        for (int j = 0; j < M; ++j) seisRow[r + (uint64_t)R * j] = xv[rcvGid[r] * M + j];
    crsUpdate(m.ptrSp, m.indSp, m.valSp, m.nsp, M, dt, xv, xs);
  }
  return 0;
}

int orc_num_threads(int nthreads) { return setThreads(nthreads); }

// rom_compute_jacobians.hpp:83-102. phi are LayoutLeft (col-major) n x k.
// romJvp (kv x ks) = PhiVp^T (Jvp PhiSp), romJsp (ks x kv) = PhiSp^T (Jsp PhiVp); outputs row-major.
int orc_rom_operators(const void* h, const double* phiVp, uint64_t kv, const double* phiSp, uint64_t ks,
                      double* romJvp, double* romJsp, int nthreads) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  if (!m.assembled) { g_err = "material not set"; return 1; }
  setThreads(nthreads);
  {
    std::vector<double> tmp(m.nvp * ks, 0.0);  // col-major nvp x ks
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < (int64_t)ks; ++c)
      for (uint64_t r = 0; r < m.nvp; ++r) {
        double sum = 0.0;
        for (uint64_t k = m.ptrVp[r]; k < m.ptrVp[r + 1]; ++k) sum += m.valVp[k] * phiSp[m.indVp[k] + m.nsp * c];
        tmp[r + m.nvp * c] = sum;
      }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)kv; ++i)
      for (uint64_t j = 0; j < ks; ++j) {
        double sum = 0.0;
        for (uint64_t r = 0; r < m.nvp; ++r) sum += phiVp[r + m.nvp * i] * tmp[r + m.nvp * j];
        romJvp[i * ks + j] = sum;
      }
  }
  {
    std::vector<double> tmp(m.nsp * kv, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < (int64_t)kv; ++c)
      for (uint64_t r = 0; r < m.nsp; ++r) {
        double sum = 0.0;
        for (uint64_t k = m.ptrSp[r]; k < m.ptrSp[r + 1]; ++k) sum += m.valSp[k] * phiVp[m.indSp[k] + m.nvp * c];
        tmp[r + m.nsp * c] = sum;
      }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)ks; ++i)
      for (uint64_t j = 0; j < kv; ++j) {
        double sum = 0.0;
        for (uint64_t r = 0; r < m.nsp; ++r) sum += phiSp[r + m.nsp * i] * tmp[r + m.nsp * j];
        romJsp[i * kv + j] = sum;
      }
  }
  return 0;
}

// rom_problem_rank_one.hpp:137-147: b = rhoInv[src] * PhiVp[src, :]
void orc_rom_forcing_vector(const void* h, const double* phiVp, uint64_t kv, uint64_t srcGid, double* b) {
  const Mesh& m = *static_cast<const Mesh*>(h);
  const double rhoInv = m.rhoInvVp[srcGid];
  for (uint64_t i = 0; i < kv; ++i) b[i] = rhoInv * phiVp[srcGid + m.nvp * i];
}

// ROM leapfrog (rom_run_rank_one.hpp:112-151 and the rank-2 form of
// torevise/run_rom_rank_two_forcing.hpp:149-188):
//   xv += dt * Av xs ; xv[:,j] += (f_j(t_{n-1}) * dt) * b[:,j] ; xs += dt * As xv
// romJvp kv x ks row-major, romJsp ks x kv row-major, b kv x M col-major.
// Outputs LayoutLeft: snapVp [kv x T x M], snapSp [ks x T x M], finalVp [kv x M], finalSp [ks x M].
int orc_rom_run(uint64_t kv, uint64_t ks, const double* Av, const double* As, int M, const double* b,
                uint64_t nsteps, double dt, const int32_t* kind, const double* period, const double* delay,
                uint64_t freqVp, uint64_t freqSp, double* snapVp, double* snapSp,
                double* finalVp, double* finalSp, int nthreads) {
  setThreads(nthreads);
  std::vector<double> xv(kv * (uint64_t)M, 0.0), xs(ks * (uint64_t)M, 0.0);  // col-major
  const uint64_t Tvp = freqVp ? nsteps / freqVp : 0, Tsp = freqSp ? nsteps / freqSp : 0;
  uint64_t cVp = 0, cSp = 0;
  std::vector<double> fdt(M);
  double time = 0.0;
  for (uint64_t step = 1; step <= nsteps; ++step) {
    for (int j = 0; j < M; ++j) fdt[j] = signal(kind[j], delay[j], period[j], time) * dt;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < M; ++j) {
      for (uint64_t i = 0; i < kv; ++i) {
        double sum = 0.0;
        for (uint64_t k = 0; k < ks; ++k) sum += Av[i * ks + k] * xs[k + ks * j];
        xv[i + kv * j] = 1.0 * xv[i + kv * j] + dt * sum;
      }
      for (uint64_t i = 0; i < kv; ++i) xv[i + kv * j] = xv[i + kv * j] + fdt[j] * b[i + kv * j];
    }
    if (snapVp && freqVp && step % freqVp == 0) {
      for (int j = 0; j < M; ++j) for (uint64_t i = 0; i < kv; ++i) snapVp[i + kv * (cVp + Tvp * j)] = xv[i + kv * j];
      ++cVp;
    }
    time = step * dt;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < M; ++j)
      for (uint64_t i = 0; i < ks; ++i) {
        double sum = 0.0;
        for (uint64_t k = 0; k < kv; ++k) sum += As[i * kv + k] * xv[k + kv * j];
        xs[i + ks * j] = 1.0 * xs[i + ks * j] + dt * sum;
      }
    if (snapSp && freqSp && step % freqSp == 0) {
      for (int j = 0; j < M; ++j) for (uint64_t i = 0; i < ks; ++i) snapSp[i + ks * (cSp + Tsp * j)] = xs[i + ks * j];
      ++cSp;
    }
  }
  if (finalVp) std::memcpy(finalVp, xv.data(), xv.size() * sizeof(double));
  if (finalSp) std::memcpy(finalSp, xs.data(), xs.size() * sizeof(double));
  return 0;
}

// main_reconstruct_seismo.cc:157-185: S(r, t) = sum_i PhiVp[gid_r, i] * X(i, t)
void orc_rom_seismogram(const double* phiVp, uint64_t nvp, uint64_t kv, int R, const uint64_t* rcvGid,
                        const double* X, uint64_t T, double* S) {
  for (uint64_t t = 0; t < T; ++t)
    for (int r = 0; r < R; ++r) {
      double sum = 0.0;
      for (uint64_t i = 0; i < kv; ++i) sum += phiVp[rcvGid[r] + nvp * i] * X[i + kv * t];
      S[r + (uint64_t)R * t] = sum;
    }
}

// ---- the reference mesher's full mesh with two variable groups, written as files ----
// Cells are visited j-major (r), i-minor (theta); each cell holds its vp point, an srp
// point above it (j < nr-1) and an stp point to its right (i < nth-1), numbered in that
// order (meshing/helpers/full_mesh_utils.py:8-89, unit_cell.py:58-66).  Graphs and the
// boundary factors of the vp stencil follow build_graph_impl.py:58-127; the files use the
// mesher's formats (write_files.py: "%.20f" floats, "%.1f" factors, a trailing space).
int orc_write_full_mesh(uint64_t nth, uint64_t nr, double thLDeg, double thRDeg, double rCmb, double rSurf,
                        const char* dir) {
  if (nth < 2 || nr < 2 || !dir) { g_err = "bad mesh arguments"; return 1; }
  const double pi = 3.14159265358979311600;  // numpy.pi
  const double thL = thLDeg * pi / 180., thR = thRDeg * pi / 180.;
  const double dth = (thR - thL) / (double)(nth - 1), dr = (rSurf - rCmb) / (double)(nr - 1);
  const uint64_t nvp = nth * nr, nsp = (nr - 1) * nth + nr * (nth - 1), row = 2 * nth - 1;
  auto srp = [&](uint64_t j, uint64_t i) { return j * row + 2 * i; };
  auto stp = [&](uint64_t j, uint64_t i) { return (j + 1 < nr) ? j * row + 2 * i + 1 : j * row + i; };
  const std::string d(dir);
  FILE* fi = std::fopen((d + "/mesh_info.dat").c_str(), "w");
  FILE* fv = std::fopen((d + "/graph_vp.dat").c_str(), "w");
  FILE* fc = std::fopen((d + "/coeff_vp.dat").c_str(), "w");
  FILE* fs = std::fopen((d + "/graph_sp.dat").c_str(), "w");
  if (!fi || !fv || !fc || !fs) {
    for (FILE* f : {fi, fv, fc, fs}) if (f) std::fclose(f);
    g_err = "cannot write mesh files in " + d;
    return 1;
  }
  std::fprintf(fi, "thL   %.20f\nthR   %.20f\nrCmb  %.20f\nrSurf %.20f\ndth   %.20f\ndr    %.20f\n", thLDeg, thRDeg,
               rCmb, rSurf, dth, dr);
  std::fprintf(fi, "numPtsVp %llu\nnumPtsSp %llu\nnth %llu\nnr %llu\n", (unsigned long long)nvp,
               (unsigned long long)nsp, (unsigned long long)nth, (unsigned long long)nr);
  // sp points are written in gid order, which is the cell order: srp then stp per cell
  for (uint64_t j = 0; j < nr; ++j) {
    for (uint64_t i = 0; i < nth; ++i) {
      const uint64_t p = j * nth + i;
      const double th = thL + (double)i * dth, r = rCmb + (double)j * dr;
      const int onSym = (i == 0 || i == nth - 1) ? 1 : 0;
      const uint64_t W = i >= 1 ? stp(j, i - 1) : stp(j, i), E = i + 1 < nth ? stp(j, i) : stp(j, i - 1);
      const uint64_t N = j + 1 < nr ? srp(j, i) : srp(j - 1, i), S = j >= 1 ? srp(j - 1, i) : srp(j, i);
      double c[4] = {i >= 1 ? 1. : 0., j + 1 < nr ? 1. : -1., i + 1 < nth ? 1. : 0., j >= 1 ? 1. : -1.};
      if (onSym) c[0] = c[1] = c[2] = c[3] = 0.;
      std::fprintf(fv, "%llu %d %.20f %.20f %llu %llu %llu %llu \n", (unsigned long long)p, onSym, th, r,
                   (unsigned long long)W, (unsigned long long)N, (unsigned long long)E, (unsigned long long)S);
      std::fprintf(fc, "%llu %.1f %.1f %.1f %.1f \n", (unsigned long long)p, c[0], c[1], c[2], c[3]);
      if (j + 1 < nr)
        std::fprintf(fs, "%llu 1 %d %.20f %.20f %llu %llu \n", (unsigned long long)srp(j, i), onSym, th, r + dr * 0.5,
                     (unsigned long long)((j + 1) * nth + i), (unsigned long long)p);
      if (i + 1 < nth)
        std::fprintf(fs, "%llu 2 0 %.20f %.20f %llu %llu \n", (unsigned long long)stp(j, i), th + dth * 0.5, r,
                     (unsigned long long)p, (unsigned long long)(p + 1));
    }
  }
  int bad = 0;
  for (FILE* f : {fi, fv, fc, fs}) bad |= std::fclose(f) != 0;
  if (bad) { g_err = "error writing mesh files in " + d; return 1; }
  return 0;
}

}  // extern "C"
