// host.cpp -- host-side setup and drivers around the GPU hot path: what the
// reference's main.cc, MeshInfo, mesh readers, material models, grid mappers,
// checkers, input parser, problem classes and writers do, re-written for this
// library.  Everything here is O(mesh) setup or I/O; the time loop itself runs
// in fom.cu / rom.cu.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "shaw_gpu.h"
#include "host_internal.h"
#include "yaml_lite.h"

namespace shaw {
int fail(int code, const std::string& msg);
}


namespace shaw {
namespace host {

namespace {

bool essentiallyEqual(double a, double b) {
  const double eps = std::numeric_limits<double>::epsilon();
  return std::abs(a - b) <= ((std::abs(a) > std::abs(b) ? std::abs(b) : std::abs(a)) * eps);
}

// angular_helpers.hpp:52-64
double cotangent(double th) {
  const double c = std::cos(th), s = std::sin(th);
  if (essentiallyEqual(s, 0.0)) return 0.0;
  return c / s;
}

double degToRad(double v) { return v * (M_PI / 180.0); }

double polarDistance(double r1, double th1, double r2, double th2) {
  return std::sqrt((r1 * r1) + (r2 * r2) - 2.0 * r1 * r2 * std::cos(th2 - th1));
}

int mesh_error(const std::string& m) { return fail(SHAW_ERR_MESH, m); }

// mesh_info.hpp:116-214
int read_mesh_info(shaw_mesh_s& m, const std::string& dir) {
  std::ifstream f(dir + "/mesh_info.dat");
  if (!f) return mesh_error("File named: mesh_info.dat not found in " + dir);
  std::string line;
  try {
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
  } catch (const std::exception& e) {
    return mesh_error(std::string("malformed mesh_info.dat: ") + e.what());
  }
  if (m.nvp == 0 || m.nsp == 0) return mesh_error("mesh_info.dat lacks numPtsVp/numPtsSp");
  return SHAW_OK;
}

// read_graph_file.hpp:54-124
int read_graph(shaw_mesh_s& m, const std::string& dir, bool sp) {
  const std::string path = dir + (sp ? "/graph_sp.dat" : "/graph_vp.dat");
  std::ifstream f(path);
  if (!f) return mesh_error("graph file: " + path + " not found");
  const uint64_t n = sp ? m.nsp : m.nvp;
  const int nnb = sp ? 2 : 4;
  auto& g = sp ? m.gsp : m.gvp;
  auto& c = sp ? m.csp : m.cvp;
  auto& cot = sp ? m.cotsp : m.cotvp;
  g.assign(n * (nnb + 1), -1);
  c.assign(n * 2, 0.0);
  cot.assign(n, 0.0);
  if (sp) m.labels.assign(n, 0);
  std::string line, col;
  uint64_t rows = 0;
  try {
    while (std::getline(f, line)) {
      std::istringstream ss(line);
      if (!(ss >> col)) continue;
      const long long gid = std::stoll(col);
      if (gid < 0 || (uint64_t)gid >= n) return mesh_error("gid out of range in " + path);
      g[gid * (nnb + 1)] = gid;
      if (sp) { if (!(ss >> col)) throw std::runtime_error("short line"); m.labels[gid] = std::stoi(col); }
      if (!(ss >> col)) throw std::runtime_error("short line");
      const int onSym = std::stoi(col);
      if (!(ss >> col)) throw std::runtime_error("short line");
      c[gid * 2] = std::stod(col);
      if (!(ss >> col)) throw std::runtime_error("short line");
      c[gid * 2 + 1] = 1.0 / (std::stod(col) * 1000.0);
      cot[gid] = (onSym == 1) ? 0.0 : cotangent(c[gid * 2]);
      for (int i = 1; i <= nnb; ++i) {
        if (!(ss >> col)) throw std::runtime_error("short line");
        g[gid * (nnb + 1) + i] = std::stoll(col);
      }
      ++rows;
    }
  } catch (const std::exception& e) {
    return mesh_error("malformed " + path + ": " + e.what());
  }
  if (rows != n) return mesh_error(path + ": row count differs from mesh_info.dat");
  return SHAW_OK;
}

// read_vpcoeff_file.hpp:52-81
int read_coeff(shaw_mesh_s& m, const std::string& dir) {
  const std::string path = dir + "/coeff_vp.dat";
  std::ifstream f(path);
  if (!f) return mesh_error(" file: " + path + "not found");
  m.coeffvp.assign(m.nvp * 4, 0.0);
  std::string line, col;
  try {
    while (std::getline(f, line)) {
      std::istringstream ss(line);
      if (!(ss >> col)) continue;
      const long long gid = std::stoll(col);
      if (gid < 0 || (uint64_t)gid >= m.nvp) return mesh_error("gid out of range in " + path);
      for (int i = 0; i < 4; ++i) {
        if (!(ss >> col)) throw std::runtime_error("short line");
        m.coeffvp[gid * 4 + i] = std::stod(col);
      }
    }
  } catch (const std::exception& e) {
    return mesh_error("malformed " + path + ": " + e.what());
  }
  return SHAW_OK;
}

std::string fmt20(double v) {
  char buf[128];
  std::snprintf(buf, sizeof(buf), "%.20f", v);
  return buf;
}

}  // namespace

// ---- the full-mesh generator: meshing/helpers/full_mesh_utils.py:8-89,
//      build_graph_impl.py:7-172, create_single_mesh.py:24-60 ----------------
int generate_mesh(uint64_t nth, uint64_t nr, double thLDeg, double thRDeg, double rCmb, double rSurf,
                  shaw_mesh_s& m) {
  if (nth < 2 || nr < 2) return fail(SHAW_ERR_INVALID_ARG, "nth and nr must be >= 2");
  if (!(rCmb < rSurf) || !(rCmb > 0)) return fail(SHAW_ERR_INVALID_ARG, "need 0 < rCmb < rSurf");
  if (!(thLDeg < thRDeg)) return fail(SHAW_ERR_INVALID_ARG, "thLeft must be < thRight");
  const double thL = thLDeg * M_PI / 180.;
  const double thR = thRDeg * M_PI / 180.;
  const double L0 = thR - thL, L1 = rSurf - rCmb;
  const double dth = L0 / (double)(nth - 1), dr = L1 / (double)(nr - 1);
  m.nth = nth; m.nr = nr;
  m.nvp = nth * nr;
  m.nsp = (nr - 1) * nth + nr * (nth - 1);
  m.bounds[0] = thLDeg; m.bounds[1] = thRDeg;
  m.bounds[2] = rCmb * 1000.0; m.bounds[3] = rSurf * 1000.0;
  m.dth = dth; m.dthInv = 1.0 / dth;
  m.drr = dr * 1000.0; m.drrInv = 1.0 / m.drr;
  m.gvp.assign(m.nvp * 5, 0);
  m.gsp.assign(m.nsp * 3, 0);
  m.labels.assign(m.nsp, 0);
  m.cvp.assign(m.nvp * 2, 0.0); m.csp.assign(m.nsp * 2, 0.0);
  m.cotvp.assign(m.nvp, 0.0); m.cotsp.assign(m.nsp, 0.0);
  m.coeffvp.assign(m.nvp * 4, 0.0);
  m.thvp.assign(m.nvp, 0.0); m.rvp_km.assign(m.nvp, 0.0);
  m.thsp.assign(m.nsp, 0.0); m.rsp_km.assign(m.nsp, 0.0);
  m.raw_info[0] = thLDeg; m.raw_info[1] = thRDeg; m.raw_info[2] = rCmb; m.raw_info[3] = rSurf;
  m.raw_info[4] = dth; m.raw_info[5] = dr;
  m.onsymvp.assign(m.nvp, 0); m.onsymsp.assign(m.nsp, 0);
  const uint64_t row = 2 * nth - 1;
  auto srp = [&](uint64_t j, uint64_t i) { return (int64_t)(j * row + 2 * i); };
  auto stp = [&](uint64_t j, uint64_t i) { return (int64_t)((j + 1 < nr) ? j * row + 2 * i + 1 : j * row + i); };
  for (uint64_t j = 0; j < nr; ++j) {
    for (uint64_t i = 0; i < nth; ++i) {
      const uint64_t p = j * nth + i;
      const double vpTh = thL + (double)i * dth, vpR = rCmb + (double)j * dr;
      const int onSym = (i == 0 || i == nth - 1) ? 1 : 0;
      m.thvp[p] = vpTh; m.rvp_km[p] = vpR; m.onsymvp[p] = onSym;
      // vp neighbours and boundary factors (build_graph_impl.py:58-127)
      int64_t W, N, E, S;
      double c[4];
      if (i >= 1) { W = stp(j, i - 1); c[0] = 1.; } else { W = stp(j, i); c[0] = 0.; }
      if (i < nth - 1) { E = stp(j, i); c[2] = 1.; } else { E = stp(j, i - 1); c[2] = 0.; }
      if (j < nr - 1) { N = srp(j, i); c[1] = 1.; } else { N = srp(j - 1, i); c[1] = -1.; }
      if (j >= 1) { S = srp(j - 1, i); c[3] = 1.; } else { S = srp(j, i); c[3] = -1.; }
      if (onSym) c[0] = c[1] = c[2] = c[3] = 0.;
      int64_t* g = &m.gvp[p * 5];
      g[0] = (int64_t)p; g[1] = W; g[2] = N; g[3] = E; g[4] = S;
      for (int k = 0; k < 4; ++k) m.coeffvp[p * 4 + k] = c[k];
      if (j < nr - 1) {
        const int64_t q = srp(j, i);
        m.thsp[q] = vpTh; m.rsp_km[q] = vpR + dr * 0.5; m.onsymsp[q] = onSym; m.labels[q] = 1;
        int64_t* h = &m.gsp[q * 3];
        h[0] = q; h[1] = (int64_t)((j + 1) * nth + i); h[2] = (int64_t)p;
      }
      if (i < nth - 1) {
        const int64_t q = stp(j, i);
        m.thsp[q] = vpTh + dth * 0.5; m.rsp_km[q] = vpR; m.onsymsp[q] = 0; m.labels[q] = 2;
        int64_t* h = &m.gsp[q * 3];
        h[0] = q; h[1] = (int64_t)p; h[2] = (int64_t)(p + 1);
      }
    }
  }
  // The solver reads coordinates back through "%.20f" text: round-trip them the same way.
  for (uint64_t p = 0; p < m.nvp; ++p) {
    m.cvp[p * 2] = std::stod(fmt20(m.thvp[p]));
    m.cvp[p * 2 + 1] = 1.0 / (std::stod(fmt20(m.rvp_km[p])) * 1000.0);
    m.cotvp[p] = m.onsymvp[p] ? 0.0 : cotangent(m.cvp[p * 2]);
  }
  for (uint64_t q = 0; q < m.nsp; ++q) {
    m.csp[q * 2] = std::stod(fmt20(m.thsp[q]));
    m.csp[q * 2 + 1] = 1.0 / (std::stod(fmt20(m.rsp_km[q])) * 1000.0);
    m.cotsp[q] = m.onsymsp[q] ? 0.0 : cotangent(m.csp[q * 2]);
  }
  // mesh_info.dat is read back through "%.20f" too
  m.bounds[0] = std::stod(fmt20(thLDeg));
  m.bounds[1] = std::stod(fmt20(thRDeg));
  m.bounds[2] = std::stod(fmt20(rCmb)) * 1000.0;
  m.bounds[3] = std::stod(fmt20(rSurf)) * 1000.0;
  m.dth = std::stod(fmt20(dth)); m.dthInv = 1.0 / m.dth;
  m.drr = std::stod(fmt20(dr)) * 1000.0; m.drrInv = 1.0 / m.drr;
  return SHAW_OK;
}

// meshing/helpers/write_files.py:23-119
int write_mesh(const shaw_mesh_s& m, const std::string& dir) {
  if (m.thvp.empty()) return fail(SHAW_ERR_STATE, "only generated meshes can be written");
  const double* ri = m.raw_info;
  {
    std::ofstream f(dir + "/mesh_info.dat");
    if (!f) return fail(SHAW_ERR_IO, "cannot write " + dir + "/mesh_info.dat");
    f << "thL   " << fmt20(ri[0]) << "\n" << "thR   " << fmt20(ri[1]) << "\n"
      << "rCmb  " << fmt20(ri[2]) << "\n" << "rSurf " << fmt20(ri[3]) << "\n"
      << "dth   " << fmt20(ri[4]) << "\n" << "dr    " << fmt20(ri[5]) << "\n"
      << "numPtsVp " << m.nvp << "\n" << "numPtsSp " << m.nsp << "\n"
      << "nth " << m.nth << "\n" << "nr " << m.nr << "\n";
  }
  {
    std::ofstream f(dir + "/graph_vp.dat");
    if (!f) return fail(SHAW_ERR_IO, "cannot write graph_vp.dat");
    for (uint64_t p = 0; p < m.nvp; ++p) {
      const int64_t* g = &m.gvp[p * 5];
      f << p << " " << m.onsymvp[p] << " " << fmt20(m.thvp[p]) << " " << fmt20(m.rvp_km[p]) << " "
        << g[1] << " " << g[2] << " " << g[3] << " " << g[4] << " \n";
    }
  }
  {
    std::ofstream f(dir + "/coeff_vp.dat");
    if (!f) return fail(SHAW_ERR_IO, "cannot write coeff_vp.dat");
    char buf[64];
    for (uint64_t p = 0; p < m.nvp; ++p) {
      f << p << " ";
      for (int k = 0; k < 4; ++k) {
        std::snprintf(buf, sizeof(buf), "%.1f ", m.coeffvp[p * 4 + k]);
        f << buf;
      }
      f << "\n";
    }
  }
  {
    std::ofstream f(dir + "/graph_sp.dat");
    if (!f) return fail(SHAW_ERR_IO, "cannot write graph_sp.dat");
    for (uint64_t q = 0; q < m.nsp; ++q) {
      const int64_t* g = &m.gsp[q * 3];
      f << q << " " << m.labels[q] << " " << m.onsymsp[q] << " " << fmt20(m.thsp[q]) << " "
        << fmt20(m.rsp_km[q]) << " " << g[1] << " " << g[2] << " \n";
    }
  }
  return SHAW_OK;
}

int load_mesh(const std::string& dir, shaw_mesh_s& m) {
  int rc;
  if ((rc = read_mesh_info(m, dir))) return rc;
  if ((rc = read_graph(m, dir, false))) return rc;
  if ((rc = read_graph(m, dir, true))) return rc;
  if ((rc = read_coeff(m, dir))) return rc;
  return SHAW_OK;
}

// material_model_{unilayer,bilayer,prem}.hpp computeAt
struct Material {
  int kind = SHAW_MATERIAL_UNILAYER;
  double rho[2][3] = {{0}}, vs[2][3] = {{0}};
  double discKm = 0, surfM = 0;
  void at(double rM, double& rho_, double& vs_) const {
    if (kind == SHAW_MATERIAL_UNILAYER) {
      const double dM = surfM - rM;
      rho_ = rho[0][0] + rho[0][1] * dM + rho[0][2] * dM * dM;
      vs_ = vs[0][0] + vs[0][1] * dM + vs[0][2] * dM * dM;
      return;
    }
    if (kind == SHAW_MATERIAL_BILAYER) {
      const double d = surfM - rM;
      if (d < discKm * 1000.0) {
        rho_ = rho[0][0] + rho[0][1] * d + rho[0][2] * d * d;
        vs_ = vs[0][0] + vs[0][1] * d + vs[0][2] * d * d;
      } else {
        const double dM = d - (discKm * 1000.0);
        rho_ = rho[1][0] + rho[1][1] * dM + rho[1][2] * dM * dM;
        vs_ = vs[1][0] + vs[1][1] * dM + vs[1][2] * dM * dM;
      }
      return;
    }
    // PREM (Dziewonski & Anderson 1981), material_model_prem.hpp:85-176
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
      r = 12.5815 - 1.2638 * x - 3.6426 * xSq - 5.5281 * xCu;
      v = 0.0;
    } else {
      r = 13.0885 - 8.8381 * xSq;
      v = 3.6678 - 4.4475 * xSq;
    }
    v *= 1000.0;
    r *= 1000.0;
    rho_ = r;
    vs_ = v;
  }
};

// shwavepp.hpp:246-286
int set_material(shaw_mesh_s& m, int kind, const double* params, uint32_t np) {
  Material mat;
  mat.kind = kind;
  mat.surfM = m.bounds[3];
  if (kind == SHAW_MATERIAL_UNILAYER || kind == SHAW_MATERIAL_BILAYER) {
    if (!params || np < 6) return fail(SHAW_ERR_INVALID_ARG, "layer coefficients missing");
    for (int i = 0; i < 3; ++i) { mat.rho[0][i] = params[i]; mat.vs[0][i] = params[3 + i]; }
  }
  if (kind == SHAW_MATERIAL_BILAYER) {
    if (np < 13) return fail(SHAW_ERR_INVALID_ARG, "bilayer needs 13 parameters");
    mat.discKm = params[6];
    for (int i = 0; i < 3; ++i) { mat.rho[1][i] = params[7 + i]; mat.vs[1][i] = params[10 + i]; }
  }
  if (kind == SHAW_MATERIAL_PREM) {
    const double d1 = std::abs(m.bounds[3] / 1000. - 6371.), d2 = std::abs(m.bounds[2] / 1000. - 3480.);
    if (d1 > 1e-13 || d2 > 1e-13)
      return fail(SHAW_ERR_INVALID_ARG,
                  "To use the PREM model, your Earth domain must have r_cmb=3480 km and r_surface=6371 km.");
  }
  if (kind < SHAW_MATERIAL_UNILAYER || kind > SHAW_MATERIAL_PREM)
    return fail(SHAW_ERR_INVALID_ARG, "Cannot create material object, invalid material model kind");
  m.rhoInvVp.assign(m.nvp, 0.0);
  m.shearSp.assign(m.nsp, 0.0);
  m.minVs = std::numeric_limits<double>::max();
  m.maxVs = std::numeric_limits<double>::min();
  double rho, vs;
  for (uint64_t p = 0; p < m.nvp; ++p) {
    mat.at(1.0 / m.cvp[p * 2 + 1], rho, vs);
    m.rhoInvVp[p] = 1.0 / rho;
  }
  for (uint64_t q = 0; q < m.nsp; ++q) {
    mat.at(1.0 / m.csp[q * 2 + 1], rho, vs);
    m.shearSp[q] = rho * vs * vs;
    if (vs != 0.) m.minVs = std::min(m.minVs, vs);
    m.maxVs = std::max(m.maxVs, vs);
  }
  m.hasMaterial = true;
  return SHAW_OK;
}

// map_point_source_to_velocity_grid_point.hpp:61-133
int map_source(const shaw_mesh_s& m, double depthKm, double angleDeg, uint64_t& gid) {
  const double radiusKm = m.bounds[3] / 1000.0 - depthKm;
  if (angleDeg < m.bounds[0] || angleDeg > m.bounds[1])
    return fail(SHAW_ERR_INVALID_ARG, "Source angle is outside theta axis");
  if (radiusKm * 1000.0 < m.bounds[2] || radiusKm * 1000.0 > m.bounds[3])
    return fail(SHAW_ERR_INVALID_ARG, "Source angle is outside radius axis");
  double angRad = degToRad(angleDeg);
  if (essentiallyEqual(angleDeg, m.bounds[0])) angRad = degToRad(m.bounds[0]) + m.dth;
  if (essentiallyEqual(angleDeg, m.bounds[1])) angRad = degToRad(m.bounds[1]) - m.dth;
  double best = std::numeric_limits<double>::max();
  uint64_t res = 0;
  for (uint64_t p = 0; p < m.nvp; ++p) {
    const double th = m.cvp[p * 2], r = 1.0 / m.cvp[p * 2 + 1];
    const double d = polarDistance(r, th, radiusKm * 1000.0, angRad);
    if (d <= best) { best = d; res = p; }
  }
  gid = res;
  return SHAW_OK;
}

// map_nominal_location_to_velocity_grid_point.hpp:57-117 (receivers on the surface)
int map_receiver(const shaw_mesh_s& m, double angleDeg, uint64_t& gid) {
  const double rM = m.bounds[3];
  if (angleDeg < m.bounds[0] || angleDeg > m.bounds[1])
    return fail(SHAW_ERR_INVALID_ARG, "Target angle is outside theta axis");
  const double angRad = degToRad(angleDeg);
  double best = std::numeric_limits<double>::max();
  uint64_t res = 0;
  for (uint64_t p = 0; p < m.nvp; ++p) {
    const double th = m.cvp[p * 2], r = 1.0 / m.cvp[p * 2 + 1];
    const double d = polarDistance(r, th, rM, angRad);
    if (d <= best) { best = d; res = p; }
  }
  gid = res;
  return SHAW_OK;
}

// check_cfl.hpp:53-75
int check_cfl(const shaw_mesh_s& m, double dt, double& value) {
  const double maxArc = m.dth * m.bounds[3], minArc = m.dth * m.bounds[2];
  const double hRef = std::min(m.drr, std::min(maxArc, minArc));
  value = (dt * std::sqrt(2.0) * m.maxVs) / hRef;
  if (value <= 0.28) return SHAW_OK;
  return fail(SHAW_ERR_CFL, "CFL error (cfl = " + std::to_string(value) + ")");
}

// check_dispersion_criterion.hpp:53-84
int check_dispersion(const shaw_mesh_s& m, double maxfreq) {
  const double maxArc = m.dth * m.bounds[3];
  const double ratio = m.minVs / (10.0 * maxfreq);
  if (!(m.drr <= ratio)) return fail(SHAW_ERR_DISPERSION, "Numerical dispersion criterion violated by radial spacing");
  if (!(maxArc <= ratio)) return fail(SHAW_ERR_DISPERSION, "Numerical dispersion criterion violated along theta");
  return SHAW_OK;
}

void operator_desc(const shaw_mesh_s& m, shaw_fom_operator_desc& d) {
  d.nth = m.nth; d.nr = m.nr; d.nvp = m.nvp; d.nsp = m.nsp;
  d.dth_inv = m.dthInv; d.drr_inv = m.drrInv;
  d.graph_vp = m.gvp.data(); d.graph_sp = m.gsp.data(); d.labels_sp = m.labels.data();
  d.coords_vp = m.cvp.data(); d.coords_sp = m.csp.data();
  d.cot_vp = m.cotvp.data(); d.cot_sp = m.cotsp.data();
  d.coeff_vp = m.coeffvp.data();
  d.rho_inv_vp = m.rhoInvVp.data(); d.shear_mod_sp = m.shearSp.data();
}

}  // namespace host
}  // namespace shaw

using namespace shaw::host;

extern "C" {

int shaw_mesh_load(const char* dir, shaw_mesh_t* out) {
  if (!dir || !out) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  shaw_mesh_s* m = new shaw_mesh_s();
  const int rc = load_mesh(dir, *m);
  if (rc) { delete m; return rc; }
  *out = m;
  return SHAW_OK;
}

int shaw_mesh_generate(uint64_t nth, uint64_t nr, double thL, double thR, double rCmb, double rSurf,
                       shaw_mesh_t* out) {
  if (!out) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  shaw_mesh_s* m = new shaw_mesh_s();
  const int rc = generate_mesh(nth, nr, thL, thR, rCmb, rSurf, *m);
  if (rc) { delete m; return rc; }
  *out = m;
  return SHAW_OK;
}

int shaw_mesh_write(shaw_mesh_t m, const char* dir) {
  if (!m || !dir) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  return write_mesh(*m, dir);
}

int shaw_mesh_info(shaw_mesh_t m, double* out) {
  if (!m || !out) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  for (int i = 0; i < 4; ++i) out[i] = m->bounds[i];
  out[4] = m->dth; out[5] = m->drr; out[6] = m->dthInv; out[7] = m->drrInv;
  out[8] = (double)m->nvp; out[9] = (double)m->nsp; out[10] = (double)m->nth; out[11] = (double)m->nr;
  out[12] = m->dth * m->bounds[2]; out[13] = m->dth * m->bounds[3];
  return SHAW_OK;
}

int shaw_mesh_set_material(shaw_mesh_t m, int kind, const double* params, uint32_t np) {
  if (!m) return shaw::fail(SHAW_ERR_INVALID_ARG, "null mesh");
  return set_material(*m, kind, params, np);
}

int shaw_mesh_set_material_arrays(shaw_mesh_t m, const double* rhoInvVp, const double* shearSp) {
  if (!m || !rhoInvVp || !shearSp) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  m->rhoInvVp.assign(rhoInvVp, rhoInvVp + m->nvp);
  m->shearSp.assign(shearSp, shearSp + m->nsp);
  // vs = sqrt(G / rho) is unknown without rho at sp points: report the range as unset
  m->minVs = std::numeric_limits<double>::max();
  m->maxVs = std::numeric_limits<double>::min();
  m->hasMaterial = true;
  return SHAW_OK;
}

int shaw_mesh_min_max_vs(shaw_mesh_t m, double* mm) {
  if (!m || !mm) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  mm[0] = m->minVs; mm[1] = m->maxVs;
  return SHAW_OK;
}

int shaw_mesh_operator_desc(shaw_mesh_t m, shaw_fom_operator_desc* d) {
  if (!m || !d) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  if (!m->hasMaterial) return shaw::fail(SHAW_ERR_STATE, "set a material before building operators");
  operator_desc(*m, *d);
  return SHAW_OK;
}

int shaw_mesh_map_source(shaw_mesh_t m, double depthKm, double angleDeg, uint64_t* gid) {
  if (!m || !gid) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  return map_source(*m, depthKm, angleDeg, *gid);
}

int shaw_mesh_map_receiver(shaw_mesh_t m, double angleDeg, uint64_t* gid) {
  if (!m || !gid) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  return map_receiver(*m, angleDeg, *gid);
}

int shaw_mesh_check_cfl(shaw_mesh_t m, double dt, double* value) {
  if (!m) return shaw::fail(SHAW_ERR_INVALID_ARG, "null mesh");
  double v = 0;
  const int rc = check_cfl(*m, dt, v);
  if (value) *value = v;
  return rc;
}

int shaw_mesh_check_dispersion(shaw_mesh_t m, double maxfreq) {
  if (!m) return shaw::fail(SHAW_ERR_INVALID_ARG, "null mesh");
  return check_dispersion(*m, maxfreq);
}

void shaw_mesh_destroy(shaw_mesh_t m) { delete m; }

}  // extern "C"
