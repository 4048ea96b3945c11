// host_internal.h -- host-side mesh object and setup helpers shared by the
// C ABI (host.cpp) and the input-file driver (driver.cpp).
#pragma once

#include <cstdint>
#include <limits>
#include <string>
#include <vector>

#include "shaw_gpu.h"

struct shaw_mesh_s {
  double bounds[4] = {0, 0, 0, 0};  // thL [deg], thR [deg], rCmb [m], rSurf [m]
  double dth = 0, drr = 0, dthInv = 0, drrInv = 0;
  uint64_t nvp = 0, nsp = 0, nth = 0, nr = 0;
  std::vector<int64_t> gvp, gsp;
  std::vector<int32_t> labels;
  std::vector<double> cvp, csp, cotvp, cotsp, coeffvp;
  std::vector<double> rhoInvVp, shearSp;
  double minVs = std::numeric_limits<double>::max();
  double maxVs = std::numeric_limits<double>::min();
  bool hasMaterial = false;
  // generated coordinates (before text round-trip), for byte-identical mesh files
  std::vector<double> thvp, rvp_km, thsp, rsp_km;
  std::vector<int> onsymvp, onsymsp;
  double raw_info[6] = {0, 0, 0, 0, 0, 0};  // thL, thR [deg], rCmb, rSurf [km], dth, dr as generated
};

namespace shaw {
int fail(int code, const std::string& msg);
namespace host {
int load_mesh(const std::string& dir, shaw_mesh_s& m);
int generate_mesh(uint64_t nth, uint64_t nr, double thLDeg, double thRDeg, double rCmb, double rSurf,
                  shaw_mesh_s& m);
int write_mesh(const shaw_mesh_s& m, const std::string& dir);
int set_material(shaw_mesh_s& m, int kind, const double* params, uint32_t np);
int map_source(const shaw_mesh_s& m, double depthKm, double angleDeg, uint64_t& gid);
int map_receiver(const shaw_mesh_s& m, double angleDeg, uint64_t& gid);
int check_cfl(const shaw_mesh_s& m, double dt, double& value);
int check_dispersion(const shaw_mesh_s& m, double maxfreq);
void operator_desc(const shaw_mesh_s& m, shaw_fom_operator_desc& d);
}  // namespace host
}  // namespace shaw
