// driver.h -- parsed input of a SHAW run and the driver entry points.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "host_internal.h"

namespace shaw {
namespace driver {

constexpr int kMaterialCustom = 99;

// What InputParser<...> holds after parsing (src/shared/parser/*.hpp), with the
// reference's defaults.
struct Input {
  // general
  std::string meshDir = "empty";
  bool checkDispersion = true, checkCfl = true, exploitForcingSparsity = true;
  double dt = 0, finalTime = 0;
  uint64_t nsteps = 0;
  // io
  bool snapEnabled = false, snapBinary = true;
  uint64_t snapFreqVp = 0, snapFreqSp = 0;
  std::string snapFileVp = "snaps_vp", snapFileSp = "snaps_sp";
  bool seisEnabled = false, seisBinary = true;
  uint64_t seisFreq = 0;
  std::string seisFile = "seismogram";
  std::vector<double> receivers = {5, 30, 60, 90, 120, 150, 175};
  // material
  int matKind = 0;
  std::vector<double> matParams;
  // source
  int signalKind = -1;
  std::vector<double> depths, angles, periods, delays;
  bool rank2 = false, multiForcing = false;
  int forcingSize = 1;
  // rom
  bool romEnabled = false, romDummyBasis = false, disableRomJacs = false;
  uint64_t romModesVp = 0, romModesSp = 0;
  std::string romFileVp = "empty", romFileSp = "empty";
  bool romBinaryVp = true, romBinarySp = true;
};

int parse_input(const std::string& path, Input& in);
int run_input_file(const std::string& path);
int run_fom(const Input& in, const shaw_mesh_s& mesh);
int run_rom(const Input& in, const shaw_mesh_s& mesh);

int write_matrix(const std::string& file, const double* A, uint64_t m, uint64_t n, bool binary, bool writeSize);
int write_3d(const std::string& file, const double* A, uint64_t s0, uint64_t s1, uint64_t s2, bool binary,
             bool writeSize);
int write_observed(const std::string& file, const double* A, uint64_t s0, uint64_t s1, uint64_t s2, bool binary,
                   bool writeSize);

}  // namespace driver
}  // namespace shaw
