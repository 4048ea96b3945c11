// rom_driver.cpp -- RomProblemRankOneForcing (src/kokkos/rom_problem_rank_one.hpp).
#include "driver.h"

namespace shaw {
namespace driver {

int run_rom(const Input&, const shaw_mesh_s&) {
  return fail(SHAW_ERR_UNSUPPORTED, "ROM runs from an input file are not wired yet");
}

}  // namespace driver
}  // namespace shaw
