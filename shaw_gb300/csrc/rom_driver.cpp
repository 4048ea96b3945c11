// rom_driver.cpp -- RomProblemRankOneForcing (src/kokkos/rom_problem_rank_one.hpp:90-191)
// on top of the C ABI: FOM operators on the GPU, basis loading (rom_load_basis.hpp,
// src/shared/io/read_basis.hpp), GPU projection of the reduced operators, the
// forcing vector phiVpRhoInv, the checkers, the ROM leapfrog and the reduced
// snapshots written like the reference's StateObserver.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "driver.h"

namespace shaw {
namespace driver {

namespace {

// fillMatrixFromBinary / fillMatrixFromAscii with extents (src/shared/io/matrix_read.hpp:57-157):
// returns a column-major rows x cols matrix.
int read_matrix(const std::string& file, bool binary, std::vector<double>& out, uint64_t& rows, uint64_t& cols) {
  if (binary) {
    std::ifstream f(file, std::ios::in | std::ios::binary);
    if (!f) return fail(SHAW_ERR_IO, "cannot open basis file " + file);
    size_t r = 0, c = 0;
    f.read((char*)&r, sizeof(size_t));
    f.read((char*)&c, sizeof(size_t));
    if (!f) return fail(SHAW_ERR_IO, "ERROR READING binary file " + file);
    rows = r; cols = c;
    out.assign(r * c, 0.0);
    f.read((char*)out.data(), (std::streamsize)(r * c * sizeof(double)));
    if (!f) return fail(SHAW_ERR_IO, "ERROR READING binary file " + file);
    return SHAW_OK;
  }
  std::ifstream f(file);
  if (!f) return fail(SHAW_ERR_IO, "cannot open basis file " + file);
  std::string line, col;
  if (!std::getline(f, line)) return fail(SHAW_ERR_IO, "empty basis file " + file);
  {
    std::istringstream in(line);
    std::string a, b;
    in >> a >> b;
    try {
      rows = std::stoull(a);
      cols = std::stoull(b);
    } catch (const std::exception&) {
      return fail(SHAW_ERR_IO, "bad extents in " + file);
    }
  }
  out.assign(rows * cols, 0.0);
  uint64_t i = 0;
  while (std::getline(f, line) && i < rows) {
    std::istringstream in(line);
    for (uint64_t j = 0; j < cols; ++j) {
      if (!(in >> col)) return fail(SHAW_ERR_IO, "short row in " + file);
      out[i + rows * j] = std::atof(col.c_str());
    }
    ++i;
  }
  if (i != rows) return fail(SHAW_ERR_IO, "row count differs from extents in " + file);
  return SHAW_OK;
}

// readBasis (read_basis.hpp:54-96): keep the first numModes columns.
int load_basis(const std::string& file, bool binary, uint64_t nrows, uint64_t k, std::vector<double>& phi) {
  std::vector<double> all;
  uint64_t r = 0, c = 0;
  int rc = read_matrix(file, binary, all, r, c);
  if (rc) return rc;
  if (r != nrows) return fail(SHAW_ERR_INVALID_ARG, "basis rows differ from the mesh's point count: " + file);
  if (c < k) return fail(SHAW_ERR_INVALID_ARG, "basis has fewer columns than numModes: " + file);
  phi.assign(all.begin(), all.begin() + (size_t)(nrows * k));
  return SHAW_OK;
}

struct FomGuard {
  shaw_fom_t h = nullptr;
  ~FomGuard() { shaw_fom_destroy(h); }
};
struct RomGuard {
  shaw_rom_t h = nullptr;
  ~RomGuard() { shaw_rom_destroy(h); }
};

}  // namespace

int run_rom(const Input& in, const shaw_mesh_s& mesh) {
  int rc;
  const uint64_t kv = in.romModesVp, ks = in.romModesSp;
  // fillBasis (rom_load_basis.hpp:62-101)
  std::vector<double> phiVp, phiSp;
  if (in.romDummyBasis) {
    // random dummy basis for scaling runs: uniform in [0, 1e-3), seed 13718
    std::mt19937_64 gen(13718);
    std::uniform_real_distribution<double> u(0.0, 0.001);
    phiVp.resize(mesh.nvp * kv);
    phiSp.resize(mesh.nsp * ks);
    for (auto& x : phiVp) x = u(gen);
    for (auto& x : phiSp) x = u(gen);
  } else {
    if ((rc = load_basis(in.romFileVp, in.romBinaryVp, mesh.nvp, kv, phiVp))) return rc;
    if ((rc = load_basis(in.romFileSp, in.romBinarySp, mesh.nsp, ks, phiSp))) return rc;
  }
  // reduced operators
  std::vector<double> Av(kv * ks, 0.0), As(ks * kv, 0.0);
  if (!in.disableRomJacs) {
    shaw_fom_operator_desc d;
    host::operator_desc(mesh, d);
    FomGuard f;
    if ((rc = shaw_fom_create(&d, 1, 1, SHAW_FP64, &f.h))) return rc;
    const auto t0 = std::chrono::steady_clock::now();
    if ((rc = shaw_rom_project(f.h, phiVp.data(), kv, phiSp.data(), ks, Av.data(), As.data()))) return rc;
    // the log line of computeRomOperatorsUsingFomJacsWithMatProp (rom_compute_jacobians.hpp:107-108)
    std::printf("romJac time: %.10f\n",
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
  }
  // RankOneForcing source mapping and phiVpRhoInv (rom_problem_rank_one.hpp:133-147)
  uint64_t src = 0;
  if ((rc = host::map_source(mesh, in.depths[0], in.angles[0], src))) return rc;
  std::vector<double> b(kv);
  const double rhoInv = mesh.rhoInvVp[src];
  for (uint64_t i = 0; i < kv; ++i) b[i] = rhoInv * phiVp[src + mesh.nvp * i];
  double cfl = 0;
  if (in.checkCfl && (rc = host::check_cfl(mesh, in.dt, cfl))) return rc;
  if (in.checkDispersion && (rc = host::check_dispersion(mesh, 1.0 / in.periods[0]))) return rc;
  RomGuard r;
  if ((rc = shaw_rom_create(kv, ks, Av.data(), As.data(), 1, 1, b.data(), SHAW_FP64, &r.h))) return rc;
  const int32_t kind = in.signalKind;
  if ((rc = shaw_rom_set_signals(r.h, &kind, &in.periods[0], &in.delays[0]))) return rc;
  std::vector<double> snapVp, snapSp;
  if (in.snapEnabled) {
    if (in.nsteps % in.snapFreqVp != 0)
      return fail(SHAW_ERR_FREQ_DIVISOR, "Snapshot Vp frequency not a divisor of steps");
    if (in.nsteps % in.snapFreqSp != 0)
      return fail(SHAW_ERR_FREQ_DIVISOR, "Snapshot Sp frequency not a divisor of steps");
    snapVp.assign(kv * (in.nsteps / in.snapFreqVp), 0.0);
    snapSp.assign(ks * (in.nsteps / in.snapFreqSp), 0.0);
    if ((rc = shaw_rom_set_snapshots(r.h, in.snapFreqVp, in.snapFreqSp, in.nsteps, snapVp.data(), snapSp.data())))
      return rc;
  }
  if ((rc = shaw_rom_run(r.h, in.dt, in.nsteps))) return rc;
  // processCollectedData: only with a real basis (rom_problem_rank_one.hpp:168-189)
  if (!in.romDummyBasis && in.snapEnabled) {
    if ((rc = write_observed(in.snapFileVp + "_0", snapVp.data(), kv, in.nsteps / in.snapFreqVp, 1, in.snapBinary,
                             true)))
      return rc;
    if ((rc = write_observed(in.snapFileSp + "_0", snapSp.data(), ks, in.nsteps / in.snapFreqSp, 1, in.snapBinary,
                             true)))
      return rc;
  }
  return SHAW_OK;
}

}  // namespace driver
}  // namespace shaw
