// driver.cpp -- the shawExe replacement: input parsing (src/shared/parser/*.hpp
// semantics), the FOM/ROM problem drivers (src/kokkos/fom_problem_rank_{one,two}.hpp,
// src/kokkos/rom_problem_rank_one.hpp) and the output writers
// (src/shared/io/matrix_write.hpp).  All stepping goes through the C ABI.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "driver.h"
#include "host_internal.h"
#include "shaw_gpu.h"
#include "yaml_lite.h"

namespace shaw {
namespace driver {

using yaml::Node;

namespace {

int parse_error(const std::string& m) { return fail(SHAW_ERR_PARSE, m); }

int signal_kind_from(const std::string& s) {
  if (s == "ricker" || s == "Ricker") return SHAW_SIGNAL_RICKER;
  if (s == "sinusoid" || s == "Sinusoid") return SHAW_SIGNAL_SINUSOID;
  if (s == "gaussDer" || s == "gaussianDeriv") return SHAW_SIGNAL_GAUSS_DER;
  return -1;
}

std::vector<double> scalar_or_list(const Node& n) {
  if (n.is_scalar()) return {n.as_double()};
  return n.as_double_vector();
}

void fill3(const Node* n, double* out) {
  out[0] = out[1] = out[2] = 0.0;
  if (!n) throw std::runtime_error("missing layer coefficients");
  const auto v = n->as_double_vector();
  for (size_t i = 0; i < v.size() && i < 3; ++i) out[i] = v[i];
}

}  // namespace

// InputParser<general, io, material, forcing, rom> (src/kokkos/types.hpp:64-69)
int parse_input(const std::string& path, Input& in) {
  Node root;
  try {
    root = yaml::parse_file(path);
  } catch (const std::exception& e) {
    return parse_error(e.what());
  }
  try {
    // parser_general_section.hpp:78-125
    const Node* g = root.get("general");
    if (!g) return parse_error("General section in yaml input is mandatory!");
    if (const Node* n = g->get("meshDir")) in.meshDir = n->as_string(); else return parse_error("Empty meshDir");
    if (const Node* n = g->get("checkNumericalDispersion")) in.checkDispersion = n->as_bool();
    if (const Node* n = g->get("checkCfl")) in.checkCfl = n->as_bool();
    if (const Node* n = g->get("dt")) in.dt = n->as_double(); else return parse_error("Empty dt");
    if (const Node* n = g->get("finalTime")) in.finalTime = n->as_double(); else return parse_error("Empty final time");
    if (const Node* n = g->get("exploitForcingSparsity")) in.exploitForcingSparsity = n->as_bool();
    in.nsteps = (uint64_t)(in.finalTime / in.dt);
    if (in.dt <= 0.) return parse_error("Cannot have dt <= 0");
    if (in.finalTime <= 0.) return parse_error("Cannot have finalT <= 0");

    // parser_io_section.hpp:110-190
    if (const Node* io = root.get("io")) {
      if (const Node* sm = io->get("snapshotMatrix")) {
        in.snapEnabled = true;
        if (const Node* b = sm->get("binary")) in.snapBinary = b->as_bool();
        const Node* v = sm->get("velocity");
        if (!v) return parse_error("Cannot find io inputs for velocity");
        if (const Node* f = v->get("freq")) in.snapFreqVp = f->as_size();
        else return parse_error("You must set snapshot freq for velocity");
        if (const Node* f = v->get("fileName")) in.snapFileVp = f->as_string();
        const Node* s = sm->get("stress");
        if (!s) return parse_error("Cannot find io inputs for stress");
        if (const Node* f = s->get("freq")) in.snapFreqSp = f->as_size();
        else return parse_error("You must set snapshot freq for stress");
        if (const Node* f = s->get("fileName")) in.snapFileSp = f->as_string();
      }
      if (const Node* se = io->get("seismogram")) {
        in.seisEnabled = true;
        if (const Node* b = se->get("binary")) in.seisBinary = b->as_bool();
        if (const Node* f = se->get("fileName")) in.seisFile = f->as_string();
        if (const Node* f = se->get("freq")) in.seisFreq = f->as_size();
        else return parse_error("You must set freq for seismogram");
        if (const Node* r = se->get("receivers"))
          if (r->is_seq()) in.receivers = r->as_double_vector();
      }
      if (in.snapEnabled) {
        if (in.snapFreqVp == 0) return parse_error("cannot have vpSnapshotsFreq <=0 ");
        if (in.snapFreqSp == 0) return parse_error("cannot have spSnapshotsFreq <=0 ");
      }
      if (in.seisEnabled && in.seisFreq == 0) return parse_error("cannot have seismoFreq <=0 ");
    }

    // parser_material_model.hpp:98-181
    const Node* mat = root.get("material");
    if (!mat) return parse_error("Cannot find material section in yaml");
    const Node* kind = mat->get("kind");
    if (!kind) return parse_error("material kind missing");
    const std::string k = kind->as_string();
    in.matParams.assign(13, 0.0);
    if (k == "unilayer" || k == "Unilayer" || k == "UniLayer") {
      in.matKind = SHAW_MATERIAL_UNILAYER;
      const Node* l = mat->get("layer");
      if (!l) return parse_error("unilayer needs a layer entry");
      fill3(l->get("density"), &in.matParams[0]);
      fill3(l->get("velocity"), &in.matParams[3]);
    } else if (k == "bilayer" || k == "Bilayer" || k == "BiLayer") {
      in.matKind = SHAW_MATERIAL_BILAYER;
      const Node* l1 = mat->get("layer1");
      const Node* l2 = mat->get("layer2");
      if (!l1 || !l2) return parse_error("bilayer needs layer1 and layer2");
      fill3(l1->get("density"), &in.matParams[0]);
      fill3(l1->get("velocity"), &in.matParams[3]);
      const Node* d = l2->get("depth");
      if (!d) return parse_error("layer2 needs a depth");
      in.matParams[6] = d->as_double();
      fill3(l2->get("density"), &in.matParams[7]);
      fill3(l2->get("velocity"), &in.matParams[10]);
    } else if (k == "prem" || k == "PREM") {
      in.matKind = SHAW_MATERIAL_PREM;
    } else if (k == "custom") {
      in.matKind = kMaterialCustom;
    } else {
      return parse_error("Unknown material model kind, maybe mispelled it?");
    }

    // parser_forcing_section.hpp:93-287
    const Node* src = root.get("source");
    if (!src) return parse_error("Cannot find source section in inputfile, must be set!");
    const Node* sig = src->get("signal");
    if (!sig) return parse_error("Signal node in inputfile is missing, it is mandatory!");
    const Node* sk = sig->get("kind");
    if (!sk) return parse_error("You must set the kind of the signal");
    in.signalKind = signal_kind_from(sk->as_string());
    if (const Node* n = sig->get("depth")) in.depths = scalar_or_list(*n);
    else return parse_error("You must set the depth of the signal");
    if (const Node* n = sig->get("angle")) in.angles = scalar_or_list(*n);
    else in.angles = {0.};
    if (const Node* n = sig->get("period")) in.periods = scalar_or_list(*n);
    else return parse_error("You must set the period of the signal");
    if (const Node* n = sig->get("delay")) in.delays = scalar_or_list(*n);
    else return parse_error("You must set the delay of the signal");
    if (const Node* n = sig->get("forcingSize")) {
      in.forcingSize = (int)n->as_int();
      in.rank2 = true;
    }
    if (in.depths.empty() || in.angles.empty() || in.periods.empty() || in.delays.empty())
      return parse_error("source lists must not be empty");
    in.multiForcing = in.depths.size() >= 2 || in.angles.size() >= 2 || in.periods.size() >= 2 ||
                      in.delays.size() >= 2;
    if (in.signalKind < 0)
      return parse_error("Invalid source kind: unknown, maybe you mispelled it in input file?");
    for (double d : in.depths)
      if (d <= 0.) return parse_error("The depth of the source must be a positive number");
    for (double a : in.angles)
      if (a < 0.) return parse_error("The angle of source must be zero or a positive value");
    for (double p : in.periods)
      if (p <= 0.) return parse_error("Period for signal must be positive. ");
    for (double d : in.delays)
      if (d < 0.) return parse_error("Delay time of the signal must be >=0");
    if (in.rank2 && in.forcingSize < 1) return parse_error("forcingSize must be >= 1");

    // parser_rom_section.hpp:107-165
    if (const Node* rom = root.get("rom")) {
      in.romEnabled = true;
      if (const Node* n = rom->get("disableCompRomJacs")) in.disableRomJacs = n->as_bool();
      const Node* v = rom->get("velocity");
      if (!v) return parse_error("Cannot find rom inputs for velocity");
      if (const Node* n = v->get("numModes")) in.romModesVp = n->as_size();
      else return parse_error("You must set # of modes for velocity");
      if (const Node* n = v->get("modesFile")) in.romFileVp = n->as_string();
      if (const Node* n = v->get("binary")) in.romBinaryVp = n->as_bool();
      const Node* s = rom->get("stress");
      if (!s) return parse_error("Cannot find rom inputs for stress");
      if (const Node* n = s->get("numModes")) in.romModesSp = n->as_size();
      else return parse_error("You must set # of modes for stress");
      if (const Node* n = s->get("modesFile")) in.romFileSp = n->as_string();
      if (const Node* n = s->get("binary")) in.romBinarySp = n->as_bool();
      if (in.romFileVp == "empty" || in.romFileSp == "empty") in.romDummyBasis = true;
      if (in.romModesVp == 0) return parse_error("Cannot have vpRomSize <=0 ");
      if (in.romModesSp == 0) return parse_error("Cannot have spRomSize <=0 ");
    }
  } catch (const std::exception& e) {
    return parse_error(e.what());
  }
  return SHAW_OK;
}

// ---- writers: src/shared/io/matrix_write.hpp:60-191 ------------------------

int write_matrix(const std::string& file, const double* A, uint64_t m, uint64_t n, bool binary, bool writeSize) {
  if (binary) {
    std::ofstream out(file, std::ios::out | std::ios::binary | std::ios::trunc);
    if (!out) return fail(SHAW_ERR_IO, "cannot write " + file);
    if (writeSize) {
      const size_t mm = m, nn = n;
      out.write((const char*)&mm, sizeof(size_t));
      out.write((const char*)&nn, sizeof(size_t));
    }
    out.write((const char*)A, (std::streamsize)(m * n * sizeof(double)));
    return out ? SHAW_OK : fail(SHAW_ERR_IO, "write failed: " + file);
  }
  FILE* f = std::fopen(file.c_str(), "w");
  if (!f) return fail(SHAW_ERR_IO, "cannot write " + file);
  if (writeSize) std::fprintf(f, "%llu %llu\n", (unsigned long long)m, (unsigned long long)n);
  for (uint64_t i = 0; i < m; ++i) {
    for (uint64_t j = 0; j < n; ++j) std::fprintf(f, "%.17g ", A[i + m * j]);
    std::fputc('\n', f);
  }
  std::fclose(f);
  return SHAW_OK;
}

int write_3d(const std::string& file, const double* A, uint64_t s0, uint64_t s1, uint64_t s2, bool binary,
             bool writeSize) {
  if (binary) {
    std::ofstream out(file, std::ios::out | std::ios::binary | std::ios::trunc);
    if (!out) return fail(SHAW_ERR_IO, "cannot write " + file);
    if (writeSize) {
      const size_t a = s0, b = s1, c = s2;
      out.write((const char*)&a, sizeof(size_t));
      out.write((const char*)&b, sizeof(size_t));
      out.write((const char*)&c, sizeof(size_t));
    }
    out.write((const char*)A, (std::streamsize)(s0 * s1 * s2 * sizeof(double)));
    return out ? SHAW_OK : fail(SHAW_ERR_IO, "write failed: " + file);
  }
  FILE* f = std::fopen(file.c_str(), "w");
  if (!f) return fail(SHAW_ERR_IO, "cannot write " + file);
  if (writeSize)
    std::fprintf(f, "%llu %llu %llu\n", (unsigned long long)s0, (unsigned long long)s1, (unsigned long long)s2);
  for (uint64_t k = 0; k < s2; ++k)
    for (uint64_t i = 0; i < s0; ++i) {
      for (uint64_t j = 0; j < s1; ++j) std::fprintf(f, "%.17g ", A[i + s0 * (j + s1 * k)]);
      std::fputc('\n', f);
    }
  std::fclose(f);
  return SHAW_OK;
}

// Seismogram::writeReceiversToFile / StateObserver::writeSnapshotMatrixToFile: a
// 2-D write when the third extent is 1, else a 3-D write.
int write_observed(const std::string& file, const double* A, uint64_t s0, uint64_t s1, uint64_t s2, bool binary,
                   bool writeSize) {
  if (s2 == 1) return write_matrix(file, A, s0, s1, binary, writeSize);
  return write_3d(file, A, s0, s1, s2, binary, writeSize);
}

// ShWavePP::writeCoordinatesToFile (shwavepp.hpp:231-243)
int write_coordinates(const shaw_mesh_s& m) {
  for (int dof = 0; dof < 2; ++dof) {
    const std::string file = dof == 0 ? "coords_vp.txt" : "coords_sp.txt";
    const auto& c = dof == 0 ? m.cvp : m.csp;
    const uint64_t n = dof == 0 ? m.nvp : m.nsp;
    FILE* f = std::fopen(file.c_str(), "w");
    if (!f) return fail(SHAW_ERR_IO, "cannot write " + file);
    for (uint64_t i = 0; i < n; ++i) std::fprintf(f, "%.17g %.17g\n", c[i * 2], 1.0 / c[i * 2 + 1]);
    std::fclose(f);
  }
  return SHAW_OK;
}

namespace {

struct FomGuard {
  shaw_fom_t h = nullptr;
  ~FomGuard() { shaw_fom_destroy(h); }
};

// The reference's cost model of one leapfrog step (fom_complexities.hpp:57-137 with the
// Spmv / Spmm / Mult formulas of src/shared/complexities/: FP64 values, size_t ordinals)
// and its log lines (print_perf.hpp:57-84), which the reference's scaling scripts parse.
// nnz(Jvp) = 4 nvp - 2 nth - 2 nr (merged CMB/surface and axis entries), nnz(Jsp) = 2 nsp.
void print_perf(int rank, uint64_t M, const shaw_mesh_s& mesh, uint64_t nsteps, const double perf[3]) {
  const double sc = sizeof(double), ord = sizeof(uint64_t), MB = 1024.0 * 1024.0;
  const double nvp = (double)mesh.nvp, nsp = (double)mesh.nsp;
  const double nnzVp = 4.0 * nvp - 2.0 * (double)mesh.nth - 2.0 * (double)mesh.nr, nnzSp = 2.0 * nsp;
  const double k = (double)M;
  auto sparse = [&](double nnz, double rows, double& mem, double& fl) {  // spmv (k == 1) / spmm
    mem = (nnz * (sc + ord) + rows * ord + nnz * k * sc + 2.0 * rows * k * sc) / MB;
    fl = 2.0 * nnz * k + rows * k;
  };
  double m0, f0, m2, f2, m1, f1;
  sparse(nnzVp, nvp, m0, f0);
  sparse(nnzSp, nsp, m2, f2);
  if (rank == 1) { m1 = 4.0 * nvp * sc / MB; f1 = 3.0 * nvp; }  // mult with beta = 1
  else { m1 = 4.0 * k * sc / MB; f1 = 3.0 * k; }                // the rank-2 forcing loop
  const double memMB = m0 + m1 + m2, flops = f0 + f1 + f2;
  const double minT = perf[0], maxT = perf[1], tot = perf[2], ave = tot / (double)nsteps;
  const double GB = memMB / 1024.;
  std::cout << "flops = " << flops << std::endl;
  std::cout << "memMB = " << memMB << std::endl;
  std::cout << "flops/bytes = " << flops / (memMB * MB) << std::endl;
  std::printf("aveBandwidth(GB/s) = %8.2lf \n", GB / ave);
  std::printf("minBandwidth(GB/s) = %8.2lf \n", GB / maxT);
  std::printf("maxBandwidth(GB/s) = %8.2lf \n", GB / minT);
  std::printf("aveGFlop = %7.4lf \n", flops / ave / 1e9);
  std::printf("minGFlop = %7.4lf \n", flops / maxT / 1e9);
  std::printf("maxGFlop = %7.4lf \n", flops / minT / 1e9);
  std::printf("totTime(se) = %7.4lf \n", tot);
  std::printf("aveTime(ms) = %7.4lf \n", ave * 1000);
  std::printf("maxTime(ms) = %7.4lf \n", maxT * 1000);
  std::printf("minTime(ms) = %7.4lf \n", minT * 1000);
  std::printf("dofUpdatesPerSec = %.6e \n", (nvp + nsp) * k / ave);
  std::fflush(stdout);
}

}  // namespace

// One runFom over a set of forcings (rank-1 single, one multi-forcing sample, or
// one rank-2 set), then processCollectedData for run id `runId`.
int run_fom_set(const Input& in, const shaw_mesh_s& mesh, int rank, const std::vector<uint64_t>& srcGids,
                const std::vector<double>& periods, const std::vector<double>& delays,
                const std::vector<uint64_t>& rcvGids, uint64_t runId) {
  const uint32_t M = (uint32_t)srcGids.size();
  shaw_fom_operator_desc d;
  host::operator_desc(mesh, d);
  FomGuard g;
  int rc = shaw_fom_create(&d, rank, M, SHAW_FP64, &g.h);
  if (rc) return rc;
  std::vector<int32_t> kinds(M, in.signalKind);
  if ((rc = shaw_fom_set_sources(g.h, srcGids.data(), kinds.data(), periods.data(), delays.data()))) return rc;
  if (in.seisEnabled) {
    if ((rc = shaw_fom_set_receivers(g.h, rcvGids.data(), (uint32_t)rcvGids.size(), in.seisFreq, in.nsteps)))
      return rc;
  }
  std::vector<double> snapVp, snapSp;
  if (in.snapEnabled) {
    if (in.nsteps % in.snapFreqVp != 0)
      return fail(SHAW_ERR_FREQ_DIVISOR, "Snapshot Vp frequency not a divisor of steps");
    if (in.nsteps % in.snapFreqSp != 0)
      return fail(SHAW_ERR_FREQ_DIVISOR, "Snapshot Sp frequency not a divisor of steps");
    snapVp.assign(mesh.nvp * (in.nsteps / in.snapFreqVp) * M, 0.0);
    snapSp.assign(mesh.nsp * (in.nsteps / in.snapFreqSp) * M, 0.0);
    if ((rc = shaw_fom_set_snapshots(g.h, in.snapFreqVp, in.snapFreqSp, in.nsteps, snapVp.data(), snapSp.data())))
      return rc;
  }
  // runFom: the steps run in chunks (multiples of the 64-step CUDA-graph chunk, at most
  // about 64 chunks), each timed on the host after its work completes; the per-step
  // min / max / total of the reference's log come from the chunks' per-step averages.
  if ((rc = shaw_fom_reset(g.h))) return rc;
  const uint64_t chunk = std::max<uint64_t>(64, (in.nsteps / 64 + 63) / 64 * 64);
  double perf[3] = {1e32, 0.0, 0.0};
  const auto t0 = std::chrono::steady_clock::now();
  for (uint64_t done = 0; done < in.nsteps;) {
    const uint64_t c = std::min(chunk, in.nsteps - done);
    const auto c0 = std::chrono::steady_clock::now();
    if ((rc = shaw_fom_advance(g.h, in.dt, c))) return rc;
    if ((rc = shaw_fom_synchronize(g.h))) return rc;
    const double per = std::chrono::duration<double>(std::chrono::steady_clock::now() - c0).count() / (double)c;
    perf[0] = std::min(perf[0], per);
    perf[1] = std::max(perf[1], per);
    perf[2] += per * (double)c;
    done += c;
  }
  const double loop = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf("\nloopTime = %.10f", loop);
  // release the page-locked snapshot registration before writing
  if (in.snapEnabled && (rc = shaw_fom_set_snapshots(g.h, 0, 0, 0, nullptr, nullptr))) return rc;
  const std::string id = "_" + std::to_string(runId);
  if (in.snapEnabled) {
    if ((rc = write_observed(in.snapFileVp + id, snapVp.data(), mesh.nvp, in.nsteps / in.snapFreqVp, M,
                             in.snapBinary, true)))
      return rc;
    if ((rc = write_observed(in.snapFileSp + id, snapSp.data(), mesh.nsp, in.nsteps / in.snapFreqSp, M,
                             in.snapBinary, true)))
      return rc;
  }
  // dataCollectionTime: the observers' host work outside the device loop (the sampled
  // snapshot columns arrive during the loop; the seismogram is read back once here)
  const auto d0 = std::chrono::steady_clock::now();
  std::vector<double> seis;
  if (in.seisEnabled) {
    seis.resize(rcvGids.size() * (in.nsteps / in.seisFreq) * M);
    if ((rc = shaw_fom_get_seismogram(g.h, seis.data()))) return rc;
  }
  std::printf("\ndataCollectionTime = %.10f\n",
              std::chrono::duration<double>(std::chrono::steady_clock::now() - d0).count());
  print_perf(rank, M, mesh, in.nsteps, perf);
  if (in.seisEnabled) {
    const uint64_t T = in.nsteps / in.seisFreq;
    if ((rc = write_observed(in.seisFile + id, seis.data(), rcvGids.size(), T, M, in.seisBinary, false))) return rc;
  }
  return SHAW_OK;
}

// FomProblemRankOneForcing (fom_problem_rank_one.hpp:105-191) and
// FomProblemRankTwoForcing (fom_problem_rank_two.hpp:109-193).
int run_fom(const Input& in, const shaw_mesh_s& mesh) {
  int rc;
  std::vector<uint64_t> rcv;
  if (in.seisEnabled) {
    if (in.nsteps % in.seisFreq != 0)
      return fail(SHAW_ERR_FREQ_DIVISOR, "Seismogram sampling frequency not a divisor of steps");
    for (double a : in.receivers) {
      uint64_t g = 0;
      if ((rc = host::map_receiver(mesh, a, g))) return rc;
      rcv.push_back(g);
    }
  }
  double cfl = 0;
  if (in.checkCfl && (rc = host::check_cfl(mesh, in.dt, cfl))) return rc;
  if (in.checkDispersion)
    for (double T : in.periods)
      if ((rc = host::check_dispersion(mesh, 1.0 / T))) return rc;

  // realizations in the reference's order: depth > period > angle > delay
  struct Real { double depth, period, angle, delay; };
  std::vector<Real> reals;
  for (double d : in.depths)
    for (double p : in.periods)
      for (double a : in.angles)
        for (double de : in.delays) reals.push_back({d, p, a, de});

  if (!in.rank2) {
    const size_t n = in.multiForcing ? reals.size() : 1;
    for (size_t s = 0; s < n; ++s) {
      uint64_t g = 0;
      if ((rc = host::map_source(mesh, reals[s].depth, reals[s].angle, g))) return rc;
      if ((rc = run_fom_set(in, mesh, 1, {g}, {reals[s].period}, {reals[s].delay}, rcv, s))) return rc;
    }
  } else {
    const size_t fs = (size_t)in.forcingSize;
    if (reals.size() % fs != 0)
      return fail(SHAW_ERR_FORCING_SETS,
                  "totFRealizations & fSize != 0: tot num of forcing realizations must be divisible by fSize");
    for (size_t set = 0; set < reals.size() / fs; ++set) {
      std::vector<uint64_t> gids;
      std::vector<double> per, del;
      for (size_t k = set * fs; k < (set + 1) * fs; ++k) {
        uint64_t g = 0;
        if ((rc = host::map_source(mesh, reals[k].depth, reals[k].angle, g))) return rc;
        gids.push_back(g);
        per.push_back(reals[k].period);
        del.push_back(reals[k].delay);
      }
      if ((rc = run_fom_set(in, mesh, 2, gids, per, del, rcv, set))) return rc;
    }
  }
  if (in.snapEnabled && (rc = write_coordinates(mesh))) return rc;
  return SHAW_OK;
}

int run_input_file(const std::string& path) {
  Input in;
  int rc = parse_input(path, in);
  if (rc) return rc;
  // ParserGeneralSection::print (parser_general_section.hpp:127-134)
  std::cout << "\nmeshDir = " << in.meshDir << " \n"
            << "checkDispersion = " << std::boolalpha << in.checkDispersion << " \n"
            << "timeStep = " << in.dt << " \n"
            << "finalT = " << in.finalTime << " \n"
            << "numSteps = " << in.nsteps << " \n"
            << "exploitForcingSparsity " << true << " \n" << std::noboolalpha;
  shaw_mesh_s mesh;
  if ((rc = host::load_mesh(in.meshDir, mesh))) return rc;
  // MeshInfo's log lines (mesh_info.hpp:196-212)
  std::cout << "numGptVp = " << mesh.nvp << "\nnumGptSp = " << mesh.nsp << "\nnth = " << mesh.nth
            << "\nnr = " << mesh.nr << std::endl;
  if (in.matKind == kMaterialCustom)
    return fail(SHAW_ERR_UNSUPPORTED,
                "custom material: supply per-point arrays through shaw_mesh_set_material_arrays");
  if ((rc = host::set_material(mesh, in.matKind, in.matParams.data(), (uint32_t)in.matParams.size()))) return rc;
  if (in.romEnabled) return run_rom(in, mesh);
  return run_fom(in, mesh);
}

}  // namespace driver
}  // namespace shaw

extern "C" int shaw_run_input_file(const char* yaml_path) {
  if (!yaml_path) return shaw::fail(SHAW_ERR_INVALID_ARG, "null path");
  return shaw::driver::run_input_file(yaml_path);
}

extern "C" int shaw_parse_input(const char* yaml_path, char* out, size_t cap) {
  if (!yaml_path || (!out && cap)) return shaw::fail(SHAW_ERR_INVALID_ARG, "null argument");
  shaw::driver::Input in;
  const int rc = shaw::driver::parse_input(yaml_path, in);
  if (rc) return rc;
  std::ostringstream s;
  s.precision(17);
  auto list = [&](const std::vector<double>& v) {
    std::ostringstream t;
    t.precision(17);
    for (size_t i = 0; i < v.size(); ++i) t << (i ? "," : "") << v[i];
    return t.str();
  };
  static const char* kinds[] = {"ricker", "sinusoid", "gaussDer"};
  static const char* mats[] = {"unilayer", "bilayer", "prem"};
  s << "getMeshDir=" << in.meshDir << "\n"
    << "checkDispersion=" << (in.checkDispersion ? "true" : "false") << "\n"
    << "checkCfl=" << (in.checkCfl ? "true" : "false") << "\n"
    << "getTimeStepSize=" << in.dt << "\n"
    << "getNumSteps=" << in.nsteps << "\n"
    << "enableSnapshotMatrix=" << (in.snapEnabled ? "true" : "false") << "\n"
    << "writeSnapshotsBinary=" << (in.snapBinary ? "true" : "false") << "\n"
    << "getSnapshotFreq(vp)=" << in.snapFreqVp << "\n"
    << "getSnapshotFreq(sp)=" << in.snapFreqSp << "\n"
    << "getSnapshotFileName(vp)=" << in.snapFileVp << "\n"
    << "getSnapshotFileName(sp)=" << in.snapFileSp << "\n"
    << "enableSeismogram=" << (in.seisEnabled ? "true" : "false") << "\n"
    << "writeSeismogramBinary=" << (in.seisBinary ? "true" : "false") << "\n"
    << "getSeismogramFileName=" << in.seisFile << "\n"
    << "getSeismoFreq=" << in.seisFreq << "\n"
    << "getSeismoReceiversAnglesDeg=" << list(in.receivers) << "\n"
    << "getSourceSignalKind=" << (in.signalKind >= 0 ? kinds[in.signalKind] : "unknown") << "\n"
    << "viewDepths=" << list(in.depths) << "\n"
    << "viewAngles=" << list(in.angles) << "\n"
    << "viewPeriods=" << list(in.periods) << "\n"
    << "viewDelays=" << list(in.delays) << "\n"
    << "multiForcing=" << (in.multiForcing ? "true" : "false") << "\n"
    << "rank2Enabled=" << (in.rank2 ? "true" : "false") << "\n"
    << "getForcingSize=" << in.forcingSize << "\n"
    << "getMaterialModelKind=" << (in.matKind == shaw::driver::kMaterialCustom ? "custom" : mats[in.matKind]) << "\n"
    << "materialParams=" << list(in.matParams) << "\n"
    << "enableRom=" << (in.romEnabled ? "true" : "false") << "\n"
    << "getRomSize(vp)=" << in.romModesVp << "\n"
    << "getRomSize(sp)=" << in.romModesSp << "\n"
    << "getBasisFileName(vp)=" << in.romFileVp << "\n"
    << "getBasisFileName(sp)=" << in.romFileSp << "\n"
    << "enableRandomDummyBasis=" << (in.romDummyBasis ? "true" : "false") << "\n"
    << "disableCompRomJacobians=" << (in.disableRomJacs ? "true" : "false") << "\n";
  const std::string t = s.str();
  if (t.size() + 1 > cap) return shaw::fail(SHAW_ERR_INVALID_ARG, "output buffer too small");
  std::memcpy(out, t.c_str(), t.size() + 1);
  return SHAW_OK;
}
