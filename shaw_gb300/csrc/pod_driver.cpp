// pod_driver.cpp -- the computeThinSVD tool (src/tools/main_eigen_svd.cc:199-305) on top
// of shaw_pod: read snaps_<dof>_0 from each directory, concatenate the snapshot
// columns, take the thin SVD on the GPU, write sva_<dof> and lsv_<dof> to the current
// directory, first for "vp", then for "sp".
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "driver.h"
#include "shaw_gpu.h"

namespace shaw {
namespace driver {
namespace {

// readBinaryMatrixWithSize (main_eigen_svd.cc:62-86): size_t rows, size_t cols, then
// rows*cols doubles in column-major order.
int read_binary_with_size(const std::string& file, uint64_t& rows, uint64_t& cols, std::vector<double>& M) {
  std::ifstream fin(file, std::ios::in | std::ios::binary);
  if (!fin) return fail(SHAW_ERR_IO, "ERROR READING binary file " + file);
  size_t r = 0, c = 0;
  fin.read((char*)&r, sizeof(size_t));
  fin.read((char*)&c, sizeof(size_t));
  if (!fin) return fail(SHAW_ERR_IO, "ERROR READING binary file " + file);
  M.resize(r * c);
  fin.read((char*)M.data(), (std::streamsize)(r * c * sizeof(double)));
  if (!fin) return fail(SHAW_ERR_IO, "ERROR READING binary file " + file);
  std::cout << fin.gcount() << " bytes read\n";
  rows = r;
  cols = c;
  return SHAW_OK;
}

// `file << std::setprecision(17) << singVal << '\n'` with Eigen's default IOFormat
// (Eigen/src/Core/IO.h print_matrix): one value per line, right-aligned to the widest
// value, no newline after the last value, then the caller's '\n'.
int write_singular_values(const std::string& file, const std::vector<double>& sv) {
  std::vector<std::string> txt(sv.size());
  size_t width = 0;
  char buf[64];
  for (size_t i = 0; i < sv.size(); ++i) {
    std::snprintf(buf, sizeof(buf), "%.17g", sv[i]);
    txt[i] = buf;
    width = std::max(width, txt[i].size());
  }
  std::ofstream out(file, std::ios::out | std::ios::trunc);
  if (!out) return fail(SHAW_ERR_IO, "cannot write " + file);
  for (size_t i = 0; i < sv.size(); ++i) {
    out << std::string(width - txt[i].size(), ' ') << txt[i];
    if (i + 1 < sv.size()) out << '\n';
  }
  out << '\n';
  return out ? SHAW_OK : fail(SHAW_ERR_IO, "write failed: " + file);
}

int process_dof(const std::string& dof, const std::vector<std::string>& dirs, const std::string& readerFormat,
                int method) {
  const auto t0 = std::chrono::high_resolution_clock::now();
  std::vector<double> all;
  uint64_t nrows = 0, ncols = 0;
  for (size_t d = 0; d < dirs.size(); ++d) {
    const std::string file = dirs[d] + "/snaps_" + dof + "_0";
    std::cout << "\nReading snapshots: " << file << std::endl;
    uint64_t r = 0, c = 0;
    std::vector<double> M;
    // loadTargetSnapshotMatrix (:88-111) reads binary files only; any other format
    // leaves the matrix empty.
    if (readerFormat == "binary") {
      std::cout << "Using Binary " << std::endl;
      if (int rc = read_binary_with_size(file, r, c, M)) return rc;
    }
    std::cout << "Current snapshots size: " << r << " " << c << std::endl;
    if (d == 0) {
      nrows = r;
    } else if (r != nrows) {
      return fail(SHAW_ERR_INVALID_ARG, "Mismatching # rows of current data with previous");
    }
    all.insert(all.end(), M.begin(), M.end());  // column-major: new columns append
    ncols += c;
  }
  std::cout << "Final snapshot matrix size: " << nrows << " " << ncols << std::endl;
  const auto t1 = std::chrono::high_resolution_clock::now();
  std::printf("svd:read:%s: %.10f\n", dof.c_str(), std::chrono::duration<double>(t1 - t0).count());
  std::fflush(stdout);
  if (method != 1 && method != 2) return SHAW_OK;  // processDirs (:261-267) does nothing
  if (nrows == 0 || ncols == 0)
    return fail(SHAW_ERR_INVALID_ARG, "empty snapshot matrix (" + dof +
                                          "): snapshots are read only when the format that reaches the reader "
                                          "(the --outformat value) is binary");
  std::cout << "Computing SVD method " << method << std::endl;
  const uint64_t k = std::min(nrows, ncols);
  std::vector<double> U(nrows * k), sv(k);
  if (int rc = shaw_pod(all.data(), nrows, ncols, method, U.data(), sv.data())) return rc;
  std::cout << "Printing sing values" << std::endl;
  if (int rc = write_singular_values("sva_" + dof, sv)) return rc;
  std::cout << "\nPrinting left-sing vectors to file" << std::endl;
  // writeToFile (:52-59) is always binary with extents, whatever --outformat says
  if (int rc = write_matrix("lsv_" + dof, U.data(), nrows, k, true, true)) return rc;
  std::cout << "Done with SVD" << std::endl << "----------------" << std::endl;
  const auto t2 = std::chrono::high_resolution_clock::now();
  std::printf("svd:time%s: %.10f\n", dof.c_str(), std::chrono::duration<double>(t2 - t0).count());
  std::fflush(stdout);
  return SHAW_OK;
}

}  // namespace
}  // namespace driver
}  // namespace shaw

extern "C" int shaw_pod_tool(const char* const* dirs, uint32_t ndirs, const char* informat, const char* outformat,
                             int method) {
  using namespace shaw::driver;
  if (method == -1) return shaw::fail(SHAW_ERR_INVALID_ARG, "Invalid method");
  if (!dirs || ndirs == 0 || !informat || !outformat)
    return shaw::fail(SHAW_ERR_INVALID_ARG, "--dirs, --informat, --outformat and --method are required");
  std::vector<std::string> d(dirs, dirs + ndirs);
  (void)informat;  // main_eigen_svd.cc:302-303 hands --outformat to the snapshot reader
  if (int rc = process_dof("vp", d, outformat, method)) return rc;
  return process_dof("sp", d, outformat, method);
}
