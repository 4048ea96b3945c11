// main.cpp -- `shaw_exe <input.yaml>`: the drop-in for the reference's
// `shawExe <input.yaml>` (src/kokkos/main.cc:41-94).  Outputs go to the
// current directory with the reference's names and formats.
#include <cstdio>

#include "shaw_gpu.h"

int main(int argc, char* argv[]) {
  if (argc != 2) {
    std::fprintf(stderr, "Wrong # of cmd line args, should be: ./exe <path-to-inputfile>\n");
    return 1;
  }
  const int rc = shaw_run_input_file(argv[1]);
  if (rc != SHAW_OK) {
    std::fprintf(stderr, "shaw_exe: error %d: %s\n", rc, shaw_last_error());
    return 1;
  }
  return 0;
}
