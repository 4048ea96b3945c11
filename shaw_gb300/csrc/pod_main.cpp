// pod_main.cpp -- `computeThinSVD --dirs <d1> [<d2> ...] --informat <f> --outformat <f>
// --method <1|2>`: the drop-in for the reference's POD tool (src/tools/main_eigen_svd.cc:
// 279-305, built as computeThinSVD by CMakeLists.txt:57).  Options may also be given as
// --opt=value.  As in the reference, a malformed command line is not an error by
// itself; a missing --method is ("Invalid method").
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "shaw_gpu.h"

int main(int argc, char* argv[]) {
  std::vector<std::string> dirs;
  std::string informat, outformat;
  int method = -1;
  bool haveIn = false, haveOut = false;
  for (int i = 1; i < argc; ++i) {
    std::string opt = argv[i], val;
    bool inlineVal = false;
    const size_t eq = opt.find('=');
    if (opt.rfind("--", 0) == 0 && eq != std::string::npos) {
      val = opt.substr(eq + 1);
      opt = opt.substr(0, eq);
      inlineVal = true;
    }
    auto next = [&](std::string& out) {
      if (inlineVal) {
        out = val;
        return true;
      }
      if (i + 1 < argc && std::strncmp(argv[i + 1], "--", 2) != 0) {
        out = argv[++i];
        return true;
      }
      return false;
    };
    if (opt == "--dirs") {
      if (inlineVal) {
        dirs.push_back(val);
      } else {
        while (i + 1 < argc && std::strncmp(argv[i + 1], "--", 2) != 0) dirs.push_back(argv[++i]);
      }
    } else if (opt == "--informat") {
      haveIn = next(informat);
    } else if (opt == "--outformat") {
      haveOut = next(outformat);
    } else if (opt == "--method") {
      std::string m;
      if (next(m)) method = std::atoi(m.c_str());
    }
  }
  if (method == -1) {
    std::fprintf(stderr, "computeThinSVD: Invalid method\n");
    return 1;
  }
  if (dirs.empty() || !haveIn || !haveOut) {
    std::fprintf(stderr, "computeThinSVD: --dirs, --informat and --outformat are required\n");
    return 1;
  }
  std::vector<const char*> d;
  for (const auto& s : dirs) d.push_back(s.c_str());
  const int rc = shaw_pod_tool(d.data(), (uint32_t)d.size(), informat.c_str(), outformat.c_str(), method);
  if (rc != SHAW_OK) {
    std::fprintf(stderr, "computeThinSVD: error %d: %s\n", rc, shaw_last_error());
    return 1;
  }
  return 0;
}
