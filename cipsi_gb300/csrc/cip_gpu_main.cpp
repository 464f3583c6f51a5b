// cip_gpu: executable drop-in for cip.exe / cipsym.exe.
// Usage (same as the reference, run in the calculation directory):
//     cip_gpu [--sym] [--json out.json] [--device N] < namelist-input
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/cipsi_gb300.h"

int main(int argc, char** argv) {
  int sym = 0, device = 0;
  const char* json = nullptr;
  for (int a = 1; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--sym")) sym = 1;
    else if (!std::strcmp(argv[a], "--json") && a + 1 < argc) json = argv[++a];
    else if (!std::strcmp(argv[a], "--device") && a + 1 < argc) device = std::atoi(argv[++a]);
    else {
      std::fprintf(stderr, "usage: cip_gpu [--sym] [--json out.json] [--device N] < input\n");
      return 2;
    }
  }
  char err[1024] = {0};
  const int rc = cipsi_cip_main(".", "/dev/stdin", sym, json, nullptr, device, err, sizeof err);
  if (rc) {
    std::fprintf(stderr, "cip_gpu: %s\n", err);
    return 1;
  }
  return 0;
}
