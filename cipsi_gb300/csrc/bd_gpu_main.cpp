// bd_gpu: executable drop-in for bd.exe.
// Usage (same as the reference, run in the calculation directory):
//     bd_gpu [--json out.json] [--device N] < namelist-input
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/cipsi_gb300.h"

int main(int argc, char** argv) {
  int device = 0;
  const char* json = nullptr;
  for (int a = 1; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--json") && a + 1 < argc) json = argv[++a];
    else if (!std::strcmp(argv[a], "--device") && a + 1 < argc) device = std::atoi(argv[++a]);
    else {
      std::fprintf(stderr, "usage: bd_gpu [--json out.json] [--device N] < input\n");
      return 2;
    }
  }
  char err[1024] = {0};
  const int rc = cipsi_bd_main(".", "/dev/stdin", json, device, err, sizeof err);
  if (rc) {
    std::fprintf(stderr, "bd_gpu: %s\n", err);
    return 1;
  }
  return 0;
}
