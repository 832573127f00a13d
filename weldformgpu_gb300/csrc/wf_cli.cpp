// wf_cli.cpp — command-line driver, the equivalent of the reference's
// WeldFormGPU executable (src/WeldFormGPU.cu:142-926):
//
//   wf <input.json> [output directory]
//
// runs the input file through the library (wf_run_json) and writes the CSV
// snapshots into the output directory (default: the current directory).
#include <cstdio>

#include "../../include/weldform_gb300.h"

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <input.json> [output directory]\n", argv[0]);
    return 2;
  }
  char err[512] = {0};
  const int rc = wf_run_json(argv[1], argc > 2 ? argv[2] : ".", err, sizeof err);
  if (rc != WF_OK) {
    fprintf(stderr, "%s: error %d: %s\n", argv[0], rc, err);
    return 1;
  }
  printf("%s: done (%s)\n", argv[0], wf_version());
  return 0;
}
