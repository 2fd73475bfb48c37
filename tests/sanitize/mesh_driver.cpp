// Runs the product's host setup (input deck, mesh files, connectivity, periodic pairing,
// operators, metrics) on one case, for a build with -fsanitize=address,undefined
// (tests/test_sanitizers.py).  Usage: mesh_driver <case dir>
#include <cstdio>
#include <string>

#include "chorus_internal.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  chorus::Mesh m;
  std::string err;
  const int rc = chorus::mesh_load(argv[1], m, err);
  if (rc) {
    std::fprintf(stderr, "mesh_load: %s\n", err.c_str());
    return 3;
  }
  std::printf("ok NCELL %d NFACE %d NPAIR %d\n", m.NCELL, m.NFACE, m.NPAIR);
  return 0;
}
