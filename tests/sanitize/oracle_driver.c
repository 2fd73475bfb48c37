/* Runs the oracle through setup, time steps, the plot output and the restart stream on
 * one case, for a build with -fsanitize=address,undefined (tests/test_sanitizers.py).
 * Usage: oracle_driver <case dir> <scratch dir> <steps> */
#include <stdio.h>
#include <stdlib.h>

#include "chorus_oracle.h"

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  char err[512];
  orc_t* o = orc_load(argv[1], err, sizeof err);
  if (!o) {
    fprintf(stderr, "load: %s\n", err);
    return 3;
  }
  double r = 0.0, b = 0.0;
  const int steps = atoi(argv[3]);
  for (int i = 0; i < steps; i++) orc_step(o, &r, &b);
  char path[1024];
  if (orc_plot_setup(o, 3) < 0 || orc_plot_eval(o) != 0) return 4;
  snprintf(path, sizeof path, "%s/plot.plt", argv[2]);
  if (orc_plot_write(o, orc_getd(o, "ctime"), path) != 0) return 5;
  snprintf(path, sizeof path, "%s/restart.dat", argv[2]);
  if (orc_write_restart(o, path) != 0 || orc_read_restart(o, path) != 0) return 6;
  orc_compresid(o);
  orc_nablaQsp(o, 1, 9);
  orc_correct_B_via_curl_Az(o);
  printf("ok %d steps residglob %.6e divB %.6e\n", steps, r, b);
  orc_free(o);
  return 0;
}
