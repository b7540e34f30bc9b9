// `tara [file.ini] [output_dir] [max_steps]`: the reference program's command
// line (src/main.f95:15-24: default input.ini) over libtara.
#include <cstdio>
#include <cstdlib>

#include "../../include/tara.h"

int main(int argc, char** argv) {
  const char* ini = argc > 1 ? argv[1] : "input.ini";
  if (argc <= 1) std::printf(" No input file provided. Default input.ini is being used.\n");
  const char* out = argc > 2 ? argv[2] : "output";
  const int max_steps = argc > 3 ? std::atoi(argv[3]) : 0;
  const int rc = tara_run_ini(ini, out, max_steps);
  if (rc) std::fprintf(stderr, "tara: %s\n", tara_last_error_message());
  return rc;
}
