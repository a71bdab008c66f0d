// cli.cpp — `cudebye <file.deb>`: drop-in for the reference's command line
// `cuDebye.exe <file.deb>` (cuDebye-v15.cu:599-1004, README.md section 3).
// Reads the .deb, uses its device index (line 1, :644), and writes
// <file.deb>x<row>x<col> and/or <file.deb>I next to it, as the reference
// does. Options (all optional):
//   --out <prefix>   write outputs to <prefix>I / <prefix>x<i>x<j>
//   --device <n>     override the .deb's device index
//   --quiet          no progress log
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/cudebye.h"

int main(int argc, char **argv) {
  const char *in = nullptr, *prefix = nullptr;
  int device = -1, verbose = 1;
  for (int i = 1; i < argc; ++i) {
    if (!strcmp(argv[i], "--out") && i + 1 < argc)
      prefix = argv[++i];
    else if (!strcmp(argv[i], "--device") && i + 1 < argc)
      device = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--quiet"))
      verbose = 0;
    else
      in = argv[i];
  }
  if (!in) {
    fprintf(stderr, "usage: cudebye <file.deb> [--out prefix] [--device n] "
                    "[--quiet]\n");
    return 2;
  }
  if (device < 0) {
    FILE *f = fopen(in, "rb");
    if (!f) {
      printf("\nERROR: >>%s<< does not exist\n", in);  // cuDebye-v15.cu:620
      return 1;
    }
    if (fscanf(f, "%d", &device) != 1) device = 0;
    fclose(f);
  }
  dbx_ctx *ctx = nullptr;
  int rc = dbx_create(&ctx, device, 0);
  if (rc) {
    fprintf(stderr, "ERROR: cannot open CUDA device %d: %s\n", device,
            dbx_strerror(rc));
    return 1;
  }
  rc = dbx_run_deb(ctx, in, prefix, verbose);
  if (rc)
    fprintf(stderr, "ERROR: %s: %s\n", dbx_strerror(rc), dbx_last_error(ctx));
  dbx_destroy(ctx);
  return rc ? 1 : 0;
}
