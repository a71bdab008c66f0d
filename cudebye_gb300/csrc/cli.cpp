// cli.cpp — `cudebye <file.deb>`: drop-in for the reference's command line
// `cuDebye.exe <file.deb>` (cuDebye-v15.cu:599-1004, README.md section 3).
// Reads the .deb, uses its device index (line 1, :644), and writes
// <file.deb>x<row>x<col> and/or <file.deb>I next to it, as the reference
// does. Options (all optional):
//   --out <prefix>   write outputs to <prefix>I / <prefix>x<i>x<j>
//   --device <n>     override the .deb's device index
//   --quiet          no progress log
// Further commands, equivalents of the reference's Matlab helpers:
//   cudebye --dir <folder> [--table <file>] [--device n] [--quiet]
//       multisim (Matlab/multisim.m): convert .xyz without .deb, compute
//       every .deb without .debI, batched on one GPU
//   cudebye xyz2deb <file.xyz> --table <file> [--out <file.deb>]
//       [--lambda L] [--tt-min a] [--tt-max b] [--tt-step s] [--rstep r]
//       [--device n] [--block b] [--grid g] [--intensity 0|1]
//       [--distances 0|1]
//       xyz2deb (Matlab/xyz2deb.m), no GPU needed
//   cudebye pack <file.deb> <out>
//       the binary form of a .deb (read by all commands), no GPU needed
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/cudebye.h"

static int usage() {
  fprintf(stderr,
          "usage: cudebye <file.deb> [--out prefix] [--device n] [--quiet]\n"
          "       cudebye --dir <folder> [--table file] [--device n] [--quiet]\n"
          "       cudebye xyz2deb <file.xyz> --table <file> [--out file.deb]\n"
          "               [--lambda L] [--tt-min a] [--tt-max b] [--tt-step s]\n"
          "               [--rstep r] [--device n] [--block b] [--grid g]\n"
          "               [--intensity 0|1] [--distances 0|1]\n"
          "       cudebye pack <file.deb> <out>\n");
  return 2;
}

static int run_xyz2deb(int argc, char **argv) {
  const char *in = nullptr, *table = nullptr, *out = nullptr;
  dbx_xyz2deb_params p;
  dbx_xyz2deb_defaults(&p);
  for (int i = 2; i < argc; ++i) {
    const std::string a = argv[i];
    const bool has = i + 1 < argc;
    if (a == "--table" && has) table = argv[++i];
    else if (a == "--out" && has) out = argv[++i];
    else if (a == "--lambda" && has) p.lambda = atof(argv[++i]);
    else if (a == "--tt-min" && has) p.tt_min = atof(argv[++i]);
    else if (a == "--tt-max" && has) p.tt_max = atof(argv[++i]);
    else if (a == "--tt-step" && has) p.tt_step = atof(argv[++i]);
    else if (a == "--rstep" && has) p.rstep = atof(argv[++i]);
    else if (a == "--device" && has) p.device = atoi(argv[++i]);
    else if (a == "--block" && has) p.block = atoi(argv[++i]);
    else if (a == "--grid" && has) p.grid = atoi(argv[++i]);
    else if (a == "--intensity" && has) p.intensity = atoi(argv[++i]);
    else if (a == "--distances" && has) p.distances = atoi(argv[++i]);
    else if (a.rfind("--", 0) == 0) return usage();
    else in = argv[i];
  }
  if (!in || !table) return usage();
  char msg[512] = {0};
  const int rc = dbx_xyz2deb(in, table, &p, out, msg, sizeof msg);
  if (rc) fprintf(stderr, "ERROR: %s: %s\n", dbx_strerror(rc), msg);
  return rc ? 1 : 0;
}

int main(int argc, char **argv) {
  if (argc >= 2 && !strcmp(argv[1], "xyz2deb")) return run_xyz2deb(argc, argv);
  if (argc >= 2 && !strcmp(argv[1], "pack")) {
    if (argc != 4) return usage();
    char msg[512] = {0};
    const int rc = dbx_deb_pack(argv[2], argv[3], msg, sizeof msg);
    if (rc) fprintf(stderr, "ERROR: %s: %s\n", dbx_strerror(rc), msg);
    return rc ? 1 : 0;
  }
  const char *in = nullptr, *prefix = nullptr, *dir = nullptr, *table = nullptr;
  int device = -1, verbose = 1;
  for (int i = 1; i < argc; ++i) {
    if (!strcmp(argv[i], "--out") && i + 1 < argc)
      prefix = argv[++i];
    else if (!strcmp(argv[i], "--device") && i + 1 < argc)
      device = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--dir") && i + 1 < argc)
      dir = argv[++i];
    else if (!strcmp(argv[i], "--table") && i + 1 < argc)
      table = argv[++i];
    else if (!strcmp(argv[i], "--quiet"))
      verbose = 0;
    else
      in = argv[i];
  }
  if (!in && !dir) return usage();
  if (device < 0 && in) {
    FILE *f = fopen(in, "rb");
    if (!f) {
      printf("\nERROR: >>%s<< does not exist\n", in);  // cuDebye-v15.cu:620
      return 1;
    }
    // line 1 of a text .deb; a binary one holds it after its 8-byte magic
    char magic[8] = {0};
    if (fread(magic, 1, 8, f) == 8 && !memcmp(magic, "DBXDEB1", 8)) {
      int dev = 0;
      device = fread(&dev, sizeof dev, 1, f) == 1 ? dev : 0;
    } else {
      rewind(f);
      if (fscanf(f, "%d", &device) != 1) device = 0;
    }
    fclose(f);
  }
  if (device < 0) device = 0;
  dbx_ctx *ctx = nullptr;
  int rc = dbx_create(&ctx, device, 0);
  if (rc) {
    fprintf(stderr, "ERROR: cannot open CUDA device %d: %s\n", device,
            dbx_strerror(rc));
    return 1;
  }
  rc = dir ? dbx_run_dir(ctx, dir, table, verbose)
           : dbx_run_deb(ctx, in, prefix, verbose);
  if (rc)
    fprintf(stderr, "ERROR: %s: %s\n", dbx_strerror(rc), dbx_last_error(ctx));
  dbx_destroy(ctx);
  return rc ? 1 : 0;
}
