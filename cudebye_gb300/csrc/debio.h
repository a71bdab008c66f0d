// debio.h — .deb reader and .debI / .debx writers (host C++).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/cudebye.h"

namespace dbx {

struct DebSpecies {
  int64_t n = 0;
  std::string name;
  dbx_species p{};
};

struct DebFile {
  int device = 0, block = 0, grid = 0;           // line 1 (cuDebye-v15.cu:644)
  double lambda = 0, tt_min = 0, tt_max = 0, tt_step = 0;  // line 2 (:689)
  double rmax = 0, rstep = 0;                    // line 3 (:730)
  int hist = 0;                                  // 0/1/2 (:745-754)
  std::vector<DebSpecies> species;               // (:782-804)
  std::vector<float> x, y, z;                    // (:819-827)
};

// Reads a text .deb or its binary form (detected by the "DBXDEB1" magic).
// Returns DBX_OK, DBX_ERR_FILE, DBX_ERR_PARSE or DBX_ERR_COUNT; msg is set
// on error.
int deb_read(const std::string &path, DebFile *out, std::string *msg);
// Writes the binary form of d (debio.cpp documents the layout).
int debb_write(const std::string &path, const DebFile &d);

// Non-zero bins as "%.7g\t%lld\n" of (k*rstep, count) (cuDebye-v15.cu:421-423).
int write_debx(const std::string &path, const int64_t *counts, int64_t nbins,
               double rstep);
// "%.6g\t%.6g\n" of (2theta, I) (cuDebye-v15.cu:995-997).
int write_debI(const std::string &path, const double *two_theta,
               const double *I, int n);

}  // namespace dbx
