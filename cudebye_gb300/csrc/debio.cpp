// debio.cpp — .deb reader and .debI / .debx writers (host C++).
//
// Input format (cuDebye-v15.cu:629-833, README.md section 2): four header
// lines, one line per species, then "x y z" per atom in species order.
// Header fields are parsed as istringstream >> int/double would; the
// coordinates with strtof, i.e. correctly rounded to FP32 like >> float.
// A line holding only whitespace (a CR of a CRLF file included) counts as
// empty and is skipped, as in the reference's Windows text-mode build
// (:821). A coordinate line that does not start with three numbers is an
// error here; the reference would silently read zeros.
//
// Outputs are written with "\n" line ends, which is what the reference's
// ostream code writes on a POSIX host; the shipped Windows files differ
// only by CRLF.
#include "debio.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>

namespace dbx {

static bool blank(const std::string &l) {
  for (char c : l)
    if (c != ' ' && c != '\t' && c != '\r' && c != '\v' && c != '\f')
      return false;
  return true;
}

int deb_read(const std::string &path, DebFile *d, std::string *msg) {
  std::ifstream f(path, std::ios::binary);
  if (!f.good()) {
    *msg = ">>" + path + "<< does not exist";  // cuDebye-v15.cu:620
    return DBX_ERR_FILE;
  }
  std::string l1, l2, l3, l4;
  if (!std::getline(f, l1) || !std::getline(f, l2) || !std::getline(f, l3) ||
      !std::getline(f, l4)) {
    *msg = "truncated .deb header";
    return DBX_ERR_PARSE;
  }
  int nsp = 0;
  if (sscanf(l1.c_str(), "%d %d %d", &d->device, &d->block, &d->grid) != 3 ||
      sscanf(l2.c_str(), "%lf %lf %lf %lf", &d->lambda, &d->tt_min,
             &d->tt_max, &d->tt_step) != 4 ||
      sscanf(l3.c_str(), "%lf %lf %d", &d->rmax, &d->rstep, &d->hist) != 3 ||
      sscanf(l4.c_str(), "%d", &nsp) != 1 || nsp < 1) {
    *msg = "malformed .deb header (lines 1-4)";
    return DBX_ERR_PARSE;
  }
  if (d->hist != 1 && d->hist != 2) d->hist = 0;  // cuDebye-v15.cu:751-753
  if (!(d->rstep > 0) || !(d->tt_step > 0)) {
    *msg = "rstep and the 2theta step must be positive";
    return DBX_ERR_PARSE;
  }
  d->species.resize(nsp);
  int64_t total = 0;
  for (int i = 0; i < nsp; ++i) {
    std::string l;
    char name[64] = {0};
    long long n = 0;
    dbx_species &s = d->species[i].p;
    if (!std::getline(f, l) ||
        sscanf(l.c_str(),
               "%lld %63s %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf",
               &n, name, &s.occ, &s.beq, &s.a[0], &s.a[1], &s.a[2], &s.a[3],
               &s.a[4], &s.b[0], &s.b[1], &s.b[2], &s.b[3], &s.b[4],
               &s.c) != 15 ||
        n < 0) {
      *msg = "malformed species line " + std::to_string(i + 5);
      return DBX_ERR_PARSE;
    }
    d->species[i].n = n;
    d->species[i].name = name;
    total += n;
  }
  d->x.resize(total);
  d->y.resize(total);
  d->z.resize(total);
  int64_t i = 0, lineno = 4 + nsp;
  std::string l;
  while (std::getline(f, l)) {
    ++lineno;
    if (blank(l)) continue;
    if (i < total) {
      const char *p = l.c_str();
      char *e;
      float v[3];
      for (int c = 0; c < 3; ++c) {
        v[c] = strtof(p, &e);
        if (e == p) {
          *msg = "malformed coordinate line " + std::to_string(lineno);
          return DBX_ERR_PARSE;
        }
        p = e;
      }
      d->x[i] = v[0];
      d->y[i] = v[1];
      d->z[i] = v[2];
    }
    ++i;
  }
  if (i != total) {  // cuDebye-v15.cu:830-833
    *msg = "Number of extracted Atoms (" + std::to_string(i) +
           ") doesn't match the number specified in the preamble (" +
           std::to_string(total) + ")";
    return DBX_ERR_COUNT;
  }
  return DBX_OK;
}

namespace {
struct FileCloser {
  void operator()(FILE *f) const {
    if (f) fclose(f);
  }
};
}  // namespace

int write_debx(const std::string &path, const int64_t *counts, int64_t nbins,
               double rstep) {
  std::unique_ptr<FILE, FileCloser> f(fopen(path.c_str(), "wb"));
  if (!f) return DBX_ERR_IO;
  std::vector<char> buf(1 << 20);
  setvbuf(f.get(), buf.data(), _IOFBF, buf.size());
  for (int64_t k = 0; k < nbins; ++k)
    if (counts[k] != 0)
      fprintf(f.get(), "%.7g\t%lld\n", (double)k * rstep, (long long)counts[k]);
  if (fflush(f.get())) return DBX_ERR_IO;
  return fclose(f.release()) ? DBX_ERR_IO : DBX_OK;
}

int write_debI(const std::string &path, const double *two_theta,
               const double *I, int n) {
  std::unique_ptr<FILE, FileCloser> f(fopen(path.c_str(), "wb"));
  if (!f) return DBX_ERR_IO;
  for (int i = 0; i < n; ++i)
    fprintf(f.get(), "%.6g\t%.6g\n", two_theta[i], I[i]);
  if (fflush(f.get())) return DBX_ERR_IO;
  return fclose(f.release()) ? DBX_ERR_IO : DBX_OK;
}

}  // namespace dbx
