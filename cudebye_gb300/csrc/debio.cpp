// debio.cpp — .deb reader and .debI / .debx writers (host C++).
//
// Input format (cuDebye-v15.cu:629-833, README.md section 2): four header
// lines, one line per species, then "x y z" per atom in species order.
// Header fields are parsed as istringstream >> int/double would; the
// coordinates with from_chars / strtof, i.e. correctly rounded to FP32 like
// >> float. The file is read in one piece and scanned in place. A binary
// form of the same content (the reference's wish list, cuDebye-v15.cu:7) is
// read as well.
// A line holding only whitespace (a CR of a CRLF file included) counts as
// empty and is skipped, as in the reference's Windows text-mode build
// (:821). A coordinate line that does not start with three numbers is an
// error here; the reference would silently read zeros.
//
// Outputs are written with "\n" line ends, which is what the reference's
// ostream code writes on a POSIX host; the shipped Windows files differ
// only by CRLF.
#include "debio.h"

#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>

namespace dbx {

// ---- binary .deb ("DBXDEB1"), little-endian -----------------------------
// magic[8]; int32 device, block, grid, hist; float64 lambda, tt_min,
// tt_max, tt_step, rmax, rstep; int32 nspecies, int32 0; per species int64 n,
// char name[32], float64 occ, beq, a[5], b[5], c; then float32 x[N], y[N],
// z[N] (N = sum of n). The text header's meaning field by field; the
// coordinates are the FP32 values the text parser would produce.
const char kDebbMagic[8] = {'D', 'B', 'X', 'D', 'E', 'B', '1', '\0'};

namespace {
template <typename T>
void put(std::string *b, const T &v) {
  b->append(reinterpret_cast<const char *>(&v), sizeof(T));
}
template <typename T>
bool get(const std::string &b, size_t *pos, T *v) {
  if (*pos + sizeof(T) > b.size()) return false;
  memcpy(v, b.data() + *pos, sizeof(T));
  *pos += sizeof(T);
  return true;
}
}  // namespace

static int debb_parse(const std::string &buf, DebFile *d, std::string *msg) {
  size_t pos = 8;
  int32_t dev, blk, grd, hist, nsp, zero;
  bool good = get(buf, &pos, &dev) && get(buf, &pos, &blk) &&
              get(buf, &pos, &grd) && get(buf, &pos, &hist) &&
              get(buf, &pos, &d->lambda) && get(buf, &pos, &d->tt_min) &&
              get(buf, &pos, &d->tt_max) && get(buf, &pos, &d->tt_step) &&
              get(buf, &pos, &d->rmax) && get(buf, &pos, &d->rstep) &&
              get(buf, &pos, &nsp) && get(buf, &pos, &zero);
  if (!good || nsp < 1 || nsp > (1 << 20) || !(d->rstep > 0) ||
      !(d->tt_step > 0)) {
    *msg = "malformed binary .deb header";
    return DBX_ERR_PARSE;
  }
  d->device = dev;
  d->block = blk;
  d->grid = grd;
  d->hist = (hist == 1 || hist == 2) ? hist : 0;
  d->species.resize(nsp);
  int64_t total = 0;
  for (int i = 0; i < nsp; ++i) {
    DebSpecies &s = d->species[i];
    char name[32];
    good = get(buf, &pos, &s.n) && pos + 32 <= buf.size();
    if (good) {
      memcpy(name, buf.data() + pos, 32);
      pos += 32;
      name[31] = 0;
      s.name = name;
      good = get(buf, &pos, &s.p.occ) && get(buf, &pos, &s.p.beq);
      for (int k = 0; good && k < 5; ++k) good = get(buf, &pos, &s.p.a[k]);
      for (int k = 0; good && k < 5; ++k) good = get(buf, &pos, &s.p.b[k]);
      good = good && get(buf, &pos, &s.p.c);
    }
    if (!good || s.n < 0 || s.n > (int64_t(1) << 40)) {
      *msg = "malformed binary .deb species " + std::to_string(i);
      return DBX_ERR_PARSE;
    }
    total += s.n;
  }
  const size_t bytes = sizeof(float) * (size_t)total;
  if (pos + 3 * bytes != buf.size()) {
    *msg = "binary .deb holds " + std::to_string((buf.size() - pos) / 12) +
           " atoms, the species say " + std::to_string(total);
    return DBX_ERR_COUNT;
  }
  d->x.resize(total);
  d->y.resize(total);
  d->z.resize(total);
  if (total) {
    memcpy(d->x.data(), buf.data() + pos, bytes);
    memcpy(d->y.data(), buf.data() + pos + bytes, bytes);
    memcpy(d->z.data(), buf.data() + pos + 2 * bytes, bytes);
  }
  return DBX_OK;
}

int debb_write(const std::string &path, const DebFile &d) {
  std::string b(kDebbMagic, 8);
  put(&b, (int32_t)d.device);
  put(&b, (int32_t)d.block);
  put(&b, (int32_t)d.grid);
  put(&b, (int32_t)d.hist);
  for (double v : {d.lambda, d.tt_min, d.tt_max, d.tt_step, d.rmax, d.rstep})
    put(&b, v);
  put(&b, (int32_t)d.species.size());
  put(&b, (int32_t)0);
  for (const DebSpecies &s : d.species) {
    put(&b, (int64_t)s.n);
    char name[32] = {0};
    snprintf(name, sizeof name, "%s", s.name.c_str());
    b.append(name, 32);
    put(&b, s.p.occ);
    put(&b, s.p.beq);
    for (double v : s.p.a) put(&b, v);
    for (double v : s.p.b) put(&b, v);
    put(&b, s.p.c);
  }
  for (const std::vector<float> *v : {&d.x, &d.y, &d.z})
    b.append(reinterpret_cast<const char *>(v->data()), sizeof(float) * v->size());
  std::unique_ptr<FILE, int (*)(FILE *)> f(fopen(path.c_str(), "wb"), fclose);
  if (!f || fwrite(b.data(), 1, b.size(), f.get()) != b.size()) return DBX_ERR_IO;
  return fclose(f.release()) ? DBX_ERR_IO : DBX_OK;
}

// One FP32 number at p (leading blanks skipped): from_chars, which rounds
// correctly like strtof, with strtof for what it does not take (a '+'
// sign, "inf", ...). Returns the end, or nullptr if there is no number.
static const char *parse_f32(const char *p, const char *end, float *v) {
  while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' ||
                     *p == '\f'))
    ++p;
  auto r = std::from_chars(p, end, *v);
  if (r.ec == std::errc() && r.ptr != p) return r.ptr;
  // strtof needs a terminated string: copy the token
  char tok[64];
  size_t n = 0;
  while (p + n < end && n < sizeof tok - 1 && p[n] != ' ' && p[n] != '\t' &&
         p[n] != '\r' && p[n] != '\n')
    ++n;
  memcpy(tok, p, n);
  tok[n] = 0;
  char *e = nullptr;
  *v = strtof(tok, &e);
  if (e == tok) return nullptr;
  return p + (e - tok);
}

static bool read_file(const std::string &path, std::string *out) {
  std::unique_ptr<FILE, int (*)(FILE *)> f(fopen(path.c_str(), "rb"), fclose);
  if (!f) return false;
  if (fseek(f.get(), 0, SEEK_END) != 0) return false;
  const long n = ftell(f.get());
  if (n < 0 || fseek(f.get(), 0, SEEK_SET) != 0) return false;
  out->resize((size_t)n);
  return n == 0 || fread(&(*out)[0], 1, (size_t)n, f.get()) == (size_t)n;
}

// Next line of [*pos, end) without its '\n'; false at the end.
static bool next_line(const std::string &buf, size_t *pos, const char **b,
                      const char **e) {
  if (*pos >= buf.size()) return false;
  const char *s = buf.data() + *pos;
  const char *end = buf.data() + buf.size();
  const char *nl = static_cast<const char *>(memchr(s, '\n', end - s));
  *b = s;
  *e = nl ? nl : end;
  *pos = (size_t)((nl ? nl + 1 : end) - buf.data());
  return true;
}

static int deb_read_text(const std::string &buf, DebFile *d, std::string *msg) {
  size_t pos = 0;
  const char *b, *e;
  std::string l[4];
  for (int i = 0; i < 4; ++i) {
    if (!next_line(buf, &pos, &b, &e)) {
      *msg = "truncated .deb header";
      return DBX_ERR_PARSE;
    }
    l[i].assign(b, e);
  }
  int nsp = 0;
  if (sscanf(l[0].c_str(), "%d %d %d", &d->device, &d->block, &d->grid) != 3 ||
      sscanf(l[1].c_str(), "%lf %lf %lf %lf", &d->lambda, &d->tt_min,
             &d->tt_max, &d->tt_step) != 4 ||
      sscanf(l[2].c_str(), "%lf %lf %d", &d->rmax, &d->rstep, &d->hist) != 3 ||
      sscanf(l[3].c_str(), "%d", &nsp) != 1 || nsp < 1) {
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
    char name[64] = {0};
    long long n = 0;
    dbx_species &s = d->species[i].p;
    std::string line;
    if (next_line(buf, &pos, &b, &e)) line.assign(b, e);
    if (line.empty() ||
        sscanf(line.c_str(),
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
  while (next_line(buf, &pos, &b, &e)) {
    ++lineno;
    const char *q = b;
    while (q < e && (*q == ' ' || *q == '\t' || *q == '\r' || *q == '\v' ||
                     *q == '\f'))
      ++q;
    if (q == e) continue;  // blank line
    if (i < total) {
      float v[3];
      const char *p = b;
      for (int c = 0; c < 3; ++c) {
        p = p ? parse_f32(p, e, &v[c]) : nullptr;
        if (!p) {
          *msg = "malformed coordinate line " + std::to_string(lineno);
          return DBX_ERR_PARSE;
        }
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

int deb_read(const std::string &path, DebFile *d, std::string *msg) {
  std::string buf;
  if (!read_file(path, &buf)) {
    *msg = ">>" + path + "<< does not exist";  // cuDebye-v15.cu:620
    return DBX_ERR_FILE;
  }
  if (buf.size() >= 8 && memcmp(buf.data(), kDebbMagic, 8) == 0)
    return debb_parse(buf, d, msg);
  return deb_read_text(buf, d, msg);
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

extern "C" int dbx_deb_pack(const char *deb_path, const char *out_path,
                            char *msg, size_t msg_len) {
  if (!deb_path || !out_path) return DBX_ERR_ARG;
  dbx::DebFile d;
  std::string m;
  int rc = dbx::deb_read(deb_path, &d, &m);
  if (rc == DBX_OK) {
    rc = dbx::debb_write(out_path, d);
    if (rc) m = std::string("cannot write ") + out_path;
  }
  if (rc && msg && msg_len) snprintf(msg, msg_len, "%s", m.c_str());
  return rc;
}
