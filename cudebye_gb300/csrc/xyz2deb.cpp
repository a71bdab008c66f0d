// xyz2deb.cpp — .xyz -> .deb conversion (host C++), the equivalent of the
// reference's Matlab converter (Matlab/xyz2deb.m:154-263) without its GUI.
//
// Steps, each as the Matlab function does them:
//  * Columns are counted on the first line; the whole file is then read as
//    one token stream in records of that many tokens ("%s" + "%f" ...,
//    :155-172): element, x, y, z [, occupancy [, Beq]]; a missing occupancy
//    is 1 and a missing Beq 0 (:180-186).
//  * Elements are numbered by their place in the sorted list of distinct
//    names (:173-179); rows are sorted stably by (element, occupancy, Beq)
//    (:189) and cut into species where the sum of the three differences to
//    the previous row is non-zero (:190-194) — kept as it is, so two rows
//    whose changes cancel (e.g. element +1, occupancy -1) stay in one
//    species, as with the reference.
//  * Each coordinate column is centred on the middle of its range,
//    x - min - (max - min)/2 (:198-202); rmax = 2 ceil(1.025 max r) with
//    r = hypot(hypot(x, y), z) (:203-204).
//  * Header lines and species lines with the script's fprintf formats
//    (:236-259), coefficients from a Waasmaier-Kirfel table file in the
//    RIETAN layout (element a1..a5 c b1..b5; leading '#' lines and the first
//    line after them skipped; names compared without case, :268-300), then
//    the centred coordinates as "%.7g\t%.7g\t%.7g" lines (dlmwrite
//    precision 7, :262), with the decimal rounding of mfmt_g below.
//  * The output goes to the input path with its last three characters
//    replaced by "deb" (:235).
// An element missing from the table is an error here (the script would
// write a species line without coefficients).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cudebye.h"

namespace {

struct Row {
  double type, x, y, z, occ, beq;
};

struct TableRow {
  std::string name;
  double v[11];  // a1..a5, c, b1..b5
};

bool read_all(const char *path, std::string *out) {
  std::ifstream f(path, std::ios::binary);
  if (!f.good()) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  *out = ss.str();
  return true;
}

bool is_space(char c) {
  return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' ||
         c == '\f';
}

// Whitespace-separated tokens of [b, e).
void tokens(const char *b, const char *e, std::vector<std::string> *out) {
  while (b < e) {
    while (b < e && is_space(*b)) ++b;
    const char *s = b;
    while (b < e && !is_space(*b)) ++b;
    if (b > s) out->emplace_back(s, b);
  }
}

bool to_double(const std::string &t, double *v) {
  char *e = nullptr;
  *v = strtod(t.c_str(), &e);
  return e && *e == '\0' && e != t.c_str();
}

bool same_name(const std::string &a, const std::string &b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i]))
      return false;
  return true;
}

// Decimal formatting as the converter's output shows it: the value is first
// written with 17 significant digits (correctly rounded), and that decimal
// string is rounded half away from zero to the requested digits. A correctly
// rounded printf differs on decimal ties of the 17-digit form: -12.256335
// (the double -12.25633499999999998) prints as -12.25634 in the reference's
// files. Shapes follow printf's %g / %f.
struct Dec {
  bool neg = false;
  char d[18] = {0};  // 17 significant digits, d[0] != '0'
  int exp = 0;       // value = 0.d[0..16] * 10^(exp+1) = d[0].d[1..] * 10^exp
};

Dec decimal17(double v) {
  Dec r;
  char buf[64];
  snprintf(buf, sizeof buf, "%.16e", v);
  const char *p = buf;
  if (*p == '-') {
    r.neg = true;
    ++p;
  }
  int k = 0;
  for (; *p && *p != 'e'; ++p)
    if (*p >= '0' && *p <= '9') r.d[k++] = *p;
  r.exp = atoi(p + 1);
  return r;
}

// Keep `keep` significant digits (1..17), rounding half away from zero.
void round_digits(Dec *r, int keep) {
  if (keep >= 17) return;
  if (keep < 0) keep = 0;
  const bool up = r->d[keep] >= '5';
  for (int i = keep; i < 17; ++i) r->d[i] = '0';
  if (!up) return;
  int i = keep - 1;
  for (; i >= 0; --i) {
    if (r->d[i] == '9') {
      r->d[i] = '0';
    } else {
      ++r->d[i];
      break;
    }
  }
  if (i < 0) {  // 99..9 -> 100..0
    for (int j = 16; j > 0; --j) r->d[j] = r->d[j - 1];
    r->d[0] = '1';
    ++r->exp;
  }
}

std::string fmt_fixed_digits(const Dec &r, int decimals) {
  // digits of the integer part and `decimals` fraction digits
  std::string out = r.neg ? "-" : "";
  std::string ip;
  for (int e = r.exp; e >= 0; --e) {
    const int idx = r.exp - e;
    ip += (idx >= 0 && idx < 17) ? r.d[idx] : '0';
  }
  out += ip.empty() ? "0" : ip;
  if (decimals > 0) {
    out += '.';
    for (int k = 1; k <= decimals; ++k) {
      const int idx = r.exp + k;  // digit of 10^-k
      out += (idx >= 0 && idx < 17) ? r.d[idx] : '0';
    }
  }
  return out;
}

// %.{p}g
std::string mfmt_g(double v, int p) {
  if (v == 0) return std::signbit(v) ? "-0" : "0";
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v < 0 ? "-Inf" : "Inf";
  Dec r = decimal17(v);
  round_digits(&r, p);
  std::string out;
  if (r.exp < -4 || r.exp >= p) {
    int last = p - 1;
    while (last > 0 && r.d[last] == '0') --last;
    out = r.neg ? "-" : "";
    out += r.d[0];
    if (last > 0) {
      out += '.';
      out.append(r.d + 1, r.d + 1 + last);
    }
    char e[16];
    snprintf(e, sizeof e, "e%c%02d", r.exp < 0 ? '-' : '+', std::abs(r.exp));
    return out + e;
  }
  out = fmt_fixed_digits(r, std::max(0, p - 1 - r.exp));
  if (out.find('.') != std::string::npos) {
    while (out.back() == '0') out.pop_back();
    if (out.back() == '.') out.pop_back();
  }
  return out;
}

// %.{decimals}f
std::string mfmt_f(double v, int decimals) {
  if (v == 0) return fmt_fixed_digits(Dec{std::signbit(v), "00000000000000000", 0},
                                      decimals);
  if (!std::isfinite(v)) return mfmt_g(v, 1);
  Dec r = decimal17(v);
  round_digits(&r, r.exp + 1 + decimals);
  return fmt_fixed_digits(r, decimals);
}

int fail(char *msg, size_t len, int code, const std::string &m) {
  if (msg && len) snprintf(msg, len, "%s", m.c_str());
  return code;
}

int read_table(const char *path, std::vector<TableRow> *rows, std::string *err) {
  std::string txt;
  if (!read_all(path, &txt)) {
    *err = std::string("cannot read scattering-factor table ") + path;
    return DBX_ERR_FILE;
  }
  // skip the leading '#' lines and the first line after them (the column
  // header)
  size_t pos = 0;
  for (;;) {
    size_t eol = txt.find('\n', pos);
    if (eol == std::string::npos) eol = txt.size();
    size_t s = pos;
    while (s < eol && is_space(txt[s])) ++s;
    const bool comment = s < eol && txt[s] == '#';
    pos = eol < txt.size() ? eol + 1 : eol;
    if (!comment || pos >= txt.size()) break;
  }
  std::vector<std::string> tok;
  tokens(txt.data() + pos, txt.data() + txt.size(), &tok);
  for (size_t i = 0; i + 12 <= tok.size(); i += 12) {
    TableRow r;
    r.name = tok[i];
    for (int k = 0; k < 11; ++k)
      if (!to_double(tok[i + 1 + k], &r.v[k])) {
        *err = "malformed scattering-factor table row for " + r.name;
        return DBX_ERR_PARSE;
      }
    rows->push_back(r);
  }
  return DBX_OK;
}

}  // namespace

extern "C" {

void dbx_xyz2deb_defaults(dbx_xyz2deb_params *p) {
  if (!p) return;
  // the script's defaults (Matlab/xyz2deb.m:13-25)
  p->device = 0;
  p->block = 16;
  p->grid = 2048;
  p->lambda = 1.5418;
  p->tt_min = 10;
  p->tt_max = 140;
  p->tt_step = 0.02;
  p->rstep = 0.0001;
  p->intensity = 1;
  p->distances = 0;
}

int dbx_xyz2deb(const char *xyz_path, const char *table_path,
                const dbx_xyz2deb_params *prm, const char *deb_path,
                char *msg, size_t msg_len) {
  if (!xyz_path || !table_path)
    return fail(msg, msg_len, DBX_ERR_ARG, "need the .xyz and table paths");
  dbx_xyz2deb_params p;
  if (prm)
    p = *prm;
  else
    dbx_xyz2deb_defaults(&p);
  std::string txt;
  if (!read_all(xyz_path, &txt))
    return fail(msg, msg_len, DBX_ERR_FILE,
                std::string(">>") + xyz_path + "<< does not exist");
  // columns of the first line
  size_t eol = txt.find('\n');
  if (eol == std::string::npos) eol = txt.size();
  std::vector<std::string> first;
  tokens(txt.data(), txt.data() + eol, &first);
  const int cols = (int)first.size();
  if (cols < 4 || cols > 6)
    return fail(msg, msg_len, DBX_ERR_PARSE,
                "an .xyz line needs 4 to 6 columns (element x y z [occ [Beq]])");
  std::vector<std::string> tok;
  tokens(txt.data(), txt.data() + txt.size(), &tok);
  if (tok.size() % cols != 0)
    return fail(msg, msg_len, DBX_ERR_PARSE, "ragged .xyz records");
  const size_t n = tok.size() / cols;
  if (n == 0) return fail(msg, msg_len, DBX_ERR_PARSE, "no atoms in the .xyz");
  std::vector<std::string> names(n);
  std::vector<Row> rows(n);
  for (size_t i = 0; i < n; ++i) {
    const std::string *t = &tok[i * cols];
    names[i] = t[0];
    double v[5] = {0, 0, 0, 1, 0};
    for (int c = 1; c < cols; ++c)
      if (!to_double(t[c], &v[c - 1]))
        return fail(msg, msg_len, DBX_ERR_PARSE,
                    "malformed number in .xyz record " + std::to_string(i + 1));
    rows[i] = Row{0, v[0], v[1], v[2], v[3], v[4]};
  }
  std::vector<std::string> uniq = names;
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  for (size_t i = 0; i < n; ++i)
    rows[i].type = (double)(std::lower_bound(uniq.begin(), uniq.end(), names[i]) -
                            uniq.begin() + 1);
  std::stable_sort(rows.begin(), rows.end(), [](const Row &a, const Row &b) {
    if (a.type != b.type) return a.type < b.type;
    if (a.occ != b.occ) return a.occ < b.occ;
    return a.beq < b.beq;
  });
  std::vector<size_t> start(1, 0);
  for (size_t i = 1; i < n; ++i) {
    const double d = (rows[i].type - rows[i - 1].type) +
                     (rows[i].occ - rows[i - 1].occ) +
                     (rows[i].beq - rows[i - 1].beq);
    if (d != 0) start.push_back(i);
  }
  start.push_back(n);
  double *col[3];
  std::vector<double> xs(n), ys(n), zs(n);
  for (size_t i = 0; i < n; ++i) {
    xs[i] = rows[i].x;
    ys[i] = rows[i].y;
    zs[i] = rows[i].z;
  }
  col[0] = xs.data();
  col[1] = ys.data();
  col[2] = zs.data();
  for (int c = 0; c < 3; ++c) {
    const double mx = *std::max_element(col[c], col[c] + n);
    const double mn = *std::min_element(col[c], col[c] + n);
    for (size_t i = 0; i < n; ++i) col[c][i] = col[c][i] - mn - (mx - mn) / 2;
  }
  double rmax_r = 0;
  for (size_t i = 0; i < n; ++i)
    rmax_r = std::max(rmax_r, std::hypot(std::hypot(xs[i], ys[i]), zs[i]));
  const double rmax = 2 * std::ceil(rmax_r * 1.025);
  std::vector<TableRow> table;
  std::string err;
  int rc = read_table(table_path, &table, &err);
  if (rc) return fail(msg, msg_len, rc, err);
  const int output = p.distances ? (p.intensity ? 2 : 1) : 0;
  std::string out = deb_path ? deb_path : "";
  if (out.empty()) {
    out = xyz_path;
    out = out.substr(0, out.size() >= 3 ? out.size() - 3 : 0) + "deb";
  }
  FILE *f = fopen(out.c_str(), "wb");
  if (!f) return fail(msg, msg_len, DBX_ERR_IO, "cannot write " + out);
  std::vector<char> buf(1 << 20);
  setvbuf(f, buf.data(), _IOFBF, buf.size());
  fprintf(f, "%s %s %s", mfmt_f(p.device, 0).c_str(),
          mfmt_f(p.block, 0).c_str(), mfmt_f(p.grid, 0).c_str());
  fprintf(f, "\n%s %s %s %s", mfmt_f(p.lambda, 6).c_str(),
          mfmt_f(p.tt_min, 2).c_str(), mfmt_f(p.tt_max, 2).c_str(),
          mfmt_f(p.tt_step, 2).c_str());
  fprintf(f, "\n%s %s %s", mfmt_f(rmax, 0).c_str(), mfmt_f(p.rstep, 4).c_str(),
          mfmt_f(output, 0).c_str());
  fprintf(f, "\n%s", mfmt_f((double)(start.size() - 1), 0).c_str());
  for (size_t s = 0; s + 1 < start.size(); ++s) {
    const Row &r0 = rows[start[s]];
    const std::string &el = uniq[(size_t)r0.type - 1];
    const TableRow *tr = nullptr;
    for (const TableRow &t : table)
      if (same_name(t.name, el)) {
        tr = &t;
        break;
      }
    if (!tr) {
      fclose(f);
      remove(out.c_str());
      return fail(msg, msg_len, DBX_ERR_PARSE,
                  "element " + el + " is not in the scattering-factor table");
    }
    fprintf(f, "\n%s %s %s %s", mfmt_f((double)(start[s + 1] - start[s]), 0).c_str(),
            el.c_str(), mfmt_f(r0.occ, 4).c_str(), mfmt_f(r0.beq, 4).c_str());
    for (int k = 0; k < 5; ++k) fprintf(f, " %s", mfmt_f(tr->v[k], 6).c_str());  // a
    for (int k = 0; k < 5; ++k)
      fprintf(f, " %s", mfmt_f(tr->v[6 + k], 6).c_str());  // b
    fprintf(f, " %s", mfmt_f(tr->v[5], 6).c_str());           // c
  }
  fprintf(f, "\n");
  for (size_t i = 0; i < n; ++i)
    fprintf(f, "%s\t%s\t%s\n", mfmt_g(xs[i], 7).c_str(), mfmt_g(ys[i], 7).c_str(),
            mfmt_g(zs[i], 7).c_str());
  const bool bad = fflush(f) != 0;
  if (fclose(f) != 0 || bad)
    return fail(msg, msg_len, DBX_ERR_IO, "cannot write " + out);
  return DBX_OK;
}

}  // extern "C"
