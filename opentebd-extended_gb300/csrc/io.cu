// io.cu -- chain state I/O in the reference's record formats
// (ToolsCore_v_2.0/io_module.f90), so that checkpoints move between a Fortran
// host (or the reference's MPI extension) and this library:
//   tebd_record_lambdas            RecordLambdas  :191-220
//   tebd_record_gammas             RecordGammas   :222-264
//   tebd_record_labels             RecordLabel    :267-287 (LabelLeft and LabelRight)
//   tebd_read_gamma_lambda         readGammaLambda        :289-373
//   tebd_read_gamma_lambda_labels  readGammaLambdaLabels  :376-472
// Record layouts (one record = one text line):
//   Lambdas: L+1 records of chi values;
//   Gammas: for each site, left index i, right index j (j fastest, i next) a record
//           of the d real parts Re Gamma(i,k,j), k = 1..d; then the same sweep
//           for the imaginary parts;
//   labels: L+1 records of chi integers, I16.
// Kind 'S' writes each real as Fortran E30.15 (0.ddd...dE+xx, 15 significant
// digits, right-justified in 30 columns; exponents beyond +-99 as +-xxx without
// the E); kind 'B' as B80, the 64 bits of the IEEE double in binary without
// leading zeros, right-justified in 80 columns (exact).  Host code only.
#include <errno.h>
#include <inttypes.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "tebd_internal.cuh"

using tebd::set_error;

namespace {

// Fortran Ew.d with w = 30, d = 15 and no exponent width given
void put_e30_15(std::string &out, double x) {
  char body[64];
  if (isnan(x)) {
    snprintf(body, sizeof body, "NaN");
  } else if (isinf(x)) {
    snprintf(body, sizeof body, "%s", x < 0 ? "-Infinity" : "Infinity");
  } else if (x == 0.0) {
    snprintf(body, sizeof body, "%s0.000000000000000E+00", signbit(x) ? "-" : "");
  } else {
    char m[64];
    snprintf(m, sizeof m, "%.14E", fabs(x));  // d.dddddddddddddd E+xx, correctly rounded
    const char *ep = strchr(m, 'E');
    const int e10 = atoi(ep + 1) + 1;        // 0.d1d2... x 10^e10
    char digits[16];
    digits[0] = m[0];
    memcpy(digits + 1, m + 2, 14);
    digits[15] = 0;
    char ex[24];
    if (e10 >= -99 && e10 <= 99)
      snprintf(ex, sizeof ex, "E%c%02d", e10 < 0 ? '-' : '+', e10 < 0 ? -e10 : e10);
    else
      snprintf(ex, sizeof ex, "%c%03d", e10 < 0 ? '-' : '+', e10 < 0 ? -e10 : e10);
    snprintf(body, sizeof body, "%s0.%s%s", x < 0 ? "-" : "", digits, ex);
  }
  char field[96];
  snprintf(field, sizeof field, "%30s", body);
  out += field;
}

// B80: the bit pattern of the double in binary, leading zeros dropped
void put_b80(std::string &out, double x) {
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  char bits[65];
  int n = 0;
  bool lead = true;
  for (int b = 63; b >= 0; --b) {
    const int v = (int)((u >> b) & 1u);
    if (lead && v == 0 && b > 0) continue;
    lead = false;
    bits[n++] = (char)('0' + v);
  }
  bits[n] = 0;
  char field[96];
  snprintf(field, sizeof field, "%80s", bits);
  out += field;
}

void put_real(std::string &out, double x, char kind) {
  if (kind == 'S')
    put_e30_15(out, x);
  else
    put_b80(out, x);
}

// one fixed-width field back to a double (E30.15 as written above, also with D or
// without the E before a three-digit exponent; B80 as a bit pattern)
bool get_real(const char *f, int w, char kind, double *x) {
  char buf[128];
  if (w > 120) return false;
  memcpy(buf, f, w);
  buf[w] = 0;
  char *s = buf;
  while (*s == ' ') ++s;
  char *e = s + strlen(s);
  while (e > s && (e[-1] == ' ' || e[-1] == '\r' || e[-1] == '\n')) *--e = 0;
  if (!*s) return false;
  if (kind == 'B') {
    uint64_t u = 0;
    for (char *p = s; *p; ++p) {
      if (*p != '0' && *p != '1') return false;
      u = (u << 1) | (uint64_t)(*p - '0');
    }
    memcpy(x, &u, sizeof u);
    return true;
  }
  std::string t(s);
  for (char &c : t)
    if (c == 'D' || c == 'd') c = 'E';
  if (t.find('E') == std::string::npos && t.find('e') == std::string::npos) {
    // mantissa followed directly by a signed exponent (|exponent| > 99)
    const size_t p = t.find_last_of("+-");
    if (p != std::string::npos && p > 0) t.insert(p, "E");
  }
  errno = 0;
  char *end = nullptr;
  *x = strtod(t.c_str(), &end);
  return end && *end == 0 && errno != ERANGE;
}

struct Reader {
  FILE *f = nullptr;
  std::string line;
  bool next() {
    line.clear();
    int c;
    while ((c = fgetc(f)) != EOF && c != '\n') line.push_back((char)c);
    return !(c == EOF && line.empty());
  }
};

int width(char kind) { return kind == 'S' ? 30 : 80; }

bool kind_ok(char k) { return k == 'S' || k == 'B'; }

FILE *open_out(const char *path, int append) { return fopen(path, append ? "a" : "w"); }

int write_all(tebd_handle *h, FILE *f, const std::string &s, const char *path) {
  const bool ok = fwrite(s.data(), 1, s.size(), f) == s.size();
  const bool closed = fclose(f) == 0;
  if (!ok || !closed) return set_error(h, TEBD_ERR_ARG, std::string("write failed: ") + path);
  return TEBD_OK;
}

int read_lambdas(tebd_handle *h, const char *path, char kind, int chi_now, std::vector<double> &lam) {
  FILE *f = fopen(path, "r");
  if (!f) return set_error(h, TEBD_ERR_ARG, std::string("cannot open ") + path);
  Reader r;
  r.f = f;
  const int w = width(kind);
  for (int link = 0; link < h->L + 1; ++link) {
    if (!r.next() || (int)r.line.size() < w * chi_now) {
      fclose(f);
      return set_error(h, TEBD_ERR_ARG, std::string("short Lambda record in ") + path);
    }
    for (int j = 0; j < chi_now; ++j)
      if (!get_real(r.line.data() + (size_t)w * j, w, kind, &lam[(size_t)link * h->chi + j])) {
        fclose(f);
        return set_error(h, TEBD_ERR_ARG, std::string("bad Lambda field in ") + path);
      }
  }
  fclose(f);
  return TEBD_OK;
}

int read_gammas(tebd_handle *h, const char *path, char kind, int chi_now, std::vector<double> &gam) {
  FILE *f = fopen(path, "r");
  if (!f) return set_error(h, TEBD_ERR_ARG, std::string("cannot open ") + path);
  Reader r;
  r.f = f;
  const int w = width(kind), d = h->d, chi = h->chi;
  const size_t csz = (size_t)chi * d * chi;
  for (int part = 0; part < 2; ++part)  // real parts, then imaginary parts
    for (int l = 0; l < h->L; ++l)
      for (int i = 0; i < chi_now; ++i)
        for (int j = 0; j < chi_now; ++j) {
          if (!r.next() || (int)r.line.size() < w * d) {
            fclose(f);
            return set_error(h, TEBD_ERR_ARG, std::string("short Gamma record in ") + path);
          }
          for (int k = 0; k < d; ++k) {
            double v;
            if (!get_real(r.line.data() + (size_t)w * k, w, kind, &v)) {
              fclose(f);
              return set_error(h, TEBD_ERR_ARG, std::string("bad Gamma field in ") + path);
            }
            gam[2 * (l * csz + i + (size_t)chi * (k + (size_t)d * j)) + part] = v;
          }
        }
  fclose(f);
  return TEBD_OK;
}

int read_labels(tebd_handle *h, const char *path, int chi_now, std::vector<int> &lab) {
  FILE *f = fopen(path, "r");
  if (!f) return set_error(h, TEBD_ERR_ARG, std::string("cannot open ") + path);
  Reader r;
  r.f = f;
  for (int link = 0; link < h->L + 1; ++link) {
    if (!r.next() || (int)r.line.size() < 16 * chi_now) {
      fclose(f);
      return set_error(h, TEBD_ERR_ARG, std::string("short label record in ") + path);
    }
    for (int j = 0; j < chi_now; ++j) {
      char buf[20];
      memcpy(buf, r.line.data() + 16 * j, 16);
      buf[16] = 0;
      char *end = nullptr;
      const long v = strtol(buf, &end, 10);
      while (end && *end == ' ') ++end;
      if (!end || *end != 0) {
        fclose(f);
        return set_error(h, TEBD_ERR_ARG, std::string("bad label field in ") + path);
      }
      lab[(size_t)link * h->chi + j] = (int)v;
    }
  }
  fclose(f);
  return TEBD_OK;
}

// the whole chain <-> host arrays (Gammas interleaved complex, Fortran order)
int get_chain(tebd_handle *h, std::vector<double> &gam, std::vector<double> &lam) {
  const size_t csz = (size_t)h->chi * h->d * h->chi;
  gam.resize(2 * csz * h->L);
  lam.resize((size_t)h->chi * (h->L + 1));
  int rc;
  for (int s = 1; s <= h->L; ++s)
    if ((rc = tebd_get_gamma(h, s, gam.data() + 2 * csz * (s - 1)))) return rc;
  for (int l = 1; l <= h->L + 1; ++l)
    if ((rc = tebd_get_lambda(h, l, lam.data() + (size_t)h->chi * (l - 1)))) return rc;
  return TEBD_OK;
}

int put_chain(tebd_handle *h, const std::vector<double> &gam, const std::vector<double> &lam) {
  const size_t csz = (size_t)h->chi * h->d * h->chi;
  int rc;
  for (int s = 1; s <= h->L; ++s)
    if ((rc = tebd_set_gamma(h, s, gam.data() + 2 * csz * (s - 1)))) return rc;
  for (int l = 1; l <= h->L + 1; ++l)
    if ((rc = tebd_set_lambda(h, l, lam.data() + (size_t)h->chi * (l - 1)))) return rc;
  return TEBD_OK;
}

}  // namespace

extern "C" int tebd_record_lambdas(tebd_handle *h, const char *path, char kind, int append) {
  if (!h || !path) return TEBD_ERR_ARG;
  if (!kind_ok(kind)) return set_error(h, TEBD_ERR_ARG, "tebd_record_lambdas: kind must be 'S' or 'B'");
  std::vector<double> lam((size_t)h->chi * (h->L + 1));
  int rc;
  for (int l = 1; l <= h->L + 1; ++l)
    if ((rc = tebd_get_lambda(h, l, lam.data() + (size_t)h->chi * (l - 1)))) return rc;
  std::string s;
  for (int l = 0; l < h->L + 1; ++l) {
    for (int j = 0; j < h->chi; ++j) put_real(s, lam[(size_t)l * h->chi + j], kind);
    s += '\n';
  }
  FILE *f = open_out(path, append);
  if (!f) return set_error(h, TEBD_ERR_ARG, std::string("cannot open ") + path);
  return write_all(h, f, s, path);
}

extern "C" int tebd_record_gammas(tebd_handle *h, const char *path, char kind, int append) {
  if (!h || !path) return TEBD_ERR_ARG;
  if (!kind_ok(kind)) return set_error(h, TEBD_ERR_ARG, "tebd_record_gammas: kind must be 'S' or 'B'");
  std::vector<double> gam, lam;
  int rc;
  if ((rc = get_chain(h, gam, lam))) return rc;
  const int d = h->d, chi = h->chi;
  const size_t csz = (size_t)chi * d * chi;
  std::string s;
  s.reserve(2 * csz * h->L * (width(kind) + 1));
  for (int part = 0; part < 2; ++part)
    for (int l = 0; l < h->L; ++l)
      for (int i = 0; i < chi; ++i)
        for (int j = 0; j < chi; ++j) {
          for (int k = 0; k < d; ++k) put_real(s, gam[2 * (l * csz + i + (size_t)chi * (k + (size_t)d * j)) + part], kind);
          s += '\n';
        }
  FILE *f = open_out(path, append);
  if (!f) return set_error(h, TEBD_ERR_ARG, std::string("cannot open ") + path);
  return write_all(h, f, s, path);
}

extern "C" int tebd_record_labels(tebd_handle *h, const char *path_left, const char *path_right) {
  if (!h) return TEBD_ERR_ARG;
  if (h->mode != TEBD_MODE_NC) return set_error(h, TEBD_ERR_STATE, "tebd_record_labels: NC mode only");
  const char *paths[2] = {path_left, path_right};
  for (int side = 0; side < 2; ++side) {
    if (!paths[side]) continue;
    std::vector<int> lab((size_t)h->chi * (h->L + 1));
    int rc;
    for (int l = 1; l <= h->L + 1; ++l)
      if ((rc = tebd_get_labels(h, l, side == 0 ? lab.data() + (size_t)h->chi * (l - 1) : nullptr,
                                side == 1 ? lab.data() + (size_t)h->chi * (l - 1) : nullptr)))
        return rc;
    std::string s;
    for (int l = 0; l < h->L + 1; ++l) {
      for (int j = 0; j < h->chi; ++j) {
        char fld[32];
        snprintf(fld, sizeof fld, "%16d", lab[(size_t)l * h->chi + j]);
        s += fld;
      }
      s += '\n';
    }
    FILE *f = open_out(paths[side], 0);
    if (!f) return set_error(h, TEBD_ERR_ARG, std::string("cannot open ") + paths[side]);
    if ((rc = write_all(h, f, s, paths[side]))) return rc;
  }
  return TEBD_OK;
}

extern "C" int tebd_read_gamma_lambda(tebd_handle *h, const char *lambda_path, const char *gamma_path, char kind,
                                      int chi_now) {
  if (!h || !lambda_path || !gamma_path) return TEBD_ERR_ARG;
  if (!kind_ok(kind)) return set_error(h, TEBD_ERR_ARG, "tebd_read_gamma_lambda: kind must be 'S' or 'B'");
  if (chi_now < 1 || chi_now > h->chi)
    return set_error(h, TEBD_ERR_ARG, "tebd_read_gamma_lambda: need 1 <= chi_now <= chi");
  std::vector<double> gam, lam;
  int rc;
  if ((rc = get_chain(h, gam, lam))) return rc;  // entries beyond chi_now stay as they are
  if ((rc = read_lambdas(h, lambda_path, kind, chi_now, lam))) return rc;
  if ((rc = read_gammas(h, gamma_path, kind, chi_now, gam))) return rc;
  return put_chain(h, gam, lam);
}

extern "C" int tebd_read_gamma_lambda_labels(tebd_handle *h, const char *lambda_path, const char *gamma_path,
                                             const char *label_left_path, const char *label_right_path,
                                             char kind, int chi_now) {
  if (!h || !label_left_path || !label_right_path) return TEBD_ERR_ARG;
  if (h->mode != TEBD_MODE_NC) return set_error(h, TEBD_ERR_STATE, "tebd_read_gamma_lambda_labels: NC mode only");
  int rc;
  if ((rc = tebd_read_gamma_lambda(h, lambda_path, gamma_path, kind, chi_now))) return rc;
  std::vector<int> ll((size_t)h->chi * (h->L + 1)), lr(ll.size());
  for (int l = 1; l <= h->L + 1; ++l)
    if ((rc = tebd_get_labels(h, l, ll.data() + (size_t)h->chi * (l - 1), lr.data() + (size_t)h->chi * (l - 1))))
      return rc;
  if ((rc = read_labels(h, label_left_path, chi_now, ll))) return rc;
  if ((rc = read_labels(h, label_right_path, chi_now, lr))) return rc;
  for (int l = 1; l <= h->L + 1; ++l)
    if ((rc = tebd_set_labels(h, l, ll.data() + (size_t)h->chi * (l - 1), lr.data() + (size_t)h->chi * (l - 1))))
      return rc;
  return TEBD_OK;
}
