// input.ini reader: cfgio semantics (lib/iniparser/cfgio_mod.f90) and Fortran
// list-directed number reads.  Host code only.
#include "ini.h"

#include <algorithm>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <new>
#include <stdexcept>
#include <thread>

#include "../../include/tara.h"
#include "status.h"

namespace tara {

namespace {

const char* kDefaults = "DEFAULTS";  // cfgio_mod.f90:17
const size_t kLine = 512;            // character(len=512):: text (parse_cfg)
const size_t kMxn = 256;             // MXNSTR (cfgio_mod.f90:13)

std::string adjustl(const std::string& s) {
  size_t i = 0;
  while (i < s.size() && s[i] == ' ') ++i;
  return s.substr(i);
}

std::string trim(const std::string& s) {
  size_t n = s.size();
  while (n > 0 && (s[n - 1] == ' ' || s[n - 1] == '\r' || s[n - 1] == '\n')) --n;
  return s.substr(0, n);
}

// Fortran CHARACTER comparison: trailing blanks do not matter.
bool feq(const std::string& a, const std::string& b) { return trim(a) == trim(b); }

int find_section(const IniFile& ini, const std::string& name) {
  for (size_t i = 0; i < ini.sections.size(); ++i)
    if (feq(adjustl(ini.sections[i].name), name)) return (int)i;  // find_isect (:139-152)
  return -1;
}

int find_key(const IniSection& s, const std::string& key) {
  for (size_t i = 0; i < s.pars.size(); ++i)
    if (feq(s.pars[i].first, key)) return (int)i;  // find_ikey (:167-179), first match wins
  return -1;
}

// parse_text (cfgio_mod.f90:781-815)
bool parse_line(IniFile& ini, std::string text, int& isect, std::string& err) {
  if (text.size() > kLine) text.resize(kLine);
  // tabs are ordinary characters to Fortran; only blanks are adjusted
  std::string str = adjustl(text);
  if (str.size() > kMxn) str.resize(kMxn);
  const char c1 = str.empty() ? ' ' : str[0];
  if (c1 == '#' || c1 == ';') return true;
  if (c1 == '[') {
    const size_t id = str.find(']');
    if (id == std::string::npos) {
      err = "Wrong section title";
      return false;
    }
    const std::string section = trim(adjustl(str.substr(1, id - 1)));
    const int found = find_section(ini, section);
    if (found >= 0) {
      isect = found;
    } else {
      ini.sections.push_back(IniSection{section, {}});
      isect = (int)ini.sections.size() - 1;
    }
    return true;
  }
  const size_t id = str.find('=');
  if (id == std::string::npos) return true;
  std::string key = trim(adjustl(str.substr(0, id)));   // split_kv (:874-881)
  std::string val = trim(adjustl(str.substr(id + 1)));
  if (key.size() > kMxn) key.resize(kMxn);
  if (val.size() > kMxn) val.resize(kMxn);
  ini.sections[isect].pars.emplace_back(key, val);
  return true;
}

std::string unquote(const std::string& s) {  // string_conv_mod unquote
  if (!s.empty() && (s[0] == '"' || s[0] == '\'')) {
    const size_t l = trim(s).size();
    return l >= 2 ? s.substr(1, l - 2) : std::string();
  }
  return s;
}

// cfg_gets_basic (cfgio_mod.f90:399-424)
bool get_basic(const IniFile& ini, const std::string& section, const std::string& key,
               std::string& val, std::string& err) {
  int isect = find_section(ini, section);
  if (isect < 0) {
    isect = find_section(ini, kDefaults);
    if (isect < 0) {
      err = "Cannot find the section:" + section;
      return false;
    }
  }
  int ikey = find_key(ini.sections[isect], key);
  if (ikey < 0) {
    isect = find_section(ini, kDefaults);
    if (isect < 0 || (ikey = find_key(ini.sections[isect], key)) < 0) {
      err = "Cannot find the key:" + key;
      return false;
    }
  }
  val = unquote(ini.sections[isect].pars[ikey].second);
  return true;
}

bool is_sep(char c) { return c == ' ' || c == '\t' || c == ',' || c == '/' || c == '\0'; }

// Skip blanks and an optional repeat count "r*"; returns false on a null value.
bool lead_in(const std::string& s, size_t& i, std::string& err) {
  while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
  size_t j = i;
  while (j < s.size() && std::isdigit((unsigned char)s[j])) ++j;
  if (j > i && j < s.size() && s[j] == '*') i = j + 1;
  if (i >= s.size() || s[i] == ',' || s[i] == '/' || s[i] == ' ' || s[i] == '\t') {
    err = "null value in list-directed read";
    return false;
  }
  return true;
}

}  // namespace

bool ini_parse_text(const std::string& text, IniFile& ini, std::string& err) {
  ini.sections.clear();
  ini.sections.push_back(IniSection{kDefaults, {}});  // cfg_init
  int isect = 0;
  std::istringstream in(text);
  std::string line;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (!parse_line(ini, line, isect, err)) return false;
  }
  return true;
}

bool ini_parse_file(const std::string& path, IniFile& ini, std::string& err) {
  std::ifstream f(path);
  if (!f) {
    err = "cannot open " + path;
    return false;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  return ini_parse_text(ss.str(), ini, err);
}

// cfg_gets = cfg_gets_basic + interpolate_str (cfgio_mod.f90:426-470)
bool ini_get(const IniFile& ini, const std::string& section, const std::string& key,
             std::string& val, std::string& err) {
  if (!get_basic(ini, section, key, val, err)) return false;
  for (int guard = 0; guard < 64; ++guard) {
    const size_t a = val.find("${");
    if (a == std::string::npos) return true;
    const size_t b = val.find('}', a + 2);
    if (b == std::string::npos) return true;
    std::string ref = val.substr(a + 2, b - a - 2), sec = section, k = ref;
    const size_t c = trim(ref).find(':');
    if (c != std::string::npos) {
      sec = ref.substr(0, c);
      k = trim(ref.substr(c + 1));
    }
    std::string sub;
    if (!get_basic(ini, sec, k, sub, err)) return false;
    val = val.substr(0, a) + trim(sub) + trim(val.substr(b + 1));
  }
  err = "interpolation does not terminate";
  return false;
}

bool fortran_read_double(const std::string& s, double& v, std::string& err) {
  size_t i = 0;
  if (!lead_in(s, i, err)) return false;
  // Inf / Infinity / NaN (gfortran accepts them in list-directed input)
  {
    size_t j = i;
    std::string sign;
    if (j < s.size() && (s[j] == '+' || s[j] == '-')) sign = s[j++];
    std::string word;
    while (j < s.size() && std::isalpha((unsigned char)s[j])) word += (char)std::tolower(s[j++]);
    if ((word == "inf" || word == "infinity" || word == "nan") && (j >= s.size() || is_sep(s[j]))) {
      v = word == "nan" ? std::nan("") : (sign == "-" ? -INFINITY : INFINITY);
      return true;
    }
  }
  std::string num;
  size_t j = i;
  if (j < s.size() && (s[j] == '+' || s[j] == '-')) num += s[j++];
  int digits = 0;
  while (j < s.size() && std::isdigit((unsigned char)s[j])) { num += s[j++]; ++digits; }
  if (j < s.size() && s[j] == '.') {
    num += s[j++];
    while (j < s.size() && std::isdigit((unsigned char)s[j])) { num += s[j++]; ++digits; }
  }
  if (!digits) {
    err = "bad real number '" + s + "'";
    return false;
  }
  if (j < s.size()) {
    const char c = s[j];
    bool exp = false;
    if (std::strchr("eEdDqQ", c)) {
      ++j;
      exp = true;
    } else if (c == '+' || c == '-') {
      exp = true;  // 1.0+05 means 1.0e+05
    }
    if (exp) {
      num += 'e';
      if (j < s.size() && (s[j] == '+' || s[j] == '-')) num += s[j++];
      int ed = 0;
      while (j < s.size() && std::isdigit((unsigned char)s[j])) { num += s[j++]; ++ed; }
      if (!ed) {
        err = "bad real number '" + s + "'";
        return false;
      }
    }
  }
  if (j < s.size() && !is_sep(s[j])) {
    err = "bad real number '" + s + "'";
    return false;
  }
  v = std::strtod(num.c_str(), nullptr);  // correctly rounded, as gfortran's reader
  return true;
}

bool fortran_read_int(const std::string& s, long long& v, std::string& err) {
  size_t i = 0;
  if (!lead_in(s, i, err)) return false;
  size_t j = i;
  std::string num;
  if (j < s.size() && (s[j] == '+' || s[j] == '-')) num += s[j++];
  int digits = 0;
  while (j < s.size() && std::isdigit((unsigned char)s[j])) { num += s[j++]; ++digits; }
  if (!digits || (j < s.size() && !is_sep(s[j]))) {
    err = "bad integer '" + s + "'";
    return false;
  }
  v = std::strtoll(num.c_str(), nullptr, 10);
  return true;
}

// One REAL(8) item of a list-directed record: a separating blank, then G25.17
// (F20.(16 - e) plus five blanks for 0.1 <= |x| < 1e17, where e is the decimal
// exponent after rounding to 17 significant digits; otherwise 1P E25.17 with a
// three-digit exponent).  Always kItem characters.  The 17 digits come from one
// correctly rounded conversion (std::to_chars, the digits printf's %.16E gives);
// the F form places the same digits around the decimal point, which is what
// printf's %.*f gives at 16 - e decimals, since both round at the 17th
// significant digit.
constexpr int kItem = 26;

char* fortran_item(char* out, double x) {
  char* p = out;
  *p++ = ' ';
  if (!std::isfinite(x)) {
    const char* w = std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity");
    const int len = (int)std::strlen(w);
    std::memset(p, ' ', 25 - len);
    std::memcpy(p + 25 - len, w, len);
    return p + 25;
  }
  char s[48];
  const std::to_chars_result r = std::to_chars(s, s + sizeof s, x, std::chars_format::scientific, 16);
  const bool neg = s[0] == '-';
  const char* d = s + (neg ? 1 : 0);  // d[0] '.' d[2..17] 'e' sign exponent
  int ex = 0;
  for (const char* q = d + 20; q < r.ptr; ++q) ex = 10 * ex + (*q - '0');
  if (d[19] == '-') ex = -ex;
  char f[32];
  int n = 0;
  if (neg) f[n++] = '-';
  if (x == 0.0 || (ex >= -1 && ex < 17)) {
    char dig[17];
    dig[0] = d[0];
    std::memcpy(dig + 1, d + 2, 16);
    if (x == 0.0) {
      f[n++] = '0';
      f[n++] = '.';
      std::memset(f + n, '0', 16);
      n += 16;
    } else if (ex >= 0) {
      std::memcpy(f + n, dig, ex + 1);
      n += ex + 1;
      f[n++] = '.';
      std::memcpy(f + n, dig + ex + 1, 16 - ex);
      n += 16 - ex;
    } else {  // ex == -1: 0.ddddddddddddddddd
      f[n++] = '0';
      f[n++] = '.';
      std::memcpy(f + n, dig, 17);
      n += 17;
    }
    std::memset(p, ' ', 20 - n);
    std::memcpy(p + 20 - n, f, n);
    std::memset(p + 20, ' ', 5);
    return p + 25;
  }
  std::memcpy(f + n, d, 18);  // d.dddddddddddddddd
  n += 18;
  f[n++] = 'E';
  f[n++] = ex < 0 ? '-' : '+';
  const int a = ex < 0 ? -ex : ex;
  f[n++] = (char)('0' + a / 100);
  f[n++] = (char)('0' + a / 10 % 10);
  f[n++] = (char)('0' + a % 10);
  std::memset(p, ' ', 25 - n);
  std::memcpy(p + 25 - n, f, n);
  return p + 25;
}

std::string fortran_list_record(const double* v, int n) {
  std::string rec((size_t)kItem * (n > 0 ? n : 0), ' ');
  for (int k = 0; k < n; ++k) fortran_item(&rec[(size_t)k * kItem], v[k]);
  return rec;
}

int write_grid_records(const std::string& path, int nx, int ny, const double* xs, const double* ys,
                       const std::vector<const double*>& fields) {
  const size_t items = 2 + fields.size(), rec = items * kItem + 1;
  // blocks of whole x columns (ny records each), formatted in parallel into
  // their final offsets, then written in order; about 64 MB of text per block
  const int cols = std::max(1, (int)std::min<size_t>((size_t)nx, (64u << 20) / (rec * (size_t)ny)));
  std::vector<char> buf;
  try {
    buf.resize(rec * (size_t)ny * cols);
  } catch (const std::bad_alloc&) {
    return set_error(TARA_ERR_NOMEM, "write_grid_records: no host memory for the text buffer");
  }
  FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) return set_error(TARA_ERR_ARGS, "cannot open " + path + " for writing");
  const int hw = (int)std::thread::hardware_concurrency();
  const int nthreads = std::max(1, std::min(hw > 0 ? hw : 1, 64));
  int rc = TARA_OK;
  for (int i0 = 0; i0 < nx && rc == TARA_OK; i0 += cols) {
    const int ncol = std::min(cols, nx - i0);
    auto work = [&](int t) {
      for (int c = t; c < ncol; c += nthreads) {
        const int i = i0 + c;
        char* o = buf.data() + rec * (size_t)ny * c;
        for (int j = 0; j < ny; ++j) {
          const size_t q = (size_t)j * nx + i;
          o = fortran_item(o, xs[i]);
          o = fortran_item(o, ys[j]);
          for (const double* fld : fields) o = fortran_item(o, fld[q]);
          *o++ = '\n';
        }
      }
    };
    const int nt = std::min(nthreads, ncol);
    std::vector<std::thread> pool;
    int started = 1;
    try {
      for (; started < nt; ++started) pool.emplace_back(work, started);
    } catch (const std::exception&) {  // no more threads: this one takes the rest
    }
    for (int t = started; t < nt; ++t) work(t);
    work(0);
    for (std::thread& th : pool) th.join();
    const size_t bytes = rec * (size_t)ny * ncol;
    if (std::fwrite(buf.data(), 1, bytes, fp) != bytes) rc = set_error(TARA_ERR_ARGS, "short write to " + path);
  }
  if (std::fclose(fp) != 0 && rc == TARA_OK) rc = set_error(TARA_ERR_ARGS, "cannot close " + path);
  return rc;
}

}  // namespace tara

using namespace tara;

extern "C" {

int tara_fortran_read_double(const char* s, double* out) {
  if (!s || !out) return set_error(TARA_ERR_ARGS, "null argument");
  std::string err;
  if (!fortran_read_double(s, *out, err)) return set_error(TARA_ERR_INI, err);
  return set_ok();
}

int tara_fortran_read_int(const char* s, long long* out) {
  if (!s || !out) return set_error(TARA_ERR_ARGS, "null argument");
  std::string err;
  if (!fortran_read_int(s, *out, err)) return set_error(TARA_ERR_INI, err);
  return set_ok();
}

int tara_ini_get(const char* path, const char* section, const char* key, char* buf, int buflen) {
  if (!path || !section || !key || !buf || buflen <= 0) return set_error(TARA_ERR_ARGS, "null argument");
  IniFile ini;
  std::string err, val;
  if (!ini_parse_file(path, ini, err) || !ini_get(ini, section, key, val, err))
    return set_error(TARA_ERR_INI, err);
  std::snprintf(buf, (size_t)buflen, "%s", val.c_str());
  return set_ok();
}

int tara_write_grid_records(const char* path, int nx, int ny, const double* xs, const double* ys,
                            const double* fields, int nfields) {
  if (!path || !xs || !ys || nx < 1 || ny < 1 || nfields < 0 || (nfields > 0 && !fields))
    return set_error(TARA_ERR_ARGS, "tara_write_grid_records: bad argument");
  std::vector<const double*> f;
  for (int k = 0; k < nfields; ++k) f.push_back(fields + (size_t)k * nx * ny);
  const int rc = write_grid_records(path, nx, ny, xs, ys, f);
  return rc ? rc : set_ok();
}

int tara_fortran_list_record(const double* v, int n, char* buf, int buflen) {
  if (!v || n < 0 || !buf || buflen <= 0) return set_error(TARA_ERR_ARGS, "null argument");
  const std::string rec = fortran_list_record(v, n);
  if (rec.size() + 1 > (size_t)buflen) {
    buf[0] = '\0';
    return set_error(TARA_ERR_ARGS, "tara_fortran_list_record: the record needs " + std::to_string(rec.size() + 1) +
                                        " bytes, buflen is " + std::to_string(buflen));
  }
  std::memcpy(buf, rec.c_str(), rec.size() + 1);
  return set_ok();
}

}  // extern "C"
