// input.ini reading with the semantics of the reference's cfgio module
// (lib/iniparser/cfgio_mod.f90) and Fortran list-directed number reads
// (lib/iniparser/string_conv_mod.f90:95-99, `read(str,*) v`).
#pragma once
#include <string>
#include <utility>
#include <vector>

namespace tara {

struct IniSection {
  std::string name;
  std::vector<std::pair<std::string, std::string>> pars;  // in file order
};

struct IniFile {
  std::vector<IniSection> sections;  // sections[0] is DEFAULTS
};

// Parse a file.  On failure returns false and sets err (the reference stops the
// program with errexit instead).
bool ini_parse_file(const std::string& path, IniFile& ini, std::string& err);
bool ini_parse_text(const std::string& text, IniFile& ini, std::string& err);

// cfg%gets: raw value with the DEFAULTS fallback, quotes stripped, ${sec:key} /
// ${key} interpolated.
bool ini_get(const IniFile& ini, const std::string& section, const std::string& key,
             std::string& val, std::string& err);

// Fortran list-directed reads of one item from a string: leading blanks
// skipped, optional repeat count r*, the value ends at a blank, comma, slash or
// the end of the string; reals accept d/D/e/E/q/Q exponents and a signed
// exponent without a letter.  A slash therefore ends "3.0d0/128.0d0" after 3.0.
bool fortran_read_double(const std::string& s, double& v, std::string& err);
bool fortran_read_int(const std::string& s, long long& v, std::string& err);

// One list-directed output record of REAL(8) values in gfortran's style
// (G25.17 per item: F form for 0.1 <= |x| < 1e17, otherwise 1P E form with a
// three-digit exponent), each item preceded by one separating blank.
std::string fortran_list_record(const double* v, int n);

// A snapshot file of the reference's drivers: one record per grid point, x
// outer and y inner (do i = 1, Nx; do j = 1, Ny), holding xs[i], ys[j] and each
// field's value at index j * nx + i, in fortran_list_record's format.  Records
// are formatted in parallel on the host's cores and written in order.
int write_grid_records(const std::string& path, int nx, int ny, const double* xs, const double* ys,
                       const std::vector<const double*>& fields);

}  // namespace tara
