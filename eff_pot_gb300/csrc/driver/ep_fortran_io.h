// ep_fortran_io.h - the Fortran I/O forms the eff_pot driver and its files use:
//   * NAMELIST input (`&input name = value, ... /`, DFT4He3d.f90:106-140),
//   * list-directed text (`read(1,*)` / `write(10,*)`, readenc.f90:83-176,
//     printoutc.f90:98-125) with comment lines skipped as titols.f90 does,
//   * sequential unformatted records (printoutc.f90:73-80, iprint < 0).
// Host-only C++17; no dependence on the CUDA toolkit.
#pragma once
#include <cstdint>
#include <istream>
#include <map>
#include <ostream>
#include <string>
#include <vector>

namespace fio {

// One namelist group: variable name (lower case) -> its value items, each
// already expanded from repeat counts (r*c).  Strings keep their quotes off.
struct Namelist {
  std::map<std::string, std::vector<std::string>> vars;
  std::vector<std::string> order;  // first-assignment order, for echoing
  bool has(const std::string& k) const { return vars.count(k) != 0; }
};

// Parses the group named `group` (case-insensitive) from `in`.  Returns false
// with a message in err if the group is missing or malformed.
bool parse_namelist(std::istream& in, const std::string& group, Namelist& nml, std::string& err);

// Conversions of namelist / list-directed items (Fortran spellings: 1.5d-3,
// .true., T, 'text').  They throw std::invalid_argument on bad input.
double to_real(const std::string& s);
long to_int(const std::string& s);
bool to_logical(const std::string& s);

// List-directed reader over a whole stream: blanks, commas and line ends
// separate values, r*c repeats c r times, a slash ends the current read,
// complex values are (re,im).  skip_comments() positions the reader after the
// leading lines whose first column is `c` (titols.f90).
class ListReader {
 public:
  explicit ListReader(std::istream& in) : in_(in) {}
  void skip_comments(char c = '#');
  bool real(double& v);
  bool integer(long& v);
  bool logical(bool& v);
  bool complex(double& re, double& im);
  bool reals(double* v, size_t n);
  bool complexes(double* v, size_t n);  // interleaved re, im
  // ends the current READ statement: pending repeats are dropped and the
  // next value comes from the next line (Fortran starts a new record)
  void end_statement();

 private:
  bool token(std::string& t);
  bool raw(std::string& t);
  std::istream& in_;
  std::string pending_;
  long repeat_ = 0;
  std::string line_;
  size_t pos_ = 0;
  bool have_line_ = false;
};

// List-directed style writers (values as Fortran reads them back).
void write_reals(std::ostream& os, const double* v, size_t n, int per_line = 4);
void write_complexes(std::ostream& os, const double* v, size_t n, int per_line = 2);

// Sequential unformatted records: 4-byte length before and after the data.
bool write_record(std::ostream& os, const void* data, uint32_t bytes);
bool read_record(std::istream& is, std::vector<char>& data);

}  // namespace fio
