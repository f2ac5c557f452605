// ep_fortran_io.cpp - see ep_fortran_io.h.
#include "ep_fortran_io.h"

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <stdexcept>

namespace fio {

namespace {

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

bool is_sep(char c) { return c == ' ' || c == '\t' || c == ',' || c == '\r' || c == '\n'; }

// Splits "r*value" into (r, value); r = 1 when there is no repeat prefix.
long split_repeat(const std::string& t, std::string& value) {
  size_t i = 0;
  while (i < t.size() && std::isdigit((unsigned char)t[i])) ++i;
  if (i > 0 && i < t.size() && t[i] == '*') {
    value = t.substr(i + 1);
    return std::strtol(t.substr(0, i).c_str(), nullptr, 10);
  }
  value = t;
  return 1;
}

std::string unquote(const std::string& s) {
  if (s.size() >= 2 && (s[0] == '\'' || s[0] == '"') && s.back() == s[0]) {
    const char q = s[0];
    std::string out;
    for (size_t i = 1; i + 1 < s.size(); ++i) {
      out.push_back(s[i]);
      if (s[i] == q && i + 2 < s.size() && s[i + 1] == q) ++i;  // doubled quote
    }
    return out;
  }
  return s;
}

// Namelist tokens: names, '=', values (strings keep their quotes, complex
// values their parentheses), with '!' comments removed.
std::vector<std::string> nml_tokens(const std::string& text, size_t begin, size_t& end_out, bool& closed) {
  std::vector<std::string> tok;
  size_t i = begin;
  closed = false;
  while (i < text.size()) {
    const char c = text[i];
    if (is_sep(c)) { ++i; continue; }
    if (c == '!') {
      while (i < text.size() && text[i] != '\n') ++i;
      continue;
    }
    if (c == '/') { closed = true; ++i; break; }
    if (c == '&' || c == '$') {  // &end / $end
      size_t j = i + 1;
      while (j < text.size() && std::isalpha((unsigned char)text[j])) ++j;
      if (lower(text.substr(i + 1, j - i - 1)) == "end") { closed = true; i = j; break; }
    }
    if (c == '=') { tok.push_back("="); ++i; continue; }
    if (c == '\'' || c == '"') {
      size_t j = i + 1;
      while (j < text.size()) {
        if (text[j] == c) {
          if (j + 1 < text.size() && text[j + 1] == c) { j += 2; continue; }
          break;
        }
        ++j;
      }
      tok.push_back(text.substr(i, j + 1 - i));
      i = j + 1;
      continue;
    }
    size_t j = i;
    std::string t;
    while (j < text.size() && !is_sep(text[j]) && text[j] != '=' && text[j] != '/' && text[j] != '!') {
      if (text[j] == '(') {  // complex value, possibly with blanks inside
        while (j < text.size() && text[j] != ')') {
          if (!std::isspace((unsigned char)text[j])) t.push_back(text[j]);
          ++j;
        }
        if (j < text.size()) t.push_back(text[j++]);
        continue;
      }
      if (text[j] == '\'' || text[j] == '"') break;
      t.push_back(text[j++]);
    }
    if (j < text.size() && (text[j] == '\'' || text[j] == '"') && !t.empty() && t.back() == '*') {
      // r*'string'
      const char q = text[j];
      size_t k = j + 1;
      while (k < text.size() && text[k] != q) ++k;
      t += text.substr(j, k + 1 - j);
      j = k + 1;
    }
    tok.push_back(t);
    i = j;
  }
  end_out = i;
  return tok;
}

}  // namespace

bool parse_namelist(std::istream& in, const std::string& group, Namelist& nml, std::string& err) {
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string text = ss.str();
  const std::string lt = lower(text);
  const std::string g = lower(group);
  size_t at = std::string::npos;
  for (size_t p = 0; (p = lt.find(g, p)) != std::string::npos; ++p) {
    if (p > 0 && (lt[p - 1] == '&' || lt[p - 1] == '$') &&
        (p + g.size() >= lt.size() || !std::isalnum((unsigned char)lt[p + g.size()]))) {
      at = p + g.size();
      break;
    }
  }
  if (at == std::string::npos) {
    err = "namelist group &" + group + " not found";
    return false;
  }
  size_t end = 0;
  bool closed = false;
  const std::vector<std::string> tok = nml_tokens(text, at, end, closed);
  if (!closed) {
    err = "namelist group &" + group + " is not terminated by '/'";
    return false;
  }
  size_t i = 0;
  while (i < tok.size()) {
    if (i + 1 >= tok.size() || tok[i + 1] != "=") {
      err = "namelist: expected 'name =' at '" + tok[i] + "'";
      return false;
    }
    const std::string name = lower(tok[i]);
    i += 2;
    std::vector<std::string> vals;
    while (i < tok.size() && !(i + 1 < tok.size() && tok[i + 1] == "=")) {
      if (tok[i] == "=") { err = "namelist: misplaced '='"; return false; }
      std::string v;
      const long r = split_repeat(tok[i], v);
      for (long k = 0; k < r; ++k) vals.push_back(unquote(v));
      ++i;
    }
    if (!nml.has(name)) nml.order.push_back(name);
    nml.vars[name] = vals;
  }
  return true;
}

double to_real(const std::string& s0) {
  std::string s = s0;
  for (char& c : s)
    if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
  char* endp = nullptr;
  const double v = std::strtod(s.c_str(), &endp);
  if (s.empty() || endp == s.c_str() || *endp != 0) throw std::invalid_argument("not a real: '" + s0 + "'");
  return v;
}

long to_int(const std::string& s) {
  char* endp = nullptr;
  const long v = std::strtol(s.c_str(), &endp, 10);
  if (s.empty() || *endp != 0) throw std::invalid_argument("not an integer: '" + s + "'");
  return v;
}

bool to_logical(const std::string& s0) {
  std::string s = lower(s0);
  size_t i = 0;
  if (i < s.size() && s[i] == '.') ++i;
  if (i < s.size() && s[i] == 't') return true;
  if (i < s.size() && s[i] == 'f') return false;
  throw std::invalid_argument("not a logical: '" + s0 + "'");
}

// ---------------------------------------------------------------------------
void ListReader::skip_comments(char c) {
  std::string l;
  while (true) {
    const std::streampos p = in_.tellg();
    if (!std::getline(in_, l)) return;
    if (l.empty() || l[0] != c) {
      in_.clear();
      in_.seekg(p);
      return;
    }
  }
}

void ListReader::end_statement() {
  repeat_ = 0;
  pending_.clear();
  have_line_ = false;
}

bool ListReader::raw(std::string& t) {
  t.clear();
  while (true) {
    if (!have_line_) {
      if (!std::getline(in_, line_)) return false;
      pos_ = 0;
      have_line_ = true;
    }
    while (pos_ < line_.size() && is_sep(line_[pos_])) ++pos_;
    if (pos_ >= line_.size()) { have_line_ = false; continue; }
    if (line_[pos_] == '/') { pos_ = line_.size(); return false; }
    // a value, a repeat prefix, or a complex that may span lines
    while (true) {
      while (pos_ < line_.size() && !is_sep(line_[pos_]) && line_[pos_] != '(') t.push_back(line_[pos_++]);
      if (pos_ < line_.size() && line_[pos_] == '(') {
        while (true) {
          while (pos_ < line_.size() && line_[pos_] != ')') {
            if (!std::isspace((unsigned char)line_[pos_])) t.push_back(line_[pos_]);
            ++pos_;
          }
          if (pos_ < line_.size()) { t.push_back(line_[pos_++]); break; }
          if (!std::getline(in_, line_)) return false;
          pos_ = 0;
        }
        continue;
      }
      break;
    }
    return true;
  }
}

bool ListReader::token(std::string& t) {
  if (repeat_ > 0) {
    --repeat_;
    t = pending_;
    return true;
  }
  std::string r;
  if (!raw(r)) return false;
  const long n = split_repeat(r, pending_);
  repeat_ = n - 1;
  t = pending_;
  return true;
}

bool ListReader::real(double& v) {
  std::string t;
  if (!token(t)) return false;
  v = to_real(t);
  return true;
}

bool ListReader::integer(long& v) {
  std::string t;
  if (!token(t)) return false;
  v = to_int(t);
  return true;
}

bool ListReader::logical(bool& v) {
  std::string t;
  if (!token(t)) return false;
  v = to_logical(t);
  return true;
}

bool ListReader::complex(double& re, double& im) {
  std::string t;
  if (!token(t)) return false;
  if (t.size() < 5 || t.front() != '(' || t.back() != ')') throw std::invalid_argument("not a complex: '" + t + "'");
  const size_t c = t.find(',');
  if (c == std::string::npos) throw std::invalid_argument("not a complex: '" + t + "'");
  re = to_real(t.substr(1, c - 1));
  im = to_real(t.substr(c + 1, t.size() - c - 2));
  return true;
}

bool ListReader::reals(double* v, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!real(v[i])) return false;
  return true;
}

bool ListReader::complexes(double* v, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!complex(v[2 * i], v[2 * i + 1])) return false;
  return true;
}

// ---------------------------------------------------------------------------
void write_reals(std::ostream& os, const double* v, size_t n, int per_line) {
  char buf[64];
  for (size_t i = 0; i < n; ++i) {
    std::snprintf(buf, sizeof buf, " %24.16E", v[i]);
    os << buf;
    if ((i + 1) % per_line == 0 || i + 1 == n) os << '\n';
  }
}

void write_complexes(std::ostream& os, const double* v, size_t n, int per_line) {
  char buf[96];
  for (size_t i = 0; i < n; ++i) {
    std::snprintf(buf, sizeof buf, " (%.16E,%.16E)", v[2 * i], v[2 * i + 1]);
    os << buf;
    if ((i + 1) % per_line == 0 || i + 1 == n) os << '\n';
  }
}

bool write_record(std::ostream& os, const void* data, uint32_t bytes) {
  os.write(reinterpret_cast<const char*>(&bytes), 4);
  os.write(reinterpret_cast<const char*>(data), bytes);
  os.write(reinterpret_cast<const char*>(&bytes), 4);
  return (bool)os;
}

bool read_record(std::istream& is, std::vector<char>& data) {
  uint32_t a = 0, b = 0;
  if (!is.read(reinterpret_cast<char*>(&a), 4)) return false;
  data.resize(a);
  if (a && !is.read(data.data(), a)) return false;
  if (!is.read(reinterpret_cast<char*>(&b), 4)) return false;
  return a == b;
}

}  // namespace fio
