// ep_select_pot.cu - Select_Pot by name (V_impur.f90:87-932), host code.
//
// The closed forms the library evaluates are built in.  The inverse-power
// fits (the Param_LJ_* family: V = f_core / |aa x^2 + bb x + cc| / sum_k
// Pg(k) x^-(k+k0), e.g. V_Fausto_Rb_gs, V_impur.f90:2206-2250) are read
// from the reference's own V_impur.f90: the Select_Pot chain maps the name
// to a function, the function's COMMON block names the BLOCK DATA that
// holds Npg, Pg, rcutoff, fcutoff, r0, aa, bb, cc and k0, and the function
// itself gives the precision of its sum (Real*16 or Real*8 Sto) and, where
// it writes x**(k+5), the exponent offset.  Every literal keeps its Fortran
// kind: without exponent letter or with E it is default REAL (binary32)
// before DATA widens it, D is double, Q is Real*16 (kept here as a
// double-double pair, 106 bits).  Two fits of their own form are read the
// same way: Func_Ba_plus_gs behind 'Ba_plus_old_gs' (even inverse powers)
// and V_Cs_7s (exponentials times powers of x).
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/eff_pot.h"
#include "ep_pairpot.h"

namespace {

struct Stmt {
  std::string raw;  // comments stripped, continuations joined
  std::string cl;   // lower case, blanks removed
};

std::string lower_compact(const std::string& s) {
  std::string o;
  for (char ch : s)
    if (!isspace((unsigned char)ch)) o.push_back((char)tolower((unsigned char)ch));
  return o;
}

// Free-form statements: '!' comments (outside quotes) removed, '&'
// continuations joined, ';' separated statements split.
std::vector<Stmt> statements(const std::string& text) {
  std::vector<Stmt> out;
  std::istringstream in(text);
  std::string line, acc;
  bool cont = false;
  while (std::getline(in, line)) {
    std::string code;
    char q = 0;
    for (char ch : line) {
      if (q) {
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
      } else if (ch == '!') {
        break;
      }
      code.push_back(ch);
    }
    size_t a = code.find_first_not_of(" \t\r");
    if (a == std::string::npos) {
      if (!cont) acc.clear();
      continue;
    }
    code = code.substr(a);
    if (cont && !code.empty() && code[0] == '&') code = code.substr(1);
    size_t b = code.find_last_not_of(" \t\r");
    code = code.substr(0, b + 1);
    cont = !code.empty() && code.back() == '&';
    if (cont) code.pop_back();
    acc += code;
    acc.push_back(' ');
    if (cont) continue;
    // split on ';' outside quotes
    std::string cur;
    q = 0;
    for (char ch : acc) {
      if (q) {
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
      } else if (ch == ';') {
        if (!lower_compact(cur).empty()) out.push_back({cur, lower_compact(cur)});
        cur.clear();
        continue;
      }
      cur.push_back(ch);
    }
    if (!lower_compact(cur).empty()) out.push_back({cur, lower_compact(cur)});
    acc.clear();
  }
  return out;
}

bool starts(const std::string& s, const char* p) { return s.compare(0, strlen(p), p) == 0; }

bool is_end(const std::string& cl) {
  return cl == "end" || starts(cl, "endfunction") || starts(cl, "endblockdata") || starts(cl, "endsubroutine");
}

// name of the function a statement opens ("" if none)
std::string function_name(const std::string& cl) {
  size_t f = cl.find("function");
  if (f == std::string::npos || starts(cl, "end")) return "";
  const std::string pre = cl.substr(0, f);
  if (!(pre.empty() || pre == "doubleprecision" || pre == "real*8" || pre == "real(kind=8)" || pre == "real(8)"))
    return "";
  size_t p = cl.find('(', f);
  if (p == std::string::npos) return "";
  return cl.substr(f + 8, p - f - 8);
}

// ---------------------------------------------------------------- literals
struct Lit {
  int kind = 0;  // 0 integer, 4 default real, 8 double, 16 quad
  double hi = 0, lo = 0;
  long long ival = 0;
  bool ok = false;
};

// decimal digits d (no dot) times 10^e10, sign s, as a double-double:
// d is split into chunks of at most 18 digits (exact in uint64, exact as a
// double pair); powers of ten up to 10^22 are exact doubles.
ep_dd dd_from_uint(uint64_t u) {
  const double hi = (double)(u >> 11 << 11);
  const double lo = (double)(u & 2047u);
  return ep_dd_quick(hi + lo, (hi - (hi + lo)) + lo);
}
ep_dd dd_pow10(int e) {  // e >= 0
  ep_dd r{1.0, 0.0};
  while (e > 0) {
    const int k = e > 22 ? 22 : e;
    double p = 1.0;
    for (int i = 0; i < k; ++i) p *= 10.0;
    r = ep_dd_mul(r, ep_dd{p, 0.0});
    e -= k;
  }
  return r;
}
ep_dd dd_div(ep_dd a, ep_dd b) {
  const double q1 = a.hi / b.hi;
  const ep_dd r = ep_dd_add(a, ep_dd_mul(ep_dd{-q1, 0.0}, b));
  const double q2 = r.hi / b.hi;
  const ep_dd r2 = ep_dd_add(r, ep_dd_mul(ep_dd{-q2, 0.0}, b));
  const double q3 = r2.hi / b.hi;
  const ep_dd q = ep_dd_quick(q1, q2);
  return ep_dd_add(q, ep_dd{q3, 0.0});
}
ep_dd dd_decimal(const std::string& digits, int e10) {
  ep_dd m{0.0, 0.0};
  size_t i = 0;
  while (i < digits.size()) {
    const size_t k = std::min<size_t>(18, digits.size() - i);
    uint64_t u = 0;
    for (size_t j = 0; j < k; ++j) u = u * 10 + (uint64_t)(digits[i + j] - '0');
    m = ep_dd_add(ep_dd_mul(m, dd_pow10((int)k)), dd_from_uint(u));
    i += k;
  }
  if (e10 >= 0) return ep_dd_mul(m, dd_pow10(e10));
  return dd_div(m, dd_pow10(-e10));
}

Lit literal(const std::string& tok0) {
  Lit L;
  std::string t = lower_compact(tok0);
  if (t.empty()) return L;
  bool neg = false;
  size_t i = 0;
  if (t[i] == '+' || t[i] == '-') neg = t[i++] == '-';
  std::string digits;
  int frac = 0;
  bool dot = false, any = false;
  for (; i < t.size(); ++i) {
    const char ch = t[i];
    if (isdigit((unsigned char)ch)) {
      digits.push_back(ch);
      any = true;
      if (dot) ++frac;
    } else if (ch == '.' && !dot) {
      dot = true;
    } else {
      break;
    }
  }
  if (!any) return L;
  char letter = 0;
  int ex = 0;
  if (i < t.size()) {
    letter = t[i++];
    if (letter != 'e' && letter != 'd' && letter != 'q') return L;
    bool eneg = false;
    if (i < t.size() && (t[i] == '+' || t[i] == '-')) eneg = t[i++] == '-';
    if (i >= t.size()) return L;
    for (; i < t.size(); ++i) {
      if (!isdigit((unsigned char)t[i])) return L;
      ex = ex * 10 + (t[i] - '0');
    }
    if (eneg) ex = -ex;
  }
  const std::string txt = (neg ? "-" : "") + digits.substr(0, digits.size() - frac) + "." +
                          digits.substr(digits.size() - frac) + "e" + std::to_string(ex);
  if (!dot && !letter) {
    L.kind = 0;
    L.ival = std::strtoll(tok0.c_str(), nullptr, 10);
    L.hi = (double)L.ival;
  } else if (letter == 'q') {
    L.kind = 16;
    ep_dd v = dd_decimal(digits, ex - frac);
    if (neg) v = ep_dd{-v.hi, -v.lo};
    L.hi = v.hi;
    L.lo = v.lo;
  } else if (letter == 'd') {
    L.kind = 8;
    L.hi = std::strtod(txt.c_str(), nullptr);
  } else {
    L.kind = 4;
    L.hi = (double)std::strtof(txt.c_str(), nullptr);
  }
  L.ok = true;
  return L;
}

// DATA name/v1, v2, .../ [, name/.../] -> (name, literals)
struct DataItem {
  std::string name;
  std::vector<std::string> vals;
};
std::vector<DataItem> data_items(const std::string& raw) {
  std::vector<DataItem> out;
  const std::string& s = raw;
  size_t k = 0;
  while (k < s.size() && isspace((unsigned char)s[k])) ++k;
  k += 4;  // "data"
  while (k < s.size()) {
    size_t sl = s.find('/', k);
    if (sl == std::string::npos) break;
    DataItem it;
    it.name = lower_compact(s.substr(k, sl - k));
    if (!it.name.empty() && it.name[0] == ',') it.name = it.name.substr(1);
    size_t e = s.find('/', sl + 1);
    if (e == std::string::npos) break;
    std::string body = s.substr(sl + 1, e - sl - 1);
    std::stringstream ss(body);
    std::string v;
    while (std::getline(ss, v, ','))
      if (!lower_compact(v).empty()) it.vals.push_back(v);
    out.push_back(it);
    k = e + 1;
  }
  return out;
}

int put_err(char* err, int cap, const std::string& m) {
  if (err && cap > 0) snprintf(err, (size_t)cap, "%s", m.c_str());
  return EP_ERR_INVALID_ARG;
}

int builtin(const std::string& sel, ep_potential* p) {
  static const char* kout[4] = {"Na_plus_Koutselos", "K_plus_Koutselos", "Rb_plus_Koutselos", "Cs_plus_Koutselos"};
  static const char* patil[5] = {"LI", "NA", "K", "RB", "CS"};
  if (sel == "null") {
    p->kind = EP_POT_NULL;
    return 1;
  }
  for (int i = 0; i < 4; ++i)
    if (sel == kout[i]) {
      p->kind = EP_POT_KOUTSELOS;
      p->par[0] = i;
      return 1;
    }
  for (int i = 0; i < 5; ++i)
    if (sel == patil[i]) {
      p->kind = EP_POT_PATIL;
      p->par[0] = i;
      return 1;
    }
  if (sel == "Aziz_He") {
    p->kind = EP_POT_AZIZ;
    return 1;
  }
  if (sel == "Ar_He" || sel == "Xe_He") {
    p->kind = EP_POT_TANG_TOENNIES;
    p->par[0] = sel == "Ar_He" ? 0 : 1;
    return 1;
  }
  static const char* ag[3] = {"Ag_gs", "Ag_Pi", "Ag_Sig"};
  for (int i = 0; i < 3; ++i)
    if (sel == ag[i]) {
      p->kind = EP_POT_AG;
      p->par[0] = i;
      return 1;
    }
  if (sel == "Ba_gs") {
    p->kind = EP_POT_BA_GS;
    return 1;
  }
  static const char* surf[10] = {"Grafeno", "Grafeno_sin_dispersion", "TiO2", "Au", "Au_TiO2",
                                 "dAu_TiO2", "Ag_Graphene", "dz_Ag_Graphene", "Au_Graphene", "dz_Au_Graphene"};
  for (int i = 0; i < 10; ++i)
    if (sel == surf[i]) {
      p->kind = EP_POT_SURFACE;
      p->par[0] = i;
      return 1;
    }
  if (sel.size() == 6 && sel.compare(0, 5, "CH3I_") == 0 && sel[5] >= '0' && sel[5] <= '4') {
    p->kind = EP_POT_CH3I;
    p->par[0] = sel[5] - '0';
    return 1;
  }
  return 0;
}

}  // namespace

extern "C" int ep_select_pot(const char* selec, double r_cutoff, double umax, const char* source_path, ep_potential* p,
                             ep_series* series, char* err, int cap) {
  if (!selec || !p) return put_err(err, cap, "null argument");
  *p = ep_potential{};
  p->r_cutoff = r_cutoff;
  p->umax = umax;
  std::string sel(selec);
  while (!sel.empty() && isspace((unsigned char)sel.back())) sel.pop_back();
  while (!sel.empty() && isspace((unsigned char)sel.front())) sel.erase(sel.begin());
  if (builtin(sel, p)) return EP_OK;
  if (!source_path || !series)
    return put_err(err, cap, "selec '" + sel + "' is not a built-in closed form; give the V_impur.f90 source");
  std::ifstream f(source_path, std::ios::binary);
  if (!f) return put_err(err, cap, std::string("cannot read ") + source_path);
  std::stringstream buf;
  buf << f.rdbuf();
  const std::vector<Stmt> st = statements(buf.str());

  // 1. the Select_Pot chain: name -> function
  std::string func;
  {
    bool in_sel = false, match = false;
    for (const Stmt& s : st) {
      if (!in_sel) {
        if (function_name(s.cl) == "select_pot") in_sel = true;
        continue;
      }
      if (is_end(s.cl) && (s.cl == "end" || starts(s.cl, "endfunction"))) break;
      if (s.cl.find("trim(selec).eq.'") != std::string::npos) {
        match = false;
        size_t k = 0;
        while ((k = s.raw.find('\'', k)) != std::string::npos) {
          size_t e = s.raw.find('\'', k + 1);
          if (e == std::string::npos) break;
          if (s.raw.substr(k + 1, e - k - 1) == sel) match = true;
          k = e + 1;
        }
        continue;
      }
      if (match && starts(s.cl, "select_pot=")) {
        size_t par = s.cl.find('(');
        if (par != std::string::npos) {
          func = s.cl.substr(11, par - 11);
          break;
        }
      }
    }
  }
  if (func.empty()) return put_err(err, cap, "selec '" + sel + "' is not in the Select_Pot chain of " + source_path);

  // 2. the function: its COMMON block and its form -- the inverse-power fit
  // (core constant, |parabola|, sum of Pg(k) x^-(k+k0), Real*16 or Real*8
  // Sto), Func_Ba_plus_gs's even powers, or V_Cs_7s's exponential fit; a
  // function that only returns another one (V_Ba_plus_old_gs) is followed
  enum { F_SERIES, F_EVENPOW, F_EXPFIT, F_NONE };
  std::string common;
  bool quad = false, has_core = false, has_par = false, has_sum = false;
  bool even_sum = false, plain_par = false, exp_first = false, exp_sum = false, clamp = false;
  int k0_lit = -1;
  Lit x0;
  for (int hop = 0; hop < 2; ++hop) {
    size_t i = 0;
    for (; i < st.size(); ++i)
      if (function_name(st[i].cl) == func) break;
    if (i == st.size()) return put_err(err, cap, "function " + func + " not found");
    std::string forward;
    int stmts = 0;
    for (++i; i < st.size() && !is_end(st[i].cl); ++i) {
      const std::string& c = st[i].cl;
      if (starts(c, "implicit") || starts(c, "parameter") || starts(c, "real") || starts(c, "integer") ||
          c == "return")
        continue;
      ++stmts;
      if (starts(c, (func + "=").c_str()) && c.size() > func.size() + 4 &&
          c.compare(c.size() - 3, 3, "(x)") == 0)
        forward = c.substr(func.size() + 1, c.size() - func.size() - 4);
      if (starts(c, "common/")) common = c.substr(7, c.find('/', 7) - 7);
      if (c.find("x.le.rcutoff") != std::string::npos) has_core = true;
      if (c.find("abs(aa*x**2+bb*x+cc)") != std::string::npos) has_par = true;
      if (c.find("=aa*x**2+bb*x+cc") != std::string::npos) plain_par = true;
      if (c.find("sto=sto+pg(k)/x**(2*(k-1)+6)") != std::string::npos) even_sum = true;
      else if (c.find("sto=sto+pg(k)*x**(k-1)*dexp(-ps(k)*x)") != std::string::npos) exp_sum = true;
      else if (c.find("sto=sto+pg(k)") != std::string::npos) {
        has_sum = true;
        size_t q = c.find("x**(k+");
        if (q != std::string::npos) k0_lit = std::atoi(c.c_str() + q + 6);
      }
      if (c.find("sto=pg(1)*dexp(-ps(1)*x)/x") != std::string::npos) exp_first = true;
      if (c.find("if(xx.lt.x0)") != std::string::npos) clamp = true;
      if (starts(c, "data")) {
        for (const DataItem& d : data_items(st[i].raw))
          if (d.name == "x0" && d.vals.size() == 1) x0 = literal(d.vals[0]);
      }
    }
    // function bodies hold their statements between a declaration and END;
    // the Real*16 / Real*8 declaration of Sto decides the sum's precision
    if (forward.empty() || stmts != 1) break;
    func = forward;
  }
  {
    size_t i = 0;
    for (; i < st.size(); ++i)
      if (function_name(st[i].cl) == func) break;
    for (++i; i < st.size() && !is_end(st[i].cl); ++i)
      if (starts(st[i].cl, "real*16") && st[i].cl.find("sto") != std::string::npos) quad = true;
  }
  const int form = (has_core && has_par && has_sum) ? F_SERIES
                   : (even_sum && plain_par)        ? F_EVENPOW
                   : (exp_first && exp_sum && plain_par && clamp && x0.ok) ? F_EXPFIT
                                                                            : F_NONE;
  if (common.empty() || form == F_NONE)
    return put_err(err, cap, "'" + sel + "' (" + func + ") is not an inverse-power fit with a parabolic core");

  // 3. the BLOCK DATA holding that COMMON
  int npg = -1;
  bool pg16 = false;
  std::vector<std::string> pg, ps;
  Lit sc[6];
  const char* scn[6] = {"rcutoff", "fcutoff", "r0", "aa", "bb", "cc"};
  int k0 = -1;
  {
    size_t i = 0, b0 = st.size();
    for (; i < st.size(); ++i) {
      if (starts(st[i].cl, "blockdata")) b0 = i;
      if (starts(st[i].cl, ("common/" + common + "/").c_str()) && b0 < i) {
        bool inside = true;
        for (size_t j = b0 + 1; j < i; ++j)
          if (is_end(st[j].cl)) inside = false;
        if (inside) break;
      }
    }
    if (i == st.size()) return put_err(err, cap, "no BLOCK DATA for COMMON /" + common + "/");
    for (size_t j = b0 + 1; j < st.size() && !is_end(st[j].cl); ++j) {
      const std::string& c = st[j].cl;
      if (starts(c, "parameter(npg=")) npg = std::atoi(c.c_str() + 14);
      if (starts(c, "real*16") && (c.find("pg") != std::string::npos)) pg16 = true;
      if (!starts(c, "data")) continue;
      for (const DataItem& d : data_items(st[j].raw)) {
        if (d.name == "pg") pg = d.vals;
        if (d.name == "ps") ps = d.vals;
        for (int q = 0; q < 6; ++q)
          if (d.name == scn[q] && d.vals.size() == 1) sc[q] = literal(d.vals[0]);
        if (d.name == "k0" && d.vals.size() == 1) k0 = (int)literal(d.vals[0]).ival;
      }
    }
  }
  if (k0_lit >= 0) k0 = k0_lit;
  if (form != F_SERIES) k0 = 0;
  if (npg < 1 || npg > EP_SERIES_MAX || (int)pg.size() != npg || k0 < 0 ||
      (form == F_EXPFIT && (int)ps.size() != npg))
    return put_err(err, cap, "BLOCK DATA of /" + common + "/: Npg, Pg, Ps or k0 unreadable or above EP_SERIES_MAX");
  for (int q = form == F_SERIES ? 0 : 2; q < 6; ++q)
    if (!sc[q].ok) return put_err(err, cap, std::string("BLOCK DATA of /") + common + "/: no " + scn[q]);
  ep_series s{};
  s.r_core = form == F_SERIES ? sc[0].hi : (form == F_EXPFIT ? x0.hi : 0.0);
  s.f_core = form == F_SERIES ? sc[1].hi : 0.0;
  s.r0 = sc[2].hi;
  s.aa = sc[3].hi;
  s.bb = sc[4].hi;
  s.cc = sc[5].hi;
  s.k0 = k0;
  s.n = npg;
  s.quad = (form == F_SERIES && quad) ? 1 : 0;
  for (int k = 0; k < npg; ++k) {
    const Lit L = literal(pg[k]);
    if (!L.ok) return put_err(err, cap, "Pg(" + std::to_string(k + 1) + ") of /" + common + "/ unreadable");
    s.c_hi[k] = L.hi;
    // a Real*8 Pg keeps the literal rounded to double; Real*16 keeps its kind
    s.c_lo[k] = (pg16 && L.kind == 16) ? L.lo : 0.0;
    if (!pg16 && L.kind == 16) s.c_hi[k] = L.hi + L.lo;
    if (form == F_EXPFIT) {
      const Lit M = literal(ps[k]);
      if (!M.ok) return put_err(err, cap, "Ps(" + std::to_string(k + 1) + ") of /" + common + "/ unreadable");
      s.c_lo[k] = M.hi + M.lo;
    }
  }
  *series = s;
  p->kind = form == F_SERIES ? EP_POT_SERIES : (form == F_EVENPOW ? EP_POT_EVENPOW : EP_POT_EXPFIT);
  p->series = series;
  return EP_OK;
}
