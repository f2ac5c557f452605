// ep_dft4he3d - the DFT4He3d driver (DFT4He3d.f90:104-474) on the GPU solver.
//
// Reads the &input namelist from standard input (or the file named by the
// first argument), echoes it to DFT4He3d.namelist.read, reads the density or
// wave function of `filedenin` in the readenc formats (readenc.f90:83-176),
// and prints the first energy balance exactly as the reference does
// (potenimp, poten, energy, forceimp, potinvar; formats 6050 / 6060).  All
// arithmetic runs behind the C ABI (include/eff_pot.h).
//
// Beyond the reference (whose snapshot stops after that balance): niter > 0
// runs niter Hamming predictor-corrector steps after three Runge-Kutta-Gill
// steps, in imaginary time (timemode = 'imaginary', renormalised to n4) or
// real time, printing mu and the energy every `pener` steps, and writes
// `filedenout` in the printoutc layout (printoutc.f90:85-125; binary when
// iprint < 0).  Namelist keys the reference does not know: morse_de,
// morse_re, morse_alpha (selec_* = 'Morse'), potentials_source (the
// V_impur.f90 whose fits selec_* may name), precision ('fp64' | 'fp32'),
// refine (final FP64 steps of an FP32 run), timemode, iprint.
//
// `ep_dft4he3d --scan file...` (namelist on standard input) is the U*/U+
// post-processing scan of loop.sh / get_impurity_energy.sh as one job: the
// first energy balance of every saved wave function, printed as the table
// those scripts assemble (time, X-He centre-of-mass distance, Ekin(X), U*,
// U+, E_SO per file).
//
// The internal variables of the P (instate 0..2) and D (Lstate = 'D',
// instate 0..4) states are built as instates.f90 does in its default branch
// (ep_instates.h); Lexcite_state_fix gives the fixed P vectors, instate 5
// reads invar.dat, Ldiag_jz picks the state of given <Jz> in a j manifold.
// Pair potentials: Select_Pot by name through ep_select_pot (the closed
// forms built into the library; the inverse-power fits of V_impur.f90 read
// from the file named by the key potentials_source), 'Morse', or 'table'
// from a file of (r, V) rows.  Not built here: the Laverage_P_value /
// Lmixture / exciplex variants of instates.f90 (they sum eigenvectors, so
// they depend on EISPACK's phase convention).
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <fstream>
#include <future>
#include <iostream>
#include <thread>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/eff_pot.h"
#include "ep_fortran_io.h"
#include "ep_instates.h"

namespace {

const double kKtops = 7.63822291;  // ps K (DFT4He3d.f90:55)

struct Input {
  fio::Namelist nml;
  template <class T> T get(const char* k, T dflt) const;
};

template <> double Input::get<double>(const char* k, double d) const {
  auto it = nml.vars.find(k);
  return (it == nml.vars.end() || it->second.empty()) ? d : fio::to_real(it->second[0]);
}
template <> long Input::get<long>(const char* k, long d) const {
  auto it = nml.vars.find(k);
  return (it == nml.vars.end() || it->second.empty()) ? d : fio::to_int(it->second[0]);
}
template <> bool Input::get<bool>(const char* k, bool d) const {
  auto it = nml.vars.find(k);
  return (it == nml.vars.end() || it->second.empty()) ? d : fio::to_logical(it->second[0]);
}
template <> std::string Input::get<std::string>(const char* k, std::string d) const {
  auto it = nml.vars.find(k);
  return (it == nml.vars.end() || it->second.empty()) ? d : it->second[0];
}

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(' '), b = s.find_last_not_of(' ');
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

[[noreturn]] void stop(const std::string& msg, int code = 1) {
  std::fprintf(stdout, "%s\n", msg.c_str());
  std::fflush(stdout);
  std::exit(code);
}

void check(int st, ep_ctx* c, const char* what) {
  if (st != EP_OK) stop(std::string(what) + " failed: " + (c ? ep_last_error(c) : ep_create_error()), 2);
}

// selec_* -> ep_potential: 'Morse' (this project's selector), 'table'
// (tabulated by pair_tables below), everything else through Select_Pot by
// name (ep_select_pot: the built-in closed forms, and the inverse-power fits
// read from the reference's V_impur.f90 named by potentials_source).  *store
// holds a fit for as long as the potential is used.
ep_potential potential_of(const Input& in, const char* which, const char* dflt_sel, double dflt_rc,
                          double dflt_umax, ep_series* store) {
  const std::string key = std::string("selec_") + which;
  const std::string sel = trim(in.get<std::string>(key.c_str(), dflt_sel));
  ep_potential p{};
  p.r_cutoff = in.get<double>((std::string("r_cutoff_") + which).c_str(), dflt_rc);
  p.umax = in.get<double>((std::string("umax_") + which).c_str(), dflt_umax);
  if (sel == "table") {
    p.kind = EP_POT_NULL;
  } else if (sel == "Morse" || sel == "morse") {
    p.kind = EP_POT_MORSE;
    p.par[0] = in.get<double>("morse_de", 10.0);
    p.par[1] = in.get<double>("morse_re", 4.5);
    p.par[2] = in.get<double>("morse_alpha", 1.2);
  } else {
    const std::string src = trim(in.get<std::string>("potentials_source", ""));
    char err[512];
    if (ep_select_pot(sel.c_str(), p.r_cutoff, p.umax, src.empty() ? nullptr : src.c_str(), &p, store, err,
                      (int)sizeof err) != EP_OK)
      stop("selec_" + std::string(which) + "='" + sel + "': " + err +
           " (built in: 'null', 'Morse', '{Na,K,Rb,Cs}_plus_Koutselos', 'LI', 'NA', 'K', 'RB', 'CS', "
           "'Aziz_He', 'Ar_He', 'Xe_He', 'Ag_gs', 'Ag_Pi', 'Ag_Sig', 'Ba_gs', 'CH3I_0'..'CH3I_4', "
           "the graphene/TiO2/Au surface names; "
           "the inverse-power fits of V_impur.f90 with potentials_source = "
           "its path; any potential as 'table' with table_" + std::string(which) +
           " = a file of r (A), V (K) rows)");
  }
  return p;
}

// A pair potential given as a file of (r [A], V [K]) rows (comment lines
// starting with '#'), evaluated as Select_Pot does: umax inside r_cutoff,
// else the linear interpolant of the rows (the first / last value beyond
// them).
struct PairTable {
  std::vector<double> r, v;
  double r_cutoff = 0, umax = 0;
  double operator()(double x) const {
    if (x < r_cutoff) return umax;
    if (x <= r.front()) return v.front();
    if (x >= r.back()) return v.back();
    const size_t j = std::upper_bound(r.begin(), r.end(), x) - r.begin();
    const double f = (x - r[j - 1]) / (r[j] - r[j - 1]);
    return v[j - 1] + f * (v[j] - v[j - 1]);
  }
};

PairTable read_pair_table(const Input& in, const char* which) {
  const std::string fn = trim(in.get<std::string>((std::string("table_") + which).c_str(), ""));
  if (fn.empty()) stop(std::string("selec_") + which + "='table' needs table_" + which + " = a file name");
  std::ifstream f(fn);
  if (!f) stop("cannot open the potential table '" + fn + "'");
  PairTable t;
  t.r_cutoff = in.get<double>((std::string("r_cutoff_") + which).c_str(), 0.0);
  t.umax = in.get<double>((std::string("umax_") + which).c_str(), 0.0);
  fio::ListReader rd(f);
  rd.skip_comments('#');
  double a, b;
  while (rd.real(a) && rd.real(b)) {
    if (!t.r.empty() && !(a > t.r.back())) stop("potential table '" + fn + "': r must increase");
    t.r.push_back(a);
    t.v.push_back(b);
  }
  if (t.r.size() < 2) stop("potential table '" + fn + "' has fewer than two rows");
  return t;
}

// potenimpini (potenimpini.f90:12-55) for tabulated pi / sigma channels:
// V_Pi and V_Sigma - V_Pi on r_i = (i-1) rmax/(npot-1), npot = 100 max(n)+1,
// rmax = 4 max(xmax, ymax, zmax), ends repeated.
bool pair_tables(const Input& in, const ep_config& cfg, ep_ctx* ctx) {
  const bool tpi = trim(in.get<std::string>("selec_pi", "")) == "table";
  const bool tsg = trim(in.get<std::string>("selec_sigma", "")) == "table";
  const bool dst = cfg.state == EP_STATE_D;
  const bool tdl = dst && trim(in.get<std::string>("selec_delta", "")) == "table";
  if (!tpi && !tsg && !tdl) return false;
  if (!(tpi && tsg && (tdl || !dst)))
    stop(dst ? "selec_pi, selec_sigma and selec_delta must all be 'table' when one is"
             : "selec_pi and selec_sigma must both be 'table' when one is");
  const PairTable vp = read_pair_table(in, "pi"), vs = read_pair_table(in, "sigma");
  const int npot = 100 * std::max(cfg.nx, std::max(cfg.ny, cfg.nz)) + 1;
  const double rmax = 4.0 * std::max(cfg.xmax, std::max(cfg.ymax, cfg.zmax));
  const double del = rmax / (double)(npot - 1);
  if (dst) {  // potenimpini.f90:28-50: V_Delta, V_Pi - V_Delta, V_Sigma - V_Delta
    const PairTable vd = read_pair_table(in, "delta");
    std::vector<double> td(npot + 2), tpd(npot + 2), tsd(npot + 2);
    for (int i = 1; i <= npot; ++i) {
      const double r = (double)(i - 1) * del;
      td[i] = vd(r);
      tpd[i] = vp(r) - td[i];
      tsd[i] = vs(r) - td[i];
    }
    for (std::vector<double>* t : {&td, &tpd, &tsd}) {
      (*t)[0] = (*t)[1];
      (*t)[npot + 1] = (*t)[npot];
    }
    check(ep_set_impurity_tables_d(ctx, td.data(), tpd.data(), tsd.data(), npot, del, vp.umax, vs.umax), ctx,
          "impurity tables");
    return true;
  }
  std::vector<double> tp(npot + 2), td(npot + 2);
  for (int i = 1; i <= npot; ++i) {
    const double r = (double)(i - 1) * del;
    tp[i] = vp(r);
    td[i] = vs(r) - tp[i];
  }
  tp[0] = tp[1];
  tp[npot + 1] = tp[npot];
  td[0] = td[1];
  td[npot + 1] = td[npot];
  check(ep_set_impurity_tables(ctx, tp.data(), td.data(), npot, del, vs.umax), ctx, "impurity tables");
  return true;
}

// Echo of the namelist as read (DFT4He3d.f90:164-166).
void echo_namelist(const Input& in, const char* path) {
  std::ofstream os(path);
  os << "&INPUT\n";
  for (const std::string& k : in.nml.order) {
    os << " " << k << " =";
    for (const std::string& v : in.nml.vars.at(k)) os << " " << v;
    os << ",\n";
  }
  os << "/\n";
}

struct State {
  std::vector<double> psi;  // complex, interleaved
  std::vector<double> den;
  double rimp[3] = {0, 0, 0}, vimp[3] = {0, 0, 0};
  std::vector<double> invar = std::vector<double>(20, 0.0);
  bool have_invar = false;
  double time_ps = 0.0;                       // from the file's comment lines
  int p_instate = -1;                         // P state to build from the field moments
  int d_instate = -1;                         // D state to build from the field matrix
  int jz_ki = 0, jz_n = 0, jz_il = -1;        // Ldiag_jz: manifold and <Jz> index
  double auxn4 = 0, xc = 0, yc = 0, zc = 0;   // helium number and centre of mass
};

// readenc(mode) (readenc.f90:83-176); the grid of the file must match the
// namelist's (the reference does not check and would misread).
void readenc(const Input& in, const ep_config& cfg, int mode, const std::string& fn, State& s) {
  std::ifstream f(fn);
  if (!f) stop("readenc: cannot open '" + fn + "'");
  {  // the evolution time printoutc records in the comment lines (read by loop.sh)
    std::string l;
    while (std::getline(f, l) && !l.empty() && l[0] == '#') {
      const size_t k = l.find("Total evolution time");
      if (k != std::string::npos && l.find(':', k) != std::string::npos) {
        try {
          s.time_ps = fio::to_real(trim(l.substr(l.find(':', k) + 1)));
        } catch (const std::invalid_argument&) {
        }
      }
    }
    f.clear();
    f.seekg(0);
  }
  const size_t N = (size_t)cfg.nx * cfg.ny * cfg.nz;
  fio::ListReader r(f);
  r.skip_comments('#');
  double hdr[6];
  long n[3];
  bool ok = r.reals(hdr, 6) && r.integer(n[0]) && r.integer(n[1]) && r.integer(n[2]);
  if (!ok) stop("readenc: short header in '" + fn + "'");
  if (n[0] != cfg.nx || n[1] != cfg.ny || n[2] != cfg.nz)
    stop("readenc: the grid of '" + fn + "' differs from nx, ny, nz of the namelist");
  try {
    if (mode == 0) {
      bool limp = false;
      ok = r.logical(limp) && r.reals(s.rimp, 3);
      r.end_statement();
      s.den.resize(N);
      ok = ok && r.reals(s.den.data(), N);
    } else if (mode >= 1 && mode <= 3) {
      r.end_statement();
      ok = r.reals(s.rimp, 3);
      r.end_statement();
      ok = ok && r.reals(s.vimp, 3);
      r.end_statement();
      if (mode >= 2) {
        long nin = 0;
        ok = ok && r.integer(nin);
        r.end_statement();
        std::vector<double> iv(2 * (size_t)std::max(nin, 0L));
        ok = ok && r.complexes(iv.data(), (size_t)nin);
        r.end_statement();
        if (mode == 2) {  // P state: the first six (readenc.f90:130-137)
          const std::string lstate = trim(in.get<std::string>("lstate", "P"));
          const long keep = (nin < 10 || lstate == "P") ? std::min(nin, 6L) : std::min(nin, 10L);
          for (long k = 0; k < keep; ++k) {
            s.invar[2 * k] = iv[2 * k];
            s.invar[2 * k + 1] = iv[2 * k + 1];
          }
          s.have_invar = true;
        }
      }
      s.psi.resize(2 * N);
      ok = ok && r.complexes(s.psi.data(), N);
    } else {
      stop("ERROR READEN: This mode is still not programmed");
    }
  } catch (const std::invalid_argument& e) {
    stop("readenc: " + std::string(e.what()) + " in '" + fn + "'");
  }
  if (!ok) stop("readenc: '" + fn + "' ended early");
}

// The invar preparation that follows in readenc (readenc.f90:180-245).
void prepare_invar(const Input& in, State& s) {
  const long instate = in.get<long>("instate", -1L);
  if (instate < 0) stop("instate less than 0, still not programmed " + std::to_string(instate));
  if (instate == 5) {
    std::ifstream f("invar.dat");
    if (!f) stop("readenc: cannot open 'invar.dat'");
    fio::ListReader r(f);
    for (int k = 0; k < 10; ++k) {
      if (!r.complex(s.invar[2 * k], s.invar[2 * k + 1])) stop("readenc: 'invar.dat' ended early");
      r.end_statement();
    }
    return;
  }
  if (instate > 5) stop("instate value invalid " + std::to_string(instate));
  const std::string lstate = trim(in.get<std::string>("lstate", "P"));
  if (lstate != "P" && lstate != "D") stop("Lstate='" + lstate + "' is neither 'P' nor 'D'");
  if (in.get<bool>("ldiag_jz", false)) {  // instates.f90:228-300 (P), :613-690 (D)
    if (instate > (lstate == "D" ? 4 : 2)) stop("instate " + std::to_string(instate) + " has no Ldiag_jz state");
    const std::string ljz = trim(in.get<std::string>("ljz", ""));
    instates::jz_selection(lstate == "D", (int)instate, ljz, s.jz_ki, s.jz_n, s.jz_il);
    if (s.jz_il < 0) stop("Wrong Ljz value...:" + ljz);
    (lstate == "D" ? s.d_instate : s.p_instate) = (int)instate;
    return;
  }
  if (lstate == "D") {  // instates.f90:440-647, default branch
    s.d_instate = (int)instate;
    return;
  }
  if (in.get<bool>("lexcite_state_fix", false) && instate <= 2) {  // fixed P states, instates.f90:300-320
    std::fill(s.invar.begin(), s.invar.end(), 0.0);
    const int n = (int)instate + 1;
    for (int k = 0; k < n; ++k) s.invar[2 * (2 * k)] = 1.0 / std::sqrt((double)n);
    return;
  }
  for (const char* k : {"laverage_p_value", "lmixture", "lexciplex_state_fix"})
    if (in.get<bool>(k, false)) stop(std::string(k) + ": this instates.f90 variant is not built in this driver");
  if (instate > 2) stop("instate " + std::to_string(instate) + " has no P state (0..2)");
  s.p_instate = (int)instate;  // built from the field moments once the density is on the GPU
}

// instates.f90, P state: the moments of the impurity field on the current
// density give the 6x6 V + (Als/2) SO; its pair of eigenvectors selected by
// instate gives invar, then the impurity field is recomputed with it.
void build_p_state(ep_ctx* ctx, const ep_config& cfg, State& s) {
  if (s.d_instate >= 0) {  // D state: the 5x5 field matrix, MatDSO, instate's pair
    double M[25];
    check(ep_impurity_matrix_d(ctx, M), ctx, "impurity matrix");
    instates::d_state(M, cfg.als_d, s.d_instate, s.invar.data(), s.jz_ki, s.jz_n, s.jz_il);
    check(ep_set_impurity_state(ctx, s.rimp, s.vimp, s.invar.data()), ctx, "impurity state");
    check(ep_potenimp(ctx), ctx, "potenimp");
    return;
  }
  if (s.p_instate < 0) return;
  double m[6];
  check(ep_impurity_moments(ctx, m), ctx, "impurity moments");
  instates::p_state(m, cfg.als_p, s.p_instate, s.invar.data(), s.jz_ki, s.jz_n, s.jz_il);
  check(ep_set_impurity_state(ctx, s.rimp, s.vimp, s.invar.data()), ctx, "impurity state");
  check(ep_potenimp(ctx), ctx, "potenimp");
}

// The state of one input file as DFT4He3d prepares it: impurity start values
// from the namelist (DFT4He3d.f90:230-240, v in A/ps -> A K), readenc, the
// initial-velocity phases (:314-330, :414-432), the helium number and centre
// of mass.
void load_state(const Input& in, const ep_config& cfg, const std::string& file, State& s) {
  s.rimp[0] = in.get<double>("ximp", 0.0);
  s.rimp[1] = in.get<double>("yimp", 0.0);
  s.rimp[2] = in.get<double>("zimp", 0.0);

  double vimp0[3] = {in.get<double>("vximp", 0.0) * kKtops, in.get<double>("vyimp", 0.0) * kKtops,
                     in.get<double>("vzimp", 0.0) * kKtops};
  const double n4 = cfg.n4, mimp = cfg.mimpur;
  const double h2 = cfg.h2o2m4;
  double xl0[3];
  for (int k = 0; k < 3; ++k) {
    s.vimp[k] = vimp0[k];
    xl0[k] = -(vimp0[k] / kKtops) * mimp / (4.0 * n4);
  }
  const int mode = (int)in.get<long>("mode", 0L);
  readenc(in, cfg, mode, file, s);
  if (mode != 2) prepare_invar(in, s);
  const size_t N = (size_t)cfg.nx * cfg.ny * cfg.nz;
  const double hx = 2 * cfg.xmax / cfg.nx, hy = 2 * cfg.ymax / cfg.ny, hz = 2 * cfg.zmax / cfg.nz;
  auto X = [&](int i) { return -cfg.xmax + hx * i; };
  auto Y = [&](int i) { return -cfg.ymax + hy * i; };
  auto Z = [&](int i) { return -cfg.zmax + hz * i; };
  const bool vadd = in.get<bool>("l_v_aditional", false);
  if (mode == 0) {
    // psi = sqrt(den) exp(i k.r) with the initial-velocity phase (DFT4He3d.f90:414-432)
    double xlx = in.get<double>("xlamdax", 0.0), xly = in.get<double>("xlamday", 0.0),
           xlz = in.get<double>("xlamdaz", 0.0);
    const double xlam = in.get<double>("xlamda", 0.0);
    if (xlam != 0.0) xlz = xlam * kKtops / (2.0 * h2);
    s.psi.resize(2 * N);
    for (int iz = 0; iz < cfg.nz; ++iz)
      for (int iy = 0; iy < cfg.ny; ++iy)
        for (int ix = 0; ix < cfg.nx; ++ix) {
          const size_t p = ix + (size_t)cfg.nx * (iy + (size_t)cfg.ny * iz);
          const double a = X(ix) * xlx + Y(iy) * xly + Z(iz) * xlz, r = std::sqrt(s.den[p]);
          s.psi[2 * p] = r * std::cos(a);
          s.psi[2 * p + 1] = r * std::sin(a);
        }
  }
  if (vadd) {  // DFT4He3d.f90:314-330 (for mode 0 the phase is overwritten there by sqrt(den))
    for (int k = 0; k < 3; ++k) {
      s.vimp[k] += vimp0[k];
      xl0[k] = xl0[k] * kKtops / (2.0 * h2);
    }
    for (int iz = 0; iz < (mode == 0 ? 0 : cfg.nz); ++iz)
      for (int iy = 0; iy < cfg.ny; ++iy)
        for (int ix = 0; ix < cfg.nx; ++ix) {
          const size_t p = ix + (size_t)cfg.nx * (iy + (size_t)cfg.ny * iz);
          const std::complex<double> z(s.psi[2 * p], s.psi[2 * p + 1]);
          const double a = X(ix) * xl0[0] + Y(iy) * xl0[1] + Z(iz) * xl0[2];
          const std::complex<double> w = z * std::complex<double>(std::cos(a), std::sin(a));
          s.psi[2 * p] = w.real();
          s.psi[2 * p + 1] = w.imag();
        }
  }
  // helium count and centre of mass of the density used
  double auxn4 = 0, xc = 0, yc = 0, zc = 0;
  for (int iz = 0; iz < cfg.nz; ++iz)
    for (int iy = 0; iy < cfg.ny; ++iy)
      for (int ix = 0; ix < cfg.nx; ++ix) {
        const size_t p = ix + (size_t)cfg.nx * (iy + (size_t)cfg.ny * iz);
        const double d = s.psi[2 * p] * s.psi[2 * p] + s.psi[2 * p + 1] * s.psi[2 * p + 1];
        auxn4 += d;
        xc += X(ix) * d;
        yc += Y(iy) * d;
        zc += Z(iz) * d;
      }
  xc /= auxn4;
  yc /= auxn4;
  zc /= auxn4;
  auxn4 *= hx * hy * hz;
  s.auxn4 = auxn4;
  s.xc = xc;
  s.yc = yc;
  s.zc = zc;}

void printoutc(const std::string& fn, int iprint, long iter, double time_ps, const ep_config& cfg,
               const State& s, double deltatps) {
  const size_t N = (size_t)cfg.nx * cfg.ny * cfg.nz;
  const double hx = 2 * cfg.xmax / cfg.nx, hy = 2 * cfg.ymax / cfg.ny, hz = 2 * cfg.zmax / cfg.nz;
  const int ninvar = 10;
  if (iprint < 0) {
    std::ofstream os(fn, std::ios::binary);
    struct {
      double v[6];
      int n[3];
    } __attribute__((packed)) h{{cfg.xmax, cfg.ymax, cfg.zmax, hx, hy, hz}, {cfg.nx, cfg.ny, cfg.nz}};
    fio::write_record(os, &h, sizeof h);
    fio::write_record(os, s.rimp, sizeof s.rimp);
    fio::write_record(os, s.vimp, sizeof s.vimp);
    fio::write_record(os, &ninvar, sizeof ninvar);
    fio::write_record(os, s.invar.data(), (uint32_t)(s.invar.size() * sizeof(double)));
    fio::write_record(os, s.psi.data(), (uint32_t)(s.psi.size() * sizeof(double)));
    return;
  }
  // centre of mass of the helium (printoutc.f90:38-61)
  double xn = 0, xc = 0, yc = 0, zc = 0;
  for (int iz = 0; iz < cfg.nz; ++iz)
    for (int iy = 0; iy < cfg.ny; ++iy)
      for (int ix = 0; ix < cfg.nx; ++ix) {
        const size_t p = ix + (size_t)cfg.nx * (iy + (size_t)cfg.ny * iz);
        const double d = s.psi[2 * p] * s.psi[2 * p] + s.psi[2 * p + 1] * s.psi[2 * p + 1];
        xn += d;
        xc += (-cfg.xmax + ix * hx) * d;
        yc += (-cfg.ymax + iy * hy) * d;
        zc += (-cfg.zmax + iz * hz) * d;
      }
  std::ofstream os(fn);
  char buf[256];
  std::snprintf(buf, sizeof buf, "#  Density after %15ld iterations.\n#  Actual delatatps....:%20.10E\n", iter, deltatps);
  os << buf;
  std::snprintf(buf, sizeof buf, "#  Total evolution time(ps)...:%20.12E\n#  xcm,ycm,zcm:%16.8E%16.8E%16.8E\n", time_ps,
                xc / xn, yc / xn, zc / xn);
  os << buf;
  os << (iprint == 1 ? "#  Last printout of the run.\n" : iprint == 2 ? "#  Change of Paflov parameter.\n"
                                                                      : "#  Backup copy.\n");
  double h6[6] = {cfg.xmax, cfg.ymax, cfg.zmax, hx, hy, hz};
  fio::write_reals(os, h6, 6, 6);
  os << " " << cfg.nx << " " << cfg.ny << " " << cfg.nz << "\n";
  fio::write_reals(os, s.rimp, 3, 3);
  fio::write_reals(os, s.vimp, 3, 3);
  os << " " << ninvar << "\n";
  fio::write_complexes(os, s.invar.data(), 10, 2);
  fio::write_complexes(os, s.psi.data(), N, 2);
}

void balance(const ep_energies& e, double auxn4) {
  std::printf("\n\n    FIRST ENERGY BALANCE: \n\n");
  std::printf("    Number of particles ..........: %18.6f  \n", auxn4);
  std::printf("    TOTAL   energy (He) ..........: %18.6f K\n", e.etot4);
  std::printf("    Energy per particle (He) .....: %18.6f K\n", e.etot4 / auxn4);
  std::printf("    Kinetic energy (He) ..........: %18.6f K\n", e.ekin4);
  std::printf("    Lennard-Jones energy (He) ....: %18.6f K\n", e.elj4);
  std::printf("    Alpha_s term  energy (He) ....: %18.6f K\n", e.ealphas);
  std::printf("    Solid energy (He)  ...........: %18.6f K\n", e.esolid);
  std::printf("    Correlation energy   (He) ....: %18.6f K\n", e.ecor4);
  std::printf("    Impurity energy (X) ..........: %18.6f K\n", e.eimpu);
  std::printf("    Kinetic energy (X) ...........: %18.6f K\n", e.ekinx);
  std::printf("    Interaction energy (X*-He) ...: %18.6f K\n", e.eHeX);
  std::printf("    Interaction energy (X+-He) ...: %18.6f K\n", e.uplus);
  std::printf("    Spin-Orbit energy (X) ........: %18.6f K\n", e.eso);
  std::printf("    TOTAL ENERGY (He+X) ..........: %18.6f K\n\n", e.etot);
}

}  // namespace

int main(int argc, char** argv) {
  Input in;
  std::vector<std::string> scan;  // --scan file...: the U*/U+ scan of loop.sh
  if (argc > 1 && std::string(argv[1]) == "--scan") {
    for (int i = 2; i < argc; ++i) scan.push_back(argv[i]);
    if (scan.empty()) stop("--scan needs at least one wave-function file");
  }
  {
    std::string err;
    bool ok;
    if (argc > 1 && scan.empty()) {
      std::ifstream f(argv[1]);
      ok = f && fio::parse_namelist(f, "input", in.nml, err);
    } else {
      ok = fio::parse_namelist(std::cin, "input", in.nml, err);
    }
    if (!ok) stop("DFT3He3d. Error in input master file. " + err);
  }
  echo_namelist(in, "DFT4He3d.namelist.read");
  try {
    // time step consistency (DFT4He3d.f90:176-196)
    double deltat = in.get<double>("deltat", 0.0), deltatps = in.get<double>("deltatps", 0.0);
    if (deltat == 0.0) {
      if (deltatps == 0.0) stop("You must specify either Deltat (in kelvin) or Deltatps (in picosecond)");
      deltat = deltatps / kKtops;
    } else if (deltatps == 0.0) {
      deltatps = deltat * kKtops;
    } else if (deltatps != deltat * kKtops) {
      stop("Inconsistent deltat - deltatps");
    }
    std::printf(" Time step is %24.16E kelvins or %24.16E picoseconds.\n", deltat, deltatps);

    ep_config cfg;
    ep_config_init(&cfg);
    cfg.nx = (int)in.get<long>("nx", 64L);
    cfg.ny = (int)in.get<long>("ny", 64L);
    cfg.nz = (int)in.get<long>("nz", 64L);
    cfg.xmax = std::fabs(in.get<double>("xmax", 64.0));
    cfg.ymax = std::fabs(in.get<double>("ymax", 64.0));
    cfg.zmax = std::fabs(in.get<double>("zmax", 64.0));
    cfg.npd = (int)in.get<long>("npd", 13L);
    cfg.icon = (int)in.get<long>("icon", 13L);
    const std::string core = trim(in.get<std::string>("core4", "OT "));
    if (core == "OT") cfg.core = EP_CORE_OT;
    else if (core == "OTC") cfg.core = EP_CORE_OTC;
    else if (core == "OP") cfg.core = EP_CORE_OP;
    else stop(" I do not know how to work with the core: " + core);
    cfg.l = in.get<double>("l", cfg.l);
    cfg.cp4 = in.get<double>("cp4", cfg.cp4);
    cfg.cpp4 = in.get<double>("cpp4", cfg.cpp4);
    cfg.den4c = in.get<double>("den4c", cfg.den4c);
    cfg.alphas = in.get<double>("alphas", cfg.alphas);
    cfg.h2o2m4 = in.get<double>("h2o2m4", cfg.h2o2m4);
    cfg.eps4 = in.get<double>("eps4", cfg.eps4);
    cfg.sigma4 = in.get<double>("sigma4", cfg.sigma4);
    cfg.n4 = (double)in.get<long>("n4", 300L);
    cfg.mimpur = in.get<double>("mimpur", cfg.mimpur);
    cfg.fix_lambda = in.get<bool>("lfix_lambda", false) ? 1 : 0;
    cfg.als_p = in.get<double>("als_p", 0.0);
    cfg.als_d = in.get<double>("als_d", 0.0);
    {
      const std::string ls = trim(in.get<std::string>("lstate", "P"));
      if (ls != "P" && ls != "D") stop("Lstate='" + ls + "' is neither 'P' nor 'D'");
      cfg.state = ls == "D" ? EP_STATE_D : EP_STATE_P;
    }
    cfg.ev0 = in.get<double>("ev0", 0.0);
    cfg.z_exciplex_exclusion = in.get<double>("z_exciplex_exclusion", cfg.z_exciplex_exclusion);
    cfg.filter_exciplex_force = in.get<bool>("lfilter_exciplex_force", false) ? 1 : 0;
    cfg.impurity = EP_IMPURITY_MOVING;
    const std::string tm = trim(in.get<std::string>("timemode", "imaginary"));
    cfg.time_mode = (tm == "real") ? EP_REAL_TIME : EP_IMAGINARY_TIME;
    cfg.renormalize = cfg.time_mode == EP_IMAGINARY_TIME;
    const std::string prec = trim(in.get<std::string>("precision", "fp64"));
    cfg.precision = prec == "fp32" ? EP_FP32 : EP_FP64;

    // the pair potentials first: a name the registry does not know stops the
    // run before any device work
    ep_series fits[4] = {};
    const ep_potential ppi = potential_of(in, "pi", "Ba_plus_2D1", 1.05, 5.216077e4, &fits[0]);
    const ep_potential psg = potential_of(in, "sigma", "Ba_plus_2D0", 1.05, 9.674836e4, &fits[1]);
    const ep_potential ppl = potential_of(in, "plus", "Ba_plus_2D2", 1.05, 6.260015e4, &fits[2]);
    const ep_potential pdl = cfg.state == EP_STATE_D
                                 ? potential_of(in, "delta", "Ba_plus_2D2", 1.05, 6.260015e4, &fits[3])
                                 : ep_potential{};
    ep_ctx* ctx = nullptr;
    check(ep_create(&cfg, &ctx), nullptr, "ep_create");
    auto set_potentials = [&](ep_ctx* x) {
      if (cfg.state == EP_STATE_D)
        check(ep_set_impurity_potentials_d(x, &ppi, &psg, &pdl, &ppl), x, "impurity potentials");
      else
        check(ep_set_impurity_potentials(x, &ppi, &psg, &ppl), x, "impurity potentials");
      pair_tables(in, cfg, x);
    };
    set_potentials(ctx);

    if (!scan.empty()) {
      // loop.sh + get_impurity_energy.sh in one job: every file's first energy
      // balance, files parsed on host threads ahead of the GPU, one table line
      // per file with the columns loop.sh extracts
      std::printf("# time (ps)\tdX-HeCM (AA)\tEkin (K)\tU* (K)\t\tU+ (K)\t\tESO (K)\n");
      const size_t nf = scan.size();
      const size_t T = std::max<size_t>(1, std::min<size_t>(16, std::thread::hardware_concurrency()));
      std::vector<std::future<State>> fut(nf);
      size_t next = 0;
      auto launch = [&] {
        const size_t i = next++;
        fut[i] = std::async(std::launch::async, [&in, &cfg, &scan, i] {
          State st;
          load_state(in, cfg, scan[i], st);
          return st;
        });
      };
      while (next < nf && next < T) launch();
      for (size_t i = 0; i < nf; ++i) {
        State st = fut[i].get();
        if (next < nf) launch();
        check(ep_upload_psi(ctx, st.psi.data()), ctx, "upload psi");
        check(ep_set_impurity_state(ctx, st.rimp, st.vimp, st.invar.data()), ctx, "impurity state");
        check(ep_potenimp(ctx), ctx, "potenimp");
        build_p_state(ctx, cfg, st);
        check(ep_poten(ctx), ctx, "poten");
        ep_energies e{};
        check(ep_energy(ctx, &e), ctx, "energy");
        const double rcm = std::sqrt((st.rimp[0] - st.xc) * (st.rimp[0] - st.xc) +
                                     (st.rimp[1] - st.yc) * (st.rimp[1] - st.yc) +
                                     (st.rimp[2] - st.zc) * (st.rimp[2] - st.zc));
        std::printf("%.1f\t\t%f\t%f\t%f\t%f\t%f\n", st.time_ps, rcm, e.ekinx, e.eHeX, e.uplus, e.eso);
        std::fflush(stdout);
      }
      ep_destroy(ctx);
      return 0;
    }
    State s;
    load_state(in, cfg, trim(in.get<std::string>("filedenin", "he4.input.density")), s);
    const double auxn4 = s.auxn4, xc = s.xc, yc = s.yc, zc = s.zc;
    std::printf("\n\n     Title of the run: %s\n", in.get<std::string>("title", "Helium4 - 3dim.  ").c_str());

    check(ep_upload_psi(ctx, s.psi.data()), ctx, "upload psi");
    check(ep_set_impurity_state(ctx, s.rimp, s.vimp, s.invar.data()), ctx, "impurity state");
    check(ep_potenimp(ctx), ctx, "potenimp");
    build_p_state(ctx, cfg, s);
    check(ep_poten(ctx), ctx, "poten");
    ep_energies e{};
    check(ep_energy(ctx, &e), ctx, "energy");
    if (cfg.ev0 == 0.0 && !cfg.fix_lambda) {
      // Ev0 = eHeX + eso (DFT4He3d.f90:446): the phase reference of potinvar
      cfg.ev0 = e.eHeX + e.eso;
      std::vector<double> keep = s.psi;
      check(ep_destroy(ctx), nullptr, "ep_destroy");
      ctx = nullptr;
      check(ep_create(&cfg, &ctx), nullptr, "ep_create");
      set_potentials(ctx);
      check(ep_upload_psi(ctx, keep.data()), ctx, "upload psi");
      check(ep_set_impurity_state(ctx, s.rimp, s.vimp, s.invar.data()), ctx, "impurity state");
      check(ep_potenimp(ctx), ctx, "potenimp");
      check(ep_poten(ctx), ctx, "poten");
    }
    double F[3];
    check(ep_forceimp(ctx, F), ctx, "forceimp");
    if (!cfg.fix_lambda) {
      std::vector<double> hiv(20);
      check(ep_potinvar(ctx, hiv.data()), ctx, "potinvar");
    }
    std::printf("Number of He4 atoms%15.6E\n", auxn4);
    balance(e, auxn4);
    std::printf(" X-HE CoM distance: %24.16E\n",
                std::sqrt((s.rimp[0] - xc) * (s.rimp[0] - xc) + (s.rimp[1] - yc) * (s.rimp[1] - yc) +
                          (s.rimp[2] - zc) * (s.rimp[2] - zc)));

    const long niter = in.get<long>("niter", 0L);
    if (niter > 0) {
      const long pener = std::max(1L, in.get<long>("pener", 50L));
      const long refine = in.get<long>("refine", 0L);
      for (int k = 0; k < 3; ++k) check(ep_steprk(ctx, deltat), ctx, "steprk");
      long done = 3;
      std::printf("\n Iter     Mu(K)             Etot(K)            errHe\n");
      while (done < niter) {
        long chunk = std::min(pener, niter - done);
        if (cfg.precision == EP_FP32 && refine > 0 && done + chunk > niter - refine && done < niter - refine)
          chunk = niter - refine - done;
        if (cfg.precision == EP_FP32 && refine > 0 && done == niter - refine)
          check(ep_set_precision(ctx, EP_FP64), ctx, "set_precision");
        ep_run_stats st{};
        check(ep_run(ctx, (int)chunk, deltat, &st), ctx, "run");
        done += chunk;
        check(ep_poten(ctx), ctx, "poten");
        check(ep_energy(ctx, &e), ctx, "energy");
        std::printf("%6ld %18.10f %18.10f %12.4E\n", done, st.mu, e.etot, st.errHe);
      }
      check(ep_download_psi(ctx, s.psi.data()), ctx, "download psi");
      double aimp[3];
      check(ep_get_impurity_state(ctx, s.rimp, s.vimp, aimp, s.invar.data()), ctx, "impurity state");
      const int iprint = (int)in.get<long>("iprint", 1L);
      printoutc(trim(in.get<std::string>("filedenout", "he4.output.density")), iprint, niter,
                niter * deltatps, cfg, s, deltatps);
    }
    ep_destroy(ctx);
  } catch (const std::invalid_argument& e) {
    stop(std::string("DFT3He3d. Error in input master file: ") + e.what());
  }
  return 0;
}
