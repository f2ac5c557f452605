/*
 * eff_pot.h - C ABI of the GB300-native Orsay-Trento helium order-parameter
 * time-evolution hot path (libeffpot.so).
 *
 * The reference program keeps all state in Fortran modules and calls
 * argument-light external subroutines.  This ABI replaces those subroutines
 * one for one behind an opaque solver context; every array lives in HBM and
 * is owned by the context.  Host pointers passed in are borrowed for the
 * duration of the call only.  Arrays are column-major (x fastest), exactly
 * the Fortran layout (nx,ny,nz); complex arrays are interleaved (re,im)
 * doubles, i.e. Fortran complex(kind=8) / C double _Complex.
 *
 * Every entry point returns an ep_status; none aborts or traps.  The text of
 * the last failure is available from ep_last_error().
 */
#ifndef EFF_POT_H
#define EFF_POT_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference STOPs instead) ------------------------ */
typedef enum ep_status {
  EP_OK = 0,
  EP_ERR_INVALID_ARG = 1,   /* bad pointer / value                         */
  EP_ERR_BAD_GRID = 2,      /* grid size not a product of 2,3,5 or odd     */
  EP_ERR_CUDA = 3,          /* CUDA runtime error                          */
  EP_ERR_OOM = 4,           /* device allocation failed                    */
  EP_ERR_NONFINITE = 5,     /* NaN / Inf / non-positive density detected   */
  EP_ERR_STATE = 6,         /* call made in the wrong order                */
  EP_ERR_NO_DEVICE = 7,     /* no CUDA device visible                      */
  EP_ERR_UNSUPPORTED = 8,   /* option not built                            */
  EP_ERR_TIMEOUT = 9        /* a bounded device wait ran out               */
} ep_status;

/* ---- functional cores (DFT4He3d.f90:346-363) --------------------------- */
enum { EP_CORE_OT = 0, EP_CORE_OTC = 1, EP_CORE_OP = 2 };
/* ---- evolution kind: timec = 1 (imaginary) or i (real) ----------------- */
enum { EP_IMAGINARY_TIME = 0, EP_REAL_TIME = 1 };
/* ---- impurity treatment ------------------------------------------------- */
enum { EP_IMPURITY_NONE = 0, EP_IMPURITY_FIXED = 1, EP_IMPURITY_MOVING = 2 };
/* ---- arithmetic of the bulk field updates ------------------------------ */
/* Field arithmetic: FP64; FP32; double-float (each real an unevaluated sum
 * of two FP32 values, about 48 significant bits, computed on the FP32 pipes:
 * the FP64-class path that is not bound by the FP64 pipe). */
enum { EP_FP64 = 0, EP_FP32 = 1, EP_DFLOAT = 2 };
/* ---- boundary modes of the finite differences (newder.f ICON) ---------- */
enum { EP_ICON_PERIODIC = 8, EP_ICON_ZERO_OUTSIDE = 13 };
/* ---- electronic state of the impurity (Lstate, modules.f90:303) -------- */
enum { EP_STATE_P = 0, EP_STATE_D = 1 };

/*
 * Solver configuration.  ep_config_init() fills every field with the
 * defaults of the reference modules (modules.f90:15-19,116-135,187-199;
 * V_impur.f90:1-16; DFT4He3d.f90 namelist defaults).
 */
typedef struct ep_config {
  int nx, ny, nz;            /* grid points (even, factors 2,3,5)           */
  double xmax, ymax, zmax;   /* box half-widths, x(i) = -xmax + hx*(i-1)    */
  int npd;                   /* FD stencil points, odd 3..25 (default 13)   */
  int icon;                  /* EP_ICON_PERIODIC or EP_ICON_ZERO_OUTSIDE    */
  int core;                  /* EP_CORE_*                                   */
  /* Orsay-Trento functional (module he4 / lenard4)                         */
  double cp4, cpp4, den4c, alphas, l, den0s, h2o2m4;
  double C, beta, den_m;     /* solid penalty                               */
  double h4ot, h4op, eps4, sigma4, b4;
  /* evolution                                                              */
  int time_mode;             /* EP_IMAGINARY_TIME / EP_REAL_TIME            */
  int renormalize;           /* imaginary time: rescale psi to n4 per step  */
  double n4;                 /* number of helium atoms                      */
  /* classical impurity (module classicimp)                                 */
  int impurity;              /* EP_IMPURITY_*                               */
  double mimpur;             /* impurity mass in u (mAg_u = mimpur*mp_u)    */
  int fix_lambda;            /* Lfix_lambda: freeze the internal variables  */
  double als_p;              /* spin-orbit splitting, P state               */
  double ev0;                /* phase reference of potinvar                 */
  double z_exciplex_exclusion;
  int precision;             /* EP_FP64 / EP_FP32 / EP_DFLOAT               */
  int device;                /* CUDA device ordinal                         */
  int state;                 /* Lstate: EP_STATE_P (default) / EP_STATE_D   */
  double als_d;              /* spin-orbit splitting, D state (Als_D)       */
  int filter_exciplex_force; /* Lfilter_exciplex_force: F_z of forceimp only
                                over the planes beyond z_exciplex_exclusion
                                on the far side (potenimp.f90:211-248)      */
} ep_config;

/* Pair potentials (the Select_Pot registry, V_impur.f90:87-932, plus the
 * Morse selector this project adds).  r < r_cutoff -> umax.
 * EP_POT_KOUTSELOS: the He-M+ potentials 'Na_plus_Koutselos',
 *   'K_plus_Koutselos', 'Rb_plus_Koutselos', 'Cs_plus_Koutselos'
 *   (V_impur.f90:232-290,1704-1883), par[0] = 0, 1, 2, 3 for Na+, K+, Rb+, Cs+.
 * EP_POT_PATIL: Patil's alkali-He potentials 'LI', 'NA', 'K', 'RB', 'CS'
 *   (V_alka, V_impur.f90:1097-1192), par[0] = 0 .. 4 for Li .. Cs.
 * EP_POT_AZIZ: the He-He potential 'Aziz_He' (V_impur.f90:970-990).
 * EP_POT_TANG_TOENNIES: 'Ar_He', 'Xe_He' (V_impur.f90:2681-2782),
 *   par[0] = 0 Ar, 1 Xe.
 * EP_POT_SERIES: the inverse-power fits of V_impur.f90 ('Rb_gs_Fausto',
 *   'Ba_plus_gs', 'He2S_fci', 'LJ_OT', ...): the fit in *series.
 * EP_POT_AG: 'Ag_gs', 'Ag_Pi', 'Ag_Sig' (V_impur.f90:1038-1096),
 *   par[0] = 0, 1, 2.
 * EP_POT_BA_GS: 'Ba_gs' (V_impur.f90:1197-1210).
 * EP_POT_CH3I: 'CH3I_0' .. 'CH3I_4' (V_impur.f90:3079-3243), par[0] = l.
 * EP_POT_SURFACE: the He-surface and adatom potentials of the registry,
 *   functions of one distance like the rest: par[0] = 0 'Grafeno',
 *   1 'Grafeno_sin_dispersion', 2 'TiO2', 3 'Au', 4 'Au_TiO2', 5 'dAu_TiO2',
 *   6 'Ag_Graphene', 7 'dz_Ag_Graphene', 8 'Au_Graphene', 9 'dz_Au_Graphene'
 *   (V_impur.f90:939-965,2417-2554,3013-3030).
 * EP_POT_EVENPOW: 'Ba_plus_old_gs' (Func_Ba_plus_gs, V_impur.f90:1440-1497):
 *   aa x^2 + bb x + cc for x <= r0, sum_k c_hi[k-1] x^-(2k+4) beyond, in
 *   *series (r0, aa, bb, cc, n, c_hi).
 * EP_POT_EXPFIT: 'Cs_7s' (V_Cs_7s, V_impur.f90:1660-1702): x = max(r, x0);
 *   aa x^2 + bb x + cc for x <= r0, else Pg(1) e^(-Ps(1) x)/x + sum_{k>=2}
 *   Pg(k) x^(k-1) e^(-Ps(k) x), in *series (r_core = x0, r0, aa, bb, cc,
 *   n, c_hi = Pg, c_lo = Ps). */
enum {
  EP_POT_NULL = 0,
  EP_POT_MORSE = 1,
  EP_POT_KOUTSELOS = 2,
  EP_POT_PATIL = 3,
  EP_POT_AZIZ = 4,
  EP_POT_TANG_TOENNIES = 5,
  EP_POT_SERIES = 6,
  EP_POT_AG = 7,
  EP_POT_BA_GS = 8,
  EP_POT_CH3I = 9,
  EP_POT_SURFACE = 10,
  EP_POT_EVENPOW = 11,
  EP_POT_EXPFIT = 12
};

#define EP_SERIES_MAX 24
/* An inverse-power fit with a parabolic core (the Param_LJ_* blocks of
 * V_impur.f90), x in A, V in K:
 *   V = f_core                         x <= r_core
 *   V = |aa x^2 + bb x + cc|           x <= r0
 *   V = sum_{k=1..n} c_k x^-(k + k0)   beyond,
 * c_k = c_hi[k-1] + c_lo[k-1].  quad = 1 forms the sum in double-double
 * arithmetic (106-bit: the fits the reference sums in Real*16), 0 in
 * double. */
typedef struct ep_series {
  double r_core, f_core, r0, aa, bb, cc;
  int k0, n, quad;
  double c_hi[EP_SERIES_MAX], c_lo[EP_SERIES_MAX];
} ep_series;

typedef struct ep_potential {
  int kind;                  /* EP_POT_*                                    */
  double r_cutoff, umax;
  double par[4];             /* Morse: De (K), re (A), alpha (1/A);
                                Koutselos, Patil, Tang-Toennies: the atom   */
  const ep_series* series;   /* EP_POT_SERIES, _EVENPOW, _EXPFIT: the fit
                                (read during the call that takes the
                                potential, not kept)                        */
} ep_potential;

/* V(r_i), i < n, of p in the library's host arithmetic (no GPU needed): the
 * values potenimpini tabulates and energy() sums for U+. */
int ep_potential_values(const ep_potential* p, const double* r, double* v,
                        int n);

/* Select_Pot by name (V_impur.f90:87-932): selec as the namelist gives it,
 * with its r_cutoff and umax.  The closed forms are built in ('null',
 * '*_plus_Koutselos', 'LI' .. 'CS', 'Aziz_He', 'Ar_He', 'Xe_He', 'Ag_gs',
 * 'Ag_Pi', 'Ag_Sig', 'Ba_gs', 'CH3I_0' .. 'CH3I_4' and the ten surface
 * names of EP_POT_SURFACE); the
 * inverse-power fits (and the two fits of their own form, 'Ba_plus_old_gs'
 * and 'Cs_7s') are read from the reference's V_impur.f90 at
 * source_path (NULL: closed forms only): its Select_Pot chain names the
 * function, whose COMMON block names the BLOCK DATA with the coefficients.
 * Fortran literal kinds are kept: a constant without exponent letter or
 * with E is default REAL (rounded to binary32 before it is widened), D is
 * double, Q is Real*16.  *series receives the fit (p->series points to
 * it).  EP_ERR_INVALID_ARG with a message in err (cap bytes) for unknown
 * names, forms this library does not evaluate, or unreadable sources. */
int ep_select_pot(const char* selec, double r_cutoff, double umax,
                  const char* source_path, ep_potential* p, ep_series* series,
                  char* err, int cap);

/* Energies printed by DFT4He3d.f90:460-463 (module energies). */
typedef struct ep_energies {
  double etot, etot4, ekin4, elj4, ecor4, ealphas, esolid;
  double eimpu, ekinx, eHeX, uplus, eso;
  double n4;                 /* integral of the density                    */
} ep_energies;

/* Per-call diagnostics of one predictor-corrector step (steppc.f90:1). */
typedef struct ep_step_errors {
  double errHe, errimp, errvimp, erriv;
} ep_step_errors;

/* Statistics of ep_run (the time loop this project adds). */
typedef struct ep_run_stats {
  double errHe;              /* last step                                   */
  double mu;                 /* <psi|H|psi>/N of the last corrector         */
  double norm;               /* integral |psi|^2 before renormalisation     */
  int steps_done;
} ep_run_stats;

/* Field identifiers for ep_download_field. */
enum {
  EP_FIELD_DEN = 0, EP_FIELD_POT4 = 1, EP_FIELD_UIMP = 2, EP_FIELD_DENCG = 3,
  EP_FIELD_DELJ4 = 4, EP_FIELD_DXDEN = 5, EP_FIELD_DYDEN = 6, EP_FIELD_DZDEN = 7,
  EP_FIELD_FALFS = 8, EP_FIELD_INTXALF = 9, EP_FIELD_INTYALF = 10,
  EP_FIELD_INTZALF = 11, EP_FIELD_UALPHAS = 12, EP_FIELD_VPI = 13,
  EP_FIELD_DELTA = 14, EP_FIELD_SIGDEL = 15, EP_FIELD_COUNT = 16
};
/* The impurity fields by state (updatepoten, potenimp.f90:531-566):
 *   P: VPI = V_Pi(r), DELTA = (V_Sigma - V_Pi)(r) / r^2;
 *   D: DELTA = V_Delta(r), VPI = Pi_Del = (V_Pi - V_Delta)(r) / r^4,
 *      SIGDEL = Sig_Del = (V_Sigma - V_Delta)(r) / r^4 (D state only). */
/* Complex-field identifiers for ep_download_cfield. */
enum {
  EP_CFIELD_PSI = 0, EP_CFIELD_PSIOLD1 = 1, EP_CFIELD_PSIOLD2 = 2,
  EP_CFIELD_PSIOLD3 = 3, EP_CFIELD_HPSIOLD1 = 4, EP_CFIELD_HPSIOLD2 = 5,
  EP_CFIELD_PC = 6, EP_CFIELD_Q = 7
};

typedef struct ep_ctx ep_ctx;

/* Defaults of the reference modules. */
int ep_config_init(ep_config* cfg);

/* Replaces dimen() + fftini() + fforma() + initcg() + kalfs + Init_deriv_p
 * (dimen.f90:8, fft.f90:233, fforma.f90:11, initcg.f90:5,
 * DFT4He3d.f90:170,396-400).  Grid validity replaces tstgrid (widened to any
 * even size whose prime factors are 2, 3 and 5). */
int ep_create(const ep_config* cfg, ep_ctx** out);
int ep_destroy(ep_ctx* ctx);
const char* ep_last_error(const ep_ctx* ctx);
/* Text of the last ep_create failure (no context exists yet). */
const char* ep_create_error(void);

/* Impurity pair potentials; builds the 1-D tables of potenimpini
 * (potenimpini.f90:1-72).  plus = selec_plus used for U+ in energy(). */
int ep_set_impurity_potentials(ep_ctx* ctx, const ep_potential* pi,
                               const ep_potential* sigma,
                               const ep_potential* plus);
/* Raw tables potpi(0:npot+1), potdel(0:npot+1) with spacing delinter, for
 * callers that tabulate Select_Pot themselves (interpol module). */
int ep_set_impurity_tables(ep_ctx* ctx, const double* potpi,
                           const double* potdel, int npot, double delinter,
                           double umax_sigma);
/* D state (Lstate = 'D'): the three tables of potenimpini's D branch
 * (potenimpini.f90:28-50): potdel = V_Delta, potpidel = V_Pi - V_Delta,
 * potsigdel = V_Sigma - V_Delta at r_i = (i-1)*delinter.  umax of pi and
 * sigma are the values updatepoten stores at r <= 1e-3 (potenimp.f90:
 * 555-562). */
int ep_set_impurity_potentials_d(ep_ctx* ctx, const ep_potential* pi,
                                 const ep_potential* sigma,
                                 const ep_potential* delta,
                                 const ep_potential* plus);
int ep_set_impurity_tables_d(ep_ctx* ctx, const double* potdel,
                             const double* potpidel, const double* potsigdel,
                             int npot, double delinter, double umax_pi,
                             double umax_sigma);
/* rimp(3), vimp(3) (A, A*K), invar(10) complex as 20 doubles. */
int ep_set_impurity_state(ep_ctx* ctx, const double* rimp, const double* vimp,
                          const double* invar);
int ep_get_impurity_state(ep_ctx* ctx, double* rimp, double* vimp,
                          double* aimp, double* invar);

/* psi in, den = |psi|^2 (readenc.f90:104-105, DFT4He3d.f90:436). */
int ep_upload_psi(ep_ctx* ctx, const double* psi);
int ep_download_psi(ep_ctx* ctx, double* psi);
int ep_download_cfield(ep_ctx* ctx, int which, double* out);
int ep_download_field(ep_ctx* ctx, int which, double* out);

/* potenimp(rimp,invar) incl. updatepoten (potenimp.f90:1-189,515-632). */
int ep_potenimp(ep_ctx* ctx);
/* poten() incl. derden() and term_alfa() (poten.f90:5, term_alfa.f90:5). */
int ep_poten(ep_ctx* ctx);
/* energy() (energy.f90:12-202), eHeX/uplus accumulators zeroed. */
int ep_energy(ep_ctx* ctx, ep_energies* e);
/* The six density-weighted moments of the impurity field,
 * v6 = (Vx, Vy, Vz, Vxy, Vxz, Vyz), V_ij = sum den (V_Pi d_ij + Delta x_i x_j)
 * dxyz with x = r - rimp, from the fields of the last ep_potenimp: the
 * matrix of the P-state internal variables (instates.f90:123-147). */
int ep_impurity_moments(ep_ctx* ctx, double* v6);
/* D state: the 5x5 matrix m25 (row-major, symmetric) of the density-
 * weighted impurity field, sum den (Delta delta_ij + Pi_Del d_i d_j +
 * Sig_Del P_ij) dxyz over the d harmonics d_i of x = r - rimp, from the
 * fields of the last ep_potenimp: the MP + MS + sumVdel of potinvar and
 * instates (potenimp.f90:331-405, instates.f90:457-534). */
int ep_impurity_matrix_d(ep_ctx* ctx, double* m25);
/* forceimp(rimp,F) (potenimp.f90:193-258); for a moving impurity also
 * stores aimp = F / mAg_u, as every reference call site does next
 * (DFT4He3d.f90:454-455). */
int ep_forceimp(ep_ctx* ctx, double* F);
/* potinvar(rimp,invar,Hinvar), P and D states (potenimp.f90:261-492). */
int ep_potinvar(ep_ctx* ctx, double* hinvar);

/* steprk(deltat) (steprk.f90:1-191). */
int ep_steprk(ep_ctx* ctx, double deltat);
/* steppc(deltat,errHe,errimp,errvimp,erriv) (steppc.f90:1-230).  err may be
 * NULL, in which case the call does not wait for the device. */
int ep_steppc(ep_ctx* ctx, double deltat, ep_step_errors* err);
/* Time loop: nsteps steppc calls with imaginary-time renormalisation as
 * configured; stats may be NULL (no device wait). */
int ep_run(ep_ctx* ctx, int nsteps, double deltat, ep_run_stats* stats);
/* Renormalise psi to n4 now (imaginary time). */
int ep_renormalize(ep_ctx* ctx, double* norm_before);

/* Switch the arithmetic of the bulk fields between EP_FP32, EP_FP64 and
 * EP_DFLOAT, keeping the state: psi, the multistep history (psiold,
 * hpsiold, pc, q) and every field are converted and the next steps run in
 * the new precision.  FP32 -> FP64 (or -> EP_DFLOAT) starts the refinement
 * sweeps of a FP32 run; the first switch to a precision allocates its
 * buffers. */
int ep_set_precision(ep_ctx* ctx, int precision);
int ep_get_precision(const ep_ctx* ctx);

/* ---- batches: many independent instances (droplets / impurity positions,
 * grids of any size) advanced together, each on its own stream so their
 * kernels overlap on the GPU.  This replaces the one-process-per-density
 * scan of loop.sh / get_impurity_energy.sh. ------------------------------ */
typedef struct ep_batch ep_batch;
int ep_batch_create(const ep_config* cfgs, int n, ep_batch** out);
int ep_batch_destroy(ep_batch* b);
int ep_batch_size(const ep_batch* b);
/* The context of instance i (to upload psi, set the impurity, read
 * energies with the single-instance calls). */
ep_ctx* ep_batch_ctx(ep_batch* b, int i);
/* nsteps steppc steps of every instance (imaginary-time renormalisation as
 * configured); stats (n entries) may be NULL: then the call does not wait. */
int ep_batch_run(ep_batch* b, int nsteps, double deltat, ep_run_stats* stats);
int ep_batch_steprk(ep_batch* b, double deltat);
int ep_batch_set_precision(ep_batch* b, int precision);
int ep_batch_synchronize(ep_batch* b);
/* Events on the batch stream, which every ep_batch_run forks from and joins
 * back into: elapsed time of whole-batch work. */
int ep_batch_event_record(ep_batch* b, int slot);
int ep_batch_event_elapsed(ep_batch* b, int slot_a, int slot_b, double* ms);
long long ep_batch_kernel_launches(const ep_batch* b);

/* Autotuner: times the poten() pipeline on the current density for
 * candidate launch shapes of the FFT passes (lines and threads per CTA of
 * the X, Y and Z passes) and keeps the fastest.  Needs a density (after
 * ep_upload_psi).  report (cap bytes, may be NULL) receives a summary.
 * shapes[6] = {x lines, x threads, y lines, y threads, z lines, z threads}. */
int ep_autotune(ep_ctx* ctx, char* report, int cap);
int ep_get_launch_shapes(const ep_ctx* ctx, int* shapes);
int ep_set_launch_shapes(ep_ctx* ctx, const int* shapes);
/* Tunes each distinct grid of the batch once and gives the shapes to every
 * instance with that grid. */
int ep_batch_autotune(ep_batch* b);

/* Device synchronisation, timing and counters. */
int ep_synchronize(ep_ctx* ctx);
/* The CUDA stream all work of this context is launched on (cudaStream_t). */
void* ep_stream(ep_ctx* ctx);
/* Events on the context stream for device-side timing: record into one of
 * 16 slots; elapsed ms between two recorded slots (waits for the second). */
int ep_event_record(ep_ctx* ctx, int slot);
int ep_event_elapsed(ep_ctx* ctx, int slot_a, int slot_b, double* ms);
/* Kernel launches made by this context since creation (kernels replayed
 * from step graphs included). */
long long ep_kernel_launches(const ep_ctx* ctx);
/* Step graphs (default on = 1): ep_run / ep_batch_run capture one steppc
 * of a context (or of every context of a batch) with a fixed or no impurity
 * into a CUDA graph once and replay it, updating only the predictor /
 * corrector nodes to the rotated history buffers.  on = 2: whole periods of
 * the history rotation (10 steps) are captured once more and replayed with
 * no node updates (single steps realign the phase and take the remainder).
 * on = 0: every kernel is launched directly.  Results are bit-identical in
 * all three modes.  No reference counterpart (the reference loop calls
 * steppc per step, DFT4He3d.f90). */
int ep_set_step_graphs(ep_ctx* ctx, int on);
int ep_batch_set_step_graphs(ep_batch* b, int on);
/* Per-kernel-class event timing of every launch made while enabled. */
int ep_profile_enable(ep_ctx* ctx, int on);
/* Fills names (NUL-separated, cap bytes), per-class total ms and launch
 * counts; returns the number of classes in *n. */
int ep_profile_read(ep_ctx* ctx, char* names, int cap, double* ms,
                    long long* launches, int maxn, int* n);
/* Bytes of device memory held by the context. */
long long ep_device_bytes(const ep_ctx* ctx);

/*
 * Context-free density convolution that allocates nothing.  It has no
 * counterpart in the reference: it exists for callers that can't call
 * cudaMalloc (a host running inside a framework that owns the device memory
 * pool, or code that runs while a CUDA graph is captured).
 *
 *   d_out = IFFT( FFT(d_in) * d_kernel ) / (nx*ny*nz)
 *
 * the k-space product poten() applies with wcgk, fvlj4 and kalfs
 * (poten.f90:27-50).  d_in and d_out are real (nx,ny,nz) device arrays,
 * d_kernel the real half-spectrum table (nx/2+1,ny,nz) on the device;
 * stream is a cudaStream_t (NULL: the default stream).  The call is
 * asynchronous on that stream.
 *
 * Scratch lives in one fixed device array of the library (4.3 MB, held on
 * every GPU that loads the library until the process exits), so:
 *  - sizes are limited to (nx/2+1)*ny*nz <= 33*64*64 (a 64^3 grid) and axes
 *    of at most 320 points; larger grids return EP_ERR_UNSUPPORTED, odd nx
 *    or axes with prime factors other than 2, 3, 5 EP_ERR_BAD_GRID;
 *  - every call shares that array, so calls that overlap on the GPU (other
 *    streams, other host threads) race; serialise them;
 *  - the first call on a device looks the array up on that device (make it
 *    before any stream capture); it calls no cudaMalloc or cudaFree.
 */
int ep_convolve_noalloc(const double* d_in, const double* d_kernel,
                        double* d_out, int nx, int ny, int nz, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* EFF_POT_H */
