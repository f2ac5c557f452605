/*
 * oracle.h - CPU FP64 restatement of the reference hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the parity checker for the CUDA
 * library and the timed CPU baseline of bench.py; nothing in the product
 * links, loads or calls it.  Every routine follows the reference Fortran
 * line by line (citations at each function in oracle.cpp); the FFT is this
 * file's own FP64 mixed-radix transform, pinned against numpy.fft because
 * the reference delegates it to FFTW/MKL (not vendored).
 *
 * The API mirrors include/eff_pot.h with an oc_ prefix.
 */
#ifndef EP_ORACLE_H
#define EP_ORACLE_H
#include "../include/eff_pot.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oc_ctx oc_ctx;

int oc_create(const ep_config* cfg, oc_ctx** out);
int oc_destroy(oc_ctx* c);
const char* oc_last_error(const oc_ctx* c);
int oc_set_threads(int n);
int oc_potential_values(const ep_potential* p, const double* r, double* v, int n);

int oc_set_impurity_potentials(oc_ctx* c, const ep_potential* pi,
                               const ep_potential* sigma,
                               const ep_potential* plus);
int oc_set_impurity_tables(oc_ctx* c, const double* potpi, const double* potdel,
                           int npot, double delinter, double umax_sigma);
int oc_get_impurity_tables(oc_ctx* c, double* potpi, double* potdel, int* npot,
                           double* delinter);
int oc_set_impurity_potentials_d(oc_ctx* c, const ep_potential* pi,
                                 const ep_potential* sigma,
                                 const ep_potential* delta,
                                 const ep_potential* plus);
int oc_set_impurity_tables_d(oc_ctx* c, const double* potdel,
                             const double* potpidel, const double* potsigdel,
                             int npot, double delinter, double umax_pi,
                             double umax_sigma);
int oc_impurity_matrix_d(oc_ctx* c, double* m25);
int oc_set_impurity_state(oc_ctx* c, const double* rimp, const double* vimp,
                          const double* invar);
int oc_get_impurity_state(oc_ctx* c, double* rimp, double* vimp, double* aimp,
                          double* invar);

int oc_upload_psi(oc_ctx* c, const double* psi);
int oc_download_psi(oc_ctx* c, double* psi);
int oc_download_cfield(oc_ctx* c, int which, double* out);
int oc_download_field(oc_ctx* c, int which, double* out);

int oc_potenimp(oc_ctx* c);
int oc_poten(oc_ctx* c);
int oc_energy(oc_ctx* c, ep_energies* e);
int oc_forceimp(oc_ctx* c, double* F);
int oc_potinvar(oc_ctx* c, double* hinvar);
int oc_impurity_moments(oc_ctx* c, double* v6);
int oc_steprk(oc_ctx* c, double deltat);
int oc_steppc(oc_ctx* c, double deltat, ep_step_errors* err);
int oc_run(oc_ctx* c, int nsteps, double deltat, ep_run_stats* stats);
int oc_renormalize(oc_ctx* c, double* norm_before);

/* Building blocks exposed for unit tests. */
int oc_rfft3(int nx, int ny, int nz, const double* in, double* out_c);
int oc_irfft3(int nx, int ny, int nz, const double* in_c, double* out);
int oc_fd_weights(int npd, int id, double* w);  /* central row, unscaled */
int oc_deriv(const oc_ctx* c, int id, int axis, int is_complex,
             const double* f, double* df);
double oc_sinint(double x);                     /* Si(x) */
int oc_form_factors(oc_ctx* c, double* fvlj4, double* wcgk, double* kalfs);
double oc_bforce(int core, double eps, double sigma, double hc);

#ifdef __cplusplus
}
#endif
#endif
