/* dmd_host.h -- host side of the GB300 DMD path: the reference's set-up and driver code restated in
 * C++ on top of the GPU ABI (dmd_gpu.h). All arrays are caller-owned; complex128 is interleaved.
 *
 * Reference interfaces mirrored (file:line in the reference tree):
 *   dmdh_parse_param     parameters::map_input / get (parameters.cpp:530-623)
 *   dmdh_load            electron::read_ldbd_size/kvec/ek/smat (electron.cpp:100-314),
 *                        electronphonon::get_brange/get_nkpair/read_ldbd_kpair/read_ldbd_eph
 *                        (ElectronPhonon.cpp:132-253), electronimpurity::read_ldbd_imp_P
 *                        (ElectronImpurity.cpp:3-49), lattice::read_ldbd_R (lattice.h:48-56),
 *                        parameters::read_jdftx (parameters.cpp:7-23); file sizes are checked as
 *                        check_file_size does (comm/myio.cpp:126-132) but reported as DMD_E_FILE
 *   dmdh_fermi           electron::fermi (electron.h:119-124)
 *   dmdh_dm_bpert        electron::compute_dm_Bpert_1st (electron.cpp:62-98) + singdenmat_k::init_dm
 *                        (DenMat.cpp:65-81)
 *   dmdh_H_BS            electron::set_H_BS (electron.cpp:19-42) + singdenmat_k::init_Hcoh (DenMat.cpp:7-28)
 *   dmdh_run             dm_dynamics_jdftx + dm_dynamics::evolve_gsl / evolve_euler
 *                        (main.cpp:38-84, DensityMatrix_Dynamics.h:177-225), S files as
 *                        ob_1dmk::measure writes them (observable.h:145-193, 368-404)
 *   dmdh_tau             ob_1dmk::measure_brange with ddmdt (observable.h:185-191, 297-336, 356-365, 392-401)
 *   dmdh_report_tau      dm_dynamics::report_tau (DensityMatrix_Dynamics.h:347-354, dt_tiny :236-238)
 */
#ifndef DMD_HOST_H
#define DMD_HOST_H
#include <stddef.h>
#include <stdint.h>

#include "dmd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dmdh_system dmdh_system;

/* scalar set-up values of a loaded system */
typedef struct dmdh_info {
  int32_t nk, nb_dm, bstart, bend, nb_total, nv_dm; /* nv_dm = max(nv - bStart_dm, 0) */
  int64_t nkpair;
  double nk_full, temperature, mu, prefac_eph, cell_size, cell_size_cmd, ob_prefac;
  double t0, tend, tstep;
  double ode_hstart, ode_hmin, ode_hmax, ode_epsabs;
  double Bpert[3], B[3];
  int32_t picture, expt, has_H, ode_method; /* ode_method: 0 rkf45, 1 euler, 2 rk4 */
  double eimp_fraction;
  double mue, muh;  /* chemical potentials of the equilibrium occupations (set_dm_eq), = mu otherwise */
  int32_t ddmdteq;  /* alg_ddmdteq: the equilibrium drift is subtracted from the scattering term */
  int32_t linear;   /* alg_linearize: P1, P2 of the system hold the linear operators Lscij, Lscji */
} dmdh_info;

/* Read param.in + ldbd_data/ from directory dir (the reference's working directory layout) and
 * perform DMD's set-up: band windows, chemical potential (carrier_density, electron.h:141-160),
 * occupations, folded P (scale_eph and |n_i V| * D1), initial density matrix, coherent Hamiltonian
 * and, with alg_ddmdteq, the equilibrium occupations of singdenmat_k::set_dm_eq (DenMat.cpp:97-225). */
int dmdh_load(const char* dir, dmdh_system** out);
void dmdh_free(dmdh_system* s);
const char* dmdh_error(void);
int dmdh_info_get(const dmdh_system* s, dmdh_info* info);
/* descriptor for dmd_create pointing into the loaded arrays (valid while s lives); with alg_sparseP
 * the descriptor asks for the sparse contraction (DMD_FLAG_SPARSE), which needs DMD_PREC_F64 */
int dmdh_desc(const dmdh_system* s, int32_t precision, int32_t device, dmd_desc* d);
/* copies of set-up arrays: dm0 (complex [nk][nb_dm^2]), f (double [nk][nb_dm]),
 * spin matrices (complex [nk][3][nb_dm^2]) */
int dmdh_get_dm0(const dmdh_system* s, double* dm0);
int dmdh_get_f(const dmdh_system* s, double* f);
int dmdh_get_smat(const dmdh_system* s, double* smat);
/* equilibrium occupations f_eq (double [nk][nb_dm]); DMD_E_ARG unless alg_ddmdteq */
int dmdh_get_f_eq(const dmdh_system* s, double* f_eq);
/* Per-handle set-up after dmd_create: attaches the e-e model of param.in (dmd_ee_attach); with
 * alg_ddmdteq, computes the equilibrium drift on the GPU
 * (electronphonon::compute_ddmdt_eq, evolve_eph.cpp:3-19, via dmd_evolve_driver at t = 0) and
 * installs it with dmd_set_ddmdt_eq; otherwise clears it. */
int dmdh_prepare(const dmdh_system* s, dmd_handle* h);
/* The e-e model of param.in (eeMode = Pee_update or Pee_fixed_at_eq with static screening) as the
 * descriptor dmdh_prepare passes to dmd_ee_attach (pointers into s); *on = 0 without one. */
int dmdh_ee_desc(const dmdh_system* s, dmd_ee_desc* ee, int32_t* on);

/* value of a param.in key after get()'s unit conversion; returns 0 and *found = 1 if present */
int dmdh_param(const dmdh_system* s, const char* key, double unit, double* value, int* found);

/* stand-alone set-up pieces */
int dmdh_fermi(double T, double mu, const double* e, double* f, size_t n);
int dmdh_dm_bpert(int32_t nk, int32_t nb, const double* smat, const double* e, const double* f, double T,
                  const double Bpert[3], double t0, int32_t picture, double* dm);
int dmdh_H_BS(int32_t nk, int32_t nb, const double* smat, const double B[3], const double* e, int32_t picture,
              double* H);

/* Fixed-step RK4 over the GSL-callback entry dmd_func, driven from the host the way GSL's stepper
 * drives func (DensityMatrix_Dynamics.h:358-369): nsteps steps of dt from t on the host state y (n
 * doubles, updated in place), 4 dmd_func calls per step (each copies its input to the device and
 * dydt back), stage combinations in host loops. work: 5 n doubles, caller-owned (page-locked memory
 * makes the copies direct). */
int dmdh_rk4_func(dmd_handle* h, double t, double dt, int64_t nsteps, double* y, size_t n, double* work);

/* Instantaneous lifetimes of one observable over bands [bstart, bend) of nb from the state dm and
 * its time derivative ddmdt at time t (complex [nk][nb^2] each; obs: complex [nk][nb^2], the
 * observable's matrices; e, f: double [nk][nb]; prefac: the observable's density prefactor):
 * out[0] = -S dt / (S(t + dt) - S) with S(t + dt) from dm + dt ddmdt (0 when dt = 0),
 * out[1] = -S / dS (without the precession term), out[2] = -S / (dS + precession term); atomic
 * units; the precession term is that of the interaction picture (0 in the Schrodinger picture). */
int dmdh_tau(int32_t nk, int32_t nb, const double* obs, const double* e, const double* f, const double* dm,
             const double* ddmdt, double t, double dt, int32_t picture, int32_t bstart, int32_t bend,
             double prefac, double out[3]);
/* DMD's report_tau for a loaded system at (t, y) with dydt = the right-hand side there (dmd_func):
 * appends one line per spin direction that param.in's Bpert selects (all three without Bpert) to
 * tau_s{x,y,z}_elec_tot.out (and _hole with valence bands) in dir, with dt = min(ode_hstart,
 * tstep / 10). */
int dmdh_report_tau(const dmdh_system* s, const char* dir, double t, const double* y, const double* dydt);

/* DMD's time loop on the GPU: evolve_gsl (rkf45), evolve_euler, or fixed-step RK4, writing
 * sx/sy/sz_elec_tot.out into dir every freq_measure-th step (the t0 line unless restart = 1; with
 * print_tot_band = 1 a column per band before the amplitude) and the
 * tau files (dmdh_report_tau) every freq_compute_tau-th step; with compute_tau_only = 1 only the t0
 * line and the tau files at t0. restart = 0 with a restart/ folder in dir is refused (DMD_E_ARG).
 * nsteps_max < 0 runs to tend. */
int dmdh_run(const char* dir, int32_t precision, int64_t nsteps_max);

#ifdef __cplusplus
}
#endif
#endif
