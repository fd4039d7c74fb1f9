/* dmd_gpu.h -- C ABI of the GB300 (sm_103a) Lindblad density-matrix right-hand side and steppers.
 *
 * Drop-in boundary for DMD's scattering/coherent RHS and its ODE stepping. Every entry point takes
 * plain pointers and sizes and returns an int status (DMD_OK = 0); nothing throws across the ABI.
 * complex128 arrays are interleaved (re, im) doubles; density matrices are k-major, then row-major
 * nb_dm x nb_dm; P operators are [nkpair][nb^4] with row (i1*nb+i2), column (i3*nb+i4).
 *
 * A handle owns one CUDA stream on one device and is not thread-safe.
 *
 * Reference interfaces replaced (file:line in the reference tree):
 *   dmd_create          electronphonon::set_eph / alloc_ephmat / read_ldbd_eph + add_scatt_contrib
 *                       (ElectronPhonon.cpp:3-14, 44-113, 209-304), singdenmat_k::init_Hcoh
 *                       (DenMat.cpp:7-28)
 *   dmd_func            GSL callback func(t, y, dydt, params) (DensityMatrix_Dynamics.h:358-369)
 *                       = dm_dynamics::compute (DensityMatrix_Dynamics.h:243-278)
 *   dmd_evolve_driver   electronphonon::evolve_driver (evolve_eph.cpp:21-32) -> evolve (:34-166)
 *   dmd_evolve_coh      singdenmat_k::evolve_coh (DenMat.cpp:29-55)
 *   dmd_set_ddmdt_eq    electronphonon::ddmdt_eq subtraction (evolve_eph.cpp:154-162)
 *   dmd_rk4             fixed-step RK4 over func (device resident; DMD's stepper loop
 *                       DensityMatrix_Dynamics.h:189-225 with the state kept on the GPU)
 *   dmd_rkf45_apply     gsl_odeiv2_driver_apply with gsl_odeiv2_step_rkf45 and the y_new control
 *                       (DensityMatrix_Dynamics.h:197-224)
 *   dmd_euler           evolve_euler_one_step + singdenmat_k::update_dm_euler
 *                       (DensityMatrix_Dynamics.h:227-234, DenMat.cpp:236-248)
 *   dmd_measure         ob_1dmk::measure("sx"/"sy"/"sz"...) totals (observable.h:301-366)
 *   dmd_set_state / dmd_get_state   copy_complex_from_real / copy_real_from_complex (comm/ODE.h:6-15)
 */
#ifndef DMD_GPU_H
#define DMD_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define DMD_OK 0
#define DMD_E_ARG 1        /* invalid argument or size */
#define DMD_E_NOMEM 2      /* device or host allocation failed */
#define DMD_E_FILE 3       /* input file missing or of the wrong size */
#define DMD_E_CUDA 4       /* CUDA runtime error */
#define DMD_E_TIMEOUT 5    /* a bounded device wait gave up */
#define DMD_E_NAN 6        /* non-finite value in the state */
#define DMD_E_STATE 7      /* call made in the wrong state */
#define DMD_E_NODEV 8      /* no CUDA device */
#define DMD_E_ODE 9        /* step size underflow (GSL_ENOPROG) or bad step direction */

/* arithmetic of the k-pair contraction */
#define DMD_PREC_F64 0     /* P complex128, native FP64 multiply-adds */
#define DMD_PREC_F64X 1    /* P and rho as (hi, lo) FP32 pairs: ~2^-46 products, double-FP32 sums */
#define DMD_PREC_F32 2     /* P stored complex64, FP32 products; rho enters as its deviation from f_ref */
#define DMD_PREC_BF16X2 3  /* P stored as bf16 hi + bf16 lo per component (8 bytes per complex), FP32
                              products; rho enters as its deviation from f_ref */

/* dmd_desc.flags */
#define DMD_FLAG_LINEAR 1u /* alg_linearize: P1, P2 hold Lscij, Lscji (ElectronPhonon_linear.cpp) and the
                              RHS is sum herm(L(t) (rho_k' - diag f_ref)) (evolve_eph_linear.cpp:3-51);
                              f_ref (the f_eq of the linearization) is required */
#define DMD_FLAG_ADJOINT 2u /* keep the pair operators in their stored order as well, for dmd_adjoint_rk4
                               (one extra copy of P on the device; single state only) */
#define DMD_FLAG_EE 4u      /* keep the operators P_eph (+ P_eimp) in their stored order and the
                               column-block map, for the e-e model (dmd_ee_attach); single state,
                               not linearized, not with DMD_FLAG_ADJOINT, operators given as arrays */
#define DMD_FLAG_SPARSE 8u  /* alg_sparseP / alg_Pin_is_sparse (evolve_eph.cpp:67-82, sparse_zgemm in
                               comm/sparse_matrix.cpp:6-40): keep only the elements with |P| > 1e-40
                               (the reference's default thr_sparseP; explicit zeros of sparse files are
                               dropped as well) and contract those; DMD_PREC_F64, a single state, not
                               with DMD_FLAG_LINEAR, DMD_FLAG_ADJOINT or DMD_FLAG_EE. It pays below
                               about a third of the elements stored (bench --sparse) */

/* pictures (alg.picture) */
#define DMD_PICTURE_INTERACTION 0
#define DMD_PICTURE_SCHRODINGER 1

typedef struct dmd_handle dmd_handle;

typedef struct dmd_desc {
  int32_t nk;            /* k-points (elec->nk) */
  int32_t nb_dm;         /* bands of the density matrix (elec->nb_dm), <= 8 */
  int32_t bstart, bend;  /* e-ph band window relative to bStart_dm; nb = bend - bstart in 1..4 */
  int64_t nkpair;        /* stored k-pairs */
  double prefac_eph;     /* 2*pi / nk_full (ElectronPhonon.h:61) */
  const double* e_dm;    /* [nk][nb_dm] band energies (Hartree) */
  const uint64_t* k1st;  /* [nkpair] first k of each pair (k1st <= k2nd) */
  const uint64_t* k2nd;  /* [nkpair] */
  const double* P1;      /* complex128 [nkpair][nb^4], scaled by scale_eph */
  const double* P2;      /* complex128 [nkpair][nb^4] */
  const double* P1_add;  /* optional complex128 [nkpair][nb^4] added as P1 += add_scale * P1_add */
  const double* P2_add;  /*   (ab-initio e-imp "D1" operators, ElectronImpurity.cpp:3-49) */
  double add_scale;      /* |n_i * V_cell| */
  const double* Hcoh;    /* optional complex128 [nk][nb_dm^2] coherent Hamiltonian (H_BS [+ H_Ez]) */
  int32_t picture;       /* DMD_PICTURE_* */
  int32_t expt;          /* 1: time-dependent P phases (alg.expt) */
  int32_t precision;     /* DMD_PREC_* */
  int32_t device;        /* CUDA device ordinal */
  uint32_t flags;        /* reserved, 0 */
  const double* f_ref;   /* optional [nk][nb_dm] reference occupations (e.g. f_dm) of the reduced-
                            precision forms: the contraction of diag(f_ref) is formed once in FP64 at
                            dmd_create and each evaluation contracts only rho - diag(f_ref) in FP32 */
  int32_t nrhs;          /* batched form: states that share P (0 or 1: a single state). With nrhs > 1 the
                            state of every call is nrhs consecutive [nk][nb_dm^2] states, stepped
                            together; precision DMD_PREC_F32 or DMD_PREC_BF16X2, nb = 2 or 4 */
  int32_t reserved;
} dmd_desc;

int dmd_create(const dmd_desc* desc, dmd_handle** out);
/* dmd_create with the pair operators read from DMD's files (ldbd_P1_lindblad.bin, ldbd_P2_lindblad.bin
 * and, optionally, the _D1 impurity files scaled by desc->add_scale; complex128 [nkpair][nb^4],
 * ElectronPhonon.cpp:209-253); desc->P1/P2/P1_add/P2_add are ignored. The column-block forms stream
 * the files in chunks through pinned buffers and convert them on the device (two chunks of 256 MB in
 * host memory at a time); the other forms read the files into host memory first. A file whose size
 * is not nkpair * nb^4 * 16 bytes gives DMD_E_FILE (check_file_size). */
int dmd_create_from_files(const dmd_desc* desc, const char* p1_path, const char* p2_path, const char* p1_add_path,
                          const char* p2_add_path, dmd_handle** out);
/* dmd_create_from_files for DMD's sparse operator input (alg.Pin_is_sparse, ElectronPhonon.cpp:240-247):
 * <prefix>_ns.bin (int32 count per pair), _s.bin (complex128 values), _i.bin and _j.bin (int32 row
 * and column in the nb^2 x nb^2 operator) for P1 and P2, plus optional dense additive files. The
 * operators are densified chunk by chunk on the host and converted on the device; the column-block
 * forms only (DMD_E_ARG otherwise). */
int dmd_create_from_sparse_files(const dmd_desc* desc, const char* sp1_prefix, const char* sp2_prefix,
                                 const char* p1_add_path, const char* p2_add_path, dmd_handle** out);
int dmd_destroy(dmd_handle* h);
const char* dmd_last_error(const dmd_handle* h);
const char* dmd_strerror(int status);

/* optional equilibrium drift subtracted from the scattering term, complex128 [nk][nb^2] */
int dmd_set_ddmdt_eq(dmd_handle* h, const double* ddmdt_eq);

/* RHS on host buffers (each call copies y in and the result out) */
int dmd_func(dmd_handle* h, double t, const double* y, double* dydt);
int dmd_evolve_driver(dmd_handle* h, double t, const double* dm, const double* dm1, double* ddmdt_eph);
int dmd_evolve_coh(dmd_handle* h, double t, const double* dm, double* ddmdt_coh);

/* device-resident state */
int dmd_set_state(dmd_handle* h, double t, const double* y);
int dmd_get_state(dmd_handle* h, double* t, double* y);
int dmd_rk4(dmd_handle* h, double dt, int64_t nsteps);
int dmd_euler(dmd_handle* h, double dt, int64_t nsteps);
/* One gsl_odeiv2_driver_apply call from the current time to t1. *hstep carries the driver's step
 * size between calls (initialise it with hstart). nfev (optional) receives the RHS evaluations. */
int dmd_rkf45_apply(dmd_handle* h, double t1, double* hstep, double hmin, double hmax, double epsabs,
                    double epsrel, int64_t* nfev);

/* observables: slot 0..7 holds complex128 [nk][nb_dm^2] matrix elements (e.g. s_z), the occupations
 * f [nk][nb_dm] and the prefactor 1/(nk_full*cell_size_cmd); measure returns (tot, tot_amp) over
 * bands [bstart, bend) of the density matrix. */
int dmd_set_observable(dmd_handle* h, int slot, const double* obs, const double* f, double prefac);
int dmd_measure(dmd_handle* h, int slot, int bstart, int bend, double* tot, double* tot_amp);
/* batched form: the totals of every state (tot, tot_amp: nrhs doubles each) */
int dmd_measure_batch(dmd_handle* h, int slot, int bstart, int bend, double* tot, double* tot_amp);

/* counters: kernel launches issued by this handle since creation */
int dmd_launch_count(const dmd_handle* h, int64_t* launches);
/* No counterpart in the reference: device bytes of the stored k-pair operators in the handle's
 * layout (what one contraction pass streams from HBM) */
int dmd_pair_bytes(const dmd_handle* h, int64_t* bytes);

/* No counterpart in the reference (DMD computes no gradients). Reverse mode of nsteps fixed-step RK4
 * steps of size dt from (t0, y0) (y0: 2 nk nb_dm^2 doubles, as dmd_func's y), for the objective
 * J = sum_i obs_weight[i] * S(t0 + obs_step[i] dt), S = the total of observable `slot` over bands
 * [bstart, bend) as dmd_measure returns it. When the stage inputs and forward sums of all steps fit
 * in 40 % of the free device memory the forward pass keeps them all; otherwise it keeps the state
 * every `checkpoint` steps and the backward pass recomputes each stretch from its checkpoint (also
 * when the environment sets DMD_ADJ_KEEP_ALL=0). The
 * adjoint runs through the exact discrete RK4 map with the transposed k-pair contraction. Outputs (any
 * may be null): s_obs [nobs] the observed totals, dJdP [2][nkpair][nb^4] complex (dJ/dRe P, dJ/dIm P
 * interleaved, P1 then P2, of the folded operators P = P + add_scale P_add), dJdy0 [2 nk nb_dm^2]
 * (the gradient with respect to y0's real and imaginary parts). Requires DMD_FLAG_ADJOINT, a single
 * state, no linearized form and no equilibrium drift; obs_step ascending in [0, nsteps]. The
 * handle's own state and time are left unchanged. */
int dmd_adjoint_rk4(dmd_handle* h, double t0, const double* y0, double dt, int64_t nsteps, int64_t checkpoint,
                    int slot, int bstart, int bend, int64_t nobs, const int64_t* obs_step,
                    const double* obs_weight, double* s_obs, double* dJdP, double* dJdy0);
/* No counterpart in the reference (its operators are fixed after set-up, apart from the e-e model).
 * P += scale * P_add on the device for both operators (complex128 [nkpair][nb^4] each, in the stored
 * pair order), then the handle's stored form is rebuilt from them: how central differences of a
 * trajectory with respect to an operator set's scale are taken without a second copy of P. Needs a
 * handle made with DMD_FLAG_ADJOINT (or DMD_FLAG_EE before an e-e model is attached), nb = 2 or 4, a
 * single state, not linearized. Synchronous; the state and time are unchanged. */
int dmd_add_operators(dmd_handle* h, const double* P1_add, const double* P2_add, double scale);
/* wait for the handle's stream */
int dmd_sync(dmd_handle* h);

/* page-locked host buffers for the host-buffer calls (cudaHostAlloc / cudaFreeHost) */
int dmd_pinned_alloc(size_t bytes, void** out);
int dmd_pinned_free(void* p);

/* CUDA-event timing on the handle's stream: op 0 records the start event, op 1 records the stop
 * event, waits for it and returns the elapsed milliseconds in *ms */
int dmd_timer(dmd_handle* h, int op, double* ms);

/* per-kernel profiling: while on, steppers launch kernels one by one (no graph) with CUDA events
 * around each launch; dmd_profile_get returns the accumulated device time and launch count of
 * kernel class 0 (prep), 1 (k-pair contraction), 2 (finish/stepper update), 3 (other) */
int dmd_set_profiling(dmd_handle* h, int on);

/* No counterpart in the reference. A group steps several handles of one device together (separate
 * P sets: temperatures, materials, uneven nk), each possibly batched: dmd_group_rk4 advances every
 * member by nsteps RK4 steps of size dt from its own time, one CUDA graph launch per step in which
 * each member's kernels form a parallel branch. Members keep their own state, observables and
 * errors; a member must not be stepped on its own while the group steps it. */
typedef struct dmd_group dmd_group;
int dmd_group_create(dmd_handle* const* members, int n, dmd_group** out);
int dmd_group_rk4(dmd_group* g, double dt, int64_t nsteps);
int dmd_group_destroy(dmd_group* g);

/* No counterpart in the reference. Self-test of the bounded waits that every bulk-copy pipeline
 * uses: a kernel waits on an mbarrier phase that nothing completes, gives up after `polls` polls and
 * raises the device error flag; *status receives what the steppers would return then
 * (DMD_E_TIMEOUT) and the call checks that the context still runs a kernel afterwards. */
int dmd_selftest_wait_timeout(int device, uint32_t polls, int* status);

/* No counterpart in the reference. Measured fused multiply-add throughput of the device (fp64 = 1:
 * FP64, 0: FP32) in TFLOP/s (2 flops per FMA), from CUDA-event-timed launches of a kernel whose
 * threads run 8 independent FMA chains (best of three after a warm-up launch, ~20 ms each). The
 * FP64 figure is the ceiling of the plain FP64 contraction, whose work is FP64 multiply-adds. */
int dmd_peak_fma(int device, int fp64, double* tflops);

/* ---- e-e scattering rebuilt from the density matrix (eeMode = Pee_update) ------------------------
 * The e-e operators P_ee(rho) of elecelec_model::calc_P (ElecElec_Model.h:186-262) for every stored
 * k-pair, with the static screened Coulomb interaction of coulomb_model::vq (Coulomb_Model.h:632-660),
 * are added to the handle's operators: P = P_eph (+ P_eimp) + scale P_ee (ElectronPhonon.cpp:44-113).
 * dmd_ee_attach replaces electronphonon::set_eph's e-e contribution (ElectronPhonon.cpp:12: P_ee at the
 * equilibrium occupations with the set-up screening density); dmd_ee_update replaces reset_scatt's
 * e-e update (ElectronPhonon.cpp:15-42, called by update_scatt_outside, DensityMatrix_Dynamics.h:290-
 * 299) on the handle's state; with every_rhs the update runs on the device before every RHS
 * evaluation, inside the captured RK4 step as well (update_scatt_inside, DensityMatrix_Dynamics.h:
 * 280-289). Requires a handle made with DMD_FLAG_EE and nb = 2 or 4. */
#define DMD_SCREEN_UNSCREENED 0 /* clp.scrFormula = "unscreened" */
#define DMD_SCREEN_DEBYE 1      /* "debye" */
#define DMD_SCREEN_BECHSTEDT 2  /* "Bechstedt" */
#define DMD_SCREEN_RPA 3        /* "RPA": the q table of calc_qscr2_static_RPA (Coulomb_Model.h:690-736,
                                   819-826) from f and U, built at attach (with the plasmon-pole
                                   terms of calc_vq_RPA, :780-874, when dynamic) */

typedef struct dmd_ee_desc {
  int32_t nbw;              /* Wannier functions (elec->nb_wannier) */
  const double* kvec;       /* [nk][3] fractional k-points (ldbd_kvec.bin) */
  int32_t kmesh[3];         /* elec->kmesh */
  const double* U;          /* complex128 [nk][nbw][nb]: the window's columns of U (ldbd_Umat.bin) */
  const double* f;          /* [nk][nb] window occupations of the set-up (coul_model->f; also the
                               occupations of the static RPA screening, which later updates keep) */
  double GGT[9];            /* reciprocal metric, row-major (lattice.h:41-42) */
  double cell_size;         /* latt->cell_size */
  double nk_full;           /* elec->nk_full */
  double temperature;       /* Hartree */
  double eps_background;    /* clp.eps (epsilon_background) */
  double meff;              /* clp.meff (meff_screening) */
  int32_t formula;          /* DMD_SCREEN_* */
  double nfree;             /* screening density of the set-up (clp.nfreetot), bohr^-dim */
  int32_t update_screening; /* clp.update: the density from rho's diagonal at each update */
  int32_t nv;               /* window bands below nv are valence (holes) in that density */
  double degauss;           /* eep.degauss (degauss_ee) */
  double ethr;              /* energy-conservation window: degauss * ndegauss (param) */
  int32_t antisymmetry;     /* eep.antisymmetry: the exchange term */
  double scale;             /* scale_ee */
  int32_t every_rhs;        /* freq_update_ee_model < 0: update before every RHS evaluation */
  /* dynamic screening (clp.dynamic, Coulomb_Model.h:572-575, 780-874, 659-687; ElecElec_Model.h:
   * 81-138): 0 static, 1 the plasmon-pole approximation ("ppa", DMD_SCREEN_RPA only). The
   * interaction of each matrix element is vq(q, w) at its energy transfer, the exchange factor
   * vq(k1 - k4, w_ex) applied as the reference applies it (to the direct term) */
  int32_t dynamic;
  int32_t ppa_gn;           /* clp.ppamodel: 1 "gn" (Godby-Needs), 0 "hl" (Hybertsen-Louie) */
  double eppa;              /* clp.eppa (eppa_screening, Hartree); 0: the plasma frequency of nfree */
  double smearing;          /* clp.smearing (smearing_screening, Hartree); <= 0: 0.5 T, except for gn */
  int32_t two_freqs;        /* clp.dynamic_screening_ee_two_freqs */
} dmd_ee_desc;

int dmd_ee_attach(dmd_handle* h, const dmd_ee_desc* ee);
/* Update from the handle's state at its time (set_state / after stepping). */
int dmd_ee_update(dmd_handle* h);
/* The e-e source of the linearized operators (electronphonon::set_Lsc's add_Lsc_contrib("ee"),
 * ElectronPhonon_linear.cpp:17-22, 44-100): for every stored pair, P_ee at the occupations f_eq
 * ([nk][nb] window; elecelec_model::calc_P with f = f_eq, ElecElec_Model.h:186-262) and the terms of
 * calc_P3P4 and calc_P5P6 (ElecElec_Model_linear.cpp:3-112; P3, P4 zero with the exchange term), with
 * the screening of density nfree (the set-up density, or coulomb_model::init(f_eq)'s when the model
 * updates it) and the attached model's static RPA table. Outputs complex128 [npair][nb^4] each
 * (prefactor included, scale_ee not; any may be NULL). Needs an attached e-e model; the handle's
 * own operators and screening are left as they were. */
int dmd_ee_linear_terms(dmd_handle* h, const double* f_eq, double nfree, double* P1ee, double* P2ee, double* P3,
                        double* P4, double* P5, double* P6);
/* The last P_ee (complex128 [npair][nb^4] each, prefactor included, scale not; either may be NULL)
 * and the screening density it used (may be NULL). */
int dmd_ee_read(dmd_handle* h, double* P1ee, double* P2ee, double* nfree);

/* No counterpart in the reference. Shape autotuner: times every compiled shape variant of the
 * handle's contraction (f64x, nb = 2: lines per stage, ring depth, CTAs per SM; f64, nb = 2: forward
 * sums reduced over the warp or added in L2, CTAs per SM (1 by default); CUDA-core batches:
 * states per warp; tensor-core batches: pipeline stages, 2 of which leave room for 2 CTAs per SM) on
 * `evals` right-hand-side evaluations of the current device state (CUDA events,
 * after one warm-up evaluation each), keeps the fastest and returns its index in *chosen (0 when
 * the handle's form has a single shape). The state is not modified. */
int dmd_autotune(dmd_handle* h, int evals, int* chosen);
int dmd_profile_get(const dmd_handle* h, int kernel_class, double* total_ms, int64_t* launches);

/* No counterpart in the reference. The scattering right-hand side of dmd_evolve_driver for callers
 * that cannot allocate device memory (code running inside a CUDA graph capture, host frameworks
 * whose memory pools own the device, plug-ins handed device pointers but no allocator). Every
 * pointer is a caller-owned DEVICE buffer: k1st/k2nd uint64 [nkpair], P1/P2 complex128
 * [nkpair][nb^4] in DMD's layout, e_dm [nk][nb_dm], dm and ddmdt_eph complex128 [nk][nb_dm^2];
 * stream is a cudaStream_t (NULL for the default stream). Nothing is allocated: the scratch lives in
 * a static device array of 16 MiB that every GPU loading this library keeps until exit, which
 * limits nk * (bend - bstart)^2 to 262144 (DMD_E_ARG above that). The first call on a device looks
 * up the array's device address and should come before any stream capture; a device reset after it
 * is not supported. All calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller. Pairs whose indices fall outside [0, nk) are skipped. The call is
 * asynchronous on `stream`; a CUDA error already pending when it is made gives DMD_E_CUDA and is
 * left pending for the caller. */
int dmd_evolve_driver_noalloc(int32_t nk, int32_t nb_dm, int32_t bstart, int32_t bend, int64_t nkpair,
                              const uint64_t* k1st, const uint64_t* k2nd, const double* P1, const double* P2,
                              const double* e_dm, double prefac_eph, int32_t expt, double t, const double* dm,
                              double* ddmdt_eph, void* stream);

#ifdef __cplusplus
}
#endif
#endif
