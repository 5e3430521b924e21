/*
 * jurassic_unified_library.h -- the reference's external GPU-library seam
 * on top of libjurassic_gb300.
 *
 * The reference's formod.c includes this header after jurassic.h when built
 * with UNIFIED=1 (formod.c:26-27) and calls jur_unified_init and
 * jur_unified_formod_multiple_packages (formod.c:72-73); its Makefile links
 * the library that provides them (Makefile:57-71).  This file declares those
 * two functions and, with the same conventions, drop-ins for kernel()
 * (jurassic.h:1006-1010, jurassic.c:4004-4099) and for the retrieval's
 * optimal_estimation (retrieval.c:448-749).  Built with the reference's own
 * jurassic.h (its ctl_t, atm_t, obs_t and dimension macros) and
 * include/jurassic_gb300.h; link -ljurassic_gb300 -lcudart.
 *
 * Errors end the program through the reference's ERRMSG, as the reference
 * does; the message is the library's (jgb_last_error).
 */
#ifndef JURASSIC_UNIFIED_LIBRARY_H
#define JURASSIC_UNIFIED_LIBRARY_H

#include "jurassic.h"
#include "jurassic_gb300.h"

/* Reads the control file with the reference's read_ctl and sets up the
   device context: control set, emissivity tables (TBLBASE/TBLFMT files,
   read_tbl's names), source functions from the filter files
   "<TBLBASE>_<nu>.filt" and, when FOV is set, the field of view.  Two
   control parameters of this library: JGB_PRECISION (1 = mixed, the
   default; 0 = FP64, rounding-level agreement with the reference) and
   JGB_DEVICE (CUDA device, default 0).  formod.c:72. */
void jur_unified_init(int argc, char *argv[]);

/* The same for a caller that holds a ctl_t already (read_ctl done). */
void jur_unified_init_ctl(const ctl_t *ctl, int device, int precision);

/* Forward model of n independent (atm, obs) packages in ONE batched call of
   the library (formod(), jurassic.c:3026-3071, of every package): obs[i]
   gets rad, tau and the tangent points (channels whose rad is NaN on entry
   stay NaN), atm[i].p the pressures after hydrostatic equilibrium when HYDZ
   is set.  unused must be NULL.  formod.c:73. */
void jur_unified_formod_multiple_packages(atm_t *atm, obs_t *obs, int n, void *unused);

/* kernel(ctl, atm, obs, k): finite-difference Jacobian k (m x n, the
   caller's gsl_matrix, row-major with its tda) of obs2y with respect to
   atm2x, every perturbation in one batched device launch sequence; obs and
   atm get the unperturbed forward model like kernel()'s own formod call.
   ctl must be the control set given to jur_unified_init; k's sizes must be
   the measurement and state sizes (ERRMSG otherwise). */
void jur_unified_kernel(ctl_t *ctl, atm_t *atm, obs_t *obs, gsl_matrix *k);

/* kernel() of n packages in one batched call; k[i] is package i's matrix. */
void jur_unified_kernel_multiple_packages(atm_t *atm, obs_t *obs, int n, gsl_matrix **k);

/* optimal_estimation(ret, ctl, obs_meas, obs_i, atm_apr, atm_i) of n
   packages, all submitted at once to the library's retrieval engine: from
   the a priori atm_apr[i] and the measurement obs_meas[i] (NaN = channel not
   used), atm_i[i] becomes the final atmosphere (x2atm of the final state on
   atm_apr[i], pressures of the final forward model) and obs_i[i] the
   measurement geometry with the final forward model.  cov (may be NULL, or
   hold NULL entries) receives the retrieval covariance of package i when
   ret->err_ana is set (matrix_cov_ret.tab).  The settings come as a jgb_ret:
   the retrieval's ret_t is private to retrieval.c, whose driver fills one
   from it field by field.  Writing the result files stays with the caller
   (write_atm, write_obs, write_matrix). */
void jur_unified_optimal_estimation_multiple_packages(const jgb_ret *ret, obs_t *obs_meas,
                                                      obs_t *obs_i, atm_t *atm_apr,
                                                      atm_t *atm_i, int n, gsl_matrix **cov);

/* Fills the jgb_ret *r from the retrieval settings ret_t *ret (read_ret,
   retrieval.c:753-804; ret_t, retrieval.c:32-112).  A macro, because ret_t
   is defined inside retrieval.c: it expands where ret_t is visible.  The
   arrays of r point into *ret, which must outlive r. */
#define JUR_UNIFIED_RET_FROM(ret, r)                                              \
  do {                                                                          \
    memset((r), 0, sizeof *(r));                                                \
    (r)->kernel_recomp = (ret)->kernel_recomp;                                  \
    (r)->conv_itmax = (ret)->conv_itmax;                                        \
    (r)->err_ana = (ret)->err_ana;                                              \
    (r)->conv_dmin = (ret)->conv_dmin;                                          \
    (r)->err_formod = (ret)->err_formod;                                        \
    (r)->err_noise = (ret)->err_noise;                                          \
    (r)->err_press = (ret)->err_press;                                          \
    (r)->err_press_cz = (ret)->err_press_cz;                                    \
    (r)->err_press_ch = (ret)->err_press_ch;                                    \
    (r)->err_temp = (ret)->err_temp;                                            \
    (r)->err_temp_cz = (ret)->err_temp_cz;                                      \
    (r)->err_temp_ch = (ret)->err_temp_ch;                                      \
    (r)->err_q = (ret)->err_q;                                                  \
    (r)->err_q_cz = (ret)->err_q_cz;                                            \
    (r)->err_q_ch = (ret)->err_q_ch;                                            \
    (r)->err_k = (ret)->err_k;                                                  \
    (r)->err_k_cz = (ret)->err_k_cz;                                            \
    (r)->err_k_ch = (ret)->err_k_ch;                                            \
    (r)->err_clz = (ret)->err_clz;                                              \
    (r)->err_cldz = (ret)->err_cldz;                                            \
    (r)->err_clk = (ret)->err_clk;                                              \
    (r)->err_sfz = (ret)->err_sfz;                                              \
    (r)->err_sfp = (ret)->err_sfp;                                              \
    (r)->err_sft = (ret)->err_sft;                                              \
    (r)->err_sfeps = (ret)->err_sfeps;                                          \
  } while (0)

/* One package: the drop-in for a single optimal_estimation call. */
void jur_unified_optimal_estimation(const jgb_ret *ret, obs_t *obs_meas, obs_t *obs_i,
                                    atm_t *atm_apr, atm_t *atm_i, gsl_matrix *cov);

/* The context created by jur_unified_init (for direct use of the C ABI),
   and its release. */
jgb_ctx *jur_unified_context(void);
void jur_unified_finalize(void);

#endif
