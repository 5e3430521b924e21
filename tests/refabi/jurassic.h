/*
 * Reference-layout declarations for running the binding
 * (jurassic_gb300/binding/jurassic_unified_library.c) where the reference
 * tree is absent (the GPU machine).  TEST INFRASTRUCTURE ONLY.
 *
 * The binding is written against the reference's jurassic.h; this header
 * restates the parts of that interface the binding uses: the dimension
 * macros, ERRMSG, and the value layouts of ctl_t, atm_t and obs_t
 * (jurassic.h:488-538, 541-675, 734-775) with the same member order and
 * types, so that packed structs look the same to the binding.
 * tests/test_abi.py compiles a probe against this header and against the
 * reference's own with the same dimensions and requires identical sizes and
 * member offsets.
 */
#ifndef JGB_REFABI_JURASSIC_H
#define JGB_REFABI_JURASSIC_H

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <gsl/gsl_matrix.h>

/* dimensions (compile-time, as in the reference) */
#ifndef NCL
#define NCL 8
#endif
#ifndef ND
#define ND 128
#endif
#ifndef NG
#define NG 8
#endif
#ifndef NP
#define NP 256
#endif
#ifndef NR
#define NR 256
#endif
#ifndef NSF
#define NSF 8
#endif
#ifndef NW
#define NW 4
#endif
#ifndef LEN
#define LEN 10000
#endif
#ifndef NLOS
#define NLOS 4096
#endif
#ifndef NSHAPE
#define NSHAPE 20000
#endif
#ifndef TBLNP
#define TBLNP 41
#endif
#ifndef TBLNT
#define TBLNT 30
#endif
#ifndef TBLNU
#define TBLNU 320
#endif

/* error exit with position, like the reference's */
#define ERRMSG(...)                                                  \
  do {                                                               \
    fprintf(stderr, "\nError (%s, %s, l%d): ", __FILE__, __func__, __LINE__); \
    fprintf(stderr, __VA_ARGS__);                                    \
    fprintf(stderr, "\n\n");                                         \
    exit(EXIT_FAILURE);                                              \
  } while (0)

/* one atmosphere: level arrays, then cloud and surface scalars */
typedef struct {
  int np;
  double time[NP], z[NP], lon[NP], lat[NP], p[NP], t[NP];
  double q[NG][NP];
  double k[NW][NP];
  double clz, cldz;
  double clk[NCL];
  double sfz, sfp, sft;
  double sfeps[NSF];
} atm_t;

/* forward-model control parameters */
typedef struct {
  int ng;
  char emitter[NG][LEN];
  int nd;
  double nu[ND];
  int nw;
  int window[ND];
  int ncl;
  double clnu[NCL];
  int nsf;
  double sfnu[NSF];
  int sftype;
  double sfsza;
  char tblbase[LEN];
  int tblfmt;
  double hydz;
  int ctm_co2, ctm_h2o, ctm_n2, ctm_o2;
  int refrac;
  double rayds, raydz;
  char fov[LEN];
  double retp_zmin, retp_zmax, rett_zmin, rett_zmax;
  double retq_zmin[NG], retq_zmax[NG];
  double retk_zmin[NW], retk_zmax[NW];
  int ret_clz, ret_cldz, ret_clk, ret_sfz, ret_sfp, ret_sft, ret_sfeps;
  int write_bbt, write_matrix, formod;
  char rfmbin[LEN], rfmhit[LEN];
  char rfmxsc[NG][LEN];
} ctl_t;

/* observation geometry and results: per-ray arrays, then channel x ray */
typedef struct {
  int nr;
  double time[NR], obsz[NR], obslon[NR], obslat[NR], vpz[NR], vplon[NR], vplat[NR];
  double tpz[NR], tplon[NR], tplat[NR];
  double tau[ND][NR];
  double rad[ND][NR];
} obs_t;

/* control-file reader of the reference (jur_unified_init calls it; the
   test driver defines stand-ins, the tests call jur_unified_init_ctl) */
void read_ctl(int argc, char *argv[], ctl_t *ctl);
double scan_ctl(int argc, char *argv[], const char *varname, int arridx, const char *defvalue,
                char *value);

#endif
