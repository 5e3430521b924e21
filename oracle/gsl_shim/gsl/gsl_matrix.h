/* GSL-compat shim header (test infrastructure): all definitions live in gsl_shim_core.h. */
#include "gsl_shim_core.h"
