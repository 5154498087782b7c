#include "gsl_shim_decls.h"
