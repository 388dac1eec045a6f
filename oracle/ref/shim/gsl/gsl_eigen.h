/* GSL declarations for the reference checker build: see gsl_linalg.h. */
#include "gsl_linalg.h"
