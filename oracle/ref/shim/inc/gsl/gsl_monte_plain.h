/* Empty stand-in: the reference includes this header but calls nothing from it on the surface path. */
#include "gsl_math.h"
