// Stand-in: the reference includes this header but its hot path calls nothing from it.
#include "gsl_integration.h"
