#ifndef REFSHIM_GSL_POLY_H
#define REFSHIM_GSL_POLY_H
#include <cstddef>
extern "C" {
typedef struct gsl_poly_complex_workspace gsl_poly_complex_workspace;
gsl_poly_complex_workspace* gsl_poly_complex_workspace_alloc(size_t n);
void gsl_poly_complex_workspace_free(gsl_poly_complex_workspace* w);
int gsl_poly_complex_solve(const double* a, size_t n, gsl_poly_complex_workspace* w, double* z);
double gsl_poly_eval(const double c[], const int len, const double x);
}
#endif
