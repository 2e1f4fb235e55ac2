// Definitions for the stand-in GSL declarations. None is on the path the
// oracle driver exercises; each aborts loudly if it is ever reached.
#include <cstdio>
#include <cstdlib>
#include "gsl/gsl_integration.h"
#include "gsl/gsl_poly.h"
static void refshim_unreachable(const char* f) {
  std::fprintf(stderr, "refshim: %s is not available in the oracle build\n", f);
  std::abort();
}
extern "C" {
gsl_integration_workspace* gsl_integration_workspace_alloc(size_t) { refshim_unreachable("gsl_integration_workspace_alloc"); return nullptr; }
void gsl_integration_workspace_free(gsl_integration_workspace*) {}
int gsl_integration_qags(const gsl_function*, double, double, double, double, size_t, gsl_integration_workspace*, double*, double*) { refshim_unreachable("gsl_integration_qags"); return 0; }
int gsl_integration_qagiu(gsl_function*, double, double, double, size_t, gsl_integration_workspace*, double*, double*) { refshim_unreachable("gsl_integration_qagiu"); return 0; }
int gsl_integration_qng(const gsl_function*, double, double, double, double, double*, double*, size_t*) { refshim_unreachable("gsl_integration_qng"); return 0; }
gsl_integration_glfixed_table* gsl_integration_glfixed_table_alloc(size_t) { refshim_unreachable("gsl_integration_glfixed_table_alloc"); return nullptr; }
int gsl_integration_glfixed_point(double, double, size_t, double*, double*, const gsl_integration_glfixed_table*) { refshim_unreachable("gsl_integration_glfixed_point"); return 0; }
gsl_poly_complex_workspace* gsl_poly_complex_workspace_alloc(size_t) { refshim_unreachable("gsl_poly_complex_workspace_alloc"); return nullptr; }
void gsl_poly_complex_workspace_free(gsl_poly_complex_workspace*) {}
int gsl_poly_complex_solve(const double*, size_t, gsl_poly_complex_workspace*, double*) { refshim_unreachable("gsl_poly_complex_solve"); return 0; }
double gsl_poly_eval(const double[], const int, const double) { refshim_unreachable("gsl_poly_eval"); return 0; }
}
