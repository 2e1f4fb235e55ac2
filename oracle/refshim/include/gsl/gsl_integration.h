// Stand-in declarations for the GSL quadrature routines the reference headers
// name. The oracle driver never calls them (the hard-sphere diameter is passed
// in explicitly); the stub definitions abort if reached.
#ifndef REFSHIM_GSL_INTEGRATION_H
#define REFSHIM_GSL_INTEGRATION_H
#include <cstddef>
extern "C" {
typedef struct { double (*function)(double x, void* params); void* params; } gsl_function;
typedef struct gsl_integration_workspace gsl_integration_workspace;
typedef struct gsl_integration_glfixed_table gsl_integration_glfixed_table;
gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace* w);
int gsl_integration_qags(const gsl_function* f, double a, double b, double epsabs, double epsrel, size_t limit,
                         gsl_integration_workspace* w, double* result, double* abserr);
int gsl_integration_qagiu(gsl_function* f, double a, double epsabs, double epsrel, size_t limit,
                          gsl_integration_workspace* w, double* result, double* abserr);
int gsl_integration_qng(const gsl_function* f, double a, double b, double epsabs, double epsrel, double* result,
                        double* abserr, size_t* neval);
gsl_integration_glfixed_table* gsl_integration_glfixed_table_alloc(size_t n);
int gsl_integration_glfixed_point(double a, double b, size_t i, double* xi, double* wi,
                                  const gsl_integration_glfixed_table* t);
}
#endif
