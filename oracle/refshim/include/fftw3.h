// Stand-in for the four FFTW3 entry points the reference calls
// (fftw_plan_dft_r2c_3d / fftw_plan_dft_c2r_3d / fftw_execute / fftw_destroy_plan).
// The implementation (fftw_dft.cpp) restates the transforms FFTW documents:
// the unnormalised forward r2c DFT (sign -1) onto the Nz/2+1 half spectrum and
// the unnormalised backward c2r DFT (sign +1), c2r(r2c(x)) = Nx*Ny*Nz * x.
#ifndef REFSHIM_FFTW3_H
#define REFSHIM_FFTW3_H
extern "C" {
typedef double fftw_complex[2];
typedef struct refshim_fftw_plan_s* fftw_plan;
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_PATIENT (1U << 5)
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex* in, double* out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int n);
}
#endif
