/* or_fft.h -- CPU DFT for the oracle and the MEX stand-in (test infrastructure). */
#ifndef OR_FFT_H
#define OR_FFT_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_fft_plan or_fft_plan;

or_fft_plan* or_fft_plan_create(int n);
void or_fft_plan_destroy(or_fft_plan* p);
void or_fft_exec(const or_fft_plan* p, double* re, double* im, int unit_stride_unused, int inverse);

/* MATLAB fft2/ifft2 on a column-major My x Mx array; ifft2 divides by Mx*My. */
int or_fft2(int My, int Mx, double* re, double* im, int inverse);
/* MATLAB fft/ifft on a length-n vector; ifft divides by n. */
int or_fft1(int n, double* re, double* im, int inverse);

#ifdef __cplusplus
}
#endif
#endif
