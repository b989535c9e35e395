/* fftw3.h -- clean-room stand-in for the FFTW 3.x C interface.
 *
 * TEST INFRASTRUCTURE ONLY.  This header and fftw3_shim.cc exist so that the
 * reference implementation (FFTW++ convolve.cc / fftw++.cc, which call FFTW3,
 * a third-party library that is neither vendored with the reference nor
 * installed on this machine) can be compiled into the CPU oracle under
 * oracle/_ref/.  Nothing in the GPU product links against it.
 *
 * Interface: the declarations below reproduce the public FFTW 3.3 API that
 * FFTW++ calls (fftw++.h:234-1543, fftw++.cc:41-72): the type names,
 * function signatures, sign and flag constants have to match the published
 * interface for the reference to compile unmodified.  The arithmetic behind
 * them is written from the DFT definition in fftw3_shim.cc.
 *
 * Semantics honoured (FFTW 3 manual, "What FFTW Really Computes"):
 *   complex DFT  Y[k] = sum_j X[j] exp(sign*2*pi*i*j*k/n), unnormalised;
 *   r2c          sign -1, n real inputs -> n/2+1 complex outputs;
 *   c2r          sign +1, n/2+1 Hermitian inputs -> n real outputs;
 *   rank-0 r2r   plain strided copy (FFTW++'s Transpose).
 * Execution is reentrant: every execute call gathers all inputs into private
 * scratch before writing any output, so in-place and aliased layouts work and
 * concurrent calls on one plan (fftw++.h:742-756) are safe.
 */
#ifndef ORACLE_FFTW3_SHIM_H
#define ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct oracle_fftw_plan *fftw_plan;

typedef struct oracle_fftw_iodim {
  int n;
  int is;
  int os;
} fftw_iodim;

typedef enum oracle_fftw_r2r_kind {
  FFTW_R2HC=0, FFTW_HC2R=1, FFTW_DHT=2,
  FFTW_REDFT00=3, FFTW_REDFT01=4, FFTW_REDFT10=5, FFTW_REDFT11=6,
  FFTW_RODFT00=7, FFTW_RODFT01=8, FFTW_RODFT10=9, FFTW_RODFT11=10
} fftw_r2r_kind;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)

#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_CONSERVE_MEMORY (1U << 2)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)
#define FFTW_NO_SIMD (1U << 17)

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in,
                           fftw_complex *out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in,
                           fftw_complex *out, int sign, unsigned flags);
fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany,
                             fftw_complex *in, const int *inembed,
                             int istride, int idist,
                             fftw_complex *out, const int *onembed,
                             int ostride, int odist,
                             int sign, unsigned flags);

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in,
                               fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany,
                                 double *in, const int *inembed,
                                 int istride, int idist,
                                 fftw_complex *out, const int *onembed,
                                 int ostride, int odist, unsigned flags);

fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in,
                               double *out, unsigned flags);
fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany,
                                 fftw_complex *in, const int *inembed,
                                 int istride, int idist,
                                 double *out, const int *onembed,
                                 int ostride, int odist, unsigned flags);

fftw_plan fftw_plan_guru_r2r(int rank, const fftw_iodim *dims,
                             int howmany_rank, const fftw_iodim *howmany_dims,
                             double *in, double *out,
                             const fftw_r2r_kind *kind, unsigned flags);

void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out);
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out);
void fftw_execute_r2r(const fftw_plan p, double *in, double *out);
void fftw_destroy_plan(fftw_plan p);

int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);
void fftw_cleanup(void);

int fftw_import_wisdom_from_string(const char *input_string);
char *fftw_export_wisdom_to_string(void);
void fftw_forget_wisdom(void);

void *fftw_malloc(size_t n);
void fftw_free(void *p);
int fftw_alignment_of(double *p);

#ifdef __cplusplus
}
#endif

#endif
