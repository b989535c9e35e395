/* cfftw++.h -- C ABI of the GB300 hybrid dealiased convolution library
 * (lib_fftwpp.so), binary compatible with FFTW++'s C wrapper.
 *
 * Every entry point below replaces the FFTW++ function of the same name
 * (reference: wrappers/cfftw++.h declares them, wrappers/cfftw++.cc defines
 * them; defaults come from wrappers/HybridConvolution.h).  Arrays are
 * interleaved complex128 (double _Complex) in host memory, exactly as FFTW++
 * expects; the library copies them to the GPU, runs the hand-written sm_103a
 * kernels and copies the result back.  Convolutions are computed in place:
 * the result overwrites the first argument and is normalised by the padded
 * size, as Convolution::convolve does (convolve.h:1157-1160).
 *
 * Differences from the reference, all in error handling: the reference
 * exit()s on invalid parameters (convolve.h:226-232, convolve.cc:480-500);
 * here a create_* call returns NULL and a convolve call leaves its data
 * untouched, and fgb_last_error() (fftwpp_gb300.h) says why.
 */
#ifndef FFTWPP_GB300_CFFTWPP_H
#define FFTWPP_GB300_CFFTWPP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
typedef struct { double re, im; } fftwpp_complex128;
#define FFTWPP_C128 fftwpp_complex128
#else
#define FFTWPP_C128 double _Complex
#endif

/* Aligned host allocation (wrappers/cfftw++.cc:27-41).  Memory comes from
 * page-locked host memory when a GPU is present, so the convolve calls copy
 * it at full PCIe/C2C bandwidth; it is 64-byte aligned either way. */
double *create_doubleAlign(size_t n);              /* cfftw++.cc:27 */
void delete_doubleAlign(double *p);                /* cfftw++.cc:31 */
FFTWPP_C128 *create_complexAlign(size_t n);        /* cfftw++.cc:35 */
void delete_complexAlign(FFTWPP_C128 *p);          /* cfftw++.cc:39 */

/* Thread count kept for ABI compatibility (cfftw++.cc:44-50); the GPU path
 * ignores it. */
size_t get_fftwpp_maxthreads(void);                /* cfftw++.cc:44 */
void set_fftwpp_maxthreads(size_t nthreads);       /* cfftw++.cc:48 */

/* 1D complex, fftPad + multBinary, M = 2L-1 (HybridConvolution.h:12-30). */
typedef struct HybridConvolution HybridConvolution;
HybridConvolution *fftwpp_create_conv1d(size_t L);          /* cfftw++.cc:53 */
void fftwpp_conv1d_delete(HybridConvolution *conv);        /* cfftw++.cc:57 */
void fftwpp_conv1d_convolve(HybridConvolution *conv,
                            FFTWPP_C128 *a, FFTWPP_C128 *b); /* cfftw++.cc:61 */

/* 1D Hermitian, fftPadHermitian + realMultBinary, ceil(L/2) stored modes,
 * M = 3 ceil(L/2) - 2 (L mod 2) (HybridConvolution.h:32-50). */
typedef struct HybridConvolutionHermitian HybridConvolutionHermitian;
HybridConvolutionHermitian *fftwpp_create_hconv1d(size_t L); /* cfftw++.cc:68 */
void fftwpp_hconv1d_delete(HybridConvolutionHermitian *conv); /* cfftw++.cc:72 */
void fftwpp_HermitianSymmetrize(FFTWPP_C128 *f);            /* cfftw++.cc:76 */
void fftwpp_hconv1d_convolve(HybridConvolutionHermitian *conv,
                             FFTWPP_C128 *a, FFTWPP_C128 *b); /* cfftw++.cc:80 */

/* 2D complex, fftPad x fftPad (HybridConvolution.h:52-78). */
typedef struct HybridConvolution2 HybridConvolution2;
HybridConvolution2 *fftwpp_create_conv2d(size_t Lx, size_t Ly); /* cfftw++.cc:87 */
void fftwpp_conv2d_delete(HybridConvolution2 *conv);          /* cfftw++.cc:92 */
void fftwpp_HermitianSymmetrizeX(size_t Hx, size_t Hy, size_t x0,
                                 FFTWPP_C128 *f);              /* cfftw++.cc:96 */
void fftwpp_conv2d_convolve(HybridConvolution2 *conv,
                            FFTWPP_C128 *a, FFTWPP_C128 *b);   /* cfftw++.cc:101 */

/* 2D centred Hermitian, fftPadCentered x fftPadHermitian, data Lx x
 * ceil(Ly/2) (HybridConvolution.h:80-111). */
typedef struct HybridConvolutionHermitian2 HybridConvolutionHermitian2;
HybridConvolutionHermitian2 *fftwpp_create_hconv2d(size_t Lx, size_t Ly); /* cfftw++.cc:109 */
void fftwpp_hconv2d_delete(HybridConvolutionHermitian2 *conv); /* cfftw++.cc:114 */
void fftwpp_hconv2d_convolve(HybridConvolutionHermitian2 *conv,
                             FFTWPP_C128 *a, FFTWPP_C128 *b);  /* cfftw++.cc:118 */

/* 3D complex (HybridConvolution.h:113-146). */
typedef struct HybridConvolution3 HybridConvolution3;
HybridConvolution3 *fftwpp_create_conv3d(size_t Lx, size_t Ly,
                                         size_t Lz);          /* cfftw++.cc:125 */
void fftwpp_conv3d_delete(HybridConvolution3 *conv);          /* cfftw++.cc:131 */
void fftwpp_HermitianSymmetrizeXY(size_t Hx, size_t Hy, size_t Hz,
                                  size_t x0, size_t y0,
                                  FFTWPP_C128 *f);             /* cfftw++.cc:135 */
void fftwpp_conv3d_convolve(HybridConvolution3 *conv,
                            FFTWPP_C128 *a, FFTWPP_C128 *b);   /* cfftw++.cc:142 */

/* 3D centred Hermitian, data Lx x Ly x ceil(Lz/2)
 * (HybridConvolution.h:148-182). */
typedef struct HybridConvolutionHermitian3 HybridConvolutionHermitian3;
HybridConvolutionHermitian3 *fftwpp_create_hconv3d(size_t Lx, size_t Ly,
                                                   size_t Lz); /* cfftw++.cc:149 */
void fftwpp_hconv3d_delete(HybridConvolutionHermitian3 *conv); /* cfftw++.cc:155 */
void fftwpp_hconv3d_convolve(HybridConvolutionHermitian3 *conv,
                             FFTWPP_C128 *a, FFTWPP_C128 *b);  /* cfftw++.cc:159 */

/* Dot-product and work-array forms.  FFTW++'s header declares these but
 * its wrapper never defines them (cfftw++.h:18, 30-47, 53-71, 77-99,
 * 104-129, 136-153, 161-188); here they are defined with the meaning their
 * signatures carry:
 *   m (mx, my, mz): data lengths, as L of the plain forms;
 *   M: number of products; the result is sum_{k<M} a_k * b_k (Hermitian
 *      forms: lane-wise real products, like realMultBinary), normalised
 *      like the plain forms and written over a[0] (dotf: the first block);
 *   _dot(a, b): arrays of M host pointers; _dotf(a, b): M arrays back to
 *      back in one host array each;
 *   _work(..., u, v, w, ...): the caller's host scratch of the CPU code;
 *      the GPU allocates its own device scratch, so these are ignored.
 * A plain handle passed to a _dot call computes one product (M = 1). */
double *create_doublealign(size_t n);                     /* cfftw++.h:18 */

HybridConvolution *fftwpp_create_conv1d_dot(size_t m, size_t M);  /* cfftw++.h:30 */
HybridConvolution *fftwpp_create_conv1d_work(size_t m, FFTWPP_C128 *u,
                                             FFTWPP_C128 *v);     /* cfftw++.h:32 */
HybridConvolution *fftwpp_create_conv1d_work_dot(size_t m, FFTWPP_C128 *u,
                                                 FFTWPP_C128 *v,
                                                 size_t M);       /* cfftw++.h:35 */
void fftwpp_conv1d_convolve_dot(HybridConvolution *conv, FFTWPP_C128 **a,
                                FFTWPP_C128 **b);                 /* cfftw++.h:42 */
void fftwpp_conv1d_convolve_dotf(HybridConvolution *conv, FFTWPP_C128 *a,
                                 FFTWPP_C128 *b);                 /* cfftw++.h:45 */

HybridConvolutionHermitian *fftwpp_create_hconv1d_dot(size_t m,
                                                      size_t M);  /* cfftw++.h:53 */
HybridConvolutionHermitian *fftwpp_create_hconv1d_work(size_t m,
    FFTWPP_C128 *u, FFTWPP_C128 *v, FFTWPP_C128 *w);              /* cfftw++.h:55 */
HybridConvolutionHermitian *fftwpp_create_hconv1d_work_dot(size_t m,
    FFTWPP_C128 *u, FFTWPP_C128 *v, FFTWPP_C128 *w, size_t M);    /* cfftw++.h:59 */
void fftwpp_hconv1d_convolve_dot(HybridConvolutionHermitian *conv,
                                 FFTWPP_C128 **a, FFTWPP_C128 **b); /* cfftw++.h:66 */
void fftwpp_hconv1d_convolve_dotf(HybridConvolutionHermitian *conv,
                                  FFTWPP_C128 *a, FFTWPP_C128 *b); /* cfftw++.h:69 */

HybridConvolution2 *fftwpp_create_conv2d_dot(size_t mx, size_t my,
                                             size_t M);           /* cfftw++.h:77 */
HybridConvolution2 *fftwpp_create_conv2d_work(size_t mx, size_t my,
    FFTWPP_C128 *u1, FFTWPP_C128 *v1, FFTWPP_C128 *u2,
    FFTWPP_C128 *v2);                                             /* cfftw++.h:79 */
HybridConvolution2 *fftwpp_create_conv2d_work_dot(size_t mx, size_t my,
    FFTWPP_C128 *u1, FFTWPP_C128 *v1, FFTWPP_C128 *u2,
    FFTWPP_C128 *v2, size_t M);                                   /* cfftw++.h:85 */
void fftwpp_conv2d_convolve_dot(HybridConvolution2 *conv, FFTWPP_C128 **a,
                                FFTWPP_C128 **b);                 /* cfftw++.h:95 */
void fftwpp_conv2d_convolve_dotf(HybridConvolution2 *conv, FFTWPP_C128 *a,
                                 FFTWPP_C128 *b);                 /* cfftw++.h:97 */

HybridConvolutionHermitian2 *fftwpp_create_hconv2d_dot(size_t mx, size_t my,
                                                       size_t M); /* cfftw++.h:104 */
HybridConvolutionHermitian2 *fftwpp_create_hconv2d_work(size_t mx, size_t my,
    FFTWPP_C128 *u1, FFTWPP_C128 *v1, FFTWPP_C128 *w1, FFTWPP_C128 *u2,
    FFTWPP_C128 *v2);                                             /* cfftw++.h:107 */
HybridConvolutionHermitian2 *fftwpp_create_hconv2d_work_dot(size_t mx,
    size_t my, FFTWPP_C128 *u1, FFTWPP_C128 *v1, FFTWPP_C128 *w1,
    FFTWPP_C128 *u2, FFTWPP_C128 *v2, size_t M);                  /* cfftw++.h:114 */
void fftwpp_hconv2d_convolve_dot(HybridConvolutionHermitian2 *conv,
                                 FFTWPP_C128 **a, FFTWPP_C128 **b); /* cfftw++.h:124 */
void fftwpp_hconv2d_convolve_dotf(HybridConvolutionHermitian2 *conv,
                                  FFTWPP_C128 *a, FFTWPP_C128 *b); /* cfftw++.h:127 */

HybridConvolution3 *fftwpp_create_conv3d_work(size_t mx, size_t my,
    size_t mz, FFTWPP_C128 *u1, FFTWPP_C128 *v1, FFTWPP_C128 *u2,
    FFTWPP_C128 *v2, FFTWPP_C128 *u3, FFTWPP_C128 *v3);           /* cfftw++.h:136 */
HybridConvolution3 *fftwpp_create_conv3d_dot(size_t mx, size_t my,
                                             size_t mz, size_t M); /* cfftw++.h:145 */
void fftwpp_conv3d_convolve_dot(HybridConvolution3 *conv, FFTWPP_C128 **a,
                                FFTWPP_C128 **b);                 /* cfftw++.h:151 */
void fftwpp_conv3d_convolve_dotf(HybridConvolution3 *conv, FFTWPP_C128 *a,
                                 FFTWPP_C128 *b);                 /* cfftw++.h:153 */

HybridConvolutionHermitian3 *fftwpp_create_hconv3d_dot(size_t mx, size_t my,
                                                       size_t mz,
                                                       size_t M); /* cfftw++.h:161 */
HybridConvolutionHermitian3 *fftwpp_create_hconv3d_work(size_t mx, size_t my,
    size_t mz, FFTWPP_C128 *u1, FFTWPP_C128 *v1, FFTWPP_C128 *w1,
    FFTWPP_C128 *u2, FFTWPP_C128 *v2, FFTWPP_C128 *u3,
    FFTWPP_C128 *v3);                                             /* cfftw++.h:165 */
HybridConvolutionHermitian3 *fftwpp_create_hconv3d_work_dot(size_t mx,
    size_t my, size_t mz, FFTWPP_C128 *u1, FFTWPP_C128 *v1,
    FFTWPP_C128 *w1, FFTWPP_C128 *u2, FFTWPP_C128 *v2, FFTWPP_C128 *u3,
    FFTWPP_C128 *v3, size_t M);                                   /* cfftw++.h:175 */
void fftwpp_hconv3d_convolve_dot(HybridConvolutionHermitian3 *conv,
                                 FFTWPP_C128 **a, FFTWPP_C128 **b); /* cfftw++.h:188 */

#ifdef __cplusplus
}
#endif

#endif
