/* fftwpp_gb300.h -- device-pointer C ABI of the GB300 hybrid dealiased
 * convolution (lib_fftwpp.so).
 *
 * These entry points generalise the reference's C wrapper
 * (wrappers/cfftw++.h) to everything its C++ API can wire
 * (convolve.h:471-1893): any dimension 1-3, any padded-transform kind per
 * axis, any minimum padded length, A inputs / B outputs, a built-in
 * multiplier, FP64 or FP32-compensated arithmetic, a batch of independent
 * 1D problems, and device pointers on a caller-supplied CUDA stream.  No
 * PyTorch types appear: pointers and sizes only.
 *
 * Layout: every array is dense row-major in its stored shape (a Hermitian
 * innermost axis stores ceil(L/2) modes; a real outermost axis means real
 * data throughout); complex values are interleaved (re, im).
 * Status codes: 0 on success, negative on error (fgb_last_error()).
 */
#ifndef FFTWPP_GB300_H
#define FFTWPP_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Padded-transform kinds (convolve.h:471, 592, 701, 805). */
#define FGB_PAD 0        /* fftPad */
#define FGB_CENTERED 1   /* fftPadCentered */
#define FGB_HERMITIAN 2  /* fftPadHermitian (innermost axis only) */
#define FGB_REAL 3       /* fftPadReal (outermost axis only) */

/* Built-in multipliers (convolve.cc:26-110) and additions. */
#define FGB_MULT_NONE 0
#define FGB_MULT_BINARY 1          /* multBinary: F0 *= F1 */
#define FGB_MULT_REALBINARY 2      /* realMultBinary, lane-wise doubles */
#define FGB_MULT_CORRELATION 3     /* multcorrelation: F0 *= conj(F1) */
#define FGB_MULT_REALJACOBIAN 4    /* F0 = F0 F3 - F1 F2 on real data */
#define FGB_MULT_JACOBIAN 5        /* same on complex data */
#define FGB_MULT_REALJACADJ 6      /* adjoint of FGB_MULT_REALJACOBIAN */
#define FGB_MULT_DOT 7             /* F0 = sum_k F_k F_{A/2+k} */
#define FGB_MULT_REALDOT 8         /* the same, lane-wise on doubles */
#define FGB_MULT_USER 9            /* a caller's device functor, compiled
                                      into the row kernels by
                                      fftwpp_gb300_mult.cuh */

#define FGB_F64 0
#define FGB_F32 1                  /* FP32 data, split hi+lo twiddles */
#define FGB_FF 2                   /* FP64 data, float-float arithmetic */

typedef struct fgb_conv fgb_conv;

/* Plan a convolution.  kinds, L, M: per axis, outermost first.  m: NULL or
 * per-axis forced residue block length (0 = planner's choice), the
 * Application m of the reference (convolve.h:103-111); a Hermitian axis is
 * always transformed explicitly, at the padded length m q the reference
 * would use for that m.  Plans are then autotuned (fgb_set_autotune,
 * fgb_set_residue_search); the results do not depend on m (beyond
 * rounding), tiles or rows per CTA.  batch > 1 runs
 * independent 1D problems stored back to back.  Replaces the constructors
 * fftPad*(L,M,app,...) + Convolution{,2,3}(...) (convolve.h:515-1603).
 * Returns NULL on error. */
fgb_conv *fgb_create(int dim, const int *kinds, const size_t *L,
                     const size_t *M, const size_t *m, int A, int B,
                     int mult, int precision, size_t batch);

/* Convolve device arrays on `stream` (a cudaStream_t, NULL = legacy
 * default stream): in[A] inputs, out[B] outputs (out[b] may equal in[b]).
 * Inputs in[B..A-1] are preserved.  Replaces Convolution::convolve
 * (convolve.h:1157-1160) with normalisation by 1/prod(m q). */
int fgb_convolve_device(fgb_conv *c, void *const *in, void *const *out,
                        void *stream);

/* Same on host arrays, synchronous.  Page-locked arrays (create_*Align,
 * cudaHostAlloc) are read by the first kernel and written by the last one
 * directly over the host link (zero copy: on Grace the NVLink-C2C
 * transfers overlap the transforms); other host memory is copied in and
 * out.  This is also the path of the FFTW++-compatible convolve calls. */
int fgb_convolve_host(fgb_conv *c, void *const *in, void *const *out);

/* Strided layouts (the reference's fftPad(L, M, app, C, S) with S > C,
 * convolve.h:515-536, and the Sx / Sy strides of Convolution2 /
 * Convolution3, convolve.h:1274, 1556; driven by tests/hybridconv2.cc,
 * hybridconvh2.cc, hybridconv3.cc): stride[d] for each outer axis
 * d < dim-1 is the number of elements between consecutive entries of axis
 * d in every input and output array (2D: entry (i, j) at i*stride[0] + j;
 * 3D: (i, j, k) at i*stride[0] + j*stride[1] + k); the innermost axis is
 * contiguous.  Entries in the gaps are neither read nor written.  NULL
 * restores the dense layout.  2D and 3D plans only; -1 for strides
 * smaller than the data they step over. */
int fgb_set_strides(fgb_conv *c, const size_t *stride);

/* Convolve with a caller's device multiplier (the reference's user
 * multiplier hook, typedef multiplier in convolve.h:78-79, with the slot
 * positions of its Indices, convolve.h:48-82).  The plan is made by
 * fgb_create with mult = FGB_MULT_USER; `launchers` is the row-kernel
 * instantiation for the functor that fgb::convolveWith /
 * fgb::convolveHostWith (fftwpp_gb300_mult.cuh, a CUDA C++ header) build
 * and pass here -- C callers use those templates rather than these entry
 * points directly.  Device arrays on `stream`, or host arrays
 * (synchronous), as fgb_convolve_device / fgb_convolve_host; -1 when the
 * plan's multiplier is not FGB_MULT_USER or the functor's A, B differ from
 * the plan's. */
int fgb_convolve_device_with(fgb_conv *c, const void *launchers,
                             void *const *in, void *const *out, void *stream);
int fgb_convolve_host_with(fgb_conv *c, const void *launchers,
                           void *const *in, void *const *out);

/* Arithmetic of the FFTW++-compatible entry points (cfftw++.h creators,
 * the _dot forms and include/convolve.h), whose arrays are FP64: FGB_F64
 * (default) or FGB_FF (float-float: FP64-grade accuracy, about 3x faster
 * on GB300).  Applies to plans created afterwards; -1 for other values. */
int fgb_set_drop_in_precision(int precision);
int fgb_get_drop_in_precision(void);

/* Range guard of the float-float mode, process-wide (default on).  Floats
 * span exponents of about +-126 against a double's +-1022, so before each
 * float-float convolution a scan of the FP64 inputs finds each array's
 * largest exponent, the first kernel scales the inputs by exact powers of
 * two and the last kernel scales the outputs back: inputs of any FP64
 * magnitude (1e-300 to 1e300) keep FP64-grade accuracy.  Multipliers whose
 * outputs are single products (binary, correlation, the Jacobian adjoint)
 * scale each input separately; sums of products share a scale per factor
 * group (the Jacobian u0 u3 - u1 u2: one for u0 and u1, one for u2 and u3;
 * dot products: one per half); a caller's functor (FGB_MULT_USER) is not
 * scaled.  Values below about 2^-120 of
 * their array's largest magnitude lose relative accuracy (their share of
 * the L2 norm is below 1e-36).  0 turns the scan off. */
void fgb_set_ff_range_guard(int on);

/* Failure injection for tests, on the host: the n-th following device
 * allocation of the library (0: the next one) fails as cudaMalloc would, so
 * error paths (NULL plans, released partial allocations) can be exercised;
 * -1 turns it off. */
void fgb_debug_fail_allocation_after(long n);

/* Process-wide switch of the zero-copy host path (default on); 0 always
 * copies page-locked arrays in and out as well. */
void fgb_set_zero_copy(int on);

/* Process-wide choice of how page-locked inputs and outputs of the
 * host-pointer entries cross the host link, each side on its own:
 * 0 copies whole arrays through device memory (SM copies), 1 has the first
 * kernel read (or the last kernel write) the caller's arrays in place with
 * the plan's device-tuned outer column tiles, 2 the same with the fastest
 * tiles whose rows span at least 64 bytes.  -1 for either side (default)
 * lets each plan's first host call whose device-tuned tiles are narrower
 * than 64 bytes time every combination on page-locked scratch arrays and
 * keep the fastest.  Results are identical every way. */
void fgb_set_host_path(int inputs, int outputs);

/* The ways (0, 1, 2 as for fgb_set_host_path) this plan's host-pointer
 * calls take for page-locked inputs and outputs: the measured choice, or
 * -1 before the first call that measures.  Returns 0, or -1 for a null
 * handle. */
int fgb_host_path(const fgb_conv *c, int *inputs, int *outputs);

/* Plan parameters: for each axis d, info[8d..8d+7] = m, p, q, N, stored
 * length, centred offset, outer tile, rows produced.  info[24] = kernels per
 * convolution, info[25] = staging bytes, info[26] = 1 if the 1D long path
 * is used, info[27+d] = backward tile of axis d, info[30] = rows per CTA of
 * the innermost-axis kernel, info[31] = its threads per CTA (info holds 32
 * longs).  Mirrors the public members m,p,q,M of fftBase
 * (convolve.h:123-145). */
int fgb_info(const fgb_conv *c, long *info);

/* Plan-time autotuning, process-wide (default on): fgb_create times the
 * candidate rows-per-CTA of the innermost-axis kernel and column tiles of
 * the outer-axis kernels (each with 128 or 256 threads) on scratch data and
 * keeps the fastest, the GPU counterpart of FFTW++'s optimiser
 * (convolve.cc:177-470).  0 keeps the planner's cost-model choice and turns
 * the residue search below off as well.  Schedules regroup work across CTAs
 * only: results are bit-identical either way. */
void fgb_set_autotune(int on);

/* Plan wisdom, the counterpart of the FFTW wisdom FFTW++ keeps in
 * wisdom3.txt (fftw++.cc:31-72).  Every plan fgb_create tunes is recorded
 * (its residue blocks and schedule, under a key of the problem and the
 * GPU); a later fgb_create of the same key rebuilds the plan from the record
 * without timing, so plans are deterministic across runs that share it.
 * fgb_wisdom_export writes the records as text, one line per plan, into buf
 * (at most size bytes, NUL-terminated when there is room) and returns the
 * full length; fgb_wisdom_import merges such text (a line replaces the
 * record of its key) and returns the lines taken, or -1, taking none, for
 * text that does not parse; fgb_wisdom_forget drops every record.  A
 * record whose schedule no longer fits the plan is ignored and replaced. */
size_t fgb_wisdom_export(char *buf, size_t size);
int fgb_wisdom_import(const char *text);
void fgb_wisdom_forget(void);

/* Timed residue search, process-wide (default on, effective while
 * autotuning is on): for every fftPad / fftPadCentered axis whose m is not
 * forced, fgb_create times whole convolutions with up to three residue
 * block lengths m the cost model ranks best (within 1.5x of its estimate),
 * axis by axis from the outermost, and keeps a candidate only if it is at
 * least 3 % faster, as the reference's OptBase times its candidate m
 * (convolve.cc:177-470).  Like the reference's choice of m, it changes the
 * rounding of the results (within the same error bounds), not the values. */
void fgb_set_residue_search(int on);

/* Normalisation switch: 1 (default) scales the result by 1/prod(m q) as
 * Convolution::convolve does; 0 returns the unnormalised sum of
 * Convolution::convolveRaw (convolve.h:1151-1160). */
int fgb_set_normalize(fgb_conv *c, int normalize);

/* Per-kernel timing (no reference counterpart: the reference times whole
 * convolutions on the CPU, convolve.cc:177-232).  With timing enabled every
 * convolve call records a CUDA event on its stream before the first and
 * after each kernel; after synchronising the stream, fgb_timing_collect
 * adds the elapsed milliseconds of launch i to ms[i] (i < n) and returns
 * the number of launches of the last call. */
int fgb_timing(fgb_conv *c, int enable);
int fgb_timing_collect(fgb_conv *c, double *ms, int n);

void fgb_destroy(fgb_conv *c);

/* Many independent 1D convolutions of uneven lengths in ONE persistent
 * kernel launch (no reference counterpart: the reference constructs one
 * Convolution per problem, convolve.h:1018-1022, and runs them one after
 * another).  Problem i has L[i] values padded to >= M[i]; the data of all
 * problems is packed back to back in each of the A input and B output
 * device arrays (problem i starts at sum_{j<i} L[j]).  kind: FGB_PAD or
 * FGB_CENTERED.  tune != 0 times the candidate plans of every distinct
 * (L, M) on the GPU and keeps the fastest, the GPU counterpart of the
 * reference's CPU optimiser (convolve.cc:177-470). */
typedef struct fgb_batch fgb_batch;
fgb_batch *fgb_batch_create(int n, const size_t *L, const size_t *M, int A,
                            int B, int mult, int precision, int kind,
                            int tune);
/* use_graph != 0: capture the launch in a CUDA graph (once per pointer set)
 * and replay it on `stream`. */
int fgb_batch_convolve_device(fgb_batch *b, void *const *in,
                              void *const *out, void *stream, int use_graph);
/* info[0] tasks, [1] persistent grid, [2] shared bytes per CTA,
 * [3] one-CTA problems, [4] long problems, [5] total packed length. */
int fgb_batch_info(const fgb_batch *b, long *info);
/* Plan of problem i: > 0 residue block m (one CTA), < 0 minus the row
 * length of a long problem. */
long fgb_batch_choice(const fgb_batch *b, int i);
/* Nonzero if a bounded in-kernel wait gave up since the last call. */
int fgb_batch_error(fgb_batch *b);
void fgb_batch_destroy(fgb_batch *b);

/* Failure detection.  Every dependency wait of the persistent kernel polls
 * at most `polls` times (default 2e7, seconds) and then gives up: its task
 * is skipped, fgb_batch_error() reports it, the launch still finishes and
 * the CUDA context stays usable.  fgb_batch_block_problem makes the waits
 * of long problem i (fgb_batch_choice(i) < 0) unreachable (blocked != 0)
 * or restores them, so tests can make a wait run out on purpose. */
int fgb_batch_set_spin_limit(fgb_batch *b, long long polls);
int fgb_batch_block_problem(fgb_batch *b, int i, int blocked);

/* Standalone padded transforms: the forward and backward transforms of
 * fftPad / fftPadCentered / fftPadReal (convolve.h:515-536, 623-646,
 * 855-877; driven stand-alone by the reference's tests/hybrid.cc and
 * tests/hybridr.cc), for callers that work in padded space themselves.
 * kind: FGB_PAD, FGB_CENTERED or FGB_REAL; L data length, M
 * minimum padded length, C interleaved columns (element (s, c) at s*C + c),
 * m forced residue block length (0: planner's choice).
 * Complex kinds: F is N x C complex, row r*m + j holding residue r, entry j,
 *   the padded DFT (sign +1) at transformed index fgb_pad_index(r, j) =
 *   q*j + r, measured from the centred origin floor(L/2) for
 *   FGB_CENTERED.  Real kind: f is L x C real, F is (N/2+1) x C
 *   complex in natural frequency order (fgb_pad_index(0, k) = k).
 *   Hermitian kind (fftPadHermitian, convolve.h:737-757; tests/hybridh.cc):
 *   f is ceil(L/2) x C complex (the stored modes k >= 0, f_0 real), F is
 *   N x C real, the physical values at grid points t = 0..N-1 of the
 *   Hermitian-extended spectrum (explicit padding to an even N, as
 *   fftPadHermitian with m = N, D = 1; fgb_pad_index(0, t) = t).
 * backward is the unnormalised adjoint (sign -1) accumulated over residues,
 * so backward(forward(f)) = N f.  Device pointers, asynchronous on stream. */
typedef struct fgb_pad fgb_pad;
fgb_pad *fgb_pad_create(int kind, size_t L, size_t M, size_t C, size_t m,
                        int precision);
int fgb_pad_forward_device(fgb_pad *t, const void *f, void *F, void *stream);
int fgb_pad_backward_device(fgb_pad *t, const void *F, void *f, void *stream);
/* info[0] m, [1] p, [2] q, [3] N, [4] L, [5] C, [6] rows of F, [7] centred
 * origin offset, [8] forward columns per CTA, [9] backward columns per CTA. */
int fgb_pad_info(const fgb_pad *t, long *info);
size_t fgb_pad_index(const fgb_pad *t, size_t r, size_t j);
void fgb_pad_destroy(fgb_pad *t);

/* Plain unnormalised FFTs on the same shared-memory radix kernels: the
 * fft1d / mfft1d (FGB_FFT_C2C, sign +1 or -1), rcfft1d / mrcfft1d
 * (FGB_FFT_R2C, n reals -> n/2+1 complex, sign -1) and crfft1d / mcrfft1d
 * (FGB_FFT_C2R, sign +1) classes of fftw++.h:556-1197; the 2D and 3D
 * classes (fftw++.h:1199-1585) are passes of these (fftwpp_gb300/fft.py).
 * C interleaved sequences in each of B batches: element s of sequence c in
 * batch b at b*batch + s*stride + c, counted in the element type of each
 * side (stride >= C when C > 1).  n: a product of 2, 3, 5, 7 (even for
 * real transforms).  Lengths beyond one CTA's shared memory are taken by
 * complex transforms of contiguous sequences (C == 1, unit strides) in two
 * passes through a scratch array the plan allocates (n = n1 n2, the
 * four-step FFT).  Complex transforms may run in place, real ones only
 * with C == 1.  Device pointers, asynchronous on stream.  No normalisation
 * (fftNormalized divides by n). */
#define FGB_FFT_C2C 0
#define FGB_FFT_R2C 1
#define FGB_FFT_C2R 2
typedef struct fgb_fft fgb_fft;
fgb_fft *fgb_fft_create(int kind, size_t n, int sign, size_t C, size_t B,
                        size_t istride, size_t ibatch, size_t ostride,
                        size_t obatch, int precision);
int fgb_fft_execute_device(fgb_fft *t, const void *in, void *out,
                           void *stream);
void fgb_fft_destroy(fgb_fft *t);

/* The origin shift of the fft0 transforms (fftw++.h:144-228, Shift; used by
 * rcfft2d/crfft2d/rcfft3d/crfft3d::fft0): negate the real values (i, j, k)
 * of a device array of nx x ny x nz reals with i + j odd (nz == 1: i
 * odd), which moves the Fourier origin to (nx/2, 0) or (nx/2, ny/2, 0).
 * nx (and ny in 3D) must be even. */
int fgb_fft_origin_shift_device(void *f, size_t nx, size_t ny, size_t nz,
                                int precision, void *stream);

/* Text of the last error on this thread. */
const char *fgb_last_error(void);

/* The reference's integer rules, exported for tests:
 * fftBase::parameters (convolve.cc:403-410) and nextfftsize
 * (convolve.cc:114-124). */
void fgb_parameters(size_t L, size_t M, size_t m, int centered,
                    size_t *p, size_t *n, size_t *q);
size_t fgb_nextfftsize(size_t m);

/* Queue order of the batched launch's tasks (host arithmetic, no GPU), for
 * nlong long problems with the given staging bytes, forward column tiles,
 * row tasks and backward column tiles, and nsmall one-CTA problems
 * (numbered after the long ones).  Writes at most max (type, problem)
 * pairs, type 0 a small problem, 1 a forward column tile (once per input),
 * 2 a row task, 3 a backward column tile (once per output), and returns
 * the task count. */
int fgb_batch_task_order(int nlong, const size_t *staging,
                         const int *fwdTiles, const int *rows,
                         const int *bwdTiles, int nsmall, int inputs,
                         int outputs, size_t groupBytes, int *type,
                         int *problem, int max);

/* Radices, stage by stage, of the shared-memory transforms of length n
 * (host arithmetic, no GPU): inplace != 0 for the in-place
 * decimation-in-frequency/time form (odd radices first), wide != 0 for the
 * FP32 row and in-place outer transforms that may take radix 16 and 6.
 * Writes at most max radices and returns their count, or -1 for a length
 * that is not 2^a 3^b 5^c 7^d. */
int fgb_fft_radices(size_t n, int precision, int inplace, int wide,
                    int *radix, int max);

/* Transformed index of entry i of residue block r (fftBase::index,
 * convolve.h:297-326, and fftPadReal::index, convolve.h:956-979) for the
 * reference's parameters (m,p,q,n,D) of a 1D transform. */
size_t fgb_index(int kind, size_t m, size_t p, size_t q, size_t n, size_t D,
                 size_t r, size_t i);

/* 2D centred-Hermitian FP64 convolution that allocates no memory.  No
 * counterpart in the reference (FFTW++ allocates its work arrays in every
 * Convolution constructor).  For callers that cannot call cudaMalloc: an
 * application whose own allocator owns the device memory, or a
 * latency-critical loop in which an allocation would synchronise the
 * device.  f, g, h: device arrays of Lx x ceil(Ly/2) complex128 modes in the
 * layout of fftwpp_hconv2d_convolve (h may equal f); the result, normalised
 * as Convolution::convolve does, goes to h.  Padding: the reference's
 * default 3/2 rule (HybridConvolution.h:94-95).  All scratch (staging rows
 * and twiddle tables) lives in one file-scope device array of
 * FGB_NOALLOC_SCRATCH_BYTES = 32 MiB, held by every GPU that loads the
 * library until the process exits; sizes that need more are rejected with
 * an error (up to 1023 x 1023 fits).  The array is shared by all calls on a
 * device and keeps the last call's contents; each call rewrites everything
 * it reads.  Calls that overlap on the GPU race on it.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress); make
 * it before any stream capture.  That address is kept until the process
 * exits, so do not call this entry point again on a device after
 * cudaDeviceReset.  Returns 0, or -1 with fgb_last_error(). */
int fgb_hconv2d_convolve_noalloc(const void *f, const void *g, void *h,
                                 size_t Lx, size_t Ly, void *stream);

/* Measured FP64 (DFMA) and FP32 (FFMA) instruction issue rates of the
 * current GPU, per second, from dependent-chain probes on every SM -- the
 * denominators of the compute roofline of the FP64-bound kernels (no
 * reference counterpart). */
int fgb_measure_fma_rate(double *dfma_per_s, double *ffma_per_s);

/* f[i][j] *= (j == 0 ? s0 : s1) on a rows x cols complex device array: the
 * weight of the k_y = 0 column of half-plane Hermitian data, used by the
 * adjoint of the Hermitian convolutions (no reference counterpart). */
int fgb_scale_columns_device(size_t rows, size_t cols, double s0, double s1,
                             void *f, int precision, void *stream);

/* Hermitian symmetrisation of device arrays (convolve.h:1175-1258). */
int fgb_hermitian_symmetrize_x_device(size_t Hx, size_t Hy, size_t x0,
                                      void *f, int precision, void *stream);

#ifdef __cplusplus
}
#endif

#endif
