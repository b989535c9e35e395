// engine.h -- host side of the GB300 hybrid dealiased convolution.
//
// A Conv object is the GPU counterpart of a chain of FFTW++ padded
// transforms plus a Convolution/Convolution2/Convolution3 driver
// (convolve.h:982-1893): it owns the per-axis padding plans, the device
// twiddle tables and the HBM staging buffers of the outer axes, and launches
// the kernel sequence on a caller-supplied stream.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace fgb {

struct RowLaunchers;       // kernels.cuh
template<typename T> struct RowPlan;
template<typename T> struct HermRowPlan;
struct IndexMap;

enum AxisKind {KIND_PAD=0, KIND_CENTERED=1, KIND_HERMITIAN=2, KIND_REAL=3};
// PREC_FF: FP64 data at the interface, float-float arithmetic inside.
enum Precision {PREC_F64=0, PREC_F32=1, PREC_FF=2};
// How a side (inputs or outputs) of a host-pointer call crosses the host
// link: whole arrays copied through device memory, or read / written in
// place by the first / last kernel with the device-tuned axis-0 tiles or
// with tiles whose rows span at least 64 bytes.
enum HostWay {HOST_COPY=0, HOST_INPLACE=1, HOST_INPLACE64=2};

// Integer rules shared with the reference (convolve.cc:114-175, 403-410).
size_t ceilquotient(size_t a, size_t b);
size_t nextfftsize(size_t m);
size_t nextpuresize(size_t m);
bool ispure(size_t m);
void refParameters(size_t L, size_t M, size_t m, bool centered,
                   size_t& p, size_t& n, size_t& q);
bool smooth(size_t n);   // n = 2^a 3^b 5^c 7^d
// Radices of the shared-memory transforms of length n (engine.cu).
int fftRadices(long n, int prec, bool oddFirst, bool allow16, int *radix);

struct AxisPlan {
  int kind;
  long L, M;          // data length, minimum padded length
  long stored;        // values stored along the axis (ceil(L/2) if Hermitian)
  long m, q, N, p;    // residue block length, residues, padded length, folds
  int cshift;         // centred origin offset
  int tile, tileB;    // outer kernels: columns per CTA (forward, backward)
  int rpc;            // innermost axis: rows per CTA of the row kernel
  int thr, thrB;      // threads per CTA of the forward (or row) and the
                      // backward launch of this axis
  long rows;          // outer axis: rows produced (N, or N/2+1 if real)
};

struct ConvInfo {
  int dim;
  int A, B, mult, prec;
  AxisPlan axis[3];
  bool longRow;       // 1D data too long for one CTA: outer/row/outer path
  long rowM, rowQ;    // long path: row length and column DFT length
};

class Conv {
public:
  // kinds/L/M/mForce: per dimension, outermost first.  mForce[d] = 0 lets
  // the planner choose.  Throws std::runtime_error on invalid input.
  // tuneSchedule = false skips the timed tile and thread search (the cost
  // model's schedule stays).
  Conv(int dim, const int *kinds, const long *L, const long *M,
       const long *mForce, int A, int B, int mult, int prec, long batch=1,
       bool tuneSchedule=true);
  ~Conv();

  // A plan whose residue block lengths are chosen by timing (the GPU
  // counterpart of the reference's OptBase search over m, convolve.cc:177-
  // 470): for every complex axis not forced, up to three cost-model
  // candidates are timed in whole convolutions, axis by axis from the
  // outermost, and a candidate replaces the current choice only if at least
  // 3 % faster.  Plain construction when autotuning or the residue search
  // is off process-wide.  Throws like the constructor.
  static Conv *create(int dim, const int *kinds, const long *L,
                      const long *M, const long *mForce, int A, int B,
                      int mult, int prec, long batch=1);
  // Residue search in create() on or off, process-wide (default on).
  static void setResidueSearch(bool on);

  // Device pointers: A inputs, B outputs (outputs may alias inputs), each a
  // dense row-major array in the stored layout; `batch` independent
  // problems back to back in every array.
  cudaError_t run(const void *const *in, void *const *out, cudaStream_t s);

  // The same for a plan made with MULT_USER: the innermost-axis launches go
  // through the caller's instantiation of the row kernels with its own
  // device functor (fftwpp_gb300_mult.cuh), whose arity must match A and B.
  cudaError_t runWith(const RowLaunchers *L, const void *const *in,
                      void *const *out, cudaStream_t s);
  cudaError_t runHostWith(const RowLaunchers *L, const void *const *in,
                          void *const *out, cudaStream_t s);

  // Host pointers (synchronous on s).  Page-locked arrays are read and
  // written by the kernels in place (zero copy) unless disabled
  // process-wide; other host memory is copied in and out.
  cudaError_t runHost(const void *const *in, void *const *out,
                      cudaStream_t s);
  static void setZeroCopy(bool on);
  // How page-locked inputs and outputs cross the host link (HostWay), set
  // process-wide; -1 for either lets each plan's first host call time every
  // combination and keep the fastest.
  static void setHostPath(int inputs, int outputs);
  // The ways this plan's host calls take (forced, fixed by the tiles, or
  // measured), -1 while still to be measured.
  void hostPath(int *inputs, int *outputs) const;

  // Strided layouts of the caller's arrays (fftPad(L,M,app,C,S) with S > C,
  // convolve.h:515-536; the Sx / Sy strides of Convolution2/3,
  // convolve.h:1274, 1556): S[d], d < dim-1, elements between consecutive
  // entries of outer axis d; the innermost axis stays contiguous.  NULL
  // restores the dense layout.  Throws std::runtime_error on strides
  // smaller than the data they step over.
  void setStrides(const long *S);
  bool strided() const {return isStrided;}
  // Elements a strided array spans (the dense count otherwise).
  size_t spanElements() const;

  const ConvInfo& info() const {return I;}
  size_t elemBytes() const;        // bytes per stored element
  size_t elements() const;         // stored elements per array (x batch)
  int launches() const;            // kernels launched per run()
  size_t stagingBytes() const {return staging;}

  // Optional per-launch timing: when enabled, run() records a CUDA event on
  // its stream before the first and after every kernel; collect() (after
  // the stream is synchronised) adds each launch's elapsed time to ms[].
  cudaError_t enableTiming(bool on);
  int collect(double *ms, int n);

  // Normalise by 1/prod(N) (Convolution::convolve) or not (convolveRaw).
  void setNormalize(bool on) {normalize=on;}

  // Range guard of the float-float mode, process-wide (default on): each
  // convolution first scans its FP64 inputs for their largest exponents and
  // scales inputs and outputs by exact powers of two (launchFFScale), so
  // FP64 data of any magnitude fit the float exponent range.
  static void setRangeGuard(bool on);

  // Plan-time autotuning (the GPU counterpart of FFTW++'s optimiser,
  // convolve.cc:177-470): rows per CTA of the innermost-axis kernel and the
  // column tiles of the outer-axis kernels are chosen by timing every
  // candidate on scratch data; each launch depends on its own parameter
  // only, so one timed convolution per candidate index serves them all.
  // Runs in the constructor unless disabled process-wide.
  static void setAutotune(bool on);

  // Plan wisdom (the counterpart of the FFTW wisdom FFTW++ keeps in
  // wisdom3.txt, fftw++.cc:31-72): create() records the timed choices of
  // every plan it tunes (the residue blocks it forced and the schedule:
  // column tiles, rows per CTA, threads, host-line tiles) under a key of
  // the problem and the GPU, and a later create() of the same key rebuilds
  // the plan from them without timing.  Text form: one "key<TAB>value"
  // line per plan.  importWisdom merges (an imported line replaces one of
  // the same key) and returns the lines taken, or -1 (nothing taken) for
  // text that does not parse.
  static std::string exportWisdom();
  static int importWisdom(const std::string& text);
  static void forgetWisdom();

private:
  std::string schedule() const;
  bool applySchedule(const std::string& s);
  static Conv *createSearched(int dim, const int *kinds, const long *L,
                              const long *M, const long *mForce, int A,
                              int B, int mult, int prec, long batch,
                              long *mUsed);
  ConvInfo I;
  long batch;
  const RowLaunchers *user;        // row launches of a MULT_USER plan
  bool isStrided;
  long strideS[3];                 // outer-axis strides (setStrides)
  int *ffState;                    // float-float range guard (32 ints)
  static bool rangeGuard;
  cudaError_t runHostStrided(const void *const *in, void *const *out,
                             cudaStream_t s);
  bool tuning;                     // inside tune(): MULT_USER runs without
                                   // a functor (no multiplication)
  template<typename T> cudaError_t rowLaunch(const RowPlan<T>& P, int thr,
                                             long long grid, cudaStream_t s);
  template<typename T> cudaError_t hermLaunch(const HermRowPlan<T>& P,
                                              int thr, long long grid,
                                              cudaStream_t s);
  cudaError_t checkUser(const RowLaunchers *L);
  std::vector<void *> bufs;        // device staging buffers
  size_t longBuf;                  // index in bufs of the long rows' A
                                   // column-transformed copies
  size_t staging;
  void *hostIn, *hostOut;          // device copies for runHost
  int nlaunch;
  bool timing;
  bool normalize;
  static bool autotune;
  static bool residueSearch;
  static bool zeroCopy;
  static int hostPathIn, hostPathOut;
  std::vector<cudaEvent_t> events;
  int marks;
  void tick(cudaStream_t s);
  template<typename T> cudaError_t runT(const void *const *in,
                                        void *const *out, cudaStream_t s);
  // The innermost axis on the long path: nrows rows of rowStride stored
  // entries in in[] (FP64 values in float-float mode when io64 bit 0 is
  // set) convolved into out[] (bit 1); three launches.
  template<typename T> cudaError_t runLong(const void *const *in,
                                           void *const *out, long long nrows,
                                           long long rowStride, int io64,
                                           const int *guard,
                                           const IndexMap *im,
                                           double scale, cudaStream_t s);
  // Axis-0 schedule for runs that read or write page-locked host arrays
  // in place: the fastest column tiles (and threads) whose rows span at
  // least 64 bytes, 0 where no candidate does; and the ways (HostWay) the
  // first host call measured fastest for inputs and outputs, -1 before.
  int hostTile, hostThr, hostTileB, hostThrB;
  int hostWay[2];
  // Inputs copied in from the host on a side stream while the first outer
  // transform runs.  Input 0 arrives in `chunks` column ranges
  // [chunkCol[k], chunkCol[k+1]); the transform of range k runs on lanes[k]
  // (lanes[0]: the call's stream) after chunkReady[k], so the ranges run
  // concurrently as they land.  Input a > 0 arrives whole; its transform
  // waits for ready[a].  chunks = 0 outside such a host call.
  static const int CHUNKS=4;
  cudaStream_t side;
  cudaStream_t lanes[CHUNKS];
  std::vector<cudaEvent_t> ready;            // per input, then a start mark
  cudaEvent_t chunkReady[CHUNKS], chunkDone[CHUNKS];
  int chunks;
  long chunkCol[CHUNKS+1];
  cudaError_t pipeInputs(const void *const *in, void *const *dev,
                         cudaStream_t s);
  // Outputs copied out to the host on the side stream while the last outer
  // transform still runs: a host call sets outChunks, and that transform
  // is launched in column ranges [outCol[k], outCol[k+1]), outDone[k]
  // recorded after range k; the copy of range k waits for it.
  static const int OUT_CHUNKS=2;
  int outChunks;
  long outCol[CHUNKS+1];
  cudaEvent_t outDone[CHUNKS], outCopied;
  cudaError_t planOutputs(cudaStream_t s);
  void allocate();
  void tune();
  bool directSegments() const;
  cudaError_t runZeroCopy(const void *const *hin, const void *const *in,
                          void *const *hout, void *const *out, int wayIn,
                          int wayOut, cudaStream_t s);
  void measureHostPath(cudaStream_t s);
};

// Twiddle table W_n^t = exp(2 pi i t/n), t < n, on the current device,
// cached for the life of the process.  prec selects double2 or the float4
// (hi, lo) split.
// Standalone padded transform along one axis of C interleaved columns: the
// forward and backward transforms of fftPad / fftPadCentered / fftPadReal
// as a public device API (convolve.h:515-536, 623-646, 855-877; the
// reference's tests/hybrid.cc drives them the same way).
//   complex kinds: f is L x C complex (element (s, c) at s*C + c); F is
//     N x C complex with row k = r*m + j holding residue r, entry j, the
//     padded DFT (sign +1) at transformed index q*j + r:
//       F[r*m+j][c] = sum_s f[s][c] exp(+2 pi i (s - cshift)(q j + r) / N);
//     backward is the unnormalised adjoint, accumulated over residues:
//       f[s][c] = sum_{r,j} F[r*m+j][c] exp(-2 pi i (s - cshift)(q j + r)/N).
//   real kind: f is L x C real; F is (N/2+1) x C complex in natural order
//     (row k: frequency k); backward is the matching complex-to-real sum.
//   Hermitian kind: f is ceil(L/2) x C complex (the stored modes k >= 0,
//     f_0 real); F is N x C real, F[t][c] = sum_{|k|<H} f_k w^{k t} with
//     f_{-k} = conj(f_k) (fftPadHermitian's explicit forward, m = N);
//     backward is the real-to-complex sum over t with w^{-k t}.
// backward(forward(f)) = N f.
class PadTransform {
public:
  PadTransform(int kind, long L, long M, long C, long mForce, int prec);
  cudaError_t forward(const void *f, void *F, cudaStream_t s);
  cudaError_t backward(const void *F, void *f, cudaStream_t s);
  const AxisPlan& plan() const {return a;}
  long columns() const {return C;}
  int precision() const {return prec;}
  size_t inElements() const;
  size_t outElements() const;
  // Whether f (data side) and F (transform side) meet the element
  // alignment the kernels' vector accesses need.
  bool aligned(const void *f, const void *F) const;
private:
  AxisPlan a;
  long C;
  int prec;
  template<typename T> cudaError_t runT(const void *in, void *out, bool fwd,
                                        cudaStream_t s);
};

// Plain unnormalised FFTs of length n, the fft1d / mfft1d / rcfft1d /
// mrcfft1d / crfft1d / mcrfft1d classes of fftw++.h (fftw++.h:556-1197; the
// 2D and 3D classes compose passes of these), on the shared-memory radix
// kernels of the convolutions.  C interleaved sequences in each of B
// batches: element s of sequence c in batch b is at b*batch + s*stride + c,
// counted in the element type of each side (real values on the real side
// of r2c/c2r).  Signs follow FFTW: c2c either, r2c -1, c2r +1.  n is a
// product of 2, 3, 5 and 7 (even for real transforms).  Lengths beyond one
// CTA's shared memory (complex, contiguous sequences: C = 1, unit strides)
// take two passes through a device scratch array: n = n1 n2, columns of
// length n1 with the W_n twiddle, then rows of length n2 (the four-step
// FFT; sign +1 in decimation-in-frequency order, sign -1 in
// decimation-in-time order, so the twiddle always sits on the side of the
// kernel that applies it).
enum FFTKind {FFT_C2C=0, FFT_R2C=1, FFT_C2R=2};

class PlainFFT {
public:
  PlainFFT(int kind, long n, int sign, long C, long B, long istride,
           long ibatch, long ostride, long obatch, int prec);
  ~PlainFFT();
  cudaError_t execute(const void *in, void *out, cudaStream_t s);
  int columnsPerCTA() const {return tile;}
  bool aligned(const void *in, const void *out) const;
  bool twoPass() const {return n1 > 0;}
private:
  int kind, sign, prec;
  long n, C, B, istride, ibatch, ostride, obatch;
  int tile;
  long n1, n2;                 // two-pass factors (0: one pass)
  int tile1, tile2;
  void *scratch;               // n x B complex (two-pass only)
  template<typename T> cudaError_t runT(const void *in, void *out,
                                        cudaStream_t s);
  template<typename T> cudaError_t runTwoPass(const void *in, void *out,
                                              cudaStream_t s);
};

const void *twiddles(long n, int prec);

// Every device allocation of the library goes through devAlloc.  Failure
// injection for tests (host side): failAllocationAfter(n) makes the n-th
// following allocation (0: the next one) fail as cudaMalloc would; -1
// turns it off.
cudaError_t devAlloc(void **p, size_t bytes);
void failAllocationAfter(long n);

std::string lastError();
void setLastError(const std::string& s);

} // namespace fgb
