// kernels.cuh -- parameter blocks of the GB300 hybrid-convolution kernels.
//
// Three kernel families cover every padded-transform kind of FFTW++'s
// convolve.h on one GPU:
//
//  * row kernels: the whole padded sub-convolution along the contiguous
//    (innermost) axis of one row, on chip: load the A input rows, for every
//    residue r form the folded, pre-twiddled length-m block, FFT (+1), apply
//    the multiplier, inverse FFT (-1) and accumulate the post-twiddled block
//    into the B output rows.  Padded data never leaves shared memory
//    (fftPad/fftPadCentered residue loop, convolve.cc:849-1965; multiplier
//    convolve.cc:26-110; Convolution::convolveRaw convolve.cc:7513-7575).
//    A Hermitian variant runs the complex-to-real / real-to-complex pair
//    through a half-length complex FFT (fftPadHermitian, convolve.cc:4309).
//  * outer forward kernels: one CTA per (column tile, residue r, batch,
//    input) computes the residue block r of the padded transform along a
//    strided axis for a tile of adjacent columns and writes it to an HBM
//    staging buffer laid out [residue][j][column] (fftPad*::forward*Many,
//    the x/y stages of Convolution2/3, convolve.h:1415-1420).
//  * outer backward kernels: one CTA per (column tile, batch, output) loops
//    over all residues, inverse-transforms each block and accumulates into
//    its output tile (fftPad*::backward*Many).  Real data along the outer
//    axis (fftPadReal) uses an explicit packed real FFT instead.
#pragma once

#include "fft_smem.cuh"

#include <type_traits>

namespace fgb {

// The row and outer kernels transform in place (fftDIF/fftDIT, one buffer)
// on the FP32 pipe; the FP64 form keeps the ping-pong Stockham transform,
// which measured faster on GB300's FP64 pipe.
template<typename T> __host__ __device__ constexpr bool inplaceFFT()
{
  return !std::is_same<T,double>::value;
}

#define FGB_MAXA 8

enum MultKind {
  MULT_NONE=0, MULT_BINARY=1, MULT_REALBINARY=2, MULT_CORRELATION=3,
  MULT_REALJACOBIAN=4, MULT_JACOBIAN=5, MULT_REALJACADJ=6, MULT_DOT=7,
  MULT_REALDOT=8,
  MULT_USER=9              // a device functor compiled by the caller
                           // (fftwpp_gb300_mult.cuh); the built-in kernels
                           // treat it as no multiplication
};

// Where every multiplier slot of the innermost-axis kernels lies on the
// padded grid, for multipliers that depend on position (the counterpart of
// the reference's Indices, convolve.h:48-82, whose index[] holds the outer
// axes' transformed indices and whose fft->index(r, i) gives the inner
// one, convolve.h:297-326).  A row of the innermost kernel is a staging row
// of the outer axes: in 2D the row of axis 0, in 3D row0 * rowsY + row1.
// A complex outer axis stores residue r, entry j in row r*m + j (entries
// in mixed-radix digit-reversed order when rev is set), transformed index
// q*j + r; a real outer axis stores frequency k in row k.
struct IndexMap {
  int dim;                 // axes of the convolution
  int N[3];                // padded length of each axis
  int m[2], q[2];          // outer axes: residue block length and count
  int real0;               // axis 0 is real (rows are frequencies)
  int rev[2];              // outer axis rows digit-reversed within a block
  int nst[2];              // ... over these radices (fftDIF order)
  unsigned char radix[2][FGB_MAXSTAGES];
  long long rowsY;         // 3D: staging rows of axis 1 per row of axis 0
  int longQ;               // innermost axis on the long path: its column
                           // DFT length q (row = outer row * q + k1, inner
                           // index k1 + q k2); 0 otherwise
};

template<typename T>
struct RowPlan {
  const cplx<T> *in[FGB_MAXA];
  cplx<T> *out[FGB_MAXA];
  long long rowStride;     // elements between consecutive rows
  long long nrows;
  int L;                   // stored complex values per row
  int m, q, N;             // residue block length, residues, padded length
  int cshift;              // centred origin offset (0 for fftPad)
  int A, B, mult;
  int realIO;              // real data in and out (1D fftPadReal rows)
  int rpc;                 // rows per CTA (their columns are interleaved)
  int io64;                // float-float mode: bit 0, in[] holds FP64
                           // values; bit 1, out[] takes FP64 values
  int direct;              // one residue and one fold (q = 1, L <= m): rows
                           // load straight into the transform buffer and
                           // store straight from it (no staging, no
                           // accumulator)
  const int *ioShift;      // float-float range guard: device exponents,
                           // [a] input a, [8+b] output b (NULL: none)
  T scale;
  FFTPlanDev fp;           // length-m complex FFT
  const typename TwT<T>::type *twN;   // W_N^t, t < N
  IndexMap im;             // slot positions (position-dependent multipliers)
};

template<typename T>
struct HermRowPlan {
  const cplx<T> *in[FGB_MAXA];
  cplx<T> *out[FGB_MAXA];
  long long rowStride;
  long long nrows;
  int H;                   // stored Hermitian modes (k = 0..H-1)
  int N, Nh;               // real padded length (even) and N/2
  int A, B, mult;
  int rpc;                 // rows per CTA
  int io64;                // as RowPlan::io64
  const int *ioShift;      // as RowPlan::ioShift
  T scale;
  FFTPlanDev fp;           // length-Nh complex FFT
  const typename TwT<T>::type *twN;   // W_N^t, t < N
  IndexMap im;             // slot positions (position-dependent multipliers)
};

enum FlatMode {FLAT_PAD=0, FLAT_CENTERED=1, FLAT_HERMITIAN=2, FLAT_REAL=3};

template<typename T>
struct OuterPlan {
  const cplx<T> *in[FGB_MAXA];
  cplx<T> *out[FGB_MAXA];
  int count;               // arrays processed (A forward, B backward)
  long long inBatch, outBatch;   // elements between batches
  int nbatch;
  long long inRow, outRow; // elements between consecutive axis positions
  int C;                   // columns per axis position
  long long Ltot;          // element (s,c) of the data side is valid iff
                           // s*dataRow + c < Ltot
  int L, m, q, N, cshift;
  int tile;
  int io64;                // as RowPlan::io64
  const int *ioShift;      // as RowPlan::ioShift
  int inplace;             // FP32-pipe modes with L <= m and no twX: fold
                           // from memory and transform in place, rows of
                           // a residue block in digit-reversed order
  int conj;                // real kernels: conjugate the complex side
                           // (the sign -1 r2c / sign +1 c2r of plain FFTs)
  int cz;                  // data side with strides: column c lies at
  long long cs;            // (c / cz) cs + c % cz (cz = 0: at c)
  int kc;                  // real kernels: complex-side rows stored (the
                           // ceil(L/2) Hermitian modes), 0 for all N/2+1
  int flat;                // long rows (twX set, q = 1): position n of the
                           // flattened q x C view holds data index
                           // FLAT_PAD n, FLAT_CENTERED (n + flatC) mod NX,
                           // FLAT_HERMITIAN the Hermitian-mirrored modes
                           // (n < Ltot, conj of NX - n), FLAT_REAL n of a
                           // real array
  long long flatC;
  T scale;
  FFTPlanDev fp;           // length-m (complex) or length-N/2 (real) FFT
  const typename TwT<T>::type *twN;
  const typename TwT<T>::type *twX;  // optional W_NX^{col*k} (1D long path)
  long long NX;
};

// ---------------------------------------------------------------------------
// Persistent batched launch of many independent 1D convolutions of uneven
// lengths (no reference counterpart: the reference runs one Convolution
// object per problem).  Tasks are dequeued in topological order from one
// global counter: the column-forward tiles of every long problem, then every
// short problem as a whole row convolution, then the rows of the long
// problems, then their column-backward tiles.  A row task waits until all
// forward tiles of its problem are done, a backward tile until all rows are;
// both waits are bounded (spinLimit polls), and a wait that gives up sets
// *err and skips its task instead of hanging.
enum BatchTaskType {TASK_SMALL=0, TASK_COLFWD=1, TASK_ROW=2, TASK_COLBWD=3};

struct BatchTask {
  int type, prob, i, j;     // i: row or column tile, j: array index
};

// Pointer fields of the plans hold offsets into the caller's packed arrays
// when the matching bit of `rel` is set (bit 0 row.in, 1 row.out, 2 fwd.in,
// 3 bwd.out); otherwise they are absolute staging-buffer addresses.
template<typename T>
struct BatchProblem {
  RowPlan<T> row;
  OuterPlan<T> fwd, bwd;
  int rel;
  int nfwd;                 // forward tiles of a long problem (tiles x A)
  int nrows;                // rows of a long problem
};

template<typename T>
struct BatchArgs {
  const BatchProblem<T> *probs;
  const BatchTask *tasks;
  int ntasks;
  int *queue;               // dequeue counter (zeroed before every launch)
  int *done;                // 2 counters per problem (zeroed likewise)
  int *err;                 // set when a wait gave up
  long long spinLimit;
  int mult, A, B;           // shared by every problem of the batch
  void *inBase[FGB_MAXA];
  void *outBase[FGB_MAXA];
};

template<typename T> cudaError_t launchBatch(const BatchArgs<T>& P, int grid,
                                             int threads, size_t smem,
                                             cudaStream_t s);
template<typename T> int batchBlocksPerSM(int threads, size_t smem, int mult,
                                          int A, int B);

// Host launchers (kernels.cu).
template<typename T> cudaError_t launchRow(const RowPlan<T>& P, int threads,
                                           long long grid, cudaStream_t s);
template<typename T> cudaError_t launchHermRow(const HermRowPlan<T>& P,
                                               int threads, long long grid,
                                               cudaStream_t s);
template<typename T> cudaError_t launchOuterFwd(const OuterPlan<T>& P,
                                                int threads, cudaStream_t s);
template<typename T> cudaError_t launchOuterBwd(const OuterPlan<T>& P,
                                                int threads, cudaStream_t s);
template<typename T> cudaError_t launchOuterRealFwd(const OuterPlan<T>& P,
                                                    int threads,
                                                    cudaStream_t s);
template<typename T> cudaError_t launchOuterRealBwd(const OuterPlan<T>& P,
                                                    int threads,
                                                    cudaStream_t s);

// Range guard of the float-float mode: the largest exponent of each of the
// `count` FP64 input arrays (n doubles each) gives the power-of-two scale
// of its values on the way in and, by the multiplier's algebra, of every
// output on the way out; written to state[16+a] and state[24+b] (state:
// 32 ints, zero before the first launch; the launch leaves its
// accumulators zeroed again).
struct FFScaleArgs {
  const unsigned long long *in[FGB_MAXA];
  int count, B, mult;
  long long n;
  int *state;
};
cudaError_t launchFFScale(const FFScaleArgs& P, cudaStream_t s);

// Copy `count` arrays of `bytes` bytes each (16-byte aligned, a multiple of
// 16) with the SMs.
struct CopyArgs {
  const void *src[FGB_MAXA];
  void *dst[FGB_MAXA];
  int count;
  size_t bytes;
};
cudaError_t launchBulkCopy(const CopyArgs& P, cudaStream_t s);

// fft0 origin shift: negate the real entries (i, j, k) of an nx x ny x nz
// array with i + j odd (nz = 1: with i odd).
cudaError_t launchOriginShift(void *f, long long nx, long long ny,
                              long long nz, bool f64, cudaStream_t s);

// The innermost-axis launches of a convolution whose multiplier is a
// caller's device functor: the functor's header (fftwpp_gb300_mult.cuh)
// implements this interface by instantiating the row kernels with it, and
// Conv routes its row launches through it.  Unsupported precisions return
// cudaErrorNotSupported.
struct RowLaunchers {
  virtual ~RowLaunchers() {}
  virtual int inputs() const=0;       // the functor's A
  virtual int outputs() const=0;      // and B
  virtual cudaError_t row(const RowPlan<double>& P, int threads,
                          long long grid, cudaStream_t s) const=0;
  virtual cudaError_t row(const RowPlan<float>& P, int threads,
                          long long grid, cudaStream_t s) const=0;
  virtual cudaError_t row(const RowPlan<ff>& P, int threads,
                          long long grid, cudaStream_t s) const=0;
  virtual cudaError_t herm(const HermRowPlan<double>& P, int threads,
                           long long grid, cudaStream_t s) const=0;
  virtual cudaError_t herm(const HermRowPlan<float>& P, int threads,
                           long long grid, cudaStream_t s) const=0;
  virtual cudaError_t herm(const HermRowPlan<ff>& P, int threads,
                           long long grid, cudaStream_t s) const=0;
};

// Shared-memory bytes each kernel needs (for plan-time sizing).
template<typename T> size_t rowSmem(int L, int m, int A, int B, int rpc=1,
                                    int direct=0);
template<typename T> size_t hermRowSmem(int H, int Nh, int A, int rpc=1);
template<typename T> size_t outerFwdSmem(int L, int m, int tile,
                                         int inplace=0);
// q == 1: the backward writes its outputs without an accumulator; q = 0
// sizes for any residue count.
template<typename T> size_t outerBwdSmem(int L, int m, int tile, int q=0,
                                         int inplace=0);
template<typename T> size_t outerRealSmem(int L, int Nh, int tile);

} // namespace fgb
