// rowkernels.cuh -- the innermost-axis kernels of the GB300 hybrid
// convolution (complex rows and Hermitian rows), templated on the
// multiplier so that both the library's built-in multipliers and a
// caller's device functor (include/fftwpp_gb300_mult.cuh) are compiled into
// the row kernel itself: the multiply stays straight-line code on registers
// between the forward and inverse transforms, as FFTW++ calls its
// multiplier between them (Convolution::operate, convolve.h:1120-1135).
#pragma once

#include "kernels.cuh"

#include <algorithm>
#include <climits>
#include <type_traits>

namespace fgb {

// ---------------------------------------------------------------------------
// Multipliers (convolve.cc:26-110 and the 2D advection Jacobian), applied to
// the A values X[0..A-1] of one transformed slot; results overwrite
// X[0..B-1].  "Real" multipliers act lane-wise on the two doubles of a slot,
// which is how the reference applies them to its double-valued buffers
// (realMultBinary, convolve.cc:60-83).
template<typename T>
__device__ __forceinline__ void applyMult(int kind, cplx<T> *X, int A)
{
  switch(kind) {
    case MULT_BINARY:
      X[0]=cmul(X[0],X[1]);
      break;
    case MULT_REALBINARY:
      X[0]=mk(X[0].x*X[1].x,X[0].y*X[1].y);
      break;
    case MULT_CORRELATION:
      X[0]=cmulconj(X[0],X[1]);
      break;
    case MULT_REALJACOBIAN:
      X[0]=mk(fma(X[0].x,X[3].x,-X[1].x*X[2].x),
              fma(X[0].y,X[3].y,-X[1].y*X[2].y));
      break;
    case MULT_JACOBIAN:
      X[0]=cmul(X[0],X[3])-cmul(X[1],X[2]);
      break;
    case MULT_REALJACADJ: {
      // Inputs u0..u3 and the back-propagated field g; outputs the four
      // lane-wise partial products dJ/du_i * g of J = u0 u3 - u1 u2.
      cplx<T> g=X[4];
      cplx<T> u0=X[0], u1=X[1], u2=X[2], u3=X[3];
      X[0]=mk(g.x*u3.x,g.y*u3.y);
      X[1]=mk(-g.x*u2.x,-g.y*u2.y);
      X[2]=mk(-g.x*u1.x,-g.y*u1.y);
      X[3]=mk(g.x*u0.x,g.y*u0.y);
      break;
    }
    case MULT_DOT: {
      // Sum of A/2 binary products: X[0] = sum_k X[k] X[A/2+k].
      int K=A/2;
      cplx<T> s=cmul(X[0],X[K]);
      for(int k=1; k < K; ++k) s=s+cmul(X[k],X[K+k]);
      X[0]=s;
      break;
    }
    case MULT_REALDOT: {
      // The same on real data (two doubles per complex slot).
      int K=A/2;
      cplx<T> s=mk(X[0].x*X[K].x,X[0].y*X[K].y);
      for(int k=1; k < K; ++k)
        s=mk(fma(X[k].x,X[K+k].x,s.x),fma(X[k].y,X[K+k].y,s.y));
      X[0]=s;
      break;
    }
    default:
      break;
  }
}

// Compile-time input/output counts of the fixed-arity multipliers; the
// row kernels are instantiated per multiplier so that the fused multiply is
// straight-line code on registers (MULT_GENERIC: runtime kind and counts).
#define MULT_GENERIC (-1)
template<int K> struct MultArity {static const int A=0, B=0;};
template<> struct MultArity<MULT_BINARY> {static const int A=2, B=1;};
template<> struct MultArity<MULT_REALBINARY> {static const int A=2, B=1;};
template<> struct MultArity<MULT_REALJACOBIAN> {static const int A=4, B=1;};
template<> struct MultArity<MULT_REALJACADJ> {static const int A=5, B=4;};

// Multiply one transformed slot: the A values at X[sp(base+a*stride)] in,
// the B results back to X[sp(base+b*stride)].
template<int K, typename T>
__device__ __forceinline__ void multiplySlot(cplx<T> *X, int base, int stride,
                                             int A, int B, int kind)
{
  if constexpr(MultArity<K>::A > 0) {
    constexpr int KA=MultArity<K>::A, KB=MultArity<K>::B;
    cplx<T> v[KA];
#pragma unroll
    for(int a=0; a < KA; ++a) v[a]=nrm(X[sp(base+a*stride)]);
    applyMult(K,v,KA);
#pragma unroll
    for(int b=0; b < KB; ++b) X[sp(base+b*stride)]=v[b];
  } else {
    cplx<T> v[FGB_MAXA];
    for(int a=0; a < A; ++a) v[a]=nrm(X[sp(base+a*stride)]);
    applyMult(kind,v,A);
    for(int b=0; b < B; ++b) X[sp(base+b*stride)]=v[b];
  }
}

// The specialised instantiation serving a (mult, A, B), or MULT_GENERIC.
inline int multVariant(int mult, int A, int B)
{
  switch(mult) {
    case MULT_BINARY: return A == 2 && B == 1 ? MULT_BINARY : MULT_GENERIC;
    case MULT_REALBINARY:
      return A == 2 && B == 1 ? MULT_REALBINARY : MULT_GENERIC;
    case MULT_REALJACOBIAN:
      return A == 4 && B == 1 ? MULT_REALJACOBIAN : MULT_GENERIC;
    case MULT_REALJACADJ:
      return A == 5 && B == 4 ? MULT_REALJACADJ : MULT_GENERIC;
    default: return MULT_GENERIC;
  }
}

// ---------------------------------------------------------------------------
// The multiplier as a type parameter of the innermost-axis kernels.  A
// built-in multiplier K is BuiltinMult<K>; a caller's device functor F is
// UserMult<F> (include/fftwpp_gb300_mult.cuh), which also receives each
// slot's position on the padded grid.

template<int K> struct BuiltinMult {
  static constexpr bool positional=false;
  template<typename T>
  __device__ __forceinline__ void operator()(cplx<T> *X, int base, int stride,
                                             int A, int B, int kind) const
  {
    multiplySlot<K>(X,base,stride,A,B,kind);
  }
};

// The position of a slot handed to a position-dependent multiplier: for
// every axis d (outermost first) the transformed index index[d], the
// position on the padded grid of axis d, 0 <= index[d] < size[d] (the
// padded length); on a real outer axis the frequency 0 <= index[0] <=
// size[0]/2.  These are the values the reference's Indices::index[] and
// fftBase::index(r, i) give a multiplier (convolve.h:48-82, 297-326).
struct Indices {
  int dim;
  int index[3];
  int size[3];
};

// Natural index of position p after a decimation-in-frequency transform
// (fftDIF) over the given radices: p = sum_s d_s n/(R_0...R_s) maps to
// k = d_0 + R_0 (d_1 + R_1 (d_2 + ...)).
template<typename R>
__device__ __forceinline__ int digitRev(int p, int n, int nst, const R *radix)
{
  int k=0, w=n, mul=1;
  for(int s=0; s < nst; ++s) {
    const int r=radix[s];
    w /= r;
    const int d=p/w;
    p -= d*w;
    k += d*mul;
    mul *= r;
  }
  return k;
}

__device__ __forceinline__ int outerAxisIndex(const IndexMap& im, int d,
                                              long long row)
{
  if(d == 0 && im.real0) return (int) row;
  const int m=im.m[d];
  const int r=(int) (row/m);
  int j=(int) (row-(long long) r*m);
  if(im.rev[d]) j=digitRev(j,m,im.nst[d],im.radix[d]);
  return im.q[d]*j+r;
}

// Indices of the outer axes of innermost-kernel row `row`; the caller
// fills in the inner entry.
__device__ __forceinline__ Indices outerIndices(const IndexMap& im,
                                                long long row)
{
  Indices ix;
  ix.dim=im.dim;
  for(int d=0; d < 3; ++d) {
    ix.size[d]=d < im.dim ? im.N[d] : 1;
    ix.index[d]=0;
  }
  if(im.dim == 2) ix.index[0]=outerAxisIndex(im,0,row);
  else if(im.dim == 3) {
    const long long r0=row/im.rowsY;
    ix.index[0]=outerAxisIndex(im,0,r0);
    ix.index[1]=outerAxisIndex(im,1,row-r0*im.rowsY);
  }
  return ix;
}

__device__ __forceinline__ double nrmS(double a) {return a;}
__device__ __forceinline__ float nrmS(float a) {return a;}
__device__ __forceinline__ ff nrmS(ff a) {return nrm(a);}

// A caller's functor F: static constexpr int A, B (values in, results out)
// and a device call operator template<class V> void operator()(V *v, const
// Indices& ix) const, V = cplx<T> on complex data and T on real data (a
// Hermitian innermost axis: one real value per grid point, as the reference
// presents double buffers to its real multipliers).
template<class F> struct UserMult {
  static constexpr bool positional=true;
  F f;
  template<typename T>
  __device__ __forceinline__ void at(cplx<T> *X, int base, int stride,
                                     const Indices& ix) const
  {
    cplx<T> v[F::A];
#pragma unroll
    for(int a=0; a < F::A; ++a) v[a]=nrm(X[sp(base+a*stride)]);
    f(v,ix);
#pragma unroll
    for(int b=0; b < F::B; ++b) X[sp(base+b*stride)]=v[b];
  }
  // The two real grid points k and k+1 held by one complex slot.
  template<typename T>
  __device__ __forceinline__ void atReal(cplx<T> *X, int base, int stride,
                                         Indices ix, int k) const
  {
    T u[F::A], w[F::A];
#pragma unroll
    for(int a=0; a < F::A; ++a) {
      const cplx<T> c=X[sp(base+a*stride)];
      u[a]=nrmS(c.x);
      w[a]=nrmS(c.y);
    }
    ix.index[ix.dim-1]=k;
    f(u,ix);
    ix.index[ix.dim-1]=k+1;
    f(w,ix);
#pragma unroll
    for(int b=0; b < F::B; ++b) X[sp(base+b*stride)]=mk(u[b],w[b]);
  }
};

// One slot of a complex row: entry j of residue r (REV: j in the
// digit-reversed order of the row FFT) of row `row`.
template<class Mul, bool REV, typename T>
__device__ __forceinline__ void mulRowSlot(const Mul& mul, const RowPlan<T>& P,
                                           cplx<T> *X, int base, int stride,
                                           long long row, int j, int r)
{
  if constexpr(Mul::positional) {
    const int jn=REV ? digitRev(j,P.fp.n,P.fp.nst,P.fp.radix) : j;
    int k=P.q*jn+r;
    long long orow=row;
    if(P.im.longQ > 0) {               // long rows: column k1 of outer row
      orow=row/P.im.longQ;
      k=(int) (row-orow*P.im.longQ)+P.im.longQ*jn;
    }
    Indices ix=outerIndices(P.im,orow);
    ix.index[P.im.dim-1]=k;
    mul.at(X,base,stride,ix);
  } else {
    mul(X,base,stride,P.A,P.B,P.mult);
  }
}

// One slot t of a Hermitian row (real grid points 2t and 2t+1).
template<class Mul, bool REV, typename T>
__device__ __forceinline__ void mulHermSlot(const Mul& mul,
                                            const HermRowPlan<T>& P,
                                            cplx<T> *X, int base, int stride,
                                            long long row, int t)
{
  if constexpr(Mul::positional) {
    const int tn=REV ? digitRev(t,P.fp.n,P.fp.nst,P.fp.radix) : t;
    mul.atReal(X,base,stride,outerIndices(P.im,row),2*tn);
  } else {
    mul(X,base,stride,P.A,P.B,P.mult);
  }
}

// ---------------------------------------------------------------------------
// FP64 values at the interface of the float-float mode.  The first kernel of
// a convolution reads the caller's FP64 arrays and the last one writes them
// (RowPlan::io64); complex FP64 and float-float elements are both 16 bytes,
// so offsets are unchanged.  The split avoids the FP64 pipe: hi keeps the
// leading 24 significand bits of x, lo the float nearest to the remaining
// 29, so hi + lo = x to 2^-48 relative; values outside [2^-70, 2^101)
// (zero, subnormals, huge values) take the FP64 conversion.
//
// Range guard: FP64 data span exponents far beyond a float's, so every
// input array a is scaled by an exact power of two 2^-sh[a] on the way in
// (its largest magnitude then lies in [1, 2)) and every output b by
// 2^sh[8+b] on the way out (ffScaleKernel in kernels.cu chooses them from
// the data and the multiplier).  Scaling by a power of two only moves the
// exponent, so it costs no accuracy.

__device__ __forceinline__ ff toFF(double x, int sh=0)
{
  unsigned long long b=(unsigned long long) __double_as_longlong(x);
  const int ef=(int) ((b >> 52) & 0x7ff);
  const int e=ef-1023-sh;
  if(ef == 0 || ef == 0x7ff || e < -70 || e > 100) {
    // keep 2^(e-52) a normal float: the FP64 conversion
    const double xs=sh ? scalbn(x,-sh) : x;
    float h=__double2float_rn(xs);
    return ff(h,__double2float_rn(xs-(double) h));
  }
  unsigned sign=(unsigned) (b >> 32) & 0x80000000u;
  float hi=__uint_as_float(sign | ((unsigned) (e+127) << 23) |
                           (unsigned) ((b >> 29) & 0x7fffffu));
  // The remaining 29 significand bits R as a float without an integer
  // conversion: R = 64 Ra + Rb, each part exact through the 2^23 bias,
  // rounded once by the multiply-add.
  unsigned R=(unsigned) (b & 0x1fffffffull);
  float ra=__fsub_rn(__uint_as_float(0x4b000000u | (R >> 6)),8388608.0f);
  float rb=__fsub_rn(__uint_as_float(0x4b000000u | (R & 63u)),8388608.0f);
  float lo=fmaf(ra,64.0f,rb);
  lo=__fmul_rn(lo,__uint_as_float((unsigned) (e-52+127) << 23)); // * 2^(e-52)
  lo=__uint_as_float(__float_as_uint(lo) | sign);
  return ffFast(hi,lo);
}

// f 2^sh widened to double exactly by moving its fields (the FP64 pipe only
// for subnormals, infinities, NaNs and results outside the double range).
__device__ __forceinline__ double widen(float f, int sh=0)
{
  unsigned u=__float_as_uint(f);
  unsigned ef=(u >> 23) & 0xffu;
  unsigned long long sign=(unsigned long long) (u & 0x80000000u) << 32;
  if((u & 0x7fffffffu) == 0) return __longlong_as_double((long long) sign);
  const int E=(int) ef+896+sh;
  if(ef == 0 || ef == 255 || E <= 0 || E >= 2047)
    return sh ? scalbn((double) f,sh) : (double) f;
  return __longlong_as_double((long long) (sign |
    ((unsigned long long) E << 52) |
    ((unsigned long long) (u & 0x7fffffu) << 29)));
}

__device__ __forceinline__ double fromFF(ff v, int sh=0)
{
  return widen(v.hi,sh)+widen(v.lo,sh);
}

// The range-guard exponent of input a (io < 8) or output io-8 of the
// float-float mode; 0 for the other modes or without a guard.
template<typename T>
__device__ __forceinline__ int ioShift(const int *sh, int io)
{
  if constexpr(std::is_same<T,ff>::value) return sh ? __ldg(sh+io) : 0;
  else return 0;
}

template<typename T>
__device__ __forceinline__ cplx<T> loadIO(const cplx<T> *p, bool f64,
                                          int sh=0)
{
  if constexpr(std::is_same<T,ff>::value) {
    if(f64) {
      double2 d=*(const double2 *) p;
      return mk(toFF(d.x,sh),toFF(d.y,sh));
    }
  }
  return *p;
}

template<typename T>
__device__ __forceinline__ T loadIOr(const T *p, bool f64, int sh=0)
{
  if constexpr(std::is_same<T,ff>::value)
    if(f64) return toFF(*(const double *) p,sh);
  return *p;
}

template<typename T>
__device__ __forceinline__ void storeIO(cplx<T> *p, cplx<T> v, bool f64,
                                        int sh=0)
{
  if constexpr(std::is_same<T,ff>::value) {
    if(f64) {
      *(double2 *) p=make_double2(fromFF(v.x,sh),fromFF(v.y,sh));
      return;
    }
  }
  *p=v;
}

template<typename T>
__device__ __forceinline__ void storeIOr(T *p, T v, bool f64, int sh=0)
{
  if constexpr(std::is_same<T,ff>::value) {
    if(f64) {
      *(double *) p=fromFF(v,sh);
      return;
    }
  }
  *p=v;
}

// Convert n elements staged in shared memory as FP64 (by cp.async) to
// float-float in place; each thread converts the elements it copied.
template<typename T>
__device__ __forceinline__ void convertStaged(cplx<T> *y, int i, int sh=0)
{
  if constexpr(std::is_same<T,ff>::value) {
    double2 d=*(double2 *) (y+i);
    y[i]=mk(toFF(d.x,sh),toFF(d.y,sh));
  }
}

// Exponent ((s-c) mod N)*r mod N of a residue twiddle (r < N; 32-bit
// arithmetic while the product fits).
__device__ __forceinline__ int twExp(int s, int c, int r, int N)
{
  int d=s-c;
  if(d < 0) d += N;
  if(N <= 65536) return (int) (((unsigned) d*(unsigned) r) % (unsigned) N);
  return (int) (((unsigned long long) d*(unsigned long long) r) %
                (unsigned long long) N);
}

// The exponent step m*r mod N between the terms s and s+m of a fold.
__device__ __forceinline__ int twStep(int m, int r, int N)
{
  return (int) (((unsigned long long) m*(unsigned long long) r) %
                (unsigned long long) N);
}

__device__ __forceinline__ int posmod(int a, int m)
{
  int r=a % m;
  return r < 0 ? r+m : r;
}

// ---------------------------------------------------------------------------
// Row kernel, complex data (fftPad / fftPadCentered along the contiguous
// axis): fold + pre-twiddle (forwardInner: Zetaqp/Zetaqm), m-point FFT, fused
// multiplier, inverse FFT, post-twiddle and accumulation over residues
// (backwardInner), normalisation (Convolution::normalize).
// Load of data another CTA of the same launch may have written: CG bypasses
// the (non-coherent) L1 with ld.global.cg.
template<bool CG>
__device__ __forceinline__ cplx<double> ldx(const cplx<double> *p)
{
  if(CG) {
    double2 v=__ldcg((const double2 *) p);
    return mk(v.x,v.y);
  }
  return *p;
}

template<bool CG>
__device__ __forceinline__ cplx<float> ldx(const cplx<float> *p)
{
  if(CG) {
    float2 v=__ldcg((const float2 *) p);
    return mk(v.x,v.y);
  }
  return *p;
}

template<bool CG>
__device__ __forceinline__ cplx<ff> ldx(const cplx<ff> *p)
{
  if(CG) {
    float4 v=__ldcg((const float4 *) p);
    return mk(ff(v.x,v.y),ff(v.z,v.w));
  }
  return *p;
}

// Asynchronous global->shared copy of one complex element (cp.async; the
// 16-byte form bypasses L1).  cpAsyncWait() waits for all of the thread's
// copies; a __syncthreads() must follow before other threads read them.
__device__ __forceinline__ void cpAsync(cplx<double> *dst,
                                        const cplx<double> *src)
{
  unsigned s=(unsigned) __cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n"
               :: "r"(s), "l"(src) : "memory");
}

__device__ __forceinline__ void cpAsync(cplx<ff> *dst, const cplx<ff> *src)
{
  unsigned s=(unsigned) __cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n"
               :: "r"(s), "l"(src) : "memory");
}

__device__ __forceinline__ void cpAsync(cplx<float> *dst,
                                        const cplx<float> *src)
{
  unsigned s=(unsigned) __cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n"
               :: "r"(s), "l"(src) : "memory");
}

__device__ __forceinline__ void cpAsyncWait()
{
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Global loads a thread issues back to back in the row kernels' load loops
// (more bytes in flight per thread than one dependent load per iteration).
#define FGB_LOADS 4

// One group of P.rpc rows of the complex row convolution (all residues),
// using the block's shared memory.  The A x rpc input rows are transformed
// together as interleaved columns col = a*rpc + rho, so the B x rpc output
// columns are a contiguous prefix for the inverse transforms.  Every thread
// of the block calls it.
template<typename T, bool CG, class Mul, bool D=false, bool R16=false>
__device__ __forceinline__ void rowConvRow(const RowPlan<T>& P,
                                           long long group,
                                           unsigned char *smemRaw,
                                           const Mul& mul)
{
  const int A=P.A, B=P.B, L=P.L, m=P.m, N=P.N, c=P.cshift, R=P.rpc;
  const int ld=A*R, lb=B*R;
  cplx<T> *fin=(cplx<T> *) smemRaw;
  cplx<T> *acc=fin+ld*L;
  cplx<T> *x=acc+lb*L;
  cplx<T> *y=x+padded(m*ld);         // ping-pong buffer of the FP64 form
  const int tid=threadIdx.x, nthr=blockDim.x;
  const typename TwT<T>::type *tw=P.twN;
  const UDiv dL(L), dLd(ld);
  const UDiv dR(R);
  const long long row0=group*R;

  if constexpr(D) {
    // One residue, one fold (RowPlan::direct; its own instantiation, so
    // that the staged path's registers do not weigh on it or it on them): slot t of column col holds f[(t + c) mod m]
    // (zero beyond L).  Reads run along each row (coalesced), FGB_LOADS
    // iterations of loads issued before any is used.
    cplx<T> *x=(cplx<T> *) smemRaw;
    cplx<T> *y=x+padded(m*ld);
    const UDiv dM(m);
    for(int i0=tid; i0 < m*ld; i0 += FGB_LOADS*nthr) {
      cplx<T> v[FGB_LOADS];
#pragma unroll
      for(int u=0; u < FGB_LOADS; ++u) {
        const int i=i0+u*nthr;
        v[u]=mk((T) 0,(T) 0);
        if(i >= m*ld) continue;
        int col=dM(i), s=i-col*m;
        int a=dR(col);
        long long row=row0+col-a*R;
        if(s < L && row < P.nrows) {
          long long off=row*P.rowStride+s;
          if(P.realIO)
            v[u]=mk(loadIOr((const T *) P.in[a]+off,P.io64 & 1,
                            ioShift<T>(P.ioShift,a)),(T) 0);
          else if(P.io64 & 1)
            v[u]=loadIO(P.in[a]+off,true,ioShift<T>(P.ioShift,a));
          else v[u]=ldx<CG>(P.in[a]+off);
        }
      }
#pragma unroll
      for(int u=0; u < FGB_LOADS; ++u) {
        const int i=i0+u*nthr;
        if(i >= m*ld) break;
        int col=dM(i), s=i-col*m;
        x[sp(posmod(s-c,m)*ld+col)]=v[u];
      }
    }
    __syncthreads();
    const cplx<T> *Z;
    if constexpr(inplaceFFT<T>() || D) {
      fftDIF<T,1,R16>(x,P.fp,ld,ld,tid,nthr);
      for(int i=tid; i < m*R; i += nthr) {
        int j=dR(i), rho=i-j*R;
        mulRowSlot<Mul,true>(mul,P,x,j*ld+rho,R,row0+rho,j,0);
      }
      __syncthreads();
      fftDIT<T,-1,R16>(x,P.fp,lb,ld,tid,nthr);
      Z=x;
    } else {
      cplx<T> *X=fftSmem<T,1>(x,y,P.fp,ld,ld,tid,nthr);
      cplx<T> *Y=X == x ? y : x;
      for(int i=tid; i < m*R; i += nthr) {
        int j=dR(i), rho=i-j*R;
        mulRowSlot<Mul,false>(mul,P,X,j*ld+rho,R,row0+rho,j,0);
      }
      __syncthreads();
      Z=fftSmem<T,-1>(X,Y,P.fp,lb,ld,tid,nthr);
    }
    for(int i=tid; i < lb*L; i += nthr) {
      int col=dL(i), s=i-col*L;
      int b=dR(col);
      long long row=row0+col-b*R;
      if(row >= P.nrows) continue;
      cplx<T> v=Z[sp(posmod(s-c,m)*ld+col)];
      long long off=row*P.rowStride+s;
      const int sh=ioShift<T>(P.ioShift,8+b);
      if(P.realIO) storeIOr((T *) P.out[b]+off,v.x*P.scale,P.io64 & 2,sh);
      else storeIO(P.out[b]+off,v*P.scale,P.io64 & 2,sh);
    }
    __syncthreads();
  } else {
    // The loads of FGB_LOADS iterations are issued before any is used.
    for(int i0=tid; i0 < ld*L; i0 += FGB_LOADS*nthr) {
      cplx<T> v[FGB_LOADS];
#pragma unroll
      for(int u=0; u < FGB_LOADS; ++u) {
        const int i=i0+u*nthr;
        v[u]=mk((T) 0,(T) 0);
        if(i >= ld*L) continue;
        int col=dL(i), s=i-col*L;
        int a=dR(col);
        long long row=row0+col-a*R;
        if(row < P.nrows) {
          long long off=row*P.rowStride+s;
          if(P.realIO)
            v[u]=mk(loadIOr((const T *) P.in[a]+off,P.io64 & 1,
                            ioShift<T>(P.ioShift,a)),(T) 0);
          else if(P.io64 & 1)
            v[u]=loadIO(P.in[a]+off,true,ioShift<T>(P.ioShift,a));
          else v[u]=ldx<CG>(P.in[a]+off);
        }
      }
#pragma unroll
      for(int u=0; u < FGB_LOADS; ++u)
        if(i0+u*nthr < ld*L) fin[i0+u*nthr]=v[u];
    }
    for(int i=tid; i < lb*L; i += nthr) acc[i]=mk((T) 0,(T) 0);
    __syncthreads();

    for(int r=0; r < P.q; ++r) {
      // Fold the data into one length-m block with the residue twiddles.
      for(int i=tid; i < m*ld; i += nthr) {
        int t=dLd(i), col=i-t*ld;
        int s0=posmod(t+c,m);
        cplx<T> sum=mk((T) 0,(T) 0);
        // The twiddle exponent advances by m r mod N from term to term.
        int e=r != 0 ? twExp(s0,c,r,N) : 0;
        const int de=r != 0 ? twStep(m,r,N) : 0;
        for(int s=s0; s < L; s += m) {
          cplx<T> v=fin[col*L+s];
          if(r != 0) {
            v=twmul<1>(v,tw[e]);
            e += de;
            if(e >= N) e -= N;
          }
          sum=accum(sum,v);
        }
        x[sp(i)]=sum;
      }
      __syncthreads();
      const cplx<T> *Z;
      if constexpr(inplaceFFT<T>()) {
        fftDIF<T,1,R16>(x,P.fp,ld,ld,tid,nthr);
        for(int i=tid; i < m*R; i += nthr) {
          int j=dR(i), rho=i-j*R;
          mulRowSlot<Mul,true>(mul,P,x,j*ld+rho,R,row0+rho,j,r);
        }
        __syncthreads();
        fftDIT<T,-1,R16>(x,P.fp,lb,ld,tid,nthr);
        Z=x;
      } else {
        cplx<T> *X=fftSmem<T,1>(x,y,P.fp,ld,ld,tid,nthr);
        cplx<T> *Y=X == x ? y : x;
        for(int i=tid; i < m*R; i += nthr) {
          int j=dR(i), rho=i-j*R;
          mulRowSlot<Mul,false>(mul,P,X,j*ld+rho,R,row0+rho,j,r);
        }
        __syncthreads();
        Z=fftSmem<T,-1>(X,Y,P.fp,lb,ld,tid,nthr);
      }
      for(int i=tid; i < lb*L; i += nthr) {
        int col=dL(i), s=i-col*L;
        int t=posmod(s-c,m);
        cplx<T> v=Z[sp(t*ld+col)];
        if(r != 0) v=twmul<-1>(v,tw[twExp(s,c,r,N)]);
        acc[i]=accum(acc[i],v);
      }
      __syncthreads();
    }
    for(int i=tid; i < lb*L; i += nthr) {
      int col=dL(i), s=i-col*L;
      int b=dR(col);
      long long row=row0+col-b*R;
      if(row >= P.nrows) continue;
      long long off=row*P.rowStride+s;
      const int sh=ioShift<T>(P.ioShift,8+b);
      if(P.realIO)
        storeIOr((T *) P.out[b]+off,acc[i].x*P.scale,P.io64 & 2,sh);
      else storeIO(P.out[b]+off,acc[i]*P.scale,P.io64 & 2,sh);
    }
    __syncthreads();
  }
}

template<typename T, class Mul, bool D>
__global__ void __launch_bounds__(256)
rowConvKernel(const RowPlan<T> P, const Mul mul)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  const long long groups=(P.nrows+P.rpc-1)/P.rpc;
  for(long long g=blockIdx.x; g < groups; g += gridDim.x)
    rowConvRow<T,false,Mul,D>(P,g,smemRaw,mul);
}

// The same for FP32 plans with a radix-16 stage: the radix-16 code needs
// more registers, so only those plans launch it, capped at 85 registers a
// thread (three CTAs of 256 threads per SM).
template<typename T, class Mul, bool D>
__global__ void __launch_bounds__(256,3)
rowConvKernel16(const RowPlan<T> P, const Mul mul)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  const long long groups=(P.nrows+P.rpc-1)/P.rpc;
  for(long long g=blockIdx.x; g < groups; g += gridDim.x)
    rowConvRow<T,false,Mul,D,true>(P,g,smemRaw,mul);
}

// ---------------------------------------------------------------------------
// Row kernel, Hermitian data (fftPadHermitian along the contiguous axis,
// explicit padding to an even real length N): the H stored modes are packed
// into a length-N/2 complex sequence whose sign +1 FFT yields the N real
// physical values as (u[2t], u[2t+1]) pairs; the multiplier acts on those
// doubles; the sign -1 FFT of the packed product is unpacked into the H
// output modes (real-to-complex).
template<typename T, class Mul, bool R16>
__device__ __forceinline__ void hermRows(const HermRowPlan<T>& P,
                                         const Mul& mul,
                                         unsigned char *smemRaw)
{
  const int A=P.A, B=P.B, H=P.H, Nh=P.Nh, R=P.rpc;
  const int ld=A*R, lb=B*R;
  cplx<T> *x=(cplx<T> *) smemRaw;
  cplx<T> *y=x+padded(Nh*ld);        // ping-pong buffer of the FP64 form
  const int tid=threadIdx.x, nthr=blockDim.x;
  const typename TwT<T>::type *tw=P.twN;
  const T half=(T) 0.5;
  const UDiv dH(H), dLd(ld);
  const UDiv dR(R);
  const long long groups=(P.nrows+R-1)/R;

  // Rows g*R .. g*R+R-1 are transformed together; column col = a*R + rho.
  for(long long g=blockIdx.x; g < groups; g += gridDim.x) {
    const long long row0=g*R;
    // Y[k] = S + i W_N^k D with S = Z[k] + conj Z[Nh-k], D = Z[k] -
    // conj Z[Nh-k], Z read from the row itself.  One thread forms the pair
    // k, Nh-k from the same two loads: Y[Nh-k] = conj(S) + i conj(W_N^k D)
    // (since W_N^{Nh} = -1), so the pair costs one twiddle multiply.
    // Every read of the group precedes its writes, so in = out is safe.
    // The loads of FGB_LOADS iterations are issued before any is used.
    const int np=Nh/2+1;                 // k = 0 .. floor(Nh/2)
    for(int i0=tid; i0 < np*ld; i0 += FGB_LOADS*nthr) {
      cplx<T> zk[FGB_LOADS], zc[FGB_LOADS];
#pragma unroll
      for(int u=0; u < FGB_LOADS; ++u) {
        const int i=i0+u*nthr;
        int k=dLd(i), col=i-k*ld;       // col < ld: a < A for every i
        int a=dR(col);
        long long row=row0+col-a*R;
        const cplx<T> *zr=P.in[a]+row*P.rowStride;
        const bool live=i < np*ld && row < P.nrows;
        const int kk=Nh-k;
        const int sh=ioShift<T>(P.ioShift,a);
        zk[u]=live && k < H ? loadIO(zr+k,P.io64 & 1,sh) : mk((T) 0,(T) 0);
        zc[u]=live && kk < H ? loadIO(zr+kk,P.io64 & 1,sh) : mk((T) 0,(T) 0);
      }
#pragma unroll
      for(int u=0; u < FGB_LOADS; ++u) {
        const int i=i0+u*nthr;
        if(i >= np*ld) break;
        const int k=dLd(i), col=i-k*ld;
        cplx<T> a=zk[u];
        if(k == 0) a.y=(T) 0;
        const cplx<T> b=conjg(zc[u]);
        const cplx<T> S=a+b;
        cplx<T> Y, Yc;
        if constexpr(std::is_same<T,double>::value) {
          // FP64: S + (i D) W as four DFMAs, the partner as conj(2S - Y).
          const cplx<T> D=a-b;
          Y=fmaTw<1>(S,mk(-D.y,D.x),tw[k]);
          Yc=mk(fma((T) 2,S.x,-Y.x),fma((T) -2,S.y,Y.y));
        } else {
          const cplx<T> Pw=twmul<1>(a-b,tw[k]);
          Y=mk(S.x-Pw.y,S.y+Pw.x);
          Yc=mk(S.x+Pw.y,Pw.x-S.y);
        }
        x[sp(i)]=Y;
        if(k != 0 && 2*k != Nh) x[sp((Nh-k)*ld+col)]=Yc;
      }
    }
    __syncthreads();
    const cplx<T> *Z;
    if constexpr(inplaceFFT<T>()) {
      fftDIF<T,1,R16>(x,P.fp,ld,ld,tid,nthr);
      for(int i=tid; i < Nh*R; i += nthr) {
        int t=dR(i), rho=i-t*R;
        mulHermSlot<Mul,true>(mul,P,x,t*ld+rho,R,row0+rho,t);
      }
      __syncthreads();
      fftDIT<T,-1,R16>(x,P.fp,lb,ld,tid,nthr);
      Z=x;
    } else {
      cplx<T> *X=fftSmem<T,1>(x,y,P.fp,ld,ld,tid,nthr);
      cplx<T> *Y=X == x ? y : x;
      for(int i=tid; i < Nh*R; i += nthr) {
        int t=dR(i), rho=i-t*R;
        mulHermSlot<Mul,false>(mul,P,X,t*ld+rho,R,row0+rho,t);
      }
      __syncthreads();
      Z=fftSmem<T,-1>(X,Y,P.fp,lb,ld,tid,nthr);
    }
    // V[k] = (s + Q)/2 with s = Z[k] + conj Z[m], Q = W_N^{-k} (-i)(Z[k] -
    // conj Z[m]), m = Nh-k (m = 0 for k = 0).  When both k and Nh-k are
    // stored modes the lower one also writes V[Nh-k] = conj(s - Q)/2, and
    // the upper one skips.
    const T hs=half*P.scale;
    for(int i=tid; i < lb*H; i += nthr) {
      int col=dH(i), k=i-col*H;
      int b=dR(col);
      long long row=row0+col-b*R;
      const int km=k == 0 ? 0 : Nh-k;
      const bool pair=k != 0 && km < H && km != k;
      if(row >= P.nrows || (pair && km < k)) continue;
      const cplx<T> zk=Z[sp(k*ld+col)];
      const cplx<T> zm=conjg(Z[sp(km*ld+col)]);
      cplx<T> V, Vc;
      if constexpr(std::is_same<T,double>::value) {
        // FP64: hs sum, hs dd = 2 hs zk - hs sum, V = hs sum + hs Q as
        // four DFMAs, the partner as conj(2 hs sum - V).
        const cplx<T> hsum=(zk+zm)*hs;
        const T h2=hs+hs;
        const cplx<T> hdd=mk(fma(h2,zk.x,-hsum.x),fma(h2,zk.y,-hsum.y));
        V=fmaTw<-1>(hsum,mk(hdd.y,-hdd.x),tw[k]);
        Vc=mk(fma((T) 2,hsum.x,-V.x),fma((T) -2,hsum.y,V.y));
      } else {
        const cplx<T> sum=zk+zm, dd=zk-zm;
        const cplx<T> Q=twmul<-1>(mk(dd.y,-dd.x),tw[k]);
        V=(sum+Q)*hs;
        Vc=conjg(sum-Q)*hs;
      }
      cplx<T> *o=P.out[b]+row*P.rowStride;
      const int sh=ioShift<T>(P.ioShift,8+b);
      storeIO(o+k,V,P.io64 & 2,sh);
      if(pair) storeIO(o+km,Vc,P.io64 & 2,sh);
    }
    __syncthreads();
  }
}

template<typename T, class Mul>
__global__ void __launch_bounds__(256)
hermRowKernel(const HermRowPlan<T> P, const Mul mul)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  hermRows<T,Mul,false>(P,mul,smemRaw);
}

// FP32 plans with a radix-16 stage (as rowConvKernel16).
template<typename T, class Mul>
__global__ void __launch_bounds__(256,3)
hermRowKernel16(const HermRowPlan<T> P, const Mul mul)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  hermRows<T,Mul,true>(P,mul,smemRaw);
}

// ---------------------------------------------------------------------------
// Launchers of the row kernels for any multiplier type.

template<typename K>
inline cudaError_t setRowSmem(K kernel, size_t bytes)
{
  if(bytes > 48*1024)
    return cudaFuncSetAttribute(kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int) bytes);
  return cudaSuccess;
}

template<typename T, class Mul>
cudaError_t launchRowWith(const RowPlan<T>& P, const Mul& mul, int threads,
                          long long grid, cudaStream_t s)
{
  const size_t sm=rowSmem<T>(P.L,P.m,P.A,P.B,P.rpc,P.direct);
  const long long groups=(P.nrows+P.rpc-1)/P.rpc;
  grid=std::min(std::min(grid,groups),(long long) INT_MAX);
  if(grid < 1) return cudaSuccess;
  auto go=[&](auto kernel) {
    cudaError_t e=setRowSmem(kernel,sm);
    if(e != cudaSuccess) return e;
    kernel<<<(unsigned) grid,threads,sm,s>>>(P,mul);
    return cudaGetLastError();
  };
  if constexpr(std::is_same<T,float>::value)
    if(hasWideRadix(P.fp)) {
      if(P.direct) return go(rowConvKernel16<T,Mul,true>);
      return go(rowConvKernel16<T,Mul,false>);
    }
  if(P.direct) return go(rowConvKernel<T,Mul,true>);
  return go(rowConvKernel<T,Mul,false>);
}

template<typename T, class Mul>
cudaError_t launchHermRowWith(const HermRowPlan<T>& P, const Mul& mul,
                              int threads, long long grid, cudaStream_t s)
{
  const size_t sm=hermRowSmem<T>(P.H,P.Nh,P.A,P.rpc);
  const long long groups=(P.nrows+P.rpc-1)/P.rpc;
  grid=std::min(std::min(grid,groups),(long long) INT_MAX);
  if(grid < 1) return cudaSuccess;
  auto go=[&](auto kernel) {
    cudaError_t e=setRowSmem(kernel,sm);
    if(e != cudaSuccess) return e;
    kernel<<<(unsigned) grid,threads,sm,s>>>(P,mul);
    return cudaGetLastError();
  };
  if constexpr(std::is_same<T,float>::value)
    if(hasWideRadix(P.fp)) return go(hermRowKernel16<T,Mul>);
  return go(hermRowKernel<T,Mul>);
}

} // namespace fgb
