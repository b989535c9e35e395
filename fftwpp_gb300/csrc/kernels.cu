// kernels.cu -- GB300 (sm_103a) kernels of the hybrid dealiased convolution.
// See kernels.cuh for the decomposition; reference routines are cited per
// kernel.
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
static int multVariant(int mult, int A, int B)
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
// FP64 values at the interface of the float-float mode.  The first kernel of
// a convolution reads the caller's FP64 arrays and the last one writes them
// (RowPlan::io64); complex FP64 and float-float elements are both 16 bytes,
// so offsets are unchanged.  The split avoids the FP64 pipe: hi keeps the
// leading 24 significand bits of x, lo the float nearest to the remaining
// 29, so hi + lo = x to 2^-48 relative; values outside [2^-70, 2^101)
// (zero, subnormals, huge values) take the FP64 conversion.

__device__ __forceinline__ ff toFF(double x)
{
  unsigned long long b=(unsigned long long) __double_as_longlong(x);
  int e=(int) ((b >> 52) & 0x7ff)-1023;
  if(e < -70 || e > 100) {          // keep 2^(e-52) a normal float
    float h=__double2float_rn(x);
    return ff(h,__double2float_rn(x-(double) h));
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

// A float widened to double exactly by moving its fields (the FP64 pipe
// only for subnormals, infinities and NaNs).
__device__ __forceinline__ double widen(float f)
{
  unsigned u=__float_as_uint(f);
  unsigned ef=(u >> 23) & 0xffu;
  unsigned long long sign=(unsigned long long) (u & 0x80000000u) << 32;
  if((u & 0x7fffffffu) == 0) return __longlong_as_double((long long) sign);
  if(ef == 0 || ef == 255) return (double) f;
  return __longlong_as_double((long long) (sign |
    ((unsigned long long) (ef+896) << 52) |
    ((unsigned long long) (u & 0x7fffffu) << 29)));
}

__device__ __forceinline__ double fromFF(ff v)
{
  return widen(v.hi)+widen(v.lo);
}

template<typename T>
__device__ __forceinline__ cplx<T> loadIO(const cplx<T> *p, bool f64)
{
  if constexpr(std::is_same<T,ff>::value) {
    if(f64) {
      double2 d=*(const double2 *) p;
      return mk(toFF(d.x),toFF(d.y));
    }
  }
  return *p;
}

template<typename T>
__device__ __forceinline__ T loadIOr(const T *p, bool f64)
{
  if constexpr(std::is_same<T,ff>::value)
    if(f64) return toFF(*(const double *) p);
  return *p;
}

template<typename T>
__device__ __forceinline__ void storeIO(cplx<T> *p, cplx<T> v, bool f64)
{
  if constexpr(std::is_same<T,ff>::value) {
    if(f64) {
      *(double2 *) p=make_double2(fromFF(v.x),fromFF(v.y));
      return;
    }
  }
  *p=v;
}

template<typename T>
__device__ __forceinline__ void storeIOr(T *p, T v, bool f64)
{
  if constexpr(std::is_same<T,ff>::value) {
    if(f64) {
      *(double *) p=fromFF(v);
      return;
    }
  }
  *p=v;
}

// Convert n elements staged in shared memory as FP64 (by cp.async) to
// float-float in place; each thread converts the elements it copied.
template<typename T>
__device__ __forceinline__ void convertStaged(cplx<T> *y, int i)
{
  if constexpr(std::is_same<T,ff>::value) {
    double2 d=*(double2 *) (y+i);
    y[i]=mk(toFF(d.x),toFF(d.y));
  }
}

// Exponent ((s-c) mod N)*r mod N of a residue twiddle.
__device__ __forceinline__ int twExp(int s, int c, int r, int N)
{
  int d=s-c;
  if(d < 0) d += N;
  return (int) (((unsigned long long) d*(unsigned long long) r) %
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
template<typename T, bool CG, int K, bool D=false>
__device__ __forceinline__ void rowConvRow(const RowPlan<T>& P,
                                           long long group,
                                           unsigned char *smemRaw)
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
          if(P.realIO) v[u]=mk(loadIOr((const T *) P.in[a]+off,P.io64 & 1),(T) 0);
          else if(P.io64 & 1) v[u]=loadIO(P.in[a]+off,true);
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
      fftDIF<T,1>(x,P.fp,ld,ld,tid,nthr);
      for(int i=tid; i < m*R; i += nthr) {
        int j=dR(i), rho=i-j*R;
        multiplySlot<K>(x,j*ld+rho,R,A,B,P.mult);
      }
      __syncthreads();
      fftDIT<T,-1>(x,P.fp,lb,ld,tid,nthr);
      Z=x;
    } else {
      cplx<T> *X=fftSmem<T,1>(x,y,P.fp,ld,ld,tid,nthr);
      cplx<T> *Y=X == x ? y : x;
      for(int i=tid; i < m*R; i += nthr) {
        int j=dR(i), rho=i-j*R;
        multiplySlot<K>(X,j*ld+rho,R,A,B,P.mult);
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
      if(P.realIO) storeIOr((T *) P.out[b]+off,v.x*P.scale,P.io64 & 2);
      else storeIO(P.out[b]+off,v*P.scale,P.io64 & 2);
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
          if(P.realIO) v[u]=mk(loadIOr((const T *) P.in[a]+off,P.io64 & 1),(T) 0);
          else if(P.io64 & 1) v[u]=loadIO(P.in[a]+off,true);
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
        for(int s=s0; s < L; s += m) {
          cplx<T> v=fin[col*L+s];
          if(r != 0) v=twmul<1>(v,tw[twExp(s,c,r,N)]);
          sum=accum(sum,v);
        }
        x[sp(i)]=sum;
      }
      __syncthreads();
      const cplx<T> *Z;
      if constexpr(inplaceFFT<T>()) {
        fftDIF<T,1>(x,P.fp,ld,ld,tid,nthr);
        for(int i=tid; i < m*R; i += nthr) {
          int j=dR(i), rho=i-j*R;
          multiplySlot<K>(x,j*ld+rho,R,A,B,P.mult);
        }
        __syncthreads();
        fftDIT<T,-1>(x,P.fp,lb,ld,tid,nthr);
        Z=x;
      } else {
        cplx<T> *X=fftSmem<T,1>(x,y,P.fp,ld,ld,tid,nthr);
        cplx<T> *Y=X == x ? y : x;
        for(int i=tid; i < m*R; i += nthr) {
          int j=dR(i), rho=i-j*R;
          multiplySlot<K>(X,j*ld+rho,R,A,B,P.mult);
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
      if(P.realIO) storeIOr((T *) P.out[b]+off,acc[i].x*P.scale,P.io64 & 2);
      else storeIO(P.out[b]+off,acc[i]*P.scale,P.io64 & 2);
    }
    __syncthreads();
  }
}

template<typename T, int K, bool D>
__global__ void __launch_bounds__(256)
rowConvKernel(const RowPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  const long long groups=(P.nrows+P.rpc-1)/P.rpc;
  for(long long g=blockIdx.x; g < groups; g += gridDim.x)
    rowConvRow<T,false,K,D>(P,g,smemRaw);
}

// ---------------------------------------------------------------------------
// Row kernel, Hermitian data (fftPadHermitian along the contiguous axis,
// explicit padding to an even real length N): the H stored modes are packed
// into a length-N/2 complex sequence whose sign +1 FFT yields the N real
// physical values as (u[2t], u[2t+1]) pairs; the multiplier acts on those
// doubles; the sign -1 FFT of the packed product is unpacked into the H
// output modes (real-to-complex).
template<typename T, int K>
__global__ void __launch_bounds__(256)
hermRowKernel(const HermRowPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
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
    // Y[k] = (Z[k] + conj Z[Nh-k]) + i W_N^k (Z[k] - conj Z[Nh-k]), with
    // Z read from the row itself (the two reads of an element are L1/L2
    // hits; every read of the group precedes its writes, so in = out is
    // safe).
    // The loads of FGB_LOADS iterations are issued before any is used.
    for(int i0=tid; i0 < Nh*ld; i0 += FGB_LOADS*nthr) {
      cplx<T> zk[FGB_LOADS], zc[FGB_LOADS];
#pragma unroll
      for(int u=0; u < FGB_LOADS; ++u) {
        const int i=i0+u*nthr;
        int k=dLd(i), col=i-k*ld;       // col < ld: a < A for every i
        int a=dR(col);
        long long row=row0+col-a*R;
        const cplx<T> *zr=P.in[a]+row*P.rowStride;
        const bool live=i < Nh*ld && row < P.nrows;
        const int kk=Nh-k;
        zk[u]=live && k < H ? loadIO(zr+k,P.io64 & 1) : mk((T) 0,(T) 0);
        zc[u]=live && kk < H ? loadIO(zr+kk,P.io64 & 1) : mk((T) 0,(T) 0);
      }
#pragma unroll
      for(int u=0; u < FGB_LOADS; ++u) {
        const int i=i0+u*nthr;
        if(i >= Nh*ld) break;
        const int k=dLd(i);
        cplx<T> a=zk[u];
        if(k == 0) a.y=(T) 0;
        cplx<T> b=conjg(zc[u]);
        cplx<T> s=a+b;
        cplx<T> d=twmul<1>(a-b,tw[k]);
        x[sp(i)]=mk(s.x-d.y,s.y+d.x);
      }
    }
    __syncthreads();
    const cplx<T> *Z;
    if constexpr(inplaceFFT<T>()) {
      fftDIF<T,1>(x,P.fp,ld,ld,tid,nthr);
      for(int i=tid; i < Nh*R; i += nthr) {
        int t=dR(i), rho=i-t*R;
        multiplySlot<K>(x,t*ld+rho,R,A,B,P.mult);
      }
      __syncthreads();
      fftDIT<T,-1>(x,P.fp,lb,ld,tid,nthr);
      Z=x;
    } else {
      cplx<T> *X=fftSmem<T,1>(x,y,P.fp,ld,ld,tid,nthr);
      cplx<T> *Y=X == x ? y : x;
      for(int i=tid; i < Nh*R; i += nthr) {
        int t=dR(i), rho=i-t*R;
        multiplySlot<K>(X,t*ld+rho,R,A,B,P.mult);
      }
      __syncthreads();
      Z=fftSmem<T,-1>(X,Y,P.fp,lb,ld,tid,nthr);
    }
    // V[k] = E[k] + W_N^{-k} O[k],  E=(Zk+conj Zm)/2, O=(Zk-conj Zm)/(2i)
    for(int i=tid; i < lb*H; i += nthr) {
      int col=dH(i), k=i-col*H;
      int b=dR(col);
      long long row=row0+col-b*R;
      if(row >= P.nrows) continue;
      cplx<T> zk=Z[sp(k*ld+col)];
      int km=k == 0 ? 0 : Nh-k;
      cplx<T> zm=conjg(Z[sp(km*ld+col)]);
      cplx<T> e=(zk+zm)*half;
      cplx<T> dd=zk-zm;
      cplx<T> o=mk(dd.y*half,-dd.x*half);
      cplx<T> v=e+twmul<-1>(o,tw[k]);
      storeIO(P.out[b]+row*P.rowStride+k,v*P.scale,P.io64 & 2);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Outer forward, complex data: residue block r of the padded transform along
// a strided axis for `tile` adjacent columns.
template<typename T, bool CG>
__device__ __forceinline__ void outerFwdTile(const OuterPlan<T>& P, int ctile,
                                             int r, int z,
                                             unsigned char *smemRaw)
{
  const int tile=P.tile, m=P.m, N=P.N, c=P.cshift, L=P.L;
  cplx<T> *x=(cplx<T> *) smemRaw;
  cplx<T> *y=x+padded(m*tile);
  const int tid=threadIdx.x, nthr=blockDim.x;
  const int col0=ctile*tile;
  const int a=z % P.count;
  const long long batch=z/P.count;
  const cplx<T> *src=P.in[a]+batch*P.inBatch;
  cplx<T> *dst=P.out[a]+batch*P.outBatch;
  const typename TwT<T>::type *tw=P.twN;
  const UDiv dTile(tile);

  if(L <= m) {
    // One term per output: asynchronous copies straight to each value's
    // transform slot, then the conversion and residue twiddle in place by
    // the same thread.
    for(int i=tid; i < m*tile; i += nthr) {
      int t=dTile(i), cc=i-t*tile;
      int col=col0+cc;
      int s=posmod(t+c,m);
      long long off=(long long) s*P.inRow+col;
      if(s < L && col < P.C && off < P.Ltot) cpAsync(x+sp(i),src+off);
      else x[sp(i)]=mk((T) 0,(T) 0);
    }
    cpAsyncWait();
    if(r != 0 || (P.io64 & 1)) {
      for(int i=tid; i < m*tile; i += nthr) {
        int t=dTile(i), cc=i-t*tile;
        int col=col0+cc;
        int s=posmod(t+c,m);
        long long off=(long long) s*P.inRow+col;
        if(s < L && col < P.C && off < P.Ltot) {
          if(P.io64 & 1) convertStaged(x,sp(i));
          if(r != 0) x[sp(i)]=twmul<1>(x[sp(i)],tw[twExp(s,c,r,N)]);
        }
      }
    }
    __syncthreads();
  } else {
    // Stage the L x tile input block in y with asynchronous copies (many
    // loads in flight per thread instead of one dependent load per
    // output), then fold it into x with the residue twiddles.
    for(int i=tid; i < L*tile; i += nthr) {
      int s=dTile(i), cc=i-s*tile;
      int col=col0+cc;
      long long off=(long long) s*P.inRow+col;
      if(col < P.C && off < P.Ltot) cpAsync(y+i,src+off);
      else y[i]=mk((T) 0,(T) 0);
    }
    cpAsyncWait();
    if(std::is_same<T,ff>::value && (P.io64 & 1)) {
      // The caller's FP64 values were staged as they are: convert them.
      for(int i=tid; i < L*tile; i += nthr) {
        int s=dTile(i), cc=i-s*tile;
        int col=col0+cc;
        long long off=(long long) s*P.inRow+col;
        if(col < P.C && off < P.Ltot) convertStaged(y,i);
      }
    }
    __syncthreads();
    for(int i=tid; i < m*tile; i += nthr) {
      int t=dTile(i), cc=i-t*tile;
      cplx<T> sum=mk((T) 0,(T) 0);
      int s0=posmod(t+c,m);
      for(int s=s0; s < L; s += m) {
        cplx<T> v=y[s*tile+cc];
        if(r != 0) v=twmul<1>(v,tw[twExp(s,c,r,N)]);
        sum=accum(sum,v);
      }
      x[sp(i)]=sum;
    }
    __syncthreads();
  }

  if constexpr(inplaceFFT<T>()) {
    if(P.inplace) {
      // Transform in place (digit-reversed j; the row kernels do not
      // depend on row order and the backward undoes it).
      fftDIF<T,1>(x,P.fp,tile,tile,tid,nthr);
      for(int i=tid; i < m*tile; i += nthr) {
        int j=dTile(i), cc=i-j*tile;
        int col=col0+cc;
        if(col < P.C) dst[((long long) r*m+j)*P.outRow+col]=x[sp(i)];
      }
      __syncthreads();
      return;
    }
  }

  cplx<T> *X=fftSmem<T,1>(x,y,P.fp,tile,tile,tid,nthr);
  for(int i=tid; i < m*tile; i += nthr) {
    int j=dTile(i), cc=i-j*tile;
    int col=col0+cc;
    if(col < P.C) {
      cplx<T> v=X[sp(i)];
      long long k=(long long) r*m+j;
      if(P.twX) {
        unsigned long long e=((unsigned long long) col*(unsigned long long) k)
          % (unsigned long long) P.NX;
        v=twmul<1>(v,P.twX[e]);
      }
      dst[k*P.outRow+col]=v;
    }
  }
  __syncthreads();
}

template<typename T>
__global__ void __launch_bounds__(256)
outerFwdKernel(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  outerFwdTile<T,false>(P,blockIdx.x,blockIdx.y,blockIdx.z,smemRaw);
}

// Outer backward, complex data: all residues of a column tile, accumulated.
template<typename T, bool CG>
__device__ __forceinline__ void outerBwdTile(const OuterPlan<T>& P, int ctile,
                                             int z, unsigned char *smemRaw)
{
  const int tile=P.tile, m=P.m, N=P.N, c=P.cshift, L=P.L;
  // One residue: the outputs come straight from the transform, with no
  // accumulator in shared memory.
  const bool direct=P.q == 1;
  cplx<T> *acc=(cplx<T> *) smemRaw;
  cplx<T> *x=direct ? acc : acc+L*tile;
  cplx<T> *y=x+padded(m*tile);
  const int tid=threadIdx.x, nthr=blockDim.x;
  const int col0=ctile*tile;
  const int b=z % P.count;
  const long long batch=z/P.count;
  const cplx<T> *src=P.in[b]+batch*P.inBatch;
  cplx<T> *dst=P.out[b]+batch*P.outBatch;
  const typename TwT<T>::type *tw=P.twN;
  const UDiv dTile(tile);

  if(!direct)
    for(int i=tid; i < L*tile; i += nthr) acc[i]=mk((T) 0,(T) 0);
  for(int r=0; r < P.q; ++r) {
    if(CG) {
      // Data written by other CTAs of this launch: L2 loads.
      for(int i=tid; i < m*tile; i += nthr) {
        int j=dTile(i), cc=i-j*tile;
        int col=col0+cc;
        cplx<T> v=mk((T) 0,(T) 0);
        if(col < P.C) v=ldx<CG>(src+((long long) r*m+j)*P.inRow+col);
        x[sp(i)]=v;
      }
    } else {
      for(int i=tid; i < m*tile; i += nthr) {
        int j=dTile(i), cc=i-j*tile;
        int col=col0+cc;
        if(col < P.C) cpAsync(x+sp(i),src+((long long) r*m+j)*P.inRow+col);
        else x[sp(i)]=mk((T) 0,(T) 0);
      }
      cpAsyncWait();
    }
    __syncthreads();
    if(P.twX) {
      for(int i=tid; i < m*tile; i += nthr) {
        int j=dTile(i), cc=i-j*tile;
        unsigned long long e=((unsigned long long) (col0+cc)*
                              (unsigned long long) ((long long) r*m+j)) %
          (unsigned long long) P.NX;
        x[sp(i)]=twmul<-1>(x[sp(i)],P.twX[e]);
      }
      __syncthreads();
    }
    cplx<T> *X;
    if(inplaceFFT<T>() && P.inplace) {
      fftDIT<T,-1>(x,P.fp,tile,tile,tid,nthr);
      X=x;
    } else {
      X=fftSmem<T,-1>(x,y,P.fp,tile,tile,tid,nthr);
    }
    if(direct) {
      for(int i=tid; i < L*tile; i += nthr) {
        int s=dTile(i), cc=i-s*tile;
        int col=col0+cc;
        long long off=(long long) s*P.outRow+col;
        if(col < P.C && off < P.Ltot)
          storeIO(dst+off,X[sp(posmod(s-c,m)*tile+cc)]*P.scale,P.io64 & 2);
      }
      __syncthreads();
      return;
    }
    for(int i=tid; i < L*tile; i += nthr) {
      int s=dTile(i), cc=i-s*tile;
      int t=posmod(s-c,m);
      cplx<T> v=X[sp(t*tile+cc)];
      if(r != 0) v=twmul<-1>(v,tw[twExp(s,c,r,N)]);
      acc[i]=accum(acc[i],v);
    }
    __syncthreads();
  }
  for(int i=tid; i < L*tile; i += nthr) {
    int s=dTile(i), cc=i-s*tile;
    int col=col0+cc;
    long long off=(long long) s*P.outRow+col;
    if(col < P.C && off < P.Ltot) storeIO(dst+off,acc[i]*P.scale,P.io64 & 2);
  }
  __syncthreads();
}

template<typename T>
__global__ void __launch_bounds__(256)
outerBwdKernel(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  outerBwdTile<T,false>(P,blockIdx.x,blockIdx.z,smemRaw);
}

// ---------------------------------------------------------------------------
// Outer forward, real data (fftPadReal with explicit padding to even N):
// pack z[t] = f[2t] + i f[2t+1], sign +1 FFT of length N/2, unpack the
// N/2+1 non-negative modes F(k) = E[k] + W_N^k O[k].
template<typename T>
__global__ void __launch_bounds__(256)
outerRealFwdKernel(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  const int tile=P.tile, L=P.L, Nh=P.N/2;
  cplx<T> *x=(cplx<T> *) smemRaw;
  cplx<T> *y=x+padded(Nh*tile);
  const int tid=threadIdx.x, nthr=blockDim.x;
  const int col0=blockIdx.x*tile;
  const int a=blockIdx.z % P.count;
  const long long batch=blockIdx.z/P.count;
  const T *src=(const T *) P.in[a]+batch*P.inBatch;
  cplx<T> *dst=P.out[a]+batch*P.outBatch;
  const typename TwT<T>::type *tw=P.twN;
  const T half=(T) 0.5;
  const UDiv dTile(tile);

  for(int i=tid; i < Nh*tile; i += nthr) {
    int t=dTile(i), cc=i-t*tile;
    int col=col0+cc;
    T re=(T) 0, im=(T) 0;
    if(col < P.C) {
      int s=2*t;
      if(s < L) re=loadIOr(src+(long long) s*P.inRow+col,P.io64 & 1);
      if(s+1 < L) im=loadIOr(src+(long long) (s+1)*P.inRow+col,P.io64 & 1);
    }
    x[sp(i)]=mk(re,im);
  }
  __syncthreads();
  cplx<T> *X=fftSmem<T,1>(x,y,P.fp,tile,tile,tid,nthr);
  for(int i=tid; i < (Nh+1)*tile; i += nthr) {
    int k=dTile(i), cc=i-k*tile;
    int col=col0+cc;
    if(col >= P.C) continue;
    int k0=k == Nh ? 0 : k;
    int km=k == 0 || k == Nh ? 0 : Nh-k;
    cplx<T> zk=X[sp(k0*tile+cc)];
    cplx<T> zm=conjg(X[sp(km*tile+cc)]);
    cplx<T> e=(zk+zm)*half;
    cplx<T> dd=zk-zm;
    cplx<T> o=mk(dd.y*half,-dd.x*half);
    cplx<T> v;
    if(k == Nh) v=e-o;
    else v=e+twmul<1>(o,tw[k]);
    dst[(long long) k*P.outRow+col]=P.conj ? conjg(v) : v;
  }
}

// Outer backward, real data: Hermitian-extend the N/2+1 modes, pack
// Y[k] = (G[k] + conj G[Nh-k]) + i W_N^{-k} (G[k] - conj G[Nh-k]), sign -1
// FFT of length N/2, unpack h[2t] = Re y[t], h[2t+1] = Im y[t].
template<typename T>
__global__ void __launch_bounds__(256)
outerRealBwdKernel(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  const int tile=P.tile, L=P.L, Nh=P.N/2;
  cplx<T> *x=(cplx<T> *) smemRaw;
  cplx<T> *y=x+padded(Nh*tile);
  const int tid=threadIdx.x, nthr=blockDim.x;
  const int col0=blockIdx.x*tile;
  const int b=blockIdx.z % P.count;
  const long long batch=blockIdx.z/P.count;
  const cplx<T> *src=P.in[b]+batch*P.inBatch;
  T *dst=(T *) P.out[b]+batch*P.outBatch;
  const typename TwT<T>::type *tw=P.twN;
  const UDiv dTile(tile);

  for(int i=tid; i < Nh*tile; i += nthr) {
    int k=dTile(i), cc=i-k*tile;
    int col=col0+cc;
    cplx<T> v=mk((T) 0,(T) 0);
    if(col < P.C) {
      cplx<T> gk=src[(long long) k*P.inRow+col];
      cplx<T> gm=src[(long long) (Nh-k)*P.inRow+col];
      if(P.conj) {
        gk=conjg(gk);
        gm=conjg(gm);
      }
      if(k == 0) gk.y=(T) 0;
      if(k == 0) gm.y=(T) 0;
      gm=conjg(gm);
      cplx<T> s=gk+gm;
      cplx<T> d=twmul<-1>(gk-gm,tw[k]);
      v=mk(s.x-d.y,s.y+d.x);
    }
    x[sp(i)]=v;
  }
  __syncthreads();
  cplx<T> *X=fftSmem<T,-1>(x,y,P.fp,tile,tile,tid,nthr);
  for(int i=tid; i < Nh*tile; i += nthr) {
    int t=dTile(i), cc=i-t*tile;
    int col=col0+cc;
    if(col >= P.C) continue;
    cplx<T> v=X[sp(i)]*P.scale;
    int s=2*t;
    if(s < L) storeIOr(dst+(long long) s*P.outRow+col,v.x,P.io64 & 2);
    if(s+1 < L) storeIOr(dst+(long long) (s+1)*P.outRow+col,v.y,P.io64 & 2);
  }
}

// ---------------------------------------------------------------------------
// Persistent batched kernel (see kernels.cuh).

template<typename T, template<typename> class Plan>
__device__ __forceinline__ void rebase(Plan<T>& plan, int count, bool relIn,
                                       bool relOut, void *const *inBase,
                                       void *const *outBase)
{
  for(int a=0; a < count; ++a) {
    if(relIn)
      plan.in[a]=(const cplx<T> *) ((char *) inBase[a]+(size_t) plan.in[a]);
    if(relOut)
      plan.out[a]=(cplx<T> *) ((char *) outBase[a]+(size_t) plan.out[a]);
  }
}

// Copy a task's plan from the problem table into shared memory (one copy per
// CTA, read by every thread through broadcast loads) and rebase its pointers
// there: a per-thread copy would live in local memory.
template<typename Plan>
__device__ __forceinline__ Plan& stagePlan(unsigned char *buf, const Plan& src)
{
  static_assert(sizeof(Plan) % sizeof(int) == 0, "plan size");
  int *d=(int *) buf;
  const int *s=(const int *) &src;
  for(int i=threadIdx.x; i < (int) (sizeof(Plan)/sizeof(int)); i += blockDim.x)
    d[i]=s[i];
  return *(Plan *) buf;
}

template<typename T, int K>
__global__ void __launch_bounds__(256)
batchKernel(const BatchArgs<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  constexpr size_t planBytes=sizeof(RowPlan<T>) > sizeof(OuterPlan<T>) ?
    sizeof(RowPlan<T>) : sizeof(OuterPlan<T>);
  __shared__ __align__(16) unsigned char planBuf[planBytes];
  __shared__ int slot;
  __shared__ int gaveUp;
  for(;;) {
    if(threadIdx.x == 0) slot=atomicAdd(P.queue,1);
    __syncthreads();
    const int t=slot;
    __syncthreads();
    if(t >= P.ntasks) return;
    const BatchTask tk=P.tasks[t];
    const BatchProblem<T> *B=P.probs+tk.prob;
    if(tk.type == TASK_ROW || tk.type == TASK_COLBWD) {
      if(threadIdx.x == 0) {
        volatile int *d=P.done+2*tk.prob+(tk.type == TASK_ROW ? 0 : 1);
        const int target=tk.type == TASK_ROW ? B->nfwd : B->nrows;
        long long it=0;
        gaveUp=0;
        while(*d < target) {
          if(++it > P.spinLimit) {
            gaveUp=1;
            atomicExch(P.err,1);
            break;
          }
          __nanosleep(100);
        }
        __threadfence();
      }
      __syncthreads();
      if(gaveUp) continue;
    }
    const int rel=B->rel;
    if(tk.type == TASK_SMALL || tk.type == TASK_ROW) {
      RowPlan<T>& R=stagePlan(planBuf,B->row);
      __syncthreads();
      if(threadIdx.x == 0 && tk.type == TASK_SMALL)
        rebase(R,R.A,rel & 1,rel & 2,P.inBase,P.outBase);
      __syncthreads();
      if(tk.type == TASK_SMALL) rowConvRow<T,false,K>(R,tk.i,smemRaw);
      else if(R.direct) rowConvRow<T,true,K,true>(R,tk.i,smemRaw);
      else rowConvRow<T,true,K>(R,tk.i,smemRaw);
    } else {
      const bool fwd=tk.type == TASK_COLFWD;
      OuterPlan<T>& O=stagePlan(planBuf,fwd ? B->fwd : B->bwd);
      __syncthreads();
      if(threadIdx.x == 0)
        rebase(O,O.count,fwd && (rel & 4),!fwd && (rel & 8),P.inBase,
               P.outBase);
      __syncthreads();
      if(fwd) outerFwdTile<T,false>(O,tk.i,0,tk.j,smemRaw);
      else outerBwdTile<T,true>(O,tk.i,tk.j,smemRaw);
    }
    if(tk.type == TASK_COLFWD || tk.type == TASK_ROW) {
      __threadfence();
      __syncthreads();
      if(threadIdx.x == 0)
        atomicAdd(P.done+2*tk.prob+(tk.type == TASK_COLFWD ? 0 : 1),1);
    }
  }
}

template<typename T, int K>
static cudaError_t launchBatchK(const BatchArgs<T>& P, int grid, int threads,
                                size_t smem, cudaStream_t s)
{
  if(smem > 48*1024) {
    cudaError_t e=cudaFuncSetAttribute(batchKernel<T,K>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int) smem);
    if(e != cudaSuccess) return e;
  }
  batchKernel<T,K><<<grid,threads,smem,s>>>(P);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launchBatch(const BatchArgs<T>& P, int grid, int threads,
                        size_t smem, cudaStream_t s)
{
  switch(multVariant(P.mult,P.A,P.B)) {
    case MULT_BINARY: return launchBatchK<T,MULT_BINARY>(P,grid,threads,smem,s);
    case MULT_REALBINARY:
      return launchBatchK<T,MULT_REALBINARY>(P,grid,threads,smem,s);
    default: return launchBatchK<T,MULT_GENERIC>(P,grid,threads,smem,s);
  }
}

template<typename T, int K>
static int batchBlocksK(int threads, size_t smem)
{
  if(smem > 48*1024)
    cudaFuncSetAttribute(batchKernel<T,K>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,(int) smem);
  int n=0;
  if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n,batchKernel<T,K>,threads,
                                                   smem) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

template<typename T>
int batchBlocksPerSM(int threads, size_t smem, int mult, int A, int B)
{
  switch(multVariant(mult,A,B)) {
    case MULT_BINARY: return batchBlocksK<T,MULT_BINARY>(threads,smem);
    case MULT_REALBINARY: return batchBlocksK<T,MULT_REALBINARY>(threads,smem);
    default: return batchBlocksK<T,MULT_GENERIC>(threads,smem);
  }
}

// ---------------------------------------------------------------------------
// Launchers.

// Shared-memory bytes: FFT ping-pong buffers are padded (sp()); the forward
// outer kernel also stages its L x tile input block in the second buffer.
template<typename T> size_t rowSmem(int L, int m, int A, int B, int rpc,
                                    int direct)
{
  size_t nbuf=inplaceFFT<T>() || direct ? 1 : 2;
  size_t stage=direct ? 0 : (size_t) (A+B)*rpc*L;
  return sizeof(cplx<T>)*(stage+nbuf*(size_t) padded(m*A*rpc));
}
template<typename T> size_t hermRowSmem(int H, int Nh, int A, int rpc)
{
  size_t nbuf=inplaceFFT<T>() ? 1 : 2;
  return sizeof(cplx<T>)*nbuf*(size_t) padded(Nh*A*rpc);
}
template<typename T> size_t outerFwdSmem(int L, int m, int tile, int inplace)
{
  size_t pm=padded(m*tile);
  if(inplaceFFT<T>() && inplace) return sizeof(cplx<T>)*pm;
  return sizeof(cplx<T>)*(pm+std::max(pm,(size_t) L*tile));
}
template<typename T> size_t outerBwdSmem(int L, int m, int tile, int q,
                                         int inplace)
{
  size_t acc=q == 1 ? 0 : (size_t) L*tile;
  size_t nbuf=inplaceFFT<T>() && inplace ? 1 : 2;
  return sizeof(cplx<T>)*(acc+nbuf*(size_t) padded(m*tile));
}
template<typename T> size_t outerRealSmem(int L, int Nh, int tile)
{
  return sizeof(cplx<T>)*2*(size_t) padded((Nh+1)*tile);
}

template<typename K>
static cudaError_t setSmem(K kernel, size_t bytes)
{
  if(bytes > 48*1024)
    return cudaFuncSetAttribute(kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int) bytes);
  return cudaSuccess;
}

template<typename T>
cudaError_t launchRow(const RowPlan<T>& P, int threads, long long grid,
                      cudaStream_t s)
{
  size_t sm=rowSmem<T>(P.L,P.m,P.A,P.B,P.rpc,P.direct);
  long long groups=(P.nrows+P.rpc-1)/P.rpc;
  grid=std::min(std::min(grid,groups),(long long) INT_MAX);
  auto go=[&](auto kernel) {
    cudaError_t e=setSmem(kernel,sm);
    if(e != cudaSuccess) return e;
    kernel<<<(unsigned) grid,threads,sm,s>>>(P);
    return cudaGetLastError();
  };
  if(P.direct)
    switch(multVariant(P.mult,P.A,P.B)) {
      case MULT_BINARY: return go(rowConvKernel<T,MULT_BINARY,true>);
      case MULT_REALBINARY: return go(rowConvKernel<T,MULT_REALBINARY,true>);
      default: return go(rowConvKernel<T,MULT_GENERIC,true>);
    }
  switch(multVariant(P.mult,P.A,P.B)) {
    case MULT_BINARY: return go(rowConvKernel<T,MULT_BINARY,false>);
    case MULT_REALBINARY: return go(rowConvKernel<T,MULT_REALBINARY,false>);
    default: return go(rowConvKernel<T,MULT_GENERIC,false>);
  }
}

template<typename T>
cudaError_t launchHermRow(const HermRowPlan<T>& P, int threads,
                          long long grid, cudaStream_t s)
{
  size_t sm=hermRowSmem<T>(P.H,P.Nh,P.A,P.rpc);
  long long groups=(P.nrows+P.rpc-1)/P.rpc;
  grid=std::min(std::min(grid,groups),(long long) INT_MAX);
  auto go=[&](auto kernel) {
    cudaError_t e=setSmem(kernel,sm);
    if(e != cudaSuccess) return e;
    kernel<<<(unsigned) grid,threads,sm,s>>>(P);
    return cudaGetLastError();
  };
  switch(multVariant(P.mult,P.A,P.B)) {
    case MULT_REALBINARY: return go(hermRowKernel<T,MULT_REALBINARY>);
    case MULT_REALJACOBIAN: return go(hermRowKernel<T,MULT_REALJACOBIAN>);
    case MULT_REALJACADJ: return go(hermRowKernel<T,MULT_REALJACADJ>);
    default: return go(hermRowKernel<T,MULT_GENERIC>);
  }
}

template<typename T>
cudaError_t launchOuterFwd(const OuterPlan<T>& P, int threads, cudaStream_t s)
{
  size_t sm=outerFwdSmem<T>(P.L,P.m,P.tile,P.inplace);
  cudaError_t e=setSmem(outerFwdKernel<T>,sm);
  if(e != cudaSuccess) return e;
  dim3 grid((P.C+P.tile-1)/P.tile,P.q,P.nbatch*P.count);
  outerFwdKernel<T><<<grid,threads,sm,s>>>(P);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launchOuterBwd(const OuterPlan<T>& P, int threads, cudaStream_t s)
{
  size_t sm=outerBwdSmem<T>(P.L,P.m,P.tile,P.q,P.inplace);
  cudaError_t e=setSmem(outerBwdKernel<T>,sm);
  if(e != cudaSuccess) return e;
  dim3 grid((P.C+P.tile-1)/P.tile,1,P.nbatch*P.count);
  outerBwdKernel<T><<<grid,threads,sm,s>>>(P);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launchOuterRealFwd(const OuterPlan<T>& P, int threads,
                               cudaStream_t s)
{
  size_t sm=outerRealSmem<T>(P.L,P.N/2,P.tile);
  cudaError_t e=setSmem(outerRealFwdKernel<T>,sm);
  if(e != cudaSuccess) return e;
  dim3 grid((P.C+P.tile-1)/P.tile,1,P.nbatch*P.count);
  outerRealFwdKernel<T><<<grid,threads,sm,s>>>(P);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launchOuterRealBwd(const OuterPlan<T>& P, int threads,
                               cudaStream_t s)
{
  size_t sm=outerRealSmem<T>(P.L,P.N/2,P.tile);
  cudaError_t e=setSmem(outerRealBwdKernel<T>,sm);
  if(e != cudaSuccess) return e;
  dim3 grid((P.C+P.tile-1)/P.tile,1,P.nbatch*P.count);
  outerRealBwdKernel<T><<<grid,threads,sm,s>>>(P);
  return cudaGetLastError();
}

#define FGB_INSTANTIATE(T) \
  template cudaError_t launchRow<T>(const RowPlan<T>&,int,long long,cudaStream_t); \
  template cudaError_t launchHermRow<T>(const HermRowPlan<T>&,int,long long,cudaStream_t); \
  template cudaError_t launchOuterFwd<T>(const OuterPlan<T>&,int,cudaStream_t); \
  template cudaError_t launchOuterBwd<T>(const OuterPlan<T>&,int,cudaStream_t); \
  template cudaError_t launchOuterRealFwd<T>(const OuterPlan<T>&,int,cudaStream_t); \
  template cudaError_t launchOuterRealBwd<T>(const OuterPlan<T>&,int,cudaStream_t); \
  template size_t rowSmem<T>(int,int,int,int,int,int); \
  template size_t hermRowSmem<T>(int,int,int,int); \
  template size_t outerFwdSmem<T>(int,int,int,int); \
  template size_t outerBwdSmem<T>(int,int,int,int,int); \
  template size_t outerRealSmem<T>(int,int,int); \
  template cudaError_t launchBatch<T>(const BatchArgs<T>&,int,int,size_t,cudaStream_t); \
  template int batchBlocksPerSM<T>(int,size_t,int,int,int);

#if !defined(FGB_ONLY_FLOAT) && !defined(FGB_ONLY_FF)
// Bulk copy by the SMs (16-byte vectors, four in flight per thread): between
// page-locked host memory and the device it reads and writes whole lines
// over the host link.
__global__ void __launch_bounds__(256) bulkCopyKernel(CopyArgs P)
{
  const size_t n=P.bytes/16;
  const size_t stride=(size_t) gridDim.x*blockDim.x;
  for(int a=0; a < P.count; ++a) {
    const uint4 *src=(const uint4 *) P.src[a];
    uint4 *dst=(uint4 *) P.dst[a];
    size_t i=blockIdx.x*(size_t) blockDim.x+threadIdx.x;
    for(; i+3*stride < n; i += 4*stride) {
      uint4 v0=src[i], v1=src[i+stride], v2=src[i+2*stride],
        v3=src[i+3*stride];
      dst[i]=v0; dst[i+stride]=v1; dst[i+2*stride]=v2; dst[i+3*stride]=v3;
    }
    for(; i < n; i += stride) dst[i]=src[i];
  }
}

cudaError_t launchBulkCopy(const CopyArgs& P, cudaStream_t s)
{
  if(P.bytes % 16) return cudaErrorInvalidValue;
  for(int a=0; a < P.count; ++a)
    if(((size_t) P.src[a] | (size_t) P.dst[a]) % 16)
      return cudaErrorInvalidValue;
  if(P.bytes == 0 || P.count == 0) return cudaSuccess;
  bulkCopyKernel<<<152*8,256,0,s>>>(P);
  return cudaGetLastError();
}
#endif

// Each precision may be compiled as its own translation unit (build.py
// compiles this file once per precision, in parallel): FGB_ONLY_<P> keeps
// one of DOUBLE, FLOAT and FF.
#if !defined(FGB_ONLY_FLOAT) && !defined(FGB_ONLY_FF)
FGB_INSTANTIATE(double)
#endif
#if !defined(FGB_ONLY_DOUBLE) && !defined(FGB_ONLY_FF)
FGB_INSTANTIATE(float)
#endif
#if !defined(FGB_ONLY_DOUBLE) && !defined(FGB_ONLY_FLOAT)
FGB_INSTANTIATE(ff)

#endif

} // namespace fgb
