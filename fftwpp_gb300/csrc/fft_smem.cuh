// fft_smem.cuh -- shared-memory staged Stockham FFT with register radix
// codelets (radix 2, 3, 4, 5, 7, 8), for the GB300 engine.
//
// A transform of length n = prod(radix[s]) runs on `ncol` interleaved
// columns held in shared memory: element i of column c lives at x[i*ld+c].
// Stage s (radix R, Ns = product of earlier radices) maps, for every
// butterfly j < n/R and column c,
//     a_r = x[j + r n/R] * W_{Ns R}^{S r (j mod Ns)}            (r < R)
//     y[(j - j mod Ns) R + (j mod Ns) + r Ns] = DFT_R^S(a)_r
// which is the self-sorting Stockham formulation: the output of the last
// stage is in natural order, and every stage reads and writes with unit
// column stride so neighbouring threads touch neighbouring words.
// Twiddles W_n^t = exp(2 pi i t/n), t < n, come from one precomputed table
// of the transform length (generated on the host in long double); the
// stage twiddle W_{Ns R}^{rk} is table entry r*k*n/(Ns R).
//
// DFT sign convention: S = +1 computes sum_j x_j exp(+2 pi i jk/n), the sign
// FFTW++ uses for its forward padded transforms; S = -1 the inverse (both
// unnormalised).
#pragma once

#include "complex.cuh"

#include <type_traits>

namespace fgb {

#define FGB_MAXSTAGES 20

// Shared-memory element index with one pad element every 32: the first
// Stockham stages write with power-of-two strides, which without padding
// put a whole warp on one bank.
__host__ __device__ __forceinline__ int sp(int a) {return a+(a >> 5);}
// Elements to allocate for n logical elements.
__host__ __device__ __forceinline__ int padded(int n) {return n+(n >> 5)+1;}

// floor(a/b) for 0 <= a < 2^21 through a float reciprocal (exact in that
// range: the rounded product is within 2^-22 relative of a/b while the
// nearest integer boundary is at least 1/(2b) away from (a+0.5)/b).
__device__ __forceinline__ int fdiv(int a, float invb)
{
  return __float2int_rz(((float) a+0.5f)*invb);
}

// Division by a block-uniform divisor d >= 1: a shift when d is a power of
// two (the common case), else fdiv's float reciprocal.
struct UDiv {
  float inv;
  int sh;
  bool p2;
  __device__ __forceinline__ explicit UDiv(int d)
    : inv(1.0f/(float) d), sh(0), p2((d & (d-1)) == 0)
  {
#ifdef __CUDA_ARCH__
    sh=__ffs(d)-1;
#endif
  }
  __device__ __forceinline__ int operator()(int a) const
  {
    return p2 ? a >> sh : fdiv(a,inv);
  }
};

struct FFTPlanDev {
  int n;
  int nst;
  int radix[FGB_MAXSTAGES];
  const void *tw;         // TwT<T>::type[n]
};

// Whether a plan holds a radix-16 or radix-6 stage (its kernels need the
// R16 form).
inline bool hasWideRadix(const FFTPlanDev& p)
{
  for(int s=0; s < p.nst; ++s)
    if(p.radix[s] == 16 || p.radix[s] == 6) return true;
  return false;
}

// Radix constants (exact decimal expansions of the algebraic values).
#define FGB_SQRT1_2 0.707106781186547524400844362105
#define FGB_SQRT3_2 0.866025403784438646763723170753
#define FGB_C51 0.309016994374947424102293417183
#define FGB_S51 0.951056516295153572116439333379
#define FGB_C52 -0.809016994374947424102293417183
#define FGB_S52 0.587785252292473129168705954639
#define FGB_C71 0.623489801858733530525004884004
#define FGB_S71 0.781831482468029808708444526674
#define FGB_C72 -0.222520933956314404288902564497
#define FGB_S72 0.974927912181823607018131682994
#define FGB_C73 -0.900968867902419126236102319507
#define FGB_S73 0.433883739117558120475768332849

template<int R, int S, typename T> struct Codelet;

template<int S, typename T> struct Codelet<2,S,T> {
  static __device__ __forceinline__ void run(cplx<T> *a) {
    cplx<T> t=a[0];
    a[0]=t+a[1];
    a[1]=t-a[1];
  }
};

template<int S, typename T> struct Codelet<4,S,T> {
  static __device__ __forceinline__ void run(cplx<T> *a) {
    cplx<T> s02=a[0]+a[2], d02=a[0]-a[2];
    cplx<T> s13=a[1]+a[3], d13=mulI<S>(a[1]-a[3]);
    a[0]=s02+s13;
    a[2]=s02-s13;
    a[1]=d02+d13;
    a[3]=d02-d13;
  }
};

template<int S, typename T> struct Codelet<8,S,T> {
  static __device__ __forceinline__ void run(cplx<T> *a) {
    const T h=(T) FGB_SQRT1_2;
    cplx<T> e[4]={a[0],a[2],a[4],a[6]};
    cplx<T> o[4]={a[1],a[3],a[5],a[7]};
    Codelet<4,S,T>::run(e);
    Codelet<4,S,T>::run(o);
    // o[k] *= W_8^{S k}
    cplx<T> o1=o[1], o3=o[3];
    if(S > 0) {
      o[1]=mk((o1.x-o1.y)*h,(o1.y+o1.x)*h);                     // (1+i)/sqrt2
      o[3]=mk((-o3.x-o3.y)*h,(o3.x-o3.y)*h);                    // (-1+i)/sqrt2
    } else {
      o[1]=mk((o1.x+o1.y)*h,(o1.y-o1.x)*h);                     // (1-i)/sqrt2
      o[3]=mk((o3.y-o3.x)*h,(-o3.y-o3.x)*h);                    // (-1-i)/sqrt2
    }
    o[2]=mulI<S>(o[2]);
#pragma unroll
    for(int k=0; k < 4; ++k) {
      a[k]=e[k]+o[k];
      a[k+4]=e[k]-o[k];
    }
  }
};

// Radix 16 as 4 x 4 (FP32 in-place transforms of row kernels compiled
// with it): radix-4 over the inputs k + 4r, the products with W_16^{ks},
// radix-4 over k; outputs in natural order.
#define FGB_C161 0.923879532511286756128183189397
#define FGB_S161 0.382683432365089771728459984030
template<int S, typename T> struct Codelet<16,S,T> {
  static __device__ __forceinline__ cplx<T> rot(cplx<T> a, T c, T s) {
    // a (c + i S s)
    const T ss=(T) S*s;
    return mk(fma(a.x,c,-a.y*ss),fma(a.x,ss,a.y*c));
  }
  static __device__ __forceinline__ void run(cplx<T> *a) {
    const T h=(T) FGB_SQRT1_2, c1=(T) FGB_C161, s1=(T) FGB_S161;
    cplx<T> b[4][4];
#pragma unroll
    for(int k=0; k < 4; ++k) {
      cplx<T> t[4]={a[k],a[k+4],a[k+8],a[k+12]};
      Codelet<4,S,T>::run(t);
#pragma unroll
      for(int s=0; s < 4; ++s) b[s][k]=t[s];
    }
    // W_16^{ks}: (k,s) = (1,1) W, (1,2) W^2, (1,3) W^3, (2,1) W^2,
    // (2,2) W^4 = S i, (2,3) W^6, (3,1) W^3, (3,2) W^6, (3,3) W^9.
    b[1][1]=rot(b[1][1],c1,s1);
    b[2][1]=rot(b[2][1],h,h);
    b[3][1]=rot(b[3][1],s1,c1);
    b[1][2]=rot(b[1][2],h,h);
    b[2][2]=mulI<S>(b[2][2]);
    b[3][2]=rot(b[3][2],-h,h);
    b[1][3]=rot(b[1][3],s1,c1);
    b[2][3]=rot(b[2][3],-h,h);
    b[3][3]=rot(b[3][3],-c1,-s1);
#pragma unroll
    for(int s=0; s < 4; ++s) {
      Codelet<4,S,T>::run(b[s]);
#pragma unroll
      for(int t=0; t < 4; ++t) a[s+4*t]=b[s][t];
    }
  }
};

// Radix 6 as 3 x 2 (with radix 16, for FP32 in-place transforms of
// lengths 3 * 2^k where it saves a stage): radix-3 over the inputs k + 2r,
// the products with W_6^{ks}, radix-2 over k; outputs in natural order.
template<int S, typename T> struct Codelet<6,S,T> {
  static __device__ __forceinline__ void run(cplx<T> *a) {
    const T h=(T) 0.5, s3=(T) (S*FGB_SQRT3_2);
    cplx<T> e[3]={a[0],a[2],a[4]}, o[3]={a[1],a[3],a[5]};
    Codelet<3,S,T>::run(e);
    Codelet<3,S,T>::run(o);
    // W_6^S = (1/2, S sqrt3/2), W_6^{2S} = (-1/2, S sqrt3/2)
    const cplx<T> o1=o[1], o2=o[2];
    o[1]=mk(fma(o1.x,h,-o1.y*s3),fma(o1.x,s3,o1.y*h));
    o[2]=mk(fma(o2.x,-h,-o2.y*s3),fma(o2.x,s3,-o2.y*h));
#pragma unroll
    for(int s=0; s < 3; ++s) {
      a[s]=e[s]+o[s];
      a[s+3]=e[s]-o[s];
    }
  }
};

// FP64 radix 8 and 3 without twiddles: the constant rotations fused into
// the combining additions (see the fused butterflies below).
template<int S> struct Codelet<8,S,double>;
template<int S> struct Codelet<3,S,double>;

template<int S, typename T> struct Codelet<3,S,T> {
  static __device__ __forceinline__ void run(cplx<T> *a) {
    const T c=(T) -0.5;
    const T s=(T) (S*FGB_SQRT3_2);
    cplx<T> t=a[1]+a[2];
    cplx<T> d=a[1]-a[2];
    cplx<T> b=mk(fma(c,t.x,a[0].x),fma(c,t.y,a[0].y));
    cplx<T> r=mk(-s*d.y,s*d.x);                                 // i*s*d
    a[0]=a[0]+t;
    a[1]=b+r;
    a[2]=b-r;
  }
};

template<int S, typename T> struct Codelet<5,S,T> {
  static __device__ __forceinline__ void run(cplx<T> *a) {
    const T c1=(T) FGB_C51, c2=(T) FGB_C52;
    const T s1=(T) (S*FGB_S51), s2=(T) (S*FGB_S52);
    cplx<T> t1=a[1]+a[4], d1=a[1]-a[4];
    cplx<T> t2=a[2]+a[3], d2=a[2]-a[3];
    cplx<T> x0=a[0];
    cplx<T> b1=mk(fma(c1,t1.x,fma(c2,t2.x,x0.x)),fma(c1,t1.y,fma(c2,t2.y,x0.y)));
    cplx<T> b2=mk(fma(c2,t1.x,fma(c1,t2.x,x0.x)),fma(c2,t1.y,fma(c1,t2.y,x0.y)));
    // i*(s1 d1 + s2 d2) and i*(s2 d1 - s1 d2)
    cplx<T> e1=mk(fma(s1,d1.x,s2*d2.x),fma(s1,d1.y,s2*d2.y));
    cplx<T> e2=mk(fma(s2,d1.x,-s1*d2.x),fma(s2,d1.y,-s1*d2.y));
    cplx<T> i1=mk(-e1.y,e1.x), i2=mk(-e2.y,e2.x);
    a[0]=x0+t1+t2;
    a[1]=b1+i1;
    a[4]=b1-i1;
    a[2]=b2+i2;
    a[3]=b2-i2;
  }
};

template<int S, typename T> struct Codelet<7,S,T> {
  static __device__ __forceinline__ void run(cplx<T> *a) {
    const T C1=(T) FGB_C71, C2=(T) FGB_C72, C3=(T) FGB_C73;
    const T S1=(T) (S*FGB_S71), S2=(T) (S*FGB_S72), S3=(T) (S*FGB_S73);
    cplx<T> t1=a[1]+a[6], d1=a[1]-a[6];
    cplx<T> t2=a[2]+a[5], d2=a[2]-a[5];
    cplx<T> t3=a[3]+a[4], d3=a[3]-a[4];
    cplx<T> x0=a[0];
    // cos(2 pi jk/7), sin(2 pi jk/7) for j=1,2,3 and k=1,2,3:
    // j=1: (C1,C2,C3), (S1,S2,S3); j=2: (C2,C3,C1), (S2,-S3,-S1);
    // j=3: (C3,C1,C2), (S3,-S1,S2).
    cplx<T> b1=mk(x0.x+C1*t1.x+C2*t2.x+C3*t3.x,x0.y+C1*t1.y+C2*t2.y+C3*t3.y);
    cplx<T> b2=mk(x0.x+C2*t1.x+C3*t2.x+C1*t3.x,x0.y+C2*t1.y+C3*t2.y+C1*t3.y);
    cplx<T> b3=mk(x0.x+C3*t1.x+C1*t2.x+C2*t3.x,x0.y+C3*t1.y+C1*t2.y+C2*t3.y);
    cplx<T> e1=mk(S1*d1.x+S2*d2.x+S3*d3.x,S1*d1.y+S2*d2.y+S3*d3.y);
    cplx<T> e2=mk(S2*d1.x-S3*d2.x-S1*d3.x,S2*d1.y-S3*d2.y-S1*d3.y);
    cplx<T> e3=mk(S3*d1.x-S1*d2.x+S2*d3.x,S3*d1.y-S1*d2.y+S2*d3.y);
    a[0]=x0+t1+t2+t3;
    cplx<T> i1=mk(-e1.y,e1.x), i2=mk(-e2.y,e2.x), i3=mk(-e3.y,e3.x);
    a[1]=b1+i1; a[6]=b1-i1;
    a[2]=b2+i2; a[5]=b2-i2;
    a[3]=b3+i3; a[4]=b3-i3;
  }
};

// ---------------------------------------------------------------------------
// FP64 butterflies with the twiddles of their inputs fused in (the FP64
// kernels are bound by GB300's FP64 pipe, so every DADD/DMUL/DFMA saved is
// time saved).  Two rules do it: a + w b is four DFMAs (fmaTw) instead of a
// multiply and an add, and the difference a - w b of a pair is taken from
// its sum s as 2a - s (one DFMA per component).  Radix 2, 3, 4 and 8 take
// 6, 18, 24 and 72 FP64 instructions with their twiddles, against 8, 22,
// 28 and 84 for a twiddle multiply per input followed by the plain
// butterfly; radix 8 and 3 without twiddles take 52 and 12 (56 and 14):
// the rotations by W_8 and the sqrt(3)/2 terms go into the combining
// additions as DFMAs.

// acc + a w^S (w a stored twiddle exp(+i theta)): four DFMAs.
template<int S>
__device__ __forceinline__ cplx<double> fmaTw(cplx<double> acc, cplx<double> a,
                                              double2 w)
{
  const double wy=S > 0 ? w.y : -w.y;
  return mk(fma(a.x,w.x,fma(-a.y,wy,acc.x)),fma(a.y,w.x,fma(a.x,wy,acc.y)));
}

// 2a - s: the difference a - b of a pair from its sum s = a + b.
__device__ __forceinline__ cplx<double> twoMinus(cplx<double> a,
                                                 cplx<double> s)
{
  return mk(fma(2.0,a.x,-s.x),fma(2.0,a.y,-s.y));
}

// Radix 4 on (a0, a1 w1, a2 w2, a3 w3), a0 untwiddled.
template<int S>
__device__ __forceinline__ void tw4(cplx<double> *o, cplx<double> a0,
                                    cplx<double> a1, double2 w1,
                                    cplx<double> a2, double2 w2,
                                    cplx<double> a3, double2 w3)
{
  const cplx<double> s02=fmaTw<S>(a0,a2,w2);
  const cplx<double> d02=twoMinus(a0,s02);
  const cplx<double> b1=twmul<S>(a1,w1);
  const cplx<double> s13=fmaTw<S>(b1,a3,w3);
  const cplx<double> d13=mulI<S>(twoMinus(b1,s13));
  o[0]=s02+s13;
  o[2]=s02-s13;
  o[1]=d02+d13;
  o[3]=d02-d13;
}

// The last layer of radix 8 from the radix-4 transforms e (even inputs)
// and o (odd inputs): a[k] = e[k] + W_8^{S k} o[k], a[k+4] = e[k] - ...
template<int S>
__device__ __forceinline__ void combine8(cplx<double> *a, const cplx<double> *e,
                                         const cplx<double> *o)
{
  const double h=FGB_SQRT1_2;
  a[0]=e[0]+o[0];
  a[4]=e[0]-o[0];
  const cplx<double> o2=mulI<S>(o[2]);
  a[2]=e[2]+o2;
  a[6]=e[2]-o2;
  // W_8^{S} o1 = h (p + i q); W_8^{3S} o3 = h (-u + i v) (S > 0) or
  // h (u' - i v') (S < 0).
  const double p=S > 0 ? o[1].x-o[1].y : o[1].x+o[1].y;
  const double q=S > 0 ? o[1].y+o[1].x : o[1].y-o[1].x;
  a[1]=mk(fma(h,p,e[1].x),fma(h,q,e[1].y));
  a[5]=mk(fma(-h,p,e[1].x),fma(-h,q,e[1].y));
  if(S > 0) {
    const double u=o[3].x+o[3].y, v=o[3].x-o[3].y;
    a[3]=mk(fma(-h,u,e[3].x),fma(h,v,e[3].y));
    a[7]=mk(fma(h,u,e[3].x),fma(-h,v,e[3].y));
  } else {
    const double u=o[3].y-o[3].x, v=o[3].x+o[3].y;
    a[3]=mk(fma(h,u,e[3].x),fma(-h,v,e[3].y));
    a[7]=mk(fma(-h,u,e[3].x),fma(h,v,e[3].y));
  }
}

template<int S>
__device__ __forceinline__ void radix3(cplx<double> *a, cplx<double> t,
                                       cplx<double> d)
{
  const double s=S*FGB_SQRT3_2;
  const cplx<double> b=mk(fma(-0.5,t.x,a[0].x),fma(-0.5,t.y,a[0].y));
  a[0]=a[0]+t;
  a[1]=mk(fma(-s,d.y,b.x),fma(s,d.x,b.y));
  a[2]=mk(fma(s,d.y,b.x),fma(-s,d.x,b.y));
}

template<int R, int S> struct TwButterfly;   // a[r] *= w[r] (r >= 1), DFT

template<int S> struct TwButterfly<2,S> {
  static __device__ __forceinline__ void run(cplx<double> *a, const double2 *w) {
    const cplx<double> b=fmaTw<S>(a[0],a[1],w[1]);
    a[1]=twoMinus(a[0],b);
    a[0]=b;
  }
};

template<int S> struct TwButterfly<4,S> {
  static __device__ __forceinline__ void run(cplx<double> *a, const double2 *w) {
    cplx<double> o[4];
    tw4<S>(o,a[0],a[1],w[1],a[2],w[2],a[3],w[3]);
    a[0]=o[0]; a[1]=o[1]; a[2]=o[2]; a[3]=o[3];
  }
};

template<int S> struct TwButterfly<8,S> {
  static __device__ __forceinline__ void run(cplx<double> *a, const double2 *w) {
    cplx<double> e[4], o[4];
    tw4<S>(e,a[0],a[2],w[2],a[4],w[4],a[6],w[6]);
    tw4<S>(o,twmul<S>(a[1],w[1]),a[3],w[3],a[5],w[5],a[7],w[7]);
    combine8<S>(a,e,o);
  }
};

template<int S> struct TwButterfly<3,S> {
  static __device__ __forceinline__ void run(cplx<double> *a, const double2 *w) {
    const cplx<double> b1=twmul<S>(a[1],w[1]);
    const cplx<double> t=fmaTw<S>(b1,a[2],w[2]);
    radix3<S>(a,t,twoMinus(b1,t));
  }
};

// Whether a fused butterfly serves (T, R).
template<typename T, int R> __host__ __device__ constexpr bool fusedTw()
{
  return std::is_same<T,double>::value && (R == 2 || R == 3 || R == 4 ||
                                           R == 8);
}

// Inputs r >= 1 multiplied by tw[r*step] (S: its conjugate for S < 0),
// then the radix-R DFT.
template<int S> struct Codelet<8,S,double> {
  static __device__ __forceinline__ void run(cplx<double> *a) {
    cplx<double> e[4]={a[0],a[2],a[4],a[6]};
    cplx<double> o[4]={a[1],a[3],a[5],a[7]};
    Codelet<4,S,double>::run(e);
    Codelet<4,S,double>::run(o);
    combine8<S>(a,e,o);
  }
};

template<int S> struct Codelet<3,S,double> {
  static __device__ __forceinline__ void run(cplx<double> *a) {
    const cplx<double> t=a[1]+a[2];
    radix3<S>(a,t,a[1]-a[2]);
  }
};

template<typename T, int R, int S>
__device__ __forceinline__ void twiddledDFT(cplx<T> *a,
                                            const typename TwT<T>::type *tw,
                                            int step)
{
  if constexpr(fusedTw<T,R>()) {
    double2 w[R];
#pragma unroll
    for(int r=1; r < R; ++r) w[r]=tw[r*step];
    TwButterfly<R,S>::run(a,w);
  } else {
#pragma unroll
    for(int r=1; r < R; ++r) a[r]=twmul<S>(a[r],tw[r*step]);
    Codelet<R,S,T>::run(a);
  }
}

template<typename T, int R, int S>
__device__ __forceinline__ void fftStage(const cplx<T> *__restrict__ x,
                                         cplx<T> *__restrict__ y,
                                         int n, int Ns, int ncol, int ld,
                                         const typename TwT<T>::type *__restrict__ tw,
                                         int tid, int nthr)
{
  const int nR=n/R;
  const int tstride=n/(Ns*R);
  const int total=nR*ncol;
  const float invNcol=1.0f/(float) ncol;
  const float invNs=1.0f/(float) Ns;
  // Power-of-two column counts and spans (the common case) divide by
  // shifts and masks; the others through the float reciprocal.
  const bool p2c=(ncol & (ncol-1)) == 0, p2s=(Ns & (Ns-1)) == 0;
  const int lc=__ffs(ncol)-1;
  for(int idx=tid; idx < total; idx += nthr) {
    int j=p2c ? idx >> lc : fdiv(idx,invNcol);
    int c=idx-j*ncol;
    int k=p2s ? j & (Ns-1) : j-fdiv(j,invNs)*Ns;
    cplx<T> a[R];
#pragma unroll
    for(int r=0; r < R; ++r) a[r]=nrm(x[sp((j+r*nR)*ld+c)]);
    // Uniform per stage: the first stage has no twiddles; later stages apply
    // them to every element (W^0 = 1 exactly, so k = 0 needs no branch).
    if(Ns > 1) twiddledDFT<T,R,S>(a,tw,k*tstride);
    else Codelet<R,S,T>::run(a);
    int base=(j-k)*R+k;
#pragma unroll
    for(int r=0; r < R; ++r) y[sp((base+r*Ns)*ld+c)]=a[r];
  }
}

// Transform ncol columns (stride ld) of x in place through the ping-pong
// buffer y; element (i, c) lives at x[sp(i*ld+c)].  Every thread of the
// block must call it; the caller has synchronised after filling x.  Returns
// the buffer holding the result (x or y) and leaves the block synchronised.
template<typename T, int S>
__device__ cplx<T> *fftSmem(cplx<T> *x, cplx<T> *y, const FFTPlanDev& p,
                            int ncol, int ld, int tid, int nthr)
{
  const typename TwT<T>::type *tw=(const typename TwT<T>::type *) p.tw;
  int Ns=1;
  for(int s=0; s < p.nst; ++s) {
    int R=p.radix[s];
    switch(R) {
      case 8: fftStage<T,8,S>(x,y,p.n,Ns,ncol,ld,tw,tid,nthr); break;
      case 4: fftStage<T,4,S>(x,y,p.n,Ns,ncol,ld,tw,tid,nthr); break;
      case 2: fftStage<T,2,S>(x,y,p.n,Ns,ncol,ld,tw,tid,nthr); break;
      case 3: fftStage<T,3,S>(x,y,p.n,Ns,ncol,ld,tw,tid,nthr); break;
      case 5: fftStage<T,5,S>(x,y,p.n,Ns,ncol,ld,tw,tid,nthr); break;
      case 7: fftStage<T,7,S>(x,y,p.n,Ns,ncol,ld,tw,tid,nthr); break;
      default: break;
    }
    __syncthreads();
    cplx<T> *t=x; x=y; y=t;
    Ns *= R;
  }
  return x;
}

// ---------------------------------------------------------------------------
// In-place transforms for convolutions.  A decimation-in-frequency pass
// (fftDIF) takes natural order and leaves the spectrum in mixed-radix
// digit-reversed order; a decimation-in-time pass (fftDIT) over the same
// radices takes that order back to natural.  A pointwise product between
// them does not care about the order, so a convolution needs no
// permutation, and since every butterfly reads and writes the same R
// elements one buffer suffices (half the shared memory of the ping-pong
// Stockham form).  Stage with span Ls (m = Ls/R): butterfly (b, j) takes
// elements b Ls + j + r m; DIF multiplies output r by W_Ls^{S r j} after
// the R-point DFT, DIT multiplies input r by it before.
template<typename T, int R, int S, bool DIF>
__device__ __forceinline__ void ipStage(cplx<T> *__restrict__ x, int n, int Ls,
                                        int ncol, int ld,
                                        const typename TwT<T>::type *__restrict__ tw,
                                        int tid, int nthr)
{
  const int m=Ls/R;
  const int tstride=n/Ls;
  const int total=(n/R)*ncol;
  const float invNcol=1.0f/(float) ncol;
  const float invM=1.0f/(float) m;
  const bool p2c=(ncol & (ncol-1)) == 0, p2m=(m & (m-1)) == 0;
  const int lc=__ffs(ncol)-1, lm=__ffs(m)-1;
  for(int idx=tid; idx < total; idx += nthr) {
    int q=p2c ? idx >> lc : fdiv(idx,invNcol);
    int c=idx-q*ncol;
    int b=p2m ? q >> lm : fdiv(q,invM);
    int j=q-b*m;
    int base=b*Ls+j;
    cplx<T> a[R];
#pragma unroll
    for(int r=0; r < R; ++r) a[r]=nrm(x[sp((base+r*m)*ld+c)]);
    if(!DIF && m > 1) twiddledDFT<T,R,S>(a,tw,j*tstride);
    else Codelet<R,S,T>::run(a);
    if(DIF && m > 1) {
#pragma unroll
      for(int r=1; r < R; ++r) a[r]=twmul<S>(a[r],tw[r*j*tstride]);
    }
#pragma unroll
    for(int r=0; r < R; ++r) x[sp((base+r*m)*ld+c)]=a[r];
  }
}

// R16: the caller is compiled with the radix-16 and radix-6 stages (FP32
// plans made with allow16 may hold them; no other plan does).
template<typename T, int S, bool DIF, bool R16>
__device__ __forceinline__ void ipDispatch(int R, cplx<T> *x, int n, int Ls,
                                           int ncol, int ld,
                                           const typename TwT<T>::type *tw,
                                           int tid, int nthr)
{
  switch(R) {
    case 16:
      if constexpr(R16) ipStage<T,16,S,DIF>(x,n,Ls,ncol,ld,tw,tid,nthr);
      break;
    case 6:
      if constexpr(R16) ipStage<T,6,S,DIF>(x,n,Ls,ncol,ld,tw,tid,nthr);
      break;
    case 8: ipStage<T,8,S,DIF>(x,n,Ls,ncol,ld,tw,tid,nthr); break;
    case 4: ipStage<T,4,S,DIF>(x,n,Ls,ncol,ld,tw,tid,nthr); break;
    case 2: ipStage<T,2,S,DIF>(x,n,Ls,ncol,ld,tw,tid,nthr); break;
    case 3: ipStage<T,3,S,DIF>(x,n,Ls,ncol,ld,tw,tid,nthr); break;
    case 5: ipStage<T,5,S,DIF>(x,n,Ls,ncol,ld,tw,tid,nthr); break;
    case 7: ipStage<T,7,S,DIF>(x,n,Ls,ncol,ld,tw,tid,nthr); break;
    default: break;
  }
}

// Natural order in, digit-reversed spectrum out (in place).  Every thread
// of the block calls it after the block has synchronised; it returns
// synchronised.
template<typename T, int S, bool R16=false>
__device__ void fftDIF(cplx<T> *x, const FFTPlanDev& p, int ncol, int ld,
                       int tid, int nthr)
{
  const typename TwT<T>::type *tw=(const typename TwT<T>::type *) p.tw;
  int Ls=p.n;
  for(int s=0; s < p.nst; ++s) {
    int R=p.radix[s];
    ipDispatch<T,S,true,R16>(R,x,p.n,Ls,ncol,ld,tw,tid,nthr);
    __syncthreads();
    Ls /= R;
  }
}

// Digit-reversed spectrum (as fftDIF leaves it) in, natural order out.
template<typename T, int S, bool R16=false>
__device__ void fftDIT(cplx<T> *x, const FFTPlanDev& p, int ncol, int ld,
                       int tid, int nthr)
{
  const typename TwT<T>::type *tw=(const typename TwT<T>::type *) p.tw;
  int Ls=1;
  for(int s=p.nst-1; s >= 0; --s) {
    int R=p.radix[s];
    Ls *= R;
    ipDispatch<T,S,false,R16>(R,x,p.n,Ls,ncol,ld,tw,tid,nthr);
    __syncthreads();
  }
}

} // namespace fgb
