// complex.cuh -- complex arithmetic and twiddle types for the GB300 engine.
//
// Three arithmetic types are supported:
//   double : FP64 drop-in mode, twiddles stored as double2;
//   float  : FP32 compensated mode, every twiddle stored as an unevaluated
//            sum hi+lo of two floats derived from the FP64 value, so a
//            twiddle multiply a*(hi+lo) keeps ~2^-48 relative twiddle
//            accuracy while the butterfly data stays FP32;
//   ff     : float-float mode, data and arithmetic both hi+lo pairs (FP64
//            data at the interface, FP64-grade accuracy on the FP32 pipe).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fgb {

// The CUDA fma overloads (double, float) stay visible next to the
// float-float one below.
using ::fma;

// ---------------------------------------------------------------------------
// Float-float arithmetic: a real number held as the unevaluated sum hi + lo
// of two floats with |lo| <= ulp(hi)/2, about 48 significant bits.  GB300
// issues FP32 instructions at 64 times its FP64 rate, so transforms in this
// type keep FP64-grade normwise accuracy at a fraction of the FP64 cost.
// The operations are the error-free transformations of Knuth (TwoSum),
// Dekker (FastTwoSum) and the FMA-based TwoProduct; the addition is the
// "sloppy" double-word sum, whose error is bounded by 2^-46 (|a| + |b|),
// which is the normwise bound an FFT needs.  Renormalisation is lazy: the
// arithmetic operators return hi + lo unrenormalised (|lo| may exceed
// ulp(hi)/2 by a small factor) and the transforms renormalise every value
// they load (nrm), so a chain of at most one radix stage runs between
// renormalisations.  The _rn intrinsics keep the compiler from fusing the
// error terms into multiply-adds.
struct ff {
  float hi, lo;
  ff() = default;
  __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr explicit ff(double d)
    : hi((float) d), lo((float) (d-(double) (float) d)) {}
};

__device__ __forceinline__ ff ffTwoSum(float a, float b)
{
  float s=__fadd_rn(a,b);
  float bb=__fsub_rn(s,a);
  float e=__fadd_rn(__fsub_rn(a,__fsub_rn(s,bb)),__fsub_rn(b,bb));
  return ff(s,e);
}

// Renormalise s + e for |s| >= |e|.
__device__ __forceinline__ ff ffFast(float s, float e)
{
  float t=__fadd_rn(s,e);
  return ff(t,__fsub_rn(e,__fsub_rn(t,s)));
}

__device__ __forceinline__ ff nrm(ff a) {return ffFast(a.hi,a.lo);}

__device__ __forceinline__ ff operator+(ff a, ff b)
{
  ff s=ffTwoSum(a.hi,b.hi);
  return ff(s.hi,__fadd_rn(s.lo,__fadd_rn(a.lo,b.lo)));
}
__device__ __forceinline__ ff operator-(ff a) {return ff(-a.hi,-a.lo);}
__device__ __forceinline__ ff operator-(ff a, ff b) {return a+(-b);}

__device__ __forceinline__ ff operator*(ff a, ff b)
{
  float p=__fmul_rn(a.hi,b.hi);
  float e=fmaf(a.hi,b.hi,-p);
  e=fmaf(a.hi,b.lo,e);
  e=fmaf(a.lo,b.hi,e);
  return ff(p,e);
}

// a*b + c.
__device__ __forceinline__ ff fma(ff a, ff b, ff c)
{
  float p=__fmul_rn(a.hi,b.hi);
  float e=fmaf(a.hi,b.hi,-p);
  ff s=ffTwoSum(p,c.hi);
  float l=__fadd_rn(__fadd_rn(s.lo,e),c.lo);
  l=fmaf(a.hi,b.lo,l);
  l=fmaf(a.lo,b.hi,l);
  return ff(s.hi,l);
}

// a*b + c*d with one renormalisation (complex multiplies).
__device__ __forceinline__ ff ffDot2(ff a, ff b, ff c, ff d)
{
  float p1=__fmul_rn(a.hi,b.hi);
  float e1=fmaf(a.hi,b.hi,-p1);
  float p2=__fmul_rn(c.hi,d.hi);
  float e2=fmaf(c.hi,d.hi,-p2);
  ff s=ffTwoSum(p1,p2);
  float l=__fadd_rn(s.lo,__fadd_rn(e1,e2));
  l=fmaf(a.hi,b.lo,l);
  l=fmaf(a.lo,b.hi,l);
  l=fmaf(c.hi,d.lo,l);
  l=fmaf(c.lo,d.hi,l);
  return ff(s.hi,l);
}

template<typename T> struct cplx { T x, y; };
// Complex values move as one vector (8 bytes for FP32, 16 for FP64 and
// float-float): aligned to their size, so every shared and global access of
// an element is a single 64- or 128-bit load or store.
template<> struct __align__(8) cplx<float> { float x, y; };
template<> struct __align__(16) cplx<double> { double x, y; };
template<> struct __align__(16) cplx<ff> { ff x, y; };

template<typename T> struct TwT;
template<> struct TwT<double> { typedef double2 type; };
template<> struct TwT<float>  { typedef float4 type; };   // (hi.x, hi.y, lo.x, lo.y)
template<> struct TwT<ff>     { typedef float4 type; };   // the same split

template<typename T>
__host__ __device__ __forceinline__ cplx<T> mk(T a, T b) { cplx<T> r; r.x=a; r.y=b; return r; }

template<typename T>
__device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk(a.x+b.x,a.y+b.y); }
template<typename T>
__device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk(a.x-b.x,a.y-b.y); }
template<typename T>
__device__ __forceinline__ cplx<T> operator*(cplx<T> a, T s) { return mk(a.x*s,a.y*s); }

// FP32 complex values as float2 pairs for the packed FP32 instructions of
// sm_100-class GPUs (one FADD2 / FMUL2 / FFMA2 does both components).
__device__ __forceinline__ float2 f2(cplx<float> a) {return make_float2(a.x,a.y);}
__device__ __forceinline__ cplx<float> c2(float2 v) {return mk(v.x,v.y);}
__device__ __forceinline__ cplx<float> operator+(cplx<float> a, cplx<float> b)
{
  return c2(__fadd2_rn(f2(a),f2(b)));
}
__device__ __forceinline__ cplx<float> operator-(cplx<float> a, cplx<float> b)
{
  return c2(__fadd2_rn(f2(a),make_float2(-b.x,-b.y)));
}
__device__ __forceinline__ cplx<float> operator*(cplx<float> a, float s)
{
  return c2(__fmul2_rn(f2(a),make_float2(s,s)));
}

template<typename T>
__device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b)
{
  return mk(fma(a.x,b.x,-a.y*b.y),fma(a.x,b.y,a.y*b.x));
}

template<typename T>
__device__ __forceinline__ cplx<T> cmulconj(cplx<T> a, cplx<T> b)   // a*conj(b)
{
  return mk(fma(a.x,b.x,a.y*b.y),fma(a.y,b.x,-a.x*b.y));
}

__device__ __forceinline__ cplx<ff> cmul(cplx<ff> a, cplx<ff> b)
{
  return mk(ffDot2(a.x,b.x,-a.y,b.y),ffDot2(a.x,b.y,a.y,b.x));
}

__device__ __forceinline__ cplx<ff> cmulconj(cplx<ff> a, cplx<ff> b)
{
  return mk(ffDot2(a.x,b.x,a.y,b.y),ffDot2(a.y,b.x,-a.x,b.y));
}

template<typename T>
__device__ __forceinline__ cplx<T> conjg(cplx<T> a) { return mk(a.x,-a.y); }

// One step of a long running sum (folds over p blocks, accumulation over
// q residues): float-float renormalises every step, since an unrenormalised
// chain of hundreds of additions loses accuracy in its lo parts.
template<typename T>
__device__ __forceinline__ cplx<T> accum(cplx<T> a, cplx<T> b) { return a+b; }
__device__ __forceinline__ cplx<ff> accum(cplx<ff> a, cplx<ff> b);

// Renormalise a loaded value (float-float only).
template<typename T>
__device__ __forceinline__ cplx<T> nrm(cplx<T> a) { return a; }
__device__ __forceinline__ cplx<ff> nrm(cplx<ff> a)
{
  return mk(nrm(a.x),nrm(a.y));
}

__device__ __forceinline__ cplx<ff> accum(cplx<ff> a, cplx<ff> b)
{
  return nrm(a+b);
}

// s*i*a for s = +1 or -1 (compile time).
template<int S, typename T>
__device__ __forceinline__ cplx<T> mulI(cplx<T> a)
{
  return S > 0 ? mk(-a.y,a.x) : mk(a.y,-a.x);
}

// a * w^S where w is a stored twiddle exp(+i theta); S=-1 uses conj(w).
template<int S>
__device__ __forceinline__ cplx<double> twmul(cplx<double> a, double2 w)
{
  if(S > 0) return mk(fma(a.x,w.x,-a.y*w.y),fma(a.x,w.y,a.y*w.x));
  return mk(fma(a.x,w.x,a.y*w.y),fma(a.y,w.x,-a.x*w.y));
}

template<int S>
__device__ __forceinline__ cplx<float> twmul(cplx<float> a, float4 w)
{
  // (hi + lo) applied as a*lo first, then the dominant a*hi term fused in;
  // both components at once with the packed FP32 instructions, in the
  // rounding order of the scalar form rx = ax wx + (-ay wy + (ax lx +
  // (-ay ly))), ry likewise.
  const float wy=S > 0 ? w.y : -w.y;
  const float ly=S > 0 ? w.w : -w.w;
  const float2 ax=make_float2(a.x,a.x), ay=make_float2(a.y,a.y);
  float2 r=__fmul2_rn(ay,make_float2(-ly,w.z));
  r=__ffma2_rn(ax,make_float2(w.z,ly),r);
  r=__ffma2_rn(ay,make_float2(-wy,w.x),r);
  r=__ffma2_rn(ax,make_float2(w.x,wy),r);
  return c2(r);
}

template<int S>
__device__ __forceinline__ cplx<ff> twmul(cplx<ff> a, float4 w)
{
  ff wx(w.x,w.z);
  ff wy=S > 0 ? ff(w.y,w.w) : ff(-w.y,-w.w);
  return mk(ffDot2(a.x,wx,-a.y,wy),ffDot2(a.x,wy,a.y,wx));
}

} // namespace fgb
