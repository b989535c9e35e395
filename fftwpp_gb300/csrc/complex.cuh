// complex.cuh -- complex arithmetic and twiddle types for the GB300 engine.
//
// Two arithmetic types are supported:
//   double : FP64 drop-in mode, twiddles stored as double2;
//   float  : FP32 compensated mode, every twiddle stored as an unevaluated
//            sum hi+lo of two floats derived from the FP64 value, so a
//            twiddle multiply a*(hi+lo) keeps ~2^-48 relative twiddle
//            accuracy while the butterfly data stays FP32.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fgb {

template<typename T> struct cplx { T x, y; };

template<typename T> struct TwT;
template<> struct TwT<double> { typedef double2 type; };
template<> struct TwT<float>  { typedef float4 type; };   // (hi.x, hi.y, lo.x, lo.y)

template<typename T>
__host__ __device__ __forceinline__ cplx<T> mk(T a, T b) { cplx<T> r; r.x=a; r.y=b; return r; }

template<typename T>
__device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk(a.x+b.x,a.y+b.y); }
template<typename T>
__device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk(a.x-b.x,a.y-b.y); }
template<typename T>
__device__ __forceinline__ cplx<T> operator*(cplx<T> a, T s) { return mk(a.x*s,a.y*s); }

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

template<typename T>
__device__ __forceinline__ cplx<T> conjg(cplx<T> a) { return mk(a.x,-a.y); }

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
  // (hi + lo) applied as a*lo first, then the dominant a*hi term fused in.
  float wy=S > 0 ? w.y : -w.y;
  float ly=S > 0 ? w.w : -w.w;
  float rx=fmaf(a.x,w.z,-a.y*ly);
  float ry=fmaf(a.x,ly,a.y*w.z);
  rx=fmaf(a.x,w.x,fmaf(-a.y,wy,rx));
  ry=fmaf(a.x,wy,fmaf(a.y,w.x,ry));
  return mk(rx,ry);
}

// Runtime-sign variants.
__device__ __forceinline__ cplx<double> twmulr(cplx<double> a, double2 w, int s)
{
  return s > 0 ? twmul<1>(a,w) : twmul<-1>(a,w);
}
__device__ __forceinline__ cplx<float> twmulr(cplx<float> a, float4 w, int s)
{
  return s > 0 ? twmul<1>(a,w) : twmul<-1>(a,w);
}

__device__ __forceinline__ cplx<double> twval(double2 w) { return mk(w.x,w.y); }
__device__ __forceinline__ cplx<float> twval(float4 w) { return mk(w.x,w.y); }

} // namespace fgb
