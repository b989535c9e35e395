// fftwpp_gb300_mult.cuh -- multipliers written by the caller, compiled into
// the GB300 row kernels.
//
// The reference lets a caller hand Convolution any function of type
// multiplier (convolve.h:78-79), called between the forward and backward
// padded transforms with the transformed indices of the current block in an
// Indices object (convolve.h:48-82; fftBase::index, convolve.h:297-326).  A
// host function cannot run inside a GPU kernel and there is no CPU
// fallback, so here the multiplier is a device functor that this header
// compiles into the library's innermost-axis (row) kernels, where it runs
// on registers between the forward and inverse row transforms exactly as
// the built-in multipliers do.  Include this header from a .cu file
// compiled with nvcc for sm_103a (-I <repo>/include), link lib_fftwpp.so.
//
// The functor:
//
//   struct MyMult {
//     static constexpr int A=2, B=1;          // values in, results out
//     template<class V>
//     __device__ void operator()(V *v, const fgb::Indices& ix) const {
//       v[0]=fgb::scale(v[0]*v[1],1.0+0.5*cospi(2.0*ix.index[0]/ix.size[0]));
//     }
//   };
//
// v[0..A-1] hold the A transformed inputs at one point of the padded grid;
// the functor overwrites v[0..B-1] with the B results.  V is
// fgb::cplx<double>, fgb::cplx<float> or fgb::cplx<fgb::ff> on complex
// data, and double, float or fgb::ff on real data (a Hermitian innermost
// axis: the reference's real multipliers see the same real values,
// convolve.cc:60-83).  ix.index[d] is the point's transformed index on axis
// d (outermost first), 0 <= ix.index[d] < ix.size[d] = the GPU plan's padded
// length N of that axis (a real outermost axis: the frequency, 0 ..
// N/2).  The functor must be trivially copyable (it is a kernel parameter).
//
// Plans: fgb_create(..., mult = FGB_MULT_USER, ...).  Then
//   fgb::convolveWith(plan, MyMult(), in, out, stream);   // device arrays
//   fgb::convolveHostWith(plan, MyMult(), in, out);       // host arrays
// PRECS (a bit mask: 1 FP64, 2 FP32, 4 float-float) limits the precisions
// instantiated, to save compile time; a plan of another precision then
// fails with an error.
#ifndef FFTWPP_GB300_MULT_CUH
#define FFTWPP_GB300_MULT_CUH

#include <memory>

#include "fftwpp_gb300.h"
#include "../fftwpp_gb300/csrc/rowkernels.cuh"

namespace fgb {

// Complex product for functors written once for every V.
template<typename T>
__device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b)
{
  return cmul(a,b);
}

// The real type underneath V and a double converted to it.
template<class V> struct Scalar {typedef V type;};
template<typename T> struct Scalar<cplx<T>> {typedef T type;};

template<class V>
__device__ __forceinline__ typename Scalar<V>::type scalar(double d)
{
  return (typename Scalar<V>::type) d;
}
template<>
__device__ __forceinline__ ff scalar<ff>(double d) {return ff(d);}
template<>
__device__ __forceinline__ ff scalar<cplx<ff>>(double d) {return ff(d);}

// v scaled by the real weight w (computed in FP64, rounded to V's type).
template<class V>
__device__ __forceinline__ V scale(V v, double w) {return v*scalar<V>(w);}

template<class F, int PRECS=7>
class FunctorLaunchers : public RowLaunchers {
public:
  explicit FunctorLaunchers(const F& f) {mul.f=f;}
  int inputs() const override {return F::A;}
  int outputs() const override {return F::B;}
  cudaError_t row(const RowPlan<double>& P, int t, long long g,
                  cudaStream_t s) const override {return rowT<1>(P,t,g,s);}
  cudaError_t row(const RowPlan<float>& P, int t, long long g,
                  cudaStream_t s) const override {return rowT<2>(P,t,g,s);}
  cudaError_t row(const RowPlan<ff>& P, int t, long long g,
                  cudaStream_t s) const override {return rowT<4>(P,t,g,s);}
  cudaError_t herm(const HermRowPlan<double>& P, int t, long long g,
                   cudaStream_t s) const override {return hermT<1>(P,t,g,s);}
  cudaError_t herm(const HermRowPlan<float>& P, int t, long long g,
                   cudaStream_t s) const override {return hermT<2>(P,t,g,s);}
  cudaError_t herm(const HermRowPlan<ff>& P, int t, long long g,
                   cudaStream_t s) const override {return hermT<4>(P,t,g,s);}
private:
  static_assert(F::A >= 1 && F::B >= 1 && F::B <= F::A && F::A <= FGB_MAXA,
                "a multiplier functor needs 1 <= B <= A <= 8");
  UserMult<F> mul;
  template<int BIT, typename T>
  cudaError_t rowT(const RowPlan<T>& P, int t, long long g,
                   cudaStream_t s) const
  {
    if constexpr((PRECS & BIT) != 0) return launchRowWith(P,mul,t,g,s);
    else return cudaErrorNotSupported;
  }
  template<int BIT, typename T>
  cudaError_t hermT(const HermRowPlan<T>& P, int t, long long g,
                    cudaStream_t s) const
  {
    if constexpr((PRECS & BIT) != 0) return launchHermRowWith(P,mul,t,g,s);
    else return cudaErrorNotSupported;
  }
};

// Convolve device arrays (in[A], out[B], as fgb_convolve_device) with the
// functor f on `stream`.  Returns 0, or a negative status with
// fgb_last_error().
template<int PRECS=7, class F>
int convolveWith(fgb_conv *plan, const F& f, void *const *in,
                 void *const *out, cudaStream_t stream=0)
{
  const FunctorLaunchers<F,PRECS> L(f);
  const RowLaunchers *base=&L;      // the library reads a RowLaunchers *
  return fgb_convolve_device_with(plan,base,in,out,(void *) stream);
}

// The row-kernel instantiation for f as a type-erased handle, for the C++
// drop-in API: Application(A, B, fftwpp::DeviceMultiplier{
// fgb::deviceLaunchers(f)}, ...) (include/convolve.h).
template<int PRECS=7, class F>
std::shared_ptr<const void> deviceLaunchers(const F& f)
{
  std::shared_ptr<const RowLaunchers> p=
    std::make_shared<const FunctorLaunchers<F,PRECS>>(f);
  // The erased pointer is the RowLaunchers base, which the library reads.
  return std::shared_ptr<const void>(p,static_cast<const void *>(p.get()));
}

// The same on host arrays (as fgb_convolve_host), synchronous.
template<int PRECS=7, class F>
int convolveHostWith(fgb_conv *plan, const F& f, void *const *in,
                     void *const *out)
{
  const FunctorLaunchers<F,PRECS> L(f);
  const RowLaunchers *base=&L;
  return fgb_convolve_host_with(plan,base,in,out);
}

} // namespace fgb

#endif
