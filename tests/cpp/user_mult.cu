// Multipliers written as caller device functors (fftwpp_gb300_mult.cuh),
// compiled by tests/test_gpu_user_mult.py into a small shared library next
// to lib_fftwpp.so and called through ctypes.
#include "fftwpp_gb300_mult.cuh"

// The advection Jacobian J = u0 u3 - u1 u2 on real physical values, the
// same product as the built-in realjacobian multiplier.
struct Jacobian {
  static constexpr int A=4, B=1;
  template<class V>
  __device__ void operator()(V *v, const fgb::Indices&) const
  {
    v[0]=v[0]*v[3]-v[1]*v[2];
  }
};

// A binary product weighted by a smooth function of the grid position:
// w = 1 + sum_d 0.25 (d+1) cos(2 pi index[d]/size[d]) (complex or real
// data alike).
struct Weighted {
  static constexpr int A=2, B=1;
  template<class V>
  __device__ void operator()(V *v, const fgb::Indices& ix) const
  {
    double w=1.0;
    for(int d=0; d < ix.dim; ++d)
      w += 0.25*(d+1)*cospi(2.0*(double) ix.index[d]/(double) ix.size[d]);
    v[0]=fgb::scale(v[0]*v[1],w);
  }
};

// Three outputs from three inputs that depend on the position in
// different ways (checks every output slot and the index of each axis).
struct Mixed {
  static constexpr int A=3, B=3;
  template<class V>
  __device__ void operator()(V *v, const fgb::Indices& ix) const
  {
    const V a=v[0], b=v[1], c=v[2];
    const double x=(double) ix.index[0]/(double) ix.size[0];
    const double y=(double) ix.index[ix.dim-1]/(double) ix.size[ix.dim-1];
    v[0]=fgb::scale(a*b,1.0+x);
    v[1]=fgb::scale(b*c,2.0-y);
    v[2]=a*c;
  }
};

extern "C" {

int user_jacobian_device(fgb_conv *c, void **in, void **out, void *s)
{
  return fgb::convolveWith<1>(c,Jacobian(),in,out,(cudaStream_t) s);
}

int user_weighted_device(fgb_conv *c, void **in, void **out, void *s)
{
  return fgb::convolveWith(c,Weighted(),in,out,(cudaStream_t) s);
}

int user_weighted_host(fgb_conv *c, void **in, void **out)
{
  return fgb::convolveHostWith(c,Weighted(),in,out);
}

int user_mixed_device(fgb_conv *c, void **in, void **out, void *s)
{
  return fgb::convolveWith<5>(c,Mixed(),in,out,(cudaStream_t) s);
}

}

// The same weighted product through the FFTW++-compatible C++ classes
// (include/convolve.h): a 2D centred-Hermitian Convolution2 whose y
// Application carries the functor, on host arrays with x stride Sx.
#include "convolve.h"

extern "C" int cpp_weighted_her2(const double *f, const double *g, double *h,
                                 size_t Lx, size_t Ly, size_t Sx, long *N)
{
  using namespace fftwpp;
  try {
    size_t Hy=utils::ceilquotient(Ly,2);
    Application appx(2,1,multNone);
    Application appy(2,1,DeviceMultiplier{fgb::deviceLaunchers(Weighted())},
                     appx);
    fftPadCentered fftx(Lx,3*utils::ceilquotient(Lx,2)-2*(Lx%2),appx,Hy,Sx);
    fftPadHermitian ffty(Ly,3*Hy-2*(Ly%2),appy);
    Convolution2 C(&fftx,&ffty);
    Complex **F=utils::ComplexAlign(2,Lx*Sx);
    for(size_t i=0; i < Lx; ++i)
      for(size_t j=0; j < Hy; ++j) {
        F[0][i*Sx+j]=Complex(f[2*(i*Hy+j)],f[2*(i*Hy+j)+1]);
        F[1][i*Sx+j]=Complex(g[2*(i*Hy+j)],g[2*(i*Hy+j)+1]);
      }
    C.convolve(F);
    for(size_t i=0; i < Lx; ++i)
      for(size_t j=0; j < Hy; ++j) {
        h[2*(i*Hy+j)]=F[0][i*Sx+j].re;
        h[2*(i*Hy+j)+1]=F[0][i*Sx+j].im;
      }
    N[0]=(long) fftx.paddedSize();
    N[1]=(long) ffty.paddedSize();
    utils::deleteAlign(F[0]);
    delete [] F;
  } catch(std::exception& e) {
    fprintf(stderr,"cpp_weighted_her2: %s\n",e.what());
    return -1;
  }
  return 0;
}
