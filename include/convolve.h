// convolve.h -- the FFTW++ C++ convolution API, served by the GB300 engine.
//
// Drop-in for the reference's convolve.h class set (convolve.h:48-1893):
// Application, the padded transforms fftPad / fftPadCentered /
// fftPadHermitian / fftPadReal, the drivers Convolution / Convolution2 /
// Convolution3, the multipliers multNone / multBinary / realMultBinary /
// multcorrelation, HermitianSymmetrize{,X,XY}, and the aligned allocators of
// align.h (utils::ComplexAlign, utils::doubleAlign, utils::deleteAlign).
// User code written against the reference compiles unchanged against this
// header and lib_fftwpp.so; every convolve() copies the host arrays to the
// GB300, runs the sm_103a kernels and copies the B results back into
// f[0..B-1], normalised by 1/prod(m q) (convolveRaw: unnormalised).
//
// Differences, all stated in the library's documentation:
//  * the optimiser times GPU plans instead of CPU ones, so the public
//    members m, p, q, n of a transform are those of the GPU plan, filled in
//    when the Convolution that uses it is constructed; a forced
//    Application m is honoured (convolve.h:103-111);
//  * a host function pointer cannot run on the device and there is no CPU
//    fallback, so a multiplier is one of the built-ins (or
//    jacobianMultiplier), recognised by address, or a device functor
//    compiled into the row kernels: Application(A, B, DeviceMultiplier{
//    fgb::deviceLaunchers(functor)}, ...) from a .cu file that includes
//    fftwpp_gb300_mult.cuh; any other host multiplier throws
//    std::invalid_argument;
//  * errors throw std::runtime_error instead of exit() (convolve.h:226-232).
#ifndef FFTWPP_GB300_CONVOLVE_H
#define FFTWPP_GB300_CONVOLVE_H

#include <cmath>
#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "cfftw++.h"
#include "fftwpp_gb300.h"

#ifndef __Complex_h__
// Interleaved complex double (the reference's Complex.h:30-45 layout).
class Complex {
public:
  double re, im;
  Complex() : re(0.0), im(0.0) {}
  Complex(double r, double i=0.0) : re(r), im(i) {}
  double real() const {return re;}
  double imag() const {return im;}
  Complex& operator+=(const Complex& b) {re += b.re; im += b.im; return *this;}
  Complex& operator-=(const Complex& b) {re -= b.re; im -= b.im; return *this;}
  Complex& operator*=(const Complex& b) {
    double r=re*b.re-im*b.im;
    im=re*b.im+im*b.re;
    re=r;
    return *this;
  }
  Complex& operator*=(double s) {re *= s; im *= s; return *this;}
};
inline Complex operator+(Complex a, const Complex& b) {return a += b;}
inline Complex operator-(Complex a, const Complex& b) {return a -= b;}
inline Complex operator*(Complex a, const Complex& b) {return a *= b;}
inline Complex operator*(Complex a, double s) {return a *= s;}
inline Complex conj(const Complex& a) {return Complex(a.re,-a.im);}
inline double abs2(const Complex& a) {return a.re*a.re+a.im*a.im;}
#endif

namespace utils {

inline size_t ceilquotient(size_t a, size_t b) {return (a+b-1)/b;}

// Page-locked (when a GPU is present) 64-byte aligned host memory
// (align.h:114-160).
inline Complex *ComplexAlign(size_t size)
{
  if(size == 0) return NULL;
  return (Complex *) create_complexAlign(size);
}

inline Complex **ComplexAlign(size_t n, size_t size)
{
  if(n == 0 || size == 0) return NULL;
  Complex **v=new Complex*[n];
  size_t Size=(size+3)/4*4;
  Complex *B=ComplexAlign((n-1)*Size+size);
  for(size_t i=0; i < n; ++i) v[i]=B+i*Size;
  return v;
}

inline double *doubleAlign(size_t size) {return create_doubleAlign(size);}

inline double **doubleAlign(size_t n, size_t size)
{
  if(n == 0 || size == 0) return NULL;
  double **v=new double*[n];
  size_t Size=(size+7)/8*8;
  double *B=doubleAlign((n-1)*Size+size);
  for(size_t i=0; i < n; ++i) v[i]=B+i*Size;
  return v;
}

inline void deleteAlign(Complex *p) {delete_complexAlign((FFTWPP_C128 *) p);}
inline void deleteAlign(double *p) {delete_doubleAlign(p);}

} // namespace utils

namespace fftwpp {

struct fftw {
  static size_t& maxthreadsRef() {static size_t n=1; return n;}
};

class fftBase;

class Indices {
public:
  fftBase *fft;
  size_t *index;
  size_t size, maxsize;
  size_t r;
  size_t offset;
  Indices() : fft(NULL), index(NULL), size(0), maxsize(0), r(0), offset(0) {}
};

typedef void multiplier(Complex **F, size_t n, Indices *indices,
                        size_t threads);

// Host bodies of the built-in multipliers (convolve.cc:26-110).  The GPU
// path recognises them by address and runs its fused device versions.
inline void multNone(Complex **, size_t, Indices *, size_t) {}
inline void multBinary(Complex **F, size_t n, Indices *, size_t)
{
  for(size_t j=0; j < n; ++j) F[0][j] *= F[1][j];
}
inline void realMultBinary(Complex **F, size_t n, Indices *, size_t)
{
  double *F0=(double *) F[0], *F1=(double *) F[1];
  for(size_t j=0; j < n; ++j) F0[j] *= F1[j];
}
inline void multcorrelation(Complex **F, size_t n, Indices *, size_t)
{
  for(size_t j=0; j < n; ++j) F[0][j] *= conj(F[1][j]);
}
// Physical-space Jacobian of four real fields: F0 = F0 F3 - F1 F2.
inline void jacobianMultiplier(Complex **F, size_t n, Indices *, size_t)
{
  double *F0=(double *) F[0], *F1=(double *) F[1], *F2=(double *) F[2],
    *F3=(double *) F[3];
  for(size_t j=0; j < n; ++j) F0[j]=F0[j]*F3[j]-F1[j]*F2[j];
}

// A multiplier compiled for the device from a caller's functor: the
// row-kernel instantiation built by fgb::deviceLaunchers (declared in
// fftwpp_gb300_mult.cuh, which needs nvcc), kept alive by this handle.
struct DeviceMultiplier {
  std::shared_ptr<const void> launchers;
};

inline int multiplierCode(multiplier *m)
{
  if(m == multNone) return FGB_MULT_NONE;
  if(m == multBinary) return FGB_MULT_BINARY;
  if(m == realMultBinary) return FGB_MULT_REALBINARY;
  if(m == multcorrelation) return FGB_MULT_CORRELATION;
  if(m == jacobianMultiplier) return FGB_MULT_REALJACOBIAN;
  throw std::invalid_argument("fftwpp_gb300: user multipliers have no "
                              "device form; use a built-in multiplier");
}

// Application (convolve.h:84-121).
class Application {
public:
  size_t A, B;
  multiplier *mult;
  size_t threads;
  bool verbose;
  size_t m, D;
  ptrdiff_t I;
  size_t maxthreads;
  DeviceMultiplier device;
  Application(size_t A, size_t B, multiplier *mult,
              size_t threads=fftw::maxthreadsRef(), bool verbose=false,
              size_t m=0, size_t D=0, ptrdiff_t I=-1)
    : A(A), B(B), mult(mult), threads(threads), verbose(verbose),
      m(m == 1 ? 0 : m), D(D), I(I), maxthreads(threads) {}
  Application(size_t A, size_t B, multiplier *mult, Application& parent,
              size_t m=0, size_t D=0, ptrdiff_t I=-1)
    : A(A), B(B), mult(mult), threads(1), verbose(parent.verbose),
      m(m == 1 ? 0 : m), D(D), I(I), maxthreads(parent.maxthreads) {}
  // A device functor in place of the host multiplier.
  Application(size_t A, size_t B, DeviceMultiplier device,
              size_t threads=fftw::maxthreadsRef(), bool verbose=false,
              size_t m=0, size_t D=0, ptrdiff_t I=-1)
    : A(A), B(B), mult(NULL), threads(threads), verbose(verbose),
      m(m == 1 ? 0 : m), D(D), I(I), maxthreads(threads), device(device) {}
  Application(size_t A, size_t B, DeviceMultiplier device,
              Application& parent, size_t m=0, size_t D=0, ptrdiff_t I=-1)
    : A(A), B(B), mult(NULL), threads(1), verbose(parent.verbose),
      m(m == 1 ? 0 : m), D(D), I(I), maxthreads(parent.maxthreads),
      device(device) {}
};

// fftBase (convolve.h:123-464): the padding specification of one axis.
class fftBase {
public:
  size_t L, M, C, S;
  size_t m, p, q, n, D;
  bool inplace;
  Application app;
  bool centered;
  int kind;
  fftBase(int kind, size_t L, size_t M, Application& app, size_t C,
          size_t S, bool centered)
    : L(L), M(M), C(C), S(S == 0 ? C : S), m(0), p(0), q(0), n(0), D(1),
      inplace(false), app(app), centered(centered), kind(kind) {
    if(L > M) throw std::runtime_error("L="+std::to_string(L)+
                                       " is greater than M="+std::to_string(M));
    if(this->S < C) throw std::runtime_error("stride S cannot be less than "
                                             "count C");
    m=app.m;
  }
  virtual ~fftBase() {}
  size_t normalization() const {return m*q;}
  size_t paddedSize() const {return m*q;}
  virtual size_t inputLength() const {return L;}
  void setPlan(const long *info) {   // from fgb_info
    m=info[0]; p=info[1]; q=info[2]; n=q; M=info[3];
  }
};

class fftPad : public fftBase {
public:
  fftPad(size_t L, size_t M, Application& app, size_t C=1, size_t S=0,
         bool Explicit=false)
    : fftBase(FGB_PAD,L,M,app,C,S,false) {if(Explicit && !m) m=M;}
  fftPad(size_t L, size_t M, Application& app, size_t C, size_t S,
         size_t m, size_t D, bool inplace)
    : fftBase(FGB_PAD,L,M,app,C,S,false) {this->m=m; this->D=D;
      this->inplace=inplace;}
protected:
  fftPad(int kind, size_t L, size_t M, Application& app, size_t C, size_t S,
         bool centered) : fftBase(kind,L,M,app,C,S,centered) {}
};

class fftPadCentered : public fftPad {
public:
  fftPadCentered(size_t L, size_t M, Application& app, size_t C=1,
                 size_t S=0, bool Explicit=false)
    : fftPad(FGB_CENTERED,L,M,app,C,S,true) {if(Explicit && !m) m=M;}
  fftPadCentered(size_t L, size_t M, Application& app, size_t C, size_t S,
                 size_t m, size_t D, bool inplace)
    : fftPad(FGB_CENTERED,L,M,app,C,S,true) {this->m=m; this->D=D;
      this->inplace=inplace;}
};

class fftPadHermitian : public fftBase {
public:
  fftPadHermitian(size_t L, size_t M, Application& app, size_t C=1,
                  bool Explicit=false)
    : fftBase(FGB_HERMITIAN,L,M,app,C,C,true) {if(Explicit && !m) m=M;}
  fftPadHermitian(size_t L, size_t M, Application& app, size_t C, size_t m,
                  size_t D, bool inplace)
    : fftBase(FGB_HERMITIAN,L,M,app,C,C,true) {this->m=m; this->D=D;
      this->inplace=inplace;}
  size_t inputLength() const {return utils::ceilquotient(L,2);}
};

class fftPadReal : public fftBase {
public:
  fftPadReal(size_t L, size_t M, Application& app, size_t C=1, size_t S=0,
             bool Explicit=false)
    : fftBase(FGB_REAL,L,M,app,C,S,false) {if(Explicit && !m) m=M;}
  fftPadReal(size_t L, size_t M, Application& app, size_t C, size_t S,
             size_t m, size_t D, bool inplace)
    : fftBase(FGB_REAL,L,M,app,C,S,false) {this->m=m; this->D=D;
      this->inplace=inplace;}
};

// Shared driver: one GPU plan over 1-3 axes.
class ConvolutionBase {
protected:
  fgb_conv *plan;
  std::vector<fftBase *> ffts;
  size_t A, B;
  std::shared_ptr<const void> launchers;     // device functor, if any
  void build(std::vector<fftBase *> axes) {
    ffts=axes;
    int dim=(int) axes.size();
    Application& app=axes.back()->app;
    A=app.A;
    B=app.B;
    int kinds[3];
    size_t L[3], M[3], m[3];
    for(int d=0; d < dim; ++d) {
      kinds[d]=axes[d]->kind;
      L[d]=axes[d]->L;
      M[d]=axes[d]->M;
      m[d]=axes[d]->m;
    }
    // Layouts (convolve.h:1274, 1556, 1614-1622): in 2D the x axis has C =
    // the stored y entries and stride S = Sx >= C; in 3D the y axis has
    // C = the stored z entries and S = Sy, the x axis S = Sx >= Ly Sy and
    // C = Ly Sy when Sy is the z extent, else the z extent.
    size_t S[3]={0,0,0};
    bool dense=true;
    if(dim == 2) {
      size_t Hy=axes[1]->inputLength();
      if(axes[0]->C != Hy)
        throw std::invalid_argument("fftwpp_gb300: the x transform's count C "
                                    "must be the stored y extent");
      S[0]=axes[0]->S;
      dense=S[0] == Hy;
    } else if(dim == 3) {
      size_t Hz=axes[2]->inputLength();
      if(axes[1]->C != Hz)
        throw std::invalid_argument("fftwpp_gb300: the y transform's count C "
                                    "must be the stored z extent");
      S[1]=axes[1]->S;
      S[0]=axes[0]->S;
      if(axes[0]->C != (S[1] == Hz ? L[1]*S[1] : Hz))
        throw std::invalid_argument("fftwpp_gb300: the x transform's count C "
                                    "must be Ly Sy (contiguous y-z planes) "
                                    "or the stored z extent");
      dense=S[1] == Hz && S[0] == L[1]*Hz;
    }
    launchers=app.device.launchers;
    int code=launchers ? FGB_MULT_USER : multiplierCode(app.mult);
    plan=fgb_create(dim,kinds,L,M,m,(int) A,(int) B,code,
                    fgb_get_drop_in_precision(),1);
    if(!plan) throw std::runtime_error(fgb_last_error());
    if(!dense && fgb_set_strides(plan,S) != 0) {
      std::string why=fgb_last_error();
      fgb_destroy(plan);
      plan=NULL;
      throw std::invalid_argument(why);
    }
    long info[32];
    fgb_info(plan,info);
    for(int d=0; d < dim; ++d) axes[d]->setPlan(info+8*d);
  }
  void run(Complex **f, size_t offset, bool normalize) {
    void *in[8];
    for(size_t a=0; a < A; ++a) in[a]=(void *) (f[a]+offset);
    fgb_set_normalize(plan,normalize ? 1 : 0);
    int rc=launchers ? fgb_convolve_host_with(plan,launchers.get(),in,in) :
      fgb_convolve_host(plan,in,in);
    if(rc != 0) throw std::runtime_error(fgb_last_error());
  }
public:
  ConvolutionBase() : plan(NULL), A(0), B(0) {}
  virtual ~ConvolutionBase() {if(plan) fgb_destroy(plan);}
  double normalization() const {
    double N=1;
    for(fftBase *f : ffts) N *= (double) f->normalization();
    return N;
  }
};

// Convolution (convolve.h:982-1166).
class Convolution : public ConvolutionBase {
public:
  fftBase *fft;
  Convolution(fftBase *fft, Complex **F=NULL, Complex *W=NULL,
              Complex *V=NULL) : fft(fft) {
    if(fft->C != 1)
      throw std::invalid_argument("fftwpp_gb300: a 1D Convolution needs C=1");
    build({fft});
  }
  void convolveRaw(Complex **f) {run(f,0,false);}
  void convolveRaw(double **f) {run((Complex **) f,0,false);}
  void convolve(Complex **f) {run(f,0,true);}
  void convolve(Complex **f, size_t offset) {run(f,offset,true);}
  void convolve(double **f) {run((Complex **) f,0,true);}
};

// Convolution2 (convolve.h:1269-1548).
class Convolution2 : public ConvolutionBase {
public:
  fftBase *fftx, *ffty;
  Convolution2(fftBase *fftx, fftBase *ffty, Complex **F=NULL,
               Complex *W=NULL, Complex *V=NULL) : fftx(fftx), ffty(ffty) {
    build({fftx,ffty});
  }
  void convolveRaw(Complex **f, size_t offset=0) {run(f,offset,false);}
  void convolve(Complex **f, size_t offset=0) {run(f,offset,true);}
  void convolve(double **f, size_t offset=0) {run((Complex **) f,offset,true);}
};

// Convolution3 (convolve.h:1550-1893).
class Convolution3 : public ConvolutionBase {
public:
  fftBase *fftx, *ffty, *fftz;
  Convolution3(fftBase *fftx, fftBase *ffty, fftBase *fftz,
               Complex **F=NULL, Complex *W=NULL, Complex *V=NULL)
    : fftx(fftx), ffty(ffty), fftz(fftz) {
    build({fftx,ffty,fftz});
  }
  void convolveRaw(Complex **f, size_t offset=0) {run(f,offset,false);}
  void convolve(Complex **f, size_t offset=0) {run(f,offset,true);}
  void convolve(double **f, size_t offset=0) {run((Complex **) f,offset,true);}
};

// Hermitian symmetrisation of host data (convolve.h:1168-1267).
inline void HermitianSymmetrize(Complex *f) {f[0].im=0.0;}

inline void HermitianSymmetrizeX(size_t Hx, size_t Hy, size_t x0, Complex *f,
                                 size_t Sx, size_t=0)
{
  Complex *F=f+x0*Sx;
  for(size_t i=1; i < Hx; ++i) *(F-i*Sx)=conj(F[i*Sx]);
  F[0].im=0.0;
  if(x0 == Hx)
    for(size_t j=0; j < Hy; ++j) f[j]=Complex(0.0,0.0);
}

inline void HermitianSymmetrizeX(size_t Hx, size_t Hy, size_t x0, Complex *f)
{
  HermitianSymmetrizeX(Hx,Hy,x0,f,Hy);
}

inline void HermitianSymmetrizeXY(size_t Hx, size_t Hy, size_t Hz, size_t x0,
                                  size_t y0, Complex *f)
{
  fftwpp_HermitianSymmetrizeXY(Hx,Hy,Hz,x0,y0,(FFTWPP_C128 *) f);
}

// The convenience classes of wrappers/HybridConvolution.h, also under the
// ConvolutionHermitian names.
class ConvolutionHermitian {
public:
  Application app;
  fftPadHermitian fft;
  Convolution conv;
  ConvolutionHermitian(size_t L, multiplier *mult=realMultBinary, size_t M=0,
                       size_t A=2, size_t B=1)
    : app(A,B,mult), fft(L,M ? M : 3*utils::ceilquotient(L,2)-2*(L%2),app),
      conv(&fft) {}
  void convolve(Complex **f) {conv.convolve(f);}
};

class ConvolutionHermitian2 {
public:
  Application appx, appy;
  fftPadCentered fftx;
  fftPadHermitian ffty;
  Convolution2 conv;
  ConvolutionHermitian2(size_t Lx, size_t Ly, multiplier *mult=realMultBinary,
                        size_t Mx=0, size_t My=0, size_t A=2, size_t B=1)
    : appx(A,B,multNone), appy(A,B,mult,appx),
      fftx(Lx,Mx ? Mx : 3*utils::ceilquotient(Lx,2)-2*(Lx%2),appx,
           utils::ceilquotient(Ly,2),utils::ceilquotient(Ly,2)),
      ffty(Ly,My ? My : 3*utils::ceilquotient(Ly,2)-2*(Ly%2),appy),
      conv(&fftx,&ffty) {}
  void convolve(Complex **f) {conv.convolve(f);}
};

class ConvolutionHermitian3 {
public:
  Application appx, appy, appz;
  fftPadCentered fftx, ffty;
  fftPadHermitian fftz;
  Convolution3 conv;
  ConvolutionHermitian3(size_t Lx, size_t Ly, size_t Lz,
                        multiplier *mult=realMultBinary, size_t Mx=0,
                        size_t My=0, size_t Mz=0, size_t A=2, size_t B=1)
    : appx(A,B,multNone), appy(A,B,multNone,appx), appz(A,B,mult,appy),
      fftx(Lx,Mx ? Mx : 3*utils::ceilquotient(Lx,2)-2*(Lx%2),appx,
           Ly*utils::ceilquotient(Lz,2),Ly*utils::ceilquotient(Lz,2)),
      ffty(Ly,My ? My : 3*utils::ceilquotient(Ly,2)-2*(Ly%2),appy,
           utils::ceilquotient(Lz,2),utils::ceilquotient(Lz,2)),
      fftz(Lz,Mz ? Mz : 3*utils::ceilquotient(Lz,2)-2*(Lz%2),appz),
      conv(&fftx,&ffty,&fftz) {}
  void convolve(Complex **f) {conv.convolve(f);}
};

typedef ConvolutionHermitian HybridConvolutionHermitian;
typedef ConvolutionHermitian2 HybridConvolutionHermitian2;
typedef ConvolutionHermitian3 HybridConvolutionHermitian3;

} // namespace fftwpp

#endif
