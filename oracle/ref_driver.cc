// ref_driver.cc -- ctypes-callable driver over the REFERENCE implementation.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile together with the
// reference's own convolve.cc / fftw++.cc / parallel.cc (FFTW++, compiled
// from its sources where they lie) and the clean-room FFTW3 backend in
// oracle/fftw3_shim, into oracle/_ref/libfftwpp_ref.so.  It is used to
// generate golden fixtures (tests/golden/) and to pin the numpy oracle.
//
// It wires the padded transforms exactly as the reference's own test drivers
// do (tests/hybridconv.cc:46-48, hybridconvh.cc:41-43, hybridconvr.cc:38-40,
// hybridconv2.cc:43-47, hybridconvh2.cc:47-51, hybridconvr2.cc:43-47,
// hybridconv3.cc:46-52, hybridconvh3.cc:50-56, hybridconvr3.cc:46-52) and
// reports the (m,p,q,n,D,I) the reference's optimizer chose.
#include <cstring>
#include <vector>

#include "convolve.h"

using namespace fftwpp;
using namespace utils;

namespace {

enum Kind {PAD=0, CENTERED=1, HERMITIAN=2, REAL=3};
enum Mult {M_NONE=0, M_BINARY=1, M_REALBINARY=2, M_CORRELATION=3,
           M_JACOBIAN=4, M_CJACOBIAN=5};

// Physical-space Jacobian for four real inputs (ux, uy, wx, wy):
// F0 <- F0*F3 - F1*F2 (advection term u.grad(w) in 2D).
void realJacobian(Complex **F, size_t n, Indices *, size_t)
{
  double *F0=(double *) F[0];
  double *F1=(double *) F[1];
  double *F2=(double *) F[2];
  double *F3=(double *) F[3];
  for(size_t j=0; j < n; ++j)
    F0[j]=F0[j]*F3[j]-F1[j]*F2[j];
}

// Same on complex physical-space data.
void complexJacobian(Complex **F, size_t n, Indices *, size_t)
{
  Complex *F0=F[0], *F1=F[1], *F2=F[2], *F3=F[3];
  for(size_t j=0; j < n; ++j)
    F0[j]=F0[j]*F3[j]-F1[j]*F2[j];
}

multiplier *pick(int mult)
{
  switch(mult) {
    case M_BINARY: return multBinary;
    case M_REALBINARY: return realMultBinary;
    case M_CORRELATION: return multcorrelation;
    case M_JACOBIAN: return realJacobian;
    case M_CJACOBIAN: return complexJacobian;
    default: return multNone;
  }
}

fftBase *makeFFT(int kind, size_t L, size_t M, Application& app,
                 size_t C, size_t S)
{
  switch(kind) {
    case CENTERED: return new fftPadCentered(L,M,app,C,S);
    case HERMITIAN: return new fftPadHermitian(L,M,app,C);
    case REAL: return new fftPadReal(L,M,app,C,S);
    default: return new fftPad(L,M,app,C,S);
  }
}

void report(fftBase *fft, size_t *info)
{
  if(!info) return;
  info[0]=fft->m;
  info[1]=fft->p;
  info[2]=fft->q;
  info[3]=fft->n;
  info[4]=fft->D;
  info[5]=fft->inplace;
}

// Number of stored elements along the last axis for a kind.
size_t stored(int kind, size_t L)
{
  return kind == HERMITIAN ? ceilquotient(L,2) : L;
}

} // namespace

extern "C" {

// Convolve A dense inputs (stored back to back in `data`, each of `words`
// doubles) and write the B normalised outputs over the first B inputs.
//   dim        1, 2 or 3
//   kinds[d]   0 fftPad, 1 fftPadCentered, 2 fftPadHermitian, 3 fftPadReal
//   L[d], M[d] data length and minimum padded length per dimension
//   m[d], D[d], I[d]  forced parameters (0, 0, -1 = let the optimizer choose)
//   info       6 entries per dimension: m, p, q, n, D, inplace (may be NULL)
// Layout: dense row-major; real kinds store doubles, others Complex; a
// Hermitian last axis stores ceil(L/2) values.
int ref_convolve(int dim, const int *kinds, const size_t *L, const size_t *M,
                 const size_t *m, const size_t *D, const long *I,
                 size_t A, size_t B, int mult, double *data, size_t *info,
                 int threads)
{
  if(threads > 0) fftw::maxthreads=threads;
  bool real=kinds[0] == REAL;
  size_t w=real ? 1 : 2;
  size_t N=std::max(A,B);
  multiplier *mul=pick(mult);

  if(dim == 1) {
    size_t n1=stored(kinds[0],L[0]);
    size_t words=w*n1;
    Application app(A,B,mul,fftw::maxthreads,false,m[0],D[0],I[0]);
    fftBase *fft=makeFFT(kinds[0],L[0],M[0],app,1,1);
    report(fft,info);
    double **f=doubleAlign(N,std::max(words,(size_t) 2));
    for(size_t a=0; a < A; ++a)
      memcpy(f[a],data+a*words,words*sizeof(double));
    Convolution C(fft);
    C.convolve((Complex **) f);
    for(size_t b=0; b < B; ++b)
      memcpy(data+b*words,f[b],words*sizeof(double));
    deleteAlign(f[0]); delete [] f;
    delete fft;
    return 0;
  }

  if(dim == 2) {
    size_t Lx=L[0], Ly=L[1];
    size_t ny=stored(kinds[1],Ly);
    size_t Sx=ny;
    size_t words=w*Lx*Sx;
    Application appx(A,B,multNone,fftw::maxthreads,false,m[0],D[0],I[0]);
    fftBase *fftx=makeFFT(kinds[0],Lx,M[0],appx,ny,Sx);
    Application appy(A,B,mul,appx,m[1],D[1],I[1]);
    fftBase *ffty=makeFFT(kinds[1],Ly,M[1],appy,1,1);
    report(fftx,info);
    report(ffty,info ? info+6 : NULL);
    double **f=doubleAlign(N,words);
    for(size_t a=0; a < A; ++a)
      memcpy(f[a],data+a*words,words*sizeof(double));
    Convolution2 C(fftx,ffty);
    C.convolve((Complex **) f);
    for(size_t b=0; b < B; ++b)
      memcpy(data+b*words,f[b],words*sizeof(double));
    deleteAlign(f[0]); delete [] f;
    delete ffty;
    delete fftx;
    return 0;
  }

  if(dim == 3) {
    size_t Lx=L[0], Ly=L[1], Lz=L[2];
    size_t nz=stored(kinds[2],Lz);
    size_t Sy=nz, Sx=Ly*Sy;
    size_t words=w*Lx*Sx;
    Application appx(A,B,multNone,fftw::maxthreads,false,m[0],D[0],I[0]);
    fftBase *fftx=makeFFT(kinds[0],Lx,M[0],appx,Ly*Sy,Sx);
    Application appy(A,B,multNone,appx,m[1],D[1],I[1]);
    fftBase *ffty=makeFFT(kinds[1],Ly,M[1],appy,nz,Sy);
    Application appz(A,B,mul,appy,m[2],D[2],I[2]);
    fftBase *fftz=makeFFT(kinds[2],Lz,M[2],appz,1,1);
    report(fftx,info);
    report(ffty,info ? info+6 : NULL);
    report(fftz,info ? info+12 : NULL);
    double **f=doubleAlign(N,words);
    for(size_t a=0; a < A; ++a)
      memcpy(f[a],data+a*words,words*sizeof(double));
    Convolution3 C(fftx,ffty,fftz);
    C.convolve((Complex **) f);
    for(size_t b=0; b < B; ++b)
      memcpy(data+b*words,f[b],words*sizeof(double));
    deleteAlign(f[0]); delete [] f;
    delete fftz;
    delete ffty;
    delete fftx;
    return 0;
  }
  return -1;
}

// Forward-layout probe for a 1D complex padded transform (tests/hybrid.cc
// :69-105): for every residue block r of the optimiser-chosen (or forced)
// plan, write the forward output F and the transformed index of each entry.
// out_F receives `total` Complex values, out_index `total` indices, where
// total = sum over blocks of noutputs(r); returns total (or -1 on error).
// kind: 0 fftPad, 1 fftPadCentered.  C = 1, S = 1.
long ref_forward_layout(int kind, size_t L, size_t M, size_t m, size_t D,
                        long I, const double *in, double *out_F,
                        size_t *out_index, size_t capacity, size_t *info)
{
  Application app(1,1,multNone,1,false,m,D,I);
  fftPad *fft=kind == CENTERED ?
    (fftPad *) new fftPadCentered(L,M,app,1,1) : new fftPad(L,M,app,1,1);
  report(fft,info);
  if(fft->overwrite) {delete fft; return -2;}
  Complex *f=ComplexAlign(L);
  Complex *F=ComplexAlign(fft->outputSize());
  // In-place plans take W=NULL (tests/hybrid.cc:63: ComplexAlign(0) is NULL).
  size_t wsize=fft->workSizeW();
  Complex *W0=wsize ? ComplexAlign(wsize) : NULL;
  memcpy((double *) f,in,2*L*sizeof(double));
  fft->pad(W0);
  size_t total=0;
  for(size_t r=0; r < fft->R; r += fft->increment(r)) {
    fft->forward(f,F,r,W0);
    size_t n=fft->noutputs(r);
    for(size_t k=0; k < n; ++k) {
      if(total >= capacity) {total=capacity+1; break;}
      out_F[2*total]=F[k].re;
      out_F[2*total+1]=F[k].im;
      out_index[total]=fft->index(r,k);
      ++total;
    }
  }
  if(info) {
    info[6]=fft->R;
    info[7]=fft->M;
  }
  if(W0) deleteAlign(W0);
  deleteAlign(F);
  deleteAlign(f);
  delete fft;
  return (long) total;
}

// Forward layout of a 1D fftPadHermitian (the loop of tests/hybridh.cc:
// 74-99, C = 1): for every residue r and copy d < D, the noutputs(r) real
// values of block d and their transformed indices.  out_F receives `total`
// doubles.  Returns total (or -1 on error).
long ref_forward_layout_hermitian(size_t L, size_t M, size_t m, size_t D,
                                  long I, const double *in, double *out_F,
                                  size_t *out_index, size_t capacity,
                                  size_t *info)
{
  Application app(1,1,multNone,1,false,m,D,I);
  fftPadHermitian *fft=new fftPadHermitian(L,M,app,1);
  report(fft,info);
  size_t H=ceilquotient(L,2);
  Complex *f=ComplexAlign(H);
  Complex *F=ComplexAlign(fft->outputSize());
  size_t wsize=fft->workSizeW();
  Complex *W0=wsize ? ComplexAlign(wsize) : NULL;
  memcpy((double *) f,in,2*H*sizeof(double));
  fft->pad(W0);
  size_t total=0;
  size_t stride=fft->noutputs(0);
  for(size_t r=0; r < fft->R; r += fft->increment(r)) {
    fft->forward(f,F,r,W0);
    size_t D1=r == 0 ? fft->D0 : fft->D;
    for(size_t d=0; d < D1; ++d) {
      double *Fr=(double *) (F+fft->b*d);
      for(size_t k=0; k < stride; ++k) {
        if(total >= capacity) {total=capacity+1; break;}
        out_F[total]=Fr[k];
        out_index[total]=fft->index(r,k+stride*d);
        ++total;
      }
    }
  }
  if(info) {
    info[6]=fft->R;
    info[7]=fft->M;
  }
  if(W0) deleteAlign(W0);
  deleteAlign(F);
  deleteAlign(f);
  delete fft;
  return (long) total;
}

// The reference's parameter rule (convolve.cc:403-410) for direct testing.
void ref_parameters(size_t L, size_t M, size_t m, int centered,
                    size_t *p, size_t *n, size_t *q)
{
  fftBase::parameters(L,M,m,centered != 0,*p,*n,*q);
}

size_t ref_nextfftsize(size_t m)
{
  return nextfftsize(m);
}

}
