// capi.cu -- C ABI of lib_fftwpp.so: the FFTW++-compatible entry points of
// include/cfftw++.h and the device-pointer API of include/fftwpp_gb300.h.
#include "batch.h"
#include "engine.h"
#include "kernels.cuh"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <vector>

using namespace fgb;

struct fgb_pad {
  std::unique_ptr<PadTransform> t;
};

struct fgb_fft {
  std::unique_ptr<PlainFFT> t;
  bool inplaceOK;
};

struct fgb_conv {
  std::unique_ptr<Conv> conv;
  cudaStream_t stream;
  // Dot-product handles (the *_dot entry points): products summed per call;
  // 0 for a plain handle.  Sums of more than FGB_MAXA/2 products run in
  // chunks of the plan's A/2 pairs, accumulated on the device.
  size_t pairs=0;
  std::vector<void *> dotBuf;     // device: A chunk inputs, accumulator, temp
  ~fgb_conv() {for(void *p : dotBuf) cudaFree(p);}
};

namespace {

size_t maxthreads=1;

// Arithmetic of the FFTW++-compatible creators (their arrays are FP64):
// FP64 or float-float (fgb_set_drop_in_precision).
int dropInPrec=PREC_F64;

// Host allocations handed out by create_*Align: page-locked when a GPU is
// present, else posix_memalign; remembered so delete_* frees correctly.
std::mutex allocMutex;
std::map<void *,bool> allocPinned;

void *alignedAlloc(size_t bytes)
{
  if(bytes == 0) bytes=16;
  void *p=NULL;
  bool pinned=cudaMallocHost(&p,bytes) == cudaSuccess;
  if(!pinned) {
    cudaGetLastError();
    p=NULL;
    if(posix_memalign(&p,64,bytes) != 0) return NULL;
  }
  std::lock_guard<std::mutex> lock(allocMutex);
  allocPinned[p]=pinned;
  return p;
}

void alignedFree(void *p)
{
  if(!p) return;
  bool pinned=false;
  {
    std::lock_guard<std::mutex> lock(allocMutex);
    auto it=allocPinned.find(p);
    if(it == allocPinned.end()) return;
    pinned=it->second;
    allocPinned.erase(it);
  }
  if(pinned) cudaFreeHost(p);
  else free(p);
}

void report(const char *where, const std::string& what)
{
  setLastError(what);
  fprintf(stderr,"fftwpp_gb300: %s: %s\n",where,what.c_str());
}

// Every kernel moves whole elements with vector accesses (16-byte for
// complex FP64): a misaligned array would fault the GPU, so it is refused.
bool aligned(const void *p, size_t a) {return (size_t) p % a == 0;}

bool alignedAll(const void *const *p, int n, size_t a)
{
  for(int i=0; i < n; ++i) if(!aligned(p[i],a)) return false;
  return true;
}

fgb_conv *make(int dim, const int *kinds, const long *L, const long *M,
               const long *m, int A, int B, int mult, int prec, long batch,
               const char *where)
{
  try {
    std::unique_ptr<fgb_conv> c(new fgb_conv);
    c->conv.reset(Conv::create(dim,kinds,L,M,m,A,B,mult,prec,batch));
    if(cudaStreamCreateWithFlags(&c->stream,cudaStreamNonBlocking) !=
       cudaSuccess) {
      cudaGetLastError();
      report(where,"cannot create a CUDA stream");
      return NULL;
    }
    return c.release();
  } catch(std::exception& e) {
    report(where,e.what());
    return NULL;
  }
}

void destroy(fgb_conv *c)
{
  if(!c) return;
  cudaStreamDestroy(c->stream);
  delete c;
}

int convolveHost(fgb_conv *c, void *a, void *b, const char *where)
{
  if(!c) {report(where,"null handle"); return -1;}
  void *in[2]={a,b};
  cudaError_t e=c->conv->runHost(in,in,c->stream);
  if(e != cudaSuccess) {
    report(where,cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

__global__ void accumulateKernel(double *acc, const double *t, size_t n)
{
  for(size_t i=blockIdx.x*(size_t) blockDim.x+threadIdx.x; i < n;
      i += (size_t) gridDim.x*blockDim.x)
    acc[i] += t[i];
}

// A handle summing `pairs` binary products (realdot: lane-wise on doubles,
// for Hermitian data).  The old FFTW++ C interface declares these entry
// points without defining them (wrappers/cfftw++.h:30-47, 53-71, 77-99,
// 104-129, 136-153, 161-188); the sum of products is the convolution of
// the dot product, h = sum_k a_k * b_k.
long defaultM(int kind, long L);

fgb_conv *makeDot(int dim, const int *kinds, const long *L, size_t pairs,
                  bool hermitian, const char *where)
{
  if(pairs < 1) {report(where,"the number of products must be positive");
    return NULL;}
  long Ms[3];
  for(int d=0; d < dim; ++d) Ms[d]=defaultM(kinds[d],L[d]);
  int K=(int) std::min<size_t>(pairs,FGB_MAXA/2);
  fgb_conv *c=make(dim,kinds,L,Ms,NULL,2*K,1,
                   hermitian ? MULT_REALDOT : MULT_DOT,dropInPrec,1,where);
  if(c) c->pairs=pairs;
  return c;
}

// a[k], b[k] (k < pairs): host arrays of the stored layout; the sum of the
// pairs' convolutions overwrites a[0].
int convolveDot(fgb_conv *c, void *const *a, void *const *b,
                const char *where)
{
  if(!c) {report(where,"null handle"); return -1;}
  if(c->pairs == 0) return convolveHost(c,a[0],b[0],where);
  Conv& C=*c->conv;
  const int K=C.info().A/2;
  const size_t bytes=C.elements()*C.elemBytes();
  cudaStream_t s=c->stream;
  cudaError_t e=cudaSuccess;
  if(c->dotBuf.empty()) {
    c->dotBuf.assign(2*K+2,NULL);
    for(void *&p : c->dotBuf)
      if(e == cudaSuccess) e=devAlloc((void **) &p,bytes);
    if(e != cudaSuccess) {
      for(void *&p : c->dotBuf) {if(p) cudaFree(p); p=NULL;}
      c->dotBuf.clear();
      report(where,cudaGetErrorString(e));
      return -2;
    }
  }
  void **in=c->dotBuf.data();
  void *acc=c->dotBuf[2*K], *tmp=c->dotBuf[2*K+1];
  for(size_t c0=0; c0 < c->pairs && e == cudaSuccess; c0 += K) {
    for(int k=0; k < K && e == cudaSuccess; ++k) {
      if(c0+k < c->pairs) {
        e=cudaMemcpyAsync(in[k],a[c0+k],bytes,cudaMemcpyHostToDevice,s);
        if(e == cudaSuccess)
          e=cudaMemcpyAsync(in[K+k],b[c0+k],bytes,cudaMemcpyHostToDevice,s);
      } else {        // a short last chunk: zero pairs add nothing
        e=cudaMemsetAsync(in[k],0,bytes,s);
        if(e == cudaSuccess) e=cudaMemsetAsync(in[K+k],0,bytes,s);
      }
    }
    if(e != cudaSuccess) break;
    void *out[1]={c0 == 0 ? acc : tmp};
    e=C.run(in,out,s);
    if(e == cudaSuccess && c0 > 0) {
      size_t n=bytes/sizeof(double);
      unsigned grid=(unsigned) std::min<size_t>((n+255)/256,4096);
      accumulateKernel<<<grid,256,0,s>>>((double *) acc,(const double *) tmp,
                                         n);
      e=cudaGetLastError();
    }
  }
  if(e == cudaSuccess)
    e=cudaMemcpyAsync(a[0],acc,bytes,cudaMemcpyDeviceToHost,s);
  if(e == cudaSuccess) e=cudaStreamSynchronize(s);
  if(e != cudaSuccess) {
    report(where,cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

// *_dotf: the pairs' arrays back to back in one flat array each.
int convolveDotFlat(fgb_conv *c, void *a, void *b, const char *where)
{
  if(!c) {report(where,"null handle"); return -1;}
  size_t P=c->pairs ? c->pairs : 1;
  size_t bytes=c->conv->elements()*c->conv->elemBytes();
  std::vector<void *> pa(P), pb(P);
  for(size_t k=0; k < P; ++k) {
    pa[k]=(char *) a+k*bytes;
    pb[k]=(char *) b+k*bytes;
  }
  return convolveDot(c,pa.data(),pb.data(),where);
}

long defaultM(int kind, long L)
{
  if(kind == KIND_CENTERED || kind == KIND_HERMITIAN)
    return 3*(long) ceilquotient(L,2)-2*(L % 2);
  return 2*L-1;
}

// Host restatement of HermitianSymmetrizeX/XY for interleaved complex data
// (convolve.h:1175-1258); these prepare host inputs before a convolve call.
void symX(size_t Hx, size_t Hy, size_t x0, double *f, size_t Sx)
{
  double *F=f+2*x0*Sx;
  for(size_t i=1; i < Hx; ++i) {
    F[-2*(long) (i*Sx)]=F[2*i*Sx];
    F[-2*(long) (i*Sx)+1]=-F[2*i*Sx+1];
  }
  F[1]=0.0;
  if(x0 == Hx)
    for(size_t j=0; j < 2*Hy; ++j) f[j]=0.0;
}

void symXY(size_t Hx, size_t Hy, size_t Hz, size_t x0, size_t y0, double *f)
{
  size_t Ly=y0+Hy;
  size_t Sy=Hz, Sx=Ly*Hz;
  size_t origin=x0*Sx+y0*Sy;
  double *F=f+2*origin;
  for(size_t i=1; i < Hx; ++i) {
    F[-2*(long) (i*Sx)]=F[2*i*Sx];
    F[-2*(long) (i*Sx)+1]=-F[2*i*Sx+1];
  }
  F[1]=0.0;
  for(long i=-(long) Hx+1; i < (long) Hx; ++i) {
    long mm=(long) origin-i*(long) Sx;
    long pp=(long) origin+i*(long) Sx;
    for(size_t j=1; j < Hy; ++j) {
      long dst=mm-(long) (j*Sy), src=pp+(long) (j*Sy);
      f[2*dst]=f[2*src];
      f[2*dst+1]=-f[2*src+1];
    }
  }
  if(x0 == Hx)
    for(size_t j=0; j < Ly; ++j)
      for(size_t k=0; k < Hz; ++k) f[2*(Sy*j+k)]=f[2*(Sy*j+k)+1]=0.0;
  if(y0 == Hy) {
    size_t Lx=x0+Hx;
    for(size_t i=0; i < Lx; ++i)
      for(size_t k=0; k < Hz; ++k) f[2*(Sx*i+k)]=f[2*(Sx*i+k)+1]=0.0;
  }
}

template<typename T>
__global__ void symXKernel(size_t Hx, size_t Hy, size_t x0, cplx<T> *f)
{
  // One thread per mirrored row i; row 0 of the Nyquist case is zeroed by
  // a separate grid-stride loop below.
  size_t i=blockIdx.x*(size_t) blockDim.x+threadIdx.x;
  cplx<T> *F=f+x0*Hy;
  if(i >= 1 && i < Hx) {
    cplx<T> v=F[i*Hy];
    F[-(long) (i*Hy)]=mk(v.x,-v.y);
  }
  if(i == 0) F[0].y=(T) 0;
}

template<typename T>
__global__ void zeroRowKernel(size_t n, cplx<T> *f)
{
  size_t i=blockIdx.x*(size_t) blockDim.x+threadIdx.x;
  if(i < n) f[i]=mk((T) 0,(T) 0);
}

// Issue-rate probes for the compute roofline: eight independent FMA chains
// per thread.  The final sum is stored only if impossible, so the chains are
// kept without writing anything.
__global__ void dfmaProbe(double *sink, int iters, double b, double c)
{
  double a[8];
  for(int k=0; k < 8; ++k) a[k]=(threadIdx.x+k)*1e-9;
  for(int i=0; i < iters; ++i)
#pragma unroll
    for(int k=0; k < 8; ++k) a[k]=fma(a[k],b,c);
  double s=0;
  for(int k=0; k < 8; ++k) s += a[k];
  if(s == -1.0) sink[0]=s;
}

__global__ void ffmaProbe(float *sink, int iters, float b, float c)
{
  float a[8];
  for(int k=0; k < 8; ++k) a[k]=(threadIdx.x+k)*1e-6f;
  for(int i=0; i < iters; ++i)
#pragma unroll
    for(int k=0; k < 8; ++k) a[k]=fmaf(a[k],b,c);
  float s=0;
  for(int k=0; k < 8; ++k) s += a[k];
  if(s == -1.0f) sink[0]=s;
}

// f[i][j] *= (j == 0 ? s0 : s1) on a rows x cols complex array.
template<typename T>
__global__ void scaleColumnsKernel(size_t rows, size_t cols, T s0, T s1,
                                   cplx<T> *f)
{
  size_t n=rows*cols;
  for(size_t i=blockIdx.x*(size_t) blockDim.x+threadIdx.x; i < n;
      i += (size_t) gridDim.x*blockDim.x) {
    T s=i % cols == 0 ? s0 : s1;
    f[i]=f[i]*s;
  }
}

} // namespace

extern "C" {

// ---------------------------------------------------------------------------
// FFTW++-compatible ABI (wrappers/cfftw++.cc).

double *create_doubleAlign(size_t n)
{
  return (double *) alignedAlloc(n*sizeof(double));
}

void delete_doubleAlign(double *p) {alignedFree(p);}

void *create_complexAlign(size_t n)
{
  return alignedAlloc(n*2*sizeof(double));
}

void delete_complexAlign(void *p) {alignedFree(p);}

size_t get_fftwpp_maxthreads(void) {return maxthreads;}
void set_fftwpp_maxthreads(size_t n) {maxthreads=n;}

void *fftwpp_create_conv1d(size_t L)
{
  int k[]={KIND_PAD};
  long Ls[]={(long) L}, Ms[]={defaultM(KIND_PAD,L)};
  return make(1,k,Ls,Ms,NULL,2,1,MULT_BINARY,dropInPrec,1,"fftwpp_create_conv1d");
}
void fftwpp_conv1d_delete(void *c) {destroy((fgb_conv *) c);}
void fftwpp_conv1d_convolve(void *c, void *a, void *b)
{
  convolveHost((fgb_conv *) c,a,b,"fftwpp_conv1d_convolve");
}

void *fftwpp_create_hconv1d(size_t L)
{
  int k[]={KIND_HERMITIAN};
  long Ls[]={(long) L}, Ms[]={defaultM(KIND_HERMITIAN,L)};
  return make(1,k,Ls,Ms,NULL,2,1,MULT_REALBINARY,dropInPrec,1,
              "fftwpp_create_hconv1d");
}
void fftwpp_hconv1d_delete(void *c) {destroy((fgb_conv *) c);}
void fftwpp_HermitianSymmetrize(double *f) {f[1]=0.0;}
void fftwpp_hconv1d_convolve(void *c, void *a, void *b)
{
  convolveHost((fgb_conv *) c,a,b,"fftwpp_hconv1d_convolve");
}

void *fftwpp_create_conv2d(size_t Lx, size_t Ly)
{
  int k[]={KIND_PAD,KIND_PAD};
  long Ls[]={(long) Lx,(long) Ly};
  long Ms[]={defaultM(KIND_PAD,Lx),defaultM(KIND_PAD,Ly)};
  return make(2,k,Ls,Ms,NULL,2,1,MULT_BINARY,dropInPrec,1,"fftwpp_create_conv2d");
}
void fftwpp_conv2d_delete(void *c) {destroy((fgb_conv *) c);}
void fftwpp_HermitianSymmetrizeX(size_t Hx, size_t Hy, size_t x0, double *f)
{
  symX(Hx,Hy,x0,f,Hy);
}
void fftwpp_conv2d_convolve(void *c, void *a, void *b)
{
  convolveHost((fgb_conv *) c,a,b,"fftwpp_conv2d_convolve");
}

void *fftwpp_create_hconv2d(size_t Lx, size_t Ly)
{
  int k[]={KIND_CENTERED,KIND_HERMITIAN};
  long Ls[]={(long) Lx,(long) Ly};
  long Ms[]={defaultM(KIND_CENTERED,Lx),defaultM(KIND_HERMITIAN,Ly)};
  return make(2,k,Ls,Ms,NULL,2,1,MULT_REALBINARY,dropInPrec,1,
              "fftwpp_create_hconv2d");
}
void fftwpp_hconv2d_delete(void *c) {destroy((fgb_conv *) c);}
void fftwpp_hconv2d_convolve(void *c, void *a, void *b)
{
  convolveHost((fgb_conv *) c,a,b,"fftwpp_hconv2d_convolve");
}

void *fftwpp_create_conv3d(size_t Lx, size_t Ly, size_t Lz)
{
  int k[]={KIND_PAD,KIND_PAD,KIND_PAD};
  long Ls[]={(long) Lx,(long) Ly,(long) Lz};
  long Ms[]={defaultM(KIND_PAD,Lx),defaultM(KIND_PAD,Ly),defaultM(KIND_PAD,Lz)};
  return make(3,k,Ls,Ms,NULL,2,1,MULT_BINARY,dropInPrec,1,"fftwpp_create_conv3d");
}
void fftwpp_conv3d_delete(void *c) {destroy((fgb_conv *) c);}
void fftwpp_HermitianSymmetrizeXY(size_t Hx, size_t Hy, size_t Hz, size_t x0,
                                  size_t y0, double *f)
{
  symXY(Hx,Hy,Hz,x0,y0,f);
}
void fftwpp_conv3d_convolve(void *c, void *a, void *b)
{
  convolveHost((fgb_conv *) c,a,b,"fftwpp_conv3d_convolve");
}

void *fftwpp_create_hconv3d(size_t Lx, size_t Ly, size_t Lz)
{
  int k[]={KIND_CENTERED,KIND_CENTERED,KIND_HERMITIAN};
  long Ls[]={(long) Lx,(long) Ly,(long) Lz};
  long Ms[]={defaultM(KIND_CENTERED,Lx),defaultM(KIND_CENTERED,Ly),
             defaultM(KIND_HERMITIAN,Lz)};
  return make(3,k,Ls,Ms,NULL,2,1,MULT_REALBINARY,dropInPrec,1,
              "fftwpp_create_hconv3d");
}
void fftwpp_hconv3d_delete(void *c) {destroy((fgb_conv *) c);}
void fftwpp_hconv3d_convolve(void *c, void *a, void *b)
{
  convolveHost((fgb_conv *) c,a,b,"fftwpp_hconv3d_convolve");
}

// ---------------------------------------------------------------------------
// Dot-product and work-array forms declared by the old FFTW++ C interface
// (wrappers/cfftw++.h).  m: data length per axis as in the plain forms;
// M: number of products summed.  The work arrays u, v, w were host scratch
// of the CPU implementation; device scratch is allocated internally, so
// they are accepted and not used.

double *create_doublealign(size_t n) {return create_doubleAlign(n);}

void *fftwpp_create_conv1d_dot(size_t m, size_t M)
{
  int k[]={KIND_PAD};
  long Ls[]={(long) m};
  return makeDot(1,k,Ls,M,false,"fftwpp_create_conv1d_dot");
}
void *fftwpp_create_conv1d_work(size_t m, void *, void *)
{
  return fftwpp_create_conv1d(m);
}
void *fftwpp_create_conv1d_work_dot(size_t m, void *, void *, size_t M)
{
  return fftwpp_create_conv1d_dot(m,M);
}
void fftwpp_conv1d_convolve_dot(void *c, void **a, void **b)
{
  convolveDot((fgb_conv *) c,a,b,"fftwpp_conv1d_convolve_dot");
}
void fftwpp_conv1d_convolve_dotf(void *c, void *a, void *b)
{
  convolveDotFlat((fgb_conv *) c,a,b,"fftwpp_conv1d_convolve_dotf");
}

void *fftwpp_create_hconv1d_dot(size_t m, size_t M)
{
  int k[]={KIND_HERMITIAN};
  long Ls[]={(long) m};
  return makeDot(1,k,Ls,M,true,"fftwpp_create_hconv1d_dot");
}
void *fftwpp_create_hconv1d_work(size_t m, void *, void *, void *)
{
  return fftwpp_create_hconv1d(m);
}
void *fftwpp_create_hconv1d_work_dot(size_t m, void *, void *, void *,
                                     size_t M)
{
  return fftwpp_create_hconv1d_dot(m,M);
}
void fftwpp_hconv1d_convolve_dot(void *c, void **a, void **b)
{
  convolveDot((fgb_conv *) c,a,b,"fftwpp_hconv1d_convolve_dot");
}
void fftwpp_hconv1d_convolve_dotf(void *c, void *a, void *b)
{
  convolveDotFlat((fgb_conv *) c,a,b,"fftwpp_hconv1d_convolve_dotf");
}

void *fftwpp_create_conv2d_dot(size_t mx, size_t my, size_t M)
{
  int k[]={KIND_PAD,KIND_PAD};
  long Ls[]={(long) mx,(long) my};
  return makeDot(2,k,Ls,M,false,"fftwpp_create_conv2d_dot");
}
void *fftwpp_create_conv2d_work(size_t mx, size_t my, void *, void *, void *,
                                void *)
{
  return fftwpp_create_conv2d(mx,my);
}
void *fftwpp_create_conv2d_work_dot(size_t mx, size_t my, void *, void *,
                                    void *, void *, size_t M)
{
  return fftwpp_create_conv2d_dot(mx,my,M);
}
void fftwpp_conv2d_convolve_dot(void *c, void **a, void **b)
{
  convolveDot((fgb_conv *) c,a,b,"fftwpp_conv2d_convolve_dot");
}
void fftwpp_conv2d_convolve_dotf(void *c, void *a, void *b)
{
  convolveDotFlat((fgb_conv *) c,a,b,"fftwpp_conv2d_convolve_dotf");
}

void *fftwpp_create_hconv2d_dot(size_t mx, size_t my, size_t M)
{
  int k[]={KIND_CENTERED,KIND_HERMITIAN};
  long Ls[]={(long) mx,(long) my};
  return makeDot(2,k,Ls,M,true,"fftwpp_create_hconv2d_dot");
}
void *fftwpp_create_hconv2d_work(size_t mx, size_t my, void *, void *, void *,
                                 void *, void *)
{
  return fftwpp_create_hconv2d(mx,my);
}
void *fftwpp_create_hconv2d_work_dot(size_t mx, size_t my, void *, void *,
                                     void *, void *, void *, size_t M)
{
  return fftwpp_create_hconv2d_dot(mx,my,M);
}
void fftwpp_hconv2d_convolve_dot(void *c, void **a, void **b)
{
  convolveDot((fgb_conv *) c,a,b,"fftwpp_hconv2d_convolve_dot");
}
void fftwpp_hconv2d_convolve_dotf(void *c, void *a, void *b)
{
  convolveDotFlat((fgb_conv *) c,a,b,"fftwpp_hconv2d_convolve_dotf");
}

void *fftwpp_create_conv3d_dot(size_t mx, size_t my, size_t mz, size_t M)
{
  int k[]={KIND_PAD,KIND_PAD,KIND_PAD};
  long Ls[]={(long) mx,(long) my,(long) mz};
  return makeDot(3,k,Ls,M,false,"fftwpp_create_conv3d_dot");
}
void *fftwpp_create_conv3d_work(size_t mx, size_t my, size_t mz, void *,
                                void *, void *, void *, void *, void *)
{
  return fftwpp_create_conv3d(mx,my,mz);
}
void fftwpp_conv3d_convolve_dot(void *c, void **a, void **b)
{
  convolveDot((fgb_conv *) c,a,b,"fftwpp_conv3d_convolve_dot");
}
void fftwpp_conv3d_convolve_dotf(void *c, void *a, void *b)
{
  convolveDotFlat((fgb_conv *) c,a,b,"fftwpp_conv3d_convolve_dotf");
}

void *fftwpp_create_hconv3d_dot(size_t mx, size_t my, size_t mz, size_t M)
{
  int k[]={KIND_CENTERED,KIND_CENTERED,KIND_HERMITIAN};
  long Ls[]={(long) mx,(long) my,(long) mz};
  return makeDot(3,k,Ls,M,true,"fftwpp_create_hconv3d_dot");
}
void *fftwpp_create_hconv3d_work(size_t mx, size_t my, size_t mz, void *,
                                 void *, void *, void *, void *, void *,
                                 void *)
{
  return fftwpp_create_hconv3d(mx,my,mz);
}
void *fftwpp_create_hconv3d_work_dot(size_t mx, size_t my, size_t mz, void *,
                                     void *, void *, void *, void *, void *,
                                     void *, size_t M)
{
  return fftwpp_create_hconv3d_dot(mx,my,mz,M);
}
void fftwpp_hconv3d_convolve_dot(void *c, void **a, void **b)
{
  convolveDot((fgb_conv *) c,a,b,"fftwpp_hconv3d_convolve_dot");
}

// ---------------------------------------------------------------------------
// Device-pointer API (include/fftwpp_gb300.h).

fgb_conv *fgb_create(int dim, const int *kinds, const size_t *L,
                     const size_t *M, const size_t *m, int A, int B, int mult,
                     int precision, size_t batch)
{
  if(dim < 1 || dim > 3 || !kinds || !L || !M) {
    report("fgb_create","bad arguments");
    return NULL;
  }
  long Ls[3], Ms[3], ms[3];
  for(int d=0; d < dim; ++d) {
    Ls[d]=(long) L[d];
    Ms[d]=(long) M[d];
    ms[d]=m ? (long) m[d] : 0;
  }
  return make(dim,kinds,Ls,Ms,ms,A,B,mult,precision,(long) batch,"fgb_create");
}

int fgb_convolve_device(fgb_conv *c, void *const *in, void *const *out,
                        void *stream)
{
  if(!c || !in || !out) {report("fgb_convolve_device","bad arguments"); return -1;}
  const ConvInfo& I=c->conv->info();
  if(!alignedAll(in,I.A,c->conv->elemBytes()) ||
     !alignedAll(out,I.B,c->conv->elemBytes())) {
    report("fgb_convolve_device","arrays must be aligned to their element "
           "size ("+std::to_string(c->conv->elemBytes())+" bytes)");
    return -1;
  }
  if(I.mult == MULT_USER) {
    report("fgb_convolve_device","this plan multiplies with a caller's "
           "device functor: convolve through fgb::convolveWith "
           "(fftwpp_gb300_mult.cuh)");
    return -1;
  }
  cudaError_t e=c->conv->run(in,out,(cudaStream_t) stream);
  if(e != cudaSuccess) {
    report("fgb_convolve_device",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

int fgb_convolve_host(fgb_conv *c, void *const *in, void *const *out)
{
  if(!c || !in || !out) {report("fgb_convolve_host","bad arguments"); return -1;}
  if(c->conv->info().mult == MULT_USER) {
    report("fgb_convolve_host","this plan multiplies with a caller's "
           "device functor: convolve through fgb::convolveHostWith "
           "(fftwpp_gb300_mult.cuh)");
    return -1;
  }
  cudaError_t e=c->conv->runHost(in,out,c->stream);
  if(e != cudaSuccess) {
    report("fgb_convolve_host",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

void fgb_set_ff_range_guard(int on) {Conv::setRangeGuard(on != 0);}

int fgb_set_strides(fgb_conv *c, const size_t *stride)
{
  if(!c) {report("fgb_set_strides","bad arguments"); return -1;}
  try {
    if(!stride) c->conv->setStrides(NULL);
    else {
      long S[3]={0,0,0};
      for(int d=0; d+1 < c->conv->info().dim; ++d) S[d]=(long) stride[d];
      c->conv->setStrides(S);
    }
  } catch(std::exception& e) {
    report("fgb_set_strides",e.what());
    return -1;
  }
  return 0;
}

int fgb_convolve_device_with(fgb_conv *c, const void *launchers,
                             void *const *in, void *const *out, void *stream)
{
  const char *where="fgb_convolve_device_with";
  if(!c || !launchers || !in || !out) {report(where,"bad arguments"); return -1;}
  const ConvInfo& I=c->conv->info();
  if(!alignedAll(in,I.A,c->conv->elemBytes()) ||
     !alignedAll(out,I.B,c->conv->elemBytes())) {
    report(where,"arrays must be aligned to their element size ("+
           std::to_string(c->conv->elemBytes())+" bytes)");
    return -1;
  }
  setLastError("");
  cudaError_t e=c->conv->runWith((const RowLaunchers *) launchers,in,out,
                                 (cudaStream_t) stream);
  if(e != cudaSuccess) {
    std::string why=lastError();
    report(where,why.empty() ? cudaGetErrorString(e) : why);
    return e == cudaErrorInvalidValue ? -1 : -2;
  }
  return 0;
}

int fgb_convolve_host_with(fgb_conv *c, const void *launchers,
                           void *const *in, void *const *out)
{
  const char *where="fgb_convolve_host_with";
  if(!c || !launchers || !in || !out) {report(where,"bad arguments"); return -1;}
  setLastError("");
  cudaError_t e=c->conv->runHostWith((const RowLaunchers *) launchers,in,out,
                                     c->stream);
  if(e != cudaSuccess) {
    std::string why=lastError();
    report(where,why.empty() ? cudaGetErrorString(e) : why);
    return e == cudaErrorInvalidValue ? -1 : -2;
  }
  return 0;
}

int fgb_info(const fgb_conv *c, long *info)
{
  if(!c || !info) return -1;
  const ConvInfo& I=c->conv->info();
  for(int k=0; k < 32; ++k) info[k]=0;
  for(int d=0; d < I.dim; ++d) {
    const AxisPlan& a=I.axis[d];
    long *o=info+8*d;
    o[0]=a.m; o[1]=a.p; o[2]=a.q; o[3]=a.N; o[4]=a.stored; o[5]=a.cshift;
    o[6]=a.tile; o[7]=a.rows;
  }
  info[24]=c->conv->launches();
  info[25]=(long) c->conv->stagingBytes();
  info[26]=I.longRow ? 1 : 0;
  for(int d=0; d < I.dim; ++d) info[27+d]=I.axis[d].tileB;
  info[30]=I.axis[I.dim-1].rpc;
  info[31]=I.axis[I.dim-1].thr;
  return 0;
}

void fgb_set_autotune(int on) {Conv::setAutotune(on != 0);}

size_t fgb_wisdom_export(char *buf, size_t size)
{
  const std::string t=Conv::exportWisdom();
  if(buf && size > 0) {
    const size_t n=std::min(size-1,t.size());
    std::memcpy(buf,t.data(),n);
    buf[n]=0;
  }
  return t.size();
}

int fgb_wisdom_import(const char *text)
{
  if(!text) return -1;
  const int n=Conv::importWisdom(text);
  if(n < 0) setLastError("wisdom text does not parse");
  return n;
}

void fgb_wisdom_forget(void) {Conv::forgetWisdom();}
void fgb_set_residue_search(int on) {Conv::setResidueSearch(on != 0);}

void fgb_debug_fail_allocation_after(long n) {failAllocationAfter(n);}

int fgb_set_drop_in_precision(int precision)
{
  if(precision != PREC_F64 && precision != PREC_FF) {
    report("fgb_set_drop_in_precision","the FFTW++-compatible entry points "
           "take FP64 arrays: FGB_F64 or FGB_FF");
    return -1;
  }
  dropInPrec=precision;
  return 0;
}

int fgb_get_drop_in_precision(void) {return dropInPrec;}
void fgb_set_zero_copy(int on) {Conv::setZeroCopy(on != 0);}
int fgb_host_path(const fgb_conv *c, int *inputs, int *outputs)
{
  if(!c) return -1;
  c->conv->hostPath(inputs,outputs);
  return 0;
}

void fgb_set_host_path(int inputs, int outputs)
{
  Conv::setHostPath(inputs,outputs);
}

int fgb_set_normalize(fgb_conv *c, int normalize)
{
  if(!c) return -1;
  c->conv->setNormalize(normalize != 0);
  return 0;
}

int fgb_timing(fgb_conv *c, int enable)
{
  if(!c) return -1;
  cudaError_t e=c->conv->enableTiming(enable != 0);
  if(e != cudaSuccess) {
    report("fgb_timing",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

int fgb_timing_collect(fgb_conv *c, double *ms, int n)
{
  if(!c || !ms) return -1;
  return c->conv->collect(ms,n);
}

void fgb_destroy(fgb_conv *c) {destroy(c);}

// ---------------------------------------------------------------------------
// Batched uneven 1D convolutions (include/fftwpp_gb300.h).

struct fgb_batch {
  std::unique_ptr<BatchConv> b;
};

fgb_batch *fgb_batch_create(int n, const size_t *L, const size_t *M, int A,
                            int B, int mult, int precision, int kind,
                            int tune)
{
  if(n < 1 || !L || !M) {report("fgb_batch_create","bad arguments"); return NULL;}
  try {
    std::vector<long> Ls(L,L+n), Ms(M,M+n);
    fgb_batch *h=new fgb_batch;
    h->b.reset(new BatchConv(n,Ls.data(),Ms.data(),NULL,A,B,mult,precision,
                             kind,tune != 0));
    return h;
  } catch(std::exception& e) {
    report("fgb_batch_create",e.what());
    return NULL;
  }
}

int fgb_batch_convolve_device(fgb_batch *h, void *const *in, void *const *out,
                              void *stream, int use_graph)
{
  if(!h || !in || !out) {report("fgb_batch_convolve_device","bad arguments"); return -1;}
  size_t eb=h->b->precision() == PREC_F64 ? 16 : 8;
  if(!alignedAll(in,h->b->inputs(),eb) || !alignedAll(out,h->b->outputs(),eb)) {
    report("fgb_batch_convolve_device","packed arrays must be aligned to "
           "their element size ("+std::to_string(eb)+" bytes)");
    return -1;
  }
  cudaError_t e=use_graph ? h->b->runGraph(in,out,(cudaStream_t) stream) :
    h->b->run(in,out,(cudaStream_t) stream);
  if(e != cudaSuccess) {
    report("fgb_batch_convolve_device",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

int fgb_batch_info(const fgb_batch *h, long *info)
{
  if(!h || !info) return -1;
  info[0]=h->b->tasks();
  info[1]=h->b->gridSize();
  info[2]=(long) h->b->smemBytes();
  info[3]=h->b->shortProblems();
  info[4]=h->b->longProblems();
  info[5]=h->b->totalLength();
  return 0;
}

long fgb_batch_choice(const fgb_batch *h, int i)
{
  return h ? h->b->choice(i) : 0;
}

int fgb_batch_error(fgb_batch *h)
{
  return h ? h->b->error() : -1;
}

void fgb_batch_destroy(fgb_batch *h) {delete h;}

int fgb_batch_set_spin_limit(fgb_batch *h, long long polls)
{
  if(!h || polls < 0) {report("fgb_batch_set_spin_limit","bad arguments");
    return -1;}
  h->b->setSpinLimit(polls);
  return 0;
}

int fgb_batch_block_problem(fgb_batch *h, int i, int blocked)
{
  if(!h) {report("fgb_batch_block_problem","null handle"); return -1;}
  cudaError_t e=h->b->blockProblem(i,blocked != 0);
  if(e != cudaSuccess) {
    report("fgb_batch_block_problem","problem "+std::to_string(i)+
           " is not a long problem of this batch");
    return -1;
  }
  return 0;
}

// Standalone padded transforms (engine.h, class PadTransform).
fgb_pad *fgb_pad_create(int kind, size_t L, size_t M, size_t C, size_t m,
                        int precision)
{
  try {
    fgb_pad *h=new fgb_pad;
    h->t.reset(new PadTransform(kind,(long) L,(long) M,(long) C,(long) m,
                                precision));
    return h;
  } catch(std::exception& e) {
    report("fgb_pad_create",e.what());
    return NULL;
  }
}

int fgb_pad_forward_device(fgb_pad *h, const void *f, void *F, void *stream)
{
  if(!h || !f || !F) {report("fgb_pad_forward_device","null argument");
    return -1;}
  if(!h->t->aligned(f,F)) {
    report("fgb_pad_forward_device","arrays must be aligned to their "
           "element size");
    return -1;
  }
  cudaError_t e=h->t->forward(f,F,(cudaStream_t) stream);
  if(e != cudaSuccess) {
    report("fgb_pad_forward_device",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

int fgb_pad_backward_device(fgb_pad *h, const void *F, void *f, void *stream)
{
  if(!h || !f || !F) {report("fgb_pad_backward_device","null argument");
    return -1;}
  if(!h->t->aligned(f,F)) {
    report("fgb_pad_backward_device","arrays must be aligned to their "
           "element size");
    return -1;
  }
  cudaError_t e=h->t->backward(F,f,(cudaStream_t) stream);
  if(e != cudaSuccess) {
    report("fgb_pad_backward_device",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

int fgb_pad_info(const fgb_pad *h, long *info)
{
  if(!h || !info) {report("fgb_pad_info","null argument"); return -1;}
  const AxisPlan& a=h->t->plan();
  long v[10]={a.m,a.p,a.q,a.N,a.L,h->t->columns(),a.rows,a.cshift,a.tile,
              a.tileB};
  for(int i=0; i < 10; ++i) info[i]=v[i];
  return 0;
}

size_t fgb_pad_index(const fgb_pad *h, size_t r, size_t j)
{
  if(!h) return 0;
  const AxisPlan& a=h->t->plan();
  return a.kind == KIND_REAL || a.kind == KIND_HERMITIAN ? j : a.q*j+r;
}

void fgb_pad_destroy(fgb_pad *h) {delete h;}

// Plain FFTs (engine.h, class PlainFFT).
fgb_fft *fgb_fft_create(int kind, size_t n, int sign, size_t C, size_t B,
                        size_t istride, size_t ibatch, size_t ostride,
                        size_t obatch, int precision)
{
  try {
    fgb_fft *h=new fgb_fft;
    h->t.reset(new PlainFFT(kind,(long) n,sign,(long) C,(long) B,
                            (long) istride,(long) ibatch,(long) ostride,
                            (long) obatch,precision));
    // Interleaved real transforms read and write columns of different
    // widths, so other CTAs' columns would overlap in place.
    h->inplaceOK=kind == FFT_C2C || C == 1;
    return h;
  } catch(std::exception& e) {
    report("fgb_fft_create",e.what());
    return NULL;
  }
}

int fgb_fft_execute_device(fgb_fft *h, const void *in, void *out,
                           void *stream)
{
  if(!h || !in || !out) {report("fgb_fft_execute_device","null argument");
    return -1;}
  if(!h->t->aligned(in,out)) {
    report("fgb_fft_execute_device","arrays must be aligned to their "
           "element size");
    return -1;
  }
  if(in == out && !h->inplaceOK) {
    report("fgb_fft_execute_device","interleaved real transforms must be "
           "out of place");
    return -1;
  }
  cudaError_t e=h->t->execute(in,out,(cudaStream_t) stream);
  if(e != cudaSuccess) {
    report("fgb_fft_execute_device",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

void fgb_fft_destroy(fgb_fft *h) {delete h;}

int fgb_fft_origin_shift_device(void *f, size_t nx, size_t ny, size_t nz,
                                int precision, void *stream)
{
  const char *where="fgb_fft_origin_shift_device";
  if(!f || nx < 1 || ny < 1 || nz < 1) {report(where,"bad arguments"); return -1;}
  if(precision != PREC_F64 && precision != PREC_F32) {
    report(where,"precision must be FGB_F64 or FGB_F32");
    return -1;
  }
  if(nx % 2 || (nz > 1 && ny % 2)) {
    report(where,"shifting the Fourier origin needs an even nx (and an "
           "even ny in 3D)");
    return -1;
  }
  if((size_t) f % (precision == PREC_F64 ? 8 : 4)) {
    report(where,"array must be aligned to its element size");
    return -1;
  }
  cudaError_t e=launchOriginShift(f,(long long) nx,(long long) ny,
                                  (long long) nz,precision == PREC_F64,
                                  (cudaStream_t) stream);
  if(e != cudaSuccess) {
    report(where,cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

const char *fgb_last_error(void)
{
  static thread_local std::string s;
  s=lastError();
  return s.c_str();
}

void fgb_parameters(size_t L, size_t M, size_t m, int centered,
                    size_t *p, size_t *n, size_t *q)
{
  refParameters(L,M,m,centered != 0,*p,*n,*q);
}

size_t fgb_nextfftsize(size_t m) {return nextfftsize(m);}

int fgb_batch_task_order(int nlong, const size_t *staging,
                         const int *fwdTiles, const int *rows,
                         const int *bwdTiles, int nsmall, int inputs,
                         int outputs, size_t groupBytes, int *type,
                         int *problem, int max)
{
  std::vector<LongTasks> lt;
  for(int i=0; i < nlong; ++i)
    lt.push_back({i,staging[i],fwdTiles[i],rows[i],bwdTiles[i]});
  std::vector<int> sm;
  for(int i=0; i < nsmall; ++i) sm.push_back(nlong+i);
  const std::vector<BatchTask> t=orderBatchTasks(lt,sm,inputs,outputs,
                                                 groupBytes);
  for(int k=0; k < (int) t.size() && k < max; ++k) {
    type[k]=t[k].type;
    problem[k]=t[k].prob;
  }
  return (int) t.size();
}

int fgb_fft_radices(size_t n, int precision, int inplace, int wide,
                    int *radix, int max)
{
  int r[FGB_MAXSTAGES];
  const int nst=fftRadices((long) n,precision,inplace != 0,wide != 0,r);
  if(nst < 0) {
    setLastError("transform length "+std::to_string(n)+" has no radix plan");
    return -1;
  }
  for(int s=0; s < nst && s < max; ++s) radix[s]=r[s];
  return nst;
}

// Transformed index (fftBase::index, convolve.h:297-326; fftPadReal::index,
// convolve.h:956-979).  D0 = n mod D (or D), the remainder block of the
// residue loop (convolve.cc:701-703); overwrite is not modelled.
size_t fgb_index(int kind, size_t m, size_t p, size_t q, size_t n, size_t D,
                 size_t r, size_t i)
{
  if(q == 1) return i;
  if(kind == KIND_REAL) {
    size_t s=i % m;
    size_t P=p == 2 ? 1 : p;
    r += i/(P*m);
    if(p <= 2) {
      if(r == 0) return q*i;
      if(2*r == q) return q*m-(q*2*i+r);
    } else {
      size_t u=(i/m) % p;
      if(r == 0) {
        if(2*u == p) return q*m-(q*2*s+u*n);
        return s == 0 ? u*n : q*m-(q*s-u*n);
      } else if(2*r == n)
        return q*m-(q*s+2*u*n+r);
      else
        return q*(m-s)-(u*n+r);
    }
    return q*(m-s)-r;
  }
  bool centered=kind == KIND_CENTERED || kind == KIND_HERMITIAN;
  size_t D0=n % D;
  if(D0 == 0) D0=D;
  size_t P=(p+1)/2;
  size_t s=i % m;
  size_t u;
  if(D > 1 && ((centered && p % 2 == 0) || p <= 2)) {
    u=(i/m) % P;
    size_t offset=r == 0 && i >= P*m && D0 % 2 == 1 ? 1 : 0;
    size_t incr=(i+P*m*offset)/(2*P*m);
    r += incr;
    if(i/(P*m)-2*incr+offset == 1) {
      if((!centered && p == 2) || (r > 0 && u == 0))
        s=s > 0 ? s-1 : m-1;
      if(r == 0)
        r=n/2;
      else {
        r=n-r;
        u=u > 0 ? u-1 : P-1;
      }
    }
  } else {
    u=(i/m) % p;
    r += i/(p*m);
  }
  return q*s+n*u+r;
}

int fgb_measure_fma_rate(double *dfma_per_s, double *ffma_per_s)
{
  int dev=0, nsm=0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm,cudaDevAttrMultiProcessorCount,dev);
  cudaEvent_t e0, e1;
  if(cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return -2;
  const int blocks=nsm*8, threads=256;
  const int itd=2048, itf=65536;
  float ms=0;
  double *sink=NULL;
  if(cudaMalloc(&sink,sizeof(double)) != cudaSuccess) return -2;
  dfmaProbe<<<blocks,threads>>>(sink,itd/8,0.999999,1e-7);   // warm-up
  cudaEventRecord(e0);
  dfmaProbe<<<blocks,threads>>>(sink,itd,0.999999,1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(&ms,e0,e1);
  if(dfma_per_s) *dfma_per_s=(double) blocks*threads*8.0*itd/(ms*1e-3);
  ffmaProbe<<<blocks,threads>>>((float *) sink,itf/8,0.9999f,1e-4f);
  cudaEventRecord(e0);
  ffmaProbe<<<blocks,threads>>>((float *) sink,itf,0.9999f,1e-4f);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(&ms,e0,e1);
  if(ffma_per_s) *ffma_per_s=(double) blocks*threads*8.0*itf/(ms*1e-3);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  cudaError_t e=cudaGetLastError();
  if(e != cudaSuccess) {
    report("fgb_measure_fma_rate",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

int fgb_scale_columns_device(size_t rows, size_t cols, double s0, double s1,
                             void *f, int precision, void *stream)
{
  cudaStream_t s=(cudaStream_t) stream;
  size_t n=rows*cols;
  unsigned grid=(unsigned) std::min<size_t>((n+255)/256,4096);
  if(grid == 0) return 0;
  if(precision == PREC_F64)
    scaleColumnsKernel<double><<<grid,256,0,s>>>(rows,cols,s0,s1,
                                                 (cplx<double> *) f);
  else
    scaleColumnsKernel<float><<<grid,256,0,s>>>(rows,cols,(float) s0,
                                                (float) s1,(cplx<float> *) f);
  cudaError_t e=cudaGetLastError();
  if(e != cudaSuccess) {
    report("fgb_scale_columns_device",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

int fgb_hermitian_symmetrize_x_device(size_t Hx, size_t Hy, size_t x0,
                                      void *f, int precision, void *stream)
{
  cudaStream_t s=(cudaStream_t) stream;
  unsigned grid=(unsigned) ((Hx+255)/256);
  if(precision == PREC_F64) {
    symXKernel<double><<<grid,256,0,s>>>(Hx,Hy,x0,(cplx<double> *) f);
    if(x0 == Hx)
      zeroRowKernel<double><<<(unsigned) ((Hy+255)/256),256,0,s>>>(Hy,(cplx<double> *) f);
  } else {
    symXKernel<float><<<grid,256,0,s>>>(Hx,Hy,x0,(cplx<float> *) f);
    if(x0 == Hx)
      zeroRowKernel<float><<<(unsigned) ((Hy+255)/256),256,0,s>>>(Hy,(cplx<float> *) f);
  }
  cudaError_t e=cudaGetLastError();
  if(e != cudaSuccess) {
    report("fgb_hermitian_symmetrize_x_device",cudaGetErrorString(e));
    return -2;
  }
  return 0;
}

} // extern "C"
