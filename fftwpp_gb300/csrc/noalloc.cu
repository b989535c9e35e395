// noalloc.cu -- a 2D centred-Hermitian FP64 convolution that allocates
// nothing: fgb_hconv2d_convolve_noalloc (include/fftwpp_gb300.h).
//
// Who needs it: callers that cannot call cudaMalloc -- for instance a host
// application whose memory manager takes all device memory up front and
// hands out pieces from its own pool (a cudaMalloc would fail or fragment
// that pool), or a latency-critical loop in which cudaMalloc/cudaFree would
// synchronise the device.  The regular plan-based entry points allocate a
// staging buffer and twiddle tables per plan; this one instead uses one
// file-scope device array, FGB_NOALLOC_SCRATCH_BYTES large, that every GPU
// which loads the library holds until the process exits.
//
// Contract:
//  * the caller passes device pointers to the two inputs and the output;
//  * the scratch array is shared by every call on a device and keeps the
//    last call's contents; each call writes every scratch word it later
//    reads (staging rows and twiddle tables), so nothing needs to start at
//    zero;
//  * calls whose work overlaps on the GPU (different streams, or host
//    threads without ordering) race on the scratch array and must be
//    serialised by the caller;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (host code cannot use the array's name as a device
//    address); make that first call before any stream capture.  The address
//    is kept for the life of the process: after cudaDeviceReset the module
//    is loaded again, possibly elsewhere, so an application that resets a
//    device must not call this entry point on it again;
//  * sizes whose staging does not fit in the array are rejected with an
//    error before anything is launched.
//
// It reuses the engine's kernels unchanged (outerFwdKernel, hermRowKernel,
// outerBwdKernel) with explicit padding on both axes.
#include "engine.h"
#include "kernels.cuh"

#include <mutex>
#include <string>

#define FGB_NOALLOC_SCRATCH_BYTES (32u*1024u*1024u)
#define FGB_NOALLOC_MAX_DEVICES 64

namespace {

static __device__ __align__(256) unsigned char noallocScratch[FGB_NOALLOC_SCRATCH_BYTES];

std::mutex scratchMutex;
void *scratchAddr[FGB_NOALLOC_MAX_DEVICES];

// Device address of noallocScratch on the current device (looked up once
// per device).
cudaError_t scratchPointer(void **ptr)
{
  int dev=0;
  cudaError_t e=cudaGetDevice(&dev);
  if(e != cudaSuccess) return e;
  if(dev < 0 || dev >= FGB_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(scratchMutex);
  if(!scratchAddr[dev]) {
    void *p=NULL;
    e=cudaGetSymbolAddress(&p,noallocScratch);
    if(e != cudaSuccess) return e;
    scratchAddr[dev]=p;
  }
  *ptr=scratchAddr[dev];
  return cudaSuccess;
}

// W_n^t = exp(2 pi i t/n), t < n, written into the scratch array.
__global__ void fillTwiddles(double2 *tw, int n)
{
  int t=blockIdx.x*blockDim.x+threadIdx.x;
  if(t >= n) return;
  double s, c;
  sincospi(2.0*(double) t/(double) n,&s,&c);
  tw[t]=make_double2(c,s);
}

long evenSmoothLen(long M)
{
  long N=M < 2 ? 2 : M;
  if(N % 2) ++N;
  while(!fgb::smooth(N/2)) N += 2;
  return N;
}

fgb::FFTPlanDev radixPlan(long n, const void *tw)
{
  fgb::FFTPlanDev p;
  p.n=(int) n;
  p.nst=0;
  long r=n;
  while(r % 8 == 0) {p.radix[p.nst++]=8; r /= 8;}
  if(r % 4 == 0) {p.radix[p.nst++]=4; r /= 4;}
  if(r % 2 == 0) {p.radix[p.nst++]=2; r /= 2;}
  while(r % 7 == 0) {p.radix[p.nst++]=7; r /= 7;}
  while(r % 5 == 0) {p.radix[p.nst++]=5; r /= 5;}
  while(r % 3 == 0) {p.radix[p.nst++]=3; r /= 3;}
  p.tw=tw;
  return p;
}

size_t align256(size_t b) {return (b+255)/256*256;}

int fail(const std::string& what)
{
  fgb::setLastError("fgb_hconv2d_convolve_noalloc: "+what);
  return -1;
}

} // namespace

extern "C" int fgb_hconv2d_convolve_noalloc(const void *f, const void *g,
                                            void *h, size_t Lx, size_t Ly,
                                            void *stream)
{
  using namespace fgb;
  typedef cplx<double> Cx;
  if(!f || !g || !h || Lx < 1 || Ly < 1) return fail("bad arguments");
  if(((size_t) f | (size_t) g | (size_t) h) % 16)
    return fail("arrays must be 16-byte aligned (complex128 elements)");
  const long Hy=(long) ceilquotient(Ly,2);
  // Default padding of the reference's hconv2d (HybridConvolution.h:94-95).
  const long Mx=3*(long) ceilquotient(Lx,2)-2*(long) (Lx % 2);
  const long My=3*Hy-2*(long) (Ly % 2);
  const long Nx=(long) nextfftsize(std::max<long>(Mx,(long) Lx));
  const long Ny=evenSmoothLen(std::max<long>(My,(long) Ly));
  const long Nyh=Ny/2;

  // Scratch layout: 2 staging arrays [Nx][Hy], then the three tables
  // W_Nx (x transform), W_Ny (Hermitian packing), W_{Ny/2} (row FFT).
  const size_t stageBytes=sizeof(Cx)*(size_t) Nx*(size_t) Hy;
  const size_t twx=align256(2*stageBytes);
  const size_t twy=twx+align256(sizeof(double2)*(size_t) Nx);
  const size_t twyh=twy+align256(sizeof(double2)*(size_t) Ny);
  const size_t need=twyh+align256(sizeof(double2)*(size_t) Nyh);
  if(need > FGB_NOALLOC_SCRATCH_BYTES)
    return fail("Lx="+std::to_string(Lx)+", Ly="+std::to_string(Ly)+
                " needs "+std::to_string(need)+" scratch bytes; the maximum "
                "is "+std::to_string(FGB_NOALLOC_SCRATCH_BYTES));
  const size_t smx=outerBwdSmem<double>((int) Lx,(int) Nx,1);
  if(smx > 227*1024 || hermRowSmem<double>((int) Hy,(int) Nyh,2) > 227*1024)
    return fail("rows too long for shared memory");

  void *base=NULL;
  cudaError_t e=scratchPointer(&base);
  if(e != cudaSuccess) return fail(cudaGetErrorString(e));
  cudaStream_t s=(cudaStream_t) stream;
  char *sc=(char *) base;
  Cx *stage0=(Cx *) sc;
  Cx *stage1=(Cx *) (sc+stageBytes);
  double2 *tx=(double2 *) (sc+twx);
  double2 *ty=(double2 *) (sc+twy);
  double2 *tyh=(double2 *) (sc+twyh);

  fillTwiddles<<<(unsigned) ((Nx+255)/256),256,0,s>>>(tx,(int) Nx);
  fillTwiddles<<<(unsigned) ((Ny+255)/256),256,0,s>>>(ty,(int) Ny);
  fillTwiddles<<<(unsigned) ((Nyh+255)/256),256,0,s>>>(tyh,(int) Nyh);
  e=cudaGetLastError();
  if(e != cudaSuccess) return fail(cudaGetErrorString(e));

  // Column tiles: widest power of two (<= 8) that fits and gives >= 3 waves.
  auto tileFor=[&](long count, bool bwd) {
    int t=8;
    while(t > 1 && ((bwd ? outerBwdSmem<double>((int) Lx,(int) Nx,t) :
                     outerFwdSmem<double>((int) Lx,(int) Nx,t)) > 227*1024 ||
                    ceilquotient(Hy,t)*count < 3*152))
      t /= 2;
    return t;
  };

  OuterPlan<double> O{};
  O.io64=0; O.inplace=0; O.conj=0;
  O.L=(int) Lx; O.m=(int) Nx; O.q=1; O.N=(int) Nx;
  O.cshift=(int) (Lx/2);
  O.fp=radixPlan(Nx,tx);
  O.twN=tx; O.twX=NULL; O.NX=1;
  O.count=2; O.nbatch=1; O.inBatch=O.outBatch=0;
  O.inRow=Hy; O.outRow=Hy; O.C=(int) Hy; O.Ltot=(long long) Lx*Hy;
  O.scale=1.0;
  O.tile=tileFor(2,false);
  O.in[0]=(const Cx *) f; O.in[1]=(const Cx *) g;
  O.out[0]=stage0; O.out[1]=stage1;
  e=launchOuterFwd<double>(O,256,s);
  if(e != cudaSuccess) return fail(cudaGetErrorString(e));

  HermRowPlan<double> P{};
  P.io64=0;
  P.H=(int) Hy; P.N=(int) Ny; P.Nh=(int) Nyh;
  P.A=2; P.B=1; P.mult=MULT_REALBINARY; P.rpc=1;
  P.fp=radixPlan(Nyh,tyh);
  P.twN=ty;
  P.in[0]=stage0; P.in[1]=stage1; P.out[0]=stage0;
  P.rowStride=Hy; P.nrows=Nx; P.scale=1.0;
  e=launchHermRow<double>(P,256,Nx,s);
  if(e != cudaSuccess) return fail(cudaGetErrorString(e));

  O.count=1;
  O.tile=tileFor(1,true);
  O.scale=1.0/((double) Nx*(double) Ny);
  O.in[0]=stage0; O.out[0]=(Cx *) h;
  e=launchOuterBwd<double>(O,256,s);
  if(e != cudaSuccess) return fail(cudaGetErrorString(e));
  return 0;
}
