// fftw3_shim.cc -- clean-room DFT backend behind the FFTW3 C interface.
//
// TEST INFRASTRUCTURE ONLY (see fftw3.h).  It lets the reference's own
// convolve.cc be compiled into oracle/_ref/ on a machine without FFTW3.
//
// Algorithm (written from the DFT definition, not from FFTW):
//   * mixed-radix recursive decimation-in-time Cooley-Tukey: n = p*m with p
//     the smallest prime factor; p sub-DFTs of length m, then a radix-p
//     butterfly with twiddles w_n^{j1*k2};
//   * prime lengths above 64 use Bluestein's chirp-z identity
//     jk = (j^2 + k^2 - (k-j)^2)/2, evaluated as a circular convolution of
//     power-of-two length (Bluestein 1968); small primes use the direct sum;
//   * every twiddle exp(2*pi*i*t/n) is computed in long double from the exact
//     rational angle t/n (t reduced mod n) and then rounded to double.
// Real transforms are computed through the complex DFT of the full length:
// r2c keeps outputs 0..n/2, c2r Hermitian-extends its n/2+1 inputs and keeps
// the real part (which discards Im X[0] and, for even n, Im X[n/2], exactly as
// a Hermitian c2r must).
#include "fftw3.h"

#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

typedef std::complex<double> cplx;

namespace {

// ---------------------------------------------------------------------------
// Twiddle tables, cached per (n, sign); guarded for concurrent planning.
struct Roots {
  std::vector<cplx> w;   // w[t] = exp(sign*2*pi*i*t/n), t < n
};

std::mutex rootsMutex;
std::map<std::pair<long,int>,std::shared_ptr<Roots>> rootsCache;

std::shared_ptr<Roots> roots(long n, int sign)
{
  std::lock_guard<std::mutex> lock(rootsMutex);
  auto key=std::make_pair(n,sign);
  auto it=rootsCache.find(key);
  if(it != rootsCache.end()) return it->second;
  auto r=std::make_shared<Roots>();
  r->w.resize(n);
  const long double twopi=6.283185307179586476925286766559005768L;
  for(long t=0; t < n; ++t) {
    long double a=twopi*(long double) t/(long double) n;
    r->w[t]=cplx((double) cosl(a),(double) (sign*sinl(a)));
  }
  rootsCache[key]=r;
  return r;
}

long smallestFactor(long n)
{
  if(n % 2 == 0) return 2;
  for(long f=3; f*f <= n; f += 2)
    if(n % f == 0) return f;
  return n;
}

long ceilpow2(long n)
{
  long p=1;
  while(p < n) p <<= 1;
  return p;
}

void dft(const cplx *in, long istride, cplx *out, long n, int sign);

// Bluestein chirp-z transform for prime n.
void bluestein(const cplx *in, long istride, cplx *out, long n, int sign)
{
  long N2=2*n;
  auto w2=roots(N2,sign);   // exp(sign*2*pi*i*t/(2n)); chirp = w2[j^2 mod 2n]
  long K=ceilpow2(2*n-1);
  std::vector<cplx> a(K,0.0), b(K,0.0), A(K), B(K);
  std::vector<cplx> chirp(n);
  for(long j=0; j < n; ++j)
    chirp[j]=w2->w[(j*j) % N2];
  for(long j=0; j < n; ++j)
    a[j]=in[j*istride]*chirp[j];
  b[0]=std::conj(chirp[0]);
  for(long j=1; j < n; ++j)
    b[j]=b[K-j]=std::conj(chirp[j]);
  dft(a.data(),1,A.data(),K,-1);
  dft(b.data(),1,B.data(),K,-1);
  for(long k=0; k < K; ++k) A[k] *= B[k];
  dft(A.data(),1,a.data(),K,+1);
  double scale=1.0/(double) K;
  for(long k=0; k < n; ++k)
    out[k]=a[k]*scale*chirp[k];
}

// out[k] = sum_j in[j*istride] exp(sign*2*pi*i*j*k/n), k < n.
void dft(const cplx *in, long istride, cplx *out, long n, int sign)
{
  if(n == 1) {
    out[0]=in[0];
    return;
  }
  long p=smallestFactor(n);
  if(p == n) {
    if(n > 64) {
      bluestein(in,istride,out,n,sign);
      return;
    }
    auto w=roots(n,sign);
    for(long k=0; k < n; ++k) {
      cplx s=0.0;
      for(long j=0; j < n; ++j)
        s += in[j*istride]*w->w[(j*k) % n];
      out[k]=s;
    }
    return;
  }
  long m=n/p;
  // p sub-transforms of the decimated sequences x[j1 + p*j2].
  for(long j1=0; j1 < p; ++j1)
    dft(in+j1*istride,istride*p,out+j1*m,m,sign);
  auto w=roots(n,sign);
  std::vector<cplx> t(p), u(p);
  for(long k2=0; k2 < m; ++k2) {
    for(long j1=0; j1 < p; ++j1)
      t[j1]=out[j1*m+k2]*w->w[(j1*k2) % n];
    for(long k1=0; k1 < p; ++k1) {
      cplx s=0.0;
      for(long j1=0; j1 < p; ++j1)
        s += t[j1]*w->w[((j1*k1) % p)*m];
      u[k1]=s;
    }
    for(long k1=0; k1 < p; ++k1)
      out[k2+m*k1]=u[k1];
  }
}

// ---------------------------------------------------------------------------
// Plans.

struct Dim {
  long n, is, os;
};

enum Kind {KIND_DFT, KIND_R2C, KIND_C2R, KIND_COPY};

} // namespace

struct oracle_fftw_plan {
  Kind kind;
  int sign;
  std::vector<Dim> dims;     // transform dimensions, row-major (last fastest)
  std::vector<Dim> howmany;  // loop dimensions
  void *in;
  void *out;
};

namespace {

// Enumerate the flattened loop space: offsets of each iteration.
void loopOffsets(const std::vector<Dim>& loops,
                 std::vector<long>& ioff, std::vector<long>& ooff)
{
  ioff.assign(1,0);
  ooff.assign(1,0);
  for(const Dim& d : loops) {
    std::vector<long> ni, no;
    ni.reserve(ioff.size()*d.n);
    no.reserve(ooff.size()*d.n);
    for(size_t k=0; k < ioff.size(); ++k)
      for(long i=0; i < d.n; ++i) {
        ni.push_back(ioff[k]+i*d.is);
        no.push_back(ooff[k]+i*d.os);
      }
    ioff.swap(ni);
    ooff.swap(no);
  }
}

// In-place multi-dimensional complex DFT of a dense row-major array.
void dftDense(cplx *x, const std::vector<long>& n, int sign)
{
  long total=1;
  for(long v : n) total *= v;
  std::vector<cplx> line, res;
  long inner=total;
  for(size_t d=0; d < n.size(); ++d) {
    long nd=n[d];
    inner /= nd;
    long outer=total/(nd*inner);
    line.resize(nd);
    res.resize(nd);
    for(long o=0; o < outer; ++o)
      for(long i=0; i < inner; ++i) {
        cplx *base=x+o*nd*inner+i;
        for(long j=0; j < nd; ++j) line[j]=base[j*inner];
        dft(line.data(),1,res.data(),nd,sign);
        for(long j=0; j < nd; ++j) base[j*inner]=res[j];
      }
  }
}

long product(const std::vector<long>& v)
{
  long p=1;
  for(long x : v) p *= x;
  return p;
}

void executePlan(const oracle_fftw_plan *p, void *in, void *out)
{
  std::vector<long> ioff, ooff;
  loopOffsets(p->howmany,ioff,ooff);
  size_t count=ioff.size();

  std::vector<long> n;
  for(const Dim& d : p->dims) n.push_back(d.n);
  size_t rank=n.size();

  if(p->kind == KIND_COPY) {
    std::vector<long> ti, to;
    loopOffsets(p->howmany,ti,to);
    const double *src=(const double *) in;
    double *dst=(double *) out;
    std::vector<double> buf(ti.size());
    for(size_t k=0; k < ti.size(); ++k) buf[k]=src[ti[k]];
    for(size_t k=0; k < to.size(); ++k) dst[to[k]]=buf[k];
    return;
  }

  // Logical (input-side) and output-side element offsets inside one transform.
  std::vector<long> nLogical=n;   // complex DFT index space
  std::vector<long> nIn=n, nOut=n;
  if(p->kind == KIND_R2C) nOut[rank-1]=n[rank-1]/2+1;
  if(p->kind == KIND_C2R) nIn[rank-1]=n[rank-1]/2+1;

  auto offsets=[&](const std::vector<long>& shape, bool input) {
    std::vector<long> off(1,0);
    for(size_t d=0; d < rank; ++d) {
      long stride=input ? p->dims[d].is : p->dims[d].os;
      std::vector<long> no;
      no.reserve(off.size()*shape[d]);
      for(long base : off)
        for(long j=0; j < shape[d]; ++j) no.push_back(base+j*stride);
      off.swap(no);
    }
    return off;
  };
  std::vector<long> inOff=offsets(nIn,true);
  std::vector<long> outOff=offsets(nOut,false);

  long N=product(nLogical);
  std::vector<cplx> work(count*N);

  // Gather every input before any output is written (aliasing-safe).
  if(p->kind == KIND_DFT) {
    const cplx *src=(const cplx *) in;
    for(size_t c=0; c < count; ++c)
      for(long e=0; e < N; ++e)
        work[c*N+e]=src[ioff[c]+inOff[e]];
  } else if(p->kind == KIND_R2C) {
    const double *src=(const double *) in;
    for(size_t c=0; c < count; ++c)
      for(long e=0; e < N; ++e)
        work[c*N+e]=cplx(src[ioff[c]+inOff[e]],0.0);
  } else { // C2R: Hermitian-extend the last dimension
    const cplx *src=(const cplx *) in;
    long nl=n[rank-1], hl=nl/2+1;
    long outerN=N/nl;
    for(size_t c=0; c < count; ++c) {
      cplx *w=work.data()+c*N;
      for(long o=0; o < outerN; ++o)
        for(long j=0; j < hl; ++j)
          w[o*nl+j]=src[ioff[c]+inOff[o*hl+j]];
      // Full multi-dimensional Hermitian extension: X[-k] = conj X[k].
      std::vector<long> idx(rank,0);
      for(long e=0; e < N; ++e) {
        long rem=e;
        for(size_t d=rank; d-- > 0;) {
          idx[d]=rem % n[d];
          rem /= n[d];
        }
        if(idx[rank-1] < hl) continue;
        long mirror=0;
        for(size_t d=0; d < rank; ++d)
          mirror=mirror*n[d]+((n[d]-idx[d]) % n[d]);
        w[e]=std::conj(w[mirror]);
      }
    }
  }

  int sign=p->kind == KIND_R2C ? FFTW_FORWARD :
    p->kind == KIND_C2R ? FFTW_BACKWARD : p->sign;
  for(size_t c=0; c < count; ++c)
    dftDense(work.data()+c*N,nLogical,sign);

  if(p->kind == KIND_DFT) {
    cplx *dst=(cplx *) out;
    for(size_t c=0; c < count; ++c)
      for(long e=0; e < N; ++e)
        dst[ooff[c]+outOff[e]]=work[c*N+e];
  } else if(p->kind == KIND_R2C) {
    cplx *dst=(cplx *) out;
    long nl=n[rank-1], hl=nl/2+1, outerN=N/nl;
    for(size_t c=0; c < count; ++c)
      for(long o=0; o < outerN; ++o)
        for(long j=0; j < hl; ++j)
          dst[ooff[c]+outOff[o*hl+j]]=work[c*N+o*nl+j];
  } else {
    double *dst=(double *) out;
    for(size_t c=0; c < count; ++c)
      for(long e=0; e < N; ++e)
        dst[ooff[c]+outOff[e]]=work[c*N+e].real();
  }
}

// Dense row-major strides for a shape, scaled by a unit stride.
std::vector<Dim> denseDims(int rank, const int *n, const int *iembed,
                           const int *oembed, long istride, long ostride,
                           long lastIn, long lastOut)
{
  std::vector<Dim> dims(rank);
  long is=istride, os=ostride;
  for(int d=rank-1; d >= 0; --d) {
    dims[d].n=n[d];
    dims[d].is=is;
    dims[d].os=os;
    long ie=iembed ? iembed[d] : (d == rank-1 ? lastIn : n[d]);
    long oe=oembed ? oembed[d] : (d == rank-1 ? lastOut : n[d]);
    is *= ie;
    os *= oe;
  }
  return dims;
}

fftw_plan makePlan(Kind kind, int sign, std::vector<Dim> dims,
                   std::vector<Dim> howmany, void *in, void *out)
{
  oracle_fftw_plan *p=new oracle_fftw_plan;
  p->kind=kind;
  p->sign=sign;
  p->dims=dims;
  p->howmany=howmany;
  p->in=in;
  p->out=out;
  // Build the twiddle tables now so that execute only reads the cache.
  for(const Dim& d : dims) {
    roots(d.n,sign);
    roots(d.n,-1);
    roots(d.n,+1);
  }
  return p;
}

} // namespace

extern "C" {

fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany,
                             fftw_complex *in, const int *inembed,
                             int istride, int idist,
                             fftw_complex *out, const int *onembed,
                             int ostride, int odist,
                             int sign, unsigned)
{
  std::vector<Dim> dims=denseDims(rank,n,inembed,onembed,istride,ostride,
                                  n[rank-1],n[rank-1]);
  return makePlan(KIND_DFT,sign,dims,{{howmany,idist,odist}},in,out);
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags)
{
  return fftw_plan_many_dft(1,&n,1,in,NULL,1,n,out,NULL,1,n,sign,flags);
}

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in,
                           fftw_complex *out, int sign, unsigned flags)
{
  int n[]={n0,n1};
  return fftw_plan_many_dft(2,n,1,in,NULL,1,0,out,NULL,1,0,sign,flags);
}

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in,
                           fftw_complex *out, int sign, unsigned flags)
{
  int n[]={n0,n1,n2};
  return fftw_plan_many_dft(3,n,1,in,NULL,1,0,out,NULL,1,0,sign,flags);
}

fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany,
                                 double *in, const int *inembed,
                                 int istride, int idist,
                                 fftw_complex *out, const int *onembed,
                                 int ostride, int odist, unsigned)
{
  long last=n[rank-1];
  long lastIn=((void *) in == (void *) out) ? 2*(last/2+1) : last;
  std::vector<Dim> dims=denseDims(rank,n,inembed,onembed,istride,ostride,
                                  lastIn,last/2+1);
  return makePlan(KIND_R2C,FFTW_FORWARD,dims,{{howmany,idist,odist}},in,out);
}

fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany,
                                 fftw_complex *in, const int *inembed,
                                 int istride, int idist,
                                 double *out, const int *onembed,
                                 int ostride, int odist, unsigned)
{
  long last=n[rank-1];
  long lastOut=((void *) in == (void *) out) ? 2*(last/2+1) : last;
  std::vector<Dim> dims=denseDims(rank,n,inembed,onembed,istride,ostride,
                                  last/2+1,lastOut);
  return makePlan(KIND_C2R,FFTW_BACKWARD,dims,{{howmany,idist,odist}},in,out);
}

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out,
                               unsigned flags)
{
  return fftw_plan_many_dft_r2c(1,&n,1,in,NULL,1,0,out,NULL,1,0,flags);
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out,
                               unsigned flags)
{
  int n[]={n0,n1};
  return fftw_plan_many_dft_r2c(2,n,1,in,NULL,1,0,out,NULL,1,0,flags);
}

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in,
                               fftw_complex *out, unsigned flags)
{
  int n[]={n0,n1,n2};
  return fftw_plan_many_dft_r2c(3,n,1,in,NULL,1,0,out,NULL,1,0,flags);
}

fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out,
                               unsigned flags)
{
  return fftw_plan_many_dft_c2r(1,&n,1,in,NULL,1,0,out,NULL,1,0,flags);
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out,
                               unsigned flags)
{
  int n[]={n0,n1};
  return fftw_plan_many_dft_c2r(2,n,1,in,NULL,1,0,out,NULL,1,0,flags);
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in,
                               double *out, unsigned flags)
{
  int n[]={n0,n1,n2};
  return fftw_plan_many_dft_c2r(3,n,1,in,NULL,1,0,out,NULL,1,0,flags);
}

fftw_plan fftw_plan_guru_r2r(int rank, const fftw_iodim *dims,
                             int howmany_rank, const fftw_iodim *howmany_dims,
                             double *in, double *out,
                             const fftw_r2r_kind *, unsigned)
{
  if(rank != 0) return NULL;   // only the rank-0 copy (transpose) is used
  std::vector<Dim> loops;
  for(int d=0; d < howmany_rank; ++d)
    loops.push_back({howmany_dims[d].n,howmany_dims[d].is,howmany_dims[d].os});
  return makePlan(KIND_COPY,0,{},loops,in,out);
}

void fftw_execute(const fftw_plan p)
{
  executePlan(p,p->in,p->out);
}

void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out)
{
  executePlan(p,in,out);
}

void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out)
{
  executePlan(p,in,out);
}

void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out)
{
  executePlan(p,in,out);
}

void fftw_execute_r2r(const fftw_plan p, double *in, double *out)
{
  executePlan(p,in,out);
}

void fftw_destroy_plan(fftw_plan p)
{
  delete p;
}

int fftw_init_threads(void) {return 1;}
void fftw_plan_with_nthreads(int) {}
void fftw_cleanup_threads(void) {}
void fftw_cleanup(void) {}

int fftw_import_wisdom_from_string(const char *) {return 1;}

char *fftw_export_wisdom_to_string(void)
{
  char *s=(char *) malloc(1);
  s[0]=0;
  return s;
}

void fftw_forget_wisdom(void) {}

void *fftw_malloc(size_t n)
{
  void *p=NULL;
  if(posix_memalign(&p,64,n ? n : 1) != 0) return NULL;
  return p;
}

void fftw_free(void *p) {free(p);}

int fftw_alignment_of(double *p) {return (int) (((size_t) p) % 16);}

}
