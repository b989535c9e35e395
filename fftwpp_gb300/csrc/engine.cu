// engine.cu -- planning and launch sequences of the GB300 hybrid convolution.
#include "engine.h"
#include "kernels.cuh"

#include <atomic>
#include <climits>
#include <cstring>
#include <cmath>
#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <tuple>
#include <type_traits>

namespace fgb {

// ---------------------------------------------------------------------------
// Integer rules (restated from convolve.cc:114-175 and :403-410).

size_t ceilquotient(size_t a, size_t b) {return (a+b-1)/b;}

static size_t ceilpow2(size_t n)
{
  size_t p=1;
  while(p < n) p <<= 1;
  return p;
}

static size_t ceilpow(size_t b, size_t n)
{
  size_t p=1;
  while(p < n) p *= b;
  return p;
}

size_t nextfftsize(size_t m)
{
  size_t N=ceilpow2(m);
  if(m == N) return m;
  for(size_t ni=1; ni < N; ni *= 7)
    for(size_t nj=ni; nj < N; nj *= 5)
      for(size_t nk=nj; nk < N; nk *= 3)
        N=std::min(N,nk*ceilpow2(ceilquotient(m,nk)));
  return N;
}

size_t nextpuresize(size_t m)
{
  size_t M=ceilpow2(m);
  if(m == M) return m;
  M=std::min(M,ceilpow(3,m));
  if(m == M) return m;
  M=std::min(M,ceilpow(5,m));
  if(m == M) return m;
  return std::min(M,ceilpow(7,m));
}

bool ispure(size_t m)
{
  return m == ceilpow(2,m) || m == ceilpow(3,m) || m == ceilpow(5,m) ||
    m == ceilpow(7,m);
}

void refParameters(size_t L, size_t M, size_t m, bool centered,
                   size_t& p, size_t& n, size_t& q)
{
  p=ceilquotient(L,m);
  size_t P=(centered && p % 2 == 0) || p == 2 ? p/2 : p;
  n=ceilquotient(M,P*m);
  q=P*n;
}

bool smooth(size_t n)
{
  if(n == 0) return false;
  for(size_t f : {2,3,5,7})
    while(n % f == 0) n /= f;
  return n == 1;
}

// ---------------------------------------------------------------------------
// Errors.

static thread_local std::string errorText;
std::string lastError() {return errorText;}
void setLastError(const std::string& s) {errorText=s;}

// ---------------------------------------------------------------------------
// Device allocation with host-side failure injection.

static std::atomic<long> allocCountdown(-1);

void failAllocationAfter(long n) {allocCountdown=n;}

cudaError_t devAlloc(void **p, size_t bytes)
{
  long c=allocCountdown.load();
  while(c >= 0 && !allocCountdown.compare_exchange_weak(c,c-1)) {}
  if(c == 0) {
    *p=NULL;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p,bytes);
}

// ---------------------------------------------------------------------------
// Twiddle tables.

const void *twiddles(long n, int prec)
{
  if(prec == PREC_FF) prec=PREC_F32;        // the same hi+lo float4 table
  static std::mutex mu;
  static std::map<std::tuple<int,long,int>,void *> cache;
  int dev=0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  auto key=std::make_tuple(dev,n,prec);
  auto it=cache.find(key);
  if(it != cache.end()) return it->second;

  // exp(2 pi i t/n) from the exact rational angle t/n, reduced to the
  // first octant so that the long double evaluation stays accurate.
  std::vector<double> c(n), s(n);
  const long double pi=3.141592653589793238462643383279502884L;
  for(long t=0; t < n; ++t) {
    // angle = 2 pi t/n; fold by symmetry into [0, pi/4].
    long tt=t;
    long double sign_c=1, sign_s=1;
    long u=tt;
    // Use 8t vs n comparisons with exact integer arithmetic.
    long double a;
    bool swap=false;
    if(2*u > n) {u=n-u; sign_s=-1;}                 // [0, pi]
    if(4*u > n) {u=n-2*u; sign_c=-sign_c;           // pi - angle
      // angle' = pi - angle = 2 pi (n/2 - u)/n  -> represent as 2*pi*u'/(2n)
      a=pi*(long double) u/(long double) n;
      // a in [0, pi/2)
    } else
      a=2*pi*(long double) u/(long double) n;
    if(a > pi/4) {a=pi/2-a; swap=true;}
    long double cv=cosl(a), sv=sinl(a);
    if(swap) std::swap(cv,sv);
    c[t]=(double) (sign_c*cv);
    s[t]=(double) (sign_s*sv);
  }
  void *d=NULL;
  if(prec == PREC_F64) {
    std::vector<double2> h(n);
    for(long t=0; t < n; ++t) h[t]=make_double2(c[t],s[t]);
    if(devAlloc((void **) &d,n*sizeof(double2)) != cudaSuccess) return NULL;
    cudaMemcpy(d,h.data(),n*sizeof(double2),cudaMemcpyHostToDevice);
  } else {
    std::vector<float4> h(n);
    for(long t=0; t < n; ++t) {
      float hx=(float) c[t], hy=(float) s[t];
      h[t]=make_float4(hx,hy,(float) (c[t]-(double) hx),
                       (float) (s[t]-(double) hy));
    }
    if(devAlloc((void **) &d,n*sizeof(float4)) != cudaSuccess) return NULL;
    cudaMemcpy(d,h.data(),n*sizeof(float4),cudaMemcpyHostToDevice);
  }
  cache[key]=d;
  return d;
}

// Radices of an n-point transform into radix[] (at most FGB_MAXSTAGES);
// returns their count, or -1 when n is not 2^a 3^b 5^c 7^d or needs too
// many stages.  The Stockham form wants the products of earlier radices to
// be powers of two (odd radices last); the in-place decimation forms want
// the spans n/(R0...Rs) to be powers of two (odd radices first).  Either
// way the stage divisions become shifts.
int fftRadices(long n, int prec, bool oddFirst, bool allow16, int *radix)
{
  if(n < 1 || !smooth(n)) return -1;
  int nst=0, tmp[64];
  long r=n;
  // Largest radices first: 8, then 4 or 2, then odd primes.  FP32 in-place
  // transforms (allow16) also take radix 16 (4 x 4 in registers) where that
  // saves a stage: a power-of-two factor 2^k takes ceil(k/3) stages of
  // radix <= 8 but s = ceil(k/4) of radix <= 16, as k - 3s radix-16 stages
  // and the rest radix 8.  A factor 3 with k >= 1 may take one factor 2
  // into a radix-6 stage when that saves one more (1536 = 6 16 16).
  int k2=0;
  for(long t=n; t % 2 == 0; t /= 2) ++k2;
  const bool wide=allow16 && prec == PREC_F32 && oddFirst;
  const bool six=wide && n % 3 == 0 && k2 >= 1 &&
    1+(k2+2)/4 < 1+(k2+3)/4;
  if(six) {k2 -= 1; r /= 2;}           // the factor 2 of the radix-6 stage
  if(wide && (k2+3)/4 < (k2+2)/3)
    for(int i=0; i < k2-3*((k2+3)/4); ++i) {tmp[nst++]=16; r /= 16;}
  while(r % 8 == 0) {tmp[nst++]=8; r /= 8;}
  if(r % 4 == 0) {tmp[nst++]=4; r /= 4;}
  if(r % 2 == 0) {tmp[nst++]=2; r /= 2;}
  while(r % 7 == 0) {tmp[nst++]=7; r /= 7;}
  while(r % 5 == 0) {tmp[nst++]=5; r /= 5;}
  while(r % 3 == 0) {tmp[nst++]=3; r /= 3;}
  if(nst > FGB_MAXSTAGES) return -1;
  if(six) {                              // one radix 3 becomes the radix 6
    for(int s=nst-1; s >= 0; --s)
      if(tmp[s] == 3) {tmp[s]=6; break;}
  }
  int k=0;
  if(oddFirst) {
    // Odd radices first (the radix 6 with them, last), then the powers of
    // two, each group in order: every span after them is a power of two.
    for(int s=0; s < nst; ++s)
      if(tmp[s] % 2) radix[k++]=tmp[s];
    for(int s=0; s < nst; ++s)
      if(tmp[s] == 6) radix[k++]=tmp[s];
    for(int s=0; s < nst; ++s)
      if(tmp[s] % 2 == 0 && tmp[s] != 6) radix[k++]=tmp[s];
  } else {
    for(int s=0; s < nst; ++s) radix[k++]=tmp[s];
  }
  return nst;
}

static FFTPlanDev fftPlan(long n, int prec, bool oddFirst=false,
                          bool allow16=false)
{
  FFTPlanDev p;
  p.n=(int) n;
  p.nst=fftRadices(n,prec,oddFirst,allow16,p.radix);
  if(p.nst < 0) {
    if(!smooth(n))
      throw std::runtime_error("transform length "+std::to_string(n)+
                               " is not a product of 2, 3, 5 and 7");
    throw std::runtime_error("too many FFT stages");
  }
  p.tw=twiddles(n,prec);
  if(!p.tw) throw std::runtime_error("twiddle table allocation failed");
  return p;
}

FFTPlanDev fftPlanPublic(long n, int prec, bool oddFirst)
{
  return fftPlan(n,prec,oddFirst);
}

// ---------------------------------------------------------------------------
// Planning.

static const size_t SMEM_MAX=227*1024;

// 16-byte complex elements (FP64 and float-float) or 8-byte ones (FP32).
static bool wide(int prec) {return prec != PREC_F32;}

// A kernel-side size function evaluated for the arithmetic type of prec.
#define FGB_BY_PREC(prec,F,...) ((prec) == PREC_F64 ? F<double>(__VA_ARGS__) : \
  (prec) == PREC_FF ? F<ff>(__VA_ARGS__) : F<float>(__VA_ARGS__))
static size_t elem(int prec) {return wide(prec) ? 16 : 8;}

// direct: a row plan with one residue and one fold (RowPlan::direct).
static size_t rowNeed(int prec, long L, long m, int A, int B, int rpc=1,
                      int direct=0)
{
  return FGB_BY_PREC(prec,rowSmem,L,m,A,B,rpc,direct);
}

static size_t hermNeed(int prec, long H, long Nh, int A, int rpc=1)
{
  return FGB_BY_PREC(prec,hermRowSmem,H,Nh,A,rpc);
}

static size_t outerNeed(int prec, long L, long m, int tile)
{
  size_t f=FGB_BY_PREC(prec,outerFwdSmem,L,m,tile);
  size_t b=FGB_BY_PREC(prec,outerBwdSmem,L,m,tile);
  return std::max(f,b);
}


static double fftInstr(long n);

// Rows per CTA of a row kernel: enough that a radix-8 stage has >= 512
// butterflies for 256 threads, at most 8 and at most nrows, within half of
// the shared memory (two CTAs per SM).
template<typename F>
static int pickRpc(long n, int A, long nrows, F smem)
{
  long per=std::max(1L,n/8)*A;
  int rpc=(int) std::min<long>(8,std::max<long>(1,(512+per-1)/per));
  rpc=(int) std::min<long>(rpc,std::max(1L,nrows));
  while(rpc > 1 && smem(rpc) > SMEM_MAX/2) --rpc;
  return rpc;
}

// Estimated arithmetic instructions of a row axis with residue blocks of m
// points and q residues: transforms, the fold (a complex twiddle per term
// for residues r > 0) and the post-twiddled accumulation.
static double rowCost(const AxisPlan& a, long m, long q, int A, int B)
{
  long p=ceilquotient(a.L,m);
  return q*(A+B)*fftInstr(m)+A*(double) m*(2.0*p+(q-1)*6.0*p)+
    B*(double) a.L*(2.0+(q-1)*6.0);
}

// The same for an outer axis: residue r > 0 folds p terms with a complex
// twiddle each (forward) and post-twiddles every output (backward); r = 0
// only adds.
static double outerCost(const AxisPlan& a, long m, long q, int A, int B)
{
  long p=ceilquotient(a.L,m);
  double fwd=q*fftInstr(m)+m*(2.0*p+(q-1)*6.0*p);
  double bwd=q*fftInstr(m)+a.L*(2.0+(q-1)*6.0);
  return A*fwd+B*bwd;
}

// Inner (row) axis, complex data: residue block m and residue count q.
static bool planRowComplex(AxisPlan& a, long mForce, int A, int B, int prec)
{
  bool centered=a.kind == KIND_CENTERED;
  if(mForce > 0) {
    size_t p,n,q;
    refParameters(a.L,a.M,mForce,centered,p,n,q);
    if(!smooth(mForce)) return false;
    a.m=mForce; a.q=q;
  } else {
    double best=1e300;
    long bm=0, bq=0;
    for(long q=1; q <= 64; ++q) {
      long m=nextfftsize(ceilquotient(a.M,q));
      if(m*q < a.M) continue;
      if(rowNeed(prec,a.L,m,A,B) > SMEM_MAX) continue;
      double cost=rowCost(a,m,q,A,B);
      if(cost < best) {best=cost; bm=m; bq=q;}
    }
    if(!bm) return false;
    a.m=bm; a.q=bq;
  }
  a.N=a.m*a.q;
  a.p=ceilquotient(a.L,a.m);
  a.cshift=centered ? (int) (a.L/2) : 0;
  return rowNeed(prec,a.L,a.m,A,B) <= SMEM_MAX;
}

static long evenSmooth(long M)
{
  long N=std::max(M,2L);
  if(N % 2) ++N;
  while(!smooth(N/2)) N += 2;
  return N;
}

static bool planRowHermitian(AxisPlan& a, long mForce, int A, int prec)
{
  long M=a.M;
  if(mForce > 0) {
    size_t p,n,q;
    refParameters(a.L,a.M,mForce,true,p,n,q);
    M=std::max<long>(M,mForce*q);
  }
  a.N=evenSmooth(M);
  a.m=a.N; a.q=1; a.p=1;
  a.cshift=0;
  return hermNeed(prec,a.stored,a.N/2,A) <= SMEM_MAX;
}

// Estimated FP64/FP32 arithmetic instructions of one length-n transform in
// the radix order fftPlan uses (codelet + twiddles per point, stage 0 has
// unit twiddles).
static double fftInstr(long n)
{
  std::vector<int> rad;
  long r=n;
  while(r % 8 == 0) {rad.push_back(8); r /= 8;}
  if(r % 4 == 0) {rad.push_back(4); r /= 4;}
  if(r % 2 == 0) {rad.push_back(2); r /= 2;}
  while(r % 7 == 0) {rad.push_back(7); r /= 7;}
  while(r % 5 == 0) {rad.push_back(5); r /= 5;}
  while(r % 3 == 0) {rad.push_back(3); r /= 3;}
  double per=0;
  for(size_t i=0; i < rad.size(); ++i) {
    int R=rad[i];
    double code=R == 8 ? 7.0 : R == 4 ? 4.0 : R == 2 ? 2.0 : R == 3 ? 4.7 :
      R == 5 ? 6.8 : 8.6;
    double tw=i == 0 ? 0.0 : 4.0*(R-1)/R;
    per += code+tw;
  }
  return per*n;
}

static const int NSM=152;

// Largest power-of-two tile <= maxTile whose kernel fits in shared memory
// and gives at least two waves of CTAs over the SMs, but not narrower than
// one 32-byte sector per row (minTile columns) unless shared memory forces
// it.
template<typename F>
static int pickTile(int maxTile, long C, long factor, F smem, int minTile=1)
{
  int tile=maxTile;
  while(tile > minTile && (smem(tile) > SMEM_MAX ||
                           ceilquotient(C,tile)*factor < 2*NSM))
    tile /= 2;
  while(tile > 1 && smem(tile) > SMEM_MAX) tile /= 2;
  return tile;
}

static void planOuter(AxisPlan& a, long mForce, int prec, long C, long nbatch,
                      int A, int B)
{
  int maxTile=wide(prec) ? 8 : 16;
  int minTile=wide(prec) ? 2 : 4;
  if(a.kind == KIND_REAL) {
    a.N=evenSmooth(mForce > 0 ? std::max(a.M,mForce) : a.M);
    a.m=a.N; a.q=1; a.p=1; a.cshift=0;
    a.rows=a.N/2+1;
    long Nh=a.N/2;
    auto sm=[&](int t) {
      return FGB_BY_PREC(prec,outerRealSmem,a.L,Nh,t);
    };
    a.tile=pickTile(maxTile,C,nbatch*A,sm,minTile);
    a.tileB=pickTile(maxTile,C,nbatch*B,sm,minTile);
    return;
  }
  bool centered=a.kind == KIND_CENTERED;
  if(mForce > 0) {
    size_t p,n,q;
    refParameters(a.L,a.M,mForce,centered,p,n,q);
    if(!smooth(mForce))
      throw std::runtime_error("forced m must be a product of 2,3,5,7");
    a.m=mForce; a.q=q;
  } else {
    long N=nextfftsize(a.M);
    double best=1e300;
    long bm=0;
    for(long m=1; m <= N; ++m) {
      if(N % m || !smooth(m)) continue;
      if(outerNeed(prec,a.L,m,1) > SMEM_MAX) continue;
      double cost=outerCost(a,m,N/m,A,B);
      if(cost < best) {best=cost; bm=m;}
    }
    if(!bm) throw std::runtime_error("no outer padding plan fits");
    a.m=bm; a.q=N/bm;
  }
  a.N=a.m*a.q;
  a.p=ceilquotient(a.L,a.m);
  a.cshift=centered ? (int) (a.L/2) : 0;
  a.rows=a.N;
  const int ip=a.p == 1;     // in-place outer transforms (FP32-pipe modes)
  auto smf=[&](int t) {
    return FGB_BY_PREC(prec,outerFwdSmem,a.L,a.m,t,ip);
  };
  auto smb=[&](int t) {
    return FGB_BY_PREC(prec,outerBwdSmem,a.L,a.m,t,(int) a.q,ip);
  };
  a.tile=pickTile(maxTile,C,nbatch*a.q*A,smf,minTile);
  a.tileB=pickTile(maxTile,C,nbatch*B,smb,minTile);
  if(smf(a.tile) > SMEM_MAX || smb(a.tileB) > SMEM_MAX)
    throw std::runtime_error("outer axis too long for shared memory");
}

Conv::Conv(int dim, const int *kinds, const long *L, const long *M,
           const long *mForce, int A, int B, int mult, int prec, long batch,
           bool tuneSchedule)
  : batch(batch), user(NULL), isStrided(false), ffState(NULL), longBuf(0),
    tuning(false), staging(0), hostIn(NULL),
    hostOut(NULL), nlaunch(0),
    timing(false), normalize(true), marks(0), hostTile(0), hostThr(0),
    hostTileB(0), hostThrB(0), side(NULL), chunks(0), outChunks(0),
    outCopied(NULL)
{
  for(int k=0; k < CHUNKS; ++k) {
    lanes[k]=NULL;
    outDone[k]=NULL;
    chunkReady[k]=chunkDone[k]=NULL;
  }
  hostWay[0]=hostWay[1]=-1;
  if(dim < 1 || dim > 3) throw std::runtime_error("dimension must be 1, 2 or 3");
  if(A < 1 || A > FGB_MAXA || B < 1 || B > A)
    throw std::runtime_error("need 1 <= B <= A <= 8");
  if(prec != PREC_F64 && prec != PREC_F32 && prec != PREC_FF)
    throw std::runtime_error("unknown precision");
  if(batch < 1) throw std::runtime_error("batch must be positive");
  switch(mult) {
    case MULT_NONE: break;
    case MULT_BINARY: case MULT_REALBINARY: case MULT_CORRELATION:
      if(A < 2) throw std::runtime_error("a binary multiplier needs A >= 2");
      break;
    case MULT_REALJACOBIAN: case MULT_JACOBIAN:
      if(A < 4) throw std::runtime_error("a Jacobian multiplier needs A >= 4");
      break;
    case MULT_REALJACADJ:
      if(A != 5 || B != 4)
        throw std::runtime_error("the Jacobian adjoint needs A = 5, B = 4");
      break;
    case MULT_DOT: case MULT_REALDOT:
      if(A % 2 || B != 1)
        throw std::runtime_error("a dot-product multiplier needs an even A "
                                 "and B = 1");
      break;
    case MULT_USER: break;
    default: throw std::runtime_error("unknown multiplier");
  }
  I.dim=dim; I.A=A; I.B=B; I.mult=mult; I.prec=prec;
  I.longRow=false; I.rowM=I.rowQ=0;
  for(int d=0; d < dim; ++d) {
    AxisPlan& a=I.axis[d];
    a.kind=kinds[d];
    a.L=L[d];
    a.M=M[d];
    if(a.kind < 0 || a.kind > 3) throw std::runtime_error("unknown axis kind");
    if(a.L < 1) throw std::runtime_error("L must be positive");
    if(a.L > a.M)
      throw std::runtime_error("L="+std::to_string(a.L)+" is greater than M="+
                               std::to_string(a.M));
    if(a.kind == KIND_HERMITIAN && d != dim-1)
      throw std::runtime_error("a Hermitian axis must be the innermost");
    if(a.kind == KIND_REAL && d != 0)
      throw std::runtime_error("a real axis must be the outermost");
    a.stored=a.kind == KIND_HERMITIAN ? (long) ceilquotient(a.L,2) : a.L;
    a.tile=a.tileB=1;
    a.rpc=1;
    a.thr=a.thrB=256;
    a.rows=0;
  }
  if(dim > 1 && batch != 1)
    throw std::runtime_error("batched problems are one-dimensional");

  for(int d=0; d < dim-1; ++d) {
    long C=1, nb=1;
    for(int e=d+1; e < dim; ++e) C *= I.axis[e].stored;
    for(int e=0; e < d; ++e) nb *= I.axis[e].rows;
    planOuter(I.axis[d],mForce ? mForce[d] : 0,prec,C,nb,A,B);
  }
  AxisPlan& in=I.axis[dim-1];
  long mf=mForce ? mForce[dim-1] : 0;
  bool ok;
  if(in.kind == KIND_HERMITIAN) ok=planRowHermitian(in,mf,A,prec);
  else ok=planRowComplex(in,mf,A,B,prec);
  if(in.kind == KIND_REAL && dim == 1) in.rows=0;
  if(!ok) {
    // Long rows (beyond one CTA's shared memory), any kind: the row is a
    // cyclic convolution of length N = rowM * rowQ >= M (explicit padding,
    // which is dealiased for every kind once N >= M), computed as columns
    // of length rowQ (outer, with the W_N^{t r} twiddle), rows of length
    // rowM and the inverse columns.  Centred data sit cyclically shifted
    // by floor(L/2), Hermitian data as their mirrored full spectrum, real
    // data with zero imaginary parts (FlatMode).
    long N=nextfftsize(in.M);
    long best=0;
    for(long m=1; m <= N; ++m)
      if(N % m == 0 && smooth(m) && rowNeed(prec,m,m,A,B) <= SMEM_MAX / 2)
        best=m;
    if(!best) throw std::runtime_error("no long-row plan");
    I.longRow=true;
    I.rowM=best;
    I.rowQ=N/best;
    in.N=N; in.m=best; in.q=N/best; in.p=ceilquotient(in.stored,best);
    in.cshift=in.kind == KIND_CENTERED ? (int) (in.L/2) : 0;
    // The column kernels of the other kinds cover all rowQ rows.
    const long colRows=in.kind == KIND_PAD || in.kind == KIND_REAL ? in.p :
      I.rowQ;
    long outerRows=batch;
    for(int d=0; d < dim-1; ++d) outerRows *= I.axis[d].rows;
    auto sm=[&](int t) {return outerNeed(prec,colRows,I.rowQ,t);};
    in.tile=pickTile(wide(prec) ? 8 : 16,I.rowM,A*outerRows,sm);
    in.tileB=pickTile(wide(prec) ? 8 : 16,I.rowM,B*outerRows,sm);
    if(mForce && mForce[dim-1] > 0)
      throw std::runtime_error("forced m not supported on the long path");
    if(outerRows*A > 65535 || outerRows*B > 65535)
      throw std::runtime_error("too many long rows for one launch");
  }
  // Rows per CTA of the row kernel.
  long nrows=batch;
  for(int d=0; d < dim-1; ++d) nrows *= I.axis[d].rows;
  if(I.longRow) {
    in.rpc=pickRpc(I.rowM,A,I.rowQ*nrows,[&](int r) {
      return rowNeed(prec,I.rowM,I.rowM,A,B,r,1);});
  } else if(in.kind == KIND_HERMITIAN) {
    in.rpc=pickRpc(in.N/2,A,nrows,[&](int r) {
      return hermNeed(prec,in.stored,in.N/2,A,r);});
  } else {
    in.rpc=pickRpc(in.m,A,nrows,[&](int r) {
      return rowNeed(prec,in.stored,in.m,A,B,r,
                     in.q == 1 && in.stored <= in.m);});
  }
  try {
    allocate();
    if(autotune && tuneSchedule) tune();
  } catch(...) {
    // A throwing constructor runs no destructor: release what was taken.
    for(void *p : bufs) cudaFree(p);
    bufs.clear();
    if(ffState) cudaFree(ffState);
    ffState=NULL;
    throw;
  }
}

bool Conv::rangeGuard=true;
void Conv::setRangeGuard(bool on) {rangeGuard=on;}

bool Conv::autotune=true;
void Conv::setAutotune(bool on) {autotune=on;}
bool Conv::residueSearch=true;
void Conv::setResidueSearch(bool on) {residueSearch=on;}

// Candidate residue block lengths of a complex axis for the timed search:
// at most three, cheapest estimate first, each within 1.5x of the cheapest.
static std::vector<long> residueCandidates(const AxisPlan& a, bool outer,
                                           int prec, int A, int B)
{
  std::vector<std::pair<double,long>> c;
  if(outer) {
    long N=nextfftsize(a.M);
    for(long m=1; m <= N; ++m)
      if(N % m == 0 && smooth(m) && outerNeed(prec,a.L,m,1) <= SMEM_MAX)
        c.push_back({outerCost(a,m,N/m,A,B),m});
  } else {
    for(long q=1; q <= 64; ++q) {
      long m=nextfftsize(ceilquotient(a.M,q));
      if(m*q < a.M || rowNeed(prec,a.L,m,A,B) > SMEM_MAX) continue;
      bool seen=false;
      for(const auto& x : c) seen=seen || x.second == m;
      if(!seen) c.push_back({rowCost(a,m,q,A,B),m});
    }
  }
  std::sort(c.begin(),c.end());
  std::vector<long> out;
  for(const auto& x : c)
    if(out.size() < 3 && x.first <= 1.5*c[0].first) out.push_back(x.second);
  return out;
}

// ---------------------------------------------------------------------------
// Plan wisdom (engine.h).

static std::mutex wisdomMutex;
static std::map<std::string,std::string> wisdomMap;

// The problem and the GPU a plan was tuned for, and whether its residue
// blocks were searched.
static std::string wisdomKey(int dim, const int *kinds, const long *L,
                             const long *M, const long *mForce, int A, int B,
                             int mult, int prec, long batch, bool searched)
{
  int dev=0, sms=0, major=0, minor=0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms,cudaDevAttrMultiProcessorCount,dev);
  cudaDeviceGetAttribute(&major,cudaDevAttrComputeCapabilityMajor,dev);
  cudaDeviceGetAttribute(&minor,cudaDevAttrComputeCapabilityMinor,dev);
  cudaGetLastError();
  std::string k="fgb1 sm"+std::to_string(major)+std::to_string(minor)+"x"+
    std::to_string(sms)+" d"+std::to_string(dim);
  for(int d=0; d < dim; ++d)
    k += " "+std::to_string(kinds[d])+":"+std::to_string(L[d])+":"+
      std::to_string(M[d])+":"+std::to_string(mForce ? mForce[d] : 0);
  k += " A"+std::to_string(A)+" B"+std::to_string(B)+" u"+
    std::to_string(mult)+" p"+std::to_string(prec)+" n"+std::to_string(batch)+
    (searched ? " r1" : " r0");          // m searched or the cost model's
  return k;
}

std::string Conv::exportWisdom()
{
  std::lock_guard<std::mutex> g(wisdomMutex);
  std::string t;
  for(const auto& kv : wisdomMap) t += kv.first+"\t"+kv.second+"\n";
  return t;
}

int Conv::importWisdom(const std::string& text)
{
  std::vector<std::pair<std::string,std::string>> lines;
  size_t pos=0;
  while(pos < text.size()) {
    size_t end=text.find('\n',pos);
    if(end == std::string::npos) end=text.size();
    const std::string line=text.substr(pos,end-pos);
    pos=end+1;
    if(line.empty()) continue;
    const size_t tab=line.find('\t');
    if(tab == std::string::npos || tab == 0 || line.compare(0,5,"fgb1 ") != 0)
      return -1;
    std::string value=line.substr(tab+1);
    // 3 residue blocks, then per axis tile, threads, backward tile,
    // threads, rows per CTA, then the four host-line tile numbers.
    std::istringstream in(value);
    long v;
    int count=0;
    while(in >> v) {
      if(v < 0 || v > (1L << 40)) return -1;
      ++count;
    }
    if(count != 22 || !in.eof()) return -1;
    lines.push_back({line.substr(0,tab),value});
  }
  std::lock_guard<std::mutex> g(wisdomMutex);
  for(const auto& kv : lines) wisdomMap[kv.first]=kv.second;
  return (int) lines.size();
}

void Conv::forgetWisdom()
{
  std::lock_guard<std::mutex> g(wisdomMutex);
  wisdomMap.clear();
}

std::string Conv::schedule() const
{
  std::string s;
  for(int d=0; d < 3; ++d) {
    const AxisPlan *a=d < I.dim ? &I.axis[d] : NULL;
    for(int v : {a ? a->tile : 0,a ? a->thr : 0,a ? a->tileB : 0,
                 a ? a->thrB : 0,a ? a->rpc : 0})
      s += std::to_string(v)+" ";
  }
  for(int v : {hostTile,hostThr,hostTileB,hostThrB})
    s += std::to_string(v)+" ";
  s.pop_back();
  return s;
}

// The schedule of a wisdom line, checked against what this plan's launches
// can take (threads 128 or 256, tiles and rows per CTA the tuner would try
// and that fit shared memory); false leaves the plan untouched.
bool Conv::applySchedule(const std::string& text)
{
  std::istringstream in(text);
  long v[19];
  for(long& x : v)
    if(!(in >> x)) return false;
  const int dim=I.dim, prec=I.prec, A=I.A, B=I.B;
  auto thrOk=[](long t) {return t == 128 || t == 256;};
  auto p2=[](long t) {return t >= 1 && (t & (t-1)) == 0;};
  AxisPlan ax[3];
  for(int d=0; d < dim; ++d) ax[d]=I.axis[d];
  for(int d=0; d < dim; ++d) {
    const long *s=v+5*d;
    AxisPlan& a=ax[d];
    if(!thrOk(s[1]) || !thrOk(s[3])) return false;
    a.thr=(int) s[1];
    a.thrB=(int) s[3];
    if(d < dim-1 && !I.longRow) {
      const int tmax=wide(prec) ? 8 : 16;
      if(!p2(s[0]) || !p2(s[2]) || s[0] > tmax || s[2] > tmax) return false;
      size_t sf, sb;
      if(a.kind == KIND_REAL) {
        sf=FGB_BY_PREC(prec,outerRealSmem,a.L,a.N/2,(int) s[0]);
        sb=FGB_BY_PREC(prec,outerRealSmem,a.L,a.N/2,(int) s[2]);
      } else {
        sf=FGB_BY_PREC(prec,outerFwdSmem,a.L,a.m,(int) s[0],(int) (a.p == 1));
        sb=FGB_BY_PREC(prec,outerBwdSmem,a.L,a.m,(int) s[2],(int) a.q,
                       (int) (a.p == 1));
      }
      if(sf > SMEM_MAX || sb > SMEM_MAX) return false;
      a.tile=(int) s[0];
      a.tileB=(int) s[2];
    }
    if(d == dim-1) {
      const long r=s[4];
      if(r != 1 && r != 2 && r != 3 && r != 4 && r != 6 && r != 8)
        return false;
      const size_t need=I.longRow ? rowNeed(prec,I.rowM,I.rowM,A,B,r,1) :
        a.kind == KIND_HERMITIAN ? hermNeed(prec,a.stored,a.N/2,A,r) :
        rowNeed(prec,a.stored,a.m,A,B,r,a.q == 1 && a.stored <= a.m);
      if(need > SMEM_MAX) return false;
      a.rpc=(int) r;
    }
  }
  const long *h=v+15;
  for(int k=0; k < 4; ++k)
    if(h[k] != 0 && !(k % 2 ? thrOk(h[k]) : p2(h[k]) && h[k] <= 16))
      return false;
  for(int d=0; d < dim; ++d) I.axis[d]=ax[d];
  hostTile=(int) h[0]; hostThr=(int) h[1];
  hostTileB=(int) h[2]; hostThrB=(int) h[3];
  return true;
}

Conv *Conv::create(int dim, const int *kinds, const long *L, const long *M,
                   const long *mForce, int A, int B, int mult, int prec,
                   long batch)
{
  if(!autotune)
    return new Conv(dim,kinds,L,M,mForce,A,B,mult,prec,batch);
  const std::string key=wisdomKey(dim,kinds,L,M,mForce,A,B,mult,prec,batch,
                                  residueSearch);
  std::string value;
  {
    std::lock_guard<std::mutex> g(wisdomMutex);
    auto it=wisdomMap.find(key);
    if(it != wisdomMap.end()) value=it->second;
  }
  if(!value.empty()) {
    std::istringstream in(value);
    long mw[3]={0,0,0};
    bool ok=true;
    for(long& m : mw) ok=ok && (bool) (in >> m);
    std::string rest;
    std::getline(in,rest);
    if(ok) {
      try {
        std::unique_ptr<Conv> c(new Conv(dim,kinds,L,M,mw,A,B,mult,prec,batch,
                                         false));
        if(c->applySchedule(rest)) return c.release();
      } catch(std::exception& x) {
        // A record that no longer plans: plan afresh.  Failures of the
        // device (allocations) are the caller's to see.
        const std::string why=x.what();
        if(why.find("allocation") != std::string::npos ||
           why.find("memory") != std::string::npos) throw;
      }
    }
  }
  long mUsed[3]={0,0,0};
  Conv *c=createSearched(dim,kinds,L,M,mForce,A,B,mult,prec,batch,mUsed);
  std::lock_guard<std::mutex> g(wisdomMutex);
  wisdomMap[key]=std::to_string(mUsed[0])+" "+std::to_string(mUsed[1])+" "+
    std::to_string(mUsed[2])+" "+c->schedule();
  return c;
}

Conv *Conv::createSearched(int dim, const int *kinds, const long *L,
                           const long *M, const long *mForce, int A, int B,
                           int mult, int prec, long batch, long *mUsed)
{
  for(int d=0; d < dim && d < 3; ++d) mUsed[d]=mForce ? mForce[d] : 0;
  // A caller's functor is not available at plan time: its plans keep the
  // cost model's residue blocks (the tiles are still timed).
  if(!residueSearch || mult == MULT_USER)
    return new Conv(dim,kinds,L,M,mForce,A,B,mult,prec,batch);
  long mf[3]={0,0,0};
  for(int d=0; d < dim && d < 3; ++d) mf[d]=mForce ? mForce[d] : 0;
  std::unique_ptr<Conv> base(new Conv(dim,kinds,L,M,mf,A,B,mult,prec,batch,
                                      false));
  const ConvInfo I0=base->info();
  std::vector<std::vector<long>> cands(dim);
  bool any=false;
  for(int d=0; d < dim; ++d) {
    const AxisPlan& a=I0.axis[d];
    if(I0.longRow || mf[d] > 0 ||
       (a.kind != KIND_PAD && a.kind != KIND_CENTERED)) continue;
    cands[d]=residueCandidates(a,d < dim-1,prec,A,B);
    any=any || cands[d].size() > 1;
  }
  if(!any) {
    base.reset();
    for(int d=0; d < dim; ++d) mUsed[d]=mf[d];
    return new Conv(dim,kinds,L,M,mf,A,B,mult,prec,batch);
  }

  // Zero-filled scratch arrays, shared by every candidate (the stored
  // layout does not depend on m).
  const size_t bytes=base->elements()*base->elemBytes();
  std::vector<void *> tin(A,NULL), tout(B,NULL);
  cudaStream_t s=NULL;
  cudaEvent_t e0=NULL, e1=NULL;
  bool ok=cudaStreamCreateWithFlags(&s,cudaStreamNonBlocking) == cudaSuccess &&
    cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  for(auto& p : tin)
    ok=ok && devAlloc((void **) &p,bytes) == cudaSuccess &&
      cudaMemsetAsync(p,0,bytes,s) == cudaSuccess;
  for(auto& p : tout) ok=ok && devAlloc((void **) &p,bytes) == cudaSuccess;
  // Best of two timed convolutions after an untimed one (ms), or "never".
  auto timeOf=[&](Conv& c) {
    double best=1e300;
    for(int rep=0; rep < 3 && ok; ++rep) {
      float ms=0;
      if(cudaEventRecord(e0,s) != cudaSuccess ||
         c.run(tin.data(),tout.data(),s) != cudaSuccess ||
         cudaEventRecord(e1,s) != cudaSuccess ||
         cudaStreamSynchronize(s) != cudaSuccess ||
         cudaEventElapsedTime(&ms,e0,e1) != cudaSuccess) {
        cudaGetLastError();
        return 1e300;
      }
      if(rep > 0) best=std::min(best,(double) ms);
    }
    return best;
  };
  double bestT=ok ? timeOf(*base) : 1e300;
  base.reset();
  for(int d=0; d < dim && ok && bestT < 1e300; ++d) {
    if(cands[d].size() < 2) continue;
    for(long m : cands[d]) {
      long trial[3]={mf[0],mf[1],mf[2]};
      trial[d]=m;
      try {
        Conv c(dim,kinds,L,M,trial,A,B,mult,prec,batch,false);
        double t=timeOf(c);
        if(t < 0.97*bestT) {bestT=t; mf[d]=m;}
      } catch(std::exception&) {}     // a candidate that does not plan
    }
  }
  if(s) cudaStreamSynchronize(s);
  cudaGetLastError();
  for(void *p : tin) if(p) cudaFree(p);
  for(void *p : tout) if(p) cudaFree(p);
  if(e0) cudaEventDestroy(e0);
  if(e1) cudaEventDestroy(e1);
  if(s) cudaStreamDestroy(s);
  for(int d=0; d < dim; ++d) mUsed[d]=mf[d];
  return new Conv(dim,kinds,L,M,mf,A,B,mult,prec,batch);
}

void Conv::tune()
{
  // A launch's tunables: one schedule parameter (rows per CTA or column
  // tile) and its threads per CTA, tried as pairs.
  struct Tunable {
    int *param, *thr;
    std::vector<std::pair<int,int>> cands;
    int launch;
  };
  const int thrs[]={128,256};
  std::vector<Tunable> tn;
  const int dim=I.dim, prec=I.prec, A=I.A, B=I.B;
  AxisPlan& in=I.axis[dim-1];
  long nrows=batch;
  for(int d=0; d < dim-1; ++d) nrows *= I.axis[d].rows;

  // Rows per CTA of the innermost-axis kernel.
  {
    Tunable t;
    t.param=&in.rpc;
    t.thr=&in.thr;
    t.launch=I.longRow ? dim : dim-1;
    long avail=I.longRow ? I.rowQ*nrows : nrows;
    for(int r : {1,2,3,4,6,8}) {
      if(r > avail) break;
      size_t need=I.longRow ? rowNeed(prec,I.rowM,I.rowM,A,B,r,1) :
        in.kind == KIND_HERMITIAN ? hermNeed(prec,in.stored,in.N/2,A,r) :
        rowNeed(prec,in.stored,in.m,A,B,r,in.q == 1 && in.stored <= in.m);
      if(need <= SMEM_MAX)
        for(int th : thrs) t.cands.push_back({r,th});
    }
    if(t.cands.size() > 1) tn.push_back(t);
  }
  // Column tiles of the outer-axis kernels (forward and backward).
  if(!I.longRow) {
    for(int d=0; d < dim-1; ++d) {
      AxisPlan& a=I.axis[d];
      long C=1;
      for(int e=d+1; e < dim; ++e) C *= I.axis[e].stored;
      Tunable f, b;
      f.param=&a.tile;
      b.param=&a.tileB;
      f.thr=&a.thr;
      b.thr=&a.thrB;
      f.launch=d;
      b.launch=2*(dim-1)-d;
      for(int t=1; t <= (wide(prec) ? 8 : 16) && t <= C; t *= 2) {
        size_t sf, sb;
        if(a.kind == KIND_REAL) {
          sf=sb=FGB_BY_PREC(prec,outerRealSmem,a.L,a.N/2,t);
        } else {
          sf=FGB_BY_PREC(prec,outerFwdSmem,a.L,a.m,t,(int) (a.p == 1));
          sb=FGB_BY_PREC(prec,outerBwdSmem,a.L,a.m,t,(int) a.q,
                         (int) (a.p == 1));
        }
        for(int th : thrs) {
          if(sf <= SMEM_MAX) f.cands.push_back({t,th});
          if(sb <= SMEM_MAX) b.cands.push_back({t,th});
        }
      }
      if(f.cands.size() > 1) tn.push_back(f);
      if(b.cands.size() > 1) tn.push_back(b);
    }
  }
  if(tn.empty()) return;
  // A MULT_USER plan is timed without its functor (no multiplication).
  struct Tuning {
    bool& f;
    explicit Tuning(bool& f) : f(f) {f=true;}
    ~Tuning() {f=false;}
  } tuningScope(tuning);

  // Scratch arrays (zeros: the kernels' timing does not depend on values).
  const size_t bytes=elements()*elemBytes();
  std::vector<void *> tin(A,NULL), tout(B,NULL);
  cudaStream_t s=NULL;
  bool ok=cudaStreamCreateWithFlags(&s,cudaStreamNonBlocking) == cudaSuccess;
  for(auto& p : tin)
    ok=ok && devAlloc((void **) &p,bytes) == cudaSuccess &&
      cudaMemsetAsync(p,0,bytes,s) == cudaSuccess;
  for(auto& p : tout) ok=ok && devAlloc((void **) &p,bytes) == cudaSuccess;
  const bool wasTiming=timing;
  ok=ok && enableTiming(true) == cudaSuccess;
  std::vector<std::pair<int,int>> keep;
  for(auto& t : tn) keep.push_back({*t.param,*t.thr});
  if(ok) {
    size_t K=0;
    for(auto& t : tn) K=std::max(K,t.cands.size());
    std::vector<std::vector<double>> ms(tn.size(),
                                        std::vector<double>(K,1e300));
    std::vector<double> lt(nlaunch);
    for(size_t k=0; k < K && ok; ++k) {
      for(auto& t : tn) {
        const auto& c=t.cands[std::min(k,t.cands.size()-1)];
        *t.param=c.first;
        *t.thr=c.second;
      }
      for(int rep=0; rep < 3 && ok; ++rep) {
        ok=run(tin.data(),tout.data(),s) == cudaSuccess &&
          cudaStreamSynchronize(s) == cudaSuccess;
        if(!ok || rep == 0) continue;
        std::fill(lt.begin(),lt.end(),0.0);
        collect(lt.data(),nlaunch);
        for(size_t i=0; i < tn.size(); ++i)
          if(k < tn[i].cands.size())
            ms[i][k]=std::min(ms[i][k],lt[tn[i].launch]);
      }
    }
    const size_t e=elemBytes();
    AxisPlan& a0=I.axis[0];
    if(ok)
      for(size_t i=0; i < tn.size(); ++i) {
        size_t bk=0;
        for(size_t k=1; k < tn[i].cands.size(); ++k)
          if(ms[i][k] < ms[i][bk]) bk=k;
        keep[i]=tn[i].cands[bk];
        // The fastest axis-0 tile whose rows are whole 64-byte host lines.
        if(tn[i].param != &a0.tile && tn[i].param != &a0.tileB) continue;
        long hk=-1;
        for(size_t k=0; k < tn[i].cands.size(); ++k)
          if((size_t) tn[i].cands[k].first*e >= 64 &&
             (hk < 0 || ms[i][k] < ms[i][hk])) hk=k;
        if(hk < 0) continue;
        const bool fwd=tn[i].param == &a0.tile;
        (fwd ? hostTile : hostTileB)=tn[i].cands[hk].first;
        (fwd ? hostThr : hostThrB)=tn[i].cands[hk].second;
      }
  }
  // The planner's choice stays wherever timing failed.
  for(size_t i=0; i < tn.size(); ++i) {
    *tn[i].param=keep[i].first;
    *tn[i].thr=keep[i].second;
  }
  timing=wasTiming;
  cudaGetLastError();
  if(s) cudaStreamSynchronize(s);
  for(void *p : tin) if(p) cudaFree(p);
  for(void *p : tout) if(p) cudaFree(p);
  if(s) cudaStreamDestroy(s);
}

Conv::~Conv()
{
  for(cudaEvent_t ev : events) cudaEventDestroy(ev);
  for(cudaEvent_t ev : ready) cudaEventDestroy(ev);
  if(outCopied) cudaEventDestroy(outCopied);
  for(int k=0; k < CHUNKS; ++k) {
    if(outDone[k]) cudaEventDestroy(outDone[k]);
    if(chunkReady[k]) cudaEventDestroy(chunkReady[k]);
    if(chunkDone[k]) cudaEventDestroy(chunkDone[k]);
    if(k > 0 && lanes[k]) cudaStreamDestroy(lanes[k]);
  }
  if(side) cudaStreamDestroy(side);
  for(void *p : bufs) cudaFree(p);
  if(hostIn) cudaFree(hostIn);
  if(hostOut) cudaFree(hostOut);
  if(ffState) cudaFree(ffState);
}

size_t Conv::elemBytes() const   // user-facing element (FP64 in ff mode)
{
  if(I.axis[0].kind == KIND_REAL) return elem(I.prec)/2;
  return elem(I.prec);
}

size_t Conv::elements() const
{
  size_t n=batch;
  for(int d=0; d < I.dim; ++d) n *= I.axis[d].stored;
  return n;
}

void Conv::setStrides(const long *S)
{
  if(!S) {
    isStrided=false;
    return;
  }
  if(I.dim < 2 || batch != 1)
    throw std::runtime_error("strides apply to the outer axes of 2D and 3D "
                             "convolutions");
  const long inner=I.axis[I.dim-1].stored;
  if(S[I.dim-2] < inner)
    throw std::runtime_error("the stride of axis "+std::to_string(I.dim-2)+
                             " is less than the "+std::to_string(inner)+
                             " entries of the axis inside it");
  if(I.dim == 3 && S[0] < I.axis[1].L*S[1])
    throw std::runtime_error("the stride of axis 0 is less than Ly times "
                             "the stride of axis 1");
  bool dense=S[I.dim-2] == inner && (I.dim == 2 || S[0] == I.axis[1].L*S[1]);
  for(int d=0; d < I.dim-1; ++d) strideS[d]=S[d];
  isStrided=!dense;
  if(hostIn) {                     // host copies are now sized by the span
    cudaFree(hostIn);
    hostIn=NULL;
  }
}

size_t Conv::spanElements() const
{
  if(!isStrided) return elements();
  return (size_t) I.axis[0].L*(size_t) strideS[0];
}

void Conv::allocate()
{
  size_t e=elem(I.prec);
  int A=I.A;
  if(I.prec == PREC_FF) {
    if(devAlloc((void **) &ffState,32*sizeof(int)) != cudaSuccess ||
       cudaMemset(ffState,0,32*sizeof(int)) != cudaSuccess) {
      ffState=NULL;
      throw std::runtime_error("device allocation of the range guard's "
                               "state failed");
    }
  }
  auto get=[&](size_t bytes) {
    void *p=NULL;
    if(devAlloc((void **) &p,bytes) != cudaSuccess)
      throw std::runtime_error("device allocation of "+std::to_string(bytes)+
                               " bytes failed");
    bufs.push_back(p);
    staging += bytes;
  };
  if(I.dim == 1) {
    nlaunch=1;
  } else if(I.dim == 2) {
    size_t rows=I.axis[0].rows;
    size_t C=I.axis[1].stored;
    for(int a=0; a < A; ++a) get(e*rows*C);
    nlaunch=3;
  } else {
    size_t rx=I.axis[0].rows, ry=I.axis[1].rows;
    size_t Ly=I.axis[1].L, nz=I.axis[2].stored;
    for(int a=0; a < A; ++a) get(e*rx*Ly*nz);
    for(int a=0; a < A; ++a) get(e*rx*ry*nz);
    nlaunch=5;
  }
  if(I.longRow) {
    // Long rows: A column-transformed copies of every inner row, N each;
    // two more launches (the column kernels around the row kernel).
    size_t rows=batch;
    for(int d=0; d < I.dim-1; ++d) rows *= I.axis[d].rows;
    longBuf=bufs.size();
    for(int a=0; a < A; ++a) get(e*rows*(size_t) I.axis[I.dim-1].N);
    nlaunch += 2;
  }
}

int Conv::launches() const {return nlaunch;}

cudaError_t Conv::enableTiming(bool on)
{
  timing=on;
  if(on && events.empty()) {
    events.resize(nlaunch+1);
    for(auto& ev : events) {
      cudaError_t e=cudaEventCreate(&ev);
      if(e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

void Conv::tick(cudaStream_t s)
{
  if(timing && marks < (int) events.size()) cudaEventRecord(events[marks++],s);
}

int Conv::collect(double *ms, int n)
{
  int k=std::min(n,marks-1);
  for(int i=0; i < k; ++i) {
    float t=0;
    if(cudaEventElapsedTime(&t,events[i],events[i+1]) == cudaSuccess)
      ms[i] += t;
  }
  return k;
}

// ---------------------------------------------------------------------------
// Launch sequences.

template<typename T>
cudaError_t Conv::runT(const void *const *in, void *const *out, cudaStream_t s)
{
  typedef cplx<T> Cx;
  const int A=I.A, B=I.B;
  const int threads=256;
  cudaError_t e;
  double scale=1.0;
  if(normalize)
    for(int d=0; d < I.dim; ++d) scale /= (double) I.axis[d].N;
  // Float-float mode: the first launch reads the caller's FP64 arrays and
  // the last one writes them, scaled by the range guard's exponents, which
  // a scan of the inputs sets first (its time counts with the first
  // launch's).
  const int IN64=std::is_same<T,ff>::value ? 1 : 0, OUT64=2*IN64;
  const int *guard=NULL;
  if(IN64 && rangeGuard && ffState && I.mult != MULT_USER) {
    FFScaleArgs G;
    for(int a=0; a < A; ++a) G.in[a]=(const unsigned long long *) in[a];
    G.count=A; G.B=B; G.mult=I.mult;
    G.n=(long long) (elements()*(I.axis[0].kind == KIND_REAL ? 1 : 2));
    G.state=ffState;
    if(isStrided) G.n=(long long) (spanElements()*
                                   (I.axis[0].kind == KIND_REAL ? 1 : 2));
    if((e=launchFFScale(G,s)) != cudaSuccess) return e;
    guard=ffState+16;
  }
  // Slot positions for position-dependent (caller's) multipliers.
  IndexMap im;
  std::memset(&im,0,sizeof(im));
  im.dim=I.dim;
  for(int d=0; d < I.dim; ++d) im.N[d]=(int) I.axis[d].N;
  im.real0=I.dim > 1 && I.axis[0].kind == KIND_REAL;
  im.rowsY=I.dim == 3 ? I.axis[1].rows : 1;
  if(I.mult == MULT_USER) {
    for(int d=0; d < I.dim-1; ++d) {
      const AxisPlan& a=I.axis[d];
      im.m[d]=(int) a.m;
      im.q[d]=(int) a.q;
      im.rev[d]=inplaceFFT<T>() && a.kind != KIND_REAL && a.p == 1;
      if(im.rev[d]) {
        FFTPlanDev f=fftPlan(a.m,I.prec,true,true);   // as outerPlan
        im.nst[d]=f.nst;
        for(int k=0; k < f.nst; ++k) im.radix[d][k]=(unsigned char) f.radix[k];
      }
    }
    if(I.longRow) im.longQ=(int) I.rowQ;    // long rows: k = k1 + q k2
  }
  auto rowPlan=[&](RowPlan<T>& P, const AxisPlan& a) {
    P.im=im;
    P.ioShift=guard;
    P.L=(int) a.stored; P.m=(int) a.m; P.q=(int) a.q; P.N=(int) a.N;
    P.cshift=a.cshift; P.A=A; P.B=B; P.mult=I.mult;
    P.realIO=a.kind == KIND_REAL && I.dim == 1;
    P.rpc=I.axis[I.dim-1].rpc;
    P.io64=0;
    P.direct=a.q == 1 && a.stored <= a.m;
    P.fp=fftPlan(a.m,I.prec,inplaceFFT<T>() || P.direct,true);
    P.twN=(const typename TwT<T>::type *) twiddles(a.N,I.prec);
  };
  auto hermPlan=[&](HermRowPlan<T>& P, const AxisPlan& a) {
    P.im=im;
    P.ioShift=guard;
    P.H=(int) a.stored; P.N=(int) a.N; P.Nh=(int) (a.N/2);
    P.A=A; P.B=B; P.mult=I.mult;
    P.rpc=a.rpc;
    P.io64=0;
    P.fp=fftPlan(a.N/2,I.prec,inplaceFFT<T>(),true);
    P.twN=(const typename TwT<T>::type *) twiddles(a.N,I.prec);
  };
  auto outerPlan=[&](OuterPlan<T>& P, const AxisPlan& a) {
    P.ioShift=guard;
    P.L=(int) a.L; P.m=(int) a.m; P.q=(int) a.q; P.N=(int) a.N;
    P.cshift=a.cshift; P.tile=a.tile;
    P.io64=0;
    P.inplace=inplaceFFT<T>() && a.kind != KIND_REAL && a.p == 1;
    P.conj=0;
    P.fp=fftPlan(a.kind == KIND_REAL ? a.N/2 : a.m,I.prec,P.inplace != 0,
                 true);
    P.twN=(const typename TwT<T>::type *) twiddles(a.N,I.prec);
    P.twX=NULL; P.NX=1;
  };
  // The first outer-axis launch.  While a host call copies the inputs in
  // (chunks > 0): input 0 one launch per column range, each on its own
  // stream after its range has landed, and every other input one launch
  // after its copy; the call's stream then joins the range streams.  With
  // per-launch timing on, one launch after every copy.
  auto firstOuter=[&](OuterPlan<T>& O, const AxisPlan& a) {
    auto go=[&](OuterPlan<T>& Q, cudaStream_t st) {
      return a.kind == KIND_REAL ? launchOuterRealFwd<T>(Q,a.thr,st) :
        launchOuterFwd<T>(Q,a.thr,st);
    };
    if(!chunks) return go(O,s);
    cudaError_t e;
    if(timing) {
      for(int k=0; k < chunks; ++k)
        if((e=cudaStreamWaitEvent(s,chunkReady[k],0)) != cudaSuccess) return e;
      for(int i=1; i < A; ++i)
        if((e=cudaStreamWaitEvent(s,ready[i],0)) != cudaSuccess) return e;
      return go(O,s);
    }
    OuterPlan<T> Q=O;
    Q.count=1;
    const size_t eb=elemBytes();       // the caller's element on the input side
    for(int k=0; k < chunks; ++k) {
      cudaStream_t st=k == 0 ? s : lanes[k];
      const long c0=chunkCol[k];
      if((e=cudaStreamWaitEvent(st,chunkReady[k],0)) != cudaSuccess) return e;
      Q.in[0]=(const Cx *) ((const char *) O.in[0]+c0*eb);
      Q.out[0]=O.out[0]+c0;
      Q.C=(int) (chunkCol[k+1]-c0);
      if((e=go(Q,st)) != cudaSuccess) return e;
      if(k > 0 && (e=cudaEventRecord(chunkDone[k],st)) != cudaSuccess) return e;
    }
    Q.C=O.C;
    for(int i=1; i < A; ++i) {
      if((e=cudaStreamWaitEvent(s,ready[i],0)) != cudaSuccess) return e;
      Q.in[0]=O.in[i];
      Q.out[0]=O.out[i];
      if((e=go(Q,s)) != cudaSuccess) return e;
    }
    for(int k=1; k < chunks; ++k)
      if((e=cudaStreamWaitEvent(s,chunkDone[k],0)) != cudaSuccess) return e;
    return cudaSuccess;
  };

  // The last outer-axis launch.  While a host call copies the outputs out
  // (outChunks > 0, complex outer axis): one launch per column range, each
  // followed by the event its copy waits for.
  auto lastOuter=[&](OuterPlan<T>& O, const AxisPlan& a) {
    if(a.kind == KIND_REAL) return launchOuterRealBwd<T>(O,a.thrB,s);
    if(!outChunks || timing) return launchOuterBwd<T>(O,a.thrB,s);
    OuterPlan<T> Q=O;
    const size_t eb=elemBytes();       // the caller's element on the output side
    cudaError_t e;
    for(int k=0; k < outChunks; ++k) {
      const long c0=outCol[k];
      Q.C=(int) (outCol[k+1]-c0);
      for(int i=0; i < O.count; ++i) {
        Q.in[i]=O.in[i]+c0;
        Q.out[i]=(Cx *) ((char *) O.out[i]+c0*eb);
      }
      if((e=launchOuterBwd<T>(Q,a.thrB,s)) != cudaSuccess ||
         (e=cudaEventRecord(outDone[k],s)) != cudaSuccess) return e;
    }
    return cudaSuccess;
  };

  if(I.dim == 1 && !I.longRow) {
    const AxisPlan& a=I.axis[0];
    if(a.kind == KIND_HERMITIAN) {
      HermRowPlan<T> P{};
      hermPlan(P,a);
      for(int i=0; i < A; ++i) P.in[i]=(const Cx *) in[i];
      for(int i=0; i < B; ++i) P.out[i]=(Cx *) out[i];
      P.rowStride=a.stored; P.nrows=batch; P.scale=(T) scale;
      P.io64=IN64 | OUT64;
      e=hermLaunch<T>(P,a.thr,batch,s);
      tick(s);
      return e;
    }
    RowPlan<T> P{};
    rowPlan(P,a);
    for(int i=0; i < A; ++i) P.in[i]=(const Cx *) in[i];
    for(int i=0; i < B; ++i) P.out[i]=(Cx *) out[i];
    P.rowStride=a.stored; P.nrows=batch; P.scale=(T) scale;
    P.io64=IN64 | OUT64;
    e=rowLaunch<T>(P,a.thr,batch,s);
    tick(s);
    return e;
  }

  if(I.dim == 1)             // long 1D rows
    return runLong<T>(in,out,batch,I.axis[0].stored,IN64 | OUT64,guard,&im,
                      scale,s);

  if(I.dim == 2) {
    const AxisPlan& ax=I.axis[0];
    const AxisPlan& ay=I.axis[1];
    long C=ay.stored;
    OuterPlan<T> O{};
    outerPlan(O,ax);
    O.count=A; O.nbatch=1; O.inBatch=O.outBatch=0;
    O.inRow=C; O.outRow=C; O.C=(int) C; O.Ltot=(long long) ax.L*C;
    if(isStrided) {                 // data side (the caller's arrays)
      O.inRow=strideS[0];
      O.Ltot=LLONG_MAX;
    }
    O.scale=(T) 1;
    O.io64=IN64;
    for(int i=0; i < A; ++i) {O.in[i]=(const Cx *) in[i]; O.out[i]=(Cx *) bufs[i];}
    e=firstOuter(O,ax);
    tick(s);
    if(e != cudaSuccess) return e;
    if(I.longRow) {
      e=runLong<T>((const void *const *) bufs.data(),bufs.data(),ax.rows,C,0,
                   NULL,&im,1.0,s);
    } else if(ay.kind == KIND_HERMITIAN) {
      HermRowPlan<T> P{};
      hermPlan(P,ay);
      for(int i=0; i < A; ++i) P.in[i]=(const Cx *) bufs[i];
      for(int i=0; i < B; ++i) P.out[i]=(Cx *) bufs[i];
      P.rowStride=C; P.nrows=ax.rows; P.scale=(T) 1;
      e=hermLaunch<T>(P,ay.thr,ax.rows,s);
      tick(s);
    } else {
      RowPlan<T> P{};
      rowPlan(P,ay);
      for(int i=0; i < A; ++i) P.in[i]=(const Cx *) bufs[i];
      for(int i=0; i < B; ++i) P.out[i]=(Cx *) bufs[i];
      P.rowStride=C; P.nrows=ax.rows; P.scale=(T) 1;
      e=rowLaunch<T>(P,ay.thr,ax.rows,s);
      tick(s);
    }
    if(e != cudaSuccess) return e;
    O.count=B;
    O.tile=ax.tileB;
    O.scale=(T) scale;
    O.io64=OUT64;
    O.inRow=C;                                  // staging side
    O.outRow=isStrided ? strideS[0] : C;        // data side
    for(int i=0; i < B; ++i) {O.in[i]=(const Cx *) bufs[i]; O.out[i]=(Cx *) out[i];}
    e=lastOuter(O,ax);
    tick(s);
    return e;
  }

  // dim == 3
  const AxisPlan& ax=I.axis[0];
  const AxisPlan& ay=I.axis[1];
  const AxisPlan& az=I.axis[2];
  long nz=az.stored;
  long Cx_=ay.L*nz;
  void **bx=bufs.data();
  void **by=bufs.data()+A;

  OuterPlan<T> X{};
  outerPlan(X,ax);
  X.count=A; X.nbatch=1; X.inBatch=X.outBatch=0;
  X.inRow=Cx_; X.outRow=Cx_; X.C=(int) Cx_; X.Ltot=(long long) ax.L*Cx_;
  X.scale=(T) 1;
  X.io64=IN64;
  if(isStrided) {                   // data side (the caller's arrays)
    X.inRow=strideS[0];
    X.Ltot=LLONG_MAX;
    if(strideS[1] != nz) {X.cz=(int) nz; X.cs=strideS[1];}
  }
  for(int i=0; i < A; ++i) {X.in[i]=(const Cx *) in[i]; X.out[i]=(Cx *) bx[i];}
  e=firstOuter(X,ax);
  tick(s);
  if(e != cudaSuccess) return e;

  OuterPlan<T> Y{};
  outerPlan(Y,ay);
  Y.count=A; Y.nbatch=(int) ax.rows;
  Y.inBatch=ay.L*nz; Y.outBatch=ay.rows*nz;
  Y.inRow=nz; Y.outRow=nz; Y.C=(int) nz; Y.Ltot=(long long) ay.L*nz;
  Y.scale=(T) 1;
  for(int i=0; i < A; ++i) {Y.in[i]=(const Cx *) bx[i]; Y.out[i]=(Cx *) by[i];}
  e=launchOuterFwd<T>(Y,ay.thr,s);
  tick(s);
  if(e != cudaSuccess) return e;

  long nrows=ax.rows*ay.rows;
  if(I.longRow) {
    e=runLong<T>((const void *const *) by,by,nrows,nz,0,NULL,&im,1.0,s);
  } else if(az.kind == KIND_HERMITIAN) {
    HermRowPlan<T> P{};
    hermPlan(P,az);
    for(int i=0; i < A; ++i) P.in[i]=(const Cx *) by[i];
    for(int i=0; i < B; ++i) P.out[i]=(Cx *) by[i];
    P.rowStride=nz; P.nrows=nrows; P.scale=(T) 1;
    e=hermLaunch<T>(P,az.thr,nrows,s);
    tick(s);
  } else {
    RowPlan<T> P{};
    rowPlan(P,az);
    for(int i=0; i < A; ++i) P.in[i]=(const Cx *) by[i];
    for(int i=0; i < B; ++i) P.out[i]=(Cx *) by[i];
    P.rowStride=nz; P.nrows=nrows; P.scale=(T) 1;
    e=rowLaunch<T>(P,az.thr,nrows,s);
    tick(s);
  }
  if(e != cudaSuccess) return e;

  Y.count=B;
  Y.tile=ay.tileB;
  for(int i=0; i < B; ++i) {Y.in[i]=(const Cx *) by[i]; Y.out[i]=(Cx *) bx[i];}
  std::swap(Y.inBatch,Y.outBatch);
  e=launchOuterBwd<T>(Y,ay.thrB,s);
  tick(s);
  if(e != cudaSuccess) return e;

  X.count=B;
  X.tile=ax.tileB;
  X.scale=(T) scale;
  X.io64=OUT64;
  X.inRow=Cx_;                                  // staging side
  X.outRow=isStrided ? strideS[0] : Cx_;        // data side
  for(int i=0; i < B; ++i) {X.in[i]=(const Cx *) bx[i]; X.out[i]=(Cx *) out[i];}
  e=lastOuter(X,ax);
  tick(s);
  return e;
}

template<typename T>
cudaError_t Conv::runLong(const void *const *in, void *const *out,
                          long long nrows, long long rowStride, int io64,
                          const int *guard, const IndexMap *im, double scale,
                          cudaStream_t s)
{
  typedef cplx<T> Cx;
  const AxisPlan& a=I.axis[I.dim-1];
  const int A=I.A, B=I.B;
  const long m=I.rowM, q=I.rowQ, N=a.N;
  void *const *lb=bufs.data()+longBuf;
  const int flat=a.kind == KIND_CENTERED ? FLAT_CENTERED :
    a.kind == KIND_HERMITIAN ? FLAT_HERMITIAN :
    a.kind == KIND_REAL ? FLAT_REAL : FLAT_PAD;
  const int threads=256;
  cudaError_t e;
  // Columns of length q over the q x m view of every row, with the
  // W_N^{col k} twiddle (explicit padding of the row to N).
  OuterPlan<T> O{};
  O.L=(int) (flat == FLAT_PAD || flat == FLAT_REAL ? a.p : q);
  O.m=(int) q; O.q=1; O.N=(int) q; O.cshift=0;
  O.tile=a.tile;
  O.fp=fftPlan(q,I.prec);
  O.twN=(const typename TwT<T>::type *) twiddles(q,I.prec);
  O.twX=(const typename TwT<T>::type *) twiddles(N,I.prec);
  O.NX=N;
  O.io64=io64 & 1; O.ioShift=guard;
  O.inplace=0; O.conj=0;
  O.flat=flat; O.flatC=a.cshift;
  O.count=A; O.nbatch=(int) nrows; O.inBatch=rowStride; O.outBatch=N;
  O.inRow=m; O.outRow=m; O.C=(int) m; O.Ltot=a.stored;
  O.scale=(T) 1;
  for(int i=0; i < A; ++i) {O.in[i]=(const Cx *) in[i]; O.out[i]=(Cx *) lb[i];}
  e=launchOuterFwd<T>(O,threads,s);
  tick(s);
  if(e != cudaSuccess) return e;
  // Rows of length m: one residue, one fold (the direct row variant).
  RowPlan<T> P{};
  P.im=*im;
  P.L=(int) m; P.m=(int) m; P.q=1; P.N=(int) m; P.cshift=0;
  P.A=A; P.B=B; P.mult=I.mult; P.realIO=0;
  P.rpc=a.rpc; P.io64=0; P.direct=1; P.ioShift=NULL;
  P.fp=fftPlan(m,I.prec,true,true);
  P.twN=(const typename TwT<T>::type *) twiddles(m,I.prec);
  for(int i=0; i < A; ++i) P.in[i]=(const Cx *) lb[i];
  for(int i=0; i < B; ++i) P.out[i]=(Cx *) lb[i];
  P.rowStride=m; P.nrows=nrows*q; P.scale=(T) 1;
  e=rowLaunch<T>(P,a.thr,nrows*q,s);
  tick(s);
  if(e != cudaSuccess) return e;
  // Inverse columns, back into the rows' stored entries.
  O.count=B;
  O.tile=a.tileB;
  O.io64=io64 & 2;
  O.scale=(T) scale;
  O.inBatch=N; O.outBatch=rowStride;
  for(int i=0; i < B; ++i) {O.in[i]=(const Cx *) lb[i]; O.out[i]=(Cx *) out[i];}
  e=launchOuterBwd<T>(O,threads,s);
  tick(s);
  return e;
}

template<typename T>
cudaError_t Conv::rowLaunch(const RowPlan<T>& P, int thr, long long grid,
                            cudaStream_t s)
{
  return user ? user->row(P,thr,grid,s) : launchRow<T>(P,thr,grid,s);
}

template<typename T>
cudaError_t Conv::hermLaunch(const HermRowPlan<T>& P, int thr, long long grid,
                             cudaStream_t s)
{
  return user ? user->herm(P,thr,grid,s) : launchHermRow<T>(P,thr,grid,s);
}

cudaError_t Conv::checkUser(const RowLaunchers *L)
{
  if(I.mult != MULT_USER) {
    setLastError("this plan has a built-in multiplier; a device functor "
                 "needs a plan made with the user multiplier");
    return cudaErrorInvalidValue;
  }
  if(!L || L->inputs() != I.A || L->outputs() != I.B) {
    setLastError("the functor's inputs and outputs (A, B) differ from the "
                 "plan's");
    return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

cudaError_t Conv::runWith(const RowLaunchers *L, const void *const *in,
                          void *const *out, cudaStream_t s)
{
  cudaError_t e=checkUser(L);
  if(e != cudaSuccess) return e;
  user=L;
  e=run(in,out,s);
  user=NULL;
  return e;
}

cudaError_t Conv::runHostWith(const RowLaunchers *L, const void *const *in,
                              void *const *out, cudaStream_t s)
{
  cudaError_t e=checkUser(L);
  if(e != cudaSuccess) return e;
  user=L;
  e=runHost(in,out,s);
  user=NULL;
  return e;
}

cudaError_t Conv::run(const void *const *in, void *const *out, cudaStream_t s)
{
  if(I.mult == MULT_USER && !user && !tuning) {
    setLastError("this plan multiplies with a caller's device functor: "
                 "convolve through fgb::convolveWith "
                 "(fftwpp_gb300_mult.cuh)");
    return cudaErrorInvalidValue;
  }
  marks=0;
  tick(s);
  if(I.prec == PREC_F64) return runT<double>(in,out,s);
  if(I.prec == PREC_F32) return runT<float>(in,out,s);
  return runT<ff>(in,out,s);        // float-float, FP64 at the interface
}

bool Conv::zeroCopy=true;
void Conv::setZeroCopy(bool on) {zeroCopy=on;}
int Conv::hostPathIn=-1, Conv::hostPathOut=-1;
void Conv::setHostPath(int inputs, int outputs)
{
  auto way=[](int w) {return w < 0 ? -1 : std::min(w,(int) HOST_INPLACE64);};
  hostPathIn=way(inputs);
  hostPathOut=way(outputs);
}

// The device address of page-locked host memory, or NULL for memory the GPU
// cannot address directly.
static void *mappedAddress(const void *p)
{
  cudaPointerAttributes at;
  if(cudaPointerGetAttributes(&at,p) != cudaSuccess) {
    cudaGetLastError();
    return NULL;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : NULL;
}

// Whether the first and last kernels touch the caller's arrays in runs of at
// least 64 contiguous bytes (then they may read and write host memory
// directly without wasting the link's lines).
bool Conv::directSegments() const
{
  const AxisPlan& a=I.axis[0];
  if(I.dim == 1 && !I.longRow) return true;        // whole rows
  size_t e=elemBytes();
  return (size_t) a.tile*e >= 64 && (size_t) a.tileB*e >= 64;
}

// Queues the copies of the inputs (host addresses) into device memory on
// the side stream, after the work already queued on s: input 0 in column
// ranges (2D copies, copy engines) so that its first transform starts on
// the first range, the other inputs whole.  Sets chunks, chunkCol and the
// events the first outer launch waits for.
cudaError_t Conv::pipeInputs(const void *const *in, void *const *dev,
                             cudaStream_t s)
{
  cudaError_t e;
  const int A=I.A;
  auto event=[](cudaEvent_t& ev) {
    return ev ? cudaSuccess :
      cudaEventCreateWithFlags(&ev,cudaEventDisableTiming);
  };
  if(!side && (e=cudaStreamCreateWithFlags(&side,cudaStreamNonBlocking)) !=
     cudaSuccess) {
    side=NULL;
    return e;
  }
  while((int) ready.size() < A+1) {
    cudaEvent_t ev=NULL;
    if((e=event(ev)) != cudaSuccess) return e;
    ready.push_back(ev);
  }
  // Column ranges of input 0, whole forward tiles each.
  const size_t eb=elemBytes(), bytes=elements()*eb;
  const long rows=I.axis[0].L, C=(long) elements()/rows;
  const long unit=std::max(1,I.axis[0].tile);
  const long units=(C+unit-1)/unit;
  const long per=(units+CHUNKS-1)/CHUNKS;
  int n=0;
  chunkCol[0]=0;
  while(chunkCol[n] < C) {
    chunkCol[n+1]=std::min(C,chunkCol[n]+per*unit);
    ++n;
  }
  for(int k=0; k < n; ++k) {
    if((e=event(chunkReady[k])) != cudaSuccess ||
       (e=event(chunkDone[k])) != cudaSuccess) return e;
    if(k > 0 && !lanes[k] &&
       (e=cudaStreamCreateWithFlags(&lanes[k],cudaStreamNonBlocking)) !=
       cudaSuccess) {
      lanes[k]=NULL;
      return e;
    }
  }
  // Copies (and the range streams) follow the work already queued on s.
  if((e=cudaEventRecord(ready[A],s)) != cudaSuccess ||
     (e=cudaStreamWaitEvent(side,ready[A],0)) != cudaSuccess) return e;
  for(int k=0; k < n; ++k) {
    const size_t off=chunkCol[k]*eb;
    if((e=cudaMemcpy2DAsync((char *) dev[0]+off,C*eb,
                            (const char *) in[0]+off,C*eb,
                            (chunkCol[k+1]-chunkCol[k])*eb,rows,
                            cudaMemcpyDefault,side)) != cudaSuccess ||
       (e=cudaEventRecord(chunkReady[k],side)) != cudaSuccess) return e;
  }
  for(int a=1; a < A; ++a)
    if((e=cudaMemcpyAsync(dev[a],in[a],bytes,cudaMemcpyDefault,side)) !=
       cudaSuccess ||
       (e=cudaEventRecord(ready[a],side)) != cudaSuccess) return e;
  chunks=n;
  return cudaSuccess;
}

// One convolution over page-locked arrays: hin the inputs' host addresses
// (for the copy engines), in and out the mapped device addresses.  Each
// side takes its own way over the host link: wayIn for the inputs, wayOut
// for the outputs, HOST_COPY (whole arrays moved through device memory,
// 16-byte aligned), HOST_INPLACE (the first kernel reads, or the
// last one writes, the caller's arrays with the device-tuned axis-0 tiles)
// or HOST_INPLACE64 (the same with the fastest tiles whose rows span at
// least 64 bytes, whole lines of the link).
cudaError_t Conv::runZeroCopy(const void *const *hin, const void *const *in,
                              void *const *hout, void *const *out,
                              int wayIn, int wayOut, cudaStream_t s)
{
  const size_t bytes=elements()*elemBytes();
  const int A=I.A, B=I.B;
  const bool copyIn=wayIn == HOST_COPY, copyOut=wayOut == HOST_COPY;
  if((copyIn || copyOut) && !hostIn &&
     devAlloc((void **) &hostIn,bytes*A) != cudaSuccess)
    return cudaErrorMemoryAllocation;
  std::vector<const void *> src(A);
  std::vector<void *> dst(B);
  for(int a=0; a < A; ++a)
    src[a]=copyIn ? (const void *) ((char *) hostIn+a*bytes) : in[a];
  for(int b=0; b < B; ++b)
    dst[b]=copyOut ? (void *) ((char *) hostIn+b*bytes) : out[b];
  CopyArgs C;
  C.bytes=bytes;
  cudaError_t e;
  // With an outer axis, the inputs are copied on a side stream and the
  // first transform of each piece starts as soon as it has arrived.
  // (Float-float plans scan all inputs before the first transform, so
  // their inputs arrive whole.)
  const bool pipeline=copyIn && I.dim > 1 && !I.longRow &&
    !(I.prec == PREC_FF && rangeGuard);
  if(pipeline) {
    std::vector<void *> dev(A);
    for(int a=0; a < A; ++a) dev[a]=(void *) src[a];
    if((e=pipeInputs(hin,dev.data(),s)) != cudaSuccess) {
      chunks=0;
      return e;
    }
  } else if(copyIn) {
    C.count=A;
    for(int a=0; a < A; ++a) {C.src[a]=in[a]; C.dst[a]=(void *) src[a];}
    if((e=launchBulkCopy(C,s)) != cudaSuccess) return e;
  }
  AxisPlan& a0=I.axis[0];
  const int keep[4]={a0.tile,a0.thr,a0.tileB,a0.thrB};
  if(wayIn == HOST_INPLACE64 && hostTile) {a0.tile=hostTile; a0.thr=hostThr;}
  if(wayOut == HOST_INPLACE64 && hostTileB) {
    a0.tileB=hostTileB; a0.thrB=hostThrB;
  }
  // With a complex outer axis the outputs leave in column ranges (2D
  // copies on the side stream, copy engines), each as soon as the last
  // transform has written it.
  const bool pipeOut=copyOut && I.dim > 1 && !I.longRow &&
    I.axis[0].kind != KIND_REAL;
  if(pipeOut && (e=planOutputs(s)) != cudaSuccess) return e;
  e=run(src.data(),dst.data(),s);
  chunks=0;
  const int nOut=outChunks;
  outChunks=0;
  a0.tile=keep[0]; a0.thr=keep[1];
  a0.tileB=keep[2]; a0.thrB=keep[3];
  if(e != cudaSuccess || !copyOut) return e;
  if(pipeOut && !timing) {
    const size_t eb=elemBytes();
    const long rows=I.axis[0].L, Cn=(long) elements()/rows;
    for(int k=0; k < nOut; ++k) {
      const size_t off=outCol[k]*eb;
      if((e=cudaStreamWaitEvent(side,outDone[k],0)) != cudaSuccess) return e;
      for(int b=0; b < B; ++b)
        if((e=cudaMemcpy2DAsync((char *) hout[b]+off,Cn*eb,
                                (const char *) dst[b]+off,Cn*eb,
                                (outCol[k+1]-outCol[k])*eb,rows,
                                cudaMemcpyDefault,side)) != cudaSuccess)
          return e;
    }
    if((e=cudaEventRecord(outCopied,side)) != cudaSuccess) return e;
    return cudaStreamWaitEvent(s,outCopied,0);
  }
  C.count=B;
  for(int b=0; b < B; ++b) {C.src[b]=dst[b]; C.dst[b]=out[b];}
  return launchBulkCopy(C,s);
}

// Column ranges of the last outer transform for a host call's output
// copies (whole backward tiles each), their events and the side stream.
cudaError_t Conv::planOutputs(cudaStream_t s)
{
  cudaError_t e;
  auto event=[](cudaEvent_t& ev) {
    return ev ? cudaSuccess :
      cudaEventCreateWithFlags(&ev,cudaEventDisableTiming);
  };
  if(!side && (e=cudaStreamCreateWithFlags(&side,cudaStreamNonBlocking)) !=
     cudaSuccess) {
    side=NULL;
    return e;
  }
  if((e=event(outCopied)) != cudaSuccess) return e;
  const long rows=I.axis[0].L, C=(long) elements()/rows;
  const long unit=std::max(1,I.axis[0].tileB);
  const long units=(C+unit-1)/unit;
  const long per=(units+OUT_CHUNKS-1)/OUT_CHUNKS;
  int n=0;
  outCol[0]=0;
  while(outCol[n] < C) {
    outCol[n+1]=std::min(C,outCol[n]+per*unit);
    if((e=event(outDone[n])) != cudaSuccess) return e;
    ++n;
  }
  outChunks=n;
  return cudaSuccess;
}

// Times every combination of input and output ways on page-locked scratch
// arrays of this plan's size (the best of three runs each, after one
// untimed) and keeps the fastest; whole-array copies both ways if timing
// fails.  The host writes the inputs before every timed run, as a caller
// producing new data does, so the link reads lines the CPU holds dirty
// (up to DIRTY_MAX bytes; larger plans time clean lines rather than spend
// seconds rewriting them before every run).
static const size_t DIRTY_MAX=(size_t) 512 << 20;

void Conv::measureHostPath(cudaStream_t s)
{
  hostWay[0]=hostWay[1]=HOST_COPY;
  const size_t bytes=elements()*elemBytes();
  const size_t stride=(bytes+255)/256*256;
  const int n=std::max(I.A,I.B);
  void *h=NULL;
  if(cudaHostAlloc(&h,stride*n,cudaHostAllocMapped) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  std::memset(h,0,stride*n);
  void *d=mappedAddress(h);
  std::vector<const void *> hin(I.A), in(I.A);
  std::vector<void *> hout(I.B), out(I.B);
  for(int a=0; a < I.A; ++a) {
    hin[a]=(char *) h+a*stride;
    in[a]=(char *) d+a*stride;
  }
  for(int b=0; b < I.B; ++b) {
    hout[b]=(char *) h+b*stride;
    out[b]=(char *) d+b*stride;
  }
  std::vector<std::pair<int,int>> ways;
  for(int wi=HOST_COPY; wi <= HOST_INPLACE64; ++wi)
    for(int wo=HOST_COPY; wo <= HOST_INPLACE64; ++wo)
      if((wi != HOST_INPLACE64 || hostTile) &&
         (wo != HOST_INPLACE64 || hostTileB)) ways.push_back({wi,wo});
  cudaEvent_t e0=NULL, e1=NULL;
  bool ok=d && cudaEventCreate(&e0) == cudaSuccess &&
    cudaEventCreate(&e1) == cudaSuccess;
  ok=ok && runZeroCopy(hin.data(),in.data(),hout.data(),out.data(),HOST_COPY,
                       HOST_COPY,s) ==
    cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess;
  double best=1e300;
  for(int rep=0; rep < 3 && ok; ++rep)
    for(const auto& w : ways) {
      if(stride*n <= DIRTY_MAX) std::memset(h,0,stride*n);
      ok=cudaEventRecord(e0,s) == cudaSuccess &&
        runZeroCopy(hin.data(),in.data(),hout.data(),out.data(),w.first,
                    w.second,s) ==
        cudaSuccess &&
        cudaEventRecord(e1,s) == cudaSuccess &&
        cudaStreamSynchronize(s) == cudaSuccess;
      float ms=0;
      if(!ok || cudaEventElapsedTime(&ms,e0,e1) != cudaSuccess) break;
      if(ms < best) {
        best=ms;
        hostWay[0]=w.first;
        hostWay[1]=w.second;
      }
    }
  if(!ok) hostWay[0]=hostWay[1]=HOST_COPY;
  cudaStreamSynchronize(s);
  if(e0) cudaEventDestroy(e0);
  if(e1) cudaEventDestroy(e1);
  cudaFreeHost(h);
  cudaGetLastError();
}

void Conv::hostPath(int *inputs, int *outputs) const
{
  int wi=hostWay[0], wo=hostWay[1];
  if(hostPathIn >= 0 && hostPathOut >= 0) {wi=hostPathIn; wo=hostPathOut;}
  else if(directSegments()) wi=wo=HOST_INPLACE;
  if(inputs) *inputs=wi;
  if(outputs) *outputs=wo;
}

// Host arrays in a strided layout: page-locked ones are read and written
// in place by the first and last kernels; other host memory is copied in
// whole (gaps included) and the stored entries copied back row by row, so
// that the gaps of separate output arrays stay untouched.
cudaError_t Conv::runHostStrided(const void *const *in, void *const *out,
                                 cudaStream_t s)
{
  const int A=I.A, B=I.B;
  const size_t eb=elemBytes(), span=spanElements()*eb;
  if(zeroCopy) {
    std::vector<const void *> min(A);
    std::vector<void *> mout(B);
    bool ok=true;
    for(int a=0; a < A && ok; ++a) ok=(min[a]=mappedAddress(in[a])) != NULL;
    for(int b=0; b < B && ok; ++b) ok=(mout[b]=mappedAddress(out[b])) != NULL;
    if(ok) {
      cudaError_t e=run(min.data(),mout.data(),s);
      return e != cudaSuccess ? e : cudaStreamSynchronize(s);
    }
  }
  if(!hostIn && devAlloc((void **) &hostIn,span*A) != cudaSuccess)
    return cudaErrorMemoryAllocation;
  std::vector<void *> din(A);
  cudaError_t e;
  for(int a=0; a < A; ++a) {
    din[a]=(char *) hostIn+a*span;
    if((e=cudaMemcpyAsync(din[a],in[a],span,cudaMemcpyHostToDevice,s)) !=
       cudaSuccess) return e;
  }
  if((e=run(din.data(),din.data(),s)) != cudaSuccess) return e;
  // Stored rows: of the innermost axis (3D: per plane of axis 0).
  const size_t inner=(size_t) I.axis[I.dim-1].stored*eb;
  const long planes=I.dim == 3 ? I.axis[0].L : 1;
  const long rows=I.dim == 3 ? I.axis[1].L : I.axis[0].L;
  const size_t pitch=(size_t) strideS[I.dim-2]*eb;
  const size_t plane=(size_t) strideS[0]*eb;
  for(int b=0; b < B; ++b)
    for(long k=0; k < planes; ++k)
      if((e=cudaMemcpy2DAsync((char *) out[b]+k*plane,pitch,
                              (const char *) din[b]+k*plane,pitch,inner,rows,
                              cudaMemcpyDeviceToHost,s)) != cudaSuccess)
        return e;
  return cudaStreamSynchronize(s);
}

cudaError_t Conv::runHost(const void *const *in, void *const *out,
                          cudaStream_t s)
{
  if(isStrided) return runHostStrided(in,out,s);
  size_t bytes=elements()*elemBytes();
  int A=I.A, B=I.B;
  if(zeroCopy) {
    // Page-locked arrays are addressed directly by the kernels.
    std::vector<const void *> min(A);
    std::vector<void *> mout(B);
    bool ok=true;
    for(int a=0; a < A && ok; ++a) ok=(min[a]=mappedAddress(in[a])) != NULL;
    for(int b=0; b < B && ok; ++b) ok=(mout[b]=mappedAddress(out[b])) != NULL;
    for(int a=0; a < A && ok; ++a) ok=(size_t) min[a] % elemBytes() == 0;
    for(int b=0; b < B && ok; ++b) ok=(size_t) mout[b] % elemBytes() == 0;
    if(ok) {
      bool aligned=bytes % 16 == 0;
      for(int a=0; a < A; ++a) aligned=aligned && (size_t) min[a] % 16 == 0;
      for(int b=0; b < B; ++b) aligned=aligned && (size_t) mout[b] % 16 == 0;
      int wi, wo;
      if(hostPathIn >= 0 && hostPathOut >= 0) {
        wi=hostPathIn;
        wo=hostPathOut;
      } else if(directSegments()) {
        wi=wo=HOST_INPLACE;                 // whole lines already
      } else {
        if(hostWay[0] < 0) measureHostPath(s);
        wi=hostWay[0];
        wo=hostWay[1];
      }
      if(!aligned) {                        // the SM copies move 16-byte units
        if(wi == HOST_COPY) wi=HOST_INPLACE;
        if(wo == HOST_COPY) wo=HOST_INPLACE;
      }
      cudaError_t e=runZeroCopy(in,min.data(),out,mout.data(),wi,wo,s);
      return e != cudaSuccess ? e : cudaStreamSynchronize(s);
    }
  }
  if(!hostIn) {
    if(devAlloc((void **) &hostIn,bytes*A) != cudaSuccess) return cudaErrorMemoryAllocation;
  }
  std::vector<void *> din(A), dout(B);
  for(int a=0; a < A; ++a) {
    din[a]=(char *) hostIn+a*bytes;
    cudaError_t e=cudaMemcpyAsync(din[a],in[a],bytes,cudaMemcpyHostToDevice,s);
    if(e != cudaSuccess) return e;
  }
  for(int b=0; b < B; ++b) dout[b]=din[b];
  cudaError_t e=run(din.data(),dout.data(),s);
  if(e != cudaSuccess) return e;
  for(int b=0; b < B; ++b) {
    e=cudaMemcpyAsync(out[b],dout[b],bytes,cudaMemcpyDeviceToHost,s);
    if(e != cudaSuccess) return e;
  }
  return cudaStreamSynchronize(s);
}

// ---------------------------------------------------------------------------
// Standalone padded transform (engine.h).

PadTransform::PadTransform(int kind, long L, long M, long C, long mForce,
                           int prec) : C(C), prec(prec)
{
  if(kind < KIND_PAD || kind > KIND_REAL)
    throw std::runtime_error("unknown padded-transform kind");
  if(prec != PREC_F64 && prec != PREC_F32)
    throw std::runtime_error("standalone padded transforms run in FP64 or "
                             "FP32");
  if(L < 1 || C < 1) throw std::runtime_error("L and C must be positive");
  if(L > M)
    throw std::runtime_error("L="+std::to_string(L)+" is greater than M="+
                             std::to_string(M));
  if(L*C > (long) INT_MAX || M*C > (long) INT_MAX)
    throw std::runtime_error("transform too large");
  a.kind=kind; a.L=L; a.M=M; a.stored=L; a.tile=a.tileB=1; a.rpc=1;
  a.rows=0;
  if(kind == KIND_HERMITIAN) {
    // Explicit padding to an even N: the ceil(L/2) stored modes to N real
    // values and back (fftPadHermitian with m = N, D = 1; a forced m gives
    // the N = m q of the reference's parameters, convolve.cc:403-410).
    long Mh=M;
    if(mForce > 0) {
      size_t p,n,q;
      refParameters(L,M,mForce,true,p,n,q);
      Mh=std::max<long>(M,mForce*(long) q);
    }
    a.stored=(long) ceilquotient(L,2);
    a.N=evenSmooth(Mh);
    a.m=a.N; a.q=1; a.p=1; a.cshift=0;
    a.rows=a.N;
    const long Nh=a.N/2;
    auto sm=[&](int t) {return FGB_BY_PREC(prec,outerRealSmem,a.N,Nh,t);};
    if(sm(1) > SMEM_MAX)
      throw std::runtime_error("transform too long for one CTA's shared "
                               "memory");
    a.tile=pickTile(wide(prec) ? 8 : 16,C,1,sm,wide(prec) ? 2 : 4);
    a.tileB=a.tile;
    return;
  }
  planOuter(a,mForce,prec,C,1,1,1);
}

size_t PadTransform::inElements() const {return (size_t) a.stored*C;}
size_t PadTransform::outElements() const {return (size_t) a.rows*C;}

bool PadTransform::aligned(const void *f, const void *F) const
{
  size_t cplx=elem(prec), data=a.kind == KIND_REAL ? cplx/2 : cplx;
  size_t trans=a.kind == KIND_HERMITIAN ? cplx/2 : cplx;
  return (size_t) f % data == 0 && (size_t) F % trans == 0;
}

template<typename T>
cudaError_t PadTransform::runT(const void *in, void *out, bool fwd,
                               cudaStream_t s)
{
  typedef cplx<T> Cx;
  OuterPlan<T> P{};
  P.L=(int) a.L; P.m=(int) a.m; P.q=(int) a.q; P.N=(int) a.N;
  P.cshift=a.cshift; P.tile=fwd ? a.tile : a.tileB;
  P.fp=fftPlan(a.kind == KIND_REAL ? a.N/2 : a.m,prec);
  P.twN=(const typename TwT<T>::type *) twiddles(a.N,prec);
  P.twX=NULL; P.NX=1;
  P.io64=0; P.inplace=0;     // the public layout is natural order
  P.conj=0;
  P.count=1; P.nbatch=1; P.inBatch=P.outBatch=0;
  P.inRow=C; P.outRow=C; P.C=(int) C; P.Ltot=(long long) a.L*C;
  P.scale=(T) 1;
  P.in[0]=(const Cx *) in;
  P.out[0]=(Cx *) out;
  const int threads=256;
  if(a.kind == KIND_HERMITIAN) {
    // Forward: the H stored modes (complex side) to N reals with sign +1
    // (the complex-to-real kernel with the complex side conjugated);
    // backward: N reals to the H modes with sign -1 (real-to-complex,
    // conjugated).
    P.L=(int) a.N;
    P.fp=fftPlan(a.N/2,prec);
    P.conj=1;
    P.kc=(int) a.stored;
    return fwd ? launchOuterRealBwd<T>(P,threads,s) :
      launchOuterRealFwd<T>(P,threads,s);
  }
  if(a.kind == KIND_REAL)
    return fwd ? launchOuterRealFwd<T>(P,threads,s) :
      launchOuterRealBwd<T>(P,threads,s);
  return fwd ? launchOuterFwd<T>(P,threads,s) : launchOuterBwd<T>(P,threads,s);
}

cudaError_t PadTransform::forward(const void *f, void *F, cudaStream_t s)
{
  return prec == PREC_F64 ? runT<double>(f,F,true,s) :
    runT<float>(f,F,true,s);
}

cudaError_t PadTransform::backward(const void *F, void *f, cudaStream_t s)
{
  return prec == PREC_F64 ? runT<double>(F,f,false,s) :
    runT<float>(F,f,false,s);
}

// ---------------------------------------------------------------------------
// Plain FFTs (engine.h).

PlainFFT::PlainFFT(int kind, long n, int sign, long C, long B, long istride,
                   long ibatch, long ostride, long obatch, int prec)
  : kind(kind), sign(sign), prec(prec), n(n), C(C), B(B), istride(istride),
    ibatch(ibatch), ostride(ostride), obatch(obatch), tile(1), n1(0), n2(0),
    tile1(1), tile2(1), scratch(NULL)
{
  if(kind != FFT_C2C && kind != FFT_R2C && kind != FFT_C2R)
    throw std::runtime_error("unknown transform kind");
  if(prec != PREC_F64 && prec != PREC_F32)
    throw std::runtime_error("plain FFTs run in FP64 or FP32");
  if(sign != 1 && sign != -1) throw std::runtime_error("sign must be +1 or -1");
  if(n < 1 || C < 1 || B < 1 || istride < 1 || ostride < 1 ||
     (B > 1 && (ibatch < 1 || obatch < 1)))
    throw std::runtime_error("sizes and strides must be positive");
  if(C > 1 && (istride < C || ostride < C))
    throw std::runtime_error("interleaved sequences need stride >= C");
  if(C > INT_MAX || B > INT_MAX)
    throw std::runtime_error("too many sequences");
  if(!smooth(n))
    throw std::runtime_error("length "+std::to_string(n)+
                             " is not a product of 2, 3, 5 and 7");
  if(kind != FFT_C2C && n % 2)
    throw std::runtime_error("real transforms need an even length");
  int maxTile=wide(prec) ? 8 : 16;
  auto sm=[&](int t) -> size_t {
    if(kind == FFT_C2C)
      return std::max(FGB_BY_PREC(prec,outerFwdSmem,n,n,t,0),
                      FGB_BY_PREC(prec,outerBwdSmem,n,n,t,1,0));
    return FGB_BY_PREC(prec,outerRealSmem,n,n/2,t);
  };
  if(sm(1) > SMEM_MAX) {
    if(kind != FFT_C2C || C != 1 || istride != 1 || ostride != 1)
      throw std::runtime_error("length "+std::to_string(n)+" is too long for "
                               "one CTA's shared memory (longer transforms "
                               "take complex contiguous sequences)");
    if(B > 1 && (ibatch < n || obatch < n))
      throw std::runtime_error("long sequences must not overlap");
    // n = n1 n2 with both passes in one CTA, n1 as close to sqrt(n) as
    // the factors allow.
    auto fits=[&](long k, int t) {
      return std::max(FGB_BY_PREC(prec,outerFwdSmem,k,k,t,0),
                      FGB_BY_PREC(prec,outerBwdSmem,k,k,t,1,0)) <= SMEM_MAX;
    };
    long best=0;
    for(long a=2; a*a <= n*4 && a < n; ++a)
      if(n % a == 0 && smooth(a) && fits(a,1) && fits(n/a,1) &&
         (!best || std::labs(a*a-n) < std::labs(best*best-n))) best=a;
    if(!best)
      throw std::runtime_error("no two-pass plan for length "+
                               std::to_string(n));
    n1=best;
    n2=n/best;
    // Coalesced side: the pass that reads (or writes) with unit column
    // stride takes whole tiles; the strided one single columns.
    auto smw=[&](long k) {
      return [&,k](int t) {
        return std::max(FGB_BY_PREC(prec,outerFwdSmem,k,k,t,0),
                        FGB_BY_PREC(prec,outerBwdSmem,k,k,t,1,0));
      };
    };
    tile1=pickTile(maxTile,sign > 0 ? n2 : n1,B,smw(sign > 0 ? n1 : n2));
    tile2=pickTile(maxTile,sign > 0 ? n1 : n2,B,smw(sign > 0 ? n2 : n1));
    if(devAlloc(&scratch,elem(prec)*(size_t) n*(size_t) B) != cudaSuccess) {
      scratch=NULL;
      throw std::runtime_error("device allocation of the scratch array "
                               "failed");
    }
    return;
  }
  tile=C > 1 ? pickTile(maxTile,C,B,sm) : 1;
}

PlainFFT::~PlainFFT()
{
  if(scratch) cudaFree(scratch);
}

// Two passes over the n1 x n2 view of each sequence (see engine.h).
//   sign +1: s = i n2 + t.  Columns of length n1 over i (n2 of them,
//     adjacent), the W_n^{t k1} twiddle after: Z[k1][t]; then the rows of Z
//     read as single columns of stride 1 (column k1 at k1 n2), transformed
//     over t into X[k1 + n1 k2].
//   sign -1: s = i + n1 t.  Columns of length n2 over t (n1 of them,
//     adjacent) written transposed as Y[i][k2] (column i at i n2); then
//     columns of length n1 over i (n2 of them, adjacent) with the
//     W_n^{-i k2} twiddle before: X[k2 + n2 k1].
template<typename T>
cudaError_t PlainFFT::runTwoPass(const void *in, void *out, cudaStream_t s)
{
  typedef cplx<T> Cx;
  const int threads=256;
  cudaError_t e;
  auto base=[&](OuterPlan<T>& P, long len) {
    P.L=(int) len; P.m=(int) len; P.q=1; P.N=(int) len; P.cshift=0;
    P.fp=fftPlan(len,prec);
    P.twN=(const typename TwT<T>::type *) twiddles(len,prec);
    P.twX=NULL; P.NX=1;
    P.io64=0; P.inplace=0; P.conj=0;
    P.count=1; P.nbatch=(int) B;
    P.Ltot=LLONG_MAX;
    P.scale=(T) 1;
  };
  OuterPlan<T> P{};
  if(sign > 0) {
    base(P,n1);
    P.twX=(const typename TwT<T>::type *) twiddles(n,prec); P.NX=n;
    P.tile=tile1;
    P.C=(int) n2; P.inRow=n2; P.outRow=n2;
    P.inBatch=ibatch; P.outBatch=n;
    P.in[0]=(const Cx *) in; P.out[0]=(Cx *) scratch;
    if((e=launchOuterFwd<T>(P,threads,s)) != cudaSuccess) return e;
    OuterPlan<T> Q{};
    base(Q,n2);
    Q.tile=tile2;
    Q.C=(int) n1; Q.inRow=1; Q.cz=1; Q.cs=n2; Q.outRow=n1;
    Q.inBatch=n; Q.outBatch=obatch;
    Q.in[0]=(const Cx *) scratch; Q.out[0]=(Cx *) out;
    return launchOuterFwd<T>(Q,threads,s);
  }
  base(P,n2);
  P.tile=tile1;
  P.C=(int) n1; P.inRow=n1; P.outRow=1; P.cz=1; P.cs=n2;
  P.inBatch=ibatch; P.outBatch=n;
  P.in[0]=(const Cx *) in; P.out[0]=(Cx *) scratch;
  if((e=launchOuterBwd<T>(P,threads,s)) != cudaSuccess) return e;
  OuterPlan<T> Q{};
  base(Q,n1);
  Q.twX=(const typename TwT<T>::type *) twiddles(n,prec); Q.NX=n;
  Q.tile=tile2;
  Q.C=(int) n2; Q.inRow=n2; Q.outRow=n2;
  Q.inBatch=n; Q.outBatch=obatch;
  Q.in[0]=(const Cx *) scratch; Q.out[0]=(Cx *) out;
  return launchOuterBwd<T>(Q,threads,s);
}

template<typename T>
cudaError_t PlainFFT::runT(const void *in, void *out, cudaStream_t s)
{
  typedef cplx<T> Cx;
  OuterPlan<T> P{};
  const bool real=kind != FFT_C2C;
  P.L=(int) n; P.m=(int) n; P.q=1; P.N=(int) n; P.cshift=0;
  P.tile=tile;
  P.fp=fftPlan(real ? n/2 : n,prec);
  P.twN=(const typename TwT<T>::type *) twiddles(n,prec);
  P.twX=NULL; P.NX=1;
  P.io64=0; P.inplace=0;
  // The real kernels compute the sign +1 r2c and sign -1 c2r; FFTW's r2c
  // (-1) and c2r (+1) are their conjugates on the complex side.
  P.conj=real ? 1 : 0;
  P.count=1;
  P.C=(int) C;
  P.nbatch=(int) B;
  P.inRow=istride; P.outRow=ostride;
  P.inBatch=ibatch; P.outBatch=obatch;
  P.Ltot=LLONG_MAX;
  P.scale=(T) 1;
  P.in[0]=(const Cx *) in;
  P.out[0]=(Cx *) out;
  const int threads=256;
  if(kind == FFT_R2C) return launchOuterRealFwd<T>(P,threads,s);
  if(kind == FFT_C2R) return launchOuterRealBwd<T>(P,threads,s);
  return sign > 0 ? launchOuterFwd<T>(P,threads,s) :
    launchOuterBwd<T>(P,threads,s);
}

bool PlainFFT::aligned(const void *in, const void *out) const
{
  size_t cplx=elem(prec), real=cplx/2;
  size_t ai=kind == FFT_R2C ? real : cplx, ao=kind == FFT_C2R ? real : cplx;
  return (size_t) in % ai == 0 && (size_t) out % ao == 0;
}

cudaError_t PlainFFT::execute(const void *in, void *out, cudaStream_t s)
{
  if(n1 > 0)
    return prec == PREC_F64 ? runTwoPass<double>(in,out,s) :
      runTwoPass<float>(in,out,s);
  return prec == PREC_F64 ? runT<double>(in,out,s) : runT<float>(in,out,s);
}

} // namespace fgb
