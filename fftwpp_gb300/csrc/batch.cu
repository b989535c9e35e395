// batch.cu -- host side of the persistent batched launch (kernels.cuh):
// per-problem plans, the task list, the completion counters, CUDA-graph
// capture and the timing autotuner that picks each problem's plan.
//
// The autotuner replaces the reference's CPU optimiser (fftBase::OptBase,
// convolve.cc:177-470: it times whole convolutions for candidate m, D, I and
// keeps the fastest) with the same idea on the GPU: for every distinct
// padded length it times the candidate plans of that length on a batch of
// copies inside the persistent kernel and keeps the fastest; results are
// cached for the life of the process.
#include "batch.h"

#include <climits>
#include <cstddef>
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <tuple>

namespace fgb {

static const int NSM=152;
static const int THREADS=256;

static size_t elemBytes(int prec) {return prec == PREC_F64 ? 16 : 8;}

static size_t rowNeedB(int prec, long L, long m, int A, int B, int rpc=1,
                       int direct=0)
{
  return prec == PREC_F64 ? rowSmem<double>(L,m,A,B,rpc,direct) :
    rowSmem<float>(L,m,A,B,rpc,direct);
}

static size_t outerNeedB(int prec, long L, long m, int tile)
{
  size_t f=prec == PREC_F64 ? outerFwdSmem<double>(L,m,tile) :
    outerFwdSmem<float>(L,m,tile);
  size_t b=prec == PREC_F64 ? outerBwdSmem<double>(L,m,tile) :
    outerBwdSmem<float>(L,m,tile);
  return std::max(f,b);
}

static double fftCostB(long m) {return m*std::log2((double) std::max(m,2L));}

FFTPlanDev fftPlanPublic(long n, int prec, bool oddFirst);   // engine.cu

// Candidate plans of one problem, cheapest (by the cost model) first.
// choice > 0: short problem with residue block m = choice;
// choice < 0: long problem with row length -choice.
std::vector<long> BatchConv::candidates(long L, long M, int A, int B,
                                        int prec, size_t budget)
{
  std::vector<std::pair<double,long>> c;
  for(long q=1; q <= 16; ++q) {
    long m=nextfftsize(ceilquotient(M,q));
    if(m*q < M || rowNeedB(prec,L,m,A,B) > budget) continue;
    long p=ceilquotient(L,m);
    double cost=q*((A+B)*fftCostB(m)+A*p*(double) m+(A+B)*(double) m);
    bool dup=false;
    for(auto& x : c) if(x.second == m) dup=true;
    if(!dup) c.push_back({cost,m});
  }
  if(c.empty()) {
    long N=nextfftsize(M);
    for(long m=N; m >= 16; --m) {
      if(N % m || !smooth(m) || rowNeedB(prec,m,m,A,B) > budget) continue;
      long qc=N/m;
      long pc=ceilquotient(L,m);
      if(outerNeedB(prec,pc,qc,1) > budget) continue;
      double cost=(A+B)*(fftCostB(m)*qc+fftCostB(qc)*m);
      c.push_back({cost,-m});
      if(c.size() >= 4) break;
    }
  }
  std::sort(c.begin(),c.end());
  std::vector<long> out;
  for(auto& x : c) out.push_back(x.second);
  return out;
}

BatchConv::BatchConv(int nprob, const long *L, const long *M,
                     const long *choice, int A, int B, int mult, int prec,
                     int kind, bool tune)
  : n(nprob), A(A), B(B), mult(mult), prec(prec), kind(kind),
    dProbs(NULL), dTasks(NULL), dCounters(NULL), staging(NULL),
    graph(NULL), exec(NULL), captureStream(NULL), smem(0), grid(0),
    stagingSize(0), ntasks(0), nsmall(0), nlong(0)
{
  if(nprob < 1) throw std::runtime_error("empty batch");
  if(A < 1 || A > FGB_MAXA || B < 1 || B > A)
    throw std::runtime_error("need 1 <= B <= A <= 8");
  if(kind != KIND_PAD && kind != KIND_CENTERED)
    throw std::runtime_error("batched problems are fftPad or fftPadCentered");
  if(prec != PREC_F64 && prec != PREC_F32)
    throw std::runtime_error("batched problems run in FP64 or FP32");
  // Per-task shared memory: three CTAs per SM (a larger FP64 budget with
  // two CTAs per SM measured slower).
  budget=72*1024;
  Ls.assign(L,L+nprob);
  Ms.assign(M,M+nprob);
  offsets.resize(nprob);
  long off=0;
  for(int i=0; i < nprob; ++i) {
    if(Ls[i] < 1 || Ls[i] > Ms[i])
      throw std::runtime_error("need 1 <= L <= M for every problem");
    offsets[i]=off;
    off += Ls[i];
  }
  total=off;
  choices.resize(nprob);
  for(int i=0; i < nprob; ++i) {
    if(choice && choice[i]) {choices[i]=choice[i]; continue;}
    std::vector<long> cand=candidates(Ls[i],Ms[i],A,B,prec,budget);
    if(cand.empty())
      throw std::runtime_error("no batched plan for L="+std::to_string(Ls[i]));
    choices[i]=tune ? tuned(Ls[i],Ms[i],cand) : cand[0];
  }
  try {
    if(tune && nlongCount() > 0) {
      // Tile shapes: time the whole batch under each cap on the column
      // tiles of its long problems and keep the fastest.
      double best=1e300;
      int bestCap=tileCap;
      for(int cap : {16,32,64,128}) {
        tileCap=cap;
        if(prec == PREC_F64) build<double>(); else build<float>();
        double t=timeLaunch(3);
        if(t < best) {best=t; bestCap=cap;}
        release();
      }
      tileCap=bestCap;
    }
    if(prec == PREC_F64) build<double>(); else build<float>();
  } catch(...) {
    // A throwing constructor runs no destructor: release what was taken.
    release();
    throw;
  }
}

int BatchConv::nlongCount() const
{
  int k=0;
  for(long c : choices) k += c < 0;
  return k;
}

void BatchConv::release()
{
  if(exec) {cudaGraphExecDestroy(exec); exec=NULL;}
  if(graph) {cudaGraphDestroy(graph); graph=NULL;}
  graphKey.clear();
  if(dProbs) cudaFree(dProbs);
  if(dTasks) cudaFree(dTasks);
  if(dCounters) cudaFree(dCounters);
  if(staging) cudaFree(staging);
  dProbs=dTasks=dCounters=staging=NULL;
  stagingSize=0;
  nsmall=nlong=0;
}

// Milliseconds of one launch of the current build on zero-filled scratch
// arrays (median of reps after a warm-up), or a huge value on failure.
double BatchConv::timeLaunch(int reps)
{
  size_t bytes=elemBytes(prec)*(size_t) total;
  std::vector<void *> bufs(std::max(A,B),NULL);
  cudaStream_t s=NULL;
  cudaEvent_t e0=NULL, e1=NULL;
  bool ok=cudaStreamCreateWithFlags(&s,cudaStreamNonBlocking) == cudaSuccess &&
    cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  for(auto& p : bufs)
    ok=ok && devAlloc((void **) &p,bytes) == cudaSuccess &&
      cudaMemsetAsync(p,0,bytes,s) == cudaSuccess;
  std::vector<float> t;
  if(ok) ok=run(bufs.data(),bufs.data(),s) == cudaSuccess;
  for(int r=0; r < reps && ok; ++r) {
    ok=cudaEventRecord(e0,s) == cudaSuccess &&
      run(bufs.data(),bufs.data(),s) == cudaSuccess &&
      cudaEventRecord(e1,s) == cudaSuccess &&
      cudaEventSynchronize(e1) == cudaSuccess;
    float ms=0;
    if(ok && cudaEventElapsedTime(&ms,e0,e1) == cudaSuccess) t.push_back(ms);
  }
  if(s) cudaStreamSynchronize(s);
  ok=ok && error() == 0;
  for(void *p : bufs) if(p) cudaFree(p);
  if(e0) cudaEventDestroy(e0);
  if(e1) cudaEventDestroy(e1);
  if(s) cudaStreamDestroy(s);
  cudaGetLastError();
  if(!ok || t.empty()) return 1e300;
  std::sort(t.begin(),t.end());
  return t[t.size()/2];
}

// Timing autotuner: per (L, M, A, B, prec, mult, kind) the fastest
// candidate, timed on a batch of copies.
long BatchConv::tuned(long L, long M, const std::vector<long>& cand)
{
  static std::mutex mu;
  static std::map<std::tuple<long,long,int,int,int,int,int>,long> cache;
  auto key=std::make_tuple(L,M,A,B,prec,mult,kind);
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it=cache.find(key);
    if(it != cache.end()) return it->second;
  }
  long best=cand[0];
  if(cand.size() > 1) {
    int copies=std::max(8L,std::min(256L,(long) (1L<<22)/std::max(L,1L)));
    double bestT=1e300;
    size_t bytes=elemBytes(prec)*(size_t) L*copies;
    std::vector<void *> bufs(A,NULL);
    bool ok=true;
    for(int a=0; a < A && ok; ++a)
      ok=devAlloc((void **) &bufs[a],bytes) == cudaSuccess &&
        cudaMemset(bufs[a],0,bytes) == cudaSuccess;
    cudaStream_t s;
    cudaEvent_t e0, e1;
    if(ok && cudaStreamCreate(&s) == cudaSuccess) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      for(long c : cand) {
        std::vector<long> Lv(copies,L), Mv(copies,M), Cv(copies,c);
        try {
          BatchConv trial(copies,Lv.data(),Mv.data(),Cv.data(),A,B,mult,prec,
                          kind,false);
          trial.run(bufs.data(),bufs.data(),s);
          cudaEventRecord(e0,s);
          for(int k=0; k < 3; ++k) trial.run(bufs.data(),bufs.data(),s);
          cudaEventRecord(e1,s);
          cudaEventSynchronize(e1);
          float ms=0;
          cudaEventElapsedTime(&ms,e0,e1);
          if(trial.error() == 0 && ms < bestT) {bestT=ms; best=c;}
        } catch(std::exception&) {
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      cudaStreamDestroy(s);
    }
    for(void *p : bufs) if(p) cudaFree(p);
    cudaGetLastError();
  }
  std::lock_guard<std::mutex> lock(mu);
  cache[key]=best;
  return best;
}

// Queue order of a batched launch (host logic only).  The long problems
// pass through their staging: forward column tasks, row tasks, backward
// column tasks.  They go in groups of about groupBytes of staging,
// software-pipelined: step g queues the forward columns of group g, a share
// of the small problems, the rows of group g-1 and the backward columns of
// group g-2.  A problem's staging is then written and read back within
// three groups, while the L2 still holds it, and every task's producers
// were queued at least one group earlier, so a consumer rarely waits.
std::vector<BatchTask> orderBatchTasks(const std::vector<LongTasks>& lng,
                                       const std::vector<int>& small, int A,
                                       int B, size_t groupBytes)
{
  std::vector<std::vector<const LongTasks *>> groups;
  size_t acc=0;
  for(const auto& o : lng) {
    if(groups.empty() || (acc > 0 && acc+o.staging > groupBytes)) {
      groups.emplace_back();
      acc=0;
    }
    groups.back().push_back(&o);
    acc += o.staging;
  }
  const int ng=(int) groups.size();
  std::vector<BatchTask> tasks;
  size_t nextSmall=0;
  for(int g=0; g < ng+2; ++g) {
    if(g < ng)
      for(const LongTasks *p : groups[g])
        for(int t=0; t < p->fwdTiles; ++t)
          for(int a=0; a < A; ++a) tasks.push_back({TASK_COLFWD,p->prob,t,a});
    const size_t endSmall=small.size()*(size_t) (g+1)/(size_t) (ng+2);
    for(; nextSmall < endSmall; ++nextSmall)
      tasks.push_back({TASK_SMALL,small[nextSmall],0,0});
    if(g >= 1 && g-1 < ng)
      for(const LongTasks *p : groups[g-1])
        for(int r=0; r < p->rows; ++r) tasks.push_back({TASK_ROW,p->prob,r,0});
    if(g >= 2)
      for(const LongTasks *p : groups[g-2])
        for(int t=0; t < p->bwdTiles; ++t)
          for(int b=0; b < B; ++b) tasks.push_back({TASK_COLBWD,p->prob,t,b});
  }
  return tasks;
}

template<typename T>
void BatchConv::build()
{
  typedef typename TwT<T>::type Tw;
  const size_t e=elemBytes(prec);
  std::vector<BatchProblem<T>> probs(n);
  std::vector<long> stagingOff(n,-1);
  size_t stagingBytes=0;
  smem=0;
  struct Ord {double cost; int i;};
  std::vector<Ord> small, lng;
  for(int i=0; i < n; ++i) {
    BatchProblem<T>& P=probs[i];
    memset(&P,0,sizeof(P));
    long L=Ls[i], M=Ms[i], c=choices[i];
    if(c > 0) {
      long m=c;
      long q=ceilquotient(M,m);
      RowPlan<T>& R=P.row;
      R.L=(int) L; R.m=(int) m; R.q=(int) q; R.N=(int) (m*q);
      R.cshift=kind == KIND_CENTERED ? (int) (L/2) : 0;
      R.A=A; R.B=B; R.mult=mult; R.realIO=0; R.rpc=1;
      R.scale=(T) (1.0/(double) (m*q));
      R.fp=fftPlanPublic(m,prec,prec != PREC_F64);   // in-place rows in FP32
      R.direct=0;
      R.twN=(const Tw *) twiddles(m*q,prec);
      R.rowStride=L; R.nrows=1;
      for(int a=0; a < A; ++a) R.in[a]=(const cplx<T> *) (offsets[i]*e);
      for(int b=0; b < B; ++b) R.out[b]=(cplx<T> *) (offsets[i]*e);
      P.rel=1|2;
      smem=std::max(smem,rowNeedB(prec,L,m,A,B));
      small.push_back({q*fftCostB(m)*(A+B),i});
      ++nsmall;
    } else {
      if(kind != KIND_PAD)
        throw std::runtime_error("long batched problems must be fftPad");
      long m=-c;
      long N=nextfftsize(M);
      if(N % m) throw std::runtime_error("row length must divide N");
      long qc=N/m, pc=ceilquotient(L,m);
      // Column tasks take as many columns as the shared-memory budget
      // allows (each column is only a qc-point transform, so narrow tiles
      // would be dominated by per-task overhead).
      int tile=tileCap;
      while(tile > 1 && (tile > m || outerNeedB(prec,pc,qc,tile) > budget))
        tile /= 2;
      stagingOff[i]=(long) stagingBytes;
      stagingBytes += e*(size_t) N*A;
      OuterPlan<T>& F=P.fwd;
      F.L=(int) pc; F.m=(int) qc; F.q=1; F.N=(int) qc; F.cshift=0;
      F.tile=tile; F.fp=fftPlanPublic(qc,prec,false);
      F.twN=(const Tw *) twiddles(qc,prec);
      F.twX=(const Tw *) twiddles(N,prec); F.NX=N;
      F.count=A; F.nbatch=1; F.inBatch=F.outBatch=0;
      F.inRow=m; F.outRow=m; F.C=(int) m; F.Ltot=L; F.scale=(T) 1;
      for(int a=0; a < A; ++a) F.in[a]=(const cplx<T> *) (offsets[i]*e);
      OuterPlan<T>& G=P.bwd;
      G=F;
      G.count=B;
      G.scale=(T) (1.0/(double) N);
      for(int b=0; b < B; ++b) G.out[b]=(cplx<T> *) (offsets[i]*e);
      // Several rows per row task where they fit the budget.
      // The rows hold one residue of one fold: the direct row variant
      // (no staging, in-place transforms).
      int rpc=1;
      while(rpc < 8 && rpc < qc &&
            rowNeedB(prec,m,m,A,B,rpc+1,1) <= budget) ++rpc;
      RowPlan<T>& R=P.row;
      R.L=(int) m; R.m=(int) m; R.q=1; R.N=(int) m; R.cshift=0;
      R.A=A; R.B=B; R.mult=mult; R.realIO=0; R.rpc=rpc; R.scale=(T) 1;
      R.fp=fftPlanPublic(m,prec,true);
      R.direct=1;
      R.twN=(const Tw *) twiddles(m,prec);
      R.rowStride=m; R.nrows=qc;
      P.rel=4|8;
      P.nfwd=(int) (ceilquotient(m,tile)*A);
      P.nrows=(int) ceilquotient(qc,rpc);   // row tasks the backward waits for
      smem=std::max(smem,rowNeedB(prec,m,m,A,B,rpc,1));
      smem=std::max(smem,outerNeedB(prec,pc,qc,tile));
      lng.push_back({(double) N*std::log2((double) N),i});
      ++nlong;
    }
  }
  if(stagingBytes) {
    if(devAlloc((void **) &staging,stagingBytes) != cudaSuccess)
      throw std::runtime_error("batched staging allocation failed");
    stagingSize=stagingBytes;
  }
  for(int i=0; i < n; ++i) {
    if(stagingOff[i] < 0) continue;
    BatchProblem<T>& P=probs[i];
    long N=(long) P.fwd.NX;
    char *base=(char *) staging+stagingOff[i];
    for(int a=0; a < A; ++a) {
      cplx<T> *buf=(cplx<T> *) (base+e*(size_t) N*a);
      P.fwd.out[a]=buf;
      P.row.in[a]=buf;
      P.bwd.in[a]=buf;
      if(a < B) P.row.out[a]=buf;
    }
  }
  auto byCost=[](const Ord& x, const Ord& y) {return x.cost > y.cost;};
  std::sort(small.begin(),small.end(),byCost);
  std::sort(lng.begin(),lng.end(),byCost);
  std::vector<LongTasks> lt;
  for(auto& o : lng) {
    const BatchProblem<T>& P=probs[o.i];
    lt.push_back({o.i,e*(size_t) P.fwd.NX*A,
                  (int) ceilquotient(P.fwd.C,P.fwd.tile),P.nrows,
                  (int) ceilquotient(P.bwd.C,P.bwd.tile)});
  }
  std::vector<int> sm;
  for(auto& o : small) sm.push_back(o.i);
  // Measured on the 512-problem workload: 8 MB groups halve the FP32
  // launch's DRAM traffic (714 -> 364 MB) at the same speed; the FP64
  // launch, bound by its FP64 pipe, loses 12 % to the waits of groups that
  // small and keeps 24 MB groups (1260 -> 1105 MB).
  std::vector<BatchTask> tasks=orderBatchTasks(lt,sm,A,B,
                                               (prec == PREC_F64 ? 24u : 8u)
                                               << 20);
  ntasks=(int) tasks.size();
  nfwd0.resize(n);
  for(int i=0; i < n; ++i) nfwd0[i]=probs[i].nfwd;
  probBytes=sizeof(BatchProblem<T>);
  nfwdOffset=offsetof(BatchProblem<T>,nfwd);
  size_t pb=sizeof(BatchProblem<T>)*n, tb=sizeof(BatchTask)*tasks.size();
  if(devAlloc((void **) &dProbs,pb) != cudaSuccess ||
     devAlloc((void **) &dTasks,tb) != cudaSuccess ||
     devAlloc((void **) &dCounters,sizeof(int)*(2+2*(size_t) n)) != cudaSuccess)
    throw std::runtime_error("batched plan allocation failed");
  cudaMemcpy(dProbs,probs.data(),pb,cudaMemcpyHostToDevice);
  cudaMemcpy(dTasks,tasks.data(),tb,cudaMemcpyHostToDevice);
  cudaMemset(dCounters,0,sizeof(int)*(2+2*(size_t) n));
  int per=batchBlocksPerSM<T>(THREADS,smem,mult,A,B);
  grid=std::min(ntasks,NSM*per);
}

BatchConv::~BatchConv()
{
  release();
  if(captureStream) cudaStreamDestroy(captureStream);
}

template<typename T>
cudaError_t BatchConv::launch(const void *const *in, void *const *out,
                              cudaStream_t s)
{
  BatchArgs<T> P;
  P.probs=(const BatchProblem<T> *) dProbs;
  P.tasks=(const BatchTask *) dTasks;
  P.ntasks=ntasks;
  P.queue=(int *) dCounters;
  P.err=(int *) dCounters+1;
  P.done=(int *) dCounters+2;
  P.spinLimit=spinLimit;
  P.mult=mult;
  P.A=A;
  P.B=B;
  for(int a=0; a < FGB_MAXA; ++a) {
    P.inBase[a]=a < A ? (void *) in[a] : NULL;
    P.outBase[a]=a < B ? out[a] : NULL;
  }
  // Reset the dequeue and completion counters; keep the error flag sticky
  // until error() reads it.
  cudaError_t e=cudaMemsetAsync(P.queue,0,sizeof(int),s);
  if(e != cudaSuccess) return e;
  e=cudaMemsetAsync(P.done,0,sizeof(int)*2*(size_t) n,s);
  if(e != cudaSuccess) return e;
  return launchBatch<T>(P,grid,THREADS,smem,s);
}

cudaError_t BatchConv::run(const void *const *in, void *const *out,
                           cudaStream_t s)
{
  return prec == PREC_F64 ? launch<double>(in,out,s) : launch<float>(in,out,s);
}

cudaError_t BatchConv::runGraph(const void *const *in, void *const *out,
                                cudaStream_t s)
{
  std::vector<const void *> key(in,in+A);
  for(int b=0; b < B; ++b) key.push_back(out[b]);
  if(!exec || key != graphKey) {
    if(exec) {cudaGraphExecDestroy(exec); exec=NULL;}
    if(graph) {cudaGraphDestroy(graph); graph=NULL;}
    if(!captureStream) {
      cudaError_t e=cudaStreamCreateWithFlags(&captureStream,
                                              cudaStreamNonBlocking);
      if(e != cudaSuccess) return e;
    }
    cudaError_t e=cudaStreamBeginCapture(captureStream,
                                         cudaStreamCaptureModeThreadLocal);
    if(e != cudaSuccess) return e;
    cudaError_t el=run(in,out,captureStream);
    e=cudaStreamEndCapture(captureStream,&graph);
    if(el != cudaSuccess) return el;
    if(e != cudaSuccess) return e;
    e=cudaGraphInstantiate(&exec,graph,0);
    if(e != cudaSuccess) return e;
    graphKey=key;
  }
  return cudaGraphLaunch(exec,s);
}

int BatchConv::error()
{
  int v=0;
  cudaMemcpy(&v,(int *) dCounters+1,sizeof(int),cudaMemcpyDeviceToHost);
  if(v) cudaMemset((int *) dCounters+1,0,sizeof(int));
  return v;
}

long BatchConv::choice(int i) const {return choices[i];}

void BatchConv::setSpinLimit(long long polls)
{
  spinLimit=polls;
  graphKey.clear();                // the limit is a launch argument
}

cudaError_t BatchConv::blockProblem(int i, bool blocked)
{
  if(i < 0 || i >= n || choices[i] > 0) return cudaErrorInvalidValue;
  int v=blocked ? INT_MAX : nfwd0[i];
  return cudaMemcpy((char *) dProbs+(size_t) i*probBytes+nfwdOffset,&v,
                    sizeof(int),cudaMemcpyHostToDevice);
}

} // namespace fgb
