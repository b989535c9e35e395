// kernels.cu -- GB300 (sm_103a) kernels of the hybrid dealiased convolution.
// See kernels.cuh for the decomposition; reference routines are cited per
// kernel.  The innermost-axis (row) kernels live in rowkernels.cuh, templated
// on the multiplier; this file instantiates them for the built-in
// multipliers and holds the outer-axis, batched and copy kernels.
#include "rowkernels.cuh"

#include <algorithm>
#include <climits>
#include <type_traits>

namespace fgb {


// ---------------------------------------------------------------------------
// Offset of column col on the data side of an outer kernel (the caller's
// arrays): col itself for dense layouts, (col / cz) cs + col % cz for the
// strided layouts of fftPad(L, M, app, C, S) with S > C (convolve.h:515-536;
// Convolution2/3's Sx, Sy, convolve.h:1274, 1556).
template<typename T>
__device__ __forceinline__ long long dataCol(const OuterPlan<T>& P, int col)
{
  if(P.cz <= 0) return col;
  const int g=col/P.cz;
  return (long long) g*P.cs+(col-g*P.cz);
}

// ---------------------------------------------------------------------------
// Outer forward, complex data: residue block r of the padded transform along
// a strided axis for `tile` adjacent columns.
template<typename T, bool CG, bool R16=false>
__device__ __forceinline__ void outerFwdTile(const OuterPlan<T>& P, int ctile,
                                             int r, int z,
                                             unsigned char *smemRaw)
{
  const int tile=P.tile, m=P.m, N=P.N, c=P.cshift, L=P.L;
  cplx<T> *x=(cplx<T> *) smemRaw;
  cplx<T> *y=x+padded(m*tile);
  const int tid=threadIdx.x, nthr=blockDim.x;
  const int col0=ctile*tile;
  const int a=z % P.count;
  const long long batch=z/P.count;
  const cplx<T> *src=P.in[a]+batch*P.inBatch;
  cplx<T> *dst=P.out[a]+batch*P.outBatch;
  const typename TwT<T>::type *tw=P.twN;
  const UDiv dTile(tile);

  if(P.flat != FLAT_PAD) {
    // Long rows of the other kinds: every position n = t*C + col of the
    // flattened row holds the data index of its kind (FlatMode); loaded
    // and converted directly (conjugated mirror, real values).
    const T *srcR=(const T *) P.in[a]+batch*P.inBatch;
    const int sh=ioShift<T>(P.ioShift,a);
    for(int i=tid; i < m*tile; i += nthr) {
      int t=dTile(i), cc=i-t*tile;
      int col=col0+cc;
      cplx<T> v=mk((T) 0,(T) 0);
      if(col < P.C) {
        const long long n=(long long) t*P.inRow+col;
        if(P.flat == FLAT_CENTERED) {
          long long sx=n+P.flatC;
          if(sx >= P.NX) sx -= P.NX;
          if(sx < P.Ltot) v=loadIO(src+sx,P.io64 & 1,sh);
        } else if(P.flat == FLAT_HERMITIAN) {
          if(n < P.Ltot) {
            v=loadIO(src+n,P.io64 & 1,sh);
            if(n == 0) v.y=(T) 0;
          } else if(P.NX-n < P.Ltot) v=conjg(loadIO(src+(P.NX-n),P.io64 & 1,sh));
        } else if(n < P.Ltot) {
          v=mk(loadIOr(srcR+n,P.io64 & 1,sh),(T) 0);
        }
      }
      x[sp(i)]=v;
    }
    __syncthreads();
  } else if(L <= m) {
    // One term per output: asynchronous copies straight to each value's
    // transform slot, then the conversion and residue twiddle in place by
    // the same thread.
    for(int i=tid; i < m*tile; i += nthr) {
      int t=dTile(i), cc=i-t*tile;
      int col=col0+cc;
      int s=posmod(t+c,m);
      long long off=(long long) s*P.inRow+dataCol(P,col);
      if(s < L && col < P.C && off < P.Ltot) cpAsync(x+sp(i),src+off);
      else x[sp(i)]=mk((T) 0,(T) 0);
    }
    cpAsyncWait();
    if(r != 0 || (P.io64 & 1)) {
      for(int i=tid; i < m*tile; i += nthr) {
        int t=dTile(i), cc=i-t*tile;
        int col=col0+cc;
        int s=posmod(t+c,m);
        long long off=(long long) s*P.inRow+dataCol(P,col);
        if(s < L && col < P.C && off < P.Ltot) {
          if(P.io64 & 1) convertStaged(x,sp(i),ioShift<T>(P.ioShift,a));
          if(r != 0) x[sp(i)]=twmul<1>(x[sp(i)],tw[twExp(s,c,r,N)]);
        }
      }
    }
    __syncthreads();
  } else {
    // Stage the L x tile input block in y with asynchronous copies (many
    // loads in flight per thread instead of one dependent load per
    // output), then fold it into x with the residue twiddles.
    for(int i=tid; i < L*tile; i += nthr) {
      int s=dTile(i), cc=i-s*tile;
      int col=col0+cc;
      long long off=(long long) s*P.inRow+dataCol(P,col);
      if(col < P.C && off < P.Ltot) cpAsync(y+i,src+off);
      else y[i]=mk((T) 0,(T) 0);
    }
    cpAsyncWait();
    if(std::is_same<T,ff>::value && (P.io64 & 1)) {
      // The caller's FP64 values were staged as they are: convert them.
      for(int i=tid; i < L*tile; i += nthr) {
        int s=dTile(i), cc=i-s*tile;
        int col=col0+cc;
        long long off=(long long) s*P.inRow+dataCol(P,col);
        if(col < P.C && off < P.Ltot)
          convertStaged(y,i,ioShift<T>(P.ioShift,a));
      }
    }
    __syncthreads();
    for(int i=tid; i < m*tile; i += nthr) {
      int t=dTile(i), cc=i-t*tile;
      cplx<T> sum=mk((T) 0,(T) 0);
      int s0=posmod(t+c,m);
      // The twiddle exponent advances by m r mod N from term to term.
      int e=r != 0 ? twExp(s0,c,r,N) : 0;
      const int de=r != 0 ? twStep(m,r,N) : 0;
      for(int s=s0; s < L; s += m) {
        cplx<T> v=y[s*tile+cc];
        if(r != 0) {
          v=twmul<1>(v,tw[e]);
          e += de;
          if(e >= N) e -= N;
        }
        sum=accum(sum,v);
      }
      x[sp(i)]=sum;
    }
    __syncthreads();
  }

  if constexpr(inplaceFFT<T>()) {
    if(P.inplace) {
      // Transform in place (digit-reversed j; the row kernels do not
      // depend on row order and the backward undoes it).
      fftDIF<T,1,R16>(x,P.fp,tile,tile,tid,nthr);
      for(int i=tid; i < m*tile; i += nthr) {
        int j=dTile(i), cc=i-j*tile;
        int col=col0+cc;
        if(col < P.C) dst[((long long) r*m+j)*P.outRow+col]=x[sp(i)];
      }
      __syncthreads();
      return;
    }
  }

  cplx<T> *X=fftSmem<T,1>(x,y,P.fp,tile,tile,tid,nthr);
  for(int i=tid; i < m*tile; i += nthr) {
    int j=dTile(i), cc=i-j*tile;
    int col=col0+cc;
    if(col < P.C) {
      cplx<T> v=X[sp(i)];
      long long k=(long long) r*m+j;
      if(P.twX) {
        unsigned long long e=((unsigned long long) col*(unsigned long long) k)
          % (unsigned long long) P.NX;
        v=twmul<1>(v,P.twX[e]);
      }
      dst[k*P.outRow+col]=v;
    }
  }
  __syncthreads();
}

template<typename T>
__global__ void __launch_bounds__(256)
outerFwdKernel(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  outerFwdTile<T,false>(P,blockIdx.x,blockIdx.y,blockIdx.z,smemRaw);
}

// Outer backward, complex data: all residues of a column tile, accumulated.
template<typename T, bool CG, bool R16=false>
__device__ __forceinline__ void outerBwdTile(const OuterPlan<T>& P, int ctile,
                                             int z, unsigned char *smemRaw)
{
  const int tile=P.tile, m=P.m, N=P.N, c=P.cshift, L=P.L;
  // One residue: the outputs come straight from the transform, with no
  // accumulator in shared memory.
  const bool direct=P.q == 1;
  cplx<T> *acc=(cplx<T> *) smemRaw;
  cplx<T> *x=direct ? acc : acc+L*tile;
  cplx<T> *y=x+padded(m*tile);
  const int tid=threadIdx.x, nthr=blockDim.x;
  const int col0=ctile*tile;
  const int b=z % P.count;
  const long long batch=z/P.count;
  const cplx<T> *src=P.in[b]+batch*P.inBatch;
  cplx<T> *dst=P.out[b]+batch*P.outBatch;
  const typename TwT<T>::type *tw=P.twN;
  const UDiv dTile(tile);

  if(!direct)
    for(int i=tid; i < L*tile; i += nthr) acc[i]=mk((T) 0,(T) 0);
  for(int r=0; r < P.q; ++r) {
    if(CG) {
      // Data written by other CTAs of this launch: L2 loads.
      for(int i=tid; i < m*tile; i += nthr) {
        int j=dTile(i), cc=i-j*tile;
        int col=col0+cc;
        cplx<T> v=mk((T) 0,(T) 0);
        if(col < P.C) v=ldx<CG>(src+((long long) r*m+j)*P.inRow+col);
        x[sp(i)]=v;
      }
    } else {
      for(int i=tid; i < m*tile; i += nthr) {
        int j=dTile(i), cc=i-j*tile;
        int col=col0+cc;
        if(col < P.C) cpAsync(x+sp(i),src+((long long) r*m+j)*P.inRow+col);
        else x[sp(i)]=mk((T) 0,(T) 0);
      }
      cpAsyncWait();
    }
    __syncthreads();
    if(P.twX) {
      for(int i=tid; i < m*tile; i += nthr) {
        int j=dTile(i), cc=i-j*tile;
        unsigned long long e=((unsigned long long) (col0+cc)*
                              (unsigned long long) ((long long) r*m+j)) %
          (unsigned long long) P.NX;
        x[sp(i)]=twmul<-1>(x[sp(i)],P.twX[e]);
      }
      __syncthreads();
    }
    cplx<T> *X;
    if(inplaceFFT<T>() && P.inplace) {
      fftDIT<T,-1,R16>(x,P.fp,tile,tile,tid,nthr);
      X=x;
    } else {
      X=fftSmem<T,-1>(x,y,P.fp,tile,tile,tid,nthr);
    }
    if(direct && P.flat != FLAT_PAD) {
      // Long rows of the other kinds: the output of data index sx is the
      // flattened position n of its kind (FlatMode).
      T *dstR=(T *) P.out[b]+batch*P.outBatch;
      const int sh=ioShift<T>(P.ioShift,8+b);
      for(int i=tid; i < m*tile; i += nthr) {
        int t=dTile(i), cc=i-t*tile;
        int col=col0+cc;
        if(col >= P.C) continue;
        const long long n=(long long) t*P.outRow+col;
        const cplx<T> v=X[sp(i)]*P.scale;
        if(P.flat == FLAT_CENTERED) {
          long long sx=n+P.flatC;
          if(sx >= P.NX) sx -= P.NX;
          if(sx < P.Ltot) storeIO(dst+sx,v,P.io64 & 2,sh);
        } else if(n < P.Ltot) {
          if(P.flat == FLAT_REAL) storeIOr(dstR+n,v.x,P.io64 & 2,sh);
          else storeIO(dst+n,v,P.io64 & 2,sh);
        }
      }
      __syncthreads();
      return;
    }
    if(direct) {
      for(int i=tid; i < L*tile; i += nthr) {
        int s=dTile(i), cc=i-s*tile;
        int col=col0+cc;
        long long off=(long long) s*P.outRow+dataCol(P,col);
        if(col < P.C && off < P.Ltot)
          storeIO(dst+off,X[sp(posmod(s-c,m)*tile+cc)]*P.scale,P.io64 & 2,
                  ioShift<T>(P.ioShift,8+b));
      }
      __syncthreads();
      return;
    }
    for(int i=tid; i < L*tile; i += nthr) {
      int s=dTile(i), cc=i-s*tile;
      int t=posmod(s-c,m);
      cplx<T> v=X[sp(t*tile+cc)];
      if(r != 0) v=twmul<-1>(v,tw[twExp(s,c,r,N)]);
      acc[i]=accum(acc[i],v);
    }
    __syncthreads();
  }
  for(int i=tid; i < L*tile; i += nthr) {
    int s=dTile(i), cc=i-s*tile;
    int col=col0+cc;
    long long off=(long long) s*P.outRow+dataCol(P,col);
    if(col < P.C && off < P.Ltot)
      storeIO(dst+off,acc[i]*P.scale,P.io64 & 2,ioShift<T>(P.ioShift,8+b));
  }
  __syncthreads();
}

template<typename T>
__global__ void __launch_bounds__(256)
outerBwdKernel(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  outerBwdTile<T,false>(P,blockIdx.x,blockIdx.z,smemRaw);
}

// FP32 in-place plans with radix-16 or radix-6 stages: their own
// instantiations, capped at 85 registers a thread (the wider codelets need
// more registers than the others may take).
template<typename T>
__global__ void __launch_bounds__(256,3)
outerFwdKernel16(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  outerFwdTile<T,false,true>(P,blockIdx.x,blockIdx.y,blockIdx.z,smemRaw);
}

template<typename T>
__global__ void __launch_bounds__(256,3)
outerBwdKernel16(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  outerBwdTile<T,false,true>(P,blockIdx.x,blockIdx.z,smemRaw);
}

// ---------------------------------------------------------------------------
// Outer forward, real data (fftPadReal with explicit padding to even N):
// pack z[t] = f[2t] + i f[2t+1], sign +1 FFT of length N/2, unpack the
// N/2+1 non-negative modes F(k) = E[k] + W_N^k O[k].
template<typename T>
__global__ void __launch_bounds__(256)
outerRealFwdKernel(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  const int tile=P.tile, L=P.L, Nh=P.N/2;
  cplx<T> *x=(cplx<T> *) smemRaw;
  cplx<T> *y=x+padded(Nh*tile);
  const int tid=threadIdx.x, nthr=blockDim.x;
  const int col0=blockIdx.x*tile;
  const int a=blockIdx.z % P.count;
  const long long batch=blockIdx.z/P.count;
  const T *src=(const T *) P.in[a]+batch*P.inBatch;
  cplx<T> *dst=P.out[a]+batch*P.outBatch;
  const typename TwT<T>::type *tw=P.twN;
  const T half=(T) 0.5;
  const UDiv dTile(tile);

  for(int i=tid; i < Nh*tile; i += nthr) {
    int t=dTile(i), cc=i-t*tile;
    int col=col0+cc;
    T re=(T) 0, im=(T) 0;
    if(col < P.C) {
      int s=2*t;
      const long long dc=dataCol(P,col);
      const int sh=ioShift<T>(P.ioShift,a);
      if(s < L) re=loadIOr(src+(long long) s*P.inRow+dc,P.io64 & 1,sh);
      if(s+1 < L) im=loadIOr(src+(long long) (s+1)*P.inRow+dc,P.io64 & 1,sh);
    }
    x[sp(i)]=mk(re,im);
  }
  __syncthreads();
  cplx<T> *X=fftSmem<T,1>(x,y,P.fp,tile,tile,tid,nthr);
  for(int i=tid; i < (Nh+1)*tile; i += nthr) {
    int k=dTile(i), cc=i-k*tile;
    int col=col0+cc;
    if(col >= P.C) continue;
    if(P.kc > 0 && k >= P.kc) continue;
    int k0=k == Nh ? 0 : k;
    int km=k == 0 || k == Nh ? 0 : Nh-k;
    cplx<T> zk=X[sp(k0*tile+cc)];
    cplx<T> zm=conjg(X[sp(km*tile+cc)]);
    cplx<T> e=(zk+zm)*half;
    cplx<T> dd=zk-zm;
    cplx<T> o=mk(dd.y*half,-dd.x*half);
    cplx<T> v;
    if(k == Nh) v=e-o;
    else v=e+twmul<1>(o,tw[k]);
    dst[(long long) k*P.outRow+col]=P.conj ? conjg(v) : v;
  }
}

// Outer backward, real data: Hermitian-extend the N/2+1 modes, pack
// Y[k] = (G[k] + conj G[Nh-k]) + i W_N^{-k} (G[k] - conj G[Nh-k]), sign -1
// FFT of length N/2, unpack h[2t] = Re y[t], h[2t+1] = Im y[t].
template<typename T>
__global__ void __launch_bounds__(256)
outerRealBwdKernel(const OuterPlan<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  const int tile=P.tile, L=P.L, Nh=P.N/2;
  cplx<T> *x=(cplx<T> *) smemRaw;
  cplx<T> *y=x+padded(Nh*tile);
  const int tid=threadIdx.x, nthr=blockDim.x;
  const int col0=blockIdx.x*tile;
  const int b=blockIdx.z % P.count;
  const long long batch=blockIdx.z/P.count;
  const cplx<T> *src=P.in[b]+batch*P.inBatch;
  T *dst=(T *) P.out[b]+batch*P.outBatch;
  const typename TwT<T>::type *tw=P.twN;
  const UDiv dTile(tile);

  for(int i=tid; i < Nh*tile; i += nthr) {
    int k=dTile(i), cc=i-k*tile;
    int col=col0+cc;
    cplx<T> v=mk((T) 0,(T) 0);
    if(col < P.C) {
      const int kc=P.kc > 0 ? P.kc : Nh+1;
      cplx<T> gk=k < kc ? src[(long long) k*P.inRow+col] : mk((T) 0,(T) 0);
      cplx<T> gm=Nh-k < kc ? src[(long long) (Nh-k)*P.inRow+col] :
        mk((T) 0,(T) 0);
      if(P.conj) {
        gk=conjg(gk);
        gm=conjg(gm);
      }
      if(k == 0) gk.y=(T) 0;
      if(k == 0) gm.y=(T) 0;
      gm=conjg(gm);
      cplx<T> s=gk+gm;
      cplx<T> d=twmul<-1>(gk-gm,tw[k]);
      v=mk(s.x-d.y,s.y+d.x);
    }
    x[sp(i)]=v;
  }
  __syncthreads();
  cplx<T> *X=fftSmem<T,-1>(x,y,P.fp,tile,tile,tid,nthr);
  for(int i=tid; i < Nh*tile; i += nthr) {
    int t=dTile(i), cc=i-t*tile;
    int col=col0+cc;
    if(col >= P.C) continue;
    cplx<T> v=X[sp(i)]*P.scale;
    int s=2*t;
    const long long dc=dataCol(P,col);
    const int sh=ioShift<T>(P.ioShift,8+b);
    if(s < L) storeIOr(dst+(long long) s*P.outRow+dc,v.x,P.io64 & 2,sh);
    if(s+1 < L) storeIOr(dst+(long long) (s+1)*P.outRow+dc,v.y,P.io64 & 2,sh);
  }
}

// ---------------------------------------------------------------------------
// Persistent batched kernel (see kernels.cuh).

template<typename T, template<typename> class Plan>
__device__ __forceinline__ void rebase(Plan<T>& plan, int count, bool relIn,
                                       bool relOut, void *const *inBase,
                                       void *const *outBase)
{
  for(int a=0; a < count; ++a) {
    if(relIn)
      plan.in[a]=(const cplx<T> *) ((char *) inBase[a]+(size_t) plan.in[a]);
    if(relOut)
      plan.out[a]=(cplx<T> *) ((char *) outBase[a]+(size_t) plan.out[a]);
  }
}

// Copy a task's plan from the problem table into shared memory (one copy per
// CTA, read by every thread through broadcast loads) and rebase its pointers
// there: a per-thread copy would live in local memory.
template<typename Plan>
__device__ __forceinline__ Plan& stagePlan(unsigned char *buf, const Plan& src)
{
  static_assert(sizeof(Plan) % sizeof(int) == 0, "plan size");
  int *d=(int *) buf;
  const int *s=(const int *) &src;
  for(int i=threadIdx.x; i < (int) (sizeof(Plan)/sizeof(int)); i += blockDim.x)
    d[i]=s[i];
  return *(Plan *) buf;
}

template<typename T, int K>
__global__ void __launch_bounds__(256)
batchKernel(const BatchArgs<T> P)
{
  extern __shared__ __align__(16) unsigned char smemRaw[];
  constexpr size_t planBytes=sizeof(RowPlan<T>) > sizeof(OuterPlan<T>) ?
    sizeof(RowPlan<T>) : sizeof(OuterPlan<T>);
  __shared__ __align__(16) unsigned char planBuf[planBytes];
  __shared__ int slot;
  __shared__ int gaveUp;
  for(;;) {
    if(threadIdx.x == 0) slot=atomicAdd(P.queue,1);
    __syncthreads();
    const int t=slot;
    __syncthreads();
    if(t >= P.ntasks) return;
    const BatchTask tk=P.tasks[t];
    const BatchProblem<T> *B=P.probs+tk.prob;
    if(tk.type == TASK_ROW || tk.type == TASK_COLBWD) {
      if(threadIdx.x == 0) {
        volatile int *d=P.done+2*tk.prob+(tk.type == TASK_ROW ? 0 : 1);
        const int target=tk.type == TASK_ROW ? B->nfwd : B->nrows;
        long long it=0;
        gaveUp=0;
        while(*d < target) {
          if(++it > P.spinLimit) {
            gaveUp=1;
            atomicExch(P.err,1);
            break;
          }
          __nanosleep(100);
        }
        __threadfence();
      }
      __syncthreads();
      if(gaveUp) continue;
    }
    const int rel=B->rel;
    if(tk.type == TASK_SMALL || tk.type == TASK_ROW) {
      RowPlan<T>& R=stagePlan(planBuf,B->row);
      __syncthreads();
      if(threadIdx.x == 0 && tk.type == TASK_SMALL)
        rebase(R,R.A,rel & 1,rel & 2,P.inBase,P.outBase);
      __syncthreads();
      const BuiltinMult<K> mul;
      if(tk.type == TASK_SMALL)
        rowConvRow<T,false,BuiltinMult<K>>(R,tk.i,smemRaw,mul);
      else if(R.direct)
        rowConvRow<T,true,BuiltinMult<K>,true>(R,tk.i,smemRaw,mul);
      else rowConvRow<T,true,BuiltinMult<K>>(R,tk.i,smemRaw,mul);
    } else {
      const bool fwd=tk.type == TASK_COLFWD;
      OuterPlan<T>& O=stagePlan(planBuf,fwd ? B->fwd : B->bwd);
      __syncthreads();
      if(threadIdx.x == 0)
        rebase(O,O.count,fwd && (rel & 4),!fwd && (rel & 8),P.inBase,
               P.outBase);
      __syncthreads();
      if(fwd) outerFwdTile<T,false>(O,tk.i,0,tk.j,smemRaw);
      else outerBwdTile<T,true>(O,tk.i,tk.j,smemRaw);
    }
    if(tk.type == TASK_COLFWD || tk.type == TASK_ROW) {
      __threadfence();
      __syncthreads();
      if(threadIdx.x == 0)
        atomicAdd(P.done+2*tk.prob+(tk.type == TASK_COLFWD ? 0 : 1),1);
    }
  }
}

template<typename T, int K>
static cudaError_t launchBatchK(const BatchArgs<T>& P, int grid, int threads,
                                size_t smem, cudaStream_t s)
{
  if(smem > 48*1024) {
    cudaError_t e=cudaFuncSetAttribute(batchKernel<T,K>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int) smem);
    if(e != cudaSuccess) return e;
  }
  batchKernel<T,K><<<grid,threads,smem,s>>>(P);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launchBatch(const BatchArgs<T>& P, int grid, int threads,
                        size_t smem, cudaStream_t s)
{
  switch(multVariant(P.mult,P.A,P.B)) {
    case MULT_BINARY: return launchBatchK<T,MULT_BINARY>(P,grid,threads,smem,s);
    case MULT_REALBINARY:
      return launchBatchK<T,MULT_REALBINARY>(P,grid,threads,smem,s);
    default: return launchBatchK<T,MULT_GENERIC>(P,grid,threads,smem,s);
  }
}

template<typename T, int K>
static int batchBlocksK(int threads, size_t smem)
{
  if(smem > 48*1024)
    cudaFuncSetAttribute(batchKernel<T,K>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,(int) smem);
  int n=0;
  if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n,batchKernel<T,K>,threads,
                                                   smem) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

template<typename T>
int batchBlocksPerSM(int threads, size_t smem, int mult, int A, int B)
{
  switch(multVariant(mult,A,B)) {
    case MULT_BINARY: return batchBlocksK<T,MULT_BINARY>(threads,smem);
    case MULT_REALBINARY: return batchBlocksK<T,MULT_REALBINARY>(threads,smem);
    default: return batchBlocksK<T,MULT_GENERIC>(threads,smem);
  }
}

// ---------------------------------------------------------------------------
// Launchers.

// Shared-memory bytes: FFT ping-pong buffers are padded (sp()); the forward
// outer kernel also stages its L x tile input block in the second buffer.
template<typename T> size_t rowSmem(int L, int m, int A, int B, int rpc,
                                    int direct)
{
  size_t nbuf=inplaceFFT<T>() || direct ? 1 : 2;
  size_t stage=direct ? 0 : (size_t) (A+B)*rpc*L;
  return sizeof(cplx<T>)*(stage+nbuf*(size_t) padded(m*A*rpc));
}
template<typename T> size_t hermRowSmem(int H, int Nh, int A, int rpc)
{
  size_t nbuf=inplaceFFT<T>() ? 1 : 2;
  return sizeof(cplx<T>)*nbuf*(size_t) padded(Nh*A*rpc);
}
template<typename T> size_t outerFwdSmem(int L, int m, int tile, int inplace)
{
  size_t pm=padded(m*tile);
  if(inplaceFFT<T>() && inplace) return sizeof(cplx<T>)*pm;
  return sizeof(cplx<T>)*(pm+std::max(pm,(size_t) L*tile));
}
template<typename T> size_t outerBwdSmem(int L, int m, int tile, int q,
                                         int inplace)
{
  size_t acc=q == 1 ? 0 : (size_t) L*tile;
  size_t nbuf=inplaceFFT<T>() && inplace ? 1 : 2;
  return sizeof(cplx<T>)*(acc+nbuf*(size_t) padded(m*tile));
}
template<typename T> size_t outerRealSmem(int L, int Nh, int tile)
{
  return sizeof(cplx<T>)*2*(size_t) padded((Nh+1)*tile);
}

template<typename K>
static cudaError_t setSmem(K kernel, size_t bytes)
{
  if(bytes > 48*1024)
    return cudaFuncSetAttribute(kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int) bytes);
  return cudaSuccess;
}

template<typename T>
cudaError_t launchRow(const RowPlan<T>& P, int threads, long long grid,
                      cudaStream_t s)
{
  switch(multVariant(P.mult,P.A,P.B)) {
    case MULT_BINARY:
      return launchRowWith(P,BuiltinMult<MULT_BINARY>(),threads,grid,s);
    case MULT_REALBINARY:
      return launchRowWith(P,BuiltinMult<MULT_REALBINARY>(),threads,grid,s);
    default:
      return launchRowWith(P,BuiltinMult<MULT_GENERIC>(),threads,grid,s);
  }
}

template<typename T>
cudaError_t launchHermRow(const HermRowPlan<T>& P, int threads,
                          long long grid, cudaStream_t s)
{
  switch(multVariant(P.mult,P.A,P.B)) {
    case MULT_REALBINARY:
      return launchHermRowWith(P,BuiltinMult<MULT_REALBINARY>(),threads,grid,
                               s);
    case MULT_REALJACOBIAN:
      return launchHermRowWith(P,BuiltinMult<MULT_REALJACOBIAN>(),threads,
                               grid,s);
    case MULT_REALJACADJ:
      return launchHermRowWith(P,BuiltinMult<MULT_REALJACADJ>(),threads,grid,
                               s);
    default:
      return launchHermRowWith(P,BuiltinMult<MULT_GENERIC>(),threads,grid,s);
  }
}

template<typename T>
cudaError_t launchOuterFwd(const OuterPlan<T>& P, int threads, cudaStream_t s)
{
  size_t sm=outerFwdSmem<T>(P.L,P.m,P.tile,P.inplace);
  dim3 grid((P.C+P.tile-1)/P.tile,P.q,P.nbatch*P.count);
  auto go=[&](auto kernel) {
    cudaError_t e=setSmem(kernel,sm);
    if(e != cudaSuccess) return e;
    kernel<<<grid,threads,sm,s>>>(P);
    return cudaGetLastError();
  };
  if constexpr(std::is_same<T,float>::value)
    if(P.inplace && hasWideRadix(P.fp)) return go(outerFwdKernel16<T>);
  return go(outerFwdKernel<T>);
}

template<typename T>
cudaError_t launchOuterBwd(const OuterPlan<T>& P, int threads, cudaStream_t s)
{
  size_t sm=outerBwdSmem<T>(P.L,P.m,P.tile,P.q,P.inplace);
  dim3 grid((P.C+P.tile-1)/P.tile,1,P.nbatch*P.count);
  auto go=[&](auto kernel) {
    cudaError_t e=setSmem(kernel,sm);
    if(e != cudaSuccess) return e;
    kernel<<<grid,threads,sm,s>>>(P);
    return cudaGetLastError();
  };
  if constexpr(std::is_same<T,float>::value)
    if(P.inplace && hasWideRadix(P.fp)) return go(outerBwdKernel16<T>);
  return go(outerBwdKernel<T>);
}

template<typename T>
cudaError_t launchOuterRealFwd(const OuterPlan<T>& P, int threads,
                               cudaStream_t s)
{
  size_t sm=outerRealSmem<T>(P.L,P.N/2,P.tile);
  cudaError_t e=setSmem(outerRealFwdKernel<T>,sm);
  if(e != cudaSuccess) return e;
  dim3 grid((P.C+P.tile-1)/P.tile,1,P.nbatch*P.count);
  outerRealFwdKernel<T><<<grid,threads,sm,s>>>(P);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launchOuterRealBwd(const OuterPlan<T>& P, int threads,
                               cudaStream_t s)
{
  size_t sm=outerRealSmem<T>(P.L,P.N/2,P.tile);
  cudaError_t e=setSmem(outerRealBwdKernel<T>,sm);
  if(e != cudaSuccess) return e;
  dim3 grid((P.C+P.tile-1)/P.tile,1,P.nbatch*P.count);
  outerRealBwdKernel<T><<<grid,threads,sm,s>>>(P);
  return cudaGetLastError();
}

#define FGB_INSTANTIATE(T) \
  template cudaError_t launchRow<T>(const RowPlan<T>&,int,long long,cudaStream_t); \
  template cudaError_t launchHermRow<T>(const HermRowPlan<T>&,int,long long,cudaStream_t); \
  template cudaError_t launchOuterFwd<T>(const OuterPlan<T>&,int,cudaStream_t); \
  template cudaError_t launchOuterBwd<T>(const OuterPlan<T>&,int,cudaStream_t); \
  template cudaError_t launchOuterRealFwd<T>(const OuterPlan<T>&,int,cudaStream_t); \
  template cudaError_t launchOuterRealBwd<T>(const OuterPlan<T>&,int,cudaStream_t); \
  template size_t rowSmem<T>(int,int,int,int,int,int); \
  template size_t hermRowSmem<T>(int,int,int,int); \
  template size_t outerFwdSmem<T>(int,int,int,int); \
  template size_t outerBwdSmem<T>(int,int,int,int,int); \
  template size_t outerRealSmem<T>(int,int,int); \
  template cudaError_t launchBatch<T>(const BatchArgs<T>&,int,int,size_t,cudaStream_t); \
  template int batchBlocksPerSM<T>(int,size_t,int,int,int);

#if !defined(FGB_ONLY_FLOAT) && !defined(FGB_ONLY_FF)
// Bulk copy by the SMs (16-byte vectors, four in flight per thread): between
// page-locked host memory and the device it reads and writes whole lines
// over the host link.
__global__ void __launch_bounds__(256) bulkCopyKernel(CopyArgs P)
{
  const size_t n=P.bytes/16;
  const size_t stride=(size_t) gridDim.x*blockDim.x;
  for(int a=0; a < P.count; ++a) {
    const uint4 *src=(const uint4 *) P.src[a];
    uint4 *dst=(uint4 *) P.dst[a];
    size_t i=blockIdx.x*(size_t) blockDim.x+threadIdx.x;
    for(; i+3*stride < n; i += 4*stride) {
      uint4 v0=src[i], v1=src[i+stride], v2=src[i+2*stride],
        v3=src[i+3*stride];
      dst[i]=v0; dst[i+stride]=v1; dst[i+2*stride]=v2; dst[i+3*stride]=v3;
    }
    for(; i < n; i += stride) dst[i]=src[i];
  }
}

// Float-float range guard (kernels.cuh, FFScaleArgs).  Block b takes the
// largest biased exponent of chunk b % chunks of array b / chunks (integer
// work on the bit patterns, no FP64 pipe; infinities and NaNs ignored)
// into state[a]; the last block to finish (a wrapping counter in state[8])
// turns them into the scales and zeroes the accumulators.  A chunk is
// FGB_SCAN_CHUNK doubles, all of a thread's loads issued before any is
// used, so the whole scan is one round trip to HBM per wave.  Multipliers
// whose every output is one product of two inputs (or one input) take a
// scale per input, and the output scale is the sum (binary, correlation,
// the Jacobian adjoint).  Those whose outputs add products take one scale
// per factor group so that every term scales alike: the Jacobian
// u0 u3 - u1 u2 shares a scale between u0 and u1 and one between u2 and u3
// (the derivatives of psi and of omega), a dot product sum_k u_k u_{K+k}
// one per half.  A caller's functor gets no scaling.
#define FGB_SCAN_CHUNK 2048
__global__ void __launch_bounds__(256) ffScaleKernel(const FFScaleArgs P)
{
  __shared__ bool last;
  __shared__ unsigned wmax[8];
  const long long chunks=(P.n+FGB_SCAN_CHUNK-1)/FGB_SCAN_CHUNK;
  const int a=(int) (blockIdx.x/chunks);
  const long long c0=(blockIdx.x-a*chunks)*FGB_SCAN_CHUNK;
  const long long c1=min(c0+FGB_SCAN_CHUNK,P.n);
  const unsigned long long *src=P.in[a];
  unsigned m=0;
  auto take=[&](unsigned long long b) {
    const unsigned e=(unsigned) ((b >> 52) & 0x7ff);
    if(e != 0x7ff && e > m) m=e;
  };
  if(((size_t) src & 15) == 0) {
    // Pairs of doubles by 16-byte loads (four per thread); an odd last
    // double is read alone.
    const ulonglong2 *v=(const ulonglong2 *) src;
    const long long p0=c0/2, p1=c1/2;
    ulonglong2 b[FGB_SCAN_CHUNK/512];
#pragma unroll
    for(int u=0; u < FGB_SCAN_CHUNK/512; ++u) {
      const long long i=p0+threadIdx.x+u*256;
      b[u]=i < p1 ? __ldg(v+i) : make_ulonglong2(0,0);
    }
#pragma unroll
    for(int u=0; u < FGB_SCAN_CHUNK/512; ++u) {take(b[u].x); take(b[u].y);}
    if((c1 & 1) && threadIdx.x == 0) take(__ldg(src+c1-1));
  } else {
    unsigned long long b[FGB_SCAN_CHUNK/256];
#pragma unroll
    for(int u=0; u < FGB_SCAN_CHUNK/256; ++u) {
      const long long i=c0+threadIdx.x+u*256;
      b[u]=i < c1 ? __ldg(src+i) : 0ull;
    }
#pragma unroll
    for(int u=0; u < FGB_SCAN_CHUNK/256; ++u) take(b[u]);
  }
  // Block maximum (warp reduction, then across the warps): one atomic per
  // block reaches the shared accumulator of its array.
  m=__reduce_max_sync(0xffffffffu,m);
  if((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5]=m;
  __syncthreads();
  if(threadIdx.x < 32) {
    unsigned v=threadIdx.x < (blockDim.x+31)/32 ? wmax[threadIdx.x] : 0u;
    v=__reduce_max_sync(0xffffffffu,v);
    if(threadIdx.x == 0 && v) atomicMax((unsigned *) P.state+a,v);
  }
  __threadfence();
  __syncthreads();
  if(threadIdx.x == 0)
    last=atomicInc((unsigned *) P.state+8,gridDim.x-1) == gridDim.x-1;
  __syncthreads();
  if(!last || threadIdx.x != 0) return;
  __threadfence();
  int sh[FGB_MAXA];
  for(int a=0; a < P.count; ++a) {
    const unsigned m=atomicExch((unsigned *) P.state+a,0u);
    sh[a]=m ? (int) m-1023 : 0;
  }
  int in[FGB_MAXA], out[FGB_MAXA];
  const bool user=P.mult == MULT_USER;
  for(int a=0; a < P.count; ++a) in[a]=user ? 0 : sh[a];
  if(P.mult == MULT_REALJACOBIAN || P.mult == MULT_JACOBIAN) {
    in[0]=in[1]=max(sh[0],sh[1]);
    in[2]=in[3]=max(sh[2],sh[3]);
  } else if(P.mult == MULT_DOT || P.mult == MULT_REALDOT) {
    const int K=P.count/2;
    int t1=sh[0], t2=sh[K];
    for(int k=1; k < K; ++k) {
      t1=max(t1,sh[k]);
      t2=max(t2,sh[K+k]);
    }
    for(int k=0; k < K; ++k) {
      in[k]=t1;
      in[K+k]=t2;
    }
  }
  for(int b=0; b < P.B; ++b) out[b]=in[b];
  switch(P.mult) {
    case MULT_BINARY: case MULT_REALBINARY: case MULT_CORRELATION:
    case MULT_REALJACOBIAN: case MULT_JACOBIAN:
      out[0]=in[0]+in[P.mult == MULT_REALJACOBIAN ||
                     P.mult == MULT_JACOBIAN ? 3 : 1];
      break;
    case MULT_DOT: case MULT_REALDOT:
      out[0]=in[0]+in[P.count/2];
      break;
    case MULT_REALJACADJ:
      for(int b=0; b < 4; ++b) out[b]=in[4]+in[3-b];
      break;
    default:
      break;
  }
  for(int a=0; a < FGB_MAXA; ++a) {
    P.state[16+a]=a < P.count ? in[a] : 0;
    P.state[24+a]=a < P.B ? out[a] : 0;
  }
}

cudaError_t launchFFScale(const FFScaleArgs& P, cudaStream_t s)
{
  if(P.count < 1 || P.count > FGB_MAXA || P.n < 1) return cudaErrorInvalidValue;
  const long long blocks=(P.n+FGB_SCAN_CHUNK-1)/FGB_SCAN_CHUNK*P.count;
  if(blocks > INT_MAX) return cudaErrorInvalidValue;
  ffScaleKernel<<<(unsigned) blocks,256,0,s>>>(P);
  return cudaGetLastError();
}

// The origin shift of the fft0 transforms (fftw++.h:144-228, fftw::Shift):
// the real values of an nx x ny (x nz) array with (i + j) odd (2D: i odd)
// change sign, which moves the Fourier origin to (nx/2, 0) or
// (nx/2, ny/2, 0).
template<typename R>
__global__ void __launch_bounds__(256) originShiftKernel(R *f, long long nx,
                                                         long long ny,
                                                         long long nz)
{
  const long long n=nx*ny*nz;
  const long long stride=(long long) gridDim.x*blockDim.x;
  for(long long e=blockIdx.x*(long long) blockDim.x+threadIdx.x; e < n;
      e += stride) {
    const long long row=e/nz;        // i*ny + j
    const long long i=row/ny, j=row-i*ny;
    const long long parity=nz > 1 ? i+j : i;
    if(parity & 1) f[e]=-f[e];
  }
}

cudaError_t launchOriginShift(void *f, long long nx, long long ny,
                              long long nz, bool f64, cudaStream_t s)
{
  const long long n=nx*ny*nz;
  if(n <= 0) return cudaSuccess;
  const int grid=(int) std::min<long long>((n+255)/256,152*8);
  if(f64) originShiftKernel<double><<<grid,256,0,s>>>((double *) f,nx,ny,nz);
  else originShiftKernel<float><<<grid,256,0,s>>>((float *) f,nx,ny,nz);
  return cudaGetLastError();
}

cudaError_t launchBulkCopy(const CopyArgs& P, cudaStream_t s)
{
  if(P.bytes % 16) return cudaErrorInvalidValue;
  for(int a=0; a < P.count; ++a)
    if(((size_t) P.src[a] | (size_t) P.dst[a]) % 16)
      return cudaErrorInvalidValue;
  if(P.bytes == 0 || P.count == 0) return cudaSuccess;
  bulkCopyKernel<<<152*8,256,0,s>>>(P);
  return cudaGetLastError();
}
#endif

// Each precision may be compiled as its own translation unit (build.py
// compiles this file once per precision, in parallel): FGB_ONLY_<P> keeps
// one of DOUBLE, FLOAT and FF.
#if !defined(FGB_ONLY_FLOAT) && !defined(FGB_ONLY_FF)
FGB_INSTANTIATE(double)
#endif
#if !defined(FGB_ONLY_DOUBLE) && !defined(FGB_ONLY_FF)
FGB_INSTANTIATE(float)
#endif
#if !defined(FGB_ONLY_DOUBLE) && !defined(FGB_ONLY_FLOAT)
FGB_INSTANTIATE(ff)

#endif

} // namespace fgb
