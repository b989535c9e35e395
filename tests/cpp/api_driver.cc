// api_driver.cc -- exercises the FFTW++-compatible C++ API (include/convolve.h)
// the way the reference's own test programs wire it (tests/hybridconv.cc,
// hybridconvh2.cc, hybridconvr3.cc, ...), reading inputs from and writing
// the first output to raw binary files so that tests/test_gpu_api.py can
// compare against the CPU oracle.
//
//   api_driver <case> <A> <infile> <outfile> L... M...
// cases: pad1, cen1, her1, real1, pad2, her2, real2, pad3, her3, real3,
//        jac2 (A=4, Jacobian multiplier), raw1 (convolveRaw), and the
//        strided layouts of tests/hybridconv2.cc, hybridconvh2.cc and
//        hybridconv3.cc: pad2s, her2s (Sx beyond the stored rows), pad3s,
//        real3s (Sy beyond Lz, Sx beyond Ly Sy).  Strided cases fill the
//        gaps with a sentinel and exit with status 4 if any gap changed.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "convolve.h"

using namespace fftwpp;
using namespace utils;

static std::vector<double> slurp(const char *fn)
{
  FILE *f=fopen(fn,"rb");
  if(!f) {perror(fn); exit(2);}
  fseek(f,0,SEEK_END);
  long n=ftell(f);
  fseek(f,0,SEEK_SET);
  std::vector<double> v(n/sizeof(double));
  if(fread(v.data(),1,n,f) != (size_t) n) exit(2);
  fclose(f);
  return v;
}

int main(int argc, char **argv)
{
  if(argc < 6) {fprintf(stderr,"usage\n"); return 2;}
  std::string c=argv[1];
  size_t A=atoi(argv[2]);
  std::vector<double> in=slurp(argv[3]);
  std::vector<size_t> nums;
  for(int i=5; i < argc; ++i) nums.push_back(strtoull(argv[i],NULL,10));
  size_t dim=nums.size()/2;
  std::vector<size_t> L(nums.begin(),nums.begin()+dim);
  std::vector<size_t> M(nums.begin()+dim,nums.end());
  size_t words=in.size()/A;
  // Strided cases: the dense input rows (of `run` doubles) are laid out
  // with `pitch` doubles between consecutive rows of the innermost axis
  // (3D: `plane` doubles between planes of axis 0).
  bool strided=c.size() > 4 && c.back() == 's';
  size_t run=words, pitch=words, plane=words, rows=1, planes=1, Sx=0, Sy=0;
  if(strided) {
    size_t w=c.substr(0,3) == "rea" ? 1 : 2;      // doubles per element
    if(dim == 2) {
      size_t Hy=c == "her2s" ? ceilquotient(L[1],2) : L[1];
      Sx=Hy+3;
      run=w*Hy; pitch=w*Sx; rows=L[0]; plane=pitch*rows; planes=1;
    } else {
      Sy=L[2]+2;
      Sx=L[1]*Sy+5;
      run=w*L[2]; pitch=w*Sy; rows=L[1]; plane=w*Sx; planes=L[0];
    }
  }
  size_t span=strided ? plane*planes : words;
  const double sentinel=12345.0;
  double **f=doubleAlign(A,span);
  for(size_t a=0; a < A; ++a) {
    for(size_t i=0; i < span; ++i) f[a][i]=sentinel;
    for(size_t k=0; k < planes; ++k)
      for(size_t r=0; r < rows; ++r)
        memcpy(f[a]+k*plane+r*pitch,in.data()+a*words+(k*rows+r)*run,
               run*sizeof(double));
  }
  try {
    if(c == "pad1" || c == "raw1") {
      Application app(A,1,multBinary);
      fftPad fft(L[0],M[0],app);
      Convolution C(&fft);
      if(c == "raw1") {
        // convolveRaw leaves the sum unnormalised; divide by the plan's
        // normalization() (convolve.h:1024-1026) to compare.
        C.convolveRaw((Complex **) f);
        double s=1.0/C.normalization();
        for(size_t j=0; j < 2*L[0]; ++j) f[0][j] *= s;
      } else C.convolve((Complex **) f);
    } else if(c == "cen1") {
      Application app(A,1,multBinary);
      fftPadCentered fft(L[0],M[0],app);
      Convolution C(&fft);
      C.convolve((Complex **) f);
    } else if(c == "her1") {
      Application app(A,1,realMultBinary);
      fftPadHermitian fft(L[0],M[0],app);
      Convolution C(&fft);
      C.convolve((Complex **) f);
    } else if(c == "real1") {
      Application app(A,1,multBinary);
      fftPadReal fft(L[0],M[0],app);
      Convolution C(&fft);
      C.convolve(f);
    } else if(c == "pad2") {
      Application appx(A,1,multNone);
      fftPad fftx(L[0],M[0],appx,L[1]);
      Application appy(A,1,multBinary,appx);
      fftPad ffty(L[1],M[1],appy);
      Convolution2 C(&fftx,&ffty);
      C.convolve((Complex **) f);
    } else if(c == "her2" || c == "jac2") {
      size_t Hy=ceilquotient(L[1],2);
      Application appx(A,1,multNone);
      fftPadCentered fftx(L[0],M[0],appx,Hy,Hy);
      Application appy(A,1,c == "jac2" ? jacobianMultiplier : realMultBinary,
                       appx);
      fftPadHermitian ffty(L[1],M[1],appy);
      Convolution2 C(&fftx,&ffty);
      C.convolve((Complex **) f);
    } else if(c == "real2") {
      Application appx(A,1,multNone);
      fftPadReal fftx(L[0],M[0],appx,L[1]);
      Application appy(A,1,multBinary,appx);
      fftPad ffty(L[1],M[1],appy);
      Convolution2 C(&fftx,&ffty);
      C.convolve(f);
    } else if(c == "pad3" || c == "real3") {
      Application appx(A,1,multNone);
      fftBase *fftx=c == "pad3" ?
        (fftBase *) new fftPad(L[0],M[0],appx,L[1]*L[2]) :
        (fftBase *) new fftPadReal(L[0],M[0],appx,L[1]*L[2]);
      Application appy(A,1,multNone,appx);
      fftPad ffty(L[1],M[1],appy,L[2]);
      Application appz(A,1,multBinary,appy);
      fftPad fftz(L[2],M[2],appz);
      Convolution3 C(fftx,&ffty,&fftz);
      C.convolve((Complex **) f);
      delete fftx;
    } else if(c == "pad2s") {
      Application appx(A,1,multNone);
      fftPad fftx(L[0],M[0],appx,L[1],Sx);
      Application appy(A,1,multBinary,appx);
      fftPad ffty(L[1],M[1],appy);
      Convolution2 C(&fftx,&ffty);
      C.convolve((Complex **) f);
    } else if(c == "her2s") {
      size_t Hy=ceilquotient(L[1],2);
      Application appx(A,1,multNone);
      fftPadCentered fftx(L[0],M[0],appx,Hy,Sx);
      Application appy(A,1,realMultBinary,appx);
      fftPadHermitian ffty(L[1],M[1],appy);
      Convolution2 C(&fftx,&ffty);
      C.convolve((Complex **) f);
    } else if(c == "pad3s" || c == "real3s") {
      // tests/hybridconv3.cc:43-49: y-z planes not contiguous (Sy != Lz),
      // so the x transform counts Lz columns.
      Application appx(A,1,multNone);
      fftBase *fftx=c == "pad3s" ?
        (fftBase *) new fftPad(L[0],M[0],appx,L[2],Sx) :
        (fftBase *) new fftPadReal(L[0],M[0],appx,L[2],Sx);
      Application appy(A,1,multNone,appx);
      fftPad ffty(L[1],M[1],appy,L[2],Sy);
      Application appz(A,1,multBinary,appy);
      fftPad fftz(L[2],M[2],appz);
      Convolution3 C(fftx,&ffty,&fftz);
      C.convolve((Complex **) f);
      delete fftx;
    } else if(c == "her3") {
      ConvolutionHermitian3 C(L[0],L[1],L[2],realMultBinary,M[0],M[1],M[2]);
      C.convolve((Complex **) f);
    } else {
      fprintf(stderr,"unknown case %s\n",c.c_str());
      return 2;
    }
  } catch(std::exception& e) {
    fprintf(stderr,"error: %s\n",e.what());
    return 3;
  }
  std::vector<double> dense(words);
  for(size_t k=0; k < planes; ++k)
    for(size_t r=0; r < rows; ++r)
      memcpy(dense.data()+(k*rows+r)*run,f[0]+k*plane+r*pitch,
             run*sizeof(double));
  FILE *o=fopen(argv[4],"wb");
  fwrite(dense.data(),sizeof(double),words,o);
  fclose(o);
  if(strided)          // every gap entry of every array must be untouched
    for(size_t a=0; a < A; ++a)
      for(size_t i=0; i < span; ++i) {
        size_t k=i/plane, in_plane=i-k*plane, r=in_plane/pitch,
          col=in_plane-r*pitch;
        bool data=k < planes && r < rows && col < run;
        if(!data && f[a][i] != sentinel) {
          fprintf(stderr,"gap entry %zu of array %zu changed\n",i,a);
          return 4;
        }
      }
  deleteAlign(f[0]);
  delete [] f;
  return 0;
}
