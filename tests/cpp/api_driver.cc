// api_driver.cc -- exercises the FFTW++-compatible C++ API (include/convolve.h)
// the way the reference's own test programs wire it (tests/hybridconv.cc,
// hybridconvh2.cc, hybridconvr3.cc, ...), reading inputs from and writing
// the first output to raw binary files so that tests/test_gpu_api.py can
// compare against the CPU oracle.
//
//   api_driver <case> <A> <infile> <outfile> L... M...
// cases: pad1, cen1, her1, real1, pad2, her2, real2, pad3, her3, real3,
//        jac2 (A=4, Jacobian multiplier), raw1 (convolveRaw).
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
  double **f=doubleAlign(A,words);
  for(size_t a=0; a < A; ++a) memcpy(f[a],in.data()+a*words,words*sizeof(double));
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
  FILE *o=fopen(argv[4],"wb");
  fwrite(f[0],sizeof(double),words,o);
  fclose(o);
  deleteAlign(f[0]);
  delete [] f;
  return 0;
}
