// batch.h -- many independent 1D convolutions of uneven lengths in one
// persistent launch (kernels.cuh, BatchArgs), optionally replayed from a
// captured CUDA graph.
#pragma once

#include "engine.h"
#include "kernels.cuh"

#include <vector>

namespace fgb {

// A long problem's task counts for the queue order: staging bytes, forward
// column tiles (each once per input), row tasks, backward column tiles
// (each once per output).
struct LongTasks {
  int prob;
  size_t staging;
  int fwdTiles, rows, bwdTiles;
};
std::vector<BatchTask> orderBatchTasks(const std::vector<LongTasks>& lng,
                                       const std::vector<int>& small, int A,
                                       int B, size_t groupBytes);

class BatchConv {
public:
  // n problems of lengths L[i] padded to >= M[i]; data packed back to back
  // in every input/output array.  choice: NULL or per-problem plan
  // (> 0 residue block m of a one-CTA problem, < 0 minus the row length of
  // a long problem); tune: time the candidate plans (autotuner).
  BatchConv(int n, const long *L, const long *M, const long *choice, int A,
            int B, int mult, int prec, int kind, bool tune);
  ~BatchConv();

  cudaError_t run(const void *const *in, void *const *out, cudaStream_t s);
  // Capture the launch (counter reset + persistent kernel) once per set of
  // array pointers and replay the graph on s.
  cudaError_t runGraph(const void *const *in, void *const *out,
                       cudaStream_t s);
  // Nonzero if a bounded wait inside the kernel gave up (reading clears it).
  int error();

  // Failure detection: polls before a dependency wait gives up (default
  // 2e7, seconds), and a test hook that makes the waits of long problem i
  // unreachable so that they time out (blocked) or restores them.
  void setSpinLimit(long long polls);
  cudaError_t blockProblem(int i, bool blocked);

  long choice(int i) const;
  int tasks() const {return ntasks;}
  int gridSize() const {return grid;}
  size_t smemBytes() const {return smem;}
  long totalLength() const {return total;}
  int shortProblems() const {return nsmall;}
  int longProblems() const {return nlong;}
  int precision() const {return prec;}
  int inputs() const {return A;}
  int outputs() const {return B;}

  static std::vector<long> candidates(long L, long M, int A, int B, int prec,
                                      size_t budget);

private:
  int n, A, B, mult, prec, kind;
  long long spinLimit=20000000LL;
  int tileCap=128;                 // widest column tile of a long problem
  void release();
  double timeLaunch(int reps);
  int nlongCount() const;
  std::vector<int> nfwd0;          // per problem: forward tasks a row waits for
  size_t probBytes=0, nfwdOffset=0;
  std::vector<long> Ls, Ms, offsets, choices;
  long total;
  void *dProbs, *dTasks, *dCounters, *staging;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  cudaStream_t captureStream;
  std::vector<const void *> graphKey;
  size_t smem, budget;
  int grid;
  size_t stagingSize;
  int ntasks, nsmall, nlong;

  long tuned(long L, long M, const std::vector<long>& cand);
  template<typename T> void build();
  template<typename T> cudaError_t launch(const void *const *in,
                                          void *const *out, cudaStream_t s);
};

} // namespace fgb
