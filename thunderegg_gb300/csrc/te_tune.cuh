// te_tune.cuh -- the project's autotuner for launch shapes and kernel variants.
//
// A tunable launch site names a family ("dft_tc", "bcg_patch", ...) and a
// shape key (dimension, patch size, patch-count bucket, types ...) and offers
// a list of candidates.  The first time a (device, family, key) is met on a
// stream that is not being captured, every candidate runs `reps` times after
// one warm-up, timed with CUDA events on that stream, and the fastest median
// is kept for the rest of the process.  Launches made during stream capture
// use the kept choice, or candidate 0 (the default) when nothing has been
// tuned yet; cycles therefore tune their levels before they capture a graph.
//
// TE_TUNE=0 turns tuning off (candidate 0 everywhere).  TE_TUNE_CACHE=<file>
// keeps choices across processes (one line per choice: device name, family,
// key, candidate label); a cached choice is used without timing.
// te_tune_report (te_gpu.h) returns the choices with every candidate's time.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <string>
#include <vector>

namespace te {

struct TuneCandidate {
  std::string label;          // e.g. "tmem ctas=3"
  std::function<void()> run;  // one launch on the tuning stream
};

// Index of the candidate to launch for (family, key) on stream s.
int tune_select(const std::string& family, const std::string& key, const std::vector<TuneCandidate>& cands,
                cudaStream_t s, int reps = 5);

// true when (family, key) already has a choice on the current device, or tuning is off:
// the caller can skip preparing its candidates' scratch buffers
bool tune_settled(const std::string& family, const std::string& key);

// patch-count bucket of a shape key: powers of two, so near sizes share a choice
inline int tune_bucket(long long P) {
  int b = 0;
  while ((1ll << (b + 1)) <= P) b++;
  return b;
}

}  // namespace te
