// Online tuning of the base-chunk count of the distance passes.
//
// The chunk count sets how many CTAs share one query tile (grid = query tiles
// x chunks): more chunks fill the last wave of the GPU better but cost CTA
// start-up (query tile load, TMEM allocation, pipeline fill) and longer
// candidate lists.  For each shape class the tuner tries the heuristic's
// choice and the two next most wave-efficient counts on the calls after a
// first, untimed one (each trial is scored by the CUDA-event time of the pass
// plus the re-rank of its candidates), then keeps the fastest.  Results do not depend on the chunk count.  YAEL_GPU_AUTOTUNE=0
// turns it off (the heuristic's choice is used).
#pragma once
#include "common.cuh"

namespace yg {

struct TuneKey {
  int kind;   // pass: 0 TOPC main, 1 THRESH main, 2 threshold sample, 3 grouped assignment
  int prec;   // distance precision
  int nqt;    // query tiles
  int ntb;    // base tiles
  int C;      // list length
  bool operator<(const TuneKey &o) const;
};

// The chunk count for this call, in [1, cmax].  *ticket >= 0 marks a trial
// whose pass time must be reported with tune_report().
int tune_chunks(const TuneKey &key, int c0, int cmax, int slots, int *ticket);
void tune_report(int ticket, float ms);

// The same scheme over n <= 3 kernel variants (index 0: the default): the
// variant for this call; *ticket >= 0 marks a trial to report.  trial_ok =
// false (a launch being captured into a CUDA graph) returns the best variant
// found so far without taking part; *settled tells whether the choice is final.
int tune_variant(const TuneKey &key, int n, bool trial_ok, int *ticket, bool *settled);

// Per host thread: calls made while it is off use the heuristic (the batched
// k-NN workers share the GPU, so their timings would not be comparable).
void tune_set_thread_enabled(bool on);

}  // namespace yg
