// Test shim: the GPU library's host-side k-means draws (km_host.h) on host
// arrays, so that a CPU test compares them with the oracle's restatements:
// the random initialisation, and the empty-cluster split with the device
// gather and scatter of the touched rows replaced by host copies.
#include <string.h>

#include "../yael_gb300/csrc/km_host.h"

// the first k of the partial Fisher-Yates shuffle of 0..n-1 from seed
extern "C" void shim_random_init(int n, int k, unsigned seed, long *sel) {
  yg::random_init_first_k(n, k, seed, sel);
}

// ni instances of k centroids (C: ni * k * d floats, nassign: ni * k counts),
// each split with its own seed when it has an empty cluster; nre receives
// the splits per instance.  Returns the total.
extern "C" int shim_split(int d, int k, int ni, float *C, const int *nassign,
                          const unsigned *seeds, int *nre) {
  using namespace yg;
  std::vector<SplitStep> plan;
  std::vector<int> pinst, pat;
  for (int i = 0; i < ni; i++) {
    const int *cnt = nassign + (long)i * k;
    bool empty = false;
    for (int c = 0; c < k; c++) empty |= cnt[c] == 0;
    nre[i] = 0;
    if (!empty) continue;
    pinst.push_back(i);
    pat.push_back((int)plan.size());
    nre[i] = split_plan(k, cnt, seeds[i], plan);
  }
  if (plan.empty()) return 0;
  SplitRows sr;
  split_rows(k, plan, pinst, pat, sr);
  std::vector<float> R(sr.rows.size() * (size_t)d);
  for (size_t r = 0; r < sr.rows.size(); r++)
    memcpy(&R[r * d], C + sr.rows[r] * d, sizeof(float) * d);
  split_apply_rows(d, k, plan, pinst, pat, sr, R.data());
  for (size_t r = 0; r < sr.rows.size(); r++)
    memcpy(C + sr.rows[r] * d, &R[r * d], sizeof(float) * d);
  return (int)plan.size();
}
