// Online chunk-count tuner (autotune.cuh).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <mutex>
#include <vector>

#include "autotune.cuh"

namespace yg {

bool TuneKey::operator<(const TuneKey &o) const {
  if (kind != o.kind) return kind < o.kind;
  if (prec != o.prec) return prec < o.prec;
  if (nqt != o.nqt) return nqt < o.nqt;
  if (ntb != o.ntb) return ntb < o.ntb;
  return C < o.C;
}

namespace {

struct Entry {
  bool warm = false;   // the first call of a shape runs untimed (module load, cold caches)
  int n = 0;           // candidates
  int cand[3] = {0, 0, 0};
  float ms[3] = {-1.f, -1.f, -1.f};
  int best = -1;       // index once every candidate has a time
};

std::mutex g_m;
std::map<TuneKey, int> g_index;
std::vector<Entry> g_entries;
thread_local bool t_enabled = true;

bool enabled() {
  static const bool on = [] {
    const char *e = getenv("YAEL_GPU_AUTOTUNE");
    return !(e && strcmp(e, "0") == 0);
  }();
  return on && t_enabled;
}

// chunk count after rounding the tiles per chunk
int effective(int c, int ntb) {
  const int per = (ntb + c - 1) / c;
  return (ntb + per - 1) / per;
}

double wave_eff(int nqt, int c, int slots) {
  const long total = (long)nqt * c;
  const long waves = (total + slots - 1) / slots;
  return (double)total / (double)(waves * slots);
}

}  // namespace

void tune_set_thread_enabled(bool on) { t_enabled = on; }

int tune_chunks(const TuneKey &key, int c0, int cmax, int slots, int *ticket) {
  *ticket = -1;
  c0 = effective(c0 < 1 ? 1 : (c0 > cmax ? cmax : c0), key.ntb);
  if (!enabled()) return c0;
  std::lock_guard<std::mutex> g(g_m);
  auto it = g_index.find(key);
  if (it == g_index.end()) {
    Entry e;
    e.cand[e.n++] = c0;
    // the two most wave-efficient other counts in [c0/2, 3 c0 + 2]
    const int lo = c0 / 2 > 1 ? c0 / 2 : 1, hi = 3 * c0 + 2 < cmax ? 3 * c0 + 2 : cmax;
    for (int pick = 0; pick < 2; pick++) {
      int bc = -1;
      double be = -1;
      for (int c = lo; c <= hi; c++) {
        const int ce = effective(c, key.ntb);
        bool used = false;
        for (int i = 0; i < e.n; i++) used |= e.cand[i] == ce;
        if (used) continue;
        const double ef = wave_eff(key.nqt, ce, slots) - 1e-3 * ce / (double)c0;
        if (ef > be) { be = ef; bc = ce; }
      }
      if (bc > 0) e.cand[e.n++] = bc;
    }
    g_entries.push_back(e);
    it = g_index.emplace(key, (int)g_entries.size() - 1).first;
  }
  Entry &e = g_entries[it->second];
  if (e.best >= 0) return e.cand[e.best];
  if (!e.warm) {
    e.warm = true;
    return e.cand[0];
  }
  for (int i = 0; i < e.n; i++) {
    if (e.ms[i] < 0.f) {
      e.ms[i] = 0.f;  // claimed: a concurrent caller takes the next one
      *ticket = it->second * 4 + i;
      return e.cand[i];
    }
  }
  return e.cand[0];  // every trial is running: the heuristic's choice
}

int tune_variant(const TuneKey &key, int n, bool trial_ok, int *ticket, bool *settled) {
  *ticket = -1;
  *settled = true;
  n = n < 1 ? 1 : (n > 3 ? 3 : n);
  if (!enabled() || n == 1) return 0;
  std::lock_guard<std::mutex> g(g_m);
  auto it = g_index.find(key);
  if (!trial_ok) {
    if (it == g_index.end() || g_entries[it->second].best < 0) {
      *settled = false;
      return 0;
    }
    const Entry &e = g_entries[it->second];
    return e.cand[e.best];
  }
  *settled = false;
  if (it == g_index.end()) {
    Entry e;
    for (int i = 0; i < n; i++) e.cand[e.n++] = i;
    g_entries.push_back(e);
    it = g_index.emplace(key, (int)g_entries.size() - 1).first;
  }
  Entry &e = g_entries[it->second];
  if (e.best >= 0) {
    *settled = true;
    return e.cand[e.best];
  }
  if (!e.warm) {
    e.warm = true;
    return e.cand[0];
  }
  for (int i = 0; i < e.n; i++) {
    if (e.ms[i] < 0.f) {
      e.ms[i] = 0.f;
      *ticket = it->second * 4 + i;
      return e.cand[i];
    }
  }
  return e.cand[0];
}

void tune_report(int ticket, float ms) {
  if (ticket < 0) return;
  std::lock_guard<std::mutex> g(g_m);
  Entry &e = g_entries[ticket / 4];
  e.ms[ticket % 4] = ms > 0.f ? ms : 1e-6f;
  int b = 0;
  for (int i = 0; i < e.n; i++) {
    if (e.ms[i] <= 0.f) return;  // untried or still running
    if (e.ms[i] < e.ms[b]) b = i;
  }
  e.best = b;
  if (trace_enabled()) {
    for (const auto &kv : g_index) {
      if (kv.second != ticket / 4) continue;
      fprintf(stderr, "[yael_gpu] autotune kind=%d key=(%d,%d,%d): candidate %d (", kv.first.kind,
              kv.first.nqt, kv.first.ntb, kv.first.C, e.cand[b]);
      for (int i = 0; i < e.n; i++) fprintf(stderr, "%s%d: %.3f ms", i ? ", " : "", e.cand[i], e.ms[i]);
      fprintf(stderr, ")\n");
    }
  }
}

}  // namespace yg
