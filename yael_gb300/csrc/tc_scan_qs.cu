// Streamed-query instantiation of the tcgen05 distance kernel, single CTAs on
// a persistent grid (any Kp; used when the query tile is too large to stay
// resident, and when a work unit holds at most two base tiles).
#include "tc_kernel.cuh"

namespace yg {

int tc_dispatch_s1(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st) {
  return tck::dispatch_metric<true, false>(op, nq, nb, sel, st);
}

}  // namespace yg
