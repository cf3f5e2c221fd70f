// Streamed-query instantiation of the tcgen05 distance kernel, single CTAs
// (any Kp; used by the split 3xBF16 packing, whose K is three times d).
#include "tc_kernel.cuh"

namespace yg {

int tc_dispatch_s1(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st) {
  return tck::dispatch_metric<true, false>(op, nq, nb, sel, st);
}

}  // namespace yg
