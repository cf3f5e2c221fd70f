// Streamed-query instantiation of the tcgen05 distance kernel (any Kp; used by
// the split 3xBF16 packing, whose K is three times d).
#include "tc_kernel.cuh"

namespace yg {

int tc_dispatch_streaming(const TcOperands &op, int nq, int nb, const ScanSel &sel,
                          cudaStream_t st) {
  if (op.metric == METRIC_L2) return tck::dispatch<true, true>(op, nq, nb, sel, st);
  return tck::dispatch<false, true>(op, nq, nb, sel, st);
}

}  // namespace yg
