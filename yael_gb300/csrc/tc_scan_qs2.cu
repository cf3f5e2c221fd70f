// Streamed-query instantiation of the tcgen05 distance kernel, CTA pairs
// (one 256-row MMA over two SMs, tcgen05 cta_group::2).
#include "tc_kernel.cuh"

namespace yg {

int tc_dispatch_s2(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st) {
  return tck::dispatch_metric<true, true>(op, nq, nb, sel, st);
}

}  // namespace yg
