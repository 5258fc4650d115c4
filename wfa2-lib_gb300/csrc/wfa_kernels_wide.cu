// wfa_kernels_wide.cu -- the CTA-per-pair alignment kernel (256 threads on one
// pair, full CIGAR, choice bytes in the block pool), instantiated from
// wfa_align.cuh.  Long pairs have rows spanning thousands of diagonals: eight
// warps split each row, share one staged copy of the sequences, and keep one
// pair's back-trace in flight where a warp per pair would keep eight.
#include "wfa_align.cuh"

namespace wf2g {
WF2G_FAULT_READER(wf2g_fault_info_wide)
}  // namespace wf2g

extern "C" void* wf2g_kernel_ptr_wide(int a2p, int enc, int off_bytes, int heur, int lin) {
  return heur ? wf2g::align_kernel<true, 256, false>(a2p, 1, enc, off_bytes, lin)
              : wf2g::align_kernel<false, 256, false>(a2p, 1, enc, off_bytes, lin);
}
