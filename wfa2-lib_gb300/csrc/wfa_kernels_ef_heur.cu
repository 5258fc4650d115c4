// wfa_kernels_ef_heur.cu -- the warp-per-pair alignment kernel in the
// ends-free and extension forms with the wf-adaptive heuristic, instantiated
// from wfa_align.cuh.
#include "wfa_align.cuh"

namespace wf2g {
WF2G_FAULT_READER(wf2g_fault_info_ef_heur)
}  // namespace wf2g

extern "C" void* wf2g_kernel_ptr_ef_heur(int a2p, int cigar, int enc, int off_bytes, int lin) {
  return wf2g::align_kernel<true, 32, true>(a2p, cigar, enc, off_bytes, lin);
}
