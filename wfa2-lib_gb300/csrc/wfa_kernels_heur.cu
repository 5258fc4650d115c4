// wfa_kernels_heur.cu -- the warp-per-pair alignment kernel with the
// wf-adaptive heuristic compiled in (wavefront/wavefront_heuristic.c:229-289),
// instantiated from wfa_align.cuh.
#include "wfa_align.cuh"

namespace wf2g {
WF2G_FAULT_READER(wf2g_fault_info_heur)
}  // namespace wf2g

extern "C" void* wf2g_kernel_ptr_heur(int a2p, int cigar, int enc, int off_bytes, int lin) {
  return wf2g::align_kernel<true, 32, false>(a2p, cigar, enc, off_bytes, lin);
}
