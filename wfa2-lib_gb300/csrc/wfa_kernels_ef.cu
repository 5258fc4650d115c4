// wfa_kernels_ef.cu -- the warp-per-pair alignment kernel in the ends-free and
// extension forms (wavefront/wavefront_attributes.h:55-69), exact,
// instantiated from wfa_align.cuh.
#include "wfa_align.cuh"

namespace wf2g {
WF2G_FAULT_READER(wf2g_fault_info_ef)
}  // namespace wf2g

extern "C" void* wf2g_kernel_ptr_ef(int a2p, int cigar, int enc, int off_bytes, int lin) {
  return wf2g::align_kernel<false, 32, true>(a2p, cigar, enc, off_bytes, lin);
}
