// wfa_kernels_wide_ef.cu -- the CTA-per-pair alignment kernel in the ends-free
// and extension forms, instantiated from wfa_align.cuh.
#include "wfa_align.cuh"

namespace wf2g {
WF2G_FAULT_READER(wf2g_fault_info_wide_ef)
}  // namespace wf2g

extern "C" void* wf2g_kernel_ptr_wide_ef(int a2p, int enc, int off_bytes, int heur, int lin) {
  return heur ? wf2g::align_kernel<true, 256, true>(a2p, 1, enc, off_bytes, lin)
              : wf2g::align_kernel<false, 256, true>(a2p, 1, enc, off_bytes, lin);
}
