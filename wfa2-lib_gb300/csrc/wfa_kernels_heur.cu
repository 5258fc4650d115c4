// wfa_kernels_heur.cu -- the warp-per-pair alignment kernel with the
// wf-adaptive heuristic compiled in (wavefront/wavefront_heuristic.c:229-289),
// instantiated from wfa_align.cuh.
#include "wfa_align.cuh"

namespace wf2g {

#define WF2G_INST(A2P, CIG, ENC, T) \
  template __global__ void wfa_align_kernel<A2P, CIG, ENC, T, true, 32>(const KParams p);
#define WF2G_INST_T(T)          \
  WF2G_INST(false, false, 2, T) \
  WF2G_INST(false, true, 2, T)  \
  WF2G_INST(true, false, 2, T)  \
  WF2G_INST(true, true, 2, T)   \
  WF2G_INST(false, false, 8, T) \
  WF2G_INST(false, true, 8, T)  \
  WF2G_INST(true, false, 8, T)  \
  WF2G_INST(true, true, 8, T)
WF2G_INST_T(int16_t)
WF2G_INST_T(int32_t)

template <typename T>
static void* pick(int a2p, int cigar, int enc) {
  if (enc == 2) {
    if (!a2p) return cigar ? (void*)wfa_align_kernel<false, true, 2, T, true, 32> : (void*)wfa_align_kernel<false, false, 2, T, true, 32>;
    return cigar ? (void*)wfa_align_kernel<true, true, 2, T, true, 32> : (void*)wfa_align_kernel<true, false, 2, T, true, 32>;
  }
  if (!a2p) return cigar ? (void*)wfa_align_kernel<false, true, 8, T, true, 32> : (void*)wfa_align_kernel<false, false, 8, T, true, 32>;
  return cigar ? (void*)wfa_align_kernel<true, true, 8, T, true, 32> : (void*)wfa_align_kernel<true, false, 8, T, true, 32>;
}

WF2G_FAULT_READER(wf2g_fault_info_heur)

}  // namespace wf2g

extern "C" void* wf2g_kernel_ptr_heur(int a2p, int cigar, int enc, int off_bytes) {
  return off_bytes == 2 ? wf2g::pick<int16_t>(a2p, cigar, enc) : wf2g::pick<int32_t>(a2p, cigar, enc);
}
