// wfa_kernels_wide.cu -- the CTA-per-pair alignment kernel (256 threads on one
// pair, full CIGAR, choice bytes in the block pool), instantiated from
// wfa_align.cuh.  Long pairs have rows spanning thousands of diagonals: eight
// warps split each row, share one staged copy of the sequences, and keep one
// pair's back-trace in flight where a warp per pair would keep eight.
#include "wfa_align.cuh"

namespace wf2g {

#define WF2G_INST(A2P, ENC, T, H) \
  template __global__ void wfa_align_kernel<A2P, true, ENC, T, H, 256>(const KParams p);
#define WF2G_INST_H(H)          \
  WF2G_INST(false, 2, int16_t, H) \
  WF2G_INST(true, 2, int16_t, H)  \
  WF2G_INST(false, 8, int16_t, H) \
  WF2G_INST(true, 8, int16_t, H)  \
  WF2G_INST(false, 2, int32_t, H) \
  WF2G_INST(true, 2, int32_t, H)  \
  WF2G_INST(false, 8, int32_t, H) \
  WF2G_INST(true, 8, int32_t, H)
WF2G_INST_H(false)
WF2G_INST_H(true)

template <typename T, bool H>
static void* pick(int a2p, int enc) {
  if (enc == 2) return a2p ? (void*)wfa_align_kernel<true, true, 2, T, H, 256> : (void*)wfa_align_kernel<false, true, 2, T, H, 256>;
  return a2p ? (void*)wfa_align_kernel<true, true, 8, T, H, 256> : (void*)wfa_align_kernel<false, true, 8, T, H, 256>;
}

WF2G_FAULT_READER(wf2g_fault_info_wide)

}  // namespace wf2g

extern "C" void* wf2g_kernel_ptr_wide(int a2p, int enc, int off_bytes, int heur) {
  if (heur) return off_bytes == 2 ? wf2g::pick<int16_t, true>(a2p, enc) : wf2g::pick<int32_t, true>(a2p, enc);
  return off_bytes == 2 ? wf2g::pick<int16_t, false>(a2p, enc) : wf2g::pick<int32_t, false>(a2p, enc);
}
