// wfa_kernels.cu -- sm_103a kernels of the GB300 wavefront aligner: the
// warp-per-pair exact end-to-end variants, the block-pool set-up and the
// kernel table.  The alignment kernel itself is the template of
// wfa_align.cuh; its other families (wf-adaptive, ends-free, CTA per pair)
// are built by the wfa_kernels_*.cu units, in parallel with this one.
#include "wfa_align.cuh"

namespace wf2g {

// Pool set-up before a pooled pass: every block free, lock released.
__global__ void wfa_pool_init_kernel(int32_t* stack, int32_t* count, int32_t* lock, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    stack[i] = i;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *count = n;
    *lock = 0;
  }
}

WF2G_FAULT_READER(wf2g_fault_info_exact)

}  // namespace wf2g

extern "C" void* wf2g_kernel_ptr_heur(int a2p, int cigar, int enc, int off_bytes, int lin);
extern "C" void* wf2g_kernel_ptr_ef(int a2p, int cigar, int enc, int off_bytes, int lin);
extern "C" void* wf2g_kernel_ptr_ef_heur(int a2p, int cigar, int enc, int off_bytes, int lin);
extern "C" void* wf2g_kernel_ptr_wide(int a2p, int enc, int off_bytes, int heur, int lin);
extern "C" void* wf2g_kernel_ptr_wide_ef(int a2p, int enc, int off_bytes, int heur, int lin);
extern "C" int wf2g_fault_info_exact(unsigned long long* out);
extern "C" int wf2g_fault_info_heur(unsigned long long* out);
extern "C" int wf2g_fault_info_ef(unsigned long long* out);
extern "C" int wf2g_fault_info_ef_heur(unsigned long long* out);
extern "C" int wf2g_fault_info_wide(unsigned long long* out);
extern "C" int wf2g_fault_info_wide_ef(unsigned long long* out);

// Kernel variant for (affine2p?, full CIGAR?, 2- or 8-bit sequences, 2- or
// 4-byte offsets, wf-adaptive heuristic?, a CTA per pair?, ends-free form?,
// single-component metric?).  The CTA-per-pair variants exist for full-CIGAR
// runs only.
extern "C" void* wf2g_kernel_ptr(int a2p, int cigar, int enc, int off_bytes, int heur, int wide,
                                 int ef, int lin) {
  if (wide) {
    if (!cigar) return nullptr;
    return ef ? wf2g_kernel_ptr_wide_ef(a2p, enc, off_bytes, heur, lin)
              : wf2g_kernel_ptr_wide(a2p, enc, off_bytes, heur, lin);
  }
  if (ef) return heur ? wf2g_kernel_ptr_ef_heur(a2p, cigar, enc, off_bytes, lin)
                      : wf2g_kernel_ptr_ef(a2p, cigar, enc, off_bytes, lin);
  if (heur) return wf2g_kernel_ptr_heur(a2p, cigar, enc, off_bytes, lin);
  return wf2g::align_kernel<false, 32, false>(a2p, cigar, enc, off_bytes, lin);
}

extern "C" void* wf2g_pool_init_ptr(void) { return (void*)wf2g::wfa_pool_init_kernel; }

// First bounds violation seen by a checked build: {site, index, pair, count}
// (the first unit that recorded one; counts add up).
extern "C" int wf2g_fault_info(unsigned long long* out) {
  int (*const readers[6])(unsigned long long*) = {
      wf2g_fault_info_exact, wf2g_fault_info_heur,    wf2g_fault_info_ef,
      wf2g_fault_info_ef_heur, wf2g_fault_info_wide, wf2g_fault_info_wide_ef};
  for (int i = 0; i < 4; ++i) out[i] = 0;
  for (int r = 0; r < 6; ++r) {
    unsigned long long f[4];
    const int rc = readers[r](f);
    if (rc) return rc;
    if (out[0] == 0 && f[0] != 0) {
      out[0] = f[0];
      out[1] = f[1];
      out[2] = f[2];
    }
    out[3] += f[3];
  }
  return 0;
}

// Bytes of both staged sequences of one group for an encoding and length bound.
extern "C" int wf2g_seq_bytes(int enc, int max_len) {
  return enc == 2 ? 2 * wf2g::Seq<2>::words(max_len) * 4 : 2 * wf2g::Seq<8>::words(max_len) * 8;
}
