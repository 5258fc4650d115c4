/*
 * Source-compatibility shim: a caller of smarco/WFA2-lib includes
 * "wavefront/wavefront_align.h" (examples/wfa_basic.c:32); with -I<this
 * repo>/include it gets the GB300 library's declarations instead.
 */
#ifndef WFA2GPU_WAVEFRONT_ALIGN_H_
#define WFA2GPU_WAVEFRONT_ALIGN_H_
#include "../wfa2gpu.h"
#endif
