/*
 * Source-compatibility shim: the reference's top-level C header
 * "wavefront/wfa.h" (included by its C++ binding through wfa.hpp); with
 * -I<this repo>/include it gets the GB300 library's declarations instead.
 */
#ifndef WFA2GPU_WFA_H_
#define WFA2GPU_WFA_H_
#include "../wfa2gpu.h"
#endif
