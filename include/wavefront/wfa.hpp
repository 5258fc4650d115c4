/*
 * Source-compatibility shim for C++ callers of "wavefront/wfa.hpp": the GB300
 * library's C declarations with C linkage.
 */
#pragma once

extern "C" {
#include "wfa.h"
}
