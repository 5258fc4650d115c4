/*
 * Source-compatibility shim: reference callers include "utils/commons.h"
 * (examples/wfa_basic.c:31) for the C standard headers; with -I<this
 * repo>/include they get those headers and the GB300 library's API.
 */
#ifndef WFA2GPU_UTILS_COMMONS_H_
#define WFA2GPU_UTILS_COMMONS_H_
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#endif
