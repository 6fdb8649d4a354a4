/*
 * Prelude for compiling one reference kernel file as C++ (TEST
 * INFRASTRUCTURE ONLY). Standard headers must come first: the reference's
 * include/device_types.h defines bool/true/false as macros when it is not
 * compiled as OpenCL, which would break any header included after it.
 */
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include "../../sampo_gb300/csrc/sampo_math.h"

extern thread_local size_t clc_tls_gid;
extern thread_local size_t clc_tls_gsize;
