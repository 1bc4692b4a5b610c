/* Stand-in for the reference's gpu_session.h when its GPU workers are compiled against this
 * repository's C ABI (oracle/ref.mk target "dropin"): the structs and entry points
 * the reference header declares are declared, with the same layouts and names, by
 * include/bw_gpu.h.  Test infrastructure only. */
#pragma once
#include "bw_gpu.h"
