// bw_replay_noalloc.cu -- the event-model replay for callers that cannot allocate
// device memory.
//
// Some hosts of this library cannot call cudaMalloc at the point where they run a
// replay: a plugin that executes inside a database engine's query thread with a
// fixed device-memory budget handed out up front, a real-time loop that must not
// block in the driver's allocator, or a process that forbids allocations after
// start-up.  bw_replay_launch_noalloc gives them the same replay with its scratch
// memory taken from a fixed region compiled into this library instead of a
// caller-provided workspace.  The caller still passes the inputs and the answer
// buffer; nothing is allocated or freed by the call (no cudaMalloc, no cudaFree,
// no allocating library routine).
//
// The region, kNoAllocScratchBytes (32 MiB), is a file-scope __device__ array: every
// GPU that loads this library holds it until the process exits.  Its device address
// is looked up on every call (cudaGetSymbolAddress, with the caller's device
// current): the lookup allocates nothing, and the address stays right when the
// module is reloaded at a different address after the primary context was torn
// down (cudaDeviceReset).  The first call on a device loads the module there, so
// make it before any stream capture.  All calls share the one region and the replay
// initialises every scratch word it reads, so nothing is carried over between
// calls; calls whose work overlaps on the GPU (different streams, or host threads
// racing) would overwrite each other's scratch and must not be issued.  With a
// non-NULL `status` the call waits for its stream and reports the device's input
// check (BW_STATUS_*); with NULL it returns as soon as the work is enqueued and
// that check is not reported (the next call resets the status word).
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "bw_gpu.h"

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

int fail(cudaError_t e, const char* what) {
  std::fprintf(stderr, "bw_replay_launch_noalloc: %s failed: %s\n", what, cudaGetErrorString(e));
  return (int)e;
}

}  // namespace

extern "C" int bw_replay_launch_noalloc(const BwReplayArgs* a, int32_t* status) {
  if (!a) return BW_EINVAL;
  if (a->workspace || a->workspace_bytes) {
    std::fprintf(stderr, "bw_replay_launch_noalloc: leave workspace NULL; the library's own region is used\n");
    return BW_EINVAL;
  }
  void* scratch = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);   // current device's copy
  if (e != cudaSuccess) return fail(e, "cudaGetSymbolAddress");
  size_t need = 0;
  int rc = bw_replay_workspace_size(a, &need);
  if (rc) return rc;
  if (need > kNoAllocScratchBytes) {
    std::fprintf(stderr,
                 "bw_replay_launch_noalloc: this workload needs %zu bytes of scratch, more than the "
                 "library's fixed %zu-byte region; use bw_replay_launch with a workspace\n",
                 need, kNoAllocScratchBytes);
    return BW_EINVAL;
  }
  BwReplayArgs b = *a;
  b.workspace = scratch;
  b.workspace_bytes = kNoAllocScratchBytes;
  rc = bw_replay_launch(&b);
  if (rc || !status) return rc;
  // Input errors found on the device (BW_STATUS_*): reading them waits for the stream.
  return bw_replay_status(&b, status);
}
