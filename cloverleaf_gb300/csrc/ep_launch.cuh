// ep_launch.cuh -- launches of the per-batch kernel chain with programmatic
// dependent launch (sm_90+).
//
// Every kernel of a batch depends on the one before it.  Launched with the
// programmatic-stream-serialization attribute, a kernel's CTAs may be
// scheduled while its predecessor's last wave drains; each such kernel
// begins with pdl_wait() (griddepcontrol.wait: blocks until the predecessor
// grid has completed and its writes are visible) and then pdl_trigger()
// (griddepcontrol.launch_dependents), so its own successor can be scheduled
// once all of its CTAs are running.  A kernel launched without the attribute
// returns from pdl_wait() at once.  Launches recorded into a CUDA graph do
// not use the attribute: a replayed graph already hides launch latency, and
// measured on GB300 the programmatic edges made the replay about 2% slower.
// EP_PDL=0 in the environment launches every chain with ordinary stream
// order.
#pragma once
#include <cuda_runtime.h>

#include <cstdlib>

namespace ep {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

inline bool pdl_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("EP_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

template <typename... KArgs, typename... Args>
inline void launch_chain(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                         Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap);
    attr[0].val.programmaticStreamSerializationAllowed = pdl_enabled() && cap == cudaStreamCaptureStatusNone ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace ep
