// Programmatic dependent launch for the engine's kernels.
//
// Every gradient kernel is launched with programmatic stream serialization and
// begins with dependent_launch_begin(): it lets the next kernel on its stream
// be scheduled at once (griddepcontrol.launch_dependents), then waits until
// the work before it on the stream has completed and its memory is visible
// (griddepcontrol.wait) before it reads or writes anything.  Stream order is
// unchanged; what overlaps is the next launch's scheduling and CTA start with
// this launch's last tiles, a few microseconds per launch that back-to-back
// launches (solver iterations, plan replays) otherwise spend idle.  A kernel
// before it that does not trigger early (another library's, a copy) is simply
// waited for, as without the attribute.
#pragma once
#include <cuda_runtime.h>

namespace frg {

__device__ __forceinline__ void dependent_launch_begin() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Brings the line holding p into L2.  Only a hint: a kernel may issue it
// before dependent_launch_begin() for the inputs of its first tile, so their
// DRAM latency overlaps the end of the work ahead of it on the stream.  The
// loads that use the data come after the wait, and L2 is the GPU's point of
// coherence, so an input that the work ahead still writes is read correctly.
__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// A lane's knot inputs (q, qd, u of a KnotPtrs) into L2; idle lanes
// (q == nullptr) issue nothing.
template <typename Ptrs>
__device__ __forceinline__ void prefetch_knot_inputs(const Ptrs &kp) {
    if (kp.q) {
        prefetch_l2(kp.q);
        prefetch_l2(kp.qd);
        prefetch_l2(kp.u);
    }
}

template <typename... KArgs, typename... Args>
cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                             Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace frg
