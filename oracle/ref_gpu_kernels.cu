// The reference's own GPU kernel, compiled UNMODIFIED from the reference tree
// into a device-only module (oracle/_ref/ref_gpu.cubin) for sm_103a.
//
// ORACLE TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile where the
// reference sources are present; a cubin is device code, so the file also runs
// on a GPU machine of another host architecture.  tests/test_gpu_reference_kernel.py
// loads it through the CUDA driver API, checks the engine's gradient against it
// on the same GB300 and times both.  Never linked into the product library.
//
// dynamicsGradientKernel<T, KNOT_POINTS, MPC_MODE, VEL_DAMPING>
// (helpers_GPU/dynamicsGradient.cuh:1257-1292) is the reference's "Completely
// Fused" kernel, launched <<<KNOT_POINTS, dim3(32, NUM_POS)>>> at
// time_GPU.cu:314 and :326: per knot it takes [q | qd | u | qdd | Minv]
// (4 NUM_POS + NUM_POS^2 floats, time_GPU.cu:137-158) and the 72 NUM_POS model
// constants, and writes the 2 NUM_POS^2-float gradient.  Instantiated here for
// the batch sizes of time_GPU.cu's main in the reference's default mode
// (MPC_MODE_GLOBAL = VEL_DAMPING_GLOBAL = false, utils/experiment_helpers.h:
// 19-20), and for the other three modes at 1024 knots.
#include "utils/experiment_helpers.h"
#include "helpers_CPU/dynamicsGradient.h"
#include "helpers_GPU/dynamicsGradient.cuh"

template __global__ void dynamicsGradientKernel<float, 16, false, false>(float *, float *, float *);
template __global__ void dynamicsGradientKernel<float, 32, false, false>(float *, float *, float *);
template __global__ void dynamicsGradientKernel<float, 64, false, false>(float *, float *, float *);
template __global__ void dynamicsGradientKernel<float, 128, false, false>(float *, float *, float *);
template __global__ void dynamicsGradientKernel<float, 1024, false, false>(float *, float *, float *);
template __global__ void dynamicsGradientKernel<float, 65536, false, false>(float *, float *, float *);
template __global__ void dynamicsGradientKernel<float, 1024, false, true>(float *, float *, float *);
template __global__ void dynamicsGradientKernel<float, 1024, true, false>(float *, float *, float *);
template __global__ void dynamicsGradientKernel<float, 1024, true, true>(float *, float *, float *);
