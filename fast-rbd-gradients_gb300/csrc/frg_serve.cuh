// Addressing of one knot of a served call (frg_server), shared by the
// server's two thread mappings.
#pragma once
#include "frg_kernels.cuh"
#include "frg_knot.cuh"

namespace frg {

// Knot i of a served call: inputs and device-slot results (kp); the input
// mirror into the device slot and the host-slot results (mr, null where not
// wanted).
__device__ __forceinline__ void serve_knot(const ServeSegment &sg, long long i, KnotPtrs &kp, KnotPtrs &mr) {
    const long long h = sg.h;
    float *d = sg.dev, *hs = sg.host;
    kp = KnotPtrs{sg.q + 7 * i, sg.qd + 7 * i, sg.u + 7 * i, d + 21 * h + 98 * i, d + 119 * h + 7 * i,
                  d + 126 * h + 49 * i};
    const bool mirror_in = sg.q != d;
    mr = KnotPtrs{mirror_in ? d + 7 * i : nullptr, mirror_in ? d + 7 * h + 7 * i : nullptr,
                  mirror_in ? d + 14 * h + 7 * i : nullptr, hs ? hs + 21 * h + 98 * i : nullptr,
                  hs ? hs + 119 * h + 7 * i : nullptr, hs ? hs + 126 * h + 49 * i : nullptr};
}

}  // namespace frg
