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
    const long long h = sg.h;  // each block of the slot is h knots long
    float *d = sg.dev, *hs = sg.host;
    kp = KnotPtrs{sg.q + kN * i, sg.qd + kN * i, sg.u + kN * i, d + kSlotDqdd * h + kDqddN * i,
                  d + kSlotQdd * h + kN * i, d + kSlotMinv * h + kMinvN * i};
    const bool mirror_in = sg.q != d;
    mr = KnotPtrs{mirror_in ? d + kN * i : nullptr, mirror_in ? d + kSlotQd * h + kN * i : nullptr,
                  mirror_in ? d + kSlotU * h + kN * i : nullptr, hs ? hs + kSlotDqdd * h + kDqddN * i : nullptr,
                  hs ? hs + kSlotQdd * h + kN * i : nullptr, hs ? hs + kSlotMinv * h + kMinvN * i : nullptr};
}

}  // namespace frg
