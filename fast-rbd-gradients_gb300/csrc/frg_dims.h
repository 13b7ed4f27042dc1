// Per-knot sizes of the robot compiled into this build (host and device code).
//
// The reference fixes the joint count with a macro (NUM_POS,
// helpers_CPU/dynamicsGradient.h:7-12) and sizes every per-knot array from it;
// here it comes from the model tables (FRG_MODEL_NUM_JOINTS, written by
// frg/urdf.py), 7 for the iiwa_14.
#pragma once
#include "frg_model_select.h"

#ifndef FRG_MODEL_NUM_JOINTS
#define FRG_MODEL_NUM_JOINTS 7
#endif

namespace frg {

constexpr int kN = FRG_MODEL_NUM_JOINTS;     // q, qd, u, qdd per knot
constexpr int kMinvN = kN * kN;              // dense symmetric Minv
// Minv's upper triangle, column by column (entries (r, c), r <= c), padded to
// a multiple of N floats per knot: the form the pipelined host-buffer call
// sends over the host link before expanding it to dense in host memory.
constexpr int kMinvPackedN = kN * ((kN + 2) / 2);
constexpr int kDqddN = 2 * kN * kN;          // [dqdd/dq | dqdd/dqd], N x 2N column-major
constexpr int kFextN = 6 * kN;               // external spatial force per link
constexpr int kRecordN = 4 * kN + kN * kN;   // the reference's knot record [q|qd|u|qdd|Minv]
constexpr int kSlotN = 4 * kN + 3 * kN * kN; // server slot [q|qd|u|dqdd|qdd|minv]
static_assert(kN >= 1 && kN <= 8, "the kernels take 1 to 8 joints");

// Block offsets, in floats per knot, of the [q | qd | u | dqdd | qdd | minv]
// layout of a server slot (and of the engine's own scratch of that shape):
// block b of an h-knot slot starts at kSlot<b> * h.
constexpr int kSlotQd = kN, kSlotU = 2 * kN, kSlotDqdd = 3 * kN, kSlotQdd = 3 * kN + kDqddN,
              kSlotMinv = 4 * kN + kDqddN;

}  // namespace frg
