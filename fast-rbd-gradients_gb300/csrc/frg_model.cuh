// iiwa_14 model and spatial algebra for the sm_103a kernels.
//
// The reference code-generates the model as dense 6x6 constants
// (helpers_CPU/dynamicsGradient.h:124-229, :231-587; helpers_GPU/
// dynamicsGradient.cuh:313-407).  Here each joint transform is described by
// its structure instead:
//
//   iX(i-1) = [E 0; -E r^ E],   E = Rz(q)^T F,
//
// F a fixed signed permutation (the joint frame's rpy from utils/iiwa_14.urdf)
// and r = t * e_axis the joint origin (one nonzero component for every iiwa
// joint).  Applying X or X^T then costs two plane rotations and two FMAs.  The
// spatial inertias use the structure I = [Ibar, m c^; m c^T, m 1] with
// compile-time constants, so structurally zero terms drop out at compile time.
#pragma once
#include <cuda_runtime.h>

#include "frg_dims.h"

// Scalar type of the device code: float for the engine; the FP64 verification
// build (frg_f64_kernels.cu) compiles the same code with FRG_REAL=double into
// namespace frg64.
#ifndef FRG_REAL
#define FRG_REAL float
#endif
#ifndef FRG_NS
#define FRG_NS frg
#endif

namespace FRG_NS {

using real = FRG_REAL;
__device__ __forceinline__ real fmaR(real a, real b, real c) {
    if constexpr (sizeof(real) == sizeof(float)) return fmaf(a, b, c);
    else return fma(a, b, c);
}

constexpr int kJoints = FRG_MODEL_NUM_JOINTS;
constexpr real kGravity = real(9.81);  // GRAVITY default, dynamicsGradient.h:7-9

template <int N> struct IC { static constexpr int value = N; };

// Compile-time loops (the link index must be a constant expression so that the
// per-joint structure and the register arrays indexed by it resolve statically).
template <int B, int E, typename F> __device__ __forceinline__ void static_for(F &&f) {
    if constexpr (B < E) {
        f(IC<B>{});
        static_for<B + 1, E>(f);
    }
}
template <int B, int E, typename F> __device__ __forceinline__ void static_for_down(F &&f) {
    if constexpr (B >= E) {
        f(IC<B>{});
        static_for_down<B - 1, E>(f);
    }
}

// ------------------------------------------------------------------ model ---

// The robot comes from one header of tables (written by frg/urdf.py from a
// URDF): the build defines FRG_MODEL_TABLES to select another robot; the
// default is the iiwa_14 of utils/iiwa_14.urdf, the reference's only model.
#include "frg_model_select.h"

// Link inertia at the COM (xx xy xz yy yz zz), COM position (x y z), mass, in
// the link frame.  For the iiwa these are the reference's l0..l6 constants
// (dynamicsGradient.h:127-202).
struct LinkInertial { double ixx, ixy, ixz, iyy, iyz, izz, cx, cy, cz, m; };
constexpr LinkInertial kLinks[kJoints] = FRG_MODEL_LINK_INERTIAL;
// Joint frames: F = R^T of the joint frame in its parent (column-major), the
// joint origin r in the parent frame (the iiwa's tz_j1..ty_j7,
// dynamicsGradient.h:223-229).
constexpr double kModelF[kJoints][9] = FRG_MODEL_JOINT_F;
constexpr double kModelOrigin[kJoints][3] = FRG_MODEL_JOINT_ORIGIN;
// Column 0 of d tau / dq vanishes identically when gravity lies along the
// first joint's axis (the iiwa; the reference relies on it at :797-813).
constexpr bool kDqColumn0Zero = FRG_MODEL_DQ_COLUMN0_ZERO != 0;

// Spatial inertia about the joint origin: rotational block Ibar = Icom +
// m (|c|^2 1 - c c^T) (the parallel-axis shift buildI6x6 applies,
// dynamicsGradient.h:78-118), coupling m c, mass m.
template <int k> struct Link {
    static constexpr LinkInertial L = kLinks[k];
    static constexpr real Ixx = real(L.ixx + L.m * (L.cy * L.cy + L.cz * L.cz));
    static constexpr real Iyy = real(L.iyy + L.m * (L.cx * L.cx + L.cz * L.cz));
    static constexpr real Izz = real(L.izz + L.m * (L.cx * L.cx + L.cy * L.cy));
    static constexpr real Ixy = real(L.ixy - L.m * L.cx * L.cy);
    static constexpr real Ixz = real(L.ixz - L.m * L.cx * L.cz);
    static constexpr real Iyz = real(L.iyz - L.m * L.cy * L.cz);
    static constexpr real mcx = real(L.m * L.cx), mcy = real(L.m * L.cy), mcz = real(L.m * L.cz);
    static constexpr real m = real(L.m);
};

// Structure of each joint frame, found at compile time.  A signed
// permutation F (frames in multiples of pi/2, as every iiwa joint) maps w to
// (F w)[p_i] = s_i w_i; an origin on one axis (every iiwa joint) is
// r = t e_axis.  Other frames take the general 3x3 / cross-product forms.
//   iiwa rpy (0,0,0):                 p = {0,1,2}, s = {+,+,+}
//   iiwa rpy (pi/2,0,pi), (-pi/2,pi,0): p = {0,2,1}, s = {-,+,+}   w -> (-w0, w2, w1)
//   iiwa rpy (pi/2,0,0):              p = {0,2,1}, s = {+,-,+}   w -> (w0, w2, -w1)
__host__ __device__ constexpr double kF(int k, int r, int c) { return kModelF[k][r + 3 * c]; }
__host__ __device__ constexpr int perm_row(int k, int c) {
    int row = -1, n = 0;
    for (int r = 0; r < 3; r++)
        if (kF(k, r, c) != 0.0) { row = r; n++; }
    return (n == 1 && (kF(k, row, c) == 1.0 || kF(k, row, c) == -1.0)) ? row : -1;
}
__host__ __device__ constexpr bool signed_perm(int k) {
    const int a = perm_row(k, 0), b = perm_row(k, 1), c = perm_row(k, 2);
    return a >= 0 && b >= 0 && c >= 0 && a != b && b != c && a != c;
}
__host__ __device__ constexpr int origin_axis(int k) {  // 0..2: one nonzero component; 3: r = 0; -1: general
    int axis = 3, n = 0;
    for (int i = 0; i < 3; i++)
        if (kModelOrigin[k][i] != 0.0) { axis = i; n++; }
    return n <= 1 ? axis : -1;
}
template <int k> struct Joint {
    static constexpr bool perm = signed_perm(k);
    static constexpr int p0 = perm ? perm_row(k, 0) : 0, p1 = perm ? perm_row(k, 1) : 1, p2 = perm ? perm_row(k, 2) : 2;
    static constexpr real s0 = real(kF(k, p0, 0)), s1 = real(kF(k, p1, 1)), s2 = real(kF(k, p2, 2));
    static constexpr int axis = origin_axis(k);
    static constexpr real t = (axis >= 0 && axis < 3) ? real(kModelOrigin[k][axis]) : real(0);
    static constexpr real r0 = real(kModelOrigin[k][0]), r1 = real(kModelOrigin[k][1]), r2 = real(kModelOrigin[k][2]);
};

// acc += K x for a compile-time K, dropped when K == 0
template <typename KC> __device__ __forceinline__ void fma_const(real &acc, KC, real x) {
    if constexpr (KC::value != 0.0) acc = fmaR(real(KC::value), x, acc);
}
template <int k, int r, int c> struct FEntry { static constexpr double value = kModelF[k][r + 3 * c]; };

// ------------------------------------------------------- 3-vector pieces ---

// F w for joint k (general frames)
template <int k> __device__ __forceinline__ void mul_F(real o[3], const real w[3]) {
    static_for<0, 3>([&](auto R) {
        constexpr int r = decltype(R)::value;
        real acc = real(0);
        fma_const(acc, FEntry<k, r, 0>{}, w[0]);
        fma_const(acc, FEntry<k, r, 1>{}, w[1]);
        fma_const(acc, FEntry<k, r, 2>{}, w[2]);
        o[r] = acc;
    });
}
// F^T w for joint k (general frames)
template <int k> __device__ __forceinline__ void mul_FT(real o[3], const real w[3]) {
    static_for<0, 3>([&](auto C) {
        constexpr int c = decltype(C)::value;
        real acc = real(0);
        fma_const(acc, FEntry<k, 0, c>{}, w[0]);
        fma_const(acc, FEntry<k, 1, c>{}, w[1]);
        fma_const(acc, FEntry<k, 2, c>{}, w[2]);
        o[c] = acc;
    });
}

// E w = Rz(q)^T (F w)
template <int k> __device__ __forceinline__ void rot_E(real o[3], const real w[3], real c, real s) {
    using J = Joint<k>;
    real fw[3];
    if constexpr (J::perm) {
        fw[J::p0] = J::s0 * w[0];
        fw[J::p1] = J::s1 * w[1];
        fw[J::p2] = J::s2 * w[2];
    } else {
        mul_F<k>(fw, w);
    }
    o[0] = fmaR(c, fw[0], s * fw[1]);
    o[1] = fmaR(c, fw[1], -s * fw[0]);
    o[2] = fw[2];
}

// E^T w = F^T (Rz(q) w),  (F^T x)_i = s_i x[p_i] for a signed permutation
template <int k> __device__ __forceinline__ void rot_ET(real o[3], const real w[3], real c, real s) {
    using J = Joint<k>;
    real x[3];
    x[0] = fmaR(c, w[0], -s * w[1]);
    x[1] = fmaR(c, w[1], s * w[0]);
    x[2] = w[2];
    if constexpr (J::perm) {
        o[0] = J::s0 * x[J::p0];
        o[1] = J::s1 * x[J::p1];
        o[2] = J::s2 * x[J::p2];
    } else {
        mul_FT<k>(o, x);
    }
}

// o = u + sgn (r x w)  (sgn = -1: u - r x w)
template <int k, int sgn> __device__ __forceinline__ void r_cross_acc(real o[3], const real u[3], const real w[3]) {
    using J = Joint<k>;
    constexpr real g = real(sgn);
    if constexpr (J::axis == 2) {  // r x w = (-t w1, t w0, 0)
        o[0] = fmaR(-g * J::t, w[1], u[0]);
        o[1] = fmaR(g * J::t, w[0], u[1]);
        o[2] = u[2];
    } else if constexpr (J::axis == 1) {  // r x w = (t w2, 0, -t w0)
        o[0] = fmaR(g * J::t, w[2], u[0]);
        o[1] = u[1];
        o[2] = fmaR(-g * J::t, w[0], u[2]);
    } else if constexpr (J::axis == 0) {  // r x w = (0, -t w2, t w1)
        o[0] = u[0];
        o[1] = fmaR(-g * J::t, w[2], u[1]);
        o[2] = fmaR(g * J::t, w[1], u[2]);
    } else if constexpr (J::axis == 3) {  // r = 0
        o[0] = u[0]; o[1] = u[1]; o[2] = u[2];
    } else {  // r x w = (r1 w2 - r2 w1, r2 w0 - r0 w2, r0 w1 - r1 w0)
        o[0] = fmaR(-g * J::r2, w[1], fmaR(g * J::r1, w[2], u[0]));
        o[1] = fmaR(-g * J::r0, w[2], fmaR(g * J::r2, w[0], u[1]));
        o[2] = fmaR(-g * J::r1, w[0], fmaR(g * J::r0, w[1], u[2]));
    }
}

// o = u - r x w
template <int k> __device__ __forceinline__ void sub_r_cross(real o[3], const real u[3], const real w[3]) {
    r_cross_acc<k, -1>(o, u, w);
}

// o = u + r x w
template <int k> __device__ __forceinline__ void add_r_cross(real o[3], const real u[3], const real w[3]) {
    r_cross_acc<k, 1>(o, u, w);
}

// ------------------------------------------------------- spatial vectors ---

// y = X_k x  (motion vector to the child frame):  [E w; E (v - r x w)]
template <int k> __device__ __forceinline__ void xmotion(real y[6], const real x[6], real c, real s) {
    real u[3];
    rot_E<k>(y, x, c, s);
    sub_r_cross<k>(u, x + 3, x);
    rot_E<k>(y + 3, u, c, s);
}

// y = X_k^T x  (force vector to the parent frame):  [E^T n + r x (E^T f); E^T f]
template <int k> __device__ __forceinline__ void xforce_T(real y[6], const real x[6], real c, real s) {
    real n[3];
    rot_ET<k>(y + 3, x + 3, c, s);
    rot_ET<k>(n, x, c, s);
    add_r_cross<k>(y, n, y + 3);
}

#define FRG_ACC(acc, K, x)                   \
    if constexpr ((K) != real(0)) {             \
        acc = fmaR((K), (x), acc);           \
    }

// y = I_k w:  [Ibar w + mc x v; m v - mc x w]
template <int k> __device__ __forceinline__ void imul(real y[6], const real x[6]) {
    using L = Link<k>;
    const real w0 = x[0], w1 = x[1], w2 = x[2], v0 = x[3], v1 = x[4], v2 = x[5];
    real t0 = L::Ixx * w0, t1 = L::Iyy * w1, t2 = L::Izz * w2;
    FRG_ACC(t0, L::Ixy, w1) FRG_ACC(t0, L::Ixz, w2)
    FRG_ACC(t1, L::Ixy, w0) FRG_ACC(t1, L::Iyz, w2)
    FRG_ACC(t2, L::Ixz, w0) FRG_ACC(t2, L::Iyz, w1)
    // + mc x v = (mcy v2 - mcz v1, mcz v0 - mcx v2, mcx v1 - mcy v0)
    FRG_ACC(t0, L::mcy, v2) FRG_ACC(t0, -L::mcz, v1)
    FRG_ACC(t1, L::mcz, v0) FRG_ACC(t1, -L::mcx, v2)
    FRG_ACC(t2, L::mcx, v1) FRG_ACC(t2, -L::mcy, v0)
    real b0 = L::m * v0, b1 = L::m * v1, b2 = L::m * v2;
    // - mc x w
    FRG_ACC(b0, -L::mcy, w2) FRG_ACC(b0, L::mcz, w1)
    FRG_ACC(b1, -L::mcz, w0) FRG_ACC(b1, L::mcx, w2)
    FRG_ACC(b2, -L::mcx, w1) FRG_ACC(b2, L::mcy, w0)
    y[0] = t0; y[1] = t1; y[2] = t2; y[3] = b0; y[4] = b1; y[5] = b2;
}

// y = I_k S = I_k e_2 (third column, constant)
template <int k> __device__ __forceinline__ void icol2(real y[6]) {
    using L = Link<k>;
    y[0] = L::Ixz; y[1] = L::Iyz; y[2] = L::Izz;
    y[3] = -L::mcy; y[4] = L::mcx; y[5] = 0.0f;
}

// y += crf(v) h = v x* h
__device__ __forceinline__ void crf_acc(real y[6], const real v[6], const real h[6]) {
    y[0] = fmaR(v[1], h[2], fmaR(-v[2], h[1], fmaR(v[4], h[5], fmaR(-v[5], h[4], y[0]))));
    y[1] = fmaR(v[2], h[0], fmaR(-v[0], h[2], fmaR(v[5], h[3], fmaR(-v[3], h[5], y[1]))));
    y[2] = fmaR(v[0], h[1], fmaR(-v[1], h[0], fmaR(v[3], h[4], fmaR(-v[4], h[3], y[2]))));
    y[3] = fmaR(v[1], h[5], fmaR(-v[2], h[4], y[3]));
    y[4] = fmaR(v[2], h[3], fmaR(-v[0], h[5], y[4]));
    y[5] = fmaR(v[0], h[4], fmaR(-v[1], h[3], y[5]));
}

}  // namespace FRG_NS
