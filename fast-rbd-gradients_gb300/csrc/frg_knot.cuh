// Per-knot forward-dynamics gradient, one knot per lane.
//
// Every lane of a warp carries one knot through the whole path, so the
// inherently serial joint sweeps run without any block barrier, and all 32
// lanes do useful work in every phase.  Lanes only meet at the per-warp
// staging buffer that turns the knot-major HBM layout into coalesced 128-byte
// loads and stores (__syncwarp only).
//
// Path per knot (the reference's forwardDynamicsGradientThreaded with
// QDD_MINV_PASSED_IN=false, helpers_CPU/dynamicsGradient.h:869-934):
//   1. sincos(q), RNEA with qdd = 0 -> bias = u - c (- 0.5 qd)     (:876-885)
//   2. articulated-inertia sweep + Minv column passes            (minv.h:392-477)
//   3. qdd = Minv bias, RNEA again with qdd                        (:892-895)
//   4. d tau/dq, d tau/dqd as 13 independent tangent sweeps        (:787-857)
//   5. dqdd = -Minv [d tau/dq | d tau/dqd]                         (:933)
#pragma once
#include "frg_model.cuh"

namespace FRG_NS {

// Per-link data that the tangent sweeps re-read, as real4 slots:
//   0: v[0..3]   1: v[4..5] Iv[0..1]   2: Iv[2..5]   3: (X a_{k-1})[0,1,3,4]
//   4: f_k[0,1,3,4] after the backward pass
constexpr int kSlotsPerLink = 5;
constexpr int kLinkSlots = kSlotsPerLink * kJoints;
// per lane: a knot's dense Minv (N x N) or half of its N x 2N gradient, its
// 3N inputs, or its 6N external-force values
constexpr int kStageFloats = kJoints * kJoints > 6 * kJoints ? kJoints * kJoints : 6 * kJoints;
constexpr int kMinvFloats = kJoints * kJoints;
constexpr int kMinvPackedFloats = kJoints * ((kJoints + 2) / 2);  // upper triangle, padded to groups of N
constexpr int kDqddFloats = 2 * kJoints * kJoints;

// Four reals as one 16-byte-aligned shared-memory slot.
template <typename T> struct Real4Of;
template <> struct Real4Of<float> { using type = float4; };
struct alignas(16) double4x { double x, y, z, w; };
template <> struct Real4Of<double> { using type = double4x; };
using real4 = Real4Of<real>::type;
__device__ __forceinline__ real4 make_real4(real a, real b, real c, real d) {
    real4 v;
    v.x = a; v.y = b; v.z = c; v.w = d;
    return v;
}
// Read-only 16-byte loads of one slot.
__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }
__device__ __forceinline__ double4x ldg4(const double4x *p) {
    const double2 *d = reinterpret_cast<const double2 *>(p);
    const double2 a = __ldg(d), b = __ldg(d + 1);
    double4x v;
    v.x = a.x; v.y = a.y; v.z = b.x; v.w = b.y;
    return v;
}

struct WarpSmem {
    real4 link[kLinkSlots][32];
    real stage[32 * kStageFloats];
    const real *knot[32];  // each lane's knot pointer, for tiles that are not one contiguous run
};

// A lane's knot: input and output bases (q == nullptr: idle lane).
struct KnotPtrs {
    const real *q, *qd, *u;
    real *dqdd, *qdd, *minv;
    const real *fext = nullptr;  // [kJoints][6] external spatial force per link (link frame), optional
};

// Persistent work loop: a warp draws tickets from a device counter,
//     for (unsigned int t; next_ticket(items, counter, lane, t);) work(t);
// until the `items` work items are exhausted.  The warp that draws the very
// last ticket (items + total warps - 1: every warp draws one failing ticket)
// resets the counter, so back-to-back and repeated plan launches need no
// memset.
__device__ __forceinline__ bool next_ticket(unsigned int items, unsigned int *counter, int lane,
                                            unsigned int &ticket) {
    unsigned int t = 0;
    if (lane == 0) t = atomicAdd(counter, 1u);
    ticket = __shfl_sync(0xffffffffu, t, 0);
    if (ticket < items) return true;
    if (lane == 0 && ticket == items + gridDim.x * (blockDim.x >> 5) - 1u) atomicExch(counter, 0u);
    return false;
}

// The segment of a ragged knot list that holds knot g (segs[nseg].knot_begin
// is the total knot count, g below it): the last one starting at or before g,
// searched upward from s, the segment of g's tile's first knot.
template <typename Seg>
__device__ __forceinline__ int segment_of(const Seg *segs, int nseg, int s, long long g) {
    while (s + 1 < nseg && segs[s + 1].knot_begin <= g) s++;
    return s;
}

__device__ __forceinline__ const real *shfl_ptr(const real *p, int src) {
    return reinterpret_cast<const real *>(
        __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(p), src));
}
__device__ __forceinline__ real *shfl_ptr(real *p, int src) {
    return reinterpret_cast<real *>(__shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(p), src));
}

// The tile's knot count n when its knots are one run in memory: lanes 0..n-1
// hold knots, lane i's base = lane 0's base + i * STRIDE, and the other lanes
// are idle (null).  Otherwise 0.  b0 = lane 0's base.  Warp-uniform.
template <int STRIDE, typename P>
__device__ __forceinline__ int tile_run(P base, int lane, P &b0) {
    b0 = shfl_ptr(base, 0);
    const unsigned valid = __ballot_sync(0xffffffffu, base != nullptr);
    const bool mine = base == nullptr || (b0 != nullptr && base == b0 + lane * STRIDE);
    if (!__all_sync(0xffffffffu, mine) || (valid & (valid + 1u)) != 0u) return 0;  // valid lanes: a prefix
    return __popc(valid);
}

__device__ __forceinline__ bool aligned16(const void *p) {
    return (reinterpret_cast<unsigned long long>(p) & 15ull) == 0;
}

// Element e = lane + 32 m (m < W) of a tile's W reals per knot is entry
// j = e % W of knot kn = e / W.  Computed afresh for every element (a
// multiply-high by a constant, independent across elements) rather than
// stepped from the previous one, whose serial chain of adds and compares
// held each store or load back by the one before.
template <int W>
__device__ __forceinline__ int element_knot(int e) {
    return static_cast<int>(static_cast<unsigned int>(e) / W);
}

// Gather of W reals per knot (knot-major) into stage[lane*W + j].  Tiles of
// one run copy their n*W reals straight and coalesced (16-byte slots when the
// run is 32 knots and aligned); idle lanes get zeros.  Other tiles (knots of
// several trajectories, strided records) read element by element through the
// knots' pointers in the warp's table (see scatter_out), coalesced: first all
// pointers, then all W loads in flight, then the shared-memory stores.
template <int W>
__device__ __forceinline__ void gather_in(real *stage, const real *base, int lane, const real **knot) {
    const real *b0;
    const int n = tile_run<W>(base, lane, b0);
    if (n == 32 && aligned16(b0)) {
        const real4 *src = reinterpret_cast<const real4 *>(b0);
        real4 *dst = reinterpret_cast<real4 *>(stage);
#pragma unroll
        for (int e = lane; e < 8 * W; e += 32) dst[e] = ldg4(src + e);
        return;
    }
    if (n > 0) {
        const int lim = n * W;
#pragma unroll
        for (int e = lane; e < 32 * W; e += 32) stage[e] = e < lim ? __ldg(b0 + e) : real(0);
        return;
    }
    if constexpr (W <= 8) {
        knot[lane] = base;
        __syncwarp();
        const real *p[W];
#pragma unroll
        for (int m = 0; m < W; m++) {
            const int e = lane + 32 * m, kn = element_knot<W>(e);
            p[m] = knot[kn];
            if (p[m]) p[m] += e - kn * W;
        }
        real v[W];
#pragma unroll
        for (int m = 0; m < W; m++) v[m] = p[m] ? __ldg(p[m]) : real(0);
        __syncwarp();  // every lane has read the table
#pragma unroll
        for (int m = 0; m < W; m++) stage[lane + 32 * m] = v[m];
    } else {  // wider knots (external forces): each lane reads its own, all loads in flight
#pragma unroll
        for (int j = 0; j < W; j++) stage[lane * W + j] = base ? __ldg(base + j) : real(0);
    }
}

// Scatter of stage[lane*W + j] to each knot's W reals at base (knots STRIDE
// reals apart in tiles of one run).  Other tiles (knots of several
// trajectories, strided records) store element by element through
// each knot's pointer in the warp's table: consecutive elements of a knot are
// consecutive in memory, so each store instruction still covers whole runs of
// a few cache lines.  A lane storing only its own knot would turn every store
// instruction into 32 separate cache-line writes; with many such tiles in
// flight the L2 request rate, not the arithmetic, then sets the time.  The
// stores go in groups of kJoints after the group's table and stage reads: the
// compiler cannot tell a table pointer from shared memory, so a read placed
// after a store would wait for it.
template <int W, int STRIDE = W>
__device__ __forceinline__ void scatter_out(const real *stage, real *base, int lane, const real **knot) {
    __syncwarp();
    real *b0;
    const int n = tile_run<STRIDE>(base, lane, b0);
    if (n > 0) {
        if constexpr (STRIDE == W) {
            if (n == 32 && aligned16(b0)) {
                const real4 *src = reinterpret_cast<const real4 *>(stage);
                real4 *dst = reinterpret_cast<real4 *>(b0);
#pragma unroll
                for (int e = lane; e < 8 * W; e += 32) dst[e] = src[e];
            } else {
                const int lim = n * W;
#pragma unroll 7
                for (int e = lane; e < 32 * W; e += 32)
                    if (e < lim) b0[e] = stage[e];
            }
        } else {
#pragma unroll 7
            for (int m = 0; m < W; m++) {
                const int e = lane + 32 * m, kn = element_knot<W>(e);
                if (kn < n) b0[e + kn * (STRIDE - W)] = stage[e];
            }
        }
    } else {
        constexpr int G = kJoints;  // every W here is a multiple of the joint count
        static_assert(W % G == 0, "split-tile stores go in groups of kJoints");
        knot[lane] = base;
        __syncwarp();
#pragma unroll 1
        for (int m0 = 0; m0 < W; m0 += G) {
            real *p[G];
            real v[G];
#pragma unroll
            for (int i = 0; i < G; i++) {
                const int e = lane + 32 * (m0 + i), kn = element_knot<W>(e);
                p[i] = const_cast<real *>(knot[kn]);
                if (p[i]) p[i] += e - kn * W;
                v[i] = stage[e];
            }
#pragma unroll
            for (int i = 0; i < G; i++)
                if (p[i]) *p[i] = v[i];
        }
    }
    __syncwarp();  // also: the table is rewritten by the next scatter
}

__device__ __forceinline__ void lds_link(const WarpSmem *ws, int k, int lane, real v[6], real Iv[6]) {
    const real4 a = ws->link[kSlotsPerLink * k + 0][lane];
    const real4 b = ws->link[kSlotsPerLink * k + 1][lane];
    const real4 c = ws->link[kSlotsPerLink * k + 2][lane];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y;
    Iv[0] = b.z; Iv[1] = b.w; Iv[2] = c.x; Iv[3] = c.y; Iv[4] = c.z; Iv[5] = c.w;
}
__device__ __forceinline__ void sts_link(WarpSmem *ws, int k, int lane, const real v[6], const real Iv[6]) {
    ws->link[kSlotsPerLink * k + 0][lane] = make_real4(v[0], v[1], v[2], v[3]);
    ws->link[kSlotsPerLink * k + 1][lane] = make_real4(v[4], v[5], Iv[0], Iv[1]);
    ws->link[kSlotsPerLink * k + 2][lane] = make_real4(Iv[2], Iv[3], Iv[4], Iv[5]);
}

// sin and cos of a joint angle: the hardware approximation __sincosf
// (absolute error below 2^-21 on [-pi, pi], far inside the 1e-4 parity bar).
// An angle outside [-pi, pi] is first reduced by the nearest multiple of 2 pi
// with Cody and Waite's additive reduction (W. J. Cody, W. Waite, Software
// Manual for the Elementary Functions, 1980): r = (x - k C1) - k C2 with
// k = rint(x / 2 pi) and C1 + C2 = 2 pi, C1 = 201/32 short enough that k C1 is
// exact for |k| < 2^15; each step is one fma, so r is within a few ulp of the
// true remainder for |x| up to about 10^4 rad.  (The library sincosf's
// general reduction, never needed for joint angles, cost the kernel a stack
// frame and 12 % of its time by its code alone.)
__device__ __forceinline__ void sincos_angle(float x, float *s, float *c) {
    if (fabsf(x) > 3.14159f) {
        const float k = rintf(x * 0.159154943f);  // 1 / (2 pi)
        x = fmaf(-k, 6.28125f, x);                // C1 = 201 / 32
        x = fmaf(-k, 1.93530718e-3f, x);          // C2 = 2 pi - C1
    }
    __sincosf(x, s, c);
}
// FP64 verification build: the double-precision library routine throughout.
__device__ __forceinline__ void sincos_angle(double x, double *s, double *c) { sincos(x, s, c); }

// ------------------------------------------------ articulated inertia ------

// G = Rz N Rz^T for symmetric N (upper entries used), result symmetric.
__device__ __forceinline__ void rotz_sym(real G[3][3], const real N[3][3], real c, real s) {
    const real cc = c * c, ss = s * s, cs = c * s, d = cc - ss;
    G[0][0] = fmaR(cc, N[0][0], fmaR(ss, N[1][1], -2.0f * cs * N[0][1]));
    G[1][1] = fmaR(ss, N[0][0], fmaR(cc, N[1][1], 2.0f * cs * N[0][1]));
    G[0][1] = fmaR(cs, N[0][0] - N[1][1], d * N[0][1]);
    G[0][2] = fmaR(c, N[0][2], -s * N[1][2]);
    G[1][2] = fmaR(s, N[0][2], c * N[1][2]);
    G[2][2] = N[2][2];
    G[1][0] = G[0][1]; G[2][0] = G[0][2]; G[2][1] = G[1][2];
}

// G = Rz N Rz^T for general N.
__device__ __forceinline__ void rotz_gen(real G[3][3], const real N[3][3], real c, real s) {
    real H[3][3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
        H[0][j] = fmaR(c, N[0][j], -s * N[1][j]);
        H[1][j] = fmaR(s, N[0][j], c * N[1][j]);
        H[2][j] = N[2][j];
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        G[i][0] = fmaR(c, H[i][0], -s * H[i][1]);
        G[i][1] = fmaR(s, H[i][0], c * H[i][1]);
        G[i][2] = H[i][2];
    }
}

// O = F^T G F:  O[i][j] = s_i s_j G[p_i][p_j] for a signed permutation F,
// else the general product (structural zeros of F dropped at compile time).
template <int k> __device__ __forceinline__ void perm_FT_G_F(real O[3][3], const real G[3][3]) {
    using J = Joint<k>;
    if constexpr (J::perm) {
        constexpr int p[3] = {J::p0, J::p1, J::p2};
        constexpr real sg[3] = {J::s0, J::s1, J::s2};
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) O[i][j] = (sg[i] * sg[j]) * G[p[i]][p[j]];
    } else {
        real GF[3][3];  // G F: row a of G F is F^T applied to row a of G
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const real row[3] = {G[a][0], G[a][1], G[a][2]};
            mul_FT<k>(GF[a], row);
        }
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const real col[3] = {GF[0][j], GF[1][j], GF[2][j]};
            real o[3];
            mul_FT<k>(o, col);  // O[i][j] = sum_a F[a][i] (G F)[a][j]
            O[0][j] = o[0]; O[1][j] = o[1]; O[2][j] = o[2];
        }
    }
}

// X_k^T [A B; B^T M] X_k for the joint transform X_k = [E 0; -E r^ E].
// With At = E^T A E, Bt = E^T B E, Mt = E^T M E:
//   M' = Mt,  B' = Bt + r^ Mt,  A' = At + r^ Bt^T - B' r^.
template <int k>
__device__ __forceinline__ void congruence(real Ao[3][3], real Bo[3][3], real Mo[3][3], const real A[3][3],
                                           const real B[3][3], const real M[3][3], real c, real s) {
    using J = Joint<k>;
    real G[3][3], At[3][3], Bt[3][3];
    rotz_sym(G, A, c, s);
    perm_FT_G_F<k>(At, G);
    rotz_gen(G, B, c, s);
    perm_FT_G_F<k>(Bt, G);
    rotz_sym(G, M, c, s);
    perm_FT_G_F<k>(Mo, G);
    const real t = J::t;
    if constexpr (J::axis == 2) {
        // r^ = [0 -t 0; t 0 0; 0 0 0]
#pragma unroll
        for (int j = 0; j < 3; j++) {
            Bo[0][j] = fmaR(-t, Mo[1][j], Bt[0][j]);
            Bo[1][j] = fmaR(t, Mo[0][j], Bt[1][j]);
            Bo[2][j] = Bt[2][j];
        }
        // (r^ Bt^T)[i][j]: i=0: -t Bt[j][1]; i=1: t Bt[j][0]; i=2: 0
        // (B' r^)[i][j]:   j=0: t B'[i][1]; j=1: -t B'[i][0]; j=2: 0
        Ao[0][0] = fmaR(-t, Bt[0][1], fmaR(-t, Bo[0][1], At[0][0]));
        Ao[0][1] = fmaR(-t, Bt[1][1], fmaR(t, Bo[0][0], At[0][1]));
        Ao[0][2] = fmaR(-t, Bt[2][1], At[0][2]);
        Ao[1][1] = fmaR(t, Bt[1][0], fmaR(t, Bo[1][0], At[1][1]));
        Ao[1][2] = fmaR(t, Bt[2][0], At[1][2]);
        Ao[2][2] = At[2][2];
    } else if constexpr (J::axis == 1) {
        // r^ = [0 0 t; 0 0 0; -t 0 0]
#pragma unroll
        for (int j = 0; j < 3; j++) {
            Bo[0][j] = fmaR(t, Mo[2][j], Bt[0][j]);
            Bo[1][j] = Bt[1][j];
            Bo[2][j] = fmaR(-t, Mo[0][j], Bt[2][j]);
        }
        // (r^ Bt^T)[i][j]: i=0: t Bt[j][2]; i=1: 0; i=2: -t Bt[j][0]
        // (B' r^)[i][j]:   j=0: -t B'[i][2]; j=1: 0; j=2: t B'[i][0]
        Ao[0][0] = fmaR(t, Bt[0][2], fmaR(t, Bo[0][2], At[0][0]));
        Ao[0][1] = fmaR(t, Bt[1][2], At[0][1]);
        Ao[0][2] = fmaR(t, Bt[2][2], fmaR(-t, Bo[0][0], At[0][2]));
        Ao[1][1] = At[1][1];
        Ao[1][2] = fmaR(-t, Bo[1][0], At[1][2]);
        Ao[2][2] = fmaR(-t, Bt[2][0], fmaR(-t, Bo[2][0], At[2][2]));
    } else {
        // other origins: r^ = [0 -r2 r1; r2 0 -r0; -r1 r0 0]
        constexpr real rh[3][3] = {{0, -J::r2, J::r1}, {J::r2, 0, -J::r0}, {-J::r1, J::r0, 0}};
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                real acc = Bt[i][j];
#pragma unroll
                for (int a = 0; a < 3; a++)
                    if (rh[i][a] != real(0)) acc = fmaR(rh[i][a], Mo[a][j], acc);
                Bo[i][j] = acc;  // Bt + r^ Mt
            }
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = i; j < 3; j++) {
                real acc = At[i][j];
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    if (rh[i][a] != real(0)) acc = fmaR(rh[i][a], Bt[j][a], acc);   // + r^ Bt^T
                    if (rh[a][j] != real(0)) acc = fmaR(-rh[a][j], Bo[i][a], acc);  // - B' r^
                }
                Ao[i][j] = acc;
            }
    }
    Ao[1][0] = Ao[0][1]; Ao[2][0] = Ao[0][2]; Ao[2][1] = Ao[1][2];
}

// IA_k = I_k + child carry, as blocks [A B; B^T M].
template <int k>
__device__ __forceinline__ void add_link_inertia(real A[3][3], real B[3][3], real M[3][3]) {
    using L = Link<k>;
    A[0][0] += L::Ixx; A[1][1] += L::Iyy; A[2][2] += L::Izz;
    A[0][1] += L::Ixy; A[1][0] += L::Ixy;
    A[0][2] += L::Ixz; A[2][0] += L::Ixz;
    A[1][2] += L::Iyz; A[2][1] += L::Iyz;
    // m c^ = [0 -mcz mcy; mcz 0 -mcx; -mcy mcx 0]
    B[0][1] += -L::mcz; B[0][2] += L::mcy;
    B[1][0] += L::mcz;  B[1][2] += -L::mcx;
    B[2][0] += -L::mcy; B[2][1] += L::mcx;
    M[0][0] += L::m; M[1][1] += L::m; M[2][2] += L::m;
}

// ------------------------------------------------------------- phase 1 -----

// sincos, RNEA(q, qd, 0), bias, Minv (upper triangle, Mi[i][j] for i <= j), qdd.
// Leaves v_k and I_k v_k of every link in the warp's link slots.
template <bool DAMP, bool MPC, bool FEXT = false>
__device__ __forceinline__ void phase1(WarpSmem *ws, int lane, const real q[kJoints], const real qd[kJoints],
                                       const real u[kJoints], real sq[kJoints], real cq[kJoints],
                                       real Mi[kJoints][kJoints], real qdd[kJoints],
                                       const real *fx = nullptr) {
#pragma unroll
    for (int k = 0; k < kJoints; k++) sincos_angle(q[k], &sq[k], &cq[k]);

    // RNEA forward with qdd = 0 (RNEA_fp, dynamicsGradient.h:620-659)
    real f[kJoints][6];
    {
        real v[6], a[6];
        static_for<0, kJoints>([&](auto K) {
            constexpr int k = decltype(K)::value;
            if constexpr (k == 0) {
                v[0] = v[1] = 0.0f; v[2] = qd[0]; v[3] = v[4] = v[5] = 0.0f;
                if constexpr (MPC) {
#pragma unroll
                    for (int i = 0; i < 6; i++) a[i] = 0.0f;
                } else {
                    const real g[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, kGravity};
                    xmotion<0>(a, g, cq[0], sq[0]);
                }
            } else {
                real nv[6], na[6];
                xmotion<k>(nv, v, cq[k], sq[k]);
                nv[2] += qd[k];
                xmotion<k>(na, a, cq[k], sq[k]);
                na[0] = fmaR(nv[1], qd[k], na[0]);
                na[1] = fmaR(-nv[0], qd[k], na[1]);
                na[3] = fmaR(nv[4], qd[k], na[3]);
                na[4] = fmaR(-nv[3], qd[k], na[4]);
#pragma unroll
                for (int i = 0; i < 6; i++) { v[i] = nv[i]; a[i] = na[i]; }
            }
            real Iv[6];
            imul<k>(Iv, v);
            imul<k>(f[k], a);
            crf_acc(f[k], v, Iv);
            if constexpr (FEXT) {  // f_k -= fext_k (RNEA_fp, dynamicsGradient.h:654-657)
#pragma unroll
                for (int i = 0; i < 6; i++) f[k][i] -= fx[6 * k + i];
            }
            sts_link(ws, k, lane, v, Iv);
        });
    }
    // backward (RNEA_bp :662-670) -> c, bias (computeBias :677-683)
    real bias[kJoints];
    static_for_down<kJoints - 1, 0>([&](auto K) {
        constexpr int k = decltype(K)::value;
        const real c = f[k][2];
        bias[k] = DAMP ? u[k] - fmaR(0.5f, qd[k], c) : u[k] - c;
        if constexpr (k > 0) {
            real t[6];
            xforce_T<k>(t, f[k], cq[k], sq[k]);
#pragma unroll
            for (int i = 0; i < 6; i++) f[k - 1][i] += t[i];
        }
    });

    // articulated-inertia sweep: U_k = IA_k[:,2], D_k = U_k[2]
    // (Minv_bp :424-436; compute_Ia_revolute :147; ctransform_Ia_revolute :222)
    real U[kJoints][6], Dinv[kJoints];
    {
        real A[3][3], B[3][3], M[3][3];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) A[i][j] = B[i][j] = M[i][j] = 0.0f;
        static_for_down<kJoints - 1, 0>([&](auto K) {
            constexpr int k = decltype(K)::value;
            add_link_inertia<k>(A, B, M);
            U[k][0] = A[0][2]; U[k][1] = A[1][2]; U[k][2] = A[2][2];
            U[k][3] = B[2][0]; U[k][4] = B[2][1]; U[k][5] = B[2][2];
            Dinv[k] = 1.0f / U[k][2];
            if constexpr (k > 0) {
                // Ia = IA - U U^T / D with the joint row/column exactly zero
                real Ud[6];
#pragma unroll
                for (int i = 0; i < 6; i++) Ud[i] = U[k][i] * Dinv[k];
                real Aa[3][3], Ba[3][3], Ma[3][3];
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        Aa[i][j] = (i == 2 || j == 2) ? 0.0f : fmaR(-U[k][i], Ud[j], A[i][j]);
                        Ba[i][j] = (i == 2) ? 0.0f : fmaR(-U[k][i], Ud[3 + j], B[i][j]);
                        Ma[i][j] = fmaR(-U[k][3 + i], Ud[3 + j], M[i][j]);
                    }
                congruence<k>(A, B, M, Aa, Ba, Ma, cq[k], sq[k]);
            }
        });
    }

    // Minv columns: backward pass (bwdPassMinvFUpdate, minv.h:392-412) then
    // forward pass (fwdPassUpdate, :440-461), each column carrying one F vector.
    static_for<0, kJoints>([&](auto JJ) {
        constexpr int j = decltype(JJ)::value;
        real F[6];
        static_for_down<j, 0>([&](auto II) {
            constexpr int i = decltype(II)::value;
            if constexpr (i == j) {
                Mi[j][j] = Dinv[j];
#pragma unroll
                for (int r = 0; r < 6; r++) F[r] = U[j][r] * Dinv[j];
            } else {
                const real m = -Dinv[i] * F[2];
                Mi[i][j] = m;
#pragma unroll
                for (int r = 0; r < 6; r++) F[r] = fmaR(U[i][r], m, F[r]);
            }
            if constexpr (i > 0) {
                real t[6];
                xforce_T<i>(t, F, cq[i], sq[i]);
#pragma unroll
                for (int r = 0; r < 6; r++) F[r] = t[r];
            }
        });
        static_for<0, j + 1>([&](auto II) {
            constexpr int i = decltype(II)::value;
            if constexpr (i == 0) {
#pragma unroll
                for (int r = 0; r < 6; r++) F[r] = 0.0f;
                F[2] = Mi[0][j];
            } else {
                // Minv[i][j] -= D_i^-1 U_i^T X_i F_{i-1};  F_i = S Minv[i][j] + X_i F_{i-1}
                real y[6];
                xmotion<i>(y, F, cq[i], sq[i]);
                real d = U[i][0] * y[0];
#pragma unroll
                for (int r = 1; r < 6; r++) d = fmaR(U[i][r], y[r], d);
                Mi[i][j] = fmaR(-Dinv[i], d, Mi[i][j]);
#pragma unroll
                for (int r = 0; r < 6; r++) F[r] = y[r];
                F[2] += Mi[i][j];
            }
        });
    });

    // qdd = Minv_sym bias (matVMultSym, math.h:29-37)
#pragma unroll
    for (int r = 0; r < kJoints; r++) {
        real acc = 0.0f;
#pragma unroll
        for (int k = 0; k < kJoints; k++) acc = fmaR(r <= k ? Mi[r][k] : Mi[k][r], bias[k], acc);
        qdd[r] = acc;
    }
}

// RNEA(q, qd, qdd) forward + backward: stores (X_k a_{k-1})[0,1,3,4] and the
// accumulated f_k[0,1,3,4] in the link slots (read at the diagonal step of the
// d/dq sweeps).
template <bool MPC, bool FEXT = false>
__device__ __forceinline__ void rnea_with_qdd(WarpSmem *ws, int lane, const real qd[kJoints],
                                              const real qdd[kJoints], const real sq[kJoints], const real cq[kJoints],
                                              const real *fx = nullptr) {
    real f[kJoints][6];
    real a[6];
    static_for<0, kJoints>([&](auto K) {
        constexpr int k = decltype(K)::value;
        real v[6], Iv[6];
        lds_link(ws, k, lane, v, Iv);
        if constexpr (k == 0) {
            if constexpr (MPC) {
#pragma unroll
                for (int i = 0; i < 6; i++) a[i] = 0.0f;
            } else {
                const real g[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, kGravity};
                xmotion<0>(a, g, cq[0], sq[0]);
            }
            if constexpr (!kDqColumn0Zero)  // X_0 a_base, read by d tau / dq column 0
                ws->link[kSlotsPerLink * 0 + 3][lane] = make_real4(a[0], a[1], a[3], a[4]);
            a[2] += qdd[0];
        } else {
            real xa[6];
            xmotion<k>(xa, a, cq[k], sq[k]);
            ws->link[kSlotsPerLink * k + 3][lane] = make_real4(xa[0], xa[1], xa[3], xa[4]);
            a[0] = fmaR(v[1], qd[k], xa[0]);
            a[1] = fmaR(-v[0], qd[k], xa[1]);
            a[2] = xa[2] + qdd[k];
            a[3] = fmaR(v[4], qd[k], xa[3]);
            a[4] = fmaR(-v[3], qd[k], xa[4]);
            a[5] = xa[5];
        }
        imul<k>(f[k], a);
        crf_acc(f[k], v, Iv);
        if constexpr (FEXT) {
#pragma unroll
            for (int i = 0; i < 6; i++) f[k][i] -= fx[6 * k + i];
        }
    });
    static_for_down<kJoints - 1, 1>([&](auto K) {
        constexpr int k = decltype(K)::value;
        ws->link[kSlotsPerLink * k + 4][lane] = make_real4(f[k][0], f[k][1], f[k][3], f[k][4]);
        real t[6];
        xforce_T<k>(t, f[k], cq[k], sq[k]);
#pragma unroll
        for (int i = 0; i < 6; i++) f[k - 1][i] += t[i];
    });
}

// ------------------------------------------------------------- phase 2 -----

// One column of d tau / dq (QSIDE) or d tau / dqd for the differentiated joint c
// (compute_vafdu :787-829 and compute_cdu :832-857 restricted to column c).
// df_k = I_k da + dv x* (I_k v_k) + v_k x* (I_k dv): the force tangent of
// link k from its velocity / acceleration tangents (dv, da).
template <int k>
__device__ __forceinline__ void link_force_tangent(real df[6], const real v[6], const real Iv[6],
                                                   const real dv[6], const real da[6]) {
    real Idv[6];
    imul<k>(Idv, dv);
    imul<k>(df, da);
    crf_acc(df, dv, Iv);
    crf_acc(df, v, Idv);
}

// Seed of the tangent sweep for the differentiated joint k, from link k's
// velocity v: d tau / dq_k (QSIDE) or d tau / dqd_k.
template <bool QSIDE>
__device__ __forceinline__ void seed_column(const WarpSmem *ws, int lane, int k, real qdk, const real v[6],
                                            real dv[6], real da[6]) {
    if constexpr (QSIDE) {
        // dv = crm(X_k v_{k-1}) S; (X_k v_{k-1}) and v_k agree outside entry 2
        dv[0] = v[1]; dv[1] = -v[0]; dv[2] = 0.0f;
        dv[3] = v[4]; dv[4] = -v[3]; dv[5] = 0.0f;
        // da = crm(dv) S qd_k + crm(X_k a_{k-1}) S
        const real4 xa = ws->link[kSlotsPerLink * k + 3][lane];  // (Xa0, Xa1, Xa3, Xa4)
        da[0] = fmaR(dv[1], qdk, xa.y);
        da[1] = fmaR(-dv[0], qdk, -xa.x);
        da[2] = 0.0f;
        da[3] = fmaR(dv[4], qdk, xa.w);
        da[4] = fmaR(-dv[3], qdk, -xa.z);
        da[5] = 0.0f;
    } else {
        // dv = S, da = crm(v_k) S
        dv[0] = dv[1] = 0.0f; dv[2] = 1.0f; dv[3] = dv[4] = dv[5] = 0.0f;
        da[0] = v[1]; da[1] = -v[0]; da[2] = 0.0f;
        da[3] = v[4]; da[4] = -v[3]; da[5] = 0.0f;
    }
}

// Velocity / acceleration tangents carried from link k - 1 into link k.
template <int k>
__device__ __forceinline__ void advance_column(real dv[6], real da[6], real qdk, real ck, real sk) {
    real ndv[6], nda[6];
    xmotion<k>(ndv, dv, ck, sk);
    xmotion<k>(nda, da, ck, sk);
    nda[0] = fmaR(ndv[1], qdk, nda[0]);
    nda[1] = fmaR(-ndv[0], qdk, nda[1]);
    nda[3] = fmaR(ndv[4], qdk, nda[3]);
    nda[4] = fmaR(-ndv[3], qdk, nda[4]);
#pragma unroll
    for (int i = 0; i < 6; i++) { dv[i] = ndv[i]; da[i] = nda[i]; }
}

// Columns c and c + 1 of d tau / dq (QSIDE) or d tau / dqd, for the
// differentiated joints c and c + 1 (compute_vafdu :787-829 and compute_cdu
// :832-857 restricted to those columns); c + 1 == kJoints or !PAIR computes
// column c only.  The two columns are independent dependency chains through the same
// link loads; each does exactly the operations of a single-column sweep, so
// the bits do not depend on the pairing.  The forward sweep is also
// software-pipelined: the block of link k computes the force tangents of link
// k - 1 with the velocity / acceleration tangents of link k.  The link loop is
// unrolled; c is a warp-uniform runtime value.
template <bool QSIDE, bool DAMP, bool PAIR>
__device__ __forceinline__ void dtau_column_pair(const WarpSmem *ws, int lane, int c, const real qd[kJoints],
                                                 const real sq[kJoints], const real cq[kJoints], real dtA[kJoints],
                                                 real dtB[kJoints]) {
    const int cb = PAIR ? c + 1 : kJoints;
    real dfA[kJoints][6], dfB[kJoints][6];
    real dvA[6], daA[6], dvB[6], daB[6];
#pragma unroll
    for (int i = 0; i < 6; i++) dvB[i] = daB[i] = 0.0f;
    static_for<0, kJoints>([&](auto K) {
        constexpr int k = decltype(K)::value;
        if (k == c) {
            real v[6], Iv[6];
            lds_link(ws, k, lane, v, Iv);
            seed_column<QSIDE>(ws, lane, k, qd[k], v, dvA, daA);
        } else if (k > c) {
            if constexpr (k >= 1) {
                real v[6], Iv[6];
                lds_link(ws, k - 1, lane, v, Iv);
                link_force_tangent<k - 1>(dfA[k - 1], v, Iv, dvA, daA);
                if (k > cb) link_force_tangent<k - 1>(dfB[k - 1], v, Iv, dvB, daB);
                advance_column<k>(dvA, daA, qd[k], cq[k], sq[k]);
                if (k > cb) advance_column<k>(dvB, daB, qd[k], cq[k], sq[k]);
                if (k == cb) {
                    real vb[6], Ivb[6];
                    lds_link(ws, k, lane, vb, Ivb);
                    seed_column<QSIDE>(ws, lane, k, qd[k], vb, dvB, daB);
                }
            }
        }
    });
    {
        real v[6], Iv[6];
        lds_link(ws, kJoints - 1, lane, v, Iv);
        link_force_tangent<kJoints - 1>(dfA[kJoints - 1], v, Iv, dvA, daA);
        if (cb < kJoints) link_force_tangent<kJoints - 1>(dfB[kJoints - 1], v, Iv, dvB, daB);
    }
    real dFA[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f}, dFB[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    static_for_down<kJoints - 1, 0>([&](auto K) {
        constexpr int k = decltype(K)::value;
        if (k >= c) {
#pragma unroll
            for (int i = 0; i < 6; i++) dFA[i] += dfA[k][i];
        }
        if (k >= cb) {
#pragma unroll
            for (int i = 0; i < 6; i++) dFB[i] += dfB[k][i];
        }
        dtA[k] = dFA[2];
        dtB[k] = dFB[2];
        if constexpr (k > 0) {
            if (QSIDE && (k == c || k == cb)) {
                // + X_k^T (S x* f_k)
                const real4 fs = ws->link[kSlotsPerLink * k + 4][lane];  // (f0, f1, f3, f4)
                real *dF = k == c ? dFA : dFB;
                dF[0] -= fs.y; dF[1] += fs.x; dF[3] -= fs.w; dF[4] += fs.z;
            }
            real t[6];
            xforce_T<k>(t, dFA, cq[k], sq[k]);
#pragma unroll
            for (int i = 0; i < 6; i++) dFA[i] = t[i];
            xforce_T<k>(t, dFB, cq[k], sq[k]);
#pragma unroll
            for (int i = 0; i < 6; i++) dFB[i] = t[i];
        }
    });
    if constexpr (!QSIDE && DAMP) {  // compile-time indices: no local-memory array
#pragma unroll
        for (int k = 0; k < kJoints; k++) {
            if (k == c) dtA[k] += 0.5f;
            if (k == cb) dtB[k] += 0.5f;
        }
    }
}

// out = -Minv_sym dtau
__device__ __forceinline__ void minv_times(real out[kJoints], const real Mi[kJoints][kJoints],
                                           const real dtau[kJoints]) {
#pragma unroll
    for (int r = 0; r < kJoints; r++) {
        real acc = 0.0f;
#pragma unroll
        for (int k = 0; k < kJoints; k++) acc = fmaR(r <= k ? Mi[r][k] : Mi[k][r], dtau[k], acc);
        out[r] = -acc;
    }
}

// Full path for the 32 knots of one warp tile.  With MIRROR, inputs are also
// stored at mr.q / qd / u and results at mr.dqdd / qdd / minv, for the lanes
// whose mirror pointers are set (the server mirrors inputs that did not come
// from a trajectory's device slot into it, and sends results to the pinned
// host slot when the caller asked for them); a mirror that no lane of the
// tile wants is skipped.  With FEXT, kp.fext holds each knot's external link
// forces; with FDONLY only q̈ and Minv are produced (forward dynamics); with
// MINV_PACKED, kp.minv receives Minv's upper triangle (kMinvPackedFloats per
// knot, column by column) instead of the dense matrix.
template <bool DAMP, bool MPC, bool MIRROR = false, bool FEXT = false, bool FDONLY = false,
          bool MINV_PACKED = false>
__device__ __forceinline__ void process_tile(WarpSmem *ws, int lane, const KnotPtrs &kp,
                                             const KnotPtrs &mr = KnotPtrs{}) {
    constexpr int N = kJoints, NN = kMinvFloats;
    real *const st_q = ws->stage, *const st_qd = ws->stage + 32 * N, *const st_u = ws->stage + 64 * N;
    real q[N], qd[N], u[N];
    gather_in<N>(st_q, kp.q, lane, ws->knot);
    gather_in<N>(st_qd, kp.qd, lane, ws->knot);
    gather_in<N>(st_u, kp.u, lane, ws->knot);
    __syncwarp();
#pragma unroll
    for (int j = 0; j < N; j++) {
        q[j] = st_q[lane * N + j];
        qd[j] = st_qd[lane * N + j];
        u[j] = st_u[lane * N + j];
    }
    __syncwarp();
    bool mirror_out = false;
    if constexpr (MIRROR) {
        mirror_out = __any_sync(0xffffffffu, mr.minv != nullptr);
        if (__any_sync(0xffffffffu, mr.q != nullptr)) {
            scatter_out<N>(st_q, const_cast<real *>(mr.q), lane, ws->knot);
            scatter_out<N>(st_qd, const_cast<real *>(mr.qd), lane, ws->knot);
            scatter_out<N>(st_u, const_cast<real *>(mr.u), lane, ws->knot);
        }
    }
    const real *fx = nullptr;
    if constexpr (FEXT) {  // the lane's 6N external-force values stay staged through both RNEA passes
        gather_in<6 * N>(ws->stage, kp.fext, lane, ws->knot);
        __syncwarp();
        fx = ws->stage + lane * 6 * N;
    }

    real sq[N], cq[N], Mi[N][N], qdd[N];
    phase1<DAMP, MPC, FEXT>(ws, lane, q, qd, u, sq, cq, Mi, qdd, fx);
    // with FEXT the second RNEA runs while the forces are still staged;
    // otherwise after the Minv / qdd stores (fewer live registers)
    if constexpr (FEXT && !FDONLY) rnea_with_qdd<MPC, FEXT>(ws, lane, qd, qdd, sq, cq, fx);
    __syncwarp();

    // Minv (dense, or its packed upper triangle) and qdd out
    if constexpr (MINV_PACKED) {
        static_assert(!MIRROR, "the server's slots hold dense Minv");
        constexpr int P = kMinvPackedFloats;
        static_assert(P <= kStageFloats && P % N == 0, "packed Minv rows fit the staging buffer in groups of N");
#pragma unroll
        for (int c = 0, e = 0; c < N; c++)
#pragma unroll
            for (int r = 0; r <= c; r++, e++) ws->stage[lane * P + e] = Mi[r][c];
#pragma unroll
        for (int e = N * (N + 1) / 2; e < P; e++) ws->stage[lane * P + e] = real(0);
        scatter_out<P>(ws->stage, kp.minv, lane, ws->knot);
    } else {
#pragma unroll
        for (int c = 0; c < N; c++)
#pragma unroll
            for (int r = 0; r < N; r++) ws->stage[lane * NN + r + N * c] = r <= c ? Mi[r][c] : Mi[c][r];
        scatter_out<NN>(ws->stage, kp.minv, lane, ws->knot);
        if (MIRROR && mirror_out) scatter_out<NN>(ws->stage, mr.minv, lane, ws->knot);
    }
#pragma unroll
    for (int r = 0; r < N; r++) ws->stage[lane * N + r] = qdd[r];
    scatter_out<N>(ws->stage, kp.qdd, lane, ws->knot);
    if (MIRROR && mirror_out) scatter_out<N>(ws->stage, mr.qdd, lane, ws->knot);
    if constexpr (FDONLY) return;
    if constexpr (!FEXT) {
        rnea_with_qdd<MPC>(ws, lane, qd, qdd, sq, cq);
        __syncwarp();
    }

    // d qdd / dq: columns 0..N-1 (column 0 is identically zero when the base
    // joint axis is parallel to gravity, as for the iiwa and as
    // dynamicsGradient.h:797-813 uses; other models compute it)
    if constexpr (kDqColumn0Zero) {
#pragma unroll
        for (int r = 0; r < N; r++) ws->stage[lane * NN + r] = 0.0f;
    }
    // two columns per sweep; one with FEXT, whose staged forces leave fewer registers
    constexpr bool kPair = !FEXT;
#pragma unroll 1
    for (int c = kDqColumn0Zero ? 1 : 0; c < N; c += kPair ? 2 : 1) {
        real dtA[N], dtB[N], out[N];
        dtau_column_pair<true, DAMP, kPair>(ws, lane, c, qd, sq, cq, dtA, dtB);
        minv_times(out, Mi, dtA);
#pragma unroll
        for (int r = 0; r < N; r++) ws->stage[lane * NN + N * c + r] = out[r];
        if (kPair && c + 1 < N) {
            minv_times(out, Mi, dtB);
#pragma unroll
            for (int r = 0; r < N; r++) ws->stage[lane * NN + N * (c + 1) + r] = out[r];
        }
    }
    scatter_out<NN, 2 * NN>(ws->stage, kp.dqdd, lane, ws->knot);
    if (MIRROR && mirror_out) scatter_out<NN, 2 * NN>(ws->stage, mr.dqdd, lane, ws->knot);
    // d qdd / dqd: columns N..2N-1
#pragma unroll 1
    for (int c = 0; c < N; c += kPair ? 2 : 1) {
        real dtA[N], dtB[N], out[N];
        dtau_column_pair<false, DAMP, kPair>(ws, lane, c, qd, sq, cq, dtA, dtB);
        minv_times(out, Mi, dtA);
#pragma unroll
        for (int r = 0; r < N; r++) ws->stage[lane * NN + N * c + r] = out[r];
        if (kPair && c + 1 < N) {
            minv_times(out, Mi, dtB);
#pragma unroll
            for (int r = 0; r < N; r++) ws->stage[lane * NN + N * (c + 1) + r] = out[r];
        }
    }
    scatter_out<NN, 2 * NN>(ws->stage, kp.dqdd ? kp.dqdd + NN : nullptr, lane, ws->knot);
    if (MIRROR && mirror_out)
        scatter_out<NN, 2 * NN>(ws->stage, mr.dqdd ? mr.dqdd + NN : nullptr, lane, ws->knot);
}

}  // namespace FRG_NS
