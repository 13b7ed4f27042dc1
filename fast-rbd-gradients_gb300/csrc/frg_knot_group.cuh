// Latency mapping: one knot per group of 8 lanes (4 knots per warp).
//
// The knot-per-lane mapping (frg_knot.cuh) maximises throughput, but one warp
// then walks ~15k instructions for its 32 knots, and a small batch (a served
// MPC request of tens of knots) waits for all of them.  Here the 8 lanes of a
// group share a knot:
//   - phase 1 (sincos, RNEA, articulated inertias, q̈) runs replicated in all
//     8 lanes, except the Minv column passes: lane g computes column g;
//   - the dtau columns are split so that every lane walks about N link steps
//     (N joints, at most 8): lane g takes dtau/dqd column g and dtau/dq
//     column N - g (dtau/dq column 0, where the model needs it, on lane N, or
//     on lane 0 for N = 8), which for the 7-joint iiwa gives every lane 7;
//   - each lane then writes its output columns of -Minv dtau.
// Lane-dependent work is predicated (selects), so a group never diverges.
// About 2.5x less latency per knot than the knot-per-lane mapping, at about
// 3x its instructions per knot: the autotuner and the server pick by size.
#pragma once
#include "frg_knot.cuh"

namespace frg {

constexpr int kGroupLanes = 8;
constexpr int kGroupKnots = 32 / kGroupLanes;  // knots per warp

static_assert(kJoints <= kGroupLanes, "one lane per joint column");

struct GroupSmem {
    float4 link[kGroupKnots][kLinkSlots];  // per knot, slot layout as WarpSmem
    float minv[kGroupKnots][kMinvN];       // dense Minv
    float out[kGroupKnots][kDqddN];        // dqdd staging
    float qdd[kGroupKnots][8];
};

// The dtau/dq column of group lane g (kJoints: none): column N - g for
// g = 1..N-1, column 0 on lane N (lane 0 when N = 8, the only free lane).
__device__ __forceinline__ int g_q_column(int g) {
    if (g >= 1 && g < kJoints) return kJoints - g;
    const int lane0 = kJoints < kGroupLanes ? kJoints : 0;
    return (g == lane0 && !kDqColumn0Zero) ? 0 : kJoints;
}

template <int k> __device__ __forceinline__ void g_sts(GroupSmem *gs, int ks, int slot, float4 v) {
    gs->link[ks][kSlotsPerLink * k + slot] = v;
}

__device__ __forceinline__ void g_lds_link(const GroupSmem *gs, int ks, int k, float v[6], float Iv[6]) {
    const float4 a = gs->link[ks][kSlotsPerLink * k + 0];
    const float4 b = gs->link[ks][kSlotsPerLink * k + 1];
    const float4 c = gs->link[ks][kSlotsPerLink * k + 2];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y;
    Iv[0] = b.z; Iv[1] = b.w; Iv[2] = c.x; Iv[3] = c.y; Iv[4] = c.z; Iv[5] = c.w;
}

// One dtau column per lane, lane-dependent c (0..N-1; c == N: no column).
// Same recursions as dtau_column in frg_knot.cuh, with the k >= c / k == c
// choices made by selects so that the 8 lanes of a group stay converged.
template <bool QSIDE, bool DAMP>
__device__ __forceinline__ void g_dtau_column(const GroupSmem *gs, int ks, int c, const float qd[kJoints],
                                              const float sq[kJoints], const float cq[kJoints],
                                              float dtau[kJoints]) {
    float df[kJoints][6];
    float dv[6] = {0, 0, 0, 0, 0, 0}, da[6] = {0, 0, 0, 0, 0, 0};
    static_for<0, kJoints>([&](auto K) {
        constexpr int k = decltype(K)::value;
        if constexpr (QSIDE && k == 0 && kDqColumn0Zero) {
#pragma unroll
            for (int i = 0; i < 6; i++) df[0][i] = 0.0f;  // dq column 0 is zero; c >= 1 on this side
            return;
        }
        float v[6], Iv[6];
        g_lds_link(gs, ks, k, v, Iv);
        // transform branch (k > c)
        float tdv[6], tda[6];
        xmotion<k>(tdv, dv, cq[k], sq[k]);
        xmotion<k>(tda, da, cq[k], sq[k]);
        // initial branch (k == c)
        float idv[6], ida[6];
        if constexpr (QSIDE) {
            idv[0] = v[1]; idv[1] = -v[0]; idv[2] = 0.0f; idv[3] = v[4]; idv[4] = -v[3]; idv[5] = 0.0f;
            const float4 xa = gs->link[ks][kSlotsPerLink * k + 3];
            ida[0] = xa.y; ida[1] = -xa.x; ida[2] = 0.0f; ida[3] = xa.w; ida[4] = -xa.z; ida[5] = 0.0f;
        } else {
            idv[0] = idv[1] = 0.0f; idv[2] = 1.0f; idv[3] = idv[4] = idv[5] = 0.0f;
            ida[0] = v[1]; ida[1] = -v[0]; ida[2] = 0.0f; ida[3] = v[4]; ida[4] = -v[3]; ida[5] = 0.0f;
        }
        const bool init = (k == c), live = (k >= c);
        float ndv[6], nda[6];
#pragma unroll
        for (int i = 0; i < 6; i++) {
            ndv[i] = init ? idv[i] : (live ? tdv[i] : 0.0f);
            nda[i] = init ? ida[i] : (live ? tda[i] : 0.0f);
        }
        nda[0] = fmaf(ndv[1], qd[k], nda[0]);
        nda[1] = fmaf(-ndv[0], qd[k], nda[1]);
        nda[3] = fmaf(ndv[4], qd[k], nda[3]);
        nda[4] = fmaf(-ndv[3], qd[k], nda[4]);
        float Idv[6];
        imul<k>(Idv, ndv);
        imul<k>(df[k], nda);
        crf_acc(df[k], ndv, Iv);
        crf_acc(df[k], v, Idv);
#pragma unroll
        for (int i = 0; i < 6; i++) { dv[i] = ndv[i]; da[i] = nda[i]; }
    });
    float dF[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    static_for_down<kJoints - 1, 0>([&](auto K) {
        constexpr int k = decltype(K)::value;
#pragma unroll
        for (int i = 0; i < 6; i++) dF[i] += df[k][i];  // df[k] is zero for k < c
        dtau[k] = dF[2];
        if constexpr (k > 0) {
            if constexpr (QSIDE) {
                const float4 fs = gs->link[ks][kSlotsPerLink * k + 4];  // (f0, f1, f3, f4)
                const float on = (k == c) ? 1.0f : 0.0f;
                dF[0] = fmaf(-on, fs.y, dF[0]);
                dF[1] = fmaf(on, fs.x, dF[1]);
                dF[3] = fmaf(-on, fs.w, dF[3]);
                dF[4] = fmaf(on, fs.z, dF[4]);
            }
            float t[6];
            xforce_T<k>(t, dF, cq[k], sq[k]);
#pragma unroll
            for (int i = 0; i < 6; i++) dF[i] = t[i];
        }
    });
    if (!QSIDE && DAMP) {
#pragma unroll
        for (int k = 0; k < kJoints; k++) dtau[k] += (k == c) ? 0.5f : 0.0f;
    }
}

// Full path for the (up to) 4 knots of one warp; lane = 8 * ks + g.
template <bool DAMP, bool MPC, bool MIRROR = false>
__device__ __forceinline__ void process_group(GroupSmem *gs, int lane, const KnotPtrs &kp,
                                              const KnotPtrs &mr = KnotPtrs{}) {
    constexpr int N = kJoints, NN = kMinvN;
    const int ks = lane >> 3, g = lane & 7;
    float q[N], qd[N], u[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
        q[j] = kp.q ? __ldg(kp.q + j) : 0.0f;
        qd[j] = kp.q ? __ldg(kp.qd + j) : 0.0f;
        u[j] = kp.q ? __ldg(kp.u + j) : 0.0f;
    }
    if constexpr (MIRROR) {
        if (mr.q && g < N) {  // entry g, picked with compile-time indices (no local-memory arrays)
            float qg = q[0], qdg = qd[0], ug = u[0];
#pragma unroll
            for (int j = 1; j < N; j++) {
                if (j == g) {
                    qg = q[j];
                    qdg = qd[j];
                    ug = u[j];
                }
            }
            const_cast<float *>(mr.q)[g] = qg;
            const_cast<float *>(mr.qd)[g] = qdg;
            const_cast<float *>(mr.u)[g] = ug;
        }
    }
    float sq[N], cq[N];
#pragma unroll
    for (int k = 0; k < kJoints; k++) sincos_angle(q[k], &sq[k], &cq[k]);

    // RNEA(q, qd, 0) -> bias, storing v_k, I v_k (every lane writes the same values)
    float bias[kJoints];
    {
        float f[kJoints][6], v[6], a[6];
        static_for<0, kJoints>([&](auto K) {
            constexpr int k = decltype(K)::value;
            if constexpr (k == 0) {
                v[0] = v[1] = 0.0f; v[2] = qd[0]; v[3] = v[4] = v[5] = 0.0f;
                if constexpr (MPC) {
#pragma unroll
                    for (int i = 0; i < 6; i++) a[i] = 0.0f;
                } else {
                    const float g6[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, kGravity};
                    xmotion<0>(a, g6, cq[0], sq[0]);
                }
            } else {
                float nv[6], na[6];
                xmotion<k>(nv, v, cq[k], sq[k]);
                nv[2] += qd[k];
                xmotion<k>(na, a, cq[k], sq[k]);
                na[0] = fmaf(nv[1], qd[k], na[0]);
                na[1] = fmaf(-nv[0], qd[k], na[1]);
                na[3] = fmaf(nv[4], qd[k], na[3]);
                na[4] = fmaf(-nv[3], qd[k], na[4]);
#pragma unroll
                for (int i = 0; i < 6; i++) { v[i] = nv[i]; a[i] = na[i]; }
            }
            float Iv[6];
            imul<k>(Iv, v);
            imul<k>(f[k], a);
            crf_acc(f[k], v, Iv);
            g_sts<k>(gs, ks, 0, make_float4(v[0], v[1], v[2], v[3]));
            g_sts<k>(gs, ks, 1, make_float4(v[4], v[5], Iv[0], Iv[1]));
            g_sts<k>(gs, ks, 2, make_float4(Iv[2], Iv[3], Iv[4], Iv[5]));
        });
        static_for_down<kJoints - 1, 0>([&](auto K) {
            constexpr int k = decltype(K)::value;
            const float c = f[k][2];
            bias[k] = DAMP ? u[k] - fmaf(0.5f, qd[k], c) : u[k] - c;
            if constexpr (k > 0) {
                float t[6];
                xforce_T<k>(t, f[k], cq[k], sq[k]);
#pragma unroll
                for (int i = 0; i < 6; i++) f[k - 1][i] += t[i];
            }
        });
    }

    // articulated-inertia sweep (replicated)
    float U[kJoints][6], Dinv[kJoints];
    {
        float A[3][3], B[3][3], M[3][3];
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
                float Ud[6];
#pragma unroll
                for (int i = 0; i < 6; i++) Ud[i] = U[k][i] * Dinv[k];
                float Aa[3][3], Ba[3][3], Ma[3][3];
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        Aa[i][j] = (i == 2 || j == 2) ? 0.0f : fmaf(-U[k][i], Ud[j], A[i][j]);
                        Ba[i][j] = (i == 2) ? 0.0f : fmaf(-U[k][i], Ud[3 + j], B[i][j]);
                        Ma[i][j] = fmaf(-U[k][3 + i], Ud[3 + j], M[i][j]);
                    }
                congruence<k>(A, B, M, Aa, Ba, Ma, cq[k], sq[k]);
            }
        });
    }

    // Minv column j = g (lanes g >= N repeat column N - 1): backward then
    // forward pass with the rows i > j masked to zero (minv.h:392-469
    // restricted to column j)
    {
        const int j = g < N ? g : N - 1;
        float col[kJoints];
        float F[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        static_for_down<kJoints - 1, 0>([&](auto II) {
            constexpr int i = decltype(II)::value;
            const float m = (i == j) ? Dinv[i] : ((i < j) ? -Dinv[i] * F[2] : 0.0f);
            col[i] = m;
#pragma unroll
            for (int r = 0; r < 6; r++) F[r] = fmaf(U[i][r], m, F[r]);
            if constexpr (i > 0) {
                float t[6];
                xforce_T<i>(t, F, cq[i], sq[i]);
#pragma unroll
                for (int r = 0; r < 6; r++) F[r] = t[r];
            }
        });
        static_for<0, kJoints>([&](auto II) {
            constexpr int i = decltype(II)::value;
            if constexpr (i == 0) {
#pragma unroll
                for (int r = 0; r < 6; r++) F[r] = 0.0f;
                F[2] = col[0];
            } else {
                float y[6];
                xmotion<i>(y, F, cq[i], sq[i]);
                float d = U[i][0] * y[0];
#pragma unroll
                for (int r = 1; r < 6; r++) d = fmaf(U[i][r], y[r], d);
                col[i] = (i <= j) ? fmaf(-Dinv[i], d, col[i]) : 0.0f;
#pragma unroll
                for (int r = 0; r < 6; r++) F[r] = y[r];
                F[2] += col[i];
            }
        });
        if (g < N) {
#pragma unroll
            for (int i = 0; i < kJoints; i++)
                if (i <= j) {
                    gs->minv[ks][i + N * j] = col[i];
                    gs->minv[ks][j + N * i] = col[i];
                }
        }
    }
    __syncwarp();
    // qdd = Minv bias (lane g < N computes entry g, shares it through smem)
    if (g < N) {
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < kJoints; k++) acc = fmaf(gs->minv[ks][g + N * k], bias[k], acc);
        gs->qdd[ks][g] = acc;
    }
    __syncwarp();
    float qdd[N];
#pragma unroll
    for (int k = 0; k < kJoints; k++) qdd[k] = gs->qdd[ks][k];

    // RNEA(q, qd, qdd): (X a)[0,1,3,4] and accumulated f[0,1,3,4] per link
    {
        float f[kJoints][6], a[6];
        static_for<0, kJoints>([&](auto K) {
            constexpr int k = decltype(K)::value;
            float v[6], Iv[6];
            g_lds_link(gs, ks, k, v, Iv);
            if constexpr (k == 0) {
                if constexpr (MPC) {
#pragma unroll
                    for (int i = 0; i < 6; i++) a[i] = 0.0f;
                } else {
                    const float g6[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, kGravity};
                    xmotion<0>(a, g6, cq[0], sq[0]);
                }
                if constexpr (!kDqColumn0Zero)  // X_0 a_base, read by d tau / dq column 0
                    g_sts<0>(gs, ks, 3, make_float4(a[0], a[1], a[3], a[4]));
                a[2] += qdd[0];
            } else {
                float xa[6];
                xmotion<k>(xa, a, cq[k], sq[k]);
                g_sts<k>(gs, ks, 3, make_float4(xa[0], xa[1], xa[3], xa[4]));
                a[0] = fmaf(v[1], qd[k], xa[0]);
                a[1] = fmaf(-v[0], qd[k], xa[1]);
                a[2] = xa[2] + qdd[k];
                a[3] = fmaf(v[4], qd[k], xa[3]);
                a[4] = fmaf(-v[3], qd[k], xa[4]);
                a[5] = xa[5];
            }
            imul<k>(f[k], a);
            crf_acc(f[k], v, Iv);
        });
        static_for_down<kJoints - 1, 1>([&](auto K) {
            constexpr int k = decltype(K)::value;
            g_sts<k>(gs, ks, 4, make_float4(f[k][0], f[k][1], f[k][3], f[k][4]));
            float t[6];
            xforce_T<k>(t, f[k], cq[k], sq[k]);
#pragma unroll
            for (int i = 0; i < 6; i++) f[k - 1][i] += t[i];
        });
    }
    __syncwarp();

    // tangent columns: dqd column g (lanes g < N) and dq column g_q_column(g)
    float mrow[N][N];
#pragma unroll
    for (int r = 0; r < N; r++)
#pragma unroll
        for (int k = 0; k < N; k++) mrow[r][k] = gs->minv[ks][r + N * k];
    {
        float dtau[N];
        g_dtau_column<false, DAMP>(gs, ks, g < N ? g : N, qd, sq, cq, dtau);  // c = N: all-zero column, unused
        if (g < N) {
#pragma unroll
            for (int r = 0; r < N; r++) {
                float acc = 0.0f;
#pragma unroll
                for (int k = 0; k < N; k++) acc = fmaf(mrow[r][k], dtau[k], acc);
                gs->out[ks][NN + N * g + r] = -acc;
            }
        }
    }
    {
        const int cq_col = g_q_column(g);  // N: no column
        float dtau[N];
        g_dtau_column<true, DAMP>(gs, ks, cq_col, qd, sq, cq, dtau);
        if (cq_col < N) {
#pragma unroll
            for (int r = 0; r < N; r++) {
                float acc = 0.0f;
#pragma unroll
                for (int k = 0; k < N; k++) acc = fmaf(mrow[r][k], dtau[k], acc);
                gs->out[ks][N * cq_col + r] = -acc;
            }
        } else if (kDqColumn0Zero && g == 0) {
#pragma unroll
            for (int r = 0; r < N; r++) gs->out[ks][r] = 0.0f;  // dq column 0 is identically zero
        }
    }
    __syncwarp();
    // write the knot's outputs: group lanes stride over its floats
    if (kp.q) {
        for (int e = g; e < kDqddN; e += kGroupLanes) kp.dqdd[e] = gs->out[ks][e];
        for (int e = g; e < NN; e += kGroupLanes) kp.minv[e] = gs->minv[ks][e];
        if (g < N) kp.qdd[g] = gs->qdd[ks][g];
        if constexpr (MIRROR) {
            if (mr.dqdd) {
                for (int e = g; e < kDqddN; e += kGroupLanes) mr.dqdd[e] = gs->out[ks][e];
                for (int e = g; e < NN; e += kGroupLanes) mr.minv[e] = gs->minv[ks][e];
                if (g < N) mr.qdd[g] = gs->qdd[ks][g];
            }
        }
    }
    __syncwarp();
}

}  // namespace frg
