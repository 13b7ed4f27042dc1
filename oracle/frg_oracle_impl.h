/* CPU restatement of the reference's iiwa_14 forward-dynamics gradient.
 *
 * ORACLE TEST INFRASTRUCTURE ONLY.  Included twice by frg_oracle.c (REAL =
 * double and REAL = float, FN() adds the suffix).  It is the checker for the
 * CUDA path and the timed CPU baseline; the product library never links it.
 *
 * It follows the reference's algorithm (helpers_CPU/dynamicsGradient.h,
 * helpers_CPU/minv.h) step for step with plain dense 6x6 column-major
 * arithmetic: every matrix is stored A[r + 6*c] exactly like the reference.
 * Where the reference hard-codes the model as generated code, this file derives
 * the same numbers from the URDF joint frames and link inertias.
 */

#define SZ6 6
#define NJ FRG_MODEL_NUM_JOINTS

/* ---------------------------------------------------------------- model ---- */

/* 6x6 spatial inertia about the joint origin from (mass, COM, inertia at COM):
 * [ Icom + m (c.c 1 - c c^T)   m c^ ]
 * [ m c^T                      m 1  ]   (c^ = cross-product matrix of c).
 * Same matrix as buildI6x6, helpers_CPU/dynamicsGradient.h:78-118. */
static void FN(spatial_inertia)(REAL *I, const double p[10]) {
    const REAL Ixx = (REAL)p[0], Ixy = (REAL)p[1], Ixz = (REAL)p[2], Iyy = (REAL)p[3], Iyz = (REAL)p[4],
               Izz = (REAL)p[5], cx = (REAL)p[6], cy = (REAL)p[7], cz = (REAL)p[8], m = (REAL)p[9];
    for (int i = 0; i < 36; i++) I[i] = (REAL)0;
    I[0 + 6 * 0] = Ixx + m * (cy * cy + cz * cz);
    I[1 + 6 * 1] = Iyy + m * (cx * cx + cz * cz);
    I[2 + 6 * 2] = Izz + m * (cx * cx + cy * cy);
    I[1 + 6 * 0] = I[0 + 6 * 1] = Ixy - m * cx * cy;
    I[2 + 6 * 0] = I[0 + 6 * 2] = Ixz - m * cx * cz;
    I[2 + 6 * 1] = I[1 + 6 * 2] = Iyz - m * cy * cz;
    /* m c^ in the top-right block, its transpose bottom-left */
    const REAL mc[3] = {m * cx, m * cy, m * cz};
    const REAL C[9] = {0, mc[2], -mc[1], -mc[2], 0, mc[0], mc[1], -mc[0], 0}; /* c^ column-major */
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) {
            I[r + 6 * (c + 3)] = C[r + 3 * c];
            I[(c + 3) + 6 * r] = C[r + 3 * c];
        }
    I[3 + 6 * 3] = I[4 + 6 * 4] = I[5 + 6 * 5] = m;
}

/* All NJ link inertias (initInertiaTensors, dynamicsGradient.h:124-212). */
static void FN(model_inertias)(REAL *I) {
    for (int k = 0; k < NJ; k++) FN(spatial_inertia)(&I[36 * k], kLinkInertial[k]);
}

/* Motion transform  iX(i-1) = [E 0; -E r^ E]  of each joint for its q, where
 * E = Rz(q)^T * F (F: the fixed frame rotation of the joint, transposed) and r
 * the joint origin in the parent frame.  Gives the same 7 matrices that
 * buildTransforms / updateTransforms write out (dynamicsGradient.h:231-587). */
static void FN(model_transforms)(REAL *X, const REAL *sinq, const REAL *cosq) {
    for (int k = 0; k < NJ; k++) {
        REAL *Xk = &X[36 * k];
        const REAL s = sinq[k], c = cosq[k];
        const REAL RzT[9] = {c, -s, 0, s, c, 0, 0, 0, 1}; /* column-major Rz(q)^T */
        REAL E[9], rx[9], Erx[9];
        for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) {
                REAL acc = 0;
                for (int l = 0; l < 3; l++) {
                    const REAL f = (REAL)kJointFT[k][l + 3 * j];
                    if (f != 0) acc += RzT[i + 3 * l] * f;
                }
                E[i + 3 * j] = acc;
            }
        const REAL r0 = (REAL)kJointOrigin[k][0], r1 = (REAL)kJointOrigin[k][1], r2 = (REAL)kJointOrigin[k][2];
        /* r^ column-major */
        rx[0] = 0;   rx[1] = r2;  rx[2] = -r1;
        rx[3] = -r2; rx[4] = 0;   rx[5] = r0;
        rx[6] = r1;  rx[7] = -r0; rx[8] = 0;
        for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) {
                REAL acc = 0;
                for (int l = 0; l < 3; l++)
                    if (rx[l + 3 * j] != 0 && E[i + 3 * l] != 0) acc += E[i + 3 * l] * rx[l + 3 * j];
                Erx[i + 3 * j] = acc;
            }
        for (int i = 0; i < 36; i++) Xk[i] = 0;
        for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) {
                Xk[i + 6 * j] = E[i + 3 * j];
                Xk[(i + 3) + 6 * (j + 3)] = E[i + 3 * j];
                Xk[(i + 3) + 6 * j] = -Erx[i + 3 * j];
            }
    }
}

/* --------------------------------------------------------- small algebra ---- */

/* y (+)= X x for a joint transform; the top-right 3x3 block of X is zero
 * (the sparsity matVMult_Tmat uses, helpers_CPU/math.h:65-88). */
static void FN(xform_motion)(REAL *y, const REAL *X, const REAL *x, int accumulate) {
    for (int r = 0; r < 6; r++) {
        REAL acc = 0;
        const int cmax = (r < 3) ? 3 : 6;
        for (int c = 0; c < cmax; c++) acc += X[r + 6 * c] * x[c];
        y[r] = accumulate ? y[r] + acc : acc;
    }
}

/* y (+)= X^T x (force transform to the parent). */
static void FN(xform_force_T)(REAL *y, const REAL *X, const REAL *x, int accumulate) {
    for (int r = 0; r < 6; r++) {
        REAL acc = 0;
        const int c0 = (r < 3) ? 0 : 3;
        for (int c = c0; c < 6; c++) acc += X[c + 6 * r] * x[c];
        y[r] = accumulate ? y[r] + acc : acc;
    }
}

/* y (+)= A x, dense 6x6. */
static void FN(mat6_vec)(REAL *y, const REAL *A, const REAL *x, int accumulate) {
    for (int r = 0; r < 6; r++) {
        REAL acc = 0;
        for (int c = 0; c < 6; c++) acc += A[r + 6 * c] * x[c];
        y[r] = accumulate ? y[r] + acc : acc;
    }
}

/* crf(v) h : spatial force cross product (v x* h). */
static void FN(cross_force)(REAL *y, const REAL *v, const REAL *h) {
    y[0] = v[1] * h[2] - v[2] * h[1] + v[4] * h[5] - v[5] * h[4];
    y[1] = v[2] * h[0] - v[0] * h[2] + v[5] * h[3] - v[3] * h[5];
    y[2] = v[0] * h[1] - v[1] * h[0] + v[3] * h[4] - v[4] * h[3];
    y[3] = v[1] * h[5] - v[2] * h[4];
    y[4] = v[2] * h[3] - v[0] * h[5];
    y[5] = v[0] * h[4] - v[1] * h[3];
}

/* crm(x) S * s for S = e_z (revolute about z): (x1, -x0, 0, x4, -x3, 0) * s. */
static void FN(cross_motion_S)(REAL *y, const REAL *x, REAL s, int accumulate) {
    const REAL t[6] = {x[1] * s, -x[0] * s, 0, x[4] * s, -x[3] * s, 0};
    for (int i = 0; i < 6; i++) y[i] = accumulate ? y[i] + t[i] : t[i];
}

/* ------------------------------------------------------------------ RNEA ---- */

/* Forward sweep for v, a, f (RNEA_fp, dynamicsGradient.h:620-659):
 *   v_k = X_k v_{k-1} + S qd_k,  a_k = X_k a_{k-1} + (v_k x S) qd_k + S qdd_k,
 *   f_k = I_k a_k + v_k x* I_k v_k - fext_k;  a_0 carries gravity as the base
 *   acceleration X_0 [0 0 0 0 0 g]^T unless mpc (gravity compensated). */
static void FN(rnea_forward)(REAL *v, REAL *a, REAL *f, const REAL *X, const REAL *I, const REAL *qd,
                             const REAL *qdd, const REAL *fext, int mpc) {
    for (int k = 0; k < NJ; k++) {
        REAL *vk = &v[6 * k], *ak = &a[6 * k], *fk = &f[6 * k];
        const REAL *Xk = &X[36 * k], *Ik = &I[36 * k];
        if (k == 0) {
            for (int i = 0; i < 6; i++) vk[i] = 0;
            vk[2] = qd[0];
            ak[0] = ak[1] = 0;
            ak[2] = qdd ? qdd[0] : 0;
            for (int i = 3; i < 6; i++) ak[i] = mpc ? (REAL)0 : Xk[i + 6 * 5] * (REAL)kGravity;
        } else {
            FN(xform_motion)(vk, Xk, &v[6 * (k - 1)], 0);
            vk[2] += qd[k];
            FN(cross_motion_S)(ak, vk, qd[k], 0);
            FN(xform_motion)(ak, Xk, &a[6 * (k - 1)], 1);
            if (qdd) ak[2] += qdd[k];
        }
        REAL Iv[6];
        FN(mat6_vec)(Iv, Ik, vk, 0);
        FN(cross_force)(fk, vk, Iv);
        FN(mat6_vec)(fk, Ik, ak, 1);
        if (fext)
            for (int i = 0; i < 6; i++) fk[i] -= fext[6 * k + i];
    }
}

/* Backward sweep f_{k-1} += X_k^T f_k, tau_k = f_k[2] (RNEA_bp, :662-670). */
static void FN(rnea_backward)(REAL *tau, REAL *f, const REAL *X) {
    for (int k = NJ - 1; k >= 0; k--) {
        if (tau) tau[k] = f[6 * k + 2];
        if (k > 0) FN(xform_force_T)(&f[6 * (k - 1)], &X[36 * k], &f[6 * k], 1);
    }
}

/* ------------------------------------------------------------------ Minv ---- */

/* Minv by the ABA-style backward/forward passes of helpers_CPU/minv.h:392-477
 * (Carpentier 2018 structure, RobCoGen articulated-inertia helpers).  Writes
 * the upper triangle of Minv (Minv[i + 7 j], j >= i) and zeros the rest, the
 * layout computeMinv returns (minv.h:472-477, forwardDynamics :700). */
static void FN(compute_minv)(REAL *Minv, const REAL *X, const REAL *I) {
    REAL IA[NJ * 36], F[NJ * 6 * NJ], U[NJ * 6], Dinv[NJ];
    for (int i = 0; i < NJ * 36; i++) IA[i] = I[i];
    for (int i = 0; i < NJ * 6 * NJ; i++) F[i] = 0;
    for (int i = 0; i < NJ * NJ; i++) Minv[i] = 0;
    /* backward pass: Minv_bp :424-436 with bwdPassMinvFUpdate :392-412 and
     * bwdPassIUpdate :415-421 (compute_Ia_revolute :147, ctransform :222) */
    for (int i = NJ - 1; i >= 0; i--) {
        REAL *Ui = &U[6 * i], *IAi = &IA[36 * i], *Fi = &F[6 * NJ * i];
        for (int r = 0; r < 6; r++) Ui[r] = IAi[r + 6 * 2];
        Dinv[i] = (REAL)1 / Ui[2];
        Minv[i + NJ * i] = Dinv[i];
        for (int j = i + 1; j < NJ; j++) Minv[i + NJ * j] = -Dinv[i] * Fi[2 + 6 * j];
        for (int j = i; j < NJ; j++)
            for (int r = 0; r < 6; r++) Fi[r + 6 * j] += Ui[r] * Minv[i + NJ * j];
        if (i == 0) continue;
        const REAL *Xi = &X[36 * i];
        REAL *Fp = &F[6 * NJ * (i - 1)];
        for (int j = i; j < NJ; j++) FN(xform_force_T)(&Fp[6 * j], Xi, &Fi[6 * j], 1);
        /* Ia = IA_i - U U^T / D with the joint row/column exactly zero,
         * then IA_parent += X^T Ia X */
        REAL Ia[36], Y[36];
        for (int c = 0; c < 6; c++)
            for (int r = 0; r < 6; r++) Ia[r + 6 * c] = IAi[r + 6 * c] - Ui[r] * (Ui[c] * Dinv[i]);
        for (int t = 0; t < 6; t++) Ia[2 + 6 * t] = Ia[t + 6 * 2] = 0;
        for (int c = 0; c < 6; c++) FN(mat6_vec)(&Y[6 * c], Ia, &Xi[6 * c], 0);
        REAL *IAp = &IA[36 * (i - 1)];
        for (int c = 0; c < 6; c++)
            for (int r = 0; r < 6; r++) {
                REAL acc = 0;
                for (int l = 0; l < 6; l++) acc += Xi[l + 6 * r] * Y[l + 6 * c];
                IAp[r + 6 * c] += acc;
            }
    }
    /* forward pass: Minv_fp :463-469 with fwdPassUpdate :440-461 */
    for (int i = 0; i < NJ; i++) {
        REAL *Fi = &F[6 * NJ * i];
        const REAL *Xi = &X[36 * i];
        if (i > 0) {
            const REAL *Fp = &F[6 * NJ * (i - 1)];
            REAL w[6];
            for (int r = 0; r < 6; r++) {
                REAL acc = 0;
                for (int l = 0; l < 6; l++) acc += Xi[l + 6 * r] * U[6 * i + l];
                w[r] = acc; /* X_i^T U_i */
            }
            for (int j = i; j < NJ; j++) {
                REAL acc = 0;
                for (int l = 0; l < 6; l++) acc += w[l] * Fp[l + 6 * j];
                Minv[i + NJ * j] += -Dinv[i] * acc;
            }
        }
        for (int j = i; j < NJ; j++) {
            for (int r = 0; r < 6; r++) Fi[r + 6 * j] = 0;
            Fi[2 + 6 * j] = Minv[i + NJ * j];
            if (i > 0) FN(mat6_vec)(&Fi[6 * j], Xi, &F[6 * NJ * (i - 1) + 6 * j], 1);
        }
    }
}

/* ----------------------------------------------------- derivative sweeps ---- */

/* d tau / d q and d tau / d qd, one column (one differentiated joint) at a
 * time.  Same recursions as compute_vafdu (dynamicsGradient.h:787-829) and
 * compute_cdu (:832-857), which interleave the columns inside the link loop;
 * every column's arithmetic is identical, only the loop nesting differs.
 *   forward  (links k >= c):
 *     dv_k = X_k dv_{k-1}  or, at k == c, crm(X_k v_{k-1}) S (q) / S (qd)
 *     da_k = X_k da_{k-1} + crm(dv_k) S qd_k  (+ crm(X_k a_{k-1}) S (q, k == c)
 *            or crm(v_k) S (qd, k == c))
 *     df_k = I_k da_k + dv_k x* (I_k v_k) + v_k x* (I_k dv_k)
 *   backward (links k = 6..1): dF_{k-1} += X_k^T dF_k  (+ X_k^T (S x* f_k) for
 *     q at k == c),  dtau_k = dF_k[2];  damping adds 0.5 to d tau_c / d qd_c.
 * Column 0 of d tau / d q is identically zero when the base joint is parallel
 * to gravity (the iiwa; the reference sets it so, :797-813): it is skipped
 * then, and computed from the base's zero velocity and gravity otherwise. */
static void FN(dtau_columns)(REAL *cdq, REAL *cdqd, const REAL *v, const REAL *a, const REAL *f, const REAL *X,
                             const REAL *I, const REAL *qd, int damping, int mpc) {
    /* X_0 v_base = 0 and X_0 a_base (gravity as base acceleration) for column 0 */
    REAL v_base[6] = {0, 0, 0, 0, 0, 0}, a_base[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 3; i < 6; i++) a_base[i] = mpc ? (REAL)0 : X[i + 6 * 5] * (REAL)kGravity;
    for (int side = 0; side < 2; side++) {
        REAL *out = side == 0 ? cdq : cdqd;
        for (int c = 0; c < NJ; c++) {
            REAL dF[NJ * 6];
            for (int i = 0; i < NJ * 6; i++) dF[i] = 0;
            if (!(side == 0 && c == 0 && FRG_MODEL_DQ_COLUMN0_ZERO)) {
                REAL dv[6], da[6];
                for (int k = c; k < NJ; k++) {
                    const REAL *Xk = &X[36 * k], *Ik = &I[36 * k], *vk = &v[6 * k];
                    REAL ndv[6], nda[6];
                    if (k == c) {
                        if (side == 0) {
                            REAL Xv[6];
                            if (k > 0) FN(xform_motion)(Xv, Xk, &v[6 * (k - 1)], 0);
                            else for (int i = 0; i < 6; i++) Xv[i] = v_base[i];
                            FN(cross_motion_S)(ndv, Xv, 1, 0);
                        } else {
                            for (int i = 0; i < 6; i++) ndv[i] = 0;
                            ndv[2] = 1;
                        }
                    } else {
                        FN(xform_motion)(ndv, Xk, dv, 0);
                    }
                    FN(cross_motion_S)(nda, ndv, qd[k], 0);
                    if (k == c) {
                        if (side == 0) {
                            REAL Xa[6];
                            if (k > 0) FN(xform_motion)(Xa, Xk, &a[6 * (k - 1)], 0);
                            else for (int i = 0; i < 6; i++) Xa[i] = a_base[i];
                            FN(cross_motion_S)(nda, Xa, 1, 1);
                        } else {
                            FN(cross_motion_S)(nda, vk, 1, 1);
                        }
                    } else {
                        FN(xform_motion)(nda, Xk, da, 1);
                    }
                    REAL Iv[6], Idv[6], t[6];
                    FN(mat6_vec)(Iv, Ik, vk, 0);
                    FN(mat6_vec)(Idv, Ik, ndv, 0);
                    REAL *dfk = &dF[6 * k];
                    FN(cross_force)(dfk, ndv, Iv);
                    FN(mat6_vec)(dfk, Ik, nda, 1);
                    FN(cross_force)(t, vk, Idv);
                    for (int i = 0; i < 6; i++) dfk[i] += t[i];
                    for (int i = 0; i < 6; i++) { dv[i] = ndv[i]; da[i] = nda[i]; }
                }
            }
            for (int k = NJ - 1; k >= 0; k--) {
                out[k + NJ * c] = dF[6 * k + 2];
                if (k == 0) break;
                FN(xform_force_T)(&dF[6 * (k - 1)], &X[36 * k], &dF[6 * k], 1);
                if (side == 0 && k == c && c > 0) {
                    const REAL *fk = &f[6 * k];
                    const REAL g[6] = {-fk[1], fk[0], 0, -fk[4], fk[3], 0}; /* S x* f_k */
                    FN(xform_force_T)(&dF[6 * (k - 1)], &X[36 * k], g, 1);
                }
            }
            if (side == 1 && damping) out[c + NJ * c] += (REAL)0.5;
        }
    }
}

/* ------------------------------------------------------------- per knot ---- */

/* One knot of the full path, forwardDynamicsGradientThreaded with
 * QDD_MINV_PASSED_IN=false (dynamicsGradient.h:925-934 via :869-897):
 *   RNEA(q, qd, 0) -> bias = u - c (- 0.5 qd) -> Minv -> qdd = Minv bias
 *   -> RNEA(q, qd, qdd) -> d tau -> dqdd = -Minv [d tau/dq | d tau/dqd].
 * Outputs: dqdd[2 NJ^2] (NJ x 2NJ column-major), qdd[NJ], Minv[NJ^2] dense
 * (98, 7 and 49 floats for the 7-joint iiwa). */
static void FN(knot_gradient)(const REAL *q, const REAL *qd, const REAL *u, const REAL *fext, int damping,
                              int mpc, REAL *dqdd, REAL *qdd, REAL *minv_dense) {
    REAL sq[NJ], cq[NJ], X[NJ * 36], I[NJ * 36];
    for (int k = 0; k < NJ; k++) { sq[k] = (REAL)sin(q[k]); cq[k] = (REAL)cos(q[k]); }
    FN(model_transforms)(X, sq, cq);
    FN(model_inertias)(I);
    REAL v[NJ * 6], a[NJ * 6], f[NJ * 6], c[NJ], bias[NJ], Minv[NJ * NJ];
    FN(rnea_forward)(v, a, f, X, I, qd, NULL, fext, mpc);
    FN(rnea_backward)(c, f, X);
    for (int k = 0; k < NJ; k++) bias[k] = damping ? u[k] - (c[k] + (REAL)0.5 * qd[k]) : u[k] - c[k];
    FN(compute_minv)(Minv, X, I);
    /* qdd = Minv_sym * bias with the upper triangle (matVMultSym, math.h:29-37) */
    for (int r = 0; r < NJ; r++) {
        REAL acc = 0;
        for (int k = 0; k < NJ; k++) acc += (r <= k ? Minv[r + NJ * k] : Minv[k + NJ * r]) * bias[k];
        qdd[r] = acc;
    }
    FN(rnea_forward)(v, a, f, X, I, qd, qdd, fext, mpc);
    FN(rnea_backward)(NULL, f, X);
    REAL cdu[2 * NJ * NJ];
    FN(dtau_columns)(cdu, &cdu[NJ * NJ], v, a, f, X, I, qd, damping, mpc);
    /* dqdd = -Minv_sym * cdu (matMultSym, math.h:17-25, call :933) */
    for (int col = 0; col < 2 * NJ; col++)
        for (int r = 0; r < NJ; r++) {
            REAL acc = 0;
            for (int k = 0; k < NJ; k++) acc += (r <= k ? Minv[r + NJ * k] : Minv[k + NJ * r]) * cdu[k + NJ * col];
            dqdd[r + NJ * col] = -acc;
        }
    for (int cc = 0; cc < NJ; cc++)
        for (int r = 0; r < NJ; r++) minv_dense[r + NJ * cc] = r <= cc ? Minv[r + NJ * cc] : Minv[cc + NJ * r];
}

/* The reference's time_CPU mode, QDD_MINV_PASSED_IN=true (dynamicsGradient.h:
 * 869-897 with the flag set, :925-934): q̈ and Minv (dense) come in, RNEA runs
 * once with that q̈, then d tau and dqdd = -Minv [d tau/dq | d tau/dqd]. */
static void FN(knot_gradient_given)(const REAL *q, const REAL *qd, const REAL *qdd, const REAL *minv_dense,
                                    int damping, int mpc, REAL *dqdd) {
    REAL sq[NJ], cq[NJ], X[NJ * 36], I[NJ * 36];
    for (int k = 0; k < NJ; k++) { sq[k] = (REAL)sin(q[k]); cq[k] = (REAL)cos(q[k]); }
    FN(model_transforms)(X, sq, cq);
    FN(model_inertias)(I);
    REAL v[NJ * 6], a[NJ * 6], f[NJ * 6];
    FN(rnea_forward)(v, a, f, X, I, qd, qdd, NULL, mpc);
    FN(rnea_backward)(NULL, f, X);
    REAL cdu[2 * NJ * NJ];
    FN(dtau_columns)(cdu, &cdu[NJ * NJ], v, a, f, X, I, qd, damping, mpc);
    for (int col = 0; col < 2 * NJ; col++)
        for (int r = 0; r < NJ; r++) {
            REAL acc = 0;
            for (int k = 0; k < NJ; k++) acc += (r <= k ? minv_dense[r + NJ * k] : minv_dense[k + NJ * r]) * cdu[k + NJ * col];
            dqdd[r + NJ * col] = -acc;
        }
}
