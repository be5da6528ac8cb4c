// prim_math.cuh -- per-primitive device math shared by the drop-in operator
// kernels (prim.cu) and the fused per-view kernels.
//
// Every function restates one step of the reference path; the operation
// order of the projection follows the reference (glm's row-by-column sums,
// left-to-right products) so that, compiled with the same flags, radii and
// tile boxes come out identical.
#pragma once

#include "ubs_common.cuh"

namespace ubs {

// 3x3 row-major helpers ------------------------------------------------------
struct M3 {
    float m[9];
    __device__ __forceinline__ float &operator()(int r, int c) { return m[r * 3 + c]; }
    __device__ __forceinline__ float operator()(int r, int c) const { return m[r * 3 + c]; }
};
// (A B)(r,c) = A(r,0)B(0,c) + A(r,1)B(1,c) + A(r,2)B(2,c), in that order
__device__ __forceinline__ M3 mm(const M3 &A, const M3 &B) {
    M3 C;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) C(r, c) = A(r, 0) * B(0, c) + A(r, 1) * B(1, c) + A(r, 2) * B(2, c);
    return C;
}
__device__ __forceinline__ M3 tr(const M3 &A) {
    M3 B;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) B(r, c) = A(c, r);
    return B;
}

// Camera ----------------------------------------------------------------------
struct Cam {
    M3 R;
    float t[3];
    float fx, fy, cx, cy;
};
__device__ __forceinline__ Cam load_cam(const float *vm, const float *K) {
    Cam c;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int k = 0; k < 3; ++k) c.R(r, k) = vm[r * 4 + k];
        c.t[r] = vm[r * 4 + 3];
    }
    c.fx = K[0];
    c.cx = K[2];
    c.fy = K[4];
    c.cy = K[5];
    return c;
}
__device__ __forceinline__ void world_to_cam(const Cam &c, const float *p, float *pc) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
        pc[r] = (c.R(r, 0) * p[0] + c.R(r, 1) * p[1] + c.R(r, 2) * p[2]) + c.t[r];
}

// Unit-quaternion rotation (w, x, y, z), utils.cuh:13-36.
__device__ __forceinline__ M3 quat_to_R(const float *q) {
    float w = q[0], x = q[1], y = q[2], z = q[3];
    const float inv = rsqrtf(x * x + y * y + z * z + w * w);
    x *= inv;
    y *= inv;
    z *= inv;
    w *= inv;
    const float x2 = x * x, y2 = y * y, z2 = z * z;
    const float xy = x * y, xz = x * z, yz = y * z;
    const float wx = w * x, wy = w * y, wz = w * z;
    M3 R;
    R(0, 0) = 1.f - 2.f * (y2 + z2);
    R(1, 0) = 2.f * (xy + wz);
    R(2, 0) = 2.f * (xz - wy);
    R(0, 1) = 2.f * (xy - wz);
    R(1, 1) = 1.f - 2.f * (x2 + z2);
    R(2, 1) = 2.f * (yz + wx);
    R(0, 2) = 2.f * (xz + wy);
    R(1, 2) = 2.f * (yz - wx);
    R(2, 2) = 1.f - 2.f * (x2 + y2);
    return R;
}

// Perspective projection state, utils.cuh:253-292.
struct Persp {
    float rz, rz2, tx, ty, limxp, limxn, limyp, limyn;
    float J[6]; // row-major 2x3
};
__device__ __forceinline__ Persp persp_setup(const float *pc, float fx, float fy, float cx,
                                             float cy, uint32_t W, uint32_t H) {
    Persp p;
    const float x = pc[0], y = pc[1], z = pc[2];
    const float tan_fovx = 0.5f * W / fx;
    const float tan_fovy = 0.5f * H / fy;
    p.limxp = (W - cx) / fx + 0.3f * tan_fovx;
    p.limxn = cx / fx + 0.3f * tan_fovx;
    p.limyp = (H - cy) / fy + 0.3f * tan_fovy;
    p.limyn = cy / fy + 0.3f * tan_fovy;
    p.rz = 1.f / z;
    p.rz2 = p.rz * p.rz;
    p.tx = z * fminf(p.limxp, fmaxf(-p.limxn, x * p.rz));
    p.ty = z * fminf(p.limyp, fmaxf(-p.limyn, y * p.rz));
    p.J[0] = fx * p.rz;
    p.J[1] = 0.f;
    p.J[2] = -fx * p.tx * p.rz2;
    p.J[3] = 0.f;
    p.J[4] = fy * p.rz;
    p.J[5] = -fy * p.ty * p.rz2;
    return p;
}

// cov2d = (J S) J^T, returned row-major 2x2
__device__ __forceinline__ void project_cov(const float *J, const M3 &S, float *c2) {
    float JS[6];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            JS[r * 3 + c] = J[r * 3 + 0] * S(0, c) + J[r * 3 + 1] * S(1, c) + J[r * 3 + 2] * S(2, c);
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c)
            c2[r * 2 + c] = JS[r * 3 + 0] * J[c * 3 + 0] + JS[r * 3 + 1] * J[c * 3 + 1] +
                            JS[r * 3 + 2] * J[c * 3 + 2];
}

// Result of the 2-D part of the projection for one (camera, primitive).
struct Proj2D {
    float mx, my, depth;
    float conic[3];
    float comp;
    int32_t radius; // 0 = culled
};

// Projection of a camera-space mean and covariance: blur, inverse, 1-sigma
// radius, image cull (fully_fused_projection_fwd.cu:104-176, utils.cuh:438-466).
__device__ __forceinline__ Proj2D project_2d(const float *pc, const M3 &Sc, const Cam &cam,
                                             uint32_t W, uint32_t H, float eps2d,
                                             float radius_clip) {
    Proj2D o;
    o.radius = 0;
    o.comp = 0.f;
    const Persp pp = persp_setup(pc, cam.fx, cam.fy, cam.cx, cam.cy, W, H);
    float c2[4];
    project_cov(pp.J, Sc, c2);
    o.mx = cam.fx * pc[0] * pp.rz + cam.cx;
    o.my = cam.fy * pc[1] * pp.rz + cam.cy;
    o.depth = pc[2];
    // add_blur: c2 row-major; glm covar[0][1] is element (1,0)
    const float det_orig = c2[0] * c2[3] - c2[2] * c2[1];
    c2[0] += eps2d;
    c2[3] += eps2d;
    const float det = c2[0] * c2[3] - c2[2] * c2[1];
    o.comp = sqrtf(fmaxf(0.f, det_orig / det));
    if (det <= 0.f) return o;
    const float invdet = 1.f / det;
    o.conic[0] = c2[3] * invdet;
    o.conic[1] = -c2[2] * invdet;
    o.conic[2] = c2[0] * invdet;
    const float b = 0.5f * (c2[0] + c2[3]);
    const float v1 = b + sqrtf(fmaxf(0.01f, b * b - det));
    const float radius = ceilf(sqrtf(v1));
    if (radius <= radius_clip) return o;
    if (o.mx + radius <= 0 || o.mx - radius >= (float)(int32_t)W || o.my + radius <= 0 ||
        o.my - radius >= (float)(int32_t)H)
        return o;
    o.radius = (int32_t)radius;
    return o;
}

// VJP of the perspective projection given d cov2d (row-major 2x2) and d mean2d:
// utils.cuh:295-372.  Adds into v_Sc and v_pc.
__device__ __forceinline__ void persp_vjp(const float *pc, const M3 &Sc, const Cam &cam,
                                          uint32_t W, uint32_t H, const float *vc2, float vmx,
                                          float vmy, M3 &vSc, float *vpc) {
    const Persp pp = persp_setup(pc, cam.fx, cam.fy, cam.cx, cam.cy, W, H);
    const float *J = pp.J;
    const float fx = cam.fx, fy = cam.fy, rz = pp.rz, rz2 = pp.rz2;
    // v_Sc += J^T vc2 J
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 2; ++b) acc += J[a * 3 + r] * vc2[a * 2 + b] * J[b * 3 + c];
            vSc(r, c) += acc;
        }
    vpc[0] += fx * rz * vmx;
    vpc[1] += fy * rz * vmy;
    vpc[2] += -(fx * pc[0] * vmx + fy * pc[1] * vmy) * rz2;
    // v_J = vc2 J Sc^T + vc2^T J Sc
    float vJ[6];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int m = 0; m < 3; ++m)
                    acc += vc2[r * 2 + b] * J[b * 3 + m] * Sc(c, m) +
                           vc2[b * 2 + r] * J[b * 3 + m] * Sc(m, c);
            vJ[r * 3 + c] = acc;
        }
    const float rz3 = rz2 * rz;
    const float xr = pc[0] * rz, yr = pc[1] * rz;
    if (xr <= pp.limxp && xr >= -pp.limxn) vpc[0] += -fx * rz2 * vJ[2];
    else vpc[2] += -fx * rz3 * vJ[2] * pp.tx;
    if (yr <= pp.limyp && yr >= -pp.limyn) vpc[1] += -fy * rz2 * vJ[5];
    else vpc[2] += -fy * rz3 * vJ[5] * pp.ty;
    vpc[2] += -fx * rz2 * vJ[0] - fy * rz2 * vJ[4] + 2.f * fx * pp.tx * rz3 * vJ[2] +
              2.f * fy * pp.ty * rz3 * vJ[5];
}

// d cov2d from d conic (inverse VJP) plus the optional compensation term
// (fully_fused_projection_bwd.cu:69-83, utils.cuh:451-502).
__device__ __forceinline__ void conic_vjp(const float *cn, const float *vcn, float eps2d,
                                          bool with_comp, float comp, float vcomp, float *vc2) {
    const float P[4] = {cn[0], cn[1], cn[1], cn[2]};
    const float vP[4] = {vcn[0], vcn[1] * .5f, vcn[1] * .5f, vcn[2]};
    float t[4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) t[r * 2 + c] = P[r * 2] * vP[c] + P[r * 2 + 1] * vP[2 + c];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) vc2[r * 2 + c] = -(t[r * 2] * P[c] + t[r * 2 + 1] * P[2 + c]);
    if (with_comp) {
        const float detc = P[0] * P[3] - P[1] * P[2];
        const float vsq = vcomp * 0.5f / (comp + 1e-6f);
        const float om = 1.f - comp * comp;
        vc2[0] += vsq * (om * P[0] - eps2d * detc);
        vc2[1] += vsq * (om * P[1]);
        vc2[2] += vsq * (om * P[2]);
        vc2[3] += vsq * (om * P[3] - eps2d * detc);
    }
}

// VJP of the unit-quaternion rotation (utils.cuh:38-62).
__device__ __forceinline__ void quat_vjp(const float *q, const M3 &vR, float *vq) {
    float w = q[0], x = q[1], y = q[2], z = q[3];
    const float inv = rsqrtf(x * x + y * y + z * z + w * w);
    x *= inv;
    y *= inv;
    z *= inv;
    w *= inv;
    // g(c, r) = vR(r, c)
#define G(c, r) vR(r, c)
    float vn[4];
    vn[0] = 2.f * (x * (G(1, 2) - G(2, 1)) + y * (G(2, 0) - G(0, 2)) + z * (G(0, 1) - G(1, 0)));
    vn[1] = 2.f * (-2.f * x * (G(1, 1) + G(2, 2)) + y * (G(0, 1) + G(1, 0)) +
                   z * (G(0, 2) + G(2, 0)) + w * (G(1, 2) - G(2, 1)));
    vn[2] = 2.f * (x * (G(0, 1) + G(1, 0)) - 2.f * y * (G(0, 0) + G(2, 2)) +
                   z * (G(1, 2) + G(2, 1)) + w * (G(2, 0) - G(0, 2)));
    vn[3] = 2.f * (x * (G(0, 2) + G(2, 0)) + y * (G(1, 2) + G(2, 1)) -
                   2.f * z * (G(0, 0) + G(1, 1)) + w * (G(0, 1) - G(1, 0)));
#undef G
    const float qn[4] = {w, x, y, z};
    const float dot = vn[0] * qn[0] + vn[1] * qn[1] + vn[2] * qn[2] + vn[3] * qn[3];
#pragma unroll
    for (int k = 0; k < 4; ++k) vq[k] += (vn[k] - dot * qn[k]) * inv;
}

// ---------------------------------------------------------------- conditioning
// cond_mean_convariance_opacity_fwd.cu:107-290 / _bwd.cu:102-563 for K = D - 3
// conditional dimensions (1 <= K <= 8).
__device__ __forceinline__ float nz20(float d) { return d == 0.f ? 1e-20f : d; }

template <int K> __device__ __forceinline__ void inv_small(const float *A, float *out) {
    if (K == 3) {
        const float *a = A;
        const float c00 = a[4] * a[8] - a[5] * a[7];
        const float c01 = -(a[3] * a[8] - a[5] * a[6]);
        const float c02 = a[3] * a[7] - a[4] * a[6];
        const float c10 = -(a[1] * a[8] - a[2] * a[7]);
        const float c11 = a[0] * a[8] - a[2] * a[6];
        const float c12 = -(a[0] * a[7] - a[1] * a[6]);
        const float c20 = a[1] * a[5] - a[2] * a[4];
        const float c21 = -(a[0] * a[5] - a[2] * a[3]);
        const float c22 = a[0] * a[4] - a[1] * a[3];
        float det = a[0] * c00 + a[1] * c01 + a[2] * c02;
        if (det == 0.f) det = 1e-20f;
        const float id = 1.f / det;
        out[0] = c00 * id; out[1] = c10 * id; out[2] = c20 * id;
        out[3] = c01 * id; out[4] = c11 * id; out[5] = c21 * id;
        out[6] = c02 * id; out[7] = c12 * id; out[8] = c22 * id;
        return;
    }
    float aug[K][2 * K];
#pragma unroll
    for (int r = 0; r < K; ++r)
#pragma unroll
        for (int c = 0; c < 2 * K; ++c)
            aug[r][c] = (c < K) ? A[r * K + c] : ((c - K == r) ? 1.f : 0.f);
#pragma unroll
    for (int col = 0; col < K; ++col) {
        int piv = col;
        float best = fabsf(aug[col][col]);
#pragma unroll
        for (int r = col + 1; r < K; ++r)
            if (fabsf(aug[r][col]) > best) {
                best = fabsf(aug[r][col]);
                piv = r;
            }
        if (piv != col) {
#pragma unroll
            for (int c = 0; c < 2 * K; ++c) {
                // swap rows col and piv without dynamic register indexing on col
                float tmp = aug[col][c];
#pragma unroll
                for (int r = col + 1; r < K; ++r)
                    if (r == piv) {
                        aug[col][c] = aug[r][c];
                        aug[r][c] = tmp;
                    }
            }
        }
        float d = aug[col][col];
        if (d == 0.f) d = 1e-20f;
        const float id = 1.f / d;
#pragma unroll
        for (int c = 0; c < 2 * K; ++c) aug[col][c] *= id;
#pragma unroll
        for (int r = 0; r < K; ++r) {
            if (r == col) continue;
            const float f = aug[r][col];
            if (f != 0.f) {
#pragma unroll
                for (int c = 0; c < 2 * K; ++c) aug[r][c] -= f * aug[col][c];
            }
        }
    }
#pragma unroll
    for (int r = 0; r < K; ++r)
#pragma unroll
        for (int c = 0; c < K; ++c) out[r * K + c] = aug[r][K + c];
}

template <int K> struct CondState {
    float x[K], beta[K], ba[K], i22[K * K], r[3 * K], rb[3 * K], v12[3 * K], v21[3 * K],
        Lc[K * K], y[K];
};

// m: [D] means, V: [D*D] row-major covariance (D = K + 3)
template <int K>
__device__ __forceinline__ void cond_prepare(const float *m, const float *V, const float *b,
                                             const float *q, CondState<K> &s) {
    constexpr int D = K + 3;
    float v22[K * K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        s.x[j] = q[j] - m[3 + j];
        s.beta[j] = b[j];
        const float t = b[j] * 0.25f;
        s.ba[j] = (t < 1.f) ? t : 1.f;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < K; ++c) s.v12[r * K + c] = V[r * D + 3 + c];
#pragma unroll
    for (int r = 0; r < K; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) s.v21[r * 3 + c] = V[(3 + r) * D + c];
#pragma unroll
    for (int r = 0; r < K; ++r)
#pragma unroll
        for (int c = 0; c < K; ++c) v22[r * K + c] = V[(3 + r) * D + 3 + c];
    inv_small<K>(v22, s.i22);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < K; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) acc += s.v12[r * K + k] * s.i22[k * K + c];
            s.r[r * K + c] = acc;
            s.rb[r * K + c] = acc * s.ba[c];
        }
    // Cholesky of v22 (lower triangle read), guarded like the reference
#pragma unroll
    for (int i = 0; i < K * K; ++i) s.Lc[i] = 0.f;
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            float sum = v22[i * K + j];
#pragma unroll
            for (int k = 0; k < j; ++k) sum -= s.Lc[i * K + k] * s.Lc[j * K + k];
            if (i == j) {
                float sv = sum;
                if (sv <= 0.f) sv = 1e-20f;
                s.Lc[i * K + j] = sqrtf(sv);
            } else {
                s.Lc[i * K + j] = sum / nz20(s.Lc[j * K + j]);
            }
        }
#pragma unroll
    for (int i = 0; i < K; ++i) {
        float sum = s.x[i];
#pragma unroll
        for (int k = 0; k < i; ++k) sum -= s.Lc[i * K + k] * s.y[k];
        s.y[i] = sum / nz20(s.Lc[i * K + i]);
    }
}

template <int K>
__device__ __forceinline__ void cond_forward(const float *m, const float *V, float o,
                                             const float *b, const float *q, float *om, float *oV,
                                             float *oo) {
    constexpr int D = K + 3;
    CondState<K> s;
    cond_prepare<K>(m, V, b, q, s);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float acc = 0.f;
#pragma unroll
        for (int c = 0; c < K; ++c) acc += s.rb[r * K + c] * s.x[c];
        om[r] = m[r] + acc;
#pragma unroll
        for (int c2 = 0; c2 < 3; ++c2) {
            float a2 = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) a2 += s.rb[r * K + k] * s.v21[k * 3 + c2];
            oV[r * 3 + c2] = V[r * D + c2] - a2;
        }
    }
    float oc = 1.f;
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const float d = clamp01_eps(tanhf(s.y[j] * s.y[j]));
        oc *= powf(1.f - d, s.beta[j]);
    }
    *oo = o * oc;
}

// VJP; gm [D], gV [D*D] (row-major), go, gb [K] are overwritten.
template <int K>
__device__ __forceinline__ void cond_backward(const float *m, const float *V, float o,
                                              const float *b, const float *q, const float *gM,
                                              const float *gVc, float gO, bool exact, float *gm,
                                              float *gV, float *go, float *gb) {
    constexpr int D = K + 3;
    const float upper = 1.0f - 1.1920928955078125e-07f;
    CondState<K> s;
    cond_prepare<K>(m, V, b, q, s);
#pragma unroll
    for (int k = 0; k < D; ++k) gm[k] = 0.f;
#pragma unroll
    for (int k = 0; k < D * D; ++k) gV[k] = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) gb[k] = 0.f;
#pragma unroll
    for (int r = 0; r < 3; ++r) gm[r] = gM[r];
    float Gr[3 * K], gx[K];
#pragma unroll
    for (int c = 0; c < K; ++c) {
        gx[c] = 0.f;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            Gr[r * K + c] = gM[r] * s.x[c] -
                            (gVc[r * 3 + 0] * s.v21[c * 3 + 0] + gVc[r * 3 + 1] * s.v21[c * 3 + 1] +
                             gVc[r * 3 + 2] * s.v21[c * 3 + 2]);
        }
        gx[c] += s.rb[0 * K + c] * gM[0] + s.rb[1 * K + c] * gM[1] + s.rb[2 * K + c] * gM[2];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) gV[r * D + c] += gVc[r * 3 + c];
#pragma unroll
    for (int rr = 0; rr < K; ++rr)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            gV[(3 + rr) * D + c] += -(s.rb[0 * K + rr] * gVc[0 * 3 + c] +
                                      s.rb[1 * K + rr] * gVc[1 * 3 + c] +
                                      s.rb[2 * K + rr] * gVc[2 * 3 + c]);
    float dba[K], G_r[3 * K];
#pragma unroll
    for (int c = 0; c < K; ++c) {
        dba[c] = Gr[0 * K + c] * s.r[0 * K + c] + Gr[1 * K + c] * s.r[1 * K + c] +
                 Gr[2 * K + c] * s.r[2 * K + c];
#pragma unroll
        for (int r = 0; r < 3; ++r) G_r[r * K + c] = Gr[r * K + c] * s.ba[c];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < K; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) acc += G_r[r * K + k] * s.i22[c * K + k];
            gV[r * D + 3 + c] += acc;
        }
    float Gi22[K * K];
#pragma unroll
    for (int rr = 0; rr < K; ++rr)
#pragma unroll
        for (int c = 0; c < K; ++c)
            Gi22[rr * K + c] = s.v12[0 * K + rr] * G_r[0 * K + c] +
                               s.v12[1 * K + rr] * G_r[1 * K + c] +
                               s.v12[2 * K + rr] * G_r[2 * K + c];
    // opacity path
    float dv[K], base[K], oc = 1.f;
#pragma unroll
    for (int j = 0; j < K; ++j) {
        float d = tanhf(s.y[j] * s.y[j]);
        if (d < 0.f) d = 0.f;
        if (d > upper) d = upper;
        dv[j] = d;
        base[j] = 1.f - d;
        oc *= powf(base[j], s.beta[j]);
    }
    *go = gO * oc;
    const float goc = gO * o;
    float gy[K], a[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        float gd = 0.f;
        if (base[j] > 0.f) {
            gb[j] += goc * oc * logf(base[j]);
            if (dv[j] > 0.f && dv[j] < upper) gd += goc * (-oc * s.beta[j] / base[j]);
        }
        gy[j] = gd * (2.f * s.y[j] * (1.f - dv[j] * dv[j]));
    }
#pragma unroll
    for (int ii = K - 1; ii >= 0; --ii) {
        float sum = gy[ii];
#pragma unroll
        for (int k = ii + 1; k < K; ++k) sum -= s.Lc[k * K + ii] * a[k];
        a[ii] = sum / nz20(s.Lc[ii * K + ii]);
    }
#pragma unroll
    for (int j = 0; j < K; ++j) gx[j] += a[j];
    float S[K * K], U[K * K], Gm[K * K];
#pragma unroll
    for (int r = 0; r < K; ++r)
#pragma unroll
        for (int c = 0; c < K; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float gl = (c <= k) ? -(a[k] * s.y[c]) : 0.f; // gL = -a y^T, lower
                acc += s.Lc[k * K + r] * gl;
            }
            S[r * K + c] = (c > r) ? 0.f : acc;
        }
#pragma unroll
    for (int r = 0; r < K; ++r) S[r * K + r] *= 0.5f;
#pragma unroll
    for (int col = 0; col < K; ++col)
#pragma unroll
        for (int ii = K - 1; ii >= 0; --ii) {
            float sum = S[ii * K + col];
#pragma unroll
            for (int k = ii + 1; k < K; ++k) sum -= s.Lc[k * K + ii] * U[k * K + col];
            U[ii * K + col] = sum / nz20(s.Lc[ii * K + ii]);
        }
    if (!exact) {
#pragma unroll
        for (int col = 0; col < K; ++col)
#pragma unroll
            for (int ii = 0; ii < K; ++ii) {
                float sum = U[col * K + ii];
#pragma unroll
                for (int k = 0; k < ii; ++k) sum -= s.Lc[ii * K + k] * Gm[k * K + col];
                Gm[ii * K + col] = sum / nz20(s.Lc[ii * K + ii]);
            }
    } else {
#pragma unroll
        for (int r = 0; r < K; ++r)
#pragma unroll
            for (int ii = K - 1; ii >= 0; --ii) {
                float sum = U[r * K + ii];
#pragma unroll
                for (int k = ii + 1; k < K; ++k) sum -= s.Lc[k * K + ii] * Gm[r * K + k];
                Gm[r * K + ii] = sum / nz20(s.Lc[ii * K + ii]);
            }
    }
#pragma unroll
    for (int r = 0; r < K; ++r)
#pragma unroll
        for (int c = 0; c < K; ++c)
            gV[(3 + r) * D + 3 + c] += 0.5f * (Gm[r * K + c] + Gm[c * K + r]);
#pragma unroll
    for (int j = 0; j < K; ++j) gm[3 + j] += -gx[j];
#pragma unroll
    for (int j = 0; j < K; ++j) gb[j] += dba[j] * ((s.beta[j] < 4.f) ? 0.25f : 0.f);
    float tmp[K * K];
#pragma unroll
    for (int r = 0; r < K; ++r)
#pragma unroll
        for (int c = 0; c < K; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) acc += Gi22[r * K + k] * s.i22[c * K + k];
            tmp[r * K + c] = acc;
        }
#pragma unroll
    for (int r = 0; r < K; ++r)
#pragma unroll
        for (int c = 0; c < K; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) acc += s.i22[k * K + r] * tmp[k * K + c];
            gV[(3 + r) * D + 3 + c] += -acc;
        }
}

// ------------------------------------------------------ D x D covariance
// V = L L^T (V: [D*D] row-major, both triangles) with the summation shapes of
// rot_scale_l_triangle_to_covar_fwd.cu:37-183, so that the covariance -- and
// with it the conditioned mean and the projected depth that keys the sort --
// rounds identically: each spatial 3x3 entry is one three-term expression
// (the way it is written decides which product the compiler fuses into an
// FMA); a diagonal entry of rows >= 3 starts from the rounded squared scale
// and adds the row's lower-triangle squares by FMA; every other entry
// accumulates over k in ascending order (L's zeros add nothing).
template <int D> __device__ __forceinline__ void covar_from_L(const float *L, float *V) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c) {
            const float v = L[r * D] * L[c * D] + L[r * D + 1] * L[c * D + 1] +
                            L[r * D + 2] * L[c * D + 2];
            V[r * D + c] = v;
            V[c * D + r] = v;
        }
#pragma unroll
    for (int r = 3; r < D; ++r) {
#pragma unroll
        for (int c = 0; c < r; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) acc += L[r * D + k] * L[c * D + k];
            V[r * D + c] = acc;
            V[c * D + r] = acc;
        }
        // the reference adds each square to a running sum that starts from
        // the rounded s_r^2 (its loop fuses the added product, never s_r^2):
        // an explicitly rounded first product keeps the compiler from
        // fusing it into the first addition instead
        float sq = __fmul_rn(L[r * D + r], L[r * D + r]);
#pragma unroll
        for (int k = 0; k < r; ++k) sq += L[r * D + k] * L[r * D + k];
        V[r * D + r] = sq;
    }
}

// L: [D*D] row-major factor of rot_scale_l_triangle_to_covar_fwd.cu:8-188
template <int D>
__device__ __forceinline__ void build_L(const float *R, const float *s, const float *lrest,
                                        const int32_t *ri, const int32_t *rj, int m_rest,
                                        float *L) {
#pragma unroll
    for (int k = 0; k < D * D; ++k) L[k] = 0.f;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) L[r * D + c] = R[r * 3 + c] * s[c];
#pragma unroll
    for (int r = 3; r < D; ++r) L[r * D + r] = s[r];
    for (int m = 0; m < m_rest; ++m) {
        const int r = ri[m], c = rj[m];
        // scatter through a compile-time loop to keep L in registers
#pragma unroll
        for (int k = 3 * D; k < D * D; ++k)
            if (k == r * D + c) L[k] = lrest[m];
    }
}

} // namespace ubs
