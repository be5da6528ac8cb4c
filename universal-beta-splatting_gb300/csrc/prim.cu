// prim.cu -- per-primitive operators of the reference path as C-ABI kernels:
// rotation (a2), D x D covariance (a3), conditioning (a4) and EWA projection
// (a6), forward and backward.  One thread per primitive (per camera and
// primitive for the projection); the math lives in prim_math.cuh.
#include "prim_math.cuh"

namespace ubs {

// ------------------------------------------------------------------ a2
__global__ void rotmat_fwd_kernel(int64_t n, const float *__restrict__ l, int64_t stride,
                                  float *__restrict__ R) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a0 = l[i * stride], a1 = l[i * stride + 1], a2 = l[i * stride + 2];
    float *o = R + i * 9;
    o[0] = 1.f; o[1] = a0; o[2] = a1;
    o[3] = -a0; o[4] = 1.f; o[5] = a2;
    o[6] = -a1; o[7] = -a2; o[8] = 1.f;
}
__global__ void rotmat_bwd_kernel(int64_t n, const float *__restrict__ g, float *__restrict__ vl) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *r = g + i * 9;
    vl[i * 3 + 0] = r[1] - r[3];
    vl[i * 3 + 1] = r[2] - r[6];
    vl[i * 3 + 2] = r[5] - r[7];
}

// ------------------------------------------------- coalesced output rows
// The per-primitive outputs are [n, w] rows, one per thread; stored directly,
// every warp store would touch 32 different sectors.  Kernels with rows of
// up to 49 floats stage a block's rows in shared memory (rows padded to an odd
// stride, so a thread's own writes are free of bank conflicts) and copy them
// out with consecutive threads on consecutive floats.
constexpr int ROW_BLOCK = 128;
template <int W> struct RowBuf {
    static constexpr int S = W | 1;
    float v[ROW_BLOCK * S];
    __device__ __forceinline__ float &at(int t, int k) { return v[t * S + k]; }
    // after a barrier: rows [0, cnt) to dst rows [i0, i0 + cnt)
    __device__ __forceinline__ void flush(float *__restrict__ dst, int64_t i0, int cnt) const {
        float *d = dst + i0 * W;
        for (int e = threadIdx.x; e < cnt * W; e += blockDim.x) {
            const int t = e / W;
            d[e] = v[t * S + (e - t * W)];
        }
    }
};

// ------------------------------------------------------------------ a3
template <int D>
__global__ void __launch_bounds__(ROW_BLOCK) covar_fwd_kernel(int64_t n, const float *__restrict__ rot,
                                 const float *__restrict__ scale, const float *__restrict__ ltri,
                                 const int32_t *__restrict__ ri_g, const int32_t *__restrict__ rj_g,
                                 int m_rest, int spatial, float *__restrict__ covar) {
    __shared__ int32_t ri[64], rj[64];
    for (int m = threadIdx.x; m < m_rest && m < 64; m += blockDim.x) {
        ri[m] = ri_g[m];
        rj[m] = rj_g[m];
    }
    constexpr bool STAGE = D <= 7;
    __shared__ RowBuf<STAGE ? D * D : 1> full;
    __shared__ RowBuf<STAGE ? 9 : 1> block3;
    __syncthreads();
    const int t = threadIdx.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x, i = i0 + t;
    const int cnt = (int)(n - i0 < (int64_t)blockDim.x ? n - i0 : (int64_t)blockDim.x);
    const bool sp = spatial || D == 3;
    if (i < n) {
        constexpr int full_m = D * (D - 1) / 2;
        float L[D * D];
        build_L<D>(rot + i * 9, scale + i * D, ltri + i * full_m + 3, ri, rj, m_rest, L);
        if (sp) {
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float v = L[r * D] * L[c * D] + L[r * D + 1] * L[c * D + 1] +
                                    L[r * D + 2] * L[c * D + 2];
                    if (STAGE) block3.at(t, r * 3 + c) = v;
                    else covar[i * 9 + r * 3 + c] = v;
                }
        } else {
            float V[D * D];
            covar_from_L<D>(L, V);
#pragma unroll
            for (int k = 0; k < D * D; ++k) {
                if (STAGE) full.at(t, k) = V[k];
                else covar[i * D * D + k] = V[k];
            }
        }
    }
    if (!STAGE) return;
    __syncthreads();
    if (sp) block3.flush(covar, i0, cnt);
    else full.flush(covar, i0, cnt);
}

// One primitive of covar_bwd_kernel: rows go to the shared row buffers when
// given (strides 9|1, D|1, full_m|1), else straight to global memory.
template <int D>
__device__ __forceinline__ void covar_bwd_row(int64_t i, int t, const float *__restrict__ rot,
                                              const float *__restrict__ scale,
                                              const float *__restrict__ ltri, const int32_t *ri,
                                              const int32_t *rj, int m_rest, int spatial,
                                              const float *__restrict__ v_covar,
                                              float *__restrict__ v_rot,
                                              float *__restrict__ v_scale,
                                              float *__restrict__ v_ltri, float *stR, float *stS,
                                              float *stL) {
    constexpr int full_m = D * (D - 1) / 2;
    const int dim = (spatial || D == 3) ? 3 : D;
    const float *R = rot + i * 9;
    const float *s = scale + i * D;
    float L[D * D];
    build_L<D>(R, s, ltri + i * full_m + 3, ri, rj, m_rest, L);
    const float *G = v_covar + i * dim * dim;
    float *gR = stR ? stR + t * (9 | 1) : v_rot + i * 9;
    float *gs = stS ? stS + t * (D | 1) : v_scale + i * D;
    float *gl = stL ? stL + t * (full_m | 1) : v_ltri + i * full_m;
    // dL = (G + G^T) L over the output rows
    float dL[D * D];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int c = 0; c < D; ++c) {
            float acc = 0.f;
            if (r < dim) {
#pragma unroll
                for (int k = 0; k < D; ++k)
                    if (k < dim) acc += (G[r * dim + k] + G[k * dim + r]) * L[k * D + c];
            }
            dL[r * D + c] = acc;
        }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) gR[r * 3 + c] = dL[r * D + c] * s[c];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        gs[c] = dL[0 * D + c] * R[0 * 3 + c] + dL[1 * D + c] * R[1 * 3 + c] + dL[2 * D + c] * R[2 * 3 + c];
#pragma unroll
    for (int k = 0; k < full_m; ++k) gl[k] = 0.f;
#pragma unroll
    for (int r = 3; r < D; ++r) gs[r] = (dim == 3) ? 0.f : dL[r * D + r];
    if (dim == 3) return;
    for (int m = 0; m < m_rest; ++m) {
        const int idx = ri[m] * D + rj[m];
        float v = 0.f;
#pragma unroll
        for (int k = 3 * D; k < D * D; ++k)
            if (k == idx) v = dL[k];
        gl[3 + m] = v;
    }
}

template <int D>
__global__ void __launch_bounds__(ROW_BLOCK) covar_bwd_kernel(int64_t n, const float *__restrict__ rot,
                                 const float *__restrict__ scale, const float *__restrict__ ltri,
                                 const int32_t *__restrict__ ri_g, const int32_t *__restrict__ rj_g,
                                 int m_rest, int spatial, const float *__restrict__ v_covar,
                                 float *__restrict__ v_rot, float *__restrict__ v_scale,
                                 float *__restrict__ v_ltri) {
    __shared__ int32_t ri[64], rj[64];
    for (int m = threadIdx.x; m < m_rest && m < 64; m += blockDim.x) {
        ri[m] = ri_g[m];
        rj[m] = rj_g[m];
    }
    constexpr int full_m = D * (D - 1) / 2;
    constexpr bool STAGE = D <= 7;
    __shared__ RowBuf<STAGE ? 9 : 1> sR;
    __shared__ RowBuf<STAGE ? D : 1> sS;
    __shared__ RowBuf<STAGE ? full_m : 1> sL;
    __syncthreads();
    const int t = threadIdx.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x, i = i0 + t;
    const int cnt = (int)(n - i0 < (int64_t)blockDim.x ? n - i0 : (int64_t)blockDim.x);
    if (i < n)
        covar_bwd_row<D>(i, t, rot, scale, ltri, ri, rj, m_rest, spatial, v_covar, v_rot, v_scale,
                         v_ltri, STAGE ? sR.v : nullptr, STAGE ? sS.v : nullptr,
                         STAGE ? sL.v : nullptr);
    if (!STAGE) return;
    __syncthreads();
    sR.flush(v_rot, i0, cnt);
    sS.flush(v_scale, i0, cnt);
    sL.flush(v_ltri, i0, cnt);
}

// ------------------------------------------------------------------ a4
template <int K>
__global__ void cond_fwd_kernel(int64_t n, const float *__restrict__ means,
                                const float *__restrict__ covars, const float *__restrict__ opac,
                                const float *__restrict__ betas, const float *__restrict__ query,
                                float *__restrict__ om, float *__restrict__ oV,
                                float *__restrict__ oo) {
    constexpr int D = K + 3;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float m[D], V[D * D], b[K], q[K];
#pragma unroll
    for (int k = 0; k < D; ++k) m[k] = means[i * D + k];
#pragma unroll
    for (int k = 0; k < D * D; ++k) V[k] = covars[i * D * D + k];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        b[k] = betas[i * K + k];
        q[k] = query[i * K + k];
    }
    cond_forward<K>(m, V, opac[i], b, q, om + i * 3, oV + i * 9, oo + i);
}

// One primitive of cond_bwd_kernel: the [D, D] and [D] gradient rows go to the
// shared row buffers when given (strides (D*D)|1 and D|1), else to global memory.
template <int K>
__device__ __forceinline__ void cond_bwd_row(int64_t i, int t, const float *__restrict__ means,
                                             const float *__restrict__ covars,
                                             const float *__restrict__ opac,
                                             const float *__restrict__ betas,
                                             const float *__restrict__ query,
                                             const float *__restrict__ vm,
                                             const float *__restrict__ vV,
                                             const float *__restrict__ vo,
                                             float *__restrict__ gm, float *__restrict__ gV,
                                             float *__restrict__ go, float *__restrict__ gb,
                                             int exact, float *stV, float *stM) {
    constexpr int D = K + 3;
    float m[D], V[D * D], b[K], q[K], gM[3], gVc[9];
#pragma unroll
    for (int k = 0; k < D; ++k) m[k] = means[i * D + k];
#pragma unroll
    for (int k = 0; k < D * D; ++k) V[k] = covars[i * D * D + k];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        b[k] = betas[i * K + k];
        q[k] = query[i * K + k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) gM[k] = vm[i * 3 + k];
#pragma unroll
    for (int k = 0; k < 9; ++k) gVc[k] = vV[i * 9 + k];
    float lm[D], lV[D * D], lb[K], lo;
    cond_backward<K>(m, V, opac[i], b, q, gM, gVc, vo[i], exact != 0, lm, lV, &lo, lb);
    float *dm = stM ? stM + t * (D | 1) : gm + i * D;
    float *dV = stV ? stV + t * ((D * D) | 1) : gV + i * D * D;
#pragma unroll
    for (int k = 0; k < D; ++k) dm[k] = lm[k];
#pragma unroll
    for (int k = 0; k < D * D; ++k) dV[k] = lV[k];
    go[i] = lo;
#pragma unroll
    for (int k = 0; k < K; ++k) gb[i * K + k] = lb[k];
}


template <int K>
__global__ void __launch_bounds__(ROW_BLOCK) cond_bwd_kernel(
    int64_t n, const float *__restrict__ means, const float *__restrict__ covars,
    const float *__restrict__ opac, const float *__restrict__ betas,
    const float *__restrict__ query, const float *__restrict__ vm, const float *__restrict__ vV,
    const float *__restrict__ vo, float *__restrict__ gm, float *__restrict__ gV,
    float *__restrict__ go, float *__restrict__ gb, int exact) {
    constexpr int D = K + 3;
    constexpr bool STAGE = D <= 7;
    __shared__ RowBuf<STAGE ? D * D : 1> sV;
    __shared__ RowBuf<STAGE ? D : 1> sM;
    const int t = threadIdx.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x, i = i0 + t;
    const int cnt = (int)(n - i0 < (int64_t)blockDim.x ? n - i0 : (int64_t)blockDim.x);
    if (i < n) cond_bwd_row<K>(i, t, means, covars, opac, betas, query, vm, vV, vo, gm, gV, go, gb,
                               exact, STAGE ? sV.v : nullptr, STAGE ? sM.v : nullptr);
    if (!STAGE) return;
    __syncthreads();
    sV.flush(gV, i0, cnt);
    sM.flush(gm, i0, cnt);
}

// ------------------------------------------------------------------ a6
struct ProjArgs {
    int C;
    int64_t N;
    const float *means, *covars, *quats, *scales, *viewmats, *Ks;
    int layout; // 6 or 9
    uint32_t W, H;
    float eps2d, near_p, far_p, radius_clip;
    int32_t *radii;
    float *means2d, *depths, *conics, *comps;
    // backward
    const int32_t *radii_in;
    const float *conics_in, *comps_in, *v_m2, *v_d, *v_cn, *v_cp;
    float *v_means, *v_covars, *v_quats, *v_scales, *v_view;
};

__device__ __forceinline__ M3 load_world_covar(const ProjArgs &a, int64_t g) {
    M3 S;
    if (a.covars) {
        if (a.layout == 6) {
            const float *c = a.covars + g * 6;
            S(0, 0) = c[0]; S(0, 1) = c[1]; S(0, 2) = c[2];
            S(1, 0) = c[1]; S(1, 1) = c[3]; S(1, 2) = c[4];
            S(2, 0) = c[2]; S(2, 1) = c[4]; S(2, 2) = c[5];
        } else {
            // the reference first packs the upper triangle: (0,0) (0,1) (0,2) (1,1) (1,2) (2,2)
            const float *c = a.covars + g * 9;
            S(0, 0) = c[0]; S(0, 1) = c[1]; S(0, 2) = c[2];
            S(1, 0) = c[1]; S(1, 1) = c[4]; S(1, 2) = c[5];
            S(2, 0) = c[2]; S(2, 1) = c[5]; S(2, 2) = c[8];
        }
    } else {
        const M3 R = quat_to_R(a.quats + g * 4);
        const float *s = a.scales + g * 3;
        M3 Sd;
#pragma unroll
        for (int k = 0; k < 9; ++k) Sd.m[k] = 0.f;
        Sd(0, 0) = s[0];
        Sd(1, 1) = s[1];
        Sd(2, 2) = s[2];
        const M3 M = mm(R, Sd);
        S = mm(M, tr(M));
    }
    return S;
}

__global__ void projection_fwd_kernel(ProjArgs a) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)a.C * a.N) return;
    const int cid = (int)(idx / a.N);
    const int64_t g = idx - (int64_t)cid * a.N;
    const Cam cam = load_cam(a.viewmats + cid * 16, a.Ks + cid * 9);
    float pc[3];
    world_to_cam(cam, a.means + g * 3, pc);
    a.radii[idx] = 0;
    a.means2d[idx * 2] = 0.f;
    a.means2d[idx * 2 + 1] = 0.f;
    a.depths[idx] = 0.f;
    a.conics[idx * 3] = 0.f;
    a.conics[idx * 3 + 1] = 0.f;
    a.conics[idx * 3 + 2] = 0.f;
    if (a.comps) a.comps[idx] = 0.f;
    if (pc[2] < a.near_p || pc[2] > a.far_p) return;
    const M3 Sw = load_world_covar(a, g);
    const M3 Sc = mm(mm(cam.R, Sw), tr(cam.R));
    const Proj2D p = project_2d(pc, Sc, cam, a.W, a.H, a.eps2d, a.radius_clip);
    if (p.radius <= 0) return;
    a.radii[idx] = p.radius;
    a.means2d[idx * 2] = p.mx;
    a.means2d[idx * 2 + 1] = p.my;
    a.depths[idx] = p.depth;
    a.conics[idx * 3] = p.conic[0];
    a.conics[idx * 3 + 1] = p.conic[1];
    a.conics[idx * 3 + 2] = p.conic[2];
    if (a.comps) a.comps[idx] = p.comp;
}

__device__ __forceinline__ void add_out(float *p, float v, bool direct) {
    if (direct) *p = v;
    else atomicAdd(p, v);
}

__global__ void projection_bwd_kernel(ProjArgs a) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in_range = idx < (int64_t)a.C * a.N;
    const bool direct = a.C == 1; // one camera: plain stores (outputs pre-zeroed otherwise)
    int cid = 0;
    int64_t g = 0;
    bool active = false;
    float vR[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) vR[k] = 0.f;
    if (in_range) {
        cid = (int)(idx / a.N);
        g = idx - (int64_t)cid * a.N;
        active = a.radii_in[idx] > 0;
    }
    if (in_range && !active && direct) {
        // culled: zero gradient (written explicitly for the single-camera case)
#pragma unroll
        for (int k = 0; k < 3; ++k) a.v_means[g * 3 + k] = 0.f;
        if (a.covars) {
            const int nc = a.layout;
#pragma unroll
            for (int k = 0; k < 9; ++k)
                if (k < nc) a.v_covars[g * nc + k] = 0.f;
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) a.v_quats[g * 4 + k] = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k) a.v_scales[g * 3 + k] = 0.f;
        }
    }
    if (active) {
        const Cam cam = load_cam(a.viewmats + cid * 16, a.Ks + cid * 9);
        float vc2[4];
        conic_vjp(a.conics_in + idx * 3, a.v_cn + idx * 3, a.eps2d, a.v_cp != nullptr,
                  a.v_cp ? a.comps_in[idx] : 0.f, a.v_cp ? a.v_cp[idx] : 0.f, vc2);
        const float *p = a.means + g * 3;
        float pc[3];
        world_to_cam(cam, p, pc);
        const M3 Sw = load_world_covar(a, g);
        const M3 Sc = mm(mm(cam.R, Sw), tr(cam.R));
        M3 vSc;
#pragma unroll
        for (int k = 0; k < 9; ++k) vSc.m[k] = 0.f;
        float vpc[3] = {0.f, 0.f, 0.f};
        persp_vjp(pc, Sc, cam, a.W, a.H, vc2, a.v_m2[idx * 2], a.v_m2[idx * 2 + 1], vSc, vpc);
        if (a.v_d) vpc[2] += a.v_d[idx];
        // rigid transform
#pragma unroll
        for (int r = 0; r < 3; ++r) {
#pragma unroll
            for (int k = 0; k < 3; ++k) vR[r * 4 + k] += vpc[r] * p[k];
            vR[r * 4 + 3] += vpc[r];
        }
        float vp[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
            vp[k] = cam.R(0, k) * vpc[0] + cam.R(1, k) * vpc[1] + cam.R(2, k) * vpc[2];
        const M3 a1 = mm(mm(vSc, cam.R), tr(Sw));
        const M3 a2 = mm(mm(tr(vSc), cam.R), Sw);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int k = 0; k < 3; ++k) vR[r * 4 + k] += a1(r, k) + a2(r, k);
        const M3 vSw = mm(mm(tr(cam.R), vSc), cam.R);
#pragma unroll
        for (int k = 0; k < 3; ++k) add_out(&a.v_means[g * 3 + k], vp[k], direct);
        if (a.covars) {
            if (a.layout == 6) {
                float *vc = a.v_covars + g * 6;
                add_out(vc + 0, vSw(0, 0), direct);
                add_out(vc + 1, vSw(0, 1) + vSw(1, 0), direct);
                add_out(vc + 2, vSw(0, 2) + vSw(2, 0), direct);
                add_out(vc + 3, vSw(1, 1), direct);
                add_out(vc + 4, vSw(1, 2) + vSw(2, 1), direct);
                add_out(vc + 5, vSw(2, 2), direct);
            } else {
                // gradient through the upper-triangle gather: packed entry -> its slot
                float *vc = a.v_covars + g * 9;
                add_out(vc + 0, vSw(0, 0), direct);
                add_out(vc + 1, vSw(0, 1) + vSw(1, 0), direct);
                add_out(vc + 2, vSw(0, 2) + vSw(2, 0), direct);
                add_out(vc + 4, vSw(1, 1), direct);
                add_out(vc + 5, vSw(1, 2) + vSw(2, 1), direct);
                add_out(vc + 8, vSw(2, 2), direct);
                if (direct) {
                    vc[3] = 0.f;
                    vc[6] = 0.f;
                    vc[7] = 0.f;
                }
            }
        } else {
            const float *q = a.quats + g * 4;
            const float *s = a.scales + g * 3;
            const M3 R = quat_to_R(q);
            M3 M;
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int k = 0; k < 3; ++k) M(r, k) = R(r, k) * s[k];
            M3 sym;
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int k = 0; k < 3; ++k) sym(r, k) = vSw(r, k) + vSw(k, r);
            const M3 vM = mm(sym, M);
            M3 vRq;
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int k = 0; k < 3; ++k) vRq(r, k) = vM(r, k) * s[k];
            float vq[4] = {0.f, 0.f, 0.f, 0.f};
            quat_vjp(q, vRq, vq);
#pragma unroll
            for (int k = 0; k < 4; ++k) add_out(&a.v_quats[g * 4 + k], vq[k], direct);
#pragma unroll
            for (int k = 0; k < 3; ++k)
                add_out(&a.v_scales[g * 3 + k],
                        R(0, k) * vM(0, k) + R(1, k) * vM(1, k) + R(2, k) * vM(2, k), direct);
        }
    }
    if (a.v_view) {
        // sum the viewmat gradient over the warp when all lanes share a camera
        const unsigned full = 0xffffffffu;
        const int key = in_range ? cid : -1;
        const unsigned same = __match_any_sync(full, key);
        if (same == full) {
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                float v = vR[k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(full, v, o);
                vR[k] = v;
            }
            if ((threadIdx.x & 31) == 0 && in_range)
#pragma unroll
                for (int k = 0; k < 12; ++k)
                    if (vR[k] != 0.f) atomicAdd(&a.v_view[cid * 16 + k], vR[k]);
        } else if (active) {
#pragma unroll
            for (int k = 0; k < 12; ++k)
                if (vR[k] != 0.f) atomicAdd(&a.v_view[cid * 16 + k], vR[k]);
        }
    }
}

} // namespace ubs

using namespace ubs;

static inline int finish(const char *what) { return check_launch(what); }

extern "C" {

int ubs_l_triangle_to_rotmat_fwd(int64_t n, const float *l_triangle, int64_t row_stride,
                                 float *rotmats, void *stream) {
    UBS_REQUIRE(n >= 0 && row_stride >= 3, "rotmat_fwd: bad sizes");
    if (n == 0) return UBS_OK;
    UBS_TIMED("rotmat_fwd", (cudaStream_t)stream,
              rotmat_fwd_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                  n, l_triangle, row_stride, rotmats));
    ::ubs::note_launch();
    return finish("rotmat_fwd");
}

int ubs_l_triangle_to_rotmat_bwd(int64_t n, const float *v_rotmats, float *v_l_triangle,
                                 void *stream) {
    UBS_REQUIRE(n >= 0, "rotmat_bwd: bad sizes");
    if (n == 0) return UBS_OK;
    UBS_TIMED("rotmat_bwd", (cudaStream_t)stream,
              rotmat_bwd_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                  n, v_rotmats, v_l_triangle));
    ::ubs::note_launch();
    return finish("rotmat_bwd");
}

#define UBS_DIM_SWITCH(dim, ...)                                                          \
    switch (dim) {                                                                        \
    case 3: { constexpr int DD = 3; __VA_ARGS__; } break;                                 \
    case 4: { constexpr int DD = 4; __VA_ARGS__; } break;                                 \
    case 5: { constexpr int DD = 5; __VA_ARGS__; } break;                                 \
    case 6: { constexpr int DD = 6; __VA_ARGS__; } break;                                 \
    case 7: { constexpr int DD = 7; __VA_ARGS__; } break;                                 \
    case 8: { constexpr int DD = 8; __VA_ARGS__; } break;                                 \
    case 9: { constexpr int DD = 9; __VA_ARGS__; } break;                                 \
    case 10: { constexpr int DD = 10; __VA_ARGS__; } break;                               \
    case 11: { constexpr int DD = 11; __VA_ARGS__; } break;                               \
    default: return set_error(UBS_ERR_UNSUPPORTED, "dimension %d (supported 3..11)", dim); \
    }

int ubs_rot_scale_l_triangle_to_covar_fwd(int64_t n, int32_t dim, const float *rot,
                                          const float *scale, const float *l_triangle,
                                          const int32_t *rest_i, const int32_t *rest_j,
                                          int32_t m_rest, int32_t spatial_block, float *covar,
                                          void *stream) {
    UBS_REQUIRE(n >= 0 && m_rest >= 0 && m_rest <= 64, "covar_fwd: bad sizes");
    UBS_REQUIRE(m_rest <= dim * (dim - 1) / 2 - 3 || dim == 3, "covar_fwd: m_rest %d too large",
                m_rest);
    if (n == 0) return UBS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    UBS_TIMED("covar_fwd", st,
              UBS_DIM_SWITCH(dim, covar_fwd_kernel<DD><<<grid_for(n, 128), 128, 0, st>>>(
                                      n, rot, scale, l_triangle, rest_i, rest_j, m_rest,
                                      spatial_block, covar)));
    ::ubs::note_launch();
    return finish("covar_fwd");
}

int ubs_rot_scale_l_triangle_to_covar_bwd(int64_t n, int32_t dim, const float *rot,
                                          const float *scale, const float *l_triangle,
                                          const int32_t *rest_i, const int32_t *rest_j,
                                          int32_t m_rest, int32_t spatial_block,
                                          const float *v_covar, float *v_rot, float *v_scale,
                                          float *v_l_triangle, void *stream) {
    UBS_REQUIRE(n >= 0 && m_rest >= 0 && m_rest <= 64, "covar_bwd: bad sizes");
    if (n == 0) return UBS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    UBS_TIMED("covar_bwd", st,
              UBS_DIM_SWITCH(dim, covar_bwd_kernel<DD><<<grid_for(n, 128), 128, 0, st>>>(
                                      n, rot, scale, l_triangle, rest_i, rest_j, m_rest,
                                      spatial_block, v_covar, v_rot, v_scale, v_l_triangle)));
    ::ubs::note_launch();
    return finish("covar_bwd");
}

#define UBS_K_SWITCH(k, ...)                                                               \
    switch (k) {                                                                           \
    case 1: { constexpr int KK = 1; __VA_ARGS__; } break;                                  \
    case 2: { constexpr int KK = 2; __VA_ARGS__; } break;                                  \
    case 3: { constexpr int KK = 3; __VA_ARGS__; } break;                                  \
    case 4: { constexpr int KK = 4; __VA_ARGS__; } break;                                  \
    case 5: { constexpr int KK = 5; __VA_ARGS__; } break;                                  \
    case 6: { constexpr int KK = 6; __VA_ARGS__; } break;                                  \
    case 7: { constexpr int KK = 7; __VA_ARGS__; } break;                                  \
    case 8: { constexpr int KK = 8; __VA_ARGS__; } break;                                  \
    default: return set_error(UBS_ERR_UNSUPPORTED, "conditioning dims %d (supported 1..8)", k); \
    }

int ubs_cond_fwd(int64_t n, int32_t dim, const float *means, const float *covars,
                 const float *opacities, const float *betas, const float *query,
                 float *out_means, float *out_covars, float *out_opacities, void *stream) {
    UBS_REQUIRE(n >= 0 && dim >= 4, "cond_fwd: bad sizes (dim %d)", dim);
    if (n == 0) return UBS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    UBS_TIMED("cond_fwd", st,
              UBS_K_SWITCH(dim - 3, cond_fwd_kernel<KK><<<grid_for(n, 128), 128, 0, st>>>(
                                        n, means, covars, opacities, betas, query, out_means,
                                        out_covars, out_opacities)));
    ::ubs::note_launch();
    return finish("cond_fwd");
}

int ubs_cond_bwd(int64_t n, int32_t dim, const float *means, const float *covars,
                 const float *opacities, const float *betas, const float *query,
                 const float *v_out_means, const float *v_out_covars,
                 const float *v_out_opacities, float *v_means, float *v_covars,
                 float *v_opacities, float *v_betas, int32_t exact, void *stream) {
    UBS_REQUIRE(n >= 0 && dim >= 4, "cond_bwd: bad sizes (dim %d)", dim);
    if (n == 0) return UBS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    UBS_TIMED("cond_bwd", st,
              UBS_K_SWITCH(dim - 3, cond_bwd_kernel<KK><<<grid_for(n, 128), 128, 0, st>>>(
                                        n, means, covars, opacities, betas, query, v_out_means,
                                        v_out_covars, v_out_opacities, v_means, v_covars,
                                        v_opacities, v_betas, exact)));
    ::ubs::note_launch();
    return finish("cond_bwd");
}

static int proj_common(ProjArgs &a, int32_t C, int64_t N, const float *means,
                       const float *covars, int32_t layout, const float *quats,
                       const float *scales, const float *viewmats, const float *Ks, int32_t W,
                       int32_t H) {
    UBS_REQUIRE(C >= 1 && N >= 0 && W >= 0 && H >= 0, "projection: bad sizes");
    UBS_REQUIRE(N == 0 || (covars ? (layout == 6 || layout == 9) : (quats && scales)),
                "projection: need covars (layout 6 or 9) or quats + scales");
    a.C = C;
    a.N = N;
    a.means = means;
    a.covars = covars;
    a.layout = layout;
    a.quats = quats;
    a.scales = scales;
    a.viewmats = viewmats;
    a.Ks = Ks;
    a.W = (uint32_t)W;
    a.H = (uint32_t)H;
    return UBS_OK;
}

int ubs_projection_fwd(int32_t C, int64_t N, const float *means, const float *covars,
                       int32_t covar_layout, const float *quats, const float *scales,
                       const float *viewmats, const float *Ks, int32_t width, int32_t height,
                       float eps2d, float near_plane, float far_plane, float radius_clip,
                       int32_t *radii, float *means2d, float *depths, float *conics,
                       float *compensations, void *stream) {
    ProjArgs a{};
    if (int e = proj_common(a, C, N, means, covars, covar_layout, quats, scales, viewmats, Ks,
                            width, height))
        return e;
    a.eps2d = eps2d;
    a.near_p = near_plane;
    a.far_p = far_plane;
    a.radius_clip = radius_clip;
    a.radii = radii;
    a.means2d = means2d;
    a.depths = depths;
    a.conics = conics;
    a.comps = compensations;
    const int64_t CN = (int64_t)C * N;
    if (CN == 0) return UBS_OK;
    UBS_TIMED("projection_fwd", (cudaStream_t)stream,
              projection_fwd_kernel<<<grid_for(CN, 256), 256, 0, (cudaStream_t)stream>>>(a));
    ::ubs::note_launch();
    return finish("projection_fwd");
}

int ubs_projection_bwd(int32_t C, int64_t N, const float *means, const float *covars,
                       int32_t covar_layout, const float *quats, const float *scales,
                       const float *viewmats, const float *Ks, int32_t width, int32_t height,
                       float eps2d, const int32_t *radii, const float *conics,
                       const float *compensations, const float *v_means2d,
                       const float *v_depths, const float *v_conics,
                       const float *v_compensations, float *v_means, float *v_covars,
                       float *v_quats, float *v_scales, float *v_viewmats, void *stream) {
    ProjArgs a{};
    if (int e = proj_common(a, C, N, means, covars, covar_layout, quats, scales, viewmats, Ks,
                            width, height))
        return e;
    UBS_REQUIRE(!v_compensations || compensations,
                "projection_bwd: v_compensations needs compensations");
    a.eps2d = eps2d;
    a.radii_in = radii;
    a.conics_in = conics;
    a.comps_in = compensations;
    a.v_m2 = v_means2d;
    a.v_d = v_depths;
    a.v_cn = v_conics;
    a.v_cp = v_compensations;
    a.v_means = v_means;
    a.v_covars = v_covars;
    a.v_quats = v_quats;
    a.v_scales = v_scales;
    a.v_view = v_viewmats;
    cudaStream_t st = (cudaStream_t)stream;
    if (C > 1 || N == 0) {
        const int nc = covars ? covar_layout : 0;
        if (cudaMemsetAsync(v_means, 0, N * 3 * 4, st) ||
            (covars && cudaMemsetAsync(v_covars, 0, N * nc * 4, st)) ||
            (!covars && (cudaMemsetAsync(v_quats, 0, N * 16, st) ||
                         cudaMemsetAsync(v_scales, 0, N * 12, st))))
            return finish("projection_bwd memset");
    }
    if (v_viewmats && cudaMemsetAsync(v_viewmats, 0, (size_t)C * 64, st))
        return finish("projection_bwd memset");
    const int64_t CN = (int64_t)C * N;
    if (CN == 0) return UBS_OK;
    UBS_TIMED("projection_bwd", st, projection_bwd_kernel<<<grid_for(CN, 256), 256, 0, st>>>(a));
    ::ubs::note_launch();
    return finish("projection_bwd");
}

} // extern "C"
