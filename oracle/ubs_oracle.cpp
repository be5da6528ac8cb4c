// ubs_oracle.cpp -- CPU oracle for the Universal Beta Splatting rasteriser path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, on the CPU, the arithmetic of
// every function on the reference's rasteriser path so that the GB300 kernels
// can be checked against it.  Only the test-suite, the smoke check and the CPU
// baseline leg of bench.py load the library built from it; the product path in
// universal-beta-splatting_gb300/ never does (it fails loudly without its CUDA
// library instead).
//
// Every function is templated on the scalar type: float mirrors the reference's
// FP32 kernels for parity tests, double drives FP64 central finite-difference
// checks of the backward passes.  Citations are to files of the reference
// project (RongLiu-Leo/universal-beta-splatting).
//
// Build: see oracle/build_oracle.py (g++ -O2 -fopenmp -ffp-contract=off).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace ubs_oracle {

// ---------------------------------------------------------------- small math
template <typename T> struct M3 {
    T a[9]; // row-major
    T &operator()(int r, int c) { return a[r * 3 + c]; }
    T operator()(int r, int c) const { return a[r * 3 + c]; }
};
template <typename T> static M3<T> mul(const M3<T> &A, const M3<T> &B) {
    M3<T> C;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            T s = 0;
            for (int k = 0; k < 3; ++k) s += A(r, k) * B(k, c);
            C(r, c) = s;
        }
    return C;
}
template <typename T> static M3<T> tr(const M3<T> &A) {
    M3<T> B;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) B(r, c) = A(c, r);
    return B;
}
template <typename T> static M3<T> add(const M3<T> &A, const M3<T> &B) {
    M3<T> C;
    for (int i = 0; i < 9; ++i) C.a[i] = A.a[i] + B.a[i];
    return C;
}

// ------------------------------------------------------------- a2: rotation
// R = I + A(a01, a02, a12), the first-order rotation of
// submodules/gsplat/cuda/csrc/l_triagnle_to_rotmat_fwd.cu:8-36 (torch twin
// submodules/gsplat/cuda/_torch_impl.py:60-88).  l has row stride l_stride.
template <typename T>
void rotmat_fwd(int64_t n, const T *l, int64_t l_stride, T *R) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const T *p = l + i * l_stride;
        T *o = R + i * 9;
        o[0] = 1; o[1] = p[0]; o[2] = p[1];
        o[3] = -p[0]; o[4] = 1; o[5] = p[2];
        o[6] = -p[1]; o[7] = -p[2]; o[8] = 1;
    }
}
// VJP of the above: l_triagnle_to_rotmat_bwd.cu:8-25.
template <typename T> void rotmat_bwd(int64_t n, const T *vR, T *vl) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const T *g = vR + i * 9;
        vl[i * 3 + 0] = g[1] - g[3];
        vl[i * 3 + 1] = g[2] - g[6];
        vl[i * 3 + 2] = g[5] - g[7];
    }
}

// -------------------------------------------------------- a3: D x D covariance
// Builds the D x D factor L of rot_scale_l_triangle_to_covar_fwd.cu:8-188 /
// _torch_impl.py:94-129: top-left block R*diag(s[0:3]), L[r][r] = s[r] for r>=3,
// L[rest_i[m]][rest_j[m]] = l_tri[3+m].
template <typename T>
static void build_L(int D, const T *R, const T *s, const T *ltri,
                    const int32_t *ri, const int32_t *rj, int m_rest, T *L) {
    std::fill(L, L + D * D, T(0));
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) L[r * D + c] = R[r * 3 + c] * s[c];
    for (int r = 3; r < D; ++r) L[r * D + r] = s[r];
    for (int m = 0; m < m_rest; ++m) L[ri[m] * D + rj[m]] = ltri[3 + m];
}

// Sigma = L L^T (full D x D, or the 3 x 3 spatial block when spatial != 0).
template <typename T>
void covar_fwd(int64_t n, int D, const T *rot, const T *scale, const T *ltri,
               const int32_t *ri, const int32_t *rj, int m_rest, int spatial,
               T *covar) {
    const int dim = (spatial || D == 3) ? 3 : D;
    const int full_m = D * (D - 1) / 2;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        std::vector<T> L(D * D);
        build_L(D, rot + i * 9, scale + i * D, ltri + i * full_m, ri, rj, m_rest,
                L.data());
        T *o = covar + i * dim * dim;
        for (int r = 0; r < dim; ++r)
            for (int c = 0; c < dim; ++c) {
                T acc = 0;
                // In the spatial block only the 3 spatial columns of L exist.
                const int kmax = (dim == 3) ? 3 : D;
                for (int k = 0; k < kmax; ++k) acc += L[r * D + k] * L[c * D + k];
                o[r * dim + c] = acc;
            }
    }
}

// VJP of Sigma = L L^T: dL = (G + G^T) L read at the parameterised entries,
// as rot_scale_l_triangle_to_covar_bwd.cu:8-235 does; the first three l_tri
// entries (rotation parameters) receive no gradient from this op.
template <typename T>
void covar_bwd(int64_t n, int D, const T *rot, const T *scale, const T *ltri,
               const int32_t *ri, const int32_t *rj, int m_rest, int spatial,
               const T *v_covar, T *v_rot, T *v_scale, T *v_ltri) {
    const int dim = (spatial || D == 3) ? 3 : D;
    const int full_m = D * (D - 1) / 2;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const T *R = rot + i * 9;
        const T *s = scale + i * D;
        std::vector<T> L(D * D), S(dim * dim), dL(D * D, T(0));
        build_L(D, R, s, ltri + i * full_m, ri, rj, m_rest, L.data());
        const T *G = v_covar + i * dim * dim;
        for (int r = 0; r < dim; ++r)
            for (int c = 0; c < dim; ++c) S[r * dim + c] = G[r * dim + c] + G[c * dim + r];
        // dL = S * L restricted to the rows/cols of the op's output
        for (int r = 0; r < dim; ++r)
            for (int c = 0; c < D; ++c) {
                T acc = 0;
                for (int k = 0; k < dim; ++k) acc += S[r * dim + k] * L[k * D + c];
                dL[r * D + c] = acc;
            }
        T *gR = v_rot + i * 9;
        T *gs = v_scale + i * D;
        T *gl = v_ltri + i * full_m;
        for (int k = 0; k < full_m; ++k) gl[k] = 0;
        for (int k = 0; k < D; ++k) gs[k] = 0;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) gR[r * 3 + c] = dL[r * D + c] * s[c];
        for (int c = 0; c < 3; ++c) {
            T acc = 0;
            for (int r = 0; r < 3; ++r) acc += dL[r * D + c] * R[r * 3 + c];
            gs[c] = acc;
        }
        if (dim == 3) continue;
        for (int r = 3; r < D; ++r) gs[r] = dL[r * D + r];
        for (int m = 0; m < m_rest; ++m) gl[3 + m] = dL[ri[m] * D + rj[m]];
    }
}

// ------------------------------------------------------- a4: conditioning
// Explicit 3x3 inverse through the adjugate with the 1e-20 zero-determinant
// guard of cond_mean_convariance_opacity_fwd.cu:75-104.
template <typename T> static void inv3(const T *a, T *o) {
    const T c00 = a[4] * a[8] - a[5] * a[7];
    const T c01 = -(a[3] * a[8] - a[5] * a[6]);
    const T c02 = a[3] * a[7] - a[4] * a[6];
    const T c10 = -(a[1] * a[8] - a[2] * a[7]);
    const T c11 = a[0] * a[8] - a[2] * a[6];
    const T c12 = -(a[0] * a[7] - a[1] * a[6]);
    const T c20 = a[1] * a[5] - a[2] * a[4];
    const T c21 = -(a[0] * a[5] - a[2] * a[3]);
    const T c22 = a[0] * a[4] - a[1] * a[3];
    T det = a[0] * c00 + a[1] * c01 + a[2] * c02;
    if (det == T(0)) det = T(1e-20f);
    const T id = T(1) / det;
    o[0] = c00 * id; o[1] = c10 * id; o[2] = c20 * id;
    o[3] = c01 * id; o[4] = c11 * id; o[5] = c21 * id;
    o[6] = c02 * id; o[7] = c12 * id; o[8] = c22 * id;
}
// Gauss-Jordan inverse with partial pivoting (fwd.cu:26-73), used for K != 3.
template <typename T> static void inv_gj(const T *A, T *out, int n) {
    T aug[8][16];
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < 2 * n; ++c)
            aug[r][c] = (c < n) ? A[r * n + c] : (c - n == r ? T(1) : T(0));
    for (int col = 0; col < n; ++col) {
        int piv = col;
        T best = std::fabs(aug[col][col]);
        for (int r = col + 1; r < n; ++r)
            if (std::fabs(aug[r][col]) > best) { best = std::fabs(aug[r][col]); piv = r; }
        if (piv != col)
            for (int c = 0; c < 2 * n; ++c) std::swap(aug[col][c], aug[piv][c]);
        T d = aug[col][col];
        if (d == T(0)) d = T(1e-20f);
        const T id = T(1) / d;
        for (int c = 0; c < 2 * n; ++c) aug[col][c] *= id;
        for (int r = 0; r < n; ++r) {
            if (r == col) continue;
            const T f = aug[r][col];
            if (f != T(0))
                for (int c = 0; c < 2 * n; ++c) aug[r][c] -= f * aug[col][c];
        }
    }
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) out[r * n + c] = aug[r][n + c];
}

// Lower Cholesky factor of the K x K block (reads its lower triangle), with the
// guards of fwd.cu:250-268 (non-positive pivot -> 1e-20, zero divisor -> 1e-20).
template <typename T> static void chol(const T *A, T *Lc, int K) {
    for (int i = 0; i < K * K; ++i) Lc[i] = 0;
    for (int i = 0; i < K; ++i)
        for (int j = 0; j <= i; ++j) {
            T sum = A[i * K + j];
            for (int k = 0; k < j; ++k) sum -= Lc[i * K + k] * Lc[j * K + k];
            if (i == j) {
                T s = sum;
                if (s <= T(0)) s = T(1e-20f);
                Lc[i * K + j] = std::sqrt(s);
            } else {
                T d = Lc[j * K + j];
                if (d == T(0)) d = T(1e-20f);
                Lc[i * K + j] = sum / d;
            }
        }
}
template <typename T> static T nz(T d) { return d == T(0) ? T(1e-20f) : d; }

template <typename T> struct CondState {
    int K;
    T x[8], beta[8], ba[8], i22[64], r[24], rb[24], v12[24], v21[24], Lc[64], y[8];
};

template <typename T>
static void cond_prepare(int D, const T *m, const T *V, const T *b, const T *q,
                         CondState<T> &st) {
    const int K = D - 3;
    st.K = K;
    T v22[64];
    for (int j = 0; j < K; ++j) {
        st.x[j] = q[j] - m[3 + j];
        st.beta[j] = b[j];
        const T t = b[j] * T(0.25f);
        st.ba[j] = (t < T(1)) ? t : T(1);
    }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < K; ++c) st.v12[r * K + c] = V[r * D + 3 + c];
    for (int r = 0; r < K; ++r)
        for (int c = 0; c < 3; ++c) st.v21[r * 3 + c] = V[(3 + r) * D + c];
    for (int r = 0; r < K; ++r)
        for (int c = 0; c < K; ++c) v22[r * K + c] = V[(3 + r) * D + 3 + c];
    if (K == 3) inv3(v22, st.i22);
    else inv_gj(v22, st.i22, K);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < K; ++c) {
            T acc = 0;
            for (int k = 0; k < K; ++k) acc += st.v12[r * K + k] * st.i22[k * K + c];
            st.r[r * K + c] = acc;
            st.rb[r * K + c] = acc * st.ba[c];
        }
    chol(v22, st.Lc, K);
    for (int i = 0; i < K; ++i) {
        T sum = st.x[i];
        for (int k = 0; k < i; ++k) sum -= st.Lc[i * K + k] * st.y[k];
        st.y[i] = sum / nz(st.Lc[i * K + i]);
    }
}

// Schur-complement conditioning with per-dimension beta damping and the
// Cholesky-whitened opacity falloff: cond_mean_convariance_opacity_fwd.cu:107-290,
// torch twin _torch_impl.py:9-57.
template <typename T>
void cond_fwd(int64_t n, int D, const T *means, const T *covars, const T *opac,
              const T *betas, const T *query, T *om, T *oV, T *oo) {
    const int K = D - 3;
    const T upper = T(1) - std::numeric_limits<T>::epsilon();
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        CondState<T> st;
        const T *m = means + i * D;
        const T *V = covars + i * D * D;
        cond_prepare(D, m, V, betas + i * K, query + i * K, st);
        for (int r = 0; r < 3; ++r) {
            T acc = 0;
            for (int c = 0; c < K; ++c) acc += st.rb[r * K + c] * st.x[c];
            om[i * 3 + r] = m[r] + acc;
            for (int c2 = 0; c2 < 3; ++c2) {
                T a2 = 0;
                for (int k = 0; k < K; ++k) a2 += st.rb[r * K + k] * st.v21[k * 3 + c2];
                oV[i * 9 + r * 3 + c2] = V[r * D + c2] - a2;
            }
        }
        T oc = 1;
        for (int j = 0; j < K; ++j) {
            T d = std::tanh(st.y[j] * st.y[j]);
            if (d < T(0)) d = 0;
            if (d > upper) d = upper;
            oc *= std::pow(T(1) - d, st.beta[j]);
        }
        oo[i] = opac[i] * oc;
    }
}

// VJP of cond_fwd, the same hand derivation as
// cond_mean_convariance_opacity_bwd.cu:102-563 (query gets no gradient).
// exact == 0 reproduces the reference kernel, whose Cholesky backward forms
// G = L^-1 U^T (bwd.cu:501-518) where the derivative of A = L L^T needs
// G = U L^-1; exact != 0 uses U L^-1 and matches autograd / finite differences.
template <typename T>
void cond_bwd(int64_t n, int D, const T *means, const T *covars, const T *opac,
              const T *betas, const T *query, const T *gM, const T *gVc,
              const T *gO, T *g_means, T *g_covars, T *g_opac, T *g_betas, int exact) {
    const int K = D - 3;
    const T upper = T(1) - std::numeric_limits<T>::epsilon();
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        CondState<T> st;
        const T *m = means + i * D;
        const T *V = covars + i * D * D;
        cond_prepare(D, m, V, betas + i * K, query + i * K, st);
        T *gm = g_means + i * D;
        T *gV = g_covars + i * D * D;
        T *gb = g_betas + i * K;
        for (int k = 0; k < D; ++k) gm[k] = 0;
        for (int k = 0; k < D * D; ++k) gV[k] = 0;
        for (int k = 0; k < K; ++k) gb[k] = 0;
        const T *gm3 = gM + i * 3;
        const T *gv = gVc + i * 9;
        for (int r = 0; r < 3; ++r) gm[r] = gm3[r];
        T Gr[24], gx[8];
        for (int c = 0; c < K; ++c) {
            gx[c] = 0;
            for (int r = 0; r < 3; ++r) {
                T acc = gm3[r] * st.x[c];
                for (int k = 0; k < 3; ++k) acc -= gv[r * 3 + k] * st.v21[c * 3 + k];
                Gr[r * K + c] = acc;
                gx[c] += st.rb[r * K + c] * gm3[r];
            }
        }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) gV[r * D + c] += gv[r * 3 + c];
        for (int rr = 0; rr < K; ++rr)
            for (int c = 0; c < 3; ++c) {
                T acc = 0;
                for (int k = 0; k < 3; ++k) acc += st.rb[k * K + rr] * gv[k * 3 + c];
                gV[(3 + rr) * D + c] -= acc;
            }
        T dba[8], G_r[24], Gi22[64];
        for (int c = 0; c < K; ++c) {
            dba[c] = 0;
            for (int r = 0; r < 3; ++r) dba[c] += Gr[r * K + c] * st.r[r * K + c];
            for (int r = 0; r < 3; ++r) G_r[r * K + c] = Gr[r * K + c] * st.ba[c];
        }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < K; ++c) {
                T acc = 0;
                for (int k = 0; k < K; ++k) acc += G_r[r * K + k] * st.i22[c * K + k];
                gV[r * D + 3 + c] += acc;
            }
        for (int rr = 0; rr < K; ++rr)
            for (int c = 0; c < K; ++c) {
                T acc = 0;
                for (int k = 0; k < 3; ++k) acc += st.v12[k * K + rr] * G_r[k * K + c];
                Gi22[rr * K + c] = acc;
            }
        // opacity path
        T dv[8], base[8], oc = 1;
        for (int j = 0; j < K; ++j) {
            T d = std::tanh(st.y[j] * st.y[j]);
            if (d < T(0)) d = 0;
            if (d > upper) d = upper;
            dv[j] = d;
            base[j] = T(1) - d;
            oc *= std::pow(base[j], st.beta[j]);
        }
        g_opac[i] = gO[i] * oc;
        const T goc = gO[i] * opac[i];
        T gy[8], a[8];
        for (int j = 0; j < K; ++j) {
            T gd = 0;
            if (base[j] > T(0)) {
                gb[j] += goc * oc * std::log(base[j]);
                if (dv[j] > T(0) && dv[j] < upper) gd = goc * (-oc * st.beta[j] / base[j]);
            }
            gy[j] = gd * (T(2) * st.y[j] * (T(1) - dv[j] * dv[j]));
        }
        for (int ii = K - 1; ii >= 0; --ii) {
            T sum = gy[ii];
            for (int k = ii + 1; k < K; ++k) sum -= st.Lc[k * K + ii] * a[k];
            a[ii] = sum / nz(st.Lc[ii * K + ii]);
        }
        for (int j = 0; j < K; ++j) gx[j] += a[j];
        // Cholesky backward: S = tril(L^T gL) with halved diagonal,
        // G = L^-T S L^-1, gA = (G + G^T) / 2 with gL = -a y^T (lower part).
        T gL[64], S[64], U[64], Gm[64];
        for (int r = 0; r < K; ++r)
            for (int c = 0; c < K; ++c) gL[r * K + c] = (c <= r) ? -(a[r] * st.y[c]) : T(0);
        for (int r = 0; r < K; ++r)
            for (int c = 0; c < K; ++c) {
                T acc = 0;
                for (int k = 0; k < K; ++k) acc += st.Lc[k * K + r] * gL[k * K + c];
                S[r * K + c] = (c > r) ? T(0) : acc;
            }
        for (int r = 0; r < K; ++r) S[r * K + r] *= T(0.5f);
        for (int col = 0; col < K; ++col)
            for (int ii = K - 1; ii >= 0; --ii) {
                T sum = S[ii * K + col];
                for (int k = ii + 1; k < K; ++k) sum -= st.Lc[k * K + ii] * U[k * K + col];
                U[ii * K + col] = sum / nz(st.Lc[ii * K + ii]);
            }
        if (!exact) {
            for (int col = 0; col < K; ++col)
                for (int ii = 0; ii < K; ++ii) {
                    T sum = U[col * K + ii];
                    for (int k = 0; k < ii; ++k) sum -= st.Lc[ii * K + k] * Gm[k * K + col];
                    Gm[ii * K + col] = sum / nz(st.Lc[ii * K + ii]);
                }
        } else {
            // G L = U, row by row: back substitution with L^T
            for (int r = 0; r < K; ++r)
                for (int ii = K - 1; ii >= 0; --ii) {
                    T sum = U[r * K + ii];
                    for (int k = ii + 1; k < K; ++k) sum -= st.Lc[k * K + ii] * Gm[r * K + k];
                    Gm[r * K + ii] = sum / nz(st.Lc[ii * K + ii]);
                }
        }
        for (int r = 0; r < K; ++r)
            for (int c = 0; c < K; ++c)
                gV[(3 + r) * D + 3 + c] += T(0.5f) * (Gm[r * K + c] + Gm[c * K + r]);
        for (int j = 0; j < K; ++j) gm[3 + j] -= gx[j];
        for (int j = 0; j < K; ++j) gb[j] += dba[j] * ((st.beta[j] < T(4)) ? T(0.25f) : T(0));
        // inverse VJP for the regression path: -i22^T Gi22 i22^T
        T tmp[64];
        for (int r = 0; r < K; ++r)
            for (int c = 0; c < K; ++c) {
                T acc = 0;
                for (int k = 0; k < K; ++k) acc += Gi22[r * K + k] * st.i22[c * K + k];
                tmp[r * K + c] = acc;
            }
        for (int r = 0; r < K; ++r)
            for (int c = 0; c < K; ++c) {
                T acc = 0;
                for (int k = 0; k < K; ++k) acc += st.i22[k * K + r] * tmp[k * K + c];
                gV[(3 + r) * D + 3 + c] -= acc;
            }
    }
}

// ------------------------------------------------------- a6: EWA projection
// Unit-quaternion rotation (w, x, y, z), utils.cuh:13-36.
template <typename T> static M3<T> quat_R(const T *q) {
    T w = q[0], x = q[1], y = q[2], z = q[3];
    const T inv = T(1) / std::sqrt(x * x + y * y + z * z + w * w);
    x *= inv; y *= inv; z *= inv; w *= inv;
    M3<T> R;
    R(0, 0) = 1 - 2 * (y * y + z * z); R(0, 1) = 2 * (x * y - w * z); R(0, 2) = 2 * (x * z + w * y);
    R(1, 0) = 2 * (x * y + w * z); R(1, 1) = 1 - 2 * (x * x + z * z); R(1, 2) = 2 * (y * z - w * x);
    R(2, 0) = 2 * (x * z - w * y); R(2, 1) = 2 * (y * z + w * x); R(2, 2) = 1 - 2 * (x * x + y * y);
    return R;
}

template <typename T>
static M3<T> world_covar(int64_t g, const T *covars6, const T *quats, const T *scales) {
    M3<T> S;
    if (covars6) {
        const T *c = covars6 + g * 6;
        S(0, 0) = c[0]; S(0, 1) = c[1]; S(0, 2) = c[2];
        S(1, 0) = c[1]; S(1, 1) = c[3]; S(1, 2) = c[4];
        S(2, 0) = c[2]; S(2, 1) = c[4]; S(2, 2) = c[5];
    } else {
        M3<T> R = quat_R(quats + g * 4), M;
        const T *s = scales + g * 3;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) M(r, c) = R(r, c) * s[c];
        S = mul(M, tr(M));
    }
    return S;
}

template <typename T> struct Cam {
    M3<T> R;
    T t[3], fx, fy, cx, cy;
};
template <typename T> static Cam<T> load_cam(int c, const T *viewmats, const T *Ks) {
    Cam<T> cam;
    const T *v = viewmats + c * 16;
    for (int r = 0; r < 3; ++r) {
        for (int k = 0; k < 3; ++k) cam.R(r, k) = v[r * 4 + k];
        cam.t[r] = v[r * 4 + 3];
    }
    const T *K = Ks + c * 9;
    cam.fx = K[0]; cam.cx = K[2]; cam.fy = K[4]; cam.cy = K[5];
    return cam;
}

// Perspective Jacobian with the 1.3x frustum clamp of utils.cuh:253-292.
template <typename T> struct Persp {
    T rz, rz2, tx, ty, limxp, limxn, limyp, limyn, J[6];
};
template <typename T>
static Persp<T> persp(const T *pc, T fx, T fy, T cx, T cy, int W, int H) {
    Persp<T> p;
    const T x = pc[0], y = pc[1], z = pc[2];
    const T tfx = T(0.5f) * T(W) / fx, tfy = T(0.5f) * T(H) / fy;
    p.limxp = (T(W) - cx) / fx + T(0.3f) * tfx;
    p.limxn = cx / fx + T(0.3f) * tfx;
    p.limyp = (T(H) - cy) / fy + T(0.3f) * tfy;
    p.limyn = cy / fy + T(0.3f) * tfy;
    p.rz = T(1) / z;
    p.rz2 = p.rz * p.rz;
    p.tx = z * std::min(p.limxp, std::max(-p.limxn, x * p.rz));
    p.ty = z * std::min(p.limyp, std::max(-p.limyn, y * p.rz));
    p.J[0] = fx * p.rz; p.J[1] = 0; p.J[2] = -fx * p.tx * p.rz2;
    p.J[3] = 0; p.J[4] = fy * p.rz; p.J[5] = -fy * p.ty * p.rz2;
    return p;
}

// Per (camera, primitive): world->camera, near/far cull, EWA 2-D covariance,
// eps2d blur, conic, 1-sigma radius and image cull.
// fully_fused_projection_fwd.cu:20-177 (perspective only: the path never
// requests the orthographic camera).
template <typename T>
void project_fwd(int C, int64_t N, const T *means, const T *covars6, const T *quats,
                 const T *scales, const T *viewmats, const T *Ks, int W, int H,
                 T eps2d, T near_p, T far_p, T radius_clip, int32_t *radii,
                 T *means2d, T *depths, T *conics, T *comps) {
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < (int64_t)C * N; ++idx) {
        const int c = (int)(idx / N);
        const int64_t g = idx % N;
        const Cam<T> cam = load_cam(c, viewmats, Ks);
        const T *p = means + g * 3;
        T pc[3];
        for (int r = 0; r < 3; ++r)
            pc[r] = cam.R(r, 0) * p[0] + cam.R(r, 1) * p[1] + cam.R(r, 2) * p[2] + cam.t[r];
        radii[idx] = 0;
        if (comps) comps[idx] = 0;
        if (pc[2] < near_p || pc[2] > far_p) continue;
        const M3<T> Sw = world_covar<T>(g, covars6, quats, scales);
        const M3<T> Sc = mul(mul(cam.R, Sw), tr(cam.R));
        const Persp<T> pp = persp(pc, cam.fx, cam.fy, cam.cx, cam.cy, W, H);
        // cov2d = J Sc J^T
        T JS[6];
        for (int r = 0; r < 2; ++r)
            for (int k = 0; k < 3; ++k) {
                T acc = 0;
                for (int m = 0; m < 3; ++m) acc += pp.J[r * 3 + m] * Sc(m, k);
                JS[r * 3 + k] = acc;
            }
        T c2[4];
        for (int r = 0; r < 2; ++r)
            for (int k = 0; k < 2; ++k) {
                T acc = 0;
                for (int m = 0; m < 3; ++m) acc += JS[r * 3 + m] * pp.J[k * 3 + m];
                c2[r * 2 + k] = acc;
            }
        const T mx = cam.fx * pc[0] * pp.rz + cam.cx;
        const T my = cam.fy * pc[1] * pp.rz + cam.cy;
        const T det_orig = c2[0] * c2[3] - c2[1] * c2[2];
        c2[0] += eps2d;
        c2[3] += eps2d;
        const T det = c2[0] * c2[3] - c2[1] * c2[2];
        const T comp = std::sqrt(std::max(T(0), det_orig / det));
        if (det <= T(0)) continue;
        const T invdet = T(1) / det;
        const T b = T(0.5f) * (c2[0] + c2[3]);
        const T v1 = b + std::sqrt(std::max(T(0.01f), b * b - det));
        const T radius = std::ceil(std::sqrt(v1));
        if (radius <= radius_clip) continue;
        if (mx + radius <= 0 || mx - radius >= T(W) || my + radius <= 0 || my - radius >= T(H))
            continue;
        radii[idx] = (int32_t)radius;
        means2d[idx * 2] = mx;
        means2d[idx * 2 + 1] = my;
        depths[idx] = pc[2];
        conics[idx * 3] = c2[3] * invdet;
        conics[idx * 3 + 1] = -c2[1] * invdet;
        conics[idx * 3 + 2] = c2[0] * invdet;
        if (comps) comps[idx] = comp;
    }
}

// VJP of the unit-quaternion rotation (utils.cuh:38-62).
template <typename T> static void quat_vjp(const T *q, const M3<T> &vR, T *vq) {
    T w = q[0], x = q[1], y = q[2], z = q[3];
    const T inv = T(1) / std::sqrt(x * x + y * y + z * z + w * w);
    x *= inv; y *= inv; z *= inv; w *= inv;
    // vR(r, c) is dL/dR[r][c]; the formulas below are written on the
    // column-major convention g[c][r] = vR(r, c).
    auto g = [&](int col, int row) { return vR(row, col); };
    T vn[4];
    vn[0] = 2 * (x * (g(1, 2) - g(2, 1)) + y * (g(2, 0) - g(0, 2)) + z * (g(0, 1) - g(1, 0)));
    vn[1] = 2 * (-2 * x * (g(1, 1) + g(2, 2)) + y * (g(0, 1) + g(1, 0)) + z * (g(0, 2) + g(2, 0)) +
                 w * (g(1, 2) - g(2, 1)));
    vn[2] = 2 * (x * (g(0, 1) + g(1, 0)) - 2 * y * (g(0, 0) + g(2, 2)) + z * (g(1, 2) + g(2, 1)) +
                 w * (g(2, 0) - g(0, 2)));
    vn[3] = 2 * (x * (g(0, 2) + g(2, 0)) + y * (g(1, 2) + g(2, 1)) - 2 * z * (g(0, 0) + g(1, 1)) +
                 w * (g(0, 1) - g(1, 0)));
    const T qn[4] = {w, x, y, z};
    const T dot = vn[0] * qn[0] + vn[1] * qn[1] + vn[2] * qn[2] + vn[3] * qn[3];
    for (int k = 0; k < 4; ++k) vq[k] += (vn[k] - dot * qn[k]) * inv;
}

// VJP of project_fwd: fully_fused_projection_bwd.cu:20-240 with
// utils.cuh:295-372 (perspective), 386-435 (rigid transform), 451-502 (inverse,
// blur).  Gradients of all cameras are summed per primitive.
template <typename T>
void project_bwd(int C, int64_t N, const T *means, const T *covars6, const T *quats,
                 const T *scales, const T *viewmats, const T *Ks, int W, int H,
                 T eps2d, const int32_t *radii, const T *conics, const T *comps,
                 const T *v_means2d, const T *v_depths, const T *v_conics,
                 const T *v_comps, T *v_means, T *v_covars6, T *v_quats, T *v_scales,
                 T *v_viewmats) {
    // serial over cameras so that per-primitive sums need no atomics
    for (int c = 0; c < C; ++c) {
        const Cam<T> cam = load_cam(c, viewmats, Ks);
        std::vector<T> vview(16, T(0));
#pragma omp parallel
        {
            std::vector<T> vloc(16, T(0));
#pragma omp for schedule(static)
            for (int64_t g = 0; g < N; ++g) {
                const int64_t idx = (int64_t)c * N + g;
                if (radii[idx] <= 0) continue;
                const T *cn = conics + idx * 3;
                const T P[4] = {cn[0], cn[1], cn[1], cn[2]};
                const T vP[4] = {v_conics[idx * 3], T(0.5f) * v_conics[idx * 3 + 1],
                                 T(0.5f) * v_conics[idx * 3 + 1], v_conics[idx * 3 + 2]};
                // v_cov2d = -P vP P
                T tmp[4], vc2[4];
                for (int r = 0; r < 2; ++r)
                    for (int k = 0; k < 2; ++k) tmp[r * 2 + k] = P[r * 2] * vP[k] + P[r * 2 + 1] * vP[2 + k];
                for (int r = 0; r < 2; ++r)
                    for (int k = 0; k < 2; ++k)
                        vc2[r * 2 + k] = -(tmp[r * 2] * P[k] + tmp[r * 2 + 1] * P[2 + k]);
                if (v_comps && comps) {
                    const T comp = comps[idx], vcomp = v_comps[idx];
                    const T detc = P[0] * P[3] - P[1] * P[2];
                    const T vsq = vcomp * T(0.5) / (comp + T(1e-6f));
                    const T om = T(1) - comp * comp;
                    vc2[0] += vsq * (om * P[0] - eps2d * detc);
                    vc2[1] += vsq * (om * P[1]);
                    vc2[2] += vsq * (om * P[2]);
                    vc2[3] += vsq * (om * P[3] - eps2d * detc);
                }
                const T *p = means + g * 3;
                T pc[3];
                for (int r = 0; r < 3; ++r)
                    pc[r] = cam.R(r, 0) * p[0] + cam.R(r, 1) * p[1] + cam.R(r, 2) * p[2] + cam.t[r];
                const M3<T> Sw = world_covar<T>(g, covars6, quats, scales);
                const M3<T> Sc = mul(mul(cam.R, Sw), tr(cam.R));
                const Persp<T> pp = persp(pc, cam.fx, cam.fy, cam.cx, cam.cy, W, H);
                const T *J = pp.J;
                // v_Sc = J^T vc2 J
                M3<T> vSc;
                for (int r = 0; r < 3; ++r)
                    for (int k = 0; k < 3; ++k) {
                        T acc = 0;
                        for (int a = 0; a < 2; ++a)
                            for (int b = 0; b < 2; ++b) acc += J[a * 3 + r] * vc2[a * 2 + b] * J[b * 3 + k];
                        vSc(r, k) = acc;
                    }
                const T fx = cam.fx, fy = cam.fy, rz = pp.rz, rz2 = pp.rz2, rz3 = rz2 * rz;
                const T vm0 = v_means2d[idx * 2], vm1 = v_means2d[idx * 2 + 1];
                T vpc[3] = {fx * rz * vm0, fy * rz * vm1, -(fx * pc[0] * vm0 + fy * pc[1] * vm1) * rz2};
                // v_J = vc2 J Sc^T + vc2^T J Sc   (2 x 3)
                T vJ[6];
                for (int r = 0; r < 2; ++r)
                    for (int k = 0; k < 3; ++k) {
                        T acc = 0;
                        for (int b = 0; b < 2; ++b)
                            for (int m = 0; m < 3; ++m)
                                acc += vc2[r * 2 + b] * J[b * 3 + m] * Sc(k, m) +
                                       vc2[b * 2 + r] * J[b * 3 + m] * Sc(m, k);
                        vJ[r * 3 + k] = acc;
                    }
                const T xr = pc[0] * rz, yr = pc[1] * rz;
                if (xr <= pp.limxp && xr >= -pp.limxn) vpc[0] += -fx * rz2 * vJ[2];
                else vpc[2] += -fx * rz3 * vJ[2] * pp.tx;
                if (yr <= pp.limyp && yr >= -pp.limyn) vpc[1] += -fy * rz2 * vJ[5];
                else vpc[2] += -fy * rz3 * vJ[5] * pp.ty;
                vpc[2] += -fx * rz2 * vJ[0] - fy * rz2 * vJ[4] + T(2) * fx * pp.tx * rz3 * vJ[2] +
                          T(2) * fy * pp.ty * rz3 * vJ[5];
                vpc[2] += v_depths ? v_depths[idx] : T(0);
                // rigid transform VJPs
                for (int r = 0; r < 3; ++r) {
                    for (int k = 0; k < 3; ++k) vloc[r * 4 + k] += vpc[r] * p[k];
                    vloc[r * 4 + 3] += vpc[r];
                }
                T vp[3];
                for (int k = 0; k < 3; ++k)
                    vp[k] = cam.R(0, k) * vpc[0] + cam.R(1, k) * vpc[1] + cam.R(2, k) * vpc[2];
                // v_R += vSc R Sw^T + vSc^T R Sw ; v_Sw = R^T vSc R
                const M3<T> a1 = mul(mul(vSc, cam.R), tr(Sw));
                const M3<T> a2 = mul(mul(tr(vSc), cam.R), Sw);
                for (int r = 0; r < 3; ++r)
                    for (int k = 0; k < 3; ++k) vloc[r * 4 + k] += a1(r, k) + a2(r, k);
                const M3<T> vSw = mul(mul(tr(cam.R), vSc), cam.R);
                for (int k = 0; k < 3; ++k) v_means[g * 3 + k] += vp[k];
                if (covars6) {
                    T *vc = v_covars6 + g * 6;
                    vc[0] += vSw(0, 0);
                    vc[1] += vSw(0, 1) + vSw(1, 0);
                    vc[2] += vSw(0, 2) + vSw(2, 0);
                    vc[3] += vSw(1, 1);
                    vc[4] += vSw(1, 2) + vSw(2, 1);
                    vc[5] += vSw(2, 2);
                } else {
                    // quat/scale chain: utils.cuh:98-134
                    const T *q = quats + g * 4;
                    const T *s = scales + g * 3;
                    const M3<T> R = quat_R(q);
                    M3<T> M;
                    for (int r = 0; r < 3; ++r)
                        for (int k = 0; k < 3; ++k) M(r, k) = R(r, k) * s[k];
                    const M3<T> vM = mul(add(vSw, tr(vSw)), M);
                    M3<T> vR;
                    for (int r = 0; r < 3; ++r)
                        for (int k = 0; k < 3; ++k) vR(r, k) = vM(r, k) * s[k];
                    quat_vjp(q, vR, v_quats + g * 4);
                    for (int k = 0; k < 3; ++k)
                        v_scales[g * 3 + k] += R(0, k) * vM(0, k) + R(1, k) * vM(1, k) + R(2, k) * vM(2, k);
                }
            }
#pragma omp critical
            for (int k = 0; k < 16; ++k) vview[k] += vloc[k];
        }
        if (v_viewmats)
            for (int k = 0; k < 16; ++k) v_viewmats[c * 16 + k] += vview[k];
    }
}

// ------------------------------------------------ a7/a8: tiles, keys, sort
static inline uint32_t sat_u32(double f) {
    // float -> uint32 conversion of the GPU: truncation, saturating, NaN -> 0
    if (!(f > 0.0)) return 0u;
    if (f >= 4294967295.0) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

struct TileBox { uint32_t x0, y0, x1, y1; };

// Tile bounding box of isect_tiles.cu:46-66 (min inclusive, max exclusive).
static TileBox tile_box(float mx, float my, int32_t radius, uint32_t tile_size,
                        uint32_t tw, uint32_t th) {
    const float r = (float)radius;
    const float ts = (float)tile_size;
    const float tr = r / ts, tx = mx / ts, ty = my / ts;
    TileBox b;
    b.x0 = std::min(sat_u32(std::floor(tx - tr)), tw);
    b.y0 = std::min(sat_u32(std::floor(ty - tr)), th);
    b.x1 = std::min(sat_u32(std::ceil(tx + tr)), tw);
    b.y1 = std::min(sat_u32(std::ceil(ty + tr)), th);
    return b;
}

static uint32_t bit_width(uint32_t v) {
    uint32_t b = 0;
    while (v) { ++b; v >>= 1; }
    return b;
}

// Pass 1 of isect_tiles.cu:99-181: tiles per (camera, primitive); returns the
// total number of intersections.
int64_t isect_count(int C, int64_t N, const float *means2d, const int32_t *radii,
                    uint32_t tile_size, uint32_t tw, uint32_t th, int32_t *tiles_per_gauss) {
    int64_t total = 0;
#pragma omp parallel for reduction(+ : total) schedule(static)
    for (int64_t idx = 0; idx < (int64_t)C * N; ++idx) {
        if (radii[idx] <= 0) { tiles_per_gauss[idx] = 0; continue; }
        const TileBox b = tile_box(means2d[idx * 2], means2d[idx * 2 + 1], radii[idx], tile_size, tw, th);
        const int32_t n = (int32_t)((b.y1 - b.y0) * (b.x1 - b.x0));
        tiles_per_gauss[idx] = n;
        total += n;
    }
    return total;
}

// Pass 2 + stable LSD radix sort over bits [0, 32 + tile_bits + cam_bits) of the
// 64-bit keys (isect_tiles.cu:76-96, 137-141, 224-278; the sort is the stable
// ascending order cub::DeviceRadixSort::SortPairs produces).
void isect_emit_sort(int C, int64_t N, const float *means2d, const int32_t *radii,
                     const float *depths, uint32_t tile_size, uint32_t tw, uint32_t th,
                     const int32_t *tiles_per_gauss, int64_t n_isects, int sort,
                     int64_t *isect_ids, int32_t *flatten_ids) {
    const uint32_t n_tiles = tw * th;
    const uint32_t tile_bits = bit_width(n_tiles);
    const uint32_t cam_bits = bit_width((uint32_t)C);
    std::vector<int64_t> start((size_t)C * N + 1, 0);
    for (int64_t i = 0; i < (int64_t)C * N; ++i) start[i + 1] = start[i] + tiles_per_gauss[i];
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < (int64_t)C * N; ++idx) {
        if (radii[idx] <= 0) continue;
        const TileBox b = tile_box(means2d[idx * 2], means2d[idx * 2 + 1], radii[idx], tile_size, tw, th);
        const int64_t cid = idx / N;
        int32_t dbits;
        std::memcpy(&dbits, depths + idx, 4);
        const int64_t denc = (int64_t)dbits; // sign-extended like the reference
        int64_t cur = start[idx];
        for (uint32_t i = b.y0; i < b.y1; ++i)
            for (uint32_t j = b.x0; j < b.x1; ++j) {
                const int64_t tile = (int64_t)i * tw + j;
                isect_ids[cur] = (cid << (32 + tile_bits)) | (tile << 32) | denc;
                flatten_ids[cur] = (int32_t)idx;
                ++cur;
            }
    }
    if (!sort || n_isects == 0) return;
    const uint32_t end_bit = 32 + tile_bits + cam_bits;
    std::vector<uint64_t> k0(n_isects), k1(n_isects);
    std::vector<int32_t> v0(flatten_ids, flatten_ids + n_isects), v1(n_isects);
    for (int64_t i = 0; i < n_isects; ++i) k0[i] = (uint64_t)isect_ids[i];
    for (uint32_t bit = 0; bit < end_bit; bit += 8) {
        const uint32_t nb = std::min(8u, end_bit - bit);
        const uint64_t mask = (1ull << nb) - 1;
        std::vector<int64_t> cnt(257, 0);
        for (int64_t i = 0; i < n_isects; ++i) cnt[((k0[i] >> bit) & mask) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (int64_t i = 0; i < n_isects; ++i) {
            const int64_t dst = cnt[(k0[i] >> bit) & mask]++;
            k1[dst] = k0[i];
            v1[dst] = v0[i];
        }
        k0.swap(k1);
        v0.swap(v1);
    }
    for (int64_t i = 0; i < n_isects; ++i) {
        isect_ids[i] = (int64_t)k0[i];
        flatten_ids[i] = v0[i];
    }
}

// isect_offset_encode (isect_tiles.cu:287-367): first sorted index per
// (camera, tile); tiles past the last intersection get n_isects; no
// intersections -> all zeros.
void offset_encode(int64_t n_isects, const int64_t *isect_ids, int C, uint32_t tw,
                   uint32_t th, int32_t *offsets) {
    const int64_t n_tiles = (int64_t)tw * th;
    const uint32_t tile_bits = bit_width((uint32_t)n_tiles);
    const int64_t total = (int64_t)C * n_tiles;
    if (n_isects == 0) {
        std::fill(offsets, offsets + total, 0);
        return;
    }
    auto bucket = [&](int64_t key) {
        const int64_t hi = key >> 32;
        return (hi >> tile_bits) * n_tiles + (hi & ((1ll << tile_bits) - 1));
    };
    int64_t cur = bucket(isect_ids[0]);
    for (int64_t i = 0; i <= cur && i < total; ++i) offsets[i] = 0;
    for (int64_t k = 1; k < n_isects; ++k) {
        const int64_t b = bucket(isect_ids[k]);
        if (b == cur) continue;
        for (int64_t i = cur + 1; i <= b && i < total; ++i) offsets[i] = (int32_t)k;
        cur = b;
    }
    for (int64_t i = cur + 1; i < total; ++i) offsets[i] = (int32_t)n_isects;
}

// ------------------------------------------------------- a9: blend forward
// Per tile, per pixel, front to back over the tile's sorted range
// (row_sel = row_step | row_offset << 16 with row_step > 1 blends only the
// tile rows ty with ty % row_step == row_offset: a timing sample):
// rasterize_to_pixels_fwd.cu:17-191.  Beta kernel alpha = min(0.999,
// o * (1 - sigma)^beta) for 0 <= sigma < 1, exclusive termination at T <= 1e-4.
template <typename T>
void raster_fwd(int C, int64_t N, int cdim, int64_t n_isects, const T *means2d,
                const T *conics, const T *colors, const T *opac, const T *betas,
                const T *bg, const uint8_t *masks, int W, int H, int tile_size,
                int tw, int th, const int32_t *offsets, const int32_t *flatten_ids,
                T *out_c, T *out_a, int32_t *last_ids, int row_step) {
    const int64_t n_tiles = (int64_t)tw * th;
    (void)N;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t bt = 0; bt < (int64_t)C * n_tiles; ++bt) {
        const int c = (int)(bt / n_tiles);
        const int64_t tile = bt % n_tiles;
        const int ty = (int)(tile / tw), tx = (int)(tile % tw);
        if (ty % (row_step & 0xffff) != (row_step >> 16)) continue;
        const int32_t rs = offsets[bt];
        const int32_t re = (c == C - 1 && tile == n_tiles - 1) ? (int32_t)n_isects : offsets[bt + 1];
        std::vector<T> acc(cdim);
        for (int py_ = 0; py_ < tile_size; ++py_)
            for (int px_ = 0; px_ < tile_size; ++px_) {
                const int i = ty * tile_size + py_, j = tx * tile_size + px_;
                if (i >= H || j >= W) continue;
                const int64_t pix = (int64_t)c * H * W + (int64_t)i * W + j;
                if (masks && !masks[bt]) {
                    for (int k = 0; k < cdim; ++k) out_c[pix * cdim + k] = bg ? bg[c * cdim + k] : T(0);
                    out_a[pix] = 0;
                    last_ids[pix] = 0;
                    continue;
                }
                const T px = (T)j + T(0.5f), py = (T)i + T(0.5f);
                T Tr = 1;
                int32_t cur = 0;
                std::fill(acc.begin(), acc.end(), T(0));
                for (int32_t idx = rs; idx < re; ++idx) {
                    const int32_t g = flatten_ids[idx];
                    const T *cn = conics + (int64_t)g * 3;
                    const T dx = means2d[(int64_t)g * 2] - px, dy = means2d[(int64_t)g * 2 + 1] - py;
                    const T sigma = (cn[0] * dx * dx + cn[2] * dy * dy) + T(2) * cn[1] * dx * dy;
                    if (sigma < T(0) || sigma >= T(1)) continue;
                    const T alpha = std::min(T(0.999f), opac[g] * std::pow(T(1) - sigma, betas[g]));
                    const T nT = Tr * (T(1) - alpha);
                    if (nT <= T(1e-4)) break;
                    const T vis = alpha * Tr;
                    for (int k = 0; k < cdim; ++k) acc[k] += colors[(int64_t)g * cdim + k] * vis;
                    cur = idx;
                    Tr = nT;
                }
                out_a[pix] = T(1) - Tr;
                for (int k = 0; k < cdim; ++k) out_c[pix * cdim + k] = bg ? acc[k] + Tr * bg[c * cdim + k] : acc[k];
                last_ids[pix] = cur;
            }
    }
}

// ------------------------------------------------------ a10: blend backward
// Back to front from each pixel's last contributor, recomputing transmittance
// from 1 - render_alpha: rasterize_to_pixels_bwd.cu:17-276.  Gradients are
// summed over pixels; background gradients are left to the caller (the
// reference computes them in Python, _wrapper.py:1029-1033).
template <typename T>
void raster_bwd(int C, int64_t N, int cdim, int64_t n_isects, const T *means2d,
                const T *conics, const T *colors, const T *opac, const T *betas,
                const T *bg, const uint8_t *masks, int W, int H, int tile_size,
                int tw, int th, const int32_t *offsets, const int32_t *flatten_ids,
                const T *render_alphas, const int32_t *last_ids, const T *v_colors_out,
                const T *v_alphas_out, T *v_means2d, T *v_conics, T *v_colors,
                T *v_opac, T *v_betas, int row_step) {
    const int64_t n_tiles = (int64_t)tw * th;
    (void)N;
    if (n_isects == 0) return;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t bt = 0; bt < (int64_t)C * n_tiles; ++bt) {
        if (masks && !masks[bt]) continue;
        const int c = (int)(bt / n_tiles);
        const int64_t tile = bt % n_tiles;
        const int ty = (int)(tile / tw), tx = (int)(tile % tw);
        if (ty % (row_step & 0xffff) != (row_step >> 16)) continue;
        const int32_t rs = offsets[bt];
        const int32_t re = (c == C - 1 && tile == n_tiles - 1) ? (int32_t)n_isects : offsets[bt + 1];
        std::vector<T> buf(cdim), vrc(cdim);
        for (int py_ = 0; py_ < tile_size; ++py_)
            for (int px_ = 0; px_ < tile_size; ++px_) {
                const int i = ty * tile_size + py_, j = tx * tile_size + px_;
                if (i >= H || j >= W) continue;
                const int64_t pix = (int64_t)c * H * W + (int64_t)i * W + j;
                const T px = (T)j + T(0.5f), py = (T)i + T(0.5f);
                const T Tf = T(1) - render_alphas[pix];
                T Tr = Tf;
                const int32_t bin_final = last_ids[pix];
                for (int k = 0; k < cdim; ++k) { buf[k] = 0; vrc[k] = v_colors_out[pix * cdim + k]; }
                const T vra = v_alphas_out[pix];
                T bgdot = 0;
                if (bg)
                    for (int k = 0; k < cdim; ++k) bgdot += bg[c * cdim + k] * vrc[k];
                for (int32_t idx = std::min(re - 1, bin_final); idx >= rs; --idx) {
                    const int32_t g = flatten_ids[idx];
                    const T *cn = conics + (int64_t)g * 3;
                    const T dx = means2d[(int64_t)g * 2] - px, dy = means2d[(int64_t)g * 2 + 1] - py;
                    const T sigma = (cn[0] * dx * dx + cn[2] * dy * dy) + T(2) * cn[1] * dx * dy;
                    if (sigma < T(0) || sigma >= T(1)) continue;
                    const T o = opac[g], be = betas[g];
                    const T vis = std::pow(T(1) - sigma, be);
                    const T alpha = std::min(T(0.999f), o * vis);
                    const T ra = T(1) / (T(1) - alpha);
                    Tr *= ra;
                    const T fac = alpha * Tr;
                    T v_alpha = 0;
                    for (int k = 0; k < cdim; ++k) {
                        const T ck = colors[(int64_t)g * cdim + k];
#pragma omp atomic
                        v_colors[(int64_t)g * cdim + k] += fac * vrc[k];
                        v_alpha += (ck * Tr - buf[k] * ra) * vrc[k];
                    }
                    v_alpha += Tf * ra * vra;
                    if (bg) v_alpha += -Tf * ra * bgdot;
                    if (o * vis <= T(0.999f)) {
                        const T v_sigma = -v_alpha * o * be * std::pow(T(1) - sigma, be - T(1));
                        const T vcx = dx * dx * v_sigma, vcy = T(2) * dx * dy * v_sigma, vcz = dy * dy * v_sigma;
                        const T vx = T(2) * v_sigma * (cn[0] * dx + cn[1] * dy);
                        const T vy = T(2) * v_sigma * (cn[1] * dx + cn[2] * dy);
                        const T vo = vis * v_alpha;
                        const T vb = v_alpha * o * std::pow(T(1) - sigma, be) * std::log(T(1) - sigma);
#pragma omp atomic
                        v_conics[(int64_t)g * 3] += vcx;
#pragma omp atomic
                        v_conics[(int64_t)g * 3 + 1] += vcy;
#pragma omp atomic
                        v_conics[(int64_t)g * 3 + 2] += vcz;
#pragma omp atomic
                        v_means2d[(int64_t)g * 2] += vx;
#pragma omp atomic
                        v_means2d[(int64_t)g * 2 + 1] += vy;
#pragma omp atomic
                        v_opac[g] += vo;
#pragma omp atomic
                        v_betas[g] += vb;
                    }
                    for (int k = 0; k < cdim; ++k) buf[k] += colors[(int64_t)g * cdim + k] * fac;
                }
            }
    }
}

} // namespace ubs_oracle

// ====================================================================== C ABI
using namespace ubs_oracle;

#define UBS_ORACLE_BOTH(X) X(float, f32) X(double, f64)

extern "C" {

int ubso_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void ubso_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

#define DEF(T, S)                                                                          \
    void ubso_rotmat_fwd_##S(int64_t n, const T *l, int64_t ls, T *R) { rotmat_fwd(n, l, ls, R); } \
    void ubso_rotmat_bwd_##S(int64_t n, const T *vR, T *vl) { rotmat_bwd(n, vR, vl); }        \
    void ubso_covar_fwd_##S(int64_t n, int D, const T *rot, const T *s, const T *l,           \
                            const int32_t *ri, const int32_t *rj, int m, int sp, T *out) {   \
        covar_fwd(n, D, rot, s, l, ri, rj, m, sp, out);                                        \
    }                                                                                          \
    void ubso_covar_bwd_##S(int64_t n, int D, const T *rot, const T *s, const T *l,           \
                            const int32_t *ri, const int32_t *rj, int m, int sp, const T *g,  \
                            T *vr, T *vs, T *vl) {                                             \
        covar_bwd(n, D, rot, s, l, ri, rj, m, sp, g, vr, vs, vl);                              \
    }                                                                                          \
    void ubso_cond_fwd_##S(int64_t n, int D, const T *m, const T *V, const T *o,              \
                           const T *b, const T *q, T *om, T *oV, T *oo) {                      \
        cond_fwd(n, D, m, V, o, b, q, om, oV, oo);                                             \
    }                                                                                          \
    void ubso_cond_bwd_##S(int64_t n, int D, const T *m, const T *V, const T *o,              \
                           const T *b, const T *q, const T *gm, const T *gv, const T *go,      \
                           T *rm, T *rv, T *ro, T *rb, int ex) {                               \
        cond_bwd(n, D, m, V, o, b, q, gm, gv, go, rm, rv, ro, rb, ex);                         \
    }                                                                                          \
    void ubso_project_fwd_##S(int C, int64_t N, const T *m, const T *c6, const T *q,          \
                              const T *s, const T *vm, const T *K, int W, int H, T e, T nr,   \
                              T fr, T rc, int32_t *radii, T *m2, T *d, T *cn, T *cp) {         \
        project_fwd(C, N, m, c6, q, s, vm, K, W, H, e, nr, fr, rc, radii, m2, d, cn, cp);      \
    }                                                                                          \
    void ubso_project_bwd_##S(int C, int64_t N, const T *m, const T *c6, const T *q,          \
                              const T *s, const T *vm, const T *K, int W, int H, T e,         \
                              const int32_t *radii, const T *cn, const T *cp, const T *vm2,   \
                              const T *vd, const T *vcn, const T *vcp, T *vmeans, T *vc6,      \
                              T *vq, T *vs, T *vview) {                                        \
        project_bwd(C, N, m, c6, q, s, vm, K, W, H, e, radii, cn, cp, vm2, vd, vcn, vcp,      \
                    vmeans, vc6, vq, vs, vview);                                               \
    }                                                                                          \
    void ubso_raster_fwd_##S(int C, int64_t N, int cd, int64_t ni, const T *m2, const T *cn,  \
                             const T *col, const T *o, const T *b, const T *bg,               \
                             const uint8_t *mk, int W, int H, int ts, int tw, int th,         \
                             const int32_t *off, const int32_t *fl, T *oc, T *oa,             \
                             int32_t *li, int rs) {                                            \
        raster_fwd(C, N, cd, ni, m2, cn, col, o, b, bg, mk, W, H, ts, tw, th, off, fl, oc, oa, \
                   li, rs < 1 ? 1 : rs);                                                       \
    }                                                                                          \
    void ubso_raster_bwd_##S(int C, int64_t N, int cd, int64_t ni, const T *m2, const T *cn,  \
                             const T *col, const T *o, const T *b, const T *bg,               \
                             const uint8_t *mk, int W, int H, int ts, int tw, int th,         \
                             const int32_t *off, const int32_t *fl, const T *ra,              \
                             const int32_t *li, const T *vc, const T *va, T *vm2, T *vcn,     \
                             T *vcol, T *vo, T *vb, int rs) {                                  \
        raster_bwd(C, N, cd, ni, m2, cn, col, o, b, bg, mk, W, H, ts, tw, th, off, fl, ra, li, \
                   vc, va, vm2, vcn, vcol, vo, vb, rs < 1 ? 1 : rs);                           \
    }

UBS_ORACLE_BOTH(DEF)
#undef DEF

int64_t ubso_isect_count(int C, int64_t N, const float *m2, const int32_t *radii,
                         uint32_t ts, uint32_t tw, uint32_t th, int32_t *tpg) {
    return isect_count(C, N, m2, radii, ts, tw, th, tpg);
}
void ubso_isect_emit_sort(int C, int64_t N, const float *m2, const int32_t *radii,
                          const float *depths, uint32_t ts, uint32_t tw, uint32_t th,
                          const int32_t *tpg, int64_t n_isects, int sort, int64_t *ids,
                          int32_t *fl) {
    isect_emit_sort(C, N, m2, radii, depths, ts, tw, th, tpg, n_isects, sort, ids, fl);
}
void ubso_offset_encode(int64_t n_isects, const int64_t *ids, int C, uint32_t tw,
                        uint32_t th, int32_t *offsets) {
    offset_encode(n_isects, ids, C, tw, th, offsets);
}

} // extern "C"
