// The vertex stage of the splat pipeline (Lichtso/splatter src/shaders.wgsl:63-294, 507-573) as one
// template over the scalar type:
//   S = float -> the forward preprocess kernel (FP32, WGSL operation order, bit-identical to the
//                oracle's restatement);
//   S = Df    -> the same arithmetic on forward-mode dual numbers (value, derivative).  The value
//                part of every Df operation is exactly the float operation, so the backward kernel
//                differentiates precisely what the forward computed.
// Compiled with -fmad=false; explicit fmaf() only where written.
#pragma once
#include "spl_device.cuh"

namespace spl {

// ---- forward-mode dual number ------------------------------------------------------------------
struct Df {
    float v, d;
};
__device__ __forceinline__ Df operator+(Df a, Df b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Df operator-(Df a, Df b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Df operator*(Df a, Df b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Df operator/(Df a, Df b) {
    const float q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Df operator-(Df a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Df operator+(Df a, float b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Df operator+(float a, Df b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Df operator-(Df a, float b) { return {a.v - b, a.d}; }
__device__ __forceinline__ Df operator-(float a, Df b) { return {a - b.v, -b.d}; }
__device__ __forceinline__ Df operator*(Df a, float b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Df operator*(float a, Df b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Df operator/(Df a, float b) { return {a.v / b, a.d / b}; }
__device__ __forceinline__ Df operator/(float a, Df b) {
    const float q = a / b.v;
    return {q, (-q * b.d) / b.v};
}

__device__ __forceinline__ float val(float x) { return x; }
__device__ __forceinline__ float val(Df x) { return x.v; }
__device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ Df sqrt_(Df x) {
    const float r = sqrtf(x.v);
    return {r, r > 0.0f ? x.d / (2.0f * r) : 0.0f};
}
__device__ __forceinline__ float abs_(float x) { return fabsf(x); }
__device__ __forceinline__ Df abs_(Df x) { return {fabsf(x.v), x.v < 0.0f ? -x.d : x.d}; }
// fminf/fmaxf semantics on the value (NaN loses); the derivative follows the chosen operand
__device__ __forceinline__ float min_(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float max_(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ Df min_(Df a, float b) {
    const float m = fminf(a.v, b);
    return {m, m == a.v ? a.d : 0.0f};
}
__device__ __forceinline__ Df max_(Df a, float b) {
    const float m = fmaxf(a.v, b);
    return {m, m == a.v ? a.d : 0.0f};
}
__device__ __forceinline__ Df max_(Df a, Df b) { return fmaxf(a.v, b.v) == a.v ? a : b; }
template <class S>
__device__ __forceinline__ S cst(float c) {
    return S(c);
}
template <>
__device__ __forceinline__ Df cst<Df>(float c) {
    return Df{c, 0.0f};
}
template <class S>
__device__ __forceinline__ float sign_(S x) {
    const float v = val(x);
    return v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : 0.0f);
}

// ---- mat3 (column-major m[c*3 + r]); (A*B) column j = A * B[j] in column order ------------------
template <class S>
struct M3T {
    S m[9];
};
template <class S>
__device__ __forceinline__ M3T<S> mul3(const M3T<S>& A, const M3T<S>& B) {
    M3T<S> t;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i)
            t.m[j * 3 + i] = (A.m[0 * 3 + i] * B.m[j * 3 + 0] + A.m[1 * 3 + i] * B.m[j * 3 + 1]) + A.m[2 * 3 + i] * B.m[j * 3 + 2];
    return t;
}
template <class S>
__device__ __forceinline__ M3T<S> transpose3(const M3T<S>& A) {
    M3T<S> t;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) t.m[c * 3 + r] = A.m[r * 3 + c];
    return t;
}
// camera rotation (constant)
template <class S>
__device__ __forceinline__ M3T<S> camera3(const Uniforms& u) {
    M3T<S> c;
#pragma unroll
    for (int col = 0; col < 3; ++col)
#pragma unroll
        for (int r = 0; r < 3; ++r) c.m[col * 3 + r] = cst<S>(u.camera[col * 4 + r]);
    return c;
}

// quatToMat (shaders.wgsl:63-79); q = (scalar, i, j, k)
template <class S>
__device__ __forceinline__ M3T<S> quat_to_mat(S px, S py, S pz, S pw) {
    const float s2 = 1.41421356237309504880f;
    const S qx = px * s2, qy = py * s2, qz = pz * s2, qw = pw * s2;
    const S yy = qy * qy, yz = qy * qz, yw = qy * qw, yx = qy * qx;
    const S zz = qz * qz, zw = qz * qw, zx = qz * qx;
    const S ww = qw * qw, wx = qw * qx;
    M3T<S> m;
    m.m[0] = (1.0f - zz) - ww; m.m[1] = yz + wx;          m.m[2] = yw - zx;
    m.m[3] = yz - wx;          m.m[4] = (1.0f - yy) - ww; m.m[5] = zw + yx;
    m.m[6] = yw + zx;          m.m[7] = zw - yx;          m.m[8] = (1.0f - yy) - zz;
    return m;
}

// projectedContourOfEllipsoid (shaders.wgsl:125-169)
template <class S>
__device__ __forceinline__ M3T<S> projected_contour(const Uniforms& u, S sx, S sy, S sz, S q0, S q1, S q2, S q3,
                                                    S tx, S ty, S tz) {
    const M3T<S> C = camera3<S>(u);
    M3T<S> T = quat_to_mat(q0, q1, q2, q3);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        T.m[0 * 3 + r] = T.m[0 * 3 + r] / sx;
        T.m[1 * 3 + r] = T.m[1 * 3 + r] / sy;
        T.m[2 * 3 + r] = T.m[2 * 3 + r] / sz;
    }
    const S ro0 = u.camera[12] - tx, ro1 = u.camera[13] - ty, ro2 = u.camera[14] - tz;
    S l[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) l[i] = (ro0 * T.m[i * 3 + 0] + ro1 * T.m[i * 3 + 1]) + ro2 * T.m[i * 3 + 2];
    const S l0 = l[0] * l[0], l1 = l[1] * l[1], l2 = l[2] * l[2];
    const S dx = (1.0f - l1) - l2, dy = (1.0f - l0) - l2, dz = (1.0f - l0) - l1;
    const S trx = l[1] * l[2], try_ = l[0] * l[2], trz = l[0] * l[1];
    M3T<S> A;
    A.m[0] = dx;   A.m[1] = trz;  A.m[2] = try_;
    A.m[3] = trz;  A.m[4] = dy;   A.m[5] = trx;
    A.m[6] = try_; A.m[7] = trx;  A.m[8] = dz;
    const M3T<S> T2 = mul3(transpose3(C), T);
    return mul3(mul3(T2, A), transpose3(T2));
}

// projectedCovarianceOfEllipsoid (shaders.wgsl:99-118)
template <class S>
__device__ __forceinline__ M3T<S> projected_covariance(const Uniforms& u, S sx, S sy, S sz, S q0, S q1, S q2, S q3,
                                                       S tx, S ty, S tz) {
    const M3T<S> C = camera3<S>(u);
    M3T<S> T = quat_to_mat(q0, q1, q2, q3);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        T.m[0 * 3 + r] = T.m[0 * 3 + r] * sx;
        T.m[1 * 3 + r] = T.m[1 * 3 + r] * sy;
        T.m[2 * 3 + r] = T.m[2 * 3 + r] * sz;
    }
    S v[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
        v[r] = ((u.view[0 * 4 + r] * tx + u.view[1 * 4 + r] * ty) + u.view[2 * 4 + r] * tz) + u.view[3 * 4 + r] * 1.0f;
    v[0] = min_(max_(v[0] / v[2], -1.0f), 1.0f) * v[2];
    v[1] = min_(max_(v[1] / v[2], -1.0f), 1.0f) * v[2];
    const S zz = v[2] * v[2];
    M3T<S> J;
    J.m[0] = 1.0f / v[2];  J.m[1] = cst<S>(0.0f); J.m[2] = (-v[0]) / zz;
    J.m[3] = cst<S>(0.0f); J.m[4] = 1.0f / v[2];  J.m[5] = (-v[1]) / zz;
    J.m[6] = cst<S>(0.0f); J.m[7] = cst<S>(0.0f); J.m[8] = cst<S>(0.0f);
    const M3T<S> Tm = mul3(mul3(transpose3(T), C), J);
    return mul3(transpose3(Tm), Tm);
}

__constant__ float c_shc[16] = {
    0.28209479177387814f,  -0.4886025119029199f, 0.4886025119029199f,  -0.4886025119029199f,
    1.0925484305920792f,   -1.0925484305920792f, 0.31539156525252005f, -1.0925484305920792f,
    0.5462742152960396f,   -0.5900435899266435f, 2.890611442640554f,   -0.4570457994644658f,
    0.3731763325901154f,   -0.4570457994644658f, 1.445305721320277f,   -0.5900435899266435f,
};

// sphericalHarmonicsLookup (shaders.wgsl:268-294), one channel; sh coefficients are constants here
template <int SHO, class S>
__device__ __forceinline__ S sh_channel(const float* sh, int c, S x, S y, S z, S xx, S yy, S zz) {
    S col = cst<S>(0.5f);
    col = col + c_shc[0] * sh[c];
    if (SHO > 0) {
        col = col + (c_shc[1] * sh[3 + c]) * y;
        col = col + (c_shc[2] * sh[6 + c]) * z;
        col = col + (c_shc[3] * sh[9 + c]) * x;
    }
    if (SHO > 1) {
        col = col + ((c_shc[4] * sh[12 + c]) * x) * y;
        col = col + ((c_shc[5] * sh[15 + c]) * y) * z;
        col = col + (c_shc[6] * sh[18 + c]) * ((2.0f * zz - xx) - yy);
        col = col + ((c_shc[7] * sh[21 + c]) * x) * z;
        col = col + (c_shc[8] * sh[24 + c]) * (xx - yy);
    }
    if (SHO > 2) {
        col = col + ((c_shc[9] * sh[27 + c]) * y) * (3.0f * xx - yy);
        col = col + (((c_shc[10] * sh[30 + c]) * x) * y) * z;
        col = col + ((c_shc[11] * sh[33 + c]) * y) * ((4.0f * zz - xx) - yy);
        col = col + ((c_shc[12] * sh[36 + c]) * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
        col = col + ((c_shc[13] * sh[39 + c]) * x) * ((4.0f * zz - xx) - yy);
        col = col + ((c_shc[14] * sh[42 + c]) * z) * (xx - yy);
        col = col + ((c_shc[15] * sh[45 + c]) * x) * (xx - 3.0f * yy);
    }
    return col;
}

// The SH basis values B_k(d) with rgb_c = 0.5 + sum_k B_k * sh[3k + c] (the gradient of the colour
// with respect to coefficient k of every channel).
template <int SHO>
__device__ __forceinline__ void sh_basis(float x, float y, float z, float* B) {
    const float xx = x * x, yy = y * y, zz = z * z;
    B[0] = c_shc[0];
    if (SHO > 0) {
        B[1] = c_shc[1] * y;
        B[2] = c_shc[2] * z;
        B[3] = c_shc[3] * x;
    }
    if (SHO > 1) {
        B[4] = (c_shc[4] * x) * y;
        B[5] = (c_shc[5] * y) * z;
        B[6] = c_shc[6] * ((2.0f * zz - xx) - yy);
        B[7] = (c_shc[7] * x) * z;
        B[8] = c_shc[8] * (xx - yy);
    }
    if (SHO > 2) {
        B[9] = (c_shc[9] * y) * (3.0f * xx - yy);
        B[10] = ((c_shc[10] * x) * y) * z;
        B[11] = (c_shc[11] * y) * ((4.0f * zz - xx) - yy);
        B[12] = (c_shc[12] * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
        B[13] = (c_shc[13] * x) * ((4.0f * zz - xx) - yy);
        B[14] = (c_shc[14] * z) * (xx - yy);
        B[15] = (c_shc[15] * x) * (xx - 3.0f * yy);
    }
}

template <class S>
struct is_df {
    static constexpr bool value = false;
};
template <>
struct is_df<Df> {
    static constexpr bool value = true;
};

// The splat's outline ellipse in the camera's z = 1 plane from the bounding elliptic cone: centre
// (t0, t1) (extractTranslationOfEllipse, shaders.wgsl:179-191), axis directions (rk, -rj) and (rj, rk)
// (extractRotationOfEllipse, shaders.wgsl:193-215) and, unless COV, the semi-axes along them
// (extractScaleOfEllipse, shaders.wgsl:217-237).  Float only: the forward's exact arithmetic.
template <bool COV>
__device__ __forceinline__ void outline_ellipse(const Uniforms& u, float sx, float sy, float sz, float q0, float q1,
                                                float q2, float q3, float cx, float cy, float cz, float& t0, float& t1,
                                                float& rj, float& rk, float& ax0, float& ax1) {
    const M3T<float> M = projected_contour(u, sx, sy, sz, q0, q1, q2, q3, cx, cy, cz);
    const float Mxx = M.m[0], Mxy = M.m[1], Mxz = M.m[2], Myy = M.m[4], Myz = M.m[5], Mzz = M.m[8];
    const float disc = Mxx * Myy - Mxy * Mxy;
    const float inv = 1.0f / disc;
    t0 = (Mxy * Myz - Myy * Mxz) * inv;
    t1 = (Mxy * Mxz - Mxx * Myz) * inv;
    const float ra = (Mxx - Myy) * (Mxx - Myy);
    const float rb = ra + (4.0f * Mxy) * Mxy;
    const float rc = 0.5f * sqrtf(ra / rb);
    rj = sqrtf(0.5f - rc);
    rk = ((-sqrtf(0.5f + rc)) * sign_(Mxy)) * sign_(Mxx - Myy);
    if (Mxy < 0.0f || Mxx - Myy < 0.0f) {
        rk = -rk;
        rj = -rj;
    }
    if (Mxx - Myy < 0.0f) {
        const float tmp = rj;
        rj = -rk;
        rk = tmp;
    }
    ax0 = ax1 = 0.0f;
    if (!COV) {
        const float d = ((2.0f * Mxy) * rj) * rk;
        const float e = Mzz - (((Mxx * t0) * t0 + (Myy * t1) * t1) + ((2.0f * Mxy) * t0) * t1);
        ax0 = sqrtf(fabsf(e / (((Mxx * rk) * rk + (Myy * rj) * rj) - d)));
        ax1 = sqrtf(fabsf(e / (((Mxx * rj) * rj + (Myy * rk) * rk) + d)));
    }
}

// Derivatives of the outline ellipse for the backward.  The cone matrix M = G A G^T above has
// A = (1 - |l|^2) I + l l^T, whose eigenvalues are 1 and 1 - |l|^2 (|l| = the camera's distance in
// units of the splat's radii): for a distant splat the outline is the small difference of terms of
// size |l|^2, which float carries to only ~|l|^2 * 2^-24 relative, and so do their derivatives.  The
// same ellipse (exactly, in real arithmetic) follows from the dual conic
//   D = (1 - |l|^2) M^-1 = Sigma - w w^T,  w = C^T (camera - centre),  Sigma = C^T R^-T S^2 R^-1 C
// (the splat's covariance in camera axes; R^-1 as the adjugate over the determinant, so that
// non-unit quaternions differentiate correctly): with k = w_z^2 - Sigma_zz the centre is
// m = (w_xy w_z - Sigma_xy,z) / k and the semi-axis matrix E = N / k^2,
//   N = Sigma_2 w_z^2 - w_z (w_2 s^T + s w_2^T) + Sigma_zz w_2 w_2^T - (Sigma_2 Sigma_zz - s s^T),
//   s = (Sigma_xz, Sigma_yz),
// whose terms have the size of the result.  Along the forward's axes U = (rk, -rj), V = (rj, rk):
// d ax0 = U^T dE U / (2 ax0), d ax1 = V^T dE V / (2 ax1), and the axes turn by
// dpsi = V^T dE U / (U^T E U - V^T E V) (eigenvector perturbation): d rk = rj dpsi, d rj = -rk dpsi.
// The values returned are the forward's (t0v ... a1v).
__device__ __forceinline__ void outline_derivatives(const Uniforms& u, Df sx, Df sy, Df sz, Df q0, Df q1, Df q2,
                                                    Df q3, Df cx, Df cy, Df cz, float t0v, float t1v, float rjv,
                                                    float rkv, float a0v, float a1v, Df& t0, Df& t1, Df& rj, Df& rk,
                                                    Df& ax0, Df& ax1) {
    const M3T<Df> R = quat_to_mat(q0, q1, q2, q3);
    // adjugate: Ri(r, c) = cofactor(c, r) / det
    const Df c00 = R.m[4] * R.m[8] - R.m[7] * R.m[5];
    const Df c01 = R.m[7] * R.m[2] - R.m[1] * R.m[8];
    const Df c02 = R.m[1] * R.m[5] - R.m[4] * R.m[2];
    const Df det = (R.m[0] * c00 + R.m[3] * c01) + R.m[6] * c02;
    const Df idet = 1.0f / det;
    M3T<Df> Ri;  // column-major, R(r, c) = R.m[c * 3 + r]
    Ri.m[0] = c00 * idet;
    Ri.m[3] = (R.m[6] * R.m[5] - R.m[3] * R.m[8]) * idet;
    Ri.m[6] = (R.m[3] * R.m[7] - R.m[6] * R.m[4]) * idet;
    Ri.m[1] = c01 * idet;
    Ri.m[4] = (R.m[0] * R.m[8] - R.m[6] * R.m[2]) * idet;
    Ri.m[7] = (R.m[6] * R.m[1] - R.m[0] * R.m[7]) * idet;
    Ri.m[2] = c02 * idet;
    Ri.m[5] = (R.m[3] * R.m[2] - R.m[0] * R.m[5]) * idet;
    Ri.m[8] = (R.m[0] * R.m[4] - R.m[3] * R.m[1]) * idet;
    const M3T<Df> K = mul3(Ri, camera3<Df>(u));  // R^-1 C
    // Sigma(i, j) = sum_a s_a^2 K(a, i) K(a, j)
    const Df s2[3] = {sx * sx, sy * sy, sz * sz};
    Df Sg[6];  // xx, xy, yy, xz, yz, zz
    const int ii[6] = {0, 0, 1, 0, 1, 2}, jj[6] = {0, 1, 1, 2, 2, 2};
#pragma unroll
    for (int e = 0; e < 6; ++e)
        Sg[e] = (s2[0] * K.m[ii[e] * 3 + 0]) * K.m[jj[e] * 3 + 0] + (s2[1] * K.m[ii[e] * 3 + 1]) * K.m[jj[e] * 3 + 1] +
                (s2[2] * K.m[ii[e] * 3 + 2]) * K.m[jj[e] * 3 + 2];
    const Df ro0 = u.camera[12] - cx, ro1 = u.camera[13] - cy, ro2 = u.camera[14] - cz;
    Df w[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = (u.camera[i * 4 + 0] * ro0 + u.camera[i * 4 + 1] * ro1) + u.camera[i * 4 + 2] * ro2;
    const Df Sxx = Sg[0], Sxy = Sg[1], Syy = Sg[2], Sxz = Sg[3], Syz = Sg[4], Szz = Sg[5];
    const Df wz2 = w[2] * w[2];
    const Df k = wz2 - Szz;
    const Df mx = (w[0] * w[2] - Sxz) / k, my = (w[1] * w[2] - Syz) / k;
    const Df Nxx = ((Sxx * wz2 - (2.0f * w[2]) * (w[0] * Sxz)) + Szz * (w[0] * w[0])) - (Sxx * Szz - Sxz * Sxz);
    const Df Nyy = ((Syy * wz2 - (2.0f * w[2]) * (w[1] * Syz)) + Szz * (w[1] * w[1])) - (Syy * Szz - Syz * Syz);
    const Df Nxy = ((Sxy * wz2 - w[2] * (w[0] * Syz + w[1] * Sxz)) + Szz * (w[0] * w[1])) - (Sxy * Szz - Sxz * Syz);
    const Df ik2 = 1.0f / (k * k);
    const Df Exx = Nxx * ik2, Exy = Nxy * ik2, Eyy = Nyy * ik2;
    const float U0 = rkv, U1 = -rjv, V0 = rjv, V1 = rkv;
    const Df quu = ((U0 * U0) * Exx + (2.0f * (U0 * U1)) * Exy) + (U1 * U1) * Eyy;
    const Df qvv = ((V0 * V0) * Exx + (2.0f * (V0 * V1)) * Exy) + (V1 * V1) * Eyy;
    const Df quv = ((U0 * V0) * Exx + (U0 * V1 + U1 * V0) * Exy) + (U1 * V1) * Eyy;
    const float gap = quu.v - qvv.v;
    const float dpsi = gap != 0.0f ? quv.d / gap : 0.0f;
    t0 = Df{t0v, mx.d};
    t1 = Df{t1v, my.d};
    rk = Df{rkv, rjv * dpsi};
    rj = Df{rjv, -(rkv * dpsi)};
    const float r0 = sqrtf(quu.v), r1 = sqrtf(qvv.v);
    ax0 = Df{a0v, r0 > 0.0f ? quu.d / (2.0f * r0) : 0.0f};
    ax1 = Df{a1v, r1 > 0.0f ? qvv.d / (2.0f * r1) : 0.0f};
}

// Everything the vertex stage derives from one splat that the raster uses and that depends on the
// splat's parameters: the affine pixel -> tc map, the colour, and (for the box) the rect basis.
template <class S>
struct VertexOut {
    S A00, A01, B0, A10, A11, B1;  // tc = (A00 X + A01 Y + B0, A10 X + A11 Y + B1)
    S cr, cg, cb;                  // colour before the fragment falloff
    S Xx, Xy, Yx, Yy, t0, t1;      // rect basis (shaders.wgsl:543-547)
    float bx, by;                  // AA-square offsets (value only)
    S B0r, B1r;                    // tc at a reference pixel centre (backward only, see vertex_math)
};

// With REF, also B0r/B1r = tc at the reference pixel centre (Xr, Yr) given as its view-plane position
// (rx, ry), computed from the small offset (rx - t0, ry - t1).  The backward differentiates
// tc = A (X - Xr, Y - Yr) + Br instead of A (X, Y) + B: the same function, but without the large,
// cancelling terms that absolute pixel coordinates put into dB/dp.
// Without COLOUR the colour is left out (o.cr, o.cg, o.cb zero): the backward's rotation and scale
// directions, on which the colour does not depend.
template <int SHO, bool COV, class S, bool REF = false, bool COLOUR = true>
__device__ __forceinline__ void vertex_math(const Uniforms& u, S cx, S cy, S cz, S q0, S q1, S q2, S q3, S scx, S scy,
                                            S scz, const float* sh, VertexOut<S>& o, float rx = 0.0f,
                                            float ry = 0.0f) {
    if constexpr (COLOUR) {
        // colour (shaders.wgsl:531-532)
        const S vx = cx - u.camera[12], vy = cy - u.camera[13], vz = cz - u.camera[14];
        const S len = sqrt_((vx * vx + vy * vy) + vz * vz);
        const S dx = vx / len, dy = vy / len, dz = vz / len;
        const S dxx = dx * dx, dyy = dy * dy, dzz = dz * dz;
        o.cr = sh_channel<SHO>(sh, 0, dx, dy, dz, dxx, dyy, dzz);
        o.cg = sh_channel<SHO>(sh, 1, dx, dy, dz, dxx, dyy, dzz);
        o.cb = sh_channel<SHO>(sh, 2, dx, dy, dz, dxx, dyy, dzz);
    } else {
        o.cr = o.cg = o.cb = cst<S>(0.0f);
    }
    // conic + decomposition (shaders.wgsl:533-542)
    const S sx = scx * u.splat_scale, sy = scy * u.splat_scale, sz = scz * u.splat_scale;
    S t0, t1, rj, rk, ax0, ax1;
    if constexpr (!is_df<S>::value) {
        outline_ellipse<COV>(u, sx, sy, sz, q0, q1, q2, q3, cx, cy, cz, t0, t1, rj, rk, ax0, ax1);
    } else {
        // values: the forward's float arithmetic; derivatives: the dual conic (outline_derivatives)
        float t0v, t1v, rjv, rkv, a0v, a1v;
        outline_ellipse<COV>(u, val(sx), val(sy), val(sz), val(q0), val(q1), val(q2), val(q3), val(cx), val(cy),
                             val(cz), t0v, t1v, rjv, rkv, a0v, a1v);
        outline_derivatives(u, sx, sy, sz, q0, q1, q2, q3, cx, cy, cz, t0v, t1v, rjv, rkv, a0v, a1v, t0, t1, rj, rk,
                            ax0, ax1);
    }
    if (COV) {
        // extractScaleOfCovariance(projectedCovarianceOfEllipsoid) (shaders.wgsl:240-246, 99-118)
        const M3T<S> P = projected_covariance(u, sx, sy, sz, q0, q1, q2, q3, cx, cy, cz);
        const S pxx = P.m[0], pxy = P.m[1], pyy = P.m[4];
        const S a = (pxx - pyy) * (pxx - pyy);
        const S b = sqrt_(a + (4.0f * pxy) * pxy);
        ax0 = sqrt_(((pxx + pyy) + b) * 0.5f);
        ax1 = sqrt_(((pxx + pyy) - b) * 0.5f);
    }
    // rect basis (shaders.wgsl:543-547) and its inverse (shaders.wgsl:563-566), folded with the
    // pixel -> view-plane mapping so that tc is affine in the pixel centre
    const S sa = u.bias + ax0, sb = u.bias + ax1;
    o.Xx = rk * sa;
    o.Xy = (-rj) * sa;
    o.Yx = rj * sb;
    o.Yy = rk * sb;
    o.t0 = t0;
    o.t1 = t1;
    const S det = o.Xx * o.Yy - o.Xy * o.Yx;
    const S idet = 1.0f / det;
    const S i00 = o.Yy * idet, i01 = (-o.Yx) * idet, i10 = (-o.Xy) * idet, i11 = o.Xx * idet;
    const float vw = u.view_size[0], vh = u.view_size[1];
    const float Wf = (float)u.image_size[0], Hf = (float)u.image_size[1];
    const float psx = (2.0f * vw) / Wf, psy = -((2.0f * vh) / Hf);
    const S bx = (-vw) - t0, by = vh - t1;
    o.A00 = i00 * psx;
    o.A01 = i01 * psy;
    o.B0 = i00 * bx + i01 * by;
    o.A10 = i10 * psx;
    o.A11 = i11 * psy;
    o.B1 = i10 * bx + i11 * by;
    o.bx = val(bx);
    o.by = val(by);
    if (REF) {
        const S ox = rx - t0, oy = ry - t1;
        o.B0r = i00 * ox + i01 * oy;
        o.B1r = i10 * ox + i11 * oy;
    }
}

}  // namespace spl
