// The vertex stage of the splat pipeline (Lichtso/splatter src/shaders.wgsl:63-294, 507-573):
//   vertex_math  -> the forward preprocess kernel (FP32, WGSL operation order, bit-identical to the
//                   oracle's restatement);
//   vertex_vjp_t -> its vector-Jacobian product for the backward, in reverse mode (float, or double
//                   for needles and discs), around the forward's own float values.
// Compiled with -fmad=false; explicit fmaf() only where written.
#pragma once
#include "spl_device.cuh"

namespace spl {

__device__ __forceinline__ float val(float x) { return x; }
__device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ float abs_(float x) { return fabsf(x); }
__device__ __forceinline__ float min_(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float max_(float a, float b) { return fmaxf(a, b); }
template <class S>
__device__ __forceinline__ S cst(float c) {
    return S(c);
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

// Everything the vertex stage derives from one splat that the raster uses and that depends on the
// splat's parameters: the affine pixel -> tc map, the colour, and (for the box) the rect basis.
template <class S>
struct VertexOut {
    S A00, A01, B0, A10, A11, B1;  // tc = (A00 X + A01 Y + B0, A10 X + A11 Y + B1)
    S cr, cg, cb;                  // colour before the fragment falloff
    S Xx, Xy, Yx, Yy, t0, t1;      // rect basis (shaders.wgsl:543-547)
    float bx, by;                  // AA-square offsets
};

template <int SHO, bool COV, class S>
__device__ __forceinline__ void vertex_math(const Uniforms& u, S cx, S cy, S cz, S q0, S q1, S q2, S q3, S scx, S scy,
                                            S scz, const float* sh, VertexOut<S>& o) {
    // colour (shaders.wgsl:531-532)
    {
        const S vx = cx - u.camera[12], vy = cy - u.camera[13], vz = cz - u.camera[14];
        const S len = sqrt_((vx * vx + vy * vy) + vz * vz);
        const S dx = vx / len, dy = vy / len, dz = vz / len;
        const S dxx = dx * dx, dyy = dy * dy, dzz = dz * dz;
        o.cr = sh_channel<SHO>(sh, 0, dx, dy, dz, dxx, dyy, dzz);
        o.cg = sh_channel<SHO>(sh, 1, dx, dy, dz, dxx, dyy, dzz);
        o.cb = sh_channel<SHO>(sh, 2, dx, dy, dz, dxx, dyy, dzz);
    }
    // conic + decomposition (shaders.wgsl:533-542)
    const S sx = scx * u.splat_scale, sy = scy * u.splat_scale, sz = scz * u.splat_scale;
    S t0, t1, rj, rk, ax0, ax1;
    outline_ellipse<COV>(u, sx, sy, sz, q0, q1, q2, q3, cx, cy, cz, t0, t1, rj, rk, ax0, ax1);
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
}

// ---- reverse mode -------------------------------------------------------------------------------
// Column-major 3x3 helpers: X(r, c) = X.m[c * 3 + r].
template <class T>
__device__ __forceinline__ T m3(const M3T<T>& X, int r, int c) {
    return X.m[c * 3 + r];
}

// Gradient of one SH colour channel with respect to the unit view direction (x, y, z): the derivative
// of sh_channel's polynomial term by term (xx = x^2 ...), accumulated with weight gc into gd.
template <int SHO, class T>
__device__ __forceinline__ void sh_channel_grad(const float* sh, int c, T gc, T x, T y, T z, T xx, T yy, T zz, T* gd) {
    T gx = 0.0f, gy = 0.0f, gz = 0.0f;
    if (SHO > 0) {
        gy += c_shc[1] * sh[3 + c];
        gz += c_shc[2] * sh[6 + c];
        gx += c_shc[3] * sh[9 + c];
    }
    if (SHO > 1) {
        const float k4 = c_shc[4] * sh[12 + c], k5 = c_shc[5] * sh[15 + c], k6 = c_shc[6] * sh[18 + c];
        const float k7 = c_shc[7] * sh[21 + c], k8 = c_shc[8] * sh[24 + c];
        gx += (k4 * y + k7 * z) + (k8 - k6) * (2.0f * x);
        gy += (k4 * x + k5 * z) - (k6 + k8) * (2.0f * y);
        gz += (k5 * y + k7 * x) + k6 * (4.0f * z);
    }
    if (SHO > 2) {
        const float k9 = c_shc[9] * sh[27 + c], k10 = c_shc[10] * sh[30 + c], k11 = c_shc[11] * sh[33 + c];
        const float k12 = c_shc[12] * sh[36 + c], k13 = c_shc[13] * sh[39 + c], k14 = c_shc[14] * sh[42 + c];
        const float k15 = c_shc[15] * sh[45 + c];
        const float f11 = (4.0f * zz - xx) - yy;  // the factor of y (k11) and of x (k13)
        gx += k9 * (6.0f * x * y) + k10 * (y * z) - k11 * (2.0f * x * y) - k12 * (6.0f * x * z) +
              k13 * (f11 - 2.0f * xx) + k14 * (2.0f * x * z) + k15 * (3.0f * xx - 3.0f * yy);
        gy += k9 * (3.0f * xx - 3.0f * yy) + k10 * (x * z) + k11 * (f11 - 2.0f * yy) - k12 * (6.0f * y * z) -
              k13 * (2.0f * x * y) - k14 * (2.0f * y * z) - k15 * (6.0f * x * y);
        gz += k10 * (x * y) + k11 * (8.0f * y * z) + k12 * ((2.0f * zz - 3.0f * xx) - 3.0f * yy + 4.0f * zz) +
              k13 * (8.0f * x * z) + k14 * (xx - yy);
    }
    gd[0] += gc * gx;
    gd[1] += gc * gy;
    gd[2] += gc * gz;
}

// The vertex stage's vector-Jacobian product, in reverse mode: the gradients of the record's affine map
// and colour, g = dL/d(A00, A01, Br0, A10, A11, Br1, -, r, g, b), pulled back to the splat's centre
// (gin[0..2]), rotation (gin[3..6]) and scale (gin[7..9]).  Br = I (rx - t0, ry - t1) is tc at a
// reference pixel centre (Xr, Yr) whose view-plane position is (rx, ry), I the inverse rectangle basis:
// the backward differentiates tc = A (X - Xr, Y - Yr) + Br instead of A (X, Y) + B, the same function
// without the large, cancelling terms that absolute pixel coordinates put into dB/dp.
//
// One sweep of values and one of adjoints, in T (float, or double for needles and discs), around the
// forward's own float outline (centre t, axis directions (rk, -rj), (rj, rk), and semi-axes):
// * the outline's derivatives follow from its dual conic, not from the cone matrix M = G A G^T the
//   forward uses.  A = (1 - |l|^2) I + l l^T has eigenvalues 1 and 1 - |l|^2 (|l| = the camera's
//   distance in units of the splat's radii), so for a distant splat the outline is the small
//   difference of terms of size |l|^2, which float carries only to ~|l|^2 2^-24 relative.  The same
//   ellipse (exactly, in real arithmetic) is
//     D = (1 - |l|^2) M^-1 = Sigma - w w^T,  w = C^T (camera - centre),  Sigma = C^T R^-T S^2 R^-1 C
//   (the covariance in camera axes; R^-1 as the adjugate over the determinant, so that non-unit
//   quaternions differentiate correctly): with k = w_z^2 - Sigma_zz the centre is
//   m = (w_xy w_z - Sigma_xy,z) / k and the semi-axis matrix E = N / k^2, N written below as a sum
//   of squares whose terms have the size of the result.  Along the forward's axes U, V:
//   d ax0 = U^T dE U / (2 ax0), d ax1 = V^T dE V / (2 ax1), and the axes turn by
//   dpsi = V^T dE U / (U^T E U - V^T E V) (eigenvector perturbation);
// * the covariance semi-axes (projected_covariance) through the eigenvectors of the projected 2x2;
// * the rectangle basis and its inverse, and the SH colour of the view direction.
template <class T, int SHO, bool COV>
__device__ __forceinline__ void vertex_vjp_t(const Uniforms& u, float cxf, float cyf, float czf, float q0f, float q1f,
                                             float q2f, float q3f, float scx, float scy, float scz, const float* sh,
                                             float rxf, float ryf, const float* gf, float* gin) {
    // the outline's centre and axes: the forward's float values
    float t0f, t1f, rjf, rkf, ax0f, ax1f;
    outline_ellipse<COV>(u, scx * u.splat_scale, scy * u.splat_scale, scz * u.splat_scale, q0f, q1f, q2f, q3f, cxf,
                         cyf, czf, t0f, t1f, rjf, rkf, ax0f, ax1f);
    const T cx = cxf, cy = cyf, cz = czf, q0 = q0f, q1 = q1f, q2 = q2f, q3 = q3f, rx = rxf, ry = ryf;
    const T sx = (T)(scx * u.splat_scale), sy = (T)(scy * u.splat_scale), sz = (T)(scz * u.splat_scale);
    T g[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) g[i] = gf[i];
    // ---- forward values ----
    T t0 = t0f, t1 = t1f, rj = rjf, rk = rkf, ax0 = ax0f, ax1 = ax1f;
    const M3T<T> C = camera3<T>(u);
    const M3T<T> R = quat_to_mat(q0, q1, q2, q3);
    M3T<T> Ri;  // R^-1 by the adjugate over the determinant
    {
        const T c00 = R.m[4] * R.m[8] - R.m[7] * R.m[5];
        const T c01 = R.m[7] * R.m[2] - R.m[1] * R.m[8];
        const T c02 = R.m[1] * R.m[5] - R.m[4] * R.m[2];
        const T det = (R.m[0] * c00 + R.m[3] * c01) + R.m[6] * c02;
        const T idet = 1.0f / det;
        Ri.m[0] = c00 * idet;
        Ri.m[3] = (R.m[6] * R.m[5] - R.m[3] * R.m[8]) * idet;
        Ri.m[6] = (R.m[3] * R.m[7] - R.m[6] * R.m[4]) * idet;
        Ri.m[1] = c01 * idet;
        Ri.m[4] = (R.m[0] * R.m[8] - R.m[6] * R.m[2]) * idet;
        Ri.m[7] = (R.m[6] * R.m[1] - R.m[0] * R.m[7]) * idet;
        Ri.m[2] = c02 * idet;
        Ri.m[5] = (R.m[3] * R.m[2] - R.m[0] * R.m[5]) * idet;
        Ri.m[8] = (R.m[0] * R.m[4] - R.m[3] * R.m[1]) * idet;
    }
    const M3T<T> K = mul3(Ri, C);
    const T s2[3] = {sx * sx, sy * sy, sz * sz};
    const int ii[6] = {0, 0, 1, 0, 1, 2}, jj[6] = {0, 1, 1, 2, 2, 2};
    T Sg[6];  // Sigma: xx, xy, yy, xz, yz, zz (the first three only through N below)
#pragma unroll
    for (int e = 3; e < 6; ++e)
        Sg[e] = (s2[0] * m3(K, 0, ii[e])) * m3(K, 0, jj[e]) + (s2[1] * m3(K, 1, ii[e])) * m3(K, 1, jj[e]) +
                (s2[2] * m3(K, 2, ii[e])) * m3(K, 2, jj[e]);
    const T ro[3] = {u.camera[12] - cx, u.camera[13] - cy, u.camera[14] - cz};
    T w[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = (u.camera[i * 4 + 0] * ro[0] + u.camera[i * 4 + 1] * ro[1]) + u.camera[i * 4 + 2] * ro[2];
    const T Sxz = Sg[3], Syz = Sg[4], Szz = Sg[5];
    const T wz2 = w[2] * w[2];
    const T k = wz2 - Szz;
    const T mx = (w[0] * w[2] - Sxz) / k, my = (w[1] * w[2] - Syz) / k;
    // N = F - M without cancellation between the splat's scales:
    //   F = sum_a s_a^2 v_a v_a^T,  v_a = w_z K(a, xy) - K(a, z) w_xy   (Sigma_2 w_z^2 - w_z (w_2 s^T + s w_2^T) + Szz w_2 w_2^T)
    //   M = sum_{a<b} s_a^2 s_b^2 u_ab u_ab^T,  u_ab = K(b, z) K(a, xy) - K(a, z) K(b, xy)   (Sigma_2 Szz - s s^T, by
    //   Cauchy-Binet: its s_z^4 terms vanish identically instead of cancelling in T, which matters for
    //   needle-like splats)
    T va[3][2], uab[3][2];
    const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
    T Nxx = 0.0f, Nxy = 0.0f, Nyy = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        va[a][0] = w[2] * m3(K, a, 0) - m3(K, a, 2) * w[0];
        va[a][1] = w[2] * m3(K, a, 1) - m3(K, a, 2) * w[1];
        Nxx += s2[a] * (va[a][0] * va[a][0]);
        Nxy += s2[a] * (va[a][0] * va[a][1]);
        Nyy += s2[a] * (va[a][1] * va[a][1]);
    }
#pragma unroll
    for (int pq = 0; pq < 3; ++pq) {
        const int a = pa[pq], b = pb[pq];
        uab[pq][0] = m3(K, b, 2) * m3(K, a, 0) - m3(K, a, 2) * m3(K, b, 0);
        uab[pq][1] = m3(K, b, 2) * m3(K, a, 1) - m3(K, a, 2) * m3(K, b, 1);
        const T p = s2[a] * s2[b];
        Nxx -= p * (uab[pq][0] * uab[pq][0]);
        Nxy -= p * (uab[pq][0] * uab[pq][1]);
        Nyy -= p * (uab[pq][1] * uab[pq][1]);
    }
    const T ik2 = 1.0f / (k * k);
    const T Exx = Nxx * ik2, Exy = Nxy * ik2, Eyy = Nyy * ik2;
    const T U0 = rk, U1 = -rj, V0 = rj, V1 = rk;
    const T quu = ((U0 * U0) * Exx + (2.0f * (U0 * U1)) * Exy) + (U1 * U1) * Eyy;
    const T qvv = ((V0 * V0) * Exx + (2.0f * (V0 * V1)) * Exy) + (V1 * V1) * Eyy;
    const T gap = quu - qvv;
    const T r0 = sqrt(quu), r1 = sqrt(qvv);
    // covariance semi-axes (projected_covariance), values kept for the sweep back
    M3T<T> Q, Tm;
    T v[3], v2 = 0.0f, zzv = 0.0f, qr[2] = {0.0f, 0.0f}, pxx = 0.0f, pxy = 0.0f, pyy = 0.0f, bsq = 0.0f;
    bool pass[2] = {false, false};
    if (COV) {
        M3T<T> Ts = R;  // R with its columns scaled
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            Ts.m[0 * 3 + r] = Ts.m[0 * 3 + r] * sx;
            Ts.m[1 * 3 + r] = Ts.m[1 * 3 + r] * sy;
            Ts.m[2 * 3 + r] = Ts.m[2 * 3 + r] * sz;
        }
#pragma unroll
        for (int r = 0; r < 3; ++r)
            v[r] = ((u.view[0 * 4 + r] * cx + u.view[1 * 4 + r] * cy) + u.view[2 * 4 + r] * cz) + u.view[3 * 4 + r] * 1.0f;
        v2 = v[2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const T q = v[i] / v2;
            const T mlo = fmax(q, (T)-1.0f), mhi = fmin(mlo, (T)1.0f);
            pass[i] = mlo == q && mhi == mlo;  // inside the clamp: the derivative follows q
            qr[i] = mhi;
            v[i] = mhi * v2;
        }
        zzv = v2 * v2;
        M3T<T> J;
        J.m[0] = 1.0f / v2; J.m[1] = 0.0f; J.m[2] = (-v[0]) / zzv;
        J.m[3] = 0.0f; J.m[4] = 1.0f / v2; J.m[5] = (-v[1]) / zzv;
        J.m[6] = 0.0f; J.m[7] = 0.0f; J.m[8] = 0.0f;
        Q = mul3(transpose3(Ts), C);
        Tm = mul3(Q, J);
        const M3T<T> P = mul3(transpose3(Tm), Tm);
        pxx = P.m[0];
        pxy = P.m[1];
        pyy = P.m[4];
        const T a = (pxx - pyy) * (pxx - pyy);
        bsq = sqrt(a + (4.0f * pxy) * pxy);
        ax0 = sqrt(((pxx + pyy) + bsq) * 0.5f);
        ax1 = sqrt(((pxx + pyy) - bsq) * 0.5f);
    }
    // rectangle basis and its inverse
    const T sa = u.bias + ax0, sb = u.bias + ax1;
    const T Xx = rk * sa, Xy = (-rj) * sa, Yx = rj * sb, Yy = rk * sb;
    const T det2 = Xx * Yy - Xy * Yx;
    const T idet2 = 1.0f / det2;
    const T i00 = Yy * idet2, i01 = (-Yx) * idet2, i10 = (-Xy) * idet2, i11 = Xx * idet2;
    const T psx = (2.0f * u.view_size[0]) / (T)u.image_size[0];
    const T psy = -((2.0f * u.view_size[1]) / (T)u.image_size[1]);
    const T ox = rx - t0, oy = ry - t1;

    // ---- sweep back: affine map -> ellipse ----
    const T bi00 = g[0] * psx + g[2] * ox, bi01 = g[1] * psy + g[2] * oy;
    const T bi10 = g[3] * psx + g[5] * ox, bi11 = g[4] * psy + g[5] * oy;
    const T bt0 = -(g[2] * i00 + g[5] * i10), bt1 = -(g[2] * i01 + g[5] * i11);
    T bXx = bi11 * idet2, bXy = -(bi10 * idet2), bYx = -(bi01 * idet2), bYy = bi00 * idet2;
    const T bidet = ((bi00 * Yy - bi01 * Yx) - bi10 * Xy) + bi11 * Xx;
    const T bdet = bidet * (-(idet2 * idet2));
    bXx += bdet * Yy;
    bYy += bdet * Xx;
    bXy -= bdet * Yx;
    bYx -= bdet * Xy;
    const T brk = bXx * sa + bYy * sb, brj = bYx * sb - bXy * sa;
    const T bax0 = bXx * rk - bXy * rj, bax1 = bYx * rj + bYy * rk;

    T gc[3] = {0.0f, 0.0f, 0.0f}, gs[3] = {0.0f, 0.0f, 0.0f};
    M3T<T> bR;
#pragma unroll
    for (int e = 0; e < 9; ++e) bR.m[e] = 0.0f;
    // ---- covariance semi-axes ----
    if (COV) {
        // ax0^2, ax1^2 are the eigenvalues of the 2x2 (pxx pxy; pxy pyy); each eigenvalue's gradient is its
        // unit eigenvector's outer product (u for the larger, v for the smaller), which has none of the
        // cancellation of differentiating ((pxx + pyy) -+ b) / 2 for a needle's thin axis
        const T bh0 = ax0 > 0.0f ? bax0 / (2.0f * ax0) : 0.0f, bh1 = ax1 > 0.0f ? bax1 / (2.0f * ax1) : 0.0f;
        T bpxx, bpyy, bpxy;
        if (bsq > 0.0f) {
            const T c2 = (pxx - pyy) / bsq, sn2 = (2.0f * pxy) / bsq;  // cos, sin of twice the axis angle
            const T cu = sqrt(fmax((T)0.0f, (T)0.5f * ((T)1.0f + c2)));
            const T su = copysign(sqrt(fmax((T)0.0f, (T)0.5f * ((T)1.0f - c2))), sn2);
            bpxx = bh0 * (cu * cu) + bh1 * (su * su);
            bpyy = bh0 * (su * su) + bh1 * (cu * cu);
            bpxy = 2.0f * (bh0 - bh1) * (cu * su);
        } else {  // equal eigenvalues: the derivative the formula takes there (b's derivative is zero)
            bpxx = bpyy = 0.5f * (bh0 + bh1);
            bpxy = 0.0f;
        }
        // P = Tm^T Tm: pxx = |Tm(:,0)|^2, pyy = |Tm(:,1)|^2, pxy = Tm(:,1) . Tm(:,0)
        M3T<T> bTm;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            bTm.m[0 * 3 + r] = 2.0f * bpxx * m3(Tm, r, 0) + bpxy * m3(Tm, r, 1);
            bTm.m[1 * 3 + r] = 2.0f * bpyy * m3(Tm, r, 1) + bpxy * m3(Tm, r, 0);
            bTm.m[2 * 3 + r] = 0.0f;
        }
        // Tm = Q J: bQ = bTm J^T, bJ = Q^T bTm (only J's non-zero entries matter)
        const T J00 = 1.0f / v2, J20 = (-v[0]) / zzv, J21 = (-v[1]) / zzv;
        M3T<T> bQ;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            bQ.m[0 * 3 + r] = m3(bTm, r, 0) * J00;           // J(0, 0)
            bQ.m[1 * 3 + r] = m3(bTm, r, 1) * J00;           // J(1, 1)
            bQ.m[2 * 3 + r] = m3(bTm, r, 0) * J20 + m3(bTm, r, 1) * J21;
        }
        T bJ00 = 0.0f, bJ11 = 0.0f, bJ20 = 0.0f, bJ21 = 0.0f;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            bJ00 += m3(Q, r, 0) * m3(bTm, r, 0);
            bJ11 += m3(Q, r, 1) * m3(bTm, r, 1);
            bJ20 += m3(Q, r, 2) * m3(bTm, r, 0);
            bJ21 += m3(Q, r, 2) * m3(bTm, r, 1);
        }
        T bv[3] = {0.0f, 0.0f, 0.0f};
        bv[2] -= (bJ00 + bJ11) / (v2 * v2);
        const T bzz = (bJ20 * v[0] + bJ21 * v[1]) / (zzv * zzv);
        bv[2] += bzz * (2.0f * v2);
        const T bvc[2] = {-(bJ20 / zzv), -(bJ21 / zzv)};
#pragma unroll
        for (int i = 0; i < 2; ++i) {  // v_i = clamp(v_i / v2, -1, 1) v2
            const T bm = bvc[i] * v2;
            bv[2] += bvc[i] * qr[i];
            if (pass[i]) {
                bv[i] += bm / v2;
                bv[2] -= bm * qr[i] / v2;
            }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) gc[i] += (u.view[i * 4 + 0] * bv[0] + u.view[i * 4 + 1] * bv[1]) + u.view[i * 4 + 2] * bv[2];
        // Q = T^T C: bT(m, i) = sum_j bQ(i, j) C(m, j); T(:, a) = R(:, a) s_a
        const T sc[3] = {sx, sy, sz};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int mm = 0; mm < 3; ++mm) {
                const T bT = (m3(bQ, a, 0) * m3(C, mm, 0) + m3(bQ, a, 1) * m3(C, mm, 1)) + m3(bQ, a, 2) * m3(C, mm, 2);
                bR.m[a * 3 + mm] += bT * sc[a];
                gs[a] += bT * m3(R, mm, a);
            }
    }
    // ---- the outline through the dual conic ----
    {
        const T bmx = bt0, bmy = bt1;
        const T bpsi = brk * rj - brj * rk;
        const T bquv = gap != 0.0f ? bpsi / gap : 0.0f;
        const T bquu = (!COV && r0 > 0.0f) ? bax0 / (2.0f * r0) : 0.0f;
        const T bqvv = (!COV && r1 > 0.0f) ? bax1 / (2.0f * r1) : 0.0f;
        const T bExx = (bquu * (U0 * U0) + bqvv * (V0 * V0)) + bquv * (U0 * V0);
        const T bExy = (bquu * (2.0f * (U0 * U1)) + bqvv * (2.0f * (V0 * V1))) + bquv * (U0 * V1 + U1 * V0);
        const T bEyy = (bquu * (U1 * U1) + bqvv * (V1 * V1)) + bquv * (U1 * V1);
        const T bNxx = bExx * ik2, bNxy = bExy * ik2, bNyy = bEyy * ik2;
        const T bik2 = (bExx * Nxx + bExy * Nxy) + bEyy * Nyy;
        T bk = bik2 * (-2.0f * ik2 / k);
        T bw[3] = {0.0f, 0.0f, 0.0f}, bS[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};  // xx xy yy xz yz zz
        // centre
        bw[0] += bmx * w[2] / k;
        bw[1] += bmy * w[2] / k;
        bw[2] += (bmx * w[0] + bmy * w[1]) / k;
        bS[3] -= bmx / k;
        bS[4] -= bmy / k;
        bk -= (bmx * mx + bmy * my) / k;
        // N = F - M (above): back to the scales, K and w
        M3T<T> bK;
#pragma unroll
        for (int e = 0; e < 9; ++e) bK.m[e] = 0.0f;
        T bs2[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            bs2[a] += (bNxx * (va[a][0] * va[a][0]) + bNxy * (va[a][0] * va[a][1])) + bNyy * (va[a][1] * va[a][1]);
            const T bv0 = s2[a] * (2.0f * bNxx * va[a][0] + bNxy * va[a][1]);
            const T bv1 = s2[a] * (2.0f * bNyy * va[a][1] + bNxy * va[a][0]);
            bw[2] += bv0 * m3(K, a, 0) + bv1 * m3(K, a, 1);
            bK.m[0 * 3 + a] += w[2] * bv0;
            bK.m[1 * 3 + a] += w[2] * bv1;
            bK.m[2 * 3 + a] -= bv0 * w[0] + bv1 * w[1];
            bw[0] -= m3(K, a, 2) * bv0;
            bw[1] -= m3(K, a, 2) * bv1;
        }
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int a = pa[pq], b = pb[pq];
            const T p = s2[a] * s2[b];
            const T bp = -((bNxx * (uab[pq][0] * uab[pq][0]) + bNxy * (uab[pq][0] * uab[pq][1])) +
                               bNyy * (uab[pq][1] * uab[pq][1]));
            bs2[a] += bp * s2[b];
            bs2[b] += bp * s2[a];
            const T bu0 = -p * (2.0f * bNxx * uab[pq][0] + bNxy * uab[pq][1]);
            const T bu1 = -p * (2.0f * bNyy * uab[pq][1] + bNxy * uab[pq][0]);
            bK.m[2 * 3 + b] += bu0 * m3(K, a, 0) + bu1 * m3(K, a, 1);
            bK.m[0 * 3 + a] += m3(K, b, 2) * bu0;
            bK.m[1 * 3 + a] += m3(K, b, 2) * bu1;
            bK.m[2 * 3 + a] -= bu0 * m3(K, b, 0) + bu1 * m3(K, b, 1);
            bK.m[0 * 3 + b] -= m3(K, a, 2) * bu0;
            bK.m[1 * 3 + b] -= m3(K, a, 2) * bu1;
        }
        gs[0] += bs2[0] * (2.0f * sx);
        gs[1] += bs2[1] * (2.0f * sy);
        gs[2] += bs2[2] * (2.0f * sz);
        // k = wz2 - Szz, wz2 = w2^2
        T bwz2 = bk;
        bS[5] -= bk;
        bw[2] += bwz2 * (2.0f * w[2]);
        // w_i = sum_r C(r, i) (camera_r - c_r)
#pragma unroll
        for (int r = 0; r < 3; ++r) gc[r] -= (bw[0] * m3(C, r, 0) + bw[1] * m3(C, r, 1)) + bw[2] * m3(C, r, 2);
        // Sigma_e = sum_a s2_a K(a, i_e) K(a, j_e) (only xz, yz and zz are left with adjoints)
#pragma unroll
        for (int e = 3; e < 6; ++e)
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const T kai = m3(K, a, ii[e]), kaj = m3(K, a, jj[e]);
                gs[a] += bS[e] * (kai * kaj) * (2.0f * (a == 0 ? sx : (a == 1 ? sy : sz)));
                bK.m[ii[e] * 3 + a] += bS[e] * s2[a] * kaj;
                bK.m[jj[e] * 3 + a] += bS[e] * s2[a] * kai;
            }
        // K = Ri C: bRi(r, kk) = sum_c bK(r, c) C(kk, c); Ri = R^-1: bR -= Ri^T bRi Ri^T
        M3T<T> bRi;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
                bRi.m[kk * 3 + r] = (m3(bK, r, 0) * m3(C, kk, 0) + m3(bK, r, 1) * m3(C, kk, 1)) + m3(bK, r, 2) * m3(C, kk, 2);
        const M3T<T> X1 = mul3(transpose3(Ri), bRi);
        const M3T<T> X2 = mul3(X1, transpose3(Ri));
#pragma unroll
        for (int e = 0; e < 9; ++e) bR.m[e] -= X2.m[e];
    }
    // ---- rotation matrix -> quaternion (quat_to_mat) ----
    {
        const T s2c = (T)1.41421356237309504880f;  // quat_to_mat's float constant
        const T qx = q0 * s2c, qy = q1 * s2c, qz = q2 * s2c, qw = q3 * s2c;
        const T* b = bR.m;
        const T gqx = ((b[1] - b[3]) * qw + (b[6] - b[2]) * qz) + (b[5] - b[7]) * qy;
        const T gqy = ((b[1] + b[3]) * qz + (b[2] + b[6]) * qw) + (b[5] - b[7]) * qx - 2.0f * qy * (b[4] + b[8]);
        const T gqz = ((b[1] + b[3]) * qy + (b[5] + b[7]) * qw) + (b[6] - b[2]) * qx - 2.0f * qz * (b[0] + b[8]);
        const T gqw = ((b[1] - b[3]) * qx + (b[2] + b[6]) * qy) + (b[5] + b[7]) * qz - 2.0f * qw * (b[0] + b[4]);
        gin[3] = (float)(gqx * s2c);
        gin[4] = (float)(gqy * s2c);
        gin[5] = (float)(gqz * s2c);
        gin[6] = (float)(gqw * s2c);
    }
    // ---- colour of the view direction ----
    {
        const T vx = cx - u.camera[12], vy = cy - u.camera[13], vz = cz - u.camera[14];
        const T len = sqrt((vx * vx + vy * vy) + vz * vz);
        const T dx = vx / len, dy = vy / len, dz = vz / len;
        T gd[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int c = 0; c < 3; ++c)
            sh_channel_grad<SHO, T>(sh, c, g[7 + c], dx, dy, dz, dx * dx, dy * dy, dz * dz, gd);
        const T dd = (dx * gd[0] + dy * gd[1]) + dz * gd[2];
        gc[0] += (gd[0] - dx * dd) / len;
        gc[1] += (gd[1] - dy * dd) / len;
        gc[2] += (gd[2] - dz * dd) / len;
    }
    gin[0] = (float)gc[0];
    gin[1] = (float)gc[1];
    gin[2] = (float)gc[2];
    gin[7] = (float)(gs[0] * u.splat_scale);
    gin[8] = (float)(gs[1] * u.splat_scale);
    gin[9] = (float)(gs[2] * u.splat_scale);
#pragma unroll
    for (int i = 0; i < 10; ++i) gin[i] = isfinite(gin[i]) ? gin[i] : 0.0f;
}

// Splats whose largest scale exceeds NEEDLE_RATIO times their smallest (needles and discs).  A rotation
// about a needle's long axis, or about a disc's normal, moves only the short axes: the exact gradient
// is a sum of adjoints of order s_max^2 (through the dual conic's N and the inverse rotation) that
// cancel to order s_min^2.  In float that sum keeps a rounding error of about eps (s_max / s_min)^2 of
// the gradient's scale, and the error changes with the last bits of the record gradients (which the
// raster backward sums with float atomics in no fixed order): measured on GB300 as the run-to-run change
// of the float sweep's gradients, relative to the largest gradient of the frame, 5e-6 at ratio 33,
// 2.4e-5 at 55, 2.4e-4 at 400 and 7e-2 at 3000.  Above ratio 32 the sweep runs in double (below 1e-6
// at every ratio measured).
constexpr float NEEDLE_RATIO = 32.0f;
__device__ __forceinline__ bool needs_double_sweep(float sx, float sy, float sz) {
    const float hi = fmaxf(fmaxf(sx, sy), sz), lo = fminf(fminf(sx, sy), sz);
    return hi > NEEDLE_RATIO * lo;
}

}  // namespace spl
