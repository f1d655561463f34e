// TEST INFRASTRUCTURE ONLY — the oracle. Nothing in the product links, loads or calls this file;
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may use it, and only as
// the checker (or as the timed CPU baseline), never as the thing measured or shipped.
//
// What this is: a CPU restatement of splatter's per-frame splat pipeline (Lichtso/splatter,
// src/shaders.wgsl + src/renderer.rs + src/scene.rs + src/utils.rs), written from the WGSL/Rust
// source as a transliteration with a FIXED floating-point operation order, so that the CUDA path
// can be compared with it bit for bit in FP32.  The projection math is a template; the FP32
// instance is the bit-exact checker and the FP64 instance is the "true math" reference for
// conics, colours and gradients.
//
// PARITY UNPINNED.  The reference is a Rust + wgpu 0.17 crate: it cannot be compiled here (no
// cargo/rustc, crates not vendored, no network) and its GPU programs cannot run anywhere we have
// (no graphics stack).  It ships no tests, golden vectors or fixtures.  The restatement is therefore
// pinned only by closed-form known-answer tests (tests/test_oracle_kat.py) and by reading.  The
// following behaviours of the reference's dependencies are assumptions, not measurements:
//   * geometric_algebra 0.3.0: Rotor::signum() = component-wise multiply by 1/sqrt(sum of squares),
//     component order preserved (scene.rs:227); the camera is given as a camera-to-world 4x4
//     (what motor3d_to_mat4 returns, utils.rs:31-42) and the view matrix is its rigid inverse
//     (renderer.rs:365 uses Motor::inverse).
//   * WGSL/naga/driver float semantics: IEEE division and sqrt, no FMA contraction, left-to-right
//     evaluation, mat*vec as a column combination in column order; u32(f32) truncates and saturates
//     (NaN -> 0).  exp() is this file's own Cody–Waite/Taylor exp (o_expf below), which the CUDA
//     path implements with the same method and constants.
//   * Fixed-function raster + Bgra8Unorm blending: a pixel centre (x+0.5, y+0.5) is covered iff it
//     lies in the splat's pixel bounding box and |tc.x|,|tc.y| <= ellipse_margin (rotated rects) or
//     the axis-aligned square test (AA quads); tc is the exact affine inverse of the quad mapping
//     (what linear interpolation of gl_TexCoord gives without sub-pixel snapping).  Blending clamps
//     the source to [0,1], blends in f32 against the dequantised (k/255) destination and re-quantises
//     with round-to-nearest-even after every splat ("unorm8" mode).  "fp32" mode keeps the
//     destination in f32 and stops a pixel once T < 1e-4.
//
// Build: oracle/build_oracle.py (g++ -O2 -ffp-contract=off -fno-fast-math; no -march flags so the
// FP32 results are identical on x86-64 and aarch64).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#define OAPI extern "C" __attribute__((visibility("default")))

namespace {

// ----------------------------------------------------------------------------------------------
// exp: Cody–Waite range reduction (x = n*ln2 + r, ln2 split into a 16-bit head and a tail) and a
// degree-7 Taylor polynomial for e^r on |r| <= ln2/2, Horner with fused multiply-adds, then a
// two-factor scaling by 2^n so that every factor stays a normal number.  Used for the loader
// (scale exp, sigmoid) and the fragment falloff; the CUDA path uses the same method and constants.
// ----------------------------------------------------------------------------------------------
inline float bits_to_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline uint32_t float_to_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

float o_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return INFINITY;
    if (x < -103.97208404541015625f) return 0.0f;
    const float n = rintf(x * 1.44269502162933349609375f);
    float r = std::fmaf(n, -0.693145751953125f, x);
    r = std::fmaf(n, -1.428606765330187045e-06f, r);
    float p = 1.98412698412698412e-04f;           // 1/7!
    p = std::fmaf(p, r, 1.38888888888888889e-03f);  // 1/6!
    p = std::fmaf(p, r, 8.33333333333333333e-03f);  // 1/5!
    p = std::fmaf(p, r, 4.16666666666666667e-02f);  // 1/4!
    p = std::fmaf(p, r, 1.66666666666666667e-01f);  // 1/3!
    p = std::fmaf(p, r, 0.5f);
    p = std::fmaf(p, r, 1.0f);
    p = std::fmaf(p, r, 1.0f);
    const int ni = (int)n;
    const int h = ni / 2;
    const float s1 = bits_to_float((uint32_t)(h + 127) << 23);
    const float s2 = bits_to_float((uint32_t)(ni - h + 127) << 23);
    return (p * s1) * s2;
}

template <typename F>
struct Num;
template <>
struct Num<float> {
    static float exp(float x) { return o_expf(x); }
    static float sqrt(float x) { return std::sqrt(x); }
    static constexpr float SQRT2 = 1.41421356237309504880f;
};
template <>
struct Num<double> {
    static double exp(double x) { return std::exp(x); }
    static double sqrt(double x) { return std::sqrt(x); }
    static constexpr double SQRT2 = 1.41421356237309504880;
};

// Forward-mode dual number in FP64 (value, derivative): the FP64 reference gradient of the vertex
// stage runs the same template on it, once per input direction.
struct Dd {
    double v, d;
    Dd(double x = 0.0) : v(x), d(0.0) {}
    Dd(double x, double dx) : v(x), d(dx) {}
};
inline Dd operator+(Dd a, Dd b) { return {a.v + b.v, a.d + b.d}; }
inline Dd operator-(Dd a, Dd b) { return {a.v - b.v, a.d - b.d}; }
inline Dd operator*(Dd a, Dd b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dd operator/(Dd a, Dd b) {
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
inline Dd operator-(Dd a) { return {-a.v, -a.d}; }
inline bool operator<(Dd a, Dd b) { return a.v < b.v; }
inline bool operator>(Dd a, Dd b) { return a.v > b.v; }
template <>
struct Num<Dd> {
    static Dd sqrt(Dd x) {
        const double r = std::sqrt(x.v);
        return {r, r > 0.0 ? x.d / (2.0 * r) : 0.0};
    }
    static constexpr double SQRT2 = 1.41421356237309504880;
};
inline float o_min(float a, float b) { return std::fmin(a, b); }
inline float o_max(float a, float b) { return std::fmax(a, b); }
inline double o_min(double a, double b) { return std::fmin(a, b); }
inline double o_max(double a, double b) { return std::fmax(a, b); }
inline Dd o_min(Dd a, Dd b) { return std::fmin(a.v, b.v) == a.v ? a : b; }
inline Dd o_max(Dd a, Dd b) { return std::fmax(a.v, b.v) == a.v ? a : b; }
inline float o_abs(float a) { return std::fabs(a); }
inline double o_abs(double a) { return std::fabs(a); }
inline Dd o_abs(Dd a) { return a.v < 0.0 ? -a : a; }
inline double o_val(float a) { return a; }
inline double o_val(double a) { return a; }
inline double o_val(Dd a) { return a.v; }

// Uniform block, byte-compatible with `Uniforms` (renderer.rs:49-61; shaders.wgsl:1-11).
struct OU {
    float camera[16];  // column-major, camera-to-world
    float view[16];
    float vp[16];
    float view_size[2];
    uint32_t image_size[2];
    float tol, bias, margin, splat_scale;
};
static_assert(sizeof(OU) == 224, "uniform block is 224 bytes");

// Configuration flags the device programs are specialised on (renderer.rs:101-132).
struct OCfg {
    int32_t depth_sorting;  // 0 None, 1 Cpu, 2 Gpu, 3 GpuIndirectDraw (renderer.rs:14-23)
    int32_t use_covariance_for_scale;
    int32_t use_unaligned_rectangles;
    int32_t sh_order;
    int32_t blend_mode;  // 0 unorm8, 1 fp32
};

inline float clamp01(float x) { return std::fmin(std::fmax(x, 0.0f), 1.0f); }

// u32(f32) in WGSL: truncate toward zero, saturate, NaN -> 0.
inline uint32_t sat_u32(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)x;
}

// ---------------------------------------------------------------------------------------------
// mat3 helpers, column-major m[c*3 + r]; (A*B) column j = A * B[j] as a column combination,
// summed in column order (WGSL mat3x3 * mat3x3).
// ---------------------------------------------------------------------------------------------
template <typename F>
inline void mul3(const F* A, const F* B, F* out) {
    F t[9];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
            t[j * 3 + i] = (A[0 * 3 + i] * B[j * 3 + 0] + A[1 * 3 + i] * B[j * 3 + 1]) + A[2 * 3 + i] * B[j * 3 + 2];
    for (int k = 0; k < 9; ++k) out[k] = t[k];
}
template <typename F>
inline void transpose3(const F* A, F* out) {
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) out[c * 3 + r] = A[r * 3 + c];
}

// quatToMat (shaders.wgsl:63-79); p = (scalar, i, j, k) (scene.rs:227-231).
template <typename F>
inline void quat_to_mat(const F* p, F* m) {
    F q[4];
    for (int i = 0; i < 4; ++i) q[i] = p[i] * Num<F>::SQRT2;
    const F yy = q[1] * q[1], yz = q[1] * q[2], yw = q[1] * q[3], yx = q[1] * q[0];
    const F zz = q[2] * q[2], zw = q[2] * q[3], zx = q[2] * q[0];
    const F ww = q[3] * q[3], wx = q[3] * q[0];
    m[0] = (F(1) - zz) - ww; m[1] = yz + wx;             m[2] = yw - zx;
    m[3] = yz - wx;          m[4] = (F(1) - yy) - ww;    m[5] = zw + yx;
    m[6] = yw + zx;          m[7] = zw - yx;             m[8] = (F(1) - yy) - zz;
}

template <typename F>
inline void camera3(const OU& u, F* c) {
    for (int col = 0; col < 3; ++col)
        for (int r = 0; r < 3; ++r) c[col * 3 + r] = (F)u.camera[col * 4 + r];
}

// projectedContourOfEllipsoid (shaders.wgsl:125-169).
template <typename F>
void projected_contour(const OU& u, const F* s, const F* rot, const F* t, F* M) {
    F C[9], T[9];
    camera3(u, C);
    quat_to_mat(rot, T);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) T[c * 3 + r] = T[c * 3 + r] / s[c];
    F ro[3];
    for (int r = 0; r < 3; ++r) ro[r] = (F)u.camera[12 + r] - t[r];
    F l[3], l2[3];
    for (int i = 0; i < 3; ++i) l[i] = (ro[0] * T[i * 3 + 0] + ro[1] * T[i * 3 + 1]) + ro[2] * T[i * 3 + 2];
    for (int i = 0; i < 3; ++i) l2[i] = l[i] * l[i];
    const F dx = (F(1) - l2[1]) - l2[2], dy = (F(1) - l2[0]) - l2[2], dz = (F(1) - l2[0]) - l2[1];
    const F tx = l[1] * l[2], ty = l[0] * l[2], tz = l[0] * l[1];
    const F A[9] = {dx, tz, ty, tz, dy, tx, ty, tx, dz};
    F Ct[9], T2[9], T2t[9], TA[9];
    transpose3(C, Ct);
    mul3(Ct, T, T2);
    mul3(T2, A, TA);
    transpose3(T2, T2t);
    mul3(TA, T2t, M);
}

// projectedCovarianceOfEllipsoid (shaders.wgsl:99-118).
template <typename F>
void projected_covariance(const OU& u, const F* s, const F* rot, const F* t, F* cov) {
    F C[9], T[9];
    camera3(u, C);
    quat_to_mat(rot, T);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) T[c * 3 + r] = T[c * 3 + r] * s[c];
    F v[3];
    for (int r = 0; r < 3; ++r)
        v[r] = (((F)u.view[0 * 4 + r] * t[0] + (F)u.view[1 * 4 + r] * t[1]) + (F)u.view[2 * 4 + r] * t[2]) +
               (F)u.view[3 * 4 + r] * F(1);
    v[0] = o_min(o_max(v[0] / v[2], F(-1)), F(1)) * v[2];
    v[1] = o_min(o_max(v[1] / v[2], F(-1)), F(1)) * v[2];
    const F zz = v[2] * v[2];
    const F J[9] = {F(1) / v[2], F(0), (-v[0]) / zz, F(0), F(1) / v[2], (-v[1]) / zz, F(0), F(0), F(0)};
    F Tt[9], TC[9], Tm[9], Tmt[9];
    transpose3(T, Tt);
    mul3(Tt, C, TC);
    mul3(TC, J, Tm);
    transpose3(Tm, Tmt);
    mul3(Tmt, Tm, cov);
}

template <typename F>
inline F wgsl_sign(F x) {
    return x > F(0) ? F(1) : (x < F(0) ? F(-1) : F(0));
}

// extractTranslationOfEllipse (shaders.wgsl:179-191).
template <typename F>
void ellipse_translation(const F* M, F* t) {
    const F xx = M[0], xy = M[1], xz = M[2], yy = M[4], yz = M[5];
    const F disc = xx * yy - xy * xy;
    const F inv = F(1) / disc;
    t[0] = (xy * yz - yy * xz) * inv;
    t[1] = (xy * xz - xx * yz) * inv;
}

// extractRotationOfEllipse (shaders.wgsl:193-215).
template <typename F>
void ellipse_rotation(const F* M, F* r) {
    const F xx = M[0], xy = M[1], yy = M[4];
    const F a = (xx - yy) * (xx - yy);
    const F b = a + (F(4) * xy) * xy;
    const F c = F(0.5) * Num<F>::sqrt(a / b);
    F j = Num<F>::sqrt(F(0.5) - c);
    F k = ((-Num<F>::sqrt(F(0.5) + c)) * wgsl_sign(xy)) * wgsl_sign(xx - yy);
    if (xy < F(0) || xx - yy < F(0)) {
        k = -k;
        j = -j;
    }
    if (xx - yy < F(0)) {
        const F tmp = j;
        j = -k;
        k = tmp;
    }
    r[0] = j;
    r[1] = k;
}

// extractScaleOfEllipse (shaders.wgsl:217-237).
template <typename F>
void ellipse_scale(const F* M, const F* t, const F* r, F* out) {
    const F xx = M[0], xy = M[1], yy = M[4], zz = M[8];
    const F d = ((F(2) * xy) * r[0]) * r[1];
    const F e = zz - (((xx * t[0]) * t[0] + (yy * t[1]) * t[1]) + ((F(2) * xy) * t[0]) * t[1]);
    out[0] = Num<F>::sqrt(o_abs(e / (((xx * r[1]) * r[1] + (yy * r[0]) * r[0]) - d)));
    out[1] = Num<F>::sqrt(o_abs(e / (((xx * r[0]) * r[0] + (yy * r[1]) * r[1]) + d)));
}

// extractScaleOfCovariance (shaders.wgsl:240-246).
template <typename F>
void covariance_scale(const F* M, F* out) {
    const F xx = M[0], xy = M[1], yy = M[4];
    const F a = (xx - yy) * (xx - yy);
    const F b = Num<F>::sqrt(a + (F(4) * xy) * xy);
    out[0] = Num<F>::sqrt(((xx + yy) + b) * F(0.5));
    out[1] = Num<F>::sqrt(((xx + yy) - b) * F(0.5));
}

// Spherical-harmonics constants (shaders.wgsl:249-266), rounded to f32 like the WGSL literals
// (SHC_F) and kept in double for the FP64 instance (SHC_D).
const float SHC_F[16] = {
    0.28209479177387814f,  -0.4886025119029199f, 0.4886025119029199f,  -0.4886025119029199f,
    1.0925484305920792f,   -1.0925484305920792f, 0.31539156525252005f, -1.0925484305920792f,
    0.5462742152960396f,   -0.5900435899266435f, 2.890611442640554f,   -0.4570457994644658f,
    0.3731763325901154f,   -0.4570457994644658f, 1.445305721320277f,   -0.5900435899266435f,
};
const double SHC_D[16] = {
    0.28209479177387814,  -0.4886025119029199, 0.4886025119029199,  -0.4886025119029199,
    1.0925484305920792,   -1.0925484305920792, 0.31539156525252005, -1.0925484305920792,
    0.5462742152960396,   -0.5900435899266435, 2.890611442640554,   -0.4570457994644658,
    0.3731763325901154,   -0.4570457994644658, 1.445305721320277,   -0.5900435899266435,
};
template <typename F>
inline F shc(int i);
template <>
inline float shc<float>(int i) { return SHC_F[i]; }
template <>
inline double shc<double>(int i) { return SHC_D[i]; }
template <>
inline Dd shc<Dd>(int i) { return Dd(SHC_D[i]); }

template <typename F>
void sh_lookup(const F* d, const F* sh, int order, F* rgb) {
    F k[16];
    for (int i = 0; i < 16; ++i) k[i] = shc<F>(i);
    const F x = d[0], y = d[1], z = d[2];
    const F xx = x * x, yy = y * y, zz = z * z;
    for (int c = 0; c < 3; ++c) {
        F col = F(0.5);
        col = col + k[0] * sh[c];
        if (order > 0) {
            col = col + (k[1] * sh[3 + c]) * y;
            col = col + (k[2] * sh[6 + c]) * z;
            col = col + (k[3] * sh[9 + c]) * x;
        }
        if (order > 1) {
            col = col + ((k[4] * sh[12 + c]) * x) * y;
            col = col + ((k[5] * sh[15 + c]) * y) * z;
            col = col + (k[6] * sh[18 + c]) * ((F(2) * zz - xx) - yy);
            col = col + ((k[7] * sh[21 + c]) * x) * z;
            col = col + (k[8] * sh[24 + c]) * (xx - yy);
        }
        if (order > 2) {
            col = col + ((k[9] * sh[27 + c]) * y) * (F(3) * xx - yy);
            col = col + (((k[10] * sh[30 + c]) * x) * y) * z;
            col = col + ((k[11] * sh[33 + c]) * y) * ((F(4) * zz - xx) - yy);
            col = col + ((k[12] * sh[36 + c]) * z) * ((F(2) * zz - F(3) * xx) - F(3) * yy);
            col = col + ((k[13] * sh[39 + c]) * x) * ((F(4) * zz - xx) - yy);
            col = col + ((k[14] * sh[42 + c]) * z) * (xx - yy);
            col = col + ((k[15] * sh[45 + c]) * x) * (xx - F(3) * yy);
        }
        rgb[c] = col;
    }
}

// Per-splat result of the vertex stage (shaders.wgsl:507-573), restated as the data a compute
// rasteriser needs.  Record layout (16 floats) is identical to the CUDA path's:
//   [A00 A01 B0 A10 | A11 B1 alpha bbox_lo | r g b bbox_hi | bx by R 0]
// where tc = (A00*X + A01*Y + B0, A10*X + A11*Y + B1) for the pixel centre (X, Y), bbox_lo/hi pack
// the inclusive pixel bounding box as (x | y<<16) and (bx, by, R) are the AA-square test.
template <typename F>
struct Dbg {
    F M[9];
    F t[2], r[2], axes[2], rgb[3];
};

// What the vertex stage derives from one splat (the quantities the raster and the gradients use).
template <typename F>
struct VOut {
    F A00, A01, B0, A10, A11, B1;  // tc = A (X, Y) + B at the pixel centre (X, Y)
    F rgb[3];
    F Xx, Xy, Yx, Yy, Zx, Zy;      // rect basis and centre in view-plane units
    F bx, by;                      // AA-square offsets
    Dbg<F> dbg;
};

// The vertex stage (shaders.wgsl:507-573) restated; scale is the splat's scale before splat_scale.
template <typename F>
void vertex_core(const OU& u, const OCfg& cfg, const F* c, const F* q, const F* scale, const F* shf, VOut<F>& o) {
    F se[3];
    for (int i = 0; i < 3; ++i) se[i] = scale[i] * (F)u.splat_scale;
    // colour (shaders.wgsl:531-532)
    F v[3];
    for (int i = 0; i < 3; ++i) v[i] = c[i] - (F)u.camera[12 + i];
    const F len = Num<F>::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    F d[3] = {v[0] / len, v[1] / len, v[2] / len};
    sh_lookup(d, shf, cfg.sh_order, o.rgb);
    // conic and its decomposition (shaders.wgsl:533-542)
    F M[9], t[2], r[2], axes[2];
    projected_contour(u, se, q, c, M);
    ellipse_translation(M, t);
    ellipse_rotation(M, r);
    if (cfg.use_covariance_for_scale) {
        F cov[9];
        projected_covariance(u, se, q, c, cov);
        covariance_scale(cov, axes);
    } else {
        ellipse_scale(M, t, r, axes);
    }
    for (int i = 0; i < 9; ++i) o.dbg.M[i] = M[i];
    o.dbg.t[0] = t[0]; o.dbg.t[1] = t[1];
    o.dbg.r[0] = r[0]; o.dbg.r[1] = r[1];
    o.dbg.axes[0] = axes[0]; o.dbg.axes[1] = axes[1];
    for (int i = 0; i < 3; ++i) o.dbg.rgb[i] = o.rgb[i];
    // rect basis (shaders.wgsl:543-547)
    const F bias = (F)u.bias;
    const F sa = bias + axes[0], sb = bias + axes[1];
    o.Xx = r[1] * sa; o.Xy = (-r[0]) * sa;
    o.Yx = r[0] * sb; o.Yy = r[1] * sb;
    o.Zx = t[0]; o.Zy = t[1];
    // inverse of the 2x2 basis (shaders.wgsl:563-566), folded with pixel -> view-plane mapping
    const F det = o.Xx * o.Yy - o.Xy * o.Yx;
    const F idet = F(1) / det;
    const F i00 = o.Yy * idet, i01 = (-o.Yx) * idet, i10 = (-o.Xy) * idet, i11 = o.Xx * idet;
    const F vw = (F)u.view_size[0], vh = (F)u.view_size[1];
    const F Wf = (F)u.image_size[0], Hf = (F)u.image_size[1];
    const F sx = (F(2) * vw) / Wf, sy = -((F(2) * vh) / Hf);
    o.bx = (-vw) - o.Zx;
    o.by = vh - o.Zy;
    o.A00 = i00 * sx; o.A01 = i01 * sy; o.B0 = i00 * o.bx + i01 * o.by;
    o.A10 = i10 * sx; o.A11 = i11 * sy; o.B1 = i10 * o.bx + i11 * o.by;
}

template <typename F>
bool preprocess_one(const OU& u, const OCfg& cfg, const float* center, const float* rot, const float* scale,
                    float alpha, const float* sh, float* rec, Dbg<F>* dbg) {
    F c[3] = {(F)center[0], (F)center[1], (F)center[2]};
    F q[4] = {(F)rot[0], (F)rot[1], (F)rot[2], (F)rot[3]};
    F sc[3] = {(F)scale[0], (F)scale[1], (F)scale[2]};
    F shf[48];
    const int nsh = 3 * (cfg.sh_order + 1) * (cfg.sh_order + 1);
    for (int i = 0; i < nsh; ++i) shf[i] = (F)sh[i];
    VOut<F> o;
    vertex_core(u, cfg, c, q, sc, shf, o);
    if (dbg) *dbg = o.dbg;
    const F Xx = o.Xx, Xy = o.Xy, Yx = o.Yx, Yy = o.Yy, Zx = o.Zx, Zy = o.Zy;
    const F A00 = o.A00, A01 = o.A01, B0 = o.B0, A10 = o.A10, A11 = o.A11, B1 = o.B1, bx = o.bx, by = o.by;
    const F* rgb = o.rgb;
    const F vw = (F)u.view_size[0], vh = (F)u.view_size[1];
    const F Wf = (F)u.image_size[0], Hf = (F)u.image_size[1];
    const F sx = (F(2) * vw) / Wf, sy = -((F(2) * vh) / Hf);
    const F m = (F)u.margin;
    F ex, ey, R = F(0);
    if (cfg.use_unaligned_rectangles) {
        ex = m * (std::fabs(Xx) + std::fabs(Yx));
        ey = m * (std::fabs(Xy) + std::fabs(Yy));
    } else {
        R = Num<F>::sqrt(std::fmax(Xx * Xx + Xy * Xy, Yx * Yx + Yy * Yy)) * m;
        ex = R;
        ey = R;
    }
    const F cxp = (Zx + vw) / sx, exp_ = ex / sx;
    const F cyp = (Zy - vh) / sy, eyp = ey / (-sy);
    // pixels whose centre (p + 0.5) lies in the exact box, widened by 1/64 px against rounding
    const F eps = (F)0.015625f;
    const F fx0 = std::ceil(((cxp - exp_) - eps) - F(0.5)), fx1 = std::floor(((cxp + exp_) + eps) - F(0.5));
    const F fy0 = std::ceil(((cyp - eyp) - eps) - F(0.5)), fy1 = std::floor(((cyp + eyp) + eps) - F(0.5));
    const F al = (F)alpha;
    bool ok = std::isfinite(A00) && std::isfinite(A01) && std::isfinite(B0) && std::isfinite(A10) &&
              std::isfinite(A11) && std::isfinite(B1) && std::isfinite(rgb[0]) && std::isfinite(rgb[1]) &&
              std::isfinite(rgb[2]) && std::isfinite(fx0) && std::isfinite(fx1) && std::isfinite(fy0) &&
              std::isfinite(fy1) && std::isfinite(R) && std::isfinite(bx) && std::isfinite(by) &&
              (al >= (F)(1.0f / 255.0f));
    int x0 = 0, x1 = -1, y0 = 0, y1 = -1;
    if (ok) {
        const F xmax = Wf - F(1), ymax = Hf - F(1);
        const F cx0 = std::fmax(fx0, F(0)), cx1 = std::fmin(fx1, xmax);
        const F cy0 = std::fmax(fy0, F(0)), cy1 = std::fmin(fy1, ymax);
        if (cx0 <= cx1 && cy0 <= cy1) {
            x0 = (int)cx0; x1 = (int)cx1; y0 = (int)cy0; y1 = (int)cy1;
        } else {
            ok = false;
        }
    }
    uint32_t lo = 0xFFFFFFFFu, hi = 0u;  // empty box
    if (ok) {
        lo = (uint32_t)x0 | ((uint32_t)y0 << 16);
        hi = (uint32_t)x1 | ((uint32_t)y1 << 16);
    }
    rec[0] = (float)A00; rec[1] = (float)A01; rec[2] = (float)B0; rec[3] = (float)A10;
    rec[4] = (float)A11; rec[5] = (float)B1; rec[6] = alpha; rec[7] = bits_to_float(lo);
    rec[8] = (float)rgb[0]; rec[9] = (float)rgb[1]; rec[10] = (float)rgb[2]; rec[11] = bits_to_float(hi);
    if (cfg.use_unaligned_rectangles) {
        rec[12] = 0.0f; rec[13] = 0.0f; rec[14] = 0.0f;
    } else {
        rec[12] = (float)bx; rec[13] = (float)by; rec[14] = (float)R;
    }
    rec[15] = 0.0f;
    return ok;
}

// worldToClipSpace + isInFrustum + key (shaders.wgsl:54-61, 318-324).
inline void clip_gpu(const OU& u, float x, float y, float z, float* c) {
    float h[4];
    for (int r = 0; r < 4; ++r)
        h[r] = ((u.vp[0 * 4 + r] * x + u.vp[1 * 4 + r] * y) + u.vp[2 * 4 + r] * z) + u.vp[3 * 4 + r] * 1.0f;
    const float den = h[3] + 1e-7f;
    c[0] = h[0] / den;
    c[1] = h[1] / den;
    c[2] = h[2] / den;
}
inline bool in_frustum(const OU& u, const float* c) {
    return std::fabs(c[0]) < u.tol && std::fabs(c[1]) < u.tol && std::fabs(c[2] - 0.5f) < 0.5f;
}
inline uint32_t gpu_key(const float* c) {
    uint32_t key = sat_u32(c[2] * 65535.0f) << 16;
    key |= sat_u32((c[0] * 0.5f + 0.5f) * 255.0f) << 8;
    key |= sat_u32((c[1] * 0.5f + 0.5f) * 255.0f);
    return key;
}
// CPU depth-sort fallback rule (renderer.rs:372-392): reciprocal multiply, no epsilon, key = bits(z).
inline bool cpu_rule(const OU& u, float x, float y, float z, uint32_t* key) {
    float h[4];
    for (int r = 0; r < 4; ++r)
        h[r] = ((u.vp[0 * 4 + r] * x + u.vp[1 * 4 + r] * y) + u.vp[2 * 4 + r] * z) + u.vp[3 * 4 + r] * 1.0f;
    const float rw = 1.0f / h[3];
    const float c[3] = {h[0] * rw, h[1] * rw, h[2] * rw};
    *key = float_to_bits(c[2]);
    return std::fabs(c[0]) < u.tol && std::fabs(c[1]) < u.tol && std::fabs(c[2] - 0.5f) < 0.5f;
}

template <typename Fn>
void parallel_for(int64_t n, int threads, Fn fn) {
    if (threads <= 1 || n < 4096) {
        fn(0, n);
        return;
    }
    std::vector<std::thread> pool;
    const int64_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        pool.emplace_back([=] { fn(b, e); });
    }
    for (auto& th : pool) th.join();
}

float g_lut[256];
struct LutInit {
    LutInit() {
        for (int k = 0; k < 256; ++k) g_lut[k] = (float)k / 255.0f;
    }
} g_lut_init;

const float FP32_T_MIN = 1e-4f;
const float ALPHA_MIN = 1.0f / 255.0f;

// Rasterise the ordered draw list into one 16x16 tile (fragment + blend, shaders.wgsl:580-592,
// renderer.rs:260-271; clear renderer.rs:441-442).  With COUNT the tile is not written; work[0..2]
// gain the tile's (pixel, record) pairs with the pixel inside the record's pixel box, those whose
// pixel centre also passes the coverage test (every pair, also after the pixel has finished), and
// the blend steps the pixel performs (coverage, alpha >= 1/255, before it finishes).
template <bool COUNT>
void raster_tile(const OU& u, const OCfg& cfg, const float* recs, const uint32_t* list, size_t nlist, int tx, int ty,
                 void* out, uint64_t* work = nullptr) {
    const int W = (int)u.image_size[0], H = (int)u.image_size[1];
    const float m = u.margin;
    for (int py = ty * 16; py < std::min(H, ty * 16 + 16); ++py) {
        for (int px = tx * 16; px < std::min(W, tx * 16 + 16); ++px) {
            const float X = (float)px + 0.5f, Y = (float)py + 0.5f;
            int cr = 0, cg = 0, cb = 0, ta = 255;
            float fr = 0.f, fg = 0.f, fb = 0.f, ft = 1.f;
            bool finished = false;
            for (size_t li = 0; li < nlist; ++li) {
                const float* rc = recs + (size_t)list[li] * 16;
                const uint32_t lo = float_to_bits(rc[7]), hi = float_to_bits(rc[11]);
                const int x0 = (int)(lo & 0xFFFFu), y0 = (int)(lo >> 16), x1 = (int)(hi & 0xFFFFu), y1 = (int)(hi >> 16);
                if (px < x0 || px > x1 || py < y0 || py > y1) continue;
                if (COUNT) ++work[0];
                const float tcx = std::fmaf(rc[1], Y, std::fmaf(rc[0], X, rc[2]));
                const float tcy = std::fmaf(rc[4], Y, std::fmaf(rc[3], X, rc[5]));
                if (cfg.use_unaligned_rectangles) {
                    if (!(std::fabs(tcx) <= m && std::fabs(tcy) <= m)) continue;
                } else {
                    const float sx = (2.0f * u.view_size[0]) / (float)W;
                    const float sy = -((2.0f * u.view_size[1]) / (float)H);
                    const float dx = std::fmaf(sx, X, rc[12]), dy = std::fmaf(sy, Y, rc[13]);
                    if (!(std::fabs(dx) <= rc[14] && std::fabs(dy) <= rc[14])) continue;
                }
                if (COUNT) {
                    ++work[1];
                    if (finished) continue;
                }
                const float power = std::fmaf(tcx, tcx, tcy * tcy);
                const float alpha = rc[6] * o_expf(-0.5f * power);
                if (alpha < ALPHA_MIN) continue;
                if (COUNT) ++work[2];
                const float sr = clamp01(rc[8] * alpha), sg = clamp01(rc[9] * alpha), sb = clamp01(rc[10] * alpha);
                const float sa = clamp01(alpha);
                if (cfg.blend_mode == 0) {
                    const float dA = g_lut[ta];
                    cr = (int)rintf(clamp01(sr * dA + g_lut[cr]) * 255.0f);
                    cg = (int)rintf(clamp01(sg * dA + g_lut[cg]) * 255.0f);
                    cb = (int)rintf(clamp01(sb * dA + g_lut[cb]) * 255.0f);
                    ta = (int)rintf(clamp01(dA * (1.0f - sa)) * 255.0f);
                    finished = ta == 0;
                } else {
                    fr = sr * ft + fr;
                    fg = sg * ft + fg;
                    fb = sb * ft + fb;
                    ft = ft * (1.0f - sa);
                    finished = ft < FP32_T_MIN;
                }
                if (!COUNT && finished) break;
            }
            if (COUNT) continue;
            const size_t pix = (size_t)py * W + px;
            if (cfg.blend_mode == 0) {
                uint8_t* o = (uint8_t*)out + pix * 4;
                o[0] = (uint8_t)cr; o[1] = (uint8_t)cg; o[2] = (uint8_t)cb; o[3] = (uint8_t)ta;
            } else {
                float* o = (float*)out + pix * 4;
                o[0] = fr; o[1] = fg; o[2] = fb; o[3] = ft;
            }
        }
    }
}

}  // namespace

// =============================================================================================
// C API (ctypes)
// =============================================================================================

OAPI int oracle_version() { return 1; }

OAPI float oracle_expf(float x) { return o_expf(x); }

// Uniforms for a frame (renderer.rs:364-409, utils.rs:45-70), with the documented extension
// `field_of_view_y` (reference hard-codes pi/2, renderer.rs:366) and view_width = aspect*view_height
// (equal to the reference's aspect/view_height at pi/2, where view_height == 1).
OAPI void oracle_uniforms(const float* cam, uint32_t W, uint32_t H, float fovy, float tol, float margin,
                          float splat_scale, void* out) {
    OU u;
    std::memcpy(u.camera, cam, 64);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) u.view[c * 4 + r] = cam[r * 4 + c];
    for (int r = 0; r < 3; ++r)
        u.view[12 + r] = -((cam[r * 4 + 0] * cam[12] + cam[r * 4 + 1] * cam[13]) + cam[r * 4 + 2] * cam[14]);
    u.view[3] = 0.0f; u.view[7] = 0.0f; u.view[11] = 0.0f; u.view[15] = 1.0f;
    const float half = fovy * 0.5f;
    const float vh = (float)std::tan((double)half);
    const float aspect = (float)W / (float)H;
    const float vw = aspect * vh;
    const float nearp = 1.0f, farp = 1000.0f;
    const float den = 1.0f / (nearp - farp);
    const float P[16] = {1.0f / vw, 0, 0, 0, 0, 1.0f / vh, 0, 0, 0, 0, -farp * den, 1.0f, 0, 0, nearp * farp * den, 0};
    for (int i = 0; i < 4; ++i)
        for (int r = 0; r < 4; ++r)
            u.vp[i * 4 + r] = ((P[0 * 4 + r] * u.view[i * 4 + 0] + P[1 * 4 + r] * u.view[i * 4 + 1]) +
                               P[2 * 4 + r] * u.view[i * 4 + 2]) +
                              P[3 * 4 + r] * u.view[i * 4 + 3];
    u.view_size[0] = vw;
    u.view_size[1] = vh;
    u.image_size[0] = W;
    u.image_size[1] = H;
    u.tol = tol;
    u.bias = (0.2f * vw) / (float)W;
    u.margin = margin;
    u.splat_scale = splat_scale;
    std::memcpy(out, &u, sizeof(u));
}

// Cull + key per splat.  mode 1 = CPU rule (renderer.rs:372-392), else the GPU rule
// (radixSortA, shaders.wgsl:318-324).  keys[i] = 0xFFFFFFFF for culled splats in GPU mode.
OAPI void oracle_cull_keys(const void* uni, int mode, const float* centers, uint64_t n, uint32_t* keys,
                           uint8_t* visible) {
    const OU& u = *(const OU*)uni;
    for (uint64_t i = 0; i < n; ++i) {
        const float* p = centers + 3 * i;
        if (mode == 1) {
            uint32_t k;
            const bool v = cpu_rule(u, p[0], p[1], p[2], &k);
            keys[i] = k;
            visible[i] = v;
        } else {
            float c[3];
            clip_gpu(u, p[0], p[1], p[2], c);
            const bool v = in_frustum(u, c);
            keys[i] = v ? gpu_key(c) : 0xFFFFFFFFu;
            visible[i] = v;
        }
    }
}

// Ordered draw list for a depth-sorting mode.  entries_key/entries_index receive the visible
// splats (stable-sorted by key for Cpu/Gpu/GpuIndirectDraw, index order for None); *n_visible and
// *n_draw receive V and the number of entries actually drawn:
//   None, Cpu: V;  Gpu: entries whose key != 0xFFFFFFFF (vertex stage discard, shaders.wgsl:520);
//   GpuIndirectDraw: entries whose top key byte != 0xFF (instance count, shaders.wgsl:458-461).
OAPI void oracle_draw_list(const void* uni, int mode, const float* centers, uint64_t n, uint32_t* entries_key,
                           uint32_t* entries_index, uint64_t* n_visible, uint64_t* n_draw) {
    std::vector<uint32_t> keys(n);
    std::vector<uint8_t> vis(n);
    oracle_cull_keys(uni, mode, centers, n, keys.data(), vis.data());
    std::vector<std::pair<uint32_t, uint32_t>> e;
    e.reserve(n);
    for (uint64_t i = 0; i < n; ++i)
        if (vis[i]) e.emplace_back(keys[i], (uint32_t)i);
    if (mode != 0)
        std::stable_sort(e.begin(), e.end(),
                         [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
                             return a.first < b.first;
                         });
    uint64_t draw = e.size();
    if (mode == 2) {
        draw = 0;
        for (auto& p : e) draw += p.first != 0xFFFFFFFFu;
    } else if (mode == 3) {
        draw = 0;
        for (auto& p : e) draw += (p.first >> 24) != 0xFFu;
    }
    for (size_t i = 0; i < e.size(); ++i) {
        entries_key[i] = e[i].first;
        entries_index[i] = e[i].second;
    }
    *n_visible = e.size();
    *n_draw = draw;
}

// Vertex-stage restatement for a list of splat indices.  recs: 16 floats per entry (layout above);
// dbg (optional): 18 values per entry = M[9], t[2], rot[2], axes[2], rgb[3].  Returns #valid.
template <typename F>
static uint64_t preprocess_impl(const void* uni, const OCfg* cfg, const float* centers, const float* rots,
                                const float* scales, const float* alphas, const float* shs, const uint32_t* idx,
                                uint64_t n, float* recs, F* dbg, int threads) {
    const OU& u = *(const OU*)uni;
    std::atomic<uint64_t> valid{0};
    parallel_for((int64_t)n, threads, [&](int64_t b, int64_t e) {
        uint64_t v = 0;
        for (int64_t i = b; i < e; ++i) {
            const uint32_t s = idx[i];
            Dbg<F> d;
            v += preprocess_one<F>(u, *cfg, centers + 3 * (size_t)s, rots + 4 * (size_t)s, scales + 3 * (size_t)s,
                                   alphas[s], shs + 48 * (size_t)s, recs + 16 * (size_t)i, dbg ? &d : nullptr);
            if (dbg) {
                F* o = dbg + 18 * (size_t)i;
                for (int k = 0; k < 9; ++k) o[k] = d.M[k];
                o[9] = d.t[0]; o[10] = d.t[1]; o[11] = d.r[0]; o[12] = d.r[1];
                o[13] = d.axes[0]; o[14] = d.axes[1];
                o[15] = d.rgb[0]; o[16] = d.rgb[1]; o[17] = d.rgb[2];
            }
        }
        valid += v;
    });
    return valid.load();
}

OAPI uint64_t oracle_preprocess_f32(const void* uni, const void* cfg, const float* centers, const float* rots,
                                    const float* scales, const float* alphas, const float* shs, const uint32_t* idx,
                                    uint64_t n, float* recs, float* dbg, int threads) {
    return preprocess_impl<float>(uni, (const OCfg*)cfg, centers, rots, scales, alphas, shs, idx, n, recs, dbg,
                                  threads);
}
OAPI uint64_t oracle_preprocess_f64(const void* uni, const void* cfg, const float* centers, const float* rots,
                                    const float* scales, const float* alphas, const float* shs, const uint32_t* idx,
                                    uint64_t n, float* recs, double* dbg, int threads) {
    return preprocess_impl<double>(uni, (const OCfg*)cfg, centers, rots, scales, alphas, shs, idx, n, recs, dbg,
                                   threads);
}

// Rasterise records (16 floats each, in draw order) into out (RGBA8 for unorm8, float4 for fp32).
// tile_stride > 1 renders only every tile_stride-th 16x16 tile (a bounded sample for timing).  With
// work != nullptr nothing is rendered and work[0..2] receive raster_tile<true>'s counts.
static void raster_impl(const void* uni, const void* cfgp, const float* recs, uint64_t n, void* out, int threads,
                        int tile_stride, uint64_t* work = nullptr);
OAPI void oracle_raster(const void* uni, const void* cfgp, const float* recs, uint64_t n, void* out, int threads) {
    raster_impl(uni, cfgp, recs, n, out, threads, 1);
}
// The raster's work for a frame's records: work[0] (pixel, record) pairs inside the records' pixel
// boxes, work[1] of those whose pixel centre passes the coverage test, work[2] blend steps performed.
OAPI void oracle_raster_work(const void* uni, const void* cfgp, const float* recs, uint64_t n, int threads,
                             uint64_t* work) {
    work[0] = work[1] = work[2] = 0;
    raster_impl(uni, cfgp, recs, n, nullptr, threads, 1, work);
}
static void raster_impl(const void* uni, const void* cfgp, const float* recs, uint64_t n, void* out, int threads,
                        int tile_stride, uint64_t* work) {
    const OU& u = *(const OU*)uni;
    const OCfg& cfg = *(const OCfg*)cfgp;
    const int W = (int)u.image_size[0], H = (int)u.image_size[1];
    const int TX = (W + 15) / 16, TY = (H + 15) / 16;
    std::vector<std::vector<uint32_t>> lists((size_t)TX * TY);
    for (uint64_t i = 0; i < n; ++i) {
        const float* rc = recs + 16 * i;
        const uint32_t lo = float_to_bits(rc[7]), hi = float_to_bits(rc[11]);
        const int x0 = (int)(lo & 0xFFFFu), y0 = (int)(lo >> 16), x1 = (int)(hi & 0xFFFFu), y1 = (int)(hi >> 16);
        if (x0 > x1 || y0 > y1) continue;
        for (int ty = y0 / 16; ty <= y1 / 16; ++ty)
            for (int tx = x0 / 16; tx <= x1 / 16; ++tx) lists[(size_t)ty * TX + tx].push_back((uint32_t)i);
    }
    std::atomic<int64_t> next{0};
    std::atomic<uint64_t> total[3] = {{0}, {0}, {0}};
    auto worker = [&] {
        uint64_t mine[3] = {0, 0, 0};
        for (;;) {
            const int64_t t = next.fetch_add(1) * (int64_t)tile_stride;
            if (t >= (int64_t)TX * TY) break;
            if (work)
                raster_tile<true>(u, cfg, recs, lists[t].data(), lists[t].size(), (int)(t % TX), (int)(t / TX), out,
                                  mine);
            else
                raster_tile<false>(u, cfg, recs, lists[t].data(), lists[t].size(), (int)(t % TX), (int)(t / TX), out);
        }
        for (int k = 0; k < 3; ++k) total[k] += mine[k];
    };
    if (threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
        for (auto& th : pool) th.join();
    }
    if (work)
        for (int k = 0; k < 3; ++k) work[k] = total[k];
}

OAPI uint64_t oracle_cpu_sort_fallback(const void* uni, const float* positions, uint64_t n, uint32_t* entries);

// Whole frame: cull/key, draw list, vertex stage (FP32), raster.  Returns the number of drawn
// entries; stats[0..2] = V, n_draw, n_valid_records.
OAPI uint64_t oracle_render(const void* uni, const void* cfgp, const float* centers, const float* rots,
                            const float* scales, const float* alphas, const float* shs, uint64_t n, void* out,
                            int threads, uint64_t* stats) {
    const OCfg& cfg = *(const OCfg*)cfgp;
    std::vector<uint32_t> ek(n), ei(n);
    uint64_t nv = 0, nd = 0;
    oracle_draw_list(uni, cfg.depth_sorting, centers, n, ek.data(), ei.data(), &nv, &nd);
    std::vector<float> recs(16 * (size_t)nd);
    const uint64_t valid = preprocess_impl<float>(uni, &cfg, centers, rots, scales, alphas, shs, ei.data(), nd,
                                                  recs.data(), (float*)nullptr, threads);
    oracle_raster(uni, cfgp, recs.data(), nd, out, threads);
    if (stats) {
        stats[0] = nv;
        stats[1] = nd;
        stats[2] = valid;
    }
    return nd;
}

// The reference's CPU path for one frame, timed by stage (seconds): [0] CPU depth-sort fallback
// (cull + key + stable sort, single-threaded like renderer.rs:372-395), [1] vertex stage over the
// drawn entries (threads), [2] raster of every tile_stride-th tile (threads).
OAPI uint64_t oracle_cpu_frame_timed(const void* uni, const void* cfgp, const float* centers, const float* rots,
                                     const float* scales, const float* alphas, const float* shs, uint64_t n,
                                     void* out, int threads, int tile_stride, double* seconds) {
    using clk = std::chrono::steady_clock;
    const OCfg& cfg = *(const OCfg*)cfgp;
    auto t0 = clk::now();
    std::vector<uint32_t> ent(2 * (size_t)n + 2);
    const uint64_t v = oracle_cpu_sort_fallback(uni, centers, n, ent.data());
    std::vector<uint32_t> ei(v);
    for (uint64_t i = 0; i < v; ++i) ei[i] = ent[2 * i + 1];
    auto t1 = clk::now();
    std::vector<float> recs(16 * (size_t)v + 16);
    preprocess_impl<float>(uni, &cfg, centers, rots, scales, alphas, shs, ei.data(), v, recs.data(), (float*)nullptr,
                           threads);
    auto t2 = clk::now();
    raster_impl(uni, cfgp, recs.data(), v, out, threads, tile_stride < 1 ? 1 : tile_stride);
    auto t3 = clk::now();
    seconds[0] = std::chrono::duration<double>(t1 - t0).count();
    seconds[1] = std::chrono::duration<double>(t2 - t1).count();
    seconds[2] = std::chrono::duration<double>(t3 - t2).count();
    return v;
}

// Scene::load_chunk transform (scene.rs:225-250) from 62-float PLY records (scene.rs:15-24):
// [center 3 | normal 3 | colour 48 | alpha-logit | log-scale 3 | rotation 4].
OAPI void oracle_load_transform(const float* records, uint64_t n, float* centers, float* rots, float* scales,
                                float* alphas, float* shs) {
    const float MAX_SIZE_VARIANCE = 5.0f;  // scene.rs:13
    for (uint64_t i = 0; i < n; ++i) {
        const float* s = records + 62 * i;
        const float* q = s + 58;
        const float inv = 1.0f / std::sqrt(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
        for (int k = 0; k < 4; ++k) rots[4 * i + k] = q[k] * inv;
        for (int k = 0; k < 3; ++k) centers[3 * i + k] = s[k];
        const float* ls = s + 55;
        const float avg = ((ls[0] + ls[1]) + ls[2]) / 3.0f;
        for (int k = 0; k < 3; ++k)
            scales[3 * i + k] = o_expf(std::fmin(std::fmax(ls[k], avg - MAX_SIZE_VARIANCE), avg + MAX_SIZE_VARIANCE));
        alphas[i] = 1.0f / (1.0f + o_expf(-s[54]));
        std::memcpy(shs + 48 * i, s + 6, 48 * sizeof(float));
    }
}

// The reference's CPU depth-sort fallback (renderer.rs:372-395) as the timed CPU baseline: cull with
// the CPU rule, key = bits(z_clip), stable sort (Rust sort_by is stable).  Single-threaded, as in
// the reference.  Returns the number of entries written.
OAPI uint64_t oracle_cpu_sort_fallback(const void* uni, const float* positions, uint64_t n, uint32_t* entries) {
    const OU& u = *(const OU*)uni;
    std::vector<std::pair<uint32_t, uint32_t>> e;
    e.reserve(n);
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t k;
        if (cpu_rule(u, positions[3 * i], positions[3 * i + 1], positions[3 * i + 2], &k)) e.emplace_back(k, (uint32_t)i);
    }
    std::stable_sort(e.begin(), e.end(),
                     [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
                         return a.first < b.first;
                     });
    for (size_t i = 0; i < e.size(); ++i) {
        entries[2 * i] = e[i].first;
        entries[2 * i + 1] = e[i].second;
    }
    return e.size();
}

// =============================================================================================
// FP64 reference gradients and finite differences for the backward pass (test infrastructure).
//
// The differentiable function is the fp32 blend mode of the frame above, evaluated in FP64:
// L = sum over pixels and RGB of (C - target)^2, with the depth order fixed by the FP32 keys of the
// splat centres (as on the GPU).  Parameters per splat (59): centre 3, rotation 4 (used as given),
// scale 3 (before splat_scale), opacity 1, SH 48.
//   * oracle_grad_loss: full-frame loss and the analytic FP64 gradient — compositing backward
//     back-to-front (suffix sums, no recomputation) and the vertex stage through FP64 dual numbers.
//   * oracle_grad_fd: central difference of the loss in one parameter, re-rendering only the tiles
//     the splat touches; returns 0 (excluded) when the perturbation changes anything discrete: the
//     depth key, the set of tiles, or any pixel's list of contributing splats (coverage edge, 1/255
//     discard, early stop).
// =============================================================================================
namespace {

constexpr int NPARAM = 59;

struct GRec {
    double A00, A01, B0, A10, A11, B1, a, rgb[3], bx, by, R;
    int x0, y0, x1, y1;  // inclusive pixel box; x0 > x1 when empty
    bool valid;
};

struct GradCtx {
    OU u;
    OCfg cfg;
    int W, H, TX, TY;
    size_t n;
    std::vector<double> c, q, s, a, sh, target;
    std::vector<double> gimg;  // when set: dL/dC per pixel and channel used by the backward instead of 2 (C - target)
    std::vector<uint32_t> order, key;   // drawn splats in depth order, and their FP32 keys
    std::vector<int64_t> pos_of;        // splat -> draw position (-1: not drawn)
    std::vector<GRec> rec;              // per draw position
    std::vector<std::vector<uint32_t>> tiles;  // per tile: draw positions, ascending
};

GRec make_rec(const GradCtx& g, const double* c, const double* q, const double* s, double a, const double* sh) {
    VOut<double> o;
    double shf[48];
    const int nsh = 3 * (g.cfg.sh_order + 1) * (g.cfg.sh_order + 1);
    for (int i = 0; i < 48; ++i) shf[i] = i < nsh ? sh[i] : 0.0;
    vertex_core<double>(g.u, g.cfg, c, q, s, shf, o);
    GRec r{};
    r.A00 = o.A00; r.A01 = o.A01; r.B0 = o.B0; r.A10 = o.A10; r.A11 = o.A11; r.B1 = o.B1;
    r.a = a;
    for (int i = 0; i < 3; ++i) r.rgb[i] = o.rgb[i];
    r.bx = o.bx; r.by = o.by;
    const double vw = g.u.view_size[0], vh = g.u.view_size[1];
    const double Wf = g.W, Hf = g.H;
    const double sx = (2.0 * vw) / Wf, sy = -((2.0 * vh) / Hf);
    const double m = g.u.margin;
    double ex, ey;
    r.R = 0.0;
    if (g.cfg.use_unaligned_rectangles) {
        ex = m * (std::fabs(o.Xx) + std::fabs(o.Yx));
        ey = m * (std::fabs(o.Xy) + std::fabs(o.Yy));
    } else {
        r.R = std::sqrt(std::fmax(o.Xx * o.Xx + o.Xy * o.Xy, o.Yx * o.Yx + o.Yy * o.Yy)) * m;
        ex = ey = r.R;
    }
    const double cxp = (o.Zx + vw) / sx, exq = ex / sx, cyp = (o.Zy - vh) / sy, eyq = ey / (-sy);
    const double eps = 0.015625;
    const double fx0 = std::ceil(cxp - exq - eps - 0.5), fx1 = std::floor(cxp + exq + eps - 0.5);
    const double fy0 = std::ceil(cyp - eyq - eps - 0.5), fy1 = std::floor(cyp + eyq + eps - 0.5);
    r.valid = std::isfinite(r.A00) && std::isfinite(r.A01) && std::isfinite(r.B0) && std::isfinite(r.A10) &&
              std::isfinite(r.A11) && std::isfinite(r.B1) && std::isfinite(r.rgb[0]) && std::isfinite(r.rgb[1]) &&
              std::isfinite(r.rgb[2]) && std::isfinite(fx0) && std::isfinite(fx1) && std::isfinite(fy0) &&
              std::isfinite(fy1) && a >= 1.0 / 255.0;
    r.x0 = 1; r.x1 = 0; r.y0 = 1; r.y1 = 0;
    if (r.valid) {
        const double cx0 = std::fmax(fx0, 0.0), cx1 = std::fmin(fx1, Wf - 1.0);
        const double cy0 = std::fmax(fy0, 0.0), cy1 = std::fmin(fy1, Hf - 1.0);
        if (cx0 <= cx1 && cy0 <= cy1) {
            r.x0 = (int)cx0; r.x1 = (int)cx1; r.y0 = (int)cy0; r.y1 = (int)cy1;
        }
    }
    return r;
}

GRec rec_of_splat(const GradCtx& g, size_t k, const double* override_params = nullptr) {
    double p[NPARAM];
    if (override_params) {
        std::memcpy(p, override_params, sizeof(p));
    } else {
        for (int i = 0; i < 3; ++i) p[i] = g.c[3 * k + i];
        for (int i = 0; i < 4; ++i) p[3 + i] = g.q[4 * k + i];
        for (int i = 0; i < 3; ++i) p[7 + i] = g.s[3 * k + i];
        p[10] = g.a[k];
        for (int i = 0; i < 48; ++i) p[11 + i] = g.sh[48 * k + i];
    }
    return make_rec(g, p, p + 3, p + 7, p[10], p + 11);
}

struct Contrib {
    uint32_t pos;
    double alpha, E, tcx, tcy, s[3], sa, T;
};

// FP64 compositing of one pixel over the given draw positions; returns the contributors.
void shade_pixel(const GradCtx& g, const GRec* recs, const uint32_t* list, size_t nl, int px, int py,
                 std::vector<Contrib>* contribs, double* C, double* Tout) {
    const double X = px + 0.5, Y = py + 0.5;
    const double m = g.u.margin;
    const double sx = (2.0 * g.u.view_size[0]) / g.W, sy = -((2.0 * g.u.view_size[1]) / g.H);
    double T = 1.0;
    C[0] = C[1] = C[2] = 0.0;
    for (size_t li = 0; li < nl; ++li) {
        const GRec& r = recs[li];
        if (!r.valid || px < r.x0 || px > r.x1 || py < r.y0 || py > r.y1) continue;
        const double tcx = r.A00 * X + r.A01 * Y + r.B0, tcy = r.A10 * X + r.A11 * Y + r.B1;
        if (g.cfg.use_unaligned_rectangles) {
            if (!(std::fabs(tcx) <= m && std::fabs(tcy) <= m)) continue;
        } else {
            const double dx = sx * X + r.bx, dy = sy * Y + r.by;
            if (!(std::fabs(dx) <= r.R && std::fabs(dy) <= r.R)) continue;
        }
        const double E = std::exp(-0.5 * (tcx * tcx + tcy * tcy));
        const double alpha = r.a * E;
        if (alpha < 1.0 / 255.0) continue;
        Contrib k;
        k.pos = list[li];
        k.alpha = alpha; k.E = E; k.tcx = tcx; k.tcy = tcy; k.T = T;
        for (int ch = 0; ch < 3; ++ch) {
            k.s[ch] = std::fmin(std::fmax(r.rgb[ch] * alpha, 0.0), 1.0);
            C[ch] += k.s[ch] * T;
        }
        k.sa = std::fmin(std::fmax(alpha, 0.0), 1.0);
        T = T * (1.0 - k.sa);
        if (contribs) contribs->push_back(k);
        if (T < 1e-4) break;
    }
    *Tout = T;
}

void atomic_add_d(std::atomic<uint64_t>* p, double v) {
    uint64_t old = p->load(std::memory_order_relaxed), nw;
    do {
        double d;
        std::memcpy(&d, &old, 8);
        d += v;
        std::memcpy(&nw, &d, 8);
    } while (!p->compare_exchange_weak(old, nw, std::memory_order_relaxed));
}

}  // namespace

OAPI void* oracle_grad_create(const void* uni, const void* cfgp, uint64_t n, const double* c, const double* q,
                              const double* s, const double* a, const double* sh, const double* target) {
    GradCtx* g = new GradCtx();
    g->u = *(const OU*)uni;
    g->cfg = *(const OCfg*)cfgp;
    g->W = (int)g->u.image_size[0];
    g->H = (int)g->u.image_size[1];
    g->TX = (g->W + 15) / 16;
    g->TY = (g->H + 15) / 16;
    g->n = n;
    g->c.assign(c, c + 3 * n);
    g->q.assign(q, q + 4 * n);
    g->s.assign(s, s + 3 * n);
    g->a.assign(a, a + n);
    g->sh.assign(sh, sh + 48 * n);
    g->target.assign(target, target + 3 * (size_t)g->W * g->H);
    std::vector<float> cf(3 * n);
    for (size_t i = 0; i < 3 * n; ++i) cf[i] = (float)c[i];
    std::vector<uint32_t> ek(n + 1), ei(n + 1);
    uint64_t nv = 0, nd = 0;
    oracle_draw_list(uni, g->cfg.depth_sorting, cf.data(), n, ek.data(), ei.data(), &nv, &nd);
    g->order.assign(ei.begin(), ei.begin() + nd);
    g->key.assign(ek.begin(), ek.begin() + nd);
    g->pos_of.assign(n, -1);
    for (size_t p = 0; p < nd; ++p) g->pos_of[g->order[p]] = (int64_t)p;
    g->rec.resize(nd);
    parallel_for((int64_t)nd, 16, [&](int64_t b, int64_t e) {
        for (int64_t p = b; p < e; ++p) g->rec[p] = rec_of_splat(*g, g->order[p]);
    });
    g->tiles.assign((size_t)g->TX * g->TY, {});
    for (size_t p = 0; p < nd; ++p) {
        const GRec& r = g->rec[p];
        if (!r.valid || r.x0 > r.x1) continue;
        for (int ty = r.y0 / 16; ty <= r.y1 / 16; ++ty)
            for (int tx = r.x0 / 16; tx <= r.x1 / 16; ++tx) g->tiles[(size_t)ty * g->TX + tx].push_back((uint32_t)p);
    }
    return g;
}

OAPI void oracle_grad_destroy(void* h) { delete (GradCtx*)h; }

namespace {
void rebuild_tiles(GradCtx& g) {
    g.tiles.assign((size_t)g.TX * g.TY, {});
    for (size_t p = 0; p < g.rec.size(); ++p) {
        const GRec& r = g.rec[p];
        if (!r.valid || r.x0 > r.x1) continue;
        for (int ty = r.y0 / 16; ty <= r.y1 / 16; ++ty)
            for (int tx = r.x0 / 16; tx <= r.x1 / 16; ++tx) g.tiles[(size_t)ty * g.TX + tx].push_back((uint32_t)p);
    }
}
}  // namespace

// Replaces the screen-space records of the given splats by FP32 records in the renderer's 16-float
// layout (A00 A01 B0 A10 | A11 B1 opacity box_lo | r g b box_hi | bx by R 0), e.g. the ones a
// renderer produced: compositing and its gradient then run in FP64 on exactly those records, while
// the vertex-stage Jacobian stays the FP64 one at the splat's parameters.  Isolates the compositing
// backward from the precision of the FP32 vertex stage.
OAPI void oracle_grad_pin_records(void* h, const float* recs16, const uint32_t* splat_idx, uint64_t count) {
    GradCtx& g = *(GradCtx*)h;
    for (uint64_t i = 0; i < count; ++i) {
        const uint32_t k = splat_idx[i];
        if (k >= g.n || g.pos_of[k] < 0) continue;
        const float* rc = recs16 + 16 * i;
        GRec& r = g.rec[(size_t)g.pos_of[k]];
        r.A00 = rc[0]; r.A01 = rc[1]; r.B0 = rc[2]; r.A10 = rc[3];
        r.A11 = rc[4]; r.B1 = rc[5]; r.a = rc[6];
        r.rgb[0] = rc[8]; r.rgb[1] = rc[9]; r.rgb[2] = rc[10];
        r.bx = rc[12]; r.by = rc[13]; r.R = rc[14];
        const uint32_t lo = float_to_bits(rc[7]), hi = float_to_bits(rc[11]);
        r.x0 = (int)(lo & 0xFFFFu); r.y0 = (int)(lo >> 16); r.x1 = (int)(hi & 0xFFFFu); r.y1 = (int)(hi >> 16);
        r.valid = r.x0 <= r.x1 && r.y0 <= r.y1;
        if (!r.valid) { r.x0 = 1; r.x1 = 0; r.y0 = 1; r.y1 = 0; }
    }
    rebuild_tiles(g);
}

// The backward's upstream gradient dL/dC (H x W x 3) taken as given instead of 2 (C - target) of the
// FP64 frame: e.g. the FP32 frame's own 2 (C32 - target), so that the FP64 backward and a renderer's
// FP32 backward start from the same upstream gradient and differ only by their own arithmetic.  NULL
// restores 2 (C - target).
OAPI void oracle_grad_set_image_gradient(void* h, const double* grad_image) {
    GradCtx& g = *(GradCtx*)h;
    if (grad_image)
        g.gimg.assign(grad_image, grad_image + 3 * (size_t)g.W * g.H);
    else
        g.gimg.clear();
}

// Full-frame FP64 loss; grads (n x 59) receive the analytic FP64 gradient (zero for splats not drawn).
OAPI double oracle_grad_loss_ex(void* h, double* grads, double* image_out, int threads, double* rec_grads_out,
                                uint32_t* order_out);
OAPI double oracle_grad_loss(void* h, double* grads, double* image_out, int threads) {
    return oracle_grad_loss_ex(h, grads, image_out, threads, nullptr, nullptr);
}
// rec_grads_out (optional): per draw position, the 10 record gradients (d/dA against the pixel-centre
// coordinates X = px + 0.5, Y = py + 0.5, d/dB, d/dopacity, d/drgb); order_out: splat index of each
// draw position.
OAPI double oracle_grad_loss_ex(void* h, double* grads, double* image_out, int threads, double* rec_grads_out,
                                uint32_t* order_out) {
    GradCtx& g = *(GradCtx*)h;
    const size_t nd = g.order.size();
    std::vector<std::atomic<uint64_t>> rg(nd * 10);
    for (auto& x : rg) x.store(0);

    std::atomic<int64_t> next{0};
    std::vector<double> loss_t(threads > 0 ? threads : 1, 0.0);
    auto worker = [&](int tid) {
        std::vector<Contrib> cs;
        std::vector<GRec> lrec;
        for (;;) {
            const int64_t t = next.fetch_add(1);
            if (t >= (int64_t)g.tiles.size()) break;
            const auto& L = g.tiles[t];
            lrec.resize(L.size());
            for (size_t i = 0; i < L.size(); ++i) lrec[i] = g.rec[L[i]];
            const int tx = (int)(t % g.TX), ty = (int)(t / g.TX);
            for (int py = ty * 16; py < std::min(g.H, ty * 16 + 16); ++py)
                for (int px = tx * 16; px < std::min(g.W, tx * 16 + 16); ++px) {
                    cs.clear();
                    double C[3], Tf;
                    shade_pixel(g, lrec.data(), L.data(), L.size(), px, py, &cs, C, &Tf);
                    const size_t pix = (size_t)py * g.W + px;
                    double gC[3];
                    for (int ch = 0; ch < 3; ++ch) {
                        const double d = C[ch] - g.target[3 * pix + ch];
                        loss_t[tid] += d * d;
                        gC[ch] = g.gimg.empty() ? 2.0 * d : g.gimg[3 * pix + ch];
                        if (image_out) image_out[4 * pix + ch] = C[ch];
                    }
                    if (image_out) image_out[4 * pix + 3] = Tf;
                    // back to front; S = colour of the splats behind
                    double S[3] = {0.0, 0.0, 0.0};
                    for (size_t ii = cs.size(); ii-- > 0;) {
                        const Contrib& k = cs[ii];
                        const GRec& r = g.rec[k.pos];
                        double dS[3];
                        for (int ch = 0; ch < 3; ++ch) dS[ch] = gC[ch] * k.T;
                        const double om = 1.0 - k.sa;
                        const double dsa = om > 0.0 ? -(gC[0] * S[0] + gC[1] * S[1] + gC[2] * S[2]) / om : 0.0;
                        for (int ch = 0; ch < 3; ++ch) S[ch] += k.s[ch] * k.T;
                        double dalpha = k.alpha < 1.0 ? dsa : 0.0;
                        double out[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
                        for (int ch = 0; ch < 3; ++ch) {
                            const double v = r.rgb[ch] * k.alpha;
                            if (v > 0.0 && v < 1.0) {
                                dalpha += dS[ch] * r.rgb[ch];
                                out[7 + ch] = dS[ch] * k.alpha;
                            }
                        }
                        out[6] = dalpha * k.E;
                        const double dpow = -0.5 * dalpha * r.a * k.E;
                        const double X = px + 0.5, Y = py + 0.5;
                        const double dtx = 2.0 * dpow * k.tcx, dty = 2.0 * dpow * k.tcy;
                        out[0] = dtx * X; out[1] = dtx * Y; out[2] = dtx;
                        out[3] = dty * X; out[4] = dty * Y; out[5] = dty;
                        for (int kk = 0; kk < 10; ++kk)
                            if (out[kk] != 0.0) atomic_add_d(&rg[(size_t)k.pos * 10 + kk], out[kk]);

                    }
                }
        }
    };
    const int nt = threads > 0 ? threads : 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker, t);
    for (auto& th : pool) th.join();
    double loss = 0.0;
    for (double v : loss_t) loss += v;
    if (rec_grads_out) {
        for (size_t p = 0; p < nd; ++p) {
            for (int kk = 0; kk < 10; ++kk) {
                uint64_t bits = rg[p * 10 + kk].load();
                std::memcpy(&rec_grads_out[p * 10 + kk], &bits, 8);
            }
            if (order_out) order_out[p] = g.order[p];
        }
    }
    if (grads) {
        std::memset(grads, 0, sizeof(double) * NPARAM * g.n);
        parallel_for((int64_t)nd, nt, [&](int64_t b, int64_t e) {
            for (int64_t p = b; p < e; ++p) {
                double gr[10];
                bool any = false;
                for (int kk = 0; kk < 10; ++kk) {
                    const uint64_t bits = rg[(size_t)p * 10 + kk].load();
                    std::memcpy(&gr[kk], &bits, 8);
                    any = any || gr[kk] != 0.0;
                }
                if (!any) continue;
                const size_t k = g.order[p];
                double* out = grads + NPARAM * k;
                // vertex stage through dual numbers: one pass per centre/rotation/scale direction
                Dd shd[48];
                const int nsh = 3 * (g.cfg.sh_order + 1) * (g.cfg.sh_order + 1);
                for (int i = 0; i < 48; ++i) shd[i] = Dd(i < nsh ? g.sh[48 * k + i] : 0.0);
                for (int dir = 0; dir < 10; ++dir) {
                    Dd cc[3], qq[4], ss[3];
                    for (int i = 0; i < 3; ++i) cc[i] = Dd(g.c[3 * k + i], dir == i ? 1.0 : 0.0);
                    for (int i = 0; i < 4; ++i) qq[i] = Dd(g.q[4 * k + i], dir == 3 + i ? 1.0 : 0.0);
                    for (int i = 0; i < 3; ++i) ss[i] = Dd(g.s[3 * k + i], dir == 7 + i ? 1.0 : 0.0);
                    VOut<Dd> o;
                    vertex_core<Dd>(g.u, g.cfg, cc, qq, ss, shd, o);
                    out[dir] = gr[0] * o.A00.d + gr[1] * o.A01.d + gr[2] * o.B0.d + gr[3] * o.A10.d +
                               gr[4] * o.A11.d + gr[5] * o.B1.d + gr[7] * o.rgb[0].d + gr[8] * o.rgb[1].d +
                               gr[9] * o.rgb[2].d;
                }
                out[10] = gr[6];
                // SH coefficients enter linearly: basis value times the colour gradient
                double cc[3] = {g.c[3 * k], g.c[3 * k + 1], g.c[3 * k + 2]};
                double v[3], d[3];
                for (int i = 0; i < 3; ++i) v[i] = cc[i] - (double)g.u.camera[12 + i];
                const double len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                for (int i = 0; i < 3; ++i) d[i] = v[i] / len;
                const int nk = (g.cfg.sh_order + 1) * (g.cfg.sh_order + 1);
                for (int kk = 0; kk < nk; ++kk) {
                    double one[48] = {0.0};
                    one[3 * kk] = 1.0;
                    double rgb[3];
                    sh_lookup(d, one, g.cfg.sh_order, rgb);
                    const double basis = rgb[0] - 0.5;
                    for (int ch = 0; ch < 3; ++ch) out[11 + 3 * kk + ch] = basis * gr[7 + ch];
                }
            }
        });
    }
    return loss;
}

// FP64 Jacobian of splat k's record (A00, A01, B0, A10, A11, B1, r, g, b; A against pixel-centre
// coordinates) with respect to its centre, rotation and scale (10 directions): J[dir * 9 + out].
OAPI void oracle_grad_jacobian(void* h, uint64_t k, double* J) {
    GradCtx& g = *(GradCtx*)h;
    Dd shd[48];
    const int nsh = 3 * (g.cfg.sh_order + 1) * (g.cfg.sh_order + 1);
    for (int i = 0; i < 48; ++i) shd[i] = Dd(i < nsh ? g.sh[48 * k + i] : 0.0);
    for (int dir = 0; dir < 10; ++dir) {
        Dd cc[3], qq[4], ss[3];
        for (int i = 0; i < 3; ++i) cc[i] = Dd(g.c[3 * k + i], dir == i ? 1.0 : 0.0);
        for (int i = 0; i < 4; ++i) qq[i] = Dd(g.q[4 * k + i], dir == 3 + i ? 1.0 : 0.0);
        for (int i = 0; i < 3; ++i) ss[i] = Dd(g.s[3 * k + i], dir == 7 + i ? 1.0 : 0.0);
        VOut<Dd> o;
        vertex_core<Dd>(g.u, g.cfg, cc, qq, ss, shd, o);
        const double v[9] = {o.A00.d, o.A01.d, o.B0.d, o.A10.d, o.A11.d, o.B1.d, o.rgb[0].d, o.rgb[1].d, o.rgb[2].d};
        for (int j = 0; j < 9; ++j) J[dir * 9 + j] = v[j];
    }
}

namespace {
// Central difference of the loss between two parameter vectors of splat k (59 activated values
// each): (loss(p[0]) - loss(p[1])) / denom, re-rendering only the tiles the splat touches.  Returns
// 0 (excluded) when anything discrete differs between the two or from the base frame; a splat this
// frame does not draw has difference 0 unless a step would draw it.
int fd_between(GradCtx& g, uint64_t k, const double* const p[2], double denom, double* fd) {
    *fd = 0.0;
    if (k >= g.n) return 0;
    if (g.pos_of[k] < 0) {
        // not drawn in this frame: the difference is 0 when it stays undrawn under both steps (culled,
        // or a key the mode does not draw), excluded when a step would draw it
        for (int sgn = 0; sgn < 2; ++sgn) {
            float cf[3] = {(float)p[sgn][0], (float)p[sgn][1], (float)p[sgn][2]};
            uint32_t kk;
            uint8_t vis;
            oracle_cull_keys(&g.u, g.cfg.depth_sorting, cf, 1, &kk, &vis);
            const bool drawn = vis && !(g.cfg.depth_sorting == 2 && kk == 0xFFFFFFFFu) &&
                               !(g.cfg.depth_sorting == 3 && (kk >> 24) == 0xFFu);
            if (drawn) return 0;
        }
        return 1;
    }
    const uint32_t pos = (uint32_t)g.pos_of[k];
    GRec rr[2];
    for (int sgn = 0; sgn < 2; ++sgn) {
        const double* q = p[sgn];
        if (q[0] != g.c[3 * k] || q[1] != g.c[3 * k + 1] || q[2] != g.c[3 * k + 2]) {
            // the FP32 depth key (and culling) must not change
            float cf[3] = {(float)q[0], (float)q[1], (float)q[2]};
            uint32_t kk;
            uint8_t vis;
            oracle_cull_keys(&g.u, g.cfg.depth_sorting, cf, 1, &kk, &vis);
            if (!vis || kk != g.key[pos]) return 0;
        }
        rr[sgn] = rec_of_splat(g, k, q);
        if (!rr[sgn].valid) return 0;
    }
    const GRec& r0 = g.rec[pos];
    auto tiles_of = [&](const GRec& r, std::vector<int64_t>& out) {
        if (!r.valid || r.x0 > r.x1) return;
        for (int ty = r.y0 / 16; ty <= r.y1 / 16; ++ty)
            for (int tx = r.x0 / 16; tx <= r.x1 / 16; ++tx) out.push_back((int64_t)ty * g.TX + tx);
    };
    std::vector<int64_t> t0, tp, tm;
    tiles_of(r0, t0);
    tiles_of(rr[0], tp);
    tiles_of(rr[1], tm);
    if (t0 != tp || t0 != tm) return 0;  // the splat enters or leaves a tile
    double loss[2] = {0.0, 0.0};
    for (int64_t t : t0) {
        const auto& L = g.tiles[t];
        std::vector<GRec> lrec(L.size());
        const int tx = (int)(t % g.TX), ty = (int)(t / g.TX);
        std::vector<std::vector<uint32_t>> sig(2);
        for (int sgn = 0; sgn < 2; ++sgn) {
            for (size_t i = 0; i < L.size(); ++i) lrec[i] = L[i] == pos ? rr[sgn] : g.rec[L[i]];
            std::vector<Contrib> cs;
            for (int py = ty * 16; py < std::min(g.H, ty * 16 + 16); ++py)
                for (int px = tx * 16; px < std::min(g.W, tx * 16 + 16); ++px) {
                    cs.clear();
                    double C[3], Tf;
                    shade_pixel(g, lrec.data(), L.data(), L.size(), px, py, &cs, C, &Tf);
                    const size_t pix = (size_t)py * g.W + px;
                    for (int ch = 0; ch < 3; ++ch) {
                        const double d = C[ch] - g.target[3 * pix + ch];
                        loss[sgn] += d * d;
                    }
                    for (auto& c : cs) sig[sgn].push_back(c.pos);
                    sig[sgn].push_back(0xFFFFFFFFu);
                }
        }
        if (sig[0] != sig[1]) return 0;
    }
    *fd = (loss[0] - loss[1]) / denom;
    return 1;
}

void base_params(const GradCtx& g, uint64_t k, double* base) {
    for (int i = 0; i < 3; ++i) base[i] = g.c[3 * k + i];
    for (int i = 0; i < 4; ++i) base[3 + i] = g.q[4 * k + i];
    for (int i = 0; i < 3; ++i) base[7 + i] = g.s[3 * k + i];
    base[10] = g.a[k];
    for (int i = 0; i < 48; ++i) base[11 + i] = g.sh[48 * k + i];
}
}  // namespace

// Central difference of the loss in parameter `param` (0..58) of splat k with step hstep.  Returns 1
// and writes *fd when nothing discrete changes under +-hstep, 0 otherwise (excluded).
OAPI int oracle_grad_fd(void* h, uint64_t k, int param, double hstep, double* fd) {
    GradCtx& g = *(GradCtx*)h;
    *fd = 0.0;
    if (k >= g.n || param < 0 || param >= NPARAM) return 0;
    double pp[NPARAM], pm[NPARAM];
    base_params(g, k, pp);
    std::memcpy(pm, pp, sizeof(pp));
    pp[param] += hstep;
    pm[param] -= hstep;
    const double* const p[2] = {pp, pm};
    return fd_between(g, k, p, 2.0 * hstep, fd);
}

// The same difference between two explicit parameter vectors of splat k (59 activated values each,
// centre 3, rotation 4, scale 3, opacity, SH 48), divided by `denom`: for steps in parameters that
// the loss sees only through an activation moving several of these at once (a raw log-scale moves
// all three scales when its clamp is active, a raw quaternion component all four rotation values).
OAPI int oracle_grad_fd_params(void* h, uint64_t k, const double* p_plus, const double* p_minus, double denom,
                               double* fd) {
    GradCtx& g = *(GradCtx*)h;
    const double* const p[2] = {p_plus, p_minus};
    return fd_between(g, k, p, denom, fd);
}

// Splats whose gradient depends on a decision that the FP32 frame and the FP64 frame take
// differently: for every pixel, the FP32 contributors (the GPU's frame, bit for bit: same records,
// coverage, falloff, 1/255 discard, early stop) and their saturation regimes are compared with the
// FP64 ones; every splat contributing to a pixel where they differ is flagged (1).  Gradients of
// flagged splats differ between FP32 and FP64 by construction (a threshold is crossed within
// rounding), so comparisons exclude them.  Returns the number of differing pixels.
OAPI uint64_t oracle_grad_ambiguous(void* h, uint8_t* flags, int threads) {
    GradCtx& g = *(GradCtx*)h;
    const size_t nd = g.order.size();
    // FP32 records of the drawn entries, exactly as the GPU computes them
    std::vector<float> rec32(16 * nd);
    parallel_for((int64_t)nd, threads, [&](int64_t b, int64_t e) {
        for (int64_t p = b; p < e; ++p) {
            const size_t k = g.order[p];
            float c[3], q[4], s[3], sh[48];
            for (int i = 0; i < 3; ++i) c[i] = (float)g.c[3 * k + i];
            for (int i = 0; i < 4; ++i) q[i] = (float)g.q[4 * k + i];
            for (int i = 0; i < 3; ++i) s[i] = (float)g.s[3 * k + i];
            for (int i = 0; i < 48; ++i) sh[i] = (float)g.sh[48 * k + i];
            preprocess_one<float>(g.u, g.cfg, c, q, s, (float)g.a[k], sh, rec32.data() + 16 * p, nullptr);
        }
    });
    // FP32 tile lists (the GPU bins with the FP32 boxes)
    std::vector<std::vector<uint32_t>> tl32((size_t)g.TX * g.TY);
    for (size_t p = 0; p < nd; ++p) {
        const float* rc = rec32.data() + 16 * p;
        const uint32_t lo = float_to_bits(rc[7]), hi = float_to_bits(rc[11]);
        const int x0 = (int)(lo & 0xFFFFu), y0 = (int)(lo >> 16), x1 = (int)(hi & 0xFFFFu), y1 = (int)(hi >> 16);
        if (x0 > x1 || y0 > y1) continue;
        for (int ty = y0 / 16; ty <= y1 / 16; ++ty)
            for (int tx = x0 / 16; tx <= x1 / 16; ++tx) tl32[(size_t)ty * g.TX + tx].push_back((uint32_t)p);
    }
    std::vector<std::atomic<uint8_t>> fl(g.n);
    for (auto& f : fl) f.store(0);
    std::atomic<uint64_t> npix{0};
    std::atomic<int64_t> next{0};
    const float m = g.u.margin;
    auto worker = [&] {
        std::vector<Contrib> cs;
        std::vector<GRec> lrec;
        std::vector<uint64_t> s32, s64;
        for (;;) {
            const int64_t t = next.fetch_add(1);
            if (t >= (int64_t)g.tiles.size()) break;
            const auto& L64 = g.tiles[t];
            const auto& L32 = tl32[t];
            lrec.resize(L64.size());
            for (size_t i = 0; i < L64.size(); ++i) lrec[i] = g.rec[L64[i]];
            const int tx = (int)(t % g.TX), ty = (int)(t / g.TX);
            for (int py = ty * 16; py < std::min(g.H, ty * 16 + 16); ++py)
                for (int px = tx * 16; px < std::min(g.W, tx * 16 + 16); ++px) {
                    // FP32 frame
                    s32.clear();
                    const float X = (float)px + 0.5f, Y = (float)py + 0.5f;
                    float ft = 1.0f;
                    for (uint32_t p : L32) {
                        const float* rc = rec32.data() + 16 * (size_t)p;
                        const uint32_t lo = float_to_bits(rc[7]), hi = float_to_bits(rc[11]);
                        if (px < (int)(lo & 0xFFFFu) || px > (int)(hi & 0xFFFFu) || py < (int)(lo >> 16) ||
                            py > (int)(hi >> 16))
                            continue;
                        const float tcx = std::fmaf(rc[1], Y, std::fmaf(rc[0], X, rc[2]));
                        const float tcy = std::fmaf(rc[4], Y, std::fmaf(rc[3], X, rc[5]));
                        if (g.cfg.use_unaligned_rectangles) {
                            if (!(std::fabs(tcx) <= m && std::fabs(tcy) <= m)) continue;
                        } else {
                            const float sx = (2.0f * g.u.view_size[0]) / (float)g.W;
                            const float sy = -((2.0f * g.u.view_size[1]) / (float)g.H);
                            const float dx = std::fmaf(sx, X, rc[12]), dy = std::fmaf(sy, Y, rc[13]);
                            if (!(std::fabs(dx) <= rc[14] && std::fabs(dy) <= rc[14])) continue;
                        }
                        const float alpha = rc[6] * o_expf(-0.5f * std::fmaf(tcx, tcx, tcy * tcy));
                        if (alpha < ALPHA_MIN) continue;
                        uint64_t regime = 0;
                        for (int ch = 0; ch < 3; ++ch) {
                            const float v = rc[8 + ch] * alpha;
                            regime |= (uint64_t)(v > 0.0f && v < 1.0f) << ch;
                        }
                        regime |= (uint64_t)(alpha < 1.0f) << 3;
                        s32.push_back(((uint64_t)p << 4) | regime);
                        ft = ft * (1.0f - clamp01(alpha));
                        if (ft < FP32_T_MIN) break;
                    }
                    // FP64 frame
                    cs.clear();
                    double C[3], Tf;
                    shade_pixel(g, lrec.data(), L64.data(), L64.size(), px, py, &cs, C, &Tf);
                    s64.clear();
                    for (auto& k : cs) {
                        const GRec& r = g.rec[k.pos];
                        uint64_t regime = 0;
                        for (int ch = 0; ch < 3; ++ch) {
                            const double v = r.rgb[ch] * k.alpha;
                            regime |= (uint64_t)(v > 0.0 && v < 1.0) << ch;
                        }
                        regime |= (uint64_t)(k.alpha < 1.0) << 3;
                        s64.push_back(((uint64_t)k.pos << 4) | regime);
                    }
                    if (s32 != s64) {
                        ++npix;
                        for (uint64_t v : s32) fl[g.order[v >> 4]].store(1);
                        for (uint64_t v : s64) fl[g.order[v >> 4]].store(1);
                    }
                }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < (threads > 0 ? threads : 1); ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    for (size_t i = 0; i < g.n; ++i) flags[i] = fl[i].load();
    return npix.load();
}
