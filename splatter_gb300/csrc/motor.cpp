// Camera motors of 3D projective geometric algebra (host only).
//
// The reference takes the camera as a PGA motor (`render_frame(.., camera_motor: Motor, ..)`,
// renderer.rs:355-363) and turns it into matrices with `motor3d_to_mat4` (utils.rs:31-42: the images of
// the x, y, z directions and of the origin under the motor, as columns) and `Motor::inverse`
// (renderer.rs:365).  Its algebra comes from the crate geometric_algebra 0.3.0, which is not
// available here, so this file builds the same objects from first principles: the algebra
// Cl(3,0,1) with basis vectors e0 (e0^2 = 0), e1, e2, e3 (squares +1), blades as bit masks over
// (e0, e1, e2, e3), the geometric product from the reordering sign and the metric, and the sandwich
// M X ~M that moves points.  Layouts (fixed here, documented in include/splatter.h):
//   motor  [s, e23, e31, e12, e01, e02, e03, e0123]
//   point  [e123, e032, e013, e021] = (w, x, y, z), a finite point x e032 + y e013 + z e021 + e123
// The arithmetic is double precision and rounds once to float at the API.
#include <cmath>
#include <cstring>

#include "spl_internal.h"

namespace {

using MV = double[16];  // coefficients by blade bit mask: bit 0 = e0, bit 1 = e1, bit 2 = e2, bit 3 = e3

// Sign of the product of two canonically ordered blades from moving the factors of b past those
// of a (each swap of distinct basis vectors flips the sign).
int reorder_sign(unsigned a, unsigned b) {
    int swaps = 0;
    for (a >>= 1; a; a >>= 1) swaps += __builtin_popcount(a & b);
    return (swaps & 1) ? -1 : 1;
}

void gp(const MV a, const MV b, MV out) {
    double r[16] = {0};
    for (unsigned i = 0; i < 16; ++i) {
        if (a[i] == 0.0) continue;
        for (unsigned j = 0; j < 16; ++j) {
            if (b[j] == 0.0) continue;
            if (i & j & 1u) continue;  // e0 e0 = 0
            r[i ^ j] += reorder_sign(i, j) * a[i] * b[j];
        }
    }
    std::memcpy(out, r, sizeof(r));
}

void reverse(const MV a, MV out) {
    for (unsigned i = 0; i < 16; ++i) {
        const int k = __builtin_popcount(i);
        out[i] = ((k * (k - 1) / 2) & 1) ? -a[i] : a[i];
    }
}

// API components -> blades, with the sign of the written basis order against the canonical one.
struct Slot {
    unsigned blade;
    int sign;
};
constexpr Slot MOTOR[8] = {{0x0, 1},  // s
                           {0xC, 1},  // e23
                           {0xA, -1}, // e31 = -e13
                           {0x6, 1},  // e12
                           {0x3, 1},  // e01
                           {0x5, 1},  // e02
                           {0x9, 1},  // e03
                           {0xF, 1}}; // e0123
constexpr Slot POINT[4] = {{0xE, 1},   // e123
                           {0xD, -1},  // e032 = -e023
                           {0xB, 1},   // e013
                           {0x7, -1}}; // e021 = -e012

void motor_in(const float m[8], MV out) {
    std::memset(out, 0, sizeof(MV));
    for (int k = 0; k < 8; ++k) out[MOTOR[k].blade] = MOTOR[k].sign * (double)m[k];
}
void motor_out(const MV a, float m[8]) {
    for (int k = 0; k < 8; ++k) m[k] = (float)(MOTOR[k].sign * a[MOTOR[k].blade]);
}

// M P ~M for the point (w, x, y, z); returns (w', x', y', z').
void transform_point(const MV M, const double p[4], double out[4]) {
    MV P = {0}, Mr, t, r;
    for (int k = 0; k < 4; ++k) P[POINT[k].blade] = POINT[k].sign * p[k];
    reverse(M, Mr);
    gp(M, P, t);
    gp(t, Mr, r);
    for (int k = 0; k < 4; ++k) out[k] = POINT[k].sign * r[POINT[k].blade];
}

}  // namespace

extern "C" {

int spl_motor_to_mat4(const float motor[8], float camera_to_world[16]) {
    if (!motor || !camera_to_world) return spl::fail(SPL_ERR_INVALID, "NULL argument");
    MV M;
    motor_in(motor, M);
    // utils.rs:31-42: columns are the images of the directions x, y, z (point components 1, 2, 3) and
    // of the origin (component 0), each written as (x, y, z, w)
    const int basis[4] = {1, 2, 3, 0};
    for (int c = 0; c < 4; ++c) {
        double p[4] = {0, 0, 0, 0}, q[4];
        p[basis[c]] = 1.0;
        transform_point(M, p, q);
        camera_to_world[4 * c + 0] = (float)q[1];
        camera_to_world[4 * c + 1] = (float)q[2];
        camera_to_world[4 * c + 2] = (float)q[3];
        camera_to_world[4 * c + 3] = (float)q[0];
    }
    return SPL_OK;
}

int spl_motor_inverse(const float motor[8], float out[8]) {
    if (!motor || !out) return spl::fail(SPL_ERR_INVALID, "NULL argument");
    MV M, Mr, n;
    motor_in(motor, M);
    reverse(M, Mr);
    gp(M, Mr, n);  // a motor times its reverse: scalar (its squared norm) + e0123 part
    const double s = n[0];
    if (!(s > 0.0) || !std::isfinite(s)) return spl::fail(SPL_ERR_INVALID, "motor has no inverse (norm %g)", s);
    // (s + p I)^-1 = (s - p I) / s^2 because I^2 = 0; the inverse is ~M (s + p I)^-1
    MV inv_n = {0}, res;
    inv_n[0] = 1.0 / s;
    inv_n[15] = -n[15] / (s * s);
    gp(Mr, inv_n, res);
    motor_out(res, out);
    return SPL_OK;
}

int spl_motor_product(const float a[8], const float b[8], float out[8]) {
    if (!a || !b || !out) return spl::fail(SPL_ERR_INVALID, "NULL argument");
    MV A, B, R;
    motor_in(a, A);
    motor_in(b, B);
    gp(A, B, R);
    motor_out(R, out);
    return SPL_OK;
}

int spl_motor_from_rotor_translation(const float rotor[4], const float translation[3], float out[8]) {
    if (!rotor || !translation || !out) return spl::fail(SPL_ERR_INVALID, "NULL argument");
    const double n = std::sqrt((double)rotor[0] * rotor[0] + (double)rotor[1] * rotor[1] +
                               (double)rotor[2] * rotor[2] + (double)rotor[3] * rotor[3]);
    if (!(n > 0.0) || !std::isfinite(n)) return spl::fail(SPL_ERR_INVALID, "rotor of norm %g", n);
    // the rotor (s, e23, e31, e12) turns by 2 acos(s) about the axis (e23, e31, e12) / sin, right-handed;
    // the translator 1 - (t_x e01 + t_y e02 + t_z e03) / 2 moves the origin to t; motor = T R (R first)
    MV R = {0}, T = {0}, M;
    R[0] = rotor[0] / n;
    R[MOTOR[1].blade] = MOTOR[1].sign * (-(double)rotor[1] / n);
    R[MOTOR[2].blade] = MOTOR[2].sign * (-(double)rotor[2] / n);
    R[MOTOR[3].blade] = MOTOR[3].sign * (-(double)rotor[3] / n);
    T[0] = 1.0;
    T[MOTOR[4].blade] = MOTOR[4].sign * (-0.5 * translation[0]);
    T[MOTOR[5].blade] = MOTOR[5].sign * (-0.5 * translation[1]);
    T[MOTOR[6].blade] = MOTOR[6].sign * (-0.5 * translation[2]);
    gp(T, R, M);
    motor_out(M, out);
    return SPL_OK;
}

}  // extern "C"
