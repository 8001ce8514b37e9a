// Host-side vector/matrix maths with glam 0.30's operation order.
//
// The reference does all of its camera, node and bounding-sphere maths with
// glam (Cargo.lock: glam 0.30.10). Rounding depends on the order of the
// adds, so every function here states the order it follows. Where glam's
// SIMD backends differ (a 4-wide horizontal dot product sums
// (x*x+z*z)+(y*y+w*w) on SSE2 but (x*x+y*y)+(z*z+w*w) on NEON), the NEON
// (aarch64) order is used; it equals the sequential scalar order whenever
// w == 0, which covers every use on the render path.
//
// Compiled with -ffp-contract=off: glam never fuses a multiply and an add.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace swr {

struct V3 {
    float x, y, z;
};
struct V4 {
    float x, y, z, w;
};
// Column-major 4x4 (glam Mat4: x_axis, y_axis, z_axis, w_axis).
struct M4 {
    V4 c[4];
};
struct Quat {
    float x, y, z, w;
};

inline V3 v3(float x, float y, float z) { return {x, y, z}; }
inline V4 v4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 mul(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 mulv(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 v3min(V3 a, V3 b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
inline V3 v3max(V3 a, V3 b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
inline V4 add4(V4 a, V4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline V4 mul4(V4 a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }

// Vec3A::dot: (x*x' + y*y') + z*z' (glam dot3 on SSE2 and NEON alike).
inline float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
// Vec4::dot, NEON pairwise order: (x*x' + y*y') + (z*z' + w*w').
inline float dot4(V4 a, V4 b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }
inline float length3(V3 a) { return std::sqrt(dot3(a, a)); }
inline float length4(V4 a) { return std::sqrt(dot4(a, a)); }
// Vec3A::normalize = self * (1 / length).
inline V3 normalize3(V3 a) {
    float r = 1.0f / length3(a);
    return mul(a, r);
}
inline V3 cross3(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

inline M4 identity4() {
    M4 m;
    m.c[0] = {1, 0, 0, 0};
    m.c[1] = {0, 1, 0, 0};
    m.c[2] = {0, 0, 1, 0};
    m.c[3] = {0, 0, 0, 1};
    return m;
}
inline M4 from_array(const float* a) {
    M4 m;
    std::memcpy(&m, a, sizeof(float) * 16);
    return m;
}
inline void to_array(const M4& m, float* a) { std::memcpy(a, &m, sizeof(float) * 16); }

// Mat4::mul_vec4: ((x_axis*x + y_axis*y) + z_axis*z) + w_axis*w.
inline V4 mulmv(const M4& m, V4 v) {
    V4 r = mul4(m.c[0], v.x);
    r = add4(r, mul4(m.c[1], v.y));
    r = add4(r, mul4(m.c[2], v.z));
    r = add4(r, mul4(m.c[3], v.w));
    return r;
}
// Mat4 * Mat4: column i = self * rhs.col(i).
inline M4 mulmm(const M4& a, const M4& b) {
    M4 r;
    for (int i = 0; i < 4; ++i) r.c[i] = mulmv(a, b.c[i]);
    return r;
}
// Mat4::transform_point3a: ((x_axis*x + y_axis*y) + z_axis*z) + w_axis.
inline V3 transform_point3(const M4& m, V3 p) {
    V4 r = mul4(m.c[0], p.x);
    r = add4(r, mul4(m.c[1], p.y));
    r = add4(r, mul4(m.c[2], p.z));
    r = add4(r, m.c[3]);
    return {r.x, r.y, r.z};
}
inline M4 transpose4(const M4& m) {
    M4 r;
    const float* a = &m.c[0].x;
    float* o = &r.c[0].x;
    for (int c = 0; c < 4; ++c)
        for (int rr = 0; rr < 4; ++rr) o[c * 4 + rr] = a[rr * 4 + c];
    return r;
}

// Mat4::inverse, the cofactor expansion glam derives from GLM. The
// determinant's final horizontal add is (x+y)+(z+w) as on the SIMD paths.
inline M4 inverse4(const M4& m) {
    const float m00 = m.c[0].x, m01 = m.c[0].y, m02 = m.c[0].z, m03 = m.c[0].w;
    const float m10 = m.c[1].x, m11 = m.c[1].y, m12 = m.c[1].z, m13 = m.c[1].w;
    const float m20 = m.c[2].x, m21 = m.c[2].y, m22 = m.c[2].z, m23 = m.c[2].w;
    const float m30 = m.c[3].x, m31 = m.c[3].y, m32 = m.c[3].z, m33 = m.c[3].w;
    const float coef00 = m22 * m33 - m32 * m23;
    const float coef02 = m12 * m33 - m32 * m13;
    const float coef03 = m12 * m23 - m22 * m13;
    const float coef04 = m21 * m33 - m31 * m23;
    const float coef06 = m11 * m33 - m31 * m13;
    const float coef07 = m11 * m23 - m21 * m13;
    const float coef08 = m21 * m32 - m31 * m22;
    const float coef10 = m11 * m32 - m31 * m12;
    const float coef11 = m11 * m22 - m21 * m12;
    const float coef12 = m20 * m33 - m30 * m23;
    const float coef14 = m10 * m33 - m30 * m13;
    const float coef15 = m10 * m23 - m20 * m13;
    const float coef16 = m20 * m32 - m30 * m22;
    const float coef18 = m10 * m32 - m30 * m12;
    const float coef19 = m10 * m22 - m20 * m12;
    const float coef20 = m20 * m31 - m30 * m21;
    const float coef22 = m10 * m31 - m30 * m11;
    const float coef23 = m10 * m21 - m20 * m11;
    const V4 fac0 = {coef00, coef00, coef02, coef03};
    const V4 fac1 = {coef04, coef04, coef06, coef07};
    const V4 fac2 = {coef08, coef08, coef10, coef11};
    const V4 fac3 = {coef12, coef12, coef14, coef15};
    const V4 fac4 = {coef16, coef16, coef18, coef19};
    const V4 fac5 = {coef20, coef20, coef22, coef23};
    const V4 vec0 = {m10, m00, m00, m00};
    const V4 vec1 = {m11, m01, m01, m01};
    const V4 vec2 = {m12, m02, m02, m02};
    const V4 vec3 = {m13, m03, m03, m03};
    auto mv = [](V4 a, V4 b) { return V4{a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; };
    auto sv = [](V4 a, V4 b) { return V4{a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; };
    const V4 inv0 = add4(sv(mv(vec1, fac0), mv(vec2, fac1)), mv(vec3, fac2));
    const V4 inv1 = add4(sv(mv(vec0, fac0), mv(vec2, fac3)), mv(vec3, fac4));
    const V4 inv2 = add4(sv(mv(vec0, fac1), mv(vec1, fac3)), mv(vec3, fac5));
    const V4 inv3 = add4(sv(mv(vec0, fac2), mv(vec1, fac4)), mv(vec2, fac5));
    const V4 sign_a = {1.0f, -1.0f, 1.0f, -1.0f};
    const V4 sign_b = {-1.0f, 1.0f, -1.0f, 1.0f};
    M4 inv;
    inv.c[0] = mv(inv0, sign_a);
    inv.c[1] = mv(inv1, sign_b);
    inv.c[2] = mv(inv2, sign_a);
    inv.c[3] = mv(inv3, sign_b);
    const V4 col0 = {inv.c[0].x, inv.c[1].x, inv.c[2].x, inv.c[3].x};
    const V4 d0 = mv(m.c[0], col0);
    const float det = (d0.x + d0.y) + (d0.z + d0.w);
    const float rcp = 1.0f / det;
    for (int i = 0; i < 4; ++i) inv.c[i] = mul4(inv.c[i], rcp);
    return inv;
}

// Quat::from_rotation_{x,y,z}: (s, c) = sin_cos(angle * 0.5).
inline Quat quat_rot_x(float a) {
    float h = a * 0.5f;
    return {std::sin(h), 0.0f, 0.0f, std::cos(h)};
}
inline Quat quat_rot_y(float a) {
    float h = a * 0.5f;
    return {0.0f, std::sin(h), 0.0f, std::cos(h)};
}
inline Quat quat_rot_z(float a) {
    float h = a * 0.5f;
    return {0.0f, 0.0f, std::sin(h), std::cos(h)};
}
// Hamilton product in the grouping of glam's SIMD quat_mul:
// (w0*q1 + x0*(w,-z,y,-x)) + (y0*(z,w,-x,-y) + z0*(-y,x,w,-z)).
inline Quat quat_mul(Quat a, Quat b) {
    const float r0x = a.w * b.x + a.x * b.w;
    const float r0y = a.w * b.y + -(a.x * b.z);
    const float r0z = a.w * b.z + a.x * b.y;
    const float r0w = a.w * b.w + -(a.x * b.x);
    const float r1x = a.y * b.z + -(a.z * b.y);
    const float r1y = a.y * b.w + a.z * b.x;
    const float r1z = -(a.y * b.x) + a.z * b.w;
    const float r1w = -(a.y * b.y) + -(a.z * b.z);
    return {r0x + r1x, r0y + r1y, r0z + r1z, r0w + r1w};
}
inline Quat quat_conj(Quat q) { return {-q.x, -q.y, -q.z, q.w}; }
// Quat * Vec3A: v*(w*w - b.b) + b*(2*(v.b)) + (b x v)*(2*w).
inline V3 quat_rotate(Quat q, V3 v) {
    const V3 b = {q.x, q.y, q.z};
    const float w = q.w;
    const float b2 = dot3(b, b);
    const V3 t0 = mul(v, w * w - b2);
    const V3 t1 = mul(b, dot3(v, b) * 2.0f);
    const V3 t2 = mul(cross3(b, v), w * 2.0f);
    return add(add(t0, t1), t2);
}
// Mat4::from_quat (glam quat_to_axes).
inline M4 mat_from_quat(Quat q) {
    const float x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    const float xx = q.x * x2, xy = q.x * y2, xz = q.x * z2;
    const float yy = q.y * y2, yz = q.y * z2, zz = q.z * z2;
    const float wx = q.w * x2, wy = q.w * y2, wz = q.w * z2;
    M4 m;
    m.c[0] = {1.0f - (yy + zz), xy + wz, xz - wy, 0.0f};
    m.c[1] = {xy - wz, 1.0f - (xx + zz), yz + wx, 0.0f};
    m.c[2] = {xz + wy, yz - wx, 1.0f - (xx + yy), 0.0f};
    m.c[3] = {0.0f, 0.0f, 0.0f, 1.0f};
    return m;
}
inline M4 mat_translation(V3 t) {
    M4 m = identity4();
    m.c[3] = {t.x, t.y, t.z, 1.0f};
    return m;
}
inline M4 mat_scale(V3 s) {
    M4 m = identity4();
    m.c[0].x = s.x;
    m.c[1].y = s.y;
    m.c[2].z = s.z;
    return m;
}
// Mat4::perspective_rh: depth mapped to [0, 1].
inline M4 perspective_rh(float fov_y, float aspect, float z_near, float z_far) {
    const float h2 = 0.5f * fov_y;
    const float sin_fov = std::sin(h2), cos_fov = std::cos(h2);
    const float h = cos_fov / sin_fov;
    const float w = h / aspect;
    const float r = z_far / (z_near - z_far);
    M4 m;
    m.c[0] = {w, 0.0f, 0.0f, 0.0f};
    m.c[1] = {0.0f, h, 0.0f, 0.0f};
    m.c[2] = {0.0f, 0.0f, r, -1.0f};
    m.c[3] = {0.0f, 0.0f, r * z_near, 0.0f};
    return m;
}

}  // namespace swr
