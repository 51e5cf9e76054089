// ref_math.hpp -- scalar math of the CPU oracle (test infrastructure only).
//
// The oracle is the checker for the GPU step: only tests, the smoke check and
// the CPU-baseline leg of the benchmark load it. Nothing in the product links it.
//
// Every operation is written out element by element in the order nalgebra
// 0.28 evaluates it (sequential sums, no fused multiply-add: the oracle is
// compiled with -ffp-contract=off), so that the f32 instantiation is a
// faithful single-precision restatement of the reference and the CUDA kernels
// can reproduce it operation for operation.
#pragma once
#include <cmath>
#include <cstdint>
#include <algorithm>

namespace oracle {

template <class R> struct V3 {
    R x, y, z;
};
template <class R> inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> vdiv(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
// Vector3::dot: a0*b0 + a1*b1 + a2*b2 evaluated left to right.
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// Vector3::cross.
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R norm2(V3<R> a) { return dot(a, a); }
template <class R> inline R norm(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> inline V3<R> cmul(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline R comp(V3<R> a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
template <class R> inline void setc(V3<R>& a, int k, R v) {
    if (k == 0) a.x = v; else if (k == 1) a.y = v; else a.z = v;
}

// nalgebra Quaternion storage: (i, j, k, w).
template <class R> struct Quat {
    R i, j, k, w;
};
template <class R> inline V3<R> qvec(Quat<R> q) { return {q.i, q.j, q.k}; }
// UnitQuaternion * Vector3 (nalgebra): t = 2 (q_v x v); v' = t*w + q_v x t + v.
template <class R> inline V3<R> qrot(Quat<R> q, V3<R> v) {
    V3<R> qv = qvec(q);
    V3<R> c = cross(qv, v);
    V3<R> t = c * R(2);
    V3<R> c2 = cross(qv, t);
    return (t * q.w + c2) + v;
}
template <class R> inline Quat<R> qconj(Quat<R> q) { return {-q.i, -q.j, -q.k, q.w}; }
template <class R> inline V3<R> qrot_inv(Quat<R> q, V3<R> v) { return qrot(qconj(q), v); }
// Quaternion * Quaternion (Hamilton product in nalgebra's expression order).
template <class R> inline Quat<R> qmul(Quat<R> a, Quat<R> b) {
    Quat<R> r;
    r.w = a.w * b.w - a.i * b.i - a.j * b.j - a.k * b.k;
    r.i = a.w * b.i + a.i * b.w + a.j * b.k - a.k * b.j;
    r.j = a.w * b.j - a.i * b.k + a.j * b.w + a.k * b.i;
    r.k = a.w * b.k + a.i * b.j - a.j * b.i + a.k * b.w;
    return r;
}
// UnitQuaternion::new(axisangle) = exp(axisangle / 2): w = cos(n), v = h sin(n)/n
// with h = axisangle/2 and n = |h|.
// f32: for n < 1/4, cos(n) and sin(n)/n are their Maclaurin series truncated
// after the n^10 term, by Horner's rule in f32 (the GPU evaluates the same
// polynomial); larger angles use sin and cos in double, rounded to f32.
// f64: std::sin / std::cos.
inline void sinc_cos_small(float nn, float& sinc, float& c) {
    c = 1.0f + nn * (-0.5f + nn * (4.16666679e-02f + nn * (-1.38888892e-03f + nn * (2.48015876e-05f +
                                                                                   nn * (-2.75573188e-07f)))));
    sinc = 1.0f + nn * (-1.66666672e-01f + nn * (8.33333377e-03f + nn * (-1.98412701e-04f + nn * (2.75573188e-06f +
                                                                                                 nn * (-2.50521079e-08f)))));
}
template <class R> inline void sinc_cos(R nn, R& f, R& c) {
    R n = std::sqrt(nn);
    c = std::cos(n);
    f = std::sin(n) / n;
}
template <> inline void sinc_cos<float>(float nn, float& f, float& c) {
    if (nn < 0.0625f) {
        sinc_cos_small(nn, f, c);
        return;
    }
    float n = std::sqrt(nn);
    float s = float(std::sin(double(n)));
    c = float(std::cos(double(n)));
    f = s / n;
}
template <class R> inline Quat<R> qexp_scaled_axis(V3<R> axisangle) {
    V3<R> h = vdiv(axisangle, R(2));
    R nn = dot(h, h);
    if (nn == R(0)) return Quat<R>{R(0), R(0), R(0), R(1)};
    R f, c;
    sinc_cos(nn, f, c);
    V3<R> v = h * f;
    return Quat<R>{v.x, v.y, v.z, c};
}

// Row-major 3x3.
// UnitQuaternion::scaled_axis: the axis (the vector part, negated when
// w < 0, normalised; zero when it vanishes) times the angle 2 acos(|w|)
// (0 when |w| >= 1). In f32 acos is taken in double and rounded, as the GPU does.
template <class R> inline V3<R> qscaled_axis(Quat<R> q) {
    V3<R> v = q.w >= R(0) ? qvec(q) : -qvec(q);
    R sq = dot(v, v);
    if (!(sq > R(0))) return v3<R>(R(0), R(0), R(0));
    V3<R> axis = vdiv(v, R(std::sqrt(sq)));
    R aw = std::fabs(q.w);
    R angle = aw >= R(1) ? R(0) : R(std::acos(double(aw))) * R(2);
    return axis * angle;
}

template <class R> struct M3 {
    R m[3][3];
};
template <class R> inline M3<R> mzero() {
    M3<R> r;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) r.m[a][b] = R(0);
    return r;
}
template <class R> inline V3<R> mrow(const M3<R>& a, int r) { return {a.m[r][0], a.m[r][1], a.m[r][2]}; }
template <class R> inline V3<R> mcol(const M3<R>& a, int c) { return {a.m[0][c], a.m[1][c], a.m[2][c]}; }
// Matrix3 * Vector3 (gemv: columns accumulated in order).
template <class R> inline V3<R> mv(const M3<R>& a, V3<R> v) {
    return {a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z,
            a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
            a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z};
}
template <class R> inline M3<R> mm(const M3<R>& a, const M3<R>& b) {
    M3<R> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return r;
}
template <class R> inline M3<R> mtr(const M3<R>& a) {
    M3<R> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i];
    return r;
}
template <class R> inline M3<R> madd(const M3<R>& a, const M3<R>& b) {
    M3<R> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j];
    return r;
}
template <class R> inline M3<R> msub(const M3<R>& a, const M3<R>& b) {
    M3<R> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] - b.m[i][j];
    return r;
}
template <class R> inline M3<R> mscale(const M3<R>& a, R s) {
    M3<R> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] * s;
    return r;
}
// Vector3::cross_matrix (gcross_matrix in 3D, src/utils/generalized_cross.rs:69-84).
template <class R> inline M3<R> cross_matrix(V3<R> v) {
    M3<R> r = mzero<R>();
    r.m[0][1] = -v.z; r.m[0][2] = v.y;
    r.m[1][0] = v.z;  r.m[1][2] = -v.x;
    r.m[2][0] = -v.y; r.m[2][1] = v.x;
    return r;
}
// UnitQuaternion::to_rotation_matrix (nalgebra).
template <class R> inline M3<R> qmat(Quat<R> q) {
    R i = q.i, j = q.j, k = q.k, w = q.w;
    R ww = w * w, ii = i * i, jj = j * j, kk = k * k;
    R ij = i * j * R(2), wk = w * k * R(2), wj = w * j * R(2);
    R ik = i * k * R(2), jk = j * k * R(2), wi = w * i * R(2);
    M3<R> r;
    r.m[0][0] = ww + ii - jj - kk; r.m[0][1] = ij - wk;           r.m[0][2] = wj + ik;
    r.m[1][0] = wk + ij;           r.m[1][1] = ww - ii + jj - kk; r.m[1][2] = jk - wi;
    r.m[2][0] = ik - wj;           r.m[2][1] = wi + jk;           r.m[2][2] = ww - ii - jj + kk;
    return r;
}
// Matrix3::try_inverse (cofactor expansion along the first row; zero when singular),
// as used by Inertia3::inverse (src/algebra/inertia3.rs:75-86).
template <class R> inline M3<R> minv_or_zero(const M3<R>& a) {
    R m11 = a.m[0][0], m12 = a.m[0][1], m13 = a.m[0][2];
    R m21 = a.m[1][0], m22 = a.m[1][1], m23 = a.m[1][2];
    R m31 = a.m[2][0], m32 = a.m[2][1], m33 = a.m[2][2];
    R minor_m12_m23 = m22 * m33 - m32 * m23;
    R minor_m11_m23 = m21 * m33 - m31 * m23;
    R minor_m11_m22 = m21 * m32 - m31 * m22;
    R det = m11 * minor_m12_m23 - m12 * minor_m11_m23 + m13 * minor_m11_m22;
    M3<R> r = mzero<R>();
    if (det == R(0)) return r;
    r.m[0][0] = minor_m12_m23 / det;
    r.m[0][1] = (m13 * m32 - m33 * m12) / det;
    r.m[0][2] = (m12 * m23 - m22 * m13) / det;
    r.m[1][0] = -minor_m11_m23 / det;
    r.m[1][1] = (m11 * m33 - m31 * m13) / det;
    r.m[1][2] = (m13 * m21 - m23 * m11) / det;
    r.m[2][0] = minor_m11_m22 / det;
    r.m[2][1] = (m12 * m31 - m32 * m11) / det;
    r.m[2][2] = (m11 * m22 - m21 * m12) / det;
    return r;
}

template <class R> struct Iso {
    V3<R> t;
    Quat<R> q;
};
template <class R> inline Iso<R> iso_identity() { return Iso<R>{{R(0), R(0), R(0)}, {R(0), R(0), R(0), R(1)}}; }
// Isometry * Point.
template <class R> inline V3<R> iso_pt(const Iso<R>& a, V3<R> p) { return qrot(a.q, p) + a.t; }
// Isometry::inverse_transform_point.
template <class R> inline V3<R> iso_inv_pt(const Iso<R>& a, V3<R> p) { return qrot_inv(a.q, p - a.t); }
// Isometry * Isometry (nalgebra: t = t1 + q1*t2, q = q1 q2).
template <class R> inline Iso<R> iso_mul(const Iso<R>& a, const Iso<R>& b) {
    Iso<R> r;
    r.t = a.t + qrot(a.q, b.t);
    r.q = qmul(a.q, b.q);
    return r;
}

// Symmetric-or-not inertia: mass + angular 3x3 (Inertia3, src/algebra/inertia3.rs).
template <class R> struct Inertia {
    R linear;
    M3<R> angular;
};

}  // namespace oracle
