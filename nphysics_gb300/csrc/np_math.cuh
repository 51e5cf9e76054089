// np_math.cuh -- f32 vector / quaternion / 3x3 math shared by the device
// kernels and the library's host code.
//
// Every expression is written element by element in nalgebra 0.28's
// evaluation order (sequential sums). The library is compiled without
// floating-point contraction (nvcc --fmad=false, host -ffp-contract=off), so
// each operation rounds exactly once, on the device as on the host.
#pragma once
#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define NP_HD __host__ __device__ __forceinline__
#else
#define NP_HD inline
#endif

namespace np {

struct V {
    float x, y, z;
};
NP_HD V mk(float x, float y, float z) { return V{x, y, z}; }
NP_HD V add(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
NP_HD V sub(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
NP_HD V neg(V a) { return V{-a.x, -a.y, -a.z}; }
NP_HD V mul(V a, float s) { return V{a.x * s, a.y * s, a.z * s}; }
NP_HD V divs(V a, float s) { return V{a.x / s, a.y / s, a.z / s}; }
NP_HD float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
NP_HD V cross(V a, V b) { return V{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
NP_HD float norm(V a) { return sqrtf(dot(a, a)); }
NP_HD float comp(V a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
NP_HD void setc(V& a, int k, float v) {
    if (k == 0) a.x = v;
    else if (k == 1) a.y = v;
    else a.z = v;
}

struct Q {
    float i, j, k, w;
};
NP_HD V qv(Q q) { return V{q.i, q.j, q.k}; }
// UnitQuaternion * Vector3: t = 2 (q_v x v); t*w + q_v x t + v.
NP_HD V qrot(Q q, V v) {
    V u = qv(q);
    V c = cross(u, v);
    V t = mul(c, 2.0f);
    V c2 = cross(u, t);
    return add(add(mul(t, q.w), c2), v);
}
NP_HD Q qconj(Q q) { return Q{-q.i, -q.j, -q.k, q.w}; }
NP_HD V qrot_inv(Q q, V v) { return qrot(qconj(q), v); }
NP_HD Q qmul(Q a, Q b) {
    Q r;
    r.w = a.w * b.w - a.i * b.i - a.j * b.j - a.k * b.k;
    r.i = a.w * b.i + a.i * b.w + a.j * b.k - a.k * b.j;
    r.j = a.w * b.j - a.i * b.k + a.j * b.w + a.k * b.i;
    r.k = a.w * b.k + a.i * b.j - a.j * b.i + a.k * b.w;
    return r;
}
// UnitQuaternion::new(axisangle): the quaternion exponential of axisangle / 2,
// w = cos(n), v = h sin(n) / n with h = axisangle / 2, n = |h|.
// For n < 1/4 (every rotation of less than 1/2 rad per step) cos(n) and
// sin(n)/n come from their Maclaurin series truncated after the n^10 term
// (remainder below 2e-16), evaluated by Horner's rule in f32; larger angles
// take sin and cos in double, rounded to f32.
NP_HD void sinc_cos_small(float nn, float& sinc, float& c) {
    c = 1.0f + nn * (-0.5f + nn * (4.16666679e-02f + nn * (-1.38888892e-03f + nn * (2.48015876e-05f +
                                                                                   nn * (-2.75573188e-07f)))));
    sinc = 1.0f + nn * (-1.66666672e-01f + nn * (8.33333377e-03f + nn * (-1.98412701e-04f + nn * (2.75573188e-06f +
                                                                                                 nn * (-2.50521079e-08f)))));
}
NP_HD Q qexp(V axisangle) {
    V h = divs(axisangle, 2.0f);
    float nn = dot(h, h);
    if (nn == 0.0f) return Q{0.0f, 0.0f, 0.0f, 1.0f};
    float f, c;
    if (nn < 0.0625f) {
        sinc_cos_small(nn, f, c);
    } else {
        float n = sqrtf(nn);
        float s = (float)sin((double)n);
        c = (float)cos((double)n);
        f = s / n;
    }
    V v = mul(h, f);
    return Q{v.x, v.y, v.z, c};
}

// UnitQuaternion::scaled_axis: the axis (the vector part, negated when
// w < 0, normalised; zero when it vanishes) times the angle 2 acos(|w|)
// (0 when |w| >= 1). acos is taken in double and rounded to f32.
NP_HD V qscaled_axis(Q q) {
    V v = q.w >= 0.0f ? qv(q) : neg(qv(q));
    float sq = dot(v, v);
    if (!(sq > 0.0f)) return V{0.0f, 0.0f, 0.0f};
    V axis = divs(v, sqrtf(sq));
    float aw = fabsf(q.w);
    float angle = aw >= 1.0f ? 0.0f : (float)acos((double)aw) * 2.0f;
    return mul(axis, angle);
}

struct M {
    float m[3][3];
};
NP_HD M mzero() {
    M r;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) r.m[a][b] = 0.0f;
    return r;
}
NP_HD V mcol(const M& a, int c) { return V{a.m[0][c], a.m[1][c], a.m[2][c]}; }
NP_HD V mv(const M& a, V v) {
    return V{a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z, a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
             a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z};
}
NP_HD M mm(const M& a, const M& b) {
    M r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return r;
}
NP_HD M mtr(const M& a) {
    M r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i];
    return r;
}
NP_HD M madd(const M& a, const M& b) {
    M r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j];
    return r;
}
NP_HD M msub(const M& a, const M& b) {
    M r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] - b.m[i][j];
    return r;
}
NP_HD M mscale(const M& a, float s) {
    M r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] * s;
    return r;
}
NP_HD M cross_matrix(V v) {
    M r = mzero();
    r.m[0][1] = -v.z;
    r.m[0][2] = v.y;
    r.m[1][0] = v.z;
    r.m[1][2] = -v.x;
    r.m[2][0] = -v.y;
    r.m[2][1] = v.x;
    return r;
}
NP_HD M qmat(Q q) {
    float i = q.i, j = q.j, k = q.k, w = q.w;
    float ww = w * w, ii = i * i, jj = j * j, kk = k * k;
    float ij = i * j * 2.0f, wk = w * k * 2.0f, wj = w * j * 2.0f;
    float ik = i * k * 2.0f, jk = j * k * 2.0f, wi = w * i * 2.0f;
    M r;
    r.m[0][0] = ww + ii - jj - kk;
    r.m[0][1] = ij - wk;
    r.m[0][2] = wj + ik;
    r.m[1][0] = wk + ij;
    r.m[1][1] = ww - ii + jj - kk;
    r.m[1][2] = jk - wi;
    r.m[2][0] = ik - wj;
    r.m[2][1] = wi + jk;
    r.m[2][2] = ww - ii - jj + kk;
    return r;
}
// Inverse by cofactors (zero when singular).
NP_HD M minv_or_zero(const M& a) {
    float m11 = a.m[0][0], m12 = a.m[0][1], m13 = a.m[0][2];
    float m21 = a.m[1][0], m22 = a.m[1][1], m23 = a.m[1][2];
    float m31 = a.m[2][0], m32 = a.m[2][1], m33 = a.m[2][2];
    float c11 = m22 * m33 - m32 * m23;
    float c12 = m21 * m33 - m31 * m23;
    float c13 = m21 * m32 - m31 * m22;
    float det = m11 * c11 - m12 * c12 + m13 * c13;
    M r = mzero();
    if (det == 0.0f) return r;
    r.m[0][0] = c11 / det;
    r.m[0][1] = (m13 * m32 - m33 * m12) / det;
    r.m[0][2] = (m12 * m23 - m22 * m13) / det;
    r.m[1][0] = -c12 / det;
    r.m[1][1] = (m11 * m33 - m31 * m13) / det;
    r.m[1][2] = (m13 * m21 - m23 * m11) / det;
    r.m[2][0] = c13 / det;
    r.m[2][1] = (m12 * m31 - m32 * m11) / det;
    r.m[2][2] = (m11 * m22 - m21 * m12) / det;
    return r;
}

struct Iso {
    V t;
    Q q;
};
NP_HD V iso_pt(const Iso& a, V p) { return add(qrot(a.q, p), a.t); }
NP_HD V iso_inv_pt(const Iso& a, V p) { return qrot_inv(a.q, sub(p, a.t)); }
NP_HD Iso iso_mul(const Iso& a, const Iso& b) {
    Iso r;
    r.t = add(a.t, qrot(a.q, b.t));
    r.q = qmul(a.q, b.q);
    return r;
}

}  // namespace np
