// geom.cuh — orientation geometry of the icosahedral path, host + device.
//
// FP32 with the reference's operation order.  Translation units that include this
// header are compiled without multiply-add contraction (-fmad=false on the device,
// -ffp-contract=off on the host) so each expression rounds exactly where the
// Fortran does.
#pragma once
#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define CI_HD __host__ __device__ __forceinline__
#else
#define CI_HD inline
#endif

namespace cryoim {

// pi and the degree conversions as every reference routine derives them:
// atan2(1.,1.) = pi/4 in FP32, then 4*, 8*, /45, 45/ (all one rounding).
struct Angles {
    float q, pi, tpi, deg2rad, rad2deg;
};
inline Angles host_angles() {
    Angles a;
    a.q = std::atan2(1.0f, 1.0f);
    a.pi = 4.0f * a.q;
    a.tpi = 8.0f * a.q;
    a.deg2rad = a.q / 45.0f;
    a.rad2deg = 45.0f / a.q;
    return a;
}

// icosprocess/SRC/euler_mat.f90:3-21  (ZYZ, R = Rz(phi) Ry(theta) Rz(omega)), m[r*3+c].
CI_HD void euler_mat(float theta0, float phi0, float omega0, float d2r, float* m) {
    float theta = theta0 * d2r, phi = phi0 * d2r, omega = omega0 * d2r;
    float c1 = cosf(phi), c2 = cosf(theta), c3 = cosf(omega);
    float s1 = sinf(phi), s2 = sinf(theta), s3 = sinf(omega);
    m[0] = c1 * c2 * c3 - s1 * s3;  m[1] = -c1 * c2 * s3 - c3 * s1; m[2] = c1 * s2;
    m[3] = c2 * c3 * s1 + c1 * s3;  m[4] = -c2 * s1 * s3 + c1 * c3; m[5] = s1 * s2;
    m[6] = -c3 * s2;                m[7] = s2 * s3;                 m[8] = c2;
}

CI_HD void mv3(const float* a, const float* v, float* o) {
    float t0 = a[0] * v[0]; t0 = t0 + a[1] * v[1]; t0 = t0 + a[2] * v[2];
    float t1 = a[3] * v[0]; t1 = t1 + a[4] * v[1]; t1 = t1 + a[5] * v[2];
    float t2 = a[6] * v[0]; t2 = t2 + a[7] * v[1]; t2 = t2 + a[8] * v[2];
    o[0] = t0; o[1] = t1; o[2] = t2;
}
CI_HD void mtv3(const float* a, const float* v, float* o) {  // transpose(a) * v
    float t0 = a[0] * v[0]; t0 = t0 + a[3] * v[1]; t0 = t0 + a[6] * v[2];
    float t1 = a[1] * v[0]; t1 = t1 + a[4] * v[1]; t1 = t1 + a[7] * v[2];
    float t2 = a[2] * v[0]; t2 = t2 + a[5] * v[1]; t2 = t2 + a[8] * v[2];
    o[0] = t0; o[1] = t1; o[2] = t2;
}
CI_HD void mm3(const float* a, const float* b, float* c) {
    float t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            float s = a[i * 3 + 0] * b[0 * 3 + j];
            s = s + a[i * 3 + 1] * b[1 * 3 + j];
            s = s + a[i * 3 + 2] * b[2 * 3 + j];
            t[i * 3 + j] = s;
        }
    for (int k = 0; k < 9; ++k) c[k] = t[k];
}

// icosprocess/SRC/icos_crosslin_angle.f90:2-37 for one symmetry operator s:
// the common line of image 1 (e1) and the s-rotated image 2 (e2), as in-plane angles
// alpha1/alpha2 in degrees; both 1000 when |z1 x s z2| < 0.5.
CI_HD void crosslin_pair(const float* e1, const float* e2, const float* s, float r2d,
                         float* alpha1, float* alpha2) {
    float z1[3] = {e1[2], e1[5], e1[8]};
    float z2[3] = {e2[2], e2[5], e2[8]};
    float z2a[3];
    mv3(s, z2, z2a);
    float v[3];
    v[0] = z1[1] * z2a[2] - z1[2] * z2a[1];
    v[1] = z1[2] * z2a[0] - z1[0] * z2a[2];
    v[2] = z1[0] * z2a[1] - z1[1] * z2a[0];
    float vv = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (vv < 0.5f) { *alpha1 = 1000.0f; *alpha2 = 1000.0f; return; }
    v[0] = v[0] / vv; v[1] = v[1] / vv; v[2] = v[2] / vv;
    float v10[3], t[3], v20[3];
    mtv3(e1, v, v10);
    mtv3(s, v, t);
    mtv3(e2, t, v20);
    *alpha1 = atan2f(v10[1], v10[0]) * r2d;
    *alpha2 = atan2f(v20[1], v20[0]) * r2d;
}

// Asymmetric-unit planes: icosprocess/SRC/ort_globesearch.f90:17-18 and
// return_icos_asymmetry_unit.f90:9-12 (same six numbers).
struct AsuPlanes {
    float A1, B1, C1, A2, B2, C2;
};
CI_HD AsuPlanes asu_planes(float d2r) {
    float c31 = cosf(31.717f * d2r), s31 = sinf(31.717f * d2r);
    float c69 = cosf(69.09f * d2r), s69 = sinf(69.09f * d2r);
    AsuPlanes p;
    p.A1 = -s31 * c69; p.B1 = -c31 * c69; p.C1 = s31 * s69;
    p.A2 = -s31 * c69; p.B2 = c31 * c69;  p.C2 = s31 * s69;
    return p;
}
CI_HD bool asu_inside(const AsuPlanes& p, float x, float y, float z) {
    float z1 = -(p.A1 * x + p.B1 * y) / p.C1;
    float z2 = -(p.A2 * x + p.B2 * y) / p.C2;
    return (z >= 0.0f) && (z <= z1) && (z <= z2);
}

// icosprocess/SRC/return_icos_asymmetry_unit.f90:1-33: the first operator (table
// order) that brings the view direction into the asymmetric unit.  The acos argument
// is clamped to [-1, 1] (the Fortran would return NaN just outside it).
CI_HD void asu_fold(float* theta, float* phi, float* omega, const float* ops, float d2r) {
    AsuPlanes pl = asu_planes(d2r);
    float e[9];
    euler_mat(*theta, *phi, *omega, d2r, e);
    float th = 0.f, ph = 0.f, om = 0.f;
    for (int i = 0; i < 60; ++i) {
        float m[9];
        mm3(ops + i * 9, e, m);
        float m33 = fminf(1.0f, fmaxf(-1.0f, m[8]));
        th = acosf(m33);
        ph = atan2f(m[5], m[2]);
        om = atan2f(m[7], -m[6]);
        float x = sinf(th) * cosf(ph);
        float y = sinf(th) * sinf(ph);
        float z = cosf(th);
        if (asu_inside(pl, x, y, z)) break;
    }
    *theta = th / d2r;
    *phi = ph / d2r;
    *omega = om / d2r;
}

}  // namespace cryoim
