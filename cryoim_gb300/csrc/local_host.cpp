// local_host.cpp — host side of the localized-reconstruction inputs: the symmetry
// rotations and sub-particle coordinates of local_box, and local_refine's parameters.
// FP32 throughout, built with -ffp-contract=off so every product and sum rounds where
// the Fortran reference rounds.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/cryoim.h"

namespace {

using M3 = float[3][3];  // m[i][j] = row i, column j

void matmul(const M3 a, const M3 b, M3 out) {
    float t[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            float s = a[i][0] * b[0][j];
            s = s + a[i][1] * b[1][j];
            s = s + a[i][2] * b[2][j];
            t[i][j] = s;
        }
    std::memcpy(out, t, sizeof(t));
}

void transpose(const M3 a, M3 out) {
    float t[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i][j] = a[j][i];
    std::memcpy(out, t, sizeof(t));
}

// C_matrix.f90:1-17: rotations by 2 pi k / N about z, k = 1..N (the last is identity)
void c_matrix(int n, float* out) {
    const float pi = 4.0f * std::atan2(1.0f, 1.0f);
    const float phi = 2.0f * pi / (float)n;
    M3 r1 = {{std::cos(phi), -std::sin(phi), 0.0f}, {std::sin(phi), std::cos(phi), 0.0f}, {0.0f, 0.0f, 1.0f}};
    M3 cur;
    std::memcpy(cur, r1, sizeof(M3));
    std::memcpy(out, cur, sizeof(M3));
    for (int i = 1; i < n; ++i) {
        matmul(cur, r1, cur);
        std::memcpy(out + 9 * i, cur, sizeof(M3));
    }
}

// icos_matrix_i2.f90:1-58: 5-fold about the axis tilted by v from z, then the 2-folds
// about x and y and the 3-fold permutation, 60 rotations in that generation order
void icos_i2(float* out) {
    const float d2r = 4.0f * std::atan2(1.0f, 1.0f) / 180.0f;
    const float a5 = 72.0f * d2r;
    const float v = std::acos(std::cos(60.0f * d2r) / std::sin(36.0f * d2r));
    M3 rz5 = {{std::cos(a5), -std::sin(a5), 0.0f}, {std::sin(a5), std::cos(a5), 0.0f}, {0.0f, 0.0f, 1.0f}};
    M3 ryv = {{std::cos(v), 0.0f, std::sin(v)}, {0.0f, 1.0f, 0.0f}, {-std::sin(v), 0.0f, std::cos(v)}};
    M3 t, ryvT;
    transpose(ryv, ryvT);
    matmul(rz5, ryvT, t);
    matmul(ryv, t, rz5);
    M3 rx2 = {{1.0f, 0.0f, 0.0f}, {0.0f, -1.0f, 0.0f}, {0.0f, 0.0f, -1.0f}};
    M3 ry2 = {{-1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, -1.0f}};
    M3 r3 = {{0.0f, 0.0f, 1.0f}, {1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}};
    M3 r[60];
    std::memset(r, 0, sizeof(r));
    r[0][0][0] = r[0][1][1] = r[0][2][2] = 1.0f;
    for (int i = 1; i < 5; ++i) matmul(r[i - 1], rz5, r[i]);
    for (int i = 5; i < 10; ++i) matmul(rx2, r[i - 5], r[i]);
    for (int i = 10; i < 20; ++i) matmul(ry2, r[i - 10], r[i]);
    for (int i = 20; i < 40; ++i) matmul(r3, r[i - 20], r[i]);
    for (int i = 40; i < 60; ++i) matmul(r3, r[i - 20], r[i]);
    std::memcpy(out, r, sizeof(r));
}

// icos_matrix_i3.f90 / icos_matrix_i5.f90: the i2 set conjugated by a frame rotation
void icos_conj(float* out, const M3 rot0) {
    icos_i2(out);
    M3 t, rT;
    transpose(rot0, rT);
    for (int i = 0; i < 60; ++i) {
        M3 m;
        std::memcpy(m, out + 9 * i, sizeof(M3));
        matmul(m, rT, t);
        matmul(rot0, t, m);
        std::memcpy(out + 9 * i, m, sizeof(M3));
    }
}

// Eularmatrix.f90 (local_box): R = Rz(phi) Ry(theta) Rz(omega), degrees
void eularmatrix(float th0, float ph0, float om0, M3 r) {
    const float d2r = 4.0f * std::atan2(1.0f, 1.0f) / 180.0f;
    const float th = th0 * d2r, ph = ph0 * d2r, om = om0 * d2r;
    r[0][0] = std::cos(ph) * std::cos(th) * std::cos(om) - std::sin(ph) * std::sin(om);
    r[0][1] = -std::cos(ph) * std::cos(th) * std::sin(om) - std::sin(ph) * std::cos(om);
    r[0][2] = std::cos(ph) * std::sin(th);
    r[1][0] = std::sin(ph) * std::cos(th) * std::cos(om) + std::cos(ph) * std::sin(om);
    r[1][1] = -std::sin(ph) * std::cos(th) * std::sin(om) + std::cos(ph) * std::cos(om);
    r[1][2] = std::sin(ph) * std::sin(th);
    r[2][0] = -std::sin(th) * std::cos(om);
    r[2][1] = std::sin(th) * std::sin(om);
    r[2][2] = std::cos(th);
}

}  // namespace

extern "C" {

int cryoim_local_sym_matrices(const char* sym, float* out, int32_t* n) {
    if (!sym || !out || !n) return CRYOIM_ERR_ARG;
    const std::string s(sym);
    if (s == "i2" || s == "I2") {
        icos_i2(out);
        *n = 60;
    } else if (s == "i3" || s == "I3" || s == "i5" || s == "I5") {
        const float d2r = 4.0f * std::atan2(1.0f, 1.0f) / 180.0f;
        M3 rot0;
        if (s == "i5" || s == "I5") {
            const float v = std::acos(std::cos(60.0f * d2r) / std::sin(36.0f * d2r));
            M3 r = {{std::cos(v), 0.0f, std::sin(v)}, {0.0f, 1.0f, 0.0f}, {-std::sin(v), 0.0f, std::cos(v)}};
            std::memcpy(rot0, r, sizeof(M3));
        } else {
            const float w = std::acos(std::cos(36.0f * d2r) / std::sin(60.0f * d2r));
            M3 r = {{1.0f, 0.0f, 0.0f}, {0.0f, std::cos(-w), std::sin(-w)}, {0.0f, -std::sin(-w), std::cos(-w)}};
            std::memcpy(rot0, r, sizeof(M3));
        }
        icos_conj(out, rot0);
        *n = 60;
    } else if (s.size() >= 2 && (s[0] == 'c' || s[0] == 'C')) {
        const int k = std::atoi(s.c_str() + 1);
        if (k < 1 || k > 60) return CRYOIM_ERR_ARG;
        c_matrix(k, out);
        *n = k;
    } else {
        return CRYOIM_ERR_ARG;
    }
    return CRYOIM_OK;
}

int cryoim_local_box_coordinates(const cryoim_particle* parts, int32_t P, const float* sym, int32_t nsym,
                                 float loc_x, float loc_y, float loc_z, float apix, int32_t fftsize,
                                 float pr_threshold, float boundx, cryoim_local_particle* out,
                                 int32_t* nout) {
    if (!parts || !sym || !out || !nout || P < 0 || nsym < 1 || fftsize < 2) return CRYOIM_ERR_ARG;
    const float r2d = 45.0f / std::atan2(1.0f, 1.0f);
    const float x0[3] = {loc_x, loc_y, loc_z};
    const float h = (float)(fftsize / 2);
    int k = 0, np = 0;
    for (int i = 0; i < P; ++i) {
        const cryoim_particle& q = parts[i];
        if (!(q.pr <= pr_threshold && std::fabs(q.x) <= boundx && std::fabs(q.y) <= boundx)) continue;
        M3 e;
        eularmatrix(q.theta, q.phi, q.omega, e);
        for (int s = 0; s < nsym; ++s) {
            // equalort.f90:9-21
            M3 S, r;
            std::memcpy(S, sym + 9 * s, sizeof(M3));
            matmul(S, e, r);
            float th;
            if (r[2][2] >= 1.0f) th = 0.0f;
            else if (r[2][2] < -1.0f) th = 180.0f;
            else th = std::acos(r[2][2]) * r2d;
            const float ph = std::atan2(r[1][2], r[0][2]) * r2d;
            const float om = std::atan2(r[2][1], -r[2][0]) * r2d;
            // loc_box_coordinate.f90:20-32
            M3 rot;
            eularmatrix(th, ph, om, rot);
            float c[3];
            for (int a = 0; a < 3; ++a) {
                float t = rot[0][a] * x0[0];
                t = t + rot[1][a] * x0[1];
                t = t + rot[2][a] * x0[2];
                c[a] = t + h;
            }
            c[0] = c[0] + q.x;
            c[1] = c[1] + q.y;
            ++np;
            const int hx0 = (int)c[0], ky0 = (int)c[1];
            cryoim_local_particle& o = out[k++];
            std::memset(&o, 0, sizeof(o));
            o.particle_id = q.particle_id;
            o.img_id = q.img_id;
            o.img_particle_id = q.img_particle_id;
            o.theta = q.theta; o.phi = q.phi; o.omega = q.omega; o.x = q.x; o.y = q.y; o.pr = q.pr;
            o.df1 = q.df1 * 10000.0f;
            o.df2 = q.df2 * 10000.0f;
            o.astigang = q.astigang;
            o.local_img_id = s + 1;
            o.local_hx0 = hx0;
            o.local_ky0 = ky0;
            o.local_theta0 = th; o.local_phi0 = ph; o.local_omega0 = om;
            o.local_x0 = c[0] - (float)hx0;
            o.local_y0 = c[1] - (float)ky0;
            o.local_z0 = (c[2] - h) * apix;
            o.local_pr0 = q.pr;
        }
    }
    (void)np;
    *nout = k;
    return CRYOIM_OK;
}

}  // extern "C"

namespace cryoim {

// loc_box.f90:43-88 (the sub-image stack mode), geometry only: for every selected
// particle (load_ort.f90:30-34) and rotation s, the equivalent orientation
// (equalort.f90), the sub-image centre R^T (loc_x, loc_y, loc_z) split into an integer
// pixel (truncated) and a fraction, and the box's first pixel hx0 + nx0/2 - sub/2.
// Records as loc_box.f90:86-88 writes them (particle_id = the running sub-particle
// count, df as read); src[k] = the whole particle of record k.  Returns the count.
int local_box_stack_geometry(const cryoim_particle* parts, int P, const float* sym, int nsym, float loc_x,
                             float loc_y, float loc_z, float apix, int nx0, int sub, float pr_threshold,
                             float boundx, cryoim_local_particle* out, int* src) {
    const float r2d = 45.0f / std::atan2(1.0f, 1.0f);
    const float x0[3] = {loc_x, loc_y, loc_z};
    int k = 0;
    for (int i = 0; i < P; ++i) {
        const cryoim_particle& q = parts[i];
        if (!(q.pr <= pr_threshold && std::fabs(q.x) <= boundx && std::fabs(q.y) <= boundx)) continue;
        M3 e;
        eularmatrix(q.theta, q.phi, q.omega, e);
        for (int s = 0; s < nsym; ++s) {
            M3 S, r;
            std::memcpy(S, sym + 9 * s, sizeof(M3));
            matmul(S, e, r);
            float th;
            if (r[2][2] >= 1.0f) th = 0.0f;
            else if (r[2][2] < -1.0f) th = 180.0f;
            else th = std::acos(r[2][2]) * r2d;
            const float ph = std::atan2(r[1][2], r[0][2]) * r2d;
            const float om = std::atan2(r[2][1], -r[2][0]) * r2d;
            M3 rot;
            eularmatrix(th, ph, om, rot);
            float c[3];
            for (int a = 0; a < 3; ++a) {
                float t = rot[0][a] * x0[0];
                t = t + rot[1][a] * x0[1];
                t = t + rot[2][a] * x0[2];
                c[a] = t;
            }
            int hx0 = (int)c[0];
            const float fx = c[0] - (float)hx0;
            int ky0 = (int)c[1];
            const float fy = c[1] - (float)ky0;
            hx0 = hx0 + nx0 / 2 - sub / 2;
            ky0 = ky0 + nx0 / 2 - sub / 2;
            cryoim_local_particle& o = out[k];
            std::memset(&o, 0, sizeof(o));
            o.particle_id = k + 1;
            o.img_id = q.img_id;
            o.img_particle_id = q.img_particle_id;
            o.theta = q.theta; o.phi = q.phi; o.omega = q.omega; o.x = q.x; o.y = q.y; o.pr = q.pr;
            o.df1 = q.df1; o.df2 = q.df2; o.astigang = q.astigang;
            o.local_img_id = s + 1;
            o.local_hx0 = hx0;
            o.local_ky0 = ky0;
            o.local_theta0 = th; o.local_phi0 = ph; o.local_omega0 = om;
            o.local_x0 = fx;
            o.local_y0 = fy;
            o.local_z0 = c[2] * apix;
            o.local_pr0 = q.pr;
            src[k] = i;
            ++k;
        }
    }
    return k;
}

}  // namespace cryoim

extern "C" {

int cryoim_local_params_default(cryoim_local_params* p, int32_t fftsize, int32_t fftsize0) {
    if (!p || fftsize < 8 || fftsize0 < fftsize) return CRYOIM_ERR_ARG;
    std::memset(p, 0, sizeof(*p));
    p->fftsize = fftsize;
    p->fftsize0 = fftsize0;
    p->nsym = 1;
    p->ncycle = 12;
    p->apply_ctf = 1;
    p->normalize = 1;
    p->apix = 1.0f;
    p->max_res = 10.0f;
    p->imgmask = 0.0f;
    p->vol = 200.0f;
    p->cs = 2.7f;
    p->ampwg = 0.1f;
    p->refine_angle = 0.0f;
    p->refine_shift = 0.0f;
    p->convf = 0.8f;
    return cryoim_local_params_derive(p);
}

int cryoim_local_params_derive(cryoim_local_params* p) {
    if (!p || p->fftsize < 8 || !(p->apix > 0) || !(p->max_res > 0) || p->nsym < 1) return CRYOIM_ERR_ARG;
    // 0calc_initialvalue.f90:65-76
    p->imgmask_px = p->imgmask > 0.0f ? p->imgmask / p->apix : (float)(p->fftsize / 2 - 2);
    p->max_r = p->apix * (float)p->fftsize / p->max_res;
    if (p->refine_angle <= 0.0f) p->refine_angle = 360.0f / (p->max_r * std::sqrt(5.0f) * 3.14159f);
    if (p->refine_shift <= 0.0f) p->refine_shift = (float)p->fftsize / (p->max_r * std::sqrt(5.0f));
    return CRYOIM_OK;
}

}  // extern "C"
