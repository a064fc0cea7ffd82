/*
 * cryoim_oracle.cpp — CPU oracle of cryoIM's projection-matching path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, routine by routine, the Fortran of
 * chenwenyuan2009/cryoIM (icosprocess/SRC, proc_icos/SRC) so that the GPU library
 * can be checked against it.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py load it; libcryoim_gb300.so never links or calls it.
 *
 * Every routine is a template on the arithmetic type R:
 *   R = float  -> "_f32" exports: FP32 with the Fortran's evaluation order (left to
 *                 right, one rounding per operation; build with -ffp-contract=off),
 *                 the same single-precision libm calls the reference makes;
 *   R = double -> "_f64" exports: the same algorithm in FP64 (the precision judge).
 *
 * Parity status: the reference is Fortran and cannot be built in this image (no
 * Fortran compiler, no FFTW/MKL) and ships no tests or fixtures, so the oracle is
 * pinned only by (1) the 60-operator table extracted from icos2f_sym_mat.f90 into
 * tests/golden, (2) analytic known-answer tests, (3) scipy.fft for the FFT.
 * Everything else is "parity unpinned" against the running reference.
 *
 * Conventions: arrays are 0-based; the reference's 1-based index i maps to i-1.
 * Images are nx*nx with x fastest; 3D arrays nx^3 with x fastest.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/cryoim.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* ------------------------------------------------------------------------ */
/* constants: every routine of the reference derives pi from atan2(1.,1.)    */
/* ------------------------------------------------------------------------ */
template <class R> struct C {
    static R q() { return std::atan2(R(1), R(1)); }
    static R pi() { return R(4) * q(); }                 /* 4.0*atan2(1.0,1.0)  */
    static R tpi() { return R(8) * q(); }                /* 8.0*atan2(1.0,1.0)  */
    static R deg2rad() { return q() / R(45); }           /* atan2(1.0,1.0)/45.0 */
    static R rad2deg() { return R(45) / q(); }           /* 45.0/atan2(1.0,1.0) */
};

/* Fortran int() truncates toward zero. */
template <class R> inline int fint(R x) { return (int)x; }

/* ------------------------------------------------------------------------ */
/* geometry                                                                  */
/* ------------------------------------------------------------------------ */

/* icosprocess/SRC/euler_mat.f90:3-21 (ZYZ: R = Rz(phi) Ry(theta) Rz(omega)). m[r*3+c]. */
template <class R> void euler_mat(R theta0, R phi0, R omega0, R* m) {
    const R d2r = C<R>::deg2rad();
    R theta = theta0 * d2r, phi = phi0 * d2r, omega = omega0 * d2r;
    R c1 = std::cos(phi), c2 = std::cos(theta), c3 = std::cos(omega);
    R s1 = std::sin(phi), s2 = std::sin(theta), s3 = std::sin(omega);
    m[0] = c1 * c2 * c3 - s1 * s3;  m[1] = -c1 * c2 * s3 - c3 * s1; m[2] = c1 * s2;
    m[3] = c2 * c3 * s1 + c1 * s3;  m[4] = -c2 * s1 * s3 + c1 * c3; m[5] = s1 * s2;
    m[6] = -c3 * s2;                m[7] = s2 * s3;                 m[8] = c2;
}

/* proc_icos/SRC/Eularmatrix.f90:1-15: the same rotation with its own product order. */
template <class R> void eular_matrix(R theta0, R phi0, R omega0, R* r) {
    const R d2r = R(4) * C<R>::q() / R(180);
    R theta = theta0 * d2r, phi = phi0 * d2r, omega = omega0 * d2r;
    r[0] = std::cos(phi) * std::cos(theta) * std::cos(omega) - std::sin(phi) * std::sin(omega);
    r[1] = -std::cos(phi) * std::cos(theta) * std::sin(omega) - std::sin(phi) * std::cos(omega);
    r[2] = std::cos(phi) * std::sin(theta);
    r[3] = std::sin(phi) * std::cos(theta) * std::cos(omega) + std::cos(phi) * std::sin(omega);
    r[4] = -std::sin(phi) * std::cos(theta) * std::sin(omega) + std::cos(phi) * std::cos(omega);
    r[5] = std::sin(phi) * std::sin(theta);
    r[6] = -std::sin(theta) * std::cos(omega);
    r[7] = std::sin(theta) * std::sin(omega);
    r[8] = std::cos(theta);
}

/* c = a*b for 3x3 (sequential k sum, as matmul). */
template <class R> void mm3(const R* a, const R* b, R* c) {
    R t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            R s = a[i * 3 + 0] * b[0 * 3 + j];
            s = s + a[i * 3 + 1] * b[1 * 3 + j];
            s = s + a[i * 3 + 2] * b[2 * 3 + j];
            t[i * 3 + j] = s;
        }
    std::memcpy(c, t, sizeof(t));
}
template <class R> void mv3(const R* a, const R* v, R* o) {
    R t[3];
    for (int i = 0; i < 3; ++i) {
        R s = a[i * 3 + 0] * v[0];
        s = s + a[i * 3 + 1] * v[1];
        s = s + a[i * 3 + 2] * v[2];
        t[i] = s;
    }
    o[0] = t[0]; o[1] = t[1]; o[2] = t[2];
}
template <class R> void mtv3(const R* a, const R* v, R* o) { /* transpose(a)*v */
    R t[3];
    for (int i = 0; i < 3; ++i) {
        R s = a[0 * 3 + i] * v[0];
        s = s + a[1 * 3 + i] * v[1];
        s = s + a[2 * 3 + i] * v[2];
        t[i] = s;
    }
    o[0] = t[0]; o[1] = t[1]; o[2] = t[2];
}

/* The 60 rotations of the icosahedral group, 2-fold axes on x, y, z.
 * proc_icos/SRC/icos2f_operation_matrix.f90:7-55 builds them from generators:
 * a 5-fold about the axis tilted by v = acos(cos60/sin36) from z, the 2-folds about
 * x and y, and the 3-fold permutation about (1,1,1).  gen_ops() restates that
 * construction (arithmetic in R, as proc_icos does in FP32). */
template <class R> void gen_ops(R* r /* 60*9, generator order */) {
    const R d2r = R(4) * C<R>::q() / R(180);
    R a5 = R(72) * d2r;
    R v = std::acos(std::cos(R(60) * d2r) / std::sin(R(36) * d2r));
    R rz5[9] = {std::cos(a5), -std::sin(a5), 0, std::sin(a5), std::cos(a5), 0, 0, 0, 1};
    R ryv[9] = {std::cos(v), 0, std::sin(v), 0, 1, 0, -std::sin(v), 0, std::cos(v)};
    R ryvt[9] = {ryv[0], ryv[3], ryv[6], ryv[1], ryv[4], ryv[7], ryv[2], ryv[5], ryv[8]};
    R t[9];
    mm3(rz5, ryvt, t);
    mm3(ryv, t, rz5);
    const R rx2[9] = {1, 0, 0, 0, -1, 0, 0, 0, -1};
    const R ry2[9] = {-1, 0, 0, 0, 1, 0, 0, 0, -1};
    const R r3[9] = {0, 0, 1, 1, 0, 0, 0, 1, 0};
    for (int k = 0; k < 9; ++k) r[k] = (k % 4 == 0) ? R(1) : R(0);
    for (int i = 1; i < 5; ++i) mm3(r + (i - 1) * 9, rz5, r + i * 9);
    for (int i = 5; i < 10; ++i) mm3(rx2, r + (i - 5) * 9, r + i * 9);
    for (int i = 10; i < 20; ++i) mm3(ry2, r + (i - 10) * 9, r + i * 9);
    for (int i = 20; i < 60; ++i) mm3(r3, r + (i - 20) * 9, r + i * 9);
}

/* icosprocess/SRC/icos2f_sym_mat.f90:5-243 lists the same 60 matrices (14-digit
 * decimals) in its own order.  TABLE_FROM_GEN[k] is the generator index of table
 * entry k; the golden fixture extracted from that file pins it. */
const int TABLE_FROM_GEN[60] = {
    0, 26, 34, 48, 42, 24, 56, 28, 17, 23, 6, 52, 49, 41, 58, 9, 37, 18, 32, 54,
    36, 1, 2, 3, 4, 8, 29, 35, 45, 40, 20, 31, 7, 38, 22, 55, 30, 59, 51, 25,
    50, 19, 47, 43, 16, 27, 13, 12, 33, 15, 44, 14, 5, 11, 46, 57, 53, 21, 10, 39};

/* Table order; values are the exact group elements rounded to R (the table's
 * decimals round to the same floats). Entries are 0, +-1/2, +-phi/2, +-1/(2phi), +-1. */
template <class R> void icos_table(R* rot) {
    double g[540];
    gen_ops<double>(g);
    for (int k = 0; k < 60; ++k)
        for (int e = 0; e < 9; ++e) {
            double x = g[TABLE_FROM_GEN[k] * 9 + e];
            /* snap to the exact algebraic value (removes FP64 generator noise) */
            const double cand[5] = {0.0, 0.5, 1.0, 0.80901699437494742, 0.30901699437494742};
            double ax = std::fabs(x), best = cand[0];
            for (double c : cand)
                if (std::fabs(ax - c) < std::fabs(ax - best)) best = c;
            rot[k * 9 + e] = (R)(x < 0 ? -best : best);
        }
}

template <class R> const R* icos_ops() {
    static R tab[540];
    static bool init = false;
    if (!init) { icos_table<R>(tab); init = true; }
    return tab;
}

/* icosprocess/SRC/icos_crosslin_angle.f90:2-37. alpha in degrees; 1000 = no line. */
template <class R>
void crosslin_angle(R th1, R ph1, R om1, R th2, R ph2, R om2, R* alpha1, R* alpha2) {
    const R r2d = C<R>::rad2deg();
    R e1[9], e2[9];
    euler_mat(th1, ph1, om1, e1);
    euler_mat(th2, ph2, om2, e2);
    R z1[3] = {e1[2], e1[5], e1[8]}, z2[3] = {e2[2], e2[5], e2[8]};
    const R* rot = icos_ops<R>();
    for (int i = 0; i < 60; ++i) {
        const R* s = rot + i * 9;
        R z2a[3];
        mv3(s, z2, z2a);
        R v[3];
        v[0] = z1[1] * z2a[2] - z1[2] * z2a[1];
        v[1] = z1[2] * z2a[0] - z1[0] * z2a[2];
        v[2] = z1[0] * z2a[1] - z1[1] * z2a[0];
        R vv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (vv < R(0.5)) { alpha1[i] = R(1000); alpha2[i] = R(1000); continue; }
        v[0] = v[0] / vv; v[1] = v[1] / vv; v[2] = v[2] / vv;
        R v10[3], t[3], v20[3];
        mtv3(e1, v, v10);
        mtv3(s, v, t);
        mtv3(e2, t, v20);
        alpha1[i] = std::atan2(v10[1], v10[0]) * r2d;
        alpha2[i] = std::atan2(v20[1], v20[0]) * r2d;
    }
}

/* ASU planes of icosprocess/SRC/ort_globesearch.f90:17-18 / return_icos_asymmetry_unit.f90:9-12. */
template <class R> struct Asu {
    R A1, B1, C1, A2, B2, C2;
    Asu() {
        const R d2r = C<R>::deg2rad();
        R c31 = std::cos(R(31.717) * d2r), s31 = std::sin(R(31.717) * d2r);
        R c69 = std::cos(R(69.09) * d2r), s69 = std::sin(R(69.09) * d2r);
        A1 = -s31 * c69; B1 = -c31 * c69; C1 = s31 * s69;
        A2 = -s31 * c69; B2 = c31 * c69;  C2 = s31 * s69;
    }
    bool inside(R x, R y, R z) const {
        R z1 = -(A1 * x + B1 * y) / C1;
        R z2 = -(A2 * x + B2 * y) / C2;
        return (z >= R(0)) && (z <= z1) && (z <= z2);
    }
};

/* icosprocess/SRC/return_icos_asymmetry_unit.f90:1-33: first of the 60 ops (table
 * order) whose view direction lands in the ASU.  acos argument clamped to [-1,1]. */
template <class R> void asu_fold(R* theta, R* phi, R* omega) {
    const R d2r = C<R>::deg2rad();
    Asu<R> asu;
    R e[9];
    euler_mat(*theta, *phi, *omega, e);
    const R* rot = icos_ops<R>();
    R th = 0, ph = 0, om = 0;
    for (int i = 0; i < 60; ++i) {
        R m[9];
        mm3(rot + i * 9, e, m);
        R m33 = std::max(R(-1), std::min(R(1), m[8]));
        th = std::acos(m33);
        ph = std::atan2(m[5], m[2]);
        om = std::atan2(m[7], -m[6]);
        R x = std::sin(th) * std::cos(ph);
        R y = std::sin(th) * std::sin(ph);
        R z = std::cos(th);
        if (asu.inside(x, y, z)) break;
    }
    *theta = th / d2r;
    *phi = ph / d2r;
    *omega = om / d2r;
}

/* ------------------------------------------------------------------------ */
/* FFT (replaces FFTW3 via MKL, icosprocess/SRC/FFTW.f90:179-219)             */
/* ------------------------------------------------------------------------ */

/* In-place 1D complex DFT of length n with stride; sign -1 = forward (FFTW_FORWARD).
 * Radix-2 iterative for powers of two, direct O(n^2) otherwise.  Twiddles in FP64. */
template <class R> void dft1d(R* re, R* im, int n, long stride, int sign) {
    std::vector<R> xr(n), xi(n);
    for (int k = 0; k < n; ++k) { xr[k] = re[k * stride]; xi[k] = im[k * stride]; }
    const double PI = 3.14159265358979323846;
    if ((n & (n - 1)) == 0) {
        for (int i = 1, j = 0; i < n; ++i) {
            int bit = n >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) { std::swap(xr[i], xr[j]); std::swap(xi[i], xi[j]); }
        }
        for (int len = 2; len <= n; len <<= 1) {
            int h = len >> 1;
            for (int k = 0; k < h; ++k) {
                double ang = sign * 2.0 * PI * k / len;
                R wr = (R)std::cos(ang), wi = (R)std::sin(ang);
                for (int s = 0; s < n; s += len) {
                    R ur = xr[s + k], ui = xi[s + k];
                    R vr = xr[s + k + h] * wr - xi[s + k + h] * wi;
                    R vi = xr[s + k + h] * wi + xi[s + k + h] * wr;
                    xr[s + k] = ur + vr; xi[s + k] = ui + vi;
                    xr[s + k + h] = ur - vr; xi[s + k + h] = ui - vi;
                }
            }
        }
        for (int k = 0; k < n; ++k) { re[k * stride] = xr[k]; im[k * stride] = xi[k]; }
    } else {
        for (int k = 0; k < n; ++k) {
            double sr = 0, si = 0;
            for (int t = 0; t < n; ++t) {
                double ang = sign * 2.0 * PI * (double)((long)k * t % n) / n;
                sr += xr[t] * std::cos(ang) - xi[t] * std::sin(ang);
                si += xr[t] * std::sin(ang) + xi[t] * std::cos(ang);
            }
            re[k * stride] = (R)sr; im[k * stride] = (R)si;
        }
    }
}

/* icosprocess/SRC/img2d_FFT.f90:4-32 with FFTW.f90:179-194: forward normalised by
 * 1/(n1*n2), backward not; the result is returned as a = Re, b = -Im. */
template <class R> void img2d_fft(R* a, R* b, int n1, int n2, int nbit) {
    int sign = (nbit == 1) ? -1 : +1;
    for (int y = 0; y < n2; ++y) dft1d(a + (long)y * n1, b + (long)y * n1, n1, 1, sign);
    for (int x = 0; x < n1; ++x) dft1d(a + x, b + x, n2, n1, sign);
    long nn = (long)n1 * n2;
    if (nbit == 1) {
        R s = (R)(float)nn;
        for (long i = 0; i < nn; ++i) { a[i] = a[i] / s; b[i] = b[i] / s; }
    }
    for (long i = 0; i < nn; ++i) b[i] = -b[i];
}

/* 3D complex FFT on (re, im), n^3, x fastest; sign -1 forward (not normalised here). */
template <class R> void fft3d(R* re, R* im, int n, int sign) {
    long n2 = (long)n * n;
    for (long zy = 0; zy < n2; ++zy) dft1d(re + zy * n, im + zy * n, n, 1, sign);
    for (int z = 0; z < n; ++z)
        for (int x = 0; x < n; ++x) dft1d(re + z * n2 + x, im + z * n2 + x, n, n, sign);
    for (long yx = 0; yx < n2; ++yx) dft1d(re + yx, im + yx, n, n2, sign);
}

/* ------------------------------------------------------------------------ */
/* 2D image operations                                                       */
/* ------------------------------------------------------------------------ */

/* icosprocess/SRC/getCTF2d.f90:2-29 (defocus in um, Cs in mm, centred at nx/2). */
template <class R>
void get_ctf2d(int nx, R df10, R df20, R astig0, R apix, R vol, R cs0, R ampwg, R* ctf) {
    const R PI = C<R>::pi();
    const R d2r = PI / R(180);
    R lam = R(0.387818) / std::sqrt(R(1) * vol * (R(1) + R(0.978459E-3) * vol));
    R cs = cs0 * R(1.0e7), df1 = df10 * R(1.0e4), df2 = df20 * R(1.0e4);
    R astig = astig0 * d2r;
    R lam3 = lam * lam * lam;
    R sq = std::sqrt(R(1) - ampwg * ampwg);
    for (int i = 0; i < nx * nx; ++i) {
        int ky = i / nx - nx / 2, hx = i % nx - nx / 2;
        R phi = std::atan2((R)ky, (R)hx);
        if (phi < R(0)) phi = phi + R(2) * PI;
        phi = phi - astig;
        R c = std::cos(phi), s = std::sin(phi);
        R df = df1 * (c * c) + df2 * (s * s);
        R res = std::sqrt((R)(hx * hx + ky * ky)) / (R)nx / apix;
        R r2 = res * res, r4 = r2 * r2;
        R phase = R(2) * PI * (-(cs * lam3 * r4 / R(4)) + df * lam * r2 / R(2));
        ctf[i] = -(sq * std::sin(phase) + ampwg * std::cos(phase));
    }
}

/* icosprocess/SRC/img2d_mask.f90:2-49: cosine edge of half-width 6 px around
 * (OrigX+nx/2, OrigY+nx/2); outside filled with the edge-ring mean (FP64 sum). */
template <class R> void img2d_mask(R* d, int nx, R mask, R ox, R oy) {
    const R pi = C<R>::pi();
    const int halfw = 6;
    R R1 = mask - (R)(halfw / 2);
    if (R1 <= R(0)) R1 = R(0);
    R R2 = mask + (R)(halfw / 2);
    if (R2 > (R)(nx / 2)) R2 = (R)(nx / 2);
    R x0 = ox + (R)(nx / 2), y0 = oy + (R)(nx / 2);
    double summ = 0;
    int num = 0;
    for (int i = 0; i < nx * nx; ++i) {
        int iy = i / nx, ix = i % nx;
        R yy = (-y0 + (R)iy) * (-y0 + (R)iy);
        R xx = (-x0 + (R)ix) * (-x0 + (R)ix);
        R ra = std::sqrt(yy + xx);
        if (ra > R1 && ra <= R2) { summ = summ + (double)d[i]; num = num + 1; }
    }
    if (num != 0) summ = summ / (double)(float)num;
    for (int i = 0; i < nx * nx; ++i) {
        int iy = i / nx, ix = i % nx;
        R yy = (-y0 + (R)iy) * (-y0 + (R)iy);
        R xx = (-x0 + (R)ix) * (-x0 + (R)ix);
        R ra = std::sqrt(yy + xx);
        if (ra > R1 && ra <= R2) {
            R edge = (R(1) + std::cos(pi * (ra - R1) / (R)halfw)) / R(2);
            d[i] = (R)((double)(d[i] * edge) + (double)(R(1) - edge) * summ);
        }
        if (ra > R2) d[i] = (R)summ;
    }
}

/* icosprocess/SRC/img2d_FT_centshift.f90:2-18: F <- F exp(-i phase). */
template <class R> void centshift(R* a, R* b, int nx, R x0, R y0) {
    const R pi = C<R>::pi();
    for (int i = 0; i < nx * nx; ++i) {
        int ky = i / nx - nx / 2, hx = i % nx - nx / 2;
        R phase = R(2) * pi * ((x0 + (R)(nx / 2)) * (R)hx + (y0 + (R)(nx / 2)) * (R)ky) / (R)nx;
        R c = std::cos(phase), s = std::sin(phase);
        R fr = (a[i] * c + b[i] * s);
        R fi = (-a[i] * s + b[i] * c);
        a[i] = fr; b[i] = fi;
    }
}

/* icosprocess/SRC/img2d_norm.f90:1-22. */
template <class R> void img2d_norm(R* img, int nx) {
    R avg = 0, nd = 0;
    long nn = (long)nx * nx;
    for (long i = 0; i < nn; ++i) avg = avg + img[i];
    avg = avg / (R)(float)nn;
    for (long i = 0; i < nn; ++i) img[i] = img[i] - avg;
    for (long i = 0; i < nn; ++i) nd = nd + img[i] * img[i];
    nd = std::sqrt(nd / (R)(float)nn);
    for (long i = 0; i < nn; ++i) img[i] = img[i] / nd;
}

/* icosprocess/SRC/FT_amp_expfit.f90:2-47: least-squares fit of ln<|F|>(r) = x1 r + x2
 * over rings minR..maxR of the ky>=0 half plane; Fcut = 0.8 exp(x1 r + x2). */
template <class R> void ft_amp_expfit(const R* a, const R* b, int nx, int minR, int maxR, R* fcut) {
    int nr = maxR - minR + 1;
    std::vector<R> favg(nr, R(0)), resln(nr, R(0));
    std::vector<int> num(nr, 0);
    for (int ky = 0; ky <= maxR; ++ky)
        for (int hx = -maxR; hx <= maxR; ++hx) {
            R rad = std::sqrt((R)(hx * hx + ky * ky));
            int ir = fint(rad + R(0.5));
            if (ir >= minR && ir <= maxR) {
                int i = (ky + nx / 2) * nx + (hx + nx / 2);
                R amp = std::sqrt(a[i] * a[i] + b[i] * b[i]);
                favg[ir - minR] = favg[ir - minR] + amp;
                num[ir - minR] += 1;
                resln[ir - minR] = resln[ir - minR] + rad;
            }
        }
    for (int k = 0; k < nr; ++k) {
        if (num[k] > 0 && favg[k] > R(0)) {
            resln[k] = resln[k] / (R)num[k];
            favg[k] = std::log(favg[k] / (R)num[k]);
        } else {
            favg[k] = R(0);
        }
    }
    R aa11 = 0, aa12 = 0, aa22 = 0, bb1 = 0, bb2 = 0;
    for (int k = 0; k < nr; ++k) aa11 = aa11 + resln[k] * resln[k];
    for (int k = 0; k < nr; ++k) aa12 = aa12 + resln[k] * R(1);
    for (int k = 0; k < nr; ++k) aa22 = aa22 + R(1) * R(1);
    for (int k = 0; k < nr; ++k) bb1 = bb1 + resln[k] * favg[k];
    for (int k = 0; k < nr; ++k) bb2 = bb2 + R(1) * favg[k];
    R aa21 = aa12;
    R x2 = (bb2 - bb1 * aa21 / aa11) / (aa22 - aa12 * aa21 / aa11);
    R x1 = (bb1 - aa12 * x2) / aa11;
    for (int k = 0; k < nr; ++k) fcut[k] = std::exp(resln[k] * x1 + x2) * R(0.8);
}

/* ------------------------------------------------------------------------ */
/* common-line sampling and phase residual                                   */
/* ------------------------------------------------------------------------ */

template <class R> inline void bilin(const R* a, const R* b, int nx, R x, R y, R* o_re, R* o_im) {
    int lx = fint(x), ly = fint(y);
    R ax = x - (R)lx, ay = y - (R)ly;
    int n1 = nx * ly + lx, n2 = nx * (ly + 1) + lx;
    *o_re = (R(1) - ax) * (R(1) - ay) * a[n1] + ax * (R(1) - ay) * a[n1 + 1] +
            (R(1) - ax) * ay * a[n2] + ax * ay * a[n2 + 1];
    *o_im = (R(1) - ax) * (R(1) - ay) * b[n1] + ax * (R(1) - ay) * b[n1 + 1] +
            (R(1) - ax) * ay * b[n2] + ax * ay * b[n2 + 1];
}

/* icosprocess/SRC/img2d_fill_line.f90:1-36.  out: [nlin][nR][2] (zero for invalid). */
template <class R>
void fill_lin(int nlin, const R* a, const R* b, int nx, int minR, int maxR, const R* alpha, R* out) {
    const R d2r = C<R>::deg2rad();
    int nr = maxR - minR + 1;
    std::fill(out, out + (long)nlin * nr * 2, R(0));
    for (int i = 0; i < nlin; ++i) {
        if (!(alpha[i] < R(999))) continue;
        for (int fr = minR; fr <= maxR; ++fr) {
            R x = (R)fr * std::cos(alpha[i] * d2r) + (R)(nx / 2);
            R y = (R)fr * std::sin(alpha[i] * d2r) + (R)(nx / 2);
            R* o = out + ((long)i * nr + (fr - minR)) * 2;
            bilin(a, b, nx, x, y, o, o + 1);
        }
    }
}

/* icosprocess/SRC/img2d_fill_lin_omegearray.f90:1-42.  out: [nomega][nlin][nR][2]
 * (999 for invalid lines). */
template <class R>
void fill_lin_omega(int nlin, int nomega, R step, const R* a, const R* b, int nx, int minR,
                    int maxR, const R* alpha, R* out) {
    const R d2r = C<R>::deg2rad();
    int nr = maxR - minR + 1;
    std::fill(out, out + (long)nomega * nlin * nr * 2, R(999));
    for (int i = 0; i < nlin; ++i) {
        if (!(alpha[i] < R(999))) continue;
        for (int jj = 0; jj < nomega; ++jj) {
            R om = alpha[i] - step * (R)jj;
            R tmp = om * d2r;
            R cs = std::cos(tmp), sn = std::sin(tmp);
            for (int fr = minR; fr <= maxR; ++fr) {
                R x = (R)fr * cs + (R)(nx / 2);
                R y = (R)fr * sn + (R)(nx / 2);
                R* o = out + (((long)jj * nlin + i) * nr + (fr - minR)) * 2;
                bilin(a, b, nx, x, y, o, o + 1);
            }
        }
    }
}

/* Template FT times CTF (cal_crosslin_PR_omega.f90:34-42) and its amplitude cut. */
template <class R>
void tmpl_ctf(const R* tmpl, const R* ctf, int nx, int minR, int maxR, const R* fcut_noctf,
              std::vector<R>& a2, std::vector<R>& b2, R* fcut) {
    long nn = (long)nx * nx;
    a2.resize(nn); b2.resize(nn);
    int nr = maxR - minR + 1;
    if (ctf) {
        for (long k = 0; k < nn; ++k) { a2[k] = tmpl[k] * ctf[k]; b2[k] = tmpl[nn + k] * ctf[k]; }
        ft_amp_expfit(a2.data(), b2.data(), nx, minR, maxR, fcut);
    } else {
        for (long k = 0; k < nn; ++k) { a2[k] = tmpl[k]; b2[k] = tmpl[nn + k]; }
        std::copy(fcut_noctf, fcut_noctf + nr, fcut);
    }
}

/* icosprocess/SRC/cal_crosslin_PR_omega.f90:3-82.
 * pa/pb: shifted particle FT; fcut0: particle Fcut; tmpl: T x (a,b) x nx^2;
 * tort: T x (theta,phi,omega); tfcut: T x nR (no-CTF cuts); ctf: nx^2 or null. */
template <class R>
void pr_omega(const R* pa, const R* pb, const R* fcut0, const R* tmpl, const R* tort,
              const R* tfcut, const R* ctf, int T, int nx, int minR, int maxR, R step,
              int nomega, R theta, R phi, R omega, R* pr) {
    const R pi = C<R>::pi(), tpi = C<R>::tpi(), r2d = R(180) / pi, d2r = C<R>::deg2rad();
    int nr = maxR - minR + 1;
    long nn = (long)nx * nx;
    std::vector<R> pr1(nomega, R(0)), pr2(nomega, R(0));
    std::vector<R> a2, b2, fc(nr), line2((long)60 * nr * 2);
    std::vector<R> cs(nomega), sn(nomega);
    R al1[60], al2[60];
    for (int i = 0; i < T; ++i) {
        crosslin_angle(theta, phi, omega, tort[i * 3], tort[i * 3 + 1], tort[i * 3 + 2], al1, al2);
        tmpl_ctf(tmpl + (long)i * 2 * nn, ctf, nx, minR, maxR, tfcut + (long)i * nr, a2, b2, fc.data());
        fill_lin(60, a2.data(), b2.data(), nx, minR, maxR, al2, line2.data());
        for (int j = 0; j < 60; ++j) {
            if (!(al1[j] < R(999) && al2[j] < R(999))) continue;
            for (int jj = 0; jj < nomega; ++jj) {
                R om = al1[j] - step * (R)jj;
                R tmp = om * d2r;
                cs[jj] = std::cos(tmp); sn[jj] = std::sin(tmp);
            }
            for (int fr = minR; fr <= maxR; ++fr) {
                const R* l2 = line2.data() + ((long)j * nr + (fr - minR)) * 2;
                R amp2 = std::sqrt(l2[0] * l2[0] + l2[1] * l2[1]);
                if (!(amp2 >= fc[fr - minR])) continue;
                R ph2 = std::atan2(l2[1], l2[0]);
                for (int jj = 0; jj < nomega; ++jj) {
                    R x = (R)fr * cs[jj] + (R)(nx / 2);
                    R y = (R)fr * sn[jj] + (R)(nx / 2);
                    R re, im;
                    bilin(pa, pb, nx, x, y, &re, &im);
                    R amp1 = std::sqrt(re * re + im * im);
                    if (!(amp1 >= fcut0[fr - minR])) continue;
                    R ph1 = std::atan2(im, re);
                    R diff = std::fabs(ph2 - ph1);
                    diff = std::fmod(diff, tpi);
                    if (diff > pi) diff = tpi - diff;
                    amp1 = R(0.5) * (amp1 + amp2);
                    pr1[jj] = pr1[jj] + diff * amp1;
                    pr2[jj] = pr2[jj] + amp1;
                }
            }
        }
    }
    for (int jj = 0; jj < nomega; ++jj)
        pr[jj] = (pr2[jj] > R(1.0e-10)) ? pr1[jj] / pr2[jj] * r2d : R(999);
}

/* icosprocess/SRC/cal_crosslin_PR.f90:2-71 (candidate origin applied to a copy of
 * the unshifted particle FT). */
template <class R>
R pr_single(const R* pa0, const R* pb0, const R* fcut0, const R* tmpl, const R* tort,
            const R* tfcut, const R* ctf, int T, int nx, int minR, int maxR, R theta, R phi,
            R omega, R x0, R y0) {
    const R pi = C<R>::pi(), tpi = R(2) * pi;
    int nr = maxR - minR + 1;
    long nn = (long)nx * nx;
    std::vector<R> a1(pa0, pa0 + nn), b1(pb0, pb0 + nn);
    centshift(a1.data(), b1.data(), nx, x0, y0);
    std::vector<R> a2, b2, fc(nr), l1((long)60 * nr * 2), l2((long)60 * nr * 2);
    R al1[60], al2[60];
    R p1 = 0, p2 = 0;
    for (int i = 0; i < T; ++i) {
        crosslin_angle(theta, phi, omega, tort[i * 3], tort[i * 3 + 1], tort[i * 3 + 2], al1, al2);
        tmpl_ctf(tmpl + (long)i * 2 * nn, ctf, nx, minR, maxR, tfcut + (long)i * nr, a2, b2, fc.data());
        fill_lin(60, a1.data(), b1.data(), nx, minR, maxR, al1, l1.data());
        fill_lin(60, a2.data(), b2.data(), nx, minR, maxR, al2, l2.data());
        for (int j = 0; j < 60; ++j) {
            if (!(al1[j] < R(999) && al2[j] < R(999))) continue;
            for (int fr = minR; fr <= maxR; ++fr) {
                const R* u = l1.data() + ((long)j * nr + fr - minR) * 2;
                const R* w = l2.data() + ((long)j * nr + fr - minR) * 2;
                R amp1 = std::sqrt(u[0] * u[0] + u[1] * u[1]);
                R amp2 = std::sqrt(w[0] * w[0] + w[1] * w[1]);
                if (amp1 >= fcut0[fr - minR] && amp2 >= fc[fr - minR]) {
                    R ph1 = std::atan2(u[1], u[0]), ph2 = std::atan2(w[1], w[0]);
                    R diff = std::fabs(ph2 - ph1);
                    diff = std::fmod(diff, tpi);
                    if (diff > pi) diff = tpi - diff;
                    amp1 = R(0.5) * (amp1 + amp2);
                    p1 = p1 + diff * amp1;
                    p2 = p2 + amp1;
                }
            }
        }
    }
    if (p2 > R(1.0e-10)) return p1 / p2 * R(180) / pi;
    return R(1000);
}

/* Particle preprocessing of ort_globesearch.f90:49-55 / ort_refinement.f90:46-51:
 * mask, checkerboard, forward FFT, Fcut fit, optional origin shift. */
template <class R>
void prep_particle(const float* img, int nx, int use_mask, R imgmask, R x, R y, int shift,
                   int minR, int maxR, R* a, R* b, R* fcut) {
    long nn = (long)nx * nx;
    for (long i = 0; i < nn; ++i) a[i] = (R)img[i];
    if (use_mask) img2d_mask(a, nx, imgmask, x, y);
    for (long i = 0; i < nn; ++i) {
        int ky = (int)(i / nx), hx = (int)(i % nx);
        if ((hx + ky) & 1) a[i] = -a[i];
        b[i] = R(0);
    }
    img2d_fft(a, b, nx, nx, 1);
    ft_amp_expfit(a, b, nx, minR, maxR, fcut);
    if (shift) centshift(a, b, nx, x, y);
}

/* CTF cache of ort_globesearch.f90:60-66 / reconstruct.f90:84-90: a particle uses the
 * defocus of the first particle of its run of equal imgID. */
std::vector<int> ctf_source(const cryoim_particle* parts, int P) {
    std::vector<int> src(P);
    int id0 = -100, cur = -1;
    for (int i = 0; i < P; ++i) {
        if (parts[i].img_id != id0) { cur = i; id0 = parts[i].img_id; }
        src[i] = cur;
    }
    return src;
}

/* icosprocess/SRC/load_template.f90:35-48. */
template <class R>
void load_templates(const float* imgs, const cryoim_template* t, int T, const cryoim_params* p,
                    R* tmpl, R* tfcut) {
    int nx = p->fftsize, nr = p->max_r - p->min_r + 1;
    long nn = (long)nx * nx;
    for (int i = 0; i < T; ++i) {
        R* a = tmpl + (long)i * 2 * nn;
        R* b = a + nn;
        for (long k = 0; k < nn; ++k) a[k] = (R)imgs[(long)i * nn + k];
        if (p->use_imgmask) img2d_mask(a, nx, (R)p->imgmask_px, (R)t[i].x, (R)t[i].y);
        for (long k = 0; k < nn; ++k) {
            int ky = (int)(k / nx), hx = (int)(k % nx);
            if ((hx + ky) & 1) a[k] = -a[k];
            b[k] = R(0);
        }
        img2d_fft(a, b, nx, nx, 1);
        centshift(a, b, nx, (R)t[i].x, (R)t[i].y);
        ft_amp_expfit(a, b, nx, p->min_r, p->max_r, tfcut + (long)i * nr);
    }
}

/* Search grid of ort_globesearch.f90:19-21. */
inline void grid_sizes(float step, int* nth, int* nph, int* nom) {
    *nth = (int)(21.0f / step);
    *nph = (int)(32.0f / step);
    *nom = (int)(360.0f / step);
}

/* icosprocess/SRC/ort_globesearch.f90:34-133 for particles [0, P).  pr_array optional. */
template <class R>
int globesearch(const cryoim_params* p, const R* tmpl, const R* tfcut, const cryoim_template* t,
                int T, const float* imgs, cryoim_particle* parts, int P, float* pr_array,
                int nthreads) {
    int nx = p->fftsize, minR = p->min_r, maxR = p->max_r, nr = maxR - minR + 1;
    long nn = (long)nx * nx;
    const R step = (R)p->searchstep;
    int nth, nph, nom;
    grid_sizes(p->searchstep, &nth, &nph, &nom);
    long per = (long)nom * (2 * nph + 1) * (nth + 1);
    std::vector<R> tort(T * 3);
    for (int i = 0; i < T; ++i) { tort[i * 3] = t[i].theta; tort[i * 3 + 1] = t[i].phi; tort[i * 3 + 2] = t[i].omega; }
    std::vector<int> src = ctf_source(parts, P);
    // The view set is the reference's, decided in its single precision (ort_globesearch.f90
    // declares theta, phi, x, y, z real): at theta = 90 degrees cos() rounds below zero in
    // FP32 and the equator's views are left out, whatever precision scores the kept views.
    const Asu<float> asu32;
    const float step32 = p->searchstep, d2r32 = C<float>::deg2rad();
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int ip = 0; ip < P; ++ip) {
        cryoim_particle& q = parts[ip];
        std::vector<R> a(nn), b(nn), fcut0(nr), ctf, pra(per, R(1000)), pro(nom);
        prep_particle(imgs + (long)ip * nn, nx, 1, (R)p->imgmask_px, (R)q.x, (R)q.y, 1, minR, maxR,
                      a.data(), b.data(), fcut0.data());
        const R* ctfp = nullptr;
        if (p->apply_ctf) {
            const cryoim_particle& s = parts[src[ip]];
            ctf.resize(nn);
            get_ctf2d(nx, (R)s.df1, (R)s.df2, (R)s.astigang, (R)p->apix, (R)p->vol, (R)p->cs,
                      (R)p->ampwg, ctf.data());
            ctfp = ctf.data();
        }
        for (int it = 0; it <= nth; ++it) {
            R theta = R(69.0) + step * (R)it;
            const float t32 = (69.0f + step32 * (float)it) * d2r32;
            const float z = std::cos(t32), z0 = std::sin(t32);
            for (int iph = 0; iph <= nph; ++iph) {
                R phi = step * (R)iph;
                const float p32 = (step32 * (float)iph) * d2r32;
                const float x = z0 * std::cos(p32), y = z0 * std::sin(p32);
                if (!asu32.inside(x, y, z)) continue;
                pr_omega(a.data(), b.data(), fcut0.data(), tmpl, tort.data(), tfcut, ctfp, T, nx,
                         minR, maxR, step, nom, theta, phi, R(0), pro.data());
                std::copy(pro.begin(), pro.end(), pra.begin() + ((long)it * (2 * nph + 1) + (iph + nph)) * nom);
                pr_omega(a.data(), b.data(), fcut0.data(), tmpl, tort.data(), tfcut, ctfp, T, nx,
                         minR, maxR, step, nom, theta, -phi, R(0), pro.data());
                std::copy(pro.begin(), pro.end(), pra.begin() + ((long)it * (2 * nph + 1) + (-iph + nph)) * nom);
            }
        }
        /* minval / minloc: first minimum in column-major order (omega fastest) */
        long best = 0;
        for (long k = 1; k < per; ++k)
            if (pra[k] < pra[best]) best = k;
        int iom = (int)(best % nom), iph = (int)((best / nom) % (2 * nph + 1)), it = (int)(best / ((long)nom * (2 * nph + 1)));
        float theta = 69.0f + p->searchstep * (float)it;
        float phi = p->searchstep * (float)(iph - nph);
        float omega = p->searchstep * (float)iom;
        q.theta0 = q.theta; q.phi0 = q.phi; q.omega0 = q.omega; q.x0 = q.x; q.y0 = q.y; q.pr0 = q.pr;
        q.theta = theta; q.phi = phi; q.omega = omega; q.pr = (float)pra[best];
        q.dtheta = q.theta - q.theta0; q.dphi = q.phi - q.phi0; q.domega = q.omega - q.omega0;
        q.dx = q.x - q.x0; q.dy = q.y - q.y0; q.dpr = q.pr - q.pr0;
        if (pr_array)
            for (long k = 0; k < per; ++k) pr_array[(long)ip * per + k] = (float)pra[k];
    }
    return 0;
}

/* A bounded sample of the global search for the timed CPU baseline: one particle,
 * the listed views (theta, phi), OpenMP over views.  Same per-view arithmetic as
 * globesearch(); out: nv x Nomega. */
template <class R>
int search_views(const cryoim_params* p, const R* tmpl, const R* tfcut, const cryoim_template* t,
                 int T, const float* img, const cryoim_particle* q, const float* views, int nv,
                 int nthreads, float* out) {
    int nx = p->fftsize, minR = p->min_r, maxR = p->max_r, nr = maxR - minR + 1;
    long nn = (long)nx * nx;
    int nth, nph, nom;
    grid_sizes(p->searchstep, &nth, &nph, &nom);
    std::vector<R> tort(T * 3);
    for (int i = 0; i < T; ++i) { tort[i * 3] = t[i].theta; tort[i * 3 + 1] = t[i].phi; tort[i * 3 + 2] = t[i].omega; }
    std::vector<R> a(nn), b(nn), fcut0(nr), ctf;
    prep_particle(img, nx, 1, (R)p->imgmask_px, (R)q->x, (R)q->y, 1, minR, maxR, a.data(), b.data(),
                  fcut0.data());
    const R* ctfp = nullptr;
    if (p->apply_ctf) {
        ctf.resize(nn);
        get_ctf2d(nx, (R)q->df1, (R)q->df2, (R)q->astigang, (R)p->apix, (R)p->vol, (R)p->cs,
                  (R)p->ampwg, ctf.data());
        ctfp = ctf.data();
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int v = 0; v < nv; ++v) {
        std::vector<R> pro(nom);
        pr_omega(a.data(), b.data(), fcut0.data(), tmpl, tort.data(), tfcut, ctfp, T, nx, minR, maxR,
                 (R)p->searchstep, nom, (R)views[2 * v], (R)views[2 * v + 1], R(0), pro.data());
        for (int k = 0; k < nom; ++k) out[(long)v * nom + k] = (float)pro[k];
    }
    return 0;
}

/* icosprocess/SRC/ort_cent_11.f90:1-94 (folds theta0..omega0 in place, as the
 * by-reference Fortran call does). oc: 11 x 5. */
template <class R> void ort_cent_11(R* th0, R* ph0, R* om0, R x0, R y0, R dang, R dtran, R* oc) {
    asu_fold(th0, ph0, om0);
    for (int jj = 0; jj <= 10; ++jj) {
        R th = *th0, ph = *ph0, om = *om0, x = x0, y = y0;
        switch (jj) {
            case 1: th = *th0 - dang; break;
            case 2: th = *th0 + dang; break;
            case 3: ph = *ph0 - dang; break;
            case 4: ph = *ph0 + dang; break;
            case 5: om = *om0 - dang; break;
            case 6: om = *om0 + dang; break;
            case 7: x = x0 - dtran; break;
            case 8: x = x0 + dtran; break;
            case 9: y = y0 - dtran; break;
            case 10: y = y0 + dtran; break;
            default: break;
        }
        asu_fold(&th, &ph, &om);
        R* o = oc + jj * 5;
        o[0] = th; o[1] = ph; o[2] = om; o[3] = x; o[4] = y;
    }
}

/* icosprocess/SRC/ort_refinement.f90:31-124 for particles [0, P). */
template <class R>
int refine(const cryoim_params* p, const R* tmpl, const R* tfcut, const cryoim_template* t, int T,
           const float* imgs, cryoim_particle* parts, int P, int nthreads) {
    int nx = p->fftsize, minR = p->min_r, maxR = p->max_r, nr = maxR - minR + 1;
    long nn = (long)nx * nx;
    std::vector<R> tort(T * 3);
    for (int i = 0; i < T; ++i) { tort[i * 3] = t[i].theta; tort[i * 3 + 1] = t[i].phi; tort[i * 3 + 2] = t[i].omega; }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int ip = 0; ip < P; ++ip) {
        cryoim_particle& q = parts[ip];
        std::vector<R> a(nn), b(nn), fcut0(nr), ctf;
        prep_particle(imgs + (long)ip * nn, nx, p->use_imgmask, (R)p->imgmask_px, (R)q.x, (R)q.y, 0,
                      minR, maxR, a.data(), b.data(), fcut0.data());
        const R* ctfp = nullptr;
        if (p->apply_ctf) {
            ctf.resize(nn);
            get_ctf2d(nx, (R)q.df1, (R)q.df2, (R)q.astigang, (R)p->apix, (R)p->vol, (R)p->cs,
                      (R)p->ampwg, ctf.data());
            ctfp = ctf.data();
        }
        R th0 = q.theta, ph0 = q.phi, om0 = q.omega, x0 = q.x, y0 = q.y, pr0 = 0;
        R fac = R(1);
        for (int cyc = 1; cyc <= p->ncycle; ++cyc) {
            R dang = (R)p->delta_angle * fac, dtran = (R)p->delta_trans * fac;
            fac = fac * R(0.8);
            R oc[55], prv[11];
            ort_cent_11(&th0, &ph0, &om0, x0, y0, dang, dtran, oc);
            for (int jj = 0; jj <= 10; ++jj)
                prv[jj] = pr_single(a.data(), b.data(), fcut0.data(), tmpl, tort.data(), tfcut, ctfp,
                                    T, nx, minR, maxR, oc[jj * 5], oc[jj * 5 + 1], oc[jj * 5 + 2],
                                    oc[jj * 5 + 3], oc[jj * 5 + 4]);
            int mn = 0;
            for (int jj = 1; jj <= 10; ++jj)
                if (prv[jj] < prv[mn]) mn = jj;
            pr0 = prv[mn];
            th0 = oc[mn * 5]; ph0 = oc[mn * 5 + 1]; om0 = oc[mn * 5 + 2]; x0 = oc[mn * 5 + 3]; y0 = oc[mn * 5 + 4];
        }
        q.theta0 = q.theta; q.phi0 = q.phi; q.omega0 = q.omega; q.x0 = q.x; q.y0 = q.y; q.pr0 = q.pr;
        q.theta = (float)th0; q.phi = (float)ph0; q.omega = (float)om0; q.x = (float)x0; q.y = (float)y0;
        q.pr = (float)pr0;
        q.dtheta = q.theta - q.theta0; q.dphi = q.phi - q.phi0; q.domega = q.omega - q.omega0;
        q.dx = q.x - q.x0; q.dy = q.y - q.y0; q.dpr = q.pr - q.pr0;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* projections and central sections                                           */
/* ------------------------------------------------------------------------ */

/* icosprocess/SRC/project_template2d.f90:25-76 for one orientation. */
template <class R> void project_template2d(const float* map, int nx, R th, R ph, R om, R* slice) {
    R rot[9];
    euler_mat(th, ph, om, rot);
    long nn = (long)nx * nx;
    std::fill(slice, slice + nn, R(0));
    int h = nx / 2;
    for (long i3 = 0; i3 < nn * nx; ++i3) {
        int iz = (int)(i3 / nn), iy = (int)((i3 % nn) / nx), ix = (int)((i3 % nn) % nx);
        long i2 = (long)iy * nx + ix;
        R xp[3] = {(R)ix - (R)h, (R)iy - (R)h, (R)iz - (R)h};
        if (std::sqrt(xp[0] * xp[0] + xp[1] * xp[1] + xp[2] * xp[2]) >= (R)(h - 1)) continue;
        R x[3];
        mv3(rot, xp, x);
        x[0] = x[0] + (R)h; x[1] = x[1] + (R)h; x[2] = x[2] + (R)h;
        int jx = fint(x[0]), jy = fint(x[1]), jz = fint(x[2]);
        R xb = x[0] - (R)jx, yb = x[1] - (R)jy, zb = x[2] - (R)jz;
        long n1 = (long)jz * nn + (long)jy * nx + jx;
        const float* m = map;
        /* slice(i2) = slice(i2) + t1 + ... + t8, evaluated left to right */
        R s = slice[i2];
        s = s + (R(1) - xb) * (R(1) - yb) * (R(1) - zb) * (R)m[n1];
        s = s + xb * (R(1) - yb) * (R(1) - zb) * (R)m[n1 + 1];
        s = s + (R(1) - xb) * yb * (R(1) - zb) * (R)m[n1 + nx];
        s = s + xb * yb * (R(1) - zb) * (R)m[n1 + nx + 1];
        s = s + (R(1) - xb) * (R(1) - yb) * zb * (R)m[n1 + nn];
        s = s + xb * (R(1) - yb) * zb * (R)m[n1 + nn + 1];
        s = s + (R(1) - xb) * yb * zb * (R)m[n1 + nn + nx];
        s = s + xb * yb * zb * (R)m[n1 + nn + nx + 1];
        slice[i2] = s;
    }
}

/* icosprocess/SRC/project2d_FT3dTo2d.f90:19-84: trilinear central section of a 3D FT. */
template <class R>
void central_section(const R* fr, const R* fi, int nx, R th, R ph, R om, R* o_re, R* o_im) {
    R rot[9];
    euler_mat(th, ph, om, rot);
    long nn = (long)nx * nx;
    int h = nx / 2;
    std::fill(o_re, o_re + nn, R(0));
    std::fill(o_im, o_im + nn, R(0));
    long n = 0;
    for (int iy = -h; iy <= h - 1; ++iy)
        for (int ix = -h; ix <= h - 1; ++ix, ++n) {
            R xp[3] = {(R)ix, (R)iy, R(0)}, xx[3];
            mv3(rot, xp, xx);
            if (std::sqrt(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]) > (R)(h - 2)) continue;
            xx[0] = xx[0] + (R)h; xx[1] = xx[1] + (R)h; xx[2] = xx[2] + (R)h;
            int hx = fint(xx[0]), ky = fint(xx[1]), lz = fint(xx[2]);
            R xb = xx[0] - (R)hx, yb = xx[1] - (R)ky, zb = xx[2] - (R)lz;
            long b0 = (long)lz * nn + (long)ky * nx + hx;
            const R* srcs[2] = {fr, fi};
            R* outs[2] = {o_re, o_im};
            for (int c = 0; c < 2; ++c) {
                const R* f = srcs[c];
                outs[c][n] = (R(1) - xb) * (R(1) - yb) * (R(1) - zb) * f[b0] +
                             xb * (R(1) - yb) * (R(1) - zb) * f[b0 + 1] +
                             (R(1) - xb) * yb * (R(1) - zb) * f[b0 + nx] +
                             xb * yb * (R(1) - zb) * f[b0 + nx + 1] +
                             (R(1) - xb) * (R(1) - yb) * zb * f[b0 + nn] +
                             xb * (R(1) - yb) * zb * f[b0 + nn + 1] +
                             (R(1) - xb) * yb * zb * f[b0 + nn + nx] +
                             xb * yb * zb * f[b0 + nn + nx + 1];
            }
        }
}

/* The central section with a Gaussian interpolation kernel instead of the trilinear
 * one (the reference interpolates trilinearly only; this restates the library's
 * alternative, cryoim_set_interpolation kind 1): the geometry of central_section, and
 * per sample the 27 voxels around the nearest one weighted exp(-d^2 / (2 sigma^2)),
 * normalised by the weights' sum. */
template <class R>
void central_section_gauss(const R* fr, const R* fi, int nx, R th, R ph, R om, R sigma, R* o_re, R* o_im) {
    R rot[9];
    euler_mat(th, ph, om, rot);
    long nn = (long)nx * nx;
    int h = nx / 2;
    std::fill(o_re, o_re + nn, R(0));
    std::fill(o_im, o_im + nn, R(0));
    const R g = R(1) / (R(2) * sigma * sigma);
    long n = 0;
    for (int iy = -h; iy <= h - 1; ++iy)
        for (int ix = -h; ix <= h - 1; ++ix, ++n) {
            R xp[3] = {(R)ix, (R)iy, R(0)}, xx[3];
            mv3(rot, xp, xx);
            if (std::sqrt(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]) > (R)(h - 2)) continue;
            int c0[3];
            R w[3][3], ws[3];
            for (int a = 0; a < 3; ++a) {
                c0[a] = (int)std::nearbyint(xx[a]);
                ws[a] = 0;
                for (int d = 0; d < 3; ++d) {
                    const R e = xx[a] - (R)(c0[a] + d - 1);
                    w[a][d] = std::exp(-g * e * e);
                    ws[a] += w[a][d];
                }
            }
            R sr = 0, si = 0;
            for (int dz = 0; dz < 3; ++dz)
                for (int dy = 0; dy < 3; ++dy)
                    for (int dx = 0; dx < 3; ++dx) {
                        const long q = (long)(c0[2] + dz - 1 + h) * nn + (long)(c0[1] + dy - 1 + h) * nx +
                                       (c0[0] + dx - 1 + h);
                        const R wt = w[0][dx] * w[1][dy] * w[2][dz];
                        sr += wt * fr[q];
                        si += wt * fi[q];
                    }
            const R inv = R(1) / (ws[0] * ws[1] * ws[2]);
            o_re[n] = sr * inv;
            o_im[n] = si * inv;
        }
}

/* ------------------------------------------------------------------------ */
/* reconstruction                                                              */
/* ------------------------------------------------------------------------ */

/* icosprocess/SRC/reconstruct.f90:53-256 (sym = icos, no real-space average).
 * map_out: nx^3.  acc_out (optional): the fa, fb, wg accumulators (3*nx^3) before
 * the Friedel fold. */
template <class R>
int reconstruct(const cryoim_params* p, const float* imgs, const cryoim_particle* parts, int P,
                float* map_out, R* acc_out) {
    int nx = p->fftsize, maxR = p->max_r, h = nx / 2;
    long nn = (long)nx * nx, n3 = nn * nx;
    std::vector<R> fa(n3, R(0)), fb(n3, R(0)), wg(n3, R(0.01));
    const R* sym = icos_ops<R>();
    /* the imgID cache (reconstruct.f90:84-90) only advances on selected particles */
    std::vector<int> src(P, -1);
    {
        int id0 = -100, cur = -1;
        for (int i = 0; i < P; ++i) {
            const cryoim_particle& q = parts[i];
            if (!(q.pr <= p->pr_threshold && std::fabs(q.x) <= p->boundx && std::fabs(q.y) <= p->boundx))
                continue;
            if (q.img_id != id0) { cur = i; id0 = q.img_id; }
            src[i] = cur;
        }
    }
    std::vector<R> a(nn), b(nn), ctf(nn, R(1));
    const R ox = (R)parts[0].x, oy = (R)parts[0].y; /* reconstruct.f90:92 passes particle%x */
    for (int ip = 0; ip < P; ++ip) {
        const cryoim_particle& q = parts[ip];
        if (!(q.pr <= p->pr_threshold && std::fabs(q.x) <= p->boundx && std::fabs(q.y) <= p->boundx))
            continue;
        for (long k = 0; k < nn; ++k) a[k] = (R)imgs[(long)ip * nn + k];
        img2d_norm(a.data(), nx);
        if (p->imgstck || p->apply_ctf) {
            const cryoim_particle& s = p->imgstck ? q : parts[src[ip]];
            get_ctf2d(nx, (R)s.df1, (R)s.df2, (R)s.astigang, (R)p->apix, (R)p->vol, (R)p->cs,
                      (R)p->ampwg, ctf.data());
        }
        if (p->use_imgmask) img2d_mask(a.data(), nx, (R)p->imgmask_px, ox, oy);
        for (long k = 0; k < nn; ++k) {
            int ky = (int)(k / nx), hx = (int)(k % nx);
            if ((hx + ky) & 1) a[k] = -a[k];
            b[k] = R(0);
        }
        img2d_fft(a.data(), b.data(), nx, nx, 1);
        centshift(a.data(), b.data(), nx, (R)q.x, (R)q.y);
        R rot[9];
        euler_mat((R)q.theta, (R)q.phi, (R)q.omega, rot);
        for (int ky = -maxR; ky <= maxR; ++ky)
            for (int hx = 0; hx <= maxR; ++hx) {
                R dr = std::sqrt((R)(hx * hx + ky * ky));
                if (!(dr <= (R)maxR)) continue;
                long i2 = (long)(ky + h) * nx + (hx + h);
                R xv[3] = {(R)hx, (R)ky, R(0)}, x00[3];
                mv3(rot, xv, x00);
                for (int is = 0; is < p->nsym; ++is) {
                    R x0[3];
                    mv3(sym + is * 9, x00, x0);
                    R signz = R(1);
                    if (x0[2] < R(0)) { x0[0] = -x0[0]; x0[1] = -x0[1]; x0[2] = -x0[2]; signz = R(-1); }
                    x0[0] = x0[0] + (R)h; x0[1] = x0[1] + (R)h; x0[2] = x0[2] + (R)h;
                    int lx[3] = {fint(x0[0]), fint(x0[1]), fint(x0[2])};
                    R ax[3] = {x0[0] - (R)lx[0], x0[1] - (R)lx[1], x0[2] - (R)lx[2]};
                    R dx[8];
                    dx[0] = (R(1) - ax[0]) * (R(1) - ax[1]) * (R(1) - ax[2]);
                    dx[1] = (ax[0]) * (R(1) - ax[1]) * (R(1) - ax[2]);
                    dx[2] = (R(1) - ax[0]) * (ax[1]) * (R(1) - ax[2]);
                    dx[3] = (ax[0]) * (ax[1]) * (R(1) - ax[2]);
                    dx[4] = (R(1) - ax[0]) * (R(1) - ax[1]) * (ax[2]);
                    dx[5] = (ax[0]) * (R(1) - ax[1]) * (ax[2]);
                    dx[6] = (R(1) - ax[0]) * (ax[1]) * (ax[2]);
                    dx[7] = (ax[0]) * (ax[1]) * (ax[2]);
                    long c1 = (long)lx[2] * nn + (long)lx[1] * nx + lx[0];
                    long cub[8] = {c1, c1 + 1, c1 + nx, c1 + nx + 1, c1 + nn, c1 + nn + 1, c1 + nn + nx, c1 + nn + nx + 1};
                    R c = ctf[i2];
                    for (int j = 0; j < 8; ++j) {
                        fa[cub[j]] = fa[cub[j]] + a[i2] * dx[j] * c;
                        fb[cub[j]] = fb[cub[j]] + b[i2] * dx[j] * c * signz;
                        wg[cub[j]] = wg[cub[j]] + dx[j] * (c * c);
                    }
                }
            }
    }
    if (acc_out) {
        std::copy(fa.begin(), fa.end(), acc_out);
        std::copy(fb.begin(), fb.end(), acc_out + n3);
        std::copy(wg.begin(), wg.end(), acc_out + 2 * n3);
    }
    /* Friedel completion and weight division: reconstruct.f90:151-237 */
    auto idx = [&](int hx, int ky, int lz) { return (long)(lz + h) * nn + (long)(ky + h) * nx + (hx + h); };
    auto fold_pair = [&](int hx, int ky, int lz, bool z0plane) {
        long n1 = idx(hx, ky, lz), n2 = idx(-hx, -ky, -lz);
        R dr = std::sqrt((R)(hx * hx + ky * ky + lz * lz));
        if (dr <= (R)maxR) {
            if (z0plane) {
                wg[n1] = wg[n1] + wg[n2];
                fa[n1] = (fa[n1] + fa[n2]) / wg[n1];
                fb[n1] = (fb[n1] - fb[n2]) / wg[n1];
            } else {
                fa[n1] = fa[n1] / wg[n1];
                fb[n1] = fb[n1] / wg[n1];
            }
            if (((hx + ky + lz) % 2 + 2) % 2 == 0) {
                fa[n2] = fa[n1]; fb[n2] = -fb[n1];
            } else {
                fa[n1] = -fa[n1]; fb[n1] = -fb[n1];
                fa[n2] = fa[n1]; fb[n2] = -fb[n1];
            }
        } else {
            fa[n1] = 0; fb[n1] = 0; fa[n2] = 0; fb[n2] = 0;
        }
    };
    for (int ky = 1; ky <= maxR; ++ky)
        for (int hx = -maxR; hx <= maxR; ++hx) fold_pair(hx, ky, 0, true);
    for (int hx = 1; hx <= maxR; ++hx) fold_pair(hx, 0, 0, true);
    {
        long n1 = idx(0, 0, 0);
        fa[n1] = fa[n1] / wg[n1];
        fb[n1] = 0;
    }
    for (int lz = 1; lz <= maxR; ++lz)
        for (int ky = -maxR; ky <= maxR; ++ky)
            for (int hx = -maxR; hx <= maxR; ++hx) fold_pair(hx, ky, lz, false);
    /* FFT3d = cmplx(fa, -fb); backward 3D FFT; shift3dComplex; real part */
    for (long k = 0; k < n3; ++k) fb[k] = -fb[k];
    fft3d(fa.data(), fb.data(), nx, +1);
    for (long k = 0; k < n3; ++k) {
        int lz = (int)(k / nn), ky = (int)((k / nx) % nx), hx = (int)(k % nx);
        R v = fa[k];
        if ((hx + ky + lz) & 1) v = -v;
        map_out[k] = (float)v;
    }
    return 0;
}

/* icosprocess/SRC/reconstruct_half.f90:4-151: particles parity, parity+2, ... of the
 * range, accumulated into the tnf half box (R+1)(2R+1)^2 (fa, fb, wg start at 0).  Masks
 * every image at parts[0]'s origin (the reference passes particle%x, whose first element
 * is particle(first) of the whole range for both halves), samples r <= maxR, x0(1:2) +=
 * maxR.  A trilinear corner past the box's row/plane end lands, as in the reference's
 * linear cubID, on the next row/plane; one past the last plane is dropped. */
template <class R>
int reconstruct_half(const cryoim_params* p, const float* imgs, const cryoim_particle* parts, int P,
                     int parity, R* fa, R* fb, R* wg) {
    int nx = p->fftsize, maxR = p->max_r, h = nx / 2, t = 2 * maxR + 1;
    long nn = (long)nx * nx, tnf = (long)(maxR + 1) * t * t;
    std::fill(fa, fa + tnf, R(0));
    std::fill(fb, fb + tnf, R(0));
    std::fill(wg, wg + tnf, R(0));
    if (P < 1) return 0;
    const R* sym = icos_ops<R>();
    std::vector<R> a(nn), b(nn), ctf(nn, R(1));
    const R ox = (R)parts[0].x, oy = (R)parts[0].y;
    int id0 = -100;
    for (int ip = parity; ip < P; ip += 2) {
        const cryoim_particle& q = parts[ip];
        if (!(q.pr <= p->pr_threshold && std::fabs(q.x) <= p->boundx && std::fabs(q.y) <= p->boundx))
            continue;
        for (long k = 0; k < nn; ++k) a[k] = (R)imgs[(long)ip * nn + k];
        img2d_norm(a.data(), nx);
        /* reconstruct_half.f90:71-81: every particle's CTF for imgstck, else cached per imgID */
        if (p->imgstck || (p->apply_ctf && q.img_id != id0)) {
            get_ctf2d(nx, (R)q.df1, (R)q.df2, (R)q.astigang, (R)p->apix, (R)p->vol, (R)p->cs,
                      (R)p->ampwg, ctf.data());
            if (!p->imgstck) id0 = q.img_id;
        }
        if (p->use_imgmask) img2d_mask(a.data(), nx, (R)p->imgmask_px, ox, oy);
        for (long k = 0; k < nn; ++k) {
            int ky = (int)(k / nx), hx = (int)(k % nx);
            if ((hx + ky) & 1) a[k] = -a[k];
            b[k] = R(0);
        }
        img2d_fft(a.data(), b.data(), nx, nx, 1);
        centshift(a.data(), b.data(), nx, (R)q.x, (R)q.y);
        R rot[9];
        euler_mat((R)q.theta, (R)q.phi, (R)q.omega, rot);
        for (int ky = -maxR; ky <= maxR; ++ky)
            for (int hx = 0; hx <= maxR; ++hx) {
                R dr = std::sqrt((R)(hx * hx + ky * ky));
                if (!(dr <= (R)maxR)) continue;
                long i2 = (long)(ky + h) * nx + (hx + h);
                R xv[3] = {(R)hx, (R)ky, R(0)}, x00[3];
                mv3(rot, xv, x00);
                for (int is = 0; is < p->nsym; ++is) {
                    R x0[3];
                    mv3(sym + is * 9, x00, x0);
                    R signz = R(1);
                    if (x0[2] < R(0)) { x0[0] = -x0[0]; x0[1] = -x0[1]; x0[2] = -x0[2]; signz = R(-1); }
                    x0[0] = x0[0] + (R)maxR; x0[1] = x0[1] + (R)maxR;
                    int lx[3] = {fint(x0[0]), fint(x0[1]), fint(x0[2])};
                    R ax[3] = {x0[0] - (R)lx[0], x0[1] - (R)lx[1], x0[2] - (R)lx[2]};
                    R dx[8];
                    dx[0] = (R(1) - ax[0]) * (R(1) - ax[1]) * (R(1) - ax[2]);
                    dx[1] = (ax[0]) * (R(1) - ax[1]) * (R(1) - ax[2]);
                    dx[2] = (R(1) - ax[0]) * (ax[1]) * (R(1) - ax[2]);
                    dx[3] = (ax[0]) * (ax[1]) * (R(1) - ax[2]);
                    dx[4] = (R(1) - ax[0]) * (R(1) - ax[1]) * (ax[2]);
                    dx[5] = (ax[0]) * (R(1) - ax[1]) * (ax[2]);
                    dx[6] = (R(1) - ax[0]) * (ax[1]) * (ax[2]);
                    dx[7] = (ax[0]) * (ax[1]) * (ax[2]);
                    long c1 = ((long)lx[2] * t + lx[1]) * t + lx[0];
                    long tt = (long)t * t;
                    long cub[8] = {c1, c1 + 1, c1 + t, c1 + t + 1, c1 + tt, c1 + tt + 1, c1 + tt + t, c1 + tt + t + 1};
                    R c = ctf[i2];
                    for (int j = 0; j < 8; ++j) {
                        if (cub[j] < 0 || cub[j] >= tnf) continue;
                        fa[cub[j]] = fa[cub[j]] + a[i2] * dx[j] * c;
                        fb[cub[j]] = fb[cub[j]] + b[i2] * dx[j] * c * signz;
                        wg[cub[j]] = wg[cub[j]] + dx[j] * (c * c);
                    }
                }
            }
    }
    return 0;
}

/* icosprocess/SRC/reconstruct_FSC.f90:25-178: FSC per integer shell of the odd (1) and
 * even (2) tnf partials, FSC weighting sqrt(2F/(1+F)) of their sum, Friedel fold to the
 * full cube, FFT3d = cmplx(fa, fb), backward 3D FFT, shift3dComplex, real part.
 * fsc_out: R+1 raw FSC values (as written to FSC.txt); map_out: nx^3. */
template <class R>
int fsc_combine(int nx, int maxR, const float* fa1, const float* fb1, const float* wg1,
                const float* fa2, const float* fb2, const float* wg2, R* fsc_out, float* map_out,
                bool merge = false, R imgmask = R(0)) {
    int t = 2 * maxR + 1, h = nx / 2;
    long tnf = (long)(maxR + 1) * t * t, nn = (long)nx * nx, n3 = nn * nx;
    std::vector<R> a1(tnf), b1(tnf), w1(tnf), a2(tnf), b2(tnf), w2(tnf);
    for (long i = 0; i < tnf; ++i) {
        w1[i] = (R)wg1[i] + R(1); w2[i] = (R)wg2[i] + R(1);
        a1[i] = (R)fa1[i] / w1[i]; b1[i] = (R)fb1[i] / w1[i];
        a2[i] = (R)fa2[i] / w2[i]; b2[i] = (R)fb2[i] / w2[i];
    }
    std::vector<R> F(maxR + 1, R(0)), F1(maxR + 1, R(1e-10)), F2(maxR + 1, R(1e-10));
    auto tidx = [&](int hx, int ky, int lz) { return ((long)lz * t + (ky + maxR)) * t + (hx + maxR); };
    auto shell = [&](int hx, int ky, int lz) { return fint(std::sqrt((float)(hx * hx + ky * ky + lz * lz))); };
    for (int lz = 0; lz <= maxR; ++lz)
        for (int ky = -maxR; ky <= maxR; ++ky)
            for (int hx = -maxR; hx <= maxR; ++hx) {
                int ir = shell(hx, ky, lz);
                if (ir > maxR) continue;
                long i3 = tidx(hx, ky, lz);
                F[ir] = F[ir] + (a1[i3] * a2[i3] + b1[i3] * b2[i3]);
                F1[ir] = F1[ir] + (a1[i3] * a1[i3] + b1[i3] * b1[i3]);
                F2[ir] = F2[ir] + (a2[i3] * a2[i3] + b2[i3] * b2[i3]);
            }
    for (int ir = 0; ir <= maxR; ++ir) {
        F[ir] = F[ir] / std::sqrt(F1[ir] * F2[ir]);
        fsc_out[ir] = F[ir];
        F[ir] = F[ir] <= R(0) ? R(0) : std::sqrt(R(2) * F[ir] / (R(1) + F[ir]));
    }
    for (long i = 0; i < tnf; ++i) {
        a1[i] = a1[i] * w1[i] + a2[i] * w2[i];
        b1[i] = b1[i] * w1[i] + b2[i] * w2[i];
        w1[i] = w1[i] + w2[i] - R(2);
    }
    for (int lz = 0; lz <= maxR; ++lz)
        for (int ky = -maxR; ky <= maxR; ++ky)
            for (int hx = -maxR; hx <= maxR; ++hx) {
                int ir = shell(hx, ky, lz);
                long i3 = tidx(hx, ky, lz);
                if (ir <= maxR) { a1[i3] = a1[i3] * F[ir]; b1[i3] = b1[i3] * F[ir]; w1[i3] = w1[i3] * F[ir]; }
                else { a1[i3] = R(0); b1[i3] = R(0); }
            }
    for (long i = 0; i < tnf; ++i) w1[i] = w1[i] + R(1);
    std::vector<R> fa(n3, R(0)), fb(n3, R(0));
    auto vidx = [&](int hx, int ky, int lz) { return (long)(lz + h) * nn + (long)(ky + h) * nx + (hx + h); };
    auto pair0 = [&](int hx, int ky) {
        if (shell(hx, ky, 0) > maxR) return;
        long ia = tidx(hx, ky, 0), ib = tidx(-hx, -ky, 0), n1 = vidx(hx, ky, 0), n2 = vidx(-hx, -ky, 0);
        w1[ia] = w1[ia] + w1[ib];
        fa[n1] = (a1[ia] + a1[ib]) / w1[ia];
        fb[n1] = (b1[ia] - b1[ib]) / w1[ia];
        if (((hx + ky) % 2 + 2) % 2 == 0) { fa[n2] = fa[n1]; fb[n2] = -fb[n1]; }
        else { fa[n1] = -fa[n1]; fb[n1] = -fb[n1]; fa[n2] = fa[n1]; fb[n2] = -fb[n1]; }
    };
    for (int ky = 1; ky <= maxR; ++ky)
        for (int hx = -maxR; hx <= maxR; ++hx) pair0(hx, ky);
    for (int hx = 1; hx <= maxR; ++hx) pair0(hx, 0);
    fa[vidx(0, 0, 0)] = a1[tidx(0, 0, 0)] / w1[tidx(0, 0, 0)];
    fb[vidx(0, 0, 0)] = R(0);
    for (int lz = 1; lz <= maxR; ++lz)
        for (int ky = -maxR; ky <= maxR; ++ky)
            for (int hx = -maxR; hx <= maxR; ++hx) {
                if (shell(hx, ky, lz) > maxR) continue;
                long i3 = tidx(hx, ky, lz), n1 = vidx(hx, ky, lz), n2 = vidx(-hx, -ky, -lz);
                R s = (((hx + ky + lz) % 2 + 2) % 2 == 0) ? R(1) : R(-1);
                fa[n1] = a1[i3] / w1[i3] * s;
                fb[n1] = b1[i3] / w1[i3] * s;
                fa[n2] = fa[n1];
                fb[n2] = -fb[n1];
            }
    if (merge) {
        /* merge_reconstruct_FSC.f90:184-198: Singleton FFT with isn = -1 (exponent sign
         * negative) along each axis, then (-1)^(x+y+z) inside radius imgmask, 0 outside */
        fft3d(fa.data(), fb.data(), nx, -1);
        for (long k = 0; k < n3; ++k) {
            int lz = (int)(k / nn), ky = (int)((k / nx) % nx), hx = (int)(k % nx);
            float r = std::sqrt((float)((hx - h) * (hx - h) + (ky - h) * (ky - h) + (lz - h) * (lz - h)));
            R v = R(0);
            if (r <= (float)imgmask) v = ((hx + ky + lz) & 1) ? -fa[k] : fa[k];
            map_out[k] = (float)v;
        }
        return 0;
    }
    /* FFT3d = cmplx(fa, fb) (reconstruct_FSC.f90:173; reconstruct.f90:241 conjugates) */
    fft3d(fa.data(), fb.data(), nx, +1);
    for (long k = 0; k < n3; ++k) {
        int lz = (int)(k / nn), ky = (int)((k / nx) % nx), hx = (int)(k % nx);
        R v = fa[k];
        if ((hx + ky + lz) & 1) v = -v;
        map_out[k] = (float)v;
    }
    return 0;
}

/* merge_icosprocess_subrec/SRC/merge_reconstruct.f90:20-140 on the summed tnf partials
 * (fa, fb, wg in the tnf layout): a (2maxR+1)^3 box with wg = 0.01, the partials in its
 * lz >= 0 half, the Friedel fold keeping int(|h|) <= maxR (the radius is an integer
 * there), cmplx(fa, -fb) in the nx^3 cube, backward FFT, shift3dComplex, real part. */
template <class R>
int merge_finish(int nx, int maxR, const float* fa0, const float* fb0, const float* wg0, float* map_out) {
    const int t = 2 * maxR + 1, h = nx / 2;
    const long tt = (long)t * t, box = tt * t, nn = (long)nx * nx, n3 = nn * nx;
    std::vector<R> fa(box, R(0)), fb(box, R(0)), wg(box, R(0.01));
    for (long i = 0; i < tt * (maxR + 1); ++i) {
        fa[tt * maxR + i] += (R)fa0[i];
        fb[tt * maxR + i] += (R)fb0[i];
        wg[tt * maxR + i] += (R)wg0[i];
    }
    auto bidx = [&](int hx, int ky, int lz) { return ((long)(lz + maxR) * t + (ky + maxR)) * t + (hx + maxR); };
    auto inside = [&](int d2) { return fint(std::sqrt((float)d2)) <= maxR; };
    auto pair0 = [&](int hx, int ky) {
        long n1 = bidx(hx, ky, 0), n2 = bidx(-hx, -ky, 0);
        if (inside(hx * hx + ky * ky)) {
            wg[n1] = wg[n1] + wg[n2];
            R s = (((hx + ky) % 2 + 2) % 2 == 0) ? R(1) : R(-1);
            fa[n1] = (fa[n1] + fa[n2]) / wg[n1] * s;
            fb[n1] = (fb[n1] - fb[n2]) / wg[n1] * s;
            fa[n2] = fa[n1];
            fb[n2] = -fb[n1];
        } else {
            fa[n1] = fb[n1] = fa[n2] = fb[n2] = R(0);
        }
    };
    for (int ky = 1; ky <= maxR; ++ky)
        for (int hx = -maxR; hx <= maxR; ++hx) pair0(hx, ky);
    for (int hx = 1; hx <= maxR; ++hx) pair0(hx, 0);
    fa[bidx(0, 0, 0)] = fa[bidx(0, 0, 0)] / wg[bidx(0, 0, 0)];
    fb[bidx(0, 0, 0)] = R(0);
    for (int lz = 1; lz <= maxR; ++lz)
        for (int ky = -maxR; ky <= maxR; ++ky)
            for (int hx = -maxR; hx <= maxR; ++hx) {
                long n1 = bidx(hx, ky, lz), n2 = bidx(-hx, -ky, -lz);
                if (inside(hx * hx + ky * ky + lz * lz)) {
                    R s = (((hx + ky + lz) % 2 + 2) % 2 == 0) ? R(1) : R(-1);
                    fa[n1] = fa[n1] * s / wg[n1];
                    fb[n1] = fb[n1] * s / wg[n1];
                    fa[n2] = fa[n1];
                    fb[n2] = -fb[n1];
                } else {
                    fa[n1] = fb[n1] = fa[n2] = fb[n2] = R(0);
                }
            }
    std::vector<R> va(n3, R(0)), vb(n3, R(0));
    for (int lz = -maxR; lz <= maxR; ++lz)
        for (int ky = -maxR; ky <= maxR; ++ky)
            for (int hx = -maxR; hx <= maxR; ++hx) {
                long n = (long)(lz + h) * nn + (long)(ky + h) * nx + (hx + h);
                va[n] = fa[bidx(hx, ky, lz)];
                vb[n] = -fb[bidx(hx, ky, lz)];
            }
    fft3d(va.data(), vb.data(), nx, +1);
    for (long k = 0; k < n3; ++k) {
        int lz = (int)(k / nn), ky = (int)((k / nx) % nx), hx = (int)(k % nx);
        R v = va[k];
        if ((hx + ky + lz) & 1) v = -v;
        map_out[k] = (float)v;
    }
    return 0;
}

/* icosprocess/SRC/img3d_icosavg.f90:45-123 (sym = icos): voxels beyond r0 become 0, the
 * others the mean over the 60 operators of the trilinear sample at S x + nx/2.  Corners
 * outside the array (r0 beyond nx/2 - 2) count as 0. */
template <class R> void icosavg(const float* in, int nx, R r0, float* out) {
    const R* sym = icos_ops<R>();
    const long nn = (long)nx * nx, n3 = nn * nx;
    const int h = nx / 2;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < n3; ++q) {
        int hx = (int)(q % nx) - h, ky = (int)((q / nx) % nx) - h, lz = (int)(q / nn) - h;
        R r = std::sqrt((R)(hx * hx + ky * ky + lz * lz));
        if (r > r0) { out[q] = 0.0f; continue; }
        R x0[3] = {(R)hx, (R)ky, (R)lz}, acc = R(0);
        for (int s = 0; s < 60; ++s) {
            R x[3];
            mv3(sym + 9 * s, x0, x);
            for (int i = 0; i < 3; ++i) x[i] = x[i] + (R)h;
            int ix = fint(x[0]), iy = fint(x[1]), iz = fint(x[2]);
            R ax = x[0] - (R)ix, ay = x[1] - (R)iy, az = x[2] - (R)iz;
            long n1 = (long)iz * nn + (long)iy * nx + ix;
            long nb[8] = {n1, n1 + 1, n1 + nx, n1 + nx + 1, n1 + nn, n1 + nn + 1, n1 + nn + nx, n1 + nn + nx + 1};
            R v[8];
            for (int j = 0; j < 8; ++j) v[j] = (nb[j] >= 0 && nb[j] < n3) ? (R)in[nb[j]] : R(0);
            acc = acc + (R(1) - ax) * (R(1) - ay) * (R(1) - az) * v[0];
            acc = acc + (ax) * (R(1) - ay) * (R(1) - az) * v[1];
            acc = acc + (R(1) - ax) * (ay) * (R(1) - az) * v[2];
            acc = acc + (ax) * (ay) * (R(1) - az) * v[3];
            acc = acc + (R(1) - ax) * (R(1) - ay) * (az) * v[4];
            acc = acc + (ax) * (R(1) - ay) * (az) * v[5];
            acc = acc + (R(1) - ax) * (ay) * (az) * v[6];
            acc = acc + (ax) * (ay) * (az) * v[7];
        }
        out[q] = (float)(acc / R(60));
    }
}

/* ------------------------------------------------------------------------ */
/* origin centring (icosprocess mode 3)                                        */
/* ------------------------------------------------------------------------ */

/* icosprocess/SRC/img2d_lowpass.f90:2-33: exp(-r^2 / (2 lp^2)) in Fourier space. */
template <class R> void img2d_lowpass(R* a, int nx, int lp) {
    const long nn = (long)nx * nx;
    std::vector<R> b(nn, R(0));
    const R lowpass = R(2) * (R)(lp * lp);
    for (long i = 0; i < nn; ++i)
        if (((i / nx) + (i % nx)) & 1) a[i] = -a[i];
    img2d_fft(a, b.data(), nx, nx, 1);
    for (long i = 0; i < nn; ++i) {
        int ky = (int)(i / nx), hx = (int)(i % nx);
        R r2 = (R)((hx - nx / 2) * (hx - nx / 2) + (ky - nx / 2) * (ky - nx / 2));
        R huv = std::exp(-r2 / lowpass);
        a[i] = a[i] * huv / (R)(float)nn;
        b[i] = b[i] * huv / (R)(float)nn;
    }
    img2d_fft(a, b.data(), nx, nx, -1);
    for (long i = 0; i < nn; ++i)
        if (((i / nx) + (i % nx)) & 1) a[i] = -a[i];
}

/* icosprocess/SRC/img2d_applyCTF.f90:2-28. */
template <class R> void img2d_apply_ctf(R* a, int nx, const R* ctf) {
    const long nn = (long)nx * nx;
    std::vector<R> b(nn, R(0));
    for (long i = 0; i < nn; ++i)
        if (((i / nx) + (i % nx)) & 1) a[i] = -a[i];
    img2d_fft(a, b.data(), nx, nx, 1);
    for (long i = 0; i < nn; ++i) { a[i] = a[i] * ctf[i]; b[i] = b[i] * ctf[i]; }
    img2d_fft(a, b.data(), nx, nx, -1);
    for (long i = 0; i < nn; ++i)
        if (((i / nx) + (i % nx)) & 1) a[i] = -a[i];
}

/* icosprocess/SRC/cross_correlation.f90:1-26: a1 <- the centred cross-correlation map. */
template <class R> void cross_correlation(R* a1, R* a2, int nx) {
    const long nn = (long)nx * nx;
    std::vector<R> b1(nn, R(0)), b2(nn, R(0));
    img2d_fft(a1, b1.data(), nx, nx, 1);
    img2d_fft(a2, b2.data(), nx, nx, 1);
    for (long i = 0; i < nn; ++i) {
        R x = a1[i] * a2[i] + b1[i] * b2[i];
        R y = b1[i] * a2[i] - a1[i] * b2[i];
        if (((i / nx) + (i % nx)) & 1) { x = -x; y = -y; }
        a1[i] = x; b1[i] = y;
    }
    img2d_fft(a1, b1.data(), nx, nx, -1);
}

/* icosprocess/SRC/guass_regression.f90:1-56; z[j+1][i+1] = z(i, j). */
template <class R> void gauss_regression(const R z[3][3], R* dx, R* dy, R* cc) {
    R c10 = 0, c01 = 0, c11 = 0, c20 = 0, c02 = 0, c00 = 0;
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c10 = c10 + (R)i * std::log(z[j + 1][i + 1]);
    c10 = c10 / R(6);
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c01 = c01 + (R)j * std::log(z[j + 1][i + 1]);
    c01 = c01 / R(6);
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c11 = c11 + (R)(i * j) * std::log(z[j + 1][i + 1]);
    c11 = c11 / R(4);
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c20 = c20 + (R)(3 * i * i - 2) * std::log(z[j + 1][i + 1]);
    c20 = c20 / R(6);
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c02 = c02 + (R)(3 * j * j - 2) * std::log(z[j + 1][i + 1]);
    c02 = c02 / R(6);
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c00 = c00 + (R)(5 - 3 * i * i - 3 * j * j) * std::log(z[j + 1][i + 1]);
    c00 = c00 / R(9);
    R den = R(4) * c20 * c02 - c11 * c11;
    *dx = (c11 * c01 - R(2) * c10 * c02) / den;
    *dy = (c11 * c10 - R(2) * c01 * c20) / den;
    *cc = std::exp(c00 - c20 * (*dx * *dx) - c11 * *dx * *dy - c02 * (*dy * *dy));
}

/* icosprocess/SRC/img3d_mask.f90:3-56 at the box centre. */
template <class R> void img3d_mask(R* d, int nx, R mask) {
    const R pi = C<R>::pi();
    R R1 = mask - R(3);
    if (R1 <= R(0)) R1 = R(0);
    R R2 = mask + R(3);
    if (R2 > (R)(nx / 2)) R2 = (R)(nx / 2);
    const R c = (R)(nx / 2);
    const long n3 = (long)nx * nx * nx;
    auto radius = [&](long q) {
        int iz = (int)(q / ((long)nx * nx)), iy = (int)((q / nx) % nx), ix = (int)(q % nx);
        R yy = (-c + (R)iy) * (-c + (R)iy), xx = (-c + (R)ix) * (-c + (R)ix), zz = (-c + (R)iz) * (-c + (R)iz);
        return std::sqrt(xx + yy + zz);
    };
    double summ = 0;
    long num = 0;
    for (long q = 0; q < n3; ++q) {
        R ra = radius(q);
        if (ra > R1 && ra <= R2) { summ = summ + (double)d[q]; ++num; }
    }
    if (num != 0) summ = summ / (double)(float)num;
    for (long q = 0; q < n3; ++q) {
        R ra = radius(q);
        if (ra > R1 && ra <= R2) {
            R edge = (R(1) + std::cos(pi * (ra - R1) / R(6))) / R(2);
            d[q] = (R)((double)(d[q] * edge) + (double)(R(1) - edge) * summ);
        }
        if (ra > R2) d[q] = (R)summ;
    }
}

/* The peak of calc_center.f90:71-86 (first maximum; 3 x 3 neighbourhood with its linear
 * index clamped to the image, where the reference reads past it), then the Gaussian fit;
 * half = 1 halves the offset (calc_center_selfrot180.f90:72-73). */
template <class R> void cc_peak(const R* a1, int nx, int half, R* cx, R* cy, R* cc) {
    const long nn = (long)nx * nx;
    long n0 = 0;
    for (long i = 1; i < nn; ++i)
        if (a1[i] > a1[n0]) n0 = i;
    int iy0 = (int)(n0 / nx), ix0 = (int)(n0 % nx);
    R z[3][3];
    for (int ky = -1; ky <= 1; ++ky)
        for (int hx = -1; hx <= 1; ++hx) {
            long j = (long)(iy0 + ky) * nx + (ix0 + hx);
            j = j < 0 ? 0 : (j >= nn ? nn - 1 : j);
            z[ky + 1][hx + 1] = a1[j];
        }
    R dx, dy;
    gauss_regression(z, &dx, &dy, cc);
    *cx = (R)(ix0 - nx / 2) + dx;
    *cy = (R)(iy0 - nx / 2) + dy;
    if (half) { *cx = *cx / R(2); *cy = *cy / R(2); }
    if (std::fabs(*cx) >= (R)nx / R(16)) *cx = R(0);
    if (std::fabs(*cy) >= (R)nx / R(16)) *cy = R(0);
}

/* icosprocess/SRC/calc_center.f90:22-105 (map given) or calc_center_selfrot180.f90:22-86
 * (map NULL); out: (centx, centy, cc) per particle before the record update. */
template <class R>
int center(const cryoim_params* p, const float* map, const float* imgs, const cryoim_particle* parts, int P,
           R* out) {
    const int nx = p->fftsize, maxR = p->max_r;
    const long nn = (long)nx * nx, n3 = nn * nx;
    std::vector<R> fr, fi;
    if (map) {
        std::vector<R> re(map, map + n3), im(n3, R(0));
        if (p->use_imgmask) img3d_mask(re.data(), nx, (R)p->imgmask_px);
        for (long q = 0; q < n3; ++q)
            if (((q / nn) + (q / nx) % nx + q % nx) & 1) re[q] = -re[q];
        fft3d(re.data(), im.data(), nx, -1);
        const R s = (R)(float)n3;
        fr.resize(n3); fi.resize(n3);
        for (long q = 0; q < n3; ++q) {
            R a = re[q] / s, b = im[q] / s;
            if (((q / nn) + (q / nx) % nx + q % nx) & 1) { a = -a; b = -b; }
            fr[q] = a; fi[q] = -b;
        }
    }
    std::vector<R> a1(nn), a2(nn), si(nn), ctf(nn, R(1));
    int id0 = -100;
    for (int ip = 0; ip < P; ++ip) {
        const cryoim_particle& q = parts[ip];
        for (long i = 0; i < nn; ++i) a1[i] = (R)imgs[(long)ip * nn + i];
        if (map) {
            if (p->use_imgmask) img2d_mask(a1.data(), nx, (R)p->imgmask_px, (R)q.x, (R)q.y);
            img2d_lowpass(a1.data(), nx, maxR);
            central_section(fr.data(), fi.data(), nx, (R)q.theta, (R)q.phi, (R)q.omega, a2.data(), si.data());
            for (long i = 0; i < nn; ++i)
                if (((i / nx) + (i % nx)) & 1) { a2[i] = -a2[i]; si[i] = -si[i]; }
            img2d_fft(a2.data(), si.data(), nx, nx, -1);
            for (long i = 0; i < nn; ++i)
                if (((i / nx) + (i % nx)) & 1) a2[i] = -a2[i];
            if (p->apply_ctf) {
                if (q.img_id != id0) {
                    get_ctf2d(nx, (R)q.df1, (R)q.df2, (R)q.astigang, (R)p->apix, (R)p->vol, (R)p->cs, (R)p->ampwg,
                              ctf.data());
                    id0 = q.img_id;
                }
                img2d_apply_ctf(a2.data(), nx, ctf.data());
            }
            if (p->use_imgmask) img2d_mask(a2.data(), nx, (R)p->imgmask_px, R(0), R(0));
            img2d_lowpass(a2.data(), nx, maxR);
            img2d_norm(a1.data(), nx);
            img2d_norm(a2.data(), nx);
        } else {
            img2d_lowpass(a1.data(), nx, maxR);
            if (p->use_imgmask) img2d_mask(a1.data(), nx, (R)p->imgmask_px, R(0), R(0));
            img2d_norm(a1.data(), nx);
            std::fill(a2.begin(), a2.end(), R(0));
            for (long i = 0; i < nn; ++i) {
                int ky = (int)(i / nx), hx = (int)(i % nx);
                if (hx == 0 || ky == 0) a1[i] = R(0);
                else a2[(long)(nx - ky) * nx + (nx - hx)] = a1[i];
            }
        }
        cross_correlation(a1.data(), a2.data(), nx);
        cc_peak(a1.data(), nx, map ? 0 : 1, &out[3 * ip], &out[3 * ip + 1], &out[3 * ip + 2]);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* local_box (coordinate mode) and local_refine (refine_PR)                   */
/* ------------------------------------------------------------------------ */

/* local_box/SRC/Eularmatrix.f90 (row-major). */
template <class R> void eularmatrix(R th0, R ph0, R om0, R* r) {
    const R d2r = R(4) * std::atan2(R(1), R(1)) / R(180);
    R th = th0 * d2r, ph = ph0 * d2r, om = om0 * d2r;
    r[0] = std::cos(ph) * std::cos(th) * std::cos(om) - std::sin(ph) * std::sin(om);
    r[1] = -std::cos(ph) * std::cos(th) * std::sin(om) - std::sin(ph) * std::cos(om);
    r[2] = std::cos(ph) * std::sin(th);
    r[3] = std::sin(ph) * std::cos(th) * std::cos(om) + std::cos(ph) * std::sin(om);
    r[4] = -std::sin(ph) * std::cos(th) * std::sin(om) + std::cos(ph) * std::cos(om);
    r[5] = std::sin(ph) * std::sin(th);
    r[6] = -std::sin(th) * std::cos(om);
    r[7] = std::sin(th) * std::sin(om);
    r[8] = std::cos(th);
}

/* C_matrix.f90 / icos2f_sym_matc.f90: rotations by 2 pi k / n about z, k = 1..n. */
template <class R> void c_matrix(int n, R* out) {
    const R pi = R(4) * std::atan2(R(1), R(1));
    const R phi = R(2) * pi / (R)n;
    R r1[9] = {std::cos(phi), -std::sin(phi), 0, std::sin(phi), std::cos(phi), 0, 0, 0, 1};
    std::copy(r1, r1 + 9, out);
    for (int k = 1; k < n; ++k) {
        R t[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                t[3 * i + j] = out[9 * (k - 1) + 3 * i] * r1[j] + out[9 * (k - 1) + 3 * i + 1] * r1[3 + j] +
                               out[9 * (k - 1) + 3 * i + 2] * r1[6 + j];
        std::copy(t, t + 9, out + 9 * k);
    }
}

/* local_box/SRC/loc_box_coordinate.f90:13-40 with equalort.f90 and load_ort.f90's
 * selection; sym: nsym row-major rotations. */
template <class R>
int local_box_coordinates(const cryoim_particle* parts, int P, const float* sym, int nsym, R lx, R ly, R lz,
                          R apix, int fftsize, R prthr, R boundx, cryoim_local_particle* out) {
    const R r2d = R(45) / std::atan2(R(1), R(1));
    const R h = (R)(fftsize / 2);
    const R x0[3] = {lx, ly, lz};
    int k = 0;
    for (int i = 0; i < P; ++i) {
        const cryoim_particle& q = parts[i];
        if (!((R)q.pr <= prthr && std::fabs((R)q.x) <= boundx && std::fabs((R)q.y) <= boundx)) continue;
        R e[9];
        eularmatrix((R)q.theta, (R)q.phi, (R)q.omega, e);
        for (int s = 0; s < nsym; ++s) {
            R r[9];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    r[3 * a + b] = (R)sym[9 * s + 3 * a] * e[b] + (R)sym[9 * s + 3 * a + 1] * e[3 + b] +
                                   (R)sym[9 * s + 3 * a + 2] * e[6 + b];
            R th = r[8] >= R(1) ? R(0) : (r[8] < R(-1) ? R(180) : std::acos(r[8]) * r2d);
            R ph = std::atan2(r[5], r[2]) * r2d, om = std::atan2(r[7], -r[6]) * r2d;
            R rot[9];
            eularmatrix(th, ph, om, rot);
            R c[3];
            for (int a = 0; a < 3; ++a) c[a] = rot[a] * x0[0] + rot[3 + a] * x0[1] + rot[6 + a] * x0[2] + h;
            c[0] = c[0] + (R)q.x;
            c[1] = c[1] + (R)q.y;
            int hx0 = fint(c[0]), ky0 = fint(c[1]);
            cryoim_local_particle& o = out[k++];
            std::memset(&o, 0, sizeof(o));
            o.particle_id = q.particle_id; o.img_id = q.img_id; o.img_particle_id = q.img_particle_id;
            o.theta = q.theta; o.phi = q.phi; o.omega = q.omega; o.x = q.x; o.y = q.y; o.pr = q.pr;
            o.df1 = (float)((R)q.df1 * R(10000)); o.df2 = (float)((R)q.df2 * R(10000)); o.astigang = q.astigang;
            o.local_img_id = s + 1; o.local_hx0 = hx0; o.local_ky0 = ky0;
            o.local_theta0 = (float)th; o.local_phi0 = (float)ph; o.local_omega0 = (float)om;
            o.local_x0 = (float)(c[0] - (R)hx0); o.local_y0 = (float)(c[1] - (R)ky0);
            o.local_z0 = (float)((c[2] - h) * apix);
            o.local_pr0 = q.pr;
        }
    }
    return k;
}

/* local_box/SRC/loc_box.f90:34-91, the sub-image stack mode: for every selected particle
 * (load_ort.f90:30-34) the whole image is shifted to centre (img2d_centshift.f90 of
 * local_box: checkerboard, forward transform /N^2, the phase ramp of (-x, -y), inverse
 * transform, checkerboard) and normalised (img2d_norm.f90); for each of the nsym
 * equivalent orientations (equalort.f90) the sub-image centre R^T (lx, ly, lz) is split
 * into an integer pixel and a fraction, the sub_FFTsize box around it is cut with
 * periodic wrap (:60-79) and normalised.  imgs: P whole images of nx0^2 in record order;
 * out: nsym records per selected particle, sub_out: their sub images (sub^2 each).
 * Record fields as loc_box.f90:86-88 writes them: local_theta0..omega0 the equivalent
 * orientation, local_x0/y0 the fractions, local_z0 = z * apix, local_img_id the rotation
 * index, local_hx0/ky0 the box's first pixel (hx0 + nx0/2 - sub/2), particle_id the
 * running sub-particle count (format 900's Nparticle), df1/df2/astigang as read (um). */
template <class R>
int local_box_extract(const float* imgs, const cryoim_particle* parts, int P, int nx0, const float* sym, int nsym,
                      R lx, R ly, R lz, R apix, int sub, R prthr, R boundx, float* sub_out,
                      cryoim_local_particle* out) {
    const R r2d = R(45) / std::atan2(R(1), R(1));
    const R pi = R(4) * std::atan2(R(1), R(1));
    const R x0[3] = {lx, ly, lz};
    const long nn0 = (long)nx0 * nx0, ns = (long)sub * sub;
    std::vector<R> a(nn0), b(nn0), cut(ns);
    int k = 0;
    for (int i = 0; i < P; ++i) {
        const cryoim_particle& q = parts[i];
        if (!((R)q.pr <= prthr && std::fabs((R)q.x) <= boundx && std::fabs((R)q.y) <= boundx)) continue;
        const float* im = imgs + (long)i * nn0;
        for (long t = 0; t < nn0; ++t) {
            const int ky = (int)(t / nx0), hx = (int)(t % nx0);
            a[t] = (R)im[t] * (((hx + ky) & 1) ? R(-1) : R(1));
            b[t] = 0;
        }
        img2d_fft<R>(a.data(), b.data(), nx0, nx0, 1);
        const R xs = -(R)q.x, ys = -(R)q.y;
        for (long t = 0; t < nn0; ++t) {
            b[t] = -b[t];
            const int ky = (int)(t / nx0) - nx0 / 2, hx = (int)(t % nx0) - nx0 / 2;
            const R ph = R(2) * pi * (xs * (R)hx + ys * (R)ky) / (R)(float)nx0;
            const R c = std::cos(ph), sn = std::sin(ph);
            const R fr = a[t] * c + b[t] * sn, fi = -a[t] * sn + b[t] * c;
            a[t] = fr;
            b[t] = fi;
        }
        img2d_fft<R>(a.data(), b.data(), nx0, nx0, -1);
        for (long t = 0; t < nn0; ++t) {
            const int ky = (int)(t / nx0), hx = (int)(t % nx0);
            if ((hx + ky) & 1) a[t] = -a[t];
        }
        img2d_norm<R>(a.data(), nx0);
        R e[9];
        eularmatrix((R)q.theta, (R)q.phi, (R)q.omega, e);
        for (int s = 0; s < nsym; ++s) {
            R r[9];
            for (int u = 0; u < 3; ++u)
                for (int v = 0; v < 3; ++v)
                    r[3 * u + v] = (R)sym[9 * s + 3 * u] * e[v] + (R)sym[9 * s + 3 * u + 1] * e[3 + v] +
                                   (R)sym[9 * s + 3 * u + 2] * e[6 + v];
            R th = r[8] >= R(1) ? R(0) : (r[8] < R(-1) ? R(180) : std::acos(r[8]) * r2d);
            R ph = std::atan2(r[5], r[2]) * r2d, om = std::atan2(r[7], -r[6]) * r2d;
            R rot[9];
            eularmatrix(th, ph, om, rot);
            R c[3];
            for (int u = 0; u < 3; ++u) c[u] = rot[u] * x0[0] + rot[3 + u] * x0[1] + rot[6 + u] * x0[2];
            int hx0 = fint(c[0]);
            const R fx = c[0] - (R)hx0;
            int ky0 = fint(c[1]);
            const R fy = c[1] - (R)ky0;
            hx0 = hx0 + nx0 / 2 - sub / 2;
            ky0 = ky0 + nx0 / 2 - sub / 2;
            for (long t = 0; t < ns; ++t) {
                int ky = (int)(t / sub) + ky0, hx = (int)(t % sub) + hx0;
                if (hx < 0) hx += nx0;
                if (hx >= nx0) hx -= nx0;
                if (ky < 0) ky += nx0;
                if (ky >= nx0) ky -= nx0;
                cut[t] = a[(long)ky * nx0 + hx];
            }
            img2d_norm<R>(cut.data(), sub);
            for (long t = 0; t < ns; ++t) sub_out[(long)k * ns + t] = (float)cut[t];
            cryoim_local_particle& o = out[k];
            std::memset(&o, 0, sizeof(o));
            o.particle_id = k + 1;
            o.img_id = q.img_id; o.img_particle_id = q.img_particle_id;
            o.theta = q.theta; o.phi = q.phi; o.omega = q.omega; o.x = q.x; o.y = q.y; o.pr = q.pr;
            o.df1 = q.df1; o.df2 = q.df2; o.astigang = q.astigang;
            o.local_img_id = s + 1; o.local_hx0 = hx0; o.local_ky0 = ky0;
            o.local_theta0 = (float)th; o.local_phi0 = (float)ph; o.local_omega0 = (float)om;
            o.local_x0 = (float)fx; o.local_y0 = (float)fy;
            o.local_z0 = (float)(c[2] * apix);
            o.local_pr0 = q.pr;
            ++k;
        }
    }
    return k;
}

/* local_refine/SRC/getCTF2d.f90 (defocus already in Angstrom). */
template <class R> void local_ctf2d(int nx, R df1, R df2, R astig0, R apix, R vol, R cs0, R ampwg, R* ctf) {
    get_ctf2d(nx, df1 / R(1.0e4), df2 / R(1.0e4), astig0, apix, vol, cs0, ampwg, ctf);
}

/* refine_PR.f90:128-143 for one candidate: FFT3d_slice, img2d_FTphase, shift x CTF x
 * weight, cal_PR_FT against the sub-particle's weighted transform (a2, b2). */
template <class R>
R local_score(const R* fr, const R* fi, int nx, const R* cand, const R* a2, const R* b2, const R* ctf, const R* w,
              R maxR) {
    const long nn = (long)nx * nx;
    std::vector<R> sa(nn), sb(nn);
    central_section(fr, fi, nx, cand[0], cand[1], cand[2], sa.data(), sb.data());
    const R pi = R(4) * std::atan2(R(1), R(1)), tpi = R(2) * pi;
    R pr1 = 0, pr2 = 0;
    for (long i = 0; i < nn; ++i) {
        int ky = (int)(i / nx) - nx / 2, hx = (int)(i % nx) - nx / 2;
        R ph = R(2) * pi * (cand[3] * (R)hx + cand[4] * (R)ky) / (R)nx;
        R a1 = sa[i] * std::cos(ph) + sb[i] * std::sin(ph);
        R b1 = -sa[i] * std::sin(ph) + sb[i] * std::cos(ph);
        R s = (((i / nx) + (i % nx)) & 1) ? R(-1) : R(1);
        a1 = a1 * s * ctf[i] * w[i];
        b1 = b1 * s * ctf[i] * w[i];
        R dr = std::sqrt((R)(hx * hx + ky * ky));
        if (!(dr >= R(-1) && dr <= maxR)) continue;
        R amp1 = std::sqrt(a1 * a1 + b1 * b1), amp2 = std::sqrt(a2[i] * a2[i] + b2[i] * b2[i]);
        R diff = std::fabs(std::atan2(b2[i], a2[i]) - std::atan2(b1, a1));
        diff = std::fmod(diff, tpi);
        if (diff > pi) diff = tpi - diff;
        amp1 = amp1 + amp2;
        pr1 = diff * amp1 + pr1;
        pr2 = amp1 + pr2;
    }
    return pr2 > R(1.0e-10) ? pr1 / pr2 * R(180) / pi : R(1000);
}

/* local_refine/SRC/refine_PR.f90:24-232 (sym cN: nsym = N; the refine_PR path). */
template <class R>
int local_refine(const cryoim_local_params* p, const float* map, const float* imgs, cryoim_local_particle* parts,
                 int P) {
    const int nx = p->fftsize, nx0 = p->fftsize0, nsym = p->nsym;
    const long nn = (long)nx * nx, nn0 = (long)nx0 * nx0, n3 = nn * nx;
    const R pi = R(4) * std::atan2(R(1), R(1));
    /* img3d_softmask.f90 */
    std::vector<R> re(map, map + n3), im(n3, R(0));
    {
        R inn = (R)p->imgmask_px - R(3);
        if (inn <= R(0)) inn = R(0);
        R out = (R)p->imgmask_px + R(3);
        if (out > (R)(nx / 2)) out = (R)(nx / 2);
        auto rad = [&](long q) {
            int iz = (int)(q / nn) - nx / 2, iy = (int)((q / nx) % nx) - nx / 2, ix = (int)(q % nx) - nx / 2;
            return std::sqrt((R)(ix * ix + iy * iy + iz * iz));
        };
        R summ = 0;
        long num = 0;
        for (long q = 0; q < n3; ++q) {
            R r = rad(q);
            if (r > inn && r <= out) { summ = re[q] + summ; ++num; }
        }
        if (num != 0) summ = summ / (R)(float)num;
        for (long q = 0; q < n3; ++q) {
            R r = rad(q);
            if (r > inn && r <= out) {
                R edge = (R(1) + std::cos(pi * (r - inn) / R(6))) / R(2);
                re[q] = re[q] * edge + (R(1) - edge) * summ;
            }
            if (r > out) re[q] = summ;
        }
    }
    /* refine_PR.f90:48-52 */
    for (long q = 0; q < n3; ++q)
        if (((q / nn) + (q / nx) % nx + q % nx) & 1) re[q] = -re[q];
    fft3d(re.data(), im.data(), nx, -1);
    const R s3 = (R)(float)n3;
    for (long q = 0; q < n3; ++q) {
        re[q] = re[q] / s3; im[q] = im[q] / s3;
        if (((q / nn) + (q / nx) % nx + q % nx) & 1) { re[q] = -re[q]; im[q] = -im[q]; }
    }
    const R maxR = (R)p->max_r;
    std::vector<R> w(nn);
    for (long i = 0; i < nn; ++i) {
        int ky = (int)(i / nx), hx = (int)(i % nx);
        R r2 = (R)((hx - nx / 2) * (hx - nx / 2) + (ky - nx / 2) * (ky - nx / 2)) / R(2) / (maxR * maxR);
        w[i] = std::exp(-r2);
    }
    std::vector<R> symr(9 * (size_t)nsym);
    c_matrix<R>(nsym, symr.data());
    std::vector<R> img(nn0), a2(nn), b2(nn), ctf(nn, R(1));
    for (int ip = 0; ip < P; ++ip) {
        cryoim_local_particle& q = parts[ip];
        for (long i = 0; i < nn0; ++i) img[i] = (R)imgs[(long)ip * nn0 + i];
        if (p->normalize) img2d_norm(img.data(), nx0);
        /* img2d_local_box.f90 */
        for (long i = 0; i < nn; ++i) {
            int hx = (int)(i % nx) + q.local_hx0 - nx / 2, ky = (int)(i / nx) + q.local_ky0 - nx / 2;
            if (hx < 0) hx += nx0;
            if (hx >= nx0) hx -= nx0;
            if (ky < 0) ky += nx0;
            if (ky >= nx0) ky -= nx0;
            long i2 = (long)ky * nx0 + hx;
            a2[i] = (i2 >= 0 && i2 < nn0) ? img[i2] : R(0);
        }
        img2d_mask(a2.data(), nx, (R)p->imgmask_px, (R)q.local_x0, (R)q.local_y0);
        for (long i = 0; i < nn; ++i) {
            if (((i / nx) + (i % nx)) & 1) a2[i] = -a2[i];
            b2[i] = R(0);
        }
        img2d_fft(a2.data(), b2.data(), nx, nx, 1);
        for (long i = 0; i < nn; ++i) { a2[i] = a2[i] * w[i]; b2[i] = b2[i] * w[i]; }
        if (p->apply_ctf)
            local_ctf2d(nx, (R)q.df1, (R)q.df2, (R)q.astigang, (R)p->apix, (R)p->vol, (R)p->cs, (R)p->ampwg,
                        ctf.data());
        R st[5] = {(R)q.local_theta0, (R)q.local_phi0, (R)q.local_omega0, (R)q.local_x0, (R)q.local_y0};
        R best = 0;
        if (nsym > 1) {
            /* icos_equalort.f90 */
            const R r2d = R(45) / std::atan2(R(1), R(1));
            R e[9];
            euler_mat(st[0], -st[1], R(180) - st[2], e);
            R bst[5];
            for (int s = 0; s < nsym; ++s) {
                R m[9];
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        m[3 * a + b] = symr[9 * s + 3 * a] * e[b] + symr[9 * s + 3 * a + 1] * e[3 + b] +
                                       symr[9 * s + 3 * a + 2] * e[6 + b];
                R cand[5] = {std::acos(m[8]) * r2d, -std::atan2(m[5], m[2]) * r2d, std::atan2(m[7], m[6]) * r2d,
                             st[3], st[4]};
                R v = local_score(re.data(), im.data(), nx, cand, a2.data(), b2.data(), ctf.data(), w.data(), maxR);
                if (s == 0 || v < best) { best = v; std::copy(cand, cand + 5, bst); }
            }
            std::copy(bst, bst + 5, st);
        }
        R fac = 1;
        for (int cyc = 1; cyc <= p->ncycle; ++cyc) {
            R dang = (R)p->refine_angle * fac, dtran = (R)p->refine_shift * fac;
            fac = fac * (R)p->convf;
            R c11[11][5];
            for (int j = 0; j < 11; ++j) std::copy(st, st + 5, c11[j]);
            c11[1][3] -= dtran; c11[2][3] += dtran; c11[3][4] -= dtran; c11[4][4] += dtran;
            c11[5][0] -= dang; c11[6][0] += dang; c11[7][1] -= dang; c11[8][1] += dang;
            c11[9][2] -= dang; c11[10][2] += dang;
            int kb = 0;
            for (int j = 0; j < 11; ++j) {
                R v = local_score(re.data(), im.data(), nx, c11[j], a2.data(), b2.data(), ctf.data(), w.data(), maxR);
                if (j == 0 || v < best) { best = v; kb = j; }
            }
            std::copy(c11[kb], c11[kb] + 5, st);
        }
        q.local_dtheta = (float)(st[0] - (R)q.local_theta0);
        q.local_dphi = (float)(st[1] - (R)q.local_phi0);
        q.local_domega = (float)(st[2] - (R)q.local_omega0);
        q.local_dx = (float)(st[3] - (R)q.local_x0);
        q.local_dy = (float)(st[4] - (R)q.local_y0);
        q.local_theta = (float)st[0]; q.local_phi = (float)st[1]; q.local_omega = (float)st[2];
        q.local_x = (float)st[3]; q.local_y = (float)st[4];
        q.local_z = q.local_z0;
        q.local_pr = (float)best;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* proc_icos                                                                   */
/* ------------------------------------------------------------------------ */

template <class R> void euler_from(const R* r, R* th, R* ph, R* om) {
    const R r2d = C<R>::rad2deg();
    if (r[8] >= R(1)) *th = R(0);
    else if (r[8] < R(-1)) *th = R(180);
    else *th = std::acos(r[8]) * r2d;
    *ph = std::atan2(r[5], r[2]) * r2d;
    *om = std::atan2(r[7], -r[6]) * r2d;
}

/* proc_icos/SRC/equalort.f90:1-24 (generator order, as proc_icos uses). */
template <class R> void equalort(R th, R ph, R om, R* out) {
    R e[9], g[540];
    eular_matrix(th, ph, om, e);
    gen_ops<R>(g);
    for (int i = 0; i < 60; ++i) {
        R r[9];
        mm3(g + i * 9, e, r);
        euler_from(r, out + i * 3, out + i * 3 + 1, out + i * 3 + 2);
    }
}

/* proc_icos/SRC/transform_ort_2fTo5f.f90:11-30 (to=5), transform_ort_2fTo3f.f90:11-32 (to=3). */
template <class R> void transform_ort(int to, R* th, R* ph, R* om, int n) {
    const R d2r = R(4) * C<R>::q() / R(180);
    R rot0[9];
    if (to == 5) {
        R v = std::acos(std::cos(R(60) * d2r) / std::sin(R(36) * d2r));
        R t[9] = {std::cos(v), 0, std::sin(v), 0, 1, 0, -std::sin(v), 0, std::cos(v)};
        std::memcpy(rot0, t, sizeof(t));
    } else {
        R w = std::acos(std::cos(R(36) * d2r) / std::sin(R(60) * d2r));
        R t[9] = {1, 0, 0, 0, std::cos(-w), std::sin(-w), 0, -std::sin(-w), std::cos(-w)};
        std::memcpy(rot0, t, sizeof(t));
    }
    for (int i = 0; i < n; ++i) {
        R e[9], r[9];
        eular_matrix(th[i], ph[i], om[i], e);
        mm3(rot0, e, r);
        euler_from(r, th + i, ph + i, om + i);
    }
}

}  // namespace

/* ------------------------------------------------------------------------ */
/* exports                                                                     */
/* ------------------------------------------------------------------------ */
#define ORC_EXPORTS(R, S)                                                                              \
    extern "C" void orc_ctf2d_##S(int nx, R df1, R df2, R ast, R apix, R vol, R cs, R w, R* ctf) {  \
        get_ctf2d<R>(nx, df1, df2, ast, apix, vol, cs, w, ctf);                                        \
    }                                                                                                  \
    extern "C" void orc_mask_##S(R* d, int nx, R mask, R ox, R oy) { img2d_mask<R>(d, nx, mask, ox, oy); } \
    extern "C" void orc_fft2d_##S(R* a, R* b, int n1, int n2, int nbit) { img2d_fft<R>(a, b, n1, n2, nbit); } \
    extern "C" void orc_fft3d_##S(R* re, R* im, int n, int sign) { fft3d<R>(re, im, n, sign); }      \
    extern "C" void orc_expfit_##S(const R* a, const R* b, int nx, int mn, int mx, R* f) {           \
        ft_amp_expfit<R>(a, b, nx, mn, mx, f);                                                          \
    }                                                                                                  \
    extern "C" void orc_centshift_##S(R* a, R* b, int nx, R x0, R y0) { centshift<R>(a, b, nx, x0, y0); } \
    extern "C" void orc_norm_##S(R* img, int nx) { img2d_norm<R>(img, nx); }                          \
    extern "C" void orc_euler_##S(R th, R ph, R om, R* m) { euler_mat<R>(th, ph, om, m); }            \
    extern "C" void orc_icos_ops_##S(R* rot) { std::memcpy(rot, icos_ops<R>(), sizeof(R) * 540); }    \
    extern "C" void orc_icos_gen_##S(R* rot) { gen_ops<R>(rot); }                                      \
    extern "C" void orc_crosslin_##S(R a, R b, R c, R d, R e, R f, R* al1, R* al2) {                 \
        crosslin_angle<R>(a, b, c, d, e, f, al1, al2);                                                 \
    }                                                                                                  \
    extern "C" void orc_asu_fold_##S(R* th, R* ph, R* om) { asu_fold<R>(th, ph, om); }                \
    extern "C" void orc_fill_lin_##S(int nl, const R* a, const R* b, int nx, int mn, int mx,         \
                                      const R* al, R* out) {                                           \
        fill_lin<R>(nl, a, b, nx, mn, mx, al, out);                                                    \
    }                                                                                                  \
    extern "C" void orc_fill_lin_omega_##S(int nl, int nom, R st, const R* a, const R* b, int nx,   \
                                            int mn, int mx, const R* al, R* out) {                     \
        fill_lin_omega<R>(nl, nom, st, a, b, nx, mn, mx, al, out);                                     \
    }                                                                                                  \
    extern "C" void orc_pr_omega_##S(const R* pa, const R* pb, const R* f0, const R* tm,             \
                                      const R* to, const R* tf, const R* ctf, int T, int nx, int mn, \
                                      int mx, R st, int nom, R th, R ph, R om, R* pr) {               \
        pr_omega<R>(pa, pb, f0, tm, to, tf, ctf, T, nx, mn, mx, st, nom, th, ph, om, pr);              \
    }                                                                                                  \
    extern "C" R orc_pr_single_##S(const R* pa, const R* pb, const R* f0, const R* tm, const R* to,  \
                                    const R* tf, const R* ctf, int T, int nx, int mn, int mx, R th,   \
                                    R ph, R om, R x, R y) {                                            \
        return pr_single<R>(pa, pb, f0, tm, to, tf, ctf, T, nx, mn, mx, th, ph, om, x, y);            \
    }                                                                                                  \
    extern "C" void orc_prep_particle_##S(const float* img, int nx, int um, R mask, R x, R y,        \
                                           int shift, int mn, int mx, R* a, R* b, R* f) {             \
        prep_particle<R>(img, nx, um, mask, x, y, shift, mn, mx, a, b, f);                             \
    }                                                                                                  \
    extern "C" void orc_load_templates_##S(const float* im, const cryoim_template* t, int T,         \
                                            const cryoim_params* p, R* tm, R* tf) {                    \
        load_templates<R>(im, t, T, p, tm, tf);                                                        \
    }                                                                                                  \
    extern "C" int orc_globesearch_##S(const cryoim_params* p, const R* tm, const R* tf,             \
                                        const cryoim_template* t, int T, const float* im,            \
                                        cryoim_particle* pa, int P, float* pra, int nth) {            \
        return globesearch<R>(p, tm, tf, t, T, im, pa, P, pra, nth);                                   \
    }                                                                                                  \
    extern "C" int orc_refine_##S(const cryoim_params* p, const R* tm, const R* tf,                  \
                                   const cryoim_template* t, int T, const float* im,                  \
                                   cryoim_particle* pa, int P, int nth) {                              \
        return refine<R>(p, tm, tf, t, T, im, pa, P, nth);                                             \
    }                                                                                                  \
    extern "C" int orc_search_views_##S(const cryoim_params* p, const R* tm, const R* tf,            \
                                         const cryoim_template* t, int T, const float* img,          \
                                         const cryoim_particle* q, const float* views, int nv,       \
                                         int nth, float* out) {                                       \
        return search_views<R>(p, tm, tf, t, T, img, q, views, nv, nth, out);                          \
    }                                                                                                  \
    extern "C" void orc_project_template2d_##S(const float* map, int nx, R th, R ph, R om, R* o) {  \
        project_template2d<R>(map, nx, th, ph, om, o);                                                 \
    }                                                                                                  \
    extern "C" void orc_central_section_gauss_##S(const R* fr, const R* fi, int nx, R th, R ph, R om, R sg,   \
                                                   R* ore, R* oim) {                                       \
        central_section_gauss<R>(fr, fi, nx, th, ph, om, sg, ore, oim);                                   \
    }                                                                                                  \
    extern "C" void orc_central_section_##S(const R* fr, const R* fi, int nx, R th, R ph, R om,     \
                                             R* orr, R* oi) {                                          \
        central_section<R>(fr, fi, nx, th, ph, om, orr, oi);                                           \
    }                                                                                                  \
    extern "C" int orc_reconstruct_##S(const cryoim_params* p, const float* im,                      \
                                        const cryoim_particle* pa, int P, float* map, R* acc) {       \
        return reconstruct<R>(p, im, pa, P, map, acc);                                                 \
    }                                                                                                  \
    extern "C" int orc_reconstruct_half_##S(const cryoim_params* p, const float* im,                 \
                                             const cryoim_particle* pa, int P, int parity, R* fa,      \
                                             R* fb, R* wg) {                                           \
        return reconstruct_half<R>(p, im, pa, P, parity, fa, fb, wg);                                  \
    }                                                                                                  \
    extern "C" int orc_fsc_combine_##S(int nx, int maxR, const float* a1, const float* b1,           \
                                        const float* w1, const float* a2, const float* b2,             \
                                        const float* w2, R* fsc, float* map) {                         \
        return fsc_combine<R>(nx, maxR, a1, b1, w1, a2, b2, w2, fsc, map);                             \
    }                                                                                                  \
    extern "C" int orc_merge_fsc_##S(int nx, int maxR, const float* a1, const float* b1,             \
                                      const float* w1, const float* a2, const float* b2,               \
                                      const float* w2, R imgmask, R* fsc, float* map) {                \
        return fsc_combine<R>(nx, maxR, a1, b1, w1, a2, b2, w2, fsc, map, true, imgmask);              \
    }                                                                                                  \
    extern "C" int orc_merge_finish_##S(int nx, int maxR, const float* a, const float* b,            \
                                         const float* w, float* map) {                                 \
        return merge_finish<R>(nx, maxR, a, b, w, map);                                                \
    }                                                                                                  \
    extern "C" void orc_icosavg_##S(const float* in, int nx, R r0, float* out) {                     \
        icosavg<R>(in, nx, r0, out);                                                                   \
    }                                                                                                  \
    extern "C" int orc_center_##S(const cryoim_params* p, const float* map, const float* im,         \
                                   const cryoim_particle* pa, int P, R* out) {                         \
        return center<R>(p, map, im, pa, P, out);                                                      \
    }                                                                                                  \
    extern "C" void orc_lowpass_##S(R* a, int nx, int lp) { img2d_lowpass<R>(a, nx, lp); }          \
    extern "C" int orc_local_box_coordinates_##S(const cryoim_particle* pa, int P, const float* sym,   \
                                                  int nsym, R lx, R ly, R lz, R apix, int nx, R prt,   \
                                                  R bx, cryoim_local_particle* out) {                  \
        return local_box_coordinates<R>(pa, P, sym, nsym, lx, ly, lz, apix, nx, prt, bx, out);         \
    }                                                                                                  \
    extern "C" int orc_local_box_extract_##S(const float* im, const cryoim_particle* pa, int P, int nx0, \
                                              const float* sym, int nsym, R lx, R ly, R lz, R apix,      \
                                              int sub, R prt, R bx, float* so, cryoim_local_particle* o) { \
        return local_box_extract<R>(im, pa, P, nx0, sym, nsym, lx, ly, lz, apix, sub, prt, bx, so, o);   \
    }                                                                                                  \
    extern "C" int orc_local_refine_##S(const cryoim_local_params* p, const float* map,              \
                                         const float* im, cryoim_local_particle* pa, int P) {          \
        return local_refine<R>(p, map, im, pa, P);                                                     \
    }                                                                                                  \
    extern "C" void orc_gauss_regression_##S(const R* z, R* out) {                                   \
        R zz[3][3];                                                                                    \
        for (int k = 0; k < 9; ++k) zz[k / 3][k % 3] = z[k];                                           \
        gauss_regression<R>(zz, &out[0], &out[1], &out[2]);                                            \
    }                                                                                                  \
    extern "C" void orc_equalort_##S(R th, R ph, R om, R* out) { equalort<R>(th, ph, om, out); }      \
    extern "C" void orc_transform_ort_##S(int to, R* th, R* ph, R* om, int n) {                      \
        transform_ort<R>(to, th, ph, om, n);                                                           \
    }

ORC_EXPORTS(float, f32)
ORC_EXPORTS(double, f64)

extern "C" void orc_grid_sizes(float step, int* nth, int* nph, int* nom) { grid_sizes(step, nth, nph, nom); }
extern "C" int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* icosprocess/SRC/0initialvalue.f90:26-45: the code defaults for a stack of nx =
 * fftsize (the keys 0input_parameters.f90 does not set: mode 0, first 1, applyCTF and
 * imgmask y, the rest n). */
extern "C" void orc_params_default(cryoim_params* p, int fftsize) {
    std::memset(p, 0, sizeof(*p));
    p->fftsize = fftsize;
    p->first = 1;
    p->ncycle = 6;
    p->apply_ctf = 1;
    p->use_imgmask = 1;
    p->imgmask = (float)(fftsize / 2 - 2);
    p->boundx = (float)(fftsize / 2 - 2);
    p->pr_threshold = 90.0f;
    p->vol = 300.0f;
    p->cs = 2.7f;
    p->ampwg = 0.1f;
    p->bfactor = 0.0f;
    p->min_res = 300.0f;
    p->max_res = 8.0f;
    p->apix = 1.0f;
    p->nsym = 60;
    p->nlin = 60;
    p->searchstep = 2.0f;
    p->maxcentshift = 100.0f;
}

/* icosprocess/SRC/0calc_initialvalues.f90:4-20 (mode != 6, icosahedral symmetry):
 * resolutions to radii in FP32, maxR rounded up to even, the mask to pixels, and the
 * refinement steps. */
extern "C" void orc_params_derive(cryoim_params* p) {
    float minres = p->apix * (float)p->fftsize / p->min_res;
    float maxres = p->apix * (float)p->fftsize / p->max_res;
    p->min_r = (int)minres;
    p->max_r = (int)maxres;
    if (p->max_r % 2 != 0) p->max_r += 1;
    p->imgmask_px = p->use_imgmask ? p->imgmask / p->apix : p->imgmask;
    p->delta_angle = 360.0f / (maxres * std::sqrt(5.0f) * 3.14159f);
    p->delta_trans = (float)p->fftsize / (maxres * std::sqrt(5.0f));
}
