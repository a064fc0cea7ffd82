// proc_icos — drop-in for the reference's `proc_icos` orientation utility.
//
// Keys (proc_icos/SRC/0inputpars.f90:3-11): ort0, newort, calc_randort_2f,
// calc_matrix_2f, calc_matrix_5f, transform_ort_2fTo5f, PR_threshold, calc_matrix_3f,
// transform_ort_2fTo3f.  Orientation rows are read as 13 list-directed columns and
// written with proc_icos's a64 row (transform_ort_2fTo5f.f90:36).
//  * transform_ort_2fTo5f / 2fTo3f: the 2-fold -> 5-fold / 3-fold frame change.
//  * calc_randort_2f: one random symmetry-equivalent orientation per particle.  The
//    reference seeds from the clock and draws int(u*60), which can index operator 0
//    (calc_randort_2f.f90:20); here the seed is the `seed` extension key (default 1) and
//    the index is int(u*60)+1 in 1..60.
//  * calc_matrix_2f / 3f / 5f: print the 60 rotations in the 2-fold frame (table order of
//    icos2f_sym_mat.f90) or conjugated into the 3-fold / 5-fold frame.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <vector>

#include "cryoim.h"

namespace {
const char* kKeys[] = {"ort0", "newort", "calc_randort_2f", "calc_matrix_2f", "calc_matrix_5f",
                       "transform_ort_2fTo5f", "PR_threshold", "calc_matrix_3f", "transform_ort_2fTo3f",
                       "seed"};
void usage() {
    std::puts("proc_icos (cryoim_gb300): icosahedral orientation utilities\n"
              "usage: proc_icos ort0=in.dat newort=out.dat [transform_ort_2fTo5f=y | transform_ort_2fTo3f=y |\n"
              "       calc_randort_2f=y | calc_matrix_2f=y | calc_matrix_3f=y | calc_matrix_5f=y] [seed=1]");
}
bool yes(const std::string& v) { return !v.empty() && (v[0] == 'y' || v[0] == 'Y'); }

void print_matrices(int frame) {
    float r[540];
    cryoim_icos_ops(r);
    const double d2r = 3.14159265358979323846 / 180.0;
    double rot0[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (frame == 5) {
        double v = std::acos(std::cos(60 * d2r) / std::sin(36 * d2r));
        double t[9] = {std::cos(v), 0, std::sin(v), 0, 1, 0, -std::sin(v), 0, std::cos(v)};
        std::memcpy(rot0, t, sizeof(t));
    } else if (frame == 3) {
        double w = std::acos(std::cos(36 * d2r) / std::sin(60 * d2r));
        double t[9] = {1, 0, 0, 0, std::cos(-w), std::sin(-w), 0, -std::sin(-w), std::cos(-w)};
        std::memcpy(rot0, t, sizeof(t));
    }
    for (int k = 0; k < 60; ++k) {
        double m[9];  // rot0 * R * rot0^T
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) s += rot0[i * 3 + a] * r[k * 9 + a * 3 + b] * rot0[j * 3 + b];
                m[i * 3 + j] = s;
            }
        for (int i = 0; i < 3; ++i) std::printf("%14.8f%14.8f%14.8f\n", m[i * 3], m[i * 3 + 1], m[i * 3 + 2]);
        std::puts("");
    }
}
}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) { usage(); return 0; }
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        size_t e = a.find('=');
        std::string k = e == std::string::npos ? a : a.substr(0, e);
        bool known = false;
        for (const char* x : kKeys) known |= (k == x);
        if (!known || e == std::string::npos) { usage(); return 0; }
        kv[k] = a.substr(e + 1);
    }
    auto on = [&](const char* k) { return kv.count(k) && yes(kv[k]); };
    if (on("calc_matrix_2f")) print_matrices(2);
    if (on("calc_matrix_3f")) print_matrices(3);
    if (on("calc_matrix_5f")) print_matrices(5);
    const bool t5 = on("transform_ort_2fTo5f"), t3 = on("transform_ort_2fTo3f"), rnd = on("calc_randort_2f");
    if (!(t5 || t3 || rnd)) return 0;
    if (!kv.count("ort0") || !kv.count("newort")) { usage(); return 0; }
    int32_t n = 0;
    if (cryoim_ort_count(kv["ort0"].c_str(), &n) || n < 1) { std::fprintf(stderr, "proc_icos: cannot read ort0\n"); return 2; }
    std::vector<cryoim_particle> parts(n);
    std::vector<char> names((size_t)n * 64);
    if (cryoim_ort_read(kv["ort0"].c_str(), 1, n, parts.data(), names.data(), 64)) {
        std::fprintf(stderr, "proc_icos: malformed ort0\n");
        return 2;
    }
    std::vector<float> th(n), ph(n), om(n);
    for (int i = 0; i < n; ++i) { th[i] = parts[i].theta; ph[i] = parts[i].phi; om[i] = parts[i].omega; }
    if (t5 || t3) {
        cryoim_transform_ort(t5 ? 5 : 3, th.data(), ph.data(), om.data(), n);
    } else {
        std::mt19937 g((unsigned)std::atoi(kv.count("seed") ? kv["seed"].c_str() : "1"));
        std::uniform_real_distribution<float> u(0.0f, 1.0f);
        for (int i = 0; i < n; ++i) {
            float eq[180];
            cryoim_equalort(th[i], ph[i], om[i], eq);
            int k = (int)(u(g) * 60.0f);
            if (k > 59) k = 59;
            th[i] = eq[3 * k]; ph[i] = eq[3 * k + 1]; om[i] = eq[3 * k + 2];
            parts[i].particle_id = i + 1;  // calc_randort_2f.f90:22 writes the running count
        }
    }
    for (int i = 0; i < n; ++i) { parts[i].theta = th[i]; parts[i].phi = ph[i]; parts[i].omega = om[i]; }
    if (cryoim_ort_write(kv["newort"].c_str(), parts.data(), names.data(), 64, n, 64, 0)) {
        std::fprintf(stderr, "proc_icos: cannot write newort\n");
        return 2;
    }
    std::printf(" the new ortfile is written in %s\n", kv["newort"].c_str());
    return 0;
}
