// io.cpp — the reference's file formats, byte-compatible.
//
//  * MRC: the 1024-byte `mrchead` type of icosprocess/SRC/0common_icosproc.f90:61-112
//    followed by float32 data (mode 2), x fastest; stream access, no record markers.
//  * orientation files: list-directed rows `stck particleID theta phi omega x y PR imgID
//    imgparticleID df1 df2 astigang` (load_original_ortcent.f90:12-16) and the 19-column
//    output row of format 900 (ort_globesearch.f90:139):
//    (a54,i8,6f10.4,i12,i6,9f10.4); proc_icos writes a64 and 13 columns
//    (transform_ort_2fTo5f.f90:36).
//  * template orientations: `particleID theta phi omega x y` (load_template.f90:19).
//  * tnf partial reconstruction: FFTsize, maxR (int32), apix, imgmask (float32),
//    flagFSC, flagAvg (int32), then fa, fb, wg of (2 maxR + 1)^2 (maxR + 1) float32
//    (reconstruct_substep.f90:152-155).
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cryoim.h"

namespace {

static_assert(sizeof(cryoim_mrc_header) == 1024, "MRC header must be 1024 bytes");

// Fortran Fw.d / Iw edit descriptors: right-justified, '*' fill on overflow.
void put_f(std::string& s, double v, int w, int d) {
    char b[64];
    int n = std::snprintf(b, sizeof(b), "%*.*f", w, d, v);
    if (n > w) s.append((size_t)w, '*');
    else s.append(b);
}
void put_i(std::string& s, long v, int w) {
    char b[64];
    int n = std::snprintf(b, sizeof(b), "%*ld", w, v);
    if (n > w) s.append((size_t)w, '*');
    else s.append(b);
}
void put_a(std::string& s, const char* name, int w) {
    std::string t(name ? name : "");
    if ((int)t.size() > w) t.resize(w);
    s += t;
    s.append((size_t)(w - (int)t.size()), ' ');
}

// Tokens of a list-directed record (blanks, tabs and commas separate values).
std::vector<std::string> tokens(const char* line) {
    std::vector<std::string> out;
    std::string cur;
    bool q = false;
    char qc = 0;
    for (const char* p = line; *p && *p != '\n' && *p != '\r'; ++p) {
        char ch = *p;
        if (q) {
            if (ch == qc) q = false;
            else cur += ch;
            continue;
        }
        if (ch == '\'' || ch == '"') { q = true; qc = ch; continue; }
        if (ch == ' ' || ch == '\t' || ch == ',') {
            if (!cur.empty()) { out.push_back(cur); cur.clear(); }
            continue;
        }
        cur += ch;
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

bool to_f(const std::string& s, float* v) {
    char* e = nullptr;
    std::string t = s;
    for (char& c : t)
        if (c == 'd' || c == 'D') c = 'e';  // Fortran double exponent
    *v = std::strtof(t.c_str(), &e);
    return e && *e == 0;
}
bool to_i(const std::string& s, int32_t* v) {
    char* e = nullptr;
    long x = std::strtol(s.c_str(), &e, 10);
    if (!e || *e != 0) {
        float f;  // list-directed integer input also accepts a real with no fraction
        if (!to_f(s, &f) || f != std::floor(f)) return false;
        x = (long)f;
    }
    *v = (int32_t)x;
    return true;
}

}  // namespace

extern "C" {

int cryoim_mrc_read_header(const char* path, cryoim_mrc_header* h) {
    if (!path || !h) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return CRYOIM_ERR_IO;
    size_t n = std::fread(h, 1, sizeof(*h), f);
    std::fclose(f);
    return n == sizeof(*h) ? CRYOIM_OK : CRYOIM_ERR_IO;
}

int cryoim_mrc_read_sections(const char* path, int32_t first, int32_t count, float* out) {
    if (!path || !out || first < 1 || count < 0) return CRYOIM_ERR_ARG;
    cryoim_mrc_header h;
    int r = cryoim_mrc_read_header(path, &h);
    if (r) return r;
    if (h.mode != 2) return CRYOIM_ERR_IO;
    if (first - 1 + count > h.nz) return CRYOIM_ERR_MISMATCH;
    FILE* f = std::fopen(path, "rb");
    if (!f) return CRYOIM_ERR_IO;
    const long long sec = (long long)h.nx * h.ny;
    const long long off = 1024 + (long long)h.nsymbt + (long long)(first - 1) * sec * 4;
    if (std::fseek(f, (long)off, SEEK_SET) != 0) { std::fclose(f); return CRYOIM_ERR_IO; }
    size_t want = (size_t)(sec * count), n = std::fread(out, sizeof(float), want, f);
    std::fclose(f);
    return n == want ? CRYOIM_OK : CRYOIM_ERR_IO;
}

// mrchead.f90:2-58 (maphead): header of an FFTsize^3 float map.
int cryoim_map_header(cryoim_mrc_header* h, int32_t nx, int32_t ny, int32_t nz, float apix) {
    if (!h) return CRYOIM_ERR_ARG;
    std::memset(h, 0, sizeof(*h));
    h->nx = nx; h->ny = ny; h->nz = nz; h->mode = 2;
    h->nxstart = -nx / 2; h->nystart = -ny / 2; h->nzstart = -nz / 2;
    h->mx = nx - 1; h->my = ny - 1; h->mz = nz - 1;
    h->a = (float)h->mx * apix; h->b = (float)h->my * apix; h->c = (float)h->my * apix;
    h->alpha = 90; h->beta = 90; h->gamma = 90;
    h->mapc = 1; h->mapr = 2; h->maps = 3;
    h->xorigin = -1.0f * (float)nx; h->yorigin = -1.0f * (float)ny; h->zorigin = -1.0f * (float)nz;
    // mrchead.f90:60-66 assigns 'map ', 'lhr' and 'Hongrong Liu' to arrays of single
    // characters (0common_icosproc.f90:104-111): every element takes the first letter.
    std::memset(h->map, 'm', 4);
    std::memset(h->machinestamp, 'l', 4);
    std::memset(h->label, 'H', sizeof(h->label));
    return CRYOIM_OK;
}

int cryoim_mrc_write(const char* path, const cryoim_mrc_header* h, const float* data, int64_t n) {
    if (!path || !h || (!data && n > 0) || n < 0) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return CRYOIM_ERR_IO;
    bool ok = std::fwrite(h, 1, sizeof(*h), f) == sizeof(*h);
    ok = ok && std::fwrite(data, sizeof(float), (size_t)n, f) == (size_t)n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? CRYOIM_OK : CRYOIM_ERR_IO;
}

int cryoim_ort_count(const char* path, int32_t* n) {
    if (!path || !n) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) return CRYOIM_ERR_IO;
    char line[4096];
    int32_t c = 0;
    while (std::fgets(line, sizeof(line), f))
        if (!tokens(line).empty()) ++c;
    std::fclose(f);
    *n = c;
    return CRYOIM_OK;
}

// load_original_ortcent.f90:9-16: rows first..last (1-based) of a 13-column ort file.
int cryoim_ort_read(const char* path, int32_t first, int32_t last, cryoim_particle* parts,
                    char* stck, int32_t stck_len) {
    if (!path || !parts || first < 1 || last < first || (stck && stck_len < 1)) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) return CRYOIM_ERR_IO;
    char line[4096];
    int32_t row = 0, k = 0;
    int rc = CRYOIM_OK;
    while (std::fgets(line, sizeof(line), f)) {
        std::vector<std::string> t = tokens(line);
        if (t.empty()) continue;
        ++row;
        if (row < first) continue;
        if (row > last) break;
        if (t.size() < 13) { rc = CRYOIM_ERR_IO; break; }
        cryoim_particle& q = parts[k];
        std::memset(&q, 0, sizeof(q));
        bool ok = to_i(t[1], &q.particle_id) && to_f(t[2], &q.theta) && to_f(t[3], &q.phi) &&
                  to_f(t[4], &q.omega) && to_f(t[5], &q.x) && to_f(t[6], &q.y) && to_f(t[7], &q.pr) &&
                  to_i(t[8], &q.img_id) && to_i(t[9], &q.img_particle_id) && to_f(t[10], &q.df1) &&
                  to_f(t[11], &q.df2) && to_f(t[12], &q.astigang);
        if (!ok) { rc = CRYOIM_ERR_INPUT; break; }
        if (stck) {
            char* dst = stck + (size_t)k * stck_len;
            std::memset(dst, 0, (size_t)stck_len);
            std::strncpy(dst, t[0].c_str(), (size_t)stck_len - 1);
        }
        ++k;
    }
    std::fclose(f);
    if (rc == CRYOIM_OK && k != last - first + 1) rc = CRYOIM_ERR_IO;  // short file
    return rc;
}

// format 900 of ort_globesearch.f90:139 (width 54) or proc_icos's 13 columns (width 64).
int cryoim_ort_write(const char* path, const cryoim_particle* parts, const char* stck,
                     int32_t stck_len, int32_t n, int32_t name_width, int32_t append) {
    if (!path || (!parts && n > 0) || n < 0 || (stck && stck_len < 1)) return CRYOIM_ERR_ARG;
    if (name_width != 54 && name_width != 64) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, append ? "a" : "w");
    if (!f) return CRYOIM_ERR_IO;
    std::string s;
    for (int32_t i = 0; i < n; ++i) {
        const cryoim_particle& q = parts[i];
        s.clear();
        put_a(s, stck ? stck + (size_t)i * stck_len : "", name_width);
        put_i(s, q.particle_id, 8);
        for (float v : {q.theta, q.phi, q.omega, q.x, q.y, q.pr}) put_f(s, v, 10, 4);
        put_i(s, q.img_id, 12);
        put_i(s, q.img_particle_id, 6);
        if (name_width == 54) {
            for (float v : {q.df1, q.df2, q.astigang, q.dtheta, q.dphi, q.domega, q.dx, q.dy, q.dpr})
                put_f(s, v, 10, 4);
        } else {
            put_f(s, q.df1, 15, 4);
            put_f(s, q.df2, 15, 4);
            put_f(s, q.astigang, 10, 4);
        }
        s += '\n';
        std::fputs(s.c_str(), f);
    }
    return std::fclose(f) == 0 ? CRYOIM_OK : CRYOIM_ERR_IO;
}

// local_refine/SRC/load_original_ort.f90:12-15: the 23 list-directed columns of rows
// first..last.
int cryoim_local_ort_read(const char* path, int32_t first, int32_t last, cryoim_local_particle* parts,
                          char* stck, int32_t stck_len) {
    if (!path || !parts || first < 1 || last < first || (stck && stck_len < 1)) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) return CRYOIM_ERR_IO;
    char line[8192];
    int32_t row = 0, k = 0;
    int rc = CRYOIM_OK;
    while (std::fgets(line, sizeof(line), f)) {
        std::vector<std::string> t = tokens(line);
        if (t.empty()) continue;
        ++row;
        if (row < first) continue;
        if (row > last) break;
        if (t.size() < 23) { rc = CRYOIM_ERR_IO; break; }
        cryoim_local_particle& q = parts[k];
        std::memset(&q, 0, sizeof(q));
        bool ok = to_i(t[1], &q.particle_id) && to_f(t[2], &q.theta) && to_f(t[3], &q.phi) &&
                  to_f(t[4], &q.omega) && to_f(t[5], &q.x) && to_f(t[6], &q.y) && to_f(t[7], &q.pr) &&
                  to_i(t[8], &q.img_id) && to_i(t[9], &q.img_particle_id) && to_f(t[10], &q.df1) &&
                  to_f(t[11], &q.df2) && to_f(t[12], &q.astigang) && to_i(t[13], &q.local_img_id) &&
                  to_i(t[14], &q.local_hx0) && to_i(t[15], &q.local_ky0) && to_f(t[16], &q.local_theta0) &&
                  to_f(t[17], &q.local_phi0) && to_f(t[18], &q.local_omega0) && to_f(t[19], &q.local_x0) &&
                  to_f(t[20], &q.local_y0) && to_f(t[21], &q.local_z0) && to_f(t[22], &q.local_pr0);
        if (!ok) { rc = CRYOIM_ERR_INPUT; break; }
        if (stck) {
            char* dst = stck + (size_t)k * stck_len;
            std::memset(dst, 0, (size_t)stck_len);
            std::strncpy(dst, t[0].c_str(), (size_t)stck_len - 1);
        }
        ++k;
    }
    std::fclose(f);
    if (rc == CRYOIM_OK && k != last - first + 1) rc = CRYOIM_ERR_IO;
    return rc;
}

// format 900 of local_box/SRC/loc_box_coordinate.f90:46 (23 columns), format 901 of
// local_refine/SRC/refine_PR.f90:246-253 (28 columns; its PR column is local_PR), or
// format 900 of local_box/SRC/loc_box.f90:93 (14 columns: the sub-image stack mode).
int cryoim_local_ort_write(const char* path, const cryoim_local_particle* parts, const char* stck,
                           int32_t stck_len, int32_t n, int32_t columns, int32_t append) {
    if (!path || (!parts && n > 0) || n < 0 || (stck && stck_len < 1)) return CRYOIM_ERR_ARG;
    if (columns != 23 && columns != 28 && columns != 14) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, append ? "a" : "w");
    if (!f) return CRYOIM_ERR_IO;
    std::string s;
    const bool box = columns == 23;
    for (int32_t i = 0; i < n; ++i) {
        const cryoim_local_particle& q = parts[i];
        s.clear();
        put_a(s, stck ? stck + (size_t)i * stck_len : "", 64);
        if (columns == 14) {  // (a64,i8,f10.4 x 6,i12,i6,f10.4 x 3,f12.4)
            put_i(s, q.particle_id, 8);
            for (float v : {q.local_theta0, q.local_phi0, q.local_omega0, q.local_x0, q.local_y0, q.pr})
                put_f(s, v, 10, 4);
            put_i(s, q.img_id, 12);
            put_i(s, q.local_img_id, 6);
            for (float v : {q.df1, q.df2, q.astigang}) put_f(s, v, 10, 4);
            put_f(s, q.local_z0, 12, 4);
            s += '\n';
            std::fputs(s.c_str(), f);
            continue;
        }
        put_i(s, q.particle_id, box ? 8 : 9);
        for (float v : {q.theta, q.phi, q.omega, q.x, q.y}) put_f(s, v, 10, 4);
        put_f(s, box ? q.pr : q.local_pr, 10, 4);
        put_i(s, q.img_id, box ? 12 : 11);
        put_i(s, q.img_particle_id, box ? 6 : 7);
        put_f(s, q.df1, 15, 4);
        put_f(s, q.df2, 15, 4);
        put_f(s, q.astigang, 10, 4);
        put_i(s, q.local_img_id, 9);
        put_i(s, q.local_hx0, 6);
        put_i(s, q.local_ky0, 6);
        if (box) {
            for (float v : {q.local_theta0, q.local_phi0, q.local_omega0, q.local_x0, q.local_y0}) put_f(s, v, 10, 4);
            put_f(s, q.local_z0, 11, 4);
            put_f(s, q.local_pr0, 11, 4);
        } else {
            for (float v : {q.local_theta, q.local_phi, q.local_omega, q.local_x, q.local_y}) put_f(s, v, 10, 4);
            put_f(s, q.local_z, 11, 4);
            put_f(s, q.local_pr, 10, 4);
            for (float v : {q.local_dtheta, q.local_dphi, q.local_domega, q.local_dx, q.local_dy})
                put_f(s, v, 10, 4);
        }
        s += '\n';
        std::fputs(s.c_str(), f);
    }
    return std::fclose(f) == 0 ? CRYOIM_OK : CRYOIM_ERR_IO;
}

// load_template.f90:18-21 (the file's first rows; 0main.f90:53-58 counts them).
int cryoim_template_ort_read(const char* path, cryoim_template* t, int32_t maxn, int32_t* n) {
    if (!path || !n || maxn < 0 || (!t && maxn > 0)) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) return CRYOIM_ERR_IO;
    char line[4096];
    int32_t k = 0;
    int rc = CRYOIM_OK;
    while (std::fgets(line, sizeof(line), f)) {
        std::vector<std::string> tk = tokens(line);
        if (tk.empty()) continue;
        if (tk.size() < 6) { rc = CRYOIM_ERR_INPUT; break; }
        if (k < maxn) {
            cryoim_template& x = t[k];
            if (!(to_i(tk[0], &x.particle_id) && to_f(tk[1], &x.theta) && to_f(tk[2], &x.phi) &&
                  to_f(tk[3], &x.omega) && to_f(tk[4], &x.x) && to_f(tk[5], &x.y))) {
                rc = CRYOIM_ERR_INPUT;
                break;
            }
        }
        ++k;
    }
    std::fclose(f);
    *n = k;
    return rc;
}

int cryoim_tnf_write(const char* path, int32_t fftsize, int32_t max_r, float apix, float imgmask,
                     int32_t flag_fsc, int32_t flag_avg, const float* fa, const float* fb,
                     const float* wg) {
    if (!path || !fa || !fb || !wg || max_r < 1) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return CRYOIM_ERR_IO;
    const size_t n = (size_t)(2 * max_r + 1) * (2 * max_r + 1) * (max_r + 1);
    bool ok = std::fwrite(&fftsize, 4, 1, f) == 1 && std::fwrite(&max_r, 4, 1, f) == 1 &&
              std::fwrite(&apix, 4, 1, f) == 1 && std::fwrite(&imgmask, 4, 1, f) == 1 &&
              std::fwrite(&flag_fsc, 4, 1, f) == 1 && std::fwrite(&flag_avg, 4, 1, f) == 1;
    ok = ok && std::fwrite(fa, 4, n, f) == n && std::fwrite(fb, 4, n, f) == n && std::fwrite(wg, 4, n, f) == n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? CRYOIM_OK : CRYOIM_ERR_IO;
}

// hdr: fftsize, max_r, flag_fsc, flag_avg (int32) and apix, imgmask (float).  fa/fb/wg may
// be NULL to read the header only.
int cryoim_tnf_read(const char* path, int32_t* ihdr, float* fhdr, float* fa, float* fb, float* wg) {
    if (!path || !ihdr || !fhdr) return CRYOIM_ERR_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return CRYOIM_ERR_IO;
    int32_t a[2], b[2];
    float c[2];
    bool ok = std::fread(a, 4, 2, f) == 2 && std::fread(c, 4, 2, f) == 2 && std::fread(b, 4, 2, f) == 2;
    if (ok && (a[1] < 1 || a[1] > 4096)) ok = false;
    if (ok) {
        ihdr[0] = a[0]; ihdr[1] = a[1]; ihdr[2] = b[0]; ihdr[3] = b[1];
        fhdr[0] = c[0]; fhdr[1] = c[1];
        if (fa && fb && wg) {
            const size_t n = (size_t)(2 * a[1] + 1) * (2 * a[1] + 1) * (a[1] + 1);
            ok = std::fread(fa, 4, n, f) == n && std::fread(fb, 4, n, f) == n && std::fread(wg, 4, n, f) == n;
        }
    }
    std::fclose(f);
    return ok ? CRYOIM_OK : CRYOIM_ERR_IO;
}

}  // extern "C"
