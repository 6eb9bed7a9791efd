// sph_host.cpp -- host-only parts of the C ABI: parameter defaults and
// validation, the exact FP32 cutoff, grid geometry and the scene generators.
// No CUDA call here: these work on a machine without a GPU.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/sph_gb300.h"
#include "sph_host.h"

namespace sphgb {

float cutoff_d2(float h) {
    // sqrtf is correctly rounded and monotone, so {d2 : sqrtf(d2) < h} = {d2 < T}.
    float t = h * h;
    while (t > 0.0f && std::sqrt(std::nextafter(t, 0.0f)) >= h) t = std::nextafter(t, 0.0f);
    while (std::sqrt(t) < h) t = std::nextafter(t, INFINITY);
    return t;
}

float smoothing_length(const sph_params& p) {
    return p.smoothing_coeff * p.particle_radius;  // rho_pres_comp.glsl:40, FP32 product
}

float cell_edge(const sph_params& p, int stencil) {
    const float smin = 1.0f + 1.0f / 1024.0f;  // margin for the rounding of the cell index
    float s = p.cell_scale;
    if (!(s >= smin)) s = smin;
    return smoothing_length(p) * s / (float)stencil;
}

bool grid_dims(const sph_params& p, int stencil, float* edge_out, int dims[3]) {
    float e = cell_edge(p, stencil);
    if (!(e > 0.0f) || !std::isfinite(e)) return false;
    long long total = 1;
    for (int a = 0; a < 3; ++a) {
        double ext = (double)p.upper[a] - (double)p.lower[a];
        double d = std::ceil(ext / (double)e);
        if (!(d >= 1.0)) d = 1.0;
        if (d > (double)(1 << 20)) return false;
        dims[a] = (int)d;
        total *= dims[a];
    }
    if (edge_out) *edge_out = e;
    return total <= (1ll << 30);
}

SceneDev make_scene_dev(const sph_params& p, int stencil, int cell_base, int first, int count, bool keep_force) {
    SceneDev s{};
    const float hf = smoothing_length(p);
    const double h = hf, PI = 3.141592741f, m = p.mass;
    s.h = hf;
    s.cut_d2 = cutoff_d2(hf);
    s.h2 = hf * hf;
    float e = 1.0f;
    grid_dims(p, stencil, &e, s.dim);
    s.inv_edge = 1.0f / e;
    for (int a = 0; a < 3; ++a) { s.lo[a] = p.lower[a]; s.up[a] = p.upper[a]; s.g[a] = p.gravity[a]; }
    s.cell_base = cell_base;
    s.first = first;
    s.count = count;
    s.poly6c = (float)(m * 315.0 / (64.0 * PI * std::pow(h, 9)));
    s.gas_k = p.gas_const;
    s.rho0 = p.resting_rho;
    s.pres_c = (float)(m * 45.0 / (PI * std::pow(h, 6)) / 2.0);
    s.visc_c = (float)((double)p.visc * m * 45.0 / (PI * std::pow(h, 6)));
    s.dt = p.dt;
    s.damp = p.damping;
    s.mass = p.mass;
    s.keep_force = keep_force ? 1 : 0;
    return s;
}

// splitmix64 of (seed, counter): the jitter stream of the scene generators.
static inline uint64_t splitmix(uint64_t seed, uint64_t ctr) {
    uint64_t z = seed + (ctr + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// Uniform in [-1, 1) with 24-bit resolution.
static inline double unit_pm(uint64_t seed, uint64_t ctr) {
    return (double)(splitmix(seed, ctr) >> 40) / (double)(1ull << 23) - 1.0;
}

}  // namespace sphgb

using namespace sphgb;

extern "C" {

const char* sph_version(void) { return "sph_gb300 1.0 sm_103a"; }

void sph_params_default(sph_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->mass = 0.02f;             // Main.cpp:112
    p->smoothing_coeff = 4.0f;   // Main.cpp:113
    p->visc = 3000.0f;           // Main.cpp:114
    p->resting_rho = 1000.0f;    // Main.cpp:115
    const float up[4] = {0.5f, 1.0f, 0.5f, 1.0f}, lo[4] = {-0.1f, -0.35f, -0.1f, 1.0f};  // Main.cpp:120-121
    std::memcpy(p->upper, up, sizeof(up));
    std::memcpy(p->lower, lo, sizeof(lo));
    p->particle_radius = 0.005f; // rho_pres_comp.glsl:5
    p->gas_const = 2000.0f;      // rho_pres_comp.glsl:33
    p->gravity[0] = 0.0f;        // force_comp.glsl:33
    p->gravity[1] = -9806.65f;
    p->gravity[2] = 0.0f;
    p->dt = 1.0f / 10000;        // integrate_comp.glsl:33 (1/NUM_PARTICLES)
    p->damping = 0.3f;           // integrate_comp.glsl:8
    p->cell_scale = 0.0f;
    p->flags = 0;
}

sph_status sph_params_validate(const sph_params* p) {
    if (!p) return SPH_ERR_INVALID_ARG;
    const float f[] = {p->mass, p->smoothing_coeff, p->visc, p->resting_rho, p->particle_radius, p->gas_const,
                       p->gravity[0], p->gravity[1], p->gravity[2], p->dt, p->damping, p->cell_scale};
    for (float x : f)
        if (!std::isfinite(x)) return SPH_ERR_INVALID_ARG;
    if (!(p->mass > 0.0f) || !(p->smoothing_coeff > 0.0f) || !(p->particle_radius > 0.0f) ||
        !(p->resting_rho > 0.0f) || !(p->dt > 0.0f) || p->cell_scale < 0.0f)
        return SPH_ERR_INVALID_ARG;
    float h = smoothing_length(*p);
    if (!(h > 0.0f) || !std::isfinite(h * h * h)) return SPH_ERR_INVALID_ARG;
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(p->lower[a]) || !std::isfinite(p->upper[a]) || !(p->lower[a] < p->upper[a]))
            return SPH_ERR_INVALID_ARG;
    if (p->flags & ~SPH_FLAG_KEEP_FORCE) return SPH_ERR_INVALID_ARG;
    if (p->reserved[0] || p->reserved[1] || p->reserved[2]) return SPH_ERR_INVALID_ARG;
    int dims[3];
    if (!grid_dims(*p, 2, nullptr, dims)) return SPH_ERR_INVALID_ARG;  // also fits at stencil 2
    return SPH_OK;
}

float sph_cutoff_d2(float h) { return cutoff_d2(h); }

sph_status sph_grid_dims(const sph_params* p, float* edge, int32_t dims[3]) {
    if (!p || !dims) return SPH_ERR_INVALID_ARG;
    int d[3];
    if (!grid_dims(*p, 1, edge, d)) return SPH_ERR_INVALID_ARG;
    for (int a = 0; a < 3; ++a) dims[a] = d[a];
    return SPH_OK;
}

sph_status sph_scene_reference_grid(sph_particle* out, uint32_t n, float spacing) {
    if (!out || n != 10000u || !(spacing > 0.0f)) return SPH_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(sph_particle) * n);
    uint32_t idx = 0;
    for (int i = 0; i < 10; ++i)            // Main.cpp:493-503: i (x), j (y), k (z) loops
        for (int j = 0; j < 100; ++j)
            for (int k = 0; k < 10; ++k) {
                sph_particle& r = out[idx++];
                r.pos[0] = (float)i * spacing;
                r.pos[1] = (float)j * spacing;
                r.pos[2] = (float)k * spacing;
                r.pos[3] = 1.0f;
            }
    return SPH_OK;
}

sph_status sph_scene_fill(sph_particle* out, uint32_t n, const float lo[3], const float hi[3], float spacing,
                          float jitter, uint64_t seed) {
    if (!out || !lo || !hi || !(spacing > 0.0f) || !(jitter >= 0.0f)) return SPH_ERR_INVALID_ARG;
    long long cnt[3];
    for (int a = 0; a < 3; ++a) {
        double ext = (double)hi[a] - (double)lo[a];
        cnt[a] = ext > 0 ? (long long)std::floor(ext / (double)spacing + 1e-6) : 0;
    }
    if ((long double)cnt[0] * cnt[1] * cnt[2] < (long double)n) return SPH_ERR_CAPACITY;
    std::memset(out, 0, sizeof(sph_particle) * n);
    for (uint32_t idx = 0; idx < n; ++idx) {
        long long ix = idx % cnt[0], iz = (idx / cnt[0]) % cnt[2], iy = idx / (cnt[0] * cnt[2]);
        long long ic[3] = {ix, iy, iz};
        sph_particle& r = out[idx];
        for (int a = 0; a < 3; ++a)
            r.pos[a] = (float)((double)lo[a] + ((double)ic[a] + 0.5) * spacing +
                               jitter * unit_pm(seed, 3ull * idx + a));
        r.pos[3] = 1.0f;
    }
    return SPH_OK;
}

sph_status sph_scene_ball(sph_particle* out, uint32_t n, const float center[3], float spacing, float jitter,
                          uint64_t seed) {
    if (!out || !center || !(spacing > 0.0f) || !(jitter >= 0.0f) || n == 0) return SPH_ERR_INVALID_ARG;
    int R = (int)std::ceil(std::cbrt(3.0 * n / (4.0 * M_PI))) + 2;
    struct Pt { long long d2; int i, j, k; };
    std::vector<Pt> pts;
    pts.reserve((size_t)(2 * R) * (2 * R) * (2 * R));
    for (int k = -R; k < R; ++k)
        for (int j = -R; j < R; ++j)
            for (int i = -R; i < R; ++i) {
                long long a = 2 * i + 1, b = 2 * j + 1, c = 2 * k + 1;  // offsets in half-spacings
                pts.push_back({a * a + b * b + c * c, i, j, k});
            }
    if (pts.size() < n) return SPH_ERR_CAPACITY;
    std::stable_sort(pts.begin(), pts.end(), [](const Pt& x, const Pt& y) { return x.d2 < y.d2; });
    std::memset(out, 0, sizeof(sph_particle) * n);
    for (uint32_t idx = 0; idx < n; ++idx) {
        const Pt& q = pts[idx];
        int ic[3] = {q.i, q.j, q.k};
        sph_particle& r = out[idx];
        for (int a = 0; a < 3; ++a)
            r.pos[a] = (float)((double)center[a] + ((double)ic[a] + 0.5) * spacing +
                               jitter * unit_pm(seed, 3ull * idx + a));
        r.pos[3] = 1.0f;
    }
    return SPH_OK;
}

sph_status sph_scene_slosh(sph_particle* out, uint32_t n, float amplitude, float x0, float length) {
    if (!out || !(length > 0.0f)) return SPH_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; ++i)
        out[i].vel[0] += (float)(amplitude * std::sin(M_PI * ((double)out[i].pos[0] - x0) / length));
    return SPH_OK;
}

}  // extern "C"

// ---- views for sph_render ----------------------------------------------------------------
// Column-major 4x4 matrices as glm stores them: m[4 * column + row]. The formulas are the
// standard OpenGL ones (glm::rotate, glm::scale, glm::lookAt, glm::perspective), computed in
// FP64 and rounded once.
namespace {

void mat_mul(const double* a, const double* b, double* out) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += a[4 * k + r] * b[4 * c + k];
            out[4 * c + r] = s;
        }
}

// M = rotate(angle, (0, 1, 0)) * scale(s, s, s) (Main.cpp:256)
void model_matrix(double angle, double s, double* m) {
    const double c = std::cos(angle), sn = std::sin(angle);
    double rot[16] = {c, 0, -sn, 0, 0, 1, 0, 0, sn, 0, c, 0, 0, 0, 0, 1};
    double sc[16] = {s, 0, 0, 0, 0, s, 0, 0, 0, 0, s, 0, 0, 0, 0, 1};
    mat_mul(rot, sc, m);
}

// V = lookAt(eye, center, up = (0, 1, 0)) (Main.cpp:257), right-handed
void view_matrix(const double* eye, const double* center, double* v) {
    double f[3] = {center[0] - eye[0], center[1] - eye[1], center[2] - eye[2]};
    const double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& x : f) x /= fl;
    const double up[3] = {0.0, 1.0, 0.0};
    double s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    const double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    for (double& x : s) x /= sl;
    const double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    std::memset(v, 0, 16 * sizeof(double));
    for (int k = 0; k < 3; ++k) {
        v[4 * k + 0] = s[k];
        v[4 * k + 1] = u[k];
        v[4 * k + 2] = -f[k];
    }
    v[12] = -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2]);
    v[13] = -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]);
    v[14] = f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2];
    v[15] = 1.0;
}

// P = perspective(fovy, aspect, near, far) (Main.cpp:258), clip depth -1..1
void proj_matrix(double fovy, double aspect, double zn, double zf, double* p) {
    const double t = std::tan(fovy / 2.0);
    std::memset(p, 0, 16 * sizeof(double));
    p[0] = 1.0 / (aspect * t);
    p[5] = 1.0 / t;
    p[10] = -(zf + zn) / (zf - zn);
    p[11] = -1.0;
    p[14] = -(2.0 * zf * zn) / (zf - zn);
}

void put(float* dst, const double* src) {
    for (int i = 0; i < 16; ++i) dst[i] = (float)src[i];
}

void set4(float* d, float a, float b, float c, float w) {
    d[0] = a;
    d[1] = b;
    d[2] = c;
    d[3] = w;
}

}  // namespace

extern "C" {

sph_status sph_view_camera(sph_view* v, float angle, float scale, const float eye[3], const float center[3]) {
    if (!v || !eye || !center || v->width <= 0 || v->height <= 0) return SPH_ERR_INVALID_ARG;
    const double e[3] = {eye[0], eye[1], eye[2]}, c[3] = {center[0], center[1], center[2]};
    if (e[0] == c[0] && e[1] == c[1] && e[2] == c[2]) return SPH_ERR_INVALID_ARG;
    double m[16], vw[16], pr[16];
    model_matrix(angle, scale, m);
    view_matrix(e, c, vw);
    proj_matrix(M_PI / 4.0, (double)v->width / (double)v->height, 0.1, 100.0, pr);
    put(v->model, m);
    put(v->view, vw);
    put(v->proj, pr);
    set4(v->eye_w, eye[0], eye[1], eye[2], 1.0f);
    return SPH_OK;
}

sph_status sph_view_default(sph_view* v, int32_t width, int32_t height, float model_scale) {
    if (!v || width <= 0 || height <= 0 || !(model_scale > 0.0f)) return SPH_ERR_INVALID_ARG;
    std::memset(v, 0, sizeof(*v));
    v->width = width;
    v->height = height;
    const float eye[3] = {10.0f, 2.0f, 0.0f}, center[3] = {0.0f, 0.0f, 0.0f};  // Main.cpp:89, :105
    sph_status st = sph_view_camera(v, 0.75f, 2.5f * model_scale, eye, center);  // Main.cpp:82-83
    if (st) return st;
    set4(v->light_w, 0.0f, 1.0f, 1.0f, 1.0f);        // Main.cpp:106
    set4(v->dark, 0.0f, 0.0f, 0.0f, 1.0f);           // Main.cpp:127-130
    set4(v->midtone, 0.5f, 0.5f, 0.5f, 1.0f);
    set4(v->highlight, 1.0f, 1.0f, 1.0f, 1.0f);
    set4(v->outline, 0.0f, 0.0f, 0.0f, 1.0f);
    set4(v->clear_color, 0.5f, 0.5f, 0.5f, 1.0f);    // Main.cpp:80
    v->shininess = 0.3f;                             // Main.cpp:131
    v->point_size = 10.0f;                           // simulation_radius, Main.cpp:88
    return SPH_OK;
}

sph_status sph_image_write_ppm(const char* path, const uint8_t* rgba, int32_t width, int32_t height) {
    if (!path || !rgba || width <= 0 || height <= 0) return SPH_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return SPH_ERR_INVALID_ARG;
    std::fprintf(f, "P6\n%d %d\n255\n", width, height);
    std::vector<unsigned char> row((size_t)width * 3);
    bool ok = true;
    for (int y = height - 1; y >= 0 && ok; --y) {  // GL rows are bottom to top
        const uint8_t* src = rgba + (size_t)y * width * 4;
        for (int x = 0; x < width; ++x)
            for (int k = 0; k < 3; ++k) row[(size_t)3 * x + k] = src[(size_t)4 * x + k];
        ok = std::fwrite(row.data(), 1, row.size(), f) == row.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? SPH_OK : SPH_ERR_INVALID_ARG;
}

}  // extern "C"

// ---- Wavefront OBJ reader (the mesh input of sph_sdf_from_mesh) ---------------------------
// Reads `v x y z` and `f i j k ...` lines; a face vertex is "a", "a/b", "a/b/c" or "a//c"
// (1-based, negative = counted back from the last vertex read so far); a polygon with m
// vertices becomes the m - 2 triangles (v0, v_k, v_k+1). Other lines are skipped.
extern "C" sph_status sph_obj_read(const char* path, float* verts, uint32_t* nv, uint32_t* tris, uint32_t* nt) {
    if (!path || !nv || !nt) return SPH_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return SPH_ERR_INVALID_ARG;
    std::vector<float> v;
    std::vector<uint32_t> t;
    sph_status st = SPH_OK;
    char line[4096];
    std::vector<long long> poly;
    while (st == SPH_OK && std::fgets(line, sizeof line, f)) {
        const char* s = line;
        while (*s == ' ' || *s == '\t') ++s;
        if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
            float x, y, z;
            if (std::sscanf(s + 2, "%f %f %f", &x, &y, &z) != 3) { st = SPH_ERR_INVALID_ARG; break; }
            v.push_back(x); v.push_back(y); v.push_back(z);
        } else if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
            poly.clear();
            const char* q = s + 2;
            const long long nvert = (long long)(v.size() / 3);
            while (true) {
                while (*q == ' ' || *q == '\t') ++q;
                if (*q == '\0' || *q == '\n' || *q == '\r' || *q == '#') break;
                char* end = nullptr;
                const long long idx = std::strtoll(q, &end, 10);
                if (end == q) { st = SPH_ERR_INVALID_ARG; break; }
                const long long k = idx > 0 ? idx - 1 : nvert + idx;  // idx == 0 is invalid
                if (idx == 0 || k < 0 || k >= nvert) { st = SPH_ERR_INVALID_ARG; break; }
                poly.push_back(k);
                q = end;
                while (*q && *q != ' ' && *q != '\t' && *q != '\n' && *q != '\r') ++q;  // skip /vt/vn
            }
            if (st == SPH_OK && poly.size() < 3) st = SPH_ERR_INVALID_ARG;
            for (size_t k = 1; st == SPH_OK && k + 1 < poly.size(); ++k) {
                t.push_back((uint32_t)poly[0]);
                t.push_back((uint32_t)poly[k]);
                t.push_back((uint32_t)poly[k + 1]);
            }
        }
    }
    std::fclose(f);
    if (st != SPH_OK) return st;
    const uint32_t cv = (uint32_t)(v.size() / 3), ct = (uint32_t)(t.size() / 3);
    const uint32_t cap_v = *nv, cap_t = *nt;
    *nv = cv;
    *nt = ct;
    if (!verts || !tris) return SPH_OK;
    if (cap_v < cv || cap_t < ct) return SPH_ERR_CAPACITY;
    std::memcpy(verts, v.data(), sizeof(float) * v.size());
    std::memcpy(tris, t.data(), sizeof(uint32_t) * t.size());
    return SPH_OK;
}
