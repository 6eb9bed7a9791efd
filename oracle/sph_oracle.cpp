// sph_oracle.cpp -- CPU restatement of the reference SPH step. TEST INFRASTRUCTURE ONLY.
//
// This file is the correctness oracle and the timed CPU baseline of the GB300
// SPH step. Only tests/, the smoke check of __graft_entry__ and the CPU legs
// of bench.py load it; the product library never links or calls it.
//
// It restates the three GLSL compute shaders of NPR-SPH:
//   rho_pres_comp.glsl:35-59  density (poly6, self included, strict r<h) + EOS p=max(k(rho-rho0),0)
//   force_comp.glsl:35-67     spiky pressure + Laplacian viscosity over j!=i, r<h; *mu; + rho_i*G
//   integrate_comp.glsl:35-82 a=F/rho; v+=dt*a; x+=dt*v; per-axis if/else-if wall clamp, v*=-damping
// Constants come from Main.cpp:110-122 and the shader #defines, all carried in
// sph_params (include/sph_gb300.h).
//
// Two instances:
//   oracle_step_f64      FP64 arithmetic (the oracle). The neighbour predicate is the
//                        FP32 expression below on the FP32-rounded positions, so that
//                        neighbour sets are the ones the FP32 GPU step sees.
//   oracle_step_f32_aos  FP32 literal mirror of the shader arithmetic, operation by
//                        operation, on the 64-byte AoS record; it is checked bit-exact
//                        against the shader source compiled as C++ (oracle/ref_shader).
// Two neighbour back-ends: brute force (the reference's O(N^2) j-loops,
// rho_pres_comp.glsl:46 / force_comp.glsl:48) and a uniform grid of cell edge >= h.
//
// Documented divergence from the shader: for i != j at r == 0, normalize(delta)
// (force_comp.glsl:59) is 0/0 = NaN in the shader. Here (and on the GPU) the
// pressure term of such a pair is skipped; the viscosity term is kept.
// oracle_step_f32_aos(..., literal_nan=1) reproduces the shader's NaN instead.
//
// Build: make -C oracle  (g++ -O2 -fopenmp -ffp-contract=off; no fast-math, so
// FP32 results are the same on x86-64 and aarch64).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

#include "../include/sph_gb300.h"

namespace {

// The shaders' PI (rho_pres_comp.glsl:8).
constexpr float kPiF = 3.141592741f;

// ---- canonical FP32 neighbour predicate -------------------------------------
// rho_pres_comp.glsl:48-50: delta = pos_i - pos_j; r = length(delta); r < h.
// length() = sqrt(dot(delta, delta)) with dot = (x*x + y*y) + z*z, evaluated in
// FP32 without contraction (this file is compiled with -ffp-contract=off).
inline float canon_d2(float xi, float yi, float zi, float xj, float yj, float zj) {
    float dx = xi - xj, dy = yi - yj, dz = zi - zj;
    float a = dx * dx;
    float b = dy * dy;
    float c = dz * dz;
    return (a + b) + c;
}
inline bool canon_pred(float d2, float h) { return std::sqrt(d2) < h; }

inline uint64_t mix64(uint64_t z) {
    // splitmix64 finaliser of (z + golden gamma); the neighbour digest term.
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// ---- uniform grid (neighbour back-end) -----------------------------------------
// Cell edge >= h (times 1 + 2^-10), so every pair with r < h lies in the same or
// an adjacent cell; coordinates clamp into the box, which only shrinks distances.
struct Grid {
    float lo[3], inv_edge;
    int dim[3];
    std::vector<int64_t> start;  // ncells + 1
    std::vector<int64_t> items;  // particle indices, by cell
    int cell_coord(float x, int a) const {
        float t = (x - lo[a]) * inv_edge;
        int c = (int)std::floor(t);
        if (!(t == t)) c = 0;  // NaN position: put it in cell 0
        return c < 0 ? 0 : (c >= dim[a] ? dim[a] - 1 : c);
    }
    int64_t key(int cx, int cy, int cz) const {
        return (int64_t)cx + (int64_t)dim[0] * ((int64_t)cy + (int64_t)dim[1] * cz);
    }
};

float grid_edge(const sph_params* P, float h) {
    float s = P->cell_scale;
    const float smin = 1.0f + 1.0f / 1024.0f;
    if (!(s >= smin)) s = smin;
    return h * s;
}

template <class GetPos>
void build_grid(Grid& g, const sph_params* P, float h, int64_t n, GetPos getpos) {
    float edge = grid_edge(P, h);
    g.inv_edge = 1.0f / edge;
    for (int a = 0; a < 3; ++a) {
        g.lo[a] = P->lower[a];
        double ext = (double)P->upper[a] - (double)P->lower[a];
        int d = (int)std::ceil(ext / (double)edge);
        g.dim[a] = d < 1 ? 1 : d;
    }
    int64_t ncell = (int64_t)g.dim[0] * g.dim[1] * g.dim[2];
    g.start.assign(ncell + 1, 0);
    std::vector<int64_t> key(n);
    for (int64_t i = 0; i < n; ++i) {
        float p[3];
        getpos(i, p);
        key[i] = g.key(g.cell_coord(p[0], 0), g.cell_coord(p[1], 1), g.cell_coord(p[2], 2));
        g.start[key[i] + 1]++;
    }
    for (int64_t c = 0; c < ncell; ++c) g.start[c + 1] += g.start[c];
    std::vector<int64_t> fill(g.start.begin(), g.start.end() - 1);
    g.items.resize(n);
    for (int64_t i = 0; i < n; ++i) g.items[fill[key[i]]++] = i;  // stable: ascending i per cell
}

// Visit every candidate j of particle i (brute force: all j; grid: 27 cells).
template <class GetPos, class Fn>
inline void for_candidates(const Grid* g, int64_t n, int64_t i, GetPos getpos, Fn fn) {
    if (!g) {
        for (int64_t j = 0; j < n; ++j) fn(j);
        return;
    }
    float p[3];
    getpos(i, p);
    int cx = g->cell_coord(p[0], 0), cy = g->cell_coord(p[1], 1), cz = g->cell_coord(p[2], 2);
    for (int z = cz - 1; z <= cz + 1; ++z) {
        if (z < 0 || z >= g->dim[2]) continue;
        for (int y = cy - 1; y <= cy + 1; ++y) {
            if (y < 0 || y >= g->dim[1]) continue;
            int x0 = cx > 0 ? cx - 1 : 0, x1 = cx + 1 < g->dim[0] ? cx + 1 : g->dim[0] - 1;
            int64_t k0 = g->key(x0, y, z), k1 = g->key(x1, y, z);
            for (int64_t t = g->start[k0]; t < g->start[k1 + 1]; ++t) fn(g->items[t]);
        }
    }
}

// ---- GLSL-like FP32 helpers for the literal mirror ----------------------------------
struct v3 { float x, y, z; };
inline v3 operator-(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline v3 operator+(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline v3 operator*(float s, v3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline v3 operator*(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline v3 operator/(v3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float glsl_length(v3 a) { return std::sqrt((a.x * a.x + a.y * a.y) + a.z * a.z); }
inline v3 glsl_normalize(v3 a) { return a / glsl_length(a); }
inline float glsl_max(float x, float y) { return x < y ? y : x; }
inline v3 ld3(const float* f) { return {f[0], f[1], f[2]}; }
inline void st3(float* f, v3 a) { f[0] = a.x; f[1] = a.y; f[2] = a.z; }

}  // namespace

extern "C" {

float oracle_cutoff_d2(float h) {
    // Smallest float T with sqrtf(T) >= h; sqrtf is monotone, so d2 < T <=> sqrtf(d2) < h.
    float t = h * h;
    while (t > 0.0f && std::sqrt(std::nextafter(t, 0.0f)) >= h) t = std::nextafter(t, 0.0f);
    while (std::sqrt(t) < h) t = std::nextafter(t, INFINITY);
    return t;
}

uint64_t oracle_mix64(uint64_t j) { return mix64(j); }

// One FP64 step from the state (pos, vel), all arrays n*3 (xyz) except the
// per-particle scalars. Outputs may be NULL except rho/pres/pos_out/vel_out.
//   fscale[i]      = sum_j |f_ij(pressure)| + mu*|f_ij(viscosity)| + rho_i*|G|, the
//                    scale of the force error metric (pressure terms cancel inside).
//   wall_margin[i] = distance of the unclamped new position to the nearest wall plane.
//   backend: 0 brute force, 1 grid.
//   rho_given: 0 computes rho/pres (pass 1); 1 takes them as inputs and runs the force and
//              integrate passes only (the check of a force pass fed the same densities).
static int step_f64_impl(const sph_params* P, int64_t n, const double* pos, const double* vel,
                         int backend, int nthreads, double* rho, double* pres, double* force,
                         double* fscale, double* pos_out, double* vel_out, double* wall_margin,
                         int rho_given) {
    if (!P || n < 0 || !pos || !vel || !rho || !pres || !pos_out || !vel_out) return -1;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    const float hf = P->smoothing_coeff * P->particle_radius;  // rho_pres_comp.glsl:40 (FP32)
    const double h = hf, m = P->mass, PI = kPiF, mu = P->visc, rho0 = P->resting_rho;
    const double k = P->gas_const, dt = P->dt, damp = P->damping;
    const double G[3] = {P->gravity[0], P->gravity[1], P->gravity[2]};
    const double poly6 = 64.0 * PI * std::pow(h, 9);  // rho_pres_comp.glsl:52 denominator
    const double spiky = -45.0 / (PI * std::pow(h, 6));  // force_comp.glsl:41
    const double lap = 45.0 / (PI * std::pow(h, 6));     // force_comp.glsl:42

    std::vector<float> pf(3 * n);
    for (int64_t t = 0; t < 3 * n; ++t) pf[t] = (float)pos[t];
    auto getpos = [&](int64_t i, float* p) { p[0] = pf[3 * i]; p[1] = pf[3 * i + 1]; p[2] = pf[3 * i + 2]; };
    Grid grid;
    const Grid* g = nullptr;
    if (backend == 1) { build_grid(grid, P, hf, n, getpos); g = &grid; }

    // Pass 1: density + pressure (rho_pres_comp.glsl:43-58).
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
    for (int64_t i = 0; i < (rho_given ? 0 : n); ++i) {
        double r_acc = 0.0;
        for_candidates(g, n, i, getpos, [&](int64_t j) {
            float d2f = canon_d2(pf[3*i], pf[3*i+1], pf[3*i+2], pf[3*j], pf[3*j+1], pf[3*j+2]);
            if (!canon_pred(d2f, hf)) return;  // :50, strict r < h
            double dx = pos[3*i] - pos[3*j], dy = pos[3*i+1] - pos[3*j+1], dz = pos[3*i+2] - pos[3*j+2];
            double r = std::sqrt(dx * dx + dy * dy + dz * dz);
            double w = h * h - r * r;
            r_acc += m * 315.0 * (w * w * w) / poly6;  // :52 (j == i included)
        });
        rho[i] = r_acc;                                  // :55
        double pp = k * (r_acc - rho0);
        pres[i] = pp < 0.0 ? 0.0 : pp;                   // :58
    }

    // Pass 2 + 3: force (force_comp.glsl:43-66), integrate (integrate_comp.glsl:41-77).
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        double fp[3] = {0, 0, 0}, fv[3] = {0, 0, 0}, scale = 0.0;
        for_candidates(g, n, i, getpos, [&](int64_t j) {
            if (j == i) return;  // force_comp.glsl:50-53
            float d2f = canon_d2(pf[3*i], pf[3*i+1], pf[3*i+2], pf[3*j], pf[3*j+1], pf[3*j+2]);
            if (!canon_pred(d2f, hf)) return;  // :57
            double d[3] = {pos[3*i] - pos[3*j], pos[3*i+1] - pos[3*j+1], pos[3*i+2] - pos[3*j+2]};
            double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double hr = h - r;
            if (r > 0.0) {  // divergence: skip the undefined normalize(0)
                double s = m * (pres[i] + pres[j]) / (2.0 * rho[j]) * spiky * hr * hr / r;  // :59
                for (int a = 0; a < 3; ++a) fp[a] -= s * d[a];
                scale += std::fabs(s) * r;
            }
            double c = m / rho[j] * lap * hr;  // :60
            double vn = 0.0;
            for (int a = 0; a < 3; ++a) {
                double dv = vel[3*j+a] - vel[3*i+a];
                fv[a] += c * dv;
                vn += dv * dv;
            }
            scale += mu * std::fabs(c) * std::sqrt(vn);
        });
        double F[3], gnorm = 0.0;
        for (int a = 0; a < 3; ++a) {
            F[a] = fp[a] + fv[a] * mu + rho[i] * G[a];  // :63-66
            gnorm += G[a] * G[a];
        }
        scale += rho[i] * std::sqrt(gnorm);
        if (force) for (int a = 0; a < 3; ++a) force[3*i+a] = F[a];
        if (fscale) fscale[i] = scale;
        // integrate_comp.glsl:41-77
        double margin = INFINITY;
        for (int a = 0; a < 3; ++a) {
            double acc = F[a] / rho[i];
            double nv = vel[3*i+a] + dt * acc;
            double np = pos[3*i+a] + dt * nv;
            margin = std::min(margin, std::min(std::fabs(np - (double)P->lower[a]),
                                               std::fabs(np - (double)P->upper[a])));
            if (np < (double)P->lower[a]) { np = P->lower[a]; nv *= -damp; }
            else if (np > (double)P->upper[a]) { np = P->upper[a]; nv *= -damp; }
            pos_out[3*i+a] = np;
            vel_out[3*i+a] = nv;
        }
        if (wall_margin) wall_margin[i] = margin;
    }
    return 0;
}

int oracle_step_f64(const sph_params* P, int64_t n, const double* pos, const double* vel,
                    int backend, int nthreads, double* rho, double* pres, double* force,
                    double* fscale, double* pos_out, double* vel_out, double* wall_margin) {
    return step_f64_impl(P, n, pos, vel, backend, nthreads, rho, pres, force, fscale, pos_out, vel_out,
                         wall_margin, 0);
}

// Force + integrate passes (force_comp.glsl, integrate_comp.glsl) from given rho/pres.
int oracle_force_f64(const sph_params* P, int64_t n, const double* pos, const double* vel,
                     const double* rho, const double* pres, int backend, int nthreads, double* force,
                     double* fscale, double* pos_out, double* vel_out, double* wall_margin) {
    return step_f64_impl(P, n, pos, vel, backend, nthreads, const_cast<double*>(rho),
                         const_cast<double*>(pres), force, fscale, pos_out, vel_out, wall_margin, 1);
}

// Conditioning of the force pass: fcond[i] = sum_j |f_ij(p)| * 2r/(h-r) + mu*|f_ij(v)| * r/(h-r),
// the first-order change of F_i under a relative perturbation of every pair distance r
// (d ln (h-r)^2 / d ln r = -2r/(h-r); d ln (h-r) / d ln r = -r/(h-r)). Any FP32 evaluation of
// force_comp.glsl:59-60 from FP32 positions (the shader itself included) rounds r by a few
// 2^-24, so its force error is bounded by a few 2^-24 * fcond on top of the usual scale.
int oracle_force_cond_f64(const sph_params* P, int64_t n, const double* pos, const double* vel,
                          const double* rho, const double* pres, int backend, int nthreads, double* fcond) {
    if (!P || n < 0 || !pos || !vel || !rho || !pres || !fcond) return -1;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    const float hf = P->smoothing_coeff * P->particle_radius;
    const double h = hf, m = P->mass, PI = kPiF, mu = P->visc;
    const double lap = 45.0 / (PI * std::pow(h, 6));
    std::vector<float> pf(3 * n);
    for (int64_t t = 0; t < 3 * n; ++t) pf[t] = (float)pos[t];
    auto getpos = [&](int64_t i, float* p) { p[0] = pf[3 * i]; p[1] = pf[3 * i + 1]; p[2] = pf[3 * i + 2]; };
    Grid grid;
    const Grid* g = nullptr;
    if (backend == 1) { build_grid(grid, P, hf, n, getpos); g = &grid; }
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        double cond = 0.0;
        for_candidates(g, n, i, getpos, [&](int64_t j) {
            if (j == i) return;
            float d2f = canon_d2(pf[3*i], pf[3*i+1], pf[3*i+2], pf[3*j], pf[3*j+1], pf[3*j+2]);
            if (!canon_pred(d2f, hf)) return;
            double d[3] = {pos[3*i] - pos[3*j], pos[3*i+1] - pos[3*j+1], pos[3*i+2] - pos[3*j+2]};
            double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double hr = h - r;
            if (!(hr > 0.0)) hr = 1e-300;
            double fp = std::fabs(m * (pres[i] + pres[j]) / (2.0 * rho[j]) * lap * hr * hr);
            double vn = 0.0;
            for (int a = 0; a < 3; ++a) { double dv = vel[3*j+a] - vel[3*i+a]; vn += dv * dv; }
            double fv = mu * std::fabs(m / rho[j] * lap * hr) * std::sqrt(vn);
            cond += fp * 2.0 * r / hr + fv * r / hr;
        });
        fcond[i] = cond;
    }
    return 0;
}

// n_steps FP64 steps in place (state in double). The CPU baseline.
int oracle_run_f64(const sph_params* P, int64_t n, double* pos, double* vel, double* rho,
                   double* pres, int n_steps, int backend, int nthreads) {
    std::vector<double> po(3 * n), vo(3 * n);
    for (int s = 0; s < n_steps; ++s) {
        int rc = oracle_step_f64(P, n, pos, vel, backend, nthreads, rho, pres, nullptr, nullptr,
                                 po.data(), vo.data(), nullptr);
        if (rc) return rc;
        std::memcpy(pos, po.data(), sizeof(double) * 3 * n);
        std::memcpy(vel, vo.data(), sizeof(double) * 3 * n);
    }
    return 0;
}

// FP32 literal mirror: n_steps steps in place on the 64-byte records, three full
// passes per step as in Main.cpp:295-303. Every expression keeps the shader's
// operation order (rho_pres_comp.glsl:52, force_comp.glsl:59-66,
// integrate_comp.glsl:41-77). literal_nan = 1 keeps normalize(0) = NaN.
int oracle_step_f32_aos(const sph_params* P, sph_particle* pa, int64_t n, int n_steps,
                        int backend, int nthreads, int literal_nan) {
    if (!P || !pa || n < 0) return -1;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    const float h = P->smoothing_coeff * P->particle_radius;
    const float mass = P->mass, visc = P->visc, rho0 = P->resting_rho, K = P->gas_const;
    const float dt = P->dt, D = P->damping;
    const v3 G = {P->gravity[0], P->gravity[1], P->gravity[2]};
    auto getpos = [&](int64_t i, float* p) { p[0] = pa[i].pos[0]; p[1] = pa[i].pos[1]; p[2] = pa[i].pos[2]; };
    for (int s = 0; s < n_steps; ++s) {
        Grid grid;
        const Grid* g = nullptr;
        if (backend == 1) { build_grid(grid, P, h, n, getpos); g = &grid; }
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
        for (int64_t i = 0; i < n; ++i) {
            float rho = 0.0f;
            for_candidates(g, n, i, getpos, [&](int64_t j) {
                v3 delta = ld3(pa[i].pos) - ld3(pa[j].pos);
                float r = glsl_length(delta);
                if (r < h)
                    rho += mass * 315.0f * std::pow(h * h - r * r, 3.0f) /
                           (64.0f * kPiF * std::pow(h, 9.0f));
            });
            pa[i].extras[0] = rho;
            pa[i].extras[1] = glsl_max(K * (rho - rho0), 0.0f);
        }
        const float spiky = -45.0f / (kPiF * std::pow(h, 6.0f));
        const float laplacian = 45.0f / (kPiF * std::pow(h, 6.0f));
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
        for (int64_t i = 0; i < n; ++i) {
            v3 pf = {0, 0, 0}, vf = {0, 0, 0};
            for_candidates(g, n, i, getpos, [&](int64_t j) {
                if (i == j) return;
                v3 delta = ld3(pa[i].pos) - ld3(pa[j].pos);
                float r = glsl_length(delta);
                if (r < h) {
                    if (r > 0.0f || literal_nan) {
                        float s = mass * (pa[i].extras[1] + pa[j].extras[1]) / (2.0f * pa[j].extras[0]) *
                                  spiky * std::pow(h - r, 2.0f);
                        pf = pf - s * glsl_normalize(delta);
                    }
                    vf = vf + mass * (ld3(pa[j].vel) - ld3(pa[i].vel)) / pa[j].extras[0] * laplacian * (h - r);
                }
            });
            vf = vf * visc;
            v3 gf = pa[i].extras[0] * G;
            st3(pa[i].force, (pf + vf) + gf);
        }
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int64_t i = 0; i < n; ++i) {
            v3 acc = ld3(pa[i].force) / pa[i].extras[0];
            v3 nv = ld3(pa[i].vel) + dt * acc;
            v3 np = ld3(pa[i].pos) + dt * nv;
            float* pp = &np.x;
            float* vv = &nv.x;
            for (int a = 0; a < 3; ++a) {
                if (pp[a] < P->lower[a]) { pp[a] = P->lower[a]; vv[a] *= -D; }
                else if (pp[a] > P->upper[a]) { pp[a] = P->upper[a]; vv[a] *= -D; }
            }
            st3(pa[i].vel, nv);
            st3(pa[i].pos, np);
        }
    }
    return 0;
}

// Neighbour sets of the query particles: count and order-independent digest
// sum_j mix64(j) over {j : length(x_i - x_j) < h} (self included).
int oracle_neighbors(const sph_params* P, int64_t n, const float* pos4, int64_t nq,
                     const int64_t* query, int backend, int nthreads, uint32_t* count,
                     uint64_t* digest) {
    if (!P || !pos4 || !query || !count || !digest) return -1;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    const float h = P->smoothing_coeff * P->particle_radius;
    auto getpos = [&](int64_t i, float* p) { p[0] = pos4[4*i]; p[1] = pos4[4*i+1]; p[2] = pos4[4*i+2]; };
    Grid grid;
    const Grid* g = nullptr;
    if (backend == 1) { build_grid(grid, P, h, n, getpos); g = &grid; }
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (int64_t q = 0; q < nq; ++q) {
        int64_t i = query[q];
        uint32_t c = 0;
        uint64_t d = 0;
        for_candidates(g, n, i, getpos, [&](int64_t j) {
            float d2 = canon_d2(pos4[4*i], pos4[4*i+1], pos4[4*i+2], pos4[4*j], pos4[4*j+1], pos4[4*j+2]);
            if (canon_pred(d2, h)) { ++c; d += mix64((uint64_t)j); }
        });
        count[q] = c;
        digest[q] = d;
    }
    return 0;
}

// Full neighbour lists (CSR) for small cases: offsets[n+1], and up to cap
// indices, ascending per particle. Returns the total count (may exceed cap).
int64_t oracle_neighbor_lists(const sph_params* P, int64_t n, const float* pos4, int backend,
                              int64_t* offsets, int64_t* items, int64_t cap) {
    const float h = P->smoothing_coeff * P->particle_radius;
    auto getpos = [&](int64_t i, float* p) { p[0] = pos4[4*i]; p[1] = pos4[4*i+1]; p[2] = pos4[4*i+2]; };
    Grid grid;
    const Grid* g = nullptr;
    if (backend == 1) { build_grid(grid, P, h, n, getpos); g = &grid; }
    int64_t total = 0;
    std::vector<int64_t> tmp;
    for (int64_t i = 0; i < n; ++i) {
        offsets[i] = total;
        tmp.clear();
        for_candidates(g, n, i, getpos, [&](int64_t j) {
            float d2 = canon_d2(pos4[4*i], pos4[4*i+1], pos4[4*i+2], pos4[4*j], pos4[4*j+1], pos4[4*j+2]);
            if (canon_pred(d2, h)) tmp.push_back(j);
        });
        std::sort(tmp.begin(), tmp.end());
        for (int64_t j : tmp) { if (total < cap) items[total] = j; ++total; }
    }
    offsets[n] = total;
    return total;
}

// Static obstacle rule of the library (sph_set_obstacle; no reference counterpart), in FP64,
// applied to states that already went through the wall clamp: phi = trilinear interpolation of
// the samples (sample (i, j, k) at origin + spacing (i, j, k), x fastest; none outside the
// sampled box); where phi < 0: x -= phi n, n = g / |g| with g the trilinear interpolant of the
// samples' central-difference gradients;
// v -= (1 + damping)(v.n) n if v.n < 0; then x is clamped into [lower, upper]. phi_out[i]
// receives phi at the input position (NaN outside the sampled box).
int oracle_obstacle_f64(const sph_params* P, const float* sdf, const int32_t* dims, const double* origin,
                        double spacing, int64_t n, double* pos, double* vel, double* phi_out) {
    if (!P || !sdf || !dims || !origin || !pos || !vel || !(spacing > 0.0)) return -1;
    const double inv = 1.0 / spacing, damp = P->damping;
    const int64_t sy = dims[0], sz = (int64_t)dims[0] * dims[1];
    for (int64_t q = 0; q < n; ++q) {
        double* x = pos + 3 * q;
        double* v = vel + 3 * q;
        const double u[3] = {(x[0] - origin[0]) * inv, (x[1] - origin[1]) * inv, (x[2] - origin[2]) * inv};
        bool in = true;
        for (int a = 0; a < 3; ++a) in = in && u[a] >= 0.0 && u[a] <= (double)(dims[a] - 1);
        if (phi_out) phi_out[q] = NAN;
        if (!in) continue;
        int c[3];
        double t[3];
        for (int a = 0; a < 3; ++a) {
            c[a] = std::min((int)std::floor(u[a]), dims[a] - 2);
            t[a] = u[a] - c[a];
        }
        auto S = [&](const int* q) { return (double)sdf[q[2] * sz + q[1] * sy + q[0]]; };
        // phi: the trilinear interpolant; g: the trilinear interpolant of the samples'
        // central-difference gradients (one-sided on the grid's faces)
        double phi = 0.0, g[3] = {0.0, 0.0, 0.0};
        for (int corner = 0; corner < 8; ++corner) {
            const int o[3] = {corner & 1, (corner >> 1) & 1, (corner >> 2) & 1};
            int q[3];
            double w = 1.0;
            for (int a = 0; a < 3; ++a) {
                w *= o[a] ? t[a] : 1.0 - t[a];
                q[a] = c[a] + o[a];
            }
            phi += w * S(q);
            for (int a = 0; a < 3; ++a) {
                int qh[3] = {q[0], q[1], q[2]}, ql[3] = {q[0], q[1], q[2]};
                qh[a] = std::min(q[a] + 1, dims[a] - 1);
                ql[a] = std::max(q[a] - 1, 0);
                g[a] += w * (S(qh) - S(ql)) / (double)(qh[a] - ql[a]) * inv;
            }
        }
        if (phi_out) phi_out[q] = phi;
        const double gl = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        if (!(phi < 0.0) || !(gl > 0.0)) continue;
        const double nrm[3] = {g[0] / gl, g[1] / gl, g[2] / gl};
        const double vn = v[0] * nrm[0] + v[1] * nrm[1] + v[2] * nrm[2];
        for (int a = 0; a < 3; ++a) {
            x[a] -= phi * nrm[a];
            if (vn < 0.0) v[a] -= (1.0 + damp) * vn * nrm[a];
            x[a] = std::min(std::max(x[a], (double)P->lower[a]), (double)P->upper[a]);
        }
    }
    return 0;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
