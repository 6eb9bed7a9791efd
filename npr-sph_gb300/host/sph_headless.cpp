// sph_headless.cpp -- the reference's host loop without a window, over the C ABI.
//
// Mirrors NPR-SPH/Main.cpp:
//   init_particles()   Main.cpp:510-539  make_grid() lattice -> sph_scene_reference_grid + sph_upload_aos
//   sendUniforms()     Main.cpp:254-279  ConstantsUniform/BoundaryUniform -> sph_set_params, every frame,
//                                        after the step (so a step uses the previous frame's uniforms)
//   display()          Main.cpp:285-305  if simulate: the three dispatches -> sph_step(ctx, 1)
//   keyboard()         Main.cpp:454-476  'p' toggles simulate (which starts false, Main.cpp:87),
//                                        'r' re-initialises the particles
// Keys come from a script instead of GLFW: --keys "p@0,r@500,p@501" presses a key at a frame.
// Every --report frames one JSON line goes to stdout: frame, steps, wall time per frame and the
// FP64 diagnostics (sph_reduce). --scene dam_break runs the 1,048,576-particle dam break instead
// of the reference's 10,000-particle lattice. --render-every N draws the particles every N
// frames (the toon pass of display(), Main.cpp:311-337, through sph_render) and writes
// <prefix>_<frame>.ppm: the headless stand-in for the window and the video capture
// (Main.cpp:377-384).
//
//   sph_headless [--frames N] [--keys "p@0"] [--report N] [--scene reference|dam_break]
//                [--visc V] [--smoothing S] [--mass M] [--rest-rho R]
//                [--render-every N] [--render-prefix P] [--size WxH]
//                [--obstacle mesh.obj] [--obstacle-spacing S]
// --obstacle loads a Wavefront OBJ mesh (the reference's LoadMesh, LoadMesh.cpp:16-55) and makes
// it a static obstacle of the step: its signed distance field sampled over the box
// (sph_sdf_from_mesh), handed to sph_set_obstacle.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "sph_gb300.h"

namespace {

struct Options {
    int frames = 600;
    int report = 60;
    std::string scene = "reference";
    std::map<int, std::string> keys;  // frame -> keys pressed
    float visc = -1, smoothing = -1, mass = -1, rest_rho = -1;
    int render_every = 0;
    std::string render_prefix = "frame";
    int width = 720, height = 720;  // init_window_width/height (Main.cpp:39-40)
    std::string obstacle;           // OBJ mesh to collide with (README.md:59; meshes load in LoadMesh.cpp:16-55)
    float obstacle_spacing = 0.0f;  // SDF sample spacing; 0: h / 2
};

bool parse(int argc, char** argv, Options& o) {
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&](const char* what) -> const char* {
            if (i + 1 >= argc) { std::fprintf(stderr, "%s needs a value\n", what); std::exit(2); }
            return argv[++i];
        };
        if (a == "--frames") o.frames = std::atoi(next("--frames"));
        else if (a == "--report") o.report = std::atoi(next("--report"));
        else if (a == "--scene") o.scene = next("--scene");
        else if (a == "--visc") o.visc = (float)std::atof(next("--visc"));
        else if (a == "--smoothing") o.smoothing = (float)std::atof(next("--smoothing"));
        else if (a == "--mass") o.mass = (float)std::atof(next("--mass"));
        else if (a == "--rest-rho") o.rest_rho = (float)std::atof(next("--rest-rho"));
        else if (a == "--render-every") o.render_every = std::atoi(next("--render-every"));
        else if (a == "--render-prefix") o.render_prefix = next("--render-prefix");
        else if (a == "--obstacle") o.obstacle = next("--obstacle");
        else if (a == "--obstacle-spacing") o.obstacle_spacing = (float)std::atof(next("--obstacle-spacing"));
        else if (a == "--size") {
            if (std::sscanf(next("--size"), "%dx%d", &o.width, &o.height) != 2) return false;
        }
        else if (a == "--keys") {
            std::string s = next("--keys");
            size_t p = 0;
            while (p < s.size()) {
                size_t q = s.find(',', p);
                if (q == std::string::npos) q = s.size();
                std::string tok = s.substr(p, q - p);
                size_t at = tok.find('@');
                if (at == std::string::npos || at == 0) { std::fprintf(stderr, "bad key event '%s'\n", tok.c_str()); return false; }
                o.keys[std::atoi(tok.c_str() + at + 1)] += tok.substr(0, at);
                p = q + 1;
            }
        } else {
            std::fprintf(stderr, "unknown argument %s\n", a.c_str());
            return false;
        }
    }
    return o.frames >= 0 && o.report > 0 && o.render_every >= 0 && o.width > 0 && o.height > 0 &&
           (o.scene == "reference" || o.scene == "dam_break");
}

// The scene the 'r' key re-creates.
std::vector<sph_particle> make_particles(const Options& o, sph_params& p) {
    std::vector<sph_particle> parts;
    if (o.scene == "reference") {
        parts.resize(10000);
        sph_scene_reference_grid(parts.data(), 10000, p.particle_radius);  // make_grid(), Main.cpp:488-505
    } else {
        // 64 x 128 x 128 block at 0.5h against the x = 0 wall of a 5.12 x 1.28 x 1.28 box
        const float s = 0.5f * p.smoothing_coeff * p.particle_radius;
        const float lo[3] = {0, 0, 0}, hi[3] = {64 * s, 128 * s, 128 * s};
        p.lower[0] = p.lower[1] = p.lower[2] = 0.0f;
        p.upper[0] = 4 * 128 * s;
        p.upper[1] = p.upper[2] = 128 * s;
        p.gravity[1] = -9.81f;
        parts.resize(64u * 128u * 128u);
        sph_scene_fill(parts.data(), (uint32_t)parts.size(), lo, hi, s, 0.01f * 2 * s, 2);
    }
    return parts;
}

void report(sph_ctx* ctx, int frame, double ms_per_frame) {
    sph_diag d;
    if (sph_reduce(ctx, &d) != SPH_OK) {
        std::printf("{\"frame\": %d, \"error\": \"%s\"}\n", frame, sph_last_error(ctx));
        return;
    }
    std::printf("{\"frame\": %d, \"steps\": %llu, \"ms_per_frame\": %.4f, \"mean_rho\": %.6g, \"max_rho\": %.6g, "
                "\"kinetic_energy\": %.6g, \"momentum\": [%.6g, %.6g, %.6g], \"nonfinite\": %llu}\n",
                frame, (unsigned long long)d.step, ms_per_frame, d.mean_rho, d.max_rho, d.kinetic_energy,
                d.momentum[0], d.momentum[1], d.momentum[2], (unsigned long long)d.nonfinite);
    std::fflush(stdout);
}

}  // namespace

// The mesh of --obstacle as a static obstacle: its signed distance field sampled over the box
// (sph_sdf_from_mesh on the GPU), handed to sph_set_obstacle.
bool load_obstacle(sph_ctx* ctx, const Options& o, const sph_params& p) {
    uint32_t nv = 0, nt = 0;
    if (sph_obj_read(o.obstacle.c_str(), nullptr, &nv, nullptr, &nt) != SPH_OK || nt == 0) {
        std::fprintf(stderr, "cannot read the mesh %s\n", o.obstacle.c_str());
        return false;
    }
    std::vector<float> v(3ull * nv);
    std::vector<uint32_t> t(3ull * nt);
    if (sph_obj_read(o.obstacle.c_str(), v.data(), &nv, t.data(), &nt) != SPH_OK) return false;
    const float sp = o.obstacle_spacing > 0 ? o.obstacle_spacing : 0.5f * p.smoothing_coeff * p.particle_radius;
    int32_t dims[3];
    float org[3];
    size_t total = 1;
    for (int a = 0; a < 3; ++a) {
        org[a] = p.lower[a];
        dims[a] = std::max(2, (int)std::ceil((p.upper[a] - p.lower[a]) / sp) + 1);
        total *= (size_t)dims[a];
    }
    std::vector<float> sdf(total);
    if (sph_sdf_from_mesh(v.data(), nv, t.data(), nt, dims, org, sp, sdf.data()) != SPH_OK ||
        sph_set_obstacle(ctx, sdf.data(), dims, org, sp) != SPH_OK) {
        std::fprintf(stderr, "obstacle: %s\n", sph_last_error(ctx));
        return false;
    }
    std::fprintf(stderr, "obstacle %s: %u triangles, %d x %d x %d samples at %g\n", o.obstacle.c_str(), nt, dims[0],
                 dims[1], dims[2], sp);
    return true;
}

// The view of a scene: the reference's initial camera for its own lattice; for the dam break a
// camera that sees its 5.12 x 1.28 x 1.28 box.
sph_view make_view(const Options& o) {
    sph_view v;
    sph_view_default(&v, o.width, o.height, 1.0f);
    if (o.scene == "dam_break") {
        const float eye[3] = {2.56f, 2.5f, 6.0f}, center[3] = {2.56f, 0.5f, 0.64f};
        sph_view_camera(&v, 0.0f, 1.0f, eye, center);
        v.point_size = 4.0f;
    }
    return v;
}

int main(int argc, char** argv) {
    Options o;
    if (!parse(argc, argv, o)) {
        std::fprintf(stderr, "usage: %s [--frames N] [--keys \"p@0,r@500\"] [--report N] "
                             "[--scene reference|dam_break] [--visc V] [--smoothing S] [--mass M] [--rest-rho R] "
                             "[--render-every N] [--render-prefix P] [--size WxH] [--obstacle mesh.obj] "
                             "[--obstacle-spacing S]\n",
                     argv[0]);
        return 2;
    }
    sph_params p;
    sph_params_default(&p);  // ConstantsData / BoundaryData initial values (Main.cpp:110-122)
    std::vector<sph_particle> parts = make_particles(o, p);
    sph_ctx* ctx = nullptr;
    if (sph_create(&p, (uint32_t)parts.size(), nullptr, &ctx) != SPH_OK) {
        std::fprintf(stderr, "sph_create failed\n");
        return 1;
    }
    if (sph_upload_aos(ctx, parts.data(), (uint32_t)parts.size()) != SPH_OK) {
        std::fprintf(stderr, "upload: %s\n", sph_last_error(ctx));
        return 1;
    }
    if (!o.obstacle.empty() && !load_obstacle(ctx, o, p)) return 1;
    const sph_view view = make_view(o);
    std::vector<uint8_t> image(o.render_every > 0 ? (size_t)o.width * o.height * 4 : 0);
    bool simulate = false;  // Main.cpp:87: a zero-initialised global, so the simulation starts paused
    auto t0 = std::chrono::steady_clock::now();
    int frames_since = 0;
    for (int frame = 0; frame < o.frames; ++frame) {
        auto it = o.keys.find(frame);
        if (it != o.keys.end()) {
            for (char k : it->second) {
                if (k == 'p' || k == 'P') simulate = !simulate;  // Main.cpp:466-468
                if (k == 'r' || k == 'R') {                      // Main.cpp:460-464
                    parts = make_particles(o, p);
                    if (sph_upload_aos(ctx, parts.data(), (uint32_t)parts.size()) != SPH_OK) {
                        std::fprintf(stderr, "reset: %s\n", sph_last_error(ctx));
                        return 1;
                    }
                }
            }
        }
        if (simulate && sph_step(ctx, 1) != SPH_OK) {  // display(), Main.cpp:291-304
            std::fprintf(stderr, "step: %s\n", sph_last_error(ctx));
            return 1;
        }
        // sendUniforms() after the dispatches (Main.cpp:314): slider edits reach the next frame
        if (o.visc > 0) p.visc = o.visc;
        if (o.smoothing > 0) p.smoothing_coeff = o.smoothing;
        if (o.mass > 0) p.mass = o.mass;
        if (o.rest_rho > 0) p.resting_rho = o.rest_rho;
        if (sph_set_params(ctx, &p) != SPH_OK) std::fprintf(stderr, "uniforms: %s\n", sph_last_error(ctx));
        if (o.render_every > 0 && (frame + 1) % o.render_every == 0) {
            char name[4096];
            std::snprintf(name, sizeof(name), "%s_%05d.ppm", o.render_prefix.c_str(), frame + 1);
            if (sph_render(ctx, &view, 0, image.data(), 0) != SPH_OK ||
                sph_image_write_ppm(name, image.data(), o.width, o.height) != SPH_OK) {
                std::fprintf(stderr, "render: %s\n", sph_last_error(ctx));
                return 1;
            }
        }
        ++frames_since;
        if ((frame + 1) % o.report == 0 || frame + 1 == o.frames) {
            if (sph_synchronize(ctx) != SPH_OK) {
                std::fprintf(stderr, "device: %s\n", sph_last_error(ctx));
                return 1;
            }
            auto t1 = std::chrono::steady_clock::now();
            double ms = std::chrono::duration<double, std::milli>(t1 - t0).count() / frames_since;
            report(ctx, frame + 1, ms);
            frames_since = 0;
            t0 = std::chrono::steady_clock::now();
        }
    }
    sph_destroy(ctx);
    return 0;
}
