// ref_shader.cpp -- runs the reference's SPH compute shaders, compiled as C++
// through glsl_shim.hpp, on the CPU. TEST INFRASTRUCTURE ONLY: it pins the
// oracle (sph_oracle.cpp) to the reference's own code. Built by
// `make -C oracle ref` into oracle/_ref/ from the shader files in the
// reference tree; nothing of the reference is committed.
//
// ref_shader_step() reproduces one frame of Main.cpp:291-304: three dispatches
// of NUM_WORK_GROUPS x WORK_GROUP_SIZE invocations, each pass finished before
// the next (glMemoryBarrier). The shaders hard-code NUM_PARTICLES = 10000
// (rho_pres_comp.glsl:4), G, GAS_CONST and dt, so the particle array must hold
// exactly 10000 records.
#include "glsl_shim.hpp"

#include <omp.h>
#include <stdint.h>

namespace glslref {

struct RhoPresShader : ShaderEnv {
#include "rho_pres_comp.inc"
};
struct ForceShader : ShaderEnv {
#include "force_comp.inc"
};
struct IntegrateShader : ShaderEnv {
#include "integrate_comp.inc"
};

}  // namespace glslref

#undef particles

extern "C" {

int ref_shader_num_particles(void) { return NUM_PARTICLES; }

// particles: 10000 records of 64 bytes (pos, vel, force, extras).
// constants: ConstantsUniform {mass, smoothing_coeff, visc, resting_rho}.
// upper/lower: BoundaryUniform.
int ref_shader_step(void* particles, int n_steps, const float constants[4], const float upper[4],
                    const float lower[4], int nthreads) {
    using namespace glslref;
    if (!particles || !constants || !upper || !lower) return -1;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    const uint invocations = 10u * WORK_GROUP_SIZE;  // glDispatchCompute(NUM_WORK_GROUPS = 10, 1, 1)
    for (int s = 0; s < n_steps; ++s) {
#pragma omp parallel num_threads(nthreads)
        {
            RhoPresShader sh;
            sh.particles_ptr_ = reinterpret_cast<RhoPresShader::Particle(*)[]>(particles);
            sh.mass = constants[0]; sh.smoothing_coeff = constants[1];
            sh.visc = constants[2]; sh.resting_rho = constants[3];
#pragma omp for schedule(dynamic, 64)
            for (uint i = 0; i < invocations; ++i) { sh.gl_GlobalInvocationID = {i, 0, 0}; sh.main(); }
        }
#pragma omp parallel num_threads(nthreads)
        {
            ForceShader sh;
            sh.particles_ptr_ = reinterpret_cast<ForceShader::Particle(*)[]>(particles);
            sh.mass = constants[0]; sh.smoothing_coeff = constants[1];
            sh.visc = constants[2]; sh.resting_rho = constants[3];
#pragma omp for schedule(dynamic, 64)
            for (uint i = 0; i < invocations; ++i) { sh.gl_GlobalInvocationID = {i, 0, 0}; sh.main(); }
        }
#pragma omp parallel num_threads(nthreads)
        {
            IntegrateShader sh;
            sh.particles_ptr_ = reinterpret_cast<IntegrateShader::Particle(*)[]>(particles);
            for (int a = 0; a < 4; ++a) { sh.upper[a] = upper[a]; sh.lower[a] = lower[a]; }
#pragma omp for schedule(static)
            for (uint i = 0; i < invocations; ++i) { sh.gl_GlobalInvocationID = {i, 0, 0}; sh.main(); }
        }
    }
    return 0;
}

}  // extern "C"
