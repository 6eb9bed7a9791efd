// sph_host.h -- host helpers shared by sph_host.cpp and the engine.
#pragma once

#include "sph_internal.h"

namespace sphgb {

float cutoff_d2(float h);
float smoothing_length(const sph_params& p);
float cell_edge(const sph_params& p, int stencil);
bool grid_dims(const sph_params& p, int stencil, float* edge_out, int dims[3]);
SceneDev make_scene_dev(const sph_params& p, int stencil, int cell_base, int first, int count, bool keep_force);

}  // namespace sphgb
