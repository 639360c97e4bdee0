// Dispersion / stability limits of Modeling::checkDispersionAndStability
// (cpp/Modeling.cu:184-327), host code shared by the engine's check and the
// engine-free pam_stability_limits.
#pragma once

#include <cstddef>

namespace pam {

// Limits for the n cells of a model (theta in radians, TTI only; eps/delta
// for VTI and TTI): *dt_lim, *dx_lim; returns 1 if dx, dz <= dx_lim and
// dt <= dt_lim, else 0.
int stability_limits(int approximation, size_t n, const float* vp, const float* eps, const float* del,
                     const float* theta_rad, float dx, float dz, float dt, float fcut, float* dt_lim,
                     float* dx_lim);

}  // namespace pam
