// Dispersion / stability check of the modeller (Modeling::
// checkDispersionAndStability, cpp/Modeling.cu:184-327), on the host.
//
// Acoustic: the shortest wavelength vmin / fcut needs 4.28 cells, and the
// leapfrog limit is dt <= dx_lim / (4 vmax).  VTI/TTI: the limit follows the
// largest phase velocity of the pseudo-acoustic operator over the cells with
// the 8th-order stencil's amplification sum; the wavelength criterion uses
// the smallest phase velocity over propagation angles (0 .. 90 degrees for
// VTI, 0 .. 180 for TTI, relative to each cell's tilt).
#include "stability.hpp"

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/pam.h"

namespace pam {

namespace {
const float kPiF = 3.14159265358979323846f;
}

int stability_limits(int approximation, size_t n, const float* vp, const float* eps, const float* del,
                     const float* theta_rad, float dx, float dz, float dt, float fcut, float* dt_lim_out,
                     float* dx_lim_out) {
    float vmin = INFINITY, vmax = 0.0f;
    for (size_t i = 0; i < n; i++) { vmin = std::min(vmin, vp[i]); vmax = std::max(vmax, vp[i]); }
    float dx_lim, dt_lim;
    if (approximation == PAM_ACOUSTIC) {
        const float lmin = vmin / fcut;
        dx_lim = lmin / 4.28f;
        dt_lim = dx_lim / (4.0f * vmax);
    } else {
        const float c8[4] = {8.0f / 5.0f, -1.0f / 5.0f, 8.0f / 315.0f, -1.0f / 560.0f};
        float soma = 0.0f;
        for (int m = 1; m <= 4; m++) soma += c8[m - 1] * (1.0f - std::pow(-1.0f, (float)m));
        // the reference's inverse powers: 1/dx squared, that squared (cpp/Modeling.cu:218-223)
        const float idx = 1.0f / dx, idz = 1.0f / dz;
        const float idx2 = idx * idx, idz2 = idz * idz;
        const float idx4 = idx2 * idx2, idz4 = idz2 * idz2;
        float maxst = 0.0f;
        for (size_t i = 0; i < n; i++) {
            const float e = eps[i], d = del[i];
            const float num = -2.0f * (e - d) * idx2 * idz2;
            const float den = (1.0f + 2.0f * e) * idx4 + idz4 + 2.0f * (1.0f + d) * idx2 * idz2;
            const float Sk = std::fabs(den) > 1e-12f ? num / den : 0.0f;
            const float f = ((1.0f + 2.0f * e) + Sk) * idx2 + (1.0f + Sk) * idz2;
            maxst = std::max(maxst, vp[i] * std::sqrt(f));
        }
        dt_lim = std::sqrt(2.0f) / (std::sqrt(soma) * maxst);
        const bool tti = approximation == PAM_TTI;
        const int nang = tti ? 361 : 181;
        const float amax = tti ? kPiF : 0.5f * kPiF;
        float pmin = INFINITY;
        for (int ia = 0; ia < nang; ia++) {
            const float phi = amax * ia / (nang - 1);
            for (size_t i = 0; i < n; i++) {
                const float beta = tti ? phi - theta_rad[i] : phi;
                const float sn = std::sin(beta), cs = std::cos(beta);
                const float s2 = sn * sn, c2 = cs * cs;
                const float e = eps[i], d = del[i];
                const float num = -2.0f * (e - d) * s2 * c2;
                const float den = (1.0f + 2.0f * e) * s2 * s2 + c2 * c2 + 2.0f * (1.0f + d) * s2 * c2;
                const float Sk = std::fabs(den) > 1e-12f ? num / den : 0.0f;
                pmin = std::min(pmin, vp[i] * std::sqrt((1.0f + 2.0f * e) * s2 + c2 + Sk));
            }
        }
        dx_lim = (pmin / fcut) / 4.28f;
    }
    if (dt_lim_out) *dt_lim_out = dt_lim;
    if (dx_lim_out) *dx_lim_out = dx_lim;
    return (dx <= dx_lim && dz <= dx_lim && dt <= dt_lim) ? 1 : 0;
}

}  // namespace pam

extern "C" int pam_stability_limits(int approximation, int nz, int nx, const float* vp, const float* eps,
                                    const float* delta, const float* theta_deg, float dx, float dz, float dt,
                                    float fcut, float* dt_lim, float* dx_lim) {
    if (!vp || nz < 1 || nx < 1 || !(dx > 0.0f) || !(dz > 0.0f) || !(fcut > 0.0f)) return PAM_E_ARG;
    if (approximation != PAM_ACOUSTIC && approximation != PAM_VTI && approximation != PAM_TTI) return PAM_E_ARG;
    if (approximation != PAM_ACOUSTIC && (!eps || !delta)) return PAM_E_ARG;
    if (approximation == PAM_TTI && !theta_deg) return PAM_E_ARG;
    const size_t n = (size_t)nz * nx;
    std::vector<float> th;
    if (approximation == PAM_TTI) {
        th.resize(n);
        for (size_t i = 0; i < n; i++) th[i] = theta_deg[i] * pam::kPiF / 180.0f;   // cpp/Modeling.cu:364-367
    }
    return pam::stability_limits(approximation, n, vp, eps, delta, th.empty() ? nullptr : th.data(), dx, dz, dt, fcut,
                                 dt_lim, dx_lim);
}
