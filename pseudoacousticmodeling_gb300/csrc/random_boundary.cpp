// Random boundary for the source field (the reference's "RBC" migration,
// src/Migration.py:327-458): the absorbing border's velocities are replaced
// by random ones, so the source wavefield scatters there instead of being
// absorbed, and the undamped scheme can be run backwards in time exactly -
// nothing needs storing.  Host code; the engine uploads kappa of the result.
//
// Per padding cell the velocity is drawn from a normal distribution centred
// on the edge-replicated value with a spread growing from 0 at the interior
// to `dvel` at the outer edge, clamped to [dvel, dvel + v] like the
// reference's get_randomvalue; then Gaussian velocity blobs (radius in
// [0.1, 1] x ratio, amplitude +-[0.5, 1] x dvel) are added around points
// dart-thrown at least `ratio` apart in the outer half of the border.  Unlike
// the reference, the blobs are added inside the border only, so the interior
// model stays exact.  Velocities are clipped to [vmin - dvel, vmax + dvel]
// (the reference's clip) and to `vcap`, the caller's stability limit.
#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

extern "C" int pam_random_boundary(const float* vp, int nz, int nx, int N, float dx, float dz, float dvel,
                                   float ratio, float vcap, unsigned long long seed, float* out) {
    if (!vp || !out || nz < 1 || nx < 1 || N < 1 || !(dx > 0.0f) || !(dz > 0.0f) || !(dvel >= 0.0f) ||
        !(ratio > 0.0f) || !(vcap > 0.0f))
        return -1;
    const int nza = nz + 2 * N, nxa = nx + 2 * N;
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    float vmin = vp[0], vmax = vp[0];
    for (long long i = 0; i < (long long)nz * nx; i++) {
        vmin = std::min(vmin, vp[i]);
        vmax = std::max(vmax, vp[i]);
    }
    const double lo = std::max(1.0, (double)vmin - dvel), hi = std::min((double)vmax + dvel, (double)vcap);
    // depth of a cell into the border: 0 inside, 1 .. N outwards
    auto depth = [&](int z, int x) {
        int d = 0;
        d = std::max(d, N - z);
        d = std::max(d, z - (N + nz - 1));
        d = std::max(d, N - x);
        d = std::max(d, x - (N + nx - 1));
        return d;
    };
    for (int z = 0; z < nza; z++)
        for (int x = 0; x < nxa; x++) {
            const int zi = std::min(std::max(z - N, 0), nz - 1), xi = std::min(std::max(x - N, 0), nx - 1);
            const double v = vp[(long long)zi * nx + xi];
            double r = v;
            const int d = depth(z, x);
            if (d > 0) {
                const double f = N > 1 ? (double)(d - 1) / (double)(N - 1) : 1.0;
                std::normal_distribution<double> g(v, std::max(1e-6, (double)dvel * f));
                const double p = g(rng);
                r = p < dvel ? (double)dvel : (p > dvel + v ? dvel + v : p);
                r = std::min(std::max(r, lo), hi);
            }
            out[(long long)z * nxa + x] = (float)r;
        }
    // blobs: dart throwing over the expanded domain, kept in the outer half of the border
    const double W = (nxa - 1) * (double)dx, H = (nza - 1) * (double)dz;
    const double half_x = 0.5 * N * dx, half_z = 0.5 * N * dz;
    std::vector<double> px, pz;
    const long long tries = std::max(64LL, (long long)(30.0 * W * H / ((double)ratio * ratio)));
    for (long long t = 0; t < tries; t++) {
        const double x = uni(rng) * W, z = uni(rng) * H;
        const bool outer = x < half_x || x > W - half_x || z < half_z || z > H - half_z;
        bool ok = outer;
        for (size_t k = 0; ok && k < px.size(); k++)
            ok = (px[k] - x) * (px[k] - x) + (pz[k] - z) * (pz[k] - z) >= (double)ratio * ratio;
        if (ok) {
            px.push_back(x);
            pz.push_back(z);
        }
    }
    for (size_t k = 0; k < px.size(); k++) {
        const double r = (0.1 + 0.9 * uni(rng)) * ratio;
        const double A = (0.5 + 0.5 * uni(rng)) * dvel * (uni(rng) < 0.5 ? -1.0 : 1.0);
        const int x0 = std::max(0, (int)std::floor((px[k] - 4 * r) / dx)), x1 = std::min(nxa - 1, (int)std::ceil((px[k] + 4 * r) / dx));
        const int z0 = std::max(0, (int)std::floor((pz[k] - 4 * r) / dz)), z1 = std::min(nza - 1, (int)std::ceil((pz[k] + 4 * r) / dz));
        for (int z = z0; z <= z1; z++)
            for (int x = x0; x <= x1; x++) {
                if (depth(z, x) == 0) continue;
                const double ddx = x * (double)dx - px[k], ddz = z * (double)dz - pz[k];
                float& c = out[(long long)z * nxa + x];
                const double v = c + A * std::exp(-0.5 * (ddx * ddx + ddz * ddz) / (r * r));
                c = (float)std::min(std::max(v, lo), hi);
            }
    }
    return (int)px.size();
}
