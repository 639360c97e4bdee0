// Host harness for the reference's own host code (test infrastructure, never
// part of the product).  The reference's cpp/Migration.cu and cpp/Modeling.cu
// are compiled unmodified into this library, and plain C entry points drive,
// on the CPU, the routines that touch no GPU:
//   Migration::createMask + Migration::smoothModel   (cpp/Migration.cu:131-236)
//   Migration::Mute                                   (cpp/Migration.cu:86-115)
//   Modeling::checkDispersionAndStability             (cpp/Modeling.cu:184-327)
//   Modeling::expandModel                             (cpp/Modeling.cu:130-182)
// cpp/Survey.cpp needs nlohmann/json, which is absent, so the Survey default
// constructor declared in the unmodified cpp/Survey.hpp is defined here; it
// leaves the fields to the caller, which sets the ones each routine reads.
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "Migration.cuh"

Survey::Survey() {}

// f [nz][nx] is smoothed in place, as smoothModel does: slowness smoothing of
// a velocity (parameter = 0) or value smoothing (parameter = 1), with the
// water mask that createMask derives from water_model.
extern "C" int ref_smooth_model(float* f, int nz, int nx, float sigma, int parameter, const float* water_model) {
    Survey s;
    s.nz = nz;
    s.nx = nx;
    s.sigma = sigma;
    Migration m(&s, nullptr);
    bool* mask = m.createMask(water_model);
    m.smoothModel(f, mask, parameter != 0);
    delete[] mask;
    return 0;
}

// seis [nt][nrec] of shot 0 muted in place; receiver and shot coordinates in
// metres, as Survey holds them.
extern "C" int ref_mute(float* seis, int nt, int nrec, const float* rec_x, const float* rec_z, float shot_x,
                        float shot_z, float dt, float v0, float shift, float window) {
    Survey s;
    s.nt_data = nt;
    s.Nrec = nrec;
    s.rec_x.assign(rec_x, rec_x + nrec);
    s.rec_z.assign(rec_z, rec_z + nrec);
    s.shot_x.assign(1, shot_x);
    s.shot_z.assign(1, shot_z);
    s.dt = dt;
    s.v0 = v0;
    s.shift = shift;
    s.window = window;
    Migration m(&s, nullptr);
    m.Mute(seis, 0);
    return 0;
}

// The report of checkDispersionAndStability, printed with 9 significant
// digits (every float exactly) into out[out_len]; theta in degrees, converted
// to radians as Modeling::setModel does before the check (cpp/Modeling.cu:364-367).
extern "C" int ref_stability(int approximation, int nz, int nx, const float* vp, const float* eps, const float* delta,
                             const float* theta_deg, float dx, float dz, float dt, float fcut, char* out, int out_len) {
    Survey s;
    s.nz = nz;
    s.nx = nx;
    s.dx = dx;
    s.dz = dz;
    s.dt = dt;
    s.fcut = fcut;
    s.approximation = approximation == 0 ? "acoustic" : (approximation == 1 ? "VTI" : "TTI");
    std::vector<float> th;
    if (approximation == 2) {
        th.resize((size_t)nz * nx);
        for (size_t i = 0; i < th.size(); i++) th[i] = theta_deg[i] * pi / 180.0f;
    }
    Modeling m(&s);
    std::ostringstream os;
    std::streambuf* old = std::cout.rdbuf(os.rdbuf());
    const std::streamsize prec = std::cout.precision(9);
    m.checkDispersionAndStability(vp, eps, delta, th.empty() ? nullptr : th.data());
    std::cout.precision(prec);
    std::cout.rdbuf(old);
    const std::string r = os.str();
    if ((int)r.size() + 1 > out_len) return -1;
    std::memcpy(out, r.c_str(), r.size() + 1);
    return 0;
}

// model [nz][nx] padded by edge replication into out [nz + 2N][nx + 2N].
extern "C" int ref_expand_model(const float* model, int nz, int nx, int N, float* out) {
    Survey s;
    s.nz = nz;
    s.nx = nx;
    s.N_abc = N;
    s.nz_abc = nz + 2 * N;
    s.nx_abc = nx + 2 * N;
    Modeling m(&s);
    std::vector<float> in(model, model + (size_t)nz * nx);
    m.expandModel(in.data(), out);
    return 0;
}
