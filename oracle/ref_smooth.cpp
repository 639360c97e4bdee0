// Host harness for the reference's model smoothing (test infrastructure,
// never part of the product): the reference's own Migration::createMask and
// Migration::smoothModel (cpp/Migration.cu:131-236), compiled unmodified
// together with cpp/Modeling.cu (which Migration.cu links against), driven
// on the CPU through a plain C entry point.  Neither function touches the
// GPU.  cpp/Survey.cpp needs nlohmann/json, which is absent, so the Survey
// default constructor declared in the unmodified cpp/Survey.hpp is defined
// here (it leaves the fields to the caller; smoothModel reads nz, nx and
// sigma).
#include "Migration.cuh"

Survey::Survey() {}

// f [nz][nx] is smoothed in place, as smoothModel does: slowness smoothing of
// a velocity (parameter = 0) or value smoothing (parameter = 1), with the
// water mask that createMask derives from mask_model (cells within 1e-3 of
// its minimum keep their value).
extern "C" int ref_smooth_model(float* f, int nz, int nx, float sigma, int parameter, const float* mask_model) {
    Survey s;
    s.nz = nz;
    s.nx = nx;
    s.sigma = sigma;
    Migration m(&s, nullptr);
    bool* mask = m.createMask(mask_model);
    m.smoothModel(f, mask, parameter != 0);
    delete[] mask;
    return 0;
}
