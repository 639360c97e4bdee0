// Job description in the reference's formats, for the C++ drivers:
// Parameters.json (flat object), source/receiver CSV files (header, then
// index,coordx,coordz rows), raw float32 .bin models and outputs.
// Field names follow the reference's Survey class (cpp/Survey.hpp:11-125);
// derived sizes use std::round like cpp/Survey.cpp:101-108.
#pragma once
#include <map>
#include <string>
#include <vector>

namespace pam {

struct JsonValue {
    enum Kind { Null, Bool, Number, String, Array } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<double> arr;
};

class Survey {
public:
    // throws std::invalid_argument with the offending key / file on error
    explicit Survey(const std::string& parameters_path);

    std::string unit, approximation, migration, ABC;
    float dx = 0, dz = 0, dt = 0, L = 0, D = 0, T = 0;
    int N_abc = 0;
    float fcut = 0, tlag = 0;
    int nx = 0, nz = 0, nt = 0, itlag = 0, nt_data = 0, nx_abc = 0, nz_abc = 0;
    float sigma = 20, v0 = 1500, shift = 0.1f, window = 0.05f;
    float dvel = 1000, ratio = 200;   // random border of the "RBC" migration
    int step = 0;
    bool fwi = false, reciprocity = false, mirror = false, multiparameter = false;
    int idx_water = 0;
    int batch = 0, ckpt_interval = 0;
    std::string ckpt_store = "f32";
    std::string rec_file, src_file, vpFile, epsilonFile, deltaFile, thetaFile;
    std::string seismogramFolder, imageFolder, gradientsFolder;
    std::vector<float> rec_x, rec_z, shot_x, shot_z;
    std::vector<int> rx, rz, sx, sz;
    int Nrec = 0, Nshot = 0;

    std::string seismogramFile(int shot) const;   // cpp/Modeling.cu:400
    std::string imageFile() const;                // cpp/Migration.cu:338
    // src/Migration.py:1095-1104; parameter "" (vp), "epsilon", "delta" or "theta"
    std::string gradientFile(const std::string& parameter = "") const;

private:
    std::map<std::string, JsonValue> kv_;
    std::string base_;
    void readParameters(const std::string& path);
    void readGeometry();
    std::string path_of(const std::string& key) const;
};

std::vector<float> import_bin(const std::string& path, size_t n);
void save_bin(const std::string& path, const float* data, size_t n);

}  // namespace pam
