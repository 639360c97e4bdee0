#include "survey.hpp"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace pam {

namespace {

// Minimal reader for the flat JSON object of Parameters.json: string, number,
// boolean and numeric-array values.
class JsonReader {
public:
    explicit JsonReader(const std::string& s) : s_(s) {}
    std::map<std::string, JsonValue> object() {
        std::map<std::string, JsonValue> out;
        ws();
        expect('{');
        ws();
        if (peek() == '}') { ++i_; return out; }
        while (true) {
            ws();
            std::string key = string();
            ws();
            expect(':');
            ws();
            out[key] = value();
            ws();
            if (peek() == ',') { ++i_; continue; }
            expect('}');
            break;
        }
        return out;
    }

private:
    const std::string& s_;
    size_t i_ = 0;
    char peek() const { return i_ < s_.size() ? s_[i_] : '\0'; }
    void ws() { while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_; }
    void expect(char c) {
        if (peek() != c) throw std::invalid_argument(std::string("Parameters.json: expected '") + c + "' at offset " +
                                                     std::to_string(i_));
        ++i_;
    }
    std::string string() {
        expect('"');
        std::string out;
        while (i_ < s_.size() && s_[i_] != '"') {
            if (s_[i_] == '\\' && i_ + 1 < s_.size()) ++i_;
            out.push_back(s_[i_++]);
        }
        expect('"');
        return out;
    }
    double number() {
        size_t j = i_;
        while (j < s_.size() && (std::isdigit((unsigned char)s_[j]) || s_[j] == '-' || s_[j] == '+' || s_[j] == '.' ||
                                 s_[j] == 'e' || s_[j] == 'E'))
            ++j;
        if (j == i_) throw std::invalid_argument("Parameters.json: bad value at offset " + std::to_string(i_));
        double v = std::stod(s_.substr(i_, j - i_));
        i_ = j;
        return v;
    }
    JsonValue value() {
        JsonValue v;
        const char c = peek();
        if (c == '"') { v.kind = JsonValue::String; v.str = string(); }
        else if (c == 't' && s_.compare(i_, 4, "true") == 0) { v.kind = JsonValue::Bool; v.b = true; i_ += 4; }
        else if (c == 'f' && s_.compare(i_, 5, "false") == 0) { v.kind = JsonValue::Bool; v.b = false; i_ += 5; }
        else if (c == 'n' && s_.compare(i_, 4, "null") == 0) { i_ += 4; }
        else if (c == '[') {
            ++i_;
            v.kind = JsonValue::Array;
            ws();
            if (peek() == ']') { ++i_; return v; }
            while (true) {
                ws();
                v.arr.push_back(number());
                ws();
                if (peek() == ',') { ++i_; continue; }
                expect(']');
                break;
            }
        } else { v.kind = JsonValue::Number; v.num = number(); }
        return v;
    }
};

void read_csv(const std::string& path, std::vector<float>& x, std::vector<float>& z) {
    std::ifstream f(path);
    if (!f.is_open()) throw std::invalid_argument("Could not open geometry file " + path);
    std::string line;
    std::getline(f, line);   // header
    while (std::getline(f, line)) {
        if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
        std::stringstream ss(line);
        std::string idx, cx, cz;
        std::getline(ss, idx, ',');
        std::getline(ss, cx, ',');
        std::getline(ss, cz, ',');
        x.push_back(std::stof(cx));
        z.push_back(std::stof(cz));
    }
}

}  // namespace

Survey::Survey(const std::string& path) {
    readParameters(path);
    readGeometry();
}

std::string Survey::path_of(const std::string& key) const {
    auto it = kv_.find(key);
    if (it == kv_.end() || it->second.kind != JsonValue::String) return "";
    const std::string& v = it->second.str;
    if (v.empty() || v[0] == '/') return v;
    return base_ + v;
}

void Survey::readParameters(const std::string& path) {
    std::ifstream f(path);
    if (!f.is_open()) throw std::invalid_argument("Could not open " + path);
    std::stringstream buf;
    buf << f.rdbuf();
    const std::string text = buf.str();
    kv_ = JsonReader(text).object();
    const size_t slash = path.find_last_of('/');
    base_ = slash == std::string::npos ? "" : path.substr(0, slash + 1);

    auto need = [&](const char* k) -> const JsonValue& {
        auto it = kv_.find(k);
        if (it == kv_.end()) throw std::invalid_argument(std::string("Parameters.json: missing key '") + k + "'");
        return it->second;
    };
    auto num = [&](const char* k, double d) {
        auto it = kv_.find(k);
        return it == kv_.end() ? d : it->second.num;
    };
    auto flag = [&](const char* k) {
        auto it = kv_.find(k);
        return it != kv_.end() && it->second.b;
    };
    auto str = [&](const char* k, const char* d) {
        auto it = kv_.find(k);
        return it == kv_.end() ? std::string(d) : it->second.str;
    };
    unit = need("unit").str;
    approximation = need("approximation").str;
    migration = need("migration").str;
    ABC = need("ABC").str;
    dx = (float)need("dx").num;
    dz = (float)need("dz").num;
    dt = (float)need("dt").num;
    L = (float)need("L").num;
    D = (float)need("D").num;
    T = (float)need("T").num;
    N_abc = (int)need("N_abc").num;
    fcut = (float)need("fcut").num;
    if (approximation != "acoustic" && approximation != "VTI" && approximation != "TTI")
        throw std::invalid_argument("Parameters.json: unknown approximation '" + approximation + "'");
    if (ABC != "cerjan" && ABC != "CPML") throw std::invalid_argument("Parameters.json: unknown ABC '" + ABC + "'");
    sigma = (float)num("sigma", 20.0);
    dvel = (float)num("dvel", 1000.0);
    ratio = (float)num("ratio", 200.0);
    v0 = (float)num("v0", 1500.0);
    shift = (float)num("shift", 0.1);
    window = (float)num("window", 0.05);
    step = (int)num("step", 0);
    fwi = flag("fwi");
    reciprocity = flag("reciprocity");
    multiparameter = flag("multiparameter");
    mirror = flag("mirror");
    idx_water = (int)num("idx_water", 0);
    batch = (int)num("batch", 0);
    ckpt_interval = (int)num("ckpt_interval", 0);
    ckpt_store = str("ckpt_store", "f32");
    rec_file = path_of("rec_file");
    src_file = path_of("src_file");
    vpFile = path_of("vpFile");
    epsilonFile = path_of("epsilonFile");
    deltaFile = path_of("deltaFile");
    thetaFile = path_of("thetaFile");
    seismogramFolder = path_of("seismogramFolder");
    imageFolder = path_of("imageFolder");
    gradientsFolder = path_of("gradientsFolder");

    // derived sizes, float arithmetic then std::round (cpp/Survey.cpp:101-108)
    const float pi = 3.14159265358979323846f;
    tlag = 2.0f * std::sqrt(pi) / fcut;
    itlag = (int)std::round(tlag / dt);
    nt_data = (int)std::round(T / dt) + 1;
    nx = (int)std::round(L / dx) + 1;
    nz = (int)std::round(D / dz) + 1;
    nt = itlag + nt_data;
    nx_abc = nx + 2 * N_abc;
    nz_abc = nz + 2 * N_abc;
}

void Survey::readGeometry() {
    read_csv(rec_file, rec_x, rec_z);
    read_csv(src_file, shot_x, shot_z);
    if (reciprocity) {
        std::swap(shot_x, rec_x);
        std::swap(shot_z, rec_z);
    }
    Nrec = (int)rec_x.size();
    Nshot = (int)shot_x.size();
    rx.resize(Nrec);
    rz.resize(Nrec);
    sx.resize(Nshot);
    sz.resize(Nshot);
    for (int i = 0; i < Nrec; i++) {
        rx[i] = (int)std::round(rec_x[i] / dx) + N_abc;
        rz[i] = (int)std::round(rec_z[i] / dz) + N_abc - (mirror ? idx_water : 0);
    }
    for (int i = 0; i < Nshot; i++) {
        sx[i] = (int)std::round(shot_x[i] / dx) + N_abc;
        sz[i] = (int)std::round(shot_z[i] / dz) + N_abc - (mirror ? idx_water : 0);
    }
}

std::string Survey::seismogramFile(int shot) const {
    char f[32];
    snprintf(f, sizeof(f), "%.1f", fcut);
    return seismogramFolder + "seismogram_shot_" + std::to_string(shot + 1) + "_Nt" + std::to_string(nt_data) +
           "_Nrec" + std::to_string(Nrec) + "_fcut" + f + ".bin";
}

std::string Survey::imageFile() const {
    return imageFolder + "image_" + approximation + "_Nx" + std::to_string(nx) + "_Nz" + std::to_string(nz) + ".bin";
}

std::string Survey::gradientFile(const std::string& parameter) const {
    return gradientsFolder + (parameter.empty() ? "" : parameter + "_") + "gradient_" + approximation + "_Nx" +
           std::to_string(nx) + "_Nz" + std::to_string(nz) + ".bin";
}

std::vector<float> import_bin(const std::string& path, size_t n) {
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open()) throw std::invalid_argument("Could not open file " + path + ". Please verify the file path.");
    std::vector<float> v(n);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(float)));
    if ((size_t)f.gcount() != n * sizeof(float))
        throw std::invalid_argument(path + " is shorter than " + std::to_string(n) + " floats");
    return v;
}

void save_bin(const std::string& path, const float* data, size_t n) {
    std::ofstream f(path, std::ios::binary);
    if (!f.is_open()) throw std::invalid_argument("Could not open file " + path + " for writing");
    f.write(reinterpret_cast<const char*>(data), (std::streamsize)(n * sizeof(float)));
}

}  // namespace pam
