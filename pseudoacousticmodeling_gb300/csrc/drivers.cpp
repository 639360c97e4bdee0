// Command-line drivers with the behaviour of the reference's executables
// (cpp/modeling_main.cpp, cpp/migration_main.cpp, and the gradient evaluation
// the empty cpp/inversion_main.cpp was meant to hold), built three times from
// this file with PAM_DRIVER = 1 (modeling), 2 (migration), 3 (inversion).
//
//   pam_modeling  [Parameters.json]   writes seismogram_shot_<i>_Nt.._Nrec.._fcut...bin per shot
//   pam_migration [Parameters.json]   reads them, mutes, smooths the models, writes image_<approx>_Nx.._Nz...bin
//   pam_inversion [Parameters.json]   FWI gradient of the model in vpFile against the observed
//                                     seismograms, writes gradient_<approx>_Nx.._Nz...bin
//
// The default path is ../inputs/Parameters.json, as in cpp/Survey.cpp:42.
//
// Several processes, one per GPU (RANK and WORLD_SIZE in the environment, as
// torchrun sets them): each handles its contiguous share of the shots (shots
// are independent, cpp/Modeling.cu:441).  pam_modeling writes its shots'
// files; pam_migration and pam_inversion write their raw (unnormalised)
// partial sums and illumination to <output>.rank<r>of<w>, and
//   pam_migration --reduce <w> [Parameters.json]   (pam_inversion likewise)
// adds the w partial files and writes the normalised output.
#include <chrono>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pam.h"
#include "survey.hpp"

#ifndef PAM_DRIVER
#define PAM_DRIVER 1
#endif

namespace {

int check(pam_engine* e, int rc, const char* what) {
    if (rc < 0) {
        std::cerr << "Error: " << what << ": " << pam_last_error(e) << std::endl;
        throw std::runtime_error(what);
    }
    return rc;
}

struct Shard {
    int rank = 0, world = 1, first = 0, count = 0;
};

Shard shard_of(int nshot) {
    Shard sh;
    const char* r = std::getenv("RANK");
    const char* w = std::getenv("WORLD_SIZE");
    if (r && w) {
        sh.rank = std::atoi(r);
        sh.world = std::atoi(w);
    }
    if (sh.world < 1 || sh.rank < 0 || sh.rank >= sh.world)
        throw std::runtime_error("RANK / WORLD_SIZE do not describe a rank of a world");
    const int base = nshot / sh.world, extra = nshot % sh.world;
    sh.first = sh.rank * base + std::min(sh.rank, extra);
    sh.count = base + (sh.rank < extra ? 1 : 0);
    return sh;
}

std::string partial_name(const std::string& out, int rank, int world) {
    return out + ".rank" + std::to_string(rank) + "of" + std::to_string(world);
}

// Sum the partial files of `world` ranks (each: `fields` arrays of nmodel
// floats, the last one the illumination) in double, rank order.
[[maybe_unused]] std::vector<double> sum_partials(const std::string& out, int world, int fields, int nmodel) {
    std::vector<double> acc((size_t)fields * nmodel, 0.0);
    for (int r = 0; r < world; r++) {
        const std::vector<float> part = pam::import_bin(partial_name(out, r, world), (size_t)fields * nmodel);
        for (size_t i = 0; i < acc.size(); i++) acc[i] += part[i];
    }
    return acc;
}

#if PAM_DRIVER != 1
int reduce(const std::string& params, int world) {
    pam::Survey s(params);
    const int nmodel = s.nz * s.nx;
#if PAM_DRIVER == 2
    const std::vector<double> acc = sum_partials(s.imageFile(), world, 2, nmodel);
    std::vector<float> img((size_t)nmodel);
    for (int i = 0; i < nmodel; i++) {
        const float num = (float)acc[i], den = (float)acc[(size_t)nmodel + i];
        img[i] = den > 1e-12f ? num / den : 0.0f;      // cpp/Migration.cu:470-484
    }
    pam::save_bin(s.imageFile(), img.data(), img.size());
    std::cout << "Info: File saved to " << s.imageFile() << std::endl;
#else
    const bool multi = s.multiparameter && s.approximation != "acoustic";
    const int nfields = multi ? (s.approximation == "TTI" ? 5 : 4) : 2;   // gradient(s), then illumination
    const std::vector<double> acc = sum_partials(s.gradientFile(), world, nfields, nmodel);
    const double* il = acc.data() + (size_t)(nfields - 1) * nmodel;
    float mx = 0.0f;
    for (int i = 0; i < nmodel; i++) mx = std::max(mx, (float)il[i]);
    const char* names[4] = {"", "epsilon", "delta", "theta"};
    for (int f = 0; f < nfields - 1; f++) {
        std::vector<float> g((size_t)nmodel);
        for (int i = 0; i < nmodel; i++) g[i] = (float)acc[(size_t)f * nmodel + i] / ((float)il[i] + 1e-5f * mx);
        const std::string name = s.gradientFile(names[f]);
        pam::save_bin(name, g.data(), g.size());
        std::cout << "Info: File saved to " << name << std::endl;
    }
#endif
    return 0;
}
#endif

[[maybe_unused]] void write_partial(const std::string& out, const Shard& sh,
                                    const std::vector<const std::vector<float>*>& fields) {
    std::vector<float> all;
    for (const auto* f : fields) all.insert(all.end(), f->begin(), f->end());
    const std::string name = partial_name(out, sh.rank, sh.world);
    pam::save_bin(name, all.data(), all.size());
    std::cout << "Info: partial sums of rank " << sh.rank << " saved to " << name << std::endl;
}

int run(const std::string& params) {
    pam::Survey s(params);
    const Shard sh = shard_of(s.Nshot);
    const int nmodel = s.nz * s.nx;
    std::vector<float> vp = pam::import_bin(s.vpFile, nmodel), eps, dl, th;
    if (s.approximation != "acoustic") {
        eps = pam::import_bin(s.epsilonFile, nmodel);
        dl = pam::import_bin(s.deltaFile, nmodel);
    }
    if (s.approximation == "TTI") th = pam::import_bin(s.thetaFile, nmodel);
    const int batch = std::max(1, s.batch > 0 ? std::min(s.batch, sh.count) : sh.count);
    pam_config c{s.nz, s.nx, s.N_abc, s.dz, s.dx, s.dt, s.nt, s.itlag, s.fcut,
                 s.approximation == "acoustic" ? PAM_ACOUSTIC : (s.approximation == "VTI" ? PAM_VTI : PAM_TTI),
                 s.ABC == "cerjan" ? PAM_CERJAN : PAM_CPML, batch};
    pam_engine* e = nullptr;
    if (pam_create(&c, 0, &e) != PAM_OK) {
        std::cerr << "Error: " << pam_last_error(e) << std::endl;
        pam_destroy(e);
        return 1;
    }
    const int store = s.ckpt_store == "bf16" ? PAM_STORE_BF16 : (s.ckpt_store == "f16" ? PAM_STORE_F16 : PAM_STORE_F32);
    // source-field strategy (src/Migration.py:1563-1583): "onthefly" stores every
    // step, "checkpoint" every ckpt_interval (else `step`) steps, "SB" saves the
    // boundary band, "RBC" runs the source field through a random border
    const int K = s.migration == "onthefly" ? 0
                : s.migration == "SB"      ? PAM_BOUNDARY_SAVING
                : s.migration == "RBC"     ? PAM_RANDOM_BOUNDARY
                                           : (s.ckpt_interval > 0 ? s.ckpt_interval : s.step);
    const bool multi = PAM_DRIVER == 3 && s.multiparameter && s.approximation != "acoustic";
    if (multi && pam_set_multiparameter(e, 1) != PAM_OK) {
        std::cerr << "Error: " << pam_last_error(e) << std::endl;
        pam_destroy(e);
        return 1;
    }
    if (s.migration == "RBC" && pam_set_random_boundary(e, s.dvel, s.ratio, 0) != PAM_OK) {
        std::cerr << "Error: " << pam_last_error(e) << std::endl;
        pam_destroy(e);
        return 1;
    }
    const size_t nseis = (size_t)s.nt_data * s.Nrec;
    int rc = 0;
    try {
#if PAM_DRIVER == 2
        // Migration::setModel smooths slowness and the anisotropy (cpp/Migration.cu:252-309)
        // on the GPU (pam_smooth_model), every field with the water mask of the
        // unsmoothed velocity (createMask(vp) before any smoothing, :265)
        const std::vector<float> vp_raw = vp;
        auto smooth = [&](std::vector<float>& m, bool parameter) {
            if (!m.empty() && pam_smooth_model(m.data(), s.nz, s.nx, s.sigma, parameter ? 1 : 0, vp_raw.data()) != PAM_OK)
                throw std::runtime_error("model smoothing failed");
        };
        smooth(vp, false);
        smooth(eps, true);
        smooth(dl, true);
        smooth(th, true);
#endif
        check(e, pam_set_models(e, vp.data(), eps.empty() ? nullptr : eps.data(), dl.empty() ? nullptr : dl.data(),
                                th.empty() ? nullptr : th.data()), "set models");
        float dt_lim = 0, dx_lim = 0;
        const int ok = check(e, pam_check_stability(e, &dt_lim, &dx_lim), "stability check");
        std::cout << "info: Critical dx for dispersion: " << dx_lim << " m" << std::endl;
        std::cout << "info: Critical dt for stability: " << dt_lim << " s" << std::endl;
        std::cout << (ok ? "info: Dispersion and stability conditions satisfied."
                         : "WARNING: Dispersion or stability conditions not satisfied.") << std::endl;
        check(e, pam_set_receivers(e, s.Nrec, s.rz.data(), s.rx.data(), 0), "set receivers");
        std::vector<float> buf((size_t)batch * nseis);
        double misfit = 0.0;
        const int shot_end = sh.first + sh.count;
        for (int b0 = sh.first; b0 < shot_end; b0 += batch) {
            const int n = std::min(batch, shot_end - b0);
            std::cout << "info: Shots " << b0 + 1 << "-" << b0 + n << " of " << s.Nshot << std::endl;
#if PAM_DRIVER == 1
            check(e, pam_forward(e, n, &s.sz[b0], &s.sx[b0], buf.data(), nullptr), "forward modelling");
            for (int i = 0; i < n; i++) {
                pam::save_bin(s.seismogramFile(b0 + i), buf.data() + (size_t)i * nseis, nseis);
                std::cout << "Info: File saved to " << s.seismogramFile(b0 + i) << std::endl;
            }
#else
            for (int i = 0; i < n; i++) {
                std::vector<float> d = pam::import_bin(s.seismogramFile(b0 + i), nseis);
                std::copy(d.begin(), d.end(), buf.begin() + (size_t)i * nseis);
            }
#if PAM_DRIVER == 2
            // Migration::Mute of each gather (cpp/Migration.cu:86-115), on the GPU after the upload
            check(e, pam_set_mute(e, n, &s.shot_x[b0], &s.shot_z[b0], s.Nrec, s.rec_x.data(), s.rec_z.data(), 0,
                                  s.v0, s.shift, s.window), "mute");
            check(e, pam_rtm(e, n, &s.sz[b0], &s.sx[b0], buf.data(), K, store, nullptr), "migration");
#else
            check(e, pam_fwi_gradient(e, n, &s.sz[b0], &s.sx[b0], buf.data(), K, store, &misfit,
                                      nullptr), "gradient");
#endif
#endif
        }
#if PAM_DRIVER == 2
        std::vector<float> img((size_t)nmodel), ilum((size_t)nmodel);
        if (sh.world > 1) {
            check(e, pam_rtm_result(e, img.data(), ilum.data(), PAM_NORM_NONE), "image");
            write_partial(s.imageFile(), sh, {&img, &ilum});
        } else {
            check(e, pam_rtm_result(e, img.data(), ilum.data(), PAM_NORM_CPP), "image");
            pam::save_bin(s.imageFile(), img.data(), img.size());
            std::cout << "Info: File saved to " << s.imageFile() << std::endl;
        }
#elif PAM_DRIVER == 3
        std::vector<float> g((size_t)nmodel), ilum((size_t)nmodel);
        check(e, pam_fwi_result(e, g.data(), ilum.data()), "gradient");
        if (sh.world > 1) {
            std::vector<float> ge((size_t)nmodel), gd((size_t)nmodel), gt((size_t)nmodel);
            std::vector<const std::vector<float>*> parts = {&g};
            if (multi) {
                const bool tti = s.approximation == "TTI";
                check(e, pam_fwi_multiparameter_result(e, ge.data(), gd.data(), tti ? gt.data() : nullptr),
                      "gradient");
                parts.push_back(&ge);
                parts.push_back(&gd);
                if (tti) parts.push_back(&gt);
            }
            parts.push_back(&ilum);
            write_partial(s.gradientFile(), sh, parts);
            std::cout << "info: misfit of rank " << sh.rank << " " << misfit << std::endl;
            pam_destroy(e);
            return 0;
        }
        float mx = 0.0f;
        for (float v : ilum) mx = std::max(mx, v);
        for (size_t i = 0; i < g.size(); i++) g[i] /= ilum[i] + 1e-5f * mx;    // src/Migration.py:1086
        pam::save_bin(s.gradientFile(), g.data(), g.size());
        if (multi) {
            // epsilon, delta (theta) gradients, same normalisation (src/Migration.py:1087-1104)
            std::vector<float> ge((size_t)nmodel), gd((size_t)nmodel), gt((size_t)nmodel);
            const bool tti = s.approximation == "TTI";
            check(e, pam_fwi_multiparameter_result(e, ge.data(), gd.data(), tti ? gt.data() : nullptr), "gradient");
            const char* names[3] = {"epsilon", "delta", "theta"};
            std::vector<float>* fields[3] = {&ge, &gd, &gt};
            for (int f = 0; f < (tti ? 3 : 2); f++) {
                std::vector<float>& v = *fields[f];
                for (size_t i = 0; i < v.size(); i++) v[i] /= ilum[i] + 1e-5f * mx;
                pam::save_bin(s.gradientFile(names[f]), v.data(), v.size());
                std::cout << "Info: File saved to " << s.gradientFile(names[f]) << std::endl;
            }
        }
        std::cout << "info: misfit " << misfit << std::endl;
        std::cout << "Info: File saved to " << s.gradientFile() << std::endl;
#endif
        (void)misfit;
        (void)store;
        (void)K;
        (void)multi;
    } catch (const std::exception& ex) {
        std::cerr << "Error: " << ex.what() << std::endl;
        rc = 1;
    }
    pam_destroy(e);
    return rc;
}

}  // namespace

int main(int argc, char** argv) {
    const auto t0 = std::chrono::system_clock::now();
    int rc;
    try {
#if PAM_DRIVER != 1
        if (argc > 2 && std::strcmp(argv[1], "--reduce") == 0) {
            const int world = std::atoi(argv[2]);
            if (world < 1) throw std::runtime_error("--reduce needs the number of ranks");
            return reduce(argc > 3 ? argv[3] : "../inputs/Parameters.json", world);
        }
#endif
        const std::string params = argc > 1 ? argv[1] : "../inputs/Parameters.json";
        rc = run(params);
    } catch (const std::exception& ex) {
        std::cerr << "Error: " << ex.what() << std::endl;
        rc = 1;
    }
    const std::chrono::duration<double> el = std::chrono::system_clock::now() - t0;
    std::cout << "\nRun time: " << el.count() << " s." << std::endl;
    return rc;
}
