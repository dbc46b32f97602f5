// fastreg_compat.hpp -- the reference's C++ surface (struct Params, class FastReg) over the
// C ABI of fastreg_gb300, header only, without OpenCV.
//
// A caller of the reference (src/apps/demo.cpp) switches by including this header in
// place of <fastreg.hpp>/<params.hpp> and linking libfastreg_gb300.so; the member
// names and the in-place semantics of FastReg::operator() are those of
// include/fastreg.hpp:12-38 and src/fastreg/fastreg.cpp:58-75.  Errors throw
// fastreg_gb300::Error instead of printing and calling exit(0)
// (src/fastreg/device_memory.cpp:10-13).
#pragma once

#include <cuda_runtime_api.h>

#include <stdexcept>
#include <string>

#include "fastreg_gb300.h"

namespace cv {
#ifndef FASTREG_GB300_HAVE_OPENCV
// the two OpenCV vector types Params uses (include/params.hpp:8-9)
template <typename T, int n>
struct Vec {
    T val[n];
    Vec() {
        for (int i = 0; i < n; ++i) val[i] = T(0);
    }
    Vec(T a, T b, T c) {
        val[0] = a;
        val[1] = b;
        val[2] = c;
    }
    T& operator[](int i) { return val[i]; }
    const T& operator[](int i) const { return val[i]; }
};
typedef Vec<int, 3> Vec3i;
typedef Vec<float, 3> Vec3f;
#endif
}  // namespace cv

namespace fastreg_gb300 {

struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(int status, const fr_handle* h, const char* what) {
    if (status != FR_OK) throw Error(status, std::string(what) + ": " + fr_status_string(status) + ": " + fr_last_error(h));
}

}  // namespace fastreg_gb300

// struct Params (include/params.hpp:7-26); defaults are the reference's params.ini
struct Params {
    cv::Vec3i volume_dims = cv::Vec3i(193, 229, 193);
    cv::Vec3f volume_size = cv::Vec3f(1.f, 1.f, 1.f);

    int reset_iter = -1;
    int verbosity = 0;

    int no_labels = 6;
    int max_iter = 2048;
    float max_update_norm = -1e-10f, tau = 0.2f, rho_0 = 1.f, alpha = 0.004f, w_reg = 0.2f, p = 2.f, C = 0.25f;

    // additions of fastreg_gb300 (params.ini keys SOLVER, SMOOTH_SIGMA, SMOOTH_WIDTH, DAMPING, STEP, KEEP_STATE,
    // AUTOTUNE, STAGING)
    int solver = FR_SOLVER_REFERENCE;
    float smooth_sigma = 1.5f;
    int smooth_width = 7;
    float damping = 0.9f, step = 0.5f;
    int keep_state = 0;
    int autotune = 1;
    int staging = 0;

    int no_voxels() { return volume_dims[0] * volume_dims[1] * volume_dims[2]; }
    cv::Vec3f voxel_sizes() {
        return cv::Vec3f(volume_size[0] / volume_dims[0], volume_size[1] / volume_dims[1],
                         volume_size[2] / volume_dims[2]);
    }

    // params.ini with the keys of demo.cpp:96-138 (plus the additions)
    static Params from_ini(const std::string& path) {
        fr_params c;
        fr_params_default(&c);
        fastreg_gb300::check(fr_params_load_ini(path.c_str(), &c), nullptr, "params.ini");
        Params P;
        P.from_c(c);
        return P;
    }

    fr_params to_c() const {
        fr_params c;
        fr_params_default(&c);
        for (int i = 0; i < 3; ++i) {
            c.volume_dims[i] = volume_dims[i];
            c.volume_size[i] = volume_size[i];
        }
        c.no_labels = no_labels;
        c.max_iter = max_iter;
        c.max_update_norm = max_update_norm;
        c.rho_0 = rho_0;
        c.tau = tau;
        c.w_reg = w_reg;
        c.alpha = alpha;
        c.p = p;
        c.C = C;
        c.reset_iter = reset_iter;
        c.verbosity = verbosity;
        c.solver = solver;
        c.smooth_sigma = smooth_sigma;
        c.smooth_width = smooth_width;
        c.damping = damping;
        c.step = step;
        c.keep_state = keep_state;
        c.autotune = autotune;
        c.staging = staging;
        return c;
    }

    void from_c(const fr_params& c) {
        for (int i = 0; i < 3; ++i) {
            volume_dims[i] = c.volume_dims[i];
            volume_size[i] = c.volume_size[i];
        }
        no_labels = c.no_labels;
        max_iter = c.max_iter;
        max_update_norm = c.max_update_norm;
        rho_0 = c.rho_0;
        tau = c.tau;
        w_reg = c.w_reg;
        alpha = c.alpha;
        p = c.p;
        C = c.C;
        reset_iter = c.reset_iter;
        verbosity = c.verbosity;
        solver = c.solver;
        smooth_sigma = c.smooth_sigma;
        smooth_width = c.smooth_width;
        damping = c.damping;
        step = c.step;
        keep_state = c.keep_state;
        autotune = c.autotune;
        staging = c.staging;
    }
};

// class FastReg (include/fastreg.hpp:12-38)
class FastReg {
public:
    explicit FastReg(const Params& params_) : params(params_), frame_counter_(0) {
        fr_params c = params.to_c();
        fastreg_gb300::check(fr_create(&c, &h_), nullptr, "FastReg");
    }
    ~FastReg() {
        if (h_) fr_destroy(h_);
    }
    FastReg(const FastReg&) = delete;
    FastReg& operator=(const FastReg&) = delete;

    Params& getParams() { return params; }

    // psi of the last registration into a caller buffer of 3*N floats (3 planes, device)
    void getDeformationField(float* d_psi, cudaStream_t stream = 0) {
        fastreg_gb300::check(fr_get_field(h_, 0, FR_FIELD_PSI, d_psi, stream), h_, "getDeformationField");
        fastreg_gb300::check(cudaStreamSynchronize(stream) == cudaSuccess ? FR_OK : FR_ERR_CUDA, h_,
                             "getDeformationField");
    }

    // registers image_data_2 (source) to image_data_1 (target); all four are device
    // buffers of the volume's size and are overwritten in place: target <- T o psi_inv,
    // source <- S o psi.  Returns when the outputs are ready, like the reference.
    bool operator()(float* image_data_1, short* labels_data_1, float* image_data_2, short* labels_data_2) {
        fastreg_gb300::check(fr_register(h_, image_data_1, reinterpret_cast<int16_t*>(labels_data_1), image_data_2,
                                         reinterpret_cast<int16_t*>(labels_data_2), nullptr),
                             h_, "FastReg::operator()");
        fr_stats st;
        fastreg_gb300::check(fr_get_stats(h_, 0, &st), h_, "FastReg::operator()");  // synchronises
        last_stats_ = st;
        return ++frame_counter_, true;
    }

    // statistics of the last registration (energy, max update norm, folds, Dice)
    const fr_stats& stats() const { return last_stats_; }
    fr_handle* handle() { return h_; }

private:
    Params params;
    int frame_counter_;
    fr_handle* h_ = nullptr;
    fr_stats last_stats_{};
};
