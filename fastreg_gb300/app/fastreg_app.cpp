// fastreg_app -- the reference's command-line app (src/apps/demo.cpp) on fastreg_gb300:
//
//   fastreg_app [--verbose|--vverbose] <ini path> <target path> <target labels path>
//               <source path> <source labels path> <out path>
//
// Reads params.ini and four NIfTI-1 volumes (float32 images, int16 labels), registers the
// source to the target with FastReg (include/fastreg_compat.hpp), prints the registration
// time like demo.cpp:306-310, and writes target_psi_inv_<name>.nii, source_psi_<name>.nii,
// target_psi_inv_labels_<name>.nii and source_psi_labels_<name>.nii into <out path>
// (demo.cpp:201-257; <name> is the source image's file name).  Exit status 0 on success,
// 1 on any error (the reference exits 0 from cudaSafeCall).
#include <cuda_runtime_api.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/fastreg_compat.hpp"
#include "nifti.hpp"

namespace {

std::string file_name(const std::string& s) {
    const size_t i = s.rfind('/');
    return i == std::string::npos ? "" : s.substr(i + 1);  // as demo.cpp:29-42 (empty without a '/')
}

void usage() {
    std::cout << "USAGE: fastreg [OPTIONS] <ini path> <target path> <target labels path> <source path> "
                 "<source labels path> <out path>\n"
                 "\t--help -h:    display help\n"
                 "\t--verbose: low verbosity\n"
                 "\t--vverbose: high verbosity\n";
}

template <typename T>
T* to_device(const std::vector<T>& h) {
    T* d = nullptr;
    if (cudaMalloc((void**)&d, h.size() * sizeof(T)) != cudaSuccess)
        throw std::runtime_error("cudaMalloc failed");
    if (cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        throw std::runtime_error("cudaMemcpy failed");
    return d;
}

template <typename T>
void to_host(std::vector<T>& h, const T* d) {
    if (cudaMemcpy(h.data(), d, h.size() * sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess)
        throw std::runtime_error("cudaMemcpy failed");
}

}  // namespace

int main(int argc, char** argv) {
    std::vector<std::string> paths;
    bool verbose = false, vverbose = false;
    for (int k = 1; k < argc; ++k) {
        const std::string a = argv[k];
        if (a == "-h" || a == "--help") {
            usage();
            return 0;
        }
        if (a == "--verbose") verbose = true;
        else if (a == "--vverbose") vverbose = true;
        else paths.push_back(a);
    }
    if (paths.size() < 6) {
        std::cerr << "error: incorrect number of arguments; please supply path to source and target data and .ini "
                     "file; exiting...\n";
        return 1;
    }
    try {
        Params params = Params::from_ini(paths[0]);
        if (vverbose) params.verbosity = 2;
        else if (verbose) params.verbosity = 1;
        nifti::Volume T = nifti::read_float(paths[1]), labT = nifti::read_int16(paths[2]);
        nifti::Volume S = nifti::read_float(paths[3]), labS = nifti::read_int16(paths[4]);
        for (const nifti::Volume* v : {&labT, &S, &labS})
            if (!std::equal(v->dims, v->dims + 3, T.dims)) throw std::runtime_error("the four volumes differ in size");
        for (int k = 0; k < 3; ++k) params.volume_dims[k] = T.dims[k];
        const std::string& out = paths[5];

        std::cout << "-------\nTARGET: " << paths[1] << ", " << paths[2] << "\nSOURCE: " << paths[3] << ", "
                  << paths[4] << "\n-------\nRUNNING NON-RIGID REGISTRATION" << std::endl;
        float* d_img_T = to_device(T.f);
        short* d_lab_T = (short*)to_device(labT.s);
        float* d_img_S = to_device(S.f);
        short* d_lab_S = (short*)to_device(labS.s);
        FastReg fastreg(params);
        const auto t0 = std::chrono::steady_clock::now();
        fastreg(d_img_T, d_lab_T, d_img_S, d_lab_S);
        const auto t1 = std::chrono::steady_clock::now();
        std::cout << "--- REGISTRATION TIME: " << std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count()
                  << "ms" << std::endl;
        const fr_stats& st = fastreg.stats();
        std::printf("iterations %d, energy %.9g (data %.9g, reg %.9g), folds %lld, dice (all labels) %.6f\n",
                    st.iterations, st.energy, st.e_data, st.e_reg, (long long)st.folds, st.dice_all);
        to_host(T.f, d_img_T);
        to_host(S.f, d_img_S);
        to_host(labT.s, (const int16_t*)d_lab_T);
        to_host(labS.s, (const int16_t*)d_lab_S);
        cudaFree(d_img_T);
        cudaFree(d_lab_T);
        cudaFree(d_img_S);
        cudaFree(d_lab_S);
        const std::string name = file_name(paths[3]);
        nifti::write(out + "/target_psi_inv_" + name + ".nii", T.hdr, T.dims, T.f.data());
        nifti::write(out + "/source_psi_" + name + ".nii", S.hdr, S.dims, S.f.data());
        nifti::write(out + "/target_psi_inv_labels_" + name + ".nii", labT.hdr, labT.dims, labT.s.data());
        nifti::write(out + "/source_psi_labels_" + name + ".nii", labS.hdr, labS.dims, labS.s.data());
        std::cout << "--- SAVED OUTPUT" << std::endl;
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 1;
    }
    return 0;
}
