// nifti.hpp -- a small NIfTI-1 (.nii, single file) reader and writer for the fastreg_gb300
// command-line app.  Reads uint8/int16/int32/uint16/float32/float64 voxels (either byte
// order) into float32 or int16 arrays, applying scl_slope/scl_inter to intensities;
// writes float32 or int16 volumes with the geometry (pixdim, qform, sform) of a template
// header.  Gzipped files (.nii.gz) are not supported.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace nifti {

#pragma pack(push, 1)
struct Header {  // the 348-byte NIfTI-1 header
    int32_t sizeof_hdr;
    char data_type[10];
    char db_name[18];
    int32_t extents;
    int16_t session_error;
    char regular;
    char dim_info;
    int16_t dim[8];
    float intent_p1, intent_p2, intent_p3;
    int16_t intent_code;
    int16_t datatype;
    int16_t bitpix;
    int16_t slice_start;
    float pixdim[8];
    float vox_offset;
    float scl_slope, scl_inter;
    int16_t slice_end;
    char slice_code;
    char xyzt_units;
    float cal_max, cal_min;
    float slice_duration;
    float toffset;
    int32_t glmax, glmin;
    char descrip[80];
    char aux_file[24];
    int16_t qform_code, sform_code;
    float quatern_b, quatern_c, quatern_d;
    float qoffset_x, qoffset_y, qoffset_z;
    float srow_x[4], srow_y[4], srow_z[4];
    char intent_name[16];
    char magic[4];
};
#pragma pack(pop)
static_assert(sizeof(Header) == 348, "NIfTI-1 header is 348 bytes");

enum : int16_t { DT_UINT8 = 2, DT_INT16 = 4, DT_INT32 = 8, DT_FLOAT32 = 16, DT_FLOAT64 = 64, DT_UINT16 = 512 };

template <typename T>
inline void swap_bytes(T& v) {
    unsigned char* p = reinterpret_cast<unsigned char*>(&v);
    for (size_t i = 0; i < sizeof(T) / 2; ++i) std::swap(p[i], p[sizeof(T) - 1 - i]);
}

inline void swap_header(Header& h) {
    swap_bytes(h.sizeof_hdr);
    swap_bytes(h.extents);
    swap_bytes(h.session_error);
    for (auto& d : h.dim) swap_bytes(d);
    swap_bytes(h.intent_p1);
    swap_bytes(h.intent_p2);
    swap_bytes(h.intent_p3);
    swap_bytes(h.intent_code);
    swap_bytes(h.datatype);
    swap_bytes(h.bitpix);
    swap_bytes(h.slice_start);
    for (auto& p : h.pixdim) swap_bytes(p);
    swap_bytes(h.vox_offset);
    swap_bytes(h.scl_slope);
    swap_bytes(h.scl_inter);
    swap_bytes(h.slice_end);
    swap_bytes(h.cal_max);
    swap_bytes(h.cal_min);
    swap_bytes(h.slice_duration);
    swap_bytes(h.toffset);
    swap_bytes(h.glmax);
    swap_bytes(h.glmin);
    swap_bytes(h.qform_code);
    swap_bytes(h.sform_code);
    swap_bytes(h.quatern_b);
    swap_bytes(h.quatern_c);
    swap_bytes(h.quatern_d);
    swap_bytes(h.qoffset_x);
    swap_bytes(h.qoffset_y);
    swap_bytes(h.qoffset_z);
    for (int i = 0; i < 4; ++i) {
        swap_bytes(h.srow_x[i]);
        swap_bytes(h.srow_y[i]);
        swap_bytes(h.srow_z[i]);
    }
}

struct Volume {
    Header hdr{};
    int dims[3] = {0, 0, 0};
    std::vector<float> f;    // intensities (read_float)
    std::vector<int16_t> s;  // labels (read_int16)
};

inline Header read_header(std::ifstream& in, const std::string& path, bool* swapped) {
    Header h{};
    in.read(reinterpret_cast<char*>(&h), sizeof h);
    if (!in) throw std::runtime_error("cannot read a NIfTI header from " + path);
    *swapped = false;
    if (h.sizeof_hdr != 348) {
        Header t = h;
        swap_header(t);
        if (t.sizeof_hdr != 348) throw std::runtime_error(path + " is not a NIfTI-1 file");
        h = t;
        *swapped = true;
    }
    if (std::strncmp(h.magic, "n+1", 3) != 0) throw std::runtime_error(path + ": only single-file .nii is supported");
    if (h.dim[0] < 3) throw std::runtime_error(path + ": fewer than 3 dimensions");
    for (int k = 4; k <= h.dim[0] && k < 8; ++k)
        if (h.dim[k] > 1) throw std::runtime_error(path + ": only 3-D volumes are supported");
    return h;
}

template <typename Out>
inline Volume read(const std::string& path, bool scale) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open " + path);
    bool sw = false;
    Volume v;
    v.hdr = read_header(in, path, &sw);
    for (int k = 0; k < 3; ++k) v.dims[k] = v.hdr.dim[k + 1];
    const size_t n = (size_t)v.dims[0] * v.dims[1] * v.dims[2];
    in.seekg((std::streamoff)v.hdr.vox_offset);
    const float slope = (scale && v.hdr.scl_slope != 0.f && std::isfinite(v.hdr.scl_slope)) ? v.hdr.scl_slope : 1.f;
    const float inter = (scale && v.hdr.scl_slope != 0.f && std::isfinite(v.hdr.scl_inter)) ? v.hdr.scl_inter : 0.f;
    std::vector<Out> out(n);
    auto conv = [&](auto tag) {
        using T = decltype(tag);
        std::vector<T> raw(n);
        in.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)(n * sizeof(T)));
        if (!in) throw std::runtime_error(path + ": truncated voxel data");
        for (size_t i = 0; i < n; ++i) {
            T x = raw[i];
            if (sw) swap_bytes(x);
            out[i] = scale ? (Out)((float)x * slope + inter) : (Out)x;
        }
    };
    switch (v.hdr.datatype) {
        case DT_UINT8: conv(uint8_t{}); break;
        case DT_INT16: conv(int16_t{}); break;
        case DT_UINT16: conv(uint16_t{}); break;
        case DT_INT32: conv(int32_t{}); break;
        case DT_FLOAT32: conv(float{}); break;
        case DT_FLOAT64: conv(double{}); break;
        default: throw std::runtime_error(path + ": unsupported NIfTI datatype " + std::to_string(v.hdr.datatype));
    }
    if constexpr (std::is_same<Out, float>::value) v.f.swap(out);
    else v.s.swap(out);
    return v;
}

inline Volume read_float(const std::string& path) { return read<float>(path, true); }
inline Volume read_int16(const std::string& path) { return read<int16_t>(path, false); }

// writes data (float32 or int16) with the geometry of `tmpl`
template <typename T>
inline void write(const std::string& path, const Header& tmpl, const int dims[3], const T* data) {
    Header h = tmpl;
    h.sizeof_hdr = 348;
    h.dim[0] = 3;
    for (int k = 0; k < 3; ++k) h.dim[k + 1] = (int16_t)dims[k];
    for (int k = 4; k < 8; ++k) h.dim[k] = 1;
    h.datatype = std::is_same<T, float>::value ? DT_FLOAT32 : DT_INT16;
    h.bitpix = (int16_t)(8 * sizeof(T));
    h.vox_offset = 352.f;
    h.scl_slope = 0.f;
    h.scl_inter = 0.f;
    std::memcpy(h.magic, "n+1\0", 4);
    std::ofstream out(path, std::ios::binary);
    if (!out) throw std::runtime_error("cannot write " + path);
    out.write(reinterpret_cast<const char*>(&h), sizeof h);
    const char ext[4] = {0, 0, 0, 0};
    out.write(ext, 4);
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    out.write(reinterpret_cast<const char*>(data), (std::streamsize)(n * sizeof(T)));
    if (!out) throw std::runtime_error("write failed: " + path);
}

}  // namespace nifti
