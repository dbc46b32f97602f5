// Minimal stand-in for the one OpenCV type the reference's CUDA headers use
// (cv::Vec3i / cv::Vec3f in include/params.hpp and include/types.hpp), so that the
// reference's src/fastreg/cuda/*.cu compile without OpenCV.  Test infrastructure
// only: used by oracle/ref_build.py to build the reference kernels.
#pragma once

// standard headers the real OpenCV header brings in transitively
#include <cmath>
#include <iostream>
#include <limits>

namespace cv {

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

}  // namespace cv
