// Drop-in replacement of the reference's include/complex_defines.cuh:
// Complex (x = re, y = im) and ComplexVec, the split re/im structure of arrays
// (one allocation of 2*vecsize elements: data_re = data, data_im = data + vecsize).
// With libsq the pointers are device pointers owned by the engine.
#pragma once
#include <cstddef>
#include <stdio.h>

typedef unsigned int uint;

struct cuDoubleComplexHost {
    double x;
    double y;
    cuDoubleComplexHost() = default;
    cuDoubleComplexHost(double xx, double yy) : x(xx), y(yy) {}
};
typedef cuDoubleComplexHost Complex;

struct ComplexVec {
    uint vecsize;
    double* data = nullptr;
    double* data_re = nullptr;
    double* data_im = nullptr;

    ComplexVec() : vecsize(0U), data(nullptr), data_re(nullptr), data_im(nullptr) {}

    size_t size() const { return vecsize; }
};

static inline double norm(const double& re, const double& im) { return re * re + im * im; }
