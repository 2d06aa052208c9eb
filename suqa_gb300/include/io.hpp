// Drop-in replacement of the reference's include/io.hpp: debug/error macros and
// small IO helpers used by the drivers.
#pragma once
#include <algorithm>
#include <bitset>
#include <chrono>
#include <cmath>
#include <complex>
#include <iostream>
#include <vector>
#include <unistd.h>
#include <sys/time.h>

typedef unsigned int uint;
#ifndef M_PI
#define M_PI 3.141592653589793
#endif

#ifndef NDEBUG
#define DEBUG_CALL(x) x
#else
#define DEBUG_CALL(x)
#endif

// Evaluates its argument once (the reference macro expands it three times).
#define HANDLE_CUDACALL(fzcall)                                                     \
    do {                                                                            \
        auto hc_rc_ = (fzcall);                                                     \
        if ((int)hc_rc_ != 0)                                                       \
            printf("ERROR: in %s:%d, call %s, errno %d\n", __FILE__, __LINE__,      \
                   #fzcall, (int)hc_rc_);                                           \
    } while (0)

#define CHECK_ERROR(fzcall)                                                         \
    {                                                                               \
        int erri;                                                                   \
        if ((erri = (fzcall)))                                                      \
            fprintf(stderr, "ERROR no. %d on call %s, %s:%d\n", erri, #fzcall,      \
                    __FILE__, __LINE__);                                            \
    }

int get_time(struct timeval* tp, struct timezone* tzp);
bool file_exists(const char* fname);
void sparse_print(double* v_re, double* v_im, size_t size);
