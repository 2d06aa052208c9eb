// Pass-kernel instantiation for FP64 states with double-float arithmetic
// (multi-tile passes without tables or dense blocks).
#define SQK_PASS_DEFINE
#include "sq_pass_host.cuh"

SQK_PASS_INSTANTIATE(sqk::df64, 256, 0)
