// Pass-kernel instantiations for FP32 passes with dense blocks on the tensor
// cores (tcgen05): multi-tile passes (512 threads) and single-tile passes.
#define SQK_PASS_DEFINE
#include "sq_pass_host.cuh"

SQK_PASS_INSTANTIATE(float, 512, sqk::PF_DENSE | sqk::PF_TC)
SQK_PASS_INSTANTIATE(float, 1024, sqk::PF_DENSE | sqk::PF_TC)
