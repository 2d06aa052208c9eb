// Pass-kernel instantiations for FP32 states without tensor-core blocks:
// multi-tile passes plain, with bulk staging, with dense blocks on the CUDA
// cores (tiles below 2^12 amplitudes, or the CUDA-core dense engine);
// single-tile passes plain and with dense blocks.
#define SQK_PASS_DEFINE
#include "sq_pass_host.cuh"

SQK_PASS_INSTANTIATE(float, 256, 0)
SQK_PASS_INSTANTIATE(float, 256, sqk::PF_BULK)
SQK_PASS_INSTANTIATE(float, 256, sqk::PF_DENSE)
SQK_PASS_INSTANTIATE(float, 1024, 0)
SQK_PASS_INSTANTIATE(float, 1024, sqk::PF_DENSE)
