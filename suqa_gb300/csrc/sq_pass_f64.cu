// Pass-kernel instantiations for FP64 states (FP64 arithmetic): multi-tile
// passes plain, with bulk staging, with dense blocks; single-tile passes plain
// and with dense blocks.
#define SQK_PASS_DEFINE
#include "sq_pass_host.cuh"

SQK_PASS_INSTANTIATE(double, 256, 0)
SQK_PASS_INSTANTIATE(double, 256, sqk::PF_BULK)
SQK_PASS_INSTANTIATE(double, 256, sqk::PF_DENSE)
SQK_PASS_INSTANTIATE(double, 1024, 0)
SQK_PASS_INSTANTIATE(double, 1024, sqk::PF_DENSE)
