// Batched QMS kernel, float amplitudes, storage mode 2 (one translation unit
// per instantiation so they compile in parallel).
#include "sq_batch_dev.cuh"

namespace sqb {
template <>
const void* kernel_for<float, 2>() {
    return (const void*)&k_qms_tfim<float, 2>;
}
}  // namespace sqb
