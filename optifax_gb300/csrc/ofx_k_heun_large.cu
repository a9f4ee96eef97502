// Heun crystal-pass kernels with 4096 and 2048 points per CTA.
#include "ofx_kernels.cuh"
namespace ofx {
void register_kernels_heun_large(std::vector<KernelEntry>& v) {
    v.push_back(kernel_entry<4096, 1, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<4096, 2, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<4096, 4, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<4096, 8, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<4096, 16, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<2048, 1, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<2048, 2, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<2048, 4, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<2048, 8, OPTIFAX_HEUN>());
}
}  // namespace ofx
