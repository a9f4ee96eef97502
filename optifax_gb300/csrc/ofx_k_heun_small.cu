// Heun crystal-pass kernels with 1024 and 512 points per CTA.
#include "ofx_kernels.cuh"
namespace ofx {
void register_kernels_heun_small(std::vector<KernelEntry>& v) {
    v.push_back(kernel_entry<1024, 1, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<1024, 2, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<1024, 4, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<1024, 8, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<1024, 16, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<512, 1, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<512, 2, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<512, 4, OPTIFAX_HEUN>());
    v.push_back(kernel_entry<512, 8, OPTIFAX_HEUN>());
}
}  // namespace ofx
