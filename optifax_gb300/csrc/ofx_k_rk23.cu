// RK23 (Bogacki-Shampine) crystal-pass kernels.
#include "ofx_kernels.cuh"
namespace ofx {
void register_kernels_rk23(std::vector<KernelEntry>& v) {
    v.push_back(kernel_entry<4096, 1, OPTIFAX_RK23>());
    v.push_back(kernel_entry<4096, 2, OPTIFAX_RK23>());
    v.push_back(kernel_entry<4096, 4, OPTIFAX_RK23>());
    v.push_back(kernel_entry<2048, 1, OPTIFAX_RK23>());
    v.push_back(kernel_entry<2048, 2, OPTIFAX_RK23>());
    v.push_back(kernel_entry<2048, 4, OPTIFAX_RK23>());
    v.push_back(kernel_entry<1024, 1, OPTIFAX_RK23>());
    v.push_back(kernel_entry<1024, 2, OPTIFAX_RK23>());
    v.push_back(kernel_entry<512, 1, OPTIFAX_RK23>());
    v.push_back(kernel_entry<512, 2, OPTIFAX_RK23>());
}
}  // namespace ofx
