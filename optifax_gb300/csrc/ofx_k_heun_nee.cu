// Heun crystal-pass kernels with NEE_CPU.m step control (variant NEE): grids up to
// 2^14 points (clusters of up to 4 CTAs of 4096 points).
#include "ofx_kernels.cuh"
namespace ofx {
void register_kernels_heun_nee(std::vector<KernelEntry>& v) {
    v.push_back(kernel_entry<4096, 1, kHeunNee>());
    v.push_back(kernel_entry<4096, 2, kHeunNee>());
    v.push_back(kernel_entry<4096, 4, kHeunNee>());
    v.push_back(kernel_entry<2048, 1, kHeunNee>());
    v.push_back(kernel_entry<2048, 2, kHeunNee>());
    v.push_back(kernel_entry<2048, 4, kHeunNee>());
    v.push_back(kernel_entry<1024, 1, kHeunNee>());
    v.push_back(kernel_entry<1024, 2, kHeunNee>());
    v.push_back(kernel_entry<512, 1, kHeunNee>());
    v.push_back(kernel_entry<512, 2, kHeunNee>());
}
}  // namespace ofx
