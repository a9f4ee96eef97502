// ofx_kernels.cuh -- registry of the compiled (cta_points, cluster, method)
// instantiations of the crystal-pass kernel.  Each ofx_k_*.cu translation
// unit instantiates a subset so the library builds in parallel.
#pragma once
#include <vector>
#include "ofx_pass.cuh"

namespace ofx {

typedef void (*KernelFn)(const PulseDev*, FftTables, KernelCfg);

struct KernelEntry { KernelFn fn; size_t smem; int M, C, method; };

template <int M, int C, int METH>
KernelEntry kernel_entry() {
    return KernelEntry{&pass_kernel<M, C, METH>, Smem<M, METH, C>::bytes, M, C, METH};
}

void register_kernels_heun_large(std::vector<KernelEntry>& v);
void register_kernels_heun_small(std::vector<KernelEntry>& v);
void register_kernels_rk23(std::vector<KernelEntry>& v);
void register_kernels_heun_nee(std::vector<KernelEntry>& v);

}  // namespace ofx
