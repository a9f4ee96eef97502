// ofx_f32x2.cu -- the float-float crystal pass (compensated FP32 field state).
//
// The persistent crystal-pass kernel (ofx_passx.cuh) with the field, the stage
// sums, the nonlinear drive and every transform in float-float arithmetic
// (ofx_num.cuh: ~48-bit significands built from FP32 operations), step
// decisions in FP64 precision.  On GB300, whose FP64 rate is about 1/64 of its
// FP32 rate, this reaches FP64-level agreement on passes where the FP32 field's
// rounding, amplified by a large parametric gain, dominates the result (the
// 20 mm chirped-PPLN precision study), at a fraction of the FP64 kernel's time.
// Compiled with -fmad=false (see ofx_num.cuh).
#include <mutex>
#include <vector>

#include "ofx_passx_host.cuh"

using namespace ofx;

namespace {

const std::vector<XKernel<ff>>& ff_kernels() {
    static const std::vector<XKernel<ff>> v = {
        xkernel<ff, 512, 1, false>(),   xkernel<ff, 512, 2, false>(),   xkernel<ff, 512, 4, false>(),
        xkernel<ff, 512, 8, false>(),   xkernel<ff, 1024, 8, false>(),  xkernel<ff, 1024, 16, false>(),
        xkernel<ff, 2048, 16, false>(), xkernel<ff, 4096, 16, false>(),
    };
    return v;
}

XWork<ff> g_w[64];
std::mutex g_mu[64];

}  // namespace

extern "C" int optifax_propagate_f32x2(int32_t n_points, int32_t n_pulses, int32_t n_steps,
                                    const double* E_in, double* A_out, const double* alpha, const double* beta,
                                    const double* G, int32_t g_per_pulse, double w0, double bdiffw0,
                                    double step_h, double dt, double max_err, double min_err, double sel,
                                    int32_t variant, int32_t* trace_host, int32_t trace_cap,
                                    optifax_pulse_stats* stats_host, void* stream) {
    if (variant == OPTIFAX_VARIANT_NEE) return OPTIFAX_ERR_UNSUPPORTED;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return OPTIFAX_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu[dev]);
    return passx_run<ff>(ff_kernels(), g_w[dev], n_points, n_pulses, n_steps, E_in, A_out, alpha, beta, G,
                         g_per_pulse, w0, bdiffw0, step_h, dt, max_err, min_err, sel, variant, trace_host,
                         trace_cap, stats_host, (cudaStream_t)stream);
}
