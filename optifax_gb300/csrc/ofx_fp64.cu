// ofx_fp64.cu -- the plain full-FP64 crystal-pass solver on the GPU.
//
// The persistent crystal-pass kernel (ofx_passx.cuh) with every value in
// double precision: the same Heun schedule as the FP32 propagator and the
// reference driver (OPO_CUDA_BATCH_XTAL.cu:373-525 and its BATCH_OP / NO_BC /
// HARD_BC variants; NEE_CPU.m:1-122), one launch per pass, the field held on
// chip by a thread-block cluster of up to 16 CTAs.  It is the FP64 comparator
// of the FP32 propagator (the "plain FP64 solver" of the OPO speed-up, and the
// FP64 side of the precision study).  GB300's FP64 rate is a small fraction of
// its FP32 rate, so this kernel spreads each pulse over as many SMs as a
// cluster allows.
#include <mutex>
#include <vector>

#include "ofx_passx_host.cuh"

using namespace ofx;

namespace {

const std::vector<XKernel<double>>& fp64_kernels() {
    static const std::vector<XKernel<double>> v = {
        xkernel<double, 512, 1, false>(),   xkernel<double, 1024, 1, false>(),
        xkernel<double, 1024, 2, false>(),  xkernel<double, 1024, 4, false>(),
        xkernel<double, 1024, 8, false>(),  xkernel<double, 1024, 16, false>(),
        xkernel<double, 2048, 16, false>(), xkernel<double, 4096, 16, false>(),
        xkernel<double, 512, 1, true>(),    xkernel<double, 1024, 1, true>(),
        xkernel<double, 1024, 2, true>(),   xkernel<double, 1024, 4, true>(),
        xkernel<double, 1024, 8, true>(),   xkernel<double, 1024, 16, true>(),
    };
    return v;
}

XWork<double> g_w[64];        // per device
std::mutex g_mu[64];

}  // namespace

extern "C" int optifax_propagate_fp64(int32_t n_points, int32_t n_pulses, int32_t n_steps,
                                      const double* E_in, double* A_out, const double* alpha, const double* beta,
                                      const double* G, int32_t g_per_pulse, double w0, double bdiffw0,
                                      double step_h, double dt, double max_err, double min_err, double sel,
                                      int32_t variant, int32_t* trace_host, int32_t trace_cap,
                                      optifax_pulse_stats* stats_host, void* stream) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return OPTIFAX_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu[dev]);
    return passx_run<double>(fp64_kernels(), g_w[dev], n_points, n_pulses, n_steps, E_in, A_out, alpha, beta, G,
                             g_per_pulse, w0, bdiffw0, step_h, dt, max_err, min_err, sel, variant, trace_host,
                             trace_cap, stats_host, (cudaStream_t)stream);
}
