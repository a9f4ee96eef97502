// ofx_gnlse.cuh -- the chi(3) fibre GNLSE kernel's descriptor and launcher
// (toolbox/lib/internal/main/gnlsefib.m; see ofx_gnlse.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "ofx_common.cuh"
#include "../../include/optifax.h"

namespace ofx {

// One pulse on the device (built from optifax_gnlse_pulse by the C ABI).
struct GnlseDev {
    const float2* A;          // input field, natural time order
    const double* B;          // dispersion per mode (rad/m), FFT order
    const float* W;           // shock weight per mode, FFT order
    const float2* RW;         // Raman response per mode, FFT order (nullptr: no Raman)
    float2* AT_out;           // n_saves x n
    float2* AW_out;           // n_saves x n
    long long* trace;         // 2 per attempt
    optifax_gnlse_stats* stats;
    float2* K;                // scratch: 8 x n (seven stage derivatives, then y_new; slot order)
    double gamma, fr, dT, alpha, length, rtol, atol;
    int n_saves, trace_cap, max_attempts, pad;
};

// Launches one CTA per pulse for M = n points in {512, 1024, 2048, 4096}.
// tw1/tw2: the pass-twiddle tables of the M-point FFT.
cudaError_t launch_gnlse(int M, const GnlseDev* d, int n_pulses, const Twiddle* tw1, const Twiddle* tw2,
                         cudaStream_t st);

}  // namespace ofx
