/*
 * ref_mex.cpp -- runs the reference's own CUDA kernels (TEST INFRASTRUCTURE ONLY).
 *
 * The reference's MEX crystal pass (toolbox/lib/MEXlib/src/OPO_CUDA_BATCH_XTAL.cu)
 * is device kernels plus a host driver, OPO_TEST_CUDA (:373-524), that needs
 * MATLAB's gpuArray glue.  The kernels are compiled, unmodified, from the
 * reference source into a cubin (oracle/Makefile, target `ref`, output in
 * oracle/_ref/); this file loads that cubin with the driver API and drives its
 * kernels -- NLFN_kernel, KN_kernel, Error_kernel, complex_ScaleVec,
 * Dispersion_kernel -- with cuFFT, in the order and with the argument values
 * OPO_TEST_CUDA uses.  The driver's control flow (step accept/reject, chunk
 * clamps, step growth) is restated here in the driver's own FP32 scalar
 * arithmetic; nothing of the reference's source is copied.
 *
 * Its results are the reference's FP32 arithmetic on the GPU (FP32 phase
 * argument, hypotf error norm, cuFFT), used by the tests to pin the FP64
 * oracle and the propagator to the reference's behaviour.  Only tests/ and
 * bench.py load it.  Optionally a decision sequence is forced (bit 0: above
 * maxErr, bit 1: above minErr per attempt) so that runs with a different
 * error norm can be compared on one step schedule; the reference's own flags
 * are still computed and recorded in the trace.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace {

constexpr int kThreads = 128;   // threadsPerBlock, OPO_CUDA_BATCH_XTAL.cu:14

std::string g_err;

struct Fn {
    const char* tag;
    CUfunction f;
};

bool set_err(const char* what, int code) {
    char b[256];
    std::snprintf(b, sizeof b, "%s failed (%d)", what, code);
    g_err = b;
    return false;
}

#define DRV(x) do { CUresult r_ = (x); if (r_ != CUDA_SUCCESS) { set_err(#x, (int)r_); goto fail; } } while (0)
#define RT(x) do { cudaError_t r_ = (x); if (r_ != cudaSuccess) { set_err(#x, (int)r_); goto fail; } } while (0)
#define FFT(x) do { cufftResult r_ = (x); if (r_ != CUFFT_SUCCESS) { set_err(#x, (int)r_); goto fail; } } while (0)

// Kernel handles found by name in the module (the cubin keeps C++ mangled names).
bool find_kernels(CUmodule mod, Fn* fns, int n) {
    unsigned count = 0;
    if (cuModuleGetFunctionCount(&count, mod) != CUDA_SUCCESS || count == 0) return set_err("cuModuleGetFunctionCount", 0);
    std::vector<CUfunction> all(count);
    if (cuModuleEnumerateFunctions(all.data(), count, mod) != CUDA_SUCCESS) return set_err("cuModuleEnumerateFunctions", 0);
    for (int i = 0; i < n; ++i) {
        fns[i].f = nullptr;
        for (unsigned j = 0; j < count; ++j) {
            const char* name = nullptr;
            if (cuFuncGetName(&name, all[j]) != CUDA_SUCCESS || !name) continue;
            if (std::strstr(name, fns[i].tag)) { fns[i].f = all[j]; break; }
        }
        if (!fns[i].f) { g_err = std::string("kernel not in cubin: ") + fns[i].tag; return false; }
    }
    return true;
}

bool launch(CUfunction f, int N, int B, void** args, int threads = kThreads) {
    const unsigned gx = (unsigned)((N + threads - 1) / threads);
    CUresult r = cuLaunchKernel(f, gx, (unsigned)B, 1, (unsigned)threads, 1, 1, 0, nullptr, args, nullptr);
    if (r != CUDA_SUCCESS) return set_err("cuLaunchKernel", (int)r);
    return true;
}

}  // namespace

extern "C" {

const char* refmex_last_error() { return g_err.c_str(); }

/*
 * One MEX crystal pass (OPO_mex_BATCH.cpp:41-122 + OPO_CUDA_BATCH_XTAL.cu:373-524)
 * on B pulses of N points.  variant selects the driver of the cubin passed:
 *   0 BATCH_XTAL  (G row per pulse: KN_kernel takes Nsteps, :195-252; float sel,
 *                  chunk count rounded up, k < Nsteps guard, absorber 6N/16..10N/16)
 *   1 BATCH_OP    (OPO_CUDA_BATCH_OP.cu:372-520: as XTAL with one shared G,
 *                  KN_kernel without Nsteps, :197-221)
 *   2 NO_BC       (OPO_CUDA_NO_BC.cu:364-510: int sel, truncated chunk count (:397),
 *                  no guard, absorber range empty (:401-402))
 *   3 HARD_BC     (OPO_CUDA_HARD_BC.cu:365-509: as NO_BC with the absorber range
 *                  of XTAL (:400-401); its complex_ScaleVec zeroes it, :105-129)
 * The time convention and the absorber's shape are inside each file's kernels.
 * Host arrays:
 *   E[B*N] (float2 as interleaved floats), alpha[N], G[S*B], beta[N] -- the
 *   MEX inputs 0, 1, 2, 8;  Ap[nchunks*N*B] and stepmods[S] are in/out
 *   (inputs 12 and 13, copied in and returned as the reference does);
 *   A_out[B*N] receives output 0.
 * trace (optional, 3 ints per attempt: k, stepmod, flags | 8 when accepted),
 * forced (optional decisions), seconds (wall time of the pass on the device).
 * Returns 0, or -1 with refmex_last_error() set.
 */
int refmex_run(const char* cubin, int variant, const float* E, int N, int B, const float* alpha, const float* G,
               const float* beta, float w0, double bdiffw0, float h, int S, double dt,
               float max_pct_err, float min_pct_err, float sel, float* Ap, long long ap_len,
               float* stepmods, float* A_out, int* trace, int trace_cap, int* n_attempts,
               const int* forced, int n_forced, double* seconds) {
    g_err.clear();
    if (N < kThreads || N % kThreads != 0 || B < 1 || S < 1 || !(sel > 0.f))
        return set_err("refmex_run: N must be a multiple of 128 (KN_kernel has no bounds guard), B, S, sel > 0", 0), -1;

    if (variant < 0 || variant > 3) return set_err("refmex_run: variant must be 0..3", variant), -1;
    const bool g_rows = (variant == 0);              // KN_kernel(..., Nsteps, ...) and G[k + row S]
    const bool int_sel = (variant >= 2);             // int sel, truncated chunks, no k < Nsteps guard
    if (int_sel) sel = (float)(int)sel;
    if (!(sel >= 1.f)) return set_err("refmex_run: sel < 1", 0), -1;
    // chunk count as each driver computes it (XTAL :403-407; NO_BC :397)
    int nchunks = (int)((float)S / sel);
    if (int_sel) nchunks = S / (int)sel;
    else if ((float)nchunks * sel < (float)S) nchunks += 1;
    if (ap_len < (long long)nchunks * N * B * 2)
        return set_err("refmex_run: Ap holds fewer than nchunks*N*B complex values", nchunks), -1;

    const size_t fb = sizeof(float) * 2 * (size_t)N * B;
    const size_t g_len = g_rows ? (size_t)S * B : (size_t)S;
    CUmodule mod = nullptr;
    cufftHandle plan = 0;
    bool have_plan = false;
    float2 *dE = nullptr, *dA0 = nullptr, *dA1 = nullptr, *dNL = nullptr, *dK1 = nullptr, *dK2 = nullptr, *dAp = nullptr;
    float *dG = nullptr, *dal = nullptr, *dbe = nullptr, *dsm = nullptr;
    bool* dflag = nullptr;
    Fn fns[5] = {{"NLFN_kernel", nullptr}, {"KN_kernel", nullptr}, {"Error_kernel", nullptr},
                 {"complex_ScaleVec", nullptr}, {"Dispersion_kernel", nullptr}};
    int rc = -1;
    int attempt = 0;
    std::chrono::steady_clock::time_point t0, t1;

    RT(cudaFree(nullptr));                           // bind the runtime's primary context
    DRV(cuModuleLoad(&mod, cubin));
    if (!find_kernels(mod, fns, 5)) goto fail;

    RT(cudaMalloc(&dE, fb)); RT(cudaMalloc(&dA0, fb)); RT(cudaMalloc(&dA1, fb));
    RT(cudaMalloc(&dNL, fb)); RT(cudaMalloc(&dK1, fb)); RT(cudaMalloc(&dK2, fb));
    RT(cudaMalloc(&dG, sizeof(float) * g_len));
    RT(cudaMalloc(&dal, sizeof(float) * N)); RT(cudaMalloc(&dbe, sizeof(float) * N));
    RT(cudaMalloc(&dAp, sizeof(float) * (size_t)ap_len));
    RT(cudaMalloc(&dsm, sizeof(float) * (size_t)S));
    RT(cudaMalloc(&dflag, 2));
    // E and A0 both start as copies of the input (OPO_mex_BATCH.cpp:41,86)
    RT(cudaMemcpy(dE, E, fb, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dA0, E, fb, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dG, G, sizeof(float) * g_len, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dal, alpha, sizeof(float) * N, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dbe, beta, sizeof(float) * N, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dAp, Ap, sizeof(float) * (size_t)ap_len, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dsm, stepmods, sizeof(float) * (size_t)S, cudaMemcpyHostToDevice));
    FFT(cufftPlan1d(&plan, N, CUFFT_C2C, B));
    have_plan = true;
    RT(cudaDeviceSynchronize());

    {
        // FP32 driver scalars, as declared in OPO_TEST_CUDA (:395-407)
        const float invdt2 = (float)(1.0 / (2.0 * dt));
        const float invSize = (float)(1.0 / N);
        const int gi1 = (variant == 2) ? 0 : (int)(6.0 * (N / 16));
        const int gi2 = (variant == 2) ? 0 : (int)(10.0 * (N / 16));
        const float one = 1.0f, half = 0.5f;
        float k = 0.f, stepprev = 4.f, stepmod = 4.f, hmod = 0.f;
        const long long max_attempts = 64LL * S + 1024;
        t0 = std::chrono::steady_clock::now();
        for (int chunk = 0; chunk < nchunks; ++chunk) {
            stepmod = stepprev;
            hmod = stepmod * h;
            for (; k < (float)(chunk + 1) * sel && (int_sel || k < (float)S); k = k + stepmod) {
                if (attempt >= max_attempts) { set_err("refmex_run: attempt limit", attempt); goto fail; }
                const int ki = (int)k, si = (int)stepmod;
                // stage 1 at z = k h, stage 2 at z = (k + stepmod) h (:431-446)
                double bdwz = bdiffw0 * (double)k * (double)h;
                {
                    void* a1[] = {&dNL, &dA0, &dA0, (void*)&dt, &w0, &bdwz, &N};
                    if (!launch(fns[0].f, N, B, a1)) goto fail;
                    int Sv = S;
                    void* a2[] = {&dA0, &dK1, &dK1, &dNL, &dG, &w0, &hmod, (void*)&ki, (void*)&invdt2,
                                  &N, &Sv, &dA1, (void*)&half};
                    void* a2s[] = {&dA0, &dK1, &dK1, &dNL, &dG, &w0, &hmod, (void*)&ki, (void*)&invdt2,
                                   &N, &dA1, (void*)&half};
                    if (!launch(fns[1].f, N, B, g_rows ? a2 : a2s)) goto fail;
                    bdwz = bdiffw0 * (double)(k + stepmod) * (double)h;
                    void* a3[] = {&dNL, &dA1, &dA1, (void*)&dt, &w0, &bdwz, &N};
                    if (!launch(fns[0].f, N, B, a3)) goto fail;
                    void* a4[] = {&dA0, &dK2, &dK1, &dNL, &dG, &w0, &hmod, (void*)&ki, (void*)&invdt2,
                                  &N, &Sv, &dE, (void*)&half};
                    void* a4s[] = {&dA0, &dK2, &dK1, &dNL, &dG, &w0, &hmod, (void*)&ki, (void*)&invdt2,
                                   &N, &dE, (void*)&half};
                    if (!launch(fns[1].f, N, B, g_rows ? a4 : a4s)) goto fail;
                }
                RT(cudaDeviceSynchronize());
                RT(cudaMemset(dflag, 0, 2));
                {
                    void* a5[] = {&dA1, &dE, &dE, (void*)&ki, (void*)&si, &N, &max_pct_err, &min_pct_err, &dflag};
                    if (!launch(fns[2].f, N, B, a5)) goto fail;
                }
                RT(cudaDeviceSynchronize());
                bool hf[2] = {false, false};
                RT(cudaMemcpy(hf, dflag, 2, cudaMemcpyDeviceToHost));
                const int own = (hf[0] ? 1 : 0) | (hf[1] ? 2 : 0);
                const int fl = (forced && attempt < n_forced) ? (forced[attempt] & 3) : own;
                const bool reject = (fl & 1) && stepmod > 1.f && (k - stepmod) > 0.f;
                if (trace && attempt < trace_cap) {
                    trace[3 * attempt] = ki;
                    trace[3 * attempt + 1] = si;
                    trace[3 * attempt + 2] = fl | (reject ? 0 : 8) | (own << 4);
                }
                ++attempt;
                if (reject) {
                    // the loop increment then adds the new stepmod: net k - 1 (:460-466)
                    k = k - stepmod;
                    stepmod = stepmod - 1.f;
                    hmod = stepmod * h;
                    stepprev = stepmod;
                    continue;
                }
                // accepted: absorber, FFT, dispersion (+ Ap, stepmods), IFFT, 1/N (:469-485)
                {
                    void* a6[] = {&dE, (void*)&one, &N, (void*)&gi1, (void*)&gi2};
                    if (!launch(fns[3].f, N, B, a6)) goto fail;
                }
                FFT(cufftExecC2C(plan, (cufftComplex*)dE, (cufftComplex*)dE, CUFFT_FORWARD));
                {
                    int nc = nchunks;
                    void* a7[] = {&dAp, &dE, &dal, &dbe, &N, (void*)&si, &chunk, &nc, &dsm, (void*)&ki};
                    if (!launch(fns[4].f, N, B, a7)) goto fail;
                }
                FFT(cufftExecC2C(plan, (cufftComplex*)dE, (cufftComplex*)dA0, CUFFT_INVERSE));
                {
                    int z0 = 0;
                    void* a8[] = {&dA0, (void*)&invSize, &N, &z0, &z0};
                    if (!launch(fns[3].f, N, B, a8)) goto fail;
                }
                // step control (:487-506)
                const float cend = (float)(chunk + 1) * sel;
                if (k + stepmod >= cend && k < cend - 1.f) {
                    const float stepend = (cend - k) - 1.f;
                    hmod = stepend * h;
                    stepprev = stepmod;
                    stepmod = stepend;
                } else {
                    if (!(fl & 2) && !(fl & 1) && (k + stepmod + 1.f) < cend - 1.f) {
                        stepmod = stepmod + 1.f;
                        hmod = stepmod * h;
                    }
                    stepprev = stepmod;
                }
            }
            RT(cudaDeviceSynchronize());
        }
        RT(cudaDeviceSynchronize());
        t1 = std::chrono::steady_clock::now();
    }
    RT(cudaMemcpy(A_out, dA0, fb, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(Ap, dAp, sizeof(float) * (size_t)ap_len, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(stepmods, dsm, sizeof(float) * (size_t)S, cudaMemcpyDeviceToHost));
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    rc = 0;
fail:
    if (n_attempts) *n_attempts = attempt;
    if (have_plan) cufftDestroy(plan);
    cudaFree(dE); cudaFree(dA0); cudaFree(dA1); cudaFree(dNL); cudaFree(dK1); cudaFree(dK2);
    cudaFree(dG); cudaFree(dal); cudaFree(dbe); cudaFree(dAp); cudaFree(dsm); cudaFree(dflag);
    if (mod) cuModuleUnload(mod);
    return rc;
}

/*
 * One ODE23 crystal pass (ode23/OPO_mex_ode23.cpp + ode23/OPO_CUDA_ODE23.cu:375-557):
 * Bogacki-Shampine 3(2) with the reference's own kernels (256 threads per block,
 * :15), FSAL K1 <- K4 swapped in after the dispersion sub-step, step doubling,
 * the K1 recomputation at z = k + stepmod after a reject, integer sel and a
 * truncated chunk count.  One pulse only: the reference's complex_AddVec
 * (:87-104) ignores the batch row, so its batched runs update only row 0.
 * Arguments as refmex_run (sel is converted to int as the gateway does).
 */
int refmex_run_ode23(const char* cubin, const float* E, int N, const float* alpha, const float* G,
                     const float* beta, float w0, double bdiffw0, float h, int S, double dt,
                     float max_pct_err, float min_pct_err, int sel, float* Ap, long long ap_len,
                     float* stepmods, float* A_out, int* trace, int trace_cap, int* n_attempts,
                     const int* forced, int n_forced, double* seconds) {
    g_err.clear();
    constexpr int T = 256;
    const int B = 1;
    if (N < T || N % T != 0 || S < 1 || sel < 1)
        return set_err("refmex_run_ode23: N must be a multiple of 256 (KN_kernel has no bounds guard), S, sel > 0", 0), -1;
    const int nchunks = S / sel;                      // truncated (:411)
    if (ap_len < (long long)nchunks * N * 2)
        return set_err("refmex_run_ode23: Ap holds fewer than nchunks*N complex values", nchunks), -1;

    const size_t fb = sizeof(float) * 2 * (size_t)N;
    CUmodule mod = nullptr;
    cufftHandle plan = 0;
    bool have_plan = false;
    float2 *dE = nullptr, *dA0 = nullptr, *dA1 = nullptr, *dNL = nullptr, *dK1 = nullptr, *dK2 = nullptr,
           *dK3 = nullptr, *dK4 = nullptr, *dAp = nullptr;
    float *dG = nullptr, *dal = nullptr, *dbe = nullptr, *dsm = nullptr;
    bool* dflag = nullptr;
    Fn fns[6] = {{"NLFN_kernel", nullptr}, {"KN_kernel", nullptr}, {"Error_kernel", nullptr},
                 {"complex_ScaleVec", nullptr}, {"Dispersion_kernel", nullptr}, {"complex_AddVec", nullptr}};
    int rc = -1;
    int attempt = 0;
    std::chrono::steady_clock::time_point t0, t1;

    RT(cudaFree(nullptr));
    DRV(cuModuleLoad(&mod, cubin));
    if (!find_kernels(mod, fns, 6)) goto fail;
    RT(cudaMalloc(&dE, fb)); RT(cudaMalloc(&dA0, fb)); RT(cudaMalloc(&dA1, fb)); RT(cudaMalloc(&dNL, fb));
    RT(cudaMalloc(&dK1, fb)); RT(cudaMalloc(&dK2, fb)); RT(cudaMalloc(&dK3, fb)); RT(cudaMalloc(&dK4, fb));
    RT(cudaMalloc(&dG, sizeof(float) * (size_t)S));
    RT(cudaMalloc(&dal, sizeof(float) * N)); RT(cudaMalloc(&dbe, sizeof(float) * N));
    RT(cudaMalloc(&dAp, sizeof(float) * (size_t)ap_len));
    RT(cudaMalloc(&dsm, sizeof(float) * (size_t)S));
    RT(cudaMalloc(&dflag, 2));
    RT(cudaMemcpy(dE, E, fb, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dA0, E, fb, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dG, G, sizeof(float) * (size_t)S, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dal, alpha, sizeof(float) * N, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dbe, beta, sizeof(float) * N, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dAp, Ap, sizeof(float) * (size_t)ap_len, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dsm, stepmods, sizeof(float) * (size_t)S, cudaMemcpyHostToDevice));
    FFT(cufftPlan1d(&plan, N, CUFFT_C2C, B));
    have_plan = true;
    RT(cudaDeviceSynchronize());
    {
        const float invdt2 = (float)(1.0 / (2.0 * dt));
        const float invSize = (float)(1.0 / N);
        const int gi1 = (int)(6.0 * (N / 16)), gi2 = (int)(10.0 * (N / 16));
        // Butcher coefficients as the driver's FP32 tables (:426-429)
        const float as[5] = {1.0f / 2.0f, 3.0f / 4.0f, 4.0f / 9.0f, 1.0f / 3.0f, 2.0f / 9.0f};
        const float bs[4] = {1.0f / 8.0f, 1.0f / 3.0f, 1.0f / 4.0f, 7.0f / 24.0f};
        const float one = 1.0f, zero = 0.0f;
        float k = 0.f, stepprev = 4.f, stepmod = 4.f, hmod;
        const long long max_attempts = 64LL * S + 1024;
        // stage helpers: NL at z = pos h of field X, then K = f(X), AN = A0 + b1 K + b2 K2
        auto nl = [&](float2* X, double bdwz) {
            void* a[] = {&dNL, &X, &X, (void*)&dt, &w0, &bdwz, &N};
            return launch(fns[0].f, N, B, a, T);
        };
        auto kn = [&](float2* K, float2* K2, float2* AN, int ki, float b1, float b2) {
            void* a[] = {&dA0, &K, &K2, &dNL, &dG, &w0, &hmod, &ki, (void*)&invdt2, &N, &AN, &b1, &b2};
            return launch(fns[1].f, N, B, a, T);
        };
        auto addv = [&](float2* A, float2* Bv, float2* Cv, float sc) {
            void* a[] = {&A, &Bv, &Cv, &sc, &N};
            return launch(fns[5].f, N, B, a, T);
        };
        t0 = std::chrono::steady_clock::now();
        // initial K1 at k = 0 with stepmod = 4 (:431-436)
        hmod = stepmod * h;
        if (!nl(dA0, bdiffw0 * (double)k * (double)h)) goto fail;
        if (!kn(dK1, dK1, dA1, (int)k, as[0], zero)) goto fail;
        for (int chunk = 0; chunk < nchunks; ++chunk) {
            stepmod = stepprev;
            hmod = stepmod * h;
            for (; k < (float)((chunk + 1) * sel); k = k + stepmod) {
                if (attempt >= max_attempts) { set_err("refmex_run_ode23: attempt limit", attempt); goto fail; }
                const int ki = (int)k, si = (int)stepmod;
                // K2 at k + s/2, K3 at k + 3s/4, E, K4 at k + s, A1 (:444-458)
                if (!nl(dA1, bdiffw0 * (double)(k + as[0] * stepmod) * (double)h)) goto fail;
                if (!kn(dK2, dK2, dA1, ki, as[1], zero)) goto fail;
                if (!nl(dA1, bdiffw0 * (double)(k + as[1] * stepmod) * (double)h)) goto fail;
                if (!kn(dK3, dK2, dE, ki, as[2], as[3])) goto fail;
                if (!addv(dE, dE, dK1, as[4])) goto fail;
                if (!nl(dE, bdiffw0 * (double)(k + stepmod) * (double)h)) goto fail;
                if (!kn(dK4, dK3, dA1, ki, bs[0], bs[1])) goto fail;
                if (!addv(dA1, dA1, dK2, bs[2])) goto fail;
                if (!addv(dA1, dA1, dK1, bs[3])) goto fail;
                RT(cudaDeviceSynchronize());
                RT(cudaMemset(dflag, 0, 2));
                {
                    void* a5[] = {&dA1, &dE, &dE, (void*)&ki, (void*)&si, &N, &max_pct_err, &min_pct_err, &dflag};
                    if (!launch(fns[2].f, N, B, a5, T)) goto fail;
                }
                RT(cudaDeviceSynchronize());
                bool hf[2] = {false, false};
                RT(cudaMemcpy(hf, dflag, 2, cudaMemcpyDeviceToHost));
                const int own = (hf[0] ? 1 : 0) | (hf[1] ? 2 : 0);
                const int fl = (forced && attempt < n_forced) ? (forced[attempt] & 3) : own;
                const bool reject = (fl & 1) && stepmod > 1.f && (k - stepmod) > 0.f;
                if (trace && attempt < trace_cap) {
                    trace[3 * attempt] = ki;
                    trace[3 * attempt + 1] = si;
                    trace[3 * attempt + 2] = fl | (reject ? 0 : 8) | (own << 4);
                }
                ++attempt;
                if (reject) {
                    // net k - 1; K1 recomputed at z = k + stepmod with G[k] (:466-476)
                    k = k - stepmod;
                    stepmod = stepmod - 1.f;
                    hmod = stepmod * h;
                    stepprev = stepmod;
                    if (!nl(dA0, bdiffw0 * (double)(k + stepmod) * (double)h)) goto fail;
                    if (!kn(dK1, dK1, dA1, (int)k, as[0], zero)) goto fail;
                    continue;
                }
                {
                    void* a6[] = {&dE, (void*)&one, &N, (void*)&gi1, (void*)&gi2};
                    if (!launch(fns[3].f, N, B, a6, T)) goto fail;
                }
                FFT(cufftExecC2C(plan, (cufftComplex*)dE, (cufftComplex*)dE, CUFFT_FORWARD));
                {
                    int nc = nchunks;
                    void* a7[] = {&dAp, &dE, &dal, &dbe, &N, (void*)&si, &chunk, &nc, &dsm, (void*)&ki};
                    if (!launch(fns[4].f, N, B, a7, T)) goto fail;
                }
                FFT(cufftExecC2C(plan, (cufftComplex*)dE, (cufftComplex*)dA0, CUFFT_INVERSE));
                {
                    int z0 = 0;
                    void* a8[] = {&dA0, (void*)&invSize, &N, &z0, &z0};
                    if (!launch(fns[3].f, N, B, a8, T)) goto fail;
                }
                std::swap(dK1, dK4);                        // FSAL (:494-496)
                RT(cudaDeviceSynchronize());
                if (!addv(dA1, dA0, dK1, as[0])) goto fail;
                // step control with doubling (:500-519)
                const int cend = (chunk + 1) * sel;
                if (k + stepmod >= (float)cend && k < (float)(cend - 1)) {
                    const float stepend = ((float)cend - k) - 1.f;
                    hmod = stepend * h;
                    stepprev = stepmod;
                    stepmod = stepend;
                } else {
                    if (!(fl & 2) && !(fl & 1) && (k + stepmod + stepmod) < (float)(cend - 1)) {
                        stepmod = stepmod * 2.f;
                        hmod = stepmod * h;
                    }
                    stepprev = stepmod;
                }
            }
            RT(cudaDeviceSynchronize());
        }
        RT(cudaDeviceSynchronize());
        t1 = std::chrono::steady_clock::now();
    }
    RT(cudaMemcpy(A_out, dA0, fb, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(Ap, dAp, sizeof(float) * (size_t)ap_len, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(stepmods, dsm, sizeof(float) * (size_t)S, cudaMemcpyDeviceToHost));
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    rc = 0;
fail:
    if (n_attempts) *n_attempts = attempt;
    if (have_plan) cufftDestroy(plan);
    cudaFree(dE); cudaFree(dA0); cudaFree(dA1); cudaFree(dNL); cudaFree(dK1); cudaFree(dK2);
    cudaFree(dK3); cudaFree(dK4); cudaFree(dG); cudaFree(dal); cudaFree(dbe); cudaFree(dAp);
    cudaFree(dsm); cudaFree(dflag);
    if (mod) cuModuleUnload(mod);
    return rc;
}

}  // extern "C"
