// ofx_passx_host.cuh -- host driver of the wide-state crystal pass (ofx_passx.cuh),
// shared by optifax_propagate_fp64 (R = double, ofx_fp64.cu) and
// optifax_propagate_f32x2 (R = float-float, ofx_f32x2.cu).
//
// Interface of both entries: the reference's MEX argument list with double
// arrays (E N x B complex, alpha and beta N, G S or S x B), every pulse of the
// call on one adaptive step schedule (the reference's batch rule, error flags
// OR-ed over the batch through a grid barrier of a cooperative launch), the
// trace and statistics of the schedule returned on the host.  Calls on one
// device are serialised; each call synchronises its stream before returning.
#pragma once
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "ofx_desc.cuh"
#include "ofx_passx.cuh"
#include "../../include/optifax.h"

namespace ofx {

template <typename R>
struct XKernel {
    void (*fn)(const PulseX*, XTables<R>, KernelCfg);
    size_t smem;
    int M, C;
    bool nee;
};

template <typename R, int M, int C, bool NEE>
XKernel<R> xkernel() {
    return XKernel<R>{&passx_kernel<R, M, C, NEE>, SmemX<R, M>::bytes, M, C, NEE};
}

// W_N^e for e < N in FP64, rounded to R
template <typename R>
__global__ void passx_twiddles(typename Num<R>::cplx* out, int n) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    double s, c;
    sincospi(-2.0 * (double)e / (double)n, &s, &c);
    out[e] = Num<R>::from(make_double2(c, s));
}

// points per CTA: clusters of up to 16 CTAs, at most 1024 points per CTA below
// 2^15 points (the FP64 rate bounds this kernel, so more SMs per pulse pay).
// Float-float spreads further up to 2^12 points, 512 per CTA (GB300, 0.3 mm pass:
// 2^11 13.6 against 18.6 us per attempt, 2^12 16.3 against 19.3); at 2^13, 16 CTAs
// of 512 points lose to 8 of 1024 (26.6 against 21.7 us), and 2048 or 4096 points
// per CTA lose at every size (2^14: 50.1 and 90.6 against 38.6 us).
template <typename R>
inline int passx_cta_points(int n) {
    int m = n < 1024 ? n : 1024;
    if (std::is_same<R, ff>::value && n <= 4096) m = n < 512 ? n : 512;
    if (n / m > 16) m = n / 16;
    return m;
}

template <typename R>
struct XWork {
    int n_tab = 0;
    typename Num<R>::cplx* tab = nullptr;
    void* cph = nullptr;
    size_t cph_bytes = 0;
    double* abc = nullptr;
    size_t abc_bytes = 0;
    void* ztab = nullptr;
    size_t ztab_bytes = 0;
    PulseX* desc = nullptr;
    size_t desc_n = 0;
    int* trace = nullptr;
    size_t trace_n = 0;
    optifax_pulse_stats* stats = nullptr;
    int* flags = nullptr;
};

template <typename T>
inline int grow_dev(T** p, size_t* have, size_t need_bytes) {
    if (*p && *have >= need_bytes) return OPTIFAX_OK;
    if (*p) { cudaFree(*p); *p = nullptr; *have = 0; }
    if (cudaMalloc((void**)p, need_bytes) != cudaSuccess) return OPTIFAX_ERR_NO_MEMORY;
    *have = need_bytes;
    return OPTIFAX_OK;
}

template <typename R>
int passx_run(const std::vector<XKernel<R>>& kernels, XWork<R>& w, int n, int B, int S, const double* E_in,
              double* A_out, const double* alpha, const double* beta, const double* G, int g_per_pulse,
              double w0, double bdiffw0, double step_h, double dt, double max_err, double min_err, double sel,
              int variant, int32_t* trace_host, int32_t trace_cap, optifax_pulse_stats* stats_host,
              cudaStream_t st) {
    if (!is_pow2(n) || n < 512 || n > 65536 || B < 1 || S < 1 || !(sel >= 1.0) || !E_in || !A_out || !alpha ||
        !beta || !G || !(step_h > 0.0) || !(dt > 0.0) || !(w0 > 0.0) || (trace_host && trace_cap < 0))
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    if (64LL * (S + 16) + 64 > 0x7fffffffLL) return OPTIFAX_ERR_INVALID_ARGUMENT;
    VariantCfg vc;
    if (variant == OPTIFAX_VARIANT_ODE23 || !variant_cfg(variant, &vc)) return OPTIFAX_ERR_INVALID_ARGUMENT;
    const int M = passx_cta_points<R>(n), C = n / M;
    const XKernel<R>* ke = nullptr;
    for (const auto& k : kernels)
        if (k.M == M && k.C == C && k.nee == (vc.nee != 0)) ke = &k;
    if (!ke) return OPTIFAX_ERR_UNSUPPORTED;
    if (B > 1 && B * C > 148) return OPTIFAX_ERR_UNSUPPORTED;   // one co-resident wave (cooperative launch)

    int rc;
    using cplx = typename Num<R>::cplx;
    if (w.n_tab != n) {
        size_t have = w.tab ? sizeof(cplx) * (size_t)w.n_tab : 0;
        if ((rc = grow_dev(&w.tab, &have, sizeof(cplx) * (size_t)n))) { w.n_tab = 0; return rc; }
        passx_twiddles<R><<<(n + 255) / 256, 256, 0, st>>>(w.tab, n);
        if (cudaGetLastError() != cudaSuccess) { w.n_tab = 0; return OPTIFAX_ERR_CUDA; }
        w.n_tab = n;
    }
    if ((rc = grow_dev(&w.cph, &w.cph_bytes, sizeof(cplx) * (size_t)n * B))) return rc;
    if ((rc = grow_dev(&w.abc, &w.abc_bytes, sizeof(double) * (size_t)n * B))) return rc;
    const int zcap = S + 64;     // z-samples k + stepmod of a pass stay below S + stepmod's clamp
    if ((rc = grow_dev(&w.ztab, &w.ztab_bytes, sizeof(cplx) * (size_t)zcap * B))) return rc;
    size_t dn = w.desc_n * sizeof(PulseX);
    if ((rc = grow_dev(&w.desc, &dn, sizeof(PulseX) * (size_t)B))) return rc;
    w.desc_n = dn / sizeof(PulseX);
    const size_t tcap = trace_host ? (size_t)trace_cap : 0;
    size_t tn = w.trace_n * 3 * sizeof(int);
    if (tcap && (rc = grow_dev(&w.trace, &tn, 3 * sizeof(int) * tcap))) return rc;
    if (tcap) w.trace_n = tn / (3 * sizeof(int));
    size_t sb = w.stats ? sizeof(optifax_pulse_stats) : 0;
    if ((rc = grow_dev(&w.stats, &sb, sizeof(optifax_pulse_stats)))) return rc;
    size_t fb = w.flags ? 4 * sizeof(int) : 0;
    if ((rc = grow_dev(&w.flags, &fb, 4 * sizeof(int)))) return rc;

    std::vector<PulseX> d((size_t)B);
    int nchunks = (int)((double)S / sel);
    if (vc.guard && (double)nchunks * sel < (double)S) nchunks += 1;
    for (int b = 0; b < B; ++b) {
        PulseX& x = d[(size_t)b];
        memset(&x, 0, sizeof(x));
        x.E_in = reinterpret_cast<const double2*>(E_in) + (size_t)b * n;
        x.A_out = reinterpret_cast<double2*>(A_out) + (size_t)b * n;
        x.alpha = alpha;
        x.beta = beta;
        x.G = G + (g_per_pulse ? (size_t)b * S : 0);
        x.trace = (b == 0 && tcap) ? w.trace : nullptr;
        x.trace_cap = (b == 0) ? (int)tcap : 0;
        x.stats = (b == 0) ? w.stats : nullptr;
        x.cph = reinterpret_cast<cplx*>(w.cph) + (size_t)b * n;
        x.abc = w.abc + (size_t)b * n;
        x.ztab = reinterpret_cast<cplx*>(w.ztab) + (size_t)b * zcap;
        x.zcap = zcap;
        x.tau_theta = turns_fixed((long double)w0 * (long double)dt);
        x.tau_z = turns_fixed((long double)bdiffw0 * (long double)step_h);
        x.w0 = w0; x.h = step_h; x.dt = dt;
        x.max_err = max_err; x.min_err = min_err; x.sel = sel;
        x.c_shock = 1.0 / (2.0 * dt * w0);
        x.N = n; x.S = S; x.nchunks = nchunks;
    }
    if (cudaMemcpyAsync(w.desc, d.data(), sizeof(PulseX) * (size_t)B, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(w.flags, 0, 4 * sizeof(int), st) != cudaSuccess ||
        cudaMemsetAsync(w.stats, 0, sizeof(optifax_pulse_stats), st) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    if (cudaFuncSetAttribute(ke->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ke->smem) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    if (C > 8 && cudaFuncSetAttribute(ke->fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    KernelCfg cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.time_mode = vc.time_mode;
    cfg.abc_mode = vc.abc_mode;
    cfg.guard = vc.guard;
    cfg.shared_sched = B > 1 ? 1 : 0;
    cfg.max_attempts_mul = 64;
    cfg.grid_flags = w.flags;
    XTables<R> tabs;
    tabs.wn = w.tab;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)(B * C), 1, 1);
    lc.blockDim = dim3(kXThreads, 1, 1);
    lc.dynamicSmemBytes = ke->smem;
    lc.stream = st;
    cudaLaunchAttribute attrs[2];
    int na = 0;
    attrs[na].id = cudaLaunchAttributeClusterDimension;
    attrs[na].val.clusterDim.x = C; attrs[na].val.clusterDim.y = 1; attrs[na].val.clusterDim.z = 1;
    ++na;
    if (B > 1) {
        attrs[na].id = cudaLaunchAttributeCooperative;
        attrs[na].val.cooperative = 1;
        ++na;
    }
    lc.attrs = attrs;
    lc.numAttrs = na;
    const PulseX* dd = w.desc;
    if (cudaLaunchKernelEx(&lc, ke->fn, dd, tabs, cfg) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    optifax_pulse_stats hs;
    if (cudaMemcpyAsync(&hs, w.stats, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    if (tcap) {
        const size_t nt = (size_t)(hs.attempts < trace_cap ? hs.attempts : trace_cap);
        if (nt && cudaMemcpy(trace_host, w.trace, 3 * sizeof(int) * nt, cudaMemcpyDeviceToHost) != cudaSuccess)
            return OPTIFAX_ERR_CUDA;
    }
    if (stats_host) *stats_host = hs;
    return OPTIFAX_OK;
}

}  // namespace ofx
