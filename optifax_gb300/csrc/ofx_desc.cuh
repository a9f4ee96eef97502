// ofx_desc.cuh -- argument checks and descriptor fill shared by every entry
// point that launches the crystal-pass kernel (ofx_api.cu, ofx_noalloc.cu).
//
// One place decides which optifax_pulse is valid and how its fields become a
// PulseDev, so the handle-based and the allocation-free entry points accept and
// reject exactly the same arguments.
#pragma once
#include <cmath>
#include <cstring>
#include <string>

#include "ofx_pass.cuh"
#include "../../include/optifax.h"

namespace ofx {

// Conventions of each reference source variant (OPO_CUDA_BATCH_XTAL.cu,
// OPO_CUDA_BATCH_OP.cu, OPO_CUDA_NO_BC.cu, OPO_CUDA_HARD_BC.cu,
// ode23/OPO_CUDA_ODE23.cu, NEE_CPU.m).
struct VariantCfg { int time_mode, abc_mode, guard, g_per_pulse, stepmods_rule, nee = 0; };

inline bool variant_cfg(int variant, VariantCfg* v) {
    switch (variant) {
        case OPTIFAX_VARIANT_BATCH_XTAL: *v = {TIME_SHIFTED, ABC_SOFT, 1, 1, 128}; return true;
        case OPTIFAX_VARIANT_BATCH_OP:   *v = {TIME_SHIFTED, ABC_SOFT, 1, 0, 128}; return true;
        case OPTIFAX_VARIANT_NO_BC:      *v = {TIME_UNSHIFTED, ABC_NONE, 0, 0, 128}; return true;
        case OPTIFAX_VARIANT_HARD_BC:    *v = {TIME_UNSHIFTED, ABC_HARD, 0, 0, 128}; return true;
        case OPTIFAX_VARIANT_ODE23:      *v = {TIME_UNSHIFTED, ABC_SOFT, 0, 0, 256}; return true;
        case OPTIFAX_VARIANT_NEE:        *v = {TIME_NEE, ABC_NEE, 0, 0, 128, 1}; return true;
        default: return false;
    }
}

inline bool is_pow2(long long x) { return x > 0 && (x & (x - 1)) == 0; }

// Dispersion_kernel records stepmods[k] in the thread with gx == k, gx in
// [0, gridDim.x * blockDim.x): ceil(N/128)*128 (BATCH kernels) or
// (N/256)*256 (ODE23, which launches N/256 blocks).
inline int stepmods_limit_for(int N, int rule) {
    return rule == 128 ? ((N + 127) / 128) * 128 : (N / 256) * 256;
}

inline int n_chunks_for(int S, float sel, int guard) {
    int nc = (int)((float)S / sel);
    if (guard && (float)nc * sel < (float)S) nc += 1;
    return nc;
}

// radians -> unsigned 64-bit fixed-point turns (2^64 = one turn)
inline uint64_t turns_fixed(long double radians) {
    long double tw = radians / (2.0L * 3.14159265358979323846264338327950288L);
    tw -= floorl(tw);                        // [0, 1)
    long double x = tw * 18446744073709551616.0L;
    if (x >= 18446744073709551615.0L) return 0;
    return (uint64_t)x;
}

// Validate one pulse and fill its kernel descriptor.  Returns OPTIFAX_OK, or an
// optifax_status with the reason in *why.
inline int fill_pulse_desc(const optifax_pulse& in, const VariantCfg& vc, PulseDev* d,
                           optifax_pulse_stats* stats, std::string* why) {
    auto bad = [&](const char* msg) { if (why) *why = msg; return (int)OPTIFAX_ERR_INVALID_ARGUMENT; };
    if (!is_pow2(in.n_points) || in.n_points < 512 || in.n_points > 65536)
        return bad("n_points must be a power of two in [512, 65536]");
    if (in.n_steps < 1) return bad("n_steps must be >= 1");
    if (!(in.sel >= 1.0f)) return bad("sel must be >= 1");
    if (!(in.h > 0.0f) || !(in.dt > 0.0) || !(in.w0 > 0.0f)) return bad("h, dt and w0 must be positive");
    if (!in.E_in || !in.A_out || !in.alpha || !in.beta || !in.G)
        return bad("E_in, A_out, alpha, beta and G are required");
    if ((in.trace && in.trace_cap < 0) || (in.forced && in.n_forced < 0)) return bad("negative trace/forced length");
    const long long n_att_bound = 64LL * (in.n_steps + 16) + 64;
    if (n_att_bound > 0x7fffffffLL || (long long)in.n_steps * 4 > (1LL << 24))
        return bad("n_steps too large (4*S must stay below 2^24)");
    memset(d, 0, sizeof(*d));
    d->E_in = (const float2*)in.E_in;
    d->A_out = (float2*)in.A_out;
    d->alpha = in.alpha;
    d->beta = in.beta;
    d->G = in.G;
    d->Ap = (float2*)in.Ap;
    d->stepmods = in.stepmods;
    d->trace = in.trace;
    d->forced = in.forced;
    d->stats = stats;
    d->bdiffw0 = in.bdiffw0;
    d->dt = in.dt;
    d->tau_theta = turns_fixed((long double)(double)in.w0 * (long double)in.dt);
    d->tau_z4 = turns_fixed((long double)in.bdiffw0 * (long double)(double)in.h / 4.0L);
    d->w0 = in.w0;
    d->h = in.h;
    d->max_err = in.max_err;
    d->min_err = in.min_err;
    d->sel = in.sel;
    float invdt2 = (float)(1.0 / (2.0 * in.dt));
    d->c_shock = invdt2 / in.w0;
    d->N = in.n_points;
    d->S = in.n_steps;
    d->nchunks = n_chunks_for(in.n_steps, in.sel, vc.guard);
    d->stepmods_limit = in.stepmods_limit > 0 ? in.stepmods_limit : stepmods_limit_for(in.n_points, vc.stepmods_rule);
    d->trace_cap = in.trace ? in.trace_cap : 0;
    d->n_forced = in.forced ? in.n_forced : 0;
    return OPTIFAX_OK;
}

}  // namespace ofx
