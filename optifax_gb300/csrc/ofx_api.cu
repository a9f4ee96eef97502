// ofx_api.cu -- C ABI (include/optifax.h): context, twiddle tables,
// descriptor staging, validation and launch of the crystal-pass kernels.
//
// Replaces the MEX gateway mexFunction (toolbox/lib/MEXlib/src/OPO_mex_BATCH.cpp:19-141)
// and the host driver OPO_TEST_CUDA (OPO_CUDA_BATCH_XTAL.cu:373-525,
// ode23/OPO_CUDA_ODE23.cu:375-557): instead of ~10 launches, two cuFFT calls
// and two device synchronisations per step, one launch runs every step of
// every pulse.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ofx_kernels.cuh"
#include "ofx_desc.cuh"
#include "ofx_gnlse.cuh"
#include "../../include/optifax.h"

using namespace ofx;

struct optifax_context {
    int device = 0;
    std::map<int, Twiddle*> tw;          // N -> W_N^i, i < 64 (cluster exchange)
    std::map<int, Twiddle*> quadtw;      // M -> W_M^y, y < M/4 (cluster exchange)
    std::map<int, Twiddle*> passtw;      // M -> pass-1 table [16][M/16] then pass-2 [16][M/256]
    PulseDev* d_desc = nullptr;
    size_t desc_cap = 0;
    float2* d_xch = nullptr;             // cluster exchange scratch
    size_t xch_cap = 0;                  // in complex values
    std::vector<cudaStream_t> side;      // streams for concurrent launch groups
    std::vector<cudaEvent_t> ev;         // fork/join events
    int* d_grid_flags = nullptr;
    ofx::GnlseDev* d_gnlse_desc = nullptr;   // GNLSE: descriptors and stage scratch
    size_t gnlse_desc_cap = 0;
    float2* d_gnlse_k = nullptr;
    size_t gnlse_k_cap = 0;                  // complex values
    cudaEvent_t done_ev = nullptr;           // end of the last call's work on the GPU
    bool done_pending = false;               // done_ev has been recorded
    std::string last_error;
};

namespace {

// out[e] = W_n^e = exp(-2 pi i e / n) for e < count, rounded to FP32, with
// d = 1/|w|^2 - 1 in FP64.  The cluster exchange's tables: the quarter period of
// W_M (count M/4) and W_N^i for i < 64.
__global__ void twiddle_kernel(Twiddle* out, int n, int count) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    double s, c;
    sincospi(-2.0 * (double)e / (double)n, &s, &c);
    float cf = (float)c, sf = (float)s;
    double m2 = (double)cf * (double)cf + (double)sf * (double)sf;
    Twiddle w;
    w.c = cf; w.s = sf; w.d = (float)(1.0 / m2 - 1.0); w.pad = 0.f;
    out[e] = w;
}

// outer twiddles of one FFT pass over blocks of length L with radix 16:
// out[r * (L/16) + off] = W_L^{off r}
__global__ void pass_twiddle_kernel(Twiddle* out, int L) {
    int lr = L / 16;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 16 * lr) return;
    int r = idx / lr, off = idx - r * lr;
    double s, c;
    sincospi(-2.0 * (double)(off * r) / (double)L, &s, &c);
    float cf = (float)c, sf = (float)s;
    double m2 = (double)cf * (double)cf + (double)sf * (double)sf;
    Twiddle w;
    w.c = cf; w.s = sf; w.d = (float)(1.0 / m2 - 1.0); w.pad = 0.f;
    out[idx] = w;
}

int fail(optifax_context* h, int code, const std::string& msg) {
    if (h) h->last_error = msg;
    return code;
}

int cuda_fail(optifax_context* h, cudaError_t e, const char* what) {
    return fail(h, OPTIFAX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Every call stages its descriptors into, and runs on, device scratch owned by the
// handle, so its work waits for the previous call's (done_ev).  On the previous
// call's own stream the wait adds nothing to stream order; it is made on every
// stream because a stream handle's value can be reused after the stream is destroyed.
int order_after_previous(optifax_context* h, cudaStream_t st) {
    if (!h->done_pending) return OPTIFAX_OK;
    cudaError_t e = cudaStreamWaitEvent(st, h->done_ev, 0);
    return e == cudaSuccess ? OPTIFAX_OK : cuda_fail(h, e, "cudaStreamWaitEvent(previous call)");
}

int mark_done(optifax_context* h, cudaStream_t st) {
    cudaError_t e = cudaEventRecord(h->done_ev, st);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventRecord(end of call)");
    h->done_pending = true;
    return OPTIFAX_OK;
}

// Grow a handle-owned scratch buffer in stream order: the old buffer goes back
// with cudaFreeAsync once the previous call's work is done (the stream waits on
// done_ev first), the new one comes from cudaMallocAsync on the same stream, so
// no other work on the device is waited for.
int grow_scratch(optifax_context* h, void** buf, size_t* cap_bytes, size_t need_bytes, cudaStream_t st,
                 const char* what) {
    if (*buf && need_bytes <= *cap_bytes) return OPTIFAX_OK;
    int rc = order_after_previous(h, st);
    if (rc) return rc;
    if (*buf) {
        cudaError_t e = cudaFreeAsync(*buf, st);
        if (e != cudaSuccess) return cuda_fail(h, e, what);
        *buf = nullptr;
        *cap_bytes = 0;
    }
    cudaError_t e = cudaMallocAsync(buf, need_bytes, st);
    if (e != cudaSuccess) { *buf = nullptr; return cuda_fail(h, e, what); }
    *cap_bytes = need_bytes;
    return OPTIFAX_OK;
}

// W_n^e for e < count, built once per (n, count) map and kept for the context
const Twiddle* get_table(optifax_context* h, std::map<int, Twiddle*>& cache, int n, int count,
                         cudaStream_t st, int* rc) {
    auto it = cache.find(n);
    if (it != cache.end()) return it->second;
    Twiddle* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(Twiddle) * (size_t)count);
    if (e != cudaSuccess) { *rc = cuda_fail(h, e, "cudaMalloc(twiddles)"); return nullptr; }
    twiddle_kernel<<<(count + 255) / 256, 256, 0, st>>>(d, n, count);
    e = cudaGetLastError();
    if (e != cudaSuccess) { cudaFree(d); *rc = cuda_fail(h, e, "twiddle_kernel"); return nullptr; }
    // tables are shared by every stream of the context: finish building them now
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { cudaFree(d); *rc = cuda_fail(h, e, "twiddle_kernel sync"); return nullptr; }
    cache[n] = d;
    return d;
}

const Twiddle* get_pass_twiddles(optifax_context* h, int M, cudaStream_t st, int* rc) {
    auto it = h->passtw.find(M);
    if (it != h->passtw.end()) return it->second;
    int n1 = M, n2 = 16 * (M / 256);
    Twiddle* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(Twiddle) * (size_t)(n1 + n2));
    if (e != cudaSuccess) { *rc = cuda_fail(h, e, "cudaMalloc(pass twiddles)"); return nullptr; }
    pass_twiddle_kernel<<<(n1 + 255) / 256, 256, 0, st>>>(d, M);
    pass_twiddle_kernel<<<(n2 + 255) / 256, 256, 0, st>>>(d + n1, M / 16);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { cudaFree(d); *rc = cuda_fail(h, e, "pass_twiddle_kernel"); return nullptr; }
    h->passtw[M] = d;
    return d;
}

const std::vector<KernelEntry>& kernel_table() {
    static const std::vector<KernelEntry> tbl = [] {
        std::vector<KernelEntry> v;
        register_kernels_heun_large(v);
        register_kernels_heun_small(v);
        register_kernels_rk23(v);
        register_kernels_heun_nee(v);
        return v;
    }();
    return tbl;
}

const KernelEntry* find_kernel(int M, int C, int method) {
    for (const auto& k : kernel_table())
        if (k.M == M && k.C == C && k.method == method) return &k;
    return nullptr;
}

int choose_M(int N, int cta_points) {
    if (cta_points > 0) return cta_points;
    return N <= 4096 ? N : 4096;
}

struct Group {
    int M, C;
    std::vector<PulseDev> d;
};

double pulse_cost(const PulseDev& d) {
    return (double)d.N * std::log2((double)d.N) * (double)d.S;
}

int ensure_sync_objects(optifax_context* h, size_t n_streams) {
    while (h->side.size() < n_streams) {
        cudaStream_t s_;
        cudaError_t e = cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamCreate");
        h->side.push_back(s_);
    }
    while (h->ev.size() < n_streams + 1) {
        cudaEvent_t e_;
        cudaError_t e = cudaEventCreateWithFlags(&e_, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventCreate");
        h->ev.push_back(e_);
    }
    return OPTIFAX_OK;
}

// Order the groups for launch (longest work first within a group; groups in order
// of their longest pulse, longest first: the block scheduler serves earlier
// launches first, so the critical path starts at once and large clusters find
// whole GPCs free only at the start) and return the exchange scratch they need
// (complex values).
size_t order_groups(std::vector<Group>& groups) {
    for (auto& g : groups) {
        std::stable_sort(g.d.begin(), g.d.end(),
                         [](const PulseDev& x, const PulseDev& y) { return pulse_cost(x) > pulse_cost(y); });
    }
    auto group_key = [](const Group& g) { return g.d.empty() ? 0.0 : pulse_cost(g.d.front()); };
    std::stable_sort(groups.begin(), groups.end(),
                     [&](const Group& x, const Group& y) { return group_key(x) > group_key(y); });
    size_t need_xch = 0;
    for (auto& g : groups) {
        if (g.C > 1) need_xch += g.d.size() * 2 * (size_t)g.M * g.C;
        for (const auto& d : g.d)
            if (d.fb) need_xch += (size_t)g.M * g.C;    // OPO: the trip's crystal output (cavity scratch)
    }
    return need_xch;
}

// Descriptors in launch order with their exchange scratch carved from xch.
std::vector<PulseDev> place_descriptors(std::vector<Group>& groups, float2* xch) {
    std::vector<PulseDev> all;
    size_t xoff = 0;
    for (auto& g : groups)
        for (auto& d : g.d) {
            if (g.C > 1) { d.xch = xch + xoff; xoff += 2 * (size_t)g.M * g.C; }
            if (d.fb) { d.xs = xch + xoff; xoff += (size_t)g.M * g.C; }
            all.push_back(d);
        }
    return all;
}

// The FFT tables of every group, built (once per context) before any launch:
// building one synchronises the stream, which must not happen between launches.
int group_tables(optifax_context* h, const std::vector<Group>& groups, cudaStream_t st, std::vector<FftTables>* tabv) {
    int rc = OPTIFAX_OK;
    tabv->assign(groups.size(), FftTables{});
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        const int M = groups[gi].M;
        const Twiddle* twp = get_pass_twiddles(h, M, st, &rc);
        if (!twp) return rc;
        (*tabv)[gi].tw1 = twp;
        (*tabv)[gi].tw2 = twp + M;
        (*tabv)[gi].quad = get_table(h, h->quadtw, M, M / 4, st, &rc);       // quarter period of W_M
        if (!(*tabv)[gi].quad) return rc;
        (*tabv)[gi].low = get_table(h, h->tw, M * groups[gi].C, 64, st, &rc);  // W_N^i, i < 64
        if (!(*tabv)[gi].low) return rc;
    }
    return rc;
}

// Kernel attributes of every group's kernel (dynamic shared memory, 16-CTA clusters);
// not stream work, so set before the launches (and outside any capture).
int group_attributes(optifax_context* h, const std::vector<Group>& groups, int method, const VariantCfg& vc) {
    for (const auto& g : groups) {
        const KernelEntry* ke = find_kernel(g.M, g.C, vc.nee ? kHeunNee : method);
        if (!ke) return fail(h, OPTIFAX_ERR_UNSUPPORTED,
                             "no kernel for cta_points=" + std::to_string(g.M) + " cluster=" + std::to_string(g.C));
        cudaError_t e = cudaFuncSetAttribute(ke->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ke->smem);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaFuncSetAttribute(smem)");
        if (g.C > 8) {
            e = cudaFuncSetAttribute(ke->fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            if (e != cudaSuccess) return cuda_fail(h, e, "cudaFuncSetAttribute(cluster 16)");
        }
    }
    return OPTIFAX_OK;
}

// One grid per (cta_points, cluster) group; groups after the first run on side
// streams forked from and joined back into `st`, so the block scheduler
// interleaves them: CTAs of a long group fill SMs as short ones end.
int enqueue_groups(optifax_context* h, const std::vector<Group>& groups, int method, const VariantCfg& vc,
                   bool shared, const PulseDev* d_desc, const std::vector<FftTables>& tabv, int* grid_flags,
                   cudaStream_t st, const std::vector<cudaStream_t>& side, const std::vector<cudaEvent_t>& ev) {
    cudaError_t e;
    if (groups.size() > 1) {
        e = cudaEventRecord(ev[0], st);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventRecord");
    }
    size_t off = 0;
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        const Group& g = groups[gi];
        const int M = g.M, C = g.C;
        const KernelEntry* ke = find_kernel(M, C, vc.nee ? kHeunNee : method);
        if (!ke) return fail(h, OPTIFAX_ERR_UNSUPPORTED,
                             "no kernel for cta_points=" + std::to_string(M) + " cluster=" + std::to_string(C));
        const FftTables tabs = tabv[gi];
        KernelCfg cfg;
        cfg.time_mode = vc.time_mode;
        cfg.abc_mode = vc.abc_mode;
        cfg.guard = vc.guard;
        cfg.shared_sched = shared ? 1 : 0;
        cfg.max_attempts_mul = 64;
        cfg.grid_flags = grid_flags;
        cudaStream_t ls = st;
        if (gi > 0) {
            ls = side[gi - 1];
            e = cudaStreamWaitEvent(ls, ev[0], 0);
            if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamWaitEvent(fork)");
        }
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3((unsigned)(g.d.size() * C), 1, 1);
        lc.blockDim = dim3(M / 16, 1, 1);
        lc.dynamicSmemBytes = ke->smem;
        lc.stream = ls;
        cudaLaunchAttribute attrs[2];
        int na = 0;
        attrs[na].id = cudaLaunchAttributeClusterDimension;
        attrs[na].val.clusterDim.x = C; attrs[na].val.clusterDim.y = 1; attrs[na].val.clusterDim.z = 1;
        ++na;
        if (shared) {
            attrs[na].id = cudaLaunchAttributeCooperative;
            attrs[na].val.cooperative = 1;
            ++na;
        }
        lc.attrs = attrs;
        lc.numAttrs = na;
        const PulseDev* dd = d_desc + off;
        e = cudaLaunchKernelEx(&lc, ke->fn, dd, tabs, cfg);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaLaunchKernelEx(pass_kernel)");
        if (gi > 0) {
            e = cudaEventRecord(ev[gi], ls);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev[gi], 0);
            if (e != cudaSuccess) return cuda_fail(h, e, "join side stream");
        }
        off += g.d.size();
    }
    return OPTIFAX_OK;
}

// Stage every group's descriptors into the handle's scratch and launch the groups.
int launch_groups(optifax_context* h, std::vector<Group>& groups, int method, const VariantCfg& vc,
                  bool shared, cudaStream_t st) {
    const size_t need_xch = order_groups(groups);
    if (need_xch > h->xch_cap) {
        size_t cap = h->xch_cap * sizeof(float2);
        int grc = grow_scratch(h, (void**)&h->d_xch, &cap, need_xch * sizeof(float2), st,
                               "cudaMallocAsync(exchange scratch)");
        h->xch_cap = cap / sizeof(float2);
        if (grc) return grc;
    }
    std::vector<PulseDev> all = place_descriptors(groups, h->d_xch);
    size_t nb = all.size() * sizeof(PulseDev);
    if (nb > h->desc_cap) {
        int grc = grow_scratch(h, (void**)&h->d_desc, &h->desc_cap, nb < 4096 ? 4096 : nb * 2, st,
                               "cudaMallocAsync(descriptors)");
        if (grc) return grc;
    }
    int rc = order_after_previous(h, st);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(h->d_desc, all.data(), nb, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemcpyAsync(descriptors)");
    if (shared) {
        e = cudaMemsetAsync(h->d_grid_flags, 0, 4 * sizeof(int), st);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemsetAsync(grid flags)");
    }
    rc = ensure_sync_objects(h, groups.size());
    if (rc) return rc;
    std::vector<FftTables> tabv;
    rc = group_tables(h, groups, st, &tabv);
    if (rc) return rc;
    rc = group_attributes(h, groups, method, vc);
    if (rc) return rc;
    rc = enqueue_groups(h, groups, method, vc, shared, h->d_desc, tabv, h->d_grid_flags, st, h->side, h->ev);
    if (rc) return rc;
    return mark_done(h, st);
}

int launch_group(optifax_context* h, const std::vector<PulseDev>& descs, int M, int C, int method,
                 const VariantCfg& vc, bool shared, cudaStream_t st) {
    std::vector<Group> groups(1);
    groups[0].M = M;
    groups[0].C = C;
    groups[0].d = descs;
    return launch_groups(h, groups, method, vc, shared, st);
}

int fill_desc(optifax_context* h, const optifax_pulse& in, const VariantCfg& vc, PulseDev* d,
              optifax_pulse_stats* stats) {
    std::string why;
    int rc = fill_pulse_desc(in, vc, d, stats, &why);
    return rc ? fail(h, rc, why) : OPTIFAX_OK;
}

}  // namespace

extern "C" {

int optifax_create(optifax_handle* out, int device) {
    if (!out) return OPTIFAX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= 0) return OPTIFAX_ERR_CUDA;
    if (device < 0 || device >= n) return OPTIFAX_ERR_INVALID_ARGUMENT;
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return OPTIFAX_ERR_CUDA;
    optifax_context* h = new (std::nothrow) optifax_context();
    if (!h) return OPTIFAX_ERR_NO_MEMORY;
    h->device = device;
    e = cudaMalloc(&h->d_grid_flags, 4 * sizeof(int));
    if (e != cudaSuccess) { delete h; return OPTIFAX_ERR_CUDA; }
    e = cudaEventCreateWithFlags(&h->done_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) { cudaFree(h->d_grid_flags); delete h; return OPTIFAX_ERR_CUDA; }
    *out = h;
    return OPTIFAX_OK;
}

int optifax_destroy(optifax_handle h) {
    if (!h) return OPTIFAX_ERR_NULL_HANDLE;
    cudaSetDevice(h->device);
    cudaDeviceSynchronize();
    for (auto& kv : h->tw) cudaFree(kv.second);
    for (auto& kv : h->passtw) cudaFree(kv.second);
    for (auto& kv : h->quadtw) cudaFree(kv.second);
    if (h->d_desc) cudaFree(h->d_desc);
    if (h->d_grid_flags) cudaFree(h->d_grid_flags);
    if (h->d_xch) cudaFree(h->d_xch);
    if (h->d_gnlse_desc) cudaFree(h->d_gnlse_desc);
    if (h->d_gnlse_k) cudaFree(h->d_gnlse_k);
    for (auto s_ : h->side) cudaStreamDestroy(s_);
    for (auto e_ : h->ev) cudaEventDestroy(e_);
    if (h->done_ev) cudaEventDestroy(h->done_ev);
    delete h;
    return OPTIFAX_OK;
}

const char* optifax_status_string(int status) {
    switch (status) {
        case OPTIFAX_OK: return "ok";
        case OPTIFAX_ERR_INVALID_ARGUMENT: return "invalid argument";
        case OPTIFAX_ERR_UNSUPPORTED: return "unsupported configuration";
        case OPTIFAX_ERR_CUDA: return "CUDA error";
        case OPTIFAX_ERR_NO_MEMORY: return "out of memory";
        case OPTIFAX_ERR_NULL_HANDLE: return "null handle";
        default: return "unknown status";
    }
}

const char* optifax_last_error(optifax_handle h) {
    return h ? h->last_error.c_str() : "null handle";
}

}  // extern "C"

namespace {

// Validation and grouping by (cta_points, cluster) shared by optifax_propagate and
// optifax_propagate_graph.
int propagate_groups(optifax_handle h, const optifax_pulse* pulses, int32_t n_pulses, int32_t method,
                     int32_t variant, int32_t cta_points, optifax_pulse_stats* stats, VariantCfg* vc,
                     std::vector<Group>* gv) {
    if (!pulses || n_pulses < 1) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "no pulses");
    if (method != OPTIFAX_HEUN && method != OPTIFAX_RK23)
        return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "unknown method");
    if (!variant_cfg(variant, vc)) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "unknown variant");
    if (vc->nee && method != OPTIFAX_HEUN)
        return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "the NEE variant is a Heun schedule (NEE_CPU.m)");
    if (cta_points != 0 && (!is_pow2(cta_points) || cta_points < 512 || cta_points > 4096))
        return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "cta_points must be 0 or a power of two in [512, 4096]");
    std::map<std::pair<int, int>, std::vector<PulseDev>> groups;
    for (int i = 0; i < n_pulses; ++i) {
        PulseDev d;
        int rc = fill_desc(h, pulses[i], *vc, &d, stats ? stats + i : nullptr);
        if (rc) return rc;
        int want = pulses[i].cta_points > 0 ? pulses[i].cta_points : cta_points;
        if (want != 0 && (!is_pow2(want) || want < 512 || want > 4096))
            return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "pulse cta_points must be 0 or a power of two in [512, 4096]");
        int M = choose_M(pulses[i].n_points, want);
        if (M > pulses[i].n_points) M = pulses[i].n_points;
        int C = pulses[i].n_points / M;
        if (C > 16) return fail(h, OPTIFAX_ERR_UNSUPPORTED, "n_points / cta_points exceeds 16");
        groups[{M, C}].push_back(d);
    }
    gv->clear();
    for (auto& g : groups) gv->push_back(Group{g.first.first, g.first.second, std::move(g.second)});
    return OPTIFAX_OK;
}

}  // namespace

struct optifax_graph_s {
    int device = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    PulseDev* d_desc = nullptr;
    float2* d_xch = nullptr;
    int kernels = 0;
};

extern "C" {

int optifax_propagate(optifax_handle h, const optifax_pulse* pulses, int32_t n_pulses,
                      int32_t method, int32_t variant, int32_t cta_points,
                      optifax_pulse_stats* stats, void* stream) {
    if (!h) return OPTIFAX_ERR_NULL_HANDLE;
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    VariantCfg vc;
    std::vector<Group> gv;
    int rc = propagate_groups(h, pulses, n_pulses, method, variant, cta_points, stats, &vc, &gv);
    if (rc) return rc;
    return launch_groups(h, gv, method, vc, false, (cudaStream_t)stream);
}

int optifax_graph_destroy(optifax_graph g) {
    if (!g) return OPTIFAX_ERR_INVALID_ARGUMENT;
    cudaSetDevice(g->device);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->d_desc) cudaFree(g->d_desc);       // synchronises with any launch still running
    if (g->d_xch) cudaFree(g->d_xch);
    delete g;
    return OPTIFAX_OK;
}

int optifax_propagate_graph(optifax_handle h, const optifax_pulse* pulses, int32_t n_pulses,
                            int32_t method, int32_t variant, int32_t cta_points,
                            optifax_pulse_stats* stats, optifax_graph* out) {
    if (!h) return OPTIFAX_ERR_NULL_HANDLE;
    if (!out) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "no output graph");
    *out = nullptr;
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    VariantCfg vc;
    std::vector<Group> gv;
    int rc = propagate_groups(h, pulses, n_pulses, method, variant, cta_points, stats, &vc, &gv);
    if (rc) return rc;
    optifax_graph g = new (std::nothrow) optifax_graph_s();
    if (!g) return fail(h, OPTIFAX_ERR_NO_MEMORY, "graph object");
    g->device = h->device;
    // the graph owns its descriptors and exchange scratch: later calls on the handle
    // neither move nor overwrite them
    const size_t need_xch = order_groups(gv);
    std::vector<PulseDev> all;
    cudaStream_t s0 = nullptr;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> ev;
    std::vector<FftTables> tabv;
    auto cleanup = [&](int code) {
        for (auto s_ : side) cudaStreamDestroy(s_);
        for (auto e_ : ev) cudaEventDestroy(e_);
        if (s0) cudaStreamDestroy(s0);
        if (code) optifax_graph_destroy(g);
        return code;
    };
    if ((e = cudaMalloc(&g->d_xch, (need_xch ? need_xch : 1) * sizeof(float2))) != cudaSuccess)
        return cleanup(cuda_fail(h, e, "cudaMalloc(graph exchange scratch)"));
    all = place_descriptors(gv, g->d_xch);
    if ((e = cudaMalloc(&g->d_desc, all.size() * sizeof(PulseDev))) != cudaSuccess)
        return cleanup(cuda_fail(h, e, "cudaMalloc(graph descriptors)"));
    if ((e = cudaMemcpy(g->d_desc, all.data(), all.size() * sizeof(PulseDev), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cleanup(cuda_fail(h, e, "cudaMemcpy(graph descriptors)"));
    if ((e = cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking)) != cudaSuccess)
        return cleanup(cuda_fail(h, e, "cudaStreamCreate"));
    for (size_t i = 0; i < gv.size(); ++i) {
        cudaStream_t s_;
        cudaEvent_t e_;
        if (i + 1 < gv.size()) {
            if ((e = cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking)) != cudaSuccess)
                return cleanup(cuda_fail(h, e, "cudaStreamCreate"));
            side.push_back(s_);
        }
        if ((e = cudaEventCreateWithFlags(&e_, cudaEventDisableTiming)) != cudaSuccess)
            return cleanup(cuda_fail(h, e, "cudaEventCreate"));
        ev.push_back(e_);
    }
    if ((rc = group_tables(h, gv, s0, &tabv))) return cleanup(rc);
    if ((rc = group_attributes(h, gv, method, vc))) return cleanup(rc);
    if ((e = cudaStreamSynchronize(s0)) != cudaSuccess) return cleanup(cuda_fail(h, e, "table build"));
    if ((e = cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return cleanup(cuda_fail(h, e, "cudaStreamBeginCapture"));
    rc = enqueue_groups(h, gv, method, vc, false, g->d_desc, tabv, h->d_grid_flags, s0, side, ev);
    e = cudaStreamEndCapture(s0, &g->graph);
    if (rc) return cleanup(rc);
    if (e != cudaSuccess) return cleanup(cuda_fail(h, e, "cudaStreamEndCapture"));
    if ((e = cudaGraphInstantiate(&g->exec, g->graph, 0)) != cudaSuccess)
        return cleanup(cuda_fail(h, e, "cudaGraphInstantiate"));
    g->kernels = (int)gv.size();
    *out = g;
    return cleanup(OPTIFAX_OK);
}

int optifax_graph_launch(optifax_graph g, void* stream) {
    if (!g || !g->exec) return OPTIFAX_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(g->device) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    return cudaGraphLaunch(g->exec, (cudaStream_t)stream) == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

int optifax_graph_kernels(optifax_graph g) { return g ? g->kernels : 0; }

int optifax_opo_run(optifax_handle h, const optifax_opo* cavities, int32_t n_cavities,
                    int32_t variant, int32_t cta_points, optifax_pulse_stats* stats, void* stream) {
    if (!h) return OPTIFAX_ERR_NULL_HANDLE;
    if (!cavities || n_cavities < 1) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "no cavities");
    VariantCfg vc;
    if (!variant_cfg(variant, &vc)) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "unknown variant");
    if (cta_points != 0 && (!is_pow2(cta_points) || cta_points < 512 || cta_points > 4096))
        return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "cta_points must be 0 or a power of two in [512, 4096]");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    std::map<std::pair<int, int>, std::vector<PulseDev>> groups;
    for (int i = 0; i < n_cavities; ++i) {
        const optifax_opo& cv = cavities[i];
        if (!cv.feedback || !cv.pump) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "feedback and pump are required");
        if (cv.n_trips < 1) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "n_trips must be >= 1");
        if (cv.n_tally < 0 || cv.n_tally > 4 || (cv.n_tally > 0 && !cv.tally_w))
            return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "n_tally must be 0..4 with tally_w");
        if (cv.steady_trips < 0 || cv.steady_tally < 0 || cv.steady_tally >= 4)
            return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "bad steady-state settings");
        PulseDev d;
        int rc = fill_desc(h, cv.pass, vc, &d, stats ? stats + i : nullptr);
        if (rc) return rc;
        d.fb = (const float2*)cv.feedback;
        d.pump = (const float2*)cv.pump;
        d.tally_w = cv.tally_w;
        d.trips = cv.trips;
        d.n_trips = cv.n_trips;
        d.n_tally = cv.n_tally;
        d.steady_trips = cv.steady_trips;
        d.steady_tally = cv.steady_tally;
        d.steady_tol = cv.steady_tol;
        d.hist = (float2*)cv.history;
        if (cv.n_esd < 0 || cv.n_esd > 4 || (cv.n_esd > 0 && (!cv.esd_w || !cv.esd)))
            return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "n_esd must be 0..4 with esd_w and esd");
        d.esd_w = cv.n_esd > 0 ? cv.esd_w : nullptr;
        d.esd = cv.n_esd > 0 ? cv.esd : nullptr;
        d.n_esd = cv.n_esd;
        d.smt = cv.stepmods_trips;
        int M = choose_M(cv.pass.n_points, cta_points);
        if (M > cv.pass.n_points) M = cv.pass.n_points;
        int C = cv.pass.n_points / M;
        if (C > 16) return fail(h, OPTIFAX_ERR_UNSUPPORTED, "n_points / cta_points exceeds 16");
        groups[{M, C}].push_back(d);
    }
    std::vector<Group> gv;
    for (auto& g : groups) gv.push_back(Group{g.first.first, g.first.second, std::move(g.second)});
    return launch_groups(h, gv, OPTIFAX_HEUN, vc, false, (cudaStream_t)stream);
}

int optifax_opo_mex_batch(optifax_handle h,
                          const void* E, const float* alpha_w, const float* G,
                          float w0, double bdiffw0, float step_h, int32_t n_steps, double dt,
                          const float* beta_op, float max_pct_err, float min_pct_err, float sel,
                          const void* Ap_in, const float* stepmods_in,
                          int32_t n_points, int32_t n_pulses, int32_t ap_chunks, int32_t variant,
                          void* A_out, void* Ap_out, float* stepmods_out, void* stream) {
    if (!h) return OPTIFAX_ERR_NULL_HANDLE;
    VariantCfg vc;
    if (!variant_cfg(variant, &vc)) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "unknown variant");
    if (n_pulses < 1) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "n_pulses must be >= 1");
    if (!Ap_out || !stepmods_out) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "Ap_out and stepmods_out are required");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    cudaStream_t st = (cudaStream_t)stream;
    int method = (variant == OPTIFAX_VARIANT_ODE23) ? OPTIFAX_RK23 : OPTIFAX_HEUN;
    int nchunks = n_chunks_for(n_steps, sel, vc.guard);
    if (nchunks > ap_chunks)
        return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "Ap has fewer chunks than ceil(n_steps/sel)");
    size_t n = (size_t)n_points;
    // outputs start as copies of the inputs (mxGPUCopyFromMxArray, OPO_mex_BATCH.cpp:55-56)
    if (Ap_in && Ap_in != Ap_out) {
        e = cudaMemcpyAsync(Ap_out, Ap_in, sizeof(float2) * n * (size_t)ap_chunks * (size_t)n_pulses,
                            cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(h, e, "copy Ap");
    }
    if (stepmods_in && stepmods_in != stepmods_out) {
        e = cudaMemcpyAsync(stepmods_out, stepmods_in, sizeof(float) * (size_t)n_steps,
                            cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(h, e, "copy stepmods");
    }
    std::vector<PulseDev> descs((size_t)n_pulses);
    for (int b = 0; b < n_pulses; ++b) {
        optifax_pulse p;
        memset(&p, 0, sizeof(p));
        p.n_points = n_points;
        p.n_steps = n_steps;
        p.E_in = (const float2*)E + n * b;
        p.A_out = (float2*)A_out + n * b;
        p.alpha = alpha_w;
        p.beta = beta_op;
        p.G = vc.g_per_pulse ? G + (size_t)n_steps * b : G;
        // reference layout: (b * Nchunks + chunk) * N + i (OPO_CUDA_BATCH_XTAL.cu:302)
        p.Ap = (float2*)Ap_out + (size_t)b * (size_t)nchunks * n;
        p.stepmods = stepmods_out;
        p.w0 = w0; p.h = step_h; p.bdiffw0 = bdiffw0; p.dt = dt;
        p.max_err = max_pct_err; p.min_err = min_pct_err; p.sel = sel;
        int rc = fill_desc(h, p, vc, &descs[b], nullptr);
        if (rc) return rc;
    }
    int M = choose_M(n_points, 0);
    int C = n_points / M;
    if (n_pulses * C > 148)
        return fail(h, OPTIFAX_ERR_UNSUPPORTED, "shared-schedule batch larger than one wave of SMs");
    return launch_group(h, descs, M, C, method, vc, n_pulses > 1, st);
}

}  // extern "C"

// chi(3) fibre GNLSE (gnlsefib.m): validation, scratch, descriptors, launch
extern "C" int optifax_gnlse(optifax_handle h, const optifax_gnlse_pulse* pulses, int32_t n_pulses,
                             void* stream) {
    if (!h) return OPTIFAX_ERR_NULL_HANDLE;
    if (!pulses || n_pulses < 1) return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "gnlse: no pulses");
    const int M = pulses[0].n_points, S = pulses[0].n_saves;
    if (M != 512 && M != 1024 && M != 2048 && M != 4096)
        return fail(h, OPTIFAX_ERR_UNSUPPORTED, "gnlse: n_points must be 512, 1024, 2048 or 4096");
    std::vector<GnlseDev> d((size_t)n_pulses);
    for (int i = 0; i < n_pulses; ++i) {
        const optifax_gnlse_pulse& p = pulses[i];
        if (p.n_points != M || p.n_saves != S)
            return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "gnlse: pulses of one call share n_points and n_saves");
        if (S < 2 || !p.A || !p.B || !p.W || !p.AT_out || !p.AW_out || !(p.length > 0.0) || !(p.dT > 0.0) ||
            !(p.rtol > 0.0) || !(p.atol > 0.0) || !std::isfinite(p.gamma) || !std::isfinite(p.alpha) ||
            !std::isfinite(p.fr) || (p.trace && p.trace_cap < 0))
            return fail(h, OPTIFAX_ERR_INVALID_ARGUMENT, "gnlse: pulse " + std::to_string(i) + " arguments");
        GnlseDev& g = d[(size_t)i];
        memset(&g, 0, sizeof(g));
        g.A = (const float2*)p.A;
        g.B = p.B;
        g.W = p.W;
        g.RW = (p.RW && p.fr != 0.0) ? (const float2*)p.RW : nullptr;
        g.AT_out = (float2*)p.AT_out;
        g.AW_out = (float2*)p.AW_out;
        g.trace = (long long*)p.trace;
        g.trace_cap = p.trace ? p.trace_cap : 0;
        g.max_attempts = p.max_attempts > 0 ? p.max_attempts : 1000000;
        g.stats = p.stats;
        g.gamma = p.gamma; g.fr = p.fr; g.dT = p.dT; g.alpha = p.alpha; g.length = p.length;
        g.rtol = p.rtol; g.atol = p.atol;
        g.n_saves = S;
    }
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t de = cudaSetDevice(h->device);
    if (de != cudaSuccess) return cuda_fail(h, de, "cudaSetDevice");
    int rc = OPTIFAX_OK;
    const Twiddle* twp = get_pass_twiddles(h, M, st, &rc);
    if (!twp) return rc;
    const size_t need_k = (size_t)8 * M * n_pulses;
    if (need_k > h->gnlse_k_cap) {
        size_t cap = h->gnlse_k_cap * sizeof(float2);
        rc = grow_scratch(h, (void**)&h->d_gnlse_k, &cap, need_k * sizeof(float2), st,
                          "cudaMallocAsync(gnlse stage scratch)");
        h->gnlse_k_cap = cap / sizeof(float2);
        if (rc) return rc;
    }
    if ((size_t)n_pulses > h->gnlse_desc_cap) {
        size_t cap = h->gnlse_desc_cap * sizeof(GnlseDev);
        rc = grow_scratch(h, (void**)&h->d_gnlse_desc, &cap, sizeof(GnlseDev) * (size_t)n_pulses, st,
                          "cudaMallocAsync(gnlse descriptors)");
        h->gnlse_desc_cap = cap / sizeof(GnlseDev);
        if (rc) return rc;
    }
    for (int i = 0; i < n_pulses; ++i) d[(size_t)i].K = h->d_gnlse_k + (size_t)8 * M * i;
    rc = order_after_previous(h, st);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(h->d_gnlse_desc, d.data(), sizeof(GnlseDev) * (size_t)n_pulses,
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemcpyAsync(gnlse descriptors)");
    e = launch_gnlse(M, h->d_gnlse_desc, n_pulses, twp, twp + M, st);
    if (e != cudaSuccess) return cuda_fail(h, e, "gnlse_kernel launch");
    return mark_done(h, st);
}
