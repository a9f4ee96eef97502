// ofx_noalloc.cu -- a crystal pass that allocates no device memory.
//
// Some callers cannot allocate GPU memory while they run: a solver called from
// inside a MATLAB MEX function shares the device with MATLAB's own gpuArray
// memory manager, an application may hand all device memory to a caching
// allocator up front, and a latency-critical loop cannot afford cudaMalloc /
// cudaFree, which may synchronise the whole device.  optifax_propagate_noalloc
// serves them.  The caller still passes every input and output; everything else
// the pass needs -- the pulse descriptor, the FFT twiddle tables and the
// cluster exchange buffer -- lives in one file-scope static device array of
// fixed size (g_noalloc_scratch, about 0.45 MB), which every GPU that loads
// this library reserves until the process exits.
//
// The kernel is the clustered Heun crystal pass (4096 points per CTA, clusters
// of 2 or 4 CTAs), so n_points must be 8192 or 16384; anything else, in
// particular anything beyond 16384 points, is rejected with
// OPTIFAX_ERR_UNSUPPORTED.  The first call on a device fills the twiddle
// tables (set-up); make that first call before any stream capture.  All calls
// share the array and it keeps the last call's contents; nothing in it has to
// start at zero (each call rewrites the descriptor and every exchange value
// before reading it).  Calls that overlap on the GPU (other streams, other host
// threads) race on the array and must be serialised by the caller.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "ofx_kernels.cuh"
#include "../../include/optifax.h"

using namespace ofx;

namespace {

constexpr int kM = 4096;                 // points per CTA
constexpr int kMaxN = 16384;             // cluster of 4
constexpr size_t kDescBytes = 512;
constexpr size_t kPassTw = kM + 16 * (kM / 256);          // pass-1 + pass-2 outer twiddles
constexpr size_t kQuadTw = kM / 4;                         // W_M^y, y < M/4 (cluster exchange)
constexpr size_t kLowTw = 64;                              // W_N^i, i < 64 (cluster exchange)
constexpr size_t kXch = 2 * (size_t)kMaxN;                 // exchange buffer (complex)
constexpr size_t kOffPass = kDescBytes;
constexpr size_t kOffQuad = kOffPass + sizeof(Twiddle) * kPassTw;
constexpr size_t kOffN = kOffQuad + sizeof(Twiddle) * kQuadTw;
constexpr size_t kOffXch = kOffN + sizeof(Twiddle) * kLowTw;
constexpr size_t kBytes = kOffXch + sizeof(float2) * kXch;
static_assert(sizeof(PulseDev) <= kDescBytes, "descriptor slot too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

struct DeviceSetup {
    unsigned char* base = nullptr;       // device address of g_noalloc_scratch
    int n_table = 0;                     // N of the W_N table currently in the array
    bool pass_tables = false;
};
std::mutex g_mutex;
DeviceSetup g_setup[64];

__global__ void noalloc_pass_twiddles(Twiddle* out, int L) {
    int lr = L / 16;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 16 * lr) return;
    int r = idx / lr, off = idx - r * lr;
    double s, c;
    sincospi(-2.0 * (double)(off * r) / (double)L, &s, &c);
    float cf = (float)c, sf = (float)s;
    double m2 = (double)cf * (double)cf + (double)sf * (double)sf;
    out[idx] = Twiddle{cf, sf, (float)(1.0 / m2 - 1.0), 0.f};
}

// out[e] = W_n^e for e < count (FP32, d = 1/|w|^2 - 1 in FP64)
__global__ void noalloc_twiddles(Twiddle* out, int n, int count) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    double s, c;
    sincospi(-2.0 * (double)e / (double)n, &s, &c);
    float cf = (float)c, sf = (float)s;
    double m2 = (double)cf * (double)cf + (double)sf * (double)sf;
    out[e] = Twiddle{cf, sf, (float)(1.0 / m2 - 1.0), 0.f};
}

uint64_t noalloc_turns(long double radians) {
    long double tw = radians / (2.0L * 3.14159265358979323846264338327950288L);
    tw -= floorl(tw);
    long double x = tw * 18446744073709551616.0L;
    if (x >= 18446744073709551615.0L) return 0;
    return (uint64_t)x;
}

}  // namespace

extern "C" int optifax_propagate_noalloc(const optifax_pulse* pulse, int32_t variant,
                                         optifax_pulse_stats* stats, void* stream) {
    if (!pulse) return OPTIFAX_ERR_INVALID_ARGUMENT;
    const optifax_pulse& in = *pulse;
    if (in.n_points != 8192 && in.n_points != kMaxN) return OPTIFAX_ERR_UNSUPPORTED;
    if (in.n_steps < 1 || !(in.sel >= 1.0f) || !(in.h > 0.0f) || !(in.dt > 0.0) || !(in.w0 > 0.0f) ||
        !in.E_in || !in.A_out || !in.alpha || !in.beta || !in.G || (long long)in.n_steps * 4 > (1LL << 24))
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    int time_mode, abc_mode, guard, rule;
    switch (variant) {
        case OPTIFAX_VARIANT_BATCH_XTAL:
        case OPTIFAX_VARIANT_BATCH_OP: time_mode = TIME_SHIFTED; abc_mode = ABC_SOFT; guard = 1; rule = 128; break;
        case OPTIFAX_VARIANT_NO_BC: time_mode = TIME_UNSHIFTED; abc_mode = ABC_NONE; guard = 0; rule = 128; break;
        case OPTIFAX_VARIANT_HARD_BC: time_mode = TIME_UNSHIFTED; abc_mode = ABC_HARD; guard = 0; rule = 128; break;
        default: return OPTIFAX_ERR_INVALID_ARGUMENT;
    }
    const int N = in.n_points, C = N / kM;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return OPTIFAX_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;

    // kernel of this cluster size (no device memory involved)
    static std::vector<KernelEntry> table = [] {
        std::vector<KernelEntry> v;
        register_kernels_heun_large(v);
        return v;
    }();
    const KernelEntry* ke = nullptr;
    for (const auto& k : table)
        if (k.M == kM && k.C == C && k.method == OPTIFAX_HEUN) ke = &k;
    if (!ke) return OPTIFAX_ERR_UNSUPPORTED;

    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mutex);
        DeviceSetup& ds = g_setup[dev];
        if (!ds.base) {
            // set-up, once per device, with that device current
            unsigned char* p = nullptr;
            if (cudaGetSymbolAddress((void**)&p, g_noalloc_scratch) != cudaSuccess || !p) return OPTIFAX_ERR_CUDA;
            ds.base = p;
        }
        base = ds.base;
        if (!ds.pass_tables) {
            Twiddle* tw = reinterpret_cast<Twiddle*>(base + kOffPass);
            noalloc_pass_twiddles<<<(kM + 255) / 256, 256, 0, st>>>(tw, kM);
            noalloc_pass_twiddles<<<1, 256, 0, st>>>(tw + kM, kM / 16);
            noalloc_twiddles<<<(int)((kQuadTw + 255) / 256), 256, 0, st>>>(
                reinterpret_cast<Twiddle*>(base + kOffQuad), kM, (int)kQuadTw);
            if (cudaGetLastError() != cudaSuccess) return OPTIFAX_ERR_CUDA;
            ds.pass_tables = true;
        }
        if (ds.n_table != N) {
            noalloc_twiddles<<<1, 64, 0, st>>>(reinterpret_cast<Twiddle*>(base + kOffN), N, (int)kLowTw);
            if (cudaGetLastError() != cudaSuccess) return OPTIFAX_ERR_CUDA;
            ds.n_table = N;
        }
    }

    PulseDev d;
    memset(&d, 0, sizeof(d));
    d.E_in = (const float2*)in.E_in;
    d.A_out = (float2*)in.A_out;
    d.alpha = in.alpha;
    d.beta = in.beta;
    d.G = in.G;
    d.Ap = (float2*)in.Ap;
    d.stepmods = in.stepmods;
    d.trace = in.trace;
    d.forced = in.forced;
    d.stats = stats;
    d.bdiffw0 = in.bdiffw0;
    d.dt = in.dt;
    d.tau_theta = noalloc_turns((long double)(double)in.w0 * (long double)in.dt);
    d.tau_z4 = noalloc_turns((long double)in.bdiffw0 * (long double)(double)in.h / 4.0L);
    d.w0 = in.w0;
    d.h = in.h;
    d.max_err = in.max_err;
    d.min_err = in.min_err;
    d.sel = in.sel;
    d.c_shock = (float)(1.0 / (2.0 * in.dt)) / in.w0;
    d.N = N;
    d.S = in.n_steps;
    int nc = (int)((float)in.n_steps / in.sel);
    if (guard && (float)nc * in.sel < (float)in.n_steps) nc += 1;
    d.nchunks = nc;
    d.stepmods_limit = in.stepmods_limit > 0 ? in.stepmods_limit : ((N + rule - 1) / rule) * rule;
    d.trace_cap = in.trace ? in.trace_cap : 0;
    d.n_forced = in.forced ? in.n_forced : 0;
    d.xch = reinterpret_cast<float2*>(base + kOffXch);
    if (cudaMemcpyAsync(base, &d, sizeof(d), cudaMemcpyHostToDevice, st) != cudaSuccess) return OPTIFAX_ERR_CUDA;

    if (cudaFuncSetAttribute(ke->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ke->smem) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    KernelCfg cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.time_mode = time_mode;
    cfg.abc_mode = abc_mode;
    cfg.guard = guard;
    cfg.shared_sched = 0;
    cfg.max_attempts_mul = 64;
    cfg.grid_flags = nullptr;
    FftTables tabs;
    tabs.tw1 = reinterpret_cast<const Twiddle*>(base + kOffPass);
    tabs.tw2 = tabs.tw1 + kM;
    tabs.quad = reinterpret_cast<const Twiddle*>(base + kOffQuad);
    tabs.low = reinterpret_cast<const Twiddle*>(base + kOffN);
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)C, 1, 1);
    lc.blockDim = dim3(kM / 16, 1, 1);
    lc.dynamicSmemBytes = ke->smem;
    lc.stream = st;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = C; attr.val.clusterDim.y = 1; attr.val.clusterDim.z = 1;
    lc.attrs = &attr;
    lc.numAttrs = 1;
    const PulseDev* dd = reinterpret_cast<const PulseDev*>(base);
    if (cudaLaunchKernelEx(&lc, ke->fn, dd, tabs, cfg) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    return OPTIFAX_OK;
}
