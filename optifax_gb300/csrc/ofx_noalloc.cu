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
// fixed size (g_noalloc_scratch, 350,720 bytes, about 0.35 MB), which every GPU
// that loads this library reserves until the process exits.
//
// The kernel is the clustered Heun crystal pass (4096 points per CTA, clusters
// of 2 or 4 CTAs), so n_points must be 8192 or 16384; anything else, in
// particular anything beyond 16384 points, is rejected with
// OPTIFAX_ERR_UNSUPPORTED.
//
// Set-up: the first call in a CUDA context (the first on a device, and the
// first after that device's context was replaced, e.g. by cudaDeviceReset)
// looks up the array's device address with cudaGetSymbolAddress and fills the
// twiddle tables of both sizes.  That call must come before any stream capture;
// made while its stream captures, it returns OPTIFAX_ERR_UNSUPPORTED and sets
// nothing up.  Each call writes its descriptor with a one-thread kernel that
// receives it as a kernel parameter (no host staging buffer), and every
// exchange value is written before it is read, so nothing in the array has to
// start at zero.  All calls share the array and it keeps the last call's
// contents: calls that overlap on the GPU (other streams, other host threads)
// race on it and must be serialised by the caller.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ofx_kernels.cuh"
#include "ofx_desc.cuh"
#include "../../include/optifax.h"

using namespace ofx;

namespace {

constexpr int kM = 4096;                 // points per CTA
constexpr int kMaxN = 16384;             // cluster of 4
constexpr size_t kDescBytes = 512;
constexpr size_t kPassTw = kM + 16 * (kM / 256);          // pass-1 + pass-2 outer twiddles
constexpr size_t kQuadTw = kM / 4;                         // W_M^y, y < M/4 (cluster exchange)
constexpr size_t kLowTw = 64;                              // W_N^i, i < 64 (cluster exchange), per N
constexpr size_t kXch = 2 * (size_t)kMaxN;                 // exchange buffer (complex)
constexpr size_t kOffPass = kDescBytes;
constexpr size_t kOffQuad = kOffPass + sizeof(Twiddle) * kPassTw;
constexpr size_t kOffLow8k = kOffQuad + sizeof(Twiddle) * kQuadTw;     // W_8192^i
constexpr size_t kOffLow16k = kOffLow8k + sizeof(Twiddle) * kLowTw;    // W_16384^i
constexpr size_t kOffXch = kOffLow16k + sizeof(Twiddle) * kLowTw;
constexpr size_t kBytes = kOffXch + sizeof(float2) * kXch;
static_assert(sizeof(PulseDev) <= kDescBytes, "descriptor slot too small");
static_assert(kBytes == 350720, "the documented size of the static array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

// Per device: the CUDA context the tables were built in and the array's device
// address there.  A new context (a device reset, a context the caller created
// and made current) reloads the module with a zeroed array, so set-up reruns.
struct DeviceSetup {
    unsigned char* base = nullptr;
    unsigned long long ctx_id = 0;
    bool ready = false;
};
std::mutex g_mutex;
DeviceSetup g_setup[64];

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points (the
// library does not link the driver library itself)
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

bool current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (CtxGetCurrentFn)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (CtxGetIdFn)f;
    });
    void* ctx = nullptr;
    return get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, id) == 0;
}

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

// The call's descriptor arrives as a kernel parameter (copied at launch) and is
// written into its slot of the array in stream order.
__global__ void noalloc_put_desc(PulseDev* slot, PulseDev d) { *slot = d; }

int setup_tables(unsigned char* base, cudaStream_t st) {
    Twiddle* tw = reinterpret_cast<Twiddle*>(base + kOffPass);
    noalloc_pass_twiddles<<<(kM + 255) / 256, 256, 0, st>>>(tw, kM);
    noalloc_pass_twiddles<<<1, 256, 0, st>>>(tw + kM, kM / 16);
    noalloc_twiddles<<<(int)((kQuadTw + 255) / 256), 256, 0, st>>>(
        reinterpret_cast<Twiddle*>(base + kOffQuad), kM, (int)kQuadTw);
    noalloc_twiddles<<<1, 64, 0, st>>>(reinterpret_cast<Twiddle*>(base + kOffLow8k), 8192, (int)kLowTw);
    noalloc_twiddles<<<1, 64, 0, st>>>(reinterpret_cast<Twiddle*>(base + kOffLow16k), 16384, (int)kLowTw);
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

}  // namespace

extern "C" int optifax_propagate_noalloc(const optifax_pulse* pulse, int32_t variant,
                                         optifax_pulse_stats* stats, void* stream) {
    if (!pulse) return OPTIFAX_ERR_INVALID_ARGUMENT;
    const optifax_pulse& in = *pulse;
    if (in.n_points != 8192 && in.n_points != kMaxN) return OPTIFAX_ERR_UNSUPPORTED;
    if (variant != OPTIFAX_VARIANT_BATCH_XTAL && variant != OPTIFAX_VARIANT_BATCH_OP &&
        variant != OPTIFAX_VARIANT_NO_BC && variant != OPTIFAX_VARIANT_HARD_BC)
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    VariantCfg vc;
    if (!variant_cfg(variant, &vc)) return OPTIFAX_ERR_INVALID_ARGUMENT;
    PulseDev d;
    if (fill_pulse_desc(in, vc, &d, stats, nullptr) != OPTIFAX_OK) return OPTIFAX_ERR_INVALID_ARGUMENT;
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

    // the array's address in the current context (loads the module if needed)
    unsigned char* base = nullptr;
    if (cudaGetSymbolAddress((void**)&base, g_noalloc_scratch) != cudaSuccess || !base) return OPTIFAX_ERR_CUDA;
    unsigned long long ctx_id = 0;
    if (!current_context_id(&ctx_id)) return OPTIFAX_ERR_CUDA;
    {
        std::lock_guard<std::mutex> lk(g_mutex);
        DeviceSetup& ds = g_setup[dev];
        if (!ds.ready || ds.ctx_id != ctx_id || ds.base != base) {
            // set-up, once per context, with this device current; never under capture
            cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
            if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
                return OPTIFAX_ERR_UNSUPPORTED;
            ds.ready = false;
            if (setup_tables(base, st) != OPTIFAX_OK) return OPTIFAX_ERR_CUDA;
            ds.base = base;
            ds.ctx_id = ctx_id;
            ds.ready = true;
        }
    }

    d.xch = reinterpret_cast<float2*>(base + kOffXch);
    PulseDev* slot = reinterpret_cast<PulseDev*>(base);
    noalloc_put_desc<<<1, 1, 0, st>>>(slot, d);
    if (cudaGetLastError() != cudaSuccess) return OPTIFAX_ERR_CUDA;

    if (cudaFuncSetAttribute(ke->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ke->smem) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    KernelCfg cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.time_mode = vc.time_mode;
    cfg.abc_mode = vc.abc_mode;
    cfg.guard = vc.guard;
    cfg.shared_sched = 0;
    cfg.max_attempts_mul = 64;
    cfg.grid_flags = nullptr;
    FftTables tabs;
    tabs.tw1 = reinterpret_cast<const Twiddle*>(base + kOffPass);
    tabs.tw2 = tabs.tw1 + kM;
    tabs.quad = reinterpret_cast<const Twiddle*>(base + kOffQuad);
    tabs.low = reinterpret_cast<const Twiddle*>(base + (N == 8192 ? kOffLow8k : kOffLow16k));
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
    if (cudaLaunchKernelEx(&lc, ke->fn, (const PulseDev*)slot, tabs, cfg) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    return OPTIFAX_OK;
}
