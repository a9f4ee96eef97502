// ofx_fno.cu -- Fourier-neural-operator surrogate of one crystal pass: forward,
// backward and AdamW on the GPU.  No reference counterpart (the reference has no
// learned component).
//
// Network (fixed sizes): input x[b][6][L] (4 field channels, one constant
// conditioning channel and the bin coordinate over L frequency bins), lifting to
// width 64, four Fourier
// layers h <- act(SpecConv(h) + Wp h + bias) with 32 retained modes (no activation
// after the last), projection to 4 channels plus a residual connection to the
// first 4 input channels: y = x[:4] + Q h + q.
//
// Data layouts (per batch of B samples): "channel-major" Hc[c][b][x] and
// "point-major" Ht[b][x][c] copies of every activation, so that every product is
// an A . B^T GEMM with both operands K-major for the tensor-core kernel
// (optifax_gemm_bf16):
//   spectral transform   S[(c,b)][m'] = Hc . F^T         (F: 64 x L, m' = 2m + re/im)
//   inverse transform    Y1[(o,b)][x] = T . G^T          (G: L x 64)
//   pointwise mix        Y2[(b,x)][o] = Ht . Wp^T        (Wp: 64 x 64, [o][c])
//   weight gradient      dWp[o][c]    = dZc[o][(b,x)] . Hc[c][(b,x)]^T
//   backward transforms  dT = dZc . GT^T, dHs = dS . FT^T, dHp = dZt . WpT^T
// The per-mode complex channel mixing T[(o,b)][m] = sum_c S[(c,b)][m] W[c][o][m]
// and the element-wise parts run on the CUDA cores.  GEMM operands and
// activations are BF16; accumulation, pre-activations, gradients, biases, the
// master weights and the Adam moments are FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/optifax.h"

typedef __nv_bfloat16 bf16;

namespace {

constexpr int W = 64, MODES = 32, NLAYER = 4, CIN = 6, COUT = 4, SPEC = 2 * MODES;
constexpr long long LAYER_WS = (long long)W * W * MODES * 2;   // [c][o][m][re,im]
constexpr long long LAYER_SIZE = LAYER_WS + W * W + W;         // Ws, Wp [o][c], bias [o]
constexpr long long OFF_P = 0;                                 // [W][CIN]
constexpr long long OFF_PB = OFF_P + W * CIN;                  // [W]
constexpr long long OFF_L0 = OFF_PB + W;
constexpr long long OFF_Q = OFF_L0 + NLAYER * LAYER_SIZE;      // [COUT][W]
constexpr long long OFF_QB = OFF_Q + COUT * W;                 // [COUT]
constexpr long long N_PARAMS = OFF_QB + COUT;
constexpr long long off_ws(int l) { return OFF_L0 + l * LAYER_SIZE; }
constexpr long long off_wp(int l) { return off_ws(l) + LAYER_WS; }
constexpr long long off_b(int l) { return off_wp(l) + W * W; }
static_assert(off_wp(0) % 8 == 0 && LAYER_SIZE % 8 == 0, "BF16 GEMM operands must stay 16-byte aligned");

constexpr int XT = 4;   // 32-point x tiles per block in the transposing kernels

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// ---- tables --------------------------------------------------------------
__global__ void k_dft_tables(int L, bf16* F, bf16* FT, bf16* G, bf16* GT) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)SPEC * L) return;
    const int mp = (int)(i / L), x = (int)(i % L), m = mp >> 1;
    const long long ph = ((long long)m * x) % L;
    float s, c;
    sincospif(2.f * (float)ph / (float)L, &s, &c);
    const float f = (mp & 1) ? -s : c;
    const float g = f * (m == 0 ? 1.f : 2.f) / (float)L;
    F[(long long)mp * L + x] = __float2bfloat16(f);
    FT[(long long)x * SPEC + mp] = __float2bfloat16(f);
    G[(long long)x * SPEC + mp] = __float2bfloat16(g);
    GT[(long long)mp * L + x] = __float2bfloat16(g);
}

__global__ void k_refresh(const float* __restrict__ master, bf16* wb, bf16* wpt) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < N_PARAMS) wb[i] = __float2bfloat16(master[i]);
    if (i < (long long)NLAYER * W * W) {
        const int l = (int)(i / (W * W)), r = (int)(i % (W * W)), c = r / W, o = r % W;
        wpt[i] = __float2bfloat16(master[off_wp(l) + (long long)o * W + c]);
    }
}

// ---- forward -------------------------------------------------------------
__global__ void k_lift(const float* __restrict__ x, const bf16* __restrict__ Pw, const float* __restrict__ pb, int B,
                       int L, bf16* __restrict__ Hc, bf16* __restrict__ Ht) {
    __shared__ float sP[W * CIN];
    __shared__ float sb[W];
    for (int i = threadIdx.x; i < W * CIN; i += blockDim.x) sP[i] = __bfloat162float(Pw[i]);
    for (int i = threadIdx.x; i < W; i += blockDim.x) sb[i] = pb[i];
    __syncthreads();
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)B * L) return;
    const int b = (int)(idx / L), xx = (int)(idx % L);
    float in[CIN];
#pragma unroll
    for (int i = 0; i < CIN; ++i) in[i] = x[((long long)b * CIN + i) * L + xx];
    uint4 pack[W / 8];
    bf16* hp = reinterpret_cast<bf16*>(pack);
#pragma unroll
    for (int c = 0; c < W; ++c) {
        float h = sb[c];
#pragma unroll
        for (int i = 0; i < CIN; ++i) h = fmaf(sP[c * CIN + i], in[i], h);
        const bf16 hb = __float2bfloat16(h);
        hp[c] = hb;
        Hc[((long long)c * B + b) * L + xx] = hb;
    }
    uint4* dst = reinterpret_cast<uint4*>(Ht + idx * W);
#pragma unroll
    for (int j = 0; j < W / 8; ++j) dst[j] = pack[j];
}

// T[(o,b)][m] = sum_c S[(c,b)][m] W[c][o][m]   (complex)
__global__ void k_mix_fwd(const float* __restrict__ S, const bf16* __restrict__ Ws, int B, bf16* __restrict__ T) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)W * B * MODES) return;
    const int m = (int)(idx % MODES);
    const long long t = idx / MODES;
    const int b = (int)(t % B), o = (int)(t / B);
    float ar = 0.f, ai = 0.f;
    for (int c = 0; c < W; ++c) {
        const float* s = S + ((long long)c * B + b) * SPEC + 2 * m;
        const __nv_bfloat162 w = *reinterpret_cast<const __nv_bfloat162*>(Ws + (((long long)c * W + o) * MODES + m) * 2);
        const float wr = __low2float(w), wi = __high2float(w);
        ar = fmaf(s[0], wr, fmaf(-s[1], wi, ar));
        ai = fmaf(s[0], wi, fmaf(s[1], wr, ai));
    }
    bf16* d = T + ((long long)o * B + b) * SPEC + 2 * m;
    d[0] = __float2bfloat16(ar);
    d[1] = __float2bfloat16(ai);
}

// Z = Y1[c][b][x] + Y2[b][x][c] + bias[c]; h = act(Z) -> Hc, Ht (and Z kept for the backward)
__global__ void k_combine_fwd(const float* __restrict__ Y1, const float* __restrict__ Y2, const float* __restrict__ bias,
                              int B, int L, int act, float* __restrict__ Zs, bf16* __restrict__ Hc,
                              bf16* __restrict__ Ht) {
    __shared__ float tile[32][W + 1];
    const int b = blockIdx.y;
    for (int xt = 0; xt < XT; ++xt) {
        const int x0 = (blockIdx.x * XT + xt) * 32;
        if (x0 >= L) break;
        for (int r = 0; r < 8; ++r) {
            const int i = threadIdx.x + 256 * r, xi = i / W, c = i % W;
            tile[xi][c] = Y2[((long long)b * L + x0 + xi) * W + c];
        }
        __syncthreads();
        float hv[8];
        for (int r = 0; r < 8; ++r) {
            const int i = threadIdx.x + 256 * r, c = i / 32, xi = i % 32;
            const long long o = ((long long)c * B + b) * L + x0 + xi;
            const float z = Y1[o] + tile[xi][c] + bias[c];
            if (Zs) Zs[o] = z;
            const float h = act ? gelu(z) : z;
            Hc[o] = __float2bfloat16(h);
            hv[r] = h;
        }
        __syncthreads();
        for (int r = 0; r < 8; ++r) {
            const int i = threadIdx.x + 256 * r, c = i / 32, xi = i % 32;
            tile[xi][c] = hv[r];
        }
        __syncthreads();
        for (int r = 0; r < 8; ++r) {
            const int i = threadIdx.x + 256 * r, xi = i / W, c = i % W;
            Ht[((long long)b * L + x0 + xi) * W + c] = __float2bfloat16(tile[xi][c]);
        }
        __syncthreads();
    }
}

// y[b][j][x] = x[b][j][x] + q[j] + sum_c Q[j][c] h[b][x][c]
__global__ void k_proj_fwd(const bf16* __restrict__ Ht, const bf16* __restrict__ Qw, const float* __restrict__ qb,
                           const float* __restrict__ xin, int B, int L, float* __restrict__ y) {
    __shared__ float sQ[COUT * W];
    for (int i = threadIdx.x; i < COUT * W; i += blockDim.x) sQ[i] = __bfloat162float(Qw[i]);
    __syncthreads();
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)B * L) return;
    const int b = (int)(idx / L), xx = (int)(idx % L);
    float acc[COUT];
#pragma unroll
    for (int j = 0; j < COUT; ++j) acc[j] = qb[j];
    const uint4* src = reinterpret_cast<const uint4*>(Ht + idx * W);
#pragma unroll
    for (int q8 = 0; q8 < W / 8; ++q8) {
        const uint4 u = src[q8];
        const bf16* hp = reinterpret_cast<const bf16*>(&u);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const float h = __bfloat162float(hp[e]);
#pragma unroll
            for (int j = 0; j < COUT; ++j) acc[j] = fmaf(sQ[j * W + q8 * 8 + e], h, acc[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < COUT; ++j)
        y[((long long)b * COUT + j) * L + xx] = xin[((long long)b * CIN + j) * L + xx] + acc[j];
}

// ---- loss and backward ---------------------------------------------------
// loss = sum_i w_(sample of i) (y_i - t_i)^2 / n  (w = 1 without sample weights)
__global__ void k_loss(const float* __restrict__ y, const float* __restrict__ t, const float* __restrict__ w,
                       long long per_sample, long long n, float inv_n, float* __restrict__ dy,
                       float* __restrict__ loss) {
    __shared__ float red[32];
    float part = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float d = y[i] - t[i];
        const float wi = w ? w[i / per_sample] : 1.f;
        dy[i] = 2.f * d * inv_n * wi;
        part = fmaf(wi * d, d, part);
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) atomicAdd(loss, v * inv_n);
    }
}

// dH4 = Q^T dy (the last layer has no activation, so this is dZ of layer 3) -> dZc, dZt; bias grad
__global__ void k_proj_bwd(const float* __restrict__ dy, const bf16* __restrict__ Qw, int B, int L,
                           bf16* __restrict__ dZc, bf16* __restrict__ dZt, float* __restrict__ db) {
    __shared__ float sQ[COUT * W];
    __shared__ float sdb[W];
    for (int i = threadIdx.x; i < COUT * W; i += blockDim.x) sQ[i] = __bfloat162float(Qw[i]);
    for (int i = threadIdx.x; i < W; i += blockDim.x) sdb[i] = 0.f;
    __syncthreads();
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = idx < (long long)B * L;
    float d[COUT] = {0.f, 0.f, 0.f, 0.f};
    int b = 0, xx = 0;
    if (live) {
        b = (int)(idx / L);
        xx = (int)(idx % L);
#pragma unroll
        for (int j = 0; j < COUT; ++j) d[j] = dy[((long long)b * COUT + j) * L + xx];
    }
    uint4 pack[W / 8];
    bf16* gp = reinterpret_cast<bf16*>(pack);
#pragma unroll
    for (int c = 0; c < W; ++c) {
        float g = 0.f;
#pragma unroll
        for (int j = 0; j < COUT; ++j) g = fmaf(sQ[j * W + c], d[j], g);
        gp[c] = __float2bfloat16(g);
        if (live) dZc[((long long)c * B + b) * L + xx] = gp[c];
        float s = g;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&sdb[c], s);
    }
    if (live) {
        uint4* dst = reinterpret_cast<uint4*>(dZt + idx * W);
#pragma unroll
        for (int j = 0; j < W / 8; ++j) dst[j] = pack[j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < W; i += blockDim.x) atomicAdd(&db[i], sdb[i]);
}

// dQ[j][c] = sum_(b,x) dy[b][j][x] h[b][x][c];  dq[j] = sum dy[b][j][x]
__global__ void k_proj_wgrad(const float* __restrict__ dy, const bf16* __restrict__ Ht, int B, int L, int rows_per_block,
                             float* __restrict__ dQ, float* __restrict__ dq) {
    __shared__ float hs[64][W + 1];
    __shared__ float ds[COUT][64];
    const int t = threadIdx.x, j = t / W, c = t % W;
    const long long total = (long long)B * L;
    const long long r0 = (long long)blockIdx.x * rows_per_block;
    float acc = 0.f, accq = 0.f;
    for (long long base = r0; base < r0 + rows_per_block && base < total; base += 64) {
        for (int r = 0; r < 16; ++r) {
            const int i = t + 256 * r, row = i / W, cc = i % W;
            const long long g = base + row;
            hs[row][cc] = g < total ? __bfloat162float(Ht[g * W + cc]) : 0.f;
        }
        {
            const int jj = t / 64, rr = t % 64;
            const long long g = base + rr;
            ds[jj][rr] = g < total ? dy[((g / L) * COUT + jj) * L + (g % L)] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int rr = 0; rr < 64; ++rr) acc = fmaf(ds[j][rr], hs[rr][c], acc);
        if (c == 0)
            for (int rr = 0; rr < 64; ++rr) accq += ds[j][rr];
        __syncthreads();
    }
    atomicAdd(&dQ[j * W + c], acc);
    if (c == 0) atomicAdd(&dq[j], accq);
}

// dS[(c,b)][m] = sum_o dT[(o,b)][m] conj(W[c][o][m])
__global__ void k_mix_bwd_ds(const float* __restrict__ dT, const bf16* __restrict__ Ws, int B, bf16* __restrict__ dS) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)W * B * MODES) return;
    const int m = (int)(idx % MODES);
    const long long t = idx / MODES;
    const int b = (int)(t % B), c = (int)(t / B);
    float ar = 0.f, ai = 0.f;
    for (int o = 0; o < W; ++o) {
        const float* d = dT + ((long long)o * B + b) * SPEC + 2 * m;
        const __nv_bfloat162 w = *reinterpret_cast<const __nv_bfloat162*>(Ws + (((long long)c * W + o) * MODES + m) * 2);
        const float wr = __low2float(w), wi = __high2float(w);
        ar = fmaf(d[0], wr, fmaf(d[1], wi, ar));
        ai = fmaf(d[1], wr, fmaf(-d[0], wi, ai));
    }
    bf16* o_ = dS + ((long long)c * B + b) * SPEC + 2 * m;
    o_[0] = __float2bfloat16(ar);
    o_[1] = __float2bfloat16(ai);
}

// dW[c][o][m] = sum_b conj(S[(c,b)][m]) dT[(o,b)][m]
__global__ void k_mix_bwd_dw(const float* __restrict__ dT, const float* __restrict__ S, int B, float* __restrict__ dW) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)W * W * MODES) return;
    const int m = (int)(idx % MODES);
    const long long t = idx / MODES;
    const int o = (int)(t % W), c = (int)(t / W);
    float ar = 0.f, ai = 0.f;
    for (int b = 0; b < B; ++b) {
        const float* s = S + ((long long)c * B + b) * SPEC + 2 * m;
        const float* d = dT + ((long long)o * B + b) * SPEC + 2 * m;
        ar = fmaf(s[0], d[0], fmaf(s[1], d[1], ar));
        ai = fmaf(s[0], d[1], fmaf(-s[1], d[0], ai));
    }
    dW[(((long long)c * W + o) * MODES + m) * 2] = ar;
    dW[(((long long)c * W + o) * MODES + m) * 2 + 1] = ai;
}

// g = dHs[c][b][x] + dHp[b][x][c]; with Zprev: dZ = g act'(Zprev) -> dZc, dZt, bias grad;
// without (layer 0): g written back into dHs (the gradient of the lifted input)
__global__ void k_combine_bwd(float* __restrict__ dHs, const float* __restrict__ dHp, const float* __restrict__ Zprev,
                              int B, int L, bf16* __restrict__ dZc, bf16* __restrict__ dZt, float* __restrict__ db) {
    __shared__ float tile[32][W + 1];
    const int b = blockIdx.y;
    float bsum[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int xt = 0; xt < XT; ++xt) {
        const int x0 = (blockIdx.x * XT + xt) * 32;
        if (x0 >= L) break;
        for (int r = 0; r < 8; ++r) {
            const int i = threadIdx.x + 256 * r, xi = i / W, c = i % W;
            tile[xi][c] = dHp[((long long)b * L + x0 + xi) * W + c];
        }
        __syncthreads();
        float gv[8];
        for (int r = 0; r < 8; ++r) {
            const int i = threadIdx.x + 256 * r, c = i / 32, xi = i % 32;
            const long long o = ((long long)c * B + b) * L + x0 + xi;
            float g = dHs[o] + tile[xi][c];
            if (Zprev) {
                g *= gelu_d(Zprev[o]);
                dZc[o] = __float2bfloat16(g);
                bsum[r] += g;
            } else {
                dHs[o] = g;
            }
            gv[r] = g;
        }
        __syncthreads();
        if (Zprev) {
            for (int r = 0; r < 8; ++r) {
                const int i = threadIdx.x + 256 * r, c = i / 32, xi = i % 32;
                tile[xi][c] = gv[r];
            }
            __syncthreads();
            for (int r = 0; r < 8; ++r) {
                const int i = threadIdx.x + 256 * r, xi = i / W, c = i % W;
                dZt[((long long)b * L + x0 + xi) * W + c] = __float2bfloat16(tile[xi][c]);
            }
            __syncthreads();
        }
    }
    if (Zprev) {
        // every warp holds channels warp + 8 r (r = 0..7) across its 32 lanes
        for (int r = 0; r < 8; ++r) {
            float s = bsum[r];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if ((threadIdx.x & 31) == 0) atomicAdd(&db[(threadIdx.x >> 5) + 8 * r], s);
        }
    }
}

// dP[c][i] = sum_(b,x) dH0[c][b][x] x[b][i][x];  dp[c] = sum dH0[c][b][x]
__global__ void k_lift_wgrad(const float* __restrict__ dH0, const float* __restrict__ x, int B, int L,
                             float* __restrict__ dP, float* __restrict__ dp) {
    __shared__ float red[CIN + 1][8];
    const int c = blockIdx.x;
    const long long total = (long long)B * L;
    float acc[CIN + 1];
#pragma unroll
    for (int i = 0; i <= CIN; ++i) acc[i] = 0.f;
    for (long long g = blockIdx.y * (long long)blockDim.x + threadIdx.x; g < total;
         g += (long long)gridDim.y * blockDim.x) {
        const int b = (int)(g / L), xx = (int)(g % L);
        const float d = dH0[((long long)c * B + b) * L + xx];
        acc[CIN] += d;
#pragma unroll
        for (int i = 0; i < CIN; ++i) acc[i] = fmaf(d, x[((long long)b * CIN + i) * L + xx], acc[i]);
    }
#pragma unroll
    for (int i = 0; i <= CIN; ++i) {
        float s = acc[i];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[i][threadIdx.x >> 5] = s;
    }
    __syncthreads();
    if (threadIdx.x <= CIN) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x][w];
        if (threadIdx.x < CIN) atomicAdd(&dP[c * CIN + threadIdx.x], s);
        else atomicAdd(&dp[c], s);
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float wd, float bc1, float bc2) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * ((mi / bc1) / (sqrtf(vi / bc2) + eps) + wd * p[i]);
}

// ---- OPO fast-forward: spectra <-> network channels ------------------------
// The crop is n_bins consecutive bins of an N-point spectrum (natural FFT order)
// starting at bin k0 (wrapping at N); bins j < split form the signal band.
__global__ void k_ff_encode(const float2* __restrict__ Y, long long ystride, int N, int k0, int L, int split,
                            float pump_scale, const float* __restrict__ sigma_in, float* __restrict__ x, int nch,
                            float* __restrict__ sigma_out) {
    __shared__ float red[32];
    __shared__ float s_sigma;
    const int p = blockIdx.x;
    const float2* y = Y + p * ystride;
    if (sigma_in) {
        if (threadIdx.x == 0) s_sigma = sigma_in[p];
    } else {
        float acc = 0.f;
        for (int j = threadIdx.x; j < split; j += blockDim.x) {
            const float2 v = y[(k0 + j) % N];
            acc = fmaf(v.x, v.x, fmaf(v.y, v.y, acc));
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            float tot = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
            float sg = sqrtf(tot / (float)(split > 0 ? split : 1));
            const float floor_ = 1e-30f * pump_scale;
            if (!(sg > floor_)) sg = floor_;
            s_sigma = sg;
            if (sigma_out) sigma_out[p] = sg;
        }
    }
    __syncthreads();
    const float sg = s_sigma, inv_s = 1.f / sg, inv_p = 1.f / pump_scale;
    const float lg = log10f(sg * inv_p);
    float* xo = x + (long long)p * nch * L;
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        const float2 v = y[(k0 + j) % N];
        const bool sb = j < split;
        xo[j] = sb ? 0.f : v.x * inv_p;
        xo[L + j] = sb ? 0.f : v.y * inv_p;
        xo[2 * L + j] = sb ? v.x * inv_s : 0.f;
        xo[3 * L + j] = sb ? v.y * inv_s : 0.f;
        if (nch > 4) {
            xo[4 * L + j] = lg;
            xo[5 * L + j] = (float)j / (float)L;
        }
    }
}

// X = (decoded network output or X_in) times lin; Y_next = X fb + pump; energy += sum tally_w |X|^2
__global__ void k_ff_step(const float* __restrict__ y, const float* __restrict__ sigma, const float2* __restrict__ X_in,
                          const float2* __restrict__ fb, const float2* __restrict__ pump,
                          const float2* __restrict__ lin, const float* __restrict__ tw, int N, int k0, int L,
                          int split, float pump_scale, float2* __restrict__ X_out, float2* __restrict__ Y_next,
                          double* __restrict__ energy) {
    __shared__ double red[32];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (k < N) {
        float2 X = make_float2(0.f, 0.f);
        if (y) {
            const int j = (k - k0 + N) % N;
            if (j < L) {
                if (j < split) {
                    const float sg = sigma[0];
                    X = make_float2(y[2 * L + j] * sg, y[3 * L + j] * sg);
                } else {
                    X = make_float2(y[j] * pump_scale, y[L + j] * pump_scale);
                }
            }
        } else {
            X = X_in[k];
        }
        if (lin) {
            const float2 d = lin[k];
            X = make_float2(X.x * d.x - X.y * d.y, X.x * d.y + X.y * d.x);
        }
        if (X_out) X_out[k] = X;
        const float2 f = fb[k], pp = pump[k];
        Y_next[k] = make_float2(X.x * f.x - X.y * f.y + pp.x, X.x * f.y + X.y * f.x + pp.y);
        if (tw) e = (double)tw[k] * ((double)X.x * X.x + (double)X.y * X.y);
    }
    if (energy) {
        for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
            atomicAdd(energy, tot);
        }
    }
}

// ---- OPO fast-forward, envelope representation ---------------------------
// A band is the set of bins whose signed offset o from the band's carrier bin kc
// (natural FFT order of the N-point spectrum) lies in [lo, hi), |o| < L/2.  Its
// envelope is e_j = sum_o b_o exp(+2 pi i o j / L), j < L: the band demodulated to
// its carrier and sampled L times over the window.
struct EnvBand {
    int kc, lo, hi;
};

__device__ __forceinline__ int env_bin(const EnvBand& b, int N, int L, int j, bool* in) {
    const int o = j < L / 2 ? j : j - L;
    *in = o >= b.lo && o < b.hi;
    int k = (b.kc + o) % N;
    return k < 0 ? k + N : k;
}

// in-place radix-2 DIT FFT of L points in shared memory (input already in
// bit-reversed order); sign +1: exp(+2 pi i ...), -1: exp(-2 pi i ...)
__device__ void smem_fft(float2* sm, int L, float sign) {
    for (int len = 2; len <= L; len <<= 1) {
        const int half = len >> 1;
        for (int b = threadIdx.x; b < L / 2; b += blockDim.x) {
            const int grp = b / half, j = b - grp * half;
            const int i0 = grp * len + j, i1 = i0 + half;
            float sn, cs;
            sincospif(sign * 2.f * (float)j / (float)len, &sn, &cs);
            const float2 u = sm[i0], v0 = sm[i1];
            const float2 v = make_float2(v0.x * cs - v0.y * sn, v0.x * sn + v0.y * cs);
            sm[i0] = make_float2(u.x + v.x, u.y + v.y);
            sm[i1] = make_float2(u.x - v.x, u.y - v.y);
        }
        __syncthreads();
    }
}

// grid (spectra, 2 bands): envelopes -> channels 0/1 (pump / pump_scale), 2/3
// (signal / sigma), 4 log10(sigma / pump_scale), 5 j / L
__global__ void k_ff_encode_env(const float2* __restrict__ Y, long long ystride, int N, int L, int logL, EnvBand bp,
                                EnvBand bs, float pump_scale, const float* __restrict__ sigma_in,
                                float* __restrict__ x, int nch, float* __restrict__ sigma_out) {
    __shared__ float2 sm[4096];
    __shared__ float red[32];
    __shared__ float s_sig;
    const int p = blockIdx.x, band = blockIdx.y;
    const EnvBand bd = band ? bs : bp;
    const float2* y = Y + p * ystride;
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        bool in;
        const int k = env_bin(bd, N, L, j, &in);
        sm[__brev((unsigned)j) >> (32 - logL)] = in ? y[k] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    smem_fft(sm, L, 1.f);
    float scale = 1.f / pump_scale, sg = 1.f;
    if (band == 1) {
        if (sigma_in) {
            if (threadIdx.x == 0) s_sig = sigma_in[p];
        } else {
            float acc = 0.f;
            for (int j = threadIdx.x; j < L; j += blockDim.x) acc = fmaf(sm[j].x, sm[j].x, fmaf(sm[j].y, sm[j].y, acc));
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
            __syncthreads();
            if (threadIdx.x == 0) {
                float tot = 0.f;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
                float v = sqrtf(tot / (float)L);
                const float floor_ = 1e-30f * pump_scale;
                if (!(v > floor_)) v = floor_;
                s_sig = v;
                if (sigma_out) sigma_out[p] = v;
            }
        }
        __syncthreads();
        sg = s_sig;
        scale = 1.f / sg;
    }
    float* xo = x + (long long)p * nch * L;
    const float lg = log10f(sg / pump_scale);
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        xo[(2 * band) * L + j] = sm[j].x * scale;
        xo[(2 * band + 1) * L + j] = sm[j].y * scale;
        if (band == 1 && nch > 4) {
            xo[4 * L + j] = lg;
            xo[5 * L + j] = (float)j / (float)L;
        }
    }
}

// grid (2 bands): network output envelopes -> band bins of X (X zeroed by the host)
__global__ void k_ff_decode_env(const float* __restrict__ y, const float* __restrict__ sigma, int N, int L, int logL,
                                EnvBand bp, EnvBand bs, float pump_scale, float2* __restrict__ X) {
    __shared__ float2 sm[4096];
    const int band = blockIdx.x;
    const EnvBand bd = band ? bs : bp;
    for (int j = threadIdx.x; j < L; j += blockDim.x)
        sm[__brev((unsigned)j) >> (32 - logL)] = make_float2(y[(2 * band) * L + j], y[(2 * band + 1) * L + j]);
    __syncthreads();
    smem_fft(sm, L, -1.f);
    const float scale = (band ? sigma[0] : pump_scale) / (float)L;
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        bool in;
        const int k = env_bin(bd, N, L, j, &in);
        if (in) X[k] = make_float2(sm[j].x * scale, sm[j].y * scale);
    }
}

inline unsigned nblk(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

struct optifax_fno_s {
    int device = 0, L = 0, maxB = 0;
    float *master = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    bf16 *wb = nullptr, *wpt = nullptr;
    bf16 *F = nullptr, *FT = nullptr, *G = nullptr, *GT = nullptr;
    bf16 *Hc[NLAYER + 1] = {}, *Ht[NLAYER + 1] = {};
    float* Z[NLAYER - 1] = {};
    float* S[NLAYER] = {};
    bf16 *T = nullptr, *dS = nullptr, *dZc = nullptr, *dZt = nullptr;
    float *Y1 = nullptr, *Y2 = nullptr, *y = nullptr, *dy = nullptr, *dT = nullptr, *loss = nullptr;
};

namespace {

template <typename P>
int alloc0(P** p, size_t bytes) {
    if (cudaMalloc(reinterpret_cast<void**>(p), bytes) != cudaSuccess) return OPTIFAX_ERR_NO_MEMORY;
    if (cudaMemset(*p, 0, bytes) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    return OPTIFAX_OK;
}

#define OFX_TRY(x)                    \
    do {                              \
        int rc_ = (x);                \
        if (rc_) return rc_;          \
    } while (0)

int fno_forward(optifax_fno_s* f, const float* x, int B, cudaStream_t st) {
    const int L = f->L;
    const long long WB = (long long)W * B, rowsA = WB > 128 ? WB : 128;
    k_lift<<<nblk((long long)B * L), 256, 0, st>>>(x, f->wb + OFF_P, f->master + OFF_PB, B, L, f->Hc[0], f->Ht[0]);
    for (int l = 0; l < NLAYER; ++l) {
        OFX_TRY(optifax_gemm_bf16(f->Hc[l], L, rowsA, f->F, L, SPEC, f->S[l], SPEC, (int)WB, SPEC, L, 8, 0, st));
        k_mix_fwd<<<nblk(WB * MODES), 256, 0, st>>>(f->S[l], f->wb + off_ws(l), B, f->T);
        OFX_TRY(optifax_gemm_bf16(f->T, SPEC, rowsA, f->G, SPEC, L, f->Y1, L, (int)WB, L, SPEC, 1, 0, st));
        OFX_TRY(optifax_gemm_bf16(f->Ht[l], W, (long long)B * L, f->wb + off_wp(l), W, W, f->Y2, W, B * L, W, W, 1,
                                  0, st));
        const int act = l < NLAYER - 1;
        k_combine_fwd<<<dim3((L + 32 * XT - 1) / (32 * XT), B), 256, 0, st>>>(
            f->Y1, f->Y2, f->master + off_b(l), B, L, act, act ? f->Z[l] : nullptr, f->Hc[l + 1], f->Ht[l + 1]);
    }
    k_proj_fwd<<<nblk((long long)B * L), 256, 0, st>>>(f->Ht[NLAYER], f->wb + OFF_Q, f->master + OFF_QB, x, B, L,
                                                       f->y);
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

int fno_backward(optifax_fno_s* f, const float* x, const float* target, const float* sample_w, int B,
                 cudaStream_t st) {
    const int L = f->L;
    const long long WB = (long long)W * B, rowsA = WB > 128 ? WB : 128, BL = (long long)B * L;
    if (cudaMemsetAsync(f->grad, 0, sizeof(float) * N_PARAMS, st) != cudaSuccess ||
        cudaMemsetAsync(f->loss, 0, sizeof(float), st) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    const long long ny = BL * COUT;
    k_loss<<<256, 256, 0, st>>>(f->y, target, sample_w, (long long)COUT * L, ny, 1.f / (float)ny, f->dy, f->loss);
    k_proj_bwd<<<nblk(BL), 256, 0, st>>>(f->dy, f->wb + OFF_Q, B, L, f->dZc, f->dZt, f->grad + off_b(NLAYER - 1));
    const int rpb = 2048;
    k_proj_wgrad<<<nblk(BL, rpb), 256, 0, st>>>(f->dy, f->Ht[NLAYER], B, L, rpb, f->grad + OFF_Q, f->grad + OFF_QB);
    for (int l = NLAYER - 1; l >= 0; --l) {
        const int splits = (int)((BL + 2047) / 2048);
        OFX_TRY(optifax_gemm_bf16(f->dZc, BL, 128, f->Hc[l], BL, W, f->grad + off_wp(l), W, W, W, (int)BL, splits, 1,
                                  st));
        OFX_TRY(optifax_gemm_bf16(f->dZc, L, 2 * WB, f->GT, L, SPEC, f->dT, SPEC, (int)WB, SPEC, L, 8, 0, st));
        k_mix_bwd_ds<<<nblk(WB * MODES), 256, 0, st>>>(f->dT, f->wb + off_ws(l), B, f->dS);
        k_mix_bwd_dw<<<nblk((long long)W * W * MODES), 256, 0, st>>>(f->dT, f->S[l], B, f->grad + off_ws(l));
        OFX_TRY(optifax_gemm_bf16(f->dS, SPEC, rowsA, f->FT, SPEC, L, f->Y1, L, (int)WB, L, SPEC, 1, 0, st));
        OFX_TRY(optifax_gemm_bf16(f->dZt, W, BL, f->wpt + (long long)l * W * W, W, W, f->Y2, W, (int)BL, W, W, 1, 0,
                                  st));
        const dim3 cg((L + 32 * XT - 1) / (32 * XT), B);
        if (l > 0) {
            k_combine_bwd<<<cg, 256, 0, st>>>(f->Y1, f->Y2, f->Z[l - 1], B, L, f->dZc, f->dZt, f->grad + off_b(l - 1));
        } else {
            k_combine_bwd<<<cg, 256, 0, st>>>(f->Y1, f->Y2, nullptr, B, L, nullptr, nullptr, nullptr);
            k_lift_wgrad<<<dim3(W, 8), 256, 0, st>>>(f->Y1, x, B, L, f->grad + OFF_P, f->grad + OFF_PB);
        }
    }
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

void fno_free(optifax_fno_s* f) {
    void* ps[] = {f->master, f->grad, f->m, f->v, f->wb, f->wpt, f->F, f->FT, f->G, f->GT, f->T, f->dS, f->dZc,
                  f->dZt, f->Y1, f->Y2, f->y, f->dy, f->dT, f->loss};
    for (void* p : ps)
        if (p) cudaFree(p);
    for (int l = 0; l <= NLAYER; ++l) {
        if (f->Hc[l]) cudaFree(f->Hc[l]);
        if (f->Ht[l]) cudaFree(f->Ht[l]);
    }
    for (int l = 0; l < NLAYER; ++l)
        if (f->S[l]) cudaFree(f->S[l]);
    for (int l = 0; l < NLAYER - 1; ++l)
        if (f->Z[l]) cudaFree(f->Z[l]);
    delete f;
}

}  // namespace

extern "C" int64_t optifax_fno_param_count(void) { return N_PARAMS; }

extern "C" int optifax_fno_create(optifax_fno* out, int32_t n_bins, int32_t max_batch, int32_t device) {
    if (!out) return OPTIFAX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n_bins < 128 || n_bins % 64 || n_bins > (1 << 20) || max_batch < 1 || max_batch > 4096)
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    optifax_fno_s* f = new optifax_fno_s();
    f->device = device;
    f->L = n_bins;
    f->maxB = max_batch;
    const long long L = n_bins, WB = (long long)W * max_batch, rowsA = WB > 128 ? WB : 128, BL = max_batch * L;
    int rc = OPTIFAX_OK;
    auto A = [&](auto** p, size_t bytes) {
        if (!rc) rc = alloc0(p, bytes);
    };
    A(&f->master, sizeof(float) * N_PARAMS);
    A(&f->grad, sizeof(float) * N_PARAMS);
    A(&f->m, sizeof(float) * N_PARAMS);
    A(&f->v, sizeof(float) * N_PARAMS);
    A(&f->wb, sizeof(bf16) * N_PARAMS);
    A(&f->wpt, sizeof(bf16) * NLAYER * W * W);
    A(&f->F, sizeof(bf16) * SPEC * L);
    A(&f->FT, sizeof(bf16) * SPEC * L);
    A(&f->G, sizeof(bf16) * SPEC * L);
    A(&f->GT, sizeof(bf16) * SPEC * L);
    for (int l = 0; l <= NLAYER; ++l) {
        A(&f->Hc[l], sizeof(bf16) * rowsA * L);
        A(&f->Ht[l], sizeof(bf16) * BL * W);
    }
    for (int l = 0; l < NLAYER - 1; ++l) A(&f->Z[l], sizeof(float) * WB * L);
    for (int l = 0; l < NLAYER; ++l) A(&f->S[l], sizeof(float) * WB * SPEC);
    A(&f->T, sizeof(bf16) * rowsA * SPEC);
    A(&f->dS, sizeof(bf16) * rowsA * SPEC);
    A(&f->dZc, sizeof(bf16) * 2 * WB * L);     // the [o][(b,x)] view is read as 128 rows
    A(&f->dZt, sizeof(bf16) * BL * W);
    A(&f->Y1, sizeof(float) * WB * L);
    A(&f->Y2, sizeof(float) * BL * W);
    A(&f->y, sizeof(float) * BL * COUT);
    A(&f->dy, sizeof(float) * BL * COUT);
    A(&f->dT, sizeof(float) * WB * SPEC);
    A(&f->loss, sizeof(float));
    if (!rc) {
        k_dft_tables<<<nblk((long long)SPEC * L), 256>>>((int)L, f->F, f->FT, f->G, f->GT);
        if (cudaDeviceSynchronize() != cudaSuccess) rc = OPTIFAX_ERR_CUDA;
    }
    if (rc) {
        fno_free(f);
        return rc;
    }
    *out = f;
    return OPTIFAX_OK;
}

extern "C" int optifax_fno_destroy(optifax_fno f) {
    if (!f) return OPTIFAX_ERR_NULL_HANDLE;
    cudaSetDevice(f->device);
    cudaDeviceSynchronize();
    fno_free(f);
    return OPTIFAX_OK;
}

extern "C" int optifax_fno_set_params(optifax_fno f, const float* params, void* stream) {
    if (!f) return OPTIFAX_ERR_NULL_HANDLE;
    if (!params) return OPTIFAX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(f->master, params, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(f->m, 0, sizeof(float) * N_PARAMS, st) != cudaSuccess ||
        cudaMemsetAsync(f->v, 0, sizeof(float) * N_PARAMS, st) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    k_refresh<<<nblk(N_PARAMS), 256, 0, st>>>(f->master, f->wb, f->wpt);
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

extern "C" int optifax_fno_get_params(optifax_fno f, float* params, void* stream) {
    if (!f) return OPTIFAX_ERR_NULL_HANDLE;
    if (!params) return OPTIFAX_ERR_INVALID_ARGUMENT;
    return cudaMemcpyAsync(params, f->master, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToDevice,
                           static_cast<cudaStream_t>(stream)) == cudaSuccess
               ? OPTIFAX_OK
               : OPTIFAX_ERR_CUDA;
}

extern "C" int optifax_fno_forward(optifax_fno f, const float* x, float* y, int32_t batch, void* stream) {
    if (!f) return OPTIFAX_ERR_NULL_HANDLE;
    if (!x || batch < 1 || batch > f->maxB) return OPTIFAX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    OFX_TRY(fno_forward(f, x, batch, st));
    if (y && cudaMemcpyAsync(y, f->y, sizeof(float) * (size_t)batch * COUT * f->L, cudaMemcpyDeviceToDevice, st) !=
                 cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    return OPTIFAX_OK;
}

extern "C" int optifax_fno_backward(optifax_fno f, const float* x, const float* target, const float* sample_w,
                                    int32_t batch, float* loss, float* grads, void* stream) {
    if (!f) return OPTIFAX_ERR_NULL_HANDLE;
    if (!x || !target || batch < 1 || batch > f->maxB) return OPTIFAX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    OFX_TRY(fno_forward(f, x, batch, st));
    OFX_TRY(fno_backward(f, x, target, sample_w, batch, st));
    if (loss && cudaMemcpyAsync(loss, f->loss, sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    if (grads && cudaMemcpyAsync(grads, f->grad, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    return OPTIFAX_OK;
}

// Data-parallel training: replace the gradients of the last backward (for example by
// their mean over ranks) before optifax_fno_adam.
extern "C" int optifax_fno_set_grads(optifax_fno f, const float* grads, void* stream) {
    if (!f) return OPTIFAX_ERR_NULL_HANDLE;
    if (!grads) return OPTIFAX_ERR_INVALID_ARGUMENT;
    return cudaMemcpyAsync(f->grad, grads, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToDevice,
                           static_cast<cudaStream_t>(stream)) == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

extern "C" int optifax_fno_adam(optifax_fno f, float lr, float beta1, float beta2, float eps, float weight_decay,
                                int32_t step, void* stream) {
    if (!f) return OPTIFAX_ERR_NULL_HANDLE;
    if (step < 1 || !(lr >= 0.f)) return OPTIFAX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
    k_adam<<<nblk(N_PARAMS), 256, 0, st>>>(f->master, f->grad, f->m, f->v, N_PARAMS, lr, beta1, beta2, eps,
                                           weight_decay, bc1, bc2);
    k_refresh<<<nblk(N_PARAMS), 256, 0, st>>>(f->master, f->wb, f->wpt);
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

extern "C" int optifax_ff_encode(const void* spectra, int64_t stride, int32_t n_spectra, int32_t n_points, int32_t k0,
                                 int32_t n_bins, int32_t split, float pump_scale, const float* sigma_in, float* x,
                                 int32_t n_channels, float* sigma_out, void* stream) {
    if (!spectra || !x || n_spectra < 1 || n_points < 1 || n_bins < 1 || n_bins > n_points || k0 < 0 ||
        k0 >= n_points || split < 0 || split > n_bins || stride < n_points || !(pump_scale > 0.f) ||
        (n_channels != 4 && n_channels != 6))
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    k_ff_encode<<<n_spectra, 1024, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float2*>(spectra), stride, n_points, k0, n_bins, split, pump_scale, sigma_in, x, n_channels,
        sigma_out);
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

extern "C" int optifax_ff_step(const float* y, const float* sigma, const void* X_in, const void* feedback,
                               const void* pump, const void* lin, const float* tally_w, int32_t n_points, int32_t k0,
                               int32_t n_bins, int32_t split, float pump_scale, void* X_out, void* Y_next,
                               double* energy, void* stream) {
    if ((!y && !X_in) || (y && !sigma) || !feedback || !pump || !Y_next || n_points < 1 || n_bins < 1 ||
        n_bins > n_points || k0 < 0 || k0 >= n_points || split < 0 || split > n_bins || !(pump_scale > 0.f))
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (energy && cudaMemsetAsync(energy, 0, sizeof(double), st) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    k_ff_step<<<nblk(n_points), 256, 0, st>>>(y, sigma, static_cast<const float2*>(X_in),
                                              static_cast<const float2*>(feedback), static_cast<const float2*>(pump),
                                              static_cast<const float2*>(lin), tally_w, n_points, k0, n_bins, split,
                                              pump_scale, static_cast<float2*>(X_out), static_cast<float2*>(Y_next),
                                              energy);
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

namespace {
int env_args(int32_t n_points, int32_t n_bins, const int32_t* band, EnvBand* bp, EnvBand* bs, int* logL) {
    if (!band || n_points < 1 || n_bins < 2 || n_bins > 4096 || (n_bins & (n_bins - 1)) || n_bins > n_points)
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    *bp = {band[0], band[1], band[2]};
    *bs = {band[3], band[4], band[5]};
    for (const EnvBand* b : {bp, bs})
        if (b->kc < 0 || b->kc >= n_points || b->lo < -n_bins / 2 || b->hi > n_bins / 2 || b->lo >= b->hi)
            return OPTIFAX_ERR_INVALID_ARGUMENT;
    int l = 0;
    while ((1 << l) < n_bins) ++l;
    *logL = l;
    return OPTIFAX_OK;
}
}  // namespace

extern "C" int optifax_ff_encode_env(const void* spectra, int64_t stride, int32_t n_spectra, int32_t n_points,
                                     int32_t n_bins, const int32_t* band, float pump_scale, const float* sigma_in,
                                     float* x, int32_t n_channels, float* sigma_out, void* stream) {
    EnvBand bp, bs;
    int logL = 0;
    if (!spectra || !x || n_spectra < 1 || stride < n_points || !(pump_scale > 0.f) ||
        (n_channels != 4 && n_channels != 6))
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    int rc = env_args(n_points, n_bins, band, &bp, &bs, &logL);
    if (rc) return rc;
    k_ff_encode_env<<<dim3(n_spectra, 2), 512, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float2*>(spectra), stride, n_points, n_bins, logL, bp, bs, pump_scale, sigma_in, x,
        n_channels, sigma_out);
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

extern "C" int optifax_ff_decode_env(const float* y, const float* sigma, int32_t n_points, int32_t n_bins,
                                     const int32_t* band, float pump_scale, void* X_out, void* stream) {
    EnvBand bp, bs;
    int logL = 0;
    if (!y || !sigma || !X_out || !(pump_scale > 0.f)) return OPTIFAX_ERR_INVALID_ARGUMENT;
    int rc = env_args(n_points, n_bins, band, &bp, &bs, &logL);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(X_out, 0, sizeof(float2) * (size_t)n_points, st) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    k_ff_decode_env<<<2, 512, 0, st>>>(y, sigma, n_points, n_bins, logL, bp, bs, pump_scale,
                                       static_cast<float2*>(X_out));
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}
