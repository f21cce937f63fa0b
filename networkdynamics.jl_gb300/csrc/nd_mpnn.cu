// Learned warm start for swing-network steady states: a message-passing network on one
// fixed graph maps per-instance power injections P and line weights K to steady-state
// phases, trained and evaluated by the kernels below (FP32).  It has no counterpart in
// the reference, whose find_fixpoint (src/initialization.jl:44-144) starts Newton from a
// caller-given guess; its prediction only replaces that guess.
//
// Architecture (hidden width H = 64, L layers), per instance b and vertex i:
//   s_i  = Σ_j K_ij / κ                        (κ = kWeightScale; j over the neighbours)
//   x_i  = [P_i, log(1 + s_i)]
//   h0_i = tanh(W_in x_i + b_in)
//   m    = M^k h,  (M h)_i = (1 / s_i) Σ_j (K_ij / κ) h_j    (k = hops weighted-mean steps)
//   a_i  = tanh(W_s h_i + W_m m_i + b),  h'_i = h_i + a_i          (L residual layers)
//   y_i  = w_out · h_i + b_out,  θ̂_i = y_i - mean_i(y)          (phases up to a shift)
// The steady-state frequency is ω* = 0 at every fixpoint of the swing equations, so only
// θ is predicted.  Loss = mean over instances and vertices of (θ̂ - (θ* - mean θ*))².
//
// Parameters are one flat FP32 vector: W_in[H][2], b_in[H], per layer W_s[H][H],
// W_m[H][H], b[H] (row = output unit), then w_out[H], b_out.  Rows of every activation
// array are r = b * nv + i with H contiguous floats.  Weight gradients are reduced as
// fixed per-block partials followed by an ordered sum, so a training run is
// deterministic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "nd_internal.h"

namespace nd {
namespace mpnn {

constexpr int kH = 64;
constexpr float kWeightScale = 10.0f;
constexpr int kBlock = 256;
constexpr int kTileRows = 64;                // rows per block in the dense layer kernels
constexpr int kGradBlocks = 304;             // blocks of the weight-gradient reductions
constexpr int kPartialStride = 2 * kH * kH + kH;
constexpr int kDenseSmem = (2 * kH * kH + kTileRows * (2 * kH + 1)) * (int)sizeof(float);

__host__ __device__ inline int64_t off_win() { return 0; }
__host__ __device__ inline int64_t off_bin() { return 2 * kH; }
__host__ __device__ inline int64_t off_layer(int l) { return 3 * kH + (int64_t)l * (2 * kH * kH + kH); }
__host__ __device__ inline int64_t off_wout(int L) { return off_layer(L); }
__host__ __device__ inline int64_t off_bout(int L) { return off_layer(L) + kH; }
inline int64_t num_params(int L) { return off_bout(L) + 1; }

__host__ __device__ inline int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }

inline unsigned grid_for(int64_t n, int block = kBlock) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + block - 1) / block, 152 * 16));
}

// ---- forward --------------------------------------------------------------------------------

// x = [P, log1p(s)], inv_s = 1 / s (0 for isolated vertices)
__global__ void features_kernel(int64_t R, int64_t nv, int64_t ne, const uint32_t* __restrict__ row_ptr,
                                const int32_t* __restrict__ eid, const float* __restrict__ P,
                                const float* __restrict__ K, float* __restrict__ x, float* __restrict__ inv_s) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < R; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = r / nv, i = r - b * nv;
        float s = 0.f;
        for (uint32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) s += K[b * ne + eid[k]] / kWeightScale;
        x[2 * r] = P[r];
        x[2 * r + 1] = log1pf(s);
        inv_s[r] = s > 0.f ? 1.f / s : 0.f;
    }
}

// h0 = tanh(W_in x + b_in), a thread per (row, unit)
__global__ void encode_kernel(int64_t R, const float* __restrict__ x, const float* __restrict__ prm,
                              float* __restrict__ h0) {
    const float* W = prm + off_win();
    const float* bb = prm + off_bin();
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < R * kH; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / kH;
        const int o = (int)(t - r * kH);
        h0[t] = tanhf(fmaf(W[2 * o], x[2 * r], fmaf(W[2 * o + 1], x[2 * r + 1], bb[o])));
    }
}

// out_r (=, or += with accumulate) post_r · Σ_k (K_k / κ) · pre_n · in_n over the neighbours
// n of row r (pre / post may be NULL = 1).  A warp per row, two units per lane.
__global__ void aggregate_kernel(int64_t R, int64_t nv, int64_t ne, const uint32_t* __restrict__ row_ptr,
                                 const int32_t* __restrict__ nbr, const int32_t* __restrict__ eid,
                                 const float* __restrict__ K, const float* __restrict__ pre,
                                 const float* __restrict__ post, const float* __restrict__ in, float* __restrict__ out,
                                 int accumulate) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < R; r += warps) {
        const int64_t b = r / nv, i = r - b * nv;
        float2 acc = make_float2(0.f, 0.f);
        for (uint32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            const int64_t n = b * nv + nbr[k];
            float w = K[b * ne + eid[k]] / kWeightScale;
            if (pre) w *= pre[n];
            const float2 hv = reinterpret_cast<const float2*>(in + n * kH)[lane];
            acc.x = fmaf(w, hv.x, acc.x);
            acc.y = fmaf(w, hv.y, acc.y);
        }
        if (post) {
            const float sc = post[r];
            acc.x *= sc;
            acc.y *= sc;
        }
        float2* o = reinterpret_cast<float2*>(out + r * kH) + lane;
        if (accumulate) {
            const float2 prev = *o;
            acc.x += prev.x;
            acc.y += prev.y;
        }
        *o = acc;
    }
}

// One residual layer forward for a tile of 64 rows: a = tanh([h | m] · Wᵀ + b), h' = h + a.
// Shared memory: Wt[128][64] (Wt[i][o] = W_s[o][i] for i < 64, W_m[o][i-64] above) and the
// input tile [64][129].  Each thread computes 16 units of one row.
__global__ void __launch_bounds__(kBlock) layer_forward_kernel(int64_t R, const float* __restrict__ h,
                                                               const float* __restrict__ m,
                                                               const float* __restrict__ Wl, float* __restrict__ a,
                                                               float* __restrict__ hn) {
    extern __shared__ __align__(16) float smem[];
    float* Wt = smem;                  // [2H][H]
    float* tile = smem + 2 * kH * kH;  // [kTileRows][2H + 1]
    const float* Ws = Wl;
    const float* Wm = Wl + kH * kH;
    const float* bias = Wl + 2 * kH * kH;
    const int tid = threadIdx.x;
    for (int t = tid; t < 2 * kH * kH; t += kBlock) {
        const int i = t / kH, o = t - (t / kH) * kH;
        Wt[t] = i < kH ? Ws[o * kH + i] : Wm[o * kH + (i - kH)];
    }
    const int rr = tid >> 2, c0 = (tid & 3) * 16;
    float bj[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) bj[c] = bias[c0 + c];
    for (int64_t r0 = (int64_t)blockIdx.x * kTileRows; r0 < R; r0 += (int64_t)gridDim.x * kTileRows) {
        __syncthreads();
        for (int t = tid; t < kTileRows * 2 * kH; t += kBlock) {
            const int row = t / (2 * kH), i = t - row * (2 * kH);
            const int64_t r = r0 + row;
            float v = 0.f;
            if (r < R) v = i < kH ? h[r * kH + i] : m[r * kH + (i - kH)];
            tile[row * (2 * kH + 1) + i] = v;
        }
        __syncthreads();
        float acc[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) acc[c] = bj[c];
        const float* trow = tile + rr * (2 * kH + 1);
        for (int i = 0; i < 2 * kH; ++i) {
            const float xi = trow[i];
            const float4* w4 = reinterpret_cast<const float4*>(Wt + i * kH + c0);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 w = w4[q];
                acc[4 * q] = fmaf(xi, w.x, acc[4 * q]);
                acc[4 * q + 1] = fmaf(xi, w.y, acc[4 * q + 1]);
                acc[4 * q + 2] = fmaf(xi, w.z, acc[4 * q + 2]);
                acc[4 * q + 3] = fmaf(xi, w.w, acc[4 * q + 3]);
            }
        }
        const int64_t r = r0 + rr;
        if (r < R) {
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                const float av = tanhf(acc[c]);
                a[r * kH + c0 + c] = av;
                hn[r * kH + c0 + c] = trow[c0 + c] + av;
            }
        }
    }
}

// y_r = w_out · h_r + b_out, a warp per row
__global__ void decode_kernel(int64_t R, const float* __restrict__ h, const float* __restrict__ prm, int L,
                              float* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const float* w = prm + off_wout(L);
    const float b = prm[off_bout(L)];
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < R; r += warps) {
        const float2 hv = reinterpret_cast<const float2*>(h + r * kH)[lane];
        float s = fmaf(w[2 * lane], hv.x, w[2 * lane + 1] * hv.y);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) y[r] = s + b;
    }
}

// Fixed-order block sum (256 threads).
__device__ float block_sum(float v, float* red) {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int off = kBlock / 2; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    const float r = red[0];
    __syncthreads();
    return r;
}

// A block per instance: θ̂ = y - mean(y) into theta (if not NULL); with a target also the
// instance's loss term (into loss_part[b]) and dy = 2 (e - mean e) / count, e = θ̂ - (t - mean t).
__global__ void __launch_bounds__(kBlock) center_loss_kernel(int64_t nv, int64_t count, const float* __restrict__ y,
                                                             const float* __restrict__ target,
                                                             float* __restrict__ theta, float* __restrict__ dy,
                                                             float* __restrict__ loss_part) {
    __shared__ float red[kBlock];
    const int64_t b = blockIdx.x;
    const float* yb = y + b * nv;
    float s = 0.f;
    for (int64_t i = threadIdx.x; i < nv; i += kBlock) s += yb[i];
    const float ym = block_sum(s, red) / (float)nv;
    if (theta)
        for (int64_t i = threadIdx.x; i < nv; i += kBlock) theta[b * nv + i] = yb[i] - ym;
    if (!target) return;
    const float* tb = target + b * nv;
    s = 0.f;
    for (int64_t i = threadIdx.x; i < nv; i += kBlock) s += tb[i];
    const float tm = block_sum(s, red) / (float)nv;
    float l = 0.f, es = 0.f;
    for (int64_t i = threadIdx.x; i < nv; i += kBlock) {
        const float e = (yb[i] - ym) - (tb[i] - tm);
        l = fmaf(e, e, l);
        es += e;
    }
    const float lsum = block_sum(l, red);
    const float em = block_sum(es, red) / (float)nv;
    for (int64_t i = threadIdx.x; i < nv; i += kBlock) {
        const float e = (yb[i] - ym) - (tb[i] - tm);
        dy[b * nv + i] = 2.f * (e - em) / (float)count;
    }
    if (threadIdx.x == 0) loss_part[b] = lsum / (float)count;
}

// ---- backward -------------------------------------------------------------------------------

// dh_r = dy_r · w_out
__global__ void decode_back_kernel(int64_t R, const float* __restrict__ dy, const float* __restrict__ prm, int L,
                                   float* __restrict__ dh) {
    const float* w = prm + off_wout(L);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < R * kH; t += (int64_t)gridDim.x * blockDim.x)
        dh[t] = dy[t / kH] * w[t % kH];
}

// dz = dh ⊙ (1 - a²)
__global__ void tanh_back_kernel(int64_t n, const float* __restrict__ dh, const float* __restrict__ a,
                                 float* __restrict__ dz) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        dz[t] = dh[t] * (1.f - a[t] * a[t]);
}

// Input gradients of one layer for a tile of 64 rows: [g_h | g_m] = dz · [W_s | W_m];
// dh += g_h (the residual path already holds dh'), dmsc = g_m ⊙ inv_s (the scaled message
// gradient, aggregated into dh afterwards).  Each thread computes 32 of the 128 outputs.
__global__ void __launch_bounds__(kBlock) layer_backward_kernel(int64_t R, const float* __restrict__ dz,
                                                                const float* __restrict__ Wl,
                                                                const float* __restrict__ inv_s,
                                                                float* __restrict__ dh, float* __restrict__ dmsc) {
    extern __shared__ __align__(16) float smem[];
    float* Wc = smem;                  // [H][2H]: Wc[o][j] = W_s[o][j] (j < H), W_m[o][j - H]
    float* tile = smem + 2 * kH * kH;  // [kTileRows][H + 1]
    const float* Ws = Wl;
    const float* Wm = Wl + kH * kH;
    const int tid = threadIdx.x;
    for (int t = tid; t < 2 * kH * kH; t += kBlock) {
        const int o = t / (2 * kH), j = t - o * (2 * kH);
        Wc[t] = j < kH ? Ws[o * kH + j] : Wm[o * kH + (j - kH)];
    }
    const int rr = tid >> 2, c0 = (tid & 3) * 32;
    for (int64_t r0 = (int64_t)blockIdx.x * kTileRows; r0 < R; r0 += (int64_t)gridDim.x * kTileRows) {
        __syncthreads();
        for (int t = tid; t < kTileRows * kH; t += kBlock) {
            const int row = t / kH, o = t - row * kH;
            const int64_t r = r0 + row;
            tile[row * (kH + 1) + o] = r < R ? dz[r * kH + o] : 0.f;
        }
        __syncthreads();
        float acc[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) acc[c] = 0.f;
        const float* trow = tile + rr * (kH + 1);
        for (int o = 0; o < kH; ++o) {
            const float d = trow[o];
            const float4* w4 = reinterpret_cast<const float4*>(Wc + o * 2 * kH + c0);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float4 w = w4[q];
                acc[4 * q] = fmaf(d, w.x, acc[4 * q]);
                acc[4 * q + 1] = fmaf(d, w.y, acc[4 * q + 1]);
                acc[4 * q + 2] = fmaf(d, w.z, acc[4 * q + 2]);
                acc[4 * q + 3] = fmaf(d, w.w, acc[4 * q + 3]);
            }
        }
        const int64_t r = r0 + rr;
        if (r < R) {
            if (c0 < kH) {
#pragma unroll
                for (int c = 0; c < 32; ++c) dh[r * kH + c0 + c] += acc[c];
            } else {
                const float sc = inv_s[r];
#pragma unroll
                for (int c = 0; c < 32; ++c) dmsc[r * kH + (c0 - kH) + c] = acc[c] * sc;
            }
        }
    }
}

// Per-block partials of one layer's weight gradients over its row range:
// [o][i] Σ dz_o h_i, then [o][i] Σ dz_o m_i, then [o] Σ dz_o.  Thread t owns unit o = t / 4
// and inputs i0..i0+15, i0 = 16 (t % 4).
__global__ void __launch_bounds__(kBlock) layer_wgrad_kernel(int64_t R, const float* __restrict__ dz,
                                                             const float* __restrict__ h,
                                                             const float* __restrict__ m,
                                                             float* __restrict__ partial) {
    constexpr int kRows = 32;
    __shared__ float sdz[kRows][kH + 1], sh[kRows][kH], sm[kRows][kH];
    const int tid = threadIdx.x;
    const int o = tid >> 2, i0 = (tid & 3) * 16;
    const int64_t per = (R + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = (int64_t)blockIdx.x * per, r1 = imin64(R, r0 + per);
    float gs[16], gm[16], gb = 0.f;
#pragma unroll
    for (int c = 0; c < 16; ++c) gs[c] = gm[c] = 0.f;
    for (int64_t rb = r0; rb < r1; rb += kRows) {
        const int nr = (int)imin64(kRows, r1 - rb);
        __syncthreads();
        for (int t = tid; t < kRows * kH; t += kBlock) {
            const int row = t / kH, i = t - row * kH;
            const bool in = row < nr;
            sdz[row][i] = in ? dz[(rb + row) * kH + i] : 0.f;
            sh[row][i] = in ? h[(rb + row) * kH + i] : 0.f;
            sm[row][i] = in ? m[(rb + row) * kH + i] : 0.f;
        }
        __syncthreads();
        for (int row = 0; row < nr; ++row) {
            const float d = sdz[row][o];
            gb += d;
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                gs[c] = fmaf(d, sh[row][i0 + c], gs[c]);
                gm[c] = fmaf(d, sm[row][i0 + c], gm[c]);
            }
        }
    }
    float* out = partial + (int64_t)blockIdx.x * kPartialStride;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
        out[o * kH + i0 + c] = gs[c];
        out[kH * kH + o * kH + i0 + c] = gm[c];
    }
    if (i0 == 0) out[2 * kH * kH + o] = gb;
}

// Per-block partials of the encoder gradients: [o][k] Σ dz_o x_k (k < 2), then [o] Σ dz_o.
__global__ void encode_wgrad_kernel(int64_t R, const float* __restrict__ dz, const float* __restrict__ x,
                                    float* __restrict__ partial) {
    const int64_t per = (R + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = (int64_t)blockIdx.x * per, r1 = imin64(R, r0 + per);
    float* out = partial + (int64_t)blockIdx.x * kPartialStride;
    for (int t = threadIdx.x; t < 3 * kH; t += blockDim.x) {
        const int o = t / 3, k = t - o * 3;
        float s = 0.f;
        for (int64_t r = r0; r < r1; ++r) s = fmaf(dz[r * kH + o], k < 2 ? x[2 * r + k] : 1.f, s);
        if (k < 2) out[2 * o + k] = s;
        else out[2 * kH + o] = s;
    }
}

// Per-block partials of the decoder gradients: [i] Σ dy h_i, then Σ dy.
__global__ void decode_wgrad_kernel(int64_t R, const float* __restrict__ dy, const float* __restrict__ h,
                                    float* __restrict__ partial) {
    const int64_t per = (R + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = (int64_t)blockIdx.x * per, r1 = imin64(R, r0 + per);
    float* out = partial + (int64_t)blockIdx.x * kPartialStride;
    for (int i = threadIdx.x; i <= kH; i += blockDim.x) {
        float s = 0.f;
        for (int64_t r = r0; r < r1; ++r) s = fmaf(dy[r], i < kH ? h[r * kH + i] : 1.f, s);
        out[i] = s;
    }
}

// g[j] = Σ_blk partial[blk][j] in block order, j < n
__global__ void reduce_partials_kernel(int nblk, int n, const float* __restrict__ partial, float* __restrict__ g) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblk; ++b) s += partial[(int64_t)b * kPartialStride + j];
        g[j] = s;
    }
}

// loss = Σ_b loss_part[b] in order
__global__ void sum_loss_kernel(int64_t n, const float* __restrict__ part, float* __restrict__ loss) {
    __shared__ float red[kBlock];
    float s = 0.f;
    const int64_t per = (n + kBlock - 1) / kBlock;
    for (int64_t i = threadIdx.x * per; i < imin64(n, (threadIdx.x + 1) * per); ++i) s += part[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) *loss = s;
}

// Adam (Kingma & Ba 2015, Algorithm 1) with bias corrections c1 = 1 - β1^t, c2 = 1 - β2^t.
__global__ void adam_kernel(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace mpnn
}  // namespace nd

using namespace nd::mpnn;

struct nd_mpnn {
    int64_t nv = 0, ne = 0;
    int layers = 0;
    int hops = 1;  // weighted-mean steps per message (receptive field = layers * hops)
    int64_t nparams = 0;
    int device = 0;
    uint32_t* row_ptr = nullptr;  // [nv + 1] CSR over both endpoints of every edge
    int32_t* nbr = nullptr;       // [2 ne]
    int32_t* eid = nullptr;       // [2 ne]
    float* params = nullptr;
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    int64_t adam_t = 0;
    int64_t cap = 0;  // instances the activation buffers hold
    float* x = nullptr;      // [R][2]
    float* inv_s = nullptr;  // [R]
    float* h = nullptr;      // [L + 1][R][H]
    float* a = nullptr;      // [L][R][H]
    float* m = nullptr;      // [L][R][H]
    float* y = nullptr;      // [R]
    float* dy = nullptr;     // [R]
    float* dh = nullptr;     // [R][H]
    float* dz = nullptr;     // [R][H]
    float* dmsc = nullptr;   // [R][H]
    float* partial = nullptr;    // [kGradBlocks][kPartialStride]
    float* loss_part = nullptr;  // [cap]
};

namespace {

void free_batch(nd_mpnn* m) {
    float** bufs[] = {&m->x, &m->inv_s, &m->h, &m->a, &m->m, &m->y, &m->dy, &m->dh, &m->dz, &m->dmsc, &m->loss_part};
    for (float** b : bufs) {
        cudaFree(*b);
        *b = nullptr;
    }
    m->cap = 0;
}

cudaError_t ensure_batch(nd_mpnn* m, int64_t batch) {
    if (batch <= m->cap) return cudaSuccess;
    free_batch(m);
    const int64_t R = batch * m->nv;
    const int64_t L = m->layers;
    struct Want {
        float** p;
        int64_t n;
    } want[] = {{&m->x, 2 * R},          {&m->inv_s, R},         {&m->h, (L + 1) * R * kH}, {&m->a, L * R * kH},
                {&m->m, L * R * kH},     {&m->y, R},             {&m->dy, R},               {&m->dh, R * kH},
                {&m->dz, R * kH},        {&m->dmsc, R * kH},     {&m->loss_part, batch}};
    for (const Want& w : want) {
        cudaError_t err = cudaMalloc(w.p, sizeof(float) * std::max<int64_t>(w.n, 1));
        if (err != cudaSuccess) {
            free_batch(m);
            return err;
        }
    }
    m->cap = batch;
    return cudaSuccess;
}

cudaError_t set_dense_smem() {
    static std::once_flag once;
    static cudaError_t status = cudaSuccess;
    std::call_once(once, [] {
        status = cudaFuncSetAttribute(layer_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kDenseSmem);
        if (status == cudaSuccess)
            status =
                cudaFuncSetAttribute(layer_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kDenseSmem);
    });
    return status;
}

unsigned dense_grid(int64_t R) { return (unsigned)std::min<int64_t>((R + kTileRows - 1) / kTileRows, 152 * 3); }

// Forward pass over `batch` instances; with a target also the loss terms and dy.
cudaError_t forward(nd_mpnn* m, int64_t batch, const float* P, const float* K, const float* target, float* theta,
                    cudaStream_t s) {
    const int64_t R = batch * m->nv;
    const int L = m->layers;
    cudaError_t err = set_dense_smem();
    if (err != cudaSuccess) return err;
    features_kernel<<<grid_for(R), kBlock, 0, s>>>(R, m->nv, m->ne, m->row_ptr, m->eid, P, K, m->x, m->inv_s);
    encode_kernel<<<grid_for(R * kH), kBlock, 0, s>>>(R, m->x, m->params, m->h);
    for (int l = 0; l < L; ++l) {
        const float* hl = m->h + (int64_t)l * R * kH;
        float* ml = m->m + (int64_t)l * R * kH;
        // m = M^hops h, ping-ponging through the (idle in the forward pass) dz / dmsc buffers
        const float* src = hl;
        for (int k = 0; k < m->hops; ++k) {
            float* dst = k == m->hops - 1 ? ml : ((k & 1) ? m->dmsc : m->dz);
            aggregate_kernel<<<grid_for(R * 32), kBlock, 0, s>>>(R, m->nv, m->ne, m->row_ptr, m->nbr, m->eid, K,
                                                                 nullptr, m->inv_s, src, dst, 0);
            src = dst;
        }
        layer_forward_kernel<<<dense_grid(R), kBlock, kDenseSmem, s>>>(
            R, hl, ml, m->params + off_layer(l), m->a + (int64_t)l * R * kH, m->h + (int64_t)(l + 1) * R * kH);
    }
    decode_kernel<<<grid_for(R * 32), kBlock, 0, s>>>(R, m->h + (int64_t)L * R * kH, m->params, L, m->y);
    center_loss_kernel<<<(unsigned)batch, kBlock, 0, s>>>(m->nv, R, m->y, target, theta, m->dy, m->loss_part);
    return cudaGetLastError();
}

// Backward pass after forward() with a target: gradients into m->grads.
cudaError_t backward(nd_mpnn* m, int64_t batch, const float* K, cudaStream_t s) {
    const int64_t R = batch * m->nv;
    const int L = m->layers;
    float* G = m->grads;
    decode_wgrad_kernel<<<kGradBlocks, 128, 0, s>>>(R, m->dy, m->h + (int64_t)L * R * kH, m->partial);
    reduce_partials_kernel<<<1, 128, 0, s>>>(kGradBlocks, kH + 1, m->partial, G + off_wout(L));
    decode_back_kernel<<<grid_for(R * kH), kBlock, 0, s>>>(R, m->dy, m->params, L, m->dh);
    for (int l = L - 1; l >= 0; --l) {
        const float* al = m->a + (int64_t)l * R * kH;
        const float* hl = m->h + (int64_t)l * R * kH;
        const float* ml = m->m + (int64_t)l * R * kH;
        tanh_back_kernel<<<grid_for(R * kH), kBlock, 0, s>>>(R * kH, m->dh, al, m->dz);
        layer_wgrad_kernel<<<kGradBlocks, kBlock, 0, s>>>(R, m->dz, hl, ml, m->partial);
        reduce_partials_kernel<<<grid_for(kPartialStride), kBlock, 0, s>>>(kGradBlocks, kPartialStride, m->partial,
                                                                          G + off_layer(l));
        layer_backward_kernel<<<dense_grid(R), kBlock, kDenseSmem, s>>>(R, m->dz, m->params + off_layer(l), m->inv_s,
                                                                        m->dh, m->dmsc);
        // dh += (Mᵀ)^hops dm with Mᵀ x = A (x / s) (the weights are symmetric); dmsc already
        // holds dm / s, dz is free again as the second ping-pong buffer
        const float* src = m->dmsc;
        for (int k = 0; k < m->hops; ++k) {
            const bool last = k == m->hops - 1;
            float* dst = last ? m->dh : ((k & 1) ? m->dmsc : m->dz);
            aggregate_kernel<<<grid_for(R * 32), kBlock, 0, s>>>(R, m->nv, m->ne, m->row_ptr, m->nbr, m->eid, K,
                                                                 k == 0 ? nullptr : m->inv_s, nullptr, src, dst,
                                                                 last ? 1 : 0);
            src = dst;
        }
    }
    tanh_back_kernel<<<grid_for(R * kH), kBlock, 0, s>>>(R * kH, m->dh, m->h, m->dz);
    encode_wgrad_kernel<<<kGradBlocks, 192, 0, s>>>(R, m->dz, m->x, m->partial);
    reduce_partials_kernel<<<1, 192, 0, s>>>(kGradBlocks, 3 * kH, m->partial, G + off_win());
    return cudaGetLastError();
}

uint64_t splitmix64(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Glorot-uniform weights (scaled by 1/2 on the residual layers), zero biases.
std::vector<float> init_params(int L, uint64_t seed) {
    std::vector<float> p((size_t)num_params(L), 0.f);
    uint64_t st = seed;
    auto fill = [&](int64_t off, int64_t n, int fan_in, int fan_out, float gain) {
        const double a = gain * std::sqrt(6.0 / (fan_in + fan_out));
        for (int64_t k = 0; k < n; ++k) {
            const double u01 = (double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0);
            p[(size_t)(off + k)] = (float)((2.0 * u01 - 1.0) * a);
        }
    };
    fill(off_win(), 2 * kH, 2, kH, 1.f);
    for (int l = 0; l < L; ++l) {
        fill(off_layer(l), kH * kH, kH, kH, 0.5f);
        fill(off_layer(l) + kH * kH, kH * kH, kH, kH, 0.5f);
    }
    fill(off_wout(L), kH, kH, 1, 1.f);
    return p;
}

void destroy(nd_mpnn* m) {
    if (!m) return;
    free_batch(m);
    cudaFree(m->row_ptr);
    cudaFree(m->nbr);
    cudaFree(m->eid);
    cudaFree(m->params);
    cudaFree(m->grads);
    cudaFree(m->adam_m);
    cudaFree(m->adam_v);
    cudaFree(m->partial);
    delete m;
}

}  // namespace

extern "C" {

int nd_mpnn_create(int64_t nv, int64_t ne, const int64_t* src, const int64_t* dst, int layers, int hidden,
                   uint64_t seed, nd_mpnn** out) {
    nd::clear_error();
    if (!out) return nd::fail(ND_ERR_ARG, "nd_mpnn_create: out is NULL");
    *out = nullptr;
    if (nv <= 0 || ne < 0 || (ne > 0 && (!src || !dst)))
        return nd::fail(ND_ERR_ARG, "nd_mpnn_create: need nv > 0 and src / dst for ne > 0");
    if (hidden != kH) return nd::fail(ND_ERR_UNSUPPORTED, "nd_mpnn_create: the hidden width must be 64");
    if (layers < 1 || layers > 16) return nd::fail(ND_ERR_ARG, "nd_mpnn_create: layers must be in 1..16");
    if (nv > INT32_MAX || 2 * ne > UINT32_MAX) return nd::fail(ND_ERR_ARG, "nd_mpnn_create: graph too large");
    std::vector<uint32_t> rp((size_t)nv + 1, 0);
    for (int64_t e = 0; e < ne; ++e) {
        if (src[e] < 0 || src[e] >= nv || dst[e] < 0 || dst[e] >= nv)
            return nd::fail(ND_ERR_ARG, "nd_mpnn_create: edge endpoint out of range");
        ++rp[(size_t)src[e] + 1];
        ++rp[(size_t)dst[e] + 1];
    }
    for (int64_t v = 0; v < nv; ++v) rp[(size_t)v + 1] += rp[(size_t)v];
    std::vector<int32_t> nbr((size_t)(2 * ne)), eid((size_t)(2 * ne));
    std::vector<uint32_t> fillp(rp.begin(), rp.end() - 1);
    for (int64_t e = 0; e < ne; ++e) {
        const uint32_t a = fillp[(size_t)dst[e]]++;
        nbr[a] = (int32_t)src[e];
        eid[a] = (int32_t)e;
        const uint32_t b = fillp[(size_t)src[e]]++;
        nbr[b] = (int32_t)dst[e];
        eid[b] = (int32_t)e;
    }
    nd_mpnn* m = new nd_mpnn();
    m->nv = nv;
    m->ne = ne;
    m->layers = layers;
    m->nparams = num_params(layers);
    cudaGetDevice(&m->device);
    const std::vector<float> p0 = init_params(layers, seed);
    cudaError_t err;
    const size_t pb = sizeof(float) * (size_t)m->nparams;
    if ((err = cudaMalloc(&m->row_ptr, sizeof(uint32_t) * rp.size())) != cudaSuccess ||
        (err = cudaMalloc(&m->nbr, sizeof(int32_t) * std::max<size_t>(nbr.size(), 1))) != cudaSuccess ||
        (err = cudaMalloc(&m->eid, sizeof(int32_t) * std::max<size_t>(eid.size(), 1))) != cudaSuccess ||
        (err = cudaMalloc(&m->params, pb)) != cudaSuccess || (err = cudaMalloc(&m->grads, pb)) != cudaSuccess ||
        (err = cudaMalloc(&m->adam_m, pb)) != cudaSuccess || (err = cudaMalloc(&m->adam_v, pb)) != cudaSuccess ||
        (err = cudaMalloc(&m->partial, sizeof(float) * (size_t)kGradBlocks * kPartialStride)) != cudaSuccess ||
        (err = cudaMemcpy(m->row_ptr, rp.data(), sizeof(uint32_t) * rp.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (err = cudaMemcpy(m->nbr, nbr.data(), sizeof(int32_t) * nbr.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (err = cudaMemcpy(m->eid, eid.data(), sizeof(int32_t) * eid.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (err = cudaMemcpy(m->params, p0.data(), pb, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (err = cudaMemset(m->grads, 0, pb)) != cudaSuccess || (err = cudaMemset(m->adam_m, 0, pb)) != cudaSuccess ||
        (err = cudaMemset(m->adam_v, 0, pb)) != cudaSuccess) {
        destroy(m);
        return nd::cuda_fail(err, "nd_mpnn_create");
    }
    *out = m;
    return ND_OK;
}

int nd_mpnn_destroy(nd_mpnn* m) {
    nd::clear_error();
    destroy(m);
    return ND_OK;
}

int nd_mpnn_num_params(const nd_mpnn* m, int64_t* n) {
    nd::clear_error();
    if (!m || !n) return nd::fail(ND_ERR_ARG, "nd_mpnn_num_params: NULL argument");
    *n = m->nparams;
    return ND_OK;
}

int nd_mpnn_get_params(const nd_mpnn* m, float* dst, void* stream) {
    nd::clear_error();
    if (!m || !dst) return nd::fail(ND_ERR_ARG, "nd_mpnn_get_params: NULL argument");
    cudaError_t err = cudaMemcpyAsync(dst, m->params, sizeof(float) * (size_t)m->nparams, cudaMemcpyDefault,
                                      (cudaStream_t)stream);
    return err == cudaSuccess ? ND_OK : nd::cuda_fail(err, "nd_mpnn_get_params");
}

int nd_mpnn_set_params(nd_mpnn* m, const float* src, void* stream) {
    nd::clear_error();
    if (!m || !src) return nd::fail(ND_ERR_ARG, "nd_mpnn_set_params: NULL argument");
    cudaError_t err = cudaMemcpyAsync(m->params, src, sizeof(float) * (size_t)m->nparams, cudaMemcpyDefault,
                                      (cudaStream_t)stream);
    return err == cudaSuccess ? ND_OK : nd::cuda_fail(err, "nd_mpnn_set_params");
}

int nd_mpnn_get_grads(const nd_mpnn* m, float* dst, void* stream) {
    nd::clear_error();
    if (!m || !dst) return nd::fail(ND_ERR_ARG, "nd_mpnn_get_grads: NULL argument");
    cudaError_t err = cudaMemcpyAsync(dst, m->grads, sizeof(float) * (size_t)m->nparams, cudaMemcpyDefault,
                                      (cudaStream_t)stream);
    return err == cudaSuccess ? ND_OK : nd::cuda_fail(err, "nd_mpnn_get_grads");
}

int nd_mpnn_forward(nd_mpnn* m, int64_t batch, const float* P, const float* K, float* theta, void* stream) {
    nd::clear_error();
    if (!m || batch <= 0 || !P || (m->ne > 0 && !K) || !theta)
        return nd::fail(ND_ERR_ARG, "nd_mpnn_forward: bad arguments");
    cudaError_t err = ensure_batch(m, batch);
    if (err != cudaSuccess) return nd::fail(ND_ERR_NOMEM, "nd_mpnn_forward: activation buffers");
    err = forward(m, batch, P, K, nullptr, theta, (cudaStream_t)stream);
    return err == cudaSuccess ? ND_OK : nd::cuda_fail(err, "nd_mpnn_forward");
}

int nd_mpnn_loss_grad(nd_mpnn* m, int64_t batch, const float* P, const float* K, const float* theta_star, float* loss,
                      void* stream) {
    nd::clear_error();
    if (!m || batch <= 0 || !P || (m->ne > 0 && !K) || !theta_star || !loss)
        return nd::fail(ND_ERR_ARG, "nd_mpnn_loss_grad: bad arguments");
    cudaError_t err = ensure_batch(m, batch);
    if (err != cudaSuccess) return nd::fail(ND_ERR_NOMEM, "nd_mpnn_loss_grad: activation buffers");
    cudaStream_t s = (cudaStream_t)stream;
    if ((err = forward(m, batch, P, K, theta_star, nullptr, s)) != cudaSuccess ||
        (err = backward(m, batch, K, s)) != cudaSuccess)
        return nd::cuda_fail(err, "nd_mpnn_loss_grad");
    sum_loss_kernel<<<1, kBlock, 0, s>>>(batch, m->loss_part, loss);
    err = cudaGetLastError();
    return err == cudaSuccess ? ND_OK : nd::cuda_fail(err, "nd_mpnn_loss_grad");
}

int nd_mpnn_adam(nd_mpnn* m, double lr, double beta1, double beta2, double eps, void* stream) {
    nd::clear_error();
    if (!m || !(lr > 0) || !(beta1 >= 0 && beta1 < 1) || !(beta2 >= 0 && beta2 < 1) || !(eps > 0))
        return nd::fail(ND_ERR_ARG, "nd_mpnn_adam: bad arguments");
    ++m->adam_t;
    const double c1 = 1.0 - std::pow(beta1, (double)m->adam_t), c2 = 1.0 - std::pow(beta2, (double)m->adam_t);
    adam_kernel<<<grid_for(m->nparams), kBlock, 0, (cudaStream_t)stream>>>(
        m->nparams, m->params, m->grads, m->adam_m, m->adam_v, (float)lr, (float)beta1, (float)beta2, (float)eps,
        (float)c1, (float)c2);
    cudaError_t err = cudaGetLastError();
    return err == cudaSuccess ? ND_OK : nd::cuda_fail(err, "nd_mpnn_adam");
}

int nd_mpnn_set_hops(nd_mpnn* m, int hops) {
    nd::clear_error();
    if (!m || hops < 1 || hops > 64) return nd::fail(ND_ERR_ARG, "nd_mpnn_set_hops: hops must be in 1..64");
    m->hops = hops;
    return ND_OK;
}

int nd_mpnn_reset_optimizer(nd_mpnn* m, void* stream) {
    nd::clear_error();
    if (!m) return nd::fail(ND_ERR_ARG, "nd_mpnn_reset_optimizer: NULL handle");
    m->adam_t = 0;
    const size_t pb = sizeof(float) * (size_t)m->nparams;
    cudaError_t err = cudaMemsetAsync(m->adam_m, 0, pb, (cudaStream_t)stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(m->adam_v, 0, pb, (cudaStream_t)stream);
    return err == cudaSuccess ? ND_OK : nd::cuda_fail(err, "nd_mpnn_reset_optimizer");
}

}  // extern "C"
