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
constexpr int kGradBlocks = 304;             // blocks of the weight-gradient reductions
constexpr int kPartialStride = 2 * kH * kH + kH;

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

// The dense layers are register-tiled FP32 products over tiles of kTileRowsD rows: thread
// (ty, tx) of a 16 x 16 block computes rows 8 ty .. 8 ty + 7 and units 4 tx .. 4 tx + 3,
// reading for every k eight tile values (broadcast along the warp) and one float4 of the
// weights, i.e. 32 FMAs per 9 shared-memory loads.  Tiles are loaded with float4 reads.
constexpr int kTileRowsD = 128;
constexpr int kLdA = 2 * kH + 4;  // padded row stride of the [h | m] tile
constexpr int kLdG = kH + 4;      // padded row stride of a dz tile
constexpr int kFwdSmem = (2 * kH * kH + kTileRowsD * kLdA) * (int)sizeof(float);
constexpr int kBwdSmem = (2 * kH * kH + kTileRowsD * kLdG) * (int)sizeof(float);

// One residual layer forward for a tile of rows: a = tanh([h | m] · Wᵀ + b), h' = h + a.
// Shared memory: Bt[128][64] (Bt[k][n] = W_s[n][k] for k < 64, W_m[n][k - 64] above) and the
// input tile [kTileRowsD][kLdA].
__global__ void __launch_bounds__(kBlock) layer_forward_kernel(int64_t R, const float* __restrict__ h,
                                                               const float* __restrict__ m,
                                                               const float* __restrict__ Wl, float* __restrict__ a,
                                                               float* __restrict__ hn) {
    extern __shared__ __align__(16) float smem[];
    float* Bt = smem;                  // [2H][H]
    float* As = smem + 2 * kH * kH;    // [kTileRowsD][kLdA]
    const float* Ws = Wl;
    const float* Wm = Wl + kH * kH;
    const float* bias = Wl + 2 * kH * kH;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    for (int t = tid; t < 2 * kH * kH; t += kBlock) {
        const int k = t / kH, n = t - (t / kH) * kH;
        Bt[t] = k < kH ? Ws[n * kH + k] : Wm[n * kH + (k - kH)];
    }
    const float4 bj = reinterpret_cast<const float4*>(bias)[tx];
    for (int64_t r0 = (int64_t)blockIdx.x * kTileRowsD; r0 < R; r0 += (int64_t)gridDim.x * kTileRowsD) {
        __syncthreads();
        // 128 rows x 32 float4 (16 of h, 16 of m)
#pragma unroll 4
        for (int f = tid; f < kTileRowsD * 32; f += kBlock) {
            const int row = f >> 5, qd = f & 31;
            const int64_t r = r0 + row;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r < R)
                v = qd < 16 ? reinterpret_cast<const float4*>(h + r * kH)[qd]
                            : reinterpret_cast<const float4*>(m + r * kH)[qd - 16];
            *reinterpret_cast<float4*>(As + row * kLdA + 4 * qd) = v;
        }
        __syncthreads();
        float acc[8][4];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            acc[i][0] = bj.x;
            acc[i][1] = bj.y;
            acc[i][2] = bj.z;
            acc[i][3] = bj.w;
        }
        const float* arow = As + (ty * 8) * kLdA;
#pragma unroll 4
        for (int k = 0; k < 2 * kH; ++k) {
            const float4 bv = reinterpret_cast<const float4*>(Bt + k * kH)[tx];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const float av = arow[i * kLdA + k];
                acc[i][0] = fmaf(av, bv.x, acc[i][0]);
                acc[i][1] = fmaf(av, bv.y, acc[i][1]);
                acc[i][2] = fmaf(av, bv.z, acc[i][2]);
                acc[i][3] = fmaf(av, bv.w, acc[i][3]);
            }
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int row = ty * 8 + i;
            const int64_t r = r0 + row;
            if (r < R) {
                const float4 hv = *reinterpret_cast<const float4*>(As + row * kLdA + 4 * tx);
                float4 av, nv;
                av.x = tanhf(acc[i][0]);
                av.y = tanhf(acc[i][1]);
                av.z = tanhf(acc[i][2]);
                av.w = tanhf(acc[i][3]);
                nv.x = hv.x + av.x;
                nv.y = hv.y + av.y;
                nv.z = hv.z + av.z;
                nv.w = hv.w + av.w;
                reinterpret_cast<float4*>(a + r * kH)[tx] = av;
                reinterpret_cast<float4*>(hn + r * kH)[tx] = nv;
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

// Input gradients of one layer for a tile of rows: g_h = dz · W_s and g_m = dz · W_m (the
// weights are [out][in], so dz · W needs no transpose); dh += g_h (the residual path already
// holds dh'), dmsc = g_m ⊙ inv_s (the scaled message gradient, aggregated into dh
// afterwards).  Register-tiled like the forward layer, the two products one after the other.
__global__ void __launch_bounds__(kBlock) layer_backward_kernel(int64_t R, const float* __restrict__ dz,
                                                                const float* __restrict__ Wl,
                                                                const float* __restrict__ inv_s,
                                                                float* __restrict__ dh, float* __restrict__ dmsc) {
    extern __shared__ __align__(16) float smem[];
    float* Bw = smem;                  // [2][H][H]: W_s then W_m, as stored
    float* As = smem + 2 * kH * kH;    // [kTileRowsD][kLdG]
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    for (int t = tid; t < 2 * kH * kH / 4; t += kBlock)
        reinterpret_cast<float4*>(Bw)[t] = reinterpret_cast<const float4*>(Wl)[t];
    for (int64_t r0 = (int64_t)blockIdx.x * kTileRowsD; r0 < R; r0 += (int64_t)gridDim.x * kTileRowsD) {
        __syncthreads();
#pragma unroll 4
        for (int f = tid; f < kTileRowsD * 16; f += kBlock) {
            const int row = f >> 4, qd = f & 15;
            const int64_t r = r0 + row;
            const float4 v = r < R ? reinterpret_cast<const float4*>(dz + r * kH)[qd] : make_float4(0.f, 0.f, 0.f, 0.f);
            *reinterpret_cast<float4*>(As + row * kLdG + 4 * qd) = v;
        }
        __syncthreads();
        const float* arow = As + (ty * 8) * kLdG;
#pragma unroll 1
        for (int part = 0; part < 2; ++part) {
            const float* B = Bw + part * kH * kH;
            float acc[8][4];
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll 4
            for (int k = 0; k < kH; ++k) {
                const float4 bv = reinterpret_cast<const float4*>(B + k * kH)[tx];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float av = arow[i * kLdG + k];
                    acc[i][0] = fmaf(av, bv.x, acc[i][0]);
                    acc[i][1] = fmaf(av, bv.y, acc[i][1]);
                    acc[i][2] = fmaf(av, bv.z, acc[i][2]);
                    acc[i][3] = fmaf(av, bv.w, acc[i][3]);
                }
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int64_t r = r0 + ty * 8 + i;
                if (r >= R) continue;
                if (part == 0) {
                    float4* o = reinterpret_cast<float4*>(dh + r * kH) + tx;
                    float4 v = *o;
                    v.x += acc[i][0];
                    v.y += acc[i][1];
                    v.z += acc[i][2];
                    v.w += acc[i][3];
                    *o = v;
                } else {
                    const float sc = inv_s[r];
                    reinterpret_cast<float4*>(dmsc + r * kH)[tx] =
                        make_float4(acc[i][0] * sc, acc[i][1] * sc, acc[i][2] * sc, acc[i][3] * sc);
                }
            }
        }
    }
}

// Per-block partials of one layer's weight gradients over its row range:
// [o][i] Σ dz_o h_i, then [o][i] Σ dz_o m_i, then [o] Σ dz_o.  Thread (to, ti) owns units
// 4 to .. 4 to + 3 and inputs 4 ti .. 4 ti + 3 of both matrices: per row three float4 loads
// from the staged tiles feed 32 FMAs.
__global__ void __launch_bounds__(kBlock) layer_wgrad_kernel(int64_t R, const float* __restrict__ dz,
                                                             const float* __restrict__ h,
                                                             const float* __restrict__ m,
                                                             float* __restrict__ partial) {
    constexpr int kRows = 64;
    __shared__ __align__(16) float sdz[kRows][kH], sh[kRows][kH], sm[kRows][kH];
    const int tid = threadIdx.x, ti = tid & 15, to = tid >> 4;
    const int64_t per = (R + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = (int64_t)blockIdx.x * per, r1 = imin64(R, r0 + per);
    float gs[4][4], gm[4][4], gb[4];
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        gb[x] = 0.f;
#pragma unroll
        for (int z = 0; z < 4; ++z) gs[x][z] = gm[x][z] = 0.f;
    }
    for (int64_t rb = r0; rb < r1; rb += kRows) {
        const int nr = (int)imin64(kRows, r1 - rb);
        __syncthreads();
        for (int f = tid; f < kRows * 16; f += kBlock) {
            const int row = f >> 4, qd = f & 15;
            const bool in = row < nr;
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            reinterpret_cast<float4*>(sdz[row])[qd] = in ? reinterpret_cast<const float4*>(dz + (rb + row) * kH)[qd] : z4;
            reinterpret_cast<float4*>(sh[row])[qd] = in ? reinterpret_cast<const float4*>(h + (rb + row) * kH)[qd] : z4;
            reinterpret_cast<float4*>(sm[row])[qd] = in ? reinterpret_cast<const float4*>(m + (rb + row) * kH)[qd] : z4;
        }
        __syncthreads();
        for (int row = 0; row < nr; ++row) {
            const float4 d = reinterpret_cast<const float4*>(sdz[row])[to];
            const float4 hv = reinterpret_cast<const float4*>(sh[row])[ti];
            const float4 mv = reinterpret_cast<const float4*>(sm[row])[ti];
            const float dd[4] = {d.x, d.y, d.z, d.w};
            const float hh[4] = {hv.x, hv.y, hv.z, hv.w};
            const float mm[4] = {mv.x, mv.y, mv.z, mv.w};
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                gb[x] += dd[x];
#pragma unroll
                for (int z = 0; z < 4; ++z) {
                    gs[x][z] = fmaf(dd[x], hh[z], gs[x][z]);
                    gm[x][z] = fmaf(dd[x], mm[z], gm[x][z]);
                }
            }
        }
    }
    float* out = partial + (int64_t)blockIdx.x * kPartialStride;
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const int o = 4 * to + x;
        reinterpret_cast<float4*>(out + o * kH)[ti] = make_float4(gs[x][0], gs[x][1], gs[x][2], gs[x][3]);
        reinterpret_cast<float4*>(out + kH * kH + o * kH)[ti] = make_float4(gm[x][0], gm[x][1], gm[x][2], gm[x][3]);
        if (ti == 0) out[2 * kH * kH + o] = gb[x];
    }
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
        status = cudaFuncSetAttribute(layer_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem);
        if (status == cudaSuccess)
            status =
                cudaFuncSetAttribute(layer_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kBwdSmem);
    });
    return status;
}

unsigned dense_grid(int64_t R) { return (unsigned)std::min<int64_t>((R + kTileRowsD - 1) / kTileRowsD, 152 * 2); }

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
        layer_forward_kernel<<<dense_grid(R), kBlock, kFwdSmem, s>>>(
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
        layer_backward_kernel<<<dense_grid(R), kBlock, kBwdSmem, s>>>(R, m->dz, m->params + off_layer(l), m->inv_s,
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
    ND_NVTX("nd_mpnn_forward");
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
    ND_NVTX("nd_mpnn_loss_grad");
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
    ND_NVTX("nd_mpnn_adam");
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
