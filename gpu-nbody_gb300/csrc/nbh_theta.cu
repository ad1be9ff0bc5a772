// nbh_theta.cu — learned per-body opening angle (no counterpart in the reference).
//
// A small MLP 12 -> 64 -> 64 -> 1 (ReLU) maps per-body features of the current tree and
// of the previous force walk to log(theta).  Inference runs once per step between the sort
// and the force stages: BF16 weights and activations on the tensor cores (mma.sync
// m16n8k16, FP32 accumulation), one warp per 32 bodies of the depth-first order.  Training
// uses the FP32 kernels at the end of this file (forward, backward, batch reductions, Adam).
//
// Parameter layout (row-major FP32, kMlpParams floats):
//   W1[64][12] b1[64] W2[64][64] b2[64] W3[64] b3
#include "nbh_common.cuh"
#include "nbh_kernels.h"
#include "nbh_theta.h"

#include <algorithm>

#include <cuda_bf16.h>

namespace nbh {

// ---- features -------------------------------------------------------------------------
// Per body, from the current tree (after sort) and the previous force walk (acc: previous
// acceleration, acc.w: its quadrupole error bound; theta_prev: the angle that walk used):
//   0 log10|a|             1 log10(bound/|a|)      2 log10 theta_prev
//   3 log10(d/R)           4 log10(n_leaf + 1)     5 level(leaf)/20
//   6 log10(n_up2 + 1)     7 log10(n_leaf/h^3)     8 log10(m_leaf/M)
//   9 log10(|a| d^2 / M)  10 log10(eps/h)         11 log10(h/d)
// d: distance to the universe's centre of mass, R and M: root half-width and mass, leaf:
// the cell holding the body, h: its half-width, up2: the leaf's parent (or the leaf if it
// is the root).
__device__ __forceinline__ void body_features(const StepParams& p, const ThetaDev& m, int b, int u, float4 a,
                                              float theta_prev, float f[kMlpIn]) {
    const int nbody = p.nbody;
    const float4 x = p.node4[b];
    const int root = p.nnodes - u;
    const float4 rc = p.node4[root];
    const float R = p.uradius[u];
    const float M = rc.w;
    const int leaf = p.parent[b];
    const int up = p.parent[leaf] >= 0 ? p.parent[leaf] : leaf;
    const int lv = p.clevel[leaf - nbody];
    const float h = ldexpf(R, -lv);
    const float nl = (float)p.count[leaf - nbody];
    const float nu = (float)p.count[up - nbody];
    const float ml = p.node4[leaf].w;
    const float dx = x.x - rc.x, dy = x.y - rc.y, dz = x.z - rc.z;
    const float d = sqrtf(dx * dx + dy * dy + dz * dz) + 1e-12f;
    const float am = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z) + 1e-30f;
    const float eps = sqrtf(p.eps2);
    f[0] = log10f(am);
    f[1] = log10f(fmaxf(a.w, 0.0f) / am + 1e-30f);
    f[2] = log10f(fmaxf(theta_prev, 1e-6f));
    f[3] = log10f(d / R + 1e-12f);
    f[4] = log10f(nl + 1.0f);
    f[5] = (float)lv * 0.05f;
    f[6] = log10f(nu + 1.0f);
    f[7] = log10f(nl / (h * h * h) + 1e-30f);
    f[8] = log10f(fmaxf(ml, 0.0f) / M + 1e-30f);
    f[9] = log10f(am * d * d / M + 1e-30f);
    f[10] = log10f(eps / h);
    f[11] = log10f(h / d);
}

// ---- BF16 tensor-core inference -------------------------------------------------------
__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const unsigned*>(&v);
}

__device__ __forceinline__ void mma_bf16(float c[4], const unsigned a[4], const unsigned b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr int kThetaThreads = 128;

// Shared-memory image of the model: weights as BF16 (W1 padded to K = 16, W3 as an 8 x 64
// tile whose row 0 is W3), biases FP32.
struct ThetaSmem {
    __nv_bfloat16 w1[kMlpHid * 16];
    __nv_bfloat16 w2[kMlpHid * kMlpHid];
    __nv_bfloat16 w3[8 * kMlpHid];
    float b1[kMlpHid];
    float b2[kMlpHid];
    float x[kThetaThreads / 32][32][16];   // normalized features of the warp's 32 bodies
};

// One warp: 32 bodies (rows) through the three layers.  Fragment layouts of
// mma.m16n8k16: A reg0 = (row g, k 2t..2t+1), reg1 = (row g+8, ...), reg2 = (row g, k+8),
// reg3 = (row g+8, k+8); B reg0 = (k 2t..2t+1, col g), reg1 = (k+8); C c0,c1 = (row g,
// cols 2t, 2t+1), c2,c3 = (row g+8).  A C tile pair (cols 16k..16k+15) is the A fragment
// of the next layer's k-tile k.
__device__ __forceinline__ void mlp_warp(const ThetaSmem& S, const float (*xs)[16], float b3, int lane,
                                         float out[2][2]) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const int r0 = mt * 16 + g, r1 = r0 + 8;
        unsigned a1[4];
        a1[0] = pack_bf16(xs[r0][2 * t], xs[r0][2 * t + 1]);
        a1[1] = pack_bf16(xs[r1][2 * t], xs[r1][2 * t + 1]);
        a1[2] = pack_bf16(xs[r0][2 * t + 8], xs[r0][2 * t + 9]);
        a1[3] = pack_bf16(xs[r1][2 * t + 8], xs[r1][2 * t + 9]);
        // layer 1
        unsigned a2[4][4];
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            float c[2][4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int nt = 2 * kt + h;
                const int n = nt * 8 + g;
                unsigned bf[2];
                bf[0] = *reinterpret_cast<const unsigned*>(&S.w1[n * 16 + 2 * t]);
                bf[1] = *reinterpret_cast<const unsigned*>(&S.w1[n * 16 + 2 * t + 8]);
                c[h][0] = c[h][1] = c[h][2] = c[h][3] = 0.f;
                mma_bf16(c[h], a1, bf);
                const float bb0 = S.b1[nt * 8 + 2 * t], bb1 = S.b1[nt * 8 + 2 * t + 1];
                c[h][0] = fmaxf(c[h][0] + bb0, 0.f);
                c[h][1] = fmaxf(c[h][1] + bb1, 0.f);
                c[h][2] = fmaxf(c[h][2] + bb0, 0.f);
                c[h][3] = fmaxf(c[h][3] + bb1, 0.f);
            }
            a2[kt][0] = pack_bf16(c[0][0], c[0][1]);
            a2[kt][1] = pack_bf16(c[0][2], c[0][3]);
            a2[kt][2] = pack_bf16(c[1][0], c[1][1]);
            a2[kt][3] = pack_bf16(c[1][2], c[1][3]);
        }
        // layer 2, with layer 3 folded in k-tile by k-tile
        float c3[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt3 = 0; kt3 < 4; ++kt3) {
            float c[2][4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int nt = 2 * kt3 + h;
                const int n = nt * 8 + g;
                c[h][0] = c[h][1] = c[h][2] = c[h][3] = 0.f;
#pragma unroll
                for (int kt = 0; kt < 4; ++kt) {
                    unsigned bf[2];
                    bf[0] = *reinterpret_cast<const unsigned*>(&S.w2[n * kMlpHid + kt * 16 + 2 * t]);
                    bf[1] = *reinterpret_cast<const unsigned*>(&S.w2[n * kMlpHid + kt * 16 + 2 * t + 8]);
                    mma_bf16(c[h], a2[kt], bf);
                }
                const float bb0 = S.b2[nt * 8 + 2 * t], bb1 = S.b2[nt * 8 + 2 * t + 1];
                c[h][0] = fmaxf(c[h][0] + bb0, 0.f);
                c[h][1] = fmaxf(c[h][1] + bb1, 0.f);
                c[h][2] = fmaxf(c[h][2] + bb0, 0.f);
                c[h][3] = fmaxf(c[h][3] + bb1, 0.f);
            }
            unsigned a3[4];
            a3[0] = pack_bf16(c[0][0], c[0][1]);
            a3[1] = pack_bf16(c[0][2], c[0][3]);
            a3[2] = pack_bf16(c[1][0], c[1][1]);
            a3[3] = pack_bf16(c[1][2], c[1][3]);
            unsigned bf[2];
            bf[0] = *reinterpret_cast<const unsigned*>(&S.w3[g * kMlpHid + kt3 * 16 + 2 * t]);
            bf[1] = *reinterpret_cast<const unsigned*>(&S.w3[g * kMlpHid + kt3 * 16 + 2 * t + 8]);
            mma_bf16(c3, a3, bf);
        }
        // column 0 of the output tile: thread t == 0 holds rows g (c3[0]) and g+8 (c3[2])
        out[mt][0] = c3[0] + b3;
        out[mt][1] = c3[2] + b3;
    }
}

__device__ __forceinline__ void load_model(ThetaSmem& S, const ThetaDev& m) {
    for (int i = threadIdx.x; i < kMlpHid * 16; i += blockDim.x) S.w1[i] = m.w1[i];
    for (int i = threadIdx.x; i < kMlpHid * kMlpHid; i += blockDim.x) S.w2[i] = m.w2[i];
    for (int i = threadIdx.x; i < 8 * kMlpHid; i += blockDim.x) S.w3[i] = m.w3[i];
    for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) {
        S.b1[i] = m.b1[i];
        S.b2[i] = m.b2[i];
    }
}

// Per-body theta of this step.  Up to the step at which the model was switched on
// (theta_since; the first step after a load) there is no previous walk with error bounds:
// every body gets the fixed theta.  Otherwise theta = clamp(exp(MLP(features)), min, max).
__global__ void __launch_bounds__(kThetaThreads) theta_kernel(StepParams p, const ThetaDev* __restrict__ mdl,
                                                              float* theta_out) {
    if (load_status(p.st)) return;
    __shared__ ThetaSmem S;
    const ThetaDev& m = *mdl;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int step = p.st->step;
    const bool use_fixed = step <= p.st->theta_since;   // no previous walk with bounds yet
    if (!use_fixed && !theta_model_step(p.st, step)) return;   // angles kept from the last evaluation
    const float fixed = sqrtf(p.theta2);
    if (!use_fixed) load_model(S, m);
    __syncthreads();
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int item = blockIdx.x * (blockDim.x >> 5) + wid; item < p.nwarps; item += warps) {
        const int2 wi = p.warps[item];
        const int u = wi.y;
        const int s = wi.x + lane;
        const bool valid = s < p.ubody[u + 1];
        const int b = p.sorted[valid ? s : wi.x];
        if (use_fixed) {
            if (valid) theta_out[b] = fixed;
            continue;
        }
        float f[kMlpIn];
        body_features(p, m, b, u, p.acc[b], theta_out[b], f);
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) S.x[wid][lane][k] = (f[k] - m.mean[k]) * m.inv_std[k];
#pragma unroll
        for (int k = kMlpIn; k < 16; ++k) S.x[wid][lane][k] = 0.f;
        __syncwarp();
        float out[2][2];
        mlp_warp(S, S.x[wid], m.b3, lane, out);
        __syncwarp();
        if ((lane & 3) == 0) {
            const int g = lane >> 2;
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int row = mt * 16 + g + 8 * h;
                    if (wi.x + row < p.ubody[u + 1]) {
                        const int br = p.sorted[wi.x + row];
                        theta_out[br] = fminf(fmaxf(__expf(out[mt][h]), m.theta_min), m.theta_max);
                    }
                }
        }
    }
}

// Raw features of every body (for training data and tests).  src: previous acceleration
// and bound per body; theta_prev: per-body angle of that walk.
__global__ void features_kernel(StepParams p, const ThetaDev* __restrict__ mdl, const float4* src,
                                const float* theta_prev, float* feat) {
    const int stride = gridDim.x * blockDim.x;
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < p.nbody; item += stride) {
        // position item of the depth-first order, so neighbouring threads share cells
        int u = 0;
        while (p.ubody[u + 1] <= item) ++u;
        const int b = p.sorted[item];
        float f[kMlpIn];
        body_features(p, *mdl, b, u, src[b], theta_prev[b], f);
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) feat[(size_t)b * kMlpIn + k] = f[k];
    }
}

// Model upload: FP32 parameters -> BF16 tiles + FP32 biases.
__global__ void model_convert_kernel(const float* __restrict__ prm, ThetaDev* mdl) {
    const float* W1 = prm;
    const float* b1 = W1 + kMlpHid * kMlpIn;
    const float* W2 = b1 + kMlpHid;
    const float* b2 = W2 + kMlpHid * kMlpHid;
    const float* W3 = b2 + kMlpHid;
    const float b3 = W3[kMlpHid];
    for (int i = threadIdx.x; i < kMlpHid * 16; i += blockDim.x) {
        const int n = i / 16, k = i % 16;
        mdl->w1[i] = __float2bfloat16_rn(k < kMlpIn ? W1[n * kMlpIn + k] : 0.f);
    }
    for (int i = threadIdx.x; i < kMlpHid * kMlpHid; i += blockDim.x) mdl->w2[i] = __float2bfloat16_rn(W2[i]);
    for (int i = threadIdx.x; i < 8 * kMlpHid; i += blockDim.x)
        mdl->w3[i] = __float2bfloat16_rn(i < kMlpHid ? W3[i] : 0.f);
    for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) {
        mdl->b1[i] = b1[i];
        mdl->b2[i] = b2[i];
    }
    if (threadIdx.x == 0) mdl->b3 = b3;
}

void launch_theta(const StepParams& p, const ThetaDev* mdl, float* theta_out, int grid, cudaStream_t s) {
    theta_kernel<<<grid, kThetaThreads, 0, s>>>(p, mdl, theta_out);
}
void launch_features(const StepParams& p, const ThetaDev* mdl, const float4* src, const float* theta_prev,
                     float* feat, int grid, cudaStream_t s) {
    features_kernel<<<grid, 256, 0, s>>>(p, mdl, src, theta_prev, feat);
}
void launch_model_convert(const float* prm, ThetaDev* mdl, cudaStream_t s) {
    model_convert_kernel<<<1, 256, 0, s>>>(prm, mdl);
}

// ---- FP32 training kernels ------------------------------------------------------------
// X: [kMlpIn][n] (feature-major), T: [n] targets (log theta), activations [kMlpHid][n].
constexpr int kTrainThreads = 128;

// Layer 1: H1 = relu(W1 x + b1).
__global__ void __launch_bounds__(kTrainThreads) mlp_fwd1_kernel(const float* __restrict__ prm,
                                                                 const float* __restrict__ X, int n, float* H1) {
    __shared__ float w[kMlpHid * kMlpIn + kMlpHid];
    for (int i = threadIdx.x; i < kMlpHid * kMlpIn + kMlpHid; i += blockDim.x) w[i] = prm[i];
    __syncthreads();
    const float* W1 = w;
    const float* b1 = W1 + kMlpHid * kMlpIn;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        float x[kMlpIn];
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) x[k] = X[(size_t)k * n + s];
#pragma unroll 4
        for (int j = 0; j < kMlpHid; ++j) {
            float a = b1[j];
#pragma unroll
            for (int k = 0; k < kMlpIn; ++k) a = fmaf(W1[j * kMlpIn + k], x[k], a);
            H1[(size_t)j * n + s] = fmaxf(a, 0.f);
        }
    }
}

// Layers 2 and 3: H2 = relu(W2 h1 + b2), y = W3 h2 + b3.
__global__ void __launch_bounds__(kTrainThreads) mlp_fwd2_kernel(const float* __restrict__ prm, int n,
                                                                 const float* __restrict__ H1, float* H2, float* Y) {
    __shared__ float w[kMlpHid * kMlpHid + 2 * kMlpHid + 1];
    const float* g = prm + kMlpHid * kMlpIn + kMlpHid;
    for (int i = threadIdx.x; i < kMlpHid * kMlpHid + 2 * kMlpHid + 1; i += blockDim.x) w[i] = g[i];
    __syncthreads();
    const float* W2 = w;
    const float* b2 = W2 + kMlpHid * kMlpHid;
    const float* W3 = b2 + kMlpHid;
    const float b3 = W3[kMlpHid];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        float h1[kMlpHid];
#pragma unroll
        for (int k = 0; k < kMlpHid; ++k) h1[k] = H1[(size_t)k * n + s];
        float y = b3;
#pragma unroll 1
        for (int j = 0; j < kMlpHid; ++j) {
            float a = b2[j];
#pragma unroll
            for (int k = 0; k < kMlpHid; ++k) a = fmaf(W2[j * kMlpHid + k], h1[k], a);
            a = fmaxf(a, 0.f);
            H2[(size_t)j * n + s] = a;
            y = fmaf(W3[j], a, y);
        }
        Y[s] = y;
    }
}

// Pinball (quantile q) loss on y vs target t, mean over the batch, and its back-propagation
// to the hidden layers: dY, dH2 = dY W3 (h2 > 0), dH1 = W2^T dH2 (h1 > 0).
__global__ void __launch_bounds__(kTrainThreads) mlp_bwd_kernel(const float* __restrict__ prm,
                                                                const float* __restrict__ T, int n, float q,
                                                                const float* H1, const float* H2,
                                                                const float* Y, float* dH1, float* dH2,
                                                                float* dY, float* loss) {
    __shared__ float w[kMlpHid * kMlpHid + kMlpHid];
    const float* W2g = prm + kMlpHid * kMlpIn + kMlpHid;
    const float* W3g = W2g + kMlpHid * kMlpHid + kMlpHid;
    for (int i = threadIdx.x; i < kMlpHid * kMlpHid; i += blockDim.x) w[i] = W2g[i];
    for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) w[kMlpHid * kMlpHid + i] = W3g[i];
    __syncthreads();
    const float* W2 = w;
    const float* W3 = w + kMlpHid * kMlpHid;
    float lsum = 0.f;
    const float inv_n = 1.0f / (float)n;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const float r = T[s] - Y[s];
        lsum += r > 0.f ? q * r : (q - 1.f) * r;
        const float dy = (r > 0.f ? -q : 1.f - q) * inv_n;
        dY[s] = dy;
        float dh2[kMlpHid];
#pragma unroll
        for (int j = 0; j < kMlpHid; ++j) {
            const float h = H2[(size_t)j * n + s];
            dh2[j] = h > 0.f ? dy * W3[j] : 0.f;
            dH2[(size_t)j * n + s] = dh2[j];
        }
        for (int k = 0; k < kMlpHid; ++k) {
            float a = 0.f;
#pragma unroll
            for (int j = 0; j < kMlpHid; ++j) a = fmaf(W2[j * kMlpHid + k], dh2[j], a);
            const float h = H1[(size_t)k * n + s];
            dH1[(size_t)k * n + s] = h > 0.f ? a : 0.f;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, lsum * inv_n);
}

// G[i][j] += sum_s A[i][s] * B[j][s] (B row rb == nullptr means a row of ones: bias
// gradients).  One block per (i-tile of 16, j-tile of 16, chunk of samples).
__global__ void __launch_bounds__(256) outer_reduce_kernel(const float* __restrict__ A, int ra,
                                                           const float* __restrict__ B, int rb, int n,
                                                           float* G, int ldg) {
    __shared__ float sa[16][65];
    __shared__ float sb[16][65];
    const int i0 = blockIdx.x * 16, j0 = blockIdx.y * 16;
    const int chunk = (n + gridDim.z - 1) / gridDim.z;
    const int s0 = blockIdx.z * chunk, s1 = min(n, s0 + chunk);
    const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
    float acc = 0.f;
    for (int base = s0; base < s1; base += 64) {
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            const int r = e / 64, c = e % 64, sidx = base + c;
            const bool in = sidx < s1;
            sa[r][c] = (in && i0 + r < ra) ? A[(size_t)(i0 + r) * n + sidx] : 0.f;
            float bv = 0.f;
            if (in && j0 + r < rb) bv = B ? B[(size_t)(j0 + r) * n + sidx] : 1.f;
            sb[r][c] = bv;
        }
        __syncthreads();
#pragma unroll 8
        for (int c = 0; c < 64; ++c) acc = fmaf(sa[ti][c], sb[tj][c], acc);
        __syncthreads();
    }
    if (i0 + ti < ra && j0 + tj < rb) atomicAdd(&G[(i0 + ti) * ldg + j0 + tj], acc);
}

__global__ void adam_kernel(float* prm, const float* g, float* m1, float* m2, int np, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = v;
        prm[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
    }
}

// One forward + backward pass: grad (kMlpParams, zeroed here) and loss of the batch.
void mlp_grad(const float* prm, const float* X, const float* T, int n, float q, MlpWork& w, float* grad, float* loss,
              cudaStream_t s) {
    const int grid = std::max(1, std::min((n + kTrainThreads - 1) / kTrainThreads, 1024));
    cudaMemsetAsync(grad, 0, sizeof(float) * kMlpParams, s);
    cudaMemsetAsync(loss, 0, sizeof(float), s);
    mlp_fwd1_kernel<<<grid, kTrainThreads, 0, s>>>(prm, X, n, w.H1);
    mlp_fwd2_kernel<<<grid, kTrainThreads, 0, s>>>(prm, n, w.H1, w.H2, w.Y);
    mlp_bwd_kernel<<<grid, kTrainThreads, 0, s>>>(prm, T, n, q, w.H1, w.H2, w.Y, w.dH1, w.dH2, w.dY, loss);
    float* gW1 = grad;
    float* gb1 = gW1 + kMlpHid * kMlpIn;
    float* gW2 = gb1 + kMlpHid;
    float* gb2 = gW2 + kMlpHid * kMlpHid;
    float* gW3 = gb2 + kMlpHid;
    float* gb3 = gW3 + kMlpHid;
    const int z = std::max(1, std::min(64, n / 2048));
    outer_reduce_kernel<<<dim3(4, 1, z), 256, 0, s>>>(w.dH1, kMlpHid, X, kMlpIn, n, gW1, kMlpIn);
    outer_reduce_kernel<<<dim3(4, 1, z), 256, 0, s>>>(w.dH1, kMlpHid, nullptr, 1, n, gb1, 1);
    outer_reduce_kernel<<<dim3(4, 4, z), 256, 0, s>>>(w.dH2, kMlpHid, w.H1, kMlpHid, n, gW2, kMlpHid);
    outer_reduce_kernel<<<dim3(4, 1, z), 256, 0, s>>>(w.dH2, kMlpHid, nullptr, 1, n, gb2, 1);
    outer_reduce_kernel<<<dim3(1, 4, z), 256, 0, s>>>(w.dY, 1, w.H2, kMlpHid, n, gW3, kMlpHid);
    outer_reduce_kernel<<<dim3(1, 1, z), 256, 0, s>>>(w.dY, 1, nullptr, 1, n, gb3, 1);
}

void mlp_forward(const float* prm, const float* X, int n, MlpWork& w, cudaStream_t s) {
    const int grid = std::max(1, std::min((n + kTrainThreads - 1) / kTrainThreads, 1024));
    mlp_fwd1_kernel<<<grid, kTrainThreads, 0, s>>>(prm, X, n, w.H1);
    mlp_fwd2_kernel<<<grid, kTrainThreads, 0, s>>>(prm, n, w.H1, w.H2, w.Y);
}

void adam_step(float* prm, const float* g, float* m1, float* m2, float lr, int t, cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
    adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(prm, g, m1, m2, kMlpParams, lr, b1, b2, 1e-8f, c1, c2);
}

}  // namespace nbh
