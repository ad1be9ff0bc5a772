// nbh_diag.cu — diagnostics of each universe as GPU reductions
// (GPUBarnesHutNBodySimulation.java:305-365: printEnergy, printDepth, printImpulse).
//
// Per universe, in FP64: mass, mass-weighted position (centre of mass), momentum sum m v
// (printImpulse, :347-365), angular momentum sum m x cross v, kinetic energy sum m |v|^2/2
// (:318-324) and, on request, the potential energy sum over pairs i < j of -G m_i m_j / r,
// softened (r^2 + eps^2, the potential of the force the step integrates) and unsoftened (the
// form of :326-335, which adds each pair twice -- `2 * e` at :334 -- and is counted once
// here).  Reductions run in a fixed order (warp shuffles, then warps in order, then chunks
// in order), so the results do not depend on scheduling.
#include "nbh_common.cuh"
#include "nbh_kernels.h"

namespace nbh {

constexpr int kDiagThreads = 256;   // one block per 256-body chunk

// Sums v over the block into red[field] of thread 0's view, in a fixed order.
template <int F>
__device__ __forceinline__ void block_sum(double (&v)[F], double (*red)[F], double* out) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int f = 0; f < F; ++f)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[f] += __shfl_xor_sync(0xffffffffu, v[f], o);
    if (lane == 0)
#pragma unroll
        for (int f = 0; f < F; ++f) red[wid][f] = v[f];
    __syncthreads();
    if (threadIdx.x < F) {
        double a = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += red[w][threadIdx.x];
        out[threadIdx.x] = a;
    }
    __syncthreads();
}

// Moments of one chunk: fields 0..10 of its partial row.
__global__ void __launch_bounds__(kDiagThreads) diag_moments_kernel(const float4* __restrict__ node4,
                                                                    const float4* __restrict__ vel,
                                                                    const int4* __restrict__ chunks, double* part) {
    __shared__ double red[kDiagThreads / 32][kDiagMoments];
    const int4 ck = chunks[blockIdx.x];
    const int b = ck.y + threadIdx.x;
    double v[kDiagMoments];
#pragma unroll
    for (int f = 0; f < kDiagMoments; ++f) v[f] = 0.0;
    if (b < ck.z) {
        const float4 q = node4[b];
        const float4 w = vel[b];
        const double m = q.w, x = q.x, y = q.y, z = q.z, vx = w.x, vy = w.y, vz = w.z;
        v[0] = m;
        v[1] = m * x; v[2] = m * y; v[3] = m * z;
        v[4] = m * vx; v[5] = m * vy; v[6] = m * vz;
        v[7] = m * (y * vz - z * vy); v[8] = m * (z * vx - x * vz); v[9] = m * (x * vy - y * vx);
        v[10] = 0.5 * m * (vx * vx + vy * vy + vz * vz);
    }
    block_sum<kDiagMoments>(v, red, part + (size_t)blockIdx.x * kDiagFields);
}

// Pair potential of one chunk's bodies against every other body of their universe:
// fields 11 (softened) and 12 (unsoftened) of the chunk's row hold sum_i m_i phi_i, with
// phi_i = -sum_{j != i} m_j / r_ij; each pair appears twice, the caller halves.  Pair terms
// are FP32 (1/sqrt of the FP32 squared distance), summed per 256-source tile in FP32 and
// the tile sums in FP64.
__global__ void __launch_bounds__(kDiagThreads) diag_potential_kernel(const float4* __restrict__ node4,
                                                                      const int4* __restrict__ chunks,
                                                                      const int* __restrict__ ubody, float eps2,
                                                                      double* part) {
    __shared__ float4 tile[kDiagThreads];
    __shared__ double red[kDiagThreads / 32][2];
    const int4 ck = chunks[blockIdx.x];
    const int lo = ubody[ck.x], hi = ubody[ck.x + 1];
    const int i = ck.y + threadIdx.x;
    const bool valid = i < ck.z;
    const float4 qi = node4[valid ? i : ck.y];
    double ps = 0.0, pu = 0.0;
    for (int base = lo; base < hi; base += kDiagThreads) {
        const int j = base + threadIdx.x;
        __syncthreads();
        if (j < hi) tile[threadIdx.x] = node4[j];
        __syncthreads();
        const int cnt = min(kDiagThreads, hi - base);
        float ts = 0.0f, tu = 0.0f;
        for (int k = 0; k < cnt; ++k) {
            const float4 q = tile[k];
            const float dx = q.x - qi.x, dy = q.y - qi.y, dz = q.z - qi.z;
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const bool other = base + k != i;
            ts += other ? q.w * rsqrtf(r2 + eps2) : 0.0f;
            tu += other ? q.w * rsqrtf(r2) : 0.0f;
        }
        ps += ts;
        pu += tu;
    }
    double v[2] = {valid ? -(double)qi.w * ps : 0.0, valid ? -(double)qi.w * pu : 0.0};
    block_sum<2>(v, red, part + (size_t)blockIdx.x * kDiagFields + kDiagMoments);
}

// One block per universe: its chunks' rows summed in chunk order.
__global__ void __launch_bounds__(kDiagThreads) diag_reduce_kernel(const int4* __restrict__ chunks, int nchunks,
                                                                   const double* __restrict__ part, int fields,
                                                                   double* out) {
    __shared__ double red[kDiagThreads / 32][kDiagFields];
    const int u = blockIdx.x;
    // chunks are ordered by universe: binary search for [c0, c1)
    int a = 0, b = nchunks;
    while (a < b) {
        const int m = (a + b) >> 1;
        if (chunks[m].x < u) a = m + 1;
        else b = m;
    }
    const int c0 = a;
    b = nchunks;
    while (a < b) {
        const int m = (a + b) >> 1;
        if (chunks[m].x <= u) a = m + 1;
        else b = m;
    }
    const int c1 = a;
    double v[kDiagFields];
#pragma unroll
    for (int f = 0; f < kDiagFields; ++f) v[f] = 0.0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x)
#pragma unroll
        for (int f = 0; f < kDiagFields; ++f)
            if (f < fields) v[f] += part[(size_t)c * kDiagFields + f];
    block_sum<kDiagFields>(v, red, out + (size_t)u * kDiagFields);
}

void launch_diagnostics(const float4* node4, const float4* vel, const int4* chunks, int nchunks, const int* ubody,
                        int nuniv, bool potential, float eps2, double* part, double* out, cudaStream_t s) {
    diag_moments_kernel<<<nchunks, kDiagThreads, 0, s>>>(node4, vel, chunks, part);
    if (potential) diag_potential_kernel<<<nchunks, kDiagThreads, 0, s>>>(node4, chunks, ubody, eps2, part);
    diag_reduce_kernel<<<nuniv, kDiagThreads, 0, s>>>(chunks, nchunks, part,
                                                      potential ? kDiagFields : kDiagMoments, out);
}

}  // namespace nbh
