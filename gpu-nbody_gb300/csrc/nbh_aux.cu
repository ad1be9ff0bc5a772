// nbh_aux.cu — leapfrog integration, host<->device packing, the float4 export, the FP64
// direct sum used to measure force error, and the FP32 throughput probe.
#include "nbh_common.cuh"
#include "nbh_kernels.h"

namespace nbh {

// -------------------------------------------------------------------------------------
// Integrate (integrate.cl:27-43): dv = a*dt*0.5; v' = v + dv; x += v'*dt; v = v' + dv.
// Precise mode: the drift v'*dt and the kick a*dt are Kahan-compensated sums.
template <bool REF, bool PRECISE>
__global__ void __launch_bounds__(256) integrate_kernel(StepParams p) {
    if (load_status(p.st)) return;
    const float dt = p.dt;
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.nbody; i += stride) {
        float4 x = p.node4[i];
        float4 v = p.vel[i];
        const float4 a = p.acc[i];
        const float dvx = __fmul_rn(__fmul_rn(a.x, dt), 0.5f);
        const float dvy = __fmul_rn(__fmul_rn(a.y, dt), 0.5f);
        const float dvz = __fmul_rn(__fmul_rn(a.z, dt), 0.5f);
        const float hx = __fadd_rn(v.x, dvx), hy = __fadd_rn(v.y, dvy), hz = __fadd_rn(v.z, dvz);
        if constexpr (PRECISE) {
            float4 kx = p.kpos[i], kv = p.kvel[i];
            float y1, t1;
            y1 = __fsub_rn(__fmul_rn(hx, dt), kx.x); t1 = __fadd_rn(x.x, y1); kx.x = __fsub_rn(__fsub_rn(t1, x.x), y1); x.x = t1;
            y1 = __fsub_rn(__fmul_rn(hy, dt), kx.y); t1 = __fadd_rn(x.y, y1); kx.y = __fsub_rn(__fsub_rn(t1, x.y), y1); x.y = t1;
            y1 = __fsub_rn(__fmul_rn(hz, dt), kx.z); t1 = __fadd_rn(x.z, y1); kx.z = __fsub_rn(__fsub_rn(t1, x.z), y1); x.z = t1;
            y1 = __fsub_rn(__fmul_rn(a.x, dt), kv.x); t1 = __fadd_rn(v.x, y1); kv.x = __fsub_rn(__fsub_rn(t1, v.x), y1); v.x = t1;
            y1 = __fsub_rn(__fmul_rn(a.y, dt), kv.y); t1 = __fadd_rn(v.y, y1); kv.y = __fsub_rn(__fsub_rn(t1, v.y), y1); v.y = t1;
            y1 = __fsub_rn(__fmul_rn(a.z, dt), kv.z); t1 = __fadd_rn(v.z, y1); kv.z = __fsub_rn(__fsub_rn(t1, v.z), y1); v.z = t1;
            p.kpos[i] = kx;
            p.kvel[i] = kv;
        } else {
            x.x = madd<REF>(hx, dt, x.x);
            x.y = madd<REF>(hy, dt, x.y);
            x.z = madd<REF>(hz, dt, x.z);
            v.x = __fadd_rn(hx, dvx);
            v.y = __fadd_rn(hy, dvy);
            v.z = __fadd_rn(hz, dvz);
        }
        p.node4[i] = x;
        p.vel[i] = v;
    }
}

// -------------------------------------------------------------------------------------
// SoA <-> float4 packing for nbh_load / nbh_write / nbh_read and the float4 export of
// copyvertices.cl:14-17.  mask bits: 1 pos, 2 vel, 4 acc, 8 mass.
__global__ void pack_kernel(int n, const float* __restrict__ soa, int mask, float4* node4,
                            float4* vel, float4* acc) {
    const int stride = gridDim.x * blockDim.x;
    const float* X = soa;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (mask & 9) {
            float4 q = node4[i];
            if (mask & 1) { q.x = X[i]; q.y = X[n + i]; q.z = X[2 * n + i]; }
            if (mask & 8) q.w = X[9 * n + i];
            node4[i] = q;
        }
        if (mask & 2) vel[i] = make_float4(X[3 * n + i], X[4 * n + i], X[5 * n + i], 0.f);
        if (mask & 4) acc[i] = make_float4(X[6 * n + i], X[7 * n + i], X[8 * n + i], 0.f);
    }
}

__global__ void unpack_kernel(int n, float* __restrict__ soa, const float4* node4, const float4* vel,
                              const float4* acc) {
    const int stride = gridDim.x * blockDim.x;
    float* X = soa;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float4 q = node4[i], v = vel[i], a = acc[i];
        X[i] = q.x; X[n + i] = q.y; X[2 * n + i] = q.z;
        X[3 * n + i] = v.x; X[4 * n + i] = v.y; X[5 * n + i] = v.z;
        X[6 * n + i] = a.x; X[7 * n + i] = a.y; X[8 * n + i] = a.z;
    }
}

__global__ void export4_kernel(int n, const float4* node4, const float4* vel, float4* pos4, float4* vel4) {
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (pos4) { float4 q = node4[i]; q.w = 1.0f; pos4[i] = q; }
        if (vel4) { float4 v = vel[i]; v.w = 1.0f; vel4[i] = v; }
    }
}

// -------------------------------------------------------------------------------------
// FP64 direct sum a_i = G sum_j m_j (x_j - x_i) / (|x_j - x_i|^2 + eps^2)^(3/2) for a list
// of bodies, each over the bodies [lo, hi) of its own universe.  Sources are split across
// blockIdx.y and the partial sums added atomically (outputs zeroed by the caller).
constexpr int kDirectTile = 256;
struct Src64 {
    double x, y, z, m;
};
__global__ void __launch_bounds__(kDirectTile) direct_f64_kernel(const float4* __restrict__ node4, int nidx,
                                                                 const int* __restrict__ idx,
                                                                 const int2* __restrict__ range, double eps2,
                                                                 double G, double* out) {
    __shared__ Src64 tile[kDirectTile];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = t < nidx;
    int i = 0;
    int2 rg = make_int2(0, 0);
    if (valid) {
        i = idx[t];
        rg = range[t];
    }
    // the block's source range: union of its targets' universes
    __shared__ int blo, bhi;
    if (threadIdx.x == 0) { blo = 0x7fffffff; bhi = 0; }
    __syncthreads();
    if (valid) { atomicMin(&blo, rg.x); atomicMax(&bhi, rg.y); }
    __syncthreads();
    const int lo = blo, hi = bhi;
    if (lo >= hi) return;
    const int len = hi - lo;
    const int per = (len + gridDim.y - 1) / gridDim.y;
    const int s0 = lo + blockIdx.y * per;
    const int s1 = min(hi, s0 + per);
    double xi = 0, yi = 0, zi = 0;
    if (valid) {
        const float4 q = node4[i];
        xi = q.x; yi = q.y; zi = q.z;
    }
    double sx = 0, sy = 0, sz = 0;
    for (int base = s0; base < s1; base += kDirectTile) {
        const int j = base + threadIdx.x;
        __syncthreads();
        if (j < s1) {
            const float4 q = node4[j];
            tile[threadIdx.x] = Src64{q.x, q.y, q.z, q.w};
        }
        __syncthreads();
        const int cnt = min(kDirectTile, s1 - base);
        if (valid) {
            for (int k = 0; k < cnt; ++k) {
                const int jj = base + k;
                if (jj < rg.x || jj >= rg.y) continue;
                const Src64 q = tile[k];
                const double dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
                const double d2 = dx * dx + dy * dy + dz * dz + eps2;
                const double inv = 1.0 / sqrt(d2);
                const double f = q.m * inv * inv * inv;
                sx += dx * f;
                sy += dy * f;
                sz += dz * f;
            }
        }
    }
    if (valid) {
        atomicAdd(out + 3 * t + 0, G * sx);
        atomicAdd(out + 3 * t + 1, G * sy);
        atomicAdd(out + 3 * t + 2, G * sz);
    }
}

// -------------------------------------------------------------------------------------
// FP32 FMA throughput probe: 8 independent dependency chains per thread keep the FMA
// pipes busy; the result is stored so nothing is optimised away.
__global__ void __launch_bounds__(256) fma_peak_kernel(float* sink, int iters) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
    const float b = 0.999f, c = 1e-4f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = __fmaf_rn(a[k], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    sink[(blockIdx.x * blockDim.x + threadIdx.x) & (1024 * 1024 - 1)] = s;
}

void launch_fma_peak(float* sink, int iters, int grid, int block, cudaStream_t s) {
    fma_peak_kernel<<<grid, block, 0, s>>>(sink, iters);
}

void launch_integrate(const StepParams& p, bool ref, int grid, cudaStream_t s) {
    if (ref) {
        if (p.precise) integrate_kernel<true, true><<<grid, 256, 0, s>>>(p);
        else integrate_kernel<true, false><<<grid, 256, 0, s>>>(p);
    } else {
        if (p.precise) integrate_kernel<false, true><<<grid, 256, 0, s>>>(p);
        else integrate_kernel<false, false><<<grid, 256, 0, s>>>(p);
    }
}

void launch_pack(int n, const float* soa, int mask, float4* node4, float4* vel, float4* acc, int grid,
                 cudaStream_t s) {
    pack_kernel<<<grid, 256, 0, s>>>(n, soa, mask, node4, vel, acc);
}
void launch_unpack(int n, float* soa, const float4* node4, const float4* vel, const float4* acc, int grid,
                   cudaStream_t s) {
    unpack_kernel<<<grid, 256, 0, s>>>(n, soa, node4, vel, acc);
}
void launch_export4(int n, const float4* node4, const float4* vel, float4* pos4, float4* vel4, int grid,
                    cudaStream_t s) {
    export4_kernel<<<grid, 256, 0, s>>>(n, node4, vel, pos4, vel4);
}
void launch_direct_f64(const float4* node4, int nidx, const int* idx, const int2* range, double eps2, double G,
                       double* out, int ysplit, cudaStream_t s) {
    dim3 grid((nidx + kDirectTile - 1) / kDirectTile, ysplit);
    direct_f64_kernel<<<grid, kDirectTile, 0, s>>>(node4, nidx, idx, range, eps2, G, out);
}

// Self-test of the bounded wait: waits on a flag that nothing changes and must come back
// with NBH_ERR_TIMEOUT in the status word (no fault, no hang), after which the context is
// still usable.
__global__ void wait_selftest_kernel(const int* flag, unsigned long long limit_ns, DevState* st) {
    if (threadIdx.x == 0 && blockIdx.x == 0) bounded_wait_ne(flag, kLock, limit_ns, st, 256, nullptr);
}

void launch_wait_selftest(const int* flag, unsigned long long limit_ns, DevState* st, cudaStream_t s) {
    wait_selftest_kernel<<<1, 32, 0, s>>>(flag, limit_ns, st);
}

}  // namespace nbh
