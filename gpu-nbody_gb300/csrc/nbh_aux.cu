// nbh_aux.cu — leapfrog integration, host<->device packing, the float4 export, the FP64
// direct sum used to measure force error, and the FP32 throughput probe.
#include "nbh_common.cuh"
#include "nbh_kernels.h"

#include <cstdint>

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

// The same as pack / unpack, reading or writing the caller's pinned host arrays directly
// (device-mapped pinned memory over NVLink-C2C): one launch in place of up to nine copies
// and a staging pass.  Null entries are skipped.  Each thread moves four consecutive bodies
// with 16-byte host accesses when every array is 16-byte aligned (vec4), else one body.
__global__ void pack_host_kernel(int n, HostArrays h, int mask, bool vec4, float4* node4, float4* vel,
                                 float4* acc) {
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (vec4) {
        for (int i4 = t0; 4 * i4 < n; i4 += stride) {
            const int i = 4 * i4;
            if (i + 3 >= n) {                         // ragged end: one body at a time
                for (int j = i; j < n; ++j) {
                    if (mask & 1) { float4 q = node4[j]; q.x = h.p[0][j]; q.y = h.p[1][j]; q.z = h.p[2][j]; node4[j] = q; }
                    if (mask & 2) vel[j] = make_float4(h.p[3][j], h.p[4][j], h.p[5][j], 0.f);
                    if (mask & 4) acc[j] = make_float4(h.p[6][j], h.p[7][j], h.p[8][j], 0.f);
                }
                continue;
            }
            if (mask & 1) {
                const float4 X = reinterpret_cast<const float4*>(h.p[0])[i4];
                const float4 Y = reinterpret_cast<const float4*>(h.p[1])[i4];
                const float4 Z = reinterpret_cast<const float4*>(h.p[2])[i4];
                const float xs[4] = {X.x, X.y, X.z, X.w}, ys[4] = {Y.x, Y.y, Y.z, Y.w}, zs[4] = {Z.x, Z.y, Z.z, Z.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    float4 q = node4[i + j];
                    q.x = xs[j]; q.y = ys[j]; q.z = zs[j];
                    node4[i + j] = q;
                }
            }
#pragma unroll
            for (int g = 0; g < 2; ++g) {
                if (!(mask & (2 << g))) continue;
                const float4 X = reinterpret_cast<const float4*>(h.p[3 + 3 * g])[i4];
                const float4 Y = reinterpret_cast<const float4*>(h.p[4 + 3 * g])[i4];
                const float4 Z = reinterpret_cast<const float4*>(h.p[5 + 3 * g])[i4];
                float4* out = g == 0 ? vel : acc;
                out[i] = make_float4(X.x, Y.x, Z.x, 0.f);
                out[i + 1] = make_float4(X.y, Y.y, Z.y, 0.f);
                out[i + 2] = make_float4(X.z, Y.z, Z.z, 0.f);
                out[i + 3] = make_float4(X.w, Y.w, Z.w, 0.f);
            }
        }
        return;
    }
    for (int i = t0; i < n; i += stride) {
        if (mask & 1) {
            float4 q = node4[i];
            q.x = h.p[0][i]; q.y = h.p[1][i]; q.z = h.p[2][i];
            node4[i] = q;
        }
        if (mask & 2) vel[i] = make_float4(h.p[3][i], h.p[4][i], h.p[5][i], 0.f);
        if (mask & 4) acc[i] = make_float4(h.p[6][i], h.p[7][i], h.p[8][i], 0.f);
    }
}

__global__ void unpack_host_kernel(int n, HostArrays h, bool vec4, const float4* node4, const float4* vel,
                                   const float4* acc) {
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (vec4) {
        for (int i4 = t0; 4 * i4 < n; i4 += stride) {
            const int i = 4 * i4;
            if (i + 3 >= n) {
                for (int j = i; j < n; ++j) {
                    const float4 q = node4[j], v = vel[j], a = acc[j];
                    const float vals[9] = {q.x, q.y, q.z, v.x, v.y, v.z, a.x, a.y, a.z};
#pragma unroll
                    for (int k = 0; k < 9; ++k)
                        if (h.p[k]) const_cast<float*>(h.p[k])[j] = vals[k];
                }
                continue;
            }
            float4 q[4], v[4], a[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                q[j] = node4[i + j];
                v[j] = vel[i + j];
                a[j] = acc[i + j];
            }
            const float4 out[9] = {make_float4(q[0].x, q[1].x, q[2].x, q[3].x), make_float4(q[0].y, q[1].y, q[2].y, q[3].y),
                                   make_float4(q[0].z, q[1].z, q[2].z, q[3].z), make_float4(v[0].x, v[1].x, v[2].x, v[3].x),
                                   make_float4(v[0].y, v[1].y, v[2].y, v[3].y), make_float4(v[0].z, v[1].z, v[2].z, v[3].z),
                                   make_float4(a[0].x, a[1].x, a[2].x, a[3].x), make_float4(a[0].y, a[1].y, a[2].y, a[3].y),
                                   make_float4(a[0].z, a[1].z, a[2].z, a[3].z)};
#pragma unroll
            for (int k = 0; k < 9; ++k)
                if (h.p[k]) reinterpret_cast<float4*>(const_cast<float*>(h.p[k]))[i4] = out[k];
        }
        return;
    }
    for (int i = t0; i < n; i += stride) {
        const float4 q = node4[i], v = vel[i], a = acc[i];
        const float vals[9] = {q.x, q.y, q.z, v.x, v.y, v.z, a.x, a.y, a.z};
#pragma unroll
        for (int k = 0; k < 9; ++k)
            if (h.p[k]) const_cast<float*>(h.p[k])[i] = vals[k];
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
static bool aligned16(const HostArrays& h) {
    for (const float* q : h.p)
        if (q && (reinterpret_cast<uintptr_t>(q) & 15)) return false;
    return true;
}
void launch_pack_host(int n, const HostArrays& h, int mask, float4* node4, float4* vel, float4* acc, int grid,
                      cudaStream_t s) {
    const bool v4 = aligned16(h);
    pack_host_kernel<<<v4 ? (grid + 3) / 4 : grid, 256, 0, s>>>(n, h, mask, v4, node4, vel, acc);
}
void launch_unpack_host(int n, const HostArrays& h, const float4* node4, const float4* vel, const float4* acc,
                        int grid, cudaStream_t s) {
    const bool v4 = aligned16(h);
    unpack_host_kernel<<<v4 ? (grid + 3) / 4 : grid, 256, 0, s>>>(n, h, v4, node4, vel, acc);
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
