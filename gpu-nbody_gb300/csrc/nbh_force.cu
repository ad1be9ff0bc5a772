// nbh_force.cu — force traversal, leapfrog integration, host<->device packing and the
// FP64 direct sum used to measure force error.
#include "nbh_common.cuh"
#include "nbh_kernels.h"

namespace nbh {

constexpr int kForceThreads = 256;
constexpr int kForceWarps = kForceThreads / 32;

// Opening threshold of tree level L (root = 0): r^2/theta^2 * 4^-L + eps^2
// (calculateforce.cl:52-67; the reference's repeated *0.25 equals ldexp in the normal
// range and eps^2 absorbs the term below it).
__device__ __forceinline__ float level_dq(float t0, int level, float eps2) {
    return __fadd_rn(ldexpf(t0, -2 * level), eps2);
}

// -------------------------------------------------------------------------------------
// Force (calculateforce.cl:52-185).  A group of W lanes (W = 32: one warp; W = 16: the
// reference's work-group, :99,145) takes W consecutive bodies of the depth-first order and
// walks its universe's tree with one shared stack of (cell, next child) per level.  A body
// child is always accepted; a cell child only if every body of the group sees
// d^2 + eps^2 >= dq[level] (work_group_all, :145), else it is opened.  Children are
// compacted, so the first empty slot ends a cell.  The walk is depth-first in child order,
// so every body accumulates its interactions in the reference's order.  Work items (32
// bodies) are handed out dynamically for balance.  After the walk: the leapfrog velocity
// correction for step > 0 (:174-181) and the acceleration store (:183-185).
//
// REF: reference arithmetic (rounded products, 1/sqrt correctly rounded); otherwise FMA and
// the hardware inverse square root.  PB: per-body opening angle from theta_body.
template <int W, bool REF, bool PB>
__global__ void __launch_bounds__(kForceThreads) force_kernel(StepParams p) {
    if (load_status(p.st)) return;
    constexpr int kGroups = kForceWarps * (32 / W);
    __shared__ int s_node[kGroups][kMaxDepth];
    __shared__ int s_next[kGroups][kMaxDepth];
    const int lane = threadIdx.x & 31;
    const int grp = (threadIdx.x >> 5) * (32 / W) + lane / W;
    const unsigned gmask = (W == 32) ? 0xffffffffu : (0xffffu << (16 * (lane >> 4)));
    int* const snode = s_node[grp];
    int* const snext = s_next[grp];
    const int nbody = p.nbody;
    const float eps2 = p.eps2;
    const int step = p.st->step;
    const float4* __restrict__ node4 = p.node4;
    const int* __restrict__ child = p.child;
    unsigned long long my_inter = 0;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(&p.st->force_next, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= p.nwarps) break;
        const int2 wi = p.warps[item];
        const int u = wi.y;
        const int s = wi.x + lane;
        const bool valid = s < p.ubody[u + 1];
        int b = 0;
        float4 pb = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid) {
            b = p.sorted[s];
            pb = node4[b];
        }
        const float r = p.uradius[u];
        const float rr = __fmul_rn(r, r);
        float th2 = p.theta2;
        if constexpr (PB) {
            if (valid) {
                const float th = p.theta_body[b];
                th2 = __fmul_rn(th, th);
            }
        }
        const float t0 = th2 > 0.0f ? __fdiv_rn(rr, th2) : rr;
        float ax = 0.f, ay = 0.f, az = 0.f;
        int ninter = 0;

        if (__any_sync(gmask, valid)) {
            int depth = 0;
            int node = p.nnodes - u;
            int k = 0;
            float dq = level_dq(t0, 0, eps2);
            for (;;) {
                int ch = kNull;
                if (k < 8) ch = __ldg(child + ((size_t)(node - nbody) << 3) + k);
                if (ch < 0) {
                    // end of this cell (:165-171): back to the parent's next child
                    if (depth == 0) break;
                    --depth;
                    node = snode[depth];
                    k = snext[depth];
                    dq = level_dq(t0, depth, eps2);
                    continue;
                }
                ++k;
                const float4 q = __ldg(node4 + ch);
                const float dx = __fsub_rn(q.x, pb.x);
                const float dy = __fsub_rn(q.y, pb.y);
                const float dz = __fsub_rn(q.z, pb.z);
                float d2;
                if constexpr (REF)
                    d2 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)), eps2);
                else
                    d2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmaf_rn(dz, dz, eps2)));
                const bool accept = ch < nbody || __all_sync(gmask, !valid || d2 >= dq);
                if (accept) {
                    if (valid) {
                        float rd;
                        if constexpr (REF) rd = __fdiv_rn(1.0f, __fsqrt_rn(d2));
                        else rd = rsqrtf(d2);
                        const float f = __fmul_rn(__fmul_rn(__fmul_rn(q.w, rd), rd), rd);
                        ax = madd<REF>(dx, f, ax);
                        ay = madd<REF>(dy, f, ay);
                        az = madd<REF>(dz, f, az);
                        ++ninter;
                    }
                } else {
                    // open the cell (:155-163); every lane writes the same stack entry
                    if (depth + 1 >= kMaxDepth) {   // unreachable for a tree the build accepted
                        raise_error(p.st, NBH_ERR_DEPTH);
                        break;
                    }
                    snode[depth] = node;
                    snext[depth] = k;
                    ++depth;
                    node = ch;
                    k = 0;
                    dq = level_dq(t0, depth, eps2);
                }
            }
        }

        if (valid) {
            if (p.G != 1.0f) {
                ax = __fmul_rn(ax, p.G);
                ay = __fmul_rn(ay, p.G);
                az = __fmul_rn(az, p.G);
            }
            float4 v = p.vel[b];
            const float4 ao = p.acc[b];
            if (step > 0) {
                const float tx = __fmul_rn(__fsub_rn(ax, ao.x), p.dt);
                const float ty = __fmul_rn(__fsub_rn(ay, ao.y), p.dt);
                const float tz = __fmul_rn(__fsub_rn(az, ao.z), p.dt);
                if (p.precise) {
                    float4 kv = p.kvel[b];
                    float y1, t1;
                    y1 = __fsub_rn(__fmul_rn(tx, 0.5f), kv.x); t1 = __fadd_rn(v.x, y1); kv.x = __fsub_rn(__fsub_rn(t1, v.x), y1); v.x = t1;
                    y1 = __fsub_rn(__fmul_rn(ty, 0.5f), kv.y); t1 = __fadd_rn(v.y, y1); kv.y = __fsub_rn(__fsub_rn(t1, v.y), y1); v.y = t1;
                    y1 = __fsub_rn(__fmul_rn(tz, 0.5f), kv.z); t1 = __fadd_rn(v.z, y1); kv.z = __fsub_rn(__fsub_rn(t1, v.z), y1); v.z = t1;
                    p.kvel[b] = kv;
                } else {
                    v.x = madd<REF>(tx, 0.5f, v.x);
                    v.y = madd<REF>(ty, 0.5f, v.y);
                    v.z = madd<REF>(tz, 0.5f, v.z);
                }
                p.vel[b] = v;
            }
            p.acc[b] = make_float4(ax, ay, az, 0.0f);
            my_inter += (unsigned long long)ninter;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_inter += __shfl_xor_sync(0xffffffffu, my_inter, o);
    if (lane == 0 && my_inter) atomicAdd(&p.st->interactions, my_inter);
}

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

template <int W, bool REF>
static void launch_force_t(const StepParams& p, bool pb, int grid, cudaStream_t s) {
    if (pb) force_kernel<W, REF, true><<<grid, kForceThreads, 0, s>>>(p);
    else force_kernel<W, REF, false><<<grid, kForceThreads, 0, s>>>(p);
}

void launch_force(const StepParams& p, int vote, bool ref, int grid, cudaStream_t s) {
    const bool pb = p.theta_body != nullptr;
    if (vote == 16) {
        if (ref) launch_force_t<16, true>(p, pb, grid, s);
        else launch_force_t<16, false>(p, pb, grid, s);
    } else {
        if (ref) launch_force_t<32, true>(p, pb, grid, s);
        else launch_force_t<32, false>(p, pb, grid, s);
    }
}

int occupancy_force(int vote, bool ref, int* blocks_per_sm) {
    if (vote == 16)
        return ref ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_kernel<16, true, false>, kForceThreads, 0)
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_kernel<16, false, false>, kForceThreads, 0);
    return ref ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_kernel<32, true, false>, kForceThreads, 0)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_kernel<32, false, false>, kForceThreads, 0);
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

}  // namespace nbh
