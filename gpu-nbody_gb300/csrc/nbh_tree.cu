// nbh_tree.cu — bounding box, octree build, summarize and sort stages.
//
// Each stage restates one reference kernel (kernels/nbody/*.cl) and produces the same
// tree: same cells, same child order, same centres of mass and body order.  The
// scheduling is GB300-first: chunked grid-stride loops over float4 node records,
// warp-shuffle reductions, acquire/release atomics at device scope, bounded waits, and a
// wait-free bottom-up summarize in place of the reference's spin-waiting one.
#include "nbh_common.cuh"
#include "nbh_kernels.h"

#include <cfloat>

namespace nbh {

// -------------------------------------------------------------------------------------
// Bounding box (boundingbox.cl:43-196).  Every block folds chunks of one universe with
// warp shuffles and publishes them with atomicMin/atomicMax on order-preserving integer
// images of the floats (min/max are order independent, so the result equals the
// reference's tree reduction).  The last block to finish (ticket, as the reference's
// _blockCount) creates every root: centre 0.5*(min+max), half-width 0.5*max extent,
// empty children, start = the universe's first sorted position; it resets bottom and the
// per-step counters and increments the step counter (boundingbox.cl:170-195).
template <bool PRECISE>
__global__ void __launch_bounds__(256) bbox_kernel(StepParams p) {
    if (load_status(p.st)) return;
    __shared__ float red[6][8];
    __shared__ int last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int ci = blockIdx.x; ci < p.nchunks;) {
        // fold this block's consecutive chunks of one universe, then publish once
        const int u = p.chunks[ci].x;
        float v[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (; ci < p.nchunks && p.chunks[ci].x == u; ci += gridDim.x) {
            const int4 ck = p.chunks[ci];
            for (int i = ck.y + threadIdx.x; i < ck.z; i += blockDim.x) {
                const float4 q = p.node4[i];
                v[0] = fminf(v[0], q.x); v[1] = fminf(v[1], q.y); v[2] = fminf(v[2], q.z);
                v[3] = fmaxf(v[3], q.x); v[4] = fmaxf(v[4], q.y); v[5] = fmaxf(v[5], q.z);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 3; ++k) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
#pragma unroll
            for (int k = 3; k < 6; ++k) v[k] = fmaxf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
        }
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < 6; ++k) red[k][wid] = v[k];
        }
        __syncthreads();
        if (threadIdx.x < 6) {
            const int k = threadIdx.x;
            float a = red[k][0];
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
                a = k < 3 ? fminf(a, red[k][w]) : fmaxf(a, red[k][w]);
            unsigned* box = p.ubox + 6 * u;
            if (k < 3) atomicMin(box + k, f2ord(a));
            else atomicMax(box + k, f2ord(a));
        }
        __syncthreads();
    }
    __threadfence();
    if (threadIdx.x == 0) last = (atomicAdd(&p.st->bbox_ticket, 1) == (int)gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int u = threadIdx.x; u < p.nuniv; u += blockDim.x) {
        unsigned* box = p.ubox + 6 * u;
        float mn[3], mx[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            mn[k] = ord2f(atomicAdd(box + k, 0u));
            mx[k] = ord2f(atomicAdd(box + 3 + k, 0u));
        }
        float cx, cy, cz, radius;
        if constexpr (PRECISE) {
            double e = fmax(fmax((double)mx[0] - (double)mn[0], (double)mx[1] - (double)mn[1]),
                            (double)mx[2] - (double)mn[2]);
            cx = (float)(0.5 * ((double)mn[0] + (double)mx[0]));
            cy = (float)(0.5 * ((double)mn[1] + (double)mx[1]));
            cz = (float)(0.5 * ((double)mn[2] + (double)mx[2]));
            radius = (float)(0.5 * e);
        } else {
            cx = __fmul_rn(0.5f, __fadd_rn(mn[0], mx[0]));
            cy = __fmul_rn(0.5f, __fadd_rn(mn[1], mx[1]));
            cz = __fmul_rn(0.5f, __fadd_rn(mn[2], mx[2]));
            radius = __fmul_rn(0.5f, fmaxf(fmaxf(__fsub_rn(mx[0], mn[0]), __fsub_rn(mx[1], mn[1])),
                                           __fsub_rn(mx[2], mn[2])));
        }
        const int root = p.nnodes - u;
        const int k = root - p.nbody;
        p.node4[root] = make_float4(cx, cy, cz, -1.0f);
        int4* c4 = reinterpret_cast<int4*>(cell_child(p, root));
        c4[0] = make_int4(kNull, kNull, kNull, kNull);
        c4[1] = make_int4(kNull, kNull, kNull, kNull);
        p.parent[root] = -1;
        p.arrive[k] = 0;
        p.clevel[k] = 0;
        p.count[k] = 0;
        p.start[k] = p.ubody[u];
        p.uradius[u] = radius;
        // fresh extents for the next step
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            box[j] = 0xffffffffu;
            box[3 + j] = 0u;
        }
    }
    if (threadIdx.x == 0) {
        DevState* st = p.st;
        st->bottom = p.nnodes - p.nuniv + 1;
        st->bbox_ticket = 0;
        st->step += 1;
        st->force_next = 0;
        for (int j = 0; j < kDiagSlots; ++j) st->lock_waits[j] = st->cas_misses[j] = 0;
        st->interactions = 0ull;
    }
}

// -------------------------------------------------------------------------------------
// Octree build (buildtree.cl:42-199).  One thread per body descends from its universe's
// root by octant, locks the leaf slot with an acquire CAS (LOCK = -2, :97), and either
// stores the body (:98-101) or splits: cells are taken from the pool top-down with one
// atomic (:109), centred at parent - r/2 + bit*r (:124-136), the old body is re-inserted
// (:148-152) until the two bodies separate (:106-165).  The new subtree is published with
// one release store into the locked slot (:173-180), which orders every write made under
// the lock.  Failed locks retry from the same node (the tree only grows) with a bounded,
// backed-off wait.
//
// Insertion runs in three phases (three launches): first one body of every 256-body
// chunk, then one in 16, then the rest.  The octree of a set of bodies does not depend
// on the order the bodies arrive in, so the phases build exactly the tree a single pass
// would; what they change is contention.  In one pass every body of a universe that is
// resident at once descends into the same empty top levels and waits on each split there
// in turn (in a batch of small universes that is every body).  After the first two
// phases the top of each tree already holds about 1/16 of its bodies, so the last phase's
// descents spread over many cells and rarely meet a locked slot.
constexpr int kBuildPhases = 3;
__host__ __device__ constexpr int phase_bodies(int phase) {   // per full 256-body chunk
    return phase < 0 ? 256 : (phase == 0 ? 1 : (phase == 1 ? 15 : 240));
}
// Offset inside its chunk of the phase's idx-th body: 0; 16, 32, ..., 240; the rest.
// Phase -1 is a single pass over every body.
__device__ __forceinline__ int phase_offset(int phase, int idx) {
    return phase < 0 ? idx : (phase == 0 ? 0 : (phase == 1 ? 16 * (idx + 1) : idx + idx / 15 + 1));
}

__global__ void __launch_bounds__(256) build_kernel(StepParams p, int phase) {
    if (load_status(p.st)) return;
    int local_max = 1;
    int waits = 0, misses = 0;
    const int nbody = p.nbody;
    const int per = phase_bodies(phase);
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // one body per thread
    if (g < (long long)p.nchunks * per) {
        const int4 ck = p.chunks[g / per];
        const int b = ck.y + phase_offset(phase, (int)(g % per));
        if (b < ck.z) {
            const int root = p.nnodes - ck.x;
            const float4 rc = p.node4[root];
            const float radius = p.uradius[ck.x];
            const float4 bp = p.node4[b];
            int node = root, depth = 1;
            float r = radius;
            float cx = rc.x, cy = rc.y, cz = rc.z;
            int path = octant(cx, cy, cz, bp.x, bp.y, bp.z);
            int* slot = cell_child(p, node) + path;
            // Slots are read through L1.  A slot that holds a cell index keeps it for the
            // rest of the build, and each cell's slots are one 32-byte sector first read
            // after the cell was published, so a cell index read from L1 is always right;
            // any other value is only acted on through the CAS below, which fails if it is
            // stale and returns the current value.  This keeps the descents off the L2
            // lines of the top cells.
            int ch = __ldca(slot);
            for (;;) {
                while (ch >= nbody) {                      // :77-89
                    if (ch >= node || depth >= kMaxDepth) {  // children sit below parents
                        raise_error(p.st, NBH_ERR_DEPTH);
                        goto finish;
                    }
                    node = ch;
                    ++depth;
                    // The child's centre is the one its creator computed (:124-136) from this
                    // centre and half-width, so it is derived here instead of loaded.
                    const float h = r * 0.5f;
                    cx = __fadd_rn(__fsub_rn(cx, h), (path & 1) ? r : 0.0f);
                    cy = __fadd_rn(__fsub_rn(cy, h), (path & 2) ? r : 0.0f);
                    cz = __fadd_rn(__fsub_rn(cz, h), (path & 4) ? r : 0.0f);
                    r = h;
                    path = octant(cx, cy, cz, bp.x, bp.y, bp.z);
                    slot = cell_child(p, node) + path;
                    ch = __ldca(slot);
                }
                int seen = kLock;
                if (ch != kLock && (seen = atomicCAS(slot, ch, kLock)) == ch) {
                    if (ch == kNull) {
                        // nothing but the index itself is published: no fence needed
                        st_relaxed(slot, b);
                    } else {
                        const int old = ch;
                        const float4 op = p.node4[old];
                        int patch = -1, cur = node, cpath = path;
                        for (;;) {
                            ++depth;
                            if (depth > kMaxDepth) {
                                raise_error(p.st, NBH_ERR_DEPTH);
                                goto finish;
                            }
                            // Cells of the lanes splitting together come from one atomic on
                            // the shared counter (contiguous, still below every parent).
                            const unsigned act = __activemask();
                            const int lane = threadIdx.x & 31;
                            const int leader = __ffs(act) - 1;
                            int base = 0;
                            if (lane == leader) base = atomicSub(&p.st->bottom, __popc(act));
                            base = __shfl_sync(act, base, leader);
                            const int cell = base - 1 - __popc(act & ((1u << lane) - 1u));
                            if (cell <= nbody) {
                                raise_error(p.st, NBH_ERR_POOL);
                                goto finish;
                            }
                            const float ox = (cpath & 1) ? r : 0.0f;
                            const float oy = (cpath & 2) ? r : 0.0f;
                            const float oz = (cpath & 4) ? r : 0.0f;
                            r *= 0.5f;
                            cx = __fadd_rn(__fsub_rn(cx, r), ox);
                            cy = __fadd_rn(__fsub_rn(cy, r), oy);
                            cz = __fadd_rn(__fsub_rn(cz, r), oz);
                            int* cc = cell_child(p, cell);
                            reinterpret_cast<int4*>(cc)[0] = make_int4(kNull, kNull, kNull, kNull);
                            reinterpret_cast<int4*>(cc)[1] = make_int4(kNull, kNull, kNull, kNull);
                            p.arrive[cell - nbody] = 0;
                            p.clevel[cell - nbody] = depth - 1;   // root = level 0
                            if (patch < 0) patch = cell;
                            else cell_child(p, cur)[cpath] = cell;
                            const int opath = octant(cx, cy, cz, op.x, op.y, op.z);
                            cc[opath] = old;
                            cur = cell;
                            cpath = octant(cx, cy, cz, bp.x, bp.y, bp.z);
                            if (cpath != opath) break;
                        }
                        cell_child(p, cur)[cpath] = b;
                        // the new cells' centres and slots become visible before their index
                        st_release(slot, patch);
                    }
                    local_max = max(local_max, depth);
                    break;
                }
                if (seen != kLock) {        // the slot moved on: continue from its value
                    if (ch != kLock) ++misses;
                    ch = seen;
                    continue;
                }
                // the slot is locked by a split in progress: wait (bounded, backed off)
                // until it holds the new subtree
                ch = bounded_wait_ne(slot, kLock, kWaitNs, p.st, kBackoffMinNs, &waits);
                if (ch == kLock) goto finish;
            }
        }
    }
finish:
    // :199; the maximum persists across steps, so the atomic is rarely needed
    if (local_max > ld_relaxed(&p.st->max_depth)) atomicMax(&p.st->max_depth, local_max);
    if (waits) atomicAdd(&p.st->lock_waits[blockIdx.x % kDiagSlots], waits);
    if (misses) atomicAdd(&p.st->cas_misses[blockIdx.x % kDiagSlots], misses);
}

// -------------------------------------------------------------------------------------
// Link: parent[] of every node from the finished tree (one pass over the cells), for the
// bottom-up summarize.  Keeping it out of the build means an insertion publishes nothing
// but a slot value.
__global__ void __launch_bounds__(256) link_kernel(StepParams p) {
    if (load_status(p.st)) return;
    const int nbody = p.nbody;
    const int bottom = p.st->bottom;
    const int stride = gridDim.x * blockDim.x;
    for (int c = bottom + (int)(blockIdx.x * blockDim.x + threadIdx.x); c <= p.nnodes; c += stride) {
        const int* ch8 = cell_child(p, c);
        const int4 s0 = reinterpret_cast<const int4*>(ch8)[0];
        const int4 s1 = reinterpret_cast<const int4*>(ch8)[1];
        const int sl[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (sl[j] >= 0) p.parent[sl[j]] = c;
    }
}

// -------------------------------------------------------------------------------------
// Summarize (summarizetree.cl:37-178), bottom-up without waiting.  Every body arrives at
// its parent cell with one atomic; the last of a cell's k children to arrive sums the
// cell: children compacted to the front in octant order (:77-81), mass and mass-weighted
// position summed in that order, centre = sum * (1/mass) (:161-167), body count
// (:98-118,160); then it arrives at the cell's parent.  The order of the sums is fixed by
// the octant order, independent of timing (the reference's depends on which children
// were ready).  Precise mode sums the roots' centres of mass in FP64.  The last arriver
// also stores, from the registers it already holds:
//   * the children's records as the cell's kids4 block, so the force walk reads a cell's
//     children with one contiguous load;
//   * each child cell's offset inside the cell's depth-first range (loff), from which the
//     sort stage derives every start without waiting (sort.cl:44-58 hands these offsets
//     down from the root instead).
// Arrivals after a write are release atomics and the last arriver acquires, in place of
// full fences.
__device__ __forceinline__ int arrive_relaxed(int* p) {
    int old;
    asm volatile("atom.relaxed.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}
__device__ __forceinline__ int arrive_acq_rel(int* p) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}
__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

template <bool REF, bool PRECISE>
__global__ void __launch_bounds__(256) summarize_kernel(StepParams p) {
    if (load_status(p.st)) return;
    const int nbody = p.nbody;
    const int first_root = p.nnodes - p.nuniv + 1;
    const int stride = gridDim.x * blockDim.x;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbody; b += stride) {
        int c = p.parent[b];
        bool from_body = true;
        while (c >= 0) {
            int* ch8 = cell_child(p, c);
            const int4 s0 = reinterpret_cast<const int4*>(ch8)[0];
            const int4 s1 = reinterpret_cast<const int4*>(ch8)[1];
            const int sl[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
            int k = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) k += sl[j] >= 0;
            int* ctr = p.arrive + (c - nbody);
            if (from_body) {
                if (arrive_relaxed(ctr) != k - 1) break;
                fence_acquire();
            } else {
                if (arrive_acq_rel(ctr) != k - 1) break;
            }
            int used = 0, cnt = 0;
            float cm = 0.0f, sx = 0.0f, sy = 0.0f, sz = 0.0f;
            double dm = 0.0, dx = 0.0, dy = 0.0, dz = 0.0;
            const bool froot = PRECISE && c >= first_root;
            float4* kb = p.kids4 + ((size_t)(c - nbody) << 3);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int ch = sl[j];
                if (ch < 0) continue;
                const float4 q = ld_cg4(p.node4 + ch);
                if (ch >= nbody) {
                    p.loff[ch - nbody] = cnt;
                    cnt += __ldcg(p.count + (ch - nbody));
                } else {
                    cnt += 1;
                }
                if (froot) {
                    dm += (double)q.w;
                    dx += (double)q.x * (double)q.w;
                    dy += (double)q.y * (double)q.w;
                    dz += (double)q.z * (double)q.w;
                } else {
                    cm = __fadd_rn(cm, q.w);
                    sx = madd<REF>(q.x, q.w, sx);
                    sy = madd<REF>(q.y, q.w, sy);
                    sz = madd<REF>(q.z, q.w, sz);
                }
                // compacted slot and the child's record, at the running position
                ch8[used] = ch;
                kb[used] = q;
                ++used;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (j >= used) {
                    ch8[j] = kNull;
                    kb[j] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            p.count[c - nbody] = cnt;
            if (froot) {
                p.node4[c] = make_float4((float)(dx / dm), (float)(dy / dm), (float)(dz / dm), (float)dm);
            } else {
                const float inv = __fdiv_rn(1.0f, cm);
                p.node4[c] = make_float4(__fmul_rn(sx, inv), __fmul_rn(sy, inv), __fmul_rn(sz, inv), cm);
            }
            const int pc = p.parent[c];
            if (pc >= 0 && pc <= c) {   // parents always have higher indices
                raise_error(p.st, NBH_ERR_STATE);
                break;
            }
            c = pc;
            from_body = false;
        }
    }
}

// -------------------------------------------------------------------------------------
// Sort (sort.cl:24-75): bodies in depth-first octant order.  A cell's first position is
// its universe's first position plus the offsets (loff, from summarize) of the cell and
// of each ancestor inside its parent's range -- the sum sort.cl:44-58 accumulates from
// the root down.  Each cell walks up to its root to form that sum (no thread waits for
// another), records it in start[], and places its body children: in child order, a cell
// child advances the position by its body count, a body child takes the next position.
__global__ void __launch_bounds__(256) sort_kernel(StepParams p) {
    if (load_status(p.st)) return;
    const int nbody = p.nbody;
    const int bottom = p.st->bottom;
    const int stride = gridDim.x * blockDim.x;
    for (int c = bottom + (int)(blockIdx.x * blockDim.x + threadIdx.x); c <= p.nnodes; c += stride) {
        int s = 0;
        int x = c;
        for (int guard = 0;; ++guard) {
            const int px = p.parent[x];
            if (px < 0) {
                s += p.start[x - nbody];         // a root: its universe's first position
                break;
            }
            if (px <= x || guard > kMaxDepth) {  // parents have higher indices; depth <= 64
                raise_error(p.st, NBH_ERR_STATE);
                return;
            }
            s += p.loff[x - nbody];
            x = px;
        }
        if (x != c) p.start[c - nbody] = s;
        const int* ch8 = cell_child(p, c);
        const int4 s0 = reinterpret_cast<const int4*>(ch8)[0];
        const int4 s1 = reinterpret_cast<const int4*>(ch8)[1];
        const int sl[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int ch = sl[j];
            if (ch >= nbody) s += p.count[ch - nbody];
            else if (ch >= 0) p.sorted[s++] = ch;
        }
    }
}

// -------------------------------------------------------------------------------------
void launch_bbox(const StepParams& p, int grid, cudaStream_t s) {
    if (p.precise) bbox_kernel<true><<<grid, 256, 0, s>>>(p);
    else bbox_kernel<false><<<grid, 256, 0, s>>>(p);
}
void launch_build(const StepParams& p, int phases, cudaStream_t s) {
    if (phases == 1) {      // a single pass over every body (phase index -1)
        const long long bodies = (long long)p.nchunks * 256;
        build_kernel<<<(unsigned)((bodies + 255) / 256), 256, 0, s>>>(p, -1);
        return;
    }
    for (int phase = 0; phase < kBuildPhases; ++phase) {
        const long long bodies = (long long)p.nchunks * phase_bodies(phase);
        build_kernel<<<(unsigned)((bodies + 255) / 256), 256, 0, s>>>(p, phase);
    }
}
void launch_link(const StepParams& p, int grid, cudaStream_t s) {
    link_kernel<<<grid, 256, 0, s>>>(p);
}
void launch_summarize(const StepParams& p, bool ref, int grid, cudaStream_t s) {
    if (ref) {
        if (p.precise) summarize_kernel<true, true><<<grid, 256, 0, s>>>(p);
        else summarize_kernel<true, false><<<grid, 256, 0, s>>>(p);
    } else {
        if (p.precise) summarize_kernel<false, true><<<grid, 256, 0, s>>>(p);
        else summarize_kernel<false, false><<<grid, 256, 0, s>>>(p);
    }
}
void launch_sort(const StepParams& p, int grid, cudaStream_t s) {
    sort_kernel<<<grid, 256, 0, s>>>(p);
}

int occupancy_sort(int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, sort_kernel, 256, 0);
}

}  // namespace nbh
