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
    {
        // Empty the slots of every cell a build may have written since the last reset (the
        // whole pool after a load, when bottom is 0), so that the insertion of this step
        // finds in any slot only kNull or a value written during this step -- see
        // build_kernel for why that matters.  Every block reads the bounds before the last
        // block moves them (below, after all blocks have taken their ticket).
        const int lo = max(p.nbody + 1, min(p.st->pool_low, p.st->bottom));
        const int hi = p.nnodes - p.nuniv;     // the roots above are reset below
        int4* const c4 = reinterpret_cast<int4*>(p.child);
        const int4 empty = make_int4(kNull, kNull, kNull, kNull);
        for (long long i = 2LL * lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; i <= 2LL * hi + 1;
             i += (long long)gridDim.x * blockDim.x)
            c4[i - 2LL * p.nbody] = empty;
    }
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
        int4* bc = reinterpret_cast<int4*>(p.kids4 + ((size_t)k << 3));   // bucket counters
        bc[0] = make_int4(0, 0, 0, 0);
        bc[1] = make_int4(0, 0, 0, 0);
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
        st->pool_low = st->bottom;          // nothing below the roots is written now
        st->bbox_ticket = 0;
        st->step += 1;
        st->force_next = 0;
        st->bucket_fill = 0;
        st->nbuckets = 0;
        st->bucket_next = 0;
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
// Insertion runs in phases (one launch each): first one body of every 256-body chunk,
// then more and more of each chunk (3 phases: 1 in 16, then the rest; 5 phases: 1 in 64,
// 1 in 16, 1 in 4, then the rest).  The octree of a set of bodies does not depend on the
// order the bodies arrive in, so the phases build exactly the tree a single pass would;
// what they change is contention.  In one pass every body of a universe that is resident
// at once descends into the same empty top levels and waits on each split there in turn
// (in a batch of small universes that is every body).  After the early phases the top of
// each tree already holds a sample of its bodies, so later descents spread over many cells
// and rarely meet a locked slot.
//
// A phase takes, in each chunk, the offsets that are multiples of `stride` but (ratio > 0)
// not multiples of stride * ratio, i.e. the ones an earlier phase did not take.
struct BuildPhase {
    int stride, ratio;
};
__host__ __device__ constexpr int phase_bodies(BuildPhase ph) {   // per full 256-body chunk
    return ph.ratio > 0 ? 256 / ph.stride - 256 / (ph.stride * ph.ratio) : 256 / ph.stride;
}
// Offset inside chunk ci of the phase's idx-th body.  The lattice is rotated by
// 7 ci mod 16 positions (a bijection of the 256 offsets), so that an input order with a
// period of 16 (two data sets interleaved 1:15, say) is sampled in every residue class
// across chunks instead of in one.
__device__ __forceinline__ int phase_offset(BuildPhase ph, int idx, long long ci) {
    const int j = ph.ratio > 0 ? ph.stride * (idx + idx / (ph.ratio - 1) + 1) : ph.stride * idx;
    return (j + (int)((ci * 7) & 15)) & 255;
}
constexpr BuildPhase kOnePass[1] = {{1, 0}};
constexpr BuildPhase kThreePhases[3] = {{256, 0}, {16, 16}, {1, 16}};
constexpr BuildPhase kFivePhases[5] = {{256, 0}, {64, 4}, {16, 4}, {4, 4}, {1, 4}};

// One body's lock insertion into its universe's tree (see build_kernel).  Returns false
// after raising an error (depth, pool, timeout).
__device__ bool lock_insert(const StepParams& p, int b, int u, bool zero_counts, int& local_max, int& waits,
                            int& misses) {
    const int nbody = p.nbody;
    const int root = p.nnodes - u;
    const float4 rc = p.node4[root];
    const float radius = p.uradius[u];
    const float4 bp = p.node4[b];
    int node = root, depth = 1;
    float r = radius;
    float cx = rc.x, cy = rc.y, cz = rc.z;
    int path = octant(cx, cy, cz, bp.x, bp.y, bp.z);
    int* slot = cell_child(p, node) + path;
    // Slots are read through L1 and without acquire, so a read may return an older
    // value of the slot.  That is safe because of what a slot can have held: the
    // bbox stage empties every pool slot a build wrote (kNull), and during the
    // build a slot only goes kNull -> body -> cell, with kLock in between; a cell
    // index, once stored, stays.  A cell index read is therefore always the
    // current one, and any other value is only acted on through the CAS below,
    // which fails if it is stale and returns the current value.  The reset keeps
    // this true whatever the L1 holds: a sector of a newly taken cell cached before
    // the cell was initialised can only show kNull, never a child index left by
    // the previous step's tree.  Reading through L1 keeps the descents off the L2
    // lines of the top cells.
    int ch = __ldca(slot);
    for (;;) {
        while (ch >= nbody) {                      // :77-89
            if (ch >= node || depth >= kMaxDepth) {  // children sit below parents
                raise_error(p.st, NBH_ERR_DEPTH);
                return false;
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
                        return false;
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
                        return false;
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
                    if (zero_counts) {   // bucket counters of the sampled tree
                        int4* bc = reinterpret_cast<int4*>(p.kids4 + ((size_t)(cell - nbody) << 3));
                        bc[0] = make_int4(0, 0, 0, 0);
                        bc[1] = make_int4(0, 0, 0, 0);
                    }
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
        if (ch == kLock) return false;
    }
    return true;
}

__global__ void __launch_bounds__(256) build_kernel(StepParams p, BuildPhase phase, bool zero_counts) {
    if (load_status(p.st)) return;
    int local_max = 1;
    int waits = 0, misses = 0;
    const int per = phase_bodies(phase);
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // one body per thread
    if (g < (long long)p.nchunks * per) {
        const int4 ck = p.chunks[g / per];
        const int b = ck.y + phase_offset(phase, (int)(g % per), g / per);
        if (b < ck.z) lock_insert(p, b, ck.x, zero_counts, local_max, waits, misses);
    }
    // :199; the maximum persists across steps, so the atomic is rarely needed
    if (local_max > ld_relaxed(&p.st->max_depth)) atomicMax(&p.st->max_depth, local_max);
    if (waits) atomicAdd(&p.st->lock_waits[blockIdx.x % kDiagSlots], waits);
    if (misses) atomicAdd(&p.st->cas_misses[blockIdx.x % kDiagSlots], misses);
}

// -------------------------------------------------------------------------------------
// The first insertion phase (one body of every 256-body chunk) in shared memory.  On an
// empty tree that phase is the slowest one: every sampled body of a universe descends into
// the same few top slots at once and waits on each split there in turn, through global
// locks and release fences.  Here one block per universe, or eight (one per octant of the
// root: more parallelism for a large sample, more blocks for many small ones), build those
// top levels in their shared memory instead -- the same descents, the same centre
// arithmetic and the same CAS locks, but on shared slots, where a lock round trip takes tens
// of cycles -- and then publish them: each block takes its new cells from the pool with one
// atomic, writes every slot once with its final value, and writes its root slots.  The tree is the one the global phase builds (an octree does not depend on
// insertion order).  Cells are numbered in the order they are made, and every cell is made
// after its parent, so the pool indices stay below their parents'.  If a block's sample
// needs more cells than it holds, or a split goes deeper than the depth limit, that block
// inserts its octant's sample through the global locks instead.
//
// Shared slots hold 16-bit values: a local cell (kTopCell | index), a sample (its index
// within the universe's chunks), kTopNull or kTopLock.  Every slot is emptied before the
// first descent, so a slot read before the write that fills it can only show kTopNull, and
// acting on that goes through the CAS, which fails and returns the current value.
constexpr int kTopThreads = 1024;
constexpr int kTopCells = 12288;               // largest shared tree of one block
constexpr unsigned short kTopNull = 0xffffu, kTopLock = 0xfffeu, kTopCell = 0x8000u;
constexpr BuildPhase kFirstPhase = {256, 0};
constexpr long long kTopSpin = 1ll << 22;     // polls of a locked shared slot before giving up

constexpr int kTopMaxSamples = 0x7ffe;       // sample indices stay below kTopLock and kTopCell
int top_build_max_samples() { return kTopMaxSamples; }
// Cells a block's shared tree holds for universes of at most max_chunks chunks: an octree of
// k bodies has about k/2 cells, and a block holds one octant's share; chains of single-child
// cells between close pairs take more, and a block that runs out falls back.
int top_build_cells(int max_chunks) {
    const int want = ((max_chunks + 64) + 63) / 64 * 64;
    return want < kTopCells ? want : kTopCells;
}
static size_t top_build_smem(int cells) { return (size_t)cells * 8 * sizeof(unsigned short) + cells; }

__device__ __forceinline__ unsigned short ld_shared_volatile(const unsigned short* a) {
    return *reinterpret_cast<const volatile unsigned short*>(a);
}

__global__ void __launch_bounds__(kTopThreads) top_build_kernel(StepParams p, bool zero_counts, int cap,
                                                                 int split) {
    extern __shared__ __align__(16) unsigned char top_smem[];
    unsigned short* slots = reinterpret_cast<unsigned short*>(top_smem);          // [cap][8]
    unsigned char* lvl = top_smem + (size_t)cap * 8 * sizeof(unsigned short);
    __shared__ int ncell, failed, c0, gbase, depth_max, status;
    // one read of the status word for the whole block: threads that saw different values
    // would part at the barriers below
    if (threadIdx.x == 0) status = load_status(p.st);
    __syncthreads();
    if (status) return;
    const int u = split == 8 ? (int)(blockIdx.x >> 3) : (int)blockIdx.x;   // universe
    const int oct = split == 8 ? (int)(blockIdx.x & 7) : -1;   // this block's octant of the root (-1: all)
    const int nbody = p.nbody;
    const int nsamp = (p.ubody[u + 1] - p.ubody[u] + 255) / 256;    // chunks of universe u
    if (threadIdx.x == 0) {
        int lo = 0, hi = p.nchunks;              // first chunk of universe u
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (p.chunks[mid].x < u) lo = mid + 1;
            else hi = mid;
        }
        c0 = lo;
        ncell = 1;                               // local cell 0 is the root
        failed = nsamp > kTopMaxSamples ? 1 : 0;
        depth_max = 1;
        lvl[0] = 0;
    }
    for (int i = threadIdx.x; i < cap * 4; i += blockDim.x) reinterpret_cast<unsigned*>(slots)[i] = 0xffffffffu;
    __syncthreads();
    const int root = p.nnodes - u;
    const float4 rc = p.node4[root];
    const float radius = p.uradius[u];
    int local_max = 1;
    if (!failed) {
        for (int smp = threadIdx.x; smp < nsamp; smp += blockDim.x) {
            const long long ci = c0 + smp;
            const int4 ck = p.chunks[ci];
            const int b = ck.y + phase_offset(kFirstPhase, 0, ci);
            if (b >= ck.z) continue;
            const float4 bp = p.node4[b];
            int node = 0, depth = 1;
            float r = radius, cx = rc.x, cy = rc.y, cz = rc.z;
            int path = octant(cx, cy, cz, bp.x, bp.y, bp.z);
            if (oct >= 0 && path != oct) continue;     // another block's octant
            unsigned short* slot = slots + node * 8 + path;
            unsigned short ch = ld_shared_volatile(slot);
            bool done = false;
            long long spins = 0;
            while (!done) {
                while (ch != kTopNull && ch != kTopLock && (ch & kTopCell)) {
                    if (depth >= kMaxDepth) {
                        atomicExch(&failed, 1);
                        break;
                    }
                    node = ch & 0x7fff;
                    ++depth;
                    const float h = r * 0.5f;
                    cx = __fadd_rn(__fsub_rn(cx, h), (path & 1) ? r : 0.0f);
                    cy = __fadd_rn(__fsub_rn(cy, h), (path & 2) ? r : 0.0f);
                    cz = __fadd_rn(__fsub_rn(cz, h), (path & 4) ? r : 0.0f);
                    r = h;
                    path = octant(cx, cy, cz, bp.x, bp.y, bp.z);
                    slot = slots + node * 8 + path;
                    ch = ld_shared_volatile(slot);
                }
                if (*reinterpret_cast<volatile int*>(&failed)) break;
                if (ch == kTopLock) {                  // a split in progress: wait, bounded
                    if (++spins > kTopSpin) {
                        raise_error(p.st, NBH_ERR_TIMEOUT);
                        atomicExch(&failed, 2);
                        break;
                    }
                    __nanosleep(32);
                    ch = ld_shared_volatile(slot);
                    continue;
                }
                const unsigned short seen = atomicCAS(slot, ch, kTopLock);
                if (seen != ch) {
                    ch = seen;
                    continue;
                }
                if (ch == kTopNull) {
                    *reinterpret_cast<volatile unsigned short*>(slot) = (unsigned short)smp;
                    local_max = max(local_max, depth);
                    done = true;
                    break;
                }
                // split: the slot held sample `ch`; cells until the two separate
                const int4 ock = p.chunks[c0 + ch];
                const float4 op = p.node4[ock.y + phase_offset(kFirstPhase, 0, c0 + ch)];
                int patch = -1, cur = node, cpath = path;
                bool ok = true;
                for (;;) {
                    ++depth;
                    const int cell = atomicAdd(&ncell, 1);
                    if (depth > kMaxDepth || cell >= cap) {
                        atomicExch(&failed, 1);
                        ok = false;
                        break;
                    }
                    const float ox = (cpath & 1) ? r : 0.0f;
                    const float oy = (cpath & 2) ? r : 0.0f;
                    const float oz = (cpath & 4) ? r : 0.0f;
                    r *= 0.5f;
                    cx = __fadd_rn(__fsub_rn(cx, r), ox);
                    cy = __fadd_rn(__fsub_rn(cy, r), oy);
                    cz = __fadd_rn(__fsub_rn(cz, r), oz);
                    lvl[cell] = (unsigned char)(depth - 1);
                    if (patch < 0) patch = cell;
                    else slots[cur * 8 + cpath] = (unsigned short)(kTopCell | cell);
                    const int opath = octant(cx, cy, cz, op.x, op.y, op.z);
                    slots[cell * 8 + opath] = ch;
                    cur = cell;
                    cpath = octant(cx, cy, cz, bp.x, bp.y, bp.z);
                    if (cpath != opath) break;
                }
                if (!ok) break;
                slots[cur * 8 + cpath] = (unsigned short)smp;
                __threadfence_block();                 // the new cells before their index
                *reinterpret_cast<volatile unsigned short*>(slot) = (unsigned short)(kTopCell | patch);
                local_max = max(local_max, depth);
                done = true;
            }
        }
    }
    atomicMax(&depth_max, local_max);
    __syncthreads();
    if (failed == 2) return;                           // a wait gave up: the status says so
    if (failed) {
        // more cells than the block holds, or a very deep split: the global lock insertion
        int lm = 1, waits = 0, misses = 0;
        const float4 rc0 = p.node4[root];
        for (int smp = threadIdx.x; smp < nsamp; smp += blockDim.x) {
            const long long ci = c0 + smp;
            const int4 ck = p.chunks[ci];
            const int b = ck.y + phase_offset(kFirstPhase, 0, ci);
            if (b >= ck.z) continue;
            const float4 bp = p.node4[b];
            if (oct >= 0 && octant(rc0.x, rc0.y, rc0.z, bp.x, bp.y, bp.z) != oct) continue;   // another block's
            if (!lock_insert(p, b, u, zero_counts, lm, waits, misses)) break;
        }
        if (lm > ld_relaxed(&p.st->max_depth)) atomicMax(&p.st->max_depth, lm);
        if (waits) atomicAdd(&p.st->lock_waits[blockIdx.x % kDiagSlots], waits);
        if (misses) atomicAdd(&p.st->cas_misses[blockIdx.x % kDiagSlots], misses);
        return;
    }
    // publish: local cell c (c >= 1) becomes pool cell gbase - c
    const int nc = ncell;
    if (threadIdx.x == 0) {
        gbase = nc > 1 ? atomicSub(&p.st->bottom, nc - 1) : 0;
        status = 0;
        if (nc > 1 && gbase - (nc - 1) <= nbody) {
            raise_error(p.st, NBH_ERR_POOL);
            status = NBH_ERR_POOL;
        }
        if (depth_max > ld_relaxed(&p.st->max_depth)) atomicMax(&p.st->max_depth, depth_max);
    }
    __syncthreads();
    if (status) return;
    const int gb = gbase;
    for (int i = threadIdx.x; i < nc * 8; i += blockDim.x) {
        const int c = i >> 3;
        if (c == 0 && oct >= 0 && (i & 7) != oct) continue;   // the root's other slots are other blocks'
        const unsigned short v = slots[i];
        int g = kNull;
        if (v != kTopNull) {
            if (v & kTopCell) {
                g = gb - (v & 0x7fff);
            } else {
                const long long ci = c0 + v;
                g = p.chunks[ci].y + phase_offset(kFirstPhase, 0, ci);
            }
        }
        const int gc = c == 0 ? root : gb - c;
        cell_child(p, gc)[i & 7] = g;
    }
    for (int c = 1 + (int)threadIdx.x; c < nc; c += blockDim.x) {
        const int k = gb - c - nbody;
        p.arrive[k] = 0;
        p.clevel[k] = lvl[c];
        if (zero_counts) {   // bucket counters of the sampled tree
            int4* bc = reinterpret_cast<int4*>(p.kids4 + ((size_t)k << 3));
            bc[0] = make_int4(0, 0, 0, 0);
            bc[1] = make_int4(0, 0, 0, 0);
        }
    }
}

// -------------------------------------------------------------------------------------
// Bucketed completion of the build.  After the lock phases have inserted a sample of every
// chunk (the "sampled tree": 1/16, or 1/256 before a first pass that completes the 1/16
// sample the same way), each remaining body of the pass finds, by a read-only descent, the
// slot of the sampled tree it would be inserted into.  The bodies headed for one slot
// (its bucket, plus the body already in it) are exactly those of the subtree that replaces
// the slot in the final tree, and no other body touches that subtree, so one warp builds
// it alone: no locks, no release fences (later kernels read it across the kernel
// boundary).  The tree is the one the lock insertion builds (it is order independent):
// a cell exists for every octant prefix shared by two or more bodies, with the same
// centres (the same arithmetic from the same parent centre and half-width).
//
// Bucket counters of a sampled-tree cell live in its kids4 block, which summarize
// overwrites later in the step: ints 0..7 = bodies headed for slot j (zeroed when the cell
// is made; the scatter counts them back to zero, so a second pass starts from zero too),
// 8..15 = first entry of slot j's bucket in the work list (written by the allocation for
// every slot with bodies before the scatter reads it), 16..19 = the cell's centre and
// half-width.
__device__ __forceinline__ int* bucket_counters(const StepParams& p, int c) {
    return reinterpret_cast<int*>(p.kids4 + ((size_t)(c - p.nbody) << 3));
}
constexpr BuildPhase kBucketBodies = {1, 16};   // the bodies outside the 1/16 sample

// (1) locate: read-only descent of each remaining body to its slot; the slot index goes
// to parent[b] (scratch: the link pass writes the body's parent later).
__global__ void __launch_bounds__(256) bucket_locate_kernel(StepParams p, BuildPhase set, bool reset_counters) {
    if (load_status(p.st)) return;
    if (reset_counters && blockIdx.x == 0 && threadIdx.x == 0) {
        // a second pass: the work-list counters start over (the first pass is complete)
        p.st->bucket_fill = 0;
        p.st->nbuckets = 0;
        p.st->bucket_next = 0;
    }
    const int nbody = p.nbody;
    const int per = phase_bodies(set);
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)p.nchunks * per) return;
    const int4 ck = p.chunks[g / per];
    const int b = ck.y + phase_offset(set, (int)(g % per), g / per);
    if (b >= ck.z) return;
    const int root = p.nnodes - ck.x;
    const float4 rc = p.node4[root];
    const float4 bp = p.node4[b];
    float r = p.uradius[ck.x];
    float cx = rc.x, cy = rc.y, cz = rc.z;
    int node = root, depth = 1;
    int path = octant(cx, cy, cz, bp.x, bp.y, bp.z);
    int ch = __ldg(cell_child(p, node) + path);
    while (ch >= nbody) {
        if (ch >= node || ++depth > kMaxDepth) {
            raise_error(p.st, NBH_ERR_DEPTH);
            return;
        }
        node = ch;
        const float h = r * 0.5f;
        cx = __fadd_rn(__fsub_rn(cx, h), (path & 1) ? r : 0.0f);
        cy = __fadd_rn(__fsub_rn(cy, h), (path & 2) ? r : 0.0f);
        cz = __fadd_rn(__fsub_rn(cz, h), (path & 4) ? r : 0.0f);
        r = h;
        path = octant(cx, cy, cz, bp.x, bp.y, bp.z);
        ch = __ldg(cell_child(p, node) + path);
    }
    p.parent[b] = ((node - nbody) << 3) | path;
    int* bc = bucket_counters(p, node);
    if (atomicAdd(bc + path, 1) == 0) {
        // the first body headed for a slot of `node` records the cell's centre and
        // half-width for the subtree builder (every descent computes the same values)
        reinterpret_cast<float4*>(bc)[4] = make_float4(cx, cy, cz, r);
    }
}

// (2) allocate: per sampled-tree cell, the work-list entries of its non-empty slots
// (bodies headed there, plus the body the slot holds) and one bucket record each.
__global__ void __launch_bounds__(256) bucket_alloc_kernel(StepParams p) {
    if (load_status(p.st)) return;
    const int nbody = p.nbody;
    const int bottom = ld_relaxed(&p.st->bottom);
    // block-uniform stride over every cell of the tree so far (the grid is sized for the
    // usual count; chains of single-child cells between close bodies can exceed it)
    for (int base = bottom + (int)(blockIdx.x * blockDim.x); base <= p.nnodes; base += (int)(gridDim.x * blockDim.x)) {
        const int c = base + (int)threadIdx.x;
        const bool valid = c <= p.nnodes;
        int cnt[8], held[8];
        int total = 0, nb = 0;
        if (valid) {
            const int4* bc = reinterpret_cast<const int4*>(bucket_counters(p, c));
            const int4 a0 = bc[0], a1 = bc[1];
            const int4* ch = reinterpret_cast<const int4*>(cell_child(p, c));
            const int4 s0 = ch[0], s1 = ch[1];
            const int cc[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const int ss[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                cnt[j] = cc[j];
                held[j] = (cc[j] > 0 && ss[j] >= 0 && ss[j] < nbody) ? ss[j] : kNull;
                total += cc[j] > 0 ? cc[j] + (held[j] >= 0 ? 1 : 0) : 0;
                nb += cc[j] > 0 ? 1 : 0;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) cnt[j] = 0, held[j] = kNull;
        }
        // warp-aggregated allocation of entries and bucket records
        const int lane = threadIdx.x & 31;
        int te = total, tb = nb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int ue = __shfl_up_sync(0xffffffffu, te, o), ub = __shfl_up_sync(0xffffffffu, tb, o);
            if (lane >= o) te += ue, tb += ub;
        }
        int be = 0, bb = 0;
        if (lane == 31) {
            be = atomicAdd(&p.st->bucket_fill, te);
            bb = atomicAdd(&p.st->nbuckets, tb);
        }
        be = __shfl_sync(0xffffffffu, be, 31) + te - total;
        bb = __shfl_sync(0xffffffffu, bb, 31) + tb - nb;
        if (!valid || total == 0) continue;
        int* bcw = bucket_counters(p, c);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (cnt[j] <= 0) continue;
            bcw[8 + j] = be;
            p.buckets[bb++] = make_int4(((c - nbody) << 3) | j, be, cnt[j], held[j]);
            be += cnt[j] + (held[j] >= 0 ? 1 : 0);
        }
    }
}

// (3) scatter: each remaining body takes an entry of its slot's bucket.
__global__ void __launch_bounds__(256) bucket_scatter_kernel(StepParams p, BuildPhase set) {
    if (load_status(p.st)) return;
    const int per = phase_bodies(set);
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)p.nchunks * per) return;
    const int4 ck = p.chunks[g / per];
    const int b = ck.y + phase_offset(set, (int)(g % per), g / per);
    if (b >= ck.z) return;
    const int slot = p.parent[b];
    int* bc = bucket_counters(p, p.nbody + (slot >> 3));
    const int j = slot & 7;
    p.bwork[bc[8 + j] + atomicSub(bc + j, 1) - 1] = b;
}

// (4) build: one warp per bucket builds the bucket's subtree by splitting its bodies by
// octant, level by level (depth first over a task stack), writing each new cell's 8 slots
// once with their final values, then stores the subtree's root into the slot.  Subtrees of
// at most 32 bodies are built in registers (one body per lane, octants grouped by
// match_any).  A warp takes kBucketChunk buckets per work-counter atomic; a counting pass
// sizes the register subtrees of the whole chunk so that one allocator atomic takes all
// their cells, then the writing pass hands each subtree its share, parents first.  (Both
// counters sit on one L2 slice: one atomic per bucket each was the kernel's limit.)  Larger
// buckets split through the two halves of bwork until a part has at most 32 bodies.
struct BucketTask {
    int cell, level, lo, hi, buf;
    float cx, cy, cz, r;       // centre and half-width of `cell`
};
struct SmallTask {
    unsigned mask;             // lanes holding the task's bodies
    int cell, level;
    float cx, cy, cz, r;
};
constexpr int kBucketWarps = 4;
// Children are pushed largest first, so every stacked sibling holds at most half of its
// parent's bodies: the stack stays within 7 log2(m) + 8 entries for a bucket of m bodies --
// 225 for any m < 2^31 (the large-bucket stacks live in global memory, one slice per warp
// of the grid) and 43 for the register subtrees of at most 32 bodies (shared memory).
constexpr int kBucketStack = 232;
constexpr int kSmallStack = 48;
constexpr int kBucketBlocksPerSm = 9;
constexpr int kBucketChunk = 4;      // buckets a warp takes per work-counter atomic

// Stack position of each child cell among the nc cells pushed now: the largest deepest.
__device__ __forceinline__ int deeper_rank(int mycnt, int lane) {
    int deeper = 0;
#pragma unroll
    for (int o2 = 0; o2 < 8; ++o2) {
        const int n2 = __shfl_sync(0xffffffffu, mycnt, o2);
        deeper += (n2 >= 2 && (n2 > mycnt || (n2 == mycnt && o2 < lane))) ? 1 : 0;
    }
    return deeper;
}

// The subtree of the m <= 32 bodies src[lo, lo + m) below a cell of level `level` with the
// given centre and half-width, in one of two passes over the same traversal.  Counting
// (build = false) returns the number of new cells the subtree takes and writes nothing.
// Building (build = true) takes them as base - 1, base - 2, ... (parents first, so every
// parent index is above its children's) and returns the subtree's root: `cell` when it
// exists already (its slots are written here), else base - 1.  Returns -1 after raising
// an error.  Whole-warp call.  Lanes with a body are grouped by octant (match_any); each
// group's lowest lane writes its octant's slot -- its own body when alone, else a new cell
// -- and lanes 0..7 write the empty octants.
__device__ int small_subtree(const StepParams& p, const int* __restrict__ src, int lo, int m, int cell, int level,
                             float cx, float cy, float cz, float r, SmallTask* st, int& local_max, bool build,
                             int base, bool zero_counts) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int nbody = p.nbody;
    int b = 0;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lane < m) {
        b = src[lo + lane];
        q = p.node4[b];
    }
    const unsigned all = m >= 32 ? 0xffffffffu : ((1u << m) - 1u);
    int made = 0;
    int root = cell;
    if (cell < 0) root = build ? base - 1 - made++ : (made++, 0);
    if (lane == 0) st[0] = SmallTask{all, root, level, cx, cy, cz, r};
    int top = 1;
    __syncwarp();
    while (top > 0) {
        const SmallTask t = st[--top];
        __syncwarp();
        const bool member = (t.mask >> lane) & 1u;
        const int o = member ? octant(t.cx, t.cy, t.cz, q.x, q.y, q.z) : -1;
        const unsigned grp = __match_any_sync(0xffffffffu, o);
        const bool leader = member && (__ffs(grp) - 1) == lane;
        const int cnt = __popc(grp);
        const unsigned balc = __ballot_sync(0xffffffffu, leader && cnt >= 2);
        const int nc = __popc(balc);
        if (nc > 0 && (t.level + 2 > kMaxDepth || top + nc > kSmallStack)) {   // coincident bodies
            raise_error(p.st, NBH_ERR_DEPTH);
            return -1;
        }
        if (build) {
            const unsigned occ = __reduce_or_sync(0xffffffffu, member ? 1u << o : 0u);
            if (lane < 8 && !((occ >> lane) & 1u)) cell_child(p, t.cell)[lane] = kNull;
            if (lane == 0) {
                p.arrive[t.cell - nbody] = 0;
                p.clevel[t.cell - nbody] = t.level;
            }
            if (zero_counts && lane < 2)   // bucket counters for a pass into this tree
                reinterpret_cast<int4*>(p.kids4 + ((size_t)(t.cell - nbody) << 3))[lane] = make_int4(0, 0, 0, 0);
        }
        // the largest child cell is pushed deepest (popped last); the others above it
        int pos = 0;
        if (nc > 1) {
            const unsigned key = (leader && cnt >= 2) ? ((unsigned)cnt << 5) | (31u - lane) : 0u;
            const unsigned kmax = __reduce_max_sync(0xffffffffu, key);
            const int largest = 31 - (int)(kmax & 31u);
            const unsigned others = balc & ~(1u << largest);
            pos = lane == largest ? 0 : 1 + __popc(others & lt);
        }
        if (leader) {
            if (cnt == 1) {
                if (build) cell_child(p, t.cell)[o] = b;
                local_max = max(local_max, t.level + 1);
            } else {
                const int v = build ? base - 1 - made - __popc(balc & lt) : 0;
                if (build) cell_child(p, t.cell)[o] = v;
                const float h = t.r * 0.5f;
                st[top + pos] = SmallTask{grp, v, t.level + 1,
                                          __fadd_rn(__fsub_rn(t.cx, h), (o & 1) ? t.r : 0.0f),
                                          __fadd_rn(__fsub_rn(t.cy, h), (o & 2) ? t.r : 0.0f),
                                          __fadd_rn(__fsub_rn(t.cz, h), (o & 4) ? t.r : 0.0f), h};
            }
        }
        made += nc;
        top += nc;
        __syncwarp();
    }
    return build ? root : made;
}

// Both passes with an allocation of their own in between (the large-bucket path).
__device__ int build_small(const StepParams& p, const int* __restrict__ src, int lo, int m, int cell, int level,
                           float cx, float cy, float cz, float r, SmallTask* st, int& local_max, bool zero_counts) {
    const int need = small_subtree(p, src, lo, m, cell, level, cx, cy, cz, r, st, local_max, false, 0, false);
    if (need < 0) return -1;
    int base = 0;
    if (need > 0) {
        if ((threadIdx.x & 31) == 0) base = atomicSub(&p.st->bottom, need);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base - need <= p.nbody) {
            raise_error(p.st, NBH_ERR_POOL);
            return -1;
        }
    }
    return small_subtree(p, src, lo, m, cell, level, cx, cy, cz, r, st, local_max, true, base, zero_counts);
}

__global__ void __launch_bounds__(32 * kBucketWarps) bucket_build_kernel(StepParams p, bool zero_counts) {
    __shared__ SmallTask small_all[kBucketWarps][kSmallStack];
    if (load_status(p.st)) return;
    BucketTask* stack = static_cast<BucketTask*>(p.bstack) +
                        (size_t)(blockIdx.x * kBucketWarps + (threadIdx.x >> 5)) * kBucketStack;
    SmallTask* sstack = small_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int nbody = p.nbody;
    const int nb = ld_relaxed(&p.st->nbuckets);
    int local_max = 1;
    for (;;) {
        // a chunk of buckets per warp: one atomic hands out kBucketChunk of them
        int item0 = 0;
        if (lane == 0) item0 = atomicAdd(&p.st->bucket_next, kBucketChunk);
        item0 = __shfl_sync(0xffffffffu, item0, 0);
        if (item0 >= nb) break;
        const int nitem = min(kBucketChunk, nb - item0);
        // lane l < nitem holds bucket item0 + l; the body its slot already held joins the
        // bucket's entries
        int4 bkt = make_int4(0, 0, 0, kNull);
        if (lane < nitem) {
            bkt = p.buckets[item0 + lane];
            if (bkt.w >= 0) p.bwork[bkt.y + bkt.z] = bkt.w;
        }
        __syncwarp();
        // (A) count the new cells of every bucket of 2..32 bodies, then take them for the whole
        // chunk with one allocation: bucket l's cells lie below chunk_base minus the cells of
        // the chunk's buckets before it
        int need = 0;                                // lane l: cells of bucket l
        for (int it = 0; it < nitem; ++it) {
            const int bx = __shfl_sync(0xffffffffu, bkt.x, it), start = __shfl_sync(0xffffffffu, bkt.y, it);
            const int m = __shfl_sync(0xffffffffu, bkt.z, it) + (__shfl_sync(0xffffffffu, bkt.w, it) >= 0 ? 1 : 0);
            if (m < 2 || m > 32) continue;
            const int c = nbody + (bx >> 3), j = bx & 7;
            const float4 g = reinterpret_cast<const float4*>(bucket_counters(p, c))[4];
            const int clev = p.clevel[c - nbody];
            if (clev + 2 > kMaxDepth) {
                raise_error(p.st, NBH_ERR_DEPTH);
                return;
            }
            const float h0 = g.w * 0.5f;
            const int cells = small_subtree(p, p.bwork, start, m, -1, clev + 1,
                                            __fadd_rn(__fsub_rn(g.x, h0), (j & 1) ? g.w : 0.0f),
                                            __fadd_rn(__fsub_rn(g.y, h0), (j & 2) ? g.w : 0.0f),
                                            __fadd_rn(__fsub_rn(g.z, h0), (j & 4) ? g.w : 0.0f), h0, sstack,
                                            local_max, false, 0, false);
            if (cells < 0) return;
            if (lane == it) need = cells;
        }
        int incl = need;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        int chunk_base = 0;
        if (total > 0) {
            if (lane == 0) chunk_base = atomicSub(&p.st->bottom, total);
            chunk_base = __shfl_sync(0xffffffffu, chunk_base, 0);
            if (chunk_base - total <= nbody) {
                raise_error(p.st, NBH_ERR_POOL);
                return;
            }
        }
        const int my_base = chunk_base - (incl - need);
        // (B) build each bucket's subtree
        for (int it = 0; it < nitem; ++it) {
            const int bx = __shfl_sync(0xffffffffu, bkt.x, it);
            const int c = nbody + (bx >> 3), j = bx & 7;
            const int start = __shfl_sync(0xffffffffu, bkt.y, it);
            const int m = __shfl_sync(0xffffffffu, bkt.z, it) + (__shfl_sync(0xffffffffu, bkt.w, it) >= 0 ? 1 : 0);
            const int sub_base = __shfl_sync(0xffffffffu, my_base, it);
            // cell c's centre and half-width, recorded by the locate pass
            const float4 g = reinterpret_cast<const float4*>(bucket_counters(p, c))[4];
            const int clev = p.clevel[c - nbody];
            int* slot = cell_child(p, c) + j;
            if (m == 1) {                                 // a single body: the slot takes it
                if (lane == 0) *slot = p.bwork[start];
                local_max = max(local_max, clev + 1);
                continue;
            }
            if (clev + 2 > kMaxDepth) {
                raise_error(p.st, NBH_ERR_DEPTH);
                return;
            }
            // the subtree's root: the child of c in octant j
            const float h0 = g.w * 0.5f;
            const float rcx = __fadd_rn(__fsub_rn(g.x, h0), (j & 1) ? g.w : 0.0f);
            const float rcy = __fadd_rn(__fsub_rn(g.y, h0), (j & 2) ? g.w : 0.0f);
            const float rcz = __fadd_rn(__fsub_rn(g.z, h0), (j & 4) ? g.w : 0.0f);
            int root;
            if (m <= 32) {
                root = small_subtree(p, p.bwork, start, m, -1, clev + 1, rcx, rcy, rcz, h0, sstack, local_max, true,
                                     sub_base, zero_counts);
                if (root < 0) return;
                if (lane == 0) *slot = root;
                continue;
            }
            if (lane == 0) root = atomicSub(&p.st->bottom, 1) - 1;
            root = __shfl_sync(0xffffffffu, root, 0);
            if (root <= nbody) {
                raise_error(p.st, NBH_ERR_POOL);
                return;
            }
            if (lane == 0) stack[0] = BucketTask{root, clev + 1, start, start + m, 0, rcx, rcy, rcz, h0};
            int top = 1;
            __syncwarp();
            bool ok = true;
            while (top > 0) {
                const BucketTask t = stack[--top];
                __syncwarp();
                const int* src = p.bwork + (t.buf ? nbody : 0);
                int* dst = p.bwork + (t.buf ? 0 : nbody);
                if (t.hi - t.lo <= 32) {                  // small enough for the register builder
                    if (build_small(p, src, t.lo, t.hi - t.lo, t.cell, t.level, t.cx, t.cy, t.cz, t.r, sstack,
                                    local_max, zero_counts) < 0) {
                        ok = false;
                        break;
                    }
                    continue;
                }
                // pass 1: bodies per octant (lane o < 8 holds octant o's count)
                int mycnt = 0;
                for (int base = t.lo; base < t.hi; base += 32) {
                    const int i = base + lane;
                    int o = -1;
                    if (i < t.hi) {
                        const float4 q = p.node4[src[i]];
                        o = octant(t.cx, t.cy, t.cz, q.x, q.y, q.z);
                    }
#pragma unroll
                    for (int oc = 0; oc < 8; ++oc) {
                        const int n = __popc(__ballot_sync(0xffffffffu, o == oc));
                        if (lane == oc) mycnt += n;
                    }
                }
                // exclusive offsets of the octants (lanes 0..7)
                int myoff = mycnt;
#pragma unroll
                for (int o2 = 1; o2 < 8; o2 <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, myoff, o2);
                    if (lane >= o2) myoff += v;
                }
                myoff -= mycnt;
                // pass 2: bodies to dst in octant order
                int run = 0;                              // lane o: bodies of octant o placed so far
                for (int base = t.lo; base < t.hi; base += 32) {
                    const int i = base + lane;
                    int o = -1, b = 0;
                    if (i < t.hi) {
                        b = src[i];
                        const float4 q = p.node4[b];
                        o = octant(t.cx, t.cy, t.cz, q.x, q.y, q.z);
                    }
                    unsigned mine = 0;
#pragma unroll
                    for (int oc = 0; oc < 8; ++oc) {
                        const unsigned bal = __ballot_sync(0xffffffffu, o == oc);
                        if (o == oc) mine = bal;
                        if (lane == oc) run += __popc(bal);
                    }
                    const int slot_base = __shfl_sync(0xffffffffu, myoff + run, o < 0 ? 0 : o);
                    // slot_base counts this chunk's bodies of octant o already: subtract them
                    if (o >= 0) dst[t.lo + slot_base - __popc(mine) + __popc(mine & lt)] = b;
                }
                __syncwarp();
                // children: empty, one body, or a cell (allocated together)
                const bool is_cell = lane < 8 && mycnt >= 2;
                const unsigned balc = __ballot_sync(0xffffffffu, is_cell);
                const int nc = __popc(balc);
                int cbase = 0;
                if (nc > 0) {
                    if (t.level + 2 > kMaxDepth || top + nc > kBucketStack) {   // coincident bodies
                        raise_error(p.st, NBH_ERR_DEPTH);
                        ok = false;
                        break;
                    }
                    if (lane == 0) cbase = atomicSub(&p.st->bottom, nc);
                    cbase = __shfl_sync(0xffffffffu, cbase, 0);
                    if (cbase - nc <= nbody) {
                        raise_error(p.st, NBH_ERR_POOL);
                        ok = false;
                        break;
                    }
                }
                const int deeper = deeper_rank(mycnt, lane);
                if (lane < 8) {
                    int v = kNull;
                    if (mycnt == 1) {
                        v = dst[t.lo + myoff];
                        local_max = max(local_max, t.level + 1);
                    } else if (mycnt >= 2) {
                        v = cbase - 1 - __popc(balc & lt);
                        const float h = t.r * 0.5f;
                        stack[top + deeper] = BucketTask{v, t.level + 1, t.lo + myoff, t.lo + myoff + mycnt, t.buf ^ 1,
                                                         __fadd_rn(__fsub_rn(t.cx, h), (lane & 1) ? t.r : 0.0f),
                                                         __fadd_rn(__fsub_rn(t.cy, h), (lane & 2) ? t.r : 0.0f),
                                                         __fadd_rn(__fsub_rn(t.cz, h), (lane & 4) ? t.r : 0.0f), h};
                    }
                    cell_child(p, t.cell)[lane] = v;
                }
                if (lane == 0) {
                    p.arrive[t.cell - nbody] = 0;
                    p.clevel[t.cell - nbody] = t.level;
                }
                if (zero_counts && lane < 2)
                    reinterpret_cast<int4*>(p.kids4 + ((size_t)(t.cell - nbody) << 3))[lane] = make_int4(0, 0, 0, 0);
                top += nc;
                __syncwarp();
            }
            if (!ok) return;
            if (lane == 0) *slot = root;
        }
    }
    // :199; the maximum persists across steps, so the atomic is rarely needed
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local_max = max(local_max, __shfl_xor_sync(0xffffffffu, local_max, o));
    if (lane == 0 && local_max > ld_relaxed(&p.st->max_depth)) atomicMax(&p.st->max_depth, local_max);
}

// -------------------------------------------------------------------------------------
// Link: parent[] of every node from the finished tree (one pass over the cells), for the
// bottom-up summarize, the sort's walk-up and the learned angle's features (a body's leaf
// cell).  Keeping it out of the build means an insertion publishes nothing but a slot value.
// It also tags each cell's count with its number of cell children k, as -1 - k: summarize
// decides from this tag, which nothing changes until the cell is summed, and never from the
// cell's slots, which the cell's summation rewrites (compaction) while other threads run.
__global__ void __launch_bounds__(256) link_kernel(StepParams p) {
    if (load_status(p.st)) return;
    const int bottom = p.st->bottom;
    const int nbody = p.nbody;
    const int stride = gridDim.x * blockDim.x;
    for (int c = bottom + (int)(blockIdx.x * blockDim.x + threadIdx.x); c <= p.nnodes; c += stride) {
        const int* ch8 = cell_child(p, c);
        const int4 s0 = reinterpret_cast<const int4*>(ch8)[0];
        const int4 s1 = reinterpret_cast<const int4*>(ch8)[1];
        const int sl[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
        int kc = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (sl[j] >= 0) p.parent[sl[j]] = c;
            kc += sl[j] >= nbody;
        }
        p.count[c - nbody] = -1 - kc;
    }
}

// -------------------------------------------------------------------------------------
// Summarize (summarizetree.cl:37-178), bottom-up without waiting.  One thread per cell
// starts at the cells whose children are all bodies and sums them at once; every other
// cell is summed by the last of its cell children to finish (one atomic arrival per cell):
// children compacted to the front in octant order (:77-81), mass and mass-weighted
// position summed in that order, centre = sum * (1/mass) (:161-167), body count
// (:98-118,160); then the climb continues at the cell's parent.  The order of the sums is fixed by
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
__device__ __forceinline__ int arrive_acq_rel(int* p) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

// One cell's children, in slot order: compacts the slots and writes each child's record into
// the cell's kids4 block, records each child cell's offset (loff) and the cell's body count,
// and returns the centre of mass and mass -- summed in FP32 (F64 = false) or, for a root in
// precise mode, in FP64.
template <bool REF, bool F64>
__device__ __forceinline__ float4 sum_children(const StepParams& p, int c, const int (&sl)[8], int* ch8) {
    const int nbody = p.nbody;
    int used = 0, cnt = 0;
    float cm = 0.0f, sx = 0.0f, sy = 0.0f, sz = 0.0f;
    double dm = 0.0, dx = 0.0, dy = 0.0, dz = 0.0;
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
        if constexpr (F64) {
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
    if constexpr (F64) {
        return make_float4((float)(dx / dm), (float)(dy / dm), (float)(dz / dm), (float)dm);
    } else {
        const float inv = __fdiv_rn(1.0f, cm);
        return make_float4(__fmul_rn(sx, inv), __fmul_rn(sy, inv), __fmul_rn(sz, inv), cm);
    }
}

template <bool REF, bool PRECISE>
__global__ void __launch_bounds__(256) summarize_kernel(StepParams p) {
    if (load_status(p.st)) return;
    const int nbody = p.nbody;
    const int first_root = p.nnodes - p.nuniv + 1;
    const int stride = gridDim.x * blockDim.x;
    const int bottom = ld_relaxed(&p.st->bottom);
    for (int c0 = bottom + (int)(blockIdx.x * blockDim.x + threadIdx.x); c0 <= p.nnodes; c0 += stride) {
        // link's tag -1 - (cell children): only a cell without cell children starts here; the
        // others are summed by their last cell child (tag < -1), perhaps already (tag >= 0)
        if (p.count[c0 - nbody] != -1) continue;
        int c = c0;
        for (;;) {
            // Every cell child of c has been summed and no other thread touches c now, so
            // its slots are stable until the compaction below.
            int* ch8 = cell_child(p, c);
            const int4 s0 = reinterpret_cast<const int4*>(ch8)[0];
            const int4 s1 = reinterpret_cast<const int4*>(ch8)[1];
            const int sl[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
            // (precise mode: the roots in FP64, as a path of its own -- folded into the
            // FP32 loop as a per-child branch, it ran the FP64 arithmetic for every cell)
            const float4 com = (PRECISE && c >= first_root) ? sum_children<REF, true>(p, c, sl, ch8)
                                                            : sum_children<REF, false>(p, c, sl, ch8);
            p.node4[c] = com;
            const int pc = p.parent[c];
            if (pc < 0) break;          // a root
            if (pc <= c) {              // parents always have higher indices
                raise_error(p.st, NBH_ERR_STATE);
                break;
            }
            // pc is summed only after all its cell children arrive, this one included, so
            // its tag still holds link's value
            const int kc = -1 - __ldcg(p.count + (pc - nbody));
            if (arrive_acq_rel(p.arrive + (pc - nbody)) != kc - 1) break;   // another child is to come
            c = pc;
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
// One bucketed completion: the bodies of `set` join the subtrees of the slots of the tree
// built so far.  zero_counts: the new cells get bucket counters for a later pass.
static void launch_bucket_pass(const StepParams& p, BuildPhase set, bool first, bool zero_counts, int sms,
                               cudaStream_t s) {
    const long long rest = (long long)p.nchunks * phase_bodies(set);
    const unsigned grid_rest = (unsigned)((rest + 255) / 256);
    bucket_locate_kernel<<<grid_rest, 256, 0, s>>>(p, set, !first);
    // every cell of the tree so far: at most one per inserted body (1/16 of each chunk) plus
    // the roots
    const long long cells = (long long)p.nchunks * 16 + p.nuniv;
    bucket_alloc_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(p);
    bucket_scatter_kernel<<<grid_rest, 256, 0, s>>>(p, set);
    bucket_build_kernel<<<kBucketBlocksPerSm * sms, 32 * kBucketWarps, 0, s>>>(p, zero_counts);
}

// The first phase (one body per chunk) of the multi-phase schedules: in shared memory (one
// block per universe) when `top`, else through the global locks.
static void launch_first_phase(const StepParams& p, bool zero_counts, int top_cells, int split, cudaStream_t s) {
    if (top_cells > 0)
        top_build_kernel<<<split * p.nuniv, kTopThreads, top_build_smem(top_cells), s>>>(p, zero_counts, top_cells,
                                                                                       split);
    else
        build_kernel<<<(unsigned)((p.nchunks * (long long)phase_bodies(kFirstPhase) + 255) / 256), 256, 0, s>>>(
            p, kFirstPhase, zero_counts);
}

void launch_build(const StepParams& p, int phases, bool buckets, int sms, int top, int split, cudaStream_t s) {
    buckets = buckets && phases != 1;
    if (buckets && phases == 3) {
        // one lock phase (1/256 of each chunk), then the rest of the 1/16 sample as bucket
        // subtrees of that tree, then every other body as bucket subtrees of the sample's
        launch_first_phase(p, true, top, split, s);
        launch_bucket_pass(p, kThreePhases[1], true, true, sms, s);
        launch_bucket_pass(p, kBucketBodies, false, false, sms, s);
        return;
    }
    const BuildPhase* sched = phases == 1 ? kOnePass : (phases == 5 ? kFivePhases : kThreePhases);
    int count = phases == 1 ? 1 : (phases == 5 ? 5 : 3);
    if (buckets) count -= 2;   // five phases: the lock phases insert the 1/16 sample only
    for (int k = 0; k < count; ++k) {
        if (k == 0 && phases != 1) {
            launch_first_phase(p, buckets, top, split, s);
            continue;
        }
        const long long bodies = (long long)p.nchunks * phase_bodies(sched[k]);
        build_kernel<<<(unsigned)((bodies + 255) / 256), 256, 0, s>>>(p, sched[k], buckets);
    }
    if (buckets) launch_bucket_pass(p, kBucketBodies, true, false, sms, s);
}

cudaError_t prepare_tree_kernels() {
    return cudaFuncSetAttribute(top_build_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)top_build_smem(kTopCells));
}

size_t bucket_stack_bytes(int sms) {
    return (size_t)kBucketBlocksPerSm * sms * kBucketWarps * kBucketStack * sizeof(BucketTask);
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
