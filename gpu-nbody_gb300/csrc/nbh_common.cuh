// nbh_common.cuh — device data layout and helpers shared by the step kernels.
//
// Node index space (one pool shared by every universe of a sim):
//   [0, nbody)                 bodies, universe after universe
//   (bottom, nnodes - nuniv]    cells, allocated downward by an atomic counter
//   (nnodes - nuniv, nnodes]   the roots: universe u has root nnodes - u
// As in the reference (buildtree.cl:109, boundingbox.cl:180-193) every cell is allocated
// after its parent, so a child always has a lower index than its parent.
//
// Per node:   float4 node4[i]   = (x, y, z, mass): body position, cell centre during the
//                                  build, cell centre of mass after summarize
//             int    parent[i]  = enclosing cell (-1 for roots), set by the link pass
// Per cell c (offset k = c - nbody):
//             int    child[8k .. 8k+7]  child slots, -1 empty, -2 locked (buildtree.cl:7-8)
//             float4 kids4[8k .. 8k+7]  copies of the children's node records, in slot
//                                       order, written by summarize for the force walk
//             int    count[k], start[k], loff[k], arrive[k], clevel[k]
// Per body:   float4 vel[b], acc[b] (w: quadrupole error bound of the last force walk when
//             the learned opening angle is on), sorted[s] = body at depth-first position s
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/nbh.h"

namespace nbh {

constexpr int kNull = -1;
constexpr int kLock = -2;
constexpr int kMaxDepth = NBH_MAXDEPTH;

// Bounded device-side waits: a wait that has not ended after this many nanoseconds sets
// NBH_ERR_TIMEOUT and returns (the reference's spin-waits have no bound).
constexpr unsigned long long kWaitNs = 4000000000ull;

// Back-off of a descent that finds its slot locked: starts at kBackoffMinNs and doubles up
// to kBackoffMaxNs (compile-time tunables).
#ifndef NBH_BACKOFF_MIN_NS
#define NBH_BACKOFF_MIN_NS 64
#endif
#ifndef NBH_BACKOFF_MAX_NS
#define NBH_BACKOFF_MAX_NS 64
#endif
constexpr unsigned kBackoffMinNs = NBH_BACKOFF_MIN_NS;
constexpr unsigned kBackoffMaxNs = NBH_BACKOFF_MAX_NS;
constexpr int kDiagSlots = 32;

struct DevState {
    int status;          // NBH_OK or the first NBH_ERR_* raised by a stage
    int bottom;          // lowest allocated cell (reference _bottom)
    int max_depth;       // reference _maxDepth, kept across steps (atom_max)
    int step;            // reference _step: -1 after load, incremented by the bbox stage
    int bbox_ticket;     // last-block ticket of the bbox stage (reference _blockCount)
    int force_next;      // work counter of the force stage
    int theta_since;     // learned theta: steps up to this index use the fixed theta
    int theta_every;     // learned theta: steps between evaluations of the model (>= 1)
    unsigned long long interactions;   // accepted force evaluations of the last step
    int bucket_fill;     // bucketed build: entries handed out in the bucket work list
    int nbuckets;        // bucketed build: non-empty slots of the sampled tree
    int bucket_next;     // bucketed build: work counter of the subtree builders
    int pool_low;        // lowest cell whose slots a build may have written since the last reset
    unsigned long long pad2;
    // Build contention meters, spread over kDiagSlots addresses so that counting does not
    // itself serialise: descents that found their slot locked, and lost lock races.
    int lock_waits[32];
    int cas_misses[32];
};

// Read-only per-step parameters (passed by value).
struct StepParams {
    float4* node4;
    float4* vel;
    float4* acc;
    float4* kpos;        // Kahan compensation of positions (precise mode), may be null
    float4* kvel;        // Kahan compensation of velocities (precise mode), may be null
    int* child;          // 8 * ncells
    float4* kids4;       // 8 * ncells: node records of each cell's children (slot order)
    int* count;          // ncells
    int* start;          // ncells: first depth-first position of each cell
    int* loff;           // ncells: offset of a cell inside its parent's depth-first range
    int* arrive;         // ncells
    int* clevel;         // ncells: tree level of each cell (root = 0)
    float4* probe;       // nbody: force-probe output (x, y, z, error bound), or null
    int* parent;         // nnodes + 1
    int* sorted;         // nbody
    const float* theta_body;   // per-body theta, or null for fixed theta
    DevState* st;
    // universes
    const int* ubody;    // nuniv + 1 body offsets
    unsigned* ubox;      // nuniv * 6 ordered-int extents (min x,y,z, max x,y,z)
    float* uradius;      // nuniv root half-widths
    const int4* chunks;  // (universe, begin, end, 0) body chunks that never span universes
    const int2* warps;   // (first sorted position, universe) of each 32-body work item
    const int2* items64; // the same for 64-body items (vote width 64)
    const int2* items128;// the same for 128-body items (vote width 128)
    int nchunks;
    int nwarps;
    int nitems64;
    int nitems128;
    int nbody;
    int nnodes;          // NUMBER_OF_NODES (top of the pool)
    int nuniv;
    float theta2;        // theta^2 (reference THETA)
    float eps2;          // eps^2 (reference EPSILON)
    float dt;
    float G;
    int precise;
    int4* buckets;       // bucketed build: (slot, first entry, bodies, 0) per non-empty slot
    int* bwork;          // bucketed build: 2 * nbody entries (bodies of each bucket, ping-pong)
    void* bstack;        // bucketed build: per-warp task stacks of the large-bucket builder
    const int* item_order; // force: work items in the order to hand them out (null: in index order)
    int* item_cost;      // force: visits of each work item's walk, for the next step's order (may be null)
    int stack_cap;       // entries of each force group's shared-memory stack
    int theta_group;     // per-body theta: 1 = each vote group walks with its smallest angle
    int feat_gate;       // force launch gated on the learned-theta schedule: 0 none,
                         // 1 run only on bound-recording steps, 2 only on the others
    int force_list;      // 1: 64-wide walks without features take the lane-parallel list walk
};

__device__ __forceinline__ int* cell_child(const StepParams& p, int c) {
    return p.child + (static_cast<size_t>(c - p.nbody) << 3);
}

// Raise an error once; later stages see status != 0 and return at entry.
__device__ __forceinline__ void raise_error(DevState* st, int code) {
    atomicCAS(&st->status, 0, code);
}

// Learned opening angle schedule (steps >= theta_since, where theta_since is the first
// step after the model was switched on): the walks of steps since, since + k, since + 2k,
// ... record each body's error bound, and the model sets new angles on the step after
// each of them (k = theta_every; with k = 1 every walk records and every later step
// evaluates).  In between, bodies keep their angles and the walk records nothing.
__device__ __forceinline__ bool theta_bound_step(const DevState* st, int step) {
    const int k = st->theta_every > 0 ? st->theta_every : 1;
    return (step - st->theta_since) % k == 0;
}
__device__ __forceinline__ bool theta_model_step(const DevState* st, int step) {
    const int k = st->theta_every > 0 ? st->theta_every : 1;
    return step > st->theta_since && (step - st->theta_since) % k == 1 % k;
}

__device__ __forceinline__ int load_status(const DevState* st) {
    return *reinterpret_cast<const volatile int*>(&st->status);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Relaxed load/store at device scope: served by L2, never a stale L1 line.
__device__ __forceinline__ int ld_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(int* p, int v) {
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int cas_acquire(int* p, int cmp, int val) {
    int old;
    asm volatile("atom.acquire.gpu.global.cas.b32 %0, [%1], %2, %3;"
                 : "=r"(old) : "l"(p), "r"(cmp), "r"(val) : "memory");
    return old;
}
// L2 (cache-global) vector load: bypasses L1, so a line another SM just wrote is current.
__device__ __forceinline__ float4 ld_cg4(const float4* p) { return __ldcg(p); }

// Bounded wait until *p != value: polls from L2 with exponential back-off (min_ns doubling
// to kBackoffMaxNs) and gives up after limit_ns, raising NBH_ERR_TIMEOUT, or as soon as
// another stage raised an error.  Returns the value seen, or `value` when it gave up.
__device__ __forceinline__ int bounded_wait_ne(const int* p, int value, unsigned long long limit_ns, DevState* st,
                                               unsigned min_ns, int* polls) {
    const unsigned long long t0 = global_ns();
    unsigned backoff = min_ns;
    for (;;) {
        const int v = ld_relaxed(p);
        if (v != value) return v;
        if (load_status(st)) return value;
        if (global_ns() - t0 > limit_ns) {
            raise_error(st, NBH_ERR_TIMEOUT);
            return value;
        }
        if (polls) ++*polls;
        __nanosleep(backoff);
        backoff = backoff * 2 < kBackoffMaxNs ? backoff * 2 : kBackoffMaxNs;
    }
}

// Order-preserving float <-> uint mapping for atomicMin/atomicMax on extents.
__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Octant of body b in a cell with centre c: bit k set when the centre is below the body on
// axis k (buildtree.cl:65-68, 83-86).
__device__ __forceinline__ int octant(float cx, float cy, float cz, float bx, float by, float bz) {
    return (cx < bx ? 1 : 0) | (cy < by ? 2 : 0) | (cz < bz ? 4 : 0);
}

// a*b+c in the configured arithmetic: fused, or rounded product then rounded sum (the
// latter is what the reference kernels compute when the OpenCL compiler does not contract).
template <bool REF>
__device__ __forceinline__ float madd(float a, float b, float c) {
    if constexpr (REF) return __fadd_rn(__fmul_rn(a, b), c);
    else return __fmaf_rn(a, b, c);
}

}  // namespace nbh
