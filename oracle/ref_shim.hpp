// ref_shim.hpp — OpenCL C environment on the host, so that the reference project's own
// kernels (kernels/nbody/*.cl) compile unchanged as C++ and run on CPU threads.
// TEST INFRASTRUCTURE ONLY: it pins the oracle restatement (oracle/refbh.c) to the
// reference's behaviour.  Nothing in the product links it.
//
// Emulation model (the reference host launches global = 256, local = 16, 1-D,
// GPUBarnesHutNBodySimulation.java:126-129,274):
//  * each work-item is one OS thread; all 256 run concurrently, so the kernels'
//    cross-group spin-waits (summarizetree.cl:122-153, sort.cl:31-75) make progress;
//  * `__kernel` becomes a function template over the group id and `__local` becomes
//    `static`, so every group gets its own instance of the kernel's local arrays;
//  * barrier() is a per-group barrier that work-items leave when they return, which
//    gives the divergent "throttle" barriers (buildtree.cl:195, sort.cl:74) the meaning
//    of "wait for the items still in the loop";
//  * work_group_all() is the same barrier with an AND over the arriving items;
//  * atomics map to GCC __atomic builtins (sequentially consistent), and every atomic
//    load yields the CPU so that spinning items let the others run;
//  * calculateForce is warp-synchronous: work-item 0 advances and pushes the group's
//    shared stack with no barrier (calculateforce.cl:113-116,128-131,157-160), which is
//    correct only when the 16 items run in lockstep, as on the SIMD16 hardware the code
//    was written for.  Built with -DREF_LOCKSTEP, get_local_id() and mem_fence() are
//    group barriers: in that kernel every call to them is made by all 16 items in the
//    same order, so each shared-stack write is ordered after every item's read of the
//    previous value and before every item's next read;
//  * rsqrt(x) is 1/sqrtf(x) (correctly rounded in two steps), like the oracle's
//    reference arithmetic mode.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <array>
#include <utility>
#include <sched.h>

struct RefArgs {
    float *posX, *posY, *posZ, *velX, *velY, *velZ, *accX, *accY, *accZ;
    int *step, *blockCount, *bodyCount;
    float* radius;
    int *maxDepth, *bottom;
    float* mass;
    int *child, *start, *sorted, *error;
};

struct RefItem {
    int lid, grp, gid;
};
extern thread_local RefItem ref_item;

// Per-group barrier / vote (implemented in ref_emul.cpp).
void ref_group_barrier();
int ref_group_all(int pred);

#ifndef REF_RUNNER
typedef int atomic_int;
typedef float atomic_float;

enum { CLK_LOCAL_MEM_FENCE = 1, CLK_GLOBAL_MEM_FENCE = 2 };
enum { memory_order_relaxed = 0, memory_order_acquire = 2, memory_order_release = 3,
       memory_order_acq_rel = 4, memory_order_seq_cst = 5 };
enum { memory_scope_work_item = 0, memory_scope_work_group = 1, memory_scope_device = 2,
       memory_scope_all_svm_devices = 3 };

#ifdef REF_LOCKSTEP
static inline int get_local_id(int) { ref_group_barrier(); return ref_item.lid; }
static inline void mem_fence(int) { ref_group_barrier(); }
#else
static inline int get_local_id(int) { return ref_item.lid; }
static inline void mem_fence(int) { __atomic_thread_fence(__ATOMIC_SEQ_CST); }
#endif
static inline int get_group_id(int) { return ref_item.grp; }
static inline int get_global_id(int) { return ref_item.gid; }
static inline int get_local_size(int) { return WORKGROUP_SIZE; }
static inline int get_num_groups(int) { return NUM_WORK_GROUPS; }
static inline int get_global_size(int) { return WORKGROUP_SIZE * NUM_WORK_GROUPS; }
static inline int get_work_dim() { return 1; }

static inline void barrier(int) { ref_group_barrier(); }
static inline int work_group_all(int pred) { return ref_group_all(pred); }
static inline void atomic_work_item_fence(int, int, int) { __atomic_thread_fence(__ATOMIC_SEQ_CST); }

static inline int atom_inc(volatile int* p) { return __atomic_fetch_add(p, 1, __ATOMIC_SEQ_CST); }
static inline int atom_dec(volatile int* p) { return __atomic_fetch_sub(p, 1, __ATOMIC_SEQ_CST); }
static inline int atom_cmpxchg(volatile int* p, int cmp, int val) {
    int expected = cmp;
    __atomic_compare_exchange_n(p, &expected, val, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
    return expected;
}
static inline int atom_max(volatile int* p, int v) {
    int old = __atomic_load_n(p, __ATOMIC_SEQ_CST);
    while (old < v && !__atomic_compare_exchange_n(p, &old, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
    }
    return old;
}
static inline int atomic_load_explicit(volatile int* p, int, int) {
    sched_yield();
    return __atomic_load_n(p, __ATOMIC_SEQ_CST);
}
static inline float atomic_load_explicit(volatile float* p, int, int) {
    sched_yield();
    int bits = __atomic_load_n(reinterpret_cast<volatile int*>(p), __ATOMIC_SEQ_CST);
    float v;
    std::memcpy(&v, &bits, sizeof v);
    return v;
}
static inline void atomic_store_explicit(volatile int* p, int v, int, int) {
    __atomic_store_n(p, v, __ATOMIC_SEQ_CST);
}
static inline void atomic_store_explicit(volatile float* p, float v, int, int) {
    int bits;
    std::memcpy(&bits, &v, sizeof bits);
    __atomic_store_n(reinterpret_cast<volatile int*>(p), bits, __ATOMIC_SEQ_CST);
}

static inline float ocl_fmin(float a, float b) { return std::fmin(a, b); }
static inline float ocl_fmax(float a, float b) { return std::fmax(a, b); }
static inline int ocl_max(int a, int b) { return a > b ? a : b; }
static inline float ocl_rsqrt(float x) { return 1.0f / std::sqrt(x); }

#define fmin(a, b) ocl_fmin((a), (b))
#define fmax(a, b) ocl_fmax((a), (b))
#define max(a, b) ocl_max((a), (b))
#define rsqrt(x) ocl_rsqrt((x))

// Address-space and kernel qualifiers.  No system header may be included after this.
#define __kernel template <int REF_GROUP>
#define __global
#define __local static
#define local static
#define __attribute__(x)

#endif  // REF_RUNNER

// Exported per kernel by ref_kernel_tu.cpp: run one work-item of `group`.
extern "C" void ref_item_boundingBox(int group, const RefArgs* a);
extern "C" void ref_item_buildTree(int group, const RefArgs* a);
extern "C" void ref_item_summarizeTree(int group, const RefArgs* a);
extern "C" void ref_item_sort(int group, const RefArgs* a);
extern "C" void ref_item_calculateForce(int group, const RefArgs* a);
extern "C" void ref_item_integrate(int group, const RefArgs* a);
