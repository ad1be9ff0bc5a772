// nbh_force.cu — the force stage: Barnes-Hut tree walk with a group-voted opening test.
#include "nbh_common.cuh"
#include "nbh_kernels.h"

namespace nbh {

// Launch geometry is chosen at run time (nbh_autotune): threads per block (64 / 128 / 256)
// and the entries of each group's shared-memory stack of pending children, each with its
// preloaded node record.  Opening a cell at level l while every ancestor still has 7
// pending children needs 7*l + 8 entries, so a stack of `cap` entries covers trees up to
// fast_max_depth(cap) levels; deeper trees take the per-level (cell, next child) walk.
constexpr int kForceThreadsMax = 256;
constexpr int kStackCapMax = 256;
constexpr int kStackCapMin = 64;     // the deep walk keeps 2 * kMaxDepth ints in the same space
__host__ __device__ constexpr int fast_max_depth(int cap) { return (cap - 8) / 7 + 1; }

// Lanes of one vote group: W bodies on W lanes for W <= 32; W = 64 puts two bodies on
// each lane of one warp.
template <int W>
__host__ __device__ constexpr int group_lanes() {
    return W < 32 ? W : 32;
}

template <int W>
constexpr size_t force_smem_bytes(int threads, int cap) {
    return (size_t)(threads / group_lanes<W>()) * cap * (sizeof(float4) + sizeof(int2));
}

// The list walk (64-wide groups): per group, the records of accepted nodes awaiting
// evaluation (at most 31 wait after an evaluation and one round adds at most 32) with each
// record's full cell width^2 (for the error bound; 0 for a body), the undecided cells of a
// round (at most 32), and a stack of `cap` cells whose children are still to be tested,
// with their levels (a 64-entry stack also holds the per-level walk's 2 * kMaxDepth ints).
constexpr int kListCap = 64;
constexpr size_t list_group_bytes(int cap) {
    return kListCap * (sizeof(float4) + sizeof(float)) + 32 * sizeof(float4) + (size_t)cap * sizeof(int2);
}
constexpr size_t force_list_smem_bytes(int threads, int cap) { return (size_t)(threads / 32) * list_group_bytes(cap); }
static_assert(kStackCapMin * sizeof(int2) >= 2 * kMaxDepth * sizeof(int), "the per-level walk fits the cell stack");

// Opening threshold of tree level L (root = 0): r^2/theta^2 * 4^-L + eps^2
// (calculateforce.cl:52-67).  The walk carries s = 4^-L (exact powers of two) and forms
// t0*s + eps^2, which equals ldexp(t0, -2L) + eps^2 in the normal range; below it eps^2
// absorbs the term either way.
__device__ __forceinline__ float level_dq(float t0, int level, float eps2) {
    return __fadd_rn(ldexpf(t0, -2 * level), eps2);
}

// 1/sqrt(d2).  d2 >= eps^2 > 0 is never subnormal, so the flush-to-zero form of the
// hardware approximation returns exactly what rsqrtf would.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// One accepted interaction (calculateforce.cl:146-151).  With FEAT it also accumulates
// the quadrupole error bound m s^2 / d^4 of an accepted cell of full width^2 s2 (0 for a
// body), the feature the learned opening angle is predicted from.
template <bool REF, bool FEAT>
__device__ __forceinline__ void interact(const float4 q, const float dx, const float dy, const float dz,
                                         const float d2, float& ax, float& ay, float& az, float& eb,
                                         const float s2) {
    float rd;
    if constexpr (REF) rd = __fdiv_rn(1.0f, __fsqrt_rn(d2));
    else rd = rsqrt_ftz(d2);
    const float f = __fmul_rn(__fmul_rn(__fmul_rn(q.w, rd), rd), rd);
    ax = madd<REF>(dx, f, ax);
    ay = madd<REF>(dy, f, ay);
    az = madd<REF>(dz, f, az);
    if constexpr (FEAT) eb = __fmaf_rn(__fmul_rn(f, rd), s2, eb);
}

template <bool REF>
__device__ __forceinline__ float dist2(const float dx, const float dy, const float dz, const float eps2) {
    if constexpr (REF)
        return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)), eps2);
    else
        return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmaf_rn(dz, dz, eps2)));
}

// The first 32 records: unrolled completely for two or more bodies per lane (the 64-wide
// walk's force 2.6 % faster than unrolled by 8), by 8 for one (the 32-wide walk on a 16K
// ball measured the same either way).
template <int BPL, bool FEAT>
__device__ __forceinline__ void eval_list32(const float4* lst, const float* lw, const float4 (&pb)[BPL],
                                            const float eps2, float (&ax)[BPL], float (&ay)[BPL], float (&az)[BPL],
                                            float (&eb)[BPL]) {
#pragma unroll(BPL >= 2 ? 32 : 8)
    for (int i = 0; i < 32; ++i) {
        const float4 q = lst[i];
        const float s2 = FEAT ? lw[i] : 0.0f;
#pragma unroll
        for (int k = 0; k < BPL; ++k) {
            const float dx = __fsub_rn(q.x, pb[k].x);
            const float dy = __fsub_rn(q.y, pb[k].y);
            const float dz = __fsub_rn(q.z, pb[k].z);
            const float d2 = dist2<false>(dx, dy, dz, eps2);
            interact<false, FEAT>(q, dx, dy, dz, d2, ax[k], ay[k], az[k], eb[k], s2);
        }
    }
}

// Evaluate the first cnt records of a group's list for the lane's bodies, in list order
// (with FEAT also their error bounds, from the widths in lw).
template <int BPL, bool FEAT>
__device__ __forceinline__ void eval_list(const float4* lst, const float* lw, const int cnt, const float4 (&pb)[BPL],
                                          const float eps2, float (&ax)[BPL], float (&ay)[BPL], float (&az)[BPL],
                                          float (&eb)[BPL]) {
#pragma unroll 4
    for (int i = 0; i < cnt; ++i) {
        const float4 q = lst[i];
        const float s2 = FEAT ? lw[i] : 0.0f;
#pragma unroll
        for (int k = 0; k < BPL; ++k) {
            const float dx = __fsub_rn(q.x, pb[k].x);
            const float dy = __fsub_rn(q.y, pb[k].y);
            const float dz = __fsub_rn(q.z, pb[k].z);
            const float d2 = dist2<false>(dx, dy, dz, eps2);
            interact<false, FEAT>(q, dx, dy, dz, d2, ax[k], ay[k], az[k], eb[k], s2);
        }
    }
}

// -------------------------------------------------------------------------------------
// Force (calculateforce.cl:52-185).  A group of W bodies (W = 32: one warp; W = 16: the
// reference's work-group, :99,145; W = 64: one warp with two bodies per lane) takes W
// consecutive bodies of the depth-first order and walks its universe's tree.  A body
// child is always accepted; a cell child only if every body of the group sees
// d^2 + eps^2 >= dq[level] (work_group_all, :145), else it is opened.  The walk is
// depth-first in child order (children are compacted, so the first empty slot ends a
// cell), so every body accumulates its interactions in the reference's order.  Every lane
// of a group accepts the same children, so the group's interaction count is counted once
// per opened cell, not per visit.
//
// GB300 schedule: opening a cell loads its 8 child slots and the 8 node records that
// summarize stored next to them (kids4) with one load per lane -- one round trip per
// opened cell -- and pushes them, first child on top, onto the group's shared-memory
// stack with their opening threshold (fixed angle: t0 * 4^-level + eps^2, formed once at
// the push; per-body angle: the level factor 4^-level) or -1 for bodies, which makes the
// test pass; each visit reads one record from shared memory and needs no branch on its
// kind.  With W = 64 every stack pop, vote and cell opening serves two bodies per lane.
// Lanes past the end of a universe walk with their group's first body, so they never
// change a vote and need no predicate.  Work items (32 bodies; 64 for W = 64) are handed
// out dynamically.  After the walk: the leapfrog velocity correction for step > 0
// (:174-181) and the acceleration store (:183-185).
//
// REF: reference arithmetic (rounded products, 1/sqrt correctly rounded); otherwise FMA and
// the hardware inverse square root.  PB: per-body opening angle from theta_body (with
// p.theta_group, the smallest angle of the group for all its bodies).  FEAT:
// also accumulate each body's quadrupole error bound into acc.w.  With p.probe set the
// results go to p.probe (x, y, z, bound) and no body state changes (force probe).  With
// p.feat_gate set, a launch that does not match the step's place in the learned-theta
// schedule returns at once (the step graph holds a recording and a plain launch).
//
// LIST (W = 32, 64 or 128: one warp per group; FMA arithmetic): the same votes, taken
// lane-parallel.  Each round the lanes take the children of up to four cells from the
// group's cell stack, one child per lane (8 lanes per cell), and decide each child on its
// own lane: a body is accepted; a cell is accepted when even the group's bounding box
// passes the test (the box's distance components bound every body's from below, and the
// rounded subtractions, the fused squares and the comparison are monotone, so every body's
// own test passes), and opened when the group's body nearest the box centre fails it (then
// the vote fails; with per-body angles also when the body with the smallest angle fails
// it).  Only the remaining cells take the vote of every body, one after another.  Accepted records go to a list in shared memory, evaluated 32 at a time in a
// loop of arithmetic alone: the same interactions as the per-visit walk, accumulated in
// list order (rounding may differ from it in the last bits).  A cell stack that would
// overflow restarts the group on the per-level walk (stack_cap entries: 256 by default,
// enough for every 64-body group of the benchmarked spheres, which needed at most 99).
template <int W, bool REF, bool PB, bool FEAT, bool LIST = false>
__device__ __forceinline__ void force_walk(const StepParams& p) {
    static_assert(!LIST || (W >= 32 && !REF), "the list walk takes whole-warp groups and FMA arithmetic");
    if (load_status(p.st)) return;
    if (p.feat_gate && theta_bound_step(p.st, p.st->step) != (p.feat_gate == 1)) return;
    constexpr int GL = group_lanes<W>();            // lanes per group
    constexpr int BPL = W / GL;                     // bodies per lane
    const int cap = p.stack_cap;
    const int groups = blockDim.x / GL;
    // The stack entry carries the finished threshold when it is the same for every body
    // of the group (fixed angle) and nothing else needs the level factor.
    constexpr bool kStoreDq = !PB && !FEAT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4* const sq_all = reinterpret_cast<float4*>(smem_raw);
    int2* const se_all = reinterpret_cast<int2*>(sq_all + groups * cap);
    const int lane = threadIdx.x & 31;
    const int grp = threadIdx.x / GL;
    const int glane = threadIdx.x % GL;
    const unsigned gmask = (GL == 32) ? 0xffffffffu : (0xffffu << (16 * (lane >> 4)));
    float4* const sq = sq_all + grp * cap;           // node record of each pending child
    int2* const se = se_all + grp * cap;             // (node index, bits of threshold or level factor)
    // list walk: the group's list of accepted records and its stack of (cell, level)
    float4* const lst = reinterpret_cast<float4*>(smem_raw + (size_t)grp * list_group_bytes(cap));
    float* const lw = reinterpret_cast<float*>(lst + kListCap);
    float4* const ud = reinterpret_cast<float4*>(lw + kListCap);   // undecided cells of a round
    int2* const cst = reinterpret_cast<int2*>(ud + 32);
    // deep-tree walk: (cell, next) per level
    int* const snode = LIST ? reinterpret_cast<int*>(cst) : reinterpret_cast<int*>(se);
    int* const snext = snode + kMaxDepth;
    const int nbody = p.nbody;
    const float eps2 = p.eps2;
    const int step = p.st->step;
    const bool fast = p.st->max_depth <= fast_max_depth(cap);
    const float4* __restrict__ node4 = p.node4;
    const int* __restrict__ child = p.child;
    const float4* __restrict__ kids4 = p.kids4;
    const int2* __restrict__ items = BPL == 4 ? p.items128 : (BPL == 2 ? p.items64 : p.warps);
    const int nitems = BPL == 4 ? p.nitems128 : (BPL == 2 ? p.nitems64 : p.nwarps);
    unsigned long long my_inter = 0;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(&p.st->force_next, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nitems) break;
        if (p.item_order) item = p.item_order[item];   // costly items first (see item_order_kernel)
        const int2 wi = items[item];
        const int u = wi.y;
        const int uend = p.ubody[u + 1];
        // Lanes past the universe's end take their group's first body.
        const int gfirst = wi.x + (GL < 32 ? (lane / GL) * GL : 0);
        const bool gvalid = gfirst < uend;       // the group has any body at all
        const float r = p.uradius[u];
        const float rr = __fmul_rn(r, r);
        bool valid[BPL];
        int b[BPL];
        float4 pb[BPL];
        float t0[BPL];
        float ax[BPL], ay[BPL], az[BPL], eb[BPL];
#pragma unroll
        for (int k = 0; k < BPL; ++k) {
            const int sk = wi.x + 32 * k + lane;
            valid[k] = sk < uend;
            b[k] = gvalid ? p.sorted[valid[k] ? sk : gfirst] : 0;
            pb[k] = node4[b[k]];
            float th2 = p.theta2;
            if constexpr (PB) {
                const float th = p.theta_body[b[k]];
                th2 = __fmul_rn(th, th);
            }
            t0[k] = th2 > 0.0f ? __fdiv_rn(rr, th2) : rr;
            ax[k] = ay[k] = az[k] = eb[k] = 0.f;
        }
        if constexpr (PB) {
            if (p.theta_group) {
                // the group walks with its smallest angle (largest r^2 / theta^2), the walk
                // of a fixed angle; lanes past the end hold the first body's angle
                float tm = t0[0];
#pragma unroll
                for (int k = 1; k < BPL; ++k) tm = fmaxf(tm, t0[k]);
#pragma unroll
                for (int o = GL / 2; o > 0; o >>= 1) tm = fmaxf(tm, __shfl_xor_sync(gmask, tm, o));
#pragma unroll
                for (int k = 0; k < BPL; ++k) t0[k] = tm;
            }
        }
        long long ninter = 0;
        int visits = 0;                                 // cost of this group's walk
        const int root = p.nnodes - u;

        if (gvalid) {
            bool walked = false;
            if constexpr (LIST) {
                walked = true;
                // the group's bounding box (lanes past the end hold the first body)
                float lox = pb[0].x, loy = pb[0].y, loz = pb[0].z, hix = pb[0].x, hiy = pb[0].y, hiz = pb[0].z;
#pragma unroll
                for (int k = 1; k < BPL; ++k) {
                    lox = fminf(lox, pb[k].x), loy = fminf(loy, pb[k].y), loz = fminf(loz, pb[k].z);
                    hix = fmaxf(hix, pb[k].x), hiy = fmaxf(hiy, pb[k].y), hiz = fmaxf(hiz, pb[k].z);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    lox = fminf(lox, __shfl_xor_sync(0xffffffffu, lox, o));
                    loy = fminf(loy, __shfl_xor_sync(0xffffffffu, loy, o));
                    loz = fminf(loz, __shfl_xor_sync(0xffffffffu, loz, o));
                    hix = fmaxf(hix, __shfl_xor_sync(0xffffffffu, hix, o));
                    hiy = fmaxf(hiy, __shfl_xor_sync(0xffffffffu, hiy, o));
                    hiz = fmaxf(hiz, __shfl_xor_sync(0xffffffffu, hiz, o));
                }
                // the representative: the body nearest the box centre (lowest index on ties)
                const float cx = 0.5f * (lox + hix), cy = 0.5f * (loy + hiy), cz = 0.5f * (loz + hiz);
                float best = 0.0f;
                int bid = 0;
#pragma unroll
                for (int k = 0; k < BPL; ++k) {
                    const float ex = pb[k].x - cx, ey = pb[k].y - cy, ez = pb[k].z - cz;
                    const float d = ex * ex + ey * ey + ez * ez;
                    if (k == 0 || d < best) {
                        best = d;
                        bid = lane * BPL + k;
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bid, o);
                    if (ob < best || (ob == best && oi < bid)) {
                        best = ob;
                        bid = oi;
                    }
                }
                const int rsrc = bid / BPL, rk = bid % BPL;
                float4 rp = pb[0];
                float rt = t0[0];
#pragma unroll
                for (int k = 1; k < BPL; ++k)
                    if (rk == k) {
                        rp = pb[k];
                        rt = t0[k];
                    }
                rp.x = __shfl_sync(0xffffffffu, rp.x, rsrc);
                rp.y = __shfl_sync(0xffffffffu, rp.y, rsrc);
                rp.z = __shfl_sync(0xffffffffu, rp.z, rsrc);
                // thresholds: the box takes the group's largest r^2/theta^2 (the smallest angle)
                float tlb = t0[0], trep = t0[0];
                if constexpr (PB) {
#pragma unroll
                    for (int k = 1; k < BPL; ++k) tlb = fmaxf(tlb, t0[k]);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) tlb = fmaxf(tlb, __shfl_xor_sync(0xffffffffu, tlb, o));
                    trep = __shfl_sync(0xffffffffu, rt, rsrc);
                }
                // per-body angles: a second representative, the body with the smallest angle
                // (the largest r^2/theta^2, the box's threshold; lowest index on ties) -- a
                // vote fails most often on it (learned step 2.36 -> 2.32 ms at 1M)
                float4 rp2 = rp;
                if constexpr (PB) {
                    float bt = t0[0];
                    int bi = lane * BPL;
#pragma unroll
                    for (int k = 1; k < BPL; ++k)
                        if (t0[k] > bt) {
                            bt = t0[k];
                            bi = lane * BPL + k;
                        }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        const float ob = __shfl_xor_sync(0xffffffffu, bt, o);
                        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                        if (ob > bt || (ob == bt && oi < bi)) {
                            bt = ob;
                            bi = oi;
                        }
                    }
                    const int r2src = bi / BPL, r2k = bi % BPL;
                    float4 mine2 = pb[0];
#pragma unroll
                    for (int k = 1; k < BPL; ++k)
                        if (r2k == k) mine2 = pb[k];
                    rp2.x = __shfl_sync(0xffffffffu, mine2.x, r2src);
                    rp2.y = __shfl_sync(0xffffffffu, mine2.y, r2src);
                    rp2.z = __shfl_sync(0xffffffffu, mine2.z, r2src);
                }
                const unsigned lt = (1u << lane) - 1u;
                if (lane == 0) cst[0] = make_int2(root, 0);
                int ctop = 1, lcnt = 0, opened = 0;    // every tested child is accepted or opened
                long long accepted = 0;
                __syncwarp();
                while (ctop > 0) {
                    const int k4 = min(4, ctop);
                    const int ci = lane >> 3;
                    int chk = kNull, lv = 0;
                    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (ci < k4) {
                        const int2 e = cst[ctop - 1 - ci];
                        lv = e.y;
                        const size_t o8 = ((size_t)(e.x - nbody) << 3) + (lane & 7);
                        chk = __ldg(child + o8);
                        q = __ldg(kids4 + o8);
                    }
                    ctop -= k4;
                    __syncwarp();          // the popped entries are read before pushes reuse them
                    // children of a level-lv cell: t0 * 4^-lv + eps^2 (4^-lv exact)
                    const float sl = __int_as_float((127 - 2 * lv) << 23);
                    bool acc = chk >= 0 && chk < nbody;
                    bool opn = false, inc = false;
                    if (chk >= nbody) {
                        const float gx = fmaxf(fmaxf(__fsub_rn(q.x, hix), __fsub_rn(lox, q.x)), 0.0f);
                        const float gy = fmaxf(fmaxf(__fsub_rn(q.y, hiy), __fsub_rn(loy, q.y)), 0.0f);
                        const float gz = fmaxf(fmaxf(__fsub_rn(q.z, hiz), __fsub_rn(loz, q.z)), 0.0f);
                        const float dlb = dist2<false>(gx, gy, gz, eps2);
                        const float qlb = PB ? __fmaf_rn(tlb, sl, eps2) : __fadd_rn(__fmul_rn(tlb, sl), eps2);
                        if (dlb >= qlb) {
                            acc = true;
                        } else {
                            const float rx = __fsub_rn(q.x, rp.x), ry = __fsub_rn(q.y, rp.y), rz = __fsub_rn(q.z, rp.z);
                            const float qr = PB ? __fmaf_rn(trep, sl, eps2) : qlb;
                            if (dist2<false>(rx, ry, rz, eps2) < qr) {
                                opn = true;
                            } else if constexpr (PB) {
                                // the smallest-angle body's own test (its threshold is the box's)
                                const float sx = __fsub_rn(q.x, rp2.x), sy = __fsub_rn(q.y, rp2.y),
                                            sz = __fsub_rn(q.z, rp2.z);
                                if (dist2<false>(sx, sy, sz, eps2) < qlb) opn = true;
                                else inc = true;
                            } else {
                                inc = true;
                            }
                        }
                    }
                    // undecided cells: the vote of every body, one cell after another
                    const unsigned im = __ballot_sync(0xffffffffu, inc);
                    if (im) {
                        // their records go to shared memory and every lane reads them back in turn
                        const int nud = __popc(im);
                        const int mine = __popc(im & lt);
                        if (inc) ud[mine] = make_float4(q.x, q.y, q.z, sl);
                        __syncwarp();
                        unsigned res = 0;
#pragma unroll 2
                        for (int j = 0; j < nud; ++j) {
                            const float4 uq = ud[j];
                            bool pass = true;
#pragma unroll
                            for (int k = 0; k < BPL; ++k) {
                                const float dx = __fsub_rn(uq.x, pb[k].x);
                                const float dy = __fsub_rn(uq.y, pb[k].y);
                                const float dz = __fsub_rn(uq.z, pb[k].z);
                                const float dq =
                                    PB ? __fmaf_rn(t0[k], uq.w, eps2) : __fadd_rn(__fmul_rn(t0[k], uq.w), eps2);
                                pass = pass && dist2<false>(dx, dy, dz, eps2) >= dq;
                            }
                            res |= (__all_sync(0xffffffffu, pass) ? 1u : 0u) << j;
                        }
                        if (inc) {
                            acc = (res >> mine) & 1u;
                            opn = !acc;
                        }
                    }
                    const unsigned am = __ballot_sync(0xffffffffu, acc);
                    const unsigned om = __ballot_sync(0xffffffffu, opn);
                    const int on = __popc(om);
                    opened += on;
                    if (ctop + on > cap) {               // group-uniform
                        walked = false;
                        break;
                    }
                    if (acc) {
                        const int at = lcnt + __popc(am & lt);
                        lst[at] = q;
                        // full width^2 of an accepted cell, r^2 * 4^-level (0 for a body)
                        if constexpr (FEAT) lw[at] = chk >= nbody ? __fmul_rn(rr, sl) : 0.0f;
                    }
                    if (opn) cst[ctop + __popc(om & lt)] = make_int2(chk, min(lv + 1, kMaxDepth - 1));
                    lcnt += __popc(am);
                    ctop += on;
                    __syncwarp();          // list and stack written before they are read
                    if (lcnt >= 32) {
                        // 32 records at a time; the rest (at most 31) move to the front
                        eval_list32<BPL, FEAT>(lst, lw, pb, eps2, ax, ay, az, eb);
                        accepted += 32;
                        __syncwarp();
                        const int rest = lcnt - 32;
                        if (lane < rest) {
                            lst[lane] = lst[32 + lane];
                            if constexpr (FEAT) lw[lane] = lw[32 + lane];
                        }
                        lcnt = rest;
                        __syncwarp();
                    }
                    if (ctop == 0 && lcnt > 0) {
                        eval_list<BPL, FEAT>(lst, lw, lcnt, pb, eps2, ax, ay, az, eb);
                        accepted += lcnt;
                        lcnt = 0;
                        __syncwarp();
                    }
                }
                if (walked) {
                    ninter = accepted;
                    visits = (int)accepted + opened;
                } else {
#pragma unroll
                    for (int k = 0; k < BPL; ++k) ax[k] = ay[k] = az[k] = eb[k] = 0.f;
                    __syncwarp();
                }
            } else if (fast) {
                walked = true;
                int top = 0;
                int pushed = 0, opened = -1;
                int open = root;
                float open_s = 1.0f;                      // 4^-level of open's children
                bool ok = true;
                for (;;) {
                    // push the children of `open`, first child on top
                    int chk = kNull;
                    float4 qk = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (glane < 8) {
                        const size_t o8 = ((size_t)(open - nbody) << 3) + glane;
                        chk = __ldg(child + o8);
                        qk = __ldg(kids4 + o8);
                    }
                    float tag = open_s;
                    if constexpr (kStoreDq) {
                        // level factor of open's children, 4^-level(open), exact; the same
                        // threshold the visit would form from it
                        const int lv = __ldg(p.clevel + (open - nbody));
                        tag = __fadd_rn(__fmul_rn(t0[0], __int_as_float((127 - 2 * lv) << 23)), eps2);
                    }
                    const unsigned bal = __ballot_sync(gmask, glane < 8 && chk >= 0) & gmask;
                    const int cnt = __popc(bal);
                    if (top + cnt > cap) {                 // unreachable below fast_max_depth(cap)
                        raise_error(p.st, NBH_ERR_DEPTH);
                        ok = false;
                        break;
                    }
                    if (glane < cnt) {
                        const int slot = top + cnt - 1 - glane;
                        sq[slot] = qk;
                        se[slot] = make_int2(chk, __float_as_int(chk >= nbody ? tag : -1.0f));
                    }
                    top += cnt;
                    pushed += cnt;
                    ++opened;
                    __syncwarp(gmask);
                    // visit until a cell has to be opened or the stack is empty
                    open = -1;
                    while (top > 0) {
                        --top;
                        const int2 e = se[top];
                        const float4 q = sq[top];
                        const float sl = __int_as_float(e.y);
                        float dx[BPL], dy[BPL], dz[BPL], d2[BPL];
                        bool pass = true;
#pragma unroll
                        for (int k = 0; k < BPL; ++k) {
                            dx[k] = __fsub_rn(q.x, pb[k].x);
                            dy[k] = __fsub_rn(q.y, pb[k].y);
                            dz[k] = __fsub_rn(q.z, pb[k].z);
                            d2[k] = dist2<REF>(dx[k], dy[k], dz[k], eps2);
                            // t0 * 4^-level is exact (a power of two), so one fused op gives the
                            // same threshold as the rounded product and sum
                            const float dq = kStoreDq ? sl : __fmaf_rn(t0[k], sl, eps2);
                            pass = pass && d2[k] >= dq;
                        }
                        if (__all_sync(gmask, pass)) {
                            const float s2 = FEAT ? __fmul_rn(rr, fmaxf(sl, 0.0f)) : 0.0f;
#pragma unroll
                            for (int k = 0; k < BPL; ++k)
                                interact<REF, FEAT>(q, dx[k], dy[k], dz[k], d2[k], ax[k], ay[k], az[k], eb[k], s2);
                        } else {
                            open = e.x;
                            if constexpr (!kStoreDq) open_s = __fmul_rn(sl, 0.25f);
                            break;
                        }
                    }
                    if (open < 0) break;
                    __syncwarp(gmask);     // every lane has read the stack before it is refilled
                }
                if (ok) ninter = pushed - opened;
                visits = pushed;
            }
            if (!walked) {
                // Deep trees: per-level (cell, next child) walk (calculateforce.cl:112-172).
                int depth = 0;
                int node = root;
                int k8 = 0;
                float dq[BPL];
#pragma unroll
                for (int k = 0; k < BPL; ++k) dq[k] = level_dq(t0[k], 0, eps2);
                for (;;) {
                    int ch = kNull;
                    if (k8 < 8) ch = __ldg(child + ((size_t)(node - nbody) << 3) + k8);
                    if (ch < 0) {
                        if (depth == 0) break;
                        --depth;
                        node = snode[depth];
                        k8 = snext[depth];
#pragma unroll
                        for (int k = 0; k < BPL; ++k) dq[k] = level_dq(t0[k], depth, eps2);
                        continue;
                    }
                    ++k8;
                    const float4 q = __ldg(node4 + ch);
                    float dx[BPL], dy[BPL], dz[BPL], d2[BPL];
                    bool pass = true;
#pragma unroll
                    for (int k = 0; k < BPL; ++k) {
                        dx[k] = __fsub_rn(q.x, pb[k].x);
                        dy[k] = __fsub_rn(q.y, pb[k].y);
                        dz[k] = __fsub_rn(q.z, pb[k].z);
                        d2[k] = dist2<REF>(dx[k], dy[k], dz[k], eps2);
                        pass = pass && d2[k] >= dq[k];
                    }
                    if (ch < nbody || __all_sync(gmask, pass)) {
                        const float s2 = ch >= nbody ? ldexpf(rr, -2 * depth) : 0.0f;
#pragma unroll
                        for (int k = 0; k < BPL; ++k)
                            interact<REF, FEAT>(q, dx[k], dy[k], dz[k], d2[k], ax[k], ay[k], az[k], eb[k], s2);
                        ++ninter;
                    } else {
                        if (depth + 1 >= kMaxDepth) {   // unreachable for a tree the build accepted
                            raise_error(p.st, NBH_ERR_DEPTH);
                            break;
                        }
                        // every lane writes the same entry, so no lane reads a stale one
                        snode[depth] = node;
                        snext[depth] = k8;
                        ++depth;
                        node = ch;
                        k8 = 0;
#pragma unroll
                        for (int k = 0; k < BPL; ++k) dq[k] = level_dq(t0[k], depth, eps2);
                    }
                }
            }
        }

#pragma unroll
        for (int k = 0; k < BPL; ++k) {
            if (!valid[k]) continue;
            if (p.G != 1.0f) {
                ax[k] = __fmul_rn(ax[k], p.G);
                ay[k] = __fmul_rn(ay[k], p.G);
                az[k] = __fmul_rn(az[k], p.G);
                eb[k] = __fmul_rn(eb[k], p.G);
            }
            my_inter += (unsigned long long)ninter;
            if (p.probe) {
                p.probe[b[k]] = make_float4(ax[k], ay[k], az[k], eb[k]);
                continue;
            }
            float4 v = p.vel[b[k]];
            const float4 ao = p.acc[b[k]];
            if (step > 0) {
                const float tx = __fmul_rn(__fsub_rn(ax[k], ao.x), p.dt);
                const float ty = __fmul_rn(__fsub_rn(ay[k], ao.y), p.dt);
                const float tz = __fmul_rn(__fsub_rn(az[k], ao.z), p.dt);
                if (p.precise) {
                    float4 kv = p.kvel[b[k]];
                    float y1, t1;
                    y1 = __fsub_rn(__fmul_rn(tx, 0.5f), kv.x); t1 = __fadd_rn(v.x, y1); kv.x = __fsub_rn(__fsub_rn(t1, v.x), y1); v.x = t1;
                    y1 = __fsub_rn(__fmul_rn(ty, 0.5f), kv.y); t1 = __fadd_rn(v.y, y1); kv.y = __fsub_rn(__fsub_rn(t1, v.y), y1); v.y = t1;
                    y1 = __fsub_rn(__fmul_rn(tz, 0.5f), kv.z); t1 = __fadd_rn(v.z, y1); kv.z = __fsub_rn(__fsub_rn(t1, v.z), y1); v.z = t1;
                    p.kvel[b[k]] = kv;
                } else {
                    v.x = madd<REF>(tx, 0.5f, v.x);
                    v.y = madd<REF>(ty, 0.5f, v.y);
                    v.z = madd<REF>(tz, 0.5f, v.z);
                }
                p.vel[b[k]] = v;
            }
            p.acc[b[k]] = make_float4(ax[k], ay[k], az[k], eb[k]);
        }
        if (p.item_cost) {
            // the item's cost: its group's visits (the deep walk counts accepted children);
            // two half-warp groups (W = 16) add up
            int c = visits > 0 ? visits : (int)min(ninter, (long long)0x7fffffff);
            if (GL < 32) c += __shfl_down_sync(0xffffffffu, c, 16);
            if (lane == 0) p.item_cost[item] = c;
        }
        __syncwarp();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_inter += __shfl_xor_sync(0xffffffffu, my_inter, o);
    if (lane == 0 && my_inter) atomicAdd(&p.st->interactions, my_inter);
}

// The kernels.  The 64-wide walks ask for at least 3 resident blocks of the largest
// geometry: the compiler then keeps up to 85 registers per thread and compiles them to
// 63-64 registers without spills (left to itself it compiles the per-body-angle walk to 48,
// with less overlap in the visit loop: 1.6 % slower, the fixed-angle walk 0.7 % slower).
// The other widths keep the compiler's own choice (with the same hint the 32-wide walk ran
// 5-10 % slower).
template <int W, bool REF, bool PB, bool FEAT, bool LIST = false>
__global__ void __launch_bounds__(kForceThreadsMax) force_kernel(StepParams p) {
    force_walk<W, REF, PB, FEAT, LIST>(p);
}
template <bool PB, bool FEAT, bool LIST>
__global__ void __launch_bounds__(kForceThreadsMax, 3) force_kernel64(StepParams p) {
    force_walk<64, false, PB, FEAT, LIST>(p);
}

template <int W, bool REF, bool PB, bool FEAT, bool LIST = false>
static auto force_entry() {
    if constexpr (W == 64 && !REF) return force_kernel64<PB, FEAT, LIST>;
    else return force_kernel<W, REF, PB, FEAT, LIST>;
}

// -------------------------------------------------------------------------------------
template <int W, bool REF, bool PB>
static void launch_force_pf(const StepParams& p, bool feat, int grid, int threads, cudaStream_t s) {
    if constexpr (W >= 32 && !REF) {
        if (p.force_list) {
            const size_t sm = force_list_smem_bytes(threads, p.stack_cap);
            if (feat) force_entry<W, false, PB, true, true>()<<<grid, threads, sm, s>>>(p);
            else force_entry<W, false, PB, false, true>()<<<grid, threads, sm, s>>>(p);
            return;
        }
    }
    const size_t sm = force_smem_bytes<W>(threads, p.stack_cap);
    if (feat) force_entry<W, REF, PB, true>()<<<grid, threads, sm, s>>>(p);
    else force_entry<W, REF, PB, false>()<<<grid, threads, sm, s>>>(p);
}

template <int W, bool REF>
static void launch_force_t(const StepParams& p, bool pb, bool feat, int grid, int threads, cudaStream_t s) {
    if (pb) launch_force_pf<W, REF, true>(p, feat, grid, threads, s);
    else launch_force_pf<W, REF, false>(p, feat, grid, threads, s);
}

// Every variant may be launched with up to the largest geometry's shared memory.
template <int W, bool REF, bool PB, bool FEAT>
static cudaError_t prep_force() {
    return cudaFuncSetAttribute(force_entry<W, REF, PB, FEAT>(), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)force_smem_bytes<W>(kForceThreadsMax, kStackCapMax));
}

template <int W, bool REF>
static cudaError_t prep_force_w() {
    cudaError_t e = cudaSuccess, t;
    if ((t = prep_force<W, REF, false, false>()) != cudaSuccess) e = t;
    if ((t = prep_force<W, REF, false, true>()) != cudaSuccess) e = t;
    if ((t = prep_force<W, REF, true, false>()) != cudaSuccess) e = t;
    if ((t = prep_force<W, REF, true, true>()) != cudaSuccess) e = t;
    return e;
}

template <int W>
static cudaError_t prep_list_w() {
    cudaError_t e = cudaSuccess, t;
    const int sm = (int)force_list_smem_bytes(kForceThreadsMax, kStackCapMax);
    if ((t = cudaFuncSetAttribute(force_entry<W, false, false, false, true>(),
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, sm)) != cudaSuccess)
        e = t;
    if ((t = cudaFuncSetAttribute(force_entry<W, false, false, true, true>(),
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, sm)) != cudaSuccess)
        e = t;
    if ((t = cudaFuncSetAttribute(force_entry<W, false, true, false, true>(),
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, sm)) != cudaSuccess)
        e = t;
    if ((t = cudaFuncSetAttribute(force_entry<W, false, true, true, true>(),
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, sm)) != cudaSuccess)
        e = t;
    return e;
}

int prepare_force_kernels() {
    cudaError_t e = cudaSuccess, t;
    if ((t = prep_list_w<32>()) != cudaSuccess) e = t;
    if ((t = prep_list_w<64>()) != cudaSuccess) e = t;
    if ((t = prep_list_w<128>()) != cudaSuccess) e = t;
    if ((t = prep_force_w<128, false>()) != cudaSuccess) e = t;
    if ((t = prep_force_w<64, false>()) != cudaSuccess) e = t;
    if ((t = prep_force_w<32, false>()) != cudaSuccess) e = t;
    if ((t = prep_force_w<32, true>()) != cudaSuccess) e = t;
    if ((t = prep_force_w<16, false>()) != cudaSuccess) e = t;
    if ((t = prep_force_w<16, true>()) != cudaSuccess) e = t;
    return (int)e;
}

bool force_geometry_valid(int vote, int threads, int cap) {
    const int gl = vote < 32 ? vote : 32;
    return (threads == 64 || threads == 128 || threads == 256) && threads % gl == 0 && cap >= kStackCapMin &&
           cap <= kStackCapMax && cap % 8 == 0;
}

int force_fast_max_depth(int cap) { return fast_max_depth(cap); }

void launch_force(const StepParams& p, int vote, bool ref, bool feat, int grid, int threads, cudaStream_t s) {
    const bool pb = p.theta_body != nullptr;
    if (vote == 128) {
        launch_force_t<128, false>(p, pb, feat, grid, threads, s);  // FMA arithmetic only
    } else if (vote == 64) {
        launch_force_t<64, false>(p, pb, feat, grid, threads, s);   // FMA arithmetic only
    } else if (vote == 16) {
        if (ref) launch_force_t<16, true>(p, pb, feat, grid, threads, s);
        else launch_force_t<16, false>(p, pb, feat, grid, threads, s);
    } else {
        if (ref) launch_force_t<32, true>(p, pb, feat, grid, threads, s);
        else launch_force_t<32, false>(p, pb, feat, grid, threads, s);
    }
}

// Order of the force work items for the next step: longest walks first (longest-
// processing-time first), so the few long walks -- bodies near a dense centre, or small
// per-body angles -- start early instead of running alone at the end of the launch.  A
// counting sort by cost class, descending: four classes per power of two (the two bits
// below the leading one), so that items of one class differ by at most 19 %; within a
// class the order is arbitrary.  One block; warp-aggregated shared-memory atomics.
constexpr int kOrderThreads = 1024;
constexpr int kOrderClasses = 128;
__device__ __forceinline__ int cost_class(int c) {
    c = max(c, 1);
    const int e = 31 - __clz(c);
    const int frac = e >= 2 ? (c >> (e - 2)) & 3 : (c << (2 - e)) & 3;
    return 4 * e + frac;
}
__global__ void __launch_bounds__(kOrderThreads) item_order_kernel(const int* __restrict__ cost, int nitems,
                                                                   int* order) {
    __shared__ int cnt[kOrderClasses], off[kOrderClasses];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    if (threadIdx.x < kOrderClasses) cnt[threadIdx.x] = 0;
    __syncthreads();
    // four items per thread per round: their cost loads are in flight together
    constexpr int kU = 4;
    const int stride = blockDim.x;
    for (int i0 = 0; i0 < nitems; i0 += kU * stride) {
        int c[kU];
#pragma unroll
        for (int k = 0; k < kU; ++k) {
            const int i = i0 + k * stride + threadIdx.x;
            c[k] = i < nitems ? cost[i] : -1;
        }
#pragma unroll
        for (int k = 0; k < kU; ++k) {
            const bool v = c[k] >= 0;
            const int cls = v ? cost_class(c[k]) : -1;
            const unsigned grp = __match_any_sync(0xffffffffu, cls);
            if (v && lane == __ffs(grp) - 1) atomicAdd(&cnt[cls], __popc(grp));
        }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        // first position of each class, largest costs first: lane l holds classes
        // 127 - 4l .. 124 - 4l; a warp scan of the lanes' sums
        static_assert(kOrderClasses == 128, "four classes per lane");
        const int c0 = kOrderClasses - 1 - 4 * lane;
        const int n0 = cnt[c0], n1 = cnt[c0 - 1], n2 = cnt[c0 - 2], n3 = cnt[c0 - 3];
        const int mine = n0 + n1 + n2 + n3;
        int incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int base = incl - mine;
        off[c0] = base;
        off[c0 - 1] = base + n0;
        off[c0 - 2] = base + n0 + n1;
        off[c0 - 3] = base + n0 + n1 + n2;
    }
    __syncthreads();
    for (int i0 = 0; i0 < nitems; i0 += kU * stride) {
        int c[kU];
#pragma unroll
        for (int k = 0; k < kU; ++k) {
            const int i = i0 + k * stride + threadIdx.x;
            c[k] = i < nitems ? cost[i] : -1;
        }
#pragma unroll
        for (int k = 0; k < kU; ++k) {
            const int i = i0 + k * stride + threadIdx.x;
            const bool v = c[k] >= 0;
            const int cls = v ? cost_class(c[k]) : -1;
            const unsigned grp = __match_any_sync(0xffffffffu, cls);
            const int leader = __ffs(grp) - 1;
            int base = 0;
            if (v && lane == leader) base = atomicAdd(&off[cls], __popc(grp));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (v) order[base + __popc(grp & lt)] = i;
        }
    }
}

__global__ void item_order_reset_kernel(int nitems, int* order, int* cost) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += gridDim.x * blockDim.x) {
        order[i] = i;
        cost[i] = 0;
    }
}

void launch_item_order(const int* cost, int nitems, int* order, cudaStream_t s) {
    if (nitems > 0) item_order_kernel<<<1, kOrderThreads, 0, s>>>(cost, nitems, order);
}
void launch_item_order_reset(int nitems, int* order, int* cost, cudaStream_t s) {
    if (nitems > 0) item_order_reset_kernel<<<(nitems + 255) / 256, 256, 0, s>>>(nitems, order, cost);
}

int occupancy_force(int vote, bool ref, int threads, int cap, bool list, int* blocks_per_sm) {
    if (list && !ref && vote >= 32) {
        const size_t sm = force_list_smem_bytes(threads, cap);
        if (vote == 128)
            return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_entry<128, false, false, false, true>(),
                                                                 threads, sm);
        if (vote == 64)
            return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_entry<64, false, false, false, true>(),
                                                                 threads, sm);
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_entry<32, false, false, false, true>(),
                                                             threads, sm);
    }
    if (vote == 128)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_kernel<128, false, false, false>,
                                                             threads, force_smem_bytes<128>(threads, cap));
    if (vote == 64)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_entry<64, false, false, false>(),
                                                             threads, force_smem_bytes<64>(threads, cap));
    if (vote == 16)
        return ref ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_kernel<16, true, false, false>,
                                                                   threads, force_smem_bytes<16>(threads, cap))
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_kernel<16, false, false, false>,
                                                                   threads, force_smem_bytes<16>(threads, cap));
    return ref ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_kernel<32, true, false, false>,
                                                               threads, force_smem_bytes<32>(threads, cap))
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, force_kernel<32, false, false, false>,
                                                               threads, force_smem_bytes<32>(threads, cap));
}

}  // namespace nbh
