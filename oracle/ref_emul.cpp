// ref_emul.cpp — host driver for the reference kernels compiled as C++ (ref_kernel_tu.cpp).
// TEST INFRASTRUCTURE ONLY: it plays the part of GPUBarnesHutNBodySimulation's OpenCL
// host (buffer set-up of loadBuffers, GPUBarnesHutNBodySimulation.java:153-181, and the
// six launches of step(), :248-275) so that the oracle can be checked against the
// reference's own code.  Compiled with -DREF_RUNNER so the OpenCL macros stay out.
#define REF_RUNNER 1
#include "ref_shim.hpp"

#include <chrono>
#include <cstdlib>
#include <mutex>
#include <thread>
#include <vector>

thread_local RefItem ref_item;

namespace {

struct GroupSync {
    std::mutex mu;
    int live = 0;
    int arrived = 0;
    int vote_and = 1;
    int result[2] = {1, 1};
    volatile unsigned gen = 0;
};

GroupSync g_groups[NUM_WORK_GROUPS];
std::vector<float> g_last_tree;
std::vector<int> g_last_child, g_last_count;

void release_locked(GroupSync& g) {
    g.result[g.gen & 1u] = g.vote_and;
    g.vote_and = 1;
    g.arrived = 0;
    __atomic_store_n(&g.gen, g.gen + 1, __ATOMIC_SEQ_CST);
}

int arrive(int pred) {
    GroupSync& g = g_groups[ref_item.grp];
    unsigned my;
    {
        std::lock_guard<std::mutex> lk(g.mu);
        my = g.gen;
        g.vote_and &= pred ? 1 : 0;
        if (++g.arrived == g.live) {
            release_locked(g);
            return g.result[my & 1u];
        }
    }
    while (__atomic_load_n(&g.gen, __ATOMIC_SEQ_CST) == my) sched_yield();
    return g.result[my & 1u];
}

void leave() {
    GroupSync& g = g_groups[ref_item.grp];
    std::lock_guard<std::mutex> lk(g.mu);
    g.live--;
    if (g.arrived > 0 && g.arrived == g.live) release_locked(g);
}

typedef void (*ItemFn)(int, const RefArgs*);

void launch(ItemFn fn, const RefArgs* a) {
    for (int g = 0; g < NUM_WORK_GROUPS; ++g) {
        g_groups[g].live = WORKGROUP_SIZE;
        g_groups[g].arrived = 0;
        g_groups[g].vote_and = 1;
    }
    std::vector<std::thread> th;
    th.reserve(NUM_WORK_GROUPS * WORKGROUP_SIZE);
    for (int g = 0; g < NUM_WORK_GROUPS; ++g) {
        for (int l = 0; l < WORKGROUP_SIZE; ++l) {
            th.emplace_back([=] {
                ref_item.lid = l;
                ref_item.grp = g;
                ref_item.gid = g * WORKGROUP_SIZE + l;
                fn(g, a);
                leave();
            });
        }
    }
    for (auto& t : th) t.join();
}

}  // namespace

void ref_group_barrier() { (void)arrive(1); }
int ref_group_all(int pred) { return arrive(pred); }

extern "C" {

int ref_nbodies() { return NBODIES; }
int ref_number_of_nodes() { return NUMBER_OF_NODES; }

// Runs nsteps reference steps from the given initial state.  After step s the body state
// goes to out_*[s*NBODIES ...]; the tree of the last step to out_sorted (NBODIES ints),
// out_info = {maxDepth, bottom, error, step, bodyCount[root]}, out_root = {x,y,z,mass,radius}.
int ref_run(const float* x, const float* y, const float* z, const float* vx, const float* vy,
            const float* vz, const float* m, int nsteps, float* out_x, float* out_y, float* out_z,
            float* out_vx, float* out_vy, float* out_vz, float* out_ax, float* out_ay,
            float* out_az, int* out_sorted, int* out_info, float* out_root) {
    const int n = NBODIES, nn = NUMBER_OF_NODES;
    const size_t nodes = (size_t)nn + 1;
    std::vector<float> px(nodes), py(nodes), pz(nodes), pvx(nodes), pvy(nodes), pvz(nodes),
        pax(nodes), pay(nodes), paz(nodes), pm(nodes);
    std::vector<int> child(8 * nodes), count(nodes), start(nodes), sorted(nodes);
    int step = -1, blockCount = 0, maxDepth = 1, bottom = 0, error = 0;
    float radius = 0.0f;
    for (int i = 0; i < n; ++i) {
        px[i] = x[i]; py[i] = y[i]; pz[i] = z[i];
        pvx[i] = vx ? vx[i] : 0.0f; pvy[i] = vy ? vy[i] : 0.0f; pvz[i] = vz ? vz[i] : 0.0f;
        pm[i] = m[i];
    }
    RefArgs a{px.data(), py.data(), pz.data(), pvx.data(), pvy.data(), pvz.data(),
              pax.data(), pay.data(), paz.data(), &step, &blockCount, count.data(), &radius,
              &maxDepth, &bottom, pm.data(), child.data(), start.data(), sorted.data(), &error};
    const ItemFn kernels[6] = {ref_item_boundingBox, ref_item_buildTree, ref_item_summarizeTree,
                               ref_item_sort, ref_item_calculateForce, ref_item_integrate};
    const bool trace = std::getenv("REF_TRACE") != nullptr;
    for (int s = 0; s < nsteps; ++s) {
        for (int k = 0; k < 6; ++k) {
            auto t0 = std::chrono::steady_clock::now();
            launch(kernels[k], &a);
            if (trace) {
                double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
                std::fprintf(stderr, "ref step %d kernel %d: %.1f ms (bottom %d maxDepth %d error %d)\n", s, k, ms,
                             bottom, maxDepth, error);
            }
            if (error) break;
        }
        if (error) break;
        const size_t o = (size_t)s * n;
        for (int i = 0; i < n; ++i) {
            if (out_x) out_x[o + i] = px[i];
            if (out_y) out_y[o + i] = py[i];
            if (out_z) out_z[o + i] = pz[i];
            if (out_vx) out_vx[o + i] = pvx[i];
            if (out_vy) out_vy[o + i] = pvy[i];
            if (out_vz) out_vz[o + i] = pvz[i];
            if (out_ax) out_ax[o + i] = pax[i];
            if (out_ay) out_ay[o + i] = pay[i];
            if (out_az) out_az[o + i] = paz[i];
        }
    }
    if (out_sorted) for (int i = 0; i < n; ++i) out_sorted[i] = sorted[i];
    if (out_info) {
        out_info[0] = maxDepth;
        out_info[1] = bottom;
        out_info[2] = error;
        out_info[3] = step;
        out_info[4] = count[nn];
    }
    if (out_root) {
        out_root[0] = px[nn];
        out_root[1] = py[nn];
        out_root[2] = pz[nn];
        out_root[3] = pm[nn];
        out_root[4] = radius;
    }
    g_last_tree.assign(px.begin(), px.end());
    g_last_tree.insert(g_last_tree.end(), py.begin(), py.end());
    g_last_tree.insert(g_last_tree.end(), pz.begin(), pz.end());
    g_last_tree.insert(g_last_tree.end(), pm.begin(), pm.end());
    g_last_child = child;
    g_last_count = count;
    return error;
}

// Node x,y,z,mass (4 x (NUMBER_OF_NODES+1) floats), child slots and body counts of the
// last tree built by ref_run.
void ref_last_tree(float* node4, int* child, int* count) {
    if (node4) std::memcpy(node4, g_last_tree.data(), g_last_tree.size() * sizeof(float));
    if (child) std::memcpy(child, g_last_child.data(), g_last_child.size() * sizeof(int));
    if (count) std::memcpy(count, g_last_count.data(), g_last_count.size() * sizeof(int));
}

}  // extern "C"
