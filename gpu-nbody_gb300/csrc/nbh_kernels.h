// nbh_kernels.h — host-side launchers of the step kernels (nbh_tree.cu, nbh_force.cu).
#pragma once
#include <cuda_runtime.h>

namespace nbh {

struct StepParams;

void launch_bbox(const StepParams& p, int grid, cudaStream_t s);
// 1, 3 or 5 lock insertion phases; with `buckets` the lock phases (5: three of them; 3: one,
// of 1/256) insert the sample and the rest is built as lock-free subtrees, one per slot of
// the tree so far (3: two such passes, the first completing the 1/16 sample)
// top > 0: the first phase of a multi-phase schedule builds in shared memory, `split` (1 or
// 8) blocks per universe holding `top` cells each (for universes of at most
// top_build_max_samples() chunks; top_build_cells() sizes it); 0: through the global locks
void launch_build(const StepParams& p, int phases, bool buckets, int sms, int top, int split, cudaStream_t s);
int top_build_max_samples();
int top_build_cells(int max_chunks);
cudaError_t prepare_tree_kernels();   // raises the dynamic shared-memory limit of the top builder
size_t bucket_stack_bytes(int sms);   // global task stacks of the bucketed build's grid
void launch_link(const StepParams& p, int grid, cudaStream_t s);
void launch_summarize(const StepParams& p, bool ref, int grid, cudaStream_t s);
void launch_sort(const StepParams& p, int grid, cudaStream_t s);
void launch_force(const StepParams& p, int vote, bool ref, bool feat, int grid, int threads, cudaStream_t s);
bool force_geometry_valid(int vote, int threads, int cap);
// Work-item order of the force launches: longest walks first, from the last launch's costs.
void launch_item_order(const int* cost, int nitems, int* order, cudaStream_t s);
void launch_item_order_reset(int nitems, int* order, int* cost, cudaStream_t s);
int force_fast_max_depth(int cap);   // deepest tree the stack of `cap` entries walks without the per-level walk
void launch_integrate(const StepParams& p, bool ref, int grid, cudaStream_t s);

void launch_pack(int n, const float* soa, int mask, float4* node4, float4* vel, float4* acc, int grid,
                 cudaStream_t s);
void launch_unpack(int n, float* soa, const float4* node4, const float4* vel, const float4* acc, int grid,
                   cudaStream_t s);
// Device views of the caller's pinned host arrays (x y z vx vy vz ax ay az; null = absent).
struct HostArrays {
    const float* p[9];
};
void launch_pack_host(int n, const HostArrays& h, int mask, float4* node4, float4* vel, float4* acc, int grid,
                      cudaStream_t s);
void launch_unpack_host(int n, const HostArrays& h, const float4* node4, const float4* vel, const float4* acc,
                        int grid, cudaStream_t s);
void launch_export4(int n, const float4* node4, const float4* vel, float4* pos4, float4* vel4, int grid,
                    cudaStream_t s);
void launch_direct_f64(const float4* node4, int nidx, const int* idx, const int2* range, double eps2, double G,
                       double* out, int ysplit, cudaStream_t s);

// Diagnostics rows (nbh_diag.cu): 0 mass, 1-3 m x, 4-6 m v, 7-9 m x cross v, 10 kinetic
// energy, 11 / 12 sum_i m_i phi_i softened / unsoftened (each pair twice).
constexpr int kDiagMoments = 11;
constexpr int kDiagFields = 13;
void launch_diagnostics(const float4* node4, const float4* vel, const int4* chunks, int nchunks, const int* ubody,
                        int nuniv, bool potential, float eps2, double* part, double* out, cudaStream_t s);

struct DevState;
void launch_wait_selftest(const int* flag, unsigned long long limit_ns, DevState* st, cudaStream_t s);
void launch_fma_peak(float* sink, int iters, int grid, int block, cudaStream_t s);

int occupancy_sort(int* blocks_per_sm);
int occupancy_force(int vote, bool ref, int threads, int cap, bool list, int* blocks_per_sm);
int prepare_force_kernels();   // raises the dynamic shared-memory limit of the force kernels

}  // namespace nbh
