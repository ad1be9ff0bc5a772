/*
 * nbh.h — C ABI of the GB300 Barnes-Hut step engine (libnbh.so).
 *
 * This is the drop-in boundary for the reference's per-step pipeline
 * (bounding box -> octree build -> summarize -> sort -> force -> integrate).
 * In the reference that pipeline is driven by the Java class
 * GPUBarnesHutNBodySimulation through JOCL; here a Java FFM/JNI shim or Python
 * ctypes drives it through the plain-C entry points below.  Every entry point
 * takes plain pointers and sizes, returns an int status (0 = ok, negative =
 * one of the NBH_ERR_* codes) and never throws.  One nbh_sim is not
 * thread-safe; different nbh_sim objects may be used from different threads.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   AbstractNBodySimulation.java:16-43          step()/init()/getNumberOfBodies()
 *   GPUBarnesHutNBodySimulation.java:104-151    constructor + init()
 *   GPUBarnesHutNBodySimulation.java:153-181    loadBuffers()   (host -> device)
 *   GPUBarnesHutNBodySimulation.java:219-227    calculateNumberOfNodes()
 *   GPUBarnesHutNBodySimulation.java:229-246    initGLBuffers() (headless here)
 *   GPUBarnesHutNBodySimulation.java:248-275    step() / executeSimulationKernel()
 *   GPUBarnesHutNBodySimulation.java:276-290    error-flag read
 *   GPUBarnesHutNBodySimulation.java:305-365    printEnergy/printDepth/printImpulse
 *   universe/UniverseGenerator.java:22           generate(offset, n, x..m)
 */
#ifndef NBH_H
#define NBH_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBH_ABI_VERSION 1

/* Status codes. */
#define NBH_OK            0
#define NBH_ERR_INVALID  (-1)  /* bad argument (null pointer, n<1, non-finite input, ...) */
#define NBH_ERR_CUDA     (-2)  /* a CUDA runtime call failed; see nbh_last_error_message */
#define NBH_ERR_POOL     (-3)  /* node pool exhausted while splitting cells
                                  (reference: *_error = 1, buildtree.cl:112-119) */
#define NBH_ERR_DEPTH    (-4)  /* tree deeper than NBH_MAXDEPTH levels
                                  (reference: calculateforce.cl:69-73) */
#define NBH_ERR_TIMEOUT  (-5)  /* a bounded device-side wait gave up (no reference
                                  counterpart: the reference spins forever) */
#define NBH_ERR_STATE    (-6)  /* call made in the wrong state (e.g. step before load) */
#define NBH_ERR_NOMEM    (-7)  /* device allocation failed */
#define NBH_ERR_NODEVICE (-8)  /* no CUDA device / wrong architecture */
#define NBH_ERR_MODEL    (-9)  /* learned-theta model missing or malformed */

/* Maximum tree depth (reference MAXDEPTH, calculateforce.cl:12). */
#define NBH_MAXDEPTH 64

/* Arithmetic modes of the step.
 * NBH_ARITH_FMA       fused multiply-add where a*b+c occurs (default, fastest);
 *                     inverse square root by the hardware approximation.
 * NBH_ARITH_REFERENCE separate multiply and add, correctly rounded 1/sqrt:
 *                     the arithmetic the reference kernels perform when the
 *                     OpenCL compiler does not contract (-cl-mad-enable is a
 *                     permission, GPUBarnesHutNBodySimulation.java:210). */
#define NBH_ARITH_FMA       0
#define NBH_ARITH_REFERENCE 1

/* Run-time replacement of the reference's compile-time constants
 * (calculateforce.cl:11-18, integrate.cl:11-12, GPUBarnesHutNBodySimulation.java:44-49,207-227). */
typedef struct nbh_config {
    int32_t abi_version;   /* must be NBH_ABI_VERSION */
    int32_t device;        /* CUDA device ordinal */
    float   theta;         /* opening angle; the reference's THETA macro is theta^2 */
    float   eps;           /* softening length; the reference's EPSILON macro is eps^2 */
    float   theta2;        /* if > 0: theta^2 used verbatim (the reference's THETA, e.g. 1.5);
                              otherwise theta*theta rounded to float */
    float   eps2;          /* if > 0: eps^2 used verbatim (the reference's EPSILON, e.g. 0.0025) */
    float   dt;            /* time step (TIMESTEP) */
    float   G;             /* gravitational constant, multiplies every mass (reference: 1) */
    float   pool_factor;   /* node pool = max(pool_factor*N, 16384) rounded up to 16;
                              the reference uses 2.0 (calculateNumberOfNodes) */
    int32_t vote_width;    /* bodies voting together on opening a cell: 64 (two bodies on
                              each lane of one warp, default; FMA arithmetic), 128 (four per
                              lane; FMA), 32 (one warp) or 16 (the reference work-group,
                              calculateforce.cl:145) */
    int32_t arith;         /* NBH_ARITH_FMA or NBH_ARITH_REFERENCE */
    int32_t precise;       /* 1: Kahan-compensated position/velocity updates and FP64
                              extent / root centre of mass; 0: reference arithmetic */
    int32_t stage_timing;  /* 1: record per-stage CUDA-event times in nbh_stats */
    int32_t use_graph;     /* 1: replay each step as one captured CUDA graph (default) */
    int32_t force_threads; /* force launch geometry: threads per block, 64 / 128 / 256
                              (0: 128); set by nbh_autotune */
    int32_t stack_cap;     /* entries of each vote group's shared-memory stack, 64..256, a
                              multiple of 8 (0: 256); trees deeper than (cap - 8) / 7 + 1
                              levels take the per-level walk; in the list walk (force_list)
                              the cells whose children are pending, and a group that would
                              hold more restarts on the per-level walk */
    int32_t build_phases;  /* octree insertion launches: 1 (one pass), 3 or 5 (0: 5) */
    int32_t build_buckets; /* 1 (or 0, the default): with 5 phases the lock phases insert a
                              1/16 sample of the bodies and every other body joins the
                              subtree of the sample-tree slot it descends to, built by one
                              warp without locks (the same tree); with 3 phases one lock
                              phase inserts 1/256 and two such passes add the rest of the
                              sample, then the other bodies; 2: lock insertion only */
    int32_t top_phase;     /* the first phase of a 3- or 5-phase schedule (one body of every
                              256) may build the top levels of each universe's tree in shared
                              memory and publish them (the same tree), for universes of at
                              most 32766 * 256 bodies: 1 with one block per universe, 3 with
                              eight (one per octant of the root), 2 never (global locks);
                              0 (default): one block up to 512 * 256 bodies per universe,
                              eight up to 8192 * 256, the global locks above (the measured
                              fastest); nbh_autotune times all three where possible */
    int32_t force_list;    /* the whole-warp walks (vote width 32, 64 or 128; FMA arithmetic;
                              fixed or per-body angle): 1 decides each tested child on its own
                              lane (the group's bounding box and its most central body settle
                              most votes) and evaluates the accepted records from a list in
                              shared memory; 2 visits one child at a time with the vote of
                              every body.  The same interactions either way; the sums may
                              differ in the last bits (list order).  0: the default, 1 except
                              in precise mode, which keeps the reference's order of
                              accumulation */
    int32_t reserved[2];
} nbh_config;

/* Fills *cfg with the defaults: theta 0.5, eps 0.05, dt 0.025, G 1, pool 2.0,
 * vote 64, FMA arithmetic, precise 0, stage timing 0, graph 1. */
void nbh_config_default(nbh_config* cfg);

typedef struct nbh_stats {
    int64_t steps;             /* steps taken since the last load */
    int64_t interactions;      /* accepted body-node force evaluations in the last step
                                  (executions of calculateforce.cl:146-151) */
    int32_t max_depth;         /* deepest level of the last tree (reference _maxDepth) */
    int32_t cells;             /* cells allocated in the last tree, all universes */
    int32_t nuniverses;
    int32_t nbodies;           /* total over universes */
    int32_t pool_nodes;        /* NUMBER_OF_NODES of the shared pool */
    int32_t status;            /* device status word of the last step (NBH_OK or NBH_ERR_*) */
    int32_t lock_waits;        /* build of the last step: descents that found their slot locked */
    int32_t cas_misses;        /* build of the last step: lock attempts that lost the race */
    /* per-stage device milliseconds of the last step (stage_timing = 1 only) */
    float   ms_bbox, ms_build, ms_summarize, ms_sort, ms_force, ms_integrate, ms_step;
    float   ms_theta;          /* learned opening angle: features + MLP inference of the last
                                  step (0 without a model; stage_timing = 1 only) */
    float   reserved[7];
} nbh_stats;

typedef struct nbh_sim nbh_sim;

/* Constructor (GPUBarnesHutNBodySimulation.java:104-108 + the device part of init :110-131). */
int nbh_create(const nbh_config* cfg, nbh_sim** out);
int nbh_destroy(nbh_sim* sim);

/* Copies one universe of n bodies (SoA host arrays, like UniverseGenerator.generate's
 * outputs) to the device and resets the step counter to -1 and max depth to 1, as
 * loadBuffers does (GPUBarnesHutNBodySimulation.java:153-181).  Any pointer among
 * vx, vy, vz may be NULL (zero velocity). */
int nbh_load(nbh_sim* sim, int32_t n,
             const float* x, const float* y, const float* z,
             const float* vx, const float* vy, const float* vz,
             const float* m);

/* Batched ensemble: nuniv independent universes, universe u holding counts[u] bodies,
 * stored back to back in the SoA arrays.  Every step advances all of them. */
int nbh_load_batch(nbh_sim* sim, int32_t nuniv, const int32_t* counts,
                   const float* x, const float* y, const float* z,
                   const float* vx, const float* vy, const float* vz,
                   const float* m);

/* Runs nsteps full steps (BB -> build -> summarize -> sort -> force -> integrate) and
 * waits for them, like step() (GPUBarnesHutNBodySimulation.java:248-271).  Returns the
 * device status word (NBH_ERR_POOL / NBH_ERR_DEPTH / NBH_ERR_TIMEOUT) if a stage failed;
 * stages after a failed one do nothing. */
int nbh_step(nbh_sim* sim, int32_t nsteps);

/* Enqueues nsteps steps on the sim's stream without waiting (no status check). */
int nbh_step_async(nbh_sim* sim, int32_t nsteps);
int nbh_synchronize(nbh_sim* sim);

/* Reads the body state back (bodies in load order).  Any pointer may be NULL. */
int nbh_read(nbh_sim* sim, float* x, float* y, float* z,
             float* vx, float* vy, float* vz,
             float* ax, float* ay, float* az);

/* Overwrites positions, velocities and (optionally) accelerations without resetting the
 * step counter: resume from a checkpoint, or a host that owns the arrays between steps.
 * NULL pointers leave that component unchanged. */
int nbh_write(nbh_sim* sim, const float* x, const float* y, const float* z,
              const float* vx, const float* vy, const float* vz,
              const float* ax, const float* ay, const float* az);

/* The nine host arrays of nbh_write / nbh_read (n floats each; NULL: not copied). */
typedef struct nbh_host_state {
    float *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az;
} nbh_host_state;

/* For a host that owns the state between steps: writes `in` like nbh_write (in may be
 * NULL), runs nsteps steps like nbh_step, reads the state into `out` like nbh_read (out
 * may be NULL), and waits once at the end instead of after each of the three calls.
 * Pinned (mapped) arrays are read and written in place by the packing kernels; with pinned
 * input, velocities and accelerations are copied in on a second stream while the first
 * step builds its tree from the positions.  Results equal nbh_write + nbh_step + nbh_read.
 * Returns what nbh_step would. */
int nbh_step_io(nbh_sim* sim, int32_t nsteps, const nbh_host_state* in, const nbh_host_state* out);

int nbh_get_stats(nbh_sim* sim, nbh_stats* out);
int32_t nbh_get_number_of_bodies(nbh_sim* sim);   /* getNumberOfBodies(), :376-379 */

/* Headless stand-in for initGLBuffers + copyVertices (copyvertices.cl:8-17): writes
 * float4 (x,y,z,1) and (vx,vy,vz,1) for every body into caller-owned DEVICE buffers of
 * 4*N floats each (either may be NULL). */
int nbh_export_float4(nbh_sim* sim, float* dev_pos4, float* dev_vel4);

/* The CUDA stream (cudaStream_t) every kernel of this sim runs on, for callers that record
 * CUDA events around steps or order their own work after them. */
void* nbh_get_stream(nbh_sim* sim);

/* Measured FP32 fused-multiply-add throughput of the device (TFLOP/s, 2 flops per FMA):
 * a register-resident FMA loop over every SM, timed with CUDA events.  This is the
 * roofline denominator of the force traversal, which runs on the FP32 pipes. */
int nbh_measure_fp32_peak(int32_t device, double* tflops);

/* Failure-detection self-test: one device thread waits, with the same bounded wait the build
 * uses, on a flag that nothing changes; it must give up after limit_ns and leave
 * NBH_ERR_TIMEOUT in *status, with the context still usable. */
int nbh_selftest_wait(int32_t device, int64_t limit_ns, int32_t* status);

/* Last error text of this sim (or of the last failed nbh_create when sim is NULL). */
const char* nbh_last_error_message(nbh_sim* sim);
int nbh_last_error(nbh_sim* sim);

/* Reference pool sizing (calculateNumberOfNodes, GPUBarnesHutNBodySimulation.java:219-227),
 * generalised by pool_factor (2.0 reproduces the reference). */
int32_t nbh_number_of_nodes(int32_t n, float pool_factor);

/* ---- Tree inspection (tests and diagnostics) ------------------------------------ */

/* Copies the last tree.  Cells are node indices (N, pool_nodes]; cell c's eight child slots
 * are child[8*(c-N) .. 8*(c-N)+7] (int32[8*(pool_nodes+1-N)]), its body count and first
 * depth-first position count[c-N] and start[c-N] (int32[pool_nodes+1-N] each).  node4 gets
 * x,y,z,mass of every node (bodies, then cell centres of mass) as float[4*(pool_nodes+1)];
 * sorted the depth-first body order int32[N]; roots the root node of each universe
 * (pool_nodes - u) and radius its half-width; bottom the lowest allocated cell.
 * Any pointer may be NULL. */
int nbh_read_tree(nbh_sim* sim, int32_t* child, float* node4, int32_t* count,
                  int32_t* start, int32_t* sorted, int32_t* roots, float* radius,
                  int32_t* bottom);

/* FP64 direct-sum accelerations of the bodies listed in idx (body indices in load order),
 * each over all bodies of its own universe, with the sim's softening and G:
 * a_i = G sum_j m_j d_ij / (|d_ij|^2 + eps^2)^(3/2).  Output arrays hold nidx doubles each.
 * This is the error yardstick of every force result (median / p99 relative error). */
int nbh_direct_f64(nbh_sim* sim, int32_t nidx, const int32_t* idx,
                   double* ax, double* ay, double* az);

/* Diagnostics of each universe (GPUBarnesHutNBodySimulation.java:305-365: printEnergy,
 * printDepth, printImpulse), reduced on the GPU in FP64 from the current state, in a fixed
 * order.  Energies and momenta use the state as stored: after a step, positions and
 * velocities at the end of that step. */
#define NBH_DIAG_POTENTIAL 1   /* also the O(N^2) pair potential (0.8 s at 1M bodies on GB300) */
typedef struct nbh_diag {
    double mass;                   /* sum m */
    double com[3];                 /* sum m x / sum m */
    double momentum[3];            /* sum m v (printImpulse, :347-365) */
    double angular_momentum[3];    /* sum m x cross v, about the origin */
    double kinetic;                /* sum m |v|^2 / 2 (:318-324) */
    double potential;              /* -G sum_{i<j} m_i m_j / sqrt(r^2 + eps^2): the potential of
                                      the softened force the step integrates */
    double potential_unsoftened;   /* -G sum_{i<j} m_i m_j / r: the form of :326-335, where each
                                      pair is added twice (`2 * e`, :334); here once */
    int32_t max_depth;             /* printDepth (:341-345): the sim's tree depth, all universes */
    int32_t has_potential;         /* 1 when the potentials were computed */
} nbh_diag;
/* Fills out[0 .. min(nout, universes)) and returns the number filled (>= 0) or an error. */
int nbh_diagnostics(nbh_sim* sim, int32_t flags, nbh_diag* out, int32_t nout);

/* Autotuner of the launch geometry (no counterpart in the reference, whose work-group sizes
 * and stack depth are compile-time constants, calculateforce.cl:11-18 and the host's 16 x 16
 * geometry).  On the loaded universes at their current positions it times every force
 * geometry (threads per block 64 / 128 / 256 x stack capacities from the smallest the tree's
 * depth allows, with 2 levels of headroom, to 256) as side-effect-free force launches that
 * write a scratch buffer, and the tree stages with 1, 3 and 5 lock insertion phases and with
 * 3 and 5 phases completed by bucketed subtrees (build_buckets), then keeps the fastest of
 * each for later steps.  Neither choice changes any result: the walk order, the arithmetic
 * and the tree are the same for every geometry.  With NBH_TUNE_VOTE (FMA arithmetic only)
 * it also times vote widths 16, 32, 64 and 128 -- bodies per traversal group: half a warp,
 * or one warp with one, two or four bodies per lane -- and keeps the fastest; that choice changes the interaction set (a
 * larger group opens a few more cells), so it is off unless asked for.  Body state and the
 * step counter are left as they were. */
#define NBH_TUNE_VOTE 1
#define NBH_TUNE_MAX_TRIALS 64
typedef struct nbh_tune {
    int32_t force_threads;         /* chosen */
    int32_t stack_cap;             /* chosen */
    int32_t build_phases;          /* chosen */
    int32_t build_buckets;         /* chosen: 1 bucketed completion, 2 lock insertion only */
    int32_t vote_width;            /* chosen (the sim's own unless NBH_TUNE_VOTE) */
    int32_t max_depth;             /* tree depth the stack capacities were fitted to */
    float   ms_force;              /* force launch of the choice */
    float   ms_force_before;       /* force launch of the geometry in place before (median
                                      of the same alternating runs as ms_force) */
    float   ms_tree;               /* tree stages of the choice */
    float   ms_tree_before;        /* tree stages of the phases in place before (likewise) */
    int32_t trials;                /* entries used below */
    int32_t trial_kind[NBH_TUNE_MAX_TRIALS];    /* 0 force, 1 tree */
    int32_t trial_a[NBH_TUNE_MAX_TRIALS];       /* threads, or insertion phases */
    int32_t trial_b[NBH_TUNE_MAX_TRIALS];       /* stack capacity (force), or bucketed (tree) */
    int32_t trial_vote[NBH_TUNE_MAX_TRIALS];    /* vote width (force); blocks per universe of
                                                   the shared-memory first phase, 0 for the
                                                   global locks (tree) */
    float   trial_ms[NBH_TUNE_MAX_TRIALS];      /* mean of 3 timed launches after 1 warm-up */
    int32_t top_phase;             /* chosen first phase, as nbh_config.top_phase: 1 or 3
                                      shared memory (one or eight blocks per universe), 2 global */
} nbh_tune;
int nbh_autotune(nbh_sim* sim, int32_t flags, nbh_tune* out);

/* ---- Learned per-body opening angle (no counterpart in the reference) ---------------- */

/* Installs an MLP 12->64->64->1 (ReLU; row-major FP32 parameters W1[64][12], b1[64],
 * W2[64][64], b2[64], W3[64], b3: NBH_MLP_PARAMS floats) and the normalisation of its 12
 * features (mean[12], inv_std[12]).  Every step (or every k-th, nbh_set_theta_interval)
 * then sets each body's opening angle to clamp(exp(MLP((f - mean) * inv_std)), theta_min,
 * theta_max), evaluated with BF16 weights on the tensor cores, and the force walk before
 * it records each body's quadrupole error bound for the features.  The first step after switching on walks with the fixed
 * theta.  enable = 0 returns to the fixed theta.  Features (nbh_theta_features order):
 * log10|a|, log10(bound/|a|), log10(theta of the last walk), log10(d/R), log10(n_leaf+1),
 * level(leaf)/20, log10(n_leaf_parent+1), log10(n_leaf/h^3), log10(m_leaf/M),
 * log10(|a| d^2/M), log10(eps/h), log10(h/d); d = distance to the universe's centre of
 * mass, R, M = root half-width and mass, h = half-width of the cell holding the body. */
#define NBH_MLP_PARAMS 5057
#define NBH_MLP_FEATURES 12
int nbh_set_theta_model(nbh_sim* sim, const float* params, int32_t nparams,
                        const float* feat_mean, const float* feat_inv_std,
                        float theta_min, float theta_max, int32_t enable);

/* Evaluate the opening-angle model every `every` steps (1 <= every <= 2^20; default 1).
 * The walk of the step before each evaluation records the error bounds the features
 * need; the walks in between keep each body's angle and record nothing, so they run at
 * the cost of a plain per-body-angle walk.  May be called before or after
 * nbh_set_theta_model.  No counterpart in the reference (its opening angle is the
 * compile-time THETA, calculateforce.cl:14). */
int nbh_set_theta_interval(nbh_sim* sim, int32_t every);

/* How a vote group uses its bodies' angles: 0 (default) every body tests a cell with its
 * own angle and the group opens it unless all accept; 1 the group walks with the
 * smallest angle among its bodies (a fixed-angle walk per group).  Applies to the
 * learned angle and to nbh_force_probe.  No counterpart in the reference. */
int nbh_set_theta_grouping(nbh_sim* sim, int32_t group_min);

/* Writes the per-body opening angle of the last step into theta[N] (host). */
int nbh_read_theta(nbh_sim* sim, float* theta);

/* One force evaluation at the current positions (the tree is rebuilt; positions,
 * velocities, accelerations and the step counter are left unchanged) with a per-body theta
 * (host array, N floats; NULL = the configured fixed theta).  Writes accelerations, the
 * per-body quadrupole error bound and the interaction count.  Training data come from this. */
int nbh_force_probe(nbh_sim* sim, const float* theta_body,
                    float* ax, float* ay, float* az, float* ebound, int64_t* interactions);

/* Raw (unnormalised) features of every body, feat[N*12] (host).  use_probe = 1 takes the
 * "previous walk" inputs from the last nbh_force_probe; 0 from the last step (the tree is
 * rebuilt for the current positions). */
int nbh_theta_features(nbh_sim* sim, float* feat, int32_t use_probe);

/* Training of the model on the device with FP32 forward/backward kernels: samples X[n*12]
 * (normalised features, row-major), targets T[n] (log theta), pinball loss at `quantile`
 * (the fraction of samples whose target the prediction may exceed).  nbh_mlp_train runs
 * `iters` full-batch Adam steps from params (updated in place), the rate `lr` falling
 * linearly to zero over the last 30 % of them, and reports the final loss;
 * nbh_mlp_grad returns the gradient and loss of one pass; nbh_mlp_forward the outputs. */
int nbh_mlp_train(int32_t device, float* params, const float* X, const float* T, int32_t n,
                  float quantile, int32_t iters, float lr, float* loss);
int nbh_mlp_grad(int32_t device, const float* params, const float* X, const float* T, int32_t n,
                 float quantile, float* grad, float* loss);
int nbh_mlp_forward(int32_t device, const float* params, const float* X, int32_t n, float* y);

/* Same FP64 direct sum as nbh_direct_f64, for callers that cannot allocate device memory
 * while they run (an application whose device memory is handed out up front by its own pool
 * or budget, or a time-critical loop in which cudaMalloc/cudaFree would synchronise the
 * device).  It makes no device or host allocation: its scratch (the index list and three
 * FP64 accumulator columns) is a fixed array inside the library, holding at most
 * NBH_DIRECT_STATIC_MAX bodies per call; larger lists are rejected with NBH_ERR_INVALID.
 * That array is reserved on every GPU that loads the library until the process exits.  The
 * first call on a device looks the array's device address up (cudaGetSymbolAddress, with the
 * sim's device current), so make that first call before any stream capture.  The address is
 * kept for the life of the process: the library never resets a device, and a host
 * application that calls cudaDeviceReset must not call this entry point afterwards.  All
 * calls share the array: it is cleared at the start of every call, and calls that overlap on
 * the GPU (two sims on different streams at the same time) race on it.  No counterpart in the
 * reference. */
#define NBH_DIRECT_STATIC_MAX 65536
int nbh_direct_f64_static(nbh_sim* sim, int32_t nidx, const int32_t* idx,
                          double* ax, double* ay, double* az);

/* ---- Seeded universe generators (UniverseGenerator implementations) ------------------ */
/* All fill caller arrays of n floats at offset `offset`, deterministic in `seed`.
 * Velocity pointers may be NULL where a generator leaves velocities unset. */

/* Uniform in the ball of radius `radius`, Gaussian velocities of standard deviation
 * vsigma, masses 1/n. */
int nbh_generate_uniform_ball(uint64_t seed, int32_t offset, int32_t n, float radius, float vsigma,
                              float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m);
/* Plummer sphere, scale radius a, total mass M, velocities from the distribution function
 * (PlummerUniverseGenerator.java:6-43 without the 3*pi/16 rescale). */
int nbh_generate_plummer(uint64_t seed, int32_t offset, int32_t n, float a, float M,
                         float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m);
/* Exponential disc (scale length rd, scale height zd) with near-circular velocities, a
 * central point mass mc (body `offset`) and a Plummer halo holding halo_frac of the
 * particles, total mass 1 + mc. */
int nbh_generate_disc(uint64_t seed, int32_t offset, int32_t n, float rd, float zd, float mc,
                      float halo_frac,
                      float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m);
/* RandomCubicUniverseGenerator.java:12-18: positions uniform in [-range/2, range/2)^3,
 * masses 1/n, velocities untouched. */
int nbh_generate_random_cube(uint64_t seed, int32_t offset, int32_t n, float range,
                             float* x, float* y, float* z, float* m);
/* SphericalUniverseGenerator.java:6-20: uniform on the unit sphere, masses 1/n. */
int nbh_generate_sphere_surface(uint64_t seed, int32_t offset, int32_t n,
                                float* x, float* y, float* z, float* m);
/* MonteCarloSphericalUniverseGenerator.java:6-27: Fibonacci sphere with a seeded phase. */
int nbh_generate_fibonacci_sphere(uint64_t seed, int32_t offset, int32_t n,
                                  float* x, float* y, float* z, float* m);
/* LonLatSphericalUniverseGenerator.java:9-29: radius 5 lon/lat sphere, masses 1/n. */
int nbh_generate_lonlat_sphere(uint64_t seed, int32_t offset, int32_t n,
                               float* x, float* y, float* z, float* m);
/* RotatingDiskGalaxyGenerator.java:17-43: flat disc of radius r, centre mass at index
 * offset, orbital speeds scaled by vmul. */
int nbh_generate_rotating_disk(uint64_t seed, int32_t offset, int32_t n, float r, float vmul,
                               float center_mass,
                               float* x, float* y, float* z, float* vx, float* vy, float* vz,
                               float* m);

/* ---- .universe files (universe/serialize/*.java) ---------------------------------- */
/* Java-serialisation stream: writeInt(n) then seven float[] objects x,y,z,vx,vy,vz,m
 * (UniverseSerializer.java:25-34, SerializedUniverseGenerator.java:21-37).
 * nbh_universe_read with x == NULL only reports *n. */
int nbh_universe_read(const char* path, int32_t* n, float* x, float* y, float* z,
                      float* vx, float* vy, float* vz, float* m);
int nbh_universe_write(const char* path, int32_t n, const float* x, const float* y,
                       const float* z, const float* vx, const float* vy, const float* vz,
                       const float* m);

#ifdef __cplusplus
}
#endif
#endif /* NBH_H */
