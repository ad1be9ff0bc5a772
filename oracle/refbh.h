/*
 * refbh — CPU restatement of the reference Barnes-Hut step, used ONLY as a test
 * oracle (pytest, __graft_entry__.smoke and bench.py's CPU-baseline leg).  Nothing in
 * the product library links or calls it.
 *
 * It restates the six OpenCL kernels of the reference (kernels/nbody/*.cl) as serial
 * C with the same data layout and arithmetic: bodies at node indices [0, n), cells
 * allocated downward from NUMBER_OF_NODES (the root), child slots child[8*node+octant],
 * octant bit k set when the cell centre is below the body on axis k.  The force pass is
 * OpenMP-parallel over vote groups; every other stage is serial, so results are
 * deterministic.  Parity is pinned against the reference kernels compiled as C++
 * (oracle/ref_emul.cpp) and against the golden fixtures in tests/golden.
 */
#ifndef REFBH_H
#define REFBH_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RB_MAXDEPTH 64
#define RB_MAXVOTE 128              /* largest vote group */
#define RB_OK 0
#define RB_ERR_INVALID (-1)
#define RB_ERR_POOL (-3)
#define RB_ERR_DEPTH (-4)

typedef struct rb_sim {
    int n, nn;                      /* bodies, NUMBER_OF_NODES */
    float theta2, eps2, dt, G;
    int vote, fma, precise;
    float *x, *y, *z, *m;           /* [nn+1] node centre / centre of mass and mass */
    float *vx, *vy, *vz, *ax, *ay, *az;   /* [n] */
    float *kx, *ky, *kz, *kvx, *kvy, *kvz; /* [n] Kahan compensation (precise mode) */
    float *theta_body;              /* [n] optional per-body theta (NULL: fixed) */
    float *ebound;                  /* [n] optional: sum over accepted cells of m s^2 / d^4 */
    int *child;                     /* [8*(nn+1)] */
    int *count, *start;             /* [nn+1] */
    int *sorted;                    /* [n] */
    float radius;
    int bottom, maxdepth, step, error;
    long long interactions;
    int theta_group;                /* per-body theta: 1 = each vote group walks with the
                                       smallest angle of its bodies */
} rb_sim;

int rb_number_of_nodes(int n, float pool_factor);
/* theta2 and eps2 are the squares (the reference's THETA and EPSILON macros). */
rb_sim* rb_create(int n, int nn, float theta2, float eps2, float dt, float G,
                  int vote, int fma, int precise);
void rb_destroy(rb_sim* s);
void rb_load(rb_sim* s, const float* x, const float* y, const float* z,
             const float* vx, const float* vy, const float* vz, const float* m);
void rb_set_theta_body(rb_sim* s, const float* theta);   /* NULL: fixed theta */
void rb_enable_ebound(rb_sim* s, int enable);   /* accumulate the quadrupole error bound */
void rb_set_theta_group(rb_sim* s, int on);     /* per-body theta, group-uniform (smallest) */

int rb_bbox(rb_sim* s);
int rb_build(rb_sim* s);
int rb_summarize(rb_sim* s);
int rb_sort(rb_sim* s);
int rb_force(rb_sim* s);
int rb_integrate(rb_sim* s);
int rb_step(rb_sim* s);          /* all six, stops at the first error */
int rb_tree(rb_sim* s);          /* bbox + build + summarize + sort */

/* FP64 direct summation a_i = G sum_j m_j d / (|d|^2 + eps2)^(3/2) for the listed bodies. */
void rb_direct_f64(int n, const float* x, const float* y, const float* z, const float* m,
                   double eps2, double G, int nidx, const int* idx,
                   double* ax, double* ay, double* az);

#ifdef __cplusplus
}
#endif
#endif
