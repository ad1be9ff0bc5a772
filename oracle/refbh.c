/*
 * refbh.c — serial CPU restatement of the reference Barnes-Hut step.
 * TEST INFRASTRUCTURE ONLY (the oracle): used by tests/, __graft_entry__.smoke and
 * bench.py's CPU-baseline leg; the product library never links it.
 *
 * Every stage cites the reference kernel it restates (paths relative to the reference
 * project).  Arithmetic follows the kernels operation by operation; MADD(a,b,c) is the
 * a*b+c that -cl-mad-enable lets the OpenCL compiler contract: with fma=1 it is fmaf,
 * with fma=0 a separate multiply and add (this file is compiled with -ffp-contract=off).
 */
#include "refbh.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define NULL_BODY (-1)

static inline float madd(int fma, float a, float b, float c) {
    return fma ? fmaf(a, b, c) : a * b + c;
}

/* GPUBarnesHutNBodySimulation.java:219-227 (calculateNumberOfNodes with maxComputeUnits=16,
 * WARPSIZE=16), generalised by pool_factor (2 reproduces the reference). */
int rb_number_of_nodes(int n, float pool_factor) {
    double want = (double)pool_factor * (double)n;
    long long nn = (long long)ceil(want);
    if (nn < 1024 * 16) nn = 1024 * 16;
    if (nn < (long long)n + 16) nn = (long long)n + 16;
    while (nn & 15) ++nn;
    if (nn > 0x7ffffff0LL) nn = 0x7ffffff0LL;
    return (int)nn;
}

rb_sim* rb_create(int n, int nn, float theta2, float eps2, float dt, float G,
                  int vote, int fma, int precise) {
    if (n < 1 || nn <= n) return NULL;
    rb_sim* s = (rb_sim*)calloc(1, sizeof(rb_sim));
    s->n = n;
    s->nn = nn;
    /* THETA and EPSILON in the reference are theta^2 and eps^2 (calculateforce.cl:13-16). */
    s->theta2 = theta2;
    s->eps2 = eps2;
    s->dt = dt;
    s->G = G;
    s->vote = vote < 1 ? 1 : (vote > RB_MAXVOTE ? RB_MAXVOTE : vote);
    s->fma = fma;
    s->precise = precise;
    size_t nodes = (size_t)nn + 1;
    s->x = (float*)calloc(nodes, sizeof(float));
    s->y = (float*)calloc(nodes, sizeof(float));
    s->z = (float*)calloc(nodes, sizeof(float));
    s->m = (float*)calloc(nodes, sizeof(float));
    s->vx = (float*)calloc(n, sizeof(float));
    s->vy = (float*)calloc(n, sizeof(float));
    s->vz = (float*)calloc(n, sizeof(float));
    s->ax = (float*)calloc(n, sizeof(float));
    s->ay = (float*)calloc(n, sizeof(float));
    s->az = (float*)calloc(n, sizeof(float));
    s->kx = (float*)calloc(n, sizeof(float));
    s->ky = (float*)calloc(n, sizeof(float));
    s->kz = (float*)calloc(n, sizeof(float));
    s->kvx = (float*)calloc(n, sizeof(float));
    s->kvy = (float*)calloc(n, sizeof(float));
    s->kvz = (float*)calloc(n, sizeof(float));
    s->child = (int*)malloc(sizeof(int) * 8 * nodes);
    s->count = (int*)calloc(nodes, sizeof(int));
    s->start = (int*)calloc(nodes, sizeof(int));
    s->sorted = (int*)calloc(n, sizeof(int));
    memset(s->child, 0, sizeof(int) * 8 * nodes);
    /* Initial values of loadBuffers (GPUBarnesHutNBodySimulation.java:167-171). */
    s->step = -1;
    s->maxdepth = 1;
    s->bottom = 0;
    return s;
}

void rb_destroy(rb_sim* s) {
    if (!s) return;
    free(s->x); free(s->y); free(s->z); free(s->m);
    free(s->vx); free(s->vy); free(s->vz);
    free(s->ax); free(s->ay); free(s->az);
    free(s->kx); free(s->ky); free(s->kz);
    free(s->kvx); free(s->kvy); free(s->kvz);
    free(s->theta_body);
    free(s->ebound);
    free(s->child); free(s->count); free(s->start); free(s->sorted);
    free(s);
}

void rb_load(rb_sim* s, const float* x, const float* y, const float* z,
             const float* vx, const float* vy, const float* vz, const float* m) {
    int n = s->n;
    memcpy(s->x, x, sizeof(float) * n);
    memcpy(s->y, y, sizeof(float) * n);
    memcpy(s->z, z, sizeof(float) * n);
    memcpy(s->m, m, sizeof(float) * n);
    if (vx) memcpy(s->vx, vx, sizeof(float) * n); else memset(s->vx, 0, sizeof(float) * n);
    if (vy) memcpy(s->vy, vy, sizeof(float) * n); else memset(s->vy, 0, sizeof(float) * n);
    if (vz) memcpy(s->vz, vz, sizeof(float) * n); else memset(s->vz, 0, sizeof(float) * n);
    memset(s->ax, 0, sizeof(float) * n);
    memset(s->ay, 0, sizeof(float) * n);
    memset(s->az, 0, sizeof(float) * n);
    memset(s->kx, 0, sizeof(float) * n);
    memset(s->ky, 0, sizeof(float) * n);
    memset(s->kz, 0, sizeof(float) * n);
    memset(s->kvx, 0, sizeof(float) * n);
    memset(s->kvy, 0, sizeof(float) * n);
    memset(s->kvz, 0, sizeof(float) * n);
    s->step = -1;
    s->maxdepth = 1;
    s->error = 0;
    s->interactions = 0;
}

void rb_enable_ebound(rb_sim* s, int enable) {
    if (enable && !s->ebound) s->ebound = (float*)calloc(s->n, sizeof(float));
    if (!enable) { free(s->ebound); s->ebound = NULL; }
}

void rb_set_theta_group(rb_sim* s, int on) { s->theta_group = on ? 1 : 0; }

void rb_set_theta_body(rb_sim* s, const float* theta) {
    if (!theta) {
        free(s->theta_body);
        s->theta_body = NULL;
        return;
    }
    if (!s->theta_body) s->theta_body = (float*)malloc(sizeof(float) * s->n);
    memcpy(s->theta_body, theta, sizeof(float) * s->n);
}

/* boundingbox.cl:43-196.  min/max are order independent, so the serial fold equals the
 * reference's tree reduction; the root gets centre 0.5*(min+max), half-width
 * 0.5*max extent, mass -1, start 0, empty children; bottom = NUMBER_OF_NODES; step++. */
int rb_bbox(rb_sim* s) {
    int n = s->n, nn = s->nn;
    float minx = s->x[0], miny = s->y[0], minz = s->z[0];
    float maxx = minx, maxy = miny, maxz = minz;
    for (int i = 0; i < n; ++i) {
        minx = fminf(minx, s->x[i]); maxx = fmaxf(maxx, s->x[i]);
        miny = fminf(miny, s->y[i]); maxy = fmaxf(maxy, s->y[i]);
        minz = fminf(minz, s->z[i]); maxz = fmaxf(maxz, s->z[i]);
    }
    if (s->precise) {
        /* FP64 extent and centre (precise mode has no reference counterpart). */
        double ex = (double)maxx - (double)minx, ey = (double)maxy - (double)miny,
               ez = (double)maxz - (double)minz;
        double e = ex > ey ? ex : ey;
        e = e > ez ? e : ez;
        s->x[nn] = (float)(0.5 * ((double)minx + (double)maxx));
        s->y[nn] = (float)(0.5 * ((double)miny + (double)maxy));
        s->z[nn] = (float)(0.5 * ((double)minz + (double)maxz));
        s->radius = (float)(0.5 * e);
    } else {
        s->x[nn] = 0.5f * (minx + maxx);
        s->y[nn] = 0.5f * (miny + maxy);
        s->z[nn] = 0.5f * (minz + maxz);
        s->radius = 0.5f * fmaxf(fmaxf(maxx - minx, maxy - miny), maxz - minz);
    }
    s->bottom = nn;
    s->m[nn] = -1.0f;
    s->start[nn] = 0;
    for (int k = 0; k < 8; ++k) s->child[8 * nn + k] = NULL_BODY;
    s->step++;
    return RB_OK;
}

static inline int octant(float cx, float cy, float cz, float bx, float by, float bz) {
    int p = 0;
    if (cx < bx) p = 1;
    if (cy < by) p += 2;
    if (cz < bz) p += 4;
    return p;
}

/* buildtree.cl:42-199, one body at a time.  The point-region octree of a point set does
 * not depend on insertion order, so the serial insertion builds the reference's tree (up
 * to cell numbering).  depth counts as in the reference (root level = 1 for a body placed
 * in the root).  A split deeper than RB_MAXDEPTH stops with RB_ERR_DEPTH instead of
 * running the pool dry; the reference reports the same tree as an error later
 * (calculateforce.cl:69-73). */
int rb_build(rb_sim* s) {
    const int n = s->n, nn = s->nn;
    const float radius = s->radius;
    int maxdepth = 1;
    for (int b = 0; b < n; ++b) {
        const float bx = s->x[b], by = s->y[b], bz = s->z[b];
        int node = nn;
        int depth = 1;
        float r = radius;
        int path = octant(s->x[nn], s->y[nn], s->z[nn], bx, by, bz);
        int ch = s->child[8 * node + path];
        while (ch >= n) {                       /* :77-89 descend to the leaf slot */
            node = ch;
            ++depth;
            r *= 0.5f;
            path = octant(s->x[node], s->y[node], s->z[node], bx, by, bz);
            ch = s->child[8 * node + path];
        }
        if (ch == NULL_BODY) {                  /* :98-101 empty slot */
            s->child[8 * node + path] = b;
        } else {                                /* :102-181 split until separated */
            const int old = ch;
            do {
                depth++;
                if (depth > RB_MAXDEPTH) { s->error = RB_ERR_DEPTH; return RB_ERR_DEPTH; }
                const int cell = --s->bottom;
                if (cell <= n) { s->error = RB_ERR_POOL; s->bottom = nn; return RB_ERR_POOL; }
                float ox = (float)(path & 1) * r;
                float oy = (float)((path >> 1) & 1) * r;
                float oz = (float)((path >> 2) & 1) * r;
                r *= 0.5f;
                s->m[cell] = -1.0f;
                s->start[cell] = -1;
                const float cx = s->x[node] - r + ox;
                const float cy = s->y[node] - r + oy;
                const float cz = s->z[node] - r + oz;
                s->x[cell] = cx;
                s->y[cell] = cy;
                s->z[cell] = cz;
                for (int k = 0; k < 8; ++k) s->child[8 * cell + k] = NULL_BODY;
                s->child[8 * node + path] = cell;
                int opath = octant(cx, cy, cz, s->x[old], s->y[old], s->z[old]);
                s->child[8 * cell + opath] = old;
                node = cell;
                path = octant(cx, cy, cz, bx, by, bz);
                ch = s->child[8 * node + path];
            } while (ch >= 0);
            s->child[8 * node + path] = b;
        }
        if (depth > maxdepth) maxdepth = depth;
    }
    if (maxdepth > s->maxdepth) s->maxdepth = maxdepth;   /* atom_max, :199 */
    return RB_OK;
}

/* summarizetree.cl:37-178.  Cells are processed from bottom up to the root; a cell's
 * children always have lower indices, so each child is final when its parent is summed.
 * Used children are moved to the front in octant order (:77-81); mass and mass-weighted
 * position are summed in that order; the centre of mass is centre * (1/mass) (:161-167). */
int rb_summarize(rb_sim* s) {
    const int n = s->n, nn = s->nn, fma = s->fma;
    for (int c = s->bottom; c <= nn; ++c) {
        int* ch8 = s->child + 8 * c;
        int used = 0;
        int cnt = 0;
        if (s->precise && c == nn) {
            /* FP64 root centre of mass (precise mode). */
            double cm = 0, cx = 0, cy = 0, cz = 0;
            for (int k = 0; k < 8; ++k) {
                int ch = ch8[k];
                if (ch < 0) continue;
                if (k != used) { ch8[k] = NULL_BODY; ch8[used] = ch; }
                double mm = s->m[ch];
                cnt += ch >= n ? s->count[ch] : 1;
                cm += mm;
                cx += (double)s->x[ch] * mm;
                cy += (double)s->y[ch] * mm;
                cz += (double)s->z[ch] * mm;
                used++;
            }
            s->count[c] = cnt;
            s->x[c] = (float)(cx / cm);
            s->y[c] = (float)(cy / cm);
            s->z[c] = (float)(cz / cm);
            s->m[c] = (float)cm;
            continue;
        }
        float cm = 0.0f, cx = 0.0f, cy = 0.0f, cz = 0.0f;
        for (int k = 0; k < 8; ++k) {
            int ch = ch8[k];
            if (ch < 0) continue;
            if (k != used) { ch8[k] = NULL_BODY; ch8[used] = ch; }
            float mm = s->m[ch];
            cnt += ch >= n ? s->count[ch] : 1;
            cm += mm;
            cx = madd(fma, s->x[ch], mm, cx);
            cy = madd(fma, s->y[ch], mm, cy);
            cz = madd(fma, s->z[ch], mm, cz);
            used++;
        }
        s->count[c] = cnt;
        float inv = 1.0f / cm;
        s->x[c] = cx * inv;
        s->y[c] = cy * inv;
        s->z[c] = cz * inv;
        s->m[c] = cm;
    }
    return RB_OK;
}

/* sort.cl:24-75.  Cells from the root downward (parents have higher indices); each cell
 * hands consecutive start offsets to its child cells and places its body children at the
 * running offset, giving bodies in depth-first octant order. */
int rb_sort(rb_sim* s) {
    const int n = s->n, nn = s->nn;
    s->start[nn] = 0;
    for (int c = nn; c >= s->bottom; --c) {
        int st = s->start[c];
        for (int k = 0; k < 8; ++k) {
            int ch = s->child[8 * c + k];
            if (ch >= n) {
                s->start[ch] = st;
                st += s->count[ch];
            } else if (ch >= 0) {
                s->sorted[st] = ch;
                ++st;
            }
        }
    }
    return RB_OK;
}

/* Opening threshold of level L (root = 0): dq[L] = r^2/theta^2 * 4^-L + eps^2
 * (calculateforce.cl:52-67; the reference's repeated *0.25 is exact in the normal range,
 * and below it eps^2 absorbs the term). */
static inline float level_threshold(float t0, int L, float eps2) {
    return ldexpf(t0, -2 * L) + eps2;
}

/* calculateforce.cl:52-185.  Vote groups of s->vote consecutive sorted bodies walk the
 * tree together with one stack of (node, next child) per level; a cell child is accepted
 * only if every body of the group has d^2 >= dq[level] (work_group_all, :145), a body
 * child always.  A null child ends the cell (children are compacted).  Then the leapfrog
 * velocity correction for step > 0 (:174-181) and the acceleration store (:183-185). */
int rb_force(rb_sim* s) {
    const int n = s->n, nn = s->nn, W = s->vote, fma = s->fma;
    const float eps2 = s->eps2, dt = s->dt;
    if (s->maxdepth > RB_MAXDEPTH) { s->error = RB_ERR_DEPTH; return RB_ERR_DEPTH; }
    const float rr = s->radius * s->radius;
    const float t0fixed = s->theta2 > 0.0f ? rr / s->theta2 : rr;
    const int ngroups = (n + W - 1) / W;
    long long total = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total)
    for (int g = 0; g < ngroups; ++g) {
        int lo = g * W, hi = lo + W;
        if (hi > n) hi = n;
        const int cnt = hi - lo;
        int bidx[RB_MAXVOTE];
        float px[RB_MAXVOTE], py[RB_MAXVOTE], pz[RB_MAXVOTE], t0[RB_MAXVOTE];
        float ax[RB_MAXVOTE], ay[RB_MAXVOTE], az[RB_MAXVOTE], eb[RB_MAXVOTE];
        int inter[RB_MAXVOTE];
        for (int k = 0; k < cnt; ++k) {
            int b = s->sorted[lo + k];
            bidx[k] = b;
            px[k] = s->x[b]; py[k] = s->y[b]; pz[k] = s->z[b];
            ax[k] = ay[k] = az[k] = eb[k] = 0.0f;
            inter[k] = 0;
            if (s->theta_body) {
                float th = s->theta_body[b];
                float th2 = th * th;
                t0[k] = th2 > 0.0f ? rr / th2 : rr;
            } else {
                t0[k] = t0fixed;
            }
        }
        if (s->theta_body && s->theta_group) {
            /* the group walks with its smallest angle (largest r^2/theta^2) */
            float tm = t0[0];
            for (int k = 1; k < cnt; ++k) tm = t0[k] > tm ? t0[k] : tm;
            for (int k = 0; k < cnt; ++k) t0[k] = tm;
        }
        int snode[RB_MAXDEPTH + 2], snext[RB_MAXDEPTH + 2];
        int depth = 0;
        snode[0] = nn;
        snext[0] = 0;
        while (depth >= 0) {
            int top;
            while ((top = snext[depth]) < 8) {
                int ch = s->child[8 * snode[depth] + top];
                snext[depth] = top + 1;
                if (ch >= 0) {
                    const float cxn = s->x[ch], cyn = s->y[ch], czn = s->z[ch], cmn = s->m[ch];
                    int accept = 1;
                    float dxs[RB_MAXVOTE], dys[RB_MAXVOTE], dzs[RB_MAXVOTE], d2s[RB_MAXVOTE];
                    for (int k = 0; k < cnt; ++k) {
                        float dx = cxn - px[k], dy = cyn - py[k], dz = czn - pz[k];
                        float d2;
                        if (fma) d2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                        else d2 = dx * dx + dy * dy + dz * dz + eps2;
                        dxs[k] = dx; dys[k] = dy; dzs[k] = dz; d2s[k] = d2;
                        if (ch >= n) {
                            float dq = level_threshold(t0[k], depth, eps2);
                            if (!(d2 >= dq)) accept = 0;
                        }
                    }
                    if (ch < n || accept) {
                        /* full width of a child of a level-`depth` cell: r * 2^-depth */
                        const float s2 = ch >= n ? ldexpf(rr, -2 * depth) : 0.0f;
                        for (int k = 0; k < cnt; ++k) {
                            float rd = 1.0f / sqrtf(d2s[k]);
                            float f = cmn * rd * rd * rd;
                            ax[k] = madd(fma, dxs[k], f, ax[k]);
                            ay[k] = madd(fma, dys[k], f, ay[k]);
                            az[k] = madd(fma, dzs[k], f, az[k]);
                            eb[k] += f * rd * s2;
                            inter[k]++;
                        }
                    } else {
                        depth++;
                        snode[depth] = ch;
                        snext[depth] = 0;
                    }
                } else {
                    depth = depth - 1 > 0 ? depth - 1 : 0;
                }
            }
            depth--;
        }
        for (int k = 0; k < cnt; ++k) {
            int b = bidx[k];
            float gx = ax[k], gy = ay[k], gz = az[k];
            if (s->G != 1.0f) { gx *= s->G; gy *= s->G; gz *= s->G; }
            if (s->step > 0) {
                float tx = (gx - s->ax[b]) * dt, ty = (gy - s->ay[b]) * dt, tz = (gz - s->az[b]) * dt;
                if (s->precise) {
                    /* Kahan-compensated velocity correction. */
                    float y1, t1;
                    y1 = tx * 0.5f - s->kvx[b]; t1 = s->vx[b] + y1; s->kvx[b] = (t1 - s->vx[b]) - y1; s->vx[b] = t1;
                    y1 = ty * 0.5f - s->kvy[b]; t1 = s->vy[b] + y1; s->kvy[b] = (t1 - s->vy[b]) - y1; s->vy[b] = t1;
                    y1 = tz * 0.5f - s->kvz[b]; t1 = s->vz[b] + y1; s->kvz[b] = (t1 - s->vz[b]) - y1; s->vz[b] = t1;
                } else {
                    s->vx[b] = madd(fma, tx, 0.5f, s->vx[b]);
                    s->vy[b] = madd(fma, ty, 0.5f, s->vy[b]);
                    s->vz[b] = madd(fma, tz, 0.5f, s->vz[b]);
                }
            }
            s->ax[b] = gx;
            s->ay[b] = gy;
            s->az[b] = gz;
            if (s->ebound) s->ebound[b] = eb[k] * s->G;
            total += inter[k];
        }
    }
    s->interactions = total;
    return RB_OK;
}

/* integrate.cl:27-43: dv = a*dt*0.5; v' = v + dv; x += v'*dt; v = v' + dv.
 * Precise mode: the drift and the full kick a*dt are Kahan-compensated sums. */
int rb_integrate(rb_sim* s) {
    const int n = s->n, fma = s->fma;
    const float dt = s->dt;
    for (int i = 0; i < n; ++i) {
        float dvx = s->ax[i] * dt * 0.5f;
        float dvy = s->ay[i] * dt * 0.5f;
        float dvz = s->az[i] * dt * 0.5f;
        float vx = s->vx[i] + dvx;
        float vy = s->vy[i] + dvy;
        float vz = s->vz[i] + dvz;
        if (s->precise) {
            float y1, t1;
            y1 = vx * dt - s->kx[i]; t1 = s->x[i] + y1; s->kx[i] = (t1 - s->x[i]) - y1; s->x[i] = t1;
            y1 = vy * dt - s->ky[i]; t1 = s->y[i] + y1; s->ky[i] = (t1 - s->y[i]) - y1; s->y[i] = t1;
            y1 = vz * dt - s->kz[i]; t1 = s->z[i] + y1; s->kz[i] = (t1 - s->z[i]) - y1; s->z[i] = t1;
            y1 = s->ax[i] * dt - s->kvx[i]; t1 = s->vx[i] + y1; s->kvx[i] = (t1 - s->vx[i]) - y1; s->vx[i] = t1;
            y1 = s->ay[i] * dt - s->kvy[i]; t1 = s->vy[i] + y1; s->kvy[i] = (t1 - s->vy[i]) - y1; s->vy[i] = t1;
            y1 = s->az[i] * dt - s->kvz[i]; t1 = s->vz[i] + y1; s->kvz[i] = (t1 - s->vz[i]) - y1; s->vz[i] = t1;
        } else {
            s->x[i] = madd(fma, vx, dt, s->x[i]);
            s->y[i] = madd(fma, vy, dt, s->y[i]);
            s->z[i] = madd(fma, vz, dt, s->z[i]);
            s->vx[i] = vx + dvx;
            s->vy[i] = vy + dvy;
            s->vz[i] = vz + dvz;
        }
    }
    return RB_OK;
}

int rb_tree(rb_sim* s) {
    int e;
    if ((e = rb_bbox(s))) return e;
    if ((e = rb_build(s))) return e;
    if ((e = rb_summarize(s))) return e;
    return rb_sort(s);
}

int rb_step(rb_sim* s) {
    int e;
    if ((e = rb_tree(s))) return e;
    if ((e = rb_force(s))) return e;
    return rb_integrate(s);
}

void rb_direct_f64(int n, const float* x, const float* y, const float* z, const float* m,
                   double eps2, double G, int nidx, const int* idx,
                   double* ax, double* ay, double* az) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nidx; ++k) {
        const int i = idx[k];
        const double xi = x[i], yi = y[i], zi = z[i];
        double sx = 0, sy = 0, sz = 0;
        for (int j = 0; j < n; ++j) {
            double dx = (double)x[j] - xi, dy = (double)y[j] - yi, dz = (double)z[j] - zi;
            double d2 = dx * dx + dy * dy + dz * dz + eps2;
            double inv = 1.0 / sqrt(d2);
            double f = (double)m[j] * inv * inv * inv;
            sx += dx * f;
            sy += dy * f;
            sz += dz * f;
        }
        ax[k] = G * sx;
        ay[k] = G * sy;
        az[k] = G * sz;
    }
}
