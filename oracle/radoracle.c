/*
 * radoracle.c -- CPU restatement of hw-radiosity's progressive-refinement
 * shooting loop, used as the parity ORACLE.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg run this program, and only as the checker.  The
 * product (hw-radiosity_gb300/) never links or calls it.
 *
 * It restates, function by function, the reference's algorithm
 * (morris821028/hw-radiosity, shipped configuration of include/config.h:5-13:
 * ADAPT, ROLLBACK, DONT_PARTITION, PRE_PARTITION, PARALLEL):
 *   - scene input            src/rad.cpp:47-111      (read_scene)
 *   - octree build           src/raycast.cpp:24-233  (clip2d, crosses_cube, build_node)
 *   - visibility walk        src/raycast.cpp:235-360 (next_point, cell_of, tri_hit, cell_hit, ray_hit)
 *   - form factors           src/shade.cpp:76-168    (split_source, point_ff, adapt_ff)
 *   - energy deposit         src/shade.cpp:244-259   (deposit)
 *   - initialisation         src/rad.cpp:259-356     (init_radiosity)
 *   - pre-partition          src/shade.cpp:11-43, 171-211, 311-431, 556-598
 *   - shooter selection      src/rad.cpp:387-404     (select_shooters)
 *   - one shooting step      src/rad.cpp:406-451     (shoot_step)
 *   - output .fin            src/rad.cpp:117-242 and include/float2string.h (write_fin)
 * with every arithmetic step at the reference's own precision: FP32 values, the
 * FP64 promotions the reference's double literals and casts cause, and
 * -ffp-contract=off so no multiply-add is fused.  Built with
 * -DORACLE_REAL=double it is the FP64 restatement (every float -> double), the
 * counterpart of the reference's float->double build.
 *
 * Pinned against the reference binary built from the reference's own sources
 * (oracle/stage_ref.py + oracle/Makefile) by tests/test_oracle_pin.py, and
 * against committed fixtures from that binary (tests/golden/).
 *
 * Usage: radoracle [reference options] input -o prefix
 * Environment: RAD_DUMP, RAD_TRACE, RAD_MAX_STEPS as for oracle/ref_hooks.cpp.
 * The receiver loop runs in index order on one thread; each receiver's result
 * depends only on shooter state that is fixed during a step, so the result is
 * the same as the reference's OpenMP loop.
 */
#define _POSIX_C_SOURCE 199309L
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifndef ORACLE_REAL
#define ORACLE_REAL float
#endif
typedef ORACLE_REAL real;
typedef real vec3[3];

#define PI_D 3.1415926535897932
#define MAX_LEVEL 6
#define MAX_TRI_PER_NODE 10
#define MAX_TRI_POOL 1000000

/* ---------------------------------------------------------------- scalars */
static inline real r_sqrt(real x) { return (real)sqrt((double)x); } /* sqrt is correctly rounded either way */
static inline real dot3(const real *a, const real *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline real len3(const real *a) { return r_sqrt(dot3(a, a)); }
static inline void sub3(const real *from, const real *to, real *out) {
    out[0] = to[0] - from[0]; out[1] = to[1] - from[1]; out[2] = to[2] - from[2];
}
static inline void cross3(const real *a, const real *b, real *o) {
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}
static inline real rmin(real a, real b) { return (b < a) ? b : a; } /* std::min */
static inline real rmax(real a, real b) { return (a < b) ? b : a; } /* std::max */
/* centre: float sum of the three coordinates divided by the double 3.0 */
static inline void centre_of(const vec3 p[3], real *c) {
    for (int k = 0; k < 3; k++) c[k] = (real)((double)(p[0][k] + p[1][k] + p[2][k]) / 3.0);
}

/* ---------------------------------------------------------------- scene */
typedef struct {
    vec3 p[3];
    int Frgb[3], Brgb[3];
    vec3 accB[3], daccB[3];
    vec3 deltaB;
    real se[3][4];
    vec3 c, n;
    real area;
    int parent;
    int nb[3];
} tri_t;

static tri_t *T;
static int trinum, pool_cap;
static vec3 G0, G1;

/* options, src/rad.cpp:17-31 */
static int opt_debug = 0;
static float AreaLimit = 5.0f, SampleArea = -1.0f, ConvergeLimit = 1200.0f, DeltaFFLimit = 0.000005f;
static int TriangleLimit = 1000000, WriteIteration = 10, ParallelSource = 1;
static float LightScale = 1.0f;

static int is_light(const tri_t *t) { return t->Brgb[0] == 255 || t->Brgb[1] == 255 || t->Brgb[2] == 255; }

/* src/rad.cpp:47-111 */
static int read_scene(FILE *fp) {
    vec3 lo = {1000000.0, 1000000.0, 1000000.0}, hi = {-1000000.0, -1000000.0, -1000000.0};
    char buf[4096];
    int cap = 1024;
    T = calloc(cap, sizeof(tri_t));
    trinum = 0;
    for (;;) {
        if (fscanf(fp, "%4095s", buf) != 1 || feof(fp)) break;
        if (trinum == cap) {
            T = realloc(T, 2 * (size_t)cap * sizeof(tri_t));
            memset(T + cap, 0, (size_t)cap * sizeof(tri_t));
            cap *= 2;
        }
        tri_t *t = &T[trinum];
        if (fscanf(fp, "%d%d%d", &t->Frgb[0], &t->Frgb[1], &t->Frgb[2]) != 3) return -1;
        if (fscanf(fp, "%d%d%d", &t->Brgb[0], &t->Brgb[1], &t->Brgb[2]) != 3) return -1;
        for (int v = 0; v < 3; v++) {
            if (sizeof(real) == sizeof(double)) {
                double x[3];
                if (fscanf(fp, "%lf%lf%lf", &x[0], &x[1], &x[2]) != 3) return -1;
                for (int k = 0; k < 3; k++) t->p[v][k] = (real)x[k];
            } else {
                float x[3];
                if (fscanf(fp, "%f%f%f", &x[0], &x[1], &x[2]) != 3) return -1;
                for (int k = 0; k < 3; k++) t->p[v][k] = (real)x[k];
            }
        }
        centre_of((const vec3 *)t->p, t->c);
        vec3 e0, e1;
        sub3(t->p[0], t->p[1], e0);
        sub3(t->p[0], t->p[2], e1);
        cross3(e0, e1, t->n);
        t->area = len3(t->n) / 2;
        real nl = len3(t->n);
        t->n[0] /= nl; t->n[1] /= nl; t->n[2] /= nl;
        for (int i = 0; i < 3; i++) {
            vec3 e, s;
            sub3(t->p[i], t->p[(i + 1) % 3], e);
            cross3(t->n, e, s);
            t->se[i][0] = s[0]; t->se[i][1] = s[1]; t->se[i][2] = s[2];
            t->se[i][3] = -dot3(t->p[i], s);
        }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                lo[j] = rmin(lo[j], t->p[i][j]);
                hi[j] = rmax(hi[j], t->p[i][j]);
            }
        t->parent = trinum++;
        t->nb[0] = t->nb[1] = t->nb[2] = -1;
    }
    real m = 0;
    for (int i = 0; i < 3; i++) m = rmax(m, hi[i] - lo[i]);
    for (int i = 0; i < 3; i++) G0[i] = (real)((double)lo[i] - PI_D);
    for (int i = 0; i < 3; i++) G1[i] = (real)((double)(G0[i] + m) + 2 * PI_D);
    /* slot pool: the reference's static TriStore[MaxTri], zero-filled */
    int lim = TriangleLimit < MAX_TRI_POOL ? TriangleLimit : MAX_TRI_POOL;
    pool_cap = (trinum > lim ? trinum : lim) + 8;
    if (pool_cap > cap) {
        T = realloc(T, (size_t)pool_cap * sizeof(tri_t));
        memset(T + cap, 0, (size_t)(pool_cap - cap) * sizeof(tri_t));
    }
    return 0;
}

/* ---------------------------------------------------------------- octree */
typedef struct { vec3 g0, g1; int sub[8]; int list; } node_t;
static node_t *nodes;
static int n_nodes, nodes_cap;
static int *lists;
static int n_lists, lists_cap;
static real min_grid;
static int grid_num;

/* src/raycast.cpp:24-60: does segment p0-p1 meet rectangle [g0,g1] in dims x,y */
static int clip2d(const real *p0, const real *p1, const real *g0, const real *g1, int x, int y) {
    int m1 = (p0[x] < g0[x]) << 0 | (p0[x] > g1[x]) << 1 | (p0[y] < g0[y]) << 2 | (p0[y] > g1[y]) << 3;
    int m2 = (p1[x] < g0[x]) << 0 | (p1[x] > g1[x]) << 1 | (p1[y] < g0[y]) << 2 | (p1[y] > g1[y]) << 3;
    if (m1 & m2) return 0;
    if (!(m1 | m2)) return 1;
    real a = p1[y] - p0[y], b = p1[x] - p0[x];
    real t = a * (g0[x] - p0[x]) - b * (g0[y] - p0[y]);
    if (t == 0) return 1;
    real side = (real)(t < 0);
    real s = (real)((a * (g0[x] - p0[x]) - b * (g1[y] - p0[y])) < 0);
    if (s != side) return 1;
    s = (real)((a * (g1[x] - p0[x]) - b * (g0[y] - p0[y])) < 0);
    if (s != side) return 1;
    s = (real)((a * (g1[x] - p0[x]) - b * (g1[y] - p0[y])) < 0);
    if (s != side) return 1;
    return 0;
}

/* src/raycast.cpp:91-100 */
static void lerp_at(const real *hi, const real *lo, real g, int d, real *out) {
    real dd = hi[d] - lo[d];
    if (dd == 0.0) {
        out[0] = hi[0]; out[1] = hi[1]; out[2] = hi[2];
    } else {
        real a = (g - lo[d]) / dd, b = (hi[d] - g) / dd;
        for (int k = 0; k < 3; k++) out[k] = a * hi[k] + b * lo[k];
    }
}

/* src/raycast.cpp:66-85 (three-element sort of vertex pointers on dim d) */
static void order3(const real **mx, const real **md, const real **mn, int d) {
    const real *t;
    if ((*mx)[d] < (*md)[d]) { t = *mx; *mx = *md; *md = t; }
    if ((*mx)[d] < (*mn)[d]) { t = *mx; *mx = *mn; *mn = t; }
    if ((*md)[d] < (*mn)[d]) { t = *md; *md = *mn; *mn = t; }
}

/* src/raycast.cpp:109-155 */
static int crosses_cube(const tri_t *tr, const real *g0, const real *g1) {
    const real *mx = tr->p[0], *md = tr->p[1], *mn = tr->p[2];
    vec3 a, b;
    for (int x = 0; x < 3; x++) {
        order3(&mx, &md, &mn, x);
        int y = (x + 1) % 3, z = (x + 2) % 3;
        if (g1[x] < mn[x]) return 0;
        lerp_at(mx, mn, g1[x], x, a);
        if (g1[x] < md[x]) { lerp_at(md, mn, g1[x], x, b); return clip2d(a, b, g0, g1, y, z); }
        else if (g1[x] <= mx[x]) { lerp_at(mx, md, g1[x], x, b); return clip2d(a, b, g0, g1, y, z); }
        if (g0[x] > mx[x]) return 0;
        lerp_at(mx, mn, g0[x], x, a);
        if (g0[x] > md[x]) { lerp_at(mx, md, g0[x], x, b); return clip2d(a, b, g0, g1, y, z); }
        else if (g0[x] >= mn[x]) { lerp_at(md, mn, g0[x], x, b); return clip2d(a, b, g0, g1, y, z); }
    }
    return 1;
}

static int push_node(void) {
    if (n_nodes == nodes_cap) {
        nodes_cap = nodes_cap ? 2 * nodes_cap : 1024;
        nodes = realloc(nodes, (size_t)nodes_cap * sizeof(node_t));
    }
    return n_nodes++;
}
static void push_list(int v) {
    if (n_lists == lists_cap) {
        lists_cap = lists_cap ? 2 * lists_cap : 4096;
        lists = realloc(lists, (size_t)lists_cap * sizeof(int));
    }
    lists[n_lists++] = v;
}

/* src/raycast.cpp:168-213: depth-first, node ids and list offsets in pre-order */
static int build_node(const int *idx, int n, int level, const real *g0, const real *g1) {
    int id = push_node();
    node_t *nd = &nodes[id];
    memcpy(nd->g0, g0, sizeof(vec3));
    memcpy(nd->g1, g1, sizeof(vec3));
    nd->list = -1;
    if (n <= MAX_TRI_PER_NODE || level >= MAX_LEVEL) {
        if (g1[0] - g0[0] < min_grid) min_grid = g1[0] - g0[0];
        for (int i = 0; i < 8; i++) nd->sub[i] = -1;
        nd->list = n_lists;
        for (int i = 0; i < n; i++) push_list(idx[i]);
        push_list(-1);
        return id;
    }
    vec3 mid;
    for (int k = 0; k < 3; k++) mid[k] = (real)(0.5 * (double)g0[k] + 0.5 * (double)g1[k]);
    int *sub = malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    for (int i = 0; i < 8; i++) {
        vec3 q0, q1;
        for (int j = 0; j < 3; j++) {
            q0[j] = g0[j]; q1[j] = g1[j];
            if ((i >> j) & 1) q0[j] = mid[j]; else q1[j] = mid[j];
        }
        int m = 0;
        for (int k = 0; k < n; k++)
            if (crosses_cube(&T[idx[k]], q0, q1)) sub[m++] = idx[k];
        int child = build_node(sub, m, level + 1, q0, q1);
        nodes[id].sub[i] = child; /* nodes may have moved */
    }
    free(sub);
    return id;
}

/* src/raycast.cpp:216-233 */
static void build_octree(void) {
    int *all = malloc((size_t)(trinum > 0 ? trinum : 1) * sizeof(int));
    for (int i = 0; i < trinum; i++) all[i] = i;
    n_nodes = 0; n_lists = 0;
    min_grid = G1[0] - G0[0];
    build_node(all, trinum, 0, G0, G1);
    grid_num = (int)((G1[0] - G0[0]) / min_grid);
    free(all);
    fprintf(stderr, "[INFO] 3D-DDA #TreeNode = %d, #Trilist = %d\n", n_nodes, n_lists);
}

/* ---------------------------------------------------------------- walk */
static long long cnt_rays, cnt_cells, cnt_tris, cnt_se, cnt_prec;

/* src/raycast.cpp:235-251 */
static real next_point(const real *p, const real *v, const real *g0, const real *g1, real *q) {
    real tm = 1000000.0;
    for (int i = 0; i < 3; i++) {
        if (fabs((double)v[i]) > 1e-6) {
            real s = (v[i] > 0) ? (g1[i] - p[i]) / v[i] : (g0[i] - p[i]) / v[i];
            tm = rmin(tm, s);
        }
    }
    tm = (real)((double)tm + 0.1);
    for (int k = 0; k < 3; k++) q[k] = p[k] + tm * v[k];
    return tm;
}

/* src/raycast.cpp:254-281 */
static int cell_of(const real *p) {
    if (p[0] < G0[0] || p[0] > G1[0] || p[1] < G0[1] || p[1] > G1[1] || p[2] < G0[2] || p[2] > G1[2])
        return -1;
    int g[3];
    for (int i = 0; i < 3; i++) g[i] = (int)(((double)p[i] - (double)G0[i]) / (double)min_grid);
    int cur = 0, gs = grid_num;
    while (nodes[cur].list < 0) {
        gs >>= 1;
        int ix = 0;
        for (int i = 0; i < 3; i++)
            if (g[i] >= gs) { ix |= 1 << i; g[i] -= gs; }
        cur = nodes[cur].sub[ix];
    }
    return cur;
}

/* src/raycast.cpp:283-313 */
static int tri_hit(const real *p, const real *v, const tri_t *tp, real *tmin) {
    cnt_tris++;
    real a1 = dot3(v, tp->n);
    vec3 w;
    sub3(p, tp->c, w);
    real a2 = dot3(w, tp->n);
    real t = a2 / a1;
    if ((double)t < 0.0001) return 0;
    if (t >= *tmin) return 0;
    cnt_se++;
    vec3 q;
    for (int k = 0; k < 3; k++) q[k] = p[k] + t * v[k];
    for (int e = 0; e < 3; e++)
        if ((q[0] * tp->se[e][0] + q[1] * tp->se[e][1] + q[2] * tp->se[e][2] + tp->se[e][3]) < 0.0) return 0;
    *tmin = t;
    return 1;
}

/* src/raycast.cpp:316-333 */
static int cell_hit(const real *p, const real *v, int at, int ban) {
    if (at < 0) return -1;
    int best = -1, k;
    real tmin = 1000000.0;
    while ((k = lists[at++]) >= 0) {
        if (k == ban) continue;
        if (tri_hit(p, v, &T[k], &tmin)) best = k;
    }
    return best;
}

/* src/raycast.cpp:335-360.  The walk's state at the top of the loop is
 * (t, prev).  When it repeats, the reference's loop never ends (it only
 * notices one cell repeated on consecutive steps); this happens when
 * TreeNodeNum returns a leaf that does not contain q (GridNum truncated to 63
 * where the tree is 64 cells deep).  Brent's cycle detection finds any
 * repeated state; such a walk stops here and the ray counts as blocked (-3),
 * recorded in cnt_loops.  Walks the reference finishes are unaffected. */
static long long cnt_loops;
static int ray_hit(const real *p, const real *v, int from, int target) {
    (void)target;
    cnt_rays++;
    real t = 0;
    int prev = -1, cur, hit;
    vec3 q = {p[0], p[1], p[2]};
    real chk_t = -1;
    int chk_prev = -2, power = 1, lam = 0;
    while ((cur = cell_of(q)) >= 0) {
        if (t == chk_t && prev == chk_prev) {
            cnt_loops++;
            return -3;
        }
        if (++lam == power) { chk_t = t; chk_prev = prev; power <<= 1; lam = 0; }
        cnt_cells++;
        if (prev == cur) {
            cnt_prec++;
            t = (real)((double)t + 1.0);
            for (int k = 0; k < 3; k++) q[k] = p[k] + t * v[k];
            continue;
        }
        if ((hit = cell_hit(p, v, nodes[cur].list, from)) >= 0) return hit;
        prev = cur;
        t = next_point(p, v, nodes[cur].g0, nodes[cur].g1, q);
    }
    return -1;
}

/* ---------------------------------------------------------------- shading */
typedef struct { vec3 p[3]; vec3 c, n; real area; } patch_t;

/* src/shade.cpp:107-127: vertex-to-patch form factor with one visibility ray */
static real point_ff(const patch_t *src, int logsrc, const tri_t *des, int logdes, const real *p) {
    vec3 d;
    sub3(p, src->c, d);
    real ds = dot3(d, src->n);
    real dd = -dot3(d, des->n);
    if ((ds < 0) != (dd < 0)) return 0;
    real dl = len3(d), sl = len3(src->n), el = len3(des->n);
    real c1 = ds / dl / sl, c2 = dd / dl / el;
    real ff = c1 * c2;
    if (ff <= 0.0) return 0;
    ff = (real)((double)ff * ((double)src->area / ((double)dot3(d, d) * PI_D)));
    if (ff <= 0.0) return 0;
    if (ray_hit(p, d, logdes, logsrc) == logsrc) return ff;
    return 0;
}

/* src/shade.cpp:76-99 */
static void split_source(const patch_t *s, patch_t *t1, patch_t *t2, int e) {
    int i0 = e, i1 = (e + 1) % 3, i2 = (e + 2) % 3;
    vec3 m;
    for (int k = 0; k < 3; k++) m[k] = (real)((double)(s->p[i0][k] + s->p[i1][k]) / 2.0);
    memcpy(t1->p[0], m, sizeof(vec3));
    memcpy(t2->p[0], m, sizeof(vec3));
    memcpy(t1->p[1], s->p[i2], sizeof(vec3));
    memcpy(t1->p[2], s->p[i0], sizeof(vec3));
    centre_of((const vec3 *)t1->p, t1->c);
    memcpy(t1->n, s->n, sizeof(vec3));
    memcpy(t2->p[1], s->p[i1], sizeof(vec3));
    memcpy(t2->p[2], s->p[i2], sizeof(vec3));
    centre_of((const vec3 *)t2->p, t2->c);
    memcpy(t2->n, s->n, sizeof(vec3));
    t1->area = t2->area = (real)((double)s->area / 2.0);
}

/* src/shade.cpp:141-168.  The recursive branch is unreachable: the test at
 * shade.cpp:164 ends in a stray ';' and line 165 returns unconditionally. */
static real adapt_ff(real ff, const patch_t *src, int logsrc, const tri_t *des, int logdes, const real *p) {
    int e = 0;
    real longest = 0.0;
    for (int v = 0; v < 3; v++) {
        vec3 l;
        sub3(src->p[v], src->p[(v + 1) % 3], l);
        real len = dot3(l, l);
        if (longest < len) { longest = len; e = v; }
    }
    if ((double)longest < 0.1) return ff;
    patch_t h1, h2;
    split_source(src, &h1, &h2, e);
    real f1 = point_ff(&h1, logsrc, des, logdes, p);
    real f2 = point_ff(&h2, logsrc, des, logdes, p);
    return f1 + f2;
}

/* src/shade.cpp:244-259 */
static void deposit(const tri_t *src, tri_t *des, const real ff[3]) {
    const real k = (real)(0.5 / 255.0);
    real lo[3];
    for (int c = 0; c < 3; c++) lo[c] = (real)des->Frgb[c] * k * src->deltaB[c] / 3;
    for (int v = 0; v < 3; v++)
        for (int c = 0; c < 3; c++) {
            real x = lo[c] * ff[v];
            des->deltaB[c] += x;
            des->accB[v][c] += x;
            des->daccB[v][c] = x;
        }
}

static void as_patch(const tri_t *t, patch_t *pt) {
    memcpy(pt->p, t->p, sizeof(pt->p));
    memcpy(pt->c, t->c, sizeof(vec3));
    memcpy(pt->n, t->n, sizeof(vec3));
    pt->area = t->area;
}

/* src/shade.cpp:435-462 (shipped: DONT_PARTITION returns before the split test) */
static void shade(const tri_t *src, int logsrc, tri_t *des, int logdes) {
    patch_t sp;
    as_patch(src, &sp);
    real ff[3];
    for (int v = 0; v < 3; v++)
        ff[v] = adapt_ff(point_ff(&sp, logsrc, des, logdes, des->p[v]), &sp, logsrc, des, logdes, des->p[v]);
    deposit(src, des, ff);
}

/* ---------------------------------------------------------------- init */
/* Neighbour links, src/rad.cpp:295-334.  The reference compares every pair
 * (i, j), j ascending, and later writes win.  Only pairs that share an exact
 * vertex can write, so corners are bucketed by vertex and, for each i in
 * ascending order, the writes are applied in the reference's (j, v, n) order:
 * the final links equal those of the sequential O(N^2) scan. */
typedef struct { uint64_t k[3]; int tri, v; } corner_t;
static uint64_t coord_bits(real x) {
    if (x == 0) return 0; /* +0 and -0 compare equal */
    uint64_t b = 0;
    memcpy(&b, &x, sizeof(real));
    return b;
}
static int corner_cmp(const void *a, const void *b) {
    const corner_t *x = a, *y = b;
    for (int q = 0; q < 3; q++)
        if (x->k[q] != y->k[q]) return x->k[q] < y->k[q] ? -1 : 1;
    if (x->tri != y->tri) return x->tri < y->tri ? -1 : 1;
    return x->v - y->v;
}
typedef struct { int j, v, n; } nbw_t;
static int nbw_cmp(const void *a, const void *b) {
    const nbw_t *x = a, *y = b;
    if (x->j != y->j) return x->j < y->j ? -1 : 1;
    if (x->v != y->v) return x->v - y->v;
    return x->n - y->n;
}
static void link_neighbours(void) {
    int n = trinum, m = 0;
    corner_t *cs = malloc((size_t)(3 * n + 1) * sizeof(corner_t));
    for (int i = 0; i < n; i++)
        for (int v = 0; v < 3; v++) {
            const real *p = T[i].p[v];
            if (p[0] != p[0] || p[1] != p[1] || p[2] != p[2]) continue; /* NaN equals nothing */
            for (int q = 0; q < 3; q++) cs[m].k[q] = coord_bits(p[q]);
            cs[m].tri = i; cs[m].v = v; m++;
        }
    qsort(cs, (size_t)m, sizeof(corner_t), corner_cmp);
    int *grp = malloc((size_t)(3 * n + 1) * sizeof(int)), *gs = malloc((size_t)(m + 2) * sizeof(int));
    for (int q = 0; q < 3 * n; q++) grp[q] = -1;
    int ng = 0;
    for (int a = 0; a < m;) {
        int b = a + 1;
        while (b < m && !memcmp(cs[b].k, cs[a].k, sizeof cs[a].k)) b++;
        gs[ng] = a;
        for (int q = a; q < b; q++) grp[3 * cs[q].tri + cs[q].v] = ng;
        ng++;
        a = b;
    }
    gs[ng] = m;
    int wcap = 64;
    nbw_t *w = malloc((size_t)wcap * sizeof(nbw_t));
    for (int i = 0; i < n; i++) {
        int nw = 0;
        for (int v = 0; v < 3; v++) {
            int g = grp[3 * i + v];
            if (g < 0) continue;
            for (int q = gs[g]; q < gs[g + 1]; q++) {
                if (cs[q].tri == i) continue;
                if (nw == wcap) { wcap *= 2; w = realloc(w, (size_t)wcap * sizeof(nbw_t)); }
                w[nw].j = cs[q].tri; w[nw].v = v; w[nw].n = cs[q].v; nw++;
            }
        }
        qsort(w, (size_t)nw, sizeof(nbw_t), nbw_cmp);
        tri_t *tp = &T[i];
        for (int q = 0; q < nw; q++) {
            int j = w[q].j, v = w[q].v, nn = w[q].n;
            tri_t *tn = &T[j];
            const real *a1 = tp->p[(v + 1) % 3], *b1 = tn->p[(nn + 1) % 3], *b2 = tn->p[(nn + 2) % 3];
            real cs_ = dot3(tp->n, tn->n) / len3(tp->n) / len3(tn->n);
            if (a1[0] == b1[0] && a1[1] == b1[1] && a1[2] == b1[2]) {
                if ((double)cs_ > 0.85) { tp->nb[v] = j; tn->nb[nn] = i; }
            } else if (a1[0] == b2[0] && a1[1] == b2[1] && a1[2] == b2[2]) {
                if ((double)cs_ > 0.85) { tp->nb[v] = j; tn->nb[(nn + 2) % 3] = i; }
            }
        }
    }
    free(w); free(gs); free(grp); free(cs);
}


/* src/rad.cpp:259-356 */
static void init_radiosity(void) {
    real minarea = 100000000.0, maxarea = 0.0;
    for (int i = 0; i < trinum; i++) {
        tri_t *tp = &T[i];
        minarea = rmin(minarea, tp->area);
        maxarea = rmax(maxarea, tp->area);
        if (is_light(tp)) {
            tp->deltaB[0] = tp->deltaB[1] = tp->deltaB[2] = 0;
            real scale = (real)LightScale;
            for (int v = 0; v < 3; v++) {
                for (int c = 0; c < 3; c++) tp->accB[v][c] = (real)tp->Brgb[c] * scale;
                for (int c = 0; c < 3; c++) tp->deltaB[c] += 100 * tp->accB[v][c] / 3;
            }
        } else {
            memset(tp->accB, 0, sizeof(tp->accB));
            memset(tp->deltaB, 0, sizeof(tp->deltaB));
        }
    }
    link_neighbours();
    if (SampleArea < 0.0) SampleArea = (float)((double)maxarea / 100.0);
    printf("[INFO] Max Patch Area = %f\n", (double)maxarea);
    printf("[INFO] Min Patch Area = %f\n", (double)minarea);
}

/* ---------------------------------------------------------------- pre-partition */
static int pool_limit(void) { return TriangleLimit < MAX_TRI_POOL ? TriangleLimit : MAX_TRI_POOL; }

/* src/shade.cpp:14-25 */
static int alloc_slot(void) {
    static int first = 1;
    if (trinum == MAX_TRI_POOL || trinum == TriangleLimit) {
        if (first) { fprintf(stderr, "\n**** Max Triangle exceed : %i ***\n", trinum); first = 0; }
        return -1;
    }
    return trinum++;
}
static int pool_full(int need) { return trinum + need >= pool_limit(); } /* shade.cpp:26-30 */

/* src/shade.cpp:33-43 */
static void relink(int nb, int old_id, int new_id) {
    if (nb < 0) return;
    for (int v = 0; v < 3; v++)
        if (T[nb].nb[v] == old_id) T[nb].nb[v] = new_id;
}

/* src/shade.cpp:171-211: longest-edge bisection of a receiver */
static void bisect(const tri_t *s, tri_t *t1, tri_t *t2, int e) {
    int i0 = e, i1 = (e + 1) % 3, i2 = (e + 2) % 3;
    vec3 m;
    for (int k = 0; k < 3; k++) m[k] = (real)((double)(s->p[i0][k] + s->p[i1][k]) / 2.0);
    memcpy(t1->p[0], m, sizeof(vec3));
    memcpy(t1->p[1], s->p[i2], sizeof(vec3));
    memcpy(t1->p[2], s->p[i0], sizeof(vec3));
    memcpy(t1->n, s->n, sizeof(vec3));
    memcpy(t1->Frgb, s->Frgb, sizeof(t1->Frgb));
    memcpy(t1->deltaB, s->deltaB, sizeof(vec3));
    centre_of((const vec3 *)t1->p, t1->c);
    memcpy(t2->p[0], m, sizeof(vec3));
    memcpy(t2->p[1], s->p[i1], sizeof(vec3));
    memcpy(t2->p[2], s->p[i2], sizeof(vec3));
    memcpy(t2->n, s->n, sizeof(vec3));
    memcpy(t2->Frgb, s->Frgb, sizeof(t2->Frgb));
    memcpy(t2->deltaB, s->deltaB, sizeof(vec3));
    centre_of((const vec3 *)t2->p, t2->c);
    vec3 a;
    for (int k = 0; k < 3; k++) a[k] = (real)((double)(s->accB[i0][k] + s->accB[i1][k]) / 2.0);
    memcpy(t1->accB[0], a, sizeof(vec3));
    memcpy(t1->accB[1], s->accB[i2], sizeof(vec3));
    memcpy(t1->accB[2], s->accB[i0], sizeof(vec3));
    memcpy(t2->accB[0], a, sizeof(vec3));
    memcpy(t2->accB[1], s->accB[i1], sizeof(vec3));
    memcpy(t2->accB[2], s->accB[i2], sizeof(vec3));
    t1->area = t2->area = (real)((double)s->area / 2.0);
    t1->parent = t2->parent = s->parent;
}

/* src/shade.cpp:311-431.  Slot ids out[0..3] (-1 when not created). */
static int split_and_store(int src_id, int out[4], int *reshade) {
    tri_t *s = &T[src_id];
    *reshade = 0;
    out[0] = out[1] = out[2] = out[3] = -1;
    if (pool_full(4) || (double)s->area < 1e-8) return -1;
    int e = 0;
    real longest = 0.0;
    for (int v = 0; v < 3; v++) {
        vec3 l;
        sub3(s->p[v], s->p[(v + 1) % 3], l);
        real len = dot3(l, l);
        if (longest < len) { longest = len; e = v; }
    }
    if (longest < 1) return -1;
    int nbid = s->nb[e];
    if (nbid >= 0 && (double)T[nbid].area < 1e-1) return -1;

    int id1 = alloc_slot(), id2 = alloc_slot();
    bisect(s, &T[id1], &T[id2], e);
    int n1, n2;
    T[id1].nb[1] = n1 = s->nb[(e + 2) % 3];
    T[id2].nb[1] = n2 = s->nb[(e + 1) % 3];
    T[id1].nb[2] = T[id2].nb[0] = -1;
    int replaced = 0;
    if (s->parent == src_id) {
        s->parent = -1;
    } else {
        T[src_id] = T[id2];
        id2 = src_id;
        trinum--;
        replaced = 1;
    }
    relink(n1, src_id, id1);
    relink(n2, src_id, id2);
    T[id1].nb[0] = id2;
    T[id2].nb[2] = id1;
    out[0] = id1; out[1] = id2;
    if (nbid < 0) return replaced;

    int id3 = alloc_slot(), id4 = alloc_slot();
    tri_t *nt = &T[nbid];
    int ne = 0;
    for (int v = 0; v < 3; v++)
        if (nt->nb[v] == src_id) ne = v;
    if (nbid < src_id)
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++) nt->accB[v][k] -= nt->daccB[v][k];
    bisect(nt, &T[id3], &T[id4], ne);
    T[id3].nb[1] = n1 = nt->nb[(ne + 2) % 3];
    T[id4].nb[1] = n2 = nt->nb[(ne + 1) % 3];
    if (nt->parent == nbid) {
        nt->parent = -1;
    } else {
        T[nbid] = T[id4];
        id4 = nbid;
        trinum--;
    }
    relink(n1, nbid, id3);
    relink(n2, nbid, id4);
    T[id3].nb[0] = id4;
    T[id4].nb[2] = id3;
    /* shade.cpp:416 compares two vertex-array addresses: equal only for the same slot and edge */
    if (src_id == nbid && e == ne) {
        T[id1].nb[2] = id3; T[id3].nb[2] = id1; T[id2].nb[0] = id4; T[id4].nb[0] = id2;
    } else {
        T[id1].nb[2] = id4; T[id4].nb[0] = id1; T[id2].nb[0] = id3; T[id3].nb[2] = id2;
    }
    if (id4 < src_id) *reshade = 1;
    out[2] = id3; out[3] = id4;
    return replaced;
}

/* ordered set of (area, slot) with the std::set semantics used at shade.cpp:561-595 */
typedef struct { real a; int i; } akey;
static akey *heap;
static int heap_n, heap_cap;
static size_t hset_cap, hset_n;
static int akey_less(akey x, akey y) { return x.a < y.a || (!(y.a < x.a) && x.i < y.i); }
static uint64_t akey_bits(akey k) {
    uint64_t b = 0;
    if (sizeof(real) == 4) { float f = (float)k.a; uint32_t u; memcpy(&u, &f, 4); b = u; }
    else { double d = (double)k.a; memcpy(&b, &d, 8); }
    return (b * 0x9E3779B97F4A7C15ull) ^ (uint64_t)(uint32_t)k.i ^ ((uint64_t)(uint32_t)k.i << 40);
}
static akey *hkeys;
static unsigned char *hused;
static long hset_find(akey k) {
    if (hset_cap == 0) return -1;
    size_t h = akey_bits(k) & (hset_cap - 1);
    while (hused[h] == 1 || hused[h] == 2) {
        if (hused[h] == 1 && !akey_less(hkeys[h], k) && !akey_less(k, hkeys[h]) && hkeys[h].i == k.i) return (long)h;
        h = (h + 1) & (hset_cap - 1);
    }
    return -1;
}
static void hset_grow(void);
static int hset_insert(akey k) {
    if (hset_find(k) >= 0) return 0;
    if (2 * (hset_n + 1) > hset_cap) hset_grow();
    size_t h = akey_bits(k) & (hset_cap - 1);
    while (hused[h] == 1) h = (h + 1) & (hset_cap - 1);
    hused[h] = 1; hkeys[h] = k; hset_n++;
    return 1;
}
static void hset_erase(akey k) {
    long h = hset_find(k);
    if (h >= 0) { hused[h] = 2; hset_n--; }
}
static void hset_grow(void) {
    size_t oc = hset_cap;
    akey *ok = hkeys;
    unsigned char *ou = hused;
    hset_cap = oc ? 4 * oc : 1024;
    hkeys = calloc(hset_cap, sizeof(akey));
    hused = calloc(hset_cap, 1);
    hset_n = 0;
    for (size_t i = 0; i < oc; i++)
        if (ou[i] == 1) hset_insert(ok[i]);
    free(ok); free(ou);
}
static void set_insert(akey k) {
    if (!hset_insert(k)) return;
    if (heap_n == heap_cap) { heap_cap = heap_cap ? 2 * heap_cap : 1024; heap = realloc(heap, (size_t)heap_cap * sizeof(akey)); }
    int i = heap_n++;
    heap[i] = k;
    while (i > 0) {
        int p = (i - 1) / 2;
        if (!akey_less(heap[p], heap[i])) break;
        akey t = heap[p]; heap[p] = heap[i]; heap[i] = t; i = p;
    }
}
static akey set_pop_max(void) {
    akey top = heap[0];
    heap[0] = heap[--heap_n];
    int i = 0;
    for (;;) {
        int l = 2 * i + 1, r = l + 1, m = i;
        if (l < heap_n && akey_less(heap[m], heap[l])) m = l;
        if (r < heap_n && akey_less(heap[m], heap[r])) m = r;
        if (m == i) break;
        akey t = heap[m]; heap[m] = heap[i]; heap[i] = t; i = m;
    }
    hset_erase(top);
    return top;
}

/* src/shade.cpp:556-598 (with the empty-set guard before line 570) */
static void pre_partition(void) {
    fprintf(stderr, "[DEBUG] Before PrePartitionTriangle %d\n", trinum);
    for (int i = 0; i < trinum; i++) {
        if (T[i].area < 1.f || is_light(&T[i])) continue;
        set_insert((akey){T[i].area, i});
    }
    for (;;) {
        if (heap_n == 0) break;
        akey top = set_pop_max();
        tri_t *tp = &T[top.i];
        if (tp->area < 1) break;
        int out[4], reshade;
        if (split_and_store(top.i, out, &reshade) < 0) break;
        if (is_light(tp)) {
            for (int q = 0; q < 4; q++) {
                if (out[q] < 0 || &T[out[q]] == tp) continue;
                tri_t *c = &T[out[q]];
                memcpy(c->Brgb, tp->Brgb, sizeof(c->Brgb));
                for (int v = 0; v < 3; v++) {
                    memcpy(c->accB[v], tp->accB[v], sizeof(vec3));
                    c->deltaB[v] = tp->deltaB[v];
                }
            }
        }
        for (int q = 0; q < 4; q++)
            if (out[q] >= 0) set_insert((akey){T[out[q]].area, out[q]});
    }
    fprintf(stderr, "[DEBUG] After PrePartitionTriangle %d\n", trinum);
}

/* ---------------------------------------------------------------- loop */
typedef struct { real key; int i; } cand_t;
static int cand_cmp(const void *a, const void *b) {
    const cand_t *x = a, *y = b;
    if (x->key < y->key) return -1;
    if (y->key < x->key) return 1;
    return (x->i > y->i) - (x->i < y->i);
}

/* src/rad.cpp:387-404 */
static int select_shooters(int *out) {
    cand_t *c = malloc((size_t)(trinum > 0 ? trinum : 1) * sizeof(cand_t));
    int nc = 0;
    for (int i = 0; i < trinum; i++) {
        if (T[i].parent < 0) continue;
        real d = T[i].deltaB[0] + T[i].deltaB[1] + T[i].deltaB[2];
        if (d > ConvergeLimit) { c[nc].key = d; c[nc].i = i; nc++; }
    }
    qsort(c, (size_t)nc, sizeof(cand_t), cand_cmp);
    int n = (nc + 4) / 5;
    if (n > ParallelSource) n = ParallelSource;
    for (int k = 0; k < n; k++) out[k] = c[nc - 1 - k].i;
    free(c);
    return n;
}

/* src/rad.cpp:406-451 */
static int shoot_step(FILE *trace) {
    int *C = malloc((size_t)(ParallelSource > 0 ? ParallelSource : 1) * sizeof(int));
    int nc = select_shooters(C);
    if (trace) {
        fprintf(trace, "%d", nc);
        for (int k = 0; k < nc; k++) fprintf(trace, " %d", C[k]);
        fputc('\n', trace);
    }
    if (nc == 0) { free(C); return 0; }
    for (int i = 0; i < trinum; i++) {
        tri_t *d = &T[i];
        if (d->parent < 0) continue;
        int is_src = 0;
        for (int k = 0; k < nc; k++) is_src |= (C[k] == i);
        if (is_src) continue;
        int open = 0;
        for (int v = 0; v < 3; v++)
            for (int c = 0; c < 3; c++) open |= ((double)d->accB[v][c] < 255.0);
        if (!open) continue;
        for (int k = 0; k < nc; k++) {
            if (C[k] == i) continue;
            shade(&T[C[k]], T[C[k]].parent, d, d->parent);
        }
    }
    for (int k = 0; k < nc; k++) T[C[k]].deltaB[0] = T[C[k]].deltaB[1] = T[C[k]].deltaB[2] = 0;
    free(C);
    return 1;
}

/* ---------------------------------------------------------------- adaptive variant */
/* The reference built with include/config.h = ADAPT + ROLLBACK only: no
 * pre-partition, serialRadiosity (rad.cpp:452-490) and the full Shade
 * (shade.cpp:435-554) whose delta-FF test can split a receiver. */
static int variant_adapt = 0;

/* glibc rand(): TYPE_3 additive feedback generator, seeded with 1 (the
 * reference never calls srand).  r[0] = 1; r[i] = 16807 r[i-1] mod (2^31-1)
 * for i < 31 (Schrage's method); r[i] = r[i-31] for i = 31..33;
 * r[i] = r[i-31] + r[i-3] (mod 2^32) after that; output k is r[k+344] >> 1. */
static uint32_t rs_r[34];
static int rs_i, rs_init;
static int glibc_rand(void) {
    if (!rs_init) {
        int32_t w = 1;
        rs_r[0] = 1;
        for (int i = 1; i < 31; i++) {
            int32_t hi = w / 127773, lo = w % 127773;
            w = 16807 * lo - 2836 * hi;
            if (w < 0) w += 2147483647;
            rs_r[i] = (uint32_t)w;
        }
        for (int i = 31; i < 34; i++) rs_r[i] = rs_r[i - 31];
        rs_i = 34;
        rs_init = 1;
        for (int k = 0; k < 310; k++) glibc_rand();
    }
    /* ring of 34: r[i] = r[i-31] + r[i-3] */
    uint32_t v = rs_r[(rs_i - 31) % 34] + rs_r[(rs_i - 3) % 34];
    rs_r[rs_i % 34] = v;
    rs_i++;
    return (int)(v >> 1);
}

/* src/shade.cpp:49-68 */
static real sample_point(const tri_t *t, real *pt, const real ff[3]) {
    real r1 = (real)glibc_rand(), r2 = (real)glibc_rand(), r3 = (real)glibc_rand();
    real tot = r1 + r2 + r3;
    r1 /= tot; r2 /= tot; r3 /= tot;
    for (int v = 0; v < 3; v++) pt[v] = r1 * t->p[0][v] + r2 * t->p[1][v] + r3 * t->p[2][v];
    return r1 * ff[0] + r2 * ff[1] + r3 * ff[2];
}

static real corner_ff_at(const tri_t *src, int logsrc, const tri_t *des, int logdes, const real *pt) {
    patch_t sp;
    as_patch(src, &sp);
    return adapt_ff(point_ff(&sp, logsrc, des, logdes, pt), &sp, logsrc, des, logdes, pt);
}

static real fabs_f(real x) { return (real)fabs((double)x); }   /* ffabs, rad.h:14 */

/* src/shade.cpp:435-554 with ADAPT, ROLLBACK, no DONT_PARTITION, no PARALLEL.
 * The shooter is read from its slot each time (a split can replace it). */
static int shade_adapt(int src_id, int logsrc, int des_id, int logdes) {
    real ff[3];
    for (int v = 0; v < 3; v++) ff[v] = corner_ff_at(&T[src_id], logsrc, &T[des_id], logdes, T[des_id].p[v]);
    tri_t *des = &T[des_id];
    if (des->area < AreaLimit) { deposit(&T[src_id], des, ff); return 0; }
    if (pool_full(4) || (double)des->area < 1e-8) { deposit(&T[src_id], des, ff); return 0; }
    real ground = (real)((double)(ff[0] + ff[1] + ff[2]) / 3.0);
    real ffs = corner_ff_at(&T[src_id], logsrc, des, logdes, des->c);
    real dff;
    if ((dff = fabs_f(ground - ffs)) < DeltaFFLimit) {
        int n = (int)(des->area / SampleArea);
        for (int k = 0; k < n; k++) {
            real pt[3];
            ground = sample_point(des, pt, ff);
            ffs = corner_ff_at(&T[src_id], logsrc, des, logdes, pt);
            if ((dff = fabs_f(ground - ffs)) > DeltaFFLimit) break;
        }
        if (dff < DeltaFFLimit) { deposit(&T[src_id], des, ff); return 0; }
    }
    int out[4], reshade;
    int rep = split_and_store(des_id, out, &reshade);
    if (reshade) {
        tri_t *t4 = &T[out[3]];
        for (int v = 0; v < 3; v++) ff[v] = corner_ff_at(&T[src_id], logsrc, t4, logdes, t4->p[v]);
        deposit(&T[src_id], t4, ff);
    }
    return rep;
}

/* src/rad.cpp:359-386: the first strict maximum (ties: lowest index) */
static int max_delta_rad(void) {
    int best = -1;
    real m = 0;
    for (int i = 0; i < trinum; i++) {
        if (T[i].parent < 0) continue;
        real d = T[i].deltaB[0] + T[i].deltaB[1] + T[i].deltaB[2];
        if (d > m && d > ConvergeLimit) { best = i; m = d; }
    }
    return best;
}

/* src/rad.cpp:452-490 */
static int serial_step(FILE *trace) {
    int src = max_delta_rad();
    if (trace) {
        if (src >= 0) fprintf(trace, "1 %d\n", src);
        else fputs("0\n", trace);
    }
    if (src < 0) return 0;
    const int logsrc = T[src].parent;
    for (int d = 0; d < trinum; d++) {
        if (d == src) continue;
        if (T[d].parent < 0) continue;
        int open = 0;
        for (int v = 0; v < 3; v++)
            for (int c = 0; c < 3; c++) open |= ((double)T[d].accB[v][c] < 255.0);
        if (!open) continue;
        if (shade_adapt(src, logsrc, d, T[d].parent)) d--;
    }
    T[src].deltaB[0] = T[src].deltaB[1] = T[src].deltaB[2] = 0;
    return 1;
}

/* ---------------------------------------------------------------- output */
/* Float to text as include/float2string.h does it (fixed point, up to 8
 * truncated fraction digits, trailing zeros dropped).  Returns 0 and leaves
 * buf untouched for Inf, NaN, subnormals and |x| >= 2^64. */
static int fmt_float(float x, char *buf) {
    uint32_t raw;
    memcpy(&raw, &x, 4);
    int neg = (raw >> 31) & 1;
    int ebits = (raw >> 23) & 0xff;
    uint32_t frac = raw & 0x7fffff;
    if (ebits == 0xff || (ebits == 0 && frac != 0)) return 0;
    char *d = buf;
    if (ebits == 0) {
        if (neg) *d++ = '-';
        *d++ = '0'; *d++ = '.'; *d++ = '0'; *d = 0;
        return (int)(d - buf);
    }
    int exp = ebits - 127 - 23;
    if (exp > 0 && !(exp < 64 - 23)) return 0;
    uint64_t mant = frac | (1u << 23);
    if (neg) *d++ = '-';
    /* integer part */
    char ip[24];
    int nd = 0;
    if (exp < 0 && -exp > 23) {
        ip[nd++] = '0';
    } else {
        uint64_t iv = exp > 0 ? mant << exp : (exp < 0 ? mant >> (-exp) : mant);
        while (iv) { ip[nd++] = (char)('0' + iv % 10); iv /= 10; }
    }
    if (nd == 0) *d++ = '0';
    for (int k = nd - 1; k >= 0; k--) *d++ = ip[k];
    *d++ = '.';
    /* fraction part: 60-bit fixed point, top four bits hold the digit */
    int shift = 64 + exp - 4;
    int keep = 0;
    char fd[8];
    if (!(shift >= 60 || shift < 0)) {
        uint64_t f = mant << shift;
        int k = 0;
        while (f && k < 8) {
            f &= 0x0fffffffffffffffull;
            f *= 10;
            int dg = (int)(f >> 60);
            fd[k++] = (char)('0' + dg);
            if (dg > 0) keep = k;
        }
    }
    if (keep == 0) *d++ = '0';
    for (int k = 0; k < keep; k++) *d++ = fd[k];
    *d = 0;
    return (int)(d - buf);
}

/* src/rad.cpp:117-242 (non-OLD_FORMAT branch) */
static char g_fbuf[64];
static void write_fin(const char *prefix, int loop) {
    char fn[4096];
    if (loop == 0) snprintf(fn, sizeof fn, "%s.fin", prefix);
    else snprintf(fn, sizeof fn, "%s.%1d", prefix, loop);
    FILE *f = fopen(fn, "w");
    if (!f) {
        fprintf(stderr, "Error: output file %s open failed\n", fn);
        if (loop != 0) return;
        f = stdout;
    }
    for (int i = 0; i < trinum; i++) {
        const tri_t *t = &T[i];
        if (t->parent < 0) continue;
        fputs("Triangle \n", f);
        int col[3];
        for (int j = 0; j < 3; j++) {
            real v = 0;
            for (int k = 0; k < 3; k++) v += t->accB[k][j];
            v /= 3;
            v = ((real)255.0 < v) ? (real)255.0 : v;
            v = (v < (real)0.0) ? (real)0.0 : v;
            if (isnan(v)) v = 0;
            col[j] = (int)v;
        }
        fprintf(f, "%d %d %d 0 0 0\n", col[0], col[1], col[2]);
        char nrm[128] = {0};
        for (int k = 0; k < 3; k++) {
            fmt_float((float)t->n[k], g_fbuf);
            strcat(nrm, g_fbuf);
            strcat(nrm, k < 2 ? " " : "\n");
        }
        for (int j = 0; j < 3; j++) {
            for (int k = 0; k < 3; k++) {
                fmt_float((float)t->p[j][k], g_fbuf);
                fputs(g_fbuf, f);
                fputs(" ", f);
            }
            fputs(nrm, f);
        }
    }
    if (f != stdout) fclose(f);
}

static void put_dump(const char *path, int steps) {
    FILE *f = fopen(path, "wb");
    if (!f) return;
    fwrite("RADDUMP1", 1, 8, f);
    int n = trinum, esz = (int)sizeof(real);
    fwrite(&n, 4, 1, f); fwrite(&esz, 4, 1, f); fwrite(&steps, 4, 1, f);
    for (int i = 0; i < n; i++) fwrite(&T[i].parent, 4, 1, f);
    for (int i = 0; i < n; i++) fwrite(T[i].p, sizeof(real), 9, f);
    for (int i = 0; i < n; i++) fwrite(T[i].accB, sizeof(real), 9, f);
    for (int i = 0; i < n; i++) fwrite(T[i].deltaB, sizeof(real), 3, f);
    for (int i = 0; i < n; i++) fwrite(&T[i].area, sizeof(real), 1, f);
    for (int i = 0; i < n; i++) fwrite(T[i].n, sizeof(real), 3, f);
    for (int i = 0; i < n; i++) fwrite(T[i].c, sizeof(real), 3, f);
    for (int i = 0; i < n; i++) fwrite(T[i].Frgb, 4, 3, f);
    for (int i = 0; i < n; i++) fwrite(T[i].nb, 4, 3, f);
    fclose(f);
}

/* ---------------------------------------------------------------- queries */
/* RAD_RAYS=path: binary input of n records {real p[3], real v[3], int32 ban}
 * (after pre-partition); writes path.out with one int32 RayHitted result per
 * record.  RAD_FF=path: input int32 src, int32 n, int32 rcv[n]; writes
 * path.out with real ff[n][3] = AdaptCalFF(CalFF(...)) per receiver corner. */
static void run_queries(void) {
    const char *rp = getenv("RAD_RAYS");
    if (rp) {
        FILE *f = fopen(rp, "rb");
        char op[4096];
        snprintf(op, sizeof op, "%s.out", rp);
        FILE *g = fopen(op, "wb");
        if (f && g) {
            real pv[6];
            int ban;
            while (fread(pv, sizeof(real), 6, f) == 6 && fread(&ban, 4, 1, f) == 1) {
                int hit = ray_hit(pv, pv + 3, ban, -1);
                fwrite(&hit, 4, 1, g);
            }
        }
        if (f) fclose(f);
        if (g) fclose(g);
    }
    const char *fp = getenv("RAD_FF");
    if (fp) {
        FILE *f = fopen(fp, "rb");
        char op[4096];
        snprintf(op, sizeof op, "%s.out", fp);
        FILE *g = fopen(op, "wb");
        int src, n;
        if (f && g && fread(&src, 4, 1, f) == 1 && fread(&n, 4, 1, f) == 1) {
            patch_t sp;
            as_patch(&T[src], &sp);
            for (int k = 0; k < n; k++) {
                int r;
                if (fread(&r, 4, 1, f) != 1) break;
                real ff[3];
                for (int v = 0; v < 3; v++)
                    ff[v] = adapt_ff(point_ff(&sp, T[src].parent, &T[r], T[r].parent, T[r].p[v]), &sp, T[src].parent,
                                     &T[r], T[r].parent, T[r].p[v]);
                fwrite(ff, sizeof(real), 3, g);
            }
        }
        if (f) fclose(f);
        if (g) fclose(g);
    }
}

/* ---------------------------------------------------------------- main */
static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int main(int argc, char **argv) {
    static const char *opts[] = {"-debug", "-adapt_area", "-sample_area", "-converge", "-delta_ff", "-write_cycle",
                                 "-zip", "-triangle", "-light", "-o", "-interactive", "-jobs", "-parallel_src"};
    if (argc < 3) {
        fprintf(stderr, "Usage: %s [options] input_file -o output_file\n", argv[0]);
        return 1;
    }
    const char *in = NULL, *out = "./test";
    for (int i = 1; i < argc; i++) {
        int j, has = 0;
        for (j = 0; j < 13; j++)
            if (!strcmp(argv[i], opts[j])) { has = 1; break; }
        if (!has) {
            if (!strcmp(argv[i], "-adaptive")) { variant_adapt = 1; continue; }
            in = argv[i];
            continue;
        }
        int ok = 1, dummy;
        switch (j) {
        case 0: ok = i + 1 < argc && sscanf(argv[++i], "%d", &opt_debug) == 1; break;
        case 1: ok = i + 1 < argc && sscanf(argv[++i], "%f", &AreaLimit) == 1; break;
        case 2: ok = i + 1 < argc && sscanf(argv[++i], "%f", &SampleArea) == 1; break;
        case 3: ok = i + 1 < argc && sscanf(argv[++i], "%f", &ConvergeLimit) == 1; break;
        case 4: ok = i + 1 < argc && sscanf(argv[++i], "%f", &DeltaFFLimit) == 1; break;
        case 5: ok = i + 1 < argc && sscanf(argv[++i], "%d", &WriteIteration) == 1; break;
        case 6: break;
        case 7: ok = i + 1 < argc && sscanf(argv[++i], "%d", &TriangleLimit) == 1; break;
        case 8: ok = i + 1 < argc && sscanf(argv[++i], "%f", &LightScale) == 1; break;
        case 9: ok = i + 1 < argc; if (ok) out = argv[++i]; break;
        case 10: break;
        case 11: ok = i + 1 < argc && sscanf(argv[++i], "%d", &dummy) == 1; break;
        case 12: ok = i + 1 < argc && sscanf(argv[++i], "%d", &ParallelSource) == 1; break;
        }
        if (!ok) { fprintf(stderr, "bad option %s\n", argv[i]); return 1; }
    }
    FILE *fin = in ? fopen(in, "r") : NULL;
    if (!fin) { fprintf(stderr, "File open error::%s\n", in ? in : "(none)"); return 1; }
    double t0 = now_s();
    if (read_scene(fin) != 0) { fprintf(stderr, "parse error\n"); return 1; }
    fclose(fin);
    fprintf(stderr, "[INFO] Read #Triangle %d from input file\n", trinum);
    build_octree();
    double t1 = now_s();
    fprintf(stderr, "[INFO] Init took %f sec. time.\n", t1 - t0);

    const char *trace_path = getenv("RAD_TRACE");
    FILE *trace = trace_path ? fopen(trace_path, "w") : NULL;
    long max_steps = getenv("RAD_MAX_STEPS") ? atol(getenv("RAD_MAX_STEPS")) : -1;

    init_radiosity();
    if (!variant_adapt) pre_partition();
    run_queries();
    double t2 = now_s();
    int loop, steps = 0;
    for (loop = 1;; loop++) {
        if (WriteIteration && loop % WriteIteration == 0) fprintf(stderr, "[INFO] Loop %d BEGIN\n", loop);
        if (max_steps >= 0 && steps >= max_steps) break;
        if (!(variant_adapt ? serial_step(trace) : shoot_step(trace))) break;
        steps++;
        if (WriteIteration && loop % WriteIteration == 0) {
            write_fin(out, loop);
            fprintf(stderr, "[INFO] END Loop. There are %i triangles.\n", trinum);
        }
    }
    double t3 = now_s();
    fprintf(stderr, "[INFO] Complete in #Iterations %d\n", loop);
    write_fin(out, 0);
    if (trace) fclose(trace);
    const char *dump = getenv("RAD_DUMP");
    if (dump) put_dump(dump, steps);
    fprintf(stderr, "[COUNT] rays %lld cells %lld tri_tests %lld se_tests %lld prec %lld loops %lld\n", cnt_rays,
            cnt_cells, cnt_tris, cnt_se, cnt_prec, cnt_loops);
    fprintf(stderr, "[INFO] Shooting took %f sec for %d steps\n", t3 - t2, steps);
    return 0;
}
