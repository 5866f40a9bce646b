/*
 * CPU oracle of the XPBD cloth step -- TEST INFRASTRUCTURE ONLY (see
 * xpbd_oracle.h).  Every function cites the reference lines it restates,
 * relative to native/src/ssbl_xpbd_cuda_abi41.cu ("abi41.cu").
 */
#include "xpbd_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define K_EPS 1.0e-7f
#define NB_SLOTS 32
#define BUCKET_SLOTS 32
#define MAX_PRIM_CELLS 64
#define N_COUNTS 38

enum {
    C_SOFT = 0, C_EXACT = 1, C_EE = 2, C_HARD = 3, C_SELF_CAND = 9, C_SELF_OVF = 10, C_SDF = 11, C_LRA = 12,
    C_WINGS = 13, C_TACK_GUARD = 14, C_BEND_GUARD = 15, C_ISL_CAND = 16, C_ISL_CLUST = 17, C_ISL_REFS = 18,
    C_ISL_APPLIED = 19, C_ISL_GUARD = 20, C_ISL_MAXD = 21, C_F_SEEN = 22, C_F_ACC_VV = 23, C_F_ACC_VT = 24,
    C_F_ACC_EE = 25, C_F_REJ_REST = 26, C_F_REJ_DUP = 27, C_F_REJ_OWN = 28, C_CLUSTERS = 31, C_CLUST_OWNED = 32,
    C_FRICTION = 33, C_DP_CAND = 4, C_DP_CONTACTS = 5, C_TRI_PAIRS = 7, C_DT_CAND = 34, C_DT_REJECT = 37
};

static char g_err[256];
static int set_err(const char* m) {
    snprintf(g_err, sizeof(g_err), "%s", m);
    return 0;
}
const char* oracle_last_error(void) { return g_err; }

int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ------------------------------------------------------------ vectors -- */
typedef struct { float x, y, z; } V3;
static inline V3 v3(float x, float y, float z) { V3 r = {x, y, z}; return r; }
static inline V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 vmul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
/* abi41.cu:625-627: fma(z, fma(y, x*x)) */
static inline float vdot(V3 a, V3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
/* abi41.cu:629-636 */
static inline V3 vcross(V3 a, V3 b) {
    return v3(fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x)));
}
static inline float vlen(V3 a) { return sqrtf(fmaxf(vdot(a, a), 0.0f)); }
static inline float lensq_xyz(V3 d) { return fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z)); }
static inline int vfinite(V3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }
static inline float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }
static V3 normalize_or(V3 v, V3 fb) {
    float l = vlen(v);
    if (!isfinite(l) || l <= K_EPS) return fb;
    return vmul(v, 1.0f / l);
}
/* abi41.cu:951-960 */
static V3 limit_delta(V3 d, float max_len) {
    if (!vfinite(d) || !isfinite(max_len) || max_len <= 0.0f) return v3(0, 0, 0);
    float l = vlen(d);
    if (!isfinite(l) || l <= K_EPS) return v3(0, 0, 0);
    return l > max_len ? vmul(d, max_len / l) : d;
}
/* abi41.cu:654-656 */
static inline int cell_of(float value, float cell) { return (int)floorf(value / fmaxf(cell, K_EPS)); }
/* abi41.cu:658-664 */
static inline unsigned bucket_of(int x, int y, int z, int n) {
    unsigned h = (unsigned)x * 73856093u ^ (unsigned)y * 19349663u ^ (unsigned)z * 83492791u;
    return n > 0 ? (h & (unsigned)(n - 1)) : 0u;
}
/* abi41.cu:1589-1635 */
static V3 closest_on_tri(V3 p, V3 a, V3 b, V3 c) {
    V3 ab = vsub(b, a), ac = vsub(c, a), ap = vsub(p, a);
    float d1 = vdot(ab, ap), d2 = vdot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return a;
    V3 bp = vsub(p, b);
    float d3 = vdot(ab, bp), d4 = vdot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return b;
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return vadd(a, vmul(ab, d1 / fmaxf(d1 - d3, K_EPS)));
    V3 cp = vsub(p, c);
    float d5 = vdot(ab, cp), d6 = vdot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return c;
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return vadd(a, vmul(ac, d2 / fmaxf(d2 - d6, K_EPS)));
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
        return vadd(b, vmul(vsub(c, b), (d4 - d3) / fmaxf((d4 - d3) + (d5 - d6), K_EPS)));
    float denom = 1.0f / fmaxf(va + vb + vc, K_EPS);
    float v = vb * denom, w = vc * denom;
    return vadd(a, vadd(vmul(ab, v), vmul(ac, w)));
}
/* abi41.cu:4588-4614 */
static void barycentric(V3 p, V3 a, V3 b, V3 c, float* wa, float* wb, float* wc) {
    V3 v0 = vsub(b, a), v1 = vsub(c, a), v2 = vsub(p, a);
    float d00 = vdot(v0, v0), d01 = vdot(v0, v1), d11 = vdot(v1, v1), d20 = vdot(v2, v0), d21 = vdot(v2, v1);
    float denom = d00 * d11 - d01 * d01;
    if (fabsf(denom) <= K_EPS) { *wa = *wb = *wc = 1.0f / 3.0f; return; }
    float v = (d11 * d20 - d01 * d21) / denom, w = (d00 * d21 - d01 * d20) / denom;
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    w = fminf(fmaxf(w, 0.0f), 1.0f - v);
    float u = fmaxf(1.0f - v - w, 0.0f);
    float sum = fmaxf(u + v + w, K_EPS);
    *wa = u / sum; *wb = v / sum; *wc = w / sum;
}
/* abi41.cu:5458-5505 */
static void seg_params(V3 p1, V3 q1, V3 p2, V3 q2, float* s, float* t) {
    V3 d1 = vsub(q1, p1), d2 = vsub(q2, p2), r = vsub(p1, p2);
    float a = vdot(d1, d1), e = vdot(d2, d2), f = vdot(d2, r);
    if (a <= K_EPS && e <= K_EPS) { *s = 0; *t = 0; return; }
    if (a <= K_EPS) { *s = 0; *t = clamp01(f / fmaxf(e, K_EPS)); return; }
    float c = vdot(d1, r);
    if (e <= K_EPS) { *t = 0; *s = clamp01(-c / fmaxf(a, K_EPS)); return; }
    float b = vdot(d1, d2), denom = a * e - b * b;
    *s = fabsf(denom) > K_EPS ? clamp01((b * f - c * e) / denom) : 0.0f;
    float tnom = b * (*s) + f;
    if (tnom < 0.0f) { *t = 0; *s = clamp01(-c / fmaxf(a, K_EPS)); }
    else if (tnom > e) { *t = 1; *s = clamp01((b - c) / fmaxf(a, K_EPS)); }
    else *t = tnom / e;
}
static inline long long to_fix(float v) {
    if (!(fabsf(v) < 1.0e6f)) return 0;
    return llrintf(v * 4294967296.0f);
}
static inline float from_fix(long long v) { return (float)v * (1.0f / 4294967296.0f); }

/* ------------------------------------------------------------- solver -- */
/* One set of dynamic colliders: a cloth's own (OracleSolver.own) or a shared
 * scene's (OracleScene.d, with source ids and layers per primitive). */
typedef struct ODyn ODyn;
struct ODyn {
    int dt_n, dt_signed, dt_motion, dt_hashed, dt_nb, dt_large_n, dt_upload, dt_max_occ;
    float dt_cell;
    V3 *dt_tri, *dt_min, *dt_max, *dt_center, *dt_prev_center; float* dt_radius;
    int *dt_cmin, *dt_cmax, *dt_start, *dt_ent, *dt_large, *dt_idx; int dt_idx_n;
    int dp_n, dp_motion, dp_hashed, dp_nb, dp_upload;
    float dp_cell; unsigned long long dp_sig;
    V3 *dp_pos, *dp_prev; float* dp_rad; int *dp_cellc, *dp_start, *dp_ent;
    int *tri_src, *tri_layer, *par_src, *par_layer;
};

struct OracleSolver {
    SsblXpbdConfig cfg;
    SsblXpbdRuntimeColliders col;
    int V, E, T, B, L;
    V3 *pos, *snap, *prev, *vel, *rest;
    float *w, *inv;
    int *sp_off, *sp_other, *sp_side; float* sp_rest;
    int *te_off, *te_other, *te_side; float* te_rest;
    int *bj_off, *bj_other, *bj_side; float* bj_rest;
    int* bends; float* bend_rest; int* bend_colors; int n_bend_colors;
    int* tris; int* edges;
    float* pin_w; V3* pin_t; float* pin_relax; int pin_relax_iter;
    /* static SDF */
    float* sdf; int sdf_ready, sdf_signed, dim[3]; float origin[3], voxel;
    V3* stris; int n_stris;
    /* self collision */
    int self_on; float radius; int vhash, thash, ehash, nvb, ntb, neb; float cell;
    int *vcell, *vb_start, *vb_ent, *tb_start, *tb_ent, *eb_start, *eb_ent, *nb_count, *nb_idx;
    int tb_total, eb_total;
    long long* acc;
    unsigned long long counts[N_COUNTS];
    float max_delta;
    /* hard-stretch optimisation */
    int pcg_on; float strength;
    float *diag, *pinv; V3 *r, *z, *d, *q; float* off; /* off: 4 floats per stretch-CSR entry */
    V3* avg_sum; float* avg_cnt;
    float red[8]; unsigned long long pcg_guard; float pcg_max_delta;
    int* cap_edges; float* cap_rest; int* cap_colors; int n_cap_colors;
    int cap_jacobi; V3* snap_prev; /* caps without a caller colouring (cap_jacobi) */
    /* prediction extras: incident triangles, volume pressure, force fields */
    int *vt_off, *vt_tri;
    int pressure_on; float *p_area, *p_rest;
    float p_strength, p_accel, p_impulse, p_vrest, p_vlen;
    SsblXpbdForceField fields[64]; int nfields;
    /* dynamic colliders: the cloth's own, and an attached shared scene with
     * its source filter */
    ODyn own;
    OracleScene* scene; int gd_mode, gd_src, gd_layer;
    float dyn_sub_dt;
};

enum { R_DAD = 0, R_RZ = 1, R_RZN = 2, R_STATUS = 3, R_INIT = 4, R_ITER = 5 };
static void cnt(OracleSolver* s, int slot) {
#pragma omp atomic
    s->counts[slot] += 1ull;
}
static void cnt_add(OracleSolver* s, int slot, unsigned long long v) {
#pragma omp atomic
    s->counts[slot] += v;
}

static void* xcalloc(size_t n, size_t sz) { return n ? calloc(n, sz) : NULL; }

/* Vertex -> constraint lists in constraint order (each vertex's incident
 * constraints by increasing index; side = 1 when it is the second end). */
static void build_csr(int V, const int* pairs, const float* rest, int n, int** off, int** other, int** side, float** r) {
    *off = (int*)calloc((size_t)V + 1, sizeof(int));
    for (int k = 0; k < n; ++k) {
        int a = pairs[2 * k], b = pairs[2 * k + 1];
        if (a < 0 || b < 0 || a >= V || b >= V || a == b) continue;
        (*off)[a + 1]++; (*off)[b + 1]++;
    }
    for (int i = 0; i < V; ++i) (*off)[i + 1] += (*off)[i];
    int tot = (*off)[V];
    *other = (int*)xcalloc(tot, sizeof(int));
    *side = (int*)xcalloc(tot, sizeof(int));
    *r = (float*)xcalloc(tot, sizeof(float));
    int* cur = (int*)calloc((size_t)V + 1, sizeof(int));
    memcpy(cur, *off, sizeof(int) * (size_t)V);
    for (int k = 0; k < n; ++k) {
        int a = pairs[2 * k], b = pairs[2 * k + 1];
        if (a < 0 || b < 0 || a >= V || b >= V || a == b) continue;
        int ia = cur[a]++, ib = cur[b]++;
        (*other)[ia] = b; (*side)[ia] = 0; (*r)[ia] = rest[k];
        (*other)[ib] = a; (*side)[ib] = 1; (*r)[ib] = rest[k];
    }
    free(cur);
}

static int next_pow2(int v) {
    int r = 1;
    if (v < 1) v = 1;
    while (r < v && r < (1 << 30)) r <<= 1;
    return r;
}

/* -------------------------------------------------------- static SDF -- */
typedef struct { long long x, y, z; int id; } QV;
static int cmp_qv(const void* a, const void* b) {
    const QV* p = (const QV*)a; const QV* q = (const QV*)b;
    if (p->x != q->x) return p->x < q->x ? -1 : 1;
    if (p->y != q->y) return p->y < q->y ? -1 : 1;
    if (p->z != q->z) return p->z < q->z ? -1 : 1;
    return p->id - q->id;
}
static int cmp_u64(const void* a, const void* b) {
    uint64_t p = *(const uint64_t*)a, q = *(const uint64_t*)b;
    return p < q ? -1 : (p > q ? 1 : 0);
}
/* Closed-mesh test: weld on a 1e-6 grid, every edge used exactly twice
 * (abi41.cu:6026-6063). */
static int mesh_closed(const float* tris, int n) {
    if (!tris || n <= 0) return 0;
    int nv = n * 3;
    QV* q = (QV*)malloc(sizeof(QV) * (size_t)nv);
    for (int k = 0; k < nv; ++k) {
        const float* p = tris + 3 * k;
        if (!isfinite(p[0]) || !isfinite(p[1]) || !isfinite(p[2])) { free(q); return 0; }
        q[k].x = llround((double)p[0] * 1000000.0); q[k].y = llround((double)p[1] * 1000000.0);
        q[k].z = llround((double)p[2] * 1000000.0); q[k].id = k;
    }
    qsort(q, (size_t)nv, sizeof(QV), cmp_qv);
    int* weld = (int*)malloc(sizeof(int) * (size_t)nv);
    int uid = -1;
    for (int k = 0; k < nv; ++k) {
        if (k == 0 || q[k].x != q[k - 1].x || q[k].y != q[k - 1].y || q[k].z != q[k - 1].z) ++uid;
        weld[q[k].id] = uid;
    }
    free(q);
    uint64_t* e = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n * 3);
    int ne = 0;
    for (int t = 0; t < n; ++t) {
        int a = weld[3 * t], b = weld[3 * t + 1], c = weld[3 * t + 2];
        if (a == b || b == c || c == a) continue;
        int pr[3][2] = {{a, b}, {b, c}, {c, a}};
        for (int k = 0; k < 3; ++k) {
            unsigned lo = (unsigned)(pr[k][0] < pr[k][1] ? pr[k][0] : pr[k][1]);
            unsigned hi = (unsigned)(pr[k][0] < pr[k][1] ? pr[k][1] : pr[k][0]);
            e[ne++] = ((uint64_t)lo << 32) | hi;
        }
    }
    free(weld);
    if (ne == 0) { free(e); return 0; }
    qsort(e, (size_t)ne, sizeof(uint64_t), cmp_u64);
    int ok = 1;
    for (int k = 0; k < ne;) {
        int j = k;
        while (j < ne && e[j] == e[k]) ++j;
        if (j - k != 2) { ok = 0; break; }
        k = j;
    }
    free(e);
    return ok;
}

/* abi41.cu:1725-1747 */
static int ray_x_hits(V3 p, V3 a, V3 b, V3 c) {
    V3 dir = v3(1, 0, 0), e1 = vsub(b, a), e2 = vsub(c, a), h = vcross(dir, e2);
    float det = vdot(e1, h);
    if (fabsf(det) <= 1.0e-8f) return 0;
    float inv_det = 1.0f / det;
    V3 s = vsub(p, a);
    float u = inv_det * vdot(s, h);
    if (u < -1.0e-5f || u > 1.0f + 1.0e-5f) return 0;
    V3 q = vcross(s, e1);
    float v = inv_det * vdot(dir, q);
    if (v < -1.0e-5f || u + v > 1.0f + 1.0e-5f) return 0;
    return inv_det * vdot(e2, q) > 1.0e-6f;
}

/* Grid sizing abi41.cu:6123-6218, voxel distances abi41.cu:1787-1829. */
static int build_sdf(OracleSolver* s, const float* tris, int n) {
    s->sdf_ready = 0; s->sdf_signed = 0; s->dim[0] = s->dim[1] = s->dim[2] = 0;
    s->origin[0] = s->origin[1] = s->origin[2] = 0.0f; s->voxel = 0.0f;
    s->n_stris = n > 0 ? n : 0;
    if (n <= 0) return 1;
    if (!tris) return set_err("static triangle data is required for SDF build");
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < n * 3; ++k) {
        const float* v = tris + 3 * k;
        if (!isfinite(v[0]) || !isfinite(v[1]) || !isfinite(v[2])) return set_err("static triangle data contains non-finite coordinates");
        for (int a = 0; a < 3; ++a) { lo[a] = fminf(lo[a], v[a]); hi[a] = fmaxf(hi[a], v[a]); }
    }
    const SsblXpbdConfig* c = &s->cfg;
    float voxel = (isfinite(c->static_sdf_voxel_size) && c->static_sdf_voxel_size > 0.0f)
                      ? c->static_sdf_voxel_size : fmaxf(fmaxf(c->collision_margin, 0.0f) * 0.5f, 0.002f);
    int band = c->static_sdf_band_voxels > 0 ? c->static_sdf_band_voxels : 4; if (band < 1) band = 1;
    int max_res = c->static_sdf_max_resolution > 0 ? c->static_sdf_max_resolution : 160; if (max_res < 16) max_res = 16;
    float margin = fmaxf(c->collision_margin, 0.0f);
    float expand = margin + (float)band * voxel + voxel * 2.0f;
    float ext[3];
    for (int a = 0; a < 3; ++a) { lo[a] = lo[a] - expand; hi[a] = hi[a] + expand; ext[a] = fmaxf(hi[a] - lo[a], voxel); }
    float largest = fmaxf(ext[0], fmaxf(ext[1], ext[2]));
    if (largest / voxel + 1.0f > (float)max_res) voxel = largest / (float)(max_res - 1 > 1 ? max_res - 1 : 1);
    voxel = fmaxf(voxel, 1.0e-5f);
    for (int a = 0; a < 3; ++a) {
        int d = (int)ceilf(ext[a] / voxel) + 1;
        if (d < 2) d = 2;
        if (d > max_res) d = max_res;
        s->dim[a] = d; s->origin[a] = lo[a];
    }
    s->voxel = voxel;
    s->sdf_signed = mesh_closed(tris, n);
    long long nvox = (long long)s->dim[0] * s->dim[1] * s->dim[2];
    free(s->sdf); free(s->stris);
    s->sdf = (float*)malloc(sizeof(float) * (size_t)nvox);
    s->stris = (V3*)malloc(sizeof(V3) * (size_t)n * 3);
    for (int k = 0; k < n * 3; ++k) s->stris[k] = v3(tris[3 * k], tris[3 * k + 1], tris[3 * k + 2]);
    const int nx = s->dim[0], ny = s->dim[1];
#pragma omp parallel for schedule(dynamic, 64)
    for (long long vx = 0; vx < nvox; ++vx) {
        int x = (int)(vx % nx), y = (int)((vx / nx) % ny), z = (int)(vx / ((long long)nx * ny));
        V3 p = vadd(v3(s->origin[0], s->origin[1], s->origin[2]), v3((float)x * voxel, (float)y * voxel, (float)z * voxel));
        V3 ray = vadd(p, v3(0.0f, voxel * 1.37e-4f, voxel * 2.11e-4f));
        float best = 3.402823466e+38f;
        int parity = 0;
        for (int t = 0; t < n; ++t) {
            V3 a = s->stris[3 * t], b = s->stris[3 * t + 1], c2 = s->stris[3 * t + 2];
            V3 d = vsub(p, closest_on_tri(p, a, b, c2));
            best = fminf(best, vdot(d, d));
            if (s->sdf_signed && ray_x_hits(ray, a, b, c2)) parity ^= 1;
        }
        float dist = sqrtf(fmaxf(best, 0.0f));
        if (s->sdf_signed && parity) dist = -dist;
        s->sdf[vx] = dist;
    }
    s->sdf_ready = 1;
    return 1;
}

static inline int sdf_idx(const OracleSolver* s, int x, int y, int z) { return (z * s->dim[1] + y) * s->dim[0] + x; }
static inline float lerpf(float a, float b, float t) { return a + (b - a) * t; }
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static float sdf_tri(const OracleSolver* s, float gx, float gy, float gz) {
    int x0 = clampi((int)floorf(gx), 0, s->dim[0] - 1), y0 = clampi((int)floorf(gy), 0, s->dim[1] - 1);
    int z0 = clampi((int)floorf(gz), 0, s->dim[2] - 1);
    int x1 = clampi(x0 + 1, 0, s->dim[0] - 1), y1 = clampi(y0 + 1, 0, s->dim[1] - 1), z1 = clampi(z0 + 1, 0, s->dim[2] - 1);
    float tx = gx - (float)x0, ty = gy - (float)y0, tz = gz - (float)z0;
    const float* g = s->sdf;
    float c0 = lerpf(lerpf(g[sdf_idx(s, x0, y0, z0)], g[sdf_idx(s, x1, y0, z0)], tx),
                     lerpf(g[sdf_idx(s, x0, y1, z0)], g[sdf_idx(s, x1, y1, z0)], tx), ty);
    float c1 = lerpf(lerpf(g[sdf_idx(s, x0, y0, z1)], g[sdf_idx(s, x1, y0, z1)], tx),
                     lerpf(g[sdf_idx(s, x0, y1, z1)], g[sdf_idx(s, x1, y1, z1)], tx), ty);
    return lerpf(c0, c1, tz);
}
/* abi41.cu:1645-1691 */
static int sdf_sample(const OracleSolver* s, V3 p, float* out) {
    if (s->dim[0] < 2 || s->dim[1] < 2 || s->dim[2] < 2 || s->voxel <= 0.0f) return 0;
    float inv = 1.0f / s->voxel;
    float gx = (p.x - s->origin[0]) * inv, gy = (p.y - s->origin[1]) * inv, gz = (p.z - s->origin[2]) * inv;
    if (gx < 0.0f || gy < 0.0f || gz < 0.0f || gx > (float)(s->dim[0] - 1) || gy > (float)(s->dim[1] - 1) || gz > (float)(s->dim[2] - 1))
        return 0;
    *out = sdf_tri(s, gx, gy, gz);
    return isfinite(*out);
}
/* abi41.cu:1693-1723 */
static float sdf_clamped(const OracleSolver* s, V3 p) {
    float inv = 1.0f / fmaxf(s->voxel, K_EPS);
    float gx = fminf(fmaxf((p.x - s->origin[0]) * inv, 0.0f), (float)(s->dim[0] - 1));
    float gy = fminf(fmaxf((p.y - s->origin[1]) * inv, 0.0f), (float)(s->dim[1] - 1));
    float gz = fminf(fmaxf((p.z - s->origin[2]) * inv, 0.0f), (float)(s->dim[2] - 1));
    return sdf_tri(s, gx, gy, gz);
}
/* abi41.cu:1749-1769 */
static V3 nearest_static_normal(const OracleSolver* s, V3 p) {
    V3 best = v3(0, 0, 1);
    float best_sq = 3.402823466e+38f;
    for (int t = 0; t < s->n_stris; ++t) {
        V3 a = s->stris[3 * t], b = s->stris[3 * t + 1], c = s->stris[3 * t + 2];
        V3 d = vsub(p, closest_on_tri(p, a, b, c));
        float dsq = vdot(d, d);
        if (dsq < best_sq) {
            best_sq = dsq;
            best = dsq > K_EPS * K_EPS ? normalize_or(d, best) : normalize_or(vcross(vsub(b, a), vsub(c, a)), best);
        }
    }
    return normalize_or(best, v3(0, 0, 1));
}
/* abi41.cu:1771-1785 */
static V3 sdf_normal(const OracleSolver* s, V3 p) {
    float h = fmaxf(s->voxel, 1.0e-5f);
    float dx = sdf_clamped(s, vadd(p, v3(h, 0, 0))) - sdf_clamped(s, vadd(p, v3(-h, 0, 0)));
    float dy = sdf_clamped(s, vadd(p, v3(0, h, 0))) - sdf_clamped(s, vadd(p, v3(0, -h, 0)));
    float dz = sdf_clamped(s, vadd(p, v3(0, 0, h))) - sdf_clamped(s, vadd(p, v3(0, 0, -h)));
    V3 n = v3(dx, dy, dz);
    float lsq = vdot(n, n);
    if (!isfinite(lsq) || lsq <= 1.0e-12f) return nearest_static_normal(s, p);
    return vmul(n, 1.0f / sqrtf(lsq));
}

/* ------------------------------------------------------ vertex stages -- */
/* abi41.cu:910-949 */
static int contact_response(OracleSolver* s, V3 n, float proxy, V3* vel) {
    if (!vfinite(n) || !vfinite(*vel)) return 0;
    float vn = vdot(*vel, n);
    if (vn < 0.0f) *vel = vsub(*vel, vmul(n, vn));
    int corrected = 0;
    V3 tg = vsub(*vel, vmul(n, vdot(*vel, n)));
    float tl = vlen(tg);
    float damping = clamp01(s->cfg.contact_tangent_damping);
    if (damping > 0.0f && tl > 1.0e-6f) { *vel = vsub(*vel, vmul(tg, damping)); corrected = 1; }
    tg = vsub(*vel, vmul(n, vdot(*vel, n)));
    tl = vlen(tg);
    float fr = fmaxf(s->cfg.contact_friction, 0.0f);
    if (fr > 0.0f && proxy > 0.0f && tl > 1.0e-6f) {
        float drop = fminf(tl, fr * proxy);
        if (drop > 1.0e-7f) { *vel = vsub(*vel, vmul(tg, drop / fmaxf(tl, K_EPS))); corrected = 1; }
    }
    if (corrected) cnt(s, C_FRICTION);
    return corrected;
}

/* ---- force fields (abi41.cu:1262-1558) ----
 * Restated kind by kind; turbulence uses the same lattice hash as the GPU
 * build (an integer mix, not the Blender permutation table). */
static V3 f3a(const float* a) { return v3(a[0], a[1], a[2]); }
static float field_noise(V3 p, int seed, float salt) {
    float x = sinf(p.x * 12.9898f + p.y * 78.233f + p.z * 37.719f + ((float)seed + salt) * 19.191f) * 43758.5453f;
    return (x - floorf(x)) * 2.0f - 1.0f;
}
static int lattice_hash(int i) {
    unsigned h = (unsigned)i * 0x9E3779B1u;
    h ^= h >> 15; h *= 0x85EBCA77u; h ^= h >> 13;
    return (int)(h & 255u);
}
static float noise_grad(int h, float x, float y, float z) {
    h &= 15;
    float u = h < 8 ? x : y, v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}
static float nfade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
static float nlerp(float t, float a, float b) { return a + t * (b - a); }
static float gradient_noise(float x, float y, float z) {
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
    x -= fx; y -= fy; z -= fz;
    float u = nfade(x), v = nfade(y), w = nfade(z);
    int A = lattice_hash(X) + Y, Bq = lattice_hash(X + 1) + Y;
    int AA = lattice_hash(A) + Z, AB = lattice_hash(A + 1) + Z, BA = lattice_hash(Bq) + Z, BB = lattice_hash(Bq + 1) + Z;
    float x0 = nlerp(u, noise_grad(lattice_hash(AA), x, y, z), noise_grad(lattice_hash(BA), x - 1.0f, y, z));
    float x1 = nlerp(u, noise_grad(lattice_hash(AB), x, y - 1.0f, z), noise_grad(lattice_hash(BB), x - 1.0f, y - 1.0f, z));
    float x2 = nlerp(u, noise_grad(lattice_hash(AA + 1), x, y, z - 1.0f), noise_grad(lattice_hash(BA + 1), x - 1.0f, y, z - 1.0f));
    float x3 = nlerp(u, noise_grad(lattice_hash(AB + 1), x, y - 1.0f, z - 1.0f), noise_grad(lattice_hash(BB + 1), x - 1.0f, y - 1.0f, z - 1.0f));
    return nlerp(w, nlerp(v, x0, x1), nlerp(v, x2, x3));
}
static float turbulence3(float size, float x, float y, float z) {
    if (size != 0.0f && isfinite(size)) { float inv = 1.0f / size; x *= inv; y *= inv; z *= inv; }
    float sum = 0.0f, amp = 1.0f, sc = 1.0f;
    for (int o = 0; o < 3; ++o) { sum += (0.5f + 0.5f * gradient_noise(sc * x, sc * y, sc * z)) * amp; amp *= 0.5f; sc *= 2.0f; }
    return sum * (4.0f / 7.0f);
}
static float field_falloff(const SsblXpbdForceField* f, float dist, float rdist) {
    if (!isfinite(dist)) return 0.0f;
    float dmin = fmaxf(f->distance_min, 0.0f), dmax = fmaxf(f->distance_max, 0.0f);
    float rmin = fmaxf(f->radial_min, 0.0f), rmax = fmaxf(f->radial_max, 0.0f);
    if (f->use_max_distance && dmax > 0.0f && dist >= dmax) return 0.0f;
    if (f->use_radial_max && rmax > 0.0f && rdist >= rmax) return 0.0f;
    float k = 1.0f;
    if (f->use_max_distance && dmax > dmin && dist > dmin) k *= clamp01((dmax - dist) / fmaxf(dmax - dmin, K_EPS));
    if (f->use_min_distance && f->falloff_power > 0.0f && dist > dmin) { float r = fmaxf(dmin, 1.0e-4f); k *= powf(r / fmaxf(dist, r), f->falloff_power); }
    if (f->use_radial_max && rmax > rmin && rdist > rmin) k *= clamp01((rmax - rdist) / fmaxf(rmax - rmin, K_EPS));
    if (f->use_radial_min && f->radial_falloff > 0.0f && rdist > rmin) { float r = fmaxf(rmin, 1.0e-4f); k *= powf(r / fmaxf(rdist, r), f->radial_falloff); }
    return isfinite(k) ? k : 0.0f;
}
static V3 cap_field(V3 a) {
    float l = vlen(a);
    if (!isfinite(l) || l <= 5000.0f) return isfinite(l) ? a : v3(0, 0, 0);
    return vmul(a, 5000.0f / fmaxf(l, K_EPS));
}
static V3 with_flow(const SsblXpbdForceField* f, V3 a, V3 vel, float falloff) {
    if (f->type != 6 && f->type != 9) {
        float flow = isfinite(f->flow) ? f->flow : 0.0f;
        if (fabsf(flow) > 1.0e-6f && falloff != 0.0f) a = vadd(a, vmul(vel, -flow * falloff));
    }
    return cap_field(a);
}
static V3 field_accel(const SsblXpbdForceField* f, V3 p, V3 vel, V3 nrm, int has_n) {
    V3 zero = v3(0, 0, 0);
    if (!isfinite(f->strength) || f->strength == 0.0f || f->apply_to_location == 0) return zero;
    V3 d = vsub(p, f3a(f->origin));
    V3 axis = normalize_or(f3a(f->axis), v3(0, 0, 1));
    V3 rd = f->use_2d_force ? vsub(d, vmul(axis, vdot(d, axis))) : d;
    float dist = vlen(d), rdist = vlen(rd);
    float fo = field_falloff(f, dist, rdist);
    float st = f->strength * fo;
    if (st == 0.0f || !isfinite(st)) return zero;
    switch (f->type) {
    case 1: { /* wind */
        if (!has_n) return zero;
        V3 dir = normalize_or(f3a(f->direction), zero);
        float proj = vdot(dir, nrm);
        if (!isfinite(proj) || proj <= 0.0f) return zero;
        float m = st * proj;
        if (f->noise > 0.0f) m *= fmaxf(0.0f, 1.0f + f->noise * field_noise(p, f->seed, 0.0f));
        return with_flow(f, vmul(dir, m), vel, fo);
    }
    case 2: case 5: { /* force, charge */
        V3 sd = f->use_2d_force ? rd : d;
        float sdist = f->use_2d_force ? rdist : dist;
        if (sdist <= 1.0e-6f) return zero;
        float k = st / fmaxf(sdist, K_EPS);
        if (f->type == 5) k /= fmaxf(sdist * sdist, 0.01f);
        return with_flow(f, vmul(sd, k), vel, fo);
    }
    case 3: { /* vortex */
        V3 radial = vsub(d, vmul(axis, vdot(d, axis)));
        if (vdot(radial, radial) <= 1.0e-10f) return zero;
        return with_flow(f, vmul(normalize_or(vcross(axis, radial), zero), st), vel, fo);
    }
    case 6: { /* harmonic */
        float sdist = f->use_2d_force ? rdist : dist;
        V3 sd = f->use_2d_force ? rd : d;
        if (sdist <= 1.0e-6f) return zero;
        V3 u = vmul(sd, 1.0f / fmaxf(sdist, K_EPS));
        float spring = -st * (sdist - fmaxf(f->rest_length, 0.0f));
        float damp = -vdot(vel, u) * fmaxf(f->harmonic_damping, 0.0f) * fabsf(st);
        return with_flow(f, vmul(u, spring + damp), vel, fo);
    }
    case 7: { /* Lennard-Jones */
        if (dist <= 1.0e-6f) return zero;
        V3 u = vmul(d, 1.0f / fmaxf(dist, K_EPS));
        float radius = fmaxf(f->rest_length, fmaxf(f->size, 0.1f));
        float q = fminf(radius / fmaxf(dist, 1.0e-3f), 6.0f);
        float q2 = q * q, q6 = q2 * q2 * q2;
        return with_flow(f, vmul(u, st * (q6 * q6 - q6)), vel, fo);
    }
    case 8: { /* magnet */
        V3 ax = normalize_or(f3a(f->direction), zero);
        return with_flow(f, vmul(vcross(vel, ax), st), vel, fo);
    }
    case 9: { /* drag */
        float speed = vlen(vel);
        if (speed <= 1.0e-6f) return zero;
        float lin = fmaxf(f->linear_drag, 0.0f), quad = fmaxf(f->quadratic_drag, 0.0f);
        if (lin <= 0.0f && quad <= 0.0f) lin = fabsf(st);
        return with_flow(f, vmul(vel, -(lin + quad * speed)), vel, fo);
    }
    case 4: { /* turbulence */
        V3 q = f->use_global_coords ? p : vadd(d, axis);
        V3 n = v3(-1.0f + 2.0f * turbulence3(f->size, q.x, q.y, q.z), -1.0f + 2.0f * turbulence3(f->size, q.y, q.z, q.x),
                  -1.0f + 2.0f * turbulence3(f->size, q.z, q.x, q.y));
        return with_flow(f, vmul(n, st), vel, fo);
    }
    case 10: { /* texture */
        float freq = fmaxf(fmaxf(f->noise, f->texture_nabla), 0.25f);
        if (f->size > 1.0e-6f) freq = fmaxf(freq, 1.0f / f->size);
        V3 q = vmul(d, freq);
        V3 n = v3(field_noise(q, f->seed, 0.0f), field_noise(q, f->seed, 7.0f), field_noise(q, f->seed, 13.0f));
        return with_flow(f, vmul(n, st), vel, fo);
    }
    default: return zero;
    }
}

/* Vertex normal from the incident triangles at the substep-start positions
 * (abi41.cu:1213-1261; IEEE 1/sqrt). */
static int vertex_normal(const OracleSolver* s, int i, const V3* x, V3* out) {
    if (!s->vt_off) return 0;
    int b = s->vt_off[i], e = s->vt_off[i + 1];
    if (e <= b) return 0;
    V3 acc = v3(0, 0, 0);
    for (int k = b; k < e; ++k) {
        int t = s->vt_tri[k];
        if (t < 0 || t >= s->T) continue;
        const int* tr = s->tris + 3 * t;
        if (tr[0] < 0 || tr[1] < 0 || tr[2] < 0 || tr[0] >= s->V || tr[1] >= s->V || tr[2] >= s->V) continue;
        V3 n = vcross(vsub(x[tr[1]], x[tr[0]]), vsub(x[tr[2]], x[tr[0]]));
        float l2 = vdot(n, n);
        if (!isfinite(l2) || l2 <= 1.0e-10f) continue;
        acc = vadd(acc, vmul(n, 1.0f / sqrtf(l2)));
    }
    float a2 = vdot(acc, acc);
    if (!isfinite(a2) || a2 <= 1.0e-10f) return 0;
    *out = vmul(acc, 1.0f / sqrtf(a2));
    return 1;
}

/* abi41.cu:1869-1925: gravity, volume pressure, force fields, damping,
 * pressure speed trims; normals from the substep-start positions. */
static void integrate_all(OracleSolver* s, float dt) {
    const int needs_normal = s->pressure_on || s->nfields > 0;
#pragma omp parallel for
    for (int i = 0; i < s->V; ++i) s->prev[i] = s->pos[i];
#pragma omp parallel for
    for (int i = 0; i < s->V; ++i) {
        if (!(s->w[i] > 0.0f)) { s->vel[i] = v3(0, 0, 0); s->pos[i] = s->rest[i]; continue; }
        V3 nrm = v3(0, 0, 0);
        int has_n = needs_normal && vertex_normal(s, i, s->prev, &nrm);
        V3 a = vadd(v3(s->cfg.gravity[0], s->cfg.gravity[1], s->cfg.gravity[2]), v3(0, 0, 0));
        int pressure = s->pressure_on && has_n;
        float area = pressure ? s->p_area[i] : 0.0f;
        if (pressure && isfinite(area) && area > 0.0f) a = vadd(a, vmul(nrm, s->p_strength * s->p_accel * area * s->inv[i]));
        if (s->nfields > 0) {
            V3 fa = v3(0, 0, 0);
            for (int k = 0; k < s->nfields; ++k) fa = vadd(fa, field_accel(&s->fields[k], s->prev[i], s->vel[i], nrm, has_n));
            a = vadd(a, cap_field(fa));
        }
        V3 vel = vadd(s->vel[i], vmul(a, dt));
        vel = vmul(vel, s->cfg.damping);
        if (pressure) {
            float rest = s->p_rest[i];
            if (isfinite(rest) && rest > K_EPS && isfinite(dt) && dt > K_EPS) {
                float pa = fmaxf(s->p_strength, 0.0f) * fmaxf(s->p_accel, 0.0f) * fmaxf(area, 0.0f) * fmaxf(s->inv[i], 0.0f);
                float maxd = fmaxf(rest * fmaxf(s->p_impulse, 0.0f), 1.0e-7f);
                float del = pa * dt * dt;
                if (isfinite(del) && del > maxd) vel = vsub(vel, vmul(nrm, (del - maxd) / dt));
                float vr = fmaxf(rest, fmaxf(s->p_vlen, 0.0f));
                float maxo = fmaxf(vr * fmaxf(s->p_vrest, 0.0f) / dt, 1.0e-6f);
                float out = vdot(vel, nrm);
                if (isfinite(out) && out > maxo) vel = vsub(vel, vmul(nrm, out - maxo));
            }
        }
        s->vel[i] = vel;
        s->pos[i] = vadd(s->prev[i], vmul(vel, dt));
    }
}

/* abi41.cu:3466-3509; pins kept per vertex (last entry of a vertex wins) */
static void pin_all(OracleSolver* s, float dt) {
#pragma omp parallel for
    for (int i = 0; i < s->V; ++i) {
        float wgt = s->pin_w[i];
        if (!isfinite(wgt) || wgt < 0.05f) continue;
        V3 target = s->pin_t[i];
        if (wgt >= 0.75f || s->inv[i] <= 0.0f) { s->pos[i] = target; s->prev[i] = target; s->vel[i] = v3(0, 0, 0); continue; }
        float relax = s->pin_relax[i];
        if (relax <= 0.0f) continue;
        V3 corrected = vadd(s->pos[i], vmul(vsub(target, s->pos[i]), relax));
        V3 damped = vmul(s->vel[i], fmaxf(1.0f - relax, 0.0f));
        s->pos[i] = corrected;
        s->prev[i] = vsub(corrected, vmul(damped, fmaxf(dt, K_EPS)));
        s->vel[i] = damped;
    }
}

/* abi41.cu:1927-1980 as a snapshot-Jacobi gather */
static void spring_all(OracleSolver* s, float dt) {
    memcpy(s->snap, s->pos, sizeof(V3) * (size_t)s->V);
    const float alpha = fmaxf(s->cfg.stretch_compliance, 0.0f) / fmaxf(dt * dt, K_EPS);
#pragma omp parallel for schedule(static)
    for (int v = 0; v < s->V; ++v) {
        V3 dp = s->snap[v], dprev = s->prev[v];
        for (int k = s->sp_off[v]; k < s->sp_off[v + 1]; ++k) {
            int o = s->sp_other[k], is_j = s->sp_side[k];
            int i = is_j ? o : v, j = is_j ? v : o;
            float wi = s->w[i], wj = s->w[j], weight = wi + wj;
            if (weight <= 0.0f) continue;
            float rest = s->sp_rest[k];
            V3 delta = vsub(s->snap[j], s->snap[i]);
            float len = sqrtf(fmaxf(vdot(delta, delta), K_EPS));
            float c = len - rest;
            float dl = -c / (weight + alpha);
            V3 corr = vmul(delta, 0.18f * dl / fmaxf(len, K_EPS));
            float cl = sqrtf(fmaxf(vdot(corr, corr), 0.0f));
            float mc = fmaxf(0.0025f, fminf(fmaxf(rest, 0.0f) * 0.10f, 0.025f));
            if (cl > mc) { corr = vmul(corr, mc / fmaxf(cl, K_EPS)); if (!is_j) cnt(s, C_HARD); }
            float wself = is_j ? wj : wi;
            if (wself > 0.0f) {
                V3 d = is_j ? vmul(corr, wj) : vmul(corr, -wi);
                dp = vadd(dp, d);
                if (c > 0.0f) dprev = vadd(dprev, vmul(d, 0.08f));
            }
        }
        s->pos[v] = dp;
        s->prev[v] = dprev;
    }
}

/* abi41.cu:2710-2803 as a snapshot gather over each vertex's tethers */
static void tether_all(OracleSolver* s, float dt) {
    memcpy(s->snap, s->pos, sizeof(V3) * (size_t)s->V);
    const float th = s->cfg.cloth_thickness;
#pragma omp parallel for schedule(static)
    for (int v = 0; v < s->V; ++v) {
        V3 dp = s->snap[v], dprev = s->prev[v];
        for (int k = s->te_off[v]; k < s->te_off[v + 1]; ++k) {
            int o = s->te_other[k], is_j = s->te_side[k], counter = !is_j;
            int i = is_j ? o : v, j = is_j ? v : o;
            float wi = s->w[i], wj = s->w[j], weight = wi + wj;
            if (!isfinite(weight) || weight <= 0.0f) { if (counter) cnt(s, C_TACK_GUARD); continue; }
            V3 pi = s->snap[i], pj = s->snap[j];
            if (!vfinite(pi) || !vfinite(pj)) { if (counter) cnt(s, C_TACK_GUARD); continue; }
            V3 dx = vsub(pj, pi);
            float lsq = lensq_xyz(dx), rest = s->te_rest[k];
            if (!isfinite(lsq) || lsq <= 1.0e-10f || !isfinite(rest) || rest <= K_EPS) { if (counter) cnt(s, C_TACK_GUARD); continue; }
            float inv_len = 1.0f / sqrtf(lsq), len = lsq * inv_len, stretch = len - rest;
            if (!isfinite(stretch) || stretch <= 0.0f) continue;
            dx = vmul(dx, inv_len);
            float bc = fmaxf(s->cfg.lra_compliance, 1.0e-12f);
            float stiff = (1.0f / bc) * 500000.0f;
            float alpha = (bc / 500000.0f) / fmaxf(dt * dt, K_EPS);
            float sw = stiff / fmaxf(stiff + 500000.0f, 1.0f);
            float dl = -stretch / fmaxf(weight + alpha, K_EPS);
            V3 corr = vmul(dx, 0.35f * sw * dl);
            if (!vfinite(corr)) { if (counter) cnt(s, C_TACK_GUARD); continue; }
            float cl = vlen(corr);
            float mc = fmaxf(5.0e-4f, fminf(fmaxf(rest, th) * 0.20f, 0.035f));
            if (!isfinite(cl) || cl <= 0.0f) continue;
            if (cl > mc) { corr = vmul(corr, mc / fmaxf(cl, K_EPS)); if (counter) cnt(s, C_TACK_GUARD); }
            int has_th = th > 0.0f;
            float cap = has_th ? 0.0025f : 0.012f;
            float rest_limit = fmaxf(rest, 0.0f) * (has_th ? 0.02f : 0.08f);
            float th_limit = has_th ? th * 0.12f : cap;
            float applied = fmaxf(5.0e-4f, fminf(fminf(rest_limit, th_limit), cap));
            if (is_j) {
                if (wj > 0.0f) { V3 d = limit_delta(vmul(corr, wj / fmaxf(weight, K_EPS)), applied); dp = vadd(dp, d); dprev = vadd(dprev, vmul(d, 0.32f)); }
            } else if (wi > 0.0f) {
                V3 d = limit_delta(vmul(corr, -wi / fmaxf(weight, K_EPS)), applied); dp = vadd(dp, d); dprev = vadd(dprev, vmul(d, 0.32f));
            }
            if (counter) cnt(s, C_LRA);
        }
        s->pos[v] = dp;
        s->prev[v] = dprev;
    }
}

/* Bend correction shared by the colour kernel and the Jacobi form
 * (abi41.cu:2805-2970). Returns 1 when applied; *guard as the reference counts. */
static int bend_corr(OracleSolver* s, float dt, V3 pi, V3 pj, float wi, float wj, float rest, V3* out, int* guard) {
    *guard = 0;
    float weight = wi + wj;
    if (!isfinite(weight) || weight <= 0.0f) return 0;
    if (!isfinite(rest) || rest <= K_EPS) { *guard = 1; return 0; }
    if (!vfinite(pi) || !vfinite(pj)) { *guard = 1; return 0; }
    V3 delta = vsub(pj, pi);
    float lsq = lensq_xyz(delta);
    if (!isfinite(lsq) || lsq <= 1.0e-10f) { *guard = 1; return 0; }
    float inv_len = 1.0f / sqrtf(lsq), len = lsq * inv_len, c = len - rest;
    if (!isfinite(c) || fabsf(c) <= 1.0e-6f) return 0;
    float alpha = fmaxf(s->cfg.bend_compliance, 0.0f) / fmaxf(dt * dt, K_EPS);
    float dl = -c / fmaxf(weight + alpha, K_EPS);
    V3 corr = vmul(delta, 0.10f * dl * inv_len);
    if (!vfinite(corr)) { *guard = 1; return 0; }
    float cl = vlen(corr);
    float mc = fmaxf(2.5e-4f, fminf(fmaxf(rest, s->cfg.cloth_thickness) * 0.08f, 0.020f));
    if (!isfinite(cl) || cl <= 0.0f) return 0;
    if (cl > mc) { corr = vmul(corr, mc / fmaxf(cl, K_EPS)); *guard = 1; }
    *out = corr;
    return 1;
}

/* abi41.cu:2886-2970, per colour in order, in place */
static void bends_by_color(OracleSolver* s, float dt) {
    for (int k = 0; k + 1 < s->n_bend_colors + 1 && k < s->n_bend_colors; ++k) {
        int start = s->bend_colors[k], count = s->bend_colors[k + 1] - start;
#pragma omp parallel for
        for (int l = 0; l < count; ++l) {
            int b = start + l;
            if (b < 0 || b >= s->B) { cnt(s, C_BEND_GUARD); continue; }
            int i = s->bends[2 * b], j = s->bends[2 * b + 1];
            if (i < 0 || j < 0 || i >= s->V || j >= s->V || i == j) { cnt(s, C_BEND_GUARD); continue; }
            V3 corr; int guard;
            int ok = bend_corr(s, dt, s->pos[i], s->pos[j], s->w[i], s->w[j], s->bend_rest[b], &corr, &guard);
            if (guard) cnt(s, C_BEND_GUARD);
            if (!ok) continue;
            float wi = s->w[i], wj = s->w[j];
            if (wi > 0.0f) { V3 d = vmul(corr, -wi); s->pos[i] = vadd(s->pos[i], d); s->prev[i] = vadd(s->prev[i], vmul(d, 0.06f)); }
            if (wj > 0.0f) { V3 d = vmul(corr, wj); s->pos[j] = vadd(s->pos[j], d); s->prev[j] = vadd(s->prev[j], vmul(d, 0.06f)); }
            cnt(s, C_WINGS);
        }
    }
}

/* abi41.cu:2805-2884: all bends at once (no colours) as a snapshot gather */
static void bends_jacobi(OracleSolver* s, float dt) {
    memcpy(s->snap, s->pos, sizeof(V3) * (size_t)s->V);
#pragma omp parallel for
    for (int v = 0; v < s->V; ++v) {
        V3 dp = s->snap[v], dprev = s->prev[v];
        for (int k = s->bj_off[v]; k < s->bj_off[v + 1]; ++k) {
            int o = s->bj_other[k], is_j = s->bj_side[k];
            int i = is_j ? o : v, j = is_j ? v : o;
            V3 corr; int guard;
            int ok = bend_corr(s, dt, s->snap[i], s->snap[j], s->w[i], s->w[j], s->bj_rest[k], &corr, &guard);
            if (!is_j) { if (guard) cnt(s, C_BEND_GUARD); if (ok) cnt(s, C_WINGS); }
            if (!ok) continue;
            float wself = is_j ? s->w[j] : s->w[i];
            if (wself > 0.0f) {
                V3 d = is_j ? vmul(corr, s->w[j]) : vmul(corr, -s->w[i]);
                dp = vadd(dp, d); dprev = vadd(dprev, vmul(d, 0.06f));
            }
        }
        s->pos[v] = dp; s->prev[v] = dprev;
    }
}

/* abi41.cu:3511-3590 */
static void analytic_all(OracleSolver* s, float dt) {
    const SsblXpbdRuntimeColliders* c = &s->col;
    const float margin = fmaxf(s->cfg.collision_margin, 0.0f), sdt = fmaxf(dt, K_EPS);
#pragma omp parallel for
    for (int i = 0; i < s->V; ++i) {
        if (s->inv[i] <= 0.0f) continue;
        V3 p = s->pos[i], vel = s->vel[i];
        int hit = 0;
        if (c->use_ground && p.z < c->ground_height + margin) {
            float tz = c->ground_height + margin, pen = tz - p.z;
            V3 n = v3(0, 0, 1);
            float inward = fmaxf(-vdot(vel, n), 0.0f);
            p.z = tz;
            contact_response(s, n, inward + pen / sdt, &vel);
            hit = 1;
        }
        if (c->use_sphere && c->sphere_radius > 0.0f) {
            V3 ctr = v3(c->sphere_center[0], c->sphere_center[1], c->sphere_center[2]);
            V3 d = vsub(p, ctr);
            float dist = sqrtf(fmaxf(vdot(d, d), K_EPS)), target = c->sphere_radius + margin;
            if (dist < target) {
                V3 n = dist > K_EPS ? vmul(d, 1.0f / dist) : v3(0, 0, 1);
                float pen = target - dist, inward = fmaxf(-vdot(vel, n), 0.0f);
                p = vadd(ctr, vmul(n, target));
                contact_response(s, n, inward + pen / sdt, &vel);
                hit = 1;
            }
        }
        if (c->use_wall) {
            V3 o = v3(c->wall_origin[0], c->wall_origin[1], c->wall_origin[2]);
            V3 n = v3(c->wall_normal[0], c->wall_normal[1], c->wall_normal[2]);
            float nl = sqrtf(fmaxf(vdot(n, n), K_EPS));
            n = vmul(n, 1.0f / nl);
            float gap = vdot(vsub(p, o), n);
            if (gap < margin) {
                float pen = margin - gap, inward = fmaxf(-vdot(vel, n), 0.0f);
                p = vadd(p, vmul(n, margin - gap));
                contact_response(s, n, inward + pen / sdt, &vel);
                hit = 1;
            }
        }
        s->pos[i] = p;
        if (hit) { s->vel[i] = vel; s->prev[i] = vsub(p, vmul(vel, sdt)); }
    }
}

/* abi41.cu:1831-1867 */
static void sdf_all(OracleSolver* s, float dt) {
    const float margin = fmaxf(s->cfg.collision_margin, 0.0f);
    if (margin <= 0.0f) return;
#pragma omp parallel for
    for (int i = 0; i < s->V; ++i) {
        if (s->inv[i] <= 0.0f) continue;
        V3 p = s->pos[i];
        float d = 0.0f;
        if (!sdf_sample(s, p, &d) || d >= margin) continue;
        V3 n = sdf_normal(s, p);
        if (!vfinite(n)) continue;
        float pen = margin - d;
        if (!isfinite(pen) || pen <= 0.0f) continue;
        V3 corrected = vadd(p, vmul(n, pen)), vel = s->vel[i];
        float inward = fmaxf(-vdot(vel, n), 0.0f);
        contact_response(s, n, inward + pen / fmaxf(dt, K_EPS), &vel);
        s->pos[i] = corrected; s->vel[i] = vel; s->prev[i] = vsub(corrected, vmul(vel, fmaxf(dt, K_EPS)));
        cnt(s, C_SDF);
    }
}

/* abi41.cu:5846-5884 */
static void velocity_all(OracleSolver* s, float dt) {
    const float sdt = fmaxf(dt, K_EPS);
    const float max_delta = fmaxf(2.0e-4f, fmaxf(s->cfg.cloth_thickness, 0.0f) * 0.35f), max_speed = max_delta / sdt;
#pragma omp parallel for
    for (int i = 0; i < s->V; ++i) {
        if (!(s->w[i] > 0.0f)) { s->vel[i] = v3(0, 0, 0); continue; }
        V3 measured = vmul(vsub(s->pos[i], s->prev[i]), 1.0f / sdt), base = s->vel[i];
        if (!vfinite(measured) || !vfinite(base)) { s->vel[i] = v3(0, 0, 0); continue; }
        V3 proj = vsub(measured, base);
        float pdb = vdot(proj, base);
        float scale = (isfinite(pdb) && pdb > 0.0f) ? 0.9f : 1.0f;
        V3 fb = vmul(proj, scale);
        float fs = vlen(fb);
        if (scale < 1.0f && isfinite(fs) && fs > max_speed && fs > K_EPS) fb = vmul(fb, max_speed / fs);
        if (!vfinite(fb)) fb = v3(0, 0, 0);
        s->vel[i] = vadd(base, fb);
    }
}

/* ----------------------------------------------------- self collision -- */
static int fast_mode(const OracleSolver* s) { return s->cfg.self_collision_mode == 1; }

static void accumulate(OracleSolver* s, int i, V3 d) {
    if (i < 0 || i >= s->V || !(s->inv[i] > 0.0f)) return;
    long long* a = s->acc + 4 * (size_t)i;
    long long x = to_fix(d.x), y = to_fix(d.y), z = to_fix(d.z);
#pragma omp atomic
    a[0] += x;
#pragma omp atomic
    a[1] += y;
#pragma omp atomic
    a[2] += z;
#pragma omp atomic
    a[3] += 1;
}

/* abi41.cu:733-760 */
static int normal_bucket(float v) { return v > 0.45f ? 2 : (v < -0.45f ? 0 : 1); }
static unsigned cluster_key(int type, V3 p, V3 n, float cell) {
    float c = fmaxf(cell, 1.0e-3f);
    unsigned key = bucket_of(cell_of(p.x, c), cell_of(p.y, c), cell_of(p.z, c), 1 << 20);
    unsigned nk = (unsigned)normal_bucket(n.x) | ((unsigned)normal_bucket(n.y) << 2) | ((unsigned)normal_bucket(n.z) << 4);
    key ^= nk * 2654435761u;
    key ^= (unsigned)(type + 1) * 2246822519u;
    return key;
}
typedef struct { unsigned keys[16]; unsigned char counts[16]; int n; } Clusters;
typedef struct { int ids[64]; int n; } Seen;
static int accept_slot(int type) { return type == 0 ? C_F_ACC_VV : (type == 1 ? C_F_ACC_VT : C_F_ACC_EE); }
/* abi41.cu:793-832 */
static int local_accept(OracleSolver* s, int type, unsigned key, Clusters* cl) {
    if (!fast_mode(s)) return 1;
    if (cl) {
        int n = cl->n < 16 ? cl->n : 16;
        for (int i = 0; i < n; ++i)
            if (cl->keys[i] == key) {
                if (cl->counts[i] >= 1) { cnt(s, C_F_REJ_OWN); return 0; }
                cl->counts[i] += 1; cnt(s, C_CLUST_OWNED); cnt(s, accept_slot(type)); return 1;
            }
        if (cl->n >= 16) { cnt(s, C_F_REJ_OWN); return 0; }
        cl->keys[cl->n] = key; cl->counts[cl->n] = 1; cl->n += 1;
        cnt(s, C_CLUSTERS); cnt(s, C_CLUST_OWNED);
    }
    cnt(s, accept_slot(type));
    return 1;
}
/* abi41.cu:762-791 */
static int note_seen(OracleSolver* s, int key, Seen* seen) {
    if (!fast_mode(s)) return 1;
    cnt(s, C_F_SEEN);
    if (!seen) return 1;
    int lim = seen->n < 64 ? seen->n : 64;
    for (int i = 0; i < lim; ++i) if (seen->ids[i] == key) { cnt(s, C_F_REJ_DUP); return 0; }
    if (seen->n >= 64) { cnt(s, C_SELF_OVF); cnt(s, C_F_REJ_OWN); return 0; }
    seen->ids[seen->n++] = key;
    return 1;
}
static void filter_count(OracleSolver* s, int slot) { if (fast_mode(s)) cnt(s, slot); }

static int tri_ok(const OracleSolver* s, const int* t) {
    return t[0] >= 0 && t[1] >= 0 && t[2] >= 0 && t[0] < s->V && t[1] < s->V && t[2] < s->V && t[0] != t[1] && t[1] != t[2] && t[0] != t[2];
}
static int edge_ok(const OracleSolver* s, const int* e) { return e[0] >= 0 && e[1] >= 0 && e[0] < s->V && e[1] < s->V && e[0] != e[1]; }

/* Cell box of a primitive with the 64-cell guard (abi41.cu:871-900). */
static void prim_cells(OracleSolver* s, V3 lo, V3 hi, V3 fb, int* r, int count_guard) {
    float c = s->cell;
    r[0] = cell_of(lo.x, c); r[1] = cell_of(hi.x, c); r[2] = cell_of(lo.y, c); r[3] = cell_of(hi.y, c);
    r[4] = cell_of(lo.z, c); r[5] = cell_of(hi.z, c);
    long long sx = (long long)r[1] - r[0] + 1, sy = (long long)r[3] - r[2] + 1, sz = (long long)r[5] - r[4] + 1;
    if (sx <= 0 || sy <= 0 || sz <= 0) return;
    if (sx * sy * sz <= MAX_PRIM_CELLS) return;
    int fx = cell_of(fb.x, c), fy = cell_of(fb.y, c), fz = cell_of(fb.z, c);
    r[0] = r[1] = fx; r[2] = r[3] = fy; r[4] = r[5] = fz;
    if (count_guard) cnt(s, C_SELF_OVF);
}
/* abi41.cu:4632-4694 / 5532-5593: cell box of triangle or edge k */
static int tri_box(OracleSolver* s, int k, int* r, int count_guard) {
    const int* t = s->tris + 3 * k;
    if (!tri_ok(s, t)) return 0;
    V3 a = s->pos[t[0]], b = s->pos[t[1]], c = s->pos[t[2]];
    float m = s->radius * 1.8f;
    V3 lo = v3(fminf(a.x, fminf(b.x, c.x)) - m, fminf(a.y, fminf(b.y, c.y)) - m, fminf(a.z, fminf(b.z, c.z)) - m);
    V3 hi = v3(fmaxf(a.x, fmaxf(b.x, c.x)) + m, fmaxf(a.y, fmaxf(b.y, c.y)) + m, fmaxf(a.z, fmaxf(b.z, c.z)) + m);
    prim_cells(s, lo, hi, vmul(vadd(vadd(a, b), c), 1.0f / 3.0f), r, count_guard);
    return 1;
}
static int edge_box(OracleSolver* s, int k, int* r, int count_guard) {
    const int* e = s->edges + 2 * k;
    if (!edge_ok(s, e)) return 0;
    V3 a = s->pos[e[0]], b = s->pos[e[1]];
    float m = s->radius * 1.8f;
    V3 lo = v3(fminf(a.x, b.x) - m, fminf(a.y, b.y) - m, fminf(a.z, b.z) - m);
    V3 hi = v3(fmaxf(a.x, b.x) + m, fmaxf(a.y, b.y) + m, fmaxf(a.z, b.z) + m);
    prim_cells(s, lo, hi, vmul(vadd(a, b), 0.5f), r, count_guard);
    return 1;
}

/* Counting sort by bucket id; entries of a bucket in increasing primitive
 * order; per-bucket overflow counted beyond 32 like the reference's slot
 * insertion (abi41.cu:4550-4575, 4632-4694, 5532-5593). */
static void hash_vertices(OracleSolver* s) {
    int nb = s->nvb;
    int* count = (int*)calloc((size_t)nb, sizeof(int));
    for (int i = 0; i < s->V; ++i) {
        V3 p = s->pos[i];
        int cx = cell_of(p.x, s->cell), cy = cell_of(p.y, s->cell), cz = cell_of(p.z, s->cell);
        int b = (int)bucket_of(cx, cy, cz, nb);
        s->vcell[4 * i] = cx; s->vcell[4 * i + 1] = cy; s->vcell[4 * i + 2] = cz; s->vcell[4 * i + 3] = b;
        if (count[b]++ >= BUCKET_SLOTS) cnt(s, C_SELF_OVF);
    }
    s->vb_start[0] = 0;
    for (int b = 0; b < nb; ++b) s->vb_start[b + 1] = s->vb_start[b] + count[b];
    memcpy(count, s->vb_start, sizeof(int) * (size_t)nb);
    for (int i = 0; i < s->V; ++i) s->vb_ent[count[s->vcell[4 * i + 3]]++] = i;
    free(count);
}
static void hash_prims(OracleSolver* s, int tri) {
    int n = tri ? s->T : s->E, nb = tri ? s->ntb : s->neb;
    int* start = tri ? s->tb_start : s->eb_start;
    int* ent = tri ? s->tb_ent : s->eb_ent;
    int* count = (int*)calloc((size_t)nb, sizeof(int));
    int r[6];
    for (int pass = 0; pass < 2; ++pass) {
        for (int k = 0; k < n; ++k) {
            int ok = tri ? tri_box(s, k, r, pass == 0) : edge_box(s, k, r, pass == 0);
            if (!ok) continue;
            for (int z = r[4]; z <= r[5]; ++z)
                for (int y = r[2]; y <= r[3]; ++y)
                    for (int x = r[0]; x <= r[1]; ++x) {
                        int b = (int)bucket_of(x, y, z, nb);
                        if (pass == 0) { if (count[b]++ >= BUCKET_SLOTS) cnt(s, C_SELF_OVF); }
                        else ent[count[b]++] = k;
                    }
        }
        if (pass == 0) {
            start[0] = 0;
            for (int b = 0; b < nb; ++b) start[b + 1] = start[b] + count[b];
            memcpy(count, start, sizeof(int) * (size_t)nb);
        }
    }
    if (tri) s->tb_total = start[nb]; else s->eb_total = start[nb];
    free(count);
}

/* abi41.cu:4696-4717 */
static int vv_valid(OracleSolver* s, int src, int other, float target, float onset) {
    if (src < 0 || other < 0 || src >= s->V || other >= s->V || src == other || target <= 0.0f || onset <= target || !(s->inv[src] > 0.0f))
        return 0;
    V3 rd = vsub(s->rest[src], s->rest[other]);
    float skip = fmaxf(onset * 1.25f, target * 2.5f);
    if (vdot(rd, rd) < skip * skip) return 0;
    V3 cd = vsub(s->pos[src], s->pos[other]), pd = vsub(s->prev[src], s->prev[other]);
    return vdot(cd, cd) < onset * onset || vdot(pd, pd) < onset * onset;
}
/* abi41.cu:4738-4812 */
static void neighbors_all(OracleSolver* s) {
    const float target = s->radius, onset = fmaxf(target * 1.8f, target + K_EPS);
#pragma omp parallel for schedule(dynamic, 256)
    for (int src = 0; src < s->V; ++src) {
        if (target <= 0.0f) { s->nb_count[src] = 0; continue; }
        int acc = 0;
        if (s->vhash) {
            V3 p = s->pos[src];
            int cx = cell_of(p.x, s->cell), cy = cell_of(p.y, s->cell), cz = cell_of(p.z, s->cell);
            for (int dz = -1; dz <= 1 && acc < NB_SLOTS; ++dz)
                for (int dy = -1; dy <= 1 && acc < NB_SLOTS; ++dy)
                    for (int dx = -1; dx <= 1 && acc < NB_SLOTS; ++dx) {
                        int qx = cx + dx, qy = cy + dy, qz = cz + dz;
                        int b = (int)bucket_of(qx, qy, qz, s->nvb), st = s->vb_start[b];
                        int lim = s->vb_start[b + 1] - st; if (lim > BUCKET_SLOTS) lim = BUCKET_SLOTS;
                        for (int k = 0; k < lim && acc < NB_SLOTS; ++k) {
                            int o = s->vb_ent[st + k];
                            if (s->vcell[4 * o] != qx || s->vcell[4 * o + 1] != qy || s->vcell[4 * o + 2] != qz || !vv_valid(s, src, o, target, onset)) continue;
                            s->nb_idx[src * NB_SLOTS + acc++] = o;
                        }
                    }
        } else {
            for (int o = 0; o < s->V && acc < NB_SLOTS; ++o)
                if (vv_valid(s, src, o, target, onset)) s->nb_idx[src * NB_SLOTS + acc++] = o;
        }
        if (acc >= NB_SLOTS) cnt(s, C_SELF_OVF);
        s->nb_count[src] = acc;
    }
}

/* abi41.cu:4816-4951 */
static void vv_all(OracleSolver* s) {
    const float target = s->radius;
#pragma omp parallel for schedule(dynamic, 256)
    for (int src = 0; src < s->V; ++src) {
        if (!(s->inv[src] > 0.0f)) continue;
        int count = s->nb_count[src];
        if (count == 0) continue;
        V3 pc = s->pos[src], pp = s->prev[src];
        float r_self = target * 0.5f;
        int lim = count < NB_SLOTS ? count : NB_SLOTS;
        Clusters cl; cl.n = 0;
        for (int n = 0; n < lim; ++n) {
            int o = s->nb_idx[src * NB_SLOTS + n];
            if (o < 0 || o >= s->V || o == src) continue;
            if (fast_mode(s)) cnt(s, C_F_SEEN); else cnt(s, C_SELF_CAND);
            V3 qc = s->pos[o], qp = s->prev[o];
            float th = r_self + target * 0.5f;
            if (th <= 0.0f) continue;
            float scale = !(s->inv[o] > 0.0f) ? 1.0f : 0.5f;
            V3 resp = v3(0, 0, 0);
            int hit = 0;
            V3 dref = vsub(pp, qp);
            float cc = vdot(dref, dref) - th * th;
            V3 rel = vsub(vsub(pc, pp), vsub(qc, qp));
            float a = vdot(rel, rel), b = vdot(dref, rel);
            if (cc >= 0.0f && b < 0.0f && a > 1.0e-5f) {
                float disc = b * b - a * cc;
                if (disc >= 0.0f) {
                    float t = (-b - sqrtf(disc)) / a;
                    if (t > 0.0f && t <= 1.0f) {
                        float sg = 1.0f - t;
                        V3 ph = vadd(vmul(pp, sg), vmul(pc, t)), qh = vadd(vmul(qp, sg), vmul(qc, t));
                        V3 nrm = vsub(ph, qh);
                        float nl = vdot(nrm, nrm);
                        if (nl > K_EPS) {
                            nrm = vmul(nrm, 1.0f / sqrtf(nl));
                            float vn = vdot(vsub(vsub(pc, ph), vsub(qc, qh)), nrm);
                            if (vn > 0.0f) { resp = vmul(nrm, -vn * scale); hit = 1; }
                        }
                    }
                }
            }
            if (!hit) {
                V3 delta = vsub(pc, qc);
                float dsq = vdot(delta, delta);
                if (dsq >= th * th) continue;
                V3 nrm = v3(0, 0, 1);
                float dist = sqrtf(fmaxf(dsq, K_EPS));
                if (dsq > K_EPS) nrm = vmul(delta, 1.0f / dist);
                else {
                    V3 rd = vsub(s->rest[src], s->rest[o]);
                    float rl = vdot(rd, rd);
                    if (rl > K_EPS) nrm = vmul(rd, 1.0f / sqrtf(rl));
                    dist = 0.0f;
                }
                resp = vmul(nrm, fminf((th - dist) * scale, th * 0.35f));
                hit = 1;
            }
            if (hit && vdot(resp, resp) > K_EPS) {
                float ml = fmaxf(th * 0.35f, 1.0e-4f), rl = vlen(resp);
                if (rl > ml) resp = vmul(resp, ml / rl);
                if (fast_mode(s)) {
                    V3 nrm = vmul(resp, 1.0f / fmaxf(vlen(resp), K_EPS));
                    unsigned key = cluster_key(0, vmul(vadd(pc, qc), 0.5f), nrm, fmaxf(th * 2.5f, 1.0e-3f));
                    if (!local_accept(s, 0, key, &cl)) continue;
                    cnt(s, C_SELF_CAND);
                }
                accumulate(s, src, resp);
                cnt(s, C_EXACT);
            }
        }
    }
}

static int rest_vt_neighbor(OracleSolver* s, int vtx, const int* t, float target, float onset) {
    if (vtx == t[0] || vtx == t[1] || vtx == t[2]) return 1;
    V3 rp = s->rest[vtx];
    V3 rd = vsub(rp, closest_on_tri(rp, s->rest[t[0]], s->rest[t[1]], s->rest[t[2]]));
    float skip = fmaxf(onset * 1.25f, target * 2.5f);
    return vdot(rd, rd) < skip * skip;
}
/* abi41.cu:4990-5107 */
static int vt_pair(OracleSolver* s, int vtx, int tri, float target, float onset, Clusters* cl) {
    if (tri < 0 || tri >= s->T || target <= 0.0f || onset <= target) return 0;
    const int* t = s->tris + 3 * tri;
    if (!tri_ok(s, t)) return 0;
    if (rest_vt_neighbor(s, vtx, t, target, onset)) { filter_count(s, C_F_REJ_REST); return 0; }
    V3 p = s->pos[vtx], a = s->pos[t[0]], b = s->pos[t[1]], c = s->pos[t[2]];
    V3 q = closest_on_tri(p, a, b, c), d = vsub(p, q);
    float dsq = vdot(d, d), dist = sqrtf(fmaxf(dsq, K_EPS));
    if (dist >= onset) return 0;
    V3 nrm = v3(0, 0, 1);
    if (dsq > K_EPS) nrm = vmul(d, 1.0f / dist);
    else {
        nrm = vcross(vsub(b, a), vsub(c, a));
        float nl = vdot(nrm, nrm);
        if (nl > K_EPS) nrm = vmul(nrm, 1.0f / sqrtf(nl));
        else {
            V3 rv = s->rest[vtx];
            V3 rd = vsub(rv, closest_on_tri(rv, s->rest[t[0]], s->rest[t[1]], s->rest[t[2]]));
            float rl = vdot(rd, rd);
            if (rl > K_EPS) nrm = vmul(rd, 1.0f / sqrtf(rl));
        }
        d = vmul(nrm, dist);
        dist = 0.0f;
    }
    if (fast_mode(s)) {
        unsigned key = cluster_key(1, q, v3(0, 0, 0), fmaxf(onset * 12.0f, 1.0e-3f));
        if (!local_accept(s, 1, key, cl)) return 1;
    }
    cnt(s, C_SELF_CAND);
    float wa, wb, wc;
    barycentric(q, a, b, c, &wa, &wb, &wc);
    float pen = target - dist, push;
    if (pen > 0.0f) push = fminf(pen * 0.35f + target * 0.01f, target * 0.25f);
    else { float x = 1.0f - fminf(dist / onset, 1.0f); push = fminf(x * x * target * 0.06f, target * 0.04f); }
    float wv = s->inv[vtx], wta = s->inv[t[0]] * wa, wtb = s->inv[t[1]] * wb, wtc = s->inv[t[2]] * wc;
    float total = wv + wta + wtb + wtc;
    if (push <= 0.0f || total <= 0.0f) return 1;
    V3 delta = vmul(nrm, push / total);
    if (wv > 0.0f) accumulate(s, vtx, vmul(delta, wv));
    if (wta > 0.0f) accumulate(s, t[0], vmul(delta, -wta));
    if (wtb > 0.0f) accumulate(s, t[1], vmul(delta, -wtb));
    if (wtc > 0.0f) accumulate(s, t[2], vmul(delta, -wtc));
    cnt(s, C_SOFT);
    return 1;
}
static int budget(const OracleSolver* s) {
    int m = s->cfg.max_self_collision_neighbors;
    if (m < 1) m = 1;
    if (m > BUCKET_SLOTS) m = BUCKET_SLOTS;
    if (fast_mode(s) && m > 16) m = 16;
    return m;
}
/* abi41.cu:5109-5224 */
static void vt_all(OracleSolver* s) {
    const float target = s->radius, onset = fmaxf(target * 1.8f, target + K_EPS);
    if (target <= 0.0f) return;
    const int bud = budget(s);
#pragma omp parallel for schedule(dynamic, 256)
    for (int vtx = 0; vtx < s->V; ++vtx) {
        int acc = 0;
        Clusters cl; cl.n = 0;
        if (s->thash) {
            V3 p = s->pos[vtx];
            int b = (int)bucket_of(cell_of(p.x, s->cell), cell_of(p.y, s->cell), cell_of(p.z, s->cell), s->ntb);
            int st = s->tb_start[b], lim = s->tb_start[b + 1] - st;
            if (lim > BUCKET_SLOTS) lim = BUCKET_SLOTS;
            if (!fast_mode(s)) {
                for (int k = 0; k < lim && acc < bud; ++k) if (vt_pair(s, vtx, s->tb_ent[st + k], target, onset, NULL)) ++acc;
            } else {
                Seen seen; seen.n = 0;
                for (int k = 0; k < lim && acc < bud; ++k) {
                    int tri = s->tb_ent[st + k];
                    if (!note_seen(s, tri, &seen)) continue;
                    if (vt_pair(s, vtx, tri, target, onset, &cl)) ++acc;
                }
            }
        } else {
            for (int tri = 0; tri < s->T && acc < bud; ++tri) {
                if (!note_seen(s, tri, NULL)) continue;
                if (vt_pair(s, vtx, tri, target, onset, &cl)) ++acc;
            }
        }
    }
}

static int rest_ee_neighbor(OracleSolver* s, const int* ea, const int* eb, float target, float onset) {
    if (ea[0] == eb[0] || ea[0] == eb[1] || ea[1] == eb[0] || ea[1] == eb[1]) return 1;
    V3 a0 = s->rest[ea[0]], a1 = s->rest[ea[1]], b0 = s->rest[eb[0]], b1 = s->rest[eb[1]];
    float sp, tp;
    seg_params(a0, a1, b0, b1, &sp, &tp);
    V3 d = vsub(vadd(a0, vmul(vsub(a1, a0), sp)), vadd(b0, vmul(vsub(b1, b0), tp)));
    float skip = fmaxf(onset * 1.25f, target * 2.5f);
    return vdot(d, d) < skip * skip;
}
/* abi41.cu:5595-5722 */
static int ee_pair(OracleSolver* s, int ia, int ib, float target, float onset, Clusters* cl) {
    if (ib <= ia || ia < 0 || ib < 0 || ia >= s->E || ib >= s->E || target <= 0.0f || onset <= target) return 0;
    const int *ea = s->edges + 2 * ia, *eb = s->edges + 2 * ib;
    if (!edge_ok(s, ea) || !edge_ok(s, eb)) return 0;
    if (rest_ee_neighbor(s, ea, eb, target, onset)) { filter_count(s, C_F_REJ_REST); return 0; }
    V3 a0 = s->pos[ea[0]], a1 = s->pos[ea[1]], b0 = s->pos[eb[0]], b1 = s->pos[eb[1]];
    float sp, tp;
    seg_params(a0, a1, b0, b1, &sp, &tp);
    V3 pa = vadd(a0, vmul(vsub(a1, a0), sp)), pb = vadd(b0, vmul(vsub(b1, b0), tp)), d = vsub(pa, pb);
    float dsq = vdot(d, d), dist = sqrtf(fmaxf(dsq, K_EPS));
    if (dist >= onset) return 0;
    V3 nrm = v3(0, 0, 1);
    if (dsq > K_EPS) nrm = vmul(d, 1.0f / dist);
    else {
        nrm = vcross(vsub(a1, a0), vsub(b1, b0));
        float nl = vdot(nrm, nrm);
        if (nl > K_EPS) nrm = vmul(nrm, 1.0f / sqrtf(nl));
        else {
            V3 r0 = s->rest[ea[0]], r1 = s->rest[ea[1]], r2 = s->rest[eb[0]], r3 = s->rest[eb[1]];
            float rs, rt;
            seg_params(r0, r1, r2, r3, &rs, &rt);
            V3 rd = vsub(vadd(r0, vmul(vsub(r1, r0), rs)), vadd(r2, vmul(vsub(r3, r2), rt)));
            float rl = vdot(rd, rd);
            if (rl > K_EPS) nrm = vmul(rd, 1.0f / sqrtf(rl));
        }
        dist = 0.0f;
    }
    if (fast_mode(s)) {
        unsigned key = cluster_key(2, vmul(vadd(pa, pb), 0.5f), v3(0, 0, 0), fmaxf(onset * 12.0f, 1.0e-3f));
        if (!local_accept(s, 2, key, cl)) return 1;
    }
    cnt(s, C_SELF_CAND);
    float pen = target - dist, push;
    if (pen > 0.0f) push = fminf(pen * 0.35f + target * 0.01f, target * 0.25f);
    else { float x = 1.0f - fminf(dist / onset, 1.0f); push = fminf(x * x * target * 0.06f, target * 0.04f); }
    float ma0 = s->inv[ea[0]], ma1 = s->inv[ea[1]], mb0 = s->inv[eb[0]], mb1 = s->inv[eb[1]];
    float ws0 = 1.0f - sp, ws1 = sp, wt0 = 1.0f - tp, wt1 = tp;
    float wa0 = ma0 * ws0, wa1 = ma1 * ws1, wb0 = mb0 * wt0, wb1 = mb1 * wt1;
    float total = ma0 * ws0 * ws0 + ma1 * ws1 * ws1 + mb0 * wt0 * wt0 + mb1 * wt1 * wt1;
    if (push <= 0.0f || total <= 0.0f) return 1;
    V3 delta = vmul(nrm, push / total);
    if (wa0 > 0.0f) accumulate(s, ea[0], vmul(delta, wa0));
    if (wa1 > 0.0f) accumulate(s, ea[1], vmul(delta, wa1));
    if (wb0 > 0.0f) accumulate(s, eb[0], vmul(delta, -wb0));
    if (wb1 > 0.0f) accumulate(s, eb[1], vmul(delta, -wb1));
    cnt(s, C_EE);
    return 1;
}
/* abi41.cu:5724-5844 */
static void ee_all(OracleSolver* s) {
    const float target = s->radius, onset = fmaxf(target * 1.8f, target + K_EPS);
    if (target <= 0.0f) return;
    const int bud = budget(s);
#pragma omp parallel for schedule(dynamic, 256)
    for (int e = 0; e < s->E; ++e) {
        int acc = 0;
        Clusters cl; cl.n = 0;
        if (s->ehash) {
            const int* ed = s->edges + 2 * e;
            if (!edge_ok(s, ed)) continue;
            V3 mid = vmul(vadd(s->pos[ed[0]], s->pos[ed[1]]), 0.5f);
            int b = (int)bucket_of(cell_of(mid.x, s->cell), cell_of(mid.y, s->cell), cell_of(mid.z, s->cell), s->neb);
            int st = s->eb_start[b], lim = s->eb_start[b + 1] - st;
            if (lim > BUCKET_SLOTS) lim = BUCKET_SLOTS;
            if (!fast_mode(s)) {
                for (int k = 0; k < lim && acc < bud; ++k) if (ee_pair(s, e, s->eb_ent[st + k], target, onset, NULL)) ++acc;
            } else {
                Seen seen; seen.n = 0;
                for (int k = 0; k < lim && acc < bud; ++k) {
                    int o = s->eb_ent[st + k];
                    if (!note_seen(s, o, &seen)) continue;
                    if (ee_pair(s, e, o, target, onset, &cl)) ++acc;
                }
            }
        } else {
            for (int o = e + 1; o < s->E && acc < bud; ++o) {
                if (!note_seen(s, o, NULL)) continue;
                if (ee_pair(s, e, o, target, onset, &cl)) ++acc;
            }
        }
    }
}

/* abi41.cu:5226-5439 */
static void island_all(OracleSolver* s) {
    const float target = s->radius, onset = fmaxf(target * 1.8f, target + K_EPS);
    if (target <= 0.0f) return;
#pragma omp parallel for schedule(dynamic, 256)
    for (int vtx = 0; vtx < s->V; ++vtx) {
        if (!(s->inv[vtx] > 0.0f)) continue;
        V3 p = s->pos[vtx], pp = s->prev[vtx];
        if (!vfinite(p) || !vfinite(pp)) { cnt(s, C_ISL_GUARD); continue; }
        int maxn = s->cfg.max_self_collision_neighbors < 1 ? 1 : s->cfg.max_self_collision_neighbors;
        int maxc = maxn * 2;
        if (maxc > 48) maxc = 48;
        if (maxc < 3) maxc = 3;
        int scan_limit = maxc * 10, tris_acc[48];
        int cx = cell_of(p.x, s->cell), cy = cell_of(p.y, s->cell), cz = cell_of(p.z, s->cell);
        int scanned = 0, contacts = 0;
        float pen_sum = 0, wsum = 0, max_pen = 0;
        V3 axis = v3(0, 0, 0), best = v3(0, 0, 1);
        for (int dz = -1; dz <= 1 && contacts < maxc && scanned < scan_limit; ++dz)
            for (int dy = -1; dy <= 1 && contacts < maxc && scanned < scan_limit; ++dy)
                for (int dx = -1; dx <= 1 && contacts < maxc && scanned < scan_limit; ++dx) {
                    int b = (int)bucket_of(cx + dx, cy + dy, cz + dz, s->ntb), st = s->tb_start[b];
                    int lim = s->tb_start[b + 1] - st; if (lim > BUCKET_SLOTS) lim = BUCKET_SLOTS;
                    for (int k = 0; k < lim && contacts < maxc && scanned < scan_limit; ++k) {
                        ++scanned;
                        int tri = s->tb_ent[st + k], dup = 0;
                        for (int q = 0; q < contacts; ++q) if (tris_acc[q] == tri) { dup = 1; break; }
                        if (dup) continue;
                        if (tri < 0 || tri >= s->T) { cnt(s, C_ISL_GUARD); continue; }
                        const int* t = s->tris + 3 * tri;
                        if (!tri_ok(s, t) || rest_vt_neighbor(s, vtx, t, target, onset)) continue;
                        V3 a = s->pos[t[0]], b2 = s->pos[t[1]], c = s->pos[t[2]];
                        V3 ap = s->prev[t[0]], bp = s->prev[t[1]], cp = s->prev[t[2]];
                        if (!vfinite(a) || !vfinite(b2) || !vfinite(c) || !vfinite(ap) || !vfinite(bp) || !vfinite(cp)) { cnt(s, C_ISL_GUARD); continue; }
                        V3 q = closest_on_tri(p, a, b2, c), delta = vsub(p, q);
                        float dsq = vdot(delta, delta), dist = sqrtf(fmaxf(dsq, K_EPS));
                        if (dist >= target) continue;
                        V3 nrm = v3(0, 0, 1);
                        if (dsq > K_EPS) nrm = vmul(delta, 1.0f / dist);
                        else {
                            nrm = vcross(vsub(b2, a), vsub(c, a));
                            float nl = vdot(nrm, nrm);
                            if (nl > K_EPS) nrm = vmul(nrm, 1.0f / sqrtf(nl));
                            else {
                                V3 rv = s->rest[vtx];
                                V3 rd = vsub(rv, closest_on_tri(rv, s->rest[t[0]], s->rest[t[1]], s->rest[t[2]]));
                                float rl = vdot(rd, rd);
                                if (rl > K_EPS) nrm = vmul(rd, 1.0f / sqrtf(rl));
                            }
                            delta = vmul(nrm, dist);
                            dist = 0.0f;
                        }
                        if (!vfinite(nrm)) { cnt(s, C_ISL_GUARD); continue; }
                        V3 pd = vsub(pp, closest_on_tri(pp, ap, bp, cp));
                        if (vdot(pd, nrm) > target * 0.25f && vdot(delta, nrm) > -target * 0.10f) continue;
                        float wa, wb, wc;
                        barycentric(q, a, b2, c, &wa, &wb, &wc);
                        float pen = target - dist;
                        if (pen <= 0.0f) continue;
                        tris_acc[contacts++] = tri;
                        pen_sum += pen;
                        wsum += s->inv[t[0]] * wa + s->inv[t[1]] * wb + s->inv[t[2]] * wc;
                        axis = vadd(axis, vmul(nrm, pen));
                        if (pen > max_pen) { max_pen = pen; best = nrm; }
                    }
                }
        if (contacts <= 0) continue;
        cnt_add(s, C_ISL_CAND, (unsigned long long)contacts);
        if (contacts < 3) { cnt(s, C_ISL_GUARD); continue; }
        float avg_pen = pen_sum / (float)contacts;
        if (avg_pen < target * 0.04f) { cnt(s, C_ISL_GUARD); continue; }
        float al = vlen(axis);
        V3 agg = al > K_EPS ? vmul(axis, 1.0f / al) : best;
        float sw = s->inv[vtx], sample = wsum / (float)contacts, share = sw / fmaxf(sw + sample, K_EPS);
        float md = fmaxf(target * 0.30f, 1.0e-5f), dl = fminf(avg_pen * 0.50f * share, md);
        if (!vfinite(agg) || !isfinite(dl) || dl <= K_EPS) { cnt(s, C_ISL_GUARD); continue; }
        accumulate(s, vtx, vmul(agg, dl));
        cnt(s, C_ISL_CLUST);
        cnt_add(s, C_ISL_REFS, (unsigned long long)contacts);
        cnt(s, C_ISL_APPLIED);
        unsigned long long micro = (unsigned long long)(fminf(dl, 1024.0f) * 1000000.0f);
#pragma omp critical
        if (micro > s->counts[C_ISL_MAXD]) s->counts[C_ISL_MAXD] = micro;
    }
}

/* abi41.cu:4953-4988 */
static void self_apply_all(OracleSolver* s) {
    const float md = fmaxf(s->radius * 0.35f, 1.0e-4f);
    for (int i = 0; i < s->V; ++i) {
        long long* a = s->acc + 4 * (size_t)i;
        long long ax = a[0], ay = a[1], az = a[2], aw = a[3];
        a[0] = a[1] = a[2] = a[3] = 0;
        if (!(s->inv[i] > 0.0f) || aw <= 0) continue;
        V3 avg = vmul(v3(from_fix(ax), from_fix(ay), from_fix(az)), 1.0f / (float)aw);
        float dl = vlen(avg);
        if (dl > md) avg = vmul(avg, md / dl);
        s->pos[i] = vadd(s->pos[i], avg);
        s->prev[i] = vadd(s->prev[i], vmul(avg, 0.55f));
        float al = vlen(avg);
        if (al > s->max_delta) s->max_delta = al;
    }
}

static void build_hashes(OracleSolver* s) {
    if (s->vhash) hash_vertices(s);
    if (s->thash) hash_prims(s, 1);
    if (s->ehash) hash_prims(s, 0);
}

/* Self-collision block of one substep (abi41.cu:9255-9339). */
static void self_collision(OracleSolver* s) {
    int passes = s->cfg.fast_self_collision_passes;
    if (passes > 8) passes = 8;
    if (passes < 1) passes = 1;
    int fast = fast_mode(s);
    build_hashes(s);
    if (fast) neighbors_all(s);
    for (int pass = 0; pass < passes; ++pass) {
        if (!fast) neighbors_all(s);
        vv_all(s);
        if (s->T > 0) vt_all(s);
        if (s->E > 0) ee_all(s);
        if (pass == passes - 1 && fast && s->T > 0 && s->thash) island_all(s);
        self_apply_all(s);
    }
}


/* ------------------------------------------------ hard-stretch solve -- */
typedef struct { float m11, m12, m13, m22, m23, m33; } Sym;
static Sym sym_ld(const float* a, int i) { const float* m = a + 6 * (size_t)i; Sym r = {m[0], m[1], m[2], m[3], m[4], m[5]}; return r; }
static void sym_st(float* a, int i, Sym m) { float* o = a + 6 * (size_t)i; o[0] = m.m11; o[1] = m.m12; o[2] = m.m13; o[3] = m.m22; o[4] = m.m23; o[5] = m.m33; }
/* abi41.cu:1125-1131 */
static V3 sym_madd(Sym m, V3 v, V3 a) {
    return v3(fmaf(m.m13, v.z, fmaf(m.m12, v.y, fmaf(m.m11, v.x, a.x))), fmaf(m.m23, v.z, fmaf(m.m22, v.y, fmaf(m.m12, v.x, a.y))),
              fmaf(m.m33, v.z, fmaf(m.m23, v.y, fmaf(m.m13, v.x, a.z))));
}
static Sym sym_outer(V3 n, float s) { Sym r = {n.x * n.x * s, n.x * n.y * s, n.x * n.z * s, n.y * n.y * s, n.y * n.z * s, n.z * n.z * s}; return r; }
static Sym sym_add(Sym a, Sym b) { Sym r = {a.m11 + b.m11, a.m12 + b.m12, a.m13 + b.m13, a.m22 + b.m22, a.m23 + b.m23, a.m33 + b.m33}; return r; }
/* abi41.cu:1158-1189 */
static Sym sym_inv(OracleSolver* s, Sym m) {
    float a = m.m11, b = m.m12, c = m.m13, d = m.m22, e = m.m23, f = m.m33;
    float df_ee = fmaf(d, f, -e * e), bf_ce = fmaf(b, f, -c * e), be_cd = fmaf(b, e, -c * d);
    float det = fmaf(c, be_cd, fmaf(-b, bf_ce, a * df_ee));
    if (isfinite(det) && fabsf(det) > 1.0e-12f) {
        float inv = 1.0f / det;
        Sym r = {df_ee * inv, fmaf(c, e, -b * f) * inv, be_cd * inv, fmaf(a, f, -c * c) * inv, fmaf(b, c, -a * e) * inv, fmaf(a, d, -b * b) * inv};
        return r;
    }
#pragma omp atomic
    s->pcg_guard += 1;
    Sym r = {1.0f / fmaxf(fabsf(a), 1.0e-4f), 0, 0, 1.0f / fmaxf(fabsf(d), 1.0e-4f), 0, 1.0f / fmaxf(fabsf(f), 1.0e-4f)};
    return r;
}
/* abi41.cu:1070-1104 */
static float proj_limit(const OracleSolver* s, float rest) {
    float th = s->cfg.cloth_thickness;
    float base = fmaxf(1.0e-5f, fminf(fmaxf(rest, th) * 0.5f, 0.25f));
    if (s->strength < 0.95f || !isfinite(th) || th <= K_EPS) return base;
    return fminf(base, fmaxf(1.0e-5f, fminf(fmaxf(rest * 0.18f, th * 0.06f), 0.0035f)));
}
static float writeback_limit(const OracleSolver* s) {
    float th = s->cfg.cloth_thickness;
    if (s->strength < 0.95f || !isfinite(th) || th <= K_EPS) return 0.25f;
    return fmaxf(2.5e-4f, fminf(th * 0.035f, 9.0e-4f));
}

/* Sum of per-vertex values in the GPU's fixed order: a shuffle-down tree
 * per 32-vertex warp over a grid of ceil(V / 256) * 256 threads, then lane l
 * adds warp partials l, l + 32, ... and a final shuffle-down tree. */
static float warp_tree32(const float* x) {
    float a[32];
    memcpy(a, x, sizeof(a));
    for (int o = 16; o > 0; o >>= 1) {
        float b[32];
        for (int l = 0; l < 32; ++l) b[l] = a[l] + (l + o < 32 ? a[l + o] : a[l]);
        memcpy(a, b, sizeof(a));
    }
    return a[0];
}
static float fixed_sum(const float* vals, int V) {
    int nw = ((V + 255) / 256) * 8;
    float* part = (float*)calloc((size_t)nw + 1, sizeof(float));
    for (int w = 0; w < nw; ++w) {
        float x[32];
        for (int l = 0; l < 32; ++l) { int i = w * 32 + l; x[l] = i < V ? vals[i] : 0.0f; }
        part[w] = warp_tree32(x);
    }
    float lanes[32];
    for (int l = 0; l < 32; ++l) { float acc = 0.0f; for (int k = l; k < nw; k += 32) acc += part[k]; lanes[l] = acc; }
    free(part);
    return warp_tree32(lanes);
}

/* Assembly (abi41.cu:3085-3186) gathered per vertex in edge order, with
 * the preconditioner and initial residual (abi41.cu:3188-3226). */
static void pcg_build(OracleSolver* s, float* tmp) {
    const float strength = clamp01(s->strength * 2.5f);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->V; ++i) {
        Sym dg = {1, 0, 0, 1, 0, 1};
        V3 rhs = v3(0, 0, 0);
        for (int k = s->sp_off[i]; k < s->sp_off[i + 1]; ++k) {
            int o = s->sp_other[k], is_j = s->sp_side[k];
            int a = is_j ? o : i, b = is_j ? i : o;
            float wi = s->w[a], wj = s->w[b], weight = wi + wj, rest = s->sp_rest[k];
            int ai = wi > 0.0f, aj = wj > 0.0f;
            float* off = s->off + 4 * (size_t)k;
            off[0] = off[1] = off[2] = off[3] = 0.0f;
            V3 pi = s->pos[a], pj = s->pos[b];
            if (!(isfinite(weight) && weight > 0.0f && isfinite(rest) && rest > K_EPS && vfinite(pi) && vfinite(pj))) continue;
            V3 delta = vsub(pj, pi);
            float lsq = vdot(delta, delta);
            if (!isfinite(lsq) || lsq <= K_EPS) continue;
            float len = sqrtf(lsq), err = len - rest;
            if (!isfinite(err) || fabsf(err) <= 1.0e-6f || strength <= 0.0f) continue;
            float lim = proj_limit(s, rest);
            float projected = fmaxf(-lim, fminf(err * strength, lim));
            if (!isfinite(projected) || fabsf(projected) <= 1.0e-7f) continue;
            V3 n = vmul(delta, 1.0f / len);
            V3 desired = vmul(n, projected / weight);
            float stiff = fmaxf(strength, 1.0e-3f);
            if (is_j ? aj : ai) {
                rhs = vadd(rhs, is_j ? vmul(desired, -wj) : vmul(desired, wi));
                dg = sym_add(dg, sym_outer(n, stiff));
            }
            if (ai && aj) { off[0] = n.x; off[1] = n.y; off[2] = n.z; off[3] = stiff; }
        }
        sym_st(s->diag, i, dg);
        if (!(s->w[i] > 0.0f)) {
            s->r[i] = s->z[i] = s->d[i] = v3(0, 0, 0);
            Sym id = {1, 0, 0, 1, 0, 1};
            sym_st(s->pinv, i, id);
            tmp[i] = 0.0f;
        } else {
            Sym inv = sym_inv(s, dg);
            V3 z = sym_madd(inv, rhs, v3(0, 0, 0));
            sym_st(s->pinv, i, inv);
            s->r[i] = rhs; s->z[i] = z; s->d[i] = z;
            tmp[i] = vdot(rhs, z);
        }
    }
    float total = fixed_sum(tmp, s->V);
    s->red[R_RZ] = total; s->red[R_INIT] = total; s->red[R_ITER] = 0.0f; s->red[R_DAD] = 0.0f; s->red[R_RZN] = 0.0f;
    s->red[R_STATUS] = 0.0f;
}

/* Eight CG iterations with device alpha / beta and the incremental write-back
 * (abi41.cu:3228-3464, 7655-7674). */
static void pcg_iterate(OracleSolver* s, float* tmp) {
    for (int it = 0; it < 8; ++it) {
        /* q = A d */
        int status_ok = s->red[R_STATUS] == 0.0f;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < s->V; ++i) {
            tmp[i] = 0.0f;
            if (!status_ok) continue;
            if (!(s->w[i] > 0.0f)) { s->q[i] = v3(0, 0, 0); continue; }
            V3 qv = sym_madd(sym_ld(s->diag, i), s->d[i], v3(0, 0, 0));
            for (int k = s->sp_off[i]; k < s->sp_off[i + 1]; ++k) {
                const float* o = s->off + 4 * (size_t)k;
                Sym nb = {0, 0, 0, 0, 0, 0};
                if (o[3] != 0.0f) {
                    Sym b = sym_outer(v3(o[0], o[1], o[2]), o[3]);
                    Sym m = {-b.m11, -b.m12, -b.m13, -b.m22, -b.m23, -b.m33};
                    nb = m;
                }
                qv = sym_madd(nb, s->d[s->sp_other[k]], qv);
            }
            s->q[i] = qv;
            tmp[i] = vdot(s->d[i], qv);
        }
        s->red[R_DAD] = s->red[R_DAD] + fixed_sum(tmp, s->V);
        /* update */
        float rz_old = s->red[R_RZ], dad = s->red[R_DAD], status = 0.0f, alpha = 0.0f;
        if (!isfinite(rz_old) || rz_old < 0.0f) status = 1.0f;
        else if (rz_old <= 1.0e-14f) status = 2.0f;
        else if (!isfinite(dad) || dad <= 1.0e-14f) status = 3.0f;
        else { alpha = rz_old / dad; if (!isfinite(alpha)) status = 4.0f; }
        if (status != 0.0f) {
            s->red[R_STATUS] = status;
            if (status != 2.0f) s->pcg_guard += 1;
        } else {
            const float mdl = writeback_limit(s);
#pragma omp parallel for schedule(static)
            for (int i = 0; i < s->V; ++i) {
                tmp[i] = 0.0f;
                if (!(s->w[i] > 0.0f)) { s->r[i] = s->z[i] = v3(0, 0, 0); continue; }
                V3 di = s->d[i], qi = s->q[i], ri = s->r[i];
                V3 res = v3(fmaf(qi.x, -alpha, ri.x), fmaf(qi.y, -alpha, ri.y), fmaf(qi.z, -alpha, ri.z));
                if (!vfinite(res)) res = v3(0, 0, 0);
                V3 z = sym_madd(sym_ld(s->pinv, i), res, v3(0, 0, 0));
                s->r[i] = res; s->z[i] = z;
                tmp[i] = vdot(res, z);
                V3 delta = vmul(di, alpha);
                float len = vlen(delta);
                if (len > mdl) { delta = vmul(delta, mdl / fmaxf(len, K_EPS)); cnt(s, C_HARD); }
                s->pos[i] = vadd(s->pos[i], delta);
                s->prev[i] = vadd(s->prev[i], vmul(delta, 0.08f));
                float dl = vlen(delta);
#pragma omp critical
                if (dl > s->pcg_max_delta) s->pcg_max_delta = dl;
            }
            s->red[R_RZN] = s->red[R_RZN] + fixed_sum(tmp, s->V);
            s->red[R_ITER] = s->red[R_ITER] + 1.0f;
        }
        if (it + 1 >= 8) break;
        /* direction and advance */
        float st = s->red[R_STATUS], ro = s->red[R_RZ], rn = s->red[R_RZN];
        int ok = st == 0.0f && isfinite(ro) && isfinite(rn) && ro > 1.0e-14f && rn >= 0.0f;
        float beta = ok ? rn / ro : 0.0f;
        if (ok && isfinite(beta)) {
#pragma omp parallel for schedule(static)
            for (int i = 0; i < s->V; ++i) {
                if (!(s->w[i] > 0.0f)) { s->d[i] = v3(0, 0, 0); continue; }
                V3 dd = s->d[i], zz = s->z[i];
                s->d[i] = v3(fmaf(dd.x, beta, zz.x), fmaf(dd.y, beta, zz.y), fmaf(dd.z, beta, zz.z));
            }
        }
        if (st == 0.0f && isfinite(rn) && rn >= 0.0f) {
            s->red[R_RZ] = rn; s->red[R_DAD] = 0.0f; s->red[R_RZN] = 0.0f; s->red[R_STATUS] = 0.0f;
        }
    }
}

/* Averaged polish / tiny corrections of one vertex's edges
 * (abi41.cu:1995-2112, 2399-2494). */
static int avg_delta(OracleSolver* s, int tiny, int a, int b, float rest, int is_j, V3* out) {
    float wi = s->w[a], wj = s->w[b], weight = wi + wj;
    if (!isfinite(weight) || weight <= 0.0f) return 0;
    V3 pi = s->pos[a], pj = s->pos[b];
    if (tiny) {
        if (!isfinite(rest) || rest <= K_EPS || rest > 7.5e-4f) return 0;
        if (!vfinite(pi) || !vfinite(pj)) return 0;
    } else {
        if (!isfinite(rest) || rest <= K_EPS) return 0;
        if (!vfinite(pi) || !vfinite(pj) || !vfinite(s->prev[a]) || !vfinite(s->prev[b])) return 0;
    }
    V3 edge = vsub(pj, pi);
    float lsq = vdot(edge, edge);
    if (!isfinite(lsq) || lsq <= 1.0e-14f) return 0;
    float len = sqrtf(lsq), target, relax, md;
    if (tiny) { target = rest * 1.06f; relax = 1.0f; md = fminf(fmaxf(rest * 3.0f, 2.5e-4f), 8.0e-4f); }
    else {
        target = rest * (s->strength >= 0.95f ? 1.08f : 1.18f); relax = 0.90f;
        md = fmaxf(5.0e-4f, fminf(fmaxf(rest * 2.0f, s->cfg.cloth_thickness * 0.25f), 0.008f));
    }
    float excess = len - target;
    if (!isfinite(excess) || excess <= 0.0f) return 0;
    V3 corr = vmul(edge, -relax * excess / fmaxf(weight * len, K_EPS));
    if (!vfinite(corr)) return 0;
    float cl = vlen(corr);
    if (!isfinite(cl) || cl <= 1.0e-20f) return 0;
    float w = is_j ? wj : wi;
    if (!(w > 0.0f)) return 0;
    V3 d = limit_delta(is_j ? vmul(corr, wj) : vmul(corr, -wi), md);
    if (!vfinite(d) || !(vlen(d) > 0.0f)) return 0;
    *out = d;
    return 1;
}
static void averaged_pass(OracleSolver* s, int tiny) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->V; ++i) {
        V3 sum = v3(0, 0, 0);
        float count = 0.0f;
        for (int k = s->sp_off[i]; k < s->sp_off[i + 1]; ++k) {
            int o = s->sp_other[k], is_j = s->sp_side[k];
            V3 d;
            if (avg_delta(s, tiny, is_j ? o : i, is_j ? i : o, s->sp_rest[k], is_j, &d)) { sum = vadd(sum, d); count += 1.0f; }
        }
        s->avg_sum[i] = sum; s->avg_cnt[i] = count;
    }
    const float th = s->cfg.cloth_thickness;
    const float md = tiny ? fminf(fmaxf(th * 0.015f, 2.5e-4f), 9.0e-4f) : fmaxf(5.0e-4f, fminf(fmaxf(th * 0.20f, 1.0e-3f), 0.005f));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->V; ++i) {
        if (!(s->w[i] > 0.0f)) continue;
        float count = s->avg_cnt[i];
        if (!isfinite(count) || count <= 0.0f) continue;
        V3 delta = vmul(s->avg_sum[i], 1.0f / count);
        if (!vfinite(delta)) { cnt(s, C_HARD); continue; }
        delta = limit_delta(delta, md);
        if (!vfinite(delta) || !(vlen(delta) > 0.0f)) continue;
        s->pos[i] = vadd(s->pos[i], delta);
        s->prev[i] = vadd(s->prev[i], vmul(delta, tiny ? 0.24f : 0.16f));
    }
}

/* One edge of a ratio cap, kind 0 normal (abi41.cu:2249-2362), 1 tiny
 * (2496-2601), 2 extreme (2603-2708): the position correction d* and the
 * previous-position shift pd* of each endpoint, ok* = 0 where that endpoint
 * gets nothing.  Returns 0 when the edge is skipped. */
static int cap_edge(const OracleSolver* s, int kind, float dt, float rest, V3 pi, V3 pj, V3 qi, V3 qj, float wi, float wj,
                    V3* di, V3* pdi_out, int* oki, V3* dj, V3* pdj_out, int* okj) {
    *oki = *okj = 0;
    if (!isfinite(rest) || rest <= K_EPS) return 0;
    if (kind == 1 ? rest > 7.5e-4f : rest <= 7.5e-4f) return 0;
    float weight = wi + wj;
    if (!isfinite(weight) || weight <= 0.0f) return 0;
    if (!vfinite(pi) || !vfinite(pj) || !vfinite(qi) || !vfinite(qj)) return 0;
    V3 edge = vsub(pj, pi);
    float lsq = vdot(edge, edge);
    if (!isfinite(lsq) || lsq <= 1.0e-14f) return 0;
    float len = sqrtf(lsq);
    int high = s->strength >= 0.95f;
    float sr, tr, md, ps;
    float th = s->cfg.cloth_thickness;
    if (kind == 0) { sr = high ? 1.12f : 1.32f; tr = high ? 1.04f : 1.22f; md = fminf(fmaxf(rest * 0.60f, th * 0.10f), 0.010f); ps = 0.08f; }
    else if (kind == 1) { sr = 1.35f; tr = 1.12f; md = fminf(fmaxf(rest * 6.0f, 5.0e-4f), 1.5e-3f); ps = 1.0f; }
    else { sr = 1.24f; tr = 1.10f; md = fminf(fmaxf(rest * 1.25f, th * 0.10f), 0.006f); ps = 0.30f; }
    if (!isfinite(len) || len <= rest * sr) return 0;
    float excess = len - rest * tr;
    if (!isfinite(excess) || excess <= 0.0f) return 0;
    V3 corr = vmul(edge, -excess / fmaxf(weight * len, K_EPS));
    if (!vfinite(corr) || vlen(corr) <= 1.0e-20f) return 0;
    V3 pdi = v3(0, 0, 0), pdj = v3(0, 0, 0);
    V3 n = vmul(edge, 1.0f / fmaxf(len, K_EPS));
    float sdt = kind == 0 ? fmaxf(dt, K_EPS) : dt;
    if (isfinite(sdt) && sdt > K_EPS) {
        float inv_dt = 1.0f / sdt;
        V3 vi = vmul(vsub(pi, qi), inv_dt), vj = vmul(vsub(pj, qj), inv_dt);
        float sep = vdot(vsub(vj, vi), n);
        if (isfinite(sep) && sep > 0.0f) {
            float trim = sep * sdt * 1.0f / weight;
            if (wi > 0.0f) pdi = vadd(pdi, vmul(n, -wi * trim));
            if (wj > 0.0f) pdj = vadd(pdj, vmul(n, wj * trim));
        }
    }
    if (wi > 0.0f) {
        V3 d = limit_delta(vmul(corr, -wi), md);
        if (vfinite(d) && vlen(d) > 0.0f) { *di = d; *pdi_out = vadd(pdi, vmul(d, ps)); *oki = 1; }
    }
    if (wj > 0.0f) {
        V3 d = limit_delta(vmul(corr, wj), md);
        if (vfinite(d) && vlen(d) > 0.0f) { *dj = d; *pdj_out = vadd(pdj, vmul(d, ps)); *okj = 1; }
    }
    return 1;
}

/* Ratio caps in place one colour at a time (no two edges of a colour share
 * a vertex), as the reference runs them over a caller's edge colouring. */
static void cap_range(OracleSolver* s, int start, int count, float dt, int kind) {
#pragma omp parallel for schedule(static)
    for (int l = 0; l < count; ++l) {
        int e = start + l;
        if (e < 0 || e >= s->E) continue;
        int i = s->cap_edges[2 * e], j = s->cap_edges[2 * e + 1];
        if (i < 0 || j < 0 || i >= s->V || j >= s->V || i == j) continue;
        V3 pi = s->pos[i], pj = s->pos[j], qi = s->prev[i], qj = s->prev[j];
        V3 di, dj, pdi, pdj;
        int oki, okj;
        if (!cap_edge(s, kind, dt, s->cap_rest[e], pi, pj, qi, qj, s->w[i], s->w[j], &di, &pdi, &oki, &dj, &pdj, &okj)) continue;
        if (oki) { s->pos[i] = vadd(pi, di); s->prev[i] = vadd(qi, pdi); }
        if (okj) { s->pos[j] = vadd(pj, dj); s->prev[j] = vadd(qj, pdj); }
    }
}

/* Without a caller's colouring the reference runs a cap pass as one launch
 * over every edge, each adding its corrections to both endpoints with
 * atomics (abi41.cu:7794-7801): a Jacobi pass.  Restated deterministically:
 * every edge sees the positions and previous positions at the start of the
 * pass, and each vertex adds its edges' corrections in edge order. */
static void cap_jacobi(OracleSolver* s, float dt, int kind) {
    memcpy(s->snap, s->pos, sizeof(V3) * (size_t)s->V);
    memcpy(s->snap_prev, s->prev, sizeof(V3) * (size_t)s->V);
#pragma omp parallel for schedule(static)
    for (int v = 0; v < s->V; ++v) {
        V3 p = s->snap[v], q = s->snap_prev[v];
        for (int k = s->sp_off[v]; k < s->sp_off[v + 1]; ++k) {
            int o = s->sp_other[k], is_j = s->sp_side[k];
            int i = is_j ? o : v, j = is_j ? v : o;
            V3 di, dj, pdi, pdj;
            int oki, okj;
            if (!cap_edge(s, kind, dt, s->sp_rest[k], s->snap[i], s->snap[j], s->snap_prev[i], s->snap_prev[j], s->w[i], s->w[j],
                          &di, &pdi, &oki, &dj, &pdj, &okj))
                continue;
            if (is_j ? okj : oki) {
                p = vadd(p, is_j ? dj : di);
                q = vadd(q, is_j ? pdj : pdi);
            }
        }
        s->pos[v] = p;
        s->prev[v] = q;
    }
}

static void caps(OracleSolver* s, float dt, int kind, int passes, int both) {
    for (int p = 0; p < passes; ++p) {
        if (s->cap_jacobi) {
            cap_jacobi(s, dt, kind);
            continue;
        }
        for (int k = 0; k < s->n_cap_colors; ++k) cap_range(s, s->cap_colors[k], s->cap_colors[k + 1] - s->cap_colors[k], dt, kind);
        if (both)
            for (int k = s->n_cap_colors - 1; k >= 0; --k) cap_range(s, s->cap_colors[k], s->cap_colors[k + 1] - s->cap_colors[k], dt, kind);
    }
}
/* PCG solve + polish + extreme caps of one substep (abi41.cu:9183-9201) */
static void hard_stretch(OracleSolver* s, float dt) {
    float* tmp = (float*)calloc((size_t)s->V + 1, sizeof(float));
    pcg_build(s, tmp);
    pcg_iterate(s, tmp);
    free(tmp);
    if (s->strength >= 0.95f) {
        for (int polish = 0; polish < 2; ++polish) {
            averaged_pass(s, 0);
            caps(s, dt, 0, 2, 1);
            for (int tiny = 0; tiny < 2; ++tiny) {
                averaged_pass(s, 1);
                caps(s, dt, 1, 3, 0);
            }
        }
        caps(s, dt, 2, 3, 0);
    }
}

/* ----------------------------------------------------------- lifecycle -- */
static void odyn_free(ODyn* d);

void oracle_destroy(OracleSolver* s) {
    if (!s) return;
    void* p[] = {s->pos, s->snap, s->prev, s->vel, s->rest, s->w, s->inv, s->sp_off, s->sp_other, s->sp_side, s->sp_rest,
                 s->te_off, s->te_other, s->te_side, s->te_rest, s->bj_off, s->bj_other, s->bj_side, s->bj_rest, s->bends,
                 s->bend_rest, s->bend_colors, s->tris, s->edges, s->pin_w, s->pin_t, s->pin_relax, s->sdf, s->stris,
                 s->vcell, s->vb_start, s->vb_ent, s->tb_start, s->tb_ent, s->eb_start, s->eb_ent, s->nb_count, s->nb_idx, s->acc,
                 s->diag, s->pinv, s->r, s->z, s->d, s->q, s->off, s->avg_sum, s->avg_cnt, s->cap_edges, s->cap_rest, s->cap_colors,
                 s->snap_prev, s->vt_off, s->vt_tri, s->p_area, s->p_rest};
    for (size_t k = 0; k < sizeof(p) / sizeof(p[0]); ++k) free(p[k]);
    odyn_free(&s->own);
    free(s);
}

/* Creation and sanitising as abi41.cu:8791-8967 (without PCG / pressure). */
static float env_scale(const char* name, float value, float lo, float hi) {
    const char* raw = getenv(name);
    if (raw && raw[0]) {
        char* end = NULL;
        float v = strtof(raw, &end);
        if (end != raw && isfinite(v)) value = v;
    }
    return fmaxf(lo, fminf(value, hi));
}

/* Area shares (a third of each incident rest triangle, capped at 16 x the
 * mean), rest scales (mean incident rest length, else sqrt(area), clamped to
 * [0.02, 16] x the mean) and the outward-speed length scale. */
static void pressure_prep(OracleSolver* s, const SsblXpbdMesh* mesh, float object_scale) {
    const int V = s->V, T = s->T, E = s->E;
    const float* pos = mesh->positions;
    double total = 0.0;
    int valid = 0;
    for (int t = 0; t < T; ++t) {
        const int* tr = s->tris + 3 * t;
        if (tr[0] < 0 || tr[1] < 0 || tr[2] < 0 || tr[0] >= V || tr[1] >= V || tr[2] >= V) continue;
        V3 a = v3(pos[3 * tr[0]], pos[3 * tr[0] + 1], pos[3 * tr[0] + 2]);
        V3 b = v3(pos[3 * tr[1]], pos[3 * tr[1] + 1], pos[3 * tr[1] + 2]);
        V3 cc = v3(pos[3 * tr[2]], pos[3 * tr[2] + 1], pos[3 * tr[2] + 2]);
        V3 n = vcross(vsub(b, a), vsub(cc, a));
        float sq4 = vdot(n, n);
        if (!isfinite(sq4) || sq4 <= 0.0f) continue;
        float area = 0.5f * sqrtf(sq4);
        if (!isfinite(area) || area <= 0.0f) continue;
        float share = area / 3.0f;
        s->p_area[tr[0]] += share; s->p_area[tr[1]] += share; s->p_area[tr[2]] += share;
        total += (double)area;
        ++valid;
    }
    if (valid <= 0 || !(total > 0.0) || !isfinite(total)) {
        for (int i = 0; i < V; ++i) s->p_area[i] = 0.0f;
    } else {
        float mean = (float)(total / (double)(V > 1 ? V : 1));
        float cap = fmaxf(mean * 16.0f, 1.0e-12f);
        for (int i = 0; i < V; ++i) s->p_area[i] = (!isfinite(s->p_area[i]) || s->p_area[i] <= 0.0f) ? 0.0f : fminf(s->p_area[i], cap);
    }
    double* sum = (double*)calloc((size_t)(V > 0 ? V : 1), sizeof(double));
    int* cnt = (int*)calloc((size_t)(V > 0 ? V : 1), sizeof(int));
    for (int e = 0; e < E; ++e) {
        int i = mesh->edges ? mesh->edges[2 * e] : 0, j = mesh->edges ? mesh->edges[2 * e + 1] : 0;
        if (i < 0) i = 0;
        if (j < 0) j = 0;
        float r = mesh->edge_rest_lengths ? mesh->edge_rest_lengths[e] : 0.0f;
        if (i >= V || j >= V || !isfinite(r) || r <= 0.0f) continue;
        sum[i] += (double)r; sum[j] += (double)r; cnt[i] += 1; cnt[j] += 1;
    }
    double tot = 0.0;
    int nval = 0;
    for (int i = 0; i < V; ++i) {
        float x = 0.0f;
        if (cnt[i] > 0) x = (float)(sum[i] / (double)cnt[i]);
        else if (isfinite(s->p_area[i]) && s->p_area[i] > 0.0f) x = sqrtf(s->p_area[i]);
        if (isfinite(x) && x > 0.0f) { s->p_rest[i] = x; tot += (double)x; ++nval; }
    }
    free(sum); free(cnt);
    float mean = nval > 0 ? (float)(tot / (double)nval) : 1.0f;
    float lo = fmaxf(mean * 0.02f, 1.0e-7f), hi = fmaxf(mean * 16.0f, lo);
    for (int i = 0; i < V; ++i) {
        float x = s->p_rest[i];
        if (!isfinite(x) || x <= 0.0f) x = mean;
        s->p_rest[i] = fmaxf(lo, fminf(x, hi));
    }
    /* velocity length scale */
    float ms = 0.0f;
    int mc = 0;
    for (int i = 0; i < V; ++i) if (isfinite(s->p_rest[i]) && s->p_rest[i] > 0.0f) { ms += s->p_rest[i]; ++mc; }
    ms = mc > 0 ? ms / (float)mc : 1.0f;
    int any = 0;
    V3 lo3 = v3(0, 0, 0), hi3 = v3(0, 0, 0);
    for (int i = 0; i < V; ++i) {
        V3 p = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        if (!vfinite(p)) continue;
        if (!any) { lo3 = hi3 = p; any = 1; }
        else {
            lo3 = v3(fminf(lo3.x, p.x), fminf(lo3.y, p.y), fminf(lo3.z, p.z));
            hi3 = v3(fmaxf(hi3.x, p.x), fmaxf(hi3.y, p.y), fmaxf(hi3.z, p.z));
        }
    }
    if (!any) { s->p_vlen = fmaxf(ms, 1.0e-6f); return; }
    V3 span = vsub(hi3, lo3);
    float diag = sqrtf(fmaxf(vdot(span, span), 0.0f));
    if (!isfinite(diag) || diag <= 0.0f) { s->p_vlen = fmaxf(ms, 1.0e-6f); return; }
    float obj = isfinite(object_scale) && object_scale > 0.0f ? object_scale : 0.08f;
    s->p_vlen = fmaxf(diag * obj, ms * 4.0f);
}

int oracle_update_force_fields(OracleSolver* s, const SsblXpbdForceField* fields, int count) {
    if (!s) return set_err("invalid force field update");
    if (count < 0 || count > 64) return set_err("force field count exceeds SSBL maximum");
    if (count > 0 && !fields) return set_err("missing force field data");
    if (count > 0) memcpy(s->fields, fields, sizeof(SsblXpbdForceField) * (size_t)count);
    s->nfields = count;
    return 1;
}

OracleSolver* oracle_create(const SsblXpbdConfig* config, const SsblXpbdMesh* mesh) {
    if (!config || config->vertex_count < 0 || config->edge_count < 0 || config->triangle_count < 0 || !isfinite(config->dt) ||
        !(config->dt > 0.0f) || !mesh || !mesh->positions || !mesh->inv_mass) {
        set_err("invalid ABI41 solver create request");
        return NULL;
    }
    OracleSolver* s = (OracleSolver*)calloc(1, sizeof(OracleSolver));
    SsblXpbdConfig* c = &s->cfg;
    *c = *config;
    if (c->vertex_count < 0) c->vertex_count = 0;
    if (c->bend_count < 0) c->bend_count = 0;
    if (c->lra_count < 0) c->lra_count = 0;
    c->damping = isfinite(c->damping) ? fmaxf(0.0f, fminf(c->damping, 1.0f)) : 1.0f;
    if (!isfinite(c->bend_compliance) || c->bend_compliance < 0.0f) c->bend_compliance = 0.0f;
    if (!isfinite(c->lra_compliance) || c->lra_compliance < 0.0f) c->lra_compliance = 0.0f;
    if (!isfinite(c->stretch_optimization_strength)) c->stretch_optimization_strength = 0.0f;
    c->stretch_optimization_strength = clamp01(c->stretch_optimization_strength);
    c->stretch_optimization_enabled = (c->edge_count > 0 && c->stretch_optimization_enabled && c->stretch_optimization_strength > 0.0f);
    const int V = c->vertex_count, E = c->edge_count, B = c->bend_count, L = c->lra_count, T = c->triangle_count;
    s->V = V; s->E = E; s->B = B; s->L = L; s->T = T;
    if (B > 0 && (!mesh->bends || !mesh->bend_rest_lengths)) { set_err("ABI41 bend constraints require bend pairs and rest lengths"); oracle_destroy(s); return NULL; }
    if (L > 0 && (!mesh->lra_edges || !mesh->lra_rest_lengths)) { set_err("ABI41 LRA constraints require edge pairs and rest lengths"); oracle_destroy(s); return NULL; }
    s->col.use_ground = c->use_ground; s->col.ground_height = c->ground_height; s->col.use_wall = c->use_wall;
    memcpy(s->col.wall_origin, c->wall_origin, sizeof(c->wall_origin));
    memcpy(s->col.wall_normal, c->wall_normal, sizeof(c->wall_normal));
    s->col.use_sphere = c->use_sphere;
    memcpy(s->col.sphere_center, c->sphere_center, sizeof(c->sphere_center));
    s->col.sphere_radius = c->sphere_radius;
    size_t nv = (size_t)(V > 0 ? V : 1);
    s->pos = (V3*)calloc(nv, sizeof(V3)); s->snap = (V3*)calloc(nv, sizeof(V3)); s->prev = (V3*)calloc(nv, sizeof(V3));
    s->vel = (V3*)calloc(nv, sizeof(V3)); s->rest = (V3*)calloc(nv, sizeof(V3));
    s->w = (float*)calloc(nv, sizeof(float)); s->inv = (float*)calloc(nv, sizeof(float));
    s->pin_w = (float*)malloc(nv * sizeof(float)); s->pin_t = (V3*)calloc(nv, sizeof(V3)); s->pin_relax = (float*)calloc(nv, sizeof(float));
    s->pin_relax_iter = -1;
    for (int i = 0; i < V; ++i) {
        s->rest[i] = v3(mesh->positions[3 * i], mesh->positions[3 * i + 1], mesh->positions[3 * i + 2]);
        s->pos[i] = s->prev[i] = s->rest[i];
        s->inv[i] = mesh->inv_mass[i];
        s->w[i] = s->inv[i] > 0.0f ? s->inv[i] : 0.0f;
        s->pin_w[i] = -1.0f;
    }
    int* sp = (int*)xcalloc((size_t)E * 2, sizeof(int));
    float* spr = (float*)xcalloc((size_t)E, sizeof(float));
    s->edges = (int*)xcalloc((size_t)E * 2, sizeof(int));
    for (int e = 0; e < E; ++e) {
        int i = mesh->edges ? mesh->edges[2 * e] : 0, j = mesh->edges ? mesh->edges[2 * e + 1] : 0;
        sp[2 * e] = i > 0 ? i : 0; sp[2 * e + 1] = j > 0 ? j : 0;
        spr[e] = mesh->edge_rest_lengths ? mesh->edge_rest_lengths[e] : 0.0f;
        s->edges[2 * e] = sp[2 * e]; s->edges[2 * e + 1] = sp[2 * e + 1];
    }
    build_csr(V, sp, spr, E, &s->sp_off, &s->sp_other, &s->sp_side, &s->sp_rest);
    s->pcg_on = c->stretch_optimization_enabled;
    s->strength = c->stretch_optimization_strength;
    if (s->pcg_on) {
        if (s->sp_off[V] == 0) { free(sp); free(spr); set_err("PCG stretch optimization found no valid CSR edges"); oracle_destroy(s); return NULL; }
        s->diag = (float*)calloc(nv * 6, sizeof(float)); s->pinv = (float*)calloc(nv * 6, sizeof(float));
        s->r = (V3*)calloc(nv, sizeof(V3)); s->z = (V3*)calloc(nv, sizeof(V3)); s->d = (V3*)calloc(nv, sizeof(V3)); s->q = (V3*)calloc(nv, sizeof(V3));
        s->off = (float*)calloc((size_t)s->sp_off[V] * 4 + 4, sizeof(float));
        s->avg_sum = (V3*)calloc(nv, sizeof(V3)); s->avg_cnt = (float*)calloc(nv, sizeof(float));
        s->cap_edges = (int*)xcalloc((size_t)E * 2, sizeof(int)); s->cap_rest = (float*)xcalloc((size_t)E, sizeof(float));
        if (c->edge_color_count > 0 && mesh->edge_color_offsets) {
            s->n_cap_colors = c->edge_color_count;
            s->cap_colors = (int*)malloc(sizeof(int) * (size_t)(s->n_cap_colors + 1));
            memcpy(s->cap_colors, mesh->edge_color_offsets, sizeof(int) * (size_t)(s->n_cap_colors + 1));
            memcpy(s->cap_edges, sp, sizeof(int) * 2 * (size_t)E); memcpy(s->cap_rest, spr, sizeof(float) * (size_t)E);
        } else {
            /* no colouring: each cap pass is one Jacobi pass over all edges */
            s->cap_jacobi = 1;
            s->snap_prev = (V3*)xcalloc(nv, sizeof(V3));
        }
    }
    free(sp); free(spr);
    build_csr(V, L > 0 ? mesh->lra_edges : NULL, L > 0 ? mesh->lra_rest_lengths : NULL, L, &s->te_off, &s->te_other, &s->te_side, &s->te_rest);
    s->bends = (int*)xcalloc((size_t)B * 2, sizeof(int));
    s->bend_rest = (float*)xcalloc((size_t)B, sizeof(float));
    if (B > 0) { memcpy(s->bends, mesh->bends, sizeof(int) * 2 * (size_t)B); memcpy(s->bend_rest, mesh->bend_rest_lengths, sizeof(float) * (size_t)B); }
    if (c->bend_color_count > 0) {
        if (!mesh->bend_color_offsets) { set_err("ABI41 bend color offsets are required"); oracle_destroy(s); return NULL; }
        s->n_bend_colors = c->bend_color_count;
        s->bend_colors = (int*)malloc(sizeof(int) * (size_t)(c->bend_color_count + 1));
        memcpy(s->bend_colors, mesh->bend_color_offsets, sizeof(int) * (size_t)(c->bend_color_count + 1));
    } else if (B > 0) {
        build_csr(V, s->bends, s->bend_rest, B, &s->bj_off, &s->bj_other, &s->bj_side, &s->bj_rest);
    }
    s->tris = (int*)xcalloc((size_t)T * 3, sizeof(int));
    for (int k = 0; k < T * 3; ++k) { int v = mesh->triangles ? mesh->triangles[k] : 0; s->tris[k] = v > 0 ? v : 0; }
    /* self collision sizing (abi41.cu:4542-4548, 6784-6994) */
    float req = fmaxf(c->self_collision_distance, 0.0f);
    s->radius = req > 0.0f ? req : fmaxf(fmaxf(c->cloth_thickness, c->collision_margin), 0.0f);
    s->self_on = c->self_collision != 0;
    if (s->self_on && s->radius > 0.0f) {
        s->cell = fmaxf(s->radius * 1.8f, 1.0e-3f);
        s->vhash = V >= 128; s->thash = T >= 64; s->ehash = E >= 64;
        s->nvb = s->vhash ? next_pow2(V * 4 > 1024 ? V * 4 : 1024) : 0;
        s->ntb = s->thash ? next_pow2(T * 4 > 1024 ? T * 4 : 1024) : 0;
        s->neb = s->ehash ? next_pow2(E * 4 > 1024 ? E * 4 : 1024) : 0;
        s->nb_count = (int*)calloc(nv, sizeof(int));
        s->nb_idx = (int*)calloc(nv * NB_SLOTS, sizeof(int));
        s->acc = (long long*)calloc(nv * 4, sizeof(long long));
        if (s->vhash) { s->vcell = (int*)calloc(nv * 4, sizeof(int)); s->vb_start = (int*)calloc((size_t)s->nvb + 1, sizeof(int)); s->vb_ent = (int*)calloc(nv, sizeof(int)); }
        if (s->thash) { s->tb_start = (int*)calloc((size_t)s->ntb + 1, sizeof(int)); s->tb_ent = (int*)calloc((size_t)T * MAX_PRIM_CELLS, sizeof(int)); }
        if (s->ehash) { s->eb_start = (int*)calloc((size_t)s->neb + 1, sizeof(int)); s->eb_ent = (int*)calloc((size_t)E * MAX_PRIM_CELLS, sizeof(int)); }
    }
    /* vertex -> incident triangles in triangle order */
    s->vt_off = (int*)calloc(nv + 1, sizeof(int));
    for (int t = 0; t < T; ++t)
        for (int a = 0; a < 3; ++a) { int id = s->tris[3 * t + a]; if (id >= 0 && id < V) s->vt_off[id + 1]++; }
    for (int i = 0; i < V; ++i) s->vt_off[i + 1] += s->vt_off[i];
    s->vt_tri = (int*)xcalloc((size_t)s->vt_off[V] + 1, sizeof(int));
    {
        int* cur = (int*)calloc(nv + 1, sizeof(int));
        memcpy(cur, s->vt_off, sizeof(int) * (size_t)V);
        for (int t = 0; t < T; ++t)
            for (int a = 0; a < 3; ++a) { int id = s->tris[3 * t + a]; if (id >= 0 && id < V) s->vt_tri[cur[id]++] = t; }
        free(cur);
    }
    /* volume pressure (abi41.cu:7413-7584, 8816-8903) */
    s->pressure_on = c->use_volume_pressure && c->pressure_strength > 0.0f && isfinite(c->pressure_strength);
    s->p_strength = fmaxf(c->pressure_strength, 0.0f);
    s->p_accel = env_scale("SSBL_ABI41_PRESSURE_UI_ACCEL_SCALE", 1792.0f, 1.0f, 8192.0f);
    s->p_impulse = env_scale("SSBL_ABI41_PRESSURE_IMPULSE_REST_SCALE", 0.85f, 0.05f, 8.0f);
    s->p_vrest = env_scale("SSBL_ABI41_PRESSURE_VELOCITY_REST_SCALE", 2.25f, 0.10f, 16.0f);
    if (s->pressure_on) {
        float objs = env_scale("SSBL_ABI41_PRESSURE_VELOCITY_OBJECT_SCALE", 0.08f, 0.005f, 1.0f);
        s->p_area = (float*)calloc(nv, sizeof(float));
        s->p_rest = (float*)calloc(nv, sizeof(float));
        pressure_prep(s, mesh, objs);
    }
    int nst = config->static_triangle_count > 0 ? config->static_triangle_count : 0;
    if (!build_sdf(s, mesh->static_triangles, nst)) { oracle_destroy(s); return NULL; }
    return s;
}

int oracle_update_pin_targets(OracleSolver* s, const int* idx, const float* pos, const float* wts, int count) {
    if (!s) return set_err("invalid solver handle");
    if (count < 0) return set_err("invalid pin count");
    if (count > 0 && (!idx || !pos)) return set_err("pin arrays are required when pin count is nonzero");
    for (int i = 0; i < s->V; ++i) s->pin_w[i] = -1.0f;
    for (int k = 0; k < count; ++k) {
        int i = idx[k];
        if (i < 0 || i >= s->V) continue;
        s->pin_w[i] = wts ? wts[k] : 1.0f;
        s->pin_t[i] = v3(pos[3 * k], pos[3 * k + 1], pos[3 * k + 2]);
    }
    s->pin_relax_iter = -1;
    return 1;
}

int oracle_update_runtime_colliders(OracleSolver* s, const SsblXpbdRuntimeColliders* c) {
    if (!s || !c) return set_err("invalid runtime collider update");
    s->col = *c;
    return 1;
}

int oracle_update_positions(OracleSolver* s, const float* p, int max_floats) {
    if (!s || !p || max_floats < s->V * 3) return set_err("invalid position upload");
    for (int i = 0; i < s->V; ++i) s->pos[i] = s->prev[i] = v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    return 1;
}

int oracle_update_static_triangles(OracleSolver* s, const float* tris, int count) {
    if (!s) return set_err("invalid static triangle update");
    if (count < 0) count = 0;
    if (count > 0 && !tris) return set_err("static triangle data is required when triangle count is nonzero");
    return build_sdf(s, tris, count);
}

/* ------------------------------------------------- dynamic colliders -- */
struct OracleScene {
    ODyn d;
    float margin, thickness;
    long long overflow;
};

static void odyn_free(ODyn* d) {
    void* p[] = {d->dt_tri, d->dt_min, d->dt_max, d->dt_center, d->dt_prev_center, d->dt_radius, d->dt_cmin, d->dt_cmax,
                 d->dt_start, d->dt_ent, d->dt_large, d->dt_idx, d->dp_pos, d->dp_prev, d->dp_rad, d->dp_cellc, d->dp_start,
                 d->dp_ent, d->tri_src, d->tri_layer, d->par_src, d->par_layer};
    for (size_t k = 0; k < sizeof(p) / sizeof(p[0]); ++k) free(p[k]);
    memset(d, 0, sizeof(*d));
}

/* Triangle rows, bounds, centres, radii and cell spans grown by the collision
 * margin (abi41.cu:3686-3760); hash with members in increasing id order and
 * the large list (spans over 64 cells) in id order (abi41.cu:3763-3930,
 * 6220-6392). */
static void dyn_tri_finish(ODyn* d, float margin_in, int T, int signed_mode, int motion, float cell) {
    size_t n = (size_t)T;
    if (motion) memcpy(d->dt_prev_center, d->dt_center, sizeof(V3) * n);
    d->dt_min = (V3*)realloc(d->dt_min, sizeof(V3) * n); d->dt_max = (V3*)realloc(d->dt_max, sizeof(V3) * n);
    d->dt_center = (V3*)realloc(d->dt_center, sizeof(V3) * n); d->dt_radius = (float*)realloc(d->dt_radius, sizeof(float) * n);
    if (!motion) d->dt_prev_center = (V3*)realloc(d->dt_prev_center, sizeof(V3) * n);
    d->dt_cmin = (int*)realloc(d->dt_cmin, sizeof(int) * 3 * n); d->dt_cmax = (int*)realloc(d->dt_cmax, sizeof(int) * 3 * n);
    const int hashed = T >= 64;
    const float margin = fmaxf(margin_in, 0.0f);
    for (int t = 0; t < T; ++t) {
        V3 a = d->dt_tri[3 * t], b = d->dt_tri[3 * t + 1], c = d->dt_tri[3 * t + 2];
        V3 lo = v3(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)));
        V3 hi = v3(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)));
        V3 ce = vmul(vadd(vadd(a, b), c), 1.0f / 3.0f);
        V3 da = vsub(a, ce), db = vsub(b, ce), dc = vsub(c, ce);
        d->dt_min[t] = lo; d->dt_max[t] = hi; d->dt_center[t] = ce;
        d->dt_radius[t] = sqrtf(fmaxf(fmaxf(vdot(da, da), vdot(db, db)), vdot(dc, dc)));
        if (!hashed) continue;
        float cs = fmaxf(cell, 1.0e-3f);
        int x0 = cell_of(lo.x - margin, cs), y0 = cell_of(lo.y - margin, cs), z0 = cell_of(lo.z - margin, cs);
        int x1 = cell_of(hi.x + margin, cs), y1 = cell_of(hi.y + margin, cs), z1 = cell_of(hi.z + margin, cs);
        long long sx = (long long)x1 - x0 + 1, sy = (long long)y1 - y0 + 1, sz = (long long)z1 - z0 + 1;
        if (!(sx > 0 && sy > 0 && sz > 0)) {
            x0 = x1 = cell_of(ce.x, cs); y0 = y1 = cell_of(ce.y, cs); z0 = z1 = cell_of(ce.z, cs);
        }
        int* m0 = d->dt_cmin + 3 * t; int* m1 = d->dt_cmax + 3 * t;
        m0[0] = x0; m0[1] = y0; m0[2] = z0; m1[0] = x1; m1[1] = y1; m1[2] = z1;
    }
    if (!motion) memcpy(d->dt_prev_center, d->dt_center, sizeof(V3) * n);
    d->dt_n = T; d->dt_signed = signed_mode; d->dt_motion = motion; d->dt_hashed = hashed; d->dt_cell = cell;
    d->dt_large_n = 0; d->dt_max_occ = 0; d->dt_nb = 0;
    if (!hashed) return;
    const int nb = next_pow2(T * 4 > 1024 ? T * 4 : 1024);
    d->dt_nb = nb;
    d->dt_start = (int*)realloc(d->dt_start, sizeof(int) * ((size_t)nb + 1));
    d->dt_large = (int*)realloc(d->dt_large, sizeof(int) * n);
    int* count = (int*)calloc((size_t)nb, sizeof(int));
    for (int pass = 0; pass < 2; ++pass) {
        for (int t = 0; t < T; ++t) {
            const int* m0 = d->dt_cmin + 3 * t; const int* m1 = d->dt_cmax + 3 * t;
            long long sx = (long long)m1[0] - m0[0] + 1, sy = (long long)m1[1] - m0[1] + 1, sz = (long long)m1[2] - m0[2] + 1;
            long long cells = (sx > 0 && sy > 0 && sz > 0) ? sx * sy * sz : 0;
            if (cells <= 0) continue;
            if (cells > MAX_PRIM_CELLS) {
                if (pass == 0) d->dt_large[d->dt_large_n++] = t;
                continue;
            }
            for (int z = m0[2]; z <= m1[2]; ++z)
                for (int y = m0[1]; y <= m1[1]; ++y)
                    for (int x = m0[0]; x <= m1[0]; ++x) {
                        unsigned b = bucket_of(x, y, z, nb);
                        if (pass == 0) count[b]++;
                        else d->dt_ent[count[b]++] = t;
                    }
        }
        if (pass == 0) {
            int total = 0;
            for (int b = 0; b < nb; ++b) {
                if (count[b] > d->dt_max_occ) d->dt_max_occ = count[b];
                d->dt_start[b] = total; total += count[b]; count[b] = d->dt_start[b];
            }
            d->dt_start[nb] = total;
            d->dt_ent = (int*)realloc(d->dt_ent, sizeof(int) * (size_t)(total > 0 ? total : 1));
        }
    }
    free(count);
}

static float dyn_tri_cell(float margin_in, float thick_in, float max_extent, int indexed) {
    float margin = fmaxf(margin_in, 0.0f), thick = fmaxf(thick_in, 0.0f);
    float ext = fmaxf(fmaxf(max_extent + margin * 2.0f, thick), 1.0e-3f);
    if (!indexed) return ext;
    float fine = fmaxf(fmaxf(thick * 1.5f, margin * 4.0f), 0.02f);
    return fmaxf(fminf(ext, fine), 1.0e-3f);
}

static float tri_extent3(V3 a, V3 b, V3 c) {
    float e = fmaxf(fmaxf(a.x, fmaxf(b.x, c.x)) - fminf(a.x, fminf(b.x, c.x)),
                    fmaxf(fmaxf(a.y, fmaxf(b.y, c.y)) - fminf(a.y, fminf(b.y, c.y)),
                          fmaxf(a.z, fmaxf(b.z, c.z)) - fminf(a.z, fminf(b.z, c.z))));
    return e;
}

static void dyn_tri_clear(ODyn* d) {
    d->dt_n = 0; d->dt_signed = 0; d->dt_motion = 0; d->dt_hashed = 0; d->dt_upload = 0; d->dt_large_n = 0; d->dt_max_occ = 0;
}

/* abi41.cu:8333-8413 */
static float rows_extent(const float* tris, int count) {
    float max_extent = 0.0f;
    for (int t = 0; t < count; ++t) {
        float e = tri_extent3(f3a(tris + 9 * t), f3a(tris + 9 * t + 3), f3a(tris + 9 * t + 6));
        if (isfinite(e) && e >= 0.0f) max_extent = fmaxf(max_extent, e);
    }
    return max_extent;
}

static void dyn_put_rows(ODyn* d, const float* tris, int count) {
    d->dt_tri = (V3*)realloc(d->dt_tri, sizeof(V3) * 3 * (size_t)count);
    for (int q = 0; q < 3 * count; ++q) d->dt_tri[q] = f3a(tris + 3 * q);
}

int oracle_update_dynamic_triangles(OracleSolver* s, const float* tris, int count) {
    if (!s) return set_err("invalid dynamic triangle update");
    ODyn* d = &s->own;
    if (count < 0) count = 0;
    if (count == 0) { dyn_tri_clear(d); return 1; }
    if (!tris) return set_err("dynamic triangle data is required when triangle count is nonzero");
    float max_extent = rows_extent(tris, count);
    int motion = d->dt_upload == count;
    dyn_put_rows(d, tris, count);
    dyn_tri_finish(d, s->cfg.collision_margin, count, 0, motion, dyn_tri_cell(s->cfg.collision_margin, s->cfg.cloth_thickness, max_extent, 0));
    d->dt_upload = count;
    return 1;
}

/* abi41.cu:8415-8564, rows from indices 3663-3684 */
int oracle_update_dynamic_indexed(OracleSolver* s, const float* verts, int vcount, const int* idx, int count, int topology_changed) {
    if (!s) return set_err("invalid dynamic indexed triangle update");
    ODyn* d = &s->own;
    if (vcount < 0) vcount = 0;
    if (count < 0) count = 0;
    if (vcount == 0 || count == 0) { dyn_tri_clear(d); return 1; }
    if (!verts || !idx) return set_err("dynamic indexed triangle positions and indices are required when count is nonzero");
    float max_extent = 0.0f;
    for (int t = 0; t < count; ++t) {
        int a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
        if (a < 0 || b < 0 || c < 0 || a >= vcount || b >= vcount || c >= vcount) continue;
        float e = tri_extent3(f3a(verts + 3 * a), f3a(verts + 3 * b), f3a(verts + 3 * c));
        if (isfinite(e) && e >= 0.0f) max_extent = fmaxf(max_extent, e);
    }
    if (topology_changed || count != d->dt_idx_n || !d->dt_idx) {
        d->dt_idx = (int*)realloc(d->dt_idx, sizeof(int) * 3 * (size_t)count);
        memcpy(d->dt_idx, idx, sizeof(int) * 3 * (size_t)count);
        d->dt_idx_n = count;
    }
    int motion = !topology_changed && d->dt_upload == count;
    d->dt_tri = (V3*)realloc(d->dt_tri, sizeof(V3) * 3 * (size_t)count);
    for (int t = 0; t < count; ++t) {
        int a = d->dt_idx[3 * t], b = d->dt_idx[3 * t + 1], c = d->dt_idx[3 * t + 2];
        if (a < 0 || b < 0 || c < 0 || a >= vcount || b >= vcount || c >= vcount) {
            d->dt_tri[3 * t] = d->dt_tri[3 * t + 1] = d->dt_tri[3 * t + 2] = v3(0.0f, 0.0f, 0.0f);
            continue;
        }
        d->dt_tri[3 * t] = f3a(verts + 3 * a); d->dt_tri[3 * t + 1] = f3a(verts + 3 * b); d->dt_tri[3 * t + 2] = f3a(verts + 3 * c);
    }
    dyn_tri_finish(d, s->cfg.collision_margin, count, 1, motion, dyn_tri_cell(s->cfg.collision_margin, s->cfg.cloth_thickness, max_extent, 1));
    d->dt_upload = count;
    return 1;
}

/* abi41.cu:584-603 (radius signature), 8566-8696, hash 6395-6449.  prev:
 * the caller's previous positions (shared scene) or NULL to keep the last
 * upload's positions as previous.  Returns the particles past the 16 queried
 * slots of their buckets. */
static long long dyn_put_particles(ODyn* d, float margin, float thickness, const float* pos, const float* prev, const float* radii,
                                   int count) {
    uint64_t sig = 1469598103934665603ull ^ (uint64_t)count;
    float max_r = 0.0f;
    for (int q = 0; q < count; ++q) {
        float r = isfinite(radii[q]) ? radii[q] : 0.0f;
        r = fmaxf(r, 0.0f);
        max_r = fmaxf(max_r, r);
        uint32_t bits; memcpy(&bits, &r, 4);
        sig ^= (uint64_t)bits; sig *= 1099511628211ull;
    }
    if (d->dp_cell <= 0.0f || d->dp_sig != sig || d->dp_upload != count) {
        d->dp_cell = fmaxf(fmaxf(max_r + fmaxf(margin, 0.0f), fmaxf(thickness, 0.0f)), 1.0e-3f);
        d->dp_sig = sig;
    }
    int motion = d->dp_upload == count;
    size_t n = (size_t)count;
    if (prev) {
        d->dp_prev = (V3*)realloc(d->dp_prev, sizeof(V3) * n);
        for (int q = 0; q < count; ++q) d->dp_prev[q] = f3a(prev + 3 * q);
    } else if (motion) {
        memcpy(d->dp_prev, d->dp_pos, sizeof(V3) * n);
    } else {
        d->dp_prev = (V3*)realloc(d->dp_prev, sizeof(V3) * n);
    }
    d->dp_pos = (V3*)realloc(d->dp_pos, sizeof(V3) * n); d->dp_rad = (float*)realloc(d->dp_rad, sizeof(float) * n);
    for (int q = 0; q < count; ++q) { d->dp_pos[q] = f3a(pos + 3 * q); d->dp_rad[q] = radii[q]; }
    if (!prev && !motion) memcpy(d->dp_prev, d->dp_pos, sizeof(V3) * n);
    d->dp_n = count; d->dp_motion = motion; d->dp_hashed = count >= 128; d->dp_nb = 0;
    long long overflow = 0;
    if (d->dp_hashed) {
        int nb = next_pow2(count * 4 > 1024 ? count * 4 : 1024);
        d->dp_nb = nb;
        d->dp_cellc = (int*)realloc(d->dp_cellc, sizeof(int) * 3 * n);
        d->dp_start = (int*)realloc(d->dp_start, sizeof(int) * ((size_t)nb + 1));
        d->dp_ent = (int*)realloc(d->dp_ent, sizeof(int) * n);
        int* cntb = (int*)calloc((size_t)nb, sizeof(int));
        unsigned* bk = (unsigned*)malloc(sizeof(unsigned) * n);
        for (int q = 0; q < count; ++q) {
            int* c = d->dp_cellc + 3 * q;
            c[0] = cell_of(d->dp_pos[q].x, d->dp_cell); c[1] = cell_of(d->dp_pos[q].y, d->dp_cell); c[2] = cell_of(d->dp_pos[q].z, d->dp_cell);
            bk[q] = bucket_of(c[0], c[1], c[2], nb);
            cntb[bk[q]]++;
        }
        int total = 0;
        for (int b = 0; b < nb; ++b) {
            if (cntb[b] > 16) overflow += cntb[b] - 16;
            d->dp_start[b] = total; total += cntb[b]; cntb[b] = d->dp_start[b];
        }
        d->dp_start[nb] = total;
        for (int q = 0; q < count; ++q) d->dp_ent[cntb[bk[q]]++] = q;
        free(bk); free(cntb);
    }
    d->dp_upload = count;
    return overflow;
}

static void dyn_clear_particles(ODyn* d) { d->dp_n = 0; d->dp_motion = 0; d->dp_hashed = 0; d->dp_upload = 0; d->dp_sig = 0; }

int oracle_update_dynamic_particles(OracleSolver* s, const float* pos, const float* radii, int count) {
    if (!s) return set_err("invalid dynamic particle update");
    if (count < 0) count = 0;
    if (count == 0) { dyn_clear_particles(&s->own); return 1; }
    if (!pos || !radii) return set_err("dynamic particle position/radius data is required when particle count is nonzero");
    dyn_put_particles(&s->own, s->cfg.collision_margin, s->cfg.cloth_thickness, pos, NULL, radii, count);
    return 1;
}

/* ---- shared scene (abi41.cu:6597-6784, 8733-8789) ---- */
OracleScene* oracle_scene_create(void) { return (OracleScene*)calloc(1, sizeof(OracleScene)); }

void oracle_scene_destroy(OracleScene* g) {
    if (!g) return;
    odyn_free(&g->d);
    free(g);
}

static int* copy_ints(int* dst, const int* src, int n) {
    dst = (int*)realloc(dst, sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (n > 0) memcpy(dst, src, sizeof(int) * (size_t)n);
    return dst;
}

int oracle_scene_update(OracleScene* g, const SsblXpbdGlobalDynamicSceneInputs* in) {
    if (!g || !in) return set_err("invalid global dynamic scene update");
    int P = in->particle_count > 0 ? in->particle_count : 0, T = in->triangle_count > 0 ? in->triangle_count : 0;
    if (P > 0 && (!in->particle_positions || !in->particle_radii || !in->particle_source_ids || !in->particle_collision_layers))
        return set_err("global dynamic particle arrays are incomplete");
    if (T > 0 && (!in->triangle_vertices || !in->triangle_source_ids || !in->triangle_collision_layers))
        return set_err("global dynamic triangle arrays are incomplete");
    g->margin = fmaxf(in->collision_margin, 0.0f);
    g->thickness = fmaxf(in->cloth_thickness, 0.0f);
    g->overflow = 0;
    ODyn* d = &g->d;
    if (P == 0) {
        dyn_clear_particles(d);
    } else {
        d->par_src = copy_ints(d->par_src, in->particle_source_ids, P);
        d->par_layer = copy_ints(d->par_layer, in->particle_collision_layers, P);
        g->overflow += dyn_put_particles(d, g->margin, g->thickness, in->particle_positions,
                                         in->particle_prev_positions ? in->particle_prev_positions : in->particle_positions,
                                         in->particle_radii, P);
    }
    if (T == 0) {
        dyn_tri_clear(d);
    } else {
        d->tri_src = copy_ints(d->tri_src, in->triangle_source_ids, T);
        d->tri_layer = copy_ints(d->tri_layer, in->triangle_collision_layers, T);
        int motion = d->dt_upload == T;
        dyn_put_rows(d, in->triangle_vertices, T);
        dyn_tri_finish(d, g->margin, T, 0, motion, dyn_tri_cell(g->margin, g->thickness, rows_extent(in->triangle_vertices, T), 1));
        d->dt_upload = T;
    }
    return 1;
}

int oracle_scene_attach(OracleSolver* s, OracleScene* g, int target_source_id, int target_collision_layer, int mode) {
    if (!s || !g) return set_err("invalid global dynamic scene attach");
    s->scene = g;
    s->gd_src = target_source_id;
    s->gd_layer = target_collision_layer;
    s->gd_mode = mode;
    return 1;
}

int oracle_scene_clear(OracleSolver* s) {
    if (!s) return set_err("invalid global dynamic scene clear");
    s->scene = NULL;
    s->gd_src = s->gd_layer = s->gd_mode = 0;
    return 1;
}

long long oracle_scene_overflow(const OracleScene* g) { return g ? g->overflow : 0; }

/* abi41.cu:3984-3997 */
static int source_enabled(const OracleSolver* s, int source, int layer) {
    if (s->gd_mode == 0) return 1;
    if (s->gd_src != 0 && source == s->gd_src) return 0;
    if (s->gd_mode == 2) return layer < s->gd_layer;
    return 1;
}

typedef struct { V3 delta, vel, acc; float pen, dist, acc_w; } DynBest;

/* abi41.cu:3998-4111 */
static void dyn_tri_candidate(OracleSolver* s, const ODyn* ds, int t, V3 p, float cdt, int inside, float qm, float cm, DynBest* b, unsigned* cand,
                              unsigned* rej) {
    if (t < 0 || t >= ds->dt_n) return;
    if (ds->tri_src && !source_enabled(s, ds->tri_src[t], ds->tri_layer ? ds->tri_layer[t] : 0)) return;
    *cand += 1;
    V3 lo = ds->dt_min[t], hi = ds->dt_max[t];
    V3 q = v3(fminf(fmaxf(p.x, lo.x), hi.x), fminf(fmaxf(p.y, lo.y), hi.y), fminf(fmaxf(p.z, lo.z), hi.z));
    V3 dq = vsub(p, q);
    if (vdot(dq, dq) > qm * qm) { *rej += 1; return; }
    V3 dc = vsub(p, ds->dt_center[t]);
    float rr = ds->dt_radius[t] + qm;
    if (vdot(dc, dc) > rr * rr) { *rej += 1; return; }
    V3 a = ds->dt_tri[3 * t], bb = ds->dt_tri[3 * t + 1], c = ds->dt_tri[3 * t + 2];
    V3 cp = closest_on_tri(p, a, bb, c);
    V3 d = vsub(p, cp);
    float dsq = vdot(d, d), dist = sqrtf(fmaxf(dsq, K_EPS));
    V3 tn = vcross(vsub(bb, a), vsub(c, a));
    float tl = sqrtf(fmaxf(vdot(tn, tn), K_EPS));
    V3 trin = vmul(tn, 1.0f / tl);
    V3 normal = dsq > K_EPS * 4.0f ? vmul(d, 1.0f / fmaxf(dist, K_EPS)) : trin;
    float pen = cm - dist;
    if (ds->dt_signed) {
        float sd = vdot(d, trin);
        if (inside) {
            if (sd >= 0.001f) return;
            pen = 0.001f - sd;
        } else {
            pen = cm - sd;
        }
        normal = trin;
        if (pen <= 0.0f) return;
        V3 delta = vmul(normal, pen);
        if (!inside && vfinite(delta)) {
            float w = fmaxf(pen, K_EPS);
            b->acc = vadd(b->acc, vmul(delta, w));
            b->acc_w += w;
        }
        if (dist < b->dist) {
            V3 vel = v3(0.0f, 0.0f, 0.0f);
            if (ds->dt_motion && cdt > K_EPS) vel = vmul(vsub(ds->dt_center[t], ds->dt_prev_center[t]), 1.0f / cdt);
            b->dist = dist; b->pen = pen; b->delta = delta; b->vel = vel;
        }
    } else {
        if (dist >= cm) return;
        if (pen > b->pen) { b->pen = pen; b->delta = vmul(normal, pen); }
    }
}

/* abi41.cu:979-994 */
static V3 dyn_local_average(V3 acc, float w, V3 fb) {
    if (w > 0.0f && vfinite(acc)) {
        V3 avg = vmul(acc, 1.0f / w);
        float al = vlen(avg), fl = vlen(fb);
        if (vfinite(avg) && isfinite(al) && isfinite(fl) && al > K_EPS && fl > K_EPS) return vmul(avg, fl / al);
    }
    return fb;
}

/* abi41.cu:996-1065 */
static void dyn_signed_response(OracleSolver* s, int i, V3 p, V3 raw, V3 cvel, float proxy, float dt, int inside) {
    if (!vfinite(p) || !vfinite(raw)) return;
    float rl = vlen(raw);
    if (!isfinite(rl) || rl <= K_EPS) return;
    V3 n = vmul(raw, 1.0f / rl);
    float basis = fmaxf(fmaxf(s->cfg.cloth_thickness, 0.0f), fmaxf(s->cfg.collision_margin, 0.0f));
    float cap = inside ? fmaxf(3.0e-3f, basis * 16.0f) : fmaxf(5.0e-4f, basis * 3.0f);
    V3 applied = limit_delta(vmul(raw, 1.0f / 3.0f), cap);
    float al = vlen(applied);
    if (!isfinite(al) || al <= K_EPS) return;
    float sdt = fmaxf(dt, K_EPS);
    V3 corrected = vadd(p, applied);
    V3 vel = s->vel[i];
    V3 base = v3(0.0f, 0.0f, 0.0f);
    if (vfinite(cvel)) {
        float cn = vdot(cvel, n);
        if (isfinite(cn)) base = vmul(n, cn);
    }
    if (inside) {
        if (!vfinite(vel)) vel = v3(0.0f, 0.0f, 0.0f);
        V3 rel = vsub(vel, base);
        float ns = vdot(rel, n);
        if (isfinite(ns) && ns < 0.0f) { rel = vsub(rel, vmul(n, ns)); vel = vadd(base, rel); }
    } else {
        V3 rel = vsub(vel, base);
        float inward = fmaxf(-vdot(rel, n), 0.0f);
        float depth = fmaxf(fmaxf(proxy, rl), al);
        contact_response(s, n, inward + depth / sdt, &rel);
        float out = vdot(rel, n);
        if (out > 0.0f) rel = vsub(rel, vmul(n, out * (1.0f - 1.0f / 8.0f)));
        vel = vadd(base, rel);
    }
    if (!vfinite(vel)) vel = v3(0.0f, 0.0f, 0.0f);
    s->pos[i] = corrected;
    s->vel[i] = vel;
    s->prev[i] = vsub(corrected, vmul(vel, sdt));
}

/* abi41.cu:4114-4323 (query and response of one vertex) */
static void dyn_triangles(OracleSolver* s, const ODyn* ds, int i, int inside, unsigned* cand, unsigned* rej) {
    const float sub_dt = s->dyn_sub_dt;
    const float cdt = (isfinite(s->cfg.dt) && s->cfg.dt > K_EPS) ? s->cfg.dt : fmaxf(sub_dt, K_EPS);
    float cm = fmaxf(s->cfg.collision_margin, 0.0f);
    if (ds->dt_signed) cm = fmaxf(cm, fmaxf(s->cfg.cloth_thickness, 0.0f) * 0.75f);
    float qm = cm;
    if (ds->dt_signed) {
        float animated = fmaxf(fmaxf(cm * 2.0f, 0.04f), fmaxf(ds->dt_cell, 0.0f) * 1.25f);
        qm = fminf(fmaxf(animated, cm), 0.08f);
    }
    if (cm <= 0.0f || qm <= 0.0f) return;
    V3 p = s->pos[i];
    DynBest b = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, 0.0f, 3.402823466e+38f, 0.0f};
    if (ds->dt_hashed) {
        int cx = cell_of(p.x, ds->dt_cell), cy = cell_of(p.y, ds->dt_cell), cz = cell_of(p.z, ds->dt_cell);
        int R = 0;
        if (ds->dt_signed) {
            if (!inside) R = 1;
            else { float cs = fmaxf(ds->dt_cell, 1.0e-3f); R = clampi((int)ceilf(fmaxf(qm, 0.0f) / cs), 1, 4); }
        }
        for (int dz = -R; dz <= R; ++dz)
            for (int dy = -R; dy <= R; ++dy)
                for (int dx = -R; dx <= R; ++dx) {
                    int qx = cx + dx, qy = cy + dy, qz = cz + dz;
                    unsigned bk = bucket_of(qx, qy, qz, ds->dt_nb);
                    int s0 = ds->dt_start[bk], s1 = ds->dt_start[bk + 1];
                    if (s1 < s0) s1 = s0;
                    for (int k = s0; k < s1; ++k) {
                        int t = ds->dt_ent[k];
                        if (t < 0 || t >= ds->dt_n) continue;
                        const int* lo = ds->dt_cmin + 3 * t; const int* hi = ds->dt_cmax + 3 * t;
                        if (qx != clampi(cx, lo[0], hi[0]) || qy != clampi(cy, lo[1], hi[1]) || qz != clampi(cz, lo[2], hi[2])) continue;
                        dyn_tri_candidate(s, ds, t, p, cdt, inside, qm, cm, &b, cand, rej);
                    }
                }
        for (int k = 0; k < ds->dt_large_n; ++k) dyn_tri_candidate(s, ds, ds->dt_large[k], p, cdt, inside, qm, cm, &b, cand, rej);
    } else {
        for (int t = 0; t < ds->dt_n; ++t) dyn_tri_candidate(s, ds, t, p, cdt, inside, qm, cm, &b, cand, rej);
    }
    if (!(b.pen > 0.0f)) return;
    cnt(s, C_TRI_PAIRS);
    if (ds->dt_signed) {
        dyn_signed_response(s, i, p, dyn_local_average(b.acc, b.acc_w, b.delta), b.vel, b.pen, sub_dt, inside);
    } else {
        V3 applied = vmul(b.delta, 0.5f);
        V3 np = vadd(p, applied);
        V3 vel = s->vel[i];
        float vn = vdot(vel, applied);
        if (vn < 0.0f) {
            float l2 = fmaxf(vdot(applied, applied), K_EPS);
            vel = vsub(vel, vmul(applied, 0.5f * vn / l2));
        }
        s->pos[i] = np;
        s->vel[i] = vel;
        s->prev[i] = vsub(np, vmul(vel, fmaxf(sub_dt, K_EPS)));
    }
    cnt(s, C_EXACT);
}

/* abi41.cu:4354-4511 */
static void dyn_particles(OracleSolver* s, const ODyn* ds, int i, unsigned* cand) {
    const float sub_dt = s->dyn_sub_dt;
    const float cdt = (isfinite(s->cfg.dt) && s->cfg.dt > K_EPS) ? s->cfg.dt : fmaxf(sub_dt, K_EPS);
    V3 p = s->pos[i];
    float margin = fmaxf(s->cfg.collision_margin, 0.0f);
    V3 bd = v3(0, 0, 0), bv = v3(0, 0, 0), acc = v3(0, 0, 0);
    float best = 0.0f, acc_w = 0.0f;
    int nq = 0;
    int list[27 * 16];
    if (ds->dp_hashed) {
        int cx = cell_of(p.x, ds->dp_cell), cy = cell_of(p.y, ds->dp_cell), cz = cell_of(p.z, ds->dp_cell);
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    int qx = cx + dx, qy = cy + dy, qz = cz + dz;
                    unsigned bk = bucket_of(qx, qy, qz, ds->dp_nb);
                    int s0 = ds->dp_start[bk], n = ds->dp_start[bk + 1] - s0;
                    if (n > 16) n = 16;
                    for (int k = 0; k < n; ++k) {
                        int q = ds->dp_ent[s0 + k];
                        const int* c = ds->dp_cellc + 3 * q;
                        if (c[0] != qx || c[1] != qy || c[2] != qz) continue;
                        list[nq++] = q;
                    }
                }
    }
    int total = ds->dp_hashed ? nq : ds->dp_n;
    for (int k = 0; k < total; ++k) {
        int q = ds->dp_hashed ? list[k] : k;
        if (ds->par_src && !source_enabled(s, ds->par_src[q], ds->par_layer ? ds->par_layer[q] : 0)) continue;
        V3 c = ds->dp_pos[q];
        float r = fmaxf(ds->dp_rad[q], 0.0f) + margin;
        if (r <= 0.0f) continue;
        V3 d = vsub(p, c);
        float dist = sqrtf(fmaxf(vdot(d, d), K_EPS));
        if (dist >= r) continue;
        *cand += 1;
        V3 n = dist > K_EPS ? vmul(d, 1.0f / dist) : v3(0.0f, 0.0f, 1.0f);
        float pen = r - dist;
        V3 delta = vmul(n, pen);
        if (ds->dt_signed && vfinite(delta)) {
            float w = fmaxf(pen, K_EPS);
            acc = vadd(acc, vmul(delta, w));
            acc_w += w;
        }
        if (pen > best) {
            V3 pv = v3(0, 0, 0);
            if (ds->dp_motion && cdt > K_EPS) pv = vmul(vsub(c, ds->dp_prev[q]), 1.0f / cdt);
            best = pen; bd = delta; bv = pv;
        }
    }
    if (!(best > 0.0f)) return;
    if (ds->dt_signed) dyn_signed_response(s, i, p, dyn_local_average(acc, acc_w, bd), bv, best, sub_dt, 0);
    else s->pos[i] = vadd(p, vmul(bd, 0.5f));
    cnt(s, C_EXACT);
    cnt(s, C_DP_CONTACTS);
}

/* One dynamic-collider stage over all vertices: which 0 unsigned triangles
 * and particles, 1 signed triangles and particles, 2 signed inside-only
 * triangles (abi41.cu:4250-4323, 4447-4538, 9234-9360). */
/* The colliders a stage reads: the unsigned stage the shared scene when one
 * is attached with a non-zero mode, else the cloth's own unsigned set; the
 * signed stages the cloth's own indexed mesh (abi41.cu:9234-9360). */
static const ODyn* stage_set(const OracleSolver* s, int which) {
    if (which == 0) {
        if (s->gd_mode != 0 && s->scene) return &s->scene->d;
        return (s->own.dt_n > 0 || s->own.dp_n > 0) && !s->own.dt_signed ? &s->own : NULL;
    }
    return (s->own.dt_n > 0 || s->own.dp_n > 0) && s->own.dt_signed ? &s->own : NULL;
}

static void dynamic_all(OracleSolver* s, int which) {
    const ODyn* d = stage_set(s, which);
    if (!d || (d->dt_n == 0 && d->dp_n == 0)) return;
    unsigned long long tc = 0, tr = 0, pc = 0;
#pragma omp parallel for schedule(static) reduction(+ : tc, tr, pc)
    for (int i = 0; i < s->V; ++i) {
        if (s->inv[i] <= 0.0f) continue;
        unsigned c = 0, r = 0, q = 0;
        if (d->dt_n > 0) dyn_triangles(s, d, i, which == 2, &c, &r);
        if (which != 2 && d->dp_n > 0) dyn_particles(s, d, i, &q);
        tc += c; tr += r; pc += q;
    }
    s->counts[C_DT_CAND] += tc;
    s->counts[C_DT_REJECT] += tr;
    s->counts[C_DP_CAND] += pc;
}

/* abi41.cu:3466-3477 */
static float soft_relax(float weight, float exponent) {
    if (!isfinite(weight) || weight < 0.05f) return 0.0f;
    float total = fminf(fmaxf(weight / 0.75f, 0.0f), 1.0f);
    if (total >= 1.0f) return 1.0f;
    float rem = fmaxf(1.0f - total, 0.0f);
    float r = 1.0f - powf(rem, fmaxf(exponent, 1.0e-4f));
    return isfinite(r) ? fminf(fmaxf(r, 0.0f), 1.0f) : total;
}

/* ssbl_step_solver_ex schedule (abi41.cu:9087-9398), stage by stage. */
int oracle_step(OracleSolver* s, int substeps, int iterations) {
    if (!s) return set_err("invalid solver handle");
    if (substeps < 1) substeps = 1;
    if (iterations < 1) iterations = 1;
    memset(s->counts, 0, sizeof(s->counts));
    s->max_delta = 0.0f;
    s->pcg_guard = 0;
    s->pcg_max_delta = 0.0f;
    memset(s->red, 0, sizeof(s->red));
    if (s->pin_relax_iter != iterations) {
        float ex = 1.0f / (float)(iterations + 1 > 1 ? iterations + 1 : 1);
        for (int i = 0; i < s->V; ++i) s->pin_relax[i] = soft_relax(s->pin_w[i], ex);
        s->pin_relax_iter = iterations;
    }
    const float dt = s->cfg.dt / (float)substeps;
    s->dyn_sub_dt = dt;
    const int analytic = s->col.use_ground || s->col.use_wall || s->col.use_sphere;
    const int sdf = s->sdf_ready;
    const int interval = s->cfg.self_collision_interval > 1 ? s->cfg.self_collision_interval : 1;
    for (int st = 0; st < substeps; ++st) {
        integrate_all(s, dt);
        pin_all(s, dt);
        for (int it = 0; it < iterations; ++it) {
            int last = it == iterations - 1, final_c = st == substeps - 1 && last;
            if (s->E > 0 && !s->pcg_on) spring_all(s, dt);
            if (s->pcg_on && last) hard_stretch(s, dt);
            if (final_c && s->L > 0) tether_all(s, dt);
            if (final_c && s->B > 0) { if (s->n_bend_colors > 0) bends_by_color(s, dt); else bends_jacobi(s, dt); }
            pin_all(s, dt);
            if (analytic) analytic_all(s, dt);
            if (sdf) sdf_all(s, dt);
            if (last) dynamic_all(s, 0);
            int self_run = s->self_on && s->cfg.self_collision && last && (((st + 1) % interval) == 0 || st == substeps - 1) &&
                           s->V > 0 && s->radius > 0.0f;
            if (self_run) self_collision(s);
            if (last) dynamic_all(s, 1);
            if (s->pcg_on && final_c && s->strength >= 0.95f) {
                caps(s, dt, 0, 2, 1);
                caps(s, dt, 2, 3, 0);
                caps(s, dt, 1, 3, 0);
            }
            if (final_c && stage_set(s, 1))
                for (int pass = 0; pass < 6; ++pass) dynamic_all(s, 2);
            if (analytic || sdf || last || self_run) pin_all(s, dt);
        }
        velocity_all(s, dt);
    }
    return 1;
}

int oracle_download_positions(OracleSolver* s, float* out, int max_floats) {
    if (!s || !out || max_floats < s->V * 3) return set_err("invalid position download");
    memcpy(out, s->pos, sizeof(V3) * (size_t)s->V);
    return 1;
}

int oracle_download_state(OracleSolver* s, float* p, float* q, float* v) {
    if (!s) return set_err("invalid solver handle");
    if (p) memcpy(p, s->pos, sizeof(V3) * (size_t)s->V);
    if (q) memcpy(q, s->prev, sizeof(V3) * (size_t)s->V);
    if (v) memcpy(v, s->vel, sizeof(V3) * (size_t)s->V);
    return 1;
}

int oracle_build_self_structures(OracleSolver* s) {
    if (!s) return set_err("invalid solver handle");
    if (!s->self_on || !s->nb_count) return set_err("self collision is not enabled for this solver");
    memset(s->counts, 0, sizeof(s->counts));
    build_hashes(s);
    neighbors_all(s);
    return 1;
}

long long oracle_read_buffer(OracleSolver* s, int which, void* out, long long max_bytes) {
    if (!s || !out) { set_err("invalid buffer read"); return -1; }
    const void* src = NULL;
    long long bytes = 0;
    switch (which) {
        case 3: src = s->vcell; bytes = 16ll * s->V; break;
        case 4: src = s->vb_start; bytes = 4ll * (s->nvb + 1); break;
        case 5: src = s->vb_ent; bytes = 4ll * s->V; break;
        case 6: src = s->tb_start; bytes = 4ll * (s->ntb + 1); break;
        case 7: src = s->tb_ent; bytes = 4ll * s->tb_total; break;
        case 8: src = s->eb_start; bytes = 4ll * (s->neb + 1); break;
        case 9: src = s->eb_ent; bytes = 4ll * s->eb_total; break;
        case 10: src = s->nb_count; bytes = 4ll * s->V; break;
        case 11: src = s->nb_idx; bytes = 4ll * s->V * NB_SLOTS; break;
        case 12: src = s->sdf; bytes = s->sdf_ready ? 4ll * s->dim[0] * s->dim[1] * s->dim[2] : 0; break;
        case 13: src = s->counts; bytes = 8ll * N_COUNTS; break;
        default: set_err("unknown buffer id"); return -1;
    }
    if (!src) { set_err("buffer is not allocated for this solver"); return -1; }
    if (bytes > max_bytes) { set_err("output buffer too small"); return -1; }
    memcpy(out, src, (size_t)bytes);
    return bytes;
}

int oracle_dynamic_info(OracleSolver* s, int* o) {
    if (!s || !o) return set_err("invalid dynamic info request");
    const ODyn* d = &s->own;
    o[0] = d->dt_n; o[1] = d->dt_hashed ? d->dt_large_n : 0; o[2] = d->dt_hashed ? d->dt_max_occ : 0; o[3] = d->dt_hashed;
    o[4] = d->dp_n; o[5] = d->dp_hashed;
    return 1;
}

int oracle_hash_info(OracleSolver* s, int* o) {
    if (!s || !o) return set_err("invalid hash info request");
    o[0] = s->nvb; o[1] = s->ntb; o[2] = s->neb; o[3] = s->vhash; o[4] = s->thash; o[5] = s->ehash;
    return 1;
}
