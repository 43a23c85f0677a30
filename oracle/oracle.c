/*
 * CPU oracle for DISO's differentiable iso-surface extraction.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C with OpenMP and in
 * double precision, the algorithm of the reference's marching cubes (DiffMC) and
 * dual marching cubes (DiffDMC): forward, backward and the quad-to-triangle split.
 * It is used as the checker by tests/, __graft_entry__.smoke() and as the timed
 * CPU baseline of bench.py; the product path never links or calls it.
 *
 * It follows the reference step by step (explicit padding, per-cell flags, full
 * exclusive scans, compaction, per-used-cell passes, scatter-form backward), so
 * that each intermediate has the meaning it has there.  Every function cites the
 * reference file:line it follows (paths inside the reference project).
 *
 * Case tables come from diso_gb300/csrc/case_tables.h (MC triangulation read
 * from the reference source, DMC tables derived by rule; both compared with the
 * reference's own tables by tests/test_tables.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../diso_gb300/csrc/case_tables.h"

#define MC_METHOD 0
#define DMC_METHOD 1

static const uint8_t kEdge[12] = DISO_EDGE_TABLE;
static const int kDmcQuad[24] = DISO_DMC_QUADS;

/* src/cumc.cu:107 (MC corner order) */
static const int kMcCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                    {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
/* src/cudualmc.cu:95-104 (DMC corner order, Morton) */
static const int kDmcCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

typedef struct {
  int64_t nv;       /* vertices */
  int64_t nf;       /* faces */
  int fw;           /* face width: 3 or 4 */
  int empty_guard;  /* 1 when the reference's min/max guard returned empty output */
  double *verts;    /* [nv,3] final (shifted and, if asked, normalised) */
  int64_t *faces;   /* [nf,fw] */
  int64_t n_used;   /* diagnostics: used cells of the padded grid */
} oracle_mesh;

typedef struct {
  int P[3];
  int64_t n_cells;
  const double *g; /* padded grid [P0*P1*P2] */
  const double *d; /* padded deform [P0*P1*P2*3] or NULL */
  double iso;
} grid_t;

/* src/cumc.h:101-105 */
static inline int64_t gA(const grid_t *G, int64_t x, int64_t y, int64_t z) {
  return z + (int64_t)G->P[2] * (y + (int64_t)G->P[1] * x);
}

static void gXYZ(const grid_t *G, int64_t c, int *x, int *y, int *z) {
  *x = (int)(c / ((int64_t)G->P[2] * G->P[1]));
  *y = (int)((c / G->P[2]) % G->P[1]);
  *z = (int)(c % G->P[2]);
}

/* Parallel exclusive scan of n int32 values in place; returns the total. */
static int64_t scan_excl(int32_t *a, int64_t n) {
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  int64_t *part = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
#pragma omp parallel num_threads(nt)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    int64_t lo = n * t / nt, hi = n * (t + 1) / nt, s = 0;
    for (int64_t i = lo; i < hi; ++i) s += a[i];
    part[t + 1] = s;
#pragma omp barrier
#pragma omp single
    for (int k = 0; k < nt; ++k) part[k + 1] += part[k];
    int64_t run = part[t];
    for (int64_t i = lo; i < hi; ++i) {
      int32_t v = a[i];
      a[i] = (int32_t)run;
      run += v;
    }
  }
  int64_t total = part[nt];
  free(part);
  return total;
}

/* diso/__init__.py:52-54: F.pad of grid with isovalue+1 and of deform with 0 */
static double *pad_grid(const double *sdf, const int n[3], double padval) {
  int P[3] = {n[0] + 2, n[1] + 2, n[2] + 2};
  int64_t tot = (int64_t)P[0] * P[1] * P[2];
  double *g = (double *)malloc((size_t)tot * sizeof(double));
#pragma omp parallel for
  for (int64_t x = 0; x < P[0]; ++x)
    for (int64_t y = 0; y < P[1]; ++y)
      for (int64_t z = 0; z < P[2]; ++z) {
        int inside = x >= 1 && x <= n[0] && y >= 1 && y <= n[1] && z >= 1 && z <= n[2];
        g[z + P[2] * (y + P[1] * x)] =
            inside ? sdf[(z - 1) + (int64_t)n[2] * ((y - 1) + (int64_t)n[1] * (x - 1))] : padval;
      }
  return g;
}

static double *pad_deform(const double *dfm, const int n[3]) {
  if (!dfm) return NULL;
  int P[3] = {n[0] + 2, n[1] + 2, n[2] + 2};
  int64_t tot = (int64_t)P[0] * P[1] * P[2];
  double *d = (double *)calloc((size_t)tot * 3, sizeof(double));
#pragma omp parallel for
  for (int64_t x = 1; x <= n[0]; ++x)
    for (int64_t y = 1; y <= n[1]; ++y)
      for (int64_t z = 1; z <= n[2]; ++z) {
        int64_t o = z + P[2] * (y + P[1] * x);
        int64_t i = (z - 1) + (int64_t)n[2] * ((y - 1) + (int64_t)n[1] * (x - 1));
        d[3 * o + 0] = dfm[3 * i + 0];
        d[3 * o + 1] = dfm[3 * i + 1];
        d[3 * o + 2] = dfm[3 * i + 2];
      }
  return d;
}

/* src/cumc.cu:455-472 / src/cudualmc.cu:796-813 */
static int cell_code(const grid_t *G, int x, int y, int z, const int corner[8][3]) {
  int code = 0;
  for (int i = 0; i < 8; ++i)
    if (G->g[gA(G, x + corner[i][0], y + corner[i][1], z + corner[i][2])] >= G->iso) code |= 1 << i;
  return code;
}

static inline int crosses(double a, double b, double iso) {
  /* src/cumc.cu:334-339 */
  return (a < iso && b >= iso) || (b < iso && a >= iso);
}

/* src/cumc.cu:343-368 (computeMcVert) */
static void mc_vert(const grid_t *G, int x, int y, int z, int dim, double out[3]) {
  int off[3] = {0, 0, 0};
  off[dim] = 1;
  int64_t v0 = gA(G, x, y, z), v1 = gA(G, x + off[0], y + off[1], z + off[2]);
  double d0 = G->g[v0], d1 = G->g[v1];
  double t = (d1 != d0) ? fmin(fmax((G->iso - d0) / (d1 - d0), 0.0), 1.0) : 0.5;
  double p0[3] = {x, y, z}, p1[3] = {x + off[0], y + off[1], z + off[2]};
  if (G->d) {
    for (int k = 0; k < 3; ++k) {
      p0[k] += G->d[3 * v0 + k];
      p1[k] += G->d[3 * v1 + k];
    }
  }
  for (int k = 0; k < 3; ++k) out[k] = p0[k] + (p1[k] - p0[k]) * t;
}

/* src/cumc.cu:412-453 (adjComputeMcVert): scatter into padded adjoints */
static void adj_mc_vert(const grid_t *G, int x, int y, int z, int dim, const double g[3],
                        double *adj_g, double *adj_d) {
  int off[3] = {0, 0, 0};
  off[dim] = 1;
  int64_t v0 = gA(G, x, y, z), v1 = gA(G, x + off[0], y + off[1], z + off[2]);
  double d0 = G->g[v0], d1 = G->g[v1];
  double t = (d1 != d0) ? fmin(fmax((G->iso - d0) / (d1 - d0), 0.0), 1.0) : 0.5;
  double p0[3] = {x, y, z}, p1[3] = {x + off[0], y + off[1], z + off[2]};
  if (G->d) {
    for (int k = 0; k < 3; ++k) {
      p0[k] += G->d[3 * v0 + k];
      p1[k] += G->d[3 * v1 + k];
    }
  }
  double adj_t = 0;
  for (int k = 0; k < 3; ++k) adj_t += (p1[k] - p0[k]) * g[k];
  if (adj_d) {
    for (int k = 0; k < 3; ++k) {
#pragma omp atomic
      adj_d[3 * v0 + k] += (1 - t) * g[k];
#pragma omp atomic
      adj_d[3 * v1 + k] += t * g[k];
    }
  }
  double den = (d1 - d0) * (d1 - d0);
#pragma omp atomic
  adj_g[v0] += (G->iso - d1) / den * adj_t;
#pragma omp atomic
  adj_g[v1] += (d0 - G->iso) / den * adj_t;
}

/* Used-cell bookkeeping shared by MC and DMC:
 * src/cumc.cu:265-311 (count/index used cells) and :313-341 (count crossings). */
typedef struct {
  int32_t *first_cell_used; /* [n_cells+1] exclusive scan of the used flags */
  int32_t *used_cell_index; /* [n_used] */
  int32_t *first_vert;      /* [n_used+1] exclusive scan of owned crossings */
  int64_t n_used, n_cross;
} used_t;

static void find_used(const grid_t *G, const int corner[8][3], used_t *U) {
  int64_t n = G->n_cells;
  U->first_cell_used = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
#pragma omp parallel for
  for (int64_t c = 0; c < n; ++c) {
    int x, y, z;
    gXYZ(G, c, &x, &y, &z);
    if (x >= G->P[0] - 1 || y >= G->P[1] - 1 || z >= G->P[2] - 1) continue;
    int code = cell_code(G, x, y, z, corner);
    U->first_cell_used[c] = (code != 0 && code != 255);
  }
  U->n_used = scan_excl(U->first_cell_used, n + 1);
  U->used_cell_index = (int32_t *)malloc((size_t)(U->n_used + 1) * sizeof(int32_t));
#pragma omp parallel for
  for (int64_t c = 0; c < n; ++c)
    if (U->first_cell_used[c + 1] != U->first_cell_used[c]) U->used_cell_index[U->first_cell_used[c]] = (int32_t)c;
  U->first_vert = (int32_t *)calloc((size_t)U->n_used + 1, sizeof(int32_t));
#pragma omp parallel for
  for (int64_t u = 0; u < U->n_used; ++u) {
    int x, y, z;
    gXYZ(G, U->used_cell_index[u], &x, &y, &z);
    double d0 = G->g[gA(G, x, y, z)];
    int num = crosses(d0, G->g[gA(G, x + 1, y, z)], G->iso) + crosses(d0, G->g[gA(G, x, y + 1, z)], G->iso) +
              crosses(d0, G->g[gA(G, x, y, z + 1)], G->iso);
    U->first_vert[u] = num;
  }
  U->n_cross = scan_excl(U->first_vert, U->n_used + 1);
}

static void free_used(used_t *U) {
  free(U->first_cell_used);
  free(U->used_cell_index);
  free(U->first_vert);
}

/* diso/__init__.py:56-60: verts - 1, then / (dim - 1) */
static void finish_verts(double *v, int64_t nv, const int n[3], int normalize) {
#pragma omp parallel for
  for (int64_t i = 0; i < nv; ++i)
    for (int k = 0; k < 3; ++k) {
      double a = v[3 * i + k] - 1.0;
      v[3 * i + k] = normalize ? a / (double)(n[k] - 1) : a;
    }
}

/* ------------------------------------------------------------------ MC */

/* src/cumc.cu:370-410 (create_cell_mc_verts_kernel), also returns verts_type */
static double *mc_make_verts(const grid_t *G, const used_t *U, int8_t **vtype_out) {
  double *verts = (double *)malloc((size_t)(U->n_cross + 1) * 3 * sizeof(double));
  int8_t *vtype = (int8_t *)malloc((size_t)U->n_cross + 1);
#pragma omp parallel for
  for (int64_t u = 0; u < U->n_used; ++u) {
    int x, y, z;
    gXYZ(G, U->used_cell_index[u], &x, &y, &z);
    double d0 = G->g[gA(G, x, y, z)];
    double ds[3] = {G->g[gA(G, x + 1, y, z)], G->g[gA(G, x, y + 1, z)], G->g[gA(G, x, y, z + 1)]};
    int64_t first = U->first_vert[u];
    for (int dim = 0; dim < 3; ++dim)
      if (crosses(d0, ds[dim], G->iso)) {
        mc_vert(G, x, y, z, dim, verts + 3 * first);
        vtype[first++] = (int8_t)dim;
      }
  }
  *vtype_out = vtype;
  return verts;
}

/* src/cumc.cu:540-649 (count_cell_mc_tris_kernel, create_cell_mc_tris_kernel) */
static int64_t *mc_make_tris(const grid_t *G, const used_t *U, const int8_t *vtype, int64_t *n_tris) {
  int32_t *first_tri = (int32_t *)calloc((size_t)U->n_used + 1, sizeof(int32_t));
  uint8_t *codes = (uint8_t *)malloc((size_t)U->n_used + 1);
#pragma omp parallel for
  for (int64_t u = 0; u < U->n_used; ++u) {
    int x, y, z;
    gXYZ(G, U->used_cell_index[u], &x, &y, &z);
    int code = cell_code(G, x, y, z, kMcCorner); /* getGoodCellCode: ambiguity fix disabled, :514-538 */
    codes[u] = (uint8_t)code;
    first_tri[u] = 3 * (int32_t)(kMcTriangles[code] & 15);
  }
  int64_t n_idx = scan_excl(first_tri, U->n_used + 1);
  int64_t *tris = (int64_t *)malloc((size_t)(n_idx + 1) * sizeof(int64_t));
#pragma omp parallel for
  for (int64_t u = 0; u < U->n_used; ++u) {
    int x, y, z;
    gXYZ(G, U->used_cell_index[u], &x, &y, &z);
    uint64_t w = kMcTriangles[codes[u]];
    int num = 3 * (int)(w & 15);
    int64_t out = first_tri[u];
    for (int i = 0; i < num; ++i) {
      int eid = (int)((w >> (4 + 4 * i)) & 15);
      int ex = x + (kEdge[eid] & 1), ey = y + ((kEdge[eid] >> 1) & 1), ez = z + ((kEdge[eid] >> 2) & 1);
      int axis = kEdge[eid] >> 3;
      int64_t eu = U->first_cell_used[gA(G, ex, ey, ez)];
      int64_t id = U->first_vert[eu];
      int vnum = U->first_vert[eu + 1] - U->first_vert[eu];
      for (int k = 0; k < vnum; ++k)
        if (vtype[id + k] == axis) {
          id += k;
          break;
        }
      tris[out + i] = id;
    }
  }
  free(first_tri);
  free(codes);
  *n_tris = n_idx / 3;
  return tris;
}

/* ------------------------------------------------------------------ DMC */

/* src/cudualmc.cu:815-839 (getGoodCellCode with face-neighbour ambiguity test) */
static int dmc_good_code(const grid_t *G, int x, int y, int z) {
  int code = cell_code(G, x, y, z, kDmcCorner);
  int dir = (int)((kDmcCase[code] >> 28) & 7);
  if (dir != 7) {
    int nb[3] = {x, y, z};
    int comp = dir >> 1;
    nb[comp] += (dir & 1) ? 1 : -1;
    if (nb[comp] >= 0 && nb[comp] < G->P[comp] - 1) {
      int ncode = cell_code(G, nb[0], nb[1], nb[2], kDmcCorner);
      if (((kDmcCase[ncode] >> 28) & 7) != 7) code ^= 0xff;
    }
  }
  return code;
}

typedef struct {
  used_t U;
  uint8_t *code;        /* [n_used] resolved codes */
  int32_t *first_patch; /* [n_used+1] */
  int64_t n_patch;
} dmc_state_t;

/* src/cudualmc.cu:1058-1122 up to the patch scan */
static void dmc_prepare(const grid_t *G, dmc_state_t *S) {
  find_used(G, kDmcCorner, &S->U);
  S->code = (uint8_t *)malloc((size_t)S->U.n_used + 1);
  S->first_patch = (int32_t *)calloc((size_t)S->U.n_used + 1, sizeof(int32_t));
#pragma omp parallel for
  for (int64_t u = 0; u < S->U.n_used; ++u) {
    int x, y, z;
    gXYZ(G, S->U.used_cell_index[u], &x, &y, &z);
    int code = dmc_good_code(G, x, y, z); /* src/cudualmc.cu:841-863 */
    S->code[u] = (uint8_t)code;
    S->first_patch[u] = (int32_t)((kDmcCase[code] >> 24) & 7);
  }
  S->n_patch = scan_excl(S->first_patch, S->U.n_used + 1);
}

static void dmc_free(dmc_state_t *S) {
  free_used(&S->U);
  free(S->code);
  free(S->first_patch);
}

/* src/cudualmc.cu:907-955 (create_dmc_verts_kernel) */
static double *dmc_make_verts(const grid_t *G, const dmc_state_t *S) {
  double *verts = (double *)malloc((size_t)(S->n_patch + 1) * 3 * sizeof(double));
#pragma omp parallel for
  for (int64_t u = 0; u < S->U.n_used; ++u) {
    int x, y, z;
    gXYZ(G, S->U.used_cell_index[u], &x, &y, &z);
    uint64_t w = kDmcCase[S->code[u]];
    int np = (int)((w >> 24) & 7);
    int code = S->code[u];
    for (int p = 0; p < np; ++p) {
      double acc[3] = {0, 0, 0}, num = 0;
      for (int e = 0; e < 12; ++e) { /* patch edges in ascending edge order */
        /* edge e crosses for this (possibly flipped) code iff its end corners differ */
        int s = kEdge[e] & 7, ax = kEdge[e] >> 3;
        int cs = s, ce = s | (1 << ax); /* Morton corner ids of the two ends */
        if (((code >> cs) & 1) == ((code >> ce) & 1)) continue;
        if ((int)((w >> (2 * e)) & 3) != p) continue;
        double v[3];
        mc_vert(G, x + (s & 1), y + ((s >> 1) & 1), z + ((s >> 2) & 1), ax, v);
        for (int k = 0; k < 3; ++k) acc[k] += v[k];
        num += 1.0;
      }
      double inv = 1.0 / num;
      int64_t o = S->first_patch[u] + p;
      for (int k = 0; k < 3; ++k) verts[3 * o + k] = acc[k] * inv;
    }
  }
  return verts;
}

/* src/cudualmc.cu:753-794 and :1019-1056 (index_cell_mc_verts + create_quads) */
static int64_t *dmc_make_quads(const grid_t *G, const dmc_state_t *S) {
  int64_t *quads = (int64_t *)malloc((size_t)(S->U.n_cross + 1) * 4 * sizeof(int64_t));
#pragma omp parallel for
  for (int64_t u = 0; u < S->U.n_used; ++u) {
    int x, y, z;
    gXYZ(G, S->U.used_cell_index[u], &x, &y, &z);
    double d0 = G->g[gA(G, x, y, z)];
    double ds[3] = {G->g[gA(G, x + 1, y, z)], G->g[gA(G, x, y + 1, z)], G->g[gA(G, x, y, z + 1)]};
    int64_t id = S->U.first_vert[u];
    for (int dim = 0; dim < 3; ++dim) {
      int entering = d0 < G->iso && ds[dim] >= G->iso;
      int exiting = ds[dim] < G->iso && d0 >= G->iso;
      if (!(entering || exiting)) continue;
      int type = (exiting ? 3 : 0) + dim;
      for (int i = 0; i < 4; ++i) {
        int q = kDmcQuad[4 * type + i];
        int dx = (q & 3) - 1, dy = ((q >> 2) & 3) - 1, dz = ((q >> 4) & 3) - 1, eid = q >> 8;
        int64_t nu = S->U.first_cell_used[gA(G, x + dx, y + dy, z + dz)];
        int off = (int)((kDmcCase[S->code[nu]] >> (2 * eid)) & 3);
        quads[4 * id + i] = S->first_patch[nu] + off;
      }
      ++id;
    }
  }
  return quads;
}

/* diso/__init__.py:118-147: split each quad into the triangle pair whose largest
 * corner cosine is smaller (config 1 iff max_cos1 < max_cos2); config-1 faces
 * first, then config-2 faces, each group in quad order. */
static void normalize3(const double v[3], double o[3]) {
  double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (n < 1e-12) n = 1e-12;
  for (int k = 0; k < 3; ++k) o[k] = v[k] / n;
}

static double tri_max_cos(const double *V, int64_t a, int64_t b, int64_t c) {
  const double *p[3] = {V + 3 * a, V + 3 * b, V + 3 * c};
  double m = -INFINITY;
  for (int k = 0; k < 3; ++k) {
    const double *o = p[k], *u = p[(k + 1) % 3], *w = p[(k + 2) % 3];
    double e1[3], e2[3], n1[3], n2[3];
    for (int j = 0; j < 3; ++j) {
      e1[j] = u[j] - o[j];
      e2[j] = w[j] - o[j];
    }
    normalize3(e1, n1);
    normalize3(e2, n2);
    double cs = n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2];
    if (cs > m || k == 0) m = cs;
  }
  return m;
}

int oracle_split_config(const double *verts, const int64_t *q) {
  double a1 = tri_max_cos(verts, q[0], q[1], q[3]);
  double b1 = tri_max_cos(verts, q[1], q[2], q[3]);
  double a2 = tri_max_cos(verts, q[0], q[1], q[2]);
  double b2 = tri_max_cos(verts, q[0], q[2], q[3]);
  double m1 = a1 > b1 ? a1 : b1, m2 = a2 > b2 ? a2 : b2;
  if (m1 < m2) return 1;
  if (m1 >= m2) return 2;
  return 0; /* NaN: the reference's two boolean masks both drop the quad */
}

static int64_t *split_quads(const double *verts, const int64_t *quads, int64_t nq, int64_t *nf) {
  int8_t *cfg = (int8_t *)malloc((size_t)nq + 1);
  int64_t n1 = 0, n2 = 0;
#pragma omp parallel for reduction(+ : n1, n2)
  for (int64_t i = 0; i < nq; ++i) {
    cfg[i] = (int8_t)oracle_split_config(verts, quads + 4 * i);
    n1 += cfg[i] == 1;
    n2 += cfg[i] == 2;
  }
  int64_t *f = (int64_t *)malloc((size_t)(2 * (n1 + n2) + 1) * 3 * sizeof(int64_t));
  int64_t a = 0, b = 2 * n1;
  for (int64_t i = 0; i < nq; ++i) {
    const int64_t *q = quads + 4 * i;
    if (cfg[i] == 1) {
      int64_t t[6] = {q[0], q[1], q[3], q[1], q[2], q[3]};
      memcpy(f + 3 * a, t, sizeof t);
      a += 2;
    } else if (cfg[i] == 2) {
      int64_t t[6] = {q[0], q[1], q[2], q[0], q[2], q[3]};
      memcpy(f + 3 * b, t, sizeof t);
      b += 2;
    }
  }
  free(cfg);
  *nf = 2 * (n1 + n2);
  return f;
}

/* ------------------------------------------------------------------ API */

/* diso/__init__.py:48-50 / 102-104: the empty-surface guard */
static int guard_empty(const double *sdf, int64_t n, double iso) {
  double mn = INFINITY, mx = -INFINITY;
#pragma omp parallel for reduction(min : mn) reduction(max : mx)
  for (int64_t i = 0; i < n; ++i) {
    if (sdf[i] < mn) mn = sdf[i];
    if (sdf[i] > mx) mx = sdf[i];
  }
  return mn >= iso || mx <= iso;
}

/* Forward of DiffMC (method 0, diso/__init__.py:48-61 + src/cumc.cu:651-732) or DiffDMC
 * (method 1, diso/__init__.py:102-147 + src/cudualmc.cu:1058-1128).  iso and padval are
 * the values the reference sees in its own dtype (padval = isovalue + 1 rounded to it). */
int oracle_extract(int method, const double *sdf, const double *deform, int nx, int ny, int nz, double iso,
                   double padval, int normalize, int return_quads, oracle_mesh *out) {
  memset(out, 0, sizeof *out);
  int n[3] = {nx, ny, nz};
  out->fw = (method == DMC_METHOD) ? 4 : 3;
  if (nx < 1 || ny < 1 || nz < 1) return -1;
  if (guard_empty(sdf, (int64_t)nx * ny * nz, iso)) {
    out->empty_guard = 1;
    return 0;
  }
  grid_t G;
  G.P[0] = nx + 2;
  G.P[1] = ny + 2;
  G.P[2] = nz + 2;
  G.n_cells = (int64_t)G.P[0] * G.P[1] * G.P[2];
  double *g = pad_grid(sdf, n, padval);
  double *d = pad_deform(deform, n);
  G.g = g;
  G.d = d;
  G.iso = iso;
  if (method == MC_METHOD) {
    used_t U;
    find_used(&G, kMcCorner, &U);
    int8_t *vtype;
    out->verts = mc_make_verts(&G, &U, &vtype);
    out->nv = U.n_cross;
    out->faces = mc_make_tris(&G, &U, vtype, &out->nf);
    out->n_used = U.n_used;
    free(vtype);
    free_used(&U);
    finish_verts(out->verts, out->nv, n, normalize);
  } else {
    dmc_state_t S;
    dmc_prepare(&G, &S);
    out->verts = dmc_make_verts(&G, &S);
    out->nv = S.n_patch;
    int64_t *quads = dmc_make_quads(&G, &S);
    out->n_used = S.U.n_used;
    finish_verts(out->verts, out->nv, n, normalize);
    if (return_quads) {
      out->faces = quads;
      out->nf = S.U.n_cross;
    } else {
      out->faces = split_quads(out->verts, quads, S.U.n_cross, &out->nf);
      out->fw = 3;
      free(quads);
    }
    dmc_free(&S);
  }
  free(g);
  free(d);
  return 0;
}

void oracle_mesh_free(oracle_mesh *m) {
  free(m->verts);
  free(m->faces);
  m->verts = NULL;
  m->faces = NULL;
}

/* Backward: grad_verts is dL/d(final verts) [nv,3].  Mirrors DMCFunction/DDMCFunction.backward
 * (diso/__init__.py:30-44, 84-98): recompute the forward, then scatter through the lerp
 * adjoint (src/cumc.cu:474-512, src/cudualmc.cu:957-1005) into padded adjoints, and take
 * the interior (the F.pad backward).  The chain rule of "- 1" and "/ (dim - 1)" is applied
 * first, as autograd does.  grad_sdf [nx*ny*nz], grad_deform [nx*ny*nz*3] (if deform).
 * exact_dmc selects the true derivative for DMC cells with several patches instead of
 * the reference's (see the comment in the DMC loop). */
int oracle_backward(int method, const double *sdf, const double *deform, int nx, int ny, int nz, double iso,
                    double padval, int normalize, const double *grad_verts, int64_t nv, double *grad_sdf,
                    double *grad_deform, int exact_dmc) {
  int n[3] = {nx, ny, nz};
  int64_t nn = (int64_t)nx * ny * nz;
  memset(grad_sdf, 0, (size_t)nn * sizeof(double));
  if (grad_deform) memset(grad_deform, 0, (size_t)nn * 3 * sizeof(double));
  if (guard_empty(sdf, nn, iso)) return 0;
  grid_t G;
  G.P[0] = nx + 2;
  G.P[1] = ny + 2;
  G.P[2] = nz + 2;
  G.n_cells = (int64_t)G.P[0] * G.P[1] * G.P[2];
  double *g = pad_grid(sdf, n, padval);
  double *d = pad_deform(deform, n);
  G.g = g;
  G.d = d;
  G.iso = iso;
  double *adj_g = (double *)calloc((size_t)G.n_cells, sizeof(double));
  double *adj_d = d ? (double *)calloc((size_t)G.n_cells * 3, sizeof(double)) : NULL;
  double *gv = (double *)malloc((size_t)(nv + 1) * 3 * sizeof(double));
  for (int64_t i = 0; i < nv; ++i)
    for (int k = 0; k < 3; ++k) gv[3 * i + k] = normalize ? grad_verts[3 * i + k] / (double)(n[k] - 1) : grad_verts[3 * i + k];
  int rc = 0;
  if (method == MC_METHOD) {
    used_t U;
    find_used(&G, kMcCorner, &U);
    if (U.n_cross != nv) rc = -2;
    else {
#pragma omp parallel for
      for (int64_t u = 0; u < U.n_used; ++u) {
        int x, y, z;
        gXYZ(&G, U.used_cell_index[u], &x, &y, &z);
        double d0 = G.g[gA(&G, x, y, z)];
        double ds[3] = {G.g[gA(&G, x + 1, y, z)], G.g[gA(&G, x, y + 1, z)], G.g[gA(&G, x, y, z + 1)]};
        int64_t first = U.first_vert[u];
        for (int dim = 0; dim < 3; ++dim)
          if (crosses(d0, ds[dim], iso)) adj_mc_vert(&G, x, y, z, dim, gv + 3 * first++, adj_g, adj_d);
      }
    }
    free_used(&U);
  } else {
    dmc_state_t S;
    dmc_prepare(&G, &S);
    if (S.n_patch != nv) rc = -2;
    else {
#pragma omp parallel for
      for (int64_t u = 0; u < S.U.n_used; ++u) {
        int x, y, z;
        gXYZ(&G, S.U.used_cell_index[u], &x, &y, &z);
        int code = S.code[u];
        uint64_t w = kDmcCase[code];
        int np = (int)((w >> 24) & 7);
        for (int p = 0; p < np; ++p) {
          double num = (double)((w >> (32 + 4 * p)) & 15);
          double inv = 1.0 / num, a[3];
          /* src/cudualmc.cu:990 reads adj_verts[first] for every patch of the cell
           * (first is never advanced), so all patches of a multi-patch cell receive
           * the first patch's gradient; exact_dmc = 1 uses each patch's own. */
          int64_t o = S.first_patch[u] + (exact_dmc ? p : 0);
          for (int k = 0; k < 3; ++k) a[k] = gv[3 * o + k] * inv;
          for (int e = 0; e < 12; ++e) {
            int s = kEdge[e] & 7, ax = kEdge[e] >> 3;
            if (((code >> s) & 1) == ((code >> (s | (1 << ax))) & 1)) continue;
            if ((int)((w >> (2 * e)) & 3) != p) continue;
            adj_mc_vert(&G, x + (s & 1), y + ((s >> 1) & 1), z + ((s >> 2) & 1), ax, a, adj_g, adj_d);
          }
        }
      }
    }
    dmc_free(&S);
  }
#pragma omp parallel for
  for (int64_t x = 1; x <= nx; ++x)
    for (int64_t y = 1; y <= ny; ++y)
      for (int64_t z = 1; z <= nz; ++z) {
        int64_t o = gA(&G, x, y, z), i = (z - 1) + (int64_t)nz * ((y - 1) + (int64_t)ny * (x - 1));
        grad_sdf[i] = adj_g[o];
        if (grad_deform)
          for (int k = 0; k < 3; ++k) grad_deform[3 * i + k] = adj_d[3 * o + k];
      }
  free(gv);
  free(adj_g);
  free(adj_d);
  free(g);
  free(d);
  return rc;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
