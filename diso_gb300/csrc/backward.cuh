// Backward of a forward that kept only its segment record: one pass over the point
// tiles near the surface that writes every gradient element there once.
//
// The reference's backward runs its forward again to rebuild the crossing lists
// (diso/__init__.py:32-37, 86-91) and then scatters each vertex's gradient with
// atomics (adj_create_cell_mc_verts_kernel, src/cumc.cu:474-512;
// adj_create_dmc_verts_kernel, src/cudualmc.cu:957-1005).  Here nothing of the
// crossing lists is kept either, but they are recomputed per point tile in shared
// memory instead of as a second forward:
//
//   * the tile's point rows and a halo become row masks (one ballot per row);
//   * the crossing edges that touch the tile's points (those owned by the window
//     cells [X0, X0+TX] x [Y0, Y0+TY] x [Z0, Z0+TZ]) get window slots;
//   * MC: an edge's vertex id is the scanned crossing count of its segment (the
//     forward's record) plus its rank inside the segment;
//     DMC: the cells around the window edges ([X0-1, X0+TX] x [Y0-1, Y0+TY] x
//     [Z0-1, Z0+TZ]) get their codes after the ambiguity test and their first
//     patch id (the segment's scanned patch count plus an in-segment prefix), from
//     which each edge's four patches and their edge counts follow;
//   * each window edge's adjoint at both end points is computed once into shared
//     memory (the same arithmetic, in the same order, as the stored backward's edge
//     pass), and each point adds the adjoints of its at most six edges in a fixed
//     order: deterministic and bit-identical to the stored backward;
//   * point tiles with no crossing nearby (the forward's tile bits) only get zeros:
//     bulk copies that warp 0 issues inside the active tiles (zero_column), or
//     zero_tiles_kernel beside this one.
//
// Tiles whose window holds more crossing edges than the shared-memory cache compute
// each edge's adjoint at both of its end points instead.
#pragma once
#include "fields.cuh"
#include "kernels.cuh"

namespace diso {

// Window edges whose adjoints a tile keeps in shared memory: sized so that three
// CTAs share an SM (the tile's state is about 72 KB of dynamic shared memory in
// either precision); at 512^3 on a noisy union of spheres about 99% of the windows
// fit (the largest hold some 1900 edges, the median about 400).
template <class S>
__host__ __device__ constexpr int fb_cap() {
  return sizeof(S) == 4 ? 1664 : 832;
}

constexpr int FB_ZBLOCK = 2048;  // bytes of the zeroed block the bulk zero copies read

// REC: the DMC window cells' codes come from the forward count's cell records
template <class S, int METHOD, bool REC = false>
struct FusedShared {
  // mask rows start at (X0 - LO, Y0 - LO): the edge rows' points; for DMC codes
  // computed here two rows further, so that the ambiguity test of every window cell
  // finds its neighbour's code in the masks (on the noisy surfaces of dense fields
  // most window rows hold ambiguous cells, and a neighbour from global memory stalls
  // the row's warp)
  static constexpr bool WIDE = METHOD == DMC && !REC;
  static constexpr int LO = WIDE ? 2 : 0;
  static constexpr int WX = TX + 2 + (WIDE ? 3 : 0), WY = TY + 2 + (WIDE ? 3 : 0);
  static constexpr int CX = TX + 1, CY = TY + 1;  // edge rows: cells [X0, X0+TX] x [Y0, Y0+TY]
  static constexpr int KX = METHOD == DMC ? TX + 2 : 1, KY = METHOD == DMC ? TY + 2 : 1;  // DMC window cell rows
  uint64_t m[WX][WY];
  RowBits wb[CX][CY];
  uint32_t eb[CX][CY][2];          // scanned crossing counts of chunks zc, zc + 1 (MC vertex ids)
  uint32_t pb[KX][KY][2];          // scanned patch counts of chunks zc, zc + 1 (DMC)
  uint8_t busy[KX][KY];            // DMC: bit 0/1/2: chunk zc-1 / zc / zc+1 of the row has a non-zero count
  uint16_t wcell[CX][CY][TZ + 1];  // per edge-row cell: its first window slot | crossing flags << 13
  uint16_t witems[fb_cap<S>()];
  uint8_t w32[CX][CY];
  uint8_t rc[KX][KY][TZ + 2];     // DMC window cells (z index j + 1 for Z0 + j): code after the ambiguity test
  int32_t first[KX][KY][TZ + 2];  //   and the id of its first patch
  uint32_t wsum[NTHREADS / 32 + 1];
  uint32_t nwi;
  // DMC case words (dmc_case in common.cuh) and the cell-local edge lookup: beside
  // three CTAs' shared memory the L1 cache is small, and these lookups sit on the
  // dependent chains of the code and adjoint phases
  uint64_t cases[METHOD == DMC ? 256 : 1];
  uint8_t edge_of[24];
  __align__(16) uint4 zblock[FB_ZBLOCK / 16];  // zeros, the source of the bulk zero copies
  __align__(16) S adj[fb_cap<S>()][8];
};

// The gradient reaching the lerp vertex of window edge (x, y, j, a) (owner cell
// (X0 + x, Y0 + y, Z0 + j), x in [0, TX], y in [0, TY], j in [0, TZ]), in padded
// coordinates (the chain rule of the shift and the normalisation in `scale`), as
// the stored backward's edge pass forms it (edge_adjoint_at in kernels.cuh).
template <class S, int METHOD, class SH>
__device__ __forceinline__ void fused_edge_grad(const SH& sh, int x, int y, int j, int a,
                                                const S* __restrict__ gv, int64_t V, const S scale[3], int exact,
                                                S gvec[3], bool& bad) {
  if constexpr (METHOD == MC) {
    // the edge's vertex: the scanned crossings of its segment, then the crossings
    // of the cells before it in the segment, then its axes before a
    const int fl = sh.wcell[x][y][j] >> 13;
    int64_t v;
    if (j == TZ) {
      v = (int64_t)sh.eb[x][y][1] + __popc(fl & ((1 << a) - 1));
    } else {
      v = (int64_t)sh.eb[x][y][0] + row_prefix(sh.wb[x][y], j) + __popc(fl & ((1 << a) - 1));
    }
    if (v >= V) {
      bad = true;
      v = 0;
    }
    load_grad<S>(gv, v, scale, gvec);
  } else {
    // the four cells around the edge, one step back by db along axis b = a + 1 and
    // dc along c = a + 2, in the order db + 2 dc; in each the edge starts at the
    // cell's corner (db along b, dc along c)
    const int b = a == 2 ? 0 : a + 1, c = a == 0 ? 2 : a - 1;
    gvec[0] = gvec[1] = gvec[2] = S(0);
#pragma unroll
    for (int at = 0; at < 4; ++at) {
      const int db = at & 1, dc = at >> 1;
      const int wx = x + 1 - (b == 0 ? db : 0) - (c == 0 ? dc : 0);
      const int wy = y + 1 - (b == 1 ? db : 0) - (c == 1 ? dc : 0);
      const int wj = j + 1 - (b == 2 ? db : 0) - (c == 2 ? dc : 0);
      const int s = (db << b) | (dc << c);
      const int e = sh.edge_of[3 * s + a];
      const uint64_t w = sh.cases[sh.rc[wx][wy][wj]];
      const int q = dmc_patch_of(w, e);
      const int cnt = (int)((w >> (32 + 4 * q)) & 15);  // the edges of patch q
      int64_t p = (int64_t)sh.first[wx][wy][wj] + (exact ? q : 0);
      if (p < 0 || p >= V || cnt == 0) {
        bad = true;
        p = 0;
      }
      S v[3];
      load_grad<S>(gv, p, scale, v);
      const S inv = recip<S>(cnt);
      gvec[0] = fma_rn(v[0], inv, gvec[0]);
      gvec[1] = fma_rn(v[1], inv, gvec[1]);
      gvec[2] = fma_rn(v[2], inv, gvec[2]);
    }
  }
}

// adjoints (c0 at the edge's first point, c1 at its second) of window edge (x, y, j, a)
template <class S, int METHOD, class F, class SH>
__device__ __forceinline__ void fused_edge_adjoint(const SH& sh, const F& f, int X0, int Y0,
                                                   int Z0, int x, int y, int j, int a, const S* __restrict__ gv,
                                                   int64_t V, const S scale[3], int exact, S c0[4], S c1[4],
                                                   bool& bad) {
  S gvec[3];
  if constexpr (F::kDense) {
    // the end points' loads first, so that they overlap the patches' gradient loads
    const int X = X0 + x, Y = Y0 + y, Z = Z0 + j, ex = a == 0, ey = a == 1, ez = a == 2;
    const bool in0 = f.inside(X, Y, Z), in1 = f.inside(X + ex, Y + ey, Z + ez);
    const int64_t i0 = ((int64_t)min(max(X - 1, 0), f.n0 - 1) * f.n1 + min(max(Y - 1, 0), f.n1 - 1)) * f.n2 +
                       min(max(Z - 1, 0), f.n2 - 1);
    const int64_t i1 = ((int64_t)min(max(X - 1 + ex, 0), f.n0 - 1) * f.n1 + min(max(Y - 1 + ey, 0), f.n1 - 1)) * f.n2 +
                       min(max(Z - 1 + ez, 0), f.n2 - 1);
    const S v0 = __ldg(f.sdf + i0), v1 = __ldg(f.sdf + i1);
    S q0[3] = {S(0), S(0), S(0)}, q1[3] = {S(0), S(0), S(0)};
    if (f.def) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const S u0 = __ldg(f.def + 3 * i0 + k), u1 = __ldg(f.def + 3 * i1 + k);
        q0[k] = in0 ? u0 : S(0);
        q1[k] = in1 ? u1 : S(0);
      }
    }
    fused_edge_grad<S, METHOD, SH>(sh, x, y, j, a, gv, V, scale, exact, gvec, bad);
    edge_adjoint_math<S>(f.iso, X, Y, Z, a, in0 ? v0 : f.pad, in1 ? v1 : f.pad, q0, q1, gvec, c0, c1);
  } else {
    fused_edge_grad<S, METHOD, SH>(sh, x, y, j, a, gv, V, scale, exact, gvec, bad);
    // an evaluated field: its values where the edge's ends lie, the same arithmetic
    const int X = X0 + x, Y = Y0 + y, Z = Z0 + j, ex = a == 0, ey = a == 1, ez = a == 2;
    S q0[3], q1[3];
    f.deform(X, Y, Z, q0);
    f.deform(X + ex, Y + ey, Z + ez, q1);
    edge_adjoint_math<S>(f.iso, X, Y, Z, a, f.at(X, Y, Z), f.at(X + ex, Y + ey, Z + ez), q0, q1, gvec, c0, c1);
  }
}

template <class S>
struct Adj4 {
  S v[4];
  bool bad;
};

// the uncached path's per-point call, kept out of line (it runs only for tiles with
// more window edges than the cache holds): the adjoint at end k of window edge
// (x, y, j, a)
template <class S, int METHOD, class F, class SH>
__device__ __noinline__ Adj4<S> fused_edge_adjoint_far(const SH& sh, const F& f, int X0,
                                                       int Y0, int Z0, int x, int y, int j, int a,
                                                       const S* __restrict__ gv, int64_t V, S sx, S sy, S sz,
                                                       int exact, int k) {
  S c0[4], c1[4];
  const S scale[3] = {sx, sy, sz};
  Adj4<S> r;
  r.bad = false;
  fused_edge_adjoint<S, METHOD, F, SH>(sh, f, X0, Y0, Z0, x, y, j, a, gv, V, scale, exact, c0, c1, r.bad);
#pragma unroll
  for (int i = 0; i < 4; ++i) r.v[i] = k ? c1[i] : c0[i];
  return r;
}

// Morton code of cell (X, Y, Z) from global memory, out of line: the DMC ambiguity
// test needs it only for an ambiguous cell whose neighbour lies outside the masks
template <class S, class F>
__device__ __noinline__ int fused_code_far(const F& f, int X, int Y, int Z) {
  if constexpr (!F::kDense) {
    return cell_code_far<S, F>(f, X, Y, Z);
  } else {
  // the eight corners' loads issued together: clamped addresses, the pad value
  // selected afterwards for corners outside the grid
  S v[8];
  bool in[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int x = X - 1 + (i & 1), y = Y - 1 + ((i >> 1) & 1), z = Z - 1 + ((i >> 2) & 1);
    in[i] = (unsigned)x < (unsigned)f.n0 && (unsigned)y < (unsigned)f.n1 && (unsigned)z < (unsigned)f.n2;
    const int cx = min(max(x, 0), f.n0 - 1), cy = min(max(y, 0), f.n1 - 1), cz = min(max(z, 0), f.n2 - 1);
    v[i] = __ldg(f.sdf + ((int64_t)cx * f.n1 + cy) * f.n2 + cz);
  }
  int c = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) c |= ((in[i] ? v[i] : f.pad) >= f.iso) << i;
  return c;
  }
}

// dmc_resolve_m (kernels.cuh) with the neighbour's code from the masks when its
// corners lie in them, otherwise from fused_code_far
template <class S, class F, int WX, int WY>
__device__ __forceinline__ int fused_resolve(const uint64_t (&m)[WX][WY], const uint64_t* cases, const F& f,
                                             int WX0, int WY0, int Z0, int code, int X, int Y, int Z,
                                             const Geom& g) {
  const int dir = dmc_dir(cases[code]);
  if (dir == 7) return code;
  const int comp = dir >> 1, d = (dir & 1) ? 1 : -1;
  const int NX = X + (comp == 0 ? d : 0), NY = Y + (comp == 1 ? d : 0), NZ = Z + (comp == 2 ? d : 0);
  const int nc = comp == 0 ? NX : (comp == 1 ? NY : NZ);
  if (nc < 0 || nc >= g.c[comp]) return code;
  const unsigned x = (unsigned)(NX - WX0), y = (unsigned)(NY - WY0);
  const int sft = NZ - Z0 + 1;
  int ncode;
  if (x < (unsigned)(WX - 1) && y < (unsigned)(WY - 1) && sft >= 0 && sft + 1 <= MASK_TOP)
    ncode = code8(m[x][y], m[x + 1][y], m[x][y + 1], m[x + 1][y + 1], sft);
  else
    ncode = fused_code_far<S, F>(f, NX, NY, NZ);
  return dmc_dir(cases[ncode]) != 7 ? (code ^ 0xff) : code;
}

// The gradient at unpadded point (x, y, z) of an evaluated union of spheres (the
// first `has` lanes' points) goes to the parameters of the sphere that attains the
// field's value there: d(|p - c| - r)/dc = -(p - c) / |p - c|, d/dr = -1.  Per warp and
// sphere in a fixed order (a shuffle tree over the lanes, then part[warp][k][.] in
// the warp's tile order), so the sums repeat bit for bit.  part: [NTHREADS / 32][K][4].
template <class S>
__device__ __forceinline__ void field_param_add(const SphereField<S>& f, double* __restrict__ part, bool has, int x,
                                                int y, int z, S grad) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int k = -1;
  double c[4] = {0.0, 0.0, 0.0, 0.0};
  if (has) {
    S off[3];
    k = f.argmin(x, y, z, off);
    const double dist = sqrt((double)off[0] * off[0] + (double)off[1] * off[1] + (double)off[2] * off[2]);
    const double gg = (double)grad;
    if (dist > 0.0) {
      c[0] = -gg * (double)off[0] / dist;
      c[1] = -gg * (double)off[1] / dist;
      c[2] = -gg * (double)off[2] / dist;
    }
    c[3] = -gg;
  }
  unsigned pending = __ballot_sync(0xffffffffu, has);
  while (pending) {
    const int kk = __shfl_sync(0xffffffffu, k, __ffs(pending) - 1);
    const bool mine = has && k == kk;
    double v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      v[i] = mine ? c[i] : 0.0;
#pragma unroll
      for (int o = 16; o; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    }
    if (lane == 0) {
      double* p = part + ((int64_t)warp * f.K + kk) * 4;
      p[0] += v[0];
      p[1] += v[1];
      p[2] += v[2];
      p[3] += v[3];
    }
    pending &= ~__ballot_sync(0xffffffffu, mine);
  }
}

// Zeros of column `col` of point tiles (the 4 x 8 rows of points (x0.., y0..) along the
// whole z extent) where its tiles have no crossing nearby, by the calling warp: lane
// l takes row (x0 + l / 8, y0 + l % 8); each run of such z tiles becomes bulk copies
// of at most FB_ZBLOCK bytes from the zeroed block to the row's dL/dsdf and dL/ddeform
// (rows of a multiple of 16 bytes at 16-byte aligned addresses, checked by the host).
// The copies run on the TMA unit beside the fused pass; the lane commits them.
template <class S>
__device__ __forceinline__ void zero_column(const Geom& g, const uint8_t* __restrict__ tile_flag, int64_t col,
                                            S* __restrict__ gsdf, S* __restrict__ gdef, const void* zblock) {
  const int lane = threadIdx.x & 31;
  const int x0 = (int)(col / g.ptiles_y()) * TX, y0 = (int)(col % g.ptiles_y()) * TY;
  const int x = x0 + lane / TY, y = y0 + lane % TY;
  const bool row = x < g.n[0] && y < g.n[1];
  const int pz = g.ptiles_z();
  char* srow = reinterpret_cast<char*>(gsdf + ((int64_t)x * g.n[1] + y) * g.n[2]);
  char* drow = gdef ? reinterpret_cast<char*>(gdef + 3 * (((int64_t)x * g.n[1] + y) * g.n[2])) : nullptr;
  bool any = false;
  for (int base = 0; base < pz; base += 32) {
    const int tz = base + lane;
    bool act = true;
    if (tz < pz) {
      act = false;
#pragma unroll
      for (int k = 0; k < 8; ++k) act = act || ptile_flag(g, tile_flag, x0, y0, tz * TZ, k) != 0;
    }
    uint32_t idle = __ballot_sync(0xffffffffu, !act);
    while (idle) {
      const int a = __ffs(idle) - 1;
      const uint32_t rest = ~(idle >> a);
      const int len = rest ? __ffs(rest) - 1 : 32 - a;  // idle tiles a .. a + len - 1
      idle &= len >= 32 ? 0u : ~(((1u << len) - 1u) << a);
      if (a + len >= 32) idle &= (1u << a) - 1u;
      const int z0 = (base + a) * TZ, z1 = min((base + a + len) * TZ, g.n[2]);
      if (!row || z1 <= z0) continue;
      const int64_t sb = (int64_t)z0 * sizeof(S), se = (int64_t)z1 * sizeof(S);
      for (int64_t o = sb; o < se; o += FB_ZBLOCK)
        bulk_store(srow + o, zblock, (uint32_t)(se - o < FB_ZBLOCK ? se - o : FB_ZBLOCK));
      if (drow)
        for (int64_t o = 3 * sb; o < 3 * se; o += FB_ZBLOCK)
          bulk_store(drow + o, zblock, (uint32_t)(3 * se - o < FB_ZBLOCK ? 3 * se - o : FB_ZBLOCK));
      any = true;
    }
  }
  if (any) bulk_commit();
}

// one active point tile (see the top of this file); for an evaluated field the
// point gradients go to the spheres' parameters (field_param_add into `part`) and
// only the deform's gradient is written.  zcol >= 0: warp 0 also writes that column's
// zeros (zero_column over the tile bits zflag) while the tile's edge adjoints run.
template <class S, int METHOD, class F = Field<S>, bool REC = false>
__device__ __forceinline__ void fused_tile(FusedShared<S, METHOD, REC>& sh, const F& f, const Geom& g,
                                           const uint64_t* __restrict__ seg, int64_t ptile, const S* __restrict__ gv,
                                           int64_t V, const S scale[3], int exact, S* __restrict__ gsdf,
                                           S* __restrict__ gdef, bool& bad, double* __restrict__ part = nullptr,
                                           const CellRec* __restrict__ codes = nullptr,
                                           const uint8_t* __restrict__ zflag = nullptr, int64_t zcol = -1) {
  using SH = FusedShared<S, METHOD, REC>;
  constexpr int LO = SH::LO, CX = SH::CX, CY = SH::CY, KX = SH::KX, KY = SH::KY;
  constexpr int CAP = fb_cap<S>();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int X0, Y0, Z0;
  ptile_coords(ptile, g, X0, Y0, Z0);
  const int zc = Z0 / TZ;
  // a narrow band's record blocks around the window (read after the first barrier)
  __shared__ typename F::RecTab rtab;
  if (REC && threadIdx.x < 12) f.rec_tab_fill(rtab, g, X0, Y0, Z0, threadIdx.x);
  // segment values first, so that their loads overlap the mask loads: MC, the
  // crossing counts of chunks zc, zc + 1 of the edge rows; DMC, the scanned values of
  // chunks zc - 1 .. zc + 2 of the window cell rows (patch bases, and which chunks
  // have a non-zero count)
  constexpr int RY = METHOD == MC ? CY : KY, SLO = METHOD == MC ? 0 : 1, NSEG = METHOD == MC ? 2 : 4;
  constexpr int NSV = (METHOD == MC ? CX * CY : KX * KY) * NSEG;
  static_assert(NSV <= NTHREADS, "one segment value per thread");
  uint64_t sv = 0;
  const int si = threadIdx.x, sk = si % NSEG, sy = (si / NSEG) % RY, sx = (si / NSEG) / RY;
  const int sc = zc + (METHOD == MC ? sk : sk - 1);
  bool sin = false;
  if (si < NSV) {
    const int X = X0 - SLO + sx, Y = Y0 - SLO + sy;
    // the value after a row's last chunk is the next row's first (the scan is
    // global); after the grid's last chunk, the total
    sin = X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1] && sc >= 0 && sc <= g.nzc && (sc < g.nzc || sk >= 2);
    if (sin) sv = seg[g.seg(X, Y, 0) + sc];
  }
  S dmn, dmx;
  bool dseen = false;
  // a warp's mask rows in batches of at most eight loads (more spill registers)
  constexpr int ROWS_PW = (SH::WX * SH::WY + NTHREADS / 32 - 1) / (NTHREADS / 32);
  constexpr int MBATCH = ROWS_PW <= 10 ? ROWS_PW : (ROWS_PW + 1) / 2;
  load_masks<S, SH::WX, SH::WY, false, F, MBATCH>(sh.m, f, X0 - LO, Y0 - LO, Z0, dmn, dmx, dseen);
  if constexpr (METHOD == MC) {
    if (si < NSV) sh.eb[sx][sy][sk] = Counts::lo(sv);
  } else {
    // chunk zc - 1 + k is busy when the scanned values at it and after it differ (the
    // four values of a row sit in four consecutive lanes; every lane shuffles)
    const uint64_t nxt = __shfl_down_sync(0xffffffffu, sv, 1, 4);
    const bool nin = __shfl_down_sync(0xffffffffu, sin ? 1 : 0, 1, 4) != 0;
    const uint32_t b = (sk < 3 && sin && nin && nxt != sv) ? (1u << sk) : 0u;
    const uint32_t bits = b | __shfl_down_sync(0xffffffffu, b, 1, 4) | __shfl_down_sync(0xffffffffu, b, 2, 4);
    if (si < NSV) {
      if (sk == 1 || sk == 2) sh.pb[sx][sy][sk - 1] = Counts::hi(sv);
      if (sk == 0) sh.busy[sx][sy] = (uint8_t)bits;
    }
  }
  __syncthreads();
  // DMC with the count's cell records: the window cells' records (resolved code,
  // first patch inside the segment) are loaded first, so that their latency passes
  // under the edge rows; segments with a zero count hold trivial cells only and have
  // no records.  Warp w: rows w, w + 8, ...; threads below 2 KX KY: the row ends
  // (cells Z0 - 1 and Z0 + TZ)
  constexpr int RPW = (KX * KY + NTHREADS / 32 - 1) / (NTHREADS / 32);
  int rec[METHOD == DMC && REC ? RPW : 1];
  int rend = 0;
  if constexpr (METHOD == DMC && REC) {
#pragma unroll
    for (int k = 0; k < RPW; ++k) {
      const int r = warp + (NTHREADS / 32) * k;
      rec[k] = 0;
      if (r < KX * KY) {
        const int wx = r / KY, wy = r % KY, X = X0 - 1 + wx, Y = Y0 - 1 + wy;
        const bool row = X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1];
        const uint32_t busy = row ? sh.busy[wx][wy] : 0u;
        if ((busy & 2) && Z0 + lane < g.c[2]) rec[k] = codes[f.rec_index_tab(rtab, g, X, Y, Z0 + lane)];
      }
    }
    if (threadIdx.x < 2 * KX * KY) {
      const int r = threadIdx.x >> 1, end = threadIdx.x & 1;
      const int wx = r / KY, wy = r % KY, X = X0 - 1 + wx, Y = Y0 - 1 + wy;
      const bool row = X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1];
      const uint32_t busy = row ? sh.busy[wx][wy] : 0u;
      const int Z = end ? Z0 + TZ : Z0 - 1;
      if ((busy & (end ? 4u : 1u)) && Z >= 0 && Z < g.c[2]) rend = codes[f.rec_index_tab(rtab, g, X, Y, Z)];
    }
  }
  // edge rows: crossing bits and the crossing flags of cell Z0 + TZ, one warp per row
  const uint32_t valid = zvalid(g, Z0);
  for (int r = warp; r < CX * CY; r += NTHREADS / 32) {
    const int x = r / CY, y = r % CY;
    RowBits rw = {0u, 0u, 0u, 0u};
    int f32 = 0;
    if (X0 + x < g.c[0] && Y0 + y < g.c[1]) {
      const uint64_t ma = sh.m[x + LO][y + LO], mb = sh.m[x + 1 + LO][y + LO], mc = sh.m[x + LO][y + 1 + LO],
                     md = sh.m[x + 1 + LO][y + 1 + LO];
      rw = row_bits(ma, mb, mc, md, valid);
      if (Z0 + TZ < g.c[2]) f32 = flags_at(ma, mb, mc, TZ + 1);
    }
    if (lane == 0) {
      sh.wb[x][y] = rw;
      sh.w32[x][y] = (uint8_t)f32;
    }
  }
  if constexpr (METHOD == DMC) {
   if constexpr (REC) {
    // the records loaded above, filed as the emit reads them
#pragma unroll
    for (int k = 0; k < RPW; ++k) {
      const int r = warp + (NTHREADS / 32) * k;
      if (r < KX * KY) {
        const int wx = r / KY, wy = r % KY;
        sh.rc[wx][wy][lane + 1] = (uint8_t)(rec[k] & 0xff);
        sh.first[wx][wy][lane + 1] = (int32_t)(sh.pb[wx][wy][0] + (uint32_t)(rec[k] >> 9));
      }
    }
    if (threadIdx.x < 2 * KX * KY) {
      const int r = threadIdx.x >> 1, end = threadIdx.x & 1;
      const int wx = r / KY, wy = r % KY;
      const int rc = rend & 0xff;
      sh.rc[wx][wy][end ? TZ + 1 : 0] = (uint8_t)rc;
      sh.first[wx][wy][end ? TZ + 1 : 0] =
          (int32_t)(end ? sh.pb[wx][wy][1] : sh.pb[wx][wy][0] - (uint32_t)dmc_npatch(sh.cases[rc]));
    }
   } else {
    // window cells: codes after the ambiguity test and first patch ids.  One warp per
    // cell row, lane j for cell Z0 + j (rows without a non-trivial cell need no test
    // and no scan); then one thread per row end for cells Z0 - 1 and Z0 + TZ.
    for (int r = warp; r < KX * KY; r += NTHREADS / 32) {
      const int wx = r / KY, wy = r % KY, X = X0 - 1 + wx, Y = Y0 - 1 + wy;
      const bool row = X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1];
      const uint32_t base = sh.pb[wx][wy][0];
      const uint64_t ma = sh.m[wx + 1][wy + 1], mb = sh.m[wx + 2][wy + 1], mc = sh.m[wx + 1][wy + 2],
                     md = sh.m[wx + 2][wy + 2];
      int code = 0;
      if (row && Z0 + lane < g.c[2]) code = code8(ma, mb, mc, md, lane + 1);
      const bool nt = code != 0 && code != 255;
      if (!__any_sync(0xffffffffu, nt)) {
        sh.rc[wx][wy][lane + 1] = 0;
        sh.first[wx][wy][lane + 1] = (int32_t)base;
        continue;
      }
      const int rc = nt ? fused_resolve<S, F>(sh.m, sh.cases, f, X0 - LO, Y0 - LO, Z0, code, X, Y, Z0 + lane, g) : 0;
      const uint32_t np = (uint32_t)dmc_npatch(sh.cases[rc]);
      const uint32_t incl = warp_incl(np);
      sh.rc[wx][wy][lane + 1] = (uint8_t)rc;
      sh.first[wx][wy][lane + 1] = (int32_t)(base + incl - np);
    }
    if (threadIdx.x < 2 * KX * KY) {
      const int r = threadIdx.x >> 1, end = threadIdx.x & 1;
      const int wx = r / KY, wy = r % KY, X = X0 - 1 + wx, Y = Y0 - 1 + wy;
      const int Z = end ? Z0 + TZ : Z0 - 1;
      int rc = 0;
      if (X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1] && Z >= 0 && Z < g.c[2]) {
        const int code = code8(sh.m[wx + 1][wy + 1], sh.m[wx + 2][wy + 1], sh.m[wx + 1][wy + 2],
                               sh.m[wx + 2][wy + 2], end ? TZ + 1 : 0);
        if (code != 0 && code != 255) rc = fused_resolve<S, F>(sh.m, sh.cases, f, X0 - LO, Y0 - LO, Z0, code, X, Y, Z, g);
      }
      sh.rc[wx][wy][end ? TZ + 1 : 0] = (uint8_t)rc;
      sh.first[wx][wy][end ? TZ + 1 : 0] =
          (int32_t)(end ? sh.pb[wx][wy][1] : sh.pb[wx][wy][0] - (uint32_t)dmc_npatch(sh.cases[rc]));
    }
   }
  }
  __syncthreads();
  // window slots: rows' bases by a block scan; slots in (row, cell, axis) order
  {
    uint32_t ce = 0;
    const int ex_ = threadIdx.x / CY, ey = threadIdx.x % CY;
    if (threadIdx.x < CX * CY) {
      const RowBits w = sh.wb[ex_][ey];
      ce = __popc(w.xc) + __popc(w.yc) + __popc(w.zc) + __popc(sh.w32[ex_][ey]);
    }
    uint32_t tot;
    const uint32_t off = block_excl_scan(ce, sh.wsum, tot);
    if (threadIdx.x == 0) sh.nwi = tot;
    // the row's first slot, parked in its cell TZ entry until the row is written
    if (threadIdx.x < CX * CY) sh.wcell[ex_][ey][TZ] = (uint16_t)off;
  }
  __syncthreads();
  // one warp per row writes its cells' first slots and flags, and the items
  for (int r = warp; r < CX * CY; r += NTHREADS / 32) {
    const int x = r / CY, y = r % CY;
    const uint32_t rbase = sh.wcell[x][y][TZ];
    __syncwarp();
    const RowBits w = sh.wb[x][y];
    const int fl = row_flags(w, lane);
    uint32_t o = rbase + (uint32_t)row_prefix(w, lane);
    sh.wcell[x][y][lane] = (uint16_t)(o | (fl << 13));
#pragma unroll
    for (int a = 0; a < 3; ++a)
      if (fl & (1 << a)) {
        if (o < (uint32_t)CAP) sh.witems[o] = item_code(x, y, lane, a);
        ++o;
      }
    if (lane == 31) {
      const int f32 = sh.w32[x][y];
      sh.wcell[x][y][TZ] = (uint16_t)(o | (f32 << 13));
#pragma unroll
      for (int a = 0; a < 3; ++a)
        if (f32 & (1 << a)) {
          if (o < (uint32_t)CAP) sh.witems[o] = item_code(x, y, TZ, a);
          ++o;
        }
    }
  }
  __syncthreads();
  const uint32_t nwi = sh.nwi;
  const bool cached = nwi <= (uint32_t)CAP;
  if (cached) {
    // warp 0 takes the last 32 of each round of items (the rounds are rarely full),
    // and then writes its column of zeros (zcol) while the others finish
    uint32_t i = (threadIdx.x + blockDim.x - 32) % blockDim.x;
    for (; i < nwi; i += blockDim.x) {
      int x, y, j, a;
      item_decode(sh.witems[i], x, y, j, a);
      S c0[4], c1[4];
      fused_edge_adjoint<S, METHOD, F, SH>(sh, f, X0, Y0, Z0, x, y, j, a, gv, V, scale, exact, c0, c1, bad);
      store_adj<S>(&sh.adj[0][0], i, c0, c1);
    }
    if (zcol >= 0 && warp == 0) zero_column<S>(g, zflag, zcol, gsdf, gdef, sh.zblock);
    __syncthreads();
  } else if (zcol >= 0 && warp == 0) {
    zero_column<S>(g, zflag, zcol, gsdf, gdef, sh.zblock);
  }
  // window slot of the edge along a owned by edge-row cell (x, y, j)
  auto slot = [&](int x, int y, int j, int a) -> int {
    const int w = sh.wcell[x][y][j];
    return (w & 0x1fff) + __popc((w >> 13) & ((1 << a) - 1));
  };
#pragma unroll 1
  for (int ix = 0; ix < TX; ++ix) {
    const int x = ix + 1, y = warp + 1, j = lane + 1;
    S acc[4] = {S(0), S(0), S(0), S(0)};
    // per axis the edge from this point (its first point), then the edge ending here,
    // in the stored backward's order (gather_tile in kernels.cuh)
    const int fo = sh.wcell[x][y][j] >> 13, fx = sh.wcell[x - 1][y][j] >> 13, fy = sh.wcell[x][y - 1][j] >> 13,
              fz = sh.wcell[x][y][j - 1] >> 13;
    const int on = (fo & 1) | ((fx & 1) << 1) | ((fo & 2) << 1) | ((fy & 2) << 2) | ((fo & 4) << 2) |
                   ((fz & 4) << 3);
    if (cached) {
#pragma unroll
      for (int e = 0; e < 6; ++e)
        if ((on >> e) & 1) {
          const S* o = &sh.adj[slot(x - (e == 1), y - (e == 3), j - (e == 5), e >> 1)][4 * (e & 1)];
          acc[0] += o[0];
          acc[1] += o[1];
          acc[2] += o[2];
          acc[3] += o[3];
        }
    } else {
#pragma unroll 1
      for (int e = 0; e < 6; ++e)
        if ((on >> e) & 1) {
          const Adj4<S> o =
              fused_edge_adjoint_far<S, METHOD, F, SH>(sh, f, X0, Y0, Z0, x - (e == 1), y - (e == 3), j - (e == 5), e >> 1,
                                                gv, V, scale[0], scale[1], scale[2], exact, e & 1);
          acc[0] += o.v[0];
          acc[1] += o.v[1];
          acc[2] += o.v[2];
          acc[3] += o.v[3];
          bad = bad || o.bad;
        }
    }
    const int X = X0 + 1 + ix, Y = Y0 + 1 + warp, Z = Z0 + 1 + lane;
    const bool in = f.inside(X, Y, Z);
    const int64_t i = ((int64_t)(X - 1) * f.n1 + (Y - 1)) * f.n2 + (Z - 1);
    if constexpr (F::kGrad == 2) {
      // a narrow band: the point's slot in the bricks (none in an absent brick)
      const int64_t b = in ? f.slot_point(X - 1, Y - 1, Z - 1) : -1;
      if (b >= 0) {
        gsdf[b] = acc[0];
        if (gdef) {
          gdef[3 * b + 0] = acc[1];
          gdef[3 * b + 1] = acc[2];
          gdef[3 * b + 2] = acc[3];
        }
      }
    } else if (in) {
      if constexpr (F::kGrad == 0) gsdf[i] = acc[0];
      if (gdef) {
        gdef[3 * i + 0] = acc[1];
        gdef[3 * i + 1] = acc[2];
        gdef[3 * i + 2] = acc[3];
      }
    }
    if constexpr (F::kGrad == 1) field_param_add<S>(f, part, in && acc[0] != S(0), X - 1, Y - 1, Z - 1, acc[0]);
  }
  __syncthreads();  // the shared arrays are reused by the CTA's next tile
}

// Persistent over the active point tiles in list[0 .. *count) (active_ptiles_kernel
// in kernels.cuh), CTA b taking entries b, b + gridDim.x, ...  DMC: `codes`, when
// given, are the forward count's cell records of this grid (read instead of
// recomputing the window cells' codes).  With zbulk, warp 0
// also zeroes the point tiles with no crossing nearby, column b, b + gridDim.x, ...
// of point tiles, one inside each of its active tiles and the rest after the last
// (bulk copies, zero_column); otherwise zero_tiles_kernel writes them beside it.  Bit 3 of
// stats->error is set when an index derived from the grid falls outside the
// forward's counts (the grid no longer matches the forward's record); no access
// leaves its buffer.
template <class S, int METHOD, bool REC = false>
__host__ __device__ constexpr size_t fused_smem() {
  return sizeof(FusedShared<S, METHOD, REC>);
}

template <class S, int METHOD, bool REC>
__global__ void __launch_bounds__(NTHREADS, 3)
    fused_backward_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg, const int* __restrict__ list,
                          const unsigned* __restrict__ count, const S* __restrict__ gv, int normalize, int exact,
                          S* __restrict__ gsdf, S* __restrict__ gdef, Stats* stats, int zbulk,
                          const CellRec* __restrict__ codes) {
  extern __shared__ __align__(16) unsigned char fb_smem[];
  FusedShared<S, METHOD, REC>& sh = *reinterpret_cast<FusedShared<S, METHOD, REC>*>(fb_smem);
  const uint8_t* tile_flag = reinterpret_cast<const uint8_t*>(seg + g.nseg + 1);
  const int64_t ncol = (int64_t)g.ptiles_x() * g.ptiles_y();
  int64_t col = blockIdx.x;  // the next column of point tiles this CTA zeroes
  if (zbulk) {
    for (int i = threadIdx.x; i < FB_ZBLOCK / 16; i += blockDim.x) sh.zblock[i] = make_uint4(0u, 0u, 0u, 0u);
    fence_proxy_async();  // the zeros are read by the bulk copies
  }
  const uint64_t tot = seg[g.nseg];
  const int64_t V = METHOD == MC ? (int64_t)Counts::lo(tot) : (int64_t)Counts::hi(tot);
  S scale[3];
  grad_scale<S>(g, normalize, scale);
  if constexpr (METHOD == DMC) sh.cases[threadIdx.x & 255] = dmc_case(threadIdx.x & 255);
  if (threadIdx.x < 24) sh.edge_of[threadIdx.x] = __ldg(g_edge_of + threadIdx.x);
  __syncthreads();
  const unsigned n = *count;
  bool bad = false;
  const int warp = threadIdx.x >> 5;
#pragma unroll 1
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x) {
    // a column of zeros, written by warp 0 inside the tile
    const int64_t zcol = zbulk && col < ncol ? col : -1;
    if (zcol >= 0) col += gridDim.x;
    fused_tile<S, METHOD, Field<S>, REC>(sh, f, g, seg, list[i], gv, V, scale, exact, gsdf, gdef, bad, nullptr,
                                         codes, tile_flag, zcol);
  }
  if (zbulk && warp == 0) {
    for (; col < ncol; col += gridDim.x) zero_column<S>(g, tile_flag, col, gsdf, gdef, sh.zblock);
    bulk_wait_all();  // the copies read shared memory: the CTA stays until they have
  }
  if (bad) atomicOr(&stats->error, 8ull);
}

// The backward of a narrow band (diso_backward_bricks): as fused_backward_kernel
// over the active point tiles in list[0 .. *count), the point gradients written to
// the bricks' slots (gval [K][512], gdef [K][512][3] or null; the caller zeroed them,
// points of tiles with no crossing nearby keep the zeros).  DMC with REC: the band's
// forward's cell records (`codes`).
template <class S, int METHOD, bool REC>
__global__ void __launch_bounds__(NTHREADS, 3)
    brick_backward_kernel(BrickField<S> f, Geom g, const uint64_t* __restrict__ seg, const int* __restrict__ list,
                          const unsigned* __restrict__ count, const S* __restrict__ gv, int normalize, int exact,
                          S* __restrict__ gval, S* __restrict__ gdef, Stats* stats,
                          const CellRec* __restrict__ codes) {
  extern __shared__ __align__(16) unsigned char fb_smem[];
  FusedShared<S, METHOD, REC>& sh = *reinterpret_cast<FusedShared<S, METHOD, REC>*>(fb_smem);
  const uint64_t tot = seg[g.nseg];
  const int64_t V = METHOD == MC ? (int64_t)Counts::lo(tot) : (int64_t)Counts::hi(tot);
  S scale[3];
  grad_scale<S>(g, normalize, scale);
  if constexpr (METHOD == DMC) sh.cases[threadIdx.x & 255] = dmc_case(threadIdx.x & 255);
  if (threadIdx.x < 24) sh.edge_of[threadIdx.x] = __ldg(g_edge_of + threadIdx.x);
  __syncthreads();
  const unsigned n = *count;
  bool bad = false;
#pragma unroll 1
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x)
    fused_tile<S, METHOD, BrickField<S>, REC>(sh, f, g, seg, list[i], gv, V, scale, exact, gval, gdef, bad, nullptr,
                                              codes);
  if (bad) atomicOr(&stats->error, 8ull);
}

// ------------------------------------------------------------------ evaluated fields

// sphere parameters whose gradients one field backward accumulates (per-warp
// partials in shared memory)
constexpr int FIELD_BWD_MAX_SPHERES = 64;

template <class S, int METHOD>
__host__ __device__ constexpr size_t field_bwd_smem(int K) {
  return (sizeof(FusedShared<S, METHOD>) + 15) / 16 * 16 + (size_t)(NTHREADS / 32) * K * 4 * sizeof(double);
}

// The backward of an evaluated union of spheres (diso_backward_field): CTA b takes
// point tiles b, b + gridDim.x, ... (a fixed assignment, so that the sums repeat);
// active tiles as fused_tile, with the point gradients going to the spheres'
// parameters; the deform's gradient written, zeros in the inactive tiles.  Each
// CTA's sums (per sphere: dL/dc, dL/dr) go to cta_part[b][K][4] in a fixed order.
template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS, 2)
    field_backward_kernel(SphereField<S> f, Geom g, const uint64_t* __restrict__ seg, const S* __restrict__ gv,
                          int normalize, int exact, S* __restrict__ gdef, double* __restrict__ cta_part,
                          Stats* stats) {
  extern __shared__ __align__(16) unsigned char fb_smem[];
  FusedShared<S, METHOD>& sh = *reinterpret_cast<FusedShared<S, METHOD>*>(fb_smem);
  double* part = reinterpret_cast<double*>(fb_smem + (sizeof(FusedShared<S, METHOD>) + 15) / 16 * 16);
  const int K = f.K, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < (NTHREADS / 32) * K * 4; i += blockDim.x) part[i] = 0.0;
  if constexpr (METHOD == DMC) sh.cases[threadIdx.x & 255] = dmc_case(threadIdx.x & 255);
  if (threadIdx.x < 24) sh.edge_of[threadIdx.x] = __ldg(g_edge_of + threadIdx.x);
  __syncthreads();
  const uint8_t* tile_flag = reinterpret_cast<const uint8_t*>(seg + g.nseg + 1);
  const uint64_t tot = seg[g.nseg];
  const int64_t V = METHOD == MC ? (int64_t)Counts::lo(tot) : (int64_t)Counts::hi(tot);
  S scale[3];
  grad_scale<S>(g, normalize, scale);
  bool bad = false;
#pragma unroll 1
  for (int64_t t = blockIdx.x; t < g.nptiles(); t += gridDim.x) {
    int x0, y0, z0;
    ptile_coords(t, g, x0, y0, z0);
    const int a = lane < 8 ? ptile_flag(g, tile_flag, x0, y0, z0, lane) : 0;
    if (__any_sync(0xffffffffu, a)) {  // the same in every warp
      fused_tile<S, METHOD, SphereField<S>>(sh, f, g, seg, t, gv, V, scale, exact, nullptr, gdef, bad, part);
    } else if (gdef) {
      const int nz = min(TZ, f.n2 - z0);
      for (int q = warp; q < TX * TY; q += NTHREADS / 32) {
        const int x = x0 + q / TY, y = y0 + q % TY;
        if (x >= f.n0 || y >= f.n1) continue;
        S* row = gdef + 3 * (((int64_t)x * f.n1 + y) * f.n2 + z0);
        for (int k = lane; k < 3 * nz; k += 32) row[k] = S(0);
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < K * 4; i += blockDim.x) {
    double acc = 0.0;
    for (int w = 0; w < NTHREADS / 32; ++w) acc += part[w * K * 4 + i];
    cta_part[(int64_t)blockIdx.x * K * 4 + i] = acc;
  }
  if (bad) atomicOr(&stats->error, 8ull);
}

// out[i] = the sum of cta_part[b][i] over the n CTAs in order (i < k4)
__global__ void __launch_bounds__(256) field_grad_final_kernel(const double* __restrict__ cta_part, int n, int k4,
                                                               double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k4; i += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int b = 0; b < n; ++b) acc += cta_part[(int64_t)b * k4 + i];
    out[i] = acc;
  }
}

}  // namespace diso
