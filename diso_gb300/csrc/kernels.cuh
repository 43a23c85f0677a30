// Forward and backward kernels of DiffMC / DiffDMC.
//
//   count_kernel      all tiles: case codes, per-segment crossing / face (MC) or
//                     crossing / patch (DMC) counts, the min/max of the SDF for the
//                     empty-surface guard, and the list of tiles with crossings
//   scan              scan.cuh
//   mc_emit_kernel    active tiles: MC vertices and triangles
//   dmc_emit_kernel   active tiles: DMC dual vertices and quads
//   *_backward_kernel all point tiles: dL/dsdf and dL/ddeform, every element written
//                     once (zeros away from the surface), crossings recomputed
//   split_*           DMC quad -> triangle split (return_quads=False)
#pragma once
#include "common.cuh"

namespace diso {

enum Method { MC = 0, DMC = 1 };

// lerp vertex of the edge from padded point (X,Y,Z) along axis a, in padded
// coordinates with deform (computeMcVert, src/cumc.cu:343-368)
template <class S, class Get>
__device__ __forceinline__ void edge_vertex(const Field<S>& f, Get get, int X, int Y, int Z, int a, S out[3]) {
  const int ex = a == 0, ey = a == 1, ez = a == 2;
  const S d0 = get(X, Y, Z), d1 = get(X + ex, Y + ey, Z + ez);
  S t = S(0.5);
  if (d1 != d0) {
    S r = (f.iso - d0) / (d1 - d0);
    r = S(0) > r ? S(0) : r;
    t = r < S(1) ? r : S(1);
  }
  S q0[3], q1[3];
  f.deform(X, Y, Z, q0);
  f.deform(X + ex, Y + ey, Z + ez, q1);
  const S p0[3] = {S(X) + q0[0], S(Y) + q0[1], S(Z) + q0[2]};
  const S p1[3] = {S(X + ex) + q1[0], S(Y + ey) + q1[1], S(Z + ez) + q1[2]};
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = p0[k] + (p1[k] - p0[k]) * t;
}

// verts - 1, then / (dim - 1) (diso/__init__.py:56-60)
template <class S>
__device__ __forceinline__ void store_vertex(S* __restrict__ verts, int64_t i, const S p[3], const Geom& g,
                                             int normalize) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    S v = p[k] - S(1);
    if (normalize) v = v / S(g.n[k] - 1);
    verts[3 * i + k] = v;
  }
}

__device__ __forceinline__ void tile_coords(int64_t tile, const Geom& g, int& X0, int& Y0, int& Z0, int& tz) {
  tz = (int)(tile % g.nzc);
  const int64_t r = tile / g.nzc;
  const int ty = (int)(r % g.tiles_y());
  const int tx = (int)(r / g.tiles_y());
  X0 = tx * TX;
  Y0 = ty * TY;
  Z0 = tz * TZ;
}

// ------------------------------------------------------------------ count

template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS) count_kernel(Field<S> f, Geom g, uint64_t* __restrict__ seg,
                                                         uint8_t* __restrict__ tile_flag, Stats* stats,
                                                         int* __restrict__ active) {
  __shared__ Window<S, TX + 1, TY + 1, TZ + 1> win;
  __shared__ S red_min[TY], red_max[TY];
  __shared__ uint32_t red_nv[TY];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t tile = blockIdx.x;
  int X0, Y0, Z0, tz;
  tile_coords(tile, g, X0, Y0, Z0, tz);
  win.load(f, X0, Y0, Z0);
  __syncthreads();
  auto get = [&](int X, int Y, int Z) { return win.get(f, X0, Y0, Z0, X, Y, Z); };

  uint32_t tile_nv = 0;
  // min / max of the caller's grid (the guard of diso/__init__.py:49), in the grid's dtype
  S mn = f.pad, mx = f.pad;
  bool any = false;
  const int Y = Y0 + warp, Z = Z0 + lane;
#pragma unroll 1
  for (int ix = 0; ix < TX; ++ix) {
    const int X = X0 + ix;
    const bool row = X < g.c[0] && Y < g.c[1];
    uint32_t nv = 0, nf = 0;
    if (row && Z < g.c[2]) {
      const int m = morton_code<S>(get, X, Y, Z, f.iso);
      nv = __popc(cross_flags(m));
      if (METHOD == MC) {
        nf = (uint32_t)(mc_tri(mc_from_morton(m)) & 15);
      } else if (m != 0 && m != 255) {
        nf = dmc_npatch(dmc_case(dmc_resolve<S>(get, m, X, Y, Z, g.c, f.iso)));
      }
      if (X >= 1 && Y >= 1 && Z >= 1) {
        const S v = get(X, Y, Z);
        mn = any ? (v < mn ? v : mn) : v;
        mx = any ? (v > mx ? v : mx) : v;
        any = true;
      }
    }
    const uint32_t snv = warp_sum(nv), snf = warp_sum(nf);
    if (lane == 0 && row) seg[g.seg(X, Y, tz)] = Counts::pack(snv, snf);
    // a cell can emit faces / patches without owning a crossing edge (its
    // crossings may all sit on edges owned by its +1 neighbours)
    tile_nv += snv + snf;
  }
  // lanes without an interior point hold the pad value, which never decides the guard
  // because the guard only asks min >= iso or max <= iso of the interior values;
  // replace them by a value already seen in the warp
  const unsigned have = __ballot_sync(0xffffffffu, any);
  if (have) {
    const int src = __ffs(have) - 1;
    const S m0 = __shfl_sync(0xffffffffu, mn, src), x0 = __shfl_sync(0xffffffffu, mx, src);
    if (!any) {
      mn = m0;
      mx = x0;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const S a = __shfl_xor_sync(0xffffffffu, mn, o), b = __shfl_xor_sync(0xffffffffu, mx, o);
      mn = a < mn ? a : mn;
      mx = b > mx ? b : mx;
    }
  }
  if (lane == 0) {
    red_min[warp] = mn;
    red_max[warp] = mx;
    red_nv[warp] = tile_nv | (have ? 0x80000000u : 0u);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    bool seen = false;
    for (int w = 0; w < TY; ++w) {
      if (red_nv[w] & 0x80000000u) {
        mn = seen ? (red_min[w] < mn ? red_min[w] : mn) : red_min[w];
        mx = seen ? (red_max[w] > mx ? red_max[w] : mx) : red_max[w];
        seen = true;
      }
      t += red_nv[w] & 0x7fffffffu;
    }
    if (seen) {
      atomicMin(&stats->min_key, ord_key((double)mn));
      atomicMax(&stats->max_key, ord_key((double)mx));
    }
    tile_flag[tile] = t ? 1 : 0;
    if (t) active[atomicAdd(&stats->n_active, 1ull)] = (int)tile;
  }
}

// ------------------------------------------------------------------ MC emit

template <class S>
__global__ void __launch_bounds__(NTHREADS) mc_emit_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg,
                                                           const int* __restrict__ active, S* __restrict__ verts,
                                                           int64_t* __restrict__ faces, int normalize) {
  constexpr int CX = TX + 1, CY = TY + 1, CZ = TZ + 1;  // cells [X0, X0+TX] x [Y0, Y0+TY] x [Z0, Z0+TZ]
  __shared__ Window<S, TX + 2, TY + 2, TZ + 2> win;     // points [X0, X0+TX+1] ...
  __shared__ uint8_t flg[CX][CY][CZ];
  __shared__ uint8_t pre[CX][CY][CZ];
  __shared__ uint32_t vb[CX][CY][2];
  __shared__ uint32_t fb[TX][TY];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int X0, Y0, Z0, tz;
  tile_coords(active[blockIdx.x], g, X0, Y0, Z0, tz);
  win.load(f, X0, Y0, Z0);
  for (int i = threadIdx.x; i < CX * CY * 2; i += blockDim.x) {
    const int k = i & 1, y = (i >> 1) % CY, x = (i >> 1) / CY;
    const int X = X0 + x, Y = Y0 + y, zc = tz + k;
    uint64_t s = (X < g.c[0] && Y < g.c[1] && zc < g.nzc) ? seg[g.seg(X, Y, zc)] : 0ull;
    vb[x][y][k] = Counts::lo(s);
    if (k == 0 && x < TX && y < TY) fb[x][y] = Counts::hi(s);
  }
  __syncthreads();
  auto get = [&](int X, int Y, int Z) { return win.get(f, X0, Y0, Z0, X, Y, Z); };

  // crossing flags and in-segment prefixes of the tile's cells and their +1 halo
  for (int r = warp; r < CX * CY; r += TY) {
    const int x = r / CY, y = r % CY, X = X0 + x, Y = Y0 + y;
    const bool row = X < g.c[0] && Y < g.c[1];
    int fl = (row && Z0 + lane < g.c[2]) ? cross_flags(morton_code<S>(get, X, Y, Z0 + lane, f.iso)) : 0;
    const uint32_t c = __popc(fl);
    const uint32_t inc = warp_incl(c);
    flg[x][y][lane] = (uint8_t)fl;
    pre[x][y][lane] = (uint8_t)(inc - c);
    if (lane == 0) {
      const int Zh = Z0 + TZ;
      flg[x][y][TZ] = (uint8_t)((row && Zh < g.c[2]) ? cross_flags(morton_code<S>(get, X, Y, Zh, f.iso)) : 0);
      pre[x][y][TZ] = 0;  // first cell of the next segment
    }
  }
  __syncthreads();

  const int Y = Y0 + warp, Z = Z0 + lane;
#pragma unroll 1
  for (int ix = 0; ix < TX; ++ix) {
    const int X = X0 + ix;
    const bool valid = X < g.c[0] && Y < g.c[1] && Z < g.c[2];
    // vertices: one per crossing edge owned by the cell, in axis order (src/cumc.cu:370-410)
    const int fl = flg[ix][warp][lane];
    if (valid && fl) {
      int64_t vid = (int64_t)vb[ix][warp][0] + pre[ix][warp][lane];
#pragma unroll
      for (int a = 0; a < 3; ++a)
        if (fl & (1 << a)) {
          S p[3];
          edge_vertex<S>(f, get, X, Y, Z, a, p);
          store_vertex<S>(verts, vid++, p, g, normalize);
        }
    }
    // triangles (src/cumc.cu:564-649): each table edge -> owner cell (+0/+1) -> its vertex
    const uint64_t w = valid ? mc_tri(mc_from_morton(morton_code<S>(get, X, Y, Z, f.iso))) : 0ull;
    const uint32_t nt = (uint32_t)(w & 15);
    const uint32_t tinc = warp_incl(nt);
    if (nt) {
      const int64_t f0 = (int64_t)fb[ix][warp] + (tinc - nt);
      for (uint32_t t = 0; t < nt; ++t) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int e = (int)((w >> (4 + 4 * (3 * t + k))) & 15);
          const int ge = g_edge[e];
          const int ox = ix + (ge & 1), oy = warp + ((ge >> 1) & 1), oz = lane + ((ge >> 2) & 1), a = ge >> 3;
          const int ofl = flg[ox][oy][oz];
          const int64_t id = (int64_t)vb[ox][oy][oz == TZ ? 1 : 0] + pre[ox][oy][oz] + __popc(ofl & ((1 << a) - 1));
          faces[3 * (f0 + t) + k] = id;
        }
      }
    }
  }
}

// ------------------------------------------------------------------ DMC emit

template <class S>
__global__ void __launch_bounds__(NTHREADS) dmc_emit_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg,
                                                            const int* __restrict__ active, S* __restrict__ verts,
                                                            int64_t* __restrict__ quads, int normalize) {
  constexpr int CX = TX + 1, CY = TY + 1, CZ = TZ + 1;  // cells [X0-1, X0+TX) x [Y0-1, Y0+TY) x [Z0-1, Z0+TZ)
  __shared__ Window<S, TX + 2, TY + 2, TZ + 2> win;     // points [X0-1, X0+TX] ...
  __shared__ uint8_t rc[CX][CY][CZ];
  __shared__ int16_t pp[CX][CY][CZ];
  __shared__ uint32_t pb[CX][CY];
  __shared__ uint32_t qb[TX][TY];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int X0, Y0, Z0, tz;
  tile_coords(active[blockIdx.x], g, X0, Y0, Z0, tz);
  win.load(f, X0 - 1, Y0 - 1, Z0 - 1);
  for (int i = threadIdx.x; i < CX * CY; i += blockDim.x) {
    const int y = i % CY, x = i / CY;
    const int X = X0 - 1 + x, Y = Y0 - 1 + y;
    uint64_t s = (X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1]) ? seg[g.seg(X, Y, tz)] : 0ull;
    pb[x][y] = Counts::hi(s);
    if (x >= 1 && y >= 1) qb[x - 1][y - 1] = Counts::lo(s);
  }
  __syncthreads();
  auto get = [&](int X, int Y, int Z) { return win.get(f, X0 - 1, Y0 - 1, Z0 - 1, X, Y, Z); };

  // resolved codes and in-segment patch prefixes of the tile's cells and their -1 halo
  for (int r = warp; r < CX * CY; r += TY) {
    const int x = r / CY, y = r % CY, X = X0 - 1 + x, Y = Y0 - 1 + y;
    const bool row = X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1];
    int code = 0;
    if (row && Z0 + lane < g.c[2]) {
      const int m = morton_code<S>(get, X, Y, Z0 + lane, f.iso);
      code = (m == 0 || m == 255) ? m : dmc_resolve<S>(get, m, X, Y, Z0 + lane, g.c, f.iso);
    }
    const uint32_t np = dmc_npatch(dmc_case(code));
    const uint32_t inc = warp_incl(np);
    rc[x][y][lane + 1] = (uint8_t)code;
    pp[x][y][lane + 1] = (int16_t)(inc - np);
    if (lane == 0) {
      int c0 = 0;
      if (row && Z0 >= 1) {
        const int m = morton_code<S>(get, X, Y, Z0 - 1, f.iso);
        c0 = (m == 0 || m == 255) ? m : dmc_resolve<S>(get, m, X, Y, Z0 - 1, g.c, f.iso);
      }
      rc[x][y][0] = (uint8_t)c0;
      pp[x][y][0] = (int16_t)(-(int)dmc_npatch(dmc_case(c0)));  // last cell of the previous segment
    }
  }
  __syncthreads();

  const int Y = Y0 + warp, Z = Z0 + lane;
#pragma unroll 1
  for (int ix = 0; ix < TX; ++ix) {
    const int X = X0 + ix;
    const bool valid = X < g.c[0] && Y < g.c[1] && Z < g.c[2];
    const int code = valid ? rc[ix + 1][warp + 1][lane + 1] : 0;
    const uint64_t w = dmc_case(code);
    const int np = dmc_npatch(w);
    // dual vertices: mean of the patch's edge vertices, edges in ascending id
    // (create_dmc_verts_kernel, src/cudualmc.cu:907-955)
    if (np) {
      S acc[4][3];
      int cnt[4] = {0, 0, 0, 0};
#pragma unroll
      for (int p = 0; p < 4; ++p) acc[p][0] = acc[p][1] = acc[p][2] = S(0);
#pragma unroll
      for (int e = 0; e < 12; ++e) {
        const int ge = g_edge[e], s = ge & 7, a = ge >> 3;
        if ((((code >> s) ^ (code >> (s | (1 << a)))) & 1) == 0) continue;
        const int p = dmc_patch_of(w, e);
        S v[3];
        edge_vertex<S>(f, get, X + (s & 1), Y + ((s >> 1) & 1), Z + ((s >> 2) & 1), a, v);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (q == p) {
            acc[q][0] += v[0];
            acc[q][1] += v[1];
            acc[q][2] += v[2];
            cnt[q] += 1;
          }
      }
      const int64_t p0 = (int64_t)pb[ix + 1][warp + 1] + pp[ix + 1][warp + 1][lane + 1];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q < np) {
          const S inv = S(1) / S(cnt[q]);
          const S v[3] = {acc[q][0] * inv, acc[q][1] * inv, acc[q][2] * inv};
          store_vertex<S>(verts, p0 + q, v, g, normalize);
        }
    }
    // quads: one per crossing edge owned by the cell (src/cudualmc.cu:753-794, 1019-1056)
    const int fl = cross_flags(code);
    const uint32_t c = __popc(fl);
    const uint32_t inc = warp_incl(c);
    if (fl) {
      int64_t qid = (int64_t)qb[ix][warp] + (inc - c);
      const S d0 = get(X, Y, Z);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (!(fl & (1 << a))) continue;
        const S d1 = get(X + (a == 0), Y + (a == 1), Z + (a == 2));
        const int type = a + ((d1 < f.iso && d0 >= f.iso) ? 3 : 0);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = g_dmc_quad[4 * type + i];
          const int nx = ix + 1 + (q & 3) - 1, ny = warp + 1 + ((q >> 2) & 3) - 1, nz = lane + 1 + ((q >> 4) & 3) - 1;
          const int eid = q >> 8;
          const int64_t pid = (int64_t)pb[nx][ny] + pp[nx][ny][nz] + dmc_patch_of(dmc_case(rc[nx][ny][nz]), eid);
          quads[4 * qid + i] = pid;
        }
        ++qid;
      }
    }
  }
}

// ------------------------------------------------------------------ backward

// dL/dverts of vertex i in padded coordinates: the chain rule of "- 1" and "/ (dim - 1)"
template <class S>
__device__ __forceinline__ void load_grad(const S* __restrict__ gv, int64_t i, const Geom& g, int normalize, S out[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    S v = __ldg(gv + 3 * i + k);
    out[k] = normalize ? v / S(g.n[k] - 1) : v;
  }
}

// adjoint of edge_vertex at one endpoint (adjComputeMcVert, src/cumc.cu:412-453):
// the edge runs from padded point A along axis a; `end` = 0 when the point being
// differentiated is A, 1 when it is A + e_a.  Adds into gs (dL/dsdf) and gd.
template <class S, class Get>
__device__ __forceinline__ void edge_adjoint(const Field<S>& f, Get get, int X, int Y, int Z, int a, int end,
                                             const S gvec[3], S& gs, S gd[3]) {
  const int ex = a == 0, ey = a == 1, ez = a == 2;
  const S d0 = get(X, Y, Z), d1 = get(X + ex, Y + ey, Z + ez);
  S t = S(0.5);
  if (d1 != d0) {
    S r = (f.iso - d0) / (d1 - d0);
    r = S(0) > r ? S(0) : r;
    t = r < S(1) ? r : S(1);
  }
  S q0[3], q1[3];
  f.deform(X, Y, Z, q0);
  f.deform(X + ex, Y + ey, Z + ez, q1);
  const S dp[3] = {(S(X + ex) + q1[0]) - (S(X) + q0[0]), (S(Y + ey) + q1[1]) - (S(Y) + q0[1]),
                   (S(Z + ez) + q1[2]) - (S(Z) + q0[2])};
  const S adj_t = dp[0] * gvec[0] + dp[1] * gvec[1] + dp[2] * gvec[2];
  const S den = (d1 - d0) * (d1 - d0);
  if (end == 0) {
    gs += (f.iso - d1) / den * adj_t;
    const S w = S(1) - t;
    gd[0] += w * gvec[0];
    gd[1] += w * gvec[1];
    gd[2] += w * gvec[2];
  } else {
    gs += (d0 - f.iso) / den * adj_t;
    gd[0] += t * gvec[0];
    gd[1] += t * gvec[1];
    gd[2] += t * gvec[2];
  }
}

// Per point tile (unpadded points [x0, x0+TX) x [y0, y0+TY) x [z0, z0+TZ)), the
// cells [x0, x0+TX] x ... (padded coordinates; cell x0+i owns point x0+i as corner 0)
// own every edge that touches the tile's points.  They lie in the forward tiles
// (x0/TX + {0,1}, y0/TY + {0,1}, z0/TZ + {0,1}); the tile is inactive when none of
// them holds a crossing.
__device__ __forceinline__ bool ptile_active(const Geom& g, const uint8_t* __restrict__ tile_flag, int x0, int y0,
                                             int z0) {
  int a = 0;
  if (threadIdx.x < 8) {
    const int tx = x0 / TX + (threadIdx.x & 1), ty = y0 / TY + ((threadIdx.x >> 1) & 1),
              tz = z0 / TZ + (threadIdx.x >> 2);
    if (tx < g.tiles_x() && ty < g.tiles_y() && tz < g.nzc) a = tile_flag[((int64_t)tx * g.tiles_y() + ty) * g.nzc + tz];
  }
  return __syncthreads_or(a) != 0;
}

// zero dL/dsdf and dL/ddeform of a point tile; float4 stores when rows are 16-byte aligned
template <class S>
__device__ __forceinline__ void zero_ptile(const Field<S>& f, S* __restrict__ gsdf, S* __restrict__ gdef, int x0, int y0,
                                           int z0) {
  const int nz = min(TZ, f.n2 - z0);
  if (sizeof(S) == 4 && (f.n2 & 3) == 0) {
    const int r = threadIdx.x >> 3, k = threadIdx.x & 7;  // 32 rows x 8 float4
    const int x = x0 + r / TY, y = y0 + r % TY;
    if (x < f.n0 && y < f.n1) {
      const int64_t base = ((int64_t)x * f.n1 + y) * f.n2 + z0;
      const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
      if (4 * k < nz) reinterpret_cast<float4*>(gsdf + base)[k] = z4;
      if (gdef) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int q = k + 8 * j;
          if (4 * q < 3 * nz) reinterpret_cast<float4*>(gdef + 3 * base)[q] = z4;
        }
      }
    }
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int ix = 0; ix < TX; ++ix) {
    const int x = x0 + ix, y = y0 + warp, z = z0 + lane;
    if (x < f.n0 && y < f.n1 && z < f.n2) {
      const int64_t i = ((int64_t)x * f.n1 + y) * f.n2 + z;
      gsdf[i] = S(0);
      if (gdef) gdef[3 * i] = gdef[3 * i + 1] = gdef[3 * i + 2] = S(0);
    }
  }
}

template <class S>
__device__ __forceinline__ void ptile_coords(int64_t tile, const Geom& g, int& x0, int& y0, int& z0) {
  const int tz = (int)(tile % g.ptiles_z());
  const int64_t r = tile / g.ptiles_z();
  y0 = (int)(r % g.ptiles_y()) * TY;
  x0 = (int)(r / g.ptiles_y()) * TX;
  z0 = tz * TZ;
}

template <class S>
__device__ __forceinline__ void write_point_grads(const Field<S>& f, S* __restrict__ gsdf, S* __restrict__ gdef,
                                                  int X, int Y, int Z, S gs, const S gd[3]) {
  if (!f.inside(X, Y, Z)) return;
  const int64_t i = f.lin(X, Y, Z);
  gsdf[i] = gs;
  if (gdef) {
    gdef[3 * i + 0] = gd[0];
    gdef[3 * i + 1] = gd[1];
    gdef[3 * i + 2] = gd[2];
  }
}

// MC: dL/dsdf and dL/ddeform of every point, gathered from its (at most six)
// incident crossing edges.  Replaces adj_create_cell_mc_verts_kernel
// (src/cumc.cu:474-512) plus the zero fills and the F.pad backward.
template <class S>
__global__ void __launch_bounds__(NTHREADS) mc_backward_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg,
                                                               const uint8_t* __restrict__ tile_flag,
                                                               const S* __restrict__ gv, int normalize,
                                                               S* __restrict__ gsdf, S* __restrict__ gdef) {
  constexpr int CX = TX + 1, CY = TY + 1, CZ = TZ + 1;  // cells [X0, X0+TX] x ...
  __shared__ Window<S, TX + 2, TY + 2, TZ + 2> win;     // points [X0, X0+TX+1] ...
  __shared__ uint8_t flg[CX][CY][CZ];
  __shared__ uint8_t pre[CX][CY][CZ];
  __shared__ uint32_t vb[CX][CY][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int X0, Y0, Z0;  // padded cell origin = unpadded point origin
  ptile_coords<S>(blockIdx.x, g, X0, Y0, Z0);
  const int zc = Z0 / TZ;
  if (!ptile_active(g, tile_flag, X0, Y0, Z0)) {
    zero_ptile<S>(f, gsdf, gdef, X0, Y0, Z0);
    return;
  }
  win.load(f, X0, Y0, Z0);
  for (int i = threadIdx.x; i < CX * CY * 2; i += blockDim.x) {
    const int k = i & 1, y = (i >> 1) % CY, x = (i >> 1) / CY;
    const int X = X0 + x, Y = Y0 + y, c = zc + k;
    vb[x][y][k] = (X < g.c[0] && Y < g.c[1] && c < g.nzc) ? Counts::lo(seg[g.seg(X, Y, c)]) : 0u;
  }
  __syncthreads();
  auto get = [&](int X, int Y, int Z) { return win.get(f, X0, Y0, Z0, X, Y, Z); };
  for (int r = warp; r < CX * CY; r += TY) {
    const int x = r / CY, y = r % CY, X = X0 + x, Y = Y0 + y;
    const bool row = X < g.c[0] && Y < g.c[1];
    int fl = (row && Z0 + lane < g.c[2]) ? cross_flags(morton_code<S>(get, X, Y, Z0 + lane, f.iso)) : 0;
    const uint32_t c = __popc(fl);
    const uint32_t inc = warp_incl(c);
    flg[x][y][lane] = (uint8_t)fl;
    pre[x][y][lane] = (uint8_t)(inc - c);
    if (lane == 0) {
      const int Zh = Z0 + TZ;
      flg[x][y][TZ] = (uint8_t)((row && Zh < g.c[2]) ? cross_flags(morton_code<S>(get, X, Y, Zh, f.iso)) : 0);
      pre[x][y][TZ] = 0;
    }
  }
  __syncthreads();
  auto vid = [&](int x, int y, int z, int a) -> int64_t {
    return (int64_t)vb[x][y][z == TZ ? 1 : 0] + pre[x][y][z] + __popc(flg[x][y][z] & ((1 << a) - 1));
  };
  for (int ix = 0; ix < TX; ++ix) {
    // point (X, Y, Z) padded = cell index (ix+1, warp+1, lane+1) in the window
    const int x = ix + 1, y = warp + 1, z = lane + 1;
    const int X = X0 + x, Y = Y0 + y, Z = Z0 + z;
    S gs = S(0), gd[3] = {S(0), S(0), S(0)};
    if (f.inside(X, Y, Z)) {
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (flg[x][y][z] & (1 << a)) {
          S gvec[3];
          load_grad<S>(gv, vid(x, y, z, a), g, normalize, gvec);
          edge_adjoint<S>(f, get, X, Y, Z, a, 0, gvec, gs, gd);
        }
        const int px = x - (a == 0), py = y - (a == 1), pz = z - (a == 2);
        if (flg[px][py][pz] & (1 << a)) {
          S gvec[3];
          load_grad<S>(gv, vid(px, py, pz, a), g, normalize, gvec);
          edge_adjoint<S>(f, get, X0 + px, Y0 + py, Z0 + pz, a, 1, gvec, gs, gd);
        }
      }
    }
    write_point_grads<S>(f, gsdf, gdef, X, Y, Z, gs, gd);
  }
}

// DMC: as above, but the gradient reaching an edge vertex is the sum over the
// four cells around the edge of dL/d(dual vertex) / (edges in that patch)
// (adj_create_dmc_verts_kernel, src/cudualmc.cu:957-1005).  The reference reads
// the gradient of the cell's first patch for every patch of the cell
// (adj_verts[first] with first never advanced, src/cudualmc.cu:990); exact = 0
// reproduces that, exact = 1 uses each patch's own gradient (the true derivative).
template <class S>
__global__ void __launch_bounds__(NTHREADS) dmc_backward_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg,
                                                                const uint8_t* __restrict__ tile_flag,
                                                                const S* __restrict__ gv, int normalize, int exact,
                                                                S* __restrict__ gsdf, S* __restrict__ gdef) {
  constexpr int CX = TX + 1, CY = TY + 1, CZ = TZ + 1;  // cells [X0, X0+TX] x ...
  __shared__ Window<S, TX + 2, TY + 2, TZ + 2> win;     // points [X0, X0+TX+1] ...
  __shared__ uint8_t rc[CX][CY][CZ];
  __shared__ uint8_t pre[CX][CY][CZ];
  __shared__ uint32_t pb[CX][CY][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int X0, Y0, Z0;
  ptile_coords<S>(blockIdx.x, g, X0, Y0, Z0);
  const int zc = Z0 / TZ;
  if (!ptile_active(g, tile_flag, X0, Y0, Z0)) {
    zero_ptile<S>(f, gsdf, gdef, X0, Y0, Z0);
    return;
  }
  win.load(f, X0, Y0, Z0);
  for (int i = threadIdx.x; i < CX * CY * 2; i += blockDim.x) {
    const int k = i & 1, y = (i >> 1) % CY, x = (i >> 1) / CY;
    const int X = X0 + x, Y = Y0 + y, c = zc + k;
    pb[x][y][k] = (X < g.c[0] && Y < g.c[1] && c < g.nzc) ? Counts::hi(seg[g.seg(X, Y, c)]) : 0u;
  }
  __syncthreads();
  auto get = [&](int X, int Y, int Z) { return win.get(f, X0, Y0, Z0, X, Y, Z); };
  auto resolved = [&](int X, int Y, int Z) -> int {
    const int m = morton_code<S>(get, X, Y, Z, f.iso);
    return (m == 0 || m == 255) ? m : dmc_resolve<S>(get, m, X, Y, Z, g.c, f.iso);
  };
  for (int r = warp; r < CX * CY; r += TY) {
    const int x = r / CY, y = r % CY, X = X0 + x, Y = Y0 + y;
    const bool row = X < g.c[0] && Y < g.c[1];
    const int code = (row && Z0 + lane < g.c[2]) ? resolved(X, Y, Z0 + lane) : 0;
    const uint32_t np = dmc_npatch(dmc_case(code));
    const uint32_t inc = warp_incl(np);
    rc[x][y][lane] = (uint8_t)code;
    pre[x][y][lane] = (uint8_t)(inc - np);
    if (lane == 0) {
      const int Zh = Z0 + TZ;
      rc[x][y][TZ] = (uint8_t)((row && Zh < g.c[2]) ? resolved(X, Y, Zh) : 0);
      pre[x][y][TZ] = 0;
    }
  }
  __syncthreads();
  // dL/d(edge vertex) of the crossing edge owned by window cell (ox, oy, oz) along a
  auto edge_grad = [&](int ox, int oy, int oz, int a, S out[3]) {
    out[0] = out[1] = out[2] = S(0);
    const int b = (a + 1) % 3, c = (a + 2) % 3;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int db = k & 1, dc = k >> 1;
      int cell[3] = {ox, oy, oz};
      cell[b] -= db;
      cell[c] -= dc;
      int st[3] = {0, 0, 0};
      st[b] = db;
      st[c] = dc;
      const int code = rc[cell[0]][cell[1]][cell[2]];
      const uint64_t w = dmc_case(code);
      const int p = dmc_patch_of(w, edge_id(st[0], st[1], st[2], a));
      const S inv = S(1) / S(dmc_patch_size(w, p));
      const int64_t pid =
          (int64_t)pb[cell[0]][cell[1]][cell[2] == TZ ? 1 : 0] + pre[cell[0]][cell[1]][cell[2]] + (exact ? p : 0);
      S v[3];
      load_grad<S>(gv, pid, g, normalize, v);
      out[0] += v[0] * inv;
      out[1] += v[1] * inv;
      out[2] += v[2] * inv;
    }
  };
  for (int ix = 0; ix < TX; ++ix) {
    const int x = ix + 1, y = warp + 1, z = lane + 1;
    const int X = X0 + x, Y = Y0 + y, Z = Z0 + z;
    S gs = S(0), gd[3] = {S(0), S(0), S(0)};
    if (f.inside(X, Y, Z)) {
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (cross_flags(rc[x][y][z]) & (1 << a)) {
          S gvec[3];
          edge_grad(x, y, z, a, gvec);
          edge_adjoint<S>(f, get, X, Y, Z, a, 0, gvec, gs, gd);
        }
        const int px = x - (a == 0), py = y - (a == 1), pz = z - (a == 2);
        if (cross_flags(rc[px][py][pz]) & (1 << a)) {
          S gvec[3];
          edge_grad(px, py, pz, a, gvec);
          edge_adjoint<S>(f, get, X0 + px, Y0 + py, Z0 + pz, a, 1, gvec, gs, gd);
        }
      }
    }
    write_point_grads<S>(f, gsdf, gdef, X, Y, Z, gs, gd);
  }
}

// ------------------------------------------------------------------ quad split

// largest corner cosine of triangle (a, b, c), as diso/__init__.py:125-130 computes
// it: F.normalize(u) = u / max(|u|, 1e-12)
template <class S>
__device__ __forceinline__ S tri_max_cos(const S* __restrict__ V, int64_t ia, int64_t ib, int64_t ic) {
  S p[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    p[0][k] = V[3 * ia + k];
    p[1][k] = V[3 * ib + k];
    p[2][k] = V[3 * ic + k];
  }
  S m = S(0);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const S* o = p[i];
    const S* u = p[(i + 1) % 3];
    const S* w = p[(i + 2) % 3];
    S e1[3] = {u[0] - o[0], u[1] - o[1], u[2] - o[2]};
    S e2[3] = {w[0] - o[0], w[1] - o[1], w[2] - o[2]};
    S n1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    S n2 = sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
    n1 = n1 > S(1e-12) ? n1 : S(1e-12);
    n2 = n2 > S(1e-12) ? n2 : S(1e-12);
    const S c = (e1[0] / n1) * (e2[0] / n2) + (e1[1] / n1) * (e2[1] / n2) + (e1[2] / n1) * (e2[2] / n2);
    m = (i == 0 || c > m || c != c) ? c : m;
  }
  return m;
}

// 1: split (0,1,3),(1,2,3); 2: split (0,1,2),(0,2,3); 0: NaN (the reference drops the quad)
template <class S>
__device__ __forceinline__ int split_config(const S* __restrict__ V, const int64_t* q) {
  const S a1 = tri_max_cos<S>(V, q[0], q[1], q[3]), b1 = tri_max_cos<S>(V, q[1], q[2], q[3]);
  const S a2 = tri_max_cos<S>(V, q[0], q[1], q[2]), b2 = tri_max_cos<S>(V, q[0], q[2], q[3]);
  const S m1 = (a1 != a1 || a1 > b1) ? a1 : b1;
  const S m2 = (a2 != a2 || a2 > b2) ? a2 : b2;
  if (m1 < m2) return 1;
  if (m1 >= m2) return 2;
  return 0;
}

template <class S>
__global__ void split_count_kernel(const S* __restrict__ verts, const int64_t* __restrict__ quads, int64_t nq,
                                   uint64_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t q[4] = {quads[4 * i], quads[4 * i + 1], quads[4 * i + 2], quads[4 * i + 3]};
    const int c = split_config<S>(verts, q);
    cnt[i] = c == 1 ? 1ull : (c == 2 ? (1ull << 32) : 0ull);
  }
}

// config-1 quads' triangle pairs first, then config-2's, each in quad order
// (diso/__init__.py:140-145)
__global__ void split_scatter_kernel(const int64_t* __restrict__ quads, int64_t nq, const uint64_t* __restrict__ pos,
                                     int64_t* __restrict__ tris) {
  const uint64_t total = pos[nq];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = pos[i], b = pos[i + 1];
    const int64_t* q = quads + 4 * i;
    int64_t t[6];
    int64_t at;
    if (Counts::lo(b) != Counts::lo(a)) {
      at = 2 * (int64_t)Counts::lo(a);
      t[0] = q[0]; t[1] = q[1]; t[2] = q[3]; t[3] = q[1]; t[4] = q[2]; t[5] = q[3];
    } else if (Counts::hi(b) != Counts::hi(a)) {
      at = 2 * ((int64_t)Counts::lo(total) + Counts::hi(a));
      t[0] = q[0]; t[1] = q[1]; t[2] = q[2]; t[3] = q[0]; t[4] = q[2]; t[5] = q[3];
    } else {
      continue;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) tris[3 * at + k] = t[k];
  }
}

}  // namespace diso
