// Forward and backward kernels of DiffMC / DiffDMC.
//
//   count_kernel      all tiles: per-segment crossing / face (MC) or crossing / patch
//                     (DMC) counts, the min/max of the SDF for the empty-surface
//                     guard, one activity byte per tile and the list of active tiles
//   scan              scan.cuh
//   mc_emit_kernel    active tiles: MC vertices and triangles
//   dmc_emit_kernel   active tiles: DMC dual vertices and quads
//   backward_kernel   all point tiles: dL/dsdf and dL/ddeform, every element written
//                     once (zeros away from the surface), crossings recomputed
//   split_*           DMC quad -> triangle split (return_quads=False)
//
// Row masks.  Every kernel first turns the SDF rows its tile needs into bit masks:
// a warp reads 32 (+3) consecutive points of a row (X, Y) along z, coalesced, and
// one ballot gives bit k = (value >= iso) of padded point (X, Y, Z0 - 1 + k).
// From the masks of the four rows around a row of 32 cells, the cells' crossing
// edges, which cells are non-trivial, each cell's case code and each cell's
// offset inside its segment all follow from a few 64-bit logic ops and popcounts
// (the warp ballot / popc compaction), so a row segment without surface costs a
// handful of instructions.
#pragma once
#include "common.cuh"

namespace diso {

enum Method { MC = 0, DMC = 1 };

constexpr int MASK_TOP = 34;  // highest valid mask bit: points Z0-1 .. Z0+33

__device__ const uint8_t g_edge_of[24] = DISO_EDGE_LOOKUP;

// ------------------------------------------------------------------ geometry helpers

// lerp vertex of the edge from padded point (X,Y,Z) along axis a, in padded
// coordinates with deform (computeMcVert, src/cumc.cu:343-368)
template <class S>
__device__ __forceinline__ void edge_vertex(const Field<S>& f, int X, int Y, int Z, int a, S out[3]) {
  const int ex = a == 0, ey = a == 1, ez = a == 2;
  const S d0 = f.at(X, Y, Z), d1 = f.at(X + ex, Y + ey, Z + ez);
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

// cells Z0 + j (j < 32) that exist
__device__ __forceinline__ uint32_t zvalid(const Geom& g, int Z0) {
  const int n = g.c[2] - Z0;
  return n >= 32 ? 0xffffffffu : ((1u << n) - 1u);
}

// ------------------------------------------------------------------ row masks

// Fill m[x][y] for point rows (WX0 + x, WY0 + y); bit k = point Z0 - 1 + k >= iso.
// Warp w takes rows w, w + NW, ...; it issues the loads of BATCH rows before their
// ballots, so each warp keeps BATCH row loads in flight.  Tracks min / max of the
// caller's (interior) values when TRACK.  Needs blockDim.x == NTHREADS.
template <class S, int WX, int WY, bool TRACK>
__device__ __forceinline__ void load_masks(uint64_t (&m)[WX][WY], const Field<S>& f, int WX0, int WY0, int Z0,
                                           S& mn, S& mx, bool& seen) {
  constexpr int NW = NTHREADS / 32, NR = WX * WY, BATCH = 8;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int Z = Z0 - 1 + lane, Ze = Z0 + 31 + lane;
  const bool zin = (unsigned)(Z - 1) < (unsigned)f.n2;
  const bool ein = lane < 3 && (unsigned)(Ze - 1) < (unsigned)f.n2;
#pragma unroll 1
  for (int r0 = warp; r0 < NR; r0 += NW * BATCH) {
    S v[BATCH], e[BATCH];
    bool in[BATCH];
#pragma unroll
    for (int k = 0; k < BATCH; ++k) {
      const int r = r0 + k * NW;
      const int x = r / WY, y = r % WY, X = WX0 + x, Y = WY0 + y;
      const bool row = r < NR && (unsigned)(X - 1) < (unsigned)f.n0 && (unsigned)(Y - 1) < (unsigned)f.n1;
      const int64_t base = ((int64_t)(X - 1) * f.n1 + (Y - 1)) * f.n2 - 1;
      in[k] = row && zin;
      v[k] = in[k] ? __ldg(f.sdf + base + Z) : f.pad;
      e[k] = (row && ein) ? __ldg(f.sdf + base + Ze) : f.pad;
    }
#pragma unroll
    for (int k = 0; k < BATCH; ++k) {
      const int r = r0 + k * NW;
      const uint32_t lo = __ballot_sync(0xffffffffu, v[k] >= f.iso);
      const uint32_t hi = __ballot_sync(0xffffffffu, lane < 3 && e[k] >= f.iso);
      if (lane == 0 && r < NR) m[r / WY][r % WY] = (uint64_t)lo | ((uint64_t)(hi & 7u) << 32);
      if (TRACK && in[k]) {
        mn = seen ? (v[k] < mn ? v[k] : mn) : v[k];
        mx = seen ? (v[k] > mx ? v[k] : mx) : v[k];
        seen = true;
      }
    }
  }
}

// Morton code from the four row masks around a cell: a = (x,y), b = (x+1,y),
// c = (x,y+1), d = (x+1,y+1); s = bit of the cell's corner 0
__device__ __forceinline__ int code8(uint64_t a, uint64_t b, uint64_t c, uint64_t d, int s) {
  const uint64_t lo = ((a >> s) & 1) | (((b >> s) & 1) << 1) | (((c >> s) & 1) << 2) | (((d >> s) & 1) << 3);
  const int t = s + 1;
  const uint64_t hi = ((a >> t) & 1) | (((b >> t) & 1) << 1) | (((c >> t) & 1) << 2) | (((d >> t) & 1) << 3);
  return (int)(lo | (hi << 4));
}

// Morton code of cell (X, Y, Z) from the masks when its corners are in the
// window, otherwise from global memory
template <class S, int WX, int WY>
__device__ __forceinline__ int cell_code(const uint64_t (&m)[WX][WY], const Field<S>& f, int WX0, int WY0, int Z0,
                                         int X, int Y, int Z) {
  // rows x and x + 1 must both lie in the window (x is unsigned: a row below the
  // window wraps to a huge value and fails the test)
  const unsigned x = (unsigned)(X - WX0), y = (unsigned)(Y - WY0);
  const int s = Z - Z0 + 1;
  if (x < (unsigned)(WX - 1) && y < (unsigned)(WY - 1) && s >= 0 && s + 1 <= MASK_TOP)
    return code8(m[x][y], m[x + 1][y], m[x][y + 1], m[x + 1][y + 1], s);
  int c = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) c |= (f.at(X + (i & 1), Y + ((i >> 1) & 1), Z + ((i >> 2) & 1)) >= f.iso) << i;
  return c;
}

// DMC code after the face-neighbour ambiguity test (src/cudualmc.cu:815-839):
// a "problematic" code looks at the cell across its ambiguous face; when that
// (raw) code is problematic too, the code is complemented.
template <class S, int WX, int WY>
__device__ __forceinline__ int dmc_resolve_m(const uint64_t (&m)[WX][WY], const Field<S>& f, int WX0, int WY0, int Z0,
                                             int code, int X, int Y, int Z, const Geom& g) {
  const int dir = dmc_dir(dmc_case(code));
  if (dir == 7) return code;
  const int comp = dir >> 1, d = (dir & 1) ? 1 : -1;
  const int NX = X + (comp == 0 ? d : 0), NY = Y + (comp == 1 ? d : 0), NZ = Z + (comp == 2 ? d : 0);
  const int nc = comp == 0 ? NX : (comp == 1 ? NY : NZ);
  if (nc < 0 || nc >= g.c[comp]) return code;
  const int ncode = cell_code<S>(m, f, WX0, WY0, Z0, NX, NY, NZ);
  return dmc_dir(dmc_case(ncode)) != 7 ? (code ^ 0xff) : code;
}

// per row of 32 cells: crossing +x / +y / +z edges owned by each cell and the
// non-trivial cells (case code not 0 or 255), one bit per cell
struct RowBits {
  uint32_t xc, yc, zc, nt;
};

__device__ __forceinline__ RowBits row_bits(uint64_t a, uint64_t b, uint64_t c, uint64_t d, uint32_t valid) {
  const uint64_t a1 = a >> 1, b1 = b >> 1, c1 = c >> 1, d1 = d >> 1;
  const uint64_t a2 = a >> 2, b2 = b >> 2, c2 = c >> 2, d2 = d >> 2;
  const uint64_t o = a1 | b1 | c1 | d1 | a2 | b2 | c2 | d2;
  const uint64_t n = a1 & b1 & c1 & d1 & a2 & b2 & c2 & d2;
  RowBits r;
  r.xc = (uint32_t)(a1 ^ b1) & valid;
  r.yc = (uint32_t)(a1 ^ c1) & valid;
  r.zc = (uint32_t)(a1 ^ a2) & valid;
  r.nt = (uint32_t)(o & ~n) & valid;
  return r;
}

// crossing flags (bit a = edge along axis a) of the cell at mask bit s (a cell past the
// 32 of a row, e.g. the first cell of the next segment)
__device__ __forceinline__ int flags_at(uint64_t a, uint64_t b, uint64_t c, int s) {
  const int p = (int)((a >> s) & 1);
  return (p ^ (int)((b >> s) & 1)) | ((p ^ (int)((c >> s) & 1)) << 1) | ((p ^ (int)((a >> (s + 1)) & 1)) << 2);
}

__device__ __forceinline__ int row_flags(const RowBits& r, int j) {
  return (int)(((r.xc >> j) & 1) | (((r.yc >> j) & 1) << 1) | (((r.zc >> j) & 1) << 2));
}

// crossings owned by cells 0..j-1 of the row
__device__ __forceinline__ int row_prefix(const RowBits& r, int j) {
  const uint32_t lo = (1u << j) - 1u;
  return __popc(r.xc & lo) + __popc(r.yc & lo) + __popc(r.zc & lo);
}

// ------------------------------------------------------------------ count

// The count pass works on blocks of CP planes x CR rows x 32 cells: one warp per
// plane, one lane per row segment.  Each lane derives its segment's crossing count
// from four row masks with popcounts and walks only the segment's non-trivial
// cells for the case-table lookups.  A block covers (CP/TX) x (CR/TY) activity tiles.
//
// Persistent: CTA b handles blocks b, b + gridDim.x, ...; it keeps the min / max and
// the list of its active tiles and publishes them with a few atomics at the end
// (per-tile atomics on one address serialise in L2).  At most COUNT_LIST tiles per
// CTA: launch at least ntiles / COUNT_LIST CTAs.
constexpr int CP = 8, CR = 32;
constexpr int COUNT_LIST = 2048;
static_assert(CP * 32 == NTHREADS && CP % TX == 0 && CR % TY == 0, "count block shape");

__host__ __device__ inline int64_t count_blocks(const Geom& g) {
  return (int64_t)((g.c[0] + CP - 1) / CP) * ((g.c[1] + CR - 1) / CR) * g.nzc;
}

template <class S, int METHOD>
struct CountShared {
  // MC needs the rows of the cells' corners, DMC also those of the face neighbours
  // used by the ambiguity test
  static constexpr int H = METHOD == DMC ? 1 : 0;
  static constexpr int WX = CP + 1 + 2 * H, WY = CR + 1 + 2 * H;
  uint64_t m[WX][WY];
  uint32_t act[CP];
  int list[COUNT_LIST];
  int nlist, base;
};

// lower the grid's min / max keys (one warp's values); reads first so that most
// warps need no atomic
template <class S>
__device__ __forceinline__ void publish_minmax(Stats* stats, S mn, S mx, bool seen) {
  const int lane = threadIdx.x & 31;
  const unsigned have = __ballot_sync(0xffffffffu, seen);
  if (!have) return;
  const int src = __ffs(have) - 1;
  const S m0 = __shfl_sync(0xffffffffu, mn, src), x0 = __shfl_sync(0xffffffffu, mx, src);
  if (!seen) {
    mn = m0;
    mx = x0;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const S p = __shfl_xor_sync(0xffffffffu, mn, o), q = __shfl_xor_sync(0xffffffffu, mx, o);
    mn = p < mn ? p : mn;
    mx = q > mx ? q : mx;
  }
  if (lane == 0) {
    const unsigned long long kmn = ord_key((double)mn), kmx = ord_key((double)mx);
    if (kmn < *(volatile unsigned long long*)&stats->min_key) atomicMin(&stats->min_key, kmn);
    if (kmx > *(volatile unsigned long long*)&stats->max_key) atomicMax(&stats->max_key, kmx);
  }
}

// One count block: the per-segment counts, the activity bytes of the block's
// tiles, the grid's min / max; active tiles are appended (as tile | tag) to sh.list.
template <class S, int METHOD>
__device__ __forceinline__ void count_block(CountShared<S, METHOD>& sh, const Field<S>& f, const Geom& g,
                                            uint64_t* __restrict__ seg, uint8_t* __restrict__ tile_flag,
                                            Stats* stats, int blk, int tag) {
  constexpr int H = CountShared<S, METHOD>::H, WX = CountShared<S, METHOD>::WX, WY = CountShared<S, METHOD>::WY;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nby = (g.c[1] + CR - 1) / CR;
  const int tz = blk % g.nzc;
  const int r = blk / g.nzc;
  const int X0 = (r / nby) * CP, Y0 = (r % nby) * CR, Z0 = tz * TZ;
  const int WX0 = X0 - H, WY0 = Y0 - H;
  S mn = f.pad, mx = f.pad;
  bool seen = false;
  load_masks<S, WX, WY, true>(sh.m, f, WX0, WY0, Z0, mn, mx, seen);
  __syncthreads();
  publish_minmax<S>(stats, mn, mx, seen);
  const int X = X0 + warp, Y = Y0 + lane;
  uint32_t nv = 0, nf = 0;
  if (X < g.c[0] && Y < g.c[1]) {
    const int x = warp + H, y = lane + H;
    const uint64_t a = sh.m[x][y], b = sh.m[x + 1][y], c = sh.m[x][y + 1], d = sh.m[x + 1][y + 1];
    const RowBits rw = row_bits(a, b, c, d, zvalid(g, Z0));
    nv = __popc(rw.xc) + __popc(rw.yc) + __popc(rw.zc);
    uint32_t nt = rw.nt;
    while (nt) {
      const int j = __ffs(nt) - 1;
      nt &= nt - 1;
      const int code = code8(a, b, c, d, j + 1);
      if (METHOD == MC)
        nf += (uint32_t)(mc_tri(mc_from_morton(code)) & 15);
      else
        nf += dmc_npatch(dmc_case(dmc_resolve_m<S>(sh.m, f, WX0, WY0, Z0, code, X, Y, Z0 + j, g)));
    }
    seg[g.seg(X, Y, tz)] = Counts::pack(nv, nf);
  }
  // a cell can emit faces / patches without owning a crossing edge (its
  // crossings may all sit on edges owned by its +1 neighbours)
  const uint32_t busy = __ballot_sync(0xffffffffu, (nv | nf) != 0);
  if (lane == 0) sh.act[warp] = busy;
  __syncthreads();
  if (threadIdx.x < (CP / TX) * (CR / TY)) {
    const int tp = threadIdx.x / (CR / TY), tr = threadIdx.x % (CR / TY);
    const int tx = X0 / TX + tp, ty = Y0 / TY + tr;
    if (tx < g.tiles_x() && ty < g.tiles_y()) {
      uint32_t any = 0;
#pragma unroll
      for (int p = 0; p < TX; ++p) any |= (sh.act[tp * TX + p] >> (tr * TY)) & ((1u << TY) - 1u);
      const int64_t tile = ((int64_t)tx * g.tiles_y() + ty) * g.nzc + tz;
      tile_flag[tile] = any ? 1 : 0;
      if (any) sh.list[atomicAdd(&sh.nlist, 1)] = (int)tile | tag;
    }
  }
}

// append the CTA's active tiles to the global list
template <class S, int METHOD>
__device__ __forceinline__ void count_flush(CountShared<S, METHOD>& sh, unsigned long long* n_active,
                                            int* __restrict__ active) {
  __syncthreads();
  if (threadIdx.x == 0) sh.base = sh.nlist ? (int)atomicAdd(n_active, (unsigned long long)sh.nlist) : 0;
  __syncthreads();
  for (int i = threadIdx.x; i < sh.nlist; i += blockDim.x) active[sh.base + i] = sh.list[i];
}

// Persistent: CTA b handles blocks b, b + gridDim.x, ...; the active tiles of a CTA
// are kept in shared memory and published with one atomic at the end (per-tile
// atomics on one address serialise in L2).  At most COUNT_LIST tiles per CTA:
// launch at least ntiles / COUNT_LIST CTAs.
template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS, 3) count_kernel(Field<S> f, Geom g, uint64_t* __restrict__ seg,
                                                            uint8_t* __restrict__ tile_flag, Stats* stats,
                                                            int* __restrict__ active) {
  __shared__ CountShared<S, METHOD> sh;
  if (threadIdx.x == 0) sh.nlist = 0;
  const int nblocks = (int)count_blocks(g);
#pragma unroll 1
  for (int blk = blockIdx.x; blk < nblocks; blk += gridDim.x) count_block<S, METHOD>(sh, f, g, seg, tile_flag, stats, blk, 0);
  count_flush<S, METHOD>(sh, &stats->n_active, active);
}

// ------------------------------------------------------------------ batches

// One grid of a batch: its field, geometry, its slices of the concatenated
// per-call record (segments and tile bytes), its first flattened count block,
// active-tile and point tile, and its gradient outputs.
template <class S>
struct BatchGrid {
  Field<S> f;
  Geom g;
  uint64_t* seg;        // this grid's first segment in the concatenated, globally scanned array
  uint64_t* seg_end;    // the next grid's first segment (or the total slot)
  uint8_t* tile_flag;   // this grid's tile bytes
  int64_t cblk0;        // first count block of the grid in the flattened queue
  int64_t ptile0;       // first point tile (backward)
  S* gsdf;              // backward outputs
  S* gdef;
};
constexpr int MAX_BATCH = 256;  // grids per batch (the grid index is stored in 8 bits of a tile id)
constexpr int BATCH_TILE_BITS = 24;

// index of the grid whose range [start[i], start[i+1]) holds item b
__device__ __forceinline__ int batch_find(const int64_t* start, int n, int64_t b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// every grid of a batch in one persistent launch over the flattened queue of count
// blocks; per-grid status words in stats[grid]
template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS, 3) batch_count_kernel(const BatchGrid<S>* __restrict__ grids, int ngrids,
                                                                  int64_t nblocks, Stats* stats,
                                                                  unsigned long long* n_active,
                                                                  int* __restrict__ active) {
  __shared__ CountShared<S, METHOD> sh;
  __shared__ int64_t start[MAX_BATCH];
  for (int i = threadIdx.x; i < ngrids; i += blockDim.x) start[i] = grids[i].cblk0;
  if (threadIdx.x == 0) sh.nlist = 0;
  __syncthreads();
#pragma unroll 1
  for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x) {
    const int i = batch_find(start, ngrids, b);
    const BatchGrid<S>& G = grids[i];
    count_block<S, METHOD>(sh, G.f, G.g, G.seg, G.tile_flag, stats + i, (int)(b - start[i]), i << BATCH_TILE_BITS);
  }
  count_flush<S, METHOD>(sh, n_active, active);
}

// ------------------------------------------------------------------ work lists

// Exclusive scan of one value per thread over the block (blockDim.x == NTHREADS).
// Returns the thread's offset; `total` receives the sum.  wsum: NW + 1 words of
// shared memory, free again after the call returns.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* wsum, uint32_t& total) {
  constexpr int NW = NTHREADS / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t inc = warp_incl(v);
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < NW ? wsum[lane] : 0u;
    const uint32_t wi = warp_incl(w);
    if (lane < NW) wsum[lane] = wi - w;
    if (lane == NW - 1) wsum[NW] = wi;
  }
  __syncthreads();
  total = wsum[NW];
  const uint32_t off = wsum[warp] + inc - v;
  __syncthreads();
  return off;
}

// work item of a tile: cell-window coordinates and, for edge items, the axis
__device__ __forceinline__ uint16_t item_code(int x, int y, int j, int a) {
  return (uint16_t)(x | (y << 3) | (j << 7) | (a << 13));
}
__device__ __forceinline__ void item_decode(uint16_t c, int& x, int& y, int& j, int& a) {
  x = c & 7;
  y = (c >> 3) & 15;
  j = (c >> 7) & 63;
  a = c >> 13;
}
static_assert(TX + 1 <= 8 && TY + 1 <= 16 && TZ + 1 <= 64, "item code fields");

// append the set bits of `bits` (bit j -> cell j) as items of cell row (x, y) and axis a
__device__ __forceinline__ void put_items(uint16_t* list, uint32_t off, uint64_t bits, int x, int y, int a) {
  while (bits) {
    const int j = __ffsll((long long)bits) - 1;
    bits &= bits - 1;
    list[off++] = item_code(x, y, j, a);
  }
}

// ------------------------------------------------------------------ MC emit

constexpr int EMIT_ITEMS = 3 * TX * TY * TZ;  // every own edge crossing

// One active tile: its vertices and triangles.  Vertex ids written into faces are
// reduced by vsub (the grid's first vertex, for batches whose vertices are concatenated).
template <class S>
__device__ __forceinline__ void mc_emit_tile(const Field<S>& f, const Geom& g, const uint64_t* __restrict__ seg,
                                             int tile, S* __restrict__ verts, int64_t* __restrict__ faces,
                                             int normalize, int64_t vsub) {
  constexpr int WX = TX + 2, WY = TY + 2;  // point rows [X0, X0+TX+1] x [Y0, Y0+TY+1]
  constexpr int CX = TX + 1, CY = TY + 1;  // cell rows [X0, X0+TX] x [Y0, Y0+TY]
  __shared__ uint64_t m[WX][WY];
  __shared__ RowBits rb[CX][CY];
  __shared__ uint8_t f32[CX][CY];  // flags of cell Z0+32 (first of the next segment)
  __shared__ uint32_t vb[CX][CY][2];
  __shared__ uint32_t fb[TX][TY];
  __shared__ uint8_t fpre[TX][TY][TZ];  // triangles before the cell inside its segment
  __shared__ uint16_t vitems[EMIT_ITEMS];
  __shared__ uint16_t citems[TX * TY * TZ];
  __shared__ uint32_t wsum[NTHREADS / 32 + 1];
  __shared__ uint32_t nvi, nci;
  int X0, Y0, Z0, tz;
  tile_coords(tile, g, X0, Y0, Z0, tz);
  S dmn, dmx;
  bool dseen = false;
  load_masks<S, WX, WY, false>(m, f, X0, Y0, Z0, dmn, dmx, dseen);
  for (int i = threadIdx.x; i < CX * CY * 2; i += blockDim.x) {
    const int k = i & 1, y = (i >> 1) % CY, x = (i >> 1) / CY;
    const int X = X0 + x, Y = Y0 + y, zc = tz + k;
    const uint64_t s = (X < g.c[0] && Y < g.c[1] && zc < g.nzc) ? seg[g.seg(X, Y, zc)] : 0ull;
    vb[x][y][k] = Counts::lo(s);
    if (k == 0 && x < TX && y < TY) fb[x][y] = Counts::hi(s);
  }
  __syncthreads();
  const uint32_t valid = zvalid(g, Z0);
  for (int i = threadIdx.x; i < CX * CY; i += blockDim.x) {
    const int x = i / CY, y = i % CY;
    RowBits r = {0u, 0u, 0u, 0u};
    int fl = 0;
    if (X0 + x < g.c[0] && Y0 + y < g.c[1]) {
      r = row_bits(m[x][y], m[x + 1][y], m[x][y + 1], m[x + 1][y + 1], valid);
      if (Z0 + TZ < g.c[2]) fl = flags_at(m[x][y], m[x + 1][y], m[x][y + 1], TZ + 1);
    }
    rb[x][y] = r;
    f32[x][y] = (uint8_t)fl;
  }
  __syncthreads();
  // one thread per own row: the row's vertex items and cell items, and the
  // triangle prefix of its non-trivial cells
  uint32_t cv = 0, cc = 0;
  RowBits own = {0u, 0u, 0u, 0u};
  const int ox = threadIdx.x / TY, oy = threadIdx.x % TY;
  if (threadIdx.x < TX * TY) {
    own = rb[ox][oy];
    cv = __popc(own.xc) + __popc(own.yc) + __popc(own.zc);
    cc = __popc(own.nt);
    uint32_t nt = own.nt, run = 0;
    while (nt) {
      const int j = __ffs(nt) - 1;
      nt &= nt - 1;
      fpre[ox][oy][j] = (uint8_t)run;
      run += (uint32_t)(mc_tri(mc_from_morton(code8(m[ox][oy], m[ox + 1][oy], m[ox][oy + 1], m[ox + 1][oy + 1], j + 1))) & 15);
    }
  }
  uint32_t tot;
  const uint32_t off = block_excl_scan(cv | (cc << 16), wsum, tot);
  if (threadIdx.x == 0) {
    nvi = tot & 0xffffu;
    nci = tot >> 16;
  }
  if (threadIdx.x < TX * TY) {
    uint32_t o = off & 0xffffu;
    // vertices in (cell, axis) order: interleave the three axes per cell
    uint32_t b = own.xc | own.yc | own.zc;
    while (b) {
      const int j = __ffs(b) - 1;
      b &= b - 1;
      const int fl = row_flags(own, j);
#pragma unroll
      for (int a = 0; a < 3; ++a)
        if (fl & (1 << a)) vitems[o++] = item_code(ox, oy, j, a);
    }
    put_items(citems, off >> 16, own.nt, ox, oy, 0);
  }
  __syncthreads();
  // index of the vertex on the edge along a owned by window cell (x, y, z index j in [0, 32])
  auto vid = [&](int x, int y, int j, int a) -> int64_t {
    if (j == TZ) return (int64_t)vb[x][y][1] + __popc(f32[x][y] & ((1 << a) - 1));
    const RowBits r = rb[x][y];
    return (int64_t)vb[x][y][0] + row_prefix(r, j) + __popc(row_flags(r, j) & ((1 << a) - 1));
  };
  // vertices (src/cumc.cu:370-410)
  for (uint32_t i = threadIdx.x; i < nvi; i += blockDim.x) {
    int x, y, j, a;
    item_decode(vitems[i], x, y, j, a);
    S p[3];
    edge_vertex<S>(f, X0 + x, Y0 + y, Z0 + j, a, p);
    store_vertex<S>(verts, vid(x, y, j, a), p, g, normalize);
  }
  // triangles (src/cumc.cu:564-649): each table edge -> owner cell (+0/+1) -> its vertex
  for (uint32_t i = threadIdx.x; i < nci; i += blockDim.x) {
    int x, y, j, a;
    item_decode(citems[i], x, y, j, a);
    const uint64_t w = mc_tri(mc_from_morton(code8(m[x][y], m[x + 1][y], m[x][y + 1], m[x + 1][y + 1], j + 1)));
    const int nt = (int)(w & 15);
    const int64_t f0 = (int64_t)fb[x][y] + fpre[x][y][j];
    for (int t = 0; t < nt; ++t) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int e = (int)((w >> (4 + 4 * (3 * t + k))) & 15);
        const int ge = g_edge[e];
        faces[3 * (f0 + t) + k] = vid(x + (ge & 1), y + ((ge >> 1) & 1), j + ((ge >> 2) & 1), ge >> 3) - vsub;
      }
    }
  }
  __syncthreads();  // the shared arrays are reused by the CTA's next tile
}

template <class S>
__global__ void __launch_bounds__(NTHREADS) mc_emit_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg,
                                                           const int* __restrict__ active, S* __restrict__ verts,
                                                           int64_t* __restrict__ faces, int normalize) {
  mc_emit_tile<S>(f, g, seg, active[blockIdx.x], verts, faces, normalize, 0);
}

// ------------------------------------------------------------------ DMC emit

// One active tile: its dual vertices and quads; patch ids written into quads are
// reduced by vsub (as in mc_emit_tile).
template <class S>
__device__ __forceinline__ void dmc_emit_tile(const Field<S>& f, const Geom& g, const uint64_t* __restrict__ seg,
                                              int tile, S* __restrict__ verts, int64_t* __restrict__ quads,
                                              int normalize, int64_t vsub) {
  constexpr int WX = TX + 3, WY = TY + 3;  // point rows [X0-1, X0+TX+1] x [Y0-1, Y0+TY+1]
  constexpr int CX = TX + 1, CY = TY + 1;  // cell rows [X0-1, X0+TX) x [Y0-1, Y0+TY) (own + the -1 halo)
  __shared__ uint64_t m[WX][WY];
  __shared__ uint8_t rc[CX][CY][TZ + 1];  // resolved codes; z index j+1 for cell Z0+j, 0 for Z0-1
  __shared__ int16_t pp[CX][CY][TZ + 1];  // first patch of the cell inside its segment
  __shared__ uint32_t pb[CX][CY];
  __shared__ uint32_t qb[TX][TY];
  __shared__ uint16_t qitems[EMIT_ITEMS];
  __shared__ uint16_t citems[TX * TY * TZ];
  __shared__ uint32_t wsum[NTHREADS / 32 + 1];
  __shared__ uint32_t nqi, nci;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int X0, Y0, Z0, tz;
  tile_coords(tile, g, X0, Y0, Z0, tz);
  const int WX0 = X0 - 1, WY0 = Y0 - 1;
  S dmn, dmx;
  bool dseen = false;
  load_masks<S, WX, WY, false>(m, f, WX0, WY0, Z0, dmn, dmx, dseen);
  for (int i = threadIdx.x; i < CX * CY; i += blockDim.x) {
    const int y = i % CY, x = i / CY, X = X0 - 1 + x, Y = Y0 - 1 + y;
    const uint64_t s = (X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1]) ? seg[g.seg(X, Y, tz)] : 0ull;
    pb[x][y] = Counts::hi(s);
    if (x >= 1 && y >= 1) qb[x - 1][y - 1] = Counts::lo(s);
  }
  __syncthreads();
  const uint32_t valid = zvalid(g, Z0);
  // resolved codes and in-segment patch prefixes of the tile's cells and their -1 halo;
  // the mask row of cell (X0-1+x, Y0-1+y) is (x, y)
  for (int r = warp; r < CX * CY; r += TY) {
    const int x = r / CY, y = r % CY, X = X0 - 1 + x, Y = Y0 - 1 + y;
    const bool row = X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1];
    const uint64_t a = m[x][y], b = m[x + 1][y], c = m[x][y + 1], d = m[x + 1][y + 1];
    const uint32_t nt = row ? row_bits(a, b, c, d, valid).nt : 0u;
    int code = 0;
    if ((nt >> lane) & 1) code = dmc_resolve_m<S>(m, f, WX0, WY0, Z0, code8(a, b, c, d, lane + 1), X, Y, Z0 + lane, g);
    const uint32_t np = dmc_npatch(dmc_case(code));
    const uint32_t inc = nt ? warp_incl(np) : 0u;
    rc[x][y][lane + 1] = (uint8_t)code;
    pp[x][y][lane + 1] = (int16_t)(inc - np);
    if (lane == 0) {
      int c0 = 0;
      if (row && Z0 >= 1) {
        c0 = code8(a, b, c, d, 0);
        if (c0 != 0 && c0 != 255) c0 = dmc_resolve_m<S>(m, f, WX0, WY0, Z0, c0, X, Y, Z0 - 1, g);
      }
      rc[x][y][0] = (uint8_t)c0;
      pp[x][y][0] = (int16_t)(-(int)dmc_npatch(dmc_case(c0)));  // last cell of the previous segment
    }
  }
  // work lists of the own rows: crossing edges (quads) and non-trivial cells (dual vertices)
  uint32_t cq = 0, cc = 0;
  RowBits own = {0u, 0u, 0u, 0u};
  const int ox = threadIdx.x / TY, oy = threadIdx.x % TY;
  if (threadIdx.x < TX * TY && X0 + ox < g.c[0] && Y0 + oy < g.c[1]) {
    own = row_bits(m[ox + 1][oy + 1], m[ox + 2][oy + 1], m[ox + 1][oy + 2], m[ox + 2][oy + 2], valid);
    cq = __popc(own.xc) + __popc(own.yc) + __popc(own.zc);
    cc = __popc(own.nt);
  }
  uint32_t tot;
  const uint32_t off = block_excl_scan(cq | (cc << 16), wsum, tot);
  if (threadIdx.x == 0) {
    nqi = tot & 0xffffu;
    nci = tot >> 16;
  }
  if (threadIdx.x < TX * TY) {
    uint32_t o = off & 0xffffu;
    uint32_t b = own.xc | own.yc | own.zc;
    while (b) {
      const int j = __ffs(b) - 1;
      b &= b - 1;
      const int fl = row_flags(own, j);
#pragma unroll
      for (int a = 0; a < 3; ++a)
        if (fl & (1 << a)) qitems[o++] = item_code(ox, oy, j, a);
    }
    put_items(citems, off >> 16, own.nt, ox, oy, 0);
  }
  __syncthreads();
  // quads: one per crossing edge owned by the cell (src/cudualmc.cu:753-794, 1019-1056);
  // the edge exits (value falls through iso) when its start point is >= iso
  for (uint32_t i = threadIdx.x; i < nqi; i += blockDim.x) {
    int ix, iy, j, a;
    item_decode(qitems[i], ix, iy, j, a);
    const int x = ix + 1, y = iy + 1;  // window cell / mask row of the own row
    const RowBits r = row_bits(m[x][y], m[x + 1][y], m[x][y + 1], m[x + 1][y + 1], valid);
    const int64_t qid = (int64_t)qb[ix][iy] + row_prefix(r, j) + __popc(row_flags(r, j) & ((1 << a) - 1));
    const int type = a + 3 * (int)((m[x][y] >> (j + 1)) & 1);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int q = g_dmc_quad[4 * type + k];
      const int nx = x + (q & 3) - 1, ny = y + ((q >> 2) & 3) - 1, nz = j + 1 + ((q >> 4) & 3) - 1;
      quads[4 * qid + k] = (int64_t)pb[nx][ny] + pp[nx][ny][nz] + dmc_patch_of(dmc_case(rc[nx][ny][nz]), q >> 8) - vsub;
    }
  }
  // dual vertices: mean of the patch's edge vertices, edges in ascending id
  // (create_dmc_verts_kernel, src/cudualmc.cu:907-955)
  for (uint32_t i = threadIdx.x; i < nci; i += blockDim.x) {
    int ix, iy, j, a;
    item_decode(citems[i], ix, iy, j, a);
    const int x = ix + 1, y = iy + 1, X = X0 + ix, Y = Y0 + iy, Z = Z0 + j;
    const int code = rc[x][y][j + 1];
    const uint64_t w = dmc_case(code);
    const int np = dmc_npatch(w);
    S acc[4][3];
    int cnt[4] = {0, 0, 0, 0};
#pragma unroll
    for (int p = 0; p < 4; ++p) acc[p][0] = acc[p][1] = acc[p][2] = S(0);
#pragma unroll
    for (int e = 0; e < 12; ++e) {
      const int ge = g_edge[e], s = ge & 7, ax = ge >> 3;
      if ((((code >> s) ^ (code >> (s | (1 << ax)))) & 1) == 0) continue;
      const int p = dmc_patch_of(w, e);
      S v[3];
      edge_vertex<S>(f, X + (s & 1), Y + ((s >> 1) & 1), Z + ((s >> 2) & 1), ax, v);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q == p) {
          acc[q][0] += v[0];
          acc[q][1] += v[1];
          acc[q][2] += v[2];
          cnt[q] += 1;
        }
    }
    const int64_t p0 = (int64_t)pb[x][y] + pp[x][y][j + 1];
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (q < np) {
        const S inv = S(1) / S(cnt[q]);
        const S v[3] = {acc[q][0] * inv, acc[q][1] * inv, acc[q][2] * inv};
        store_vertex<S>(verts, p0 + q, v, g, normalize);
      }
  }
  __syncthreads();  // the shared arrays are reused by the CTA's next tile
}

template <class S>
__global__ void __launch_bounds__(NTHREADS) dmc_emit_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg,
                                                            const int* __restrict__ active, S* __restrict__ verts,
                                                            int64_t* __restrict__ quads, int normalize) {
  dmc_emit_tile<S>(f, g, seg, active[blockIdx.x], verts, quads, normalize, 0);
}

// ------------------------------------------------------------------ backward

// dL/dverts of vertex i in padded coordinates: the chain rule of "- 1" and "/ (dim - 1)"
template <class S>
__device__ __forceinline__ void load_grad(const S* __restrict__ gv, int64_t i, const S scale[3], S out[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = __ldg(gv + 3 * i + k) * scale[k];
}

// adjoint of edge_vertex (adjComputeMcVert, src/cumc.cu:412-453) for the edge from
// padded point A along axis a: c0 = (dL/dsdf, dL/ddeform) at A, c1 at A + e_a
template <class S>
__device__ __forceinline__ void edge_adjoint2(const Field<S>& f, int X, int Y, int Z, int a, const S gvec[3], S c0[4],
                                              S c1[4]) {
  const int ex = a == 0, ey = a == 1, ez = a == 2;
  const S d0 = f.at(X, Y, Z), d1 = f.at(X + ex, Y + ey, Z + ez);
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
  const S w0 = S(1) - t;
  c0[0] = (f.iso - d1) / den * adj_t;
  c1[0] = (d0 - f.iso) / den * adj_t;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    c0[k + 1] = w0 * gvec[k];
    c1[k + 1] = t * gvec[k];
  }
}

// Point tiles: unpadded points [x0, x0+TX) x [y0, y0+TY) x [z0, z0+TZ); in padded
// coordinates the points are (X0+1.., Y0+1.., Z0+1..) with (X0, Y0, Z0) = (x0, y0, z0),
// and the cells [X0, X0+TX] x [Y0, Y0+TY] x [Z0, Z0+TZ] own every edge that touches
// them.  Those cells lie in the forward tiles (x0/TX + {0,1}, y0/TY + {0,1},
// z0/TZ + {0,1}); the point tile is inactive when none of them holds a crossing.
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

__device__ __forceinline__ void ptile_coords(int64_t tile, const Geom& g, int& x0, int& y0, int& z0) {
  const int tz = (int)(tile % g.ptiles_z());
  const int64_t r = tile / g.ptiles_z();
  y0 = (int)(r % g.ptiles_y()) * TY;
  x0 = (int)(r / g.ptiles_y()) * TX;
  z0 = tz * TZ;
}

// rows of cell-window coordinates whose edges along axis a touch the tile's points:
// axis 0: x in [0, TX], y in [1, TY]; axis 1: x in [1, TX], y in [0, TY];
// axis 2: x in [1, TX], y in [1, TY]
constexpr int BW_ROWS0 = (TX + 1) * TY, BW_ROWS1 = TX * (TY + 1), BW_ROWS2 = TX * TY;
constexpr int BW_ROWS = BW_ROWS0 + BW_ROWS1 + BW_ROWS2;
constexpr int BW_ITEMS = BW_ROWS * (TZ + 1);
static_assert(BW_ROWS <= NTHREADS, "one thread per backward item row");

template <class S>
constexpr size_t backward_dyn_smem() {
  return sizeof(S) * 2 * TX * TY * TZ * 4;
}

// dL/dsdf and dL/ddeform of every point of a tile.  Work list: the crossing edges
// touching the tile, per axis.  Each edge's adjoint (adjComputeMcVert,
// src/cumc.cu:412-453 / src/cudualmc.cu:710-751) is computed once and parked in the
// slot of each endpoint inside the tile; each point then adds its (at most six)
// slots in a fixed order, so the result is deterministic.  MC: the gradient
// reaching an edge vertex is dL/dverts of that vertex (adj_create_cell_mc_verts_kernel,
// src/cumc.cu:474-512).  DMC: it is the sum over the four cells around the edge of
// dL/d(dual vertex) / (edges in that patch) (adj_create_dmc_verts_kernel,
// src/cudualmc.cu:957-1005); the reference reads the gradient of the cell's first
// patch for every patch of the cell (adj_verts[first] with first never advanced,
// src/cudualmc.cu:990): exact = 0 reproduces that, exact = 1 uses each patch's own
// gradient (the true derivative).  Replaces the forward re-run, the zero fills and
// the F.pad backward of diso/__init__.py:30-44, 84-98.
template <class S, int METHOD>
__device__ __forceinline__ void backward_tile(const Field<S>& f, const Geom& g, const uint64_t* __restrict__ seg,
                                              const uint8_t* __restrict__ tile_flag, int64_t ptile,
                                              const S* __restrict__ gv, int normalize, int exact,
                                              S* __restrict__ gsdf, S* __restrict__ gdef) {
  constexpr int H = METHOD == DMC ? 1 : 0;  // DMC: one more mask row each side for the ambiguity test
  constexpr int WX = TX + 2 + H, WY = TY + 2 + H;  // point rows [X0-H, X0+TX+1] x [Y0-H, Y0+TY+1]
  constexpr int CX = TX + 1, CY = TY + 1;          // cell rows [X0, X0+TX] x [Y0, Y0+TY]; mask row x + H
  constexpr int RX = METHOD == DMC ? CX : 1, RY = METHOD == DMC ? CY : 1;
  constexpr int NP = TX * TY * TZ;
  __shared__ uint64_t m[WX][WY];
  __shared__ RowBits rb[CX][CY];
  __shared__ uint8_t f32[CX][CY];
  __shared__ uint32_t b0[CX][CY], b1[CX][CY];  // MC vertex / DMC patch bases of chunks zc and zc+1
  __shared__ uint8_t rc[RX][RY][TZ + 1];
  __shared__ uint8_t pre[RX][RY][TZ + 1];
  __shared__ uint16_t items[BW_ITEMS];
  __shared__ uint32_t wsum[NTHREADS / 32 + 1];
  __shared__ uint32_t aoff[4];
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  S* slot = reinterpret_cast<S*>(dyn_smem);  // [2][NP][4]: end 0 / end 1 adjoints of the current axis
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int X0, Y0, Z0;
  ptile_coords(ptile, g, X0, Y0, Z0);
  if (!ptile_active(g, tile_flag, X0, Y0, Z0)) {
    zero_ptile<S>(f, gsdf, gdef, X0, Y0, Z0);
    return;
  }
  const int zc = Z0 / TZ;
  const int WX0 = X0 - H, WY0 = Y0 - H;
  S dmn, dmx;
  bool dseen = false;
  load_masks<S, WX, WY, false>(m, f, WX0, WY0, Z0, dmn, dmx, dseen);
  for (int i = threadIdx.x; i < CX * CY * 2; i += blockDim.x) {
    const int k = i & 1, y = (i >> 1) % CY, x = (i >> 1) / CY;
    const int X = X0 + x, Y = Y0 + y, c = zc + k;
    const uint64_t s = (X < g.c[0] && Y < g.c[1] && c < g.nzc) ? seg[g.seg(X, Y, c)] : 0ull;
    const uint32_t v = METHOD == MC ? Counts::lo(s) : Counts::hi(s);
    if (k) b1[x][y] = v;
    else b0[x][y] = v;
  }
  __syncthreads();
  const uint32_t valid = zvalid(g, Z0);
  for (int i = threadIdx.x; i < CX * CY; i += blockDim.x) {
    const int x = i / CY, y = i % CY;
    RowBits r = {0u, 0u, 0u, 0u};
    int fl = 0;
    if (X0 + x < g.c[0] && Y0 + y < g.c[1]) {
      const uint64_t a = m[x + H][y + H], b = m[x + H + 1][y + H], c = m[x + H][y + H + 1], d = m[x + H + 1][y + H + 1];
      r = row_bits(a, b, c, d, valid);
      if (Z0 + TZ < g.c[2]) fl = flags_at(a, b, c, TZ + 1);
    }
    rb[x][y] = r;
    f32[x][y] = (uint8_t)fl;
  }
  if constexpr (METHOD == DMC) {
    // resolved codes and in-segment patch prefixes of the window cells
    for (int r = warp; r < CX * CY; r += TY) {
      const int x = r / CY, y = r % CY, X = X0 + x, Y = Y0 + y;
      const bool row = X < g.c[0] && Y < g.c[1];
      const uint64_t a = m[x + H][y + H], b = m[x + H + 1][y + H], c = m[x + H][y + H + 1], d = m[x + H + 1][y + H + 1];
      const uint32_t nt = row ? row_bits(a, b, c, d, valid).nt : 0u;
      int code = 0;
      if ((nt >> lane) & 1) code = dmc_resolve_m<S>(m, f, WX0, WY0, Z0, code8(a, b, c, d, lane + 1), X, Y, Z0 + lane, g);
      const uint32_t np = dmc_npatch(dmc_case(code));
      const uint32_t inc = nt ? warp_incl(np) : 0u;
      rc[x][y][lane] = (uint8_t)code;
      pre[x][y][lane] = (uint8_t)(inc - np);
      if (lane == 0) {
        int c32 = 0;
        if (row && Z0 + TZ < g.c[2]) {
          c32 = code8(a, b, c, d, TZ + 1);
          if (c32 != 0 && c32 != 255) c32 = dmc_resolve_m<S>(m, f, WX0, WY0, Z0, c32, X, Y, Z0 + TZ, g);
        }
        rc[x][y][TZ] = (uint8_t)c32;
        pre[x][y][TZ] = 0;  // first cell of the next segment
      }
    }
  }
  __syncthreads();
  // work list: crossing edges touching the tile, grouped by axis
  int ra = -1, rx = 0, ry = 0;
  uint64_t bits = 0;
  {
    const int t = threadIdx.x;
    if (t < BW_ROWS0) {
      ra = 0;
      rx = t / TY;
      ry = 1 + t % TY;
    } else if (t < BW_ROWS0 + BW_ROWS1) {
      ra = 1;
      rx = 1 + (t - BW_ROWS0) / (TY + 1);
      ry = (t - BW_ROWS0) % (TY + 1);
    } else if (t < BW_ROWS) {
      ra = 2;
      rx = 1 + (t - BW_ROWS0 - BW_ROWS1) / TY;
      ry = 1 + (t - BW_ROWS0 - BW_ROWS1) % TY;
    }
    if (ra >= 0) {
      const RowBits r = rb[rx][ry];
      const uint32_t lo = ra == 0 ? r.xc : (ra == 1 ? r.yc : r.zc);
      bits = (uint64_t)lo | ((uint64_t)((f32[rx][ry] >> ra) & 1) << TZ);
      if (ra < 2) bits &= ~1ull;  // x / y edges of cell Z0 touch no point of the tile
    }
  }
  uint32_t tot;
  const uint32_t off = block_excl_scan((uint32_t)__popcll((long long)bits), wsum, tot);
  if (threadIdx.x == 0) {
    aoff[0] = 0;
    aoff[3] = tot;
  }
  if (threadIdx.x == BW_ROWS0) aoff[1] = off;
  if (threadIdx.x == BW_ROWS0 + BW_ROWS1) aoff[2] = off;
  if (ra >= 0) put_items(items, off, bits, rx, ry, ra);
  __syncthreads();

  S scale[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) scale[k] = normalize ? S(1) / S(g.n[k] - 1) : S(1);
  auto crossing = [&](int x, int y, int j, int a) -> int {
    return j == TZ ? (f32[x][y] >> a) & 1 : (row_flags(rb[x][y], j) >> a) & 1;
  };
  S acc[TX][4];
#pragma unroll
  for (int ix = 0; ix < TX; ++ix) acc[ix][0] = acc[ix][1] = acc[ix][2] = acc[ix][3] = S(0);
#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    for (uint32_t i = aoff[a] + threadIdx.x; i < aoff[a + 1]; i += blockDim.x) {
      int x, y, j, ia;
      item_decode(items[i], x, y, j, ia);
      S gvec[3];
      if constexpr (METHOD == MC) {
        const int64_t v = j == TZ ? (int64_t)b1[x][y] + __popc(f32[x][y] & ((1 << a) - 1))
                                  : (int64_t)b0[x][y] + row_prefix(rb[x][y], j) +
                                        __popc(row_flags(rb[x][y], j) & ((1 << a) - 1));
        load_grad<S>(gv, v, scale, gvec);
      } else {
        gvec[0] = gvec[1] = gvec[2] = S(0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int db = k & 1, dc = k >> 1;
          // the cell one step back along the two other axes (b, c) = (a+1, a+2) mod 3
          const int cx = x - (a == 1 ? dc : (a == 2 ? db : 0));
          const int cy = y - (a == 0 ? db : (a == 2 ? dc : 0));
          const int cz = j - (a == 0 ? dc : (a == 1 ? db : 0));
          const int start = (x - cx) | ((y - cy) << 1) | ((j - cz) << 2);
          const uint64_t w = dmc_case(rc[cx][cy][cz]);
          const int p = dmc_patch_of(w, g_edge_of[3 * start + a]);
          const S inv = S(1) / S(dmc_patch_size(w, p));
          const int64_t pid = (int64_t)(cz == TZ ? b1[cx][cy] : b0[cx][cy]) + pre[cx][cy][cz] + (exact ? p : 0);
          S v[3];
          load_grad<S>(gv, pid, scale, v);
          gvec[0] += v[0] * inv;
          gvec[1] += v[1] * inv;
          gvec[2] += v[2] * inv;
        }
      }
      S c0[4], c1[4];
      edge_adjoint2<S>(f, X0 + x, Y0 + y, Z0 + j, a, gvec, c0, c1);
      if (x >= 1 && y >= 1 && j >= 1) {
        S* s0 = slot + 4 * (((x - 1) * TY + (y - 1)) * TZ + (j - 1));
#pragma unroll
        for (int k = 0; k < 4; ++k) s0[k] = c0[k];
      }
      const int x1 = x + (a == 0), y1 = y + (a == 1), j1 = j + (a == 2);
      if (x1 <= TX && y1 <= TY && j1 <= TZ) {
        S* s1 = slot + 4 * (NP + ((x1 - 1) * TY + (y1 - 1)) * TZ + (j1 - 1));
#pragma unroll
        for (int k = 0; k < 4; ++k) s1[k] = c1[k];
      }
    }
    __syncthreads();
#pragma unroll
    for (int ix = 0; ix < TX; ++ix) {
      const int x = ix + 1, y = warp + 1, j = lane + 1;
      const int p = (ix * TY + warp) * TZ + lane;
      if (crossing(x, y, j, a)) {
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[ix][k] += slot[4 * p + k];
      }
      if (crossing(x - (a == 0), y - (a == 1), j - (a == 2), a)) {
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[ix][k] += slot[4 * (NP + p) + k];
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int ix = 0; ix < TX; ++ix) {
    const int X = X0 + 1 + ix, Y = Y0 + 1 + warp, Z = Z0 + 1 + lane;
    if (!f.inside(X, Y, Z)) continue;
    const int64_t i = f.lin(X, Y, Z);
    gsdf[i] = acc[ix][0];
    if (gdef) {
      gdef[3 * i + 0] = acc[ix][1];
      gdef[3 * i + 1] = acc[ix][2];
      gdef[3 * i + 2] = acc[ix][3];
    }
  }
  __syncthreads();  // the shared arrays are reused by the CTA's next tile
}

template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS) backward_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg,
                                                            const uint8_t* __restrict__ tile_flag,
                                                            const S* __restrict__ gv, int normalize, int exact,
                                                            S* __restrict__ gsdf, S* __restrict__ gdef) {
  backward_tile<S, METHOD>(f, g, seg, tile_flag, blockIdx.x, gv, normalize, exact, gsdf, gdef);
}

// ------------------------------------------------------------------ batch emit / backward

// Emit every active tile of a batch (persistent).  Outputs are concatenated in grid
// order; faces hold grid-local vertex ids.  When a grid's outputs would pass the
// capacities (vcap vertices, fcap faces) the grid is skipped and bit 1 of
// stats[0].error is set; the host then retries with larger buffers.
template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS) batch_emit_kernel(const BatchGrid<S>* __restrict__ grids,
                                                              const int* __restrict__ active,
                                                              const unsigned long long* __restrict__ n_active,
                                                              S* __restrict__ verts, int64_t* __restrict__ faces,
                                                              int64_t vcap, int64_t fcap, int normalize,
                                                              Stats* stats) {
  const int64_t n = (int64_t)*n_active;
#pragma unroll 1
  for (int64_t t = blockIdx.x; t < n; t += gridDim.x) {
    const int code = active[t];
    const int i = (int)((unsigned)code >> BATCH_TILE_BITS), tile = code & ((1 << BATCH_TILE_BITS) - 1);
    const BatchGrid<S>& G = grids[i];
    const uint64_t b0 = *G.seg, b1 = *G.seg_end;
    // MC: low half = vertices, high half = triangles; DMC: low = quads, high = patches
    const int64_t v0 = METHOD == MC ? Counts::lo(b0) : Counts::hi(b0);
    const int64_t v1 = METHOD == MC ? Counts::lo(b1) : Counts::hi(b1);
    const int64_t f1 = METHOD == MC ? Counts::hi(b1) : Counts::lo(b1);
    if (v1 > vcap || f1 > fcap) {
      if (threadIdx.x == 0) atomicOr(&stats->error, 2ull);
      continue;
    }
    if (METHOD == MC)
      mc_emit_tile<S>(G.f, G.g, G.seg, tile, verts, faces, normalize, v0);
    else
      dmc_emit_tile<S>(G.f, G.g, G.seg, tile, verts, faces, normalize, v0);
  }
}

// dL/dsdf and dL/ddeform of every grid of a batch (persistent over the flattened
// point tiles); dL/dverts is the concatenated [total vertices, 3] array.
template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS) batch_backward_kernel(const BatchGrid<S>* __restrict__ grids, int ngrids,
                                                                  int64_t ntiles, const S* __restrict__ gv,
                                                                  int normalize, int exact) {
  __shared__ int64_t start[MAX_BATCH];
  for (int i = threadIdx.x; i < ngrids; i += blockDim.x) start[i] = grids[i].ptile0;
  __syncthreads();
#pragma unroll 1
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int i = batch_find(start, ngrids, t);
    const BatchGrid<S>& G = grids[i];
    backward_tile<S, METHOD>(G.f, G.g, G.seg, G.tile_flag, t - start[i], gv, normalize, exact, G.gsdf, G.gdef);
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
