// Forward and backward kernels of DiffMC / DiffDMC.
//
//   count_kernel /    all tiles: per-segment crossing / face (MC) or crossing / patch
//   count_tma_kernel  (DMC) counts, the min/max of the SDF for the empty-surface
//                     guard, two activity bytes per tile, the list of active tiles,
//                     the DMC cell records, and a share of the gradient zeros
//   scan              scan.cuh (and the forward's reset kernel)
//   mc_emit_kernel    active tiles: MC vertices and triangles (and the edge record)
//   dmc_emit_kernel   active tiles: DMC dual vertices and quads (and the edge record),
//                     the rest of the gradient zeros
//   edge_adjoint_kernel  backward, every crossing edge: its adjoint at both ends
//   active_ptiles_kernel backward: the list of point tiles near the surface
//   gather_list_kernel   backward, those point tiles: dL/dsdf and dL/ddeform as sums
//                        of edge adjoints (the rest of the gradients are the zeros
//                        of the forward, or zero_tiles_kernel's)
//   iso_grad_*        dL/d(isovalue) from dL/dsdf (optional)
//   split_*           DMC quad -> triangle split (return_quads=False)
//   batch_*           the same phases over a batch of grids
// Mesh consumers (normals, weld, OBJ, PLY) are in mesh.cuh.
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
#include "tma.cuh"

namespace diso {

enum Method { MC = 0, DMC = 1 };

constexpr int MASK_TOP = 34;  // highest valid mask bit: points Z0-1 .. Z0+33

// Cell record kept by the count for the DMC emit (2 bytes per cell, in an array of
// the grid's cells with rows padded to whole chunks): bits 0-7 the Morton code after
// the ambiguity test, bit 8 the raw bit of corner 0 (value >= iso), bits 9-15 the
// patches of the segment's earlier cells.  A segment's records are valid when its
// count is not zero (0 for its trivial cells).
typedef uint16_t CellRec;

__device__ const uint8_t g_edge_of[24] = DISO_EDGE_LOOKUP;

// ------------------------------------------------------------------ small tables

__device__ const float g_recip_f[16] = {0.f,      1.f / 1,  1.f / 2,  1.f / 3,  1.f / 4,  1.f / 5,
                                        1.f / 6,  1.f / 7,  1.f / 8,  1.f / 9,  1.f / 10, 1.f / 11,
                                        1.f / 12, 1.f / 13, 1.f / 14, 1.f / 15};
__device__ const double g_recip_d[16] = {0.,      1. / 1,  1. / 2,  1. / 3,  1. / 4,  1. / 5,  1. / 6,  1. / 7,
                                         1. / 8,  1. / 9,  1. / 10, 1. / 11, 1. / 12, 1. / 13, 1. / 14, 1. / 15};
// 1 / n, correctly rounded (what S(1) / S(n) gives)
template <class S>
__device__ __forceinline__ S recip(int n);
template <>
__device__ __forceinline__ float recip<float>(int n) { return __ldg(g_recip_f + n); }
template <>
__device__ __forceinline__ double recip<double>(int n) { return __ldg(g_recip_d + n); }

// Per DMC case code, the crossing edges of each patch: bits 12p + e = edge e (the
// reference's edge order) crosses and belongs to patch p.  Derived from the case table
// at compile time.
namespace detail {
constexpr uint64_t kDmcCaseTable[256] = DISO_DMC_CASES;
struct PatchMasks {
  uint64_t m[256];
};
constexpr PatchMasks make_patch_masks() {
  PatchMasks t{};
  for (int code = 0; code < 256; ++code) {
    uint64_t out = 0;
    for (int e = 0; e < 12; ++e) {
      const int ge = kEdgeTable[e], s = ge & 7, end = s | (1 << (ge >> 3));
      if (((code >> s) ^ (code >> end)) & 1)
        out |= 1ull << (12 * (int)((kDmcCaseTable[code] >> (2 * e)) & 3) + e);
    }
    t.m[code] = out;
  }
  return t;
}
}  // namespace detail
__device__ const detail::PatchMasks g_dmc_pmask = detail::make_patch_masks();

// ------------------------------------------------------------------ geometry helpers

// lerp vertex of the edge from padded point (X,Y,Z) along axis a, in padded
// coordinates with deform (computeMcVert, src/cumc.cu:343-368)
template <class S, class F = Field<S>>
__device__ __forceinline__ void edge_vertex(const F& f, int X, int Y, int Z, int a, S out[3]) {
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

// edge_vertex for an edge whose two points lie inside the caller's grid: no pad
// tests, one index for both points
template <class S>
__device__ __forceinline__ void edge_vertex_in(const Field<S>& f, int X, int Y, int Z, int a, S out[3]) {
  const int ex = a == 0, ey = a == 1, ez = a == 2;
  const int64_t i0 = f.lin(X, Y, Z);
  const int64_t i1 = i0 + (a == 0 ? (int64_t)f.n1 * f.n2 : (a == 1 ? (int64_t)f.n2 : (int64_t)1));
  const S d0 = __ldg(f.sdf + i0), d1 = __ldg(f.sdf + i1);
  S t = S(0.5);
  if (d1 != d0) {
    S r = (f.iso - d0) / (d1 - d0);
    r = S(0) > r ? S(0) : r;
    t = r < S(1) ? r : S(1);
  }
  S q0[3] = {S(0), S(0), S(0)}, q1[3] = {S(0), S(0), S(0)};
  if (f.def) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      q0[k] = __ldg(f.def + 3 * i0 + k);
      q1[k] = __ldg(f.def + 3 * i1 + k);
    }
  }
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

// ------------------------------------------------------------------ edge record

// Per-call edge record, written by the forward emit when gradients will be wanted
// and read by the backward.  E = crossing edges (the MC vertices / the DMC quads, in
// output order), V = vertices.  Layout in 8-byte slots, ordered so that adj and ids
// are 32- and 16-byte aligned when the record is 32-byte aligned:
//   adj [E][8] S      the backward's per-edge adjoints: (dL/dsdf, dL/ddeform) at the
//                     edge's first point, then at its second point
//   ids [E][4] int32  DMC: the patch (grid-local vertex id) of each of the four cells
//                     around the edge, the cell one step back by db along axis a+1
//                     and dc along axis a+2 (mod 3) at index db + 2 dc
//   loc [E] int64     the edge's owner cell (X, Y, Z) and axis, packed by pack_loc
//   aux [V] uint8     DMC: edges of the vertex's patch | index of the patch in its cell << 4
template <class S>
struct EdgeRecord {
  S* adj;
  int64_t* loc;
  int32_t* ids;
  uint8_t* aux;
};

__host__ __device__ inline int64_t edge_record_slots(int method, int dsize, int64_t V, int64_t E) {
  return E * dsize + E + (method == 1 ? 2 * E + (V + 7) / 8 : 0);
}

template <class S>
__host__ __device__ inline EdgeRecord<S> edge_record(void* base, int method, int64_t V, int64_t E) {
  EdgeRecord<S> r;
  int64_t* p = (int64_t*)base;
  r.adj = (S*)p;
  p += E * (int64_t)sizeof(S);
  r.ids = method == 1 ? (int32_t*)p : nullptr;
  if (method == 1) p += 2 * E;
  r.loc = p;
  p += E;
  r.aux = method == 1 ? (uint8_t*)p : nullptr;
  (void)V;
  return r;
}

// cells per axis are below 2^21 (x, y) and 2^20 (z)
constexpr int LOC_MAX_XY = 1 << 21, LOC_MAX_Z = 1 << 20;
__device__ __forceinline__ int64_t pack_loc(int X, int Y, int Z, int a) {
  return ((int64_t)X << 43) | ((int64_t)Y << 22) | ((int64_t)Z << 2) | (int64_t)a;
}
__device__ __forceinline__ void unpack_loc(int64_t l, int& X, int& Y, int& Z, int& a) {
  X = (int)(l >> 43);
  Y = (int)((l >> 22) & (LOC_MAX_XY - 1));
  Z = (int)((l >> 2) & (LOC_MAX_Z - 1));
  a = (int)(l & 3);
}

// ------------------------------------------------------------------ row masks

// Fill m[x][y] for point rows (WX0 + x, WY0 + y); bit k = point Z0 - 1 + k >= iso.
// Warp w takes rows w, w + NW, ...; it issues the loads of BATCH rows before their
// ballots, so each warp keeps BATCH row loads in flight.  Tracks min / max of the
// caller's (interior) values when TRACK.  Needs blockDim.x == NTHREADS.
template <class S, int WX, int WY, bool TRACK, class F = Field<S>, int BATCH = 8>
__device__ __forceinline__ void load_masks(uint64_t (&m)[WX][WY], const F& f, int WX0, int WY0, int Z0, S& mn,
                                           S& mx, bool& seen) {
  constexpr int NW = NTHREADS / 32, NR = WX * WY;
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
      const int64_t off = ((int64_t)(X - 1) * f.n1 + (Y - 1)) * f.n2;
      in[k] = row && zin;
      v[k] = in[k] ? f.point(off, X - 1, Y - 1, Z - 1) : f.pad;
      e[k] = (row && ein) ? f.point(off, X - 1, Y - 1, Ze - 1) : f.pad;
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

// position of the n-th (from 0) set bit of v, n < popc(v)
__device__ __forceinline__ int nth_bit(uint32_t v, int n) {
  int pos = 0;
#pragma unroll
  for (int w = 16; w; w >>= 1) {
    const int c = __popc(v & ((1u << w) - 1u));  // set bits among the low w
    if (n >= c) {
      n -= c;
      v >>= w;
      pos += w;
    }
  }
  return pos;
}

// The four masks of a cell row (a, b, c, d as for code8) as eight shifted copies, so
// that the Morton code of cell j of the row (mask bits j+1 and j+2) takes one funnel
// shift and one logic op per code bit: copy k holds mask (k & 3) shifted so that
// the bit code8 reads for code bit k sits at bit j + k.
struct CodeRow {
  uint32_t lo[8], hi[8];
};
__device__ __forceinline__ CodeRow code_row(uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
  const uint64_t m[4] = {a, b, c, d};
  CodeRow r;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const uint64_t p = (k < 4 ? (m[k] << k) : (m[k - 4] << (k - 1))) >> 1;
    r.lo[k] = (uint32_t)p;
    r.hi[k] = (uint32_t)(p >> 32);
  }
  return r;
}
// Morton code of cell j in [0, 32) of the row: code8(a, b, c, d, j + 1)
__device__ __forceinline__ int code_at(const CodeRow& r, int j) {
  uint32_t c = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) c |= __funnelshift_r(r.lo[k], r.hi[k], j) & (1u << k);
  return (int)c;
}

// Morton code of cell (X, Y, Z) from global memory
template <class S, class F = Field<S>>
__device__ __forceinline__ int cell_code_far(const F& f, int X, int Y, int Z) {
  int c = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) c |= (f.at(X + (i & 1), Y + ((i >> 1) & 1), Z + ((i >> 2) & 1)) >= f.iso) << i;
  return c;
}

// Morton code of cell (X, Y, Z) from the masks when its corners are in the
// window, otherwise from global memory
template <class S, int WX, int WY, class F = Field<S>>
__device__ __forceinline__ int cell_code(const uint64_t (&m)[WX][WY], const F& f, int WX0, int WY0, int Z0,
                                         int X, int Y, int Z) {
  // rows x and x + 1 must both lie in the window (x is unsigned: a row below the
  // window wraps to a huge value and fails the test)
  const unsigned x = (unsigned)(X - WX0), y = (unsigned)(Y - WY0);
  const int s = Z - Z0 + 1;
  if (x < (unsigned)(WX - 1) && y < (unsigned)(WY - 1) && s >= 0 && s + 1 <= MASK_TOP)
    return code8(m[x][y], m[x + 1][y], m[x][y + 1], m[x + 1][y + 1], s);
  return cell_code_far<S>(f, X, Y, Z);
}

// DMC code after the face-neighbour ambiguity test (src/cudualmc.cu:815-839):
// a "problematic" code looks at the cell across its ambiguous face; when that
// (raw) code is problematic too, the code is complemented.
template <class S, int WX, int WY, class F = Field<S>>
__device__ __forceinline__ int dmc_resolve_m(const uint64_t (&m)[WX][WY], const F& f, int WX0, int WY0, int Z0,
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

// The count pass works on units of CP planes x CR rows of cells and KZ chunks of 32
// cells along z, walked in z order: one warp per plane, one lane per row segment.
// For every chunk, each point row of the unit ((CP+1) x (CR+1) rows) is read once,
// 32 points by one coalesced load, and turned into one ballot; a row's 35-bit mask
// is spliced from the ballots of three consecutive chunks (two bits of the chunk
// below, all of the chunk, one bit of the chunk above), so every point is read once
// per unit and the per-row cost is a load, a compare, a ballot and a store.  Each
// lane derives its segment's crossing count from four row masks with popcounts; the
// case-table lookups visit only non-trivial cells (MC: the lane's own; DMC: the
// warp's, dealt out over its lanes, since the ambiguity test is the longer chain and
// reads a neighbour outside the unit's rows from global memory).
//
// Persistent: CTA b handles units b, b + gridDim.x, ... (the TMA count takes them
// from a grid-wide counter); it keeps the list of its active tiles and publishes it
// with one atomic at the end (per-tile atomics on one address serialise in L2).  The
// launches size grids for at most COUNT_LIST tiles per CTA; tiles past that (a CTA
// that took more units than its share, on grids where nearly every tile is active)
// go to the global list with an atomic each.
constexpr int CROWS = (CP + 1) * (CR + 1);  // point rows of a unit
constexpr int CRPW = (CROWS + 7) / 8;       // point rows per warp
constexpr int COUNT_LIST = 2048;
constexpr int COUNT_TILES_PER_UNIT = (CP / TX) * (CR / TY) * KZ;
static_assert(CP * 32 == NTHREADS && CP % TX == 0 && CR % TY == 0 && CRPW <= 64, "count unit shape");

__host__ __device__ inline int64_t count_units(const Geom& g) {
  return (int64_t)((g.c[0] + CP - 1) / CP) * ((g.c[1] + CR - 1) / CR) * ((g.nzc + KZ - 1) / KZ);
}

template <class S, int METHOD>
struct CountShared {
  uint64_t m[CP + 1][CR + 1];  // masks of the current chunk, point row r = x * (CR + 1) + y
  int64_t rowoff[CROWS];       // offset of point row r in the SDF, -1 outside the grid
  uint32_t bal[CROWS];         // ballots of the chunk just read (each row read and used by one warp)
  uint32_t act[CP], actc[CP], actf[CP];
  uint32_t mixed[3];                       // per chunk (rotating): OR of count_combine's bits
  __align__(16) CellRec code[CP][32][TZ];  // cell records of each lane's segment (staging)
  uint32_t pfirst[CP][32];                  // DMC: the warp's patches before each segment's first (count_chunk)
  int list[COUNT_LIST];
  int nlist, base;
  unsigned long long tot[2];  // the CTA's counts (both halves) in 64 bits, for Stats::sum_lo / sum_hi
  int rec_slot;               // a narrow band's unit being counted: its block of cell records
  // the global list and its counter: tiles past COUNT_LIST go there directly (a CTA
  // that takes units from a grid-wide counter may meet more active tiles than its share)
  int* spill;
  unsigned long long* spill_n;
};

// the CTA's 64-bit count sums into the status words (after count_flush)
template <class S, int METHOD>
__device__ __forceinline__ void count_totals(CountShared<S, METHOD>& sh, Stats* stats) {
  if (threadIdx.x == 0) {
    if (sh.tot[0]) atomicAdd(&stats->sum_lo, sh.tot[0]);
    if (sh.tot[1]) atomicAdd(&stats->sum_hi, sh.tot[1]);
  }
}

__device__ __forceinline__ float smin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float smax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double smin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ double smax(double a, double b) { return fmax(a, b); }

// lower the grid's min / max keys by one warp's values (+inf / -inf: none seen);
// reads first so that most warps need no atomic
template <class S>
__device__ __forceinline__ void publish_minmax(Stats* stats, S mn, S mx) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    mn = smin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = smax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if (lane == 0 && mn <= mx) {
    const unsigned long long kmn = ord_key((double)mn), kmx = ord_key((double)mx);
    if (kmn < *(volatile unsigned long long*)&stats->min_key) atomicMin(&stats->min_key, kmn);
    if (kmx > *(volatile unsigned long long*)&stats->max_key) atomicMax(&stats->max_key, kmx);
  }
}

// ballots of chunk t (unpadded z in [32t, 32t + 32)) of the warp's point rows into
// sh.bal; min / max of the values read.  Only the lanes in `lanes` read (the chunks
// below and above a unit contribute two bits and one bit to its masks).
template <class S, int METHOD, class F = Field<S>>
__device__ __forceinline__ void count_ballots(CountShared<S, METHOD>& sh, const F& f, int t, uint32_t lanes, S& mn,
                                              S& mx, int X0, int Y0) {
  constexpr int NB = 4, HALF = (CRPW + NB - 1) / NB;  // NB batches of HALF row loads in flight
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int z = 32 * t + lane;
  const bool zin = (unsigned)z < (unsigned)f.n2 && ((lanes >> lane) & 1u);
  if constexpr (!F::kDense) {
    // an evaluated field: a chunk that is wholly on one side of iso is not evaluated;
    // its rows' ballots are uniform, and its bound (a value on that side of iso)
    // stands in for its min and max: the guard's tests (min >= iso, max <= iso) only
    // need to know on which sides the values lie
    const int l0 = __ffs(lanes) - 1, l1 = 31 - __clz(lanes);
    const int xa = max(X0 - 1, 0), xb = min(X0 + CP - 1, f.n0 - 1);
    const int ya = max(Y0 - 1, 0), yb = min(Y0 + CR - 1, f.n1 - 1);
    const int za = max(32 * t + l0, 0), zb = min(32 * t + l1, f.n2 - 1);
    const bool pads = X0 - 1 < 0 || X0 + CP - 1 >= f.n0 || Y0 - 1 < 0 || Y0 + CR - 1 >= f.n1 || 32 * t + l0 < 0 ||
                      32 * t + l1 >= f.n2;
    S bound = S(0);
    uint64_t cand = 0;
    bool all = true;
    const int cls = f.classify_warp(xa, xb, ya, yb, za, zb, pads, bound, cand, all);
    if (cls >= 0) {
      const uint32_t b = cls ? 0xffffffffu : 0u;
#pragma unroll
      for (int i = 0; i < CRPW; ++i) {
        const int r = warp + 8 * i;
        if (r < CROWS && lane == 0) sh.bal[r] = b;
      }
      if (xa <= xb && ya <= yb && za <= zb) {
        mn = smin(mn, bound);
        mx = smax(mx, bound);
      }
      __syncwarp();
      return;
    }
    if constexpr (F::kGrad == 1) {
      // a union of spheres, evaluated one row at a time (compute, not loads, is what
      // takes the time)
#pragma unroll 1
      for (int i = 0; i < CRPW; ++i) {
        const int r = warp + 8 * i;
        if (r >= CROWS) break;
        const bool in = zin && sh.rowoff[r] >= 0;
        const S v = in ? f.value_of(X0 + r / (CR + 1) - 1, Y0 + r % (CR + 1) - 1, z, cand, all) : f.pad;
        const uint32_t b = __ballot_sync(0xffffffffu, v >= f.iso);
        if (lane == 0) sh.bal[r] = b;
        if (in) {
          mn = smin(mn, v);
          mx = smax(mx, v);
        }
      }
      __syncwarp();
      return;
    }
  }
  if constexpr (F::kGrad != 1) {
    // a grid in memory, or a narrow band's chunk that holds bricks: loads in batches
#pragma unroll
    for (int h = 0; h < NB; ++h) {
      S v[HALF];
      bool in[HALF];
#pragma unroll
      for (int k = 0; k < HALF; ++k) {
        const int r = warp + 8 * (h * HALF + k);
        const int64_t off = r < CROWS ? sh.rowoff[r] : -1;
        in[k] = zin && off >= 0;
        v[k] = in[k] ? f.point(off, X0 + r / (CR + 1) - 1, Y0 + r % (CR + 1) - 1, z) : f.pad;
      }
#pragma unroll
      for (int k = 0; k < HALF; ++k) {
        const int r = warp + 8 * (h * HALF + k);
        if (h * HALF + k < CRPW && r < CROWS) {
          const uint32_t b = __ballot_sync(0xffffffffu, v[k] >= f.iso);
          if (lane == 0) sh.bal[r] = b;
        }
        if (in[k]) {
          mn = smin(mn, v[k]);
          mx = smax(mx, v[k]);
        }
      }
    }
    __syncwarp();
  }
}

// Counts of the unit's chunk tz from the masks in sh.m (complete: the caller
// synchronised), the activity bytes of the chunk's tiles; active tiles are appended
// (as tile | tag) to sh.list; the cell records of busy segments (DMC, when `codes` is
// given).  Ends with a block barrier.
//
// Two bytes per tile: tile_flag[tile] = 1 when the tile's cells have crossings or
// faces (the emit's tiles); tile_flag[ntiles + tile] bit (dx | dy << 1 | dz << 2) =
// the tile's cells own a crossing edge, among them only the first x plane when dx,
// the first y row when dy, the first z cell when dz: the cells of this tile whose
// edges can touch the point tile one step back by (dx, dy, dz) (the backward's
// activity test).
template <class S, int METHOD, class F = Field<S>>
__device__ __forceinline__ void count_chunk(CountShared<S, METHOD>& sh, const F& f, const Geom& g,
                                            uint64_t* __restrict__ seg, uint8_t* __restrict__ tile_flag,
                                            CellRec* __restrict__ codes, int X0, int Y0, int tz, int tag) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int Z0 = tz * TZ;
  const int X = X0 + warp, Y = Y0 + lane;
  uint32_t nv = 0, nf = 0, own = 0, nt = 0;
  uint4* stage = reinterpret_cast<uint4*>(sh.code[warp][lane]);
  if (codes) stage[0] = stage[1] = stage[2] = stage[3] = make_uint4(0u, 0u, 0u, 0u);
  const bool row = X < g.c[0] && Y < g.c[1];
  if (row) {
    const int x = warp, y = lane;
    const uint64_t a = sh.m[x][y], b = sh.m[x + 1][y], c = sh.m[x][y + 1], d = sh.m[x + 1][y + 1];
    const RowBits rw = row_bits(a, b, c, d, zvalid(g, Z0));
    own = rw.xc | rw.yc | rw.zc;
    nt = rw.nt;
    nv = __popc(rw.xc) + __popc(rw.yc) + __popc(rw.zc);
    if constexpr (METHOD == MC) {
      uint32_t left = nt;
      const CodeRow cr = code_row(a, b, c, d);
      while (left) {
        const int j = __ffs(left) - 1;
        left &= left - 1;
        nf += (uint32_t)(mc_tri(mc_from_morton(code_at(cr, j))) & 15);
      }
    }
  }
  if constexpr (METHOD == DMC) {
    // The warp's non-trivial cells (segment-major, z order inside a segment) are dealt
    // out to its lanes, item k to lane k mod 32: a surface along z leaves most of a
    // warp's cells in a few segments, and each cell's ambiguity test is a chain of
    // dependent lookups.  An item's patches-before-it in its segment is a scan over
    // the items since the segment's first (pfirst).
    const uint32_t cnt = __popc(nt);
    const uint32_t base = warp_incl(cnt) - cnt;  // the lane's first item
    const uint32_t total = __shfl_sync(0xffffffffu, base + cnt, 31);
    if (codes) __syncwarp();  // the staging rows are zeroed before other lanes fill them
    uint32_t carry = 0;       // patches of the rounds before
#pragma unroll 1
    for (uint32_t k0 = 0; k0 < total; k0 += 32) {
      const uint32_t k = k0 + lane;
      // the owner: the last lane whose first item is at or before k
      int s = 0;
#pragma unroll
      for (int step = 16; step; step >>= 1) {
        const int t = s + step;
        if (__shfl_sync(0xffffffffu, base, t) <= k) s = t;
      }
      const uint32_t snt = __shfl_sync(0xffffffffu, nt, s), sbase = __shfl_sync(0xffffffffu, base, s);
      const bool has = k < total;
      int code = 0, rcode = 0, j = 0;
      uint32_t np = 0;
      if (has) {
        j = nth_bit(snt, (int)(k - sbase));
        code = code8(sh.m[warp][s], sh.m[warp + 1][s], sh.m[warp][s + 1], sh.m[warp + 1][s + 1], j + 1);
        rcode = dmc_resolve_m<S>(sh.m, f, X0, Y0, Z0, code, X0 + warp, Y0 + s, Z0 + j, g);
        np = (uint32_t)dmc_npatch(dmc_case(rcode));
      }
      const uint32_t incl = warp_incl(np);
      const uint32_t before = carry + incl - np;  // the warp's patches before item k
      if (has && k == sbase) sh.pfirst[warp][s] = before;
      __syncwarp();
      if (has && codes)
        sh.code[warp][s][j] = (CellRec)(rcode | ((code & 1) << 8) | ((before - sh.pfirst[warp][s]) << 9));
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    __syncwarp();  // pfirst and the staged records are complete
    // the lane's patches: up to the next segment with items (or the warp's end)
    const uint32_t later = __ballot_sync(0xffffffffu, cnt != 0) & ~((2u << lane) - 1u);
    if (cnt) nf = (later ? sh.pfirst[warp][__ffs(later) - 1] : carry) - sh.pfirst[warp][lane];
  }
  if (row) {
    seg[g.seg(X, Y, tz)] = Counts::pack(nv, nf);
    if (codes && nt) {
      uint4* out = reinterpret_cast<uint4*>(codes + f.rec_index_slot(sh.rec_slot, g, X, Y, Z0));
      out[0] = stage[0];
      out[1] = stage[1];
      out[2] = stage[2];
      out[3] = stage[3];
    }
  }
  // the warp's counts into the CTA's 64-bit sums (a warp's fit 32 bits)
  {
    uint32_t tv = nv, tf = nf;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      tv += __shfl_xor_sync(0xffffffffu, tv, o);
      tf += __shfl_xor_sync(0xffffffffu, tf, o);
    }
    if (lane == 0 && (tv | tf)) {
      atomicAdd(&sh.tot[0], (unsigned long long)tv);
      atomicAdd(&sh.tot[1], (unsigned long long)tf);
    }
  }
  // a cell can emit faces / patches without owning a crossing edge (its
  // crossings may all sit on edges owned by its +1 neighbours)
  const uint32_t busy = __ballot_sync(0xffffffffu, (nv | nf) != 0);
  const uint32_t anyc = __ballot_sync(0xffffffffu, own != 0), first = __ballot_sync(0xffffffffu, (own & 1u) != 0);
  if (lane == 0) {
    sh.act[warp] = busy;
    sh.actc[warp] = anyc;
    sh.actf[warp] = first;
  }
  __syncthreads();
  if (threadIdx.x < (CP / TX) * (CR / TY)) {
    const int tp = threadIdx.x / (CR / TY), tr = threadIdx.x % (CR / TY);
    const int tx = X0 / TX + tp, ty = Y0 / TY + tr;
    if (tx < g.tiles_x() && ty < g.tiles_y()) {
      uint32_t any = 0;
#pragma unroll
      for (int p = 0; p < TX; ++p) any |= (sh.act[tp * TX + p] >> (tr * TY)) & ((1u << TY) - 1u);
      uint32_t bw = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
        uint32_t v = 0;
#pragma unroll
        for (int p = 0; p < (dx ? 1 : TX); ++p) v |= ((dz ? sh.actf : sh.actc)[tp * TX + p] >> (tr * TY));
        if (v & (dy ? 1u : (1u << TY) - 1u)) bw |= 1u << k;
      }
      const int64_t tile = ((int64_t)tx * g.tiles_y() + ty) * g.nzc + tz;
      tile_flag[tile] = any ? 1 : 0;
      tile_flag[g.ntiles() + tile] = (uint8_t)bw;
      if (any) {
        const int at = atomicAdd(&sh.nlist, 1);
        if (at < COUNT_LIST)
          sh.list[at] = (int)tile | tag;
        else
          sh.spill[atomicAdd(sh.spill_n, 1ull)] = (int)tile | tag;
      }
    }
  }
}

// row masks of chunk t - 1 from the ballots of chunk t in sh.bal and the history of
// the lane's rows (i = lane, lane + 32 of this warp): p2 = chunk t - 2, p1 = chunk t - 1;
// vrows: bit i = the warp's point row i lies in the grid (used rows only)
// (written masks only) bit 0: one of them is not all ones, bit 1: one is not all zeros
template <class S, int METHOD>
__device__ __forceinline__ uint32_t count_combine_cur(CountShared<S, METHOD>& sh, bool write, uint32_t (&p1)[2],
                                                      uint32_t (&p2)[2], const uint32_t (&curk)[2]) {
  constexpr uint64_t ALL = (1ull << (MASK_TOP + 1)) - 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t mixed = 0;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int i = lane + 32 * k, r = warp + 8 * i;
    if (i < CRPW && r < CROWS) {
      const uint32_t cur = curk[k];
      if (write) {
        const uint64_t m = (uint64_t)(p2[k] >> 30) | ((uint64_t)p1[k] << 2) | ((uint64_t)(cur & 1u) << 34);
        (&sh.m[0][0])[r] = m;
        mixed |= (m != ALL ? 1u : 0u) | (m != 0 ? 2u : 0u);
      }
      p2[k] = p1[k];
      p1[k] = cur;
    }
  }
  return mixed;
}

template <class S, int METHOD>
__device__ __forceinline__ uint32_t count_combine(CountShared<S, METHOD>& sh, bool write, uint32_t (&p1)[2],
                                                  uint32_t (&p2)[2]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t cur[2] = {0u, 0u};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int i = lane + 32 * k, r = warp + 8 * i;
    if (i < CRPW && r < CROWS) cur[k] = sh.bal[r];
  }
  return count_combine_cur<S, METHOD>(sh, write, p1, p2, cur);
}

// bits (value >= iso) of the points at unpadded z0 .. z0 + cnt - 1 of the lane's
// point rows (i = lane, lane + 32 of this warp; rows from padded (X0, Y0)), each at
// bit z mod 32 as in that chunk's ballot; the pad value outside the grid
template <class S>
__device__ __forceinline__ void point_bits(const Field<S>& f, int X0, int Y0, int z0, int cnt, uint32_t (&out)[2]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int i = lane + 32 * k, r = warp + 8 * i;
    uint32_t b = 0;
    if (i < CRPW && r < CROWS) {
      const int X = X0 + r / (CR + 1), Y = Y0 + r % (CR + 1);
      for (int c = 0; c < cnt; ++c) b |= (f.at(X, Y, z0 + c + 1) >= f.iso ? 1u : 0u) << ((z0 + c) & 31);
    }
    out[k] = b;
  }
}

// A chunk whose masks are all ones or all zeros has no non-trivial cell: its
// segments count zero and its tiles are idle, with no shared-memory work.
template <class S, int METHOD>
__device__ __forceinline__ void count_chunk_empty(const Geom& g, uint64_t* __restrict__ seg,
                                                  uint8_t* __restrict__ tile_flag, int X0, int Y0, int tz) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int X = X0 + warp, Y = Y0 + lane;
  if (X < g.c[0] && Y < g.c[1]) seg[g.seg(X, Y, tz)] = 0;
  if (threadIdx.x < (CP / TX) * (CR / TY)) {
    const int tx = X0 / TX + threadIdx.x / (CR / TY), ty = Y0 / TY + threadIdx.x % (CR / TY);
    if (tx < g.tiles_x() && ty < g.tiles_y()) {
      const int64_t tile = ((int64_t)tx * g.tiles_y() + ty) * g.nzc + tz;
      tile_flag[tile] = 0;
      tile_flag[g.ntiles() + tile] = 0;
    }
  }
}

// One unit: per-segment counts, activity bytes of its tiles, the grid's min / max;
// active tiles are appended (as tile | tag) to sh.list.
template <class S, int METHOD, class F = Field<S>>
__device__ __forceinline__ void count_unit(CountShared<S, METHOD>& sh, const F& f, const Geom& g,
                                           uint64_t* __restrict__ seg, uint8_t* __restrict__ tile_flag,
                                           CellRec* __restrict__ codes, Stats* stats, int64_t unit, int tag,
                                           int64_t& ck) {
  // a row of nzc chunks is cut into nbz near-equal runs of at most KZ chunks
  const int nby = (g.c[1] + CR - 1) / CR, nbz = (g.nzc + KZ - 1) / KZ, kz = (g.nzc + nbz - 1) / nbz;
  const int tz0 = (int)(unit % nbz) * kz;
  const int64_t col = unit / nbz;
  const int X0 = (int)(col / nby) * CP, Y0 = (int)(col % nby) * CR;
  const int tz1 = min(tz0 + kz, g.nzc);
  // point row r = (X0 + r / (CR+1), Y0 + r % (CR+1)) in padded coordinates
  for (int r = threadIdx.x; r < CROWS; r += NTHREADS) {
    const int X = X0 + r / (CR + 1), Y = Y0 + r % (CR + 1);
    const bool in = (unsigned)(X - 1) < (unsigned)f.n0 && (unsigned)(Y - 1) < (unsigned)f.n1;
    sh.rowoff[r] = in ? ((int64_t)(X - 1) * f.n1 + (Y - 1)) * f.n2 : -1;
  }
  __syncthreads();  // also: the previous unit's last readers of sh.m / sh.act are done
  S mn = S(INFINITY), mx = S(-INFINITY);
  // ballot history of the lane's rows i = lane and lane + 32 of this warp:
  // chunks tz - 1 (p2) and tz (p1)
  uint32_t p1[2] = {0u, 0u}, p2[2] = {0u, 0u};
  // interior z of chunk t: [32t, 32t + 32); the padded mask of chunk tz spans
  // unpadded z in [32tz - 2, 32tz + 33)
#pragma unroll 1
  for (int t = tz0 - 1; t <= tz1; ++t) {
    count_ballots<S, METHOD>(sh, f, t, t < tz0 ? 0xc0000000u : (t == tz1 ? 1u : 0xffffffffu), mn, mx, X0, Y0);
    const uint32_t mixed = count_combine<S, METHOD>(sh, t >= tz0 + 1, p1, p2);
    if (t < tz0 + 1) continue;
    // slots rotate over the CTA's chunks: slot (ck+2)%3 was last read before the
    // previous barrier and is next written after the next one
    const int slot = (int)(ck % 3);
    if (mixed) atomicOr(&sh.mixed[slot], mixed);
    __syncthreads();
    const uint32_t mx3 = sh.mixed[slot];
    if (threadIdx.x == 0) sh.mixed[(ck + 2) % 3] = 0;
    ++ck;
    if (mx3 == 3u)
      count_chunk<S, METHOD>(sh, f, g, seg, tile_flag, codes, X0, Y0, t - 1, tag);
    else
      count_chunk_empty<S, METHOD>(g, seg, tile_flag, X0, Y0, t - 1);
  }
  publish_minmax<S>(stats, mn, mx);
}

// append the CTA's active tiles to the global list
template <class S, int METHOD>
__device__ __forceinline__ void count_flush(CountShared<S, METHOD>& sh, unsigned long long* n_active,
                                            int* __restrict__ active) {
  __syncthreads();
  const int n = min(sh.nlist, COUNT_LIST);  // the others went to the list directly
  if (threadIdx.x == 0) sh.base = n ? (int)atomicAdd(n_active, (unsigned long long)n) : 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) active[sh.base + i] = sh.list[i];
}

template <class S, int METHOD, class F = Field<S>>
__global__ void __launch_bounds__(NTHREADS, F::kDense ? 3 : 2) count_kernel(F f, Geom g, uint64_t* __restrict__ seg,
                                                            uint8_t* __restrict__ tile_flag,
                                                            CellRec* __restrict__ codes, Stats* stats,
                                                            int* __restrict__ active) {
  __shared__ CountShared<S, METHOD> sh;
  if (threadIdx.x == 0) {
    sh.nlist = 0;
    sh.tot[0] = sh.tot[1] = 0ull;
    sh.spill = active;
    sh.spill_n = &stats->n_active;
    sh.mixed[0] = sh.mixed[1] = sh.mixed[2] = 0;
  }
  const int64_t nunits = count_units(g);
  int64_t ck = 0;  // chunks this CTA has counted
#pragma unroll 1
  for (int64_t u = blockIdx.x; u < nunits; u += gridDim.x)
    count_unit<S, METHOD>(sh, f, g, seg, tile_flag, codes, stats, u, 0, ck);
  count_flush<S, METHOD>(sh, &stats->n_active, active);
  count_totals<S, METHOD>(sh, stats);
}

// ------------------------------------------------------------------ evaluated fields

// The units of an evaluated field's count that may hold both sides of iso: one warp
// per unit classifies the unit's box (every point its chunks' masks read; pads: part
// of it lies outside the grid); a unit wholly on one side publishes its bound and is
// left out (its record stays as the host zeroed it), the others are appended to
// units[1 ..] (units[0] counts them) for field_count_kernel.
template <class S, class F>
__global__ void __launch_bounds__(256) field_units_kernel(F f, Geom g, Stats* stats, int* __restrict__ units,
                                                          int* __restrict__ umap) {
  const int lane = threadIdx.x & 31;
  const int nby = (g.c[1] + CR - 1) / CR, nbz = (g.nzc + KZ - 1) / KZ, kz = (g.nzc + nbz - 1) / nbz;
  const int64_t nunits = count_units(g), step = ((int64_t)gridDim.x * blockDim.x) >> 5;
#pragma unroll 1
  for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nunits; u += step) {
    const int tz0 = (int)(u % nbz) * kz, tz1 = min(tz0 + kz, g.nzc);
    const int64_t col = u / nbz;
    const int X0 = (int)(col / nby) * CP, Y0 = (int)(col % nby) * CR;
    const int xa = max(X0 - 1, 0), xb = min(X0 + CP - 1, f.n0 - 1);
    const int ya = max(Y0 - 1, 0), yb = min(Y0 + CR - 1, f.n1 - 1);
    const int za = max(32 * tz0 - 2, 0), zb = min(32 * tz1, f.n2 - 1);
    const bool pads = X0 - 1 < 0 || X0 + CP - 1 >= f.n0 || Y0 - 1 < 0 || Y0 + CR - 1 >= f.n1 || 32 * tz0 - 2 < 0 ||
                      32 * tz1 >= f.n2;
    S bound = S(0);
    uint64_t cand = 0;
    bool all = true;
    if (f.classify_warp(xa, xb, ya, yb, za, zb, pads, bound, cand, all) >= 0) {
      if (xa <= xb && ya <= yb && za <= zb) publish_minmax<S>(stats, bound, bound);
    } else if (lane == 0) {
      const int at = atomicAdd(units, 1);
      units[1 + at] = (int)u;
      if (umap) umap[u] = at;  // the unit's block of cell records (a narrow band's DMC)
    }
  }
}

// count_kernel over the units that field_units_kernel listed
template <class S, int METHOD, class F>
__global__ void __launch_bounds__(NTHREADS, 2) field_count_kernel(F f, Geom g, uint64_t* __restrict__ seg,
                                                                  uint8_t* __restrict__ tile_flag,
                                                                  CellRec* __restrict__ codes, Stats* stats,
                                                                  int* __restrict__ active,
                                                                  const int* __restrict__ units) {
  __shared__ CountShared<S, METHOD> sh;
  if (threadIdx.x == 0) {
    sh.nlist = 0;
    sh.tot[0] = sh.tot[1] = 0ull;
    sh.spill = active;
    sh.spill_n = &stats->n_active;
    sh.mixed[0] = sh.mixed[1] = sh.mixed[2] = 0;
  }
  const int n = units[0];
  int64_t ck = 0;
#pragma unroll 1
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    // the unit's block of cell records is its place in the list (read after
    // count_unit's first barrier; the previous unit's readers passed its last one)
    if (threadIdx.x == 0) sh.rec_slot = i;
    count_unit<S, METHOD>(sh, f, g, seg, tile_flag, codes, stats, units[1 + i], 0, ck);
  }
  count_flush<S, METHOD>(sh, &stats->n_active, active);
  count_totals<S, METHOD>(sh, stats);
}

// ------------------------------------------------------------------ count through TMA

// The count pass with the SDF brought into shared memory by the TMA unit: for every
// chunk of a unit one bulk tensor copy of the box of 9 x 33 point rows x 32 points
// (out-of-grid points arrive as zeros and are replaced by the pad value).  The three
// points of each row that a unit's masks take from the chunks below and above it
// (two below its first chunk, one above its last) are plain loads by the lanes that
// keep those rows' ballot history, so every pipeline step is a full box.  A ring of
// TMA_STAGES boxes per CTA keeps copies in flight while the warps turn the previous
// box into ballots; the counting itself is count_chunk.  Needs a 16-byte aligned SDF
// whose rows are a multiple of 16 bytes (the tensor map's strides); otherwise
// count_kernel runs.
constexpr int KZT = 8;                        // chunks per unit (at most)
constexpr int TMA_STAGES = 2;
constexpr int TMA_TILES_PER_UNIT = (CP / TX) * (CR / TY) * KZT;
constexpr long long TMA_WAIT_CYCLES = 1ll << 32;  // about two seconds

template <class S>
__host__ __device__ constexpr int tma_box_bytes() {
  return CROWS * 32 * (int)sizeof(S);
}
// dynamic shared memory of count_tma_kernel: the stages, plus room to align them to 128 bytes
template <class S>
__host__ __device__ constexpr size_t count_tma_smem() {
  return (size_t)TMA_STAGES * tma_box_bytes<S>() + 128;
}

__host__ __device__ inline int64_t count_tma_units(const Geom& g) {
  return (int64_t)((g.c[0] + CP - 1) / CP) * ((g.c[1] + CR - 1) / CR) * ((g.nzc + KZT - 1) / KZT);
}

// a position in a CTA's stream of boxes: the unit (rows from (X0, Y0), chunks
// [tz0, tz1)) and the box's chunk t in [tz0, tz1)
struct BoxCursor {
  int64_t unit;
  int X0, Y0, tz0, tz1, t;
  __device__ void start(const Geom& g, int64_t u) {
    const int nby = (g.c[1] + CR - 1) / CR, nbz = (g.nzc + KZT - 1) / KZT, kz = (g.nzc + nbz - 1) / nbz;
    unit = u;
    tz0 = (int)(u % nbz) * kz;
    const int64_t col = u / nbz;
    X0 = (int)(col / nby) * CP;
    Y0 = (int)(col % nby) * CR;
    tz1 = min(tz0 + kz, g.nzc);
    t = tz0;
  }
  // the next box; after a unit's last one, the unit next_unit() returns
  template <class NextUnit>
  __device__ void next(const Geom& g, int64_t nunits, NextUnit next_unit) {
    if (++t >= tz1) {
      unit = next_unit();
      if (unit < nunits) start(g, unit);
    }
  }
  __device__ bool valid(int64_t nunits) const { return unit < nunits; }
};

// Zeros written beside a forward's kernels (the gradient buffers of a forward whose
// backward writes only the point tiles near the surface): the bytes [begin, end) of
// two 16-byte aligned ranges seen as one, written by bulk copies of a zeroed block of
// shared memory, so that the writes cost the warps neither issue slots nor load/store
// bandwidth.  Round r of CTA b is the rbytes from begin + (r * gridDim.x + b) * rbytes;
// a CTA issues one round per step of its work (a box of the count, a tile of the
// emit) and the rounds left at its end.
constexpr int ZBUF = 4096;  // bytes of the zero block

struct ZeroJob {
  char* p0;
  char* p1;
  int64_t n0;          // bytes of p0 (a multiple of 16)
  int64_t begin, end;  // multiples of 16
  int64_t rounds;      // ceil((end - begin) / (gridDim.x * rbytes)), 0: no job
  int64_t rbytes;      // bytes per round (a multiple of ZBUF)
};

// zero the block (all threads; a barrier must follow before the first round)
__device__ __forceinline__ void zero_block_init(uint4* zbuf) {
  for (int i = threadIdx.x; i < ZBUF / 16; i += blockDim.x) zbuf[i] = make_uint4(0u, 0u, 0u, 0u);
  fence_proxy_async();  // the zeros are read by the bulk copies
}

// round r of this CTA, one piece of up to ZBUF bytes per lane of the calling warp
__device__ __forceinline__ void zero_round(const ZeroJob& z, const void* zbuf, int64_t r, int lane) {
  if (r >= z.rounds) return;
  const int64_t start = z.begin + (r * gridDim.x + blockIdx.x) * z.rbytes;
  const int64_t end = min(start + z.rbytes, z.end);
  bool any = false;
  for (int64_t o = start + (int64_t)lane * ZBUF; o < end; o += 32 * ZBUF) {
    const int64_t e = min(o + (int64_t)ZBUF, end);
    if (o < z.n0) {  // the piece may run past the end of p0 into p1
      const int64_t e0 = min(e, z.n0);
      bulk_store(z.p0 + o, zbuf, (uint32_t)(e0 - o));
      if (e > z.n0) bulk_store(z.p1, zbuf, (uint32_t)(e - z.n0));
    } else {
      bulk_store(z.p1 + (o - z.n0), zbuf, (uint32_t)(e - o));
    }
    any = true;
  }
  if (any) bulk_commit();
}

// the rounds from r on, then wait for all of the warp's copies
__device__ __forceinline__ void zero_finish(const ZeroJob& z, const void* zbuf, int64_t r, int lane) {
  for (; r < z.rounds; ++r) zero_round(z, zbuf, r, lane);
  bulk_wait_all();
}

template <class S>
__device__ __forceinline__ void issue_box(const CUtensorMap* wide, void* dst, uint64_t* bar, const BoxCursor& c) {
  mbar_expect_tx(bar, (uint32_t)tma_box_bytes<S>());
  tma_load_3d(dst, wide, bar, 32 * c.t, c.Y0 - 1, c.X0 - 1);
}

// ballots of chunk t from its box in shared memory (row r at box + 32 r), and the
// min / max of the values in the grid
template <class S, int METHOD>
__device__ __forceinline__ void box_ballots(CountShared<S, METHOD>& sh, const Field<S>& f, const S* box, int t,
                                            uint64_t vrows, S& mn, S& mx) {
  constexpr int NB = 4, HALF = (CRPW + NB - 1) / NB;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t used = warp + 8 * (CRPW - 1) < CROWS ? (1ull << CRPW) - 1 : (1ull << (CRPW - 1)) - 1;
  if (vrows == used && 32 * t + 32 <= f.n2) {
    // every point of the warp's rows lies in the grid: one load, compare and ballot per row
    const S* p = box + warp * 32 + lane;
#pragma unroll
    for (int i = 0; i < CRPW; ++i) {
      if (i == CRPW - 1 && !((used >> i) & 1ull)) break;
      const S v = p[8 * 32 * i];
      const uint32_t b = __ballot_sync(0xffffffffu, v >= f.iso);
      if (lane == 0) sh.bal[warp + 8 * i] = b;
      mn = smin(mn, v);
      mx = smax(mx, v);
    }
    __syncwarp();
    return;
  }
  const bool zin = 32 * t + lane < f.n2;
#pragma unroll
  for (int h = 0; h < NB; ++h) {
    S v[HALF];
    bool in[HALF];
#pragma unroll
    for (int k = 0; k < HALF; ++k) {
      const int i = h * HALF + k, r = warp + 8 * i;
      in[k] = zin && i < CRPW && ((vrows >> i) & 1ull);
      const S b = box[in[k] ? r * 32 + lane : 0];  // every read stays inside the box
      v[k] = in[k] ? b : f.pad;
    }
#pragma unroll
    for (int k = 0; k < HALF; ++k) {
      const int i = h * HALF + k, r = warp + 8 * i;
      if (i < CRPW && r < CROWS) {
        const uint32_t b = __ballot_sync(0xffffffffu, v[k] >= f.iso);
        if (lane == 0) sh.bal[r] = b;
      }
      if (in[k]) {
        mn = smin(mn, v[k]);
        mx = smax(mx, v[k]);
      }
    }
  }
  __syncwarp();
}

template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS, 2) count_tma_kernel(const __grid_constant__ CUtensorMap wide,
                                                                Field<S> f, Geom g, uint64_t* __restrict__ seg,
                                                                uint8_t* __restrict__ tile_flag,
                                                                CellRec* __restrict__ codes, Stats* stats,
                                                                int* __restrict__ active, const ZeroJob zj) {
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  __shared__ CountShared<S, METHOD> sh;
  __shared__ __align__(8) uint64_t full[TMA_STAGES];
  __shared__ __align__(128) uint4 zbuf[ZBUF / 16];
  __shared__ int64_t uq[4];  // units in the order the producer took them (a ring: it runs <= 2 boxes ahead)
  unsigned char* stage_mem = dyn_smem + ((128u - (smem_u32(dyn_smem) & 127u)) & 127u);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nunits = count_tma_units(g);
  if (zj.rounds) zero_block_init(zbuf);
  if (threadIdx.x == 0) {
    sh.nlist = 0;
    sh.tot[0] = sh.tot[1] = 0ull;
    sh.spill = active;
    sh.spill_n = &stats->n_active;
    sh.mixed[0] = sh.mixed[1] = sh.mixed[2] = 0;
#pragma unroll
    for (int st = 0; st < TMA_STAGES; ++st) mbar_init(&full[st], 1);
    mbar_fence_init();
  }
  __syncthreads();
  // Units are taken from a grid-wide counter (stats->units, zeroed by the forward's
  // reset) by the producer (thread 0) as it reaches them, so CTAs that met cheap
  // units take more; the consumers follow the producer's order through uq (each id
  // is written at least one CTA barrier before it is read).
  unsigned long long* const unit_ctr = &stats->units;
  int pseq = 0, cseq = 0;
  auto take_unit = [&]() -> int64_t {
    const int64_t u = (int64_t)atomicAdd(unit_ctr, 1ull);
    const int64_t v = u < nunits ? u : nunits;
    uq[pseq++ & 3] = v;
    return v;
  };
  BoxCursor pc, cc;  // producer (thread 0) and consumer positions
  pc.unit = cc.unit = nunits;
  int64_t issued = 0;
  if (threadIdx.x == 0) {
    const int64_t u = take_unit();
    if (u < nunits) pc.start(g, u);
    for (int st = 0; st < TMA_STAGES && pc.valid(nunits); ++st, ++issued) {
      issue_box<S>(&wide, stage_mem + st * tma_box_bytes<S>(), &full[st], pc);
      pc.next(g, nunits, take_unit);
    }
  }
  __syncthreads();  // uq holds the first units
  auto read_unit = [&]() -> int64_t { return uq[cseq++ & 3]; };
  {
    const int64_t u = read_unit();
    if (u < nunits) cc.start(g, u);
  }
  S mn = S(INFINITY), mx = S(-INFINITY);
  uint32_t p1[2] = {0u, 0u}, p2[2] = {0u, 0u};
  uint64_t vrows = 0;
  bool failed = false;
  int64_t k = 0;
  for (; cc.valid(nunits); ++k) {
    const int st = (int)(k % TMA_STAGES);
    if (cc.t == cc.tz0) {
      // a new unit: which of the warp's point rows lie in the grid, and the ballot
      // history of the lane's rows: the two points below the unit's first chunk
      vrows = 0;
#pragma unroll
      for (int i = 0; i < CRPW; ++i) {
        const int r = warp + 8 * i;
        const int X = cc.X0 + r / (CR + 1), Y = cc.Y0 + r % (CR + 1);
        if (r < CROWS && (unsigned)(X - 1) < (unsigned)f.n0 && (unsigned)(Y - 1) < (unsigned)f.n1) vrows |= 1ull << i;
      }
      point_bits<S>(f, cc.X0, cc.Y0, 32 * cc.tz0 - 2, 2, p1);
      p2[0] = p2[1] = 0u;
    }
    // at the unit's last chunk, the point above it (read before the wait)
    uint32_t above[2] = {0u, 0u};
    if (cc.t == cc.tz1 - 1) point_bits<S>(f, cc.X0, cc.Y0, 32 * cc.tz1, 1, above);
    if (warp == 1) zero_round(zj, zbuf, k, lane);
    const bool ok = mbar_wait_bounded(&full[st], (uint32_t)((k / TMA_STAGES) & 1), TMA_WAIT_CYCLES);
    box_ballots<S, METHOD>(sh, f, reinterpret_cast<const S*>(stage_mem + st * tma_box_bytes<S>()), cc.t, vrows, mn,
                           mx);
    const uint32_t mixed = count_combine<S, METHOD>(sh, cc.t >= cc.tz0 + 1, p1, p2);
    // slots rotate over the CTA's boxes: slot (k+2)%3 was last read before the
    // previous barrier and is next written after the next one
    const int slot = (int)(k % 3);
    if (mixed) atomicOr(&sh.mixed[slot], mixed);
    // every warp is done with the stage (and sh.m is complete): refill the stage
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    const uint32_t mx3 = sh.mixed[slot];
    if (threadIdx.x == 0) {
      sh.mixed[(k + 2) % 3] = 0;
      if (pc.valid(nunits)) {
        fence_proxy_async();
        issue_box<S>(&wide, stage_mem + st * tma_box_bytes<S>(), &full[st], pc);
        pc.next(g, nunits, take_unit);
        ++issued;
      }
    }
    if (cc.t >= cc.tz0 + 1) {
      if (mx3 == 3u)
        count_chunk<S, METHOD>(sh, f, g, seg, tile_flag, codes, cc.X0, cc.Y0, cc.t - 1, 0);
      else
        count_chunk_empty<S, METHOD>(g, seg, tile_flag, cc.X0, cc.Y0, cc.t - 1);
    }
    if (cc.t == cc.tz1 - 1) {
      // the unit's last chunk, its masks completed by the points above it
      __syncthreads();  // the chunk just counted is done with sh.m and sh.act
      const uint32_t m = count_combine_cur<S, METHOD>(sh, true, p1, p2, above);
      // a mask with a zero bit and a mask with a one bit: the chunk has crossings
      const bool some0 = __syncthreads_or(m & 1u), some1 = __syncthreads_or(m & 2u);
      if (some0 && some1)
        count_chunk<S, METHOD>(sh, f, g, seg, tile_flag, codes, cc.X0, cc.Y0, cc.t, 0);
      else
        count_chunk_empty<S, METHOD>(g, seg, tile_flag, cc.X0, cc.Y0, cc.t);
    }
    cc.next(g, nunits, read_unit);
  }
  if (failed && threadIdx.x == 0) {
    atomicOr(&stats->error, 4ull);
    // let the copies in flight land before the CTA's shared memory goes away
    for (int64_t j = k; j < issued; ++j)
      mbar_wait_bounded(&full[j % TMA_STAGES], (uint32_t)((j / TMA_STAGES) & 1), TMA_WAIT_CYCLES);
  }
  if (warp == 1) zero_finish(zj, zbuf, k, lane);
  publish_minmax<S>(stats, mn, mx);
  count_flush<S, METHOD>(sh, &stats->n_active, active);
  count_totals<S, METHOD>(sh, stats);
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
  CellRec* codes;       // this grid's cell records (count -> emit), null for MC
  int64_t cblk0;        // first count unit of the grid in the flattened queue
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
// units; per-grid status words in stats[grid]
template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS, 3) batch_count_kernel(const BatchGrid<S>* __restrict__ grids, int ngrids,
                                                                  int64_t nblocks, Stats* stats,
                                                                  unsigned long long* n_active,
                                                                  int* __restrict__ active) {
  __shared__ CountShared<S, METHOD> sh;
  __shared__ int64_t start[MAX_BATCH];
  for (int i = threadIdx.x; i < ngrids; i += blockDim.x) start[i] = grids[i].cblk0;
  if (threadIdx.x == 0) {
    sh.nlist = 0;
    sh.tot[0] = sh.tot[1] = 0ull;
    sh.spill = active;
    sh.spill_n = n_active;
    sh.mixed[0] = sh.mixed[1] = sh.mixed[2] = 0;
  }
  __syncthreads();
  int64_t ck = 0;  // chunks this CTA has counted
#pragma unroll 1
  for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x) {
    const int i = batch_find(start, ngrids, b);
    const BatchGrid<S>& G = grids[i];
    count_unit<S, METHOD>(sh, G.f, G.g, G.seg, G.tile_flag, G.codes, stats + i, b - start[i], i << BATCH_TILE_BITS,
                          ck);
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
template <class S, class F = Field<S>>
__device__ __forceinline__ void mc_emit_tile(const F& f, const Geom& g, const uint64_t* __restrict__ seg,
                                             int tile, S* __restrict__ verts, int64_t* __restrict__ faces,
                                             int normalize, int64_t vsub, const EdgeRecord<S>& rec) {
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
  __shared__ uint32_t nvi, nci;
  int X0, Y0, Z0, tz;
  tile_coords(tile, g, X0, Y0, Z0, tz);
  // segment values (one per thread) loaded first, so that they overlap the mask loads
  static_assert(CX * CY * 2 <= NTHREADS, "one segment value per thread");
  const int sk = threadIdx.x & 1, sy = (threadIdx.x >> 1) % CY, sx = (threadIdx.x >> 1) / CY;
  uint64_t sv = 0;
  if (threadIdx.x < CX * CY * 2 && X0 + sx < g.c[0] && Y0 + sy < g.c[1] && tz + sk < g.nzc)
    sv = seg[g.seg(X0 + sx, Y0 + sy, tz + sk)];
  S dmn, dmx;
  bool dseen = false;
  load_masks<S, WX, WY, false>(m, f, X0, Y0, Z0, dmn, dmx, dseen);
  if (threadIdx.x < CX * CY * 2) {
    vb[sx][sy][sk] = Counts::lo(sv);
    if (sk == 0 && sx < TX && sy < TY) fb[sx][sy] = Counts::hi(sv);
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
    const CodeRow cr = code_row(m[ox][oy], m[ox + 1][oy], m[ox][oy + 1], m[ox + 1][oy + 1]);
    while (nt) {
      const int j = __ffs(nt) - 1;
      nt &= nt - 1;
      fpre[ox][oy][j] = (uint8_t)run;
      run += (uint32_t)(mc_tri(mc_from_morton(code_at(cr, j))) & 15);
    }
  }
  // the own rows are warp 0's lanes: their bases by a warp scan
  static_assert(TX * TY == 32, "one own row per lane of warp 0");
  if (threadIdx.x < 32) {
    const uint32_t v = cv | (cc << 16), inc = warp_incl(v), tot = __shfl_sync(0xffffffffu, inc, 31);
    const uint32_t off = inc - v;
    if (threadIdx.x == 0) {
      nvi = tot & 0xffffu;
      nci = tot >> 16;
    }
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
    const int64_t v = vid(x, y, j, a);
    store_vertex<S>(verts, v, p, g, normalize);
    if (rec.loc) rec.loc[v] = pack_loc(X0 + x, Y0 + y, Z0 + j, a);
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
        const int ge = edge_desc(e);
        faces[3 * (f0 + t) + k] = vid(x + (ge & 1), y + ((ge >> 1) & 1), j + ((ge >> 2) & 1), ge >> 3) - vsub;
      }
    }
  }
  __syncthreads();  // the shared arrays are reused by the CTA's next tile
}

// the record of one grid (null: none), laid out for the grid's scanned totals
template <class S, int METHOD>
__device__ __forceinline__ EdgeRecord<S> grid_record(void* record, const Geom& g, const uint64_t* __restrict__ seg) {
  if (!record) return EdgeRecord<S>{nullptr, nullptr, nullptr, nullptr};
  const uint64_t tot = seg[g.nseg];
  return edge_record<S>(record, METHOD, METHOD == MC ? Counts::lo(tot) : Counts::hi(tot), Counts::lo(tot));
}

// Whether the outputs of the grid's scanned totals fit the capacities (vcap vertices,
// fcap faces); when not, nothing is emitted and bit 1 of stats->error is set.
template <int METHOD>
__device__ __forceinline__ bool emit_fits(const Geom& g, const uint64_t* __restrict__ seg, int64_t vcap, int64_t fcap,
                                          Stats* stats) {
  const uint64_t tot = seg[g.nseg];
  const int64_t V = METHOD == MC ? Counts::lo(tot) : Counts::hi(tot), F = METHOD == MC ? Counts::hi(tot) : Counts::lo(tot);
  if (V <= vcap && F <= fcap) return true;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&stats->error, 2ull);
  return false;
}

// persistent over the *n_active active tiles of the count, taken in turn from a
// counter (tiles differ much in cost)
template <class S, class F = Field<S>>
__global__ void __launch_bounds__(NTHREADS) mc_emit_kernel(F f, Geom g, const uint64_t* __restrict__ seg,
                                                           const int* __restrict__ active,
                                                           const unsigned long long* __restrict__ n_active,
                                                           S* __restrict__ verts, int64_t* __restrict__ faces,
                                                           int normalize, void* record, int64_t vcap, int64_t fcap,
                                                           Stats* stats, const ZeroJob zj) {
  __shared__ __align__(128) uint4 zbuf[ZBUF / 16];
  __shared__ int64_t next;
  if (zj.rounds) zero_block_init(zbuf);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int64_t it = 0;  // tiles of this CTA, one zero round each
  if (emit_fits<MC>(g, seg, vcap, fcap, stats)) {
    const EdgeRecord<S> rec = grid_record<S, MC>(record, g, seg);
    const int64_t n = (int64_t)*n_active;
#pragma unroll 1
    for (;; ++it) {
      if (threadIdx.x == 0) next = (int64_t)atomicAdd(&stats->emit_tile, 1ull);
      __syncthreads();
      const int64_t t = next;
      __syncthreads();
      if (t >= n) break;
      if (warp == 1) zero_round(zj, zbuf, it, lane);
      mc_emit_tile<S>(f, g, seg, active[t], verts, faces, normalize, 0, rec);
    }
  }
  __syncthreads();
  if (warp == 1) zero_finish(zj, zbuf, it, lane);
}

// ------------------------------------------------------------------ DMC emit

// Edge window of a DMC tile: the cells [X0, X0+TX] x [Y0, Y0+TY] x [Z0, Z0+TZ] own
// every edge of the tile's cells.  Their crossing edges get window slots in
// (row, cell, axis) order; when they fit, each one's lerp vertex is computed once
// into shared memory and the dual vertices read it from there (a tile's cells share
// most of their edges).  Tiles with more crossing edges compute them per patch.
constexpr int EW_ROWS = (TX + 1) * (TY + 1);
constexpr int EW_ITEMS = EW_ROWS * 3 * (TZ + 1);
static_assert(EW_ITEMS < (1 << 13), "window slots and flags share 16 bits");
constexpr int EPOS_BYTES = 24576;
template <class S>
__host__ __device__ constexpr int epos_cap() {
  return EPOS_BYTES / (3 * (int)sizeof(S));
}

// One active tile: its dual vertices and quads; patch ids written into quads are
// reduced by vsub (as in mc_emit_tile).  The cells' codes (after the ambiguity test)
// and in-segment patch offsets come from the cell records of the count (valid for the
// segments whose count is not zero; the others hold trivial cells only), so the SDF is
// read only for the edge vertices.
template <class S, class F = Field<S>>
__device__ __forceinline__ void dmc_emit_tile(const F& f, const Geom& g, const uint64_t* __restrict__ seg,
                                              const CellRec* __restrict__ codes, int tile, S* __restrict__ verts,
                                              int64_t* __restrict__ quads, int normalize, int64_t vsub,
                                              const EdgeRecord<S>& rec) {
  constexpr int KX = TX + 2, KY = TY + 2;  // window: cells [X0-1, X0+TX] x [Y0-1, Y0+TY], z index j+1 for Z0+j,
  constexpr int KZ2 = TZ + 2;              // j in [-1, TZ]
  constexpr int CX = TX + 1, CY = TY + 1;  // code rows: cells [X0-1, X0+TX) x [Y0-1, Y0+TY) (own + the -1 halo)
  constexpr int CAP = epos_cap<S>();
  __shared__ CellRec cw[KX][KY][KZ2];     // cell records of the window (0 where trivial)
  __shared__ uint8_t sact[KX][KY];        // bit 0/1/2: the row's segment tz-1 / tz / tz+1 has a non-zero count
  __shared__ uint32_t pb[CX][CY];
  __shared__ uint32_t qb[TX][TY];
  __shared__ RowBits wb[TX + 1][TY + 1];  // edge rows: cells [X0, X0+TX] x [Y0, Y0+TY]
  __shared__ uint8_t w32[TX + 1][TY + 1];  // crossing flags of the row's cell Z0 + TZ
  __shared__ uint16_t wcell[TX + 1][TY + 1][TZ + 1];  // per edge-row cell: first window slot | flags << 13
  __shared__ uint16_t witems[EW_ITEMS];
  __shared__ uint16_t pitems[4 * TX * TY * TZ];  // dual vertex items: one per patch of the tile's cells
  __shared__ uint8_t prow[TX][TY];        // patches of the own rows' segments
  __shared__ __align__(16) S epos[CAP][3];
  __shared__ typename F::RecTab rtab;  // a narrow band's record blocks around the window
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int X0, Y0, Z0, tz;
  tile_coords(tile, g, X0, Y0, Z0, tz);
  if (threadIdx.x < 12) f.rec_tab_fill(rtab, g, X0, Y0, Z0, threadIdx.x);
  // segment values of the window rows: activity of chunks tz-1, tz, tz+1, the bases
  if (threadIdx.x < KX * KY) {
    const int wx = threadIdx.x / KY, wy = threadIdx.x % KY, X = X0 - 1 + wx, Y = Y0 - 1 + wy;
    uint32_t act = 0;
    uint64_t s0 = 0, s1 = 0;
    if (X >= 0 && Y >= 0 && X < g.c[0] && Y < g.c[1]) {
      const int64_t i = g.seg(X, Y, tz);
      s0 = seg[i];
      s1 = seg[i + 1];
      if (s1 != s0) act |= 2;
      if (tz > 0 && seg[i - 1] != s0) act |= 1;
      if (tz + 1 < g.nzc && seg[i + 2] != s1) act |= 4;
    }
    sact[wx][wy] = (uint8_t)act;
    if (wx < CX && wy < CY) {
      pb[wx][wy] = Counts::hi(s0);
      if (wx >= 1 && wy >= 1) {
        qb[wx - 1][wy - 1] = Counts::lo(s0);
        prow[wx - 1][wy - 1] = (uint8_t)(Counts::hi(s1) - Counts::hi(s0));
      }
    }
  }
  __syncthreads();
  // records of the window, one warp per row, every row of the warp in flight
  // together, and with them the rows' ends (cells Z0 - 1 and Z0 + TZ: thread t below
  // 2 KX KY takes end t & 1 of row t >> 1); the edge rows' crossing bits from them
  constexpr int RPW = (KX * KY + NTHREADS / 32 - 1) / (NTHREADS / 32);
  int c[RPW], rend = 0;
#pragma unroll
  for (int k = 0; k < RPW; ++k) {
    const int r = warp + (NTHREADS / 32) * k;
    c[k] = 0;
    if (r < KX * KY) {
      const int wx = r / KY, wy = r % KY;
      if (sact[wx][wy] & 2) c[k] = codes[f.rec_index_tab(rtab, g, X0 - 1 + wx, Y0 - 1 + wy, Z0 + lane)];
    }
  }
  if (threadIdx.x < 2 * KX * KY) {
    const int r = threadIdx.x >> 1, end = threadIdx.x & 1, wx = r / KY, wy = r % KY;
    if (sact[wx][wy] & (end ? 4u : 1u))
      rend = codes[f.rec_index_tab(rtab, g, X0 - 1 + wx, Y0 - 1 + wy, end ? Z0 + TZ : Z0 - 1)];
  }
#pragma unroll
  for (int k = 0; k < RPW; ++k) {
    const int r = warp + (NTHREADS / 32) * k;
    if (r >= KX * KY) break;
    const int wx = r / KY, wy = r % KY;
    cw[wx][wy][lane + 1] = (CellRec)c[k];
    if (wx >= 1 && wy >= 1) {
      const int code = c[k] & 0xff, cf = cross_flags(code);
      RowBits w;
      w.xc = __ballot_sync(0xffffffffu, cf & 1);
      w.yc = __ballot_sync(0xffffffffu, cf & 2);
      w.zc = __ballot_sync(0xffffffffu, cf & 4);
      w.nt = __ballot_sync(0xffffffffu, code != 0 && code != 255);
      if (lane == 0) wb[wx - 1][wy - 1] = w;
    }
  }
  if (threadIdx.x < 2 * KX * KY) {
    const int r = threadIdx.x >> 1, end = threadIdx.x & 1, wx = r / KY, wy = r % KY;
    cw[wx][wy][end ? TZ + 1 : 0] = (CellRec)rend;
    if (end && wx >= 1 && wy >= 1) w32[wx - 1][wy - 1] = (uint8_t)cross_flags(rend & 0xff);
  }
  __syncthreads();
  // code after the ambiguity test, and first patch relative to its row's base pb, of
  // window cell (x, y) at z index jj (jj = 0: cell Z0-1, the last of the previous segment)
  auto rcode = [&](int x, int y, int jj) -> int { return cw[x][y][jj] & 0xff; };
  auto ppatch = [&](int x, int y, int jj) -> int {
    const int r = cw[x][y][jj];
    return jj ? (r >> 9) : -(int)dmc_npatch(dmc_case(r & 0xff));
  };
  // edge rows: crossing edges (window items) and, for the own rows, the patches
  // (dual vertex items).  Every warp scans the rows' counts itself (rows lane and
  // lane + 32), so that the row bases need no block-wide scan and no barrier; then one
  // warp per row writes the row's window items and dual vertex items
  static_assert(EW_ROWS <= 64 && EW_ROWS > 32, "two edge rows per lane");
  uint32_t base_lo, base_hi, nwi, nci;
  {
    uint32_t v[2] = {0u, 0u};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = lane + 32 * h, ex_ = r / (TY + 1), ey = r % (TY + 1);
      if (r < EW_ROWS) {
        const RowBits w = wb[ex_][ey];
        const uint32_t ce = __popc(w.xc) + __popc(w.yc) + __popc(w.zc) + __popc(w32[ex_][ey]);
        const uint32_t cc = (ex_ < TX && ey < TY) ? prow[ex_][ey] : 0u;
        v[h] = ce | (cc << 13);
      }
    }
    const uint32_t i0 = warp_incl(v[0]);
    const uint32_t i1 = warp_incl(v[1]) + __shfl_sync(0xffffffffu, i0, 31);
    const uint32_t tot = __shfl_sync(0xffffffffu, i1, 31);
    base_lo = i0 - v[0];
    base_hi = i1 - v[1];
    nwi = tot & 0x1fffu;
    nci = tot >> 13;
  }
  for (int r = warp; r < EW_ROWS; r += NTHREADS / 32) {
    const int ex_ = r / (TY + 1), ey = r % (TY + 1);
    const RowBits w = wb[ex_][ey];
    const uint32_t rbase = r < 32 ? __shfl_sync(0xffffffffu, base_lo, r) : __shfl_sync(0xffffffffu, base_hi, r - 32);
    // window items in slot order: cells ascending, axes ascending per cell
    const int fl = row_flags(w, lane);
    const uint32_t before = row_prefix(w, lane);
    uint32_t o = (rbase & 0x1fffu) + before;
    wcell[ex_][ey][lane] = (uint16_t)(o | (fl << 13));
#pragma unroll
    for (int a = 0; a < 3; ++a)
      if (fl & (1 << a)) witems[o++] = item_code(ex_, ey, lane, a);
    if (lane == 31) {
      const int f32 = w32[ex_][ey];
      wcell[ex_][ey][TZ] = (uint16_t)(o | (f32 << 13));
#pragma unroll
      for (int a = 0; a < 3; ++a)
        if (f32 & (1 << a)) witems[o++] = item_code(ex_, ey, TZ, a);
    }
    // an own row's dual vertex items, one per patch in patch order: the patches of a
    // non-trivial cell run from its record's in-segment prefix to the next
    // non-trivial cell's (the segment's total after the last one; trivial cells have
    // no record)
    if (ex_ < TX && ey < TY && ((w.nt >> lane) & 1)) {
      const int x = ex_ + 1, y = ey + 1;
      const uint32_t later = w.nt & ~((2u << lane) - 1u);
      const int p0 = cw[x][y][lane + 1] >> 9;
      const int p1 = later ? cw[x][y][__ffs(later)] >> 9 : (int)prow[ex_][ey];
      for (int q = 0; q < p1 - p0; ++q) pitems[(rbase >> 13) + p0 + q] = item_code(ex_, ey, lane, q);
    }
  }
  __syncthreads();
  const bool cached = nwi <= (uint32_t)CAP;
  // every end point of the window's edges lies inside the caller's grid
  const bool inner = X0 >= 1 && Y0 >= 1 && Z0 >= 1 && X0 + TX + 1 <= f.n0 && Y0 + TY + 1 <= f.n1 &&
                     Z0 + TZ + 1 <= f.n2;
  // window edges: lerp vertices into the cache; the tile's own edges also give its quads
  // (one per crossing edge owned by a tile cell, src/cudualmc.cu:753-794, 1019-1056);
  // the edge exits (value falls through iso) when its start point is >= iso
  for (uint32_t i = threadIdx.x; i < nwi; i += blockDim.x) {
    int ix, iy, j, a;
    item_decode(witems[i], ix, iy, j, a);
    if (cached) {
      S p[3];
      if constexpr (F::kDense) {
        if (inner)
          edge_vertex_in<S>(f, X0 + ix, Y0 + iy, Z0 + j, a, p);
        else
          edge_vertex<S>(f, X0 + ix, Y0 + iy, Z0 + j, a, p);
      } else {
        edge_vertex<S>(f, X0 + ix, Y0 + iy, Z0 + j, a, p);
      }
      epos[i][0] = p[0];
      epos[i][1] = p[1];
      epos[i][2] = p[2];
    }
    if (ix >= TX || iy >= TY || j >= TZ) continue;
    const int x = ix + 1, y = iy + 1;  // code row / mask row of the own row
    const RowBits& r = wb[ix][iy];
    const int64_t qid = (int64_t)qb[ix][iy] + row_prefix(r, j) + __popc(row_flags(r, j) & ((1 << a) - 1));
    const int type = a + 3 * ((cw[x][y][j + 1] >> 8) & 1);  // raw corner 0 of the owner cell
    int4 rid = make_int4(0, 0, 0, 0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int q = g_dmc_quad[4 * type + k];
      const int ox = (q & 3) - 1, oy = ((q >> 2) & 3) - 1, oz = ((q >> 4) & 3) - 1;
      const int nx = x + ox, ny = y + oy, nz = j + 1 + oz;
      const int64_t id = (int64_t)pb[nx][ny] + ppatch(nx, ny, nz) + dmc_patch_of(dmc_case(rcode(nx, ny, nz)), q >> 8) - vsub;
      quads[4 * qid + k] = id;
      // the record orders the cells by their steps back (db, dc) along axes a+1, a+2
      const int db = -(a == 0 ? oy : (a == 1 ? oz : ox)), dc = -(a == 0 ? oz : (a == 1 ? ox : oy));
      const int at = db + 2 * dc;
      rid.x = at == 0 ? (int)id : rid.x;
      rid.y = at == 1 ? (int)id : rid.y;
      rid.z = at == 2 ? (int)id : rid.z;
      rid.w = at == 3 ? (int)id : rid.w;
    }
    if (rec.loc) {
      rec.loc[qid] = pack_loc(X0 + ix, Y0 + iy, Z0 + j, a);
      reinterpret_cast<int4*>(rec.ids)[qid] = rid;
    }
  }
  __syncthreads();
  // window slot of the edge along a owned by edge-row cell (x, y, j), j in [0, TZ]
  auto wslot = [&](int x, int y, int j, int a) -> int {
    const int w = wcell[x][y][j];
    return (w & 0x1fff) + __popc((w >> 13) & ((1 << a) - 1));
  };
  // dual vertices: mean of the patch's edge vertices, edges in ascending id
  // (create_dmc_verts_kernel, src/cudualmc.cu:907-955); a patch's edges come from the
  // per-code patch masks
  for (uint32_t i = threadIdx.x; i < nci; i += blockDim.x) {
    int ix, iy, j, q;
    item_decode(pitems[i], ix, iy, j, q);
    const int x = ix + 1, y = iy + 1, X = X0 + ix, Y = Y0 + iy, Z = Z0 + j;
    const int rc = cw[x][y][j + 1];
    uint32_t m = (uint32_t)(__ldg(&g_dmc_pmask.m[rc & 0xff]) >> (12 * q)) & 0xfffu;
    const int64_t p = (int64_t)pb[x][y] + (rc >> 9) + q;
    const int cnt = __popc(m);
    S acc[3] = {S(0), S(0), S(0)};
    while (m) {
      const int e = __ffs(m) - 1;
      m &= m - 1;
      const int ge = edge_desc(e), s = ge & 7, ax = ge >> 3;
      S v[3];
      if (cached) {
        const int k = wslot(ix + (s & 1), iy + ((s >> 1) & 1), j + ((s >> 2) & 1), ax);
        v[0] = epos[k][0];
        v[1] = epos[k][1];
        v[2] = epos[k][2];
      } else {
        edge_vertex<S>(f, X + (s & 1), Y + ((s >> 1) & 1), Z + ((s >> 2) & 1), ax, v);
      }
      acc[0] += v[0];
      acc[1] += v[1];
      acc[2] += v[2];
    }
    const S inv = recip<S>(cnt);  // S(1) / S(cnt)
    const S v[3] = {acc[0] * inv, acc[1] * inv, acc[2] * inv};
    store_vertex<S>(verts, p, v, g, normalize);
    if (rec.aux) rec.aux[p] = (uint8_t)(cnt | (q << 4));
  }
  __syncthreads();  // the shared arrays are reused by the CTA's next tile
}

template <class S, class F = Field<S>>
__global__ void __launch_bounds__(NTHREADS, 4) dmc_emit_kernel(F f, Geom g, const uint64_t* __restrict__ seg,
                                                               const CellRec* __restrict__ codes,
                                                               const int* __restrict__ active,
                                                               const unsigned long long* __restrict__ n_active,
                                                               S* __restrict__ verts, int64_t* __restrict__ quads,
                                                               int normalize, void* record, int64_t vcap,
                                                               int64_t fcap, Stats* stats, const ZeroJob zj) {
  __shared__ __align__(128) uint4 zbuf[ZBUF / 16];
  __shared__ int64_t next;
  if (zj.rounds) zero_block_init(zbuf);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int64_t it = 0;  // tiles of this CTA, one zero round each
  if (emit_fits<DMC>(g, seg, vcap, fcap, stats)) {
    const EdgeRecord<S> rec = grid_record<S, DMC>(record, g, seg);
    const int64_t n = (int64_t)*n_active;
#pragma unroll 1
    for (;; ++it) {
      if (threadIdx.x == 0) next = (int64_t)atomicAdd(&stats->emit_tile, 1ull);
      __syncthreads();
      const int64_t t = next;
      __syncthreads();
      if (t >= n) break;
      if (warp == 1) zero_round(zj, zbuf, it, lane);
      dmc_emit_tile<S>(f, g, seg, codes, active[t], verts, quads, normalize, 0, rec);
    }
  }
  __syncthreads();
  if (warp == 1) zero_finish(zj, zbuf, it, lane);
}

// ------------------------------------------------------------------ backward

// explicitly rounded product and fused multiply-add: the same rounding wherever the
// compiler inlines them
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// dL/dverts of vertex i in padded coordinates: the chain rule of "- 1" and "/ (dim - 1)"
template <class S>
__device__ __forceinline__ void load_grad(const S* __restrict__ gv, int64_t i, const S scale[3], S out[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = mul_rn(__ldg(gv + 3 * i + k), scale[k]);
}

// the adjoint arithmetic of edge_adjoint2 from the end points' values d0, d1 and
// deforms q0, q1
template <class S>
__device__ __forceinline__ void edge_adjoint_math(S iso, int X, int Y, int Z, int a, S d0, S d1, const S q0[3],
                                                  const S q1[3], const S gvec[3], S c0[4], S c1[4]) {
  const int ex = a == 0, ey = a == 1, ez = a == 2;
  S t = S(0.5);
  if (d1 != d0) {
    S r = (iso - d0) / (d1 - d0);
    r = S(0) > r ? S(0) : r;
    t = r < S(1) ? r : S(1);
  }
  const S dp[3] = {(S(X + ex) + q1[0]) - (S(X) + q0[0]), (S(Y + ey) + q1[1]) - (S(Y) + q0[1]),
                   (S(Z + ez) + q1[2]) - (S(Z) + q0[2])};
  const S adj_t = fma_rn(dp[2], gvec[2], fma_rn(dp[1], gvec[1], mul_rn(dp[0], gvec[0])));
  const S den = (d1 - d0) * (d1 - d0);
  const S w0 = S(1) - t;
  // rounded products: the backward's two forms (the adjoints stored, then added
  // per point; or added where they are computed) must not fuse them into the sums
  c0[0] = mul_rn((iso - d1) / den, adj_t);
  c1[0] = mul_rn((d0 - iso) / den, adj_t);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    c0[k + 1] = mul_rn(w0, gvec[k]);
    c1[k + 1] = mul_rn(t, gvec[k]);
  }
}

// adjoint of edge_vertex (adjComputeMcVert, src/cumc.cu:412-453) for the edge from
// padded point A along axis a: c0 = (dL/dsdf, dL/ddeform) at A, c1 at A + e_a
template <class S>
__device__ __forceinline__ void edge_adjoint2(const Field<S>& f, int X, int Y, int Z, int a, const S gvec[3], S c0[4],
                                              S c1[4]) {
  const int ex = a == 0, ey = a == 1, ez = a == 2;
  // both end points' values and deforms loaded together from clamped addresses, the
  // pad value (and a zero deform) selected afterwards for points outside the grid
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
  const S d0 = in0 ? v0 : f.pad, d1 = in1 ? v1 : f.pad;
  edge_adjoint_math<S>(f.iso, X, Y, Z, a, d0, d1, q0, q1, gvec, c0, c1);
}

// whether forward tile k = (dx, dy, dz) of point tile (x0, y0, z0) (the tile one step
// further by (dx, dy, dz)) owns a crossing edge that can touch the point tile (the
// backward bits that count_chunk writes after the tiles' emit flags)
__device__ __forceinline__ int ptile_flag(const Geom& g, const uint8_t* __restrict__ tile_flag, int x0, int y0, int z0,
                                          int k) {
  const int tx = x0 / TX + (k & 1), ty = y0 / TY + ((k >> 1) & 1), tz = z0 / TZ + (k >> 2);
  if (tx >= g.tiles_x() || ty >= g.tiles_y() || tz >= g.nzc) return 0;
  return (tile_flag[g.ntiles() + ((int64_t)tx * g.tiles_y() + ty) * g.nzc + tz] >> k) & 1;
}

// zero dL/dsdf and dL/ddeform of a point tile with one warp: per row (x, y) of the
// tile, 8 lanes write the row's 32 gradient values and 24 lanes its 96 deform
// gradients as float4 when the rows are 16-byte aligned
template <class S>
__device__ __forceinline__ void zero_ptile_warp(const Field<S>& f, S* __restrict__ gsdf, S* __restrict__ gdef, int x0,
                                                int y0, int z0) {
  const int lane = threadIdx.x & 31;
  const int nz = min(TZ, f.n2 - z0);
  if (sizeof(S) == 4 && (f.n2 & 3) == 0 && (((uintptr_t)gsdf | (uintptr_t)gdef) & 15u) == 0) {
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
    for (int q = 0; q < TX * TY; ++q) {
      const int x = x0 + q / TY, y = y0 + q % TY;
      if (x >= f.n0 || y >= f.n1) continue;
      const int64_t base = ((int64_t)x * f.n1 + y) * f.n2 + z0;
      if (lane < 8) {
        if (4 * lane < nz) reinterpret_cast<float4*>(gsdf + base)[lane] = z4;
      } else if (gdef && 4 * (lane - 8) < 3 * nz) {
        reinterpret_cast<float4*>(gdef + 3 * base)[lane - 8] = z4;
      }
    }
    return;
  }
  for (int q = 0; q < TX * TY; ++q) {
    const int x = x0 + q / TY, y = y0 + q % TY;
    if (x >= f.n0 || y >= f.n1) continue;
    const int64_t base = ((int64_t)x * f.n1 + y) * f.n2 + z0;
    if (lane < nz) gsdf[base + lane] = S(0);
    if (gdef)
      for (int k = lane; k < 3 * nz; k += 32) gdef[3 * base + k] = S(0);
  }
}

__device__ __forceinline__ void ptile_coords(int64_t tile, const Geom& g, int& x0, int& y0, int& z0) {
  const int tz = (int)(tile % g.ptiles_z());
  const int64_t r = tile / g.ptiles_z();
  y0 = (int)(r % g.ptiles_y()) * TY;
  x0 = (int)(r / g.ptiles_y()) * TX;
  z0 = tz * TZ;
}

// The backward runs in two passes.
//
// Edge pass: one thread per crossing edge of the record.  The gradient reaching the
// edge's lerp vertex: MC, dL/dverts of that vertex (adj_create_cell_mc_verts_kernel,
// src/cumc.cu:474-512); DMC, the sum over the four cells around the edge of
// dL/d(dual vertex) / (edges in that patch) (adj_create_dmc_verts_kernel,
// src/cudualmc.cu:957-1005), where the reference reads the gradient of the cell's
// first patch for every patch of the cell (adj_verts[first] with first never
// advanced, src/cudualmc.cu:990): exact = 0 reproduces that, exact = 1 uses each
// patch's own gradient (the true derivative).  Its adjoint at both end points
// (adjComputeMcVert, src/cumc.cu:412-453) goes to the record's adj slots.
//
// Point pass: every point tile; each point adds the adjoints of its (at most six)
// crossing edges in a fixed order, so the result is deterministic without atomics,
// and every gradient element is written once (zeros away from the surface).  This
// replaces the forward re-run, the zero fills and the F.pad backward of
// diso/__init__.py:30-44, 84-98.

template <class S>
__device__ __forceinline__ void store_adj(S* __restrict__ adj, int64_t q, const S c0[4], const S c1[4]) {
  S* o = adj + 8 * q;
  if constexpr (sizeof(S) == 4) {
    reinterpret_cast<float4*>(o)[0] = make_float4(c0[0], c0[1], c0[2], c0[3]);
    reinterpret_cast<float4*>(o)[1] = make_float4(c1[0], c1[1], c1[2], c1[3]);
  } else {
    reinterpret_cast<double2*>(o)[0] = make_double2(c0[0], c0[1]);
    reinterpret_cast<double2*>(o)[1] = make_double2(c0[2], c0[3]);
    reinterpret_cast<double2*>(o)[2] = make_double2(c1[0], c1[1]);
    reinterpret_cast<double2*>(o)[3] = make_double2(c1[2], c1[3]);
  }
}

// adds adjoint slot k (0: the edge's first point, 1: its second) of edge q to acc
template <class S>
__device__ __forceinline__ void add_adj(const S* __restrict__ adj, int64_t q, int k, S acc[4]) {
  const S* o = adj + 8 * q + 4 * k;
  if constexpr (sizeof(S) == 4) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(o));
    acc[0] += v.x;
    acc[1] += v.y;
    acc[2] += v.z;
    acc[3] += v.w;
  } else {
    const double2 u = __ldg(reinterpret_cast<const double2*>(o)), w = __ldg(reinterpret_cast<const double2*>(o) + 1);
    acc[0] += u.x;
    acc[1] += u.y;
    acc[2] += w.x;
    acc[3] += w.y;
  }
}

// edge pass for edge q of the record; vbase = the grid's first vertex (batches)
template <class S, int METHOD>
__device__ __forceinline__ void edge_adjoint_at(const Field<S>& f, const EdgeRecord<S>& r, int64_t q, int64_t vbase,
                                                const S* __restrict__ gv, const S scale[3], int exact) {
  int X, Y, Z, a;
  unpack_loc(__ldg(r.loc + q), X, Y, Z, a);
  S gvec[3];
  if constexpr (METHOD == MC) {
    load_grad<S>(gv, q, scale, gvec);  // the edge's vertex has the edge's index
  } else {
    const int4 id4 = __ldg(reinterpret_cast<const int4*>(r.ids) + q);
    const int id[4] = {id4.x, id4.y, id4.z, id4.w};
    gvec[0] = gvec[1] = gvec[2] = S(0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t p = vbase + id[k];
      const unsigned x = __ldg(r.aux + p);
      const S inv = recip<S>((int)(x & 15u));
      S v[3];
      load_grad<S>(gv, exact ? p : p - (int64_t)(x >> 4), scale, v);
      gvec[0] = fma_rn(v[0], inv, gvec[0]);
      gvec[1] = fma_rn(v[1], inv, gvec[1]);
      gvec[2] = fma_rn(v[2], inv, gvec[2]);
    }
  }
  S c0[4], c1[4];
  edge_adjoint2<S>(f, X, Y, Z, a, gvec, c0, c1);
  store_adj<S>(r.adj, q, c0, c1);
}

template <class S>
__device__ __forceinline__ void grad_scale(const Geom& g, int normalize, S scale[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) scale[k] = normalize ? S(1) / S(g.n[k] - 1) : S(1);
}

// edge pass of one grid: E and V from the scanned total of the per-call record
template <class S, int METHOD>
__global__ void __launch_bounds__(256) edge_adjoint_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg,
                                                           void* record, const S* __restrict__ gv, int normalize,
                                                           int exact) {
  const int64_t E = Counts::lo(seg[g.nseg]);
  const EdgeRecord<S> r = grid_record<S, METHOD>(record, g, seg);
  S scale[3];
  grad_scale<S>(g, normalize, scale);
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < E; q += (int64_t)gridDim.x * blockDim.x)
    edge_adjoint_at<S, METHOD>(f, r, q, 0, gv, scale, exact);
}

// Point tiles: unpadded points [x0, x0+TX) x [y0, y0+TY) x [z0, z0+TZ); in padded
// coordinates the points are (X0+1.., Y0+1.., Z0+1..) with (X0, Y0, Z0) = (x0, y0, z0),
// and the cells [X0, X0+TX] x [Y0, Y0+TY] x [Z0, Z0+TZ] own every edge that touches
// them.  Those cells lie in the forward tiles (x0/TX + {0,1}, y0/TY + {0,1},
// z0/TZ + {0,1}); the point tile is inactive when none of them owns a crossing edge
// among the cells that can touch it (ptile_flag).  gather_tile handles an active
// tile; adj: the record's adjoints, indexed by the scanned crossing counts of seg.
template <class S>
__device__ __forceinline__ void gather_tile(const Field<S>& f, const Geom& g, const uint64_t* __restrict__ seg,
                                            int64_t ptile, const S* __restrict__ adj, S* __restrict__ gsdf,
                                            S* __restrict__ gdef) {
  constexpr int WX = TX + 2, WY = TY + 2;  // point rows [X0, X0+TX+1] x [Y0, Y0+TY+1]
  constexpr int CX = TX + 1, CY = TY + 1;  // cell rows [X0, X0+TX] x [Y0, Y0+TY]
  __shared__ uint64_t m[WX][WY];
  __shared__ uint32_t b0[CX][CY], b1[CX][CY];  // first edge of the cell row's chunks zc and zc + 1
  __shared__ uint32_t eb[CX][CY][TZ + 1];      // first edge of each window cell
  __shared__ uint8_t ef[CX][CY][TZ + 1];       // its crossing flags (bit a: the edge along a)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int X0, Y0, Z0;
  ptile_coords(ptile, g, X0, Y0, Z0);
  const int zc = Z0 / TZ;
  // segment bases first, so that their loads overlap the mask loads
  uint64_t sv = 0;
  const int si = threadIdx.x, sk = si & 1, sy = (si >> 1) % CY, sx = (si >> 1) / CY;
  if (si < CX * CY * 2) {
    const int X = X0 + sx, Y = Y0 + sy, c = zc + sk;
    if (X < g.c[0] && Y < g.c[1] && c < g.nzc) sv = seg[g.seg(X, Y, c)];
  }
  S dmn, dmx;
  bool dseen = false;
  load_masks<S, WX, WY, false>(m, f, X0, Y0, Z0, dmn, dmx, dseen);
  if (si < CX * CY * 2) {
    if (sk) b1[sx][sy] = Counts::lo(sv);
    else b0[sx][sy] = Counts::lo(sv);
  }
  __syncthreads();
  // per window cell: crossing flags and the index of its first crossing edge (one
  // warp per cell row, lane j for cell j, lane 31 also for cell TZ)
  const uint32_t valid = zvalid(g, Z0);
  for (int r = warp; r < CX * CY; r += NTHREADS / 32) {
    const int x = r / CY, y = r % CY;
    RowBits rw = {0u, 0u, 0u, 0u};
    int f32 = 0;
    if (X0 + x < g.c[0] && Y0 + y < g.c[1]) {
      rw = row_bits(m[x][y], m[x + 1][y], m[x][y + 1], m[x + 1][y + 1], valid);
      if (Z0 + TZ < g.c[2]) f32 = flags_at(m[x][y], m[x + 1][y], m[x][y + 1], TZ + 1);
    }
    eb[x][y][lane] = b0[x][y] + (uint32_t)row_prefix(rw, lane);
    ef[x][y][lane] = (uint8_t)row_flags(rw, lane);
    if (lane == 31) {
      eb[x][y][TZ] = b1[x][y];
      ef[x][y][TZ] = (uint8_t)f32;
    }
  }
  __syncthreads();
#pragma unroll
  for (int ix = 0; ix < TX; ++ix) {
    const int x = ix + 1, y = warp + 1, j = lane + 1;
    S acc[4] = {S(0), S(0), S(0), S(0)};
    // per axis the edge from this point (first point), then the edge ending here
    const int fo = ef[x][y][j], fx = ef[x - 1][y][j], fy = ef[x][y - 1][j], fz = ef[x][y][j - 1];
    const uint32_t bo = eb[x][y][j];
    if (fo & 1) add_adj<S>(adj, bo, 0, acc);
    if (fx & 1) add_adj<S>(adj, eb[x - 1][y][j], 1, acc);
    if (fo & 2) add_adj<S>(adj, bo + (fo & 1), 0, acc);
    if (fy & 2) add_adj<S>(adj, eb[x][y - 1][j] + (fy & 1), 1, acc);
    if (fo & 4) add_adj<S>(adj, bo + __popc(fo & 3), 0, acc);
    if (fz & 4) add_adj<S>(adj, eb[x][y][j - 1] + __popc(fz & 3), 1, acc);
    const int X = X0 + 1 + ix, Y = Y0 + 1 + warp, Z = Z0 + 1 + lane;
    if (f.inside(X, Y, Z)) {
      const int64_t i = f.lin(X, Y, Z);
      gsdf[i] = acc[0];
      if (gdef) {
        gdef[3 * i + 0] = acc[1];
        gdef[3 * i + 1] = acc[2];
        gdef[3 * i + 2] = acc[3];
      }
    }
  }
  __syncthreads();  // the shared arrays are reused by the CTA's next tile
}

// The point pass in two parts that run side by side: the point tiles with no
// crossing nearby (most of them) only get zeros, written by independent warps on a
// second stream while the edge pass and the gather of the active tiles run.

// zeros of the inactive point tiles, one warp per tile (persistent)
template <class S>
__global__ void __launch_bounds__(256) zero_tiles_kernel(Field<S> f, Geom g, const uint8_t* __restrict__ tile_flag,
                                                         S* __restrict__ gsdf, S* __restrict__ gdef) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < g.nptiles(); p += nw) {
    int x0, y0, z0;
    ptile_coords(p, g, x0, y0, z0);
    const int a = lane < 8 ? ptile_flag(g, tile_flag, x0, y0, z0, lane) : 0;
    if (!__any_sync(0xffffffffu, a)) zero_ptile_warp<S>(f, gsdf, gdef, x0, y0, z0);
  }
}

// the list of active point tiles (any order)
__global__ void __launch_bounds__(256) active_ptiles_kernel(Geom g, const uint8_t* __restrict__ tile_flag,
                                                            int* __restrict__ list, unsigned* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  const int64_t n = g.nptiles();
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = base + threadIdx.x;
    bool act = false;
    if (p < n) {
      int x0, y0, z0;
      ptile_coords(p, g, x0, y0, z0);
#pragma unroll
      for (int k = 0; k < 8; ++k) act = act || ptile_flag(g, tile_flag, x0, y0, z0, k) != 0;
    }
    const unsigned m = __ballot_sync(0xffffffffu, act);
    unsigned at = 0;
    if (lane == 0 && m) at = atomicAdd(count, (unsigned)__popc(m));
    at = __shfl_sync(0xffffffffu, at, 0);
    if (act) list[at + __popc(m & ((1u << lane) - 1u))] = (int)p;
  }
}

// dL/d(isovalue) of an extraction, which the reference does not give (its isovalue is
// a plain scalar, diso/__init__.py:48, 102): minus the sum of dL/dsdf over the grid.
// Moving the isovalue by e moves every crossing exactly as moving every grid value by
// -e (the pad value isovalue + 1 moves with the isovalue), and the lerp's adjoints of
// an edge's two ends, (iso - d1) / (d1 - d0)^2 adj_t and (d0 - iso) / (d1 - d0)^2 adj_t
// (src/cumc.cu:412-453), sum to minus the isovalue's, adj_t / (d1 - d0).  A pad end's
// adjoint, dropped from dL/dsdf, is that end's share of the pad value's own term, so
// the grid's points alone give the isovalue's.
//
// Partial sums in double, one per CTA, over a static assignment of point tiles (warp
// w of the grid takes tiles w, w + W, ...); with the forward's tile flags the tiles
// with no crossing nearby (their gradients are zeros) are skipped.  The reductions
// run in a fixed order, so the result repeats bit for bit.
constexpr int ISO_GRAD_CTAS = 512;

template <class S>
__global__ void __launch_bounds__(256) iso_grad_partial_kernel(Geom g, const uint8_t* __restrict__ tile_flag,
                                                               const S* __restrict__ gsdf,
                                                               double* __restrict__ partial) {
  __shared__ double wsum[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nw = (int64_t)gridDim.x * 8;
  double acc = 0.0;
  for (int64_t p = (int64_t)blockIdx.x * 8 + warp; p < g.nptiles(); p += nw) {
    int x0, y0, z0;
    ptile_coords(p, g, x0, y0, z0);
    if (tile_flag) {
      const int a = lane < 8 ? ptile_flag(g, tile_flag, x0, y0, z0, lane) : 0;
      if (!__any_sync(0xffffffffu, a)) continue;
    }
    const int z = z0 + lane;
    if (z >= g.n[2]) continue;
    for (int q = 0; q < TX * TY; ++q) {
      const int x = x0 + q / TY, y = y0 + q % TY;
      if (x < g.n[0] && y < g.n[1]) acc += (double)gsdf[((int64_t)x * g.n[1] + y) * g.n[2] + z];
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) wsum[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += wsum[w];
    partial[blockIdx.x] = t;
  }
}

// the partial sums in a fixed order; out = -(their sum)
__global__ void __launch_bounds__(256) iso_grad_final_kernel(const double* __restrict__ partial, int n,
                                                             double* __restrict__ out) {
  __shared__ double wsum[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) wsum[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += wsum[w];
    *out = -t;
  }
}

// gather of the active point tiles in the list (persistent)
template <class S>
__global__ void __launch_bounds__(NTHREADS, sizeof(S) == 4 ? 4 : 3) gather_list_kernel(Field<S> f, Geom g, const uint64_t* __restrict__ seg,
                                                               const int* __restrict__ list,
                                                               const unsigned* __restrict__ count,
                                                               const void* __restrict__ record, S* __restrict__ gsdf,
                                                               S* __restrict__ gdef) {
  const unsigned n = *count;
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x)
    gather_tile<S>(f, g, seg, list[i], (const S*)record, gsdf, gdef);
}

// ------------------------------------------------------------------ batch emit / backward

// MC: low half = vertices, high half = triangles; DMC: low = quads, high = patches
template <int METHOD>
__device__ __forceinline__ int64_t count_verts(uint64_t v) {
  return METHOD == MC ? Counts::lo(v) : Counts::hi(v);
}
template <int METHOD>
__device__ __forceinline__ int64_t count_faces(uint64_t v) {
  return METHOD == MC ? Counts::hi(v) : Counts::lo(v);
}

// whether grid G's outputs fit the batch's capacities (vcap vertices, fcap faces)
template <class S, int METHOD>
__device__ __forceinline__ bool batch_fits(const BatchGrid<S>& G, int64_t vcap, int64_t fcap) {
  const uint64_t b1 = *G.seg_end;
  return count_verts<METHOD>(b1) <= vcap && count_faces<METHOD>(b1) <= fcap;
}

// Emit every active tile of a batch (persistent).  Outputs are concatenated in grid
// order; faces hold grid-local vertex ids.  When a grid's outputs would pass the
// capacities (vcap vertices, fcap faces) the grid is skipped and bit 1 of
// stats[0].error is set; the host then retries with larger buffers.  The edge
// record (optional) is laid out for the capacities.
template <class S, int METHOD>
__global__ void __launch_bounds__(NTHREADS) batch_emit_kernel(const BatchGrid<S>* __restrict__ grids,
                                                              const int* __restrict__ active,
                                                              const unsigned long long* __restrict__ n_active,
                                                              S* __restrict__ verts, int64_t* __restrict__ faces,
                                                              int64_t vcap, int64_t fcap, int normalize,
                                                              Stats* stats, EdgeRecord<S> rec) {
  const int64_t n = (int64_t)*n_active;
#pragma unroll 1
  for (int64_t t = blockIdx.x; t < n; t += gridDim.x) {
    const int code = active[t];
    const int i = (int)((unsigned)code >> BATCH_TILE_BITS), tile = code & ((1 << BATCH_TILE_BITS) - 1);
    const BatchGrid<S>& G = grids[i];
    if (!batch_fits<S, METHOD>(G, vcap, fcap)) {
      if (threadIdx.x == 0) atomicOr(&stats->error, 2ull);
      continue;
    }
    const int64_t v0 = count_verts<METHOD>(*G.seg);
    if (METHOD == MC)
      mc_emit_tile<S>(G.f, G.g, G.seg, tile, verts, faces, normalize, v0, rec);
    else
      dmc_emit_tile<S>(G.f, G.g, G.seg, G.codes, tile, verts, faces, normalize, v0, rec);
  }
}

// edge pass over every edge of a batch (persistent); grids that did not fit the
// capacities were not emitted and are skipped
template <class S, int METHOD>
__global__ void __launch_bounds__(256) batch_edge_adjoint_kernel(const BatchGrid<S>* __restrict__ grids, int ngrids,
                                                                 EdgeRecord<S> r, int64_t vcap, int64_t fcap,
                                                                 const S* __restrict__ gv, int normalize,
                                                                 int exact) {
  __shared__ int64_t estart[MAX_BATCH], vstart[MAX_BATCH];
  __shared__ uint8_t fits[MAX_BATCH];
  for (int i = threadIdx.x; i < ngrids; i += blockDim.x) {
    const uint64_t b0 = *grids[i].seg;
    estart[i] = Counts::lo(b0);
    vstart[i] = count_verts<METHOD>(b0);
    fits[i] = batch_fits<S, METHOD>(grids[i], vcap, fcap) ? 1 : 0;
  }
  __syncthreads();
  const int64_t E = Counts::lo(*grids[ngrids - 1].seg_end);
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < E; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = batch_find(estart, ngrids, q);
    if (!fits[i]) continue;
    const BatchGrid<S>& G = grids[i];
    S scale[3];
    grad_scale<S>(G.g, normalize, scale);
    edge_adjoint_at<S, METHOD>(G.f, r, q, vstart[i], gv, scale, exact);
  }
}

// point pass of a batch over the flattened point tiles: zeros of the inactive tiles
// (and of every tile of a grid that did not fit the capacities), one warp per tile
template <class S, int METHOD>
__global__ void __launch_bounds__(256) batch_zero_tiles_kernel(const BatchGrid<S>* __restrict__ grids, int ngrids,
                                                               int64_t ntiles, int64_t vcap, int64_t fcap) {
  __shared__ int64_t start[MAX_BATCH];
  __shared__ uint8_t fits[MAX_BATCH];
  for (int i = threadIdx.x; i < ngrids; i += blockDim.x) {
    start[i] = grids[i].ptile0;
    fits[i] = batch_fits<S, METHOD>(grids[i], vcap, fcap) ? 1 : 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles; t += nw) {
    const int i = batch_find(start, ngrids, t);
    const BatchGrid<S>& G = grids[i];
    int x0, y0, z0;
    ptile_coords(t - start[i], G.g, x0, y0, z0);
    const int a = (fits[i] && lane < 8) ? ptile_flag(G.g, G.tile_flag, x0, y0, z0, lane) : 0;
    if (!__any_sync(0xffffffffu, a)) zero_ptile_warp<S>(G.f, G.gsdf, G.gdef, x0, y0, z0);
  }
}

// the list of active flattened point tiles of a batch (grids that fit the capacities)
template <class S, int METHOD>
__global__ void __launch_bounds__(256) batch_active_ptiles_kernel(const BatchGrid<S>* __restrict__ grids, int ngrids,
                                                                  int64_t ntiles, int64_t vcap, int64_t fcap,
                                                                  int* __restrict__ list,
                                                                  unsigned* __restrict__ count) {
  __shared__ int64_t start[MAX_BATCH];
  __shared__ uint8_t fits[MAX_BATCH];
  for (int i = threadIdx.x; i < ngrids; i += blockDim.x) {
    start[i] = grids[i].ptile0;
    fits[i] = batch_fits<S, METHOD>(grids[i], vcap, fcap) ? 1 : 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < ntiles; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = base + threadIdx.x;
    bool act = false;
    if (t < ntiles) {
      const int i = batch_find(start, ngrids, t);
      if (fits[i]) {
        const BatchGrid<S>& G = grids[i];
        int x0, y0, z0;
        ptile_coords(t - start[i], G.g, x0, y0, z0);
#pragma unroll
        for (int k = 0; k < 8; ++k) act = act || ptile_flag(G.g, G.tile_flag, x0, y0, z0, k) != 0;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, act);
    unsigned at = 0;
    if (lane == 0 && m) at = atomicAdd(count, (unsigned)__popc(m));
    at = __shfl_sync(0xffffffffu, at, 0);
    if (act) list[at + __popc(m & ((1u << lane) - 1u))] = (int)t;
  }
}

// gather of the listed point tiles of a batch (persistent)
template <class S>
__global__ void __launch_bounds__(NTHREADS) batch_gather_list_kernel(const BatchGrid<S>* __restrict__ grids,
                                                                     int ngrids, const int* __restrict__ list,
                                                                     const unsigned* __restrict__ count,
                                                                     const void* __restrict__ record) {
  __shared__ int64_t start[MAX_BATCH];
  for (int i = threadIdx.x; i < ngrids; i += blockDim.x) start[i] = grids[i].ptile0;
  __syncthreads();
  const unsigned n = *count;
  for (unsigned k = blockIdx.x; k < n; k += gridDim.x) {
    const int64_t t = list[k];
    const int i = batch_find(start, ngrids, t);
    const BatchGrid<S>& G = grids[i];
    gather_tile<S>(G.f, G.g, G.seg, t - start[i], (const S*)record, G.gsdf, G.gdef);
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
    // the cosine of the normalised edges (the reference normalises each edge, its
    // norm clamped at 1e-12, then takes the dot product) from reciprocal square roots
    // of the squared norms (clamped at 1e-24), without divisions: the same value up
    // to rounding, so the split can differ only where the two configurations' cosines
    // tie to within it (FP64 divisions and square roots are slow on this GPU)
    S q1 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
    S q2 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
    q1 = q1 > S(1e-24) ? q1 : S(1e-24);
    q2 = q2 > S(1e-24) ? q2 : S(1e-24);
    const S c = (e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2]) * rsqrt(q1) * rsqrt(q2);
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
