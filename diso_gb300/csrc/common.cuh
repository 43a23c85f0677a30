// Shared device code of the GB300 iso-surface extractor: grid geometry with the
// virtual one-voxel pad, shared-memory point windows, cube-case codes, the case
// tables, and warp/block reductions.
//
// Geometry.  The caller's SDF is an unpadded [N0][N1][N2] array (z fastest).  The
// reference pads it by one voxel on every side with isovalue+1 and the deform by
// zeros (diso/__init__.py:52-54) and then works on the padded grid of
// P = N + 2 points per axis, whose cells are (X, Y, Z) in [0, N+1)^3
// (src/cumc.cu:265-297).  Here the pad is never materialised: Field::at() returns
// the pad value outside [1, N] in padded coordinates.
//
// Row segments.  Cells are ordered as in the reference (x-major, z fastest,
// src/cumc.h:101-105), so the reference's vertex, face and patch numbering is
// "exclusive prefix over cells in that order".  Each row (X, Y) of cells is cut
// into chunks of 32 cells; a segment (X, Y, chunk) is the unit of the scan, and
// the global index of a cell's first output is the scanned base of its segment
// plus the prefix of the cell inside the segment.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "case_tables.h"

namespace diso {

constexpr int TZ = 32;        // cells per tile along z (one per lane)
// count units: CP x CR rows of cells, runs of at most KZ 32-cell chunks
constexpr int CP = 8, CR = 32, KZ = 4;
constexpr int TY = 8;         // rows per tile along y (one per warp)
constexpr int TX = 4;         // planes per tile along x (per-thread loop)
constexpr int NTHREADS = 32 * TY;

// packed per-segment / scan value: low 32 bits vertices (MC crossings, DMC patches
// are in the high half), see Counts
struct Counts {
  __host__ __device__ static uint64_t pack(uint32_t lo, uint32_t hi) { return (uint64_t)lo | ((uint64_t)hi << 32); }
  __host__ __device__ static uint32_t lo(uint64_t v) { return (uint32_t)v; }
  __host__ __device__ static uint32_t hi(uint64_t v) { return (uint32_t)(v >> 32); }
};

struct Geom {
  int n[3];      // unpadded points per axis
  int c[3];      // cells per axis = n + 1
  int nzc;       // 32-cell chunks per row
  int64_t nseg;  // c0 * c1 * nzc
  __host__ __device__ void init(int n0, int n1, int n2) {
    n[0] = n0; n[1] = n1; n[2] = n2;
    c[0] = n0 + 1; c[1] = n1 + 1; c[2] = n2 + 1;
    nzc = (c[2] + TZ - 1) / TZ;
    nseg = (int64_t)c[0] * c[1] * nzc;
  }
  __host__ __device__ int64_t seg(int X, int Y, int zc) const { return ((int64_t)X * c[1] + Y) * nzc + zc; }
  // byte of cell (X, Y, Z) in the array of cell codes (rows padded to whole chunks)
  __host__ __device__ int64_t code(int X, int Y, int Z) const { return ((int64_t)X * c[1] + Y) * (nzc * TZ) + Z; }
  __host__ __device__ int64_t ncodes() const { return (int64_t)c[0] * c[1] * nzc * TZ; }
  // tiles of cells for the forward passes
  __host__ __device__ int tiles_x() const { return (c[0] + TX - 1) / TX; }
  __host__ __device__ int tiles_y() const { return (c[1] + TY - 1) / TY; }
  __host__ __device__ int64_t ntiles() const { return (int64_t)tiles_x() * tiles_y() * nzc; }
  // tiles of (unpadded) points for the backward pass
  __host__ __device__ int ptiles_x() const { return (n[0] + TX - 1) / TX; }
  __host__ __device__ int ptiles_y() const { return (n[1] + TY - 1) / TY; }
  __host__ __device__ int ptiles_z() const { return (n[2] + TZ - 1) / TZ; }
  __host__ __device__ int64_t nptiles() const { return (int64_t)ptiles_x() * ptiles_y() * ptiles_z(); }
};

template <class S>
struct Field {
  static constexpr bool kDense = true;  // a grid in memory (fields.cuh has evaluated ones)
  static constexpr int kGrad = 0;       // the backward writes dense dL/dsdf (fields.cuh: 1 spheres, 2 bricks)
  const S* __restrict__ sdf;
  const S* __restrict__ def;  // [N0][N1][N2][3] or null
  int n0, n1, n2;
  S iso, pad;
  // value at padded point (X, Y, Z); the pad value outside the caller's grid
  __device__ __forceinline__ S at(int X, int Y, int Z) const {
    unsigned x = (unsigned)(X - 1), y = (unsigned)(Y - 1), z = (unsigned)(Z - 1);
    if (x < (unsigned)n0 && y < (unsigned)n1 && z < (unsigned)n2) return __ldg(sdf + ((int64_t)x * n1 + y) * n2 + z);
    return pad;
  }
  __device__ __forceinline__ bool inside(int X, int Y, int Z) const {
    return (unsigned)(X - 1) < (unsigned)n0 && (unsigned)(Y - 1) < (unsigned)n1 && (unsigned)(Z - 1) < (unsigned)n2;
  }
  __device__ __forceinline__ int64_t lin(int X, int Y, int Z) const {
    return ((int64_t)(X - 1) * n1 + (Y - 1)) * n2 + (Z - 1);
  }
  // position of cell (X, Y, Z)'s DMC record (rows padded to whole chunks); the per-tile
  // table and per-unit slot forms are the same here (fields.cuh: a narrow band's differ)
  __device__ __forceinline__ int64_t rec_index(const Geom& g, int X, int Y, int Z) const { return g.code(X, Y, Z); }
  struct RecTab {};
  __device__ __forceinline__ void rec_tab_fill(RecTab&, const Geom&, int, int, int, int) const {}
  __device__ __forceinline__ int64_t rec_index_tab(const RecTab&, const Geom& g, int X, int Y, int Z) const {
    return g.code(X, Y, Z);
  }
  __device__ __forceinline__ int64_t rec_index_slot(int, const Geom& g, int X, int Y, int Z) const {
    return g.code(X, Y, Z);
  }
  // unpadded point (x, y, z) of a row in the grid whose first point is at `off`
  __device__ __forceinline__ S point(int64_t off, int, int, int z) const { return __ldg(sdf + off + z); }
  // deform at padded point (zero in the pad)
  __device__ __forceinline__ void deform(int X, int Y, int Z, S d[3]) const {
    if (def && inside(X, Y, Z)) {
      const S* p = def + 3 * lin(X, Y, Z);
      d[0] = __ldg(p); d[1] = __ldg(p + 1); d[2] = __ldg(p + 2);
    } else {
      d[0] = d[1] = d[2] = S(0);
    }
  }
};

// ----------------------------------------------------------------- case codes

__device__ const uint64_t g_mc_tri[256] = DISO_MC_TRIANGLES;
__device__ const uint64_t g_dmc_case[256] = DISO_DMC_CASES;
__device__ const int g_dmc_quad[24] = DISO_DMC_QUADS;

__device__ __forceinline__ uint64_t mc_tri(int code) { return __ldg(g_mc_tri + code); }
__device__ __forceinline__ uint64_t dmc_case(int code) { return __ldg(g_dmc_case + code); }
__device__ __forceinline__ int dmc_dir(uint64_t w) { return (int)((w >> 28) & 7); }
__device__ __forceinline__ int dmc_npatch(uint64_t w) { return (int)((w >> 24) & 7); }
__device__ __forceinline__ int dmc_patch_of(uint64_t w, int e) { return (int)((w >> (2 * e)) & 3); }

// MC case code (corner order of src/cumc.cu:107) from the Morton code: swap corners 2<->3, 6<->7
__device__ __forceinline__ int mc_from_morton(int m) {
  return (m & 0x33) | ((m & 0x44) << 1) | ((m & 0x88) >> 1);
}

// crossing flags of a cell's three owned edges (+x, +y, +z from its corner 0);
// the reference tests (d0 < iso && d1 >= iso) || (d1 < iso && d0 >= iso)
// (src/cumc.cu:334-339), i.e. the two corner bits differ.  Flipping all bits of a
// code (DMC ambiguity resolution) leaves the flags unchanged.
__device__ __forceinline__ int cross_flags(int m) {
  return ((m ^ (m >> 1)) & 1) | (((m ^ (m >> 2)) & 1) << 1) | (((m ^ (m >> 4)) & 1) << 2);
}

// The twelve cell edges (DISO_EDGE_TABLE: start corner | axis << 3, in the
// reference's edge order), packed 5 bits each so that edge_desc(e) needs no load.
namespace detail {
constexpr int kEdgeTable[12] = DISO_EDGE_TABLE;
constexpr uint64_t pack_edges(int i) {
  return i == 12 ? 0ull : (((uint64_t)kEdgeTable[i] << (5 * i)) | pack_edges(i + 1));
}
}  // namespace detail
constexpr uint64_t kEdgePack = detail::pack_edges(0);
__device__ __forceinline__ int edge_desc(int e) { return (int)((kEdgePack >> (5 * e)) & 31); }

// ----------------------------------------------------------------- reductions

__device__ __forceinline__ uint64_t warp_sum64(uint64_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// inclusive scan across the warp
__device__ __forceinline__ uint32_t warp_incl(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}
__device__ __forceinline__ uint64_t warp_incl64(uint64_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// order-preserving unsigned key of a double (for atomicMin/atomicMax)
__device__ __forceinline__ unsigned long long ord_key(double d) {
  unsigned long long u = (unsigned long long)__double_as_longlong(d);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
inline double key_to_double(unsigned long long k) {
  unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  memcpy(&d, &u, 8);
  return d;
}

// status words shared by every kernel of one call
struct Stats {
  unsigned long long min_key;   // order key of min(sdf)
  unsigned long long max_key;   // order key of max(sdf)
  unsigned long long n_active;  // active forward tiles
  unsigned long long error;     // bit 0: scan look-back gave up, bit 1: output capacity exceeded,
                                // bit 2: a TMA wait gave up, bit 3: the fused backward found an
                                // index outside the forward's counts
  unsigned long long scan_tile; // dynamic tile counter of the look-back scan
  unsigned long long emit_tile; // dynamic tile counter of the emit
  unsigned long long total;      // the segment scan's total (the forward's counts)
  unsigned long long units;      // next unit of the TMA count (a grid-wide counter)
  unsigned long long sum_lo;     // the count's two halves summed in 64 bits (crossings; triangles /
  unsigned long long sum_hi;     //   patches): the scan's 32-bit halves hold them only below 2^32
};

}  // namespace diso
