// Fields evaluated where the extractor needs their values, instead of a dense grid
// read from HBM: the caller side of the extraction (the reference evaluates its SDF
// on a full meshgrid in PyTorch and passes the dense [N, N, N] tensor,
// test/example.py:8-16, 33-53).  A field type has the interface of Field<S> that the
// forward kernels use (at, inside, deform, point, iso, pad, n0..n2) and, for the
// count, a classification of whole chunks, so that chunks far from the surface are
// never evaluated.
#pragma once
#include "common.cuh"

namespace diso {

// Union of spheres: value(p) = min_k (|p - c_k| - r_k) at grid point
// p = lo + step * (x, y, z) (unpadded indices), in the dtype's arithmetic; the pad
// value outside the grid, as for a dense grid.  The reference's example field is one
// sphere (SphereSDF, test/example.py:8-16).
template <class S>
struct SphereField {
  static constexpr bool kDense = false;
  static constexpr int kGrad = 1;  // point gradients go to the spheres' parameters
  const S* __restrict__ sph;  // [K][4]: centre x, y, z, radius
  const S* __restrict__ def;  // [N0][N1][N2][3] or null: the deform, a dense input as for Field
  int K;
  S lo[3], step[3];
  int n0, n1, n2;
  S iso, pad;

  __device__ __forceinline__ S value(int x, int y, int z) const {
    const S px = lo[0] + step[0] * (S)x, py = lo[1] + step[1] * (S)y, pz = lo[2] + step[2] * (S)z;
    S m = S(INFINITY);
    for (int k = 0; k < K; ++k) {
      const S dx = px - __ldg(sph + 4 * k), dy = py - __ldg(sph + 4 * k + 1), dz = pz - __ldg(sph + 4 * k + 2);
      const S d = sqrt(dx * dx + dy * dy + dz * dz) - __ldg(sph + 4 * k + 3);
      m = d < m ? d : m;
    }
    return m;
  }
  __device__ __forceinline__ bool inside(int X, int Y, int Z) const {
    return (unsigned)(X - 1) < (unsigned)n0 && (unsigned)(Y - 1) < (unsigned)n1 && (unsigned)(Z - 1) < (unsigned)n2;
  }
  // value at padded point (X, Y, Z); the pad value outside the grid
  __device__ __forceinline__ S at(int X, int Y, int Z) const { return inside(X, Y, Z) ? value(X - 1, Y - 1, Z - 1) : pad; }
  __device__ __forceinline__ int64_t rec_index(const Geom& g, int X, int Y, int Z) const { return g.code(X, Y, Z); }
  struct RecTab {};
  __device__ __forceinline__ void rec_tab_fill(RecTab&, const Geom&, int, int, int, int) const {}
  __device__ __forceinline__ int64_t rec_index_tab(const RecTab&, const Geom& g, int X, int Y, int Z) const {
    return g.code(X, Y, Z);
  }
  __device__ __forceinline__ int64_t rec_index_slot(int, const Geom& g, int X, int Y, int Z) const {
    return g.code(X, Y, Z);
  }
  // unpadded point (x, y, z) of a row in the grid (the row offset is not used)
  __device__ __forceinline__ S point(int64_t, int x, int y, int z) const { return value(x, y, z); }
  // deform at padded point (zero in the pad)
  __device__ __forceinline__ void deform(int X, int Y, int Z, S d[3]) const {
    if (def && inside(X, Y, Z)) {
      const S* p = def + 3 * (((int64_t)(X - 1) * n1 + (Y - 1)) * n2 + (Z - 1));
      d[0] = __ldg(p); d[1] = __ldg(p + 1); d[2] = __ldg(p + 2);
    } else {
      d[0] = d[1] = d[2] = S(0);
    }
  }
  // the sphere attaining value() at unpadded point (x, y, z) (the first of equal
  // minima, as value() keeps it) and the point's offset from its centre
  __device__ __forceinline__ int argmin(int x, int y, int z, S off[3]) const {
    const S px = lo[0] + step[0] * (S)x, py = lo[1] + step[1] * (S)y, pz = lo[2] + step[2] * (S)z;
    S m = S(INFINITY);
    int best = 0;
    for (int k = 0; k < K; ++k) {
      const S dx = px - __ldg(sph + 4 * k), dy = py - __ldg(sph + 4 * k + 1), dz = pz - __ldg(sph + 4 * k + 2);
      const S d = sqrt(dx * dx + dy * dy + dz * dz) - __ldg(sph + 4 * k + 3);
      if (d < m) {
        m = d;
        best = k;
        off[0] = dx;
        off[1] = dy;
        off[2] = dz;
      }
    }
    return best;
  }

  // value() over the spheres in `cand` only (bit k: sphere k; all of them when
  // `all`): the same value when the others cannot be the minimum (classify_warp)
  __device__ __forceinline__ S value_of(int x, int y, int z, uint64_t cand, bool all) const {
    if (all) return value(x, y, z);
    const S px = lo[0] + step[0] * (S)x, py = lo[1] + step[1] * (S)y, pz = lo[2] + step[2] * (S)z;
    S m = S(INFINITY);
    while (cand) {
      const int k = __ffsll((long long)cand) - 1;
      cand &= cand - 1;
      const S dx = px - __ldg(sph + 4 * k), dy = py - __ldg(sph + 4 * k + 1), dz = pz - __ldg(sph + 4 * k + 2);
      const S d = sqrt(dx * dx + dy * dy + dz * dz) - __ldg(sph + 4 * k + 3);
      m = d < m ? d : m;
    }
    return m;
  }

  // The points with unpadded indices in [x0, x1] x [y0, y1] x [z0, z1] (the part in
  // the grid; `pads`: some of the box lies outside it), by the calling warp (one
  // sphere per lane): cls = 1 when every value is >= iso (the pad value is), 0 when
  // every value is < iso and none is a pad, -1 otherwise; `bound` a value on the
  // box's side of iso for 1 and 0; `cand` the spheres that can be the minimum
  // somewhere in the box (`all`: every sphere, for more than 64).  From bounds of
  // each sphere's distance over the box with a margin (1e-4 of the coordinates'
  // scale) far above the rounding of value().
  __device__ __forceinline__ int classify_warp(int x0, int x1, int y0, int y1, int z0, int z1, bool pads, S& bound,
                                               uint64_t& cand, bool& all) const {
    const int lane = threadIdx.x & 31;
    all = K > 64;
    cand = 0;
    if (x0 > x1 || y0 > y1 || z0 > z1) return 1;  // only pad points
    S bmin[3], bmax[3];
    const int i0[3] = {x0, y0, z0}, i1[3] = {x1, y1, z1};
    S scale = fabs(iso) + S(1);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const S u = lo[a] + step[a] * (S)i0[a], v = lo[a] + step[a] * (S)i1[a];
      bmin[a] = u < v ? u : v;
      bmax[a] = u < v ? v : u;
      scale += fabs(bmin[a]) + fabs(bmax[a]);
    }
    S lo_k[2] = {S(INFINITY), S(INFINITY)};  // this lane's spheres lane, lane + 32 (the first 64)
    S fmin_lo = S(INFINITY), fmax_hi = S(INFINITY), rmax = S(0);
    for (int k = lane; k < K; k += 32) {
      S dn = S(0), df = S(0);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const S c = __ldg(sph + 4 * k + a);
        const S near = c < bmin[a] ? bmin[a] - c : (c > bmax[a] ? c - bmax[a] : S(0));
        const S far = fabs(c - bmin[a]) > fabs(c - bmax[a]) ? fabs(c - bmin[a]) : fabs(c - bmax[a]);
        dn += near * near;
        df += far * far;
      }
      const S r = __ldg(sph + 4 * k + 3);
      const S l = sqrt(dn) - r, h = sqrt(df) - r;
      if (k < 64) lo_k[k >> 5] = l;
      fmin_lo = l < fmin_lo ? l : fmin_lo;
      fmax_hi = h < fmax_hi ? h : fmax_hi;
      rmax = fabs(r) > rmax ? fabs(r) : rmax;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const S a = __shfl_xor_sync(0xffffffffu, fmin_lo, o), b = __shfl_xor_sync(0xffffffffu, fmax_hi, o);
      const S c = __shfl_xor_sync(0xffffffffu, rmax, o);
      fmin_lo = a < fmin_lo ? a : fmin_lo;
      fmax_hi = b < fmax_hi ? b : fmax_hi;
      rmax = c > rmax ? c : rmax;
    }
    const S margin = S(1e-4) * (scale + rmax);
    if (fmin_lo >= iso + margin) {
      bound = fmin_lo;
      return 1;
    }
    if (!pads && fmax_hi < iso - margin) {
      bound = fmax_hi;
      return 0;
    }
    // a sphere whose lower bound lies above the smallest upper bound is never the minimum
    const uint32_t c0 = __ballot_sync(0xffffffffu, lane < K && lo_k[0] <= fmax_hi + margin);
    const uint32_t c1 = __ballot_sync(0xffffffffu, lane + 32 < K && lo_k[1] <= fmax_hi + margin);
    cand = (uint64_t)c0 | ((uint64_t)c1 << 32);
    return -1;
  }
};

// ------------------------------------------------------------------ narrow band

constexpr int BRICK = 8;                          // points per brick edge
constexpr int BRICK_PTS = BRICK * BRICK * BRICK;  // 512
constexpr int BRICK_OUT = -1, BRICK_IN = -2;      // index entries of absent bricks

// A narrow band: the grid's values only in the 8^3-point bricks near the surface.
// index[bx][by][bz] (ceil(n / 8) bricks per axis) is the brick's slot in
// val [K][8][8][8] (z fastest), or BRICK_OUT / BRICK_IN for an absent brick, whose
// points read +bg / -bg.  Its values are those of the dense grid with those numbers
// in the absent bricks (bricks_materialize_kernel writes it), and so are its meshes.
// The deform, when given, is [K][8][8][8][3] (zero in absent bricks).  The backward's
// point gradients go to the slots' points (kGrad 2), none to absent points.
template <class S>
struct BrickField {
  static constexpr bool kDense = false;
  static constexpr int kGrad = 2;
  const int* __restrict__ index;
  const S* __restrict__ val;
  const S* __restrict__ def;
  int nb1, nb2;  // bricks along y and z
  int K;         // slots; an entry at or above K reads as absent (the forward rejects it)
  int n0, n1, n2;
  S iso, pad, bg;
  // DMC cell records, kept only for the count units that hold the surface: umap[unit]
  // is the unit's block (UNIT_RECS records) in the records' array, -1 for the others
  // (the units of field_count_kernel: unby x unbz runs of ukz chunks per row block)
  const int* __restrict__ umap;
  int unby, unbz, ukz;
  unsigned ukz_mul;  // ceil(2^16 / ukz): chunk / ukz = chunk * ukz_mul >> 16 (ukz <= 4, chunks < 2^15)
  static constexpr int64_t UNIT_RECS = (int64_t)CP * CR * KZ * TZ;

  // offset of cell (X, Y, Z) in its unit's block, the unit along z
  __device__ __forceinline__ int64_t rec_off(int X, int Y, int Z, int& uz) const {
    uz = (int)(((unsigned)Z / TZ * ukz_mul) >> 16);
    return ((int64_t)(X % CP) * CR + Y % CR) * (KZ * TZ) + (Z - uz * ukz * TZ);
  }
  __device__ __forceinline__ int64_t rec_index(const Geom& g, int X, int Y, int Z) const {
    (void)g;
    int uz;
    const int64_t off = rec_off(X, Y, Z, uz);
    const int slot = umap[((int64_t)(X / CP) * unby + Y / CR) * unbz + uz];
    return (int64_t)(slot < 0 ? 0 : slot) * UNIT_RECS + off;  // a listed unit's block (no other is read)
  }
  // the count's form: the unit's block is known (its place in the list of units)
  __device__ __forceinline__ int64_t rec_index_slot(int slot, const Geom&, int X, int Y, int Z) const {
    int uz;
    const int64_t off = rec_off(X, Y, Z, uz);
    return (int64_t)slot * UNIT_RECS + off;
  }
  // The emit's and the backward's form: the blocks of the (at most 2 x 2 x 3) units
  // around a tile's window (cells [X0 - 1, X0 + TX] x [Y0 - 1, Y0 + TY] x [Z0 - 1,
  // Z0 + TZ]) loaded once per tile, entry i by thread i < 12, before a barrier
  struct RecTab {
    int ux0, uy0, uz0;
    int s[12];
  };
  __device__ __forceinline__ void rec_tab_fill(RecTab& t, const Geom& g, int X0, int Y0, int Z0, int i) const {
    const int ux0 = (X0 > 0 ? X0 - 1 : 0) / CP, uy0 = (Y0 > 0 ? Y0 - 1 : 0) / CR;
    const int tz = Z0 / TZ, uz0 = (int)(((unsigned)(tz > 0 ? tz - 1 : 0) * ukz_mul) >> 16);
    if (i == 0) {
      t.ux0 = ux0;
      t.uy0 = uy0;
      t.uz0 = uz0;
    }
    const int ux = ux0 + i / 6, uy = uy0 + (i / 3) % 2, uz = uz0 + i % 3;
    const int nux = (g.c[0] + CP - 1) / CP;
    t.s[i] = (ux < nux && uy < unby && uz < unbz) ? umap[((int64_t)ux * unby + uy) * unbz + uz] : -1;
  }
  __device__ __forceinline__ int64_t rec_index_tab(const RecTab& t, const Geom&, int X, int Y, int Z) const {
    int uz;
    const int64_t off = rec_off(X, Y, Z, uz);
    const int slot = t.s[(X / CP - t.ux0) * 6 + (Y / CR - t.uy0) * 3 + (uz - t.uz0)];
    return (int64_t)(slot < 0 ? 0 : slot) * UNIT_RECS + off;
  }

  __device__ __forceinline__ int entry(int x, int y, int z) const {
    const int e = __ldg(index + ((int64_t)(x >> 3) * nb1 + (y >> 3)) * nb2 + (z >> 3));
    return e < K ? e : BRICK_OUT;
  }
  __device__ __forceinline__ static int local(int x, int y, int z) {
    return ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
  }
  // position of unpadded point (x, y, z) in the slot arrays, -1 in an absent brick
  __device__ __forceinline__ int64_t slot_point(int x, int y, int z) const {
    const int e = entry(x, y, z);
    return e >= 0 ? (int64_t)e * BRICK_PTS + local(x, y, z) : -1;
  }
  __device__ __forceinline__ S value(int x, int y, int z) const {
    const int e = entry(x, y, z);
    if (e >= 0) return __ldg(val + (int64_t)e * BRICK_PTS + local(x, y, z));
    return e == BRICK_IN ? -bg : bg;
  }
  __device__ __forceinline__ bool inside(int X, int Y, int Z) const {
    return (unsigned)(X - 1) < (unsigned)n0 && (unsigned)(Y - 1) < (unsigned)n1 && (unsigned)(Z - 1) < (unsigned)n2;
  }
  __device__ __forceinline__ S at(int X, int Y, int Z) const { return inside(X, Y, Z) ? value(X - 1, Y - 1, Z - 1) : pad; }
  __device__ __forceinline__ S point(int64_t, int x, int y, int z) const { return value(x, y, z); }
  __device__ __forceinline__ S value_of(int x, int y, int z, uint64_t, bool) const { return value(x, y, z); }
  __device__ __forceinline__ void deform(int X, int Y, int Z, S d[3]) const {
    d[0] = d[1] = d[2] = S(0);
    if (def && inside(X, Y, Z)) {
      const int64_t p = slot_point(X - 1, Y - 1, Z - 1);
      if (p >= 0) {
        d[0] = __ldg(def + 3 * p);
        d[1] = __ldg(def + 3 * p + 1);
        d[2] = __ldg(def + 3 * p + 2);
      }
    }
  }

  // As SphereField::classify_warp, from the index entries of the bricks that the box
  // [x0, x1] x [y0, y1] x [z0, z1] (unpadded, in the grid) touches: -1 when one is
  // present (the box is evaluated), else the class of the absent bricks' values
  // (+bg, -bg) when they agree, with `bound` the value farthest from iso on that side.
  // Every lane of the calling warp takes part.
  __device__ __forceinline__ int classify_warp(int x0, int x1, int y0, int y1, int z0, int z1, bool pads, S& bound,
                                               uint64_t& cand, bool& all) const {
    const int lane = threadIdx.x & 31;
    cand = 0;
    all = true;
    if (x0 > x1 || y0 > y1 || z0 > z1) return 1;  // only pad points
    const int bx0 = x0 >> 3, by0 = y0 >> 3, bz0 = z0 >> 3;
    const int nx = (x1 >> 3) - bx0 + 1, ny = (y1 >> 3) - by0 + 1, nz = (z1 >> 3) - bz0 + 1;
    const int nbk = nx * ny * nz;
    bool present = false, in = false, out = false;
    // the boxes of a count unit touch at most 2 x 5 x 18 bricks: six entries per lane,
    // loaded together (a loop takes any rest)
    constexpr int PER = 6;
    int e[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int k = lane + 32 * j;
      e[j] = BRICK_OUT;
      if (k < nbk) {
        const int bz = bz0 + k % nz, r = k / nz;
        e[j] = __ldg(index + ((int64_t)(bx0 + r / ny) * nb1 + (by0 + r % ny)) * nb2 + bz);
      }
    }
    for (int k = lane + 32 * PER; k < nbk; k += 32) {
      const int bz = bz0 + k % nz, r = k / nz;
      const int v = __ldg(index + ((int64_t)(bx0 + r / ny) * nb1 + (by0 + r % ny)) * nb2 + bz);
      present = present || v >= 0;
      in = in || v == BRICK_IN;
      out = out || (v < 0 && v != BRICK_IN);
    }
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      if (lane + 32 * j < nbk) {
        present = present || e[j] >= 0;
        in = in || e[j] == BRICK_IN;
        out = out || (e[j] < 0 && e[j] != BRICK_IN);
      }
    }
    if (__any_sync(0xffffffffu, present)) return -1;
    in = __any_sync(0xffffffffu, in);
    out = __any_sync(0xffffffffu, out);
    const bool out_hi = bg >= iso, in_hi = -bg >= iso;
    const bool above = (out && out_hi) || (in && in_hi), below = (out && !out_hi) || (in && !in_hi);
    if (above && below) return -1;
    if (above) {
      bound = out ? bg : -bg;
      return 1;
    }
    if (pads) return -1;  // pad points (>= iso) beside values below it
    bound = in ? -bg : bg;
    return 0;
  }
};

// Checks of a brick index before a forward (one pass over the entries): bit 0 of
// out[0] for an entry that is neither a slot in [0, K) nor an absent tag, bit 1 for a
// slot used twice (uses[K], zeroed by the caller, counts them); out[1] += present
// bricks; out[2] += absent bricks with a 26-neighbour of the other class (value at or
// above iso / below it: an absent brick of the other tag, or the pad beyond the grid's
// edge).  A cell can cross the surface only if a corner lies in a present brick or in
// such a border brick, and 9^3 cells touch a brick, so 729 (out[1] + out[2]) bounds the
// non-trivial cells (the host checks it against the 32-bit counts).
__global__ void __launch_bounds__(256) brick_check_kernel(const int* __restrict__ index, int nb0, int nb1, int nb2,
                                                          int K, int out_hi, int in_hi, int pad_hi,
                                                          int* __restrict__ uses,
                                                          unsigned long long* __restrict__ out) {
  const int64_t n = (int64_t)nb0 * nb1 * nb2;
  unsigned long long present = 0, border = 0;
  unsigned bad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int e = index[i];
    if (e >= 0) {
      if (e >= K) {
        bad |= 1u;
      } else {
        if (atomicAdd(uses + e, 1) != 0) bad |= 2u;
        ++present;
      }
      continue;
    }
    if (e != BRICK_OUT && e != BRICK_IN) {
      bad |= 1u;
      continue;
    }
    const int hi = e == BRICK_IN ? in_hi : out_hi;
    const int bz = (int)(i % nb2);
    const int64_t r = i / nb2;
    const int by = (int)(r % nb1), bx = (int)(r / nb1);
    // the 26 neighbours' loads issued together
    bool edge = false;
#pragma unroll
    for (int d = 0; d < 27; ++d) {
      const int dx = d / 9 - 1, dy = (d / 3) % 3 - 1, dz = d % 3 - 1;
      if (d == 13) continue;
      const int x = bx + dx, y = by + dy, z = bz + dz;
      if (x < 0 || y < 0 || z < 0 || x >= nb0 || y >= nb1 || z >= nb2) {
        edge = edge || pad_hi != hi;
      } else {
        const int f = __ldg(index + ((int64_t)x * nb1 + y) * nb2 + z);
        edge = edge || (f < 0 && (f == BRICK_IN ? in_hi : out_hi) != hi);
      }
    }
    border += edge ? 1 : 0;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    present += __shfl_xor_sync(0xffffffffu, present, o);
    border += __shfl_xor_sync(0xffffffffu, border, o);
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicOr(out, (unsigned long long)bad);
    if (present) atomicAdd(out + 1, present);
    if (border) atomicAdd(out + 2, border);
  }
}

// the dense grid [n0][n1][n2] of a narrow band (and its dense deform, zero in absent
// bricks, when both are given)
template <class S>
__global__ void __launch_bounds__(256) bricks_materialize_kernel(BrickField<S> f, S* __restrict__ out,
                                                                 S* __restrict__ dout) {
  const int64_t n = (int64_t)f.n0 * f.n1 * f.n2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(i % f.n2);
    const int64_t r = i / f.n2;
    const int x = (int)(r / f.n1), y = (int)(r % f.n1);
    out[i] = f.value(x, y, z);
    if (dout) {
      S d[3];
      f.deform(x + 1, y + 1, z + 1, d);
      dout[3 * i] = d[0];
      dout[3 * i + 1] = d[1];
      dout[3 * i + 2] = d[2];
    }
  }
}

// the dense grid of a field (for callers that want it, and for checking the
// fused path against the dense one on the same values)
template <class S>
__global__ void __launch_bounds__(256) field_materialize_kernel(SphereField<S> f, S* __restrict__ out) {
  const int64_t n = (int64_t)f.n0 * f.n1 * f.n2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(i % f.n2);
    const int64_t r = i / f.n2;
    out[i] = f.value((int)(r / f.n1), (int)(r % f.n1), z);
  }
}

}  // namespace diso
