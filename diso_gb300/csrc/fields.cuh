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
  const S* __restrict__ sph;  // [K][4]: centre x, y, z, radius
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
  // unpadded point (x, y, z) of a row in the grid (the row offset is not used)
  __device__ __forceinline__ S point(int64_t, int x, int y, int z) const { return value(x, y, z); }
  __device__ __forceinline__ void deform(int, int, int, S d[3]) const { d[0] = d[1] = d[2] = S(0); }

  // The points with unpadded indices in [x0, x1] x [y0, y1] x [z0, z1] (the part in
  // the grid; `pads`: some of the box lies outside it): 1 when every value is >= iso
  // (the pad value is), 0 when every value is < iso and none is a pad, -1 otherwise.
  // From bounds of each sphere's distance over the box in double, with a margin far
  // above the rounding of value(); `bound` receives a value on the box's side of iso
  // (a lower bound of its values for 1, an upper bound for 0).
  __device__ __forceinline__ int classify(int x0, int x1, int y0, int y1, int z0, int z1, bool pads,
                                          double& bound) const {
    if (x0 > x1 || y0 > y1 || z0 > z1) return 1;  // only pad points
    double bmin[3], bmax[3];
    const int i0[3] = {x0, y0, z0}, i1[3] = {x1, y1, z1};
    double scale = fabs((double)iso) + 1.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double u = (double)lo[a] + (double)step[a] * i0[a], v = (double)lo[a] + (double)step[a] * i1[a];
      bmin[a] = fmin(u, v);
      bmax[a] = fmax(u, v);
      scale += fabs(bmin[a]) + fabs(bmax[a]);
    }
    double fmin_lo = INFINITY, fmax_hi = INFINITY;  // min over spheres of each one's lower / upper bound
    for (int k = 0; k < K; ++k) {
      double dn = 0.0, df = 0.0;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double c = (double)__ldg(sph + 4 * k + a);
        const double near = c < bmin[a] ? bmin[a] - c : (c > bmax[a] ? c - bmax[a] : 0.0);
        const double far = fmax(fabs(c - bmin[a]), fabs(c - bmax[a]));
        dn += near * near;
        df += far * far;
      }
      const double r = (double)__ldg(sph + 4 * k + 3);
      scale = fmax(scale, fabs(r));
      fmin_lo = fmin(fmin_lo, sqrt(dn) - r);
      fmax_hi = fmin(fmax_hi, sqrt(df) - r);
    }
    const double margin = 1e-4 * scale;
    if (fmin_lo >= (double)iso + margin) {
      bound = fmin_lo;
      return 1;
    }
    if (!pads && fmax_hi < (double)iso - margin) {
      bound = fmax_hi;
      return 0;
    }
    return -1;
  }
};

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
