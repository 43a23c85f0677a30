// Mesh consumers on the device, for the meshes the extractor returns (vertices
// [V][3] in the grid dtype, faces [F][k] int64 with k = 3 or 4):
//
//   vertex normals  area-weighted: the sum of the (unnormalised) normals of the
//                   faces around each vertex, normalised; accumulated in 64-bit fixed
//                   point so the result does not depend on the order of the atomics
//   weld            merges vertices whose positions agree (exactly, or after rounding
//                   to a tolerance); the lowest index of each group represents it,
//                   vertices and faces keep their order, collapsed faces are dropped
//   OBJ text        "v %.8f %.8f %.8f" lines (then "vn" lines when normals are given),
//                   "f a b c[ d]" lines with 1-based indices ("a//a" with normals);
//                   the decimal digits are correctly rounded (ties to even)
//   PLY body        binary little-endian vertex block (x y z [nx ny nz]) and face
//                   block (uchar count, int32 indices)
//
// The reference writes its meshes through trimesh (test/example.py:71-73); these
// replace that host-side step for meshes that live on the GPU.
#pragma once
#include "common.cuh"

namespace diso {

// ------------------------------------------------------------------ normals

// unnormalised normal of face f (twice its vector area): triangles (p1 - p0) x
// (p2 - p0), quads (p2 - p0) x (p3 - p1); in double
template <class S>
__device__ __forceinline__ void face_normal(const S* __restrict__ v, const int64_t* __restrict__ faces, int64_t f,
                                            int k, double n[3]) {
  double p[4][3];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    if (c < k) {
      const int64_t i = faces[k * f + c];
#pragma unroll
      for (int d = 0; d < 3; ++d) p[c][d] = (double)v[3 * i + d];
    }
  }
  double a[3], b[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    a[d] = k == 3 ? p[1][d] - p[0][d] : p[2][d] - p[0][d];
    b[d] = k == 3 ? p[2][d] - p[0][d] : p[3][d] - p[1][d];
  }
  n[0] = a[1] * b[2] - a[2] * b[1];
  n[1] = a[2] * b[0] - a[0] * b[2];
  n[2] = a[0] * b[1] - a[1] * b[0];
}

// whether every corner index of face f lies in [0, nv)
__device__ __forceinline__ bool face_ok(const int64_t* __restrict__ faces, int64_t f, int k, int64_t nv) {
  bool ok = true;
  for (int c = 0; c < k; ++c) ok = ok && (uint64_t)faces[k * f + c] < (uint64_t)nv;
  return ok;
}

// largest |component| of any face normal, as the bits of a non-negative double;
// faces with an index out of range set bit 3 of *err and are left out (here and
// in the accumulation)
template <class S>
__global__ void __launch_bounds__(256) normals_max_kernel(const S* __restrict__ v, const int64_t* __restrict__ faces,
                                                          int64_t nf, int k, int64_t nv, unsigned long long* maxbits,
                                                          unsigned long long* err) {
  double m = 0.0;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    if (!face_ok(faces, f, k, nv)) {
      atomicOr(err, 8ull);
      continue;
    }
    double n[3];
    face_normal<S>(v, faces, f, k, n);
    m = fmax(m, fmax(fabs(n[0]), fmax(fabs(n[1]), fabs(n[2]))));
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
}

// 2^50 / (largest component): every face adds at most 2^50 per component, so 2^13
// faces around one vertex stay inside 64 bits
__device__ __forceinline__ double normals_scale(const unsigned long long* maxbits) {
  const double m = __longlong_as_double((long long)*maxbits);
  return m > 0.0 ? 1125899906842624.0 / m : 0.0;
}

template <class S>
__global__ void __launch_bounds__(256) normals_acc_kernel(const S* __restrict__ v, const int64_t* __restrict__ faces,
                                                          int64_t nf, int k, int64_t nv, const unsigned long long* maxbits,
                                                          unsigned long long* __restrict__ acc) {
  const double scale = normals_scale(maxbits);
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    if (!face_ok(faces, f, k, nv)) continue;
    double n[3];
    face_normal<S>(v, faces, f, k, n);
    long long q[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) q[d] = llrint(n[d] * scale);
    for (int c = 0; c < k; ++c) {
      const int64_t i = faces[k * f + c];
#pragma unroll
      for (int d = 0; d < 3; ++d) atomicAdd(acc + 3 * i + d, (unsigned long long)q[d]);
    }
  }
}

template <class S>
__global__ void __launch_bounds__(256) normals_out_kernel(const unsigned long long* __restrict__ acc, int64_t nv,
                                                          S* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    double s[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) s[d] = (double)(long long)acc[3 * i + d];
    const double len = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
#pragma unroll
    for (int d = 0; d < 3; ++d) out[3 * i + d] = len > 0.0 ? (S)(s[d] / len) : S(0);
  }
}

// ------------------------------------------------------------------ weld

// the key of vertex i: its coordinates in double (exact weld, tol = 0; -0 counts as
// +0) or floor(x / tol + 0.5) per coordinate
struct WeldKey {
  long long k[3];
};

template <class S>
__device__ __forceinline__ WeldKey weld_key(const S* __restrict__ v, int64_t i, double tol) {
  WeldKey w;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double x = (double)v[3 * i + d];
    w.k[d] = tol > 0.0 ? (long long)floor(x / tol + 0.5) : __double_as_longlong(x == 0.0 ? 0.0 : x);
  }
  return w;
}

__device__ __forceinline__ bool same_key(const WeldKey& a, const WeldKey& b) {
  return a.k[0] == b.k[0] && a.k[1] == b.k[1] && a.k[2] == b.k[2];
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ uint64_t key_hash(const WeldKey& w) {
  return mix64((uint64_t)w.k[0] ^ mix64((uint64_t)w.k[1] ^ mix64((uint64_t)w.k[2])));
}

// open-addressing table of `mask + 1` slots (at least twice the vertices, -1 empty):
// each key's slot ends up holding the lowest index with that key.  Every probe
// sequence ends: the table is never more than half full.
template <class S>
__global__ void __launch_bounds__(256) weld_insert_kernel(const S* __restrict__ v, int64_t nv, double tol,
                                                          int* __restrict__ table, uint32_t mask) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    const WeldKey w = weld_key<S>(v, i, tol);
    uint32_t h = (uint32_t)key_hash(w) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
      int s = table[h];
      if (s < 0) {
        s = atomicCAS(table + h, -1, (int)i);
        if (s < 0) break;  // inserted
      }
      if (same_key(weld_key<S>(v, s, tol), w)) {
        atomicMin(table + h, (int)i);
        break;
      }
    }
  }
}

// rep[i] = the lowest index with i's key; keep[i] = 1 for those
template <class S>
__global__ void __launch_bounds__(256) weld_rep_kernel(const S* __restrict__ v, int64_t nv, double tol,
                                                       const int* __restrict__ table, uint32_t mask,
                                                       int* __restrict__ rep, uint64_t* __restrict__ keep) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    const WeldKey w = weld_key<S>(v, i, tol);
    uint32_t h = (uint32_t)key_hash(w) & mask;
    int r = (int)i;
    for (uint32_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
      const int s = table[h];
      if (s < 0) break;  // not reached: i itself was inserted
      if (same_key(weld_key<S>(v, s, tol), w)) {
        r = s;
        break;
      }
    }
    rep[i] = r;
    keep[i] = r == (int)i ? 1ull : 0ull;
  }
}

// faces through rep and the scanned keep flags (new index of a kept vertex); a face
// whose corners are not all distinct afterwards collapses (keepf = 0), and so does
// a face with an index out of range (bit 3 of *err)
__global__ void __launch_bounds__(256) weld_faces_kernel(const int64_t* __restrict__ faces, int64_t nf, int k,
                                                         int64_t nv, const int* __restrict__ rep,
                                                         const uint64_t* __restrict__ vidx,
                                                         int64_t* __restrict__ mapped, uint64_t* __restrict__ keepf,
                                                         unsigned long long* err) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    if (!face_ok(faces, f, k, nv)) {
      atomicOr(err, 8ull);
      keepf[f] = 0ull;
      continue;
    }
    int64_t m[4] = {0, 0, 0, 0};
    for (int c = 0; c < k; ++c) m[c] = (int64_t)vidx[rep[faces[k * f + c]]];
    bool ok = true;
    for (int a = 0; a < k; ++a)
      for (int b = a + 1; b < k; ++b) ok = ok && m[a] != m[b];
    for (int c = 0; c < k; ++c) mapped[k * f + c] = m[c];
    keepf[f] = ok ? 1ull : 0ull;
  }
}

template <class S>
__global__ void __launch_bounds__(256) weld_compact_verts_kernel(const S* __restrict__ v, int64_t nv,
                                                                 const int* __restrict__ rep,
                                                                 const uint64_t* __restrict__ vidx, S* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    if (rep[i] != (int)i) continue;
    const int64_t o = (int64_t)vidx[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) out[3 * o + d] = v[3 * i + d];
  }
}

__global__ void __launch_bounds__(256) weld_compact_faces_kernel(const int64_t* __restrict__ mapped, int64_t nf, int k,
                                                                 const uint64_t* __restrict__ fidx,
                                                                 int64_t* __restrict__ out) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    if (fidx[f + 1] == fidx[f]) continue;  // collapsed
    const int64_t o = (int64_t)fidx[f];
    for (int c = 0; c < k; ++c) out[k * o + c] = mapped[k * f + c];
  }
}

// ------------------------------------------------------------------ OBJ text

// |x| * 10^8 rounded to the nearest integer, ties to even, from the exact product
// p + e (p the rounded product, e its error from an FMA; e = 0 for float32, whose
// 24 significant bits times the 19 of 10^8 fit a double).  Below 2^53 rint(p) is
// the nearest integer to p, the even one when p lies halfway, and e only decides
// the ties of p; above, p is an even integer and e adds its own nearest integer.
// Valid for |x| < 1.8e11.
template <class S>
__device__ __forceinline__ unsigned long long fixed8(S x) {
  const double a = fabs((double)x);
  const double p = a * 1e8;
  const double e = fma(a, 1e8, -p);
  if (p >= 9007199254740992.0) return (unsigned long long)p + (unsigned long long)(long long)rint(e);
  double r = rint(p);
  const double d = p - r;  // exact
  if (d == 0.5 && e > 0.0) r += 1.0;
  else if (d == -0.5 && e < 0.0) r -= 1.0;
  return (unsigned long long)r;
}

// decimal digits of u (at least one) written backwards from `end`; returns the count
__device__ __forceinline__ int put_uint_rev(char* end, unsigned long long u) {
  int n = 0;
  do {
    *--end = (char)('0' + (int)(u % 10ull));
    u /= 10ull;
    ++n;
  } while (u);
  return n;
}

__device__ __forceinline__ int uint_len(unsigned long long u) {
  int n = 1;
  while (u >= 10ull) {
    u /= 10ull;
    ++n;
  }
  return n;
}

// length of "%.8f" of x (nan / inf / -inf spelled as Python does)
template <class S>
__device__ __forceinline__ int fixed8_len(S x) {
  const double xd = (double)x;
  if (isnan(xd)) return 3;
  if (isinf(xd)) return xd < 0 ? 4 : 3;
  const unsigned long long r = fixed8<S>(x);
  return (signbit(xd) ? 1 : 0) + uint_len(r / 100000000ull) + 9;
}

template <class S>
__device__ __forceinline__ char* put_fixed8(char* o, S x) {
  const double xd = (double)x;
  if (isnan(xd)) {
    o[0] = 'n'; o[1] = 'a'; o[2] = 'n';
    return o + 3;
  }
  if (isinf(xd)) {
    if (xd < 0) *o++ = '-';
    o[0] = 'i'; o[1] = 'n'; o[2] = 'f';
    return o + 3;
  }
  const unsigned long long r = fixed8<S>(x);
  if (signbit(xd)) *o++ = '-';
  const unsigned long long ip = r / 100000000ull, fp = r % 100000000ull;
  const int n = uint_len(ip);
  put_uint_rev(o + n, ip);
  o += n;
  *o++ = '.';
  unsigned long long f = fp;
  for (int d = 7; d >= 0; --d) {
    o[d] = (char)('0' + (int)(f % 10ull));
    f /= 10ull;
  }
  return o + 8;
}

// line lengths: vertex lines "v x y z\n" (and "vn ...\n" lines after them), then face
// lines; len[] holds one entry per line, scanned into offsets afterwards
template <class S>
__global__ void __launch_bounds__(256) obj_len_kernel(const S* __restrict__ v, const S* __restrict__ nrm, int64_t nv,
                                                      const int64_t* __restrict__ faces, int64_t nf, int k,
                                                      uint64_t* __restrict__ len) {
  const int64_t nvl = nrm ? 2 * nv : nv, total = nvl + nf;
  for (int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l < total; l += (int64_t)gridDim.x * blockDim.x) {
    int n;
    if (l < nvl) {
      const bool isn = l >= nv;
      const S* p = isn ? nrm + 3 * (l - nv) : v + 3 * l;
      n = (isn ? 3 : 2) + fixed8_len<S>(p[0]) + 1 + fixed8_len<S>(p[1]) + 1 + fixed8_len<S>(p[2]) + 1;
    } else {
      const int64_t f = l - nvl;
      n = 1;  // "f"
      for (int c = 0; c < k; ++c) {
        const int d = uint_len((unsigned long long)(faces[k * f + c] + 1));
        n += 1 + (nrm ? 2 * d + 2 : d);
      }
      n += 1;  // newline
    }
    len[l] = (uint64_t)n;
  }
}

template <class S>
__global__ void __launch_bounds__(256) obj_write_kernel(const S* __restrict__ v, const S* __restrict__ nrm, int64_t nv,
                                                        const int64_t* __restrict__ faces, int64_t nf, int k,
                                                        const uint64_t* __restrict__ off, char* __restrict__ out) {
  const int64_t nvl = nrm ? 2 * nv : nv, total = nvl + nf;
  for (int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l < total; l += (int64_t)gridDim.x * blockDim.x) {
    char* o = out + off[l];
    if (l < nvl) {
      const bool isn = l >= nv;
      const S* p = isn ? nrm + 3 * (l - nv) : v + 3 * l;
      *o++ = 'v';
      if (isn) *o++ = 'n';
      for (int d = 0; d < 3; ++d) {
        *o++ = ' ';
        o = put_fixed8<S>(o, p[d]);
      }
      *o = '\n';
    } else {
      const int64_t f = l - nvl;
      *o++ = 'f';
      for (int c = 0; c < k; ++c) {
        const unsigned long long id = (unsigned long long)(faces[k * f + c] + 1);
        const int d = uint_len(id);
        *o++ = ' ';
        put_uint_rev(o + d, id);
        o += d;
        if (nrm) {
          *o++ = '/';
          *o++ = '/';
          put_uint_rev(o + d, id);
          o += d;
        }
      }
      *o = '\n';
    }
  }
}

// ------------------------------------------------------------------ PLY body

// vertex block: per vertex x y z (and nx ny nz) in the grid dtype; then the face
// block: per face the corner count (one byte) and k little-endian int32 indices
template <class S>
__global__ void __launch_bounds__(256) ply_vertex_kernel(const S* __restrict__ v, const S* __restrict__ nrm, int64_t nv,
                                                         S* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    S* o = out + 6 * i;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      o[d] = v[3 * i + d];
      o[3 + d] = nrm[3 * i + d];
    }
  }
}

__global__ void __launch_bounds__(256) ply_face_kernel(const int64_t* __restrict__ faces, int64_t nf, int k,
                                                       uint8_t* __restrict__ out) {
  const int rec = 1 + 4 * k;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    uint8_t* o = out + rec * f;
    o[0] = (uint8_t)k;
    for (int c = 0; c < k; ++c) {
      const uint32_t id = (uint32_t)faces[k * f + c];
#pragma unroll
      for (int b = 0; b < 4; ++b) o[1 + 4 * c + b] = (uint8_t)(id >> (8 * b));
    }
  }
}

}  // namespace diso
