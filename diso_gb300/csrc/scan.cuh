// Single-pass exclusive scan of packed 64-bit counts with decoupled look-back.
//
// Replaces the reference's three cub::DeviceScan::ExclusiveSum calls
// (src/cumc.cu:668-672, 688-692, 717-721; src/cudualmc.cu:1075-1079, 1095-1099,
// 1114-1118).  Both 32-bit halves of each element are summed at once (neither
// half can carry: a grid has fewer than 2^31 crossings).
//
// a[0..n) are the inputs; on return a[i] holds the exclusive prefix for every
// i <= n, so a[n] is the total (a must have n + 1 slots).  Tiles are taken in
// launch order from a dynamic counter, so every predecessor of a tile has started
// before it looks back; each wait is bounded and, when it gives up, sets bit 0 of
// Stats::error and the host reports the failure.
#pragma once
#include "common.cuh"

namespace diso {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 16;  // a thread's elements: 128 contiguous bytes
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr unsigned SCAN_SPIN_LIMIT = 1u << 22;  // look-back polls per predecessor (64 ns sleeps), the default

struct ScanState {
  uint32_t* flag;   // 0 none, 1 aggregate published, 2 inclusive prefix published
  uint64_t* agg;
  uint64_t* incl;
};

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// total_out (may be null) also receives the total a[n]; spin_limit bounds the polls
// of each predecessor's flag
__global__ void __launch_bounds__(SCAN_THREADS) scan_lookback_kernel(uint64_t* __restrict__ a, int64_t n,
                                                                     ScanState st, Stats* stats,
                                                                     uint64_t* total_out, unsigned spin_limit) {
  __shared__ uint64_t warp_tot[SCAN_THREADS / 32];
  __shared__ uint64_t tile_excl;
  __shared__ int64_t tile_id_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) tile_id_s = (int64_t)atomicAdd(&stats->scan_tile, 1ull);
  __syncthreads();
  const int64_t tile = tile_id_s;
  const int64_t base = tile * SCAN_TILE + (int64_t)tid * SCAN_ITEMS;

  // whole tiles of a 16-byte aligned array move as 16-byte vectors
  const bool whole = (tile + 1) * SCAN_TILE <= n && ((uintptr_t)a & 15u) == 0;
  uint64_t v[SCAN_ITEMS];
  if (whole) {
    const ulonglong2* p = reinterpret_cast<const ulonglong2*>(a + base);
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS / 2; ++i) {
      const ulonglong2 w = p[i];
      v[2 * i] = w.x;
      v[2 * i + 1] = w.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      const int64_t k = base + i;
      v[i] = (k < n) ? a[k] : 0ull;
    }
  }
  uint64_t sum = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) sum += v[i];
  // block exclusive scan of the thread sums
  uint64_t incl = warp_incl64(sum);
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  uint64_t wbase = 0, agg = 0;
#pragma unroll
  for (int w = 0; w < SCAN_THREADS / 32; ++w) {
    uint64_t t = warp_tot[w];
    if (w < warp) wbase += t;
    agg += t;
  }
  const uint64_t texcl = wbase + incl - sum;

  if (warp == 0) {
    if (tile == 0) {
      if (lane == 0) {
        __stcg(st.incl, agg);
        st_release(st.flag, 2u);
        tile_excl = 0;
      }
    } else {
      if (lane == 0) {
        __stcg(st.agg + tile, agg);
        st_release(st.flag + tile, 1u);
      }
      uint64_t excl = 0;
      int64_t pred = tile - 1;
      bool failed = false;
      while (true) {
        const int64_t idx = pred - lane;
        uint32_t f = 2u;
        uint64_t val = 0;
        if (idx >= 0) {
          unsigned spins = 0;
          while ((f = ld_acquire(st.flag + idx)) == 0u) {
            if (++spins >= spin_limit) {
              failed = true;
              break;
            }
            __nanosleep(64);
          }
          if (f != 0u) val = (f == 2u) ? __ldcg(st.incl + idx) : __ldcg(st.agg + idx);
        }
        const unsigned full = __ballot_sync(0xffffffffu, f == 2u);
        const int stop = full ? (__ffs(full) - 1) : 32;
        excl += warp_sum64(lane <= stop ? val : 0ull);
        if (__any_sync(0xffffffffu, failed)) {
          if (lane == 0) atomicOr(&stats->error, 1ull);
          break;
        }
        if (full) break;
        pred -= 32;
      }
      if (lane == 0) {
        __stcg(st.incl + tile, excl + agg);
        st_release(st.flag + tile, 2u);
        tile_excl = excl;
      }
    }
  }
  __syncthreads();
  uint64_t run = tile_excl + texcl;
  if (whole) {
    ulonglong2* p = reinterpret_cast<ulonglong2*>(a + base);
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS / 2; ++i) {
      ulonglong2 w;
      w.x = run;
      run += v[2 * i];
      w.y = run;
      run += v[2 * i + 1];
      p[i] = w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      const int64_t k = base + i;
      if (k <= n) a[k] = run;
      if (k == n && total_out) *total_out = run;
      run += v[i];
    }
  }
}

// the status words of a forward (min key at its maximum, everything else zero) and
// the look-back flags of its segment scan, in one launch
__global__ void __launch_bounds__(256) count_prep_kernel(Stats* stats, uint32_t* __restrict__ scan_flag,
                                                         int64_t tiles) {
  if (threadIdx.x == 0) {
    Stats z = {};
    z.min_key = ~0ull;
    *stats = z;
  }
  for (int64_t i = threadIdx.x; i < tiles; i += blockDim.x) scan_flag[i] = 0u;
}

// Set-up of the look-back wait probe (diso_scan_wait_probe): fresh status words, the
// flags of `tiles` tiles cleared, and the scan's tile counter at `first`, so that the
// tiles before `first` are never run and never publish their flags
__global__ void scan_probe_prep_kernel(Stats* stats, uint32_t* __restrict__ scan_flag, int64_t tiles,
                                       unsigned long long first) {
  if (threadIdx.x == 0) {
    Stats z = {};
    z.min_key = ~0ull;
    z.scan_tile = first;
    *stats = z;
  }
  for (int64_t i = threadIdx.x; i < tiles; i += blockDim.x) scan_flag[i] = 0u;
}

}  // namespace diso
