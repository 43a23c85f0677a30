// Host side of the C ABI declared in include/diso_gb300.h: argument checks,
// scratch management and kernel launches on the caller's stream.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/diso_gb300.h"
#include "backward.cuh"
#include "fields.cuh"
#include "kernels.cuh"
#include "mesh.cuh"
#include "scan.cuh"

using namespace diso;

namespace {

thread_local char g_err[512] = "";

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

#define CUDA_TRY(expr)                                                                     \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess) return fail(DISO_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

// kernels timed by diso_timing
enum KernelId {
  K_COUNT, K_SCAN, K_EMIT, K_ZERO_GRADS, K_ZERO_TILES, K_ACTIVE_PTILES, K_EDGE, K_GATHER, K_SPLIT, K_FUSED_BWD,
  K_BRICK_CHECK, K_NKERNELS
};
static const char* const kKernelNames[K_NKERNELS] = {"count",       "scan", "emit",   "zero_grads", "zero_tiles",
                                                      "active_list", "edge", "gather", "split",     "fused_bwd",
                                                      "brick_check"};

struct diso_extractor {
  int method = 0, dtype = 0, device = -1;
  // optional timing of every launch (diso_timing): event pairs on the launch's stream
  struct Timed {
    int id;
    cudaEvent_t a, b;
  };
  bool timing = false;
  std::vector<Timed> timed;
  std::vector<cudaEvent_t> event_pool;
  Stats* stats = nullptr;        // device status words
  Stats* stats_host = nullptr;   // pinned mirror
  uint32_t* scan_flag = nullptr; // look-back state
  uint64_t* scan_agg = nullptr;
  uint64_t* scan_incl = nullptr;
  int64_t scan_cap = 0;          // look-back tiles
  int* active = nullptr;         // tiles with crossings (forward)
  int64_t active_cap = 0;
  CellRec* codes = nullptr;      // DMC cell records of the active segments (count -> emit)
  int64_t codes_cap = 0;
  uint64_t* split = nullptr;     // split counts (n_quads + 1)
  int64_t split_cap = 0;
  uint8_t* mesh = nullptr;       // mesh consumers' scratch (normals, weld, OBJ), bytes
  int64_t mesh_cap = 0;
  int64_t last_active = 0;       // from the last forward count
  // the `seg` and grid of the last dense DMC count, whose cell records `codes` holds
  const uint64_t* codes_seg = nullptr;
  int codes_dims[3] = {0, 0, 0};
  bool codes_band = false;       // they are a narrow band's (else a dense grid's)
  int resident_ctas = 0;         // count-kernel CTAs that fit on the device at once
  int tma_ctas = 0;              // the same for the TMA count kernel
  int gather_ctas = 0;           // the same for the point gather
  int emit_ctas = 0;             // the same for the emit
  int fused_ctas = 0;            // the same for the fused backward
  int fused_smem = 0;            // its dynamic shared memory per CTA
  int fused_smem_rec = 0;        // the same for its variant that reads the DMC cell records
  int per_sm[4] = {1, 1, 1, 1};  // resident CTAs per SM of the count (TMA), emit, gather, fused backward
  // launch widths set by diso_tune_set (0: the default), and the zeros' count share
  int tune[DISO_TUNE_N] = {};
  double zero_share = 0.35;
  int sms = 0;
  cudaStream_t side = nullptr;   // second stream of the backward (zeros of the inactive point tiles)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_zero = nullptr;  // end of the last diso_zero_grads on the side stream
  // gradient buffers of diso_zero_grads that the next count on `stream` zeroes
  struct PendingZero {
    void* p[2];
    int64_t bytes[2];
    cudaStream_t stream;
    bool set;
  } zpend = {};
  ZeroJob zemit = {};            // the emit's part of the zeros of the last count
  cudaStream_t zemit_stream = nullptr;
  bool zemit_set = false;
  cudaEvent_t ev_counts = nullptr;  // the count's results are on the host
  int* ulist = nullptr;          // an evaluated field's count units that hold the surface (count, then ids)
  int64_t ulist_cap = 0;
  int* umap = nullptr;           // a narrow band's unit -> block of DMC cell records (-1: none)
  int64_t umap_cap = 0;
  int* plist = nullptr;          // active point tiles of the backward, and their count
  int64_t plist_cap = 0;
  unsigned* plist_n = nullptr;
  double* isog = nullptr;        // per-CTA partial sums of the isovalue gradient
  int64_t isog_cap = 0;
  double* fpart = nullptr;       // per-CTA sums of a field backward's sphere gradients
  int64_t fpart_cap = 0;
  int* buses = nullptr;          // narrow band: uses of each brick slot (brick_check_kernel)
  int64_t buses_cap = 0;
  unsigned long long* bcheck = nullptr;  // its results (bad bits, present, border bricks)
  int64_t bcheck_cap = 0;
  int brick_ctas = 0;            // resident CTAs of the narrow band's backward

  // batch state (diso_batch_*): descriptors, per-grid status, layout of the record
  void* bdesc = nullptr;         // device BatchGrid<S>[MAX_BATCH]
  void* bdesc_host = nullptr;    // pinned staging
  Stats* bstats = nullptr;       // device Stats[MAX_BATCH]
  Stats* bstats_host = nullptr;
  uint64_t* bbound = nullptr;    // device: scanned value at each grid's first segment, + total
  uint64_t* bbound_host = nullptr;
  uint64_t* brecord = nullptr;   // the caller's batch record
  int bn = 0;                    // grids in the prepared batch
  int64_t bseg_total = 0, bblocks = 0, bptiles = 0, btiles = 0;
  int64_t bseg_off[MAX_BATCH + 1] = {};
  int bcount_ctas = 0, bwork_ctas = 0;

  cudaEvent_t take_event() {
    cudaEvent_t e = nullptr;
    if (!event_pool.empty()) {
      e = event_pool.back();
      event_pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
      e = nullptr;
    }
    return e;
  }

  void release_events() {
    for (const Timed& t : timed) {
      cudaEventDestroy(t.a);
      cudaEventDestroy(t.b);
    }
    for (cudaEvent_t e : event_pool) cudaEventDestroy(e);
    timed.clear();
    event_pool.clear();
  }

  void release() {
    release_events();
    cudaFree(bdesc);
    cudaFreeHost(bdesc_host);
    cudaFree(bstats);
    cudaFreeHost(bstats_host);
    cudaFree(bbound);
    cudaFreeHost(bbound_host);
    bdesc = bdesc_host = nullptr;
    bstats = bstats_host = nullptr;
    bbound = bbound_host = nullptr;
    bn = 0;
    cudaFree(stats);
    cudaFreeHost(stats_host);
    cudaFree(scan_flag);
    cudaFree(scan_agg);
    cudaFree(scan_incl);
    cudaFree(active);
    cudaFree(codes);
    codes = nullptr;
    codes_cap = 0;
    cudaFree(split);
    cudaFree(mesh);
    mesh = nullptr;
    mesh_cap = 0;
    cudaFree(plist);
    cudaFree(plist_n);
    cudaFree(isog);
    isog = nullptr;
    isog_cap = 0;
    cudaFree(fpart);
    fpart = nullptr;
    fpart_cap = 0;
    cudaFree(buses);
    buses = nullptr;
    buses_cap = 0;
    cudaFree(ulist);
    ulist = nullptr;
    ulist_cap = 0;
    cudaFree(umap);
    umap = nullptr;
    umap_cap = 0;
    cudaFree(bcheck);
    bcheck = nullptr;
    bcheck_cap = 0;
    if (side) cudaStreamDestroy(side);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_zero) cudaEventDestroy(ev_zero);
    if (ev_counts) cudaEventDestroy(ev_counts);
    side = nullptr;
    ev_fork = ev_join = ev_zero = ev_counts = nullptr;
    plist = nullptr;
    plist_n = nullptr;
    plist_cap = 0;
    stats = nullptr;
    stats_host = nullptr;
    scan_flag = nullptr;
    scan_agg = scan_incl = split = nullptr;
    active = nullptr;
    scan_cap = active_cap = split_cap = 0;
  }
};

namespace {

// brackets one launch with timing events when the extractor's timing is on
struct KernelTimer {
  diso_extractor* ex;
  int id;
  cudaStream_t s;
  cudaEvent_t a = nullptr;
  KernelTimer(diso_extractor* e, int k, cudaStream_t st) : ex(e), id(k), s(st) {
    if (ex->timing && (a = ex->take_event())) cudaEventRecord(a, s);
  }
  ~KernelTimer() {
    if (!a) return;
    cudaEvent_t b = ex->take_event();
    if (!b) {
      ex->event_pool.push_back(a);
      return;
    }
    cudaEventRecord(b, s);
    ex->timed.push_back({id, a, b});
  }
};

template <class T>
int grow(T*& p, int64_t& cap, int64_t need) {
  if (need <= cap) return DISO_OK;
  int64_t n = need + need / 4 + 1024;
  cudaFree(p);
  p = nullptr;
  cap = 0;
  CUDA_TRY(cudaMalloc((void**)&p, (size_t)n * sizeof(T)));
  cap = n;
  return DISO_OK;
}

// ------------------------------------------------------------------ launch widths

// Persistent CTAs of a kernel: `dflt` (all that fit) unless diso_tune_set chose a
// number per SM (at most the `cap` per SM that fit); every kernel's output is the
// same for any width.
inline unsigned tuned_ctas(const diso_extractor* ex, int param, int dflt, int cap) {
  const int v = ex->tune[param];
  return (unsigned)std::max(1, v > 0 ? ex->sms * std::min(v, cap) : dflt);
}
// CTAs of the kernels sized in CTAs per SM with a fixed default (zeros, edge pass, batches)
inline unsigned per_sm_ctas(const diso_extractor* ex, int param, int dflt_per_sm) {
  const int v = ex->tune[param];
  return (unsigned)std::max(1, ex->sms * (v > 0 ? v : dflt_per_sm));
}

// ------------------------------------------------------------------ TMA tensor maps

// cuTensorMapEncodeTiled from the driver, looked up once
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

// The tensor map of the SDF for the TMA count: boxes of 32 x 33 x 9 points (z
// innermost).  False when the SDF cannot be described (address not 16-byte aligned,
// rows not a multiple of 16 bytes).
template <class S>
bool count_tensor_map(const void* sdf, int nx, int ny, int nz, CUtensorMap* wide) {
  if (((uintptr_t)sdf & 15u) != 0 || ((int64_t)nz * (int64_t)sizeof(S)) % 16 != 0) return false;
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  const CUtensorMapDataType dt = sizeof(S) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  const cuuint64_t dims[3] = {(cuuint64_t)nz, (cuuint64_t)ny, (cuuint64_t)nx};
  const cuuint64_t strides[2] = {(cuuint64_t)nz * sizeof(S), (cuuint64_t)nz * ny * sizeof(S)};
  const cuuint32_t estr[3] = {1, 1, 1};
  const cuuint32_t wbox[3] = {32, (cuuint32_t)(CR + 1), (cuuint32_t)(CP + 1)};
  return enc(wide, dt, 3, const_cast<void*>(sdf), dims, strides, wbox, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// resident CTAs per SM of the TMA count kernel (sets its shared-memory size)
template <class S>
cudaError_t tma_occupancy(int method, int* per_sm) {
  const int smem = (int)count_tma_smem<S>();
  cudaError_t e;
  if (method == DISO_MC) {
    if ((e = cudaFuncSetAttribute(count_tma_kernel<S, MC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
      return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, count_tma_kernel<S, MC>, NTHREADS, smem);
  }
  if ((e = cudaFuncSetAttribute(count_tma_kernel<S, DMC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
    return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, count_tma_kernel<S, DMC>, NTHREADS, smem);
}

int bind_device(diso_extractor* ex) {
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (ex->device != dev) {
    ex->release();
    ex->device = dev;
  }
  if (!ex->stats) {
    CUDA_TRY(cudaMalloc((void**)&ex->stats, sizeof(Stats)));
    CUDA_TRY(cudaMallocHost((void**)&ex->stats_host, sizeof(Stats)));
    int sms = 0, per_sm = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (ex->dtype == DISO_F32)
      CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, ex->method == DISO_MC ? count_kernel<float, MC> : count_kernel<float, DMC>, NTHREADS, 0));
    else
      CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, ex->method == DISO_MC ? count_kernel<double, MC> : count_kernel<double, DMC>, NTHREADS, 0));
    ex->resident_ctas = sms * std::max(per_sm, 1);
    ex->sms = sms;
    int per_tma = 0;
    if (ex->dtype == DISO_F32)
      CUDA_TRY(tma_occupancy<float>(ex->method, &per_tma));
    else
      CUDA_TRY(tma_occupancy<double>(ex->method, &per_tma));
    ex->tma_ctas = sms * std::max(per_tma, 1);
    ex->per_sm[0] = std::max(per_tma, 1);
    int per_g = 0;
    if (ex->dtype == DISO_F32)
      CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_g, gather_list_kernel<float>, NTHREADS, 0));
    else
      CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_g, gather_list_kernel<double>, NTHREADS, 0));
    ex->gather_ctas = sms * std::max(per_g, 1);
    ex->per_sm[2] = std::max(per_g, 1);
    int per_e = 0;
    if (ex->dtype == DISO_F32)
      CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_e, ex->method == DISO_MC ? (const void*)mc_emit_kernel<float> : (const void*)dmc_emit_kernel<float>,
          NTHREADS, 0));
    else
      CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_e, ex->method == DISO_MC ? (const void*)mc_emit_kernel<double> : (const void*)dmc_emit_kernel<double>,
          NTHREADS, 0));
    ex->emit_ctas = sms * std::max(per_e, 1);
    ex->per_sm[1] = std::max(per_e, 1);
    int per_f = 0;
    const void* fk = ex->dtype == DISO_F32
                         ? (ex->method == DISO_MC ? (const void*)fused_backward_kernel<float, MC, false>
                                                  : (const void*)fused_backward_kernel<float, DMC, false>)
                         : (ex->method == DISO_MC ? (const void*)fused_backward_kernel<double, MC, false>
                                                  : (const void*)fused_backward_kernel<double, DMC, false>);
    ex->fused_smem = (int)(ex->dtype == DISO_F32
                               ? (ex->method == DISO_MC ? fused_smem<float, MC>() : fused_smem<float, DMC>())
                               : (ex->method == DISO_MC ? fused_smem<double, MC>() : fused_smem<double, DMC>()));
    CUDA_TRY(cudaFuncSetAttribute(fk, cudaFuncAttributeMaxDynamicSharedMemorySize, ex->fused_smem));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_f, fk, NTHREADS, ex->fused_smem));
    if (ex->method == DISO_DMC) {  // the variant that reads the count's cell records
      const void* fr = ex->dtype == DISO_F32 ? (const void*)fused_backward_kernel<float, DMC, true>
                                             : (const void*)fused_backward_kernel<double, DMC, true>;
      ex->fused_smem_rec = (int)(ex->dtype == DISO_F32 ? fused_smem<float, DMC, true>() : fused_smem<double, DMC, true>());
      CUDA_TRY(cudaFuncSetAttribute(fr, cudaFuncAttributeMaxDynamicSharedMemorySize, ex->fused_smem_rec));
    }
    ex->fused_ctas = sms * std::max(per_f, 1);
    ex->per_sm[3] = std::max(per_f, 1);
    // the narrow band's backward: the fused tile with the same shared memory
    const void* bk = ex->dtype == DISO_F32
                         ? (ex->method == DISO_MC ? (const void*)brick_backward_kernel<float, MC, false>
                                                  : (const void*)brick_backward_kernel<float, DMC, false>)
                         : (ex->method == DISO_MC ? (const void*)brick_backward_kernel<double, MC, false>
                                                  : (const void*)brick_backward_kernel<double, DMC, false>);
    int per_b = 0;
    CUDA_TRY(cudaFuncSetAttribute(bk, cudaFuncAttributeMaxDynamicSharedMemorySize, ex->fused_smem));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_b, bk, NTHREADS, ex->fused_smem));
    ex->brick_ctas = sms * std::max(per_b, 1);
    if (ex->method == DISO_DMC) {  // the variant that reads the forward's cell records
      const void* br = ex->dtype == DISO_F32 ? (const void*)brick_backward_kernel<float, DMC, true>
                                             : (const void*)brick_backward_kernel<double, DMC, true>;
      CUDA_TRY(cudaFuncSetAttribute(br, cudaFuncAttributeMaxDynamicSharedMemorySize, ex->fused_smem_rec));
    }
    CUDA_TRY(cudaStreamCreateWithFlags(&ex->side, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&ex->ev_fork, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&ex->ev_join, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&ex->ev_zero, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&ex->ev_counts, cudaEventDisableTiming));
    // recorded once so that a backward that waits on it before any zeroing proceeds
    CUDA_TRY(cudaEventRecord(ex->ev_zero, ex->side));
    CUDA_TRY(cudaMalloc((void**)&ex->plist_n, sizeof(unsigned)));
  }
  return DISO_OK;
}

int reset_stats(diso_extractor* ex, cudaStream_t s) {
  CUDA_TRY(cudaMemsetAsync(ex->stats, 0, sizeof(Stats), s));
  CUDA_TRY(cudaMemsetAsync(&ex->stats->min_key, 0xff, sizeof(unsigned long long), s));
  return DISO_OK;
}

// look-back state for a scan of n elements; returns its tiles (0 on failure)
int64_t scan_reserve(diso_extractor* ex, int64_t n) {
  const int64_t tiles = (n + 1 + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles > ex->scan_cap) {
    cudaFree(ex->scan_flag);
    cudaFree(ex->scan_agg);
    cudaFree(ex->scan_incl);
    ex->scan_flag = nullptr;
    ex->scan_agg = ex->scan_incl = nullptr;
    ex->scan_cap = 0;
    const int64_t cap = tiles + tiles / 4 + 64;
    if (cudaMalloc((void**)&ex->scan_flag, (size_t)cap * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc((void**)&ex->scan_agg, (size_t)cap * sizeof(uint64_t)) != cudaSuccess ||
        cudaMalloc((void**)&ex->scan_incl, (size_t)cap * sizeof(uint64_t)) != cudaSuccess) {
      fail(DISO_ERR_CUDA, "scan state allocation of %lld tiles failed", (long long)cap);
      return 0;
    }
    ex->scan_cap = cap;
  }
  return tiles;
}

// exclusive look-back scan of a[0..n) in place, a[n] = total (also into *total_out
// when given).  `prepared`: its flags and tile counter were zeroed by count_prep_kernel.
int run_scan(diso_extractor* ex, uint64_t* a, int64_t n, cudaStream_t s, bool prepared = false,
             uint64_t* total_out = nullptr) {
  const int64_t tiles = scan_reserve(ex, n);
  if (tiles == 0) return DISO_ERR_CUDA;
  if (!prepared) {
    CUDA_TRY(cudaMemsetAsync(ex->scan_flag, 0, (size_t)tiles * sizeof(uint32_t), s));
    CUDA_TRY(cudaMemsetAsync(&ex->stats->scan_tile, 0, sizeof(unsigned long long), s));
  }
  ScanState st{ex->scan_flag, ex->scan_agg, ex->scan_incl};
  {
    KernelTimer kt(ex, K_SCAN, s);
    scan_lookback_kernel<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(a, n, st, ex->stats, total_out, SCAN_SPIN_LIMIT);
  }
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

// A grid's counts are scanned in two 32-bit halves (crossings; triangles / patches),
// and vertex ids are 32-bit in the records: with at most 3 crossings per cell, a grid
// of fewer than 2^31 / 3 cells can never overflow them.  A larger grid (up to the
// index limits below) is checked after its count instead: the count also sums both
// halves in 64 bits (Stats::sum_lo / sum_hi), and count_read rejects counts that do
// not fit, before anything reads the record (forward_all waits for that check before
// its emit).
constexpr int kMaxDim = 16384;
constexpr double kMaxCells = 68719476736.0;  // 2^36
inline bool counts_always_fit(int nx, int ny, int nz) {
  return 3.0 * (double)(nx + 1) * (ny + 1) * (nz + 1) < 2147483647.0;
}

int check_common(diso_extractor* ex, const void* sdf, int nx, int ny, int nz) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  if (!sdf) return fail(DISO_ERR_ARG, "null sdf");
  if (nx < 1 || ny < 1 || nz < 1) return fail(DISO_ERR_ARG, "grid dims must be >= 1 (got %d x %d x %d)", nx, ny, nz);
  const double cells = (double)(nx + 1) * (ny + 1) * (nz + 1);
  if (nx > kMaxDim || ny > kMaxDim || nz > kMaxDim || cells >= kMaxCells)
    return fail(DISO_ERR_ARG, "grid too large: %d x %d x %d (at most %d points per axis and 2^36 cells)", nx, ny,
                nz, kMaxDim);
  return bind_device(ex);
}

// the per-call record: segment bases [nseg], the total [1], then two activity bytes per forward tile
inline uint8_t* tile_flags(const uint64_t* seg, const Geom& g) { return (uint8_t*)(seg + g.nseg + 1); }

template <class S>
Field<S> make_field(const void* sdf, const void* deform, int nx, int ny, int nz, double iso, double padval) {
  Field<S> f;
  f.sdf = (const S*)sdf;
  f.def = (const S*)deform;
  f.n0 = nx;
  f.n1 = ny;
  f.n2 = nz;
  f.iso = (S)iso;
  f.pad = (S)padval;
  return f;
}

int flush_zero(diso_extractor* ex, cudaStream_t z);
int take_zero_job(diso_extractor* ex, const Geom& g, int64_t units, unsigned grid, cudaStream_t s, ZeroJob* zj);
ZeroJob take_emit_zero(diso_extractor* ex, unsigned grid, cudaStream_t s);
int flush_emit_zero(diso_extractor* ex, cudaStream_t s);

// share of a forward's gradient zeros that the count writes (the emit writes the rest)
constexpr double ZERO_COUNT_SHARE = 0.35;

template <class S>
int count_launch(diso_extractor* ex, const void* sdf, int nx, int ny, int nz, double iso, double padval,
                 uint64_t* seg, cudaStream_t s) {
  Geom g;
  g.init(nx, ny, nz);
  int rc;
  if ((rc = grow(ex->active, ex->active_cap, g.ntiles())) != DISO_OK) return rc;
  if (ex->method == DISO_DMC && (rc = grow(ex->codes, ex->codes_cap, g.ncodes())) != DISO_OK) return rc;
  // status words and the scan's look-back flags in one launch
  const int64_t scan_tiles = scan_reserve(ex, g.nseg);
  if (scan_tiles == 0) return DISO_ERR_CUDA;
  count_prep_kernel<<<1, 256, 0, s>>>(ex->stats, ex->scan_flag, scan_tiles);
  CUDA_TRY(cudaGetLastError());
  ex->codes_seg = seg;
  ex->codes_dims[0] = nx;
  ex->codes_dims[1] = ny;
  ex->codes_dims[2] = nz;
  ex->codes_band = false;
  CellRec* codes = ex->method == DISO_DMC ? ex->codes : nullptr;
  Field<S> f = make_field<S>(sdf, nullptr, nx, ny, nz, iso, padval);
  // persistent grids: enough CTAs to fill the GPU, and at most COUNT_LIST tiles each
  CUtensorMap wide;
  const bool tma = count_tensor_map<S>(sdf, nx, ny, nz, &wide);
  if (tma) {
    const int64_t units = count_tma_units(g);
    const int64_t want =
        std::max<int64_t>(tuned_ctas(ex, DISO_TUNE_COUNT_CTAS, ex->tma_ctas, ex->per_sm[0]),
                          (units * TMA_TILES_PER_UNIT + COUNT_LIST - 1) / COUNT_LIST);
    const unsigned grid = (unsigned)std::min<int64_t>(want, units);
    const size_t smem = count_tma_smem<S>();
    ZeroJob zj;
    if ((rc = take_zero_job(ex, g, units, grid, s, &zj)) != DISO_OK) return rc;
    KernelTimer kt(ex, K_COUNT, s);
    if (ex->method == DISO_MC)
      count_tma_kernel<S, MC><<<grid, NTHREADS, smem, s>>>(wide, f, g, seg, tile_flags(seg, g), codes,
                                                           ex->stats, ex->active, zj);
    else
      count_tma_kernel<S, DMC><<<grid, NTHREADS, smem, s>>>(wide, f, g, seg, tile_flags(seg, g), codes,
                                                            ex->stats, ex->active, zj);
  } else {
    ex->zemit_set = false;
    if ((rc = flush_zero(ex, ex->side)) != DISO_OK) return rc;
    KernelTimer kt(ex, K_COUNT, s);
    const int64_t units = count_units(g);
    const int64_t want =
        std::max<int64_t>(ex->resident_ctas, (units * COUNT_TILES_PER_UNIT + COUNT_LIST - 1) / COUNT_LIST);
    const unsigned grid = (unsigned)std::min<int64_t>(want, units);
    if (ex->method == DISO_MC)
      count_kernel<S, MC><<<grid, NTHREADS, 0, s>>>(f, g, seg, tile_flags(seg, g), codes, ex->stats, ex->active);
    else
      count_kernel<S, DMC><<<grid, NTHREADS, 0, s>>>(f, g, seg, tile_flags(seg, g), codes, ex->stats, ex->active);
  }
  CUDA_TRY(cudaGetLastError());
  return run_scan(ex, seg, g.nseg, s, true, reinterpret_cast<uint64_t*>(&ex->stats->total));
}

// the count's results to the host (into the pinned stats mirror, the scanned total
// included), then an event
template <class S>
int count_copy(diso_extractor* ex, const Geom& g, const uint64_t* seg, cudaStream_t s) {
  (void)g;
  (void)seg;
  CUDA_TRY(cudaMemcpyAsync(ex->stats_host, ex->stats, sizeof(Stats), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaEventRecord(ex->ev_counts, s));
  return DISO_OK;
}

// waits for count_copy's event and fills `out`
template <class S>
int count_read(diso_extractor* ex, int nx, int ny, int nz, double iso, const uint64_t* seg, cudaStream_t s,
               diso_counts* out) {
  Geom g;
  g.init(nx, ny, nz);
  (void)seg;
  CUDA_TRY(cudaEventSynchronize(ex->ev_counts));
  const Stats& h = *ex->stats_host;
  const uint64_t total = h.total;
  if (h.error & 1ull) return fail(DISO_ERR_SCAN, "segment scan: look-back wait gave up");
  if (h.error & 4ull) return fail(DISO_ERR_SCAN, "count: wait for a TMA copy gave up");
  // the scanned 32-bit halves against the count's 64-bit sums
  if (h.sum_lo != Counts::lo(total) || h.sum_hi != Counts::hi(total) || h.sum_lo >= (1ull << 31) ||
      h.sum_hi >= (1ull << 31))
    return fail(DISO_ERR_ARG, "%d x %d x %d: too many crossings for 32-bit counts (%llu and %llu)", nx, ny, nz,
                (unsigned long long)h.sum_lo, (unsigned long long)h.sum_hi);
  // the low half counts crossings, the high half triangles (MC) or patches (DMC)
  if (ex->method == DISO_MC) {
    out->n_verts = Counts::lo(total);
    out->n_faces = Counts::hi(total);
  } else {
    out->n_verts = Counts::hi(total);
    out->n_faces = Counts::lo(total);
  }
  out->sdf_min = key_to_double(h.min_key);
  out->sdf_max = key_to_double(h.max_key);
  const double isoS = (double)(S)iso;
  out->empty = (out->sdf_min >= isoS || out->sdf_max <= isoS) ? 1 : 0;
  out->emitted = 0;
  out->n_active_tiles = (int64_t)h.n_active;
  ex->last_active = out->n_active_tiles;
  // the emit's part of the zeros: no emit follows a count of an empty surface
  if (out->empty) return flush_emit_zero(ex, s);
  return DISO_OK;
}

template <class S>
int forward_count(diso_extractor* ex, const void* sdf, int nx, int ny, int nz, double iso, double padval,
                  uint64_t* seg, cudaStream_t s, diso_counts* out) {
  Geom g;
  g.init(nx, ny, nz);
  int rc;
  if ((rc = count_launch<S>(ex, sdf, nx, ny, nz, iso, padval, seg, s)) != DISO_OK) return rc;
  if ((rc = count_copy<S>(ex, g, seg, s)) != DISO_OK) return rc;
  return count_read<S>(ex, nx, ny, nz, iso, seg, s, out);
}

// the emit over the count's active tiles (persistent, `grid` CTAs); the outputs are
// written only when they fit the capacities
template <class S>
int emit_launch(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz, double iso,
                double padval, const uint64_t* seg, int normalize, void* verts, int64_t* faces, void* record,
                unsigned grid, int64_t vcap, int64_t fcap, cudaStream_t s) {
  Geom g;
  g.init(nx, ny, nz);
  Field<S> f = make_field<S>(sdf, deform, nx, ny, nz, iso, padval);
  CUDA_TRY(cudaMemsetAsync(&ex->stats->emit_tile, 0, sizeof(unsigned long long), s));
  const ZeroJob zj = take_emit_zero(ex, grid, s);
  KernelTimer kt(ex, K_EMIT, s);
  if (ex->method == DISO_MC)
    mc_emit_kernel<S><<<grid, NTHREADS, 0, s>>>(f, g, seg, ex->active, &ex->stats->n_active, (S*)verts, faces,
                                                normalize, record, vcap, fcap, ex->stats, zj);
  else
    dmc_emit_kernel<S><<<grid, NTHREADS, 0, s>>>(f, g, seg, ex->codes, ex->active, &ex->stats->n_active, (S*)verts,
                                                 faces, normalize, record, vcap, fcap, ex->stats, zj);
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

template <class S>
int forward_emit(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz, double iso,
                 double padval, const uint64_t* seg, int normalize, void* verts, int64_t* faces, void* record,
                 cudaStream_t s) {
  if (ex->last_active <= 0) return flush_emit_zero(ex, s);
  const unsigned grid = (unsigned)std::min<int64_t>(
      ex->last_active, tuned_ctas(ex, DISO_TUNE_EMIT_CTAS, ex->emit_ctas, ex->per_sm[1]));
  return emit_launch<S>(ex, sdf, deform, nx, ny, nz, iso, padval, seg, normalize, verts, faces, record, grid,
                        INT64_MAX, INT64_MAX, s);
}

// count, scan and an emit into outputs of the given capacities, with one
// synchronisation at the end (counts->emitted says whether the outputs were written)
template <class S>
int forward_all(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz, double iso,
                double padval, uint64_t* seg, int normalize, void* verts, int64_t vcap, int64_t* faces,
                int64_t fcap, void* record, cudaStream_t s, diso_counts* out) {
  Geom g;
  g.init(nx, ny, nz);
  int rc;
  if ((rc = count_launch<S>(ex, sdf, nx, ny, nz, iso, padval, seg, s)) != DISO_OK) return rc;
  if ((rc = count_copy<S>(ex, g, seg, s)) != DISO_OK) return rc;
  // a grid whose counts could overflow is checked before its emit reads the record
  const bool checked = !counts_always_fit(nx, ny, nz);
  if (checked) {
    if ((rc = count_read<S>(ex, nx, ny, nz, iso, seg, s, out)) != DISO_OK) return rc;
    if (out->empty) return DISO_OK;
  }
  // otherwise the emit is queued before the host waits for the counts, and still runs
  // when it returns
  if ((rc = emit_launch<S>(ex, sdf, deform, nx, ny, nz, iso, padval, seg, normalize, verts, faces, record,
                           tuned_ctas(ex, DISO_TUNE_EMIT_CTAS, ex->emit_ctas, ex->per_sm[1]), vcap, fcap, s)) !=
      DISO_OK)
    return rc;
  if (!checked && (rc = count_read<S>(ex, nx, ny, nz, iso, seg, s, out)) != DISO_OK) return rc;
  out->emitted = (out->n_verts <= vcap && out->n_faces <= fcap) ? 1 : 0;
  return DISO_OK;
}

// CTAs of the persistent edge pass
inline unsigned edge_ctas(const diso_extractor* ex) { return per_sm_ctas(ex, DISO_TUNE_EDGE_CTAS, 8); }

// CTAs of a grid-stride pass over n items of 256 threads, at most `cap`
inline unsigned stride_ctas(int64_t n, unsigned cap) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, cap));
}

// the zeros of the inactive point tiles run on the side stream, between fork and join
int side_fork(diso_extractor* ex, cudaStream_t s) {
  CUDA_TRY(cudaEventRecord(ex->ev_fork, s));
  CUDA_TRY(cudaStreamWaitEvent(ex->side, ex->ev_fork, 0));
  return DISO_OK;
}
int side_join(diso_extractor* ex, cudaStream_t s) {
  CUDA_TRY(cudaEventRecord(ex->ev_join, ex->side));
  CUDA_TRY(cudaStreamWaitEvent(s, ex->ev_join, 0));
  return DISO_OK;
}

template <class S>
int backward(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz, double iso,
             double padval, const uint64_t* seg, void* record, int normalize, int flags, const void* gv, void* gsdf,
             void* gdef, cudaStream_t s) {
  Geom g;
  g.init(nx, ny, nz);
  Field<S> f = make_field<S>(sdf, deform, nx, ny, nz, iso, padval);
  const int exact = (flags & DISO_GRAD_EXACT) ? 1 : 0;
  const bool zeroed = (flags & DISO_GRAD_ZEROED) != 0;
  int rc;
  if ((rc = grow(ex->plist, ex->plist_cap, g.nptiles())) != DISO_OK) return rc;
  if (zeroed) {
    CUDA_TRY(cudaStreamWaitEvent(s, ex->ev_zero, 0));
  } else {
    if ((rc = side_fork(ex, s)) != DISO_OK) return rc;
    // few CTAs per SM, so that the gather of the active tiles finds room beside them
    KernelTimer kt(ex, K_ZERO_TILES, ex->side);
    zero_tiles_kernel<S><<<per_sm_ctas(ex, DISO_TUNE_ZERO_CTAS, 2), 256, 0, ex->side>>>(f, g, tile_flags(seg, g),
                                                                                        (S*)gsdf, (S*)gdef);
    CUDA_TRY(cudaGetLastError());
  }
  CUDA_TRY(cudaMemsetAsync(ex->plist_n, 0, sizeof(unsigned), s));
  {
    KernelTimer kt(ex, K_ACTIVE_PTILES, s);
    active_ptiles_kernel<<<stride_ctas(g.nptiles(), ex->sms * 8), 256, 0, s>>>(g, tile_flags(seg, g), ex->plist,
                                                                               ex->plist_n);
  }
  CUDA_TRY(cudaGetLastError());
  {
    KernelTimer kt(ex, K_EDGE, s);
    if (ex->method == DISO_MC)
      edge_adjoint_kernel<S, MC><<<edge_ctas(ex), 256, 0, s>>>(f, g, seg, record, (const S*)gv, normalize, 0);
    else
      edge_adjoint_kernel<S, DMC><<<edge_ctas(ex), 256, 0, s>>>(f, g, seg, record, (const S*)gv, normalize, exact);
  }
  CUDA_TRY(cudaGetLastError());
  {
    KernelTimer kt(ex, K_GATHER, s);
    gather_list_kernel<S><<<tuned_ctas(ex, DISO_TUNE_GATHER_CTAS, ex->gather_ctas, ex->per_sm[2]), NTHREADS, 0, s>>>(f, g, seg, ex->plist, ex->plist_n, record,
                                                                        (S*)gsdf, (S*)gdef);
  }
  CUDA_TRY(cudaGetLastError());
  return zeroed ? DISO_OK : side_join(ex, s);
}

// the backward of a forward that kept only its segment record (backward.cuh): the
// zeros of the point tiles with no crossing nearby on the second stream, the fused
// pass over the list of the others on `s`
template <class S>
int backward_fused(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz, double iso,
                   double padval, const uint64_t* seg, int normalize, int flags, const void* gv, void* gsdf,
                   void* gdef, cudaStream_t s) {
  Geom g;
  g.init(nx, ny, nz);
  Field<S> f = make_field<S>(sdf, deform, nx, ny, nz, iso, padval);
  const int exact = (flags & DISO_GRAD_EXACT) ? 1 : 0;
  int rc;
  if ((rc = grow(ex->plist, ex->plist_cap, g.nptiles())) != DISO_OK) return rc;
  // The zeros of the point tiles with no crossing nearby: bulk copies issued from
  // inside the fused pass when the gradients' rows are whole 16-byte units at
  // 16-byte aligned addresses (they then take no warps from it); otherwise a zero
  // kernel on the second stream, two CTAs per SM launched first (fewer warps make
  // the zeros, and the fused pass beside them, slower: measured).
  const bool zbulk = ((int64_t)nz * (int64_t)sizeof(S)) % 16 == 0 && ((uintptr_t)gsdf & 15u) == 0 &&
                     ((uintptr_t)gdef & 15u) == 0;
  // DMC: the cell records of the extractor's last count are this forward's when that
  // count wrote this `seg` for a grid of these sizes (no other forward ran since);
  // then the fused pass reads the window cells' codes and patch offsets from them
  // instead of running the ambiguity test again
  const bool records = ex->method == DISO_DMC && ex->codes && ex->codes_seg == seg && !ex->codes_band &&
                       ex->codes_dims[0] == nx && ex->codes_dims[1] == ny && ex->codes_dims[2] == nz;
  if (!zbulk) {
    if ((rc = side_fork(ex, s)) != DISO_OK) return rc;
    KernelTimer kt(ex, K_ZERO_TILES, ex->side);
    zero_tiles_kernel<S><<<per_sm_ctas(ex, DISO_TUNE_ZERO_CTAS, 2), 256, 0, ex->side>>>(f, g, tile_flags(seg, g),
                                                                                        (S*)gsdf, (S*)gdef);
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemsetAsync(ex->plist_n, 0, sizeof(unsigned), s));
  {
    KernelTimer kt(ex, K_ACTIVE_PTILES, s);
    active_ptiles_kernel<<<stride_ctas(g.nptiles(), ex->sms * 8), 256, 0, s>>>(g, tile_flags(seg, g), ex->plist,
                                                                               ex->plist_n);
  }
  CUDA_TRY(cudaGetLastError());
  {
    KernelTimer kt(ex, K_FUSED_BWD, s);
    if (ex->method == DISO_MC)
      fused_backward_kernel<S, MC, false><<<tuned_ctas(ex, DISO_TUNE_FUSED_CTAS, ex->fused_ctas, ex->per_sm[3]), NTHREADS,
                                     (size_t)ex->fused_smem, s>>>(f, g, seg, ex->plist, ex->plist_n, (const S*)gv,
                                                                  normalize, 0, (S*)gsdf, (S*)gdef, ex->stats,
                                                                  zbulk ? 1 : 0, nullptr);
    else if (records)
      fused_backward_kernel<S, DMC, true><<<tuned_ctas(ex, DISO_TUNE_FUSED_CTAS, ex->fused_ctas, ex->per_sm[3]),
                                            NTHREADS, (size_t)ex->fused_smem_rec, s>>>(
          f, g, seg, ex->plist, ex->plist_n, (const S*)gv, normalize, exact, (S*)gsdf, (S*)gdef, ex->stats,
          zbulk ? 1 : 0, ex->codes);
    else
      fused_backward_kernel<S, DMC, false><<<tuned_ctas(ex, DISO_TUNE_FUSED_CTAS, ex->fused_ctas, ex->per_sm[3]),
                                             NTHREADS, (size_t)ex->fused_smem, s>>>(
          f, g, seg, ex->plist, ex->plist_n, (const S*)gv, normalize, exact, (S*)gsdf, (S*)gdef, ex->stats,
          zbulk ? 1 : 0, nullptr);
  }
  CUDA_TRY(cudaGetLastError());
  if (zbulk) return DISO_OK;
  return side_join(ex, s);
}

// the zeros as memsets on stream z, after the work queued on s so far
int zero_grads_side(diso_extractor* ex, void* gsdf, int64_t sb, void* gdef, int64_t db, cudaStream_t s,
                    cudaStream_t z) {
  CUDA_TRY(cudaEventRecord(ex->ev_fork, s));
  CUDA_TRY(cudaStreamWaitEvent(z, ex->ev_fork, 0));
  {
    KernelTimer kt(ex, K_ZERO_GRADS, z);
    if (sb) CUDA_TRY(cudaMemsetAsync(gsdf, 0, (size_t)sb, z));
    if (db) CUDA_TRY(cudaMemsetAsync(gdef, 0, (size_t)db, z));
  }
  CUDA_TRY(cudaEventRecord(ex->ev_zero, z));
  return DISO_OK;
}

// a pending zero goes to a side-stream memset (when no TMA count on its stream takes it)
int flush_zero(diso_extractor* ex, cudaStream_t z) {
  if (!ex->zpend.set) return DISO_OK;
  const diso_extractor::PendingZero pz = ex->zpend;
  ex->zpend.set = false;
  return zero_grads_side(ex, pz.p[0], pz.bytes[0], pz.p[1], pz.bytes[1], pz.stream, z);
}

// Buffers whose zeros the next forward on stream s writes beside its count and emit
// (they are 16-byte aligned); others are zeroed on stream z beside the work of s.
// Zeros still pending from an earlier call are dropped, not written: that forward
// never ran, and its buffers may be gone.
int zero_grads(diso_extractor* ex, void* gsdf, int64_t sb, void* gdef, int64_t db, cudaStream_t s,
               cudaStream_t z) {
  ex->zpend.set = false;
  ex->zemit_set = false;
  const bool aligned = ((uintptr_t)gsdf & 15u) == 0 && ((uintptr_t)gdef & 15u) == 0;
  if (!aligned) return zero_grads_side(ex, gsdf, sb, gdef, db, s, z);
  ex->zpend.p[0] = gsdf;
  ex->zpend.p[1] = gdef;
  ex->zpend.bytes[0] = sb;
  ex->zpend.bytes[1] = db;
  ex->zpend.stream = s;
  ex->zpend.set = true;
  return DISO_OK;
}

// rounds of `bytes` over `grid` CTAs that take `steps` steps each at least
void zero_rate(ZeroJob* zj, unsigned grid, int64_t steps) {
  const int64_t bytes = zj->end - zj->begin;
  const int64_t per_step = (bytes + (int64_t)grid * steps - 1) / ((int64_t)grid * steps);
  zj->rbytes = std::max<int64_t>(ZBUF, (per_step + ZBUF - 1) / ZBUF * ZBUF);
  zj->rounds = bytes > 0 ? (bytes + (int64_t)grid * zj->rbytes - 1) / ((int64_t)grid * zj->rbytes) : 0;
}

// The pending zero on stream s, split between the TMA count over `units` units in
// `grid` CTAs (the first ZERO_COUNT_SHARE of the bytes, one round per box) and the
// emit that follows (the rest, kept in ex->zemit).  The bytes past the last whole
// 16-byte vector of each buffer are set here.
int take_zero_job(diso_extractor* ex, const Geom& g, int64_t units, unsigned grid, cudaStream_t s, ZeroJob* zj) {
  *zj = ZeroJob{};
  ex->zemit_set = false;
  if (!ex->zpend.set) return DISO_OK;
  if (ex->zpend.stream != s) return flush_zero(ex, ex->side);
  const diso_extractor::PendingZero pz = ex->zpend;
  ex->zpend.set = false;
  int64_t nv[2];
  for (int i = 0; i < 2; ++i) {
    nv[i] = pz.bytes[i] / 16;
    const int64_t tail = pz.bytes[i] - nv[i] * 16;
    if (tail) CUDA_TRY(cudaMemsetAsync((char*)pz.p[i] + nv[i] * 16, 0, (size_t)tail, s));
  }
  zj->p0 = (char*)pz.p[0];
  zj->p1 = (char*)pz.p[1];
  zj->n0 = nv[0] * 16;
  const int64_t n = (nv[0] + nv[1]) * 16;
  if (n == 0) return DISO_OK;
  const int64_t split = (int64_t)((double)n * ex->zero_share) / 16 * 16;
  ex->zemit = *zj;
  ex->zemit.begin = split;
  ex->zemit.end = n;
  ex->zemit_stream = s;
  ex->zemit_set = split < n;
  zj->begin = 0;
  zj->end = split;
  // the fewest boxes a CTA gets is its whole units times the boxes (chunks) of the
  // shortest unit
  const int64_t nbz = (g.nzc + KZT - 1) / KZT, kz = (g.nzc + nbz - 1) / nbz;
  const int64_t kz_min = g.nzc - (nbz - 1) * kz;
  zero_rate(zj, grid, std::max<int64_t>(1, (units / grid) * kz_min));
  return DISO_OK;
}

// the emit's part of the zeros, for an emit on stream s in `grid` CTAs (one round per
// tile, at the tile count of the last count)
ZeroJob take_emit_zero(diso_extractor* ex, unsigned grid, cudaStream_t s) {
  ZeroJob zj{};
  if (!ex->zemit_set || ex->zemit_stream != s) return zj;
  ex->zemit_set = false;
  zj = ex->zemit;
  zero_rate(&zj, grid, std::max<int64_t>(1, ex->last_active / grid));
  return zj;
}

// the emit's part of the zeros as memsets on stream s (when no emit follows the count)
int flush_emit_zero(diso_extractor* ex, cudaStream_t s) {
  if (!ex->zemit_set) return DISO_OK;
  ex->zemit_set = false;
  const ZeroJob& z = ex->zemit;
  if (z.begin < z.n0) CUDA_TRY(cudaMemsetAsync(z.p0 + z.begin, 0, (size_t)(std::min(z.end, z.n0) - z.begin), s));
  if (z.end > z.n0) {
    const int64_t b = std::max(z.begin, z.n0);
    CUDA_TRY(cudaMemsetAsync(z.p1 + (b - z.n0), 0, (size_t)(z.end - b), s));
  }
  return DISO_OK;
}

template <class S>
int split_quads(diso_extractor* ex, const void* verts, const int64_t* quads, int64_t nq, int64_t* tris,
                int64_t* n_tris, cudaStream_t s) {
  int rc;
  if ((rc = grow(ex->split, ex->split_cap, nq + 1)) != DISO_OK) return rc;
  if ((rc = reset_stats(ex, s)) != DISO_OK) return rc;
  const int threads = 256;
  const unsigned blocks = (unsigned)((nq + threads - 1) / threads);
  KernelTimer kt(ex, K_SPLIT, s);
  split_count_kernel<S><<<blocks, threads, 0, s>>>((const S*)verts, quads, nq, ex->split);
  CUDA_TRY(cudaGetLastError());
  if ((rc = run_scan(ex, ex->split, nq, s)) != DISO_OK) return rc;
  split_scatter_kernel<<<blocks, threads, 0, s>>>(quads, nq, ex->split, tris);
  CUDA_TRY(cudaGetLastError());
  uint64_t total = 0;
  CUDA_TRY(cudaMemcpyAsync(ex->stats_host, ex->stats, sizeof(Stats), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(&total, ex->split + nq, sizeof total, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (ex->stats_host->error & 1ull) return fail(DISO_ERR_SCAN, "split scan: look-back wait gave up");
  *n_tris = 2 * ((int64_t)Counts::lo(total) + (int64_t)Counts::hi(total));
  return DISO_OK;
}

// ------------------------------------------------------------------ batches

// zero the per-grid status words, min keys to the top
__global__ void init_stats_kernel(Stats* st, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    Stats z = {};
    z.min_key = ~0ull;
    st[i] = z;
  }
}

// scanned value at the first segment of every grid, and the total
__global__ void gather_bounds_kernel(const uint64_t* seg, const int64_t* off, int n, uint64_t* out) {
  for (int i = threadIdx.x; i <= n; i += blockDim.x) out[i] = seg[off[i]];
}

int64_t batch_record_slots(const diso_grid* grids, int n, int64_t* seg_total, int64_t* tiles_total) {
  int64_t segs = 0, tiles = 0;
  for (int i = 0; i < n; ++i) {
    Geom g;
    g.init(grids[i].nx, grids[i].ny, grids[i].nz);
    segs += g.nseg;
    tiles += g.ntiles();
  }
  if (seg_total) *seg_total = segs;
  if (tiles_total) *tiles_total = tiles;
  // segments of every grid, the total slot, then two activity bytes per tile of every grid
  return segs + 1 + (2 * tiles + 7) / 8;
}

template <class S>
int batch_prepare(diso_extractor* ex, const diso_grid* grids, int n, uint64_t* record, cudaStream_t s) {
  ex->codes_seg = nullptr;  // the batch's records replace the last single grid's
  if (!ex->bdesc) {
    CUDA_TRY(cudaMalloc(&ex->bdesc, sizeof(BatchGrid<double>) * MAX_BATCH));
    CUDA_TRY(cudaMallocHost(&ex->bdesc_host, sizeof(BatchGrid<double>) * MAX_BATCH + sizeof(int64_t) * (MAX_BATCH + 1)));
    CUDA_TRY(cudaMalloc((void**)&ex->bstats, sizeof(Stats) * MAX_BATCH));
    CUDA_TRY(cudaMallocHost((void**)&ex->bstats_host, sizeof(Stats) * MAX_BATCH));
    CUDA_TRY(cudaMalloc((void**)&ex->bbound, sizeof(uint64_t) * (MAX_BATCH + 1) + sizeof(int64_t) * (MAX_BATCH + 1)));
    CUDA_TRY(cudaMallocHost((void**)&ex->bbound_host, sizeof(uint64_t) * (MAX_BATCH + 1)));
    int per = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per, ex->method == DISO_MC ? batch_count_kernel<S, MC> : batch_count_kernel<S, DMC>, NTHREADS, 0));
    ex->bcount_ctas = ex->sms * std::max(per, 1);
    ex->bwork_ctas = ex->sms * 4;
  }
  // the previous prepare's upload must have left the staging buffer
  CUDA_TRY(cudaStreamSynchronize(s));
  BatchGrid<S>* d = (BatchGrid<S>*)ex->bdesc_host;
  int64_t* offs = (int64_t*)((char*)ex->bdesc_host + sizeof(BatchGrid<double>) * MAX_BATCH);
  int64_t seg_off = 0, tile_off = 0, cblk = 0, ptile = 0, code_off = 0;
  int64_t seg_total = 0, tiles_total = 0, codes_total = 0;
  batch_record_slots(grids, n, &seg_total, &tiles_total);
  uint8_t* flags = (uint8_t*)(record + seg_total + 1);
  for (int i = 0; i < n; ++i) {
    Geom g;
    g.init(grids[i].nx, grids[i].ny, grids[i].nz);
    codes_total += g.ncodes();
  }
  int rc;
  if (ex->method == DISO_DMC && (rc = grow(ex->codes, ex->codes_cap, codes_total)) != DISO_OK) return rc;
  for (int i = 0; i < n; ++i) {
    const diso_grid& q = grids[i];
    BatchGrid<S> b;
    b.f = make_field<S>(q.sdf, q.deform, q.nx, q.ny, q.nz, q.isovalue, q.padval);
    b.g.init(q.nx, q.ny, q.nz);
    b.seg = record + seg_off;
    b.seg_end = record + seg_off + b.g.nseg;
    b.tile_flag = flags + tile_off;
    b.codes = ex->method == DISO_DMC ? ex->codes + code_off : nullptr;
    b.cblk0 = cblk;
    b.ptile0 = ptile;
    b.gsdf = (S*)q.grad_sdf;
    b.gdef = q.deform ? (S*)q.grad_deform : nullptr;
    d[i] = b;
    offs[i] = seg_off;
    ex->bseg_off[i] = seg_off;
    seg_off += b.g.nseg;
    tile_off += 2 * b.g.ntiles();
    code_off += b.g.ncodes();
    cblk += count_units(b.g);
    ptile += b.g.nptiles();
  }
  offs[n] = seg_off;
  ex->bseg_off[n] = seg_off;
  ex->bn = n;
  ex->brecord = record;
  ex->bseg_total = seg_total;
  ex->btiles = tiles_total;
  ex->bblocks = cblk;
  ex->bptiles = ptile;
  if ((rc = grow(ex->active, ex->active_cap, tiles_total)) != DISO_OK) return rc;
  if ((rc = grow(ex->plist, ex->plist_cap, ex->bptiles)) != DISO_OK) return rc;
  // grow the scan state now so that count allocates nothing
  const int64_t scan_tiles = (seg_total + 1 + SCAN_TILE - 1) / SCAN_TILE;
  if (scan_tiles > ex->scan_cap) {
    cudaFree(ex->scan_flag);
    cudaFree(ex->scan_agg);
    cudaFree(ex->scan_incl);
    ex->scan_flag = nullptr;
    ex->scan_agg = ex->scan_incl = nullptr;
    ex->scan_cap = 0;
    const int64_t cap = scan_tiles + scan_tiles / 4 + 64;
    CUDA_TRY(cudaMalloc((void**)&ex->scan_flag, (size_t)cap * sizeof(uint32_t)));
    CUDA_TRY(cudaMalloc((void**)&ex->scan_agg, (size_t)cap * sizeof(uint64_t)));
    CUDA_TRY(cudaMalloc((void**)&ex->scan_incl, (size_t)cap * sizeof(uint64_t)));
    ex->scan_cap = cap;
  }
  CUDA_TRY(cudaMemcpyAsync(ex->bdesc, d, sizeof(BatchGrid<S>) * n, cudaMemcpyHostToDevice, s));
  int64_t* doffs = (int64_t*)((char*)ex->bbound + sizeof(uint64_t) * (MAX_BATCH + 1));
  CUDA_TRY(cudaMemcpyAsync(doffs, offs, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return DISO_OK;
}

template <class S>
int batch_count(diso_extractor* ex, cudaStream_t s) {
  const int n = ex->bn;
  init_stats_kernel<<<1, 256, 0, s>>>(ex->bstats, n);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemsetAsync(ex->stats, 0, sizeof(Stats), s));
  const int64_t want =
      std::max<int64_t>(ex->bcount_ctas, (ex->bblocks * COUNT_TILES_PER_UNIT + COUNT_LIST - 1) / COUNT_LIST);
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, ex->bblocks));
  const BatchGrid<S>* d = (const BatchGrid<S>*)ex->bdesc;
  if (ex->method == DISO_MC)
    batch_count_kernel<S, MC><<<grid, NTHREADS, 0, s>>>(d, n, ex->bblocks, ex->bstats, &ex->bstats->n_active,
                                                         ex->active);
  else
    batch_count_kernel<S, DMC><<<grid, NTHREADS, 0, s>>>(d, n, ex->bblocks, ex->bstats, &ex->bstats->n_active,
                                                          ex->active);
  CUDA_TRY(cudaGetLastError());
  const int64_t tiles = (ex->bseg_total + 1 + SCAN_TILE - 1) / SCAN_TILE;
  CUDA_TRY(cudaMemsetAsync(ex->scan_flag, 0, (size_t)tiles * sizeof(uint32_t), s));
  ScanState st{ex->scan_flag, ex->scan_agg, ex->scan_incl};
  scan_lookback_kernel<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(ex->brecord, ex->bseg_total, st, ex->stats, nullptr,
                                                                SCAN_SPIN_LIMIT);
  CUDA_TRY(cudaGetLastError());
  const int64_t* doffs = (const int64_t*)((char*)ex->bbound + sizeof(uint64_t) * (MAX_BATCH + 1));
  gather_bounds_kernel<<<1, 256, 0, s>>>(ex->brecord, doffs, n, ex->bbound);
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

// the batch record is laid out for the capacities: E = faces (DMC quads) or vertices (MC)
template <class S>
EdgeRecord<S> batch_record(const diso_extractor* ex, void* record, int64_t vcap, int64_t fcap) {
  if (!record) return EdgeRecord<S>{nullptr, nullptr, nullptr, nullptr};
  return edge_record<S>(record, ex->method, vcap, ex->method == DISO_MC ? vcap : fcap);
}

template <class S>
int batch_emit(diso_extractor* ex, int normalize, void* verts, int64_t vcap, int64_t* faces, int64_t fcap,
               void* record, cudaStream_t s) {
  const BatchGrid<S>* d = (const BatchGrid<S>*)ex->bdesc;
  const unsigned grid = per_sm_ctas(ex, DISO_TUNE_BATCH_CTAS, 4);
  const EdgeRecord<S> rec = batch_record<S>(ex, record, vcap, fcap);
  if (ex->method == DISO_MC)
    batch_emit_kernel<S, MC><<<grid, NTHREADS, 0, s>>>(d, ex->active, &ex->bstats->n_active, (S*)verts, faces, vcap,
                                                        fcap, normalize, ex->bstats, rec);
  else
    batch_emit_kernel<S, DMC><<<grid, NTHREADS, 0, s>>>(d, ex->active, &ex->bstats->n_active, (S*)verts, faces,
                                                         vcap, fcap, normalize, ex->bstats, rec);
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

template <class S>
int batch_backward(diso_extractor* ex, int normalize, int flags, const void* gv, void* record, int64_t vcap,
                   int64_t fcap, cudaStream_t s) {
  const BatchGrid<S>* d = (const BatchGrid<S>*)ex->bdesc;
  const unsigned grid = per_sm_ctas(ex, DISO_TUNE_BATCH_CTAS, 4);
  const int exact = (flags & DISO_GRAD_EXACT) ? 1 : 0;
  const EdgeRecord<S> rec = batch_record<S>(ex, record, vcap, fcap);
  (void)grid;
  int rc;
  if ((rc = side_fork(ex, s)) != DISO_OK) return rc;
  const unsigned zgrid = per_sm_ctas(ex, DISO_TUNE_ZERO_CTAS, 2), lgrid = stride_ctas(ex->bptiles, ex->sms * 8);
  if (ex->method == DISO_MC)
    batch_zero_tiles_kernel<S, MC><<<zgrid, 256, 0, ex->side>>>(d, ex->bn, ex->bptiles, vcap, fcap);
  else
    batch_zero_tiles_kernel<S, DMC><<<zgrid, 256, 0, ex->side>>>(d, ex->bn, ex->bptiles, vcap, fcap);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemsetAsync(ex->plist_n, 0, sizeof(unsigned), s));
  if (ex->method == DISO_MC) {
    batch_active_ptiles_kernel<S, MC><<<lgrid, 256, 0, s>>>(d, ex->bn, ex->bptiles, vcap, fcap, ex->plist,
                                                            ex->plist_n);
    CUDA_TRY(cudaGetLastError());
    batch_edge_adjoint_kernel<S, MC><<<edge_ctas(ex), 256, 0, s>>>(d, ex->bn, rec, vcap, fcap, (const S*)gv,
                                                                   normalize, 0);
  } else {
    batch_active_ptiles_kernel<S, DMC><<<lgrid, 256, 0, s>>>(d, ex->bn, ex->bptiles, vcap, fcap, ex->plist,
                                                             ex->plist_n);
    CUDA_TRY(cudaGetLastError());
    batch_edge_adjoint_kernel<S, DMC><<<edge_ctas(ex), 256, 0, s>>>(d, ex->bn, rec, vcap, fcap, (const S*)gv,
                                                                    normalize, exact);
  }
  CUDA_TRY(cudaGetLastError());
  batch_gather_list_kernel<S><<<tuned_ctas(ex, DISO_TUNE_GATHER_CTAS, ex->gather_ctas, ex->per_sm[2]), NTHREADS, 0,
                                s>>>(d, ex->bn, ex->plist, ex->plist_n,
                                                                            record);
  CUDA_TRY(cudaGetLastError());
  return side_join(ex, s);
}

int batch_results(diso_extractor* ex, diso_counts* out, int64_t* voff, int64_t* foff, int* overflow,
                  cudaStream_t s) {
  const int n = ex->bn;
  CUDA_TRY(cudaMemcpyAsync(ex->bstats_host, ex->bstats, sizeof(Stats) * n, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(ex->bbound_host, ex->bbound, sizeof(uint64_t) * (n + 1), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(ex->stats_host, ex->stats, sizeof(Stats), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (ex->stats_host->error & 1ull) return fail(DISO_ERR_SCAN, "batch segment scan: look-back wait gave up");
  const bool mc = ex->method == DISO_MC;
  for (int i = 0; i < n; ++i) {
    const uint64_t a = ex->bbound_host[i], b = ex->bbound_host[i + 1];
    const int64_t va = mc ? Counts::lo(a) : Counts::hi(a), vb = mc ? Counts::lo(b) : Counts::hi(b);
    const int64_t fa = mc ? Counts::hi(a) : Counts::lo(a), fb = mc ? Counts::hi(b) : Counts::lo(b);
    const Stats& h = ex->bstats_host[i];
    out[i].n_verts = vb - va;
    out[i].n_faces = fb - fa;
    out[i].sdf_min = key_to_double(h.min_key);
    out[i].sdf_max = key_to_double(h.max_key);
    out[i].empty = 0;  // the caller applies the guard with its own isovalue (see diso_batch_results)
    out[i].emitted = 0;
    out[i].n_active_tiles = 0;
    if (voff) voff[i] = va;
    if (foff) foff[i] = fa;
  }
  if (overflow) *overflow = (ex->bstats_host[0].error & 2ull) ? 1 : 0;
  return DISO_OK;
}

}  // namespace


// ------------------------------------------------------------------ evaluated fields

template <class S>
SphereField<S> make_sphere_field(const diso_sphere_field* d, int nx, int ny, int nz, double iso, double padval) {
  SphereField<S> f;
  f.sph = (const S*)d->spheres;
  f.def = (const S*)d->deform;
  f.K = d->count;
  const int n[3] = {nx, ny, nz};
  for (int a = 0; a < 3; ++a) {
    f.lo[a] = (S)d->lo[a];
    f.step[a] = n[a] > 1 ? (S)((d->hi[a] - d->lo[a]) / (double)(n[a] - 1)) : S(0);
  }
  f.n0 = nx;
  f.n1 = ny;
  f.n2 = nz;
  f.iso = (S)iso;
  f.pad = (S)padval;
  return f;
}

// The forward of an evaluated field (a union of spheres, a narrow band of bricks) in
// one call, as forward_all without edge record: the count evaluates the chunks near
// the surface (the others it classifies whole), the emit evaluates the end points of
// the crossing edges.
template <class S, class F>
int forward_field(diso_extractor* ex, const F& f, double iso, uint64_t* seg, int normalize,
                  void* verts, int64_t vcap, int64_t* faces, int64_t fcap, cudaStream_t s, diso_counts* out,
                  int* umap = nullptr) {
  Geom g;
  g.init(f.n0, f.n1, f.n2);
  int rc;
  // DMC cell records: dense, or (umap, a narrow band) one block per unit that holds
  // the surface, grown once the units are listed
  const bool blocks = umap != nullptr && ex->method == DISO_DMC;
  if ((rc = grow(ex->active, ex->active_cap, g.ntiles())) != DISO_OK) return rc;
  if (ex->method == DISO_DMC && !blocks && (rc = grow(ex->codes, ex->codes_cap, g.ncodes())) != DISO_OK) return rc;
  const int64_t scan_tiles = scan_reserve(ex, g.nseg);
  if (scan_tiles == 0) return DISO_ERR_CUDA;
  // a narrow band's records serve its backward (brick_backward_kernel); a sphere
  // union's backward recomputes its cells
  ex->codes_seg = F::kGrad == 2 ? seg : nullptr;
  ex->codes_dims[0] = f.n0;
  ex->codes_dims[1] = f.n1;
  ex->codes_dims[2] = f.n2;
  ex->codes_band = true;
  ex->zpend.set = ex->zemit_set = false;  // gradient zeros belong to a dense forward
  count_prep_kernel<<<1, 256, 0, s>>>(ex->stats, ex->scan_flag, scan_tiles);
  CUDA_TRY(cudaGetLastError());
  // the count leaves the units that field_units_kernel classifies whole unwritten
  CUDA_TRY(cudaMemsetAsync(seg, 0, (size_t)(g.nseg + 1 + (2 * g.ntiles() + 7) / 8) * sizeof(uint64_t), s));
  CellRec* codes = ex->method == DISO_DMC ? ex->codes : nullptr;
  {
    const int64_t units = count_units(g);
    if ((rc = grow(ex->ulist, ex->ulist_cap, units + 1)) != DISO_OK) return rc;
    CUDA_TRY(cudaMemsetAsync(ex->ulist, 0, sizeof(int), s));
    if (blocks) CUDA_TRY(cudaMemsetAsync(umap, 0xff, sizeof(int) * (size_t)units, s));
    const int64_t want =
        std::max<int64_t>(ex->resident_ctas, (units * COUNT_TILES_PER_UNIT + COUNT_LIST - 1) / COUNT_LIST);
    const unsigned grid = (unsigned)std::min<int64_t>(want, units);
    {
      KernelTimer kt(ex, K_COUNT, s);
      field_units_kernel<S, F><<<stride_ctas(units * 32, (unsigned)ex->sms * 16), 256, 0, s>>>(
          f, g, ex->stats, ex->ulist, blocks ? umap : nullptr);
    }
    CUDA_TRY(cudaGetLastError());
    if (blocks) {  // the listed units' record blocks (one host round trip)
      int listed = 0;
      CUDA_TRY(cudaMemcpyAsync(&listed, ex->ulist, sizeof(int), cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaStreamSynchronize(s));
      if ((rc = grow(ex->codes, ex->codes_cap, std::max(listed, 1) * BrickField<S>::UNIT_RECS)) != DISO_OK)
        return rc;
      codes = ex->codes;
    }
    KernelTimer kt(ex, K_COUNT, s);
    if (ex->method == DISO_MC)
      field_count_kernel<S, MC, F><<<grid, NTHREADS, 0, s>>>(f, g, seg, tile_flags(seg, g), codes, ex->stats,
                                                             ex->active, ex->ulist);
    else
      field_count_kernel<S, DMC, F><<<grid, NTHREADS, 0, s>>>(f, g, seg, tile_flags(seg, g), codes, ex->stats,
                                                              ex->active, ex->ulist);
  }
  CUDA_TRY(cudaGetLastError());
  if ((rc = run_scan(ex, seg, g.nseg, s, true, reinterpret_cast<uint64_t*>(&ex->stats->total))) != DISO_OK)
    return rc;
  if ((rc = count_copy<S>(ex, g, seg, s)) != DISO_OK) return rc;
  CUDA_TRY(cudaMemsetAsync(&ex->stats->emit_tile, 0, sizeof(unsigned long long), s));
  {
    const ZeroJob zj{};
    KernelTimer kt(ex, K_EMIT, s);
    if (ex->method == DISO_MC)
      mc_emit_kernel<S, F><<<(unsigned)ex->emit_ctas, NTHREADS, 0, s>>>(
          f, g, seg, ex->active, &ex->stats->n_active, (S*)verts, faces, normalize, nullptr, vcap, fcap, ex->stats, zj);
    else
      dmc_emit_kernel<S, F><<<(unsigned)ex->emit_ctas, NTHREADS, 0, s>>>(
          f, g, seg, codes, ex->active, &ex->stats->n_active, (S*)verts, faces, normalize, nullptr, vcap, fcap,
          ex->stats, zj);
  }
  CUDA_TRY(cudaGetLastError());
  if ((rc = count_read<S>(ex, f.n0, f.n1, f.n2, iso, seg, s, out)) != DISO_OK) return rc;
  out->emitted = (out->n_verts <= vcap && out->n_faces <= fcap) ? 1 : 0;
  return DISO_OK;
}

// the backward of an evaluated union of spheres (field_backward_kernel)
template <class S>
int backward_field(diso_extractor* ex, const SphereField<S>& f, const uint64_t* seg, int normalize, int flags,
                   const void* gv, double* grad_spheres, void* gdef, cudaStream_t s) {
  Geom g;
  g.init(f.n0, f.n1, f.n2);
  const size_t smem = ex->method == DISO_MC ? field_bwd_smem<S, MC>(f.K) : field_bwd_smem<S, DMC>(f.K);
  const void* k = ex->method == DISO_MC ? (const void*)field_backward_kernel<S, MC>
                                        : (const void*)field_backward_kernel<S, DMC>;
  CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, NTHREADS, smem));
  const unsigned grid = (unsigned)(ex->sms * std::max(per, 1));
  int rc;
  if ((rc = grow(ex->fpart, ex->fpart_cap, (int64_t)grid * f.K * 4)) != DISO_OK) return rc;
  const int exact = (flags & DISO_GRAD_EXACT) ? 1 : 0;
  {
    KernelTimer kt(ex, K_FUSED_BWD, s);
    if (ex->method == DISO_MC)
      field_backward_kernel<S, MC><<<grid, NTHREADS, smem, s>>>(f, g, seg, (const S*)gv, normalize, 0, (S*)gdef,
                                                                ex->fpart, ex->stats);
    else
      field_backward_kernel<S, DMC><<<grid, NTHREADS, smem, s>>>(f, g, seg, (const S*)gv, normalize, exact, (S*)gdef,
                                                                 ex->fpart, ex->stats);
  }
  CUDA_TRY(cudaGetLastError());
  field_grad_final_kernel<<<1, 256, 0, s>>>(ex->fpart, (int)grid, f.K * 4, grad_spheres);
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

int check_field(const diso_sphere_field* field, int nx, int ny, int nz) {
  if (!field || !field->spheres) return fail(DISO_ERR_ARG, "null field or spheres");
  if (field->count < 1 || field->count > 65536) return fail(DISO_ERR_ARG, "sphere count %d (1..65536)", field->count);
  if (nx < 1 || ny < 1 || nz < 1) return fail(DISO_ERR_ARG, "grid dims must be >= 1 (got %d x %d x %d)", nx, ny, nz);
  const double cells = (double)(nx + 1) * (ny + 1) * (nz + 1);
  if (3.0 * cells >= 2147483647.0) return fail(DISO_ERR_ARG, "grid too large: %d x %d x %d", nx, ny, nz);
  for (int a = 0; a < 3; ++a)
    if (!std::isfinite(field->lo[a]) || !std::isfinite(field->hi[a])) return fail(DISO_ERR_ARG, "non-finite bounds");
  return DISO_OK;
}

// ------------------------------------------------------------------ narrow band

template <class S>
BrickField<S> make_brick_field(const diso_brick_grid* b, double iso, double padval, const int* umap = nullptr) {
  BrickField<S> f;
  Geom g;
  g.init(b->dims[0], b->dims[1], b->dims[2]);
  f.umap = umap;
  f.unby = (g.c[1] + CR - 1) / CR;
  f.unbz = (g.nzc + KZ - 1) / KZ;
  f.ukz = (g.nzc + f.unbz - 1) / f.unbz;
  f.ukz_mul = (65536u + (unsigned)f.ukz - 1u) / (unsigned)f.ukz;
  f.index = b->index;
  f.val = (const S*)b->values;
  f.def = (const S*)b->deform;
  f.nb1 = (b->dims[1] + BRICK - 1) / BRICK;
  f.nb2 = (b->dims[2] + BRICK - 1) / BRICK;
  f.K = b->count;
  f.n0 = b->dims[0];
  f.n1 = b->dims[1];
  f.n2 = b->dims[2];
  f.iso = (S)iso;
  f.pad = (S)padval;
  f.bg = (S)b->background;
  return f;
}

// the arguments of a narrow band, before any CUDA call
int check_bricks(const diso_brick_grid* b) {
  if (!b || !b->index) return fail(DISO_ERR_ARG, "null brick grid or index");
  const int nx = b->dims[0], ny = b->dims[1], nz = b->dims[2];
  if (nx < 1 || ny < 1 || nz < 1) return fail(DISO_ERR_ARG, "grid dims must be >= 1 (got %d x %d x %d)", nx, ny, nz);
  if (nx > (1 << 30) || ny > (1 << 30) || nz > (1 << 30)) return fail(DISO_ERR_ARG, "grid dims above 2^30");
  if (b->count < 0) return fail(DISO_ERR_ARG, "negative brick count %d", b->count);
  if (b->count > 0 && !b->values) return fail(DISO_ERR_ARG, "null brick values");
  if (!std::isfinite(b->background) || !(b->background > 0.0))
    return fail(DISO_ERR_ARG, "background must be finite and > 0 (got %g)", b->background);
  return DISO_OK;
}

// One pass over the index (brick_check_kernel), read back: slots and tags valid, no
// slot used twice, and the crossings that the bricks allow fit the 32-bit counts
template <class S>
int validate_bricks(diso_extractor* ex, const diso_brick_grid* b, double iso, double padval, cudaStream_t s) {
  const int nb0 = (b->dims[0] + BRICK - 1) / BRICK, nb1 = (b->dims[1] + BRICK - 1) / BRICK,
            nb2 = (b->dims[2] + BRICK - 1) / BRICK;
  const int64_t nb = (int64_t)nb0 * nb1 * nb2;
  int rc;
  if ((rc = grow(ex->buses, ex->buses_cap, std::max(b->count, 1))) != DISO_OK) return rc;
  if ((rc = grow(ex->bcheck, ex->bcheck_cap, 4)) != DISO_OK) return rc;
  if (b->count) CUDA_TRY(cudaMemsetAsync(ex->buses, 0, sizeof(int) * (size_t)b->count, s));
  CUDA_TRY(cudaMemsetAsync(ex->bcheck, 0, 4 * sizeof(unsigned long long), s));
  const S bg = (S)b->background, isoS = (S)iso;
  {
    KernelTimer kt(ex, K_BRICK_CHECK, s);
    brick_check_kernel<<<stride_ctas(nb, ex->sms * 8), 256, 0, s>>>(b->index, nb0, nb1, nb2, b->count,
                                                                    bg >= isoS ? 1 : 0, -bg >= isoS ? 1 : 0,
                                                                    (S)padval >= isoS ? 1 : 0, ex->buses, ex->bcheck);
  }
  CUDA_TRY(cudaGetLastError());
  unsigned long long h[4] = {0, 0, 0, 0};
  CUDA_TRY(cudaMemcpyAsync(h, ex->bcheck, sizeof(h), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (h[0] & 1ull) return fail(DISO_ERR_ARG, "brick index: an entry is neither a slot in [0, %d) nor -1 / -2", b->count);
  if (h[0] & 2ull) return fail(DISO_ERR_ARG, "brick index: a slot is used by two bricks");
  // crossings are counted in 32 bits per half of the scan value: at most 3 per cell,
  // and only cells touching a present or a border brick can cross
  const double cells = std::min((double)(b->dims[0] + 1) * (b->dims[1] + 1) * (b->dims[2] + 1),
                                729.0 * (double)(h[1] + h[2]));
  if (3.0 * cells >= 2147483647.0)
    return fail(DISO_ERR_ARG, "narrow band too wide for 32-bit counts: %llu present and %llu border bricks", h[1],
                h[2]);
  return DISO_OK;
}

// the backward of a narrow band: its gradient slots zeroed, then the fused tile over
// the active point tiles with the gradients going to the slots
template <class S>
int backward_bricks(diso_extractor* ex, const BrickField<S>& f, int K, const uint64_t* seg, int normalize, int flags,
                    const void* gv, void* gval, void* gdef, cudaStream_t s) {
  Geom g;
  g.init(f.n0, f.n1, f.n2);
  int rc;
  if ((rc = grow(ex->plist, ex->plist_cap, g.nptiles())) != DISO_OK) return rc;
  if (K) {
    CUDA_TRY(cudaMemsetAsync(gval, 0, (size_t)K * BRICK_PTS * sizeof(S), s));
    if (gdef) CUDA_TRY(cudaMemsetAsync(gdef, 0, (size_t)K * BRICK_PTS * 3 * sizeof(S), s));
  }
  CUDA_TRY(cudaMemsetAsync(ex->plist_n, 0, sizeof(unsigned), s));
  {
    KernelTimer kt(ex, K_ACTIVE_PTILES, s);
    active_ptiles_kernel<<<stride_ctas(g.nptiles(), ex->sms * 8), 256, 0, s>>>(g, tile_flags(seg, g), ex->plist,
                                                                               ex->plist_n);
  }
  CUDA_TRY(cudaGetLastError());
  const int exact = (flags & DISO_GRAD_EXACT) ? 1 : 0;
  // DMC: the cell records of the extractor's last forward are this band's when that
  // forward wrote this `seg` for a band of these sizes
  const bool records = ex->method == DISO_DMC && ex->codes && ex->codes_seg == seg && ex->codes_band &&
                       ex->codes_dims[0] == f.n0 && ex->codes_dims[1] == f.n1 && ex->codes_dims[2] == f.n2;
  {
    KernelTimer kt(ex, K_FUSED_BWD, s);
    if (ex->method == DISO_MC)
      brick_backward_kernel<S, MC, false><<<(unsigned)ex->brick_ctas, NTHREADS, (size_t)ex->fused_smem, s>>>(
          f, g, seg, ex->plist, ex->plist_n, (const S*)gv, normalize, 0, (S*)gval, (S*)gdef, ex->stats, nullptr);
    else if (records)
      brick_backward_kernel<S, DMC, true><<<(unsigned)ex->brick_ctas, NTHREADS, (size_t)ex->fused_smem_rec, s>>>(
          f, g, seg, ex->plist, ex->plist_n, (const S*)gv, normalize, exact, (S*)gval, (S*)gdef, ex->stats,
          ex->codes);
    else
      brick_backward_kernel<S, DMC, false><<<(unsigned)ex->brick_ctas, NTHREADS, (size_t)ex->fused_smem, s>>>(
          f, g, seg, ex->plist, ex->plist_n, (const S*)gv, normalize, exact, (S*)gval, (S*)gdef, ex->stats,
          nullptr);
  }
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

// ------------------------------------------------------------------ mesh consumers

constexpr unsigned long long MESH_ERR_INDEX = 8ull;  // Stats::error bit 3: a face index out of range

inline unsigned mesh_ctas(const diso_extractor* ex, int64_t n) { return stride_ctas(n, (unsigned)ex->sms * 8u); }

// the extractor's mesh scratch as consecutive 256-byte aligned pieces
struct MeshCarve {
  uint8_t* base;
  int64_t used = 0;
  template <class T>
  T* take(int64_t count) {
    T* p = (T*)(base + used);
    used += (count * (int64_t)sizeof(T) + 255) / 256 * 256;
    return p;
  }
};

int mesh_scratch(diso_extractor* ex, int64_t bytes) { return grow(ex->mesh, ex->mesh_cap, bytes); }

// waits for the stream; an out-of-range face index is an argument error
int mesh_finish(diso_extractor* ex, cudaStream_t s, const char* what) {
  CUDA_TRY(cudaMemcpyAsync(ex->stats_host, ex->stats, sizeof(Stats), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (ex->stats_host->error & 1ull) return fail(DISO_ERR_SCAN, "%s: scan look-back wait gave up", what);
  if (ex->stats_host->error & MESH_ERR_INDEX) return fail(DISO_ERR_ARG, "%s: a face index is out of range", what);
  return DISO_OK;
}

template <class S>
int mesh_normals(diso_extractor* ex, const S* v, int64_t nv, const int64_t* faces, int64_t nf, int k, S* out,
                 cudaStream_t s) {
  int rc;
  if ((rc = mesh_scratch(ex, nv * 24 + 512)) != DISO_OK) return rc;
  MeshCarve c{ex->mesh};
  unsigned long long* maxbits = c.take<unsigned long long>(1);
  unsigned long long* acc = c.take<unsigned long long>(3 * nv);
  if ((rc = reset_stats(ex, s)) != DISO_OK) return rc;
  CUDA_TRY(cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long), s));
  CUDA_TRY(cudaMemsetAsync(acc, 0, (size_t)(3 * nv) * sizeof(unsigned long long), s));
  if (nf > 0) {
    normals_max_kernel<S><<<mesh_ctas(ex, nf), 256, 0, s>>>(v, faces, nf, k, nv, maxbits, &ex->stats->error);
    normals_acc_kernel<S><<<mesh_ctas(ex, nf), 256, 0, s>>>(v, faces, nf, k, nv, maxbits, acc);
  }
  normals_out_kernel<S><<<mesh_ctas(ex, nv), 256, 0, s>>>(acc, nv, out);
  CUDA_TRY(cudaGetLastError());
  return mesh_finish(ex, s, "vertex normals");
}

template <class S>
int mesh_weld(diso_extractor* ex, const S* v, int64_t nv, const int64_t* faces, int64_t nf, int k, double tol,
              S* out_v, int64_t* out_f, int64_t* nv_out, int64_t* nf_out, cudaStream_t s) {
  uint32_t slots = 1024;
  while ((int64_t)slots < 2 * nv) slots <<= 1;
  int rc;
  if ((rc = mesh_scratch(ex, (int64_t)slots * 4 + nv * 4 + (nv + 1) * 8 + (nf + 1) * 8 + nf * k * 8 + 1280)) !=
      DISO_OK)
    return rc;
  MeshCarve c{ex->mesh};
  int* table = c.take<int>(slots);
  int* rep = c.take<int>(nv);
  uint64_t* keep = c.take<uint64_t>(nv + 1);
  uint64_t* keepf = c.take<uint64_t>(nf + 1);
  int64_t* mapped = c.take<int64_t>(nf * k);
  if ((rc = reset_stats(ex, s)) != DISO_OK) return rc;
  CUDA_TRY(cudaMemsetAsync(table, 0xff, (size_t)slots * sizeof(int), s));
  weld_insert_kernel<S><<<mesh_ctas(ex, nv), 256, 0, s>>>(v, nv, tol, table, slots - 1);
  weld_rep_kernel<S><<<mesh_ctas(ex, nv), 256, 0, s>>>(v, nv, tol, table, slots - 1, rep, keep);
  CUDA_TRY(cudaGetLastError());
  if ((rc = run_scan(ex, keep, nv, s)) != DISO_OK) return rc;
  if (nf > 0) {
    weld_faces_kernel<<<mesh_ctas(ex, nf), 256, 0, s>>>(faces, nf, k, nv, rep, keep, mapped, keepf,
                                                       &ex->stats->error);
    CUDA_TRY(cudaGetLastError());
  }
  if ((rc = run_scan(ex, keepf, nf, s)) != DISO_OK) return rc;
  weld_compact_verts_kernel<S><<<mesh_ctas(ex, nv), 256, 0, s>>>(v, nv, rep, keep, out_v);
  if (nf > 0) weld_compact_faces_kernel<<<mesh_ctas(ex, nf), 256, 0, s>>>(mapped, nf, k, keepf, out_f);
  CUDA_TRY(cudaGetLastError());
  uint64_t tot[2] = {0, 0};
  CUDA_TRY(cudaMemcpyAsync(&tot[0], keep + nv, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(&tot[1], keepf + nf, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  if ((rc = mesh_finish(ex, s, "weld")) != DISO_OK) return rc;
  *nv_out = (int64_t)tot[0];
  *nf_out = (int64_t)tot[1];
  return DISO_OK;
}

template <class S>
int mesh_obj(diso_extractor* ex, const S* v, const S* nrm, int64_t nv, const int64_t* faces, int64_t nf, int k,
             char* text, int64_t cap, int64_t* bytes, cudaStream_t s) {
  const int64_t lines = (nrm ? 2 * nv : nv) + nf;
  int rc;
  if ((rc = mesh_scratch(ex, (lines + 1) * 8 + 256)) != DISO_OK) return rc;
  MeshCarve c{ex->mesh};
  uint64_t* off = c.take<uint64_t>(lines + 1);
  if ((rc = reset_stats(ex, s)) != DISO_OK) return rc;
  if (lines > 0) obj_len_kernel<S><<<mesh_ctas(ex, lines), 256, 0, s>>>(v, nrm, nv, faces, nf, k, off);
  CUDA_TRY(cudaGetLastError());
  if ((rc = run_scan(ex, off, lines, s)) != DISO_OK) return rc;
  uint64_t total = 0;
  CUDA_TRY(cudaMemcpyAsync(&total, off + lines, sizeof total, cudaMemcpyDeviceToHost, s));
  if ((rc = mesh_finish(ex, s, "OBJ text")) != DISO_OK) return rc;
  *bytes = (int64_t)total;
  if (!text || (int64_t)total > cap) return DISO_OK;  // the size only
  if (lines > 0) obj_write_kernel<S><<<mesh_ctas(ex, lines), 256, 0, s>>>(v, nrm, nv, faces, nf, k, off, text);
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

template <class S>
int mesh_ply(diso_extractor* ex, const S* v, const S* nrm, int64_t nv, const int64_t* faces, int64_t nf, int k,
             uint8_t* body, cudaStream_t s) {
  const int64_t vbytes = nv * 3 * (int64_t)sizeof(S) * (nrm ? 2 : 1);
  if (nrm) {
    if (nv > 0) ply_vertex_kernel<S><<<mesh_ctas(ex, nv), 256, 0, s>>>(v, nrm, nv, (S*)body);
  } else if (vbytes > 0) {
    CUDA_TRY(cudaMemcpyAsync(body, v, (size_t)vbytes, cudaMemcpyDeviceToDevice, s));
  }
  if (nf > 0) ply_face_kernel<<<mesh_ctas(ex, nf), 256, 0, s>>>(faces, nf, k, body + vbytes);
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

// common checks of the mesh entry points
int mesh_args(diso_extractor* ex, const void* verts, int64_t nv, const int64_t* faces, int64_t nf, int k) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  if (k != 3 && k != 4) return fail(DISO_ERR_ARG, "faces must have 3 or 4 corners (got %d)", k);
  if (nv < 0 || nf < 0) return fail(DISO_ERR_ARG, "negative vertex or face count");
  if (nv >= (1ll << 31)) return fail(DISO_ERR_ARG, "too many vertices for 32-bit indices: %lld", (long long)nv);
  if ((nv && !verts) || (nf && !faces)) return fail(DISO_ERR_ARG, "null vertices or faces");
  return bind_device(ex);
}

extern "C" {

int diso_create(int method, int dtype, diso_extractor** out) {
  if (!out) return fail(DISO_ERR_ARG, "null output pointer");
  if (method != DISO_MC && method != DISO_DMC) return fail(DISO_ERR_ARG, "unknown method %d", method);
  if (dtype != DISO_F32 && dtype != DISO_F64) return fail(DISO_ERR_ARG, "unknown dtype %d", dtype);
  diso_extractor* ex = new (std::nothrow) diso_extractor();
  if (!ex) return fail(DISO_ERR_ARG, "out of host memory");
  ex->method = method;
  ex->dtype = dtype;
  *out = ex;
  return DISO_OK;
}

void diso_destroy(diso_extractor* ex) {
  if (!ex) return;
  if (ex->device >= 0) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(ex->device);
    ex->release();
    cudaSetDevice(cur);
  }
  delete ex;
}

int64_t diso_segment_slots(int nx, int ny, int nz) {
  if (nx < 1 || ny < 1 || nz < 1) return 0;
  Geom g;
  g.init(nx, ny, nz);
  return g.nseg + 1 + (2 * g.ntiles() + 7) / 8;
}

int diso_forward_count(diso_extractor* ex, const void* sdf, int nx, int ny, int nz, double isovalue, double padval,
                       uint64_t* seg, void* stream, diso_counts* out) {
  int rc = check_common(ex, sdf, nx, ny, nz);
  if (rc) return rc;
  if (!seg || !out) return fail(DISO_ERR_ARG, "null seg or counts");
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? forward_count<float>(ex, sdf, nx, ny, nz, isovalue, padval, seg, s, out)
                               : forward_count<double>(ex, sdf, nx, ny, nz, isovalue, padval, seg, s, out);
}

int diso_forward_emit(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz,
                      double isovalue, double padval, const uint64_t* seg, int normalize, void* verts,
                      int64_t* faces, uint64_t* edge_record, void* stream) {
  int rc = check_common(ex, sdf, nx, ny, nz);
  if (rc) return rc;
  if (!seg || !verts || !faces) return fail(DISO_ERR_ARG, "null seg, verts or faces");
  if (((uintptr_t)edge_record & 31u) != 0) return fail(DISO_ERR_ARG, "edge record must be 32-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? forward_emit<float>(ex, sdf, deform, nx, ny, nz, isovalue, padval, seg, normalize,
                                                     verts, faces, edge_record, s)
                               : forward_emit<double>(ex, sdf, deform, nx, ny, nz, isovalue, padval, seg, normalize,
                                                      verts, faces, edge_record, s);
}

int diso_forward(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz, double isovalue,
                 double padval, uint64_t* seg, int normalize, void* verts, int64_t vcap, int64_t* faces, int64_t fcap,
                 uint64_t* edge_record, void* stream, diso_counts* out) {
  int rc = check_common(ex, sdf, nx, ny, nz);
  if (rc) return rc;
  if (!seg || !out) return fail(DISO_ERR_ARG, "null seg or counts");
  if (vcap < 0 || fcap < 0 || (vcap && !verts) || (fcap && !faces)) return fail(DISO_ERR_ARG, "bad output buffers");
  if (((uintptr_t)edge_record & 31u) != 0) return fail(DISO_ERR_ARG, "edge record must be 32-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? forward_all<float>(ex, sdf, deform, nx, ny, nz, isovalue, padval, seg, normalize,
                                                    verts, vcap, faces, fcap, edge_record, s, out)
                               : forward_all<double>(ex, sdf, deform, nx, ny, nz, isovalue, padval, seg, normalize,
                                                     verts, vcap, faces, fcap, edge_record, s, out);
}

int64_t diso_edge_record_slots(int method, int dtype, int64_t n_verts, int64_t n_faces) {
  if ((method != DISO_MC && method != DISO_DMC) || (dtype != DISO_F32 && dtype != DISO_F64)) return 0;
  if (n_verts < 0 || n_faces < 0) return 0;
  const int64_t E = method == DISO_MC ? n_verts : n_faces;
  return edge_record_slots(method, dtype == DISO_F32 ? 4 : 8, n_verts, E);
}

int diso_split_quads(diso_extractor* ex, const void* verts, const int64_t* quads, int64_t n_quads, int64_t* tris,
                     int64_t* n_tris, void* stream) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  if (ex->method != DISO_DMC) return fail(DISO_ERR_ARG, "quad split needs a DMC extractor");
  if (!n_tris || n_quads < 0) return fail(DISO_ERR_ARG, "bad quad count");
  *n_tris = 0;
  if (n_quads == 0) return DISO_OK;
  if (!verts || !quads || !tris) return fail(DISO_ERR_ARG, "null verts, quads or tris");
  int rc = bind_device(ex);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? split_quads<float>(ex, verts, quads, n_quads, tris, n_tris, s)
                               : split_quads<double>(ex, verts, quads, n_quads, tris, n_tris, s);
}

int diso_backward(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz, double isovalue,
                  double padval, const uint64_t* seg, uint64_t* edge_record, int normalize, int flags,
                  const void* grad_verts, void* grad_sdf, void* grad_deform, void* stream) {
  if (!seg || !grad_sdf) return fail(DISO_ERR_ARG, "null seg or grad_sdf");
  if (!edge_record) return fail(DISO_ERR_ARG, "null edge record (the forward emit must record the edges)");
  if (((uintptr_t)edge_record & 31u) != 0) return fail(DISO_ERR_ARG, "edge record must be 32-byte aligned");
  if (deform && !grad_deform) return fail(DISO_ERR_ARG, "deform given without grad_deform");
  if (!grad_verts) return fail(DISO_ERR_ARG, "null grad_verts");
  int rc = check_common(ex, sdf, nx, ny, nz);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? backward<float>(ex, sdf, deform, nx, ny, nz, isovalue, padval, seg, edge_record,
                                                 normalize, flags, grad_verts, grad_sdf,
                                                 deform ? grad_deform : nullptr, s)
                               : backward<double>(ex, sdf, deform, nx, ny, nz, isovalue, padval, seg, edge_record,
                                                  normalize, flags, grad_verts, grad_sdf,
                                                  deform ? grad_deform : nullptr, s);
}

int diso_backward_recompute(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz,
                            double isovalue, double padval, const uint64_t* seg, int normalize, int flags,
                            const void* grad_verts, void* grad_sdf, void* grad_deform, void* stream) {
  if (!seg || !grad_sdf) return fail(DISO_ERR_ARG, "null seg or grad_sdf");
  if (!grad_verts) return fail(DISO_ERR_ARG, "null grad_verts");
  if (deform && !grad_deform) return fail(DISO_ERR_ARG, "deform given without grad_deform");
  int rc = check_common(ex, sdf, nx, ny, nz);
  if (rc != DISO_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  void* gd = deform ? grad_deform : nullptr;
  return ex->dtype == DISO_F32 ? backward_fused<float>(ex, sdf, deform, nx, ny, nz, isovalue, padval, seg,
                                                        normalize, flags, grad_verts, grad_sdf, gd, s)
                               : backward_fused<double>(ex, sdf, deform, nx, ny, nz, isovalue, padval, seg,
                                                         normalize, flags, grad_verts, grad_sdf, gd, s);
}

int diso_isovalue_grad(diso_extractor* ex, const void* grad_sdf, int nx, int ny, int nz, const uint64_t* seg,
                       double* grad_iso, void* stream) {
  if (!grad_iso) return fail(DISO_ERR_ARG, "null grad_iso");
  int rc = check_common(ex, grad_sdf, nx, ny, nz);
  if (rc) return rc;
  Geom g;
  g.init(nx, ny, nz);
  if ((rc = grow(ex->isog, ex->isog_cap, ISO_GRAD_CTAS)) != DISO_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const uint8_t* flags = seg ? tile_flags(seg, g) : nullptr;
  if (ex->dtype == DISO_F32)
    iso_grad_partial_kernel<float><<<ISO_GRAD_CTAS, 256, 0, s>>>(g, flags, (const float*)grad_sdf, ex->isog);
  else
    iso_grad_partial_kernel<double><<<ISO_GRAD_CTAS, 256, 0, s>>>(g, flags, (const double*)grad_sdf, ex->isog);
  CUDA_TRY(cudaGetLastError());
  iso_grad_final_kernel<<<1, 256, 0, s>>>(ex->isog, ISO_GRAD_CTAS, grad_iso);
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

double diso_zero_count_share(void) { return ZERO_COUNT_SHARE; }

int diso_zero_grads(diso_extractor* ex, void* grad_sdf, int64_t sdf_bytes, void* grad_deform, int64_t deform_bytes,
                    void* stream, void* zero_stream) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  if (sdf_bytes < 0 || deform_bytes < 0 || (sdf_bytes && !grad_sdf) || (deform_bytes && !grad_deform))
    return fail(DISO_ERR_ARG, "bad gradient buffers");
  int rc = bind_device(ex);
  if (rc) return rc;
  cudaStream_t z = zero_stream ? (cudaStream_t)zero_stream : ex->side;
  return zero_grads(ex, grad_sdf, sdf_bytes, grad_deform, deform_bytes, (cudaStream_t)stream, z);
}

int64_t diso_batch_record_slots(const diso_grid* grids, int ngrids) {
  if (!grids || ngrids < 1 || ngrids > MAX_BATCH) return 0;
  return batch_record_slots(grids, ngrids, nullptr, nullptr);
}

int diso_batch_prepare(diso_extractor* ex, const diso_grid* grids, int ngrids, uint64_t* record, void* stream) {
  if (!ex || !grids || !record) return fail(DISO_ERR_ARG, "null extractor, grids or record");
  if (ngrids < 1 || ngrids > MAX_BATCH) return fail(DISO_ERR_ARG, "batch of %d grids (1..%d)", ngrids, MAX_BATCH);
  int64_t tiles = 0;
  for (int i = 0; i < ngrids; ++i) {
    int rc = check_common(ex, grids[i].sdf, grids[i].nx, grids[i].ny, grids[i].nz);
    if (rc) return rc;
    Geom g;
    g.init(grids[i].nx, grids[i].ny, grids[i].nz);
    if (g.ntiles() >= (1ll << BATCH_TILE_BITS)) return fail(DISO_ERR_ARG, "grid %d too large for a batch", i);
    tiles += g.ntiles();
  }
  int64_t segs = 0;
  batch_record_slots(grids, ngrids, &segs, &tiles);
  if (3.0 * (double)segs * TZ >= 2147483647.0) return fail(DISO_ERR_ARG, "batch too large for 32-bit counts");
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? batch_prepare<float>(ex, grids, ngrids, record, s)
                               : batch_prepare<double>(ex, grids, ngrids, record, s);
}

int diso_batch_count(diso_extractor* ex, void* stream) {
  if (!ex || ex->bn < 1) return fail(DISO_ERR_ARG, "no prepared batch");
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? batch_count<float>(ex, s) : batch_count<double>(ex, s);
}

int diso_batch_results(diso_extractor* ex, diso_counts* per_grid, int64_t* vert_offset, int64_t* face_offset,
                       int* overflow, void* stream) {
  if (!ex || ex->bn < 1 || !per_grid) return fail(DISO_ERR_ARG, "no prepared batch or null output");
  return batch_results(ex, per_grid, vert_offset, face_offset, overflow, (cudaStream_t)stream);
}

int diso_batch_emit(diso_extractor* ex, int normalize, void* verts, int64_t vcap, int64_t* faces, int64_t fcap,
                    uint64_t* edge_record, void* stream) {
  if (!ex || ex->bn < 1) return fail(DISO_ERR_ARG, "no prepared batch");
  if ((!verts && vcap) || (!faces && fcap) || vcap < 0 || fcap < 0) return fail(DISO_ERR_ARG, "bad output buffers");
  if (((uintptr_t)edge_record & 31u) != 0) return fail(DISO_ERR_ARG, "edge record must be 32-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? batch_emit<float>(ex, normalize, verts, vcap, faces, fcap, edge_record, s)
                               : batch_emit<double>(ex, normalize, verts, vcap, faces, fcap, edge_record, s);
}

int diso_batch_backward(diso_extractor* ex, int normalize, int flags, const void* grad_verts, uint64_t* edge_record,
                        int64_t vcap, int64_t fcap, void* stream) {
  if (!ex || ex->bn < 1) return fail(DISO_ERR_ARG, "no prepared batch");
  if (!grad_verts) return fail(DISO_ERR_ARG, "null grad_verts");
  if (!edge_record) return fail(DISO_ERR_ARG, "null edge record (the batch emit must record the edges)");
  if (((uintptr_t)edge_record & 31u) != 0) return fail(DISO_ERR_ARG, "edge record must be 32-byte aligned");
  if (vcap < 0 || fcap < 0) return fail(DISO_ERR_ARG, "bad capacities");
  for (int i = 0; i < ex->bn; ++i) {
    const bool missing = ex->dtype == DISO_F32 ? ((const BatchGrid<float>*)ex->bdesc_host)[i].gsdf == nullptr
                                               : ((const BatchGrid<double>*)ex->bdesc_host)[i].gsdf == nullptr;
    if (missing) return fail(DISO_ERR_ARG, "grid %d of the batch has no grad_sdf", i);
  }
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? batch_backward<float>(ex, normalize, flags, grad_verts, edge_record, vcap, fcap, s)
                               : batch_backward<double>(ex, normalize, flags, grad_verts, edge_record, vcap, fcap, s);
}

int diso_timing(diso_extractor* ex, int enable) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  ex->timing = enable != 0;
  for (const diso_extractor::Timed& t : ex->timed) {
    ex->event_pool.push_back(t.a);
    ex->event_pool.push_back(t.b);
  }
  ex->timed.clear();
  return DISO_OK;
}

int diso_timing_read(diso_extractor* ex, diso_kernel_time* out, int max, int* n) {
  if (!ex || !n || (max > 0 && !out)) return fail(DISO_ERR_ARG, "null extractor or output");
  double ms[K_NKERNELS] = {};
  int64_t launches[K_NKERNELS] = {};
  for (const diso_extractor::Timed& t : ex->timed) {
    CUDA_TRY(cudaEventSynchronize(t.b));
    float e = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&e, t.a, t.b));
    ms[t.id] += e;
    launches[t.id] += 1;
  }
  diso_timing(ex, ex->timing ? 1 : 0);  // recycle the events
  int k = 0;
  for (int i = 0; i < K_NKERNELS; ++i) {
    if (!launches[i]) continue;
    if (k < max) {
      snprintf(out[k].name, sizeof out[k].name, "%s", kKernelNames[i]);
      out[k].launches = launches[i];
      out[k].total_ms = ms[i];
    }
    ++k;
  }
  *n = std::min(k, max);
  return DISO_OK;
}

int diso_tune_set(diso_extractor* ex, int param, int value) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  if (param < 0 || param >= DISO_TUNE_N) return fail(DISO_ERR_ARG, "unknown launch parameter %d", param);
  const int hi = param == DISO_TUNE_ZERO_SHARE ? 1000 : 64;
  if (value < 0 || value > hi) return fail(DISO_ERR_ARG, "value %d of launch parameter %d outside [0, %d]", value, param, hi);
  ex->tune[param] = value;
  if (param == DISO_TUNE_ZERO_SHARE) ex->zero_share = value > 0 ? value / 1000.0 : ZERO_COUNT_SHARE;
  return DISO_OK;
}

int diso_tune_value(const diso_extractor* ex, int param) {
  if (!ex || param < 0 || param >= DISO_TUNE_N) return -1;
  return ex->tune[param];
}

int diso_scan_wait_probe(diso_extractor* ex, unsigned spin_limit, void* stream) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  if (spin_limit < 1 || spin_limit > SCAN_SPIN_LIMIT)
    return fail(DISO_ERR_ARG, "spin limit %u outside [1, %u]", spin_limit, SCAN_SPIN_LIMIT);
  int rc = bind_device(ex);
  if (rc != DISO_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  // two whole scan tiles in the extractor's split scratch; only tile 1 runs
  const int64_t n = 2 * (int64_t)SCAN_TILE;
  if ((rc = grow(ex->split, ex->split_cap, n + 1)) != DISO_OK) return rc;
  const int64_t tiles = scan_reserve(ex, n);
  if (tiles == 0) return DISO_ERR_CUDA;
  CUDA_TRY(cudaMemsetAsync(ex->split, 0, (size_t)(n + 1) * sizeof(uint64_t), s));
  scan_probe_prep_kernel<<<1, 64, 0, s>>>(ex->stats, ex->scan_flag, tiles, 1ull);
  CUDA_TRY(cudaGetLastError());
  ScanState st{ex->scan_flag, ex->scan_agg, ex->scan_incl};
  scan_lookback_kernel<<<1, SCAN_THREADS, 0, s>>>(ex->split, n, st, ex->stats, nullptr, spin_limit);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(ex->stats_host, ex->stats, sizeof(Stats), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (ex->stats_host->error & 1ull) return fail(DISO_ERR_SCAN, "segment scan: look-back wait gave up");
  return DISO_OK;
}

int64_t diso_scratch_bytes(const diso_extractor* ex) {
  if (!ex) return 0;
  int64_t b = ex->active_cap * (int64_t)sizeof(int) + ex->codes_cap * (int64_t)sizeof(CellRec) +
              ex->fpart_cap * (int64_t)sizeof(double) +
              ex->plist_cap * (int64_t)sizeof(int) + ex->split_cap * (int64_t)sizeof(uint64_t) + ex->mesh_cap +
              ex->isog_cap * (int64_t)sizeof(double) +
              ex->scan_cap * (int64_t)(sizeof(uint32_t) + 2 * sizeof(uint64_t));
  if (ex->stats) b += (int64_t)sizeof(Stats) + (int64_t)sizeof(unsigned);
  if (ex->bdesc)
    b += (int64_t)(sizeof(BatchGrid<double>) * MAX_BATCH + sizeof(Stats) * MAX_BATCH +
                   sizeof(uint64_t) * (MAX_BATCH + 1) + sizeof(int64_t) * (MAX_BATCH + 1));
  return b;
}

const char* diso_last_error(void) { return g_err; }

const char* diso_version(void) { return "diso_gb300 0.1.0 (sm_103a)"; }


int diso_mesh_normals(diso_extractor* ex, const void* verts, int64_t n_verts, const int64_t* faces, int64_t n_faces,
                      int corners, void* normals, void* stream) {
  int rc = mesh_args(ex, verts, n_verts, faces, n_faces, corners);
  if (rc) return rc;
  if (n_verts && !normals) return fail(DISO_ERR_ARG, "null normals");
  if (n_verts == 0) return DISO_OK;
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32
             ? mesh_normals<float>(ex, (const float*)verts, n_verts, faces, n_faces, corners, (float*)normals, s)
             : mesh_normals<double>(ex, (const double*)verts, n_verts, faces, n_faces, corners, (double*)normals, s);
}

int diso_mesh_weld(diso_extractor* ex, const void* verts, int64_t n_verts, const int64_t* faces, int64_t n_faces,
                   int corners, double tol, void* out_verts, int64_t* out_faces, int64_t* n_verts_out,
                   int64_t* n_faces_out, void* stream) {
  int rc = mesh_args(ex, verts, n_verts, faces, n_faces, corners);
  if (rc) return rc;
  if (!n_verts_out || !n_faces_out) return fail(DISO_ERR_ARG, "null output counts");
  if (!(tol >= 0.0)) return fail(DISO_ERR_ARG, "tolerance must be >= 0");
  if ((n_verts && !out_verts) || (n_faces && !out_faces)) return fail(DISO_ERR_ARG, "null output vertices or faces");
  *n_verts_out = *n_faces_out = 0;
  if (n_verts == 0) return n_faces ? fail(DISO_ERR_ARG, "weld: faces without vertices") : DISO_OK;
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? mesh_weld<float>(ex, (const float*)verts, n_verts, faces, n_faces, corners, tol,
                                                  (float*)out_verts, out_faces, n_verts_out, n_faces_out, s)
                               : mesh_weld<double>(ex, (const double*)verts, n_verts, faces, n_faces, corners, tol,
                                                   (double*)out_verts, out_faces, n_verts_out, n_faces_out, s);
}

int diso_mesh_obj(diso_extractor* ex, const void* verts, const void* normals, int64_t n_verts, const int64_t* faces,
                  int64_t n_faces, int corners, char* text, int64_t text_cap, int64_t* text_bytes, void* stream) {
  int rc = mesh_args(ex, verts, n_verts, faces, n_faces, corners);
  if (rc) return rc;
  if (!text_bytes || text_cap < 0) return fail(DISO_ERR_ARG, "null text size or negative capacity");
  *text_bytes = 0;
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? mesh_obj<float>(ex, (const float*)verts, (const float*)normals, n_verts, faces,
                                                 n_faces, corners, text, text_cap, text_bytes, s)
                               : mesh_obj<double>(ex, (const double*)verts, (const double*)normals, n_verts, faces,
                                                  n_faces, corners, text, text_cap, text_bytes, s);
}

int64_t diso_mesh_ply_bytes(int dtype, int64_t n_verts, int64_t n_faces, int corners, int with_normals) {
  if ((dtype != DISO_F32 && dtype != DISO_F64) || (corners != 3 && corners != 4) || n_verts < 0 || n_faces < 0)
    return -1;
  return n_verts * 3 * (dtype == DISO_F32 ? 4 : 8) * (with_normals ? 2 : 1) + n_faces * (1 + 4 * corners);
}

int diso_mesh_ply(diso_extractor* ex, const void* verts, const void* normals, int64_t n_verts, const int64_t* faces,
                  int64_t n_faces, int corners, void* body, void* stream) {
  int rc = mesh_args(ex, verts, n_verts, faces, n_faces, corners);
  if (rc) return rc;
  if (!body && (n_verts || n_faces)) return fail(DISO_ERR_ARG, "null body buffer");
  cudaStream_t s = (cudaStream_t)stream;
  return ex->dtype == DISO_F32 ? mesh_ply<float>(ex, (const float*)verts, (const float*)normals, n_verts, faces,
                                                 n_faces, corners, (uint8_t*)body, s)
                               : mesh_ply<double>(ex, (const double*)verts, (const double*)normals, n_verts, faces,
                                                  n_faces, corners, (uint8_t*)body, s);
}


int diso_forward_field(diso_extractor* ex, const diso_sphere_field* field, int nx, int ny, int nz, double isovalue,
                       double padval, uint64_t* seg, int normalize, void* verts, int64_t vcap, int64_t* faces,
                       int64_t fcap, void* stream, diso_counts* out) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  int rc = check_field(field, nx, ny, nz);
  if (rc) return rc;
  if (!seg || !out) return fail(DISO_ERR_ARG, "null seg or counts");
  if (vcap < 0 || fcap < 0 || (vcap && !verts) || (fcap && !faces)) return fail(DISO_ERR_ARG, "bad output buffers");
  if ((rc = bind_device(ex)) != DISO_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (ex->dtype == DISO_F32)
    return forward_field<float>(ex, make_sphere_field<float>(field, nx, ny, nz, isovalue, padval), isovalue, seg,
                                normalize, verts, vcap, faces, fcap, s, out);
  return forward_field<double>(ex, make_sphere_field<double>(field, nx, ny, nz, isovalue, padval), isovalue, seg,
                               normalize, verts, vcap, faces, fcap, s, out);
}

int diso_backward_field(diso_extractor* ex, const diso_sphere_field* field, int nx, int ny, int nz, double isovalue,
                        double padval, const uint64_t* seg, int normalize, int flags, const void* grad_verts,
                        double* grad_spheres, void* grad_deform, void* stream) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  int rc = check_field(field, nx, ny, nz);
  if (rc != DISO_OK) return rc;
  if (field->count > FIELD_BWD_MAX_SPHERES)
    return fail(DISO_ERR_ARG, "the field backward takes at most %d spheres (got %d)", FIELD_BWD_MAX_SPHERES,
                field->count);
  if (!seg || !grad_verts || !grad_spheres) return fail(DISO_ERR_ARG, "null seg, grad_verts or grad_spheres");
  if (field->deform && !grad_deform) return fail(DISO_ERR_ARG, "a field with a deform needs grad_deform");
  if ((rc = check_common(ex, field->spheres, nx, ny, nz)) != DISO_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  void* gd = field->deform ? grad_deform : nullptr;
  return ex->dtype == DISO_F32
             ? backward_field<float>(ex, make_sphere_field<float>(field, nx, ny, nz, isovalue, padval), seg, normalize,
                                     flags, grad_verts, grad_spheres, gd, s)
             : backward_field<double>(ex, make_sphere_field<double>(field, nx, ny, nz, isovalue, padval), seg,
                                      normalize, flags, grad_verts, grad_spheres, gd, s);
}

int diso_field_materialize(int dtype, const diso_sphere_field* field, int nx, int ny, int nz, void* sdf,
                           void* stream) {
  if (dtype != DISO_F32 && dtype != DISO_F64) return fail(DISO_ERR_ARG, "unknown dtype %d", dtype);
  int rc = check_field(field, nx, ny, nz);
  if (rc) return rc;
  if (!sdf) return fail(DISO_ERR_ARG, "null output grid");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n = (int64_t)nx * ny * nz;
  const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 65536);
  if (dtype == DISO_F32)
    field_materialize_kernel<float><<<blocks, 256, 0, s>>>(make_sphere_field<float>(field, nx, ny, nz, 0.0, 1.0),
                                                          (float*)sdf);
  else
    field_materialize_kernel<double><<<blocks, 256, 0, s>>>(make_sphere_field<double>(field, nx, ny, nz, 0.0, 1.0),
                                                           (double*)sdf);
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

int diso_forward_bricks(diso_extractor* ex, const diso_brick_grid* bricks, double isovalue, double padval,
                        uint64_t* seg, int normalize, void* verts, int64_t vcap, int64_t* faces, int64_t fcap,
                        void* stream, diso_counts* out) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  int rc = check_bricks(bricks);
  if (rc) return rc;
  if (!seg || !out) return fail(DISO_ERR_ARG, "null seg or counts");
  if (vcap < 0 || fcap < 0 || (vcap && !verts) || (fcap && !faces)) return fail(DISO_ERR_ARG, "bad output buffers");
  if ((rc = bind_device(ex)) != DISO_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  Geom g;
  g.init(bricks->dims[0], bricks->dims[1], bricks->dims[2]);
  if (ex->method == DISO_DMC && (rc = grow(ex->umap, ex->umap_cap, count_units(g))) != DISO_OK) return rc;
  int* umap = ex->method == DISO_DMC ? ex->umap : nullptr;
  if (ex->dtype == DISO_F32) {
    if ((rc = validate_bricks<float>(ex, bricks, isovalue, padval, s)) != DISO_OK) return rc;
    return forward_field<float>(ex, make_brick_field<float>(bricks, isovalue, padval, umap), isovalue, seg,
                                normalize, verts, vcap, faces, fcap, s, out, umap);
  }
  if ((rc = validate_bricks<double>(ex, bricks, isovalue, padval, s)) != DISO_OK) return rc;
  return forward_field<double>(ex, make_brick_field<double>(bricks, isovalue, padval, umap), isovalue, seg,
                               normalize, verts, vcap, faces, fcap, s, out, umap);
}

int diso_backward_bricks(diso_extractor* ex, const diso_brick_grid* bricks, double isovalue, double padval,
                         const uint64_t* seg, int normalize, int flags, const void* grad_verts, void* grad_values,
                         void* grad_deform, void* stream) {
  if (!ex) return fail(DISO_ERR_ARG, "null extractor");
  int rc = check_bricks(bricks);
  if (rc) return rc;
  if (!seg || !grad_verts) return fail(DISO_ERR_ARG, "null seg or grad_verts");
  if (bricks->count && !grad_values) return fail(DISO_ERR_ARG, "null grad_values");
  if (bricks->deform && !grad_deform) return fail(DISO_ERR_ARG, "a band with a deform needs grad_deform");
  if ((rc = bind_device(ex)) != DISO_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  void* gd = bricks->deform ? grad_deform : nullptr;
  return ex->dtype == DISO_F32
             ? backward_bricks<float>(ex, make_brick_field<float>(bricks, isovalue, padval, ex->umap), bricks->count, seg,
                                      normalize, flags, grad_verts, grad_values, gd, s)
             : backward_bricks<double>(ex, make_brick_field<double>(bricks, isovalue, padval, ex->umap), bricks->count,
                                       seg,
                                       normalize, flags, grad_verts, grad_values, gd, s);
}

int diso_bricks_materialize(int dtype, const diso_brick_grid* bricks, void* sdf, void* deform, void* stream) {
  if (dtype != DISO_F32 && dtype != DISO_F64) return fail(DISO_ERR_ARG, "unknown dtype %d", dtype);
  int rc = check_bricks(bricks);
  if (rc) return rc;
  if (!sdf) return fail(DISO_ERR_ARG, "null output grid");
  if (deform && !bricks->deform) return fail(DISO_ERR_ARG, "a dense deform asked of a band without one");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n = (int64_t)bricks->dims[0] * bricks->dims[1] * bricks->dims[2];
  const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 65536);
  if (dtype == DISO_F32)
    bricks_materialize_kernel<float><<<blocks, 256, 0, s>>>(make_brick_field<float>(bricks, 0.0, 1.0), (float*)sdf,
                                                            (float*)deform);
  else
    bricks_materialize_kernel<double><<<blocks, 256, 0, s>>>(make_brick_field<double>(bricks, 0.0, 1.0),
                                                             (double*)sdf, (double*)deform);
  CUDA_TRY(cudaGetLastError());
  return DISO_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// diso_forward_count_static: the forward count phase without any allocation.
//
// Its scratch (status words, the list of active tiles, the look-back state of
// the scan) lives in one file-scope device array instead of buffers owned by an
// extractor.  Host code cannot use the array's name as a device address, so at
// the first call on each device (with that device current) the address is looked
// up with cudaGetSymbolAddress and cached, keyed by the device's current context:
// a context made again after cudaDeviceReset gets a fresh lookup.
namespace {

constexpr int64_t kStaticMaxTiles = 65536;      // 4x8x32-cell tiles of one grid
// look-back tiles of SCAN_TILE (512 x 16 = 8192) segments each.  A grid of at most
// kStaticMaxTiles tiles has at most 65536 x 32 row segments (2.1M), i.e. about 256
// scan tiles, so the tile limit above is the one that applies.
constexpr int64_t kStaticMaxScanTiles = 2048;

struct StaticScratch {
  Stats stats;
  uint32_t scan_flag[kStaticMaxScanTiles];
  uint64_t scan_agg[kStaticMaxScanTiles];
  uint64_t scan_incl[kStaticMaxScanTiles];
  int active[kStaticMaxTiles];
};

__device__ __align__(256) unsigned char g_static_scratch[sizeof(StaticScratch)];

constexpr int kStaticMaxDevices = 64;
std::mutex g_static_mu;
StaticScratch* g_static_ptr[kStaticMaxDevices] = {};
void* g_static_ctx[kStaticMaxDevices] = {};    // the context the cached address belongs to
int g_static_ctas[kStaticMaxDevices][4] = {};  // resident count-kernel CTAs per (method, dtype)

// the calling thread's current driver context (cuCtxGetCurrent, looked up once)
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
void* current_context() {
  static std::once_flag once;
  static CtxGetCurrentFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (CtxGetCurrentFn)p;
  });
  CUcontext c = nullptr;
  if (fn && fn(&c) != CUDA_SUCCESS) c = nullptr;
  return (void*)c;
}

int static_setup(int dev, StaticScratch** out, int method, int dtype, int* ctas) {
  if (dev < 0 || dev >= kStaticMaxDevices) return fail(DISO_ERR_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_static_mu);
  // (before the thread's first runtime call no context may be current yet: the
  // lookup below makes the primary context current, and the key is read after it)
  void* ctx = current_context();
  if (!g_static_ptr[dev] || !ctx || g_static_ctx[dev] != ctx) {
    void* p = nullptr;
    CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
    int sms = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int per[4] = {0, 0, 0, 0};
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[0], count_kernel<float, MC>, NTHREADS, 0));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[1], count_kernel<float, DMC>, NTHREADS, 0));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[2], count_kernel<double, MC>, NTHREADS, 0));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[3], count_kernel<double, DMC>, NTHREADS, 0));
    for (int k = 0; k < 4; ++k) g_static_ctas[dev][k] = sms * std::max(per[k], 1);
    g_static_ptr[dev] = (StaticScratch*)p;
    g_static_ctx[dev] = current_context();
  }
  *out = g_static_ptr[dev];
  *ctas = g_static_ctas[dev][2 * dtype + method];
  return DISO_OK;
}

template <class S>
int forward_count_static(int method, StaticScratch* sc, int ctas, const void* sdf, int nx, int ny, int nz,
                         double iso, double padval, uint64_t* seg, cudaStream_t s, diso_counts* out) {
  Geom g;
  g.init(nx, ny, nz);
  // clear what must start at zero (the array keeps the previous call's contents)
  CUDA_TRY(cudaMemsetAsync(&sc->stats, 0, sizeof(Stats), s));
  CUDA_TRY(cudaMemsetAsync(&sc->stats.min_key, 0xff, sizeof(unsigned long long), s));
  Field<S> f = make_field<S>(sdf, nullptr, nx, ny, nz, iso, padval);
  const int64_t units = count_units(g);
  const int64_t want = std::max<int64_t>(ctas, (units * COUNT_TILES_PER_UNIT + COUNT_LIST - 1) / COUNT_LIST);
  const unsigned grid = (unsigned)std::min<int64_t>(want, units);
  if (method == DISO_MC)
    count_kernel<S, MC><<<grid, NTHREADS, 0, s>>>(f, g, seg, tile_flags(seg, g), nullptr, &sc->stats, sc->active);
  else
    count_kernel<S, DMC><<<grid, NTHREADS, 0, s>>>(f, g, seg, tile_flags(seg, g), nullptr, &sc->stats, sc->active);
  CUDA_TRY(cudaGetLastError());
  const int64_t tiles = (g.nseg + 1 + SCAN_TILE - 1) / SCAN_TILE;
  CUDA_TRY(cudaMemsetAsync(sc->scan_flag, 0, (size_t)tiles * sizeof(uint32_t), s));
  ScanState st{sc->scan_flag, sc->scan_agg, sc->scan_incl};
  scan_lookback_kernel<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(seg, g.nseg, st, &sc->stats, nullptr,
                                                                SCAN_SPIN_LIMIT);
  CUDA_TRY(cudaGetLastError());
  Stats h;
  uint64_t total = 0;
  CUDA_TRY(cudaMemcpyAsync(&h, &sc->stats, sizeof(Stats), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(&total, seg + g.nseg, sizeof total, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (h.error & 1ull) return fail(DISO_ERR_SCAN, "segment scan: look-back wait gave up");
  if (method == DISO_MC) {
    out->n_verts = Counts::lo(total);
    out->n_faces = Counts::hi(total);
  } else {
    out->n_verts = Counts::hi(total);
    out->n_faces = Counts::lo(total);
  }
  out->sdf_min = key_to_double(h.min_key);
  out->sdf_max = key_to_double(h.max_key);
  const double isoS = (double)(S)iso;
  out->empty = (out->sdf_min >= isoS || out->sdf_max <= isoS) ? 1 : 0;
  out->emitted = 0;
  out->n_active_tiles = (int64_t)h.n_active;
  return DISO_OK;
}

}  // namespace

extern "C" int diso_forward_count_static(int method, int dtype, const void* sdf, int nx, int ny, int nz,
                                         double isovalue, double padval, uint64_t* seg, void* stream,
                                         diso_counts* out) {
  if (method != DISO_MC && method != DISO_DMC) return fail(DISO_ERR_ARG, "unknown method %d", method);
  if (dtype != DISO_F32 && dtype != DISO_F64) return fail(DISO_ERR_ARG, "unknown dtype %d", dtype);
  if (!sdf || !seg || !out) return fail(DISO_ERR_ARG, "null sdf, seg or counts");
  if (nx < 1 || ny < 1 || nz < 1) return fail(DISO_ERR_ARG, "grid dims must be >= 1 (got %d x %d x %d)", nx, ny, nz);
  Geom g;
  g.init(nx, ny, nz);
  const int64_t scan_tiles = (g.nseg + 1 + SCAN_TILE - 1) / SCAN_TILE;
  if (g.ntiles() > kStaticMaxTiles || scan_tiles > kStaticMaxScanTiles)
    return fail(DISO_ERR_ARG,
                "grid %d x %d x %d too large for diso_forward_count_static: %lld tiles (max %lld), %lld scan tiles "
                "(max %lld); use diso_forward_count",
                nx, ny, nz, (long long)g.ntiles(), (long long)kStaticMaxTiles, (long long)scan_tiles,
                (long long)kStaticMaxScanTiles);
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  StaticScratch* sc = nullptr;
  int ctas = 0;
  int rc = static_setup(dev, &sc, method, dtype, &ctas);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return dtype == DISO_F32
             ? forward_count_static<float>(method, sc, ctas, sdf, nx, ny, nz, isovalue, padval, seg, s, out)
             : forward_count_static<double>(method, sc, ctas, sdf, nx, ny, nz, isovalue, padval, seg, s, out);
}
