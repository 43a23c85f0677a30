/*
 * C ABI of the GB300 differentiable iso-surface extractor.
 *
 * This is the boundary a binding of the reference's extension would call instead
 * of its pybind11 classes CUMCFloat / CUMCDouble / CUDMCFloat / CUDMCDouble
 * (src/pybind.cpp:13-397, registered at src/pybind.cpp:419-447).  Every entry
 * point takes plain device pointers, sizes, the isovalue and a CUDA stream
 * (cudaStream_t passed as void*; NULL = the legacy default stream), and returns
 * a status code (DISO_OK = 0); diso_last_error() gives the message of the last
 * failure on the calling thread.  No exception crosses the ABI.
 *
 * Layouts are the reference's: sdf [nx][ny][nz] (z fastest), deform
 * [nx][ny][nz][3], verts [V][3], faces [F][3] (MC, DMC triangles) or [F][4]
 * (DMC quads) as int64.  The pad of one voxel that the reference's Python layer
 * adds (diso/__init__.py:52-54) is applied virtually: pass the unpadded grid and
 * padval = isovalue + 1 rounded to the grid's dtype.  Vertices come out already
 * shifted and, with normalize != 0, divided by (dim - 1) (diso/__init__.py:56-60).
 *
 * A forward is two calls.  diso_forward_count classifies every cell, scans the
 * per-row-segment counts into the caller's `seg` array and returns the output
 * sizes (one device-to-host copy, the only synchronisation of the forward);
 * the caller then allocates verts/faces and calls diso_forward_emit with the
 * same inputs and `seg`.  `seg` (diso_segment_slots() uint64 values: the
 * scanned per-segment counts, their total and two activity bytes per tile) and,
 * when gradients will be wanted, the edge record that diso_forward_emit fills
 * (diso_edge_record_slots() uint64 values: every crossing edge's cell and axis,
 * for DMC the patches around it, and room for the backward's per-edge adjoints)
 * are all the per-call state: keep both to run diso_backward later.
 *
 * An extractor owns small scratch buffers (scan look-back state, the list of
 * tiles with crossings, status words) that grow on demand; calls on one
 * extractor must not overlap, and diso_forward_emit must follow the
 * diso_forward_count of the same grid on that extractor.
 */
#ifndef DISO_GB300_H
#define DISO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { DISO_MC = 0, DISO_DMC = 1 };
enum { DISO_F32 = 0, DISO_F64 = 1 };
enum { DISO_GRAD_EXACT = 1, DISO_GRAD_ZEROED = 2 }; /* diso_backward flags, see there */
enum {
  DISO_OK = 0,
  DISO_ERR_ARG = 1,      /* bad argument (size, null pointer, method, dtype) */
  DISO_ERR_CUDA = 2,     /* a CUDA call failed */
  DISO_ERR_SCAN = 3,     /* a bounded device-side wait gave up (scan look-back, TMA copy) */
  DISO_ERR_CAPACITY = 4, /* an output would exceed the caller's capacity */
};

typedef struct diso_extractor diso_extractor;

typedef struct {
  int64_t n_verts;        /* MC: crossing edges; DMC: patches (dual vertices) */
  int64_t n_faces;        /* MC: triangles; DMC: quads (= crossing edges) */
  double sdf_min;         /* min and max of the (unpadded) SDF */
  double sdf_max;
  int32_t empty;          /* 1 when the reference's guard returns an empty mesh:
                             min >= isovalue or max <= isovalue (diso/__init__.py:49, 103) */
  int32_t emitted;        /* diso_forward: 1 when the outputs fitted their capacities and were written */
  int64_t n_active_tiles; /* 4x8x32-cell tiles holding a crossing, a face or a patch */
} diso_counts;

/* Create an extractor for method DISO_MC / DISO_DMC and dtype DISO_F32 / DISO_F64.
 * Replaces constructing CUMCFloat, CUMCDouble, CUDMCFloat or CUDMCDouble
 * (src/pybind.cpp:419-447; diso/__init__.py:10-16, 64-70). */
int diso_create(int method, int dtype, diso_extractor** out);

/* Free the extractor's scratch (the reference's ~CUMC / ~CUDMC, src/pybind.cpp:27-39, 219-232). */
void diso_destroy(diso_extractor* ex);

/* Number of uint64 slots of the per-call `seg` array for an nx*ny*nz grid.  The
 * caller owns this per-call state; the reference keeps its per-cell scan buffers in
 * the extension object and grows them there (ensure_* in src/cumc.cu:177-263,
 * src/cudualmc.cu:515-603). */
int64_t diso_segment_slots(int nx, int ny, int nz);

/* Forward, phase 1: case codes, counts, scan and the empty-surface guard.
 * Replaces CuMC::forward / CUDualMC::forward up to their last scan
 * (src/cumc.cu:651-723, src/cudualmc.cu:1058-1122), the guard's min/max
 * (diso/__init__.py:49, 103) and the pad (diso/__init__.py:52-54).
 *
 * Sizes: at most 16384 points per axis and 2^36 cells.  The output counts are
 * scanned in 32 bits: a grid of fewer than 2^31 / 3 cells (about 890^3) always fits;
 * for a larger one the count's 64-bit sums are checked, and counts of 2^31 or more
 * (crossings, or triangles / patches) are DISO_ERR_ARG.  diso_forward then waits for
 * that check before its emit. */
int diso_forward_count(diso_extractor* ex, const void* sdf, int nx, int ny, int nz, double isovalue, double padval,
                       uint64_t* seg, void* stream, diso_counts* out);

/* Forward, phase 2: writes verts [n_verts][3] (grid dtype) and faces as int64
 * [n_faces][3] (MC) or [n_faces][4] (DMC quads).  deform may be NULL.
 * edge_record (32-byte aligned, diso_edge_record_slots() uint64 values) is filled
 * for a later diso_backward; pass NULL when no gradient will be taken.
 * Replaces create_cell_mc_verts / create_cell_mc_tris (src/cumc.cu:370-410, 564-649),
 * index_cell_mc_verts / create_dmc_verts / create_quads (src/cudualmc.cu:753-794,
 * 907-955, 1027-1056), the outputs' clone (src/pybind.cpp:78-87, 271-280) and the
 * shift / normalisation (diso/__init__.py:56-60). */
int diso_forward_emit(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz,
                      double isovalue, double padval, const uint64_t* seg, int normalize, void* verts,
                      int64_t* faces, uint64_t* edge_record, void* stream);

/* The whole forward in one call (CuMC::forward / CUDualMC::forward entire,
 * src/cumc.cu:652-732, src/cudualmc.cu:1059-1128, with the Python layer's guard, pad
 * and normalisation): count, scan and emit into verts [vcap][3] and faces
 * [fcap][3|4] (and edge_record, laid out for the actual counts; NULL without a
 * backward), synchronising the stream once at the end, so that the emit follows the
 * count on the GPU without a host round trip.  out->emitted = 1 when the outputs fitted
 * (n_verts <= vcap and n_faces <= fcap) and were written; otherwise nothing was
 * emitted and the caller runs diso_forward_emit with buffers of the reported sizes
 * (the count is done).  Capacities come from the caller's expectation, e.g. the last
 * call on grids of this size. */
int diso_forward(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz, double isovalue,
                 double padval, uint64_t* seg, int normalize, void* verts, int64_t vcap, int64_t* faces, int64_t fcap,
                 uint64_t* edge_record, void* stream, diso_counts* out);

/* uint64 slots of the edge record of a forward with these counts (diso_counts.n_verts,
 * .n_faces); 0 on bad input.  No counterpart in the reference, whose backward re-runs
 * the forward (diso/__init__.py:32, 86). */
int64_t diso_edge_record_slots(int method, int dtype, int64_t n_verts, int64_t n_faces);

/* DMC quads -> triangles: for each quad the triangle pair with the smaller largest
 * corner cosine, config (0,1,3),(1,2,3) first for all quads that pick it, then
 * (0,1,2),(0,2,3) (diso/__init__.py:118-147).  tris must hold 2*n_quads rows;
 * *n_tris receives the rows written (fewer only when a quad's angles are NaN,
 * which the reference also drops).  Synchronises the stream. */
int diso_split_quads(diso_extractor* ex, const void* verts, const int64_t* quads, int64_t n_quads, int64_t* tris,
                     int64_t* n_tris, void* stream);

/* Backward: dL/dsdf [nx][ny][nz] and dL/ddeform [nx][ny][nz][3] (when deform is
 * not NULL) from dL/dverts [n_verts][3] of the final (shifted, normalised)
 * vertices, with the `seg` and the edge record of the forward (the record's
 * adjoint slots are overwritten).  Every element of both outputs is written
 * (with DISO_GRAD_ZEROED: the buffers were zeroed by diso_zero_grads and only the
 * point tiles near the surface are written); the result is deterministic (no atomics).
 * flags = 0 reproduces the reference's gradients exactly, including its DMC
 * backward, which hands every patch of a multi-patch cell the gradient of the
 * cell's first patch (src/cudualmc.cu:990); flags = DISO_GRAD_EXACT gives the
 * true derivative there instead.  MC is unaffected by the flag.
 * Replaces DMCFunction.backward / DDMCFunction.backward (diso/__init__.py:30-44,
 * 84-98: the forward re-run, the zero fills and the F.pad backward) and
 * CuMC::backward / CUDualMC::backward (src/cumc.cu:734-743, src/cudualmc.cu:1130-1138). */
int diso_backward(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz, double isovalue,
                  double padval, const uint64_t* seg, uint64_t* edge_record, int normalize, int flags,
                  const void* grad_verts, void* grad_sdf, void* grad_deform, void* stream);

/* Backward of a forward that kept nothing but its `seg` (no edge record, no
 * gradient buffers): dL/dsdf [nx][ny][nz] and dL/ddeform [nx][ny][nz][3] (when
 * deform is not NULL) from dL/dverts [n_verts][3], every element of both written.
 * The crossings near each point tile, the vertex ids (MC) or the DMC cells' codes
 * after the ambiguity test and their patch ids, each edge's adjoint and each point's
 * sum are recomputed per tile in one pass (the tiles with no crossing nearby get
 * zeros on a second stream of the extractor): the same values, bit for bit, as
 * diso_backward with the forward's edge record (flags as there).  The inputs must
 * hold the values the forward saw; every index derived from them is checked against
 * the counts in `seg`, so a grid changed since the forward gives wrong gradients but
 * no access outside the buffers.  No host synchronisation.  Replaces
 * DMCFunction.backward / DDMCFunction.backward (diso/__init__.py:30-44, 84-98),
 * which re-run the forward to rebuild the crossing lists, and CuMC::backward /
 * CUDualMC::backward (src/cumc.cu:734-743, src/cudualmc.cu:1130-1138). */
int diso_backward_recompute(diso_extractor* ex, const void* sdf, const void* deform, int nx, int ny, int nz,
                            double isovalue, double padval, const uint64_t* seg, int normalize, int flags,
                            const void* grad_verts, void* grad_sdf, void* grad_deform, void* stream);

/* dL/d(isovalue) of an extraction, from the dL/dsdf [nx][ny][nz] that
 * diso_backward wrote: minus its sum (moving the isovalue by e moves every crossing
 * as moving every grid value by -e; the pad value isovalue + 1 moves with it).  The
 * result is written as one double to device memory at grad_iso on `stream`.  With
 * the forward's `seg`, only the point tiles near the surface are read (the others
 * hold zeros); with seg = NULL the whole grid.  Deterministic (a fixed reduction
 * order).  The gradient is that of the backward's flags: exact with
 * DISO_GRAD_EXACT (and for MC), the counterpart of the reference's DMC gradient
 * otherwise.  No counterpart in the reference, whose isovalue is a plain scalar
 * without a gradient (diso/__init__.py:48, 102). */
int diso_isovalue_grad(diso_extractor* ex, const void* grad_sdf, int nx, int ny, int nz, const uint64_t* seg,
                       double* grad_iso, void* stream);

/* Zero a forward's gradient buffers ahead of its backward, beside the forward's
 * kernels, which leave HBM bandwidth unused.  Call it before diso_forward_count /
 * diso_forward on `stream`; the zeros are complete once that forward's emit has run
 * (or its count found no surface).  When both buffers are 16-byte aligned, the
 * count and the emit write the zeros between their own loads; otherwise (or when the
 * count runs on another stream, or the SDF's rows are not a multiple of 16 bytes)
 * they are memsets on `zero_stream` after the work queued on `stream`, and the caller
 * keeps the buffers alive until that stream has passed them (e.g. torch's
 * Tensor.record_stream).  A second call before any forward replaces the first, whose
 * buffers are then not written.  A later diso_backward on the same extractor with
 * flags | DISO_GRAD_ZEROED waits for the zeros and writes only the point tiles near
 * the surface.  No counterpart in the reference (its backward zero-fills the padded
 * gradients, diso/__init__.py:35-37, 89-91). */
int diso_zero_grads(diso_extractor* ex, void* grad_sdf, int64_t sdf_bytes, void* grad_deform, int64_t deform_bytes,
                    void* stream, void* zero_stream);

/* Share of diso_zero_grads' bytes that the count writes (the first bytes of
 * grad_sdf then grad_deform, laid end to end); the emit writes the rest.  No
 * counterpart in the reference. */
double diso_zero_count_share(void);

/* Forward phase 1 (as diso_forward_count) for callers that cannot allocate
 * device memory: serving processes that reserve all their device memory at
 * start-up and may not grow it per request, and hosts that embed the library
 * under a memory manager of their own, where a cudaMalloc inside a request could
 * fail or stall.  No counterpart in the reference.
 *
 * It takes no extractor: its scratch (status words, active-tile list, scan state,
 * about 300 KB) is one static device array of this library, which every GPU that
 * loads the library holds until the process exits.  Nothing is allocated: no
 * cudaMalloc / cudaFree / cudaMallocHost.  Grids of at most 65536 4x8x32-cell
 * tiles (about 384^3) are accepted, larger ones fail with DISO_ERR_ARG and a
 * message.  The call copies the counts to the host and synchronises `stream`
 * before it returns.  The first call on a device (and the first after that
 * device's context was made again) looks up the array's device address.  All
 * calls share the array: calls whose GPU work overlaps (other streams, other
 * threads) race and must be serialised by the caller.  `seg` and the result have
 * the meaning they have for diso_forward_count.  A `seg` from this call alone does
 * not feed diso_forward_emit or diso_backward: those need an extractor on which
 * diso_forward_count (or diso_forward) ran for the same grid, and the backward
 * also the edge record of that extractor's emit. */
int diso_forward_count_static(int method, int dtype, const void* sdf, int nx, int ny, int nz, double isovalue,
                              double padval, uint64_t* seg, void* stream, diso_counts* out);

/* ---------------------------------------------------------------- batches
 *
 * Many grids of uneven size in one launch per phase (count, scan, emit,
 * backward) over a flattened queue of their tiles; the reference has no batched
 * call (its README runs a Python loop over one extractor, README.md:61-70), so
 * these replace that loop.  diso_batch_prepare uploads the grid descriptors and
 * grows the scratch; after it, diso_batch_count / _emit / _backward allocate
 * nothing and do not synchronise with the host, so the sequence can be captured
 * in a CUDA graph and replayed while the grids' contents change in place. */
typedef struct {
  const void* sdf;    /* [nx][ny][nz] */
  const void* deform; /* [nx][ny][nz][3] or NULL */
  void* grad_sdf;     /* backward output [nx][ny][nz] (needed by diso_batch_backward) */
  void* grad_deform;  /* backward output [nx][ny][nz][3] when deform is given */
  int nx, ny, nz;
  int pad_;
  double isovalue, padval; /* per grid, as in diso_forward_count */
} diso_grid;

/* uint64 slots of the batch record (segments of every grid, their total, tile bytes); 0 on bad input */
int64_t diso_batch_record_slots(const diso_grid* grids, int ngrids);

/* Lay out the record, upload the descriptors (1 <= ngrids <= 256), grow the scratch.  Synchronises. */
int diso_batch_prepare(diso_extractor* ex, const diso_grid* grids, int ngrids, uint64_t* record, void* stream);

/* Count and scan every grid of the prepared batch: one launch each, no host synchronisation. */
int diso_batch_count(diso_extractor* ex, void* stream);

/* Results of the last count (and emit): per-grid sizes, the grids' first vertex / face in the
 * concatenated outputs, and *overflow = 1 when an emit skipped grids past its capacities.
 * sdf_min / sdf_max are filled; `empty` is left 0: the caller applies the guard of
 * diso/__init__.py:49, 103 with each grid's isovalue.  Synchronises the stream. */
int diso_batch_results(diso_extractor* ex, diso_counts* per_grid, int64_t* vert_offset, int64_t* face_offset,
                       int* overflow, void* stream);

/* Emit every grid into concatenated verts [vcap][3] and faces [fcap][3] (MC) or [fcap][4]
 * (DMC quads); faces hold grid-local vertex ids.  A grid whose outputs would pass the
 * capacities is skipped and reported through diso_batch_results.  edge_record (32-byte
 * aligned, diso_edge_record_slots(method, dtype, vcap, fcap) slots, or NULL without a
 * backward) is filled for diso_batch_backward. */
int diso_batch_emit(diso_extractor* ex, int normalize, void* verts, int64_t vcap, int64_t* faces, int64_t fcap,
                    uint64_t* edge_record, void* stream);

/* Backward of every grid of the prepared batch from the concatenated dL/dverts, with the
 * edge record and the capacities of its diso_batch_emit; writes each grid's grad_sdf and
 * grad_deform (flags as for diso_backward).  Grids that the emit skipped get zero gradients. */
int diso_batch_backward(diso_extractor* ex, int normalize, int flags, const void* grad_verts, uint64_t* edge_record,
                        int64_t vcap, int64_t fcap, void* stream);

/* ---------------------------------------------------------------- timing
 *
 * Optional timing of every kernel an extractor launches, for benchmarks: with
 * timing on, each launch is bracketed by CUDA events on its own stream.  No
 * counterpart in the reference, which times nothing. */
typedef struct {
  char name[32];     /* count, scan, emit, zero_grads, zero_tiles, active_list, edge, gather, split */
  int64_t launches;
  double total_ms;   /* summed event time of those launches */
} diso_kernel_time;

/* Turn timing on (enable != 0) or off; drops the launches recorded so far. */
int diso_timing(diso_extractor* ex, int enable);

/* Per-kernel totals of the launches recorded since the last call (waits for their
 * end events), at most `max` entries, *n = entries written; then starts over. */
int diso_timing_read(diso_extractor* ex, diso_kernel_time* out, int max, int* n);

/* ---- Evaluated fields ----
 * The caller side of the extraction without the dense grid: the reference's caller
 * evaluates its SDF on a full meshgrid in PyTorch and passes the [N, N, N] tensor
 * (test/example.py:8-16, 33-53).  Here the extractor evaluates the field where it
 * needs values: the count classifies each chunk of 8 x 32 x 32 cells from bounds of
 * the field over it and evaluates only the chunks that may hold the surface, the
 * emit evaluates the end points of the crossing edges.  The field: a union of spheres,
 * value(p) = min_k (|p - c_k| - r_k) at grid point p = lo + (hi - lo) * i / (n - 1)
 * (per axis; step computed in double, then in the dtype), spheres [count][4] (x, y,
 * z, r) in device memory in the extractor's dtype, and optionally a dense deform of
 * the grid's points.  diso_backward_field gives the gradients with respect to the
 * spheres (and the deform). */
typedef struct diso_sphere_field {
  const void* spheres;
  int count;
  double lo[3];
  double hi[3];
  const void* deform; /* [nx][ny][nz][3] in the dtype, or NULL: the vertices' deform, as for a dense grid */
} diso_sphere_field;

/* As diso_forward for an evaluated field: count, scan and emit in one call into
 * outputs of capacities vcap / fcap; counts->emitted says whether they fitted (if not,
 * call again with larger outputs).  counts->sdf_min / sdf_max are bounds on the side
 * of the isovalue that decide the empty-surface guard, not the grid's extremes. */
int diso_forward_field(diso_extractor* ex, const diso_sphere_field* field, int nx, int ny, int nz, double isovalue,
                       double padval, uint64_t* seg, int normalize, void* verts, int64_t vcap, int64_t* faces,
                       int64_t fcap, void* stream, diso_counts* counts);

/* Backward of diso_forward_field (its `seg` record; the field unchanged since), without
 * a dense grid of the field's values: from dL/dverts [n_verts][3], the gradients of
 * the spheres' parameters as doubles grad_spheres [count][4] (dL/dx, dL/dy, dL/dz of
 * the centre, dL/dr), and, when the field has a deform, dL/ddeform [nx][ny][nz][3].
 * A point's dL/d(value) (the crossing edges' lerp adjoints, as diso_backward forms
 * them, flags as there) goes to the sphere attaining the minimum there: d(|p - c| -
 * r)/dc = -(p - c) / |p - c|, d/dr = -1.  Deterministic (fixed reduction orders); at
 * most 64 spheres.  The reference's example differentiates its analytic sphere
 * through PyTorch on a dense grid (test/example.py:8-16, 33-54, 75-81); no
 * counterpart in its library. */
int diso_backward_field(diso_extractor* ex, const diso_sphere_field* field, int nx, int ny, int nz, double isovalue,
                        double padval, const uint64_t* seg, int normalize, int flags, const void* grad_verts,
                        double* grad_spheres, void* grad_deform, void* stream);

/* The field's dense grid [nx][ny][nz] (the same values the fused forward evaluates). */
int diso_field_materialize(int dtype, const diso_sphere_field* field, int nx, int ny, int nz, void* sdf,
                           void* stream);

/* ---- Narrow-band input ----
 * A grid whose values are stored only in 8 x 8 x 8-point bricks near the surface, for
 * grids whose dense arrays are out of reach (32 B per point in fp32 with deform and
 * both gradients: 275 GB at 2048^3).  index [ceil(nx/8)][ceil(ny/8)][ceil(nz/8)] (int32, device)
 * holds each brick's slot in values [count][8][8][8] (the dtype, z fastest), or
 * DISO_BRICK_OUTSIDE / DISO_BRICK_INSIDE for an absent brick, whose points read
 * +background / -background.  The band's meshes are exactly those of the dense grid
 * with those values in the absent bricks (diso_bricks_materialize writes it): the same
 * vertices, faces and order.  The deform, when given, is [count][8][8][8][3] (zero in
 * absent bricks).  The reference takes only dense [N, N, N] grids
 * (diso/__init__.py:48, 102); no counterpart in its library. */
#define DISO_BRICK_OUTSIDE (-1)
#define DISO_BRICK_INSIDE (-2)
typedef struct diso_brick_grid {
  int dims[3];          /* nx, ny, nz: points per axis of the grid the band lies in */
  const int32_t* index; /* [ceil(nx/8)][ceil(ny/8)][ceil(nz/8)] */
  int count;            /* slots */
  const void* values;   /* [count][8][8][8] in the extractor's dtype */
  const void* deform;   /* [count][8][8][8][3] in the dtype, or NULL */
  double background;    /* > 0 */
} diso_brick_grid;

/* As diso_forward_field for a narrow band (count, scan and emit in one call into
 * outputs of capacities vcap / fcap; counts->emitted says whether they fitted).  A
 * first pass checks the index (synchronising the stream): an entry that is neither a
 * slot in [0, count) nor an absent tag, a slot used twice, or a band whose present
 * bricks and absent bricks beside an absent brick of the other side (or the grid's
 * edge) allow more crossings than the 32-bit counts hold is DISO_ERR_ARG.  The count
 * classifies chunks whose bricks are all absent from the index alone.  The `seg`
 * record has the dense grid's size (8 bytes per 32-cell row segment); DMC keeps its
 * cell records in the extractor's scratch for the count units that hold the surface
 * only (64 KB per unit of 8 x 32 x 128 cells; one more host round trip sizes them). */
int diso_forward_bricks(diso_extractor* ex, const diso_brick_grid* bricks, double isovalue, double padval,
                        uint64_t* seg, int normalize, void* verts, int64_t vcap, int64_t* faces, int64_t fcap,
                        void* stream, diso_counts* counts);

/* Backward of diso_forward_bricks (its `seg`; the band unchanged since): from
 * dL/dverts [n_verts][3], dL/dvalues [count][8][8][8] and, for a band with a deform,
 * dL/ddeform [count][8][8][8][3], every element written (zero where no crossing edge
 * ends), flags as for diso_backward.  Equal to the dense backward's gradients at the
 * bricks' points; absent points have none. */
int diso_backward_bricks(diso_extractor* ex, const diso_brick_grid* bricks, double isovalue, double padval,
                         const uint64_t* seg, int normalize, int flags, const void* grad_verts, void* grad_values,
                         void* grad_deform, void* stream);

/* The band's dense grid [nx][ny][nz] and, when `deform` is not NULL (the band has a
 * deform), its dense deform [nx][ny][nz][3]. */
int diso_bricks_materialize(int dtype, const diso_brick_grid* bricks, void* sdf, void* deform, void* stream);

/* ---- Mesh consumers on the device ----
 * For the meshes the extractor returns: vertices [n_verts][3] in the extractor's
 * dtype, faces [n_faces][corners] int64 (corners 3 or 4).  Each call runs on
 * `stream` and synchronises it at the end; a face index outside [0, n_verts) is
 * DISO_ERR_ARG.  The reference writes its meshes through trimesh on the host
 * (test/example.py:71-73, trimesh.Trimesh(...).export to OBJ); these replace that
 * step for meshes in device memory.  The extractor only supplies the dtype and
 * grow-only scratch. */

/* Area-weighted vertex normals: per vertex the sum of the normals of its faces
 * (triangles (p1-p0) x (p2-p0), quads (p2-p0) x (p3-p1), i.e. twice the vector
 * area, in double), normalised; [0, 0, 0] for a vertex without area.  The sums are
 * exact 64-bit fixed point (2^50 over the largest face normal component), so the
 * result does not depend on the order of the GPU's atomics.  normals: [n_verts][3]. */
int diso_mesh_normals(diso_extractor* ex, const void* verts, int64_t n_verts, const int64_t* faces, int64_t n_faces,
                      int corners, void* normals, void* stream);

/* Weld: vertices with equal positions (tol = 0: equal coordinates, -0 = +0;
 * tol > 0: equal floor(x / tol + 0.5) per coordinate) become one, the lowest index
 * of each group; kept vertices and faces keep their order, faces whose corners are
 * no longer distinct are dropped.  out_verts holds up to n_verts rows, out_faces up to
 * n_faces; *n_verts_out / *n_faces_out receive the counts. */
int diso_mesh_weld(diso_extractor* ex, const void* verts, int64_t n_verts, const int64_t* faces, int64_t n_faces,
                   int corners, double tol, void* out_verts, int64_t* out_faces, int64_t* n_verts_out,
                   int64_t* n_faces_out, void* stream);

/* OBJ text into a device buffer: "v x y z" lines with every coordinate as "%.8f"
 * (correctly rounded, ties to even; nan / inf / -inf spelled so), then, when normals
 * is not NULL, "vn" lines, then "f a b c[ d]" lines with 1-based indices ("a//a"
 * with normals); every line ends in "\n".  *text_bytes receives the length; the text
 * is written only when text is not NULL and the length fits text_cap (call with
 * text = NULL for the size).  Coordinates must have |x| < 1.8e11. */
int diso_mesh_obj(diso_extractor* ex, const void* verts, const void* normals, int64_t n_verts, const int64_t* faces,
                  int64_t n_faces, int corners, char* text, int64_t text_cap, int64_t* text_bytes, void* stream);

/* Bytes of a binary little-endian PLY body (-1 for bad arguments): the vertex block
 * (x y z, then nx ny nz when with_normals, in the dtype) and the face block (one
 * byte count, then `corners` int32 indices per face). */
int64_t diso_mesh_ply_bytes(int dtype, int64_t n_verts, int64_t n_faces, int corners, int with_normals);

/* The PLY body into a device buffer of diso_mesh_ply_bytes bytes; the header
 * ("ply", "format binary_little_endian 1.0", the element and property lines,
 * "end_header") is the caller's. */
int diso_mesh_ply(diso_extractor* ex, const void* verts, const void* normals, int64_t n_verts, const int64_t* faces,
                  int64_t n_faces, int corners, void* body, void* stream);

/* ---- Launch widths ----
 * Free parameters of the kernels' launches, for the package's autotuner
 * (diso_gb300/tune.py), which times candidates on the caller's GPU and grid size and
 * caches the winners.  None changes any output: every kernel gives the same bits for
 * any width.  The reference fixes its block size (BLOCK_SIZE 512, src/cumc.cu:93;
 * src/cudualmc.cu:93) and has nothing to tune. */
enum {
  DISO_TUNE_COUNT_CTAS = 0,  /* persistent CTAs per SM of the forward count (capped by occupancy) */
  DISO_TUNE_EMIT_CTAS = 1,   /* ... of the forward emit */
  DISO_TUNE_GATHER_CTAS = 2, /* ... of the stored backward's point gather (single grids and batches) */
  DISO_TUNE_FUSED_CTAS = 3,  /* ... of the recompute backward's fused pass */
  DISO_TUNE_ZERO_CTAS = 4,   /* CTAs per SM of the point-tile zeros beside a backward (default 2) */
  DISO_TUNE_EDGE_CTAS = 5,   /* CTAs per SM of the stored backward's edge pass (default 8) */
  DISO_TUNE_BATCH_CTAS = 6,  /* CTAs per SM of the batches' emit and backward passes (default 4) */
  DISO_TUNE_ZERO_SHARE = 7,  /* stored mode: per mille of the gradient zeros the count writes (default 350) */
  DISO_TUNE_N = 8
};

/* Set launch parameter `param` of the extractor's later calls to `value` (0 restores
 * the default; CTAs per SM 1..64, the zero share 1..1000 per mille).  No counterpart
 * in the reference. */
int diso_tune_set(diso_extractor* ex, int param, int value);

/* The value set for `param` (0: the default), -1 for a bad argument. */
int diso_tune_value(const diso_extractor* ex, int param);

/* Check of the bounded device-side waits: runs the segment scan's look-back on two
 * tiles of the extractor's scratch with only the second tile launched, so that the
 * flag it waits for is never published, and each poll limited to spin_limit tries
 * (1 .. 2^22; the forward's own scans use 2^22).  Returns DISO_ERR_SCAN with the
 * scan's message when the wait gave up (the expected result), after which the
 * extractor is usable as before; DISO_OK would mean the wait never ran out.  Lets a
 * caller see that a stalled look-back ends in an error status instead of a hang.
 * No counterpart in the reference.  Synchronises the stream. */
int diso_scan_wait_probe(diso_extractor* ex, unsigned spin_limit, void* stream);

/* Bytes of device memory the extractor holds as its own scratch (grow-only
 * buffers; not the caller's per-call `seg`, edge record or outputs), for memory
 * reports.  No counterpart in the reference. */
int64_t diso_scratch_bytes(const diso_extractor* ex);

/* Message of the last failed call on this thread ("" if none).  Replaces the
 * reference's error paths: AT_ASSERTM / TORCH_INTERNAL_ASSERT on the inputs
 * (src/pybind.cpp:5-11), which raise in Python, and CUDA errors that are printed and
 * ignored (src/cumc.cu:68-78); here every failure is a status code with this message. */
const char* diso_last_error(void);

/* Library version string (no counterpart in the reference). */
const char* diso_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DISO_GB300_H */
