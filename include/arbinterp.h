/*
 * arbinterp.h — C ABI of the GB300 (sm_103a) Lekien–Marsden tricubic /
 * quadcubic interpolation path.
 *
 * Every entry point takes DEVICE pointers, sizes and a CUDA stream, launches
 * work on that stream and returns an arb_status.  Nothing here allocates
 * device memory: callers (the Python drop-in, or any C/C++ host) own every
 * buffer.  Errors found on the device (an irregular grid, a cell index past
 * the table) are OR-ed into a caller-owned device status word; read it with
 * arb_status_fetch() after the stream work is done.  No C++ exception crosses
 * this boundary.
 *
 * Data layout in device memory (see arb_grid):
 *   grid64  [npts][F] float64, points z-major with x fastest (t slowest in 4D)
 *   grid32  float32 split, hi = RN(v), lo = RN(v - hi):
 *             F = 1: [npts] (hi, lo)
 *             F = 3: [npts] (hi_x, hi_y, hi_z, 0)        (values only)
 *             F = 4: [npts] (hi_x, hi_y, hi_z, hi_n), then [npts] lo_n
 *           only the field whose gradient is returned keeps its residual
 *   table   [nc][F][M] coefficients (M = 64 in 3D, 256 in 4D), float64 or
 *           float32, monomial index ex + 4 ey + 16 ez (+ 64 et)
 * F (fields) is 1 for scalar and norm modes, 3 for vector mode and 4 for
 * both mode (order Bx, By, Bz, |B|).
 *
 * The reference (DurhamDecLab/ARBInterp v1.8) is a pure Python/NumPy module
 * with no FFI; each function below cites the reference method whose work it
 * replaces (paths relative to the reference project root).
 */
#ifndef ARBINTERP_H
#define ARBINTERP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *arb_stream_t; /* same type as cudaStream_t */

enum arb_status {
  ARB_OK = 0,
  ARB_ERR_INVALID = 1,        /* bad argument: null pointer, bad sizes      */
  ARB_ERR_CUDA = 2,           /* a CUDA runtime call or launch failed        */
  ARB_ERR_IRREGULAR_GRID = 4, /* field rows are not a full tensor grid       */
  ARB_ERR_CELL_INDEX = 8,     /* a query's cell index exceeded nc            */
  ARB_ERR_CAPACITY = 16,      /* an axis has more points than axis_cap       */
  ARB_ERR_TIMEOUT = 32,       /* a bounded device wait gave up               */
  ARB_ERR_UNSUPPORTED = 64    /* combination not built (e.g. dim/F/precision) */
};

enum arb_precision {
  ARB_PREC_FP64 = 0,  /* everything in float64 (parity with the reference)  */
  ARB_PREC_MIXED = 1  /* split-precision tensor-core / float32 evaluation   */
};

enum arb_kind {
  ARB_KIND_SCALAR = 0, /* N x 4 (3D) / N x 5 (4D) input: value + gradient   */
  ARB_KIND_VECTOR = 1, /* components only                                   */
  ARB_KIND_NORM = 2,   /* |B| interpolated as its own field + gradient      */
  ARB_KIND_BOTH = 3    /* components, |B| and its gradient                  */
};

/* A constructed interpolant: grid geometry plus device buffers. */
typedef struct arb_grid {
  int32_t dim;          /* 3 or 4                                           */
  int32_t kind;         /* enum arb_kind                                    */
  int32_t nfield;       /* F                                                */
  int32_t sentinel_nan; /* cell index == nc: 1 -> NaN row, 0 -> zero row   */
  int64_t n[4];         /* grid points per axis (x, y, z, t)                */
  int64_t nc;           /* cells = prod(n[a] - 3)                           */
  double lo[4];         /* xIntMin.. : second grid coordinate per axis      */
  double hi[4];         /* xIntMax.. : second-to-last grid coordinate       */
  double h[4];          /* spacing from the first two axis samples          */
  const double *grid64; /* [npts][F]                                        */
  const float *grid32;  /* mixed-precision split (layout above) or NULL   */
  const void *table;    /* [nc][F][M] or NULL                               */
  int32_t table_prec;   /* enum arb_precision of table (FP64: double)      */
  int32_t bin_shift;    /* log2 cells per bin edge for grouped queries; 0 = default (3D: 3, 4D: 2) */
} arb_grid;

/* Query outputs.  Any pointer may be NULL when not wanted.  Rows are
 * row-major like the reference's return arrays; each of comps, norms and
 * grads has its own row stride in doubles (0 = packed: 3, 1 and dim).
 * Interleaved rows: when comps, norms and grads share rows of R doubles —
 * both mode: norms = comps + 3, grads = comps + 4, R = 8; scalar / norm
 * mode: grads = norms + 1, R = 4 (3D) or 8 (4D); vector mode: R = 4 — and
 * the first output is 32-byte aligned, the kernels store whole 32-byte
 * sectors and may write 0 into the row's unused trailing doubles. */
typedef struct arb_query_out {
  double *comps;     /* [nq][3]   vector and both modes                     */
  double *norms;     /* [nq]      scalar, norm and both modes               */
  double *grads;     /* [nq][dim] scalar, norm and both modes               */
  int64_t *inds;     /* [nq]      cell index per row (queryInds)            */
  int64_t *oob_rows; /* [nq]      rows found outside the volume, any order  */
  unsigned long long *oob_count; /* device counter for oob_rows (zeroed by caller) */
  int64_t comps_stride, norms_stride, grads_stride; /* row strides in doubles, 0 = packed */
} arb_query_out;

/* ---- ingest: replaces getFieldParams (src/ARBInterp/ARBInterp.py:528-568,
 *      1264-1320), the argsort-based lexicographic sort and exact-equality
 *      axis discovery. ------------------------------------------------------ */

/* Scratch bytes arb_ingest_axes needs in `work`. */
size_t arb_ingest_axes_work_bytes(int32_t dim);

/* Finds each axis' sample values (points on the axis lines through row 0;
 * for a full tensor grid these equal the reference's lines through its
 * first sorted row), sorted ascending.  Writes
 * axis_out[a * axis_cap + i] and axis_count[a] (device).  axis_out holds
 * 2 * dim * axis_cap doubles: the second half stages the unsorted lists.
 * field is [npts][ncol] float64 (field_is_f32 == 0) or float32. */
int arb_ingest_axes(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol,
                    int32_t dim, int64_t axis_cap, double *axis_out, int64_t *axis_count,
                    void *work, size_t work_bytes, int32_t *status, arb_stream_t stream);

/* Scatters every field row to its grid slot (the sorted order the reference
 * builds with argsort) and writes the per-mode interpolated fields: grid64,
 * optionally grid32 (hi/lo split) and, when raw_out is given, the raw value
 * columns [npts][ncol-dim] in sorted order.  claim is npts uint32 of scratch
 * (it receives the inverse permutation grid slot -> row, and detects
 * duplicate points).  n holds the host-side axis counts returned by
 * arb_ingest_axes.  grid64 may be NULL when grid32 is given (a
 * mixed-precision interpolant whose float64 values are produced later, by a
 * second call with grid32 NULL).  npts < 2^32. */
int arb_ingest_scatter(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol,
                       int32_t dim, const double *axes, int64_t axis_cap, const int64_t *n,
                       int32_t kind, double *grid64, float *grid32, double *raw_out,
                       uint32_t *claim, int32_t *status, arb_stream_t stream);

/* Single-pass ingest for rows in meshgrid order: lexicographic over the
 * axes in any axis order, each axis ascending or descending (what NumPy's
 * meshgrid + reshape and the reference's own sort, ARB:530, produce).  Reads
 * the axes off the lines through row 0 into axis_out / axis_count (as
 * arb_ingest_axes does) and writes every grid slot from the row its
 * position implies (as arb_ingest_scatter does), checking that row's
 * coordinates against the slot's axis samples.  For rows in any other order
 * (or not a full grid) it sets ARB_ERR_IRREGULAR_GRID in *status and leaves
 * the outputs undefined: the caller then runs arb_ingest_axes +
 * arb_ingest_scatter, which give the authoritative answer.  work holds
 * arb_ingest_axes_work_bytes(dim) bytes.  grid64 or grid32 may be NULL (not
 * both), as for arb_ingest_scatter.  npts < 2^32.  Replaces the same
 * reference code as the two-step ingest (ARB:528-568, 1264-1320). */
int arb_ingest_ordered(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol,
                       int32_t dim, int32_t kind, int64_t axis_cap, double *axis_out,
                       int64_t *axis_count, double *grid64, float *grid32, double *raw_out,
                       void *work, size_t work_bytes, int32_t *status, arb_stream_t stream);

/* arb_ingest_ordered in two launches on the same stream, so that the host
 * can read the axes (arb_ingest_summary after the probe) while the grid is
 * still being written: _probe reads the axes off the lines through row 0
 * (ARB_ERR_IRREGULAR_GRID in *status if those lines are not a meshgrid) and
 * writes all dim axis counts (0 for an axis it did not find);
 * _fill writes every grid slot and checks every row, with the same axes and
 * work (ARB_ERR_IRREGULAR_GRID for rows in another order; it does nothing
 * after a failed probe).  The same reference code (ARB:528-568, 1264-1320). */
int arb_ingest_ordered_probe(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol,
                             int32_t dim, int32_t kind, int64_t axis_cap, double *axis_out,
                             int64_t *axis_count, void *work, size_t work_bytes, int32_t *status,
                             arb_stream_t stream);

int arb_ingest_ordered_fill(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol,
                            int32_t dim, int32_t kind, int64_t axis_cap, const double *axis_out,
                            const void *work, size_t work_bytes, double *grid64, float *grid32,
                            double *raw_out, int32_t *status, arb_stream_t stream);

/* Everything the host needs after an ingest, for one device-to-host copy:
 * out[0] = *status (then cleared), out[1 + a] = axis_count[a], and per axis
 * a the samples 0, 1 and n_a - 2 at out[5 + 3a .. 7 + 3a] (the reference's
 * h, IntMin and IntMax come from them, ARB:541-568); 17 doubles.  No
 * counterpart in the reference (host-side arrays there). */
int arb_ingest_summary(const double *axes, int64_t axis_cap, const int64_t *axis_count, int32_t dim,
                       int32_t *status, double *out, arb_stream_t stream);

/* ---- finite-difference planes: replaces the D matrix of makeAMatrix
 *      (src/ARBInterp/ARBInterp.py:129-173, 762-876) applied per grid point.
 *      planes is [2^dim][npts][F] float64: kind r (f, fx, fy, fz, fxy, fxz,
 *      fyz, fxyz in 3D; the reference's 16 kinds in 4D) as central
 *      differences in unit-cell units.  Boundary points (no neighbour on an
 *      axis) get NaN for kinds that need it. ------------------------------ */
int arb_fd_planes(const arb_grid *g, double *planes, arb_stream_t stream);

/* ---- coefficient solve: replaces calcCoefficients1/2/3 and allCoeffs
 *      (src/ARBInterp/ARBInterp.py:523-525, 570-603; 4D 1260-1262,
 *      1322-1355).  Writes table[cell][F][M] for cells [cell0, cell0+ncells).
 *      ARB_PREC_FP64: float64 table, exact separable form of A = inv(B) D.
 *      ARB_PREC_MIXED: float32 table from the tcgen05 tensor-core GEMM with
 *      split-precision operands. ------------------------------------------ */
int arb_coef_solve(const arb_grid *g, int32_t precision, int64_t cell0, int64_t ncells,
                   void *table, int32_t *status, arb_stream_t stream);

/* ---- query evaluation from the coefficient table: replaces rQuery1/2/3
 *      (src/ARBInterp/ARBInterp.py:344-521; 4D 1064-1258).  q is [nq] rows
 *      of q_stride doubles (x, y, z[, t], ...).  Rows outside
 *      [IntMin, IntMax] on any axis come back NaN in every output; when
 *      q_writeback is nonzero those rows of q are overwritten with NaN in
 *      place, like the reference does to its caller's array. -------------- */
int arb_query_eval(const arb_grid *g, double *q, int64_t nq, int64_t q_stride,
                   int32_t q_writeback, const arb_query_out *out, int32_t *status,
                   arb_stream_t stream);

/* ---- on-the-fly evaluation straight from the grid (no table): same
 *      contract as arb_query_eval; precision selects float64 or the
 *      split float32 (hi/lo delta) evaluation that needs g->grid32. ------- */
int arb_query_eval_otf(const arb_grid *g, int32_t precision, double *q, int64_t nq,
                       int64_t q_stride, int32_t q_writeback, const arb_query_out *out,
                       int32_t *status, arb_stream_t stream);

/* ---- cell-grouped evaluation: the same contract as arb_query_eval_otf
 *      (use_table == 0) or arb_query_eval (use_table != 0, table precision
 *      must equal `precision`), but queries are first grouped by spatial bin
 *      with a counting sort so grid blocks / coefficient rows are fetched
 *      from HBM about once.  Replaces the same reference methods
 *      (rQuery1/2/3, src/ARBInterp/ARBInterp.py:344-521, 1064-1258).
 *      work: caller-owned scratch of arb_query_sorted_work_bytes() bytes.
 *      nq < 2^32. ----------------------------------------------------------- */
size_t arb_query_sorted_work_bytes(const arb_grid *g, int32_t precision, int64_t nq);

int arb_query_eval_sorted(const arb_grid *g, int32_t precision, int32_t use_table, double *q,
                          int64_t nq, int64_t q_stride, int32_t q_writeback,
                          const arb_query_out *out, void *work, size_t work_bytes,
                          int32_t *status, arb_stream_t stream);

/* ---- adjoint of the 3D scalar interpolant.  No counterpart in the
 *      reference (it has no backward pass); it is the transpose of the
 *      forward map of rQuery2 (src/ARBInterp/ARBInterp.py:399-454): values
 *      and gradients are linear in the grid samples through A = inv(B) D.
 *      Given upstream dL/dvalue dval[nq] and/or dL/dgrad dgrad[nq][3]
 *      (either may be NULL), accumulates dL/df into grid_grad[npts] (float64
 *      for ARB_PREC_FP64, float32 for ARB_PREC_MIXED; zero it first) with
 *      atomics, and writes dL/dq into q_grad[nq][3] (may be NULL).  Rows
 *      outside the volume, NaN rows and sentinel rows contribute nothing
 *      and get dL/dq = 0.  g must be 3D with F = 1 (scalar or norm mode). */
int arb_adjoint(const arb_grid *g, int32_t precision, const double *q, int64_t nq, int64_t q_stride,
                const double *dval, const double *dgrad, void *grid_grad, double *q_grad,
                int32_t *status, arb_stream_t stream);

/* ---- the same adjoint (3D scalar, ARB_PREC_MIXED only) with the queries
 *      grouped by 8^3-cell bins first, as arb_query_eval_sorted does: the
 *      scatter of dL/df goes to a shared-memory tile of each bin's points
 *      and reaches grid_grad with one atomic per point and bin (64 per query
 *      in arb_adjoint).  Same arguments and results (float32 sums in another
 *      order); work: caller-owned scratch of arb_adjoint_work_bytes(g, nq)
 *      bytes.  nq < 2^32.  No counterpart in the reference. */
size_t arb_adjoint_work_bytes(const arb_grid *g, int64_t nq);

int arb_adjoint_binned(const arb_grid *g, int32_t precision, const double *q, int64_t nq, int64_t q_stride,
                       const double *dval, const double *dgrad, void *grid_grad, double *q_grad, void *work,
                       size_t work_bytes, int32_t *status, arb_stream_t stream);

/* Replaces the sample values of a scalar (F = 1) interpolant: values[npts]
 * in grid order (z-major, x fastest), float32 (values_f32) or float64;
 * rewrites grid64 and, when given, the float32 split grid32.  The geometry
 * and any coefficient table are unchanged (solve again if one is used). */
int arb_grid_set_values(const arb_grid *g, const void *values, int32_t values_f32, double *grid64,
                        float *grid32, arb_stream_t stream);

/* ---- batched persistent evaluation of many 3D interpolants in one launch.
 *      Per field it computes what rQuery1/2/3 do
 *      (src/ARBInterp/ARBInterp.py:344-521); the batching itself has no
 *      counterpart in the reference (one Python object per field).
 *      grids: DEVICE array of nfields descriptors (a descriptor with a table
 *      is evaluated from its table, otherwise on the fly; all use
 *      `precision`).  Queries of all fields are concatenated in q (q_stride
 *      doubles per row); field f owns rows [q_off[f], q_off[f+1]) and tiles
 *      [tile_off[f], tile_off[f+1]) of tile_rows rows (device arrays of
 *      nfields+1).  Outputs are concatenated the same way.  counter is one
 *      device word of scratch (reset here).  nfield: the fields' common
 *      count F (1, 3 or 4) when every descriptor has it, which selects a
 *      kernel compiled for that count alone (fewer registers, more CTAs per
 *      SM); 0 when the counts differ.  Capturable in a CUDA graph. */
int arb_batched_launch(const arb_grid *grids, int32_t nfields, int32_t nfield, const int64_t *q_off,
                       const int64_t *tile_off, int64_t ntiles, int32_t tile_rows, int32_t precision,
                       double *q, int64_t q_stride, int32_t q_writeback, const arb_query_out *out,
                       unsigned long long *counter, int32_t *status, arb_stream_t stream);

/* ---- the two halves of arb_query_eval_sorted (same reference methods).
 *      arb_query_bin: index step, out-of-volume bookkeeping (inds, oob rows,
 *      q write-back, status) and the bin-ordered records in `work`.
 *      arb_query_eval_binned: evaluation from those records into
 *      out->comps/norms/grads.  The records depend on the query points and
 *      the grid geometry only, so the same points can be re-evaluated after
 *      the field values change (same geometry) without binning again. */
int arb_query_bin(const arb_grid *g, int32_t precision, double *q, int64_t nq, int64_t q_stride,
                  int32_t q_writeback, const arb_query_out *out, void *work, size_t work_bytes,
                  int32_t *status, arb_stream_t stream);

int arb_query_eval_binned(const arb_grid *g, int32_t precision, int32_t use_table, int64_t nq,
                          const arb_query_out *out, void *work, size_t work_bytes, arb_stream_t stream);

/* ---- allocation-free cell-grouped evaluation.  No counterpart in the
 *      reference (which has no device memory at all).
 *
 *      For callers that cannot allocate device memory while they run: hosts
 *      that own every device byte through their own pool (simulation or
 *      rendering engines), plugin hosts that forbid allocation inside
 *      callbacks, and long-running services that must not grow or fragment
 *      device memory mid-run.  Same contract as arb_query_eval_sorted, but the
 *      scratch is a fixed array inside the library: ARB_NOALLOC_SCRATCH_BYTES
 *      on every GPU that loads the library, held until the process exits.
 *      Calls whose scratch need (arb_query_sorted_work_bytes) exceeds it
 *      return ARB_ERR_CAPACITY without touching the GPU — on a 256^3 grid
 *      (32768 bins, 16 sub-bins each in mixed precision) at most 344,048
 *      query rows per call in float64 and
 *      360,416 in mixed precision (48- and 32-byte records); split larger
 *      query sets into several calls.  Arguments are checked first, as
 *      arb_query_eval_sorted checks them.
 *
 *      The first call on a device looks up the array's device address (once
 *      per device, with that device current); make that first call before
 *      any stream capture.  The lookup is repeated only if the device's
 *      context changed since (after a cudaDeviceReset).  Nothing is allocated: no cudaMalloc, no
 *      cudaFree, no allocating library call.  Every call shares the one
 *      array and leaves its contents behind; each call clears what must start
 *      at zero.  Calls that overlap on the GPU (other streams, other host
 *      threads) race on the array and must be serialised by the caller. */
#define ARB_NOALLOC_SCRATCH_BYTES (16u << 20)

int arb_query_eval_sorted_noalloc(const arb_grid *g, int32_t precision, int32_t use_table,
                                  double *q, int64_t nq, int64_t q_stride, int32_t q_writeback,
                                  const arb_query_out *out, int32_t *status, arb_stream_t stream);

/* ---- particle trajectories (no reference counterpart: the reference was
 *      written to simulate particle motion in magnetic fields and planned
 *      integrators for it, CHANGELOG.md v1.0.0).  Fourth-order Runge-Kutta on
 *      x' = v, v' = coef * grad f(x) + gravity, f the interpolated scalar
 *      (scalar / norm modes) or |B| (both mode), 3D only; one thread per
 *      particle, four on-the-fly evaluations per step in the given precision.
 *      state is [n][6] (x, y, z, vx, vy, vz), updated in place; a particle
 *      whose stage leaves the interpolation volume (or lands on a cell index
 *      >= nc) becomes NaN and increments *lost (device counter).  path, when
 *      not NULL, receives the state every record_every steps:
 *      [nsteps / record_every][n][6]. ------------------------------------- */
int arb_rk4_trajectories(const arb_grid *g, int32_t precision, double *state, int64_t n, double dt,
                         int64_t nsteps, double coef, const double *gravity, double *path,
                         int64_t record_every, unsigned long long *lost, arb_stream_t stream);

/* ---- field files: np.genfromtxt(path, delimiter=',') on the device
 *      (examples/3D_ARBInterpExample.py:14,37 and
 *      examples/4D_ARBInterpExample.py:14,38 load the N x 4..7 field tables
 *      this way; README.md:64-72).  ASCII text, universal newlines, a
 *      one-character delimiter and comment character, skip_header; every
 *      token converted as Python's float() does (correctly rounded; an
 *      empty or malformed token reads as NaN).  Three phases, each followed
 *      by a read of the device-side arb_csv_info:
 *        1. arb_csv_count  -> nlines (lines counted in byte chunks),
 *                             first_nonascii;
 *        2. arb_csv_split  -> line starts, values per line (nvals, the
 *                             caller's int32[nlines]; 0 = skipped line),
 *                             first_data_line, ncols, nrows, ninvalid;
 *        3. arb_csv_parse  -> out[nrows][ncols] float64 (lines whose value
 *                             count differs from ncols are not written).
 *      text must be 16-byte aligned; delimiter in 1..127 (not CR/LF);
 *      comment -1 (none) or 1..127 and != delimiter. ------------------- */
typedef struct arb_csv_info {
  int64_t nlines;          /* physical lines                                   */
  int64_t first_nonascii;  /* offset of the first byte >= 0x80, or -1          */
  int64_t first_data_line; /* first line with values (0-based), or -1          */
  int64_t ncols;           /* values on that line                              */
  int64_t nrows;           /* lines with exactly ncols values                  */
  int64_t ninvalid;        /* lines with values, but not ncols of them         */
  int64_t nexact;          /* tokens settled by the exact big-integer pass     */
  int64_t nqueued;         /* lines queued for that pass                       */
  int32_t error;           /* ARB_ERR_CAPACITY if a big integer overflowed     */
  int32_t reserved;
} arb_csv_info;

size_t arb_csv_count_work_bytes(int64_t nbytes);
int arb_csv_count(const uint8_t *text, int64_t nbytes, void *work, size_t work_bytes, arb_csv_info *info,
                  arb_stream_t stream);
/* lines_work: arb_csv_lines_work_bytes(nlines) bytes, 256-byte aligned;
 * count_work is phase 1's work buffer (per-chunk line offsets). */
size_t arb_csv_lines_work_bytes(int64_t nlines);
int arb_csv_split(const uint8_t *text, int64_t nbytes, int64_t nlines, int32_t delimiter, int32_t comment,
                  int64_t skip_header, const void *count_work, void *lines_work, size_t lines_work_bytes,
                  int32_t *nvals, arb_csv_info *info, arb_stream_t stream);
int arb_csv_parse(const uint8_t *text, int64_t nbytes, int64_t nlines, int32_t delimiter, int32_t comment,
                  void *lines_work, size_t lines_work_bytes, const int32_t *nvals, double *out, int64_t nrows,
                  int64_t ncols, arb_csv_info *info, arb_stream_t stream);

/* Test hook, no counterpart in the reference: sets the poll limit of the
 * 3D tensor-core solve's MMA-completion wait (arb_coef_solve, mixed
 * precision) on the current device; limit < 0 restores the default (2^22
 * polls).  With a limit of 0 that wait gives up at once: the kernel ORs
 * ARB_ERR_TIMEOUT into the status word, waits (with the full limit) for the
 * MMAs it issued, releases its tensor memory and returns.  Tests use it to
 * exercise the timeout path without faulting or hanging the GPU. */
int arb_test_set_mma_wait_limit(int64_t limit);

/* Reads (and clears) the device status word after the stream's work is
 * done; returns ARB_OK, an arb_status bit set, or ARB_ERR_CUDA. */
int arb_status_fetch(int32_t *status, arb_stream_t stream);

/* Clears a device status word on the stream (one memset; for a new word,
 * without waiting). */
int arb_status_clear(int32_t *status, arb_stream_t stream);

/* Library version string ("arbinterp-gb300 <ver> sm_103a"). */
const char *arb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* ARBINTERP_H */
