/*
 * axgb.h — C ABI of the GB300 (sm_103a) implementation of the AXIS
 * regridding hot path: first-order conservative, bilinear and
 * nearest-neighbour weight generation (with the reference's fast paths,
 * masks and coastal post-pass), and the sparse weight apply.
 *
 * Conventions (those of the AXIS Fortran/C interop layer,
 * libs/axis/src/fortran/axis_c_interop.cpp:36-62):
 *   - every entry point returns 0 (AXGB_SUCCESS) or a negative code; the
 *     message of the last failure on the calling thread is available from
 *     axgb_last_error();
 *   - objects are opaque int handles >= 1 (0 is never a valid handle),
 *     kept in a mutex-guarded registry (handle_registry.hpp:32-60);
 *   - extents are validated before any output is written
 *     (libs/axis/include/axis/solver/apply.hpp:63-71).
 * Device-pointer entry points are stream-ordered on the given CUDA stream
 * (0 = the legacy default stream) and return once the work is enqueued;
 * host-pointer entry points are synchronous.
 * Nothing here allocates on the calling thread's behalf in the apply path
 * except the first use of a matrix in a given format (see axgb_matrix_prepare).
 */
#ifndef AXGB_H
#define AXGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void *axgb_stream_t; /* a cudaStream_t */

/* Return codes. AXGB_ERROR matches AXIS_ERROR (-1). */
#define AXGB_SUCCESS 0
#define AXGB_ERROR (-1)
#define AXGB_ERR_INVALID (-2)     /* bad argument / extent mismatch (std::invalid_argument) */
#define AXGB_ERR_CUDA (-3)        /* CUDA runtime failure */
#define AXGB_ERR_UNSUPPORTED (-4) /* method/dispatch branch not provided by this library */
#define AXGB_ERR_NOMEM (-5)       /* device allocation failed */
#define AXGB_ERR_TIMEOUT (-6)     /* a bounded device wait gave up */
#define AXGB_ERR_UNMAPPED (-7)    /* UnmappedAction::Error hit an uncovered destination cell */
#define AXGB_ERR_HANDLE (-8)      /* unknown or destroyed handle */

/* Enumerations with the values of libs/axis/include/axis/solver/regrid_config.hpp:24-72
 * and libs/axis/include/axis/topology/enums.hpp:73-80. */
enum axgb_method {
    AXGB_BILINEAR = 0,
    AXGB_NEAREST_NEIGHBOR = 1,
    AXGB_BICUBIC = 2,
    AXGB_PATCH = 3,
    AXGB_CONSERVATIVE = 4,
    AXGB_CONSERVATIVE_2ND = 5
};
enum axgb_norm_type { AXGB_DSTAREA = 0, AXGB_FRACAREA = 1 };
enum axgb_line_type { AXGB_CARTESIAN = 0, AXGB_GREAT_CIRCLE = 1 };
enum axgb_unmapped { AXGB_UNMAPPED_ERROR = 0, AXGB_UNMAPPED_IGNORE = 1 };
enum axgb_extrap { AXGB_EXTRAP_NONE = 0, AXGB_EXTRAP_NEAREST_WET = 1 };
enum axgb_coord_sys { AXGB_SPHERICAL_DEG = 0, AXGB_SPHERICAL_RAD = 1, AXGB_CARTESIAN3D = 2 };

/* RegridConfig (regrid_config.hpp:80-89), one int per field. */
typedef struct axgb_regrid_config {
    int32_t method;
    int32_t norm_type;
    int32_t line_type;
    int32_t unmapped;
    int32_t use_limiter;
    int32_t extrap_method;
} axgb_regrid_config;

/* Fills the RegridConfig defaults: Bilinear, DstArea, GreatCircle, Ignore,
 * no limiter, NearestWet (regrid_config.hpp:80-89). */
void axgb_default_config(axgb_regrid_config *cfg);

/* Replaces axis_init_c (axis_c_interop.cpp:88-90): selects the CUDA device
 * for this process and creates the library context. Safe to call again. */
int axgb_init(int device);

/* Copies the message of the last failure on this thread (NUL-terminated,
 * truncated to len). Returns the full message length. */
int axgb_last_error(char *buf, size_t len);

/* Library build/identity string (arch, version). */
const char *axgb_version(void);

/* ─── Meshes ─────────────────────────────────────────────────────────────
 * Replaces UnstructuredMesh construction (unstructured_mesh.hpp:68-76) /
 * make_ugrid_mesh (python/axis_py.cpp:126-140) / axis_mesh_from_descriptor_c
 * (axis_c_interop.cpp:105-109). Host pointers:
 *   node_coords  [n_nodes, 2] LayoutLeft (all lon, then all lat), degrees
 *                for AXGB_SPHERICAL_DEG;
 *   conn_offsets [n_cells + 1], conn_indices [conn_offsets[n_cells]] (CSR);
 *   areas        optional precomputed cell areas [n_cells] or NULL;
 *   mask         optional cell mask [n_cells] (0 = masked) or NULL.
 * The arrays are copied; the caller keeps ownership. */
int axgb_mesh_create(const double *node_coords, int64_t n_nodes, const int64_t *conn_offsets,
                     const int64_t *conn_indices, int64_t n_cells, int coord_sys, const double *areas,
                     const int32_t *mask, int *mesh_handle);

/* Replaces make_regular_mesh (python/axis_py.cpp:75-103). */
int axgb_mesh_create_regular(int64_t ni, int64_t nj, double lon_start, double lat_start, double dlon, double dlat,
                             int *mesh_handle);

/* Mesh facts: n_nodes, n_cells, and the regular/rectilinear detection of
 * detail/regular_grid_detector.hpp:64-299 (flags[0] regular, flags[1]
 * rectilinear; dims = ni, nj; vals = lon_min, delta_lon, lat_min, delta_lat).
 * Any output pointer may be NULL. */
int axgb_mesh_info(int mesh_handle, int64_t *n_nodes, int64_t *n_cells, int32_t *flags, int64_t *dims,
                   double *vals);

/* Per-cell geometry computed on the device for this mesh (host outputs,
 * each may be NULL): spherical area (spherical_clipper.hpp:112-137),
 * bounding-cap centroid [n,3] and angular radius
 * (spherical_cap_filter.hpp:85-173), the dilated float AABB [n,6]
 * (weight_generator.cpp:198-262) and the degenerate class
 * (degenerate_cell_handler.hpp:115-142: 0 none, 1 zero area, 2 collapsed,
 * 3 self-intersecting). */
int axgb_mesh_cell_geometry(int mesh_handle, double *area, double *cap_centroid, double *cap_radius, float *box,
                            int32_t *degenerate);

/* Replaces axis_destroy_mesh_c (axis_c_interop.cpp:240-242). */
int axgb_destroy_mesh(int mesh_handle);

/* ─── Weight generation ──────────────────────────────────────────────────
 * Replaces WeightGenerator::generate (solver/weight_generator.hpp:60-62,
 * weight_generator.cpp:1887-2019) and python generate_weights
 * (axis_py.cpp:633-652), in the reference's dispatch order:
 *   - Conservative1stOrder: regular x regular (analytic, may decline), then
 *     rectilinear x rectilinear, then the general BVH + spherical clipper
 *     path (GreatCircle lines only);
 *   - Bilinear: regular x regular, else a rectilinear source, else the
 *     point-location path for any source mesh;
 *   - NearestNeighbor: regular index rounding, else an exact nearest search.
 * Cell masks and user areas of the meshes are honoured, and a masked source
 * goes through the coastal post-pass (renormalisation, NearestWet). Other
 * methods (Bicubic, Patch, Conservative2ndOrder) and Cartesian lines on the
 * clipper path return AXGB_ERR_UNSUPPORTED. The matrix lives on the device
 * in CSR form with its frac_a/frac_b/area_a/area_b arrays. Synchronous. */
int axgb_generate_weights(int src_mesh, int dst_mesh, const axgb_regrid_config *cfg, int *matrix_handle);

/* Replaces axis_generate_weights_c (axis_c_interop.cpp:117-145): method code
 * 0 Bilinear, 1 NearestNeighbor, 2 Conservative1stOrder, other fields default. */
int axgb_generate_weights_c(int src_mesh, int dst_mesh, int method, int *matrix_handle);

/* Statistics of the last generation into this matrix. stats (int64[8]):
 * BVH candidate pairs, pairs passing the reference gates (float AABB, cap,
 * degenerate, area, mask), pairs clipped with the 32-vertex fallback,
 * kept pairs (nnz), LBVH nodes, the kernel launches per split-FP32 apply
 * of the direct and of the blocked variants (each known after
 * axgb_matrix_prepare of its format), and 1 when the split layouts renumber
 * the source cells (known after axgb_matrix_prepare of format 1 or 2; a
 * split apply then first gathers the fields into that order, in scratch of
 * the fields' size taken with cudaMallocAsync on the apply's stream).
 * times_ms (double[8]): cell prep,
 * LBVH build, candidate search, clip, CSR assembly, total, 0, 0. */
int axgb_matrix_stats(int matrix_handle, int64_t *stats, double *times_ms);

/* n_src, n_dst, nnz of a matrix (InterpolationMatrix accessors,
 * interpolation_matrix.hpp:97-111). Any pointer may be NULL. */
int axgb_matrix_info(int matrix_handle, int64_t *n_src, int64_t *n_dst, int64_t *nnz);

/* Copies the CSR arrays to HOST buffers (to_csr order: rows ascending,
 * columns ascending within a row; interpolation_matrix.hpp:180-255) and the
 * frac/area arrays. Any pointer may be NULL. */
int axgb_matrix_export_csr(int matrix_handle, int64_t *row_ptr, int64_t *col_idx, double *values, double *frac_a,
                           double *frac_b, double *area_a, double *area_b);

/* Builds a device matrix from HOST CSR arrays (columns must lie in
 * [0, n_src); rows need not be column-sorted). frac/area may be NULL
 * (filled with 1 and 0). Mirrors the InterpolationMatrix adopting
 * constructor (interpolation_matrix.hpp:80-92) followed by to_csr(). */
/* Weight cache blob: the binary format of WeightCache
 * (include/axis/solver/weight_cache.hpp:49-157), so weights round-trip with
 * the reference. 40-byte header [magic u32 0x43574841 (bytes "AHWC")]
 * [version 1 u32][endian u8]
 * [pad 7][n_src u64][n_dst u64][nnz u64], then factor_list f64[nnz],
 * factor_row i64[nnz], factor_col i64[nnz], frac_a f64[n_src], frac_b
 * f64[n_dst], area_a f64[n_src], area_b f64[n_dst]; the triplets are written
 * in CSR order. serialize: buf NULL returns the size in *written; a smaller
 * buf_size is AXGB_ERR_INVALID. deserialize validates magic, version,
 * endianness and size (AXGB_ERR_INVALID otherwise) and builds a matrix as
 * axgb_matrix_import_csr does (triplets in any order). */
int axgb_matrix_serialize(int matrix_handle, void *buf, int64_t buf_size, int64_t *written);
int axgb_matrix_deserialize(const void *buf, int64_t buf_size, int *matrix_handle);

/* ESMF weight files: EsmfWeightIO::write_esmf / read_esmf
 * (src/io/esmf_weight_io.cpp:66-183). The file holds dimension num_wgts,
 * variables S (double), col_idx and row_idx (int, 1-based) and global int
 * attributes n_a, n_b (source / destination cell counts). It is written in
 * the NetCDF-3 64-bit-offset format, which libnetcdf (and so the reference's
 * read_esmf) opens. Reading takes NetCDF-3 classic and 64-bit-offset files;
 * a NETCDF4 (HDF5) file, the format the reference writes, or a CDF-5 file is
 * AXGB_ERR_UNSUPPORTED. A missing attribute or variable is AXGB_ERR_INVALID.
 * axgb_esmf_write / axgb_esmf_read work on host arrays and need no device;
 * axgb_esmf_read with S NULL only returns the sizes. axgb_matrix_write_esmf
 * writes a matrix's entries in CSR order; axgb_matrix_read_esmf builds a
 * matrix from a file with frac and area arrays zero, as the reference's
 * reader leaves them. */
int axgb_esmf_write(const char *path, int64_t n_a, int64_t n_b, int64_t nnz, const double *S, const int32_t *col_idx,
                    const int32_t *row_idx);
int axgb_esmf_read(const char *path, int64_t *n_a, int64_t *n_b, int64_t *nnz, double *S, int32_t *col_idx,
                   int32_t *row_idx, int64_t capacity);
int axgb_matrix_write_esmf(int matrix_handle, const char *path);
int axgb_matrix_read_esmf(const char *path, int *matrix_handle);

int axgb_matrix_import_csr(int64_t n_src, int64_t n_dst, int64_t nnz, const int64_t *row_ptr, const int64_t *col_idx,
                           const double *values, const double *frac_a, const double *frac_b, const double *area_a,
                           const double *area_b, int *matrix_handle);

/* Builds the apply layouts of a matrix ahead of time (format 0: FP64
 * sliced-ELL, 1: split-FP32 hi+lo sliced-ELL, 2: the blocked staged
 * split-FP32 layout, which also builds 1, 3: the segmented split-FP32
 * layout of variant 5, which also builds 2) so that later apply calls
 * allocate nothing. Synchronous. */
int axgb_matrix_prepare(int matrix_handle, int format);

/* Reads (and clears) the device status word of a matrix's bulk-staged apply:
 * 0 = fine, 1 = a bounded wait for staged copies gave up (the affected
 * block rows were not written). Synchronizes the device. */
int axgb_matrix_device_status(int matrix_handle, int32_t *status);

/* Measures the FP64 FMA throughput of the current device (TFLOP/s, two flops
 * per FMA): independent dependent-FMA chains on every SM, iters FMAs per
 * chain (1 .. 2^24), timed with CUDA events. The roofline denominator of the
 * FP64 apply and of the clipper, which run on the FP64 pipe. Synchronous.
 * No reference counterpart (a measurement aid). */
int axgb_probe_fp64_fma(int64_t iters, double *tflops);

/* Replaces axis_destroy_matrix_c (axis_c_interop.cpp:247-249). */
int axgb_destroy_matrix(int matrix_handle);

/* ─── Apply (device pointers) ────────────────────────────────────────────
 * y[:, v] = S x[:, v] for v < nrhs; x is [nrhs][ld_x] (field v starts at
 * x + v*ld_x, ld_x >= n_src), y is [nrhs][ld_y]. This is the LayoutLeft
 * (n_cells, n_vars) layout of batch_apply (apply.hpp:275-343); nrhs = 1 is
 * the single-field apply (apply.hpp:61-119). y is overwritten. */
int axgb_apply_f64(int matrix_handle, const double *x, int64_t ld_x, double *y, int64_t ld_y, int64_t nrhs,
                   axgb_stream_t stream);

/* FP32 fields, FP64 weights stored as an FP32 hi+lo pair, products and sums
 * carried with error-free transforms and compensated per row. New in this
 * library (the reference applies in FP64 only). */
int axgb_apply_f32split(int matrix_handle, const float *x, int64_t ld_x, float *y, int64_t ld_y, int64_t nrhs,
                        axgb_stream_t stream);

/* axgb_apply_f32split with a second output: y is bitwise the result of
 * axgb_apply_f32split (every split kernel gives the same bits), and
 * y_lo[:, v] ([nrhs][ld_lo])
 * receives the rounding error of each stored value, so that y + y_lo in
 * FP64 carries the compensated row sum to about 2^-48 relative: the form for
 * conservation-grade results (global integrals of y + y_lo meet the FP64
 * apply's), at 4 more bytes per output written. Replaces no reference
 * interface (the reference applies in FP64 only). */
int axgb_apply_f32split_hilo(int matrix_handle, const float *x, int64_t ld_x, float *y, int64_t ld_y, float *y_lo,
                             int64_t ld_lo, int64_t nrhs, axgb_stream_t stream);

/* Same, kernel choice explicit. variant 0: direct gathers from global
 * memory, fields_per_pass = RHS tile width (0 = all), unroll = fields per
 * thread iteration (1, 2 or 4). variants 1 to 3: rows in blocks of 4
 * slices grouped by source locality; per block the source values are staged
 * in shared memory as 16-byte chunks, variant 1 with cp.async by all
 * threads (two staging buffers), variant 2 with bulk (TMA) copies completing
 * on an mbarrier, variant 3 with cp.async by a producer warp into a ring of
 * two or three slots guarded by mbarriers (4 fields per stage); unroll =
 * fields per stage (2, 4 or 8),
 * fields_per_pass = fields per work item of a block (0 = all). Variants 1
 * to 3 need x 16-byte aligned and ld_x a multiple of 4 (variant 2 also n_src
 * a multiple of 4); otherwise the direct kernel runs. variant 4: the whole
 * matrix in one launch (for one or a few fields); the other knobs are
 * unused. variant 5: segmented, one lane per field: groups of 32 nearby
 * rows stage their distinct source cells (original numbering, any x
 * alignment) for 32 fields at a time; stages = staging slots (2 or 3).
 * Every variant gives the same bits. */
int axgb_apply_f32split_tuned(int matrix_handle, const float *x, int64_t ld_x, float *y, int64_t ld_y, int64_t nrhs,
                              int variant, int fields_per_pass, int unroll, axgb_stream_t stream);

/* Autotuner: times the split apply over (variant, fields_per_pass, unroll,
 * staging buffers) choices on the given device buffers, caches the best per
 * (matrix, nrhs) and returns it in best[4]. Used automatically by
 * axgb_apply_f32split when enabled with axgb_set_autotune(1). */
int axgb_autotune_f32split(int matrix_handle, const float *x, int64_t ld_x, float *y, int64_t ld_y, int64_t nrhs,
                           axgb_stream_t stream, int32_t *best);
int axgb_set_autotune(int enable);

/* Read or seed the cached kernel choice of (matrix, nrhs) that
 * axgb_apply_f32split uses: choice[4] = variant, fields_per_pass, unroll,
 * stages (staging buffers: 2 or 3 with variants 1 and 3, else 2; variant 3
 * also 0 = per row-length class the depth that lets more CTAs fit), as
 * axgb_autotune_f32split returns
 * it. Seeding lets a caller reuse a choice tuned in an earlier process
 * without timing again. When nothing is cached for (matrix, nrhs), get
 * sets *cached = 0 and returns the default choice. */
int axgb_set_kernel_choice(int matrix_handle, int64_t nrhs, const int32_t *choice);
int axgb_get_kernel_choice(int matrix_handle, int64_t nrhs, int32_t *choice, int32_t *cached);

/* NaN-aware batched FP64 apply; replaces nan_batch_apply
 * (include/axis/solver/apply.hpp:359-437, python/axis_py.cpp:764-821).
 * Device pointers, x [nrhs][ld_x], y [nrhs][ld_y] (y overwritten). Per row:
 * the total weight; per field: the weighted sum and the weight of the
 * sources that are not NaN. y is NaN where no source is valid or the valid
 * weight fraction is below 1 - na_thres - 1e-6, else the weighted sum over
 * the valid weight. Sums run in CSR order with separate multiply and add, as
 * the reference's loop, so NaN positions and values match it exactly. */
int axgb_nan_batch_apply_f64(int matrix_handle, const double *x, int64_t ld_x, double *y, int64_t ld_y,
                             int64_t nrhs, double na_thres, axgb_stream_t stream);

/* Masked single-field FP64 apply; replaces the masked solver::apply
 * (include/axis/solver/apply.hpp:458-532). Device pointers; dst_mask
 * [n_dst] int32 (0 = masked: y left unchanged) or NULL (every row). */
int axgb_apply_masked_f64(int matrix_handle, const double *x, double *y, const int32_t *dst_mask,
                          axgb_stream_t stream);

/* ─── Apply (host pointers, synchronous) ─────────────────────────────────
 * Replaces axis_apply_c (axis_c_interop.cpp:217-236): FP64, one field,
 * host arrays; returns AXGB_ERR_INVALID before touching dst on extent
 * mismatch. */
int axgb_apply_c(int matrix_handle, const double *src, double *dst, int n_src, int n_dst);

/* Replaces python batch_apply (axis_py.cpp:690-759) for host arrays laid
 * out LayoutLeft [n_src, n_vars] / [n_dst, n_vars]. */
/* axgb_nan_batch_apply_f64 on host arrays: src [n_src, n_vars] and dst
 * [n_dst, n_vars] column-major (LayoutLeft, one field after another), the
 * layout nan_batch_apply takes. Synchronous. */
int axgb_nan_batch_apply_host(int matrix_handle, const double *src, int64_t n_src, double *dst, int64_t n_dst,
                              int64_t n_vars, double na_thres);
int axgb_batch_apply_host_f64(int matrix_handle, const double *src, int64_t n_src, double *dst, int64_t n_dst,
                              int64_t n_vars);
int axgb_batch_apply_host_f32split(int matrix_handle, const float *src, int64_t n_src, float *dst, int64_t n_dst,
                                   int64_t n_vars);

/* ─── Many grid pairs in one persistent launch ───────────────────────────
 * A batch groups k matrices, each with its own field count. axgb_batch_apply
 * runs all of them (split-FP32) in persistent kernels fed by work queues: one
 * per row-length class of the staged layout over (matrix, field chunk, block)
 * items, and two direct ones over the rows and slices that layout leaves out,
 * replayed from a CUDA graph captured on first use per stream and per
 * pointer set. A batch's graphs
 * share its work counters and descriptors: a call on another stream than
 * the previous call's waits on the GPU for the previous call's work, so one
 * batch never runs on two streams at once. No reference counterpart: the
 * reference applies one matrix per call. */
int axgb_batch_create(const int *matrix_handles, const int64_t *nrhs, int count, int *batch_handle);
int axgb_batch_apply(int batch_handle, const float *const *x, const int64_t *ld_x, float *const *y,
                     const int64_t *ld_y, axgb_stream_t stream);
int axgb_destroy_batch(int batch_handle);

/* ─── Conservation (device pointers to FP64 fields) ──────────────────────
 * check_conservation (solver/conservation.hpp:96, conservation.cpp:83-96):
 * out[0] source integral sum(src*area_a*frac_a), out[1] destination integral
 * (DstArea: sum over frac_b != 0 of dst*area_b; FracArea: * frac_b),
 * out[2] |difference|, out[3] relative error. Synchronous. */
int axgb_conservation_f64(int matrix_handle, const double *src, const double *dst, int norm_type, double *out,
                          axgb_stream_t stream);
int axgb_conservation_f32(int matrix_handle, const float *src, const float *dst, int norm_type, double *out,
                          axgb_stream_t stream);

/* axgb_conservation_f64 for callers that cannot allocate device memory
 * while they run (a model whose device memory belongs to its own pool, or
 * code that must not call cudaMalloc between its set-up and tear-down). It
 * allocates nothing: its partial sums live in a fixed 128 KiB array that the
 * library places in every GPU that loads it, kept until the process exits.
 * Limit: n_src and n_dst at most 16,777,216 cells each; larger matrices get
 * AXGB_ERR_INVALID (use axgb_conservation_f64). The first call on a device
 * looks the array's device address up once; make that first call before
 * any stream capture. All calls share the one array, so calls that overlap
 * on the GPU (other streams or host threads) race; no slot needs clearing
 * between calls. Synchronous. It has no counterpart in the reference, which
 * always allocates its reduction scratch. */
int axgb_conservation_f64_noalloc(int matrix_handle, const double *src, const double *dst, int norm_type,
                                  double *out, axgb_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* AXGB_H */
