// Internal types of libaxgb: device buffers, meshes, matrices, batches and
// the entry points the C ABI layer (api.cpp) calls into the CUDA translation
// units (prep.cu, weights.cu, apply.cu, scan_sort.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/axgb.h"

namespace axgb {

using i64 = std::int64_t;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define AXGB_CUDA(x)                                                                                    \
    do {                                                                                                \
        cudaError_t e_ = (x);                                                                           \
        if (e_ != cudaSuccess)                                                                          \
            throw ::axgb::Error(e_ == cudaErrorMemoryAllocation ? AXGB_ERR_NOMEM : AXGB_ERR_CUDA,      \
                                std::string(#x) + ": " + cudaGetErrorString(e_));                       \
    } while (0)

#define AXGB_REQUIRE(cond, msg)                                                \
    do {                                                                       \
        if (!(cond)) throw ::axgb::Error(AXGB_ERR_INVALID, std::string(msg)); \
    } while (0)

// Owning device allocation (cudaMalloc / cudaFree), move-only.
template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    explicit DBuf(size_t count) { alloc(count); }
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) {
        o.p = nullptr;
        o.n = 0;
    }
    DBuf &operator=(DBuf &&o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DBuf() { release(); }
    void alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        AXGB_CUDA(cudaMalloc(reinterpret_cast<void **>(&p), count * sizeof(T)));
        n = count;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void upload(const T *h, size_t count, cudaStream_t s = 0) {
        if (count > n) alloc(count);
        if (count) AXGB_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    // Allocates at least one element and copies the vector's elements (none for an empty vector).
    template <class V>
    void upload_vec(const V &v, cudaStream_t s = 0) {
        if (v.size() + 1 > n || !p) alloc(v.size() > 0 ? v.size() : 1);
        if (!v.empty()) AXGB_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void download(T *h, size_t count, cudaStream_t s = 0) const {
        if (count) AXGB_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    void zero(cudaStream_t s = 0) {
        if (n) AXGB_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

// Result of the regular / rectilinear grid detection
// (detail/regular_grid_detector.hpp:64-299).
struct GridInfo {
    bool regular = false, rectilinear = false;
    i64 ni = 0, nj = 0;
    double lon_min = 0, lon_max = 0, dlon = 0, lat_min = 0, lat_max = 0, dlat = 0;
    std::vector<double> ulon, ulat;  // tolerance-unique sorted node coordinates
};

// Bounding cap of a cell: unit centroid and angular radius (radians).
struct __align__(32) DCap {
    double x, y, z, r;
};

// What device kernels read about a mesh (plain pointers, passed by value).
struct MeshView {
    i64 n_nodes, n_cells;
    const int *off;         // [n_cells+1] conn offsets
    const int *idx;         // conn node indices
    const double *xyz;      // [n_nodes*3] unit vectors (deg2rad trig, host libm)
    const double *lonlat;   // LayoutLeft [n_nodes,2]
    int regular;            // polygons from the node trig cache
    int ni, nj;             // regular grid shape
    const double *trig;     // [sin_lon(ni+1) cos_lon(ni+1) sin_lat(nj+1) cos_lat(nj+1)]
    const double *user_area;
    const int *mask;
    // per-cell products of the prep kernel
    double *area;
    DCap *cap;           // centroid xyz + angular radius
    float4 *capf;           // the same rounded to float (the search's cap prefilter)
    float *box;             // reference float AABB [n_cells*6]
    unsigned char *flags;   // bit0 degenerate, bit1 masked, bit2 area<=0; class in bits 4..5
};

struct Mesh {
    i64 n_nodes = 0, n_cells = 0, n_conn = 0;
    int coord_sys = AXGB_SPHERICAL_DEG;
    std::vector<double> lonlat;  // host LayoutLeft copy
    std::vector<i64> off, idx;
    GridInfo grid;
    bool has_area = false, has_mask = false;
    DBuf<int> d_off, d_idx, d_mask;
    DBuf<double> d_xyz, d_lonlat, d_trig, d_user_area, d_area;
    DBuf<DCap> d_cap;
    DBuf<float4> d_capf;
    DBuf<float> d_box;
    DBuf<unsigned char> d_flags;
    bool prepped = false;
    std::mutex mu;
    MeshView view() const;
};

// Sliced-ELL (32-row slices) apply layout. Entry k of row r of slice s is at
// base[s] + k*32 + (r % 32); padding entries have column 0 and weight 0.
struct Sell {
    bool built = false;
    i64 n_slices = 0, n_entries = 0;
    DBuf<int> base, len, col;
    DBuf<float> hi, lo;     // split weights (format 1)
    DBuf<double> w64;       // FP64 weights (format 0)
    // slice ids grouped by length class: <=8, <=16, <=32, <=64, >64
    std::vector<i64> class_begin;  // 6 entries into class_ids
    DBuf<int> class_ids;
    std::vector<int> class_maxlen;
    std::vector<int> h_slice_len;  // entries per row slot of each slice
    // Rows of more than 32 entries, row-contiguous in the layout's entry
    // order (for the warp-per-row kernels): row ids, offsets, entries.
    i64 n_lrows = 0;
    DBuf<int> lrow, lptr, lcol;
    DBuf<float> lhi, llo;   // format 1
    DBuf<double> lw64;      // format 0
};

// Blocked split-FP32 layout (staged.cu). Rows are grouped in blocks of up to
// 4 slices (128 rows) chosen for source locality; inside a block rows are
// sorted by length so each warp's trip count follows its own rows. Per block:
// the 16-byte chunks of source columns to stage (ccol), runs of consecutive
// chunks for bulk copies, and per entry the staging index (lidx; padding
// entries point at a zero slot), hi and lo weights, laid out k-major per warp.
struct Blocked {
    struct Launch {
        int L;        // row-length class (multiple of 4, <= 32)
        int us;       // staging floats per field (allocation for the class)
        i64 begin, n; // range in block_ids
    };
    bool built = false;
    i64 n_blocks = 0;
    i64 n_src = 0;  // source cells of the matrix (bounds the last staged chunk)
    DBuf<int> brow, wbase, wlen, cstart, ccol, rstart, block_ids, fallback_slices;
    DBuf<int4> runs;  // (global col of first chunk, chunks, staging offset, 0)
    DBuf<unsigned short> lidx;
    DBuf<float> hi, lo;
    std::vector<Launch> launches;
    std::vector<int> order;  // launches by size, largest first
    std::vector<int> h_us, h_block_ids;  // host copies: staging floats per block, block ids by class
    i64 n_fallback = 0;
    DBuf<int> status;  // device status word: 1 = a bounded wait timed out
    // stream pool for concurrent class launches (fork/join on the caller's stream)
    std::mutex pool_mu;
    std::vector<cudaStream_t> pool;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
    ~Blocked() {
        for (auto st : pool) cudaStreamDestroy(st);
        for (auto ev : join) cudaEventDestroy(ev);
        if (fork) cudaEventDestroy(fork);
    }
};

// Segmented split-FP32 layout (staged.cu, variant 5): lane = field. Rows in
// 8-row segments (one 32-byte sector of a field's outputs), four segments of
// nearby rows per group (a CTA: one warp per segment, one producer warp).
// Per group the distinct source cells of its rows (original numbering) are
// staged cell by cell for 32 fields, transposed ([cell][field], 33 floats a
// cell), so a warp's 32 lanes (fields) read one cell without bank
// conflicts. A segment's rows, sorted by length, are taken in pairs summed
// side by side with packed f32x2 arithmetic. Per entry pair: the staged
// offsets of both cells and (hi_a, hi_b, -lo_a, -lo_b). Rows of more than
// 32 entries, and the rows of groups with more staged cells than the
// largest bucket, are listed for the fallback kernels (original numbering).
struct Segmented {
    struct Launch {
        int usmax;     // staged-cell bucket of the launch
        i64 begin, n;  // range in gids
    };
    bool built = false;
    i64 n_groups = 0;
    DBuf<int4> grp;       // per group: (first cell in cellmap, cells, first entry pair, entry pairs)
    int max_ent = 0;      // entry pairs of the largest group
    DBuf<int4> slot;      // per group and segment: (segment id or -1, first entry pair, store mask, 0)
    DBuf<uint4> pairs;    // per group and segment: 4 x (ra | rb << 3 | has_b << 6 | length << 8)
    DBuf<int> cellmap, gids;
    DBuf<unsigned> eoff;  // per entry pair: staged float offsets (cell * 33) of row a | row b << 16
    DBuf<float4> ew;      // per entry pair: (hi_a, hi_b, -lo_a, -lo_b)
    std::vector<Launch> launches;
    // fallback rows of at most 32 entries: row ids and row-contiguous entries
    i64 n_fb = 0;
    DBuf<int> fb_row, fb_ptr, fb_col;
    DBuf<float> fb_hi, fb_lo;
    // rows of more than 32 entries, row-contiguous (original numbering)
    i64 n_long = 0;
    DBuf<int> l_row, l_ptr, l_col;
    DBuf<float> l_hi, l_lo;
    DBuf<int> status;  // 1 = a bounded wait timed out
    std::mutex pool_mu;
    std::vector<cudaStream_t> pool;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
    ~Segmented() {
        for (auto st : pool) cudaStreamDestroy(st);
        for (auto ev : join) cudaEventDestroy(ev);
        if (fork) cudaEventDestroy(fork);
    }
};

// Kernel choice for the split-FP32 apply.
struct SplitParams {
    int variant = 1;          // 0 direct gathers, 1 blocked + cp.async chunk staging,
                              // 2 blocked + bulk-copy (TMA) staging, 3 blocked + producer
                              // warp and mbarrier ring, 4 one fused launch (few fields)
    int fields_per_pass = 0;  // direct: RHS tile width; blocked: fields per work item (0 = all)
    int unroll = 4;           // direct: fields per thread iteration; staged: fields per stage
    int stages = 2;           // blocked: staging buffers (variants 1 and 3: 2-3, 2: 2)
};

struct Matrix {
    i64 n_src = 0, n_dst = 0, nnz = 0;
    DBuf<int> row_ptr, col;  // CSR (rows ascending, cols ascending in a row)
    DBuf<double> val, frac_a, frac_b, area_a, area_b;
    i64 stats[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double times_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    Sell sell64, sell32;
    Blocked blocked;
    Segmented seg;
    // Order of each row's entries in the split-FP32 layouts: split_perm[rp[r] + k]
    // is the CSR index of the k-th entry of row r. Chosen by the blocked build
    // against shared-memory bank conflicts and shared by every split layout,
    // so all split kernels sum in the same order (same bits).
    DBuf<int> split_perm;
    // Source renumbering of the split layouts (chosen by the blocked build
    // when the source cells' own numbering scatters each block's sources
    // over many 16-byte chunks): split_col holds the renumbered column of
    // every CSR entry, src_inv the original cell of every new index. A split
    // apply first gathers the fields into the new order.
    bool src_renum = false;
    DBuf<int> split_col, src_inv;
    // Per CSR entry, a key of its place in its row's generation order, for
    // the paths whose rows are not generated in column order (regular and
    // rectilinear conservative fast paths: candidate position; bilinear:
    // stencil corner). Empty: column order. Read by the coastal post-pass
    // (the reference sums a row's wet weights in generation order) and
    // released after generation.
    DBuf<int> gen_rank;
    std::vector<float> slice_xyz;  // mean unit vector of each 32-row slice (locality hint), may be empty
    std::vector<float> seg_xyz;    // the same for each 8-row segment (segmented layout)
    std::map<i64, SplitParams> tuned;  // nrhs -> best kernel choice
    std::mutex mu;
};

struct Batch;

// prep.cu
void mesh_prepare(Mesh &m, cudaStream_t s);  // cell prep kernel (once)

// weights.cu
void generate_conservative(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out);
// regular x regular fast path; false = declined (use generate_conservative)
bool generate_conservative_regular(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out);
// rectilinear x rectilinear fast path (non-uniform edges); false = an empty
// matrix under UnmappedAction::Error (use generate_conservative)
bool generate_conservative_rectilinear(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out);
// esmf_io.cpp: ESMF weight files (NetCDF-3); col1/row1 are 1-based
struct EsmfWeights {
    std::int64_t n_a = 0, n_b = 0;
    std::vector<double> S;
    std::vector<std::int32_t> col1, row1;
};
void esmf_write(const std::string &path, std::int64_t n_a, std::int64_t n_b, std::int64_t nnz, const double *S,
                const std::int32_t *col1, const std::int32_t *row1);
EsmfWeights esmf_read(const std::string &path);
// nearest.cu: nearest-neighbour weights (index rounding for two regular
// grids, else an exact float nearest query over centroid points)
void generate_nearest(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out);
// bilinear.cu: bilinear weights from a non-rectilinear source (nearest
// centroids, quad / triangle / inverse-distance stencils)
void generate_bilinear_general(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out);
// regular x regular bilinear fast path; false = no destination cells (fall through)
bool generate_bilinear_regular(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out);
void generate_bilinear(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out);

// coastal.cu: wet renormalisation and NearestWet extrapolation after any
// method when the source mesh has a cell mask
void coastal_postpass(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &m);

// apply.cu
void matrix_prepare(Matrix &m, int format, cudaStream_t s);
void apply_f64(Matrix &m, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, cudaStream_t s);
// ylo (optional): low parts of the outputs, so that y + ylo carries each row
// value s + c to about 2^-48 relative (y's bits are unchanged).
void apply_split(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, const SplitParams &p,
                 cudaStream_t s, float *ylo = nullptr, i64 ldylo = 0);
void conservation(Matrix &m, const void *src, const void *dst, bool f32, int norm_type, double *out, cudaStream_t s);
double fp64_fma_tflops(i64 iters);  // FP64 FMA throughput of the current device (TFLOP/s)
void nan_batch_apply_f64(Matrix &m, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, double na_thres,
                         cudaStream_t s);
void apply_masked_f64(Matrix &m, const double *x, const int *mask, double *y, cudaStream_t s);
void conservation_noalloc(Matrix &m, const double *src, const double *dst, int norm_type, double *out,
                          cudaStream_t s);
std::shared_ptr<Batch> batch_create(const std::vector<std::shared_ptr<Matrix>> &mats, const std::vector<i64> &nrhs);
void batch_apply(Batch &b, const float *const *x, const i64 *ldx, float *const *y, const i64 *ldy, cudaStream_t s);

// staged.cu
void build_blocked(Matrix &m, cudaStream_t s);
bool blocked_eligible(const Matrix &m, const void *x, i64 ldx, bool bulk);
void launch_long_rows(const int *row, const int *ptr, const int *col, const float *hi, const float *lo, i64 n,
                      const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s, float *ylo, i64 ldylo);
void build_segmented(Matrix &m, cudaStream_t s);
void apply_segmented(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s, float *ylo,
                     i64 ldylo, int ns);
void apply_blocked(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, int kind, int T, int ns,
                   i64 fchunk, cudaStream_t s, float *ylo = nullptr, i64 ldylo = 0);
int blocked_launches(const Matrix &m);
// persistent staged kernels over the blocked layouts of several matrices
// (batches); use[q] selects the matrices whose fields allow the staged kernels
struct BlkBatch;
std::shared_ptr<BlkBatch> blk_batch_create(const std::vector<Matrix *> &mats, const std::vector<i64> &nrhs,
                                           const std::vector<char> &use);
void blk_batch_set_fields(BlkBatch &bb, const float *const *x, const i64 *ldx, float *const *y, const i64 *ldy,
                          cudaStream_t s);
void blk_batch_launch(BlkBatch &bb, const cudaStream_t *streams, int n_streams);
void slice_centroids(const MeshView &dst, Matrix &m, cudaStream_t s);
// get_cell_areas of src/solver/weight_generator.cpp:297-312: the mesh's own
// areas where it has them, else planar shoelace areas in degrees (nearest.cu).
void planar_cell_areas(const MeshView &m, double *out, cudaStream_t s);

// scan_sort.cu: device primitives (own implementations)
// out[0..n] = exclusive prefix sum of in[0..n-1], out[n] = total.
void scan_exclusive_i32_to_i64(const int *in, i64 *out, i64 n, cudaStream_t s);
void scan_exclusive_i32(const int *in, int *out, i64 n, cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs on the low key_bits bits.
void radix_sort_pairs_u64(std::uint64_t *keys, int *vals, i64 n, int key_bits, cudaStream_t s);
void radix_sort_pairs_u32(std::uint32_t *keys, int *vals, i64 n, int key_bits, cudaStream_t s);

}  // namespace axgb
