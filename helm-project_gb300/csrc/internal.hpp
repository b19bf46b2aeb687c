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
};

// Staged split-FP32 layout: rows in blocks of 4 slices (128 rows); per block the sorted
// unique source columns (ucol[ustart[b] .. +ucount[b]]) and, per entry in the
// sliced-ELL positions of Sell, the 16-bit index of its column in that list.
struct Staged {
    bool built = false;
    i64 n_blocks = 0;
    // block b = slices bslices[b].{x,y,z,w} (-1 = none), grouped by source locality
    std::vector<int4> h_bslices;
    DBuf<int4> bslices;
    DBuf<int> blk_of_slice;
    DBuf<unsigned short> lidx;
    DBuf<int> ucol, ustart, ucount;
    // block ids by class (max slice length <= 8, <= 16, <= 32 and unique
    // columns <= kStagedMaxU = 2048); slices of all other blocks use the direct kernel
    std::vector<i64> class_begin;  // 4 entries into block_ids
    std::vector<int> class_umax;
    DBuf<int> block_ids, fallback_slices;
    i64 n_fallback = 0;
};

// Bulk-staged layout on top of Staged: per block the unique columns as runs
// of 16-byte chunks copied with cp.async.bulk, and per sliced-ELL entry the
// index into the block's staging area (padding -> the zero slot).
struct Bulk {
    bool built = false;
    DBuf<unsigned short> lidx;
    DBuf<int> rstart, bus, block_ids, fallback_slices, cstart, ccol;
    DBuf<int4> runs;
    std::vector<i64> class_begin;  // 9 entries: row-length classes 4, 8, ..., 32
    std::vector<int> class_usmax;
    i64 n_fallback = 0;
    DBuf<int> status;  // device status word: 1 = a bounded wait timed out
};

// Kernel choice for the split-FP32 apply.
struct SplitParams {
    int variant = 2;          // 0 direct, 1 cp.async 4-byte staged, 2 cp.async 16-byte chunk staged,
                              // 3 bulk-copy (TMA) staged
    int fields_per_pass = 0;  // direct: RHS tile width (0 = all)
    int unroll = 4;           // direct: fields per thread iteration; staged: fields per stage
};

struct Matrix {
    i64 n_src = 0, n_dst = 0, nnz = 0;
    DBuf<int> row_ptr, col;  // CSR (rows ascending, cols ascending in a row)
    DBuf<double> val, frac_a, frac_b, area_a, area_b;
    i64 stats[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double times_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    Sell sell64, sell32;
    Staged staged;
    Bulk bulk;
    std::map<i64, SplitParams> tuned;  // nrhs -> best kernel choice
    std::mutex mu;
};

struct Batch;

// prep.cu
void mesh_prepare(Mesh &m, cudaStream_t s);  // cell prep kernel (once)

// weights.cu
void generate_conservative(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out);
void generate_bilinear(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out);

// apply.cu
void matrix_prepare(Matrix &m, int format, cudaStream_t s);
void apply_f64(Matrix &m, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, cudaStream_t s);
void apply_split(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, const SplitParams &p,
                 cudaStream_t s);
void conservation(Matrix &m, const void *src, const void *dst, bool f32, int norm_type, double *out, cudaStream_t s);
std::shared_ptr<Batch> batch_create(const std::vector<std::shared_ptr<Matrix>> &mats, const std::vector<i64> &nrhs);
void batch_apply(Batch &b, const float *const *x, const i64 *ldx, float *const *y, const i64 *ldy, cudaStream_t s);

// scan_sort.cu: device primitives (own implementations)
// out[0..n] = exclusive prefix sum of in[0..n-1], out[n] = total.
void scan_exclusive_i32_to_i64(const int *in, i64 *out, i64 n, cudaStream_t s);
void scan_exclusive_i32(const int *in, int *out, i64 n, cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs on the low key_bits bits.
void radix_sort_pairs_u64(std::uint64_t *keys, int *vals, i64 n, int key_bits, cudaStream_t s);
void radix_sort_pairs_u32(std::uint32_t *keys, int *vals, i64 n, int key_bits, cudaStream_t s);

}  // namespace axgb
