// C ABI of libaxgb (include/axgb.h): handle registry, error barrier, host
// side of mesh ingest, and the apply entry points.
//
// Mesh ingest keeps two host steps of the reference on the host on
// purpose: node unit vectors are computed with the host libm
// (lonlat_to_xyz, libs/axis/include/axis/detail/spherical_geometry.hpp:80-83)
// so the vertex bits the clipper sees are the reference's bits, and the
// regular/rectilinear detection (detail/regular_grid_detector.hpp:64-299)
// runs on sorted node coordinates with a parallel sort. Everything after
// that runs on the GPU.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <parallel/algorithm>
#include <thread>

#include "internal.hpp"

namespace axgb {
namespace {

thread_local std::string g_last_error;
std::atomic<int> g_autotune{0};

struct Registry {
    std::mutex mu;
    int next = 1;
    std::map<int, std::shared_ptr<Mesh>> meshes;
    std::map<int, std::shared_ptr<Matrix>> mats;
    std::map<int, std::shared_ptr<Batch>> batches;
    static Registry &get() {
        static Registry r;
        return r;
    }
    template <class T>
    int add(std::map<int, std::shared_ptr<T>> &m, std::shared_ptr<T> v) {
        std::lock_guard<std::mutex> lk(mu);
        int h = next++;
        m[h] = std::move(v);
        return h;
    }
    template <class T>
    std::shared_ptr<T> find(std::map<int, std::shared_ptr<T>> &m, int h, const char *what) {
        std::lock_guard<std::mutex> lk(mu);
        auto it = m.find(h);
        if (it == m.end()) throw Error(AXGB_ERR_HANDLE, std::string("unknown ") + what + " handle " + std::to_string(h));
        return it->second;
    }
    template <class T>
    void drop(std::map<int, std::shared_ptr<T>> &m, int h, const char *what) {
        std::shared_ptr<T> keep;
        {
            std::lock_guard<std::mutex> lk(mu);
            auto it = m.find(h);
            if (it == m.end())
                throw Error(AXGB_ERR_HANDLE, std::string("unknown ") + what + " handle " + std::to_string(h));
            keep = std::move(it->second);
            m.erase(it);
        }
    }
};

#define AXGB_TRY(...)                                    \
    try {                                                \
        __VA_ARGS__;                                     \
        return AXGB_SUCCESS;                             \
    } catch (const ::axgb::Error &e) {                   \
        ::axgb::g_last_error = e.what();                 \
        return e.code;                                   \
    } catch (const std::bad_alloc &) {                   \
        ::axgb::g_last_error = "host allocation failed"; \
        return AXGB_ERR_NOMEM;                           \
    } catch (const std::exception &e) {                  \
        ::axgb::g_last_error = e.what();                 \
        return AXGB_ERROR;                               \
    } catch (...) {                                      \
        ::axgb::g_last_error = "unknown exception";      \
        return AXGB_ERROR;                               \
    }

constexpr double kPi = 3.14159265358979323846;
constexpr double kDeg2Rad = kPi / 180.0;

template <class F>
void parallel_range(i64 n, F f) {
    unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (n < 65536 || nt == 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    i64 chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        i64 b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([=] { f(b, e); });
    }
    for (auto &t : th) t.join();
}

std::vector<double> unique_tol(std::vector<double> v) {
    __gnu_parallel::sort(v.begin(), v.end());
    std::vector<double> u;
    if (v.empty()) return u;
    u.push_back(v[0]);
    for (size_t i = 1; i < v.size(); ++i)
        if (std::abs(v[i] - u.back()) > 1.0e-12) u.push_back(v[i]);
    return u;
}

bool uniform(const std::vector<double> &d) {
    if (d.empty()) return false;
    double mn = d[0], mx = d[0], s = 0.0;
    for (double x : d) {
        mn = std::min(mn, x);
        mx = std::max(mx, x);
        s += x;
    }
    if (mn <= 0.0) return false;
    double mean = s / static_cast<double>(d.size());
    return (mx - mn) < 1.0e-10 * mean;
}

// detect_regular_grid + detect_rectilinear_grid (regular_grid_detector.hpp:64-299)
GridInfo detect(const Mesh &m) {
    GridInfo g;
    if (m.n_cells == 0) return g;
    for (i64 c = 0; c < m.n_cells; ++c)
        if (m.off[c + 1] - m.off[c] != 4) return g;
    std::vector<double> lo(m.lonlat.begin(), m.lonlat.begin() + m.n_nodes);
    std::vector<double> la(m.lonlat.begin() + m.n_nodes, m.lonlat.end());
    g.ulon = unique_tol(std::move(lo));
    g.ulat = unique_tol(std::move(la));
    if (g.ulon.size() < 2 || g.ulat.size() < 2) return g;
    i64 ni = static_cast<i64>(g.ulon.size()) - 1, nj = static_cast<i64>(g.ulat.size()) - 1;
    if (ni * nj != m.n_cells) return g;
    g.rectilinear = true;
    g.ni = ni;
    g.nj = nj;
    std::vector<double> dl(ni), dt(nj);
    for (i64 i = 0; i < ni; ++i) dl[i] = g.ulon[i + 1] - g.ulon[i];
    for (i64 j = 0; j < nj; ++j) dt[j] = g.ulat[j + 1] - g.ulat[j];
    if (!uniform(dl) || !uniform(dt)) return g;
    double sl = 0.0, st = 0.0;
    for (double d : dl) sl += d;
    for (double d : dt) st += d;
    g.regular = true;
    g.lon_min = g.ulon.front();
    g.lon_max = g.ulon.back();
    g.dlon = sl / static_cast<double>(ni);
    g.lat_min = g.ulat.front();
    g.lat_max = g.ulat.back();
    g.dlat = st / static_cast<double>(nj);
    return g;
}

// Host libm node vectors + trig cache, then device copies.
void mesh_upload_impl(Mesh &m) {
    std::vector<double> xyz(3 * m.n_nodes);
    const double *lon = m.lonlat.data(), *lat = m.lonlat.data() + m.n_nodes;
    parallel_range(m.n_nodes, [&](i64 b, i64 e) {
        for (i64 n = b; n < e; ++n) {
            double lo = lon[n] * kDeg2Rad, la = lat[n] * kDeg2Rad;
            double cl = std::cos(la);
            xyz[3 * n] = cl * std::cos(lo);
            xyz[3 * n + 1] = cl * std::sin(lo);
            xyz[3 * n + 2] = std::sin(la);
        }
    });
    m.grid = detect(m);
    std::vector<int> off(m.n_cells + 1), idx(m.n_conn);
    for (i64 c = 0; c <= m.n_cells; ++c) off[c] = static_cast<int>(m.off[c]);
    for (i64 k = 0; k < m.n_conn; ++k) idx[k] = static_cast<int>(m.idx[k]);
    m.d_off.upload(off.data(), off.size());
    m.d_idx.upload(idx.data(), idx.size());
    m.d_xyz.upload(xyz.data(), xyz.size());
    m.d_lonlat.upload(m.lonlat.data(), m.lonlat.size());
    if (m.grid.regular) {
        // NodeTrigCache (trig_cache.hpp:210-267)
        const GridInfo &g = m.grid;
        std::vector<double> t(2 * (g.ni + 1) + 2 * (g.nj + 1));
        for (i64 i = 0; i <= g.ni; ++i) {
            double r = (g.lon_min + static_cast<double>(i) * g.dlon) * kDeg2Rad;
            t[i] = std::sin(r);
            t[(g.ni + 1) + i] = std::cos(r);
        }
        for (i64 j = 0; j <= g.nj; ++j) {
            double r = (g.lat_min + static_cast<double>(j) * g.dlat) * kDeg2Rad;
            t[2 * (g.ni + 1) + j] = std::sin(r);
            t[2 * (g.ni + 1) + (g.nj + 1) + j] = std::cos(r);
        }
        m.d_trig.upload(t.data(), t.size());
    }
    AXGB_CUDA(cudaDeviceSynchronize());
}

// Reusable device staging for the host-pointer entry points.
// Device staging for the host-buffer batched apply: a ring of field-chunk
// buffers and three streams (copy in, compute, copy out) with events, kept
// across calls (one set per process, for the device current at first use;
// re-created if the device changes).
struct Staging {
    static constexpr int kRing = 3;
    std::mutex mu;
    DBuf<char> a, b;
    int device = -1;
    cudaStream_t h2d = nullptr, comp = nullptr, d2h = nullptr;
    cudaEvent_t loaded[kRing] = {}, computed[kRing] = {}, drained[kRing] = {};
    void *get_a(size_t bytes) {
        if (a.n < bytes) a.alloc(bytes);
        return a.p;
    }
    void *get_b(size_t bytes) {
        if (b.n < bytes) b.alloc(bytes);
        return b.p;
    }
    void ensure_streams() {
        int dev = 0;
        AXGB_CUDA(cudaGetDevice(&dev));
        if (dev == device && h2d) return;
        release_streams();
        a.release();
        b.release();
        for (cudaStream_t *st : {&h2d, &comp, &d2h}) AXGB_CUDA(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
        for (int q = 0; q < kRing; ++q)
            for (cudaEvent_t *ev : {&loaded[q], &computed[q], &drained[q]})
                AXGB_CUDA(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
        device = dev;
    }
    void release_streams() {
        for (cudaStream_t st : {h2d, comp, d2h})
            if (st) cudaStreamDestroy(st);
        h2d = comp = d2h = nullptr;
        for (int q = 0; q < kRing; ++q)
            for (cudaEvent_t *ev : {&loaded[q], &computed[q], &drained[q]})
                if (*ev) {
                    cudaEventDestroy(*ev);
                    *ev = nullptr;
                }
    }
    static Staging &get() {
        static Staging s;
        return s;
    }
};

void check_apply(const Matrix &m, const void *x, i64 ldx, const void *y, i64 ldy, i64 nrhs) {
    AXGB_REQUIRE(nrhs >= 0, "apply: nrhs < 0");
    if (nrhs == 0) return;
    AXGB_REQUIRE(ldx >= m.n_src, "apply: ld_x (" + std::to_string(ldx) + ") < n_src (" + std::to_string(m.n_src) + ")");
    AXGB_REQUIRE(ldy >= m.n_dst, "apply: ld_y (" + std::to_string(ldy) + ") < n_dst (" + std::to_string(m.n_dst) + ")");
    AXGB_REQUIRE(m.n_src == 0 || x != nullptr, "apply: x is NULL");
    AXGB_REQUIRE(m.n_dst == 0 || y != nullptr, "apply: y is NULL");
}

// Valid kernel choices: variant 0 (direct; unroll 1, 2 or 4), 1 (blocked,
// cp.async staging; 2 or 3 buffers), 2 (blocked, bulk copies; 2 buffers),
// 1 and 2 with 2, 4 or 8 fields per stage, 3 (blocked, producer warp and
// mbarrier ring of 2 or 3 slots, or 0: per row-length class the depth that
// lets more CTAs fit; 4 fields per stage); 4 (one fused launch
// for few fields; the other knobs unused); 5 (segmented, lane = field, 32
// fields per stage, 2 or 3 staging slots).
void check_split_params(const SplitParams &p, const char *who) {
    const std::string w(who);
    AXGB_REQUIRE(p.variant >= 0 && p.variant <= 5, w + ": variant must be 0 to 5");
    AXGB_REQUIRE(p.fields_per_pass >= 0, w + ": fields_per_pass must be >= 0");
    if (p.variant == 4) return;
    if (p.variant == 5) {
        AXGB_REQUIRE(p.stages == 2 || p.stages == 3, w + ": variant 5 takes 2 or 3 staging slots");
        return;
    }
    if (p.variant == 0) {
        AXGB_REQUIRE(p.unroll == 1 || p.unroll == 2 || p.unroll == 4, w + ": direct unroll must be 1, 2 or 4");
        return;
    }
    AXGB_REQUIRE(p.unroll == 2 || p.unroll == 4 || p.unroll == 8, w + ": staged fields per stage must be 2, 4 or 8");
    AXGB_REQUIRE(p.variant != 3 || p.unroll == 4, w + ": variant 3 stages 4 fields at a time");
    AXGB_REQUIRE(p.stages == 2 || (p.stages == 3 && p.variant != 2) || (p.stages == 0 && p.variant == 3),
                 w + ": staging buffers must be 2 (variant 2), 2-3 (variant 1) or 0 (per class), 2-3 (variant 3)");
}

SplitParams tune_split(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    std::vector<SplitParams> cands;
    for (int t : {4, 8})
        for (int ns : {2, 3})
            for (int fc : {0, 128, 64, 32, 16, 8})
                if (t <= std::max<i64>(2, nrhs) && (fc == 0 || fc < nrhs)) cands.push_back({1, fc, t, ns});
    cands.push_back({2, 64, 4, 2});
    for (int fc : {256, 128, 64, 0})
        for (int ns : {3, 0})
            if (nrhs >= 8 && (fc == 0 || fc < nrhs)) cands.push_back({3, fc, 4, ns});
    std::vector<i64> tiles = {nrhs};
    for (i64 t : {32, 8})
        if (t < nrhs) tiles.push_back(t);
    for (i64 t : tiles)
        for (int u : {2, 4})
            if (u <= std::max<i64>(1, nrhs)) cands.push_back({0, static_cast<int>(t), u});
    if (nrhs == 1) cands.push_back({0, 1, 1});
    if (nrhs <= 8) cands.push_back({4, 0, 1, 2});
    cudaEvent_t e0, e1;
    AXGB_CUDA(cudaEventCreate(&e0));
    AXGB_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    SplitParams arg = cands.front();
    for (const SplitParams &c : cands) {
        apply_split(m, x, ldx, y, ldy, nrhs, c, s);  // warm-up (and layout build)
        AXGB_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < 2; ++r) apply_split(m, x, ldx, y, ldy, nrhs, c, s);
        AXGB_CUDA(cudaEventRecord(e1, s));
        AXGB_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        AXGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            arg = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return arg;
}

// Host-buffer batch apply, LayoutLeft [n, n_vars]. Fields are streamed in
// chunks through two device staging halves on two streams, so the copies of
// one chunk overlap the apply of the other.
// Host-buffer batched apply: fields [n_vars][n] in host memory (pinned for
// full copy speed). Chunks of fields flow through a 3-deep ring of device
// buffers: copy in (stream h2d) -> apply (stream comp) -> copy out (stream
// d2h), so host-to-device copies, the apply and device-to-host copies of
// different chunks overlap. A chunk holds about 2^26 values (256 MiB FP32).
// Synchronous: returns when every result is in dst.
template <class T, class F>
void host_batch(Matrix &m, const T *src, T *dst, int64_t n_vars, F apply_fn) {
    auto &st = Staging::get();
    std::lock_guard<std::mutex> lk(st.mu);
    st.ensure_streams();
    constexpr int R = Staging::kRing;
    const int64_t ns = std::max<int64_t>(1, m.n_src), nd = std::max<int64_t>(1, m.n_dst);
    const int64_t per = std::max<int64_t>(1, std::min<int64_t>(n_vars, (int64_t(1) << 26) / (ns + nd)));
    T *dx = static_cast<T *>(st.get_a(sizeof(T) * ns * per * R));
    T *dy = static_cast<T *>(st.get_b(sizeof(T) * nd * per * R));
    int64_t chunk = 0;
    for (int64_t v0 = 0; v0 < n_vars; v0 += per, ++chunk) {
        const int64_t nv = std::min(per, n_vars - v0);
        const int b = static_cast<int>(chunk % R);
        T *x = dx + static_cast<int64_t>(b) * ns * per;
        T *y = dy + static_cast<int64_t>(b) * nd * per;
        if (chunk >= R) AXGB_CUDA(cudaStreamWaitEvent(st.h2d, st.computed[b], 0));  // x[b] no longer read
        if (m.n_src)
            AXGB_CUDA(cudaMemcpyAsync(x, src + v0 * m.n_src, sizeof(T) * m.n_src * nv, cudaMemcpyHostToDevice, st.h2d));
        AXGB_CUDA(cudaEventRecord(st.loaded[b], st.h2d));
        AXGB_CUDA(cudaStreamWaitEvent(st.comp, st.loaded[b], 0));
        if (chunk >= R) AXGB_CUDA(cudaStreamWaitEvent(st.comp, st.drained[b], 0));  // y[b] copied out
        apply_fn(x, ns, y, nd, nv, st.comp);
        AXGB_CUDA(cudaEventRecord(st.computed[b], st.comp));
        AXGB_CUDA(cudaStreamWaitEvent(st.d2h, st.computed[b], 0));
        if (m.n_dst)
            AXGB_CUDA(cudaMemcpyAsync(dst + v0 * m.n_dst, y, sizeof(T) * m.n_dst * nv, cudaMemcpyDeviceToHost, st.d2h));
        AXGB_CUDA(cudaEventRecord(st.drained[b], st.d2h));
    }
    AXGB_CUDA(cudaStreamSynchronize(st.h2d));
    AXGB_CUDA(cudaStreamSynchronize(st.comp));
    AXGB_CUDA(cudaStreamSynchronize(st.d2h));
}

SplitParams default_split_params(i64 nrhs);
SplitParams pick_params(Matrix &m, i64 nrhs) {
    std::lock_guard<std::mutex> lk(m.mu);
    auto it = m.tuned.find(nrhs);
    if (it != m.tuned.end()) return it->second;
    return default_split_params(nrhs);
}

SplitParams default_split_params(i64 nrhs) {
    SplitParams p;
    if (nrhs <= 2) {  // one fused launch
        p.variant = 4;
        p.fields_per_pass = 0;
        p.unroll = 1;
        p.stages = 2;
        return p;
    }
    if (nrhs >= 8) {  // producer-warp staged kernel, ring depth per row-length class
        p.variant = 3;
        p.fields_per_pass = 128;
        p.stages = 0;
        p.unroll = 4;
        return p;
    }
    p.variant = 1;
    p.fields_per_pass = 64;
    p.stages = 2;
    p.unroll = 4;
    return p;
}

}  // namespace
}  // namespace axgb

using namespace axgb;

extern "C" {

void axgb_default_config(axgb_regrid_config *cfg) {
    if (!cfg) return;
    cfg->method = AXGB_BILINEAR;
    cfg->norm_type = AXGB_DSTAREA;
    cfg->line_type = AXGB_GREAT_CIRCLE;
    cfg->unmapped = AXGB_UNMAPPED_IGNORE;
    cfg->use_limiter = 0;
    cfg->extrap_method = AXGB_EXTRAP_NEAREST_WET;
}

int axgb_init(int device) {
    AXGB_TRY({
        int n = 0;
        AXGB_CUDA(cudaGetDeviceCount(&n));
        AXGB_REQUIRE(device >= 0 && device < n, "axgb_init: no CUDA device " + std::to_string(device));
        AXGB_CUDA(cudaSetDevice(device));
        AXGB_CUDA(cudaFree(nullptr));
    });
}

int axgb_last_error(char *buf, size_t len) {
    const std::string &e = g_last_error;
    if (buf && len) {
        size_t n = std::min(len - 1, e.size());
        std::memcpy(buf, e.data(), n);
        buf[n] = '\0';
    }
    return static_cast<int>(e.size());
}

const char *axgb_version(void) { return "axgb 0.1 sm_103a"; }

int axgb_mesh_create(const double *node_coords, int64_t n_nodes, const int64_t *conn_offsets,
                     const int64_t *conn_indices, int64_t n_cells, int coord_sys, const double *areas,
                     const int32_t *mask, int *mesh_handle) {
    AXGB_TRY({
        AXGB_REQUIRE(mesh_handle, "mesh_create: mesh_handle is NULL");
        AXGB_REQUIRE(n_nodes >= 0 && n_cells >= 0, "mesh_create: negative size");
        AXGB_REQUIRE(n_nodes < (int64_t(1) << 31), "mesh_create: more than 2^31 nodes");
        AXGB_REQUIRE(coord_sys == AXGB_SPHERICAL_DEG,
                     "mesh_create: only SphericalDeg meshes are supported by the great-circle path");
        AXGB_REQUIRE(conn_offsets, "mesh_create: conn_offsets is NULL");
        AXGB_REQUIRE(n_nodes == 0 || node_coords, "mesh_create: node_coords is NULL");
        AXGB_REQUIRE(conn_offsets[0] == 0, "mesh_create: conn_offsets[0] != 0");
        for (int64_t c = 0; c < n_cells; ++c)
            AXGB_REQUIRE(conn_offsets[c + 1] >= conn_offsets[c], "mesh_create: conn_offsets not monotone at " +
                                                                    std::to_string(c));
        int64_t nconn = conn_offsets[n_cells];
        AXGB_REQUIRE(nconn < (int64_t(1) << 31), "mesh_create: more than 2^31 connectivity entries");
        AXGB_REQUIRE(nconn == 0 || conn_indices, "mesh_create: conn_indices is NULL");
        for (int64_t k = 0; k < nconn; ++k)
            AXGB_REQUIRE(conn_indices[k] >= 0 && conn_indices[k] < n_nodes,
                         "mesh_create: conn_indices[" + std::to_string(k) + "] out of range");
        for (int64_t k = 0; k < 2 * n_nodes; ++k)
            AXGB_REQUIRE(std::isfinite(node_coords[k]), "mesh_create: non-finite node coordinate at " +
                                                            std::to_string(k % std::max<int64_t>(1, n_nodes)));
        auto m = std::make_shared<Mesh>();
        m->n_nodes = n_nodes;
        m->n_cells = n_cells;
        m->n_conn = nconn;
        m->coord_sys = coord_sys;
        m->lonlat.assign(node_coords, node_coords + 2 * n_nodes);
        m->off.assign(conn_offsets, conn_offsets + n_cells + 1);
        m->idx.assign(conn_indices, conn_indices + nconn);
        if (areas) {
            m->has_area = true;
            m->d_user_area.upload(areas, n_cells);
        }
        if (mask) {
            m->has_mask = true;
            std::vector<int> mk(mask, mask + n_cells);
            m->d_mask.upload(mk.data(), mk.size());
        }
        mesh_upload_impl(*m);
        *mesh_handle = Registry::get().add(Registry::get().meshes, m);
    });
}

int axgb_mesh_create_regular(int64_t ni, int64_t nj, double lon_start, double lat_start, double dlon, double dlat,
                             int *mesh_handle) {
    AXGB_TRY({
        AXGB_REQUIRE(ni > 0 && nj > 0, "mesh_create_regular: ni and nj must be positive");
        // make_regular_mesh (python/axis_py.cpp:75-103) via to_unstructured
        // (src/topology/structured_grid.cpp:210-270)
        const int64_t nn = (ni + 1) * (nj + 1), nc = ni * nj;
        std::vector<double> ll(2 * nn);
        for (int64_t j = 0; j <= nj; ++j)
            for (int64_t i = 0; i <= ni; ++i) {
                ll[i + j * (ni + 1)] = lon_start + static_cast<double>(i) * dlon;
                ll[nn + i + j * (ni + 1)] = lat_start + static_cast<double>(j) * dlat;
            }
        std::vector<int64_t> off(nc + 1), idx(4 * nc);
        for (int64_t j = 0; j < nj; ++j)
            for (int64_t i = 0; i < ni; ++i) {
                int64_t c = i + j * ni;
                off[c] = 4 * c;
                idx[4 * c] = i + j * (ni + 1);
                idx[4 * c + 1] = (i + 1) + j * (ni + 1);
                idx[4 * c + 2] = (i + 1) + (j + 1) * (ni + 1);
                idx[4 * c + 3] = i + (j + 1) * (ni + 1);
            }
        off[nc] = 4 * nc;
        int rc = axgb_mesh_create(ll.data(), nn, off.data(), idx.data(), nc, AXGB_SPHERICAL_DEG, nullptr, nullptr,
                                  mesh_handle);
        if (rc != AXGB_SUCCESS) return rc;
    });
}

int axgb_mesh_info(int h, int64_t *n_nodes, int64_t *n_cells, int32_t *flags, int64_t *dims, double *vals) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().meshes, h, "mesh");
        if (n_nodes) *n_nodes = m->n_nodes;
        if (n_cells) *n_cells = m->n_cells;
        if (flags) {
            flags[0] = m->grid.regular;
            flags[1] = m->grid.rectilinear;
        }
        if (dims) {
            dims[0] = m->grid.ni;
            dims[1] = m->grid.nj;
        }
        if (vals) {
            vals[0] = m->grid.lon_min;
            vals[1] = m->grid.dlon;
            vals[2] = m->grid.lat_min;
            vals[3] = m->grid.dlat;
        }
    });
}

int axgb_mesh_cell_geometry(int h, double *area, double *cap_centroid, double *cap_radius, float *box,
                            int32_t *degenerate) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().meshes, h, "mesh");
        mesh_prepare(*m, 0);
        const i64 n = m->n_cells;
        if (area) m->d_area.download(area, n);
        if (cap_centroid || cap_radius) {
            std::vector<DCap> cap(n);
            m->d_cap.download(cap.data(), n);
            AXGB_CUDA(cudaDeviceSynchronize());
            for (i64 c = 0; c < n; ++c) {
                if (cap_centroid) {
                    cap_centroid[3 * c] = cap[c].x;
                    cap_centroid[3 * c + 1] = cap[c].y;
                    cap_centroid[3 * c + 2] = cap[c].z;
                }
                if (cap_radius) cap_radius[c] = cap[c].r;
            }
        }
        if (box) m->d_box.download(box, 6 * n);
        if (degenerate) {
            std::vector<unsigned char> f(n);
            m->d_flags.download(f.data(), n);
            AXGB_CUDA(cudaDeviceSynchronize());
            for (i64 c = 0; c < n; ++c) degenerate[c] = (f[c] >> 4) & 3;
        }
        AXGB_CUDA(cudaDeviceSynchronize());
    });
}

int axgb_destroy_mesh(int h) { AXGB_TRY(Registry::get().drop(Registry::get().meshes, h, "mesh")); }

int axgb_generate_weights(int src, int dst, const axgb_regrid_config *cfg_in, int *mat) {
    AXGB_TRY({
        AXGB_REQUIRE(mat, "generate_weights: matrix_handle is NULL");
        axgb_regrid_config cfg;
        axgb_default_config(&cfg);
        if (cfg_in) cfg = *cfg_in;
        auto &R = Registry::get();
        auto S = R.find(R.meshes, src, "mesh");
        auto D = R.find(R.meshes, dst, "mesh");
        // coordinate-system check of WeightGenerator::generate (weight_generator.cpp:1891-1896)
        AXGB_REQUIRE(S->coord_sys == D->coord_sys, "generate_weights: source and destination coordinate systems differ");
        auto M = std::make_shared<Matrix>();
        if (cfg.method == AXGB_CONSERVATIVE) {
            // dispatch of generate_conservative (weight_generator.cpp:3246-3302)
            bool done = false;
            if (S->grid.regular && D->grid.regular) {
                done = generate_conservative_regular(*S, *D, cfg, *M);  // may decline
                if (!done) M = std::make_shared<Matrix>();
            }
            if (!done && S->grid.rectilinear && D->grid.rectilinear) {
                done = generate_conservative_rectilinear(*S, *D, cfg, *M);
                if (!done) M = std::make_shared<Matrix>();
            }
            if (!done) {
                if (cfg.line_type != AXGB_GREAT_CIRCLE)
                    throw Error(AXGB_ERR_UNSUPPORTED, "conservative: Cartesian line type not provided");
                generate_conservative(*S, *D, cfg, *M);
            }
        } else if (cfg.method == AXGB_BILINEAR) {
            // dispatch of generate_bilinear (weight_generator.cpp:2306-2345)
            bool done = false;
            if (S->grid.regular && D->grid.regular) done = generate_bilinear_regular(*S, *D, cfg, *M);
            if (!done) {
                if (S->grid.rectilinear)
                    generate_bilinear(*S, *D, cfg, *M);
                else
                    generate_bilinear_general(*S, *D, cfg, *M);  // point location (weight_generator.cpp:2346-2667)
            }
        } else if (cfg.method == AXGB_NEAREST_NEIGHBOR) {
            generate_nearest(*S, *D, cfg, *M);  // generate_nearest (weight_generator.cpp:2097-2118)
        } else {
            throw Error(AXGB_ERR_UNSUPPORTED, "generate_weights: method " + std::to_string(cfg.method) +
                                                  " not provided (Conservative1stOrder, Bilinear and "
                                                  "NearestNeighbor are)");
        }
        // generate() applies the coastal post-pass to every method (weight_generator.cpp:2014)
        coastal_postpass(*S, *D, cfg, *M);
        *mat = R.add(R.mats, M);
    });
}

int axgb_generate_weights_c(int src, int dst, int method, int *mat) {
    axgb_regrid_config cfg;
    axgb_default_config(&cfg);
    switch (method) {
        case 0:
            cfg.method = AXGB_BILINEAR;
            break;
        case 1:
            cfg.method = AXGB_NEAREST_NEIGHBOR;
            break;
        case 2:
            cfg.method = AXGB_CONSERVATIVE;
            break;
        default:
            g_last_error = "generate_weights_c: method code must be 0, 1 or 2";
            return AXGB_ERROR;
    }
    return axgb_generate_weights(src, dst, &cfg, mat);
}

int axgb_matrix_stats(int h, int64_t *stats, double *times_ms) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        if (stats) {
            std::copy(m->stats, m->stats + 8, stats);
            stats[7] = m->src_renum ? 1 : 0;
        }
        if (times_ms) std::copy(m->times_ms, m->times_ms + 8, times_ms);
    });
}

int axgb_matrix_info(int h, int64_t *n_src, int64_t *n_dst, int64_t *nnz) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        if (n_src) *n_src = m->n_src;
        if (n_dst) *n_dst = m->n_dst;
        if (nnz) *nnz = m->nnz;
    });
}

int axgb_matrix_export_csr(int h, int64_t *row_ptr, int64_t *col_idx, double *values, double *frac_a, double *frac_b,
                           double *area_a, double *area_b) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        if (row_ptr) {
            std::vector<int> rp(m->n_dst + 1);
            m->row_ptr.download(rp.data(), rp.size());
            AXGB_CUDA(cudaDeviceSynchronize());
            for (size_t k = 0; k < rp.size(); ++k) row_ptr[k] = rp[k];
        }
        if (col_idx) {
            std::vector<int> c(m->nnz);
            m->col.download(c.data(), c.size());
            AXGB_CUDA(cudaDeviceSynchronize());
            for (size_t k = 0; k < c.size(); ++k) col_idx[k] = c[k];
        }
        if (values) m->val.download(values, m->nnz);
        if (frac_a) m->frac_a.download(frac_a, m->n_src);
        if (frac_b) m->frac_b.download(frac_b, m->n_dst);
        if (area_a) m->area_a.download(area_a, m->n_src);
        if (area_b) m->area_b.download(area_b, m->n_dst);
        AXGB_CUDA(cudaDeviceSynchronize());
    });
}

// ─── weight cache blob (include/axis/solver/weight_cache.hpp:49-157) ─────
// [magic u32 0x43574841, the reference's value (little-endian bytes "AHWC")]
// [version u32 = 1][endian u8][pad 7][n_src u64][n_dst u64]
// [nnz u64] then factor_list f64[nnz], factor_row i64[nnz], factor_col
// i64[nnz], frac_a f64[n_src], frac_b f64[n_dst], area_a f64[n_src], area_b
// f64[n_dst]. The COO triplets are written in CSR order.
namespace {
constexpr uint32_t kCacheMagic = 0x43574841u;
constexpr uint32_t kCacheVersion = 1;
constexpr int64_t kCacheHeader = 40;
inline uint8_t native_endian() {
    const uint16_t one = 1;
    uint8_t b;
    std::memcpy(&b, &one, 1);
    return b == 1 ? 0x01 : 0x02;
}
inline int64_t cache_size(int64_t ns, int64_t nd, int64_t nnz) { return kCacheHeader + 24 * nnz + 16 * ns + 16 * nd; }
}  // namespace

// COO triplets (any order) -> CSR, stable by row, then axgb_matrix_import_csr
// (which sorts each row by column, as to_csr).
static int import_coo(int64_t ns, int64_t nd, int64_t nz, const int64_t *rows, const int64_t *cols, const double *vals,
                      const double *fa, const double *fb, const double *aa, const double *ab, int *h, const char *who) {
    std::vector<int64_t> rp(nd + 1, 0);
    for (int64_t k = 0; k < nz; ++k) {
        AXGB_REQUIRE(rows[k] >= 0 && rows[k] < nd, std::string(who) + ": row out of range");
        AXGB_REQUIRE(cols[k] >= 0 && cols[k] < ns, std::string(who) + ": column out of range");
        rp[rows[k] + 1]++;
    }
    for (int64_t j = 0; j < nd; ++j) rp[j + 1] += rp[j];
    std::vector<int64_t> pos(rp.begin(), rp.end() - 1), cc(nz);
    std::vector<double> vv(nz);
    for (int64_t k = 0; k < nz; ++k) {
        const int64_t at = pos[rows[k]]++;
        cc[at] = cols[k];
        vv[at] = vals[k];
    }
    return axgb_matrix_import_csr(ns, nd, nz, rp.data(), cc.data(), vv.data(), fa, fb, aa, ab, h);
}

int axgb_matrix_serialize(int h, void *buf, int64_t buf_size, int64_t *written) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        const int64_t need = cache_size(m->n_src, m->n_dst, m->nnz);
        if (written) *written = need;
        if (!buf) return AXGB_SUCCESS;  // size query
        AXGB_REQUIRE(buf_size >= need, "matrix_serialize: buf_size (" + std::to_string(buf_size) + ") < required (" +
                                           std::to_string(need) + ")");
        std::vector<int> rp(m->n_dst + 1), c(m->nnz);
        m->row_ptr.download(rp.data(), rp.size());
        m->col.download(c.data(), c.size());
        uint8_t *p = static_cast<uint8_t *>(buf);
        const uint64_t ns = m->n_src, nd = m->n_dst, nz = m->nnz;
        std::memset(p, 0, kCacheHeader);
        std::memcpy(p, &kCacheMagic, 4);
        std::memcpy(p + 4, &kCacheVersion, 4);
        p[8] = native_endian();
        std::memcpy(p + 16, &ns, 8);
        std::memcpy(p + 24, &nd, 8);
        std::memcpy(p + 32, &nz, 8);
        double *vals = reinterpret_cast<double *>(p + kCacheHeader);
        m->val.download(vals, m->nnz);
        AXGB_CUDA(cudaDeviceSynchronize());
        int64_t *rows = reinterpret_cast<int64_t *>(p + kCacheHeader + 8 * nz);
        int64_t *cols = rows + nz;
        for (int64_t j = 0; j < m->n_dst; ++j)
            for (int k = rp[j]; k < rp[j + 1]; ++k) rows[k] = j;
        for (int64_t k = 0; k < m->nnz; ++k) cols[k] = c[k];
        double *fa = reinterpret_cast<double *>(cols + nz);
        double *fb = fa + ns, *aa = fb + nd, *ab = aa + ns;
        m->frac_a.download(fa, ns);
        m->frac_b.download(fb, nd);
        m->area_a.download(aa, ns);
        m->area_b.download(ab, nd);
        AXGB_CUDA(cudaDeviceSynchronize());
    });
}

int axgb_matrix_deserialize(const void *buf, int64_t buf_size, int *h) {
    AXGB_TRY({
        AXGB_REQUIRE(buf && h, "matrix_deserialize: NULL argument");
        AXGB_REQUIRE(buf_size >= kCacheHeader, "matrix_deserialize: buf_size (" + std::to_string(buf_size) +
                                                   ") < minimum header size (40)");
        const uint8_t *p = static_cast<const uint8_t *>(buf);
        uint32_t magic, version;
        uint64_t ns, nd, nz;
        std::memcpy(&magic, p, 4);
        std::memcpy(&version, p + 4, 4);
        std::memcpy(&ns, p + 16, 8);
        std::memcpy(&nd, p + 24, 8);
        std::memcpy(&nz, p + 32, 8);
        AXGB_REQUIRE(magic == kCacheMagic, "matrix_deserialize: invalid magic bytes");
        AXGB_REQUIRE(version == kCacheVersion, "matrix_deserialize: format version mismatch (expected 1, got " +
                                                   std::to_string(version) + ")");
        AXGB_REQUIRE(p[8] == native_endian(), "matrix_deserialize: endianness mismatch");
        AXGB_REQUIRE(ns < (uint64_t(1) << 31) && nd < (uint64_t(1) << 31) && nz < (uint64_t(1) << 31),
                     "matrix_deserialize: sizes above 2^31");
        const int64_t need = cache_size(static_cast<int64_t>(ns), static_cast<int64_t>(nd), static_cast<int64_t>(nz));
        AXGB_REQUIRE(buf_size >= need, "matrix_deserialize: blob size mismatch (buf_size=" + std::to_string(buf_size) +
                                           ", expected=" + std::to_string(need) + ")");
        // unaligned-safe copies of the body
        std::vector<double> vals(nz), fa(ns), fb(nd), aa(ns), ab(nd);
        std::vector<int64_t> rows(nz), cols(nz);
        const uint8_t *q = p + kCacheHeader;
        std::memcpy(vals.data(), q, 8 * nz);
        std::memcpy(rows.data(), q + 8 * nz, 8 * nz);
        std::memcpy(cols.data(), q + 16 * nz, 8 * nz);
        q += 24 * nz;
        std::memcpy(fa.data(), q, 8 * ns);
        std::memcpy(fb.data(), q + 8 * ns, 8 * nd);
        std::memcpy(aa.data(), q + 8 * ns + 8 * nd, 8 * ns);
        std::memcpy(ab.data(), q + 16 * ns + 8 * nd, 8 * nd);
        return import_coo(static_cast<int64_t>(ns), static_cast<int64_t>(nd), static_cast<int64_t>(nz), rows.data(),
                          cols.data(), vals.data(), fa.data(), fb.data(), aa.data(), ab.data(), h,
                          "matrix_deserialize");
    });
}

int axgb_esmf_write(const char *path, int64_t n_a, int64_t n_b, int64_t nnz, const double *S, const int32_t *col_idx,
                    const int32_t *row_idx) {
    AXGB_TRY({
        AXGB_REQUIRE(path, "esmf_write: NULL path");
        esmf_write(path, n_a, n_b, nnz, S, col_idx, row_idx);
    });
}

int axgb_esmf_read(const char *path, int64_t *n_a, int64_t *n_b, int64_t *nnz, double *S, int32_t *col_idx,
                   int32_t *row_idx, int64_t capacity) {
    AXGB_TRY({
        AXGB_REQUIRE(path && n_a && n_b && nnz, "esmf_read: NULL argument");
        EsmfWeights w = esmf_read(path);
        *n_a = w.n_a;
        *n_b = w.n_b;
        *nnz = static_cast<int64_t>(w.S.size());
        if (!S) return AXGB_SUCCESS;  // size query
        AXGB_REQUIRE(col_idx && row_idx, "esmf_read: NULL index arrays");
        AXGB_REQUIRE(capacity >= *nnz, "esmf_read: capacity (" + std::to_string(capacity) + ") < nnz (" +
                                           std::to_string(*nnz) + ")");
        std::copy(w.S.begin(), w.S.end(), S);
        std::copy(w.col1.begin(), w.col1.end(), col_idx);
        std::copy(w.row1.begin(), w.row1.end(), row_idx);
    });
}

int axgb_matrix_write_esmf(int h, const char *path) {
    AXGB_TRY({
        AXGB_REQUIRE(path, "matrix_write_esmf: NULL path");
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        std::vector<int> rp(m->n_dst + 1), c(m->nnz);
        std::vector<double> v(m->nnz);
        m->row_ptr.download(rp.data(), rp.size());
        m->col.download(c.data(), c.size());
        m->val.download(v.data(), v.size());
        AXGB_CUDA(cudaDeviceSynchronize());
        // 0-based -> 1-based (esmf_weight_io.cpp:82-90), in CSR order
        std::vector<int32_t> col1(m->nnz), row1(m->nnz);
        for (int64_t j = 0; j < m->n_dst; ++j)
            for (int k = rp[j]; k < rp[j + 1]; ++k) {
                row1[k] = static_cast<int32_t>(j + 1);
                col1[k] = c[k] + 1;
            }
        esmf_write(path, m->n_src, m->n_dst, m->nnz, v.data(), col1.data(), row1.data());
    });
}

int axgb_matrix_read_esmf(const char *path, int *h) {
    AXGB_TRY({
        AXGB_REQUIRE(path && h, "matrix_read_esmf: NULL argument");
        EsmfWeights w = esmf_read(path);
        AXGB_REQUIRE(w.n_a >= 0 && w.n_b >= 0, "matrix_read_esmf: negative n_a / n_b");
        const int64_t nz = static_cast<int64_t>(w.S.size());
        std::vector<int64_t> rows(nz), cols(nz);
        for (int64_t k = 0; k < nz; ++k) {  // 1-based -> 0-based (esmf_weight_io.cpp:163-167)
            rows[k] = static_cast<int64_t>(w.row1[k]) - 1;
            cols[k] = static_cast<int64_t>(w.col1[k]) - 1;
        }
        // frac and area arrays are zero, as the reference's read_esmf leaves them
        std::vector<double> za(w.n_a, 0.0), zb(w.n_b, 0.0);
        return import_coo(w.n_a, w.n_b, nz, rows.data(), cols.data(), w.S.data(), za.data(), zb.data(), za.data(),
                          zb.data(), h, "matrix_read_esmf");
    });
}

int axgb_matrix_import_csr(int64_t n_src, int64_t n_dst, int64_t nnz, const int64_t *row_ptr, const int64_t *col_idx,
                           const double *values, const double *frac_a, const double *frac_b, const double *area_a,
                           const double *area_b, int *h) {
    AXGB_TRY({
        AXGB_REQUIRE(h && row_ptr, "matrix_import_csr: NULL argument");
        AXGB_REQUIRE(n_src >= 0 && n_dst >= 0 && nnz >= 0, "matrix_import_csr: negative size");
        AXGB_REQUIRE(nnz < (int64_t(1) << 31) && n_src < (int64_t(1) << 31) && n_dst < (int64_t(1) << 31),
                     "matrix_import_csr: sizes above 2^31");
        AXGB_REQUIRE(row_ptr[0] == 0 && row_ptr[n_dst] == nnz, "matrix_import_csr: row_ptr ends");
        AXGB_REQUIRE(nnz == 0 || (col_idx && values), "matrix_import_csr: NULL col/values");
        std::vector<int> rp(n_dst + 1), col(nnz);
        std::vector<double> val(nnz);
        for (int64_t j = 0; j < n_dst; ++j) {
            AXGB_REQUIRE(row_ptr[j + 1] >= row_ptr[j], "matrix_import_csr: row_ptr not monotone");
            // sort each row by column, as to_csr does
            std::vector<std::pair<int64_t, double>> r;
            for (int64_t k = row_ptr[j]; k < row_ptr[j + 1]; ++k) {
                AXGB_REQUIRE(col_idx[k] >= 0 && col_idx[k] < n_src, "matrix_import_csr: column out of range");
                r.push_back({col_idx[k], values[k]});
            }
            std::stable_sort(r.begin(), r.end(), [](auto &a, auto &b) { return a.first < b.first; });
            for (size_t q = 0; q < r.size(); ++q) {
                col[row_ptr[j] + q] = static_cast<int>(r[q].first);
                val[row_ptr[j] + q] = r[q].second;
            }
        }
        for (int64_t j = 0; j <= n_dst; ++j) rp[j] = static_cast<int>(row_ptr[j]);
        auto M = std::make_shared<Matrix>();
        M->n_src = n_src;
        M->n_dst = n_dst;
        M->nnz = nnz;
        M->row_ptr.upload(rp.data(), rp.size());
        M->col.upload(col.data(), col.size());
        M->val.upload(val.data(), val.size());
        std::vector<double> ones_s(n_src, 1.0), ones_d(n_dst, 1.0), zs(n_src, 0.0), zd(n_dst, 0.0);
        M->frac_a.upload(frac_a ? frac_a : ones_s.data(), n_src);
        M->frac_b.upload(frac_b ? frac_b : ones_d.data(), n_dst);
        M->area_a.upload(area_a ? area_a : zs.data(), n_src);
        M->area_b.upload(area_b ? area_b : zd.data(), n_dst);
        AXGB_CUDA(cudaDeviceSynchronize());
        M->stats[3] = nnz;
        *h = Registry::get().add(Registry::get().mats, M);
    });
}

int axgb_matrix_prepare(int h, int format) {
    AXGB_TRY({
        AXGB_REQUIRE(format >= 0 && format <= 3, "matrix_prepare: format must be 0, 1, 2 or 3");
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        matrix_prepare(*m, format, 0);
    });
}

int axgb_probe_fp64_fma(int64_t iters, double *tflops) {
    AXGB_TRY({
        AXGB_REQUIRE(tflops && iters > 0 && iters <= (int64_t(1) << 24), "probe_fp64_fma: iters in [1, 2^24], tflops");
        *tflops = fp64_fma_tflops(iters);
    });
}

int axgb_matrix_device_status(int h, int32_t *status) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(status, "matrix_device_status: NULL status");
        AXGB_CUDA(cudaDeviceSynchronize());
        int v = 0;
        for (DBuf<int> *st : {&m->blocked.status, &m->seg.status})
            if (st->p) {
                int w = 0;
                AXGB_CUDA(cudaMemcpy(&w, st->p, sizeof(int), cudaMemcpyDeviceToHost));
                AXGB_CUDA(cudaMemset(st->p, 0, sizeof(int)));
                v |= w;
            }
        *status = v;
    });
}

int axgb_destroy_matrix(int h) {
    AXGB_TRY({
        AXGB_CUDA(cudaDeviceSynchronize());
        Registry::get().drop(Registry::get().mats, h, "matrix");
    });
}

int axgb_apply_f64(int h, const double *x, int64_t ldx, double *y, int64_t ldy, int64_t nrhs, axgb_stream_t stream) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        check_apply(*m, x, ldx, y, ldy, nrhs);
        if (nrhs > 0) apply_f64(*m, x, ldx, y, ldy, nrhs, static_cast<cudaStream_t>(stream));
    });
}

int axgb_apply_f32split_tuned(int h, const float *x, int64_t ldx, float *y, int64_t ldy, int64_t nrhs, int variant,
                              int fields_per_pass, int unroll, axgb_stream_t stream) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        check_apply(*m, x, ldx, y, ldy, nrhs);
        SplitParams p{variant, fields_per_pass, unroll, variant == 3 || variant == 5 ? 3 : 2};
        check_split_params(p, "apply");
        if (nrhs > 0) apply_split(*m, x, ldx, y, ldy, nrhs, p, static_cast<cudaStream_t>(stream));
    });
}

int axgb_autotune_f32split(int h, const float *x, int64_t ldx, float *y, int64_t ldy, int64_t nrhs,
                           axgb_stream_t stream, int32_t *best) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        check_apply(*m, x, ldx, y, ldy, nrhs);
        AXGB_REQUIRE(nrhs > 0, "autotune: nrhs must be positive");
        auto p = tune_split(*m, x, ldx, y, ldy, nrhs, static_cast<cudaStream_t>(stream));
        {
            std::lock_guard<std::mutex> lk(m->mu);
            m->tuned[nrhs] = p;
        }
        if (best) {
            best[0] = p.variant;
            best[1] = p.fields_per_pass;
            best[2] = p.unroll;
            best[3] = p.stages;
        }
    });
}

int axgb_set_autotune(int enable) {
    g_autotune = enable ? 1 : 0;
    return AXGB_SUCCESS;
}

int axgb_set_kernel_choice(int h, int64_t nrhs, const int32_t *choice) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(choice && nrhs > 0, "set_kernel_choice: NULL choice or nrhs <= 0");
        SplitParams p{choice[0], choice[1], choice[2], choice[3]};
        check_split_params(p, "set_kernel_choice");
        std::lock_guard<std::mutex> lk(m->mu);
        m->tuned[nrhs] = p;
    });
}

int axgb_get_kernel_choice(int h, int64_t nrhs, int32_t *choice, int32_t *cached) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(choice && nrhs > 0, "get_kernel_choice: NULL choice or nrhs <= 0");
        SplitParams p = default_split_params(nrhs);
        int32_t c = 0;
        {
            std::lock_guard<std::mutex> lk(m->mu);
            auto it = m->tuned.find(nrhs);
            if (it != m->tuned.end()) {
                p = it->second;
                c = 1;
            }
        }
        choice[0] = p.variant;
        choice[1] = p.fields_per_pass;
        choice[2] = p.unroll;
        choice[3] = p.stages;
        if (cached) *cached = c;
    });
}

int axgb_apply_f32split(int h, const float *x, int64_t ldx, float *y, int64_t ldy, int64_t nrhs,
                        axgb_stream_t stream) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        check_apply(*m, x, ldx, y, ldy, nrhs);
        if (nrhs > 0) {
            cudaStream_t s = static_cast<cudaStream_t>(stream);
            SplitParams p;
            bool have = false;
            {
                std::lock_guard<std::mutex> lk(m->mu);
                auto it = m->tuned.find(nrhs);
                if (it != m->tuned.end()) {
                    p = it->second;
                    have = true;
                }
            }
            if (!have && g_autotune) {
                p = tune_split(*m, x, ldx, y, ldy, nrhs, s);
                std::lock_guard<std::mutex> lk(m->mu);
                m->tuned[nrhs] = p;
                have = true;
            }
            if (!have) p = default_split_params(nrhs);
            apply_split(*m, x, ldx, y, ldy, nrhs, p, s);
        }
    });
}

int axgb_apply_f32split_hilo(int h, const float *x, int64_t ldx, float *y, int64_t ldy, float *y_lo, int64_t ld_lo,
                             int64_t nrhs, axgb_stream_t stream) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        check_apply(*m, x, ldx, y, ldy, nrhs);
        AXGB_REQUIRE(nrhs == 0 || m->n_dst == 0 || y_lo != nullptr, "apply_hilo: y_lo is NULL");
        AXGB_REQUIRE(nrhs == 0 || ld_lo >= m->n_dst, "apply_hilo: ld_lo < n_dst");
        if (nrhs > 0) apply_split(*m, x, ldx, y, ldy, nrhs, pick_params(*m, nrhs), static_cast<cudaStream_t>(stream),
                                  y_lo, ld_lo);
    });
}

int axgb_apply_c(int h, const double *src, double *dst, int n_src, int n_dst) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(n_src == m->n_src, "apply: src extent (" + std::to_string(n_src) + ") != matrix.n_src() (" +
                                            std::to_string(m->n_src) + ")");
        AXGB_REQUIRE(n_dst == m->n_dst, "apply: dst extent (" + std::to_string(n_dst) + ") != matrix.n_dst() (" +
                                            std::to_string(m->n_dst) + ")");
        AXGB_REQUIRE((n_src == 0 || src) && (n_dst == 0 || dst), "apply: NULL field");
        auto &st = Staging::get();
        std::lock_guard<std::mutex> lk(st.mu);
        double *dx = static_cast<double *>(st.get_a(sizeof(double) * std::max(1, n_src)));
        double *dy = static_cast<double *>(st.get_b(sizeof(double) * std::max(1, n_dst)));
        if (n_src) AXGB_CUDA(cudaMemcpy(dx, src, sizeof(double) * n_src, cudaMemcpyHostToDevice));
        apply_f64(*m, dx, std::max<int64_t>(1, n_src), dy, std::max<int64_t>(1, n_dst), 1, 0);
        if (n_dst) AXGB_CUDA(cudaMemcpy(dst, dy, sizeof(double) * n_dst, cudaMemcpyDeviceToHost));
    });
}

int axgb_nan_batch_apply_f64(int h, const double *x, int64_t ldx, double *y, int64_t ldy, int64_t nrhs,
                             double na_thres, axgb_stream_t stream) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        check_apply(*m, x, ldx, y, ldy, nrhs);
        nan_batch_apply_f64(*m, x, ldx, y, ldy, nrhs, na_thres, static_cast<cudaStream_t>(stream));
    });
}

int axgb_apply_masked_f64(int h, const double *x, double *y, const int32_t *dst_mask, axgb_stream_t stream) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        check_apply(*m, x, std::max<int64_t>(1, m->n_src), y, std::max<int64_t>(1, m->n_dst), 1);
        apply_masked_f64(*m, x, dst_mask, y, static_cast<cudaStream_t>(stream));
    });
}

int axgb_nan_batch_apply_host(int h, const double *src, int64_t n_src, double *dst, int64_t n_dst, int64_t n_vars,
                              double na_thres) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(n_src == m->n_src && n_dst == m->n_dst, "nan_batch_apply: extents do not match the matrix");
        AXGB_REQUIRE(n_vars >= 0, "nan_batch_apply: n_vars < 0");
        if (n_vars > 0)
            host_batch<double>(*m, src, dst, n_vars,
                               [&](const double *x, int64_t lx, double *y, int64_t ly, int64_t nv, cudaStream_t s) {
                                   nan_batch_apply_f64(*m, x, lx, y, ly, nv, na_thres, s);
                               });
    });
}

int axgb_batch_apply_host_f64(int h, const double *src, int64_t n_src, double *dst, int64_t n_dst, int64_t n_vars) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(n_src == m->n_src && n_dst == m->n_dst, "batch_apply: extents do not match the matrix");
        AXGB_REQUIRE(n_vars >= 0, "batch_apply: n_vars < 0");
        if (n_vars > 0)
            host_batch<double>(*m, src, dst, n_vars, [&](const double *x, int64_t lx, double *y, int64_t ly, int64_t nv,
                                                         cudaStream_t s) { apply_f64(*m, x, lx, y, ly, nv, s); });
    });
}

int axgb_batch_apply_host_f32split(int h, const float *src, int64_t n_src, float *dst, int64_t n_dst,
                                   int64_t n_vars) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(n_src == m->n_src && n_dst == m->n_dst, "batch_apply: extents do not match the matrix");
        AXGB_REQUIRE(n_vars >= 0, "batch_apply: n_vars < 0");
        if (n_vars > 0)
            host_batch<float>(*m, src, dst, n_vars,
                              [&](const float *x, int64_t lx, float *y, int64_t ly, int64_t nv, cudaStream_t s) {
                                  apply_split(*m, x, lx, y, ly, nv, pick_params(*m, nv), s);
                              });
    });
}

int axgb_batch_create(const int *handles, const int64_t *nrhs, int count, int *bh) {
    AXGB_TRY({
        AXGB_REQUIRE(bh && count >= 0 && (count == 0 || (handles && nrhs)), "batch_create: bad arguments");
        std::vector<std::shared_ptr<Matrix>> mats;
        std::vector<i64> nr;
        for (int q = 0; q < count; ++q) {
            mats.push_back(Registry::get().find(Registry::get().mats, handles[q], "matrix"));
            AXGB_REQUIRE(nrhs[q] >= 0, "batch_create: negative nrhs");
            nr.push_back(nrhs[q]);
        }
        auto b = batch_create(mats, nr);
        *bh = Registry::get().add(Registry::get().batches, b);
    });
}

int axgb_batch_apply(int bh, const float *const *x, const int64_t *ldx, float *const *y, const int64_t *ldy,
                     axgb_stream_t stream) {
    AXGB_TRY({
        auto b = Registry::get().find(Registry::get().batches, bh, "batch");
        batch_apply(*b, x, ldx, y, ldy, static_cast<cudaStream_t>(stream));
    });
}

int axgb_destroy_batch(int bh) {
    AXGB_TRY({
        AXGB_CUDA(cudaDeviceSynchronize());
        Registry::get().drop(Registry::get().batches, bh, "batch");
    });
}

int axgb_conservation_f64(int h, const double *src, const double *dst, int norm_type, double *out,
                          axgb_stream_t stream) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(out && (m->n_src == 0 || src) && (m->n_dst == 0 || dst), "conservation: NULL argument");
        conservation(*m, src, dst, false, norm_type, out, static_cast<cudaStream_t>(stream));
    });
}

int axgb_conservation_f64_noalloc(int h, const double *src, const double *dst, int norm_type, double *out,
                                  axgb_stream_t stream) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(out && (m->n_src == 0 || src) && (m->n_dst == 0 || dst), "conservation_noalloc: NULL argument");
        conservation_noalloc(*m, src, dst, norm_type, out, static_cast<cudaStream_t>(stream));
    });
}

int axgb_conservation_f32(int h, const float *src, const float *dst, int norm_type, double *out,
                          axgb_stream_t stream) {
    AXGB_TRY({
        auto m = Registry::get().find(Registry::get().mats, h, "matrix");
        AXGB_REQUIRE(out && (m->n_src == 0 || src) && (m->n_dst == 0 || dst), "conservation: NULL argument");
        conservation(*m, src, dst, true, norm_type, out, static_cast<cudaStream_t>(stream));
    });
}

}  // extern "C"
