// Linear BVH over points or boxes in [-1, 1]^3 (the unit sphere's
// bounding cube): 30-bit Morton codes, the Karras (2012) radix tree over
// the sorted codes, a bottom-up refit of float boxes, and per-node ropes
// (escape links) for stackless traversal. Node layout: internal nodes
// 0..n-2, leaf q at n-1+q; lo = (box min, left child or leaf item), hi =
// (box max, rope). The caller fills the leaves; shared by the conservative
// candidate search and the nearest-neighbour query.
#pragma once

#include "internal.hpp"

namespace axgb {
namespace {

__device__ __forceinline__ unsigned spread10(unsigned v) {
    v &= 1023u;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ unsigned morton30(double x, double y, double z) {
    auto q = [](double t) {
        double u = (t + 1.0) * 512.0;
        u = fmin(fmax(u, 0.0), 1023.0);
        return static_cast<unsigned>(u);
    };
    return (spread10(q(x)) << 2) | (spread10(q(y)) << 1) | spread10(q(z));
}

struct Bvh {
    int n;          // leaves
    int root;
    float4 *lo;     // [2n-1] (lo.xyz, left child | cell)
    float4 *hi;     // [2n-1] (hi.xyz, rope)
    int *parent;    // [2n-1]
    int *right;     // [n-1] right child of internal nodes
    int *flag;      // [n-1] refit arrival counters
    const unsigned *keys;  // sorted Morton keys [n]
};

__device__ __forceinline__ int delta(const unsigned *k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned a = k[i], b = k[j];
    if (a == b) return 32 + __clz(static_cast<unsigned>(i ^ j));
    return __clz(a ^ b);
}

// Internal node i of the Karras (2012) radix tree over sorted keys.
__global__ void k_internal(Bvh t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = t.n;
    if (i >= n - 1) return;
    const unsigned *k = t.keys;
    int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(k, n, i, i - d);
    int lmax = 2;
    while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int s = lmax >> 1; s >= 1; s >>= 1)
        if (delta(k, n, i, i + (l + s) * d) > dmin) l += s;
    int j = i + l * d;
    int dn = delta(k, n, i, j);
    int s = 0;
    int step = l;
    do {
        step = (step + 1) >> 1;
        if (delta(k, n, i, i + (s + step) * d) > dn) s += step;
    } while (step > 1);
    int g = i + s * d + min(d, 0);
    int lo_i = min(i, j), hi_i = max(i, j);
    int left = (lo_i == g) ? (n - 1 + g) : g;
    int right = (hi_i == g + 1) ? (n - 1 + g + 1) : (g + 1);
    t.lo[i].w = __int_as_float(left);
    t.right[i] = right;
    t.parent[left] = i;
    t.parent[right] = i;
}

__global__ void k_refit(Bvh t) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= t.n || t.n < 2) return;
    int node = t.parent[t.n - 1 + q];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&t.flag[node], 1) == 0) return;  // first child to arrive stops
        int l = __float_as_int(__ldcg(&t.lo[node].w));
        int r = __ldcg(&t.right[node]);
        float4 al = __ldcg(&t.lo[l]), ah = __ldcg(&t.hi[l]);
        float4 bl = __ldcg(&t.lo[r]), bh = __ldcg(&t.hi[r]);
        float4 nl = t.lo[node], nh;
        nl.x = fminf(al.x, bl.x);
        nl.y = fminf(al.y, bl.y);
        nl.z = fminf(al.z, bl.z);
        nh.x = fmaxf(ah.x, bh.x);
        nh.y = fmaxf(ah.y, bh.y);
        nh.z = fmaxf(ah.z, bh.z);
        nh.w = __int_as_float(-1);
        __stcg(&t.lo[node], nl);
        __stcg(&t.hi[node], nh);
        node = (node == t.root) ? -1 : t.parent[node];
    }
}

// rope(x): the right sibling of the first left-child ancestor-or-self of x.
__global__ void k_ropes(Bvh t) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int total = 2 * t.n - 1;
    if (x >= total) return;
    int node = x, rope = -1;
    while (node != t.root) {
        int p = t.parent[node];
        int l = __float_as_int(t.lo[p].w);
        if (l == node) {
            rope = t.right[p];
            break;
        }
        node = p;
    }
    t.hi[x].w = __int_as_float(rope);
}

// ─── exact nearest point ────────────────────────────────────────────────────
// An LBVH over a point set (float4 x, y, z; w unused) and per query the point
// at the least float squared distance dx*dx + dy*dy + dz*dz, exact ties to
// the lower point index. Morton codes use (s*x + ox, s*y + oy, s*z + oz), a
// uniform scale into the unit cube (codes shape the tree only); boxes and
// distances use the points as given. A box's float distance never exceeds
// that of a point inside it (the same clamped differences, the same order of
// summation, no contraction in the including units), so the walk, which
// skips nodes farther than the best so far, never skips a nearer point.

struct PtMap {
    double s, ox, oy, oz;
};

__device__ __forceinline__ unsigned pt_code(const float4 &p, const PtMap &m) {
    return morton30(m.s * p.x + m.ox, m.s * p.y + m.oy, m.s * p.z + m.oz);
}

// keys/vals of points ids[i] (or i when ids is null)
__global__ void k_pt_keys(const float4 *pts, const int *ids, i64 n, PtMap m, unsigned *keys, int *vals) {
    const i64 i = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int id = ids ? ids[i] : static_cast<int>(i);
    keys[i] = pt_code(pts[id], m);
    vals[i] = id;
}

__global__ void k_pt_leaves(Bvh t, const float4 *pts, const int *vals) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= t.n) return;
    const int s = vals[q];
    const float4 p = pts[s];
    t.lo[t.n - 1 + q] = make_float4(p.x, p.y, p.z, __int_as_float(s));
    t.hi[t.n - 1 + q] = make_float4(p.x, p.y, p.z, __int_as_float(-1));
}

__device__ __forceinline__ float pt_d2(const float4 &a, const float4 &q) {
    const float dx = a.x - q.x, dy = a.y - q.y, dz = a.z - q.z;
    return dx * dx + dy * dy + dz * dz;
}

struct PtTreeView {
    const float4 *lo, *hi;
    const unsigned *keys;  // sorted codes
    const int *vals;       // point index per sorted code
    const float4 *pts;
    int n;
    PtMap m;
};

// Nearest point to q (-1 when the set is empty); *err set if the walk
// exceeds its bound (a malformed tree).
__device__ int pt_nearest(const PtTreeView &T, const float4 &q, int *err) {
    if (T.n <= 0) return -1;
    float best = INFINITY;
    int bi = -1;
    auto take = [&](int s) {
        const float d2 = pt_d2(T.pts[s], q);
        if (d2 < best || (d2 == best && s < bi)) {
            best = d2;
            bi = s;
        }
    };
    // seed: the points on either side of the query in Morton order
    const unsigned code = pt_code(q, T.m);
    int lo_i = 0, hi_i = T.n;
    while (lo_i < hi_i) {
        const int mid = (lo_i + hi_i) >> 1;
        if (T.keys[mid] < code) lo_i = mid + 1;
        else hi_i = mid;
    }
    for (int k = max(0, lo_i - 1); k <= min(T.n - 1, lo_i); ++k) take(T.vals[k]);
    const int n_leaf_base = T.n - 1;
    // ropes visit every node at most once
    const int max_steps = 2 * (2 * n_leaf_base + 1) + 8;
    int steps = 0, node = 0;  // root: internal node 0, or the single leaf
    while (node >= 0) {
        if (++steps > max_steps) {
            atomicOr(err, 1);
            break;
        }
        const float4 lo = T.lo[node], hi = T.hi[node];
        const float dx = fmaxf(fmaxf(lo.x - q.x, 0.f), q.x - hi.x);
        const float dy = fmaxf(fmaxf(lo.y - q.y, 0.f), q.y - hi.y);
        const float dz = fmaxf(fmaxf(lo.z - q.z, 0.f), q.z - hi.z);
        if (dx * dx + dy * dy + dz * dz <= best) {  // nodes at the best distance are entered (ties)
            if (node >= n_leaf_base) {
                take(__float_as_int(lo.w));
                node = __float_as_int(hi.w);
            } else {
                node = __float_as_int(lo.w);
            }
        } else {
            node = __float_as_int(hi.w);
        }
    }
    return bi;
}

// The K nearest points to q in ascending (distance, index) order; returns
// how many were found (min(K, n)). Nodes at the K-th distance are entered,
// so ties resolve to the lower indices.
template <int K>
__device__ int pt_knearest(const PtTreeView &T, const float4 &q, int *out, float *outd, int *err) {
    int cnt = 0;
    float bd[K];
    int bi[K];
    auto take = [&](int s) {
        const float d2 = pt_d2(T.pts[s], q);
        if (cnt == K && !(d2 < bd[K - 1] || (d2 == bd[K - 1] && s < bi[K - 1]))) return;
        for (int k = 0; k < cnt; ++k)
            if (bi[k] == s) return;  // seeded already
        int at = cnt < K ? cnt++ : K - 1;
        while (at > 0 && (d2 < bd[at - 1] || (d2 == bd[at - 1] && s < bi[at - 1]))) {
            bd[at] = bd[at - 1];
            bi[at] = bi[at - 1];
            --at;
        }
        bd[at] = d2;
        bi[at] = s;
    };
    if (T.n <= 0) return 0;
    const unsigned code = pt_code(q, T.m);
    int lo_i = 0, hi_i = T.n;
    while (lo_i < hi_i) {
        const int mid = (lo_i + hi_i) >> 1;
        if (T.keys[mid] < code) lo_i = mid + 1;
        else hi_i = mid;
    }
    for (int k = max(0, lo_i - K / 2); k < min(T.n, lo_i + K / 2); ++k) take(T.vals[k]);
    const int n_leaf_base = T.n - 1;
    const int max_steps = 2 * (2 * n_leaf_base + 1) + 8;
    int steps = 0, node = 0;
    while (node >= 0) {
        if (++steps > max_steps) {
            atomicOr(err, 1);
            break;
        }
        const float4 lo = T.lo[node], hi = T.hi[node];
        const float dx = fmaxf(fmaxf(lo.x - q.x, 0.f), q.x - hi.x);
        const float dy = fmaxf(fmaxf(lo.y - q.y, 0.f), q.y - hi.y);
        const float dz = fmaxf(fmaxf(lo.z - q.z, 0.f), q.z - hi.z);
        if (cnt < K || dx * dx + dy * dy + dz * dz <= bd[K - 1]) {
            if (node >= n_leaf_base) {
                take(__float_as_int(lo.w));
                node = __float_as_int(hi.w);
            } else {
                node = __float_as_int(lo.w);
            }
        } else {
            node = __float_as_int(hi.w);
        }
    }
    for (int k = 0; k < cnt; ++k) {
        out[k] = bi[k];
        outd[k] = bd[k];
    }
    return cnt;
}

// Owner of a point tree's device arrays.
struct PtTree {
    DBuf<float4> lo, hi;
    DBuf<int> parent, right, flag, vals;
    DBuf<unsigned> keys;
    int n = 0;
    PtMap m{};
    PtTreeView view(const float4 *pts) const { return PtTreeView{lo.p, hi.p, keys.p, vals.p, pts, n, m}; }
};

// Builds the tree over pts[ids[i]] (or pts[0..n) when ids is null).
inline void build_pt_tree(PtTree &T, const float4 *pts, const int *ids, int n, PtMap m, cudaStream_t s) {
    auto blocks = [](i64 k, int t) { return static_cast<unsigned>((k + t - 1) / t); };
    T.n = n;
    T.m = m;
    if (n <= 0) return;
    T.lo.alloc(2 * n - 1);
    T.hi.alloc(2 * n - 1);
    T.parent.alloc(2 * n - 1);
    T.right.alloc(n > 1 ? n - 1 : 1);
    T.flag.alloc(n > 1 ? n - 1 : 1);
    T.vals.alloc(n);
    T.keys.alloc(n);
    k_pt_keys<<<blocks(n, 256), 256, 0, s>>>(pts, ids, n, m, T.keys.p, T.vals.p);
    AXGB_CUDA(cudaGetLastError());
    radix_sort_pairs_u32(T.keys.p, T.vals.p, n, 30, s);
    Bvh t{n, 0, T.lo.p, T.hi.p, T.parent.p, T.right.p, T.flag.p, T.keys.p};
    AXGB_CUDA(cudaMemsetAsync(T.parent.p, 0xff, sizeof(int) * (2 * n - 1), s));
    T.flag.zero(s);
    k_pt_leaves<<<blocks(n, 256), 256, 0, s>>>(t, pts, T.vals.p);
    if (n > 1) {
        k_internal<<<blocks(n - 1, 256), 256, 0, s>>>(t);
        k_refit<<<blocks(n, 256), 256, 0, s>>>(t);
    }
    k_ropes<<<blocks(2 * n - 1, 256), 256, 0, s>>>(t);
    AXGB_CUDA(cudaGetLastError());
}

}  // namespace
}  // namespace axgb
