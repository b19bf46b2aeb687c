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

}  // namespace
}  // namespace axgb
