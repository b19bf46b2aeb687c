// FP64 spherical geometry on the device. Every expression keeps the
// operation order of the reference (libs/axis/include/axis/detail/
// spherical_clipper.hpp:39-335) and the translation units that include
// this header are compiled with --fmad=false, so additions and products
// round exactly as the reference's host build does; sqrt and division are
// IEEE round-to-nearest on the device as on the host. Only atan2/acos come
// from CUDA's libdevice and may differ from the host libm by an ulp.
#pragma once

#include <cstdint>

namespace axgb {

struct DV3 {
    double x, y, z;
};

__device__ __forceinline__ double d_dot(const DV3 &a, const DV3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ DV3 d_cross(const DV3 &a, const DV3 &b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double d_lensq(const DV3 &v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
__device__ __forceinline__ DV3 d_normalize(const DV3 &v) {
    double len = sqrt(d_lensq(v));
    if (len < 1.0e-300) return {0.0, 0.0, 0.0};
    double inv = 1.0 / len;
    return {v.x * inv, v.y * inv, v.z * inv};
}
__device__ __forceinline__ DV3 d_add(const DV3 &a, const DV3 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }

// Fixed-capacity polygon in registers/local memory. push() past CAP sets
// `over`; with CAP = 32 this is exactly the reference's silent drop
// (SphericalPolygon::push, spherical_clipper.hpp:145-150), with a smaller
// CAP the caller re-runs the pair at CAP = 32.
template <int CAP>
struct DPoly {
    double x[CAP], y[CAP], z[CAP];
    int n;
    bool over;
    __device__ __forceinline__ void clear() {
        n = 0;
        over = false;
    }
    __device__ __forceinline__ void push(const DV3 &v) {
        if (n < CAP) {
            x[n] = v.x;
            y[n] = v.y;
            z[n] = v.z;
            ++n;
        } else {
            over = true;
        }
    }
    __device__ __forceinline__ DV3 at(int i) const { return {x[i], y[i], z[i]}; }
};

// Van Oosterom-Strackee fan from vertex 0, |sum of 2*atan2|
// (spherical_clipper.hpp:112-137).
template <int CAP>
__device__ double d_poly_area(const DPoly<CAP> &p) {
    if (p.n < 3) return 0.0;
    double total = 0.0;
    DV3 a = p.at(0);
    for (int i = 1; i < p.n - 1; ++i) {
        DV3 b = p.at(i), c = p.at(i + 1);
        double ab = d_dot(a, b);
        double ac = d_dot(a, c);
        double bc = d_dot(b, c);
        DV3 bxc = d_cross(b, c);
        double num = d_dot(a, bxc);
        double den = 1.0 + ab + ac + bc;
        double tri = 2.0 * atan2(num, den);
        total += tri;
    }
    return fabs(total);
}

// Arc (v1 -> v2) against the great circle of normal n1 = ea x eb, midpoint
// fallback (spherical_clipper.hpp:265-295; the caller passes the edge
// normal it already formed, the same product).
__device__ __forceinline__ DV3 d_arc_cross(const DV3 &v1, const DV3 &v2, const DV3 &n1) {
    DV3 n2 = d_cross(v1, v2);
    DV3 d = d_cross(n1, n2);
    double dl = d_lensq(d);
    if (dl < 1.0e-30) return d_normalize(d_add(v1, v2));
    DV3 c = d_normalize(d);
    DV3 mid = d_normalize(d_add(v1, v2));
    if (d_dot(c, mid) < 0.0) c = {-c.x, -c.y, -c.z};
    return c;
}

// Clip `subject` by every edge of `clip` (Sutherland-Hodgman on great
// circles, inclusive eps = -1e-14, edges with |a x b|^2 < 1e-30 skipped;
// spherical_clipper.hpp:181-229 and :301-335). Returns the overlap area;
// sets *over when a polygon exceeded CAP.
// The previous vertex's side test is the value the loop formed one step
// earlier (the same dot product), and the two buffers swap roles per edge.
template <int CAP>
__device__ double d_overlap_area(const DPoly<CAP> &subject, const DPoly<CAP> &clip, DPoly<CAP> &bufa,
                                 DPoly<CAP> &bufb, bool *over) {
    *over = subject.over || clip.over;
    if (subject.n < 3 || clip.n < 3) return 0.0;
    bufa.n = subject.n;
    bufa.over = false;
    for (int i = 0; i < subject.n; ++i) {
        bufa.x[i] = subject.x[i];
        bufa.y[i] = subject.y[i];
        bufa.z[i] = subject.z[i];
    }
    DPoly<CAP> *in = &bufa, *out = &bufb;
    constexpr double eps = -1.0e-14;
    for (int ci = 0; ci < clip.n; ++ci) {
        DV3 ea = clip.at(ci);
        DV3 eb = clip.at(ci + 1 == clip.n ? 0 : ci + 1);
        DV3 nrm = d_cross(ea, eb);
        if (d_lensq(nrm) < 1.0e-30) continue;
        out->clear();
        const int nin = in->n;
        DV3 prv = in->at(nin - 1);
        double dp = d_dot(nrm, prv);
        for (int i = 0; i < nin; ++i) {
            DV3 cur = in->at(i);
            double dc = d_dot(nrm, cur);
            bool cin = dc >= eps;
            bool pin = dp >= eps;
            if (cin) {
                if (!pin) out->push(d_arc_cross(prv, cur, nrm));
                out->push(cur);
            } else if (pin) {
                out->push(d_arc_cross(prv, cur, nrm));
            }
            prv = cur;
            dp = dc;
        }
        if (out->over) *over = true;
        DPoly<CAP> *t = in;
        in = out;
        out = t;
        if (in->n < 3) return 0.0;
    }
    return d_poly_area(*in);
}

// Degenerate classification (degenerate_cell_handler.hpp:115-142, 259-367):
// 0 none, 1 zero area, 2 collapsed, 3 self-intersecting.
template <int CAP>
__device__ int d_classify(const DPoly<CAP> &p, double area) {
    if (p.n < 3) return 1;
    if (area < 1e-25) return 1;
    const double t2 = 1e-15 * 1e-15;
    int uniq = 1;
    for (int i = 1; i < p.n; ++i) {
        bool dup = false;
        for (int j = 0; j < i; ++j) {
            DV3 d{p.x[i] - p.x[j], p.y[i] - p.y[j], p.z[i] - p.z[j]};
            if (d_lensq(d) < t2) {
                dup = true;
                break;
            }
        }
        if (!dup) ++uniq;
    }
    if (uniq < 3) return 2;
    if (p.n >= 4) {
        for (int i = 0; i < p.n; ++i) {
            int in = (i + 1) % p.n;
            for (int j = i + 2; j < p.n; ++j) {
                int jn = (j + 1) % p.n;
                if (jn == i) continue;
                DV3 a = p.at(i), b = p.at(in), c = p.at(j), d = p.at(jn);
                DV3 nab = d_cross(a, b);
                double dc = d_dot(nab, c), dd = d_dot(nab, d);
                if (dc * dd >= 0.0) continue;
                DV3 ncd = d_cross(c, d);
                double da = d_dot(ncd, a), db = d_dot(ncd, b);
                if (da * db >= 0.0) continue;
                return 3;
            }
        }
    }
    return 0;
}

}  // namespace axgb
